"""The wavefront-trace summary (spral_gb300.wavetrace) on a synthetic trace."""
import io

import numpy as np

from spral_gb300 import wavetrace


def test_wavetrace_summary(tmp_path):
    pre = str(tmp_path / "wt")
    # two fronts: 0 (level 0, small item) and 1 (level 1: gather, two pivot
    # blocks, one contribution block); backward: gather, partial, two blocks
    items = np.array([[0, 0x30000], [1, 0x20000], [1, 0], [1, 1], [1, 0x10000],
                      [1, 0x20000], [1, 0x100000], [1, 1], [1, 0], [0, 0x30000]], dtype=np.int32)
    t = np.zeros((10, 4), dtype=np.uint64)
    for i in range(10):
        t[i] = (1000 * i, 1000 * i + 400, 1000 * i + 900, i % 3)
    items.tofile(pre + ".items")
    t.tofile(pre + ".trace")
    with open(pre + ".meta", "w") as f:
        f.write("5 5\n0 40 20\n1 200 100\n")
    out = io.StringIO()
    wavetrace.summary(pre, out)
    text = out.getvalue()
    assert "forward: 5 items, span 4.9 us" in text
    assert "backward: 5 items, span 4.9 us" in text
    assert "T:     1 items" in text and "S:     1 items" in text
    assert "widest front (200 x 100 eliminated): 2 pivot blocks, chain step median 1.00 us" in text
    assert list(wavetrace.kind_of([0x30000, 0x20001, 0x100002, 5, 0x10003])) == list("SGTPC")
