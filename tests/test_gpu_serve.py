"""The request loop on the GPU: a Poisson stream of factor and same-pattern
refactor requests served with overlapping slots gives, for every request,
bitwise the result of serving that request alone."""
import numpy as np
import pytest

from spral_gb300 import matrices as M, serve

pytestmark = pytest.mark.gpu


def test_gpu_serving_mix_equals_alone():
    reqs = serve.poisson_stream(14, rate=300.0, seed=7, nmin=1000, nmax=30000, nrhs_max=8)
    mixed = serve.Server(slots=4)
    res = mixed.run(reqs, realtime=True)
    mixed.close()
    assert all(r.error is None for r in res), [r.error for r in res if r.error]
    # the mix really overlapped on the device
    spans = [(r.admitted, r.done) for r in res]
    overlaps = sum(1 for i, a in enumerate(spans) for b in spans[i + 1:]
                   if a[0] < b[1] and b[0] < a[1])
    assert overlaps > 0
    alone = serve.Server(slots=1)
    ref = alone.run(reqs, realtime=False)
    alone.close()
    for q, a, b in zip(reqs, res, ref):
        assert a.num_neg == b.num_neg
        assert np.array_equal(a.x, b.x), f"request {q.rid} differs alone and in the mix"
    # each answer solves its own system
    vals = {}
    for q, r in zip(reqs, res):
        if q.kind == "factor":
            vals[q.key] = (q.ptr, q.row)
        p, rw = vals[q.key]
        assert M.scaled_bwd_error(p, rw, q.val, r.x, q.b).max() <= 1e-14
        neg, _, _ = M.laplacian_eig_count_3d(*(3 * [round((len(p) - 1) ** (1 / 3))]),
                                             q.val[p[0]] - 6.0)
        assert r.num_neg == neg
