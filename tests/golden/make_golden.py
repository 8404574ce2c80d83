"""Generate golden fixtures from the reference's own CPU numeric core.

Run where the reference source tree exists (``make -C oracle ref`` must have
built oracle/_ref/libspral_cpu_ref.so):

    python tests/golden/make_golden.py

For each case it stores the matrix, the ordering, right-hand sides and what
the reference returns for them: stats (inertia, delays, 2x2 count, flag),
solution, partial solves and enquire_indef output.  The GPU tests compare
against these files; the GPU host never needs the reference sources.
"""
import os
import zlib
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from spral_gb300 import matrices as M, ssids  # noqa: E402
import oracle  # noqa: E402


def cases():
    out = {}
    p, r, v = M.laplacian_2d(16, 16, -0.5)
    out["lap2d_16_shift-0.5"] = (p, r, v, M.nd_order_grid(16, 16), 3)
    p, r, v = M.laplacian_3d(8, shift=-0.3)
    out["lap3d_8_shift-0.3"] = (p, r, v, M.nd_order_grid(8, 8, 8), 2)
    p, r, v = M.random_indef(300, density=0.02, seed=3, diag_scale=0.01)
    out["rand_indef_300"] = (p, r, v, ssids.order_mindeg(p, r), 2)
    p, r, v = M.kkt(160, 60, seed=5)
    out["kkt_160_60"] = (p, r, v, ssids.order_mindeg(p, r), 2)
    return out


def main():
    oracle.build(with_ref=True)
    for name, (p, r, v, order, nrhs) in cases().items():
        ak = ssids.analyse(p, r, order)
        n = len(p) - 1
        rng = np.random.default_rng(zlib.crc32(name.encode()))
        b = rng.uniform(-1, 1, size=(n, nrhs))
        F = oracle.RefFactor(ak, v)
        x = F.solve(b)
        xf = F.solve(b, job=1)
        xd = F.solve(b, job=2)
        piv, d = F.enquire_indef()
        st = F.stats
        np.savez_compressed(os.path.join(HERE, f"{name}.npz"), ptr=p, row=r, val=v,
                            order=order, b=b, x=x, x_fwd=xf, x_diag=xd, piv_order=piv, d=d,
                            **{f"stat_{k}": np.array(val) for k, val in st.items()})
        bwd = M.scaled_bwd_error(p, r, v, x, b).max()
        print(f"{name}: n={n} neg={st['num_neg']} delay={st['num_delay']} two={st['num_two']} "
              f"flag={st['flag']} bwd={bwd:.2e}")


if __name__ == "__main__":
    main()
