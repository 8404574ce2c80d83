"""Command-line driver: read a Rutherford-Boeing matrix, analyse, factorize
on the GPU, solve, and report as the reference's driver/spral_ssids.F90.

    python -m spral_gb300.driver [options] matrix.rb

Options (the reference driver's, where they apply to this path):
  --pos            positive-definite factorisation (Cholesky)
  --posdef         make up diagonally dominant values for a pattern-only file
  --nrhs=N         number of right-hand sides (each is A times a vector of ones)
  --scale=none     no scaling (the scaling algorithms are host-side and not
                   part of this path; --scale=equil uses a simple symmetric
                   equilibration instead)
  --mixed          FP32 factors with FP64 refinement (extension)
  --refine         refine the FP64 solve to bwd err <= 1e-14 (extension)
"""
import sys
import time

import numpy as np

from . import matrices as M, rb, ssids


def main(argv=None):
    argv = sys.argv[1:] if argv is None else argv
    filename, pos, dominant, nrhs, scale, mixed, refine = "matrix.rb", False, False, 1, "none", \
        False, False
    for a in argv:
        if a == "--pos":
            pos = True
        elif a == "--posdef":
            dominant = True
        elif a.startswith("--nrhs="):
            nrhs = int(a.split("=", 1)[1])
        elif a.startswith("--scale="):
            scale = a.split("=", 1)[1]
        elif a == "--mixed":
            mixed = True
        elif a == "--refine":
            refine = True
        elif a.startswith("--"):
            print(f"Unrecognised command line argument: {a}")
            return 1
        else:
            filename = a
    if nrhs < 1:
        return 0
    print(f"Reading '{filename}'...")
    m, n, ptr, row, val, tc = rb.rb_read(filename, "dominant" if dominant else "random")
    if tc[1] not in "sh" or m != n:
        print("Rutherford-Boeing read failed: the matrix is not square symmetric")
        return 1
    print("ok")
    rhs = np.tile(M.sym_matvec(ptr, row, val, np.ones(n))[:, None], (1, nrhs))
    opts = ssids.Options(precision=ssids.PRECISION_MIXED if mixed else ssids.PRECISION_FP64)
    print(f" Number of CUDA devices: {ssids.device_count()}")
    t0 = time.perf_counter()
    ak = ssids.analyse(ptr, row, ssids.order_mindeg(ptr, row), opts)
    t_anal = time.perf_counter() - t0
    print("ok")
    print(f" Analyse took {t_anal:14.6f}")
    print(f"Predict nfact = {float(ak.nfact):10.2e}")
    print(f"Predict nflop = {float(ak.nflops):10.2e}")
    scaling = M.equilibrate(ptr, row, val) if scale == "equil" else None
    print("Factorize...")
    t0 = time.perf_counter()
    fk = ssids.Fkeep(ak, val, opts, posdef=pos, scaling=scaling)
    t_fact = time.perf_counter() - t0
    inf = fk.inform
    if inf.flag < 0:
        print(f" oops on factorize {inf.flag}")
        return 1
    print("ok")
    print(f" Factor took {t_fact:14.6f}")
    print("Solve...")
    t0 = time.perf_counter()
    soln = fk.solve_refined(rhs) if (mixed or refine) and scaling is None else fk.solve(rhs)
    t_solve = time.perf_counter() - t0
    print("ok")
    print(f" Solve took {t_solve:14.6f}")
    print(f" number bad cmp = {int((np.abs(soln[:, 0] - 1.0) >= 1e-6).sum())}")
    print(f" fwd error || ||_inf = {np.abs(soln[:, 0] - 1.0).max():.16e}")
    res = M.scaled_bwd_error(ptr, row, val, soln, rhs)
    print(" bwd error scaled = " + " ".join(f"{r:.16e}" for r in np.atleast_1d(res)))
    print(f"{'cmp:':>6}{'SMFCT':>10}")
    print(f"{'anal:':>6}{t_anal:10.2f}")
    print(f"{'fact:':>6}{t_fact:10.2f}")
    print(f"{'afact:':>6}{float(ak.nfact):10.2e}")
    print(f"{'aflop:':>6}{float(ak.nflops):10.2e}")
    print(f"{'nfact:':>6}{float(inf.num_factor):10.2e}")
    print(f"{'nflop:':>6}{float(inf.num_flops):10.2e}")
    print(f"{'delay:':>6}{inf.num_delay:10d}")
    print(f"{'inertia:':>6}{inf.num_neg:10d}{n - inf.matrix_rank:10d}"
          f"{inf.matrix_rank - inf.num_neg:10d}")
    print(f"{'2x2piv:':>6}{inf.num_two:10d}")
    print(f"{'maxfront:':>6}{inf.maxfront:10d}")
    print(f"{'maxsupernode:':>6}{inf.maxsupernode:10d}")
    print(f"{'not_first_pass:':>6}{inf.not_first_pass:10d}")
    print(f"{'not_second_pass:':>6}{inf.not_second_pass:10d}")
    fk.free()
    return 0


if __name__ == "__main__":
    sys.exit(main())
