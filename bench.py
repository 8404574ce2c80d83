#!/usr/bin/env python
"""Benchmark of the SSIDS numeric factor + solve on one GB300 per rank.

Workload (default): the 3D 7-point Laplacian on a 48^3 grid (n = 110,592),
diagonal shifted by -0.3 (indefinite), geometric nested-dissection order
(stand-in for METIS), 8 Gaussian right-hand sides from a fixed seed.  One
step = numeric factorisation of the matrix plus the solution of its 8
right-hand sides; the metric counts such solves per second and the line
records the scaled backward error actually reached.

Arms:
  default            the GB300 path (FP64 factors, the plain FP64 GPU path)
                     with inputs resident in HBM (value), the same through the
                     C-ABI with host buffers (e2e), the mixed-precision path
                     (FP32 factors + FP64 refinement) as a second line item,
                     the KKT saddle point (n = 15,000, AMD order: 2x2 pivots
                     and delays; mixed against FP64) as a third, the
                     contribution-GEMM roofline, and the CPU baseline
  --impl reference   the reference's CPU numeric path on the host cores:
                     the reference's own C++ core where it was compiled here,
                     else the oracle's C restatement (with OpenBLAS)

Multi-GPU: the factorizations are independent replicas (no data exchange in
the path), one process per GPU; value = all ranks' solves / max time.
"""
import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

METRIC = "solves/s at bwd err<=1e-14 mixed vs FP64 GPU; factor TFLOP/s; p50/p99 latency"
REFINE_TOL = 1e-14  # the metric's backward-error bound, applied to both paths


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--grid", type=int, default=48)
    ap.add_argument("--shift", type=float, default=-0.3)
    ap.add_argument("--nrhs", type=int, default=8)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-mixed", action="store_true")
    ap.add_argument("--no-kkt", action="store_true",
                    help="leave the KKT saddle-point object out of the default line")
    ap.add_argument("--mixed-only", action="store_true",
                    help="profiling aid: time only the mixed-precision path and print its object")
    ap.add_argument("--workload", default="lap3d",
                    choices=["lap3d", "batch", "serve", "tc-gemm", "kkt", "contrib"],
                    help="lap3d: the headline 48^3 Laplacian; batch: many small 2D Laplacians "
                         "factored and solved as one forest; serve: a Poisson stream of factor "
                         "and refactor requests through the request loop; tc-gemm: the "
                         "tensor-core Schur update kernel alone; contrib: the SIMT "
                         "contribution update of one thin wide front alone (HBM roofline); "
                         "kkt: a KKT saddle point "
                         "(random sparse H and A, -1e-8 I block) in mixed precision with FP64 "
                         "refinement against the FP64 path")
    ap.add_argument("--nemin", type=int, default=32,
                    help="supernode amalgamation parameter of the analyse (options%%nemin)")
    ap.add_argument("--kkt-nh", type=int, default=10000)
    ap.add_argument("--kkt-na", type=int, default=5000)
    ap.add_argument("--kkt-order", default="amd", choices=["amd", "natural"],
                    help="KKT pivot order: approximate minimum degree (interleaves the "
                         "constraint rows with H, so 2x2 pivots and delays occur) or the "
                         "natural order (H first: no 2x2 pivot is needed)")
    ap.add_argument("--kkt-cpu", action="store_true",
                    help="also time the CPU port on the kkt workload (about a minute)")
    ap.add_argument("--batch-count", type=int, default=4096)
    ap.add_argument("--serve-count", type=int, default=96)
    ap.add_argument("--serve-rate", type=float, default=8.0)
    ap.add_argument("--serve-slots", type=int, default=4)
    return ap.parse_args()


def problem(args):
    from spral_gb300 import matrices as M, ssids
    k = args.grid
    ptr, row, val = M.laplacian_3d(k, shift=args.shift)
    order = M.nd_order_grid(k, k, k)
    ak = ssids.analyse(ptr, row, order, ssids.Options(nemin=getattr(args, "nemin", 32)))
    rng = np.random.default_rng(2024)
    b = rng.standard_normal((len(ptr) - 1, args.nrhs))
    return ptr, row, val, ak, b


def config(args, ak, extra=None):
    c = {"workload": f"3D 7-point Laplacian {args.grid}^3 (n={ak.n}), shift {args.shift}, "
                     f"nested-dissection order, {args.nrhs} RHS N(0,1); one solve = numeric "
                     f"factor + {args.nrhs}-RHS solve",
         "n": ak.n, "nnz_lower": ak.nnz, "nrhs": args.nrhs, "nemin": args.nemin,
         "predicted_flops": ak.nflops, "nfactor": ak.nfact,
         "l2": "inputs larger than L2 (factors ~%.0f MB)" % (ak.nfact * 8 / 1e6),
         "parallelism": f"replicas x{args.gpus}"}
    if extra:
        c.update(extra)
    return c


class Clocks:
    """nvidia-smi sampling during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.f = tempfile.NamedTemporaryFile(mode="w+", suffix=".csv", delete=False)
        try:
            self.p = subprocess.Popen(["nvidia-smi", f"--id={index}", f"--query-gpu={self.Q}",
                                       "--format=csv,noheader,nounits", "-lms", "200"],
                                      stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.p = None

    def stop(self):
        if self.p is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.p.terminate()
        try:
            self.p.wait(timeout=5)
        except Exception:
            self.p.kill()
        self.f.flush()
        rows = []
        with open(self.f.name) as fh:
            for ln in fh:
                parts = [x.strip() for x in ln.split(",")]
                if len(parts) >= 9:
                    rows.append(parts)
        os.unlink(self.f.name)
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons, "samples": len(rows)}


def dist_setup(args):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def max_over_ranks(ms, dist, device):
    """The job's time per step: the slowest rank's (all_reduce MAX); `dist`
    is None on one rank."""
    if dist is None:
        return ms
    import torch
    t = torch.tensor([float(ms)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_value(world, ms):
    """Whole-job throughput of `world` independent replicas: all ranks'
    solves over the slowest rank's time per step (ms)."""
    return world * 1000.0 / ms


def cpu_reference_step_fn(ak, val, b, use_ref):
    import oracle
    if use_ref:
        def step():
            F = oracle.RefFactor(ak, val)
            return F.solve(b), F.stats
        kind = "reference"
    else:
        def step():
            F = oracle.OracleFactor(ak, val, blas=True)
            return F.solve(b), F.stats
        kind = "port"
    return step, kind


def run_reference(args):
    world, rank, local = dist_setup(args)
    if rank != 0:
        return
    import oracle
    from spral_gb300 import matrices as M
    oracle.build()
    ptr, row, val, ak, b = problem(args)
    use_ref = oracle.ref_available()
    step, kind = cpu_reference_step_fn(ak, val, b, use_ref)
    # warm-up steps as asked, each a full factor+solve (~1.4 s on 16 Arm
    # cores), within the time budget
    budget = 150.0
    t_w = time.perf_counter()
    nwarm = 0
    while nwarm < args.warmup and time.perf_counter() - t_w < budget / 3:
        step()
        nwarm += 1
    times = []
    x = None
    t_all = time.perf_counter()
    for i in range(args.steps):
        t0 = time.perf_counter()
        x, st = step()
        times.append(time.perf_counter() - t0)
        if time.perf_counter() - t_all > budget:
            break
    ms = 1000.0 * sum(times) / len(times)
    bwd = float(M.scaled_bwd_error(ptr, row, val, x, b).max())
    val_ = 1000.0 / ms
    cores = os.cpu_count()
    line = {"impl": "reference", "metric": METRIC, "value": val_, "unit": "solves/s",
            "n_gpus": args.gpus, "steps": len(times), "warmup": nwarm,
            "ms_per_step": ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64", "data": "synthetic",
            "config": config(args, ak, {"bwd_err": bwd, "num_neg": st["num_neg"]}),
            "cpu_baseline": {"value": val_, "unit": "solves/s", "cores": cores, "kind": kind,
                             "sample": f"{len(times)} full factor+solve steps of the workload "
                                       f"(OpenMP/OpenBLAS threads = {cores})"},
            "e2e": {"value": val_, "unit": "solves/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0},
            "p50_ms": float(np.percentile(np.array(times) * 1e3, 50)),
            "p99_ms": float(np.percentile(np.array(times) * 1e3, 99))}
    print(json.dumps(line), flush=True)


def rel_diff(x, xref):
    """max |x - xref| / max |xref| (the solution's error against the FP64
    CPU solution of the same right-hand sides)."""
    return float(np.abs(x - xref).max() / max(np.abs(xref).max(), 1e-300))


def hbm_peak_gbs():
    try:
        pk = json.load(open(os.path.join(HERE, "MEASURED_PEAKS.json")))
        return pk["hbm_gbs"], "measured copy bandwidth (MEASURED_PEAKS.json)"
    except Exception:
        return 6800.0, "fallback 6.8 TB/s"


def hbm_rooflines(ak, L, fk, ph_ms, b_d, x_d, n, nrhs, fp64_peak):
    """HBM rooflines of the solve and of the assembly (FP64 path), with the
    algorithmic byte counts: solve = 2 sum_nodes m*nelim*8 (L read in the
    forward and the backward pass) + sum_nodes 2*nelim*8 (D) + 2 sum_nodes
    m*nrhs*8*2 (local vectors gathered and scattered); assembly = sum over
    children cm(cm+1)/2 * (8 read + 8 parent write: the extend-add zeroes
    the parent's contribution columns in L2 before adding) + 4 cm (row map)
    plus loading A: nnz * (8 value + 16 index pair + 8 front).

    The FP64 solve also has a compute roofline: 2 passes x 2 flops x nrhs
    per strictly-lower entry of L, sum_nodes (m*nelim - nelim(nelim+1)/2),
    against the FP64 FMA rate.  On this GPU that bound (about 1.7 ms for the
    48^3 Laplacian's 8 right-hand sides) lies ten times above the HBM one,
    so the FP64 solve cannot reach a large fraction of HBM bandwidth."""
    import torch
    peak, src = hbm_peak_gbs()
    nrow, ncol = ak.front_sizes()
    solve_bytes = float(2 * (nrow * ncol).sum() * 8 + (2 * ncol * 8).sum()
                        + 2 * (nrow * nrhs * 8 * 2).sum())
    nrow64, ncol64 = nrow.astype(np.int64), ncol.astype(np.int64)
    solve_flops = float(2 * 2 * nrhs * (nrow64 * ncol64 - ncol64 * (ncol64 + 1) // 2).sum())
    times = []
    for _ in range(5):
        x_d.copy_(b_d)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        fk.solve_dev(x_d.data_ptr(), nrhs, n)  # returns after its stream is idle
        times.append(time.perf_counter() - t0)
    t_solve = float(np.median(times))
    cm = nrow - ncol
    parent = ak.sparent[:ak.nnodes] - 1
    has_parent = parent < ak.nnodes
    asm_bytes = float((cm[has_parent] * (cm[has_parent] + 1) / 2 * 16 + 4 * cm[has_parent]).sum()
                      + ak.nnz * 32)
    t_asm = (ph_ms[1] + ph_ms[4]) * 1e-3  # load A + extend-add phases
    return {"peak": peak, "unit": "GB/s", "peak_source": src,
            "solve": {"bytes": solve_bytes, "ms": t_solve * 1e3,
                      "achieved": solve_bytes / t_solve / 1e9,
                      "frac": solve_bytes / t_solve / 1e9 / peak,
                      "flops": solve_flops,
                      "fp64_tflops": solve_flops / t_solve / 1e12,
                      "fp64_frac": (solve_flops / t_solve / 1e12 / fp64_peak
                                    if fp64_peak > 0 else None),
                      "fp64_bound_ms": (solve_flops / fp64_peak / 1e9
                                        if fp64_peak > 0 else None),
                      "hbm_bound_ms": solve_bytes / peak / 1e6,
                      "note": f"one {nrhs}-RHS forward+backward solve, FP64 factors; "
                              "fp64_* = the same solve against the FP64 FMA rate, "
                              "its binding roofline on this GPU"},
            "assembly": {"bytes": asm_bytes, "ms": t_asm * 1e3,
                         "achieved": asm_bytes / t_asm / 1e9 if t_asm > 0 else None,
                         "frac": asm_bytes / t_asm / 1e9 / peak if t_asm > 0 else None,
                         "note": "load A + extend-add phases of one factorisation "
                                 "(phase timer, CUDA events)"}}


def solve_roofline_f32(ak, fk, b_d, x_d, n, nrhs):
    """HBM roofline of one forward+backward solve with FP32 factors: the
    FP64 path's byte count with 4-byte entries of L and of the local
    vectors (D stays FP64).  Both passes run as one persistent launch each
    and are bound by the chain of dependent pivot blocks, not by bytes."""
    import torch
    peak, src = hbm_peak_gbs()
    nrow, ncol = ak.front_sizes()
    nbytes = float(2 * (nrow * ncol).sum() * 4 + (2 * ncol * 8).sum()
                   + 2 * (nrow * nrhs * 4 * 2).sum())
    times = []
    for _ in range(5):
        x_d.copy_(b_d)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        fk.solve_dev(x_d.data_ptr(), nrhs, n)
        times.append(time.perf_counter() - t0)
    t = float(np.median(times))
    return {"bytes": nbytes, "ms": t * 1e3, "achieved": nbytes / t / 1e9, "peak": peak,
            "unit": "GB/s", "frac": nbytes / t / 1e9 / peak, "peak_source": src,
            "hbm_bound_ms": nbytes / peak / 1e6,
            "note": f"one {nrhs}-RHS forward+backward solve, FP32 factors (host clock "
                    "around a call that returns with its stream idle)"}


def tf32_peak_tflops():
    """TF32 tensor peak: the measured dense bf16 burst rate halved (tcgen05
    issues kind::tf32 at half the kind::f16 rate); fallback 1.9 PF/s bf16."""
    try:
        pk = json.load(open(os.path.join(HERE, "MEASURED_PEAKS.json")))
        return pk["bf16_tflops"] / 2.0, "measured bf16 burst / 2 (MEASURED_PEAKS.json)"
    except Exception:
        return 1900.0 / 2.0, "fallback 1.9 PF/s bf16 / 2"


def tensor_roofline(L, fk, aval_d, ak=None):
    """Roofline of the tensor-core Schur update (k_tc_gemm) inside one
    mixed-precision factorization, each launch timed with CUDA events on
    the library's stream.  Tensor flops = 3 x the FP32 update's flops
    (3xTF32 split products).  When no front takes the tensor cores (thin
    supernodes, below the depth rule) and ak is given, the roofline of the
    SIMT contribution update instead: HBM-bound, algorithmic bytes = the
    lower triangle of every contribution block read and written once in
    FP32, sum cm(cm+1)/2 * 8."""
    L.spral_ssids_gpu_set_profiling(fk.num, 1)
    fk.refactor_dev(aval_d.data_ptr())
    ps = np.zeros(6)
    L.spral_ssids_gpu_profile_stats(fk.num, ps.ctypes.data_as(ctypes.c_void_p))
    L.spral_ssids_gpu_set_profiling(fk.num, 0)
    peak, src = tf32_peak_tflops()
    if ps[3] <= 0:
        if ak is None or ps[0] <= 0:
            return None
        nrow, ncol = ak.front_sizes()
        cm = (nrow - ncol).astype(np.float64)
        nbytes = float((cm * (cm + 1) / 2 * 8).sum())
        hpk, hsrc = hbm_peak_gbs()
        gbs = nbytes / (ps[0] * 1e-3) / 1e9
        traffic = None
        tfile = os.path.join(HERE, "profiles", "contrib_f32_thin_front.md")
        if os.path.exists(tfile):
            import re
            m = re.search(r"dram_bytes_per_byte:\s*([0-9.eE+]+)", open(tfile).read())
            traffic = float(m.group(1)) * nbytes / max(int(ps[2]), 1) if m else None
        return {"bound": "hbm", "kernel": "k_syrk<float, 1> (SIMT contribution update)",
                "achieved": gbs, "peak": hpk, "unit": "GB/s", "frac": gbs / hpk,
                "traffic": traffic, "peak_source": hsrc, "launches": int(ps[2]),
                "bytes_per_step": nbytes, "contrib_update_ms": ps[0],
                "fp32_update_tflops": ps[1] / (ps[0] * 1e-3) / 1e12}
    alg = ps[4] / (ps[3] * 1e-3) / 1e12
    return {"bound": "tensor", "kernel": "k_tc_gemm (tcgen05 kind::tf32, 3xTF32 split)",
            "achieved": 3.0 * alg, "achieved_fp32_update": alg, "peak": peak,
            "unit": "TFLOP/s", "frac": 3.0 * alg / peak, "traffic": None,
            "peak_source": src, "launches": int(ps[5]), "flops_per_step": ps[4],
            "contrib_update_ms": ps[0], "tc_gemm_ms": ps[3], "autotuner": tune_table()}


def tune_table():
    """The library's autotuner table for this GPU: the SIMT / tensor-core
    crossover and the tile width per size class (largest contribution block
    of a launch, rows)."""
    from spral_gb300 import _native
    tab = np.zeros(32, dtype=np.int32)
    n = _native.lib().spral_ssids_gpu_tune_table(tab.ctypes.data_as(ctypes.c_void_p), 32)
    if n <= 0:
        return None
    t = tab[:n].tolist()
    return {"tc_min_cm": t[0],
            "tile_width_by_max_rows": {str(m): w for m, w in zip(t[2::2], t[3::2])}}


def run_gpu(args):
    import torch
    world, rank, local = dist_setup(args)
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group(backend="nccl")
    from spral_gb300 import _native, matrices as M, ssids
    L = _native.lib()
    ptr, row, val, ak, b = problem(args)
    n, nrhs = ak.n, args.nrhs
    dev = torch.device("cuda", local)
    bp = np.ascontiguousarray(b[ak.invp, :].T)  # (nrhs, n): column-major n x nrhs
    aval_d = torch.tensor(val, dtype=torch.float64, device=dev)
    b_d = torch.tensor(bp, dtype=torch.float64, device=dev)
    x_d = torch.empty_like(b_d)

    def barrier():
        if dist is not None:
            dist.barrier()

    def measure(fk, mixed):
        it = ctypes.c_int(0)
        bw = ctypes.c_double(0)

        def step():
            fk.refactor_dev(aval_d.data_ptr())
            # full solve plus FP64 refinement until bwd err <= 1e-14 (both paths)
            L.spral_ssids_gpu_solve_refined_dev(fk.num, nrhs, ctypes.c_void_p(b_d.data_ptr()),
                                                ctypes.c_void_p(x_d.data_ptr()), n,
                                                ctypes.byref(it), ctypes.byref(bw))

        for _ in range(args.warmup):
            step()
        torch.cuda.synchronize()
        barrier()
        lc0 = L.spral_ssids_gpu_launch_count()
        clk = Clocks(local) if rank == 0 else None
        ev0 = torch.cuda.Event(enable_timing=True)
        ev1 = torch.cuda.Event(enable_timing=True)
        per = []
        torch.cuda.synchronize()
        ev0.record()
        for _ in range(args.steps):
            t0 = time.perf_counter()
            step()
            torch.cuda.synchronize()
            per.append((time.perf_counter() - t0) * 1e3)
        ev1.record()
        torch.cuda.synchronize()
        clocks = clk.stop() if clk else None
        barrier()
        ms = ev0.elapsed_time(ev1) / args.steps
        launches = L.spral_ssids_gpu_launch_count() - lc0
        ms = max_over_ranks(ms, dist, dev)
        x = x_d.cpu().numpy().T
        xu = np.empty_like(x)
        xu[ak.invp, :] = x
        bwd = float(M.scaled_bwd_error(ptr, row, val, xu, b).max())
        measure.x = xu
        return ms, per, launches, clocks, bwd, it.value

    if args.mixed_only:
        fm = ssids.Fkeep(ak, val, ssids.Options(precision=ssids.PRECISION_MIXED, max_refine=20,
                                                 refine_tol=REFINE_TOL))
        mms, mper, mlaunch, _, mbwd, mit = measure(fm, mixed=True)
        if rank == 0:
            print(json.dumps({"metric": METRIC, "mixed_only": True, "ms_per_step": mms,
                              "value": world * 1000.0 / mms, "unit": "solves/s", "bwd_err": mbwd,
                              "refine_iters": mit, "gpu_launches": int(mlaunch),
                              "roofline": tensor_roofline(L, fm, aval_d)}), flush=True)
        fm.free()
        return

    opts64 = ssids.Options(precision=ssids.PRECISION_FP64, max_refine=10, refine_tol=REFINE_TOL)
    fk = ssids.Fkeep(ak, val, opts64)
    inform = fk.inform
    ms, per, launches, clocks, bwd, fp64_iters = measure(fk, mixed=False)
    x_fp64 = measure.x
    value = replica_value(world, ms)
    factor_tflops = inform.num_flops / (fk.timing()[0] * 1e-3) / 1e12

    # roofline of the dominant kernel: contribution GEMM, timed per launch
    L.spral_ssids_gpu_set_profiling(fk.num, 1)
    fk.refactor_dev(aval_d.data_ptr())
    ps = np.zeros(6)
    L.spral_ssids_gpu_profile_stats(fk.num, ps.ctypes.data_as(ctypes.c_void_p))
    ph_ms = np.zeros(32)
    ph_cnt = np.zeros(32, dtype=np.int64)
    L.spral_ssids_gpu_phase_times(fk.num, ph_ms.ctypes.data_as(ctypes.c_void_p),
                                  ph_cnt.ctypes.data_as(ctypes.c_void_p))
    L.spral_ssids_gpu_set_profiling(fk.num, 0)
    fp64_peak = L.spral_ssids_gpu_fp64_peak_tflops(local)
    bandwidth = hbm_rooflines(ak, L, fk, ph_ms, b_d, x_d, n, nrhs, fp64_peak)
    achieved = ps[1] / (ps[0] * 1e-3) / 1e12 if ps[0] > 0 else 0.0
    traffic = None
    tfile = os.path.join(HERE, "profiles", "contrib_gemm_fp64_lap3d48.md")
    if os.path.exists(tfile):
        import re
        m = re.search(r"dram_bytes_per_launch:\s*([0-9.eE+]+)", open(tfile).read())
        traffic = float(m.group(1)) if m else None
    roofline = {"bound": "fp64", "kernel": "k_syrk<double,contrib> (contribution block GEMM)",
                "achieved": achieved, "peak": fp64_peak, "unit": "TFLOP/s",
                "frac": achieved / fp64_peak if fp64_peak > 0 else None, "traffic": traffic,
                "peak_source": "FP64 FMA probe measured by bench.py on this GPU (the driver's "
                               "measured peaks cover HBM and bf16 tensor only)",
                "launches": int(ps[2]), "flops_per_step": ps[1]}

    # end to end through the C-ABI with host buffers
    copts = opts64.cpu_options()
    e2e_times = []
    xh = np.asfortranarray(b[ak.invp, :])
    for i in range(args.warmup + args.steps):
        t0 = time.perf_counter()
        st = _native.ThreadStats()
        num = L.spral_ssids_gpu_create_num_subtree_dbl(False, fk.sym,
                                                       val.ctypes.data_as(ctypes.c_void_p), None,
                                                       None, ctypes.byref(copts), ctypes.byref(st))
        xw = xh.copy(order="F")
        its = ctypes.c_int(0)
        L.spral_ssids_gpu_solve_refined(num, nrhs, xw.ctypes.data_as(ctypes.c_void_p), n,
                                        ctypes.byref(its))
        L.spral_ssids_gpu_destroy_num_subtree_dbl(False, num)
        if i >= args.warmup:
            e2e_times.append(time.perf_counter() - t0)
    e2e_ms = 1000.0 * sum(e2e_times) / len(e2e_times)
    e2e_ms = max_over_ranks(e2e_ms, dist, dev)
    e2e = {"value": replica_value(world, e2e_ms), "unit": "solves/s",
           "h2d_bytes_per_step": int(val.nbytes + n * nrhs * 8),
           "d2h_bytes_per_step": int(n * nrhs * 8),
           "path": "spral_ssids_gpu_create_num_subtree_dbl + spral_ssids_gpu_solve_refined "
                   "(host aval and x, FP64 factors)"}

    mixed = None
    if not args.no_mixed:
        fm = ssids.Fkeep(ak, val, ssids.Options(precision=ssids.PRECISION_MIXED, max_refine=20,
                                                 refine_tol=REFINE_TOL))
        mms, mper, mlaunch, _, mbwd, mit = measure(fm, mixed=True)
        x_mixed = measure.x
        mixed = {"value": world * 1000.0 / mms, "unit": "solves/s", "ms_per_step": mms,
                 "bwd_err": mbwd, "refine_iters": mit, "num_neg": fm.inform.num_neg,
                 "factor_ms": float(fm.timing()[0]),
                 "p50_ms": float(np.percentile(mper, 50)),
                 "p99_ms": float(np.percentile(mper, 99)),
                 "gpu_launches": int(mlaunch),
                 "speedup_vs_fp64_gpu": (1000.0 / mms) / (1000.0 / ms),
                 "roofline": tensor_roofline(L, fm, aval_d),
                 "solve": solve_roofline_f32(ak, fm, b_d, x_d, n, nrhs)}
        fm.free()

    cpu = None
    rel_fp64 = rel_mixed = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        import oracle
        oracle.build()
        step, kind = cpu_reference_step_fn(ak, val, b, oracle.ref_available())
        t0 = time.perf_counter()
        xc, stc = step()
        tc = time.perf_counter() - t0
        cpu = {"value": 1.0 / tc, "unit": "solves/s", "cores": os.cpu_count(), "kind": kind,
               "sample": "one full factor+solve of the workload (OpenBLAS threads = all cores)",
               "bwd_err": float(M.scaled_bwd_error(ptr, row, val, xc, b).max()),
               "num_neg": stc["num_neg"]}
        # each arm's solution against the FP64 CPU solution of the same b:
        # max |x - x_cpu| / max |x_cpu| over all right-hand sides
        rel_fp64 = rel_diff(x_fp64, xc)
        if mixed is not None:
            rel_mixed = rel_diff(x_mixed, xc)
            mixed["rel_vs_oracle"] = rel_mixed

    # the KKT saddle point (mixed precision against FP64), a compact object
    # of the same line
    kkt = None
    if not args.no_kkt and world == 1:
        import copy
        ka = copy.copy(args)
        ka.steps, ka.warmup, ka.kkt_cpu = 3, 2, not args.no_cpu_baseline
        kl = kkt_line(ka)
        if kl is not None:
            kkt = {"workload": kl["config"]["workload"], "n": kl["config"]["n"],
                   "maxfront": kl["config"]["maxfront"],
                   "num_neg_expected": kl["config"]["num_neg_expected"],
                   "value": kl["value"], "unit": "solves/s", "dtype": kl["dtype"],
                   "mixed": kl["mixed"], "fp64": kl["fp64"],
                   "speedup_mixed_vs_fp64_gpu": kl["speedup_mixed_vs_fp64_gpu"],
                   "e2e": kl["e2e"], "roofline": kl["roofline"],
                   "cpu_baseline": kl["cpu_baseline"]}

    if rank == 0:
        neg_exact, _, _ = M.laplacian_eig_count_3d(args.grid, args.grid, args.grid, args.shift)
        line = {"metric": METRIC, "value": value, "unit": "solves/s", "n_gpus": world,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
                "data": "synthetic (seeded 3D Laplacian and RHS)",
                "config": config(args, ak, {"bwd_err": bwd, "num_neg": inform.num_neg,
                                            "num_neg_exact": neg_exact,
                                            "num_delay": inform.num_delay,
                                            "refine_iters": fp64_iters,
                                            "num_flops": inform.num_flops,
                                            "rel_vs_oracle": rel_fp64}),
                "factor_tflops": factor_tflops,
                "p50_ms": float(np.percentile(per, 50)), "p99_ms": float(np.percentile(per, 99)),
                "e2e": e2e, "gpu_launches": int(launches), "roofline": roofline,
                "bandwidth": bandwidth,
                "cpu_baseline": cpu, "clocks": clocks, "mixed_precision": mixed,
                "kkt": kkt}
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()


def batch_problem(args):
    """Indefinite 2D 5-point Laplacians: side log-uniform in [8, 128], shift
    uniform in [-1, 0], one right-hand side uniform in [-1, 1] each."""
    from spral_gb300 import matrices as M
    rng = np.random.default_rng(4096)
    sides = np.exp(rng.uniform(np.log(8), np.log(128), args.batch_count)).astype(int)
    shifts = rng.uniform(-1.0, 0.0, args.batch_count)
    mats = [M.laplacian_2d(int(k), int(k), float(sh)) for k, sh in zip(sides, shifts)]
    orders = [M.nd_order_grid(int(k), int(k)) for k in sides]
    bs = [rng.uniform(-1, 1, int(k) * int(k)) for k in sides]
    return sides, shifts, mats, orders, bs


def run_batch(args):
    """One step = numeric factorisation of every matrix of the batch plus the
    solve of each one's right-hand side, refined in FP64 until every matrix's
    own scaled backward error is <= 1e-14.  Measured with FP64 factors
    (`value`) and with FP32 factors (`mixed`): at most 4 refinement steps,
    after which the matrices still above the target (shifts near an
    eigenvalue, too ill-conditioned for FP32 factors) are factored and
    solved again in FP64 as a sub-batch (BatchFkeep's per-matrix fallback)."""
    import torch
    world, rank, local = dist_setup(args)
    torch.cuda.set_device(local)
    from spral_gb300 import _native, batch, matrices as M, ssids
    L = _native.lib()
    sides, shifts, mats, orders, bs = batch_problem(args)
    bak = batch.BatchAkeep([(p, r) for p, r, _ in mats], orders)
    vals = bak.stack_values([v for _, _, v in mats])
    n = bak.n
    B, _ = bak.stack_rhs(bs)
    invp = bak.akeep.invp
    dev = torch.device("cuda", local)
    vals_d = torch.tensor(vals, dtype=torch.float64, device=dev)
    bp_d = torch.tensor(np.ascontiguousarray(B[invp, 0]), dtype=torch.float64, device=dev)
    x_d = torch.empty_like(bp_d)

    def measure(precision, max_refine):
        bf = batch.BatchFkeep(bak, [v for _, _, v in mats],
                              ssids.Options(precision=precision, max_refine=max_refine,
                                            refine_tol=REFINE_TOL))
        it = ctypes.c_int(0)

        def step():
            bf.refactor_dev(vals_d.data_ptr())
            # solve plus FP64 refinement of the whole batch to bwd err <= 1e-14
            # (FP32 factors: the matrices that miss it are refactored in FP64)
            it.value = bf.solve_refined_dev(bp_d, x_d)

        for _ in range(args.warmup):
            step()
        torch.cuda.synchronize()
        lc0 = L.spral_ssids_gpu_launch_count()
        clk = Clocks(local) if rank == 0 else None
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        per = []
        e0.record()
        for _ in range(args.steps):
            t0 = time.perf_counter()
            step()
            torch.cuda.synchronize()
            per.append((time.perf_counter() - t0) * 1e3)
        e1.record()
        torch.cuda.synchronize()
        clocks = clk.stop() if clk else None
        ms = e0.elapsed_time(e1) / args.steps
        launches = L.spral_ssids_gpu_launch_count() - lc0
        x = np.empty(n)
        x[invp] = x_d.cpu().numpy()
        xs = bak.split(x[:, None], True)
        bwd = max(float(M.scaled_bwd_error(p, r, v, xs[i], bs[i][:, None]).max())
                  for i, (p, r, v) in enumerate(mats))
        inert = bf.inertia()
        exact = all(inert[i, 0] == M.laplacian_eig_count_2d(int(k), int(k), float(sh))[0]
                    for i, (k, sh) in enumerate(zip(sides, shifts)))
        # end to end: host values and right-hand sides through the batch API
        e2e_t = []
        for i in range(args.warmup + args.steps):
            t0 = time.perf_counter()
            bf.refactor([v for _, _, v in mats])
            bf.solve_refined(bs)
            if i >= args.warmup:
                e2e_t.append(time.perf_counter() - t0)
        e2e_ms = 1000.0 * sum(e2e_t) / len(e2e_t)
        fb = bf.fk.fallbacks
        nfail = int(bf.failed.size)
        bf.free()
        return {"value": world * args.batch_count * 1000.0 / ms, "unit": "matrices/s",
                "ms_per_step": ms, "p50_ms": float(np.percentile(per, 50)),
                "p99_ms": float(np.percentile(per, 99)), "bwd_err": bwd,
                "refine_iters": it.value, "inertia_exact": bool(exact), "fp64_fallbacks": fb,
                "matrices_refactored_in_fp64": nfail,
                "gpu_launches": int(launches), "clocks": clocks,
                "e2e": {"value": args.batch_count * 1000.0 / e2e_ms, "unit": "matrices/s",
                        "h2d_bytes_per_step": int(vals.nbytes + n * 8),
                        "d2h_bytes_per_step": int(n * 8),
                        "path": "BatchFkeep.refactor + BatchFkeep.solve_refined (host values "
                                "and RHS)"}}

    fp64 = measure(ssids.PRECISION_FP64, 10)
    mixed = measure(ssids.PRECISION_MIXED, 4)
    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        import oracle
        oracle.build()
        t_all, done = 0.0, 0
        for i in range(len(mats)):  # a bounded sample, in batch order
            p, r, v = mats[i]
            ak = ssids.analyse(p, r, orders[i])
            t0 = time.perf_counter()
            F = oracle.OracleFactor(ak, v, blas=True)
            F.solve(bs[i])
            t_all += time.perf_counter() - t0
            done += 1
            if t_all > 15.0:
                break
        cpu = {"value": done / t_all, "unit": "matrices/s", "cores": os.cpu_count(),
               "kind": "port",
               "sample": f"first {done} matrices of the batch, one at a time (OpenBLAS threads = "
                         f"all cores)"}
    if rank == 0:
        line = {"metric": "matrices factored+solved per second (batched)", "workload": "batch",
                "value": fp64["value"], "unit": "matrices/s",
                "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
                "ms_per_step": fp64["ms_per_step"],
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
                "dtype": "f64",
                "data": "synthetic (seeded 2D Laplacians and right-hand sides)",
                "config": {"workload": f"{args.batch_count} indefinite 2D 5-point Laplacians, "
                                       "side log-uniform in [8,128], shift uniform[-1,0], "
                                       "nested-dissection order, FP64 values, 1 RHS "
                                       "uniform[-1,1] each; one step = factor + solve of every "
                                       "matrix refined to bwd err <= 1e-14",
                           "total_n": n, "nnodes": bak.akeep.nnodes,
                           "nflops": int(bak.akeep.nflops),
                           "bwd_err": fp64["bwd_err"], "refine_iters": fp64["refine_iters"],
                           "inertia_exact": fp64["inertia_exact"],
                           "l2": "inputs larger than L2"},
                "p50_ms": fp64["p50_ms"], "p99_ms": fp64["p99_ms"], "e2e": fp64["e2e"],
                "gpu_launches": fp64["gpu_launches"], "mixed": mixed, "cpu_baseline": cpu,
                "clocks": fp64["clocks"]}
        print(json.dumps(line), flush=True)


def run_serve(args):
    """The request loop on a seeded Poisson stream: 3D 7-point Laplacians with
    n log-uniform in [1e3, 2e5] (shift uniform[-0.5, 0]) and same-pattern
    refactorisations (diagonal x uniform[0.5, 2]), nrhs uniform in [1, 64],
    FP64, solves refined to bwd err <= 1e-14.  The timed region is the whole
    stream; `value` is requests served per second with overlapping slots and
    `alone` the same stream served one request at a time."""
    world, rank, local = dist_setup(args)
    import torch
    torch.cuda.set_device(local)
    from spral_gb300 import _native, matrices as M, serve, ssids
    L = _native.lib()
    reqs = serve.poisson_stream(args.serve_count, rate=args.serve_rate, seed=2025 + rank)
    opts = ssids.Options(max_refine=10, refine_tol=REFINE_TOL)
    # untimed warm-up: a few requests through a throw-away server
    warm = serve.Server(slots=args.serve_slots, options=opts)
    warm.run(serve.poisson_stream(4, rate=1000.0, seed=1, nmax=20000), realtime=False)
    warm.close()
    srv = serve.Server(slots=args.serve_slots, options=opts)
    for q in reqs:  # the host-side analyse is outside the timed region
        if q.kind == "factor":
            srv.akeeps[q.key] = ssids.analyse(q.ptr, q.row, q.order)
    lc0 = L.spral_ssids_gpu_launch_count()
    clk = Clocks(local) if rank == 0 else None
    t0 = time.perf_counter()
    res = srv.run(reqs, realtime=True)
    span = time.perf_counter() - t0
    clocks = clk.stop() if clk else None
    launches = L.spral_ssids_gpu_launch_count() - lc0
    srv.close()
    errors = [r.error for r in res if r.error]
    lat = np.array([r.latency for r in res if r.error is None]) * 1e3
    pats, bwd = {}, 0.0
    for q, r in zip(reqs, res):
        if q.kind == "factor":
            pats[q.key] = (q.ptr, q.row)
        if r.error is None:
            p, rw = pats[q.key]
            bwd = max(bwd, float(M.scaled_bwd_error(p, rw, q.val, r.x, q.b).max()))
    alone = serve.Server(slots=1, options=opts)
    alone.akeeps.update(srv.akeeps)
    ta = time.perf_counter()
    ref = alone.run(reqs, realtime=False)
    t_alone = time.perf_counter() - ta
    alone.close()
    same = all(a.error is None and np.array_equal(a.x, b.x) for a, b in zip(res, ref))
    # where the latency goes: waiting for a slot or memory (admitted -
    # arrival) against being served (done - admitted), and what the slowest
    # requests were; the service time alone is each request's time in the
    # one-at-a-time run
    ok = [(q, r, a) for q, r, a in zip(reqs, res, ref) if r.error is None and a.error is None]
    queue_ms = np.array([r.admitted - r.arrival for _, r, _ in ok]) * 1e3
    service_ms = np.array([r.done - r.admitted for _, r, _ in ok]) * 1e3
    alone_ms = np.array([a.done - a.admitted for _, _, a in ok]) * 1e3

    def pct(v, p):
        return float(np.percentile(v, p)) if v.size else None

    slow = sorted(ok, key=lambda t: -(t[1].done - t[1].arrival))[:3]
    breakdown = {
        "queue_ms": {"p50": pct(queue_ms, 50), "p99": pct(queue_ms, 99)},
        "service_ms": {"p50": pct(service_ms, 50), "p99": pct(service_ms, 99)},
        "service_alone_ms": {"p50": pct(alone_ms, 50), "p99": pct(alone_ms, 99)},
        "slowest": [{"kind": q.kind, "n": int(q.b.shape[0]), "nrhs": int(q.b.shape[1]),
                     "latency_ms": (r.done - r.arrival) * 1e3,
                     "queue_ms": (r.admitted - r.arrival) * 1e3,
                     "service_ms": (r.done - r.admitted) * 1e3,
                     "service_alone_ms": (a.done - a.admitted) * 1e3} for q, r, a in slow]}
    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        import oracle
        oracle.build()
        t_all, done = 0.0, 0
        for q in reqs:
            if q.kind != "factor":
                continue
            ak = srv.akeeps[q.key]
            t1 = time.perf_counter()
            F = oracle.OracleFactor(ak, q.val, blas=True)
            F.solve(q.b)
            t_all += time.perf_counter() - t1
            done += 1
            if t_all > 20.0:
                break
        cpu = {"value": done / t_all, "unit": "requests/s", "cores": os.cpu_count(),
               "kind": "port",
               "sample": f"the first {done} factor requests of the stream, one at a time, "
                         "factor + solve (OpenBLAS threads = all cores)"}
    nfac = sum(1 for q in reqs if q.kind == "factor")
    if rank == 0:
        line = {"metric": "requests served per second (Poisson stream); p50/p99 latency",
                "workload": "serve", "value": len(reqs) / span, "unit": "requests/s",
                "n_gpus": world, "steps": 1, "warmup": 1, "ms_per_step": span * 1e3,
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
                "dtype": "f64", "data": "synthetic (seeded Poisson stream of 3D Laplacians)",
                "config": {"workload": f"{len(reqs)} requests ({nfac} new matrices, "
                                       f"{len(reqs) - nfac} same-pattern refactorisations), "
                                       "3D 7-point Laplacians n log-uniform in [1e3, 2e5], "
                                       "shift uniform[-0.5,0], nrhs uniform[1,64], "
                                       f"Poisson arrivals at {args.serve_rate}/s, "
                                       f"{args.serve_slots} slots, memory-based admission",
                           "errors": errors[:3], "bwd_err": bwd,
                           "same_alone_and_in_mix": bool(same)},
                "p50_ms": float(np.percentile(lat, 50)) if lat.size else None,
                "p99_ms": float(np.percentile(lat, 99)) if lat.size else None,
                "latency_breakdown": breakdown,
                "alone": {"value": len(reqs) / t_alone, "unit": "requests/s",
                          "note": "same stream, one request at a time, no arrival waits"},
                "e2e": {"value": len(reqs) / span, "unit": "requests/s",
                        "h2d_bytes_per_step": int(sum(q.val.nbytes + q.b.nbytes for q in reqs)),
                        "d2h_bytes_per_step": int(sum(q.b.nbytes for q in reqs)),
                        "path": "serve.Server.run (host values and right-hand sides)"},
                "gpu_launches": int(launches), "cpu_baseline": cpu, "clocks": clocks}
        print(json.dumps(line), flush=True)


def run_tc_gemm(args):
    """The tensor-core Schur update alone (C -= A B^T, 3xTF32 split products,
    chunked FP32 accumulation): the largest contribution block of the 48^3
    workload (lower, 2304 x 2304, depth 1152) and a large square update;
    timed with CUDA events by the library, error against an FP64 product."""
    import torch
    from spral_gb300 import _native
    L = _native.lib()
    peak, src = tf32_peak_tflops()
    out = []
    for M_, N_, K_, lower in ((2304, 2304, 1152, 1), (8192, 8192, 2048, 0)):
        rng = np.random.default_rng(M_ + K_)
        A = rng.standard_normal((M_, K_)).astype(np.float32)
        B = rng.standard_normal((N_, K_)).astype(np.float32)
        dA = torch.tensor(A.ravel(order="F"), device="cuda")
        dB = torch.tensor(B.ravel(order="F"), device="cuda")
        dC = torch.zeros(M_ * N_, device="cuda", dtype=torch.float32)
        assert L.spral_ssids_gpu_tc_gemm_f32(M_, N_, K_, dA.data_ptr(), M_, dB.data_ptr(), N_,
                                             dC.data_ptr(), M_, lower, -1, 0, None) == 0
        got = dC.cpu().numpy().reshape(M_, N_, order="F").astype(np.float64)
        ref = -(A.astype(np.float64) @ B.astype(np.float64).T)
        mask = np.tril(np.ones((M_, N_), bool)) if lower else np.ones((M_, N_), bool)
        rms = float(np.sqrt(np.mean((got - ref)[mask] ** 2)) / np.sqrt(K_))
        ms = (ctypes.c_float * 2)()
        assert L.spral_ssids_gpu_tc_gemm_f32(M_, N_, K_, dA.data_ptr(), M_, dB.data_ptr(), N_,
                                             dC.data_ptr(), M_, lower, -1,
                                             max(args.steps, 3), ms) == 0
        flops = 2.0 * K_ * mask.sum()
        alg = flops / (ms[1] * 1e-3) / 1e12
        # every tile width of the kernel, beside the autotuned one above
        widths = {}
        for bn in (64, 128, 256):
            mw = (ctypes.c_float * 2)()
            assert L.spral_ssids_gpu_tc_gemm_f32_bn(M_, N_, K_, dA.data_ptr(), M_, dB.data_ptr(),
                                                    N_, dC.data_ptr(), M_, lower, -1,
                                                    max(args.steps, 3), mw, bn) == 0
            widths[str(bn)] = {"gemm_ms": mw[1], "tensor_tflops": 3 * flops / (mw[1] * 1e-3) / 1e12}
        out.append({"shape": f"{M_}x{N_}x{K_}" + (" lower" if lower else ""),
                    "gemm_ms": ms[1], "split_ms": ms[0], "fp32_update_tflops": alg,
                    "tensor_tflops": 3 * alg, "frac": 3 * alg / peak,
                    "rms_err_over_sqrtK": rms, "tile_widths": widths})
    tune = tune_table()
    print(json.dumps({"metric": "tensor-core Schur update TFLOP/s (3xTF32)", "workload": "tc-gemm",
                      "value": out[-1]["tensor_tflops"], "unit": "TFLOP/s",
                      "peak": peak, "peak_source": src, "autotuner": tune, "cases": out}),
          flush=True)


def run_contrib(args):
    """The SIMT contribution update of one front alone, C -= L21 (L21 D)^T on
    the lower triangle, through spral_ssids_gpu_contrib_update: the thin
    supernodes of the KKT workload's chain (k = 32 and 64 eliminated columns
    against a contribution block 9,728 rows wide) in FP32, where the update
    streams C through HBM, and the same in FP64.  Algorithmic bytes = the
    lower triangle of C read and written once (cm(cm+1)/2 entries x 2);
    C (190-380 MB) exceeds L2, so no flush between repetitions.  Timed with
    CUDA events on the stream of the launches; the first call's result is
    checked against an FP64 product on the host."""
    import torch
    from spral_gb300 import _native
    L = _native.lib()
    peak, src = hbm_peak_gbs()
    stream = torch.cuda.current_stream()
    out = []
    for dbl, cm, k in ((0, 9728, 32), (0, 9728, 64), (1, 9728, 32)):
        dt = torch.float64 if dbl else torch.float32
        npdt = np.float64 if dbl else np.float32
        rng = np.random.default_rng(cm + k + dbl)
        ld = cm + k
        Lh = (rng.standard_normal((ld, k)) * 0.1).astype(npdt)
        LDh = (rng.standard_normal((cm, k)) * 0.1).astype(npdt)
        Ch = np.tril(rng.standard_normal((cm, cm))).astype(npdt)
        dL = torch.tensor(Lh.ravel(order="F"), device="cuda")
        dLD = torch.tensor(LDh.ravel(order="F"), device="cuda")
        dC = torch.tensor(Ch.ravel(order="F"), device="cuda")
        h = stream.cuda_stream

        def call(reps):
            rc = L.spral_ssids_gpu_contrib_update(dbl, dL.data_ptr(), ld, dLD.data_ptr(),
                                                  dC.data_ptr(), cm, k, reps, h)
            assert rc == 0, rc

        call(1)
        got = dC.cpu().numpy().reshape(cm, cm, order="F").astype(np.float64)
        ref = Ch.astype(np.float64) - Lh[k:, :].astype(np.float64) @ LDh.astype(np.float64).T
        low = np.tril(np.ones((cm, cm), bool))
        err = float(np.abs(got - ref)[low].max())
        call(max(args.warmup, 3))
        reps = max(args.steps, 3)
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record(stream)
        call(reps)
        e1.record(stream)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / reps
        ent = cm * (cm + 1) / 2
        gbs = ent * 2 * (8 if dbl else 4) / (ms * 1e-3) / 1e9
        out.append({"dtype": "f64" if dbl else "f32", "cm": cm, "k": k, "ms": ms,
                    "achieved_gbs": gbs, "frac_hbm": gbs / peak,
                    "gflops": 2.0 * k * ent / (ms * 1e-3) / 1e9, "max_abs_err": err})
        del dL, dLD, dC
    print(json.dumps({"metric": "SIMT contribution update GB/s (lower C read + write)",
                      "workload": "contrib", "value": out[0]["achieved_gbs"], "unit": "GB/s",
                      "peak": peak, "peak_source": src, "cases": out}), flush=True)


def run_kkt(args):
    line = kkt_line(args)
    if line is not None:
        print(json.dumps(line), flush=True)


def kkt_line(args):
    """KKT saddle point [[H, A^T], [A, -1e-8 I]] with the benchmark
    definition's structure (H SPD with a random symmetric pattern of about 7
    entries per row, N(0,1) off-diagonals and diagonal = row abs-sum + 1; A
    with 4 N(0,1) entries per row at uniform columns) at nh x na = 10,000 x
    5,000 by default (the definition's 200,000 x 100,000 under the same
    approximate minimum-degree order has a dense root front of 105,834 rows
    and 4.1e14 predicted flops).  Approximate minimum-degree order (which
    interleaves constraint rows with H, so 2x2 pivots and delays occur), 8
    right-hand sides N(0,1).  One step = numeric factor + 8-RHS solve
    refined to bwd err <= 1e-14; `value` is the mixed-precision path (FP32
    factors, 2x2 pivots and delays decided in FP64), `fp64` the FP64 path."""
    import torch
    world, rank, local = dist_setup(args)
    torch.cuda.set_device(local)
    from spral_gb300 import _native, matrices as M, ssids
    L = _native.lib()
    nh, na = args.kkt_nh, args.kkt_na
    ptr, row, val = M.kkt(nh, na, seed=2026)
    order = ssids.order_amd(ptr, row) if args.kkt_order == "amd" else None
    ak = ssids.analyse(ptr, row, order, ssids.Options(nemin=args.nemin))
    n, nrhs = ak.n, args.nrhs
    b = np.random.default_rng(2027).standard_normal((n, nrhs))
    dev = torch.device("cuda", local)
    aval_d = torch.tensor(val, dtype=torch.float64, device=dev)
    b_d = torch.tensor(np.ascontiguousarray(b[ak.invp, :].T), dtype=torch.float64, device=dev)
    x_d = torch.empty_like(b_d)

    def measure(prec, steps):
        fk = ssids.Fkeep(ak, val, ssids.Options(precision=prec, max_refine=20,
                                                 refine_tol=REFINE_TOL))
        it = ctypes.c_int(0)
        bw = ctypes.c_double(0)

        def step():
            fk.refactor_dev(aval_d.data_ptr())
            L.spral_ssids_gpu_solve_refined_dev(fk.num, nrhs, ctypes.c_void_p(b_d.data_ptr()),
                                                ctypes.c_void_p(x_d.data_ptr()), n,
                                                ctypes.byref(it), ctypes.byref(bw))

        for _ in range(args.warmup):
            step()
        torch.cuda.synchronize()
        lc0 = L.spral_ssids_gpu_launch_count()
        clk = Clocks(local) if rank == 0 else None
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(steps):
            step()
        e1.record()
        torch.cuda.synchronize()
        clocks = clk.stop() if clk else None
        ms = e0.elapsed_time(e1) / steps
        x = x_d.cpu().numpy().T
        xu = np.empty_like(x)
        xu[ak.invp, :] = x
        if prec == ssids.PRECISION_MIXED:
            measure.x_mixed = xu
        else:
            measure.x_fp64 = xu
        # the statistics that apply after the solves: an FP32-factor handle
        # whose refinement could not reach the target was refactored in FP64
        st = _native.ThreadStats()
        nfb = L.spral_ssids_gpu_fp64_fallbacks(fk.num, ctypes.byref(st))
        out = {"value": 1000.0 / ms, "unit": "solves/s", "ms_per_step": ms,
               "factor_ms": float(fk.timing()[0]),
               "bwd_err": float(M.scaled_bwd_error(ptr, row, val, xu, b).max()),
               "refine_iters": it.value, "num_neg": int(st.num_neg),
               "num_two": int(st.num_two), "num_delay": int(st.num_delay),
               "fp64_fallbacks": int(nfb), "num_flops": fk.inform.num_flops,
               "gpu_launches": int(L.spral_ssids_gpu_launch_count() - lc0), "clocks": clocks}
        if nfb > 0:
            out["fp32_factor_num_neg"] = fk.inform.num_neg
        return fk, out

    fm, mixed = measure(ssids.PRECISION_MIXED, args.steps)
    roof = tensor_roofline(L, fm, aval_d, ak)
    # end to end through the C-ABI with host buffers (mixed precision)
    g = ssids.Options(precision=ssids.PRECISION_MIXED, max_refine=20, refine_tol=REFINE_TOL)
    copts = g.cpu_options()
    xh = np.asfortranarray(b[ak.invp, :])
    e2e_t = []
    for i in range(args.warmup + args.steps):
        t0 = time.perf_counter()
        st = _native.ThreadStats()
        num = L.spral_ssids_gpu_create_num_subtree_dbl(False, fm.sym,
                                                       val.ctypes.data_as(ctypes.c_void_p), None,
                                                       None, ctypes.byref(copts), ctypes.byref(st))
        xw = xh.copy(order="F")
        its = ctypes.c_int(0)
        L.spral_ssids_gpu_solve_refined(num, nrhs, xw.ctypes.data_as(ctypes.c_void_p), n,
                                        ctypes.byref(its))
        L.spral_ssids_gpu_destroy_num_subtree_dbl(False, num)
        if i >= args.warmup:
            e2e_t.append(time.perf_counter() - t0)
    fm.free()
    f64, fp64 = measure(ssids.PRECISION_FP64, max(1, min(args.steps, 3)))
    f64.free()
    cpu = None
    if rank == 0 and args.kkt_cpu:
        import oracle
        oracle.build()
        t0 = time.perf_counter()
        F = oracle.OracleFactor(ak, val, blas=True)
        xc = F.solve(b)
        tc = time.perf_counter() - t0
        cpu = {"value": 1.0 / tc, "unit": "solves/s", "cores": os.cpu_count(), "kind": "port",
               "sample": "one full factor+solve (OpenBLAS threads = all cores)",
               "bwd_err": float(M.scaled_bwd_error(ptr, row, val, xc, b).max()),
               "num_neg": F.stats["num_neg"], "num_two": F.stats["num_two"],
               "num_delay": F.stats["num_delay"]}
        mixed["rel_vs_oracle"] = rel_diff(measure.x_mixed, xc)
        fp64["rel_vs_oracle"] = rel_diff(measure.x_fp64, xc)
    if rank == 0:
        e2e_ms = 1000.0 * sum(e2e_t) / len(e2e_t)
        line = {"metric": METRIC, "workload": "kkt", "value": mixed["value"],
                "unit": "solves/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
                "ms_per_step": mixed["ms_per_step"], "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "f32 factors, f64 refinement",
                "data": "synthetic (seeded KKT values and RHS)",
                "config": {"workload": f"KKT [[H, A^T], [A, -1e-8 I]], H {nh}x{nh} SPD (7 "
                                       f"nnz/row), A {na}x{nh} (4 nnz/row), n={n}, "
                                       f"{'approximate minimum-degree' if args.kkt_order == 'amd' else 'natural'} "
                                       f"order, {nrhs} RHS N(0,1); one solve = "
                                       f"numeric factor + {nrhs}-RHS solve refined to bwd err "
                                       f"<= 1e-14",
                           "n": n, "nnz_lower": ak.nnz, "predicted_flops": ak.nflops,
                           "maxfront": int(ak.front_sizes()[0].max()), "nemin": args.nemin,
                           "num_neg_expected": na,
                           "l2": "inputs larger than L2 (factors ~%.0f MB in FP32)"
                                 % (ak.nfact * 4 / 1e6)},
                "mixed": mixed, "fp64": fp64,
                "speedup_mixed_vs_fp64_gpu": mixed["value"] / fp64["value"],
                "e2e": {"value": 1000.0 / e2e_ms, "unit": "solves/s",
                        "h2d_bytes_per_step": int(val.nbytes + n * nrhs * 8),
                        "d2h_bytes_per_step": int(n * nrhs * 8),
                        "path": "spral_ssids_gpu_create_num_subtree_dbl + "
                                "spral_ssids_gpu_solve_refined (host aval and x, FP32 factors)"},
                "gpu_launches": mixed["gpu_launches"], "roofline": roof, "cpu_baseline": cpu,
                "clocks": mixed["clocks"]}
        return line
    return None


def main():
    args = parse()
    if args.workload == "tc-gemm":
        run_tc_gemm(args)
        return
    if args.workload == "contrib":
        run_contrib(args)
        return
    if args.impl == "reference":
        run_reference(args)
    elif args.workload == "batch":
        run_batch(args)
    elif args.workload == "serve":
        run_serve(args)
    elif args.workload == "kkt":
        run_kkt(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
