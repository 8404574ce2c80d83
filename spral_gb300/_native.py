"""Loader for the in-tree native library ``libspral_gb300.so``.

The library holds the host analyse (C++), the CUDA kernels for sm_103a and the
C-ABI declared in ``include/spral_ssids_gpu.h``.  There is no Python or CPU
fallback for the numeric path: if the library is missing, importing the
numeric API raises.
"""
import ctypes
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libspral_gb300.so")
_lib = None


class NativeLibraryMissing(RuntimeError):
    pass


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise NativeLibraryMissing(
                f"{LIB_PATH} not built; run `python -c 'import __graft_entry__ as g; g.build()'`")
        _lib = ctypes.CDLL(LIB_PATH, mode=ctypes.RTLD_GLOBAL)
        _declare(_lib)
    return _lib


P = ctypes.c_void_p
I = ctypes.c_int
I64 = ctypes.c_int64
D = ctypes.c_double
B = ctypes.c_bool


class CpuFactorOptions(ctypes.Structure):
    """Same layout as the reference's ``struct cpu_factor_options``
    (src/ssids/cpu/cpu_iface.hxx:27-37)."""
    _fields_ = [("print_level", I), ("action", B), ("small", D), ("u", D),
                ("multiplier", D), ("small_subtree_threshold", I64),
                ("cpu_block_size", I), ("pivot_method", I), ("failed_pivot_method", I)]


class ThreadStats(ctypes.Structure):
    """Same layout as the reference's ``struct ThreadStats``
    (src/ssids/cpu/ThreadStats.hxx:42-56)."""
    _fields_ = [("flag", I), ("num_delay", I), ("num_factor", I64), ("num_flops", I64),
                ("num_neg", I), ("num_two", I), ("num_zero", I), ("maxfront", I),
                ("maxsupernode", I), ("not_first_pass", I), ("not_second_pass", I)]


class GpuOptions(ctypes.Structure):
    """Out-of-band options of the GPU path (``struct spral_ssids_gpu_options``)."""
    _fields_ = [("precision", I), ("max_refine", I), ("refine_tol", D),
                ("small_front_cols", I), ("use_graph", I), ("no_fp64_fallback", I),
                ("reserved", I * 7)]


def _declare(L):
    def f(name, res, *args):
        fn = getattr(L, name, None)
        if fn is None:
            return
        fn.restype = res
        fn.argtypes = list(args)

    f("spral_gb300_analyse", P, I, P, P, P, I, ctypes.POINTER(I))
    f("spral_gb300_akeep_sizes", None, P, P)
    f("spral_gb300_akeep_arrays", None, P, P, P, P, P, P, P, P)
    f("spral_gb300_akeep_free", None, P)
    f("spral_gb300_order_mindeg", I, I, P, P, P)
    f("spral_gb300_order_amd", I, I, P, P, P)
    f("spral_ssids_gpu_create_symbolic_subtree", P, I, I, I, I, P, P, P, P, P, P,
      ctypes.POINTER(CpuFactorOptions))
    f("spral_ssids_gpu_destroy_symbolic_subtree", None, P)
    f("spral_ssids_gpu_create_num_subtree_dbl", P, B, P, P, P, P,
      ctypes.POINTER(CpuFactorOptions), ctypes.POINTER(ThreadStats))
    f("spral_ssids_gpu_destroy_num_subtree_dbl", None, B, P)
    for nm in ("fwd", "diag", "diag_bwd", "bwd"):
        f(f"spral_ssids_gpu_subtree_solve_{nm}_dbl", I, B, P, I, P, I)
    f("spral_ssids_gpu_subtree_enquire_dbl", None, B, P, P, P)
    f("spral_ssids_gpu_subtree_alter_dbl", None, B, P, P)
    f("spral_ssids_gpu_subtree_get_contrib_dbl", I, B, P, P, P, P, P, P, P, P, P)
    f("spral_ssids_gpu_subtree_free_contrib_dbl", None, B, P)
    f("spral_ssids_gpu_set_options", I, P, ctypes.POINTER(GpuOptions))
    f("spral_ssids_gpu_refactor_dev", I, P, P, ctypes.POINTER(ThreadStats), P)
    f("spral_ssids_gpu_refactor", I, P, P, P, ctypes.POINTER(ThreadStats))
    f("spral_ssids_gpu_solve_dev", I, P, I, I, P, I, P)
    f("spral_ssids_gpu_last_timing", I, P, P)
    f("spral_ssids_gpu_device_count", I)
    f("spral_ssids_gpu_debug_front", I, P, I, P, P, P, P)
    f("spral_ssids_gpu_solve_refined_dev", I, P, I, P, P, I, P, P)
    f("spral_ssids_gpu_fp64_fallbacks", I, P, P)
    f("spral_ssids_gpu_set_row_groups", I, P, I, P)
    f("spral_ssids_gpu_solve_refined", I, P, I, P, I, P)
    f("spral_ssids_gpu_launch_count", ctypes.c_longlong)
    f("spral_ssids_gpu_node_inertia", I, P, P)
    f("spral_ssids_gpu_mem_info", I, P, P)
    f("spral_ssids_gpu_release_cache", None)
    f("spral_ssids_gpu_tc_crossover", I)
    f("spral_ssids_gpu_contrib_update", I, I, P, I, P, P, I, I, I, P)
    f("spral_ssids_gpu_set_profiling", None, P, I)
    f("spral_ssids_gpu_profile_stats", None, P, P)
    f("spral_ssids_gpu_fp64_peak_tflops", D, I)
    f("spral_ssids_gpu_phase_times", None, P, P, P)
    f("spral_ssids_gpu_recip_probe", I, P, P, I)
    f("spral_ssids_gpu_ldlt_app_factor", I, I, I, P, P, I, P, D, P, I,
      ctypes.POINTER(CpuFactorOptions), P)
    f("spral_ssids_gpu_tc_gemm_f32", I, I, I, I, P, I, P, I, P, I, I, I, I, P)
    f("spral_ssids_gpu_tc_gemm_f32_bn", I, I, I, I, P, I, P, I, P, I, I, I, I, P, I)
    f("spral_ssids_gpu_tune_table", I, P, I)
    f("spral_ssids_gpu_group_bwd_errors", I, P, P, I)
    f("spral_ssids_gpu_tune_device_key", I, ctypes.c_char_p, I)
    f("spral_ssids_gpu_tune_parse", I, ctypes.c_char_p, ctypes.c_char_p, I, P, I)
    f("spral_ssids_gpu_tune_format", I, ctypes.c_char_p, P, I, ctypes.c_char_p, I)
    f("spral_ssids_gpu_tune_cache_lookup", I, ctypes.c_char_p, ctypes.c_char_p, P, I)
    f("spral_ssids_gpu_tune_cache_store", I, ctypes.c_char_p, ctypes.c_char_p, P, I)
    f("spral_ssids_gpu_level_schedule", I, I, P, P, P, I, P, P, P)
    f("spral_ssids_gpu_mbar_timeout_probe", I, I)
    f("spral_ssids_gpu_wave_timeout_probe", I, I)
    f("spral_ssids_gpu_inject_alloc_failure", None, I)
    f("spral_ssids_gpu_ldlt_app_factor_noalloc", I, I, I, P, P, I, P, D, P, I,
      ctypes.POINTER(CpuFactorOptions), P)
