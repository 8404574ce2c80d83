/*
 * spral_ssids_gpu.h -- C-ABI of the GB300 numeric factorize-and-solve for
 * SPRAL SSIDS.
 *
 * These entry points replace the GPU subtree of SSIDS (the type-bound
 * procedures of gpu_symbolic_subtree / gpu_numeric_subtree in
 * src/ssids/gpu/subtree.f90:20-72) and are shaped exactly like the CPU
 * subtree's C interface (src/ssids/cpu/SymbolicSubtree.cxx:14-28,
 * src/ssids/cpu/NumericSubtree.cxx:29-262), so that a Fortran binding can
 * call them the way src/ssids/cpu/subtree.f90 calls the CPU ones.
 *
 * Conventions (as at the reference boundary, described in
 * src/ssids/cpu/SymbolicSubtree.hxx:20-48): all index arrays are 1-based and
 * Fortran-ordered; x is column-major n x nrhs in pivot order (already
 * permuted by invp and scaled by the caller, src/ssids/fkeep.F90:252-266).
 * Options and statistics use the reference's struct layouts.  Errors are
 * reported through ThreadStats.flag / return codes; nothing exits or throws.
 */
#ifndef SPRAL_SSIDS_GPU_H
#define SPRAL_SSIDS_GPU_H

#include <stdbool.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Same layout as struct cpu_factor_options (src/ssids/cpu/cpu_iface.hxx:27). */
struct spral_ssids_cpu_factor_options {
  int print_level;
  bool action;
  double small;
  double u;
  double multiplier;
  int64_t small_subtree_threshold;
  int cpu_block_size;
  int pivot_method;        /* 1 app_aggressive, 2 app_block, 3 tpp */
  int failed_pivot_method; /* 1 tpp, 2 pass */
};

/* Same layout as struct ThreadStats (src/ssids/cpu/ThreadStats.hxx:42). */
struct spral_ssids_thread_stats {
  int flag;
  int num_delay;
  int64_t num_factor;
  int64_t num_flops;
  int num_neg;
  int num_two;
  int num_zero;
  int maxfront;
  int maxsupernode;
  int not_first_pass;
  int not_second_pass;
};

/* Out-of-band options of the GPU path (the public spral_ssids_options
 * struct is not changed).  precision: 0 = FP64 factors, 1 = FP32 factors with
 * FP64 pivot decisions and FP64 iterative refinement in the solve. */
struct spral_ssids_gpu_options {
  int precision;
  int max_refine;
  double refine_tol;
  int small_front_cols;
  int use_graph;
  /* 1: an FP32-factor handle whose refined solve cannot reach refine_tol
   * returns its best refined solution instead of refactoring the matrix in
   * FP64 (the caller handles the rest, e.g. the matrices of a batch that
   * missed the target, spral_ssids_gpu_group_bwd_errors); 0: the default
   * FP64 fallback */
  int no_fp64_fallback;
  int reserved[7];
};

/* Replaces construct_gpu_symbolic_subtree (src/ssids/gpu/subtree.f90:76);
 * signature of spral_ssids_cpu_create_symbolic_subtree
 * (src/ssids/cpu/SymbolicSubtree.cxx:14) with the CUDA device first and
 * without the inter-subtree contribution list (the whole tree is one GPU
 * subtree).  Nodes sa..en-1 (1-based) are the subtree. Returns NULL on error. */
void* spral_ssids_gpu_create_symbolic_subtree(
    int device, int n, int sa, int en, const int* sptr, const int* sparent,
    const int64_t* rptr, const int* rlist, const int64_t* nptr, const int64_t* nlist,
    const struct spral_ssids_cpu_factor_options* options);

/* Replaces gpu_symbolic_subtree%cleanup (src/ssids/gpu/subtree.f90:283). */
void spral_ssids_gpu_destroy_symbolic_subtree(void* symbolic);

/* Out-of-band options; call before create_num_subtree.  Returns 0. */
int spral_ssids_gpu_set_options(void* symbolic, const struct spral_ssids_gpu_options* opts);

/* Replaces gpu_symbolic_subtree%factor (src/ssids/gpu/subtree.f90:304);
 * signature of spral_ssids_cpu_create_num_subtree_dbl
 * (src/ssids/cpu/NumericSubtree.cxx:30).  aval: host values in the user's
 * lower-CSC order; scaling: NULL or n scaling factors in pivot order;
 * child_contrib must be NULL.  Returns the numeric handle (also on failure,
 * with stats->flag < 0) or NULL if nothing could be allocated. */
void* spral_ssids_gpu_create_num_subtree_dbl(
    bool posdef, const void* symbolic, const double* aval, const double* scaling,
    void** child_contrib, const struct spral_ssids_cpu_factor_options* options,
    struct spral_ssids_thread_stats* stats);

/* Replaces gpu_numeric_subtree%cleanup (src/ssids/gpu/subtree.f90:484);
 * cf. spral_ssids_cpu_destroy_num_subtree_dbl (NumericSubtree.cxx:63). */
void spral_ssids_gpu_destroy_num_subtree_dbl(bool posdef, void* numeric);

/* Replace gpu_numeric_subtree%solve_fwd/_diag/_diag_bwd/_bwd
 * (src/ssids/gpu/subtree.f90:555-738); cf. spral_ssids_cpu_subtree_solve_*
 * (NumericSubtree.cxx:76-180).  x: host, pivot order, ldx >= n.  Return an
 * SSIDS flag (0 success, -50 allocation, -51 CUDA error). */
int spral_ssids_gpu_subtree_solve_fwd_dbl(bool posdef, const void* numeric, int nrhs, double* x,
                                          int ldx);
int spral_ssids_gpu_subtree_solve_diag_dbl(bool posdef, const void* numeric, int nrhs, double* x,
                                           int ldx);
int spral_ssids_gpu_subtree_solve_diag_bwd_dbl(bool posdef, const void* numeric, int nrhs,
                                               double* x, int ldx);
int spral_ssids_gpu_subtree_solve_bwd_dbl(bool posdef, const void* numeric, int nrhs, double* x,
                                          int ldx);

/* Replaces gpu_numeric_subtree%enquire_indef (src/ssids/gpu/subtree.f90:855);
 * cf. spral_ssids_cpu_subtree_enquire_dbl (NumericSubtree.cxx:183).
 * piv_order[var] (0-based, negative for 2x2) and d (2 x n), either may be NULL. */
void spral_ssids_gpu_subtree_enquire_dbl(bool posdef, const void* numeric, int* piv_order,
                                         double* d);

/* Replaces gpu_numeric_subtree%alter (src/ssids/gpu/subtree.f90:933);
 * cf. spral_ssids_cpu_subtree_alter_dbl (NumericSubtree.cxx:204). */
void spral_ssids_gpu_subtree_alter_dbl(bool posdef, void* numeric, const double* d);

/* Replaces gpu_numeric_subtree%get_contrib (src/ssids/gpu/subtree.f90:522)
 * with the copy of transfer_contrib (src/ssids/gpu/factor.f90:155-221);
 * arguments of spral_ssids_cpu_subtree_get_contrib_dbl
 * (src/ssids/cpu/NumericSubtree.cxx:218).  For a subtree whose root has a
 * parent in another subtree: the root's contribution block (n x n, full
 * symmetric, ldval = n), its 1-based rows (rlist), and the root's delayed
 * columns (delay_perm: 1-based variables; delay_val: each column from its
 * diagonal down, the ndelay x ndelay block then the n contribution rows,
 * leading dimension lddelay = n + ndelay).  Pointers are NULL when empty and
 * stay valid until free_contrib or the handle's destruction; FP32 factors
 * are widened to FP64.  Returns 0 or -51 (a CUDA error; the reference's
 * function returns nothing, so a Fortran subroutine binding may ignore it). */
int spral_ssids_gpu_subtree_get_contrib_dbl(bool posdef, void* numeric, int* n,
                                            const double** val, int* ldval, const int** rlist,
                                            int* ndelay, const int** delay_perm,
                                            const double** delay_val, int* lddelay);

/* Replaces gpu_free_contrib (src/ssids/gpu/subtree.f90:540); cf.
 * spral_ssids_cpu_subtree_free_contrib_dbl (NumericSubtree.cxx:248). */
void spral_ssids_gpu_subtree_free_contrib_dbl(bool posdef, void* numeric);

/* Same-pattern refactorisation with values already in device memory (no
 * reference counterpart: the reference re-creates the numeric subtree and
 * copies aval host-to-device each time, src/ssids/gpu/subtree.f90:375). */
int spral_ssids_gpu_refactor_dev(void* numeric, const double* aval_dev,
                                 struct spral_ssids_thread_stats* stats, void* stream);

/* Same-pattern refactorisation with host values (and optional host
 * scaling): the numeric subtree constructor's inputs, reusing the handle,
 * its device memory and, when no pivot was delayed last time, its captured
 * factorisation graph.  Returns the SSIDS flag. */
int spral_ssids_gpu_refactor(void* numeric, const double* aval, const double* scaling,
                             struct spral_ssids_thread_stats* stats);

/* Solve with x in device memory (pivot order, FP64).  job: 0 full,
 * 1 fwd, 2 diag, 3 bwd, 4 diag_bwd (ssids_solve job codes,
 * src/ssids/ssids.f90:1232-1246). */
int spral_ssids_gpu_solve_dev(void* numeric, int job, int nrhs, double* x_dev, int ldx,
                              void* stream);

/* Full solve with FP64 iterative refinement against the FP64 matrix held on
 * the device (pivot order x, host).  Used by precision = 1; for FP64
 * factors it performs max_refine steps of classical refinement.  iters
 * receives the number of refinement steps taken. */
int spral_ssids_gpu_solve_refined(void* numeric, int nrhs, double* x, int ldx, int* iters);

/* Timings of the last factor (ms): [0] total, [1] assembly, [2] dense,
 * [3] contribution GEMM, [4] host wait.  Returns number of entries. */
int spral_ssids_gpu_last_timing(const void* numeric, double* out);

/* Diagnostics (no reference counterpart): copy one front of the factors to
 * the host.  info[0..4] = m, n, nelim, ndelay_in, ld; L is m x n
 * (ld = m, FP64), D is 2 x n, perm n 0-based pivot positions (any may be
 * NULL).  node is 0-based. */
int spral_ssids_gpu_debug_front(const void* numeric, int node, int* info, double* L, double* D,
                                int* perm);

/* Full solve plus FP64 refinement with b and x in device memory (n x nrhs,
 * leading dimension ld, pivot order).  iters / bwd_err receive the largest
 * refinement count and the final scaled backward error. */
int spral_ssids_gpu_solve_refined_dev(void* numeric, int nrhs, const double* b_dev, double* x_dev,
                                      int ld, int* iters, double* bwd_err);

/* No counterpart in the reference.  Number of FP64 refactorisations taken by
 * the refined solves of an FP32-factor handle (precision = 1) since it was
 * created: when the FP32 factors cannot bring a refined solve to the
 * backward-error target (refinement stalls or runs out of steps), the same
 * values are factored in FP64 on the GPU, once per factorisation, and the
 * solve is finished with those factors.  stats (may be NULL) receives the
 * handle's current statistics, which are the FP64 factorisation's after a
 * fallback.  Returns -1 for a NULL handle. */
int spral_ssids_gpu_fp64_fallbacks(const void* numeric, struct spral_ssids_thread_stats* stats);

/* No counterpart in the reference.  Row groups for the refined solves of
 * every numeric handle of this symbolic subtree: row_group[i] (pivot order,
 * n entries) in [0, ngroups) names the group of row i, e.g. the matrix of a
 * batch of independent matrices stacked into one subtree.  The scaled
 * backward error that stops the refinement is then the largest over the
 * groups, each with its own norms (||A_g||, ||x_g||, ||b_g||), so every
 * group meets the target.  When the groups are whole trees of the assembly
 * forest (every front's columns and its parent's in one group, as for
 * stacked independent matrices), each refinement step of an FP64 handle,
 * or of an FP32 handle with no_fp64_fallback, solves only for the groups
 * still above the target.  ngroups <= 0 or row_group == NULL removes the
 * groups.  Returns 0, -1 (NULL handle), -2 (a group out of range) or -51. */
int spral_ssids_gpu_set_row_groups(void* symbolic, int ngroups, const int* row_group);

/* Benchmark support (no reference counterpart): kernels launched by this
 * library so far; per-factor timing of the contribution-block update with
 * CUDA events on the library's stream (out[0] ms, out[1] algorithmic flops,
 * out[2] timed levels; out[3..5] the same for the tensor-core GEMM kernel
 * alone, flops counted as the FP32 update); measured FP64 FMA throughput of
 * the device. */
long long spral_ssids_gpu_launch_count(void);
void spral_ssids_gpu_set_profiling(void* numeric, int on);
void spral_ssids_gpu_profile_stats(const void* numeric, double* out);
double spral_ssids_gpu_fp64_peak_tflops(int device);
void spral_ssids_gpu_phase_times(const void* numeric, double* ms, long long* counts);
/* Evaluates the device reciprocal used on the pivot-decision path for n
 * values (device pointers), for accuracy tests against IEEE division. */
int spral_ssids_gpu_recip_probe(const double* x_dev, double* y_dev, int n);

/* Dense LDL^T with a-posteriori threshold pivoting of one front, all
 * pointers in device memory: the per-front kernel of the factorization as a
 * stand-alone call.  Counterpart of ldlt_app_factor
 * (src/ssids/cpu/kernels/ldlt_app.cxx:2506) followed by the TPP finish of
 * factor_node_indef (src/ssids/cpu/factor.hxx:38-110); on the GPU path,
 * node_ldlt (src/ssids/gpu/dense_factor.f90:28).
 *   a (m x n, lda >= m): lower part of the n fully-summed columns and the
 *     rows below; on exit L (unit diagonal) of the nelim eliminated columns
 *     followed by the failed (delayed) columns, updated;
 *   d (2n): D^{-1} in the reference format; perm (n): labels, permuted;
 *   upd ((m-n) x (m-n), ldupd >= m-n) or NULL: upd = beta*upd - L21 D L21^T
 *     (beta 0 or 1), e.g. the trailing block of a with ldupd = lda.
 * Returns nelim, or a negative SSIDS flag (-5 singular with action false,
 * -50 allocation, -51 CUDA).  Allocates its workspace with cudaMalloc and
 * synchronises the stream before returning. */
int spral_ssids_gpu_ldlt_app_factor(int m, int n, int* perm_dev, double* a_dev, int lda,
                                    double* d_dev, double beta, double* upd_dev, int ldupd,
                                    const struct spral_ssids_cpu_factor_options* options,
                                    void* stream);

/* No counterpart in the reference.  The same factorization as
 * spral_ssids_gpu_ldlt_app_factor for callers that must not allocate device
 * memory at factorization time (memory owned by another allocator, a budget
 * fixed at load time, or a latency-critical path where cudaMalloc/cudaFree
 * can stall the device): the workspace is a fixed 3 MiB device array inside
 * the library, present on every GPU that loads it until the process exits.
 * lda <= 1024 (so m <= 1024); larger fronts return
 * SPRAL_SSIDS_GPU_NOALLOC_TOO_LARGE (n = 0 returns 0 whatever lda is, as
 * the allocating call does).  The first call on a device looks up the
 * array's device address and keeps it; a process that resets the device
 * (cudaDeviceReset) must not call this entry point on it again.  Like the
 * allocating call, it synchronises its stream before returning.
 * All calls share the array: calls that overlap on the GPU race and must be
 * serialised by the caller.  Calls no cudaMalloc, cudaFree or allocating
 * library routine. */
#define SPRAL_SSIDS_GPU_NOALLOC_TOO_LARGE (-60)
int spral_ssids_gpu_ldlt_app_factor_noalloc(int m, int n, int* perm_dev, double* a_dev, int lda,
                                            double* d_dev, double beta, double* upd_dev,
                                            int ldupd,
                                            const struct spral_ssids_cpu_factor_options* options,
                                            void* stream);

/* Tensor-core Schur update used by the mixed-precision path, exposed for
 * tests and measurements: C (M x N, column-major, ldc) -= A B^T with A
 * (M x K) and B (N x K) column-major FP32 device arrays; 3xTF32 split
 * products on tcgen05, accumulated in TMEM for at most `chunk` 32-deep
 * k-tiles (chunk = 0: the whole depth; chunk < 0: the library default) and
 * then in FP32 registers; lower != 0 updates only r >= c.  With reps > 0 and
 * ms != NULL the update runs reps times and ms[0], ms[1] receive the mean
 * split-kernel and GEMM-kernel times in ms.  Returns 0, -1 bad argument,
 * -50 allocation, -51 CUDA error, -52 pipeline timeout.  No reference
 * counterpart (the reference's contribution update is FP64 SIMT,
 * src/ssids/gpu/kernels/syrk.cu:185). */
int spral_ssids_gpu_tc_gemm_f32(int M, int N, int K, const float* A, int lda, const float* B,
                                int ldb, float* C, int ldc, int lower, int chunk, int reps,
                                float* ms);

/* The same with an explicit tile width bn (64, 128 or 256; 0: the
 * autotuned width).  Returns -4 for another width. */
int spral_ssids_gpu_tc_gemm_f32_bn(int M, int N, int K, const float* A, int lda, const float* B,
                                   int ldb, float* C, int ldc, int lower, int chunk, int reps,
                                   float* ms, int bn);

/* Per-node inertia of the last factorisation: out[3*node + {0, 1, 2}] =
 * (negative eigenvalues, 2x2 pivots, zero pivots) of each node's D, nodes
 * numbered 0-based as in the symbolic subtree.  Batched factorisations of
 * many independent matrices (one forest) sum these per matrix.  No
 * reference counterpart (the reference reports whole-subtree totals,
 * src/ssids/cpu/NumericSubtree.hxx:249-280).  Returns 0 or -51. */
int spral_ssids_gpu_node_inertia(const void* numeric, int* out);

/* Contribution-block size (rows) from which the FP32-factor path forms the
 * update on the tensor cores instead of the SIMT kernel: measured once per
 * device by timing both on synthetic fronts (the environment variable
 * SPRAL_GB300_TC_MIN_CM overrides it).  No reference counterpart.  Returns
 * the size, or -51 on a CUDA error. */
int spral_ssids_gpu_tc_crossover(void);

/* The autotuner's table for the current device: the crossover above and,
 * per size class of a launch (its largest contribution block, m rows or
 * fewer), the fastest tile width of the tensor-core update (128 x 64,
 * 128 x 128 or 128 x 256), all measured once per device, or read from the
 * tune cache file named by the environment variable SPRAL_GB300_TUNE_CACHE
 * when it holds a line for this device (and written there after a
 * measurement).  out = [tc_min_cm, nb, m_0, bn_0, ..., m_{nb-1}, bn_{nb-1}].
 * Returns the number of ints written, -1 if nout is too small, -51 on a
 * CUDA error.  No reference counterpart (the reference's kernel shapes are
 * fixed at compile time). */
int spral_ssids_gpu_tune_table(int* out, int nout);

/* The scaled backward error of each row group (spral_ssids_gpu_set_row_groups:
 * e.g. the matrices of a batch) after the last refined solve of the handle,
 * the largest over the right-hand sides of its last chunk of 16.  out holds
 * ngroups values.  Returns 0, -1 without row groups or refined solve, -51 on
 * a CUDA error.  No reference counterpart. */
int spral_ssids_gpu_group_bwd_errors(const void* numeric, double* out, int ngroups);

/* The current device's key in the tune cache (device name with '_' for
 * spaces, "-sm<multiprocessors>-cc<major><minor>").  Returns its length, or
 * -1 (no device, or cap too small). */
int spral_ssids_gpu_tune_device_key(char* buf, int cap);

/* Tune-cache helpers (host only, no GPU needed).  A cache line reads
 *   spral_gb300-tune v1 <key> tc_min_cm=<int> bn=<m>:<bn>,<m>:<bn>,...
 * with strictly increasing m and bn in {64, 128, 256}; tables are passed as
 * the ints of spral_ssids_gpu_tune_table.
 * _parse: parses one line into key (key_cap bytes) and out; returns the
 *   number of ints, or -1 for a malformed line or too little room.
 * _format: writes the line of (key, table) into buf; returns its length or -1.
 * _cache_lookup: the last line for key in the file at path; returns the
 *   number of ints, 0 if the file or the key is absent, -1 if out is too small.
 * _cache_store: replaces (or adds) the line for key, keeping the others;
 *   the file is replaced by a rename.  Returns 0 or -1. */
int spral_ssids_gpu_tune_parse(const char* line, char* key, int key_cap, int* out, int nout);
int spral_ssids_gpu_tune_format(const char* key, const int* in, int nin, char* buf, int cap);
int spral_ssids_gpu_tune_cache_lookup(const char* path, const char* key, int* out, int nout);
int spral_ssids_gpu_tune_cache_store(const char* path, const char* key, const int* in, int nin);

/* Level schedule of the numeric factorisation (host only, no GPU needed),
 * as spral_ssids_gpu_create_symbolic_subtree builds it.  parent[i] is node
 * i's parent (0-based, > i; -1 for a root), ncol[i] its fully-summed
 * columns, small[i] != 0 marks the nodes of small leaf subtrees (NULL: none).
 * align: 0 root-aligned when it takes at least 10% fewer APP block steps
 * (sum over levels of the widest front's ceil(ncol/32)) than leaf-aligned,
 * else leaf-aligned; 1 leaf-aligned (height above the leaves),
 * 2 root-aligned (depth below the root, as the reference's
 * assign_nodes_to_levels, src/ssids/gpu/factor.f90:824, with the small
 * subtrees kept leaf-aligned).  Writes level[i] and *nlev; *steps (if not
 * NULL) the schedule's APP block steps.  Returns 1 when root-aligned, 0 when
 * leaf-aligned, -1 on a bad argument. */
int spral_ssids_gpu_level_schedule(int nnodes, const int* parent, const int* ncol,
                                   const char* small, int align, int* level, int* nlev,
                                   int64_t* steps);

/* The contribution update of one front, C -= L21 (L21 D)^T on the lower
 * triangle of the cm x cm block C, on the SIMT kernel of the numeric
 * factorisation, applied reps times on the caller's device buffers and
 * stream (L: the front's (cm + k) x k columns, leading dimension ld >=
 * cm + k; LD = L21 D: cm x k, leading dimension cm; C: a full cm x cm
 * array, whose upper part may be read but is never written; FP64 when
 * dbl != 0, else FP32).  Serves timing the kernel alone.  No
 * reference counterpart (the reference forms this block inside its
 * factorisation: form_contrib, src/ssids/gpu/factor.f90:945, with the
 * kernel cu_multisyrk_lc_r4x4, src/ssids/gpu/kernels/syrk.cu:185).
 * Returns 0, -1 on a bad argument or -51 on a CUDA error. */
int spral_ssids_gpu_contrib_update(int dbl, const void* l, int ld, const void* l21d, void* c,
                                   int cm, int k, int reps, void* stream);

/* Free and total memory of the current device (cudaMemGetInfo), for
 * callers that admit work by device memory; free includes the blocks this
 * library keeps cached for reuse by numeric handles.  No reference
 * counterpart.  Returns 0 or -51. */
int spral_ssids_gpu_mem_info(size_t* free_bytes, size_t* total_bytes);

/* No counterpart in the reference.  Returns the device blocks that numeric
 * handles of this process gave back (kept for reuse by later handles, up to
 * a quarter of the device's memory) to the driver, for the current device. */
void spral_ssids_gpu_release_cache(void);

/* Failure detection (testing aids, no reference counterpart).  Every wait
 * of this library's kernels on another CTA or on an mbarrier is bounded:
 * when it gives up, the kernel records an error status and returns, and the
 * host reports SSIDS_ERROR_CUDA_UNKNOWN (-51) with the context still usable
 * (the reference's inter-CTA spins, src/ssids/gpu/kernels/assemble.cu:208-211,
 * are unbounded).  These probes run one such wait on a barrier or flag that
 * nothing completes, bounded to `rounds` polls, and return -51 when it gave
 * up (0 otherwise); the first is the tensor-core pipeline's mbarrier wait,
 * the second the wavefront solves' flag wait. */
int spral_ssids_gpu_mbar_timeout_probe(int rounds);
int spral_ssids_gpu_wave_timeout_probe(int rounds);
/* Testing aid: after `after` further successful device-block allocations
 * of numeric handles, the next one fails as an out-of-memory cudaMalloc
 * does (the factorization then reports SSIDS_ERROR_ALLOCATION, -50); a
 * negative value switches the injection off. */
void spral_ssids_gpu_inject_alloc_failure(int after);

/* Number of CUDA devices visible (hw_topology/guess_topology.cxx:65). */
int spral_ssids_gpu_device_count(void);

#ifdef __cplusplus
}
#endif

#endif /* SPRAL_SSIDS_GPU_H */
