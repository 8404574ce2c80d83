// Shared declarations of the GB300 numeric factor/solve for SSIDS.
//
// Layout in HBM (one numeric subtree = the whole assembly tree):
//   * front f: L is m x n column-major, leading dimension ld >= m (m, n
//     include delayed columns from children; delays follow the node's own
//     columns, as in src/ssids/cpu/kernels/assemble.hxx:227-263).  L holds the
//     true factor (unit diagonal, scaled by D^{-1}) for eliminated columns.
//   * D^{-1} per front: 2 x n doubles in the reference CPU format
//     (src/ssids/cpu/kernels/ldlt_app.cxx:338-343): 1x1 -> (d11, 0); 2x2 ->
//     (d11, d21), (+Inf, d22).  Always FP64, whatever the factor type.
//   * perm per front: n ints, 0-based pivot positions (rlist order).
//   * contribution block per front: cm x cm (cm = nrow - ncol), lower part.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace ssids300 {

constexpr int kBlk = 32;         // APP inner block (ldlt_app.cxx:41 INNER_BLOCK_SIZE)
constexpr int kApplyRows = 64;   // rows per apply/fixup CTA
constexpr int kGemmTile = 64;    // SIMT GEMM tile

// Programmatic dependent launch (PDL).  The serial chains of the path (the
// APP block steps of a level, the block steps of the solves) are strings of
// small dependent kernels; launched with launch_pdl, a kernel is scheduled
// while its predecessor in the stream is still running and blocks in
// pdl_wait() until that predecessor has completed and its memory is
// visible, which hides the launch latency of every link (also inside a
// captured graph, where the launches become programmatic edges).  Rules for
// a kernel launched this way: before pdl_wait() it may read only what the
// host wrote before the launch (front/solve descriptors, level lists) and
// writes nothing; pdl_trigger() after the wait lets the next kernel of the
// chain be scheduled.  Both are no-ops for an ordinary launch.
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;\n" ::: "memory"); }
__device__ __forceinline__ void pdl_trigger() {
  asm volatile("griddepcontrol.launch_dependents;\n" ::: "memory");
}
template <typename... KArgs, typename... Args>
inline void launch_pdl(void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem,
                       cudaStream_t s, Args... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  cudaLaunchKernelEx(&cfg, kernel, static_cast<KArgs>(args)...);
}

// Error codes written to the device status word (host maps to SSIDS flags).
enum DevStatus : int {
  kDevOk = 0,
  kDevSingular = 1,   // zero pivot with action == false  -> SSIDS_ERROR_SINGULAR
  kDevBadState = 2,   // internal consistency check failed -> SSIDS_ERROR_CUDA_UNKNOWN
  kDevNotPosdef = 3,  // posdef factorisation met a pivot that is not > 0 -> SSIDS_ERROR_NOT_POS_DEF
};

template <typename T>
struct FrontDesc {
  T* L;          // m x n, ld
  double* D;     // 2 x n
  int* perm;     // n
  int* opos;     // n: original (assembly-time) position of each final position
  T* C;          // cm x cm contribution block (nullptr if cm == 0)
  T* W;          // per-level workspace, >= ld x 32
  double* step;  // per-front step buffer: L11 (32x32) + D (64) doubles
  int* lperm;    // per-front step buffer: 32 ints (local block permutation)
  T* swapbuf;    // per-level workspace for column moves: 64 x ld
  T* LD;         // per-level workspace for L*D of the contribution rows (cm x n)
  int m, n, ld;  // rows, fully-summed columns (incl. delays), leading dim
  int nrow, ncol, ndelay_in, cm;
  int node;
  int ldc;       // leading dimension of C (cm for the tree's own blocks)
  int tc;        // contribution block formed by the tensor-core GEMM
  int panel;     // > 0: APP in panels of this many candidate columns (see below)
};

// Panels (FP32 factors, fronts wider than FrontDesc::panel): the APP block
// steps draw their candidates from a panel of `panel` columns [pstart, qend)
// and update only the panel's columns; at the panel's end the trailing
// fully-summed columns [qend, n) take the panel's pk pivots in one
// tensor-core update, and the panel's failed columns move to the end of the
// front's candidate range [.., gend).  Other fronts have one panel with
// qend = gend = n.
struct FrontState {
  int p;          // number eliminated so far (APP)
  int end;        // end of the APP candidate range (of the current panel)
  int bs;         // current block width (0 = done)
  int npass_raw;  // first failing column from the threshold test
  int npass;      // adjusted (2x2 not split)
  int nelim;      // final
  int status;     // DevStatus
  int step;       // step counter (sanity)
  int pstart;     // first position of the current panel
  int qend;       // end of the current panel's columns (bound of its updates)
  int gend;       // end of the front's candidate range
  int pk;         // pivots of the last closed panel
};

struct Stats {  // device-side reduction target (integers only -> deterministic)
  int num_neg, num_two, num_zero, num_delay;
  long long num_factor, num_flops;
};

// Count of kernels launched by this library (reported by the benchmark).
void note_launches(int k);

// Optional per-phase device timing: a CUDA event is recorded before each
// kernel of interest (and at the end); the time between consecutive events
// is attributed to the phase of the earlier one.  Only used when profiling.
enum Phase : int {
  kPhZero = 0, kPhLoadA, kPhInitPerm, kPhDelays, kPhAssemble, kPhDiag, kPhRowPerm, kPhApply,
  kPhFixup, kPhPanel, kPhSwap, kPhFinish, kPhTpp, kPhCalcLd, kPhContrib, kPhStats, kPhHost,
  kPhFwdGather = 20, kPhFwdDiag, kPhFwdUpdate, kPhFwdScatter, kPhBwdGather, kPhBwdL21,
  kPhBwdDiag, kPhBwdUpdate, kPhBwdScatter, kPhResid, kPhAxpy, kPhCount = 32
};
struct PhaseTimer {
  cudaEvent_t* ev = nullptr;
  int* ph = nullptr;
  int cap = 0, used = 0;
  double ms[kPhCount] = {0};
  long long cnt[kPhCount] = {0};
  void mark(int phase, cudaStream_t s);
  void flush();  // after a stream synchronisation
  void reset();
  ~PhaseTimer();
};
inline void pmark(PhaseTimer* t, int phase, cudaStream_t s) {
  if (t) t->mark(phase, s);
}

// ---------------- launchers (defined in the kernel .cu files) --------------
// assembly (assemble_kernels.cu)
template <typename T>
void launch_load_a(const FrontDesc<T>* fd, const int* fronts, int nf, const int64_t* nptr,
                   const int64_t* nlist, const double* aval, const int* rlist,
                   const int64_t* rptr, const double* scaling, int max_entries, cudaStream_t s);
template <typename T>
void launch_init_perm(const FrontDesc<T>* fd, const int* fronts, int nf, const int* sptr,
                      int max_n, cudaStream_t s);
// max_nd bounds the delayed columns of any child in the work list
template <typename T>
void launch_assemble_delays(const FrontDesc<T>* fd, const FrontState* st, const int4* work,
                            int nwork, int max_nd, const int* rdir, const int64_t* rdir_ptr,
                            cudaStream_t s);
// max_rows: the longest contribution-block column (parent or child) of the
// level: short columns take a warp each, long ones a CTA
template <typename T>
void launch_assemble_contrib(const FrontDesc<T>* fd, const int4* cols, int ncols,
                             const int2* pairs, const int* rdir, const int64_t* rdir_ptr,
                             int max_rows, cudaStream_t s);
template <typename T>
void launch_app_step(FrontDesc<T>* fd, FrontState* st, const int* fronts, int nf, int step,
                     int max_rows, int max_trail_rows, int max_trail_cols, bool action,
                     double u, double small, cudaStream_t s, PhaseTimer* tm, bool posdef = false);
template <typename T>
void launch_app_finish(FrontDesc<T>* fd, FrontState* st, const int* fronts, int nf,
                       cudaStream_t s);
// End of a panel for the listed fronts: fold the last block step and form
// LD = L D for the trailing rows [qend, n) of the panel's pivots into fd.LD
// (column k at fd.LD + k * n); max_n bounds n over the listed fronts.
template <typename T>
void launch_panel_end(FrontDesc<T>* fd, FrontState* st, const int* fronts, int nf, int max_n,
                      int panel, cudaStream_t s);
// After the panel's trailing update: move its failed columns to the end of
// the candidate range and open the next panel.
template <typename T>
void launch_panel_close(FrontDesc<T>* fd, FrontState* st, const int* fronts, int nf,
                        cudaStream_t s);
template <typename T>
void launch_tpp(FrontDesc<T>* fd, FrontState* st, const int* fronts, int nf, bool action,
                double u, double small, bool root_only_or_all, cudaStream_t s);
// fronts of small leaf subtrees, one persistent launch: TPP from the first
// column, then each front's contribution block (LD and C -= L21 LD^T);
// max_bytes is the dynamic shared memory of the launch (fronts whose
// staging, ((m + 1) & ~1) * (n + 2) * sizeof(T) + 8 n bytes, exceeds it
// are factored in place); threads: 32 (one warp per front) or 256
template <typename T>
void launch_tpp_level(FrontDesc<T>* fd, FrontState* st, const int* fronts, int nf, bool action,
                      double u, double small, int max_bytes, int threads, cudaStream_t s);
template <typename T>
void launch_calc_ld(FrontDesc<T>* fd, FrontState* st, const int* fronts, int nf, int max_cm,
                    int max_n, cudaStream_t s);
template <typename T>
void launch_contrib_gemm(FrontDesc<T>* fd, FrontState* st, const int* fronts, int nf, int max_cm,
                         cudaStream_t s);
template <typename T>
void launch_stats(const FrontDesc<T>* fd, const FrontState* st, const int* fronts, int nf,
                  int max_n, Stats* stats, int* node_counts, cudaStream_t s);

// ---------------- tensor-core Schur update (tc_gemm.cu) ----------------
// C_i -= A_i B_i^T (lower if requested) with 3xTF32 split products on
// tcgen05.  A_i: M_i x kmax column-major (lda), B_i: N_i x kmax (ldb); the
// effective depth may be read from device memory (kval_dev).
struct TcProblem {
  const float* A;
  int lda;
  const float* B;
  int ldb;
  float* C;
  int ldc, M, N, kmax;
  const int* kval_dev;
  int lower;
};
struct TcBuffers {  // reusable descriptor staging of tc_gemm_run
  void* h_stage = nullptr;  // pinned host copy of the descriptors
  void* d_stage = nullptr;  // device copy
  size_t cap = 0;
  cudaEvent_t uploaded = nullptr;  // the last upload from h_stage has completed
  ~TcBuffers();
};
}  // namespace ssids300
#include <vector>
namespace ssids300 {
// Default number of 32-deep k-tiles (96 split products each) accumulated in
// TMEM before the partial sum is added (round-to-nearest) into the register
// accumulator.
constexpr int kTcChunk = 3;
size_t tc_gemm_scratch_bytes(const std::vector<TcProblem>& ps);
// Descriptor tables of one tc_gemm launch pair (split + GEMM), built on the
// host; tc_gemm_launch only enqueues kernels, so it can be graph-captured
// once the blob is in device memory.
struct TcPlan {
  std::vector<char> blob;
  size_t o_jobs = 0, o_tiles = 0, o_maps = 0;
  int nsplit = 0, ntiles = 0, maxr = 0, maxk = 0, grid = 0;
  int bn = 256;  // tile width (N) of the GEMM kernel
};
// Tile widths of k_tc_gemm (128 x bn tiles): 64, 128 or 256.
bool tc_tile_width_ok(int bn);
// The autotuned tile width for a launch over ps on the current device
// (256 before the device has been tuned; SPRAL_GB300_TC_BN overrides it).
int tc_tile_width(const std::vector<TcProblem>& ps);
// bn = 0: the autotuned width; returns -4 for a width the kernel lacks.
int tc_gemm_prepare(const std::vector<TcProblem>& ps, void* scratch, TcPlan& plan, int bn = 0);
int tc_gemm_launch(const TcPlan& plan, const void* d_blob, int* status, cudaStream_t s,
                   int chunk);
// Returns 0, or a negative code: -1 allocation, -2 tensor-map encoding,
// -3 launch error, -4 unknown tile width.  Device-side pipeline timeouts are
// reported in *status.
int tc_gemm_run(const std::vector<TcProblem>& ps, void* scratch, TcBuffers& buf, int* status,
                cudaStream_t s, int chunk = kTcChunk, float* ms_split = nullptr,
                float* ms_gemm = nullptr, int bn = 0);

// syrk-like lower update C(r,c) -= sum_k A(r,k) B(c,k), r >= c
template <typename T>
struct SyrkJob {
  T* C;
  const T* A;
  const T* B;
  int ldc, lda, ldb;
  int M, N, K;
};

// ---------------- solve (solve_kernels.cu) ----------------
// Per node data for the level-set solves.  x is n x nrhs (ld = ldx) in pivot
// order, FP64.  xloc holds the node's local vector (m x nrhs, ld = m) and is
// kept for the whole forward pass: its rows [nelim, m) are the node's
// contribution to its parent.
template <typename T>
struct SolveNode {
  const T* L;
  const double* D;
  const int* perm;   // n: pivot position of each final front position
  const int* opos;   // n: original position of each final front position
  const int* rows;   // rlist of the node (0-based pivot positions), nrow entries
  const int* rdir;   // cm entries: parent position of each contribution row
  T* xloc;           // m x nrhs, in the factor precision
  const int* gp;     // nrow + 1: children's contribution pairs of each parent position
  int m, n, ld, nelim, ncol, nrow, ndelay_in, cm;
  int sptr0;         // first own pivot
  int child_beg, child_end;  // into the child arrays
  int doff;          // offset of this node's delays inside its parent's delay block
  // wavefront solves: flag[0, nblk) completion flags of the pivot blocks,
  // flag[nblk, 2 nblk) finished L21^T partial items of each pivot block,
  // flag[2 nblk] gathered row chunks, flag[2 nblk + 1] finished items of
  // the pass
  int* flag;
  T* l21p;           // backward L21^T partial sums: [nblk][nch][64][kSolveRhs]
  // inverses of the 64 x 64 unit lower diagonal blocks, [nblk][64][64]
  // row-major (FP32 factors' wavefront passes), or nullptr
  const T* binv;
  int nblk;          // ceil(nelim / 64) pivot blocks
  int ngat;          // gather items (0: the front is one small item)
  int nch;           // L21^T partial items per pivot block (0: none)
  int nitf, nitb;    // items of the forward and of the backward pass
  int parent;        // front index of the parent, -1 at a root
};

// Wavefront solves: one persistent launch per pass over the whole tree.
// The work items, items[i] = (front, code), are taken in list order from an
// atomic counter; an item waits (bounded) only for items earlier in the
// list, so every awaited item is held by a running CTA.  Codes:
//   [0, 0x10000)        pivot block b (rows [64 b, 64 b + 64) of the
//                       eliminated part);
//   [0x10000, 0x20000)  forward only: contribution row block k (rows
//                       nelim + 64 k ...);
//   [0x20000, 0x30000)  gather chunk c: rows [256 c, 256 c + 256) of the
//                       front's local vector;
//   0x30000             a small front whole (gather, its one pivot block
//                       and, forward, its contribution rows) in one item;
//   >= 0x100000         backward only: L21^T partial item t = b nch + c,
//                       the product over contribution rows
//                       [nelim + 256 c, nelim + 256 c + 256) for pivot
//                       block b.
// Forward list: levels from the leaves; per level the gathers (and small
// fronts), then the pivot blocks in increasing block order, then the
// contribution row blocks.  A gather waits until every child has finished
// all its items; pivot and contribution blocks wait for their front's
// gathers and for the pivot blocks before them.  Backward list: levels from
// the root; per level the gathers, then the pivot blocks in decreasing
// order, each after its block's L21^T partial items (which wait for their
// front's gathers); a gather waits until the parent has finished.  A wait
// that gives up sets *status.
constexpr int kWaveContrib = 0x10000;
constexpr int kWaveGather = 0x20000;
constexpr int kWaveSmall = 0x30000;
constexpr int kWaveL21 = 0x100000;
constexpr int kWaveGatherRows = 256;
constexpr int kWaveL21Rows = 256;
// a front is one small item when it has at most one pivot block and at most
// this many rows below its pivots
constexpr int kWaveSmallRows = 256;
struct WaveLevel {
  const int2* items;
  int nitems;
  int* counter;  // zeroed before the launch
  // optional trace (nullptr: off): per item, the global timer when a CTA
  // took it, when its last wait was over, when it finished, and the SM
  unsigned long long* trace;
  int ctas_per_sm;  // persistent CTAs per SM: 3 when small fronts dominate, else 2
  // optional mask (nullptr: every front): the items of front f run only when
  // active[front_group[f]] != 0; a group is one matrix of a batch stacked as
  // a forest, so the skipped fronts are whole trees that no other item waits
  // for
  const int* front_group;
  const unsigned char* active;
};

constexpr int kSolveBlk = 64;   // diagonal block of the blocked triangular solves
constexpr int kSolveRhs = 16;   // right-hand sides per pass
// doubles per row group in the refinement's residual workspace: ||A||, then
// (||x||, ||b||, ||r||) per right-hand side of a pass
constexpr int kResStride = 1 + 3 * kSolveRhs;

template <typename T>
void launch_fwd_gather(const SolveNode<T>* sn, const int* nodes, int nn, const int* children,
                       const int2* pairs, const double* x, int ldx, int nrhs, int max_m,
                       cudaStream_t s);
template <typename T>
void launch_fwd_steps(const SolveNode<T>* sn, const int* nodes, int nn, int max_nelim,
                      int max_m, int nrhs, double* x, int ldx, bool scale_sqrt, cudaStream_t s,
                      PhaseTimer* tm);
// one forward pass over the whole tree (gathers included)
template <typename T>
void launch_fwd_tree(const SolveNode<T>* sn, const int* children, const int2* pairs,
                     const WaveLevel& wl, int nrhs, double* x, int ldx, bool scale_sqrt,
                     int* status, cudaStream_t s);
// one backward pass over the whole tree (gathers, D^{-1} by diag_mode and
// the L21^T products included)
template <typename T>
void launch_bwd_tree(const SolveNode<T>* sn, const WaveLevel& wl, double* x, int ldx, int nrhs,
                     int diag_mode, int* status, cudaStream_t s);
// the inverses of the 64 x 64 unit lower diagonal blocks blocks[i] =
// (front, block) into each front's SolveNode::binv
template <typename T>
void launch_diag_inv(const SolveNode<T>* sn, const int2* blocks, int nblocks, cudaStream_t s);
// failure-detection probe of the wavefront solves' bounded flag wait
// (solve_kernels.cu): -51 when the wait gave up
int wave_timeout_probe(int rounds);
// sets the solve kernels' dynamic shared memory limits (once per process)
template <typename T>
void solve_init();
template <typename T>
// diag_mode: 0 none, 1 D^{-1}, 2 sqrt(D^{-1}) (posdef backward solve)
void launch_bwd(const SolveNode<T>* sn, const int* nodes, int nn, double* x, int ldx, int nrhs,
                int max_m, int max_nelim, int diag_mode, bool do_bwd, cudaStream_t s,
                PhaseTimer* tm);

}  // namespace ssids300
