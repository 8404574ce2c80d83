// Forward, diagonal and backward solves over the assembly tree, many
// right-hand sides at once (the reference GPU path solves one
// right-hand side per call, src/ssids/gpu/subtree.f90:570-579).
//
// Semantics follow the CPU subtree solves (src/ssids/cpu/NumericSubtree.hxx:
// 284-400 with ldlt_app_solve_fwd/diag/bwd, ldlt_app.cxx:2538-2589):
//   forward : per node, y = L11^{-1} x(fully summed); x(rows below) -= L21 y
//   diagonal: x = D^{-1} x (1x1 and 2x2 pivots)
//   backward: x(elim) -= L21^T x(rows below); x = L11^{-T} x
// The forward pass is organised multifrontally so that nodes of one level
// never update the same entry: each node gathers b for its own pivots plus
// its children's local vectors (fixed order, no atomics), solves, and leaves
// rows [nelim, m) of its local vector for its parent.  The triangular solves
// are blocked by 64 rows.  Two schedules:
//  * wavefront passes (FP32 factors by default): one persistent launch per
//    pass over the whole tree; CTAs take work items (gathers, pivot blocks,
//    contribution row blocks, or a small front whole) in a fixed order from
//    an atomic counter and wait, with bounded polls, on completion flags and
//    counters of earlier items only, so fronts of different levels overlap
//    and no level boundary drains the GPU (k_fwd_tree, k_bwd_tree);
//  * block steps (FP64 factors by default): per level a gather launch, then
//    one kernel per block step: every CTA of the step stages the step's
//    diagonal block in shared memory (cp.async) and solves it itself, each
//    right-hand side in its own warp (values in registers, the pivot row
//    broadcast by shuffles), then takes its share of the block's update
//    (rows below the block in the forward pass, columns left of it in the
//    backward pass).  No CTA waits for another and the solution is written
//    to the output vector by CTA 0 of the step, so a level needs no scatter
//    launch.
// Arithmetic is in the factor precision T; the number of right-hand sides
// per pass NR is a template parameter so that no work is spent on absent
// columns.  Every sum runs in a fixed order, so results do not depend on
// which CTA takes which item.
#include <mutex>
#include <type_traits>

#include "ssids_gpu.cuh"

namespace ssids300 {

namespace {

constexpr int SB = kSolveBlk;

// Value of assembly-order position pos of a node's local vector for
// right-hand side q: b for the node's own pivots, the delayed entry of the
// child that delayed it, and the contribution rows that the children map to
// pos (pair list gp, children in their fixed order).  Each entry is a pure
// function of b and the children's local vectors, so any number of CTAs can
// gather one node; the additions run in child order, so the sums do not
// depend on the launch shape.
// With CG the children's values are read from L2 (__ldcg): in a wavefront
// pass they were written by other CTAs of the same launch.
template <typename T, bool CG = false>
__device__ __forceinline__ T gather_value(const SolveNode<T>& sn, const SolveNode<T>* sns,
                                          const int* children, const int2* pairs,
                                          const double* x, int ldx, int q, int pos) {
  auto ld = [](const T* p) { return CG ? __ldcg(p) : *p; };
  T v = T(0);
  int P;
  if (pos < sn.ncol) {
    v = (T)x[(int64_t)q * ldx + sn.sptr0 + pos];
    P = pos;
  } else if (pos < sn.ncol + sn.ndelay_in) {
    const int k = pos - sn.ncol;
    for (int ci = sn.child_beg; ci < sn.child_end; ++ci) {
      const SolveNode<T>& cn = sns[children[ci]];
      const int nd = cn.n - cn.nelim;
      if (k >= cn.doff && k < cn.doff + nd)
        return ld(&cn.xloc[(int64_t)q * cn.m + cn.nelim + (k - cn.doff)]);
    }
    return v;
  } else {
    P = pos - sn.ndelay_in;
  }
  const int k1 = sn.gp[P + 1];
  for (int k = sn.gp[P]; k < k1; ++k) {
    const int2 pr = pairs[k];
    const SolveNode<T>& cn = sns[pr.x];
    v += ld(&cn.xloc[(int64_t)q * cn.m + cn.n + pr.y]);
  }
  return v;
}

constexpr int kSolveThreads = 256;
constexpr int kSolveWarps = kSolveThreads / 32;
constexpr int LDB = SB + 1;  // leading dimension of a staged block Lb[c * LDB + r]
constexpr int kDiagPer = SB * SB / kSolveThreads;  // entries of a staged block per thread

// stage the jb x jb diagonal block (strictly lower part) into shared memory
// with asynchronous copies (cp.async): a CTA starts it, does other work, and
// waits for it with cp_async_wait_all() and a barrier before the block is
// read; the entries outside the strictly lower part are zeroed
template <typename T>
__device__ __forceinline__ void prefetch_diag_block(const SolveNode<T>& sn, int j0, int jb, T* Lb) {
#pragma unroll
  for (int k = 0; k < kDiagPer; ++k) {
    const int e = threadIdx.x + k * kSolveThreads;
    const int c = e / SB, r = e % SB;
    T* dst = Lb + c * LDB + r;
    if (r > c && r < jb && c < jb) {
      const unsigned sa = (unsigned)__cvta_generic_to_shared(dst);
      const T* src = sn.L + (int64_t)(j0 + c) * sn.ld + j0 + r;
      if constexpr (sizeof(T) == 8)
        asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(sa), "l"(src) : "memory");
      else
        asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(sa), "l"(src) : "memory");
    } else {
      *dst = T(0);
    }
  }
  asm volatile("cp.async.commit_group;\n" ::: "memory");
}
__device__ __forceinline__ void cp_async_wait_all() {
  asm volatile("cp.async.wait_group 0;\n" ::: "memory");
}

// Unit lower (FWD) or unit upper L^T (!FWD) triangular solve of a jb x jb
// diagonal block staged in Lb (Lb[c*LDB + r] = L(j0+r, j0+c), zero on and
// above the diagonal) for values held in registers: warp w holds the
// right-hand sides w, w + 8, ...; lane l holds rows l and l + 32.  Pivot k
// changes only the rows after it (FWD) or before it (!FWD), so once the
// chain has passed a group of 32 rows that group is left out.
static_assert(SB == 64, "the register layout below holds two row groups per lane");
template <typename T, int R, bool FWD>
__device__ __forceinline__ void solve_in_regs(int jb, const T* Lb, T (&x)[R][2]) {
  const int lane = threadIdx.x & 31;
  if (jb <= 32) {
    // one row group: the second holds no rows of the block
    for (int k = 0; k < jb - 1; ++k) {
      const T l0 = FWD ? Lb[k * LDB + lane] : Lb[lane * LDB + (jb - 1 - k)];
#pragma unroll
      for (int r = 0; r < R; ++r) {
        const T v = __shfl_sync(0xffffffffu, x[r][0], FWD ? k : jb - 1 - k);
        x[r][0] -= l0 * v;
      }
    }
    return;
  }
  if (FWD) {
    const int k1 = min(jb - 1, 32);
    for (int k = 0; k < k1; ++k) {
      const T l0 = Lb[k * LDB + lane], l1 = Lb[k * LDB + lane + 32];
#pragma unroll
      for (int r = 0; r < R; ++r) {
        const T xk = __shfl_sync(0xffffffffu, x[r][0], k);
        x[r][0] -= l0 * xk;
        x[r][1] -= l1 * xk;
      }
    }
    for (int k = 32; k < jb - 1; ++k) {
      const T l1 = Lb[k * LDB + lane + 32];
#pragma unroll
      for (int r = 0; r < R; ++r) {
        const T xk = __shfl_sync(0xffffffffu, x[r][1], k & 31);
        x[r][1] -= l1 * xk;
      }
    }
  } else {
    // (L^T y)_r = y_r + sum_{c > r} L(c, r) y_c, c from the bottom
    for (int c = jb - 1; c >= 32; --c) {
      const T l0 = Lb[lane * LDB + c], l1 = Lb[(lane + 32) * LDB + c];
#pragma unroll
      for (int r = 0; r < R; ++r) {
        const T yc = __shfl_sync(0xffffffffu, x[r][1], c & 31);
        x[r][0] -= l0 * yc;
        x[r][1] -= l1 * yc;
      }
    }
    for (int c = min(jb - 1, 31); c > 0; --c) {
      const T l0 = Lb[lane * LDB + c];
#pragma unroll
      for (int r = 0; r < R; ++r) {
        const T yc = __shfl_sync(0xffffffffu, x[r][0], c);
        x[r][0] -= l0 * yc;
      }
    }
  }
}

// dynamic shared memory of the solve kernels: the staged block, the
// block's solved values yb[r * NR + q], then the partial sums of the
// update passes red[(qq * NR + q) * PR + t] (256 NR values for any pass width)
template <typename T, int NR>
constexpr size_t solve_smem_bytes() {
  return sizeof(T) * ((size_t)SB * LDB + (size_t)SB * NR + (size_t)4 * NR * 64);
}
// the wavefront passes' kernels: the same, then a small front's local
// vector (kWaveSmall items: at most SB + kWaveSmallRows rows)
template <typename T, int NR>
constexpr size_t wave_smem_bytes() {
  return solve_smem_bytes<T, NR>() + sizeof(T) * (size_t)(SB + kWaveSmallRows) * NR;
}

// Solve of diagonal block [j0, j0+jb) inside a block step, after the CTA
// started staging it with prefetch_diag_block.  Every CTA of the step solves
// the block itself: its solution feeds that CTA's share of the update, so
// no CTA waits for another.  The solution goes to yb (yb[r*NR + q], zero
// outside the block and for absent right-hand sides) and CTA 0 writes it to
// the output vector x through perm (times sqrt(D^{-1}) for the posdef
// forward solve, L_chol = L D^(1/2)).  The local vector keeps the unsolved
// values (other CTAs of the step may still be reading them) unless to_xloc
// is set by a CTA that is alone on its node.  Ends with a barrier.
template <typename T, int NR, bool FWD>
__device__ __forceinline__ void block_solve(const SolveNode<T>& sn, int j0, int jb, int nrhs,
                                            const T* Lb, T* yb, double* x, int ldx,
                                            bool scale_sqrt, bool to_xloc) {
  constexpr int R = (NR + kSolveWarps - 1) / kSolveWarps;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  T xr[R][2];
#pragma unroll
  for (int r = 0; r < R; ++r) {
    const int q = warp + r * kSolveWarps;
#pragma unroll
    for (int g = 0; g < 2; ++g) {
      const int row = lane + 32 * g;
      xr[r][g] = (q < nrhs && row < jb) ? sn.xloc[(int64_t)q * sn.m + j0 + row] : T(0);
    }
  }
  cp_async_wait_all();
  __syncthreads();
  if (warp < nrhs) solve_in_regs<T, R, FWD>(jb, Lb, xr);
#pragma unroll
  for (int r = 0; r < R; ++r) {
    const int q = warp + r * kSolveWarps;
    if (q >= NR) continue;
#pragma unroll
    for (int g = 0; g < 2; ++g) {
      const int row = lane + 32 * g;
      const bool ok = q < nrhs && row < jb;
      yb[row * NR + q] = ok ? xr[r][g] : T(0);
      if (ok && to_xloc) sn.xloc[(int64_t)q * sn.m + j0 + row] = xr[r][g];
      if (ok && blockIdx.x == 0) {
        double v = (double)xr[r][g];
        if (scale_sqrt) v *= sqrt(sn.D[2 * (j0 + row)]);
        x[(int64_t)q * ldx + sn.perm[j0 + row]] = v;
      }
    }
  }
  __syncthreads();
}

// ---- forward ----
// Gather every node of the level into its local vector (final positions:
// xloc[i] = value of assembly position opos[i] for i < n), all CTAs of a
// node grid-striding over its entries.
template <typename T>
__global__ void k_fwd_gather(const SolveNode<T>* sns, const int* nodes, const int* children,
                             const int2* pairs, const double* x, int ldx, int nrhs) {
  const SolveNode<T> sn = sns[nodes[blockIdx.y]];  // written by the host before the launch
  pdl_wait();
  pdl_trigger();
  const int m = sn.m;
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < m * nrhs;
       e += gridDim.x * blockDim.x) {
    const int i = e % m, q = e / m;
    const int pos = (i < sn.n) ? sn.opos[i] : i;
    sn.xloc[(int64_t)q * m + i] = gather_value(sn, sns, children, pairs, x, ldx, q, pos);
  }
}

// Update passes of the block steps: a CTA pass covers PR rows (forward) or
// columns (backward); thread (t, qq) = (threadIdx.x % PR, threadIdx.x / PR)
// forms the partial dot products of entry t over the block columns
// [qq CW, (qq+1) CW), CW = SB PR / 256, for every right-hand side, with
// those loads issued together, and the 256 / PR partial sums are added
// through shared memory in qq order.  FP32 passes cover 64 entries; FP64
// passes 16, because a 64-entry pass is 32k FP64 FMAs for 8 right-hand
// sides, which on GB300's FP64 pipe (about 1.7 per clock per SM) would
// keep one SM busy for about 9 us.
template <typename T>
constexpr int pass_rows() { return sizeof(T) == 8 ? 16 : 64; }

template <typename T, int NR, int CW>
__device__ __forceinline__ void partial_dots(const T* p, int64_t stride, int cq, int jb,
                                             const T* yb, T (&acc)[NR]) {
  T lv[CW];
#pragma unroll
  for (int k = 0; k < CW; ++k) lv[k] = (cq + k < jb) ? p[(int64_t)k * stride] : T(0);
#pragma unroll
  for (int q = 0; q < NR; ++q) acc[q] = T(0);
#pragma unroll
  for (int k = 0; k < CW; ++k)
#pragma unroll
    for (int q = 0; q < NR; ++q) acc[q] += lv[k] * yb[(cq + k) * NR + q];
}

// red[(qq * NR + q) * PR + t] holds the partial sums; entry t of the pass
// (global index base + t < lim) gets x -= the sum of its partials
template <typename T, int NR, int PR>
__device__ __forceinline__ void apply_partials(const SolveNode<T>& sn, const T* red, int base,
                                               int lim, int nrhs) {
  constexpr int QN = kSolveThreads / PR;
  for (int e = threadIdx.x; e < PR * NR; e += blockDim.x) {
    const int t = e % PR, q = e / PR;
    const int idx = base + t;
    if (q < nrhs && idx < lim) {
      T v = red[q * PR + t];
#pragma unroll
      for (int qq = 1; qq < QN; ++qq) v += red[(qq * NR + q) * PR + t];
      sn.xloc[(int64_t)q * sn.m + idx] -= v;
    }
  }
}

// the solved rows [j0, j0+jb) of every right-hand side into yb[r*NR + q]
// (zero outside the block), then a barrier
template <typename T, int NR>
__device__ __forceinline__ void load_y(const SolveNode<T>& sn, int j0, int jb, int nrhs, T* yb) {
  for (int e = threadIdx.x; e < SB * NR; e += blockDim.x) {
    const int r = e % SB, q = e / SB;
    yb[r * NR + q] = (r < jb && q < nrhs) ? sn.xloc[(int64_t)q * sn.m + j0 + r] : T(0);
  }
  __syncthreads();
}

// Block step kernels, three shapes (MODE):
//   kStepFused  solve block st in every CTA (block_solve), then update;
//   kStepSolve  one CTA per node solves block st and stores it in xloc;
//   kStepUpdate update only, y read back from xloc.
// The FP32 path always runs fused steps.  The FP64 path runs fused steps on
// levels with few nodes (their large fronts spread over many CTAs, where the
// latency of a step matters) and solve + update pairs on levels with many
// nodes, where the FP64 pipe is the limit and a repeated diagonal solve in
// every CTA would add FP64 work.
// All shapes use the same pass width, so a node's arithmetic (and result)
// does not depend on the level it shares with other nodes.
constexpr int kStepFused = 0, kStepSolve = 1, kStepUpdate = 2;

// Forward block step st: solve block st, then the rows i >= j0 + jb take
// x_i -= sum_c L(i, j0+c) y_c, PR rows per pass, the passes spread over the
// CTAs.
template <typename T, int NR, int MODE>
__global__ void __launch_bounds__(kSolveThreads)
    k_fwd_step(const SolveNode<T>* sns, const int* nodes, int step, int nrhs, double* x, int ldx,
               bool scale_sqrt) {
  const SolveNode<T> sn = sns[nodes[blockIdx.y]];  // written by the host before the launch
  pdl_wait();
  pdl_trigger();
  const int j0 = step * SB;
  if (j0 >= sn.nelim) return;
  const int jb = min(SB, sn.nelim - j0);
  extern __shared__ __align__(16) unsigned char solve_smem[];
  T* Lb = reinterpret_cast<T*>(solve_smem);
  T* yb = Lb + SB * LDB;
  T* red = yb + SB * NR;
  if (MODE == kStepUpdate) {
    load_y<T, NR>(sn, j0, jb, nrhs, yb);
  } else {
    prefetch_diag_block(sn, j0, jb, Lb);
    block_solve<T, NR, true>(sn, j0, jb, nrhs, Lb, yb, x, ldx, scale_sqrt, MODE == kStepSolve);
    if (MODE == kStepSolve) return;
  }
  constexpr int PR = pass_rows<T>(), CW = SB * PR / kSolveThreads;
  const int t = threadIdx.x % PR, qq = threadIdx.x / PR;
  for (int base = j0 + jb + blockIdx.x * PR; base < sn.m; base += gridDim.x * PR) {
    const int i = base + t;
    T acc[NR];
    if (i < sn.m) {
      partial_dots<T, NR, CW>(sn.L + (int64_t)(j0 + qq * CW) * sn.ld + i, sn.ld, qq * CW, jb, yb,
                              acc);
    } else {
#pragma unroll
      for (int q = 0; q < NR; ++q) acc[q] = T(0);
    }
#pragma unroll
    for (int q = 0; q < NR; ++q) red[(qq * NR + q) * PR + t] = acc[q];
    __syncthreads();
    apply_partials<T, NR, PR>(sn, red, base, sn.m, nrhs);
    __syncthreads();
  }
}

template <typename T>
__global__ void k_fwd_scatter(const SolveNode<T>* sns, const int* nodes, double* x, int ldx,
                              int nrhs, bool scale_sqrt) {
  const SolveNode<T> sn = sns[nodes[blockIdx.y]];  // written by the host before the launch
  pdl_wait();
  pdl_trigger();
  const int tot = sn.nelim * nrhs;
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < tot; e += gridDim.x * blockDim.x) {
    const int i = e % sn.nelim, q = e / sn.nelim;
    double v = (double)sn.xloc[(int64_t)q * sn.m + i];
    if (scale_sqrt) v *= sqrt(sn.D[2 * i]);
    x[(int64_t)q * ldx + sn.perm[i]] = v;
  }
}

// ---- backward ----
// diag_mode: 0 none, 1 apply D^{-1} (1x1 and 2x2), 2 apply sqrt(D^{-1}) (the
// posdef backward solve with L_chol^T = D^(1/2) L^T)
// Value of local position i for right-hand side q at the start of the
// backward pass: x at the position's pivot (for i < nelim times D^{-1}
// with 2x2 blocks, or sqrt(D^{-1}) for diag_mode 2).  With CG, x is read
// from L2 (ancestors' values written by other CTAs of the same launch).
template <bool CG, typename T>
__device__ __forceinline__ double bwd_gather_value(const SolveNode<T>& sn, const double* x,
                                                   int ldx, int diag_mode, int q, int i) {
  auto ld = [](const double* p) { return CG ? __ldcg(p) : *p; };
  const int src = (i < sn.n) ? sn.perm[i] : sn.rows[sn.ncol + i - sn.n];
  double v = ld(&x[(int64_t)q * ldx + src]);
  if (diag_mode == 2 && i < sn.nelim) {
    v *= sqrt(sn.D[2 * i]);
  } else if (diag_mode == 1 && i < sn.nelim) {
    const double di = sn.D[2 * i];
    if (isinf(di)) {
      // second half of a 2x2: d21*x1 + d22*x2
      const double d21 = sn.D[2 * (i - 1) + 1], d22 = sn.D[2 * i + 1];
      const double x1 = ld(&x[(int64_t)q * ldx + sn.perm[i - 1]]);
      v = d21 * x1 + d22 * v;
    } else if (i + 1 < sn.nelim && isinf(sn.D[2 * i + 2])) {
      const double d21 = sn.D[2 * i + 1];
      const double x2 = ld(&x[(int64_t)q * ldx + sn.perm[i + 1]]);
      v = di * v + d21 * x2;
    } else {
      v = di * v;
    }
  }
  return v;
}

template <typename T>
__global__ void k_bwd_gather(const SolveNode<T>* sns, const int* nodes, const double* x, int ldx,
                             int nrhs, int diag_mode, bool do_bwd) {
  const SolveNode<T> sn = sns[nodes[blockIdx.y]];  // written by the host before the launch
  pdl_wait();
  pdl_trigger();
  const int mm = do_bwd ? sn.m : sn.nelim;
  const int tot = mm * nrhs;
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < tot; e += gridDim.x * blockDim.x) {
    const int i = e % mm, q = e / mm;
    sn.xloc[(int64_t)q * sn.m + i] = (T)bwd_gather_value<false>(sn, x, ldx, diag_mode, q, i);
  }
}

// Partial sums of sum_{i in [nelim, m)} L(i, j) xloc[i] for column j over
// the rows i = nelim + i0, i0 + stride, ... of one lane.  Each lane takes U
// rows per round with all their loads issued before the FMAs, so a column
// costs about (m - nelim) / (stride U) memory round trips.
template <typename T, int NR>
__device__ __forceinline__ void bwd_l21_partial(const SolveNode<T>& sn, int j, int i0, int stride,
                                                int nrhs, T (&acc)[NR]) {
  constexpr int U = (NR * sizeof(T) >= 64) ? 2 : 4;
  const T* col = sn.L + (int64_t)j * sn.ld;
  int i = sn.nelim + i0;
  for (; i + stride * (U - 1) < sn.m; i += stride * U) {
    T l[U], xv[U][NR];
#pragma unroll
    for (int u = 0; u < U; ++u) l[u] = col[i + stride * u];
#pragma unroll
    for (int u = 0; u < U; ++u)
#pragma unroll
      for (int q = 0; q < NR; ++q)
        xv[u][q] = (q < nrhs) ? sn.xloc[(int64_t)q * sn.m + i + stride * u] : T(0);
#pragma unroll
    for (int u = 0; u < U; ++u)
#pragma unroll
      for (int q = 0; q < NR; ++q) acc[q] += l[u] * xv[u][q];
  }
  for (; i < sn.m; i += stride) {
    const T l = col[i];
#pragma unroll
    for (int q = 0; q < NR; ++q)
      if (q < nrhs) acc[q] += l * sn.xloc[(int64_t)q * sn.m + i];
  }
}

// warps that share one column of the L21^T product, from the node's own
// rows below its pivots (so a node is computed the same way whatever level
// it shares)
__device__ __forceinline__ int l21_warps(int rows_below) {
  return rows_below <= 128 ? 1 : rows_below <= 512 ? 2 : rows_below <= 1024 ? 4 : 8;
}
inline int l21_warps_host(int rows_below) {
  return rows_below <= 128 ? 1 : rows_below <= 512 ? 2 : rows_below <= 1024 ? 4 : 8;
}

// L21^T part of the backward solve for every eliminated column:
// xloc[j] -= sum_{i in [nelim, m)} L(i, j) xloc[i].  W warps share a column
// (rows strided over their 32 W lanes); their partial sums are added in
// shared memory in warp order.
template <typename T, int NR>
__global__ void __launch_bounds__(kSolveThreads)
    k_bwd_l21(const SolveNode<T>* sns, const int* nodes, int nrhs) {
  const SolveNode<T> sn = sns[nodes[blockIdx.y]];  // written by the host before the launch
  pdl_wait();
  pdl_trigger();
  if (sn.m <= sn.nelim) return;
  const int W = l21_warps(sn.m - sn.nelim);
  const int CPB = kSolveWarps / W;  // columns per CTA round
  __shared__ T part[kSolveWarps][NR];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int cw = warp / W, wi = warp % W;
  for (int jb = blockIdx.x * CPB; jb < sn.nelim; jb += gridDim.x * CPB) {
    const int j = jb + cw;
    T acc[NR];
#pragma unroll
    for (int q = 0; q < NR; ++q) acc[q] = T(0);
    if (j < sn.nelim) bwd_l21_partial<T, NR>(sn, j, wi * 32 + lane, 32 * W, nrhs, acc);
#pragma unroll
    for (int q = 0; q < NR; ++q)
      for (int off = 16; off > 0; off >>= 1) acc[q] += __shfl_xor_sync(0xffffffffu, acc[q], off);
    if (lane == 0) {
#pragma unroll
      for (int q = 0; q < NR; ++q) part[warp][q] = acc[q];
    }
    __syncthreads();
    if (wi == 0 && lane < nrhs && j < sn.nelim) {
      T v = part[warp][lane];
      for (int w = 1; w < W; ++w) v += part[warp + w][lane];
      sn.xloc[(int64_t)lane * sn.m + j] -= v;
    }
    __syncthreads();
  }
}

// Backward block step st, from the last block down: solve block st, then the
// columns j < j0 take x_j -= sum_c L(j0+c, j) y_c, PR columns per pass,
// spread over the CTAs (shapes as for the forward steps).
template <typename T, int NR, int MODE>
__global__ void __launch_bounds__(kSolveThreads)
    k_bwd_step(const SolveNode<T>* sns, const int* nodes, int step, int nrhs, double* x,
               int ldx) {
  const SolveNode<T> sn = sns[nodes[blockIdx.y]];  // written by the host before the launch
  pdl_wait();
  pdl_trigger();
  const int j0 = step * SB;
  if (j0 >= sn.nelim) return;
  const int jb = min(SB, sn.nelim - j0);
  extern __shared__ __align__(16) unsigned char solve_smem[];
  T* Lb = reinterpret_cast<T*>(solve_smem);
  T* yb = Lb + SB * LDB;
  T* red = yb + SB * NR;
  if (MODE == kStepUpdate) {
    load_y<T, NR>(sn, j0, jb, nrhs, yb);
  } else {
    prefetch_diag_block(sn, j0, jb, Lb);
    block_solve<T, NR, false>(sn, j0, jb, nrhs, Lb, yb, x, ldx, false, MODE == kStepSolve);
    if (MODE == kStepSolve) return;
  }
  constexpr int PR = pass_rows<T>(), CW = SB * PR / kSolveThreads;
  const int t = threadIdx.x % PR, qq = threadIdx.x / PR;
  for (int base = blockIdx.x * PR; base < j0; base += gridDim.x * PR) {
    const int j = base + t;
    T acc[NR];
    if (j < j0) {
      partial_dots<T, NR, CW>(sn.L + (int64_t)j * sn.ld + j0 + qq * CW, 1, qq * CW, jb, yb, acc);
    } else {
#pragma unroll
      for (int q = 0; q < NR; ++q) acc[q] = T(0);
    }
#pragma unroll
    for (int q = 0; q < NR; ++q) red[(qq * NR + q) * PR + t] = acc[q];
    __syncthreads();
    apply_partials<T, NR, PR>(sn, red, base, j0, nrhs);
    __syncthreads();
  }
}

// ---- wavefront solves (one persistent launch per pass, whole tree) ----
// persistent CTAs per SM of a pass, CPS (registers capped to fit them):
// 3 for trees of many small fronts (more items in flight), 2 otherwise (no
// spilled registers on the chains of the widest fronts); WaveLevel tells
// try rounds of a flag wait before it gives up (each round sleeps briefly);
// no legitimate wait comes close
constexpr long long kWaveSpinLimit = 1LL << 22;

__device__ __forceinline__ int ld_acquire(const int* p) {
  int v;
  asm volatile("ld.acquire.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_release(int* p, int v) {
  asm volatile("st.release.gpu.global.b32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
// every thread: wait until *ctr >= target, the counter being advanced by
// other CTAs (thread 0 polls); false once the wait, or another CTA's wait,
// gave up
__device__ __forceinline__ bool wave_wait_count(const int* ctr, int target, int* status,
                                                int* s_fail) {
  if (threadIdx.x == 0) {
    bool ok = true;
    for (long long it = 0; ld_acquire(ctr) < target; ++it) {
      if (it >= kWaveSpinLimit || *(volatile int*)status != 0) { ok = false; break; }
      __nanosleep(20);
    }
    if (!ok) atomicExch(status, 1);
    *s_fail = ok ? 0 : 1;
  }
  __syncthreads();
  return *s_fail == 0;
}
// completion flag of one pivot block
__device__ __forceinline__ bool wave_wait(const int* flag, int* status, int* s_fail) {
  return wave_wait_count(flag, 1, status, s_fail);
}
// after every thread of the CTA has written its part of an item: publish
// (all writes before the counter advances, as seen by any CTA)
__device__ __forceinline__ void wave_signal(int* ctr_a, int* ctr_b) {
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    if (ctr_a) atomicAdd(ctr_a, 1);
    if (ctr_b) atomicAdd(ctr_b, 1);
  }
}

// Failure-detection probe: one CTA waits on a completion flag that no
// item will ever set, with the wait bounded to `rounds` polls; the wait
// gives up and sets *status, as a wavefront solve does.
__global__ void k_wave_timeout_probe(const int* flag, long long rounds, int* status) {
  if (threadIdx.x == 0) {
    bool ok = true;
    for (long long it = 0; ld_acquire(flag) == 0; ++it)
      if (it >= rounds) { ok = false; break; }
    if (!ok) atomicExch(status, 1);
  }
}

__device__ __forceinline__ unsigned long long global_timer() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}
// trace stamp k of item it (thread 0; no-op without a trace buffer)
__device__ __forceinline__ void wave_stamp(const WaveLevel& wl, int it, int k) {
  if (wl.trace && threadIdx.x == 0) {
    wl.trace[4 * (size_t)it + k] = global_timer();
    if (k == 0) {
      unsigned sm;
      asm volatile("mov.u32 %0, %%smid;" : "=r"(sm));
      wl.trace[4 * (size_t)it + 3] = sm;
    }
  }
}

// the next item of the pass for this CTA (kept in shared memory)
__device__ __forceinline__ int wave_next(const WaveLevel& wl, int* s_item) {
  __syncthreads();  // every thread is done with the previous item
  if (threadIdx.x == 0) *s_item = atomicAdd(wl.counter, 1);
  __syncthreads();
  return *s_item;
}

template <typename T>
__device__ __forceinline__ int* wave_l21done(const SolveNode<T>& sn, int b) {
  return sn.flag + sn.nblk + b;
}
template <typename T>
__device__ __forceinline__ int* wave_gathered(const SolveNode<T>& sn) {
  return sn.flag + 2 * sn.nblk;
}
template <typename T>
__device__ __forceinline__ int* wave_finished(const SolveNode<T>& sn) {
  return sn.flag + 2 * sn.nblk + 1;
}

// Forward gather of rows [r0, r1) of a front's local vector, one row per
// thread with every right-hand side (the row's index lookups once, its
// children's values, from L2, all in flight together).  The additions run
// in the same order as gather_value's.
template <typename T, int NR>
__device__ __forceinline__ void fwd_gather_rows(const SolveNode<T>& sn, const SolveNode<T>* sns,
                                                const int* children, const int2* pairs,
                                                const double* x, int ldx, int nrhs, int r0,
                                                int r1) {
  for (int i = r0 + threadIdx.x; i < r1; i += blockDim.x) {
    const int pos = (i < sn.n) ? sn.opos[i] : i;
    T v[NR];
#pragma unroll
    for (int q = 0; q < NR; ++q) v[q] = T(0);
    int P = -1;
    if (pos < sn.ncol) {
#pragma unroll
      for (int q = 0; q < NR; ++q)
        if (q < nrhs) v[q] = (T)x[(int64_t)q * ldx + sn.sptr0 + pos];
      P = pos;
    } else if (pos < sn.ncol + sn.ndelay_in) {
      const int k = pos - sn.ncol;
      for (int ci = sn.child_beg; ci < sn.child_end; ++ci) {
        const SolveNode<T>& cn = sns[children[ci]];
        const int nd = cn.n - cn.nelim;
        if (k >= cn.doff && k < cn.doff + nd) {
          const T* src = cn.xloc + cn.nelim + (k - cn.doff);
#pragma unroll
          for (int q = 0; q < NR; ++q)
            if (q < nrhs) v[q] = __ldcg(src + (int64_t)q * cn.m);
          break;
        }
      }
    } else {
      P = pos - sn.ndelay_in;
    }
    if (P >= 0) {
      const int k1 = sn.gp[P + 1];
      for (int k = sn.gp[P]; k < k1; ++k) {
        const int2 pr = pairs[k];
        const SolveNode<T>& cn = sns[pr.x];
        const T* src = cn.xloc + cn.n + pr.y;
#pragma unroll
        for (int q = 0; q < NR; ++q)
          if (q < nrhs) v[q] += __ldcg(src + (int64_t)q * cn.m);
      }
    }
#pragma unroll
    for (int q = 0; q < NR; ++q)
      if (q < nrhs) sn.xloc[(int64_t)q * sn.m + i] = v[q];
  }
}

// Backward gather of rows [r0, r1), one row per thread (x from L2)
template <typename T, int NR>
__device__ __forceinline__ void bwd_gather_rows(const SolveNode<T>& sn, const double* x, int ldx,
                                                int nrhs, int diag_mode, int r0, int r1) {
  for (int i = r0 + threadIdx.x; i < r1; i += blockDim.x) {
    // the row's pivot positions and D^{-1} coefficients once, then every
    // right-hand side's loads together (the arithmetic of bwd_gather_value)
    const int src = (i < sn.n) ? sn.perm[i] : sn.rows[sn.ncol + i - sn.n];
    int src2 = -1;      // the other half of a 2x2 block
    double ca = 1.0, cb = 0.0;  // v = ca x(src) + cb x(src2)
    if (diag_mode == 2 && i < sn.nelim) {
      ca = sqrt(sn.D[2 * i]);
    } else if (diag_mode == 1 && i < sn.nelim) {
      const double di = sn.D[2 * i];
      if (isinf(di)) {
        src2 = sn.perm[i - 1];
        ca = sn.D[2 * i + 1];
        cb = sn.D[2 * (i - 1) + 1];
      } else if (i + 1 < sn.nelim && isinf(sn.D[2 * i + 2])) {
        src2 = sn.perm[i + 1];
        ca = di;
        cb = sn.D[2 * i + 1];
      } else {
        ca = di;
      }
    }
    double v[NR], w[NR];
#pragma unroll
    for (int q = 0; q < NR; ++q) {
      v[q] = (q < nrhs) ? __ldcg(&x[(int64_t)q * ldx + src]) : 0.0;
      w[q] = (q < nrhs && src2 >= 0) ? __ldcg(&x[(int64_t)q * ldx + src2]) : 0.0;
    }
#pragma unroll
    for (int q = 0; q < NR; ++q) {
      if (q >= nrhs) continue;
      double r;
      if (src2 < 0) r = (diag_mode == 0 || i >= sn.nelim) ? v[q] : ca * v[q];
      else if (isinf(sn.D[2 * i])) r = cb * w[q] + ca * v[q];   // d21 x1 + d22 x2
      else r = ca * v[q] + cb * w[q];                           // di x + d21 x2
      sn.xloc[(int64_t)q * sn.m + i] = (T)r;
    }
  }
}

// Forward block item.  A pivot block b takes x_b -= sum_{j < b} L(b, j) y_j,
// block by block as the flags of blocks j arrive (thread (r, cq): row r,
// columns [16 cq, 16 cq + 16) of each 64-column block), adds the four column
// quarters in shared memory, solves its unit lower diagonal block in
// registers (warp per right-hand side), writes y to the local vector and to
// x, and sets its flag.  A contribution row block takes the whole L21 y
// product the same way.  False if a wait gave up.
template <typename T, int NR>
__device__ bool fwd_block(const SolveNode<T>& sn, int code, int nrhs, double* x, int ldx,
                          bool scale_sqrt, int* status, T* Lb, T* yb, T* red, int* s_fail,
                          const WaveLevel& wl, int it) {
  constexpr int R = (NR + kSolveWarps - 1) / kSolveWarps;
  const int tid = threadIdx.x, r = tid % SB, cq = tid / SB;
  const int warp = tid >> 5, lane = tid & 31;
  const int m = sn.m, nelim = sn.nelim;
  const bool piv = code < kWaveContrib;
  const int r0 = piv ? code * SB : nelim + (code - kWaveContrib) * SB;
  const int rows = min(SB, (piv ? nelim : m) - r0);
  const int ncb = piv ? code : sn.nblk;
  T own[R][2];  // a pivot block's gathered values, final before any wait below
  T bv[16];     // with inverses: row r, columns [16 cq, 16 cq + 16) of the block's
  if (piv) {
    if (sn.binv) {
      const T* bp = sn.binv + (size_t)code * SB * SB + r * SB + cq * 16;
#pragma unroll
      for (int k = 0; k < 16; ++k) bv[k] = bp[k];
    } else {
      prefetch_diag_block(sn, r0, rows, Lb);
    }
#pragma unroll
    for (int rr = 0; rr < R; ++rr) {
      const int q = warp + rr * kSolveWarps;
#pragma unroll
      for (int g = 0; g < 2; ++g) {
        const int row = lane + 32 * g;
        own[rr][g] = (q < nrhs && q < NR && row < rows) ? __ldcg(&sn.xloc[(int64_t)q * m + r0 + row])
                                                        : T(0);
      }
    }
  }
  T acc[NR];
#pragma unroll
  for (int q = 0; q < NR; ++q) acc[q] = T(0);
  bool ok = true;
  for (int j = 0; j < ncb && ok; ++j) {
    const int c0 = j * SB, jb = min(SB, nelim - c0);
    // the tile of L does not depend on block j's result: its loads are
    // in flight while the flag is awaited
    T lv[16];
    {
      const T* Lp = sn.L + (int64_t)(c0 + cq * 16) * sn.ld + r0 + r;
#pragma unroll
      for (int k = 0; k < 16; ++k)
        lv[k] = (r < rows && cq * 16 + k < jb) ? Lp[(int64_t)k * sn.ld] : T(0);
    }
    ok = wave_wait(&sn.flag[j], status, s_fail);
    if (!ok) break;
    for (int e = tid; e < SB * NR; e += kSolveThreads) {
      const int c = e % SB, q = e / SB;
      // another CTA wrote these values: read them from L2, past this SM's L1
      yb[c * NR + q] = (c < jb && q < nrhs) ? __ldcg(&sn.xloc[(int64_t)q * m + c0 + c]) : T(0);
    }
    __syncthreads();
    // a warp's 32 rows and 16 columns are warp-uniform: a warp wholly past
    // the block's rows or columns holds zeros of L and skips the products
    // (the padded tiles of narrow fronts; with FP64 factors the passes are
    // bound by the FMA rate)
    if (cq * 16 < jb && (r & ~31) < rows) {
#pragma unroll
      for (int k = 0; k < 16; ++k)
#pragma unroll
        for (int q = 0; q < NR; ++q) acc[q] += lv[k] * yb[(cq * 16 + k) * NR + q];
    }
    __syncthreads();
  }
  if (!ok) {
    if (piv && !sn.binv) cp_async_wait_all();
    return false;
  }
  wave_stamp(wl, it, 1);
#pragma unroll
  for (int q = 0; q < NR; ++q) red[(cq * NR + q) * SB + r] = acc[q];
  __syncthreads();
  if (piv && sn.binv) {
    // y = L_bb^{-1} (b - sum): the right-hand side into yb, then the
    // block inverse's row r times it over column quarter cq, the quarters
    // added in order
#pragma unroll
    for (int rr = 0; rr < R; ++rr) {
      const int q = warp + rr * kSolveWarps;
#pragma unroll
      for (int g = 0; g < 2; ++g) {
        const int row = lane + 32 * g;
        if (q < NR)
          yb[row * NR + q] = (q < nrhs && row < rows)
                                 ? own[rr][g] - (red[q * SB + row] + red[(NR + q) * SB + row] +
                                                 red[(2 * NR + q) * SB + row] +
                                                 red[(3 * NR + q) * SB + row])
                                 : T(0);
      }
    }
    __syncthreads();
#pragma unroll
    for (int q = 0; q < NR; ++q) acc[q] = T(0);
    if (cq * 16 < rows && (r & ~31) < rows) {
#pragma unroll
      for (int k = 0; k < 16; ++k)
#pragma unroll
        for (int q = 0; q < NR; ++q) acc[q] += bv[k] * yb[(cq * 16 + k) * NR + q];
    }
#pragma unroll
    for (int q = 0; q < NR; ++q) red[(cq * NR + q) * SB + r] = acc[q];
    __syncthreads();
    for (int e = tid; e < SB * NR; e += kSolveThreads) {
      const int row = e % SB, q = e / SB;
      if (row < rows && q < nrhs) {
        const T y = red[q * SB + row] + red[(NR + q) * SB + row] + red[(2 * NR + q) * SB + row] +
                    red[(3 * NR + q) * SB + row];
        sn.xloc[(int64_t)q * m + r0 + row] = y;
        double v = (double)y;
        if (scale_sqrt) v *= sqrt(sn.D[2 * (r0 + row)]);
        x[(int64_t)q * ldx + sn.perm[r0 + row]] = v;
      }
    }
    __syncthreads();
    if (tid == 0) st_release(&sn.flag[code], 1);
  } else if (piv) {
    T xr[R][2];
#pragma unroll
    for (int rr = 0; rr < R; ++rr) {
      const int q = warp + rr * kSolveWarps;
#pragma unroll
      for (int g = 0; g < 2; ++g) {
        const int row = lane + 32 * g;
        T v = T(0);
        if (q < nrhs && q < NR && row < rows)
          v = own[rr][g] - (red[q * SB + row] + red[(NR + q) * SB + row] +
                            red[(2 * NR + q) * SB + row] + red[(3 * NR + q) * SB + row]);
        xr[rr][g] = v;
      }
    }
    cp_async_wait_all();
    __syncthreads();
    if (warp < nrhs) solve_in_regs<T, R, true>(rows, Lb, xr);
#pragma unroll
    for (int rr = 0; rr < R; ++rr) {
      const int q = warp + rr * kSolveWarps;
#pragma unroll
      for (int g = 0; g < 2; ++g) {
        const int row = lane + 32 * g;
        if (q < nrhs && q < NR && row < rows) {
          sn.xloc[(int64_t)q * m + r0 + row] = xr[rr][g];
          double v = (double)xr[rr][g];
          if (scale_sqrt) v *= sqrt(sn.D[2 * (r0 + row)]);
          x[(int64_t)q * ldx + sn.perm[r0 + row]] = v;
        }
      }
    }
    __syncthreads();
    // the release orders every thread's writes above (ordered before it by
    // the barrier) before the flag, for any CTA that acquires the flag
    if (tid == 0) st_release(&sn.flag[code], 1);
  } else {
    for (int e = tid; e < SB * NR; e += kSolveThreads) {
      const int row = e % SB, q = e / SB;
      if (row < rows && q < nrhs) {
        T* p = &sn.xloc[(int64_t)q * m + r0 + row];
        *p = __ldcg(p) - (red[q * SB + row] + red[(NR + q) * SB + row] +
                          red[(2 * NR + q) * SB + row] + red[(3 * NR + q) * SB + row]);
      }
    }
  }
  return true;
}

// Forward small-front item (kWaveSmall: at most one pivot block and
// kWaveSmallRows rows below it), the whole front in one CTA with its local
// vector in shared memory (xs[row * NR + q]).  What the children do not
// write is loaded before waiting for them: the right-hand side's entries of
// the front's own columns, the row maps and the first two contribution
// sources of every row (pair lists and child nodes), and the block inverse
// rows (or the diagonal block).  After the wait one round of loads brings
// the children's contribution rows; the pivot block and the contribution
// row blocks then read their inputs from shared memory.  The arithmetic and
// its order are those of fwd_gather_rows and fwd_block (code 0, then the
// contribution row blocks), so the results are the same bits.  False if a
// wait gave up.
template <typename T, int NR>
__device__ bool fwd_small(const SolveNode<T>& sn, const SolveNode<T>* sns, const int* children,
                          const int2* pairs, double* x, int ldx, int nrhs, bool scale_sqrt,
                          int* status, T* Lb, T* yb, T* red, T* xs, int* s_fail,
                          const WaveLevel& wl, int it) {
  constexpr int R = (NR + kSolveWarps - 1) / kSolveWarps;
  constexpr int RP = (SB + kWaveSmallRows + kSolveThreads - 1) / kSolveThreads;
  const int tid = threadIdx.x, r = tid % SB, cq = tid / SB;
  const int warp = tid >> 5, lane = tid & 31;
  const int m = sn.m, nelim = sn.nelim;
  T bv[16];
  if (nelim > 0) {
    if (sn.binv) {
      const T* bp = sn.binv + r * SB + cq * 16;
#pragma unroll
      for (int k = 0; k < 16; ++k) bv[k] = bp[k];
    } else {
      prefetch_diag_block(sn, 0, nelim, Lb);
    }
  }
  // rows tid + j * kSolveThreads: the right-hand side part into xs, the
  // first two contribution sources; delayed entries and further sources
  // are looked up after the wait
  const T* src0[RP];
  const T* src1[RP];
  int m0[RP], m1[RP], kn[RP], k1[RP], dl[RP];
#pragma unroll
  for (int j = 0; j < RP; ++j) {
    const int i = tid + j * kSolveThreads;
    src0[j] = src1[j] = nullptr;
    m0[j] = m1[j] = 0;
    kn[j] = k1[j] = 0;
    dl[j] = -1;
    if (i >= m) continue;
    const int pos = (i < sn.n) ? sn.opos[i] : i;
    int P = -1;
    if (pos < sn.ncol) {
#pragma unroll
      for (int q = 0; q < NR; ++q)
        xs[i * NR + q] = (q < nrhs) ? (T)x[(int64_t)q * ldx + sn.sptr0 + pos] : T(0);
      P = pos;
    } else {
#pragma unroll
      for (int q = 0; q < NR; ++q) xs[i * NR + q] = T(0);
      if (pos < sn.ncol + sn.ndelay_in) dl[j] = pos - sn.ncol;
      else P = pos - sn.ndelay_in;
    }
    if (P >= 0) {
      kn[j] = sn.gp[P];
      k1[j] = sn.gp[P + 1];
      if (kn[j] < k1[j]) {
        const int2 pr = pairs[kn[j]++];
        src0[j] = sns[pr.x].xloc + sns[pr.x].n + pr.y;
        m0[j] = sns[pr.x].m;
      }
      if (kn[j] < k1[j]) {
        const int2 pr = pairs[kn[j]++];
        src1[j] = sns[pr.x].xloc + sns[pr.x].n + pr.y;
        m1[j] = sns[pr.x].m;
      }
    }
  }
  // the children's contribution rows (and delayed entries) are final once
  // every item of theirs has finished
  bool ok = true;
  for (int ci = sn.child_beg; ci < sn.child_end && ok; ++ci) {
    const SolveNode<T>& cn = sns[children[ci]];
    ok = wave_wait_count(wave_finished(cn), cn.nitf, status, s_fail);
  }
  if (!ok) {
    if (nelim > 0 && !sn.binv) cp_async_wait_all();
    return false;
  }
  wave_stamp(wl, it, 1);
#pragma unroll
  for (int j = 0; j < RP; ++j) {
    const int i = tid + j * kSolveThreads;
    if (i >= m) continue;
    T v[NR];
#pragma unroll
    for (int q = 0; q < NR; ++q) v[q] = xs[i * NR + q];
    if (dl[j] >= 0) {
      const int k = dl[j];
      for (int ci = sn.child_beg; ci < sn.child_end; ++ci) {
        const SolveNode<T>& cn = sns[children[ci]];
        const int nd = cn.n - cn.nelim;
        if (k >= cn.doff && k < cn.doff + nd) {
          const T* src = cn.xloc + cn.nelim + (k - cn.doff);
#pragma unroll
          for (int q = 0; q < NR; ++q)
            if (q < nrhs) v[q] = __ldcg(src + (int64_t)q * cn.m);
          break;
        }
      }
    }
    if (src0[j]) {
#pragma unroll
      for (int q = 0; q < NR; ++q)
        if (q < nrhs) v[q] += __ldcg(src0[j] + (int64_t)q * m0[j]);
    }
    if (src1[j]) {
#pragma unroll
      for (int q = 0; q < NR; ++q)
        if (q < nrhs) v[q] += __ldcg(src1[j] + (int64_t)q * m1[j]);
    }
    for (int k = kn[j]; k < k1[j]; ++k) {
      const int2 pr = pairs[k];
      const SolveNode<T>& cn = sns[pr.x];
      const T* src = cn.xloc + cn.n + pr.y;
#pragma unroll
      for (int q = 0; q < NR; ++q)
        if (q < nrhs) v[q] += __ldcg(src + (int64_t)q * cn.m);
    }
#pragma unroll
    for (int q = 0; q < NR; ++q) xs[i * NR + q] = v[q];
  }
  __syncthreads();
  if (nelim > 0) {
    const int rows = nelim;
    if (sn.binv) {
      // y = L_bb^{-1} b: the products of the block inverse's row r over
      // column quarter cq, the quarters added in order
      for (int e = tid; e < SB * NR; e += kSolveThreads) {
        const int row = e / NR, q = e % NR;
        yb[row * NR + q] = (q < nrhs && row < rows) ? xs[row * NR + q] : T(0);
      }
      __syncthreads();
      T acc[NR];
#pragma unroll
      for (int q = 0; q < NR; ++q) acc[q] = T(0);
      if (cq * 16 < rows && (r & ~31) < rows) {
#pragma unroll
        for (int k = 0; k < 16; ++k)
#pragma unroll
          for (int q = 0; q < NR; ++q) acc[q] += bv[k] * yb[(cq * 16 + k) * NR + q];
      }
#pragma unroll
      for (int q = 0; q < NR; ++q) red[(cq * NR + q) * SB + r] = acc[q];
      __syncthreads();
      for (int e = tid; e < SB * NR; e += kSolveThreads) {
        const int row = e % SB, q = e / SB;
        if (row < rows && q < nrhs) {
          const T y = red[q * SB + row] + red[(NR + q) * SB + row] + red[(2 * NR + q) * SB + row] +
                      red[(3 * NR + q) * SB + row];
          xs[row * NR + q] = y;
          sn.xloc[(int64_t)q * m + row] = y;
          double v = (double)y;
          if (scale_sqrt) v *= sqrt(sn.D[2 * row]);
          x[(int64_t)q * ldx + sn.perm[row]] = v;
        }
      }
    } else {
      T xr[R][2];
#pragma unroll
      for (int rr = 0; rr < R; ++rr) {
        const int q = warp + rr * kSolveWarps;
#pragma unroll
        for (int g = 0; g < 2; ++g) {
          const int row = lane + 32 * g;
          xr[rr][g] = (q < nrhs && q < NR && row < rows) ? xs[row * NR + q] : T(0);
        }
      }
      cp_async_wait_all();
      __syncthreads();
      if (warp < nrhs) solve_in_regs<T, R, true>(rows, Lb, xr);
#pragma unroll
      for (int rr = 0; rr < R; ++rr) {
        const int q = warp + rr * kSolveWarps;
#pragma unroll
        for (int g = 0; g < 2; ++g) {
          const int row = lane + 32 * g;
          if (q < nrhs && q < NR && row < rows) {
            xs[row * NR + q] = xr[rr][g];
            sn.xloc[(int64_t)q * m + row] = xr[rr][g];
            double v = (double)xr[rr][g];
            if (scale_sqrt) v *= sqrt(sn.D[2 * row]);
            x[(int64_t)q * ldx + sn.perm[row]] = v;
          }
        }
      }
    }
    __syncthreads();
    if (tid == 0) st_release(&sn.flag[0], 1);
  }
  if (nelim >= m) return true;
  // the contribution rows: x_C -= L21 y, 64-row blocks (thread (r, cq): row
  // r, columns [16 cq, 16 cq + 16) of the pivot block), y staged once
  const int jb = nelim;
  for (int e = tid; e < SB * NR; e += kSolveThreads) {
    const int c = e % SB, q = e / SB;
    yb[c * NR + q] = (c < jb && q < nrhs) ? xs[c * NR + q] : T(0);
  }
  __syncthreads();
  for (int r0 = nelim; r0 < m; r0 += SB) {
    const int rows = min(SB, m - r0);
    T lv[16];
    {
      const T* Lp = sn.L + (int64_t)(cq * 16) * sn.ld + r0 + r;
#pragma unroll
      for (int k = 0; k < 16; ++k)
        lv[k] = (r < rows && cq * 16 + k < jb) ? Lp[(int64_t)k * sn.ld] : T(0);
    }
    T acc[NR];
#pragma unroll
    for (int q = 0; q < NR; ++q) acc[q] = T(0);
    if (cq * 16 < jb && (r & ~31) < rows) {
#pragma unroll
      for (int k = 0; k < 16; ++k)
#pragma unroll
        for (int q = 0; q < NR; ++q) acc[q] += lv[k] * yb[(cq * 16 + k) * NR + q];
    }
#pragma unroll
    for (int q = 0; q < NR; ++q) red[(cq * NR + q) * SB + r] = acc[q];
    __syncthreads();
    for (int e = tid; e < SB * NR; e += kSolveThreads) {
      const int row = e % SB, q = e / SB;
      if (row < rows && q < nrhs)
        sn.xloc[(int64_t)q * m + r0 + row] =
            xs[(r0 + row) * NR + q] - (red[q * SB + row] + red[(NR + q) * SB + row] +
                                       red[(2 * NR + q) * SB + row] +
                                       red[(3 * NR + q) * SB + row]);
    }
    __syncthreads();
  }
  return true;
}

// Forward pass over the whole tree (item list and waits: see WaveLevel).
template <typename T, int NR, int CPS>
__global__ void __launch_bounds__(kSolveThreads, CPS)
    k_fwd_tree(const SolveNode<T>* sns, const int* children, const int2* pairs, WaveLevel wl,
               int nrhs, double* x, int ldx, bool scale_sqrt, int* status) {
  extern __shared__ __align__(16) unsigned char solve_smem[];
  T* Lb = reinterpret_cast<T*>(solve_smem);
  T* yb = Lb + SB * LDB;
  T* red = yb + SB * NR;
  T* xs = red + 4 * NR * 64;  // a small front's local vector
  __shared__ int s_item, s_fail;
  for (;;) {
    const int it = wave_next(wl, &s_item);
    if (it >= wl.nitems) break;
    wave_stamp(wl, it, 0);
    const int2 w = wl.items[it];
    if (wl.active && !wl.active[wl.front_group[w.x]]) {
      // a row group the refinement no longer solves for: a whole tree that
      // no other item waits for
      wave_stamp(wl, it, 1);
      wave_stamp(wl, it, 2);
      continue;
    }
    const SolveNode<T>& sn = sns[w.x];
    const int code = w.y;
    bool ok = true;
    if (code == kWaveSmall) {
      ok = fwd_small<T, NR>(sn, sns, children, pairs, x, ldx, nrhs, scale_sqrt, status, Lb, yb,
                            red, xs, &s_fail, wl, it);
      if (ok) wave_signal(wave_finished(sn), nullptr);
    } else if (code >= kWaveGather) {
      // the children's contribution rows (and delayed entries) are final
      // once every item of theirs has finished
      for (int ci = sn.child_beg; ci < sn.child_end && ok; ++ci) {
        const SolveNode<T>& cn = sns[children[ci]];
        ok = wave_wait_count(wave_finished(cn), cn.nitf, status, &s_fail);
      }
      if (!ok) continue;
      wave_stamp(wl, it, 1);
      {
        const int g0 = (code - kWaveGather) * kWaveGatherRows;
        fwd_gather_rows<T, NR>(sn, sns, children, pairs, x, ldx, nrhs, g0,
                        min(sn.m, g0 + kWaveGatherRows));
        wave_signal(wave_gathered(sn), wave_finished(sn));
      }
    } else {
      ok = wave_wait_count(wave_gathered(sn), sn.ngat, status, &s_fail);
      if (ok)
        ok = fwd_block<T, NR>(sn, code, nrhs, x, ldx, scale_sqrt, status, Lb, yb, red, &s_fail,
                              wl, it);
      if (ok) wave_signal(wave_finished(sn), nullptr);
    }
    wave_stamp(wl, it, 2);
  }
}

// Backward L21^T partial item t = b nch + c: for pivot block b, the
// products sum_i L(i, 64 b + col) x_i over the contribution rows
// [nelim + 256 c, ...) of the front (thread (col, rq): rows
// [64 rq, 64 rq + 64) of the chunk), the four row groups added in order,
// into l21p[b][c][col][q].  The rows' values (gathered, from L2) are staged
// in xs (256 NR values).
template <typename T, int NR>
__device__ void bwd_l21_item(const SolveNode<T>& sn, int t, int nrhs, T* xs, T* red) {
  static_assert(kWaveL21Rows * NR <= SB * LDB, "the staged rows fit the diagonal block's space");
  static_assert(kWaveL21Rows == 4 * 64, "four row groups of 64 per chunk");
  const int b = t / sn.nch, c = t % sn.nch;
  const int m = sn.m, nelim = sn.nelim;
  const int c0 = b * SB, jb = min(SB, nelim - c0);
  const int R0 = nelim + c * kWaveL21Rows, nr = min(kWaveL21Rows, m - R0);
  const int tid = threadIdx.x, col = tid % SB, rq = tid / SB;
  for (int e = tid; e < kWaveL21Rows * NR; e += kSolveThreads) {
    const int rr = e % kWaveL21Rows, q = e / kWaveL21Rows;
    xs[rr * NR + q] = (rr < nr && q < nrhs) ? __ldcg(&sn.xloc[(int64_t)q * m + R0 + rr]) : T(0);
  }
  __syncthreads();
  T acc[NR];
#pragma unroll
  for (int q = 0; q < NR; ++q) acc[q] = T(0);
  const T* Lp = sn.L + (int64_t)(c0 + col) * sn.ld + R0 + rq * 64;
  // two batches of 32 loads in flight: the item is bound by their latency
  for (int kb = 0; kb < 64; kb += 32) {
    // warp-uniform: a warp's columns past the block, or a batch of rows
    // past the chunk, hold zeros of L
    if ((col & ~31) >= jb || rq * 64 + kb >= nr) continue;
    T lv[32];
#pragma unroll
    for (int k = 0; k < 32; ++k)
      lv[k] = (col < jb && rq * 64 + kb + k < nr) ? Lp[kb + k] : T(0);
#pragma unroll
    for (int k = 0; k < 32; ++k)
#pragma unroll
      for (int q = 0; q < NR; ++q) acc[q] += lv[k] * xs[(rq * 64 + kb + k) * NR + q];
  }
#pragma unroll
  for (int q = 0; q < NR; ++q) red[(rq * NR + q) * SB + col] = acc[q];
  __syncthreads();
  T* out = sn.l21p + (size_t)(b * sn.nch + c) * SB * kSolveRhs;
  for (int e = tid; e < SB * NR; e += kSolveThreads) {
    const int cc = e % SB, q = e / SB;
    out[cc * kSolveRhs + q] = red[q * SB + cc] + red[(NR + q) * SB + cc] +
                              red[(2 * NR + q) * SB + cc] + red[(3 * NR + q) * SB + cc];
  }
}

// Backward block item for pivot block b: x_b -= L21(:, b)^T x(rows below
// the pivots), from the block's partial items (their sums in chunk order)
// or, for a front without them (a small front taken whole), over its
// contribution rows here; then x_b -= sum_{j > b} L(j, b)^T y_j as the
// flags of the pivot blocks j arrive (thread (c, rq): column c, rows
// [16 rq, 16 rq + 16) of each 64-row tile), the four row quarters added in
// shared memory, L_bb^T solved in registers, y written to the local vector
// and to x, and the flag set.  False if a wait gave up.
template <typename T, int NR>
__device__ bool bwd_block(const SolveNode<T>& sn, int b, int nrhs, double* x, int ldx,
                          int* status, T* Lb, T* yb, T* red, int* s_fail, const WaveLevel& wl,
                          int it) {
  constexpr int R = (NR + kSolveWarps - 1) / kSolveWarps;
  const int tid = threadIdx.x, c = tid % SB, rq = tid / SB;
  const int warp = tid >> 5, lane = tid & 31;
  const int m = sn.m, nelim = sn.nelim;
  const int c0 = b * SB, jb = min(SB, nelim - c0);
  T bv[16];  // with inverses: column c, rows [16 rq, 16 rq + 16) of the block's
  if (sn.binv) {
    const T* bp = sn.binv + (size_t)b * SB * SB + (rq * 16) * SB + c;
#pragma unroll
    for (int k = 0; k < 16; ++k) bv[k] = bp[k * SB];
  } else {
    prefetch_diag_block(sn, c0, jb, Lb);
  }
  // the block's gathered values (D^{-1} applied), final before any wait
  T own[R][2];
#pragma unroll
  for (int rr = 0; rr < R; ++rr) {
    const int q = warp + rr * kSolveWarps;
#pragma unroll
    for (int g = 0; g < 2; ++g) {
      const int col = lane + 32 * g;
      own[rr][g] = (q < nrhs && q < NR && col < jb) ? __ldcg(&sn.xloc[(int64_t)q * m + c0 + col])
                                                    : T(0);
    }
  }
  T acc[NR];
#pragma unroll
  for (int q = 0; q < NR; ++q) acc[q] = T(0);
  bool ok = true;
  if (sn.nch > 0) {
    ok = wave_wait_count(wave_l21done(sn, b), sn.nch, status, s_fail);
    if (ok && rq == 0) {
      const T* pp = sn.l21p + (size_t)b * sn.nch * SB * kSolveRhs + c * kSolveRhs;
      for (int k = 0; k < sn.nch; ++k)
#pragma unroll
        for (int q = 0; q < NR; ++q)
          if (q < nrhs) acc[q] += __ldcg(pp + (size_t)k * SB * kSolveRhs + q);
    }
  } else {
    // the contribution rows, 64-row tiles
    for (int R0 = nelim; R0 < m; R0 += SB) {
      const int nr = min(SB, m - R0);
      T lv[16];
      {
        const T* Lp = sn.L + (int64_t)(c0 + c) * sn.ld + R0 + rq * 16;
#pragma unroll
        for (int k = 0; k < 16; ++k) lv[k] = (c < jb && rq * 16 + k < nr) ? Lp[k] : T(0);
      }
      for (int e = tid; e < SB * NR; e += kSolveThreads) {
        const int rr = e % SB, q = e / SB;
        yb[rr * NR + q] =
            (rr < nr && q < nrhs) ? __ldcg(&sn.xloc[(int64_t)q * m + R0 + rr]) : T(0);
      }
      __syncthreads();
      // warp-uniform skip of columns past the block or rows past the tile
      if ((c & ~31) < jb && rq * 16 < nr) {
#pragma unroll
        for (int k = 0; k < 16; ++k)
#pragma unroll
          for (int q = 0; q < NR; ++q) acc[q] += lv[k] * yb[(rq * 16 + k) * NR + q];
      }
      __syncthreads();
    }
  }
  // the pivot blocks sn.nblk-1 .. b+1, as their flags arrive
  for (int j = sn.nblk - 1; j > b && ok; --j) {
    const int R0 = j * SB, nr = min(SB, nelim - R0);
    T lv[16];
    {
      const T* Lp = sn.L + (int64_t)(c0 + c) * sn.ld + R0 + rq * 16;
#pragma unroll
      for (int k = 0; k < 16; ++k) lv[k] = (c < jb && rq * 16 + k < nr) ? Lp[k] : T(0);
    }
    ok = wave_wait(&sn.flag[j], status, s_fail);
    if (!ok) break;
    for (int e = tid; e < SB * NR; e += kSolveThreads) {
      const int rr = e % SB, q = e / SB;
      // another CTA wrote the pivot blocks' values: read them from L2
      yb[rr * NR + q] = (rr < nr && q < nrhs) ? __ldcg(&sn.xloc[(int64_t)q * m + R0 + rr]) : T(0);
    }
    __syncthreads();
    if ((c & ~31) < jb && rq * 16 < nr) {
#pragma unroll
      for (int k = 0; k < 16; ++k)
#pragma unroll
        for (int q = 0; q < NR; ++q) acc[q] += lv[k] * yb[(rq * 16 + k) * NR + q];
    }
    __syncthreads();
  }
  if (!ok) {
    if (!sn.binv) cp_async_wait_all();
    return false;
  }
  wave_stamp(wl, it, 1);
#pragma unroll
  for (int q = 0; q < NR; ++q) red[(rq * NR + q) * SB + c] = acc[q];
  __syncthreads();
  if (sn.binv) {
    // y = L_bb^{-T} (b - sum): the right-hand side into yb, then column c
    // of the block inverse times it over row quarter rq, quarters in order
#pragma unroll
    for (int rr = 0; rr < R; ++rr) {
      const int q = warp + rr * kSolveWarps;
#pragma unroll
      for (int g = 0; g < 2; ++g) {
        const int col = lane + 32 * g;
        if (q < NR)
          yb[col * NR + q] = (q < nrhs && col < jb)
                                 ? own[rr][g] - (red[q * SB + col] + red[(NR + q) * SB + col] +
                                                 red[(2 * NR + q) * SB + col] +
                                                 red[(3 * NR + q) * SB + col])
                                 : T(0);
      }
    }
    __syncthreads();
#pragma unroll
    for (int q = 0; q < NR; ++q) acc[q] = T(0);
    if ((c & ~31) < jb && rq * 16 < jb) {
#pragma unroll
      for (int k = 0; k < 16; ++k)
#pragma unroll
        for (int q = 0; q < NR; ++q) acc[q] += bv[k] * yb[(rq * 16 + k) * NR + q];
    }
#pragma unroll
    for (int q = 0; q < NR; ++q) red[(rq * NR + q) * SB + c] = acc[q];
    __syncthreads();
    for (int e = tid; e < SB * NR; e += kSolveThreads) {
      const int col = e % SB, q = e / SB;
      if (col < jb && q < nrhs) {
        const T y = red[q * SB + col] + red[(NR + q) * SB + col] + red[(2 * NR + q) * SB + col] +
                    red[(3 * NR + q) * SB + col];
        sn.xloc[(int64_t)q * m + c0 + col] = y;
        x[(int64_t)q * ldx + sn.perm[c0 + col]] = (double)y;
      }
    }
    __syncthreads();
    if (tid == 0) st_release(&sn.flag[b], 1);
    return true;
  }
  T xr[R][2];
#pragma unroll
  for (int rr = 0; rr < R; ++rr) {
    const int q = warp + rr * kSolveWarps;
#pragma unroll
    for (int g = 0; g < 2; ++g) {
      const int col = lane + 32 * g;
      T v = T(0);
      if (q < nrhs && q < NR && col < jb)
        v = own[rr][g] - (red[q * SB + col] + red[(NR + q) * SB + col] +
                          red[(2 * NR + q) * SB + col] + red[(3 * NR + q) * SB + col]);
      xr[rr][g] = v;
    }
  }
  cp_async_wait_all();
  __syncthreads();
  if (warp < nrhs) solve_in_regs<T, R, false>(jb, Lb, xr);
#pragma unroll
  for (int rr = 0; rr < R; ++rr) {
    const int q = warp + rr * kSolveWarps;
#pragma unroll
    for (int g = 0; g < 2; ++g) {
      const int col = lane + 32 * g;
      if (q < nrhs && q < NR && col < jb) {
        sn.xloc[(int64_t)q * m + c0 + col] = xr[rr][g];
        x[(int64_t)q * ldx + sn.perm[c0 + col]] = (double)xr[rr][g];
      }
    }
  }
  __syncthreads();
  // the release orders every thread's writes above (ordered before it by
  // the barrier) before the flag, for any CTA that acquires the flag
  if (tid == 0) st_release(&sn.flag[b], 1);
  return true;
}

// Backward small-front item, the whole front in one CTA with its local
// vector in shared memory (xs[row * NR + q]): the pivot rows' entries of x
// (this front's own, written by no other item of the pass) with their D^{-1}
// applied, and the block inverse (or the diagonal block), are loaded before
// waiting for the parent; after it one round of loads brings the rows below
// the pivots, solved at the ancestors.  Then x_b -= L21^T x_C over the
// contribution rows and the unit triangle, with the arithmetic and order of
// bwd_gather_rows and bwd_block (code 0, no partial items), so the results
// are the same bits.  False if a wait gave up.
template <typename T, int NR>
__device__ bool bwd_small(const SolveNode<T>& sn, const SolveNode<T>* sns, int nrhs, double* x,
                          int ldx, int diag_mode, int* status, T* Lb, T* yb, T* red, T* xs,
                          int* s_fail, const WaveLevel& wl, int it) {
  constexpr int R = (NR + kSolveWarps - 1) / kSolveWarps;
  constexpr int RP = (SB + kWaveSmallRows + kSolveThreads - 1) / kSolveThreads;
  const int tid = threadIdx.x, c = tid % SB, rq = tid / SB;
  const int warp = tid >> 5, lane = tid & 31;
  const int m = sn.m, nelim = sn.nelim, jb = min(SB, nelim);
  T bv[16];
  if (nelim > 0) {
    if (sn.binv) {
      const T* bp = sn.binv + (rq * 16) * SB + c;
#pragma unroll
      for (int k = 0; k < 16; ++k) bv[k] = bp[k * SB];
    } else {
      prefetch_diag_block(sn, 0, jb, Lb);
    }
  }
  int later[RP];  // x position of a row below the pivots, read after the wait
#pragma unroll
  for (int j = 0; j < RP; ++j) {
    const int i = tid + j * kSolveThreads;
    later[j] = -1;
    if (i >= m) continue;
    const int src = (i < sn.n) ? sn.perm[i] : sn.rows[sn.ncol + i - sn.n];
    if (i >= nelim) {
      later[j] = src;
      continue;
    }
    int src2 = -1;
    double ca = 1.0, cb = 0.0;
    if (diag_mode == 2) {
      ca = sqrt(sn.D[2 * i]);
    } else if (diag_mode == 1) {
      const double di = sn.D[2 * i];
      if (isinf(di)) {
        src2 = sn.perm[i - 1];
        ca = sn.D[2 * i + 1];
        cb = sn.D[2 * (i - 1) + 1];
      } else if (i + 1 < nelim && isinf(sn.D[2 * i + 2])) {
        src2 = sn.perm[i + 1];
        ca = di;
        cb = sn.D[2 * i + 1];
      } else {
        ca = di;
      }
    }
#pragma unroll
    for (int q = 0; q < NR; ++q) {
      T t = T(0);
      if (q < nrhs) {
        const double v = __ldcg(&x[(int64_t)q * ldx + src]);
        const double w = src2 >= 0 ? __ldcg(&x[(int64_t)q * ldx + src2]) : 0.0;
        double rv;
        if (src2 < 0) rv = (diag_mode == 0) ? v : ca * v;
        else if (isinf(sn.D[2 * i])) rv = cb * w + ca * v;
        else rv = ca * v + cb * w;
        t = (T)rv;
        sn.xloc[(int64_t)q * m + i] = t;
      }
      xs[i * NR + q] = t;
    }
  }
  // the rows below the pivots are solved at the ancestors, which are final
  // once the parent has finished (it waited for its own parent)
  bool ok = true;
  if (sn.parent >= 0) {
    const SolveNode<T>& pn = sns[sn.parent];
    ok = wave_wait_count(wave_finished(pn), pn.nitb, status, s_fail);
  }
  if (!ok) {
    if (nelim > 0 && !sn.binv) cp_async_wait_all();
    return false;
  }
  wave_stamp(wl, it, 1);
#pragma unroll
  for (int j = 0; j < RP; ++j) {
    const int i = tid + j * kSolveThreads;
    if (later[j] < 0) continue;
#pragma unroll
    for (int q = 0; q < NR; ++q) {
      T t = T(0);
      if (q < nrhs) {
        t = (T)__ldcg(&x[(int64_t)q * ldx + later[j]]);
        sn.xloc[(int64_t)q * m + i] = t;
      }
      xs[i * NR + q] = t;
    }
  }
  __syncthreads();
  if (nelim == 0) return true;
  T own[R][2];
#pragma unroll
  for (int rr = 0; rr < R; ++rr) {
    const int q = warp + rr * kSolveWarps;
#pragma unroll
    for (int g = 0; g < 2; ++g) {
      const int col = lane + 32 * g;
      own[rr][g] = (q < nrhs && q < NR && col < jb) ? xs[col * NR + q] : T(0);
    }
  }
  T acc[NR];
#pragma unroll
  for (int q = 0; q < NR; ++q) acc[q] = T(0);
  for (int R0 = nelim; R0 < m; R0 += SB) {
    const int nr = min(SB, m - R0);
    T lv[16];
    {
      const T* Lp = sn.L + (int64_t)c * sn.ld + R0 + rq * 16;
#pragma unroll
      for (int k = 0; k < 16; ++k) lv[k] = (c < jb && rq * 16 + k < nr) ? Lp[k] : T(0);
    }
    for (int e = tid; e < SB * NR; e += kSolveThreads) {
      const int rr = e % SB, q = e / SB;
      yb[rr * NR + q] = (rr < nr && q < nrhs) ? xs[(R0 + rr) * NR + q] : T(0);
    }
    __syncthreads();
    if ((c & ~31) < jb && rq * 16 < nr) {
#pragma unroll
      for (int k = 0; k < 16; ++k)
#pragma unroll
        for (int q = 0; q < NR; ++q) acc[q] += lv[k] * yb[(rq * 16 + k) * NR + q];
    }
    __syncthreads();
  }
  wave_stamp(wl, it, 1);
#pragma unroll
  for (int q = 0; q < NR; ++q) red[(rq * NR + q) * SB + c] = acc[q];
  __syncthreads();
  if (sn.binv) {
#pragma unroll
    for (int rr = 0; rr < R; ++rr) {
      const int q = warp + rr * kSolveWarps;
#pragma unroll
      for (int g = 0; g < 2; ++g) {
        const int col = lane + 32 * g;
        if (q < NR)
          yb[col * NR + q] = (q < nrhs && col < jb)
                                 ? own[rr][g] - (red[q * SB + col] + red[(NR + q) * SB + col] +
                                                 red[(2 * NR + q) * SB + col] +
                                                 red[(3 * NR + q) * SB + col])
                                 : T(0);
      }
    }
    __syncthreads();
#pragma unroll
    for (int q = 0; q < NR; ++q) acc[q] = T(0);
    if ((c & ~31) < jb && rq * 16 < jb) {
#pragma unroll
      for (int k = 0; k < 16; ++k)
#pragma unroll
        for (int q = 0; q < NR; ++q) acc[q] += bv[k] * yb[(rq * 16 + k) * NR + q];
    }
#pragma unroll
    for (int q = 0; q < NR; ++q) red[(rq * NR + q) * SB + c] = acc[q];
    __syncthreads();
    for (int e = tid; e < SB * NR; e += kSolveThreads) {
      const int col = e % SB, q = e / SB;
      if (col < jb && q < nrhs) {
        const T y = red[q * SB + col] + red[(NR + q) * SB + col] + red[(2 * NR + q) * SB + col] +
                    red[(3 * NR + q) * SB + col];
        sn.xloc[(int64_t)q * m + col] = y;
        x[(int64_t)q * ldx + sn.perm[col]] = (double)y;
      }
    }
  } else {
    T xr[R][2];
#pragma unroll
    for (int rr = 0; rr < R; ++rr) {
      const int q = warp + rr * kSolveWarps;
#pragma unroll
      for (int g = 0; g < 2; ++g) {
        const int col = lane + 32 * g;
        T v = T(0);
        if (q < nrhs && q < NR && col < jb)
          v = own[rr][g] - (red[q * SB + col] + red[(NR + q) * SB + col] +
                            red[(2 * NR + q) * SB + col] + red[(3 * NR + q) * SB + col]);
        xr[rr][g] = v;
      }
    }
    cp_async_wait_all();
    __syncthreads();
    if (warp < nrhs) solve_in_regs<T, R, false>(jb, Lb, xr);
#pragma unroll
    for (int rr = 0; rr < R; ++rr) {
      const int q = warp + rr * kSolveWarps;
#pragma unroll
      for (int g = 0; g < 2; ++g) {
        const int col = lane + 32 * g;
        if (q < nrhs && q < NR && col < jb) {
          sn.xloc[(int64_t)q * m + col] = xr[rr][g];
          x[(int64_t)q * ldx + sn.perm[col]] = (double)xr[rr][g];
        }
      }
    }
  }
  __syncthreads();
  if (tid == 0) st_release(&sn.flag[0], 1);
  return true;
}

// Backward pass over the whole tree (item list and waits: see WaveLevel).
template <typename T, int NR, int CPS>
__global__ void __launch_bounds__(kSolveThreads, CPS)
    k_bwd_tree(const SolveNode<T>* sns, WaveLevel wl, int nrhs, double* x, int ldx, int diag_mode,
               int* status) {
  extern __shared__ __align__(16) unsigned char solve_smem[];
  T* Lb = reinterpret_cast<T*>(solve_smem);
  T* yb = Lb + SB * LDB;
  T* red = yb + SB * NR;
  T* xs = red + 4 * NR * 64;  // a small front's local vector
  __shared__ int s_item, s_fail;
  for (;;) {
    const int it = wave_next(wl, &s_item);
    if (it >= wl.nitems) break;
    wave_stamp(wl, it, 0);
    const int2 w = wl.items[it];
    if (wl.active && !wl.active[wl.front_group[w.x]]) {
      // a row group the refinement no longer solves for: a whole tree that
      // no other item waits for
      wave_stamp(wl, it, 1);
      wave_stamp(wl, it, 2);
      continue;
    }
    const SolveNode<T>& sn = sns[w.x];
    const int code = w.y;
    bool ok = true;
    if (code == kWaveSmall) {
      ok = bwd_small<T, NR>(sn, sns, nrhs, x, ldx, diag_mode, status, Lb, yb, red, xs, &s_fail,
                            wl, it);
      if (ok) wave_signal(wave_finished(sn), nullptr);
    } else if (code >= kWaveL21) {
      ok = wave_wait_count(wave_gathered(sn), sn.ngat, status, &s_fail);
      if (ok) wave_stamp(wl, it, 1);
      const int t = code - kWaveL21;
      if (ok) bwd_l21_item<T, NR>(sn, t, nrhs, Lb, red);
      if (ok) wave_signal(wave_l21done(sn, t / sn.nch), wave_finished(sn));
    } else if (code >= kWaveGather) {
      // the rows below the pivots are solved at the ancestors, which are
      // final once the parent has finished (it waited for its own parent)
      if (sn.parent >= 0) {
        const SolveNode<T>& pn = sns[sn.parent];
        ok = wave_wait_count(wave_finished(pn), pn.nitb, status, &s_fail);
      }
      if (!ok) continue;
      wave_stamp(wl, it, 1);
      const int g0 = (code - kWaveGather) * kWaveGatherRows;
      bwd_gather_rows<T, NR>(sn, x, ldx, nrhs, diag_mode, g0, min(sn.m, g0 + kWaveGatherRows));
      wave_signal(wave_gathered(sn), wave_finished(sn));
    } else {
      ok = wave_wait_count(wave_gathered(sn), sn.ngat, status, &s_fail);
      if (ok) ok = bwd_block<T, NR>(sn, code, nrhs, x, ldx, status, Lb, yb, red, &s_fail, wl, it);
      if (ok) wave_signal(wave_finished(sn), nullptr);
    }
    wave_stamp(wl, it, 2);
  }
}

// Inverse of a 64 x 64 unit lower diagonal block of the FP32 factors,
// blocks[i] = (front, block): Binv(i, j) for the block's jb x jb part, zero
// elsewhere, row-major.  64 threads; thread j forms column j by forward
// substitution in FP32, the factors' precision.
__global__ void __launch_bounds__(64) k_diag_inv(const SolveNode<float>* sns, const int2* blocks) {
  using T = float;
  __shared__ T Ls[SB][SB + 1];  // Ls[r][c] = L(r, c), strictly lower
  __shared__ T X[SB][SB + 1];
  const int2 w = blocks[blockIdx.x];
  const SolveNode<float>& sn = sns[w.x];
  const int c0 = w.y * SB, jb = min(SB, sn.nelim - c0);
  const int t = threadIdx.x;
  for (int e = t; e < SB * SB; e += blockDim.x) {
    const int r = e % SB, c = e / SB;
    Ls[r][c] = (r > c && r < jb) ? sn.L[(int64_t)(c0 + c) * sn.ld + c0 + r] : T(0);
  }
  for (int i = 0; i < SB; ++i) X[i][t] = T(0);
  __syncthreads();
  if (t < jb) {
    X[t][t] = T(1);
    for (int i = t + 1; i < jb; ++i) {
      T acc = T(0);
      for (int k = t; k < i; ++k) acc += Ls[i][k] * X[k][t];
      X[i][t] = -acc;
    }
  }
  __syncthreads();
  T* out = const_cast<T*>(sn.binv) + (size_t)w.y * SB * SB;
  for (int e = t; e < SB * SB; e += blockDim.x) out[e] = X[e / SB][e % SB];
}

inline int cdiv(int a, int b) { return (a + b - 1) / b; }

// CTAs per node of a block step: every CTA repeats the step's diagonal
// solve, so a level with many nodes gets about one wave of CTAs in total
// (one per node once the level has 152 nodes or more)
inline int cta_cap(int nn) { return std::max(1, 152 / std::max(nn, 1)); }

// call f(std::integral_constant<int, NR>) with the smallest NR in
// {1, 2, 4, 8, 16} that holds q right-hand sides
template <typename F>
void with_nr(int q, F&& f) {
  if (q <= 1) f(std::integral_constant<int, 1>());
  else if (q <= 2) f(std::integral_constant<int, 2>());
  else if (q <= 4) f(std::integral_constant<int, 4>());
  else if (q <= 8) f(std::integral_constant<int, 8>());
  else f(std::integral_constant<int, 16>());
}

}  // namespace

template <typename T>
void launch_fwd_gather(const SolveNode<T>* sn, const int* nodes, int nn, const int* children,
                       const int2* pairs, const double* x, int ldx, int nrhs, int max_m,
                       cudaStream_t s) {
  if (nn <= 0) return;
  const int gx = std::max(1, std::min(cdiv(max_m * nrhs, 256), 152));
  launch_pdl(k_fwd_gather<T>, dim3(gx, nn), 256, 0, s, sn, nodes, children, pairs, x, ldx, nrhs);
  note_launches(1);
}

// levels with at least this many nodes run FP64 block steps as solve +
// update pairs (see kStepSolve)
constexpr int kSplitNodes = 8;

// block steps: solve block st, update the rows below it; the solution goes
// straight to x (pivot order)
template <typename T>
void launch_fwd_steps(const SolveNode<T>* sn, const int* nodes, int nn, int max_nelim,
                      int max_m, int nrhs, double* x, int ldx, bool scale_sqrt, cudaStream_t s,
                      PhaseTimer* tm) {
  if (nn <= 0) return;
  const int steps = cdiv(max_nelim, SB);
  const bool split = sizeof(T) == 8 && nn >= kSplitNodes;
  with_nr(nrhs, [&](auto nrc) {
    constexpr int NR = decltype(nrc)::value;
    constexpr size_t sm = solve_smem_bytes<T, NR>();
    for (int st = 0; st < steps; ++st) {
      const int below = std::max(max_m - (st + 1) * SB, 1);  // upper bound on rows to update
      pmark(tm, kPhFwdUpdate, s);
      if (split) {
        launch_pdl(k_fwd_step<T, NR, kStepSolve>, dim3(1, nn), kSolveThreads, sm, s, sn, nodes, st,
                   nrhs, x, ldx, scale_sqrt);
        const int gx = std::max(1, std::min(cdiv(below, pass_rows<T>()), 152));
        launch_pdl(k_fwd_step<T, NR, kStepUpdate>, dim3(gx, nn), kSolveThreads, sm, s, sn, nodes,
                   st, nrhs, x, ldx, scale_sqrt);
        note_launches(2);
      } else {
        const int cap = sizeof(T) == 8 ? cta_cap(nn) : 152;
        const int gx = std::max(1, std::min(cdiv(below, pass_rows<T>()), cap));
        launch_pdl(k_fwd_step<T, NR, kStepFused>, dim3(gx, nn), kSolveThreads, sm, s, sn, nodes,
                   st, nrhs, x, ldx, scale_sqrt);
        note_launches(1);
      }
    }
  });
}

template <typename T>
void launch_bwd(const SolveNode<T>* sn, const int* nodes, int nn, double* x, int ldx, int nrhs,
                int max_m, int max_nelim, int diag_mode, bool do_bwd, cudaStream_t s,
                PhaseTimer* tm) {
  if (nn <= 0) return;
  int gx = std::max(1, std::min(cdiv(max_m * nrhs, 256), 152));
  pmark(tm, kPhBwdGather, s);
  launch_pdl(k_bwd_gather<T>, dim3(gx, nn), 256, 0, s, sn, nodes, x, ldx, nrhs, diag_mode,
             do_bwd);
  note_launches(1);
  if (!do_bwd) {
    // diagonal solve only: D^{-1} x was applied by the gather
    int gs = std::max(1, std::min(cdiv(max_nelim * nrhs, 256), 64));
    pmark(tm, kPhBwdScatter, s);
    launch_pdl(k_fwd_scatter<T>, dim3(gs, nn), 256, 0, s, sn, nodes, x, ldx, nrhs, false);
    note_launches(1);
    return;
  }
  with_nr(nrhs, [&](auto nrc) {
    constexpr int NR = decltype(nrc)::value;
    // enough CTAs for the level's widest node at the most warps per column
    // any of its nodes can use (rows below the pivots <= max_m), up to 4 per SM
    const int gw = std::max(
        1, std::min(cdiv(max_nelim, kSolveWarps / l21_warps_host(max_m)), 4 * 152));
    pmark(tm, kPhBwdL21, s);
    launch_pdl(k_bwd_l21<T, NR>, dim3(gw, nn), kSolveThreads, 0, s, sn, nodes, nrhs);
    note_launches(1);
    const int steps = cdiv(max_nelim, SB);
    const bool split = sizeof(T) == 8 && nn >= kSplitNodes;
    constexpr size_t sm = solve_smem_bytes<T, NR>();
    for (int st = steps - 1; st >= 0; --st) {
      const int left = std::max(st * SB, 1);  // columns to update
      pmark(tm, kPhBwdUpdate, s);
      if (split) {
        launch_pdl(k_bwd_step<T, NR, kStepSolve>, dim3(1, nn), kSolveThreads, sm, s, sn, nodes, st,
                   nrhs, x, ldx);
        note_launches(1);
        if (st > 0) {
          const int gx = std::max(1, std::min(cdiv(left, pass_rows<T>()), 152));
          launch_pdl(k_bwd_step<T, NR, kStepUpdate>, dim3(gx, nn), kSolveThreads, sm, s, sn,
                     nodes, st, nrhs, x, ldx);
          note_launches(1);
        }
      } else {
        const int cap = sizeof(T) == 8 ? cta_cap(nn) : 152;
        const int gx = std::max(1, std::min(cdiv(left, pass_rows<T>()), cap));
        launch_pdl(k_bwd_step<T, NR, kStepFused>, dim3(gx, nn), kSolveThreads, sm, s, sn, nodes,
                   st, nrhs, x, ldx);
        note_launches(1);
      }
    }
  });
}

// returns -51 (SSIDS_ERROR_CUDA_UNKNOWN) when the bounded wait gave up, as
// it must: nothing sets the flag
int wave_timeout_probe(int rounds) {
  int* d = nullptr;
  if (cudaMalloc(&d, 2 * sizeof(int)) != cudaSuccess) { cudaGetLastError(); return -50; }
  cudaMemset(d, 0, 2 * sizeof(int));
  k_wave_timeout_probe<<<1, 32>>>(d, (long long)std::max(rounds, 1), d + 1);
  int h = 0;
  const cudaError_t e = cudaMemcpy(&h, d + 1, sizeof(int), cudaMemcpyDeviceToHost);
  cudaFree(d);
  if (e != cudaSuccess) { cudaGetLastError(); return -51; }
  return h ? -51 : 0;
}

// persistent CTAs of a wave launch: cps per SM (each may hold an item that
// waits), never more than there are items
inline int wave_grid(int nitems, int cps) {
  static const int nsm = [] {
    int dev = 0, n = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
    return n > 0 ? n : 152;
  }();
  return std::max(1, std::min(nitems, cps * nsm));
}

// FP32 factors only (FP64 factors keep the substitution in the passes)
template <typename T>
void launch_diag_inv(const SolveNode<T>* sn, const int2* blocks, int nblocks, cudaStream_t s) {
  if (nblocks <= 0) return;
  if constexpr (std::is_same<T, float>::value) {
    k_diag_inv<<<nblocks, SB, 0, s>>>(sn, blocks);
    note_launches(1);
  }
}

template <typename T>
void launch_fwd_tree(const SolveNode<T>* sn, const int* children, const int2* pairs,
                     const WaveLevel& wl, int nrhs, double* x, int ldx, bool scale_sqrt,
                     int* status, cudaStream_t s) {
  if (wl.nitems <= 0) return;
  with_nr(nrhs, [&](auto nrc) {
    constexpr int NR = decltype(nrc)::value;
    if (wl.ctas_per_sm >= 3)
      k_fwd_tree<T, NR, 3><<<wave_grid(wl.nitems, 3), kSolveThreads, wave_smem_bytes<T, NR>(),
                             s>>>(sn, children, pairs, wl, nrhs, x, ldx, scale_sqrt, status);
    else
      k_fwd_tree<T, NR, 2><<<wave_grid(wl.nitems, 2), kSolveThreads, wave_smem_bytes<T, NR>(),
                             s>>>(sn, children, pairs, wl, nrhs, x, ldx, scale_sqrt, status);
  });
  note_launches(1);
}

template <typename T>
void launch_bwd_tree(const SolveNode<T>* sn, const WaveLevel& wl, double* x, int ldx, int nrhs,
                     int diag_mode, int* status, cudaStream_t s) {
  if (wl.nitems <= 0) return;
  with_nr(nrhs, [&](auto nrc) {
    constexpr int NR = decltype(nrc)::value;
    if (wl.ctas_per_sm >= 3)
      k_bwd_tree<T, NR, 3><<<wave_grid(wl.nitems, 3), kSolveThreads, wave_smem_bytes<T, NR>(),
                             s>>>(sn, wl, nrhs, x, ldx, diag_mode, status);
    else
      k_bwd_tree<T, NR, 2><<<wave_grid(wl.nitems, 2), kSolveThreads, wave_smem_bytes<T, NR>(),
                             s>>>(sn, wl, nrhs, x, ldx, diag_mode, status);
  });
  note_launches(1);
}

// the dynamic shared memory limit of every solve kernel instantiation; called
// before solves are enqueued (never during a stream capture)
template <typename T>
void solve_init() {
  static std::once_flag once;
  std::call_once(once, [] {
    auto set = [](auto kernel, size_t bytes) {
      cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
    };
    for (int q : {1, 2, 4, 8, 16}) {
      with_nr(q, [&](auto nrc) {
        constexpr int NR = decltype(nrc)::value;
        set(k_fwd_step<T, NR, kStepFused>, solve_smem_bytes<T, NR>());
        set(k_fwd_step<T, NR, kStepSolve>, solve_smem_bytes<T, NR>());
        set(k_fwd_step<T, NR, kStepUpdate>, solve_smem_bytes<T, NR>());
        set(k_bwd_step<T, NR, kStepFused>, solve_smem_bytes<T, NR>());
        set(k_bwd_step<T, NR, kStepSolve>, solve_smem_bytes<T, NR>());
        set(k_bwd_step<T, NR, kStepUpdate>, solve_smem_bytes<T, NR>());
        set(k_fwd_tree<T, NR, 2>, wave_smem_bytes<T, NR>());
        set(k_bwd_tree<T, NR, 2>, wave_smem_bytes<T, NR>());
        set(k_fwd_tree<T, NR, 3>, wave_smem_bytes<T, NR>());
        set(k_bwd_tree<T, NR, 3>, wave_smem_bytes<T, NR>());
      });
    }
  });
}

#define INST(T)                                                                                \
  template void solve_init<T>();                                                               \
  template void launch_fwd_gather<T>(const SolveNode<T>*, const int*, int, const int*,         \
                                     const int2*, const double*, int, int, int, cudaStream_t); \
  template void launch_fwd_steps<T>(const SolveNode<T>*, const int*, int, int, int, int,       \
                                    double*, int, bool, cudaStream_t, PhaseTimer*);            \
  template void launch_bwd<T>(const SolveNode<T>*, const int*, int, double*, int, int, int, int, \
                              int, bool, cudaStream_t, PhaseTimer*);                           \
  template void launch_fwd_tree<T>(const SolveNode<T>*, const int*, const int2*,               \
                                   const WaveLevel&, int, double*, int, bool, int*,            \
                                   cudaStream_t);                                              \
  template void launch_bwd_tree<T>(const SolveNode<T>*, const WaveLevel&, double*, int, int,   \
                                   int, int*, cudaStream_t);                                   \
  template void launch_diag_inv<T>(const SolveNode<T>*, const int2*, int, cudaStream_t);
INST(double)
INST(float)
#undef INST

}  // namespace ssids300
