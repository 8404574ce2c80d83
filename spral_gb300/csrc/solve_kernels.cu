// Forward, diagonal and backward solves over the assembly tree, level by
// level, many right-hand sides at once (the reference GPU path solves one
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
// are blocked by 64 rows.  A diagonal-block solve stages the block in shared
// memory and gives each right-hand side its own warp (values in registers,
// the pivot row broadcast by shuffles), so the serial chains of different
// right-hand sides run on different SM sub-partitions.  One kernel per block
// step applies the block's update (rows below it in the forward pass,
// columns left of it in the backward pass) and, in the CTA that owns the
// next block's rows or columns, solves that next diagonal block right after
// updating it: one launch per block step instead of two.  Arithmetic is in
// the factor precision T; the number of right-hand sides per pass NR is a
// template parameter so that no work is spent on absent columns.
#include <type_traits>

#include "ssids_gpu.cuh"

namespace ssids300 {

namespace {

constexpr int SB = kSolveBlk;

// gather b and the children's local vectors into the node's local vector
// (the whole CTA works on one node)
template <typename T>
__device__ __forceinline__ void fwd_gather_node(const SolveNode<T>& sn, const SolveNode<T>* sns,
                                                const int* children, const double* x, int ldx,
                                                int nrhs) {
  const int m = sn.m;
  T* xo = sn.xorig;
  for (int e = threadIdx.x; e < m * nrhs; e += blockDim.x) {
    const int i = e % m, r = e / m;
    xo[e] = (i < sn.ncol) ? (T)x[(int64_t)r * ldx + sn.sptr0 + i] : T(0);
  }
  __syncthreads();
  for (int ci = sn.child_beg; ci < sn.child_end; ++ci) {
    const SolveNode<T> cn = sns[children[ci]];
    const int nd = cn.n - cn.nelim;
    const int tot = nd + cn.cm;
    for (int e = threadIdx.x; e < tot * nrhs; e += blockDim.x) {
      const int k = e % tot, r = e / tot;
      int pos;
      T v;
      if (k < nd) {
        pos = sn.ncol + cn.doff + k;
        v = cn.xloc[(int64_t)r * cn.m + cn.nelim + k];
      } else {
        const int ic = k - nd;
        const int Q = cn.rdir[ic];
        pos = (Q < sn.ncol) ? Q : Q + sn.ndelay_in;
        v = cn.xloc[(int64_t)r * cn.m + cn.n + ic];
      }
      xo[(int64_t)r * m + pos] += v;
    }
    __syncthreads();
  }
  for (int e = threadIdx.x; e < m * nrhs; e += blockDim.x) {
    const int i = e % m, r = e / m;
    sn.xloc[e] = (i < sn.n) ? xo[(int64_t)r * m + sn.opos[i]] : xo[e];
  }
}

// stage the jb x jb diagonal block (strictly lower part) into shared memory;
// every thread issues all of its loads before the first store so that the
// global-memory latency is paid once, not once per element
constexpr int kSolveThreads = 256;
constexpr int kSolveWarps = kSolveThreads / 32;
template <typename T>
__device__ __forceinline__ void load_diag_block(const SolveNode<T>& sn, int j0, int jb,
                                                T (*Lb)[SB + 1]) {
  constexpr int PER = SB * SB / kSolveThreads;  // 16
  T v[PER];
#pragma unroll
  for (int k = 0; k < PER; ++k) {
    const int e = threadIdx.x + k * kSolveThreads;
    const int c = e / SB, r = e % SB;
    v[k] = (r > c && r < jb && c < jb) ? sn.L[(int64_t)(j0 + c) * sn.ld + j0 + r] : T(0);
  }
#pragma unroll
  for (int k = 0; k < PER; ++k) {
    const int e = threadIdx.x + k * kSolveThreads;
    Lb[e / SB][e % SB] = v[k];
  }
}

// Unit lower (FWD) or unit upper L^T (!FWD) triangular solve of rows
// [j0, j0+jb) of xloc in place, with the block staged in Lb (Lb[c][r] =
// L(j0+r, j0+c), zero on and above the diagonal).  Warp w solves the
// right-hand sides w, w + 8, ...; lane l holds rows l and l + 32.  The
// caller has synchronised the CTA after staging Lb; nothing follows.
template <typename T, int NR, bool FWD>
__device__ __forceinline__ void diag_block_solve(const SolveNode<T>& sn, int j0, int jb,
                                                 int nrhs, T (*Lb)[SB + 1]) {
  constexpr int R = (NR + kSolveWarps - 1) / kSolveWarps;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (warp >= nrhs) return;
  T x0[R], x1[R];
#pragma unroll
  for (int r = 0; r < R; ++r) {
    const int q = warp + r * kSolveWarps;
    x0[r] = (q < nrhs && lane < jb) ? sn.xloc[(int64_t)q * sn.m + j0 + lane] : T(0);
    x1[r] = (q < nrhs && lane + 32 < jb) ? sn.xloc[(int64_t)q * sn.m + j0 + lane + 32] : T(0);
  }
  if (FWD) {
    for (int k = 0; k < jb - 1; ++k) {
      const T l0 = Lb[k][lane], l1 = Lb[k][lane + 32];
#pragma unroll
      for (int r = 0; r < R; ++r) {
        const T xk = (k < 32) ? __shfl_sync(0xffffffffu, x0[r], k & 31)
                              : __shfl_sync(0xffffffffu, x1[r], k & 31);
        x0[r] -= l0 * xk;
        x1[r] -= l1 * xk;
      }
    }
  } else {
    // (L^T y)_r = y_r + sum_{c > r} L(c, r) y_c ; process c from the bottom.
    // L(c, r) = Lb[r][c] is zero unless c > r, so no lane masks are needed.
    for (int c = jb - 1; c > 0; --c) {
      const T l0 = Lb[lane][c], l1 = Lb[lane + 32][c];
#pragma unroll
      for (int r = 0; r < R; ++r) {
        const T yc = (c < 32) ? __shfl_sync(0xffffffffu, x0[r], c & 31)
                              : __shfl_sync(0xffffffffu, x1[r], c & 31);
        x0[r] -= l0 * yc;
        x1[r] -= l1 * yc;
      }
    }
  }
#pragma unroll
  for (int r = 0; r < R; ++r) {
    const int q = warp + r * kSolveWarps;
    if (q < nrhs && lane < jb) sn.xloc[(int64_t)q * sn.m + j0 + lane] = x0[r];
    if (q < nrhs && lane + 32 < jb) sn.xloc[(int64_t)q * sn.m + j0 + lane + 32] = x1[r];
  }
}

// ---- forward ----
// gather (one CTA per node), then the first diagonal block
template <typename T, int NR>
__global__ void __launch_bounds__(kSolveThreads)
    k_fwd_gather_diag(const SolveNode<T>* sns, const int* nodes, const int* children,
                      const double* x, int ldx, int nrhs) {
  const SolveNode<T> sn = sns[nodes[blockIdx.x]];
  fwd_gather_node(sn, sns, children, x, ldx, nrhs);
  if (sn.nelim == 0) return;
  __shared__ T Lb[SB][SB + 1];
  __syncthreads();  // xloc rows written by the gather
  const int jb = min(SB, sn.nelim);
  load_diag_block(sn, 0, jb, Lb);
  __syncthreads();
  diag_block_solve<T, NR, true>(sn, 0, jb, nrhs, Lb);
}

// Thread layout of the update kernels: G = min(4, NR) groups of 256 / G
// threads; a thread owns one row (forward) or column (backward) for the
// right-hand sides g, g + G, ... of its group g.  No cross-thread reductions
// (each FP64 add of a shuffle reduction costs a full FP64 issue slot).
template <int NR>
struct UpdLayout {
  static constexpr int G = NR < 4 ? NR : 4;
  static constexpr int W = kSolveThreads / G;  // rows / columns per CTA pass
  static constexpr int R = (NR + G - 1) / G;   // right-hand sides per thread
};

// Block step st: rows i >= i0 = j0 + jb get x_i -= sum_c L(i, j0+c) y_c with
// y = the solved rows [j0, j0+jb).  CTA 0 updates rows [i0, i0 + W) first,
// which hold the whole next diagonal block (W >= 64), and then solves that
// block.
template <typename T, int NR>
__global__ void __launch_bounds__(kSolveThreads)
    k_fwd_step(const SolveNode<T>* sns, const int* nodes, int step, int nrhs) {
  using LY = UpdLayout<NR>;
  const SolveNode<T> sn = sns[nodes[blockIdx.y]];
  const int j0 = step * SB;
  if (j0 >= sn.nelim) return;
  const int jb = min(SB, sn.nelim - j0);
  const int i0 = j0 + jb;
  if (i0 >= sn.m) return;
  __shared__ T yb[SB][NR];
  __shared__ T Lb[SB][SB + 1];
  for (int e = threadIdx.x; e < SB * NR; e += blockDim.x) {
    const int r = e % SB, q = e / SB;
    yb[r][q] = (r < jb && q < nrhs) ? sn.xloc[(int64_t)q * sn.m + j0 + r] : T(0);
  }
  __syncthreads();
  const int g = threadIdx.x / LY::W, t = threadIdx.x % LY::W;
  for (int i = i0 + blockIdx.x * LY::W + t; i < sn.m; i += gridDim.x * LY::W) {
    T acc[LY::R];
#pragma unroll
    for (int r = 0; r < LY::R; ++r) acc[r] = T(0);
    const T* lrow = sn.L + (int64_t)j0 * sn.ld + i;
#pragma unroll 8
    for (int c = 0; c < jb; ++c) {
      const T l = lrow[(int64_t)c * sn.ld];
#pragma unroll
      for (int r = 0; r < LY::R; ++r) acc[r] += l * yb[c][g + r * LY::G];
    }
#pragma unroll
    for (int r = 0; r < LY::R; ++r) {
      const int q = g + r * LY::G;
      if (q < nrhs) sn.xloc[(int64_t)q * sn.m + i] -= acc[r];
    }
  }
  if (blockIdx.x != 0 || i0 >= sn.nelim) return;
  __syncthreads();  // rows [i0, i0 + jb1) updated by this CTA
  const int jb1 = min(SB, sn.nelim - i0);
  load_diag_block(sn, i0, jb1, Lb);
  __syncthreads();
  diag_block_solve<T, NR, true>(sn, i0, jb1, nrhs, Lb);
}

template <typename T>
__global__ void k_fwd_scatter(const SolveNode<T>* sns, const int* nodes, double* x, int ldx,
                              int nrhs) {
  const SolveNode<T> sn = sns[nodes[blockIdx.y]];
  const int tot = sn.nelim * nrhs;
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < tot; e += gridDim.x * blockDim.x) {
    const int i = e % sn.nelim, q = e / sn.nelim;
    x[(int64_t)q * ldx + sn.perm[i]] = (double)sn.xloc[(int64_t)q * sn.m + i];
  }
}

// ---- backward ----
template <typename T>
__global__ void k_bwd_gather(const SolveNode<T>* sns, const int* nodes, const double* x, int ldx,
                             int nrhs, bool do_diag, bool do_bwd) {
  const SolveNode<T> sn = sns[nodes[blockIdx.y]];
  const int mm = do_bwd ? sn.m : sn.nelim;
  const int tot = mm * nrhs;
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < tot; e += gridDim.x * blockDim.x) {
    const int i = e % mm, q = e / mm;
    const int src = (i < sn.n) ? sn.perm[i] : sn.rows[sn.ncol + i - sn.n];
    double v = x[(int64_t)q * ldx + src];
    if (do_diag && i < sn.nelim) {
      const double di = sn.D[2 * i];
      if (isinf(di)) {
        // second half of a 2x2: d21*x1 + d22*x2
        const double d21 = sn.D[2 * (i - 1) + 1], d22 = sn.D[2 * i + 1];
        const double x1 = x[(int64_t)q * ldx + sn.perm[i - 1]];
        v = d21 * x1 + d22 * v;
      } else if (i + 1 < sn.nelim && isinf(sn.D[2 * i + 2])) {
        const double d21 = sn.D[2 * i + 1];
        const double x2 = x[(int64_t)q * ldx + sn.perm[i + 1]];
        v = di * v + d21 * x2;
      } else {
        v = di * v;
      }
    }
    sn.xloc[(int64_t)q * sn.m + i] = (T)v;
  }
}

// xloc[j] -= sum_{i in [nelim, m)} L(i, j) xloc[i] for one column j (one warp)
template <typename T, int NR>
__device__ __forceinline__ void bwd_l21_column(const SolveNode<T>& sn, int j, int nrhs,
                                               int lane) {
  T acc[NR];
#pragma unroll
  for (int q = 0; q < NR; ++q) acc[q] = T(0);
  const T* col = sn.L + (int64_t)j * sn.ld;
  for (int i = sn.nelim + lane; i < sn.m; i += 32) {
    const T l = col[i];
#pragma unroll
    for (int q = 0; q < NR; ++q)
      if (q < nrhs) acc[q] += l * sn.xloc[(int64_t)q * sn.m + i];
  }
#pragma unroll
  for (int q = 0; q < NR; ++q)
    for (int off = 16; off > 0; off >>= 1) acc[q] += __shfl_xor_sync(0xffffffffu, acc[q], off);
  if (lane == 0)
    for (int q = 0; q < nrhs; ++q) sn.xloc[(int64_t)q * sn.m + j] -= acc[q];
}

// L21^T part of the backward solve for every eliminated column (one warp per
// column: the dot products run over the m - nelim rows below the pivots)
template <typename T, int NR>
__global__ void __launch_bounds__(kSolveThreads)
    k_bwd_l21(const SolveNode<T>* sns, const int* nodes, int nrhs) {
  const SolveNode<T> sn = sns[nodes[blockIdx.y]];
  if (sn.m <= sn.nelim) return;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int j = blockIdx.x * kSolveWarps + warp; j < sn.nelim; j += gridDim.x * kSolveWarps)
    bwd_l21_column<T, NR>(sn, j, nrhs, lane);
}

// the last diagonal block of each node (one CTA per node)
template <typename T, int NR>
__global__ void __launch_bounds__(kSolveThreads)
    k_bwd_diag_last(const SolveNode<T>* sns, const int* nodes, int nrhs) {
  const SolveNode<T> sn = sns[nodes[blockIdx.x]];
  if (sn.nelim == 0) return;
  const int jl = ((sn.nelim - 1) / SB) * SB;
  __shared__ T Lb[SB][SB + 1];
  load_diag_block(sn, jl, sn.nelim - jl, Lb);
  __syncthreads();
  diag_block_solve<T, NR, false>(sn, jl, sn.nelim - jl, nrhs, Lb);
}

// Block step st (> 0) of the backward solve: the columns j left of block st
// take x_j -= sum_c L(j0+c, j) y_c with y = its solved rows.  CTA 0 updates
// the columns of block st-1 and then solves that block; CTAs 1.. update the
// columns before it, W columns per pass.
template <typename T, int NR>
__global__ void __launch_bounds__(kSolveThreads)
    k_bwd_step(const SolveNode<T>* sns, const int* nodes, int step, int nrhs) {
  using LY = UpdLayout<NR>;
  const SolveNode<T> sn = sns[nodes[blockIdx.y]];
  const int j0 = step * SB;
  if (j0 >= sn.nelim || j0 == 0) return;
  const int jb = min(SB, sn.nelim - j0);
  __shared__ T yb[SB][NR];
  __shared__ T Lb[SB][SB + 1];
  for (int e = threadIdx.x; e < SB * NR; e += blockDim.x) {
    const int r = e % SB, q = e / SB;
    yb[r][q] = (r < jb && q < nrhs) ? sn.xloc[(int64_t)q * sn.m + j0 + r] : T(0);
  }
  __syncthreads();
  const int g = threadIdx.x / LY::W, t = threadIdx.x % LY::W;
  const int jp = j0 - SB;  // first column of block st-1 (a full block)
  int jbeg, jend, jstep;
  if (blockIdx.x == 0) {
    jbeg = jp + t; jend = j0; jstep = LY::W;
  } else {
    jbeg = (blockIdx.x - 1) * LY::W + t; jend = jp; jstep = (gridDim.x - 1) * LY::W;
  }
  for (int j = jbeg; j < jend; j += jstep) {
    const T* col = sn.L + (int64_t)j * sn.ld + j0;
    T acc[LY::R];
#pragma unroll
    for (int r = 0; r < LY::R; ++r) acc[r] = T(0);
#pragma unroll 8
    for (int c = 0; c < jb; ++c) {
      const T l = col[c];
#pragma unroll
      for (int r = 0; r < LY::R; ++r) acc[r] += l * yb[c][g + r * LY::G];
    }
#pragma unroll
    for (int r = 0; r < LY::R; ++r) {
      const int q = g + r * LY::G;
      if (q < nrhs) sn.xloc[(int64_t)q * sn.m + j] -= acc[r];
    }
  }
  if (blockIdx.x != 0) return;
  __syncthreads();
  load_diag_block(sn, jp, SB, Lb);
  __syncthreads();
  diag_block_solve<T, NR, false>(sn, jp, SB, nrhs, Lb);
}

inline int cdiv(int a, int b) { return (a + b - 1) / b; }

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

// gather plus the first diagonal block of every node of the level
template <typename T>
void launch_fwd_gather(const SolveNode<T>* sn, const int* nodes, int nn, const int* children,
                       const double* x, int ldx, int nrhs, cudaStream_t s) {
  if (nn <= 0) return;
  with_nr(nrhs, [&](auto nrc) {
    constexpr int NR = decltype(nrc)::value;
    k_fwd_gather_diag<T, NR><<<nn, kSolveThreads, 0, s>>>(sn, nodes, children, x, ldx, nrhs);
    note_launches(1);
  });
}

// block steps: update below block st, then solve block st + 1
// block steps: update below block st, then solve block st + 1
template <typename T>
void launch_fwd_steps(const SolveNode<T>* sn, const int* nodes, int nn, int max_nelim,
                      int max_m, int nrhs, cudaStream_t s, PhaseTimer* tm) {
  if (nn <= 0) return;
  const int steps = cdiv(max_nelim, SB);
  with_nr(nrhs, [&](auto nrc) {
    constexpr int NR = decltype(nrc)::value;
    constexpr int W = UpdLayout<NR>::W;
    for (int st = 0; st < steps; ++st) {
      const int rows = max_m - st * SB;  // upper bound; the kernel derives the exact range
      if (rows <= 0) break;
      const int gx = std::max(1, std::min(cdiv(rows, W), 152));
      pmark(tm, kPhFwdUpdate, s);
      k_fwd_step<T, NR><<<dim3(gx, nn), kSolveThreads, 0, s>>>(sn, nodes, st, nrhs);
      note_launches(1);
    }
  });
}

template <typename T>
void launch_fwd_scatter(const SolveNode<T>* sn, const int* nodes, int nn, double* x, int ldx,
                        int nrhs, int max_nelim, cudaStream_t s) {
  if (nn <= 0) return;
  int gx = std::max(1, std::min(cdiv(max_nelim * nrhs, 256), 64));
  { k_fwd_scatter<T><<<dim3(gx, nn), 256, 0, s>>>(sn, nodes, x, ldx, nrhs); note_launches(1); }
}

template <typename T>
void launch_bwd(const SolveNode<T>* sn, const int* nodes, int nn, double* x, int ldx, int nrhs,
                int max_m, int max_nelim, bool do_diag, bool do_bwd, cudaStream_t s,
                PhaseTimer* tm) {
  if (nn <= 0) return;
  int gx = std::max(1, std::min(cdiv(max_m * nrhs, 256), 64));
  pmark(tm, kPhBwdGather, s);
  { k_bwd_gather<T><<<dim3(gx, nn), 256, 0, s>>>(sn, nodes, x, ldx, nrhs, do_diag, do_bwd); note_launches(1); }
  if (do_bwd) {
    with_nr(nrhs, [&](auto nrc) {
      constexpr int NR = decltype(nrc)::value;
      constexpr int W = UpdLayout<NR>::W;
      const int gw = std::max(1, std::min(cdiv(max_nelim, kSolveWarps), 152));
      pmark(tm, kPhBwdL21, s);
      k_bwd_l21<T, NR><<<dim3(gw, nn), kSolveThreads, 0, s>>>(sn, nodes, nrhs);
      note_launches(1);
      pmark(tm, kPhBwdDiag, s);
      k_bwd_diag_last<T, NR><<<nn, kSolveThreads, 0, s>>>(sn, nodes, nrhs);
      note_launches(1);
      const int steps = cdiv(max_nelim, SB);
      for (int st = steps - 1; st >= 1; --st) {
        // CTA 0 takes block st-1; at least one more CTA for the columns before it
        const int gu = std::max(1, std::min(cdiv((st - 1) * SB, W), 151));
        pmark(tm, kPhBwdUpdate, s);
        k_bwd_step<T, NR><<<dim3(1 + gu, nn), kSolveThreads, 0, s>>>(sn, nodes, st, nrhs);
        note_launches(1);
      }
    });
  }
  int gs = std::max(1, std::min(cdiv(max_nelim * nrhs, 256), 64));
  pmark(tm, kPhBwdScatter, s);
  { k_fwd_scatter<T><<<dim3(gs, nn), 256, 0, s>>>(sn, nodes, x, ldx, nrhs); note_launches(1); }
}

#define INST(T)                                                                                \
  template void launch_fwd_gather<T>(const SolveNode<T>*, const int*, int, const int*,         \
                                     const double*, int, int, cudaStream_t);                   \
  template void launch_fwd_steps<T>(const SolveNode<T>*, const int*, int, int, int, int,       \
                                    cudaStream_t, PhaseTimer*);                                \
  template void launch_fwd_scatter<T>(const SolveNode<T>*, const int*, int, double*, int, int, \
                                      int, cudaStream_t);                                      \
  template void launch_bwd<T>(const SolveNode<T>*, const int*, int, double*, int, int, int, int, \
                              bool, bool, cudaStream_t, PhaseTimer*);
INST(double)
INST(float)
#undef INST

}  // namespace ssids300
