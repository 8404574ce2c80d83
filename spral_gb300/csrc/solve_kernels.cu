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
// are blocked by 64 rows: a one-warp diagonal-block solve (values in
// registers, the pivot row broadcast by shuffles) followed by a row-parallel
// (forward) or column-parallel (backward) update.  Arithmetic is in the
// factor precision T; the number of right-hand sides per pass NR is a
// template parameter so that no work is spent on absent columns.
#include <type_traits>

#include "ssids_gpu.cuh"

namespace ssids300 {

namespace {

constexpr int SB = kSolveBlk;

template <typename T>
__global__ void k_fwd_gather(const SolveNode<T>* sns, const int* nodes, const int* children,
                             const double* x, int ldx, int nrhs) {
  const SolveNode<T> sn = sns[nodes[blockIdx.x]];
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
constexpr int kSolveDiagThreads = 256;
template <typename T>
__device__ __forceinline__ void load_diag_block(const SolveNode<T>& sn, int j0, int jb,
                                                T (*Lb)[SB + 1]) {
  constexpr int PER = SB * SB / kSolveDiagThreads;  // 16
  T v[PER];
#pragma unroll
  for (int k = 0; k < PER; ++k) {
    const int e = threadIdx.x + k * kSolveDiagThreads;
    const int c = e / SB, r = e % SB;
    v[k] = (r > c && r < jb && c < jb) ? sn.L[(int64_t)(j0 + c) * sn.ld + j0 + r] : T(0);
  }
#pragma unroll
  for (int k = 0; k < PER; ++k) {
    const int e = threadIdx.x + k * kSolveDiagThreads;
    Lb[e / SB][e % SB] = v[k];
  }
}

// forward: unit lower triangular solve of rows [j0, j0+jb) in place
template <typename T, int NR>
__global__ void __launch_bounds__(kSolveDiagThreads) k_fwd_diag(const SolveNode<T>* sns, const int* nodes,
                                                 int step, int nrhs) {
  const SolveNode<T> sn = sns[nodes[blockIdx.x]];
  const int j0 = step * SB;
  if (j0 >= sn.nelim) return;
  const int jb = min(SB, sn.nelim - j0);
  __shared__ T Lb[SB][SB + 1];  // Lb[c][r] = L(j0+r, j0+c)
  load_diag_block(sn, j0, jb, Lb);
  __syncthreads();
  if (threadIdx.x >= 32) return;
  const int lane = threadIdx.x;
  T x0[NR], x1[NR];
#pragma unroll
  for (int q = 0; q < NR; ++q) {
    x0[q] = (q < nrhs && lane < jb) ? sn.xloc[(int64_t)q * sn.m + j0 + lane] : T(0);
    x1[q] = (q < nrhs && lane + 32 < jb) ? sn.xloc[(int64_t)q * sn.m + j0 + lane + 32] : T(0);
  }
  for (int k = 0; k < jb - 1; ++k) {
    const T l0 = Lb[k][lane], l1 = Lb[k][lane + 32];  // zero on and above the diagonal
#pragma unroll
    for (int q = 0; q < NR; ++q) {
      const T xk = (k < 32) ? __shfl_sync(0xffffffffu, x0[q], k & 31)
                            : __shfl_sync(0xffffffffu, x1[q], k & 31);
      x0[q] -= l0 * xk;
      x1[q] -= l1 * xk;
    }
  }
#pragma unroll
  for (int q = 0; q < NR; ++q) {
    if (q < nrhs && lane < jb) sn.xloc[(int64_t)q * sn.m + j0 + lane] = x0[q];
    if (q < nrhs && lane + 32 < jb) sn.xloc[(int64_t)q * sn.m + j0 + lane + 32] = x1[q];
  }
}

template <typename T, int NR>
__global__ void k_fwd_update(const SolveNode<T>* sns, const int* nodes, int step, int nrhs) {
  const SolveNode<T> sn = sns[nodes[blockIdx.y]];
  const int j0 = step * SB;
  if (j0 >= sn.nelim) return;
  const int jb = min(SB, sn.nelim - j0);
  const int i0 = j0 + jb;
  if (i0 >= sn.m) return;
  __shared__ T yb[SB][NR];
  for (int e = threadIdx.x; e < SB * NR; e += blockDim.x) {
    const int r = e % SB, q = e / SB;
    yb[r][q] = (r < jb && q < nrhs) ? sn.xloc[(int64_t)q * sn.m + j0 + r] : T(0);
  }
  __syncthreads();
  for (int i = i0 + blockIdx.x * blockDim.x + threadIdx.x; i < sn.m; i += gridDim.x * blockDim.x) {
    T acc[NR];
#pragma unroll
    for (int q = 0; q < NR; ++q) acc[q] = T(0);
    const T* lrow = sn.L + (int64_t)j0 * sn.ld + i;
#pragma unroll 8
    for (int c = 0; c < jb; ++c) {
      const T l = lrow[(int64_t)c * sn.ld];
#pragma unroll
      for (int q = 0; q < NR; ++q) acc[q] += l * yb[c][q];
    }
#pragma unroll
    for (int q = 0; q < NR; ++q)
      if (q < nrhs) sn.xloc[(int64_t)q * sn.m + i] -= acc[q];
  }
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

// xloc[j] -= sum_{i in [nelim, m)} L(i, j) xloc[i]   (warp per column j)
template <typename T, int NR>
__global__ void k_bwd_l21(const SolveNode<T>* sns, const int* nodes, int nrhs) {
  const SolveNode<T> sn = sns[nodes[blockIdx.y]];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  if (sn.m <= sn.nelim) return;
  for (int j = blockIdx.x * nw + warp; j < sn.nelim; j += gridDim.x * nw) {
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
}

// backward: unit upper (L^T) triangular solve of rows [j0, j0+jb) in place
template <typename T, int NR>
__global__ void __launch_bounds__(kSolveDiagThreads) k_bwd_diag(const SolveNode<T>* sns, const int* nodes,
                                                 int step, int nrhs) {
  const SolveNode<T> sn = sns[nodes[blockIdx.x]];
  const int j0 = step * SB;
  if (j0 >= sn.nelim) return;
  const int jb = min(SB, sn.nelim - j0);
  __shared__ T Lb[SB][SB + 1];  // Lb[c][r] = L(j0+r, j0+c)
  load_diag_block(sn, j0, jb, Lb);
  __syncthreads();
  if (threadIdx.x >= 32) return;
  const int lane = threadIdx.x;
  T x0[NR], x1[NR];
#pragma unroll
  for (int q = 0; q < NR; ++q) {
    x0[q] = (q < nrhs && lane < jb) ? sn.xloc[(int64_t)q * sn.m + j0 + lane] : T(0);
    x1[q] = (q < nrhs && lane + 32 < jb) ? sn.xloc[(int64_t)q * sn.m + j0 + lane + 32] : T(0);
  }
  // (L^T y)_r = y_r + sum_{c > r} L(c, r) y_c ; process c from the bottom.
  // L(c, r) = Lb[r][c] is zero unless c > r, so no lane masks are needed.
  for (int c = jb - 1; c > 0; --c) {
    const T l0 = Lb[lane][c], l1 = Lb[lane + 32][c];
#pragma unroll
    for (int q = 0; q < NR; ++q) {
      const T yc = (c < 32) ? __shfl_sync(0xffffffffu, x0[q], c & 31)
                            : __shfl_sync(0xffffffffu, x1[q], c & 31);
      x0[q] -= l0 * yc;
      x1[q] -= l1 * yc;
    }
  }
#pragma unroll
  for (int q = 0; q < NR; ++q) {
    if (q < nrhs && lane < jb) sn.xloc[(int64_t)q * sn.m + j0 + lane] = x0[q];
    if (q < nrhs && lane + 32 < jb) sn.xloc[(int64_t)q * sn.m + j0 + lane + 32] = x1[q];
  }
}

// columns j < j0: xloc[j] -= sum_{c < jb} L(j0+c, j) y_c   (warp per column)
template <typename T, int NR>
__global__ void k_bwd_update(const SolveNode<T>* sns, const int* nodes, int step, int nrhs) {
  const SolveNode<T> sn = sns[nodes[blockIdx.y]];
  const int j0 = step * SB;
  if (j0 >= sn.nelim || j0 == 0) return;
  const int jb = min(SB, sn.nelim - j0);
  __shared__ T yb[SB][NR];
  for (int e = threadIdx.x; e < SB * NR; e += blockDim.x) {
    const int r = e % SB, q = e / SB;
    yb[r][q] = (r < jb && q < nrhs) ? sn.xloc[(int64_t)q * sn.m + j0 + r] : T(0);
  }
  __syncthreads();
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  for (int j = blockIdx.x * nw + warp; j < j0; j += gridDim.x * nw) {
    const T* col = sn.L + (int64_t)j * sn.ld + j0;
    T acc[NR];
#pragma unroll
    for (int q = 0; q < NR; ++q) acc[q] = T(0);
    for (int c = lane; c < jb; c += 32) {
      const T l = col[c];
#pragma unroll
      for (int q = 0; q < NR; ++q) acc[q] += l * yb[c][q];
    }
#pragma unroll
    for (int q = 0; q < NR; ++q)
      for (int off = 16; off > 0; off >>= 1) acc[q] += __shfl_xor_sync(0xffffffffu, acc[q], off);
    if (lane == 0)
      for (int q = 0; q < nrhs; ++q) sn.xloc[(int64_t)q * sn.m + j] -= acc[q];
  }
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

template <typename T>
void launch_fwd_gather(const SolveNode<T>* sn, const int* nodes, int nn, const int* children,
                       const double* x, int ldx, int nrhs, cudaStream_t s) {
  if (nn <= 0) return;
  { k_fwd_gather<T><<<nn, 256, 0, s>>>(sn, nodes, children, x, ldx, nrhs); note_launches(1); }
}

template <typename T>
void launch_fwd_steps(const SolveNode<T>* sn, const int* nodes, int nn, int max_nelim,
                      int max_m, int nrhs, cudaStream_t s, PhaseTimer* tm) {
  if (nn <= 0) return;
  const int steps = cdiv(max_nelim, SB);
  with_nr(nrhs, [&](auto nrc) {
    constexpr int NR = decltype(nrc)::value;
    for (int st = 0; st < steps; ++st) {
      pmark(tm, kPhFwdDiag, s);
      { k_fwd_diag<T, NR><<<nn, kSolveDiagThreads, 0, s>>>(sn, nodes, st, nrhs); note_launches(1); }
      int rows = max_m - st * SB;  // upper bound; the kernel derives the exact range
      if (rows > 0) {
        int gx = std::max(1, std::min(cdiv(rows, 128), 128));
        pmark(tm, kPhFwdUpdate, s);
        { k_fwd_update<T, NR><<<dim3(gx, nn), 128, 0, s>>>(sn, nodes, st, nrhs); note_launches(1); }
      }
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
      int gw = std::max(1, std::min(cdiv(max_nelim, 8), 128));
      pmark(tm, kPhBwdL21, s);
      { k_bwd_l21<T, NR><<<dim3(gw, nn), 256, 0, s>>>(sn, nodes, nrhs); note_launches(1); }
      const int steps = cdiv(max_nelim, SB);
      for (int st = steps - 1; st >= 0; --st) {
        pmark(tm, kPhBwdDiag, s);
        { k_bwd_diag<T, NR><<<nn, kSolveDiagThreads, 0, s>>>(sn, nodes, st, nrhs); note_launches(1); }
        if (st > 0) {
          int gu = std::max(1, std::min(cdiv(st * SB, 8), 128));
          pmark(tm, kPhBwdUpdate, s);
          { k_bwd_update<T, NR><<<dim3(gu, nn), 256, 0, s>>>(sn, nodes, st, nrhs); note_launches(1); }
        }
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
