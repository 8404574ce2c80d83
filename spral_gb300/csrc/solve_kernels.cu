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
template <typename T>
__device__ __forceinline__ T gather_value(const SolveNode<T>& sn, const SolveNode<T>* sns,
                                          const int* children, const int2* pairs,
                                          const double* x, int ldx, int q, int pos) {
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
        return cn.xloc[(int64_t)q * cn.m + cn.nelim + (k - cn.doff)];
    }
    return v;
  } else {
    P = pos - sn.ndelay_in;
  }
  const int k1 = sn.gp[P + 1];
  for (int k = sn.gp[P]; k < k1; ++k) {
    const int2 pr = pairs[k];
    const SolveNode<T>& cn = sns[pr.x];
    v += cn.xloc[(int64_t)q * cn.m + cn.n + pr.y];
  }
  return v;
}

// stage the jb x jb diagonal block (strictly lower part) into shared memory;
// every thread issues a batch of loads before the stores, so the
// global-memory latency is paid once per batch, not once per element
constexpr int kSolveThreads = 256;
constexpr int kSolveWarps = kSolveThreads / 32;
constexpr int LDB = SB + 1;  // leading dimension of a staged block Lb[c * LDB + r]
constexpr int kDiagPer = SB * SB / kSolveThreads;  // entries of a staged block per thread
template <typename T>
__device__ __forceinline__ void fetch_diag_block(const SolveNode<T>& sn, int j0, int jb,
                                                 T (&v)[kDiagPer]) {
#pragma unroll
  for (int k = 0; k < kDiagPer; ++k) {
    const int e = threadIdx.x + k * kSolveThreads;
    const int c = e / SB, r = e % SB;
    v[k] = (r > c && r < jb && c < jb) ? sn.L[(int64_t)(j0 + c) * sn.ld + j0 + r] : T(0);
  }
}
template <typename T>
__device__ __forceinline__ void store_diag_block(const T (&v)[kDiagPer], T* Lb) {
#pragma unroll
  for (int k = 0; k < kDiagPer; ++k) {
    const int e = threadIdx.x + k * kSolveThreads;
    Lb[(e / SB) * LDB + e % SB] = v[k];
  }
}
// the same staging with asynchronous copies (cp.async), so that a CTA can
// start it, do other work, and wait for it with cp_async_wait_all() and a
// barrier before the block is read
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
template <typename T>
__device__ __forceinline__ void load_diag_block(const SolveNode<T>& sn, int j0, int jb, T* Lb) {
  T v[kDiagPer];
  fetch_diag_block(sn, j0, jb, v);
  store_diag_block(v, Lb);
}

// Unit lower (FWD) or unit upper L^T (!FWD) triangular solve of rows
// [j0, j0+jb) of xloc in place, with the block staged in Lb (Lb[c*LDB + r] =
// L(j0+r, j0+c), zero on and above the diagonal).  Warp w solves the
// right-hand sides w, w + 8, ...; lane l holds rows l, l + 32, ...  The
// caller has synchronised the CTA after staging Lb; nothing follows.
template <typename T, int NR, bool FWD>
__device__ __forceinline__ void diag_block_solve(const SolveNode<T>& sn, int j0, int jb,
                                                 int nrhs, const T* Lb) {
  constexpr int R = (NR + kSolveWarps - 1) / kSolveWarps;
  constexpr int G = SB / 32;  // rows per lane
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (warp >= nrhs) return;
  T x[R][G];
#pragma unroll
  for (int r = 0; r < R; ++r) {
    const int q = warp + r * kSolveWarps;
#pragma unroll
    for (int g = 0; g < G; ++g)
      x[r][g] = (q < nrhs && lane + 32 * g < jb) ? sn.xloc[(int64_t)q * sn.m + j0 + lane + 32 * g]
                                                 : T(0);
  }
  if (FWD) {
    for (int k = 0; k < jb - 1; ++k) {
      T l[G];
#pragma unroll
      for (int g = 0; g < G; ++g) l[g] = Lb[k * LDB + lane + 32 * g];
      const int kg = k >> 5;
#pragma unroll
      for (int r = 0; r < R; ++r) {
        T src = x[r][0];
#pragma unroll
        for (int g = 1; g < G; ++g) src = (kg == g) ? x[r][g] : src;
        const T xk = __shfl_sync(0xffffffffu, src, k & 31);
#pragma unroll
        for (int g = 0; g < G; ++g) x[r][g] -= l[g] * xk;
      }
    }
  } else {
    // (L^T y)_r = y_r + sum_{c > r} L(c, r) y_c ; process c from the bottom.
    // L(c, r) = Lb[r*LDB + c] is zero unless c > r, so no lane masks are needed.
    for (int c = jb - 1; c > 0; --c) {
      T l[G];
#pragma unroll
      for (int g = 0; g < G; ++g) l[g] = Lb[(lane + 32 * g) * LDB + c];
      const int cg = c >> 5;
#pragma unroll
      for (int r = 0; r < R; ++r) {
        T src = x[r][0];
#pragma unroll
        for (int g = 1; g < G; ++g) src = (cg == g) ? x[r][g] : src;
        const T yc = __shfl_sync(0xffffffffu, src, c & 31);
#pragma unroll
        for (int g = 0; g < G; ++g) x[r][g] -= l[g] * yc;
      }
    }
  }
#pragma unroll
  for (int r = 0; r < R; ++r) {
    const int q = warp + r * kSolveWarps;
#pragma unroll
    for (int g = 0; g < G; ++g)
      if (q < nrhs && lane + 32 * g < jb) sn.xloc[(int64_t)q * sn.m + j0 + lane + 32 * g] = x[r][g];
  }
}

// dynamic shared memory of the solve kernels: the staged block, the
// block's solved values yb[r * NR + q], then the partial sums of the
// update passes red[(qq * NR + q) * 64 + t] (qq = 0..3)
template <typename T, int NR>
constexpr size_t solve_smem_bytes() {
  return sizeof(T) * ((size_t)SB * LDB + (size_t)SB * NR + (size_t)4 * NR * 64);
}

// ---- forward ----
// Gather every node of the level into its local vector (final positions:
// xloc[i] = value of assembly position opos[i] for i < n), then solve the
// first diagonal block.  CTA 0 of a node gathers rows [0, SB) and solves
// block 0 from them; CTAs 1.. gather the rows after it (CTA 0 gathers all
// rows when it is alone).
template <typename T, int NR>
__global__ void __launch_bounds__(kSolveThreads)
    k_fwd_gather_diag(const SolveNode<T>* sns, const int* nodes, const int* children,
                      const int2* pairs, const double* x, int ldx, int nrhs) {
  const SolveNode<T> sn = sns[nodes[blockIdx.y]];  // written by the host before the launch
  pdl_wait();
  pdl_trigger();
  const int m = sn.m;
  const int h = (gridDim.x == 1) ? m : min(m, SB);
  int lo, len, e0, stride;
  if (blockIdx.x == 0) {
    lo = 0; len = h; e0 = threadIdx.x; stride = blockDim.x;
  } else {
    lo = h; len = m - h; e0 = (blockIdx.x - 1) * blockDim.x + threadIdx.x;
    stride = (gridDim.x - 1) * blockDim.x;
  }
  for (int e = e0; e < len * nrhs; e += stride) {
    const int i = lo + e % len, q = e / len;
    const int pos = (i < sn.n) ? sn.opos[i] : i;
    sn.xloc[(int64_t)q * m + i] = gather_value(sn, sns, children, pairs, x, ldx, q, pos);
  }
  if (blockIdx.x != 0 || sn.nelim == 0) return;
  extern __shared__ __align__(16) unsigned char solve_smem[];
  T* Lb = reinterpret_cast<T*>(solve_smem);
  __syncthreads();  // rows [0, h) written by this CTA
  const int jb = min(SB, sn.nelim);
  load_diag_block(sn, 0, jb, Lb);
  __syncthreads();
  diag_block_solve<T, NR, true>(sn, 0, jb, nrhs, Lb);
}

// Update kernels of the block steps: a CTA pass covers 64 rows (forward) or
// columns (backward); thread (t, qq) = (threadIdx.x % 64, threadIdx.x / 64)
// forms the partial dot products of entry t over the block columns
// [qq SB/4, (qq+1) SB/4) for every right-hand side, with those loads issued
// together, and the four partial sums are added through shared memory.
constexpr int kPassRows = 64;
constexpr int kQuarter = SB / 4;

template <typename T, int NR>
__device__ __forceinline__ void partial_dots(const T* p, int64_t stride, int cq, int jb,
                                             const T* yb, T (&acc)[NR]) {
  T lv[kQuarter];
#pragma unroll
  for (int k = 0; k < kQuarter; ++k) lv[k] = (cq + k < jb) ? p[(int64_t)k * stride] : T(0);
#pragma unroll
  for (int q = 0; q < NR; ++q) acc[q] = T(0);
#pragma unroll
  for (int k = 0; k < kQuarter; ++k)
#pragma unroll
    for (int q = 0; q < NR; ++q) acc[q] += lv[k] * yb[(cq + k) * NR + q];
}

// red[(qq * NR + q) * 64 + t] holds the partial sums; entry t of the pass
// (global index base + t < lim) gets x -= the sum of its four partials
template <typename T, int NR>
__device__ __forceinline__ void apply_partials(const SolveNode<T>& sn, const T* red, int base,
                                               int lim, int nrhs) {
  for (int e = threadIdx.x; e < kPassRows * NR; e += blockDim.x) {
    const int t = e % kPassRows, q = e / kPassRows;
    const int idx = base + t;
    if (q < nrhs && idx < lim) {
      const T v = red[(0 * NR + q) * kPassRows + t] + red[(1 * NR + q) * kPassRows + t] +
                  red[(2 * NR + q) * kPassRows + t] + red[(3 * NR + q) * kPassRows + t];
      sn.xloc[(int64_t)q * sn.m + idx] -= v;
    }
  }
}

// the solved rows [j0, j0+jb) of every right-hand side into yb[r*NR + q]
template <typename T, int NR>
__device__ __forceinline__ void load_y(const SolveNode<T>& sn, int j0, int jb, int nrhs, T* yb) {
  for (int e = threadIdx.x; e < SB * NR; e += blockDim.x) {
    const int r = e % SB, q = e / SB;
    yb[r * NR + q] = (r < jb && q < nrhs) ? sn.xloc[(int64_t)q * sn.m + j0 + r] : T(0);
  }
}

// Block step st: rows i >= i0 = j0 + jb get x_i -= sum_c L(i, j0+c) y_c with
// y = the solved rows [j0, j0+jb).  CTA 0 updates the next block's rows
// [i0, i0 + SB) and then solves that block; CTAs 1.. update the rows after
// it (CTA 0 as well when it is alone).
template <typename T, int NR>
__global__ void __launch_bounds__(kSolveThreads)
    k_fwd_step(const SolveNode<T>* sns, const int* nodes, int step, int nrhs) {
  const SolveNode<T> sn = sns[nodes[blockIdx.y]];  // written by the host before the launch
  pdl_wait();
  pdl_trigger();
  const int j0 = step * SB;
  if (j0 >= sn.nelim) return;
  const int jb = min(SB, sn.nelim - j0);
  const int i0 = j0 + jb;
  if (i0 >= sn.m) return;
  extern __shared__ __align__(16) unsigned char solve_smem[];
  T* Lb = reinterpret_cast<T*>(solve_smem);
  T* yb = Lb + SB * LDB;
  T* red = yb + SB * NR;
  // CTA 0 starts staging the next diagonal block first: the copies overlap
  // the update passes (L is read-only here)
  const bool solve_next = blockIdx.x == 0 && i0 < sn.nelim;
  const int jb1 = solve_next ? min(SB, sn.nelim - i0) : 0;
  if (solve_next) prefetch_diag_block(sn, i0, jb1, Lb);
  load_y<T, NR>(sn, j0, jb, nrhs, yb);
  __syncthreads();
  const int t = threadIdx.x % kPassRows, qq = threadIdx.x / kPassRows;
  const int ih = min(sn.m, i0 + SB);  // end of the next block's rows
  auto pass = [&](int base) {
    const int i = base + t;
    T acc[NR];
    if (i < sn.m) {
      partial_dots<T, NR>(sn.L + (int64_t)(j0 + qq * kQuarter) * sn.ld + i, sn.ld, qq * kQuarter,
                          jb, yb, acc);
    } else {
#pragma unroll
      for (int q = 0; q < NR; ++q) acc[q] = T(0);
    }
#pragma unroll
    for (int q = 0; q < NR; ++q) red[(qq * NR + q) * kPassRows + t] = acc[q];
    __syncthreads();
    apply_partials<T, NR>(sn, red, base, sn.m, nrhs);
    __syncthreads();
  };
  if (blockIdx.x == 0) {
    for (int base = i0; base < ih; base += kPassRows) pass(base);
  }
  if (gridDim.x == 1) {
    for (int base = ih; base < sn.m; base += kPassRows) pass(base);
  } else if (blockIdx.x > 0) {
    for (int base = ih + (blockIdx.x - 1) * kPassRows; base < sn.m;
         base += (gridDim.x - 1) * kPassRows)
      pass(base);
  }
  if (!solve_next) return;
  cp_async_wait_all();
  __syncthreads();
  diag_block_solve<T, NR, true>(sn, i0, jb1, nrhs, Lb);
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
    const int src = (i < sn.n) ? sn.perm[i] : sn.rows[sn.ncol + i - sn.n];
    double v = x[(int64_t)q * ldx + src];
    if (diag_mode == 2 && i < sn.nelim) {
      v *= sqrt(sn.D[2 * i]);
    } else if (diag_mode == 1 && i < sn.nelim) {
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

// L21^T part of the backward solve for every eliminated column:
// xloc[j] -= sum_{i in [nelim, m)} L(i, j) xloc[i].  W warps share a column
// (rows strided over their 32 W lanes); their partial sums are added in
// shared memory in warp order, so the result does not depend on the grid.
template <typename T, int NR, int W>
__global__ void __launch_bounds__(kSolveThreads)
    k_bwd_l21(const SolveNode<T>* sns, const int* nodes, int nrhs) {
  const SolveNode<T> sn = sns[nodes[blockIdx.y]];  // written by the host before the launch
  pdl_wait();
  pdl_trigger();
  if (sn.m <= sn.nelim) return;
  constexpr int CPB = kSolveWarps / W;  // columns per CTA round
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
#pragma unroll
      for (int w = 1; w < W; ++w) v += part[warp + w][lane];
      sn.xloc[(int64_t)lane * sn.m + j] -= v;
    }
    __syncthreads();
  }
}

// the last diagonal block of each node (one CTA per node)
template <typename T, int NR>
__global__ void __launch_bounds__(kSolveThreads)
    k_bwd_diag_last(const SolveNode<T>* sns, const int* nodes, int nrhs) {
  const SolveNode<T> sn = sns[nodes[blockIdx.x]];  // written by the host before the launch
  pdl_wait();
  pdl_trigger();
  if (sn.nelim == 0) return;
  const int jl = ((sn.nelim - 1) / SB) * SB;
  extern __shared__ __align__(16) unsigned char solve_smem[];
  T* Lb = reinterpret_cast<T*>(solve_smem);
  load_diag_block(sn, jl, sn.nelim - jl, Lb);
  __syncthreads();
  diag_block_solve<T, NR, false>(sn, jl, sn.nelim - jl, nrhs, Lb);
}

// Block step st (> 0) of the backward solve: the columns j left of block st
// take x_j -= sum_c L(j0+c, j) y_c with y = its solved rows.  CTA 0 updates
// the columns of block st-1 and then solves that block; CTAs 1.. update the
// columns before it (CTA 0 as well when it is alone), 64 per pass.
template <typename T, int NR>
__global__ void __launch_bounds__(kSolveThreads)
    k_bwd_step(const SolveNode<T>* sns, const int* nodes, int step, int nrhs) {
  const SolveNode<T> sn = sns[nodes[blockIdx.y]];  // written by the host before the launch
  pdl_wait();
  pdl_trigger();
  const int j0 = step * SB;
  if (j0 >= sn.nelim || j0 == 0) return;
  const int jb = min(SB, sn.nelim - j0);
  extern __shared__ __align__(16) unsigned char solve_smem[];
  T* Lb = reinterpret_cast<T*>(solve_smem);
  T* yb = Lb + SB * LDB;
  T* red = yb + SB * NR;
  const int jp = j0 - SB;  // first column of block st-1 (a full block)
  if (blockIdx.x == 0) prefetch_diag_block(sn, jp, SB, Lb);  // overlaps the passes
  load_y<T, NR>(sn, j0, jb, nrhs, yb);
  __syncthreads();
  const int t = threadIdx.x % kPassRows, qq = threadIdx.x / kPassRows;
  auto pass = [&](int base, int lim) {
    const int j = base + t;
    T acc[NR];
    if (j < lim) {
      partial_dots<T, NR>(sn.L + (int64_t)j * sn.ld + j0 + qq * kQuarter, 1, qq * kQuarter, jb,
                          yb, acc);
    } else {
#pragma unroll
      for (int q = 0; q < NR; ++q) acc[q] = T(0);
    }
#pragma unroll
    for (int q = 0; q < NR; ++q) red[(qq * NR + q) * kPassRows + t] = acc[q];
    __syncthreads();
    apply_partials<T, NR>(sn, red, base, lim, nrhs);
    __syncthreads();
  };
  if (blockIdx.x == 0) {
    for (int base = jp; base < j0; base += kPassRows) pass(base, j0);
  }
  if (gridDim.x == 1) {
    for (int base = 0; base < jp; base += kPassRows) pass(base, jp);
  } else if (blockIdx.x > 0) {
    for (int base = (blockIdx.x - 1) * kPassRows; base < jp; base += (gridDim.x - 1) * kPassRows)
      pass(base, jp);
  }
  if (blockIdx.x != 0) return;
  cp_async_wait_all();
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
                       const int2* pairs, const double* x, int ldx, int nrhs, int max_m,
                       cudaStream_t s) {
  if (nn <= 0) return;
  const int rest = std::max(0, max_m - SB) * nrhs;
  const int gx = rest > 0 ? 1 + std::min(cdiv(rest, kSolveThreads), 151) : 1;
  with_nr(nrhs, [&](auto nrc) {
    constexpr int NR = decltype(nrc)::value;
    launch_pdl(k_fwd_gather_diag<T, NR>, dim3(gx, nn), kSolveThreads, solve_smem_bytes<T, NR>(),
               s, sn, nodes, children, pairs, x, ldx, nrhs);
    note_launches(1);
  });
}

// block steps: update below block st, then solve block st + 1
template <typename T>
void launch_fwd_steps(const SolveNode<T>* sn, const int* nodes, int nn, int max_nelim,
                      int max_m, int nrhs, cudaStream_t s, PhaseTimer* tm) {
  if (nn <= 0) return;
  const int steps = cdiv(max_nelim, SB);
  with_nr(nrhs, [&](auto nrc) {
    constexpr int NR = decltype(nrc)::value;
    for (int st = 0; st < steps; ++st) {
      const int rows = max_m - st * SB;  // upper bound; the kernel derives the exact range
      if (rows <= 0) break;
      // CTA 0 takes the next block's rows, the others the rows after it
      const int tail = rows - SB - 1;
      const int gx = tail > 0 ? 1 + std::min(cdiv(tail, kPassRows), 151) : 1;
      pmark(tm, kPhFwdUpdate, s);
      launch_pdl(k_fwd_step<T, NR>, dim3(gx, nn), kSolveThreads, solve_smem_bytes<T, NR>(), s,
                 sn, nodes, st, nrhs);
      note_launches(1);
    }
  });
}

template <typename T>
void launch_fwd_scatter(const SolveNode<T>* sn, const int* nodes, int nn, double* x, int ldx,
                        int nrhs, int max_nelim, cudaStream_t s, bool scale_sqrt) {
  if (nn <= 0) return;
  int gx = std::max(1, std::min(cdiv(max_nelim * nrhs, 256), 64));
  launch_pdl(k_fwd_scatter<T>, dim3(gx, nn), 256, 0, s, sn, nodes, x, ldx, nrhs, scale_sqrt);
  note_launches(1);
}

template <typename T>
void launch_bwd(const SolveNode<T>* sn, const int* nodes, int nn, double* x, int ldx, int nrhs,
                int max_m, int max_nelim, int diag_mode, bool do_bwd, cudaStream_t s,
                PhaseTimer* tm) {
  if (nn <= 0) return;
  int gx = std::max(1, std::min(cdiv(max_m * nrhs, 256), 64));
  pmark(tm, kPhBwdGather, s);
  launch_pdl(k_bwd_gather<T>, dim3(gx, nn), 256, 0, s, sn, nodes, x, ldx, nrhs, diag_mode,
             do_bwd);
  note_launches(1);
  if (do_bwd) {
    with_nr(nrhs, [&](auto nrc) {
      constexpr int NR = decltype(nrc)::value;
      // warps per column from the level's largest front (rows below the
      // pivots <= max_m), columns spread over up to 4 CTAs per SM
      auto l21 = [&](auto wc) {
        constexpr int W = decltype(wc)::value;
        const int gw = std::max(1, std::min(cdiv(max_nelim, kSolveWarps / W), 4 * 152));
        launch_pdl(k_bwd_l21<T, NR, W>, dim3(gw, nn), kSolveThreads, 0, s, sn, nodes, nrhs);
      };
      pmark(tm, kPhBwdL21, s);
      if (max_m <= 128) l21(std::integral_constant<int, 1>());
      else if (max_m <= 512) l21(std::integral_constant<int, 2>());
      else if (max_m <= 1024) l21(std::integral_constant<int, 4>());
      else l21(std::integral_constant<int, 8>());
      note_launches(1);
      pmark(tm, kPhBwdDiag, s);
      launch_pdl(k_bwd_diag_last<T, NR>, nn, kSolveThreads, solve_smem_bytes<T, NR>(), s, sn,
                 nodes, nrhs);
      note_launches(1);
      const int steps = cdiv(max_nelim, SB);
      for (int st = steps - 1; st >= 1; --st) {
        // CTA 0 takes block st-1, the others the columns before it
        const int jp = (st - 1) * SB;
        const int gu = jp > 0 ? std::min(cdiv(jp, kPassRows), 151) : 0;
        pmark(tm, kPhBwdUpdate, s);
        launch_pdl(k_bwd_step<T, NR>, dim3(1 + gu, nn), kSolveThreads,
                   solve_smem_bytes<T, NR>(), s, sn, nodes, st, nrhs);
        note_launches(1);
      }
    });
  }
  int gs = std::max(1, std::min(cdiv(max_nelim * nrhs, 256), 64));
  pmark(tm, kPhBwdScatter, s);
  launch_pdl(k_fwd_scatter<T>, dim3(gs, nn), 256, 0, s, sn, nodes, x, ldx, nrhs, false);
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
        set(k_fwd_gather_diag<T, NR>, solve_smem_bytes<T, NR>());
        set(k_fwd_step<T, NR>, solve_smem_bytes<T, NR>());
        set(k_bwd_diag_last<T, NR>, solve_smem_bytes<T, NR>());
        set(k_bwd_step<T, NR>, solve_smem_bytes<T, NR>());
      });
    }
  });
}

#define INST(T)                                                                                \
  template void solve_init<T>();                                                               \
  template void launch_fwd_gather<T>(const SolveNode<T>*, const int*, int, const int*,         \
                                     const int2*, const double*, int, int, int, cudaStream_t); \
  template void launch_fwd_steps<T>(const SolveNode<T>*, const int*, int, int, int, int,       \
                                    cudaStream_t, PhaseTimer*);                                \
  template void launch_fwd_scatter<T>(const SolveNode<T>*, const int*, int, double*, int, int, \
                                      int, cudaStream_t, bool);                                \
  template void launch_bwd<T>(const SolveNode<T>*, const int*, int, double*, int, int, int, int, \
                              int, bool, cudaStream_t, PhaseTimer*);
INST(double)
INST(float)
#undef INST

}  // namespace ssids300
