// Small utility kernels of the numeric path: zeroing a level's fronts and
// the FP64 residual / backward-error / update kernels of iterative
// refinement.  The residual uses the matrix in pivot order as a full CSR
// whose values are read through the user's value array (no copy), so a
// same-pattern refactorisation needs no symbolic work.  The backward error is
// the scaled residual of tests/ssids/ssids.f90:1762-1810:
//   max_i |b - A x|_i / (||A||_inf ||x||_inf + ||b||_inf).
#include "ssids_gpu.cuh"

namespace ssids300 {

namespace {

// zero n elements from p (16-byte aligned) with 16-byte stores
template <typename T>
__device__ __forceinline__ void zero_range(T* p, int64_t n, int64_t i0, int64_t stride) {
  constexpr int V = 16 / sizeof(T);
  const int64_t nv = n / V;
  int4* q = reinterpret_cast<int4*>(p);
  for (int64_t i = i0; i < nv; i += stride) q[i] = make_int4(0, 0, 0, 0);
  for (int64_t i = nv * V + i0; i < n; i += stride) p[i] = T(0);
}

// Zero a level's fronts: L (ld x n, contiguous) and D.  Fronts start
// 256-byte aligned, so the stores are 16 bytes wide.  The contribution
// blocks are zeroed column by column by the extend-add, which owns them.
template <typename T>
__global__ void k_zero_fronts(FrontDesc<T>* fds, const int* fronts) {
  const FrontDesc<T> fd = fds[fronts[blockIdx.y]];
  const int64_t nl = (int64_t)fd.ld * fd.n;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  const int64_t i0 = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  zero_range(fd.L, nl, i0, stride);
  zero_range(fd.D, 2 * (int64_t)fd.n, i0, stride);
}

__device__ __forceinline__ void atomic_max_pos(double* a, double v) {
  // non-negative doubles order like their bit patterns
  atomicMax(reinterpret_cast<unsigned long long*>(a), (unsigned long long)__double_as_longlong(v));
}

// r = b - A x and the maxima of the scaled backward error in one pass.
// kResG lanes share a row (its non-zeros strided over the lanes); each
// non-zero is applied to kResQC right-hand sides at once (chunk
// blockIdx.y), so the row's index and value loads are shared by the chunk.
// Every lane of a warp runs the same number of row iterations, so the lane
// reductions use full-warp shuffles.  work: [0] ||A||_inf, then per rhs
// (||x||, ||b||, ||r||) at 1 + 3q (maxima, order-independent).
constexpr int kResG = 4;
constexpr int kResQC = 4;
// With row groups (row_group != nullptr: the group of each row, e.g. the
// matrix of a batch it belongs to) the maxima are kept per group, at
// work[g * kResStride ...], so the backward error can be judged per group.
__global__ void __launch_bounds__(256) k_resid_norms(const int64_t* aptr, const int* acol,
                                                     const int64_t* asrc, const double* aval,
                                                     int n, const double* x, const double* b,
                                                     double* r, int nrhs, int ld, double* work,
                                                     const int* row_group) {
  constexpr int G = kResG, QC = kResQC, RPW = 32 / G;
  const int lane = threadIdx.x & 31, sub = lane & (G - 1);
  const int q0 = blockIdx.y * QC;
  const int nq = min(QC, nrhs - q0);
  const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int64_t nwarp = ((int64_t)gridDim.x * blockDim.x) >> 5;
  double an = 0.0, mx[QC], mb[QC], mr[QC];
#pragma unroll
  for (int q = 0; q < QC; ++q) mx[q] = mb[q] = mr[q] = 0.0;
  for (int64_t base = warp * RPW; base < n; base += nwarp * RPW) {
    const int64_t i = base + lane / G;
    const bool ok = i < n;
    double s[QC], ra = 0.0;
#pragma unroll
    for (int q = 0; q < QC; ++q) s[q] = 0.0;
    if (ok) {
      const int64_t k1 = aptr[i + 1];
      for (int64_t k = aptr[i] + sub; k < k1; k += G) {
        const double a = aval[asrc[k]];
        const int64_t c = acol[k];
        ra += fabs(a);
#pragma unroll
        for (int q = 0; q < QC; ++q)
          if (q < nq) s[q] = fma(a, x[(int64_t)(q0 + q) * ld + c], s[q]);
      }
    }
#pragma unroll
    for (int off = G / 2; off > 0; off >>= 1) {
      ra += __shfl_xor_sync(0xffffffffu, ra, off);
#pragma unroll
      for (int q = 0; q < QC; ++q) s[q] += __shfl_xor_sync(0xffffffffu, s[q], off);
    }
    if (row_group) {
      // grouped maxima: a warp whose rows share one group reduces them and
      // makes one atomic per value; otherwise each row makes its own
      double vx[QC], vb[QC], vr[QC];
#pragma unroll
      for (int q = 0; q < QC; ++q) vx[q] = vb[q] = vr[q] = 0.0;
      const int g = ok ? row_group[i] : -1;
      if (ok && sub == 0) {
#pragma unroll
        for (int q = 0; q < QC; ++q) {
          if (q < nq) {
            const int64_t e = (int64_t)(q0 + q) * ld + i;
            const double bi = b[e], ri = bi - s[q];
            r[e] = ri;
            vx[q] = fabs(x[e]);
            vb[q] = fabs(bi);
            vr[q] = fabs(ri);
          }
        }
      }
      const double va = ok ? ra : 0.0;
      const int g0 = __shfl_sync(0xffffffffu, g, 0);
      if (__all_sync(0xffffffffu, g == g0 || g < 0)) {
        double wa = va;
        for (int off = 16; off > 0; off >>= 1) wa = fmax(wa, __shfl_xor_sync(0xffffffffu, wa, off));
#pragma unroll
        for (int q = 0; q < QC; ++q)
          for (int off = 16; off > 0; off >>= 1) {
            vx[q] = fmax(vx[q], __shfl_xor_sync(0xffffffffu, vx[q], off));
            vb[q] = fmax(vb[q], __shfl_xor_sync(0xffffffffu, vb[q], off));
            vr[q] = fmax(vr[q], __shfl_xor_sync(0xffffffffu, vr[q], off));
          }
        if (lane == 0 && g0 >= 0) {
          double* w = work + (int64_t)g0 * kResStride;
          if (blockIdx.y == 0) atomic_max_pos(&w[0], wa);
          for (int q = 0; q < nq; ++q) {
            atomic_max_pos(&w[1 + 3 * (q0 + q)], vx[q]);
            atomic_max_pos(&w[2 + 3 * (q0 + q)], vb[q]);
            atomic_max_pos(&w[3 + 3 * (q0 + q)], vr[q]);
          }
        }
      } else if (ok && sub == 0) {
        double* w = work + (int64_t)g * kResStride;
        if (blockIdx.y == 0) atomic_max_pos(&w[0], va);
        for (int q = 0; q < nq; ++q) {
          atomic_max_pos(&w[1 + 3 * (q0 + q)], vx[q]);
          atomic_max_pos(&w[2 + 3 * (q0 + q)], vb[q]);
          atomic_max_pos(&w[3 + 3 * (q0 + q)], vr[q]);
        }
      }
      continue;
    }
    if (ok && sub == 0) {
      an = fmax(an, ra);
#pragma unroll
      for (int q = 0; q < QC; ++q) {
        if (q < nq) {
          const int64_t e = (int64_t)(q0 + q) * ld + i;
          const double bi = b[e], ri = bi - s[q];
          r[e] = ri;
          mx[q] = fmax(mx[q], fabs(x[e]));
          mb[q] = fmax(mb[q], fabs(bi));
          mr[q] = fmax(mr[q], fabs(ri));
        }
      }
    }
  }
  if (row_group) return;
  // warp maxima -> block maxima in shared memory -> one atomic per value
  // and block (same-address atomics from every warp would serialise)
  constexpr int NV = 1 + 3 * QC;
  __shared__ double red[256 / 32][NV];
  const int warp_in_block = threadIdx.x >> 5;
  for (int off = 16; off > 0; off >>= 1) an = fmax(an, __shfl_xor_sync(0xffffffffu, an, off));
  if (lane == 0) red[warp_in_block][0] = an;
#pragma unroll
  for (int q = 0; q < QC; ++q) {
    double v0 = mx[q], v1 = mb[q], v2 = mr[q];
    for (int off = 16; off > 0; off >>= 1) {
      v0 = fmax(v0, __shfl_xor_sync(0xffffffffu, v0, off));
      v1 = fmax(v1, __shfl_xor_sync(0xffffffffu, v1, off));
      v2 = fmax(v2, __shfl_xor_sync(0xffffffffu, v2, off));
    }
    if (lane == 0) {
      red[warp_in_block][1 + 3 * q] = v0;
      red[warp_in_block][2 + 3 * q] = v1;
      red[warp_in_block][3 + 3 * q] = v2;
    }
  }
  __syncthreads();
  if (threadIdx.x < NV) {
    const int v = threadIdx.x;
    double m = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) m = fmax(m, red[w][v]);
    if (v == 0) {
      if (blockIdx.y == 0) atomic_max_pos(&work[0], m);
    } else if ((v - 1) / 3 < nq) {
      atomic_max_pos(&work[1 + 3 * q0 + (v - 1)], m);
    }
  }
}

// out[q] = the largest scaled backward error of right-hand side q over the
// groups (one group when rows are not grouped)
__global__ void k_bwd_finish(const double* work, int nrhs, int ngroups, double* out) {
  __shared__ double red[256];
  for (int q = 0; q < nrhs; ++q) {
    double m = 0.0;
    for (int g = threadIdx.x; g < ngroups; g += blockDim.x) {
      const double* w = work + (int64_t)g * kResStride;
      const double den = w[0] * w[1 + 3 * q] + w[2 + 3 * q];
      m = fmax(m, den > 0 ? w[3 + 3 * q] / den : 0.0);
    }
    red[threadIdx.x] = m;
    __syncthreads();
    for (int h = blockDim.x / 2; h > 0; h >>= 1) {
      if ((int)threadIdx.x < h) red[threadIdx.x] = fmax(red[threadIdx.x], red[threadIdx.x + h]);
      __syncthreads();
    }
    if (threadIdx.x == 0) out[q] = red[0];
    __syncthreads();
  }
}

__global__ void k_axpy(int64_t total, int n, int ld, double* x, const double* d,
                       const int* row_group, const unsigned char* active) {
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total;
       e += (int64_t)gridDim.x * blockDim.x) {
    int64_t q = e / n, i = e % n;
    if (active && !active[row_group[i]]) continue;
    x[q * ld + i] += d[q * ld + i];
  }
}

}  // namespace

template <typename T>
void launch_zero_fronts(FrontDesc<T>* fd, const int* fronts, int nf, int max_elems,
                        cudaStream_t s) {
  if (nf <= 0) return;
  // 16-byte stores: one thread per 8 elements (FP32) or 4 (FP64) per round
  const int per = 256 * (16 / (int)sizeof(T)) * 4;
  int gx = std::max(1, std::min((max_elems + per - 1) / per, 4 * 152));
  { k_zero_fronts<T><<<dim3(gx, nf), 256, 0, s>>>(fd, fronts); note_launches(1); }
}
template void launch_zero_fronts<double>(FrontDesc<double>*, const int*, int, int, cudaStream_t);
template void launch_zero_fronts<float>(FrontDesc<float>*, const int*, int, int, cudaStream_t);

// r = b - A x and the scaled backward error of each right-hand side, the
// largest over the row groups when row_group is given (work must hold
// nrhs + max(ngroups, 1) * (1 + 3*kSolveRhs) doubles; the result per rhs is
// written to work[0 .. nrhs)).
void launch_resid_bwd_err(const int64_t* aptr, const int* acol, const int64_t* asrc,
                          const double* aval, int n, const double* x, const double* b, double* r,
                          int nrhs, int ld, double* work, const int* row_group, int ngroups,
                          cudaStream_t s) {
  double* acc = work + nrhs;
  const int ng = row_group ? std::max(ngroups, 1) : 1;
  cudaMemsetAsync(acc, 0, (size_t)ng * kResStride * sizeof(double), s);
  const int rows_per_block = 256 / 32 * (32 / kResG);
  const int bx = std::max(1, std::min((n + rows_per_block - 1) / rows_per_block, 4 * 152));
  const int by = (nrhs + kResQC - 1) / kResQC;
  { k_resid_norms<<<dim3(bx, by), 256, 0, s>>>(aptr, acol, asrc, aval, n, x, b, r, nrhs, ld, acc, row_group); note_launches(1); }
  { k_bwd_finish<<<1, 256, 0, s>>>(acc, nrhs, ng, work); note_launches(1); }
}

// x += d; with a mask (active != nullptr) only on the rows whose group is
// active (the others' d was not solved for)
void launch_axpy(int n, int nrhs, int ld, double* x, const double* d, cudaStream_t s,
                 const int* row_group, const unsigned char* active) {
  int64_t total = (int64_t)n * nrhs;
  int blocks = (int)std::max<int64_t>(1, std::min<int64_t>((total + 255) / 256, 4096));
  { k_axpy<<<blocks, 256, 0, s>>>(total, n, ld, x, d, row_group, active); note_launches(1); }
}

}  // namespace ssids300

// FP64 FMA throughput probe: independent DFMA chains per thread, no memory
// traffic; used to state the FP64 roofline of the FP64 path (the driver's
// measured peaks cover HBM and bf16 tensor only).
namespace ssids300 {
namespace {
__global__ void k_dfma_probe(double* out, int iters, double seed) {
  double a0 = seed + threadIdx.x, a1 = a0 + 1, a2 = a0 + 2, a3 = a0 + 3;
  double a4 = a0 + 4, a5 = a0 + 5, a6 = a0 + 6, a7 = a0 + 7;
  const double m = 0.999999, c = 1e-7;
  for (int i = 0; i < iters; ++i) {
    a0 = fma(a0, m, c); a1 = fma(a1, m, c); a2 = fma(a2, m, c); a3 = fma(a3, m, c);
    a4 = fma(a4, m, c); a5 = fma(a5, m, c); a6 = fma(a6, m, c); a7 = fma(a7, m, c);
  }
  double s = a0 + a1 + a2 + a3 + a4 + a5 + a6 + a7;
  if (s == 12345.678) out[0] = s;  // keep the chains live
}
}  // namespace

double fp64_peak_tflops(int device) {
  cudaSetDevice(device);
  int sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
  double* out = nullptr;
  cudaMalloc(&out, sizeof(double));
  const int blocks = sms * 8, threads = 256, iters = 4096;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  k_dfma_probe<<<blocks, threads>>>(out, 64, 1.0);
  cudaEventRecord(e0);
  k_dfma_probe<<<blocks, threads>>>(out, iters, 1.0);
  cudaEventRecord(e1);
  cudaEventSynchronize(e1);
  float ms = 0;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(out);
  double flops = 2.0 * 8.0 * (double)iters * blocks * threads;
  return ms > 0 ? flops / (ms * 1e-3) / 1e12 : 0.0;
}
}  // namespace ssids300
