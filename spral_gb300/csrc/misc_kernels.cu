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

template <typename T>
__global__ void k_zero_fronts(FrontDesc<T>* fds, const int* fronts) {
  const FrontDesc<T> fd = fds[fronts[blockIdx.y]];
  const int64_t nl = (int64_t)fd.ld * fd.n;
  const int64_t nc = (int64_t)fd.cm * fd.cm;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nl; i += stride) fd.L[i] = T(0);
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nc; i += stride)
    fd.C[(i / fd.cm) * fd.ldc + i % fd.cm] = T(0);
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < 2 * fd.n; i += stride) fd.D[i] = 0.0;
}

// r = b - A x, warp per row
__global__ void k_spmv_resid(const int64_t* aptr, const int* acol, const int64_t* asrc,
                             const double* aval, int n, const double* x, const double* b,
                             double* r, int nrhs, int ld) {
  const int lane = threadIdx.x & 31;
  const int64_t w = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t i = w; i < n; i += nw) {
    for (int q = 0; q < nrhs; ++q) {
      double s = 0.0;
      for (int64_t k = aptr[i] + lane; k < aptr[i + 1]; k += 32)
        s += aval[asrc[k]] * x[(int64_t)q * ld + acol[k]];
      for (int off = 16; off > 0; off >>= 1) s += __shfl_xor_sync(0xffffffffu, s, off);
      if (lane == 0) r[(int64_t)q * ld + i] = b[(int64_t)q * ld + i] - s;
    }
  }
}

__device__ __forceinline__ void atomic_max_pos(double* a, double v) {
  // non-negative doubles order like their bit patterns
  atomicMax(reinterpret_cast<unsigned long long*>(a), (unsigned long long)__double_as_longlong(v));
}

// work: [0] ||A||, then per rhs (xn, bn, rn) at 1 + 3q
__global__ void k_norms(const int64_t* aptr, const int64_t* asrc, const double* aval, int n,
                        const double* x, const double* r, const double* b, int nrhs, int ld,
                        double* work) {
  double an = 0.0;
  double loc[3 * kSolveRhs];
  for (int i = 0; i < 3 * kSolveRhs; ++i) loc[i] = 0.0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    double rs = 0.0;
    for (int64_t k = aptr[i]; k < aptr[i + 1]; ++k) rs += fabs(aval[asrc[k]]);
    an = fmax(an, rs);
    for (int q = 0; q < nrhs && q < kSolveRhs; ++q) {
      loc[3 * q] = fmax(loc[3 * q], fabs(x[(int64_t)q * ld + i]));
      loc[3 * q + 1] = fmax(loc[3 * q + 1], fabs(b[(int64_t)q * ld + i]));
      loc[3 * q + 2] = fmax(loc[3 * q + 2], fabs(r[(int64_t)q * ld + i]));
    }
  }
  for (int off = 16; off > 0; off >>= 1) an = fmax(an, __shfl_xor_sync(0xffffffffu, an, off));
  if ((threadIdx.x & 31) == 0) atomic_max_pos(&work[0], an);
  for (int q = 0; q < nrhs && q < kSolveRhs; ++q)
    for (int j = 0; j < 3; ++j) {
      double v = loc[3 * q + j];
      for (int off = 16; off > 0; off >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, off));
      if ((threadIdx.x & 31) == 0) atomic_max_pos(&work[1 + 3 * q + j], v);
    }
}

__global__ void k_bwd_finish(const double* work, int nrhs, double* out) {
  int q = threadIdx.x;
  if (q < nrhs) {
    double den = work[0] * work[1 + 3 * q] + work[1 + 3 * q + 1];
    out[q] = (den > 0) ? work[1 + 3 * q + 2] / den : 0.0;
  }
}

__global__ void k_axpy(int64_t total, int n, int ld, double* x, const double* d) {
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total;
       e += (int64_t)gridDim.x * blockDim.x) {
    int64_t q = e / n, i = e % n;
    x[q * ld + i] += d[q * ld + i];
  }
}

}  // namespace

template <typename T>
void launch_zero_fronts(FrontDesc<T>* fd, const int* fronts, int nf, int max_elems,
                        cudaStream_t s) {
  if (nf <= 0) return;
  int gx = std::max(1, std::min((max_elems + 1023) / 1024, 256));
  { k_zero_fronts<T><<<dim3(gx, nf), 256, 0, s>>>(fd, fronts); note_launches(1); }
}
template void launch_zero_fronts<double>(FrontDesc<double>*, const int*, int, int, cudaStream_t);
template void launch_zero_fronts<float>(FrontDesc<float>*, const int*, int, int, cudaStream_t);

void launch_spmv_resid(const int64_t* aptr, const int* acol, const int64_t* asrc,
                       const double* aval, int n, const double* x, const double* b, double* r,
                       int nrhs, int ld, cudaStream_t s) {
  int blocks = std::max(1, std::min((n + 7) / 8, 4096));
  { k_spmv_resid<<<blocks, 256, 0, s>>>(aptr, acol, asrc, aval, n, x, b, r, nrhs, ld); note_launches(1); }
}

void launch_axpy(int n, int nrhs, int ld, double* x, const double* d, cudaStream_t s) {
  int64_t total = (int64_t)n * nrhs;
  int blocks = (int)std::max<int64_t>(1, std::min<int64_t>((total + 255) / 256, 4096));
  { k_axpy<<<blocks, 256, 0, s>>>(total, n, ld, x, d); note_launches(1); }
}

// work must hold 1 + 3*nrhs + nrhs doubles; the result (per rhs) is written
// to work[0 .. nrhs) after the reduction.
void launch_bwd_err(const int64_t* aptr, const int64_t* asrc, const double* aval, int n,
                    const double* x, const double* r, const double* b, int nrhs, int ld,
                    double* work, cudaStream_t s) {
  double* acc = work + nrhs;
  cudaMemsetAsync(acc, 0, (1 + 3 * kSolveRhs) * sizeof(double), s);
  int blocks = std::max(1, std::min((n + 255) / 256, 1024));
  { k_norms<<<blocks, 256, 0, s>>>(aptr, asrc, aval, n, x, r, b, nrhs, ld, acc); note_launches(1); }
  { k_bwd_finish<<<1, 32, 0, s>>>(acc, nrhs, work); note_launches(1); }
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
