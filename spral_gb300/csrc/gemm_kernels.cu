// Contribution block of the fronts of a level on CUDA cores (SIMT):
// C -= L21 (L21 D)^T over all eliminated columns, lower part
// (factor.hxx:96-108; gpu path: syrk.cu:185 form_contrib), batched over the
// fronts of a level (blockIdx.y = front).  The operand pointers depend on
// the elimination count (nelim), so each CTA derives its job from the
// front's FrontState; tiles are walked with a grid-stride loop over the
// lower triangle.  (The APP panel update lives in factor_kernels.cu.)
#include "ssids_gpu.cuh"

namespace ssids300 {

namespace {

constexpr int TM = kGemmTile;  // 64
constexpr int TK = 16;

template <typename T>
__device__ __forceinline__ bool make_job(const FrontDesc<T>& fd, const FrontState& st,
                                         SyrkJob<T>& j) {
  if (fd.tc) return false;  // formed on the tensor cores instead
  const int cm = fd.m - fd.n;
  j.C = fd.C;
  j.A = fd.L + fd.n;
  j.B = fd.LD;
  j.ldc = fd.ldc; j.lda = fd.ld; j.ldb = cm;
  j.M = cm; j.N = cm;
  j.K = st.nelim;
  return j.K > 0 && j.M > 0 && j.N > 0;
}

// MODE 1 (the contribution block) is the only mode
template <typename T, int MODE>
__global__ void __launch_bounds__(256) k_syrk(FrontDesc<T>* fds, const FrontState* sts,
                                              const int* fronts) {
  const int f = fronts[blockIdx.y];
  const FrontDesc<T> fd = fds[f];  // written by the host before the launch
  pdl_wait();
  pdl_trigger();
  const FrontState st = sts[f];
  SyrkJob<T> j;
  if (!make_job<T>(fd, st, j)) return;
  const int tid = threadIdx.x;
  const int tx = tid & 15, ty = tid >> 4;
  const int tc = (j.N + TM - 1) / TM, tr = (j.M + TM - 1) / TM;
  const int total = tc * tr - tc * (tc - 1) / 2;
  if constexpr (sizeof(T) == 4) {
    // FP32: a tile reads its C entries with the first 32 columns of A and B
    // in one batch of loads, then one batch per further 32 columns.  (Thin
    // supernodes update large contribution blocks with depth 32, where the
    // update is a stream of C through HBM.)
    constexpr int KC = 32, PER = TM * KC / 256;
    __shared__ T Ap[KC][TM + 4];
    __shared__ T Bp[KC][TM + 4];
    for (int t = blockIdx.x; t < total; t += gridDim.x) {
      int tj = 0, rem = t;
      while (rem >= tr - tj) { rem -= tr - tj; ++tj; }
      const int ti = tj + rem;
      const int row0 = ti * TM, col0 = tj * TM;
      T cv[4][4], acc[4][4];
#pragma unroll
      for (int y = 0; y < 4; ++y) {
        const int c = col0 + ty + 16 * y;
#pragma unroll
        for (int x = 0; x < 4; ++x) {
          const int r = row0 + tx + 16 * x;
          cv[x][y] = (r < j.M && c < j.N && r >= c) ? j.C[(int64_t)c * j.ldc + r] : T(0);
          acc[x][y] = T(0);
        }
      }
      for (int k0 = 0; k0 < j.K; k0 += KC) {
        T av[PER], bv[PER];
#pragma unroll
        for (int q = 0; q < PER; ++q) {
          const int idx = tid + 256 * q;
          const int rr = idx % TM, kk = k0 + idx / TM;
          const int r = row0 + rr, c = col0 + rr;
          av[q] = (r < j.M && kk < j.K) ? j.A[(int64_t)kk * j.lda + r] : T(0);
          bv[q] = (c < j.N && kk < j.K) ? j.B[(int64_t)kk * j.ldb + c] : T(0);
        }
#pragma unroll
        for (int q = 0; q < PER; ++q) {
          const int idx = tid + 256 * q;
          Ap[idx / TM][idx % TM] = av[q];
          Bp[idx / TM][idx % TM] = bv[q];
        }
        __syncthreads();
#pragma unroll 8
        for (int kk = 0; kk < KC; ++kk) {
          T a[4], b[4];
#pragma unroll
          for (int q = 0; q < 4; ++q) { a[q] = Ap[kk][tx + 16 * q]; b[q] = Bp[kk][ty + 16 * q]; }
#pragma unroll
          for (int x = 0; x < 4; ++x)
#pragma unroll
            for (int y = 0; y < 4; ++y) acc[x][y] += a[x] * b[y];
        }
        __syncthreads();
      }
#pragma unroll
      for (int y = 0; y < 4; ++y) {
        const int c = col0 + ty + 16 * y;
#pragma unroll
        for (int x = 0; x < 4; ++x) {
          const int r = row0 + tx + 16 * x;
          if (r < j.M && c < j.N && r >= c) j.C[(int64_t)c * j.ldc + r] = cv[x][y] - acc[x][y];
        }
      }
    }
    return;
  }
  __shared__ T As[TK][TM + 4];
  __shared__ T Bs[TK][TM + 4];
  for (int t = blockIdx.x; t < total; t += gridDim.x) {
    int tj = 0, rem = t;
    while (rem >= tr - tj) { rem -= tr - tj; ++tj; }
    const int ti = tj + rem;
    const int row0 = ti * TM, col0 = tj * TM;
    T acc[4][4];
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
      for (int b = 0; b < 4; ++b) acc[a][b] = T(0);
    for (int k0 = 0; k0 < j.K; k0 += TK) {
#pragma unroll
      for (int q = 0; q < (TM * TK) / 256; ++q) {
        int idx = tid + 256 * q;
        int rr = idx % TM, kk = idx / TM;
        int r = row0 + rr, c = col0 + rr, k = k0 + kk;
        As[kk][rr] = (r < j.M && k < j.K) ? j.A[(int64_t)k * j.lda + r] : T(0);
        Bs[kk][rr] = (c < j.N && k < j.K) ? j.B[(int64_t)k * j.ldb + c] : T(0);
      }
      __syncthreads();
#pragma unroll
      for (int kk = 0; kk < TK; ++kk) {
        T a[4], b[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) { a[q] = As[kk][tx + 16 * q]; b[q] = Bs[kk][ty + 16 * q]; }
#pragma unroll
        for (int x = 0; x < 4; ++x)
#pragma unroll
          for (int y = 0; y < 4; ++y) acc[x][y] += a[x] * b[y];
      }
      __syncthreads();
    }
#pragma unroll
    for (int y = 0; y < 4; ++y) {
      const int c = col0 + ty + 16 * y;
#pragma unroll
      for (int x = 0; x < 4; ++x) {
        const int r = row0 + tx + 16 * x;
        if (r < j.M && c < j.N && r >= c) j.C[(int64_t)c * j.ldc + r] -= acc[x][y];
      }
    }
  }
}

}  // namespace

template <typename T>
void launch_syrk_contrib(FrontDesc<T>* fd, const FrontState* st, const int* fronts, int nf,
                         int max_tiles, cudaStream_t s) {
  int gx = max_tiles < 1 ? 1 : (max_tiles > 4096 ? 4096 : max_tiles);
  { k_syrk<T, 1><<<dim3(gx, nf), 256, 0, s>>>(fd, st, fronts); note_launches(1); }
}

template void launch_syrk_contrib<double>(FrontDesc<double>*, const FrontState*, const int*, int, int, cudaStream_t);
template void launch_syrk_contrib<float>(FrontDesc<float>*, const FrontState*, const int*, int, int, cudaStream_t);

}  // namespace ssids300
