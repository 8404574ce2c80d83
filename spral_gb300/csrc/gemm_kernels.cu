// Lower-triangular rank-k updates C(r,c) -= sum_k A(r,k) B(c,k), r >= c, on
// CUDA cores (SIMT).  Two uses per front, both batched over the fronts of a
// level (blockIdx.y = front):
//   panel   : trailing update of the APP candidate columns with the block's
//             passed pivots (ldlt_app.cxx:1082-1165 Block::update)
//   contrib : contribution block C -= L21 (L21 D)^T over all eliminated
//             columns (factor.hxx:96-108; gpu path: syrk.cu:185 form_contrib)
// The operand pointers depend on device-side pivoting state (p, npass,
// nelim), so each CTA derives its job from the front's FrontState; tiles are
// walked with a grid-stride loop over the lower trapezoid.
#include "ssids_gpu.cuh"

namespace ssids300 {

namespace {

constexpr int TM = kGemmTile;  // 64
constexpr int TK = 16;

template <typename T, int MODE>
__device__ __forceinline__ bool make_job(const FrontDesc<T>& fd, const FrontState& st,
                                         SyrkJob<T>& j) {
  if (MODE == 0) {
    if (st.bs == 0) return false;
    const int p = st.p, bs = st.bs;
    j.C = fd.L + (int64_t)(p + bs) * fd.ld + (p + bs);
    j.A = fd.L + (int64_t)p * fd.ld + (p + bs);
    j.B = fd.W;
    j.ldc = fd.ld; j.lda = fd.ld; j.ldb = fd.ld;
    j.M = fd.m - (p + bs);
    j.N = fd.n - (p + bs);
    j.K = st.npass;
  } else {
    if (fd.tc) return false;  // formed on the tensor cores instead
    const int cm = fd.m - fd.n;
    j.C = fd.C;
    j.A = fd.L + fd.n;
    j.B = fd.LD;
    j.ldc = fd.ldc; j.lda = fd.ld; j.ldb = cm;
    j.M = cm; j.N = cm;
    j.K = st.nelim;
  }
  return j.K > 0 && j.M > 0 && j.N > 0;
}

template <typename T, int MODE>
__global__ void __launch_bounds__(256) k_syrk(FrontDesc<T>* fds, const FrontState* sts,
                                              const int* fronts) {
  const int f = fronts[blockIdx.y];
  const FrontDesc<T> fd = fds[f];  // written by the host before the launch
  pdl_wait();
  pdl_trigger();
  const FrontState st = sts[f];
  SyrkJob<T> j;
  if (!make_job<T, MODE>(fd, st, j)) return;
  const int tid = threadIdx.x;
  const int tx = tid & 15, ty = tid >> 4;
  const int tc = (j.N + TM - 1) / TM, tr = (j.M + TM - 1) / TM;
  const int total = tc * tr - tc * (tc - 1) / 2;
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

// Panel update C -= A B^T (lower part), K <= kBlk passed pivots: a TP x TP
// tile per CTA round, thread (tx, ty) = (tid % 16, tid / 16) computing
// (TP/16)^2 entries.  A tile stages all of its A and B columns and reads its
// C entries in one batch of loads (one memory round trip per tile).  FP32
// uses 64 x 64 tiles (latency bound); FP64 32 x 32 tiles: a 64 x 64 tile is
// about 37 us of work for one SM's FP64 pipe, and the finer tiles balance the
// last wave of the launch.
template <typename T, int TP>
__global__ void __launch_bounds__(256) k_panel(FrontDesc<T>* fds, const FrontState* sts,
                                               const int* fronts) {
  constexpr int RT = TP / 16;            // entries per thread and direction
  constexpr int PER = TP * kBlk / 256;   // A (and B) loads per thread
  const int f = fronts[blockIdx.y];
  const FrontDesc<T> fd = fds[f];  // written by the host before the launch
  pdl_wait();
  pdl_trigger();
  const FrontState st = sts[f];
  SyrkJob<T> j;
  if (!make_job<T, 0>(fd, st, j)) return;
  __shared__ T Ap[kBlk][TP + 4];
  __shared__ T Bp[kBlk][TP + 4];
  const int tid = threadIdx.x;
  const int tx = tid & 15, ty = tid >> 4;
  const int tc = (j.N + TP - 1) / TP, tr = (j.M + TP - 1) / TP;
  const int total = tc * tr - tc * (tc - 1) / 2;
  for (int t = blockIdx.x; t < total; t += gridDim.x) {
    int tj = 0, rem = t;
    while (rem >= tr - tj) { rem -= tr - tj; ++tj; }
    const int ti = tj + rem;
    const int row0 = ti * TP, col0 = tj * TP;
    T cv[RT][RT];
#pragma unroll
    for (int y = 0; y < RT; ++y) {
      const int c = col0 + ty + 16 * y;
#pragma unroll
      for (int x = 0; x < RT; ++x) {
        const int r = row0 + tx + 16 * x;
        cv[x][y] = (r < j.M && c < j.N && r >= c) ? j.C[(int64_t)c * j.ldc + r] : T(0);
      }
    }
    T av[PER], bv[PER];
#pragma unroll
    for (int q = 0; q < PER; ++q) {
      const int idx = tid + 256 * q;
      const int rr = idx % TP, kk = idx / TP;
      const int r = row0 + rr, c = col0 + rr;
      av[q] = (r < j.M && kk < j.K) ? j.A[(int64_t)kk * j.lda + r] : T(0);
      bv[q] = (c < j.N && kk < j.K) ? j.B[(int64_t)kk * j.ldb + c] : T(0);
    }
#pragma unroll
    for (int q = 0; q < PER; ++q) {
      const int idx = tid + 256 * q;
      Ap[idx / TP][idx % TP] = av[q];
      Bp[idx / TP][idx % TP] = bv[q];
    }
    __syncthreads();
    T acc[RT][RT];
#pragma unroll
    for (int a = 0; a < RT; ++a)
#pragma unroll
      for (int b = 0; b < RT; ++b) acc[a][b] = T(0);
#pragma unroll 8
    for (int kk = 0; kk < kBlk; ++kk) {
      T a[RT], b[RT];
#pragma unroll
      for (int q = 0; q < RT; ++q) { a[q] = Ap[kk][tx + 16 * q]; b[q] = Bp[kk][ty + 16 * q]; }
#pragma unroll
      for (int x = 0; x < RT; ++x)
#pragma unroll
        for (int y = 0; y < RT; ++y) acc[x][y] += a[x] * b[y];
    }
#pragma unroll
    for (int y = 0; y < RT; ++y) {
      const int c = col0 + ty + 16 * y;
#pragma unroll
      for (int x = 0; x < RT; ++x) {
        const int r = row0 + tx + 16 * x;
        if (r < j.M && c < j.N && r >= c) j.C[(int64_t)c * j.ldc + r] = cv[x][y] - acc[x][y];
      }
    }
    __syncthreads();  // Ap/Bp are rewritten by the next tile
  }
}

}  // namespace

template <typename T>
int panel_tile() { return sizeof(T) == 8 ? 32 : 64; }
template int panel_tile<double>();
template int panel_tile<float>();

template <typename T>
void launch_syrk_panel(FrontDesc<T>* fd, const FrontState* st, const int* fronts, int nf,
                       int max_tiles, cudaStream_t s) {
  int gx = max_tiles < 1 ? 1 : (max_tiles > 4096 ? 4096 : max_tiles);
  if constexpr (sizeof(T) == 8)
    launch_pdl(k_panel<T, 32>, dim3(gx, nf), 256, 0, s, fd, st, fronts);
  else
    launch_pdl(k_panel<T, 64>, dim3(gx, nf), 256, 0, s, fd, st, fronts);
  note_launches(1);
}
template <typename T>
void launch_syrk_contrib(FrontDesc<T>* fd, const FrontState* st, const int* fronts, int nf,
                         int max_tiles, cudaStream_t s) {
  int gx = max_tiles < 1 ? 1 : (max_tiles > 4096 ? 4096 : max_tiles);
  { k_syrk<T, 1><<<dim3(gx, nf), 256, 0, s>>>(fd, st, fronts); note_launches(1); }
}

template void launch_syrk_panel<double>(FrontDesc<double>*, const FrontState*, const int*, int, int, cudaStream_t);
template void launch_syrk_panel<float>(FrontDesc<float>*, const FrontState*, const int*, int, int, cudaStream_t);
template void launch_syrk_contrib<double>(FrontDesc<double>*, const FrontState*, const int*, int, int, cudaStream_t);
template void launch_syrk_contrib<float>(FrontDesc<float>*, const FrontState*, const int*, int, int, cudaStream_t);

}  // namespace ssids300
