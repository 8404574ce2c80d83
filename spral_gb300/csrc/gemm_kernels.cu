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

// Tile t of the lower triangle of a tr x tr grid of tiles, numbered down
// the columns: column tj holds tiles tj .. tr-1 and starts at
// tj*tr - tj*(tj-1)/2.  The root of the quadratic gives tj up to rounding;
// the two loops correct it.
__device__ __forceinline__ void tri_tile(int t, int tr, int& ti, int& tj) {
  const float b = 2.0f * tr + 1.0f;
  int j = (int)((b - sqrtf(fmaxf(b * b - 8.0f * t, 0.0f))) * 0.5f);
  j = max(0, min(j, tr - 1));
  auto first = [tr](int c) { return c * tr - c * (c - 1) / 2; };
  while (j > 0 && first(j) > t) --j;
  while (j + 1 < tr && first(j + 1) <= t) ++j;
  tj = j;
  ti = j + (t - first(j));
}

__device__ __forceinline__ void cp_async4(float* dst, const float* src, bool valid) {
  const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;\n" ::"r"(d), "l"(src),
               "r"(valid ? 4 : 0)
               : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory"); }

// FP32 contribution update, C -= A B^T on the lower triangle, depth K
// staged 32 columns at a time.  The update of a thin supernode (K = 32..64
// against a contribution block thousands of rows wide) streams C through
// HBM while needing most of the FP32 FMA rate to keep up, so the kernel
// overlaps the two and keeps its instruction count down:
//  * a CTA walks its tiles in a grid-stride loop, copies the next (tile,
//    batch) of A and B into the other shared buffer with cp.async while it
//    computes on the current one, and reads the next tile's C into
//    registers during the last batch of the current tile;
//  * tiles inside C (all but the last row and column of tiles) take no
//    bounds tests; the diagonal tiles test row >= column on the store only
//    (C is a full cm x cm array, so reading its upper part is in bounds);
//  * shared layout: position p of a 64-row batch holds row
//    (p % 4) * 16 + p / 4, so the 32 lanes of a copy write 32 consecutive
//    banks and thread tx reads its rows tx, tx+16, tx+32, tx+48 as one
//    float4 (likewise for the columns of B).
constexpr int kF32Threads = 256;

template <typename T>
__device__ __forceinline__ void contrib_f32(const SyrkJob<T>& j, int total, int tr) {
  constexpr int KC = 32, NT = kF32Threads, CP = TM * KC / NT;
  __shared__ __align__(16) float Ap[2][KC][TM];
  __shared__ __align__(16) float Bp[2][KC][TM];
  const int tid = threadIdx.x;
  const int tx = tid & 15, ty = tid >> 4;
  const int nb = (j.K + KC - 1) / KC;
  auto issue = [&](int t, int b, int buf) {
    int ti, tj;
    tri_tile(t, tr, ti, tj);
    const int row0 = ti * TM, col0 = tj * TM, k0 = b * KC;
    const bool full = row0 + TM <= j.M && col0 + TM <= j.N && k0 + KC <= j.K;
#pragma unroll
    for (int q = 0; q < CP; ++q) {
      const int idx = tid + NT * q;
      const int kk = idx / TM, p = idx % TM;
      const int rr = (p & 3) * 16 + (p >> 2);
      const int k = k0 + kk, r = row0 + rr, c = col0 + rr;
      const float* sa = j.A + (int64_t)k * j.lda + r;
      const float* sb = j.B + (int64_t)k * j.ldb + c;
      if (full) {
        cp_async4(&Ap[buf][kk][p], sa, true);
        cp_async4(&Bp[buf][kk][p], sb, true);
      } else {
        const bool va = k < j.K && r < j.M, vb = k < j.K && c < j.N;
        cp_async4(&Ap[buf][kk][p], va ? sa : j.A, va);
        cp_async4(&Bp[buf][kk][p], vb ? sb : j.B, vb);
      }
    }
  };
  auto load_c = [&](int t, float (&cv)[4][4]) {
    int ti, tj;
    tri_tile(t, tr, ti, tj);
    const int row0 = ti * TM, col0 = tj * TM;
    if (row0 + TM <= j.M && col0 + TM <= j.N) {
      const float* base = j.C + (int64_t)(col0 + ty) * j.ldc + row0 + tx;
#pragma unroll
      for (int y = 0; y < 4; ++y)
#pragma unroll
        for (int x = 0; x < 4; ++x) cv[x][y] = base[(int64_t)16 * y * j.ldc + 16 * x];
    } else {
#pragma unroll
      for (int y = 0; y < 4; ++y) {
        const int c = col0 + ty + 16 * y;
#pragma unroll
        for (int x = 0; x < 4; ++x) {
          const int r = row0 + tx + 16 * x;
          cv[x][y] = (r < j.M && c < j.N) ? j.C[(int64_t)c * j.ldc + r] : 0.0f;
        }
      }
    }
  };
  int t = blockIdx.x;
  if (t >= total) return;
  float cn[4][4];
  issue(t, 0, 0);
  cp_async_commit();
  load_c(t, cn);
  int buf = 0;
  for (; t < total; t += gridDim.x) {
    float acc[4][4];
#pragma unroll
    for (int x = 0; x < 4; ++x)
#pragma unroll
      for (int y = 0; y < 4; ++y) acc[x][y] = cn[x][y];
    for (int b = 0; b < nb; ++b) {
      int tn = t, bn = b + 1;
      if (bn == nb) { tn = t + gridDim.x; bn = 0; }
      if (tn < total) issue(tn, bn, buf ^ 1);
      cp_async_commit();
      if (bn == 0 && tn < total) load_c(tn, cn);
      cp_async_wait<1>();
      __syncthreads();
#pragma unroll 8
      for (int kk = 0; kk < KC; ++kk) {
        const float4 a = *reinterpret_cast<const float4*>(&Ap[buf][kk][4 * tx]);
        const float4 bq = *reinterpret_cast<const float4*>(&Bp[buf][kk][4 * ty]);
        const float av[4] = {a.x, a.y, a.z, a.w}, bv[4] = {bq.x, bq.y, bq.z, bq.w};
#pragma unroll
        for (int x = 0; x < 4; ++x)
#pragma unroll
          for (int y = 0; y < 4; ++y) acc[x][y] = fmaf(-av[x], bv[y], acc[x][y]);
      }
      __syncthreads();
      buf ^= 1;
    }
    int ti, tj;
    tri_tile(t, tr, ti, tj);
    const int row0 = ti * TM, col0 = tj * TM;
    if (row0 + TM <= j.M && col0 + TM <= j.N && ti != tj) {
      float* base = j.C + (int64_t)(col0 + ty) * j.ldc + row0 + tx;
#pragma unroll
      for (int y = 0; y < 4; ++y)
#pragma unroll
        for (int x = 0; x < 4; ++x) base[(int64_t)16 * y * j.ldc + 16 * x] = acc[x][y];
    } else {
#pragma unroll
      for (int y = 0; y < 4; ++y) {
        const int c = col0 + ty + 16 * y;
#pragma unroll
        for (int x = 0; x < 4; ++x) {
          const int r = row0 + tx + 16 * x;
          if (r < j.M && c < j.N && r >= c) j.C[(int64_t)c * j.ldc + r] = acc[x][y];
        }
      }
    }
  }
  cp_async_wait<0>();
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
  const int tr = (j.M + TM - 1) / TM;
  const int total = tr * (tr + 1) / 2;
  if constexpr (sizeof(T) == 4) {
    contrib_f32<T>(j, total, tr);
    return;
  }
  const int tid = threadIdx.x;
  const int tx = tid & 15, ty = tid >> 4;
  __shared__ T As[TK][TM + 4];
  __shared__ T Bs[TK][TM + 4];
  for (int t = blockIdx.x; t < total; t += gridDim.x) {
    int ti, tj;
    tri_tile(t, tr, ti, tj);
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
  // FP32: about four waves of the resident CTAs (four per SM) over the
  // level, so that each CTA pipelines several tiles; FP64: one tile per CTA
  // up to 4096 CTAs (its long tiles balance better in small units)
  const int cap = sizeof(T) == 4 ? std::max(1, 16 * 152 / std::max(nf, 1)) : 4096;
  int gx = max_tiles < 1 ? 1 : std::min(max_tiles, cap);
  const int threads = sizeof(T) == 4 ? kF32Threads : 256;
  { k_syrk<T, 1><<<dim3(gx, nf), threads, 0, s>>>(fd, st, fronts); note_launches(1); }
}

template void launch_syrk_contrib<double>(FrontDesc<double>*, const FrontState*, const int*, int, int, cudaStream_t);
template void launch_syrk_contrib<float>(FrontDesc<float>*, const FrontState*, const int*, int, int, cudaStream_t);

}  // namespace ssids300
