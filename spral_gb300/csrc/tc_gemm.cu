// Contribution-block Schur update on the 5th-generation tensor cores.
//
//   C(r, c) -= sum_k A(r, k) B(c, k)      (lower part, r >= c, or full)
//
// with A = L21 and B = L21 D of a front (FP32 factors of the mixed-precision
// path).  FP32-class accuracy comes from split products: each FP32 value x is
// written as x = hi + lo with hi = tf32(x) and lo = tf32(x - hi), and
//   A B^T ~ Ahi Bhi^T + Ahi Blo^T + Alo Bhi^T.
// k_split writes A' and B' K-major (row-major) with, per 32-deep k-tile, the
// 32 hi values then the 32 lo values (ld = 64 x k-tiles); k_tc_gemm is a
// persistent kernel that computes 128 x BN tiles of the result (BN = 256,
// 128 or 64, chosen per launch by the autotuner): per k-tile it loads the
// hi and lo halves of A (128 rows) and B (BN rows) with TMA (128-byte
// swizzle) through an mbarrier pipeline of 192 KiB (2, 3 or 4 stages) and
// issues the three products of the tile from them into
// tcgen05.mma.kind::tf32 (M = 128, N = BN, FP32 accumulators in TMEM), then
// subtracts the result from C.  Keeping hi and lo once each, instead of the
// three operand copies of a 3K-deep GEMM, reads two thirds of the operand
// bytes per tensor flop.
//
// Accumulation: the tensor cores accumulate at most `chunk` k-tiles
// (96 * chunk split products) in TMEM; the epilogue warps then add that
// partial sum into registers with round-to-nearest FP32 adds.  This keeps
// the tensor cores' internal accumulation short and recovers FP32-class
// accuracy for deep updates (the contribution of a front with nelim
// eliminated columns is 3 * nelim split products deep).
//
// Every mbarrier wait is bounded; on timeout the CTA records an error in
// the status word, waits (bounded) for its in-flight copies and MMAs, frees
// its TMEM and returns.
#include <cuda.h>
#include <cstdint>
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <vector>

#include "spral_ssids_gpu.h"
#include "ssids_gpu.cuh"

namespace ssids300 {

namespace {

constexpr int TC_M = 128, TC_K = 32;  // K = 32 fp32 = 128 bytes
constexpr int TC_AH_BYTES = TC_M * TC_K * 4;  // 16 KiB: the hi (or lo) half of A per stage
constexpr int TC_A_BYTES = 2 * TC_AH_BYTES;   // A hi then A lo
constexpr int TC_RING_BYTES = 192 << 10;      // the k-tile ring of every tile width
// tile width BN: B bytes per stage (hi then lo halves of BN * 128 bytes),
// stages, TMEM columns (two FP32 accumulators of BN columns; a power of two
// >= 32 as tcgen05.alloc needs)
template <int BN>
struct TcShape {
  static_assert(BN == 64 || BN == 128 || BN == 256, "tile widths of the kernel");
  static constexpr int BH_BYTES = BN * TC_K * 4;
  static constexpr int B_BYTES = 2 * BH_BYTES;
  static constexpr int STAGES = TC_RING_BYTES / (TC_A_BYTES + B_BYTES);
  static constexpr uint32_t TMEM_COLS = 2 * BN;
};
constexpr int TC_EPI_WARPS = 8;              // two per TMEM lane quarter
constexpr int TC_EPI_THREADS = 32 * TC_EPI_WARPS;
constexpr int TC_THREADS = 64 + TC_EPI_THREADS;
// try_wait rounds before a wait gives up (each round may suspend briefly);
// no legitimate wait in the pipeline comes close
constexpr long long TC_WAIT_LIMIT = 1LL << 24;

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count));
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
               "r"(bytes)
               : "memory");
}

__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

__device__ __forceinline__ bool mbar_try(uint32_t a, uint32_t parity) {
  uint32_t done;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
      " selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(done)
      : "r"(a), "r"(parity)
      : "memory");
  return done != 0;
}

// Bounded wait for the phase with the given parity.  Gives up (returns
// false) after TC_WAIT_LIMIT rounds, setting the CTA's abort flag, or as
// soon as another role has set it.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, volatile int* abort) {
  const uint32_t a = smem_u32(bar);
  for (long long it = 0; it < TC_WAIT_LIMIT; ++it) {
    if (mbar_try(a, parity)) return true;
    if ((it & 31) == 31 && *abort) return false;
  }
  *abort = 1;
  return false;
}

// Bounded wait that ignores the abort flag (used to drain after an abort).
__device__ __forceinline__ bool mbar_wait_plain(uint64_t* bar, uint32_t parity) {
  const uint32_t a = smem_u32(bar);
  for (long long it = 0; it < TC_WAIT_LIMIT; ++it)
    if (mbar_try(a, parity)) return true;
  return false;
}

// arrive on `bar` once every tcgen05 operation issued so far by this thread
// has completed
__device__ __forceinline__ void mma_commit(uint64_t* bar) {
  asm volatile(
      "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
          smem_u32(bar))
      : "memory");
}

// 16 consecutive FP32 columns of this warp's 32 TMEM lanes (one lane per thread)
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, uint32_t (&v)[16]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,"
      "%14,%15}, [%16];"
      : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]),
        "=r"(v[7]), "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]),
        "=r"(v[14]), "=r"(v[15])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* map, int x, int y,
                                            uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%2, %3}], [%4];" ::"r"(smem_u32(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(smem_u32(bar))
      : "memory");
}

// shared-memory matrix descriptor: K-major, 128-byte swizzle, 8-row atoms of
// 1024 bytes (stride byte offset), descriptor version 1
__device__ __forceinline__ uint64_t smem_desc_sw128(uint32_t saddr) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr >> 4) & 0x3FFF);
  d |= (uint64_t)1 << 16;                  // leading byte offset (unused for swizzled K-major)
  d |= (uint64_t)(1024 >> 4) << 32;        // stride byte offset
  d |= (uint64_t)1 << 46;                  // version
  d |= (uint64_t)2 << 61;                  // 128-byte swizzle
  return d;
}

// instruction descriptor: D = F32, A = B = TF32, both K-major, N = BN, M = 128
template <int BN>
__host__ __device__ constexpr uint32_t idesc_tf32() {
  return (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(BN >> 3) << 17) |
         ((uint32_t)(TC_M >> 4) << 24);
}

__device__ __forceinline__ float to_tf32(float x) {
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
  return __uint_as_float(r);
}

}  // namespace

// ---------------------------------------------------------------------------
// Split operands.  For row r < rows and k < kval, k = 32 t + j: dst[r*ld +
// 64 t + j] = hi and dst[r*ld + 64 t + 32 + j] = lo of src(r, k) (both
// sides alike); entries of k >= kval are zero.  src is column-major
// (ld_src); kpad = 64 x k-tiles.
// ---------------------------------------------------------------------------
struct SplitJob {
  const float* src;
  float* dst;
  int rows, kval, kpad, ld_src, ld_dst, is_b;
  const int* kval_dev;  // nullptr or device-side effective depth (<= kval)
};

__global__ void k_split(const SplitJob* jobs) {
  const SplitJob j = jobs[blockIdx.z];
  __shared__ float tile[32][33];
  const int r0 = blockIdx.x * 32, k0 = blockIdx.y * 32;
  if (r0 >= j.rows || 2 * k0 >= j.kpad) return;  // uniform per CTA
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;  // 32 x 8
  const int kval = j.kval_dev ? min(j.kval, *j.kval_dev) : j.kval;
  for (int i = ty; i < 32; i += 8) {
    const int r = r0 + tx, k = k0 + i;
    tile[i][tx] = (r < j.rows && k < kval) ? j.src[(int64_t)k * j.ld_src + r] : 0.f;
  }
  __syncthreads();
  for (int i = ty; i < 32; i += 8) {
    const int r = r0 + i;
    if (r >= j.rows) continue;
    const float x = tile[tx][i];
    const float hi = to_tf32(x);
    const float lo = to_tf32(x - hi);
    // k0 is a multiple of 32: this CTA's k-tile is k0 / 32
    float* d = j.dst + (int64_t)r * j.ld_dst + 2 * k0 + tx;
    d[0] = hi;
    d[32] = lo;
  }
}

// ---------------------------------------------------------------------------
// GEMM jobs: one per front; the tiles of all results are enumerated by the
// host into one flat list (job index, tile row, tile col), longest first.
// ---------------------------------------------------------------------------
struct TcJob {
  float* C;
  int ldc, M, N;
  int kpad;        // row length of A', B': 64 per 32-deep k-tile
  int lower;       // 1: only r >= c is updated
  const int* kval; // nullptr or device pointer: effective depth *kval
};

// 32-deep k-tiles of a job (each: hi and lo halves, three products)
__device__ __forceinline__ int tile_ktiles(const TcJob& j) {
  int nk = j.kpad / (2 * TC_K);
  if (j.kval) nk = min(nk, (max(*j.kval, 0) + TC_K - 1) / TC_K);
  return nk;
}

// Persistent kernel, one CTA per SM, 320 threads:
//   warp 0 lane 0   TMA producer (hi and lo halves of A' and B' per k-tile
//                   into a ring of STAGES)
//   warp 1 lane 0   MMA issuer (tcgen05.mma into one of two TMEM
//                   accumulators, the k-tile's three split products)
//   warps 2..9      accumulate / epilogue (warp w reads TMEM lanes 32*(w%4)..)
// The k range of a tile is cut into chunks of `chunk` k-tiles (0 = one chunk).
// Each chunk is accumulated by the tensor cores in a fresh TMEM accumulator;
// the epilogue warps add it, rounding to nearest, into a per-thread register
// row of the tile, so the tensor cores' own accumulation spans at most
// 96 * chunk products.  Two accumulators let the MMAs of the next chunk (or
// tile) run while the previous one is drained.
template <int BN>
__global__ void __launch_bounds__(TC_THREADS, 1)
    k_tc_gemm(const TcJob* jobs, const int4* tiles, int ntiles, const CUtensorMap* maps,
              int chunk, int* status) {
  constexpr int TC_STAGES = TcShape<BN>::STAGES;
  constexpr int TC_B_BYTES = TcShape<BN>::B_BYTES;
  constexpr int TC_BH_BYTES = TcShape<BN>::BH_BYTES;
  constexpr uint32_t TC_TMEM_COLS = TcShape<BN>::TMEM_COLS;
  constexpr int HALF = BN / 2;  // columns of a tile per epilogue warp
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  unsigned char* smem = (unsigned char*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  unsigned char* sA = smem;
  unsigned char* sB = smem + TC_STAGES * TC_A_BYTES;
  uint64_t* full = reinterpret_cast<uint64_t*>(smem + TC_STAGES * (TC_A_BYTES + TC_B_BYTES));
  uint64_t* empty = full + TC_STAGES;
  uint64_t* accf = empty + TC_STAGES;  // accumulator b holds a finished chunk
  uint64_t* acce = accf + 2;           // accumulator b has been drained
  uint64_t* drain = acce + 2;          // all MMAs of this CTA have completed
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(drain + 1);
  int* s_abort = reinterpret_cast<int*>(tmem_slot + 1);
  int* s_issued = s_abort + 1;

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (threadIdx.x == 0) {
    for (int s = 0; s < TC_STAGES; ++s) { mbar_init(&full[s], 1); mbar_init(&empty[s], 1); }
    for (int b = 0; b < 2; ++b) { mbar_init(&accf[b], 1); mbar_init(&acce[b], TC_EPI_THREADS); }
    mbar_init(drain, 1);
    *s_abort = 0;
    *s_issued = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(tmem_slot)),
                 "r"(TC_TMEM_COLS));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;");
  const uint32_t tmem = *tmem_slot;
  volatile int* abort_flag = s_abort;

  if (warp == 0) {
    if (lane == 0) {
      // ---- producer ----
      uint32_t it = 0;
      bool ok = true;
      for (int t = blockIdx.x; t < ntiles && ok; t += gridDim.x) {
        const int4 tl = tiles[t];
        const int nk = tile_ktiles(jobs[tl.x]);
        const CUtensorMap* mapA = maps + 2 * tl.x;
        const CUtensorMap* mapB = mapA + 1;
        for (int kt = 0; kt < nk; ++kt, ++it) {
          const uint32_t s = it % TC_STAGES;
          if (it >= (uint32_t)TC_STAGES &&
              !mbar_wait(&empty[s], ((it / TC_STAGES) - 1) & 1, abort_flag)) {
            ok = false;
            break;
          }
          mbar_expect_tx(&full[s], TC_A_BYTES + TC_B_BYTES);
          unsigned char* a = sA + s * TC_A_BYTES;
          unsigned char* b = sB + s * TC_B_BYTES;
          const int x = kt * 2 * TC_K;  // hi half at x, lo half at x + 32
          tma_load_2d(a, mapA, x, tl.y * TC_M, &full[s]);
          tma_load_2d(a + TC_AH_BYTES, mapA, x + TC_K, tl.y * TC_M, &full[s]);
          tma_load_2d(b, mapB, x, tl.z * BN, &full[s]);
          tma_load_2d(b + TC_BH_BYTES, mapB, x + TC_K, tl.z * BN, &full[s]);
        }
      }
      *s_issued = (int)it;
    }
  } else if (warp == 1) {
    if (lane == 0) {
      // ---- MMA issuer ----
      const uint32_t idesc = idesc_tf32<BN>();
      uint32_t it = 0, ch = 0;
      bool ok = true;
      for (int t = blockIdx.x; t < ntiles && ok; t += gridDim.x) {
        const int nk = tile_ktiles(jobs[tiles[t].x]);
        const int per = chunk > 0 ? chunk : max(nk, 1);
        for (int k0 = 0; k0 < nk && ok; k0 += per, ++ch) {
          const uint32_t b = ch & 1;
          if (ch >= 2 && !mbar_wait(&acce[b], ((ch >> 1) - 1) & 1, abort_flag)) {
            ok = false;
            break;
          }
          asm volatile("tcgen05.fence::after_thread_sync;");
          const uint32_t dacc = tmem + b * BN;
          const int k1 = min(nk, k0 + per);
          for (int kt = k0; kt < k1; ++kt, ++it) {
            const uint32_t s = it % TC_STAGES;
            if (!mbar_wait(&full[s], (it / TC_STAGES) & 1, abort_flag)) { ok = false; break; }
            asm volatile("tcgen05.fence::after_thread_sync;");
            const uint32_t ahi = smem_u32(sA + s * TC_A_BYTES), alo = ahi + TC_AH_BYTES;
            const uint32_t bhi = smem_u32(sB + s * TC_B_BYTES), blo = bhi + TC_BH_BYTES;
            // the three split products Ahi Bhi, Ahi Blo, Alo Bhi of the k-tile
#pragma unroll
            for (int pr = 0; pr < 3; ++pr) {
              const uint32_t a0 = pr == 2 ? alo : ahi, b0 = pr == 1 ? blo : bhi;
#pragma unroll
              for (int kk = 0; kk < TC_K / 8; ++kk) {  // 8 tf32 = 32 bytes per MMA
                const uint64_t ad = smem_desc_sw128(a0 + kk * 32);
                const uint64_t bd = smem_desc_sw128(b0 + kk * 32);
                const uint32_t acc = (kt > k0 || pr > 0 || kk > 0) ? 1u : 0u;
                asm volatile(
                    "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
                    " tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}\n" ::"r"(dacc),
                    "l"(ad), "l"(bd), "r"(idesc), "r"(acc));
              }
            }
            // stage s is free once these MMAs have read it
            mma_commit(&empty[s]);
          }
          if (ok) mma_commit(&accf[b]);
        }
      }
      // every MMA issued above has completed once `drain` flips
      mma_commit(drain);
      (void)mbar_wait_plain(drain, 0);
    }
  } else {
    // ---- accumulate + epilogue ----
    // warp w (2..9) reads TMEM lane quarter w % 4 and owns the column half
    // (w - 2) / 4 of the tile: one register row of BN / 2 sums per thread
    const int q = warp & 3;
    const int half = (warp - 2) >> 2;
    uint32_t ch = 0;
    bool ok = true;
    for (int t = blockIdx.x; t < ntiles && ok; t += gridDim.x) {
      const int4 tl = tiles[t];
      const TcJob job = jobs[tl.x];
      const int nk = tile_ktiles(job);
      if (nk == 0) continue;
      const int per = chunk > 0 ? chunk : nk;
      float acc[HALF];
#pragma unroll
      for (int j = 0; j < HALF; ++j) acc[j] = 0.f;
      for (int k0 = 0; k0 < nk; k0 += per, ++ch) {
        const uint32_t b = ch & 1;
        // the TMEM loads below are warp-collective: decide as a warp
        const bool got = mbar_wait(&accf[b], (ch >> 1) & 1, abort_flag);
        if (!__all_sync(0xffffffffu, got)) { *abort_flag = 1; ok = false; break; }
        asm volatile("tcgen05.fence::after_thread_sync;");
        const uint32_t base = tmem + ((uint32_t)(q * 32) << 16) + b * BN + half * HALF;
#pragma unroll
        for (int cb = 0; cb < HALF; cb += 16) {
          uint32_t v[16];
          tmem_ld16(base + (uint32_t)cb, v);
#pragma unroll
          for (int j = 0; j < 16; ++j) acc[cb + j] += __uint_as_float(v[j]);
        }
        asm volatile("tcgen05.fence::before_thread_sync;");
        mbar_arrive(&acce[b]);
      }
      if (!ok) break;
      const int r = tl.y * TC_M + q * 32 + lane;
      if (r < job.M) {
        const int col0 = tl.z * BN + half * HALF;
        float* crow = job.C + r;
        // 8 columns at a time: all loads in flight before the stores
        const int64_t ldc = job.ldc;
        const float* cbase = crow + col0 * ldc;
#pragma unroll
        for (int cb = 0; cb < HALF; cb += 8) {
          float cv[8];
#pragma unroll
          for (int j = 0; j < 8; ++j) {
            const int c = col0 + cb + j;
            cv[j] = (c < job.N && (!job.lower || r >= c)) ? cbase[(cb + j) * ldc] : 0.f;
          }
#pragma unroll
          for (int j = 0; j < 8; ++j) {
            const int c = col0 + cb + j;
            if (c < job.N && (!job.lower || r >= c))
              const_cast<float*>(cbase)[(cb + j) * ldc] = cv[j] - acc[cb + j];
          }
        }
      }
    }
  }
  __syncthreads();
  if (*abort_flag) {
    if (threadIdx.x == 0) {
      atomicExch(status, kDevBadState);
      // let the copies still in flight land before shared memory is released
      const int issued = *s_issued;
      for (int it = max(0, issued - TC_STAGES); it < issued; ++it)
        (void)mbar_wait_plain(&full[it % TC_STAGES], (it / TC_STAGES) & 1);
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                 "r"(TC_TMEM_COLS));
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
// The tensor-map encoder is a driver entry point; it is looked up through the
// runtime so that the library does not link the driver library directly
// (hosts without a GPU driver can still load it for the CPU-side tests).
typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*,
                                  const cuuint64_t*, const cuuint64_t*, const cuuint32_t*,
                                  const cuuint32_t*, CUtensorMapInterleave, CUtensorMapSwizzle,
                                  CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

static EncodeTiledFn encode_fn() {
  static EncodeTiledFn fn = nullptr;
  if (!fn) {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault,
                                         &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<EncodeTiledFn>(p);
    else
      cudaGetLastError();
  }
  return fn;
}

static CUresult encode_kmajor(CUtensorMap* map, const float* base, int rows, int kpad, int ld,
                              int box_rows) {
  EncodeTiledFn fn = encode_fn();
  if (!fn) return CUDA_ERROR_NOT_FOUND;
  cuuint64_t gdim[2] = {(cuuint64_t)kpad, (cuuint64_t)rows};
  cuuint64_t gstride[1] = {(cuuint64_t)ld * sizeof(float)};
  cuuint32_t box[2] = {(cuuint32_t)TC_K, (cuuint32_t)box_rows};
  cuuint32_t estride[2] = {1, 1};
  return fn(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, (void*)base, gdim, gstride, box, estride,
            CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
            CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
}

// dynamic shared memory of k_tc_gemm<BN>: alignment slack, the ring, the
// barriers (full and empty per stage, two accumulator pairs, drain) and the
// TMEM slot and flags
template <int BN>
static size_t tc_gemm_smem_bytes() {
  constexpr int st = TcShape<BN>::STAGES;
  return 1024 + (size_t)st * (TC_A_BYTES + TcShape<BN>::B_BYTES) + (2 * st + 5) * 8 + 16;
}
static size_t tc_gemm_smem_bytes(int bn) {
  return bn == 64 ? tc_gemm_smem_bytes<64>()
                  : bn == 128 ? tc_gemm_smem_bytes<128>() : tc_gemm_smem_bytes<256>();
}

bool tc_tile_width_ok(int bn) { return bn == 64 || bn == 128 || bn == 256; }

// one launch of k_tc_gemm with the plan's tile width
static void launch_tc_kernel(const TcPlan& plan, const char* d, int chunk, int* status,
                             cudaStream_t s) {
  const TcJob* jobs = reinterpret_cast<const TcJob*>(d + plan.o_jobs);
  const int4* tiles = reinterpret_cast<const int4*>(d + plan.o_tiles);
  const CUtensorMap* maps = reinterpret_cast<const CUtensorMap*>(d + plan.o_maps);
  const size_t sm = tc_gemm_smem_bytes(plan.bn);
  if (plan.bn == 64)
    k_tc_gemm<64><<<plan.grid, TC_THREADS, sm, s>>>(jobs, tiles, plan.ntiles, maps, chunk, status);
  else if (plan.bn == 128)
    k_tc_gemm<128><<<plan.grid, TC_THREADS, sm, s>>>(jobs, tiles, plan.ntiles, maps, chunk, status);
  else
    k_tc_gemm<256><<<plan.grid, TC_THREADS, sm, s>>>(jobs, tiles, plan.ntiles, maps, chunk, status);
  note_launches(1);
}


size_t tc_gemm_scratch_bytes(const std::vector<TcProblem>& ps) {
  size_t b = 0;
  for (auto& p : ps) {
    const size_t kpad = (size_t)((p.kmax + TC_K - 1) / TC_K) * 2 * TC_K;
    b += ((size_t)p.M * kpad * 4 + 255) / 256 * 256;
    b += ((size_t)p.N * kpad * 4 + 255) / 256 * 256;
  }
  return b + 256;
}

TcBuffers::~TcBuffers() {
  if (uploaded) cudaEventSynchronize(uploaded);
  cudaFreeHost(h_stage);
  cudaFree(d_stage);
  if (uploaded) cudaEventDestroy(uploaded);
}

static size_t up64(size_t b) { return (b + 63) & ~size_t(63); }

int tc_gemm_prepare(const std::vector<TcProblem>& ps, void* scratch, TcPlan& plan, int bn) {
  plan = TcPlan{};
  if (bn == 0) bn = tc_tile_width(ps);
  if (!tc_tile_width_ok(bn)) return -4;
  plan.bn = bn;
  if (ps.empty()) return 0;
  std::vector<SplitJob> sj;
  std::vector<TcJob> jobs;
  std::vector<int4> tiles;
  std::vector<CUtensorMap> maps;
  char* sp = static_cast<char*>(scratch);
  sp = (char*)(((uintptr_t)sp + 255) & ~(uintptr_t)255);
  int maxr = 0, maxk = 0;
  for (size_t i = 0; i < ps.size(); ++i) {
    const TcProblem& p = ps[i];
    const int kpad = (p.kmax + TC_K - 1) / TC_K * 2 * TC_K;  // hi and lo per k-tile
    float* a2 = (float*)sp; sp += ((size_t)p.M * kpad * 4 + 255) / 256 * 256;
    float* b2 = (float*)sp; sp += ((size_t)p.N * kpad * 4 + 255) / 256 * 256;
    sj.push_back({p.A, a2, p.M, p.kmax, kpad, p.lda, kpad, 0, p.kval_dev});
    sj.push_back({p.B, b2, p.N, p.kmax, kpad, p.ldb, kpad, 1, p.kval_dev});
    maxr = std::max(maxr, std::max(p.M, p.N));
    maxk = std::max(maxk, kpad / 2);  // source columns of the split
    CUtensorMap ma, mb;
    if (encode_kmajor(&ma, a2, p.M, kpad, kpad, TC_M) != CUDA_SUCCESS) return -2;
    if (encode_kmajor(&mb, b2, p.N, kpad, kpad, bn) != CUDA_SUCCESS) return -2;
    maps.push_back(ma);
    maps.push_back(mb);
    jobs.push_back({p.C, p.ldc, p.M, p.N, kpad, p.lower, p.kval_dev});
    const int tm = (p.M + TC_M - 1) / TC_M, tn = (p.N + bn - 1) / bn;
    for (int ti = 0; ti < tm; ++ti)
      for (int tj = 0; tj < tn; ++tj) {
        if (p.lower && (tj * bn > ti * TC_M + TC_M - 1)) continue;  // tile above diagonal
        tiles.push_back(make_int4((int)i, ti, tj, kpad));
      }
  }
  // deepest tiles first: the persistent CTAs take tiles round-robin
  std::stable_sort(tiles.begin(), tiles.end(),
                   [](const int4& a, const int4& b) { return a.w > b.w; });
  plan.o_jobs = up64(sj.size() * sizeof(SplitJob));
  plan.o_tiles = plan.o_jobs + up64(jobs.size() * sizeof(TcJob));
  plan.o_maps = plan.o_tiles + up64(tiles.size() * sizeof(int4));
  const size_t total = plan.o_maps + maps.size() * sizeof(CUtensorMap);
  plan.blob.assign(total, 0);
  memcpy(plan.blob.data(), sj.data(), sj.size() * sizeof(SplitJob));
  memcpy(plan.blob.data() + plan.o_jobs, jobs.data(), jobs.size() * sizeof(TcJob));
  memcpy(plan.blob.data() + plan.o_tiles, tiles.data(), tiles.size() * sizeof(int4));
  memcpy(plan.blob.data() + plan.o_maps, maps.data(), maps.size() * sizeof(CUtensorMap));
  plan.nsplit = (int)sj.size();
  plan.ntiles = (int)tiles.size();
  plan.maxr = maxr;
  plan.maxk = maxk;
  // launch configuration, fixed here so that tc_gemm_launch only enqueues
  int dev = 0, nsm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  plan.grid = std::min(plan.ntiles, std::max(nsm, 1));
  cudaError_t e;
  if (bn == 64)
    e = cudaFuncSetAttribute(k_tc_gemm<64>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)tc_gemm_smem_bytes<64>());
  else if (bn == 128)
    e = cudaFuncSetAttribute(k_tc_gemm<128>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)tc_gemm_smem_bytes<128>());
  else
    e = cudaFuncSetAttribute(k_tc_gemm<256>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)tc_gemm_smem_bytes<256>());
  return e == cudaSuccess ? 0 : -3;
}

int tc_gemm_launch(const TcPlan& plan, const void* d_blob, int* status, cudaStream_t s, int chunk) {
  if (plan.nsplit == 0) return 0;
  const char* d = static_cast<const char*>(d_blob);
  dim3 sg((plan.maxr + 31) / 32, (plan.maxk + 31) / 32, (unsigned)plan.nsplit);
  k_split<<<sg, 256, 0, s>>>(reinterpret_cast<const SplitJob*>(d));
  note_launches(1);
  if (plan.ntiles > 0) launch_tc_kernel(plan, d, chunk, status, s);
  return cudaGetLastError() == cudaSuccess ? 0 : -3;
}

int tc_gemm_run(const std::vector<TcProblem>& ps, void* scratch, TcBuffers& buf, int* status,
                cudaStream_t s, int chunk, float* ms_split, float* ms_gemm, int bn) {
  if (ps.empty()) return 0;
  TcPlan plan;
  const int rp = tc_gemm_prepare(ps, scratch, plan, bn);
  if (rp != 0) return rp;
  // one upload of all descriptors through a pinned staging buffer
  const size_t total = plan.blob.size();
  if (!buf.uploaded && cudaEventCreateWithFlags(&buf.uploaded, cudaEventDisableTiming) != cudaSuccess)
    return -1;
  if (cudaEventSynchronize(buf.uploaded) != cudaSuccess) return -3;  // staging free again
  if (total > buf.cap) {
    cudaFreeHost(buf.h_stage);
    cudaFree(buf.d_stage);
    buf.h_stage = buf.d_stage = nullptr;
    buf.cap = 0;
    const size_t nc = std::max(total, (size_t)64 << 10);
    if (cudaMallocHost(&buf.h_stage, nc) != cudaSuccess) return -1;
    if (cudaMalloc(&buf.d_stage, nc) != cudaSuccess) return -1;
    buf.cap = nc;
  }
  memcpy(buf.h_stage, plan.blob.data(), total);
  if (cudaMemcpyAsync(buf.d_stage, buf.h_stage, total, cudaMemcpyHostToDevice, s) != cudaSuccess)
    return -3;
  if (cudaEventRecord(buf.uploaded, s) != cudaSuccess) return -3;
  cudaEvent_t ev[3] = {nullptr, nullptr, nullptr};
  const bool timed = ms_split || ms_gemm;
  if (!timed) return tc_gemm_launch(plan, buf.d_stage, status, s, chunk);
  for (auto& e : ev) cudaEventCreate(&e);
  // split and GEMM timed separately
  TcPlan only_split = plan;
  only_split.ntiles = 0;
  cudaEventRecord(ev[0], s);
  int rc = tc_gemm_launch(only_split, buf.d_stage, status, s, chunk);
  cudaEventRecord(ev[1], s);
  if (rc == 0 && plan.ntiles > 0) {
    launch_tc_kernel(plan, static_cast<const char*>(buf.d_stage), chunk, status, s);
    rc = cudaGetLastError() == cudaSuccess ? 0 : -3;
  }
  cudaEventRecord(ev[2], s);
  cudaEventSynchronize(ev[2]);
  if (ms_split) cudaEventElapsedTime(ms_split, ev[0], ev[1]);
  if (ms_gemm) cudaEventElapsedTime(ms_gemm, ev[1], ev[2]);
  for (auto& e : ev) cudaEventDestroy(e);
  return rc;
}

// Failure-detection probe: one CTA waits on an mbarrier that nothing will
// ever complete, with the pipeline's bounded-wait loop cut to `limit`
// rounds; the wait gives up, records kDevBadState in *status and the CTA
// returns normally, leaving the context usable.
__global__ void k_mbar_timeout_probe(long long limit, int* status) {
  __shared__ __align__(8) uint64_t bar;
  if (threadIdx.x == 0) {
    mbar_init(&bar, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    const uint32_t a = smem_u32(&bar);
    bool done = false;
    for (long long it = 0; it < limit && !done; ++it) done = mbar_try(a, 0);
    if (!done) atomicExch(status, kDevBadState);
  }
}

}  // namespace ssids300

// ---------------------------------------------------------------------------
// Stand-alone entry point for tests and measurements: C (M x N, col-major,
// ldc) -= A B^T with A (M x K, lda) and B (N x K, ldb) column-major FP32, all
// device pointers.  chunk < 0 selects the default accumulation chunk.  With
// reps > 0 and ms != nullptr the update is repeated reps times and
// ms[0], ms[1] receive the mean split and GEMM times of the repetitions.
// ---------------------------------------------------------------------------
extern "C" int spral_ssids_gpu_mbar_timeout_probe(int rounds) {
  int* d = nullptr;
  if (cudaMalloc(&d, sizeof(int)) != cudaSuccess) { cudaGetLastError(); return -50; }
  int h = 0;
  cudaMemset(d, 0, sizeof(int));
  ssids300::k_mbar_timeout_probe<<<1, 32>>>((long long)std::max(rounds, 1), d);
  const cudaError_t e = cudaMemcpy(&h, d, sizeof(int), cudaMemcpyDeviceToHost);
  cudaFree(d);
  if (e != cudaSuccess) { cudaGetLastError(); return -51; }
  return h == ssids300::kDevBadState ? -51 : 0;  // a wait that gave up: SSIDS_ERROR_CUDA_UNKNOWN
}

extern "C" int spral_ssids_gpu_tc_gemm_f32(int M, int N, int K, const float* A, int lda,
                                           const float* B, int ldb, float* C, int ldc, int lower,
                                           int chunk, int reps, float* ms) {
  return spral_ssids_gpu_tc_gemm_f32_bn(M, N, K, A, lda, B, ldb, C, ldc, lower, chunk, reps, ms,
                                        0);
}

extern "C" int spral_ssids_gpu_tc_gemm_f32_bn(int M, int N, int K, const float* A, int lda,
                                              const float* B, int ldb, float* C, int ldc,
                                              int lower, int chunk, int reps, float* ms, int bn) {
  using namespace ssids300;
  if (M < 0 || N < 0 || K < 0 || lda < M || ldb < N || ldc < M) return -1;
  if (bn != 0 && !tc_tile_width_ok(bn)) return -4;
  if (chunk < 0) chunk = kTcChunk;
  std::vector<TcProblem> ps(1);
  ps[0] = {A, lda, B, ldb, C, ldc, M, N, K, nullptr, lower};
  void* scratch = nullptr;
  int* status = nullptr;
  const size_t bytes = tc_gemm_scratch_bytes(ps);
  if (cudaMalloc(&scratch, bytes) != cudaSuccess) return -50;
  if (cudaMalloc(&status, sizeof(int)) != cudaSuccess) { cudaFree(scratch); return -50; }
  cudaMemset(status, 0, sizeof(int));
  int rc = 0;
  {
    TcBuffers buf;
    const int n = std::max(reps, 1);
    double tsplit = 0, tgemm = 0;
    for (int i = 0; i < n && rc == 0; ++i) {
      float a = 0, b = 0;
      rc = tc_gemm_run(ps, scratch, buf, status, 0, chunk, ms ? &a : nullptr, ms ? &b : nullptr,
                       bn);
      tsplit += a;
      tgemm += b;
    }
    if (cudaDeviceSynchronize() != cudaSuccess) rc = -51;
    if (ms) { ms[0] = (float)(tsplit / n); ms[1] = (float)(tgemm / n); }
  }
  int hs = 0;
  cudaMemcpy(&hs, status, sizeof(int), cudaMemcpyDeviceToHost);
  if (rc == 0 && hs != 0) rc = -52;
  cudaFree(scratch);
  cudaFree(status);
  return rc;
}
