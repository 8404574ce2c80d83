// Dense per-front LDL^T with a-posteriori threshold pivoting on sm_103a.
//
// One APP step processes a block of up to 32 candidate columns [p, p+bs) of
// every active front of a level at once:
//   k_app_diag      diagonal block: complete pivoting (indefinite) or none (posdef)
//                   (semantics of block_ldlt, src/ssids/cpu/kernels/
//                   block_ldlt.hxx:290-413), FP64 arithmetic, writes L11, D^{-1}
//                   and the local permutation
//   k_app_apply     rows below: X = A21 L11^{-T}, L21 = X D^{-1} and the
//                   a-posteriori test |l| <= 1/u (apply_pivot/check_threshold,
//                   ldlt_app.cxx:316-436); X (= L21 D) is kept for the update;
//                   extra CTAs apply the block permutation to the eliminated
//                   L rows
//   k_app_panel     trailing update of the candidate columns and, in extra
//                   CTAs, the fixup: Column::adjust (ldlt_app.cxx:112-130)
//                   and, for failed columns, the restore-and-update of
//                   restore_if_required + update, computed as X_f L_ff^T
//                   (rows below) and L_ff D_f L_ff^T (diagonal block)
//   k_app_swap      failed columns are moved to the end of the APP range
// After ceil(n/32) steps k_app_finish records nelim; k_tpp finishes failed
// columns with threshold partial pivoting (ldlt_tpp.cxx:166-270) where the
// reference does (root fronts or failed_pivot_method = tpp); k_calc_ld and
// k_syrk (contrib) form the contribution block; k_stats counts inertia.
#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <type_traits>

#include "ssids_gpu.cuh"

namespace ssids300 {

namespace {

__device__ __forceinline__ double dinf() { return __longlong_as_double(0x7ff0000000000000LL); }

}  // namespace

// Reciprocal by Newton-Raphson iteration y <- y + y (1 - x y) from an FP32
// seed (each step squares the relative error: 2^-23 -> 2^-46 -> 2^-92), so
// the result is within one ulp of 1/x.  Two FP64 FMA pairs replace the long
// dependent sequence of a correctly rounded FP64 division, which matters on
// the serial path of the pivot decisions.  Arguments whose magnitude is
// outside [2^-100, 2^100] (or zero/Inf/NaN) use ordinary division.
__device__ __forceinline__ double recip_nr(double x) {
  const int e = (int)((__double_as_longlong(x) >> 52) & 0x7ff);
  if (e < 1023 - 100 || e > 1023 + 100) return 1.0 / x;
  double y = (double)__frcp_rn((float)x);
  double r = fma(-x, y, 1.0);
  y = fma(y, r, y);
  r = fma(-x, y, 1.0);
  return fma(y, r, y);
}

__global__ void k_recip_probe(const double* x, double* y, int n) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) y[i] = recip_nr(x[i]);
}

void launch_recip_probe(const double* x, double* y, int n, cudaStream_t s) {
  k_recip_probe<<<(n + 255) / 256, 256, 0, s>>>(x, y, n);
}

namespace {

// read symmetric entry (r, c) of a lower-stored front (both < n or r >= n > c)
template <typename T>
__device__ __forceinline__ double sym_at(const T* L, int ld, int r, int c) {
  return (r >= c) ? (double)L[(int64_t)c * ld + r] : (double)L[(int64_t)r * ld + c];
}

// ------------------------------------------------------------------------
// Start of APP block step `step` for one front (one thread): fold the
// previous step's result (npass eliminated, the rest moved to the end of the
// candidate range) and take the next block of at most 32 candidates.  A
// front with fd.panel > 0 and more columns than that starts with the panel
// [0, panel): its candidate range ends there (see FrontState).
// ------------------------------------------------------------------------
template <typename T>
__device__ __forceinline__ void app_step_begin(const FrontDesc<T>& fd, FrontState* st, int step,
                                               int& p_out, int& bs_out) {
  int p, end;
  if (step == 0) {
    p = 0;
    end = (fd.panel > 0 && fd.n > fd.panel) ? fd.panel : fd.n;
    st->pstart = 0;
    st->qend = end;
    st->gend = fd.n;
    st->pk = 0;
  } else {
    p = st->p;
    end = st->end;
    if (st->bs > 0) {
      p += st->npass;
      end -= st->bs - st->npass;
    }
  }
  int bs = min(kBlk, end - p);
  if (bs < 0) bs = 0;
  st->p = p;
  st->end = end;
  st->bs = bs;
  st->npass_raw = bs;
  st->npass = bs;
  st->step = step;
  p_out = p;
  bs_out = bs;
}

// ------------------------------------------------------------------------
// k_app_diag: advance state, factor the diagonal block with complete pivoting.
// 1024 threads, thread (R, C) = (warp, lane) owns entry (R, C) of the block,
// which is stored full-symmetric and kept exactly symmetric: for R > C the
// thread computes the update of the pair once and writes both copies.
// Pivoting never moves data: a logical <-> physical index map is updated
// instead.  Each pivot: every thread keys its entry (64-bit: magnitude, then
// the reference's column-major scan order over the logical lower triangle),
// warps reduce, warp 0 reduces the 32 partial maxima and takes the 1x1 / 2x2
// decision, and every thread applies the rank-1/2 update to its entry.  The
// block and its updates are in the factor precision T; pivot values, D^{-1}
// and 2x2 inversions are FP64.  Semantics follow block_ldlt
// (src/ssids/cpu/kernels/block_ldlt.hxx:290-413): find_maxloc, the 2x2 test
// |det| >= |a21|/2 on the scaled determinant, otherwise the larger diagonal
// as a 1x1 pivot, zero pivots below `small`.
// ------------------------------------------------------------------------
template <typename T>
struct DiagKey;
template <>
struct DiagKey<double> {
  // magnitude with its low 10 mantissa bits replaced by the inverted
  // logical position: one unsigned max gives the largest entry and, among
  // entries equal to 2^-42 relative, the first in column-major order
  static __device__ __forceinline__ unsigned long long make(double v, int pos) {
    const unsigned long long mag =
        (unsigned long long)__double_as_longlong(v) & 0x7fffffffffffffffULL;
    return ((mag | 0x3ffULL) ^ 0x3ffULL) | (unsigned long long)(1023 - pos) | (1ULL << 63);
  }
  static __device__ __forceinline__ double mag(unsigned long long k) {
    return __longlong_as_double((long long)((k & 0x7fffffffffffffffULL) | 0x3ffULL));
  }
};
template <>
struct DiagKey<float> {
  // the exact FP32 magnitude above the 10-bit inverted position
  static __device__ __forceinline__ unsigned long long make(float v, int pos) {
    const unsigned long long mag = (unsigned long long)(__float_as_uint(v) & 0x7fffffffu);
    return (mag << 10) | (unsigned long long)(1023 - pos) | (1ULL << 63);
  }
  static __device__ __forceinline__ double mag(unsigned long long k) {
    return (double)__uint_as_float((unsigned int)((k >> 10) & 0x7fffffffULL));
  }
};

// unsigned 64-bit maximum over the warp as two 32-bit redux.sync: the high
// halves, then the low halves of the lanes holding the high maximum
__device__ __forceinline__ unsigned long long warp_max_u64(unsigned long long k) {
  const unsigned hi = (unsigned)(k >> 32), lo = (unsigned)k;
  const unsigned mh = __reduce_max_sync(0xffffffffu, hi);
  const unsigned ml = __reduce_max_sync(0xffffffffu, hi == mh ? lo : 0u);
  return ((unsigned long long)mh << 32) | ml;
}

// 17 warps: thread t < 528 owns the pair {R, C}, R >= C, t = R(R+1)/2 + C
constexpr int kDiagPairs = kBlk * (kBlk + 1) / 2;
constexpr int kDiagThreads = (kDiagPairs + 31) / 32 * 32;

// POSDEF: the Cholesky case (cpu/kernels/cholesky.cxx, LAPACK potrf): no
// pivoting, pivot q is the block's q-th diagonal, and a pivot that is not
// > 0 ends the factorisation with kDevNotPosdef.  The factors are kept as
// L D L^T (unit L, D > 0); L_chol = L D^(1/2).
template <typename T, bool POSDEF>
__global__ void __launch_bounds__(kDiagThreads) k_app_diag(FrontDesc<T>* fds, FrontState* sts,
                                                           const int* fronts, int step,
                                                           bool action, double small) {
  constexpr bool kF64 = sizeof(T) == 8;
  const int f = fronts[blockIdx.x];
  FrontState* st = &sts[f];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  // owned pair (physical R >= C)
  int R = (int)((sqrtf(8.0f * tid + 1.0f) - 1.0f) * 0.5f);
  while ((R + 1) * (R + 2) / 2 <= tid) ++R;
  while (R * (R + 1) / 2 > tid) --R;
  const int C = tid - R * (R + 1) / 2;
  const bool pair = tid < kDiagPairs;
  __shared__ T blk[kBlk][kBlk + 1];   // blk[c][r] = A(r, c), physical indices, symmetric
  __shared__ T outb[kBlk][kBlk + 1];  // outb[j][X] = L(inv[X], j): logical column, physical row
  __shared__ int map[kBlk], inv[kBlk];  // logical -> physical, physical -> logical
  __shared__ unsigned long long wkey[kBlk];
  __shared__ double rdiag[kBlk];
  __shared__ double dd[2 * kBlk + 2];
  __shared__ int s_dec[3];  // pivot size (0: zero pivot), physical pivot(s)
  __shared__ int s_state[2];
  __shared__ FrontDesc<T> fd;

  if (tid == 0) fd = fds[f];  // written by the host before the launch
  pdl_wait();
  pdl_trigger();
  if (tid == 0) {
    int p, bs;
    app_step_begin(fd, st, step, p, bs);
    s_state[0] = p;
    s_state[1] = bs;
  }
  __syncthreads();
  const int p = s_state[0], bs = s_state[1];
  if (bs == 0) return;
  const bool mine = pair && R < bs;  // (C <= R < bs)
  if (pair) {
    const T v = mine ? (T)fd.L[(int64_t)(p + C) * fd.ld + p + R] : T(0);
    blk[C][R] = v;
    blk[R][C] = v;
  }
  for (int e = tid; e < kBlk * (kBlk + 1); e += kDiagThreads) (&outb[0][0])[e] = T(0);
  if (tid < kBlk) { map[tid] = tid; inv[tid] = tid; }
  if (tid < 2 * kBlk + 2) dd[tid] = 0.0;
  if (tid < kBlk) wkey[tid] = 0;
  __syncthreads();

  bool singular = false, notpd = false;
  for (int q = 0; q < bs;) {
    // ---- candidates: the logical lower triangle of the trailing block
    if (POSDEF) {
      if (kF64 && R == q && C == q) rdiag[q] = recip_nr((double)blk[q][q]);
    } else {
      const int li = inv[R], lj = inv[C];
      const int hi = max(li, lj), lo = min(li, lj);
      unsigned long long key = 0;
      if (mine && lo >= q) key = DiagKey<T>::make(blk[C][R], lo * 32 + hi);
      key = warp_max_u64(key);
      if (lane == 0) wkey[warp] = key;
    }
    __syncthreads();
    // ---- decision and the pivot's L column(s) (warp 0; every lane takes the
    // same decision, lane X then forms row X of the new L column(s))
    if (warp == 0) {
      const unsigned long long gk = POSDEF ? 0ULL : warp_max_u64(wkey[lane]);
      const int pos = 1023 - (int)(gk & 0x3ffULL);
      const int bj = pos >> 5, bi = pos & 31;  // logical column, row of the maximum
      const double bv = DiagKey<T>::mag(gk);
      int pivsiz = 1, i1 = bi, i2 = -1;
      double e11 = 0.0, e21 = 0.0, e22 = 0.0;
      if (POSDEF) {
        i1 = q;  // no pivoting
        if (!((double)blk[q][q] > 0.0)) pivsiz = -1;
      } else if (bv < small) {
        pivsiz = 0;
      } else if (bi != bj) {
        const int mm = map[bj], tt = map[bi];
        const double a11 = (double)blk[mm][mm], a22 = (double)blk[tt][tt];
        const double a21 = (double)blk[mm][tt];
        const double detscale = recip_nr(fabs(a21));
        const double detpiv = (a11 * detscale) * a22 - fabs(a21);
        if (fabs(detpiv) >= fabs(a21) / 2) {
          pivsiz = 2; i1 = bj; i2 = bi;
          const double rdet = recip_nr(detpiv);
          e11 = (a22 * detscale) * rdet;
          e21 = (-a21 * detscale) * rdet;
          e22 = (a11 * detscale) * rdet;
        } else if (fabs(a11) > fabs(a22)) {
          i1 = bj;
        } else {
          i1 = bi;
        }
      }
      if (pivsiz > 0) {
        // logical swaps q <-> i1, then q+1 <-> i2 (i2 > i1 >= q) on the
        // updated map; P1, P2 are the physical pivots at q and q+1
        const int pa = map[q], pb = map[i1];
        const int cq1 = (pivsiz == 2) ? ((i1 == q + 1) ? pa : map[q + 1]) : -1;
        const int ci2 = (pivsiz == 2) ? map[i2] : -1;
        __syncwarp();
        if (lane == 0) {
          map[q] = pb; map[i1] = pa; inv[pb] = q; inv[pa] = i1;
          if (pivsiz == 2) { map[q + 1] = ci2; map[i2] = cq1; inv[ci2] = q + 1; inv[cq1] = i2; }
          s_dec[0] = pivsiz; s_dec[1] = pb; s_dec[2] = ci2;
        }
        __syncwarp();
        const int X = lane, lx = inv[X];
        if (pivsiz == 1) {
          const int P = pb;
          T dT;
          if (kF64) {
            // the chosen pivot's reciprocal only: FP64 instructions issue
            // slowly, so the other warps compute none
            const double d11 = POSDEF ? rdiag[P] : recip_nr((double)blk[P][P]);
            dT = (T)d11;
            if (lane == 0) { dd[2 * q] = d11; dd[2 * q + 1] = 0.0; }
          } else {
            // FP32 factors: the L column uses the FP32 reciprocal; D^{-1} is
            // formed in FP64 during the trailing update, off the critical path
            dT = T(1) / blk[P][P];
          }
          if (X < bs && lx > q) outb[q][X] = blk[P][X] * dT;  // L(lx, q) = A(X, P) / A(P, P)
        } else {
          if (lane == 0) {
            dd[2 * q] = e11; dd[2 * q + 1] = e21;
            dd[2 * q + 2] = dinf(); dd[2 * q + 3] = e22;
          }
          if (X < bs && lx > q + 1) {
            const T v1 = blk[pb][X], v2 = blk[ci2][X];
            outb[q][X] = (T)e11 * v1 + (T)e21 * v2;
            outb[q + 1][X] = (T)e21 * v1 + (T)e22 * v2;
          }
        }
      } else if (lane == 0) {
        s_dec[0] = pivsiz;  // 0: zero pivot, -1: not positive definite
      }
    }
    __syncthreads();
    const int pivsiz = s_dec[0];
    if (pivsiz < 0) { notpd = true; break; }
    if (pivsiz == 0) {
      if (!action) { singular = true; break; }
      // the remaining logical columns are zero pivots: their L columns stay zero
      if (tid >= q && tid < bs) { dd[2 * tid] = 0.0; dd[2 * tid + 1] = 0.0; }
      __syncthreads();
      break;
    }
    // ---- trailing update, one pair per thread, both copies written
    const int li = inv[R], lj = inv[C];
    if (pivsiz == 1) {
      const int P = s_dec[1];
      if (!kF64 && tid == kDiagThreads - 1) {  // an idle (non-pair) thread
        dd[2 * q] = recip_nr((double)blk[P][P]);
        dd[2 * q + 1] = 0.0;
      }
      if (mine && li > q && lj > q) {
        const T nv = blk[C][R] - blk[P][R] * outb[q][C];  // A(R,P) (A(C,P) / A(P,P))
        blk[C][R] = nv;
        blk[R][C] = nv;
      }
      __syncthreads();
      q += 1;
    } else {
      const int P1 = s_dec[1], P2 = s_dec[2];
      if (mine && li > q + 1 && lj > q + 1) {
        const T nv = blk[C][R] - (blk[P1][R] * outb[q][C] + blk[P2][R] * outb[q + 1][C]);
        blk[C][R] = nv;
        blk[R][C] = nv;
      }
      __syncthreads();
      q += 2;
    }
  }
  if (singular || notpd) {
    if (tid == 0) { st->status = notpd ? kDevNotPosdef : kDevSingular; st->bs = 0; }
    return;
  }
  // ---- write L11 (logical lower part, unit diagonal), D, step buffer, perm
  for (int e = tid; e < kBlk * kBlk; e += kDiagThreads) {
    const int j = e >> 5, X = e & 31;  // logical column, physical row
    if (j < bs && X < bs) {
      const int i = inv[X];
      if (i >= j) {
        const T v = (i == j) ? T(1) : outb[j][X];
        fd.L[(int64_t)(p + j) * fd.ld + p + i] = v;
        fd.step[j * kBlk + i] = (double)v;
      }
    }
  }
  if (tid < bs) {
    fd.D[2 * (p + tid)] = dd[2 * tid];
    fd.D[2 * (p + tid) + 1] = dd[2 * tid + 1];
    fd.step[kBlk * kBlk + 2 * tid] = dd[2 * tid];
    fd.step[kBlk * kBlk + 2 * tid + 1] = dd[2 * tid + 1];
    fd.lperm[tid] = map[tid];
  }
  int oldp = 0, oldo = 0;
  if (tid < bs) { oldp = fd.perm[p + map[tid]]; oldo = fd.opos[p + map[tid]]; }
  __syncthreads();
  if (tid < bs) { fd.perm[p + tid] = oldp; fd.opos[p + tid] = oldo; }
}

// ------------------------------------------------------------------------
// k_app_diag_f32<NW>: the indefinite diagonal block for FP32 factors with
// one barrier per pivot, NW warps.  Pair ownership, keys and pivot
// semantics as k_app_diag; thread t owns the pairs t, t + 32 NW, ... of the
// lower triangle (NW = 17: one pair each).  The pivot loop is restructured
// so that no warp waits on a serial decision phase:
//   * every warp reduces the NW warp maxima itself (two 32-bit redux.sync
//     per reduction) and takes the same pivot decision;
//   * the key of an entry also carries the physical row and column of its
//     logical column and row, so the decision reads the pivot entries
//     directly;
//   * each thread keeps the logical indices of its pairs in registers and
//     applies the pivot's swaps to them;
//   * the block, the logical -> physical map and the warp maxima are double
//     buffered: pivot q reads buffer q&1 and writes the other, and the key
//     of each updated entry is formed right after its update;
//   * the 2x2 test and the L columns are FP32; D^{-1} is formed in FP64
//     after the loop, for all pivots at once, from the recorded pivot
//     entries (the same formulas as k_app_diag).
// Every pair's update is the same arithmetic whatever NW, and the key
// maxima do not depend on the grouping, so all NW give the same bits.
// Fewer warps issue fewer redundant decisions per pivot but chain a
// thread's pair updates; on GB300 one pair per thread (17 warps) is the
// fastest.
// ------------------------------------------------------------------------
constexpr int kDiagWarps = kDiagThreads / 32;

// key of entry value v at logical (lo, hi), lo <= hi, physical (plo, phi):
// magnitude, then the inverted column-major position, then the physical
// indices (never decisive: positions are distinct)
__device__ __forceinline__ unsigned long long diag_key_f32(float v, int lo, int hi, int plo,
                                                            int phi) {
  const unsigned mag = __float_as_uint(v) & 0x7fffffffu;
  const unsigned low = ((unsigned)(1023 - (lo * 32 + hi)) << 10) | ((unsigned)plo << 5) |
                       (unsigned)phi;
  return (1ULL << 63) | ((unsigned long long)mag << 32) | low;
}

template <int NW>
__global__ void __launch_bounds__(NW * 32)
    k_app_diag_f32(FrontDesc<float>* fds, FrontState* sts, const int* fronts, int step,
                   bool action, double small) {
  constexpr int NT = NW * 32;
  constexpr int PP = (kDiagPairs + NT - 1) / NT;  // pairs per thread
  const int f = fronts[blockIdx.x];
  FrontState* st = &sts[f];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  int R[PP], C[PP];
  bool pair[PP];
#pragma unroll
  for (int k = 0; k < PP; ++k) {
    const int e = tid + k * NT;
    int r = (int)((sqrtf(8.0f * e + 1.0f) - 1.0f) * 0.5f);
    while ((r + 1) * (r + 2) / 2 <= e) ++r;
    while (r * (r + 1) / 2 > e) --r;
    pair[k] = e < kDiagPairs;
    R[k] = pair[k] ? r : 0;
    C[k] = pair[k] ? e - r * (r + 1) / 2 : 0;
  }
  __shared__ float blk[2][kBlk][kBlk + 1];   // blk[b][c][r] = A(r, c), physical, symmetric
  __shared__ float outb[kBlk][kBlk + 1];     // outb[j][X] = L(inv[X], j)
  __shared__ int map[2][kBlk];               // logical -> physical
  __shared__ int inv[kBlk];                  // physical -> logical (after the loop)
  __shared__ unsigned long long wkey[2][NW];
  __shared__ float pv[kBlk][3];              // pivot entries: a11 (1x1: d), a21, a22
  __shared__ int psz[kBlk];                  // 1: 1x1, 2: first of a 2x2, 3: second, 0: zero
  __shared__ double dd[2 * kBlk + 2];
  __shared__ int s_state[2];
  __shared__ FrontDesc<float> fd;

  if (tid == 0) fd = fds[f];  // written by the host before the launch
  pdl_wait();
  pdl_trigger();
  if (tid == 0) {
    int p, bs;
    app_step_begin(fd, st, step, p, bs);
    s_state[0] = p;
    s_state[1] = bs;
  }
  __syncthreads();
  const int p = s_state[0], bs = s_state[1];
  if (bs == 0) return;
  // FP32 threshold with (bv < fsmall) == ((double)bv < small) for every float bv
  float fsmall = (float)small;
  if ((double)fsmall < small) fsmall = nextafterf(fsmall, INFINITY);
  float a[PP];  // the owned entries
  bool mine[PP];
#pragma unroll
  for (int k = 0; k < PP; ++k) {
    mine[k] = pair[k] && R[k] < bs;  // (C <= R < bs)
    a[k] = mine[k] ? fd.L[(int64_t)(p + C[k]) * fd.ld + p + R[k]] : 0.f;
    if (pair[k]) {
      blk[0][C[k]][R[k]] = a[k];
      blk[0][R[k]][C[k]] = a[k];
    }
  }
  for (int e = tid; e < kBlk * (kBlk + 1); e += NT) (&outb[0][0])[e] = 0.f;
  if (tid < kBlk) {
    map[0][tid] = tid;
    psz[tid] = 0;
  }
  {
    unsigned long long k0 = 0ULL;
#pragma unroll
    for (int k = 0; k < PP; ++k)
      if (mine[k]) k0 = max(k0, diag_key_f32(a[k], C[k], R[k], C[k], R[k]));
    k0 = warp_max_u64(k0);
    if (lane == 0) wkey[0][warp] = k0;
  }
  int li[PP], lj[PP];  // logical indices of physical R and C
#pragma unroll
  for (int k = 0; k < PP; ++k) { li[k] = R[k]; lj[k] = C[k]; }
  int lx = lane;       // warp 0: logical index of physical row `lane`
  int cur = 0;
  bool singular = false;
  for (int q = 0; q < bs;) {
    __syncthreads();
    const int nxt = cur ^ 1;
    const unsigned long long gk = warp_max_u64(lane < NW ? wkey[cur][lane] : 0ULL);
    const unsigned lo32 = (unsigned)gk;
    const int pos = 1023 - (int)(lo32 >> 10);
    const int bj = pos >> 5, bi = pos & 31;                   // logical column, row
    const int pj = (int)((lo32 >> 5) & 31), pi = (int)(lo32 & 31);  // their physical
    const float bv = __uint_as_float((unsigned)(gk >> 32) & 0x7fffffffu);
    int pivsiz = 1, i1 = bi, i2 = -1;
    float e11 = 0.f, e21 = 0.f, e22 = 0.f, a11 = 0.f, a21 = 0.f, a22 = 0.f;
    if (bv < fsmall) {
      pivsiz = 0;
    } else if (bi != bj) {
      a11 = blk[cur][pj][pj];
      a22 = blk[cur][pi][pi];
      a21 = blk[cur][pj][pi];
      const float aa21 = fabsf(a21);
      const float detscale = __frcp_rn(aa21);
      const float detpiv = (a11 * detscale) * a22 - aa21;
      if (fabsf(detpiv) >= aa21 * 0.5f) {
        pivsiz = 2; i1 = bj; i2 = bi;
        const float rdet = __frcp_rn(detpiv);
        e11 = (a22 * detscale) * rdet;
        e21 = (-a21 * detscale) * rdet;
        e22 = (a11 * detscale) * rdet;
      } else if (fabsf(a11) > fabsf(a22)) {
        i1 = bj;
      } else {
        i1 = bi;
      }
    }
    if (pivsiz == 0) {
      // the remaining logical columns are zero pivots (psz 0): L columns and
      // D^{-1} stay zero
      if (!action) singular = true;
      break;
    }
    const int* mp = map[cur];
    const int pa = mp[q], pb = mp[i1];
    const int cq1 = (pivsiz == 2) ? ((i1 == q + 1) ? pa : mp[q + 1]) : -1;
    const int ci2 = (pivsiz == 2) ? mp[i2] : -1;
    // swaps q <-> i1, then q+1 <-> i2, applied to logical indices
    auto relabel = [&](int x) {
      x = (x == q) ? i1 : (x == i1) ? q : x;
      if (pivsiz == 2) x = (x == q + 1) ? i2 : (x == i2) ? q + 1 : x;
      return x;
    };
#pragma unroll
    for (int k = 0; k < PP; ++k) { li[k] = relabel(li[k]); lj[k] = relabel(lj[k]); }
    const int qn = q + pivsiz;
    if (pivsiz == 1) {
      const int P = pb;
      const float dT = __frcp_rn(blk[cur][P][P]);
#pragma unroll
      for (int k = 0; k < PP; ++k)
        if (mine[k] && min(li[k], lj[k]) >= qn)
          a[k] = a[k] - blk[cur][P][R[k]] * (blk[cur][P][C[k]] * dT);
      if (warp == 0) {
        lx = relabel(lx);
        if (lane < bs && lx > q) outb[q][lane] = blk[cur][P][lane] * dT;
      }
      if (tid == 0) {
        psz[q] = 1;
        pv[q][0] = blk[cur][P][P];
      }
    } else {
      const int P1 = pb, P2 = ci2;
#pragma unroll
      for (int k = 0; k < PP; ++k)
        if (mine[k] && min(li[k], lj[k]) >= qn) {
          const float v1 = blk[cur][P1][C[k]], v2 = blk[cur][P2][C[k]];
          a[k] = a[k] - (blk[cur][P1][R[k]] * (e11 * v1 + e21 * v2) +
                         blk[cur][P2][R[k]] * (e21 * v1 + e22 * v2));
        }
      if (warp == 0) {
        lx = relabel(lx);
        if (lane < bs && lx > q + 1) {
          const float v1 = blk[cur][P1][lane], v2 = blk[cur][P2][lane];
          outb[q][lane] = e11 * v1 + e21 * v2;
          outb[q + 1][lane] = e21 * v1 + e22 * v2;
        }
      }
      if (tid == 0) {
        psz[q] = 2;
        psz[q + 1] = 3;
        pv[q][0] = a11;
        pv[q][1] = a21;
        pv[q][2] = a22;
      }
    }
    unsigned long long key = 0ULL;
#pragma unroll
    for (int k = 0; k < PP; ++k) {
      if (pair[k]) {
        blk[nxt][C[k]][R[k]] = a[k];
        blk[nxt][R[k]][C[k]] = a[k];
      }
      const int lo = min(li[k], lj[k]), hi = max(li[k], lj[k]);
      if (mine[k] && lo >= qn)
        key = max(key, diag_key_f32(a[k], lo, hi, li[k] <= lj[k] ? R[k] : C[k],
                                    li[k] <= lj[k] ? C[k] : R[k]));
    }
    const unsigned long long wk = warp_max_u64(key);
    if (lane == 0) wkey[nxt][warp] = wk;
    if (warp == 0) {
      int v = mp[lane];
      if (lane == q) v = pb; else if (lane == i1) v = pa;
      if (pivsiz == 2) {
        if (lane == q + 1) v = ci2; else if (lane == i2) v = cq1;
      }
      map[nxt][lane] = v;
    }
    cur = nxt;
    q = qn;
  }
  if (warp == 0) inv[lane] = lx;
  __syncthreads();
  if (singular) {
    if (tid == 0) { st->status = kDevSingular; st->bs = 0; }
    return;
  }
  // D^{-1} in FP64 from the recorded pivots
  if (tid < bs) {
    const int ps = psz[tid];
    if (ps == 1) {
      dd[2 * tid] = recip_nr((double)pv[tid][0]);
      dd[2 * tid + 1] = 0.0;
    } else if (ps == 2) {
      const double d11 = pv[tid][0], d21 = pv[tid][1], d22 = pv[tid][2];
      const double detscale = recip_nr(fabs(d21));
      const double detpiv = (d11 * detscale) * d22 - fabs(d21);
      const double rdet = recip_nr(detpiv);
      dd[2 * tid] = (d22 * detscale) * rdet;
      dd[2 * tid + 1] = (-d21 * detscale) * rdet;
      dd[2 * tid + 2] = dinf();
      dd[2 * tid + 3] = (d11 * detscale) * rdet;
    } else if (ps == 0) {
      dd[2 * tid] = 0.0;
      dd[2 * tid + 1] = 0.0;
    }
  }
  __syncthreads();
  // ---- write L11 (logical lower part, unit diagonal), D, step buffer, perm
  const int* fmap = map[cur];
  for (int e = tid; e < kBlk * kBlk; e += NT) {
    const int j = e >> 5, X = e & 31;  // logical column, physical row
    if (j < bs && X < bs) {
      const int i = inv[X];
      if (i >= j) {
        const float v = (i == j) ? 1.f : outb[j][X];
        fd.L[(int64_t)(p + j) * fd.ld + p + i] = v;
        fd.step[j * kBlk + i] = (double)v;
      }
    }
  }
  if (tid < bs) {
    fd.D[2 * (p + tid)] = dd[2 * tid];
    fd.D[2 * (p + tid) + 1] = dd[2 * tid + 1];
    fd.step[kBlk * kBlk + 2 * tid] = dd[2 * tid];
    fd.step[kBlk * kBlk + 2 * tid + 1] = dd[2 * tid + 1];
    fd.lperm[tid] = fmap[tid];
  }
  int oldp = 0, oldo = 0;
  if (tid < bs) { oldp = fd.perm[p + fmap[tid]]; oldo = fd.opos[p + fmap[tid]]; }
  __syncthreads();
  if (tid < bs) { fd.perm[p + tid] = oldp; fd.opos[p + tid] = oldo; }
}

// columns of the eliminated part that one warp of k_app_apply's permutation
// CTAs moves per round
constexpr int kPermCols = 8;

// ------------------------------------------------------------------------
// k_app_apply: rows below the block; solve, scale, threshold test
// ------------------------------------------------------------------------
// threads per apply CTA and rows per tile: FP32, one row per thread (64);
// FP64, 32 rows shared by 4 warps (column blocks, see the solve below)
template <typename T>
__host__ __device__ constexpr int apply_threads() { return sizeof(T) == 8 ? 128 : kApplyRows; }
template <typename T>
__host__ __device__ constexpr int apply_rows() { return sizeof(T) == 8 ? 32 : kApplyRows; }

template <typename T>
__global__ void __launch_bounds__(apply_threads<T>()) k_app_apply(FrontDesc<T>* fds, FrontState* sts,
                                                          const int* fronts, double u,
                                                          double small, int napply) {
  const int f = fronts[blockIdx.y];
  FrontDesc<T> fd = fds[f];  // written by the host before the launch
  pdl_wait();
  pdl_trigger();
  FrontState* st = &sts[f];
  const int bs = st->bs;
  if (bs == 0) return;
  const int p = st->p;
  if ((int)blockIdx.x >= napply) {
    // block permutation of rows [p, p+bs) in the eliminated columns [0, p)
    if (p == 0) return;
    // a warp permutes kPermCols columns per round: all loads, then all stores
    constexpr int U = kPermCols;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const int src = (lane < bs) ? fd.lperm[lane] : lane;
    const int wstride = (gridDim.x - napply) * nw;
    for (int c0 = ((blockIdx.x - napply) * nw + warp) * U; c0 < p; c0 += wstride * U) {
      T v[U];
#pragma unroll
      for (int u = 0; u < U; ++u)
        v[u] = (lane < bs && c0 + u < p) ? fd.L[(int64_t)(c0 + u) * fd.ld + p + src] : T(0);
      __syncwarp();
#pragma unroll
      for (int u = 0; u < U; ++u)
        if (lane < bs && c0 + u < p) fd.L[(int64_t)(c0 + u) * fd.ld + p + lane] = v[u];
    }
    return;
  }
  const int r0 = p + bs;
  const int nrows = fd.m - r0;
  if (nrows <= 0) return;
  // X = A21 L11^{-T} in the factor precision T; D^{-1} application and the
  // a-posteriori test in FP64.  Few warps run this kernel on an SM, so its
  // code is kept short: L11 is staged transposed (l11t[k][j] = L(j, k),
  // rows 16-byte aligned) for vector loads in the unrolled solve, and the
  // per-column epilogue is a rolled loop over X staged in shared memory,
  // driven by the pivot kind of each column.
  constexpr int VW = 16 / sizeof(T);  // elements per 16-byte vector
  constexpr int LT = kBlk + VW;       // padded row of l11t
  constexpr int NT = apply_threads<T>(), RT = apply_rows<T>();
  __shared__ __align__(16) T l11t[kBlk][LT];
  __shared__ T xs[kBlk][RT];
  __shared__ double dd[2 * kBlk + 2];
  __shared__ float ddf[kBlk];  // FP32 copies of the 1x1 D^{-1} entries
  __shared__ int kind[kBlk];   // 0 1x1, 1 first of a 2x2, 2 second of a 2x2, 3 zero pivot
  __shared__ int lp[kBlk];
  {
    // all loads first (one latency), then the shared-memory stores
    constexpr int PER = kBlk * kBlk / NT;  // 16 (FP32) or 8 (FP64)
    double v[PER];
#pragma unroll
    for (int k = 0; k < PER; ++k) {
      const int i = threadIdx.x + k * NT;
      const int c = i / kBlk, r = i % kBlk;
      v[k] = (r > c && r < bs && c < bs) ? fd.step[c * kBlk + r] : 0.0;
    }
#pragma unroll
    for (int k = 0; k < PER; ++k) {
      const int i = threadIdx.x + k * NT;
      l11t[i / kBlk][i % kBlk] = (T)v[k];
    }
  }
  for (int i = threadIdx.x; i < 2 * kBlk + 2; i += blockDim.x)
    dd[i] = (i < 2 * bs) ? fd.step[kBlk * kBlk + i] : 0.0;
  __syncthreads();
  if (threadIdx.x < kBlk) {
    const int j = threadIdx.x;
    ddf[j] = (j < bs) ? (float)dd[2 * j] : 0.f;
    lp[j] = (j < bs) ? fd.lperm[j] : 0;
    int kd = 0;
    if (j < bs) {
      if (isinf(dd[2 * j])) kd = 2;
      else if (j + 1 < bs && isinf(dd[2 * j + 2])) kd = 1;
      else if (dd[2 * j] == 0.0) kd = 3;
    }
    kind[j] = kd;
  }
  __syncthreads();
  const double thresh = 1.0 / u;
  // FP32 guard band of the threshold test (FP32 factors)
  const float thr_lo = (float)(thresh * (1.0 - 1e-6)), thr_hi = (float)(thresh * (1.0 + 1e-6));
  // |l| > 1/u tested on bit patterns (non-negative doubles order as integers)
  const long long tkey = __double_as_longlong(thresh);
  auto over = [tkey](double l) {  // Inf fails the test, NaN does not (as fabs(l) > 1/u)
    const long long b = __double_as_longlong(l) & 0x7fffffffffffffffLL;
    return b > tkey && b <= 0x7ff0000000000000LL;
  };
  int myfail = bs;
  // row of the tile: FP32, thread t; FP64, lane t of each of the 4 warps,
  // warp w owning columns [8w, 8w+8)
  const int t = (sizeof(T) == 8) ? (threadIdx.x & 31) : threadIdx.x;
  for (int tile = blockIdx.x; tile * RT < nrows; tile += napply) {
    const int rr = tile * RT + t;
    const bool valid = rr < nrows;
    const int r = r0 + rr;
    if constexpr (sizeof(T) == 8) {
      // FP64: one warp's chain of 496 dependent FMAs per row tile waits on
      // the FP64 pipe of its SM sub-partition (~75 cycles a warp
      // instruction), so the columns are split over 4 warps in blocks of 8
      // and solved block by block: warp b solves its diagonal block, then
      // the warps right of it subtract block b.  Each x[j] still takes its
      // terms in the order k = 0, 1, ..., j-1 (the single-warp result, bit
      // for bit); the critical path is 4 x 28 + 3 x 64 FMAs.
      constexpr int CB = 8;
      const int w = threadIdx.x >> 5, c0 = CB * w;
      T x[CB];
#pragma unroll
      for (int i = 0; i < CB; ++i)
        x[i] = (valid && c0 + i < bs) ? fd.L[(int64_t)(p + lp[c0 + i]) * fd.ld + r] : T(0);
      for (int b = 0; b < kBlk / CB && CB * b < bs; ++b) {
        if (w == b) {
#pragma unroll
          for (int k = 0; k < CB - 1; ++k) {
            const T xk = x[k];
#pragma unroll
            for (int i = k + 1; i < CB; ++i) x[i] -= xk * l11t[c0 + k][c0 + i];
          }
#pragma unroll
          for (int i = 0; i < CB; ++i) xs[c0 + i][t] = x[i];
        }
        __syncthreads();
        if (w > b) {
#pragma unroll
          for (int k = 0; k < CB; ++k) {
            const T xk = xs[CB * b + k][t];
#pragma unroll
            for (int i = 0; i < CB; i += 2) {
              const double2 q = *reinterpret_cast<const double2*>(&l11t[CB * b + k][c0 + i]);
              x[i] -= xk * (T)q.x;
              x[i + 1] -= xk * (T)q.y;
            }
          }
        }
      }
      // blocks past bs were never solved: their columns are not used
    } else {
      T x[kBlk];
#pragma unroll
      for (int j = 0; j < kBlk; ++j)
        x[j] = (valid && j < bs) ? fd.L[(int64_t)(p + lp[j]) * fd.ld + r] : T(0);
      // right-looking: after x[k] is final, the updates of x[k+1..] are
      // independent FMAs; L(j, k) for j > k comes in 16-byte vectors (the
      // zero entries on and above the diagonal change nothing)
#pragma unroll
      for (int k = 0; k < kBlk - 1; ++k) {
        if (k + 1 < bs) {
          const T xk = x[k];
#pragma unroll
          for (int j0 = ((k + 1) / VW) * VW; j0 < kBlk; j0 += VW) {
            T lv[VW];
            const float4 q = *reinterpret_cast<const float4*>(&l11t[k][j0]);
            lv[0] = q.x; lv[1] = q.y; lv[2] = q.z; lv[3] = q.w;
#pragma unroll
            for (int v = 0; v < VW; ++v)
              if (j0 + v > k) x[j0 + v] -= xk * lv[v];
          }
        }
      }
#pragma unroll
      for (int j = 0; j < kBlk; ++j) xs[j][t] = x[j];  // column t is this thread's
    }
    if (valid) {
      T* W = fd.W + rr;
      // FP32: every column of the row; FP64: the warp's 8 columns
      const int jb = (sizeof(T) == 8) ? 8 * (threadIdx.x >> 5) : 0;
      const int je = (sizeof(T) == 8) ? min(jb + 8, bs) : bs;
#pragma unroll 1
      for (int j = jb; j < je; ++j) {
        const int kd = kind[j];
        if (kd == 2) continue;  // second half of a 2x2: handled with the first
        const T xj = xs[j][t];
        if (kd == 1) {
          const double dj = dd[2 * j], d21 = dd[2 * j + 1], d22 = dd[2 * j + 3];
          const double x1 = (double)xj, x2 = (double)xs[j + 1][t];
          const double l1 = dj * x1 + d21 * x2, l2 = d21 * x1 + d22 * x2;
          fd.L[(int64_t)(p + j) * fd.ld + r] = (T)l1;
          fd.L[(int64_t)(p + j + 1) * fd.ld + r] = (T)l2;
          W[(int64_t)j * fd.ld] = (T)x1;
          W[(int64_t)(j + 1) * fd.ld] = (T)x2;
          const int cand = over(l1) ? j : (over(l2) ? j + 1 : bs);
          myfail = min(myfail, cand);
        } else if (kd == 3) {
          const double v = (double)xj;
          const double l = (fabs(v) < small) ? 0.0 : dinf() * v;
          fd.L[(int64_t)(p + j) * fd.ld + r] = (T)l;
          W[(int64_t)j * fd.ld] = T(0);
          if (over(l)) myfail = min(myfail, j);
        } else if (sizeof(T) == 4) {
          // FP32 factors: L in FP32; the a-posteriori test |l| <= 1/u is
          // decided in FP32 outside a relative guard band of 1e-6 around
          // the threshold and in FP64 inside it, so every decision is the
          // FP64 one
          const float lf = (float)xj * ddf[j];
          fd.L[(int64_t)(p + j) * fd.ld + r] = (T)lf;
          W[(int64_t)j * fd.ld] = xj;
          const float al = fabsf(lf);
          if (!(al <= thr_lo)) {  // above the band, in it, or NaN
            if (al > thr_hi || over((double)xj * dd[2 * j])) myfail = min(myfail, j);
          }
        } else {
          const double l = (double)xj * dd[2 * j];
          fd.L[(int64_t)(p + j) * fd.ld + r] = (T)l;
          W[(int64_t)j * fd.ld] = xj;
          if (over(l)) myfail = min(myfail, j);
        }
      }
    }
    if constexpr (sizeof(T) == 8) __syncthreads();  // the next tile rewrites xs
  }
  // block min -> atomicMin
  for (int off = 16; off > 0; off >>= 1) myfail = min(myfail, __shfl_xor_sync(0xffffffffu, myfail, off));
  if ((threadIdx.x & 31) == 0 && myfail < bs) atomicMin(&st->npass_raw, myfail);
}

__device__ __forceinline__ int adjust_npass(int np, int bs, int p, const double* D) {
  if (np > 0 && np < bs) {
    double d11 = D[2 * (p + np - 1)], d21 = D[2 * (p + np - 1) + 1];
    if (isfinite(d11) && d21 != 0.0) np--;
  }
  return np;
}

// ------------------------------------------------------------------------
// Fixup of a block step (one of nfix CTAs, index fix): CTA 0 stores npass
// (Column::adjust, ldlt_app.cxx:112-130); for failed columns the
// restore-and-update of restore_if_required + update, computed as
// X_f L_ff^T (rows below, blockDim.x rows per tile) and L_ff D_f L_ff^T
// (diagonal block, CTA 0).  Failed columns are rare, so this path keeps few
// registers rather than being fast.
// ------------------------------------------------------------------------
template <typename T>
__device__ void app_fixup_cta(const FrontDesc<T>& fd, FrontState* st, int p, int bs, int np,
                              int fix, int nfix, double (*l11)[kBlk + 1],
                              double (*ldf)[kBlk + 1]) {
  if (fix == 0 && threadIdx.x == 0) st->npass = np;
  const int nf = bs - np;
  if (nf == 0) return;
  for (int i = threadIdx.x; i < kBlk * kBlk; i += blockDim.x) {
    int c = i / kBlk, r = i % kBlk;
    double v = (r < bs && c < bs) ? ((r == c) ? 1.0 : (r > c ? fd.step[c * kBlk + r] : 0.0)) : 0.0;
    l11[r][c] = v;
  }
  __syncthreads();
  const int r0 = p + bs, nrows = fd.m - r0;
  // rows below: A(r, p+np+i) = sum_{k<=i} X(r, np+k) * L(np+i, np+k)
  for (int tile = fix; tile * (int)blockDim.x < nrows; tile += nfix) {
    const int rr = tile * blockDim.x + threadIdx.x;
    if (rr < nrows) {
      const T* W = fd.W + rr;
      for (int i = 0; i < nf; ++i) {
        double s = 0.0;
        for (int k = 0; k <= i; ++k) s += (double)W[(int64_t)(np + k) * fd.ld] * l11[np + i][np + k];
        fd.L[(int64_t)(p + np + i) * fd.ld + r0 + rr] = (T)s;
      }
    }
  }
  if (fix == 0) {
    // diagonal failed block S = L_ff D_f L_ff^T
    const double* d = fd.step + kBlk * kBlk;
    // LD = L_ff * D_f  (D_f = inverse of stored inverse)
    for (int i = threadIdx.x; i < nf * nf; i += blockDim.x) {
      int r = i % nf, c = i / nf;
      ldf[r][c] = 0.0;
    }
    __syncthreads();
    if ((int)threadIdx.x < nf) {
      int r = threadIdx.x;
      for (int c = 0; c < nf;) {
        int cc = np + c;
        if (c + 1 == nf || isfinite(d[2 * (cc + 1)])) {
          double d11 = d[2 * cc];
          if (d11 != 0.0) d11 = 1.0 / d11;
          ldf[r][c] = d11 * l11[np + r][cc];
          c += 1;
        } else {
          double d11 = d[2 * cc], d21 = d[2 * cc + 1], d22 = d[2 * cc + 3];
          double det = d11 * d22 - d21 * d21;
          d11 /= det; d21 /= det; d22 /= det;
          double a1 = l11[np + r][cc], a2 = l11[np + r][cc + 1];
          ldf[r][c] = d22 * a1 - d21 * a2;
          ldf[r][c + 1] = -d21 * a1 + d11 * a2;
          c += 2;
        }
      }
    }
    __syncthreads();
    for (int i = threadIdx.x; i < nf * nf; i += blockDim.x) {
      int r = i % nf, c = i / nf;
      if (r < c) continue;
      double s = 0.0;
      for (int k = 0; k < nf; ++k) s += l11[np + r][np + k] * ldf[c][k];
      fd.L[(int64_t)(p + np + c) * fd.ld + p + np + r] = (T)s;
    }
  }
}

// ------------------------------------------------------------------------
// k_app_panel: the block step's trailing update of the candidate columns
// (ldlt_app.cxx:1082-1165 Block::update) in CTAs [0, ptiles) and its fixup
// in CTAs [ptiles, gridDim.x).  The two touch disjoint columns (the update
// reads the passed pivots' columns and writes the columns after the block;
// the fixup rewrites the failed columns of the block), so one launch serves
// both.  Every CTA derives npass from the apply's result itself.
//
// Update C -= A B^T (lower part) with K = npass <= kBlk: a TP x TP tile per
// CTA round, thread (tx, ty) = (tid % 16, tid / 16) computing (TP/16)^2
// entries; a tile stages all of its A and B columns and reads its C entries
// in one batch of loads (one memory round trip per tile).  FP32 uses 64 x 64
// tiles (latency bound); FP64 32 x 32 tiles: a 64 x 64 tile is about 37 us
// of work for one SM's FP64 pipe, and finer tiles balance the last wave.
// ------------------------------------------------------------------------
template <typename T>
constexpr int panel_tile() { return sizeof(T) == 8 ? 32 : 64; }

template <typename T, int TP>
__global__ void __launch_bounds__(256) k_app_panel(FrontDesc<T>* fds, FrontState* sts,
                                                   const int* fronts, int ptiles) {
  constexpr int RT = TP / 16;            // entries per thread and direction
  constexpr int PER = TP * kBlk / 256;   // A (and B) loads per thread
  // update CTAs use Ap/Bp, fixup CTAs l11/ldf: one buffer serves both
  constexpr size_t kUpd = 2 * sizeof(T) * kBlk * (TP + 4);
  constexpr size_t kFix = 2 * sizeof(double) * kBlk * (kBlk + 1);
  __shared__ __align__(16) unsigned char sbuf[kUpd > kFix ? kUpd : kFix];
  T (*Ap)[TP + 4] = reinterpret_cast<T (*)[TP + 4]>(sbuf);
  T (*Bp)[TP + 4] = Ap + kBlk;
  double (*l11)[kBlk + 1] = reinterpret_cast<double (*)[kBlk + 1]>(sbuf);
  double (*ldf)[kBlk + 1] = l11 + kBlk;
  const int f = fronts[blockIdx.y];
  const FrontDesc<T> fd = fds[f];  // written by the host before the launch
  pdl_wait();
  pdl_trigger();
  FrontState* stp = &sts[f];
  const int bs = stp->bs;
  if (bs == 0) return;
  const int p = stp->p;
  const int np = adjust_npass(stp->npass_raw, bs, p, fd.D);
  if ((int)blockIdx.x >= ptiles) {
    app_fixup_cta<T>(fd, stp, p, bs, np, blockIdx.x - ptiles, gridDim.x - ptiles, l11, ldf);
    return;
  }
  // the candidate columns of the current panel (all of them for a front
  // without panels), including failed columns moved behind its candidates
  const int M = fd.m - (p + bs), N = stp->qend - (p + bs), K = np;
  if (K <= 0 || M <= 0 || N <= 0) return;
  T* C = fd.L + (int64_t)(p + bs) * fd.ld + (p + bs);
  const T* A = fd.L + (int64_t)p * fd.ld + (p + bs);
  const T* B = fd.W;
  const int ld = fd.ld;
  const int tid = threadIdx.x;
  const int tx = tid & 15, ty = tid >> 4;
  const int tc = (N + TP - 1) / TP, tr = (M + TP - 1) / TP;
  const int total = tc * tr - tc * (tc - 1) / 2;
  for (int t = blockIdx.x; t < total; t += ptiles) {
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
        cv[x][y] = (r < M && c < N && r >= c) ? C[(int64_t)c * ld + r] : T(0);
      }
    }
    T av[PER], bv[PER];
#pragma unroll
    for (int q = 0; q < PER; ++q) {
      const int idx = tid + 256 * q;
      const int rr = idx % TP, kk = idx / TP;
      const int r = row0 + rr, c = col0 + rr;
      av[q] = (r < M && kk < K) ? A[(int64_t)kk * ld + r] : T(0);
      bv[q] = (c < N && kk < K) ? B[(int64_t)kk * ld + c] : T(0);
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
        if (r < M && c < N && r >= c) C[(int64_t)c * ld + r] = cv[x][y] - acc[x][y];
      }
    }
    __syncthreads();  // Ap/Bp are rewritten by the next tile
  }
}

// ------------------------------------------------------------------------
// moving failed columns [p+np, p+bs) to the end of the range [.., end)
// ------------------------------------------------------------------------
struct SwapRanges {
  int a0, b0, npairs;  // pairs (a0+k, b0+k)
};
__device__ __forceinline__ SwapRanges swap_ranges(const FrontState& st) {
  SwapRanges s;
  const int nf = st.bs - st.npass;
  const int fs = st.p + st.npass, fe = st.p + st.bs;
  const int ts = st.end - nf, te = st.end;
  s.a0 = fs;
  s.b0 = max(ts, fe);
  int aend = min(fe, ts);
  s.npairs = max(0, aend - fs);
  (void)te;
  return s;
}
__device__ __forceinline__ int swap_partner(const SwapRanges& s, int x) {
  if (x >= s.a0 && x < s.a0 + s.npairs) return s.b0 + (x - s.a0);
  if (x >= s.b0 && x < s.b0 + s.npairs) return s.a0 + (x - s.b0);
  return x;
}

// columns per CTA of the L D kernels (k_panel_ld, k_calc_ld)
constexpr int kLdCols = 16;

// Symmetric swap of the position pairs (a0 + k, b0 + k), k < npairs, over
// the whole front (every line: eliminated L rows, columns, diagonal; perm
// and opos), by one CTA, 32 pairs at a time: gather the affected lines into
// the front's swap buffer (64 lines), barrier, scatter them permuted.
template <typename T>
__device__ void swap_lines(const FrontDesc<T>& fd, int a0, int b0, int npairs) {
  for (int base = 0; base < npairs; base += 32) {
    SwapRanges sr;
    sr.a0 = a0 + base;
    sr.b0 = b0 + base;
    sr.npairs = min(32, npairs - base);
    const int nl = 2 * sr.npairs;
    int* ib = reinterpret_cast<int*>(fd.swapbuf + (int64_t)nl * fd.ld);
    for (int li = 0; li < nl; ++li) {
      const int s = (li < sr.npairs) ? sr.a0 + li : sr.b0 + (li - sr.npairs);
      T* line = fd.swapbuf + (int64_t)li * fd.ld;
      for (int x = threadIdx.x; x < fd.m; x += blockDim.x) line[x] = (T)sym_at(fd.L, fd.ld, x, s);
      if (threadIdx.x == 0) { ib[2 * li] = fd.perm[s]; ib[2 * li + 1] = fd.opos[s]; }
    }
    __syncthreads();
    for (int li = 0; li < nl; ++li) {
      const int s = (li < sr.npairs) ? sr.a0 + li : sr.b0 + (li - sr.npairs);
      const int ps = swap_partner(sr, s);
      const int pli =
          (ps >= sr.a0 && ps < sr.a0 + sr.npairs) ? ps - sr.a0 : sr.npairs + (ps - sr.b0);
      const T* line = fd.swapbuf + (int64_t)pli * fd.ld;
      for (int x = threadIdx.x; x < fd.m; x += blockDim.x) {
        const T v = line[swap_partner(sr, x)];
        if (x <= s) fd.L[(int64_t)x * fd.ld + s] = v;
        else fd.L[(int64_t)s * fd.ld + x] = v;
      }
      if (threadIdx.x == 0) { fd.perm[s] = ib[2 * pli]; fd.opos[s] = ib[2 * pli + 1]; }
    }
    __syncthreads();  // the buffer is refilled by the next 32 pairs
  }
}

// The block step's failed columns trade places with the last candidates
// (at most 32 disjoint transpositions (a0 + i, b0 + i)).  For a line x
// outside the swapped set, the transposition only exchanges the entries
// (x, a0 + i) and (x, b0 + i): CTAs 1.. take the lines x, one thread per
// line, which touch disjoint entries (a row of contiguous entries when x
// lies left of the set, coalesced columns when it lies right of it).  CTA 0
// permutes the block of entries between the swapped lines themselves, and
// perm and opos, through shared memory.  No barrier across CTAs is needed.
template <typename T>
__device__ __forceinline__ T* sym_ptr(T* L, int ld, int r, int c) {
  return r >= c ? L + (int64_t)c * ld + r : L + (int64_t)r * ld + c;
}
template <typename T>
__global__ void __launch_bounds__(256) k_app_swap(FrontDesc<T>* fds, const FrontState* sts,
                                                  const int* fronts) {
  const int f = fronts[blockIdx.y];
  FrontDesc<T> fd = fds[f];  // written by the host before the launch
  pdl_wait();
  pdl_trigger();
  const FrontState st = sts[f];
  if (st.bs == 0 || st.bs == st.npass) return;
  const SwapRanges sr = swap_ranges(st);
  const int np = sr.npairs;
  if (np <= 0) return;
  const int nl = 2 * np;
  auto line = [&](int i) { return i < np ? sr.a0 + i : sr.b0 + (i - np); };
  if (blockIdx.x == 0) {
    __shared__ T blk[2 * kBlk][2 * kBlk + 1];
    __shared__ int pp[2 * kBlk], oo[2 * kBlk];
    for (int e = threadIdx.x; e < nl * nl; e += blockDim.x) {
      const int i = e / nl, j = e % nl;
      blk[i][j] = *sym_ptr(fd.L, fd.ld, line(i), line(j));
    }
    for (int i = threadIdx.x; i < nl; i += blockDim.x) { pp[i] = fd.perm[line(i)]; oo[i] = fd.opos[line(i)]; }
    __syncthreads();
    // new(s_i, s_j) = old(partner(s_i), partner(s_j)); partner swaps halves
    for (int e = threadIdx.x; e < nl * nl; e += blockDim.x) {
      const int i = e / nl, j = e % nl;
      if (line(i) < line(j)) continue;  // each stored entry once
      const int pi = i < np ? i + np : i - np, pj = j < np ? j + np : j - np;
      *sym_ptr(fd.L, fd.ld, line(i), line(j)) = blk[pi][pj];
    }
    for (int i = threadIdx.x; i < nl; i += blockDim.x) {
      const int pi = i < np ? i + np : i - np;
      fd.perm[line(i)] = pp[pi];
      fd.opos[line(i)] = oo[pi];
    }
    return;
  }
  for (int x = (blockIdx.x - 1) * blockDim.x + threadIdx.x; x < fd.m;
       x += (gridDim.x - 1) * blockDim.x) {
    if ((x >= sr.a0 && x < sr.a0 + np) || (x >= sr.b0 && x < sr.b0 + np)) continue;
    for (int i = 0; i < np; ++i) {
      T* pa = sym_ptr(fd.L, fd.ld, x, sr.a0 + i);
      T* pb = sym_ptr(fd.L, fd.ld, x, sr.b0 + i);
      const T va = *pa, vb = *pb;
      *pa = vb;
      *pb = va;
    }
  }
}

// ------------------------------------------------------------------------
// Panel end (fronts with panels): fold the panel's last block step, record
// pk = p - pstart, and form LD = L D of the trailing rows [qend, n) for the
// panel's pivots [pstart, p), column k at fd.LD + k * n (2x2 pivots never
// straddle a panel: Column::adjust keeps them whole).  The tensor-core
// update C[qend:m, qend:n] -= L[qend:m, pstart:p] LD^T follows.
// ------------------------------------------------------------------------
__global__ void k_panel_fold(FrontState* sts, const int* fronts, int nf) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nf) return;
  FrontState* st = &sts[fronts[i]];
  if (st->bs > 0) {
    st->p += st->npass;
    st->end -= st->bs - st->npass;
    st->bs = 0;
  }
  st->pk = st->p - st->pstart;
}

template <typename T>
__global__ void __launch_bounds__(128) k_panel_ld(FrontDesc<T>* fds, const FrontState* sts,
                                                  const int* fronts) {
  const int f = fronts[blockIdx.z];
  const FrontDesc<T> fd = fds[f];
  const FrontState st = sts[f];
  const int K = st.pk, c0 = blockIdx.y * kLdCols;
  const int q = st.qend, rows = fd.n - q;
  if (c0 >= K || rows <= 0 || st.status != kDevOk) return;
  const int nc = min(kLdCols, K - c0);
  const int pe = st.pstart + K;  // end of the panel's pivots
  __shared__ double alpha[kLdCols], beta[kLdCols];
  __shared__ int partner[kLdCols];
  if ((int)threadIdx.x < nc) {
    const int c = st.pstart + c0 + threadIdx.x;
    const double d11 = fd.D[2 * c];
    if (isinf(d11)) {  // second column of a 2x2
      const double a = fd.D[2 * (c - 1)], b = fd.D[2 * (c - 1) + 1], d = fd.D[2 * c + 1];
      const double det = a * d - b * b;
      alpha[threadIdx.x] = a / det; beta[threadIdx.x] = -b / det; partner[threadIdx.x] = c - 1;
    } else if (c + 1 < pe && isinf(fd.D[2 * c + 2])) {  // first column of a 2x2
      const double b = fd.D[2 * c + 1], d = fd.D[2 * c + 3];
      const double det = d11 * d - b * b;
      alpha[threadIdx.x] = d / det; beta[threadIdx.x] = -b / det; partner[threadIdx.x] = c + 1;
    } else {
      alpha[threadIdx.x] = (d11 != 0.0) ? 1.0 / d11 : 0.0; beta[threadIdx.x] = 0.0;
      partner[threadIdx.x] = c;
    }
  }
  __syncthreads();
  for (int rr = blockIdx.x * blockDim.x + threadIdx.x; rr < rows; rr += gridDim.x * blockDim.x) {
    const T* Lr = fd.L + q + rr;
    T lv[kLdCols], lp[kLdCols];
#pragma unroll
    for (int k = 0; k < kLdCols; ++k) {
      lv[k] = (k < nc) ? Lr[(int64_t)(st.pstart + c0 + k) * fd.ld] : T(0);
      lp[k] = (k < nc && beta[k] != 0.0) ? Lr[(int64_t)partner[k] * fd.ld] : T(0);
    }
#pragma unroll
    for (int k = 0; k < kLdCols; ++k)
      if (k < nc)
        fd.LD[(int64_t)(c0 + k) * fd.n + rr] = (T)(alpha[k] * (double)lv[k] + beta[k] * (double)lp[k]);
  }
}

// Panel close (one CTA per front): the panel's failed columns [end, qend)
// (kept up to date by every pivot of the panel, and now also complete with
// respect to the trailing update) trade places with the last candidates of
// the front [gend - nf, gend), which have all of the panel's updates too;
// the candidate range shrinks by nf and the next panel [p, min(p + panel,
// gend)) opens.
template <typename T>
__global__ void __launch_bounds__(1024) k_panel_close(FrontDesc<T>* fds, FrontState* sts,
                                                      const int* fronts) {
  const int f = fronts[blockIdx.x];
  const FrontDesc<T> fd = fds[f];
  FrontState* st = &sts[f];
  const int p = st->p, end = st->end, qend = st->qend, gend = st->gend;
  if (st->status != kDevOk) return;
  const int nf = qend - end;
  if (nf > 0) {
    const int fs = end, fe = qend, ts = gend - nf;
    const int b0 = max(ts, fe);
    const int npairs = max(0, min(fe, ts) - fs);
    swap_lines(fd, fs, b0, npairs);
  }
  if (threadIdx.x == 0) {
    const int g = gend - max(nf, 0);
    st->gend = g;
    st->pstart = p;
    st->qend = min(p + fd.panel, g);
    st->end = st->qend;
    st->bs = 0;
  }
}

template <typename T>
__global__ void k_app_finish(FrontDesc<T>* fds, FrontState* sts, const int* fronts, int nf) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nf) return;
  FrontState* st = &sts[fronts[i]];
  int p = st->p, end = st->end;
  if (st->bs > 0) { p += st->npass; end -= st->bs - st->npass; }
  st->p = p;
  st->end = end;
  st->bs = 0;
  st->nelim = p;
  st->step = p;  // number eliminated by the APP pass (before TPP)
}

// ------------------------------------------------------------------------
// k_tpp: threshold partial pivoting on the failed columns [nelim, n)
// (ldlt_tpp.cxx:166-270).  One CTA per front; FP64 arithmetic.
// ------------------------------------------------------------------------
constexpr int kTppThreads = 256;


// ------------------------------------------------------------------------
// k_tpp_small: the fronts of small leaf subtrees, factored with TPP from
// their first column as the reference's CPU path does for every node of a
// subtree below small_subtree_threshold flops (SymbolicSubtree.hxx:56-82;
// SmallLeafNumericSubtree.hxx:345-375 calls ldlt_tpp_factor on the whole
// front).  One CTA per front, the front (m x n), two workspace columns and
// its perm/opos held in shared memory.  The TPP itself (tpp_fast, which
// k_tpp also runs on the failed columns of APP fronts): each pivot, warp 0
// alone runs the pivot search of ldlt_tpp_factor (ldlt_tpp.cxx:166-270;
// every reduction a warp shuffle), performs the symmetric swaps, writes
// D^{-1} and keeps unscaled copies of the pivot column(s); after one barrier
// every warp scales the pivot column(s) and updates the trailing
// fully-summed columns (rows of the front's contribution part included);
// one more barrier ends the pivot.  A front too large for the launch's
// shared memory (delays can grow one) is factored the same way in global
// memory.  step = 0 records that no APP pass ran.
// ------------------------------------------------------------------------
namespace tpps {
enum Kind : int { kStop = 0, kZeroNel, kZeroSwap, kTwo, kOne, kSingular };
struct Decision {
  int kind, t, p;
  double d0, d1, d3;  // FP64 factors: D^{-1} of the pivot
  float f0, f1, f3;   // FP32 factors: the L columns' multipliers
};

__device__ __forceinline__ bool wall(bool b) { return __all_sync(0xffffffffu, b); }

// Magnitude keys: |v|'s bits as an unsigned integer order non-negative
// floating-point values (no NaN) as their values do, so the pivot search
// compares and reduces entries with integer instructions (on GB300 every
// FP64 instruction, conversions and maxima included, issues slowly) and
// takes exactly the decisions of the FP64 comparisons it replaces.
__device__ __forceinline__ unsigned long long mag_key(float v) {
  return __float_as_uint(v) & 0x7fffffffu;
}
__device__ __forceinline__ unsigned long long mag_key(double v) {
  return (unsigned long long)__double_as_longlong(v) & 0x7fffffffffffffffULL;
}
// the value of a key, in the factor precision (FP32 factors: no conversion
// to FP64, whose instructions issue slowly)
template <typename T>
__device__ __forceinline__ T key_value(unsigned long long k) {
  if constexpr (sizeof(T) == 4) return __uint_as_float((unsigned)k);
  else return __longlong_as_double((long long)k);
}
// the key below which an entry's magnitude is < s (s >= 0): the key of the
// smallest T not below s
template <typename T>
__device__ __forceinline__ unsigned long long below_key(double s) {
  if constexpr (sizeof(T) == 4) {
    float f = (float)s;
    if ((double)f < s) f = nextafterf(f, INFINITY);
    return mag_key(f);
  } else {
    return mag_key(s);
  }
}
// warp-wide maximum of a key
template <typename T>
__device__ __forceinline__ unsigned long long warp_key_max(unsigned long long k) {
  if constexpr (sizeof(T) == 4) return __reduce_max_sync(0xffffffffu, (unsigned)k);
  else return warp_max_u64(k);
}

// The thresholds of a TPP search, formed once per front: the key below
// which an entry counts as zero, and small and u in the factor precision
// (FP32: small rounded up, so that (v < small_t) == ((double)v < small) for
// every FP32 v; the conversions are FP64 instructions, kept off the
// per-pivot path)
template <typename T>
struct Thr {
  unsigned long long sk;
  T small, u;
};
template <typename T>
__device__ __forceinline__ Thr<T> make_thr(double u, double small) {
  Thr<T> t;
  t.sk = below_key<T>(small);
  if constexpr (sizeof(T) == 4) {
    float f = (float)small;
    if ((double)f < small) f = nextafterf(f, INFINITY);
    t.small = f;
    t.u = (float)u;
  } else {
    t.small = small;
    t.u = u;
  }
  return t;
}

// all |entries| of row/column idx (row part from `from`) below small
// (check_col_small, ldlt_tpp.cxx:21-28); sk = the threshold's key
template <typename T>
__device__ bool col_small(const T* S, int ld, int idx, int from, int m, unsigned long long sk) {
  const int lane = threadIdx.x & 31;
  bool ok = true;
  for (int c = from + lane; c < idx; c += 32) ok = ok && (mag_key(S[(size_t)c * ld + idx]) < sk);
  for (int r = idx + lane; r < m; r += 32) ok = ok && (mag_key(S[(size_t)idx * ld + r]) < sk);
  return wall(ok);
}
// largest |entry| of row/column col excluding position excl and the
// diagonal (find_rc_abs_max_exclude, ldlt_tpp.cxx:80-92)
template <typename T>
__device__ T rc_max(const T* S, int ld, int col, int nel, int m, int excl) {
  const int lane = threadIdx.x & 31;
  unsigned long long k = 0;
  for (int c = nel + lane; c < col; c += 32)
    if (c != excl) k = max(k, mag_key(S[(size_t)c * ld + col]));
  for (int r = col + 1 + lane; r < m; r += 32)
    if (r != excl) k = max(k, mag_key(S[(size_t)col * ld + r]));
  return key_value<T>(warp_key_max<T>(k));
}
// first column of the largest |a(p, c)|, c in [from, p) (find_row_abs_max)
template <typename T>
__device__ int row_argmax(const T* S, int ld, int p, int from) {
  const int lane = threadIdx.x & 31;
  unsigned long long bk = 0;
  int bi = 0x7fffffff;
  for (int c = from + lane; c < p; c += 32) {
    const unsigned long long k = mag_key(S[(size_t)c * ld + p]);
    if (k > bk || bi == 0x7fffffff) { bk = k; bi = c; }
  }
  const unsigned long long mx = warp_key_max<T>(bi == 0x7fffffff ? 0ULL : bk);
  const unsigned cand = (bi != 0x7fffffff && bk == mx) ? (unsigned)bi : 0x7fffffffu;
  return (int)__reduce_min_sync(0xffffffffu, cand);
}
// symmetric swap of positions i < j over the whole front (swap_cols,
// ldlt_tpp.cxx:44-72), perm and opos included; warp-wide
template <typename T>
__device__ void sym_swap(T* S, int ld, int m, int i, int j, int* perm, int* opos) {
  if (i == j) return;
  if (j < i) { const int t = i; i = j; j = t; }
  const int lane = threadIdx.x & 31;
  for (int c = lane; c < i; c += 32) {
    const T t = S[(size_t)c * ld + i]; S[(size_t)c * ld + i] = S[(size_t)c * ld + j]; S[(size_t)c * ld + j] = t;
  }
  for (int r = i + 1 + lane; r < j; r += 32) {
    const T t = S[(size_t)i * ld + r]; S[(size_t)i * ld + r] = S[(size_t)r * ld + j]; S[(size_t)r * ld + j] = t;
  }
  for (int r = j + 1 + lane; r < m; r += 32) {
    const T t = S[(size_t)i * ld + r]; S[(size_t)i * ld + r] = S[(size_t)j * ld + r]; S[(size_t)j * ld + r] = t;
  }
  if (lane == 0) {
    const T t = S[(size_t)i * ld + i]; S[(size_t)i * ld + i] = S[(size_t)j * ld + j]; S[(size_t)j * ld + j] = t;
    const int pt = perm[i]; perm[i] = perm[j]; perm[j] = pt;
    const int ot = opos[i]; opos[i] = opos[j]; opos[j] = ot;
  }
  __syncwarp();
}
// The 2x2 test of (t, p) (test_2x2, ldlt_tpp.cxx:95-126), then the 1x1
// test of p (ldlt_tpp.cxx:216-236): true with d set when p is taken.  FP64
// factors: FP64 arithmetic as the reference.  FP32 factors: FP32 arithmetic
// on the FP32 entries and maxima, as the FP32 APP block takes its 2x2 test,
// so the serial search issues no FP64 instruction, conversions included (on
// GB300 a division alone is a long chain of slow FP64 instructions); D^{-1}
// of the chosen pivots is formed in FP64 afterwards (tpp_finish_d), and
// f0..f3 here only scale the L columns.
template <typename T>
__device__ __forceinline__ bool test_pivots(T a11, T a21, T a22, T maxt, T maxp,
                                            const Thr<T> th, int t, int p, Decision& d) {
  if constexpr (sizeof(T) == 8) {
    const double u = th.u, small = th.small;
    const double maxpiv = fmax(fabs(a11), fmax(fabs(a21), fabs(a22)));
    if (!(maxpiv < small)) {
      const double detscale = 1 / maxpiv;
      const double det0 = (a11 * detscale) * a22, det1 = (a21 * detscale) * a21;
      const double detpiv = det0 - det1;
      if (!(fabs(detpiv) < fmax(small, fmax(fabs(det0 / 2), fabs(det1 / 2))))) {
        // the three divisions side by side in lanes 0, 1, 2 (the same
        // operations, so the same bits, in one division's latency)
        const int lane = threadIdx.x & 31;
        const double num = lane == 0 ? a22 * detscale : lane == 1 ? -a21 * detscale : a11 * detscale;
        const double q = num / detpiv;
        const double d0 = __shfl_sync(0xffffffffu, q, 0), d1 = __shfl_sync(0xffffffffu, q, 1);
        const double d3 = __shfl_sync(0xffffffffu, q, 2);
        bool ok;
        if (fmax(maxp, maxt) < small) ok = true;
        else {
          const double x1 = fabs(d0) * maxt + fabs(d1) * maxp;
          const double x2 = fabs(d1) * maxt + fabs(d3) * maxp;
          ok = (u * fmax(x1, x2) < 1.0);
        }
        if (ok) { d.kind = kTwo; d.t = t; d.p = p; d.d0 = d0; d.d1 = d1; d.d3 = d3; return true; }
      }
    }
    maxp = fmax(maxp, fabs(a21));
    if (fabs(a22) >= u * maxp) { d.kind = kOne; d.p = p; return true; }
    return false;
  } else {
    // the entries and maxima are FP32 values; thresholds in FP32
    const float fsmall = th.small, fu = th.u;
    const float b11 = a11, b21 = a21, b22 = a22;
    const float mt = maxt;
    float mp = maxp;
    const float maxpiv = fmaxf(fabsf(b11), fmaxf(fabsf(b21), fabsf(b22)));
    if (!(maxpiv < fsmall)) {
      const float detscale = 1.0f / maxpiv;
      const float det0 = (b11 * detscale) * b22, det1 = (b21 * detscale) * b21;
      const float detpiv = det0 - det1;
      if (!(fabsf(detpiv) < fmaxf(fsmall, fmaxf(fabsf(det0 * 0.5f), fabsf(det1 * 0.5f))))) {
        const float d0 = (b22 * detscale) / detpiv, d1 = (-b21 * detscale) / detpiv;
        const float d3 = (b11 * detscale) / detpiv;
        bool ok;
        if (fmaxf(mp, mt) < fsmall) ok = true;
        else {
          const float x1 = fabsf(d0) * mt + fabsf(d1) * mp;
          const float x2 = fabsf(d1) * mt + fabsf(d3) * mp;
          ok = (fu * fmaxf(x1, x2) < 1.0f);
        }
        if (ok) { d.kind = kTwo; d.t = t; d.p = p; d.f0 = d0; d.f1 = d1; d.f3 = d3; return true; }
      }
    }
    mp = fmaxf(mp, fabsf(b21));
    if (fabsf(b22) >= fu * mp) { d.kind = kOne; d.p = p; return true; }
    return false;
  }
}
// the pivot search of one step of ldlt_tpp_factor, in warp 0
template <typename T>
__device__ Decision decide(const T* S, int ld, int nel, int m, int n, bool action,
                           const Thr<T> th) {
  Decision d{kStop, 0, 0, 0.0, 0.0, 0.0};
  if (col_small(S, ld, nel, nel, m, th.sk)) { d.kind = action ? kZeroNel : kSingular; return d; }
  for (int p = nel + 1; p < n; ++p) {
    if (col_small(S, ld, p, nel, m, th.sk)) { d.kind = action ? kZeroSwap : kSingular; d.p = p; return d; }
    const int t = row_argmax(S, ld, p, nel);
    const T maxt = rc_max(S, ld, t, nel, m, p);
    const T maxp = rc_max(S, ld, p, nel, m, t);
    const T a11 = S[(size_t)t * ld + t], a21 = S[(size_t)t * ld + p];
    const T a22 = S[(size_t)p * ld + p];
    if (test_pivots<T>(a11, a21, a22, maxt, maxp, th, t, p, d)) return d;
  }
  // last resort: nel itself as a 1x1 pivot
  const T maxp = rc_max(S, ld, nel, nel, m, -1);
  if (sizeof(T) == 8 ? fabs((double)S[(size_t)nel * ld + nel]) >= (double)th.u * (double)maxp
                     : fabsf((float)S[(size_t)nel * ld + nel]) >= (float)th.u * (float)maxp) {
    d.kind = kOne;
    d.p = nel;
  }
  return d;
}
// ---- the same pivot search with every warp of the CTA (tall fronts) ----
// Per line (row part [nel, idx) then column part [idx, m) of line idx):
// all |v| < small, the first largest |v| of the row part, and the two
// largest |v| off the diagonal with their positions; reduced over the CTA
// in warp order (shuffles, then shared memory), so the result is the same
// for every thread and every launch shape.
// Magnitudes are kept as keys (mag_key); an empty record holds key 0 at
// position 0x7fffffff, which any entry beats.
struct LineInfo {
  int all_small;
  unsigned long long rv; int ri;  // row part: first maximum
  unsigned long long v1; int i1;  // off-diagonal: largest ...
  unsigned long long v2; int i2;  // ... and second largest (positions differ)
};
__device__ __forceinline__ bool better(unsigned long long va, int ia, unsigned long long vb,
                                       int ib) {
  return va > vb || (va == vb && ia < ib);
}
__device__ __forceinline__ void top2_add(LineInfo& a, unsigned long long v, int i) {
  if (better(v, i, a.v1, a.i1)) { a.v2 = a.v1; a.i2 = a.i1; a.v1 = v; a.i1 = i; }
  else if (better(v, i, a.v2, a.i2)) { a.v2 = v; a.i2 = i; }
}
__device__ __forceinline__ void line_merge(LineInfo& a, const LineInfo& b) {
  a.all_small = a.all_small && b.all_small;
  if (better(b.rv, b.ri, a.rv, a.ri)) { a.rv = b.rv; a.ri = b.ri; }
  top2_add(a, b.v1, b.i1);
  top2_add(a, b.v2, b.i2);
}
__device__ __forceinline__ LineInfo line_shfl(const LineInfo& a, int o) {
  LineInfo b;
  b.all_small = __shfl_xor_sync(0xffffffffu, a.all_small, o);
  b.rv = __shfl_xor_sync(0xffffffffu, a.rv, o); b.ri = __shfl_xor_sync(0xffffffffu, a.ri, o);
  b.v1 = __shfl_xor_sync(0xffffffffu, a.v1, o); b.i1 = __shfl_xor_sync(0xffffffffu, a.i1, o);
  b.v2 = __shfl_xor_sync(0xffffffffu, a.v2, o); b.i2 = __shfl_xor_sync(0xffffffffu, a.i2, o);
  return b;
}
template <typename T>
__device__ LineInfo line_info(const T* S, int ld, int idx, int nel, int m,
                              unsigned long long sk, LineInfo* sh) {
  LineInfo a{1, 0, 0x7fffffff, 0, 0x7fffffff, 0, 0x7fffffff};
  for (int c = nel + (int)threadIdx.x; c < idx; c += blockDim.x) {
    const unsigned long long v = mag_key(S[(size_t)c * ld + idx]);
    a.all_small = a.all_small && (v < sk);
    if (better(v, c, a.rv, a.ri)) { a.rv = v; a.ri = c; }
    top2_add(a, v, c);
  }
  for (int r = idx + (int)threadIdx.x; r < m; r += blockDim.x) {
    const unsigned long long v = mag_key(S[(size_t)idx * ld + r]);
    a.all_small = a.all_small && (v < sk);
    if (r != idx) top2_add(a, v, r);
  }
  for (int o = 1; o < 32; o <<= 1) {
    const LineInfo b = line_shfl(a, o);
    line_merge(a, b);
  }
  const int warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  __syncthreads();  // sh may still be read from the previous reduction
  if ((threadIdx.x & 31) == 0) sh[warp] = a;
  __syncthreads();
  LineInfo r = sh[0];
  for (int w = 1; w < nw; ++w) line_merge(r, sh[w]);
  return r;
}
// the line information of lines [l0, l1) (one warp per line) into
// out[idx - nel], then a barrier
template <typename T>
__device__ void line_info_batch(const T* S, int ld, int l0, int l1, int nel, int m,
                                unsigned long long sk, LineInfo* out) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  for (int idx = l0 + warp; idx < l1; idx += nw) {
    LineInfo a{1, 0, 0x7fffffff, 0, 0x7fffffff, 0, 0x7fffffff};
    for (int c = nel + lane; c < idx; c += 32) {
      const unsigned long long v = mag_key(S[(size_t)c * ld + idx]);
      a.all_small = a.all_small && (v < sk);
      if (better(v, c, a.rv, a.ri)) { a.rv = v; a.ri = c; }
      top2_add(a, v, c);
    }
    for (int r = idx + lane; r < m; r += 32) {
      const unsigned long long v = mag_key(S[(size_t)idx * ld + r]);
      a.all_small = a.all_small && (v < sk);
      if (r != idx) top2_add(a, v, r);
    }
    for (int o = 1; o < 32; o <<= 1) {
      const LineInfo b = line_shfl(a, o);
      line_merge(a, b);
    }
    if (lane == 0) out[idx - nel] = a;
  }
  __syncthreads();
}

// One candidate p of ldlt_tpp_factor's search (ldlt_tpp.cxx:196-236), from
// the line information of p and of t = the first largest entry of row p:
// returns true with d set when p is taken (as a zero column, a 2x2 pivot
// (t, p) or a 1x1 pivot).
template <typename T>
__device__ bool try_candidate(const T* S, int ld, int p, const LineInfo& lp, const LineInfo& lt,
                              bool action, const Thr<T> th, Decision& d) {
  if (lp.all_small) { d.kind = action ? kZeroSwap : kSingular; d.p = p; return true; }
  const int t = lp.ri;
  const T maxp = key_value<T>((lp.i1 == t) ? lp.v2 : lp.v1);
  // largest |entry| of line t off its diagonal, excluding position p
  const T maxt = key_value<T>((lt.i1 == p) ? lt.v2 : lt.v1);
  const T a11 = S[(size_t)t * ld + t], a21 = S[(size_t)t * ld + p];
  const T a22 = S[(size_t)p * ld + p];
  return test_pivots<T>(a11, a21, a22, maxt, maxp, th, t, p, d);
}

// the pivot search of one step of ldlt_tpp_factor with all threads (each
// gets the same Decision).  The first candidate is tested from two line
// scans; when it fails and `batch` (>= n - nel line records of global
// scratch) is given, the information of every remaining line is gathered
// in one pass, one warp per line, and the other candidates are tested from
// it: a search that runs through many candidates (failed columns, as in KKT
// systems) reads each line once instead of twice per candidate.  The
// records equal line_info's, so the decision is the same either way.
template <typename T>
__device__ Decision decide_cta(const T* S, int ld, int nel, int m, int n, bool action,
                               const Thr<T> th, LineInfo* sh, LineInfo* batch) {
  Decision d{kStop, 0, 0, 0.0, 0.0, 0.0};
  if (line_info(S, ld, nel, nel, m, th.sk, sh).all_small) {
    d.kind = action ? kZeroNel : kSingular;
    return d;
  }
  int p = nel + 1;
  if (p < n) {
    const LineInfo lp = line_info(S, ld, p, nel, m, th.sk, sh);
    const LineInfo lt = line_info(S, ld, lp.ri, nel, m, th.sk, sh);
    if (try_candidate(S, ld, p, lp, lt, action, th, d)) return d;
    ++p;
  }
  if (batch != nullptr && p < n) {
    line_info_batch(S, ld, nel, n, nel, m, th.sk, batch);
    for (; p < n; ++p) {
      const LineInfo lp = batch[p - nel];
      if (try_candidate(S, ld, p, lp, batch[(lp.all_small ? p : lp.ri) - nel], action, th, d))
        return d;
    }
    const LineInfo ln = batch[0];
    const T maxp = key_value<T>(ln.v1);
    if (sizeof(T) == 8 ? fabs((double)S[(size_t)nel * ld + nel]) >= (double)th.u * (double)maxp
                       : fabsf((float)S[(size_t)nel * ld + nel]) >= (float)th.u * (float)maxp) {
      d.kind = kOne;
      d.p = nel;
    }
    return d;
  }
  for (; p < n; ++p) {
    const LineInfo lp = line_info(S, ld, p, nel, m, th.sk, sh);
    if (lp.all_small) { d.kind = action ? kZeroSwap : kSingular; d.p = p; return d; }
    const LineInfo lt = line_info(S, ld, lp.ri, nel, m, th.sk, sh);
    if (try_candidate(S, ld, p, lp, lt, action, th, d)) return d;
  }
  const LineInfo ln = line_info(S, ld, nel, nel, m, th.sk, sh);
  const T maxp = key_value<T>(ln.v1);
  if (sizeof(T) == 8 ? fabs((double)S[(size_t)nel * ld + nel]) >= (double)th.u * (double)maxp
                     : fabsf((float)S[(size_t)nel * ld + nel]) >= (float)th.u * (float)maxp) {
    d.kind = kOne;
    d.p = nel;
  }
  return d;
}
}  // namespace tpps

// rows of a front above which the TPP pivot search uses every warp
constexpr int kTppWideRows = 1024;

// line records of the batched pivot search: the front's workspace W (ld x 32
// entries; the first two columns hold the pivot copies), 56 n <= 30 ld
// sizeof(T) bytes
template <typename T>
__device__ __forceinline__ tpps::LineInfo* tpp_batch(const FrontDesc<T>& fd) {
  return reinterpret_cast<tpps::LineInfo*>(fd.W + 2 * (size_t)fd.ld);
}

// a b + c d in FP32 with the rounding error of c d kept (an error-free
// product by FMA, then one fused add and one add): close to the sum formed
// exactly and rounded once, also where the two products cancel
__device__ __forceinline__ float dot2_f32(float a, float b, float c, float d) {
  const float p = __fmul_rn(c, d);
  const float e = __fmaf_rn(c, d, -p);
  return __fadd_rn(__fmaf_rn(a, b, p), e);
}

// FP32 factors: D^{-1} of the pivots [nel0, nel1) in FP64 from the pivot
// entries the TPP loop recorded in D (1x1: the pivot; 2x2: a11, a21, the
// second-half marker, a22), with the formulas of test_2x2 and the 1x1
// reciprocal, one pivot per thread; ends with a barrier.  FP64 factors
// already hold D^{-1}.
template <typename T>
__device__ void tpp_finish_d(double* D, int nel0, int nel1) {
  if constexpr (sizeof(T) == 4) {
    __syncthreads();
    for (int i = nel0 + (int)threadIdx.x; i < nel1; i += blockDim.x) {
      if (isinf(D[2 * i])) continue;  // second half of a 2x2: its first half converts both
      if (i + 1 < nel1 && isinf(D[2 * i + 2])) {
        const double a11 = D[2 * i], a21 = D[2 * i + 1], a22 = D[2 * i + 3];
        const double maxpiv = fmax(fabs(a11), fmax(fabs(a21), fabs(a22)));
        const double detscale = 1 / maxpiv;
        const double det0 = (a11 * detscale) * a22, det1 = (a21 * detscale) * a21;
        const double detpiv = det0 - det1;
        D[2 * i] = (a22 * detscale) / detpiv;
        D[2 * i + 1] = (-a21 * detscale) / detpiv;
        D[2 * i + 3] = (a11 * detscale) / detpiv;
      } else {
        const double a = D[2 * i];
        D[2 * i] = (a != 0.0) ? 1.0 / a : 0.0;
        D[2 * i + 1] = 0.0;
      }
    }
  }
  __syncthreads();
}

// The TPP loop of ldlt_tpp_factor on columns [nel, n), rows [nel, m), of
// the front held at S (leading dimension ld; shared or global memory), with
// two workspace columns W0, W1 (>= m entries) and the front's perm, opos
// and D^{-1}.  Swaps cover whole lines (the rows of the eliminated columns
// to the left included, as swap_cols with aleft, ldlt_tpp.cxx:44-72).
// Returns the number of columns eliminated in total, or -1 for a singular
// front with action == false.  Called by all threads of the CTA.  With
// finish == false, FP32 factors leave the recorded pivot entries (the D
// blocks themselves) in D for the caller, which forms D^{-1} with
// tpp_finish_d afterwards.
template <typename T>
__device__ int tpp_fast(T* S, int ld, int m, int n, int nel, T* W0, T* W1, int* perm, int* opos,
                        double* D, bool action, double u, double small, tpps::LineInfo* batch,
                        bool finish = true) {
  using namespace tpps;
  __shared__ Decision s_dec;
  __shared__ LineInfo s_line[kTppThreads / 32];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
  const int nel0 = nel;
  const Thr<T> th = make_thr<T>(u, small);
  while (nel < n) {
    Decision dw;
    const bool wide = m - nel > kTppWideRows;
    if (wide) dw = decide_cta(S, ld, nel, m, n, action, th, s_line, batch);
    if (warp == 0) {
      Decision d = wide ? dw : decide(S, ld, nel, m, n, action, th);
      if (d.kind == kZeroSwap) sym_swap(S, ld, m, d.p, nel, perm, opos);
      if (d.kind == kZeroNel || d.kind == kZeroSwap) {
        for (int r = nel + lane; r < m; r += 32) S[(size_t)nel * ld + r] = T(0);
        if (lane == 0) { D[2 * nel] = 0.0; D[2 * nel + 1] = 0.0; }
      } else if (d.kind == kTwo) {
        sym_swap(S, ld, m, d.t, nel, perm, opos);
        sym_swap(S, ld, m, d.p, nel + 1, perm, opos);
        for (int r = nel + 2 + lane; r < m; r += 32) {
          W0[r] = S[(size_t)nel * ld + r];
          W1[r] = S[(size_t)(nel + 1) * ld + r];
        }
        if (lane == 0) {
          if constexpr (sizeof(T) == 4) {
            // the pivot entries; D^{-1} in FP64 by tpp_finish_d
            D[2 * nel] = (double)S[(size_t)nel * ld + nel];
            D[2 * nel + 1] = (double)S[(size_t)nel * ld + nel + 1];
            D[2 * nel + 3] = (double)S[(size_t)(nel + 1) * ld + nel + 1];
          } else {
            D[2 * nel] = d.d0; D[2 * nel + 1] = d.d1; D[2 * nel + 3] = d.d3;
          }
          D[2 * nel + 2] = dinf();
          S[(size_t)nel * ld + nel] = T(1);
          S[(size_t)nel * ld + nel + 1] = T(0);
          S[(size_t)(nel + 1) * ld + nel + 1] = T(1);
        }
      } else if (d.kind == kOne) {
        sym_swap(S, ld, m, d.p, nel, perm, opos);
        const T app = S[(size_t)nel * ld + nel];
        if constexpr (sizeof(T) == 4) d.f0 = 1.0f / app;  // the L column's multiplier
        else d.d0 = 1.0 / app;
        for (int r = nel + 1 + lane; r < m; r += 32) W0[r] = S[(size_t)nel * ld + r];
        if (lane == 0) {
          S[(size_t)nel * ld + nel] = T(1);
          D[2 * nel] = sizeof(T) == 4 ? (double)app : d.d0;  // FP32: the pivot, see tpp_finish_d
          D[2 * nel + 1] = 0.0;
        }
      }
      __syncwarp();
      if (lane == 0) s_dec = d;
    }
    __syncthreads();
    const Decision d = s_dec;
    if (d.kind == kStop) break;
    if (d.kind == kSingular) {
      tpp_finish_d<T>(D, nel0, nel);
      return -1;
    }
    if (d.kind == kZeroNel || d.kind == kZeroSwap) {
      nel += 1;
      __syncthreads();  // every warp has read s_dec before warp 0 rewrites it
      continue;
    }
    const int ps = (d.kind == kTwo) ? 2 : 1;
    // scale the pivot column(s) (apply_1x1 / apply_2x2) and update the
    // trailing fully-summed columns, rows [c, m), with the unscaled copies.
    // The multipliers are taken in the factor precision (FP32 factors: the
    // FP32 D^{-1} entries, as the APP path's L columns; D^{-1} itself stays
    // FP64), so the update issues no FP64 instruction for FP32 factors.
    const int c0 = nel + ps;
    T e0, e1, e3;
    if constexpr (sizeof(T) == 4) { e0 = d.f0; e1 = d.f1; e3 = d.f3; }
    else { e0 = d.d0; e1 = d.d1; e3 = d.d3; }
    if (ps == 1) {
      for (int r = c0 + threadIdx.x; r < m; r += blockDim.x) S[(size_t)nel * ld + r] = W0[r] * e0;
    } else {
      // FP32 factors: each L entry of a 2x2 pivot is a sum of two products
      // that can cancel, formed with the second product's rounding error
      // kept (dot2_f32); FP64 factors as written
      for (int r = c0 + threadIdx.x; r < m; r += blockDim.x) {
        const T a1 = W0[r], a2 = W1[r];
        if constexpr (sizeof(T) == 4) {
          S[(size_t)nel * ld + r] = dot2_f32(e0, a1, e1, a2);
          S[(size_t)(nel + 1) * ld + r] = dot2_f32(e1, a1, e3, a2);
        } else {
          S[(size_t)nel * ld + r] = e0 * a1 + e1 * a2;
          S[(size_t)(nel + 1) * ld + r] = e1 * a1 + e3 * a2;
        }
      }
    }
    // the trailing update reads the scaled columns back (other threads wrote
    // them): one FMA per entry and pivot column instead of forming the
    // multipliers again for every column
    __syncthreads();
    if (ps == 1) {
      const T* l = S + (size_t)nel * ld;
      for (int c = c0 + warp; c < n; c += nw) {
        const T wc = W0[c];
        T* col = S + (size_t)c * ld;
        for (int r = c + lane; r < m; r += 32) col[r] -= l[r] * wc;
      }
    } else {
      const T* l1 = S + (size_t)nel * ld;
      const T* l2 = S + (size_t)(nel + 1) * ld;
      for (int c = c0 + warp; c < n; c += nw) {
        const T w0 = W0[c], w1 = W1[c];
        T* col = S + (size_t)c * ld;
        for (int r = c + lane; r < m; r += 32) col[r] -= l1[r] * w0 + l2[r] * w1;
      }
    }
    __syncthreads();
    nel += ps;
  }
  if (finish) tpp_finish_d<T>(D, nel0, nel);
  return nel;
}

template <typename T>
__global__ void __launch_bounds__(kTppThreads) k_tpp(FrontDesc<T>* fds, FrontState* sts,
                                                     const int* fronts, bool action, double u,
                                                     double small, bool all_fronts) {
  const int f = fronts[blockIdx.x];
  FrontState* st = &sts[f];
  FrontDesc<T> fd = fds[f];
  if (st->status != kDevOk) return;
  if (st->nelim >= fd.n) return;
  if (!(all_fronts || fd.m == fd.n)) return;
  const int nel = tpp_fast(fd.L, fd.ld, fd.m, fd.n, st->nelim, fd.W, fd.W + fd.ld, fd.perm,
                           fd.opos, fd.D, action, u, small, tpp_batch(fd));
  if (threadIdx.x == 0) {
    if (nel < 0) st->status = kDevSingular;
    else { st->nelim = nel; st->p = nel; }
  }
}

// ------------------------------------------------------------------------
// k_tpp_level: the fronts of the small leaf subtrees in one level set, one
// persistent launch per size class (the multinode_ldlt role of the
// reference's GPU path, src/ssids/gpu/kernels/dense_factor.cu, with the CPU
// path's pivoting for these fronts, ldlt_tpp_factor).  CTAs take fronts
// i = blockIdx.x, blockIdx.x + gridDim.x, ... of the class's list (largest
// first); per front: the TPP factorisation (in shared memory when the front
// fits the launch's dynamic shared memory, else in place in global memory),
// then, fused, the front's contribution: LD = L21 D (the front's LD
// workspace) and C -= L21 LD^T on the lower triangle of its contribution
// block, warp per column of C and lane per row, k in increasing order.  So
// a level set of small fronts takes one or two launches instead of a TPP
// launch, an LD launch and a contribution launch, and small fronts run many
// CTAs per SM (the tiny class launches one warp per CTA).
// ------------------------------------------------------------------------
// (alpha, beta, partner) of eliminated column c: column c of D = (D^{-1})^{-1}
// is alpha e_c + beta e_partner (1x1: partner = c, beta = 0)
__device__ __forceinline__ void d_column(const double* D, int c, int nel, double& alpha,
                                         double& beta, int& partner) {
  const double d11 = D[2 * c];
  if (isinf(d11)) {  // second column of a 2x2
    const double a = D[2 * (c - 1)], b = D[2 * (c - 1) + 1], d = D[2 * c + 1];
    const double det = a * d - b * b;
    alpha = a / det; beta = -b / det; partner = c - 1;
  } else if (c + 1 < nel && isinf(D[2 * c + 2])) {  // first column of a 2x2
    const double b = D[2 * c + 1], d = D[2 * c + 3];
    const double det = d11 * d - b * b;
    alpha = d / det; beta = -b / det; partner = c + 1;
  } else {
    alpha = (d11 != 0.0) ? 1.0 / d11 : 0.0; beta = 0.0; partner = c;
  }
}

// FP32 factors before tpp_finish_d: D holds the pivot blocks themselves
// (1x1: d; 2x2: a11, a21, the second-half marker, a22), exact FP32 values,
// so column c of D is read off directly, without an FP64 division
__device__ __forceinline__ void d_column_raw(const double* D, int c, int nel, float& alpha,
                                             float& beta, int& partner) {
  const double d11 = D[2 * c];
  if (isinf(d11)) {  // second column of a 2x2: (a21, a22)
    alpha = (float)D[2 * c + 1]; beta = (float)D[2 * (c - 1) + 1]; partner = c - 1;
  } else if (c + 1 < nel && isinf(D[2 * c + 2])) {  // first column of a 2x2: (a11, a21)
    alpha = (float)d11; beta = (float)D[2 * c + 1]; partner = c + 1;
  } else {
    alpha = (float)d11; beta = 0.f; partner = c;
  }
}

// the fused contribution of one front whose factor is at S (leading
// dimension ldS); all threads of the CTA.  Column c of D, (alpha, beta,
// partner), is formed once per column into shared memory: FP64 factors
// from D^{-1} (d_column, FP64 divisions), FP32 factors from the recorded
// pivot blocks (d_column_raw, before tpp_finish_d) with LD in FP32
// arithmetic (compensated for 2x2 columns), so the FP32 contribution issues
// no FP64 instruction per entry.  LD goes to ldsm (shared memory, cm x nel)
// when given, else to the front's LD workspace.  C -= L21 LD^T on the lower
// triangle: FP32 factors in 32 x 16 tiles, one per warp at a time, lane
// (lr, lc) = (lane % 8, lane / 8) holding rows lr + 8i and columns lc + 4j,
// i, j < 4, so each k takes 8 loads for 16 FMAs; FP64 factors a warp per
// column and a lane per row (their FMAs, not the loads, bound it, and the
// tile's registers would cost a CTA per SM).  Either way every entry sums
// its products in increasing k, one FMA each.
template <typename T>
__device__ void tpp_front_contrib(const FrontDesc<T>& fd, const T* S, int ldS, int nel, T* ldsm) {
  const int n = fd.n, cm = fd.m - fd.n;
  if (cm <= 0 || nel <= 0) return;
  T* LD = ldsm ? ldsm : fd.LD;  // LD(r, c) at LD[c * cm + r]
  __shared__ T s_alpha[kTppThreads], s_beta[kTppThreads];
  __shared__ int s_partner[kTppThreads];
  for (int cb = 0; cb < nel; cb += blockDim.x) {
    const int nc = min((int)blockDim.x, nel - cb);
    if ((int)threadIdx.x < nc) {
      const int c = cb + threadIdx.x;
      int partner;
      if constexpr (sizeof(T) == 4) {
        float alpha, beta;
        d_column_raw(fd.D, c, nel, alpha, beta, partner);
        s_alpha[threadIdx.x] = alpha; s_beta[threadIdx.x] = beta;
      } else {
        double alpha, beta;
        d_column(fd.D, c, nel, alpha, beta, partner);
        s_alpha[threadIdx.x] = alpha; s_beta[threadIdx.x] = beta;
      }
      s_partner[threadIdx.x] = partner;
    }
    __syncthreads();
    for (int e = threadIdx.x; e < cm * nc; e += blockDim.x) {
      const int rr = e % cm, cc = e / cm, c = cb + cc;
      const T alpha = s_alpha[cc], beta = s_beta[cc];
      const T lv = S[(size_t)c * ldS + n + rr];
      const T lp = (beta != T(0)) ? S[(size_t)s_partner[cc] * ldS + n + rr] : T(0);
      if constexpr (sizeof(T) == 4) {
        // a 2x2 column's two products can cancel (dot2_f32)
        LD[(int64_t)c * cm + rr] = dot2_f32(alpha, lv, beta, lp);
      } else {
        LD[(int64_t)c * cm + rr] = alpha * lv + beta * lp;
      }
    }
    __syncthreads();  // the coefficients are rewritten by the next chunk
  }
  __syncthreads();  // LD is read back by other threads of this CTA
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
  if constexpr (sizeof(T) == 8) {
    for (int c = warp; c < cm; c += nw) {
      const T* ldc = LD + c;
      for (int r = c + lane; r < cm; r += 32) {
        const T* lrow = S + n + r;
        T acc = T(0);
        for (int k = 0; k < nel; ++k) acc += lrow[(size_t)k * ldS] * ldc[(int64_t)k * cm];
        fd.C[(int64_t)c * fd.ldc + r] -= acc;
      }
    }
    return;
  }
  const int lr = lane & 7, lc = lane >> 3;
  const int nrt = (cm + 31) / 32, nct = (cm + 15) / 16;
  for (int t = warp; t < nrt * nct; t += nw) {
    const int rt = t % nrt, ct = t / nrt;
    const int r0 = 32 * rt + lr, c0 = 16 * ct + lc;
    if (32 * rt + 31 < 16 * ct) continue;  // wholly above the diagonal
    T acc[4][4];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
      for (int j = 0; j < 4; ++j) acc[i][j] = T(0);
    const T* Ap = S + n + r0;
    const T* Bp = LD + c0;
    for (int k = 0; k < nel; ++k) {
      T a[4], b[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) a[i] = (r0 + 8 * i < cm) ? Ap[(size_t)k * ldS + 8 * i] : T(0);
#pragma unroll
      for (int j = 0; j < 4; ++j) b[j] = (c0 + 4 * j < cm) ? Bp[(int64_t)k * cm + 4 * j] : T(0);
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] += a[i] * b[j];
    }
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const int r = r0 + 8 * i, c = c0 + 4 * j;
        if (r < cm && c <= r) fd.C[(int64_t)c * fd.ldc + r] -= acc[i][j];
      }
  }
}

template <typename T>
__global__ void __launch_bounds__(kTppThreads) k_tpp_level(FrontDesc<T>* fds, FrontState* sts,
                                                           const int* fronts, int nf,
                                                           bool action, double u, double small,
                                                           int smem_bytes) {
  extern __shared__ __align__(16) unsigned char tpp_smem[];
  // FP32 factors: the contribution reads the pivot blocks recorded in D,
  // which become D^{-1} after it
  constexpr bool raw_d = sizeof(T) == 4;
  for (int i = blockIdx.x; i < nf; i += gridDim.x) {
    const int f = fronts[i];
    FrontState* st = &sts[f];
    const FrontDesc<T> fd = fds[f];
    __syncthreads();  // the previous front is done with shared memory and st
    if (st->status != kDevOk) continue;
    const int m = fd.m, n = fd.n;
    const int ldS = (m + 1) & ~1;
    const size_t need = (size_t)ldS * (n + 2) * sizeof(T) + 2 * (size_t)n * sizeof(int);
    int nel;
    const T* F = fd.L;  // where the factor is when the contribution is formed
    int ldF = fd.ld;
    T* ldsm = nullptr;  // LD in shared memory, or the front's workspace
    if (n == 0) {
      nel = 0;
    } else if (need > (size_t)smem_bytes) {
      nel = tpp_fast(fd.L, fd.ld, m, n, 0, fd.W, fd.W + fd.ld, fd.perm, fd.opos, fd.D, action, u,
                     small, tpp_batch(fd), !raw_d);
    } else {
      // FP32 factors: LD in the shared memory after the front when it fits
      const size_t ld_off = (need + 15) & ~(size_t)15;
      if (sizeof(T) == 4 && ld_off + (size_t)(m - n) * n * sizeof(T) <= (size_t)smem_bytes)
        ldsm = reinterpret_cast<T*>(tpp_smem + ld_off);
      T* S = reinterpret_cast<T*>(tpp_smem);
      T* W0 = S + (size_t)ldS * n;
      T* W1 = W0 + ldS;
      int* sperm = reinterpret_cast<int*>(W1 + ldS);
      int* sopos = sperm + n;
      for (int c = 0; c < n; ++c)
        for (int r = threadIdx.x; r < m; r += blockDim.x)
          S[(size_t)c * ldS + r] = fd.L[(int64_t)c * fd.ld + r];
      for (int k = threadIdx.x; k < n; k += blockDim.x) { sperm[k] = fd.perm[k]; sopos[k] = fd.opos[k]; }
      __syncthreads();
      nel = tpp_fast(S, ldS, m, n, 0, W0, W1, sperm, sopos, fd.D, action, u, small, nullptr,
                     !raw_d);
      __syncthreads();
      if (nel >= 0) {
        for (int c = 0; c < n; ++c)
          for (int r = threadIdx.x; r < m; r += blockDim.x)
            fd.L[(int64_t)c * fd.ld + r] = S[(size_t)c * ldS + r];
        for (int k = threadIdx.x; k < n; k += blockDim.x) { fd.perm[k] = sperm[k]; fd.opos[k] = sopos[k]; }
      }
      F = S;
      ldF = ldS;
    }
    if (threadIdx.x == 0) {
      if (nel < 0) st->status = kDevSingular;
      else { st->nelim = nel; st->p = nel; st->step = 0; }
    }
    __syncthreads();  // D and the factor are complete
    if (nel > 0) tpp_front_contrib(fd, F, ldF, nel, ldsm);
    if (raw_d && nel > 0) tpp_finish_d<T>(fd.D, 0, nel);
  }
}

// ------------------------------------------------------------------------
// contribution block: LD = L(n:m, 0:nelim) * D, then C -= L LD^T
// ------------------------------------------------------------------------
// LD(:, c) = alpha_c L(:, c) + beta_c L(:, partner_c) for the contribution
// rows, where (alpha, beta) are the entries of D = (D^{-1})^{-1} in column c.
// Grid: (row blocks of 128, column chunks of kLdCols, fronts).  Each thread
// issues the loads of all of its chunk's columns before the first store, so
// one memory round trip covers kLdCols columns.
// alpha lv + beta lp for FP32 factors in FP32 instructions, alpha and beta
// given as float pairs (hi + lo): the two hi products with their exact
// errors (FMA), their sum with its exact error (two-sum), then the error
// and lo terms added once, so the result is within an ulp of the FP64
// expression rounded to FP32, a 2x2 column's cancelling products included
__device__ __forceinline__ float ld_entry_f32(float ahi, float alo, float bhi, float blo,
                                              float lv, float lp) {
  const float p1 = __fmul_rn(ahi, lv), e1 = __fmaf_rn(ahi, lv, -p1);
  const float p2 = __fmul_rn(bhi, lp), e2 = __fmaf_rn(bhi, lp, -p2);
  const float sm = __fadd_rn(p1, p2);
  const float bb = __fsub_rn(sm, p1);
  const float es = __fadd_rn(__fsub_rn(p1, __fsub_rn(sm, bb)), __fsub_rn(p2, bb));
  const float corr = __fmaf_rn(alo, lv, __fmaf_rn(blo, lp, __fadd_rn(__fadd_rn(e1, e2), es)));
  return __fadd_rn(sm, corr);
}

template <typename T>
__global__ void __launch_bounds__(128) k_calc_ld(FrontDesc<T>* fds, const FrontState* sts,
                                                 const int* fronts) {
  const int f = fronts[blockIdx.z];
  const FrontDesc<T> fd = fds[f];
  const int nelim = sts[f].nelim;
  const int cm = fd.m - fd.n;
  const int c0 = blockIdx.y * kLdCols;
  if (cm <= 0 || c0 >= nelim) return;
  const int nc = min(kLdCols, nelim - c0);
  __shared__ double alpha[kLdCols], beta[kLdCols];
  __shared__ int partner[kLdCols];
  if ((int)threadIdx.x < nc) {
    const int c = c0 + threadIdx.x;
    const double d11 = fd.D[2 * c];
    if (isinf(d11)) {  // second column of a 2x2
      const double a = fd.D[2 * (c - 1)], b = fd.D[2 * (c - 1) + 1], d = fd.D[2 * c + 1];
      const double det = a * d - b * b;
      alpha[threadIdx.x] = a / det; beta[threadIdx.x] = -b / det; partner[threadIdx.x] = c - 1;
    } else if (c + 1 < nelim && isinf(fd.D[2 * c + 2])) {  // first column of a 2x2
      const double b = fd.D[2 * c + 1], d = fd.D[2 * c + 3];
      const double det = d11 * d - b * b;
      alpha[threadIdx.x] = d / det; beta[threadIdx.x] = -b / det; partner[threadIdx.x] = c + 1;
    } else {
      alpha[threadIdx.x] = (d11 != 0.0) ? 1.0 / d11 : 0.0; beta[threadIdx.x] = 0.0;
      partner[threadIdx.x] = c;
    }
  }
  // FP32 factors: alpha and beta as pairs of floats, hi + lo, formed once
  // per column, so the entries need no FP64 instruction
  __shared__ float ahi[kLdCols], alo[kLdCols], bhi[kLdCols], blo[kLdCols];
  if (sizeof(T) == 4 && (int)threadIdx.x < nc) {
    const int k = threadIdx.x;
    ahi[k] = (float)alpha[k];
    alo[k] = (float)(alpha[k] - (double)ahi[k]);
    bhi[k] = (float)beta[k];
    blo[k] = (float)(beta[k] - (double)bhi[k]);
  }
  __syncthreads();
  for (int rr = blockIdx.x * blockDim.x + threadIdx.x; rr < cm; rr += gridDim.x * blockDim.x) {
    const T* Lr = fd.L + fd.n + rr;
    T lv[kLdCols], lp[kLdCols];
#pragma unroll
    for (int k = 0; k < kLdCols; ++k) {
      bool two;
      if constexpr (sizeof(T) == 4) two = bhi[k] != 0.f || blo[k] != 0.f;
      else two = beta[k] != 0.0;
      lv[k] = (k < nc) ? Lr[(int64_t)(c0 + k) * fd.ld] : T(0);
      lp[k] = (k < nc && two) ? Lr[(int64_t)partner[k] * fd.ld] : T(0);
    }
#pragma unroll
    for (int k = 0; k < kLdCols; ++k) {
      if (k >= nc) continue;
      if constexpr (sizeof(T) == 4)
        fd.LD[(int64_t)(c0 + k) * cm + rr] = ld_entry_f32(ahi[k], alo[k], bhi[k], blo[k], lv[k], lp[k]);
      else
        fd.LD[(int64_t)(c0 + k) * cm + rr] = (T)(alpha[k] * (double)lv[k] + beta[k] * (double)lp[k]);
    }
  }
}

// ------------------------------------------------------------------------
// inertia and counts (NumericSubtree.hxx:249-280, factor.hxx:117-124)
// ------------------------------------------------------------------------
template <typename T>
__global__ void k_stats(const FrontDesc<T>* fds, const FrontState* sts, const int* fronts,
                        Stats* stats, int* node_counts) {
  const int f = fronts[blockIdx.y];
  const FrontDesc<T> fd = fds[f];
  const int nelim = sts[f].nelim;
  int neg = 0, two = 0, zero = 0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nelim; i += gridDim.x * blockDim.x) {
    double a11 = fd.D[2 * i];
    if (isinf(a11)) continue;  // second half of a 2x2
    if (i + 1 < nelim && isinf(fd.D[2 * i + 2])) {
      double a21 = fd.D[2 * i + 1], a22 = fd.D[2 * i + 3];
      two++;
      double det = a11 * a22 - a21 * a21, tr = a11 + a22;
      if (det < 0) neg++;
      else if (tr < 0) neg += 2;
    } else {
      if (a11 == 0.0) zero++;
      if (a11 < 0.0) neg++;
    }
  }
  for (int off = 16; off > 0; off >>= 1) {
    neg += __shfl_xor_sync(0xffffffffu, neg, off);
    two += __shfl_xor_sync(0xffffffffu, two, off);
    zero += __shfl_xor_sync(0xffffffffu, zero, off);
  }
  if ((threadIdx.x & 31) == 0) {
    if (neg) atomicAdd(&stats->num_neg, neg);
    if (two) atomicAdd(&stats->num_two, two);
    if (zero) atomicAdd(&stats->num_zero, zero);
    if (node_counts) {  // per-node inertia (neg, two, zero), indexed by node
      int* nc = node_counts + 3 * fd.node;
      if (neg) atomicAdd(nc, neg);
      if (two) atomicAdd(nc + 1, two);
      if (zero) atomicAdd(nc + 2, zero);
    }
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    long long m = fd.m, a = fd.m - nelim + 1;
    long long sf = 0, sq = 0;
    if (nelim > 0) {
      sf = (a + m) * (m - a + 1) / 2;
      sq = m * (m + 1) * (2 * m + 1) / 6 - (a - 1) * a * (2 * a - 1) / 6;
    }
    atomicAdd(&stats->num_delay, fd.n - nelim);
    atomicAdd((unsigned long long*)&stats->num_factor, (unsigned long long)sf);
    atomicAdd((unsigned long long*)&stats->num_flops, (unsigned long long)sq);
  }
}

}  // namespace

// ---------------- syrk kernel entry points (gemm_kernels.cu) --------------
template <typename T>
void launch_syrk_contrib(FrontDesc<T>* fd, const FrontState* st, const int* fronts, int nf,
                         int max_tiles, cudaStream_t s);

static inline int cdiv(int a, int b) { return (a + b - 1) / b; }

// warps of the FP32 diagonal-block kernel: 17 (one pair per thread; the
// fastest on GB300: 24.8 ms per 48^3 mixed step against 25.9 with 8 warps
// and 27.0 with 4), or 8 or 4 through SPRAL_GB300_DIAG_WARPS
static int diag_f32_warps() {
  const char* e = getenv("SPRAL_GB300_DIAG_WARPS");
  const int v = e ? atoi(e) : 17;
  return (v == 4 || v == 8) ? v : 17;
}

template <typename T>
void launch_app_step(FrontDesc<T>* fd, FrontState* st, const int* fronts, int nf, int step,
                     int max_rows, int max_trail_rows, int max_trail_cols, bool action,
                     double u, double small, cudaStream_t s, PhaseTimer* tm, bool posdef) {
  if (nf <= 0) return;
  pmark(tm, kPhDiag, s);
  if (posdef) {
    launch_pdl(k_app_diag<T, true>, nf, kDiagThreads, 0, s, fd, st, fronts, step, action, small);
  } else if constexpr (std::is_same<T, float>::value) {
    const int nw = diag_f32_warps();
    if (nw == 4)
      launch_pdl(k_app_diag_f32<4>, nf, 4 * 32, 0, s, fd, st, fronts, step, action, small);
    else if (nw == 8)
      launch_pdl(k_app_diag_f32<8>, nf, 8 * 32, 0, s, fd, st, fronts, step, action, small);
    else
      launch_pdl(k_app_diag_f32<kDiagWarps>, nf, kDiagThreads, 0, s, fd, st, fronts, step, action,
                 small);
  } else {
    launch_pdl(k_app_diag<T, false>, nf, kDiagThreads, 0, s, fd, st, fronts, step, action, small);
  }
  note_launches(1);
  // apply (+ row permutation of the eliminated part in extra CTAs)
  const int napply = std::max(1, cdiv(max_rows, apply_rows<T>()));
  const int pcols = step * kBlk;  // upper bound on p
  const int nperm =
      pcols > 0 ? std::max(1, std::min(cdiv(pcols, (apply_threads<T>() / 32) * kPermCols), 128))
                : 0;
  pmark(tm, kPhApply, s);
  launch_pdl(k_app_apply<T>, dim3(napply + nperm, nf), apply_threads<T>(), 0, s, fd, st, fronts,
             u, small, napply);
  note_launches(1);
  // trailing update and fixup in one launch (tile estimate assumes no failed
  // columns so far; after failures the trailing region is wider and the
  // kernel's tile loop covers it, so the launch is never skipped)
  constexpr int tp = panel_tile<T>();
  int tr = std::max(0, cdiv(max_trail_rows, tp)), tc = std::max(0, cdiv(max_trail_cols, tp));
  const int ptiles = std::max(1, std::min(tc * tr - tc * (tc - 1) / 2, 4096));
  const int nfix = std::max(1, cdiv(max_rows, 256));
  pmark(tm, kPhPanel, s);
  launch_pdl(k_app_panel<T, tp>, dim3(ptiles + nfix, nf), 256, 0, s, fd, st, fronts, ptiles);
  note_launches(1);
  pmark(tm, kPhSwap, s);
  const int sx = 1 + std::max(1, std::min(cdiv(max_rows + step * kBlk, 256), 64));
  launch_pdl(k_app_swap<T>, dim3(sx, nf), 256, 0, s, fd, st, fronts);
  note_launches(1);
}

template <typename T>
void launch_app_finish(FrontDesc<T>* fd, FrontState* st, const int* fronts, int nf,
                       cudaStream_t s) {
  if (nf <= 0) return;
  { k_app_finish<T><<<cdiv(nf, 128), 128, 0, s>>>(fd, st, fronts, nf); note_launches(1); }
}

template <typename T>
void launch_panel_end(FrontDesc<T>* fd, FrontState* st, const int* fronts, int nf, int max_n,
                      int panel, cudaStream_t s) {
  if (nf <= 0) return;
  k_panel_fold<<<cdiv(nf, 128), 128, 0, s>>>(st, fronts, nf);
  const int gx = std::max(1, std::min(cdiv(max_n, 128), 64));
  const int gy = std::max(1, cdiv(panel, kLdCols));
  k_panel_ld<T><<<dim3(gx, gy, nf), 128, 0, s>>>(fd, st, fronts);
  note_launches(2);
}

template <typename T>
void launch_panel_close(FrontDesc<T>* fd, FrontState* st, const int* fronts, int nf,
                        cudaStream_t s) {
  if (nf <= 0) return;
  k_panel_close<T><<<nf, 1024, 0, s>>>(fd, st, fronts);
  note_launches(1);
}

template <typename T>
void launch_tpp(FrontDesc<T>* fd, FrontState* st, const int* fronts, int nf, bool action,
                double u, double small, bool all_fronts, cudaStream_t s) {
  if (nf <= 0) return;
  { k_tpp<T><<<nf, kTppThreads, 0, s>>>(fd, st, fronts, action, u, small, all_fronts); note_launches(1); }
}

// Largest dynamic shared memory of k_tpp_small: the fronts of small leaf
// subtrees hold m * n < ~26k entries (their flops are below 4e6), about
// 205 KB in FP64.
// dynamic shared memory ceiling of k_tpp_level: the 227 KB per CTA less its
// static shared memory (the search's records and the contribution's
// per-column coefficients, under 6 KB)
constexpr int kTppSmallSmem = 220 * 1024;

template <typename T>
void launch_tpp_level(FrontDesc<T>* fd, FrontState* st, const int* fronts, int nf, bool action,
                      double u, double small, int max_bytes, int threads, cudaStream_t s) {
  if (nf <= 0) return;
  static int smem_cap = -1;  // per template instance, once per process
  if (smem_cap < 0) {
    // without the opt-in the launch keeps to the default 48 KB: fronts that
    // do not fit are factored in global memory
    smem_cap = cudaFuncSetAttribute(k_tpp_level<T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    kTppSmallSmem) == cudaSuccess
                   ? kTppSmallSmem
                   : 48 * 1024 - 6 * 1024;
    cudaGetLastError();
  }
  const int smem = std::min(std::max(max_bytes, 0), smem_cap);
  threads = threads <= 32 ? 32 : threads <= 64 ? 64 : kTppThreads;
  int dev = 0, nsm = 0, occ = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_tpp_level<T>, threads, smem) !=
      cudaSuccess)
    occ = 1;
  const int grid = std::max(1, std::min(nf, std::max(nsm, 1) * std::max(occ, 1)));
  k_tpp_level<T><<<grid, threads, smem, s>>>(fd, st, fronts, nf, action, u, small, smem);
  note_launches(1);
}

template <typename T>
void launch_calc_ld(FrontDesc<T>* fd, FrontState* st, const int* fronts, int nf, int max_cm,
                    int max_n, cudaStream_t s) {
  if (nf <= 0 || max_cm <= 0) return;
  // column chunks cover the largest possible nelim (the front width)
  int gx = std::max(1, std::min(cdiv(max_cm, 128), 64));
  int gy = std::max(1, cdiv(max_n, kLdCols));
  { k_calc_ld<T><<<dim3(gx, gy, nf), 128, 0, s>>>(fd, st, fronts); note_launches(1); }
}
template <typename T>
void launch_contrib_gemm(FrontDesc<T>* fd, FrontState* st, const int* fronts, int nf, int max_cm,
                         cudaStream_t s) {
  if (nf <= 0 || max_cm <= 0) return;
  int t = cdiv(max_cm, kGemmTile);
  launch_syrk_contrib<T>(fd, st, fronts, nf, t * (t + 1) / 2, s);
}

template <typename T>
void launch_stats(const FrontDesc<T>* fd, const FrontState* st, const int* fronts, int nf,
                  int max_n, Stats* stats, int* node_counts, cudaStream_t s) {
  if (nf <= 0) return;
  int gx = std::max(1, std::min(cdiv(max_n, 256), 64));
  { k_stats<T><<<dim3(gx, nf), 256, 0, s>>>(fd, st, fronts, stats, node_counts); note_launches(1); }
}

#define INST(T)                                                                                 \
  template void launch_app_step<T>(FrontDesc<T>*, FrontState*, const int*, int, int, int, int,  \
                                   int, bool, double, double, cudaStream_t, PhaseTimer*, bool); \
  template void launch_app_finish<T>(FrontDesc<T>*, FrontState*, const int*, int, cudaStream_t); \
  template void launch_panel_end<T>(FrontDesc<T>*, FrontState*, const int*, int, int, int,      \
                                    cudaStream_t);                                              \
  template void launch_panel_close<T>(FrontDesc<T>*, FrontState*, const int*, int, cudaStream_t); \
  template void launch_tpp<T>(FrontDesc<T>*, FrontState*, const int*, int, bool, double, double, \
                              bool, cudaStream_t);                                              \
  template void launch_tpp_level<T>(FrontDesc<T>*, FrontState*, const int*, int, bool, double,  \
                                    double, int, int, cudaStream_t);                            \
  template void launch_calc_ld<T>(FrontDesc<T>*, FrontState*, const int*, int, int, int,        \
                                  cudaStream_t);                                                 \
  template void launch_contrib_gemm<T>(FrontDesc<T>*, FrontState*, const int*, int, int,        \
                                       cudaStream_t);                                           \
  template void launch_stats<T>(const FrontDesc<T>*, const FrontState*, const int*, int, int,    \
                                Stats*, int*, cudaStream_t);
INST(double)
INST(float)
#undef INST

}  // namespace ssids300
