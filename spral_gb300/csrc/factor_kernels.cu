// Dense per-front LDL^T with a-posteriori threshold pivoting on sm_103a.
//
// One APP step processes a block of up to 32 candidate columns [p, p+bs) of
// every active front of a level at once:
//   k_app_diag      one warp per front: complete pivoting inside the block
//                   (semantics of block_ldlt, src/ssids/cpu/kernels/
//                   block_ldlt.hxx:290-413), FP64 arithmetic, writes L11, D^{-1}
//                   and the local permutation
//   k_app_rowperm   applies the block permutation to the eliminated L rows
//   k_app_apply     rows below: X = A21 L11^{-T}, L21 = X D^{-1} and the
//                   a-posteriori test |l| <= 1/u (apply_pivot/check_threshold,
//                   ldlt_app.cxx:316-436); X (= L21 D) is kept for the update
//   k_app_fixup     Column::adjust (ldlt_app.cxx:112-130) and, for failed
//                   columns, the restore-and-update of restore_if_required +
//                   update, computed as X_f L_ff^T (rows below) and
//                   L_ff D_f L_ff^T (diagonal block)
//   k_syrk (panel)  trailing update of the candidate columns (gemm_kernels.cu)
//   k_app_swap_*    failed columns are moved to the end of the APP range
// After ceil(n/32) steps k_app_finish records nelim; k_tpp finishes failed
// columns with threshold partial pivoting (ldlt_tpp.cxx:166-270) where the
// reference does (root fronts or failed_pivot_method = tpp); k_calc_ld and
// k_syrk (contrib) form the contribution block; k_stats counts inertia.
#include <cfloat>
#include <cmath>
#include <cstdio>

#include "ssids_gpu.cuh"

namespace ssids300 {

namespace {

__device__ __forceinline__ double dinf() { return __longlong_as_double(0x7ff0000000000000LL); }

// read symmetric entry (r, c) of a lower-stored front (both < n or r >= n > c)
template <typename T>
__device__ __forceinline__ double sym_at(const T* L, int ld, int r, int c) {
  return (r >= c) ? (double)L[(int64_t)c * ld + r] : (double)L[(int64_t)r * ld + c];
}

// ------------------------------------------------------------------------
// k_app_diag: advance state, factor the diagonal block with complete pivoting
// ------------------------------------------------------------------------
template <typename T>
__global__ void __launch_bounds__(32) k_app_diag(FrontDesc<T>* fds, FrontState* sts,
                                                 const int* fronts, int step, bool action,
                                                 double small) {
  const int f = fronts[blockIdx.x];
  FrontDesc<T> fd = fds[f];
  FrontState* st = &sts[f];
  const int lane = threadIdx.x;
  __shared__ double blk[kBlk][kBlk + 1];  // blk[c][r], full symmetric
  __shared__ double wv[2][kBlk];          // unscaled pivot columns
  __shared__ double lv[2][kBlk];          // scaled pivot columns
  __shared__ double dd[2 * kBlk + 2];
  __shared__ int lp[kBlk];
  __shared__ int s_piv[3];  // pivsiz, idx1, idx2
  __shared__ double s_det[2];

  int p, end;
  if (step == 0) {
    p = 0;
    end = fd.n;
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
  __syncwarp();
  if (lane == 0) {
    st->p = p;
    st->end = end;
    st->bs = bs;
    st->npass_raw = bs;
    st->npass = bs;
    st->step = step;
  }
  if (bs == 0) return;

  // load block (lower storage) as full symmetric
  for (int c = 0; c < bs; ++c) {
    int r = lane;
    if (r < bs) blk[c][r] = sym_at(fd.L, fd.ld, p + r, p + c);
  }
  lp[lane] = lane;
  for (int i = lane; i < 2 * kBlk + 2; i += 32) dd[i] = 0.0;
  __syncwarp();

  bool singular = false;
  for (int q = 0; q < bs;) {
    // argmax over lower triangle of the active block (first in column order)
    double best = -1.0;
    int br = -1;
    const int c = lane;
    if (c >= q && c < bs) {
      for (int r = c; r < bs; ++r) {
        double v = fabs(blk[c][r]);
        if (v > best) { best = v; br = r; }
      }
    }
    int bc = (br >= 0) ? c : 1 << 20;
    for (int off = 16; off > 0; off >>= 1) {
      double ob = __shfl_xor_sync(0xffffffffu, best, off);
      int obr = __shfl_xor_sync(0xffffffffu, br, off);
      int obc = __shfl_xor_sync(0xffffffffu, bc, off);
      if (ob > best || (ob == best && obc < bc)) { best = ob; br = obr; bc = obc; }
    }
    if (best < small) {
      if (!action) { singular = true; break; }
      // remaining columns are zero pivots
      for (int cc = q; cc < bs; ++cc) {
        if (lane >= cc && lane < bs) blk[cc][lane] = 0.0;
        if (lane == 0) { dd[2 * cc] = 0.0; dd[2 * cc + 1] = 0.0; }
      }
      __syncwarp();
      break;
    }
    if (lane == 0) {
      int t = br, mm = bc;
      int pivsiz, i1, i2 = -1;
      if (t == mm) {
        pivsiz = 1; i1 = t;
      } else {
        double a11 = blk[mm][mm], a22 = blk[t][t], a21 = blk[mm][t];
        double detscale = 1.0 / fabs(a21);
        double detpiv = (a11 * detscale) * a22 - fabs(a21);
        if (fabs(detpiv) >= fabs(a21) / 2) {
          pivsiz = 2; i1 = mm; i2 = t;
          s_det[0] = detscale; s_det[1] = detpiv;
        } else if (fabs(a11) > fabs(a22)) {
          pivsiz = 1; i1 = mm;
        } else {
          pivsiz = 1; i1 = t;
        }
      }
      s_piv[0] = pivsiz; s_piv[1] = i1; s_piv[2] = i2;
    }
    __syncwarp();
    const int pivsiz = s_piv[0];
    // symmetric swaps q <-> i1 (and q+1 <-> i2)
    for (int sw = 0; sw < pivsiz; ++sw) {
      int a = q + sw, b = s_piv[1 + sw];
      if (a != b) {
        // rows
        if (lane < bs) { double tmp = blk[lane][a]; blk[lane][a] = blk[lane][b]; blk[lane][b] = tmp; }
        __syncwarp();
        if (lane < bs) { double tmp = blk[a][lane]; blk[a][lane] = blk[b][lane]; blk[b][lane] = tmp; }
        if (lane == 0) { int tmp = lp[a]; lp[a] = lp[b]; lp[b] = tmp; }
        __syncwarp();
      }
    }
    if (pivsiz == 1) {
      double d11 = 1.0 / blk[q][q];
      int r = lane;
      if (r > q && r < bs) {
        double w = blk[q][r];
        wv[0][r] = w;
        lv[0][r] = w * d11;
      }
      __syncwarp();
      int cc = lane;
      if (cc > q && cc < bs) {
        double wc = wv[0][cc];
        for (int rr = q + 1; rr < bs; ++rr) blk[cc][rr] -= wc * lv[0][rr];
      }
      __syncwarp();
      if (r > q && r < bs) blk[q][r] = lv[0][r];
      if (lane == 0) { blk[q][q] = 1.0; dd[2 * q] = d11; dd[2 * q + 1] = 0.0; }
      __syncwarp();
      q += 1;
    } else {
      double detscale = s_det[0], detpiv = s_det[1];
      double a11 = blk[q][q], a22 = blk[q + 1][q + 1], a21 = blk[q][q + 1];
      double d11 = (a22 * detscale) / detpiv;
      double d22 = (a11 * detscale) / detpiv;
      double d21 = (-a21 * detscale) / detpiv;
      int r = lane;
      if (r > q + 1 && r < bs) {
        double w1 = blk[q][r], w2 = blk[q + 1][r];
        wv[0][r] = w1; wv[1][r] = w2;
        lv[0][r] = d11 * w1 + d21 * w2;
        lv[1][r] = d21 * w1 + d22 * w2;
      }
      __syncwarp();
      int cc = lane;
      if (cc > q + 1 && cc < bs) {
        double w1 = wv[0][cc], w2 = wv[1][cc];
        for (int rr = q + 2; rr < bs; ++rr) blk[cc][rr] -= w1 * lv[0][rr] + w2 * lv[1][rr];
      }
      __syncwarp();
      if (r > q + 1 && r < bs) { blk[q][r] = lv[0][r]; blk[q + 1][r] = lv[1][r]; }
      if (lane == 0) {
        blk[q][q] = 1.0; blk[q][q + 1] = 0.0; blk[q + 1][q + 1] = 1.0;
        dd[2 * q] = d11; dd[2 * q + 1] = d21; dd[2 * q + 2] = dinf(); dd[2 * q + 3] = d22;
      }
      __syncwarp();
      q += 2;
    }
  }
  if (singular) {
    if (lane == 0) { st->status = kDevSingular; st->bs = 0; }
    return;
  }
  // write L11 (lower), D, step buffer, permutation
  for (int cc = 0; cc < bs; ++cc) {
    int r = lane;
    if (r >= cc && r < bs) {
      double v = blk[cc][r];
      fd.L[(int64_t)(p + cc) * fd.ld + p + r] = (T)v;
      fd.step[cc * kBlk + r] = v;
    }
  }
  if (lane < bs) {
    fd.D[2 * (p + lane)] = dd[2 * lane];
    fd.D[2 * (p + lane) + 1] = dd[2 * lane + 1];
    fd.step[kBlk * kBlk + 2 * lane] = dd[2 * lane];
    fd.step[kBlk * kBlk + 2 * lane + 1] = dd[2 * lane + 1];
    fd.lperm[lane] = lp[lane];
  }
  int oldp = (lane < bs) ? fd.perm[p + lp[lane]] : 0;
  int oldo = (lane < bs) ? fd.opos[p + lp[lane]] : 0;
  __syncwarp();
  if (lane < bs) { fd.perm[p + lane] = oldp; fd.opos[p + lane] = oldo; }
}

// ------------------------------------------------------------------------
// k_app_rowperm: permute rows [p, p+bs) of the eliminated columns [0, p)
// ------------------------------------------------------------------------
template <typename T>
__global__ void k_app_rowperm(FrontDesc<T>* fds, const FrontState* sts, const int* fronts) {
  const int f = fronts[blockIdx.y];
  const FrontState st = sts[f];
  if (st.bs == 0 || st.p == 0) return;
  FrontDesc<T> fd = fds[f];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  int src = (lane < st.bs) ? fd.lperm[lane] : lane;
  for (int c = blockIdx.x * nw + warp; c < st.p; c += gridDim.x * nw) {
    T* col = fd.L + (int64_t)c * fd.ld + st.p;
    T v = (lane < st.bs) ? col[src] : T(0);
    __syncwarp();
    if (lane < st.bs) col[lane] = v;
  }
}

// ------------------------------------------------------------------------
// k_app_apply: rows below the block; solve, scale, threshold test
// ------------------------------------------------------------------------
template <typename T>
__global__ void __launch_bounds__(kApplyRows) k_app_apply(FrontDesc<T>* fds, FrontState* sts,
                                                          const int* fronts, double u,
                                                          double small) {
  const int f = fronts[blockIdx.y];
  FrontState* st = &sts[f];
  const int bs = st->bs;
  if (bs == 0) return;
  const int p = st->p;
  FrontDesc<T> fd = fds[f];
  const int r0 = p + bs;
  const int nrows = fd.m - r0;
  if (nrows <= 0) return;
  __shared__ double l11[kBlk][kBlk + 1];  // l11[j][k] = L(j,k), row-major for broadcast
  __shared__ double dd[2 * kBlk + 2];
  __shared__ int lp[kBlk];
  for (int i = threadIdx.x; i < kBlk * kBlk; i += blockDim.x) {
    int c = i / kBlk, r = i % kBlk;
    l11[r][c] = (r > c && r < bs && c < bs) ? fd.step[c * kBlk + r] : 0.0;
  }
  for (int i = threadIdx.x; i < 2 * kBlk + 2; i += blockDim.x)
    dd[i] = (i < 2 * bs) ? fd.step[kBlk * kBlk + i] : 0.0;
  if (threadIdx.x < kBlk) lp[threadIdx.x] = (threadIdx.x < bs) ? fd.lperm[threadIdx.x] : 0;
  __syncthreads();
  const double thresh = 1.0 / u;
  int myfail = bs;
  for (int tile = blockIdx.x; tile * kApplyRows < nrows; tile += gridDim.x) {
    const int rr = tile * kApplyRows + threadIdx.x;
    const bool valid = rr < nrows;
    const int r = r0 + rr;
    double x[kBlk];
#pragma unroll
    for (int j = 0; j < kBlk; ++j)
      x[j] = (valid && j < bs) ? (double)fd.L[(int64_t)(p + lp[j]) * fd.ld + r] : 0.0;
#pragma unroll
    for (int j = 1; j < kBlk; ++j) {
      double s = x[j];
#pragma unroll
      for (int k = 0; k < j; ++k) s -= x[k] * l11[j][k];
      x[j] = s;
    }
    if (valid) {
      T* W = fd.W + rr;
#pragma unroll
      for (int j = 0; j < kBlk; ++j) {
        if (j < bs) {
          const double dj = dd[2 * j];
          if (!isinf(dj)) {  // (second half of a 2x2 is handled with the first)
            if (j + 1 < bs && isinf(dd[2 * j + 2])) {
              const double d21 = dd[2 * j + 1], d22 = dd[2 * j + 3];
              const double x1 = x[j], x2 = x[j + 1 < kBlk ? j + 1 : kBlk - 1];
              const double l1 = dj * x1 + d21 * x2, l2 = d21 * x1 + d22 * x2;
              fd.L[(int64_t)(p + j) * fd.ld + r] = (T)l1;
              fd.L[(int64_t)(p + j + 1) * fd.ld + r] = (T)l2;
              W[(int64_t)j * fd.ld] = (T)x1;
              W[(int64_t)(j + 1) * fd.ld] = (T)x2;
              int cand = (fabs(l1) > thresh) ? j : ((fabs(l2) > thresh) ? j + 1 : bs);
              myfail = min(myfail, cand);
            } else {
              double l, w;
              if (dj == 0.0) {
                const double v = x[j];
                l = (fabs(v) < small) ? 0.0 : dinf() * v;
                w = 0.0;
              } else {
                l = x[j] * dj;
                w = x[j];
              }
              fd.L[(int64_t)(p + j) * fd.ld + r] = (T)l;
              W[(int64_t)j * fd.ld] = (T)w;
              if (fabs(l) > thresh) myfail = min(myfail, j);
            }
          }
        }
      }
    }
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
// k_app_fixup: adjust npass; restore + update failed columns
// ------------------------------------------------------------------------
template <typename T>
__global__ void __launch_bounds__(kApplyRows) k_app_fixup(FrontDesc<T>* fds, FrontState* sts,
                                                          const int* fronts) {
  const int f = fronts[blockIdx.y];
  FrontState* st = &sts[f];
  const int bs = st->bs;
  if (bs == 0) return;
  const int p = st->p;
  FrontDesc<T> fd = fds[f];
  const int np = adjust_npass(st->npass_raw, bs, p, fd.D);
  if (blockIdx.x == 0 && threadIdx.x == 0) st->npass = np;
  const int nf = bs - np;
  if (nf == 0) return;
  __shared__ double l11[kBlk][kBlk + 1];
  __shared__ double ldf[kBlk][kBlk + 1];
  for (int i = threadIdx.x; i < kBlk * kBlk; i += blockDim.x) {
    int c = i / kBlk, r = i % kBlk;
    double v = (r < bs && c < bs) ? ((r == c) ? 1.0 : (r > c ? fd.step[c * kBlk + r] : 0.0)) : 0.0;
    l11[r][c] = v;
  }
  __syncthreads();
  const int r0 = p + bs, nrows = fd.m - r0;
  // rows below: A(r, p+np+i) = sum_{k<=i} X(r, np+k) * L(np+i, np+k)
  for (int tile = blockIdx.x; tile * kApplyRows < nrows; tile += gridDim.x) {
    int rr = tile * kApplyRows + threadIdx.x;
    if (rr < nrows) {
      const T* W = fd.W + rr;
      double xf[kBlk];
#pragma unroll
      for (int i = 0; i < kBlk; ++i) xf[i] = (i < nf) ? (double)W[(int64_t)(np + i) * fd.ld] : 0.0;
      for (int i = 0; i < nf; ++i) {
        double s = 0.0;
#pragma unroll
        for (int k = 0; k < kBlk; ++k)
          if (k <= i) s += xf[k] * l11[np + i][np + k];
        fd.L[(int64_t)(p + np + i) * fd.ld + r0 + rr] = (T)s;
      }
    }
  }
  if (blockIdx.x == 0) {
    // diagonal failed block S = L_ff D_f L_ff^T
    const double* d = fd.step + kBlk * kBlk;
    // LD = L_ff * D_f  (D_f = inverse of stored inverse)
    for (int i = threadIdx.x; i < nf * nf; i += blockDim.x) {
      int r = i % nf, c = i / nf;
      ldf[r][c] = 0.0;
    }
    __syncthreads();
    if (threadIdx.x < nf) {
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

template <typename T>
__global__ void k_app_swap_gather(FrontDesc<T>* fds, const FrontState* sts, const int* fronts) {
  const int f = fronts[blockIdx.y];
  const FrontState st = sts[f];
  if (st.bs == 0 || st.bs == st.npass) return;
  FrontDesc<T> fd = fds[f];
  SwapRanges sr = swap_ranges(st);
  const int nl = 2 * sr.npairs;
  for (int li = blockIdx.x; li < nl; li += gridDim.x) {
    int s = (li < sr.npairs) ? sr.a0 + li : sr.b0 + (li - sr.npairs);
    T* line = fd.swapbuf + (int64_t)li * fd.ld;
    for (int x = threadIdx.x; x < fd.m; x += blockDim.x) line[x] = (T)sym_at(fd.L, fd.ld, x, s);
    if (threadIdx.x == 0) {
      int* ib = reinterpret_cast<int*>(fd.swapbuf + (int64_t)nl * fd.ld);
      ib[2 * li] = fd.perm[s];
      ib[2 * li + 1] = fd.opos[s];
    }
  }
}

template <typename T>
__global__ void k_app_swap_scatter(FrontDesc<T>* fds, const FrontState* sts, const int* fronts) {
  const int f = fronts[blockIdx.y];
  const FrontState st = sts[f];
  if (st.bs == 0 || st.bs == st.npass) return;
  FrontDesc<T> fd = fds[f];
  SwapRanges sr = swap_ranges(st);
  const int nl = 2 * sr.npairs;
  for (int li = blockIdx.x; li < nl; li += gridDim.x) {
    int s = (li < sr.npairs) ? sr.a0 + li : sr.b0 + (li - sr.npairs);
    int ps = swap_partner(sr, s);
    int pli = (ps >= sr.a0 && ps < sr.a0 + sr.npairs) ? ps - sr.a0 : sr.npairs + (ps - sr.b0);
    const T* line = fd.swapbuf + (int64_t)pli * fd.ld;
    for (int x = threadIdx.x; x < fd.m; x += blockDim.x) {
      T v = line[swap_partner(sr, x)];
      if (x <= s) fd.L[(int64_t)x * fd.ld + s] = v;
      else fd.L[(int64_t)s * fd.ld + x] = v;
    }
    if (threadIdx.x == 0) {
      const int* ib = reinterpret_cast<const int*>(fd.swapbuf + (int64_t)nl * fd.ld);
      fd.perm[s] = ib[2 * pli];
      fd.opos[s] = ib[2 * pli + 1];
    }
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

__device__ __forceinline__ double block_max(double v, double* red) {
  for (int off = 16; off > 0; off >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, off));
  __syncthreads();
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  double r = red[0];
  for (int i = 1; i < (int)(blockDim.x >> 5); ++i) r = fmax(r, red[i]);
  __syncthreads();
  return r;
}

template <typename T>
__device__ void tpp_sym_swap(FrontDesc<T>& fd, int i, int j) {
  if (i == j) return;
  if (j < i) { int t = i; i = j; j = t; }
  T* L = fd.L;
  const int ld = fd.ld;
  for (int c = threadIdx.x; c < i; c += blockDim.x) {
    T t = L[(int64_t)c * ld + i]; L[(int64_t)c * ld + i] = L[(int64_t)c * ld + j]; L[(int64_t)c * ld + j] = t;
  }
  for (int r = i + 1 + threadIdx.x; r < j; r += blockDim.x) {
    T t = L[(int64_t)i * ld + r]; L[(int64_t)i * ld + r] = L[(int64_t)r * ld + j]; L[(int64_t)r * ld + j] = t;
  }
  if (threadIdx.x == 0) {
    T t = L[(int64_t)i * ld + i]; L[(int64_t)i * ld + i] = L[(int64_t)j * ld + j]; L[(int64_t)j * ld + j] = t;
    int pt = fd.perm[i]; fd.perm[i] = fd.perm[j]; fd.perm[j] = pt;
    int ot = fd.opos[i]; fd.opos[i] = fd.opos[j]; fd.opos[j] = ot;
  }
  for (int r = j + 1 + threadIdx.x; r < fd.m; r += blockDim.x) {
    T t = L[(int64_t)i * ld + r]; L[(int64_t)i * ld + r] = L[(int64_t)j * ld + r]; L[(int64_t)j * ld + r] = t;
  }
  __syncthreads();
}

template <typename T>
__device__ bool tpp_col_small(const FrontDesc<T>& fd, int idx, int from, double small, double* red) {
  double v = 0.0;
  for (int c = from + threadIdx.x; c < idx; c += blockDim.x) v = fmax(v, fabs((double)fd.L[(int64_t)c * fd.ld + idx]));
  for (int r = idx + threadIdx.x; r < fd.m; r += blockDim.x) v = fmax(v, fabs((double)fd.L[(int64_t)idx * fd.ld + r]));
  return block_max(v, red) < small;
}

template <typename T>
__device__ double tpp_rc_max_excl(const FrontDesc<T>& fd, int col, int nel, int excl, double* red) {
  double v = 0.0;
  for (int c = nel + threadIdx.x; c < col; c += blockDim.x)
    if (c != excl) v = fmax(v, fabs((double)fd.L[(int64_t)c * fd.ld + col]));
  for (int r = col + 1 + threadIdx.x; r < fd.m; r += blockDim.x)
    if (r != excl) v = fmax(v, fabs((double)fd.L[(int64_t)col * fd.ld + r]));
  return block_max(v, red);
}

template <typename T>
__device__ void tpp_zero_col(FrontDesc<T>& fd, int col) {
  for (int r = col + threadIdx.x; r < fd.m; r += blockDim.x) fd.L[(int64_t)col * fd.ld + r] = T(0);
  if (threadIdx.x == 0) { fd.D[2 * col] = 0.0; fd.D[2 * col + 1] = 0.0; }
  __syncthreads();
}

// scale pivot column(s) at nel, keep unscaled copy in W, update trailing
template <typename T>
__device__ void tpp_apply(FrontDesc<T>& fd, int nel, int ps, double d11, double d21, double d22) {
  T* L = fd.L;
  const int ld = fd.ld, m = fd.m, n = fd.n;
  T* w0 = fd.W;            // unscaled copies indexed by row
  T* w1 = fd.W + fd.ld;
  if (ps == 1) {
    for (int r = nel + 1 + threadIdx.x; r < m; r += blockDim.x) {
      double a = (double)L[(int64_t)nel * ld + r];
      w0[r] = (T)a;
      L[(int64_t)nel * ld + r] = (T)(a * d11);
    }
    if (threadIdx.x == 0) { L[(int64_t)nel * ld + nel] = T(1); fd.D[2 * nel] = d11; fd.D[2 * nel + 1] = 0.0; }
  } else {
    for (int r = nel + 2 + threadIdx.x; r < m; r += blockDim.x) {
      double a1 = (double)L[(int64_t)nel * ld + r], a2 = (double)L[(int64_t)(nel + 1) * ld + r];
      w0[r] = (T)a1; w1[r] = (T)a2;
      L[(int64_t)nel * ld + r] = (T)(d11 * a1 + d21 * a2);
      L[(int64_t)(nel + 1) * ld + r] = (T)(d21 * a1 + d22 * a2);
    }
    if (threadIdx.x == 0) {
      L[(int64_t)nel * ld + nel] = T(1);
      L[(int64_t)nel * ld + nel + 1] = T(0);
      L[(int64_t)(nel + 1) * ld + nel + 1] = T(1);
      fd.D[2 * nel] = d11; fd.D[2 * nel + 1] = d21;
      fd.D[2 * nel + 2] = dinf(); fd.D[2 * nel + 3] = d22;
    }
  }
  __syncthreads();
  // trailing update of fully-summed columns [nel+ps, n), rows [c, m)
  const int c0 = nel + ps;
  const int ncols = n - c0;
  if (ncols > 0) {
    const int64_t rows = m - c0;
    const int64_t total = rows * ncols;
    for (int64_t e = threadIdx.x; e < total; e += blockDim.x) {
      int c = c0 + (int)(e / rows);
      int r = c0 + (int)(e % rows);
      if (r < c) continue;
      double v = (double)w0[c] * (double)L[(int64_t)nel * ld + r];
      if (ps == 2) v += (double)w1[c] * (double)L[(int64_t)(nel + 1) * ld + r];
      L[(int64_t)c * ld + r] = (T)((double)L[(int64_t)c * ld + r] - v);
    }
  }
  __syncthreads();
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
  __shared__ double red[kTppThreads / 32];
  __shared__ int s_t;
  int nel = st->nelim;
  const int n = fd.n, m = fd.m;
  const T* L = fd.L;
  const int ld = fd.ld;
  while (nel < n) {
    if (tpp_col_small(fd, nel, nel, small, red)) {
      if (!action) { if (threadIdx.x == 0) st->status = kDevSingular; return; }
      tpp_zero_col(fd, nel);
      nel++;
      continue;
    }
    int p;
    bool done = false;
    for (p = nel + 1; p < n; ++p) {
      if (tpp_col_small(fd, p, nel, small, red)) {
        if (!action) { if (threadIdx.x == 0) st->status = kDevSingular; return; }
        tpp_sym_swap(fd, p, nel);
        tpp_zero_col(fd, nel);
        nel++;
        done = true;
        break;
      }
      // t = argmax_{c in [nel, p)} |a(p, c)| (first maximum)
      if (threadIdx.x == 0) {
        int t = nel;
        double bv = fabs((double)L[(int64_t)nel * ld + p]);
        for (int c = nel + 1; c < p; ++c) {
          double v = fabs((double)L[(int64_t)c * ld + p]);
          if (v > bv) { bv = v; t = c; }
        }
        s_t = t;
      }
      __syncthreads();
      const int t = s_t;
      double maxt = tpp_rc_max_excl(fd, t, nel, p, red);
      double maxp = tpp_rc_max_excl(fd, p, nel, t, red);
      {
        double a11 = (double)L[(int64_t)t * ld + t], a21 = (double)L[(int64_t)t * ld + p];
        double a22 = (double)L[(int64_t)p * ld + p];
        double maxpiv = fmax(fabs(a11), fmax(fabs(a21), fabs(a22)));
        bool ok = false;
        double d0 = 0, d1 = 0, d3 = 0;
        if (!(maxpiv < small)) {
          double detscale = 1 / maxpiv;
          double det0 = (a11 * detscale) * a22, det1 = (a21 * detscale) * a21;
          double detpiv = det0 - det1;
          if (!(fabs(detpiv) < fmax(small, fmax(fabs(det0 / 2), fabs(det1 / 2))))) {
            d0 = (a22 * detscale) / detpiv;
            d1 = (-a21 * detscale) / detpiv;
            d3 = (a11 * detscale) / detpiv;
            if (fmax(maxp, maxt) < small) ok = true;
            else {
              double x1 = fabs(d0) * maxt + fabs(d1) * maxp;
              double x2 = fabs(d1) * maxt + fabs(d3) * maxp;
              ok = (u * fmax(x1, x2) < 1.0);
            }
          }
        }
        if (ok) {
          tpp_sym_swap(fd, t, nel);
          tpp_sym_swap(fd, p, nel + 1);
          tpp_apply(fd, nel, 2, d0, d1, d3);
          nel += 2;
          done = true;
          break;
        }
      }
      maxp = fmax(maxp, fabs((double)L[(int64_t)t * ld + p]));
      if (fabs((double)L[(int64_t)p * ld + p]) >= u * maxp) {
        tpp_sym_swap(fd, p, nel);
        double d11 = 1.0 / (double)L[(int64_t)nel * ld + nel];
        tpp_apply(fd, nel, 1, d11, 0, 0);
        nel += 1;
        done = true;
        break;
      }
    }
    if (!done) {
      p = nel;
      double maxp = tpp_rc_max_excl(fd, p, nel, -1, red);
      if (fabs((double)L[(int64_t)p * ld + p]) >= u * maxp) {
        double d11 = 1.0 / (double)L[(int64_t)nel * ld + nel];
        tpp_apply(fd, nel, 1, d11, 0, 0);
        nel += 1;
      } else {
        break;
      }
    }
  }
  if (threadIdx.x == 0) { st->nelim = nel; st->p = nel; }
  (void)m;
}

// ------------------------------------------------------------------------
// contribution block: LD = L(n:m, 0:nelim) * D, then C -= L LD^T
// ------------------------------------------------------------------------
template <typename T>
__global__ void k_calc_ld(FrontDesc<T>* fds, const FrontState* sts, const int* fronts) {
  const int f = fronts[blockIdx.y];
  FrontDesc<T> fd = fds[f];
  const int nelim = sts[f].nelim;
  const int cm = fd.m - fd.n;
  if (cm <= 0 || nelim <= 0) return;
  for (int rr = blockIdx.x * blockDim.x + threadIdx.x; rr < cm; rr += gridDim.x * blockDim.x) {
    const int r = fd.n + rr;
    for (int c = 0; c < nelim;) {
      double d11 = fd.D[2 * c];
      if (c + 1 == nelim || isfinite(fd.D[2 * c + 2])) {
        if (d11 != 0.0) d11 = 1.0 / d11;
        fd.LD[(int64_t)c * cm + rr] = (T)(d11 * (double)fd.L[(int64_t)c * fd.ld + r]);
        c += 1;
      } else {
        double d21 = fd.D[2 * c + 1], d22 = fd.D[2 * c + 3];
        double det = d11 * d22 - d21 * d21;
        double e11 = d11 / det, e21 = d21 / det, e22 = d22 / det;
        double a1 = (double)fd.L[(int64_t)c * fd.ld + r], a2 = (double)fd.L[(int64_t)(c + 1) * fd.ld + r];
        fd.LD[(int64_t)c * cm + rr] = (T)(e22 * a1 - e21 * a2);
        fd.LD[(int64_t)(c + 1) * cm + rr] = (T)(-e21 * a1 + e11 * a2);
        c += 2;
      }
    }
  }
}

// ------------------------------------------------------------------------
// inertia and counts (NumericSubtree.hxx:249-280, factor.hxx:117-124)
// ------------------------------------------------------------------------
template <typename T>
__global__ void k_stats(const FrontDesc<T>* fds, const FrontState* sts, const int* fronts,
                        Stats* stats) {
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
void launch_syrk_panel(FrontDesc<T>* fd, const FrontState* st, const int* fronts, int nf,
                       int max_tiles, cudaStream_t s);
template <typename T>
void launch_syrk_contrib(FrontDesc<T>* fd, const FrontState* st, const int* fronts, int nf,
                         int max_tiles, cudaStream_t s);

static inline int cdiv(int a, int b) { return (a + b - 1) / b; }

template <typename T>
void launch_app_step(FrontDesc<T>* fd, FrontState* st, const int* fronts, int nf, int step,
                     int max_rows, int max_trail_rows, int max_trail_cols, bool action,
                     double u, double small, cudaStream_t s) {
  if (nf <= 0) return;
  { k_app_diag<T><<<nf, 32, 0, s>>>(fd, st, fronts, step, action, small); note_launches(1); }
  {
    int pcols = step * kBlk;  // columns of L to the left (upper bound on p)
    int gx = std::max(1, std::min(cdiv(pcols, 8), 64));
    if (pcols > 0) { k_app_rowperm<T><<<dim3(gx, nf), 256, 0, s>>>(fd, st, fronts); note_launches(1); }
  }
  int gx = std::max(1, cdiv(max_rows, kApplyRows));
  { k_app_apply<T><<<dim3(gx, nf), kApplyRows, 0, s>>>(fd, st, fronts, u, small); note_launches(1); }
  { k_app_fixup<T><<<dim3(gx, nf), kApplyRows, 0, s>>>(fd, st, fronts); note_launches(1); }
  // tile estimate assumes no failed columns so far; after failures the
  // trailing region is wider and the kernel's grid-stride loop covers it, so
  // the launch is never skipped
  int tr = std::max(0, cdiv(max_trail_rows, kGemmTile)), tc = std::max(0, cdiv(max_trail_cols, kGemmTile));
  int tiles = tc * tr - tc * (tc - 1) / 2;
  launch_syrk_panel<T>(fd, st, fronts, nf, std::max(tiles, 1), s);
  { k_app_swap_gather<T><<<dim3(64, nf), 256, 0, s>>>(fd, st, fronts); note_launches(1); }
  { k_app_swap_scatter<T><<<dim3(64, nf), 256, 0, s>>>(fd, st, fronts); note_launches(1); }
}

template <typename T>
void launch_app_finish(FrontDesc<T>* fd, FrontState* st, const int* fronts, int nf,
                       cudaStream_t s) {
  if (nf <= 0) return;
  { k_app_finish<T><<<cdiv(nf, 128), 128, 0, s>>>(fd, st, fronts, nf); note_launches(1); }
}

template <typename T>
void launch_tpp(FrontDesc<T>* fd, FrontState* st, const int* fronts, int nf, bool action,
                double u, double small, bool all_fronts, cudaStream_t s) {
  if (nf <= 0) return;
  { k_tpp<T><<<nf, kTppThreads, 0, s>>>(fd, st, fronts, action, u, small, all_fronts); note_launches(1); }
}

template <typename T>
void launch_calc_ld(FrontDesc<T>* fd, FrontState* st, const int* fronts, int nf, int max_cm,
                    cudaStream_t s) {
  if (nf <= 0 || max_cm <= 0) return;
  int gx = std::max(1, std::min(cdiv(max_cm, 128), 256));
  { k_calc_ld<T><<<dim3(gx, nf), 128, 0, s>>>(fd, st, fronts); note_launches(1); }
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
                  int max_n, Stats* stats, cudaStream_t s) {
  if (nf <= 0) return;
  int gx = std::max(1, std::min(cdiv(max_n, 256), 64));
  { k_stats<T><<<dim3(gx, nf), 256, 0, s>>>(fd, st, fronts, stats); note_launches(1); }
}

#define INST(T)                                                                                 \
  template void launch_app_step<T>(FrontDesc<T>*, FrontState*, const int*, int, int, int, int,  \
                                   int, bool, double, double, cudaStream_t);                    \
  template void launch_app_finish<T>(FrontDesc<T>*, FrontState*, const int*, int, cudaStream_t); \
  template void launch_tpp<T>(FrontDesc<T>*, FrontState*, const int*, int, bool, double, double, \
                              bool, cudaStream_t);                                              \
  template void launch_calc_ld<T>(FrontDesc<T>*, FrontState*, const int*, int, int, cudaStream_t); \
  template void launch_contrib_gemm<T>(FrontDesc<T>*, FrontState*, const int*, int, int,        \
                                       cudaStream_t);                                           \
  template void launch_stats<T>(const FrontDesc<T>*, const FrontState*, const int*, int, int,    \
                                Stats*, cudaStream_t);
INST(double)
INST(float)
#undef INST

}  // namespace ssids300
