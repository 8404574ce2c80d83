/*
 * ORACLE -- test infrastructure only.  CPU restatement of SSIDS's numeric
 * factorize-and-solve (indefinite LDL^T with a-posteriori threshold pivoting)
 * used to check the GPU path.  Nothing in the product links or calls this
 * file; only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline arm
 * load it.
 *
 * What it restates (reference paths relative to the SPRAL source tree):
 *   multifrontal driver      src/ssids/cpu/NumericSubtree.hxx:53-282
 *   assembly (A, delays,
 *     child contributions)   src/ssids/cpu/kernels/assemble.hxx:143-354,356-445
 *   node factor + stats      src/ssids/cpu/factor.hxx:38-136
 *   APP block pass           src/ssids/cpu/kernels/ldlt_app.cxx:1273-1472
 *     (block factor          src/ssids/cpu/kernels/block_ldlt.hxx:290-413,
 *      apply_pivot           ldlt_app.cxx:344-436,
 *      check_threshold       ldlt_app.cxx:316-336,
 *      Column::adjust        ldlt_app.cxx:112-130)
 *   TPP fallback             src/ssids/cpu/kernels/ldlt_tpp.cxx:166-270
 *   calcLD                   src/ssids/cpu/kernels/calc_ld.hxx:34-118
 *   solves                   src/ssids/cpu/NumericSubtree.hxx:284-400,
 *                            ldlt_app.cxx:2538-2589
 *   inertia count            src/ssids/cpu/NumericSubtree.hxx:249-280
 *   enquire_indef            src/ssids/cpu/NumericSubtree.hxx:402-445
 *
 * One deliberate difference in bookkeeping (not in the pivot tests): when
 * columns of a block fail the a-posteriori test they are restored, updated
 * with the block's passed pivots (as restore_if_required/update do) and then
 * swapped to the end of the APP range immediately, instead of being left in
 * place and compacted after the pass (ldlt_app.cxx:2374-2475).  Either way a
 * failed column gets no further APP attempt, is kept up to date by every later
 * pivot and is finally offered to TPP; the GPU path uses the same grouping, so
 * per-front elimination counts can be compared directly.
 *
 * Storage per front: L is m x n column-major with ld = m (m, n include
 * incoming delays), followed by D^{-1} in the reference's 2 x n format
 * (2x2 pivots marked by +Inf in d[2i+2]), perm holds 1-based pivot indices.
 */
#include <math.h>
#include <stdbool.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <dlfcn.h>

#define BLK 32

/* Same layout as struct cpu_factor_options (src/ssids/cpu/cpu_iface.hxx:27) */
typedef struct {
  int print_level;
  bool action;
  double small;
  double u;
  double multiplier;
  int64_t small_subtree_threshold;
  int cpu_block_size;
  int pivot_method;        /* 1 app_aggressive, 2 app_block, 3 tpp */
  int failed_pivot_method; /* 1 tpp, 2 pass */
} oracle_options;

/* Same layout as struct ThreadStats (src/ssids/cpu/ThreadStats.hxx:42) */
typedef struct {
  int flag;
  int num_delay;
  int64_t num_factor;
  int64_t num_flops;
  int num_neg;
  int num_two;
  int num_zero;
  int maxfront;
  int maxsupernode;
  int not_first_pass;
  int not_second_pass;
} oracle_stats;

typedef struct {
  int m, n;        /* including delays */
  int nrow, ncol;  /* symbolic */
  int ndelay_in, nelim, ndelay_out;
  double* l;       /* m*n + 2n */
  int* perm;       /* n, 1-based */
  double* contrib; /* (nrow-ncol)^2 */
  int first_child, next_child, parent;
  const int* rlist; /* 1-based, nrow entries */
} onode;

typedef struct {
  int n, nnodes;
  onode* nodes;
  oracle_stats stats;
} ofactors;

/* ---------------- optional BLAS dgemm (OpenBLAS found at run time) -------- */
typedef void (*dgemm_fn)(const char*, const char*, const int*, const int*, const int*,
                         const double*, const double*, const int*, const double*,
                         const int*, const double*, double*, const int*);
static dgemm_fn g_dgemm = NULL;
typedef void (*dtrsm_fn)(const char*, const char*, const char*, const char*, const int*,
                         const int*, const double*, const double*, const int*, double*,
                         const int*);
static dtrsm_fn g_dtrsm = NULL;

/* Load a Fortran-ABI dgemm from the shared library at `path` under symbol
 * `sym` (e.g. scipy's bundled OpenBLAS "scipy_dgemm_").  Returns 0 on
 * success.  Without it, the naive loops below are used. */
int oracle_set_blas(const char* path, const char* sym) {
  if (!path) { g_dgemm = NULL; g_dtrsm = NULL; return 0; }
  void* h = dlopen(path, RTLD_NOW | RTLD_GLOBAL);
  if (!h) return -1;
  void* f = dlsym(h, sym);
  if (!f) return -2;
  g_dgemm = (dgemm_fn)f;
  /* dtrsm under the same prefix (the solves, as ldlt_app_solve_* use it) */
  char tsym[128];
  size_t len = strlen(sym);
  g_dtrsm = NULL;
  if (len >= 6 && len < sizeof(tsym) && strcmp(sym + len - 6, "dgemm_") == 0) {
    memcpy(tsym, sym, len + 1);
    memcpy(tsym + len - 6, "dtrsm_", 6);
    g_dtrsm = (dtrsm_fn)dlsym(h, tsym);
  }
  return 0;
}

/* C(m x n, ldc) += alpha * A(m x k, lda) * B(n x k, ldb)^T ; lower_only: only
 * entries with row >= col (in C's own coordinates plus diag offset) */
static void gemm_nt(int m, int n, int k, double alpha, const double* a, int lda,
                    const double* b, int ldb, double* c, int ldc) {
  if (m <= 0 || n <= 0 || k <= 0) return;
  if (g_dgemm && (int64_t)m * n * k > 32768) {
    const double one = 1.0;
    g_dgemm("N", "T", &m, &n, &k, &alpha, a, &lda, b, &ldb, &one, c, &ldc);
    return;
  }
  for (int j = 0; j < n; ++j)
    for (int p = 0; p < k; ++p) {
      double bv = alpha * b[p * (int64_t)ldb + j];
      if (bv == 0.0) continue;
      const double* ac = a + p * (int64_t)lda;
      double* cc = c + j * (int64_t)ldc;
      for (int i = 0; i < m; ++i) cc[i] += ac[i] * bv;
    }
}

/* ---------------- helpers on a front (lower storage, ld = lda) ------------- */
static inline double* AT(double* a, int lda, int r, int c) { return &a[(int64_t)c * lda + r]; }

/* Symmetric swap of positions i<j in an m-row lower-stored front whose
 * columns 0..ncols-1 are stored (ldlt_tpp.cxx:50-77 swap_cols over the whole
 * front, including already-eliminated L rows to the left). */
static void sym_swap(int i, int j, int m, int ncols, double* a, int lda, int* perm) {
  if (i == j) return;
  if (j < i) { int t = i; i = j; j = t; }
  if (perm) { int t = perm[i]; perm[i] = perm[j]; perm[j] = t; }
  for (int c = 0; c < i; ++c) { double t = *AT(a, lda, i, c); *AT(a, lda, i, c) = *AT(a, lda, j, c); *AT(a, lda, j, c) = t; }
  for (int r = i + 1; r < j; ++r) { double t = *AT(a, lda, r, i); *AT(a, lda, r, i) = *AT(a, lda, j, r); *AT(a, lda, j, r) = t; }
  { double t = *AT(a, lda, i, i); *AT(a, lda, i, i) = *AT(a, lda, j, j); *AT(a, lda, j, j) = t; }
  if (j < ncols) {
    for (int r = j + 1; r < m; ++r) { double t = *AT(a, lda, r, i); *AT(a, lda, r, i) = *AT(a, lda, r, j); *AT(a, lda, r, j) = t; }
  } else {
    /* j beyond stored columns cannot happen for fully-summed swaps */
  }
}

/* LD = L * D for columns [c0, c0+k) of rows [r0, r1) (calc_ld.hxx:34-118) */
static void calc_ld(int r0, int r1, int k, const double* l, int ldl, const double* d,
                    double* ld, int ldld) {
  for (int c = 0; c < k;) {
    if (c + 1 == k || isfinite(d[2 * c + 2])) {
      double d11 = d[2 * c];
      if (d11 != 0.0) d11 = 1.0 / d11;
      for (int r = r0; r < r1; ++r) ld[(int64_t)c * ldld + r] = d11 * l[(int64_t)c * ldl + r];
      c += 1;
    } else {
      double d11 = d[2 * c], d21 = d[2 * c + 1], d22 = d[2 * c + 3];
      double det = d11 * d22 - d21 * d21;
      d11 /= det; d21 /= det; d22 /= det;
      for (int r = r0; r < r1; ++r) {
        double a1 = l[(int64_t)c * ldl + r], a2 = l[(int64_t)(c + 1) * ldl + r];
        ld[(int64_t)c * ldld + r] = d22 * a1 - d21 * a2;
        ld[(int64_t)(c + 1) * ldld + r] = -d21 * a1 + d11 * a2;
      }
      c += 2;
    }
  }
}

/* ------------- block_ldlt: complete pivoting inside one diagonal block ------
 * Operates on positions [p0, p0+bs) of the front; swaps act on whole rows and
 * columns of the front.  Only the diagonal block is updated.  Returns 0, or -1
 * for a singular block when action is false (block_ldlt.hxx:290-413). */
static int block_factor(int p0, int bs, int m, int ncols, double* a, int lda, double* d,
                        int* perm, bool action, double u, double small) {
  double work[2 * BLK];
  for (int p = 0; p < bs;) {
    /* find maxloc over uneliminated lower triangle of the block */
    double best = -1.0; int br = p, bc = p;
    for (int c = p; c < bs; ++c)
      for (int r = c; r < bs; ++r) {
        double v = fabs(*AT(a, lda, p0 + r, p0 + c));
        if (v > best) { best = v; br = r; bc = c; }
      }
    if (best < small) {
      if (!action) return -1;
      for (; p < bs; ++p) {
        d[2 * (p0 + p)] = 0.0; d[2 * (p0 + p) + 1] = 0.0;
        for (int r = p; r < bs; ++r) *AT(a, lda, p0 + r, p0 + p) = 0.0;
      }
      break;
    }
    int t = br, mm = bc, pivsiz;
    double a11, a21 = 0.0, a22 = 0.0, detscale = 0.0, detpiv = 0.0;
    if (t == mm) { a11 = *AT(a, lda, p0 + t, p0 + t); pivsiz = 1; }
    else {
      a11 = *AT(a, lda, p0 + mm, p0 + mm);
      a22 = *AT(a, lda, p0 + t, p0 + t);
      a21 = *AT(a, lda, p0 + t, p0 + mm);
      detscale = 1.0 / fabs(a21);
      detpiv = (a11 * detscale) * a22 - fabs(a21);
      if (fabs(detpiv) >= fabs(a21) / 2) pivsiz = 2;
      else if (fabs(a11) > fabs(a22)) { pivsiz = 1; t = mm; }
      else { pivsiz = 1; a11 = a22; mm = t; }
      (void)u;
    }
    if (pivsiz == 1) {
      double d11 = 1.0 / a11;
      sym_swap(p0 + p, p0 + t, m, ncols, a, lda, perm);
      for (int r = p + 1; r < bs; ++r) {
        work[r] = *AT(a, lda, p0 + r, p0 + p);
        *AT(a, lda, p0 + r, p0 + p) *= d11;
      }
      for (int c = p + 1; c < bs; ++c)
        for (int r = c; r < bs; ++r)
          *AT(a, lda, p0 + r, p0 + c) -= work[c] * *AT(a, lda, p0 + r, p0 + p);
      d[2 * (p0 + p)] = d11; d[2 * (p0 + p) + 1] = 0.0;
      *AT(a, lda, p0 + p, p0 + p) = 1.0;
      p += 1;
    } else {
      /* t > mm by construction (row index of the max below the diagonal) */
      sym_swap(p0 + p, p0 + mm, m, ncols, a, lda, perm);
      sym_swap(p0 + p + 1, p0 + t, m, ncols, a, lda, perm);
      double d11 = (a22 * detscale) / detpiv;
      double d22 = (a11 * detscale) / detpiv;
      double d21 = (-a21 * detscale) / detpiv;
      for (int r = p + 2; r < bs; ++r) {
        double w1 = *AT(a, lda, p0 + r, p0 + p), w2 = *AT(a, lda, p0 + r, p0 + p + 1);
        work[r] = w1; work[BLK + r] = w2;
        *AT(a, lda, p0 + r, p0 + p) = d11 * w1 + d21 * w2;
        *AT(a, lda, p0 + r, p0 + p + 1) = d21 * w1 + d22 * w2;
      }
      for (int c = p + 2; c < bs; ++c)
        for (int r = c; r < bs; ++r)
          *AT(a, lda, p0 + r, p0 + c) -= work[c] * *AT(a, lda, p0 + r, p0 + p) +
                                         work[BLK + c] * *AT(a, lda, p0 + r, p0 + p + 1);
      d[2 * (p0 + p)] = d11; d[2 * (p0 + p) + 1] = d21;
      d[2 * (p0 + p) + 2] = INFINITY; d[2 * (p0 + p) + 3] = d22;
      *AT(a, lda, p0 + p, p0 + p) = 1.0;
      *AT(a, lda, p0 + p + 1, p0 + p) = 0.0;
      *AT(a, lda, p0 + p + 1, p0 + p + 1) = 1.0;
      p += 2;
    }
  }
  return 0;
}

/* ------------- TPP (ldlt_tpp.cxx:166-270) on columns [c0, n) rows [c0, m) --- */
static bool col_small(int idx, int from, int to, const double* a, int lda, double small) {
  for (int c = from; c < idx; ++c) if (!(fabs(a[(int64_t)c * lda + idx]) < small)) return false;
  for (int r = idx; r < to; ++r) if (!(fabs(a[(int64_t)idx * lda + r]) < small)) return false;
  return true;
}
static double rc_absmax_excl(int col, int nel, int m, const double* a, int lda, int excl) {
  double best = 0.0;
  for (int c = nel; c < col; ++c) { if (c == excl) continue; double v = fabs(a[(int64_t)c * lda + col]); if (v > best) best = v; }
  for (int r = col + 1; r < m; ++r) { if (r == excl) continue; double v = fabs(a[(int64_t)col * lda + r]); if (v > best) best = v; }
  return best;
}
/* rank-1 / rank-2 trailing update of columns [c0, n) rows [c, m) */
static void tpp_update(int piv, int ps, int m, int n, double* a, int lda, const double* ld0, const double* ld1) {
  for (int c = piv + ps; c < n; ++c)
    for (int r = c; r < m; ++r) {
      double v = ld0[c] * a[(int64_t)piv * lda + r];
      if (ps == 2) v += ld1[c] * a[(int64_t)(piv + 1) * lda + r];
      a[(int64_t)c * lda + r] -= v;
    }
}
/* Returns number eliminated in [c0, n), or -1 on singular with !action. */
static int tpp_factor(int c0, int m, int n, double* a, int lda, double* d, int* perm,
                      bool action, double u, double small, double* ld0, double* ld1) {
  int nel = c0;
  while (nel < n) {
    if (col_small(nel, nel, m, a, lda, small)) {
      if (!action) return -1;
      for (int r = nel; r < m; ++r) a[(int64_t)nel * lda + r] = 0.0;
      d[2 * nel] = 0.0; d[2 * nel + 1] = 0.0;
      nel++;
      continue;
    }
    int p;
    for (p = nel + 1; p < n; ++p) {
      if (col_small(p, nel, m, a, lda, small)) {
        if (!action) return -1;
        sym_swap(p, nel, m, n, a, lda, perm);
        for (int r = nel; r < m; ++r) a[(int64_t)nel * lda + r] = 0.0;
        d[2 * nel] = 0.0; d[2 * nel + 1] = 0.0;
        nel++;
        break;
      }
      /* t: column of largest |a(p, nel:p-1)| */
      int t = nel; double bv = fabs(a[(int64_t)nel * lda + p]);
      for (int c = nel + 1; c < p; ++c) { double v = fabs(a[(int64_t)c * lda + p]); if (v > bv) { bv = v; t = c; } }
      double maxt = rc_absmax_excl(t, nel, m, a, lda, p);
      double maxp = rc_absmax_excl(p, nel, m, a, lda, t);
      /* 2x2 test (ldlt_tpp.cxx:84-112) */
      {
        double a11 = a[(int64_t)t * lda + t], a21 = a[(int64_t)t * lda + p], a22 = a[(int64_t)p * lda + p];
        double maxpiv = fmax(fabs(a11), fmax(fabs(a21), fabs(a22)));
        bool ok = false;
        double dd[4];
        if (!(maxpiv < small)) {
          double detscale = 1 / maxpiv;
          double det0 = (a11 * detscale) * a22, det1 = (a21 * detscale) * a21;
          double detpiv = det0 - det1;
          if (!(fabs(detpiv) < fmax(small, fmax(fabs(det0 / 2), fabs(det1 / 2))))) {
            dd[0] = (a22 * detscale) / detpiv; dd[1] = (-a21 * detscale) / detpiv;
            dd[2] = INFINITY; dd[3] = (a11 * detscale) / detpiv;
            if (fmax(maxp, maxt) < small) ok = true;
            else {
              double x1 = fabs(dd[0]) * maxt + fabs(dd[1]) * maxp;
              double x2 = fabs(dd[1]) * maxt + fabs(dd[3]) * maxp;
              ok = (u * fmax(x1, x2) < 1.0);
            }
          }
        }
        if (ok) {
          sym_swap(t, nel, m, n, a, lda, perm);
          sym_swap(p, nel + 1, m, n, a, lda, perm);
          memcpy(&d[2 * nel], dd, sizeof(dd));
          double* c1 = &a[(int64_t)nel * lda];
          double* c2 = &a[(int64_t)(nel + 1) * lda];
          c1[nel] = 1.0; c1[nel + 1] = 0.0; c2[nel + 1] = 1.0;
          for (int r = nel + 2; r < m; ++r) {
            ld0[r] = c1[r]; ld1[r] = c2[r];
            c1[r] = dd[0] * ld0[r] + dd[1] * ld1[r];
            c2[r] = dd[1] * ld0[r] + dd[3] * ld1[r];
          }
          tpp_update(nel, 2, m, n, a, lda, ld0, ld1);
          nel += 2;
          break;
        }
      }
      maxp = fmax(maxp, fabs(a[(int64_t)t * lda + p]));
      if (fabs(a[(int64_t)p * lda + p]) >= u * maxp) {
        sym_swap(p, nel, m, n, a, lda, perm);
        double* c1 = &a[(int64_t)nel * lda];
        d[2 * nel] = 1 / c1[nel]; d[2 * nel + 1] = 0.0;
        c1[nel] = 1.0;
        for (int r = nel + 1; r < m; ++r) { ld0[r] = c1[r]; c1[r] *= d[2 * nel]; }
        tpp_update(nel, 1, m, n, a, lda, ld0, ld1);
        nel += 1;
        break;
      }
    }
    if (p >= n) {
      p = nel;
      double maxp = rc_absmax_excl(p, nel, m, a, lda, -1);
      if (fabs(a[(int64_t)p * lda + p]) >= u * maxp) {
        double* c1 = &a[(int64_t)nel * lda];
        d[2 * nel] = 1 / c1[nel]; d[2 * nel + 1] = 0.0;
        c1[nel] = 1.0;
        for (int r = nel + 1; r < m; ++r) { ld0[r] = c1[r]; c1[r] *= d[2 * nel]; }
        tpp_update(nel, 1, m, n, a, lda, ld0, ld1);
        nel += 1;
      } else {
        break;
      }
    }
  }
  return nel - c0;
}

/* ------------- APP front factorization ------------------------------------
 * Returns nelim (>=0) or -1 (singular, action false). */
static int app_factor(int m, int n, double* a, int lda, double* d, int* perm,
                      bool action, double u, double small, double* bk, double* xw,
                      double* ldw, int* n_app_out) {
  int p = 0, end = n;
  while (p < end) {
    int bs = end - p < BLK ? end - p : BLK;
    /* backup the block column (rows p..m) before anything changes; swaps
       inside block_factor are applied to the backup afterwards by re-reading
       with the final order, so back up after the diag factor's swaps instead:
       we factor a copy of the diagonal block first to learn the swaps. */
    if (block_factor(p, bs, m, n, a, lda, d, perm, action, u, small) < 0) return -1;
    /* backup of the (permuted) original rows below, for restore */
    int rows = m - (p + bs);
    for (int j = 0; j < bs; ++j)
      memcpy(&bk[(int64_t)j * m], AT(a, lda, p + bs, p + j), sizeof(double) * (size_t)(rows > 0 ? rows : 0));
    /* apply pivot: X = A21 L11^{-T}; L21 = X D^{-1} (ldlt_app.cxx:344-384) */
    for (int j = 0; j < bs; ++j) {
      double* xj = AT(a, lda, p + bs, p + j);
      for (int k = 0; k < j; ++k) {
        double lkj = *AT(a, lda, p + j, p + k);
        if (lkj == 0.0) continue;
        const double* xk = &xw[(int64_t)k * m];
        for (int r = 0; r < rows; ++r) xj[r] -= xk[r] * lkj;
      }
      memcpy(&xw[(int64_t)j * m], xj, sizeof(double) * (size_t)(rows > 0 ? rows : 0));
    }
    for (int j = 0; j < bs;) {
      double* dj = &d[2 * (p + j)];
      if (j + 1 == bs || isfinite(dj[2])) {
        double d11 = dj[0];
        double* col = AT(a, lda, p + bs, p + j);
        if (d11 == 0.0) {
          for (int r = 0; r < rows; ++r) { double v = col[r]; col[r] = (fabs(v) < small) ? 0.0 : INFINITY * v; }
          for (int r = 0; r < rows; ++r) xw[(int64_t)j * m + r] = 0.0;
        } else {
          for (int r = 0; r < rows; ++r) col[r] *= d11;
        }
        j += 1;
      } else {
        double d11 = dj[0], d21 = dj[1], d22 = dj[3];
        double* c1 = AT(a, lda, p + bs, p + j);
        double* c2 = AT(a, lda, p + bs, p + j + 1);
        for (int r = 0; r < rows; ++r) {
          double a1 = c1[r], a2 = c2[r];
          c1[r] = d11 * a1 + d21 * a2;
          c2[r] = d21 * a1 + d22 * a2;
        }
        j += 2;
      }
    }
    /* a posteriori threshold test: first failing column over all rows */
    int npass = bs;
    for (int j = 0; j < npass; ++j) {
      const double* col = AT(a, lda, p + bs, p + j);
      for (int r = 0; r < rows; ++r)
        if (fabs(col[r]) > 1.0 / u) { npass = j; break; }
    }
    /* Column::adjust: do not split a 2x2 pivot */
    if (npass > 0 && npass < bs) {
      double d11 = d[2 * (p + npass - 1)], d21 = d[2 * (p + npass - 1) + 1];
      if (isfinite(d11) && d21 != 0.0) npass--;
    }
    int f = bs - npass;
    if (f > 0) {
      /* restore failed columns and update them with the passed pivots only */
      /* rows below: A21_fail = backup - X_pass * L11[fail, pass]^T */
      for (int j = npass; j < bs; ++j) {
        double* col = AT(a, lda, p + bs, p + j);
        memcpy(col, &bk[(int64_t)j * m], sizeof(double) * (size_t)(rows > 0 ? rows : 0));
        for (int k = 0; k < npass; ++k) {
          double lkj = *AT(a, lda, p + j, p + k);
          if (lkj == 0.0) continue;
          for (int r = 0; r < rows; ++r) col[r] -= xw[(int64_t)k * m + r] * lkj;
        }
      }
      /* diagonal block failed part: S = L_ff D_f L_ff^T where the whole block
         was factorised (restoring from A11 and removing the passed pivots'
         contribution gives the same matrix) */
      {
        double lff[BLK * BLK];
        double ldff[BLK * BLK];
        for (int j = 0; j < f; ++j)
          for (int i = 0; i < f; ++i)
            lff[j * BLK + i] = (i >= j) ? *AT(a, lda, p + npass + i, p + npass + j) : 0.0;
        for (int i = 0; i < f; ++i) lff[i * BLK + i] = 1.0;
        calc_ld(0, f, f, lff, BLK, &d[2 * (p + npass)], ldff, BLK);
        for (int j = 0; j < f; ++j)
          for (int i = j; i < f; ++i) {
            double s = 0.0;
            for (int k = 0; k < f; ++k) s += lff[k * BLK + i] * ldff[k * BLK + j];
            *AT(a, lda, p + npass + i, p + npass + j) = s;
          }
      }
    }
    /* trailing update of fully-summed columns [p+bs, n) with passed pivots */
    if (npass > 0 && p + bs < n) {
      int rr = m - (p + bs);
      calc_ld(0, rr, npass, AT(a, lda, p + bs, p), lda, &d[2 * p], ldw, m);
      /* blocked: columns [cb, cb+nb) rows [cb, m); entries above the
         diagonal inside a block are scratch in lower storage */
      for (int cb = p + bs; cb < n; cb += 128) {
        int nb = n - cb < 128 ? n - cb : 128;
        gemm_nt(m - cb, nb, npass, -1.0, AT(a, lda, cb, p), lda,
                &ldw[cb - (p + bs)], m, AT(a, lda, cb, cb), lda);
      }
    }
    /* move failed columns to the end of the APP range */
    if (f > 0) {
      int fs = p + npass, ts = end - f;
      int nf = 0, tf[BLK], tt[BLK];
      for (int i = fs; i < fs + f; ++i) if (i < ts) tf[nf++] = i;
      int nt = 0;
      for (int i = ts; i < end; ++i) if (i >= fs + f) tt[nt++] = i;
      for (int k = 0; k < nf && k < nt; ++k) {
        sym_swap(tf[k], tt[k], m, n, a, lda, perm);
        /* D entries are only meaningful for eliminated columns */
      }
      end -= f;
    }
    p += npass;
  }
  *n_app_out = p;
  return p;
}

static void free_factors(ofactors* F) {
  if (!F) return;
  if (F->nodes) {
    for (int i = 0; i < F->nnodes; ++i) { free(F->nodes[i].l); free(F->nodes[i].perm); free(F->nodes[i].contrib); }
    free(F->nodes);
  }
  free(F);
}

/* Factorize.  Inputs as for spral_ssids_cpu_create_symbolic_subtree /
 * create_num_subtree (1-based arrays, src/ssids/cpu/SymbolicSubtree.hxx:20):
 * the whole tree (sa=1, en=nnodes+1).  Returns a handle; stats filled. */
void* oracle_factor(int n, int nnodes, const int* sptr, const int* sparent, const int64_t* rptr,
                    const int* rlist, const int64_t* nptr, const int64_t* nlist, const double* aval,
                    const oracle_options* opt, oracle_stats* stats) {
  memset(stats, 0, sizeof(*stats));
  ofactors* F = (ofactors*)calloc(1, sizeof(ofactors));
  F->n = n;
  F->nnodes = nnodes;
  F->nodes = (onode*)calloc((size_t)nnodes + 1, sizeof(onode));
  for (int i = 0; i <= nnodes; ++i) F->nodes[i].first_child = -1;
  for (int i = 0; i < nnodes; ++i) {
    onode* nd = &F->nodes[i];
    nd->nrow = (int)(rptr[i + 1] - rptr[i]);
    nd->ncol = sptr[i + 1] - sptr[i];
    nd->rlist = &rlist[rptr[i] - 1];
    nd->parent = sparent[i] - 1;
  }
  /* child lists built as SymbolicSubtree.hxx:42-47 builds them (each node
   * is pushed onto its parent's list in increasing order), so children come
   * off in decreasing order: delayed columns are appended, and contributions
   * added, last child first */
  for (int i = 0; i < nnodes; ++i) {
    int par = F->nodes[i].parent;
    if (par > nnodes) par = nnodes;
    F->nodes[i].next_child = F->nodes[par].first_child;
    F->nodes[par].first_child = i;
  }
  /* Small leaf subtrees (SymbolicSubtree.hxx:56-82): subtrees below
   * small_subtree_threshold flops are factored node by node with TPP only
   * (SmallLeafNumericSubtree.hxx:345-375, ldlt_tpp_factor from column 0). */
  char* insl = (char*)calloc((size_t)nnodes + 1, 1);
  {
    int64_t* fl = (int64_t*)calloc((size_t)nnodes + 1, sizeof(int64_t));
    for (int ni = 0; ni < nnodes; ++ni) {
      const int64_t nr = F->nodes[ni].nrow;
      for (int k = 0; k < F->nodes[ni].ncol; ++k) fl[ni] += (nr - k) * (nr - k);
      int par = F->nodes[ni].parent;
      if (par > nnodes || par < 0) par = nnodes;
      fl[par] += fl[ni];
    }
    for (int ni = 0; ni < nnodes;) {
      if (F->nodes[ni].first_child != -1) { ++ni; continue; }
      int last = ni;
      for (int cur = ni; cur < nnodes;) {
        if (fl[cur] >= opt->small_subtree_threshold) break;
        last = cur;
        int par = F->nodes[cur].parent;
        cur = (par > nnodes || par < 0) ? nnodes : par;
      }
      if (last == ni) { ++ni; continue; }
      for (int i = ni; i <= last; ++i) insl[i] = 1;
      ni = last + 1;
    }
    free(fl);
  }
  int* map = (int*)malloc(sizeof(int) * ((size_t)n + 1));
  int maxm = 1;
  for (int i = 0; i < nnodes; ++i) if (F->nodes[i].nrow > maxm) maxm = F->nodes[i].nrow;
  /* delays can grow fronts; size scratch lazily */
  size_t scratch = 0;
  double *bk = NULL, *xw = NULL, *ldw = NULL;

  for (int ni = 0; ni < nnodes; ++ni) {
    onode* nd = &F->nodes[ni];
    int ndin = 0;
    for (int c = nd->first_child; c != -1; c = F->nodes[c].next_child) ndin += F->nodes[c].ndelay_out;
    nd->ndelay_in = ndin;
    int m = nd->nrow + ndin, nn = nd->ncol + ndin;
    nd->m = m; nd->n = nn;
    int cm = nd->nrow - nd->ncol;
    nd->l = (double*)calloc((size_t)m * nn + 2 * (size_t)nn + 1, sizeof(double));
    nd->perm = (int*)malloc(sizeof(int) * ((size_t)nn + 1));
    nd->contrib = cm > 0 ? (double*)calloc((size_t)cm * cm, sizeof(double)) : NULL;
    double* L = nd->l;
    int ld = m;
    for (int i = 0; i < nd->ncol; ++i) nd->perm[i] = nd->rlist[i];
    /* add A (assemble.hxx:46-75) */
    for (int64_t k = nptr[ni] - 1; k < nptr[ni + 1] - 1; ++k) {
      int64_t src = nlist[2 * k] - 1, dest = nlist[2 * k + 1] - 1;
      int c = (int)(dest / nd->nrow), r = (int)(dest % nd->nrow);
      if (r >= nd->ncol) r += ndin;
      L[(int64_t)c * ld + r] = aval[src];
    }
    /* map rows of this node (assemble.hxx:230-236) */
    for (int i = 0; i < nd->ncol; ++i) map[nd->rlist[i]] = i;
    for (int i = nd->ncol; i < nd->nrow; ++i) map[nd->rlist[i]] = i + ndin;
    int delay_col = nd->ncol;
    for (int c = nd->first_child; c != -1; c = F->nodes[c].next_child) {
      onode* ch = &F->nodes[c];
      /* delayed columns go to the back of the fully-summed block */
      for (int i = 0; i < ch->ndelay_out; ++i) {
        double* src = &ch->l[(int64_t)(ch->nelim + i) * ch->m + ch->nelim + i];
        double* dst = &L[(int64_t)delay_col * ld + delay_col];
        nd->perm[delay_col] = ch->perm[ch->nelim + i];
        for (int j = 0; j < ch->ndelay_out - i; ++j) dst[j] = src[j];
        const double* s2 = &ch->l[(int64_t)(ch->nelim + i) * ch->m + ch->ndelay_in];
        for (int j = ch->ncol; j < ch->nrow; ++j) {
          int r = map[ch->rlist[j]];
          if (r < nn) L[(int64_t)r * ld + delay_col] = s2[j];
          else L[(int64_t)delay_col * ld + r] = s2[j];
        }
        delay_col++;
      }
      /* expected contributions: into L (fully-summed) or contrib */
      int ccm = ch->nrow - ch->ncol;
      if (ch->contrib) {
        for (int jj = 0; jj < ccm; ++jj) {
          int cpos = map[ch->rlist[ch->ncol + jj]];
          const double* src = &ch->contrib[(int64_t)jj * ccm];
          for (int ii = jj; ii < ccm; ++ii) {
            int rpos = map[ch->rlist[ch->ncol + ii]];
            if (cpos < nn) L[(int64_t)cpos * ld + rpos] += src[ii];
            else nd->contrib[(int64_t)(cpos - nn) * cm + (rpos - nn)] += src[ii];
          }
        }
        free(ch->contrib);
        ch->contrib = NULL;
      }
    }
    /* factor (factor.hxx:38-136) */
    double* D = &L[(int64_t)nn * ld];
    size_t need = (size_t)m * BLK;
    if (need > scratch) {
      free(bk); free(xw); free(ldw);
      scratch = need;
      bk = (double*)malloc(sizeof(double) * scratch);
      xw = (double*)malloc(sizeof(double) * scratch);
      ldw = (double*)malloc(sizeof(double) * scratch);
    }
    int nelim = 0, napp = 0;
    if (insl[ni]) {
      double* l0 = (double*)malloc(sizeof(double) * (size_t)m);
      double* l1 = (double*)malloc(sizeof(double) * (size_t)m);
      int got = tpp_factor(0, m, nn, L, ld, D, nd->perm, opt->action, opt->u, opt->small, l0, l1);
      free(l0); free(l1);
      if (got < 0) { stats->flag = -5; break; }
      nelim = got;
    } else if (opt->pivot_method != 3) {
      nelim = app_factor(m, nn, L, ld, D, nd->perm, opt->action, opt->u, opt->small, bk, xw, ldw, &napp);
      if (nelim < 0) { stats->flag = -5; break; }
    }
    if (nelim < nn && !insl[ni]) {
      if (opt->pivot_method != 3) stats->not_first_pass += nn - nelim;
      if (m == nn || opt->pivot_method == 3 || opt->failed_pivot_method == 1) {
        double* l0 = (double*)malloc(sizeof(double) * (size_t)m);
        double* l1 = (double*)malloc(sizeof(double) * (size_t)m);
        int got = tpp_factor(nelim, m, nn, L, ld, D, nd->perm, opt->action, opt->u, opt->small, l0, l1);
        free(l0); free(l1);
        if (got < 0) { stats->flag = -5; break; }
        nelim += got;
        if (opt->pivot_method == 3) stats->not_first_pass += nn - nelim;
        else stats->not_second_pass += nn - nelim;
      }
    }
    nd->nelim = nelim;
    nd->ndelay_out = nn - nelim;
    /* contribution: C -= L_cb D L_cb^T over all eliminated columns */
    if (cm > 0 && nelim > 0) {
      double* ldc = (double*)malloc(sizeof(double) * (size_t)cm * nelim);
      calc_ld(0, cm, nelim, &L[nn], ld, D, ldc, cm);
      /* lower triangle only, column by column */
      for (int jb = 0; jb < cm; jb += 128) {
        int nb = cm - jb < 128 ? cm - jb : 128;
        gemm_nt(cm - jb, nb, nelim, -1.0, &L[nn + jb], ld, &ldc[jb], cm,
                &nd->contrib[(int64_t)jb * cm + jb], cm);
      }
      free(ldc);
    }
    stats->num_delay += nd->ndelay_out;
    for (int64_t j = m; j >= m - nelim + 1; --j) { stats->num_factor += j; stats->num_flops += j * j; }
    if (m > stats->maxfront) stats->maxfront = m;
    if (nn > stats->maxsupernode) stats->maxsupernode = nn;
  }
  free(map); free(bk); free(xw); free(ldw); free(insl);
  if (stats->flag < 0) { F->stats = *stats; return F; }
  /* inertia (NumericSubtree.hxx:249-280) */
  for (int ni = 0; ni < nnodes; ++ni) {
    onode* nd = &F->nodes[ni];
    const double* d = &nd->l[(int64_t)nd->n * nd->m];
    for (int i = 0; i < nd->nelim;) {
      double a11 = d[2 * i], a21 = d[2 * i + 1];
      if (i + 1 == nd->nelim || isfinite(d[2 * i + 2])) {
        if (a11 == 0.0) { stats->flag = 7; stats->num_zero++; }
        if (a11 < 0.0) stats->num_neg++;
        i++;
      } else {
        double a22 = d[2 * i + 3];
        stats->num_two++;
        double det = a11 * a22 - a21 * a21, tr = a11 + a22;
        if (det < 0) stats->num_neg++;
        else if (tr < 0) stats->num_neg += 2;
        i += 2;
      }
    }
  }
  F->stats = *stats;
  return F;
}

void oracle_free(void* h) { free_factors((ofactors*)h); }

/* per node: m, n, nelim, ndelay_in */
void oracle_node_info(void* h, int node, int* info) {
  ofactors* F = (ofactors*)h;
  onode* nd = &F->nodes[node];
  info[0] = nd->m; info[1] = nd->n; info[2] = nd->nelim; info[3] = nd->ndelay_in;
}

/* copy one front: L (m x n, ld m), D (2n), perm (n, 0-based) */
void oracle_node_data(void* h, int node, double* L, double* D, int* perm) {
  ofactors* F = (ofactors*)h;
  onode* nd = &F->nodes[node];
  if (L) memcpy(L, nd->l, sizeof(double) * (size_t)nd->m * nd->n);
  if (D) memcpy(D, &nd->l[(int64_t)nd->n * nd->m], sizeof(double) * 2 * (size_t)nd->n);
  if (perm) for (int i = 0; i < nd->n; ++i) perm[i] = nd->perm[i] - 1;
}

/* Solve in pivot order (x already permuted by invp), nrhs columns, ldx.
 * job: 0 full, 1 fwd, 2 diag, 3 bwd (no D), 4 diag_bwd
 * (NumericSubtree.hxx:284-400; ldlt_app.cxx:2538-2589: per node, all
 * right-hand sides at once; with BLAS loaded, dtrsm for the triangle and
 * dgemm for the rectangle, as ldlt_app_solve_fwd/bwd do). */
int oracle_solve(void* h, int job, int nrhs, double* x, int ldx) {
  ofactors* F = (ofactors*)h;
  int n = F->n;
  int maxm = 1;
  for (int ni = 0; ni < F->nnodes; ++ni) if (F->nodes[ni].m > maxm) maxm = F->nodes[ni].m;
  double* xl = (double*)malloc(sizeof(double) * (size_t)maxm * (nrhs > 0 ? nrhs : 1));
  int* map = (int*)malloc(sizeof(int) * (size_t)(n > 0 ? n : 1));
  bool fwd = (job == 0 || job == 1);
  bool diag = (job == 0 || job == 2 || job == 4);
  bool bwd = (job == 0 || job == 3 || job == 4);
  const double one = 1.0, mone = -1.0;
  if (fwd) {
    for (int ni = 0; ni < F->nnodes; ++ni) {
      onode* nd = &F->nodes[ni];
      int m = nd->m, nn = nd->n, ne = nd->nelim;
      for (int i = 0; i < nn; ++i) map[i] = nd->perm[i];
      for (int i = nd->ncol; i < nd->nrow; ++i) map[i + nd->ndelay_in] = nd->rlist[i];
      for (int r = 0; r < nrhs; ++r)
        for (int i = 0; i < m; ++i) xl[(size_t)r * m + i] = x[(size_t)r * ldx + map[i] - 1];
      const double* L = nd->l;
      if (ne > 0) {
        if (g_dtrsm && g_dgemm) {
          g_dtrsm("L", "L", "N", "U", &ne, &nrhs, &one, L, &m, xl, &m);
          int rows = m - ne;
          if (rows > 0)
            g_dgemm("N", "N", &rows, &nrhs, &ne, &mone, L + ne, &m, xl, &m, &one, xl + ne, &m);
        } else {
          for (int r = 0; r < nrhs; ++r) {
            double* xr = xl + (size_t)r * m;
            for (int j = 0; j < ne; ++j) {
              double v = xr[j];
              for (int i = j + 1; i < m; ++i) xr[i] -= L[(int64_t)j * m + i] * v;
            }
          }
        }
      }
      for (int r = 0; r < nrhs; ++r)
        for (int i = 0; i < m; ++i) x[(size_t)r * ldx + map[i] - 1] = xl[(size_t)r * m + i];
    }
  }
  if (diag || bwd) {
    for (int ni = F->nnodes - 1; ni >= 0; --ni) {
      onode* nd = &F->nodes[ni];
      int m = nd->m, nn = nd->n, ne = nd->nelim;
      for (int i = 0; i < nn; ++i) map[i] = nd->perm[i];
      for (int i = nd->ncol; i < nd->nrow; ++i) map[i + nd->ndelay_in] = nd->rlist[i];
      int blkm = bwd ? m : ne;
      for (int r = 0; r < nrhs; ++r)
        for (int i = 0; i < blkm; ++i) xl[(size_t)r * m + i] = x[(size_t)r * ldx + map[i] - 1];
      const double* L = nd->l;
      const double* d = &L[(int64_t)nn * m];
      if (diag) {
        for (int r = 0; r < nrhs; ++r) {
          double* xr = xl + (size_t)r * m;
          for (int i = 0; i < ne;) {
            if (i + 1 == ne || isfinite(d[2 * i + 2])) { xr[i] *= d[2 * i]; i++; }
            else {
              double x1 = xr[i], x2 = xr[i + 1];
              xr[i] = d[2 * i] * x1 + d[2 * i + 1] * x2;
              xr[i + 1] = d[2 * i + 1] * x1 + d[2 * i + 3] * x2;
              i += 2;
            }
          }
        }
      }
      if (bwd && ne > 0) {
        if (g_dtrsm && g_dgemm) {
          int rows = m - ne;
          if (rows > 0)
            g_dgemm("T", "N", &ne, &nrhs, &rows, &mone, L + ne, &m, xl + ne, &m, &one, xl, &m);
          g_dtrsm("L", "L", "T", "U", &ne, &nrhs, &one, L, &m, xl, &m);
        } else {
          for (int r = 0; r < nrhs; ++r) {
            double* xr = xl + (size_t)r * m;
            for (int j = ne - 1; j >= 0; --j) {
              double sacc = xr[j];
              for (int i = j + 1; i < m; ++i) sacc -= L[(int64_t)j * m + i] * xr[i];
              xr[j] = sacc;
            }
          }
        }
      }
      for (int r = 0; r < nrhs; ++r)
        for (int i = 0; i < ne; ++i) x[(size_t)r * ldx + map[i] - 1] = xl[(size_t)r * m + i];
    }
  }
  free(xl); free(map);
  return 0;
}

/* enquire_indef (NumericSubtree.hxx:402-445): piv_order (0-based variable in
 * pivot order, negative for 2x2) and d (2 x n) */
void oracle_enquire(void* h, int* piv_order, double* dout) {
  ofactors* F = (ofactors*)h;
  int piv = 0;
  for (int ni = 0; ni < F->nnodes; ++ni) {
    onode* nd = &F->nodes[ni];
    const double* d = &nd->l[(int64_t)nd->n * nd->m];
    for (int i = 0; i < nd->nelim;) {
      if (i + 1 == nd->nelim || isfinite(d[2 * i + 2])) {
        if (piv_order) piv_order[nd->perm[i] - 1] = piv++;
        if (dout) { *dout++ = d[2 * i]; *dout++ = 0.0; }
        i += 1;
      } else {
        if (piv_order) { piv_order[nd->perm[i] - 1] = -(piv++); piv_order[nd->perm[i + 1] - 1] = -(piv++); }
        if (dout) { *dout++ = d[2 * i]; *dout++ = d[2 * i + 1]; *dout++ = d[2 * i + 3]; *dout++ = 0.0; }
        i += 2;
      }
    }
  }
}
