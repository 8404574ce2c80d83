/*
 * ORACLE -- test infrastructure only.  Link-time shims that let the
 * reference's own C++ CPU numeric core (compiled from its sources into
 * oracle/_ref/ by oracle/Makefile) run without its Fortran parts:
 *   spral_c_{dgemm,dgemv,dtrsv,dtrsm,dsyrk,dpotrf,dsytrf}
 *       The reference implements these in Fortran
 *       (src/ssids/cpu/cpu_iface.f90:100-173) as thin calls into BLAS/LAPACK.
 *       Here they forward to an OpenBLAS found at run time: the library path
 *       comes from $SPRAL_REF_BLAS and the symbol prefix from
 *       $SPRAL_REF_BLAS_PREFIX (scipy bundles OpenBLAS with prefix "scipy_").
 *   spral_ssids_contrib_get_data / spral_ssids_contrib_free_dbl
 *       Fortran in the reference (src/ssids/contrib.f90:37,
 *       src/ssids/contrib_free.f90).  They are only reached when a subtree
 *       receives contribution blocks from other subtrees; the oracle always
 *       factors the whole tree as one subtree (ncontrib = 0), so they report
 *       an empty contribution.
 */
#include <dlfcn.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

static void* g_lib = NULL;
static const char* g_prefix = "";

static void* blas_sym(const char* name) {
  if (!g_lib) {
    const char* path = getenv("SPRAL_REF_BLAS");
    const char* pre = getenv("SPRAL_REF_BLAS_PREFIX");
    if (pre) g_prefix = pre;
    g_lib = dlopen(path ? path : "libopenblas.so", RTLD_NOW | RTLD_GLOBAL);
    if (!g_lib) { fprintf(stderr, "ref_shims: cannot load BLAS (%s)\n", dlerror()); abort(); }
    /* one BLAS thread: the reference runs BLAS inside OpenMP tasks */
    char nm[128];
    snprintf(nm, sizeof nm, "%sopenblas_set_num_threads", g_prefix);
    void (*setnt)(int) = (void (*)(int))dlsym(g_lib, nm);
    if (setnt) setnt(1);
  }
  char full[128];
  snprintf(full, sizeof full, "%s%s", g_prefix, name);
  void* f = dlsym(g_lib, full);
  if (!f) { fprintf(stderr, "ref_shims: missing %s\n", full); abort(); }
  return f;
}

typedef void (*gemm_t)(char*, char*, int*, int*, int*, double*, const double*, int*,
                       const double*, int*, double*, double*, int*, size_t, size_t);
typedef void (*gemv_t)(char*, int*, int*, const double*, const double*, int*, const double*,
                       int*, const double*, double*, int*, size_t);
typedef void (*trsv_t)(char*, char*, char*, int*, const double*, int*, double*, int*, size_t,
                       size_t, size_t);
typedef void (*trsm_t)(char*, char*, char*, char*, int*, int*, const double*, const double*,
                       int*, double*, int*, size_t, size_t, size_t, size_t);
typedef void (*syrk_t)(char*, char*, int*, int*, double*, const double*, int*, double*,
                       double*, int*, size_t, size_t);
typedef void (*potrf_t)(char*, int*, double*, int*, int*, size_t);
typedef void (*sytrf_t)(char*, int*, double*, int*, int*, double*, int*, int*, size_t);

void spral_c_dgemm(char* ta, char* tb, int* m, int* n, int* k, double* alpha, const double* a,
                   int* lda, const double* b, int* ldb, double* beta, double* c, int* ldc) {
  static gemm_t f = NULL;
  if (!f) f = (gemm_t)blas_sym("dgemm_");
  f(ta, tb, m, n, k, alpha, a, lda, b, ldb, beta, c, ldc, 1, 1);
}
void spral_c_dgemv(char* t, int* m, int* n, const double* alpha, const double* a, int* lda,
                   const double* x, int* incx, const double* beta, double* y, int* incy) {
  static gemv_t f = NULL;
  if (!f) f = (gemv_t)blas_sym("dgemv_");
  f(t, m, n, alpha, a, lda, x, incx, beta, y, incy, 1);
}
void spral_c_dtrsv(char* uplo, char* t, char* diag, int* n, const double* a, int* lda, double* x,
                   int* incx) {
  static trsv_t f = NULL;
  if (!f) f = (trsv_t)blas_sym("dtrsv_");
  f(uplo, t, diag, n, a, lda, x, incx, 1, 1, 1);
}
void spral_c_dtrsm(char* side, char* uplo, char* ta, char* diag, int* m, int* n,
                   const double* alpha, const double* a, int* lda, double* b, int* ldb) {
  static trsm_t f = NULL;
  if (!f) f = (trsm_t)blas_sym("dtrsm_");
  f(side, uplo, ta, diag, m, n, alpha, a, lda, b, ldb, 1, 1, 1, 1);
}
void spral_c_dsyrk(char* uplo, char* t, int* n, int* k, double* alpha, const double* a, int* lda,
                   double* beta, double* c, int* ldc) {
  static syrk_t f = NULL;
  if (!f) f = (syrk_t)blas_sym("dsyrk_");
  f(uplo, t, n, k, alpha, a, lda, beta, c, ldc, 1, 1);
}
void spral_c_dpotrf(char* uplo, int* n, double* a, int* lda, int* info) {
  static potrf_t f = NULL;
  if (!f) f = (potrf_t)blas_sym("dpotrf_");
  f(uplo, n, a, lda, info, 1);
}
void spral_c_dsytrf(char* uplo, int* n, double* a, int* lda, int* ipiv, double* work, int* lwork,
                    int* info) {
  static sytrf_t f = NULL;
  if (!f) f = (sytrf_t)blas_sym("dsytrf_");
  f(uplo, n, a, lda, ipiv, work, lwork, info, 1);
}

void spral_ssids_contrib_get_data(const void* contrib, int* n, const double** val, int* ldval,
                                  const int** rlist, int* ndelay, const int** delay_perm,
                                  const double** delay_val, int* lddelay) {
  (void)contrib;
  *n = 0; *val = NULL; *ldval = 0; *rlist = NULL;
  *ndelay = 0; *delay_perm = NULL; *delay_val = NULL; *lddelay = 0;
}
void spral_ssids_contrib_free_dbl(void* contrib) { (void)contrib; }
