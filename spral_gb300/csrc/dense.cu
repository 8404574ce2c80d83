// Dense LDL^T of one front with a-posteriori threshold pivoting, as a
// stand-alone entry point (the GPU counterpart of ldlt_app_factor,
// src/ssids/cpu/kernels/ldlt_app.cxx:2506, and of the GPU path's
// node_ldlt, src/ssids/gpu/dense_factor.f90:28).  It runs the same APP step
// kernels, TPP fallback and contribution update as the tree factorization,
// on one front held by the caller in device memory.
#include <algorithm>
#include <cstdio>

#include "spral_ssids_gpu.h"
#include "ssids_gpu.cuh"

namespace ssids300 {

namespace {

__global__ void k_iota(int* v, int n) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) v[i] = i;
}

__global__ void k_zero_upd(double* upd, int ldupd, int cm) {
  const int64_t tot = (int64_t)cm * cm;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < tot;
       e += (int64_t)gridDim.x * blockDim.x)
    upd[(e / cm) * ldupd + e % cm] = 0.0;
}

inline int cdiv(int a, int b) { return (a + b - 1) / b; }

}  // namespace

// Workspace carve-up for one front (sizes in bytes, 256-aligned pieces).
struct DenseWorkspace {
  FrontDesc<double>* desc;
  FrontState* state;
  int* front0;
  int* opos;
  int* lperm;
  double* step;
  double* W;
  double* swapbuf;
  double* LD;
};

static size_t align256(size_t b) { return (b + 255) & ~size_t(255); }

size_t dense_workspace_bytes(int m, int n, int lda) {
  const int cm = m - n;
  return align256(sizeof(FrontDesc<double>)) + align256(sizeof(FrontState)) + align256(sizeof(int)) +
         align256(sizeof(int) * (size_t)std::max(n, 1)) + align256(sizeof(int) * kBlk) +
         align256(sizeof(double) * (kBlk * kBlk + 2 * kBlk + 64)) +
         align256(sizeof(double) * (size_t)lda * kBlk) +
         align256(sizeof(double) * ((size_t)lda * 64 + 256)) +
         align256(sizeof(double) * (size_t)std::max(cm, 0) * std::max(n, 1));
}

DenseWorkspace dense_workspace_carve(void* base, int m, int n, int lda) {
  char* p = static_cast<char*>(base);
  DenseWorkspace w;
  const int cm = m - n;
  auto take = [&](size_t b) { char* r = p; p += align256(b); return r; };
  w.desc = (FrontDesc<double>*)take(sizeof(FrontDesc<double>));
  w.state = (FrontState*)take(sizeof(FrontState));
  w.front0 = (int*)take(sizeof(int));
  w.opos = (int*)take(sizeof(int) * (size_t)std::max(n, 1));
  w.lperm = (int*)take(sizeof(int) * kBlk);
  w.step = (double*)take(sizeof(double) * (kBlk * kBlk + 2 * kBlk + 64));
  w.W = (double*)take(sizeof(double) * (size_t)lda * kBlk);
  w.swapbuf = (double*)take(sizeof(double) * ((size_t)lda * 64 + 256));
  w.LD = (double*)take(sizeof(double) * (size_t)std::max(cm, 0) * std::max(n, 1));
  return w;
}

// Enqueue the factorization of one front on stream s using workspace w and
// return nelim (after a synchronisation) or a negative SSIDS flag.
int dense_factor_run(const DenseWorkspace& w, int m, int n, int* perm, double* a, int lda,
                     double* d, double beta, double* upd, int ldupd,
                     const spral_ssids_cpu_factor_options& co, cudaStream_t s) {
  FrontDesc<double> h{};
  h.L = a;
  h.D = d;
  h.perm = perm;
  h.opos = w.opos;
  h.C = (m > n) ? upd : nullptr;
  h.W = w.W;
  h.step = w.step;
  h.lperm = w.lperm;
  h.swapbuf = w.swapbuf;
  h.LD = w.LD;
  h.m = m; h.n = n; h.ld = lda;
  h.nrow = m; h.ncol = n; h.ndelay_in = 0; h.cm = m - n;
  h.node = 0;
  h.ldc = ldupd;
  const int zero = 0;
  if (cudaMemcpyAsync(w.desc, &h, sizeof(h), cudaMemcpyHostToDevice, s) != cudaSuccess) return -51;
  if (cudaMemcpyAsync(w.front0, &zero, sizeof(int), cudaMemcpyHostToDevice, s) != cudaSuccess) return -51;
  if (cudaMemsetAsync(w.state, 0, sizeof(FrontState), s) != cudaSuccess) return -51;
  k_iota<<<std::max(1, std::min(cdiv(n, 256), 64)), 256, 0, s>>>(w.opos, n);
  note_launches(1);
  if (m > n && upd && beta == 0.0) {
    k_zero_upd<<<std::max(1, std::min(cdiv((m - n) * (m - n), 256), 1024)), 256, 0, s>>>(upd, ldupd, m - n);
    note_launches(1);
  }
  const bool use_app = co.pivot_method != 3;
  if (use_app) {
    const int steps = cdiv(n, kBlk);
    for (int st = 0; st < steps; ++st)
      launch_app_step<double>(w.desc, w.state, w.front0, 1, st, std::max(m - kBlk * st, 1),
                              m - kBlk * (st + 1), n - kBlk * (st + 1), co.action, co.u,
                              co.small, s, nullptr);
  }
  launch_app_finish<double>(w.desc, w.state, w.front0, 1, s);
  const bool tpp_all = (co.pivot_method == 3) || (co.failed_pivot_method == 1);
  launch_tpp<double>(w.desc, w.state, w.front0, 1, co.action, co.u, co.small, tpp_all, s);
  if (m > n && upd) {
    launch_calc_ld<double>(w.desc, w.state, w.front0, 1, m - n, n, s);
    launch_contrib_gemm<double>(w.desc, w.state, w.front0, 1, m - n, s);
  }
  FrontState hs{};
  if (cudaMemcpyAsync(&hs, w.state, sizeof(FrontState), cudaMemcpyDeviceToHost, s) != cudaSuccess)
    return -51;
  if (cudaStreamSynchronize(s) != cudaSuccess) return -51;
  if (hs.status == kDevSingular) return -5;
  if (hs.status != kDevOk) return -51;
  return hs.nelim;
}

}  // namespace ssids300

using namespace ssids300;

extern "C" {

int spral_ssids_gpu_ldlt_app_factor(int m, int n, int* perm_dev, double* a_dev, int lda,
                                    double* d_dev, double beta, double* upd_dev, int ldupd,
                                    const struct spral_ssids_cpu_factor_options* options,
                                    void* stream) {
  if (m < n || n < 0) return -1;
  if (lda < m) return -4;
  if (m > n && upd_dev && ldupd < m - n) return -9;
  if (n == 0) return 0;
  spral_ssids_cpu_factor_options co{};
  co.action = true; co.small = 1e-20; co.u = 0.01; co.pivot_method = 2; co.failed_pivot_method = 1;
  if (options) co = *options;
  cudaStream_t s = (cudaStream_t)stream;
  void* base = nullptr;
  const size_t bytes = dense_workspace_bytes(m, n, lda);
  if (cudaMalloc(&base, bytes) != cudaSuccess) {
    cudaGetLastError();
    return -50;
  }
  DenseWorkspace w = dense_workspace_carve(base, m, n, lda);
  int r = dense_factor_run(w, m, n, perm_dev, a_dev, lda, d_dev, beta, upd_dev, ldupd, co, s);
  cudaFree(base);
  return r;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Variant of spral_ssids_gpu_ldlt_app_factor that allocates nothing.
//
// Some callers cannot call cudaMalloc at the point where they factor a
// front: their device memory may belong to another allocator (a framework's
// caching pool that has reserved most of the GPU), their memory budget may be
// fixed when the library is loaded, or they sit on a latency-critical path
// where cudaMalloc/cudaFree can stall the whole device.  For them the
// workspace lives in one fixed device array that is part of this library's
// image: every GPU that loads the library holds it until the process exits.
// ---------------------------------------------------------------------------
#include <mutex>

namespace {

// Largest leading dimension (hence front height m) the fixed scratch serves.
constexpr int kNoAllocMaxLda = 1024;
// Workspace of the largest front: desc/state/index pieces, opos, step
// buffers, W (lda x 32), column-move buffer (64 x lda) and L*D for the
// contribution rows ((m-n) x n, largest at n = m/2).  3 MiB holds it.
constexpr size_t kNoAllocScratchBytes = size_t(3) << 20;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

constexpr int kNoAllocMaxDevices = 64;
std::mutex g_noalloc_mutex;
void* g_noalloc_addr[kNoAllocMaxDevices] = {nullptr};

// Device address of the scratch array on the current device.  The host-side
// symbol g_noalloc_scratch is only a stand-in and must never reach a kernel;
// the address is looked up once per device, with that device current, and
// kept for the life of the process.  cudaDeviceReset (or anything else that
// destroys the device's primary context) unloads the module, after which the
// array may come back at another address: a process that resets a device
// must not call this entry point on it again.
int noalloc_scratch_address(void** out) {
  int dev = -1;
  if (cudaGetDevice(&dev) != cudaSuccess) { cudaGetLastError(); return -51; }
  if (dev < 0 || dev >= kNoAllocMaxDevices) return -51;
  std::lock_guard<std::mutex> lock(g_noalloc_mutex);
  if (!g_noalloc_addr[dev]) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || p == nullptr) {
      cudaGetLastError();
      fprintf(stderr, "spral_gb300: cannot locate the fixed factorization scratch on device %d: %s\n",
              dev, cudaGetErrorString(e));
      return -51;
    }
    g_noalloc_addr[dev] = p;
  }
  *out = g_noalloc_addr[dev];
  return 0;
}

}  // namespace

extern "C" {

// Same arguments and results as spral_ssids_gpu_ldlt_app_factor, but the
// workspace is the library's fixed device scratch array instead of
// cudaMalloc'd memory.  Limits and behaviour:
//  * lda must be at most 1024 (so m <= 1024); larger fronts are refused with
//    SPRAL_SSIDS_GPU_NOALLOC_TOO_LARGE (-60) and a message on stderr.
//  * The first call on each device looks up the scratch array's device
//    address (with that device current) and keeps it for later calls.
//  * Like spral_ssids_gpu_ldlt_app_factor, the call synchronises its stream
//    and reads the front's elimination count back before it returns.
//  * All calls share the one array and it keeps the previous call's contents;
//    the per-call state that must start from zero is cleared by each call.
//    Calls whose GPU work overlaps (different host threads or streams at the
//    same time on the same device) race on the array: serialise them.
//  * No cudaMalloc, cudaFree or allocating library routine is called.
int spral_ssids_gpu_ldlt_app_factor_noalloc(int m, int n, int* perm_dev, double* a_dev, int lda,
                                            double* d_dev, double beta, double* upd_dev,
                                            int ldupd,
                                            const struct spral_ssids_cpu_factor_options* options,
                                            void* stream) {
  if (m < n || n < 0) return -1;
  if (lda < m) return -4;
  if (m > n && upd_dev && ldupd < m - n) return -9;
  if (n == 0) return 0;  // nothing to factor: the same result as the allocating call
  if (lda > kNoAllocMaxLda || dense_workspace_bytes(m, n, lda) > kNoAllocScratchBytes) {
    fprintf(stderr,
            "spral_gb300: front too large for the fixed scratch (lda=%d, limit %d)\n", lda,
            kNoAllocMaxLda);
    return -60;
  }
  void* base = nullptr;
  const int st = noalloc_scratch_address(&base);
  if (st != 0) return st;
  spral_ssids_cpu_factor_options co{};
  co.action = true; co.small = 1e-20; co.u = 0.01; co.pivot_method = 2; co.failed_pivot_method = 1;
  if (options) co = *options;
  DenseWorkspace w = dense_workspace_carve(base, m, n, lda);
  return dense_factor_run(w, m, n, perm_dev, a_dev, lda, d_dev, beta, upd_dev, ldupd, co,
                          (cudaStream_t)stream);
}

}  // extern "C"
