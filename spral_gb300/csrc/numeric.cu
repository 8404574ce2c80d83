// Host orchestration and C-ABI of the GB300 numeric factor/solve.
//
// Replaces the GPU subtree of SSIDS (src/ssids/gpu/subtree.f90:20-72 and the
// level loop of src/ssids/gpu/factor.f90:240-656).  Design:
//   * the whole assembly tree is one device-resident subtree; fronts are
//     numbered level by level (leaves first) so that a level's descriptors,
//     states and contribution blocks are contiguous;
//   * per level: zero + assemble (A, delays, children) -> ceil(n/32) APP
//     steps batched over the level's fronts -> TPP for failed columns ->
//     contribution block -> inertia counts; one host synchronisation per
//     level reads back the elimination counts, which fix the sizes (delays)
//     of the next level's fronts (the reference syncs per 8 columns,
//     dense_factor.f90:185-192);
//   * factors stay resident for repeated solves and same-pattern
//     refactorisation; solves take many right-hand sides at once.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <memory>
#include <new>
#include <stdexcept>
#include <type_traits>
#include <mutex>
#include <vector>

#include <cstdlib>

#include "spral_ssids_gpu.h"
#include "ssids_gpu.cuh"
#include "tune.h"
#include "schedule.h"

namespace ssids300 {

struct CudaFail {
  cudaError_t err;
  int line;
};

static std::atomic<long long> g_launches{0};
// stream capture and graph instantiation are serialised across handles
static std::mutex g_capture_mutex;

void PhaseTimer::mark(int phase, cudaStream_t s) {
  if (used == cap) {
    int nc = cap ? 2 * cap : 1024;
    cudaEvent_t* ne = new cudaEvent_t[nc];
    int* np = new int[nc];
    for (int i = 0; i < cap; ++i) { ne[i] = ev[i]; np[i] = ph[i]; }
    for (int i = cap; i < nc; ++i) cudaEventCreate(&ne[i]);
    delete[] ev;
    delete[] ph;
    ev = ne;
    ph = np;
    cap = nc;
  }
  cudaEventRecord(ev[used], s);
  ph[used++] = phase;
}
void PhaseTimer::flush() {
  for (int i = 0; i + 1 < used; ++i) {
    float t = 0;
    if (cudaEventElapsedTime(&t, ev[i], ev[i + 1]) == cudaSuccess) {
      ms[ph[i]] += t;
      cnt[ph[i]] += 1;
    }
  }
  if (used > 0) { ev[0] = ev[0]; }
  // keep the last event as the start of the next interval
  if (used > 0) {
    std::swap(ev[0], ev[used - 1]);
    ph[0] = ph[used - 1];
    used = 1;
  }
  cudaGetLastError();
}
void PhaseTimer::reset() {
  used = 0;
  for (int i = 0; i < kPhCount; ++i) { ms[i] = 0; cnt[i] = 0; }
}
PhaseTimer::~PhaseTimer() {
  for (int i = 0; i < cap; ++i) cudaEventDestroy(ev[i]);
  delete[] ev;
  delete[] ph;
}
// launches issued by this thread (a capture counts the launches it records)
static thread_local long long t_launches = 0;
void note_launches(int k) {
  g_launches += k;
  t_launches += k;
}
double fp64_peak_tflops(int device);
void launch_recip_probe(const double* x, double* y, int n, cudaStream_t s);

#define CK(x)                                              \
  do {                                                     \
    cudaError_t e_ = (x);                                  \
    if (e_ != cudaSuccess) throw CudaFail{e_, __LINE__};   \
  } while (0)

// ---------------------------------------------------------------------------
// Device block cache.  Numeric handles take their large buffers (factor
// arena chunks, contribution blocks, workspaces, solve vectors) from here
// and give them back when they grow them or are destroyed, so a caller that
// factors one matrix after another with a new handle each time (as
// ssids_factor does) does not pay cudaMalloc and cudaFree, and the device
// synchronisation of cudaFree, for every handle.  Blocks of 4 KiB or more
// are kept per device in size classes (4 KiB steps up to 64 KiB, 64 KiB
// steps up to 2 MiB, 2 MiB steps above), up to a quarter of the device's
// memory; a request takes the
// smallest cached block of its class or at most a quarter larger.
// spral_ssids_gpu_mem_info counts cached bytes as free, and
// spral_ssids_gpu_release_cache returns them to the driver.
// ---------------------------------------------------------------------------
namespace {
constexpr int kCacheDevices = 64;
struct BlockCache {
  std::mutex mu;
  std::multimap<size_t, void*> blocks[kCacheDevices];
  size_t bytes[kCacheDevices] = {0};
  size_t limit[kCacheDevices] = {0};
};
BlockCache& block_cache() {
  static BlockCache* c = new BlockCache();  // never destroyed: blocks outlive static teardown
  return *c;
}
constexpr size_t kCacheMin = size_t(4) << 10;  // smaller blocks are not cached
size_t cache_class(size_t bytes) {
  const size_t g = bytes < (size_t(64) << 10)  ? (size_t(4) << 10)
                   : bytes < (size_t(2) << 20) ? (size_t(64) << 10)
                                               : (size_t(2) << 20);
  return (bytes + g - 1) / g * g;
}
}  // namespace

// Allocation-failure injection for tests (spral_ssids_gpu_inject_alloc_failure):
// when >= 0, the number of cache_alloc calls that still succeed; the call
// after them fails as cudaMalloc does when the device is out of memory.
static std::atomic<int> g_alloc_fail_after{-1};

// allocate `bytes` on the current device; *cls receives the block's size
void* cache_alloc(size_t bytes, size_t* cls, int* dev_out) {
  int dev = 0;
  CK(cudaGetDevice(&dev));
  if (g_alloc_fail_after.load() >= 0 && g_alloc_fail_after.fetch_sub(1) == 0)
    throw CudaFail{cudaErrorMemoryAllocation, __LINE__};
  *dev_out = dev;
  const size_t c = cache_class(std::max<size_t>(bytes, 1));
  *cls = c;
  if (c >= kCacheMin && dev >= 0 && dev < kCacheDevices) {
    BlockCache& bc = block_cache();
    std::lock_guard<std::mutex> lock(bc.mu);
    auto it = bc.blocks[dev].lower_bound(c);
    if (it != bc.blocks[dev].end() && it->first <= c + c / 4) {
      void* p = it->second;
      *cls = it->first;
      bc.bytes[dev] -= it->first;
      bc.blocks[dev].erase(it);
      return p;
    }
  }
  void* p = nullptr;
  cudaError_t e = cudaMalloc(&p, c);
  if (e == cudaErrorMemoryAllocation && dev >= 0 && dev < kCacheDevices) {
    // give the cached blocks back and retry once
    cudaGetLastError();
    BlockCache& bc = block_cache();
    {
      std::lock_guard<std::mutex> lock(bc.mu);
      for (auto& kv : bc.blocks[dev]) cudaFree(kv.second);
      bc.blocks[dev].clear();
      bc.bytes[dev] = 0;
    }
    e = cudaMalloc(&p, c);
  }
  CK(e);
  return p;
}

// return a block of size cls (from cache_alloc) allocated on device dev
void cache_free(void* p, size_t cls, int dev) {
  if (!p) return;
  if (cls >= kCacheMin && dev >= 0 && dev < kCacheDevices) {
    BlockCache& bc = block_cache();
    std::lock_guard<std::mutex> lock(bc.mu);
    if (bc.limit[dev] == 0) {
      size_t fr = 0, tot = 0;
      int cur = -1;
      cudaGetDevice(&cur);
      if (cur != dev) cudaSetDevice(dev);
      if (cudaMemGetInfo(&fr, &tot) != cudaSuccess) { cudaGetLastError(); tot = 0; }
      if (cur != dev && cur >= 0) cudaSetDevice(cur);
      bc.limit[dev] = std::max<size_t>(tot / 4, 1);
    }
    if (bc.bytes[dev] + cls <= bc.limit[dev]) {
      bc.blocks[dev].emplace(cls, p);
      bc.bytes[dev] += cls;
      return;
    }
  }
  int cur = -1;
  cudaGetDevice(&cur);
  if (cur != dev && dev >= 0) cudaSetDevice(dev);
  cudaFree(p);
  if (cur != dev && cur >= 0) cudaSetDevice(cur);
}

// cudaFree on the block's device (not cached)
void release_now(void* p, int dev) {
  int cur = -1;
  cudaGetDevice(&cur);
  if (cur != dev && dev >= 0) cudaSetDevice(dev);
  cudaFree(p);
  if (cur != dev && cur >= 0) cudaSetDevice(cur);
}

size_t cache_bytes(int dev) {
  if (dev < 0 || dev >= kCacheDevices) return 0;
  BlockCache& bc = block_cache();
  std::lock_guard<std::mutex> lock(bc.mu);
  return bc.bytes[dev];
}

void cache_release(int dev) {
  if (dev < 0 || dev >= kCacheDevices) return;
  BlockCache& bc = block_cache();
  std::lock_guard<std::mutex> lock(bc.mu);
  int cur = -1;
  cudaGetDevice(&cur);
  if (cur != dev) cudaSetDevice(dev);
  for (auto& kv : bc.blocks[dev]) cudaFree(kv.second);
  bc.blocks[dev].clear();
  bc.bytes[dev] = 0;
  if (cur != dev && cur >= 0) cudaSetDevice(cur);
}

// ---------------------------------------------------------------------------
// device arena: chunked bump allocator that can be rewound for refactorisation
// ---------------------------------------------------------------------------
struct DevArena {
  struct Chunk {
    char* p;
    size_t cap;
    int dev;
  };
  std::vector<Chunk> chunks;
  size_t ci = 0, used = 0;
  size_t min_chunk = size_t(64) << 20;
  void rewind() { ci = 0; used = 0; }
  void* alloc(size_t bytes) {
    bytes = (bytes + 255) & ~size_t(255);
    if (bytes == 0) bytes = 256;
    while (ci < chunks.size()) {
      if (used + bytes <= chunks[ci].cap) {
        void* r = chunks[ci].p + used;
        used += bytes;
        return r;
      }
      ++ci;
      used = 0;
    }
    size_t cap = std::max(bytes, min_chunk);
    int dev = 0;
    void* p = cache_alloc(cap, &cap, &dev);
    chunks.push_back({(char*)p, cap, dev});
    ci = chunks.size() - 1;
    used = bytes;
    return p;
  }
  ~DevArena() {
    for (auto& c : chunks) cache_free(c.p, c.cap, c.dev);
  }
};

template <typename T>
struct DevBuf {
  T* p = nullptr;
  size_t cap = 0;    // elements
  size_t bytes = 0;  // size of the cache block
  int dev = -1;
  void ensure(size_t n) {
    if (n <= cap) return;
    // kernels already queued may still use the old block: give it to the
    // driver (cudaFree waits for them) rather than to the cache
    if (p) release_now(p, dev);
    p = nullptr;
    size_t nc = std::max(n, cap + cap / 2);
    p = static_cast<T*>(cache_alloc(std::max<size_t>(nc, 1) * sizeof(T), &bytes, &dev));
    cap = bytes / sizeof(T);
  }
  // the owner has finished all work that uses the block (Numeric's
  // destructor synchronises its stream first)
  ~DevBuf() {
    if (p) cache_free(p, bytes, dev);
  }
};

// Size classes of the small leaf subtrees' fronts for the level-set kernel
// (launch_tpp_level): rows <= 32 one warp per front, <= 96 two warps, more
// 256 threads; a class launch stages fronts up to its cap in shared memory
// and factors larger ones in place.
constexpr int kTppClasses = 3;
inline int tpp_class(int rows) { return rows <= 32 ? 0 : rows <= 96 ? 1 : 2; }
inline int tpp_class_threads(int c) { return c == 0 ? 32 : c == 1 ? 64 : 256; }
inline int tpp_class_smem_cap(int c) { return c == 2 ? (100 << 10) : (64 << 10); }

template <typename T>
static T* upload(const std::vector<T>& v) {
  T* p = nullptr;
  CK(cudaMalloc(&p, std::max<size_t>(v.size(), 1) * sizeof(T)));
  if (!v.empty()) CK(cudaMemcpy(p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice));
  return p;
}

// ---------------------------------------------------------------------------
// symbolic subtree
// ---------------------------------------------------------------------------
struct Symbolic {
  int device = 0, n = 0, nnodes = 0, nlev = 0;
  bool root_aligned = false;  // level schedule (see build_symbolic)
  std::vector<int> sptr, ncol, nrow, parent;  // per node (0-based; parent -1 = root)
  std::vector<int64_t> rptr, nptr;
  std::vector<int> rlist;
  std::vector<std::vector<int>> children;  // node ids, decreasing (reference order)
  std::vector<int> front_of, node_of, lvl_start;
  // Small leaf subtrees (SymbolicSubtree.hxx:56-82): per front, 1 when its
  // node lies in a leaf subtree below small_subtree_threshold flops, which
  // the reference's CPU path factors with TPP only; per level, the number of
  // other (APP) fronts, listed first in the level's part of d_fronts.
  std::vector<char> tpp_only;
  std::vector<int> lvl_napp;
  // the level's TPP fronts by size class for the level-set kernel
  // (kTppClasses classes of rows, largest first within a class):
  // d_tpp[tpp_off[kTppClasses * l + c] .. tpp_off[kTppClasses * l + c + 1])
  std::vector<int> tpp_off, tpp_list;
  std::vector<int> cols_start;  // per level into cols
  std::vector<int> lvl_colrows;  // per level, the longest contribution-block column (parent or child)
  std::vector<int64_t> contrib_off;  // per front, elements
  int64_t contrib_total = 0;
  int64_t nnz = 0;
  std::vector<int> rdir_h;
  std::vector<int64_t> rdir_ptr_h;
  // device
  int64_t* d_nptr = nullptr;
  int64_t* d_nlist = nullptr;
  int* d_sptr = nullptr;
  int* d_rlist = nullptr;
  int64_t* d_rptr = nullptr;
  int* d_rdir = nullptr;
  int64_t* d_rdir_ptr = nullptr;
  int* d_fronts = nullptr;
  int* d_tpp = nullptr;
  int4* d_cols = nullptr;
  int2* d_pairs = nullptr;
  int* d_gp = nullptr;        // per front, nrow + 1 offsets into d_pairs by parent position
  // optional row groups of the refinement's backward error (pivot order)
  int ngroups = 0;
  int* d_row_group = nullptr;
  int* d_front_group = nullptr;  // the group of each front (its first column's)
  std::vector<int64_t> gp_off;
  // FP64 matrix in pivot order (full CSR, both triangles) for refinement
  int64_t* d_aptr = nullptr;
  int* d_acol = nullptr;
  int64_t* d_asrc = nullptr;
  spral_ssids_gpu_options gopts{};
  spral_ssids_cpu_factor_options copts{};
  ~Symbolic() {
    cudaFree(d_nptr); cudaFree(d_nlist); cudaFree(d_sptr); cudaFree(d_rlist); cudaFree(d_rptr);
    cudaFree(d_rdir); cudaFree(d_rdir_ptr); cudaFree(d_fronts); cudaFree(d_cols); cudaFree(d_tpp);
    cudaFree(d_pairs); cudaFree(d_gp); cudaFree(d_row_group); cudaFree(d_front_group);
    cudaFree(d_aptr); cudaFree(d_acol); cudaFree(d_asrc);
  }
};

static Symbolic* build_symbolic(int device, int n, int sa, int en, const int* sptr1,
                                const int* sparent1, const int64_t* rptr1, const int* rlist1,
                                const int64_t* nptr1, const int64_t* nlist1,
                                const spral_ssids_cpu_factor_options* opts) {
  std::unique_ptr<Symbolic> S(new Symbolic());
  S->device = device;
  S->n = n;
  const int s0 = sa - 1;  // first node (0-based)
  const int nn = en - sa;
  S->nnodes = nn;
  if (opts) S->copts = *opts;
  S->gopts.precision = 0;
  S->gopts.max_refine = 10;
  S->gopts.refine_tol = 1e-15;
  S->sptr.resize(nn + 1);
  S->ncol.resize(nn);
  S->nrow.resize(nn);
  S->parent.resize(nn);
  S->rptr.resize(nn + 1);
  S->nptr.resize(nn + 1);
  for (int i = 0; i <= nn; ++i) {
    S->sptr[i] = sptr1[s0 + i] - 1;
    S->rptr[i] = rptr1[s0 + i] - rptr1[s0];
    S->nptr[i] = nptr1[s0 + i] - nptr1[s0];
  }
  for (int i = 0; i < nn; ++i) {
    S->ncol[i] = S->sptr[i + 1] - S->sptr[i];
    S->nrow[i] = (int)(S->rptr[i + 1] - S->rptr[i]);
    int p = sparent1[s0 + i] - 1 - s0;
    S->parent[i] = (p >= 0 && p < nn) ? p : -1;
  }
  S->rlist.resize(S->rptr[nn]);
  for (int64_t k = 0; k < S->rptr[nn]; ++k) S->rlist[k] = rlist1[rptr1[s0] - 1 + k] - 1;
  // nlist: 0-based pairs
  const int64_t npairs = S->nptr[nn];
  std::vector<int64_t> nl(2 * npairs);
  int64_t maxsrc = -1;
  for (int64_t k = 0; k < npairs; ++k) {
    nl[2 * k] = nlist1[2 * (nptr1[s0] - 1 + k)] - 1;
    nl[2 * k + 1] = nlist1[2 * (nptr1[s0] - 1 + k) + 1] - 1;
    maxsrc = std::max(maxsrc, nl[2 * k]);
  }
  S->nnz = maxsrc + 1;
  // children in decreasing order, the order in which the reference's CPU
  // path visits them (SymbolicSubtree.hxx:42-47 pushes each node onto its
  // parent's list): delayed columns are appended, and contributions added,
  // last child first
  S->children.assign(nn, {});
  for (int i = nn - 1; i >= 0; --i)
    if (S->parent[i] >= 0) S->children[S->parent[i]].push_back(i);
  // small leaf subtrees: flops below each node, then from every leaf up
  // while the subtree stays below the threshold (a single node is not a
  // subtree).  Each marked set is a whole subtree: nodes are in postorder,
  // and the first leaf of an unmarked range walks up to the highest node
  // below the threshold, whose subtree starts at that leaf.
  std::vector<char> insl(nn, 0);
  {
    const int64_t thr = opts ? opts->small_subtree_threshold : int64_t(4000000);
    std::vector<int64_t> fl(nn + 1, 0);
    for (int i = 0; i < nn; ++i) {
      for (int k = 0; k < S->ncol[i]; ++k) fl[i] += (int64_t)(S->nrow[i] - k) * (S->nrow[i] - k);
      fl[S->parent[i] >= 0 ? S->parent[i] : nn] += fl[i];
    }
    for (int i = 0; i < nn;) {
      if (!S->children[i].empty()) { ++i; continue; }
      int last = i;
      for (int cur = i; cur >= 0 && cur < nn; cur = S->parent[cur]) {
        if (fl[cur] >= thr) break;
        last = cur;
      }
      if (last == i) { ++i; continue; }
      for (int j = i; j <= last; ++j) insl[j] = 1;
      i = last + 1;
    }
  }
  // levels (schedule.cpp): root-aligned where that takes at least 10%
  // fewer APP block steps, else leaf-aligned; SPRAL_GB300_LEVEL_ALIGN =
  // leaf | root forces one
  std::vector<int> lev;
  int nlev = 0;
  {
    const char* al = getenv("SPRAL_GB300_LEVEL_ALIGN");
    const LevelAlign align = !al ? LevelAlign::Choose
                             : std::string(al) == "root" ? LevelAlign::Root
                             : std::string(al) == "leaf" ? LevelAlign::Leaf
                                                         : LevelAlign::Choose;
    S->root_aligned =
        level_schedule(nn, S->parent.data(), S->ncol.data(), insl.data(), align, lev, nlev);
  }
  {
    // split crowded levels: kernels index a level's fronts in blockIdx.y
    // (at most 65535) and the tensor-core split kernel two jobs per front in
    // blockIdx.z; fronts of one level are independent, so consecutive
    // sub-levels keep the schedule valid
    constexpr int kMaxLevelFronts = 16384;
    std::vector<int> cnt(nlev, 0), base(nlev + 1, 0), seen(nlev, 0);
    for (int i = 0; i < nn; ++i) cnt[lev[i]]++;
    for (int l = 0; l < nlev; ++l)
      base[l + 1] = base[l] + std::max(1, (cnt[l] + kMaxLevelFronts - 1) / kMaxLevelFronts);
    for (int i = 0; i < nn; ++i) {
      const int l = lev[i];
      lev[i] = base[l] + seen[l]++ / kMaxLevelFronts;
    }
    nlev = base[nlev];
  }
  S->nlev = nlev;
  S->lvl_start.assign(nlev + 1, 0);
  for (int i = 0; i < nn; ++i) S->lvl_start[lev[i] + 1]++;
  for (int l = 0; l < nlev; ++l) S->lvl_start[l + 1] += S->lvl_start[l];
  S->front_of.resize(nn);
  S->node_of.resize(nn);
  {
    std::vector<int> pos(S->lvl_start.begin(), S->lvl_start.end() - 1);
    for (int i = 0; i < nn; ++i) {
      int f = pos[lev[i]]++;
      S->front_of[i] = f;
      S->node_of[f] = i;
    }
  }
  // contribution block offsets (level-major)
  S->contrib_off.resize(nn + 1);
  int64_t off = 0;
  for (int f = 0; f < nn; ++f) {
    S->contrib_off[f] = off;
    int64_t cm = S->nrow[S->node_of[f]] - S->ncol[S->node_of[f]];
    off += ((cm * cm + 63) / 64) * 64;
  }
  S->contrib_off[nn] = off;
  S->contrib_total = off;
  // rdir: parent position of each contribution row of a child
  S->rdir_ptr_h.assign(nn + 1, 0);
  for (int i = 0; i < nn; ++i) S->rdir_ptr_h[i + 1] = S->rdir_ptr_h[i] + (S->nrow[i] - S->ncol[i]);
  S->rdir_h.assign(S->rdir_ptr_h[nn], -1);
  {
    std::vector<int> pos(std::max(n, 1), -1);
    for (int p = 0; p < nn; ++p) {
      for (int k = 0; k < S->nrow[p]; ++k) pos[S->rlist[S->rptr[p] + k]] = k;
      for (int c : S->children[p]) {
        int cm = S->nrow[c] - S->ncol[c];
        for (int ic = 0; ic < cm; ++ic) {
          int var = S->rlist[S->rptr[c] + S->ncol[c] + ic];
          S->rdir_h[S->rdir_ptr_h[c] + ic] = pos[var];
        }
      }
      for (int k = 0; k < S->nrow[p]; ++k) pos[S->rlist[S->rptr[p] + k]] = -1;
    }
  }
  // extend-add work: per level, per parent column, the (child, jc) pairs
  // (the same pairs, indexed by parent position through gp, drive the
  // forward solve's gather: gp[gp_off[f] + P] .. gp[gp_off[f] + P + 1])
  std::vector<int4> cols;
  std::vector<int2> pairs;
  S->cols_start.assign(nlev + 1, 0);
  S->lvl_colrows.assign(nlev, 0);
  S->gp_off.assign(nn + 1, 0);
  for (int f = 0; f < nn; ++f) S->gp_off[f + 1] = S->gp_off[f] + S->nrow[S->node_of[f]] + 1;
  std::vector<int> gp(S->gp_off[nn] + 1, 0);
  for (int l = 0; l < nlev; ++l) {
    S->cols_start[l] = (int)cols.size();
    for (int f = S->lvl_start[l]; f < S->lvl_start[l + 1]; ++f) {
      int p = S->node_of[f];
      std::vector<std::vector<int2>> per(S->nrow[p]);
      S->lvl_colrows[l] = std::max(S->lvl_colrows[l], S->nrow[p] - S->ncol[p]);
      for (int c : S->children[p]) {
        int cm = S->nrow[c] - S->ncol[c];
        S->lvl_colrows[l] = std::max(S->lvl_colrows[l], cm);
        for (int jc = 0; jc < cm; ++jc) {
          int P = S->rdir_h[S->rdir_ptr_h[c] + jc];
          per[P].push_back(make_int2(S->front_of[c], jc));
        }
      }
      for (int P = 0; P < S->nrow[p]; ++P) {
        gp[S->gp_off[f] + P] = (int)pairs.size();
        // every column of the contribution block gets a CTA (the extend-add
        // also zeroes it), those of the fully-summed part only with children
        if (per[P].empty() && P < S->ncol[p]) continue;
        int beg = (int)pairs.size();
        for (auto& q : per[P]) pairs.push_back(q);
        cols.push_back(make_int4(f, P, beg, (int)pairs.size()));
      }
      gp[S->gp_off[f] + S->nrow[p]] = (int)pairs.size();
    }
  }
  S->cols_start[nlev] = (int)cols.size();
  // full CSR of A in pivot order: for each nlist pair, (prow, pcol, src)
  std::vector<int64_t> aptr(n + 1, 0);
  {
    std::vector<int> pr(npairs), pc(npairs);
    for (int i = 0; i < nn; ++i) {
      for (int64_t k = S->nptr[i]; k < S->nptr[i + 1]; ++k) {
        int64_t dest = nl[2 * k + 1];
        int c = (int)(dest / S->nrow[i]), r = (int)(dest % S->nrow[i]);
        pr[k] = S->rlist[S->rptr[i] + r];
        pc[k] = S->rlist[S->rptr[i] + c];
      }
    }
    for (int64_t k = 0; k < npairs; ++k) {
      aptr[pr[k] + 1]++;
      if (pr[k] != pc[k]) aptr[pc[k] + 1]++;
    }
    for (int i = 0; i < n; ++i) aptr[i + 1] += aptr[i];
    std::vector<int> acol(aptr[n]);
    std::vector<int64_t> asrc(aptr[n]);
    std::vector<int64_t> fill(aptr.begin(), aptr.end() - 1);
    for (int64_t k = 0; k < npairs; ++k) {
      acol[fill[pr[k]]] = pc[k];
      asrc[fill[pr[k]]++] = nl[2 * k];
      if (pr[k] != pc[k]) {
        acol[fill[pc[k]]] = pr[k];
        asrc[fill[pc[k]]++] = nl[2 * k];
      }
    }
    CK(cudaSetDevice(device));
    S->d_aptr = upload(aptr);
    S->d_acol = upload(acol);
    S->d_asrc = upload(asrc);
  }
  S->tpp_only.assign(nn, 0);
  for (int i = 0; i < nn; ++i) S->tpp_only[S->front_of[i]] = insl[i];
  std::vector<int> fronts(nn);
  S->lvl_napp.assign(nlev, 0);
  for (int l = 0; l < nlev; ++l) {
    int k = S->lvl_start[l];
    for (int f = S->lvl_start[l]; f < S->lvl_start[l + 1]; ++f)
      if (!S->tpp_only[f]) fronts[k++] = f;
    S->lvl_napp[l] = k - S->lvl_start[l];
    for (int f = S->lvl_start[l]; f < S->lvl_start[l + 1]; ++f)
      if (S->tpp_only[f]) fronts[k++] = f;
  }
  // size classes of the TPP fronts (rows at analysis)
  S->tpp_off.assign((size_t)kTppClasses * nlev + 1, 0);
  S->tpp_list.clear();
  for (int l = 0; l < nlev; ++l)
    for (int c = 0; c < kTppClasses; ++c) {
      S->tpp_off[(size_t)kTppClasses * l + c] = (int)S->tpp_list.size();
      std::vector<int> cls;
      for (int f = S->lvl_start[l]; f < S->lvl_start[l + 1]; ++f)
        if (S->tpp_only[f] && tpp_class(S->nrow[S->node_of[f]]) == c) cls.push_back(f);
      std::stable_sort(cls.begin(), cls.end(), [&](int a, int b) {
        return S->nrow[S->node_of[a]] > S->nrow[S->node_of[b]];
      });
      S->tpp_list.insert(S->tpp_list.end(), cls.begin(), cls.end());
    }
  S->tpp_off[(size_t)kTppClasses * nlev] = (int)S->tpp_list.size();
  std::vector<int> sp(S->sptr.begin(), S->sptr.end());
  S->d_nptr = upload(S->nptr);
  S->d_nlist = upload(nl);
  S->d_sptr = upload(sp);
  S->d_rlist = upload(S->rlist);
  S->d_rptr = upload(S->rptr);
  S->d_rdir = upload(S->rdir_h);
  S->d_rdir_ptr = upload(S->rdir_ptr_h);
  S->d_fronts = upload(fronts);
  if (!S->tpp_list.empty()) S->d_tpp = upload(S->tpp_list);
  S->d_cols = upload(cols);
  S->d_pairs = upload(pairs);
  S->d_gp = upload(gp);
  return S.release();
}

// ---------------------------------------------------------------------------
// numeric subtree
// ---------------------------------------------------------------------------
struct NumericBase {
  virtual ~NumericBase() {}
  bool posdef = false;
  int precision = 0;
  spral_ssids_thread_stats stats{};
  double timing[5] = {0, 0, 0, 0, 0};
  bool profile = false;
  double prof_ms = 0, prof_flops = 0;
  long long prof_launches = 0;
  double prof_tc_ms = 0, prof_tc_flops = 0;  // tensor-core GEMM kernel alone
  long long prof_tc_launches = 0;
  PhaseTimer ptimer;
  PhaseTimer* tm() { return profile ? &ptimer : nullptr; }
  virtual int factor(const double* aval, bool aval_on_device, const double* scaling,
                     cudaStream_t user_stream) = 0;
  virtual int solve_dev(int job, int nrhs, double* x, int ldx, cudaStream_t s) = 0;
  virtual int solve_refined(int nrhs, double* x_host, int ldx, int* iters) = 0;
  virtual int solve_refined_dev(int nrhs, const double* b, double* x, int ld, int* iters,
                                double* bwd) = 0;
  virtual void enquire(int* piv, double* d) = 0;
  virtual void alter(const double* d) = 0;
  virtual Symbolic* symbolic() = 0;
  virtual int debug_front(int node, int* info, double* L, double* D, int* perm) = 0;
  virtual int node_inertia(int* out) = 0;
  // per row group, the scaled backward error of the last refined solve
  virtual int group_bwd_errors(double* out, int ngroups) = 0;
  virtual cudaStream_t get_stream() const = 0;
  virtual int get_contrib() = 0;
  // the subtree root's contribution for a parent outside the subtree, host
  // copies filled by get_contrib() and kept until free_contrib
  std::vector<double> contrib_val, contrib_delay;
  std::vector<int> contrib_rlist, contrib_perm;
  int contrib_n = 0, contrib_ndelay = 0, contrib_lddelay = 0;
  DevBuf<double> hsolve;  // device copy of host right-hand sides (host-buffer solves)
  // FP64 refactorisations taken by the FP32-factor path's refined solves
  int fallbacks = 0;
};

template <typename T>
void launch_zero_fronts(FrontDesc<T>* fd, const int* fronts, int nf, int max_elems,
                        cudaStream_t s);
void launch_resid_bwd_err(const int64_t* aptr, const int* acol, const int64_t* asrc,
                          const double* aval, int n, const double* x, const double* b, double* r,
                          int nrhs, int ld, double* work, const int* row_group, int ngroups,
                          cudaStream_t s);
void launch_axpy(int n, int nrhs, int ld, double* x, const double* d, cudaStream_t s,
                 const int* row_group = nullptr, const unsigned char* active = nullptr);

// ---------------------------------------------------------------------------
// Autotuner, run once per device (or read from the tune cache named by
// SPRAL_GB300_TUNE_CACHE, see tune.cpp).  It times, with CUDA events (best of
// five after a warm-up run; the tensor path's host-side job tables are built
// beforehand, as they are when the factorisation is replayed from its
// graph), synthetic fronts with contribution blocks of cm rows and
// max(32, cm / 2) eliminated columns (at least 256 for the tile classes):
//  * the SIMT contribution kernel against the tensor-core update at its best
//    tile width: the crossover is the smallest cm of the grid from which the
//    tensor cores are faster for every larger size of the grid;
//  * each tile width of the tensor-core kernel (128 x 64, 128 x 128,
//    128 x 256) at the size classes cm = 256 .. 4096: a launch whose largest
//    contribution block has at most cm rows takes that class's fastest width.
// ---------------------------------------------------------------------------
static std::mutex g_tune_mutex;

static std::string tune_device_key(int dev) {
  cudaDeviceProp pr{};
  if (cudaGetDeviceProperties(&pr, dev) != cudaSuccess) {
    cudaGetLastError();
    return "unknown";
  }
  std::string name = pr.name;
  for (auto& c : name)
    if (c == ' ' || c == '\t') c = '_';
  return name + "-sm" + std::to_string(pr.multiProcessorCount) + "-cc" +
         std::to_string(pr.major) + std::to_string(pr.minor);
}

static TuneTable measure_tune_table() {
  const int xgrid[] = {64, 96, 128, 192, 256, 384, 512};
  constexpr int nx = sizeof(xgrid) / sizeof(xgrid[0]);
  const int cgrid[] = {256, 512, 1024, 2048, 4096};
  constexpr int ncls = sizeof(cgrid) / sizeof(cgrid[0]);
  const int widths[] = {64, 128, 256};
  constexpr int nw = sizeof(widths) / sizeof(widths[0]);
  const int maxcm = cgrid[ncls - 1], maxk = 1024;  // storage for the largest case
  cudaStream_t s;
  CK(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
  DevBuf<float> L, LD, C;
  DevBuf<char> scratch;
  DevBuf<int> fr;
  FrontDesc<float>* d_fd = nullptr;
  FrontState* d_st = nullptr;
  int* d_status = nullptr;
  const int ld = ((maxcm + maxk) + 3) / 4 * 4;
  L.ensure((size_t)ld * maxk);
  LD.ensure((size_t)maxcm * maxk);
  C.ensure((size_t)maxcm * maxcm);
  fr.ensure(1);
  CK(cudaMalloc(&d_fd, sizeof(FrontDesc<float>)));
  CK(cudaMalloc(&d_st, sizeof(FrontState)));
  CK(cudaMalloc(&d_status, sizeof(int)));
  CK(cudaMemsetAsync(L.p, 0, L.cap * sizeof(float), s));
  CK(cudaMemsetAsync(LD.p, 0, LD.cap * sizeof(float), s));
  CK(cudaMemsetAsync(C.p, 0, C.cap * sizeof(float), s));
  CK(cudaMemsetAsync(fr.p, 0, sizeof(int), s));
  CK(cudaMemsetAsync(d_status, 0, sizeof(int), s));

  cudaEvent_t e0, e1;
  CK(cudaEventCreate(&e0));
  CK(cudaEventCreate(&e1));
  auto best = [&](auto&& run) {
    float b = 1e30f;
    for (int r = 0; r < 6; ++r) {  // first run warms up
      CK(cudaEventRecord(e0, s));
      run();
      CK(cudaEventRecord(e1, s));
      CK(cudaEventSynchronize(e1));
      float ms = 0;
      CK(cudaEventElapsedTime(&ms, e0, e1));
      if (r > 0) b = std::min(b, ms);
    }
    return b;
  };
  void* blob = nullptr;
  // tensor-core time of one (cm, k) front at tile width bn
  auto time_tc = [&](int cm, int kk, int bn) {
    std::vector<TcProblem> ps(1);
    ps[0] = {L.p + kk, ld, LD.p, cm, C.p, cm, cm, cm, kk, &d_st->nelim, 1};
    scratch.ensure(tc_gemm_scratch_bytes(ps));
    TcPlan plan;
    if (tc_gemm_prepare(ps, scratch.p, plan, bn) != 0) throw CudaFail{cudaErrorUnknown, __LINE__};
    cudaFree(blob);
    blob = nullptr;
    CK(cudaMalloc(&blob, plan.blob.size()));
    CK(cudaMemcpy(blob, plan.blob.data(), plan.blob.size(), cudaMemcpyHostToDevice));
    return best([&] {
      if (tc_gemm_launch(plan, blob, d_status, s, kTcChunk) != 0)
        throw CudaFail{cudaErrorUnknown, __LINE__};
    });
  };
  auto set_front = [&](int cm, int kk) {
    FrontDesc<float> h{};
    h.L = L.p; h.LD = LD.p; h.C = C.p;
    h.m = cm + kk; h.n = kk; h.ld = ld; h.cm = cm; h.ldc = cm;
    h.nrow = cm + kk; h.ncol = kk;
    FrontState hs{};
    hs.nelim = kk;
    CK(cudaMemcpyAsync(d_fd, &h, sizeof(h), cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(d_st, &hs, sizeof(hs), cudaMemcpyHostToDevice, s));
  };
  TuneTable t;
  // tile width per size class
  for (int c = 0; c < ncls; ++c) {
    const int cm = cgrid[c], kk = std::max(256, std::min(cm / 2, maxk));
    set_front(cm, kk);
    float bt = 1e30f;
    int bw = kTuneDefaultBn;
    for (int w = 0; w < nw; ++w) {
      const float tt = time_tc(cm, kk, widths[w]);
      if (tt < bt) { bt = tt; bw = widths[w]; }
    }
    t.bucket_m[c] = cm;
    t.bn[c] = bw;
  }
  t.nb = ncls;
  // SIMT / tensor-core crossover, the tensor cores at the tuned width
  bool tc_wins[nx];
  for (int g = 0; g < nx; ++g) {
    const int cm = xgrid[g], kk = std::max(32, cm / 2);
    set_front(cm, kk);
    const float t_simt = best([&] { launch_contrib_gemm<float>(d_fd, d_st, fr.p, 1, cm, s); });
    tc_wins[g] = time_tc(cm, kk, tune_bn_for(t, cm)) < t_simt;
  }
  cudaFree(blob);
  int pick = xgrid[nx - 1] + 1;
  for (int g = nx - 1; g >= 0 && tc_wins[g]; --g) pick = xgrid[g];
  t.tc_min_cm = pick;
  CK(cudaStreamSynchronize(s));
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(d_fd);
  cudaFree(d_st);
  cudaFree(d_status);
  cudaStreamDestroy(s);
  return t;
}

static TuneTable autotune_device() {
  int dev = 0;
  CK(cudaGetDevice(&dev));
  std::lock_guard<std::mutex> lock(g_tune_mutex);
  TuneTable t;
  if (tune_get(dev, t)) return t;
  const char* cache = getenv("SPRAL_GB300_TUNE_CACHE");
  const std::string key = tune_device_key(dev);
  if (!(cache && *cache && tune_cache_lookup(cache, key, t))) {
    t = measure_tune_table();
    if (cache && *cache) (void)tune_cache_store(cache, key, t);  // best effort
  }
  tune_set(dev, t);
  return t;
}

static int autotune_tc_min_cm() { return autotune_device().tc_min_cm; }

int tc_tile_width(const std::vector<TcProblem>& ps) {
  if (const char* e = getenv("SPRAL_GB300_TC_BN")) {
    const int bn = atoi(e);
    if (tc_tile_width_ok(bn)) return bn;
  }
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) { cudaGetLastError(); return kTuneDefaultBn; }
  TuneTable t;
  if (!tune_get(dev, t)) return kTuneDefaultBn;
  int mm = 0;
  for (auto& p : ps) mm = std::max(mm, std::max(p.M, p.N));
  return tune_bn_for(t, mm);
}

template <typename T>
struct Numeric : NumericBase {
  Symbolic* S;
  cudaStream_t stream = nullptr;
  cudaEvent_t ev[4];
  std::vector<FrontDesc<T>> hfd;
  std::vector<FrontState> hst;
  std::vector<int> nelim_, ndin_, m_, n_, ld_, doff_, napp_;
  std::vector<int> lvl_max_m, lvl_max_nelim;
  FrontDesc<T>* d_fd = nullptr;
  FrontState* d_st = nullptr;
  Stats* d_stats = nullptr;
  int4* d_dwork = nullptr;
  DevBuf<double> aval_buf, scale_buf;
  DevBuf<T> contrib;
  DevArena farena, darena, iarena;
  DevBuf<T> ws_W, ws_swap, ws_LD;
  DevBuf<double> ws_step;
  DevBuf<int> ws_lperm;
  // solve
  bool solve_ready = false;
  SolveNode<T>* d_sn = nullptr;
  int* d_children = nullptr;
  DevBuf<SolveNode<T>> sn_buf;
  DevBuf<int> ch_buf;
  DevBuf<char> small_buf;  // d_fd, d_st, d_stats, d_dwork, d_tc_status, d_ncount
  // Captured solve sequences (CUDA graphs), replayed while the launch
  // sequence and every pointer it uses are unchanged (solve_sig).
  struct SolveGraph {
    int job, q, ldx;
    const double* x;
    uint64_t sig;
    cudaGraphExec_t exec;
    int nlaunch;
  };
  std::vector<SolveGraph> sgraphs;
  uint64_t solve_sig = 0;
  bool use_graphs = true;
  void drop_graphs() {
    for (auto& g : sgraphs) cudaGraphExecDestroy(g.exec);
    sgraphs.clear();
  }
  DevBuf<T> xloc;
  DevBuf<double> xbuf, rbuf, dbuf, bbuf, nbuf;
  // wavefront solves: per level, the forward and backward item lists (one
  // device array), the completion flags of every pivot block, and the ints
  // [status, forward counters (nlev), backward counters (nlev)]
  bool use_wave = true;
  DevBuf<int2> wave_items;
  DevBuf<int> wave_flags, wave_ints;
  // per row group, whether the refinement still solves for it (all ones
  // outside the refinement of a forest of row groups)
  DevBuf<unsigned char> group_active;
  DevBuf<T> wave_l21p;  // backward L21^T partial sums of the wavefront pass
  // inverses of the pivot blocks' unit lower diagonal blocks (FP32 factors'
  // wavefront passes; SPRAL_GB300_SOLVE_BINV=0 keeps the substitution),
  // formed once per factorisation before the first solve
  bool use_binv = false;
  DevBuf<T> wave_binv;
  DevBuf<int2> binv_blocks;
  int wave_nfwd = 0, wave_nbwd = 0;  // items of the forward pass, then of the backward pass
  int wave_nsmall = 0;  // small fronts (one item each per pass)
  size_t wave_nflags = 0;
  // optional trace of the wavefront passes (SPRAL_GB300_WAVE_TRACE = path
  // prefix): per item four stamps (taken, last wait over, finished, SM),
  // written with the item list after every pass; passes then run without
  // graphs
  std::string wave_trace;
  DevBuf<unsigned long long> wave_trace_buf;
  WaveLevel wave_pass(bool fwd) {
    WaveLevel w;
    w.items = wave_items.p + (fwd ? 0 : wave_nfwd);
    w.nitems = fwd ? wave_nfwd : wave_nbwd;
    w.counter = wave_ints.p + (fwd ? 1 : 2);
    w.trace = nullptr;
    // many small-front items: more CTAs in flight; otherwise the widest
    // fronts' chains set the time and keep their registers
    w.ctas_per_sm = 2 * wave_nsmall > wave_nfwd ? 3 : 2;
    w.front_group = S->d_front_group;
    w.active = S->d_front_group ? group_active.p : nullptr;
    if (!wave_trace.empty()) {
      wave_trace_buf.ensure(4 * (size_t)(wave_nfwd + wave_nbwd) + 4);
      w.trace = wave_trace_buf.p + (fwd ? 0 : 4 * (size_t)wave_nfwd);
    }
    return w;
  }
  void dump_wave_trace(cudaStream_t s) {
    CK(cudaStreamSynchronize(s));
    const size_t ni = (size_t)wave_nfwd + wave_nbwd;
    std::vector<int2> items(ni);
    std::vector<unsigned long long> tr(4 * ni);
    if (ni) {
      CK(cudaMemcpy(items.data(), wave_items.p, ni * sizeof(int2), cudaMemcpyDeviceToHost));
      CK(cudaMemcpy(tr.data(), wave_trace_buf.p, tr.size() * 8, cudaMemcpyDeviceToHost));
    }
    if (FILE* f = fopen((wave_trace + ".items").c_str(), "wb")) {
      fwrite(items.data(), sizeof(int2), ni, f);
      fclose(f);
    }
    if (FILE* f = fopen((wave_trace + ".trace").c_str(), "wb")) {
      fwrite(tr.data(), 8, tr.size(), f);
      fclose(f);
    }
    if (FILE* f = fopen((wave_trace + ".meta").c_str(), "w")) {
      fprintf(f, "%d %d\n", wave_nfwd, wave_nbwd);
      // per front: level, m, nelim
      for (int l = 0; l < S->nlev; ++l)
        for (int fr = S->lvl_start[l]; fr < S->lvl_start[l + 1]; ++fr)
          fprintf(f, "%d %d %d\n", l, m_[fr], nelim_[fr]);
      fclose(f);
    }
  }
  // tensor-core contribution GEMM (FP32 factors only)
  bool use_tc = false;
  int tc_chunk = kTcChunk;
  int tc_min_cm = 192;  // smallest contribution block formed on the tensor cores
  // fewest fully-summed columns (the update's depth K) of a front formed on
  // the tensor cores.  Shallower updates stream their contribution block
  // through HBM with little arithmetic per byte, so the tensor cores gain
  // little there, while their 3xTF32 products (about 22-bit operands) cost
  // the FP64 refinement a step: on the 48^3 and 32^3 Laplacians the
  // factor + refined solve was fastest with K >= 256 (48^3: 26.7 ms against
  // 28.9 ms with every front of >= 192 contribution rows on the tensor cores
  // and 28.1 ms with none).
  int tc_min_k = 256;
  TcBuffers tcbuf;
  DevBuf<char> tc_scratch;
  int panel_nb = 256;       // APP panel width (FP32 fronts with tensor cores)
  // fewest fully-summed columns of a front factored in panels: narrower
  // fronts keep the block steps' SIMT updates, which are exact in FP32
  // (the 3xTF32 products carry about 22 bits and can cost the FP64
  // refinement a step)
  int panel_min_n = 4096;
  DevBuf<int> panel_list;   // fronts ending a panel (eager mode)
  int* d_tc_status = nullptr;
  int* d_ncount = nullptr;  // per-node inertia counts (neg, two, zero)

  // Fronts of small leaf subtrees are factored by TPP alone (as the
  // reference's CPU path does), except in the positive-definite case, whose
  // small leaf subtrees use the same unpivoted factorisation as the rest,
  // and with pivot_method = tpp, where every front takes TPP after an empty
  // APP pass.  The level's APP fronts come first in d_fronts.
  bool tpp_front(int f) const {
    return !posdef && S->copts.pivot_method != 3 && S->tpp_only[f];
  }
  int app_fronts(int l) const {
    if (posdef || S->copts.pivot_method == 3) return S->lvl_start[l + 1] - S->lvl_start[l];
    return S->lvl_napp[l];
  }
  // APP panels (FP32 factors with tensor cores): a front with more than
  // panel_nb fully-summed columns is factored in panels of panel_nb columns;
  // the block steps of a panel update only the panel, and the panel's
  // trailing update (all later fully-summed columns and their rows below)
  // runs once per panel on the tensor cores with the panel's pivots as its
  // depth.  Returns the panel width of front f, or 0.
  int panel_cols(int f) const {
    if (!std::is_same<T, float>::value || !use_tc || panel_nb <= 0) return 0;
    if (tpp_front(f) || S->copts.pivot_method == 3) return 0;
    return n_[f] >= std::max(panel_min_n, panel_nb + 1) ? panel_nb : 0;
  }
  // fronts of [f0, f1) whose current panel ends with block step st
  void panel_boundary(int f0, int f1, int st, std::vector<int>& out) const {
    out.clear();
    const int per = panel_nb / kBlk;
    for (int f = f0; f < f1; ++f) {
      if (!hfd[f].panel) continue;
      const int steps_f = (n_[f] + kBlk - 1) / kBlk;
      if (st + 1 > steps_f) continue;
      if ((st + 1) % per == 0 || st + 1 == steps_f) out.push_back(f);
    }
  }
  // the tensor-core trailing update of a closed panel: pivots [pstart,
  // pstart + k) of front f, trailing block [q, m) x [q, n)
  TcProblem panel_problem(int f, int pstart, int q, int k) const {
    const FrontDesc<T>& d = hfd[f];
    TcProblem pr;
    pr.A = reinterpret_cast<const float*>(d.L + (int64_t)pstart * d.ld + q);
    pr.lda = d.ld;
    pr.B = reinterpret_cast<const float*>(d.LD);
    pr.ldb = d.n;
    pr.C = reinterpret_cast<float*>(d.L + (int64_t)q * d.ld + q);
    pr.ldc = d.ld;
    pr.M = d.m - q;
    pr.N = d.n - q;
    pr.kmax = k;
    pr.kval_dev = &d_st[f].pk;
    pr.lower = 1;
    return pr;
  }
  // end of panels in eager mode: the panels' geometry is read back (failed
  // columns move panel boundaries), then the trailing updates and the close
  void panel_end_eager(const std::vector<int>& fl, cudaStream_t s) {
    const int nfl = (int)fl.size();
    panel_list.ensure(nfl);
    CK(cudaMemcpyAsync(panel_list.p, fl.data(), nfl * sizeof(int), cudaMemcpyHostToDevice, s));
    int max_n = 0;
    for (int f : fl) max_n = std::max(max_n, n_[f]);
    launch_panel_end<T>(d_fd, d_st, panel_list.p, nfl, max_n, panel_nb, s);
    for (int f : fl)
      CK(cudaMemcpyAsync(&hst[f], &d_st[f], sizeof(FrontState), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    std::vector<TcProblem> ps;
    double fl_tc = 0;
    for (int f : fl) {
      const FrontState& q = hst[f];
      if (q.status != kDevOk || q.pk <= 0 || q.qend >= n_[f]) continue;
      ps.push_back(panel_problem(f, q.pstart, q.qend, q.pk));
      const double M = m_[f] - q.qend, N = n_[f] - q.qend;
      fl_tc += 2.0 * q.pk * (N * (N + 1) / 2 + (M - N) * N);
    }
    if (!ps.empty()) {
      tc_scratch.ensure(tc_gemm_scratch_bytes(ps));
      float ms_split = 0, ms_gemm = 0;
      if (tc_gemm_run(ps, tc_scratch.p, tcbuf, d_tc_status, s, tc_chunk,
                      profile ? &ms_split : nullptr, profile ? &ms_gemm : nullptr) != 0)
        throw CudaFail{cudaErrorUnknown, __LINE__};
      if (profile) { prof_tc_ms += ms_gemm; prof_tc_launches += 1; prof_tc_flops += fl_tc; }
    }
    launch_panel_close<T>(d_fd, d_st, panel_list.p, nfl, s);
  }

  // shared-memory staging of a small leaf front (k_tpp_small): the front,
  // two workspace columns, perm and opos, bytes
  // shared memory of a front in k_tpp_level: the front with two workspace
  // columns, perm and opos, then (FP32 factors, 16-byte aligned) its LD
  // block for the fused contribution
  int tpp_bytes(int f) const {
    const int front = ((m_[f] + 1) & ~1) * (n_[f] + 2) * (int)sizeof(T) + 8 * n_[f];
    if (sizeof(T) == 8) return front;
    return ((front + 15) & ~15) + (m_[f] - n_[f]) * n_[f] * (int)sizeof(T);
  }
  // the level-set kernel over level l's small-subtree fronts, one launch
  // per non-empty size class, shared memory sized for the class's largest
  // front (current sizes, delays included) up to the class cap
  void launch_tpp_levels(int l, cudaStream_t s) {
    const auto& co = S->copts;
    int cls[kTppClasses], nc = 0;
    for (int c = 0; c < kTppClasses; ++c)
      if (S->tpp_off[(size_t)kTppClasses * l + c + 1] > S->tpp_off[(size_t)kTppClasses * l + c])
        cls[nc++] = c;
    // the classes' fronts are independent: the first class on s, the others
    // on the side streams, joined back into s
    if (nc > 1) CK(cudaEventRecord(fork_ev, s));
    for (int k = 0; k < nc; ++k) {
      const int c = cls[k];
      const int o0 = S->tpp_off[(size_t)kTppClasses * l + c];
      const int o1 = S->tpp_off[(size_t)kTppClasses * l + c + 1];
      int mx = 0;
      for (int j = o0; j < o1; ++j) mx = std::max(mx, tpp_bytes(S->tpp_list[j]));
      cudaStream_t q = k == 0 ? s : side[k - 1];
      if (k > 0) CK(cudaStreamWaitEvent(q, fork_ev, 0));
      launch_tpp_level<T>(d_fd, d_st, S->d_tpp + o0, o1 - o0, co.action, co.u, co.small,
                          std::min(mx, tpp_class_smem_cap(c)), tpp_class_threads(c), q);
      if (k > 0) {
        CK(cudaEventRecord(join_ev[k - 1], q));
        CK(cudaStreamWaitEvent(s, join_ev[k - 1], 0));
      }
    }
  }

  std::vector<TcProblem> tc_problems(int f0, int f1) const {
    std::vector<TcProblem> ps;
    for (int f = f0; f < f1; ++f) {
      const FrontDesc<T>& d = hfd[f];
      if (!d.tc) continue;
      TcProblem p;
      p.A = reinterpret_cast<const float*>(d.L + d.n);
      p.lda = d.ld;
      p.B = reinterpret_cast<const float*>(d.LD);
      p.ldb = d.cm;
      p.C = reinterpret_cast<float*>(d.C);
      p.ldc = d.ldc;
      p.M = d.cm;
      p.N = d.cm;
      p.kmax = d.n;
      p.kval_dev = &d_st[f].nelim;
      p.lower = 1;
      ps.push_back(p);
    }
    return ps;
  }

  void run_tc_contrib(int f0, int f1, cudaStream_t s) {
    if (!use_tc) return;
    const std::vector<TcProblem> ps = tc_problems(f0, f1);
    if (ps.empty()) return;
    tc_scratch.ensure(tc_gemm_scratch_bytes(ps));
    float ms_split = 0, ms_gemm = 0;
    if (tc_gemm_run(ps, tc_scratch.p, tcbuf, d_tc_status, s, tc_chunk,
                    profile ? &ms_split : nullptr, profile ? &ms_gemm : nullptr) != 0)
      throw CudaFail{cudaErrorUnknown, __LINE__};
    if (profile) { prof_tc_ms += ms_gemm; prof_tc_launches += 1; }
  }

  // ---------------- captured factorisation (CUDA graph) ----------------
  // After an eager factorisation in which no front delayed a column, the
  // next same-pattern factorisation plans every level up front (sizes are
  // then fixed: no front receives delayed columns), uploads all front
  // descriptors and tensor-core job tables once, and captures the whole
  // level sweep as one graph.  Each replay is checked on the device's
  // results (every front OK with nelim == n); otherwise the factorisation is
  // redone eagerly.  The graph reads the values from aval_buf and the
  // scaling from scale_buf, so callers' pointers may change between calls.
  static constexpr int kGraphFallback = 1000;
  bool last_zero_delay = false;
  cudaGraphExec_t fgraph = nullptr;
  int fgraph_nlaunch = 0;
  bool fgraph_scaled = false;
  std::vector<void*> fgraph_blobs;
  std::vector<FrontDesc<T>> fg_hfd;
  std::vector<const void*> fgraph_key;
  int fg_maxfront = 0, fg_maxsn = 0;

  void drop_fgraph() {
    if (fgraph) cudaGraphExecDestroy(fgraph);
    fgraph = nullptr;
    for (void* b : fgraph_blobs) cudaFree(b);
    fgraph_blobs.clear();
    fgraph_key.clear();
  }

  std::vector<const void*> graph_key() const {
    return {aval_buf.p, scale_buf.p, ws_W.p, ws_swap.p, ws_LD.p, ws_step.p, ws_lperm.p,
            contrib.p,  tc_scratch.p, d_fd,  d_st,      d_stats, d_ncount};
  }

  void build_fgraph(bool scaled) {
    drop_fgraph();
    cudaStream_t s = stream;
    const int nn = S->nnodes;
    const auto& co = S->copts;
    // plan: no delayed columns anywhere, so front sizes are the symbolic ones
    size_t wsW = 0, wsSwap = 0, wsLD = 0, wsStep = 0, wsLp = 0;
    fg_maxfront = 0; fg_maxsn = 0;
    for (int l = 0; l < S->nlev; ++l) {
      size_t w1 = 0, w2 = 0, w3 = 0;
      const int f0 = S->lvl_start[l], f1 = S->lvl_start[l + 1];
      for (int f = f0; f < f1; ++f) {
        const int node = S->node_of[f];
        const int m = S->nrow[node], n = S->ncol[node], ld = (m + 3) / 4 * 4, cm = m - n;
        ndin_[f] = 0; m_[f] = m; n_[f] = n; ld_[f] = ld;
        w1 += (size_t)ld * kBlk;
        w2 += (size_t)ld * 64 + 256;
        w3 += (size_t)std::max(cm, panel_cols(f)) * n;
        fg_maxfront = std::max(fg_maxfront, m);
        fg_maxsn = std::max(fg_maxsn, n);
        for (int c : S->children[node]) doff_[S->front_of[c]] = 0;
      }
      wsW = std::max(wsW, w1); wsSwap = std::max(wsSwap, w2); wsLD = std::max(wsLD, w3);
      wsStep = std::max(wsStep, (size_t)(f1 - f0) * (kBlk * kBlk + 2 * kBlk + 64));
      wsLp = std::max(wsLp, (size_t)(f1 - f0) * kBlk);
    }
    ws_W.ensure(wsW + 64);
    ws_swap.ensure(wsSwap + 64);
    ws_LD.ensure(wsLD + 64);
    ws_step.ensure(wsStep);
    ws_lperm.ensure(wsLp);
    farena.rewind();
    darena.rewind();
    iarena.rewind();
    for (int l = 0; l < S->nlev; ++l) {
      const int f0 = S->lvl_start[l], f1 = S->lvl_start[l + 1];
      size_t oW = 0, oS = 0, oL = 0;
      for (int f = f0; f < f1; ++f) {
        const int node = S->node_of[f];
        FrontDesc<T>& d = hfd[f];
        d = FrontDesc<T>{};
        d.m = m_[f]; d.n = n_[f]; d.ld = ld_[f];
        d.nrow = S->nrow[node]; d.ncol = S->ncol[node];
        d.ndelay_in = 0;
        d.cm = d.nrow - d.ncol;
        d.ldc = d.cm;
        d.node = node;
        d.L = (T*)farena.alloc((size_t)d.ld * d.n * sizeof(T));
        d.D = (double*)darena.alloc((size_t)2 * d.n * sizeof(double) + 16);
        d.perm = (int*)iarena.alloc((size_t)d.n * sizeof(int));
        d.opos = (int*)iarena.alloc((size_t)d.n * sizeof(int));
        d.C = d.cm > 0 ? contrib.p + S->contrib_off[f] : nullptr;
        d.W = ws_W.p + oW; oW += (size_t)d.ld * kBlk;
        d.swapbuf = ws_swap.p + oS; oS += (size_t)d.ld * 64 + 256;
        d.LD = ws_LD.p + oL; oL += (size_t)std::max(d.cm, panel_cols(f)) * d.n;
        d.step = ws_step.p + (size_t)(f - f0) * (kBlk * kBlk + 2 * kBlk + 64);
        d.lperm = ws_lperm.p + (size_t)(f - f0) * kBlk;
        d.tc = (use_tc && d.cm >= tc_min_cm && d.n >= tc_min_k) ? 1 : 0;
        d.panel = panel_cols(f);
      }
    }
    fg_hfd = hfd;
    CK(cudaMemcpy(d_fd, hfd.data(), nn * sizeof(FrontDesc<T>), cudaMemcpyHostToDevice));
    // panel ends of the fronts with panels, with the static geometry of a
    // factorisation without failed columns (panel j covers [j nb, (j+1) nb))
    struct PanelStep {
      int l, st, off, nl, max_n, pp;  // pp: index into pps (-1: no update)
    };
    std::vector<PanelStep> psteps;
    std::vector<int> plist;
    std::vector<std::vector<TcProblem>> pps;
    {
      const int per = std::max(panel_nb / kBlk, 1);
      std::vector<int> pfl;
      for (int l = 0; l < S->nlev; ++l) {
        const int f0 = S->lvl_start[l], f1 = S->lvl_start[l + 1];
        int mx = 0;
        for (int f = f0; f < f1; ++f) if (hfd[f].panel) mx = std::max(mx, n_[f]);
        if (mx == 0) continue;
        for (int st = 0; st < (mx + kBlk - 1) / kBlk; ++st) {
          panel_boundary(f0, f1, st, pfl);
          if (pfl.empty()) continue;
          PanelStep ps{l, st, (int)plist.size(), (int)pfl.size(), 0, -1};
          std::vector<TcProblem> pr;
          for (int f : pfl) {
            plist.push_back(f);
            ps.max_n = std::max(ps.max_n, n_[f]);
            const int j = st / per, pstart = j * panel_nb;
            const int q = std::min((j + 1) * panel_nb, n_[f]);
            if (q < n_[f]) pr.push_back(panel_problem(f, pstart, q, q - pstart));
          }
          if (!pr.empty()) { ps.pp = (int)pps.size(); pps.push_back(pr); }
          psteps.push_back(ps);
        }
      }
    }
    const int* d_plist = nullptr;
    if (!plist.empty()) {
      void* b = nullptr;
      CK(cudaMalloc(&b, plist.size() * sizeof(int)));
      fgraph_blobs.push_back(b);
      CK(cudaMemcpy(b, plist.data(), plist.size() * sizeof(int), cudaMemcpyHostToDevice));
      d_plist = static_cast<const int*>(b);
    }
    // tensor-core job tables, one device blob per level and per panel end
    std::vector<TcPlan> tplans(S->nlev), pplans(pps.size());
    std::vector<const void*> tblob(S->nlev, nullptr), pblob(pps.size(), nullptr);
    if (use_tc) {
      size_t scr = 0;
      std::vector<std::vector<TcProblem>> lps(S->nlev);
      for (int l = 0; l < S->nlev; ++l) {
        lps[l] = tc_problems(S->lvl_start[l], S->lvl_start[l + 1]);
        if (!lps[l].empty()) scr = std::max(scr, tc_gemm_scratch_bytes(lps[l]));
      }
      for (auto& pr : pps) scr = std::max(scr, tc_gemm_scratch_bytes(pr));
      if (scr > 0) tc_scratch.ensure(scr);
      auto upload_plan = [&](const std::vector<TcProblem>& pr, TcPlan& plan) -> const void* {
        if (tc_gemm_prepare(pr, tc_scratch.p, plan) != 0)
          throw CudaFail{cudaErrorUnknown, __LINE__};
        void* b = nullptr;
        CK(cudaMalloc(&b, plan.blob.size()));
        fgraph_blobs.push_back(b);
        CK(cudaMemcpy(b, plan.blob.data(), plan.blob.size(), cudaMemcpyHostToDevice));
        return b;
      };
      for (int l = 0; l < S->nlev; ++l)
        if (!lps[l].empty()) tblob[l] = upload_plan(lps[l], tplans[l]);
      for (size_t i = 0; i < pps.size(); ++i) pblob[i] = upload_plan(pps[i], pplans[i]);
    }
    size_t pstep_i = 0;
    const double* d_scale = scaled ? scale_buf.p : nullptr;
    std::lock_guard<std::mutex> lock(g_capture_mutex);
    const long long l0 = t_launches;
    cudaGraph_t g = nullptr;
    CK(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
    try {
      CK(cudaMemsetAsync(d_st, 0, nn * sizeof(FrontState), s));
      CK(cudaMemsetAsync(d_tc_status, 0, sizeof(int), s));
      CK(cudaMemsetAsync(d_stats, 0, sizeof(Stats), s));
      CK(cudaMemsetAsync(d_ncount, 0, 3 * (size_t)nn * sizeof(int), s));
      for (int l = 0; l < S->nlev; ++l) {
        const int f0 = S->lvl_start[l], f1 = S->lvl_start[l + 1], nf = f1 - f0;
        const int napp = app_fronts(l);
        int max_m = 0, max_n = 0, max_cm = 0, max_ent = 0, max_app_n = 0, max_app_cm = 0;
        int64_t maxz = 0;
        for (int f = f0; f < f1; ++f) {
          const int node = S->node_of[f];
          max_m = std::max(max_m, m_[f]);
          max_n = std::max(max_n, n_[f]);
          max_cm = std::max(max_cm, hfd[f].cm);
          max_ent = std::max<int>(max_ent, (int)(S->nptr[node + 1] - S->nptr[node]));
          maxz = std::max(maxz, (int64_t)ld_[f] * n_[f]);
          if (!tpp_front(f)) {
            max_app_n = std::max(max_app_n, n_[f]);
            max_app_cm = std::max(max_app_cm, hfd[f].cm);
          }
        }
        const int* fr = S->d_fronts + f0;
        launch_zero_fronts<T>(d_fd, fr, nf, (int)std::min<int64_t>(maxz, 1 << 30), s);
        launch_load_a<T>(d_fd, fr, nf, S->d_nptr, S->d_nlist, aval_buf.p, S->d_rlist, S->d_rptr,
                         d_scale, max_ent, s);
        launch_init_perm<T>(d_fd, fr, nf, S->d_sptr, max_n, s);
        launch_assemble_contrib<T>(d_fd, S->d_cols + S->cols_start[l],
                                   S->cols_start[l + 1] - S->cols_start[l], S->d_pairs,
                                   S->d_rdir, S->d_rdir_ptr, S->lvl_colrows[l], s);
        const int steps = (max_app_n + kBlk - 1) / kBlk;
        for (int st = 0; st < steps; ++st) {
          int mr = 0, tr = 0, tc = 0;
          for (int f = f0; f < f1; ++f) {
            if (tpp_front(f)) continue;
            mr = std::max(mr, m_[f] - kBlk * st);
            tr = std::max(tr, m_[f] - kBlk * (st + 1));
            const int cols = n_[f] - kBlk * (st + 1);
            tc = std::max(tc, hfd[f].panel ? std::min(cols, hfd[f].panel) : cols);
          }
          launch_app_step<T>(d_fd, d_st, fr, napp, st, std::max(mr, 1), tr, tc, co.action,
                             posdef ? 0.0 : co.u, co.small, s, nullptr, posdef);
          if (pstep_i < psteps.size() && psteps[pstep_i].l == l && psteps[pstep_i].st == st) {
            const PanelStep& ps = psteps[pstep_i++];
            launch_panel_end<T>(d_fd, d_st, d_plist + ps.off, ps.nl, ps.max_n, panel_nb, s);
            if (ps.pp >= 0 &&
                tc_gemm_launch(pplans[ps.pp], pblob[ps.pp], d_tc_status, s, tc_chunk) != 0)
              throw CudaFail{cudaErrorUnknown, __LINE__};
            launch_panel_close<T>(d_fd, d_st, d_plist + ps.off, ps.nl, s);
          }
        }
        launch_app_finish<T>(d_fd, d_st, fr, nf, s);
        const bool tpp_all = (co.pivot_method == 3) || (co.failed_pivot_method == 1);
        launch_tpp<T>(d_fd, d_st, fr, napp, co.action, co.u, co.small, tpp_all, s);
        if (napp < nf) launch_tpp_levels(l, s);
        launch_calc_ld<T>(d_fd, d_st, fr, napp, max_app_cm, max_app_n, s);
        launch_contrib_gemm<T>(d_fd, d_st, fr, napp, max_app_cm, s);
        if (tblob[l] && tc_gemm_launch(tplans[l], tblob[l], d_tc_status, s, tc_chunk) != 0)
          throw CudaFail{cudaErrorUnknown, __LINE__};
        launch_stats<T>(d_fd, d_st, fr, nf, max_n, d_stats, d_ncount, s);
      }
    } catch (...) {
      cudaStreamEndCapture(s, &g);
      if (g) cudaGraphDestroy(g);
      g_launches -= t_launches - l0;
      t_launches = l0;
      drop_fgraph();
      throw;
    }
    CK(cudaStreamEndCapture(s, &g));
    fgraph_nlaunch = (int)(t_launches - l0);
    g_launches -= fgraph_nlaunch;  // counted at each replay instead
    t_launches = l0;
    const cudaError_t e = cudaGraphInstantiate(&fgraph, g, 0);
    cudaGraphDestroy(g);
    CK(e);
    fgraph_scaled = scaled;
    fgraph_key = graph_key();
  }

  // One factorisation by graph replay; kGraphFallback if it must be redone
  // eagerly (a front delayed columns or failed), else the SSIDS flag.
  int factor_graph(const double* aval, bool on_device, const double* scaling) {
    cudaStream_t s = stream;
    const int nn = S->nnodes;
    aval_buf.ensure(std::max<int64_t>(S->nnz, 1));
    if (scaling) scale_buf.ensure(S->n);
    if (!fgraph || fgraph_scaled != (scaling != nullptr) || graph_key() != fgraph_key)
      build_fgraph(scaling != nullptr);
    CK(cudaEventRecord(ev[0], s));
    CK(cudaMemcpyAsync(aval_buf.p, aval, S->nnz * sizeof(double),
                       on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, s));
    if (scaling)
      CK(cudaMemcpyAsync(scale_buf.p, scaling, S->n * sizeof(double), cudaMemcpyHostToDevice, s));
    // an eager factorisation since the capture may have changed the descriptors
    hfd = fg_hfd;
    CK(cudaMemcpyAsync(d_fd, hfd.data(), nn * sizeof(FrontDesc<T>), cudaMemcpyHostToDevice, s));
    CK(cudaGraphLaunch(fgraph, s));
    note_launches(fgraph_nlaunch);
    Stats hs;
    int tcs = 0;
    CK(cudaMemcpyAsync(hst.data(), d_st, nn * sizeof(FrontState), cudaMemcpyDeviceToHost, s));
    CK(cudaMemcpyAsync(&hs, d_stats, sizeof(Stats), cudaMemcpyDeviceToHost, s));
    CK(cudaMemcpyAsync(&tcs, d_tc_status, sizeof(int), cudaMemcpyDeviceToHost, s));
    CK(cudaEventRecord(ev[1], s));
    CK(cudaStreamSynchronize(s));
    cur_aval = aval_buf.p;
    bool ok = tcs == 0;
    for (int f = 0; f < nn && ok; ++f)
      ok = hst[f].status == kDevOk && hst[f].nelim == n_[f];
    if (!ok) {
      last_zero_delay = false;
      return kGraphFallback;
    }
    const auto& co = S->copts;
    const bool use_app = co.pivot_method != 3;
    const bool tpp_all = (co.pivot_method == 3) || (co.failed_pivot_method == 1);
    int nfp = 0, nsp = 0;
    lvl_max_m.assign(S->nlev, 0);
    lvl_max_nelim.assign(S->nlev, 0);
    for (int l = 0; l < S->nlev; ++l)
      for (int f = S->lvl_start[l]; f < S->lvl_start[l + 1]; ++f) {
        nelim_[f] = hst[f].nelim;
        napp_[f] = hst[f].step;
        lvl_max_m[l] = std::max(lvl_max_m[l], m_[f]);
        lvl_max_nelim[l] = std::max(lvl_max_nelim[l], nelim_[f]);
        if (tpp_front(f)) continue;  // small leaf fronts: no pass counts
        if (use_app && napp_[f] < n_[f]) nfp += n_[f] - napp_[f];
        const bool tpp_ran = tpp_all || (m_[f] == n_[f]);
        if (!use_app) nfp += n_[f] - nelim_[f];
        else if (tpp_ran && napp_[f] < n_[f]) nsp += n_[f] - nelim_[f];
      }
    float ms = 0;
    CK(cudaEventElapsedTime(&ms, ev[0], ev[1]));
    timing[0] = ms;
    return finish_stats(hs, fg_maxfront, fg_maxsn, nfp, nsp);
  }

  int finish_stats(const Stats& hs, int maxfront, int maxsn, int nfp, int nsp) {
    stats.num_delay = hs.num_delay;
    stats.num_factor = hs.num_factor;
    stats.num_flops = hs.num_flops;
    stats.num_neg = hs.num_neg;
    stats.num_two = hs.num_two;
    stats.num_zero = hs.num_zero;
    stats.maxfront = maxfront;
    stats.maxsupernode = maxsn;
    stats.not_first_pass = nfp;
    stats.not_second_pass = nsp;
    stats.flag = 0;
    // delays left at a root of the tree are unrecoverable; a subtree root
    // with rows beyond its columns has its parent in another subtree, which
    // takes the delays with the contribution block (get_contrib)
    for (int f = 0; f < S->nnodes; ++f) {
      const int node = S->node_of[f];
      if (S->parent[node] < 0 && S->nrow[node] == S->ncol[node] && nelim_[f] < n_[f])
        stats.flag = -5;
    }
    if (stats.num_zero > 0 && stats.flag == 0) stats.flag = 7;
    if (posdef) {
      if (stats.num_neg > 0 || stats.num_zero > 0 || stats.num_two > 0) stats.flag = -6;
      stats.num_neg = 0; stats.num_two = 0; stats.num_zero = 0;
    }
    return stats.flag;
  }

  const double* cur_aval = nullptr;  // device values of the last factor
  double last_bwd_err = 0.0;
  // FP32-factor path: an FP64 factorisation of the same values, formed on the
  // GPU when the FP32 factors cannot reach the refinement target (see
  // fp64_fallback); stale after every factorisation of this handle
  std::unique_ptr<NumericBase> fb;
  bool fb_stale = true, fb_ok = false;
  bool last_scaled = false;
  std::vector<cudaEvent_t> pev;

  // side streams and events that let the size-class launches of one level's
  // small-subtree fronts run concurrently (fork from and join back to the
  // handle's stream; captured into the factorisation graph as branches)
  cudaStream_t side[kTppClasses - 1] = {};
  cudaEvent_t fork_ev = nullptr, join_ev[kTppClasses - 1] = {};

  explicit Numeric(Symbolic* s) : S(s) {
    CK(cudaSetDevice(S->device));
    CK(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
    for (auto& e : ev) CK(cudaEventCreate(&e));
    for (auto& q : side) CK(cudaStreamCreateWithFlags(&q, cudaStreamNonBlocking));
    CK(cudaEventCreateWithFlags(&fork_ev, cudaEventDisableTiming));
    for (auto& e : join_ev) CK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    const int nn = S->nnodes;
    hfd.resize(nn);
    hst.resize(nn);
    nelim_.assign(nn, 0); ndin_.assign(nn, 0); m_.assign(nn, 0); n_.assign(nn, 0);
    ld_.assign(nn, 0); doff_.assign(nn, 0); napp_.assign(nn, 0);
    {
      // the per-front descriptor, state and count arrays share one block
      auto al = [](size_t b) { return (b + 255) & ~size_t(255); };
      const size_t nn1 = std::max(nn, 1);
      const size_t b_fd = al(nn1 * sizeof(FrontDesc<T>)), b_st = al(nn1 * sizeof(FrontState));
      const size_t b_stats = al(sizeof(Stats)), b_dw = al(nn1 * sizeof(int4));
      const size_t b_tcs = al(sizeof(int)), b_nc = al(3 * nn1 * sizeof(int));
      small_buf.ensure(b_fd + b_st + b_stats + b_dw + b_tcs + b_nc);
      char* q = small_buf.p;
      d_fd = reinterpret_cast<FrontDesc<T>*>(q); q += b_fd;
      d_st = reinterpret_cast<FrontState*>(q); q += b_st;
      d_stats = reinterpret_cast<Stats*>(q); q += b_stats;
      d_dwork = reinterpret_cast<int4*>(q); q += b_dw;
      d_tc_status = reinterpret_cast<int*>(q); q += b_tcs;
      d_ncount = reinterpret_cast<int*>(q);
    }
    {
      const char* gr = getenv("SPRAL_GB300_GRAPHS");
      use_graphs = !(gr && gr[0] == '0');
      // wavefront solves (one persistent launch per pass over the tree);
      // SPRAL_GB300_SOLVE_WAVE=0 selects the per-level block-step chain
      // (48^3 Laplacian, 8 right-hand sides, FP64 factors: 6.1 ms per pass
      // against 7.3 ms)
      const char* wv = getenv("SPRAL_GB300_SOLVE_WAVE");
      use_wave = !(wv && wv[0] == '0');
      const char* wt = getenv("SPRAL_GB300_WAVE_TRACE");
      if (wt && *wt) wave_trace = wt;
      const char* bi = getenv("SPRAL_GB300_SOLVE_BINV");
      use_binv = std::is_same<T, float>::value && !(bi && bi[0] == '0');
    }
    if (std::is_same<T, float>::value) {
      const char* env = getenv("SPRAL_GB300_TENSOR_CORES");
      use_tc = !(env && env[0] == '0');
      const char* ch = getenv("SPRAL_GB300_TC_CHUNK");
      if (ch) tc_chunk = std::max(0, atoi(ch));
      const char* mc = getenv("SPRAL_GB300_TC_MIN_CM");
      if (mc) tc_min_cm = std::max(1, atoi(mc));
      else if (use_tc) tc_min_cm = autotune_tc_min_cm();
      const char* mk = getenv("SPRAL_GB300_TC_MIN_K");
      if (mk) tc_min_k = std::max(0, atoi(mk));
      const char* pn = getenv("SPRAL_GB300_PANEL");
      if (pn) panel_nb = std::max(0, atoi(pn)) / kBlk * kBlk;
      const char* pm = getenv("SPRAL_GB300_PANEL_MIN_N");
      if (pm) panel_min_n = std::max(0, atoi(pm));
    }
    contrib.ensure(std::max<int64_t>(S->contrib_total, 1));
    // factor storage estimate (no delays) + 10%
    size_t est = 0;
    for (int i = 0; i < nn; ++i) est += (size_t)((S->nrow[i] + 3) / 4 * 4) * S->ncol[i];
    farena.min_chunk = std::max<size_t>(est * sizeof(T) * 11 / 10, size_t(16) << 20);
  }
  ~Numeric() override {
    // every kernel of this handle has finished before its blocks go back to
    // the device block cache (member destructors)
    if (stream) cudaStreamSynchronize(stream);
    for (auto e : pev) cudaEventDestroy(e);
    drop_graphs();
    drop_fgraph();
    for (auto& e : ev) cudaEventDestroy(e);
    for (auto q : side)
      if (q) { cudaStreamSynchronize(q); cudaStreamDestroy(q); }
    if (fork_ev) cudaEventDestroy(fork_ev);
    for (auto e : join_ev)
      if (e) cudaEventDestroy(e);
    if (stream) cudaStreamDestroy(stream);
  }
  Symbolic* symbolic() override { return S; }

  int factor(const double* aval, bool on_device, const double* scaling,
             cudaStream_t user_stream) override {
    if (user_stream) CK(cudaStreamSynchronize(user_stream));
    solve_ready = false;
    fb_stale = true;
    last_scaled = scaling != nullptr;
    if (use_graphs && !profile && last_zero_delay) {
      stats = spral_ssids_thread_stats{};
      const int r = factor_graph(aval, on_device, scaling);
      if (r != kGraphFallback) return r;
    }
    const int r = factor_eager(aval, on_device, scaling);
    bool zero_delay = r >= 0 && S->copts.pivot_method != 3;
    for (int f = 0; f < S->nnodes && zero_delay; ++f) zero_delay = nelim_[f] == n_[f];
    last_zero_delay = zero_delay;
    return r;
  }

  int factor_eager(const double* aval, bool on_device, const double* scaling) {
    cudaStream_t s = stream;
    const int nn = S->nnodes;
    const auto& co = S->copts;
    stats = spral_ssids_thread_stats{};
    CK(cudaEventRecord(ev[0], s));
    if (on_device) {
      cur_aval = aval;
    } else {
      aval_buf.ensure(std::max<int64_t>(S->nnz, 1));
      CK(cudaMemcpyAsync(aval_buf.p, aval, S->nnz * sizeof(double), cudaMemcpyHostToDevice, s));
      cur_aval = aval_buf.p;
    }
    const double* d_scale = nullptr;
    if (scaling) {
      scale_buf.ensure(S->n);
      CK(cudaMemcpyAsync(scale_buf.p, scaling, S->n * sizeof(double), cudaMemcpyHostToDevice, s));
      d_scale = scale_buf.p;
    }
    farena.rewind();
    darena.rewind();
    iarena.rewind();
    if (profile && (int)pev.size() < 2 * S->nlev) {
      for (size_t i = pev.size(); i < (size_t)2 * S->nlev; ++i) {
        cudaEvent_t e;
        CK(cudaEventCreate(&e));
        pev.push_back(e);
      }
    }
    CK(cudaMemsetAsync(d_st, 0, nn * sizeof(FrontState), s));
    CK(cudaMemsetAsync(d_tc_status, 0, sizeof(int), s));
    CK(cudaMemsetAsync(d_stats, 0, sizeof(Stats), s));
    CK(cudaMemsetAsync(d_ncount, 0, 3 * (size_t)nn * sizeof(int), s));
    lvl_max_m.assign(S->nlev, 0);
    lvl_max_nelim.assign(S->nlev, 0);
    int maxfront = 0, maxsn = 0, nfp = 0, nsp = 0;
    double host_wait = 0.0;
    std::vector<int4> dwork;
    for (int l = 0; l < S->nlev; ++l) {
      const int f0 = S->lvl_start[l], f1 = S->lvl_start[l + 1], nf = f1 - f0;
      const int napp = app_fronts(l);
      dwork.clear();
      int max_m = 0, max_n = 0, max_cm = 0, max_ent = 0, max_app_n = 0, max_app_cm = 0;
      size_t wsW = 0, wsSwap = 0, wsLD = 0;
      for (int f = f0; f < f1; ++f) {
        const int node = S->node_of[f];
        int ndin = 0;
        for (int c : S->children[node]) {
          const int fc = S->front_of[c];
          doff_[fc] = ndin;
          const int nd = n_[fc] - nelim_[fc];
          if (nd > 0) dwork.push_back(make_int4(f, fc, S->ncol[node] + ndin, 0));
          ndin += nd;
        }
        const int m = S->nrow[node] + ndin, n = S->ncol[node] + ndin;
        const int ld = (m + 3) / 4 * 4;
        const int cm = S->nrow[node] - S->ncol[node];
        ndin_[f] = ndin; m_[f] = m; n_[f] = n; ld_[f] = ld;
        max_m = std::max(max_m, m);
        max_n = std::max(max_n, n);
        max_cm = std::max(max_cm, cm);
        max_ent = std::max<int>(max_ent, (int)(S->nptr[node + 1] - S->nptr[node]));
        wsW += (size_t)ld * kBlk;
        wsSwap += (size_t)ld * 64 + 256;
        wsLD += (size_t)std::max(cm, panel_cols(f)) * n;
        maxfront = std::max(maxfront, m);
        maxsn = std::max(maxsn, n);
      }
      for (int f = f0; f < f1; ++f) {
        if (tpp_front(f)) continue;
        max_app_n = std::max(max_app_n, n_[f]);
        max_app_cm = std::max(max_app_cm, S->nrow[S->node_of[f]] - S->ncol[S->node_of[f]]);
      }
      ws_W.ensure(wsW + 64);
      ws_swap.ensure(wsSwap + 64);
      ws_LD.ensure(wsLD + 64);
      ws_step.ensure((size_t)nf * (kBlk * kBlk + 2 * kBlk + 64));
      ws_lperm.ensure((size_t)nf * kBlk);
      size_t oW = 0, oS = 0, oL = 0;
      for (int f = f0; f < f1; ++f) {
        const int node = S->node_of[f];
        FrontDesc<T>& d = hfd[f];
        const int m = m_[f], n = n_[f], ld = ld_[f];
        d.m = m; d.n = n; d.ld = ld;
        d.nrow = S->nrow[node]; d.ncol = S->ncol[node];
        d.ndelay_in = ndin_[f];
        d.cm = S->nrow[node] - S->ncol[node];
        d.ldc = d.cm;
        d.node = node;
        d.L = (T*)farena.alloc((size_t)ld * n * sizeof(T));
        d.D = (double*)darena.alloc((size_t)2 * n * sizeof(double) + 16);
        d.perm = (int*)iarena.alloc((size_t)n * sizeof(int));
        d.opos = (int*)iarena.alloc((size_t)n * sizeof(int));
        d.C = d.cm > 0 ? contrib.p + S->contrib_off[f] : nullptr;
        d.W = ws_W.p + oW; oW += (size_t)ld * kBlk;
        d.swapbuf = ws_swap.p + oS; oS += (size_t)ld * 64 + 256;
        d.LD = ws_LD.p + oL; oL += (size_t)std::max(d.cm, panel_cols(f)) * n;
        d.step = ws_step.p + (size_t)(f - f0) * (kBlk * kBlk + 2 * kBlk + 64);
        d.lperm = ws_lperm.p + (size_t)(f - f0) * kBlk;
        d.tc = (use_tc && d.cm >= tc_min_cm && d.n >= tc_min_k) ? 1 : 0;
        d.panel = panel_cols(f);
      }
      CK(cudaMemcpyAsync(d_fd + f0, hfd.data() + f0, nf * sizeof(FrontDesc<T>),
                         cudaMemcpyHostToDevice, s));
      if (!dwork.empty())
        CK(cudaMemcpyAsync(d_dwork, dwork.data(), dwork.size() * sizeof(int4),
                           cudaMemcpyHostToDevice, s));
      const int* fr = S->d_fronts + f0;
      // assembly
      int64_t maxz = 0;
      for (int f = f0; f < f1; ++f) {
        maxz = std::max(maxz, (int64_t)ld_[f] * n_[f]);
      }
      pmark(tm(), kPhZero, s);
      launch_zero_fronts<T>(d_fd, fr, nf, (int)std::min<int64_t>(maxz, 1 << 30), s);
      pmark(tm(), kPhLoadA, s);
      launch_load_a<T>(d_fd, fr, nf, S->d_nptr, S->d_nlist, cur_aval, S->d_rlist, S->d_rptr,
                       d_scale, max_ent, s);
      pmark(tm(), kPhInitPerm, s);
      launch_init_perm<T>(d_fd, fr, nf, S->d_sptr, max_n, s);
      pmark(tm(), kPhDelays, s);
      int max_nd = 0;
      for (const int4& w : dwork) max_nd = std::max(max_nd, n_[w.y] - nelim_[w.y]);
      launch_assemble_delays<T>(d_fd, d_st, d_dwork, (int)dwork.size(), max_nd, S->d_rdir,
                                S->d_rdir_ptr, s);
      pmark(tm(), kPhAssemble, s);
      launch_assemble_contrib<T>(d_fd, S->d_cols + S->cols_start[l],
                                 S->cols_start[l + 1] - S->cols_start[l], S->d_pairs, S->d_rdir,
                                 S->d_rdir_ptr, S->lvl_colrows[l], s);
      // dense factorisation
      const bool use_app = co.pivot_method != 3;
      bool any_panel = false;
      for (int f = f0; f < f1; ++f) any_panel = any_panel || hfd[f].panel > 0;
      std::vector<int> pfl;
      if (use_app) {
        const int steps = (max_app_n + kBlk - 1) / kBlk;
        for (int st = 0; st < steps; ++st) {
          int mr = 0, tr = 0, tc = 0;
          for (int f = f0; f < f1; ++f) {
            if (tpp_front(f)) continue;
            mr = std::max(mr, m_[f] - kBlk * st);
            tr = std::max(tr, m_[f] - kBlk * (st + 1));
            const int cols = n_[f] - kBlk * (st + 1);
            tc = std::max(tc, hfd[f].panel ? std::min(cols, hfd[f].panel) : cols);
          }
          launch_app_step<T>(d_fd, d_st, fr, napp, st, std::max(mr, 1), tr, tc, co.action,
                             posdef ? 0.0 : co.u, co.small, s, tm(), posdef);
          if (any_panel) {
            panel_boundary(f0, f1, st, pfl);
            if (!pfl.empty()) {
              pmark(tm(), kPhPanel, s);
              panel_end_eager(pfl, s);
            }
          }
        }
      }
      pmark(tm(), kPhFinish, s);
      launch_app_finish<T>(d_fd, d_st, fr, nf, s);
      pmark(tm(), kPhTpp, s);
      const bool tpp_all = (co.pivot_method == 3) || (co.failed_pivot_method == 1);
      launch_tpp<T>(d_fd, d_st, fr, napp, co.action, co.u, co.small, tpp_all, s);
      if (napp < nf) launch_tpp_levels(l, s);
      pmark(tm(), kPhCalcLd, s);
      launch_calc_ld<T>(d_fd, d_st, fr, napp, max_app_cm, max_app_n, s);
      pmark(tm(), kPhContrib, s);
      if (profile) CK(cudaEventRecord(pev[2 * l], s));
      launch_contrib_gemm<T>(d_fd, d_st, fr, napp, max_app_cm, s);
      run_tc_contrib(f0, f1, s);
      if (profile) CK(cudaEventRecord(pev[2 * l + 1], s));
      pmark(tm(), kPhStats, s);
      launch_stats<T>(d_fd, d_st, fr, nf, max_n, d_stats, d_ncount, s);
      pmark(tm(), kPhHost, s);
      CK(cudaMemcpyAsync(hst.data() + f0, d_st + f0, nf * sizeof(FrontState),
                         cudaMemcpyDeviceToHost, s));
      // a launch that did not start (a configuration error) fails the
      // factorisation as a CUDA error, not as the fronts it left untouched
      CK(cudaGetLastError());
      CK(cudaStreamSynchronize(s));
      if (profile) ptimer.flush();
      bool singular = false, bad = false, notpd = false;
      for (int f = f0; f < f1; ++f) {
        if (hst[f].status == kDevSingular) singular = true;
        else if (hst[f].status == kDevNotPosdef) notpd = true;
        else if (hst[f].status != kDevOk) bad = true;
        nelim_[f] = hst[f].nelim;
        napp_[f] = hst[f].step;
        lvl_max_m[l] = std::max(lvl_max_m[l], m_[f]);
        lvl_max_nelim[l] = std::max(lvl_max_nelim[l], nelim_[f]);
        if (tpp_front(f)) continue;  // small leaf fronts: no pass counts
        if (use_app && napp_[f] < n_[f]) nfp += n_[f] - napp_[f];
        bool tpp_ran = tpp_all || (m_[f] == n_[f]);
        if (!use_app) nfp += n_[f] - nelim_[f];
        else if (tpp_ran && napp_[f] < n_[f]) nsp += n_[f] - nelim_[f];
      }
      if (profile) {
        float ms = 0;
        CK(cudaEventElapsedTime(&ms, pev[2 * l], pev[2 * l + 1]));
        // the contribution launches' fronts (the small-subtree fronts form
        // theirs inside the level-set kernel)
        double fl = 0;
        for (int f = f0; f < f1; ++f) {
          if (tpp_front(f)) continue;
          const double cm = hfd[f].cm;
          fl += (double)nelim_[f] * cm * (cm + 1.0);
        }
        if (fl > 0) { prof_ms += ms; prof_flops += fl; prof_launches += 1; }
        for (int f = f0; f < f1; ++f) {
          const double cm = hfd[f].cm;
          if (hfd[f].tc) prof_tc_flops += (double)nelim_[f] * cm * (cm + 1.0);
        }
      }
      if (use_tc) {
        int tcs = 0;
        CK(cudaMemcpy(&tcs, d_tc_status, sizeof(int), cudaMemcpyDeviceToHost));
        if (tcs != 0) bad = true;
      }
      if (notpd) { stats.flag = -6; return stats.flag; }
      if (singular) { stats.flag = -5; return stats.flag; }
      if (bad) { stats.flag = -51; return stats.flag; }
    }
    Stats hs;
    CK(cudaMemcpyAsync(&hs, d_stats, sizeof(Stats), cudaMemcpyDeviceToHost, s));
    CK(cudaEventRecord(ev[1], s));
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(s));
    float ms = 0;
    CK(cudaEventElapsedTime(&ms, ev[0], ev[1]));
    timing[0] = ms;
    (void)host_wait;
    return finish_stats(hs, maxfront, maxsn, nfp, nsp);
  }

  void prepare_solve() {
    if (solve_ready) return;
    solve_init<T>();
    const int nn = S->nnodes;
    std::vector<SolveNode<T>> sn(nn);
    std::vector<int> ch;
    size_t xl = 0;
    std::vector<size_t> xoff(nn);
    for (int f = 0; f < nn; ++f) { xoff[f] = xl; xl += (size_t)m_[f] * kSolveRhs; }
    xloc.ensure(xl + 1);
    // per front: the pivot blocks' flags, the gathered-chunk counter and the
    // finished-item counter of the wavefront passes
    auto nblk_of = [&](int f) { return (nelim_[f] + kSolveBlk - 1) / kSolveBlk; };
    auto small_of = [&](int f) { return nblk_of(f) <= 1 && m_[f] - nelim_[f] <= kWaveSmallRows; };
    auto ngat_of = [&](int f) {
      return small_of(f) ? 0 : (m_[f] + kWaveGatherRows - 1) / kWaveGatherRows;
    };
    auto ncon_of = [&](int f) { return (m_[f] - nelim_[f] + kSolveBlk - 1) / kSolveBlk; };
    auto nch_of = [&](int f) {
      return small_of(f) ? 0 : (m_[f] - nelim_[f] + kWaveL21Rows - 1) / kWaveL21Rows;
    };
    std::vector<size_t> flag_off(nn + 1, 0), l21_off(nn + 1, 0);
    for (int f = 0; f < nn; ++f) {
      flag_off[f + 1] = flag_off[f] + 2 * nblk_of(f) + 2;
      l21_off[f + 1] = l21_off[f] + (size_t)nblk_of(f) * nch_of(f) * kSolveBlk * kSolveRhs;
    }
    wave_l21p.ensure(std::max<size_t>(l21_off[nn], 1));
    const bool binv = use_wave && use_binv;
    std::vector<size_t> binv_off(nn + 1, 0);
    std::vector<int2> bblocks;
    if (binv) {
      for (int f = 0; f < nn; ++f) {
        binv_off[f + 1] = binv_off[f] + (size_t)nblk_of(f) * kSolveBlk * kSolveBlk;
        for (int b = 0; b < nblk_of(f); ++b) bblocks.push_back(make_int2(f, b));
      }
      wave_binv.ensure(std::max<size_t>(binv_off[nn], 1));
      binv_blocks.ensure(std::max<size_t>(bblocks.size(), 1));
      if (!bblocks.empty())
        CK(cudaMemcpyAsync(binv_blocks.p, bblocks.data(), bblocks.size() * sizeof(int2),
                           cudaMemcpyHostToDevice, stream));
    }
    wave_nflags = flag_off[nn];
    wave_flags.ensure(std::max<size_t>(wave_nflags, 1));
    wave_ints.ensure(3);
    {
      // forward: levels from the leaves; per level the gathers and small
      // fronts, the pivot blocks by block index across the level's fronts,
      // then the contribution row blocks.  Backward: levels from the root;
      // the gathers and small fronts, then the pivot blocks from the last.
      std::vector<int2> items;
      for (int l = 0; l < S->nlev; ++l) {
        const int f0 = S->lvl_start[l], f1 = S->lvl_start[l + 1];
        int mb = 0;
        for (int f = f0; f < f1; ++f) {
          if (small_of(f)) {
            items.push_back(make_int2(f, kWaveSmall));
            continue;
          }
          for (int g = 0; g < ngat_of(f); ++g) items.push_back(make_int2(f, kWaveGather + g));
          mb = std::max(mb, nblk_of(f));
        }
        for (int b = 0; b < mb; ++b)
          for (int f = f0; f < f1; ++f)
            if (!small_of(f) && b < nblk_of(f)) items.push_back(make_int2(f, b));
        for (int f = f0; f < f1; ++f)
          if (!small_of(f))
            for (int k = 0; k < ncon_of(f); ++k) items.push_back(make_int2(f, kWaveContrib + k));
      }
      wave_nfwd = (int)items.size();
      wave_nsmall = 0;
      for (int f = 0; f < nn; ++f) wave_nsmall += small_of(f) ? 1 : 0;
      for (int l = S->nlev - 1; l >= 0; --l) {
        const int f0 = S->lvl_start[l], f1 = S->lvl_start[l + 1];
        int mb = 0;
        for (int f = f0; f < f1; ++f) {
          if (small_of(f)) {
            items.push_back(make_int2(f, kWaveSmall));
            continue;
          }
          for (int g = 0; g < ngat_of(f); ++g) items.push_back(make_int2(f, kWaveGather + g));
          mb = std::max(mb, nblk_of(f));
        }
        for (int b = mb - 1; b >= 0; --b)
          for (int f = f0; f < f1; ++f)
            if (b < nblk_of(f))
              for (int c = 0; c < nch_of(f); ++c)
                items.push_back(make_int2(f, kWaveL21 + b * nch_of(f) + c));
        for (int b = mb - 1; b >= 0; --b)
          for (int f = f0; f < f1; ++f)
            if (!small_of(f) && b < nblk_of(f)) items.push_back(make_int2(f, b));
      }
      wave_nbwd = (int)items.size() - wave_nfwd;
      wave_items.ensure(std::max<size_t>(items.size(), 1));
      if (!items.empty())
        CK(cudaMemcpyAsync(wave_items.p, items.data(), items.size() * sizeof(int2),
                           cudaMemcpyHostToDevice, stream));
      CK(cudaMemsetAsync(wave_ints.p, 0, sizeof(int), stream));  // status
    }
    for (int f = 0; f < nn; ++f) {
      const int node = S->node_of[f];
      SolveNode<T>& q = sn[f];
      q.flag = wave_flags.p + flag_off[f];
      q.l21p = wave_l21p.p + l21_off[f];
      q.binv = binv ? wave_binv.p + binv_off[f] : nullptr;
      q.nblk = nblk_of(f);
      q.ngat = ngat_of(f);
      q.nch = nch_of(f);
      q.nitf = small_of(f) ? 1 : q.ngat + q.nblk + ncon_of(f);
      q.nitb = small_of(f) ? 1 : q.ngat + q.nblk * (1 + q.nch);
      q.parent = S->parent[node] >= 0 ? S->front_of[S->parent[node]] : -1;
      q.L = hfd[f].L; q.D = hfd[f].D; q.perm = hfd[f].perm; q.opos = hfd[f].opos;
      q.rows = S->d_rlist + S->rptr[node];
      q.rdir = S->d_rdir + S->rdir_ptr_h[node];
      q.xloc = xloc.p + xoff[f];
      q.gp = S->d_gp + S->gp_off[f];
      q.m = m_[f]; q.n = n_[f]; q.ld = ld_[f]; q.nelim = nelim_[f];
      q.ncol = S->ncol[node]; q.nrow = S->nrow[node]; q.ndelay_in = ndin_[f];
      q.cm = S->nrow[node] - S->ncol[node];
      q.sptr0 = S->sptr[node];
      q.child_beg = (int)ch.size();
      for (int c : S->children[node]) ch.push_back(S->front_of[c]);
      q.child_end = (int)ch.size();
      q.doff = doff_[f];
    }
    // the tables keep their device addresses across refactorisations
    sn_buf.ensure(std::max<size_t>(sn.size(), 1));
    ch_buf.ensure(std::max<size_t>(ch.size(), 1));
    d_sn = sn_buf.p;
    d_children = ch_buf.p;
    CK(cudaMemcpyAsync(d_sn, sn.data(), sn.size() * sizeof(SolveNode<T>), cudaMemcpyHostToDevice,
                       stream));
    if (binv) launch_diag_inv<T>(d_sn, binv_blocks.p, (int)bblocks.size(), stream);
    if (!ch.empty())
      CK(cudaMemcpyAsync(d_children, ch.data(), ch.size() * sizeof(int), cudaMemcpyHostToDevice,
                         stream));
    if (S->d_front_group) {
      group_active.ensure((size_t)S->ngroups);
      CK(cudaMemsetAsync(group_active.p, 1, (size_t)S->ngroups, stream));
    }
    CK(cudaStreamSynchronize(stream));
    // signature of everything a captured solve sequence depends on
    uint64_t h = 1469598103934665603ull;
    auto mix = [&](uint64_t v) { h = (h ^ v) * 1099511628211ull; };
    for (int l = 0; l < S->nlev; ++l) { mix((uint64_t)lvl_max_m[l]); mix((uint64_t)lvl_max_nelim[l]); }
    mix((uint64_t)(uintptr_t)d_sn); mix((uint64_t)(uintptr_t)d_children);
    mix((uint64_t)(uintptr_t)xloc.p);
    mix((uint64_t)(uintptr_t)wave_items.p); mix((uint64_t)(uintptr_t)wave_flags.p);
    mix((uint64_t)(uintptr_t)wave_ints.p); mix((uint64_t)(uintptr_t)wave_l21p.p);
    mix((uint64_t)(uintptr_t)wave_binv.p); mix((uint64_t)binv);
    mix((uint64_t)wave_nfwd); mix((uint64_t)wave_nbwd);
    mix((uint64_t)(uintptr_t)S->d_front_group); mix((uint64_t)(uintptr_t)group_active.p);
    if (h != solve_sig) drop_graphs();
    solve_sig = h;
    solve_ready = true;
  }

  // enqueue one solve pass of q <= kSolveRhs right-hand sides on s.
  // Jobs: 0 full, 1 fwd, 2 diag, 3 bwd, 4 diag+bwd (L D L^T); 5 fwd and
  // 6 bwd with the Cholesky factor L_chol = L D^(1/2) (posdef).
  void enqueue_solve(int job, int q, double* xp, int ldx, cudaStream_t s) {
    const bool fwd = (job == 0 || job == 1 || job == 5);
    const bool diag = (job == 0 || job == 2 || job == 4);
    const bool bwd = (job == 0 || job == 3 || job == 4 || job == 6);
    const int diag_mode = diag ? 1 : (job == 6 ? 2 : 0);
    int* wstatus = wave_ints.p;
    if (fwd) {
      if (use_wave) {
        CK(cudaMemsetAsync(wave_flags.p, 0, std::max<size_t>(wave_nflags, 1) * sizeof(int), s));
        CK(cudaMemsetAsync(wave_ints.p + 1, 0, sizeof(int), s));
        pmark(tm(), kPhFwdUpdate, s);
        launch_fwd_tree<T>(d_sn, d_children, S->d_pairs, wave_pass(true), q, xp, ldx, job == 5,
                           wstatus, s);
      } else {
        for (int l = 0; l < S->nlev; ++l) {
          const int f0 = S->lvl_start[l], nf = S->lvl_start[l + 1] - f0;
          const int* fr = S->d_fronts + f0;
          pmark(tm(), kPhFwdGather, s);
          launch_fwd_gather<T>(d_sn, fr, nf, d_children, S->d_pairs, xp, ldx, q, lvl_max_m[l],
                               s);
          launch_fwd_steps<T>(d_sn, fr, nf, lvl_max_nelim[l], lvl_max_m[l], q, xp, ldx, job == 5,
                              s, tm());
        }
      }
    }
    if (diag || bwd) {
      if (use_wave && bwd) {
        CK(cudaMemsetAsync(wave_flags.p, 0, std::max<size_t>(wave_nflags, 1) * sizeof(int), s));
        CK(cudaMemsetAsync(wave_ints.p + 2, 0, sizeof(int), s));
        pmark(tm(), kPhBwdUpdate, s);
        launch_bwd_tree<T>(d_sn, wave_pass(false), xp, ldx, q, diag_mode, wstatus, s);
      } else {
        for (int l = S->nlev - 1; l >= 0; --l) {
          const int f0 = S->lvl_start[l], nf = S->lvl_start[l + 1] - f0;
          launch_bwd<T>(d_sn, S->d_fronts + f0, nf, xp, ldx, q, lvl_max_m[l], lvl_max_nelim[l],
                        diag_mode, bwd, s, tm());
        }
      }
    }
  }

  // the same pass through a captured graph (captured on first use)
  void run_solve(int job, int q, double* xp, int ldx, cudaStream_t s) {
    if (!wave_trace.empty()) {
      enqueue_solve(job, q, xp, ldx, s);
      dump_wave_trace(s);
      return;
    }
    if (profile || !use_graphs) { enqueue_solve(job, q, xp, ldx, s); return; }
    for (auto& g : sgraphs)
      if (g.job == job && g.q == q && g.x == xp && g.ldx == ldx && g.sig == solve_sig) {
        CK(cudaGraphLaunch(g.exec, s));
        note_launches(g.nlaunch);
        return;
      }
    if (sgraphs.size() >= 32) {
      cudaGraphExecDestroy(sgraphs.front().exec);
      sgraphs.erase(sgraphs.begin());
    }
    std::lock_guard<std::mutex> lock(g_capture_mutex);
    const long long l0 = t_launches;
    cudaGraph_t g = nullptr;
    CK(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
    try {
      enqueue_solve(job, q, xp, ldx, s);
    } catch (...) {
      cudaStreamEndCapture(s, &g);
      if (g) cudaGraphDestroy(g);
      g_launches -= t_launches - l0;
      t_launches = l0;
      throw;
    }
    CK(cudaStreamEndCapture(s, &g));
    const int nl = (int)(t_launches - l0);
    g_launches -= nl;  // counted at each replay instead
    t_launches = l0;
    cudaGraphExec_t ge = nullptr;
    const cudaError_t e = cudaGraphInstantiate(&ge, g, 0);
    cudaGraphDestroy(g);
    CK(e);
    sgraphs.push_back({job, q, ldx, xp, solve_sig, ge, nl});
    CK(cudaGraphLaunch(ge, s));
    note_launches(nl);
  }

  int solve_dev(int job, int nrhs, double* x, int ldx, cudaStream_t us) override {
    prepare_solve();
    cudaStream_t s = stream;
    if (us) CK(cudaStreamSynchronize(us));
    for (int r0 = 0; r0 < nrhs; r0 += kSolveRhs) {
      const int q = std::min(kSolveRhs, nrhs - r0);
      run_solve(job, q, x + (int64_t)r0 * ldx, ldx, s);
    }
    pmark(tm(), kPhHost, s);
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(s));
    if (profile) ptimer.flush();
    if (use_wave) {
      // a wavefront wait that gave up (never expected) fails the solve
      int wst = 0;
      CK(cudaMemcpy(&wst, wave_ints.p, sizeof(int), cudaMemcpyDeviceToHost));
      if (wst != 0) {
        CK(cudaMemset(wave_ints.p, 0, sizeof(int)));
        throw CudaFail{cudaErrorLaunchTimeout, __LINE__};
      }
    }
    return 0;
  }

  // full solve with FP64 iterative refinement; x (host) holds b on entry
  int solve_refined(int nrhs, double* xh, int ldx, int* iters) override {
    const int n = S->n;
    cudaStream_t s = stream;
    int itmax = 0;
    for (int r0 = 0; r0 < nrhs; r0 += kSolveRhs) {
      const int q = std::min(kSolveRhs, nrhs - r0);
      bbuf.ensure((size_t)n * q + 1);
      xbuf.ensure((size_t)n * q + 1);
      rbuf.ensure((size_t)n * q + 1);
      nbuf.ensure(q + (size_t)std::max(S->ngroups, 1) * (1 + 3 * kSolveRhs) + 8);
      for (int r = 0; r < q; ++r)
        CK(cudaMemcpyAsync(bbuf.p + (size_t)r * n, xh + (size_t)(r0 + r) * ldx,
                           n * sizeof(double), cudaMemcpyHostToDevice, s));
      CK(cudaMemcpyAsync(xbuf.p, bbuf.p, (size_t)n * q * sizeof(double),
                         cudaMemcpyDeviceToDevice, s));
      solve_dev(0, q, xbuf.p, n, nullptr);
      int it = refine_dev(q, xbuf.p, bbuf.p, n);
      if (NumericBase* f64 = fp64_fallback()) {
        int it64 = 0;
        double bwd64 = 0;
        f64->solve_refined_dev(q, bbuf.p, xbuf.p, n, &it64, &bwd64);
        it += it64;
        last_bwd_err = bwd64;
      }
      itmax = std::max(itmax, it);
      for (int r = 0; r < q; ++r)
        CK(cudaMemcpyAsync(xh + (size_t)(r0 + r) * ldx, xbuf.p + (size_t)r * n,
                           n * sizeof(double), cudaMemcpyDeviceToHost, s));
    }
    CK(cudaStreamSynchronize(s));
    if (iters) *iters = itmax;
    return 0;
  }

  // full solve + refinement with b and x in device memory (n x nrhs, ld)
  int solve_refined_dev(int nrhs, const double* b, double* x, int ld, int* iters,
                        double* bwd) override {
    int itmax = 0;
    double worst = 0;
    for (int r0 = 0; r0 < nrhs; r0 += kSolveRhs) {
      const int q = std::min(kSolveRhs, nrhs - r0);
      double* xp = x + (size_t)r0 * ld;
      const double* bp = b + (size_t)r0 * ld;
      CK(cudaMemcpy2DAsync(xp, ld * sizeof(double), bp, ld * sizeof(double),
                           S->n * sizeof(double), q, cudaMemcpyDeviceToDevice, stream));
      solve_dev(0, q, xp, ld, nullptr);
      int it = refine_dev(q, xp, bp, ld);
      if (NumericBase* f64 = fp64_fallback()) {
        int it64 = 0;
        double bwd64 = 0;
        f64->solve_refined_dev(q, bp, xp, ld, &it64, &bwd64);
        it += it64;
        last_bwd_err = bwd64;
      }
      itmax = std::max(itmax, it);
      worst = std::max(worst, last_bwd_err);
    }
    if (iters) *iters = itmax;
    if (bwd) *bwd = worst;
    return 0;
  }

  // FP64 fallback of the FP32-factor path.  When FP32 factors cannot bring
  // the backward error of a refined solve to the target (the refinement
  // stalled or ran out of steps: the matrix is too ill-conditioned for FP32
  // factors), the same values are factored again in FP64 on the GPU, once
  // per factorisation of this handle, and the right-hand sides are solved
  // and refined with those factors.  The FP64 factorisation's statistics
  // (inertia, delays) replace the FP32 ones.  Returns the FP64 handle to
  // solve with, or nullptr when no fallback is needed (FP64 handles, or the
  // target was met).
  NumericBase* fp64_fallback() {
    if (!std::is_same<T, float>::value) return nullptr;
    if (S->gopts.no_fp64_fallback) return nullptr;
    if (!(last_bwd_err > S->gopts.refine_tol)) return nullptr;
    if (!fb) {
      fb.reset(new Numeric<double>(S));
      fb->posdef = posdef;
      fb->precision = 0;
    }
    if (fb_stale) {
      std::vector<double> sc;
      if (last_scaled) {
        sc.resize(S->n);
        CK(cudaMemcpy(sc.data(), scale_buf.p, S->n * sizeof(double), cudaMemcpyDeviceToHost));
      }
      const int r = fb->factor(cur_aval, true, last_scaled ? sc.data() : nullptr, nullptr);
      fb_stale = false;
      fb_ok = r >= 0;
      ++fallbacks;
      stats = fb->stats;  // its flag tells a failed FP64 factorisation
    }
    return fb_ok ? fb.get() : nullptr;
  }

  // refinement of x (device, n x q, ld) against b; returns steps taken
  int refine_dev(int q, double* x, const double* b, int ld) {
    const int n = S->n;
    cudaStream_t s = stream;
    rbuf.ensure((size_t)ld * q + 1);
    nbuf.ensure(q + (size_t)std::max(S->ngroups, 1) * (1 + 3 * kSolveRhs) + 8);
    std::vector<double> h(q);
    int it = 0;
    const int maxit = S->gopts.max_refine;
    last_refine_q = q;
    group_prev.clear();
    for (;; ++it) {
      pmark(tm(), kPhResid, s);
      launch_resid_bwd_err(S->d_aptr, S->d_acol, S->d_asrc, cur_aval, n, x, b, rbuf.p, q, ld,
                           nbuf.p, S->d_row_group, S->ngroups, s);
      pmark(tm(), kPhHost, s);
      CK(cudaMemcpyAsync(h.data(), nbuf.p, q * sizeof(double), cudaMemcpyDeviceToHost, s));
      CK(cudaStreamSynchronize(s));
      if (profile) ptimer.flush();
      double worst = 0;
      for (int r = 0; r < q; ++r) worst = std::max(worst, h[r]);
      // stop at the target, after max_refine steps, or when a step did not
      // halve the backward error (the factors' precision cannot reach it).
      // Row groups whose caller handles the misses itself (no FP64
      // fallback): stalled only once no group above the target halved its
      // own error, so the other groups finish their refinement.
      bool stalled = it > 0 && !(worst < 0.5 * last_bwd_err);
      bool masked = false;
      // row groups judged one by one: FP32 factors whose caller handles
      // the misses (no FP64 fallback here), and FP64 factors
      const bool by_group = S->gopts.no_fp64_fallback || std::is_same<T, double>::value;
      if (S->d_row_group && by_group && worst > S->gopts.refine_tol) {
        last_refine_q = q;
        std::vector<double> ge(S->ngroups);
        group_bwd_errors(ge.data(), S->ngroups);
        if (S->gopts.no_fp64_fallback && it > 0 && group_prev.size() == ge.size()) {
          stalled = true;
          for (size_t g = 0; g < ge.size() && stalled; ++g)
            if (ge[g] > S->gopts.refine_tol && ge[g] < 0.5 * group_prev[g]) stalled = false;
        }
        // the next step solves only for the groups above the target: the
        // wavefront passes skip the others' trees and the update leaves
        // their rows as they are (their errors stay those just measured)
        if (use_wave && S->d_front_group && group_active.p) {
          active_h.resize(ge.size());
          for (size_t g = 0; g < ge.size(); ++g) active_h[g] = ge[g] > S->gopts.refine_tol;
          CK(cudaMemcpyAsync(group_active.p, active_h.data(), active_h.size(),
                             cudaMemcpyHostToDevice, s));
          masked = true;
        }
        group_prev.swap(ge);
      }
      last_bwd_err = worst;
      if (!(worst > S->gopts.refine_tol) || it >= maxit || stalled) break;
      solve_dev(0, q, rbuf.p, ld, nullptr);
      pmark(tm(), kPhAxpy, s);
      launch_axpy(n, q, ld, x, rbuf.p, s, masked ? S->d_row_group : nullptr,
                  masked ? group_active.p : nullptr);
      pmark(tm(), kPhHost, s);
    }
    // later solves are for every group
    if (S->d_front_group && group_active.p)
      CK(cudaMemsetAsync(group_active.p, 1, (size_t)S->ngroups, s));
    return it;
  }
  std::vector<unsigned char> active_h;  // host copy of the refinement's group mask

  cudaStream_t get_stream() const override { return stream; }

  int last_refine_q = 0;  // right-hand sides of the last refinement's residuals in nbuf
  std::vector<double> group_prev;  // per row group, the previous refinement step's error
  int group_bwd_errors(double* out, int ngroups) override {
    if (!S->d_row_group || last_refine_q <= 0 || ngroups != S->ngroups) return -1;
    std::vector<double> w((size_t)ngroups * kResStride);
    CK(cudaMemcpy(w.data(), nbuf.p + last_refine_q, w.size() * sizeof(double),
                  cudaMemcpyDeviceToHost));
    for (int g = 0; g < ngroups; ++g) {
      const double* wg = w.data() + (size_t)g * kResStride;
      double e = 0.0;
      for (int r = 0; r < last_refine_q; ++r) {
        const double den = wg[0] * wg[1 + 3 * r] + wg[2 + 3 * r];
        e = std::max(e, den > 0 ? wg[3 + 3 * r] / den : 0.0);
      }
      out[g] = e;
    }
    return 0;
  }

  int node_inertia(int* out) override {
    CK(cudaMemcpy(out, d_ncount, 3 * (size_t)S->nnodes * sizeof(int), cudaMemcpyDeviceToHost));
    return 0;
  }

  int debug_front(int node, int* info, double* Lout, double* Dout, int* Pout) override {
    const int f = S->front_of[node];
    info[0] = m_[f]; info[1] = n_[f]; info[2] = nelim_[f]; info[3] = ndin_[f]; info[4] = ld_[f];
    if (Lout) {
      std::vector<T> tmp((size_t)ld_[f] * n_[f]);
      CK(cudaMemcpy(tmp.data(), hfd[f].L, tmp.size() * sizeof(T), cudaMemcpyDeviceToHost));
      for (int c = 0; c < n_[f]; ++c)
        for (int r = 0; r < m_[f]; ++r) Lout[(size_t)c * m_[f] + r] = (double)tmp[(size_t)c * ld_[f] + r];
    }
    if (Dout) CK(cudaMemcpy(Dout, hfd[f].D, 2 * n_[f] * sizeof(double), cudaMemcpyDeviceToHost));
    if (Pout) CK(cudaMemcpy(Pout, hfd[f].perm, n_[f] * sizeof(int), cudaMemcpyDeviceToHost));
    return 0;
  }

  void download_dp(std::vector<double>& D, std::vector<int>& P, int f) {
    D.resize(2 * (size_t)n_[f]);
    P.resize(n_[f]);
    CK(cudaMemcpy(D.data(), hfd[f].D, D.size() * sizeof(double), cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(P.data(), hfd[f].perm, P.size() * sizeof(int), cudaMemcpyDeviceToHost));
  }

  // The subtree root's generalised element for a parent in another subtree,
  // as transfer_contrib (src/ssids/gpu/factor.f90:155-221) hands it over and
  // NumericSubtree::get_contrib (src/ssids/cpu/NumericSubtree.hxx:518-532)
  // describes it: the cm x cm contribution block (full, leading dimension
  // cm; the device holds its lower triangle, mirrored here), the 1-based
  // rows it belongs to, and the delayed columns (1-based perm entries; each
  // column from its diagonal down: the ndelay x ndelay block, then the cm
  // contribution rows; leading dimension cm + ndelay).  FP32 factors are
  // widened to FP64.  Returns 0 or -51.
  int get_contrib() override {
    contrib_val.clear(); contrib_delay.clear(); contrib_rlist.clear(); contrib_perm.clear();
    contrib_n = contrib_ndelay = contrib_lddelay = 0;
    const int root = S->nnodes - 1;
    if (root < 0 || nelim_.empty()) return 0;
    const int f = S->front_of[root];
    const int cm = S->nrow[root] - S->ncol[root];
    const int nel = nelim_[f], nd = n_[f] - nel;
    if (cudaStreamSynchronize(stream) != cudaSuccess) { cudaGetLastError(); return -51; }
    contrib_n = cm;
    if (cm > 0) {
      std::vector<T> c((size_t)cm * cm);
      if (cudaMemcpy(c.data(), hfd[f].C, c.size() * sizeof(T), cudaMemcpyDeviceToHost) !=
          cudaSuccess) { cudaGetLastError(); return -51; }
      contrib_val.resize((size_t)cm * cm);
      for (int j = 0; j < cm; ++j)
        for (int i = j; i < cm; ++i) {
          const double v = (double)c[(size_t)j * hfd[f].ldc + i];
          contrib_val[(size_t)j * cm + i] = v;
          contrib_val[(size_t)i * cm + j] = v;
        }
      contrib_rlist.resize(cm);
      const int64_t r0 = S->rptr[root] + S->ncol[root];
      for (int i = 0; i < cm; ++i) contrib_rlist[i] = S->rlist[r0 + i] + 1;
    }
    if (nd > 0) {
      std::vector<int> P(n_[f]);
      std::vector<T> Lc((size_t)ld_[f] * nd);
      if (cudaMemcpy(P.data(), hfd[f].perm, P.size() * sizeof(int), cudaMemcpyDeviceToHost) !=
              cudaSuccess ||
          cudaMemcpy(Lc.data(), hfd[f].L + (size_t)nel * ld_[f], Lc.size() * sizeof(T),
                     cudaMemcpyDeviceToHost) != cudaSuccess) {
        cudaGetLastError();
        return -51;
      }
      contrib_ndelay = nd;
      contrib_lddelay = cm + nd;
      contrib_perm.resize(nd);
      contrib_delay.resize((size_t)contrib_lddelay * nd);
      for (int i = 0; i < nd; ++i) {
        contrib_perm[i] = P[nel + i] + 1;
        for (int r = 0; r < contrib_lddelay; ++r)
          contrib_delay[(size_t)i * contrib_lddelay + r] = (double)Lc[(size_t)i * ld_[f] + nel + r];
      }
    }
    return 0;
  }

  // node order as the CPU enquire (NumericSubtree.hxx:402-445)
  void enquire(int* piv_order, double* d) override {
    std::vector<double> D;
    std::vector<int> P;
    if (posdef) {
      // diagonal of L_chol = L D^(1/2), node by node (NumericSubtree.hxx:424-431)
      for (int node = 0; node < S->nnodes; ++node) {
        const int f = S->front_of[node];
        download_dp(D, P, f);
        for (int i = 0; i < nelim_[f]; ++i) *d++ = 1.0 / std::sqrt(D[2 * i]);
      }
      return;
    }
    int piv = 0;
    for (int node = 0; node < S->nnodes; ++node) {
      const int f = S->front_of[node];
      download_dp(D, P, f);
      const int ne = nelim_[f];
      for (int i = 0; i < ne;) {
        if (i + 1 == ne || std::isfinite(D[2 * i + 2])) {
          if (piv_order) piv_order[P[i]] = piv++;
          if (d) { *d++ = D[2 * i]; *d++ = 0.0; }
          i += 1;
        } else {
          if (piv_order) { piv_order[P[i]] = -(piv++); piv_order[P[i + 1]] = -(piv++); }
          if (d) { *d++ = D[2 * i]; *d++ = D[2 * i + 1]; *d++ = D[2 * i + 3]; *d++ = 0.0; }
          i += 2;
        }
      }
    }
  }

  void alter(const double* d) override {
    std::vector<double> D;
    std::vector<int> P;
    for (int node = 0; node < S->nnodes; ++node) {
      const int f = S->front_of[node];
      download_dp(D, P, f);
      const int ne = nelim_[f];
      for (int i = 0; i < ne;) {
        if (i + 1 == ne || std::isfinite(D[2 * i + 2])) {
          D[2 * i] = *d++; d++;
          i += 1;
        } else {
          D[2 * i] = *d++; D[2 * i + 1] = *d++; D[2 * i + 3] = *d++; d++;
          i += 2;
        }
      }
      CK(cudaMemcpy(hfd[f].D, D.data(), D.size() * sizeof(double), cudaMemcpyHostToDevice));
    }
  }
};

}  // namespace ssids300

using namespace ssids300;

namespace {
int map_cuda_error(const CudaFail& e, spral_ssids_thread_stats* st) {
  if (st) st->flag = (e.err == cudaErrorMemoryAllocation) ? -50 : -51;
  fprintf(stderr, "spral_gb300: CUDA error %d (%s) at numeric.cu:%d\n", (int)e.err,
          cudaGetErrorString(e.err), e.line);
  cudaGetLastError();
  return (e.err == cudaErrorMemoryAllocation) ? -50 : -51;
}
}  // namespace

extern "C" {

void spral_ssids_gpu_inject_alloc_failure(int after) { g_alloc_fail_after.store(after); }

int spral_ssids_gpu_wave_timeout_probe(int rounds) { return wave_timeout_probe(rounds); }

int spral_ssids_gpu_device_count(void) {
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess) { cudaGetLastError(); return 0; }
  return n;
}

void* spral_ssids_gpu_create_symbolic_subtree(int device, int n, int sa, int en, const int* sptr,
                                              const int* sparent, const int64_t* rptr,
                                              const int* rlist, const int64_t* nptr,
                                              const int64_t* nlist,
                                              const struct spral_ssids_cpu_factor_options* options) {
  try {
    if (cudaSetDevice(device) != cudaSuccess) { cudaGetLastError(); return nullptr; }
    return build_symbolic(device, n, sa, en, sptr, sparent, rptr, rlist, nptr, nlist, options);
  } catch (CudaFail const& e) {
    map_cuda_error(e, nullptr);
    return nullptr;
  } catch (std::bad_alloc const&) {
    return nullptr;
  }
}

void spral_ssids_gpu_destroy_symbolic_subtree(void* symbolic) {
  delete static_cast<Symbolic*>(symbolic);
}

int spral_ssids_gpu_set_options(void* symbolic, const struct spral_ssids_gpu_options* opts) {
  if (!symbolic || !opts) return -1;
  static_cast<Symbolic*>(symbolic)->gopts = *opts;
  return 0;
}

void* spral_ssids_gpu_create_num_subtree_dbl(bool posdef, const void* symbolic, const double* aval,
                                             const double* scaling, void** child_contrib,
                                             const struct spral_ssids_cpu_factor_options* options,
                                             struct spral_ssids_thread_stats* stats) {
  Symbolic* S = const_cast<Symbolic*>(static_cast<const Symbolic*>(symbolic));
  if (stats) *stats = spral_ssids_thread_stats{};
  if (!S) { if (stats) stats->flag = -51; return nullptr; }
  if (child_contrib) { /* inter-subtree contributions are not supported */ }
  if (options) S->copts = *options;
  NumericBase* N = nullptr;
  try {
    CK(cudaSetDevice(S->device));
    if (S->gopts.precision == 1) N = new Numeric<float>(S);
    else N = new Numeric<double>(S);
    N->posdef = posdef;
    N->precision = S->gopts.precision;
    N->factor(aval, false, scaling, nullptr);
    if (stats) *stats = N->stats;
    return N;
  } catch (CudaFail const& e) {
    map_cuda_error(e, stats);
    if (N) N->stats.flag = stats ? stats->flag : -51;
    return N;
  } catch (std::bad_alloc const&) {
    if (stats) stats->flag = -50;
    return N;
  }
}

void spral_ssids_gpu_destroy_num_subtree_dbl(bool posdef, void* numeric) {
  (void)posdef;
  delete static_cast<NumericBase*>(numeric);
}

int spral_ssids_gpu_refactor_dev(void* numeric, const double* aval_dev,
                                 struct spral_ssids_thread_stats* stats, void* stream) {
  NumericBase* N = static_cast<NumericBase*>(numeric);
  try {
    int fl = N->factor(aval_dev, true, nullptr, (cudaStream_t)stream);
    if (stats) *stats = N->stats;
    return fl;
  } catch (CudaFail const& e) {
    return map_cuda_error(e, stats);
  } catch (std::bad_alloc const&) {
    return -50;
  }
}

int spral_ssids_gpu_refactor(void* numeric, const double* aval, const double* scaling,
                             struct spral_ssids_thread_stats* stats) {
  NumericBase* N = static_cast<NumericBase*>(numeric);
  try {
    int fl = N->factor(aval, false, scaling, nullptr);
    if (stats) *stats = N->stats;
    return fl;
  } catch (CudaFail const& e) {
    return map_cuda_error(e, stats);
  } catch (std::bad_alloc const&) {
    return -50;
  }
}

static int host_solve(const void* numeric, int job, int nrhs, double* x, int ldx) {
  NumericBase* N = const_cast<NumericBase*>(static_cast<const NumericBase*>(numeric));
  Symbolic* S = N->symbolic();
  const int n = S->n;
  try {
    CK(cudaSetDevice(S->device));
    // a per-handle device buffer and the handle's stream: no allocation and
    // no device-wide synchronisation per call
    N->hsolve.ensure(std::max<size_t>((size_t)n * nrhs, 1));
    double* dx = N->hsolve.p;
    cudaStream_t s = N->get_stream();
    for (int r = 0; r < nrhs; ++r)
      CK(cudaMemcpyAsync(dx + (size_t)r * n, x + (size_t)r * ldx, n * sizeof(double),
                         cudaMemcpyHostToDevice, s));
    N->solve_dev(job, nrhs, dx, n, nullptr);
    for (int r = 0; r < nrhs; ++r)
      CK(cudaMemcpyAsync(x + (size_t)r * ldx, dx + (size_t)r * n, n * sizeof(double),
                         cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    return 0;
  } catch (CudaFail const& e) {
    return map_cuda_error(e, nullptr);
  }
}

int spral_ssids_gpu_subtree_solve_fwd_dbl(bool posdef, const void* numeric, int nrhs, double* x,
                                          int ldx) {
  // posdef: L_chol y = b with L_chol = L D^(1/2) (cholesky_solve_fwd)
  return host_solve(numeric, posdef ? 5 : 1, nrhs, x, ldx);
}
int spral_ssids_gpu_subtree_solve_diag_dbl(bool posdef, const void* numeric, int nrhs, double* x,
                                           int ldx) {
  // the diagonal solve is a no-op for posdef (NumericSubtree.hxx:343)
  if (posdef) return 0;
  return host_solve(numeric, 2, nrhs, x, ldx);
}
int spral_ssids_gpu_subtree_solve_diag_bwd_dbl(bool posdef, const void* numeric, int nrhs,
                                               double* x, int ldx) {
  return host_solve(numeric, posdef ? 6 : 4, nrhs, x, ldx);
}
int spral_ssids_gpu_subtree_solve_bwd_dbl(bool posdef, const void* numeric, int nrhs, double* x,
                                          int ldx) {
  // posdef: L_chol^T x = y (cholesky_solve_bwd)
  return host_solve(numeric, posdef ? 6 : 3, nrhs, x, ldx);
}

int spral_ssids_gpu_solve_dev(void* numeric, int job, int nrhs, double* x_dev, int ldx,
                              void* stream) {
  NumericBase* N = static_cast<NumericBase*>(numeric);
  try {
    return N->solve_dev(job, nrhs, x_dev, ldx, (cudaStream_t)stream);
  } catch (CudaFail const& e) {
    return map_cuda_error(e, nullptr);
  }
}

int spral_ssids_gpu_solve_refined(void* numeric, int nrhs, double* x, int ldx, int* iters) {
  NumericBase* N = static_cast<NumericBase*>(numeric);
  try {
    return N->solve_refined(nrhs, x, ldx, iters);
  } catch (CudaFail const& e) {
    return map_cuda_error(e, nullptr);
  }
}

void spral_ssids_gpu_subtree_enquire_dbl(bool posdef, const void* numeric, int* piv_order,
                                         double* d) {
  (void)posdef;
  NumericBase* N = const_cast<NumericBase*>(static_cast<const NumericBase*>(numeric));
  try {
    N->enquire(piv_order, d);
  } catch (CudaFail const& e) {
    map_cuda_error(e, nullptr);
  }
}

void spral_ssids_gpu_subtree_alter_dbl(bool posdef, void* numeric, const double* d) {
  (void)posdef;
  try {
    static_cast<NumericBase*>(numeric)->alter(d);
  } catch (CudaFail const& e) {
    map_cuda_error(e, nullptr);
  }
}

int spral_ssids_gpu_subtree_get_contrib_dbl(bool posdef, void* numeric, int* n,
                                            const double** val, int* ldval, const int** rlist,
                                            int* ndelay, const int** delay_perm,
                                            const double** delay_val, int* lddelay) {
  (void)posdef;
  auto* N = static_cast<NumericBase*>(numeric);
  if (!N) return -1;
  const int rc = N->get_contrib();
  *n = N->contrib_n;
  *ldval = N->contrib_n;
  *val = N->contrib_val.empty() ? nullptr : N->contrib_val.data();
  *rlist = N->contrib_rlist.empty() ? nullptr : N->contrib_rlist.data();
  *ndelay = N->contrib_ndelay;
  *delay_perm = N->contrib_perm.empty() ? nullptr : N->contrib_perm.data();
  *delay_val = N->contrib_delay.empty() ? nullptr : N->contrib_delay.data();
  *lddelay = N->contrib_lddelay;
  return rc;
}

void spral_ssids_gpu_subtree_free_contrib_dbl(bool posdef, void* numeric) {
  (void)posdef;
  auto* N = static_cast<NumericBase*>(numeric);
  if (!N) return;
  std::vector<double>().swap(N->contrib_val);
  std::vector<double>().swap(N->contrib_delay);
  std::vector<int>().swap(N->contrib_rlist);
  std::vector<int>().swap(N->contrib_perm);
  N->contrib_n = N->contrib_ndelay = N->contrib_lddelay = 0;
}

int spral_ssids_gpu_debug_front(const void* numeric, int node, int* info, double* L, double* D,
                                int* perm) {
  NumericBase* N = const_cast<NumericBase*>(static_cast<const NumericBase*>(numeric));
  try {
    return N->debug_front(node, info, L, D, perm);
  } catch (CudaFail const& e) {
    return map_cuda_error(e, nullptr);
  }
}

int spral_ssids_gpu_last_timing(const void* numeric, double* out) {
  const NumericBase* N = static_cast<const NumericBase*>(numeric);
  for (int i = 0; i < 5; ++i) out[i] = N->timing[i];
  return 5;
}

}  // extern "C"

extern "C" {

/* Profiling and bench support (no reference counterpart). */
long long spral_ssids_gpu_launch_count(void) { return ssids300::g_launches.load(); }

void spral_ssids_gpu_set_profiling(void* numeric, int on) {
  auto* N = static_cast<ssids300::NumericBase*>(numeric);
  N->profile = on != 0;
  N->prof_ms = 0;
  N->prof_flops = 0;
  N->prof_launches = 0;
  N->prof_tc_ms = 0;
  N->prof_tc_flops = 0;
  N->prof_tc_launches = 0;
  N->ptimer.reset();
}

/* Per-phase device time (ms) and interval counts accumulated while profiling
 * (32 phases; see the Phase enum of the implementation). */
void spral_ssids_gpu_phase_times(const void* numeric, double* ms, long long* counts) {
  auto* N = static_cast<const ssids300::NumericBase*>(numeric);
  for (int i = 0; i < ssids300::kPhCount; ++i) {
    ms[i] = N->ptimer.ms[i];
    counts[i] = N->ptimer.cnt[i];
  }
}

/* Smallest contribution block (rows) formed on the tensor cores by the
 * FP32-factor path on the current device, as measured by the autotuner. */
int spral_ssids_gpu_tc_crossover(void) {
  try {
    return ssids300::autotune_tc_min_cm();
  } catch (...) {
    return -51;
  }
}

/* The autotuner's table for the current device (measured on first use, or
 * read from the tune cache): out = [tc_min_cm, nb, m_0, bn_0, ...].  Returns
 * the number of ints written, -1 if nout is too small, -51 on a CUDA error. */
int spral_ssids_gpu_group_bwd_errors(const void* numeric, double* out, int ngroups) {
  auto* N = const_cast<NumericBase*>(static_cast<const NumericBase*>(numeric));
  if (!N || !out || ngroups <= 0) return -1;
  try {
    return N->group_bwd_errors(out, ngroups);
  } catch (...) {
    return -51;
  }
}

int spral_ssids_gpu_tune_table(int* out, int nout) {
  try {
    const ssids300::TuneTable t = ssids300::autotune_device();
    const int need = 2 + 2 * t.nb;
    if (!out || nout < need) return -1;
    out[0] = t.tc_min_cm;
    out[1] = t.nb;
    for (int i = 0; i < t.nb; ++i) { out[2 + 2 * i] = t.bucket_m[i]; out[3 + 2 * i] = t.bn[i]; }
    return need;
  } catch (...) {
    return -51;
  }
}

/* The current device's key in the tune cache.  Returns its length, or -1. */
int spral_ssids_gpu_tune_device_key(char* buf, int cap) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) { cudaGetLastError(); return -1; }
  const std::string k = ssids300::tune_device_key(dev);
  if (!buf || cap <= (int)k.size()) return -1;
  std::snprintf(buf, (size_t)cap, "%s", k.c_str());
  return (int)k.size();
}

/* The contribution update of one front on the SIMT kernel, on the caller's
 * device buffers and stream: C -= L21 (L21 D)^T on the lower triangle of
 * the cm x cm block C (leading dimension cm), where the front's L is
 * (cm + k) x k with leading dimension ld (rows 0..k-1 the pivots, rows k..
 * the L21 block) and LD = L21 D is cm x k with leading dimension cm.  dbl
 * selects FP64 (1) or FP32 (0) buffers; the update is applied reps times
 * back to back (reps >= 1).  Returns 0, -1 on a bad argument or -51 on a
 * CUDA error. */
int spral_ssids_gpu_contrib_update(int dbl, const void* l, int ld, const void* l21d, void* c,
                                   int cm, int k, int reps, void* stream) {
  using namespace ssids300;
  if (cm < 0 || k < 0 || reps < 1 || ld < cm + k || !l || !l21d || !c) return -1;
  if (cm == 0 || k == 0) return 0;
  auto s = static_cast<cudaStream_t>(stream);
  auto run = [&](auto* tag) -> int {
    using T = std::remove_pointer_t<decltype(tag)>;
    struct Blk {
      FrontDesc<T> fd;
      FrontState st;
      int front;
    } h{};
    h.fd.L = const_cast<T*>(static_cast<const T*>(l));
    h.fd.LD = const_cast<T*>(static_cast<const T*>(l21d));
    h.fd.C = static_cast<T*>(c);
    h.fd.m = cm + k; h.fd.n = k; h.fd.ld = ld; h.fd.cm = cm; h.fd.ldc = cm;
    h.fd.nrow = cm + k; h.fd.ncol = k;
    h.st.nelim = k;
    h.front = 0;
    Blk* d = nullptr;
    if (cudaMallocAsync(reinterpret_cast<void**>(&d), sizeof(Blk), s) != cudaSuccess) return -51;
    cudaMemcpyAsync(d, &h, sizeof(Blk), cudaMemcpyHostToDevice, s);
    for (int r = 0; r < reps; ++r) launch_contrib_gemm<T>(&d->fd, &d->st, &d->front, 1, cm, s);
    cudaFreeAsync(d, s);
    // h is read by the copy above before the stream drains
    if (cudaStreamSynchronize(s) != cudaSuccess) return -51;
    return cudaGetLastError() == cudaSuccess ? 0 : -51;
  };
  return dbl ? run(static_cast<double*>(nullptr)) : run(static_cast<float*>(nullptr));
}

/* Free and total device memory of the current device (cudaMemGetInfo);
 * used by callers that admit work by memory.  Returns 0 or -51. */
int spral_ssids_gpu_mem_info(size_t* free_bytes, size_t* total_bytes) {
  if (cudaMemGetInfo(free_bytes, total_bytes) != cudaSuccess) {
    cudaGetLastError();
    return -51;
  }
  int dev = 0;
  if (cudaGetDevice(&dev) == cudaSuccess) *free_bytes += ssids300::cache_bytes(dev);
  return 0;
}

void spral_ssids_gpu_release_cache(void) {
  int dev = 0;
  if (cudaGetDevice(&dev) == cudaSuccess) ssids300::cache_release(dev);
  else cudaGetLastError();
}

/* Per-node inertia of the last factorisation: out[3*node + {0, 1, 2}] =
 * (negative eigenvalues, 2x2 pivots, zero pivots) of the node's D (0-based
 * node numbering of the symbolic subtree). */
int spral_ssids_gpu_node_inertia(const void* numeric, int* out) {
  auto* N = const_cast<ssids300::NumericBase*>(static_cast<const ssids300::NumericBase*>(numeric));
  try {
    return N->node_inertia(out);
  } catch (...) {
    return -51;
  }
}

/* out[0] = contribution-update time (ms) summed over profiled factors,
 * out[1] = its algorithmic flops, out[2] = number of timed levels;
 * out[3..5] = the same for the tensor-core GEMM kernel alone (flops counted
 * as the FP32 update it performs, not the 3x split products). */
void spral_ssids_gpu_profile_stats(const void* numeric, double* out) {
  auto* N = static_cast<const ssids300::NumericBase*>(numeric);
  out[0] = N->prof_ms;
  out[1] = N->prof_flops;
  out[2] = (double)N->prof_launches;
  out[3] = N->prof_tc_ms;
  out[4] = N->prof_tc_flops;
  out[5] = (double)N->prof_tc_launches;
}

int spral_ssids_gpu_solve_refined_dev(void* numeric, int nrhs, const double* b_dev, double* x_dev,
                                      int ld, int* iters, double* bwd_err) {
  auto* N = static_cast<ssids300::NumericBase*>(numeric);
  try {
    return N->solve_refined_dev(nrhs, b_dev, x_dev, ld, iters, bwd_err);
  } catch (ssids300::CudaFail const& e) {
    return map_cuda_error(e, nullptr);
  }
}

int spral_ssids_gpu_set_row_groups(void* symbolic, int ngroups, const int* row_group) {
  Symbolic* S = static_cast<Symbolic*>(symbolic);
  if (!S) return -1;
  try {
    CK(cudaSetDevice(S->device));
    if (ngroups <= 0 || !row_group) {
      cudaFree(S->d_row_group);
      cudaFree(S->d_front_group);
      S->d_row_group = nullptr;
      S->d_front_group = nullptr;
      S->ngroups = 0;
      return 0;
    }
    for (int i = 0; i < S->n; ++i)
      if (row_group[i] < 0 || row_group[i] >= ngroups) return -2;
    // a front's group: its columns' when they and its parent's share one
    // (the groups are the trees of a forest, e.g. the matrices of a batch);
    // otherwise no front groups, and the refinement never skips a group
    std::vector<int> fg(std::max(S->nnodes, 1), 0);
    bool trees = true;
    for (int i = 0; i < S->nnodes && trees; ++i) {
      const int g = S->sptr[i] < S->n ? row_group[S->sptr[i]] : 0;
      for (int c = S->sptr[i]; c < S->sptr[i + 1] && trees; ++c) trees = row_group[c] == g;
      const int p = S->parent[i];
      if (trees && p >= 0 && S->sptr[p] < S->n) trees = row_group[S->sptr[p]] == g;
      fg[S->front_of[i]] = g;
    }
    int* d = nullptr;
    int* dfg = nullptr;
    CK(cudaMalloc(&d, std::max(S->n, 1) * sizeof(int)));
    cudaError_t e = trees ? cudaMalloc(&dfg, fg.size() * sizeof(int)) : cudaSuccess;
    if (e == cudaSuccess) e = cudaMemcpy(d, row_group, S->n * sizeof(int), cudaMemcpyHostToDevice);
    if (e == cudaSuccess && dfg)
      e = cudaMemcpy(dfg, fg.data(), fg.size() * sizeof(int), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) { cudaFree(d); cudaFree(dfg); CK(e); }
    cudaFree(S->d_row_group);
    cudaFree(S->d_front_group);
    S->d_row_group = d;
    S->d_front_group = dfg;
    S->ngroups = ngroups;
    return 0;
  } catch (CudaFail const& e) {
    return -51;
  }
}

int spral_ssids_gpu_fp64_fallbacks(const void* numeric, struct spral_ssids_thread_stats* stats) {
  const auto* N = static_cast<const NumericBase*>(numeric);
  if (!N) return -1;
  if (stats) *stats = N->stats;
  return N->fallbacks;
}

int spral_ssids_gpu_recip_probe(const double* x_dev, double* y_dev, int n) {
  ssids300::launch_recip_probe(x_dev, y_dev, n, 0);
  return (int)cudaDeviceSynchronize();
}

double spral_ssids_gpu_fp64_peak_tflops(int device) {
  try {
    return ssids300::fp64_peak_tflops(device);
  } catch (ssids300::CudaFail const& e) {
    map_cuda_error(e, nullptr);
    return 0.0;
  }
}

}  // extern "C"
