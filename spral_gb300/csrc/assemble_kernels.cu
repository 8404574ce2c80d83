// Assembly of a level's fronts on the device:
//   k_load_a          L(front) <- A via the analyse map (nptr, nlist);
//                     add_a_block, src/ssids/cpu/kernels/assemble.hxx:46-75
//                     (GPU reference: cu_load_nodes, src/ssids/gpu/kernels/
//                     assemble.cu:42)
//   k_init_perm       own pivots and the identity "original position" map
//   k_assemble_delays delayed columns of each child go after the parent's
//                     own columns (assemble.hxx:227-263; add_delays,
//                     assemble.cu:248)
//   k_assemble_contrib extend-add of child contribution blocks into the
//                     parent's fully-summed columns and contribution block
//                     (assemble_expected / assemble_expected_contrib,
//                     assemble.hxx:86-141; GPU reference assemble.cu:174).
//                     One CTA per parent column: the children that map into
//                     that column are added in a fixed order, each child
//                     column read contiguously and scattered through the
//                     child->parent row map (rdir), so the result is
//                     deterministic without atomics.  The contribution
//                     block receives nothing else (A and the delayed
//                     columns go to the fully-summed part), so every one of
//                     its columns has a CTA that first zeroes the column's
//                     lower part and then adds: the zeros stay in L2 for the
//                     adds, and each entry crosses HBM once as a write.
#include "ssids_gpu.cuh"

namespace ssids300 {

namespace {

template <typename T>
__global__ void k_load_a(const FrontDesc<T>* fds, const int* fronts, const int64_t* nptr,
                         const int64_t* nlist, const double* aval, const int* rlist,
                         const int64_t* rptr, const double* scaling) {
  const int f = fronts[blockIdx.y];
  const FrontDesc<T> fd = fds[f];
  const int64_t beg = nptr[fd.node], end = nptr[fd.node + 1];
  for (int64_t k = beg + blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < end;
       k += (int64_t)gridDim.x * blockDim.x) {
    const int64_t src = nlist[2 * k], dest = nlist[2 * k + 1];
    const int c = (int)(dest / fd.nrow);
    const int r0 = (int)(dest % fd.nrow);
    const int r = (r0 >= fd.ncol) ? r0 + fd.ndelay_in : r0;
    double v = aval[src];
    if (scaling) {
      const int* rl = rlist + rptr[fd.node];
      v *= scaling[rl[r0]] * scaling[rl[c]];
    }
    fd.L[(int64_t)c * fd.ld + r] = (T)v;
  }
}

template <typename T>
__global__ void k_init_perm(const FrontDesc<T>* fds, const int* fronts, const int* sptr) {
  const int f = fronts[blockIdx.y];
  const FrontDesc<T> fd = fds[f];
  const int s0 = sptr[fd.node];
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < fd.n; i += gridDim.x * blockDim.x) {
    if (i < fd.ncol) fd.perm[i] = s0 + i;
    fd.opos[i] = i;
  }
}

// work[i] = (parent front, child front, first delay column in parent, 0);
// grid (column groups, work items): CTA x takes the child's delayed columns
// x, x + gridDim.x, ... (each column independent of the others)
template <typename T>
__global__ void k_assemble_delays(const FrontDesc<T>* fds, const FrontState* sts, const int4* work,
                                  const int* rdir, const int64_t* rdir_ptr) {
  const int4 w = work[blockIdx.y];
  const FrontDesc<T> fp = fds[w.x];
  const FrontDesc<T> fc = fds[w.y];
  const int nel = sts[w.y].nelim;
  const int nd = fc.n - nel;
  const int dcol0 = w.z;
  const int* rd = rdir + rdir_ptr[fc.node];
  const int cmc = fc.m - fc.n;
  for (int i = blockIdx.x; i < nd; i += gridDim.x) {
    const int sc = nel + i, dcol = dcol0 + i;
    const T* src = fc.L + (int64_t)sc * fc.ld;
    for (int j = i + threadIdx.x; j < nd; j += blockDim.x)
      fp.L[(int64_t)dcol * fp.ld + dcol0 + j] = src[nel + j];
    for (int ic = threadIdx.x; ic < cmc; ic += blockDim.x) {
      const int Q = rd[ic];
      const T v = src[fc.n + ic];
      if (Q < fp.ncol) fp.L[(int64_t)Q * fp.ld + dcol] = v;
      else fp.L[(int64_t)dcol * fp.ld + Q + fp.ndelay_in] = v;
    }
    if (threadIdx.x == 0) fp.perm[dcol] = fc.perm[sc];
  }
}

// cols[i] = (parent front, parent position P, first pair, end pair);
// pairs[q] = (child front, child contribution column jc).  One parent
// column per CTA, or per warp (WARP: levels whose columns are short, so that
// four columns of small fronts share a CTA instead of one leaving most of
// its threads idle); the same additions in the same order either way.
template <typename T, bool WARP>
__global__ void k_assemble_contrib(const FrontDesc<T>* fds, const int4* cols, int ncols,
                                   const int2* pairs, const int* rdir, const int64_t* rdir_ptr) {
  const int col = WARP ? blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5) : blockIdx.x;
  if (col >= ncols) return;  // warp-uniform
  const int tid = WARP ? (threadIdx.x & 31) : threadIdx.x;
  const int nt = WARP ? 32 : blockDim.x;
  auto sync = [] {
    if (WARP) __syncwarp();
    else __syncthreads();
  };
  const int4 cw = cols[col];
  const FrontDesc<T> fp = fds[cw.x];
  const int P = cw.y;
  const bool into_l = P < fp.ncol;
  T* dst = into_l ? fp.L + (int64_t)P * fp.ld : fp.C + (int64_t)(P - fp.ncol) * fp.ldc;
  if (!into_l) {
    for (int r = P - fp.ncol + tid; r < fp.cm; r += nt) dst[r] = T(0);
    sync();
  }
  // A contribution-block column fed by one child receives each entry at most
  // once: it is stored (v + 0 has the bits of 0 + v, -0 included) instead of
  // read back and added.
  const bool store = !into_l && cw.w - cw.z == 1;
  constexpr int U = 8;  // entries per thread in flight
  for (int q = cw.z; q < cw.w; ++q) {
    const int2 pr = pairs[q];
    const FrontDesc<T> fc = fds[pr.x];
    const int jc = pr.y;
    const int cmc = fc.cm;
    const T* src = fc.C + (int64_t)jc * fc.ldc;
    const int* rd = rdir + rdir_ptr[fc.node];
    for (int ic0 = jc + tid; ic0 < cmc; ic0 += U * nt) {
      int Q[U];
      T v[U];
#pragma unroll
      for (int u = 0; u < U; ++u) {
        const int ic = ic0 + u * nt;
        Q[u] = ic < cmc ? rd[ic] : -1;
        v[u] = ic < cmc ? src[ic] : T(0);
      }
#pragma unroll
      for (int u = 0; u < U; ++u) {
        if (Q[u] < 0) continue;
        int r;
        if (into_l) r = (Q[u] < fp.ncol) ? Q[u] : Q[u] + fp.ndelay_in;
        else r = Q[u] - fp.ncol;
        if (store) dst[r] = v[u] + T(0);
        else dst[r] += v[u];
      }
    }
    sync();
  }
}

inline int cdiv(int64_t a, int b) { return (int)((a + b - 1) / b); }

}  // namespace

template <typename T>
void launch_load_a(const FrontDesc<T>* fd, const int* fronts, int nf, const int64_t* nptr,
                   const int64_t* nlist, const double* aval, const int* rlist,
                   const int64_t* rptr, const double* scaling, int max_entries, cudaStream_t s) {
  if (nf <= 0 || max_entries <= 0) return;
  int gx = std::max(1, std::min(cdiv(max_entries, 256), 512));
  { k_load_a<T><<<dim3(gx, nf), 256, 0, s>>>(fd, fronts, nptr, nlist, aval, rlist, rptr, scaling); note_launches(1); }
}
template <typename T>
void launch_init_perm(const FrontDesc<T>* fd, const int* fronts, int nf, const int* sptr,
                      int max_n, cudaStream_t s) {
  if (nf <= 0) return;
  int gx = std::max(1, std::min(cdiv(max_n, 256), 64));
  { k_init_perm<T><<<dim3(gx, nf), 256, 0, s>>>(fd, fronts, sptr); note_launches(1); }
}
template <typename T>
void launch_assemble_delays(const FrontDesc<T>* fd, const FrontState* st, const int4* work,
                            int nwork, int max_nd, const int* rdir, const int64_t* rdir_ptr,
                            cudaStream_t s) {
  if (nwork <= 0) return;
  const int gx = std::max(1, std::min(max_nd, 256));
  { k_assemble_delays<T><<<dim3(gx, nwork), 128, 0, s>>>(fd, st, work, rdir, rdir_ptr); note_launches(1); }
}
// columns at most this long (rows of the parent's or a child's contribution
// block) take a warp each
constexpr int kAssembleWarpRows = 256;

template <typename T>
void launch_assemble_contrib(const FrontDesc<T>* fd, const int4* cols, int ncols,
                             const int2* pairs, const int* rdir, const int64_t* rdir_ptr,
                             int max_rows, cudaStream_t s) {
  if (ncols <= 0) return;
  if (max_rows <= kAssembleWarpRows)
    k_assemble_contrib<T, true><<<cdiv(ncols, 4), 128, 0, s>>>(fd, cols, ncols, pairs, rdir,
                                                               rdir_ptr);
  else
    k_assemble_contrib<T, false><<<ncols, 128, 0, s>>>(fd, cols, ncols, pairs, rdir, rdir_ptr);
  note_launches(1);
}

#define INST(T)                                                                                  \
  template void launch_load_a<T>(const FrontDesc<T>*, const int*, int, const int64_t*,          \
                                 const int64_t*, const double*, const int*, const int64_t*,      \
                                 const double*, int, cudaStream_t);                              \
  template void launch_init_perm<T>(const FrontDesc<T>*, const int*, int, const int*, int,      \
                                    cudaStream_t);                                               \
  template void launch_assemble_delays<T>(const FrontDesc<T>*, const FrontState*, const int4*,  \
                                          int, int, const int*, const int64_t*, cudaStream_t);   \
  template void launch_assemble_contrib<T>(const FrontDesc<T>*, const int4*, int, const int2*,  \
                                           const int*, const int64_t*, int, cudaStream_t);
INST(double)
INST(float)
#undef INST

}  // namespace ssids300
