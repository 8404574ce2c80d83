// Host-side symbolic analyse for SSIDS, restated in C++.
//
// SSIDS's analyse phase is Fortran (src/core_analyse.f90, src/ssids/anal.F90)
// and produces the arrays that the numeric subtree constructors consume:
// sptr, sparent, rptr, rlist, nptr, nlist (all 1-based, as the Fortran passes
// them across the C boundary, src/ssids/cpu/SymbolicSubtree.hxx:20).  The GPU
// numeric path plugs in below that boundary, so this file only exists to feed
// it the same inputs the Fortran analyse would:
//   * elimination tree (Liu)                 core_analyse.f90:173  find_etree
//   * postorder                              core_analyse.f90:233  find_postorder
//   * column counts                          core_analyse.f90:387  find_col_counts
//   * supernode amalgamation (nemin rule)    core_analyse.f90:536  find_supernodes,
//                                            :806 do_merge, :832 merge_nodes
//   * row lists + sort                       core_analyse.f90:911, :1007
//   * predicted factor size / flops          core_analyse.f90:856  calc_stats
//   * A -> front map (nptr, nlist)           anal.F90:1137         build_map
// The elimination tree and column counts are computed with different (simpler)
// algorithms than the Fortran; the resulting tree, supernode partition and
// row lists are the same objects.
//
// The ordering itself (METIS in the reference) is an input: callers supply
// `order` (position of each variable in the pivot sequence).  A minimum-degree
// ordering is provided for general sparse test matrices.
#include <algorithm>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <new>
#include <set>
#include <vector>

namespace {

struct Akeep {
  int n = 0;
  int nnodes = 0;
  std::vector<int> sptr;      // nnodes+1, 1-based pivot indices
  std::vector<int> sparent;   // nnodes, 1-based node index (nnodes+1 = root)
  std::vector<int64_t> rptr;  // nnodes+1, 1-based into rlist
  std::vector<int> rlist;     // 1-based pivot indices
  std::vector<int64_t> nptr;  // nnodes+1, 1-based into nlist pairs
  std::vector<int64_t> nlist; // 2 x nnz pairs (src, dest), 1-based
  std::vector<int> invp;      // invp[p] = variable (0-based) at pivot p (0-based)
  int64_t nfact = 0, nflops = 0;
  int maxfront = 0, maxsupernode = 0;
};

// Full symmetric adjacency (no diagonal) from a lower-triangle CSC.
void full_pattern(int n, const int64_t* ptr, const int* row,
                  std::vector<int64_t>& fptr, std::vector<int>& frow) {
  std::vector<int64_t> cnt(n + 1, 0);
  for (int c = 0; c < n; ++c)
    for (int64_t k = ptr[c]; k < ptr[c + 1]; ++k) {
      int r = row[k];
      if (r == c) continue;
      cnt[r + 1]++;
      cnt[c + 1]++;
    }
  fptr.assign(n + 1, 0);
  for (int i = 0; i < n; ++i) fptr[i + 1] = fptr[i] + cnt[i + 1];
  frow.assign(fptr[n], 0);
  std::vector<int64_t> pos(fptr.begin(), fptr.end() - 1);
  for (int c = 0; c < n; ++c)
    for (int64_t k = ptr[c]; k < ptr[c + 1]; ++k) {
      int r = row[k];
      if (r == c) continue;
      frow[pos[r]++] = c;
      frow[pos[c]++] = r;
    }
}

}  // namespace

extern "C" {

// Analyse a symmetric matrix given by its lower triangle in CSC form
// (0-based ptr[n+1], row[nnz]; row[k] >= column).  order[i] is the pivot
// position (0-based) of variable i; NULL means natural order.  Returns an
// opaque handle or NULL with *info set (<0 error).
void* spral_gb300_analyse(int n, const int64_t* ptr, const int* row,
                          const int* order, int nemin, int* info) {
  *info = 0;
  Akeep* ak = nullptr;
  try {
    ak = new Akeep();
    ak->n = n;
    std::vector<int64_t> fptr;
    std::vector<int> frow;
    full_pattern(n, ptr, row, fptr, frow);

    std::vector<int> perm(n), invp(n);
    for (int i = 0; i < n; ++i) perm[i] = order ? order[i] : i;
    for (int i = 0; i < n; ++i) {
      if (perm[i] < 0 || perm[i] >= n) { *info = -9; delete ak; return nullptr; }
      invp[perm[i]] = i;
    }

    // --- elimination tree (Liu, with path compression) ---
    std::vector<int> parent(n, n), vf(n, n);
    for (int piv = 0; piv < n; ++piv) {
      int v = invp[piv];
      for (int64_t k = fptr[v]; k < fptr[v + 1]; ++k) {
        int j = perm[frow[k]];
        if (j >= piv) continue;
        int a = j;
        while (vf[a] < piv) { int nxt = vf[a]; vf[a] = piv; a = nxt; }
        if (vf[a] == piv) continue;
        parent[a] = piv;
        vf[a] = piv;
      }
    }

    // --- postorder (children visited in increasing order) ---
    {
      std::vector<int> head(n + 1, -1), next(n, -1);
      for (int v = n - 1; v >= 0; --v) { next[v] = head[parent[v]]; head[parent[v]] = v; }
      std::vector<int> post(n), stack;
      stack.reserve(n + 1);
      std::vector<int> it(n + 1);
      for (int v = 0; v <= n; ++v) it[v] = head[v];
      int cnt = 0;
      stack.push_back(n);
      while (!stack.empty()) {
        int v = stack.back();
        int c = it[v];
        if (c != -1) { it[v] = next[c]; stack.push_back(c); }
        else { stack.pop_back(); if (v != n) post[v] = cnt++; }
      }
      std::vector<int> nparent(n);
      for (int v = 0; v < n; ++v) nparent[post[v]] = (parent[v] == n) ? n : post[parent[v]];
      parent.swap(nparent);
      for (int i = 0; i < n; ++i) perm[i] = post[perm[i]];
      for (int i = 0; i < n; ++i) invp[perm[i]] = i;
    }

    // --- column counts by row-subtree traversal: O(nnz(L)) ---
    std::vector<int> cc(n, 1), mark(n, -1);
    for (int i = 0; i < n; ++i) {
      mark[i] = i;
      int v = invp[i];
      for (int64_t k = fptr[v]; k < fptr[v + 1]; ++k) {
        int a = perm[frow[k]];
        if (a >= i) continue;
        while (mark[a] != i) { cc[a]++; mark[a] = i; a = parent[a]; }
      }
    }

    // --- supernode amalgamation (find_supernodes / do_merge semantics) ---
    const long long HUGE_LL = (1LL << 62);
    std::vector<int> nelim(n + 1, 1), nvert(n + 1, 1), vhead(n + 1, -1), vnext(n + 1, -1);
    std::vector<long long> ezero(n + 1, 0);
    ezero[n] = HUGE_LL;
    nelim[n] = n + 1 + nemin;
    std::vector<char> keep(n, 0);
    {
      std::vector<int> chead(n + 1, -1), cnext(n + 1, -1);
      for (int v = n - 1; v >= 0; --v) { cnext[v] = chead[parent[v]]; chead[parent[v]] = v; }
      std::vector<int> kids;
      for (int par = 0; par <= n; ++par) {
        kids.clear();
        for (int c = chead[par]; c != -1; c = cnext[c]) kids.push_back(c);
        std::stable_sort(kids.begin(), kids.end(),
                         [&](int a, int b) { return cc[a] > cc[b]; });
        for (int node : kids) {
          bool merge;
          if (ezero[par] == HUGE_LL) merge = false;
          else {
            int ccp = (par < n) ? cc[par] : 0;
            merge = (ccp == cc[node] - 1 && nelim[par] == 1) ||
                    (nelim[par] < nemin && nelim[node] < nemin);
          }
          if (merge) {
            vnext[node] = vhead[par];
            vhead[par] = node;
            ezero[par] += ezero[node] +
                (long long)(cc[par] - 1 + nelim[par] - cc[node] + 1) * nelim[par];
            nelim[par] += nelim[node];
            nvert[par] += nvert[node];
            keep[node] = 0;
          } else {
            keep[node] = 1;
          }
        }
      }
    }
    std::vector<int> sperm(n), vmap(n + 1), npar, scc;
    std::vector<int> sptr0;
    {
      int v = 0;
      std::vector<int> stack;
      for (int node = 0; node < n; ++node) {
        if (!keep[node]) continue;
        int s = (int)sptr0.size();
        sptr0.push_back(v);
        npar.push_back(parent[node]);
        scc.push_back(cc[node] + nelim[node] - 1);
        v += nvert[node];
        int k = v;
        stack.clear();
        stack.push_back(node);
        while (!stack.empty()) {
          int i = stack.back();
          stack.pop_back();
          sperm[i] = --k;
          vmap[i] = s;
          if (vnext[i] != -1) stack.push_back(vnext[i]);
          if (vhead[i] != -1) stack.push_back(vhead[i]);
        }
      }
      sptr0.push_back(v);
    }
    int nnodes = (int)npar.size();
    vmap[n] = nnodes;
    for (int i = 0; i < n; ++i) perm[i] = sperm[perm[i]];
    for (int i = 0; i < n; ++i) invp[perm[i]] = i;

    // --- row lists ---
    std::vector<int> spar(nnodes);
    for (int s = 0; s < nnodes; ++s) spar[s] = vmap[npar[s]];
    std::vector<int> chead(nnodes + 1, -1), cnext(nnodes + 1, -1);
    for (int s = nnodes - 1; s >= 0; --s) { cnext[s] = chead[spar[s]]; chead[spar[s]] = s; }
    std::vector<int64_t> rptr0(nnodes + 1, 0);
    std::vector<int> rl;
    rl.reserve(std::max<int64_t>(n, 1));
    std::vector<int> seen(n, -1);
    for (int s = 0; s < nnodes; ++s) {
      int64_t start = (int64_t)rl.size();
      rptr0[s] = start;
      for (int p = sptr0[s]; p < sptr0[s + 1]; ++p) { seen[p] = s; rl.push_back(p); }
      for (int c = chead[s]; c != -1; c = cnext[c])
        for (int64_t k = rptr0[c]; k < rptr0[c + 1]; ++k) {
          int j = rl[k];
          if (j < sptr0[s] || seen[j] == s) continue;
          seen[j] = s;
          rl.push_back(j);
        }
      for (int p = sptr0[s]; p < sptr0[s + 1]; ++p) {
        int v = invp[p];
        for (int64_t k = fptr[v]; k < fptr[v + 1]; ++k) {
          int j = perm[frow[k]];
          if (j < p || seen[j] == s) continue;
          seen[j] = s;
          rl.push_back(j);
        }
      }
      std::sort(rl.begin() + start, rl.end());
    }
    rptr0[nnodes] = (int64_t)rl.size();

    // --- statistics (calc_stats) ---
    int64_t nfact = 0, nflops = 0;
    int maxfront = 0, maxsn = 0;
    for (int s = 0; s < nnodes; ++s) {
      int64_t ne = sptr0[s + 1] - sptr0[s];
      int64_t blkm = rptr0[s + 1] - rptr0[s];
      int64_t m = blkm - ne;
      nfact += ne * (ne + 1) / 2 + ne * m;
      for (int64_t j = 1; j <= ne; ++j) nflops += (m + j) * (m + j);
      maxfront = std::max<int>(maxfront, (int)blkm);
      maxsn = std::max<int>(maxsn, (int)ne);
    }

    // --- build_map: A (lower CSC) -> front positions ---
    int64_t nnz = ptr[n];
    std::vector<int64_t> tptr(n + 1, 0);
    for (int c = 0; c < n; ++c)
      for (int64_t k = ptr[c]; k < ptr[c + 1]; ++k)
        if (row[k] != c) tptr[row[k] + 1]++;
    for (int i = 0; i < n; ++i) tptr[i + 1] += tptr[i];
    std::vector<int> trow(tptr[n]);
    std::vector<int64_t> torig(tptr[n]);
    {
      std::vector<int64_t> pos(tptr.begin(), tptr.end() - 1);
      for (int c = 0; c < n; ++c)
        for (int64_t k = ptr[c]; k < ptr[c + 1]; ++k) {
          int r = row[k];
          if (r == c) continue;
          trow[pos[r]] = c;
          torig[pos[r]] = k;
          pos[r]++;
        }
    }
    std::vector<int64_t> nptr0(nnodes + 1, 0);
    std::vector<int64_t> nl;
    nl.reserve(2 * nnz);
    std::vector<int> lmap(n, 0);
    for (int s = 0; s < nnodes; ++s) {
      int64_t blkm = rptr0[s + 1] - rptr0[s];
      nptr0[s] = (int64_t)(nl.size() / 2);
      for (int64_t k = rptr0[s]; k < rptr0[s + 1]; ++k) lmap[rl[k]] = (int)(k - rptr0[s]);
      for (int j = sptr0[s]; j < sptr0[s + 1]; ++j) {
        int col = invp[j];
        for (int64_t k = tptr[col]; k < tptr[col + 1]; ++k) {
          int kp = perm[trow[k]];
          if (kp < j) continue;
          nl.push_back(torig[k] + 1);
          nl.push_back((int64_t)(j - sptr0[s]) * blkm + lmap[kp] + 1);
        }
        for (int64_t k = ptr[col]; k < ptr[col + 1]; ++k) {
          int kp = perm[row[k]];
          if (kp < j) continue;
          nl.push_back(k + 1);
          nl.push_back((int64_t)(j - sptr0[s]) * blkm + lmap[kp] + 1);
        }
      }
    }
    nptr0[nnodes] = (int64_t)(nl.size() / 2);

    // --- export in the 1-based conventions of the subtree interface ---
    ak->nnodes = nnodes;
    ak->sptr.resize(nnodes + 1);
    for (int s = 0; s <= nnodes; ++s) ak->sptr[s] = sptr0[s] + 1;
    ak->sparent.resize(nnodes);
    for (int s = 0; s < nnodes; ++s) ak->sparent[s] = spar[s] + 1;
    ak->rptr.resize(nnodes + 1);
    for (int s = 0; s <= nnodes; ++s) ak->rptr[s] = rptr0[s] + 1;
    ak->rlist.resize(rl.size());
    for (size_t k = 0; k < rl.size(); ++k) ak->rlist[k] = rl[k] + 1;
    ak->nptr.resize(nnodes + 1);
    for (int s = 0; s <= nnodes; ++s) ak->nptr[s] = nptr0[s] + 1;
    ak->nlist.swap(nl);
    ak->invp = invp;
    ak->nfact = nfact;
    ak->nflops = nflops;
    ak->maxfront = maxfront;
    ak->maxsupernode = maxsn;
    return ak;
  } catch (std::bad_alloc const&) {
    delete ak;
    *info = -50;
    return nullptr;
  }
}

// sizes[0..7] = n, nnodes, len(rlist), number of nlist pairs, nfact, nflops,
//               maxfront, maxsupernode
void spral_gb300_akeep_sizes(const void* h, int64_t* sizes) {
  const Akeep* ak = static_cast<const Akeep*>(h);
  sizes[0] = ak->n;
  sizes[1] = ak->nnodes;
  sizes[2] = (int64_t)ak->rlist.size();
  sizes[3] = (int64_t)(ak->nlist.size() / 2);
  sizes[4] = ak->nfact;
  sizes[5] = ak->nflops;
  sizes[6] = ak->maxfront;
  sizes[7] = ak->maxsupernode;
}

// Copy out the analyse arrays (any pointer may be NULL).
void spral_gb300_akeep_arrays(const void* h, int* sptr, int* sparent, int64_t* rptr,
                              int* rlist, int64_t* nptr, int64_t* nlist, int* invp) {
  const Akeep* ak = static_cast<const Akeep*>(h);
  if (sptr) std::copy(ak->sptr.begin(), ak->sptr.end(), sptr);
  if (sparent) std::copy(ak->sparent.begin(), ak->sparent.end(), sparent);
  if (rptr) std::copy(ak->rptr.begin(), ak->rptr.end(), rptr);
  if (rlist) std::copy(ak->rlist.begin(), ak->rlist.end(), rlist);
  if (nptr) std::copy(ak->nptr.begin(), ak->nptr.end(), nptr);
  if (nlist) std::copy(ak->nlist.begin(), ak->nlist.end(), nlist);
  if (invp) std::copy(ak->invp.begin(), ak->invp.end(), invp);
}

void spral_gb300_akeep_free(void* h) { delete static_cast<Akeep*>(h); }

// Minimum-degree ordering on the quotient graph (exact external degrees,
// no supervariables).  Input: lower CSC, 0-based.  Output: order[i] = pivot
// position of variable i.  Intended for moderate test matrices; the
// reference obtains its orderings from METIS, which is not part of this path.
int spral_gb300_order_mindeg(int n, const int64_t* ptr, const int* row, int* order) {
  try {
    std::vector<int64_t> fptr;
    std::vector<int> frow;
    full_pattern(n, ptr, row, fptr, frow);
    std::vector<std::vector<int>> avar(n), aelt(n), evar(n);
    for (int v = 0; v < n; ++v) {
      avar[v].assign(frow.begin() + fptr[v], frow.begin() + fptr[v + 1]);
      std::sort(avar[v].begin(), avar[v].end());
      avar[v].erase(std::unique(avar[v].begin(), avar[v].end()), avar[v].end());
    }
    std::vector<int> deg(n), stamp(n, -1);
    std::vector<char> done(n, 0), elive(n, 0);
    std::set<std::pair<int, int>> pq;
    for (int v = 0; v < n; ++v) { deg[v] = (int)avar[v].size(); pq.insert({deg[v], v}); }
    int tag = 0;
    std::vector<int> reach;
    auto compute_reach = [&](int v) {
      ++tag;
      reach.clear();
      stamp[v] = tag;
      for (int u : avar[v]) if (!done[u] && stamp[u] != tag) { stamp[u] = tag; reach.push_back(u); }
      for (int e : aelt[v]) for (int u : evar[e])
        if (!done[u] && stamp[u] != tag) { stamp[u] = tag; reach.push_back(u); }
    };
    for (int step = 0; step < n; ++step) {
      int v = pq.begin()->second;
      pq.erase(pq.begin());
      compute_reach(v);
      std::vector<int> vars = reach;
      done[v] = 1;
      order[v] = step;
      // new element v absorbs v's elements
      for (int e : aelt[v]) { elive[e] = 0; std::vector<int>().swap(evar[e]); }
      evar[v] = vars;
      elive[v] = 1;
      for (int u : vars) {
        auto& ae = aelt[u];
        ae.erase(std::remove_if(ae.begin(), ae.end(), [&](int e) { return !elive[e]; }), ae.end());
        ae.push_back(v);
        auto& av = avar[u];
        // variables covered by the new element are no longer explicit neighbours
        ++tag;
        for (int w : vars) stamp[w] = tag;
        av.erase(std::remove_if(av.begin(), av.end(),
                                [&](int w) { return done[w] || stamp[w] == tag; }), av.end());
      }
      for (int u : vars) {
        compute_reach(u);
        int d = (int)reach.size();
        pq.erase({deg[u], u});
        deg[u] = d;
        pq.insert({d, u});
      }
    }
    return 0;
  } catch (std::bad_alloc const&) {
    return -50;
  }
}


// Approximate minimum degree ordering, written from the published algorithm
// (P. R. Amestoy, T. A. Davis, I. S. Duff, "An approximate minimum degree
// ordering algorithm", SIAM J. Matrix Anal. Appl. 17(4), 1996): elimination
// on the quotient graph (variables, and elements formed by eliminated
// pivots), approximate external degrees from |Le \ Lp|, element absorption
// (including elements that Lp covers), and supervariables of
// indistinguishable variables found by hashing their adjacency, which also
// collapses the dense end of the elimination into one pivot block.  Input:
// lower CSC, 0-based.  Output: order[i] = pivot position of variable i.  The
// reference takes its orderings from METIS, which is not part of this path;
// this ordering serves general sparse matrices here (KKT systems).
int spral_gb300_order_amd(int n, const int64_t* ptr, const int* row, int* order) {
  try {
    std::vector<int64_t> fptr;
    std::vector<int> frow;
    full_pattern(n, ptr, row, fptr, frow);
    std::vector<std::vector<int>> A(n), E(n), Le(n);
    for (int v = 0; v < n; ++v) {
      A[v].assign(frow.begin() + fptr[v], frow.begin() + fptr[v + 1]);
      std::sort(A[v].begin(), A[v].end());
      A[v].erase(std::unique(A[v].begin(), A[v].end()), A[v].end());
    }
    std::vector<int64_t>().swap(fptr);
    std::vector<int>().swap(frow);
    enum : char { kVar = 0, kElt = 1, kMerged = 2, kDead = 3 };
    std::vector<char> status(n, kVar);
    std::vector<int> nv(n, 1), deg(n), chain_next(n, -1), chain_last(n);
    for (int v = 0; v < n; ++v) { deg[v] = (int)A[v].size(); chain_last[v] = v; }
    // degree buckets (doubly linked)
    std::vector<int> head(n + 1, -1), nxt(n, -1), prv(n, -1);
    auto bucket_insert = [&](int v) {
      const int d = std::min(std::max(deg[v], 0), n);
      nxt[v] = head[d];
      prv[v] = -1;
      if (head[d] >= 0) prv[head[d]] = v;
      head[d] = v;
    };
    auto bucket_remove = [&](int v) {
      const int d = std::min(std::max(deg[v], 0), n);
      if (prv[v] >= 0) nxt[prv[v]] = nxt[v];
      else head[d] = nxt[v];
      if (nxt[v] >= 0) prv[nxt[v]] = prv[v];
      nxt[v] = prv[v] = -1;
    };
    for (int v = n - 1; v >= 0; --v) bucket_insert(v);
    std::vector<int> mark(n, 0), wstamp(n, 0);
    std::vector<long long> w(n, 0);
    int tag = 0, wtag = 0, mindeg = 0, nel = 0;
    std::vector<int> pivots;
    std::vector<int> Lp;
    std::vector<std::pair<unsigned long long, int>> hv;
    while (nel < n) {
      while (mindeg <= n && head[mindeg] < 0) ++mindeg;
      if (mindeg > n) return -1;  // inconsistent state
      const int p = head[mindeg];
      bucket_remove(p);
      // the new element Lp: p's elements' variables and p's variable neighbours
      ++tag;
      mark[p] = tag;
      Lp.clear();
      long long lpw = 0;
      for (int e : E[p]) {
        if (status[e] != kElt) continue;
        for (int j : Le[e])
          if (status[j] == kVar && mark[j] != tag) { mark[j] = tag; Lp.push_back(j); lpw += nv[j]; }
        status[e] = kDead;  // absorbed into p
        std::vector<int>().swap(Le[e]);
      }
      for (int j : A[p])
        if (status[j] == kVar && mark[j] != tag) { mark[j] = tag; Lp.push_back(j); lpw += nv[j]; }
      std::vector<int>().swap(E[p]);
      std::vector<int>().swap(A[p]);
      status[p] = kElt;
      nel += nv[p];
      pivots.push_back(p);
      for (int i : Lp) bucket_remove(i);
      // adjacency of the variables of Lp: element p replaces what it covers
      for (int i : Lp) {
        auto& Ei = E[i];
        size_t k = 0;
        for (int e : Ei) if (status[e] == kElt && e != p) Ei[k++] = e;
        Ei.resize(k);
        Ei.push_back(p);
        auto& Ai = A[i];
        k = 0;
        for (int j : Ai) if (status[j] == kVar && mark[j] != tag) Ai[k++] = j;
        Ai.resize(k);
      }
      // w(e) = |Le \ Lp| (weighted) for the other elements next to Lp
      ++wtag;
      for (int i : Lp)
        for (int e : E[i]) {
          if (e == p) continue;
          if (wstamp[e] != wtag) {
            wstamp[e] = wtag;
            auto& L = Le[e];
            size_t k = 0;
            long long s = 0;
            for (int j : L) if (status[j] == kVar) { L[k++] = j; s += nv[j]; }
            L.resize(k);
            w[e] = s;
          }
          w[e] -= nv[i];
        }
      // approximate external degrees; elements covered by Lp are absorbed
      for (int i : Lp) {
        long long dext = 0;
        auto& Ei = E[i];
        size_t k = 0;
        for (int e : Ei) {
          if (e == p) { Ei[k++] = e; continue; }
          if (status[e] != kElt) continue;
          if (w[e] <= 0) { status[e] = kDead; std::vector<int>().swap(Le[e]); continue; }
          dext += w[e];
          Ei[k++] = e;
        }
        Ei.resize(k);
        for (int j : A[i]) dext += nv[j];
        long long d = std::min<long long>((long long)deg[i] + lpw - nv[i], dext + lpw - nv[i]);
        d = std::min<long long>(d, (long long)(n - nel) - nv[i]);
        deg[i] = (int)std::max<long long>(d, 0);
      }
      // supervariables: variables of Lp with equal element and variable lists
      hv.clear();
      for (int i : Lp) {
        auto& Ei = E[i];
        size_t k = 0;
        for (int e : Ei) if (status[e] == kElt) Ei[k++] = e;
        Ei.resize(k);
        std::sort(Ei.begin(), Ei.end());
        std::sort(A[i].begin(), A[i].end());
        unsigned long long h = 1469598103934665603ull;
        for (int e : Ei) h = (h ^ (unsigned long long)e) * 1099511628211ull;
        h = (h ^ 0x9e3779b97f4a7c15ull) * 1099511628211ull;
        for (int j : A[i]) h = (h ^ (unsigned long long)j) * 1099511628211ull;
        hv.push_back({h, i});
      }
      std::sort(hv.begin(), hv.end());
      for (size_t a = 0; a < hv.size();) {
        size_t b = a;
        while (b < hv.size() && hv[b].first == hv[a].first) ++b;
        for (size_t x = a; x < b; ++x) {
          const int i = hv[x].second;
          if (status[i] != kVar) continue;
          for (size_t y = x + 1; y < b; ++y) {
            const int j = hv[y].second;
            if (status[j] != kVar) continue;
            if (E[i] != E[j] || A[i] != A[j]) continue;
            // j is indistinguishable from i: merge
            nv[i] += nv[j];
            deg[i] -= nv[j];
            nv[j] = 0;
            status[j] = kMerged;
            chain_next[chain_last[i]] = j;
            chain_last[i] = chain_last[j];
            std::vector<int>().swap(E[j]);
            std::vector<int>().swap(A[j]);
          }
        }
        a = b;
      }
      auto& Lnew = Le[p];
      for (int i : Lp) {
        if (status[i] != kVar) continue;
        deg[i] = std::max(deg[i], 0);
        bucket_insert(i);
        mindeg = std::min(mindeg, std::min(deg[i], n));
        Lnew.push_back(i);
      }
    }
    int pos = 0;
    for (int p : pivots)
      for (int v = p; v >= 0; v = chain_next[v]) order[v] = pos++;
    return pos == n ? 0 : -1;
  } catch (std::bad_alloc const&) {
    return -50;
  }
}

}  // extern "C"
