// Level schedule of the assembly tree.
//
// The numeric factorisation runs the fronts level by level, every APP
// kernel of a block step over all fronts of a level in one launch, so a
// level takes as many block steps as its widest front needs.  The
// reference's GPU path levels the tree by depth below the root, numbered
// from the bottom (src/ssids/gpu/factor.f90:824-879,
// assign_nodes_to_levels); here two valid schedules are compared by their
// block steps:
//   leaf-aligned  a node's height above its leaves (leaves = 0);
//   root-aligned  the top level minus the node's depth below its root, the
//                 small leaf subtrees (factored by TPP in their own
//                 level-set launches) keeping their leaf-aligned levels.
// A root-aligned node is never below its leaf-aligned level (induction from
// the roots: its parent's root-aligned level is at least the parent's
// height, one above the node's), so a small subtree's root stays below its
// parent in the mixed schedule.  Root alignment pays where sibling subtrees
// differ in height: their separators, which the leaf-aligned schedule
// factors one after the other, share a level.
#include "schedule.h"

#include "spral_ssids_gpu.h"

#include <algorithm>

namespace ssids300 {

int64_t level_block_steps(const std::vector<int>& lev, int nlev, const int* ncol,
                          const char* small) {
  std::vector<int> mx(std::max(nlev, 0), 0);
  for (size_t i = 0; i < lev.size(); ++i)
    if (!small || !small[i]) mx[lev[i]] = std::max(mx[lev[i]], (ncol[i] + 31) / 32);
  int64_t sum = 0;
  for (int v : mx) sum += v;
  return sum;
}

bool level_schedule(int nn, const int* parent, const int* ncol, const char* small,
                    LevelAlign align, std::vector<int>& lev, int& nlev) {
  lev.assign(nn, 0);
  nlev = 0;
  for (int i = 0; i < nn; ++i) {
    if (parent[i] >= 0) lev[parent[i]] = std::max(lev[parent[i]], lev[i] + 1);
    nlev = std::max(nlev, lev[i] + 1);
  }
  if (align == LevelAlign::Leaf || nn == 0) return false;
  std::vector<int> ra(nn);
  for (int i = nn - 1; i >= 0; --i)
    ra[i] = (small && small[i]) ? lev[i] : (parent[i] < 0 ? nlev - 1 : ra[parent[i]] - 1);
  // root alignment only for at least 10% fewer steps: the model counts the
  // widths of the analysis, and delayed columns change them (a KKT tree
  // with 5,545 delays, predicted 0.4% fewer steps root-aligned, ran 17%
  // slower)
  if (align == LevelAlign::Root ||
      (align == LevelAlign::Choose && 10 * level_block_steps(ra, nlev, ncol, small) <=
                                          9 * level_block_steps(lev, nlev, ncol, small))) {
    lev.swap(ra);
    return true;
  }
  return false;
}

}  // namespace ssids300

extern "C" int spral_ssids_gpu_level_schedule(int nnodes, const int* parent, const int* ncol,
                                              const char* small, int align, int* level,
                                              int* nlev, int64_t* steps) {
  using namespace ssids300;
  if (nnodes < 0 || (nnodes > 0 && (!parent || !ncol || !level)) || !nlev || align < 0 ||
      align > 2)
    return -1;
  for (int i = 0; i < nnodes; ++i)
    if (parent[i] != -1 && (parent[i] <= i || parent[i] >= nnodes)) return -1;
  std::vector<int> lev;
  int nl = 0;
  const bool root = level_schedule(nnodes, parent, ncol, small, static_cast<LevelAlign>(align),
                                   lev, nl);
  for (int i = 0; i < nnodes; ++i) level[i] = lev[i];
  *nlev = nl;
  if (steps) *steps = level_block_steps(lev, nl, ncol, small);
  return root ? 1 : 0;
}
