// Level schedule of the assembly tree (host side; see schedule.cpp).
#pragma once
#include <cstdint>
#include <vector>

namespace ssids300 {

enum class LevelAlign { Choose = 0, Leaf = 1, Root = 2 };

// APP block steps of a level schedule: per level the widest non-small
// front's ceil(ncol / 32), summed over levels
int64_t level_block_steps(const std::vector<int>& lev, int nlev, const int* ncol,
                          const char* small);

// Levels of a postordered tree (parent[i] > i, -1 for a root): lev[i] for
// every node, every node on a lower level than its parent; returns true when
// the root-aligned schedule was taken.  small[i] != 0 marks the nodes of the
// small leaf subtrees (whole subtrees), which keep leaf-aligned levels.
bool level_schedule(int nn, const int* parent, const int* ncol, const char* small,
                    LevelAlign align, std::vector<int>& lev, int& nlev);

}  // namespace ssids300
