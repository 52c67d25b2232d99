// adapt.hpp -- host-side tree logic of the wavelet adaptation (coarsening).
//
// The reference's adapt_tree (LIB/MESH/adapt_tree.f90:11-255) works on the
// "full tree": the leaf grid plus every ancestor down to Jmin
// (init_full_tree, adapt_tree.f90:995-1085). Every block of the full tree is
// decomposed (a mother holds its daughters' scaling coefficients,
// sync_D2M, LIB/MESH/executeCoarsening_tree.f90:125-227), flagged by the
// coarsening indicator, and the flags are made consistent
// (respectJmaxJmin_tree, ensureGradedness_tree with check_daughters,
// ensure_completeness_block); blocks still flagged -1 are deleted and the
// remaining blocks without remaining daughters are the new leaves
// (prune_fulltree2leafs, adapt_tree.f90:1235).
#pragma once
#include <cstdint>
#include <string>
#include <unordered_map>
#include <vector>

#include "forest.hpp"

namespace wg {

// flag values of the reference (module_globals.f90:25-32)
constexpr int kFlagCoarsen = -1;
constexpr int kFlagStay = 0;
constexpr int kFlagUnsignificantStay = 9;   // REF_UNSIGNIFICANT_STAY

struct FullTree {
    int dim = 2, Jmin = 0;
    int nleaves = 0;                 // blocks 0..nleaves-1 are the input leaves, in input order
    std::vector<int> level;          // per block
    std::vector<int> coords;         // 3 per block
    std::vector<int> mother;         // index or -1
    std::vector<int> daughters;      // 8 per block (2^dim used), -1 where absent
    std::unordered_map<uint64_t, int> lookup;

    int size() const { return (int)level.size(); }
    bool is_leaf(int b) const { return daughters[8 * b] < 0; }
    int find(int lv, int x, int y, int z) const;
    int max_level() const;
};

// leaves + all ancestors down to Jmin; mothers are appended level by level
// from the finest (false and a message for leaves below Jmin)
bool build_full_tree(int dim, int Jmin, int nblk, const int *level, const int *coords, FullTree &t, std::string &err);

// neighbour of block b across direction d (components -1, 0, +1) on the
// same level (periodic domain), or -1
int same_level_neighbor(const FullTree &t, int b, const int d[3]);

// Make the indicator flags of every full-tree block consistent and return
// the new leaves (full-tree indices, ascending). flags: -1 (coarsen) or 0
// (stay) per block on entry; on exit the final flags (-1 deleted).
void adapt_decide(const FullTree &t, std::vector<int> &flags, std::vector<int> &new_leaves);

// sync_D2M for CDF X0 and same-level ghost copies of the mothers of one
// level, as ghost patches (see Patch in forest.hpp) on the full layout;
// slot maps a full-tree block to its arena slot
void mother_patches(const FullTree &t, const Geometry &geo, int level, const std::vector<int> &slot,
                    std::vector<Patch> &d2m, std::vector<Patch> &ghosts);

}  // namespace wg
