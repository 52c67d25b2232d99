// lifted.hpp -- host planning of the full-tree adaptation with coarse
// extension (lifted wavelets CDF XY, Y > 0).
//
// adapt_tree (LIB/MESH/adapt_tree.f90:11-255) runs, on the full tree (leaves
// and all their ancestors), a level loop of ghost synchronisations, FWTs,
// coarse-extension modifications (LIB/MPI/reconstruction_step.f90:3-100) and
// daughter-to-mother copies, then the indicator, the security zone
// (LIB/MESH/securityZone_tree.f90:140-306), the flag consistency rules, the
// deletion, and a reconstruction limited to the blocks at coarse/fine
// interfaces (wavelet_reconstruct_full_tree_CEoptimized, :686-987). Every
// sync is sync_ghosts_generic (LIB/MPI/synchronize_ghosts_generic.f90:
// 181-694) with a case (full, MoC, MoF, ...), optional filters on the
// receiver's refinement status and level, and per sender the choice between
// the decomposed (hvy_block) and the original (hvy_tmp) data
// (LIB/MPI/xfer_block_data.f90:321-437).
//
// This file turns each of those steps into flat device work lists: patches
// with a source-buffer flag, filtered-restriction entries with their
// coarse-extension copies, strided boxes to zero or copy, block lists for
// the transforms. The reference fills the patches of a stage one after
// another; the lists are cut into waves such that no patch reads a box that
// an earlier patch of the same wave writes or writes a box an earlier patch
// reads, so each wave runs in parallel with the sequential result.
#pragma once
#include <cstdint>
#include <memory>
#include <string>
#include <utility>
#include <vector>

#include "adapt.hpp"
#include "forest.hpp"

namespace wg {

constexpr int kRefTmpEmpty = 10;   // REF_TMP_EMPTY (module_globals.f90:25)

// one box of one block: zero the points or copy them from hvy_tmp, on a
// lattice with the given first point and step per direction (0-based,
// inclusive)
struct BoxOp {
    int32_t slot;
    int16_t op;                       // 0 zero (hvy_block), 1 copy hvy_tmp -> hvy_block
    int16_t pad;
    int16_t lo[3], hi[3], step[3];
    int16_t pad2;
};
static_assert(sizeof(BoxOp) == 28, "BoxOp layout");

// filtered restriction: the HD-filtered scaling coefficients of one sender
// (blockFilterXYZ_vct with do_restriction, module_wavelets.f90:307-401) on
// the interior SC lattice, from hvy_block (src_tmp 0) or hvy_tmp (1)
struct FilterEntry {
    int32_t slot;
    int32_t src_tmp;
};
// coarse-extension SC copy into a filter entry (restrict_copy_at_CE,
// LIB/MPI/restrict_predict_data.f90:121-170): SC lattice index box
struct ScBox {
    int32_t entry;
    int16_t lo[3], hi[3];
};

// vectors of plain records whose resize leaves the new elements
// uninitialised (they are written right after, in parallel)
template <class T>
struct NoInit : std::allocator<T> {
    template <class U>
    struct rebind {
        using other = NoInit<U>;
    };
    NoInit() = default;
    template <class U>
    NoInit(const NoInit<U> &) {}
    template <class U>
    void construct(U *p) {
        ::new (static_cast<void *>(p)) U;
    }
    template <class U, class... A>
    void construct(U *p, A &&...a) {
        ::new (static_cast<void *>(p)) U(std::forward<A>(a)...);
    }
};
template <class T>
using RecVec = std::vector<T, NoInit<T>>;

struct SyncWave {
    int stage = 1;
    RecVec<Patch> copy_blk, copy_tmp;           // op 0 from hvy_block / hvy_tmp
    RecVec<FilterEntry> filters;                // restriction: filtered senders
    RecVec<ScBox> ce_copies;                    // SC copied back into the entries
    RecVec<Patch> restrict_;                    // op 1, src = filter entry index
    RecVec<Patch> pred_blk, pred_tmp;           // op 2 from hvy_block / hvy_tmp
    int max_coarse = 0;                         // shared memory of the largest prediction (doubles)
    // a stage of copies and restrictions built per chunk of senders: the
    // wave is the concatenation of these parts' lists (their filter entry
    // numbers already count the entries of the parts before them)
    std::vector<SyncWave> parts;
};

struct SyncSpecL {
    int base = 1;                  // 1 full, 2 full_leaf, 3 MoC, 4 MoF, 5 Monly
    bool by_ref = false, by_level = false;
    int s_ref = 0, s_level = 0;
    int gminus = 0, gplus = 0;
    int tmp_usage = 0;             // 0 none, 1 not_flag_is_decomposed, 2 block_is_decomposed
    bool filter = true;            // filtered restriction (lifted wavelets)
};

class LiftedTree {
public:
    Geometry geo;
    WaveletInfo wav;
    int Jmin = 1, Jmax = 1;
    int nleaves = 0;
    FullTree ft;                   // leaves 0..nleaves-1, then mothers
    std::vector<int> slot;         // arena slot per full-tree block
    std::vector<char> alive;       // block present (deleted blocks are gone)
    std::vector<int> ref;          // refinement status
    // CE widths (module_wavelets.f90:1341-1417)
    int Nscl = 0, Nscr = 0, Nwcl = 0, Nwcr = 0, Nreconl = 0, Nreconr = 0, Ndep2l = 0, Ndep2r = 0;

    bool init(const Geometry &g, const WaveletInfo &w, int fd_max_size, int Jmin, int Jmax, int nleaf,
              const int *level, const int *coords, std::string &err);
    // neighbour relations (overlapping search) and family of the alive blocks
    bool update_metadata(std::string &err);
    int size() const { return ft.size(); }
    int mother(int b) const;
    bool is_leaf(int b, bool check_empty) const;
    bool is_root(int b, bool check_empty) const;
    bool has_valid_neighbor(int b, int relation, int lvl_diff) const;
    // neighbour of b in relation r (1..168) or -1
    int nbr(int b, int r) const {
        for (int i = adj_begin_[b]; i < adj_begin_[b + 1]; i++)
            if (adj_[i].first == r) return adj_[i].second;
        return -1;
    }
    // existing neighbours of b in ascending relation order: f(relation, n)
    template <class F>
    void for_neighbors(int b, F f) const {
        for (int i = adj_begin_[b]; i < adj_begin_[b + 1]; i++) f(adj_[i].first, adj_[i].second);
    }

    void plan_sync(const SyncSpecL &sp, std::vector<SyncWave> &waves) const;
    // coarse_extension_modify: case 0 tree, 1 level, 2 ref, 3 level_ref
    void plan_ce_modify(int ce_case, int s_level, int s_ref, bool clear_wc, bool copy_sc,
                        std::vector<BoxOp> &ops) const;
    // addSecurityZone_CE_tree, pass 1 candidates: (block, relation, box)
    struct ZoneItem {
        int block, relation;
        int lo[3], hi[3], io[3];
    };
    void security_candidates(std::vector<ZoneItem> &items) const;
    // passes 2 and 3 from the significance of the candidates
    void security_apply(const std::vector<ZoneItem> &items, const std::vector<char> &significant);

private:
    std::vector<int> adj_begin_;   // neighbour lists of the alive blocks, ascending relation
    std::vector<std::pair<int, int>> adj_;
    // the same search with every block of the full tree alive (once per tree)
    bool full_ready_ = false;
    std::vector<int> full_begin_;
    std::vector<std::pair<int, int>> full_adj_;
    std::vector<int> rel_dir_, rel_part_;   // direction (0..26) and part of finer relation r-1
    void search_all_();
    std::vector<uint64_t> keys_;   // open-addressing table: block key -> full-tree index
    std::vector<int> vals_;
    uint64_t mask_ = 0;
    int find_(int lv, int x, int y, int z) const;
    void ce_clear_wc(int b, int relation, std::vector<BoxOp> &ops) const;
    void ce_copy_sc(int b, int relation, std::vector<BoxOp> &ops) const;
};

}  // namespace wg
