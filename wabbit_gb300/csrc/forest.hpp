// forest.hpp -- host-side tree bookkeeping of the GB300 hot path.
//
// The reference keeps the block tree as light data (lgt_block: level,
// treecode) and recomputes neighbour relations and ghost-patch index boxes on
// every synchronisation (LIB/MESH/find_neighbors.f90, LIB/TREE/neighborhood.f90,
// LIB/MPI/calc_data_bounds.f90, synchronize_ghosts_generic.f90:352-694). Here
// that integer work runs once per grid change and is flattened into patch
// tables that the device sync kernel consumes; the heavy data never leaves HBM.
#pragma once
#include <cstdint>
#include <string>
#include <unordered_map>
#include <vector>

namespace wg {

// neighbour-relation numbering of the reference (find_neighbors.f90:1-16):
//   1- 56 same level, 57-112 coarser neighbour, 113-168 finer neighbour
constexpr int kNumRelations = 168;

struct WaveletInfo {
    int X = 4, Y = 0;            // CDF X,Y
    bool lifted = false;
    int order_predictor = 4;     // 2,4,6,8
    int g_min = 3;               // minimal ghost width
    std::vector<double> HD, GD, HR, GR;  // coefficient arrays
    int hd_lo = 0, gd_lo = 0, hr_lo = 0, gr_lo = 0;
};
bool make_wavelet(const char *name, WaveletInfo &w);

struct Geometry {
    int dim = 2;
    int Bs[3] = {16, 16, 1};
    int g = 4;                   // ghost width of the full-state layout
    int nc = 3;
    int n(int d) const { return d < dim ? Bs[d] + 2 * g : 1; }
};

class Forest {
public:
    int dim = 2, Jmin = 1, Jmax = 1;
    std::vector<int> level;      // per block
    std::vector<int> coords;     // 3 per block
    std::vector<int> nbr;        // kNumRelations per block, -1 = none

    int size() const { return (int)level.size(); }
    void set(int nblk, const int *lv, const int *co);
    int find(int lv, int x, int y, int z) const;
    // neighbour search for all blocks; returns false and a message for an
    // invalid grid (a face without any neighbour, overlapping blocks, ...).
    // With overlapping (a full tree: leaves and their ancestors) every
    // existing same-level, finer and coarser neighbour is recorded, as
    // find_neighbor with search_overlapping (find_neighbors.f90:18-215).
    bool update_neighbors(std::string &err, bool overlapping = false);
    // maximum level difference across any face/edge/corner is 1
    bool graded() const;
    uint64_t treecode(int b) const;  // reference bit layout (y bit0, x bit1, z bit2)

private:
    // open-addressing table (linear probing) of block keys -> block index
    std::vector<uint64_t> keys_;
    std::vector<int> vals_;
    uint64_t mask_ = 0;
    bool insert_(uint64_t key, int b);
};

// One ghost patch: fill box [rlo,rhi] (0-based, inclusive) of block dst from
// block src. op: 0 copy, 1 restriction (every 2nd point), 2 prediction.
//   copy:     src index = slo + (r - rlo)
//   restrict: src index = slo + 2*(blo + r - rlo)
//   predict:  fine index f = blo + (r - rlo) into the (2n-1)-point fine array
//             interpolated from the coarse box [slo,shi] of src
struct Patch {
    int32_t src, dst;
    int16_t op, stage;
    int16_t rlo[3], rhi[3];
    int16_t slo[3], shi[3];
    int16_t blo[3], pad;
};
static_assert(sizeof(Patch) == 44, "patch layout");

struct SyncTable {
    int nstages = 2;
    std::vector<Patch> patches;        // sorted by stage
    std::vector<int> stage_begin;      // nstages+1 offsets
    std::vector<int> stage_predict;    // 1 if every patch of the stage is a prediction
    int max_points = 0;                // largest receiver box
    int max_coarse = 0;                // largest shared-memory need of a prediction (doubles)
};

// Patch of relation r (1..168) from src to dst with level difference
// lvl_diff = level(src) - level(dst), boxes in the full layout (ghost width
// geo.g): receiver box from get_indices_of_ghost_patch of the inverse
// relation, sender / buffer boxes from set_send_bounds.
Patch make_patch(const Geometry &geo, int order_predictor, int relation, int lvl_diff, int gminus, int gplus, int src,
                 int dst);
// get_indices_of_modify_patch (neighborhood.f90:23-126), 0-based inclusive
void modify_box0(const Geometry &geo, int relation, int Ns, int Ne, int gm, int gp, int lvl_diff, int lo[3], int hi[3]);
// get_indices_of_ghost_patch (neighborhood.f90:158-327), 0-based inclusive
void ghost_box0(const Geometry &geo, int relation, int gminus, int gplus, int lvl_diff, int lo[3], int hi[3]);
int relation_inverse(int relation);
// relation id 1..56 of direction d (components -1, 0, +1) and, for a finer or
// coarser neighbour, the part index along the free directions
int relation_id(const int d[3], int part, int dim);
// np_l / np_u (neighborhood.f90:439-500): relations of the same patch at
// another level difference
void relation_range(int relation, int lvl_diff, int &lo, int &hi);
// neighborhood2patchID (neighborhood.f90:413-434)
int relation_patch_id(int relation);

// Build the ghost-sync table of one forest for the reference's
// sync_ghosts_RHS_tree / sync_ghosts_tree semantics on a leaf-only grid.
// Boxes are expressed for a buffer with ghost width g_buf (<= geo.g): an
// index i of the full layout maps to i - (geo.g - g_buf).
bool make_sync_table(const Forest &f, const Geometry &geo, const WaveletInfo &w, int gminus, int gplus,
                     int g_buf, int block_offset, SyncTable &out, std::string &err);

}  // namespace wg
