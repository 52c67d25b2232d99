// wg_oracle.cpp -- CPU oracle for the WABBIT ACM block-level time-step hot path.
//
// TEST INFRASTRUCTURE ONLY. This file is a scalar, line-by-line restatement of
// the reference's Fortran algorithms for the hot path, used by tests/, by
// __graft_entry__.smoke() and by bench.py's cpu_baseline leg as the checker.
// The product (wabbit_gb300/) never links, imports or calls it.
//
// It is compiled with -ffp-contract=off so that every floating-point
// expression is evaluated with the reference's (x86-64, no FMA) rounding in the
// reference's left-to-right order. Array indices in the patch-geometry code
// are kept 1-based, as in the Fortran, and converted only at array access.
//
// Parity: pinned against the reference's committed regression files
// (TESTING/acm/3vortices/3vorticesEquiFD4_CDF40, TESTING/acm/taylorGreen/
// taylorGreenEqui_FD4_CDF40, TESTING/wavelets/adaptive_CDF4x) through fixtures
// generated by tests/golden/make_fixtures.py.
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <unordered_map>
#include <vector>
#include <algorithm>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "../include/wabbit_gb300.h"

namespace {

// ---------------------------------------------------------------------------
// wavelet filters: setup_wavelet (LIB/WAVELETS/module_wavelets.f90:1031-1561)
// ---------------------------------------------------------------------------
struct Filter {           // coefficients f(lo..hi)
    int lo = 0, hi = -1;
    std::vector<double> c;
    double operator()(int i) const { return c[i - lo]; }
    void init(int l, int h) { lo = l; hi = h; c.assign(h - l + 1, 0.0); }
};

// interpolation stencils with added zeros (module_wavelets.f90:14-22)
static void stencil_int(int order, Filter &f) {
    switch (order) {
    case 2: f.init(-1, 1); { double v[] = {1, 2, 1}; for (int i = 0; i < 3; i++) f.c[i] = v[i] / 2.0; } break;
    case 4: f.init(-3, 3); { double v[] = {-1, 0, 9, 16, 9, 0, -1}; for (int i = 0; i < 7; i++) f.c[i] = v[i] / 16.0; } break;
    case 6: f.init(-5, 5); { double v[] = {3, 0, -25, 0, 150, 256, 150, 0, -25, 0, 3}; for (int i = 0; i < 11; i++) f.c[i] = v[i] / 256.0; } break;
    case 8: f.init(-7, 7); { double v[] = {-5, 0, 49, 0, -245, 0, 1225, 2048, 1225, 0, -245, 0, 49, 0, -5}; for (int i = 0; i < 15; i++) f.c[i] = v[i] / 2048.0; } break;
    default: f.init(0, -1);
    }
}

struct Wavelet {
    int X = 4, Y = 0;
    bool lifted = false;
    Filter HD, GD, HR, GR;
    int order_predictor = 4;
    int Nscl = 0, Nscr = 0, Nwcl = 0, Nwcr = 0;
    int Nreconl = 0, Nreconr = 0, Ndep2l = 0, Ndep2r = 0;
    std::string name;
};

static bool setup_wavelet(const char *name, int fd_max_size, Wavelet &w) {
    w.name = name;
    if (std::strncmp(name, "CDF", 3) != 0 || std::strlen(name) < 5) return false;
    w.X = name[3] - '0';
    w.Y = name[4] - '0';
    if (w.X != 2 && w.X != 4 && w.X != 6 && w.X != 8) return false;
    if (w.Y != 0 && w.Y != 2 && w.Y != 4 && w.Y != 6 && w.Y != 8) return false;
    stencil_int(w.X, w.HR);
    if (w.Y == 0) {
        w.HD.init(0, 0);
        w.HD.c[0] = 1.0;
    } else if (w.X >= w.Y) {
        Filter h;
        stencil_int(w.Y, h);
        h.c[0 - h.lo] = 0.0;
        w.HD.init(w.HR.lo + h.lo, w.HR.hi + h.hi);
        for (int i = w.HD.lo; i <= w.HD.hi; i++) {
            double v = (i == 0) ? 1.0 : 0.0;
            for (int j = w.HR.lo; j <= w.HR.hi; j++) {
                if (i - j < h.lo || i - j > h.hi) continue;
                // (-1.0_rk)**j * HR(j) * h_ntilde(i-j) / 2.0_rk
                double sgn = (std::abs(j) % 2 == 0) ? 1.0 : -1.0;
                v = v + sgn * w.HR(j) * h(i - j) / 2.0;
            }
            w.HD.c[i - w.HD.lo] = v;
        }
    } else {
        return false;  // CDF24/26/28/46 not needed on this path
    }
    w.GD.init(w.HR.lo, w.HR.hi);
    for (int i = w.GD.lo; i <= w.GD.hi; i++) w.GD.c[i - w.GD.lo] = ((std::abs(i) % 2 == 0) ? 1.0 : -1.0) * w.HR(i);
    w.GR.init(w.HD.lo, w.HD.hi);
    for (int i = w.GR.lo; i <= w.GR.hi; i++) w.GR.c[i - w.GR.lo] = ((std::abs(i) % 2 == 0) ? 1.0 : -1.0) * w.HD(i);
    w.lifted = (w.Y != 0);
    w.order_predictor = w.X;
    // coarse-extension widths (module_wavelets.f90:1341-1375)
    w.Nscl = std::max(std::abs(w.HD.lo) - 1, 0);
    w.Nwcl = w.Nscl + std::abs(w.GD.lo);
    w.Nreconl = w.Nwcl + std::abs(w.GR.lo);
    w.Ndep2l = w.Nreconl + std::max((std::abs(w.HR.lo) + 1) / 2 - 1, 0);
    w.Nscr = w.HD.hi;
    w.Nwcr = w.Nscr + w.GD.hi;
    w.Nreconr = w.Nwcr + w.GR.hi;
    w.Ndep2r = w.Nreconr + (w.HR.hi + 1) / 2;
    // minimum WC width from the FD stencils (module_wavelets.f90:1405-1417)
    int i2 = 2 * fd_max_size;
    const int dl = std::max(i2 - w.Nwcl, 0), dr = std::max(i2 - w.Nwcr, 0);
    w.Nwcl += dl;
    w.Nreconl += dl;
    w.Ndep2l += dl;
    w.Nwcr += dr;
    w.Nreconr += dr;
    w.Ndep2r += dr;
    return true;
}

// ---------------------------------------------------------------------------
// forest: blocks, levels, neighbour relations
// ---------------------------------------------------------------------------
struct Block {
    int level;
    int c[3];
};

static inline uint64_t key_of(int level, int x, int y, int z) {
    return (uint64_t(level) << 60) | (uint64_t(x) << 40) | (uint64_t(y) << 20) | uint64_t(z);
}

struct Oracle {
    wg_config cfg;
    Wavelet wav;
    int nx, ny, nz, nc, npts;       // block extents incl. ghosts
    std::vector<Block> blocks;
    std::vector<double> data;       // nblk * nc * npts
    std::vector<double> mask;       // nblk * 6 * npts (optional), or per mask_slot
    std::vector<int> mask_slot;     // empty: mask is dense; else block -> slot of mask (6 * npts each)
    std::vector<int> nb;            // nblk * 168
    std::unordered_map<uint64_t, int> lookup;
    // full-tree adaptation: hvy_tmp, refinement status, family
    std::vector<double> tmp;
    std::vector<int> ref, mother, dau;   // dau: 8 per block, -1 where absent
    // refinement status of the leaves after the last adaptation (0:
    // significant, REF_UNSIGNIFICANT_STAY), read by the "significant"
    // refinement indicator
    std::vector<int> status;
    // useCoarseExtension / useSecurityZone also for unlifted wavelets (an ini
    // that sets them, ini_file_to_params.f90:543-546)
    bool ce_force = false;
    // RK registers: slot 0 = u_n, 1..4 = k1..k4 (hvy_work), interior points
    // only (the only points the RK update reads or writes)
    std::vector<double> work;
    int nthreads = 1;
    // penalisation geometry (createMask_tree); kind WG_GEOM_NONE = none
    wg_geometry geom{};

    double *blk(int b) { return data.data() + size_t(b) * nc * npts; }
    const double *blk(int b) const { return data.data() + size_t(b) * nc * npts; }
    // 1-based Fortran indexing into a block array
    inline size_t at(int ix, int iy, int iz, int ic) const {
        return ((size_t(ic - 1) * nz + (iz - 1)) * ny + (iy - 1)) * nx + (ix - 1);
    }
};

// the mask of block b (6 components of npts points), null without a mask
static inline const double *mask_of(const Oracle &o, int b) {
    if (o.mask.empty()) return nullptr;
    const size_t slot = o.mask_slot.empty() ? size_t(b) : size_t(o.mask_slot[b]);
    return o.mask.data() + slot * 6 * o.npts;
}

static inline void clear_mask(Oracle &o) {
    o.mask.clear();
    o.mask_slot.clear();
}

// treecode digit of a block at its own level: bit0 = y, bit1 = x, bit2 = z
// (LIB/TREE/module_treelib.f90 encoding_b/decoding_b, find_neighbors.f90:46)
static inline int tc_last_digit(const Block &b) {
    return 2 * (b.c[0] & 1) + (b.c[1] & 1) + 4 * (b.c[2] & 1);
}

static void rebuild_lookup(Oracle &o) {
    o.lookup.clear();
    for (int i = 0; i < (int)o.blocks.size(); i++) {
        const Block &b = o.blocks[i];
        o.lookup[key_of(b.level, b.c[0], b.c[1], b.c[2])] = i;
    }
}

static int find_block(const Oracle &o, int level, const int c[3]) {
    auto it = o.lookup.find(key_of(level, c[0], c[1], c[2]));
    return it == o.lookup.end() ? -1 : it->second;
}

// adjacent block coordinates on `level` in direction d (periodic domain)
static void adjacent(const int c[3], const int d[3], int level, int dim, int out[3]) {
    int n = 1 << level;
    for (int i = 0; i < 3; i++) {
        if (i < dim) out[i] = ((c[i] + d[i]) % n + n) % n;
        else out[i] = 0;
    }
}

// find_neighbor (LIB/MESH/find_neighbors.f90:18-215) for one direction
static void find_neighbor(Oracle &o, int ib, const int dir_dim[3], bool overlapping) {
    const int dim = o.cfg.dim;
    const Block &B = o.blocks[ib];
    const int level = B.level;
    int nzero = 0;
    for (int i = 0; i < 3; i++) if (dir_dim[i] == 0) nzero++;
    int dir_free = 1 << nzero;
    if (dim == 2) dir_free /= 2;
    int tcFiner[4] = {0, 0, 0, 0};
    const int vary_tc[3] = {2, 1, 4};
    int apply_free = 1;
    for (int i = 0; i < dim; i++) {
        if (dir_dim[i] == 0) {
            for (int k = 0; k < 4; k++) tcFiner[k] += vary_tc[i] * ((k / apply_free) % 2);
            apply_free++;
        } else if (dir_dim[i] == 1) {
            for (int k = 0; k < 4; k++) tcFiner[k] += vary_tc[i];
        }
    }
    int same = -1;
    if (nzero == 2) {
        same = 1;
        for (int i = 0; i < 3; i++) {
            if (dir_dim[i] != 0) same += 8 * i;
            if (dir_dim[i] == 1) same += 4;
        }
    } else if (nzero == 1) {
        same = 25;
        int af = 1;
        for (int i = 0; i < 3; i++) {
            if (dir_dim[i] == 0) same += 8 * (2 - i);
            else if (dir_dim[i] == 1) { same += af * 2; af++; }
            else af++;
        }
    } else {
        same = 49;
        for (int i = 0; i < 3; i++) if (dir_dim[i] == 1) same += 1 << i;
    }
    int coarser = -1;
    const int tc_last = tc_last_digit(B);
    for (int k = 0; k < dir_free; k++) if (tc_last == tcFiner[k]) coarser = same + k;

    int *nbr = o.nb.data() + size_t(ib) * 168;
    int d[3] = {dir_dim[0], dir_dim[1], dim == 3 ? dir_dim[2] : 0};
    int cn[3] = {0, 0, 0};
    // with overlapping (full-tree) search every existing same, finer and
    // coarser neighbour is recorded
    if (level == 0) {
        nbr[same - 1] = ib;
        if (!overlapping) return;
    } else {
        adjacent(B.c, d, level, dim, cn);
        int idn = find_block(o, level, cn);
        if (idn >= 0) {
            nbr[same - 1] = idn;
            if (!overlapping) return;
        }
    }
    if (level < o.cfg.Jmax) {
        for (int k = 0; k < dir_free; k++) {
            int dig = tcFiner[k];
            int vc[3] = {2 * B.c[0] + ((dig >> 1) & 1), 2 * B.c[1] + (dig & 1), 2 * B.c[2] + ((dig >> 2) & 1)};
            if (dim == 2) vc[2] = 0;
            int cf[3];
            adjacent(vc, d, level + 1, dim, cf);
            int idf = find_block(o, level + 1, cf);
            if (idf >= 0) nbr[same + k - 1 + 2 * 56] = idf;
            else break;
            if (!overlapping && k == dir_free - 1) return;
        }
    }
    if (coarser != -1 && level > o.cfg.Jmin) {
        int cp[3] = {cn[0] >> 1, cn[1] >> 1, cn[2] >> 1};
        if (dim == 2) cp[2] = 0;
        int idc = find_block(o, level - 1, cp);
        if (idc >= 0) nbr[coarser - 1 + 56] = idc;
    }
}

static void update_neighbors(Oracle &o, bool overlapping = false) {
    rebuild_lookup(o);
    const int nb = (int)o.blocks.size();
    o.nb.assign(size_t(nb) * 168, -1);
    const int dim = o.cfg.dim;
    for (int ib = 0; ib < nb; ib++) {
        for (int dz = (dim == 3 ? -1 : 0); dz <= (dim == 3 ? 1 : 0); dz++)
            for (int dy = -1; dy <= 1; dy++)
                for (int dx = -1; dx <= 1; dx++) {
                    if (dx == 0 && dy == 0 && dz == 0) continue;
                    int dd[3] = {dx, dy, dz};
                    find_neighbor(o, ib, dd, overlapping);
                }
    }
}

// ---------------------------------------------------------------------------
// patch geometry (LIB/TREE/neighborhood.f90, LIB/MPI/calc_data_bounds.f90)
// idx(1:2,1:3) kept as idx[lr][dim] with 1-based values.
// ---------------------------------------------------------------------------
static bool in_list(int r, std::initializer_list<int> l) {
    for (int v : l) if (v == r) return true;
    return false;
}

// get_indices_of_modify_patch (neighborhood.f90:23-126)
static void modify_patch(int dim, int relation, int idx[2][3], const int N[3], const int Ns[3], const int Ne[3],
                         const int gm[3], const int gp[3], int lvlDiff) {
    int r = relation > 56 ? (relation - 1) % 56 + 1 : relation;
    for (int d = 0; d < 3; d++) { idx[0][d] = 1; idx[1][d] = 1; }
    for (int d = 0; d < dim; d++) { idx[0][d] = 1 + gm[d]; idx[1][d] = N[d] - gp[d]; }
    if (in_list(r, {1, 2, 3, 4, 25, 26, 29, 30, 33, 34, 37, 38, 49, 51, 53, 55})) idx[1][0] = Ns[0] + gm[0];
    if (in_list(r, {5, 6, 7, 8, 27, 28, 31, 32, 35, 36, 39, 40, 50, 52, 54, 56})) idx[0][0] = N[0] - Ne[0] - gp[0] + 1;
    if (in_list(r, {9, 10, 11, 12, 25, 26, 27, 28, 41, 42, 45, 46, 49, 50, 53, 54})) idx[1][1] = Ns[1] + gm[1];
    if (in_list(r, {13, 14, 15, 16, 29, 30, 31, 32, 43, 44, 47, 48, 51, 52, 55, 56})) idx[0][1] = N[1] - Ne[1] - gp[1] + 1;
    if (in_list(r, {17, 18, 19, 20, 33, 34, 35, 36, 41, 42, 43, 44, 49, 50, 51, 52})) idx[1][2] = Ns[2] + gm[2];
    if (in_list(r, {21, 22, 23, 24, 37, 38, 39, 40, 45, 46, 47, 48, 53, 54, 55, 56})) idx[0][2] = N[2] - Ne[2] - gp[2] + 1;
    if (lvlDiff == -1) {
        if (in_list(r, {10, 12, 14, 16, 18, 20, 22, 24, 42, 44, 46, 48})) idx[0][0] = N[0] / 2 - Ne[0] + 2;
        if (in_list(r, {9, 11, 13, 15, 17, 19, 21, 23, 41, 43, 45, 47})) idx[1][0] = N[0] / 2 + Ns[0];
        if (in_list(r, {2, 4, 6, 8, 19, 20, 23, 24, 34, 36, 38, 40})) idx[0][1] = N[1] / 2 - Ne[1] + 2;
        if (in_list(r, {1, 3, 5, 7, 17, 18, 21, 22, 33, 35, 37, 39})) idx[1][1] = N[1] / 2 + Ns[1];
        if (dim == 3) {
            if (in_list(r, {3, 4, 7, 8, 11, 12, 15, 16, 26, 28, 30, 32})) idx[0][2] = N[2] / 2 - Ne[2] + 2;
            if (in_list(r, {1, 2, 5, 6, 9, 10, 13, 14, 25, 27, 29, 31})) idx[1][2] = N[2] / 2 + Ns[2];
        }
    }
}

// get_indices_of_ghost_patch (neighborhood.f90:158-327), neighbour relations only
static void ghost_patch(const int Bs[3], int g, int dim, int relation, int idx[2][3], int gminus, int gplus, int lvl_diff) {
    int r = relation > 56 ? (relation - 1) % 56 + 1 : relation;
    for (int d = 0; d < 3; d++) { idx[0][d] = 1; idx[1][d] = 1; }
    for (int d = 0; d < dim; d++) { idx[0][d] = g + 1; idx[1][d] = g + Bs[d]; }
    if (in_list(r, {1, 2, 3, 4, 25, 26, 29, 30, 33, 34, 37, 38, 49, 51, 53, 55})) { idx[0][0] = g - gminus + 1; idx[1][0] = g; }
    if (in_list(r, {5, 6, 7, 8, 27, 28, 31, 32, 35, 36, 39, 40, 50, 52, 54, 56})) { idx[0][0] = Bs[0] + g + 1; idx[1][0] = Bs[0] + g + gplus; }
    if (in_list(r, {9, 10, 11, 12, 25, 26, 27, 28, 41, 42, 45, 46, 49, 50, 53, 54})) { idx[0][1] = g - gminus + 1; idx[1][1] = g; }
    if (in_list(r, {13, 14, 15, 16, 29, 30, 31, 32, 43, 44, 47, 48, 51, 52, 55, 56})) { idx[0][1] = Bs[1] + g + 1; idx[1][1] = Bs[1] + g + gplus; }
    if (in_list(r, {17, 18, 19, 20, 33, 34, 35, 36, 41, 42, 43, 44, 49, 50, 51, 52})) { idx[0][2] = g - gminus + 1; idx[1][2] = g; }
    if (in_list(r, {21, 22, 23, 24, 37, 38, 39, 40, 45, 46, 47, 48, 53, 54, 55, 56})) { idx[0][2] = Bs[2] + g + 1; idx[1][2] = Bs[2] + g + gplus; }
    if (in_list(r, {10, 12, 14, 16, 18, 20, 22, 24, 42, 44, 46, 48})) {
        if (lvl_diff == +1) idx[0][0] = g - gminus + 1;
        else if (lvl_diff == -1) idx[0][0] = g + Bs[0] / 2 + 1;
        idx[1][0] = Bs[0] + g;
    }
    if (in_list(r, {9, 11, 13, 15, 17, 19, 21, 23, 41, 43, 45, 47})) {
        idx[0][0] = g + 1;
        if (lvl_diff == +1) idx[1][0] = Bs[0] + g + gplus;
        else if (lvl_diff == -1) idx[1][0] = g + Bs[0] / 2;
    }
    if (in_list(r, {2, 4, 6, 8, 19, 20, 23, 24, 34, 36, 38, 40})) {
        if (lvl_diff == +1) idx[0][1] = g - gminus + 1;
        else if (lvl_diff == -1) idx[0][1] = g + Bs[1] / 2 + 1;
        idx[1][1] = Bs[1] + g;
    }
    if (in_list(r, {1, 3, 5, 7, 17, 18, 21, 22, 33, 35, 37, 39})) {
        idx[0][1] = g + 1;
        if (lvl_diff == +1) idx[1][1] = Bs[1] + g + gplus;
        else if (lvl_diff == -1) idx[1][1] = g + Bs[1] / 2;
    }
    if (dim == 3) {
        if (in_list(r, {3, 4, 7, 8, 11, 12, 15, 16, 26, 28, 30, 32})) {
            if (lvl_diff == +1) idx[0][2] = g - gminus + 1;
            else if (lvl_diff == -1) idx[0][2] = g + Bs[2] / 2 + 1;
            idx[1][2] = Bs[2] + g;
        }
        if (in_list(r, {1, 2, 5, 6, 9, 10, 13, 14, 25, 27, 29, 31})) {
            idx[0][2] = g + 1;
            if (lvl_diff == +1) idx[1][2] = Bs[2] + g + gplus;
            else if (lvl_diff == -1) idx[1][2] = g + Bs[2] / 2;
        }
    }
}

// set_send_bounds (calc_data_bounds.f90:46-147)
static void send_bounds(const wg_config &cfg, int order_predictor, int relation, int lvl_diff, int gminus, int gplus,
                        int bounds[2][3], int buffer[2][3]) {
    const int g = cfg.g, dim = cfg.dim;
    int n[3] = {1, 1, 1};
    for (int d = 0; d < dim; d++) n[d] = cfg.Bs[d] + 2 * g;
    int a = order_predictor / 2 - 1;
    for (int d = 0; d < 3; d++) { bounds[0][d] = bounds[1][d] = 1; buffer[0][d] = buffer[1][d] = 1; }
    int gm3[3] = {g, g, g};
    if (lvl_diff == 0) {
        int Ns[3] = {gminus, gminus, gminus}, Ne[3] = {gplus, gplus, gplus};
        modify_patch(dim, relation, bounds, n, Ns, Ne, gm3, gm3, 0);
    } else if (lvl_diff == +1) {
        int Ns[3] = {gminus * 2 - 1, gminus * 2 - 1, gminus * 2 - 1}, Ne[3] = {gplus * 2 - 1, gplus * 2 - 1, gplus * 2 - 1};
        int gp[3] = {g + 1, g + 1, g + 1};
        modify_patch(dim, relation, bounds, n, Ns, Ne, gm3, gp, +1);
        for (int d = 0; d < dim; d++) {
            int Nsender = bounds[1][d] - bounds[0][d] + 1;
            buffer[1][d] = (Nsender + 1) / 2;
        }
    } else if (lvl_diff == -1) {
        int Ns[3] = {gminus / 2 + 1, gminus / 2 + 1, gminus / 2 + 1};
        int Ne[3] = {(gplus + 1) / 2 + 1, (gplus + 1) / 2 + 1, (gplus + 1) / 2 + 1};
        int gp[3] = {g - 1, g - 1, g - 1};
        modify_patch(dim, relation, bounds, n, Ns, Ne, gm3, gp, -1);
        for (int d = 0; d < dim; d++) { bounds[0][d] -= a; bounds[1][d] += a; }
        for (int d = 0; d < dim; d++) {
            if (bounds[0][d] == g + 1 - a || gminus % 2 == 0) buffer[0][d] = 1 + a * 2;
            else buffer[0][d] = 2 + a * 2;
            buffer[1][d] = buffer[0][d] + gplus - 1;
            if (bounds[1][d] - bounds[0][d] > g + a) buffer[1][d] += cfg.Bs[d];
        }
    }
}

// inverse_relation (neighborhood.f90:347-381)
static int inverse_relation(int relation) {
    int inv = (relation - 1) % 56 + 1;
    if (relation > 56) inv += (3 - (relation - 1) / 56) * 56;
    int m = (relation - 1) % 56;
    for (int i_dim = 3; i_dim >= 3 - m / 24; i_dim--) {
        int p = 1 << i_dim, h = 1 << (i_dim - 1);
        if ((relation - 1) % p >= h) inv -= h;
        else inv += h;
    }
    return inv;
}

// ---------------------------------------------------------------------------
// prediction (module_wavelets.f90:96-284): coarse(n) -> fine(2n-1), in place
// on a dense x-fastest array
// ---------------------------------------------------------------------------
static void prediction(const double *coarse, int cx, int cy, int cz, double *fine, int order) {
    const int fx = 2 * cx - 1, fy = 2 * cy - 1, fz = 2 * cz - 1;
    auto F = [&](int i, int j, int k) -> double & { return fine[((size_t)(k - 1) * fy + (j - 1)) * fx + (i - 1)]; };
    double c[8];
    int nc;
    if (order == 2) { nc = 2; c[0] = 0.5; c[1] = 0.5; }
    else if (order == 4) { nc = 4; c[0] = -1.0 / 16.0; c[1] = 9.0 / 16.0; c[2] = 9.0 / 16.0; c[3] = -1.0 / 16.0; }
    else if (order == 6) { nc = 6; double v[] = {3, -25, 150, 150, -25, 3}; for (int i = 0; i < 6; i++) c[i] = v[i] / 256.0; }
    else { nc = 8; double v[] = {-5, 49, -245, 1225, 1225, -245, 49, -5}; for (int i = 0; i < 8; i++) c[i] = v[i] / 2048.0; }
    // ( -1.0_rk, 9.0_rk, 9.0_rk, -1.0_rk ) / 16.0_rk : elementwise division
    for (int k = 1; k <= fz; k++) for (int j = 1; j <= fy; j++) for (int i = 1; i <= fx; i++)
        if (i % 2 == 0 || j % 2 == 0 || k % 2 == 0) F(i, j, k) = 0.0;
    for (int k = 1; k <= cz; k++) for (int j = 1; j <= cy; j++) for (int i = 1; i <= cx; i++)
        F(2 * i - 1, 2 * j - 1, 2 * k - 1) = coarse[((size_t)(k - 1) * cy + (j - 1)) * cx + (i - 1)];
    const int h = nc - 1;  // offsets -h,-h+2,...,+h
    auto interp = [&](auto get) -> double {
        double s = c[0] * get(-h);
        for (int m = 1; m < nc; m++) s = s + c[m] * get(-h + 2 * m);
        return s;
    };
    for (int k = 1; k <= fz; k += 2) {
        for (int j = 1; j <= fy; j += 2)
            for (int i = nc; i <= fx - (nc - 1); i += 2)
                F(i, j, k) = interp([&](int o) { return F(i + o, j, k); });
        for (int j = nc; j <= fy - (nc - 1); j += 2)
            for (int i = 1; i <= fx; i++)
                F(i, j, k) = interp([&](int o) { return F(i, j + o, k); });
    }
    for (int k = nc; k <= fz - (nc - 1); k += 2)
        for (int j = 1; j <= fy; j++)
            for (int i = 1; i <= fx; i++)
                F(i, j, k) = interp([&](int o) { return F(i, j, k + o); });
}

// ---------------------------------------------------------------------------
// ghost-node synchronisation: sync_ghosts_generic (synchronize_ghosts_generic.f90)
// with unpack_ghostlayers_internal (xfer_block_data.f90:321-437), leaf-only grid.
// The restriction is plain decimation (ignore_Filter, RHS sync) or, for
// lifted wavelets without ignore_Filter, the HD-filtered variant.
// ---------------------------------------------------------------------------
static void hd_filter_block(const Oracle &o, int b, std::vector<double> &out);

// one transfer of a sync stage: sender ib -> receiver in through relation i_n
struct Xfer {
    int ib, in, i_n, lvl_diff;
};

// per-thread scratch of the transfers (prediction patches, filtered sender)
struct XferScratch {
    std::vector<double> coarse, fine, filtered;
    int filtered_id = -1;
};

static void do_xfer(Oracle &o, const Xfer &x, int gminus, int gplus, bool ignore_filter, XferScratch &sc) {
    const wg_config &cfg = o.cfg;
    const int dim = cfg.dim;
    const int ib = x.ib, in = x.in, i_n = x.i_n, lvl_diff = x.lvl_diff;
    const int inv = inverse_relation(i_n);
    int recv[2][3], sb[2][3], buf[2][3];
    ghost_patch(cfg.Bs, cfg.g, dim, inv, recv, gminus, gplus, -lvl_diff);
    send_bounds(cfg, o.wav.order_predictor, i_n, lvl_diff, gminus, gplus, sb, buf);
    double *dst = o.blk(in);
    const double *src = o.blk(ib);
    if (lvl_diff == 0) {
        for (int c = 1; c <= o.nc; c++)
            for (int k = recv[0][2], ks = sb[0][2]; k <= recv[1][2]; k++, ks++)
                for (int j = recv[0][1], js = sb[0][1]; j <= recv[1][1]; j++, js++)
                    for (int i = recv[0][0], is = sb[0][0]; i <= recv[1][0]; i++, is++)
                        dst[o.at(i, j, k, c)] = src[o.at(is, js, ks, c)];
    } else if (lvl_diff == +1) {
        const double *srcf = src;
        if (!ignore_filter && o.wav.lifted) {
            if (sc.filtered_id != ib) { hd_filter_block(o, ib, sc.filtered); sc.filtered_id = ib; }
            srcf = sc.filtered.data();
        }
        // res_data(1:...) = src(ijk(1):ijk(2):2), then receiver takes res_data(buffer box)
        for (int c = 1; c <= o.nc; c++)
            for (int k = recv[0][2], kb = buf[0][2]; k <= recv[1][2]; k++, kb++)
                for (int j = recv[0][1], jb = buf[0][1]; j <= recv[1][1]; j++, jb++)
                    for (int i = recv[0][0], ib2 = buf[0][0]; i <= recv[1][0]; i++, ib2++) {
                        int is = sb[0][0] + 2 * (ib2 - 1);
                        int js = sb[0][1] + 2 * (jb - 1);
                        int ks = (dim == 3) ? sb[0][2] + 2 * (kb - 1) : 1;
                        dst[o.at(i, j, k, c)] = srcf[o.at(is, js, ks, c)];
                    }
    } else {
        const int cx = sb[1][0] - sb[0][0] + 1, cy = sb[1][1] - sb[0][1] + 1, cz = sb[1][2] - sb[0][2] + 1;
        const int fx = 2 * cx - 1, fy = 2 * cy - 1;
        sc.coarse.resize(size_t(cx) * cy * cz);
        sc.fine.resize(size_t(fx) * fy * (2 * cz - 1));
        for (int c = 1; c <= o.nc; c++) {
            size_t p = 0;
            for (int k = sb[0][2]; k <= sb[1][2]; k++)
                for (int j = sb[0][1]; j <= sb[1][1]; j++)
                    for (int i = sb[0][0]; i <= sb[1][0]; i++) sc.coarse[p++] = src[o.at(i, j, k, c)];
            prediction(sc.coarse.data(), cx, cy, cz, sc.fine.data(), o.wav.order_predictor);
            for (int k = recv[0][2], kb = buf[0][2]; k <= recv[1][2]; k++, kb++)
                for (int j = recv[0][1], jb = buf[0][1]; j <= recv[1][1]; j++, jb++)
                    for (int i = recv[0][0], ib2 = buf[0][0]; i <= recv[1][0]; i++, ib2++)
                        dst[o.at(i, j, k, c)] = sc.fine[(size_t(kb - 1) * fy + (jb - 1)) * fx + (ib2 - 1)];
        }
    }
}

// whether a transfer reads ghost nodes of its sender (the filtered
// restriction reads the whole block)
static bool xfer_reads_ghosts(const Oracle &o, const Xfer &x, int gminus, int gplus, bool ignore_filter) {
    const wg_config &cfg = o.cfg;
    if (x.lvl_diff == +1 && !ignore_filter && o.wav.lifted) return true;
    int sb[2][3], buf[2][3];
    send_bounds(cfg, o.wav.order_predictor, x.i_n, x.lvl_diff, gminus, gplus, sb, buf);
    for (int d = 0; d < cfg.dim; d++)
        if (sb[0][d] < cfg.g + 1 || sb[1][d] > cfg.g + cfg.Bs[d]) return true;
    return false;
}

// sync_ghosts_generic's stages on one process: in stage 1 the same-level
// copies (and, unlifted, the restrictions), then the restrictions (lifted),
// then the predictions; within a stage the transfers run in the order of the
// sending blocks and their relations (unpack_ghostlayers_internal). With
// several threads the receiving blocks of a stage are processed in parallel,
// each receiver's transfers in that same order, which gives the sequential
// result unless a sender reads ghost nodes that the same stage writes; such
// stages run sequentially.
static void sync_ghosts(Oracle &o, int gminus, int gplus, bool ignore_filter) {
    const int nstages = o.wav.lifted ? 3 : 2;
    const int isUnlifted = o.wav.lifted ? 0 : 1;
    const int nblk = (int)o.blocks.size();
    for (int istage = 1; istage <= nstages; istage++) {
        std::vector<Xfer> xs;
        for (int ib = 0; ib < nblk; ib++) {
            const int level = o.blocks[ib].level;
            for (int i_n = 1; i_n <= 168; i_n++) {
                const int in = o.nb[size_t(ib) * 168 + i_n - 1];
                if (in < 0) continue;
                const int lvl_diff = level - o.blocks[in].level;
                bool send = (istage == 1 && lvl_diff == 0) || (istage == 2 - isUnlifted && lvl_diff == +1) ||
                            (istage == 3 - isUnlifted && lvl_diff == -1);
                if (send) xs.push_back({ib, in, i_n, lvl_diff});
            }
        }
        bool parallel = o.nthreads > 1;
        if (parallel) {
            std::vector<char> recv(nblk, 0), reads(nblk, 0);
            for (const Xfer &x : xs) {
                recv[x.in] = 1;
                if (!reads[x.ib] && xfer_reads_ghosts(o, x, gminus, gplus, ignore_filter)) reads[x.ib] = 1;
            }
            for (int b = 0; b < nblk && parallel; b++)
                if (recv[b] && reads[b]) parallel = false;
        }
        if (!parallel) {
            XferScratch sc;
            for (const Xfer &x : xs) do_xfer(o, x, gminus, gplus, ignore_filter, sc);
            continue;
        }
        std::vector<int> first(nblk + 1, 0), order(xs.size());
        for (const Xfer &x : xs) first[x.in + 1]++;
        for (int b = 0; b < nblk; b++) first[b + 1] += first[b];
        {
            std::vector<int> fill(first.begin(), first.end() - 1);
            for (int k = 0; k < (int)xs.size(); k++) order[fill[xs[k].in]++] = k;
        }
#pragma omp parallel num_threads(o.nthreads)
        {
            XferScratch sc;
#pragma omp for schedule(dynamic, 4)
            for (int b = 0; b < nblk; b++)
                for (int k = first[b]; k < first[b + 1]; k++) do_xfer(o, xs[order[k]], gminus, gplus, ignore_filter, sc);
        }
    }
}

// HD filter of a whole block (blockFilterXYZ_vct with do_restriction, used by
// restrict_copy_at_CE for lifted wavelets). Filters x, then y, then z where the
// filter support stays inside the block; other points keep the input values.
static void hd_filter_block(const Oracle &o, int b, std::vector<double> &out) {
    const Filter &HD = o.wav.HD;
    const double *u = o.blk(b);
    out.assign(u, u + size_t(o.nc) * o.npts);
    std::vector<double> tmp(out);
    const int dim = o.cfg.dim;
    int n[3] = {o.nx, o.ny, o.nz};
    for (int d = 0; d < dim; d++) {
        tmp = out;
        for (int c = 1; c <= o.nc; c++)
            for (int k = 1; k <= n[2]; k++)
                for (int j = 1; j <= n[1]; j++)
                    for (int i = 1; i <= n[0]; i++) {
                        int p[3] = {i, j, k};
                        if (p[d] + HD.lo < 1 || p[d] + HD.hi > n[d]) continue;
                        double s = 0.0;
                        bool first = true;
                        for (int m = HD.lo; m <= HD.hi; m++) {
                            int q[3] = {i, j, k};
                            q[d] += m;
                            double v = HD(m) * tmp[o.at(q[0], q[1], q[2], c)];
                            s = first ? v : s + v;
                            first = false;
                        }
                        out[o.at(i, j, k, c)] = s;
                    }
    }
}

// ---------------------------------------------------------------------------
// ACM right-hand side, FD_4th_central (LIB/EQUATION/ACMnew/rhs_ACM.f90)
// ---------------------------------------------------------------------------
static const double a_FD4[5] = {1.0 / 12.0, -2.0 / 3.0, 0.0, 2.0 / 3.0, -1.0 / 12.0};
static const double b_FD4[5] = {-1.0 / 12.0, 4.0 / 3.0, -5.0 / 2.0, 4.0 / 3.0, -1.0 / 12.0};
#define A(i) a_FD4[(i) + 2]
#define B(i) b_FD4[(i) + 2]

static void rhs_2d(const Oracle &o, const double *phi, const double *mask, const double dx[3], double *rhs) {
    const wg_config &p = o.cfg;
    const int g = p.g, Bs0 = p.Bs[0], Bs1 = p.Bs[1];
    const double dx_inv = 1.0 / dx[0], dy_inv = 1.0 / dx[1];
    const double dx2_inv = 1.0 / (dx[0] * dx[0]), dy2_inv = 1.0 / (dx[1] * dx[1]);
    const double c_0 = p.c0, nu = p.nu, gamma = p.gamma_p;
    double Ceta_inv[8];
    for (int i = 0; i < 8; i++) Ceta_inv[i] = 1.0 / p.C_eta;
    Ceta_inv[0] = 0.0;
    auto P = [&](int ix, int iy, int ic) { return phi[o.at(ix, iy, 1, ic)]; };
    auto M = [&](int ix, int iy, int ic) { return mask ? mask[o.at(ix, iy, 1, ic)] : 0.0; };
    for (int iy = g + 1; iy <= Bs1 + g; iy++)
        for (int ix = g + 1; ix <= Bs0 + g; ix++) {
            double u_dx = (A(-2) * P(ix - 2, iy, 1) + A(-1) * P(ix - 1, iy, 1) + A(1) * P(ix + 1, iy, 1) + A(2) * P(ix + 2, iy, 1)) * dx_inv;
            double v_dx = (A(-2) * P(ix - 2, iy, 2) + A(-1) * P(ix - 1, iy, 2) + A(1) * P(ix + 1, iy, 2) + A(2) * P(ix + 2, iy, 2)) * dx_inv;
            double p_dx = (A(-2) * P(ix - 2, iy, 3) + A(-1) * P(ix - 1, iy, 3) + A(1) * P(ix + 1, iy, 3) + A(2) * P(ix + 2, iy, 3)) * dx_inv;
            double u_dy = (A(-2) * P(ix, iy - 2, 1) + A(-1) * P(ix, iy - 1, 1) + A(1) * P(ix, iy + 1, 1) + A(2) * P(ix, iy + 2, 1)) * dy_inv;
            double v_dy = (A(-2) * P(ix, iy - 2, 2) + A(-1) * P(ix, iy - 1, 2) + A(1) * P(ix, iy + 1, 2) + A(2) * P(ix, iy + 2, 2)) * dy_inv;
            double p_dy = (A(-2) * P(ix, iy - 2, 3) + A(-1) * P(ix, iy - 1, 3) + A(1) * P(ix, iy + 1, 3) + A(2) * P(ix, iy + 2, 3)) * dy_inv;
            double u_dxdx = (B(-2) * P(ix - 2, iy, 1) + B(-1) * P(ix - 1, iy, 1) + B(0) * P(ix, iy, 1) + B(1) * P(ix + 1, iy, 1) + B(2) * P(ix + 2, iy, 1)) * dx2_inv;
            double v_dxdx = (B(-2) * P(ix - 2, iy, 2) + B(-1) * P(ix - 1, iy, 2) + B(0) * P(ix, iy, 2) + B(1) * P(ix + 1, iy, 2) + B(2) * P(ix + 2, iy, 2)) * dx2_inv;
            double u_dydy = (B(-2) * P(ix, iy - 2, 1) + B(-1) * P(ix, iy - 1, 1) + B(0) * P(ix, iy, 1) + B(1) * P(ix, iy + 1, 1) + B(2) * P(ix, iy + 2, 1)) * dy2_inv;
            double v_dydy = (B(-2) * P(ix, iy - 2, 2) + B(-1) * P(ix, iy - 1, 2) + B(0) * P(ix, iy, 2) + B(1) * P(ix, iy + 1, 2) + B(2) * P(ix, iy + 2, 2)) * dy2_inv;
            double div_U = u_dx + v_dy;
            int color = (int)M(ix, iy, 5);
            double penalx = -M(ix, iy, 1) * Ceta_inv[color] * (P(ix, iy, 1) - M(ix, iy, 2));
            double penaly = -M(ix, iy, 1) * Ceta_inv[color] * (P(ix, iy, 2) - M(ix, iy, 3));
            double r1, r2;
            if (p.skew_symmetry) {
                double uu_dx = (A(-2) * P(ix - 2, iy, 1) * P(ix - 2, iy, 1) + A(-1) * P(ix - 1, iy, 1) * P(ix - 1, iy, 1) + A(1) * P(ix + 1, iy, 1) * P(ix + 1, iy, 1) + A(2) * P(ix + 2, iy, 1) * P(ix + 2, iy, 1)) * dx_inv;
                double uv_dy = (A(-2) * P(ix, iy - 2, 1) * P(ix, iy - 2, 2) + A(-1) * P(ix, iy - 1, 1) * P(ix, iy - 1, 2) + A(1) * P(ix, iy + 1, 1) * P(ix, iy + 1, 2) + A(2) * P(ix, iy + 2, 1) * P(ix, iy + 2, 2)) * dy_inv;
                double vu_dx = (A(-2) * P(ix - 2, iy, 2) * P(ix - 2, iy, 1) + A(-1) * P(ix - 1, iy, 2) * P(ix - 1, iy, 1) + A(1) * P(ix + 1, iy, 2) * P(ix + 1, iy, 1) + A(2) * P(ix + 2, iy, 2) * P(ix + 2, iy, 1)) * dx_inv;
                double vv_dy = (A(-2) * P(ix, iy - 2, 2) * P(ix, iy - 2, 2) + A(-1) * P(ix, iy - 1, 2) * P(ix, iy - 1, 2) + A(1) * P(ix, iy + 1, 2) * P(ix, iy + 1, 2) + A(2) * P(ix, iy + 2, 2) * P(ix, iy + 2, 2)) * dy_inv;
                r1 = -0.5 * (uu_dx + uv_dy + P(ix, iy, 1) * u_dx + P(ix, iy, 2) * u_dy) - p_dx + nu * (u_dxdx + u_dydy) + penalx;
                r2 = -0.5 * (vu_dx + vv_dy + P(ix, iy, 1) * v_dx + P(ix, iy, 2) * v_dy) - p_dy + nu * (v_dxdx + v_dydy) + penaly;
            } else {
                r1 = -P(ix, iy, 1) * u_dx - P(ix, iy, 2) * u_dy - p_dx + nu * (u_dxdx + u_dydy) + penalx;
                r2 = -P(ix, iy, 1) * v_dx - P(ix, iy, 2) * v_dy - p_dy + nu * (v_dxdx + v_dydy) + penaly;
            }
            double r3 = -(c_0 * c_0) * div_U - gamma * P(ix, iy, 3);
            if (p.use_sponge) {
                double spo = M(ix, iy, 6) * (1.0 / p.C_sponge);
                r1 = r1 - (P(ix, iy, 1) - p.u_mean_set[0]) * spo;
                r2 = r2 - (P(ix, iy, 2) - p.u_mean_set[1]) * spo;
                r3 = r3 - P(ix, iy, 3) * spo;
            }
            rhs[o.at(ix, iy, 1, 1)] = r1;
            rhs[o.at(ix, iy, 1, 2)] = r2;
            rhs[o.at(ix, iy, 1, 3)] = r3;
        }
}

static void rhs_3d(const Oracle &o, const double *phi, const double *mask, const double dx[3], double *rhs) {
    const wg_config &p = o.cfg;
    const int g = p.g;
    const double dx_inv = 1.0 / dx[0], dy_inv = 1.0 / dx[1], dz_inv = 1.0 / dx[2];
    const double dx2_inv = 1.0 / (dx[0] * dx[0]), dy2_inv = 1.0 / (dx[1] * dx[1]), dz2_inv = 1.0 / (dx[2] * dx[2]);
    const double c_0 = p.c0, nu = p.nu, gamma = p.gamma_p;
    double Ceta_inv[8];
    for (int i = 0; i < 8; i++) Ceta_inv[i] = 1.0 / p.C_eta;
    Ceta_inv[0] = 0.0;
    auto P = [&](int ix, int iy, int iz, int ic) { return phi[o.at(ix, iy, iz, ic)]; };
    auto M = [&](int ix, int iy, int iz, int ic) { return mask ? mask[o.at(ix, iy, iz, ic)] : 0.0; };
#define D1X(c) ((A(-2) * P(ix - 2, iy, iz, c) + A(-1) * P(ix - 1, iy, iz, c) + A(1) * P(ix + 1, iy, iz, c) + A(2) * P(ix + 2, iy, iz, c)) * dx_inv)
#define D1Y(c) ((A(-2) * P(ix, iy - 2, iz, c) + A(-1) * P(ix, iy - 1, iz, c) + A(1) * P(ix, iy + 1, iz, c) + A(2) * P(ix, iy + 2, iz, c)) * dy_inv)
#define D1Z(c) ((A(-2) * P(ix, iy, iz - 2, c) + A(-1) * P(ix, iy, iz - 1, c) + A(1) * P(ix, iy, iz + 1, c) + A(2) * P(ix, iy, iz + 2, c)) * dz_inv)
#define D2X(c) ((B(-2) * P(ix - 2, iy, iz, c) + B(-1) * P(ix - 1, iy, iz, c) + B(0) * P(ix, iy, iz, c) + B(1) * P(ix + 1, iy, iz, c) + B(2) * P(ix + 2, iy, iz, c)) * dx2_inv)
#define D2Y(c) ((B(-2) * P(ix, iy - 2, iz, c) + B(-1) * P(ix, iy - 1, iz, c) + B(0) * P(ix, iy, iz, c) + B(1) * P(ix, iy + 1, iz, c) + B(2) * P(ix, iy + 2, iz, c)) * dy2_inv)
#define D2Z(c) ((B(-2) * P(ix, iy, iz - 2, c) + B(-1) * P(ix, iy, iz - 1, c) + B(0) * P(ix, iy, iz, c) + B(1) * P(ix, iy, iz + 1, c) + B(2) * P(ix, iy, iz + 2, c)) * dz2_inv)
#define PX(a, b) ((A(-2) * P(ix - 2, iy, iz, a) * P(ix - 2, iy, iz, b) + A(-1) * P(ix - 1, iy, iz, a) * P(ix - 1, iy, iz, b) + A(1) * P(ix + 1, iy, iz, a) * P(ix + 1, iy, iz, b) + A(2) * P(ix + 2, iy, iz, a) * P(ix + 2, iy, iz, b)) * dx_inv)
#define PY(a, b) ((A(-2) * P(ix, iy - 2, iz, a) * P(ix, iy - 2, iz, b) + A(-1) * P(ix, iy - 1, iz, a) * P(ix, iy - 1, iz, b) + A(1) * P(ix, iy + 1, iz, a) * P(ix, iy + 1, iz, b) + A(2) * P(ix, iy + 2, iz, a) * P(ix, iy + 2, iz, b)) * dy_inv)
#define PZ(a, b) ((A(-2) * P(ix, iy, iz - 2, a) * P(ix, iy, iz - 2, b) + A(-1) * P(ix, iy, iz - 1, a) * P(ix, iy, iz - 1, b) + A(1) * P(ix, iy, iz + 1, a) * P(ix, iy, iz + 1, b) + A(2) * P(ix, iy, iz + 2, a) * P(ix, iy, iz + 2, b)) * dz_inv)
    for (int iz = g + 1; iz <= p.Bs[2] + g; iz++)
        for (int iy = g + 1; iy <= p.Bs[1] + g; iy++)
            for (int ix = g + 1; ix <= p.Bs[0] + g; ix++) {
                double u_dx = D1X(1), v_dx = D1X(2), w_dx = D1X(3), p_dx = D1X(4);
                double u_dy = D1Y(1), v_dy = D1Y(2), w_dy = D1Y(3), p_dy = D1Y(4);
                double u_dz = D1Z(1), v_dz = D1Z(2), w_dz = D1Z(3), p_dz = D1Z(4);
                double u_dxdx = D2X(1), v_dxdx = D2X(2), w_dxdx = D2X(3);
                double u_dydy = D2Y(1), v_dydy = D2Y(2), w_dydy = D2Y(3);
                double u_dzdz = D2Z(1), v_dzdz = D2Z(2), w_dzdz = D2Z(3);
                double u = P(ix, iy, iz, 1), v = P(ix, iy, iz, 2), w = P(ix, iy, iz, 3), pp = P(ix, iy, iz, 4);
                double chi = M(ix, iy, iz, 1) * Ceta_inv[(int)M(ix, iy, iz, 5)];
                double penalx = -chi * (u - M(ix, iy, iz, 2));
                double penaly = -chi * (v - M(ix, iy, iz, 3));
                double penalz = -chi * (w - M(ix, iy, iz, 4));
                double r1, r2, r3;
                if (p.skew_symmetry) {
                    double uu_dx = PX(1, 1), uv_dy = PY(1, 2), uw_dz = PZ(1, 3);
                    double vu_dx = PX(2, 1), vv_dy = PY(2, 2), vw_dz = PZ(2, 3);
                    double wu_dx = PX(3, 1), wv_dy = PY(3, 2), ww_dz = PZ(3, 3);
                    r1 = -0.5 * (uu_dx + uv_dy + uw_dz + u * u_dx + v * u_dy + w * u_dz) - p_dx + nu * (u_dxdx + u_dydy + u_dzdz) + penalx;
                    r2 = -0.5 * (vu_dx + vv_dy + vw_dz + u * v_dx + v * v_dy + w * v_dz) - p_dy + nu * (v_dxdx + v_dydy + v_dzdz) + penaly;
                    r3 = -0.5 * (wu_dx + wv_dy + ww_dz + u * w_dx + v * w_dy + w * w_dz) - p_dz + nu * (w_dxdx + w_dydy + w_dzdz) + penalz;
                } else {
                    r1 = (-u * u_dx - v * u_dy - w * u_dz) - p_dx + nu * (u_dxdx + u_dydy + u_dzdz) + penalx;
                    r2 = (-u * v_dx - v * v_dy - w * v_dz) - p_dy + nu * (v_dxdx + v_dydy + v_dzdz) + penaly;
                    r3 = (-u * w_dx - v * w_dy - w * w_dz) - p_dz + nu * (w_dxdx + w_dydy + w_dzdz) + penalz;
                }
                double r4 = -(c_0 * c_0) * (u_dx + v_dy + w_dz) - gamma * pp;
                if (p.use_sponge) {
                    double spo = M(ix, iy, iz, 6) * (1.0 / p.C_sponge);
                    r1 = r1 - (u - p.u_mean_set[0]) * spo;
                    r2 = r2 - (v - p.u_mean_set[1]) * spo;
                    r3 = r3 - (w - p.u_mean_set[2]) * spo;
                    r4 = r4 - pp * spo;
                }
                rhs[o.at(ix, iy, iz, 1)] = r1;
                rhs[o.at(ix, iy, iz, 2)] = r2;
                rhs[o.at(ix, iy, iz, 3)] = r3;
                rhs[o.at(ix, iy, iz, 4)] = r4;
            }
#undef D1X
#undef D1Y
#undef D1Z
#undef D2X
#undef D2Y
#undef D2Z
#undef PX
#undef PY
#undef PZ
}

static void block_spacing(const Oracle &o, int b, double x0[3], double dx[3]) {
    const Block &B = o.blocks[b];
    for (int d = 0; d < 3; d++) {
        x0[d] = 0.0;
        dx[d] = 0.0;
    }
    for (int d = 0; d < o.cfg.dim; d++) {
        dx[d] = std::pow(2.0, -B.level) * o.cfg.domain[d] / (double)o.cfg.Bs[d];
        x0[d] = (double)(B.c[d] * o.cfg.Bs[d]) * dx[d];
    }
}

// ---------------------------------------------------------------------------
// Penalisation mask of one block from the tree's geometry: CREATE_MASK_meta
// (LIB/EQUATION/module_physics_metamodule.f90:38-83, mask = 0, colour = 1)
// -> create_mask_2D_acm / create_mask_3D_acm "all-parts"
// (LIB/EQUATION/ACMnew/create_mask.f90:6-320): draw_circle / draw_sphere
// (LIB/EQUATION/insects/module_geometry.f90:49-117,315-381) with the cosine
// step (step_cosine4, LIB/HELPER/module_helpers.f90:467-487) of width
// h = C_smooth * dx_min(Jmax) and safety h (module_ACM.f90:468-471), then the
// sponge (sponge_2D / sponge_3D, LIB/EQUATION/ACMnew/sponge.f90) on the
// interior. m: 6 components of the full block (at(ix,iy,iz,ic)).
// ---------------------------------------------------------------------------
static const double kPi = 4.0 * std::atan(1.0);

static double step_cosine(double x, double t, double h) {
    const double x_rel = x - t;
    if (x_rel <= -h) return 1.0;
    if (x_rel >= +h) return 0.0;
    return 0.5 * (1.0 + std::cos((x_rel + h) * kPi / (2.0 * h)));
}

static void mask_block(const Oracle &o, int b, double *m) {
    const wg_config &p = o.cfg;
    const wg_geometry &G = o.geom;
    const int g = p.g, dim = p.dim;
    std::fill(m, m + 6 * size_t(o.npts), 0.0);
    for (size_t q = 0; q < size_t(o.npts); q++) m[4 * size_t(o.npts) + q] = 1.0;
    if (!p.penalization) return;
    double x0[3], dx[3];
    block_spacing(o, b, x0, dx);
    double dx_min = 9e9;
    for (int d = 0; d < dim; d++) dx_min = std::min(dx_min, std::pow(2.0, -p.Jmax) * (p.domain[d] / (double)p.Bs[d]));
    const double h = dx_min * G.C_smooth, safety = 1.0 * h;
    if (G.kind == WG_GEOM_CYLINDER || G.kind == WG_GEOM_SPHERE) {
        double dmin = dx[0];
        for (int d = 1; d < dim; d++) dmin = std::min(dmin, dx[d]);
        const int Nsafety = (int)std::ceil(safety / dmin);
        const int n[3] = {o.nx, o.ny, o.nz};
        int lo[3] = {1, 1, 1}, hi[3] = {1, 1, 1};
        for (int d = 0; d < dim; d++) {
            const int bmin = (int)((G.x_cntr[d] - G.R_cyl - x0[d]) / dx[d]) - Nsafety + (g + 1);
            const int bmax = (int)std::ceil((G.x_cntr[d] + G.R_cyl - x0[d]) / dx[d]) + Nsafety + (g + 1);
            lo[d] = std::max(bmin, g + 1);
            hi[d] = std::min(bmax, n[d] - g + 1);
        }
        for (int iz = lo[2]; iz <= hi[2]; iz++)
            for (int iy = lo[1]; iy <= hi[1]; iy++)
                for (int ix = lo[0]; ix <= hi[0]; ix++) {
                    const double xx = (double)(ix - (g + 1)) * dx[0] + x0[0];
                    const double yy = (double)(iy - (g + 1)) * dx[1] + x0[1];
                    double dist;
                    if (dim == 2) {
                        const double a = xx - G.x_cntr[0], c = yy - G.x_cntr[1];
                        dist = std::sqrt(a * a + c * c) - G.R_cyl;
                    } else {
                        const double zz = (double)(iz - (g + 1)) * dx[2] + x0[2];
                        const double a = xx - G.x_cntr[0], c = yy - G.x_cntr[1], e = zz - G.x_cntr[2];
                        dist = std::sqrt(a * a + c * c + e * e) - G.R_cyl;
                    }
                    const double tmp = step_cosine(dist, 0.0, h);
                    double &chi = m[o.at(ix, iy, iz, 1)];
                    if (tmp >= chi) {
                        chi = tmp;
                        m[o.at(ix, iy, iz, 5)] = 1.0;
                    }
                }
    }
    if (!p.use_sponge) return;
    const double Ls = G.L_sponge;
    const int z1 = dim == 3 ? g + 1 : 1, z2 = dim == 3 ? p.Bs[2] + g : 1;
    if (dim == 2) {
        for (int iy = g + 1; iy <= p.Bs[1] + g; iy++)
            for (int ix = g + 1; ix <= p.Bs[0] + g; ix++) {
                double tmp;
                if (G.sponge_type == WG_SPONGE_RECT) {
                    const double x = (double)(ix - (g + 1)) * dx[0] + x0[0];
                    const double y = (double)(iy - (g + 1)) * dx[1] + x0[1];
                    tmp = std::min(std::min(x, y), std::min(-(x - p.domain[0]), -(y - p.domain[1])));
                } else {
                    const double off = 0.5 * p.domain[0];
                    const double y = (double)(iy - (g + 1)) * dx[1] + x0[1] - off;
                    const double x = (double)(ix - (g + 1)) * dx[0] + x0[0] - off;
                    tmp = -(std::pow(std::pow(x, G.p_sponge) + std::pow(y, G.p_sponge), 1.0 / G.p_sponge) - off);
                }
                m[o.at(ix, iy, 1, 6)] = step_cosine(tmp, 0.5 * Ls, 0.5 * Ls);
            }
        return;
    }
    if (G.sponge_type == WG_SPONGE_RECT) {
        double t = 9e99;
        for (int d = 0; d < 3; d++) t = std::min(t, x0[d]);
        for (int d = 0; d < 3; d++) t = std::min(t, p.domain[d] - (x0[d] + dx[d] * (double)p.Bs[d]));
        if (t > Ls) return;
    } else {
        const double off = 0.5 * p.domain[0], pp = G.p_sponge, pinv = 1.0 / pp;
        double e[3];
        for (int d = 0; d < 3; d++)
            e[d] = std::pow(std::max(std::fabs(x0[d] - off), std::fabs(x0[d] + dx[d] * (double)p.Bs[d] - off)), pp);
        if (off - std::pow(e[0] + e[1] + e[2], pinv) > Ls) return;
    }
    for (int iz = z1; iz <= z2; iz++)
        for (int iy = g + 1; iy <= p.Bs[1] + g; iy++)
            for (int ix = g + 1; ix <= p.Bs[0] + g; ix++) {
                double tmp;
                if (G.sponge_type == WG_SPONGE_RECT) {
                    const double z = (double)(iz - (g + 1)) * dx[2] + x0[2];
                    const double y = (double)(iy - (g + 1)) * dx[1] + x0[1];
                    const double x = (double)(ix - (g + 1)) * dx[0] + x0[0];
                    const double v[6] = {x, y, z, -(x - p.domain[0]), -(y - p.domain[1]), -(z - p.domain[2])};
                    tmp = v[0];
                    for (int k = 1; k < 6; k++) tmp = std::min(tmp, v[k]);
                } else {
                    const double off = 0.5 * p.domain[0], pp = G.p_sponge, pinv = 1.0 / pp;
                    const double z = std::pow((double)(iz - (g + 1)) * dx[2] + x0[2] - off, pp);
                    const double y = std::pow((double)(iy - (g + 1)) * dx[1] + x0[1] - off, pp);
                    const double x = std::pow((double)(ix - (g + 1)) * dx[0] + x0[0] - off, pp);
                    tmp = -(std::pow(x + y + z, pinv) - off);
                }
                m[o.at(ix, iy, iz, 6)] = step_cosine(tmp, 0.5 * Ls, 0.5 * Ls);
            }
}

// masks of every block of the current grid (createMask_tree with
// dont_use_pruned_tree_mask / 2-D: createCompleteMaskDirect_tree,
// LIB/MESH/createMask_tree.f90:118-136)
static void make_masks(Oracle &o) {
    if (o.geom.kind == WG_GEOM_NONE || !o.cfg.penalization) {
        clear_mask(o);
        return;
    }
    o.mask_slot.clear();
    o.mask.assign(o.blocks.size() * 6 * size_t(o.npts), 0.0);
    for (size_t b = 0; b < o.blocks.size(); b++) mask_block(o, (int)b, o.mask.data() + b * 6 * o.npts);
}

// coarseningIndicatorMask_tree (LIB/MESH/coarseningIndicator_tree.f90:
// 333-420) for one block: 0 (stay) where chi has an interface point in the
// interior or is not constant there, else -1
static int mask_status(const Oracle &o, int b) {
    std::vector<double> m(6 * size_t(o.npts));
    mask_block(o, b, m.data());
    const wg_config &p = o.cfg;
    const int g = p.g;
    const int z1 = p.dim == 3 ? g + 1 : 1, z2 = p.dim == 3 ? p.Bs[2] + g : 1;
    bool iface = false;
    double mx = -HUGE_VAL, mn = HUGE_VAL;
    for (int iz = z1; iz <= z2; iz++)
        for (int iy = g + 1; iy <= p.Bs[1] + g; iy++)
            for (int ix = g + 1; ix <= p.Bs[0] + g; ix++) {
                const double c = m[o.at(ix, iy, iz, 1)];
                if (c > 1.0e-12 && c < 1.0 - 1.0e-12) iface = true;
                mx = std::max(mx, c);
                mn = std::min(mn, c);
            }
    if (iface || (mx - mn) > 1.0e-12) return 0;
    return -1;
}

// the two indicator switches of coarseningIndicator_tree on a flag array
// whose entries came from the block indicator: force_maxlevel_dealiasing
// (Jmax blocks -1, :287-293) and threshold_mask (max with the mask status)
static void indicator_switches(const Oracle &o, int nt, int *flags) {
    const wg_config &p = o.cfg;
    for (int b = 0; b < nt; b++) {
        if (p.force_maxlevel_dealiasing && o.blocks[b].level == p.Jmax) {
            flags[b] = -1;
            continue;
        }
        if (p.threshold_mask && o.geom.kind != WG_GEOM_NONE && p.penalization)
            flags[b] = std::max(flags[b], mask_status(o, b));
    }
}

// the divergence guard of the RHS's integral stage (rhs_ACM.f90:133-146):
// |u| > 1e12 at an interior point of any block
static bool diverged(const Oracle &o) {
    const wg_config &p = o.cfg;
    const int nblk = (int)o.blocks.size();
    const int z1 = p.dim == 3 ? p.g + 1 : 1, z2 = p.dim == 3 ? p.Bs[2] + p.g : 1;
    int bad = 0;
#pragma omp parallel for reduction(| : bad) num_threads(o.nthreads) if (o.nthreads > 1)
    for (int b = 0; b < nblk; b++) {
        const double *u = o.blk(b);
        for (int c = 1; c <= o.nc; c++)
            for (int k = z1; k <= z2; k++)
                for (int j = p.g + 1; j <= p.Bs[1] + p.g; j++)
                    for (int i = p.g + 1; i <= p.Bs[0] + p.g; i++)
                        if (std::fabs(u[o.at(i, j, k, c)]) > 1.0e12) bad = 1;
    }
    return bad != 0;
}

// RHS_wrapper local stage of one block into rhs (full-block layout; only the
// interior points are written)
static void rhs_block(const Oracle &o, int b, double *rhs) {
    double x0[3], dx[3];
    block_spacing(o, b, x0, dx);
    if (o.cfg.dim == 2) rhs_2d(o, o.blk(b), mask_of(o, b), dx, rhs);
    else rhs_3d(o, o.blk(b), mask_of(o, b), dx, rhs);
}

// RHS_wrapper local stage over all blocks, result into rhs (full-block layout)
static int rhs_all(Oracle &o, double *rhs) {
    const int nblk = (int)o.blocks.size();
    const size_t bs = size_t(o.nc) * o.npts;
    if (diverged(o)) return WG_EDIVERGED;
#pragma omp parallel for schedule(dynamic) num_threads(o.nthreads) if (o.nthreads > 1)
    for (int b = 0; b < nblk; b++) rhs_block(o, b, rhs + b * bs);
    return WG_OK;
}

// ---------------------------------------------------------------------------
// time step: calculate_time_step (LIB/TIME/calculate_time_step.f90:2-125) with
// GET_DT_BLOCK_ACM (module_ACM.f90:617-691)
// ---------------------------------------------------------------------------
static double dt_block(const Oracle &o, int b) {
    const wg_config &p = o.cfg;
    double x0[3], dx[3];
    block_spacing(o, b, x0, dx);
    const double *u = o.blk(b);
    const int g = p.g;
    double u_mag = -HUGE_VAL;
    for (int k = (p.dim == 3 ? g + 1 : 1); k <= (p.dim == 3 ? p.Bs[2] + g : 1); k++)
        for (int j = g + 1; j <= p.Bs[1] + g; j++)
            for (int i = g + 1; i <= p.Bs[0] + g; i++) {
                double s;
                if (p.dim == 2) {
                    double a = u[o.at(i, j, k, 1)], bb = u[o.at(i, j, k, 2)];
                    s = a * a + bb * bb;
                } else {
                    double a = u[o.at(i, j, k, 1)], bb = u[o.at(i, j, k, 2)], cc = u[o.at(i, j, k, 3)];
                    s = a * a + bb * bb + cc * cc;
                }
                if (s > u_mag) u_mag = s;
            }
    double u_eigen = std::sqrt(u_mag) + std::sqrt(p.c0 * p.c0 + u_mag);
    double dxmin = dx[0];
    for (int d = 1; d < p.dim; d++) dxmin = std::min(dxmin, dx[d]);
    double dt;
    if (u_eigen >= 1.0e-6) dt = p.CFL * dxmin / u_eigen;
    else dt = 1.0e-2;
    if (p.nu > 1.0e-13) dt = std::min(dt, p.CFL_nu * (dxmin * dxmin) / p.nu);
    if (p.gamma_p > 0) dt = std::min(dt, p.CFL_eta * p.gamma_p);
    if (p.penalization) dt = std::min(dt, p.CFL_eta * p.C_eta);
    if (p.use_sponge) dt = std::min(dt, p.CFL_eta * p.C_sponge);
    return dt;
}

static double calc_dt(const Oracle &o, double time) {
    const wg_config &p = o.cfg;
    double dt = 9.0e9;
    if (p.dt_fixed > 0.0) dt = p.dt_fixed;
    else {
        // the minimum does not depend on the order of the blocks
        const int nblk = (int)o.blocks.size();
#pragma omp parallel for reduction(min : dt) num_threads(o.nthreads) if (o.nthreads > 1)
        for (int b = 0; b < nblk; b++) dt = std::min(dt, dt_block(o, b));
        if (p.dt_max > 0.0) dt = std::min(p.dt_max, dt);
    }
    if (p.write_time > 0.0) {
        double wt = p.write_time;
        if (std::fmod(time + dt, wt) < std::fmod(time + 1e-12, wt) && !(std::fabs(std::fmod(time, wt)) < 1e-12) && time + 1e-12 > 0.0)
            dt = wt - std::fmod(time, wt);
    }
    if (p.tsave_stats > 0.0) {
        double ts = p.tsave_stats;
        if (std::fmod(time + dt, ts) < std::fmod(time + 1e-12, ts) && !(std::fabs(std::fmod(time, ts)) < 1e-12))
            dt = ts - std::fmod(time, ts);
    }
    if (time + dt > p.time_max && time <= p.time_max) dt = p.time_max - time;
    return dt;
}

// RungeKuttaGeneric with the default RK4 Butcher tableau
// (LIB/TIME/runge_kutta_generic.f90:1-156, ini_file_to_params.f90:640-646).
// The registers hold the interior points only; every update is a loop over
// blocks with the same expression per point as the reference, so the
// result does not depend on the number of threads.
static int rk4_step(Oracle &o, double *time_inout, double *dt_out) {
    const wg_config &p = o.cfg;
    const int nblk = (int)o.blocks.size();
    const size_t bs = size_t(o.nc) * o.npts;
    static const double rk[5][5] = {
        {0.0, 0.0, 0.0, 0.0, 0.0},
        {0.5, 0.5, 0.0, 0.0, 0.0},
        {0.5, 0.0, 0.5, 0.0, 0.0},
        {1.0, 0.0, 0.0, 1.0, 0.0},
        {0.0, 1.0 / 6.0, 1.0 / 3.0, 1.0 / 3.0, 1.0 / 6.0}};
    const double time = *time_inout;
    const int grhs = p.g_rhs;
    sync_ghosts(o, grhs, grhs, true);
    double dt = calc_dt(o, time);
    const int g = p.g;
    const int bz = p.dim == 3 ? p.Bs[2] : 1, z1 = p.dim == 2 ? 1 : g + 1;
    const size_t ni = size_t(o.nc) * bz * p.Bs[1] * p.Bs[0];   // interior values of a block
    if (o.work.size() != 5 * ni * nblk) o.work.resize(5 * ni * nblk);
    auto W = [&](int slot, int b) { return o.work.data() + (size_t(slot) * nblk + b) * ni; };
    // fn(b, index in the full block, index in the interior register)
    auto interior = [&](auto fn) {
#pragma omp parallel for schedule(static) num_threads(o.nthreads) if (o.nthreads > 1)
        for (int b = 0; b < nblk; b++) {
            size_t n = 0;
            for (int c = 1; c <= o.nc; c++)
                for (int k = z1; k < z1 + bz; k++)
                    for (int j = g + 1; j <= p.Bs[1] + g; j++)
                        for (int i = g + 1; i <= p.Bs[0] + g; i++) fn(b, o.at(i, j, k, c), n++);
        }
    };
    // RHS of every block into register `slot`
    auto stage_rhs = [&](int slot) -> int {
        if (diverged(o)) return WG_EDIVERGED;
#pragma omp parallel num_threads(o.nthreads) if (o.nthreads > 1)
        {
            std::vector<double> r(bs);
#pragma omp for schedule(dynamic)
            for (int b = 0; b < nblk; b++) {
                rhs_block(o, b, r.data());
                double *w = W(slot, b);
                size_t n = 0;
                for (int c = 1; c <= o.nc; c++)
                    for (int k = z1; k < z1 + bz; k++)
                        for (int j = g + 1; j <= p.Bs[1] + g; j++)
                            for (int i = g + 1; i <= p.Bs[0] + g; i++) w[n++] = r[o.at(i, j, k, c)];
            }
        }
        return WG_OK;
    };
    interior([&](int b, size_t q, size_t n) { W(0, b)[n] = o.blk(b)[q]; });
    int st = stage_rhs(1);
    if (st) return st;
    for (int j = 2; j <= 4; j++) {
        interior([&](int b, size_t q, size_t n) { o.blk(b)[q] = W(0, b)[n]; });
        for (int l = 2; l <= j; l++) {
            double a = rk[j - 1][l - 1];
            if (std::fabs(a) < 1.0e-8) continue;
            interior([&](int b, size_t q, size_t n) { o.blk(b)[q] = o.blk(b)[q] + dt * a * W(l - 1, b)[n]; });
        }
        sync_ghosts(o, grhs, grhs, true);
        if ((st = stage_rhs(j))) return st;
    }
    interior([&](int b, size_t q, size_t n) { o.blk(b)[q] = W(0, b)[n]; });
    for (int j = 2; j <= 5; j++) {
        double bj = rk[4][j - 1];
        if (std::fabs(bj) < 1.0e-8) continue;
        interior([&](int b, size_t q, size_t n) { o.blk(b)[q] = o.blk(b)[q] + dt * bj * W(j - 1, b)[n]; });
    }
    *time_inout = time + dt;
    *dt_out = dt;
    return WG_OK;
}

// ---------------------------------------------------------------------------
// one-level FWT of a block, interior only, spaghetti order
// (waveletDecomposition_optimized_block,
//  LIB/WAVELETS/wavelet_decomposition_reconstruction.f90:23-389)
// u and ud are full blocks (one component at a time), ud may equal u.
// ---------------------------------------------------------------------------
static void fwt_block(const Oracle &o, const double *u_in, double *u_d) {
    const wg_config &p = o.cfg;
    const Wavelet &w = o.wav;
    const int dim = p.dim;
    int g[3] = {p.g, p.g, dim == 3 ? p.g : 0};
    int Bs[3] = {p.Bs[0], p.Bs[1], dim == 3 ? p.Bs[2] : 1};
    int fmax = std::max(std::max(std::abs(w.HD.lo), std::abs(w.HD.hi)), std::max(std::abs(w.GD.lo), std::abs(w.GD.hi)));
    fmax = std::max({w.HD.lo, w.HD.hi, w.GD.lo, w.GD.hi});
    int fm[3] = {fmax, fmax, dim == 3 ? fmax : 0};
    const int nmax = std::max(o.nx, std::max(o.ny, o.nz)) + 1;
    std::vector<double> buf(nmax + 8);
    auto U = [&](const double *a, int ix, int iy, int iz) { return a[((size_t)(iz - 1) * o.ny + (iy - 1)) * o.nx + (ix - 1)]; };
    auto Ud = [&](int ix, int iy, int iz) -> double & { return u_d[((size_t)(iz - 1) * o.ny + (iy - 1)) * o.nx + (ix - 1)]; };
    // a filter applied in the reference's explicit term order (non-zero taps in ascending offset)
    auto apply = [&](const Filter &f, auto get, int at) {
        double s = 0.0;
        bool first = true;
        for (int m = f.lo; m <= f.hi; m++) {
            if (f(m) == 0.0 && !(m == 0)) continue;
            double v = get(at + m) * f(m);
            s = first ? v : s + v;
            first = false;
        }
        return s;
    };
    const bool lazy = (w.Y == 0);  // CDFX0: SC copied, only odd points filtered
    // X
    for (int iz = g[2] + 1 - fm[2]; iz <= Bs[2] + g[2] + fm[2]; iz++)
        for (int iy = g[1] + 1 - fm[1]; iy <= Bs[1] + g[1] + fm[1]; iy++) {
            auto get = [&](int ix) { return U(u_in, ix, iy, iz); };
            for (int ix = g[0] + 1; ix <= Bs[0] + g[0]; ix += 2) buf[ix] = lazy ? get(ix) : apply(w.HD, get, ix);
            for (int ix = g[0] + 2; ix <= Bs[0] + g[0]; ix += 2) buf[ix] = apply(w.GD, get, ix);
            for (int ix = g[0] + 1; ix <= Bs[0] + g[0]; ix++) Ud(ix, iy, iz) = buf[ix];
        }
    // Y
    for (int iz = g[2] + 1 - fm[2]; iz <= Bs[2] + g[2] + fm[2]; iz++)
        for (int ix = g[0] + 1; ix <= Bs[0] + g[0]; ix++) {
            auto get = [&](int iy) { return Ud(ix, iy, iz); };
            for (int iy = g[1] + 1; iy <= Bs[1] + g[1]; iy += 2) buf[iy] = lazy ? get(iy) : apply(w.HD, get, iy);
            for (int iy = g[1] + 2; iy <= Bs[1] + g[1]; iy += 2) buf[iy] = apply(w.GD, get, iy);
            for (int iy = g[1] + 1; iy <= Bs[1] + g[1]; iy++) Ud(ix, iy, iz) = buf[iy];
        }
    // Z
    if (dim == 3) {
        for (int iy = g[1] + 1; iy <= Bs[1] + g[1]; iy++)
            for (int ix = g[0] + 1; ix <= Bs[0] + g[0]; ix++) {
                auto get = [&](int iz) { return Ud(ix, iy, iz); };
                for (int iz = g[2] + 1; iz <= Bs[2] + g[2]; iz += 2) buf[iz] = lazy ? get(iz) : apply(w.HD, get, iz);
                for (int iz = g[2] + 2; iz <= Bs[2] + g[2]; iz += 2) buf[iz] = apply(w.GD, get, iz);
                for (int iz = g[2] + 1; iz <= Bs[2] + g[2]; iz++) Ud(ix, iy, iz) = buf[iz];
            }
    }
}

// ---------------------------------------------------------------------------
// one-level IWT of a block, interior only, from spaghetti order
// (waveletReconstruction_optimized_block,
//  LIB/WAVELETS/wavelet_decomposition_reconstruction.f90:426-840).
// Passes x, y, z; the x pass reads u and covers the ghost rows/planes the
// later passes need, the y and z passes read the partial result. Term order
// of the reference: unlifted wavelets keep the SC and add the odd HR taps to
// each WC (value first); lifted wavelets write at an SC position
// SC + odd GR taps, at a WC position the odd HR taps over the neighbouring
// SCs, then GR(0)*WC, then the other even GR taps, each group in ascending
// offset (non-zero taps).
// ---------------------------------------------------------------------------
static void iwt_block(const Oracle &o, const double *u_in, double *u_r) {
    const wg_config &p = o.cfg;
    const Wavelet &w = o.wav;
    const int dim = p.dim;
    int g[3] = {p.g, p.g, dim == 3 ? p.g : 0};
    int Bs[3] = {p.Bs[0], p.Bs[1], dim == 3 ? p.Bs[2] : 1};
    const int fmax = std::max({w.HR.lo, w.HR.hi, w.GR.lo, w.GR.hi});
    int fm[3] = {fmax, fmax, dim == 3 ? fmax : 0};
    const int nmax = std::max(o.nx, std::max(o.ny, o.nz)) + 2;
    std::vector<double> buf(nmax + 8);
    auto at = [&](int ix, int iy, int iz) { return ((size_t)(iz - 1) * o.ny + (iy - 1)) * o.nx + (ix - 1); };
    const bool lazy = (w.Y == 0);
    // reconstruct one line: get(i) reads the source at 1-based index i, the
    // results for the interior go to buf
    auto line = [&](auto get, int n0, int n1) {
        for (int s = n0; s <= n1; s += 2) {
            const int wpos = s + 1;
            if (lazy) {
                buf[s] = get(s);
                double v = get(wpos);
                for (int m = w.HR.lo; m <= w.HR.hi; m++)
                    if ((m & 1) && w.HR(m) != 0.0) v = v + get(wpos + m) * w.HR(m);
                buf[wpos] = v;
            } else {
                double sc = get(s);
                for (int m = w.GR.lo; m <= w.GR.hi; m++)
                    if ((m & 1) && w.GR(m) != 0.0) sc = sc + get(s + m) * w.GR(m);
                double v = 0.0;
                bool first = true;
                for (int m = w.HR.lo; m <= w.HR.hi; m++) {
                    if (!(m & 1) || w.HR(m) == 0.0) continue;
                    const double t = get(wpos + m) * w.HR(m);
                    v = first ? t : v + t;
                    first = false;
                }
                v = v + get(wpos) * w.GR(0);
                for (int m = w.GR.lo; m <= w.GR.hi; m++)
                    if (!(m & 1) && m != 0 && w.GR(m) != 0.0) v = v + get(wpos + m) * w.GR(m);
                buf[s] = sc;
                buf[wpos] = v;
            }
        }
    };
    // X: reads u_in, writes u_r (x interior) on the extended rows/planes
    for (int iz = g[2] + 1 - fm[2]; iz <= Bs[2] + g[2] + fm[2]; iz++)
        for (int iy = g[1] + 1 - fm[1]; iy <= Bs[1] + g[1] + fm[1]; iy++) {
            line([&](int ix) { return u_in[at(ix, iy, iz)]; }, g[0] + 1, Bs[0] + g[0] - 1);
            for (int ix = g[0] + 1; ix <= Bs[0] + g[0]; ix++) u_r[at(ix, iy, iz)] = buf[ix];
        }
    // Y
    for (int iz = g[2] + 1 - fm[2]; iz <= Bs[2] + g[2] + fm[2]; iz++)
        for (int ix = g[0] + 1; ix <= Bs[0] + g[0]; ix++) {
            line([&](int iy) { return u_r[at(ix, iy, iz)]; }, g[1] + 1, Bs[1] + g[1] - 1);
            for (int iy = g[1] + 1; iy <= Bs[1] + g[1]; iy++) u_r[at(ix, iy, iz)] = buf[iy];
        }
    // Z
    if (dim == 3)
        for (int iy = g[1] + 1; iy <= Bs[1] + g[1]; iy++)
            for (int ix = g[0] + 1; ix <= Bs[0] + g[0]; ix++) {
                line([&](int iz) { return u_r[at(ix, iy, iz)]; }, g[2] + 1, Bs[2] + g[2] - 1);
                for (int iz = g[2] + 1; iz <= Bs[2] + g[2]; iz++) u_r[at(ix, iy, iz)] = buf[iz];
            }
}

// wc_threshold_tree (LIB/MESH/adapt_tree.f90:1091-1180) with Linfty renorm:
// on spaghetti data, interior WC positions only. As in the reference,
// components whose threshold_state_vector_component is 1 are skipped by the
// per-component pass; 0 and >= 2 components are zeroed where |WC| < thresh;
// each group l >= 2 is also zeroed where the group's Euclidean norm is below
// the group's largest threshold.
static void wc_threshold_block(const Oracle &o, double *u, const double *thresh) {
    const wg_config &p = o.cfg;
    const int g = p.g, dim = p.dim, nc = o.nc;
    const int even_odd = (g + 1) % 2;
    const int z1 = dim == 2 ? 1 : g + 1, z2 = dim == 2 ? 1 : p.Bs[2] + g;
    auto is_sc = [&](int ix, int iy, int iz) {
        return ix % 2 == even_odd && iy % 2 == even_odd && iz % 2 == (dim == 2 ? 1 : even_odd);
    };
    auto idx = [&](int ix, int iy, int iz) { return ((size_t)(iz - 1) * o.ny + (iy - 1)) * o.nx + (ix - 1); };
    // the renormed copy (identity for Linfty) is read, the block is written
    std::vector<double> wc(u, u + (size_t)nc * o.npts);
    for (int c = 0; c < nc; c++) {
        if (p.threshold_state_vector_component[c] == 1) continue;
        for (int iz = z1; iz <= z2; iz++)
            for (int iy = g + 1; iy <= p.Bs[1] + g; iy++)
                for (int ix = g + 1; ix <= p.Bs[0] + g; ix++) {
                    if (is_sc(ix, iy, iz)) continue;
                    if (std::fabs(wc[c * o.npts + idx(ix, iy, iz)]) < thresh[c]) u[c * o.npts + idx(ix, iy, iz)] = 0.0;
                }
    }
    int maxg = 0;
    for (int c = 0; c < nc; c++) maxg = std::max(maxg, p.threshold_state_vector_component[c]);
    for (int l = 2; l <= maxg; l++) {
        double tmax = -1e300;
        for (int c = 0; c < nc; c++)
            if (p.threshold_state_vector_component[c] == l) tmax = std::max(tmax, thresh[c]);
        for (int iz = z1; iz <= z2; iz++)
            for (int iy = g + 1; iy <= p.Bs[1] + g; iy++)
                for (int ix = g + 1; ix <= p.Bs[0] + g; ix++) {
                    if (is_sc(ix, iy, iz)) continue;
                    double s = 0.0;
                    bool first = true;
                    for (int c = 0; c < nc; c++) {
                        if (p.threshold_state_vector_component[c] != l) continue;
                        const double v = wc[c * o.npts + idx(ix, iy, iz)];
                        s = first ? v * v : s + v * v;
                        first = false;
                    }
                    if (std::sqrt(s) < tmax)
                        for (int c = 0; c < nc; c++)
                            if (p.threshold_state_vector_component[c] == l) u[c * o.npts + idx(ix, iy, iz)] = 0.0;
                }
    }
}

// threshold_block (LIB/INDICATORS/threshold_block.f90) with Linfty renorm
// (wavelet_renorm_block, module_wavelets.f90:1848-1960): details are the max
// |WC| over the interior with scaling coefficients zeroed. Returns -1 (coarsen)
// or 0 (stay) and writes per-component details.
static int threshold_block(const Oracle &o, int b, const double *eps_use, double *detail_out) {
    const wg_config &p = o.cfg;
    std::vector<double> ud(size_t(o.npts));
    double detail[8];
    for (int c = 0; c < o.nc; c++) detail[c] = -1.0;
    const int g = p.g;
    const int z1 = p.dim == 2 ? 1 : g + 1, z2 = p.dim == 2 ? 1 : p.Bs[2] + g;
    std::vector<double> compv(8, 0.0);
    for (int c = 1; c <= o.nc; c++) {
        const double *u = o.blk(b) + size_t(c - 1) * o.npts;
        std::copy(u, u + o.npts, ud.begin());
        fwt_block(o, u, ud.data());
        double m = 0.0;
        bool any = false;
        for (int k = z1; k <= z2; k++)
            for (int j = g + 1; j <= p.Bs[1] + g; j++)
                for (int i = g + 1; i <= p.Bs[0] + g; i++) {
                    bool sc = ((i - g - 1) % 2 == 0) && ((j - g - 1) % 2 == 0) && (p.dim == 2 || (k - g - 1) % 2 == 0);
                    double v = sc ? 0.0 : std::fabs(ud[((size_t)(k - 1) * o.ny + (j - 1)) * o.nx + (i - 1)]);
                    if (!any || v > m) { m = v; any = true; }
                }
        compv[c - 1] = m;
    }
    // threshold_state_vector_component: 1 = own component, 0 = ignore,
    // l>=2 = vector group (max over sqrt(wc^2) of the group)
    int maxgrp = 0;
    for (int c = 0; c < o.nc; c++) maxgrp = std::max(maxgrp, p.threshold_state_vector_component[c]);
    for (int l = 2; l <= maxgrp; l++) {
        double m = 0.0;
        for (int c = 0; c < o.nc; c++) if (p.threshold_state_vector_component[c] == l) m = std::max(m, compv[c]);
        for (int c = 0; c < o.nc; c++) if (p.threshold_state_vector_component[c] == l) detail[c] = m;
    }
    for (int c = 0; c < o.nc; c++) {
        if (p.threshold_state_vector_component[c] == 1) detail[c] = compv[c];
        if (p.threshold_state_vector_component[c] == 0) detail[c] = 0.0;
    }
    bool all = true;
    for (int c = 0; c < o.nc; c++) {
        if (!(detail[c] <= eps_use[c])) all = false;
        if (detail_out) detail_out[c] = detail[c];
    }
    return all ? -1 : 0;
}

// refineBlock (LIB/MESH/refinementExecute.f90:4-116): predict the whole block
// (incl. ghosts) and cut the 2^d daughters out of the fine array, for every
// block with refine[b] != 0 (all blocks below Jmax when refine is empty).
static void refine_blocks(Oracle &o, const std::vector<int> &refine);
static void refine_everywhere(Oracle &o) { refine_blocks(o, {}); }

static void refine_blocks(Oracle &o, const std::vector<int> &refine) {
    const wg_config &p = o.cfg;
    const int dim = p.dim, g = p.g;
    const int nblk = (int)o.blocks.size();
    const int nd = 1 << dim;
    std::vector<Block> nbl;
    std::vector<double> ndata(size_t(nblk) * nd * o.nc * o.npts, 0.0);
    const int cx = o.nx, cy = o.ny, cz = o.nz;
    const int fx = 2 * cx - 1, fy = 2 * cy - 1, fz = dim == 3 ? 2 * cz - 1 : 1;
    std::vector<double> fine(size_t(fx) * fy * fz);
    std::vector<double> coarse(size_t(o.npts));
    // daughters are appended in (block, k_daughter) order; blocks on Jmax stay
    // (respectJmaxJmin_tree) and keep their place and data
    std::vector<int> first(nblk);
    auto stays = [&](int b) { return o.blocks[b].level >= p.Jmax || (!refine.empty() && !refine[b]); };
    for (int b = 0; b < nblk; b++) {
        first[b] = (int)nbl.size();
        if (stays(b)) {
            nbl.push_back(o.blocks[b]);
            continue;
        }
        for (int k = 0; k < nd; k++) {
            Block d;
            d.level = o.blocks[b].level + 1;
            int bx = (k / 2) % 2, by = k % 2, bz = k / 4;
            d.c[0] = 2 * o.blocks[b].c[0] + bx;
            d.c[1] = 2 * o.blocks[b].c[1] + by;
            d.c[2] = dim == 3 ? 2 * o.blocks[b].c[2] + bz : 0;
            nbl.push_back(d);
        }
    }
    ndata.assign(nbl.size() * o.nc * o.npts, 0.0);
    for (int b = 0; b < nblk; b++) {
        if (stays(b)) {
            std::copy(o.blk(b), o.blk(b) + size_t(o.nc) * o.npts, ndata.begin() + size_t(first[b]) * o.nc * o.npts);
            continue;
        }
        for (int c = 1; c <= o.nc; c++) {
            const double *u = o.blk(b) + size_t(c - 1) * o.npts;
            std::copy(u, u + o.npts, coarse.begin());
            prediction(coarse.data(), cx, cy, dim == 3 ? cz : 1, fine.data(), o.wav.order_predictor);
            for (int k = 0; k < nd; k++) {
                int i0 = g + 1 + p.Bs[0] * ((k / 2) % 2);
                int j0 = g + 1 + p.Bs[1] * (k % 2);
                int k0 = dim == 3 ? g + 1 + p.Bs[2] * (k / 4) : 1;
                double *dst = ndata.data() + (size_t(first[b]) + k) * o.nc * o.npts + size_t(c - 1) * o.npts;
                for (int kk = 0; kk < o.nz; kk++)
                    for (int jj = 0; jj < o.ny; jj++)
                        for (int ii = 0; ii < o.nx; ii++)
                            dst[((size_t)kk * o.ny + jj) * o.nx + ii] = fine[((size_t)(k0 - 1 + kk) * fy + (j0 - 1 + jj)) * fx + (i0 - 1 + ii)];
            }
        }
    }
    o.blocks = nbl;
    o.data.swap(ndata);
    update_neighbors(o);
}

// ---------------------------------------------------------------------------
// adapt_tree for unlifted wavelets (LIB/MESH/adapt_tree.f90:11-255; no coarse
// extension, no security zone, no WC thresholding):
//  * init_full_tree (adapt_tree.f90:995-1085): every block without a mother
//    above Jmin whose last treecode digit is 2^dim-1 creates its mother,
//    repeated until no block is added;
//  * the leaves are synchronised with g layers and flagged; the mothers, from
//    the finest level down, receive their daughters' scaling coefficients
//    (sync_D2M, executeCoarsening_tree.f90:125-227: every second interior
//    point for CDF X0) and, as ghost nodes, their same-level neighbours'
//    values (the full-tree sync of sync_TMP_from_all: a non-leaf block of a
//    graded tree has a same-level neighbour in every direction), then are
//    flagged (coarseningIndicator_tree.f90: the "everywhere" indicator flags
//    the leaves only);
//  * respectJmaxJmin_tree, then ensureGradedness_tree(check_daughters) with
//    ensure_completeness_block until nothing changes (ensureGradedness_tree.f90:
//    13-219, ensure_completeness_block.f90:7-87);
//  * blocks still at -1 are deleted, the remaining blocks without remaining
//    daughters are the new grid (prune_fulltree2leafs), their data the
//    leaves' own or the mothers' daughter coefficients; final ghost sync.
// ---------------------------------------------------------------------------
static int adapt_unlifted(Oracle &o, const double *eps_use, int everywhere) {
    const wg_config &p = o.cfg;
    const int dim = p.dim, g = p.g, nd = 1 << dim;
    const int Jmin = p.Jmin;
    sync_ghosts(o, g, g, true);
    const int nleaf = (int)o.blocks.size();
    // full tree
    std::vector<int> mother(nleaf, -1);
    auto digit_all_set = [&](const Block &b) { return tc_last_digit(b) == nd - 1; };
    size_t nold = 0;
    while (nold != o.blocks.size()) {
        nold = o.blocks.size();
        for (size_t i = 0; i < nold; i++) {
            const Block b = o.blocks[i];
            if (mother[i] >= 0 || b.level == Jmin) continue;
            if (b.level < Jmin) return WG_EGRID;
            if (!digit_all_set(b)) continue;
            Block m;
            m.level = b.level - 1;
            for (int a = 0; a < 3; a++) m.c[a] = b.c[a] >> 1;
            o.blocks.push_back(m);
            mother.push_back(-1);
            o.lookup[key_of(m.level, m.c[0], m.c[1], m.c[2])] = (int)o.blocks.size() - 1;
            mother[i] = (int)o.blocks.size() - 1;
        }
        // link the other daughters of the new mothers
        for (size_t i = 0; i < o.blocks.size(); i++) {
            const Block &b = o.blocks[i];
            if (mother[i] >= 0 || b.level == Jmin) continue;
            int c[3] = {b.c[0] >> 1, b.c[1] >> 1, b.c[2] >> 1};
            mother[i] = find_block(o, b.level - 1, c);
        }
    }
    const int nt = (int)o.blocks.size();
    std::vector<std::vector<int>> daughters(nt);
    for (int i = 0; i < nt; i++)
        if (mother[i] >= 0) daughters[mother[i]].push_back(i);
    for (int i = 0; i < nt; i++)
        if (!daughters[i].empty() && (int)daughters[i].size() != nd) return WG_EGRID;
    o.data.resize(size_t(nt) * o.nc * o.npts, 0.0);
    auto idx = [&](int ix, int iy, int iz) { return ((size_t)(iz - 1) * o.ny + (iy - 1)) * o.nx + (ix - 1); };
    int lmax = 0;
    for (const Block &b : o.blocks) lmax = std::max(lmax, b.level);
    std::vector<int> flags(nt, 0);
    // leaf flags (after the sync above)
    for (int i = 0; i < nleaf; i++)
        flags[i] = everywhere ? -1 : threshold_block(o, i, eps_use, nullptr);
    const int zlo = dim == 3 ? g + 1 : 1, zhi = dim == 3 ? g + p.Bs[2] : 1;
    const int half[3] = {p.Bs[0] / 2, p.Bs[1] / 2, dim == 3 ? p.Bs[2] / 2 : 1};
    for (int l = lmax - 1; l >= Jmin; l--) {
        // sync_D2M: the mother's interior point takes the daughter's SC
        for (int m = nleaf; m < nt; m++) {
            if (o.blocks[m].level != l) continue;
            for (int dgt : daughters[m]) {
                const Block &d = o.blocks[dgt];
                const int kx = d.c[0] & 1, ky = d.c[1] & 1, kz = dim == 3 ? (d.c[2] & 1) : 0;
                for (int c = 0; c < o.nc; c++) {
                    const double *src = o.blk(dgt) + size_t(c) * o.npts;
                    double *dst = o.blk(m) + size_t(c) * o.npts;
                    for (int k = 0; k < (dim == 3 ? half[2] : 1); k++)
                        for (int j = 0; j < half[1]; j++)
                            for (int i = 0; i < half[0]; i++) {
                                const int mi = g + 1 + kx * half[0] + i, mj = g + 1 + ky * half[1] + j;
                                const int mk = dim == 3 ? g + 1 + kz * half[2] + k : 1;
                                const int si = g + 1 + 2 * i, sj = g + 1 + 2 * j, sk = dim == 3 ? g + 1 + 2 * k : 1;
                                dst[idx(mi, mj, mk)] = src[idx(si, sj, sk)];
                            }
                }
            }
        }
        if (everywhere) continue;
        // ghost nodes of the mothers from their same-level neighbours
        for (int m = nleaf; m < nt; m++) {
            if (o.blocks[m].level != l) continue;
            const Block &mb = o.blocks[m];
            for (int dz = (dim == 3 ? -1 : 0); dz <= (dim == 3 ? 1 : 0); dz++)
                for (int dy = -1; dy <= 1; dy++)
                    for (int dx = -1; dx <= 1; dx++) {
                        if (!dx && !dy && !dz) continue;
                        const int d[3] = {dx, dy, dz};
                        const int n = 1 << l;
                        int c[3] = {0, 0, 0};
                        for (int a = 0; a < dim; a++) c[a] = ((mb.c[a] + d[a]) % n + n) % n;
                        const int nb = find_block(o, l, c);
                        if (nb < 0) continue;
                        int lo[3], hi[3], so[3];
                        for (int a = 0; a < 3; a++) {
                            if (a >= dim) { lo[a] = hi[a] = so[a] = 1; continue; }
                            const int B = p.Bs[a];
                            lo[a] = d[a] < 0 ? 1 : d[a] == 0 ? g + 1 : g + B + 1;
                            hi[a] = d[a] < 0 ? g : d[a] == 0 ? g + B : B + 2 * g;
                            so[a] = d[a] < 0 ? B + 1 : g + 1;
                        }
                        for (int c2 = 0; c2 < o.nc; c2++) {
                            const double *src = o.blk(nb) + size_t(c2) * o.npts;
                            double *dst = o.blk(m) + size_t(c2) * o.npts;
                            for (int k = lo[2]; k <= hi[2]; k++)
                                for (int j = lo[1]; j <= hi[1]; j++)
                                    for (int i = lo[0]; i <= hi[0]; i++)
                                        dst[idx(i, j, k)] = src[idx(so[0] + i - lo[0], so[1] + j - lo[1], so[2] + k - lo[2])];
                        }
                    }
        }
        for (int m = nleaf; m < nt; m++)
            if (o.blocks[m].level == l) flags[m] = threshold_block(o, m, eps_use, nullptr);
    }
    (void)zlo;
    (void)zhi;
    if (!everywhere) indicator_switches(o, nt, flags.data());
    // respectJmaxJmin_tree
    const int STAY = 9;
    for (int i = 0; i < nt; i++)
        if (flags[i] == -1 && o.blocks[i].level <= Jmin) flags[i] = STAY;
    // ensureGradedness_tree(check_daughters, stay=REF_UNSIGNIFICANT_STAY)
    bool changed = true;
    int guard = 0;
    while (changed) {
        changed = false;
        if (++guard > 10 * (p.Jmax + 1) + 100) return WG_EGRID;
        for (int i = 0; i < nt; i++) {
            if (flags[i] != -1) continue;
            // ensure_completeness_block
            const int m = mother[i];
            const std::vector<int> &sis = daughters[m];
            bool all_coarsen = true;
            for (int s2 : sis)
                if (flags[s2] >= 0) all_coarsen = false;
            if (!all_coarsen) {
                for (int s2 : sis)
                    if (flags[s2] < 0) flags[s2] = STAY;
                changed = true;
                continue;
            }
            bool dstay = false;
            for (int d2 : daughters[i])
                if (flags[d2] == 0 || flags[d2] == STAY) dstay = true;
            if (dstay) {
                for (int s2 : sis)
                    if (flags[s2] < 0) flags[s2] = STAY;
                changed = true;
                continue;
            }
            // gradedness: finer neighbours that stay
            const Block b = o.blocks[i];
            const int n = 1 << b.level;
            bool keep = false;
            for (int dz = (dim == 3 ? -1 : 0); dz <= (dim == 3 ? 1 : 0) && !keep; dz++)
                for (int dy = -1; dy <= 1 && !keep; dy++)
                    for (int dx = -1; dx <= 1 && !keep; dx++) {
                        if (!dx && !dy && !dz) continue;
                        const int d[3] = {dx, dy, dz};
                        int c[3] = {0, 0, 0};
                        for (int a = 0; a < dim; a++) c[a] = ((b.c[a] + d[a]) % n + n) % n;
                        // finer blocks touching b across d
                        for (int kz = 0; kz < (dim == 3 ? 2 : 1) && !keep; kz++)
                            for (int ky = 0; ky < 2 && !keep; ky++)
                                for (int kx = 0; kx < 2 && !keep; kx++) {
                                    const int kk[3] = {kx, ky, kz};
                                    bool adj = true;
                                    for (int a = 0; a < dim; a++)
                                        if ((d[a] == 1 && kk[a] != 0) || (d[a] == -1 && kk[a] != 1)) adj = false;
                                    if (!adj) continue;
                                    int fc[3] = {2 * c[0] + kx, 2 * c[1] + ky, dim == 3 ? 2 * c[2] + kz : 0};
                                    const int f = find_block(o, b.level + 1, fc);
                                    if (f >= 0 && (flags[f] == 0 || flags[f] == STAY)) keep = true;
                                }
                    }
            if (keep) {
                flags[i] = STAY;
                changed = true;
            }
        }
    }
    // delete -1 blocks, prune to leaves
    std::vector<Block> nbl;
    std::vector<double> ndata;
    for (int i = 0; i < nt; i++) {
        if (flags[i] == -1) continue;
        bool kept_daughter = false;
        for (int d2 : daughters[i])
            if (flags[d2] != -1) kept_daughter = true;
        if (kept_daughter) continue;
        nbl.push_back(o.blocks[i]);
        ndata.insert(ndata.end(), o.blk(i), o.blk(i) + size_t(o.nc) * o.npts);
    }
    o.blocks = nbl;
    o.data.swap(ndata);
    clear_mask(o);   // masks depend on the grid
    rebuild_lookup(o);
    update_neighbors(o);
    sync_ghosts(o, g, g, true);
    return WG_OK;
}

// ===========================================================================
// Full-tree adaptation with coarse extension (lifted wavelets, CDF XY with
// Y > 0): adapt_tree (LIB/MESH/adapt_tree.f90:11-255) with
// wavelet_decompose_full_tree (:264-523), init_full_tree (:995-1085),
// wavelet_reconstruct_full_tree_CEoptimized (:686-987) and
// prune_fulltree2leafs. The sync is sync_ghosts_generic
// (LIB/MPI/synchronize_ghosts_generic.f90:181-343) with the single-rank send
// logic of prepare_ghost_synch_metadata (:352-694) and the data source rules
// of unpack_ghostlayers_internal (LIB/MPI/xfer_block_data.f90:321-437).
// Blocks are visited in index order (the reference's results do not depend
// on the block order, which varies with the MPI partition).
// ===========================================================================
constexpr int kRefTmpEmpty = 10;          // REF_TMP_EMPTY (module_globals.f90:25)
constexpr int kRefUnsignificantStay = 9;  // REF_UNSIGNIFICANT_STAY (:28)

// updateFamily_tree (LIB/MESH/updateFamily_tree.f90:16-56): mother below
// Jmin is not searched, daughters above Jmax neither
static void update_family(Oracle &o, int Jmin) {
    const int n = (int)o.blocks.size(), dim = o.cfg.dim, nd = 1 << dim;
    o.mother.assign(n, -1);
    o.dau.assign(size_t(n) * 8, -1);
    for (int b = 0; b < n; b++) {
        const Block &B = o.blocks[b];
        if (B.level != Jmin) {
            const int c[3] = {B.c[0] >> 1, B.c[1] >> 1, dim == 3 ? B.c[2] >> 1 : 0};
            o.mother[b] = find_block(o, B.level - 1, c);
        }
        if (B.level != o.cfg.Jmax)
            for (int k = 0; k < nd; k++) {
                const int c[3] = {2 * B.c[0] + (k & 1), 2 * B.c[1] + ((k >> 1) & 1), dim == 3 ? 2 * B.c[2] + ((k >> 2) & 1) : 0};
                o.dau[size_t(b) * 8 + k] = find_block(o, B.level + 1, c);
            }
    }
}

// block_is_leaf / block_is_root / block_has_valid_neighbor
// (LIB/MPI/block_relations.f90:2-71)
static bool blk_is_leaf(const Oracle &o, int b, bool check_empty) {
    bool leaf = true;
    for (int k = 0; k < 8; k++)
        if (o.dau[size_t(b) * 8 + k] >= 0) leaf = false;
    if (leaf || !check_empty) return leaf;
    for (int k = 0; k < 8; k++) {
        const int d = o.dau[size_t(b) * 8 + k];
        if (d >= 0 && o.ref[d] != kRefTmpEmpty) return false;
    }
    return true;
}

static bool blk_is_root(const Oracle &o, int b, bool check_empty) {
    if (o.mother[b] < 0) return true;
    return check_empty && o.ref[o.mother[b]] == kRefTmpEmpty;
}

// np_l / np_u (LIB/TREE/neighborhood.f90:439-500): the relations of the
// same patch at another level difference
static void patch_range(int relation, int lvl_diff, int &lo, int &hi) {
    const int t = (relation - 1) % 56 + 1;
    int pid;
    if (t <= 24) pid = (t - 1) / 4 + 1;
    else if (t <= 48) pid = (t - 25) / 2 + 1 + 6;
    else pid = (t - 49) + 1 + 6 + 12;
    if (pid <= 6) { lo = (pid - 1) * 4 + 1; hi = pid * 4; }
    else if (pid <= 18) { lo = (pid - 7) * 2 + 25; hi = (pid - 6) * 2 + 24; }
    else { lo = (pid - 19) + 49; hi = (pid - 18) + 48; }
    const int off = lvl_diff == +1 ? 56 : lvl_diff == -1 ? 112 : 0;
    lo += off;
    hi += off;
}

static bool blk_has_valid_neighbor(const Oracle &o, int b, int relation, int lvl_diff) {
    int lo, hi;
    patch_range(relation, lvl_diff, lo, hi);
    for (int r = lo; r <= hi; r++) {
        const int n = o.nb[size_t(b) * 168 + r - 1];
        if (n >= 0 && o.ref[n] != kRefTmpEmpty) return true;
    }
    return false;
}

// coarseExtensionManipulateSC_block (module_wavelets.f90:966-1028): copy the
// SC of the patch next to a coarser neighbour from u_copy
static void ce_copy_sc(const Oracle &o, double *wc, const double *u_copy, int relation) {
    const int g = o.cfg.g, dim = o.cfg.dim;
    const int N[3] = {o.nx, o.ny, o.nz};
    const int Ns[3] = {o.wav.Nscl, o.wav.Nscl, o.wav.Nscl}, Ne[3] = {o.wav.Nscr, o.wav.Nscr, o.wav.Nscr};
    const int gg[3] = {g, g, g};
    int idx[2][3];
    modify_patch(dim, relation, idx, N, Ns, Ne, gg, gg, +1);
    int io[3] = {0, 0, 0};
    for (int d = 0; d < dim; d++) io[d] = ((g + idx[0][d] + 1) % 2 + 2) % 2;
    for (int c = 1; c <= o.nc; c++)
        for (int k = idx[0][2] + io[2]; k <= idx[1][2]; k += 2)
            for (int j = idx[0][1] + io[1]; j <= idx[1][1]; j += 2)
                for (int i = idx[0][0] + io[0]; i <= idx[1][0]; i += 2) wc[o.at(i, j, k, c)] = u_copy[o.at(i, j, k, c)];
}

// coarseExtensionManipulateWC_block (module_wavelets.f90:877-962): zero the
// WC inside the patch next to a coarser neighbour and in its ghost patch
static void ce_clear_wc(const Oracle &o, double *wc, int relation) {
    const int g = o.cfg.g, dim = o.cfg.dim;
    const int N[3] = {o.nx, o.ny, o.nz};
    const int Ns[3] = {o.wav.Nwcl, o.wav.Nwcl, o.wav.Nwcl}, Ne[3] = {o.wav.Nwcr, o.wav.Nwcr, o.wav.Nwcr};
    const int gg[3] = {g, g, g};
    for (int set = 1; set <= 2; set++) {
        int idx[2][3];
        if (set == 1) modify_patch(dim, relation, idx, N, Ns, Ne, gg, gg, +1);
        else ghost_patch(o.cfg.Bs, g, dim, relation, idx, g, g, +1);
        if (dim == 2) idx[0][2] = idx[1][2] = 1;
        int io[3] = {0, 0, 0};
        for (int d = 0; d < dim; d++) io[d] = ((g + idx[0][d] + 1) % 2 + 2) % 2;
        for (int c = 1; c <= o.nc; c++) {
            for (int k = idx[0][2] + io[2]; k <= idx[1][2]; k += 2)
                for (int j = idx[0][1] + io[1]; j <= idx[1][1]; j += 2)
                    for (int i = idx[0][0] + 1 - io[0]; i <= idx[1][0]; i += 2) wc[o.at(i, j, k, c)] = 0.0;
            for (int k = idx[0][2] + io[2]; k <= idx[1][2]; k += 2)
                for (int j = idx[0][1] + 1 - io[1]; j <= idx[1][1]; j += 2)
                    for (int i = idx[0][0]; i <= idx[1][0]; i++) wc[o.at(i, j, k, c)] = 0.0;
            if (dim == 3)
                for (int k = idx[0][2] + 1 - io[2]; k <= idx[1][2]; k += 2)
                    for (int j = idx[0][1]; j <= idx[1][1]; j++)
                        for (int i = idx[0][0]; i <= idx[1][0]; i++) wc[o.at(i, j, k, c)] = 0.0;
        }
    }
}

// blockFilterXYZ_vct with do_restriction (module_wavelets.f90:307-401):
// x pass on every second interior point over the rows the later passes
// read, then y, then z; every sum starts from 0 and runs over all taps
static void block_filter_restrict(const Oracle &o, const double *u, std::vector<double> &out) {
    const Filter &F = o.wav.HD;
    out.assign(u, u + size_t(o.nc) * o.npts);
    if (F.lo == 0 && F.hi == 0 && std::fabs(F(0) - 1.0) <= 1.0e-10) return;
    const int g = o.cfg.g, dim = o.cfg.dim;
    int ifs[3], ife[3], ils[3], ile[3];
    for (int d = 0; d < 3; d++) {
        ifs[d] = g + 1 + F.lo;
        ife[d] = o.cfg.Bs[d] + g + F.hi;
        ils[d] = g + 1;
        ile[d] = o.cfg.Bs[d] + g;
    }
    if (dim == 2) ifs[2] = ife[2] = ils[2] = ile[2] = 1;
    std::vector<double> t(o.npts);
    for (int c = 1; c <= o.nc; c++) {
        double *uf = out.data() + size_t(c - 1) * o.npts;
        auto T = [&](int i, int j, int k) { return t[((size_t)(k - 1) * o.ny + (j - 1)) * o.nx + (i - 1)]; };
        auto UF = [&](int i, int j, int k) -> double & { return uf[((size_t)(k - 1) * o.ny + (j - 1)) * o.nx + (i - 1)]; };
        std::copy(uf, uf + o.npts, t.begin());
        for (int k = ifs[2]; k <= ife[2]; k++)
            for (int j = ifs[1]; j <= ife[1]; j++)
                for (int i = ils[0]; i <= ile[0]; i += 2) {
                    double s = 0.0;
                    for (int m = F.lo; m <= F.hi; m++) s = s + T(i + m, j, k) * F(m);
                    UF(i, j, k) = s;
                }
        std::copy(uf, uf + o.npts, t.begin());
        for (int k = ifs[2]; k <= ife[2]; k++)
            for (int j = ils[1]; j <= ile[1]; j += 2)
                for (int i = ils[0]; i <= ile[0]; i += 2) {
                    double s = 0.0;
                    for (int m = F.lo; m <= F.hi; m++) s = s + T(i, j + m, k) * F(m);
                    UF(i, j, k) = s;
                }
        if (dim == 3) {
            std::copy(uf, uf + o.npts, t.begin());
            for (int k = ils[2]; k <= ile[2]; k += 2)
                for (int j = ils[1]; j <= ile[1]; j += 2)
                    for (int i = ils[0]; i <= ile[0]; i += 2) {
                        double s = 0.0;
                        for (int m = F.lo; m <= F.hi; m++) s = s + T(i, j, k + m) * F(m);
                        UF(i, j, k) = s;
                    }
        }
    }
}

// restrict_copy_at_CE (LIB/MPI/restrict_predict_data.f90:121-170): filtered
// block, with the SC next to a coarser or finer neighbour copied back for a
// leaf without a same-level neighbour on that patch
static void restrict_copy_at_ce(const Oracle &o, const double *src, int b, std::vector<double> &out) {
    block_filter_restrict(o, src, out);
    const int lvl = o.blocks[b].level;
    for (int r = 1; r <= 168; r++) {
        const int n = o.nb[size_t(b) * 168 + r - 1];
        if (n < 0) continue;
        const int ld = lvl - o.blocks[n].level;
        if ((ld == -1 || ld == 1) && blk_is_leaf(o, b, false) && !blk_has_valid_neighbor(o, b, r, 0))
            ce_copy_sc(o, out.data(), src, r);
    }
}

enum { kSyncFull = 1, kSyncFullLeaf = 2, kSyncMoC = 3, kSyncMoF = 4, kSyncMonly = 5 };
enum { kTmpNone = 0, kTmpNotFlag = 1, kTmpDecomposed = 2 };

struct SyncSpec {
    int base = kSyncFull;
    bool by_ref = false, by_level = false;
    int s_ref = 0, s_level = 0;
    int gminus = 0, gplus = 0;
    int tmp_usage = kTmpNone;
    bool ignore_filter = false;
};

static void sync_generic(Oracle &o, const SyncSpec &sp) {
    const wg_config &cfg = o.cfg;
    const int dim = cfg.dim;
    const int nstages = o.wav.lifted ? 3 : 2, isUnl = o.wav.lifted ? 0 : 1;
    const int nblk = (int)o.blocks.size();
    std::vector<double> coarse, fine, filtered;
    int filtered_id = -1;   // restricted_hvy_ID, reset once per sync
    for (int istage = 1; istage <= nstages; istage++) {
        for (int ib = 0; ib < nblk; ib++) {
            if (sp.base == kSyncFullLeaf && !blk_is_leaf(o, ib, false)) continue;
            if (o.ref[ib] == kRefTmpEmpty) continue;
            const int level = o.blocks[ib].level;
            for (int i_n = 1; i_n <= 168; i_n++) {
                const int in = o.nb[size_t(ib) * 168 + i_n - 1];
                if (in < 0) continue;
                const int lvl_diff = level - o.blocks[in].level;
                const int ref_n = o.ref[in];
                if (ref_n == kRefTmpEmpty) continue;
                const bool s1 = istage == 1 && lvl_diff == 0;
                const bool s2 = istage == 2 - isUnl && lvl_diff == +1;
                const bool s3 = istage == 3 - isUnl && lvl_diff == -1;
                bool send = false;
                switch (sp.base) {
                case kSyncFull:
                    if (s1 || s2 || s3) {
                        send = true;
                        if (lvl_diff == -1 && !blk_is_leaf(o, ib, true)) send = false;
                        if (lvl_diff == +1 && !blk_is_root(o, ib, true)) send = false;
                    }
                    break;
                case kSyncFullLeaf:
                    if (s1 || s2 || s3) {
                        send = true;
                        if (lvl_diff >= 0 && blk_has_valid_neighbor(o, ib, i_n, -1)) send = false;
                        else if (lvl_diff == +1 && blk_has_valid_neighbor(o, ib, i_n, 0)) send = false;
                    }
                    break;
                case kSyncMoC:
                    if (s1 || s3) {
                        send = true;
                        if (lvl_diff != 0 && !blk_is_leaf(o, ib, true)) send = false;
                    }
                    break;
                case kSyncMoF:
                    if (s1 || s2) {
                        send = true;
                        if (lvl_diff != 0 && !blk_is_root(o, ib, true)) send = false;
                    }
                    break;
                default:
                    send = s1;
                }
                if (send && sp.by_ref) send = sp.s_ref == ref_n;
                if (send && sp.by_level) send = sp.s_level == o.blocks[in].level;
                if (!send) continue;
                // data source of the sender (hvy_tmp_usage)
                bool tmp_rp = false, tmp_same = false;
                if (sp.tmp_usage == kTmpNotFlag && o.ref[ib] != sp.s_ref) tmp_rp = tmp_same = true;
                if (sp.tmp_usage == kTmpDecomposed) tmp_rp = true;
                const int inv = inverse_relation(i_n);
                int recv[2][3], sb[2][3], buf[2][3];
                ghost_patch(cfg.Bs, cfg.g, dim, inv, recv, sp.gminus, sp.gplus, -lvl_diff);
                send_bounds(cfg, o.wav.order_predictor, i_n, lvl_diff, sp.gminus, sp.gplus, sb, buf);
                double *dst = o.blk(in);
                if (lvl_diff == 0) {
                    const double *src = (tmp_same ? o.tmp.data() : o.data.data()) + size_t(ib) * o.nc * o.npts;
                    for (int c = 1; c <= o.nc; c++)
                        for (int k = recv[0][2], ks = sb[0][2]; k <= recv[1][2]; k++, ks++)
                            for (int j = recv[0][1], js = sb[0][1]; j <= recv[1][1]; j++, js++)
                                for (int i = recv[0][0], is = sb[0][0]; i <= recv[1][0]; i++, is++)
                                    dst[o.at(i, j, k, c)] = src[o.at(is, js, ks, c)];
                    continue;
                }
                const double *src = (tmp_rp ? o.tmp.data() : o.data.data()) + size_t(ib) * o.nc * o.npts;
                if (lvl_diff == +1) {
                    const double *srcf = src;
                    if (!sp.ignore_filter) {
                        if (filtered_id != ib) {
                            restrict_copy_at_ce(o, src, ib, filtered);
                            filtered_id = ib;
                        }
                        srcf = filtered.data();
                    }
                    for (int c = 1; c <= o.nc; c++)
                        for (int k = recv[0][2], kb = buf[0][2]; k <= recv[1][2]; k++, kb++)
                            for (int j = recv[0][1], jb = buf[0][1]; j <= recv[1][1]; j++, jb++)
                                for (int i = recv[0][0], ib2 = buf[0][0]; i <= recv[1][0]; i++, ib2++) {
                                    const int is = sb[0][0] + 2 * (ib2 - 1), js = sb[0][1] + 2 * (jb - 1);
                                    const int ks = dim == 3 ? sb[0][2] + 2 * (kb - 1) : 1;
                                    dst[o.at(i, j, k, c)] = srcf[o.at(is, js, ks, c)];
                                }
                } else {
                    const int cx = sb[1][0] - sb[0][0] + 1, cy = sb[1][1] - sb[0][1] + 1, cz = sb[1][2] - sb[0][2] + 1;
                    const int fx = 2 * cx - 1, fy = 2 * cy - 1;
                    coarse.resize(size_t(cx) * cy * cz);
                    fine.resize(size_t(fx) * fy * (2 * cz - 1));
                    for (int c = 1; c <= o.nc; c++) {
                        size_t q = 0;
                        for (int k = sb[0][2]; k <= sb[1][2]; k++)
                            for (int j = sb[0][1]; j <= sb[1][1]; j++)
                                for (int i = sb[0][0]; i <= sb[1][0]; i++) coarse[q++] = src[o.at(i, j, k, c)];
                        prediction(coarse.data(), cx, cy, cz, fine.data(), o.wav.order_predictor);
                        for (int k = recv[0][2], kb = buf[0][2]; k <= recv[1][2]; k++, kb++)
                            for (int j = recv[0][1], jb = buf[0][1]; j <= recv[1][1]; j++, jb++)
                                for (int i = recv[0][0], ib2 = buf[0][0]; i <= recv[1][0]; i++, ib2++)
                                    dst[o.at(i, j, k, c)] = fine[(size_t(kb - 1) * fy + (jb - 1)) * fx + (ib2 - 1)];
                    }
                }
            }
        }
    }
}

// coarse_extension_modify (LIB/MPI/reconstruction_step.f90:3-100); case 0
// tree, 1 level, 2 ref, 3 level_ref
static void ce_modify(Oracle &o, int ce_case, int s_level, int s_ref, bool clear_wc, bool copy_sc) {
    const int n = (int)o.blocks.size();
    for (int b = 0; b < n; b++) {
        const int lv = o.blocks[b].level;
        if ((ce_case == 1 || ce_case == 3) && lv != s_level) continue;
        if ((ce_case == 2 || ce_case == 3) && o.ref[b] != s_ref) continue;
        if (!blk_is_leaf(o, b, false)) continue;
        for (int r = 1; r <= 168; r++) {
            const int nb = o.nb[size_t(b) * 168 + r - 1];
            if (nb < 0) continue;
            if (o.blocks[nb].level < lv &&
                !(blk_has_valid_neighbor(o, b, r, 0) || blk_has_valid_neighbor(o, b, r, -1))) {
                if (clear_wc) ce_clear_wc(o, o.blk(b), r);
                if (copy_sc) ce_copy_sc(o, o.blk(b), o.tmp.data() + size_t(b) * o.nc * o.npts, r);
            }
        }
    }
}

// sync_D2M for one level (LIB/MESH/executeCoarsening_tree.f90:125-227):
// the SC of every daughter go to its quadrant of the mother's interior
static void sync_d2m(Oracle &o, int level) {
    const int dim = o.cfg.dim, g = o.cfg.g;
    const int half[3] = {o.cfg.Bs[0] / 2, o.cfg.Bs[1] / 2, dim == 3 ? o.cfg.Bs[2] / 2 : 1};
    for (int b = 0; b < (int)o.blocks.size(); b++) {
        if (o.blocks[b].level != level || o.mother[b] < 0) continue;
        const int m = o.mother[b];
        const Block &d = o.blocks[b];
        const int kx = d.c[0] & 1, ky = d.c[1] & 1, kz = dim == 3 ? (d.c[2] & 1) : 0;
        for (int c = 1; c <= o.nc; c++)
            for (int k = 0; k < half[2]; k++)
                for (int j = 0; j < half[1]; j++)
                    for (int i = 0; i < half[0]; i++) {
                        const int mk = dim == 3 ? g + 1 + kz * half[2] + k : 1, sk = dim == 3 ? g + 1 + 2 * k : 1;
                        o.blk(m)[o.at(g + 1 + kx * half[0] + i, g + 1 + ky * half[1] + j, mk, c)] =
                            o.blk(b)[o.at(g + 1 + 2 * i, g + 1 + 2 * j, sk, c)];
                    }
    }
}

// coarseningIndicator_block on decomposed data (input_is_WD): max |WC| over
// the interior per component, vector groups as threshold_block
static int threshold_wd(const Oracle &o, int b, const double *eps_use) {
    const wg_config &p = o.cfg;
    const int g = p.g;
    const int z1 = p.dim == 2 ? 1 : g + 1, z2 = p.dim == 2 ? 1 : p.Bs[2] + g;
    double compv[8] = {0, 0, 0, 0, 0, 0, 0, 0}, detail[8];
    for (int c = 1; c <= o.nc; c++) {
        const double *u = o.blk(b);
        double m = 0.0;
        bool any = false;
        for (int k = z1; k <= z2; k++)
            for (int j = g + 1; j <= p.Bs[1] + g; j++)
                for (int i = g + 1; i <= p.Bs[0] + g; i++) {
                    const bool sc = ((i - g - 1) % 2 == 0) && ((j - g - 1) % 2 == 0) && (p.dim == 2 || (k - g - 1) % 2 == 0);
                    const double v = sc ? 0.0 : std::fabs(u[o.at(i, j, k, c)]);
                    if (!any || v > m) { m = v; any = true; }
                }
        compv[c - 1] = m;
    }
    int maxgrp = 0;
    for (int c = 0; c < o.nc; c++) maxgrp = std::max(maxgrp, p.threshold_state_vector_component[c]);
    for (int c = 0; c < o.nc; c++) detail[c] = -1.0;
    for (int l = 2; l <= maxgrp; l++) {
        double m = 0.0;
        for (int c = 0; c < o.nc; c++) if (p.threshold_state_vector_component[c] == l) m = std::max(m, compv[c]);
        for (int c = 0; c < o.nc; c++) if (p.threshold_state_vector_component[c] == l) detail[c] = m;
    }
    for (int c = 0; c < o.nc; c++) {
        if (p.threshold_state_vector_component[c] == 1) detail[c] = compv[c];
        if (p.threshold_state_vector_component[c] == 0) detail[c] = 0.0;
    }
    for (int c = 0; c < o.nc; c++)
        if (!(detail[c] <= eps_use[c])) return 0;
    return -1;
}

// threshold_block on a patch of decomposed data (input_is_WD, Linfty): SC
// of the patch zeroed by parity, max |WC| per component and vector group;
// true if any component is significant
static bool patch_significant(const Oracle &o, int b, const int idx[2][3], const double *eps_use) {
    const wg_config &p = o.cfg;
    const int g = p.g;
    int io[3] = {0, 0, 0};
    for (int d = 0; d < p.dim; d++) io[d] = ((g + idx[0][d] + 1) % 2 + 2) % 2;
    double compv[8] = {0, 0, 0, 0, 0, 0, 0, 0}, detail[8];
    for (int c = 1; c <= o.nc; c++) {
        double m = 0.0;
        bool any = false;
        for (int k = idx[0][2]; k <= idx[1][2]; k++)
            for (int j = idx[0][1]; j <= idx[1][1]; j++)
                for (int i = idx[0][0]; i <= idx[1][0]; i++) {
                    const bool sc = ((i - idx[0][0] - io[0]) % 2 == 0) && ((j - idx[0][1] - io[1]) % 2 == 0) &&
                                    (p.dim == 2 || (k - idx[0][2] - io[2]) % 2 == 0);
                    const double v = sc ? 0.0 : std::fabs(o.blk(b)[o.at(i, j, k, c)]);
                    if (!any || v > m) { m = v; any = true; }
                }
        compv[c - 1] = m;
    }
    int maxgrp = 0;
    for (int c = 0; c < o.nc; c++) maxgrp = std::max(maxgrp, p.threshold_state_vector_component[c]);
    for (int c = 0; c < o.nc; c++) detail[c] = -1.0;
    for (int l = 2; l <= maxgrp; l++) {
        double m = 0.0;
        for (int c = 0; c < o.nc; c++) if (p.threshold_state_vector_component[c] == l) m = std::max(m, compv[c]);
        for (int c = 0; c < o.nc; c++) if (p.threshold_state_vector_component[c] == l) detail[c] = m;
    }
    for (int c = 0; c < o.nc; c++) {
        if (p.threshold_state_vector_component[c] == 1) detail[c] = compv[c];
        if (p.threshold_state_vector_component[c] == 0) detail[c] = 0.0;
    }
    for (int c = 0; c < o.nc; c++)
        if (!(detail[c] <= eps_use[c])) return true;
    return false;
}

// neighborhood2patchID (LIB/TREE/neighborhood.f90:413-434)
static int patch_id(int relation) {
    const int t = (relation - 1) % 56 + 1;
    if (t <= 24) return (t - 1) / 4 + 1;
    if (t <= 48) return (t - 25) / 2 + 1 + 6;
    return (t - 49) + 1 + 6 + 12;
}

// addSecurityZone_CE_tree (LIB/MESH/securityZone_tree.f90:140-306): a block
// that stays marks each same-level neighbour that wants to coarsen and whose
// adjoining patch (Nwcl / Nwcr wide) holds significant details; the marked
// neighbours stay. The marks are encoded in the status as bit patchID+3 plus
// the flag bit 30, as lgt_encode_significant_patch (:308-340) does.
static void security_zone(Oracle &o, const double *eps_use) {
    constexpr int kTmpStatus = 17;
    const int n = (int)o.blocks.size(), g = o.cfg.g, dim = o.cfg.dim;
    const int N[3] = {o.nx, o.ny, o.nz};
    const int Ns[3] = {o.wav.Nwcl, o.wav.Nwcl, o.wav.Nwcl}, Ne[3] = {o.wav.Nwcr, o.wav.Nwcr, o.wav.Nwcr};
    const int gg[3] = {g, g, g};
    auto flag_bit = [](int r) { return (r >> 30) & 1; };
    for (int b = 0; b < n; b++) {
        if (o.ref[b] != 0) continue;
        for (int r = 1; r <= 168; r++) {
            const int nb = o.nb[size_t(b) * 168 + r - 1];
            if (nb < 0 || o.ref[nb] != -1 || o.blocks[nb].level != o.blocks[b].level) continue;
            int idx[2][3];
            modify_patch(dim, r, idx, N, Ns, Ne, gg, gg, 0);
            if (patch_significant(o, b, idx, eps_use)) o.ref[b] |= (1 << (patch_id(r) + 3)) | (1 << 30);
        }
    }
    for (int b = 0; b < n; b++) {
        if (o.ref[b] != -1) continue;
        for (int r = 1; r <= 168; r++) {
            const int nb = o.nb[size_t(b) * 168 + r - 1];
            if (nb < 0 || !(o.ref[nb] > 0) || o.blocks[nb].level != o.blocks[b].level) continue;
            const int pid = patch_id(inverse_relation(r));
            if (flag_bit(o.ref[nb]) && ((o.ref[nb] >> (pid + 3)) & 1)) o.ref[b] = kTmpStatus;
        }
    }
    for (int b = 0; b < n; b++)
        if (o.ref[b] > 0 && (o.ref[b] == kTmpStatus || flag_bit(o.ref[b]))) o.ref[b] = 0;
}

// keep the blocks whose flag is not del (and the new order of the kept ones)
static void erase_blocks(Oracle &o, const std::vector<char> &del) {
    std::vector<Block> nbl;
    std::vector<double> nd, nt;
    std::vector<int> nr;
    const size_t bsz = size_t(o.nc) * o.npts;
    for (int b = 0; b < (int)o.blocks.size(); b++) {
        if (del[b]) continue;
        nbl.push_back(o.blocks[b]);
        nd.insert(nd.end(), o.data.begin() + b * bsz, o.data.begin() + (b + 1) * bsz);
        nt.insert(nt.end(), o.tmp.begin() + b * bsz, o.tmp.begin() + (b + 1) * bsz);
        nr.push_back(o.ref[b]);
    }
    o.blocks.swap(nbl);
    o.data.swap(nd);
    o.tmp.swap(nt);
    o.ref.swap(nr);
    rebuild_lookup(o);
}

static int adapt_lifted(Oracle &o, const double *eps_use, int everywhere) {
    const wg_config &p = o.cfg;
    const Wavelet &w = o.wav;
    const int dim = p.dim, g = p.g, Jmin = p.Jmin;
    const size_t bsz = size_t(o.nc) * o.npts;
    const bool use_ce = w.lifted || o.ce_force || p.use_coarse_extension;
    bool leaf_first = true;
    for (int d = 0; d < dim; d++)
        if (p.Bs[d] < 3 * std::max(std::abs(w.HD.lo), std::abs(w.HD.hi))) leaf_first = false;
    // leaf grid metadata
    const int nleaf = (int)o.blocks.size();
    o.ref.assign(nleaf, 0);
    update_neighbors(o, false);
    update_family(o, Jmin);
    int lmax = 0;
    for (const Block &b : o.blocks) {
        if (b.level < Jmin) return WG_EGRID;
        lmax = std::max(lmax, b.level);
    }
    for (int b = 0; b < nleaf; b++)
        if (o.blocks[b].level == lmax || leaf_first) o.ref[b] = -1;
    o.tmp = o.data;
    // init_full_tree: a mother per family whose last daughter exists
    {
        const int last = (1 << dim) - 1;
        size_t nold = 0;
        std::vector<char> has_mother(o.blocks.size(), 0);
        while (nold != o.blocks.size()) {
            nold = o.blocks.size();
            has_mother.resize(nold, 0);
            for (size_t i = 0; i < nold; i++) {
                const Block b = o.blocks[i];
                if (has_mother[i] || b.level == Jmin) continue;
                const int c[3] = {b.c[0] >> 1, b.c[1] >> 1, dim == 3 ? b.c[2] >> 1 : 0};
                if (find_block(o, b.level - 1, c) >= 0) { has_mother[i] = 1; continue; }
                const int digit = (b.c[0] & 1) | ((b.c[1] & 1) << 1) | (dim == 3 ? (b.c[2] & 1) << 2 : 0);
                if (digit != last) continue;
                Block m;
                m.level = b.level - 1;
                m.c[0] = c[0];
                m.c[1] = c[1];
                m.c[2] = c[2];
                o.blocks.push_back(m);
                o.lookup[key_of(m.level, m.c[0], m.c[1], m.c[2])] = (int)o.blocks.size() - 1;
                o.ref.push_back(kRefTmpEmpty);
                has_mother[i] = 1;
            }
        }
        o.data.resize(o.blocks.size() * bsz, 0.0);
        o.tmp.resize(o.blocks.size() * bsz, 0.0);
        rebuild_lookup(o);
        update_neighbors(o, true);
        update_family(o, Jmin);
    }
    const int nt = (int)o.blocks.size();
    // wavelet_decompose_full_tree
    {
        int level = lmax, iteration = 0;
        const int g_this = std::max(std::abs(w.HD.lo), w.GD.hi);
        std::vector<double> ud(o.npts);
        while (level >= Jmin) {
            SyncSpec sp;
            sp.base = (use_ce && (!leaf_first || iteration > 0)) ? kSyncMoF : kSyncFull;
            sp.by_ref = true;
            sp.s_ref = -1;
            sp.gminus = sp.gplus = g_this;
            sp.tmp_usage = kTmpNotFlag;
            sync_generic(o, sp);
            for (int b = 0; b < nt; b++) {
                if (o.ref[b] != -1) continue;
                std::copy(o.data.begin() + b * bsz, o.data.begin() + (b + 1) * bsz, o.tmp.begin() + b * bsz);
                for (int c = 0; c < o.nc; c++)
                    fwt_block(o, o.tmp.data() + b * bsz + size_t(c) * o.npts, o.blk(b) + size_t(c) * o.npts);
            }
            if (use_ce) ce_modify(o, 2, 0, -1, true, true);
            for (int b = 0; b < nt; b++) {
                if (o.ref[b] == -1) o.ref[b] = 0;
                if ((o.ref[b] == kRefTmpEmpty || !leaf_first) && o.blocks[b].level == level - 1) o.ref[b] = -1;
            }
            sync_d2m(o, level);
            iteration++;
            level--;
        }
        std::fill(o.ref.begin(), o.ref.end(), 0);
    }
    // coarseningIndicator_tree (input_is_WD) / everywhere on leaves
    for (int b = 0; b < nt; b++) {
        if (everywhere) {
            if (blk_is_leaf(o, b, false)) o.ref[b] = -1;
        } else {
            o.ref[b] = threshold_wd(o, b, eps_use);
        }
    }
    if (!everywhere) indicator_switches(o, nt, o.ref.data());
    if (!everywhere && use_ce) security_zone(o, eps_use);
    // respectJmaxJmin_tree and ensureGradedness_tree (check_daughters)
    for (int b = 0; b < nt; b++)
        if (o.ref[b] == -1 && o.blocks[b].level <= Jmin) o.ref[b] = kRefUnsignificantStay;
    auto stays = [](int f) { return f == 0 || f == kRefUnsignificantStay; };
    const int nd = 1 << dim;
    bool changed = true;
    int guard = 0;
    while (changed) {
        changed = false;
        if (++guard > 10 * (p.Jmax + 1) + 100) return WG_EGRID;
        for (int i = 0; i < nt; i++) {
            if (o.ref[i] != -1) continue;
            const int m = o.mother[i];
            auto family_stays = [&]() {
                for (int k = 0; k < nd; k++) {
                    const int s2 = o.dau[size_t(m) * 8 + k];
                    if (s2 >= 0 && o.ref[s2] < 0) o.ref[s2] = kRefUnsignificantStay;
                }
                changed = true;
            };
            bool all_coarsen = true;
            for (int k = 0; k < nd; k++) {
                const int s2 = o.dau[size_t(m) * 8 + k];
                if (s2 < 0 || o.ref[s2] >= 0) all_coarsen = false;
            }
            if (!all_coarsen) { family_stays(); continue; }
            bool dstay = false;
            for (int k = 0; k < nd; k++) {
                const int d2 = o.dau[size_t(i) * 8 + k];
                if (d2 >= 0 && stays(o.ref[d2])) dstay = true;
            }
            if (dstay) { family_stays(); continue; }
            const Block b = o.blocks[i];
            const int nn = 1 << b.level;
            bool keep = false;
            for (int dz = (dim == 3 ? -1 : 0); dz <= (dim == 3 ? 1 : 0) && !keep; dz++)
                for (int dy = -1; dy <= 1 && !keep; dy++)
                    for (int dx = -1; dx <= 1 && !keep; dx++) {
                        if (!dx && !dy && !dz) continue;
                        const int d[3] = {dx, dy, dz};
                        int c[3] = {0, 0, 0};
                        for (int a = 0; a < dim; a++) c[a] = ((b.c[a] + d[a]) % nn + nn) % nn;
                        for (int kz = 0; kz < (dim == 3 ? 2 : 1) && !keep; kz++)
                            for (int ky = 0; ky < 2 && !keep; ky++)
                                for (int kx = 0; kx < 2 && !keep; kx++) {
                                    const int kk[3] = {kx, ky, kz};
                                    bool adj = true;
                                    for (int a = 0; a < dim; a++)
                                        if ((d[a] == 1 && kk[a] != 0) || (d[a] == -1 && kk[a] != 1)) adj = false;
                                    if (!adj) continue;
                                    const int fc[3] = {2 * c[0] + kx, 2 * c[1] + ky, dim == 3 ? 2 * c[2] + kz : 0};
                                    const int f = find_block(o, b.level + 1, fc);
                                    if (f >= 0 && stays(o.ref[f])) keep = true;
                                }
                    }
            if (keep) {
                o.ref[i] = kRefUnsignificantStay;
                changed = true;
            }
        }
    }
    // delete the blocks still flagged -1; metadata of the remaining full tree
    {
        std::vector<char> del(nt, 0);
        for (int b = 0; b < nt; b++) del[b] = o.ref[b] == -1;
        erase_blocks(o, del);
        update_neighbors(o, true);
        update_family(o, Jmin);
    }
    const int n2 = (int)o.blocks.size();
    if (use_ce) ce_modify(o, 0, 0, 0, true, false);
    if (!use_ce) {
        // nothing was modified: the original values are copied back
        o.data = o.tmp;
    } else {
        // wavelet_reconstruct_full_tree_CEoptimized
        bool leaf_only = true, recon_nb = false;
        for (int d = 0; d < dim; d++) {
            if (p.Bs[d] < w.Ndep2l || p.Bs[d] < w.Ndep2r) leaf_only = false;
            if (p.Bs[d] < w.Nreconl || p.Bs[d] < w.Nreconr) recon_nb = true;
        }
        if (recon_nb) return WG_ENOTSUP;   // sync_M2D not restated (Bs below Nrecon)
        // the reconstruction marks blocks in the status; it is restored
        // afterwards (adapt_tree.f90:721-722,978)
        const std::vector<int> saved = o.ref;
        std::fill(o.ref.begin(), o.ref.end(), 0);
        for (int b = 0; b < n2; b++) {
            if (!blk_is_leaf(o, b, false)) continue;
            for (int r = 1; r <= 168; r++) {
                const int nb = o.nb[size_t(b) * 168 + r - 1];
                if (nb < 0) continue;
                if (o.blocks[nb].level < o.blocks[b].level &&
                    !(blk_has_valid_neighbor(o, b, r, 0) || blk_has_valid_neighbor(o, b, r, -1))) {
                    o.ref[b] = -1;
                    break;
                }
            }
        }
        auto reconstruct = [&](int b) {
            if (o.ref[b] == -1)
                for (int c = 0; c < o.nc; c++)
                    iwt_block(o, o.blk(b) + size_t(c) * o.npts, o.tmp.data() + b * bsz + size_t(c) * o.npts);
            std::copy(o.tmp.begin() + b * bsz, o.tmp.begin() + (b + 1) * bsz, o.data.begin() + b * bsz);
        };
        SyncSpec sp;
        sp.base = kSyncMoC;
        sp.by_ref = true;
        sp.s_ref = -1;
        sp.gminus = sp.gplus = g;
        sp.tmp_usage = kTmpDecomposed;
        if (leaf_only) {
            sync_generic(o, sp);
            if (use_ce) ce_modify(o, 0, 0, 0, true, false);
            for (int b = 0; b < n2; b++) reconstruct(b);
        } else {
            int jmax = 0;
            for (const Block &b : o.blocks) jmax = std::max(jmax, b.level);
            for (int level = Jmin; level <= jmax; level++) {
                sp.by_level = true;
                sp.s_level = level;
                sync_generic(o, sp);
                if (use_ce) ce_modify(o, 1, level, 0, true, false);
                for (int b = 0; b < n2; b++)
                    if (o.blocks[b].level == level) reconstruct(b);
            }
        }
        o.ref = saved;
    }
    // prune_fulltree2leafs
    {
        std::vector<char> del(n2, 0);
        for (int b = 0; b < n2; b++) del[b] = !blk_is_leaf(o, b, false);
        erase_blocks(o, del);
    }
    o.status = o.ref;
    clear_mask(o);
    update_neighbors(o, false);
    update_family(o, Jmin);
    // final sync_ghosts_tree (filtered restriction)
    SyncSpec sp;
    sp.gminus = sp.gplus = g;
    sync_generic(o, sp);
    o.tmp.clear();
    return WG_OK;
}

}  // namespace

// ===========================================================================
// C ABI for tests (ctypes)
// ===========================================================================
extern "C" {

void *or_create(const wg_config *cfg) {
    // ghost widths the oracle's loops rely on (the reference aborts likewise)
    if (cfg->g < 2 || cfg->g_rhs < 2 || cfg->g_rhs > cfg->g) return nullptr;
    Oracle *o = new Oracle();
    o->cfg = *cfg;
    if (!setup_wavelet(cfg->wavelet, 2, o->wav)) { delete o; return nullptr; }
    // every filter and the predictor stencil must fit into the ghost layer
    {
        const Wavelet &w = o->wav;
        int need = std::max({std::abs(w.HD.lo), w.HD.hi, std::abs(w.GD.lo), w.GD.hi, w.X - 1});
        if (cfg->g < need) { delete o; return nullptr; }
    }
    o->nx = cfg->Bs[0] + 2 * cfg->g;
    o->ny = cfg->Bs[1] + 2 * cfg->g;
    o->nz = cfg->dim == 3 ? cfg->Bs[2] + 2 * cfg->g : 1;
    o->nc = cfg->neq;
    o->npts = o->nx * o->ny * o->nz;
    return o;
}

void or_destroy(void *h) { delete (Oracle *)h; }

void or_set_threads(void *h, int n) { ((Oracle *)h)->nthreads = n < 1 ? 1 : n; }

int or_set_grid(void *h, int nblk, const int *level, const int *coords, const double *data) {
    Oracle &o = *(Oracle *)h;
    o.blocks.resize(nblk);
    for (int i = 0; i < nblk; i++) {
        o.blocks[i].level = level[i];
        for (int d = 0; d < 3; d++) o.blocks[i].c[d] = coords[3 * i + d];
    }
    o.data.assign(size_t(nblk) * o.nc * o.npts, 0.0);
    if (data) std::memcpy(o.data.data(), data, o.data.size() * sizeof(double));
    clear_mask(o);
    update_neighbors(o);
    return WG_OK;
}

int or_nblocks(void *h) { return (int)((Oracle *)h)->blocks.size(); }

int or_get_grid(void *h, int *level, int *coords) {
    Oracle &o = *(Oracle *)h;
    for (size_t i = 0; i < o.blocks.size(); i++) {
        level[i] = o.blocks[i].level;
        for (int d = 0; d < 3; d++) coords[3 * i + d] = o.blocks[i].c[d];
    }
    return WG_OK;
}

int or_get_data(void *h, double *out) {
    Oracle &o = *(Oracle *)h;
    std::memcpy(out, o.data.data(), o.data.size() * sizeof(double));
    return WG_OK;
}

int or_set_data(void *h, const double *in) {
    Oracle &o = *(Oracle *)h;
    std::memcpy(o.data.data(), in, o.data.size() * sizeof(double));
    return WG_OK;
}

int or_set_mask(void *h, const double *mask) {
    Oracle &o = *(Oracle *)h;
    if (!mask) { clear_mask(o); return WG_OK; }
    o.mask_slot.clear();
    o.mask.assign(mask, mask + o.blocks.size() * 6 * size_t(o.npts));
    return WG_OK;
}

// masks of the n listed blocks (n * 6 * npts doubles, full-block layout);
// every other block has the all-zero mask (one shared copy)
int or_set_mask_sparse(void *h, int n, const int *ids, const double *masks) {
    Oracle &o = *(Oracle *)h;
    const int nblk = (int)o.blocks.size();
    const size_t per = 6 * size_t(o.npts);
    o.mask.assign(size_t(n + 1) * per, 0.0);
    o.mask_slot.assign(nblk, n);   // slot n: zeros
    for (int i = 0; i < n; i++) {
        if (ids[i] < 0 || ids[i] >= nblk) { clear_mask(o); return WG_EINVAL; }
        o.mask_slot[ids[i]] = i;
        std::memcpy(o.mask.data() + i * per, masks + i * per, per * sizeof(double));
    }
    return WG_OK;
}

// interior points of every block ((nblk, nc, Bz, By, Bx), x fastest) into
// the state; ghost nodes are left as they are
int or_set_interior(void *h, const double *u) {
    Oracle &o = *(Oracle *)h;
    const wg_config &p = o.cfg;
    const int g = p.g, bz = p.dim == 3 ? p.Bs[2] : 1, z0 = p.dim == 3 ? g + 1 : 1;
    const int nblk = (int)o.blocks.size();
#pragma omp parallel for num_threads(o.nthreads) if (o.nthreads > 1)
    for (int b = 0; b < nblk; b++) {
        const double *src = u + size_t(b) * o.nc * bz * p.Bs[1] * p.Bs[0];
        for (int c = 1; c <= o.nc; c++)
            for (int k = 0; k < bz; k++)
                for (int j = 0; j < p.Bs[1]; j++)
                    for (int i = 0; i < p.Bs[0]; i++)
                        o.blk(b)[o.at(g + 1 + i, g + 1 + j, z0 + k, c)] = *src++;
    }
    return WG_OK;
}

// neighbour table (nblk*168, -1 = none), 0-based block ids
int or_get_neighbors(void *h, int *out) {
    Oracle &o = *(Oracle *)h;
    std::memcpy(out, o.nb.data(), o.nb.size() * sizeof(int));
    return WG_OK;
}

int or_sync_ghosts(void *h, int gminus, int gplus, int ignore_filter) {
    Oracle &o = *(Oracle *)h;
    if (gminus < 1 || gplus < 1 || gminus > o.cfg.g || gplus > o.cfg.g) return WG_EINVAL;
    if (o.wav.lifted && !ignore_filter) {
        // sync_ghosts_tree with the filtered restriction and the SC copies
        // of restrict_copy_at_CE
        o.ref.assign(o.blocks.size(), 0);
        update_family(o, o.cfg.Jmin);
        SyncSpec sp;
        sp.gminus = gminus;
        sp.gplus = gplus;
        sync_generic(o, sp);
        return WG_OK;
    }
    sync_ghosts(o, gminus, gplus, ignore_filter != 0);
    return WG_OK;
}

// rhs for all blocks (no sync); out has full-block layout, interior written
int or_rhs(void *h, double *out) {
    Oracle &o = *(Oracle *)h;
    std::memset(out, 0, o.data.size() * sizeof(double));
    return rhs_all(o, out);
}

int or_dt(void *h, double time, double *dt) {
    *dt = calc_dt(*(Oracle *)h, time);
    return WG_OK;
}

int or_timestep(void *h, double *time, double *dt) { return rk4_step(*(Oracle *)h, time, dt); }

// per-block coarsening flag (-1/0) from the FWT of the current data
// (ghosts must have been synchronised); eps_use has neq entries
int or_threshold_flags(void *h, const double *eps_use, int *flags, double *details) {
    Oracle &o = *(Oracle *)h;
    const int nblk = (int)o.blocks.size();
#pragma omp parallel for schedule(dynamic) num_threads(o.nthreads) if (o.nthreads > 1)
    for (int b = 0; b < nblk; b++) flags[b] = threshold_block(o, b, eps_use, details ? details + size_t(b) * o.nc : nullptr);
    return WG_OK;
}

// FWT of every block (spaghetti order, interior), result into out (full layout)
int or_fwt(void *h, double *out) {
    Oracle &o = *(Oracle *)h;
    std::memcpy(out, o.data.data(), o.data.size() * sizeof(double));
    for (size_t b = 0; b < o.blocks.size(); b++)
        for (int c = 0; c < o.nc; c++) {
            const double *u = o.blk((int)b) + size_t(c) * o.npts;
            fwt_block(o, u, out + (b * o.nc + c) * o.npts);
        }
    return WG_OK;
}

// IWT of every block: in holds spaghetti data with synchronised ghosts (full
// layout); out receives the reconstructed interior (ghosts copied from in)
int or_iwt(void *h, const double *in, double *out) {
    Oracle &o = *(Oracle *)h;
    const size_t n = (size_t)o.blocks.size() * o.nc * o.npts;
    std::copy(in, in + n, out);
    std::vector<double> tmp(o.npts);
    for (size_t b = 0; b < o.blocks.size(); b++)
        for (int c = 0; c < o.nc; c++) {
            const double *u = in + (b * o.nc + c) * o.npts;
            std::copy(u, u + o.npts, tmp.begin());
            iwt_block(o, u, tmp.data());
            double *dst = out + (b * o.nc + c) * o.npts;
            std::copy(tmp.begin(), tmp.end(), dst);
        }
    // ghosts: keep in's values (the passes wrote interior x on ghost rows)
    const wg_config &p = o.cfg;
    const int g = p.g;
    for (size_t b = 0; b < o.blocks.size(); b++)
        for (int c = 0; c < o.nc; c++)
            for (int iz = 1; iz <= o.nz; iz++)
                for (int iy = 1; iy <= o.ny; iy++)
                    for (int ix = 1; ix <= o.nx; ix++) {
                        const bool interior = ix > g && ix <= p.Bs[0] + g && iy > g && iy <= p.Bs[1] + g &&
                                              (p.dim == 2 || (iz > g && iz <= p.Bs[2] + g));
                        if (interior) continue;
                        const size_t q = (b * o.nc + c) * o.npts + ((size_t)(iz - 1) * o.ny + (iy - 1)) * o.nx + (ix - 1);
                        out[q] = in[q];
                    }
    return WG_OK;
}

// wc_threshold_tree on spaghetti data of every block, in place
int or_wc_threshold(void *h, double *data, const double *thresh) {
    Oracle &o = *(Oracle *)h;
    for (size_t b = 0; b < o.blocks.size(); b++) wc_threshold_block(o, data + b * o.nc * o.npts, thresh);
    return WG_OK;
}

// adapt_tree: indicator 0 threshold-state-vector (eps_use per component), 1
// everywhere; CDF X0 by decimation unless the coarse extension is forced,
// otherwise through the full tree; returns the new block count or an error
int or_adapt(void *h, const double *eps_use, int indicator) {
    Oracle &o = *(Oracle *)h;
    const int st = o.wav.Y != 0 || o.ce_force || o.cfg.use_coarse_extension ? adapt_lifted(o, eps_use, indicator == 1)
                                                                            : adapt_unlifted(o, eps_use, indicator == 1);
    return st ? st : (int)o.blocks.size();
}

// the same through the full-tree machinery of the lifted path, also for
// unlifted wavelets (checks that machinery against the CDF X0 files)
int or_adapt_full_tree(void *h, const double *eps_use, int indicator) {
    Oracle &o = *(Oracle *)h;
    const int st = adapt_lifted(o, eps_use, indicator == 1);
    return st ? st : (int)o.blocks.size();
}

int or_refine_everywhere(void *h) {
    refine_everywhere(*(Oracle *)h);
    return WG_OK;
}

// refine_tree(..., "significant") (LIB/MESH/refine_tree.f90:1-100): the
// leaves' status of the last adaptation becomes the refinement flag
// (refinementIndicator_tree.f90:152-167: 0 -> +1, REF_UNSIGNIFICANT_STAY ->
// 0), respectJmaxJmin_tree, then ensureGradedness_tree without daughters
// (ensureGradedness_tree.f90: a block next to a finer block that refines
// refines as well, repeated until nothing changes), then refineBlock of the
// flagged blocks. Returns the new block count, or WG_EINVAL where a status
// is -1 or +1 (the reference aborts) or no adaptation set the status.
int or_refine_significant(void *h) {
    Oracle &o = *(Oracle *)h;
    const int n = (int)o.blocks.size();
    if ((int)o.status.size() != n) return WG_EINVAL;
    std::vector<int> f(o.status);
    for (int b = 0; b < n; b++) {
        if (f[b] == -1 || f[b] == 1) return WG_EINVAL;
        if (f[b] == 0) f[b] = 1;
        else if (f[b] == kRefUnsignificantStay) f[b] = 0;
        if (f[b] == 1 && o.blocks[b].level >= o.cfg.Jmax) f[b] = 0;
    }
    for (bool changed = true; changed;) {
        changed = false;
        for (int b = 0; b < n; b++) {
            if (f[b] != 0 && f[b] != kRefUnsignificantStay) continue;
            for (int r = 0; r < 168; r++) {
                const int nb = o.nb[size_t(b) * 168 + r];
                if (nb >= 0 && o.blocks[nb].level == o.blocks[b].level + 1 && f[nb] == 1) {
                    f[b] = 1;
                    changed = true;
                    break;
                }
            }
        }
    }
    std::vector<int> refine(n, 0);
    for (int b = 0; b < n; b++) refine[b] = f[b] == 1;
    refine_blocks(o, refine);
    o.status.clear();
    return (int)o.blocks.size();
}

// the leaves' status after the last adaptation (out: nblk ints, or null);
// returns its length (0 when no adaptation set it)
int or_status(void *h, int *out) {
    Oracle &o = *(Oracle *)h;
    if (out) std::copy(o.status.begin(), o.status.end(), out);
    return (int)o.status.size();
}

// the leaves' status as a restarted run reads it from its field file
// (readHDF5vct_tree with read_refinement_status, InputOutput.f90:322)
int or_set_status(void *h, int n, const int *st) {
    Oracle &o = *(Oracle *)h;
    if (n != (int)o.blocks.size()) return WG_EINVAL;
    o.status.assign(st, st + n);
    return WG_OK;
}

// the FD stencil half-width the wavelet set-up widens the coarse-extension
// zones to (module_wavelets.f90:1402-1417): 2 for FD_4th_central (the
// default), 0 where no discretization is set (the reference's wavelet
// post-processing tools)
int or_set_fd_stencil(void *h, int n) {
    Oracle &o = *(Oracle *)h;
    if (n < 0 || !setup_wavelet(o.cfg.wavelet, n, o.wav)) return WG_EINVAL;
    return WG_OK;
}

// useCoarseExtension and useSecurityZone for any wavelet (on != 0)
int or_set_coarse_extension(void *h, int on) {
    ((Oracle *)h)->ce_force = on != 0;
    return WG_OK;
}

// wavelet filters for inspection: which = 0 HD, 1 GD, 2 HR, 3 GR; returns lo, hi
int or_filter(void *h, int which, int *lo, int *hi, double *coef) {
    Oracle &o = *(Oracle *)h;
    const Filter *f = which == 0 ? &o.wav.HD : which == 1 ? &o.wav.GD : which == 2 ? &o.wav.HR : &o.wav.GR;
    *lo = f->lo;
    *hi = f->hi;
    if (coef) std::memcpy(coef, f->c.data(), f->c.size() * sizeof(double));
    return WG_OK;
}

// penalisation geometry of the forest (NULL: none); masks are built by
// or_make_mask on the current grid and used by the RHS
int or_set_geometry(void *h, const wg_geometry *geo) {
    Oracle &o = *(Oracle *)h;
    if (geo) o.geom = *geo;
    else o.geom = wg_geometry{};
    clear_mask(o);
    return WG_OK;
}

int or_make_mask(void *h) {
    make_masks(*(Oracle *)h);
    return WG_OK;
}

// the forest's masks (nblk * 6 * npts doubles); 0 if it has none
int or_get_mask(void *h, double *out) {
    Oracle &o = *(Oracle *)h;
    if (o.mask.empty()) return 0;
    for (size_t b = 0; b < o.blocks.size(); b++)
        std::memcpy(out + b * 6 * o.npts, mask_of(o, (int)b), 6 * size_t(o.npts) * sizeof(double));
    return 1;
}

// mask status of every block (coarseningIndicatorMask_tree's test)
int or_mask_status(void *h, int *out) {
    Oracle &o = *(Oracle *)h;
    for (size_t b = 0; b < o.blocks.size(); b++) out[b] = mask_status(o, (int)b);
    return WG_OK;
}

// componentWiseNorm_tree (LIB/OPERATORS/componentWiseNorm_tree.f90:1-140)
// over the leaves' interiors: which 0 = Linfty (max |u|, -1 for components
// the indicator skips), 1 = L2 (sqrt of sum u^2 dV)
int or_norm(void *h, int which, double *norm) {
    Oracle &o = *(Oracle *)h;
    const wg_config &p = o.cfg;
    const int g = p.g;
    const int z1 = p.dim == 3 ? g + 1 : 1, z2 = p.dim == 3 ? p.Bs[2] + g : 1;
    for (int c = 0; c < o.nc; c++) norm[c] = which == 0 ? -1.0 : 0.0;
    for (size_t b = 0; b < o.blocks.size(); b++) {
        double x0[3], dx[3];
        block_spacing(o, (int)b, x0, dx);
        double dV = 1.0;
        for (int d = 0; d < p.dim; d++) dV *= dx[d];
        for (int c = 1; c <= o.nc; c++) {
            if (p.threshold_state_vector_component[c - 1] != 1) continue;
            double acc = which == 0 ? 0.0 : 0.0;
            bool first = true;
            for (int iz = z1; iz <= z2; iz++)
                for (int iy = g + 1; iy <= p.Bs[1] + g; iy++)
                    for (int ix = g + 1; ix <= p.Bs[0] + g; ix++) {
                        const double v = o.blk((int)b)[o.at(ix, iy, iz, c)];
                        if (which == 0) {
                            const double a = std::fabs(v);
                            if (first || a > acc) acc = a;
                            first = false;
                        } else {
                            acc += v * v;
                        }
                    }
            if (which == 0) norm[c - 1] = std::max(norm[c - 1], acc);
            else norm[c - 1] += dV * acc;
        }
    }
    if (which == 1)
        for (int c = 0; c < o.nc; c++) norm[c] = std::sqrt(norm[c]);
    return WG_OK;
}

// run nsteps RK4 steps, returns the per-step dt in dts (may be null)
int or_run(void *h, int nsteps, double *time, double *dts) {
    Oracle &o = *(Oracle *)h;
    for (int s = 0; s < nsteps; s++) {
        double dt;
        int st = rk4_step(o, time, &dt);
        if (st) return st;
        if (dts) dts[s] = dt;
        if (*time >= o.cfg.time_max - 1e-12 * std::max(1.0, std::fabs(o.cfg.time_max))) return s + 1;
    }
    return nsteps;
}

}  // extern "C"
