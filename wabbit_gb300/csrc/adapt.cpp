// adapt.cpp -- full-tree construction, mother patches and the consistency
// rules of the coarsening decision (see adapt.hpp).
#include "adapt.hpp"

#include <algorithm>

namespace wg {

static inline uint64_t ft_key(int lv, int x, int y, int z) {
    return ((uint64_t)lv << 58) | ((uint64_t)(uint32_t)x << 38) | ((uint64_t)(uint32_t)y << 19) | (uint64_t)(uint32_t)z;
}

int FullTree::find(int lv, int x, int y, int z) const {
    auto it = lookup.find(ft_key(lv, x, y, z));
    return it == lookup.end() ? -1 : it->second;
}

int FullTree::max_level() const {
    int m = -1;
    for (int l : level) m = std::max(m, l);
    return m;
}

bool build_full_tree(int dim, int Jmin, int nblk, const int *lv, const int *co, FullTree &t, std::string &err) {
    t = FullTree();
    t.dim = dim;
    t.Jmin = Jmin;
    t.nleaves = nblk;
    auto add = [&](int l, int x, int y, int z) {
        const int id = (int)t.level.size();
        t.level.push_back(l);
        t.coords.insert(t.coords.end(), {x, y, z});
        t.mother.push_back(-1);
        t.daughters.insert(t.daughters.end(), 8, -1);
        t.lookup.emplace(ft_key(l, x, y, z), id);
        return id;
    };
    int lmax = -1;
    for (int b = 0; b < nblk; b++) {
        if (lv[b] < Jmin) {
            err = "a leaf lies below Jmin";
            return false;
        }
        if (t.find(lv[b], co[3 * b], co[3 * b + 1], co[3 * b + 2]) >= 0) {
            err = "duplicate block";
            return false;
        }
        add(lv[b], co[3 * b], co[3 * b + 1], co[3 * b + 2]);
        lmax = std::max(lmax, lv[b]);
    }
    // mothers level by level from the finest, each created once
    for (int l = lmax; l > Jmin; l--) {
        const int n = t.size();
        for (int b = 0; b < n; b++) {
            if (t.level[b] != l) continue;
            const int x = t.coords[3 * b], y = t.coords[3 * b + 1], z = t.coords[3 * b + 2];
            int m = t.find(l - 1, x >> 1, y >> 1, z >> 1);
            if (m < 0) m = add(l - 1, x >> 1, y >> 1, z >> 1);
            const int k = (x & 1) | ((y & 1) << 1) | ((z & 1) << 2);
            if (t.daughters[8 * m + k] >= 0) {
                err = "blocks overlap";
                return false;
            }
            t.daughters[8 * m + k] = b;
            t.mother[b] = m;
        }
    }
    // every mother has all 2^dim daughters (the leaves form a complete tree)
    const int nd = 1 << dim;
    for (int b = 0; b < t.size(); b++) {
        if (t.is_leaf(b)) continue;
        for (int k = 0; k < nd; k++)
            if (t.daughters[8 * b + k] < 0) {
                err = "the leaves do not form a complete tree";
                return false;
            }
    }
    return true;
}

int same_level_neighbor(const FullTree &t, int b, const int d[3]) {
    const int l = t.level[b];
    const int n = 1 << l;
    int c[3];
    for (int a = 0; a < 3; a++) {
        if (a >= t.dim) {
            if (d[a] != 0) return -1;
            c[a] = 0;
            continue;
        }
        c[a] = ((t.coords[3 * b + a] + d[a]) % n + n) % n;
    }
    return t.find(l, c[0], c[1], c[2]);
}

static inline bool stays(int f) { return f == kFlagStay || f == kFlagUnsignificantStay; }

void adapt_decide(const FullTree &t, std::vector<int> &flags, std::vector<int> &new_leaves) {
    const int n = t.size(), dim = t.dim, nd = 1 << dim;
    // respectJmaxJmin_tree: no coarsening below Jmin
    for (int b = 0; b < n; b++)
        if (flags[b] == kFlagCoarsen && t.level[b] <= t.Jmin) flags[b] = kFlagUnsignificantStay;
    // ensureGradedness_tree(check_daughters) with ensure_completeness_block:
    // only -1 -> stay transitions, repeated until nothing changes
    bool changed = true;
    while (changed) {
        changed = false;
        for (int b = 0; b < n; b++) {
            if (flags[b] != kFlagCoarsen) continue;
            const int m = t.mother[b];
            auto family_stays = [&]() {
                for (int k = 0; k < nd; k++) {
                    const int s = t.daughters[8 * m + k];
                    if (flags[s] < 0) flags[s] = kFlagUnsignificantStay;
                }
                changed = true;
            };
            // completeness: all sisters must want to coarsen
            bool sister_stays = false;
            for (int k = 0; k < nd; k++)
                if (flags[t.daughters[8 * m + k]] != kFlagCoarsen) sister_stays = true;
            if (sister_stays) {
                family_stays();
                continue;
            }
            // a block whose daughters stay cannot disappear
            if (!t.is_leaf(b)) {
                bool dstay = false;
                for (int k = 0; k < nd; k++)
                    if (stays(flags[t.daughters[8 * b + k]])) dstay = true;
                if (dstay) {
                    family_stays();
                    continue;
                }
            }
            // gradedness: a finer neighbour that stays keeps this block
            bool keep = false;
            for (int dz = (dim == 3 ? -1 : 0); dz <= (dim == 3 ? 1 : 0) && !keep; dz++)
                for (int dy = -1; dy <= 1 && !keep; dy++)
                    for (int dx = -1; dx <= 1 && !keep; dx++) {
                        if (!dx && !dy && !dz) continue;
                        const int d[3] = {dx, dy, dz};
                        const int nb = same_level_neighbor(t, b, d);
                        if (nb < 0 || t.is_leaf(nb)) continue;
                        for (int k = 0; k < nd && !keep; k++) {
                            const int kk[3] = {k & 1, (k >> 1) & 1, (k >> 2) & 1};
                            bool adjacent = true;
                            for (int a = 0; a < dim; a++)
                                if ((d[a] == 1 && kk[a] != 0) || (d[a] == -1 && kk[a] != 1)) adjacent = false;
                            if (adjacent && stays(flags[t.daughters[8 * nb + k]])) keep = true;
                        }
                    }
            if (keep) {
                flags[b] = kFlagUnsignificantStay;
                changed = true;
            }
        }
    }
    // blocks still flagged -1 are deleted; the new leaves are the remaining
    // blocks without remaining daughters
    new_leaves.clear();
    for (int b = 0; b < n; b++) {
        if (flags[b] == kFlagCoarsen) continue;
        bool has = false;
        if (!t.is_leaf(b))
            for (int k = 0; k < nd; k++)
                if (flags[t.daughters[8 * b + k]] != kFlagCoarsen) has = true;
        if (!has) new_leaves.push_back(b);
    }
}

void mother_patches(const FullTree &t, const Geometry &geo, int level, const std::vector<int> &slot,
                    std::vector<Patch> &d2m, std::vector<Patch> &ghosts) {
    const int dim = t.dim, nd = 1 << dim, g = geo.g;
    for (int m = 0; m < t.size(); m++) {
        if (t.level[m] != level || t.is_leaf(m)) continue;
        for (int k = 0; k < nd; k++) {
            Patch p{};
            p.src = slot[t.daughters[8 * m + k]];
            p.dst = slot[m];
            p.op = 1;
            for (int a = 0; a < 3; a++) {
                if (a >= dim) continue;
                const int half = geo.Bs[a] / 2, ka = (k >> a) & 1;
                p.rlo[a] = (int16_t)(g + ka * half);
                p.rhi[a] = (int16_t)(g + ka * half + half - 1);
                p.slo[a] = (int16_t)g;
                p.shi[a] = (int16_t)(g + geo.Bs[a] - 1);
            }
            d2m.push_back(p);
        }
        for (int dz = (dim == 3 ? -1 : 0); dz <= (dim == 3 ? 1 : 0); dz++)
            for (int dy = -1; dy <= 1; dy++)
                for (int dx = -1; dx <= 1; dx++) {
                    if (!dx && !dy && !dz) continue;
                    const int d[3] = {dx, dy, dz};
                    const int nb = same_level_neighbor(t, m, d);
                    if (nb < 0) continue;
                    Patch p{};
                    p.src = slot[nb];
                    p.dst = slot[m];
                    p.op = 0;
                    for (int a = 0; a < dim; a++) {
                        const int B = geo.Bs[a];
                        const int lo = d[a] < 0 ? 0 : d[a] == 0 ? g : g + B;
                        const int hi = d[a] < 0 ? g - 1 : d[a] == 0 ? g + B - 1 : B + 2 * g - 1;
                        const int s0 = d[a] < 0 ? B : g;
                        p.rlo[a] = (int16_t)lo;
                        p.rhi[a] = (int16_t)hi;
                        p.slo[a] = (int16_t)s0;
                        p.shi[a] = (int16_t)(s0 + hi - lo);
                    }
                    ghosts.push_back(p);
                }
    }
}

}  // namespace wg
