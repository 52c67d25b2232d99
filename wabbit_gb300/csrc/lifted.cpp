// lifted.cpp -- host planning of the full-tree adaptation with coarse
// extension (see lifted.hpp).
#include "lifted.hpp"
#include "par.hpp"

#include <algorithm>
#include <cstring>
#include <thread>
#include <unordered_map>

namespace wg {

bool LiftedTree::init(const Geometry &g, const WaveletInfo &w, int fd_max_size, int jmin, int jmax, int nleaf,
                      const int *level, const int *coords, std::string &err) {
    geo = g;
    wav = w;
    Jmin = jmin;
    Jmax = jmax;
    nleaves = nleaf;
    if (!build_full_tree(g.dim, jmin, nleaf, level, coords, ft, err)) return false;
    alive.assign(ft.size(), 1);
    full_ready_ = false;
    ref.assign(ft.size(), 0);
    slot.assign(ft.size(), -1);
    size_t cap = 16;
    while (cap < size_t(ft.size()) * 2 + 16) cap <<= 1;
    keys_.assign(cap, 0);
    vals_.assign(cap, -1);
    mask_ = cap - 1;
    for (int b = 0; b < ft.size(); b++) {
        const uint64_t k = ((uint64_t)ft.level[b] << 60) | ((uint64_t)ft.coords[3 * b] << 40) |
                           ((uint64_t)ft.coords[3 * b + 1] << 20) | (uint64_t)ft.coords[3 * b + 2];
        uint64_t h = (k * 0x9E3779B97F4A7C15ull) >> 20 & mask_;
        while (vals_[h] >= 0) h = (h + 1) & mask_;
        keys_[h] = k;
        vals_[h] = b;
    }
    // coarse-extension widths: setup_wavelet (module_wavelets.f90:1341-1417);
    // CDF24/26/28/46 are not built, so no extra WC width applies
    const int hd_hi = w.hd_lo + (int)w.HD.size() - 1, gd_hi = w.gd_lo + (int)w.GD.size() - 1;
    const int hr_hi = w.hr_lo + (int)w.HR.size() - 1, gr_hi = w.gr_lo + (int)w.GR.size() - 1;
    Nscl = std::max(std::abs(w.hd_lo) - 1, 0);
    Nwcl = Nscl + std::abs(w.gd_lo);
    Nreconl = Nwcl + std::abs(w.gr_lo);
    Ndep2l = Nreconl + std::max((std::abs(w.hr_lo) + 1) / 2 - 1, 0);
    Nscr = hd_hi;
    Nwcr = Nscr + gd_hi;
    Nreconr = Nwcr + gr_hi;
    Ndep2r = Nreconr + (hr_hi + 1) / 2;
    const int i2 = 2 * fd_max_size, dl = std::max(i2 - Nwcl, 0), dr = std::max(i2 - Nwcr, 0);
    Nwcl += dl;
    Nreconl += dl;
    Ndep2l += dl;
    Nwcr += dr;
    Nreconr += dr;
    Ndep2r += dr;
    return true;
}

int LiftedTree::find_(int lv, int x, int y, int z) const {
    const uint64_t k = ((uint64_t)lv << 60) | ((uint64_t)x << 40) | ((uint64_t)y << 20) | (uint64_t)z;
    for (uint64_t h = (k * 0x9E3779B97F4A7C15ull) >> 20 & mask_;; h = (h + 1) & mask_) {
        if (vals_[h] < 0) return -1;
        if (keys_[h] == k) return vals_[h];
    }
}

// find_neighbor with search_overlapping (find_neighbors.f90:18-215) on the
// full tree: the same-level block, then the finer parts up to the first
// missing one, then the coarser block; only alive blocks are recorded. The
// finer blocks are daughters and the coarser block the mother of the
// same-level position's block of the full tree, when it exists.
void LiftedTree::search_all_() {
    const int dim = geo.dim, nch = host_threads();
    std::vector<std::vector<std::pair<int, int>>> part(nch);
    std::vector<std::vector<int>> count(nch);
    par_chunks(size(), nch, [&](int ch, int lo, int hi) {
        std::vector<std::pair<int, int>> &out = part[ch];
        std::vector<int> &cnt = count[ch];
        cnt.assign(hi - lo, 0);
        // neighbour per relation (each relation occurs at most once): read
        // out in ascending order without a sort
        int slot[kNumRelations];
        int used[kNumRelations], nused = 0;
        for (int b = lo; b < hi; b++) {
            const int lv = ft.level[b];
            const int *c = &ft.coords[3 * b];
            const int N = 1 << lv;
            nused = 0;
            for (int dz = (dim == 3 ? -1 : 0); dz <= (dim == 3 ? 1 : 0); dz++)
                for (int dy = -1; dy <= 1; dy++)
                    for (int dx = -1; dx <= 1; dx++) {
                        if (!dx && !dy && !dz) continue;
                        const int d[3] = {dx, dy, dz};
                        int nfree = 0;
                        for (int i = 0; i < dim; i++) nfree += (d[i] == 0);
                        const int nparts = 1 << nfree;
                        int a[3] = {0, 0, 0};
                        for (int i = 0; i < dim; i++) a[i] = (c[i] + d[i]) & (N - 1);   // periodic, N a power of two
                        const int same = lv == 0 ? b : find_(lv, a[0], a[1], a[2]);
                        if (same >= 0) {
                            const int r = relation_id(d, 0, dim) - 1;
                            slot[r] = same;
                            used[nused++] = r;
                        }
                        if (lv < Jmax && same >= 0)
                            for (int p = 0; p < nparts; p++) {
                                int k = 0, fr = 0;
                                for (int i = 0; i < dim; i++) {
                                    int bit;
                                    if (d[i] == 0) bit = (p >> fr++) & 1;
                                    else bit = d[i] > 0 ? 1 : 0;
                                    // daughter bit of the fine neighbour: (2c + bit + d) mod 2
                                    k |= ((bit + d[i]) & 1) << i;
                                }
                                const int f = ft.daughters[8 * same + k];
                                if (f < 0) break;
                                const int r = relation_id(d, p, dim) + 111;
                                slot[r] = f;
                                used[nused++] = r;
                            }
                        if (lv <= Jmin) continue;
                        int prt = 0, fr = 0;
                        bool touches = true;
                        for (int i = 0; i < dim; i++) {
                            const int bit = c[i] & 1;
                            if (d[i] == 0) prt |= bit << fr++;
                            else if ((d[i] > 0) != (bit == 1)) touches = false;
                        }
                        if (!touches) continue;
                        const int cb = same >= 0 ? ft.mother[same] : find_(lv - 1, a[0] >> 1, a[1] >> 1, a[2] >> 1);
                        if (cb >= 0) {
                            const int r = relation_id(d, prt, dim) + 55;
                            slot[r] = cb;
                            used[nused++] = r;
                        }
                    }
            // the used relations in ascending order: a 168-bit mask
            uint64_t mk[3] = {0, 0, 0};
            for (int i = 0; i < nused; i++) mk[used[i] >> 6] |= 1ull << (used[i] & 63);
            for (int w = 0; w < 3; w++)
                for (uint64_t m = mk[w]; m; m &= m - 1) {
                    const int r = w * 64 + __builtin_ctzll(m);
                    out.push_back({r + 1, slot[r]});
                }
            cnt[b - lo] = nused;
        }
    }, 2048);
    full_begin_.assign(size() + 1, 0);
    full_adj_.clear();
    size_t total = 0;
    for (const auto &v : part) total += v.size();
    full_adj_.reserve(total);
    int b = 0;
    for (int ch = 0; ch < nch; ch++) {
        for (int k : count[ch]) {
            full_begin_[b + 1] = full_begin_[b] + k;
            b++;
        }
        full_adj_.insert(full_adj_.end(), part[ch].begin(), part[ch].end());
    }
    for (; b < size(); b++) full_begin_[b + 1] = full_begin_[b];
    // direction and part of every finer relation
    rel_dir_.assign(kNumRelations, -1);
    rel_part_.assign(kNumRelations, 0);
    for (int dz = (dim == 3 ? -1 : 0); dz <= (dim == 3 ? 1 : 0); dz++)
        for (int dy = -1; dy <= 1; dy++)
            for (int dx = -1; dx <= 1; dx++) {
                if (!dx && !dy && !dz) continue;
                const int d[3] = {dx, dy, dz};
                int nfree = 0;
                for (int i = 0; i < dim; i++) nfree += (d[i] == 0);
                for (int p = 0; p < (1 << nfree); p++) {
                    const int r = relation_id(d, p, dim) + 111;
                    rel_dir_[r] = (dx + 1) + 3 * (dy + 1) + 9 * (dz + 1);
                    rel_part_[r] = p;
                }
            }
    full_ready_ = true;
}

// find_neighbor with search_overlapping restricted to the alive blocks: a
// filter of the all-alive search (computed once per tree). Same-level and
// coarser neighbours stay when alive; the finer parts of a direction stay up
// to the first part that is missing or not alive.
bool LiftedTree::update_metadata(std::string &err) {
    (void)err;
    if (!full_ready_) search_all_();
    const int n = size(), nch = host_threads();
    std::vector<int> cnt(n, 0);
    par_chunks(n, nch, [&](int, int lo, int hi) {
        for (int b = lo; b < hi; b++) {
            if (!alive[b]) continue;
            int dead[27];
            for (int k = 0; k < 27; k++) dead[k] = 1 << 20;
            for (int i = full_begin_[b]; i < full_begin_[b + 1]; i++) {
                const int r = full_adj_[i].first - 1;
                if (r >= 112 && !alive[full_adj_[i].second]) dead[rel_dir_[r]] = std::min(dead[rel_dir_[r]], rel_part_[r]);
            }
            int c = 0;
            for (int i = full_begin_[b]; i < full_begin_[b + 1]; i++) {
                const int r = full_adj_[i].first - 1;
                c += r < 112 ? alive[full_adj_[i].second] != 0 : rel_part_[r] < dead[rel_dir_[r]];
            }
            cnt[b] = c;
        }
    }, 2048);
    adj_begin_.assign(n + 1, 0);
    for (int b = 0; b < n; b++) adj_begin_[b + 1] = adj_begin_[b] + cnt[b];
    adj_.resize(adj_begin_[n]);
    par_chunks(n, nch, [&](int, int lo, int hi) {
        for (int b = lo; b < hi; b++) {
            if (!cnt[b]) continue;
            int dead[27];
            for (int k = 0; k < 27; k++) dead[k] = 1 << 20;
            for (int i = full_begin_[b]; i < full_begin_[b + 1]; i++) {
                const int r = full_adj_[i].first - 1;
                if (r >= 112 && !alive[full_adj_[i].second]) dead[rel_dir_[r]] = std::min(dead[rel_dir_[r]], rel_part_[r]);
            }
            int at = adj_begin_[b];
            for (int i = full_begin_[b]; i < full_begin_[b + 1]; i++) {
                const int r = full_adj_[i].first - 1;
                if (r < 112 ? alive[full_adj_[i].second] != 0 : rel_part_[r] < dead[rel_dir_[r]]) adj_[at++] = full_adj_[i];
            }
        }
    }, 2048);
    return true;
}

// updateFamily_tree (LIB/MESH/updateFamily_tree.f90:16-56): no mother on
// Jmin, no daughters on Jmax
int LiftedTree::mother(int b) const {
    if (ft.level[b] == Jmin) return -1;
    const int m = ft.mother[b];
    return (m >= 0 && alive[m]) ? m : -1;
}

// block_is_leaf / block_is_root / block_has_valid_neighbor
// (LIB/MPI/block_relations.f90:2-71)
bool LiftedTree::is_leaf(int b, bool check_empty) const {
    if (ft.level[b] == Jmax) return true;
    bool any = false;
    for (int k = 0; k < 8; k++) {
        const int d = ft.daughters[8 * b + k];
        if (d >= 0 && alive[d]) any = true;
    }
    if (!any) return true;
    if (!check_empty) return false;
    for (int k = 0; k < 8; k++) {
        const int d = ft.daughters[8 * b + k];
        if (d >= 0 && alive[d] && ref[d] != kRefTmpEmpty) return false;
    }
    return true;
}

bool LiftedTree::is_root(int b, bool check_empty) const {
    const int m = mother(b);
    if (m < 0) return true;
    return check_empty && ref[m] == kRefTmpEmpty;
}

bool LiftedTree::has_valid_neighbor(int b, int relation, int lvl_diff) const {
    int lo, hi;
    relation_range(relation, lvl_diff, lo, hi);
    for (int i = adj_begin_[b]; i < adj_begin_[b + 1]; i++) {
        const int r = adj_[i].first;
        if (r > hi) break;
        if (r >= lo && ref[adj_[i].second] != kRefTmpEmpty) return true;
    }
    return false;
}

namespace {
struct Box {
    int lo[3], hi[3];
};
inline bool overlap(const Box &a, const Box &b) {
    for (int d = 0; d < 3; d++)
        if (a.hi[d] < b.lo[d] || b.hi[d] < a.lo[d]) return false;
    return true;
}
// boxes read / written by the patches of the current wave, per arena slot
// (dense, cleared through the list of touched slots)
struct WaveBoxes {
    std::vector<std::vector<Box>> rd, wr;
    std::vector<int> touched;
    bool hits(const std::vector<std::vector<Box>> &m, int s, const Box &b) const {
        if (s >= (int)m.size()) return false;
        for (const Box &x : m[s])
            if (overlap(x, b)) return true;
        return false;
    }
    void add(std::vector<std::vector<Box>> &m, int s, const Box &b) {
        if (s >= (int)rd.size()) {
            rd.resize(s + 1);
            wr.resize(s + 1);
        }
        if (rd[s].empty() && wr[s].empty()) touched.push_back(s);
        m[s].push_back(b);
    }
    void clear() {
        for (int s : touched) {
            rd[s].clear();
            wr[s].clear();
        }
        touched.clear();
    }
};
int pred_need_of(const Patch &p, int order_predictor) {
    const int h = order_predictor - 1;
    const int cx = p.shi[0] - p.slo[0] + 1, cy = p.shi[1] - p.slo[1] + 1, cz = p.shi[2] - p.slo[2] + 1;
    const int Fy = 2 * cy - 1, Fz = 2 * cz - 1;
    const int ex = p.rhi[0] - p.rlo[0] + 1, ey = p.rhi[1] - p.rlo[1] + 1, ez = p.rhi[2] - p.rlo[2] + 1;
    int yw0 = std::max(0, p.blo[1] - h), yw1 = std::min(Fy - 1, p.blo[1] + ey - 1 + h);
    yw0 += yw0 & 1;
    yw1 -= yw1 & 1;
    int zw0 = std::max(0, p.blo[2] - h), zw1 = std::min(Fz - 1, p.blo[2] + ez - 1 + h);
    zw0 += zw0 & 1;
    zw1 -= zw1 & 1;
    const int ny = (yw1 - yw0) / 2 + 1, nz = (zw1 - zw0) / 2 + 1;
    return cx * cy * cz + ex * ny * nz + ex * ey * nz;
}
}  // namespace

// sync_ghosts_generic with the single-rank send logic of
// prepare_ghost_synch_metadata (synchronize_ghosts_generic.f90:352-694)
void LiftedTree::plan_sync(const SyncSpecL &sp, std::vector<SyncWave> &waves) const {
    waves.clear();
    const int nstages = wav.lifted ? 3 : 2, unl = wav.lifted ? 0 : 1;
    const int nch = host_threads();
    // candidates of every stage in sender-major order, after the cheap
    // receiver filters (one pass over the senders, in parallel chunks)
    struct Cand {
        int b, r, n, lvl_diff;
    };
    std::vector<std::vector<std::vector<Cand>>> cpart(nch, std::vector<std::vector<Cand>>(nstages + 1));
    par_chunks(size(), nch, [&](int ch, int lo, int hi) {
        for (int b = lo; b < hi; b++) {
            if (!alive[b]) continue;
            if (sp.base == 2 && !is_leaf(b, false)) continue;
            if (ref[b] == kRefTmpEmpty) continue;
            const int level = ft.level[b];
            for_neighbors(b, [&](int r, int n) {
                if (ref[n] == kRefTmpEmpty) return;
                if (sp.by_ref && ref[n] != sp.s_ref) return;
                if (sp.by_level && ft.level[n] != sp.s_level) return;
                const int lvl_diff = level - ft.level[n];
                const int stage = lvl_diff == 0 ? 1 : lvl_diff == +1 ? 2 - unl : 3 - unl;
                cpart[ch][stage].push_back({b, r, n, lvl_diff});
            });
        }
    }, 2048);
    // the boxes of a patch depend on its relation and level difference only
    std::vector<Patch> tmpl(3 * (kNumRelations + 1));
    std::vector<int> tmpl_need(3 * (kNumRelations + 1), -1);
    for (int ld = -1; ld <= 1; ld++)
        for (int r = 1; r <= kNumRelations; r++) {
            const int k = (ld + 1) * (kNumRelations + 1) + r;
            tmpl[k] = make_patch(geo, wav.order_predictor, r, ld, sp.gminus, sp.gplus, 0, 0);
            if (ld == -1) tmpl_need[k] = pred_need_of(tmpl[k], wav.order_predictor);
        }
    // send rule of the case, the data source and the patch of one candidate
    auto prepare = [&](const Cand &cd, Patch &p, int &need, bool &tmp_rp, bool &tmp_same) {
        const int b = cd.b, r = cd.r, lvl_diff = cd.lvl_diff;
        bool send = false;
        switch (sp.base) {
        case 1:
            send = true;
            if (lvl_diff == -1 && !is_leaf(b, true)) send = false;
            if (lvl_diff == +1 && !is_root(b, true)) send = false;
            break;
        case 2:
            send = true;
            if (lvl_diff >= 0 && has_valid_neighbor(b, r, -1)) send = false;
            else if (lvl_diff == +1 && has_valid_neighbor(b, r, 0)) send = false;
            break;
        case 3:
            send = lvl_diff != +1;
            if (send && lvl_diff != 0 && !is_leaf(b, true)) send = false;
            break;
        case 4:
            send = lvl_diff != -1;
            if (send && lvl_diff != 0 && !is_root(b, true)) send = false;
            break;
        default:
            send = lvl_diff == 0;
        }
        if (!send) return false;
        // hvy_tmp_usage (xfer_block_data.f90:376-395)
        tmp_rp = tmp_same = false;
        if (sp.tmp_usage == 1 && ref[b] != sp.s_ref) tmp_rp = tmp_same = true;
        if (sp.tmp_usage == 2) tmp_rp = true;
        const int k = (lvl_diff + 1) * (kNumRelations + 1) + r;
        p = tmpl[k];
        p.src = slot[b];
        p.dst = slot[cd.n];
        need = tmpl_need[k];
        return true;
    };
    // add a prepared patch to a wave (restrictions: one filter entry per
    // sender and source in the wave, with its coarse-extension SC copies)
    auto add = [&](const Cand &cd, Patch p, int need, bool tmp_rp, bool tmp_same, SyncWave &cur,
                   std::unordered_map<int, int> &entry_of) {
        const int b = cd.b, lvl_diff = cd.lvl_diff, level = ft.level[b];
        if (lvl_diff == 0) {
            (tmp_same ? cur.copy_tmp : cur.copy_blk).push_back(p);
            return;
        }
        if (lvl_diff == -1) {
            (tmp_rp ? cur.pred_tmp : cur.pred_blk).push_back(p);
            cur.max_coarse = std::max(cur.max_coarse, need);
            return;
        }
        const int key = 2 * b + (tmp_rp ? 1 : 0);
        auto it = entry_of.find(key);
        int e;
        if (it == entry_of.end()) {
            e = (int)cur.filters.size();
            entry_of[key] = e;
            cur.filters.push_back({slot[b], tmp_rp ? 1 : 0});
            // SC next to a coarser or finer neighbour without a same-level
            // one are copied, not filtered
            const int g = geo.g;
            const bool leaf = is_leaf(b, false);
            for_neighbors(b, [&](int r2, int n2) {
                if (!sp.filter || !leaf) return;
                const int ld = level - ft.level[n2];
                if ((ld != 1 && ld != -1) || has_valid_neighbor(b, r2, 0)) return;
                int lo[3], hi[3];
                modify_box0(geo, r2, Nscl, Nscr, g, g, +1, lo, hi);
                ScBox sb;
                sb.entry = e;
                bool empty = false;
                for (int d = 0; d < 3; d++) {
                    if (d >= geo.dim) {
                        sb.lo[d] = sb.hi[d] = 0;
                        continue;
                    }
                    // SC lattice g + 2m (0-based); the box starts on it
                    const int first = lo[d] + ((lo[d] - g) & 1);
                    int last = hi[d] - ((hi[d] - g) & 1);
                    if (last > g + geo.Bs[d] - 2) last = g + geo.Bs[d] - 2;
                    sb.lo[d] = (int16_t)((first - g) / 2);
                    sb.hi[d] = (int16_t)((last - g) / 2);
                    if (first > last || first < g) empty = true;
                }
                if (!empty) cur.ce_copies.push_back(sb);
            });
        } else {
            e = it->second;
        }
        p.src = e;
        cur.restrict_.push_back(p);
    };
    for (int istage = 1; istage <= nstages; istage++) {
        size_t ncand = 0;
        for (int ch = 0; ch < nch; ch++) ncand += cpart[ch][istage].size();
        if (ncand == 0) continue;
        if (wav.lifted && sp.filter && istage == 2 - unl) {
            // HD-filtered restrictions: the reference handles the senders in
            // order and filters a sender's block when it first sends, from its
            // current data, so restrictions written into its ghost nodes by
            // earlier senders of the stage are part of its filter input. A
            // wave runs all its filters before its writes: a new wave starts
            // when a sender that reads hvy_block was written in this one.
            SyncWave cur;
            cur.stage = istage;
            std::unordered_map<int, int> entry_of;
            std::vector<char> written(size(), 0);
            std::vector<int> touched;
            int sender = -1;
            auto flush = [&]() {
                if (!cur.restrict_.empty()) waves.push_back(std::move(cur));
                cur = SyncWave();
                cur.stage = istage;
                entry_of.clear();
                for (int t : touched) written[t] = 0;
                touched.clear();
            };
            for (int ch = 0; ch < nch; ch++)
                for (const Cand &cd : cpart[ch][istage]) {
                    Patch p;
                    int need;
                    bool tmp_rp, tmp_same;
                    if (!prepare(cd, p, need, tmp_rp, tmp_same)) continue;
                    if (cd.b != sender) {
                        sender = cd.b;
                        if (!tmp_rp && written[cd.b]) flush();
                    }
                    add(cd, p, need, tmp_rp, tmp_same, cur, entry_of);
                    if (!written[cd.n]) {
                        written[cd.n] = 1;
                        touched.push_back(cd.n);
                    }
                }
            flush();
            continue;
        }
        if (istage != 3 - unl) {
            // copies (and unfiltered restrictions) never conflict within a
            // stage (they read the sender's interior and write ghost nodes,
            // and the ghost boxes of the relations of one receiver are
            // disjoint): the stage is one wave, built per chunk of senders in
            // parallel
            std::vector<SyncWave> part(nch);
            auto chunk = [&](int c) {
                std::unordered_map<int, int> entry_of;
                part[c].stage = istage;
                for (const Cand &cd : cpart[c][istage]) {
                    Patch p;
                    int need;
                    bool tmp_rp, tmp_same;
                    if (prepare(cd, p, need, tmp_rp, tmp_same)) add(cd, p, need, tmp_rp, tmp_same, part[c], entry_of);
                }
            };
            if (ncand >= 2048) par_tasks(nch, chunk);
            else
                for (int c = 0; c < nch; c++) chunk(c);
            // one wave for the stage made of the chunks' lists in chunk
            // order; filter entries renumbered in place
            std::vector<int> off(nch + 1, 0);
            for (int c = 0; c < nch; c++) off[c + 1] = off[c] + (int)part[c].filters.size();
            auto renumber = [&](int c) {
                for (ScBox &x : part[c].ce_copies) x.entry += off[c];
                for (Patch &x : part[c].restrict_) x.src += off[c];
            };
            if (ncand >= 2048) par_tasks(nch, renumber);
            else
                for (int c = 0; c < nch; c++) renumber(c);
            SyncWave all;
            all.stage = istage;
            bool any = false;
            for (int c = 0; c < nch; c++) {
                any = any || !part[c].copy_blk.empty() || !part[c].copy_tmp.empty() || !part[c].restrict_.empty();
                if (!part[c].copy_blk.empty() || !part[c].copy_tmp.empty() || !part[c].filters.empty())
                    all.parts.push_back(std::move(part[c]));
            }
            if (any) waves.push_back(std::move(all));
            continue;
        }
        // predictions: in the reference's order, cut into waves where a
        // patch would see or clobber a box an earlier patch of the wave
        // touches
        SyncWave cur;
        cur.stage = istage;
        WaveBoxes wb;
        std::unordered_map<int, int> entry_of;
        auto flush = [&]() {
            if (!cur.pred_blk.empty() || !cur.pred_tmp.empty()) waves.push_back(std::move(cur));
            cur = SyncWave();
            cur.stage = istage;
            wb.clear();
        };
        for (int ch = 0; ch < nch; ch++)
            for (const Cand &cd : cpart[ch][istage]) {
                Patch p;
                int need;
                bool tmp_rp, tmp_same;
                if (!prepare(cd, p, need, tmp_rp, tmp_same)) continue;
                const bool reads_blk = !tmp_rp;
                const Box w{{p.rlo[0], p.rlo[1], p.rlo[2]}, {p.rhi[0], p.rhi[1], p.rhi[2]}};
                const Box rd{{p.slo[0], p.slo[1], p.slo[2]}, {p.shi[0], p.shi[1], p.shi[2]}};
                const bool conflict = (reads_blk && wb.hits(wb.wr, p.src, rd)) || wb.hits(wb.rd, p.dst, w) ||
                                      wb.hits(wb.wr, p.dst, w);
                if (conflict) flush();
                if (reads_blk) wb.add(wb.rd, p.src, rd);
                wb.add(wb.wr, p.dst, w);
                add(cd, p, need, tmp_rp, tmp_same, cur, entry_of);
            }
        flush();
    }
}

// coarseExtensionManipulateWC_block (module_wavelets.f90:877-962): zero the
// WC in the Nwcl/Nwcr patch and in the ghost patch, SC skipped by parity
void LiftedTree::ce_clear_wc(int b, int relation, std::vector<BoxOp> &ops) const {
    const int g = geo.g, dim = geo.dim;
    for (int set = 1; set <= 2; set++) {
        int lo[3], hi[3];
        if (set == 1) modify_box0(geo, relation, Nwcl, Nwcr, g, g, +1, lo, hi);
        else ghost_box0(geo, relation, g, g, +1, lo, hi);
        if (dim == 2) lo[2] = hi[2] = 0;
        int io[3] = {0, 0, 0};
        for (int d = 0; d < dim; d++) io[d] = ((g + lo[d]) % 2 + 2) % 2;
        auto add = [&](const int first[3], const int step[3]) {
            BoxOp o;
            std::memset(&o, 0, sizeof(o));
            o.slot = slot[b];
            o.op = 0;
            for (int d = 0; d < 3; d++) {
                if (first[d] > hi[d]) return;
                o.lo[d] = (int16_t)first[d];
                o.hi[d] = (int16_t)hi[d];
                o.step[d] = (int16_t)step[d];
            }
            ops.push_back(o);
        };
        {
            const int f[3] = {lo[0] + 1 - io[0], lo[1] + io[1], lo[2] + io[2]}, s[3] = {2, 2, 2};
            add(f, s);
        }
        {
            const int f[3] = {lo[0], lo[1] + 1 - io[1], lo[2] + io[2]}, s[3] = {1, 2, 2};
            add(f, s);
        }
        if (dim == 3) {
            const int f[3] = {lo[0], lo[1], lo[2] + 1 - io[2]}, s[3] = {1, 1, 2};
            add(f, s);
        }
    }
}

// coarseExtensionManipulateSC_block (module_wavelets.f90:966-1028) with the
// copy taken from hvy_tmp
void LiftedTree::ce_copy_sc(int b, int relation, std::vector<BoxOp> &ops) const {
    const int g = geo.g, dim = geo.dim;
    int lo[3], hi[3];
    modify_box0(geo, relation, Nscl, Nscr, g, g, +1, lo, hi);
    BoxOp o;
    std::memset(&o, 0, sizeof(o));
    o.slot = slot[b];
    o.op = 1;
    for (int d = 0; d < 3; d++) {
        const int io = d < dim ? ((g + lo[d]) % 2 + 2) % 2 : 0;
        if (lo[d] + io > hi[d]) return;
        o.lo[d] = (int16_t)(lo[d] + io);
        o.hi[d] = (int16_t)hi[d];
        o.step[d] = 2;
    }
    ops.push_back(o);
}

void LiftedTree::plan_ce_modify(int ce_case, int s_level, int s_ref, bool clear_wc, bool copy_sc,
                                std::vector<BoxOp> &ops) const {
    // per chunk of blocks on the host pool, joined in block order
    const int nch = host_threads();
    std::vector<std::vector<BoxOp>> part(nch);
    par_chunks(size(), nch, [&](int ch, int lo, int hi) {
        std::vector<BoxOp> &out = part[ch];
        for (int b = lo; b < hi; b++) {
            if (!alive[b]) continue;
            const int lv = ft.level[b];
            if ((ce_case == 1 || ce_case == 3) && lv != s_level) continue;
            if ((ce_case == 2 || ce_case == 3) && ref[b] != s_ref) continue;
            if (!is_leaf(b, false)) continue;
            for_neighbors(b, [&](int r, int n) {
                if (ft.level[n] < lv && !(has_valid_neighbor(b, r, 0) || has_valid_neighbor(b, r, -1))) {
                    if (clear_wc) ce_clear_wc(b, r, out);
                    if (copy_sc) ce_copy_sc(b, r, out);
                }
            });
        }
    }, 2048);
    ops.clear();
    for (const auto &v : part) ops.insert(ops.end(), v.begin(), v.end());
}

void LiftedTree::security_candidates(std::vector<ZoneItem> &items) const {
    items.clear();
    const int g = geo.g;
    for (int b = 0; b < size(); b++) {
        if (!alive[b] || ref[b] != 0) continue;
        for_neighbors(b, [&](int r, int n) {
            if (ref[n] != -1 || ft.level[n] != ft.level[b]) return;
            ZoneItem it;
            it.block = b;
            it.relation = r;
            modify_box0(geo, r, Nwcl, Nwcr, g, g, 0, it.lo, it.hi);
            for (int d = 0; d < 3; d++) it.io[d] = d < geo.dim ? ((g + it.lo[d]) % 2 + 2) % 2 : 0;
            items.push_back(it);
        });
    }
}

void LiftedTree::security_apply(const std::vector<ZoneItem> &items, const std::vector<char> &significant) {
    constexpr int kTmpStatus = 17;
    for (size_t i = 0; i < items.size(); i++)
        if (significant[i]) ref[items[i].block] |= (1 << (relation_patch_id(items[i].relation) + 3)) | (1 << 30);
    auto flag_bit = [](int v) { return (v >> 30) & 1; };
    for (int b = 0; b < size(); b++) {
        if (!alive[b] || ref[b] != -1) continue;
        for_neighbors(b, [&](int r, int n) {
            if (!(ref[n] > 0) || ft.level[n] != ft.level[b]) return;
            const int pid = relation_patch_id(relation_inverse(r));
            if (flag_bit(ref[n]) && ((ref[n] >> (pid + 3)) & 1)) ref[b] = kTmpStatus;
        });
    }
    for (int b = 0; b < size(); b++)
        if (alive[b] && ref[b] > 0 && (ref[b] == kTmpStatus || flag_bit(ref[b]))) ref[b] = 0;
}

}  // namespace wg
