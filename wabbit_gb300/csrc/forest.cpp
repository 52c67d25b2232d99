// forest.cpp -- neighbour search and ghost-patch tables (host side).
#include "forest.hpp"
#include "par.hpp"

#include <algorithm>
#include <cmath>
#include <cstring>

namespace wg {

// ---------------------------------------------------------------------------
// wavelet filter bank (setup_wavelet, LIB/WAVELETS/module_wavelets.f90:1031-1561)
// ---------------------------------------------------------------------------
static void interp_stencil(int order, std::vector<double> &c, int &lo) {
    // interpolation stencil with interleaved zeros, centre tap = 1
    // (Stencil_Int_*th, module_wavelets.f90:14-22)
    static const double s2[] = {1, 2, 1};
    static const double s4[] = {-1, 0, 9, 16, 9, 0, -1};
    static const double s6[] = {3, 0, -25, 0, 150, 256, 150, 0, -25, 0, 3};
    static const double s8[] = {-5, 0, 49, 0, -245, 0, 1225, 2048, 1225, 0, -245, 0, 49, 0, -5};
    const double *s = order == 2 ? s2 : order == 4 ? s4 : order == 6 ? s6 : s8;
    double den = order == 2 ? 2.0 : order == 4 ? 16.0 : order == 6 ? 256.0 : 2048.0;
    int n = 2 * order - 1;
    lo = -(order - 1);
    c.resize(n);
    for (int i = 0; i < n; i++) c[i] = s[i] / den;
}

bool make_wavelet(const char *name, WaveletInfo &w) {
    if (!name || std::strncmp(name, "CDF", 3) != 0 || std::strlen(name) != 5) return false;
    w.X = name[3] - '0';
    w.Y = name[4] - '0';
    if (w.X != 2 && w.X != 4 && w.X != 6 && w.X != 8) return false;
    if (w.Y < 0 || w.Y > w.X || (w.Y % 2)) return false;
    interp_stencil(w.X, w.HR, w.hr_lo);
    if (w.Y == 0) {
        w.HD.assign(1, 1.0);
        w.hd_lo = 0;
    } else {
        // HD(i) = delta(i) + sum_j (-1)^j HR(j) h(i-j) / 2, with h the order-Y
        // interpolation stencil with a zero centre tap
        std::vector<double> h;
        int h_lo;
        interp_stencil(w.Y, h, h_lo);
        h[-h_lo] = 0.0;
        int hi_hr = w.hr_lo + (int)w.HR.size() - 1, hi_h = h_lo + (int)h.size() - 1;
        w.hd_lo = w.hr_lo + h_lo;
        int hd_hi = hi_hr + hi_h;
        w.HD.assign(hd_hi - w.hd_lo + 1, 0.0);
        for (int i = w.hd_lo; i <= hd_hi; i++) {
            double v = (i == 0) ? 1.0 : 0.0;
            for (int j = w.hr_lo; j <= hi_hr; j++) {
                if (i - j < h_lo || i - j > hi_h) continue;
                double sgn = (std::abs(j) % 2 == 0) ? 1.0 : -1.0;
                v = v + sgn * w.HR[j - w.hr_lo] * h[i - j - h_lo] / 2.0;
            }
            w.HD[i - w.hd_lo] = v;
        }
    }
    w.gd_lo = w.hr_lo;
    w.GD.resize(w.HR.size());
    for (size_t k = 0; k < w.HR.size(); k++) {
        int i = w.gd_lo + (int)k;
        w.GD[k] = ((std::abs(i) % 2 == 0) ? 1.0 : -1.0) * w.HR[k];
    }
    w.gr_lo = w.hd_lo;
    w.GR.resize(w.HD.size());
    for (size_t k = 0; k < w.HD.size(); k++) {
        int i = w.gr_lo + (int)k;
        w.GR[k] = ((std::abs(i) % 2 == 0) ? 1.0 : -1.0) * w.HD[k];
    }
    w.lifted = (w.Y != 0);
    w.order_predictor = w.X;
    int hd_hi = w.hd_lo + (int)w.HD.size() - 1;
    w.g_min = std::max({std::abs(w.hd_lo), hd_hi, std::abs(w.hr_lo), w.X - 1});
    return true;
}

// ---------------------------------------------------------------------------
// relation table: for each of the 56 relations the side of the neighbour in
// x,y,z (-1,0,+1) and, for the directions along the shared face/edge, which
// half of it a finer neighbour covers (-1 lower, +1 upper). Derived from the
// membership lists of get_indices_of_ghost_patch (LIB/TREE/neighborhood.f90:
// 214-289) and the numbering of find_neighbor (find_neighbors.f90:1-16).
// ---------------------------------------------------------------------------
struct RelInfo {
    int side[3];
    int half[3];
};

struct RelTable {
    RelInfo t[57];
    RelTable();
};

// built once (a function-local static: thread-safe initialisation)
static const RelInfo *rel_table() {
    static const RelTable table;
    return table.t;
}

RelTable::RelTable() {
    auto in = [](int r, std::initializer_list<int> l) {
        for (int v : l) if (v == r) return true;
        return false;
    };
    for (int r = 1; r <= 56; r++) {
        RelInfo &x = t[r];
        std::memset(&x, 0, sizeof(x));
        if (in(r, {1, 2, 3, 4, 25, 26, 29, 30, 33, 34, 37, 38, 49, 51, 53, 55})) x.side[0] = -1;
        if (in(r, {5, 6, 7, 8, 27, 28, 31, 32, 35, 36, 39, 40, 50, 52, 54, 56})) x.side[0] = +1;
        if (in(r, {9, 10, 11, 12, 25, 26, 27, 28, 41, 42, 45, 46, 49, 50, 53, 54})) x.side[1] = -1;
        if (in(r, {13, 14, 15, 16, 29, 30, 31, 32, 43, 44, 47, 48, 51, 52, 55, 56})) x.side[1] = +1;
        if (in(r, {17, 18, 19, 20, 33, 34, 35, 36, 41, 42, 43, 44, 49, 50, 51, 52})) x.side[2] = -1;
        if (in(r, {21, 22, 23, 24, 37, 38, 39, 40, 45, 46, 47, 48, 53, 54, 55, 56})) x.side[2] = +1;
        if (in(r, {10, 12, 14, 16, 18, 20, 22, 24, 42, 44, 46, 48})) x.half[0] = +1;
        if (in(r, {9, 11, 13, 15, 17, 19, 21, 23, 41, 43, 45, 47})) x.half[0] = -1;
        if (in(r, {2, 4, 6, 8, 19, 20, 23, 24, 34, 36, 38, 40})) x.half[1] = +1;
        if (in(r, {1, 3, 5, 7, 17, 18, 21, 22, 33, 35, 37, 39})) x.half[1] = -1;
        if (in(r, {3, 4, 7, 8, 11, 12, 15, 16, 26, 28, 30, 32})) x.half[2] = +1;
        if (in(r, {1, 2, 5, 6, 9, 10, 13, 14, 25, 27, 29, 31})) x.half[2] = -1;
    }
}

// relation id (1..56) of a direction d[3] and, for finer/coarser neighbours,
// the part index k (0..3) along the free directions (find_neighbors.f90:54-104)
static int relation_of_scan(const int d[3], int part, int dim);

// memoised per (dim, direction, part); the table is built once, thread-safe
struct RelMemo {
    int v[2][27][4];
    RelMemo() {
        for (int dm = 2; dm <= 3; dm++)
            for (int k = 0; k < 27; k++)
                for (int p = 0; p < 4; p++) {
                    const int dd[3] = {k % 3 - 1, (k / 3) % 3 - 1, k / 9 - 1};
                    v[dm - 2][k][p] = relation_of_scan(dd, p, dm);
                }
    }
};

static int relation_of(const int d[3], int part, int dim) {
    static const RelMemo memo;
    const int k = (d[0] + 1) + 3 * (d[1] + 1) + 9 * ((dim == 3 ? d[2] : 0) + 1);
    return memo.v[dim - 2][k][part & 3];
}

static int relation_of_scan(const int d[3], int part, int dim) {
    const RelInfo *t = rel_table();
    // part bit i belongs to the i-th free direction in x,y,z order
    int free_rank[3] = {-1, -1, -1}, nfree = 0;
    for (int i = 0; i < dim; i++) if (d[i] == 0) free_rank[i] = nfree++;
    for (int r = 1; r <= 56; r++) {
        bool ok = true;
        for (int i = 0; i < 3 && ok; i++) {
            int s = i < dim ? d[i] : 0;
            if (i >= dim) {
                // 2-D: relations are the z-lower variants
                if (t[r].side[2] != 0) ok = false;
                if (t[r].half[2] == +1) ok = false;
                continue;
            }
            if (t[r].side[i] != s) ok = false;
            if (s == 0) {
                int want = ((part >> free_rank[i]) & 1) ? +1 : -1;
                if (t[r].half[i] != want) ok = false;
            }
        }
        if (ok) return r;
    }
    return -1;
}

static int inverse_relation_scan(int r);

struct InvMemo {
    int v[169];
    InvMemo() {
        for (int r = 1; r <= 168; r++) v[r] = inverse_relation_scan(r);
    }
};

static int inverse_relation(int r) {
    static const InvMemo memo;
    return memo.v[r];
}

static int inverse_relation_scan(int r) {
    const RelInfo *t = rel_table();
    int base = (r - 1) % 56 + 1, range = (r - 1) / 56;
    int inv = -1;
    for (int q = 1; q <= 56; q++) {
        bool ok = true;
        for (int i = 0; i < 3; i++)
            if (t[q].side[i] != -t[base].side[i] || t[q].half[i] != t[base].half[i]) ok = false;
        if (ok) { inv = q; break; }
    }
    int inv_range = range == 0 ? 0 : (range == 1 ? 2 : 1);
    return inv + 56 * inv_range;
}

// ---------------------------------------------------------------------------
// forest
// ---------------------------------------------------------------------------
static inline uint64_t key_of(int lv, int x, int y, int z) {
    return (uint64_t(lv) << 60) | (uint64_t(x) << 40) | (uint64_t(y) << 20) | uint64_t(z);
}

void Forest::set(int nblk, const int *lv, const int *co) {
    level.assign(lv, lv + nblk);
    coords.assign(co, co + 3 * nblk);
    if (dim == 2)
        for (int b = 0; b < nblk; b++) coords[3 * b + 2] = 0;
}

bool Forest::insert_(uint64_t k, int b) {
    for (uint64_t h = (k * 0x9E3779B97F4A7C15ull) >> 20 & mask_;; h = (h + 1) & mask_) {
        if (vals_[h] < 0) {
            keys_[h] = k;
            vals_[h] = b;
            return true;
        }
        if (keys_[h] == k) return false;
    }
}

int Forest::find(int lv, int x, int y, int z) const {
    if (keys_.empty()) return -1;
    const uint64_t k = key_of(lv, x, y, z);
    for (uint64_t h = (k * 0x9E3779B97F4A7C15ull) >> 20 & mask_;; h = (h + 1) & mask_) {
        if (vals_[h] < 0) return -1;
        if (keys_[h] == k) return vals_[h];
    }
}

uint64_t Forest::treecode(int b) const {
    uint64_t tc = 0;
    const int lv = level[b];
    for (int l = 0; l < lv; l++) {
        int sh = lv - 1 - l;
        int bx = (coords[3 * b] >> sh) & 1, by = (coords[3 * b + 1] >> sh) & 1, bz = (coords[3 * b + 2] >> sh) & 1;
        uint64_t digit = uint64_t(2 * bx + by + (dim == 3 ? 4 * bz : 0));
        tc = (tc << dim) | digit;
    }
    return tc;
}

bool Forest::update_neighbors(std::string &err, bool overlapping) {
    const int n = size();
    size_t cap = 16;
    while (cap < size_t(n) * 2 + 16) cap <<= 1;
    keys_.assign(cap, 0);
    vals_.assign(cap, -1);
    mask_ = cap - 1;
    for (int b = 0; b < n; b++) {
        int lv = level[b];
        if (lv < 0 || lv > 20) { err = "block level out of range"; return false; }
        for (int d = 0; d < dim; d++)
            if (coords[3 * b + d] < 0 || coords[3 * b + d] >= (1 << lv)) { err = "block coordinate out of range"; return false; }
        if (!insert_(key_of(lv, coords[3 * b], coords[3 * b + 1], coords[3 * b + 2]), b)) {
            err = "duplicate block";
            return false;
        }
    }
    nbr.assign(size_t(n) * kNumRelations, -1);
    // the blocks are independent (each writes its own row); the first
    // failing block in block order gives the error message
    auto one = [&](int b, std::string &e) -> bool {
        const int lv = level[b];
        const int *c = &coords[3 * b];
        int *nb = &nbr[size_t(b) * kNumRelations];
        const int N = 1 << lv;
        for (int dz = (dim == 3 ? -1 : 0); dz <= (dim == 3 ? 1 : 0); dz++)
            for (int dy = -1; dy <= 1; dy++)
                for (int dx = -1; dx <= 1; dx++) {
                    if (!dx && !dy && !dz) continue;
                    const int d[3] = {dx, dy, dz};
                    int nfree = 0;
                    for (int i = 0; i < dim; i++) nfree += (d[i] == 0);
                    const int nparts = 1 << nfree;
                    const int rel0 = relation_of(d, 0, dim);
                    if (lv == 0) {
                        nb[rel0 - 1] = b;
                        if (!overlapping) continue;
                    }
                    int a[3];
                    for (int i = 0; i < 3; i++) a[i] = i < dim ? (c[i] + d[i]) & (N - 1) : 0;   // periodic, N a power of two
                    if (lv > 0) {
                        const int s = find(lv, a[0], a[1], a[2]);
                        if (s >= 0) {
                            nb[rel0 - 1] = s;
                            if (!overlapping) continue;
                        }
                    }
                    if (overlapping) {
                        // every finer part up to the first missing one, then
                        // the coarser block
                        if (lv < Jmax)
                            for (int p = 0; p < nparts; p++) {
                                int fc[3];
                                int fr = 0;
                                for (int i = 0; i < 3; i++) {
                                    if (i >= dim) { fc[i] = 0; continue; }
                                    int bit;
                                    if (d[i] == 0) bit = (p >> fr++) & 1;
                                    else bit = d[i] > 0 ? 1 : 0;
                                    const int v = 2 * c[i] + bit + d[i];
                                    fc[i] = v & (2 * N - 1);
                                }
                                const int fb = find(lv + 1, fc[0], fc[1], fc[2]);
                                if (fb < 0) break;
                                nb[relation_of(d, p, dim) - 1 + 112] = fb;
                            }
                        if (lv <= Jmin) continue;
                        int part = 0, fr = 0;
                        bool touches = true;
                        for (int i = 0; i < dim; i++) {
                            const int bit = c[i] & 1;
                            if (d[i] == 0) part |= bit << fr++;
                            else if ((d[i] > 0) != (bit == 1)) touches = false;
                        }
                        if (!touches) continue;
                        const int cb = find(lv - 1, a[0] >> 1, a[1] >> 1, a[2] >> 1);
                        if (cb >= 0) nb[relation_of(d, part, dim) - 1 + 56] = cb;
                        continue;
                    }
                    // finer neighbours: all parts must exist
                    bool all = lv < Jmax;
                    if (all) {
                        for (int p = 0; p < nparts; p++) {
                            int fc[3];
                            int fr = 0;
                            for (int i = 0; i < 3; i++) {
                                if (i >= dim) { fc[i] = 0; continue; }
                                int bit;
                                if (d[i] == 0) bit = (p >> fr++) & 1;
                                else bit = d[i] > 0 ? 1 : 0;
                                int v = 2 * c[i] + bit + d[i];
                                fc[i] = v & (2 * N - 1);
                            }
                            int fb = find(lv + 1, fc[0], fc[1], fc[2]);
                            if (fb < 0) { all = false; break; }
                            nb[relation_of(d, p, dim) - 1 + 112] = fb;
                        }
                    }
                    if (all) continue;
                    // coarser neighbour: only if this block touches the parent's
                    // boundary in direction d (find_neighbors.f90:99-104, 178-192)
                    if (lv <= Jmin) continue;
                    int part = 0, fr = 0;
                    bool touches = true;
                    for (int i = 0; i < dim; i++) {
                        int bit = c[i] & 1;
                        if (d[i] == 0) part |= bit << fr++;
                        else if ((d[i] > 0) != (bit == 1)) touches = false;
                    }
                    if (!touches) continue;
                    int pc[3] = {a[0] >> 1, a[1] >> 1, a[2] >> 1};
                    int cb = find(lv - 1, pc[0], pc[1], pc[2]);
                    if (cb >= 0) nb[relation_of(d, part, dim) - 1 + 56] = cb;
                }
        // every face needs a neighbour on a periodic domain
        for (int f = 0; f < 2 * dim; f++) {
            int d[3] = {0, 0, 0};
            d[f / 2] = (f % 2) ? 1 : -1;
            bool found = false;
            for (int p = 0; p < (dim == 3 ? 4 : 2) && !found; p++) {
                int r = relation_of(d, p, dim);
                if (nb[r - 1] >= 0 || nb[r - 1 + 56] >= 0 || nb[r - 1 + 112] >= 0) found = true;
            }
            if (!found) { e = "block without a face neighbour (grid not complete or not graded)"; return false; }
        }
        return true;
    };
    const int nch = host_threads();
    std::vector<int> bad(nch, n);
    std::vector<std::string> msg(nch);
    par_chunks(n, nch, [&](int ch, int lo, int hi) {
        for (int b = lo; b < hi; b++)
            if (!one(b, msg[ch])) {
                bad[ch] = b;
                return;
            }
    }, 4096);
    for (int ch = 0; ch < nch; ch++)
        if (bad[ch] < n) {
            err = msg[ch];
            return false;
        }
    return true;
}

bool Forest::graded() const {
    for (int b = 0; b < size(); b++)
        for (int r = 0; r < kNumRelations; r++) {
            int n = nbr[size_t(b) * kNumRelations + r];
            if (n >= 0 && std::abs(level[n] - level[b]) > 1) return false;
        }
    return true;
}

// ---------------------------------------------------------------------------
// patch boxes (1-based, as in the reference)
// ---------------------------------------------------------------------------
// get_indices_of_ghost_patch (neighborhood.f90:158-327): receiver box
static void recv_box(const Geometry &geo, int relation, int gminus, int gplus, int lvl_diff, int idx[2][3]) {
    const RelInfo &t = rel_table()[(relation - 1) % 56 + 1];
    const int g = geo.g;
    for (int d = 0; d < 3; d++) { idx[0][d] = idx[1][d] = 1; }
    for (int d = 0; d < geo.dim; d++) {
        const int Bs = geo.Bs[d];
        int lo = g + 1, hi = g + Bs;
        if (t.side[d] == -1) { lo = g - gminus + 1; hi = g; }
        if (t.side[d] == +1) { lo = Bs + g + 1; hi = Bs + g + gplus; }
        if (t.half[d] == +1) {
            if (lvl_diff == +1) lo = g - gminus + 1;
            else if (lvl_diff == -1) lo = g + Bs / 2 + 1;
            hi = Bs + g;
        }
        if (t.half[d] == -1) {
            lo = g + 1;
            if (lvl_diff == +1) hi = Bs + g + gplus;
            else if (lvl_diff == -1) hi = g + Bs / 2;
        }
        idx[0][d] = lo;
        idx[1][d] = hi;
    }
}

// get_indices_of_modify_patch (neighborhood.f90:23-126)
static void modify_box(const Geometry &geo, int relation, const int Ns, const int Ne, int gm, int gp, int lvl_diff,
                       int idx[2][3]) {
    const RelInfo &t = rel_table()[(relation - 1) % 56 + 1];
    for (int d = 0; d < 3; d++) { idx[0][d] = idx[1][d] = 1; }
    for (int d = 0; d < geo.dim; d++) {
        const int N = geo.Bs[d] + 2 * geo.g;
        int lo = 1 + gm, hi = N - gp;
        if (t.side[d] == -1) hi = Ns + gm;
        if (t.side[d] == +1) lo = N - Ne - gp + 1;
        if (lvl_diff == -1) {
            if (t.half[d] == +1) lo = N / 2 - Ne + 2;
            if (t.half[d] == -1) hi = N / 2 + Ns;
        }
        idx[0][d] = lo;
        idx[1][d] = hi;
    }
}

// set_send_bounds (LIB/MPI/calc_data_bounds.f90:46-147): sender box and buffer box
static void send_box(const Geometry &geo, int order_predictor, int relation, int lvl_diff, int gminus, int gplus,
                     int b[2][3], int buf[2][3]) {
    const int g = geo.g;
    const int a = order_predictor / 2 - 1;
    for (int d = 0; d < 3; d++) { b[0][d] = b[1][d] = 1; buf[0][d] = buf[1][d] = 1; }
    if (lvl_diff == 0) {
        modify_box(geo, relation, gminus, gplus, g, g, 0, b);
    } else if (lvl_diff == +1) {
        modify_box(geo, relation, 2 * gminus - 1, 2 * gplus - 1, g, g + 1, +1, b);
        for (int d = 0; d < geo.dim; d++) buf[1][d] = (b[1][d] - b[0][d] + 2) / 2;
    } else {
        modify_box(geo, relation, gminus / 2 + 1, (gplus + 1) / 2 + 1, g, g - 1, -1, b);
        for (int d = 0; d < geo.dim; d++) { b[0][d] -= a; b[1][d] += a; }
        for (int d = 0; d < geo.dim; d++) {
            buf[0][d] = (b[0][d] == g + 1 - a || gminus % 2 == 0) ? 1 + 2 * a : 2 + 2 * a;
            buf[1][d] = buf[0][d] + gplus - 1;
            if (b[1][d] - b[0][d] > g + a) buf[1][d] += geo.Bs[d];
        }
    }
}

Patch make_patch(const Geometry &geo, int order_predictor, int relation, int lvl_diff, int gminus, int gplus, int src,
                 int dst) {
    int rb[2][3], sb[2][3], bb[2][3];
    recv_box(geo, inverse_relation(relation), gminus, gplus, -lvl_diff, rb);
    send_box(geo, order_predictor, relation, lvl_diff, gminus, gplus, sb, bb);
    Patch p;
    std::memset(&p, 0, sizeof(p));
    p.src = src;
    p.dst = dst;
    p.op = lvl_diff == 0 ? 0 : (lvl_diff == +1 ? 1 : 2);
    for (int k = 0; k < 3; k++) {
        p.rlo[k] = (int16_t)(rb[0][k] - 1);
        p.rhi[k] = (int16_t)(rb[1][k] - 1);
        p.slo[k] = (int16_t)(sb[0][k] - 1);
        p.shi[k] = (int16_t)(sb[1][k] - 1);
        p.blo[k] = (int16_t)(bb[0][k] - 1);
    }
    return p;
}

void modify_box0(const Geometry &geo, int relation, int Ns, int Ne, int gm, int gp, int lvl_diff, int lo[3], int hi[3]) {
    int idx[2][3];
    modify_box(geo, relation, Ns, Ne, gm, gp, lvl_diff, idx);
    for (int d = 0; d < 3; d++) {
        lo[d] = idx[0][d] - 1;
        hi[d] = idx[1][d] - 1;
    }
}

void ghost_box0(const Geometry &geo, int relation, int gminus, int gplus, int lvl_diff, int lo[3], int hi[3]) {
    int idx[2][3];
    recv_box(geo, relation, gminus, gplus, lvl_diff, idx);
    for (int d = 0; d < 3; d++) {
        lo[d] = idx[0][d] - 1;
        hi[d] = idx[1][d] - 1;
    }
}

int relation_inverse(int relation) { return inverse_relation(relation); }

int relation_id(const int d[3], int part, int dim) { return relation_of(d, part, dim); }

int relation_patch_id(int relation) {
    const int t = (relation - 1) % 56 + 1;
    if (t <= 24) return (t - 1) / 4 + 1;
    if (t <= 48) return (t - 25) / 2 + 1 + 6;
    return (t - 49) + 1 + 6 + 12;
}

void relation_range(int relation, int lvl_diff, int &lo, int &hi) {
    const int pid = relation_patch_id(relation);
    if (pid <= 6) { lo = (pid - 1) * 4 + 1; hi = pid * 4; }
    else if (pid <= 18) { lo = (pid - 7) * 2 + 25; hi = (pid - 6) * 2 + 24; }
    else { lo = (pid - 19) + 49; hi = (pid - 18) + 48; }
    const int off = lvl_diff == +1 ? 56 : lvl_diff == -1 ? 112 : 0;
    lo += off;
    hi += off;
}

bool make_sync_table(const Forest &f, const Geometry &geo, const WaveletInfo &w, int gminus, int gplus, int g_buf,
                     int block_offset, SyncTable &out, std::string &err) {
    const int nstages = w.lifted ? 3 : 2;
    const int unl = w.lifted ? 0 : 1;
    const int shift = geo.g - g_buf;
    int nbuf[3];
    for (int d = 0; d < 3; d++) nbuf[d] = d < geo.dim ? geo.Bs[d] + 2 * g_buf : 1;
    out.max_points = 0;
    out.max_coarse = 0;
    const int n = f.size();
    // the boxes of a patch depend only on (relation, level difference): one
    // template per pair that occurs, checked once
    struct Tmpl {
        Patch p;
        int npts = 0, need = 0;
        const char *bad = nullptr;
    };
    std::vector<Tmpl> tm(3 * kNumRelations);
    std::vector<char> used(3 * kNumRelations, 0);
    for (int s = 0; s < n; s++) {
        const int *nb = &f.nbr[size_t(s) * kNumRelations];
        for (int r = 1; r <= kNumRelations; r++) {
            const int d = nb[r - 1];
            if (d < 0) continue;
            const int lvl_diff = f.level[s] - f.level[d];
            if (lvl_diff < -1 || lvl_diff > 1) { err = "level jump larger than one between neighbours"; return false; }
            used[(lvl_diff + 1) * kNumRelations + r - 1] = 1;
        }
    }
    for (int lvl_diff = -1; lvl_diff <= 1; lvl_diff++)
        for (int r = 1; r <= kNumRelations; r++) {
            if (!used[(lvl_diff + 1) * kNumRelations + r - 1]) continue;
            Tmpl &t = tm[(lvl_diff + 1) * kNumRelations + r - 1];
            int rb[2][3], sb[2][3], bb[2][3];
            recv_box(geo, inverse_relation(r), gminus, gplus, -lvl_diff, rb);
            send_box(geo, w.order_predictor, r, lvl_diff, gminus, gplus, sb, bb);
            Patch &p = t.p;
            std::memset(&p, 0, sizeof(p));
            p.op = lvl_diff == 0 ? 0 : (lvl_diff == +1 ? 1 : 2);
            p.stage = (int16_t)(lvl_diff == 0 ? 1 : lvl_diff == +1 ? 2 - unl : 3 - unl);
            int npts = 1;
            for (int k = 0; k < 3 && !t.bad; k++) {
                const bool active = k < geo.dim;
                const int sh = active ? shift : 0;
                p.rlo[k] = (int16_t)(rb[0][k] - 1 - sh);
                p.rhi[k] = (int16_t)(rb[1][k] - 1 - sh);
                p.slo[k] = (int16_t)(sb[0][k] - 1 - sh);
                p.shi[k] = (int16_t)(sb[1][k] - 1 - sh);
                p.blo[k] = (int16_t)(bb[0][k] - 1);
                npts *= (rb[1][k] - rb[0][k] + 1);
                // bounds of every access in the ghost-width-g_buf buffer
                if (p.rlo[k] < 0 || p.rhi[k] >= nbuf[k] || p.rlo[k] > p.rhi[k]) { t.bad = "receiver box outside buffer"; break; }
                if (p.op == 0) {
                    if (p.slo[k] < 0 || p.slo[k] + (p.rhi[k] - p.rlo[k]) >= nbuf[k]) t.bad = "copy source outside buffer";
                } else if (p.op == 1) {
                    int hi = p.slo[k] + 2 * (p.blo[k] + p.rhi[k] - p.rlo[k]);
                    if (p.slo[k] < 0 || hi >= nbuf[k] || (active && hi > p.shi[k])) t.bad = "restriction source outside buffer";
                } else {
                    int nf = 2 * (p.shi[k] - p.slo[k] + 1) - 1;
                    if (p.slo[k] < 0 || p.shi[k] >= nbuf[k] || p.blo[k] + (p.rhi[k] - p.rlo[k]) >= nf) t.bad = "prediction box outside buffer";
                }
            }
            t.npts = npts;
            if (p.op == 2 && !t.bad) {
                // shared memory of the separable prediction: coarse box, x
                // window (even rows/planes) and x-y window (even planes)
                const int h = w.order_predictor - 1;
                const int cx = p.shi[0] - p.slo[0] + 1, cy = p.shi[1] - p.slo[1] + 1, cz = p.shi[2] - p.slo[2] + 1;
                const int Fy = 2 * cy - 1, Fz = 2 * cz - 1;
                const int ex = p.rhi[0] - p.rlo[0] + 1, ey = p.rhi[1] - p.rlo[1] + 1, ez = p.rhi[2] - p.rlo[2] + 1;
                int yw0 = std::max(0, p.blo[1] - h), yw1 = std::min(Fy - 1, p.blo[1] + ey - 1 + h);
                yw0 += yw0 & 1;
                yw1 -= yw1 & 1;
                int zw0 = std::max(0, p.blo[2] - h), zw1 = std::min(Fz - 1, p.blo[2] + ez - 1 + h);
                zw0 += zw0 & 1;
                zw1 -= zw1 & 1;
                const int wy = (yw1 - yw0) / 2 + 1, wz = (zw1 - zw0) / 2 + 1;
                t.need = cx * cy * cz + ex * wy * wz + ex * ey * wz;
            }
            if (t.bad) { err = t.bad; return false; }
            out.max_points = std::max(out.max_points, npts);
            out.max_coarse = std::max(out.max_coarse, t.need);
        }
    // a stage is a prediction stage iff all its relations predict
    out.nstages = nstages;
    out.stage_begin.assign(nstages + 1, 0);
    out.stage_predict.assign(nstages, 0);
    for (int st = 1; st <= nstages; st++) {
        bool any = false, all = true;
        for (int i = 0; i < 3 * kNumRelations; i++)
            if (used[i] && tm[i].p.stage == st) {
                any = true;
                all = all && tm[i].p.op == 2;
                if (tm[i].p.op == 2) out.stage_predict[st - 1] = 1;
            }
        if (out.stage_predict[st - 1] && !all) { err = "prediction mixed with copies in one stage"; return false; }
        if (!any) out.stage_predict[st - 1] = 0;
    }
    // patches in (stage, sender, relation) order: count per chunk of senders,
    // then every chunk writes its own ranges
    const int nch = host_threads();
    std::vector<int> cnt((size_t)nch * (nstages + 1), 0);
    auto each = [&](int lo, int hi, auto g) {
        for (int s = lo; s < hi; s++) {
            const int *nb = &f.nbr[size_t(s) * kNumRelations];
            for (int r = 1; r <= kNumRelations; r++) {
                const int d = nb[r - 1];
                if (d >= 0) g(s, d, tm[(f.level[s] - f.level[d] + 1) * kNumRelations + r - 1].p);
            }
        }
    };
    par_chunks(n, nch, [&](int ch, int lo, int hi) {
        each(lo, hi, [&](int, int, const Patch &p) { cnt[(size_t)ch * (nstages + 1) + p.stage]++; });
    }, 4096);
    std::vector<size_t> off((size_t)nch * (nstages + 1), 0);
    size_t at = 0;
    for (int st = 1; st <= nstages; st++) {
        out.stage_begin[st - 1] = (int)at;
        for (int ch = 0; ch < nch; ch++) {
            off[(size_t)ch * (nstages + 1) + st] = at;
            at += cnt[(size_t)ch * (nstages + 1) + st];
        }
    }
    out.patches.resize(at);
    par_chunks(n, nch, [&](int ch, int lo, int hi) {
        size_t *o = &off[(size_t)ch * (nstages + 1)];
        each(lo, hi, [&](int s, int d, const Patch &t) {
            Patch &p = out.patches[o[t.stage]++];
            p = t;
            p.src = s + block_offset;
            p.dst = d + block_offset;
        });
    }, 4096);
    out.stage_begin[nstages] = (int)out.patches.size();
    return true;
}

}  // namespace wg
