// capi.cu -- the C ABI of the GB300 hot path (include/wabbit_gb300.h).
//
// A context is one device arena for a fixed block geometry (dim, Bs, g, neq)
// holding up to max_blocks blocks. Blocks belong to trees: independent solves
// with their own grid, physics constants, time and dt. The host keeps each
// tree's grid (Forest) and derives flat ghost-patch tables from it whenever
// the grid changes; the heavy data stays in HBM.
//
// Device buffers per block slot:
//   A    full layout (ghost width g): the state u (hvy_block)
//   B, C thin layout (ghost width g_rhs): RK stage inputs
//   D    thin layout, FP32-pipe precision only: third stage-input buffer
//        (B keeps the double-float copy of u_n through the step)
//   acc  interior only: u_n + dt*sum b_j k_j (the RK accumulator; in the
//        FP32-pipe precision the double-float increment dt*sum b_j k_j)
//   mask interior only, 6 components, only for blocks that carry a mask;
//        the FP32-pipe precision adds a double-float copy (5 components)
#include <algorithm>
#include <cstddef>
#include <chrono>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <map>
#include <memory>
#include <string>
#include <vector>

#include <cuda.h>

#include "../../include/wabbit_gb300.h"
#include "adapt.hpp"
#include "geometry.hpp"
#include "par.hpp"
#include "lifted.hpp"
#include "common.cuh"

namespace wg {

static thread_local std::string g_err;
static thread_local int g_code = 0;   // status of the last fail() on this thread

static int fail(int code, const char *fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    g_err = buf;
    g_code = code;
    return code;
}

// status of a failed get_tree (invalid id, or a context that a timed-out
// device wait left unusable)
static int tree_err() { return g_code ? g_code : WG_EINVAL; }

int cuda_fail(cudaError_t e, const char *what, const char *file, int line) {
    return fail(WG_ECUDA, "%s failed: %s (%s:%d)", what, cudaGetErrorString(e), file, line);
}

template <class T>
struct DevArray {
    T *p = nullptr;
    size_t n = 0, cap = 0;
    ~DevArray() {
        if (p) cudaFree(p);
    }
    cudaError_t upload(const T *h, size_t count, cudaStream_t s) {
        if (count > cap) {
            if (p) cudaFree(p);
            p = nullptr;
            cap = 0;
            cudaError_t e = cudaMalloc(&p, sizeof(T) * (count ? count : 1));
            if (e != cudaSuccess) return e;
            cap = count;
        }
        n = count;
        if (!count || !h) return cudaSuccess;
        return cudaMemcpyAsync(p, h, sizeof(T) * count, cudaMemcpyHostToDevice, s);
    }
};

// Transient device lists of one adaptation: chunks of device memory kept
// between calls (no allocation per list), handed out by a bump pointer and
// reset when the stream is idle.
struct DevScratch {
    struct Chunk {
        char *p;
        size_t cap, used;
    };
    std::vector<Chunk> chunks;
    size_t cur = 0;
    void *alloc(size_t bytes) {
        bytes = std::max<size_t>(256, (bytes + 255) & ~(size_t)255);
        while (cur < chunks.size() && chunks[cur].used + bytes > chunks[cur].cap) cur++;
        if (cur == chunks.size()) {
            const size_t cap = std::max(bytes, (size_t)64 << 20);
            char *p = nullptr;
            if (cudaMalloc(&p, cap) != cudaSuccess) {
                cudaGetLastError();
                return nullptr;
            }
            chunks.push_back({p, cap, 0});
        }
        void *r = chunks[cur].p + chunks[cur].used;
        chunks[cur].used += bytes;
        return r;
    }
    void reset() {
        for (Chunk &c : chunks) c.used = 0;
        cur = 0;
    }
    ~DevScratch() {
        for (Chunk &c : chunks) cudaFree(c.p);
    }
};

// Free arena slots as a bitmap (bit set = free): take() hands out the lowest
// free slot, give() returns one; no sort of the free list per grid change.
struct SlotPool {
    std::vector<uint64_t> bits;
    size_t nfree = 0;
    size_t first = 0;   // every word below this one is empty
    void init(int n) {
        bits.assign(((size_t)n + 63) / 64, 0);
        for (int i = 0; i < n; i++) bits[(size_t)i >> 6] |= 1ull << (i & 63);
        nfree = (size_t)n;
        first = 0;
    }
    size_t size() const { return nfree; }
    void give(int s) {
        bits[(size_t)s >> 6] |= 1ull << (s & 63);
        nfree++;
        first = std::min(first, (size_t)s >> 6);
    }
    int take() {
        if (!nfree) return -1;
        while (!bits[first]) first++;
        const int b = __builtin_ctzll(bits[first]);
        bits[first] &= bits[first] - 1;
        nfree--;
        return (int)(first * 64 + b);
    }
};

// Prediction patches of the stages of a table for one launch per stage,
// sorted within each stage by the shared memory the CTA-per-patch kernel
// needs, largest first (the long CTAs start first); the launch sizes its
// shared memory for the largest and runs as many components per pass as
// keep four CTAs on an SM.
struct PredClasses {
    DevArray<Patch> patches;                 // sorted copy
    std::vector<std::vector<int>> begin;     // per stage: class offsets into patches (n_class+1)
    std::vector<std::vector<int>> need;      // per stage and class: largest need in doubles per component
};

struct SyncPlan {
    SyncTable table;
    DevArray<Patch> d;
    // gather form of the copy / restriction stages (empty: patch kernel)
    DevArray<Patch> order;             // patches in expansion order (copies first per stage)
    DevArray<unsigned> first;          // per patch of order: offset of its first point in its stage
    DevArray<uint2> pairs;             // (receiver, sender) offsets, all stages
    std::vector<unsigned> pair_begin;  // nstages+1 offsets into pairs
    std::vector<unsigned> copy_end;    // per stage: end of its copy entries
    // prediction stages split into classes of similar shared-memory need
    // (patches sorted by need), so that small patches launch small CTAs
    PredClasses pcls;
    // every copy patch is a same-level translation of a full ghost region:
    // the stage kernels may write these ghost nodes themselves (ctx->d_push)
    bool push_ok = false;
};

// The per-step work of several trees of the FP32-pipe precision fused into
// one launch per kernel: their block lists, ghost gather entries and
// prediction patches concatenated (the trees share the block geometry and
// the wavelet, so their syncs have the same stages).
struct BatchPlan {
    std::vector<int> trees;
    int version = -1;
    DevArray<int> all, plain, masked, tree_ids;
    DevArray<int> stage;                // the FP32-pipe stage order: masked blocks first (the longer CTAs)
    int n_all = 0, n_plain = 0, n_masked = 0;
    int nstages = 0;
    std::vector<int> stage_predict;
    DevArray<uint2> pairs;              // per stage: copies of all trees, then the other entries
    std::vector<unsigned> pair_begin, copy_end;
    DevArray<Patch> predict;            // per stage: prediction patches of all trees
    std::vector<int> pred_begin;
    PredClasses pcls;                   // prediction patches by shared-memory class
    int max_coarse = 0;
    bool push = false;                  // every tree's copies are pushed by the stage kernels
};

struct Tree {
    bool live = false;
    wg_config cfg;
    TreeParams tp;
    Forest forest;
    std::vector<int> slots;            // block -> arena slot
    std::vector<int> mask_slot;        // block -> mask slot or -1
    DevArray<int> d_all, d_plain, d_masked;   // slot lists
    DevArray<int> d_stage;                    // masked slots, then the others (FP32-pipe stage launches)
    int n_plain = 0, n_masked = 0;
    std::map<long long, std::unique_ptr<SyncPlan>> sync;   // key: gm, gp, buffer
    std::map<long long, std::unique_ptr<SyncPlan>> spare;  // plans of an earlier grid: device buffers to reuse
    double time = 0.0;
    bool shadow_valid = false;         // double-float copy of u_n in B is current
    std::vector<int> status;           // refinement status the last adaptation left (0 or 9 per block)
    wg_geometry geom{};                // penalisation geometry the masks are drawn from
    bool has_geom = false;             // false: masks are set by the caller (wg_set_mask*)
};

}  // namespace wg

using namespace wg;

struct wg_ctx {
    wg_config cfg;
    Geometry geo;
    WaveletInfo wav;
    int max_blocks = 0;
    BufGeo gA, gT;                      // full and thin layouts
    long long nint = 0;                 // interior points per block
    double *A = nullptr, *B = nullptr, *C = nullptr, *D = nullptr, *E = nullptr, *acc = nullptr;
    double *mask = nullptr;
    float2 *mask_df = nullptr;
    int *d_push = nullptr;              // per slot 27 same-level receivers (FP32-pipe precision)
    std::vector<int> h_push;
    CUtensorMap tm[4];                  // TMA maps over B, C, D, E (3-D FP32-pipe precision): slab boxes
    CUtensorMap tp[4];                  // ... one-plane boxes (march form)
    CUtensorMap tm2[4], tm8[4];         // ... slab boxes of 2 and 8 interior planes (tile2, tile8 forms)
    bool have_tm = false, have_march = false, have_slabs28 = false;
    int stage_form = WG_FORM_AUTO;      // requested form of the FP32-pipe stage kernel
    int tuned[4] = {0, 0, 0, 0};        // the autotuner's choice per RK stage (0: not tuned yet)
    // step profile (wg_step_profile): events recorded between the kernel
    // groups of an RK4 step while prof_on is set
    cudaEvent_t prof_ev[10] = {};
    bool prof_on = false;
    // wg_rk4_stream: stage 4 of the tree's step also writes u_n+1 into this
    // compact array (positions by block slot in d_pos), instead of a gather
    double *s4_out = nullptr;
    int s4_keep = 1;                    // stage-4 mode of rk4_enqueue_df (launch_acm_stage_df keep_state)
    const double *s4_next = nullptr;    // stage 4 (keep 3): the next step's compact input
    const double *s4_usrc = nullptr;    // dt and stage 4 read u_n from this compact input (positions d_pos), or null
    cudaEvent_t s4_wait = nullptr;      // stage 4 waits for it (the copy of s4_next), or null
    DevArray<int> d_pos;
    // set when a bounded device wait gave up (WG_ETIMEOUT): a bulk copy may
    // still have been landing in shared memory, so nothing the context holds
    // is trusted any more and every call but wg_ctx_destroy fails
    bool dead = false;
    int *d_err = nullptr;               // device error flag (a kernel's wait ran out), then the three
                                        // work counters of the fused ghost sync and the finished-CTA
                                        // counter of the dt reduction (all zero between launches)
    int mask_cap = 0;
    std::vector<int> mask_free;
    BlockDesc *d_desc = nullptr;
    std::vector<BlockDesc> h_desc;
    TreeParams *d_tp = nullptr;
    TreeClock *d_clk = nullptr;
    unsigned long long *d_usq = nullptr;   // per block slot: max |u|^2 the last RK stage stored (TreeClock::usq_ready)
    int max_trees = 64;
    std::vector<Tree> trees;
    SlotPool free_slots;
    DevScratch scratch;                 // transient lists of the lifted adaptation
    cudaStream_t stream = nullptr;
    int variant_fast = 1;               // 1: FMA stencil, 0: strict reference arithmetic
    int precision = WG_RHS_FP64;        // WG_RHS_FP32: double-float stencils on the FP32 units
    DevArray<int> d_tree_ids;
    double *T = nullptr;                // hvy_tmp arena of the lifted adaptation (slot-indexed like A)
    bool adapt_profile = false;         // time the phases of the lifted adaptation
    double adapt_ms[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    double *staging = nullptr;          // compact interior staging buffer
    cudaStream_t copy_stream = nullptr; // host<->device copies of the interior transfers
    std::vector<cudaEvent_t> copy_ev;   // one per chunk
    cudaStream_t d2h_stream = nullptr;  // results of wg_rk4_stream
    double *stream_buf = nullptr;       // wg_rk4_stream: two input and two output staging buffers
    size_t stream_buf_bytes = 0;
    cudaEvent_t io_ev[10] = {};         // wg_rk4_stream: h2d done (x3), d2h done (x2), gathered (x2), consumed (x3)
    size_t staging_bytes = 0;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t graph_exec = nullptr;
    std::vector<int> graph_trees;
    int graph_version = -1;
    BatchPlan batch;
    int grid_version = 0;
};

namespace {

// a tree's clock at time t: no dt yet, the running dt minimum at its start
// value, no anchoring constant
TreeClock fresh_clock(double t) {
    TreeClock c;
    std::memset(&c, 0, sizeof(c));
    c.time = t;
    c.dt_min_bits = kDtStartBits;
    return c;
}

// the tree's state changed outside an RK step: neither the double-float
// copy of u_n nor the per-block maxima of |u|^2 the last RK stage recorded
// (TreeClock::usq_ready) describe it any longer
static int state_changed(wg_ctx *ctx, Tree *t, int tree) {
    t->shadow_valid = false;
    WG_CUDA_OK(cudaMemsetAsync(&ctx->d_clk[tree].usq_ready, 0, sizeof(int), ctx->stream));
    return WG_OK;
}

int check_cfg(const wg_config *c) {
    if (!c) return fail(WG_EINVAL, "null config");
    if (c->dim != 2 && c->dim != 3) return fail(WG_EINVAL, "dim must be 2 or 3");
    if (c->neq != c->dim + 1) return fail(WG_ENOTSUP, "neq must be dim+1 (ACM: velocity + pressure)");
    for (int d = 0; d < c->dim; d++)
        if (c->Bs[d] < 4 || (c->Bs[d] % 2) || c->Bs[d] > 64) return fail(WG_EINVAL, "Bs must be even, 4..64");
    if (c->g_rhs < 2 || c->g < c->g_rhs) return fail(WG_EINVAL, "need g >= g_rhs >= 2 for FD_4th_central");
    WaveletInfo w;
    if (!make_wavelet(c->wavelet, w)) return fail(WG_EINVAL, "unknown wavelet '%s'", c->wavelet);
    if (c->g < w.g_min) return fail(WG_EINVAL, "%s needs g >= %d", c->wavelet, w.g_min);
    // a restriction takes 2g-1 fine points next to the interface; if that
    // exceeds the block, it would read ghost nodes of the same sync stage
    for (int d = 0; d < c->dim; d++)
        if (2 * c->g - 1 > c->Bs[d]) return fail(WG_EINVAL, "Bs=%d too small for g=%d (need Bs >= 2g-1)", c->Bs[d], c->g);
    if (c->Jmin < 0 || c->Jmax < c->Jmin || c->Jmax > 18) return fail(WG_EINVAL, "bad Jmin/Jmax");
    if (c->rhs_precision != WG_RHS_FP64 && c->rhs_precision != WG_RHS_FP32)
        return fail(WG_EINVAL, "rhs_precision must be WG_RHS_FP64 or WG_RHS_FP32");
    if (c->rhs_precision == WG_RHS_FP32 && c->skew_symmetry)
        return fail(WG_ENOTSUP, "the FP32 stencil path implements the convective form only (skew_symmetry=0)");
    return WG_OK;
}

// double -> (hi, lo) float pair
void split_df(double v, float out[2]) {
    const float h = (float)v;
    out[0] = h;
    out[1] = (float)(v - (double)h);
}

TreeParams make_params(const wg_config &c) {
    TreeParams p;
    std::memset(&p, 0, sizeof(p));
    p.c0 = c.c0;
    p.nu = c.nu;
    p.gamma_p = c.gamma_p;
    p.C_eta = c.C_eta;
    p.C_eta_inv = 1.0 / c.C_eta;
    p.C_sponge = c.C_sponge;
    p.C_sponge_inv = 1.0 / c.C_sponge;
    for (int i = 0; i < 3; i++) p.u_mean_set[i] = c.u_mean_set[i];
    p.CFL = c.CFL;
    p.CFL_nu = c.CFL_nu;
    p.CFL_eta = c.CFL_eta;
    p.dt_fixed = c.dt_fixed;
    p.dt_max = c.dt_max;
    p.time_max = c.time_max;
    p.write_time = c.write_time;
    p.tsave_stats = c.tsave_stats;
    p.penalization = c.penalization;
    p.use_sponge = c.use_sponge;
    p.skew = c.skew_symmetry;
    split_df(c.c0 * c.c0, p.f_c0sq);
    split_df(c.gamma_p, p.f_gamma);
    for (int i = 0; i < 3; i++) split_df(c.u_mean_set[i], p.f_umean[i]);
    return p;
}

Tree *get_tree(wg_ctx *ctx, int t) {
    if (ctx && ctx->dead) {
        fail(WG_ETIMEOUT, "the context is unusable after a timed-out device wait; destroy it");
        return nullptr;
    }
    if (!ctx || t < 0 || t >= (int)ctx->trees.size() || !ctx->trees[t].live) {
        fail(WG_EINVAL, "invalid tree id %d", t);
        return nullptr;
    }
    return &ctx->trees[t];
}

long long sync_key(int gm, int gp, int thin) { return ((long long)gm << 20) | ((long long)gp << 4) | thin; }

// shared memory (doubles per component) of a prediction patch in the
// CTA-per-patch kernel: coarse box, x window and x-y window
static int pred_need(const Patch &p, int order_predictor) {
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

int build_pred_classes(wg_ctx *ctx, const std::vector<Patch> &pt, const std::vector<int> &stage_begin,
                       const std::vector<int> &stage_predict, PredClasses &pc) {
    const int ns = (int)stage_predict.size();
    std::vector<Patch> sorted;
    pc.begin.assign(ns, {});
    pc.need.assign(ns, {});
    for (int st = 0; st < ns; st++) {
        if (!stage_predict[st]) continue;
        std::vector<std::pair<int, int>> byneed;
        for (int i = stage_begin[st]; i < stage_begin[st + 1]; i++)
            byneed.push_back({-pred_need(pt[i], ctx->wav.order_predictor), i});
        std::stable_sort(byneed.begin(), byneed.end());
        const int base = (int)sorted.size();
        for (const auto &e : byneed) sorted.push_back(pt[e.second]);
        pc.begin[st] = {base, base + (int)byneed.size()};
        pc.need[st] = {byneed.empty() ? 0 : -byneed.front().first};
    }
    WG_CUDA_OK(pc.patches.upload(sorted.data(), sorted.size(), ctx->stream));
    return WG_OK;
}

int run_pred_classes(wg_ctx *ctx, const PredClasses &pc, int st, double *buf, const BufGeo &geo) {
    const std::vector<int> &b = pc.begin[st];
    for (size_t k = 0; k + 1 < b.size(); k++)
        WG_CUDA_OK(launch_predict_df(pc.patches.p + b[k], b[k + 1] - b[k], pc.need[st][k], buf, geo, ctx->geo.nc,
                                     ctx->wav.order_predictor, ctx->d_desc, ctx->d_clk, ctx->stream, 4));
    return WG_OK;
}

// Check that every copy patch of a thin per-step plan is a same-level
// translation of a full ghost region (the form push_ghosts writes) and, if
// so, record per sender slot the receiver slot of each direction.
int build_push(wg_ctx *ctx, Tree &t, SyncPlan &sp, const BufGeo &geo) {
    const int gb = geo.gb, dim = ctx->cfg.dim;
    const int *Bs = ctx->cfg.Bs;
    std::vector<int> row_of(ctx->max_blocks, -1);
    for (size_t i = 0; i < t.slots.size(); i++) row_of[t.slots[i]] = (int)i;
    std::vector<int> rows(t.slots.size() * 27, -1);
    bool ok = true;
    for (const Patch &p : sp.table.patches) {
        if (p.op != 0) continue;
        int D[3] = {0, 0, 0};
        for (int a = 0; a < 3 && ok; a++) {
            const int r0 = p.rlo[a], r1 = p.rhi[a], s0 = p.slo[a], s1 = p.shi[a];
            if (a >= dim) {
                ok = r0 == 0 && r1 == 0 && s0 == 0 && s1 == 0;
                continue;
            }
            const int B = Bs[a];
            if (r0 == gb && r1 == gb + B - 1 && s0 == gb && s1 == gb + B - 1) D[a] = 0;
            else if (r0 == gb + B && r1 == gb + B + gb - 1 && s0 == gb && s1 == 2 * gb - 1) D[a] = -1;
            else if (r0 == 0 && r1 == gb - 1 && s0 == B && s1 == gb + B - 1) D[a] = 1;
            else ok = false;
        }
        if (!ok) break;
        const int r = p.src >= 0 && p.src < ctx->max_blocks ? row_of[p.src] : -1;
        const int k = (D[2] + 1) * 9 + (D[1] + 1) * 3 + (D[0] + 1);
        if (r < 0 || k == 13 || rows[(size_t)r * 27 + k] != -1) {
            ok = false;
            break;
        }
        rows[(size_t)r * 27 + k] = p.dst;
    }
    sp.push_ok = ok;
    if (!ok || t.slots.empty()) return WG_OK;
    int lo = ctx->max_blocks, hi = -1;
    for (size_t i = 0; i < t.slots.size(); i++) {
        std::memcpy(&ctx->h_push[(size_t)t.slots[i] * 27], &rows[i * 27], sizeof(int) * 27);
        lo = std::min(lo, t.slots[i]);
        hi = std::max(hi, t.slots[i]);
    }
    WG_CUDA_OK(cudaMemcpyAsync(ctx->d_push + (size_t)lo * 27, &ctx->h_push[(size_t)lo * 27],
                               sizeof(int) * 27 * (size_t)(hi - lo + 1), cudaMemcpyHostToDevice, ctx->stream));
    WG_CUDA_OK(cudaStreamSynchronize(ctx->stream));
    return WG_OK;
}

// the tree's sync plans are stale (its grid changed): their device buffers
// serve the plans of the new grid, so a grid change allocates and frees no
// device memory for them (the stream is idle at every caller)
void drop_sync(Tree &t) {
    for (auto &kv : t.sync) {
        SyncPlan &p = *kv.second;
        p.pair_begin.clear();
        p.copy_end.clear();
        p.push_ok = false;
        t.spare[kv.first] = std::move(kv.second);
    }
    t.sync.clear();
}

int get_sync(wg_ctx *ctx, Tree &t, int gm, int gp, bool thin, SyncPlan **out) {
    const long long key = sync_key(gm, gp, thin ? 1 : 0);
    auto it = t.sync.find(key);
    if (it == t.sync.end()) {
        std::unique_ptr<SyncPlan> sp;
        auto old = t.spare.find(key);
        if (old != t.spare.end()) {
            sp = std::move(old->second);
            t.spare.erase(old);
        } else {
            sp.reset(new SyncPlan());
        }
        std::string err;
        if (!make_sync_table(t.forest, ctx->geo, ctx->wav, gm, gp, thin ? ctx->gT.gb : ctx->gA.gb, 0, sp->table, err))
            return fail(WG_EGRID, "sync table: %s", err.c_str());
        for (auto &p : sp->table.patches) {
            p.src = t.slots[p.src];
            p.dst = t.slots[p.dst];
        }
        WG_CUDA_OK(sp->d.upload(sp->table.patches.data(), sp->table.patches.size(), ctx->stream));
        // the per-step syncs (g_rhs layers) get the gather form when every
        // element offset of the buffer fits 32 bits
        const BufGeo geo = thin ? ctx->gT : ctx->gA;
        const unsigned long long elems = (unsigned long long)ctx->max_blocks * ctx->geo.nc * geo.npts();
        if (gm == ctx->cfg.g_rhs && gp == ctx->cfg.g_rhs && elems < (1ull << 32)) {
            const SyncTable &tb = sp->table;
            const auto &pt = tb.patches;
            std::vector<Patch> order;
            std::vector<unsigned> first;
            std::vector<int> order_begin(tb.nstages + 1, 0);
            unsigned long long run = 0;
            sp->pair_begin.assign(tb.nstages + 1, 0);
            sp->copy_end.assign(tb.nstages, 0);
            for (int st = 0; st < tb.nstages; st++) {
                sp->pair_begin[st] = (unsigned)run;
                order_begin[st] = (int)order.size();
                sp->copy_end[st] = (unsigned)run;
                if (tb.stage_predict[st]) continue;
                for (int pass = 0; pass < 2; pass++) {
                    for (int i = tb.stage_begin[st]; i < tb.stage_begin[st + 1]; i++) {
                        if ((pt[i].op == 0) != (pass == 0)) continue;
                        order.push_back(pt[i]);
                        first.push_back((unsigned)(run - sp->pair_begin[st]));
                        run += (unsigned long long)(pt[i].rhi[0] - pt[i].rlo[0] + 1) *
                               (pt[i].rhi[1] - pt[i].rlo[1] + 1) * (pt[i].rhi[2] - pt[i].rlo[2] + 1);
                    }
                    if (pass == 0) sp->copy_end[st] = (unsigned)run;
                }
            }
            order_begin[tb.nstages] = (int)order.size();
            sp->pair_begin[tb.nstages] = (unsigned)run;
            {
                int st2 = build_pred_classes(ctx, tb.patches, tb.stage_begin, tb.stage_predict, sp->pcls);
                if (st2) return st2;
            }
            if (run < (1ull << 32)) {
                WG_CUDA_OK(sp->order.upload(order.data(), order.size(), ctx->stream));
                WG_CUDA_OK(sp->first.upload(first.data(), first.size(), ctx->stream));
                WG_CUDA_OK(sp->pairs.upload(nullptr, run, ctx->stream));
                for (int st = 0; st < tb.nstages; st++) {
                    const int b = order_begin[st], e = order_begin[st + 1];
                    if (e == b) continue;
                    const unsigned n = sp->pair_begin[st + 1] - sp->pair_begin[st];
                    WG_CUDA_OK(launch_expand(sp->order.p + b, sp->first.p + b, e - b, n, geo, ctx->geo.nc,
                                             sp->pairs.p + sp->pair_begin[st], ctx->stream));
                }
                WG_CUDA_OK(cudaStreamSynchronize(ctx->stream));
                if (thin && ctx->d_push && gm == geo.gb) {
                    int st2 = build_push(ctx, t, *sp, geo);
                    if (st2) return st2;
                }
            } else {
                sp->pair_begin.clear();
            }
        }
        it = t.sync.emplace(key, std::move(sp)).first;
    }
    *out = it->second.get();
    return WG_OK;
}

// The shape the fused sync launch covers: gather stages of which at most one
// has entries left once the pushed copies are skipped (*gst, or -1), then a
// single prediction stage, the last (*pst). False: run the stages one by one.
static bool fused_shape(const std::vector<int> &stage_predict, const std::vector<unsigned> &pair_begin,
                        const std::vector<unsigned> &copy_end, bool skip_copies, int *gst, int *pst) {
    const int ns = (int)stage_predict.size();
    if (ns == 0 || (int)pair_begin.size() != ns + 1 || !stage_predict[ns - 1]) return false;
    *gst = -1;
    *pst = ns - 1;
    for (int s = 0; s + 1 < ns; s++) {
        if (stage_predict[s]) return false;
        const unsigned from = skip_copies ? copy_end[s] : pair_begin[s];
        if (pair_begin[s + 1] == from) continue;
        if (*gst >= 0) return false;
        *gst = s;
    }
    return true;
}

// counters of the fused sync (after the error flag)
static unsigned *fused_ctr(wg_ctx *ctx) { return reinterpret_cast<unsigned *>(ctx->d_err + 1); }

// finished-CTA counter of the one-launch dt reduction
static unsigned *dt_done(wg_ctx *ctx) { return reinterpret_cast<unsigned *>(ctx->d_err + 4); }

// skip_copies: the same-level copies were written by the kernel that wrote
// buf's interiors (push); only restrictions and predictions remain
int run_sync(wg_ctx *ctx, Tree &t, double *buf, bool thin, int gm, int gp, bool df = false, bool skip_copies = false) {
    SyncPlan *sp;
    int st = get_sync(ctx, t, gm, gp, thin, &sp);
    if (st) return st;
    const BufGeo geo = thin ? ctx->gT : ctx->gA;
    int gst, pst;
    if (df && !sp->pair_begin.empty() && !sp->pcls.begin.empty() &&
        fused_shape(sp->table.stage_predict, sp->pair_begin, sp->copy_end, skip_copies && sp->push_ok, &gst, &pst) &&
        sp->pcls.begin[pst].size() == 2) {
        const unsigned from = gst < 0 ? 0 : (skip_copies && sp->push_ok ? sp->copy_end[gst] : sp->pair_begin[gst]);
        const unsigned n = gst < 0 ? 0 : sp->pair_begin[gst + 1] - from;
        const std::vector<int> &pb = sp->pcls.begin[pst];
        WG_CUDA_OK(launch_sync_df_fused(sp->pairs.p + from, n, sp->pcls.patches.p + pb[0], pb[1] - pb[0],
                                        sp->pcls.need[pst][0], buf, geo, ctx->geo.nc, ctx->wav.order_predictor,
                                        ctx->d_desc, ctx->d_clk, fused_ctr(ctx), ctx->d_err, ctx->stream, 4));
        return WG_OK;
    }
    for (int s = 0; s < sp->table.nstages; s++) {
        const int b = sp->table.stage_begin[s], e = sp->table.stage_begin[s + 1];
        // copies and decimations move 8-byte elements: the same kernel serves
        // FP64 and double-float buffers; predictions convert
        if (sp->table.stage_predict[s] && df && !sp->pcls.begin.empty()) {
            int st3 = run_pred_classes(ctx, sp->pcls, s, buf, geo);
            if (st3) return st3;
        } else if (sp->table.stage_predict[s] && df)
            WG_CUDA_OK(launch_predict_df(sp->d.p + b, e - b, sp->table.max_coarse, buf, geo, ctx->geo.nc,
                                         ctx->wav.order_predictor, ctx->d_desc, ctx->d_clk, ctx->stream));
        else if (sp->table.stage_predict[s])
            WG_CUDA_OK(launch_predict(sp->d.p + b, e - b, sp->table.max_coarse, buf, geo, ctx->geo.nc,
                                      ctx->wav.order_predictor, ctx->stream));
        else if (!sp->pair_begin.empty()) {
            const unsigned from = skip_copies && sp->push_ok ? sp->copy_end[s] : sp->pair_begin[s];
            WG_CUDA_OK(launch_gather(sp->pairs.p + from, sp->pair_begin[s + 1] - from, buf, geo, ctx->geo.nc,
                                     ctx->stream));
        }
        else
            WG_CUDA_OK(launch_sync(sp->d.p + b, e - b, buf, geo, ctx->geo.nc, ctx->wav.order_predictor, ctx->stream));
    }
    return WG_OK;
}

void release_tree_blocks(wg_ctx *ctx, Tree &t) {
    for (int s : t.slots) ctx->free_slots.give(s);
    for (int m : t.mask_slot)
        if (m >= 0) ctx->mask_free.push_back(m);
    t.slots.clear();
    t.mask_slot.clear();
    drop_sync(t);
    t.n_plain = t.n_masked = 0;
}

int upload_lists(wg_ctx *ctx, Tree &t) {
    std::vector<int> plain, masked;
    for (size_t b = 0; b < t.slots.size(); b++) (t.mask_slot[b] >= 0 ? masked : plain).push_back(t.slots[b]);
    t.n_plain = (int)plain.size();
    t.n_masked = (int)masked.size();
    WG_CUDA_OK(t.d_all.upload(t.slots.data(), t.slots.size(), ctx->stream));
    WG_CUDA_OK(t.d_plain.upload(plain.data(), plain.size(), ctx->stream));
    WG_CUDA_OK(t.d_masked.upload(masked.data(), masked.size(), ctx->stream));
    std::vector<int> order(masked);
    order.insert(order.end(), plain.begin(), plain.end());
    WG_CUDA_OK(t.d_stage.upload(order.data(), order.size(), ctx->stream));
    return WG_OK;
}

// (re)write the descriptors of a tree's blocks
int upload_desc(wg_ctx *ctx, Tree &t, int tree_id) {
    const wg_config &c = ctx->cfg;
    for (size_t b = 0; b < t.slots.size(); b++) {
        BlockDesc d;
        std::memset(&d, 0, sizeof(d));
        const int lv = t.forest.level[b];
        for (int k = 0; k < 3; k++) d.dx[k] = k < c.dim ? std::pow(2.0, -lv) * c.domain[k] / (double)c.Bs[k] : 0.0;
        const double nu = t.cfg.nu;
        d.m0 = 0.0;
        for (int k = 0; k < c.dim; k++) {
            d.k1[k] = (2.0 / 3.0) / d.dx[k];
            d.k2[k] = (1.0 / 12.0) / d.dx[k];
            d.m1[k] = nu * (4.0 / 3.0) / (d.dx[k] * d.dx[k]);
            d.m2[k] = nu * (1.0 / 12.0) / (d.dx[k] * d.dx[k]);
            d.m0 += nu * (-2.5) / (d.dx[k] * d.dx[k]);
        }
        double sc = 0.0;
        for (int k = 0; k < c.dim; k++) {
            const double s2 = nu / (12.0 * d.dx[k] * d.dx[k]);
            split_df(1.0 / (12.0 * d.dx[k]), d.fs1[k]);
            split_df(s2, d.fs2[k]);
            sc += -30.0 * s2;
        }
        split_df(sc, d.fsc);
        d.tree = tree_id;
        d.level = lv;
        d.mask = t.mask_slot[b];
        ctx->h_desc[t.slots[b]] = d;
    }
    // one copy per run of consecutive slots from the host mirror
    std::vector<int> sl(t.slots);
    std::sort(sl.begin(), sl.end());
    for (size_t i = 0; i < sl.size();) {
        size_t j = i + 1;
        while (j < sl.size() && sl[j] == sl[j - 1] + 1) j++;
        WG_CUDA_OK(cudaMemcpyAsync(ctx->d_desc + sl[i], ctx->h_desc.data() + sl[i], sizeof(BlockDesc) * (j - i),
                                   cudaMemcpyHostToDevice, ctx->stream));
        i = j;
    }
    return WG_OK;
}

int stage_launch(wg_ctx *ctx, Tree &t, int stage, const double *in, BufGeo gin, double *out, BufGeo gout) {
    const int dim = ctx->cfg.dim;
    const int base = (ctx->variant_fast ? 1 : 0) | (t.cfg.skew_symmetry ? 2 : 0);
    const int *Bs = ctx->cfg.Bs;
    WG_CUDA_OK(launch_acm_stage(base, dim, stage, t.d_plain.p, t.n_plain, ctx->d_desc, ctx->d_tp, ctx->d_clk, in,
                                gin, out, gout, ctx->A, ctx->gA, ctx->acc, ctx->mask, Bs[0], Bs[1], Bs[2],
                                ctx->geo.nc, ctx->stream));
    WG_CUDA_OK(launch_acm_stage(base | 4, dim, stage, t.d_masked.p, t.n_masked, ctx->d_desc, ctx->d_tp, ctx->d_clk,
                                in, gin, out, gout, ctx->A, ctx->gA, ctx->acc, ctx->mask, Bs[0], Bs[1], Bs[2],
                                ctx->geo.nc, ctx->stream));
    return WG_OK;
}

// the TMA map over a thin stage buffer (slab or one-plane boxes)
static const void *in_map(wg_ctx *ctx, const double *in, bool plane, int slab = 4) {
    const CUtensorMap *m = plane ? ctx->tp : slab == 2 ? ctx->tm2 : slab == 8 ? ctx->tm8 : ctx->tm;
    return in == ctx->B ? &m[0] : in == ctx->C ? &m[1] : in == ctx->D ? &m[2] : in == ctx->E ? &m[3] : nullptr;
}

// the stage-kernel form of RK stage `stage`
static int form_of(const wg_ctx *ctx, int stage) {
    if (ctx->stage_form != WG_FORM_AUTO) return ctx->stage_form;
    return ctx->tuned[stage - 1] ? ctx->tuned[stage - 1] : WG_FORM_DIRECT;
}

// kernel arguments of a form: the tensor map (null: direct) and the march flag
static void form_args(wg_ctx *ctx, int stage, const double *in, const void **tm, int *march) {
    const int form = form_of(ctx, stage);
    *tm = nullptr;
    *march = 0;
    if (form == WG_FORM_TILE && ctx->have_tm) *tm = in_map(ctx, in, false);
    if (form == WG_FORM_MARCH && ctx->have_march) {
        *tm = in_map(ctx, in, true);
        *march = 1;
    }
    if (form == WG_FORM_PIPE && ctx->have_tm) {
        *tm = in_map(ctx, in, false);
        *march = 2;
    }
    if ((form == WG_FORM_TILE2 || form == WG_FORM_TILE8) && ctx->have_tm) {
        *tm = in_map(ctx, in, false, form == WG_FORM_TILE2 ? 2 : 8);
        *march = form == WG_FORM_TILE2 ? 3 : 4;
    }
}

// the two launches of an FP32-pipe stage, one after the other: the unmasked
// blocks' kernel and the masked blocks' kernel (the mask words compiled out
// of the first; one kernel testing the mask per block was 3 % slower, and
// the two kernels side by side on two streams 25 % slower in the last stage)
// (the pipe form: one launch over `both`, the masked blocks followed by the
// others)
static int stage_pair(wg_ctx *ctx, int stage, const int *plain, int nplain, const int *masked, int nmasked,
                      const int *both, const double *in, double *out, const int *pp, int keep) {
    const int dim = ctx->cfg.dim;
    const int *Bs = ctx->cfg.Bs;
    const void *tm = nullptr;
    int march = 0;
    form_args(ctx, stage, in, &tm, &march);
    auto go = [&](int msk, const int *blk, int n) {
        return launch_acm_stage_df(dim, stage, msk, blk, n, ctx->d_desc, ctx->d_tp, ctx->d_clk, in, ctx->B, ctx->C,
                                   ctx->D, out, ctx->gT, ctx->A, ctx->gA, ctx->mask_df, pp, Bs[0], Bs[1], Bs[2], tm,
                                   march, ctx->d_err, ctx->stream, keep, ctx->s4_out, ctx->d_pos.p, ctx->s4_next,
                                   stage == 4 ? ctx->s4_usrc : nullptr, ctx->d_usq);
    };
    if (march == 2) {
        WG_CUDA_OK(go(nmasked, both, nplain + nmasked));
        return WG_OK;
    }
    WG_CUDA_OK(go(0, plain, nplain));
    WG_CUDA_OK(go(1, masked, nmasked));
    return WG_OK;
}

// u0 is always B (the anchored copy of u_n), the inputs of stages 2 and 3
// are C and D; with push the kernels also write the same-level ghost copies
// of out
int stage_launch_df(wg_ctx *ctx, Tree &t, int stage, const double *in, double *out, bool push, int keep = 1) {
    return stage_pair(ctx, stage, t.d_plain.p, t.n_plain, t.d_masked.p, t.n_masked, t.d_stage.p, in, out,
                      push ? ctx->d_push : nullptr, keep);
}

// TMA maps over the four thin double-float buffers: a 3-D tensor of 8-byte
// elements (x, y, plane-of-all-blocks-and-components), box nx * ny * (zt+4)
int make_tensor_maps(wg_ctx *ctx) {
    const int zt = tile_slab(ctx->cfg.dim, ctx->cfg.Bs[0], ctx->cfg.Bs[1], ctx->cfg.Bs[2], ctx->gT.gb);
    if (!zt) return WG_OK;
    using Encode = CUresult (*)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
    void *fn = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess || !fn) {
        cudaGetLastError();
        return WG_OK;   // no TMA maps: the direct-load kernel runs
    }
    const BufGeo &g = ctx->gT;
    const cuuint64_t dims[3] = {(cuuint64_t)g.nx, (cuuint64_t)g.ny,
                                (cuuint64_t)g.nz * ctx->geo.nc * (cuuint64_t)ctx->max_blocks};
    const cuuint64_t strides[2] = {(cuuint64_t)g.nx * 8, (cuuint64_t)g.nx * g.ny * 8};
    const cuuint32_t box[3] = {(cuuint32_t)g.nx, (cuuint32_t)g.ny, (cuuint32_t)(zt + 4)};
    const cuuint32_t pbox[3] = {(cuuint32_t)g.nx, (cuuint32_t)g.ny, 1};
    const cuuint32_t box2[3] = {(cuuint32_t)g.nx, (cuuint32_t)g.ny, 6};
    const cuuint32_t box8[3] = {(cuuint32_t)g.nx, (cuuint32_t)g.ny, 12};
    const cuuint32_t estr[3] = {1, 1, 1};
    double *bufs[4] = {ctx->B, ctx->C, ctx->D, ctx->E};
    const bool march = ctx->cfg.Bs[2] == 16;   // the march kernel walks 16 planes
    const bool slabs28 = ctx->cfg.Bs[2] % 8 == 0;   // slab heights 2 and 8 divide the block
    for (int i = 0; i < 4; i++) {
        for (int k = 0; k < 4; k++) {
            if ((k == 1 && !march) || (k >= 2 && !slabs28)) continue;
            CUtensorMap *dst = k == 0 ? &ctx->tm[i] : k == 1 ? &ctx->tp[i] : k == 2 ? &ctx->tm2[i] : &ctx->tm8[i];
            const cuuint32_t *bx = k == 0 ? box : k == 1 ? pbox : k == 2 ? box2 : box8;
            const CUresult r = reinterpret_cast<Encode>(fn)(dst, CU_TENSOR_MAP_DATA_TYPE_UINT64, 3, bufs[i], dims,
                                                            strides, bx, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                                                            CU_TENSOR_MAP_SWIZZLE_NONE,
                                                            CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                                                            CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
            if (r != CUDA_SUCCESS) return fail(WG_ECUDA, "cuTensorMapEncodeTiled failed (%d)", (int)r);
        }
    }
    ctx->have_slabs28 = slabs28;
    ctx->have_tm = true;
    ctx->have_march = march;
    return WG_OK;
}

// a kernel's bounded wait ran out (reported once, then cleared)
int check_dev_err(wg_ctx *ctx) {
    if (!ctx->d_err) return WG_OK;
    int h = 0;
    WG_CUDA_OK(cudaMemcpyAsync(&h, ctx->d_err, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    WG_CUDA_OK(cudaStreamSynchronize(ctx->stream));
    if (!h) return WG_OK;
    ctx->dead = true;
    return fail(WG_ETIMEOUT, "a bounded device wait (a stage kernel's shared-memory load or the ghost sync's "
                             "wait for its restrictions) ran out; the context is unusable, destroy it");
}

// the thin per-step plan of a tree, and whether its copies are pushed
int thin_plan(wg_ctx *ctx, Tree &t, bool *push) {
    SyncPlan *sp;
    int st = get_sync(ctx, t, ctx->cfg.g_rhs, ctx->cfg.g_rhs, true, &sp);
    if (st) return st;
    *push = sp->push_ok && !sp->pair_begin.empty();
    return WG_OK;
}

// double-float copy of u_n (interior of A) into B, needed once after the
// state changed outside an RK step
int ensure_shadow(wg_ctx *ctx, Tree &t) {
    if (ctx->precision != WG_RHS_FP32 || t.shadow_valid) return WG_OK;
    const int *Bs = ctx->cfg.Bs;
    bool push;
    int st = thin_plan(ctx, t, &push);
    if (st) return st;
    const int tid = (int)(&t - ctx->trees.data());
    WG_CUDA_OK(launch_anchor_from_state(t.d_all.p, (int)t.slots.size(), ctx->A, ctx->gA, ctx->geo.nc, Bs[0], Bs[1],
                                        ctx->cfg.dim == 3 ? Bs[2] : 1, ctx->d_desc, ctx->d_clk,
                                        ctx->d_tree_ids.p + tid, 1, 1, ctx->stream));
    WG_CUDA_OK(launch_shadow(t.d_all.p, (int)t.slots.size(), ctx->A, ctx->gA, ctx->B, ctx->gT, ctx->geo.nc, Bs[0],
                             Bs[1], ctx->cfg.dim == 3 ? Bs[2] : 1, push ? ctx->d_push : nullptr, ctx->d_desc,
                             ctx->d_clk, ctx->stream));
    t.shadow_valid = true;
    return WG_OK;
}

// Autotuner of the FP32-pipe stage kernel: for each RK stage, times every
// applicable form (direct, tile, march) on this tree's grid and keeps the
// fastest for the context. The stages are timed in step order, each reading
// the previous one's output (B -> C -> D -> E), so the timed kernels see
// realistic values. Nothing the next step reads changes: stages 1-3 write
// the scratch stage buffers, and stage 4 writes its copy of u_n+1 to C (not
// B) and neither stores u_n+1 nor records its maximum (keep = 4: it writes
// u_n back unchanged where u_n+1 would go, so its traffic is the real one). The
// autotuner may therefore run between any two steps without changing a bit
// of the results.
int autotune_stage_form(wg_ctx *ctx, Tree &t) {
    if (ctx->precision != WG_RHS_FP32 || ctx->stage_form != WG_FORM_AUTO || ctx->tuned[0]) return WG_OK;
    std::vector<int> forms = {WG_FORM_DIRECT};
    if (ctx->have_tm && !t.slots.empty()) forms.push_back(WG_FORM_TILE);
    if (ctx->have_march && !t.slots.empty()) forms.push_back(WG_FORM_MARCH);
    if (ctx->have_tm && !t.slots.empty()) forms.push_back(WG_FORM_PIPE);
    if (ctx->have_slabs28 && !t.slots.empty()) {
        forms.push_back(WG_FORM_TILE2);
        forms.push_back(WG_FORM_TILE8);
    }
    if (forms.size() == 1) {
        for (int &f : ctx->tuned) f = WG_FORM_DIRECT;
        return WG_OK;
    }
    bool push;
    int st = ensure_shadow(ctx, t);
    if (st) return st;
    if ((st = thin_plan(ctx, t, &push))) return st;
    cudaEvent_t e0, e1;
    WG_CUDA_OK(cudaEventCreate(&e0));
    WG_CUDA_OK(cudaEventCreate(&e1));
    double *in[4] = {ctx->B, ctx->C, ctx->D, ctx->E}, *out[4] = {ctx->C, ctx->D, ctx->E, ctx->C};
    for (int stage = 1; stage <= 4 && !st; stage++) {
        float best = 0.f;
        int best_form = WG_FORM_DIRECT;
        for (int form : forms) {
            ctx->tuned[stage - 1] = form;
            const int keep = stage == 4 ? 4 : 1;
            if ((st = stage_launch_df(ctx, t, stage, in[stage - 1], out[stage - 1], push, keep))) break;   // warm-up
            WG_CUDA_OK(cudaEventRecord(e0, ctx->stream));
            for (int r = 0; r < 3 && !st; r++) st = stage_launch_df(ctx, t, stage, in[stage - 1], out[stage - 1], push, keep);
            WG_CUDA_OK(cudaEventRecord(e1, ctx->stream));
            WG_CUDA_OK(cudaEventSynchronize(e1));
            float ms = 0.f;
            WG_CUDA_OK(cudaEventElapsedTime(&ms, e0, e1));
            if (form == forms[0] || ms < best) {
                best = ms;
                best_form = form;
            }
        }
        ctx->tuned[stage - 1] = best_form;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (st) return st;
    return check_dev_err(ctx);
}

// one RK4 step with double-float stencils: B holds the double-float copy of
// u_n (stage 1 input) and keeps it through the step; the stage inputs 2-4
// are C, D, C; stage 4 adds the increment to A and writes the copy of
// u_{n+1} to B
// event i of the step profile (0: step start, then after sync 1, dt,
// stage 1, sync 2, stage 2, sync 3, stage 3, sync 4, stage 4)
static inline void prof_mark(wg_ctx *ctx, int i) {
    if (ctx->prof_on) cudaEventRecord(ctx->prof_ev[i], ctx->stream);
}

int rk4_enqueue_df(wg_ctx *ctx, int tree_id) {
    Tree &t = ctx->trees[tree_id];
    const int g_rhs = ctx->cfg.g_rhs;
    const int *Bs = ctx->cfg.Bs;
    int st;
    bool push;
    if ((st = thin_plan(ctx, t, &push))) return st;
    prof_mark(ctx, 0);
    // B's same-level ghosts were written with its interior (previous stage 4
    // or the shadow copy) when push is on
    if ((st = run_sync(ctx, t, ctx->B, true, g_rhs, g_rhs, true, push))) return st;
    prof_mark(ctx, 1);
    if (ctx->s4_usrc) {   // u_n in the compact input of a streamed step
        const BufGeo gc = {Bs[0], Bs[1], ctx->cfg.dim == 3 ? Bs[2] : 1, 0};
        WG_CUDA_OK(launch_dt(ctx->cfg.dim, t.d_all.p, (int)t.slots.size(), ctx->d_desc, ctx->d_tp, ctx->d_clk,
                             ctx->s4_usrc, gc, Bs[0], Bs[1], Bs[2], 1, ctx->d_tree_ids.p + tree_id, dt_done(ctx),
                             ctx->stream, 1, ctx->d_pos.p, ctx->d_usq));
    } else {
        WG_CUDA_OK(launch_dt(ctx->cfg.dim, t.d_all.p, (int)t.slots.size(), ctx->d_desc, ctx->d_tp, ctx->d_clk, ctx->A,
                             ctx->gA, Bs[0], Bs[1], Bs[2], 1, ctx->d_tree_ids.p + tree_id, dt_done(ctx), ctx->stream, 1,
                             nullptr, ctx->d_usq));
    }
    prof_mark(ctx, 2);
    if ((st = stage_launch_df(ctx, t, 1, ctx->B, ctx->C, push))) return st;
    prof_mark(ctx, 3);
    if ((st = run_sync(ctx, t, ctx->C, true, g_rhs, g_rhs, true, push))) return st;
    prof_mark(ctx, 4);
    if ((st = stage_launch_df(ctx, t, 2, ctx->C, ctx->D, push))) return st;
    prof_mark(ctx, 5);
    if ((st = run_sync(ctx, t, ctx->D, true, g_rhs, g_rhs, true, push))) return st;
    prof_mark(ctx, 6);
    if ((st = stage_launch_df(ctx, t, 3, ctx->D, ctx->E, push))) return st;
    prof_mark(ctx, 7);
    if ((st = run_sync(ctx, t, ctx->E, true, g_rhs, g_rhs, true, push))) return st;
    prof_mark(ctx, 8);
    if (ctx->s4_wait) WG_CUDA_OK(cudaStreamWaitEvent(ctx->stream, ctx->s4_wait, 0));
    if ((st = stage_launch_df(ctx, t, 4, ctx->E, ctx->B, push, ctx->s4_keep))) return st;
    // the last stage recorded the maxima of what it wrote (the state, or in
    // a streamed step the next input) unless it ran for timing only
    WG_CUDA_OK(launch_clock_advance(ctx->d_clk, ctx->d_tree_ids.p + tree_id, 1, ctx->stream,
                                    ctx->s4_keep == 1 || ctx->s4_keep == 3));
    prof_mark(ctx, 9);
    return WG_OK;
}

// (re)build ctx->batch for the listed trees (FP32-pipe precision)
int build_batch(wg_ctx *ctx, const std::vector<int> &trees) {
    BatchPlan &bp = ctx->batch;
    if (bp.version == ctx->grid_version && bp.trees == trees) return WG_OK;
    std::vector<SyncPlan *> plans;
    bool push = true;
    for (int id : trees) {
        Tree &t = ctx->trees[id];
        SyncPlan *sp;
        int st = get_sync(ctx, t, ctx->cfg.g_rhs, ctx->cfg.g_rhs, true, &sp);
        if (st) return st;
        if (sp->pair_begin.empty()) return fail(WG_ENOTSUP, "batched step needs the gather form of the ghost sync");
        push = push && sp->push_ok;
        plans.push_back(sp);
    }
    const int ns = plans[0]->table.nstages;
    std::vector<int> all, plain, masked;
    for (int id : trees) {
        Tree &t = ctx->trees[id];
        for (size_t b = 0; b < t.slots.size(); b++) {
            all.push_back(t.slots[b]);
            (t.mask_slot[b] >= 0 ? masked : plain).push_back(t.slots[b]);
        }
    }
    bp.n_all = (int)all.size();
    bp.n_plain = (int)plain.size();
    bp.n_masked = (int)masked.size();
    WG_CUDA_OK(bp.all.upload(all.data(), all.size(), ctx->stream));
    WG_CUDA_OK(bp.plain.upload(plain.data(), plain.size(), ctx->stream));
    WG_CUDA_OK(bp.masked.upload(masked.data(), masked.size(), ctx->stream));
    {
        std::vector<int> order(masked);
        order.insert(order.end(), plain.begin(), plain.end());
        WG_CUDA_OK(bp.stage.upload(order.data(), order.size(), ctx->stream));
    }
    WG_CUDA_OK(bp.tree_ids.upload(trees.data(), trees.size(), ctx->stream));
    // gather entries and prediction patches, stage by stage
    bp.nstages = ns;
    bp.stage_predict = plans[0]->table.stage_predict;
    bp.pair_begin.assign(ns + 1, 0);
    bp.copy_end.assign(ns, 0);
    bp.pred_begin.assign(ns + 1, 0);
    bp.max_coarse = 0;
    unsigned long long total = 0;
    std::vector<Patch> pred;
    for (int st = 0; st < ns; st++) {
        bp.pair_begin[st] = (unsigned)total;
        bp.pred_begin[st] = (int)pred.size();
        for (SyncPlan *sp : plans) total += sp->pair_begin[st + 1] - sp->pair_begin[st];
        for (SyncPlan *sp : plans) {
            if (!sp->table.stage_predict[st]) continue;
            const auto &pt = sp->table.patches;
            pred.insert(pred.end(), pt.begin() + sp->table.stage_begin[st], pt.begin() + sp->table.stage_begin[st + 1]);
            bp.max_coarse = std::max(bp.max_coarse, sp->table.max_coarse);
        }
    }
    bp.pair_begin[ns] = (unsigned)total;
    bp.pred_begin[ns] = (int)pred.size();
    if (total >= (1ull << 32)) return fail(WG_ENOTSUP, "batched ghost gather exceeds 2^32 entries");
    WG_CUDA_OK(bp.pairs.upload(nullptr, total, ctx->stream));
    WG_CUDA_OK(bp.predict.upload(pred.data(), pred.size(), ctx->stream));
    {
        std::vector<int> sp_pred(ns, 0);
        for (int st = 0; st < ns; st++) sp_pred[st] = bp.stage_predict[st];
        int st2 = build_pred_classes(ctx, pred, bp.pred_begin, sp_pred, bp.pcls);
        if (st2) return st2;
    }
    for (int st = 0; st < ns; st++) {
        unsigned at = bp.pair_begin[st];
        for (int pass = 0; pass < 2; pass++) {          // copies of every tree first
            for (SyncPlan *sp : plans) {
                const unsigned b = pass == 0 ? sp->pair_begin[st] : sp->copy_end[st];
                const unsigned e = pass == 0 ? sp->copy_end[st] : sp->pair_begin[st + 1];
                if (e > b)
                    WG_CUDA_OK(cudaMemcpyAsync(bp.pairs.p + at, sp->pairs.p + b, sizeof(uint2) * (e - b),
                                               cudaMemcpyDeviceToDevice, ctx->stream));
                at += e - b;
            }
            if (pass == 0) bp.copy_end[st] = at;
        }
    }
    WG_CUDA_OK(cudaStreamSynchronize(ctx->stream));
    bp.push = push;
    bp.trees = trees;
    bp.version = ctx->grid_version;
    return WG_OK;
}

int run_sync_batch(wg_ctx *ctx, double *buf) {
    const BatchPlan &bp = ctx->batch;
    int gst, pst;
    if (!bp.pcls.begin.empty() && fused_shape(bp.stage_predict, bp.pair_begin, bp.copy_end, bp.push, &gst, &pst) &&
        bp.pcls.begin[pst].size() == 2) {
        const unsigned from = gst < 0 ? 0 : (bp.push ? bp.copy_end[gst] : bp.pair_begin[gst]);
        const unsigned n = gst < 0 ? 0 : bp.pair_begin[gst + 1] - from;
        const std::vector<int> &pb = bp.pcls.begin[pst];
        WG_CUDA_OK(launch_sync_df_fused(bp.pairs.p + from, n, bp.pcls.patches.p + pb[0], pb[1] - pb[0],
                                        bp.pcls.need[pst][0], buf, ctx->gT, ctx->geo.nc, ctx->wav.order_predictor,
                                        ctx->d_desc, ctx->d_clk, fused_ctr(ctx), ctx->d_err, ctx->stream, 4));
        return WG_OK;
    }
    for (int s = 0; s < bp.nstages; s++) {
        if (bp.stage_predict[s]) {
            int st3 = run_pred_classes(ctx, bp.pcls, s, buf, ctx->gT);
            if (st3) return st3;
        } else {
            const unsigned from = bp.push ? bp.copy_end[s] : bp.pair_begin[s];
            WG_CUDA_OK(launch_gather(bp.pairs.p + from, bp.pair_begin[s + 1] - from, buf, ctx->gT, ctx->geo.nc,
                                     ctx->stream));
        }
    }
    return WG_OK;
}

int stage_launch_batch(wg_ctx *ctx, int stage, const double *in, double *out) {
    const BatchPlan &bp = ctx->batch;
    return stage_pair(ctx, stage, bp.plain.p, bp.n_plain, bp.masked.p, bp.n_masked, bp.stage.p, in, out,
                      bp.push ? ctx->d_push : nullptr, 1);
}

// one RK4 step of every tree of ctx->batch (FP32-pipe precision): the same
// sequence as rk4_enqueue_df, each kernel launched once for all trees
int rk4_enqueue_batch(wg_ctx *ctx) {
    const BatchPlan &bp = ctx->batch;
    const int *Bs = ctx->cfg.Bs;
    int st;
    prof_mark(ctx, 0);
    if ((st = run_sync_batch(ctx, ctx->B))) return st;
    prof_mark(ctx, 1);
    WG_CUDA_OK(launch_dt(ctx->cfg.dim, bp.all.p, bp.n_all, ctx->d_desc, ctx->d_tp, ctx->d_clk, ctx->A, ctx->gA, Bs[0],
                         Bs[1], Bs[2], (int)bp.trees.size(), bp.tree_ids.p, dt_done(ctx), ctx->stream, 1, nullptr,
                         ctx->d_usq));
    prof_mark(ctx, 2);
    if ((st = stage_launch_batch(ctx, 1, ctx->B, ctx->C))) return st;
    prof_mark(ctx, 3);
    if ((st = run_sync_batch(ctx, ctx->C))) return st;
    prof_mark(ctx, 4);
    if ((st = stage_launch_batch(ctx, 2, ctx->C, ctx->D))) return st;
    prof_mark(ctx, 5);
    if ((st = run_sync_batch(ctx, ctx->D))) return st;
    prof_mark(ctx, 6);
    if ((st = stage_launch_batch(ctx, 3, ctx->D, ctx->E))) return st;
    prof_mark(ctx, 7);
    if ((st = run_sync_batch(ctx, ctx->E))) return st;
    prof_mark(ctx, 8);
    if ((st = stage_launch_batch(ctx, 4, ctx->E, ctx->B))) return st;
    WG_CUDA_OK(launch_clock_advance(ctx->d_clk, bp.tree_ids.p, (int)bp.trees.size(), ctx->stream, 1));
    prof_mark(ctx, 9);
    return WG_OK;
}

// one RK4 step of one tree, fully asynchronous on ctx->stream
int rk4_enqueue(wg_ctx *ctx, int tree_id) {
    if (ctx->precision == WG_RHS_FP32) return rk4_enqueue_df(ctx, tree_id);
    Tree &t = ctx->trees[tree_id];
    const int g_rhs = ctx->cfg.g_rhs;
    const int *Bs = ctx->cfg.Bs;
    int st;
    prof_mark(ctx, 0);
    if ((st = run_sync(ctx, t, ctx->A, false, g_rhs, g_rhs))) return st;
    prof_mark(ctx, 1);
    WG_CUDA_OK(launch_dt(ctx->cfg.dim, t.d_all.p, (int)t.slots.size(), ctx->d_desc, ctx->d_tp, ctx->d_clk, ctx->A,
                         ctx->gA, Bs[0], Bs[1], Bs[2], 1, ctx->d_tree_ids.p + tree_id, dt_done(ctx), ctx->stream, 0,
                         nullptr, ctx->d_usq));
    prof_mark(ctx, 2);
    if ((st = stage_launch(ctx, t, 1, ctx->A, ctx->gA, ctx->B, ctx->gT))) return st;
    prof_mark(ctx, 3);
    if ((st = run_sync(ctx, t, ctx->B, true, g_rhs, g_rhs))) return st;
    prof_mark(ctx, 4);
    if ((st = stage_launch(ctx, t, 2, ctx->B, ctx->gT, ctx->C, ctx->gT))) return st;
    prof_mark(ctx, 5);
    if ((st = run_sync(ctx, t, ctx->C, true, g_rhs, g_rhs))) return st;
    prof_mark(ctx, 6);
    if ((st = stage_launch(ctx, t, 3, ctx->C, ctx->gT, ctx->B, ctx->gT))) return st;
    prof_mark(ctx, 7);
    if ((st = run_sync(ctx, t, ctx->B, true, g_rhs, g_rhs))) return st;
    prof_mark(ctx, 8);
    if ((st = stage_launch(ctx, t, 4, ctx->B, ctx->gT, nullptr, ctx->gT))) return st;
    WG_CUDA_OK(launch_clock_advance(ctx->d_clk, ctx->d_tree_ids.p + tree_id, 1, ctx->stream));
    prof_mark(ctx, 9);
    return WG_OK;
}

int read_clock(wg_ctx *ctx, int tree, TreeClock *out) {
    WG_CUDA_OK(cudaMemcpyAsync(out, ctx->d_clk + tree, sizeof(TreeClock), cudaMemcpyDeviceToHost, ctx->stream));
    WG_CUDA_OK(cudaStreamSynchronize(ctx->stream));
    return check_dev_err(ctx);
}

}  // namespace

extern "C" {

const char *wg_last_error(void) { return g_err.c_str(); }

int wg_config_defaults(wg_config *c, int dim) {
    if (!c || (dim != 2 && dim != 3)) return fail(WG_EINVAL, "bad arguments");
    std::memset(c, 0, sizeof(*c));
    c->dim = dim;
    c->Bs[0] = c->Bs[1] = 16;
    c->Bs[2] = dim == 3 ? 16 : 1;
    std::strcpy(c->wavelet, "CDF40");
    c->g = 3;
    c->g_rhs = 2;
    c->neq = dim + 1;
    c->domain[0] = c->domain[1] = c->domain[2] = 1.0;
    c->Jmin = 1;
    c->Jmax = 1;
    c->c0 = 10.0;
    c->nu = 1e-1;
    c->gamma_p = 1.0;
    c->penalization = 1;
    c->C_eta = 1.0;
    c->C_sponge = 1e-2;
    c->u_mean_set[0] = 1.0;
    c->CFL = 1.0;
    c->CFL_eta = 0.99;
    c->CFL_nu = 0.95 * 2.79 / (5.333 * (double)dim);
    c->time_max = 1.0;
    c->eps = 1e-3;
    for (int i = 0; i < 8; i++) c->threshold_state_vector_component[i] = 1;
    return WG_OK;
}

size_t wg_bytes_per_block(const wg_config *c) {
    if (!c) return 0;
    const long long nA = (long long)(c->Bs[0] + 2 * c->g) * (c->Bs[1] + 2 * c->g) * (c->dim == 3 ? c->Bs[2] + 2 * c->g : 1);
    const long long nT = (long long)(c->Bs[0] + 2 * c->g_rhs) * (c->Bs[1] + 2 * c->g_rhs) *
                         (c->dim == 3 ? c->Bs[2] + 2 * c->g_rhs : 1);
    const long long nI = (long long)c->Bs[0] * c->Bs[1] * (c->dim == 3 ? c->Bs[2] : 1);
    // FP64: thin buffers B, C and the interior RK accumulator; FP32-pipe:
    // thin buffers B, C, D, E (u_n copy and the stage inputs 2-4)
    const bool df = c->rhs_precision == WG_RHS_FP32;
    return sizeof(double) * (size_t)c->neq * (size_t)(nA + (df ? 4 : 2) * nT + (df ? 0 : nI)) + sizeof(BlockDesc);
}

int wg_ctx_create(const wg_config *cfg, int max_blocks, wg_ctx **out) {
    if (!out) return fail(WG_EINVAL, "null output");
    *out = nullptr;
    int st = check_cfg(cfg);
    if (st) return st;
    if (max_blocks <= 0) return fail(WG_EINVAL, "max_blocks must be positive");
    std::unique_ptr<wg_ctx> ctx(new wg_ctx());
    ctx->cfg = *cfg;
    ctx->precision = cfg->rhs_precision;
    ctx->geo.dim = cfg->dim;
    for (int d = 0; d < 3; d++) ctx->geo.Bs[d] = d < cfg->dim ? cfg->Bs[d] : 1;
    ctx->geo.g = cfg->g;
    ctx->geo.nc = cfg->neq;
    make_wavelet(cfg->wavelet, ctx->wav);
    ctx->max_blocks = max_blocks;
    const int dim = cfg->dim;
    ctx->gA = {cfg->Bs[0] + 2 * cfg->g, cfg->Bs[1] + 2 * cfg->g, dim == 3 ? cfg->Bs[2] + 2 * cfg->g : 1, cfg->g};
    ctx->gT = {cfg->Bs[0] + 2 * cfg->g_rhs, cfg->Bs[1] + 2 * cfg->g_rhs, dim == 3 ? cfg->Bs[2] + 2 * cfg->g_rhs : 1,
               cfg->g_rhs};
    ctx->nint = (long long)cfg->Bs[0] * cfg->Bs[1] * (dim == 3 ? cfg->Bs[2] : 1);
    const size_t nc = cfg->neq;
    const size_t bytesA = sizeof(double) * nc * ctx->gA.npts() * max_blocks;
    const size_t bytesT = sizeof(double) * nc * ctx->gT.npts() * max_blocks;
    const size_t bytesI = sizeof(double) * nc * ctx->nint * max_blocks;
    if (cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking) != cudaSuccess)
        return fail(WG_ECUDA, "cudaStreamCreate failed");
    if (sync_init() != cudaSuccess || wavelet_init() != cudaSuccess) {
        cudaStreamDestroy(ctx->stream);
        return fail(WG_ECUDA, "constant-memory set-up failed");
    }
    auto alloc = [&](double **p, size_t n) { return cudaMalloc(p, n) == cudaSuccess; };
    const bool df = ctx->precision == WG_RHS_FP32;
    if (!alloc(&ctx->A, bytesA) || !alloc(&ctx->B, bytesT) || !alloc(&ctx->C, bytesT) ||
        (!df && !alloc(&ctx->acc, bytesI)) || (df && (!alloc(&ctx->D, bytesT) || !alloc(&ctx->E, bytesT)))) {
        cudaGetLastError();
        wg_ctx_destroy(ctx.release());
        return fail(WG_ENOMEM, "device allocation of %d blocks failed", max_blocks);
    }
    if (cudaMalloc(&ctx->d_desc, sizeof(BlockDesc) * max_blocks) != cudaSuccess ||
        cudaMalloc(&ctx->d_tp, sizeof(TreeParams) * ctx->max_trees) != cudaSuccess ||
        cudaMalloc(&ctx->d_clk, sizeof(TreeClock) * ctx->max_trees) != cudaSuccess ||
        cudaMalloc(&ctx->d_usq, sizeof(unsigned long long) * max_blocks) != cudaSuccess) {
        cudaGetLastError();
        wg_ctx_destroy(ctx.release());
        return fail(WG_ENOMEM, "device allocation of descriptors failed");
    }
    cudaMemsetAsync(ctx->d_usq, 0, sizeof(unsigned long long) * max_blocks, ctx->stream);
    cudaMemsetAsync(ctx->A, 0, bytesA, ctx->stream);
    cudaMemsetAsync(ctx->B, 0, bytesT, ctx->stream);
    cudaMemsetAsync(ctx->C, 0, bytesT, ctx->stream);
    if (ctx->D) cudaMemsetAsync(ctx->D, 0, bytesT, ctx->stream);
    if (ctx->E) cudaMemsetAsync(ctx->E, 0, bytesT, ctx->stream);
    if (ctx->precision == WG_RHS_FP32) {
        if (cudaMalloc(&ctx->d_push, sizeof(int) * 27 * (size_t)max_blocks) != cudaSuccess) {
            cudaGetLastError();
            wg_ctx_destroy(ctx.release());
            return fail(WG_ENOMEM, "device allocation of the ghost push table failed");
        }
        ctx->h_push.assign((size_t)27 * max_blocks, -1);
        cudaMemsetAsync(ctx->d_push, 0xff, sizeof(int) * 27 * (size_t)max_blocks, ctx->stream);
        if ((st = make_tensor_maps(ctx.get()))) {
            wg_ctx_destroy(ctx.release());
            return st;
        }
    }
    if (cudaMalloc(&ctx->d_err, 8 * sizeof(int)) != cudaSuccess) {
        cudaGetLastError();
        wg_ctx_destroy(ctx.release());
        return fail(WG_ENOMEM, "device allocation failed");
    }
    cudaMemsetAsync(ctx->d_err, 0, 8 * sizeof(int), ctx->stream);
    {
        std::vector<TreeClock> clk0(ctx->max_trees, fresh_clock(0.0));
        cudaMemcpyAsync(ctx->d_clk, clk0.data(), sizeof(TreeClock) * ctx->max_trees, cudaMemcpyHostToDevice,
                        ctx->stream);
        cudaStreamSynchronize(ctx->stream);
    }
    ctx->h_desc.resize(max_blocks);
    ctx->free_slots.init(max_blocks);
    ctx->trees.resize(ctx->max_trees);
    std::vector<int> ids(ctx->max_trees);
    for (int i = 0; i < ctx->max_trees; i++) ids[i] = i;
    if (ctx->d_tree_ids.upload(ids.data(), ids.size(), ctx->stream) != cudaSuccess)
        return fail(WG_ECUDA, "upload failed");
    if (cudaStreamSynchronize(ctx->stream) != cudaSuccess) return fail(WG_ECUDA, "stream sync failed");
    *out = ctx.release();
    return WG_OK;
}

int wg_ctx_destroy(wg_ctx *ctx) {
    if (!ctx) return WG_OK;
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    if (ctx->graph_exec) cudaGraphExecDestroy(ctx->graph_exec);
    if (ctx->graph) cudaGraphDestroy(ctx->graph);
    ctx->trees.clear();
    cudaFree(ctx->A);
    cudaFree(ctx->B);
    cudaFree(ctx->C);
    cudaFree(ctx->D);
    cudaFree(ctx->E);
    cudaFree(ctx->acc);
    cudaFree(ctx->mask);
    cudaFree(ctx->mask_df);
    cudaFree(ctx->d_push);
    cudaFree(ctx->d_err);
    cudaFree(ctx->staging);
    cudaFree(ctx->T);
    cudaFree(ctx->d_desc);
    cudaFree(ctx->d_tp);
    cudaFree(ctx->d_clk);
    cudaFree(ctx->d_usq);
    for (cudaEvent_t ev : ctx->copy_ev) cudaEventDestroy(ev);
    for (cudaEvent_t ev : ctx->prof_ev)
        if (ev) cudaEventDestroy(ev);
    if (ctx->copy_stream) cudaStreamDestroy(ctx->copy_stream);
    for (cudaEvent_t ev : ctx->io_ev)
        if (ev) cudaEventDestroy(ev);
    if (ctx->d2h_stream) cudaStreamDestroy(ctx->d2h_stream);
    cudaFree(ctx->stream_buf);
    if (ctx->stream) cudaStreamDestroy(ctx->stream);
    delete ctx;
    return WG_OK;
}

int wg_set_variant(wg_ctx *ctx, int fast) {
    if (!ctx) return fail(WG_EINVAL, "null ctx");
    ctx->variant_fast = fast ? 1 : 0;
    return WG_OK;
}

int wg_tree_create(wg_ctx *ctx, const wg_config *cfg, int *tree) {
    if (!ctx || !tree) return fail(WG_EINVAL, "null argument");
    if (ctx->dead) return fail(WG_ETIMEOUT, "the context is unusable after a timed-out device wait; destroy it");
    const wg_config *c = cfg ? cfg : &ctx->cfg;
    if (c->dim != ctx->cfg.dim || c->g != ctx->cfg.g || c->g_rhs != ctx->cfg.g_rhs || c->neq != ctx->cfg.neq ||
        std::memcmp(c->Bs, ctx->cfg.Bs, sizeof(c->Bs)) || std::strcmp(c->wavelet, ctx->cfg.wavelet))
        return fail(WG_EINVAL, "tree geometry differs from the context's");
    for (int i = 0; i < (int)ctx->trees.size(); i++) {
        if (ctx->trees[i].live) continue;
        Tree &t = ctx->trees[i];
        t = Tree();
        t.live = true;
        t.cfg = *c;
        t.tp = make_params(*c);
        t.forest.dim = c->dim;
        t.forest.Jmin = c->Jmin;
        t.forest.Jmax = c->Jmax;
        WG_CUDA_OK(cudaMemcpyAsync(ctx->d_tp + i, &t.tp, sizeof(TreeParams), cudaMemcpyHostToDevice, ctx->stream));
        const TreeClock clk = fresh_clock(0.0);
        WG_CUDA_OK(cudaMemcpyAsync(ctx->d_clk + i, &clk, sizeof(clk), cudaMemcpyHostToDevice, ctx->stream));
        WG_CUDA_OK(cudaStreamSynchronize(ctx->stream));
        *tree = i;
        ctx->grid_version++;
        return WG_OK;
    }
    return fail(WG_ENOMEM, "too many trees (max %d)", (int)ctx->trees.size());
}

int wg_tree_destroy(wg_ctx *ctx, int tree) {
    Tree *t = get_tree(ctx, tree);
    if (!t) return tree_err();
    cudaStreamSynchronize(ctx->stream);
    release_tree_blocks(ctx, *t);
    *t = Tree();
    ctx->grid_version++;
    return WG_OK;
}

static int regen_masks(wg_ctx *ctx, Tree *t, int tree);

int wg_set_grid(wg_ctx *ctx, int tree, int nblk, const int *level, const int *coords) {
    Tree *t = get_tree(ctx, tree);
    if (!t) return tree_err();
    if (nblk < 0 || (nblk && (!level || !coords))) return fail(WG_EINVAL, "bad grid arguments");
    cudaStreamSynchronize(ctx->stream);
    release_tree_blocks(ctx, *t);
    if ((size_t)nblk > ctx->free_slots.size())
        return fail(WG_ENOMEM, "grid of %d blocks does not fit (%zu free slots)", nblk, ctx->free_slots.size());
    t->forest.set(nblk, level, coords);
    std::string err;
    if (!t->forest.update_neighbors(err)) return fail(WG_EGRID, "%s", err.c_str());
    if (!t->forest.graded()) return fail(WG_EGRID, "grid is not graded (level jump > 1 between neighbours)");
    t->slots.resize(nblk);
    t->status.clear();
    t->mask_slot.assign(nblk, -1);
    if (const int sc = state_changed(ctx, t, tree)) return sc;
    // the lowest free slots in ascending order (contiguous copies)
    for (int b = 0; b < nblk; b++) t->slots[b] = ctx->free_slots.take();
    int st;
    if ((st = upload_desc(ctx, *t, tree))) return st;
    if ((st = upload_lists(ctx, *t))) return st;
    if ((st = regen_masks(ctx, t, tree))) return st;
    WG_CUDA_OK(cudaStreamSynchronize(ctx->stream));
    ctx->grid_version++;
    return WG_OK;
}

int wg_get_nblocks(wg_ctx *ctx, int tree, int *nblk) {
    Tree *t = get_tree(ctx, tree);
    if (!t) return tree_err();
    if (!nblk) return fail(WG_EINVAL, "null output");
    *nblk = t->forest.size();
    return WG_OK;
}

int wg_get_grid(wg_ctx *ctx, int tree, int cap, int *level, int *coords) {
    Tree *t = get_tree(ctx, tree);
    if (!t) return tree_err();
    const int n = t->forest.size();
    if (cap < n) return fail(WG_EINVAL, "capacity %d < %d blocks", cap, n);
    std::memcpy(level, t->forest.level.data(), sizeof(int) * n);
    std::memcpy(coords, t->forest.coords.data(), sizeof(int) * 3 * n);
    return WG_OK;
}

// host_blocks: nblk * neq * npts doubles in the reference block layout
static bool contiguous(const std::vector<int> &s) {
    for (size_t i = 1; i < s.size(); i++)
        if (s[i] != s[i - 1] + 1) return false;
    return true;
}

int wg_upload_state(wg_ctx *ctx, int tree, const double *host_blocks) {
    Tree *t = get_tree(ctx, tree);
    if (!t) return tree_err();
    if (!host_blocks) return fail(WG_EINVAL, "bad arguments");
    if (const int sc = state_changed(ctx, t, tree)) return sc;
    const size_t per = sizeof(double) * ctx->geo.nc * ctx->gA.npts();
    if (!t->slots.empty() && contiguous(t->slots)) {
        WG_CUDA_OK(cudaMemcpyAsync((char *)ctx->A + per * t->slots[0], host_blocks, per * t->slots.size(),
                                   cudaMemcpyHostToDevice, ctx->stream));
        WG_CUDA_OK(cudaStreamSynchronize(ctx->stream));
        return WG_OK;
    }
    for (size_t b = 0; b < t->slots.size(); b++)
        WG_CUDA_OK(cudaMemcpyAsync((char *)ctx->A + per * t->slots[b], (const char *)host_blocks + per * b, per,
                                   cudaMemcpyHostToDevice, ctx->stream));
    WG_CUDA_OK(cudaStreamSynchronize(ctx->stream));
    return WG_OK;
}

int wg_download_state(wg_ctx *ctx, int tree, double *host_blocks) {
    Tree *t = get_tree(ctx, tree);
    if (!t) return tree_err();
    if (!host_blocks) return fail(WG_EINVAL, "bad arguments");
    const size_t per = sizeof(double) * ctx->geo.nc * ctx->gA.npts();
    if (!t->slots.empty() && contiguous(t->slots)) {
        WG_CUDA_OK(cudaMemcpyAsync(host_blocks, (const char *)ctx->A + per * t->slots[0], per * t->slots.size(),
                                   cudaMemcpyDeviceToHost, ctx->stream));
        WG_CUDA_OK(cudaStreamSynchronize(ctx->stream));
        return WG_OK;
    }
    for (size_t b = 0; b < t->slots.size(); b++)
        WG_CUDA_OK(cudaMemcpyAsync((char *)host_blocks + per * b, (const char *)ctx->A + per * t->slots[b], per,
                                   cudaMemcpyDeviceToHost, ctx->stream));
    WG_CUDA_OK(cudaStreamSynchronize(ctx->stream));
    return WG_OK;
}

// Masks of the listed blocks of a tree: mask holds n blocks of 6*npts doubles
// (hvy_mask layout); all other blocks get no mask (chi = 0). Blocks whose
// listed mask is zero (chi, u_s and sponge; the colour is ignored) keep no
// device copy either.
// room in the mask pool for `extra` more blocks (the pool and its
// double-float copy grow by doubling; contents are kept)
static int grow_mask_pool(wg_ctx *ctx, int extra) {
    const long long ni = ctx->nint;
    const int in_use = ctx->mask_cap - (int)ctx->mask_free.size();
    const int want = in_use + extra;
    if (want <= ctx->mask_cap) return WG_OK;
    const int ncap = std::max(want, ctx->mask_cap * 2);
    double *nm = nullptr;
    float2 *nmd = nullptr;
    const bool df = ctx->precision == WG_RHS_FP32;
    if (cudaMalloc(&nm, sizeof(double) * 6 * ni * (size_t)ncap) != cudaSuccess ||
        (df && cudaMalloc(&nmd, sizeof(float2) * 5 * ni * (size_t)ncap) != cudaSuccess)) {
        cudaGetLastError();
        cudaFree(nm);
        return fail(WG_ENOMEM, "mask pool of %d blocks does not fit", ncap);
    }
    if (ctx->mask) {
        WG_CUDA_OK(cudaMemcpyAsync(nm, ctx->mask, sizeof(double) * 6 * ni * (size_t)ctx->mask_cap,
                                   cudaMemcpyDeviceToDevice, ctx->stream));
        if (df)
            WG_CUDA_OK(cudaMemcpyAsync(nmd, ctx->mask_df, sizeof(float2) * 5 * ni * (size_t)ctx->mask_cap,
                                       cudaMemcpyDeviceToDevice, ctx->stream));
        WG_CUDA_OK(cudaStreamSynchronize(ctx->stream));
        cudaFree(ctx->mask);
        cudaFree(ctx->mask_df);
    }
    for (int i = ncap - 1; i >= ctx->mask_cap; i--) ctx->mask_free.push_back(i);
    ctx->mask = nm;
    ctx->mask_df = nmd;
    ctx->mask_cap = ncap;
    return WG_OK;
}

static int install_masks(wg_ctx *ctx, Tree *t, int tree, const std::vector<int> &need,
                         const std::vector<double> &packed);

int wg_set_mask_sparse(wg_ctx *ctx, int tree, int n, const int *blocks, const double *mask) {
    Tree *t = get_tree(ctx, tree);
    if (!t) return tree_err();
    if (n < 0 || (n && (!blocks || !mask))) return fail(WG_EINVAL, "bad arguments");
    cudaStreamSynchronize(ctx->stream);
    t->has_geom = false;
    const int nb = t->forest.size();
    const long long np = ctx->gA.npts();
    const long long ni = ctx->nint;
    const int g = ctx->cfg.g, dim = ctx->cfg.dim;
    const int *Bs = ctx->cfg.Bs;
    std::vector<double> packed;
    std::vector<int> need;
    for (int k = 0; k < n; k++) {
        const int b = blocks[k];
        if (b < 0 || b >= nb) return fail(WG_EINVAL, "mask block id %d out of range", b);
        const double *m = mask + (size_t)k * 6 * np;
        bool any = false;
        std::vector<double> blk(6 * ni);
        for (int c = 0; c < 6; c++)
            for (int iz = 0; iz < (dim == 3 ? Bs[2] : 1); iz++)
                for (int iy = 0; iy < Bs[1]; iy++)
                    for (int ix = 0; ix < Bs[0]; ix++) {
                        const long long src = ((long long)(iz + (dim == 3 ? g : 0)) * ctx->gA.ny + iy + g) * ctx->gA.nx + ix + g;
                        const double v = m[c * np + src];
                        blk[c * ni + ((long long)iz * Bs[1] + iy) * Bs[0] + ix] = v;
                        if (v != 0.0 && c != 4) any = true;
                    }
        if (any) {
            need.push_back(b);
            packed.insert(packed.end(), blk.begin(), blk.end());
        }
    }
    return install_masks(ctx, t, tree, need, packed);
}

// Replace a tree's masks by the interior masks packed (6 * Bs^d doubles per
// block, the pool's layout) of the blocks listed in need; every other block
// runs without a mask.
static int install_masks(wg_ctx *ctx, Tree *t, int tree, const std::vector<int> &need,
                         const std::vector<double> &packed) {
    for (int &m : t->mask_slot) {
        if (m >= 0) ctx->mask_free.push_back(m);
        m = -1;
    }
    const long long ni = ctx->nint;
    const int dim = ctx->cfg.dim;
    {
        const int st = grow_mask_pool(ctx, (int)need.size());
        if (st) return st;
    }
    // double-float copy for the FP32-pipe stage: chi/C_eta (colour 0 -> 0),
    // u_s (three words, the third zero in 2D), sponge/C_sponge
    std::vector<float2> packed_df;
    if (ctx->precision == WG_RHS_FP32) {
        packed_df.resize(need.size() * 5 * ni);
        for (size_t k = 0; k < need.size(); k++) {
            const double *m = packed.data() + k * 6 * ni;
            float2 *o = packed_df.data() + k * 5 * ni;
            for (long long i = 0; i < ni; i++) {
                float f[2];
                const double vals[5] = {(int)m[4 * ni + i] == 0 ? 0.0 : m[i] * t->tp.C_eta_inv, m[ni + i],
                                        m[2 * ni + i], dim == 3 ? m[3 * ni + i] : 0.0,
                                        m[5 * ni + i] * t->tp.C_sponge_inv};
                for (int w = 0; w < 5; w++) {
                    split_df(vals[w], f);
                    o[w * ni + i] = make_float2(f[0], f[1]);
                }
            }
        }
    }
    for (size_t k = 0; k < need.size(); k++) {
        const int slot = ctx->mask_free.back();
        ctx->mask_free.pop_back();
        t->mask_slot[need[k]] = slot;
        WG_CUDA_OK(cudaMemcpyAsync(ctx->mask + (size_t)slot * 6 * ni, packed.data() + k * 6 * ni,
                                   sizeof(double) * 6 * ni, cudaMemcpyHostToDevice, ctx->stream));
        if (!packed_df.empty())
            WG_CUDA_OK(cudaMemcpyAsync(ctx->mask_df + (size_t)slot * 5 * ni, packed_df.data() + k * 5 * ni,
                                       sizeof(float2) * 5 * ni, cudaMemcpyHostToDevice, ctx->stream));
    }
    int st;
    if ((st = upload_desc(ctx, *t, tree))) return st;
    if ((st = upload_lists(ctx, *t))) return st;
    WG_CUDA_OK(cudaStreamSynchronize(ctx->stream));
    ctx->grid_version++;
    return WG_OK;
}

// host_mask: nblk * 6 * npts (reference layout hvy_mask) or NULL to drop it
int wg_set_mask(wg_ctx *ctx, int tree, const double *host_mask) {
    Tree *t = get_tree(ctx, tree);
    if (!t) return tree_err();
    if (!host_mask) return wg_set_mask_sparse(ctx, tree, 0, nullptr, nullptr);
    std::vector<int> ids(t->forest.size());
    for (size_t i = 0; i < ids.size(); i++) ids[i] = (int)i;
    return wg_set_mask_sparse(ctx, tree, (int)ids.size(), ids.data(), host_mask);
}

// Masks of every block of a tree drawn from its geometry (createMask_tree
// after each grid change, LIB/MESH/createMask_tree.f90:118-136), computed
// on the host pool and installed for the blocks that carry a non-zero word.
static int regen_masks(wg_ctx *ctx, Tree *t, int tree) {
    if (!t->has_geom) return WG_OK;
    const int nb = t->forest.size();
    const long long ni = ctx->nint;
    std::vector<char> any(nb, 0);
    std::vector<double> all((size_t)nb * 6 * ni);
    Pool::get().run(nb, [&](int b) {
        any[b] = geometry_mask_block(t->cfg, t->geom, t->forest.level[b], &t->forest.coords[3 * b],
                                     all.data() + (size_t)b * 6 * ni);
    });
    std::vector<int> need;
    std::vector<double> packed;
    for (int b = 0; b < nb; b++)
        if (any[b]) {
            need.push_back(b);
            packed.insert(packed.end(), all.begin() + (size_t)b * 6 * ni, all.begin() + (size_t)(b + 1) * 6 * ni);
        }
    return install_masks(ctx, t, tree, need, packed);
}

int wg_set_geometry(wg_ctx *ctx, int tree, const wg_geometry *geo) {
    Tree *t = get_tree(ctx, tree);
    if (!t) return tree_err();
    wg_geometry G{};
    if (geo) G = *geo;
    const char *why = geometry_check(t->cfg, G);
    if (*why) return fail(WG_EINVAL, "geometry: %s", why);
    cudaStreamSynchronize(ctx->stream);
    t->geom = G;
    t->has_geom = geo != nullptr;
    if (!t->has_geom) return install_masks(ctx, t, tree, {}, {});
    return regen_masks(ctx, t, tree);
}

// mask of a fixed sphere computed on the device: the blocks whose ghosted
// box comes within radius + h + 3 max(dx) of the centre are candidates,
// those with chi > 0 at an interior point get a mask slot (the selection of
// the workloads' host mask, create_mask.f90:58-61 -> draw_sphere)
int wg_set_mask_sphere(wg_ctx *ctx, int tree, const double *centre, double radius, double c_smooth) {
    Tree *t = get_tree(ctx, tree);
    if (!t) return tree_err();
    if (!centre || !(radius > 0.0) || !(c_smooth > 0.0)) return fail(WG_EINVAL, "bad arguments");
    if (ctx->cfg.dim != 3) return fail(WG_ENOTSUP, "sphere mask needs a 3-D context");
    cudaStreamSynchronize(ctx->stream);
    t->has_geom = false;
    for (int &m : t->mask_slot) {
        if (m >= 0) ctx->mask_free.push_back(m);
        m = -1;
    }
    const wg_config &c = t->cfg;
    const int g = ctx->cfg.g;
    const int *Bs = ctx->cfg.Bs;
    SphereArgs a;
    double dx_min = 0.0;
    for (int d = 0; d < 3; d++) {
        a.centre[d] = centre[d];
        a.domain[d] = c.domain[d];
        a.Bs[d] = Bs[d];
        const double v = std::ldexp(1.0, -c.Jmax) * c.domain[d] / Bs[d];
        dx_min = d == 0 ? v : std::min(dx_min, v);
    }
    a.radius = radius;
    a.h = c_smooth * dx_min;
    // candidates by the distance of the ghosted block box to the centre
    std::vector<int4> cand;
    std::vector<int> cblk;
    const int nb = t->forest.size();
    for (int b = 0; b < nb; b++) {
        const int lv = t->forest.level[b];
        double d2 = 0.0, dxmax = 0.0;
        for (int d = 0; d < 3; d++) {
            const double dx = std::ldexp(1.0, -lv) * c.domain[d] / Bs[d];
            const double x0 = (double)(t->forest.coords[3 * b + d] * Bs[d]) * dx;
            const double lo = x0 - g * dx, hi = x0 + (Bs[d] + g) * dx;
            const double e = std::max({lo - centre[d], 0.0, centre[d] - hi});
            d2 += e * e;
            dxmax = std::max(dxmax, dx);
        }
        if (std::sqrt(d2) > radius + a.h + 3.0 * dxmax) continue;
        cand.push_back(make_int4(lv, t->forest.coords[3 * b], t->forest.coords[3 * b + 1], t->forest.coords[3 * b + 2]));
        cblk.push_back(b);
    }
    std::vector<int> need;
    std::vector<int4> ncand;
    if (!cand.empty()) {
        DevArray<int4> d_cand;
        DevArray<int> d_flags;
        std::vector<int> flags(cand.size(), 0);
        cudaError_t e = d_cand.upload(cand.data(), cand.size(), ctx->stream);
        if (e == cudaSuccess) e = d_flags.upload(nullptr, cand.size(), ctx->stream);
        if (e == cudaSuccess) e = launch_sphere_flags(d_cand.p, (int)cand.size(), a, d_flags.p, ctx->stream);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(flags.data(), d_flags.p, sizeof(int) * flags.size(), cudaMemcpyDeviceToHost, ctx->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
        if (e != cudaSuccess) return cuda_fail(e, "wg_set_mask_sphere", __FILE__, __LINE__);
        for (size_t k = 0; k < cand.size(); k++)
            if (flags[k]) {
                need.push_back(cblk[k]);
                ncand.push_back(cand[k]);
            }
    }
    int st = grow_mask_pool(ctx, (int)need.size());
    if (st) return st;
    if (!need.empty()) {
        std::vector<int> slots(need.size());
        for (size_t k = 0; k < need.size(); k++) {
            slots[k] = ctx->mask_free.back();
            ctx->mask_free.pop_back();
            t->mask_slot[need[k]] = slots[k];
        }
        DevArray<int4> d_cand;
        DevArray<int> d_slot;
        cudaError_t e = d_cand.upload(ncand.data(), ncand.size(), ctx->stream);
        if (e == cudaSuccess) e = d_slot.upload(slots.data(), slots.size(), ctx->stream);
        if (e == cudaSuccess)
            e = launch_sphere_fill(d_cand.p, d_slot.p, (int)need.size(), a, ctx->mask,
                                   ctx->precision == WG_RHS_FP32 ? ctx->mask_df : nullptr, t->tp.C_eta_inv,
                                   ctx->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
        if (e != cudaSuccess) return cuda_fail(e, "wg_set_mask_sphere", __FILE__, __LINE__);
    }
    if ((st = upload_desc(ctx, *t, tree))) return st;
    if ((st = upload_lists(ctx, *t))) return st;
    WG_CUDA_OK(cudaStreamSynchronize(ctx->stream));
    ctx->grid_version++;
    return WG_OK;
}

// interior mask of one block (6 * Bs^d doubles, components chi, u_s x3,
// colour, sponge) for inspection: returns 1 and fills out when the block has
// a mask, 0 when it has none
int wg_get_mask_block(wg_ctx *ctx, int tree, int block, double *out) {
    Tree *t = get_tree(ctx, tree);
    if (!t) return tree_err();
    if (!out || block < 0 || block >= t->forest.size()) return fail(WG_EINVAL, "bad arguments");
    const int slot = t->mask_slot[block];
    if (slot < 0) return 0;
    const long long ni = ctx->nint;
    WG_CUDA_OK(cudaMemcpyAsync(out, ctx->mask + (size_t)slot * 6 * ni, sizeof(double) * 6 * ni,
                               cudaMemcpyDeviceToHost, ctx->stream));
    WG_CUDA_OK(cudaStreamSynchronize(ctx->stream));
    return 1;
}

int wg_set_time(wg_ctx *ctx, int tree, double time) {
    Tree *t = get_tree(ctx, tree);
    if (!t) return tree_err();
    const TreeClock c = fresh_clock(time);
    // time, dt and the divergence flag; the anchoring constant and running
    // max of the stage inputs stay (they describe the state, not the clock)
    WG_CUDA_OK(cudaMemcpyAsync(ctx->d_clk + tree, &c, offsetof(TreeClock, anchor_M), cudaMemcpyHostToDevice,
                               ctx->stream));
    WG_CUDA_OK(cudaStreamSynchronize(ctx->stream));
    return WG_OK;
}

int wg_get_time(wg_ctx *ctx, int tree, double *time, double *dt) {
    Tree *t = get_tree(ctx, tree);
    if (!t) return tree_err();
    TreeClock c;
    int st = read_clock(ctx, tree, &c);
    if (st) return st;
    if ((st = check_dev_err(ctx))) return st;
    if (time) *time = c.time;
    if (dt) *dt = c.dt;
    return c.diverged ? fail(WG_EDIVERGED, "ACM fail: very very large values in state vector") : WG_OK;
}

// sync_ghosts_RHS_tree / sync_ghosts_tree on the state (no HD filter)
int wg_sync_ghosts(wg_ctx *ctx, int tree, int gminus, int gplus) {
    Tree *t = get_tree(ctx, tree);
    if (!t) return tree_err();
    if (gminus < 1 || gplus < 1 || gminus > ctx->cfg.g || gplus > ctx->cfg.g)
        return fail(WG_EINVAL, "ghost widths must be in 1..g");
    int st = run_sync(ctx, *t, ctx->A, false, gminus, gplus);
    if (st) return st;
    WG_CUDA_OK(cudaStreamSynchronize(ctx->stream));
    return WG_OK;
}

// RHS_ACM local stage of every block on the current (synchronised) state;
// host_rhs receives nblk*neq*npts doubles (reference layout, interior set)
int wg_rhs(wg_ctx *ctx, int tree, double *host_rhs) {
    Tree *t = get_tree(ctx, tree);
    if (!t) return tree_err();
    if (!host_rhs) return fail(WG_EINVAL, "bad arguments");
    const size_t per = sizeof(double) * ctx->geo.nc * ctx->gA.npts();
    double *d = nullptr;
    WG_CUDA_OK(cudaMallocAsync(&d, per * ctx->max_blocks, ctx->stream));
    cudaMemsetAsync(d, 0, per * ctx->max_blocks, ctx->stream);
    const int base = (ctx->variant_fast ? 1 : 0) | (t->cfg.skew_symmetry ? 2 : 0);
    const int *Bs = ctx->cfg.Bs;
    cudaError_t e = launch_rhs_only(base, ctx->cfg.dim, t->d_plain.p, t->n_plain, ctx->d_desc, ctx->d_tp, ctx->A,
                                    ctx->gA, d, ctx->mask, Bs[0], Bs[1], Bs[2], ctx->geo.nc, ctx->stream);
    if (e == cudaSuccess)
        e = launch_rhs_only(base | 4, ctx->cfg.dim, t->d_masked.p, t->n_masked, ctx->d_desc, ctx->d_tp, ctx->A,
                            ctx->gA, d, ctx->mask, Bs[0], Bs[1], Bs[2], ctx->geo.nc, ctx->stream);
    for (size_t b = 0; e == cudaSuccess && b < t->slots.size(); b++)
        e = cudaMemcpyAsync((char *)host_rhs + per * b, (const char *)d + per * t->slots[b], per,
                            cudaMemcpyDeviceToHost, ctx->stream);
    cudaFreeAsync(d, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) return cuda_fail(e, "wg_rhs", __FILE__, __LINE__);
    return WG_OK;
}

// calculate_time_step at the tree's current time (state must be synced)
int wg_compute_dt(wg_ctx *ctx, int tree, double *dt) {
    Tree *t = get_tree(ctx, tree);
    if (!t) return tree_err();
    const int *Bs = ctx->cfg.Bs;
    WG_CUDA_OK(launch_dt(ctx->cfg.dim, t->d_all.p, (int)t->slots.size(), ctx->d_desc, ctx->d_tp, ctx->d_clk, ctx->A,
                         ctx->gA, Bs[0], Bs[1], Bs[2], 1, ctx->d_tree_ids.p + tree, dt_done(ctx), ctx->stream));
    TreeClock c;
    int st = read_clock(ctx, tree, &c);
    if (st) return st;
    if (dt) *dt = c.dt;
    return WG_OK;
}

// timeStep_tree: one RK4 step (sync, dt, four stages); time and dt are
// returned when the pointers are non-NULL (which synchronises)
int wg_rk4_step(wg_ctx *ctx, int tree, double *time, double *dt) {
    Tree *t = get_tree(ctx, tree);
    if (!t) return tree_err();
    // the stage-kernel form is chosen before the first step (stage buffers
    // C and D are scratch at this point)
    int st = autotune_stage_form(ctx, *t);
    if (st) return st;
    st = ensure_shadow(ctx, *t);
    if (st) return st;
    st = rk4_enqueue(ctx, tree);
    if (st) return st;
    if (time || dt) return wg_get_time(ctx, tree, time, dt);
    return WG_OK;
}

// nsteps RK4 steps of each listed tree without host synchronisation; with
// use_graph the per-step launch sequence is captured once and replayed
int wg_run(wg_ctx *ctx, int ntrees, const int *trees, int nsteps, int use_graph) {
    if (!ctx || ntrees <= 0 || !trees || nsteps < 0) return fail(WG_EINVAL, "bad arguments");
    if (ctx->dead) return fail(WG_ETIMEOUT, "the context is unusable after a timed-out device wait; destroy it");
    for (int i = 0; i < ntrees; i++) {
        Tree *t = get_tree(ctx, trees[i]);
        if (!t) return tree_err();
        for (int k = 0; k < i; k++)
            if (trees[k] == trees[i]) return fail(WG_EINVAL, "tree %d listed twice", trees[i]);
        int st = ensure_shadow(ctx, *t);
        if (st) return st;
    }
    // the FP32-pipe precision steps all listed trees with one launch per
    // kernel (batched); the FP64 precision tree by tree
    const bool batched = ctx->precision == WG_RHS_FP32;
    if (batched) {
        int st = build_batch(ctx, std::vector<int>(trees, trees + ntrees));
        if (st) return st;
    }
    if (!use_graph) {
        for (int s = 0; s < nsteps; s++) {
            if (batched) {
                int st = rk4_enqueue_batch(ctx);
                if (st) return st;
                continue;
            }
            for (int i = 0; i < ntrees; i++) {
                int st = rk4_enqueue(ctx, trees[i]);
                if (st) return st;
            }
        }
        return WG_OK;
    }
    const bool same = ctx->graph_exec && ctx->graph_version == ctx->grid_version &&
                      ctx->graph_trees == std::vector<int>(trees, trees + ntrees);
    if (!same) {
        // tables are built (and uploaded) before capture
        for (int i = 0; i < ntrees; i++) {
            Tree &t = ctx->trees[trees[i]];
            SyncPlan *sp;
            int st;
            if ((st = get_sync(ctx, t, ctx->cfg.g_rhs, ctx->cfg.g_rhs, false, &sp))) return st;
            if ((st = get_sync(ctx, t, ctx->cfg.g_rhs, ctx->cfg.g_rhs, true, &sp))) return st;
        }
        for (int i = 0; i < ntrees; i++) {
            int st = autotune_stage_form(ctx, ctx->trees[trees[i]]);
            if (st) return st;
        }
        WG_CUDA_OK(cudaStreamSynchronize(ctx->stream));
        if (ctx->graph_exec) cudaGraphExecDestroy(ctx->graph_exec);
        if (ctx->graph) cudaGraphDestroy(ctx->graph);
        ctx->graph_exec = nullptr;
        ctx->graph = nullptr;
        WG_CUDA_OK(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
        int st = WG_OK;
        if (batched) st = rk4_enqueue_batch(ctx);
        for (int i = 0; i < ntrees && !st && !batched; i++) st = rk4_enqueue(ctx, trees[i]);
        cudaGraph_t g = nullptr;
        cudaError_t e = cudaStreamEndCapture(ctx->stream, &g);
        if (st) {
            if (g) cudaGraphDestroy(g);
            return st;
        }
        if (e != cudaSuccess) return cuda_fail(e, "cudaStreamEndCapture", __FILE__, __LINE__);
        ctx->graph = g;
        WG_CUDA_OK(cudaGraphInstantiate(&ctx->graph_exec, g, 0));
        ctx->graph_trees.assign(trees, trees + ntrees);
        ctx->graph_version = ctx->grid_version;
    }
    for (int s = 0; s < nsteps; s++) WG_CUDA_OK(cudaGraphLaunch(ctx->graph_exec, ctx->stream));
    return WG_OK;
}

// waveletDecomposition_optimized_block / waveletReconstruction_optimized_block
// of every block of the tree, in place on the state; wc_threshold_tree
int wg_wavelet_decompose(wg_ctx *ctx, int tree) {
    Tree *t = get_tree(ctx, tree);
    if (!t) return tree_err();
    const int *Bs = ctx->cfg.Bs;
    WG_CUDA_OK(launch_wavelet_decompose(ctx->cfg.dim, t->d_all.p, (int)t->slots.size(), ctx->A, ctx->gA, Bs[0], Bs[1],
                                        Bs[2], ctx->geo.nc, ctx->wav.X, ctx->wav.Y, ctx->stream));
    if (const int sc = state_changed(ctx, t, tree)) return sc;
    WG_CUDA_OK(cudaStreamSynchronize(ctx->stream));
    return WG_OK;
}

int wg_wavelet_reconstruct(wg_ctx *ctx, int tree) {
    Tree *t = get_tree(ctx, tree);
    if (!t) return tree_err();
    const int *Bs = ctx->cfg.Bs;
    WG_CUDA_OK(launch_wavelet_reconstruct(ctx->cfg.dim, t->d_all.p, (int)t->slots.size(), ctx->A, ctx->gA, Bs[0],
                                          Bs[1], Bs[2], ctx->geo.nc, ctx->wav.X, ctx->wav.Y, ctx->stream));
    if (const int sc = state_changed(ctx, t, tree)) return sc;
    WG_CUDA_OK(cudaStreamSynchronize(ctx->stream));
    return WG_OK;
}

int wg_wavelet_threshold(wg_ctx *ctx, int tree, const double *thresh) {
    Tree *t = get_tree(ctx, tree);
    if (!t) return tree_err();
    if (!thresh) return fail(WG_EINVAL, "bad arguments");
    if (ctx->geo.nc > 8) return fail(WG_ENOTSUP, "at most 8 components");
    const int *Bs = ctx->cfg.Bs;
    WG_CUDA_OK(launch_wc_threshold(ctx->cfg.dim, t->d_all.p, (int)t->slots.size(), ctx->A, ctx->gA, Bs[0], Bs[1],
                                   Bs[2], ctx->geo.nc, thresh, t->cfg.threshold_state_vector_component, ctx->stream));
    if (const int sc = state_changed(ctx, t, tree)) return sc;
    WG_CUDA_OK(cudaStreamSynchronize(ctx->stream));
    return WG_OK;
}

int wg_set_stage_form(wg_ctx *ctx, int form) {
    if (!ctx) return fail(WG_EINVAL, "null ctx");
    if (form < WG_FORM_AUTO || form > WG_FORM_TILE8) return fail(WG_EINVAL, "unknown stage form %d", form);
    if ((form == WG_FORM_TILE2 || form == WG_FORM_TILE8) && !ctx->have_slabs28)
        return fail(WG_ENOTSUP, "slabs of 2 and 8 planes need the tile form and Bs2 a multiple of 8");
    if ((form == WG_FORM_TILE || form == WG_FORM_PIPE) && !ctx->have_tm)
        return fail(WG_ENOTSUP, "the tile and pipe forms need 3-D 16x16 planes, g_rhs = 2 and the FP32-pipe precision");
    if (form == WG_FORM_MARCH && !ctx->have_march)
        return fail(WG_ENOTSUP, "the march form needs 3-D 16^3 blocks, g_rhs = 2 and the FP32-pipe precision");
    ctx->stage_form = form;
    for (int &f : ctx->tuned) f = 0;
    ctx->graph_version = -1;   // recapture with the new form
    return WG_OK;
}

int wg_set_stage_forms(wg_ctx *ctx, const int *forms) {
    if (!ctx || !forms) return fail(WG_EINVAL, "bad arguments");
    for (int k = 0; k < 4; k++) {
        if (forms[k] < WG_FORM_DIRECT || forms[k] > WG_FORM_TILE8)
            return fail(WG_EINVAL, "stage %d: form %d is not direct, tile, march, pipe, tile2 or tile8", k + 1,
                        forms[k]);
        if (((forms[k] == WG_FORM_TILE || forms[k] == WG_FORM_PIPE) && !ctx->have_tm) ||
            ((forms[k] == WG_FORM_TILE2 || forms[k] == WG_FORM_TILE8) && !ctx->have_slabs28) ||
            (forms[k] == WG_FORM_MARCH && !ctx->have_march))
            return fail(WG_ENOTSUP, "stage %d: form %d does not apply to this configuration", k + 1, forms[k]);
    }
    ctx->stage_form = WG_FORM_AUTO;
    for (int k = 0; k < 4; k++) ctx->tuned[k] = forms[k];   // as if the autotuner had chosen them
    ctx->graph_version = -1;
    return WG_OK;
}

int wg_get_stage_form(wg_ctx *ctx, int *form) {
    if (!ctx || !form) return fail(WG_EINVAL, "bad arguments");
    *form = form_of(ctx, 2);
    return WG_OK;
}

int wg_get_stage_forms(wg_ctx *ctx, int *forms) {
    if (!ctx || !forms) return fail(WG_EINVAL, "bad arguments");
    for (int k = 0; k < 4; k++) forms[k] = form_of(ctx, k + 1);
    return WG_OK;
}

int wg_synchronize(wg_ctx *ctx) {
    if (!ctx) return fail(WG_EINVAL, "null ctx");
    if (ctx->dead) return fail(WG_ETIMEOUT, "the context is unusable after a timed-out device wait; destroy it");
    WG_CUDA_OK(cudaStreamSynchronize(ctx->stream));
    return check_dev_err(ctx);
}

// the context's stream, for callers that time or order work around it
void *wg_stream(wg_ctx *ctx) { return ctx ? (void *)ctx->stream : nullptr; }

// coarseningIndicator for every block of the tree on the current state
// (ghosts synchronised with g points first): flags[b] = -1 (may coarsen) or
// 0; details (nblk*neq, may be NULL) receives the per-component details
static int threshold_flags(wg_ctx *ctx, int tree, const double *eps_use, int *flags, double *details, int input_is_wd) {
    Tree *t = get_tree(ctx, tree);
    if (!t) return tree_err();
    if (!eps_use || !flags) return fail(WG_EINVAL, "bad arguments");
    const int nb = t->forest.size();
    const int nc = ctx->geo.nc;
    double *d_det = nullptr;
    int *d_flags = nullptr;
    cudaError_t e = cudaMallocAsync(&d_flags, sizeof(int) * (nb + 1), ctx->stream);
    if (e == cudaSuccess) e = cudaMallocAsync(&d_det, sizeof(double) * (nb + 1) * nc, ctx->stream);
    const int *Bs = ctx->cfg.Bs;
    if (e == cudaSuccess)
        e = launch_fwt_flags(ctx->cfg.dim, t->d_all.p, nb, ctx->A, ctx->gA, Bs[0], Bs[1], Bs[2], nc, ctx->wav.X,
                             ctx->wav.Y, eps_use, t->cfg.threshold_state_vector_component, d_flags, d_det,
                             ctx->stream, input_is_wd);
    if (e == cudaSuccess) e = cudaMemcpyAsync(flags, d_flags, sizeof(int) * nb, cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess && details)
        e = cudaMemcpyAsync(details, d_det, sizeof(double) * nb * nc, cudaMemcpyDeviceToHost, ctx->stream);
    cudaFreeAsync(d_flags, ctx->stream);
    cudaFreeAsync(d_det, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) return cuda_fail(e, "wg_threshold_flags", __FILE__, __LINE__);
    return WG_OK;
}

int wg_threshold_flags(wg_ctx *ctx, int tree, const double *eps_use, int *flags, double *details) {
    return threshold_flags(ctx, tree, eps_use, flags, details, 0);
}

// coarseningIndicator_tree(..., input_is_WD=.true.): the state already holds
// the one-level decomposition (wg_wavelet_decompose), the details are read
// from it without a second FWT
int wg_threshold_flags_wd(wg_ctx *ctx, int tree, const double *eps_use, int *flags, double *details) {
    return threshold_flags(ctx, tree, eps_use, flags, details, 1);
}

// adapt_tree (LIB/MESH/adapt_tree.f90:11-255) for unlifted wavelets (CDF X0,
// no coarse extension and no security zone): the full tree of the grid is
// built on the host (adapt.cpp); the mothers, level by level from the
// finest, receive their daughters' scaling coefficients (sync_D2M: every
// second interior point for CDF X0) and the same-level neighbours' values as
// ghost nodes; every block of the full tree is flagged by the coarsening
// indicator on its own data (the leaves after a sync with g layers); the
// host makes the flags consistent (Jmin, completeness, daughters,
// gradedness) and keeps the blocks that remain without remaining daughters.
// Their data is already in their slots: the old leaves' untouched, the
// promoted mothers' from their daughters. Masks are dropped (they depend on
// the grid and are set again by the caller). Ends with a ghost sync.
// adapt_tree for lifted wavelets (LIB/MESH/adapt_tree.f90:11-255): full-tree
// decomposition with coarse extension, indicator on the decomposition,
// security zone, flag consistency, deletion, reconstruction of the blocks at
// coarse/fine interfaces, pruning and the final filtered sync. The host
// plans every step (lifted.cpp); the data stays in A (hvy_block) and the
// slot-indexed hvy_tmp arena T.
// The two switches of coarseningIndicator_tree applied to the block
// indicator's flags of the full tree: force_maxlevel_dealiasing flags every
// block on Jmax for coarsening (LIB/MESH/coarseningIndicator_tree.f90:
// 287-293) and threshold_mask keeps the blocks whose mask has an interface
// (coarseningIndicatorMask_tree, :333-420; the mask status comes from the
// tree's geometry on the host pool).
static void indicator_switches(const Tree &t, const FullTree &ft, std::vector<int> &flags) {
    const wg_config &c = t.cfg;
    const bool by_mask = c.threshold_mask && t.has_geom && c.penalization;
    if (!c.force_maxlevel_dealiasing && !by_mask) return;
    Pool::get().run(ft.size(), [&](int b) {
        if (c.force_maxlevel_dealiasing && ft.level[b] == c.Jmax) {
            flags[b] = kFlagCoarsen;
            return;
        }
        if (by_mask) flags[b] = std::max(flags[b], geometry_mask_status(c, t.geom, ft.level[b], &ft.coords[3 * b]));
    });
}

// eps * norm per component (adapt_tree / coarseningIndicator_tree with
// eps_normalized: componentWiseNorm_tree's Linfty over the leaves, a norm
// <= 1e-9 replaced by 1, coarseningIndicator_tree.f90:133-152), or eps.
static int adapt_thresholds(wg_ctx *ctx, Tree *t, std::vector<double> &eps_use) {
    const int nc = ctx->geo.nc;
    const wg_config &c = t->cfg;
    eps_use.assign(nc, c.eps);
    if (!c.eps_normalized) return WG_OK;
    DevArray<double> d_norm;
    std::vector<double> norm(nc, 0.0);
    cudaError_t e = d_norm.upload(nullptr, nc, ctx->stream);
    if (e == cudaSuccess)
        e = launch_norm_linf(t->d_all.p, t->forest.size(), ctx->A, ctx->gA, ctx->cfg.Bs[0], ctx->cfg.Bs[1],
                             ctx->cfg.dim == 3 ? ctx->cfg.Bs[2] : 1, nc, d_norm.p, ctx->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(norm.data(), d_norm.p, sizeof(double) * nc, cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) return cuda_fail(e, "adapt norm", __FILE__, __LINE__);
    for (int p = 0; p < nc; p++) {
        double n = c.threshold_state_vector_component[p] == 1 ? norm[p] : -1.0;
        if (n <= 1.0e-9) n = 1.0;
        eps_use[p] = c.eps * n;
    }
    return WG_OK;
}

static int adapt_lifted(wg_ctx *ctx, Tree *t, int tree, const double *eps_use, bool thr, int *nblk_out) {
    const int dim = ctx->cfg.dim, nc = ctx->geo.nc, g = ctx->cfg.g;
    const int *Bs = ctx->cfg.Bs;
    const int nb = t->forest.size();
    const WaveletInfo &w = ctx->wav;
    const BufGeo gA = ctx->gA;
    const long long per_block = (long long)nc * gA.npts();
    WG_CUDA_OK(cudaStreamSynchronize(ctx->stream));
    LiftedTree L;
    std::string err;
    if (!L.init(ctx->geo, w, 2, t->cfg.Jmin, t->cfg.Jmax, nb, t->forest.level.data(), t->forest.coords.data(), err))
        return fail(WG_EGRID, "adapt: %s", err.c_str());
    bool leaf_only = true, recon_nb = false, leaf_first = true;
    const int hd_hi = w.hd_lo + (int)w.HD.size() - 1;
    for (int d = 0; d < dim; d++) {
        if (Bs[d] < L.Ndep2l || Bs[d] < L.Ndep2r) leaf_only = false;
        if (Bs[d] < L.Nreconl || Bs[d] < L.Nreconr) recon_nb = true;
        if (Bs[d] < 3 * std::max(std::abs(w.hd_lo), std::abs(hd_hi))) leaf_first = false;
    }
    if (recon_nb) return fail(WG_ENOTSUP, "lifted adapt with Bs below the coarse-extension reconstruction width");
    const int nt = L.size();
    if ((size_t)(nt - nb) > ctx->free_slots.size())
        return fail(WG_ENOMEM, "adapt needs %d free slots for the mothers (%zu free)", nt - nb, ctx->free_slots.size());
    if (!ctx->T) {
        const size_t bytes = sizeof(double) * (size_t)per_block * ctx->max_blocks;
        if (cudaMalloc(&ctx->T, bytes) != cudaSuccess) {
            cudaGetLastError();
            ctx->T = nullptr;
            return fail(WG_ENOMEM, "hvy_tmp arena of %zu bytes", bytes);
        }
    }
    for (int b = 0; b < nb; b++) L.slot[b] = t->slots[b];
    for (int b = nb; b < nt; b++) L.slot[b] = ctx->free_slots.take();
    // device lists from the context's scratch arena, alive until the end
    // (the stream is synchronised there and before the next reset); a null
    // list makes its launcher fail
    cudaStreamSynchronize(ctx->stream);
    ctx->scratch.reset();
    auto up = [&](const auto &v) {
        using E = typename std::decay<decltype(*v.data())>::type;
        E *p = static_cast<E *>(ctx->scratch.alloc(sizeof(E) * v.size()));
        if (p && !v.empty() &&
            cudaMemcpyAsync(p, v.data(), sizeof(E) * v.size(), cudaMemcpyHostToDevice, ctx->stream) != cudaSuccess)
            p = nullptr;
        return p;
    };
    // phase timing (wg_adapt_profile): host planning, then device phases
    // bracketed by stream synchronisations
    enum { kPlan, kSync, kFwt, kCe, kFlags, kRecon, kCopy, kTotal };
    std::fill(ctx->adapt_ms, ctx->adapt_ms + 8, 0.0);
    using clk = std::chrono::steady_clock;
    const auto t_start = clk::now();
    auto tic = [&]() {
        if (ctx->adapt_profile) cudaStreamSynchronize(ctx->stream);
        return clk::now();
    };
    auto toc = [&](int phase, clk::time_point t0) {
        if (ctx->adapt_profile) cudaStreamSynchronize(ctx->stream);
        ctx->adapt_ms[phase] += std::chrono::duration<double, std::milli>(clk::now() - t0).count();
    };
    cudaError_t e = cudaSuccess;
    const int hx = Bs[0] / 2, hy = Bs[1] / 2, hz = dim == 3 ? Bs[2] / 2 : 1;
    // one device list from the same list of every part of a wave (or of
    // the wave itself): one copy per part into consecutive scratch memory
    auto gather = [&](const std::vector<const SyncWave *> &ps, auto mem, int &n) {
        using E = typename std::decay<decltype(*(ps[0]->*mem).data())>::type;
        size_t tot = 0;
        for (const SyncWave *q : ps) tot += (q->*mem).size();
        n = (int)tot;
        E *d = tot ? static_cast<E *>(ctx->scratch.alloc(sizeof(E) * tot)) : nullptr;
        size_t at = 0;
        for (const SyncWave *q : ps) {
            const auto &v = q->*mem;
            if (d && !v.empty() &&
                cudaMemcpyAsync(d + at, v.data(), sizeof(E) * v.size(), cudaMemcpyHostToDevice, ctx->stream) != cudaSuccess)
                d = nullptr;
            at += v.size();
        }
        return d;
    };
    auto run_waves = [&](const std::vector<SyncWave> &waves) -> cudaError_t {
        for (const SyncWave &wv : waves) {
            std::vector<const SyncWave *> ps;
            if (wv.parts.empty()) ps.push_back(&wv);
            for (const SyncWave &q : wv.parts) ps.push_back(&q);
            cudaError_t r = cudaSuccess;
            int n = 0;
            const Patch *cb = gather(ps, &SyncWave::copy_blk, n);
            if (n) r = launch_xcopy(cb, n, ctx->A, ctx->A, gA, nc, ctx->stream);
            const Patch *ct = gather(ps, &SyncWave::copy_tmp, n);
            if (r == cudaSuccess && n) r = launch_xcopy(ct, n, ctx->T, ctx->A, gA, nc, ctx->stream);
            int nr = 0, nf = 0, ns = 0;
            for (const SyncWave *q : ps) nr += (int)q->restrict_.size();
            if (r == cudaSuccess && nr) {
                // every restricted point lies on the sender's interior SC lattice
                for (const SyncWave *q : ps)
                    for (const Patch &p : q->restrict_)
                        for (int d = 0; d < dim; d++) {
                            const int a = p.slo[d] + 2 * p.blo[d], z = a + 2 * (p.rhi[d] - p.rlo[d]);
                            if (((a - g) & 1) || a < g || z > g + Bs[d] - 2) return cudaErrorInvalidValue;
                        }
                const FilterEntry *fe = gather(ps, &SyncWave::filters, nf);
                const ScBox *sb = gather(ps, &SyncWave::ce_copies, ns);
                const Patch *rp = gather(ps, &SyncWave::restrict_, nr);
                double *scratch = static_cast<double *>(ctx->scratch.alloc(sizeof(double) * nf * nc * hx * hy * hz));
                r = launch_hd_filter(dim, fe, nf, ctx->A, ctx->T, gA, Bs[0], Bs[1], Bs[2], nc, w.HD.data(), w.hd_lo,
                                     (int)w.HD.size(), scratch, ctx->stream);
                if (r == cudaSuccess && ns)
                    r = launch_scbox(sb, ns, fe, ctx->A, ctx->T, gA, hx, hy, hz, nc, scratch, ctx->stream);
                if (r == cudaSuccess)
                    r = launch_restrict_scratch(rp, nr, scratch, ctx->A, gA, hx, hy, hz, nc, ctx->stream);
            }
            if (r == cudaSuccess && !wv.pred_blk.empty())
                r = launch_predict(up(wv.pred_blk), (int)wv.pred_blk.size(), wv.max_coarse, ctx->A, gA, nc,
                                   w.order_predictor, ctx->stream, ctx->A);
            if (r == cudaSuccess && !wv.pred_tmp.empty())
                r = launch_predict(up(wv.pred_tmp), (int)wv.pred_tmp.size(), wv.max_coarse, ctx->A, gA, nc,
                                   w.order_predictor, ctx->stream, ctx->T);
            if (r != cudaSuccess) return r;
        }
        return cudaSuccess;
    };
    auto sync_spec = [&](SyncSpecL sp) -> cudaError_t {
        std::vector<SyncWave> waves;
        auto t0 = clk::now();
        L.plan_sync(sp, waves);
        ctx->adapt_ms[kPlan] += std::chrono::duration<double, std::milli>(clk::now() - t0).count();
        t0 = tic();
        const cudaError_t r = run_waves(waves);
        toc(kSync, t0);
        return r;
    };
    auto ce = [&](int ce_case, int s_level, int s_ref, bool clear_wc, bool copy_sc) -> cudaError_t {
        std::vector<BoxOp> ops;
        auto t0 = clk::now();
        L.plan_ce_modify(ce_case, s_level, s_ref, clear_wc, copy_sc, ops);
        ctx->adapt_ms[kPlan] += std::chrono::duration<double, std::milli>(clk::now() - t0).count();
        if (ops.empty()) return cudaSuccess;
        t0 = tic();
        const cudaError_t r = launch_boxop(up(ops), (int)ops.size(), ctx->A, ctx->T, gA, nc, ctx->stream);
        toc(kCe, t0);
        return r;
    };
    auto slots_where = [&](auto pred) {
        std::vector<int> v;
        for (int b = 0; b < nt; b++)
            if (L.alive[b] && pred(b)) v.push_back(L.slot[b]);
        return v;
    };
    auto fail_restore = [&](cudaError_t ce2, int st) {
        cudaStreamSynchronize(ctx->stream);
        for (int b = nb; b < nt; b++) ctx->free_slots.give(L.slot[b]);
        if (ce2 != cudaSuccess) return cuda_fail(ce2, "wg_adapt (lifted)", __FILE__, __LINE__);
        return st;
    };
    // the leaf grid's filtered sync (sync_ghosts_tree)
    for (int b = 0; b < nt; b++) L.alive[b] = b < nb;
    auto meta = [&]() {
        const auto t0 = clk::now();
        const bool ok = L.update_metadata(err);
        ctx->adapt_ms[kPlan] += std::chrono::duration<double, std::milli>(clk::now() - t0).count();
        return ok;
    };
    if (!meta()) return fail_restore(cudaSuccess, fail(WG_EGRID, "adapt: %s", err.c_str()));
    {
        SyncSpecL sp;
        sp.gminus = sp.gplus = g;
        if (e == cudaSuccess) e = sync_spec(sp);
    }
    // wavelet_decompose_full_tree
    std::fill(L.alive.begin(), L.alive.end(), 1);
    if (!meta()) return fail_restore(cudaSuccess, fail(WG_EGRID, "adapt: %s", err.c_str()));
    const int lmax = L.ft.max_level();
    for (int b = 0; b < nt; b++) L.ref[b] = b < nb ? ((L.ft.level[b] == lmax || leaf_first) ? -1 : 0) : kRefTmpEmpty;
    {
        std::vector<int> leaves(t->slots.begin(), t->slots.end());
        if (e == cudaSuccess) e = launch_blockcopy(up(leaves), nb, ctx->A, ctx->T, per_block, ctx->stream);
    }
    const int g_this = std::max(std::abs(w.hd_lo), w.gd_lo + (int)w.GD.size() - 1);
    for (int level = lmax, it = 0; level >= t->cfg.Jmin && e == cudaSuccess; level--, it++) {
        SyncSpecL sp;
        sp.base = (leaf_first && it == 0) ? 1 : 4;
        sp.by_ref = true;
        sp.s_ref = -1;
        sp.gminus = sp.gplus = g_this;
        sp.tmp_usage = 1;
        e = sync_spec(sp);
        const std::vector<int> dec = slots_where([&](int b) { return L.ref[b] == -1; });
        if (e == cudaSuccess && !dec.empty()) {
            const int *d_dec = up(dec);
            auto t0 = tic();
            e = launch_blockcopy(d_dec, (int)dec.size(), ctx->A, ctx->T, per_block, ctx->stream);
            toc(kCopy, t0);
            t0 = tic();
            if (e == cudaSuccess)
                e = launch_wavelet_decompose_window(dim, d_dec, (int)dec.size(), ctx->A, gA, Bs[0], Bs[1], Bs[2], nc,
                                                    w.X, w.Y, ctx->stream);
            toc(kFwt, t0);
        }
        if (e == cudaSuccess) e = ce(2, 0, -1, true, true);
        for (int b = 0; b < nt; b++) {
            if (L.ref[b] == -1) L.ref[b] = 0;
            if ((L.ref[b] == kRefTmpEmpty || !leaf_first) && L.ft.level[b] == level - 1) L.ref[b] = -1;
        }
        std::vector<Patch> d2m, gh;
        mother_patches(L.ft, ctx->geo, level - 1, L.slot, d2m, gh);
        auto t0 = tic();
        if (e == cudaSuccess && !d2m.empty())
            e = launch_sync(up(d2m), (int)d2m.size(), ctx->A, gA, nc, w.order_predictor, ctx->stream);
        toc(kCe, t0);
    }
    std::fill(L.ref.begin(), L.ref.end(), 0);
    // coarseningIndicator_tree on the decomposition, security zone
    std::vector<int> flags(nt, 0);
    const auto t_flags = tic();
    if (e == cudaSuccess && thr) {
        std::vector<int> all(L.slot.begin(), L.slot.end());
        std::vector<int> tsvc(t->cfg.threshold_state_vector_component, t->cfg.threshold_state_vector_component + nc);
        std::vector<double> eps(eps_use, eps_use + nc);
        const int *d_all = up(all);
        std::vector<int> zeros(nt, 0);
        int *d_flags = up(zeros);
        e = launch_fwt_flags(dim, d_all, nt, ctx->A, gA, Bs[0], Bs[1], Bs[2], nc, w.X, w.Y, eps.data(), tsvc.data(),
                             d_flags, nullptr, ctx->stream, 1);
        if (e == cudaSuccess) e = cudaMemcpyAsync(flags.data(), d_flags, sizeof(int) * nt, cudaMemcpyDeviceToHost, ctx->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
        if (e == cudaSuccess) {
            indicator_switches(*t, L.ft, flags);
            L.ref = flags;
            std::vector<LiftedTree::ZoneItem> items;
            L.security_candidates(items);
            if (!items.empty()) {
                std::vector<int> zb;
                for (const auto &z : items) {
                    zb.push_back(L.slot[z.block]);
                    for (int d = 0; d < 3; d++) zb.push_back(z.lo[d]);
                    for (int d = 0; d < 3; d++) zb.push_back(z.hi[d]);
                    for (int d = 0; d < 3; d++) zb.push_back(z.io[d]);
                }
                std::vector<double> det(items.size() * nc, 0.0);
                double *d_det = static_cast<double *>(ctx->scratch.alloc(sizeof(double) * det.size()));
                e = launch_zone_detail(up(zb), (int)items.size(), ctx->A, gA, nc, dim, d_det, ctx->stream);
                if (e == cudaSuccess)
                    e = cudaMemcpyAsync(det.data(), d_det, sizeof(double) * det.size(), cudaMemcpyDeviceToHost,
                                        ctx->stream);
                if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
                // threshold_block's component / vector-group rule
                std::vector<char> sig(items.size(), 0);
                int maxg = 0;
                for (int c = 0; c < nc; c++) maxg = std::max(maxg, tsvc[c]);
                for (size_t i = 0; i < items.size(); i++) {
                    double detail[8];
                    for (int c = 0; c < nc; c++) detail[c] = -1.0;
                    for (int l = 2; l <= maxg; l++) {
                        double m = 0.0;
                        for (int c = 0; c < nc; c++) if (tsvc[c] == l) m = std::max(m, det[i * nc + c]);
                        for (int c = 0; c < nc; c++) if (tsvc[c] == l) detail[c] = m;
                    }
                    for (int c = 0; c < nc; c++) {
                        if (tsvc[c] == 1) detail[c] = det[i * nc + c];
                        if (tsvc[c] == 0) detail[c] = 0.0;
                    }
                    for (int c = 0; c < nc; c++)
                        if (!(detail[c] <= eps_use[c])) sig[i] = 1;
                }
                L.security_apply(items, sig);
            }
            flags = L.ref;
        }
    } else if (!thr) {
        for (int b = 0; b < nb; b++) flags[b] = kFlagCoarsen;   // "everywhere": the leaves
    }
    toc(kFlags, t_flags);
    if (e != cudaSuccess) return fail_restore(e, WG_ECUDA);
    std::vector<int> leaves;
    adapt_decide(L.ft, flags, leaves);
    // delete, coarse extension on the remaining full tree, reconstruct
    for (int b = 0; b < nt; b++) {
        L.alive[b] = flags[b] != kFlagCoarsen;
        L.ref[b] = 0;
    }
    if (!meta()) return fail_restore(cudaSuccess, fail(WG_EGRID, "adapt: %s", err.c_str()));
    e = ce(0, 0, 0, true, false);
    for (int b = 0; b < nt; b++) {
        if (!L.alive[b] || !L.is_leaf(b, false)) continue;
        L.for_neighbors(b, [&](int r, int n) {
            if (L.ref[b] != -1 && L.ft.level[n] < L.ft.level[b] &&
                !(L.has_valid_neighbor(b, r, 0) || L.has_valid_neighbor(b, r, -1)))
                L.ref[b] = -1;
        });
    }
    auto reconstruct = [&](auto on_level) -> cudaError_t {
        const std::vector<int> rec = slots_where([&](int b) { return on_level(b) && L.ref[b] == -1; });
        const std::vector<int> keep = slots_where([&](int b) { return on_level(b) && L.ref[b] != -1; });
        cudaError_t r = cudaSuccess;
        auto t0 = tic();
        // waveletReconstruction_optimized_block writes into hvy_tmp and
        // hvy_block takes that copy (adapt_tree.f90:921-922): the later
        // levels' syncs read these blocks from hvy_tmp
        const int *d_rec = rec.empty() ? nullptr : up(rec);
        if (!rec.empty())
            r = launch_wavelet_reconstruct(dim, d_rec, (int)rec.size(), ctx->A, gA, Bs[0], Bs[1], Bs[2], nc, w.X,
                                           w.Y, ctx->stream);
        if (r == cudaSuccess && !rec.empty())
            r = launch_blockcopy(d_rec, (int)rec.size(), ctx->A, ctx->T, per_block, ctx->stream);
        toc(kRecon, t0);
        t0 = tic();
        if (r == cudaSuccess && !keep.empty())
            r = launch_blockcopy(up(keep), (int)keep.size(), ctx->T, ctx->A, per_block, ctx->stream);
        toc(kCopy, t0);
        return r;
    };
    SyncSpecL rs;
    rs.base = 3;
    rs.by_ref = true;
    rs.s_ref = -1;
    rs.gminus = rs.gplus = g;
    rs.tmp_usage = 2;
    if (leaf_only) {
        if (e == cudaSuccess) e = sync_spec(rs);
        if (e == cudaSuccess) e = ce(0, 0, 0, true, false);
        if (e == cudaSuccess) e = reconstruct([](int) { return true; });
    } else {
        int jmax = 0;
        for (int b = 0; b < nt; b++)
            if (L.alive[b]) jmax = std::max(jmax, L.ft.level[b]);
        for (int level = t->cfg.Jmin; level <= jmax && e == cudaSuccess; level++) {
            rs.by_level = true;
            rs.s_level = level;
            e = sync_spec(rs);
            if (e == cudaSuccess) e = ce(1, level, 0, true, false);
            if (e == cudaSuccess) e = reconstruct([&](int b) { return L.ft.level[b] == level; });
        }
    }
    // prune: the new leaves; final filtered sync on the leaf grid
    std::fill(L.alive.begin(), L.alive.end(), 0);
    for (int b : leaves) L.alive[b] = 1;
    std::fill(L.ref.begin(), L.ref.end(), 0);
    if (!meta()) return fail_restore(e, fail(WG_EGRID, "adapt: %s", err.c_str()));
    {
        SyncSpecL sp;
        sp.gminus = sp.gplus = g;
        if (e == cudaSuccess) e = sync_spec(sp);
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) return fail_restore(e, WG_ECUDA);
    // install the new grid
    const int nn = (int)leaves.size();
    std::vector<int> lv(nn), co(3 * nn), sl(nn), stat(nn);
    std::vector<char> kept(nt, 0);
    for (int i = 0; i < nn; i++) {
        const int b = leaves[i];
        lv[i] = L.ft.level[b];
        for (int a = 0; a < 3; a++) co[3 * i + a] = L.ft.coords[3 * b + a];
        sl[i] = L.slot[b];
        stat[i] = flags[b];
        kept[b] = 1;
    }
    for (int b = 0; b < nt; b++)
        if (!kept[b]) ctx->free_slots.give(L.slot[b]);
    for (int m : t->mask_slot)
        if (m >= 0) ctx->mask_free.push_back(m);
    t->forest.set(nn, lv.data(), co.data());
    if (!t->forest.update_neighbors(err)) return fail(WG_EGRID, "adapt produced an invalid grid: %s", err.c_str());
    if (!t->forest.graded()) return fail(WG_EGRID, "adapt produced a grid that is not graded");
    t->slots = sl;
    t->status = stat;
    t->mask_slot.assign(nn, -1);
    drop_sync(*t);
    if (const int sc = state_changed(ctx, t, tree)) return sc;
    int st;
    if ((st = upload_desc(ctx, *t, tree))) return st;
    if ((st = upload_lists(ctx, *t))) return st;
    if ((st = regen_masks(ctx, t, tree))) return st;
    ctx->grid_version++;
    WG_CUDA_OK(cudaStreamSynchronize(ctx->stream));
    ctx->adapt_ms[kTotal] = std::chrono::duration<double, std::milli>(clk::now() - t_start).count();
    if (nblk_out) *nblk_out = nn;
    return WG_OK;
}

int wg_adapt_profile(wg_ctx *ctx, int enable, double *ms_out, int n) {
    if (!ctx) return WG_EINVAL;
    if (enable >= 0) ctx->adapt_profile = enable != 0;
    if (ms_out)
        for (int i = 0; i < n && i < 8; i++) ms_out[i] = ctx->adapt_ms[i];
    return WG_OK;
}

int wg_adapt(wg_ctx *ctx, int tree, const double *eps_use, int indicator, int *nblk_out) {
    Tree *t = get_tree(ctx, tree);
    if (!t) return tree_err();
    if (indicator != WG_ADAPT_THRESHOLD && indicator != WG_ADAPT_EVERYWHERE)
        return fail(WG_EINVAL, "unknown indicator %d", indicator);
    std::vector<double> eps_own;
    if (indicator == WG_ADAPT_THRESHOLD && !eps_use) {
        WG_CUDA_OK(cudaStreamSynchronize(ctx->stream));
        const int st0 = adapt_thresholds(ctx, t, eps_own);
        if (st0) return st0;
        eps_use = eps_own.data();
    }
    if (ctx->wav.lifted || t->cfg.use_coarse_extension)
        return adapt_lifted(ctx, t, tree, eps_use, indicator == WG_ADAPT_THRESHOLD, nblk_out);
    const int dim = ctx->cfg.dim, nc = ctx->geo.nc, g = ctx->cfg.g;
    const int *Bs = ctx->cfg.Bs;
    const int nb = t->forest.size();
    WG_CUDA_OK(cudaStreamSynchronize(ctx->stream));
    int st = run_sync(ctx, *t, ctx->A, false, g, g);
    if (st) return st;
    FullTree ft;
    std::string err;
    if (!build_full_tree(dim, t->cfg.Jmin, nb, t->forest.level.data(), t->forest.coords.data(), ft, err))
        return fail(WG_EGRID, "adapt: %s", err.c_str());
    const int nt = ft.size(), nm = nt - nb;
    if ((size_t)nm > ctx->free_slots.size())
        return fail(WG_ENOMEM, "adapt needs %d free slots for the mothers (%zu free)", nm, ctx->free_slots.size());
    std::vector<int> slot(nt);
    for (int b = 0; b < nb; b++) slot[b] = t->slots[b];
    for (int b = nb; b < nt; b++) slot[b] = ctx->free_slots.take();
    auto give_back = [&](const std::vector<int> &keep) {
        std::vector<char> kept(nt, 0);
        for (int b : keep) kept[b] = 1;
        for (int b = 0; b < nt; b++)
            if (!kept[b]) ctx->free_slots.give(slot[b]);
    };
    std::vector<int> flags(nt, 0);
    DevArray<int> d_flags;
    const bool thr = indicator == WG_ADAPT_THRESHOLD;
    cudaError_t e = cudaSuccess;
    if (thr) {
        e = d_flags.upload(nullptr, nt, ctx->stream);
        if (e == cudaSuccess)
            e = launch_fwt_flags(dim, t->d_all.p, nb, ctx->A, ctx->gA, Bs[0], Bs[1], Bs[2], nc, ctx->wav.X, ctx->wav.Y,
                                 eps_use, t->cfg.threshold_state_vector_component, d_flags.p, nullptr, ctx->stream);
    } else {
        for (int b = 0; b < nb; b++) flags[b] = kFlagCoarsen;   // "everywhere": the leaves
    }
    // mothers level by level from the finest
    const int lmax = ft.max_level();
    std::vector<std::unique_ptr<DevArray<Patch>>> keep_alive;   // alive until the stream is synchronised
    std::vector<std::unique_ptr<DevArray<int>>> keep_lists;
    for (int l = lmax - 1; l >= t->cfg.Jmin && e == cudaSuccess; l--) {
        std::vector<Patch> d2m, gh;
        mother_patches(ft, ctx->geo, l, slot, d2m, gh);
        if (d2m.empty()) continue;
        keep_alive.emplace_back(new DevArray<Patch>());
        e = keep_alive.back()->upload(d2m.data(), d2m.size(), ctx->stream);
        if (e == cudaSuccess)
            e = launch_sync(keep_alive.back()->p, (int)d2m.size(), ctx->A, ctx->gA, nc, ctx->wav.order_predictor,
                            ctx->stream);
        if (!thr || e != cudaSuccess) continue;
        keep_alive.emplace_back(new DevArray<Patch>());
        e = keep_alive.back()->upload(gh.data(), gh.size(), ctx->stream);
        if (e == cudaSuccess)
            e = launch_sync(keep_alive.back()->p, (int)gh.size(), ctx->A, ctx->gA, nc, ctx->wav.order_predictor,
                            ctx->stream);
        // indicator of this level's mothers (consecutive full-tree indices)
        std::vector<int> ms;
        int first = -1;
        for (int b = nb; b < nt; b++)
            if (ft.level[b] == l) {
                if (first < 0) first = b;
                ms.push_back(slot[b]);
            }
        keep_lists.emplace_back(new DevArray<int>());
        if (e == cudaSuccess) e = keep_lists.back()->upload(ms.data(), ms.size(), ctx->stream);
        if (e == cudaSuccess)
            e = launch_fwt_flags(dim, keep_lists.back()->p, (int)ms.size(), ctx->A, ctx->gA, Bs[0], Bs[1], Bs[2], nc,
                                 ctx->wav.X, ctx->wav.Y, eps_use, t->cfg.threshold_state_vector_component,
                                 d_flags.p + first, nullptr, ctx->stream);
    }
    if (e == cudaSuccess && thr)
        e = cudaMemcpyAsync(flags.data(), d_flags.p, sizeof(int) * nt, cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) {
        cudaStreamSynchronize(ctx->stream);
        for (int b = nb; b < nt; b++) ctx->free_slots.give(slot[b]);   // the grid is unchanged
        return cuda_fail(e, "wg_adapt", __FILE__, __LINE__);
    }
    if (thr) indicator_switches(*t, ft, flags);
    std::vector<int> leaves;
    adapt_decide(ft, flags, leaves);
    // install the new grid
    const int nn = (int)leaves.size();
    std::vector<int> lv(nn), co(3 * nn), sl(nn), stat(nn);
    for (int i = 0; i < nn; i++) {
        const int b = leaves[i];
        lv[i] = ft.level[b];
        for (int a = 0; a < 3; a++) co[3 * i + a] = ft.coords[3 * b + a];
        sl[i] = slot[b];
        stat[i] = flags[b];
    }
    give_back(leaves);
    for (int m : t->mask_slot)
        if (m >= 0) ctx->mask_free.push_back(m);
    t->forest.set(nn, lv.data(), co.data());
    if (!t->forest.update_neighbors(err)) return fail(WG_EGRID, "adapt produced an invalid grid: %s", err.c_str());
    if (!t->forest.graded()) return fail(WG_EGRID, "adapt produced a grid that is not graded");
    t->slots = sl;
    t->status = stat;
    t->mask_slot.assign(nn, -1);
    drop_sync(*t);
    if (const int sc = state_changed(ctx, t, tree)) return sc;
    if ((st = upload_desc(ctx, *t, tree))) return st;
    if ((st = upload_lists(ctx, *t))) return st;
    if ((st = regen_masks(ctx, t, tree))) return st;
    ctx->grid_version++;
    if ((st = run_sync(ctx, *t, ctx->A, false, g, g))) return st;
    WG_CUDA_OK(cudaStreamSynchronize(ctx->stream));
    if (nblk_out) *nblk_out = nn;
    return WG_OK;
}

// refine_tree(..., "everywhere") data part: every block is replaced by its
// 2^d daughters (refineBlock); ghosts must be synchronised with g points.
// Daughters of block b are blocks 2^d*b .. 2^d*b+2^d-1 of the new grid.
// refineBlock (LIB/MESH/refinementExecute.f90:4-116) as prediction patches:
// daughter k of a parent (x half (k/2)%2, y half k%2, z half k/4) holds the
// parent's full-block prediction at fine indices g + Bs*half + i, i over the
// daughter's full block. Each patch covers a slab of tz planes of one
// daughter and reads a coarse sub-box of the parent that holds every stencil
// of its points: within the sub-box no point reaches the zero fill at the
// edges unless it does in the parent's full fine array, so the separable
// prediction kernel returns the reference's values. Returns the shared
// memory (doubles) of the largest patch.
static int refine_patches(const wg_config &c, int g, int order, const std::vector<int> &parents,
                          const std::vector<int> &daughters, int tz, std::vector<Patch> &out) {
    const int dim = c.dim, nd = 1 << dim, h = order - 1;
    int nb[3];
    for (int d = 0; d < 3; d++) nb[d] = d < dim ? c.Bs[d] + 2 * g : 1;
    const int nslab = dim == 3 ? (nb[2] + tz - 1) / tz : 1;
    auto fdiv = [](int a) { return a >= 0 ? a / 2 : -((1 - a) / 2); };   // floor(a / 2)
    int need = 0;
    out.clear();
    out.reserve(parents.size() * nd * nslab);
    for (size_t p = 0; p < parents.size(); p++)
        for (int k = 0; k < nd; k++)
            for (int sl = 0; sl < nslab; sl++) {
                Patch q;
                std::memset(&q, 0, sizeof(q));
                q.src = parents[p];
                q.dst = daughters[p * nd + k];
                q.op = 2;
                const int half[3] = {(k / 2) % 2, k % 2, k / 4};
                for (int d = 0; d < dim; d++) {
                    const int ilo = d == 2 ? sl * tz : 0, ihi = d == 2 ? std::min(nb[2], (sl + 1) * tz) - 1 : nb[d] - 1;
                    const int flo = g + c.Bs[d] * half[d] + ilo, fhi = g + c.Bs[d] * half[d] + ihi;
                    const int clo = std::max(0, fdiv(flo - h)), chi = std::min(nb[d] - 1, fdiv(fhi + h + 1));
                    q.rlo[d] = (int16_t)ilo;
                    q.rhi[d] = (int16_t)ihi;
                    q.slo[d] = (int16_t)clo;
                    q.shi[d] = (int16_t)chi;
                    q.blo[d] = (int16_t)(flo - 2 * clo);
                }
                // shared memory of predict_kernel: coarse box, x window, x-y window
                const int cx = q.shi[0] - q.slo[0] + 1, cy = q.shi[1] - q.slo[1] + 1, cz = q.shi[2] - q.slo[2] + 1;
                const int ex = q.rhi[0] - q.rlo[0] + 1, ey = q.rhi[1] - q.rlo[1] + 1, ez = q.rhi[2] - q.rlo[2] + 1;
                int yw0 = std::max(0, q.blo[1] - h), yw1 = std::min(2 * cy - 2, q.blo[1] + ey - 1 + h);
                yw0 += yw0 & 1;
                yw1 -= yw1 & 1;
                int zw0 = std::max(0, q.blo[2] - h), zw1 = std::min(2 * cz - 2, q.blo[2] + ez - 1 + h);
                zw0 += zw0 & 1;
                zw1 -= zw1 & 1;
                const int wy = (yw1 - yw0) / 2 + 1, wz = (zw1 - zw0) / 2 + 1;
                need = std::max(need, cx * cy * cz + ex * wy * wz + ex * ey * wz);
                out.push_back(q);
            }
    return need;
}

// refineBlock for the blocks with refine[b] != 0 (refinementExecute.f90:
// 4-116): each is replaced, at its position, by its 2^d daughters; the
// others keep their place and data
static int refine_blocks(wg_ctx *ctx, Tree *t, int tree, const std::vector<char> &refine) {
    const int dim = ctx->cfg.dim, nd = 1 << dim;
    const int nb = t->forest.size();
    std::vector<int> ref;
    for (int b = 0; b < nb; b++)
        if (refine[b]) ref.push_back(b);
    const int nr = (int)ref.size();
    if ((size_t)nr * nd > ctx->free_slots.size()) return fail(WG_ENOMEM, "refinement needs %d free slots", nr * nd);
    const int nn = nb + nr * (nd - 1);
    std::vector<int> lv, co, slots, child_first(nb, -1), parents, bases;
    lv.reserve(nn);
    co.reserve(3 * nn);
    slots.reserve(nn);
    // the daughters take any free slots (lowest first): bases[p * nd + k]
    for (int b : ref) {
        child_first[b] = (int)bases.size();
        for (int k = 0; k < nd; k++) bases.push_back(ctx->free_slots.take());
        parents.push_back(t->slots[b]);
    }
    for (int b = 0; b < nb; b++) {
        if (child_first[b] < 0) {   // stays on Jmax
            lv.push_back(t->forest.level[b]);
            for (int a = 0; a < 3; a++) co.push_back(t->forest.coords[3 * b + a]);
            slots.push_back(t->slots[b]);
            continue;
        }
        for (int k = 0; k < nd; k++) {
            lv.push_back(t->forest.level[b] + 1);
            co.push_back(2 * t->forest.coords[3 * b + 0] + (k / 2) % 2);
            co.push_back(2 * t->forest.coords[3 * b + 1] + k % 2);
            co.push_back(dim == 3 ? 2 * t->forest.coords[3 * b + 2] + k / 4 : 0);
            slots.push_back(bases[child_first[b] + k]);
        }
    }
    if (nr > 0) {
        DevArray<int> d_par, d_base;
        const int *Bs = ctx->cfg.Bs;
        // separable prediction per daughter slab (7 planes: two CTAs per SM
        // for 16^3 blocks); the point-wise kernel where a slab's windows do
        // not fit the shared memory
        std::vector<Patch> rp;
        const int need = refine_patches(ctx->cfg, ctx->gA.gb, ctx->wav.order_predictor, parents, bases, 7, rp);
        cudaError_t e = cudaSuccess;
        DevArray<Patch> d_rp;
        if ((size_t)need * sizeof(double) <= 200 * 1024) {
            e = d_rp.upload(rp.data(), rp.size(), ctx->stream);
            if (e == cudaSuccess)
                e = launch_predict(d_rp.p, (int)rp.size(), need, ctx->A, ctx->gA, ctx->geo.nc, ctx->wav.order_predictor,
                                   ctx->stream);
        } else {
            e = d_par.upload(parents.data(), nr, ctx->stream);
            if (e == cudaSuccess) e = d_base.upload(bases.data(), bases.size(), ctx->stream);
            if (e == cudaSuccess)
                e = launch_refine(dim, d_par.p, nr, d_base.p, ctx->A, ctx->gA, Bs[0], Bs[1], Bs[2], ctx->geo.nc,
                                  ctx->wav.order_predictor, ctx->stream);
        }
        if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
        if (e != cudaSuccess) {   // the grid is unchanged
            cudaStreamSynchronize(ctx->stream);
            for (int s2 : bases) ctx->free_slots.give(s2);
            return cuda_fail(e, "refineBlock", __FILE__, __LINE__);
        }
    }
    // swap the tree onto the new blocks
    for (int s2 : parents) ctx->free_slots.give(s2);
    for (int m : t->mask_slot)
        if (m >= 0) ctx->mask_free.push_back(m);
    t->slots = slots;
    t->status.clear();
    t->mask_slot.assign(nn, -1);
    if (const int sc = state_changed(ctx, t, tree)) return sc;
    drop_sync(*t);
    t->forest.set(nn, lv.data(), co.data());
    std::string err;
    if (!t->forest.update_neighbors(err)) return fail(WG_EGRID, "%s", err.c_str());
    int st;
    if ((st = upload_desc(ctx, *t, tree))) return st;
    if ((st = upload_lists(ctx, *t))) return st;
    if ((st = regen_masks(ctx, t, tree))) return st;
    WG_CUDA_OK(cudaStreamSynchronize(ctx->stream));
    ctx->grid_version++;
    return WG_OK;
}

int wg_refine_everywhere(wg_ctx *ctx, int tree) {
    Tree *t = get_tree(ctx, tree);
    if (!t) return tree_err();
    // blocks on Jmax stay (respectJmaxJmin_tree, LIB/MESH/respectJmaxJmin_tree.f90)
    std::vector<char> refine(t->forest.size(), 0);
    for (int b = 0; b < t->forest.size(); b++) refine[b] = t->forest.level[b] < t->cfg.Jmax;
    return refine_blocks(ctx, t, tree, refine);
}

int wg_refine_significant(wg_ctx *ctx, int tree) {
    Tree *t = get_tree(ctx, tree);
    if (!t) return tree_err();
    const int nb = t->forest.size();
    if ((int)t->status.size() != nb) return fail(WG_EINVAL, "no refinement status: adapt the tree first");
    // refinementIndicator_tree "significant": 0 -> +1, REF_UNSIGNIFICANT_STAY -> 0
    std::vector<int> f(nb);
    for (int b = 0; b < nb; b++) {
        const int s0 = t->status[b];
        if (s0 == 1 || s0 == -1) return fail(WG_EINVAL, "refinement status %d on block %d", s0, b);
        f[b] = s0 == 0 ? 1 : s0 == kFlagUnsignificantStay ? 0 : s0;
        if (f[b] == 1 && t->forest.level[b] >= t->cfg.Jmax) f[b] = 0;   // respectJmaxJmin_tree
    }
    // ensureGradedness_tree: a block next to a finer block that refines refines
    for (bool changed = true; changed;) {
        changed = false;
        for (int b = 0; b < nb; b++) {
            if (f[b] != 0) continue;
            for (int r = 0; r < kNumRelations; r++) {
                const int n = t->forest.nbr[(size_t)b * kNumRelations + r];
                if (n >= 0 && t->forest.level[n] == t->forest.level[b] + 1 && f[n] == 1) {
                    f[b] = 1;
                    changed = true;
                    break;
                }
            }
        }
    }
    std::vector<char> refine(nb, 0);
    for (int b = 0; b < nb; b++) refine[b] = f[b] == 1;
    return refine_blocks(ctx, t, tree, refine);
}

int wg_set_refinement_status(wg_ctx *ctx, int tree, int nblk, const int *status) {
    Tree *t = get_tree(ctx, tree);
    if (!t) return tree_err();
    if (nblk != t->forest.size() || (nblk && !status)) return fail(WG_EINVAL, "status of %d blocks expected", t->forest.size());
    for (int b = 0; b < nblk; b++)
        if (status[b] != 0 && status[b] != kFlagUnsignificantStay)
            return fail(WG_EINVAL, "refinement status %d on block %d (0 or 9 expected)", status[b], b);
    t->status.assign(status, status + nblk);
    return WG_OK;
}

int wg_get_refinement_status(wg_ctx *ctx, int tree, int cap, int *status) {
    Tree *t = get_tree(ctx, tree);
    if (!t) return tree_err();
    const int nb = t->forest.size();
    if ((int)t->status.size() != nb) return fail(WG_EINVAL, "no refinement status: adapt the tree first");
    if (status)
        for (int b = 0; b < std::min(cap, nb); b++) status[b] = t->status[b];
    return nb;
}

// patch table of the tree's ghost sync for inspection: returns the number of
// patches; if out != NULL, writes 19 ints per patch
// (src, dst, op, stage, rlo[3], rhi[3], slo[3], shi[3], blo[3])
int wg_sync_table(wg_ctx *ctx, int tree, int gminus, int gplus, int thin, int cap, int *out) {
    Tree *t = get_tree(ctx, tree);
    if (!t) return tree_err();
    SyncPlan *sp;
    int st = get_sync(ctx, *t, gminus, gplus, thin != 0, &sp);
    if (st) return st;
    const int n = (int)sp->table.patches.size();
    if (out) {
        if (cap < n) return fail(WG_EINVAL, "capacity too small");
        for (int i = 0; i < n; i++) {
            const Patch &p = sp->table.patches[i];
            int *o = out + 19 * i;
            o[0] = p.src;
            o[1] = p.dst;
            o[2] = p.op;
            o[3] = p.stage;
            for (int k = 0; k < 3; k++) {
                o[4 + k] = p.rlo[k];
                o[7 + k] = p.rhi[k];
                o[10 + k] = p.slo[k];
                o[13 + k] = p.shi[k];
                o[16 + k] = p.blo[k];
            }
        }
    }
    return n;
}

// block slot of block b of a tree (for tests that inspect the arena)
int wg_block_slot(wg_ctx *ctx, int tree, int b) {
    Tree *t = get_tree(ctx, tree);
    if (!t) return tree_err();
    if (b < 0 || b >= (int)t->slots.size()) return fail(WG_EINVAL, "bad block");
    return t->slots[b];
}

}  // extern "C"

extern "C" {

// Host-only ghost-patch table of a grid (no device needed): the same table
// wg_sync_table returns, with block indices instead of arena slots.
int wg_sync_table_host(const wg_config *cfg, int nblk, const int *level, const int *coords, int gminus, int gplus,
                       int thin, int cap, int *out) {
    int st = check_cfg(cfg);
    if (st) return st;
    Forest f;
    f.dim = cfg->dim;
    f.Jmin = cfg->Jmin;
    f.Jmax = cfg->Jmax;
    f.set(nblk, level, coords);
    std::string err;
    if (!f.update_neighbors(err)) return fail(WG_EGRID, "%s", err.c_str());
    Geometry geo;
    geo.dim = cfg->dim;
    for (int d = 0; d < 3; d++) geo.Bs[d] = d < cfg->dim ? cfg->Bs[d] : 1;
    geo.g = cfg->g;
    geo.nc = cfg->neq;
    WaveletInfo w;
    make_wavelet(cfg->wavelet, w);
    SyncTable t;
    if (!make_sync_table(f, geo, w, gminus, gplus, thin ? cfg->g_rhs : cfg->g, 0, t, err))
        return fail(WG_EGRID, "sync table: %s", err.c_str());
    const int n = (int)t.patches.size();
    if (out) {
        if (cap < n) return fail(WG_EINVAL, "capacity too small");
        for (int i = 0; i < n; i++) {
            const Patch &p = t.patches[i];
            int *o = out + 19 * i;
            o[0] = p.src;
            o[1] = p.dst;
            o[2] = p.op;
            o[3] = p.stage;
            for (int k = 0; k < 3; k++) {
                o[4 + k] = p.rlo[k];
                o[7 + k] = p.rhi[k];
                o[10 + k] = p.slo[k];
                o[13 + k] = p.shi[k];
                o[16 + k] = p.blo[k];
            }
        }
    }
    return n;
}

}  // extern "C"

extern "C" {

// Average device time of one launch of a hot-path kernel over reps launches,
// timed with CUDA events on the context stream. which: 0 = RK stage kernel
// (stage 2, current variant, plain + masked lists), 1 = RHS ghost sync of a
// stage buffer (all stages), 2 = dt reduction. The state is left unchanged
// for which = 0 and 2 (stage 2 writes only the stage buffers).
int wg_time_kernel(wg_ctx *ctx, int tree, int which, int reps, double *ms_per_launch) {
    Tree *t = get_tree(ctx, tree);
    if (!t) return tree_err();
    if (reps <= 0 || !ms_per_launch) return fail(WG_EINVAL, "bad arguments");
    const int g_rhs = ctx->cfg.g_rhs;
    const int *Bs = ctx->cfg.Bs;
    SyncPlan *sp;
    int st = get_sync(ctx, *t, g_rhs, g_rhs, true, &sp);
    if (st) return st;
    cudaEvent_t e0, e1;
    WG_CUDA_OK(cudaEventCreate(&e0));
    WG_CUDA_OK(cudaEventCreate(&e1));
    auto once = [&]() -> int {
        const bool df = ctx->precision == WG_RHS_FP32;
        const bool push = df && sp->push_ok && !sp->pair_begin.empty();
        if (which == 0 && df) return stage_launch_df(ctx, *t, 2, ctx->C, ctx->D, push);
        if (which == 0) return stage_launch(ctx, *t, 2, ctx->B, ctx->gT, ctx->C, ctx->gT);
        if (which == 1) return run_sync(ctx, *t, ctx->D, true, g_rhs, g_rhs, df, push);
        WG_CUDA_OK(launch_dt(ctx->cfg.dim, t->d_all.p, (int)t->slots.size(), ctx->d_desc, ctx->d_tp, ctx->d_clk,
                             ctx->A, ctx->gA, Bs[0], Bs[1], Bs[2], 1, ctx->d_tree_ids.p + tree, dt_done(ctx), ctx->stream));
        return WG_OK;
    };
    if ((st = once())) return st;
    WG_CUDA_OK(cudaEventRecord(e0, ctx->stream));
    for (int r = 0; r < reps; r++)
        if ((st = once())) return st;
    WG_CUDA_OK(cudaEventRecord(e1, ctx->stream));
    WG_CUDA_OK(cudaEventSynchronize(e1));
    float ms = 0.f;
    WG_CUDA_OK(cudaEventElapsedTime(&ms, e0, e1));
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    *ms_per_launch = ms / reps;
    return WG_OK;
}

// nsteps RK4 steps of the listed trees (the same launches as wg_run without
// a graph; batched for the FP32-pipe precision), one step at a time with CUDA
// events on the context stream between the kernel groups; ms[9] receives the
// mean device time per step of: sync before stages 1-4 (ms[0..3]), dt
// (ms[4]), stages 1-4 (ms[5..8]). The state advances by nsteps steps.
int wg_step_profile(wg_ctx *ctx, int ntrees, const int *trees, int nsteps, double *ms) {
    if (!ctx || ntrees <= 0 || !trees || nsteps <= 0 || !ms) return fail(WG_EINVAL, "bad arguments");
    if (ctx->dead) return fail(WG_ETIMEOUT, "the context is unusable after a timed-out device wait; destroy it");
    for (int i = 0; i < 9; i++) ms[i] = 0.0;
    for (cudaEvent_t &ev : ctx->prof_ev)
        if (!ev) WG_CUDA_OK(cudaEventCreate(&ev));
    static const int order[9][2] = {{0, 1}, {3, 4}, {5, 6}, {7, 8}, {1, 2}, {2, 3}, {4, 5}, {6, 7}, {8, 9}};
    for (int s = 0; s < nsteps; s++) {
        if (ctx->precision == WG_RHS_FP32) {
            int st = wg_run(ctx, ntrees, trees, 0, 0);   // checks, shadows, batch plan
            if (st) return st;
            for (int i = 0; i < ntrees; i++)
                if ((st = autotune_stage_form(ctx, ctx->trees[trees[i]]))) return st;
            ctx->prof_on = true;
            st = rk4_enqueue_batch(ctx);
            ctx->prof_on = false;
            if (st) return st;
        } else {
            if (ntrees != 1) return fail(WG_EINVAL, "the FP64 precision profiles one tree");
            Tree *t = get_tree(ctx, trees[0]);
            if (!t) return tree_err();
            ctx->prof_on = true;
            int st = rk4_enqueue(ctx, trees[0]);
            ctx->prof_on = false;
            if (st) return st;
        }
        WG_CUDA_OK(cudaEventSynchronize(ctx->prof_ev[9]));
        for (int i = 0; i < 9; i++) {
            float v = 0.f;
            WG_CUDA_OK(cudaEventElapsedTime(&v, ctx->prof_ev[order[i][0]], ctx->prof_ev[order[i][1]]));
            ms[i] += v / nsteps;
        }
    }
    return check_dev_err(ctx);
}

// Per-block interior points and masked-block count of a tree (for the bench)
int wg_tree_stats(wg_ctx *ctx, int tree, int *nblocks, int *nmasked) {
    Tree *t = get_tree(ctx, tree);
    if (!t) return tree_err();
    if (nblocks) *nblocks = (int)t->slots.size();
    if (nmasked) *nmasked = t->n_masked;
    return WG_OK;
}

}  // extern "C"

namespace {
int ensure_staging(wg_ctx *ctx, size_t bytes) {
    if (ctx->staging_bytes >= bytes) return WG_OK;
    if (ctx->staging) cudaFree(ctx->staging);
    ctx->staging = nullptr;
    ctx->staging_bytes = 0;
    if (cudaMalloc(&ctx->staging, bytes) != cudaSuccess) {
        cudaGetLastError();
        return fail(WG_ENOMEM, "staging buffer of %zu bytes does not fit", bytes);
    }
    ctx->staging_bytes = bytes;
    return WG_OK;
}
}  // namespace

extern "C" {

// Interior-only state exchange: host array (nblk, neq, Bz, By, Bx), x
// fastest. The copy runs in chunks of whole blocks on a second stream so that
// the host<->device transfer of one chunk overlaps the device scatter /
// gather of the previous (next) one; ghost nodes are left to the next
// synchronisation.
static int ensure_copy_stream(wg_ctx *ctx, int nchunk) {
    if (!ctx->copy_stream &&
        cudaStreamCreateWithFlags(&ctx->copy_stream, cudaStreamNonBlocking) != cudaSuccess) {
        ctx->copy_stream = nullptr;
        return fail(WG_ECUDA, "cudaStreamCreate failed");
    }
    while ((int)ctx->copy_ev.size() < 2 * nchunk) {
        cudaEvent_t ev;
        if (cudaEventCreateWithFlags(&ev, cudaEventDisableTiming) != cudaSuccess) return fail(WG_ECUDA, "cudaEventCreate failed");
        ctx->copy_ev.push_back(ev);
    }
    return WG_OK;
}

// chunks of about 256 MB, at block granularity
static int interior_chunks(const wg_ctx *ctx, int nblk, std::vector<int> &first) {
    const size_t per = sizeof(double) * ctx->geo.nc * ctx->nint;
    const int step = std::max(1, (int)((256u << 20) / per));
    first.clear();
    for (int b = 0; b < nblk; b += step) first.push_back(b);
    first.push_back(nblk);
    return (int)first.size() - 1;
}

static int interior_transfer(wg_ctx *ctx, Tree *t, double *host, int to_device) {
    const int *Bs = ctx->cfg.Bs;
    const int Bz = ctx->cfg.dim == 3 ? Bs[2] : 1;
    const int nblk = (int)t->slots.size();
    const size_t per = (size_t)ctx->geo.nc * ctx->nint;
    int st = ensure_staging(ctx, sizeof(double) * per * nblk);
    if (st) return st;
    // an upload also writes the double-float copy of the FP32-pipe precision
    const bool shadow = to_device && ctx->precision == WG_RHS_FP32;
    bool push = false;
    if (shadow && (st = thin_plan(ctx, *t, &push))) return st;
    std::vector<int> first;
    const int nch = interior_chunks(ctx, nblk, first);
    if ((st = ensure_copy_stream(ctx, nch))) return st;
    const cudaMemcpyKind kind = cudaMemcpyDefault;   // host or device memory
    const int tid = (int)(t - ctx->trees.data());
    // the scatter records max |u|, from which the anchored copy takes its quantum
    if (shadow) WG_CUDA_OK(launch_umax_reset(ctx->d_clk, ctx->d_tree_ids.p + tid, 1, ctx->stream));
    for (int k = 0; k < nch; k++) {
        const int b0 = first[k], nb = first[k + 1] - first[k];
        double *dev = ctx->staging + per * b0, *hst = host + per * b0;
        const size_t bytes = sizeof(double) * per * nb;
        cudaEvent_t done = ctx->copy_ev[2 * k], ready = ctx->copy_ev[2 * k + 1];
        if (to_device) {
            WG_CUDA_OK(cudaMemcpyAsync(dev, hst, bytes, kind, ctx->copy_stream));
            WG_CUDA_OK(cudaEventRecord(done, ctx->copy_stream));
            WG_CUDA_OK(cudaStreamWaitEvent(ctx->stream, done, 0));
            WG_CUDA_OK(launch_interior_xfer(t->d_all.p + b0, nb, dev, ctx->A, ctx->gA, ctx->geo.nc, Bs[0], Bs[1], Bz,
                                            1, ctx->d_desc, shadow ? ctx->d_clk : nullptr, ctx->stream,
                                            shadow ? ctx->B : nullptr, ctx->gT, push ? ctx->d_push : nullptr));
        } else {
            WG_CUDA_OK(launch_interior_xfer(t->d_all.p + b0, nb, dev, ctx->A, ctx->gA, ctx->geo.nc, Bs[0], Bs[1], Bz,
                                            0, ctx->d_desc, nullptr, ctx->stream));
            WG_CUDA_OK(cudaEventRecord(ready, ctx->stream));
            WG_CUDA_OK(cudaStreamWaitEvent(ctx->copy_stream, ready, 0));
            WG_CUDA_OK(cudaMemcpyAsync(hst, dev, bytes, kind, ctx->copy_stream));
        }
    }
    if (shadow) {
        // the scatter wrote the anchored copy with the tree's current
        // constant; redone only if the new state's constant differs
        WG_CUDA_OK(launch_anchor_check(ctx->d_clk, ctx->d_tree_ids.p + tid, 1, ctx->stream));
        WG_CUDA_OK(launch_shadow(t->d_all.p, nblk, ctx->A, ctx->gA, ctx->B, ctx->gT, ctx->geo.nc, Bs[0], Bs[1], Bz,
                                 push ? ctx->d_push : nullptr, ctx->d_desc, ctx->d_clk, ctx->stream, 1));
    }
    WG_CUDA_OK(cudaStreamSynchronize(ctx->copy_stream));
    WG_CUDA_OK(cudaStreamSynchronize(ctx->stream));
    if (shadow) t->shadow_valid = true;
    return WG_OK;
}

int wg_upload_interior(wg_ctx *ctx, int tree, const double *host) {
    Tree *t = get_tree(ctx, tree);
    if (!t) return tree_err();
    if (!host) return fail(WG_EINVAL, "bad arguments");
    if (const int sc = state_changed(ctx, t, tree)) return sc;
    // the staging buffer is free once the stream's earlier work is done
    WG_CUDA_OK(cudaStreamSynchronize(ctx->stream));
    return interior_transfer(ctx, t, const_cast<double *>(host), 1);
}

int wg_download_interior(wg_ctx *ctx, int tree, double *host) {
    Tree *t = get_tree(ctx, tree);
    if (!t) return tree_err();
    if (!host) return fail(WG_EINVAL, "bad arguments");
    return interior_transfer(ctx, t, host, 0);
}

// Streaming RK4 steps with host buffers: five staging buffers, the input of
// step k+1 copied in (copy stream) while step k computes, the result of step
// k copied out (d2h stream) while step k+1 computes. FP64 precision: every
// step scatters its input into the state, steps, and gathers the result.
// FP32-pipe precision: the loop below.
int wg_rk4_stream(wg_ctx *ctx, int tree, int nsteps, const double *const *ins, double *const *outs) {
    Tree *t = get_tree(ctx, tree);
    if (!t) return tree_err();
    if (nsteps < 0 || (nsteps && (!ins || !outs))) return fail(WG_EINVAL, "bad arguments");
    for (int k = 0; k < nsteps; k++)
        if (!ins[k] || !outs[k]) return fail(WG_EINVAL, "null buffer for step %d", k);
    if (nsteps == 0) return WG_OK;
    const int *Bs = ctx->cfg.Bs;
    const int Bz = ctx->cfg.dim == 3 ? Bs[2] : 1;
    const int nblk = (int)t->slots.size();
    const size_t per = (size_t)ctx->geo.nc * ctx->nint, bytes = sizeof(double) * per * nblk;
    int st;
    if (ctx->stream_buf_bytes < 5 * bytes) {
        cudaFree(ctx->stream_buf);
        ctx->stream_buf = nullptr;
        ctx->stream_buf_bytes = 0;
        if (cudaMalloc(&ctx->stream_buf, 5 * bytes) != cudaSuccess) {
            cudaGetLastError();
            return fail(WG_ENOMEM, "staging buffers of 5 x %zu bytes do not fit", bytes);
        }
        ctx->stream_buf_bytes = 5 * bytes;
    }
    if ((st = ensure_copy_stream(ctx, 1))) return st;
    if (!ctx->d2h_stream && cudaStreamCreateWithFlags(&ctx->d2h_stream, cudaStreamNonBlocking) != cudaSuccess) {
        ctx->d2h_stream = nullptr;
        return fail(WG_ECUDA, "cudaStreamCreate failed");
    }
    for (cudaEvent_t &ev : ctx->io_ev)
        if (!ev && cudaEventCreateWithFlags(&ev, cudaEventDisableTiming) != cudaSuccess) return fail(WG_ECUDA, "cudaEventCreate failed");
    // I[k % 3] receives step k's input, O[k & 1] its result. FP32-pipe: the
    // last stage of step k also writes the anchored copy of input k+1 (the
    // scatter of the next step), and step k+1 reads its u_n (dt, last stage)
    // from I directly, so the FP64 state is written only by the last step;
    // an input is free again after its own step. The copy in of step k+1
    // waits only for the end of step k-2 (three input buffers: the copies in
    // run ahead of the steps, and a stage 4 finds its next input on the
    // device), the copy out of step k only for the end of step k, so both
    // directions use the link at once
    cudaEvent_t *h2d_done = ctx->io_ev, *d2h_done = ctx->io_ev + 3, *gathered = ctx->io_ev + 5,
                *consumed = ctx->io_ev + 7;
    const bool shadow = ctx->precision == WG_RHS_FP32;
    bool push = false;
    if (shadow && (st = thin_plan(ctx, *t, &push))) return st;
    if ((st = autotune_stage_form(ctx, *t))) return st;
    const size_t pb = per * nblk;
    double *I[3] = {ctx->stream_buf, ctx->stream_buf + pb, ctx->stream_buf + 2 * pb};
    double *O[2] = {ctx->stream_buf + 3 * pb, ctx->stream_buf + 4 * pb};
    // FP32-pipe: the last stage writes the result into O directly
    if (shadow) {
        std::vector<int> pos(ctx->max_blocks, 0);
        for (int i = 0; i < nblk; i++) pos[t->slots[i]] = i;
        WG_CUDA_OK(ctx->d_pos.upload(pos.data(), pos.size(), ctx->stream));
    }
    WG_CUDA_OK(cudaStreamSynchronize(ctx->stream));
    WG_CUDA_OK(cudaMemcpyAsync(I[0], ins[0], bytes, cudaMemcpyDefault, ctx->copy_stream));
    WG_CUDA_OK(cudaEventRecord(h2d_done[0], ctx->copy_stream));
    auto scatter = [&](double *in) -> int {   // input into the state (and its anchored copy)
        WG_CUDA_OK(cudaMemsetAsync(&ctx->d_clk[tree].usq_ready, 0, sizeof(int), ctx->stream));
        if (shadow) WG_CUDA_OK(launch_umax_reset(ctx->d_clk, ctx->d_tree_ids.p + tree, 1, ctx->stream));
        WG_CUDA_OK(launch_interior_xfer(t->d_all.p, nblk, in, ctx->A, ctx->gA, ctx->geo.nc, Bs[0], Bs[1], Bz, 1,
                                        ctx->d_desc, shadow ? ctx->d_clk : nullptr, ctx->stream,
                                        shadow ? ctx->B : nullptr, ctx->gT, push ? ctx->d_push : nullptr));
        return WG_OK;
    };
    // the quantum of the new state, the copy redone if it changed: from the
    // state after a scatter, from the compact input (src) after a stage 4
    // that loaded it
    auto reanchor = [&](const double *src) -> int {
        WG_CUDA_OK(launch_anchor_check(ctx->d_clk, ctx->d_tree_ids.p + tree, 1, ctx->stream));
        WG_CUDA_OK(launch_shadow(t->d_all.p, nblk, src ? src : ctx->A, ctx->gA, ctx->B, ctx->gT, ctx->geo.nc, Bs[0],
                                 Bs[1], Bz, push ? ctx->d_push : nullptr, ctx->d_desc, ctx->d_clk, ctx->stream, 1,
                                 src ? ctx->d_pos.p : nullptr));
        return WG_OK;
    };
    for (int k = 0; k < nsteps; k++) {
        const int cur = k % 3, nxt = (k + 1) % 3, oc = k & 1;
        if (k + 1 < nsteps) {
            if (k >= 2) WG_CUDA_OK(cudaStreamWaitEvent(ctx->copy_stream, consumed[nxt], 0));
            WG_CUDA_OK(cudaMemcpyAsync(I[nxt], ins[k + 1], bytes, cudaMemcpyDefault, ctx->copy_stream));
            WG_CUDA_OK(cudaEventRecord(h2d_done[nxt], ctx->copy_stream));
        }
        // the input of step k: scattered here (the first step, or FP64),
        // otherwise already loaded by the last stage of step k-1
        if (k == 0 || !shadow) {
            WG_CUDA_OK(cudaStreamWaitEvent(ctx->stream, h2d_done[cur], 0));
            if ((st = scatter(I[cur]))) return st;
            if (shadow && (st = reanchor(nullptr))) return st;
        }
        t->shadow_valid = shadow;
        // the result buffer O[oc] is free once the result of step k-2 is out
        if (k >= 2) WG_CUDA_OK(cudaStreamWaitEvent(ctx->stream, d2h_done[oc], 0));
        const bool chain = shadow && k + 1 < nsteps;
        if (shadow) {
            ctx->s4_out = O[oc];
            ctx->s4_keep = chain ? 3 : 1;
            ctx->s4_next = chain ? I[nxt] : nullptr;
            ctx->s4_wait = chain ? h2d_done[nxt] : nullptr;
            ctx->s4_usrc = I[cur];
        }
        st = rk4_enqueue(ctx, tree);
        ctx->s4_out = nullptr;
        ctx->s4_keep = 1;
        ctx->s4_next = nullptr;
        ctx->s4_wait = nullptr;
        ctx->s4_usrc = nullptr;
        if (st) return st;
        if (chain && (st = reanchor(I[nxt]))) return st;
        WG_CUDA_OK(cudaEventRecord(consumed[cur], ctx->stream));   // input k read for the last time
        if (!shadow)
            WG_CUDA_OK(launch_interior_xfer(t->d_all.p, nblk, O[oc], ctx->A, ctx->gA, ctx->geo.nc, Bs[0], Bs[1], Bz, 0,
                                            ctx->d_desc, nullptr, ctx->stream));
        WG_CUDA_OK(cudaEventRecord(gathered[oc], ctx->stream));
        WG_CUDA_OK(cudaStreamWaitEvent(ctx->d2h_stream, gathered[oc], 0));
        WG_CUDA_OK(cudaMemcpyAsync(outs[k], O[oc], bytes, cudaMemcpyDefault, ctx->d2h_stream));
        WG_CUDA_OK(cudaEventRecord(d2h_done[oc], ctx->d2h_stream));
    }
    WG_CUDA_OK(cudaStreamSynchronize(ctx->d2h_stream));
    WG_CUDA_OK(cudaStreamSynchronize(ctx->copy_stream));
    WG_CUDA_OK(cudaStreamSynchronize(ctx->stream));
    return WG_OK;
}

}  // extern "C"

extern "C" {

// number of kernel nodes in the captured RK4-step graph of the last
// wg_run(use_graph=1) call (the launches one replay performs)
int wg_graph_kernels(wg_ctx *ctx) {
    if (!ctx || !ctx->graph) return fail(WG_EINVAL, "no captured graph");
    size_t n = 0;
    WG_CUDA_OK(cudaGraphGetNodes(ctx->graph, nullptr, &n));
    std::vector<cudaGraphNode_t> nodes(n);
    WG_CUDA_OK(cudaGraphGetNodes(ctx->graph, nodes.data(), &n));
    int k = 0;
    for (auto nd : nodes) {
        cudaGraphNodeType t;
        WG_CUDA_OK(cudaGraphNodeGetType(nd, &t));
        if (t == cudaGraphNodeTypeKernel) k++;
    }
    return k;
}

}  // extern "C"

extern "C" {

// Coarsening indicator without any device allocation (see the header).
int wg_threshold_flags_noalloc(const wg_config *cfg, int nblk, const double *d_blocks, const double *eps_use,
                               int *d_flags, double *d_details, void *stream) {
    int st = check_cfg(cfg);
    if (st) return st;
    if (nblk < 0 || (nblk && (!d_blocks || !eps_use || !d_flags))) return fail(WG_EINVAL, "bad arguments");
    if (nblk > noalloc_max_blocks())
        return fail(WG_EINVAL, "wg_threshold_flags_noalloc handles at most %d blocks per call (got %d)",
                    noalloc_max_blocks(), nblk);
    if (cfg->neq > 8) return fail(WG_EINVAL, "at most 8 components");
    WaveletInfo w;
    make_wavelet(cfg->wavelet, w);
    const int dim = cfg->dim;
    if (!noalloc_shape_supported(dim, cfg->Bs[0], cfg->Bs[1], dim == 3 ? cfg->Bs[2] : 1, w.X, w.Y))
        return fail(WG_EINVAL, "wg_threshold_flags_noalloc: a %s transform of %dx%dx%d blocks does not fit the "
                    "shared memory of one thread block", cfg->wavelet, cfg->Bs[0], cfg->Bs[1], dim == 3 ? cfg->Bs[2] : 1);
    BufGeo geo = {cfg->Bs[0] + 2 * cfg->g, cfg->Bs[1] + 2 * cfg->g, dim == 3 ? cfg->Bs[2] + 2 * cfg->g : 1, cfg->g};
    cudaError_t e = launch_fwt_flags_noalloc(dim, nblk, d_blocks, geo, cfg->Bs[0], cfg->Bs[1],
                                             dim == 3 ? cfg->Bs[2] : 1, cfg->neq, w.X, w.Y, eps_use,
                                             cfg->threshold_state_vector_component, d_flags, d_details,
                                             (cudaStream_t)stream);
    if (e != cudaSuccess) return cuda_fail(e, "wg_threshold_flags_noalloc", __FILE__, __LINE__);
    return WG_OK;
}

}  // extern "C"
