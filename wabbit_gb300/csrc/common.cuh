// common.cuh -- shared device-side types of the GB300 hot path.
#pragma once
#include <cuda_runtime.h>
#include <cstdint>

#include "forest.hpp"

namespace wg {

// Per-solve physics and time-stepping constants, resident on the device so
// that an RK4 step (dt included) can be captured in a CUDA graph.
struct TreeParams {
    double c0, nu, gamma_p;
    double C_eta_inv;            // 1/C_eta (colour >= 1); colour 0 -> 0
    double C_sponge_inv;
    double u_mean_set[3];
    double CFL, CFL_nu, CFL_eta, C_eta, C_sponge;
    double dt_fixed, dt_max, time_max, write_time, tsave_stats;
    int    penalization, use_sponge, skew;
    int    pad;
    float  f_c0sq[2], f_gamma[2];   // c0^2 and gamma_p as double-float pairs
    float  f_umean[3][2];           // u_mean_set as double-float pairs
    float  fpad[2];
};

// Per-tree time state on the device.
// start value of a tree's running dt minimum: the bits of 9e9
constexpr unsigned long long kDtStartBits = 0x4200C388D0000000ull;

struct TreeClock {
    double time;
    double dt;
    unsigned long long dt_min_bits;  // running min over blocks (positive double bits); kDtStartBits between reductions
    int    diverged;
    int    reshadow;   // the anchored copy an upload wrote with a guessed constant must be redone
    // dt, dt/3 and dt/6 as double-float pairs (written with dt)
    float  f_dt[2], f_dt3[2], f_dt6[2];
    // FP32-pipe stage inputs are anchored: the hi float of every value is a
    // multiple of one quantum q per tree, rounded by (x + M) - M with
    // M = 1.5 * 2^23 * q (0: no anchoring). umax_f: running max |u| (float
    // bits) of the state written in this step, from which the next step's
    // M is chosen.
    float  anchor_M;
    unsigned umax_f;
    // usq_ready: the last RK stage recorded every block's max |u|^2 of the
    // state it wrote (BlockUsq, per block slot) and its divergence guard
    // (div_next), and nothing has changed the state since; the next dt
    // reduction then reads those maxima instead of the state
    int    usq_ready;
    int    div_next;
};

// Per-block descriptor. k1, k2: first-derivative weights (2/3)/dx, (1/12)/dx;
// m1, m2, m0: viscous weights nu*(4/3)/dx^2, nu*(1/12)/dx^2 and
// nu*(-5/2)*sum 1/dx^2 (regrouped FD_4th_central stencils of the fast path).
struct BlockDesc {
    double dx[3];
    double k1[3], k2[3], m1[3], m2[3], m0;
    // double-float weights of the FP32-pipe path, which evaluates the
    // integer-coefficient stencils 8(u+1 - u-1) - (u+2 - u-2) and
    // 16(u+1 + u-1) - (u+2 + u-2) and scales afterwards:
    // fs1 = 1/(12 dx), fs2 = nu/(12 dx^2), fsc = -30 sum fs2
    float fs1[3][2], fs2[3][2], fsc[2];
    int32_t tree;
    int32_t level;
    int32_t mask;                // slot in the mask pool, -1 = no mask
    int32_t pad;
};

// Layout of one block-major buffer: nc components of nx*ny*nz points with
// ghost width gb (nx = Bs+2gb).
struct BufGeo {
    int nx, ny, nz, gb;
    __host__ __device__ long long npts() const { return (long long)nx * ny * nz; }
};

// Arguments of one RHS / RK4-stage launch over a list of blocks.
struct StageArgs {
    const int *blk;
    const BlockDesc *desc;
    const TreeParams *tp;
    const TreeClock *clk;
    const double *in;
    BufGeo gin;
    double *out;
    BufGeo gout;
    double *un;
    BufGeo gun;
    double *acc;
    const double *mask;
    int Bs0, Bs1, Bs2, nc, stage, chunks;
    int rhs_only;        // 1: write the RHS to out (layout gout), no RK update
};

namespace strict {
cudaError_t stage(int dim, const StageArgs &a, int nblk, bool skew, bool mask, cudaStream_t s);
}
namespace fast {
cudaError_t stage(int dim, const StageArgs &a, int nblk, bool skew, bool mask, cudaStream_t s);
}

#define WG_CUDA_OK(call)                                                   \
    do {                                                                   \
        cudaError_t e__ = (call);                                          \
        if (e__ != cudaSuccess) return ::wg::cuda_fail(e__, #call, __FILE__, __LINE__); \
    } while (0)

int cuda_fail(cudaError_t e, const char *what, const char *file, int line);

// ---- kernel launchers (defined in the .cu files) -----------------------
// constant-memory set-up; must run before any stream capture
cudaError_t sync_init();
cudaError_t wavelet_init();
cudaError_t launch_sync(const Patch *patches, int npatch, double *buf, BufGeo geo, int nc, int order_predictor,
                        cudaStream_t s);
// gather form of copy / restriction stages: expand npatch patches (first[p]
// = offset of patch p's first point, total points < 2^32) into (receiver,
// sender) element offsets of component 0 (uint2 each), then move nc 8-byte
// components per point; every offset + (nc-1)*npts must be < 2^32
cudaError_t launch_expand(const Patch *patches, const unsigned *first, int npatch, unsigned total, BufGeo geo,
                          int nc, void *out, cudaStream_t s);
cudaError_t launch_gather(const void *pairs, unsigned n, void *buf, BufGeo geo, int nc, cudaStream_t s);
// prediction patches only; max_smem_doubles = largest shared-memory need
// (coarse box + x window + x-y window) of a patch, in doubles
// src_buf: the sender blocks' buffer when it is not buf (same layout)
cudaError_t launch_predict(const Patch *patches, int npatch, int max_smem_doubles, double *buf, BufGeo geo, int nc,
                           int order_predictor, cudaStream_t s, const double *src_buf = nullptr);
// RHS + RK stage (j = 1..4) over nblk blocks listed in blk
cudaError_t launch_acm_stage(int variant, int dim, int stage, const int *blk, int nblk, const BlockDesc *desc,
                             const TreeParams *tp, const TreeClock *clk, const double *in, BufGeo gin,
                             double *out, BufGeo gout, double *un, BufGeo gun, double *acc, const double *mask,
                             int Bs0, int Bs1, int Bs2, int nc, cudaStream_t s);
// double-float stage kernel (FP32-pipe stencils and RK stages, FP64 state;
// err: set to 1 by a CTA whose TMA load did not complete within a second;
// push: per slot 27 same-level receiver slots whose ghost copies the kernel
// writes along with its output, or null):
// in, u0, s2, s3 and out are float2 (hi, lo) buffers of layout gt: in the
// stage's input, u0 the anchored copy of u_n, s2 / s3 the inputs of stages
// 2 and 3 (read by stage 4); stage 4 adds the increment to un (FP64) and
// writes the copy of u_{n+1} to out; maskdf holds 5 float2 words per point
// (chi/C_eta with colour applied, u_s, sponge/C_sponge)
cudaError_t launch_acm_stage_df(int dim, int stage, int masked, const int *blk, int nblk, const BlockDesc *desc,
                                const TreeParams *tp, TreeClock *clk, const void *in, const void *u0, const void *s2,
                                const void *s3, void *out, BufGeo gt, double *un, BufGeo gun, const void *maskdf,
                                const int *push, int Bs0, int Bs1, int Bs2, const void *tmap, int march, int *err,
                                cudaStream_t s, int keep_state = 1, double *cout = nullptr,
                                const int *cpos = nullptr, const double *nin = nullptr,
                                const double *usrc = nullptr, unsigned long long *usq = nullptr);
// (march 0, 3, 4: tmap is a slab map of 4, 2 or 8 interior planes and the
// tile kernel of that slab height runs; 1: tmap is a map
// with one-plane boxes and the whole-block ring kernel runs; 2: tmap is a
// slab map and the persistent double-buffered slab kernel runs over masked
// and unmasked blocks at once, masked then being the number of masked blocks
// at the head of blk; keep_state: see launch_acm_stage_df in k_acm_df.cu,
// 0 times stage 4 without storing u_n+1)
// slab height of the TMA tile form of the double-float stage kernel (3-D,
// Bs0*Bs1 = 256), 0 where it does not apply; tmap (a CUtensorMap over the
// stage-input buffer: dims nx, ny, nz*nc*slots; box nx, ny, zt+4) selects it
int tile_slab(int dim, int Bs0, int Bs1, int Bs2, int g);
// double-float copy of the interiors of the listed blocks of an FP64 buffer
// (push: same-level ghost copies as in the stage kernel, or null)
// (only_if_flagged: only blocks of trees whose TreeClock::reshadow is set;
// cpos: src is a compact array (position, component, z, y, x), block b at
// position cpos[b], and gs is not used)
cudaError_t launch_shadow(const int *blk, int nblk, const double *src, BufGeo gs, void *dst, BufGeo gd, int nc,
                          int Bs0, int Bs1, int Bs2, const int *push, const BlockDesc *desc, const TreeClock *clk,
                          cudaStream_t s, int only_if_flagged = 0, const int *cpos = nullptr);
// after an upload that wrote the anchored copy with the trees' current
// constant: the constant from the merged running max, and reshadow set
// where it differs from the one used
cudaError_t launch_anchor_check(TreeClock *clk, const int *trees, int ntrees, cudaStream_t s);
// anchoring constant of the FP32-pipe stage inputs (TreeClock::anchor_M):
// reset of the running max, and the constant from the state (scan) or from
// the running max an interior upload merged
cudaError_t launch_umax_reset(TreeClock *clk, const int *trees, int ntrees, cudaStream_t s);
cudaError_t launch_anchor_from_state(const int *slots, int nblk, const double *A, BufGeo ga, int nc, int Bx, int By,
                                     int Bz, const BlockDesc *desc, TreeClock *clk, const int *trees, int ntrees,
                                     int scan, cudaStream_t s);
// the per-step ghost sync of a double-float buffer as one persistent launch:
// npairs restriction entries (gather form) and then npatch prediction
// patches (largest first; max_smem_doubles: the largest need per component);
// ctr: three zeroed counters of this stream (left zeroed), err: set when a
// wait for the restrictions ran out
cudaError_t launch_sync_df_fused(const void *pairs, unsigned npairs, const Patch *patches, int npatch,
                                 int max_smem_doubles, void *buf, BufGeo geo, int nc, int order_predictor,
                                 const BlockDesc *desc, const TreeClock *clk, unsigned *ctr, int *err, cudaStream_t s,
                                 int min_ctas);
cudaError_t launch_predict_df(const Patch *patches, int npatch, int max_smem_doubles, void *buf, BufGeo geo, int nc,
                              int order_predictor, const BlockDesc *desc, const TreeClock *clk, cudaStream_t s,
                              int min_ctas = 1);
cudaError_t launch_rhs_only(int variant, int dim, const int *blk, int nblk, const BlockDesc *desc,
                            const TreeParams *tp, const double *in, BufGeo gin, double *rhs, const double *mask,
                            int Bs0, int Bs1, int Bs2, int nc, cudaStream_t s);
// fixed sphere of the penalisation (3-D): centre, radius, smoothing width,
// domain and block size
struct SphereArgs {
    double centre[3];
    double radius, h;
    double domain[3];
    int Bs[3];
};
// cand: (level, x, y, z) of candidate blocks
cudaError_t launch_sphere_flags(const int4 *cand, int n, const SphereArgs &a, int *flags, cudaStream_t s);
cudaError_t launch_sphere_fill(const int4 *cand, const int *slot, int n, const SphereArgs &a, double *mask,
                               float2 *mask_df, double c_eta_inv, cudaStream_t s);
// dt of the listed trees in one launch (the last CTA finalises; done: a
// zeroed counter of this stream, left zeroed); every TreeClock's dt_min_bits
// holds kDtStartBits between reductions
cudaError_t launch_dt(int dim, const int *blk, int nblk, const BlockDesc *desc, const TreeParams *tp,
                      TreeClock *clk, const double *u, BufGeo geo, int Bs0, int Bs1, int Bs2, int ntrees,
                      const int *trees, unsigned *done, cudaStream_t s, int step_start = 0,
                      const int *upos = nullptr, unsigned long long *usq = nullptr);
// (upos: u is indexed by upos[slot] instead of the slot, e.g. a compact
// interior array with geo = {Bs0, Bs1, Bs2, 0}; usq: the per-slot maxima
// the last RK stage records: read instead of the state for the trees whose
// TreeClock::usq_ready is set, set back to zero for every listed block)

// time += dt for the listed trees; usq_ready: the step's last stage recorded
// the per-block maxima of the state it wrote (TreeClock::usq_ready)
cudaError_t launch_clock_advance(TreeClock *clk, const int *trees, int ntrees, cudaStream_t s, int usq_ready = 0);
// max |u| per component over the interiors of the listed blocks (Bs2 = 1 in 2-D)
cudaError_t launch_norm_linf(const int *blk, int nblk, const double *u, BufGeo geo, int Bs0, int Bs1, int Bs2, int nc,
                             double *out, cudaStream_t s);
// interior exchange state <-> compact array, one CTA row per (block,
// component); towards the state it merges max |u| into clk (when given) and
// optionally also writes the anchored double-float copy shadow (thin layout
// gs, same-level ghost pushes), anchored with the trees' current constant
// (launch_anchor_check decides whether that was the right one)
cudaError_t launch_interior_xfer(const int *slots, int nblk, double *compact, double *A, BufGeo ga, int nc, int Bx,
                                 int By, int Bz, int to_state, const BlockDesc *desc, TreeClock *clk, cudaStream_t s,
                                 void *shadow = nullptr, BufGeo gs = BufGeo{0, 0, 0, 0}, const int *push = nullptr);
cudaError_t launch_fwt_flags(int dim, const int *blk, int nblk, const double *u, BufGeo geo, int Bs0, int Bs1,
                             int Bs2, int nc, int wavelet_x, int wavelet_y, const double *eps_use,
                             const int *tsvc, int *flags, double *details, cudaStream_t s, int input_is_wd = 0);
// one-level FWT (spaghetti order) / IWT of the interiors of the listed blocks,
// in place; the ghost nodes must be synchronised (IWT: with spaghetti data)
cudaError_t launch_wavelet_decompose(int dim, const int *blk, int nblk, double *u, BufGeo geo, int Bs0, int Bs1,
                                     int Bs2, int nc, int wavelet_x, int wavelet_y, cudaStream_t s);
cudaError_t launch_wavelet_reconstruct(int dim, const int *blk, int nblk, double *u, BufGeo geo, int Bs0, int Bs1,
                                       int Bs2, int nc, int wavelet_x, int wavelet_y, cudaStream_t s);
// the FWT of waveletDecomposition_optimized_block with the pass results it
// leaves on the ghost rows/planes of its window (adapt on the full tree)
cudaError_t launch_wavelet_decompose_window(int dim, const int *blk, int nblk, double *u, BufGeo geo, int Bs0, int Bs1,
                                            int Bs2, int nc, int wavelet_x, int wavelet_y, cudaStream_t s);
// full-tree adaptation with coarse extension (k_lifted.cu); the structs are
// in lifted.hpp
struct FilterEntry;
struct ScBox;
struct BoxOp;
cudaError_t launch_xcopy(const Patch *p, int n, const double *sbuf, double *dbuf, BufGeo geo, int nc, cudaStream_t s);
cudaError_t launch_hd_filter(int dim, const FilterEntry *ent, int n, const double *A, const double *T, BufGeo geo,
                             int Bx, int By, int Bz, int nc, const double *hd, int hd_lo, int hd_n, double *scratch,
                             cudaStream_t s);
cudaError_t launch_scbox(const ScBox *b, int n, const FilterEntry *ent, const double *A, const double *T, BufGeo geo,
                         int hx, int hy, int hz, int nc, double *scratch, cudaStream_t s);
cudaError_t launch_restrict_scratch(const Patch *p, int n, const double *scratch, double *A, BufGeo geo, int hx,
                                    int hy, int hz, int nc, cudaStream_t s);
cudaError_t launch_boxop(const BoxOp *o, int n, double *A, const double *T, BufGeo geo, int nc, cudaStream_t s);
cudaError_t launch_blockcopy(const int *slots, int n, const double *src, double *dst, long long per_block,
                             cudaStream_t s);
// items: {slot, lo[3], hi[3], io[3]} ints; det: n x nc maxima
cudaError_t launch_zone_detail(const void *items, int n, const double *A, BufGeo geo, int nc, int dim, double *det,
                               cudaStream_t s);
// wc_threshold_tree on spaghetti data (thresh, tsvc: nc host values, nc <= 8)
cudaError_t launch_wc_threshold(int dim, const int *blk, int nblk, double *u, BufGeo geo, int Bs0, int Bs1, int Bs2,
                                int nc, const double *thresh, const int *tsvc, cudaStream_t s);
// allocation-free variant (static device scratch, contiguous blocks 0..nblk-1)
int noalloc_max_blocks();
bool noalloc_shape_supported(int dim, int Bs0, int Bs1, int Bs2, int wavelet_x, int wavelet_y);
cudaError_t launch_fwt_flags_noalloc(int dim, int nblk, const double *u, BufGeo geo, int Bs0, int Bs1, int Bs2,
                                     int nc, int wavelet_x, int wavelet_y, const double *eps_host,
                                     const int *tsvc_host, int *flags, double *details, cudaStream_t s);
// child_slot: 2^dim arena slots per parent, daughter k of parent p at [p * 2^dim + k]
cudaError_t launch_refine(int dim, const int *parent, int nparent, const int *child_slot, const double *u,
                          BufGeo geo, int Bs0, int Bs1, int Bs2, int nc, int order_predictor, cudaStream_t s);

}  // namespace wg
