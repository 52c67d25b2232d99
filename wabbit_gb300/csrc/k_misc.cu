// k_misc.cu -- time-step selection and stage dispatch.
//
// dt: GET_DT_BLOCK_ACM (LIB/EQUATION/ACMnew/module_ACM.f90:617-691) per block,
// min over the blocks of each tree (the reference's MPI_Allreduce(MIN),
// LIB/TIME/calculate_time_step.f90:28-48), then the output-time trimming of
// calculate_time_step.f90:50-118 -- all on the device, so that a whole RK4
// step can be captured in a CUDA graph.
#include <algorithm>

#include "common.cuh"
#include "df.cuh"
#include "exact.cuh"
#include "umag.cuh"

namespace wg {

template <int DIM>
__device__ __forceinline__ float usq_approx(const double *ub, long long np, long long o) {
    const float a = trunc_abs_f(ub[o]), b = trunc_abs_f(ub[np + o]);
    float s = a * a + b * b;
    if (DIM == 3) {
        const float c = trunc_abs_f(ub[2 * np + o]);
        s += c * c;
    }
    return s;
}

// the reference's u*u + v*v (+ w*w) with every operation rounded in order
template <int DIM>
__device__ __forceinline__ double usq_exact(const double *ub, long long np, long long o) {
    const double a = ub[o], bb = ub[np + o];
    double s = __dadd_rn(__dmul_rn(a, a), __dmul_rn(bb, bb));
    if (DIM == 3) {
        const double c = ub[2 * np + o];
        s = __dadd_rn(s, __dmul_rn(c, c));
    }
    return s;
}

// GET_DT_BLOCK_ACM of one block from its max |u|^2 (u_mag; the callers
// take the atomic min over the blocks of its tree, calculate_time_step.f90:28-48)
template <int DIM>
__device__ __forceinline__ double dt_of_block(const TreeParams &p, const BlockDesc &d, double u_mag) {
    const double u_eigen = __dadd_rn(sqrt(u_mag), sqrt(__dadd_rn(__dmul_rn(p.c0, p.c0), u_mag)));
    double dxmin = d.dx[0];
    for (int k = 1; k < DIM; k++) dxmin = fmin(dxmin, d.dx[k]);
    double dt = u_eigen >= 1.0e-6 ? __ddiv_rn(__dmul_rn(p.CFL, dxmin), u_eigen) : 1.0e-2;
    if (p.nu > 1.0e-13) dt = fmin(dt, __ddiv_rn(__dmul_rn(p.CFL_nu, __dmul_rn(dxmin, dxmin)), p.nu));
    if (p.gamma_p > 0) dt = fmin(dt, __dmul_rn(p.CFL_eta, p.gamma_p));
    if (p.penalization) dt = fmin(dt, __dmul_rn(p.CFL_eta, p.C_eta));
    if (p.use_sponge) dt = fmin(dt, __dmul_rn(p.CFL_eta, p.C_sponge));
    return dt;
}

// dt_kernel: per block the max |u|^2 over the interior -- the maximum the
// last RK stage recorded while it wrote the state (trees with
// TreeClock::usq_ready), else from the state (two passes, umag.cuh) -> the
// block's dt -> atomic min per tree; a value outside the divergence guard
// sets the tree's flag. The last CTA to finish (counter *done, set back to
// zero by it) finalises the listed trees, so the whole reduction is one
// launch.
__device__ void dt_finalize_tree(const TreeParams *tp, TreeClock *clk, int t, int step_start);

// the max |u|^2 of block b from its state (two passes, umag.cuh), its dt
// merged into the tree's minimum, the divergence guard into its flag; every
// thread of the CTA calls it
template <int DIM, int BS>
__device__ __forceinline__ void dt_scan_block(const BlockDesc &d, TreeClock *clk, const TreeParams *tp,
                                              const double *u, BufGeo geo, int Bs0_, int Bs1_, int Bs2_,
                                              const int *upos, int b) {
    const int Bs0 = BS ? BS : Bs0_, Bs1 = BS ? BS : Bs1_, Bs2 = BS ? BS : Bs2_;
    constexpr int kCache = 4096;
    __shared__ float s32[kCache];
    __shared__ float red32[8];
    __shared__ double red64[8];
    const long long np = geo.npts();
    const int nint = Bs0 * Bs1 * (DIM == 3 ? Bs2 : 1);
    const bool cache = nint <= kCache;
    const double *ub = u + (long long)(upos ? upos[b] : b) * (DIM + 1) * np;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    auto offset = [&](int q) {
        const int ix = q % Bs0, iy = (q / Bs0) % Bs1, iz = DIM == 3 ? q / (Bs0 * Bs1) : 0;
        return ((long long)(iz + (DIM == 3 ? geo.gb : 0)) * geo.ny + (iy + geo.gb)) * geo.nx + (ix + geo.gb);
    };
    float m32 = 0.f;
    bool ok = true;
    for (int q = threadIdx.x; q < nint; q += blockDim.x) {
        const long long o = offset(q);
#pragma unroll
        for (int c = 0; c <= DIM; c++) ok &= within_guard(ub[c * np + o]);
        const float v = usq_approx<DIM>(ub, np, o);
        if (cache) s32[q] = v;
        m32 = fmaxf(m32, v);
    }
    if (!ok) atomicOr(&clk[d.tree].diverged, 1);
    for (int w = 16; w; w >>= 1) m32 = fmaxf(m32, __shfl_xor_sync(0xffffffffu, m32, w));
    if (lane == 0) red32[warp] = m32;
    __syncthreads();
    m32 = red32[0];
    for (int w = 1; w < (int)(blockDim.x >> 5); w++) m32 = fmaxf(m32, red32[w]);
    const float thr = umag_threshold(m32);
    double m = -1.0;
    for (int q = threadIdx.x; q < nint; q += blockDim.x) {
        const long long o = offset(q);
        const float v = cache ? s32[q] : usq_approx<DIM>(ub, np, o);
        if (v >= thr) m = fmax(m, usq_exact<DIM>(ub, np, o));
    }
    for (int w = 16; w; w >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, w));
    if (lane == 0) red64[warp] = m;
    __syncthreads();
    if (threadIdx.x == 0) {
        double u_mag = red64[0];
        for (int w = 1; w < (int)(blockDim.x >> 5); w++) u_mag = fmax(u_mag, red64[w]);
        atomicMin(&clk[d.tree].dt_min_bits,
                  (unsigned long long)__double_as_longlong(dt_of_block<DIM>(tp[d.tree], d, u_mag)));
    }
}

// A grid of resident CTAs: the blocks whose tree's last RK stage recorded
// their maxima take one thread each (their dt merged per warp and tree), the
// others one CTA each in turn. BS: the block edge when all edges equal it
// (index arithmetic by shifts), 0 for the general case.
template <int DIM, int BS>
__global__ void __launch_bounds__(256) dt_kernel(const int *blk, int nblk, const BlockDesc *desc,
                                                 const TreeParams *tp, TreeClock *clk, const double *u, BufGeo geo,
                                                 int Bs0, int Bs1, int Bs2, const int *trees, int ntrees,
                                                 int step_start, unsigned *done, const int *upos,
                                                 unsigned long long *usq) {
    __shared__ int s_last;
    // a tree's flag was set before this launch and is cleared only by the
    // last CTA, after every CTA has read it
    if (usq) {
        const int span = (int)(gridDim.x * blockDim.x);
        for (int j0 = (int)(blockIdx.x * blockDim.x); j0 < nblk; j0 += span) {   // uniform over the CTA
            const int j = j0 + (int)threadIdx.x;
            int tree = -1;
            unsigned long long bits = ~0ull;
            if (j < nblk) {
                const int b = blk[j];
                const BlockDesc &d = desc[b];
                if (__ldcg(&clk[d.tree].usq_ready)) {
                    const unsigned long long e = usq[b];
                    usq[b] = 0ull;
                    tree = d.tree;
                    bits = (unsigned long long)__double_as_longlong(
                        dt_of_block<DIM>(tp[tree], d, e ? __longlong_as_double((long long)(e - 1ull)) : -1.0));
                }
            }
            // dt >= 0: the minimum of the bits is the minimum, per tree
            const unsigned grp = __match_any_sync(0xffffffffu, tree);
            const unsigned hi = __reduce_min_sync(grp, (unsigned)(bits >> 32));
            const unsigned lo = __reduce_min_sync(grp, (unsigned)(bits >> 32) == hi ? (unsigned)bits : 0xffffffffu);
            if (tree >= 0 && (threadIdx.x & 31) == (unsigned)(__ffs(grp) - 1))
                atomicMin(&clk[tree].dt_min_bits, ((unsigned long long)hi << 32) | lo);
        }
    }
    for (int i = (int)blockIdx.x; i < nblk; i += (int)gridDim.x) {
        const int b = blk[i];
        const BlockDesc &d = desc[b];
        if (usq && __ldcg(&clk[d.tree].usq_ready)) continue;   // uniform over the CTA
        dt_scan_block<DIM, BS>(d, clk, tp, u, geo, Bs0, Bs1, Bs2, upos, b);
        if (usq && threadIdx.x == 0) usq[b] = 0ull;
    }
    if (threadIdx.x == 0) {
        // acquire-release count of the finished CTAs: the last one sees every
        // other CTA's minimum (and flag) before it finalises
        unsigned n;
        asm volatile("atom.acq_rel.gpu.global.add.u32 %0, [%1], 1;" : "=r"(n) : "l"(done) : "memory");
        s_last = n == gridDim.x - 1;
    }
    __syncthreads();
    if (s_last) {
        for (int i = threadIdx.x; i < ntrees; i += blockDim.x) dt_finalize_tree(tp, clk, trees[i], step_start);
        if (threadIdx.x == 0) *done = 0u;
    }
}

// calculate_time_step.f90:28-118 after the MIN reduction, for tree t; the
// running minimum is read through L2 (the other CTAs' atomics) and set back
// to its start value for the next reduction
__device__ void dt_finalize_tree(const TreeParams *tp, TreeClock *clk, int t, int step_start) {
    const TreeParams &p = tp[t];
    TreeClock &c = clk[t];
    const double time = c.time;
    const unsigned long long mbits = __ldcg(&c.dt_min_bits);
    c.dt_min_bits = kDtStartBits;
    double dt;
    if (p.dt_fixed > 0.0) dt = p.dt_fixed;
    else {
        dt = __longlong_as_double((long long)mbits);
        if (p.dt_max > 0.0) dt = fmin(p.dt_max, dt);
    }
    if (p.write_time > 0.0) {
        const double wt = p.write_time;
        if (fmod(__dadd_rn(time, dt), wt) < fmod(__dadd_rn(time, 1e-12), wt) && !(fabs(fmod(time, wt)) < 1e-12) &&
            __dadd_rn(time, 1e-12) > 0.0)
            dt = __dsub_rn(wt, fmod(time, wt));
    }
    if (p.tsave_stats > 0.0) {
        const double ts = p.tsave_stats;
        if (fmod(__dadd_rn(time, dt), ts) < fmod(__dadd_rn(time, 1e-12), ts) && !(fabs(fmod(time, ts)) < 1e-12))
            dt = __dsub_rn(ts, fmod(time, ts));
    }
    if (__dadd_rn(time, dt) > p.time_max && time <= p.time_max) dt = __dsub_rn(p.time_max, time);
    c.dt = dt;
    // the divergence guard the last RK stage took on the state it wrote, if
    // this reduction used its maxima
    if (c.usq_ready && c.div_next) c.diverged = 1;
    c.usq_ready = 0;
    c.div_next = 0;
    const df2 f1 = df_from(dt), f3 = df_from(__ddiv_rn(dt, 3.0)), f6 = df_from(__ddiv_rn(dt, 6.0));
    c.f_dt[0] = f1.hi;
    c.f_dt[1] = f1.lo;
    c.f_dt3[0] = f3.hi;
    c.f_dt3[1] = f3.lo;
    c.f_dt6[0] = f6.hi;
    c.f_dt6[1] = f6.lo;
    // at the start of an RK step: the quantum of the stage inputs this step
    // writes, from the largest |u| the previous step wrote (unchanged if none
    // was recorded, e.g. in the FP64 precision)
    if (step_start) {
        if (c.umax_f) c.anchor_M = anchor_constant(c.umax_f);
        c.umax_f = 0u;
    }
}

__global__ void dt_finalize_kernel(const TreeParams *tp, TreeClock *clk, const int *trees, int ntrees, int step_start) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < ntrees) dt_finalize_tree(tp, clk, trees[i], step_start);
}

__global__ void clock_advance_kernel(TreeClock *clk, const int *trees, int ntrees, int usq_ready) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < ntrees) {
        TreeClock &c = clk[trees[i]];
        c.time = __dadd_rn(c.time, c.dt);
        c.usq_ready = usq_ready;
    }
}

cudaError_t launch_dt(int dim, const int *blk, int nblk, const BlockDesc *desc, const TreeParams *tp,
                      TreeClock *clk, const double *u, BufGeo geo, int Bs0, int Bs1, int Bs2, int ntrees,
                      const int *trees, unsigned *done, cudaStream_t s, int step_start, const int *upos,
                      unsigned long long *usq) {
    if (!done) return cudaErrorInvalidValue;
    if (nblk > 0) {
        const bool b16 = Bs0 == 16 && Bs1 == 16 && (dim == 2 || Bs2 == 16);
        auto k = dim == 2 ? (b16 ? dt_kernel<2, 16> : dt_kernel<2, 0>) : (b16 ? dt_kernel<3, 16> : dt_kernel<3, 0>);
        // as many CTAs as are resident at once (every CTA loops)
        int dev = 0, sms = 0, per_sm = 0;
        cudaError_t e = cudaGetDevice(&dev);
        if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, 256, 0);
        if (e != cudaSuccess) return e;
        const int grid = std::min(nblk, std::max(1, sms * per_sm));
        k<<<grid, 256, 0, s>>>(blk, nblk, desc, tp, clk, u, geo, Bs0, Bs1, Bs2, trees, ntrees, step_start, done,
                               upos, usq);
    } else {
        dt_finalize_kernel<<<(ntrees + 127) / 128, 128, 0, s>>>(tp, clk, trees, ntrees, step_start);
    }
    return cudaGetLastError();
}

cudaError_t launch_clock_advance(TreeClock *clk, const int *trees, int ntrees, cudaStream_t s, int usq_ready) {
    clock_advance_kernel<<<(ntrees + 127) / 128, 128, 0, s>>>(clk, trees, ntrees, usq_ready);
    return cudaGetLastError();
}

static StageArgs make_args(const int *blk, const BlockDesc *desc, const TreeParams *tp,
                                   const TreeClock *clk, const double *in, BufGeo gin, double *out, BufGeo gout,
                                   double *un, BufGeo gun, double *acc, const double *mask, int Bs0, int Bs1,
                                   int Bs2, int nc, int stage, int rhs_only) {
    StageArgs a;
    a.blk = blk;
    a.desc = desc;
    a.tp = tp;
    a.clk = clk;
    a.in = in;
    a.gin = gin;
    a.out = out;
    a.gout = gout;
    a.un = un;
    a.gun = gun;
    a.acc = acc;
    a.mask = mask;
    a.Bs0 = Bs0;
    a.Bs1 = Bs1;
    a.Bs2 = Bs2;
    a.nc = nc;
    a.stage = stage;
    a.chunks = 1;
    a.rhs_only = rhs_only;
    return a;
}

// variant bit 0: 1 = fast (FMA); bit 1: skew-symmetric; bit 2: masked block list
cudaError_t launch_acm_stage(int variant, int dim, int stage, const int *blk, int nblk, const BlockDesc *desc,
                             const TreeParams *tp, const TreeClock *clk, const double *in, BufGeo gin,
                             double *out, BufGeo gout, double *un, BufGeo gun, double *acc, const double *mask,
                             int Bs0, int Bs1, int Bs2, int nc, cudaStream_t s) {
    if (nblk <= 0) return cudaSuccess;
    StageArgs a = make_args(blk, desc, tp, clk, in, gin, out, gout, un, gun, acc, mask, Bs0, Bs1, Bs2, nc,
                                    stage, 0);
    const bool skew = variant & 2, masked = variant & 4;
    if (variant & 1) return fast::stage(dim, a, nblk, skew, masked, s);
    return strict::stage(dim, a, nblk, skew, masked, s);
}

cudaError_t launch_rhs_only(int variant, int dim, const int *blk, int nblk, const BlockDesc *desc,
                            const TreeParams *tp, const double *in, BufGeo gin, double *rhs, const double *mask,
                            int Bs0, int Bs1, int Bs2, int nc, cudaStream_t s) {
    if (nblk <= 0) return cudaSuccess;
    StageArgs a = make_args(blk, desc, tp, nullptr, in, gin, rhs, gin, nullptr, gin, nullptr, mask, Bs0, Bs1,
                                    Bs2, nc, 1, 1);
    const bool skew = variant & 2, masked = variant & 4;
    if (variant & 1) return fast::stage(dim, a, nblk, skew, masked, s);
    return strict::stage(dim, a, nblk, skew, masked, s);
}

// ---------------------------------------------------------------------------
// Penalisation mask of a fixed sphere on the device (create_mask_3D_acm
// 'sphere-fixed' -> draw_sphere, LIB/EQUATION/ACMnew/create_mask.f90:58-61,
// LIB/EQUATION/insects/module_geometry.f90:49-117; step_cosine4,
// LIB/HELPER/module_helpers.f90:467-487): chi is the cosine-smoothed step of
// the signed distance over the width h, colour 1, u_s = 0, no sponge. Block
// origin, spacing and point coordinates follow get_block_spacing_origin_b
// (LIB/TREE/module_treelib.f90:96-101) with every product and sum rounded
// separately, in the same order as the host mask of the workloads.

__device__ __forceinline__ double sphere_chi(const SphereArgs &a, const int4 &blk, int ix, int iy, int iz) {
    const int lv = blk.x;
    const int co[3] = {blk.y, blk.z, blk.w};
    const int ii[3] = {ix, iy, iz};
    double r2 = 0.0;
    for (int d = 0; d < 3; d++) {
        const double dx = __ddiv_rn(__dmul_rn(ldexp(1.0, -lv), a.domain[d]), (double)a.Bs[d]);
        const double x0 = __dmul_rn((double)(co[d] * a.Bs[d]), dx);
        const double x = __dadd_rn(x0, __dmul_rn((double)ii[d], dx));
        const double e = __dsub_rn(x, a.centre[d]);
        r2 = d == 0 ? __dmul_rn(e, e) : __dadd_rn(r2, __dmul_rn(e, e));
    }
    const double dist = __dsub_rn(__dsqrt_rn(r2), a.radius);
    if (dist <= -a.h) return 1.0;
    if (dist >= a.h) return 0.0;
    const double t = __ddiv_rn(__dmul_rn(__dadd_rn(dist, a.h), 3.141592653589793), __dmul_rn(2.0, a.h));
    return __dmul_rn(0.5, __dadd_rn(1.0, cos(t)));
}

// flags[k] = 1 if chi > 0 at an interior point of candidate k
__global__ void __launch_bounds__(256) sphere_flag_kernel(const int4 *cand, int n, SphereArgs a, int *flags) {
    const int k = blockIdx.x;
    if (k >= n) return;
    const int4 blk = cand[k];
    const int npts = a.Bs[0] * a.Bs[1] * a.Bs[2];
    int any = 0;
    for (int i = threadIdx.x; i < npts; i += blockDim.x) {
        const int ix = i % a.Bs[0], iy = (i / a.Bs[0]) % a.Bs[1], iz = i / (a.Bs[0] * a.Bs[1]);
        any |= sphere_chi(a, blk, ix, iy, iz) > 0.0;
    }
    any = __syncthreads_or(any);
    if (threadIdx.x == 0) flags[k] = any;
}

// the interior mask of block k into pool slot slot[k]: chi, u_s (3), colour,
// sponge in FP64, and the double-float words of the FP32-pipe stage
// (chi / C_eta, u_s, sponge / C_sponge)
__global__ void __launch_bounds__(256) sphere_fill_kernel(const int4 *cand, const int *slot, int n, SphereArgs a,
                                                          double *mask, float2 *mask_df, double c_eta_inv) {
    const int k = blockIdx.x;
    if (k >= n) return;
    const int4 blk = cand[k];
    const long long ni = (long long)a.Bs[0] * a.Bs[1] * a.Bs[2];
    double *m = mask + (long long)slot[k] * 6 * ni;
    float2 *md = mask_df ? mask_df + (long long)slot[k] * 5 * ni : nullptr;
    for (long long i = threadIdx.x; i < ni; i += blockDim.x) {
        const int ix = (int)(i % a.Bs[0]), iy = (int)((i / a.Bs[0]) % a.Bs[1]), iz = (int)(i / (a.Bs[0] * a.Bs[1]));
        const double chi = sphere_chi(a, blk, ix, iy, iz);
        m[i] = chi;
        m[ni + i] = 0.0;
        m[2 * ni + i] = 0.0;
        m[3 * ni + i] = 0.0;
        m[4 * ni + i] = 1.0;
        m[5 * ni + i] = 0.0;
        if (md) {
            const double v = __dmul_rn(chi, c_eta_inv);
            const float hi = __double2float_rn(v);
            md[i] = make_float2(hi, __double2float_rn(__dsub_rn(v, (double)hi)));
            for (int w = 1; w < 5; w++) md[w * ni + i] = make_float2(0.f, 0.f);
        }
    }
}

cudaError_t launch_sphere_flags(const int4 *cand, int n, const SphereArgs &a, int *flags, cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    if (!cand || !flags) return cudaErrorInvalidValue;
    sphere_flag_kernel<<<n, 256, 0, s>>>(cand, n, a, flags);
    return cudaGetLastError();
}

cudaError_t launch_sphere_fill(const int4 *cand, const int *slot, int n, const SphereArgs &a, double *mask,
                               float2 *mask_df, double c_eta_inv, cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    if (!cand || !slot || !mask) return cudaErrorInvalidValue;
    sphere_fill_kernel<<<n, 256, 0, s>>>(cand, slot, n, a, mask, mask_df, c_eta_inv);
    return cudaGetLastError();
}

// componentWiseNorm_tree (LIB/OPERATORS/componentWiseNorm_tree.f90:1-140),
// Linfty over the interiors of the listed blocks: one CTA per (block,
// component) reduces max |u| and merges it into out[c] with an integer
// atomic max on the bits (non-negative doubles order like their bits).
// out must hold zeros on entry.
__global__ void __launch_bounds__(256) norm_linf_kernel(const int *blk, const double *u, BufGeo geo, int Bs0, int Bs1,
                                                        int Bs2, int nc, unsigned long long *out) {
    __shared__ unsigned long long red[8];
    const int b = blk[blockIdx.x], c = blockIdx.y;
    const long long np = geo.npts();
    const double *ub = u + ((long long)b * nc + c) * np;
    const int z3 = geo.nz > 1;
    const int nint = Bs0 * Bs1 * Bs2;
    unsigned long long m = 0ull;
    for (int q = threadIdx.x; q < nint; q += blockDim.x) {
        const int ix = q % Bs0, iy = (q / Bs0) % Bs1, iz = q / (Bs0 * Bs1);
        const double v = ub[((long long)(iz + (z3 ? geo.gb : 0)) * geo.ny + (iy + geo.gb)) * geo.nx + (ix + geo.gb)];
        const unsigned long long a = (unsigned long long)dbits(v) & 0x7fffffffffffffffull;
        m = a > m ? a : m;
    }
    for (int o = 16; o; o >>= 1) {
        const unsigned long long t = __shfl_xor_sync(0xffffffffu, m, o);
        m = t > m ? t : m;
    }
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = m;
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int w = 1; w < (int)(blockDim.x >> 5); w++) m = red[w] > m ? red[w] : m;
        atomicMax(out + c, m);
    }
}

cudaError_t launch_norm_linf(const int *blk, int nblk, const double *u, BufGeo geo, int Bs0, int Bs1, int Bs2, int nc,
                             double *out, cudaStream_t s) {
    cudaError_t e = cudaMemsetAsync(out, 0, sizeof(double) * nc, s);
    if (e != cudaSuccess || nblk <= 0) return e;
    norm_linf_kernel<<<dim3(nblk, nc), 256, 0, s>>>(blk, u, geo, Bs0, Bs1, Bs2, nc,
                                                    reinterpret_cast<unsigned long long *>(out));
    return cudaGetLastError();
}

}  // namespace wg
