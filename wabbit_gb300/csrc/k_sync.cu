// k_sync.cu -- ghost-node synchronisation from a flat patch table.
//
// Replaces the per-block, per-neighbour loops of sync_ghosts_generic
// (LIB/MPI/synchronize_ghosts_generic.f90:181-343) and
// unpack_ghostlayers_internal (LIB/MPI/xfer_block_data.f90:321-437): one warp
// per patch copies, decimates (restrict_data, restrict_predict_data.f90:45-99)
// or interpolates (predict_data -> prediction, module_wavelets.f90:96-284)
// the sender data straight into the receiver's ghost box. A launch covers one
// stage; stages run in order so that predictions read ghost nodes that the
// previous stage filled.
//
// The interpolation is evaluated per fine point in the reference's separable
// order (x on coarse rows, then y, then z, each sum left to right) with
// explicit round-to-nearest multiplies and adds, so the ghost values are
// bit-identical to the reference's. Double-float buffers (FP32-pipe
// precision) get the same passes in double-float arithmetic
// (predict_df_kernel), and the per-step copy / restriction stages run in
// gather form (expand_kernel, gather_kernel).
#include "common.cuh"
#include "predict.cuh"
#include "df.cuh"
#include "exact.cuh"
#include <algorithm>
#include <atomic>

namespace wg {

// Division by a divisor fixed for a patch: q = floor(n / d) as the high
// word of n * ceil(2^64 / d), exact for every 32-bit n and d >= 2 (the error
// term n * (ceil(2^64/d) d - 2^64) / 2^64 stays below n d / 2^64 < 1). The
// element loops of a prediction patch divide every index by up to four such
// extents, and the generic 32-bit division was most of the kernel's
// instructions.
struct FastDiv {
    unsigned d;
    unsigned long long m;
    __device__ __forceinline__ unsigned div(unsigned n) const {
        return d > 1u ? (unsigned)__umul64hi((unsigned long long)n, m) : n;
    }
};

__device__ __forceinline__ unsigned long long fastdiv_magic(unsigned d) { return d > 1u ? ~0ull / d + 1ull : 0ull; }

// the multipliers of up to 9 divisors of a patch, formed once per CTA (a
// 64-bit division each) into shared memory mag[]; every thread calls it,
// and it ends past a barrier
__device__ __forceinline__ void fastdiv_setup(unsigned long long *mag, const unsigned (&d)[9]) {
    if (threadIdx.x < 9) {
        unsigned v = d[0];
#pragma unroll
        for (int k = 1; k < 9; k++)
            if ((int)threadIdx.x == k) v = d[k];
        mag[threadIdx.x] = fastdiv_magic(v);
    }
    __syncthreads();
}

// Copy and restriction patches: one warp per patch, one lane per receiver
// row (x fastest), so the index arithmetic is one division per row.
__global__ void __launch_bounds__(128) sync_kernel(const Patch *__restrict__ patches, int npatch, double *buf,
                                                   BufGeo geo, int nc, int order_idx, int ncoef) {
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (warp >= npatch) return;
    const Patch p = patches[warp];
    const int ex = p.rhi[0] - p.rlo[0] + 1, ey = p.rhi[1] - p.rlo[1] + 1, ez = p.rhi[2] - p.rlo[2] + 1;
    const long long npts = geo.npts();
    double *dst = buf + (long long)p.dst * nc * npts;
    const double *src = buf + (long long)p.src * nc * npts;
    const int step = p.op == 1 ? 2 : 1;
    const int rows = ey * ez;
    for (int r = lane; r < rows; r += 32) {
        const int iy = r % ey, iz = r / ey;
        const long long di = ((long long)(p.rlo[2] + iz) * geo.ny + (p.rlo[1] + iy)) * geo.nx + p.rlo[0];
        long long si;
        if (p.op == 0)
            si = ((long long)(p.slo[2] + iz) * geo.ny + (p.slo[1] + iy)) * geo.nx + p.slo[0];
        else
            si = ((long long)(p.slo[2] + 2 * (p.blo[2] + iz)) * geo.ny + (p.slo[1] + 2 * (p.blo[1] + iy))) * geo.nx +
                 p.slo[0] + 2 * p.blo[0];
        // sender and receiver boxes of one stage never overlap (checked when
        // the table is built), so the loads of a row need not wait for its
        // stores
        for (int c = 0; c < nc; c++) {
            const double *__restrict__ sr = src + c * npts + si;
            double *__restrict__ dr = dst + c * npts + di;
            for (int ix = 0; ix < ex; ix++) dr[ix] = sr[step * ix];
        }
    }
}

// Gather form of the copy and restriction stages: the patches of a stage are
// expanded once per grid into (receiver, sender) element offsets of
// component 0, in patch order with x fastest. Every ghost point is then one
// thread that moves all nc components, so the loads of the nc components are
// in flight together and consecutive threads touch consecutive addresses.
__global__ void expand_kernel(const Patch *__restrict__ patches, const unsigned *__restrict__ first, int npatch,
                              unsigned total, BufGeo geo, int nc, uint2 *__restrict__ out) {
    const unsigned i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= total) return;
    int lo = 0, hi = npatch - 1;                     // last patch with first[p] <= i
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (first[mid] <= i) lo = mid;
        else hi = mid - 1;
    }
    const Patch p = patches[lo];
    const int ex = p.rhi[0] - p.rlo[0] + 1, ey = p.rhi[1] - p.rlo[1] + 1;
    const int k = (int)(i - first[lo]);
    const int ix = k % ex, iy = (k / ex) % ey, iz = k / (ex * ey);
    const unsigned long long bs = (unsigned long long)nc * geo.npts();
    const unsigned long long d = p.dst * bs + ((unsigned long long)(p.rlo[2] + iz) * geo.ny + (p.rlo[1] + iy)) * geo.nx +
                                 (p.rlo[0] + ix);
    unsigned long long sidx;
    if (p.op == 0)
        sidx = ((unsigned long long)(p.slo[2] + iz) * geo.ny + (p.slo[1] + iy)) * geo.nx + (p.slo[0] + ix);
    else
        sidx = ((unsigned long long)(p.slo[2] + 2 * (p.blo[2] + iz)) * geo.ny + (p.slo[1] + 2 * (p.blo[1] + iy))) *
                   geo.nx + (p.slo[0] + 2 * (p.blo[0] + ix));
    out[i] = make_uint2((unsigned)d, (unsigned)(p.src * bs + sidx));
}

template <int NC>
__global__ void __launch_bounds__(256) gather_kernel(const uint2 *__restrict__ pairs, unsigned n,
                                                     unsigned long long *buf, unsigned cs) {
    const unsigned i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint2 e = __ldg(pairs + i);
    unsigned long long v[NC];
#pragma unroll
    for (int c = 0; c < NC; c++) v[c] = buf[e.y + c * cs];
#pragma unroll
    for (int c = 0; c < NC; c++) buf[e.x + c * cs] = v[c];
}

// Prediction patches: one CTA per patch, one component at a time. The coarse
// sender box is staged in shared memory; the reference's separable passes
// are then evaluated only over the windows the receiver box needs: x values
// on the even rows/planes around it, x-y values on its rows and the even
// planes around it, and finally the z pass on the receiver box itself. Each
// value is the same expression (term order, rounding) as the reference's.
__device__ __forceinline__ double interp_line(const double *c, const double *v, int stride, int first, int nc) {
    double s = __dmul_rn(c[0], v[(long long)first * stride]);
    for (int m = 1; m < nc; m++) s = __dadd_rn(s, __dmul_rn(c[m], v[(long long)(first + m) * stride]));
    return s;
}

// the order-4 predictor (-1, 9, 9, -1)/16 with its products on the integer
// pipe (exact.cuh: -2^-4 and 9 2^-4 times v, bit-identical to the FP64
// multiply); the FP64 multiplies redo it where a product left the exact range
__device__ __forceinline__ double interp_pred(const double *c, const double *v, int stride, int first, int nc) {
    if (nc == 4) {
        constexpr long long kNeg = (long long)0x8000000000000000ULL;
        const double *q = v + (long long)first * stride;
        bool bad = false;
        double s = pow2_mul(q[0], -4, kNeg, bad);
        s = __dadd_rn(s, short_mul(q[stride], 9, -4, 0, bad));
        s = __dadd_rn(s, short_mul(q[2 * (long long)stride], 9, -4, 0, bad));
        s = __dadd_rn(s, pow2_mul(q[3 * (long long)stride], -4, kNeg, bad));
        if (!bad) return s;
    }
    return interp_line(c, v, stride, first, nc);
}

__global__ void __launch_bounds__(256) predict_kernel(const Patch *__restrict__ patches, const double *sbuf,
                                                      double *buf, BufGeo geo, int nc, int order_idx, int ncoef) {
    extern __shared__ double sm[];
    const Patch p = patches[blockIdx.x];
    const int cx = p.shi[0] - p.slo[0] + 1, cy = p.shi[1] - p.slo[1] + 1, cz = p.shi[2] - p.slo[2] + 1;
    const int Fx = 2 * cx - 1, Fy = 2 * cy - 1, Fz = 2 * cz - 1;
    const int h = ncoef - 1;
    const double *cf = c_pred[order_idx];
    // receiver box in fine indices
    const int ex = p.rhi[0] - p.rlo[0] + 1, ey = p.rhi[1] - p.rlo[1] + 1, ez = p.rhi[2] - p.rlo[2] + 1;
    const int x0 = p.blo[0], y0 = p.blo[1], z0 = p.blo[2];
    // even-row / even-plane windows
    int yw0 = max(0, y0 - h), yw1 = min(Fy - 1, y0 + ey - 1 + h);
    yw0 += yw0 & 1;
    yw1 -= yw1 & 1;
    int zw0 = max(0, z0 - h), zw1 = min(Fz - 1, z0 + ez - 1 + h);
    zw0 += zw0 & 1;
    zw1 -= zw1 & 1;
    const int ny = (yw1 - yw0) / 2 + 1, nz = (zw1 - zw0) / 2 + 1;
    const int ncp = cx * cy * cz;
    __shared__ unsigned long long mag[9];
    fastdiv_setup(mag, {(unsigned)cx, (unsigned)cy, (unsigned)ex, (unsigned)ey, (unsigned)ny, 1u, 1u, 1u, 1u});
    const FastDiv f_cx{(unsigned)cx, mag[0]}, f_cy{(unsigned)cy, mag[1]}, f_ex{(unsigned)ex, mag[2]},
        f_ey{(unsigned)ey, mag[3]}, f_ny{(unsigned)ny, mag[4]};
    double *C = sm;                       // coarse box
    double *X = C + ncp;                  // ex * ny * nz
    double *XY = X + ex * ny * nz;        // ex * ey * nz
    const long long npts = geo.npts();
    for (int c = 0; c < nc; c++) {
        const double *src = sbuf + ((long long)p.src * nc + c) * npts;
        double *dst = buf + ((long long)p.dst * nc + c) * npts;
        for (int i = threadIdx.x; i < ncp; i += blockDim.x) {
            const int kx = (int)f_cx.div(i), x = i - kx * cx;
            const int z = (int)f_cy.div(kx), y = kx - z * cy;
            C[i] = src[((long long)(p.slo[2] + z) * geo.ny + (p.slo[1] + y)) * geo.nx + (p.slo[0] + x)];
        }
        __syncthreads();
        // x pass on even rows / planes
        for (int i = threadIdx.x; i < ex * ny * nz; i += blockDim.x) {
            const int kx = (int)f_ex.div(i), ix = i - kx * ex;
            const int kz = (int)f_ny.div(kx), jy = kx - kz * ny;
            const int fx = x0 + ix, cyy = (yw0 >> 1) + jy, czz = (zw0 >> 1) + kz;
            const double *row = C + ((long long)czz * cy + cyy) * cx;
            double v;
            if (!(fx & 1)) v = row[fx >> 1];
            else if (fx < h || fx > Fx - 1 - h) v = 0.0;
            else v = interp_pred(cf, row, 1, (fx - h) >> 1, ncoef);
            X[i] = v;
        }
        __syncthreads();
        // y pass on the receiver rows, even planes
        for (int i = threadIdx.x; i < ex * ey * nz; i += blockDim.x) {
            const int kx = (int)f_ex.div(i), ix = i - kx * ex;
            const int kz = (int)f_ey.div(kx), j = kx - kz * ey;
            const int fy = y0 + j;
            const double *col = X + (long long)kz * ny * ex + ix;     // stride ex along the row window
            double v;
            if (!(fy & 1)) v = col[(long long)((fy - yw0) >> 1) * ex];
            else if (fy < h || fy > Fy - 1 - h) v = 0.0;
            else v = interp_pred(cf, col, ex, (fy - h - yw0) >> 1, ncoef);
            XY[i] = v;
        }
        __syncthreads();
        // z pass on the receiver box, write out
        for (int i = threadIdx.x; i < ex * ey * ez; i += blockDim.x) {
            const int kx = (int)f_ex.div(i), ix = i - kx * ex;
            const int k = (int)f_ey.div(kx), j = kx - k * ey;
            const int fz = z0 + k;
            const double *pl = XY + (long long)j * ex + ix;            // stride ex*ey along the plane window
            double v;
            if (!(fz & 1)) v = pl[(long long)((fz - zw0) >> 1) * ex * ey];
            else if (fz < h || fz > Fz - 1 - h) v = 0.0;
            else v = interp_pred(cf, pl, ex * ey, (fz - h - zw0) >> 1, ncoef);
            dst[((long long)(p.rlo[2] + k) * geo.ny + (p.rlo[1] + j)) * geo.nx + (p.rlo[0] + ix)] = v;
        }
        __syncthreads();
    }
}

// Prediction into double-float buffers (FP32-pipe path): the same windows
// and separable passes, evaluated in double-float arithmetic on the FP32
// units with the predictors' integer weights (1)/2, (-1,9)/16,
// (3,-25,150)/256, (-5,49,-245,1225)/2048 applied to symmetric pair sums
// and the power-of-two scale applied exactly; all components of a patch in
// one pass. Accuracy a few 2^-47 relative, like the stencils it feeds.
template <int NCOEF>
__device__ __forceinline__ df2 interp_df(const float2 *v, int stride, int first) {
    constexpr float w2[1] = {1.f}, w4[2] = {-1.f, 9.f}, w6[3] = {3.f, -25.f, 150.f},
                    w8[4] = {-5.f, 49.f, -245.f, 1225.f};
    constexpr float scale = NCOEF == 2 ? 0.5f : NCOEF == 4 ? 0.0625f : NCOEF == 6 ? 0.00390625f : 0.00048828125f;
    df2 acc = {0.f, 0.f};
#pragma unroll
    for (int m = 0; m < NCOEF / 2; m++) {
        const float w = NCOEF == 2 ? w2[m] : NCOEF == 4 ? w4[m] : NCOEF == 6 ? w6[m] : w8[m];
        const float2 a = v[(long long)(first + m) * stride], b = v[(long long)(first + NCOEF - 1 - m) * stride];
        const df2 s = df_add_nr({a.x, a.y}, {b.x, b.y});
        const float p = s.hi * w;
        const df2 t = {p, fmaf(s.lo, w, fmaf(s.hi, w, -p))};
        acc = m == 0 ? t : df_add_nr(acc, t);
    }
    return df_norm(df_pow2(acc, scale));
}

// One prediction patch by the whole CTA (sf: the CTA's dynamic shared
// memory, cg components per pass). The coarse box is read through L2
// (ld.global.cg): in the fused sync the restrictions of the same launch, run
// by other CTAs, wrote some of it, and a line this SM's L1 held from before
// could be stale. Every thread ends past a barrier, so the caller may reuse
// sf at once.
template <int NCOEF>
__device__ __forceinline__ void predict_df_patch(const Patch &p, float2 *buf, BufGeo geo, int nc, int cg, float M,
                                                 float2 *sf) {
    const int cx = p.shi[0] - p.slo[0] + 1, cy = p.shi[1] - p.slo[1] + 1, cz = p.shi[2] - p.slo[2] + 1;
    const int Fx = 2 * cx - 1, Fy = 2 * cy - 1, Fz = 2 * cz - 1;
    constexpr int h = NCOEF - 1;
    const int ex = p.rhi[0] - p.rlo[0] + 1, ey = p.rhi[1] - p.rlo[1] + 1, ez = p.rhi[2] - p.rlo[2] + 1;
    const int x0 = p.blo[0], y0 = p.blo[1], z0 = p.blo[2];
    int yw0 = max(0, y0 - h), yw1 = min(Fy - 1, y0 + ey - 1 + h);
    yw0 += yw0 & 1;
    yw1 -= yw1 & 1;
    int zw0 = max(0, z0 - h), zw1 = min(Fz - 1, z0 + ez - 1 + h);
    zw0 += zw0 & 1;
    zw1 -= zw1 & 1;
    const int ny = (yw1 - yw0) / 2 + 1, nz = (zw1 - zw0) / 2 + 1;
    const int ncp = cx * cy * cz, nX = ex * ny * nz, nXY = ex * ey * nz, nR = ex * ey * ez;
    const long long npts = geo.npts();
    __shared__ unsigned long long mag[9];
    fastdiv_setup(mag, {(unsigned)cx, (unsigned)cy, (unsigned)ex, (unsigned)ey, (unsigned)ny, (unsigned)ncp,
                        (unsigned)nX, (unsigned)nXY, (unsigned)nR});
    const FastDiv f_cx{(unsigned)cx, mag[0]}, f_cy{(unsigned)cy, mag[1]}, f_ex{(unsigned)ex, mag[2]},
        f_ey{(unsigned)ey, mag[3]}, f_ny{(unsigned)ny, mag[4]};
    const FastDiv f_ncp{(unsigned)ncp, mag[5]}, f_nX{(unsigned)nX, mag[6]}, f_nXY{(unsigned)nXY, mag[7]},
        f_nR{(unsigned)nR, mag[8]};
    for (int c0 = 0; c0 < nc; c0 += cg) {
        const int ncg = min(cg, nc - c0);
        float2 *C = sf;                      // ncg coarse boxes
        float2 *X = C + ncg * ncp;           // ncg x-pass windows
        float2 *XY = X + ncg * nX;           // ncg x-y windows
        for (int i = threadIdx.x; i < ncg * ncp; i += blockDim.x) {
            const int c = (int)f_ncp.div(i), k = i - c * ncp;
            const int kx = (int)f_cx.div(k), x = k - kx * cx;
            const int z = (int)f_cy.div(kx), y = kx - z * cy;
            C[i] = __ldcg(buf + ((long long)p.src * nc + c0 + c) * npts +
                          ((long long)(p.slo[2] + z) * geo.ny + (p.slo[1] + y)) * geo.nx + (p.slo[0] + x));
        }
        __syncthreads();
        for (int i = threadIdx.x; i < ncg * nX; i += blockDim.x) {
            const int c = (int)f_nX.div(i), k = i - c * nX;
            const int kx = (int)f_ex.div(k), ix = k - kx * ex;
            const int kz = (int)f_ny.div(kx), jy = kx - kz * ny;
            const int fx = x0 + ix;
            const float2 *row = C + c * ncp + ((long long)((zw0 >> 1) + kz) * cy + (yw0 >> 1) + jy) * cx;
            float2 v;
            if (!(fx & 1)) v = row[fx >> 1];
            else if (fx < h || fx > Fx - 1 - h) v = make_float2(0.f, 0.f);
            else {
                const df2 r = interp_df<NCOEF>(row, 1, (fx - h) >> 1);
                v = make_float2(r.hi, r.lo);
            }
            X[i] = v;
        }
        __syncthreads();
        for (int i = threadIdx.x; i < ncg * nXY; i += blockDim.x) {
            const int c = (int)f_nXY.div(i), k = i - c * nXY;
            const int kx = (int)f_ex.div(k), ix = k - kx * ex;
            const int kz = (int)f_ey.div(kx), j = kx - kz * ey;
            const int fy = y0 + j;
            const float2 *col = X + c * nX + (long long)kz * ny * ex + ix;
            float2 v;
            if (!(fy & 1)) v = col[(long long)((fy - yw0) >> 1) * ex];
            else if (fy < h || fy > Fy - 1 - h) v = make_float2(0.f, 0.f);
            else {
                const df2 r = interp_df<NCOEF>(col, ex, (fy - h - yw0) >> 1);
                v = make_float2(r.hi, r.lo);
            }
            XY[i] = v;
        }
        __syncthreads();
        for (int i = threadIdx.x; i < ncg * nR; i += blockDim.x) {
            const int c = (int)f_nR.div(i), k = i - c * nR;
            const int kx = (int)f_ex.div(k), ix = k - kx * ex;
            const int kk = (int)f_ey.div(kx), j = kx - kk * ey;
            const int fz = z0 + kk;
            const float2 *pl = XY + c * nXY + (long long)j * ex + ix;
            float2 v;
            if (!(fz & 1)) v = pl[(long long)((fz - zw0) >> 1) * ex * ey];
            else if (fz < h || fz > Fz - 1 - h) v = make_float2(0.f, 0.f);
            else {
                const df2 r = interp_df<NCOEF>(pl, ex * ey, (fz - h - zw0) >> 1);
                v = make_float2(r.hi, r.lo);
            }
            const df2 va = anchor({v.x, v.y}, M);
            buf[((long long)p.dst * nc + c0 + c) * npts +
                ((long long)(p.rlo[2] + kk) * geo.ny + (p.rlo[1] + j)) * geo.nx + (p.rlo[0] + ix)] =
                make_float2(va.hi, va.lo);
        }
        __syncthreads();
    }
}

template <int NCOEF>
__global__ void __launch_bounds__(256) predict_df_kernel(const Patch *__restrict__ patches, float2 *buf, BufGeo geo,
                                                         int nc, int cg, const BlockDesc *desc, const TreeClock *clk) {
    extern __shared__ float2 sf[];
    const Patch p = patches[blockIdx.x];
    // the receiver's stage input is anchored to its tree's quantum
    predict_df_patch<NCOEF>(p, buf, geo, nc, cg, clk[desc[p.dst].tree].anchor_M, sf);
}

__device__ __forceinline__ unsigned ld_acquire_u32(const unsigned *p) {
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ void red_release_add_u32(unsigned *p, unsigned v) {
    asm volatile("red.release.gpu.global.add.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

__device__ __forceinline__ unsigned long long sync_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// The per-step ghost sync of the FP32-pipe precision as one launch: the
// restriction entries (gather form) and then the prediction patches, which
// read coarse ghost nodes the restrictions fill. CTAs take work items in
// order from a ticket counter: chunks of 512 restriction entries first, then
// one prediction patch per ticket (largest first). A CTA holding a
// prediction ticket waits until every restriction chunk is done; every chunk
// was handed to a running CTA before that ticket, and chunks wait for
// nothing, so the wait ends (bounded at one second all the same: then *err
// is set and the CTA stops). ctr[0] is the ticket counter, ctr[1] the chunks
// done, ctr[2] the CTAs that finished; the last CTA to finish sets all three
// back to zero for the next launch.
template <int NC, int NCOEF>
__global__ void __launch_bounds__(256, 4) sync_df_fused_kernel(const uint2 *__restrict__ pairs, unsigned npairs,
                                                            const Patch *__restrict__ patches, int npatch,
                                                            float2 *buf, BufGeo geo, int cg, const BlockDesc *desc,
                                                            const TreeClock *clk, unsigned *ctr, int *err) {
    extern __shared__ float2 sf[];
    __shared__ unsigned s_tk;
    __shared__ int s_ok;
    constexpr unsigned CHUNK = 512;
    const unsigned ng = (npairs + CHUNK - 1) / CHUNK;
    const unsigned nwork = ng + (unsigned)npatch;
    const unsigned cs = (unsigned)geo.npts();
    auto *b64 = reinterpret_cast<unsigned long long *>(buf);
    bool ready = ng == 0;
    for (;;) {
        if (threadIdx.x == 0) s_tk = atomicAdd(&ctr[0], 1u);
        __syncthreads();
        const unsigned tk = s_tk;
        __syncthreads();   // every thread has the ticket before thread 0 takes the next
        if (tk >= nwork) break;
        if (tk < ng) {
            const unsigned base = tk * CHUNK + threadIdx.x;
            uint2 e[2];
            unsigned long long v[2][NC];
#pragma unroll
            for (int k = 0; k < 2; k++) {
                const unsigned i = base + k * 256u;
                e[k] = i < npairs ? __ldg(pairs + i) : make_uint2(0u, 0u);
                if (i < npairs) {
#pragma unroll
                    for (int c = 0; c < NC; c++) v[k][c] = b64[e[k].y + c * cs];
                }
            }
#pragma unroll
            for (int k = 0; k < 2; k++) {
                if (base + k * 256u < npairs) {
#pragma unroll
                    for (int c = 0; c < NC; c++) b64[e[k].x + c * cs] = v[k][c];
                }
            }
            __threadfence();
            __syncthreads();
            if (threadIdx.x == 0) red_release_add_u32(&ctr[1], 1u);
            continue;
        }
        if (!ready) {
            if (threadIdx.x == 0) {
                s_ok = 1;
                const unsigned long long t0 = sync_ns();
                while (ld_acquire_u32(&ctr[1]) < ng) {
                    if (sync_ns() - t0 > 1000000000ull) {
                        s_ok = 0;
                        atomicExch(err, 1);
                        break;
                    }
                }
            }
            __syncthreads();
            if (!s_ok) break;
            ready = true;
        }
        const Patch p = patches[tk - ng];
        predict_df_patch<NCOEF>(p, buf, geo, NC, cg, clk[desc[p.dst].tree].anchor_M, sf);
    }
    if (threadIdx.x == 0) {
        __threadfence();
        if (atomicAdd(&ctr[2], 1u) == gridDim.x - 1) {
            ctr[0] = 0u;
            ctr[1] = 0u;
            ctr[2] = 0u;
            __threadfence();
        }
    }
}


cudaError_t sync_init() { return cudaSuccess; }

cudaError_t launch_predict(const Patch *patches, int npatch, int max_smem_doubles, double *buf, BufGeo geo, int nc,
                           int order_predictor, cudaStream_t s, const double *src_buf) {
    if (npatch <= 0) return cudaSuccess;
    if (!patches) return cudaErrorInvalidValue;
    const size_t smem = sizeof(double) * (size_t)max_smem_doubles;
    // the attribute belongs to the current device's context: set on every
    // launch that needs it, to the largest size asked for so far (launches
    // captured earlier in a graph keep a valid attribute)
    static std::atomic<size_t> attr_max{0};
    for (size_t cur = attr_max.load(); cur < smem && !attr_max.compare_exchange_weak(cur, smem);) {
    }
    const size_t want = std::max(smem, attr_max.load());
    if (want > 48 * 1024) {
        cudaError_t e = cudaFuncSetAttribute(predict_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)want);
        if (e != cudaSuccess) return e;
    }
    predict_kernel<<<npatch, 256, smem, s>>>(patches, src_buf ? src_buf : buf, buf, geo, nc, order_predictor / 2 - 1,
                                             order_predictor);
    return cudaGetLastError();
}

cudaError_t launch_predict_df(const Patch *patches, int npatch, int max_smem_doubles, void *buf, BufGeo geo, int nc,
                              int order_predictor, const BlockDesc *desc, const TreeClock *clk, cudaStream_t s,
                              int min_ctas) {
    if (npatch <= 0) return cudaSuccess;
    // as many components per pass as fit the shared memory of one CTA, or of
    // one of min_ctas CTAs on an SM (at least one component)
    const size_t per = sizeof(float2) * (size_t)max_smem_doubles;
    const size_t limit = 200 * 1024;
    if (per > limit) return cudaErrorInvalidValue;
    const size_t room = std::min<size_t>(limit, (size_t)(224 * 1024) / (size_t)std::max(1, min_ctas));
    const int cg = (int)std::max<size_t>(1, std::min<size_t>((size_t)nc, room / per));
    const size_t smem = per * cg;
    float2 *b = reinterpret_cast<float2 *>(buf);
    // the attribute belongs to the current device's context; it is raised to
    // the largest size this launcher has asked for on any device (launches
    // captured earlier in a graph keep a valid attribute)
    static std::atomic<size_t> attr_max[4];
    auto go = [&](auto kern, int k) -> cudaError_t {
        size_t want = smem;
        for (size_t cur = attr_max[k].load(); cur < want && !attr_max[k].compare_exchange_weak(cur, want);) {
        }
        want = std::max(want, attr_max[k].load());
        if (want > 48 * 1024) {
            cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)want);
            if (e != cudaSuccess) return e;
        }
        kern<<<npatch, 256, smem, s>>>(patches, b, geo, nc, cg, desc, clk);
        return cudaGetLastError();
    };
    switch (order_predictor) {
        case 2: return go(predict_df_kernel<2>, 0);
        case 4: return go(predict_df_kernel<4>, 1);
        case 6: return go(predict_df_kernel<6>, 2);
        case 8: return go(predict_df_kernel<8>, 3);
        default: return cudaErrorInvalidValue;
    }
}

cudaError_t launch_sync_df_fused(const void *pairs, unsigned npairs, const Patch *patches, int npatch,
                                 int max_smem_doubles, void *buf, BufGeo geo, int nc, int order_predictor,
                                 const BlockDesc *desc, const TreeClock *clk, unsigned *ctr, int *err, cudaStream_t s,
                                 int min_ctas) {
    if (npairs == 0 && npatch <= 0) return cudaSuccess;
    if (!ctr || !err || (npatch > 0 && !patches) || (npairs > 0 && !pairs)) return cudaErrorInvalidValue;
    // components per prediction pass as in launch_predict_df
    const size_t per = sizeof(float2) * (size_t)std::max(1, max_smem_doubles);
    const size_t limit = 200 * 1024;
    if (per > limit) return cudaErrorInvalidValue;
    const size_t room = std::min<size_t>(limit, (size_t)(224 * 1024) / (size_t)std::max(1, min_ctas));
    const int cg = (int)std::max<size_t>(1, std::min<size_t>((size_t)nc, room / per));
    const size_t smem = npatch > 0 ? per * cg : 0;
    const unsigned nwork = (npairs + 511u) / 512u + (unsigned)std::max(0, npatch);
    auto go = [&](auto kern) -> cudaError_t {
        cudaError_t e;
        if (smem > 48 * 1024 &&
            (e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem)) != cudaSuccess)
            return e;
        int dev = 0, nsm = 0, occ = 0;
        if ((e = cudaGetDevice(&dev)) != cudaSuccess) return e;
        if ((e = cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess) return e;
        if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kern, 256, smem)) != cudaSuccess) return e;
        const unsigned grid = std::min<unsigned>(nwork, (unsigned)std::max(1, nsm * std::max(1, occ)));
        kern<<<grid, 256, smem, s>>>(reinterpret_cast<const uint2 *>(pairs), npairs, patches, npatch,
                                     reinterpret_cast<float2 *>(buf), geo, cg, desc, clk, ctr, err);
        return cudaGetLastError();
    };
    if (nc == 4) {
        switch (order_predictor) {
            case 2: return go(sync_df_fused_kernel<4, 2>);
            case 4: return go(sync_df_fused_kernel<4, 4>);
            case 6: return go(sync_df_fused_kernel<4, 6>);
            case 8: return go(sync_df_fused_kernel<4, 8>);
        }
    } else if (nc == 3) {
        switch (order_predictor) {
            case 2: return go(sync_df_fused_kernel<3, 2>);
            case 4: return go(sync_df_fused_kernel<3, 4>);
            case 6: return go(sync_df_fused_kernel<3, 6>);
            case 8: return go(sync_df_fused_kernel<3, 8>);
        }
    }
    return cudaErrorInvalidValue;
}

cudaError_t launch_expand(const Patch *patches, const unsigned *first, int npatch, unsigned total, BufGeo geo,
                          int nc, void *out, cudaStream_t s) {
    if (total == 0) return cudaSuccess;
    expand_kernel<<<(total + 255) / 256, 256, 0, s>>>(patches, first, npatch, total, geo, nc,
                                                      reinterpret_cast<uint2 *>(out));
    return cudaGetLastError();
}

cudaError_t launch_gather(const void *pairs, unsigned n, void *buf, BufGeo geo, int nc, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    const uint2 *pp = reinterpret_cast<const uint2 *>(pairs);
    auto *b = reinterpret_cast<unsigned long long *>(buf);
    const unsigned cs = (unsigned)geo.npts();
    const unsigned blocks = (n + 255) / 256;
    switch (nc) {
        case 3: gather_kernel<3><<<blocks, 256, 0, s>>>(pp, n, b, cs); break;
        case 4: gather_kernel<4><<<blocks, 256, 0, s>>>(pp, n, b, cs); break;
        default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

cudaError_t launch_sync(const Patch *patches, int npatch, double *buf, BufGeo geo, int nc, int order_predictor,
                        cudaStream_t s) {
    if (npatch <= 0) return cudaSuccess;
    if (!patches) return cudaErrorInvalidValue;
    const int oi = order_predictor / 2 - 1;
    const int threads = 128;
    const int blocks = (npatch * 32 + threads - 1) / threads;
    sync_kernel<<<blocks, threads, 0, s>>>(patches, npatch, buf, geo, nc, oi, order_predictor);
    return cudaGetLastError();
}

}  // namespace wg
