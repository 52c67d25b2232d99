// k_acm_df.cu -- ACM RHS + RK4 stage with the stencils and the stage
// arithmetic in double-float on the FP32 units.
//
// GB300 executes FP64 at 1/58 of its FP32 rate, so the FP64 stencil is
// FP64-pipe bound. Here the RK stage inputs are stored as pairs of floats
// (hi + lo, ~47 significant bits; df.cuh) and the FD_4th_central stencils of
// RHS_3D_acm / RHS_2D_acm (convective form, LIB/EQUATION/ACMnew/
// rhs_ACM.f90:578-615, 1206-1256) run as error-free FP32 transformations:
//   du/dx   = (8 (u+1 - u-1) - (u+2 - u-2)) / (12 dx)
//   d2u/dx2 = (16 (u+1 + u-1) - (u+2 + u-2) - 30 u) / (12 dx^2)
// with the integer weights applied exactly (powers of two) and the 1/(12 dx)
// scalings applied once per term. The RK accumulator holds only the
// increment dt * sum b_j k_j (runge_kutta_generic.f90:60-154), in
// double-float; the state u_n stays FP64 and receives the increment in one
// FP64 addition per value at stage 4, so the state carries full FP64
// resolution while stages 1-3 issue no FP64 instruction. Penalisation and
// sponge use the double-float mask (chi/C_eta with the colour applied, u_s,
// sponge/C_sponge) built by the host from hvy_mask.
//
// Compiled with -fmad=false: the error-free transformations must not be
// contracted; every FMA is explicit.
#include "common.cuh"
#include "df.cuh"

namespace wg {

struct StageArgsDF {
    const int *blk;
    const BlockDesc *desc;
    const TreeParams *tp;
    const TreeClock *clk;
    const float2 *in;      // stage input (thin layout, ghosts synchronised)
    const float2 *u0;      // double-float copy of u_n (thin layout)
    float2 *out;           // next stage input; at stage 4 the copy of u_{n+1}
    BufGeo gt;
    double *un;            // u_n, FP64 (full layout)
    BufGeo gun;
    float2 *acc;           // increment, interior only
    const float2 *mask;    // 5 words per point, interior only
    const int *push;       // same-level ghost copies pushed by the writer, or null
    int Bs0, Bs1, Bs2;
    int stage;
    int chunks;
};

__device__ __forceinline__ df2 ld(const float2 *p) {
    const float2 v = *p;
    return {v.x, v.y};
}

__device__ __forceinline__ void st(float2 *p, df2 v) { *p = make_float2(v.hi, v.lo); }

__device__ __forceinline__ df2 cf(const float c[2]) { return {c[0], c[1]}; }

// Same-level ghost copies pushed by the writer. A point within gb of a face
// of block b is, in the copy stage of the ghost synchronisation
// (synchronize_ghosts_generic.f90, same-level relations), the sender of the
// ghost nodes of the same-level neighbours on that side (faces, edges and
// corners). push[b*27 + dir] is that neighbour's slot, or -1 where the
// neighbour across dir is not on the same level (restriction / prediction
// fill those nodes later); dir = (dz+1)*9 + (dy+1)*3 + (dx+1) points from b
// to the receiver. The host enables this only after checking that every copy
// patch of the table is such a translation.
template <int DIM, int NV>
__device__ __forceinline__ void push_ghosts(const int *push, int b, int ix, int iy, int iz, int Bs0, int Bs1,
                                            int Bs2, BufGeo gt, float2 *out, long long cs, const float2 *v) {
    const int g = gt.gb;
    const int sx = ix < g ? -1 : (ix >= Bs0 - g ? 1 : 0);
    const int sy = iy < g ? -1 : (iy >= Bs1 - g ? 1 : 0);
    const int sz = DIM == 3 ? (iz < g ? -1 : (iz >= Bs2 - g ? 1 : 0)) : 0;
    if (!(sx | sy | sz)) return;
    const int *row = push + b * 27;
    for (int kz = 0; kz < (sz ? 2 : 1); kz++) {
        const int dz = kz ? sz : 0;
        for (int ky = 0; ky < (sy ? 2 : 1); ky++) {
            const int dy = ky ? sy : 0;
            for (int kx = 0; kx < (sx ? 2 : 1); kx++) {
                const int dx = kx ? sx : 0;
                if (!(dx | dy | dz)) continue;
                const int nb = row[(dz + 1) * 9 + (dy + 1) * 3 + (dx + 1)];
                if (nb < 0) continue;
                const long long o = (long long)nb * NV * cs +
                                    ((long long)(DIM == 3 ? iz - dz * Bs2 + g : 0) * gt.ny + (iy - dy * Bs1 + g)) * gt.nx +
                                    (ix - dx * Bs0 + g);
#pragma unroll
                for (int c = 0; c < NV; c++) out[o + c * cs] = v[c];
            }
        }
    }
}

template <int DIM, bool MASK>
__global__ void __launch_bounds__(256) acm_stage_df_kernel(StageArgsDF a) {
    const int bi = blockIdx.x / a.chunks;
    const int chunk = blockIdx.x % a.chunks;
    const int npts_int = a.Bs0 * a.Bs1 * (DIM == 3 ? a.Bs2 : 1);
    const int q = chunk * blockDim.x + threadIdx.x;
    if (q >= npts_int) return;
    const int b = a.blk[bi];
    const BlockDesc &d = a.desc[b];
    const TreeParams &tp = a.tp[d.tree];
    const int ix = q % a.Bs0, iy = (q / a.Bs0) % a.Bs1, iz = DIM == 3 ? q / (a.Bs0 * a.Bs1) : 0;
    const long long cs = a.gt.npts();
    const long long off = (long long)b * (DIM + 1) * cs +
                          ((long long)(iz + (DIM == 3 ? a.gt.gb : 0)) * a.gt.ny + (iy + a.gt.gb)) * a.gt.nx +
                          (ix + a.gt.gb);
    const float2 *u = a.in + off;
    const int stv[3] = {1, a.gt.nx, a.gt.nx * a.gt.ny};

    df2 vel[DIM], w[DIM], r[DIM + 1];
#pragma unroll
    for (int k = 0; k < DIM; k++) {
        vel[k] = ld(u + k * cs);
        w[k] = df_mul_nr(vel[k], cf(d.fs1[k]));            // u_k / (12 dx_k)
    }
    df2 div = {0.f, 0.f};
#pragma unroll
    for (int c = 0; c < DIM; c++) {
        const float2 *uc = u + c * cs;
        df2 adv = {0.f, 0.f};
        df2 lap = df_mul_nr(cf(d.fsc), vel[c]);           // -30 u sum nu/(12 dx^2)
#pragma unroll
        for (int k = 0; k < DIM; k++) {
            const df2 A = ld(uc + stv[k]), B = ld(uc - stv[k]), E = ld(uc + 2 * stv[k]), F = ld(uc - 2 * stv[k]);
            const df2 d1 = df_sub_nr(df_pow2(df_sub_nr(A, B), 8.f), df_sub_nr(E, F));
            adv = df_add_nr(adv, df_mul_nr(w[k], d1));
            if (k == c) div = df_add_nr(div, df_mul_nr(cf(d.fs1[k]), d1));
            const df2 l = df_sub_nr(df_pow2(df_add_nr(A, B), 16.f), df_add_nr(E, F));
            lap = df_add_nr(lap, df_mul_nr(cf(d.fs2[k]), l));
        }
        r[c] = df_sub_nr(lap, adv);
    }
    const float2 *up = u + DIM * cs;
    const df2 p0 = ld(up);
#pragma unroll
    for (int k = 0; k < DIM; k++) {
        const df2 A = ld(up + stv[k]), B = ld(up - stv[k]), E = ld(up + 2 * stv[k]), F = ld(up - 2 * stv[k]);
        const df2 d1 = df_sub_nr(df_pow2(df_sub_nr(A, B), 8.f), df_sub_nr(E, F));
        r[k] = df_sub_nr(r[k], df_mul_nr(cf(d.fs1[k]), d1));
    }
    r[DIM] = df_neg(df_add_nr(df_mul_nr(cf(tp.f_c0sq), div), df_mul_nr(cf(tp.f_gamma), p0)));
    if (MASK) {
        const float2 *m = a.mask + (long long)d.mask * 5 * npts_int + q;
        const df2 chi = ld(m);
#pragma unroll
        for (int c = 0; c < DIM; c++)
            r[c] = df_sub_nr(r[c], df_mul_nr(chi, df_sub_nr(vel[c], ld(m + (1 + c) * npts_int))));
        if (tp.use_sponge) {
            const df2 spo = ld(m + 4 * npts_int);
#pragma unroll
            for (int c = 0; c < DIM; c++)
                r[c] = df_sub_nr(r[c], df_mul_nr(spo, df_sub_nr(vel[c], cf(tp.f_umean[c]))));
            r[DIM] = df_sub_nr(r[DIM], df_mul_nr(spo, p0));
        }
    }

    // RK4 stage (runge_kutta_generic.f90:60-154): b = 1/6, 1/3, 1/3, 1/6;
    // the stage inputs are u_n + dt/2 k1, u_n + dt/2 k2, u_n + dt k3
    const TreeClock &ck = a.clk[d.tree];
    const int j = a.stage;
    const df2 db = (j == 1 || j == 4) ? cf(ck.f_dt6) : cf(ck.f_dt3);
    float2 *acc = a.acc + (long long)b * (DIM + 1) * npts_int + q;
    float2 ov[DIM + 1];
    if (j < 4) {
        const df2 da = j == 3 ? cf(ck.f_dt) : df_pow2(cf(ck.f_dt), 0.5f);
        const float2 *u0 = a.u0 + off;
        float2 *o = a.out + off;
#pragma unroll
        for (int c = 0; c <= DIM; c++) {
            const df2 rc = df_norm(r[c]);
            const df2 inc = df_mul_nr(db, rc);
            st(acc + c * npts_int, df_norm(j == 1 ? inc : df_add_nr(ld(acc + c * npts_int), inc)));
            const df2 v = df_norm(df_add_nr(ld(u0 + c * cs), df_mul_nr(da, rc)));
            ov[c] = make_float2(v.hi, v.lo);
            o[c * cs] = ov[c];
        }
    } else {
        const long long us = a.gun.npts();
        double *un = a.un + (long long)b * (DIM + 1) * us +
                     ((long long)(iz + (DIM == 3 ? a.gun.gb : 0)) * a.gun.ny + (iy + a.gun.gb)) * a.gun.nx +
                     (ix + a.gun.gb);
        float2 *o = a.out + off;
#pragma unroll
        for (int c = 0; c <= DIM; c++) {
            const df2 inc = df_norm(df_add_nr(ld(acc + c * npts_int), df_mul_nr(db, df_norm(r[c]))));
            const double v = __dadd_rn(__dadd_rn(un[c * us], f2d_bits(inc.hi)), f2d_bits(inc.lo));
            un[c * us] = v;
            const df2 w = df_split(v);
            ov[c] = make_float2(w.hi, w.lo);
            o[c * cs] = ov[c];
        }
    }
    if (a.push) push_ghosts<DIM, DIM + 1>(a.push, b, ix, iy, iz, a.Bs0, a.Bs1, a.Bs2, a.gt, a.out, cs, ov);
}

cudaError_t launch_acm_stage_df(int dim, int stage, int masked, const int *blk, int nblk, const BlockDesc *desc,
                                const TreeParams *tp, const TreeClock *clk, const void *in, const void *u0,
                                void *out, BufGeo gt, double *un, BufGeo gun, void *acc, const void *maskdf,
                                const int *push, int Bs0, int Bs1, int Bs2, cudaStream_t s) {
    if (nblk <= 0) return cudaSuccess;
    StageArgsDF a;
    a.blk = blk;
    a.desc = desc;
    a.tp = tp;
    a.clk = clk;
    a.in = reinterpret_cast<const float2 *>(in);
    a.u0 = reinterpret_cast<const float2 *>(u0);
    a.out = reinterpret_cast<float2 *>(out);
    a.gt = gt;
    a.un = un;
    a.gun = gun;
    a.acc = reinterpret_cast<float2 *>(acc);
    a.mask = reinterpret_cast<const float2 *>(maskdf);
    a.push = push;
    a.Bs0 = Bs0;
    a.Bs1 = Bs1;
    a.Bs2 = Bs2;
    a.stage = stage;
    const int npts_int = Bs0 * Bs1 * (dim == 3 ? Bs2 : 1);
    const int threads = 256;
    a.chunks = (npts_int + threads - 1) / threads;
    const unsigned grid = (unsigned)((long long)nblk * a.chunks);
    if (dim == 2) {
        if (masked) acm_stage_df_kernel<2, true><<<grid, threads, 0, s>>>(a);
        else acm_stage_df_kernel<2, false><<<grid, threads, 0, s>>>(a);
    } else {
        if (masked) acm_stage_df_kernel<3, true><<<grid, threads, 0, s>>>(a);
        else acm_stage_df_kernel<3, false><<<grid, threads, 0, s>>>(a);
    }
    return cudaGetLastError();
}

// double-float copy (df_split) of the interiors of the listed blocks
__global__ void shadow_kernel(const int *blk, int nblk, const double *src, BufGeo gs, float2 *dst, BufGeo gd, int nc,
                              int Bx, int By, int Bz, const int *push) {
    const long long nint = (long long)Bx * By * Bz;
    const long long total = (long long)nblk * nc * nint;
    const int zs = gs.nz > 1 ? gs.gb : 0, zd = gd.nz > 1 ? gd.gb : 0;
    for (long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x; q < total;
         q += (long long)gridDim.x * blockDim.x) {
        const long long r = q % nint;
        const int c = (int)((q / nint) % nc);
        const int b = blk[q / (nint * nc)];
        const int ix = (int)(r % Bx), iy = (int)((r / Bx) % By), iz = (int)(r / ((long long)Bx * By));
        const double v = src[((long long)b * nc + c) * gs.npts() + ((long long)(iz + zs) * gs.ny + (iy + gs.gb)) * gs.nx +
                             (ix + gs.gb)];
        const df2 w = df_split(v);
        const float2 f = make_float2(w.hi, w.lo);
        float2 *dc = dst + (long long)c * gd.npts();
        dc[(long long)b * nc * gd.npts() + ((long long)(iz + zd) * gd.ny + (iy + gd.gb)) * gd.nx + (ix + gd.gb)] = f;
        if (push) {
            if (gd.nz > 1) push_ghosts<3, 1>(push, b, ix, iy, iz, Bx, By, Bz, gd, dc, gd.npts() * nc, &f);
            else push_ghosts<2, 1>(push, b, ix, iy, iz, Bx, By, Bz, gd, dc, gd.npts() * nc, &f);
        }
    }
}

cudaError_t launch_shadow(const int *blk, int nblk, const double *src, BufGeo gs, void *dst, BufGeo gd, int nc,
                          int Bs0, int Bs1, int Bs2, const int *push, cudaStream_t s) {
    if (nblk <= 0) return cudaSuccess;
    shadow_kernel<<<1024, 256, 0, s>>>(blk, nblk, src, gs, reinterpret_cast<float2 *>(dst), gd, nc, Bs0, Bs1, Bs2,
                                       push);
    return cudaGetLastError();
}

}  // namespace wg
