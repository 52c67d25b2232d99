// k_acm_df.cu -- ACM RHS + RK4 stage with the stencils evaluated in
// double-float arithmetic on the FP32 units.
//
// GB300 executes FP64 at 1/58 of its FP32 rate, so the FP64 stencil is
// FP64-pipe bound. Here each RK stage input is stored as a pair of floats
// (hi + lo, ~48 significant bits; df.cuh) and the FD_4th_central stencils of
// RHS_3D_acm / RHS_2D_acm (convective form, LIB/EQUATION/ACMnew/
// rhs_ACM.f90:578-615, 1206-1256) run as error-free FP32 transformations. The
// RK state (u_n, accumulator, u_{n+1}), the update arithmetic and the stiff
// penalisation and sponge terms stay in FP64. Results agree with the FP64
// path to about 1e-14 relative per step.
//
// Compiled with -fmad=false: the error-free transformations must not be
// contracted; every FMA is explicit.
#include "common.cuh"
#include "df.cuh"

namespace wg {

__device__ __forceinline__ df2 ld(const float2 *p) {
    const float2 v = *p;
    return {v.x, v.y};
}

__device__ __forceinline__ void st(float2 *p, df2 v) { *p = make_float2(v.hi, v.lo); }

__device__ __forceinline__ df2 cf(const float c[2]) { return {c[0], c[1]}; }

template <int DIM, bool MASK>
__global__ void __launch_bounds__(256) acm_stage_df_kernel(StageArgs a) {
    const int bi = blockIdx.x / a.chunks;
    const int chunk = blockIdx.x % a.chunks;
    const int npts_int = a.Bs0 * a.Bs1 * (DIM == 3 ? a.Bs2 : 1);
    const int q = chunk * blockDim.x + threadIdx.x;
    if (q >= npts_int) return;
    const int b = a.blk[bi];
    const BlockDesc &d = a.desc[b];
    const TreeParams &tp = a.tp[d.tree];
    const int ix = q % a.Bs0, iy = (q / a.Bs0) % a.Bs1, iz = DIM == 3 ? q / (a.Bs0 * a.Bs1) : 0;
    const long long cs = a.gin.npts();
    const float2 *u = reinterpret_cast<const float2 *>(a.in) + (long long)b * (DIM + 1) * cs +
                      ((long long)(iz + (DIM == 3 ? a.gin.gb : 0)) * a.gin.ny + (iy + a.gin.gb)) * a.gin.nx +
                      (ix + a.gin.gb);
    const int stv[3] = {1, a.gin.nx, a.gin.nx * a.gin.ny};
    df2 D1[DIM + 1][DIM];
    df2 L[DIM];
    df2 vel[DIM];
    df2 p0 = ld(u + DIM * cs);
#pragma unroll
    for (int c = 0; c <= DIM; c++) {
        const float2 *uc = u + c * cs;
        const df2 u0 = ld(uc);
        if (c < DIM) vel[c] = u0;
        df2 lap = c < DIM ? df_mul(cf(d.fm0), u0) : df2{0.f, 0.f};
#pragma unroll
        for (int k = 0; k < DIM; k++) {
            const df2 A = ld(uc + stv[k]), B = ld(uc - stv[k]), E = ld(uc + 2 * stv[k]), F = ld(uc - 2 * stv[k]);
            D1[c][k] = df_sub(df_mul(cf(d.fk1[k]), df_sub(A, B)), df_mul(cf(d.fk2[k]), df_sub(E, F)));
            if (c < DIM)
                lap = df_add(lap, df_sub(df_mul(cf(d.fm1[k]), df_add(A, B)), df_mul(cf(d.fm2[k]), df_add(E, F))));
        }
        if (c < DIM) L[c] = lap;
    }
    double r[DIM + 1];
#pragma unroll
    for (int c = 0; c < DIM; c++) {
        df2 t = D1[DIM][c];
#pragma unroll
        for (int k = 0; k < DIM; k++) t = df_add(t, df_mul(vel[k], D1[c][k]));
        r[c] = df_to(df_sub(L[c], t));
    }
    df2 div = D1[0][0];
#pragma unroll
    for (int k = 1; k < DIM; k++) div = df_add(div, D1[k][k]);
    r[DIM] = -df_to(df_add(df_mul(cf(tp.f_c0sq), div), df_mul(cf(tp.f_gamma), p0)));
    if (MASK) {
        // penalisation and sponge in FP64
        const double *m = a.mask + (long long)d.mask * 6 * npts_int + q;
        const long long ms = npts_int;
        const int color = (int)m[4 * ms];
        const double chi = color == 0 ? 0.0 : m[0] * tp.C_eta_inv;
#pragma unroll
        for (int c = 0; c < DIM; c++) r[c] = fma(-chi, df_to(vel[c]) - m[(1 + c) * ms], r[c]);
        if (tp.use_sponge) {
            const double spo = m[5 * ms] * tp.C_sponge_inv;
#pragma unroll
            for (int c = 0; c < DIM; c++) r[c] = fma(-(df_to(vel[c]) - tp.u_mean_set[c]), spo, r[c]);
            r[DIM] = fma(-df_to(p0), spo, r[DIM]);
        }
    }
    // RK4 update in FP64 (runge_kutta_generic.f90:60-154)
    const double dt = a.clk[d.tree].dt;
    const int j = a.stage;
    const double bj = (j == 1 || j == 4) ? 1.0 / 6.0 : 1.0 / 3.0;
    const double db = dt * bj;
    const long long us = a.gun.npts();
    double *un = a.un + (long long)b * (DIM + 1) * us +
                 ((long long)(iz + (DIM == 3 ? a.gun.gb : 0)) * a.gun.ny + (iy + a.gun.gb)) * a.gun.nx + (ix + a.gun.gb);
    double *acc = a.acc + (long long)b * (DIM + 1) * npts_int + q;
    const long long os = a.gout.npts();
    float2 *o = reinterpret_cast<float2 *>(a.out) + (long long)b * (DIM + 1) * os +
                ((long long)(iz + (DIM == 3 ? a.gout.gb : 0)) * a.gout.ny + (iy + a.gout.gb)) * a.gout.nx +
                (ix + a.gout.gb);
    if (j < 4) {
        const double da = dt * (j == 3 ? 1.0 : 0.5);
#pragma unroll
        for (int c = 0; c <= DIM; c++) {
            const double u0 = un[c * us];
            const double base = j == 1 ? u0 : acc[c * npts_int];
            acc[c * npts_int] = fma(db, r[c], base);
            st(o + c * os, df_from(fma(da, r[c], u0)));
        }
    } else {
#pragma unroll
        for (int c = 0; c <= DIM; c++) {
            const double v = fma(db, r[c], acc[c * npts_int]);
            un[c * us] = v;
            st(o + c * os, df_from(v));
        }
    }
}

cudaError_t launch_acm_stage_df(int dim, int stage, int masked, const int *blk, int nblk, const BlockDesc *desc,
                                const TreeParams *tp, const TreeClock *clk, const void *in, BufGeo gin, void *out,
                                BufGeo gout, double *un, BufGeo gun, double *acc, const double *mask, int Bs0,
                                int Bs1, int Bs2, int nc, cudaStream_t s) {
    if (nblk <= 0) return cudaSuccess;
    StageArgs a;
    a.blk = blk;
    a.desc = desc;
    a.tp = tp;
    a.clk = clk;
    a.in = reinterpret_cast<const double *>(in);
    a.gin = gin;
    a.out = reinterpret_cast<double *>(out);
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
    a.rhs_only = 0;
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

__global__ void shadow_kernel(const int *blk, int nblk, const double *src, BufGeo gs, float2 *dst, BufGeo gd, int nc,
                              int Bx, int By, int Bz) {
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
        st(dst + ((long long)b * nc + c) * gd.npts() + ((long long)(iz + zd) * gd.ny + (iy + gd.gb)) * gd.nx + (ix + gd.gb),
           df_from(v));
    }
}

cudaError_t launch_shadow(const int *blk, int nblk, const double *src, BufGeo gs, void *dst, BufGeo gd, int nc,
                          int Bs0, int Bs1, int Bs2, cudaStream_t s) {
    if (nblk <= 0) return cudaSuccess;
    shadow_kernel<<<1024, 256, 0, s>>>(blk, nblk, src, gs, reinterpret_cast<float2 *>(dst), gd, nc, Bs0, Bs1, Bs2);
    return cudaGetLastError();
}

}  // namespace wg
