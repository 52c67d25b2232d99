// acm_body.cuh -- ACM right-hand side + RK4 stage update, one thread per
// interior point. Included by k_acm_strict.cu (compiled with -fmad=false: the
// arithmetic is the reference's, term by term and left to right, so results
// are bit-identical to it) and k_acm_fast.cu (FMA contraction allowed).
//
// RHS: RHS_2D_acm / RHS_3D_acm, FD_4th_central, skew-symmetric or convective
// form, volume penalisation and sponge
// (LIB/EQUATION/ACMnew/rhs_ACM.f90:530-615, 1137-1256, 872-890, 1734-1753).
// RK4: RungeKuttaGeneric with the default Butcher tableau
// (LIB/TIME/runge_kutta_generic.f90:60-154): stage j computes k_j, adds
// dt*b_j*k_j to the accumulator (which starts from u_n) and writes the next
// stage input u_n + dt*a_{j+1,j}*k_j; stage 4 writes u_{n+1}.
#pragma once
#include "common.cuh"

#ifndef WG_NS
#error "define WG_NS"
#endif

namespace wg {
namespace WG_NS {

__device__ __constant__ double kA[5] = {1.0 / 12.0, -2.0 / 3.0, 0.0, 2.0 / 3.0, -1.0 / 12.0};
__device__ __constant__ double kB[5] = {-1.0 / 12.0, 4.0 / 3.0, -5.0 / 2.0, 4.0 / 3.0, -1.0 / 12.0};

template <bool SKEW, bool MASK>
__device__ __forceinline__ void rhs2d(const double *u, long long cs, int sx, const double *m, long long ms,
                                      const TreeParams &tp, double dx_inv, double dy_inv, double dx2_inv,
                                      double dy2_inv, double r[3]) {
#define P(c, ox, oy) u[(c)*cs + (long long)(oy)*sx + (ox)]
    auto px = [&](int c, int o) { return P(c, o, 0); };
    auto py = [&](int c, int o) { return P(c, 0, o); };
    double u_dx = (kA[0] * px(0, -2) + kA[1] * px(0, -1) + kA[3] * px(0, 1) + kA[4] * px(0, 2)) * dx_inv;
    double v_dx = (kA[0] * px(1, -2) + kA[1] * px(1, -1) + kA[3] * px(1, 1) + kA[4] * px(1, 2)) * dx_inv;
    double p_dx = (kA[0] * px(2, -2) + kA[1] * px(2, -1) + kA[3] * px(2, 1) + kA[4] * px(2, 2)) * dx_inv;
    double u_dy = (kA[0] * py(0, -2) + kA[1] * py(0, -1) + kA[3] * py(0, 1) + kA[4] * py(0, 2)) * dy_inv;
    double v_dy = (kA[0] * py(1, -2) + kA[1] * py(1, -1) + kA[3] * py(1, 1) + kA[4] * py(1, 2)) * dy_inv;
    double p_dy = (kA[0] * py(2, -2) + kA[1] * py(2, -1) + kA[3] * py(2, 1) + kA[4] * py(2, 2)) * dy_inv;
    double u_dxdx = (kB[0] * px(0, -2) + kB[1] * px(0, -1) + kB[2] * px(0, 0) + kB[3] * px(0, 1) + kB[4] * px(0, 2)) * dx2_inv;
    double v_dxdx = (kB[0] * px(1, -2) + kB[1] * px(1, -1) + kB[2] * px(1, 0) + kB[3] * px(1, 1) + kB[4] * px(1, 2)) * dx2_inv;
    double u_dydy = (kB[0] * py(0, -2) + kB[1] * py(0, -1) + kB[2] * py(0, 0) + kB[3] * py(0, 1) + kB[4] * py(0, 2)) * dy2_inv;
    double v_dydy = (kB[0] * py(1, -2) + kB[1] * py(1, -1) + kB[2] * py(1, 0) + kB[3] * py(1, 1) + kB[4] * py(1, 2)) * dy2_inv;
    const double div_U = u_dx + v_dy;
    const double uc = P(0, 0, 0), vc = P(1, 0, 0), pc = P(2, 0, 0);
    double penalx = 0.0, penaly = 0.0;
    if (MASK) {
        const double chi = m[0];
        const int color = (int)m[4 * ms];
        const double ci = color == 0 ? 0.0 : tp.C_eta_inv;
        penalx = -chi * ci * (uc - m[1 * ms]);
        penaly = -chi * ci * (vc - m[2 * ms]);
    }
    const double nu = tp.nu;
    double r1, r2;
    if (SKEW) {
        double uu_dx = (kA[0] * px(0, -2) * px(0, -2) + kA[1] * px(0, -1) * px(0, -1) + kA[3] * px(0, 1) * px(0, 1) + kA[4] * px(0, 2) * px(0, 2)) * dx_inv;
        double uv_dy = (kA[0] * py(0, -2) * py(1, -2) + kA[1] * py(0, -1) * py(1, -1) + kA[3] * py(0, 1) * py(1, 1) + kA[4] * py(0, 2) * py(1, 2)) * dy_inv;
        double vu_dx = (kA[0] * px(1, -2) * px(0, -2) + kA[1] * px(1, -1) * px(0, -1) + kA[3] * px(1, 1) * px(0, 1) + kA[4] * px(1, 2) * px(0, 2)) * dx_inv;
        double vv_dy = (kA[0] * py(1, -2) * py(1, -2) + kA[1] * py(1, -1) * py(1, -1) + kA[3] * py(1, 1) * py(1, 1) + kA[4] * py(1, 2) * py(1, 2)) * dy_inv;
        r1 = -0.5 * (uu_dx + uv_dy + uc * u_dx + vc * u_dy) - p_dx + nu * (u_dxdx + u_dydy) + penalx;
        r2 = -0.5 * (vu_dx + vv_dy + uc * v_dx + vc * v_dy) - p_dy + nu * (v_dxdx + v_dydy) + penaly;
    } else {
        r1 = -uc * u_dx - vc * u_dy - p_dx + nu * (u_dxdx + u_dydy) + penalx;
        r2 = -uc * v_dx - vc * v_dy - p_dy + nu * (v_dxdx + v_dydy) + penaly;
    }
    double r3 = -(tp.c0 * tp.c0) * div_U - tp.gamma_p * pc;
    if (MASK && tp.use_sponge) {
        const double spo = m[5 * ms] * tp.C_sponge_inv;
        r1 = r1 - (uc - tp.u_mean_set[0]) * spo;
        r2 = r2 - (vc - tp.u_mean_set[1]) * spo;
        r3 = r3 - pc * spo;
    }
    r[0] = r1;
    r[1] = r2;
    r[2] = r3;
#undef P
}

template <bool SKEW, bool MASK>
__device__ __forceinline__ void rhs3d(const double *u, long long cs, int sx, int sy, const double *m, long long ms,
                                      const TreeParams &tp, const double di[3], const double d2i[3], double r[4]) {
    auto P = [&](int c, int ox, int oy, int oz) { return u[c * cs + (long long)oz * sy + (long long)oy * sx + ox]; };
#define D1X(c) ((kA[0] * P(c, -2, 0, 0) + kA[1] * P(c, -1, 0, 0) + kA[3] * P(c, 1, 0, 0) + kA[4] * P(c, 2, 0, 0)) * di[0])
#define D1Y(c) ((kA[0] * P(c, 0, -2, 0) + kA[1] * P(c, 0, -1, 0) + kA[3] * P(c, 0, 1, 0) + kA[4] * P(c, 0, 2, 0)) * di[1])
#define D1Z(c) ((kA[0] * P(c, 0, 0, -2) + kA[1] * P(c, 0, 0, -1) + kA[3] * P(c, 0, 0, 1) + kA[4] * P(c, 0, 0, 2)) * di[2])
#define D2X(c) ((kB[0] * P(c, -2, 0, 0) + kB[1] * P(c, -1, 0, 0) + kB[2] * P(c, 0, 0, 0) + kB[3] * P(c, 1, 0, 0) + kB[4] * P(c, 2, 0, 0)) * d2i[0])
#define D2Y(c) ((kB[0] * P(c, 0, -2, 0) + kB[1] * P(c, 0, -1, 0) + kB[2] * P(c, 0, 0, 0) + kB[3] * P(c, 0, 1, 0) + kB[4] * P(c, 0, 2, 0)) * d2i[1])
#define D2Z(c) ((kB[0] * P(c, 0, 0, -2) + kB[1] * P(c, 0, 0, -1) + kB[2] * P(c, 0, 0, 0) + kB[3] * P(c, 0, 0, 1) + kB[4] * P(c, 0, 0, 2)) * d2i[2])
#define PX(a, b) ((kA[0] * P(a, -2, 0, 0) * P(b, -2, 0, 0) + kA[1] * P(a, -1, 0, 0) * P(b, -1, 0, 0) + kA[3] * P(a, 1, 0, 0) * P(b, 1, 0, 0) + kA[4] * P(a, 2, 0, 0) * P(b, 2, 0, 0)) * di[0])
#define PY(a, b) ((kA[0] * P(a, 0, -2, 0) * P(b, 0, -2, 0) + kA[1] * P(a, 0, -1, 0) * P(b, 0, -1, 0) + kA[3] * P(a, 0, 1, 0) * P(b, 0, 1, 0) + kA[4] * P(a, 0, 2, 0) * P(b, 0, 2, 0)) * di[1])
#define PZ(a, b) ((kA[0] * P(a, 0, 0, -2) * P(b, 0, 0, -2) + kA[1] * P(a, 0, 0, -1) * P(b, 0, 0, -1) + kA[3] * P(a, 0, 0, 1) * P(b, 0, 0, 1) + kA[4] * P(a, 0, 0, 2) * P(b, 0, 0, 2)) * di[2])
    double u_dx = D1X(0), v_dx = D1X(1), w_dx = D1X(2), p_dx = D1X(3);
    double u_dy = D1Y(0), v_dy = D1Y(1), w_dy = D1Y(2), p_dy = D1Y(3);
    double u_dz = D1Z(0), v_dz = D1Z(1), w_dz = D1Z(2), p_dz = D1Z(3);
    double u_dxdx = D2X(0), v_dxdx = D2X(1), w_dxdx = D2X(2);
    double u_dydy = D2Y(0), v_dydy = D2Y(1), w_dydy = D2Y(2);
    double u_dzdz = D2Z(0), v_dzdz = D2Z(1), w_dzdz = D2Z(2);
    const double uu = P(0, 0, 0, 0), vv = P(1, 0, 0, 0), ww = P(2, 0, 0, 0), pp = P(3, 0, 0, 0);
    double penalx = 0.0, penaly = 0.0, penalz = 0.0;
    if (MASK) {
        const int color = (int)m[4 * ms];
        const double chi = m[0] * (color == 0 ? 0.0 : tp.C_eta_inv);
        penalx = -chi * (uu - m[1 * ms]);
        penaly = -chi * (vv - m[2 * ms]);
        penalz = -chi * (ww - m[3 * ms]);
    }
    const double nu = tp.nu;
    double r1, r2, r3;
    if (SKEW) {
        double uu_dx = PX(0, 0), uv_dy = PY(0, 1), uw_dz = PZ(0, 2);
        double vu_dx = PX(1, 0), vv_dy = PY(1, 1), vw_dz = PZ(1, 2);
        double wu_dx = PX(2, 0), wv_dy = PY(2, 1), ww_dz = PZ(2, 2);
        r1 = -0.5 * (uu_dx + uv_dy + uw_dz + uu * u_dx + vv * u_dy + ww * u_dz) - p_dx + nu * (u_dxdx + u_dydy + u_dzdz) + penalx;
        r2 = -0.5 * (vu_dx + vv_dy + vw_dz + uu * v_dx + vv * v_dy + ww * v_dz) - p_dy + nu * (v_dxdx + v_dydy + v_dzdz) + penaly;
        r3 = -0.5 * (wu_dx + wv_dy + ww_dz + uu * w_dx + vv * w_dy + ww * w_dz) - p_dz + nu * (w_dxdx + w_dydy + w_dzdz) + penalz;
    } else {
        r1 = (-uu * u_dx - vv * u_dy - ww * u_dz) - p_dx + nu * (u_dxdx + u_dydy + u_dzdz) + penalx;
        r2 = (-uu * v_dx - vv * v_dy - ww * v_dz) - p_dy + nu * (v_dxdx + v_dydy + v_dzdz) + penaly;
        r3 = (-uu * w_dx - vv * w_dy - ww * w_dz) - p_dz + nu * (w_dxdx + w_dydy + w_dzdz) + penalz;
    }
    double r4 = -(tp.c0 * tp.c0) * (u_dx + v_dy + w_dz) - tp.gamma_p * pp;
    if (MASK && tp.use_sponge) {
        const double spo = m[5 * ms] * tp.C_sponge_inv;
        r1 = r1 - (uu - tp.u_mean_set[0]) * spo;
        r2 = r2 - (vv - tp.u_mean_set[1]) * spo;
        r3 = r3 - (ww - tp.u_mean_set[2]) * spo;
        r4 = r4 - pp * spo;
    }
    r[0] = r1;
    r[1] = r2;
    r[2] = r3;
    r[3] = r4;
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


#ifdef WG_FAST_ALGEBRA
// Regrouped convective form for the fast path: per axis the pair differences
// and sums of the +-1, +-2 neighbours give the first derivative
// k1*(u1-u_1) - k2*(u2-u_2) and the viscous term m1*(u1+u_1) - m2*(u2+u_2),
// with m0*u0 added once; about 111 FP64 instructions per point and stage
// instead of ~167 for the reference's term order.
template <int DIM, bool MASK>
__device__ __forceinline__ void rhs_opt(const double *u, long long cs, int sx, int sy, const double *m, long long ms,
                                        const TreeParams &tp, const BlockDesc &d, double r[4]) {
    const int st[3] = {1, sx, sy};
    double D1[4][3];
    double L[3];
#pragma unroll
    for (int c = 0; c < DIM + 1; c++) {
        const double *uc = u + c * cs;
        const double u0 = uc[0];
        double lap = c < DIM ? d.m0 * u0 : 0.0;
#pragma unroll
        for (int k = 0; k < DIM; k++) {
            const double a = uc[st[k]], b = uc[-st[k]], e = uc[2 * st[k]], f = uc[-2 * st[k]];
            D1[c][k] = fma(-d.k2[k], e - f, d.k1[k] * (a - b));
            if (c < DIM) lap = fma(-d.m2[k], e + f, fma(d.m1[k], a + b, lap));
        }
        if (c < DIM) L[c] = lap;
    }
    const double p0 = u[DIM * cs];
    double vel[3];
#pragma unroll
    for (int c = 0; c < DIM; c++) vel[c] = u[c * cs];
    double chi = 0.0;
    if (MASK) {
        const int color = (int)m[4 * ms];
        chi = color == 0 ? 0.0 : m[0] * tp.C_eta_inv;
    }
#pragma unroll
    for (int c = 0; c < DIM; c++) {
        double t = D1[DIM][c];                       // p_dx (pressure gradient along c)
#pragma unroll
        for (int k = 0; k < DIM; k++) t = fma(vel[k], D1[c][k], t);
        double rc = L[c] - t;
        if (MASK) rc = fma(-chi, vel[c] - m[(1 + c) * ms], rc);
        r[c] = rc;
    }
    double div = D1[0][0];
#pragma unroll
    for (int k = 1; k < DIM; k++) div += D1[k][k];
    r[DIM] = fma(-(tp.c0 * tp.c0), div, -tp.gamma_p * p0);
    if (MASK && tp.use_sponge) {
        const double spo = m[5 * ms] * tp.C_sponge_inv;
#pragma unroll
        for (int c = 0; c < DIM; c++) r[c] = fma(-(vel[c] - tp.u_mean_set[c]), spo, r[c]);
        r[DIM] = fma(-p0, spo, r[DIM]);
    }
}
#endif

// RK4 Butcher coefficients (ini_file_to_params.f90:640-646)
__device__ __forceinline__ double rk_b(int j) { return (j == 1 || j == 4) ? 1.0 / 6.0 : 1.0 / 3.0; }
__device__ __forceinline__ double rk_a(int j) { return j == 3 ? 1.0 : 0.5; }   // a_{j+1,j}

// Blocks listed for a MASK launch all own a mask slot; the host splits the
// block list into masked and unmasked blocks (a block without a mask slot has
// chi = 0 and no sponge everywhere, so the unmasked kernel is exact for it).
template <int DIM, bool SKEW, bool MASK>
__global__ void __launch_bounds__(256) acm_stage_kernel(StageArgs a) {
    const int bi = blockIdx.x / a.chunks;
    const int chunk = blockIdx.x % a.chunks;
    const int npts_int = a.Bs0 * a.Bs1 * (DIM == 3 ? a.Bs2 : 1);
    const int q = chunk * blockDim.x + threadIdx.x;
    if (q >= npts_int) return;
    const int b = a.blk[bi];
    const BlockDesc d = a.desc[b];
    const TreeParams &tp = a.tp[d.tree];
    const int ix = q % a.Bs0, iy = (q / a.Bs0) % a.Bs1, iz = DIM == 3 ? q / (a.Bs0 * a.Bs1) : 0;
    const long long cs = a.gin.npts();
    const double *u = a.in + (long long)b * a.nc * cs +
                      ((long long)(iz + (DIM == 3 ? a.gin.gb : 0)) * a.gin.ny + (iy + a.gin.gb)) * a.gin.nx + (ix + a.gin.gb);
    const double *m = nullptr;
    long long ms = npts_int;
    if (MASK) m = a.mask + (long long)d.mask * 6 * npts_int + q;
    double r[4];
#ifdef WG_FAST_ALGEBRA
    if (!SKEW) {
        rhs_opt<DIM, MASK>(u, cs, a.gin.nx, a.gin.nx * a.gin.ny, m, ms, tp, d, r);
    } else
#endif
    if (DIM == 2) {
        const double dxi = 1.0 / d.dx[0], dyi = 1.0 / d.dx[1];
        const double dx2 = 1.0 / (d.dx[0] * d.dx[0]), dy2 = 1.0 / (d.dx[1] * d.dx[1]);
        rhs2d<SKEW, MASK>(u, cs, a.gin.nx, m, ms, tp, dxi, dyi, dx2, dy2, r);
    } else {
        const double di[3] = {1.0 / d.dx[0], 1.0 / d.dx[1], 1.0 / d.dx[2]};
        const double d2i[3] = {1.0 / (d.dx[0] * d.dx[0]), 1.0 / (d.dx[1] * d.dx[1]), 1.0 / (d.dx[2] * d.dx[2])};
        rhs3d<SKEW, MASK>(u, cs, a.gin.nx, a.gin.nx * a.gin.ny, m, ms, tp, di, d2i, r);
    }
    const int nc = DIM + 1;
    if (a.rhs_only) {
        const long long os = a.gout.npts();
        double *o = a.out + (long long)b * nc * os +
                    ((long long)(iz + (DIM == 3 ? a.gout.gb : 0)) * a.gout.ny + (iy + a.gout.gb)) * a.gout.nx + (ix + a.gout.gb);
        for (int c = 0; c < nc; c++) o[c * os] = r[c];
        return;
    }
    // divergence guard of the integral stage (rhs_ACM.f90:133-146)
    const TreeClock &ck = a.clk[d.tree];
    const double dt = ck.dt;
    const long long us = a.gun.npts();
    double *un = a.un + (long long)b * nc * us +
                 ((long long)(iz + (DIM == 3 ? a.gun.gb : 0)) * a.gun.ny + (iy + a.gun.gb)) * a.gun.nx + (ix + a.gun.gb);
    double *acc = a.acc + (long long)b * nc * npts_int + q;
    const int j = a.stage;
    const double db = __dmul_rn(dt, rk_b(j));
    if (j < 4) {
        const long long os = a.gout.npts();
        double *o = a.out + (long long)b * nc * os +
                    ((long long)(iz + (DIM == 3 ? a.gout.gb : 0)) * a.gout.ny + (iy + a.gout.gb)) * a.gout.nx + (ix + a.gout.gb);
        const double da = __dmul_rn(dt, rk_a(j));
        for (int c = 0; c < nc; c++) {
            const double u0 = un[c * us];
            const double base = j == 1 ? u0 : acc[c * npts_int];
#ifdef WG_FAST_ALGEBRA
            acc[c * npts_int] = fma(db, r[c], base);
            o[c * os] = fma(da, r[c], u0);
#else
            acc[c * npts_int] = __dadd_rn(base, __dmul_rn(db, r[c]));
            o[c * os] = __dadd_rn(u0, __dmul_rn(da, r[c]));
#endif
        }
    } else {
#ifdef WG_FAST_ALGEBRA
        for (int c = 0; c < nc; c++) un[c * us] = fma(db, r[c], acc[c * npts_int]);
#else
        for (int c = 0; c < nc; c++) un[c * us] = __dadd_rn(acc[c * npts_int], __dmul_rn(db, r[c]));
#endif
    }
}

template <int DIM, bool SKEW, bool MASK>
static cudaError_t go(const StageArgs &a, int nblk, cudaStream_t s) {
    const int npts_int = a.Bs0 * a.Bs1 * (DIM == 3 ? a.Bs2 : 1);
    const int threads = 256;
    StageArgs b = a;
    b.chunks = (npts_int + threads - 1) / threads;
    const long long grid = (long long)nblk * b.chunks;
    if (grid <= 0) return cudaSuccess;
    acm_stage_kernel<DIM, SKEW, MASK><<<(unsigned)grid, threads, 0, s>>>(b);
    return cudaGetLastError();
}

template <int DIM>
static cudaError_t dispatch(const StageArgs &a, int nblk, bool skew, bool mask, cudaStream_t s) {
    if (skew) return mask ? go<DIM, true, true>(a, nblk, s) : go<DIM, true, false>(a, nblk, s);
    return mask ? go<DIM, false, true>(a, nblk, s) : go<DIM, false, false>(a, nblk, s);
}

cudaError_t stage(int dim, const StageArgs &a, int nblk, bool skew, bool mask, cudaStream_t s) {
    return dim == 2 ? dispatch<2>(a, nblk, skew, mask, s) : dispatch<3>(a, nblk, skew, mask, s);
}

}  // namespace WG_NS
}  // namespace wg
