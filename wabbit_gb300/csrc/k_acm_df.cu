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
// scalings applied once per term. The stage inputs are anchored (df.cuh), so
// neighbour differences are exact FP32 operations.
//
// RK4 (runge_kutta_generic.f90:60-154 with the classic tableau) without an
// increment register: the stage inputs s2 = u_n + dt/2 k1, s3 = u_n + dt/2 k2
// and s4 = u_n + dt k3 stay in their own buffers, and stage 4 forms
//   u_n+1 = u_n + [(s2 - u_n) + 2 (s3 - u_n) + (s4 - u_n)] / 3 + dt/6 k4,
// the reference's dt (k1/6 + k2/3 + k3/3 + k4/6) regrouped, with one FP64
// addition per value into the FP64 state. Stage 1 takes u_n from the centre
// of its own stencil input, stages 2 and 3 read the copy of u_n, stage 4
// reads s2, s3 and u_n: per point and step 2 + 3 reads and 3 + 2 writes of
// interior values beside the stencil slabs, and no read-modify-write of an
// accumulator. Penalisation and sponge use the double-float mask
// (chi/C_eta with the colour applied, u_s, sponge/C_sponge) built by the
// host from hvy_mask.
//
// Compiled with -fmad=false: the error-free transformations must not be
// contracted; every FMA is explicit.
#include "common.cuh"
#include "df.cuh"
#include "tma.cuh"
#include "umag.cuh"

namespace wg {

struct StageArgsDF {
    const int *blk;
    const BlockDesc *desc;
    const TreeParams *tp;
    TreeClock *clk;        // per tree: dt weights, anchoring constant, running max (stage 4)
    const float2 *in;      // stage input s_j (thin layout, ghosts synchronised)
    const float2 *u0;      // anchored copy of u_n = s1 (thin layout)
    const float2 *s2, *s3; // stage inputs 2 and 3 (thin layout; read by stage 4)
    float2 *out;           // next stage input; at stage 4 the copy of u_{n+1} (null: not stored)
    BufGeo gt;
    double *un;            // u_n, FP64 (full layout)
    double *un_out;        // where stage 4 stores u_n+1 (un, or null: not stored)
    double *cout;          // stage 4: u_n+1 also into a compact interior array (nblk, nc, Bz, By, Bx), or null
    const int *cpos;       // block slot -> its position in cout (and nin)
    const double *nin;     // stage 4: the next step's input (compact like cout): its anchored copy to out, or null
    const double *usrc;    // stage 4: u_n read from this compact array (positions cpos) instead of un, or null
    int record;            // stage 4: merge the maximum of what it stores into the tree's running max
    unsigned long long *usq;   // stage 4: per block slot, max |u|^2 of what it stores (bits + 1), or null
    int rewrite;           // stage 4: store u_n (unchanged) where u_n+1 would go (timing with the state's traffic)
    BufGeo gun;
    const float2 *mask;    // 5 words per point, interior only
    const int *push;       // same-level ghost copies pushed by the writer, or null
    int Bs0, Bs1, Bs2;
    int stage;
    int chunks;
    float third[2];        // 1/3 as a double-float pair
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
// (row: the 27 receiver slots of the writer's block, in global or shared
// memory)
template <int DIM, int NV>
__device__ __forceinline__ void push_ghosts_row(const int *row, int ix, int iy, int iz, int Bs0, int Bs1, int Bs2,
                                                BufGeo gt, float2 *out, long long cs, const float2 *v) {
    const int g = gt.gb;
    const int sx = ix < g ? -1 : (ix >= Bs0 - g ? 1 : 0);
    const int sy = iy < g ? -1 : (iy >= Bs1 - g ? 1 : 0);
    const int sz = DIM == 3 ? (iz < g ? -1 : (iz >= Bs2 - g ? 1 : 0)) : 0;
    const int near = (sx ? 1 : 0) | (sy ? 2 : 0) | (sz ? 4 : 0);
    if (!near) return;
    // the point's offset inside a block; a receiver across (dx, dy, dz) sees
    // it shifted by -(dx Bs0 + dy Bs1 nx + dz Bs2 nx ny)
    const long long own = ((long long)(DIM == 3 ? iz + g : 0) * gt.ny + (iy + g)) * gt.nx + (ix + g);
    for (int sub = near; sub; sub = (sub - 1) & near) {          // non-empty subsets of the near axes
        const int dx = sub & 1 ? sx : 0, dy = sub & 2 ? sy : 0, dz = sub & 4 ? sz : 0;
        const int nb = row[(dz + 1) * 9 + (dy + 1) * 3 + (dx + 1)];
        if (nb < 0) continue;
        float2 *o = out + (long long)nb * NV * cs + own - (dx * Bs0 + (dy * Bs1 + dz * Bs2 * gt.ny) * gt.nx);
#pragma unroll
        for (int c = 0; c < NV; c++) o[c * cs] = v[c];
    }
}

template <int DIM, int NV>
__device__ __forceinline__ void push_ghosts(const int *push, int b, int ix, int iy, int iz, int Bs0, int Bs1,
                                            int Bs2, BufGeo gt, float2 *out, long long cs, const float2 *v) {
    push_ghosts_row<DIM, NV>(push + b * 27, ix, iy, iz, Bs0, Bs1, Bs2, gt, out, cs, v);
}

// The per-block and per-tree constants of a stage, loaded once per thread:
// stencil weights (BlockDesc), physics (TreeParams), the RK weights of the
// stage from the tree's clock and the anchoring constant of the stage input
// this stage writes.
struct DfConst {
    df2 s1[3], s2[3];          // 1/(12 dx), nu/(12 dx^2)
    df2 c0sq, gamma, umean[3];
    df2 db, da;                // dt * b_j, dt * a_(j+1) of the stage
    float M;                   // anchoring constant of the tree (TreeClock::anchor_M)
    int sponge;
};

__device__ __forceinline__ DfConst load_const(const StageArgsDF &a, const BlockDesc &d) {
    DfConst k;
    const TreeParams &tp = a.tp[d.tree];
    const TreeClock &ck = a.clk[d.tree];
#pragma unroll
    for (int i = 0; i < 3; i++) {
        k.s1[i] = cf(d.fs1[i]);
        k.s2[i] = cf(d.fs2[i]);
        k.umean[i] = cf(tp.f_umean[i]);
    }
    k.c0sq = cf(tp.f_c0sq);
    k.gamma = cf(tp.f_gamma);
    k.sponge = tp.use_sponge;
    k.M = ck.anchor_M;
    const int j = a.stage;
    k.db = (j == 1 || j == 4) ? cf(ck.f_dt6) : cf(ck.f_dt3);
    k.da = j == 3 ? cf(ck.f_dt) : df_pow2(cf(ck.f_dt), 0.5f);
    return k;
}

// Stencil numerators of anchored inputs (df.cuh) as double-float pairs:
// the neighbour differences / second differences are formed part by part
// (hi parts exact), their weighted combination by one two-sum.
//   first derivative  8 (A - B) - (E - F)               A, B at +-1, E, F at +-2
//   second derivative 16 (A + B - 2u) - (E + F - 2u)     = 16 (A + B) - (E + F) - 30 u
// In num1 8 dh - eh is exact unless it exceeds 2^24 q, which needs
// |8 dh| > 2^23 q >= |eh|; the quick two-sum is therefore exact.
__device__ __forceinline__ df2 num1(float2 A, float2 B, float2 E, float2 F) {
    const float dh = A.x - B.x, dl = A.y - B.y;
    const float eh = E.x - F.x, el = E.y - F.y;
    const df2 s = quick_two_sum(8.f * dh, -eh);
    return {s.hi, s.lo + fmaf(8.f, dl, -el)};
}

__device__ __forceinline__ df2 num2(float2 A, float2 B, float2 E, float2 F, float2 u2) {
    const float ah = (A.x + B.x) - u2.x, al = (A.y + B.y) - u2.y;
    const float bh = (E.x + F.x) - u2.x, bl = (E.y + F.y) - u2.y;
    const df2 s = two_sum(16.f * ah, -bh);
    return {s.hi, s.lo + fmaf(16.f, al, -bl)};
}

// RHS of one interior point (convective FD_4th_central, RHS_3D_acm /
// RHS_2D_acm, rhs_ACM.f90:578-615,1206-1256, with the penalisation and the
// sponge of :1734-1753) from an anchored stencil input with strides stv
// (shared or global memory). m: the point's double-float mask words (stride
// ms), or null. Returns the RHS in r and the centre values vel, p0.
template <int DIM, typename Idx>
__device__ __forceinline__ void rhs_df(const float2 *u, Idx cs, const int stv[3], const DfConst &d,
                                       const float2 *m, int ms, df2 r[DIM + 1], df2 vel[DIM], df2 &p0) {
    df2 w[DIM];
#pragma unroll
    for (int k = 0; k < DIM; k++) {
        vel[k] = ld(u + k * cs);
        w[k] = df_mul_nr(vel[k], d.s1[k]);                 // u_k / (12 dx_k)
    }
    df2 div = {0.f, 0.f};
#pragma unroll
    for (int c = 0; c < DIM; c++) {
        const float2 *uc = u + c * cs;
        const float2 u2 = make_float2(2.f * vel[c].hi, 2.f * vel[c].lo);
        df2 adv = {0.f, 0.f}, lap = {0.f, 0.f};
#pragma unroll
        for (int k = 0; k < DIM; k++) {
            const float2 A = uc[stv[k]], B = uc[-stv[k]], E = uc[2 * stv[k]], F = uc[-2 * stv[k]];
            const df2 d1 = num1(A, B, E, F);
            const df2 ta = df_mul_nr(w[k], d1), tl = df_mul_nr(d.s2[k], num2(A, B, E, F, u2));
            adv = k == 0 ? ta : df_add_nr(adv, ta);
            lap = k == 0 ? tl : df_add_nr(lap, tl);
            if (k == c) {
                const df2 td = df_mul_nr(d.s1[k], d1);
                div = c == 0 ? td : df_add_nr(div, td);
            }
        }
        r[c] = df_sub_nr(lap, adv);
    }
    const float2 *up = u + DIM * cs;
    p0 = ld(up);
#pragma unroll
    for (int k = 0; k < DIM; k++) {
        const df2 d1 = num1(up[stv[k]], up[-stv[k]], up[2 * stv[k]], up[-2 * stv[k]]);
        r[k] = df_sub_nr(r[k], df_mul_nr(d.s1[k], d1));
    }
    r[DIM] = df_neg(df_add_nr(df_mul_nr(d.c0sq, div), df_mul_nr(d.gamma, p0)));
    if (m) {   // masked block (uniform over the CTA)
        const df2 chi = ld(m);
#pragma unroll
        for (int c = 0; c < DIM; c++) r[c] = df_sub_nr(r[c], df_mul_nr(chi, df_sub_nr(vel[c], ld(m + (1 + c) * ms))));
        if (d.sponge) {
            const df2 spo = ld(m + 4 * ms);
#pragma unroll
            for (int c = 0; c < DIM; c++)
                r[c] = df_sub_nr(r[c], df_mul_nr(spo, df_sub_nr(vel[c], d.umean[c])));
            r[DIM] = df_sub_nr(r[DIM], df_mul_nr(spo, p0));
        }
    }
}

// rhs_df for the march kernel: the x and y neighbours lie in the centre
// plane's slot, the z neighbours in the slots of planes k-2 .. k+2 of the
// ring (comp: stride of one component's ring, xy: offset in a plane).
__device__ __forceinline__ void rhs_df_ring(const float2 *sm, int comp, int k, int xy, const float2 *ctrp,
                                            const DfConst &d, const float2 *m, int ms, df2 r[4], df2 ctr[4]) {
    constexpr int NS = 5, PLANE = 400;
    const int zm2 = ((k + 0) % NS) * PLANE + xy, zm1 = ((k + 1) % NS) * PLANE + xy;
    const int zp1 = ((k + 3) % NS) * PLANE + xy, zp2 = ((k + 4) % NS) * PLANE + xy;
    auto at = [&](int c, int dir, int o) -> float2 {   // neighbour o (+-1, +-2) of component c along dir
        if (dir < 2) return ctrp[c * comp + (dir == 0 ? o : o * 20)];
        const int z = o == -2 ? zm2 : o == -1 ? zm1 : o == 1 ? zp1 : zp2;
        return sm[c * comp + z];
    };
    df2 w[3], vel[3];
#pragma unroll
    for (int kk = 0; kk < 3; kk++) {
        vel[kk] = ld(ctrp + kk * comp);
        w[kk] = df_mul_nr(vel[kk], d.s1[kk]);
    }
    df2 div = {0.f, 0.f};
#pragma unroll
    for (int c = 0; c < 3; c++) {
        const float2 u2 = make_float2(2.f * vel[c].hi, 2.f * vel[c].lo);
        df2 adv = {0.f, 0.f}, lap = {0.f, 0.f};
#pragma unroll
        for (int kk = 0; kk < 3; kk++) {
            const float2 A = at(c, kk, 1), B = at(c, kk, -1), E = at(c, kk, 2), F = at(c, kk, -2);
            const df2 d1 = num1(A, B, E, F);
            const df2 ta = df_mul_nr(w[kk], d1), tl = df_mul_nr(d.s2[kk], num2(A, B, E, F, u2));
            adv = kk == 0 ? ta : df_add_nr(adv, ta);
            lap = kk == 0 ? tl : df_add_nr(lap, tl);
            if (kk == c) {
                const df2 td = df_mul_nr(d.s1[kk], d1);
                div = c == 0 ? td : df_add_nr(div, td);
            }
        }
        r[c] = df_sub_nr(lap, adv);
    }
    const df2 p0 = ld(ctrp + 3 * comp);
#pragma unroll
    for (int kk = 0; kk < 3; kk++) {
        const df2 d1 = num1(at(3, kk, 1), at(3, kk, -1), at(3, kk, 2), at(3, kk, -2));
        r[kk] = df_sub_nr(r[kk], df_mul_nr(d.s1[kk], d1));
    }
    r[3] = df_neg(df_add_nr(df_mul_nr(d.c0sq, div), df_mul_nr(d.gamma, p0)));
    if (m) {   // masked block (uniform over the CTA)
        const df2 chi = ld(m);
#pragma unroll
        for (int c = 0; c < 3; c++) r[c] = df_sub_nr(r[c], df_mul_nr(chi, df_sub_nr(vel[c], ld(m + (1 + c) * ms))));
        if (d.sponge) {
            const df2 spo = ld(m + 4 * ms);
#pragma unroll
            for (int c = 0; c < 3; c++) r[c] = df_sub_nr(r[c], df_mul_nr(spo, df_sub_nr(vel[c], d.umean[c])));
            r[3] = df_sub_nr(r[3], df_mul_nr(spo, p0));
        }
    }
#pragma unroll
    for (int c = 0; c < 3; c++) ctr[c] = vel[c];
    ctr[3] = p0;
}

// Per-point operands of the RK4 stage update that come from memory: the
// copy of u_n (stages 2, 3), or s2, s3 and the bits of u_n (stage 4).
template <int DIM>
struct RkIn {
    float2 a[DIM + 1], b[DIM + 1], c[DIM + 1];
};

__device__ __forceinline__ float2 bits_f2(double v) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(v);
    return make_float2(__uint_as_float((unsigned)b), __uint_as_float((unsigned)(b >> 32)));
}

__device__ __forceinline__ double f2_bits(float2 v) {
    return __longlong_as_double((long long)(((unsigned long long)__float_as_uint(v.y) << 32) | __float_as_uint(v.x)));
}

template <int DIM, int STAGE>
__device__ __forceinline__ void rk_load(const StageArgsDF &a, int b, int ix, int iy, int iz, long long off,
                                        RkIn<DIM> &in) {
    const long long cs = a.gt.npts();
    if (STAGE == 2 || STAGE == 3) {
#pragma unroll
        for (int c = 0; c <= DIM; c++) in.a[c] = a.u0[off + c * cs];
    } else if (STAGE == 4) {
        long long us = a.gun.npts();
        const double *un;
        if (a.usrc) {   // compact: (position, component, z, y, x)
            const int nint = a.Bs0 * a.Bs1 * (DIM == 3 ? a.Bs2 : 1);
            us = nint;
            un = a.usrc + (long long)a.cpos[b] * (DIM + 1) * nint + ((DIM == 3 ? iz * a.Bs1 : 0) + iy) * a.Bs0 + ix;
        } else {
            un = a.un + (long long)b * (DIM + 1) * us +
                 ((long long)(iz + (DIM == 3 ? a.gun.gb : 0)) * a.gun.ny + (iy + a.gun.gb)) * a.gun.nx +
                 (ix + a.gun.gb);
        }
#pragma unroll
        for (int c = 0; c <= DIM; c++) {
            in.a[c] = a.s2[off + c * cs];
            in.b[c] = a.s3[off + c * cs];
            in.c[c] = bits_f2(a.usrc ? __ldcs(un + c * us) : un[c * us]);
        }
    }
}

// The per-block maximum of |u|^2 that the next dt reduction needs
// (k_misc.cu::dt_kernel), taken from the values the last stage stores: the
// FP64 sum u*u + v*v (+ w*w) rounded in the reduction's order, and its
// divergence guard on every component. usq_term adds component c.
template <int DIM>
__device__ __forceinline__ void usq_term(int c, double w, double &usq, bool &ok) {
    ok &= within_guard(w);
    if (c < DIM) {
        const double p = __dmul_rn(w, w);
        usq = c == 0 ? p : __dadd_rn(usq, p);
    }
}

// merge of one point's |u|^2 into the block's maximum: the warp's maximum
// (every warp of every stage form holds points of one block) by one atomic.
// The reduction's fmax skips nan sums, so they do not count here either; a
// value s >= 0 is kept as its bits + 1 (ordered like s), 0 meaning none.
__device__ __forceinline__ void usq_merge(const StageArgsDF &a, int b, double usq, bool ok) {
    unsigned long long e = (unsigned long long)__double_as_longlong(usq);
    e = (e & 0x7fffffffffffffffull) > 0x7ff0000000000000ull ? 0ull : e + 1ull;
    const unsigned am = __activemask();
    const unsigned hi = __reduce_max_sync(am, (unsigned)(e >> 32));
    const unsigned lo = __reduce_max_sync(am, (unsigned)(e >> 32) == hi ? (unsigned)e : 0u);
    if ((threadIdx.x & 31) == (unsigned)(__ffs(am) - 1) && (hi | lo))
        atomicMax(a.usq + b, ((unsigned long long)hi << 32) | lo);
    if (!ok) atomicOr(&a.clk[a.desc[b].tree].div_next, 1);
}

// RK4 stage update of one point: stages 1-3 write the anchored next stage
// input u_n + a dt k_j (a = 1/2, 1/2, 1), stage 4 writes u_n+1 to the FP64
// state (unless un_out is null), to cout (when given) and its anchored copy
// (unless out is null), and returns the largest |u_n+1| of the point in
// umax. ctr: the centre values of this stage's input (s1 = u_n at stage 1,
// s4 at stage 4). (ix, iy, iz): interior coordinates; off: the point's
// offset in the thin buffers (component 0).
template <int DIM, int STAGE>
__device__ __forceinline__ void rk_df(const StageArgsDF &a, const DfConst &k, int b, int ix, int iy, int iz,
                                      long long off, const df2 r[DIM + 1], const df2 ctr[DIM + 1],
                                      const RkIn<DIM> &in, float &umax) {
    const long long cs = a.gt.npts();
    float2 *o = a.out ? a.out + off : nullptr;
    float2 ov[DIM + 1];
    if (STAGE < 4) {
#pragma unroll
        for (int c = 0; c <= DIM; c++) {
            const df2 u0 = STAGE == 1 ? ctr[c] : df2{in.a[c].x, in.a[c].y};
            const df2 v = anchor(df_add_nr(u0, df_mul_nr(k.da, df_norm(r[c]))), k.M);
            ov[c] = make_float2(v.hi, v.lo);
            o[c * cs] = ov[c];
        }
    } else {
        const long long us = a.gun.npts();
        double *un = a.un + (long long)b * (DIM + 1) * us +
                     ((long long)(iz + (DIM == 3 ? a.gun.gb : 0)) * a.gun.ny + (iy + a.gun.gb)) * a.gun.nx +
                     (ix + a.gun.gb);
        const df2 third = {a.third[0], a.third[1]};
        float2 *const ob = a.out;
        // the point in the compact arrays cout / nin (their component stride)
        const int nint = a.Bs0 * a.Bs1 * (DIM == 3 ? a.Bs2 : 1);
        const long long cbase = a.cout || a.nin ? (long long)a.cpos[b] * (DIM + 1) * nint +
                                                      ((DIM == 3 ? iz * a.Bs1 : 0) + iy) * a.Bs0 + ix
                                                : 0;
        double usq = 0.0;   // |u|^2 of the stored velocity, in the order of the dt reduction
        bool ok = true;     // every stored component within the divergence guard
#pragma unroll
        for (int c = 0; c <= DIM; c++) {
            const double u = f2_bits(in.c[c]);
            const df2 ud = df_split(u);
            // s2 + 2 s3 + s4: the three inputs of this step share one quantum,
            // so the hi sum is exact; then - 4 u_n as a double-float difference
            const float sh = fmaf(2.f, in.b[c].x, in.a[c].x + ctr[c].hi);
            const float sl = fmaf(2.f, in.b[c].y, in.a[c].y + ctr[c].lo);
            const df2 sum = df_sub_nr({sh, sl}, df_pow2(ud, 4.f));
            const df2 inc = df_norm(df_add_nr(df_mul_nr(third, sum), df_mul_nr(k.db, df_norm(r[c]))));
            const double v = __dadd_rn(u, df_to_double(inc));
            const long long ci = cbase + (long long)c * nint;
            if (a.cout) a.cout[ci] = v;
            if (a.nin) {   // the next input takes the place of u_n+1 in the anchored copy
                const double x = __ldcs(a.nin + ci);
                if (a.usq) usq_term<DIM>(c, x, usq, ok);
                if (ob) {
                    const df2 sx = df_split(x);
                    const df2 w = anchor(sx, k.M);
                    ov[c] = make_float2(w.hi, w.lo);
                    o[c * cs] = ov[c];
                    umax = fmaxf(umax, fabsf(sx.hi));
                }
                continue;
            }
            if (a.un_out) un[c * us] = a.rewrite ? u : v;
            if (a.usq) usq_term<DIM>(c, a.rewrite ? u : v, usq, ok);
            if (ob) {   // the anchored copy of u_n+1 and its running maximum
                const df2 w = anchor(df_add_nr(ud, inc), k.M);
                ov[c] = make_float2(w.hi, w.lo);
                o[c * cs] = ov[c];
                umax = fmaxf(umax, fabsf(w.hi));
            }
        }
        if (a.usq) usq_merge(a, b, usq, ok);
        if (!ob) return;   // the result went to cout alone
    }
    if (a.push) push_ghosts<DIM, DIM + 1>(a.push, b, ix, iy, iz, a.Bs0, a.Bs1, a.Bs2, a.gt, a.out, cs, ov);
}

// block-wide max of umax merged into the tree's running max (stage 4);
// every thread of the CTA calls it
__device__ __forceinline__ void merge_umax(float umax, TreeClock *clk, int tree) {
    __shared__ float red[32];
    for (int o = 16; o; o >>= 1) umax = fmaxf(umax, __shfl_xor_sync(0xffffffffu, umax, o));
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = umax;
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int w = 1; w < (int)(blockDim.x >> 5); w++) umax = fmaxf(umax, red[w]);
        atomicMax(&clk[tree].umax_f, __float_as_uint(umax));
    }
}

// One thread per interior point, stencil values read from global memory.
// BS: the block edge when all Bs are equal to it (index arithmetic by
// shifts), 0 for the general case.
template <int DIM, int STAGE>
__device__ __forceinline__ void direct_point(const StageArgsDF &a, const DfConst &k, const float2 *u, long long cs,
                                             const int stv[3], const float2 *m, int ms, int b, int ix, int iy, int iz,
                                             long long off, float &umax) {
    df2 r[DIM + 1], ctr[DIM + 1];
    RkIn<DIM> in;
    rk_load<DIM, STAGE>(a, b, ix, iy, iz, off, in);
    rhs_df<DIM>(u, cs, stv, k, m, ms, r, ctr, ctr[DIM]);
    rk_df<DIM, STAGE>(a, k, b, ix, iy, iz, off, r, ctr, in, umax);
}

// Masked blocks (d.mask >= 0) and unmasked ones share the launch; the branch
// between the two bodies is uniform per CTA.
template <int DIM, int BS, bool MASKED>
__global__ void __launch_bounds__(256, 3) acm_stage_df_kernel(StageArgsDF a) {
    const int Bs0 = BS ? BS : a.Bs0, Bs1 = BS ? BS : a.Bs1, Bs2 = BS ? BS : a.Bs2;
    const int npts_int = Bs0 * Bs1 * (DIM == 3 ? Bs2 : 1);
    const int chunks = BS ? (npts_int + 255) / 256 : a.chunks;
    const int bi = blockIdx.x / chunks;
    const int q = (blockIdx.x - bi * chunks) * blockDim.x + threadIdx.x;
    const int b = a.blk[bi];
    const BlockDesc &d = a.desc[b];
    float umax = 0.f;
    if (q < npts_int) {
        const int ix = q % Bs0, iy = (q / Bs0) % Bs1, iz = DIM == 3 ? q / (Bs0 * Bs1) : 0;
        const long long cs = a.gt.npts();
        const long long off = (long long)b * (DIM + 1) * cs +
                              ((long long)(iz + (DIM == 3 ? a.gt.gb : 0)) * a.gt.ny + (iy + a.gt.gb)) * a.gt.nx +
                              (ix + a.gt.gb);
        const int stv[3] = {1, a.gt.nx, a.gt.nx * a.gt.ny};
        const DfConst k = load_const(a, d);
        const float2 *u = a.in + off;
        const float2 *m = MASKED ? a.mask + (long long)d.mask * 5 * npts_int + q : nullptr;
        switch (a.stage) {
            case 1: direct_point<DIM, 1>(a, k, u, cs, stv, m, npts_int, b, ix, iy, iz, off, umax); break;
            case 2: direct_point<DIM, 2>(a, k, u, cs, stv, m, npts_int, b, ix, iy, iz, off, umax); break;
            case 3: direct_point<DIM, 3>(a, k, u, cs, stv, m, npts_int, b, ix, iy, iz, off, umax); break;
            default: direct_point<DIM, 4>(a, k, u, cs, stv, m, npts_int, b, ix, iy, iz, off, umax); break;
        }
    }
    if (a.stage == 4 && a.record) merge_umax(umax, a.clk, d.tree);
}

// 3-D blocks of 16x16xBs2 points with 2 ghost layers (the stage-input
// layout of FD_4th_central): each CTA of 256 threads takes a slab of ZT
// interior planes of one block (ZT = 2, 4 or 8: 76.8, 102.4 or 153.6 KB of
// shared memory). One elected thread loads the slab's stencil
// input (ZT+4 planes of 20x20 points per component, ghosts included) with
// one TMA box per component into shared memory; every thread then walks its
// (x, y) column through the slab, reading all stencil values from shared
// memory at compile-time offsets. A TMA completion that does not arrive
// within a second on any thread sets *err and ends the CTA after giving the
// copy in flight a second bounded wait; the context's state is then
// undefined.
template <int ZT, int STAGE, bool MASKED>
__global__ void __launch_bounds__(256, 2) acm_stage_df_tile(StageArgsDF a, const __grid_constant__ CUtensorMap tin,
                                                            int nslab, int *err) {
    constexpr int NX = 20, NY = 20, GB = 2, BS = 16;
    constexpr int PLANE = NX * NY, COMP = (ZT + 4) * PLANE;
    extern __shared__ __align__(128) float2 sm[];
    __shared__ unsigned long long bar;
    const int bi = blockIdx.x / nslab, slab = blockIdx.x % nslab;
    const int b = a.blk[bi];
    const int zb = slab * ZT;
    if (threadIdx.x == 0) {
        mbar_init(&bar, 1);
        mbar_arrive_expect_tx(&bar, (unsigned)(4 * COMP * sizeof(float2)));
#pragma unroll
        for (int c = 0; c < 4; c++)
            tma_load_3d(sm + c * COMP, &tin, 0, 0, (b * 4 + c) * a.gt.nz + zb + GB - 2, &bar);
    }
    __syncthreads();   // the barrier is initialised before anyone waits on it
    const BlockDesc &d = a.desc[b];
    const DfConst kc = load_const(a, d);
    const int ix = threadIdx.x % BS, iy = threadIdx.x / BS;
    const int npts_int = BS * BS * a.Bs2;
    constexpr int stv[3] = {1, NX, PLANE};
    const long long boff = (long long)b * 4 * a.gt.npts() + (long long)(iy + GB) * NX + (ix + GB);
    // the memory operands of the RK update are fetched one plane ahead (the
    // first plane's while the TMA load is in flight)
    RkIn<3> nxt;
    rk_load<3, STAGE>(a, b, ix, iy, zb, boff + (long long)(zb + GB) * PLANE, nxt);
    // the decision to go on is the CTA's, so every thread meets the barriers
    // below or none does
    if (!__syncthreads_and(mbar_wait(&bar, 0, 1000000000ull))) {
        if (threadIdx.x == 0) {
            atomicExch(err, 1);
            mbar_wait(&bar, 0, 1000000000ull);
        }
        return;
    }
    float umax = 0.f;
#pragma unroll 1
    for (int k = 0; k < ZT; k++) {
        const int iz = zb + k;
        const int q = (iz * BS + iy) * BS + ix;
        const long long off = boff + (long long)(iz + GB) * PLANE;
        const RkIn<3> cur = nxt;
        if (k + 1 < ZT) rk_load<3, STAGE>(a, b, ix, iy, iz + 1, off + PLANE, nxt);
        const float2 *u = sm + ((k + 2) * NY + (iy + GB)) * NX + (ix + GB);
        df2 r[4], ctr[4];
        rhs_df<3>(u, COMP, stv, kc, MASKED ? a.mask + (long long)d.mask * 5 * npts_int + q : nullptr, npts_int, r, ctr,
                  ctr[3]);
        rk_df<3, STAGE>(a, kc, b, ix, iy, iz, off, r, ctr, cur, umax);
    }
    if (STAGE == 4 && a.record) merge_umax(umax, a.clk, d.tree);
}

// Whole-block form of the tile kernel ("march"): one CTA per 16x16x16
// block walks its 16 planes in z. Shared memory holds a ring of 5 planes of
// 20x20 points per component (the planes k-2 .. k+2 of the point being
// computed, ghosts included, 64 KB), so three CTAs fit on an SM beside each
// other; after plane k every thread has finished with plane k-2, whose slot
// then receives plane k+3 by TMA (one box of 20x20x1 per component) while
// the next plane is computed. The planes of a block are loaded once (20
// planes for 16) instead of twice per 4-plane slab. A TMA completion that
// does not arrive within a second on any thread sets *err and ends the CTA
// after a bounded wait for the copies in flight; the context's state is then
// undefined.
template <int STAGE, bool MASKED>
__global__ void __launch_bounds__(256, 3) acm_stage_df_march(StageArgsDF a, const __grid_constant__ CUtensorMap tin,
                                                             int *err) {
    constexpr int NX = 20, NY = 20, GB = 2, BS = 16, NS = 5, NZ = 16;
    constexpr int PLANE = NX * NY, COMP = NS * PLANE;
    extern __shared__ __align__(128) float2 sm[];
    __shared__ unsigned long long bar[NS];
    const int b = a.blk[blockIdx.x];
    // plane p (interior index -2 .. NZ+1) sits in slot (p + 2) % NS; its
    // fill of that slot is the ((p + 2) / NS)-th
    auto load_plane = [&](int p) {
        const int slot = (p + 2) % NS;
        mbar_arrive_expect_tx(&bar[slot], (unsigned)(4 * PLANE * sizeof(float2)));
#pragma unroll
        for (int c = 0; c < 4; c++)
            tma_load_3d(sm + c * COMP + slot * PLANE, &tin, 0, 0, (b * 4 + c) * a.gt.nz + p + GB, &bar[slot]);
    };
    if (threadIdx.x == 0) {
        for (int i = 0; i < NS; i++) mbar_init(&bar[i], 1);
        for (int p = -2; p <= 2; p++) load_plane(p);
    }
    __syncthreads();   // the barriers are initialised before anyone waits on them
    const BlockDesc &d = a.desc[b];
    const DfConst kc = load_const(a, d);
    const int ix = threadIdx.x % BS, iy = threadIdx.x / BS;
    const int npts_int = BS * BS * a.Bs2;
    constexpr int stv[3] = {1, NX, PLANE};
    const long long boff = (long long)b * 4 * a.gt.npts() + (long long)(iy + GB) * NX + (ix + GB);
    RkIn<3> nxt;
    rk_load<3, STAGE>(a, b, ix, iy, 0, boff + (long long)GB * PLANE, nxt);
    bool ok = true;
    for (int p = -2; p <= 1; p++) ok &= mbar_wait(&bar[(p + 2) % NS], 0, 1000000000ull);
    float umax = 0.f;
#pragma unroll 1
    for (int k = 0; k < NZ; k++) {
        // plane k+2 completes the stencil of plane k
        ok &= mbar_wait(&bar[(k + 4) % NS], ((k + 4) / NS) & 1, 1000000000ull);
        const int q = (k * BS + iy) * BS + ix;
        const long long off = boff + (long long)(k + GB) * PLANE;
        const RkIn<3> cur = nxt;
        if (k + 1 < NZ) rk_load<3, STAGE>(a, b, ix, iy, k + 1, off + PLANE, nxt);
        // the ring's slots are not in z order: the stencil reads each plane
        // through its own slot pointer
        const float2 *ctrp = sm + ((k + 2) % NS) * PLANE + (iy + GB) * NX + (ix + GB);
        df2 r[4], ctr[4];
        rhs_df_ring(sm, COMP, k, (iy + GB) * NX + (ix + GB), ctrp, kc,
                    MASKED ? a.mask + (long long)d.mask * 5 * npts_int + q : nullptr, npts_int, r, ctr);
        rk_df<3, STAGE>(a, kc, b, ix, iy, k, off, r, ctr, cur, umax);
        // every thread is done with plane k-2: its slot takes plane k+3; the
        // decision to go on is the CTA's
        if (!__syncthreads_and(ok)) {
            if (threadIdx.x == 0) {   // the copy of plane k+2 may still be landing
                atomicExch(err, 1);
                mbar_wait(&bar[(k + 4) % NS], ((k + 4) / NS) & 1, 1000000000ull);
            }
            return;
        }
        if (threadIdx.x == 0 && k + 3 <= NZ + 1) {
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            load_plane(k + 3);
        }
    }
    if (STAGE == 4 && a.record) merge_umax(umax, a.clk, d.tree);
}

// Persistent form of the tile kernel ("pipe"): one launch per RK stage for
// all blocks of all listed trees, masked and unmasked. One CTA of 512
// threads per SM walks the slabs s = blockIdx.x, blockIdx.x + gridDim.x, ...
// of the block list (4 slabs of 4 planes per 16^3 block; the masked blocks
// come first, and a slab runs the masked or the unmasked body, uniform over
// the CTA). Shared memory holds two slab buffers (2 x 102.4 KB): while the
// CTA computes the slab in one, TMA fills the other with the CTA's next
// slab, so the 16 warps keep issuing while the loads run (the tile form's
// CTAs wait for their own slab, and an SM then computes with half of its
// warps). Threads 0-255 compute planes 0-1 of their (x, y) column, threads
// 256-511 planes 2-3. Neighbouring CTAs take neighbouring slabs at the same
// time, so the halo planes two slabs share come from L2. The arithmetic is
// the tile form's, in the same order. A TMA completion that does not arrive
// within a second on any thread sets *err and ends the CTA after bounded
// waits for both buffers' copies in flight; the context's state is then
// undefined.
template <int STAGE, bool MASKED>
__device__ __forceinline__ void pipe_planes(const StageArgsDF &a, const DfConst &kc, const BlockDesc &d, int b,
                                            const float2 *sb, int zs, int z0, int ix, int iy, long long boff,
                                            RkIn<3> &nxt, float &umax) {
    constexpr int NX = 20, NY = 20, GB = 2, BS = 16, ZT = 4;
    constexpr int PLANE = NX * NY, COMP = (ZT + 4) * PLANE;
    constexpr int stv[3] = {1, NX, PLANE};
    const int npts_int = BS * BS * a.Bs2;
#pragma unroll 1
    for (int k = 0; k < 2; k++) {
        const int iz = z0 + k;
        const int q = (iz * BS + iy) * BS + ix;
        const long long off = boff + (long long)(iz + GB) * PLANE;
        const RkIn<3> cur = nxt;
        if (k == 0) rk_load<3, STAGE>(a, b, ix, iy, iz + 1, off + PLANE, nxt);
        const float2 *u = sb + ((iz - zs + 2) * NY + (iy + GB)) * NX + (ix + GB);
        df2 r[4], ctr[4];
        rhs_df<3>(u, COMP, stv, kc, MASKED ? a.mask + (long long)d.mask * 5 * npts_int + q : nullptr, npts_int, r,
                  ctr, ctr[3]);
        rk_df<3, STAGE>(a, kc, b, ix, iy, iz, off, r, ctr, cur, umax);
    }
}

template <int STAGE>
__global__ void __launch_bounds__(512, 1) acm_stage_df_pipe(StageArgsDF a, const __grid_constant__ CUtensorMap tin,
                                                            int nslab_total, int nslab_masked, int *err) {
    constexpr int NX = 20, NY = 20, GB = 2, BS = 16, ZT = 4;
    constexpr int PLANE = NX * NY, COMP = (ZT + 4) * PLANE, BUF = 4 * COMP;
    extern __shared__ __align__(128) float2 sm[];
    __shared__ unsigned long long bar[2];
    const int nsb = a.Bs2 / ZT;   // slabs per block
    const int total = nslab_total;
    const int step = (int)gridDim.x;
    auto issue = [&](int s, int buf) {
        const int b = a.blk[s / nsb], zb = (s % nsb) * ZT;
        mbar_arrive_expect_tx(&bar[buf], (unsigned)(4 * COMP * sizeof(float2)));
#pragma unroll
        for (int c = 0; c < 4; c++)
            tma_load_3d(sm + buf * BUF + c * COMP, &tin, 0, 0, (b * 4 + c) * a.gt.nz + zb + GB - 2, &bar[buf]);
    };
    if (threadIdx.x == 0) {
        mbar_init(&bar[0], 1);
        mbar_init(&bar[1], 1);
        if ((int)blockIdx.x < total) issue((int)blockIdx.x, 0);
        if ((int)blockIdx.x + step < total) issue((int)blockIdx.x + step, 1);
    }
    __syncthreads();   // the barriers are initialised before anyone waits on them
    const int col = threadIdx.x & 255, half = threadIdx.x >> 8;
    const int ix = col % BS, iy = col / BS;
    float umax = 0.f;
    int utree = -1;   // tree whose maximum umax holds (stage 4)
    int j = 0;
#pragma unroll 1
    for (int s = (int)blockIdx.x; s < total; s += step, j++) {
        const int buf = j & 1;
        const int b = a.blk[s / nsb];
        const int zs = (s % nsb) * ZT;      // first plane of the slab
        const int z0 = zs + 2 * half;       // first plane of this thread
        const BlockDesc &d = a.desc[b];
        if (STAGE == 4 && a.record && d.tree != utree) {   // uniform over the CTA
            if (utree >= 0) merge_umax(umax, a.clk, utree);
            umax = 0.f;
            utree = d.tree;
        }
        const DfConst kc = load_const(a, d);
        const long long boff = (long long)b * 4 * a.gt.npts() + (long long)(iy + GB) * NX + (ix + GB);
        RkIn<3> nxt;
        rk_load<3, STAGE>(a, b, ix, iy, z0, boff + (long long)(z0 + GB) * PLANE, nxt);
        // the n-th fill of a buffer completes its phase n; the decision to go
        // on is the CTA's, so every thread meets the barriers below or none does
        if (!__syncthreads_and(mbar_wait(&bar[buf], (unsigned)(j >> 1) & 1u, 1000000000ull))) {
            if (threadIdx.x == 0) {   // this slab's copy and the next one's may still be landing
                atomicExch(err, 1);
                mbar_wait(&bar[buf], (unsigned)(j >> 1) & 1u, 1000000000ull);
                if (s + step < total) mbar_wait(&bar[buf ^ 1], (unsigned)((j + 1) >> 1) & 1u, 1000000000ull);
            }
            return;
        }
        const float2 *sb = sm + buf * BUF;
        if (s < nslab_masked) pipe_planes<STAGE, true>(a, kc, d, b, sb, zs, z0, ix, iy, boff, nxt, umax);
        else pipe_planes<STAGE, false>(a, kc, d, b, sb, zs, z0, ix, iy, boff, nxt, umax);
        __syncthreads();   // every thread is done with this buffer: it takes the slab after next
        if (threadIdx.x == 0 && s + 2 * step < total) {
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            issue(s + 2 * step, buf);
        }
    }
    if (STAGE == 4 && a.record && utree >= 0) merge_umax(umax, a.clk, utree);
}

// slab height of the tile kernel (0: not applicable): 16x16 planes, two
// ghost layers, Bs2 a multiple of 4
int tile_slab(int dim, int Bs0, int Bs1, int Bs2, int g) {
    if (dim != 3 || Bs0 != 16 || Bs1 != 16 || g != 2 || Bs2 % 4) return 0;
    return 4;
}

cudaError_t launch_acm_stage_df(int dim, int stage, int masked, const int *blk, int nblk, const BlockDesc *desc,
                                const TreeParams *tp, TreeClock *clk, const void *in, const void *u0, const void *s2,
                                const void *s3, void *out, BufGeo gt, double *un, BufGeo gun, const void *maskdf,
                                const int *push, int Bs0, int Bs1, int Bs2, const void *tmap, int march, int *err,
                                cudaStream_t s, int keep_state, double *cout, const int *cpos, const double *nin,
                                const double *usrc, unsigned long long *usq) {
    if (nblk <= 0) return cudaSuccess;
    if (stage < 1 || stage > 4) return cudaErrorInvalidValue;
    StageArgsDF a;
    a.blk = blk;
    a.desc = desc;
    a.tp = tp;
    a.clk = clk;
    a.in = reinterpret_cast<const float2 *>(in);
    a.u0 = reinterpret_cast<const float2 *>(u0);
    a.s2 = reinterpret_cast<const float2 *>(s2);
    a.s3 = reinterpret_cast<const float2 *>(s3);
    a.out = reinterpret_cast<float2 *>(out);
    a.gt = gt;
    a.un = un;
    // keep_state 1: u_n+1 to the state, its copy to out, its maximum recorded
    // (and to cout when given); 0 (timing): the copy to out only; 4 (timing
    // with the state's traffic): as 0, and u_n written back unchanged where
    // u_n+1 would go; 2: u_n+1 to cout only (a result the next input
    // replaces); 3: u_n+1 to cout, and the anchored copy of the next step's
    // input nin (compact like cout) to out with its maximum recorded (the
    // next step reads u_n from nin: usrc). usrc (stage 4, with cpos): u_n
    // is read from that compact array instead of un.
    if (keep_state < 0 || keep_state > 4 || ((keep_state == 2 || keep_state == 3) && (stage != 4 || !cout || !cpos)) ||
        (keep_state == 3 && !nin) || (usrc && (stage != 4 || !cpos || keep_state == 4)))
        return cudaErrorInvalidValue;
    a.un_out = keep_state == 1 || keep_state == 4 ? un : nullptr;
    a.usrc = stage == 4 ? usrc : nullptr;
    a.cout = (keep_state == 1 || keep_state == 2 || keep_state == 3) && stage == 4 ? cout : nullptr;
    a.nin = keep_state == 3 ? nin : nullptr;
    a.record = keep_state == 1 || keep_state == 3;
    // (timing with the state's traffic records the maxima of the state it
    // rewrites, the values the recording of the last stage that wrote the
    // state holds: the timed kernel does the same work as the real one)
    a.usq = (a.record || keep_state == 4) && stage == 4 ? usq : nullptr;
    a.rewrite = keep_state == 4;
    if (keep_state == 2) a.out = nullptr;
    a.cpos = cpos;
    a.gun = gun;
    a.mask = reinterpret_cast<const float2 *>(maskdf);
    a.push = push;
    a.Bs0 = Bs0;
    a.Bs1 = Bs1;
    a.Bs2 = Bs2;
    a.stage = stage;
    {
        const double t = 1.0 / 3.0;
        a.third[0] = (float)t;
        a.third[1] = (float)(t - (double)a.third[0]);
    }
    const int zt = tmap ? tile_slab(dim, Bs0, Bs1, Bs2, gt.gb) : 0;
    if (march == 2 && zt == 4 && gt.nx == 20 && gt.ny == 20) {
        // masked: the number of masked blocks at the head of blk
        if (masked < 0 || masked > nblk) return cudaErrorInvalidValue;
        const long long total = (long long)nblk * (Bs2 / zt);
        if (total >= (1ll << 31)) return cudaErrorInvalidValue;
        const size_t smem = sizeof(float2) * 2 * 4 * (size_t)(zt + 4) * gt.nx * gt.ny;
        const CUtensorMap &map = *reinterpret_cast<const CUtensorMap *>(tmap);
        using K = void (*)(StageArgsDF, const CUtensorMap, int, int, int *);
        static const K kerns[4] = {acm_stage_df_pipe<1>, acm_stage_df_pipe<2>, acm_stage_df_pipe<3>,
                                   acm_stage_df_pipe<4>};
        const K kern = kerns[stage - 1];
        cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        int dev = 0, nsm = 0;
        if ((e = cudaGetDevice(&dev)) != cudaSuccess) return e;
        if ((e = cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess) return e;
        a.chunks = 0;
        const unsigned grid = (unsigned)std::min<long long>(total, (long long)std::max(1, nsm));
        kern<<<grid, 512, smem, s>>>(a, map, (int)total, masked * (Bs2 / zt), err);
        return cudaGetLastError();
    }
    if (march == 1 && zt == 4 && Bs2 == 16 && gt.nx == 20 && gt.ny == 20) {
        const size_t smem = sizeof(float2) * 4 * 5 * (size_t)gt.nx * gt.ny;
        const CUtensorMap &map = *reinterpret_cast<const CUtensorMap *>(tmap);
        using K = void (*)(StageArgsDF, const CUtensorMap, int *);
        static const K kerns[2][4] = {
            {acm_stage_df_march<1, false>, acm_stage_df_march<2, false>, acm_stage_df_march<3, false>,
             acm_stage_df_march<4, false>},
            {acm_stage_df_march<1, true>, acm_stage_df_march<2, true>, acm_stage_df_march<3, true>,
             acm_stage_df_march<4, true>}};
        const K kern = kerns[masked ? 1 : 0][stage - 1];
        cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        a.chunks = 0;
        kern<<<(unsigned)nblk, 256, smem, s>>>(a, map, err);
        return cudaGetLastError();
    }
    if ((march == 0 || march == 3 || march == 4) && zt == 4 && gt.nx == 20 && gt.ny == 20) {
        // slab height: 4 (march 0), 2 (march 3) or 8 (march 4) interior
        // planes per CTA; tmap's boxes hold that height plus four ghost planes
        const int z = march == 3 ? 2 : march == 4 ? 8 : 4;
        if (Bs2 % z) return cudaErrorInvalidValue;
        const int nslab = Bs2 / z;
        const size_t smem = sizeof(float2) * 4 * (size_t)(z + 4) * gt.nx * gt.ny;
        const CUtensorMap &map = *reinterpret_cast<const CUtensorMap *>(tmap);
        using K = void (*)(StageArgsDF, const CUtensorMap, int, int *);
        static const K kerns[3][2][4] = {
            {{acm_stage_df_tile<4, 1, false>, acm_stage_df_tile<4, 2, false>, acm_stage_df_tile<4, 3, false>,
              acm_stage_df_tile<4, 4, false>},
             {acm_stage_df_tile<4, 1, true>, acm_stage_df_tile<4, 2, true>, acm_stage_df_tile<4, 3, true>,
              acm_stage_df_tile<4, 4, true>}},
            {{acm_stage_df_tile<2, 1, false>, acm_stage_df_tile<2, 2, false>, acm_stage_df_tile<2, 3, false>,
              acm_stage_df_tile<2, 4, false>},
             {acm_stage_df_tile<2, 1, true>, acm_stage_df_tile<2, 2, true>, acm_stage_df_tile<2, 3, true>,
              acm_stage_df_tile<2, 4, true>}},
            {{acm_stage_df_tile<8, 1, false>, acm_stage_df_tile<8, 2, false>, acm_stage_df_tile<8, 3, false>,
              acm_stage_df_tile<8, 4, false>},
             {acm_stage_df_tile<8, 1, true>, acm_stage_df_tile<8, 2, true>, acm_stage_df_tile<8, 3, true>,
              acm_stage_df_tile<8, 4, true>}}};
        const K kern = kerns[march == 3 ? 1 : march == 4 ? 2 : 0][masked ? 1 : 0][stage - 1];
        cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        a.chunks = 0;
        kern<<<(unsigned)((long long)nblk * nslab), 256, smem, s>>>(a, map, nslab, err);
        return cudaGetLastError();
    }
    const int npts_int = Bs0 * Bs1 * (dim == 3 ? Bs2 : 1);
    const int threads = 256;
    a.chunks = (npts_int + threads - 1) / threads;
    const unsigned grid = (unsigned)((long long)nblk * a.chunks);
    const bool b16 = Bs0 == 16 && Bs1 == 16 && (dim == 2 || Bs2 == 16);
    using K = void (*)(StageArgsDF);
    static const K kerns[2][2][2] = {
        {{acm_stage_df_kernel<2, 0, false>, acm_stage_df_kernel<2, 0, true>},
         {acm_stage_df_kernel<2, 16, false>, acm_stage_df_kernel<2, 16, true>}},
        {{acm_stage_df_kernel<3, 0, false>, acm_stage_df_kernel<3, 0, true>},
         {acm_stage_df_kernel<3, 16, false>, acm_stage_df_kernel<3, 16, true>}}};
    kerns[dim == 3 ? 1 : 0][b16 ? 1 : 0][masked ? 1 : 0]<<<grid, threads, 0, s>>>(a);
    return cudaGetLastError();
}

// anchored double-float copy (df_split, then the tree's quantum) of the
// interiors of the listed blocks
__global__ void __launch_bounds__(256) shadow_kernel(const int *__restrict__ blk, const double *src, BufGeo gs,
                                                     float2 *dst, BufGeo gd, int nc, int Bx, int By, int Bz,
                                                     const int *push, const BlockDesc *desc, const TreeClock *clk,
                                                     int only_if_flagged, const int *cpos) {
    // one CTA per (block, component), 32-bit index arithmetic within the block
    const int b = blk[blockIdx.x], c = blockIdx.y;
    if (only_if_flagged && !clk[desc[b].tree].reshadow) return;
    const int nint = Bx * By * Bz;
    const int zs = gs.nz > 1 ? gs.gb : 0, zd = gd.nz > 1 ? gd.gb : 0;
    const double *sb = cpos ? src + ((long long)cpos[b] * nc + c) * nint : src + ((long long)b * nc + c) * gs.npts();
    float2 *dc = dst + (long long)c * gd.npts();
    float2 *db = dc + (long long)b * nc * gd.npts();
    const float M = clk[desc[b].tree].anchor_M;
    for (int i = threadIdx.x; i < nint; i += blockDim.x) {
        const int ix = i % Bx, iy = (i / Bx) % By, iz = i / (Bx * By);
        const double v = cpos ? sb[i] : sb[((iz + zs) * gs.ny + (iy + gs.gb)) * gs.nx + (ix + gs.gb)];
        const df2 w = anchor(df_split(v), M);
        const float2 f = make_float2(w.hi, w.lo);
        db[((iz + zd) * gd.ny + (iy + gd.gb)) * gd.nx + (ix + gd.gb)] = f;
        if (push) {
            if (gd.nz > 1) push_ghosts<3, 1>(push, b, ix, iy, iz, Bx, By, Bz, gd, dc, gd.npts() * nc, &f);
            else push_ghosts<2, 1>(push, b, ix, iy, iz, Bx, By, Bz, gd, dc, gd.npts() * nc, &f);
        }
    }
}

// Interior exchange with a compact array (nblk, nc, Bz, By, Bx): one CTA
// row per (block, component), 32-bit index arithmetic. Towards the state it
// also merges max |u| into the tree's running max (clk, when given), from
// which the anchored copy of the FP32-pipe precision takes its quantum.
// BS: the block edge when all edges equal it (index arithmetic by shifts),
// 0 for the general case
template <int BS>
__global__ void __launch_bounds__(256) interior_xfer_kernel(const int *__restrict__ slots, double *compact, double *A,
                                                            BufGeo ga, int nc, int Bx_, int By_, int Bz_, int to_state,
                                                            const BlockDesc *desc, TreeClock *clk, float2 *shadow,
                                                            BufGeo gs, const int *push) {
    const int Bx = BS ? BS : Bx_, By = BS ? BS : By_, Bz = BS ? (Bz_ > 1 ? BS : 1) : Bz_;
    const int b = slots[blockIdx.x], c = blockIdx.y;
    const int nint = Bx * By * Bz;
    double *cp = compact + ((long long)blockIdx.x * nc + c) * nint;
    double *ab = A + ((long long)b * nc + c) * ga.npts();
    const int za = ga.nz > 1 ? ga.gb : 0, zs = gs.nz > 1 ? gs.gb : 0;
    float2 *dc = shadow ? shadow + (long long)c * gs.npts() : nullptr;
    float2 *db = shadow ? dc + (long long)b * nc * gs.npts() : nullptr;
    const float M = shadow ? clk[desc[b].tree].anchor_M : 0.f;
    float umax = 0.f;
    for (int i = threadIdx.x; i < nint; i += blockDim.x) {
        const int ix = i % Bx, iy = (i / Bx) % By, iz = i / (Bx * By);
        double *pa = ab + ((long long)(iz + za) * ga.ny + (iy + ga.gb)) * ga.nx + (ix + ga.gb);
        if (!to_state) {
            cp[i] = *pa;
            continue;
        }
        const double v = cp[i];
        *pa = v;
        const df2 sv = df_split(v);
        umax = fmaxf(umax, fabsf(sv.hi));
        if (shadow) {
            const df2 w = anchor(sv, M);
            const float2 f = make_float2(w.hi, w.lo);
            db[((iz + zs) * gs.ny + (iy + gs.gb)) * gs.nx + (ix + gs.gb)] = f;
            if (push) {
                if (gs.nz > 1) push_ghosts<3, 1>(push, b, ix, iy, iz, Bx, By, Bz, gs, dc, gs.npts() * nc, &f);
                else push_ghosts<2, 1>(push, b, ix, iy, iz, Bx, By, Bz, gs, dc, gs.npts() * nc, &f);
            }
        }
    }
    if (to_state && clk) merge_umax(umax, clk, desc[b].tree);
}

// The upload direction of interior_xfer_kernel for 3-D 16^3 blocks with the
// double-float copy: one CTA per block, every thread moving all NV
// components of its points (the compact rows of the components are read
// side by side), the block's 27 push receivers staged in shared memory, one
// merge of the maximum per block. Values and writes are those of
// interior_xfer_kernel.
template <int NV>
__global__ void __launch_bounds__(256) interior_scatter_df_kernel(const int *__restrict__ slots,
                                                                  const double *__restrict__ compact, double *A,
                                                                  BufGeo ga, const BlockDesc *desc, TreeClock *clk,
                                                                  float2 *shadow, BufGeo gs, const int *push) {
    constexpr int BS = 16, NINT = BS * BS * BS;
    __shared__ int prow[27];
    const int b = slots[blockIdx.x];
    if (push && threadIdx.x < 27) prow[threadIdx.x] = push[b * 27 + threadIdx.x];
    __syncthreads();
    const double *cp = compact + (long long)blockIdx.x * NV * NINT;
    const long long na = ga.npts(), ns = gs.npts();
    double *ab = A + (long long)b * NV * na;
    float2 *db = shadow + (long long)b * NV * ns;
    const float M = clk[desc[b].tree].anchor_M;
    float umax = 0.f;
#pragma unroll 1
    for (int i = threadIdx.x; i < NINT; i += 256) {
        const int ix = i & (BS - 1), iy = (i >> 4) & (BS - 1), iz = i >> 8;
        double v[NV];
#pragma unroll
        for (int c = 0; c < NV; c++) v[c] = __ldcs(cp + c * NINT + i);
        const long long oa = ((long long)(iz + ga.gb) * ga.ny + (iy + ga.gb)) * ga.nx + (ix + ga.gb);
        const long long os = ((long long)(iz + gs.gb) * gs.ny + (iy + gs.gb)) * gs.nx + (ix + gs.gb);
        float2 f[NV];
#pragma unroll
        for (int c = 0; c < NV; c++) {
            ab[c * na + oa] = v[c];
            const df2 sv = df_split(v[c]);
            umax = fmaxf(umax, fabsf(sv.hi));
            const df2 w = anchor(sv, M);
            f[c] = make_float2(w.hi, w.lo);
            db[c * ns + os] = f[c];
        }
        if (push) push_ghosts_row<3, NV>(prow, ix, iy, iz, BS, BS, BS, gs, shadow, ns, f);
    }
    merge_umax(umax, clk, desc[b].tree);
}

__global__ void anchor_check_kernel(TreeClock *clk, const int *trees, int ntrees) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= ntrees) return;
    TreeClock &c = clk[trees[i]];
    const float M = anchor_constant(c.umax_f);
    c.reshadow = M != c.anchor_M;
    c.anchor_M = M;
}

// max |u| over the interiors of the listed blocks (all components) merged
// into the trees' running max: the quantum of a state that changed outside
// an RK step
__global__ void __launch_bounds__(256) umax_state_kernel(const int *__restrict__ slots, const double *A, BufGeo ga,
                                                         int nc, int Bx, int By, int Bz, const BlockDesc *desc,
                                                         TreeClock *clk) {
    const int b = slots[blockIdx.x], c = blockIdx.y;
    const int nint = Bx * By * Bz;
    const double *ab = A + ((long long)b * nc + c) * ga.npts();
    const int za = ga.nz > 1 ? ga.gb : 0;
    float umax = 0.f;
    for (int i = threadIdx.x; i < nint; i += blockDim.x) {
        const int ix = i % Bx, iy = (i / Bx) % By, iz = i / (Bx * By);
        umax = fmaxf(umax, fabsf(df_split(ab[((long long)(iz + za) * ga.ny + (iy + ga.gb)) * ga.nx + (ix + ga.gb)]).hi));
    }
    merge_umax(umax, clk, desc[b].tree);
}

__global__ void umax_reset_kernel(TreeClock *clk, const int *trees, int ntrees) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < ntrees) clk[trees[i]].umax_f = 0u;
}

__global__ void anchor_set_kernel(TreeClock *clk, const int *trees, int ntrees) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < ntrees) clk[trees[i]].anchor_M = anchor_constant(clk[trees[i]].umax_f);
}

// the anchoring constant of the listed trees from their state: the running
// max is reset, then (scan) rebuilt from A's interiors or (no scan) taken
// from what an interior upload merged since the reset
cudaError_t launch_umax_reset(TreeClock *clk, const int *trees, int ntrees, cudaStream_t s) {
    umax_reset_kernel<<<(ntrees + 127) / 128, 128, 0, s>>>(clk, trees, ntrees);
    return cudaGetLastError();
}

cudaError_t launch_anchor_from_state(const int *slots, int nblk, const double *A, BufGeo ga, int nc, int Bx, int By,
                                     int Bz, const BlockDesc *desc, TreeClock *clk, const int *trees, int ntrees,
                                     int scan, cudaStream_t s) {
    if (scan) {
        cudaError_t e = launch_umax_reset(clk, trees, ntrees, s);
        if (e != cudaSuccess) return e;
        if (nblk > 0) umax_state_kernel<<<dim3(nblk, nc), 256, 0, s>>>(slots, A, ga, nc, Bx, By, Bz, desc, clk);
    }
    anchor_set_kernel<<<(ntrees + 127) / 128, 128, 0, s>>>(clk, trees, ntrees);
    return cudaGetLastError();
}

cudaError_t launch_interior_xfer(const int *slots, int nblk, double *compact, double *A, BufGeo ga, int nc, int Bx,
                                 int By, int Bz, int to_state, const BlockDesc *desc, TreeClock *clk, cudaStream_t s,
                                 void *shadow, BufGeo gs, const int *push) {
    if (nblk <= 0) return cudaSuccess;
    if (shadow && (!to_state || !clk)) return cudaErrorInvalidValue;
    const bool b16 = Bx == 16 && By == 16 && (Bz == 1 || Bz == 16);
    if (shadow && nc == 4 && Bz == 16 && b16 && ga.nz > 1 && gs.nz > 1) {
        interior_scatter_df_kernel<4><<<(unsigned)nblk, 256, 0, s>>>(slots, compact, A, ga, desc, clk,
                                                                     reinterpret_cast<float2 *>(shadow), gs, push);
        return cudaGetLastError();
    }
    (b16 ? interior_xfer_kernel<16> : interior_xfer_kernel<0>)<<<dim3(nblk, nc), 256, 0, s>>>(
        slots, compact, A, ga, nc, Bx, By, Bz, to_state, desc, clk, reinterpret_cast<float2 *>(shadow), gs, push);
    return cudaGetLastError();
}

cudaError_t launch_anchor_check(TreeClock *clk, const int *trees, int ntrees, cudaStream_t s) {
    anchor_check_kernel<<<(ntrees + 127) / 128, 128, 0, s>>>(clk, trees, ntrees);
    return cudaGetLastError();
}

cudaError_t launch_shadow(const int *blk, int nblk, const double *src, BufGeo gs, void *dst, BufGeo gd, int nc,
                          int Bs0, int Bs1, int Bs2, const int *push, const BlockDesc *desc, const TreeClock *clk,
                          cudaStream_t s, int only_if_flagged, const int *cpos) {
    if (nblk <= 0) return cudaSuccess;
    shadow_kernel<<<dim3((unsigned)nblk, (unsigned)nc), 256, 0, s>>>(blk, src, gs, reinterpret_cast<float2 *>(dst), gd,
                                                                     nc, Bs0, Bs1, Bs2, push, desc, clk,
                                                                     only_if_flagged, cpos);
    return cudaGetLastError();
}

}  // namespace wg
