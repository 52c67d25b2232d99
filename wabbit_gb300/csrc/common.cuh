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
};

// Per-tree time state on the device.
struct TreeClock {
    double time;
    double dt;
    unsigned long long dt_min_bits;  // running min over blocks (positive double bits)
    int    diverged;
    int    pad;
};

// Per-block descriptor. k1, k2: first-derivative weights (2/3)/dx, (1/12)/dx;
// m1, m2, m0: viscous weights nu*(4/3)/dx^2, nu*(1/12)/dx^2 and
// nu*(-5/2)*sum 1/dx^2 (regrouped FD_4th_central stencils of the fast path).
struct BlockDesc {
    double dx[3];
    double k1[3], k2[3], m1[3], m2[3], m0;
    // the same weights as double-float pairs (hi, lo) for the FP32-pipe path
    float fk1[3][2], fk2[3][2], fm1[3][2], fm2[3][2], fm0[2];
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
cudaError_t probe_alu(double *fp64_tflops, double *fp32_tflops);
// constant-memory set-up; must run before any stream capture
cudaError_t sync_init();
cudaError_t wavelet_init();
cudaError_t launch_sync(const Patch *patches, int npatch, double *buf, BufGeo geo, int nc, int order_predictor,
                        cudaStream_t s);
// prediction patches only; max_smem_doubles = largest shared-memory need
// (coarse box + x window + x-y window) of a patch, in doubles
cudaError_t launch_predict(const Patch *patches, int npatch, int max_smem_doubles, double *buf, BufGeo geo, int nc,
                           int order_predictor, cudaStream_t s);
// RHS + RK stage (j = 1..4) over nblk blocks listed in blk
cudaError_t launch_acm_stage(int variant, int dim, int stage, const int *blk, int nblk, const BlockDesc *desc,
                             const TreeParams *tp, const TreeClock *clk, const double *in, BufGeo gin,
                             double *out, BufGeo gout, double *un, BufGeo gun, double *acc, const double *mask,
                             int Bs0, int Bs1, int Bs2, int nc, cudaStream_t s);
// double-float stage kernel (FP32-pipe stencils, FP64 RK state): in/out are
// float2 (hi, lo) buffers; stage 4 writes u_{n+1} to un (FP64) and its
// double-float copy to out
cudaError_t launch_acm_stage_df(int dim, int stage, int masked, const int *blk, int nblk, const BlockDesc *desc,
                                const TreeParams *tp, const TreeClock *clk, const void *in, BufGeo gin, void *out,
                                BufGeo gout, double *un, BufGeo gun, double *acc, const double *mask, int Bs0,
                                int Bs1, int Bs2, int nc, cudaStream_t s);
// double-float copy of the interiors of the listed blocks of an FP64 buffer
cudaError_t launch_shadow(const int *blk, int nblk, const double *src, BufGeo gs, void *dst, BufGeo gd, int nc,
                          int Bs0, int Bs1, int Bs2, cudaStream_t s);
cudaError_t launch_predict_df(const Patch *patches, int npatch, int max_smem_doubles, void *buf, BufGeo geo, int nc,
                              int order_predictor, cudaStream_t s);
cudaError_t launch_rhs_only(int variant, int dim, const int *blk, int nblk, const BlockDesc *desc,
                            const TreeParams *tp, const double *in, BufGeo gin, double *rhs, const double *mask,
                            int Bs0, int Bs1, int Bs2, int nc, cudaStream_t s);
cudaError_t launch_dt(int dim, const int *blk, int nblk, const BlockDesc *desc, const TreeParams *tp,
                      TreeClock *clk, const double *u, BufGeo geo, int Bs0, int Bs1, int Bs2, int ntrees,
                      const int *trees, cudaStream_t s);
cudaError_t launch_clock_advance(TreeClock *clk, const int *trees, int ntrees, cudaStream_t s);
cudaError_t launch_interior_copy(const int *slots, int nblk, double *full, BufGeo geo, double *compact, int nc,
                                 int Bx, int By, int Bz, int to_full, cudaStream_t s);
cudaError_t launch_fwt_flags(int dim, const int *blk, int nblk, const double *u, BufGeo geo, int Bs0, int Bs1,
                             int Bs2, int nc, int wavelet_x, int wavelet_y, const double *eps_use,
                             const int *tsvc, int *flags, double *details, cudaStream_t s);
// allocation-free variant (static device scratch, contiguous blocks 0..nblk-1)
int noalloc_max_blocks();
cudaError_t launch_fwt_flags_noalloc(int dim, int nblk, const double *u, BufGeo geo, int Bs0, int Bs1, int Bs2,
                                     int nc, int wavelet_x, int wavelet_y, const double *eps_host,
                                     const int *tsvc_host, int *flags, double *details, cudaStream_t s);
cudaError_t launch_refine(int dim, const int *parent, int nparent, const int *child_base, const double *u,
                          BufGeo geo, int Bs0, int Bs1, int Bs2, int nc, int order_predictor, cudaStream_t s);

}  // namespace wg
