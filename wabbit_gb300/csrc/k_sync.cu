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
// bit-identical to the reference's.
#include "common.cuh"
#include "predict.cuh"

namespace wg {

__global__ void __launch_bounds__(128) sync_kernel(const Patch *__restrict__ patches, int npatch, double *buf,
                                                   BufGeo geo, int nc, int order_idx, int ncoef) {
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (warp >= npatch) return;
    const Patch p = patches[warp];
    const int ex = p.rhi[0] - p.rlo[0] + 1, ey = p.rhi[1] - p.rlo[1] + 1, ez = p.rhi[2] - p.rlo[2] + 1;
    const int n = ex * ey * ez;
    const long long npts = geo.npts();
    double *dst = buf + (long long)p.dst * nc * npts;
    const double *src = buf + (long long)p.src * nc * npts;
    for (int q = lane; q < n; q += 32) {
        const int ix = q % ex, iy = (q / ex) % ey, iz = q / (ex * ey);
        const long long di = ((long long)(p.rlo[2] + iz) * geo.ny + (p.rlo[1] + iy)) * geo.nx + (p.rlo[0] + ix);
        if (p.op == 0) {
            const long long si = ((long long)(p.slo[2] + iz) * geo.ny + (p.slo[1] + iy)) * geo.nx + (p.slo[0] + ix);
            for (int c = 0; c < nc; c++) dst[c * npts + di] = src[c * npts + si];
        } else if (p.op == 1) {
            const int sx = p.slo[0] + 2 * (p.blo[0] + ix);
            const int sy = p.slo[1] + 2 * (p.blo[1] + iy);
            const int sz = p.slo[2] + 2 * (p.blo[2] + iz);
            const long long si = ((long long)sz * geo.ny + sy) * geo.nx + sx;
            for (int c = 0; c < nc; c++) dst[c * npts + di] = src[c * npts + si];
        } else {
            PredCtx pc;
            pc.nx = geo.nx;
            pc.ny = geo.ny;
            pc.sx = p.slo[0];
            pc.sy = p.slo[1];
            pc.sz = p.slo[2];
            pc.Fx = 2 * (p.shi[0] - p.slo[0] + 1) - 1;
            pc.Fy = 2 * (p.shi[1] - p.slo[1] + 1) - 1;
            pc.Fz = 2 * (p.shi[2] - p.slo[2] + 1) - 1;
            pc.nc = ncoef;
            pc.c = c_pred[order_idx];
            const int fx = p.blo[0] + ix, fy = p.blo[1] + iy, fz = p.blo[2] + iz;
            for (int c = 0; c < nc; c++) {
                pc.src = src + c * npts;
                dst[c * npts + di] = pred_xyz(pc, fx, fy, fz);
            }
        }
    }
}

cudaError_t sync_init() { return init_predictor(); }

cudaError_t launch_sync(const Patch *patches, int npatch, double *buf, BufGeo geo, int nc, int order_predictor,
                        cudaStream_t s) {
    if (npatch <= 0) return cudaSuccess;
    cudaError_t e = init_predictor();
    if (e != cudaSuccess) return e;
    const int oi = order_predictor / 2 - 1;
    const int threads = 128;
    const int blocks = (npatch * 32 + threads - 1) / threads;
    sync_kernel<<<blocks, threads, 0, s>>>(patches, npatch, buf, geo, nc, oi, order_predictor);
    return cudaGetLastError();
}

}  // namespace wg
