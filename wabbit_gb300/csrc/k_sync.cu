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
        for (int c = 0; c < nc; c++) {
            const double *sr = src + c * npts + si;
            double *dr = dst + c * npts + di;
            for (int ix = 0; ix < ex; ix++) dr[ix] = sr[step * ix];
        }
    }
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

// storage of a sync buffer element: FP64, or a double-float pair (hi, lo)
// held in the same 8 bytes (FP32-pipe path); predictions are always
// evaluated in FP64
template <bool DF>
__device__ __forceinline__ double load_el(const double *p) {
    if (!DF) return *p;
    const float2 v = *reinterpret_cast<const float2 *>(p);
    return (double)v.x + (double)v.y;
}

template <bool DF>
__device__ __forceinline__ void store_el(double *p, double v) {
    if (!DF) {
        *p = v;
        return;
    }
    const float h = __double2float_rn(v);
    *reinterpret_cast<float2 *>(p) = make_float2(h, __double2float_rn(v - (double)h));
}

template <bool DF>
__global__ void __launch_bounds__(256) predict_kernel(const Patch *__restrict__ patches, double *buf, BufGeo geo,
                                                      int nc, int order_idx, int ncoef) {
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
    double *C = sm;                       // coarse box
    double *X = C + ncp;                  // ex * ny * nz
    double *XY = X + ex * ny * nz;        // ex * ey * nz
    const long long npts = geo.npts();
    for (int c = 0; c < nc; c++) {
        const double *src = buf + ((long long)p.src * nc + c) * npts;
        double *dst = buf + ((long long)p.dst * nc + c) * npts;
        for (int i = threadIdx.x; i < ncp; i += blockDim.x) {
            const int x = i % cx, y = (i / cx) % cy, z = i / (cx * cy);
            C[i] = load_el<DF>(src + ((long long)(p.slo[2] + z) * geo.ny + (p.slo[1] + y)) * geo.nx + (p.slo[0] + x));
        }
        __syncthreads();
        // x pass on even rows / planes
        for (int i = threadIdx.x; i < ex * ny * nz; i += blockDim.x) {
            const int ix = i % ex, jy = (i / ex) % ny, kz = i / (ex * ny);
            const int fx = x0 + ix, cyy = (yw0 >> 1) + jy, czz = (zw0 >> 1) + kz;
            const double *row = C + ((long long)czz * cy + cyy) * cx;
            double v;
            if (!(fx & 1)) v = row[fx >> 1];
            else if (fx < h || fx > Fx - 1 - h) v = 0.0;
            else v = interp_line(cf, row, 1, (fx - h) >> 1, ncoef);
            X[i] = v;
        }
        __syncthreads();
        // y pass on the receiver rows, even planes
        for (int i = threadIdx.x; i < ex * ey * nz; i += blockDim.x) {
            const int ix = i % ex, j = (i / ex) % ey, kz = i / (ex * ey);
            const int fy = y0 + j;
            const double *col = X + (long long)kz * ny * ex + ix;     // stride ex along the row window
            double v;
            if (!(fy & 1)) v = col[(long long)((fy - yw0) >> 1) * ex];
            else if (fy < h || fy > Fy - 1 - h) v = 0.0;
            else v = interp_line(cf, col, ex, (fy - h - yw0) >> 1, ncoef);
            XY[i] = v;
        }
        __syncthreads();
        // z pass on the receiver box, write out
        for (int i = threadIdx.x; i < ex * ey * ez; i += blockDim.x) {
            const int ix = i % ex, j = (i / ex) % ey, k = i / (ex * ey);
            const int fz = z0 + k;
            const double *pl = XY + (long long)j * ex + ix;            // stride ex*ey along the plane window
            double v;
            if (!(fz & 1)) v = pl[(long long)((fz - zw0) >> 1) * ex * ey];
            else if (fz < h || fz > Fz - 1 - h) v = 0.0;
            else v = interp_line(cf, pl, ex * ey, (fz - h - zw0) >> 1, ncoef);
            store_el<DF>(dst + ((long long)(p.rlo[2] + k) * geo.ny + (p.rlo[1] + j)) * geo.nx + (p.rlo[0] + ix), v);
        }
        __syncthreads();
    }
}

cudaError_t sync_init() { return init_predictor(); }

cudaError_t launch_predict(const Patch *patches, int npatch, int max_smem_doubles, double *buf, BufGeo geo, int nc,
                           int order_predictor, cudaStream_t s) {
    if (npatch <= 0) return cudaSuccess;
    const size_t smem = sizeof(double) * (size_t)max_smem_doubles;
    static size_t attr = 0;
    if (smem > 48 * 1024 && smem > attr) {
        cudaError_t e = cudaFuncSetAttribute(predict_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        attr = smem;
    }
    predict_kernel<false><<<npatch, 256, smem, s>>>(patches, buf, geo, nc, order_predictor / 2 - 1, order_predictor);
    return cudaGetLastError();
}

cudaError_t launch_predict_df(const Patch *patches, int npatch, int max_smem_doubles, void *buf, BufGeo geo, int nc,
                              int order_predictor, cudaStream_t s) {
    if (npatch <= 0) return cudaSuccess;
    const size_t smem = sizeof(double) * (size_t)max_smem_doubles;
    static size_t attr = 0;
    if (smem > 48 * 1024 && smem > attr) {
        cudaError_t e = cudaFuncSetAttribute(predict_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        attr = smem;
    }
    predict_kernel<true><<<npatch, 256, smem, s>>>(patches, reinterpret_cast<double *>(buf), geo, nc,
                                                   order_predictor / 2 - 1, order_predictor);
    return cudaGetLastError();
}

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
