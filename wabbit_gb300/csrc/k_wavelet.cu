// k_wavelet.cu -- wavelet kernels: coarsening indicator (one-level FWT +
// detail threshold) and block refinement.
//
// FWT: waveletDecomposition_optimized_block
// (LIB/WAVELETS/wavelet_decomposition_reconstruction.f90:23-389): separable
// x -> y -> z pass in spaghetti order, the low-pass filter HD on odd (1-based)
// points, the high-pass filter GD on even points; for CDFX0 the scaling
// coefficients are copied. Threshold: threshold_block
// (LIB/INDICATORS/threshold_block.f90) with the Linfty renorm of
// wavelet_renorm_block (module_wavelets.f90:1848-1960): the detail of a
// component is max|WC| over the interior with the SC positions zeroed, and a
// block may coarsen (-1) iff every detail <= eps_use. Every filter sum uses
// explicit round-to-nearest operations in the reference's term order, so the
// details -- and therefore the grid decisions -- are bit-identical.
//
// Refinement: refineBlock (LIB/MESH/refinementExecute.f90:4-116): the whole
// parent block (ghosts included) is predicted to the fine grid and each of the
// 2^d daughters takes its (Bs+2g)^d window.
#include "common.cuh"
#include "predict.cuh"

namespace wg {

__constant__ double c_hd[32];
__constant__ double c_gd[32];
__constant__ int c_flt[4];   // hd_lo, hd_n, gd_lo, gd_n

static int g_flt_key = -1;   // wavelet whose filters sit in constant memory

struct FwtArgs {
    const int *blk;
    const double *u;
    BufGeo geo;
    int Bs[3];
    int nc, lazy, fmax;
    const double *eps_use;   // nc entries
    const int *tsvc;         // threshold_state_vector_component, nc entries
    int *flags;
    double *details;
};

__device__ __forceinline__ double filt(const double *c, int lo, int n, const double *line, int stride, int at) {
    double s = 0.0;
    bool first = true;
    for (int k = 0; k < n; k++) {
        const double w = c[k];
        const int m = lo + k;
        if (w == 0.0 && m != 0) continue;
        const double v = __dmul_rn(line[(long long)(at + m) * stride], w);
        s = first ? v : __dadd_rn(s, v);
        first = false;
    }
    return s;
}

// one CTA per (block, component); shared array holds the x-interior columns of
// all rows/planes the later passes read
template <int DIM>
__global__ void __launch_bounds__(256) fwt_detail_kernel(FwtArgs a, double *detail_scratch) {
    extern __shared__ double sm[];
    const int bi = blockIdx.x / a.nc, c = blockIdx.x % a.nc;
    const int b = a.blk[bi];
    const int g = a.geo.gb;
    const int Bx = a.Bs[0], By = a.Bs[1], Bz = DIM == 3 ? a.Bs[2] : 1;
    const int f = a.fmax;
    const int y0 = g - f, ny = By + 2 * f;                 // rows [g-f, g+By+f)
    const int z0 = DIM == 3 ? g - f : 0, nz = DIM == 3 ? Bz + 2 * f : 1;
    const long long np = a.geo.npts();
    const double *u = a.u + ((long long)b * a.nc + c) * np;
    const int hd_lo = c_flt[0], hd_n = c_flt[1], gd_lo = c_flt[2], gd_n = c_flt[3];
    // sm[(z*ny + y)*Bx + x], x interior, y in [y0,y0+ny), z in [z0,z0+nz)
    // X pass straight from global memory
    for (int r = threadIdx.x; r < ny * nz; r += blockDim.x) {
        const int yy = r % ny, zz = r / ny;
        const double *line = u + ((long long)(z0 + zz) * a.geo.ny + (y0 + yy)) * a.geo.nx;
        double *o = sm + (long long)r * Bx;
        for (int ix = 0; ix < Bx; ix++) {
            const int at = g + ix;
            if ((ix & 1) == 0) o[ix] = a.lazy ? line[at] : filt(c_hd, hd_lo, hd_n, line, 1, at);
            else o[ix] = filt(c_gd, gd_lo, gd_n, line, 1, at);
        }
    }
    __syncthreads();
    // Y pass, x-interior columns, all planes, in place through registers
    double tmp[64];
    for (int r = threadIdx.x; r < Bx * nz; r += blockDim.x) {
        const int ix = r % Bx, zz = r / Bx;
        double *col = sm + (long long)zz * ny * Bx + ix;   // stride Bx along y
        for (int iy = 0; iy < By; iy++) {
            const int at = f + iy;
            if ((iy & 1) == 0) tmp[iy] = a.lazy ? col[(long long)at * Bx] : filt(c_hd, hd_lo, hd_n, col, Bx, at);
            else tmp[iy] = filt(c_gd, gd_lo, gd_n, col, Bx, at);
        }
        for (int iy = 0; iy < By; iy++) col[(long long)(f + iy) * Bx] = tmp[iy];
    }
    __syncthreads();
    if (DIM == 3) {
        for (int r = threadIdx.x; r < Bx * By; r += blockDim.x) {
            const int ix = r % Bx, iy = r / Bx;
            double *col = sm + (long long)(f + iy) * Bx + ix;   // stride ny*Bx along z
            const int st = ny * Bx;
            for (int iz = 0; iz < Bz; iz++) {
                const int at = f + iz;
                if ((iz & 1) == 0) tmp[iz] = a.lazy ? col[(long long)at * st] : filt(c_hd, hd_lo, hd_n, col, st, at);
                else tmp[iz] = filt(c_gd, gd_lo, gd_n, col, st, at);
            }
            for (int iz = 0; iz < Bz; iz++) col[(long long)(f + iz) * st] = tmp[iz];
        }
        __syncthreads();
    }
    // max |WC| over the interior, SC positions (all indices even) excluded
    double m = 0.0;
    const int nint = Bx * By * Bz;
    for (int q = threadIdx.x; q < nint; q += blockDim.x) {
        const int ix = q % Bx, iy = (q / Bx) % By, iz = q / (Bx * By);
        if ((ix & 1) == 0 && (iy & 1) == 0 && (iz & 1) == 0) continue;
        const double v = fabs(sm[((long long)(DIM == 3 ? f + iz : 0) * ny + (f + iy)) * Bx + ix]);
        m = fmax(m, v);
    }
    __shared__ double red[256];
    red[threadIdx.x] = m;
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) red[threadIdx.x] = fmax(red[threadIdx.x], red[threadIdx.x + w]);
        __syncthreads();
    }
    if (threadIdx.x == 0) detail_scratch[(long long)bi * a.nc + c] = red[0];
}

__global__ void flag_kernel(FwtArgs a, const double *detail_scratch, int nblk) {
    const int bi = blockIdx.x * blockDim.x + threadIdx.x;
    if (bi >= nblk) return;
    double det[8];
    const double *d = detail_scratch + (long long)bi * a.nc;
    int maxg = 0;
    for (int c = 0; c < a.nc; c++) { det[c] = -1.0; maxg = max(maxg, a.tsvc[c]); }
    for (int l = 2; l <= maxg; l++) {
        double m = 0.0;
        for (int c = 0; c < a.nc; c++) if (a.tsvc[c] == l) m = fmax(m, d[c]);
        for (int c = 0; c < a.nc; c++) if (a.tsvc[c] == l) det[c] = m;
    }
    bool all = true;
    for (int c = 0; c < a.nc; c++) {
        if (a.tsvc[c] == 1) det[c] = d[c];
        if (a.tsvc[c] == 0) det[c] = 0.0;
        if (!(det[c] <= a.eps_use[c])) all = false;
        if (a.details) a.details[(long long)bi * a.nc + c] = det[c];
    }
    a.flags[bi] = all ? -1 : 0;
}

cudaError_t launch_fwt_flags(int dim, const int *blk, int nblk, const double *u, BufGeo geo, int Bs0, int Bs1,
                             int Bs2, int nc, int wavelet_x, int wavelet_y, const double *eps_use, const int *tsvc,
                             int *flags, double *details, cudaStream_t s) {
    if (nblk <= 0) return cudaSuccess;
    WaveletInfo w;
    char name[8] = {'C', 'D', 'F', (char)('0' + wavelet_x), (char)('0' + wavelet_y), 0};
    if (!make_wavelet(name, w)) return cudaErrorInvalidValue;
    const int key = wavelet_x * 10 + wavelet_y;
    if (g_flt_key != key) {
        double hd[32] = {}, gd[32] = {};
        for (size_t i = 0; i < w.HD.size(); i++) hd[i] = w.HD[i];
        for (size_t i = 0; i < w.GD.size(); i++) gd[i] = w.GD[i];
        int flt[4] = {w.hd_lo, (int)w.HD.size(), w.gd_lo, (int)w.GD.size()};
        cudaError_t e = cudaMemcpyToSymbolAsync(c_hd, hd, sizeof(hd), 0, cudaMemcpyHostToDevice, s);
        if (e == cudaSuccess) e = cudaMemcpyToSymbolAsync(c_gd, gd, sizeof(gd), 0, cudaMemcpyHostToDevice, s);
        if (e == cudaSuccess) e = cudaMemcpyToSymbolAsync(c_flt, flt, sizeof(flt), 0, cudaMemcpyHostToDevice, s);
        if (e != cudaSuccess) return e;
        g_flt_key = key;
    }
    FwtArgs a;
    a.blk = blk;
    a.u = u;
    a.geo = geo;
    a.Bs[0] = Bs0;
    a.Bs[1] = Bs1;
    a.Bs[2] = Bs2;
    a.nc = nc;
    a.lazy = w.lifted ? 0 : 1;
    const int hd_hi = w.hd_lo + (int)w.HD.size() - 1, gd_hi = w.gd_lo + (int)w.GD.size() - 1;
    a.fmax = std::max(std::max(w.hd_lo, hd_hi), std::max(w.gd_lo, gd_hi));
    a.eps_use = eps_use;
    a.tsvc = tsvc;
    a.flags = flags;
    a.details = details;
    if (a.fmax > geo.gb) return cudaErrorInvalidValue;   // filter needs more ghost nodes
    const int ny = Bs1 + 2 * a.fmax, nz = dim == 3 ? Bs2 + 2 * a.fmax : 1;
    const size_t smem = sizeof(double) * (size_t)Bs0 * ny * nz;
    double *scratch = nullptr;
    cudaError_t e = cudaMallocAsync(&scratch, sizeof(double) * (size_t)nblk * nc, s);
    if (e != cudaSuccess) return e;
    if (dim == 2) {
        cudaFuncSetAttribute(fwt_detail_kernel<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        fwt_detail_kernel<2><<<nblk * nc, 256, smem, s>>>(a, scratch);
    } else {
        cudaFuncSetAttribute(fwt_detail_kernel<3>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        fwt_detail_kernel<3><<<nblk * nc, 256, smem, s>>>(a, scratch);
    }
    flag_kernel<<<(nblk + 127) / 128, 128, 0, s>>>(a, scratch, nblk);
    e = cudaGetLastError();
    cudaFreeAsync(scratch, s);
    return e;
}

cudaError_t wavelet_init() { return init_predictor(); }

// ---------------------------------------------------------------------------
// Allocation-free coarsening indicator. Callers that must not allocate device
// memory during a call (a host code that manages its own memory pool, runs
// under a memory budget enforced outside CUDA, or links the library into a
// runtime whose allocator it may not call) get a variant of
// launch_fwt_flags whose per-block detail scratch, block list, thresholds
// and component groups live in file-scope static device arrays. Every
// device that loads the library holds these arrays (~1.2 MB) until exit.
// All calls share them: two calls whose kernels overlap on the GPU race.
// ---------------------------------------------------------------------------
#define WG_NOALLOC_MAX_BLOCKS 16384
#define WG_NOALLOC_MAX_COMP 8
static __device__ __align__(256) double g_na_detail[WG_NOALLOC_MAX_BLOCKS * WG_NOALLOC_MAX_COMP];
static __device__ __align__(256) int g_na_blocks[WG_NOALLOC_MAX_BLOCKS];
static __device__ __align__(256) double g_na_eps[WG_NOALLOC_MAX_COMP];
static __device__ __align__(256) int g_na_tsvc[WG_NOALLOC_MAX_COMP];

struct NoAllocPtrs {
    double *detail;
    int *blocks;
    double *eps;
    int *tsvc;
    bool ready;
};
static NoAllocPtrs g_na_ptrs[64];

__global__ void noalloc_iota_kernel(int *b, int n) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) b[i] = i;
}

// once per device, with that device current: resolve the device addresses of
// the static arrays (a host-side name of a __device__ array is not a device
// address) and fill the identity block list
static cudaError_t noalloc_setup(int dev, cudaStream_t s) {
    if (dev < 0 || dev >= 64) return cudaErrorInvalidDevice;
    NoAllocPtrs &p = g_na_ptrs[dev];
    if (p.ready) return cudaSuccess;
    cudaError_t e = cudaGetSymbolAddress((void **)&p.detail, g_na_detail);
    if (e == cudaSuccess) e = cudaGetSymbolAddress((void **)&p.blocks, g_na_blocks);
    if (e == cudaSuccess) e = cudaGetSymbolAddress((void **)&p.eps, g_na_eps);
    if (e == cudaSuccess) e = cudaGetSymbolAddress((void **)&p.tsvc, g_na_tsvc);
    if (e != cudaSuccess) return e;
    e = init_predictor();
    if (e != cudaSuccess) return e;
    noalloc_iota_kernel<<<64, 256, 0, s>>>(p.blocks, WG_NOALLOC_MAX_BLOCKS);
    e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e == cudaSuccess) p.ready = true;
    return e;
}

int noalloc_max_blocks() { return WG_NOALLOC_MAX_BLOCKS; }

cudaError_t launch_fwt_flags_noalloc(int dim, int nblk, const double *u, BufGeo geo, int Bs0, int Bs1, int Bs2,
                                     int nc, int wavelet_x, int wavelet_y, const double *eps_host,
                                     const int *tsvc_host, int *flags, double *details, cudaStream_t s) {
    if (nblk <= 0) return cudaSuccess;
    if (nblk > WG_NOALLOC_MAX_BLOCKS || nc > WG_NOALLOC_MAX_COMP) return cudaErrorInvalidValue;
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    e = noalloc_setup(dev, s);
    if (e != cudaSuccess) return e;
    const NoAllocPtrs &P = g_na_ptrs[dev];
    WaveletInfo w;
    char name[8] = {'C', 'D', 'F', (char)('0' + wavelet_x), (char)('0' + wavelet_y), 0};
    if (!make_wavelet(name, w)) return cudaErrorInvalidValue;
    // filters, thresholds and groups for this call (no allocation: copies
    // into constant memory and into the static arrays)
    double hd[32] = {}, gd[32] = {};
    for (size_t i = 0; i < w.HD.size(); i++) hd[i] = w.HD[i];
    for (size_t i = 0; i < w.GD.size(); i++) gd[i] = w.GD[i];
    int flt[4] = {w.hd_lo, (int)w.HD.size(), w.gd_lo, (int)w.GD.size()};
    e = cudaMemcpyToSymbolAsync(c_hd, hd, sizeof(hd), 0, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaMemcpyToSymbolAsync(c_gd, gd, sizeof(gd), 0, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaMemcpyToSymbolAsync(c_flt, flt, sizeof(flt), 0, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(P.eps, eps_host, sizeof(double) * nc, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(P.tsvc, tsvc_host, sizeof(int) * nc, cudaMemcpyHostToDevice, s);
    if (e != cudaSuccess) return e;
    g_flt_key = -1;   // the shared filter constants now hold this call's wavelet
    FwtArgs a;
    a.blk = P.blocks;
    a.u = u;
    a.geo = geo;
    a.Bs[0] = Bs0;
    a.Bs[1] = Bs1;
    a.Bs[2] = Bs2;
    a.nc = nc;
    a.lazy = w.lifted ? 0 : 1;
    const int hd_hi = w.hd_lo + (int)w.HD.size() - 1, gd_hi = w.gd_lo + (int)w.GD.size() - 1;
    a.fmax = std::max(std::max(w.hd_lo, hd_hi), std::max(w.gd_lo, gd_hi));
    a.eps_use = P.eps;
    a.tsvc = P.tsvc;
    a.flags = flags;
    a.details = details;
    if (a.fmax > geo.gb) return cudaErrorInvalidValue;
    const int ny = Bs1 + 2 * a.fmax, nz = dim == 3 ? Bs2 + 2 * a.fmax : 1;
    const size_t smem = sizeof(double) * (size_t)Bs0 * ny * nz;
    if (dim == 2) {
        e = cudaFuncSetAttribute(fwt_detail_kernel<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e == cudaSuccess) fwt_detail_kernel<2><<<nblk * nc, 256, smem, s>>>(a, P.detail);
    } else {
        e = cudaFuncSetAttribute(fwt_detail_kernel<3>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e == cudaSuccess) fwt_detail_kernel<3><<<nblk * nc, 256, smem, s>>>(a, P.detail);
    }
    if (e != cudaSuccess) return e;
    flag_kernel<<<(nblk + 127) / 128, 128, 0, s>>>(a, P.detail, nblk);
    return cudaGetLastError();
}

// refineBlock: daughter k of parent p is written to slot child_base[p] + k
__global__ void __launch_bounds__(256) refine_kernel(const int *parent, const int *child_base, const double *u,
                                                     BufGeo geo, int dim, int Bs0, int Bs1, int Bs2, int nc,
                                                     int order_idx, int ncoef, long long npts_per) {
    const int nd = 1 << dim;
    const long long np = geo.npts();
    const long long total = (long long)nd * np;
    const int pi = blockIdx.y;
    const int pb = parent[pi];
    const double *src = u + (long long)pb * nc * np;
    PredCtx pc;
    pc.nx = geo.nx;
    pc.ny = geo.ny;
    pc.sx = pc.sy = pc.sz = 0;
    pc.Fx = 2 * geo.nx - 1;
    pc.Fy = 2 * geo.ny - 1;
    pc.Fz = dim == 3 ? 2 * geo.nz - 1 : 1;
    pc.nc = ncoef;
    pc.c = c_pred[order_idx];
    const int g = geo.gb;
    for (long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x; q < total; q += (long long)gridDim.x * blockDim.x) {
        const int k = (int)(q / np);
        const long long r = q % np;
        const int ix = (int)(r % geo.nx), iy = (int)((r / geo.nx) % geo.ny), iz = (int)(r / ((long long)geo.nx * geo.ny));
        const int fx = g + Bs0 * ((k / 2) % 2) + ix;
        const int fy = g + Bs1 * (k % 2) + iy;
        const int fz = dim == 3 ? g + Bs2 * (k / 4) + iz : 0;
        double *dst = const_cast<double *>(u) + ((long long)(child_base[pi] + k) * nc) * np + r;
        for (int c = 0; c < nc; c++) {
            pc.src = src + c * np;
            dst[c * np] = pred_xyz(pc, fx, fy, fz);
        }
    }
}

cudaError_t launch_refine(int dim, const int *parent, int nparent, const int *child_base, const double *u,
                          BufGeo geo, int Bs0, int Bs1, int Bs2, int nc, int order_predictor, cudaStream_t s) {
    if (nparent <= 0) return cudaSuccess;
    cudaError_t e = init_predictor();
    if (e != cudaSuccess) return e;
    dim3 grid(64, nparent);
    refine_kernel<<<grid, 256, 0, s>>>(parent, child_base, u, geo, dim, Bs0, Bs1, Bs2, nc, order_predictor / 2 - 1,
                                       order_predictor, 0);
    return cudaGetLastError();
}

}  // namespace wg
