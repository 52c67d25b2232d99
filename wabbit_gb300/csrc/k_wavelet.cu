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
// IWT: waveletReconstruction_optimized_block
// (wavelet_decomposition_reconstruction.f90:426-840), the same separable
// passes with the reconstruction filters HR, GR in the reference's term order
// (see iwt_kernel). WC thresholding: wc_threshold_tree (LIB/MESH/
// adapt_tree.f90:1091-1180).
//
// Refinement: refineBlock (LIB/MESH/refinementExecute.f90:4-116): the whole
// parent block (ghosts included) is predicted to the fine grid and each of the
// 2^d daughters takes its (Bs+2g)^d window.
#include <mutex>
#include <type_traits>

#include "common.cuh"
#include "exact.cuh"
#include "predict.cuh"

namespace wg {

// The filters, thresholds and component groups of a launch travel in its
// parameters (read through the constant bank like __constant__ data): no
// state is shared between launches, so calls on different streams, host
// threads or devices with different wavelets cannot see each other's taps.
struct Filters {            // analysis filters HD, GD
    double hd[32], gd[32];
    int hd_lo, hd_n, gd_lo, gd_n;
};
struct RFilters {           // reconstruction filters HR, GR
    double hr[32], gr[32];
    int hr_lo, hr_n, gr_lo, gr_n;
};

static Filters make_filters(const WaveletInfo &w) {
    Filters f{};
    for (size_t i = 0; i < w.HD.size() && i < 32; i++) f.hd[i] = w.HD[i];
    for (size_t i = 0; i < w.GD.size() && i < 32; i++) f.gd[i] = w.GD[i];
    f.hd_lo = w.hd_lo;
    f.hd_n = (int)w.HD.size();
    f.gd_lo = w.gd_lo;
    f.gd_n = (int)w.GD.size();
    return f;
}

static RFilters make_rfilters(const WaveletInfo &w) {
    RFilters f{};
    for (size_t i = 0; i < w.HR.size() && i < 32; i++) f.hr[i] = w.HR[i];
    for (size_t i = 0; i < w.GR.size() && i < 32; i++) f.gr[i] = w.GR[i];
    f.hr_lo = w.hr_lo;
    f.hr_n = (int)w.HR.size();
    f.gr_lo = w.gr_lo;
    f.gr_n = (int)w.GR.size();
    return f;
}

struct FwtArgs {
    const int *blk;
    const double *u;
    BufGeo geo;
    int Bs[3];
    int nc, lazy, fmax;
    Filters F;
    double eps[8];           // per-component threshold (eps * norm)
    int tsvc[8];             // threshold_state_vector_component
    int *flags;
    double *details;
};

// FwtArgs of a wavelet, with its thresholds and groups (host arrays of nc)
static bool make_fwt_args(const WaveletInfo &w, int nc, const double *eps_host, const int *tsvc_host, FwtArgs &a) {
    if (nc > 8 || w.HD.size() > 32 || w.GD.size() > 32) return false;
    a = FwtArgs{};
    a.F = make_filters(w);
    a.nc = nc;
    a.lazy = w.lifted ? 0 : 1;
    const int hd_hi = w.hd_lo + (int)w.HD.size() - 1, gd_hi = w.gd_lo + (int)w.GD.size() - 1;
    a.fmax = std::max(std::max(w.hd_lo, hd_hi), std::max(w.gd_lo, gd_hi));
    for (int c = 0; c < nc; c++) {
        a.eps[c] = eps_host ? eps_host[c] : 0.0;
        a.tsvc[c] = tsvc_host ? tsvc_host[c] : 1;
    }
    return true;
}

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
// all rows/planes the later passes read. STORE: write the decomposed interior
// (spaghetti order) to out instead of reducing the details; out may be the
// input itself (every read of the CTA's block component precedes its writes).
template <int DIM, bool STORE = false>
__global__ void __launch_bounds__(256) fwt_detail_kernel(const __grid_constant__ FwtArgs a, double *detail_scratch,
                                                         double *out = nullptr) {
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
    const int hd_lo = a.F.hd_lo, hd_n = a.F.hd_n, gd_lo = a.F.gd_lo, gd_n = a.F.gd_n;
    const double *c_hd = a.F.hd, *c_gd = a.F.gd;
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
    const int nint = Bx * By * Bz;
    if (STORE) {
        double *o = out + ((long long)b * a.nc + c) * np;
        for (int q = threadIdx.x; q < nint; q += blockDim.x) {
            const int ix = q % Bx, iy = (q / Bx) % By, iz = q / (Bx * By);
            o[((long long)(DIM == 3 ? g + iz : 0) * a.geo.ny + (g + iy)) * a.geo.nx + (g + ix)] =
                sm[((long long)(DIM == 3 ? f + iz : 0) * ny + (f + iy)) * Bx + ix];
        }
        return;
    }
    // max |WC| over the interior, SC positions (all indices even) excluded
    double m = 0.0;
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

// details from data that is already decomposed (spaghetti order): max |WC|
// over the interior, SC positions excluded; one CTA per (block, component)
template <int DIM>
__global__ void __launch_bounds__(256) wd_detail_kernel(const __grid_constant__ FwtArgs a, double *detail_scratch) {
    const int bi = blockIdx.x / a.nc, c = blockIdx.x % a.nc;
    const int b = a.blk[bi];
    const int g = a.geo.gb;
    const int Bx = a.Bs[0], By = a.Bs[1], Bz = DIM == 3 ? a.Bs[2] : 1;
    const double *u = a.u + ((long long)b * a.nc + c) * a.geo.npts();
    double m = 0.0;
    const int nint = Bx * By * Bz;
    for (int q = threadIdx.x; q < nint; q += blockDim.x) {
        const int ix = q % Bx, iy = (q / Bx) % By, iz = q / (Bx * By);
        if ((ix & 1) == 0 && (iy & 1) == 0 && (iz & 1) == 0) continue;
        m = fmax(m, fabs(u[((long long)(DIM == 3 ? g + iz : 0) * a.geo.ny + (g + iy)) * a.geo.nx + (g + ix)]));
    }
    for (int w = 16; w; w >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, w));
    __shared__ double red[8];
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = m;
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int w = 1; w < (int)(blockDim.x >> 5); w++) m = fmax(m, red[w]);
        m = fmax(m, red[0]);
        detail_scratch[(long long)bi * a.nc + c] = m;
    }
}

__global__ void flag_kernel(const __grid_constant__ FwtArgs a, const double *detail_scratch, int nblk) {
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
        if (!(det[c] <= a.eps[c])) all = false;
        if (a.details) a.details[(long long)bi * a.nc + c] = det[c];
    }
    a.flags[bi] = all ? -1 : 0;
}

static cudaError_t launch_tpo(int mode, int dim, const int *blk, int nblk, double *u, BufGeo geo, int Bs0, int Bs1,
                              int Bs2, int nc, const WaveletInfo &w, int f, double *scratch, cudaStream_t s);

cudaError_t launch_fwt_flags(int dim, const int *blk, int nblk, const double *u, BufGeo geo, int Bs0, int Bs1,
                             int Bs2, int nc, int wavelet_x, int wavelet_y, const double *eps_use, const int *tsvc,
                             int *flags, double *details, cudaStream_t s, int input_is_wd) {
    if (nblk <= 0) return cudaSuccess;
    if (!blk || !eps_use || !tsvc || !flags) return cudaErrorInvalidValue;
    WaveletInfo w;
    char name[8] = {'C', 'D', 'F', (char)('0' + wavelet_x), (char)('0' + wavelet_y), 0};
    if (!make_wavelet(name, w)) return cudaErrorInvalidValue;
    FwtArgs a;
    if (!make_fwt_args(w, nc, eps_use, tsvc, a)) return cudaErrorInvalidValue;
    a.blk = blk;
    a.u = u;
    a.geo = geo;
    a.Bs[0] = Bs0;
    a.Bs[1] = Bs1;
    a.Bs[2] = Bs2;
    a.flags = flags;
    a.details = details;
    if (a.fmax > geo.gb) return cudaErrorInvalidValue;   // filter needs more ghost nodes
    const int ny = Bs1 + 2 * a.fmax, nz = dim == 3 ? Bs2 + 2 * a.fmax : 1;
    const size_t smem = sizeof(double) * (size_t)Bs0 * ny * nz;
    double *scratch = nullptr;
    cudaError_t e = cudaMallocAsync(&scratch, sizeof(double) * (size_t)nblk * nc, s);
    if (e != cudaSuccess) return e;
    cudaError_t et = cudaErrorNotSupported;
    if (!input_is_wd)
        et = launch_tpo(0, dim, blk, nblk, const_cast<double *>(u), geo, Bs0, Bs1, Bs2, nc, w, a.fmax, scratch, s);
    if (et != cudaSuccess && et != cudaErrorNotSupported) {
        cudaFreeAsync(scratch, s);
        return et;
    }
    if (et == cudaErrorNotSupported) cudaGetLastError();
    if (input_is_wd) {
        if (dim == 2) wd_detail_kernel<2><<<nblk * nc, 256, 0, s>>>(a, scratch);
        else wd_detail_kernel<3><<<nblk * nc, 256, 0, s>>>(a, scratch);
    } else if (et == cudaSuccess) {
        // details computed by the thread-per-output kernel
    } else if (dim == 2) {
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

// Reconstruct one line in place: src(i) for i in [at0 - F, at0 + n + F) holds
// spaghetti data (SC at at0, at0+2, ...); the n interior results go to dst
// with stride ds. Lazy (unlifted) wavelets keep the SCs and add the odd HR taps
// to each WC (value first); lifted wavelets: SC + odd GR taps at an SC,
// odd HR taps over the SCs, then GR(0) WC, then the other even GR taps at a WC.
__device__ __forceinline__ void iwt_line(const RFilters &R, const double *src, long long ss, int at0, int n, bool lazy,
                                         double *dst, long long ds) {
    const int hr_lo = R.hr_lo, hr_n = R.hr_n, gr_lo = R.gr_lo, gr_n = R.gr_n;
    const double *c_hr = R.hr, *c_gr = R.gr;
    for (int k = 0; k < n; k += 2) {
        const int s0 = at0 + k, w0 = s0 + 1;
        double sc, wc;
        if (lazy) {
            sc = src[s0 * ss];
            wc = src[w0 * ss];
            for (int t = 0; t < hr_n; t++) {
                const int m = hr_lo + t;
                if (!(m & 1) || c_hr[t] == 0.0) continue;
                wc = __dadd_rn(wc, __dmul_rn(src[(w0 + m) * ss], c_hr[t]));
            }
        } else {
            sc = src[s0 * ss];
            for (int t = 0; t < gr_n; t++) {
                const int m = gr_lo + t;
                if (!(m & 1) || c_gr[t] == 0.0) continue;
                sc = __dadd_rn(sc, __dmul_rn(src[(s0 + m) * ss], c_gr[t]));
            }
            bool first = true;
            wc = 0.0;
            for (int t = 0; t < hr_n; t++) {
                const int m = hr_lo + t;
                if (!(m & 1) || c_hr[t] == 0.0) continue;
                const double v = __dmul_rn(src[(w0 + m) * ss], c_hr[t]);
                wc = first ? v : __dadd_rn(wc, v);
                first = false;
            }
            wc = __dadd_rn(wc, __dmul_rn(src[w0 * ss], c_gr[-gr_lo]));
            for (int t = 0; t < gr_n; t++) {
                const int m = gr_lo + t;
                if ((m & 1) || m == 0 || c_gr[t] == 0.0) continue;
                wc = __dadd_rn(wc, __dmul_rn(src[(w0 + m) * ss], c_gr[t]));
            }
        }
        dst[k * ds] = sc;
        dst[(k + 1) * ds] = wc;
    }
}

// One-level IWT of every (block, component), in place on the interior; the
// ghost nodes must hold the neighbours' spaghetti data (synchronised). Shared
// memory holds the x-interior columns of the rows/planes the y and z passes
// read (F = max HR/GR half-width around the interior).
template <int DIM>
__global__ void __launch_bounds__(256) iwt_kernel(const __grid_constant__ RFilters R, const int *blk, double *u,
                                                  BufGeo geo, int Bx, int By, int Bz,
                                                  int nc, int lazy, int F) {
    extern __shared__ double sm[];
    const int bi = blockIdx.x / nc, c = blockIdx.x % nc;
    const int b = blk[bi];
    const int g = geo.gb;
    if (DIM == 2) Bz = 1;
    const int y0 = g - F, ny = By + 2 * F;
    const int z0 = DIM == 3 ? g - F : 0, nz = DIM == 3 ? Bz + 2 * F : 1;
    const long long np = geo.npts();
    double *ub = u + ((long long)b * nc + c) * np;
    // x pass from global memory on every row/plane of the extended window
    for (int r = threadIdx.x; r < ny * nz; r += blockDim.x) {
        const int yy = r % ny, zz = r / ny;
        const double *line = ub + ((long long)(z0 + zz) * geo.ny + (y0 + yy)) * geo.nx;
        iwt_line(R, line, 1, g, Bx, lazy, sm + (long long)r * Bx, 1);
    }
    __syncthreads();
    double tmp[64];
    for (int r = threadIdx.x; r < Bx * nz; r += blockDim.x) {
        const int ix = r % Bx, zz = r / Bx;
        double *col = sm + (long long)zz * ny * Bx + ix;     // stride Bx along y
        iwt_line(R, col, Bx, F, By, lazy, tmp, 1);
        for (int iy = 0; iy < By; iy++) col[(long long)(F + iy) * Bx] = tmp[iy];
    }
    __syncthreads();
    if (DIM == 3) {
        for (int r = threadIdx.x; r < Bx * By; r += blockDim.x) {
            const int ix = r % Bx, iy = r / Bx;
            double *col = sm + (long long)(F + iy) * Bx + ix;   // stride ny*Bx along z
            iwt_line(R, col, (long long)ny * Bx, F, Bz, lazy, tmp, 1);
            for (int iz = 0; iz < Bz; iz++) col[(long long)(F + iz) * ny * Bx] = tmp[iz];
        }
        __syncthreads();
    }
    const int nint = Bx * By * Bz;
    for (int q = threadIdx.x; q < nint; q += blockDim.x) {
        const int ix = q % Bx, iy = (q / Bx) % By, iz = q / (Bx * By);
        ub[((long long)(DIM == 3 ? g + iz : 0) * geo.ny + (g + iy)) * geo.nx + (g + ix)] =
            sm[((long long)(DIM == 3 ? F + iz : 0) * ny + (F + iy)) * Bx + ix];
    }
}

struct WcThresh {
    double t[8];
    int tsvc[8];
};

// wc_threshold_tree on spaghetti data, one thread per interior point of a
// block: components with threshold_state_vector_component 0 or >= 2 are
// zeroed where |WC| < thresh (1 is skipped, as in the reference), then every
// group l >= 2 where the group's Euclidean norm is below its largest threshold
template <int DIM>
__global__ void wc_threshold_kernel(const int *blk, int nblk, double *u, BufGeo geo, int Bx, int By, int Bz, int nc,
                                    WcThresh th) {
    const int nint = Bx * By * (DIM == 3 ? Bz : 1);
    const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= (long long)nblk * nint) return;
    const int bi = (int)(q / nint), p = (int)(q % nint);
    const int ix = p % Bx, iy = (p / Bx) % By, iz = DIM == 3 ? p / (Bx * By) : 0;
    if ((ix & 1) == 0 && (iy & 1) == 0 && (iz & 1) == 0) return;   // scaling coefficient
    const long long np = geo.npts();
    double *ub = u + (long long)blk[bi] * nc * np +
                 ((long long)(DIM == 3 ? geo.gb + iz : 0) * geo.ny + (geo.gb + iy)) * geo.nx + (geo.gb + ix);
    double w[8];
    for (int c = 0; c < nc; c++) w[c] = ub[c * np];
    int maxg = 0;
    for (int c = 0; c < nc; c++) {
        maxg = max(maxg, th.tsvc[c]);
        if (th.tsvc[c] != 1 && fabs(w[c]) < th.t[c]) ub[c * np] = 0.0;
    }
    for (int l = 2; l <= maxg; l++) {
        double s = 0.0, tmax = -1e300;
        bool first = true;
        for (int c = 0; c < nc; c++) {
            if (th.tsvc[c] != l) continue;
            const double v = __dmul_rn(w[c], w[c]);
            s = first ? v : __dadd_rn(s, v);
            first = false;
            tmax = fmax(tmax, th.t[c]);
        }
        if (__dsqrt_rn(s) < tmax)
            for (int c = 0; c < nc; c++)
                if (th.tsvc[c] == l) ub[c * np] = 0.0;
    }
}

// ---------------------------------------------------------------------------
// Thread-per-output form of the one-level FWT and IWT (blocks with
// Bx*By*nz_ext <= 8192): 512 threads per (block, component); the x pass goes
// from global memory into shared memory on the rows/planes the later passes
// read, the y pass keeps its results in registers across a barrier and writes
// them back in place, the z pass writes the state (FWT: every read of the
// block component happened in the x pass) or reduces the details. Filter taps
// are compacted on the host into (offset, value) lists in the reference's
// term order.
// ---------------------------------------------------------------------------
struct Taps {
    int n[5];              // 0 HD (non-zero or centre), 1 GD, 2 HR odd, 3 GR odd, 4 GR even without 0
    int off[5][16];
    double val[5][16];
    int kind[5][16], sh[5][16], mul[5][16];   // tap kinds for the integer-pipe products (exact.cuh)
    long long sgn[5][16];         // sign bit of each tap
    double gr0;            // GR(0)
    int gr0_kind, gr0_sh, gr0_mul;
    long long gr0_sgn;
    int lazy;
};

constexpr int kTpoThreads = 512;
constexpr int kTpoMaxPerThread = 16;

// sum_t src[(at + off_t) * st] * val_t in order, the first term not added to 0
__device__ __forceinline__ double tap_sum(const Taps &c_taps, int f, const double *src, long long st, int at) {
    const int n = c_taps.n[f];
    double s = __dmul_rn(src[(at + c_taps.off[f][0]) * st], c_taps.val[f][0]);
    for (int t = 1; t < n; t++) s = __dadd_rn(s, __dmul_rn(src[(at + c_taps.off[f][t]) * st], c_taps.val[f][t]));
    return s;
}

// Compile-time tap kinds of CDF4,4 (classify_tap of the lists make_taps
// builds: HD -6..6 without +-5, GD -3..3 without +-2, HR odd, GR odd, GR even
// without 0); the host checks them against the loaded taps before the
// specialised kernel runs.
struct Cdf44Taps {
    __host__ __device__ static constexpr int nt(int f) { return f == 0 ? 11 : f == 1 ? 5 : f == 4 ? 6 : 4; }
    __host__ __device__ static constexpr int kind(int f, int t) {
        return f == 0 ? ((t == 0 || t == 2 || t == 8 || t == 10) ? 1 : 3)
             : f == 1 ? ((t == 0 || t == 4) ? 1 : t == 2 ? 2 : 3)
             : f == 4 ? ((t == 0 || t == 5) ? 1 : 3)
             : ((t == 0 || t == 3) ? 1 : 3);
    }
};

// product with tap t of list F, the kind known at compile time: every kind
// but 0 is formed on the integer pipe
template <class K, int F>
__device__ __forceinline__ double ktap_mul(const Taps &c_taps, double x, int t, bool &bad) {
    if (K::kind(F, t) == 2) return x;
    if (K::kind(F, t) == 1) return pow2_mul(x, c_taps.sh[F][t], c_taps.sgn[F][t], bad);
    if (K::kind(F, t) == 3) return short_mul(x, c_taps.mul[F][t], c_taps.sh[F][t], c_taps.sgn[F][t], bad);
    return __dmul_rn(x, c_taps.val[F][t]);
}

// the same sum with the kinds of K known at compile time: the FP64 pipe
// only adds
template <class K, int F>
__device__ __forceinline__ double ktap_sum(const Taps &c_taps, const double *src, long long st, int at, bool &bad) {
    double s = 0.0;
#pragma unroll
    for (int t = 0; t < K::nt(F); t++) {
        const double p = ktap_mul<K, F>(c_taps, src[(at + c_taps.off[F][t]) * st], t, bad);
        s = t == 0 ? p : __dadd_rn(s, p);
    }
    return s;
}

// FWT output at interior offset p (position at of the line)
__device__ __forceinline__ double fwt_point(const Taps &c_taps, const double *src, long long st, int at, int p) {
    if ((p & 1) == 0) return c_taps.lazy ? src[at * st] : tap_sum(c_taps, 0, src, st, at);
    return tap_sum(c_taps, 1, src, st, at);
}

// IWT output at interior offset p (position at of the line)
__device__ __forceinline__ double iwt_point(const Taps &c_taps, const double *src, long long st, int at, int p) {
    if (c_taps.lazy) {
        double v = src[at * st];
        if (p & 1)
            for (int t = 0; t < c_taps.n[2]; t++)
                v = __dadd_rn(v, __dmul_rn(src[(at + c_taps.off[2][t]) * st], c_taps.val[2][t]));
        return v;
    }
    if ((p & 1) == 0) {
        double v = src[at * st];
        for (int t = 0; t < c_taps.n[3]; t++)
            v = __dadd_rn(v, __dmul_rn(src[(at + c_taps.off[3][t]) * st], c_taps.val[3][t]));
        return v;
    }
    double v = tap_sum(c_taps, 2, src, st, at);
    v = __dadd_rn(v, __dmul_rn(src[at * st], c_taps.gr0));
    for (int t = 0; t < c_taps.n[4]; t++)
        v = __dadd_rn(v, __dmul_rn(src[(at + c_taps.off[4][t]) * st], c_taps.val[4][t]));
    return v;
}

// fwt_point / iwt_point with compile-time tap kinds (lifted wavelets),
// without the fallback: bad is set where an integer-pipe product left the
// exact range, and the caller recomputes those outputs with fwt_point /
// iwt_point
template <class K>
__device__ __forceinline__ double fwt_point_k(const Taps &c_taps, const double *src, long long st, int at, int p,
                                              bool &bad) {
    return (p & 1) == 0 ? ktap_sum<K, 0>(c_taps, src, st, at, bad) : ktap_sum<K, 1>(c_taps, src, st, at, bad);
}

template <class K>
__device__ __forceinline__ double iwt_point_k(const Taps &c_taps, const double *src, long long st, int at, int p,
                                              bool &bad) {
    double v;
    if ((p & 1) == 0) {
        // the reference adds the odd GR taps one by one to the SC
        v = src[at * st];
#pragma unroll
        for (int t = 0; t < K::nt(3); t++) {
            v = __dadd_rn(v, ktap_mul<K, 3>(c_taps, src[(at + c_taps.off[3][t]) * st], t, bad));
        }
    } else {
        v = ktap_sum<K, 2>(c_taps, src, st, at, bad);
        v = __dadd_rn(v, tap_mul(src[at * st], c_taps.gr0, c_taps.gr0_kind, c_taps.gr0_sh, c_taps.gr0_mul,
                                 c_taps.gr0_sgn, bad));
#pragma unroll
        for (int t = 0; t < K::nt(4); t++)
            v = __dadd_rn(v, ktap_mul<K, 4>(c_taps, src[(at + c_taps.off[4][t]) * st], t, bad));
    }
    return v;
}

// Zero, or a biased exponent in [16, 2030]: the product of such a value with
// a CDF4,4 tap (2^-9 <= |c| <= 1) is zero or a normal number, so a pass
// whose inputs all lie in this band needs no range check per product.
__device__ __forceinline__ bool in_tap_band(double x) {
    const unsigned long long a = (unsigned long long)dbits(x) & 0x7fffffffffffffffULL;
    return (a == 0ULL) | ((unsigned)((int)(a >> 52) - 16) <= 2014u);
}

// MODE 0: details (max |WC|) into scratch; 1: FWT stored in place; 2: IWT
// stored in place. f: half-width of the extended window.
struct GenericTaps {};

template <int DIM, int MODE, class K = GenericTaps>
__global__ void __launch_bounds__(kTpoThreads, 2) tpo_kernel(const __grid_constant__ Taps c_taps, const int *blk,
                                                             double *u, BufGeo geo, int Bx, int By, int Bz, int nc,
                                                             int f, double *detail_scratch) {
    extern __shared__ double sm[];
    const int bi = blockIdx.x / nc, c = blockIdx.x % nc;
    const int b = blk[bi];
    const int g = geo.gb;
    if (DIM == 2) Bz = 1;
    const int ny = By + 2 * f, nz = DIM == 3 ? Bz + 2 * f : 1;
    const int y0 = g - f, z0 = DIM == 3 ? g - f : 0;
    const long long np = geo.npts();
    double *ub = u + ((long long)b * nc + c) * np;
    // slow: the reference's FP64 multiplies; fast: compile-time tap kinds
    // (products on the integer pipe), bad marks outputs to redo
    auto slow = [&](const double *src, long long st, int at, int p) {
        return MODE == 2 ? iwt_point(c_taps, src, st, at, p) : fwt_point(c_taps, src, st, at, p);
    };
    auto fast = [&](const double *src, long long st, int at, int p, bool &bad) {
        if constexpr (std::is_same<K, GenericTaps>::value)
            return slow(src, st, at, p);
        else
            return MODE == 2 ? iwt_point_k<K>(c_taps, src, st, at, p, bad) : fwt_point_k<K>(c_taps, src, st, at, p, bad);
    };
    auto point = slow;
    constexpr bool kTyped = !std::is_same<K, GenericTaps>::value;
    // inputs of every pass in the tap band (block-wide): the products skip
    // their range checks (the compiler drops the unread flags)
    bool band = false;
    if constexpr (kTyped) {
        bool ok = true;
        for (long long i = threadIdx.x; i < np; i += kTpoThreads) ok &= in_tap_band(ub[i]);
        band = __syncthreads_and(ok) != 0;
    }
    bool ok_next = true;   // this thread's outputs of the pass in the band
    // x pass, two independent outputs per step
    const int nx_out = Bx * ny * nz;
    auto xrow = [&](int o) { return ub + ((long long)(z0 + (o / Bx) / ny) * geo.ny + (y0 + (o / Bx) % ny)) * geo.nx; };
    for (int o = threadIdx.x; o < nx_out; o += 2 * kTpoThreads) {
        const int o2 = o + kTpoThreads;
        const bool two = o2 < nx_out;
        double v1, v2;
        if (band) {
            bool unread = false;
            v1 = fast(xrow(o), 1, g + o % Bx, o % Bx, unread);
            v2 = two ? fast(xrow(o2), 1, g + o2 % Bx, o2 % Bx, unread) : 0.0;
        } else {
            bool bad = false;
            v1 = fast(xrow(o), 1, g + o % Bx, o % Bx, bad);
            v2 = two ? fast(xrow(o2), 1, g + o2 % Bx, o2 % Bx, bad) : 0.0;
            if (bad) {
                v1 = slow(xrow(o), 1, g + o % Bx, o % Bx);
                if (two) v2 = slow(xrow(o2), 1, g + o2 % Bx, o2 % Bx);
            }
        }
        if constexpr (kTyped) ok_next &= in_tap_band(v1) & in_tap_band(v2);
        sm[o] = v1;
        if (two) sm[o2] = v2;
    }
    if constexpr (kTyped) band = __syncthreads_and(ok_next) != 0;
    else __syncthreads();
    if (MODE == 3) {
        // the x pass results outside the interior rows/planes stay in the
        // block, as the reference's FWT leaves them in u_d
        for (int o = threadIdx.x; o < nx_out; o += kTpoThreads) {
            const int ix = o % Bx, r = o / Bx;
            const int yy = r % ny, zz = r / ny;
            const bool inner = yy >= f && yy < f + By && (DIM == 2 || (zz >= f && zz < f + Bz));
            if (!inner) ub[((long long)(z0 + zz) * geo.ny + (y0 + yy)) * geo.nx + g + ix] = sm[o];
        }
    }
    // y pass on the interior rows of every plane of the window
    double res[kTpoMaxPerThread];
    const int ny_out = Bx * By * nz;
    if (band) {
        bool unread = false;
#pragma unroll
        for (int k = 0; k < kTpoMaxPerThread; k++) {
            const int o = threadIdx.x + k * kTpoThreads;
            if (o < ny_out) {
                const int ix = o % Bx, iy = (o / Bx) % By, zz = o / (Bx * By);
                res[k] = fast(sm + (long long)zz * ny * Bx + ix, Bx, f + iy, iy, unread);
            }
        }
    } else {
        bool bad = false;
#pragma unroll
        for (int k = 0; k < kTpoMaxPerThread; k++) {
            const int o = threadIdx.x + k * kTpoThreads;
            if (o < ny_out) {
                const int ix = o % Bx, iy = (o / Bx) % By, zz = o / (Bx * By);
                res[k] = fast(sm + (long long)zz * ny * Bx + ix, Bx, f + iy, iy, bad);
            }
        }
        if (bad) {
#pragma unroll
            for (int k = 0; k < kTpoMaxPerThread; k++) {
                const int o = threadIdx.x + k * kTpoThreads;
                if (o < ny_out) {
                    const int ix = o % Bx, iy = (o / Bx) % By, zz = o / (Bx * By);
                    res[k] = point(sm + (long long)zz * ny * Bx + ix, Bx, f + iy, iy);
                }
            }
        }
    }
    double m = 0.0;
    if (DIM == 2) {
        // the y pass results are final
#pragma unroll
        for (int k = 0; k < kTpoMaxPerThread; k++) {
            const int o = threadIdx.x + k * kTpoThreads;
            if (o >= ny_out) continue;
            const int ix = o % Bx, iy = o / Bx;
            if (MODE == 0) {
                if ((ix & 1) || (iy & 1)) m = fmax(m, fabs(res[k]));
            } else {
                ub[(long long)(g + iy) * geo.nx + (g + ix)] = res[k];
            }
        }
    } else {
        __syncthreads();
        ok_next = true;
#pragma unroll
        for (int k = 0; k < kTpoMaxPerThread; k++) {
            const int o = threadIdx.x + k * kTpoThreads;
            if (o >= ny_out) continue;
            const int ix = o % Bx, iy = (o / Bx) % By, zz = o / (Bx * By);
            sm[((long long)zz * ny + (f + iy)) * Bx + ix] = res[k];
            if (MODE == 3 && (zz < f || zz >= f + Bz))
                ub[((long long)(z0 + zz) * geo.ny + (g + iy)) * geo.nx + (g + ix)] = res[k];
            if constexpr (kTyped) ok_next &= in_tap_band(res[k]);
        }
        // the z pass reads only these y pass results
        if constexpr (kTyped) band = __syncthreads_and(ok_next) != 0;
        else __syncthreads();
        const int nint = Bx * By * Bz;
        auto zcol = [&](int o) { return sm + (long long)(f + (o / Bx) % By) * Bx + o % Bx; };
        auto put = [&](int o, double v) {
            const int ix = o % Bx, iy = (o / Bx) % By, iz = o / (Bx * By);
            if (MODE == 0) {
                if ((ix & 1) || (iy & 1) || (iz & 1)) m = fmax(m, fabs(v));
            } else {
                ub[((long long)(g + iz) * geo.ny + (g + iy)) * geo.nx + (g + ix)] = v;
            }
        };
        for (int o = threadIdx.x; o < nint; o += 2 * kTpoThreads) {
            const int o2 = o + kTpoThreads;
            const bool two = o2 < nint;
            const long long st = (long long)ny * Bx;
            double v1, v2;
            if (band) {
                bool unread = false;
                v1 = fast(zcol(o), st, f + o / (Bx * By), o / (Bx * By), unread);
                v2 = two ? fast(zcol(o2), st, f + o2 / (Bx * By), o2 / (Bx * By), unread) : 0.0;
            } else {
                bool bad = false;
                v1 = fast(zcol(o), st, f + o / (Bx * By), o / (Bx * By), bad);
                v2 = two ? fast(zcol(o2), st, f + o2 / (Bx * By), o2 / (Bx * By), bad) : 0.0;
                if (bad) {
                    v1 = slow(zcol(o), st, f + o / (Bx * By), o / (Bx * By));
                    if (two) v2 = slow(zcol(o2), st, f + o2 / (Bx * By), o2 / (Bx * By));
                }
            }
            put(o, v1);
            if (two) put(o2, v2);
        }
    }
    if (MODE == 0) {
        for (int w = 16; w; w >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, w));
        __shared__ double red[kTpoThreads / 32];
        if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = m;
        __syncthreads();
        if (threadIdx.x == 0) {
            for (int w = 0; w < kTpoThreads / 32; w++) m = fmax(m, red[w]);
            detail_scratch[(long long)bi * nc + c] = m;
        }
    }
}

// the compacted tap lists of a wavelet; cdf44: they have the kinds of the
// CDF4,4-specialised kernels
static bool make_taps(const WaveletInfo &w, Taps &t, bool &cdf44) {
    t = Taps{};
    auto add = [&](int f, int off, double v) {
        if (t.n[f] >= 16) return false;
        t.off[f][t.n[f]] = off;
        t.val[f][t.n[f]] = v;
        classify_tap(v, t.kind[f][t.n[f]], t.sh[f][t.n[f]], t.mul[f][t.n[f]]);
        t.sgn[f][t.n[f]] = v < 0.0 ? (long long)0x8000000000000000ULL : 0LL;
        t.n[f]++;
        return true;
    };
    bool ok = true;
    for (size_t i = 0; i < w.HD.size(); i++) {
        const int m = w.hd_lo + (int)i;
        if (w.HD[i] != 0.0 || m == 0) ok &= add(0, m, w.HD[i]);
    }
    for (size_t i = 0; i < w.GD.size(); i++) {
        const int m = w.gd_lo + (int)i;
        if (w.GD[i] != 0.0 || m == 0) ok &= add(1, m, w.GD[i]);
    }
    for (size_t i = 0; i < w.HR.size(); i++) {
        const int m = w.hr_lo + (int)i;
        if ((m & 1) && w.HR[i] != 0.0) ok &= add(2, m, w.HR[i]);
    }
    for (size_t i = 0; i < w.GR.size(); i++) {
        const int m = w.gr_lo + (int)i;
        if (m == 0) {
            t.gr0 = w.GR[i];
            classify_tap(t.gr0, t.gr0_kind, t.gr0_sh, t.gr0_mul);
            t.gr0_sgn = t.gr0 < 0.0 ? (long long)0x8000000000000000ULL : 0LL;
        }
        else if ((m & 1) && w.GR[i] != 0.0) ok &= add(3, m, w.GR[i]);
        else if (!(m & 1) && w.GR[i] != 0.0) ok &= add(4, m, w.GR[i]);
    }
    t.lazy = w.lifted ? 0 : 1;
    if (!ok || t.n[0] == 0 || t.n[1] == 0) return false;
    // the compile-time kinds of the CDF4,4 kernels must describe these taps
    cdf44 = !t.lazy;
    for (int f = 0; f < 5 && cdf44; f++) {
        if (t.n[f] != Cdf44Taps::nt(f)) cdf44 = false;
        for (int k = 0; k < t.n[f] && cdf44; k++)
            if (t.kind[f][k] != Cdf44Taps::kind(f, k)) cdf44 = false;
    }
    return true;
}

// launch the thread-per-output kernel if the block fits its limits; returns
// cudaErrorNotSupported otherwise (the caller then uses the column kernels)
static cudaError_t launch_tpo(int mode, int dim, const int *blk, int nblk, double *u, BufGeo geo, int Bs0, int Bs1,
                              int Bs2, int nc, const WaveletInfo &w, int f, double *scratch, cudaStream_t s) {
    const int ny = Bs1 + 2 * f, nz = dim == 3 ? Bs2 + 2 * f : 1;
    if ((long long)Bs0 * Bs1 * nz > (long long)kTpoThreads * kTpoMaxPerThread) return cudaErrorNotSupported;
    const size_t smem = sizeof(double) * (size_t)Bs0 * ny * nz;
    if (smem > 110 * 1024) return cudaErrorNotSupported;
    Taps taps;
    bool cdf44 = false;
    if (!make_taps(w, taps, cdf44)) return cudaErrorInvalidValue;
    const int bz = dim == 3 ? Bs2 : 1;
    auto go = [&](auto kern) -> cudaError_t {
        cudaError_t e2 = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e2 != cudaSuccess) return e2;
        kern<<<nblk * nc, kTpoThreads, smem, s>>>(taps, blk, u, geo, Bs0, Bs1, bz, nc, f, scratch);
        return cudaGetLastError();
    };
    if (dim == 2) {
        if (mode == 0) return go(tpo_kernel<2, 0>);
        if (cdf44) {
            if (mode == 1) return go(tpo_kernel<2, 1, Cdf44Taps>);
            if (mode == 3) return go(tpo_kernel<2, 3, Cdf44Taps>);
            return go(tpo_kernel<2, 2, Cdf44Taps>);
        }
        if (mode == 1) return go(tpo_kernel<2, 1>);
        if (mode == 3) return go(tpo_kernel<2, 3>);
        return go(tpo_kernel<2, 2>);
    }
    if (mode == 0) return go(tpo_kernel<3, 0>);
    if (cdf44) {
        if (mode == 1) return go(tpo_kernel<3, 1, Cdf44Taps>);
        if (mode == 3) return go(tpo_kernel<3, 3, Cdf44Taps>);
        return go(tpo_kernel<3, 2, Cdf44Taps>);
    }
    if (mode == 1) return go(tpo_kernel<3, 1>);
    if (mode == 3) return go(tpo_kernel<3, 3>);
    return go(tpo_kernel<3, 2>);
}

cudaError_t launch_wavelet_decompose(int dim, const int *blk, int nblk, double *u, BufGeo geo, int Bs0, int Bs1,
                                     int Bs2, int nc, int wavelet_x, int wavelet_y, cudaStream_t s) {
    if (nblk <= 0) return cudaSuccess;
    WaveletInfo w;
    char name[8] = {'C', 'D', 'F', (char)('0' + wavelet_x), (char)('0' + wavelet_y), 0};
    if (!make_wavelet(name, w)) return cudaErrorInvalidValue;
    FwtArgs a;
    if (!make_fwt_args(w, nc, nullptr, nullptr, a)) return cudaErrorInvalidValue;
    a.blk = blk;
    a.u = u;
    a.geo = geo;
    a.Bs[0] = Bs0;
    a.Bs[1] = Bs1;
    a.Bs[2] = Bs2;
    if (a.fmax > geo.gb) return cudaErrorInvalidValue;
    cudaError_t e = launch_tpo(1, dim, blk, nblk, u, geo, Bs0, Bs1, Bs2, nc, w, a.fmax, nullptr, s);
    if (e != cudaErrorNotSupported) return e;
    cudaGetLastError();
    const int ny = Bs1 + 2 * a.fmax, nz = dim == 3 ? Bs2 + 2 * a.fmax : 1;
    const size_t smem = sizeof(double) * (size_t)Bs0 * ny * nz;
    if (dim == 2) {
        cudaFuncSetAttribute(fwt_detail_kernel<2, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        fwt_detail_kernel<2, true><<<nblk * nc, 256, smem, s>>>(a, nullptr, u);
    } else {
        cudaFuncSetAttribute(fwt_detail_kernel<3, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        fwt_detail_kernel<3, true><<<nblk * nc, 256, smem, s>>>(a, nullptr, u);
    }
    return cudaGetLastError();
}

// FWT of whole blocks in the layout the reference's
// waveletDecomposition_optimized_block leaves in u_d: interior in spaghetti
// order, x-pass results on the ghost rows/planes of the filter window,
// y-pass results on the ghost planes (3-D)
cudaError_t launch_wavelet_decompose_window(int dim, const int *blk, int nblk, double *u, BufGeo geo, int Bs0, int Bs1,
                                            int Bs2, int nc, int wavelet_x, int wavelet_y, cudaStream_t s) {
    if (nblk <= 0) return cudaSuccess;
    if (!blk) return cudaErrorInvalidValue;
    WaveletInfo w;
    char name[8] = {'C', 'D', 'F', (char)('0' + wavelet_x), (char)('0' + wavelet_y), 0};
    if (!make_wavelet(name, w)) return cudaErrorInvalidValue;
    const int hd_hi = w.hd_lo + (int)w.HD.size() - 1, gd_hi = w.gd_lo + (int)w.GD.size() - 1;
    const int fmax = std::max(std::max(w.hd_lo, hd_hi), std::max(w.gd_lo, gd_hi));
    if (fmax > geo.gb) return cudaErrorInvalidValue;
    return launch_tpo(3, dim, blk, nblk, u, geo, Bs0, Bs1, Bs2, nc, w, fmax, nullptr, s);
}

cudaError_t launch_wavelet_reconstruct(int dim, const int *blk, int nblk, double *u, BufGeo geo, int Bs0, int Bs1,
                                       int Bs2, int nc, int wavelet_x, int wavelet_y, cudaStream_t s) {
    if (nblk <= 0) return cudaSuccess;
    if (!blk) return cudaErrorInvalidValue;
    WaveletInfo w;
    char name[8] = {'C', 'D', 'F', (char)('0' + wavelet_x), (char)('0' + wavelet_y), 0};
    if (!make_wavelet(name, w)) return cudaErrorInvalidValue;
    if (w.HR.size() > 32 || w.GR.size() > 32) return cudaErrorInvalidValue;
    const RFilters R = make_rfilters(w);
    const int hr_hi = w.hr_lo + (int)w.HR.size() - 1, gr_hi = w.gr_lo + (int)w.GR.size() - 1;
    const int F = std::max(std::max(w.hr_lo, hr_hi), std::max(w.gr_lo, gr_hi));
    // the x pass reads up to F+1 points beyond an interior WC position
    if (F + 1 > geo.gb + 1 || Bs0 > 64 || Bs1 > 64 || Bs2 > 64) return cudaErrorInvalidValue;
    {
        cudaError_t e = launch_tpo(2, dim, blk, nblk, u, geo, Bs0, Bs1, Bs2, nc, w, F, nullptr, s);
        if (e != cudaErrorNotSupported) return e;
        cudaGetLastError();
    }
    const int ny = Bs1 + 2 * F, nz = dim == 3 ? Bs2 + 2 * F : 1;
    const size_t smem = sizeof(double) * (size_t)Bs0 * ny * nz;
    if (dim == 2) {
        cudaFuncSetAttribute(iwt_kernel<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        iwt_kernel<2><<<nblk * nc, 256, smem, s>>>(R, blk, u, geo, Bs0, Bs1, 1, nc, w.lifted ? 0 : 1, F);
    } else {
        cudaFuncSetAttribute(iwt_kernel<3>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        iwt_kernel<3><<<nblk * nc, 256, smem, s>>>(R, blk, u, geo, Bs0, Bs1, Bs2, nc, w.lifted ? 0 : 1, F);
    }
    return cudaGetLastError();
}

cudaError_t launch_wc_threshold(int dim, const int *blk, int nblk, double *u, BufGeo geo, int Bs0, int Bs1, int Bs2,
                                int nc, const double *thresh, const int *tsvc, cudaStream_t s) {
    if (nblk <= 0) return cudaSuccess;
    if (nc > 8) return cudaErrorInvalidValue;
    WcThresh th{};
    for (int c = 0; c < nc; c++) {
        th.t[c] = thresh[c];
        th.tsvc[c] = tsvc[c];
    }
    const long long n = (long long)nblk * Bs0 * Bs1 * (dim == 3 ? Bs2 : 1);
    const unsigned grid = (unsigned)((n + 255) / 256);
    if (dim == 2) wc_threshold_kernel<2><<<grid, 256, 0, s>>>(blk, nblk, u, geo, Bs0, Bs1, Bs2, nc, th);
    else wc_threshold_kernel<3><<<grid, 256, 0, s>>>(blk, nblk, u, geo, Bs0, Bs1, Bs2, nc, th);
    return cudaGetLastError();
}

cudaError_t wavelet_init() { return cudaSuccess; }

// ---------------------------------------------------------------------------
// Allocation-free coarsening indicator. Callers that must not allocate device
// memory during a call (a host code that manages its own memory pool, runs
// under a memory budget enforced outside CUDA, or links the library into a
// runtime whose allocator it may not call) get a variant of
// launch_fwt_flags whose per-block detail scratch and block list live in
// file-scope static device arrays; filters, thresholds and component groups
// travel in the launch parameters. Every device that loads the library
// holds these arrays (~0.6 MB) until exit. All calls share them: two calls
// whose kernels overlap on the GPU race.
// ---------------------------------------------------------------------------
#define WG_NOALLOC_MAX_BLOCKS 16384
#define WG_NOALLOC_MAX_COMP 8
static __device__ __align__(256) double g_na_detail[WG_NOALLOC_MAX_BLOCKS * WG_NOALLOC_MAX_COMP];
static __device__ __align__(256) int g_na_blocks[WG_NOALLOC_MAX_BLOCKS];

struct NoAllocPtrs {
    double *detail = nullptr;
    int *blocks = nullptr;
    bool ready = false;
};
static NoAllocPtrs g_na_ptrs[64];
static std::mutex g_na_mutex;

__global__ void noalloc_iota_kernel(int *b, int n) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) b[i] = i;
}

// once per device, with that device current: resolve the device addresses of
// the static arrays (a host-side name of a __device__ array is not a device
// address) and fill the identity block list
static cudaError_t noalloc_setup(int dev, cudaStream_t s, NoAllocPtrs &out) {
    if (dev < 0 || dev >= 64) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lk(g_na_mutex);
    NoAllocPtrs &p = g_na_ptrs[dev];
    if (!p.ready) {
        NoAllocPtrs q;
        cudaError_t e = cudaGetSymbolAddress((void **)&q.detail, g_na_detail);
        if (e == cudaSuccess) e = cudaGetSymbolAddress((void **)&q.blocks, g_na_blocks);
        if (e != cudaSuccess) return e;
        noalloc_iota_kernel<<<64, 256, 0, s>>>(q.blocks, WG_NOALLOC_MAX_BLOCKS);
        e = cudaGetLastError();
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) return e;
        q.ready = true;
        p = q;
    }
    out = p;
    return cudaSuccess;
}

int noalloc_max_blocks() { return WG_NOALLOC_MAX_BLOCKS; }

// whether one of the two transform forms takes blocks of this shape
bool noalloc_shape_supported(int dim, int Bs0, int Bs1, int Bs2, int wavelet_x, int wavelet_y) {
    WaveletInfo w;
    char name[8] = {'C', 'D', 'F', (char)('0' + wavelet_x), (char)('0' + wavelet_y), 0};
    if (!make_wavelet(name, w)) return false;
    FwtArgs a;
    if (!make_fwt_args(w, 1, nullptr, nullptr, a)) return false;
    const long long ny = Bs1 + 2 * a.fmax, nz = dim == 3 ? Bs2 + 2 * a.fmax : 1;
    const long long smem = 8LL * Bs0 * ny * nz;
    const bool tpo = (long long)Bs0 * Bs1 * nz <= (long long)kTpoThreads * kTpoMaxPerThread && smem <= 110 * 1024;
    const bool column = smem <= 227 * 1024 && Bs1 <= 64 && Bs2 <= 64;
    return tpo || column;
}

cudaError_t launch_fwt_flags_noalloc(int dim, int nblk, const double *u, BufGeo geo, int Bs0, int Bs1, int Bs2,
                                     int nc, int wavelet_x, int wavelet_y, const double *eps_host,
                                     const int *tsvc_host, int *flags, double *details, cudaStream_t s) {
    if (nblk <= 0) return cudaSuccess;
    if (nblk > WG_NOALLOC_MAX_BLOCKS || nc > WG_NOALLOC_MAX_COMP) return cudaErrorInvalidValue;
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    NoAllocPtrs P;
    e = noalloc_setup(dev, s, P);
    if (e != cudaSuccess) return e;
    WaveletInfo w;
    char name[8] = {'C', 'D', 'F', (char)('0' + wavelet_x), (char)('0' + wavelet_y), 0};
    if (!make_wavelet(name, w)) return cudaErrorInvalidValue;
    FwtArgs a;
    if (!make_fwt_args(w, nc, eps_host, tsvc_host, a)) return cudaErrorInvalidValue;
    a.blk = P.blocks;
    a.u = u;
    a.geo = geo;
    a.Bs[0] = Bs0;
    a.Bs[1] = Bs1;
    a.Bs[2] = Bs2;
    a.flags = flags;
    a.details = details;
    if (a.fmax > geo.gb) return cudaErrorInvalidValue;
    // the thread-per-output transform where the block fits it, else the
    // column form
    e = launch_tpo(0, dim, P.blocks, nblk, const_cast<double *>(u), geo, Bs0, Bs1, Bs2, nc, w, a.fmax, P.detail, s);
    if (e == cudaErrorNotSupported) {
        cudaGetLastError();
        const int ny = Bs1 + 2 * a.fmax, nz = dim == 3 ? Bs2 + 2 * a.fmax : 1;
        const size_t smem = sizeof(double) * (size_t)Bs0 * ny * nz;
        if (dim == 2) {
            e = cudaFuncSetAttribute(fwt_detail_kernel<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
            if (e == cudaSuccess) fwt_detail_kernel<2><<<nblk * nc, 256, smem, s>>>(a, P.detail);
        } else {
            e = cudaFuncSetAttribute(fwt_detail_kernel<3>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
            if (e == cudaSuccess) fwt_detail_kernel<3><<<nblk * nc, 256, smem, s>>>(a, P.detail);
        }
        if (e == cudaSuccess) e = cudaGetLastError();
    }
    if (e != cudaSuccess) return e;
    flag_kernel<<<(nblk + 127) / 128, 128, 0, s>>>(a, P.detail, nblk);
    return cudaGetLastError();
}

// refineBlock: daughter k of parent p is written to slot child_slot[p * 2^d + k]
__global__ void __launch_bounds__(256) refine_kernel(const int *parent, int nparent, const int *child_slot,
                                                     const double *u, BufGeo geo, int dim, int Bs0, int Bs1, int Bs2,
                                                     int nc, int order_idx, int ncoef) {
    const int nd = 1 << dim;
    const long long np = geo.npts();
    const long long total = (long long)nd * np;
    for (int pi = blockIdx.y; pi < nparent; pi += gridDim.y) {
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
            double *dst = const_cast<double *>(u) + ((long long)child_slot[(long long)pi * nd + k] * nc) * np + r;
            for (int c = 0; c < nc; c++) {
                pc.src = src + c * np;
                dst[c * np] = pred_xyz(pc, fx, fy, fz);
            }
        }
    }
}

cudaError_t launch_refine(int dim, const int *parent, int nparent, const int *child_slot, const double *u,
                          BufGeo geo, int Bs0, int Bs1, int Bs2, int nc, int order_predictor, cudaStream_t s) {
    if (nparent <= 0) return cudaSuccess;
    dim3 grid(64, std::min(nparent, 65535));
    refine_kernel<<<grid, 256, 0, s>>>(parent, nparent, child_slot, u, geo, dim, Bs0, Bs1, Bs2, nc,
                                       order_predictor / 2 - 1, order_predictor);
    return cudaGetLastError();
}

}  // namespace wg
