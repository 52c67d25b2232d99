// k_lifted.cu -- device work of the full-tree adaptation with coarse
// extension (lifted wavelets); the lists come from lifted.cpp.
//
// * xcopy_kernel: same-level ghost copies from hvy_block or hvy_tmp into
//   hvy_block (unpack_ghostlayers_internal, LIB/MPI/xfer_block_data.f90:
//   397-409).
// * hd_filter_kernel: the HD filter of blockFilterXYZ_vct with
//   do_restriction (module_wavelets.f90:307-401) evaluated only on the
//   interior SC lattice the restriction reads: x pass on every second x over
//   the rows the later passes need, y pass, z pass; each sum starts from 0 and
//   adds every tap in ascending order with round-to-nearest multiplies and
//   adds, as the reference's loop does.
// * scbox_kernel: the SC that restrict_copy_at_CE copies back
//   (LIB/MPI/restrict_predict_data.f90:121-170).
// * restrict_scratch_kernel: the restriction gather from the filtered
//   lattice (restrict_data, :45-99).
// * boxop_kernel: coarse-extension WC zeroing / SC copies on strided boxes
//   (coarseExtensionManipulateWC/SC_block, module_wavelets.f90:877-1028).
// * blockcopy_kernel: hvy_tmp = hvy_block and back for listed blocks.
// * zone_detail_kernel: max |WC| of a patch per component with the SC
//   zeroed (threshold_block with indices, LIB/INDICATORS/threshold_block.f90)
//   for the security zone.
#include "common.cuh"
#include "lifted.hpp"
#include "exact.cuh"

namespace wg {

// HD filter taps of a launch, passed by value (no state shared between
// launches, streams or devices)
struct HdTaps {
    double v[32];
    int k[32], s[32], m[32];   // tap kinds for the integer-pipe products (exact.cuh)
    long long g[32];           // sign bit of each tap
    int lo, n;
};

__global__ void __launch_bounds__(128) xcopy_kernel(const Patch *__restrict__ patches, int npatch,
                                                    const double *__restrict__ sbuf, double *dbuf, BufGeo geo,
                                                    int nc) {
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (warp >= npatch) return;
    const Patch p = patches[warp];
    const int ex = p.rhi[0] - p.rlo[0] + 1, ey = p.rhi[1] - p.rlo[1] + 1, ez = p.rhi[2] - p.rlo[2] + 1;
    const long long npts = geo.npts();
    const int n = ex * ey * ez;
    for (int c = 0; c < nc; c++) {
        const double *src = sbuf + ((long long)p.src * nc + c) * npts;
        double *dst = dbuf + ((long long)p.dst * nc + c) * npts;
        for (int i = lane; i < n; i += 32) {
            const int ix = i % ex, iy = (i / ex) % ey, iz = i / (ex * ey);
            dst[((long long)(p.rlo[2] + iz) * geo.ny + (p.rlo[1] + iy)) * geo.nx + p.rlo[0] + ix] =
                src[((long long)(p.slo[2] + iz) * geo.ny + (p.slo[1] + iy)) * geo.nx + p.slo[0] + ix];
        }
    }
}

// one CTA per (entry, component); X: [nz][ny][hx], Y: [nz][hy][hx]
template <int DIM>
__global__ void __launch_bounds__(256) hd_filter_kernel(const __grid_constant__ HdTaps H,
                                                        const FilterEntry *__restrict__ ent, const double *A,
                                                        const double *T, BufGeo geo, int Bx, int By, int Bz, int nc,
                                                        double *scratch) {
    const double *c_lhd = H.v;
    const int *c_lhd_k = H.k, *c_lhd_s = H.s, *c_lhd_m = H.m;
    const long long *c_lhd_g = H.g;
    extern __shared__ double sm[];
    const int e = blockIdx.x / nc, c = blockIdx.x % nc;
    const FilterEntry fe = ent[e];
    const double *u = (fe.src_tmp ? T : A) + ((long long)fe.slot * nc + c) * geo.npts();
    const int g = geo.gb, lo = H.lo, nt = H.n, hi = lo + nt - 1;
    const int hx = Bx / 2, hy = By / 2, hz = DIM == 3 ? Bz / 2 : 1;
    const int y0 = g + lo, ny = By + hi - lo, z0 = DIM == 3 ? g + lo : 0, nz = DIM == 3 ? Bz + hi - lo : 1;
    double *X = sm, *Y = sm + (size_t)hx * ny * nz;
    for (int i = threadIdx.x; i < hx * ny * nz; i += blockDim.x) {
        const int mx = i % hx, yy = (i / hx) % ny, zz = i / (hx * ny);
        const double *row = u + ((long long)(z0 + zz) * geo.ny + (y0 + yy)) * geo.nx + g + 2 * mx;
        double s = 0.0;
        bool bad = false;
        for (int t = 0; t < nt; t++)
            s = __dadd_rn(s, tap_mul(row[lo + t], c_lhd[t], c_lhd_k[t], c_lhd_s[t], c_lhd_m[t], c_lhd_g[t], bad));
        if (bad) {
            s = 0.0;
            for (int t = 0; t < nt; t++) s = __dadd_rn(s, __dmul_rn(row[lo + t], c_lhd[t]));
        }
        X[i] = s;
    }
    __syncthreads();
    for (int i = threadIdx.x; i < hx * hy * nz; i += blockDim.x) {
        const int mx = i % hx, my = (i / hx) % hy, zz = i / (hx * hy);
        const double *col = X + ((size_t)zz * ny + (g + 2 * my - y0)) * hx + mx;
        double s = 0.0;
        bool bad = false;
        for (int t = 0; t < nt; t++)
            s = __dadd_rn(s, tap_mul(col[(long long)(lo + t) * hx], c_lhd[t], c_lhd_k[t], c_lhd_s[t], c_lhd_m[t],
                                     c_lhd_g[t], bad));
        if (bad) {
            s = 0.0;
            for (int t = 0; t < nt; t++) s = __dadd_rn(s, __dmul_rn(col[(long long)(lo + t) * hx], c_lhd[t]));
        }
        Y[i] = s;
    }
    __syncthreads();
    double *out = scratch + ((long long)e * nc + c) * hx * hy * hz;
    if (DIM == 2) {
        for (int i = threadIdx.x; i < hx * hy; i += blockDim.x) out[i] = Y[i];
        return;
    }
    for (int i = threadIdx.x; i < hx * hy * hz; i += blockDim.x) {
        const int mx = i % hx, my = (i / hx) % hy, mz = i / (hx * hy);
        const double *pl = Y + ((size_t)(g + 2 * mz - z0) * hy + my) * hx + mx;
        double s = 0.0;
        bool bad = false;
        for (int t = 0; t < nt; t++)
            s = __dadd_rn(s, tap_mul(pl[(long long)(lo + t) * hx * hy], c_lhd[t], c_lhd_k[t], c_lhd_s[t],
                                     c_lhd_m[t], c_lhd_g[t], bad));
        if (bad) {
            s = 0.0;
            for (int t = 0; t < nt; t++) s = __dadd_rn(s, __dmul_rn(pl[(long long)(lo + t) * hx * hy], c_lhd[t]));
        }
        out[i] = s;
    }
}

__global__ void __launch_bounds__(128) scbox_kernel(const ScBox *__restrict__ boxes, int nbox,
                                                    const FilterEntry *__restrict__ ent, const double *A,
                                                    const double *T, BufGeo geo, int hx, int hy, int hz, int nc,
                                                    double *scratch) {
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (warp >= nbox) return;
    const ScBox b = boxes[warp];
    const FilterEntry fe = ent[b.entry];
    const int g = geo.gb;
    const int ex = b.hi[0] - b.lo[0] + 1, ey = b.hi[1] - b.lo[1] + 1, ez = b.hi[2] - b.lo[2] + 1;
    const int n = ex * ey * ez;
    for (int c = 0; c < nc; c++) {
        const double *u = (fe.src_tmp ? T : A) + ((long long)fe.slot * nc + c) * geo.npts();
        double *out = scratch + ((long long)b.entry * nc + c) * hx * hy * hz;
        for (int i = lane; i < n; i += 32) {
            const int mx = b.lo[0] + i % ex, my = b.lo[1] + (i / ex) % ey, mz = b.lo[2] + i / (ex * ey);
            const int z = hz > 1 ? g + 2 * mz : 0;
            out[((long long)mz * hy + my) * hx + mx] = u[((long long)z * geo.ny + g + 2 * my) * geo.nx + g + 2 * mx];
        }
    }
}

__global__ void __launch_bounds__(128) restrict_scratch_kernel(const Patch *__restrict__ patches, int npatch,
                                                               const double *__restrict__ scratch, double *A,
                                                               BufGeo geo, int hx, int hy, int hz, int nc) {
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (warp >= npatch) return;
    const Patch p = patches[warp];
    const int g = geo.gb;
    const int ex = p.rhi[0] - p.rlo[0] + 1, ey = p.rhi[1] - p.rlo[1] + 1, ez = p.rhi[2] - p.rlo[2] + 1;
    const int n = ex * ey * ez;
    const long long npts = geo.npts();
    for (int c = 0; c < nc; c++) {
        const double *s = scratch + ((long long)p.src * nc + c) * hx * hy * hz;
        double *dst = A + ((long long)p.dst * nc + c) * npts;
        for (int i = lane; i < n; i += 32) {
            const int ix = i % ex, iy = (i / ex) % ey, iz = i / (ex * ey);
            const int mx = (p.slo[0] + 2 * (p.blo[0] + ix) - g) >> 1;
            const int my = (p.slo[1] + 2 * (p.blo[1] + iy) - g) >> 1;
            const int mz = hz > 1 ? (p.slo[2] + 2 * (p.blo[2] + iz) - g) >> 1 : 0;
            dst[((long long)(p.rlo[2] + iz) * geo.ny + (p.rlo[1] + iy)) * geo.nx + p.rlo[0] + ix] =
                s[((long long)mz * hy + my) * hx + mx];
        }
    }
}

__global__ void __launch_bounds__(128) boxop_kernel(const BoxOp *__restrict__ ops, int nop, double *A,
                                                    const double *T, BufGeo geo, int nc) {
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (warp >= nop) return;
    const BoxOp o = ops[warp];
    int ext[3];
    for (int d = 0; d < 3; d++) ext[d] = (o.hi[d] - o.lo[d]) / o.step[d] + 1;
    const int n = ext[0] * ext[1] * ext[2];
    const long long npts = geo.npts();
    for (int c = 0; c < nc; c++) {
        double *a = A + ((long long)o.slot * nc + c) * npts;
        const double *t = T + ((long long)o.slot * nc + c) * npts;
        for (int i = lane; i < n; i += 32) {
            const int x = o.lo[0] + (i % ext[0]) * o.step[0];
            const int y = o.lo[1] + ((i / ext[0]) % ext[1]) * o.step[1];
            const int z = o.lo[2] + (i / (ext[0] * ext[1])) * o.step[2];
            const long long q = ((long long)z * geo.ny + y) * geo.nx + x;
            a[q] = o.op == 0 ? 0.0 : t[q];
        }
    }
}

// dst[slot] = src[slot] for the listed blocks (all components and points)
__global__ void blockcopy_kernel(const int *__restrict__ slots, int n, const double *__restrict__ src,
                                 double *__restrict__ dst, long long per_block) {
    const long long chunks = (per_block + 1023) / 1024;
    for (long long w = blockIdx.x; w < (long long)n * chunks; w += gridDim.x) {
        const int i = (int)(w / chunks);
        const long long off = (long long)slots[i] * per_block + (w % chunks) * 1024;
        const long long end = min(per_block - (w % chunks) * 1024, 1024LL);
        for (int k = threadIdx.x; k < end; k += blockDim.x) dst[off + k] = src[off + k];
    }
}

struct ZoneBox {
    int slot;
    int lo[3], hi[3], io[3];
};

// per (item, component): max |v| over the box with the SC lattice (first
// point lo + io, step 2 in every active direction) counted as 0
__global__ void __launch_bounds__(128) zone_detail_kernel(const ZoneBox *__restrict__ items, int n,
                                                          const double *A, BufGeo geo, int nc, int dim,
                                                          double *det) {
    const int item = blockIdx.x / nc, c = blockIdx.x % nc;
    if (item >= n) return;
    const ZoneBox z = items[item];
    const int ex = z.hi[0] - z.lo[0] + 1, ey = z.hi[1] - z.lo[1] + 1, ez = z.hi[2] - z.lo[2] + 1;
    const double *u = A + ((long long)z.slot * nc + c) * geo.npts();
    double m = 0.0;
    for (int i = threadIdx.x; i < ex * ey * ez; i += blockDim.x) {
        const int ix = i % ex, iy = (i / ex) % ey, iz = i / (ex * ey);
        const bool sc = ((ix - z.io[0]) % 2 == 0) && ((iy - z.io[1]) % 2 == 0) && (dim == 2 || (iz - z.io[2]) % 2 == 0);
        const double v = fabs(u[((long long)(z.lo[2] + iz) * geo.ny + (z.lo[1] + iy)) * geo.nx + z.lo[0] + ix]);
        if (!sc) m = fmax(m, v);
    }
    for (int w = 16; w; w >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, w));
    __shared__ double red[4];
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = m;
    __syncthreads();
    if (threadIdx.x == 0) det[(long long)item * nc + c] = fmax(fmax(red[0], red[1]), fmax(red[2], red[3]));
}

// ---------------------------------------------------------------------------
static bool make_hd_taps(const double *hd, int lo, int n, HdTaps &H) {
    if (n > 32 || n < 1 || !hd) return false;
    H = HdTaps{};
    for (int i = 0; i < n; i++) {
        H.v[i] = hd[i];
        classify_tap(H.v[i], H.k[i], H.s[i], H.m[i]);
        H.g[i] = H.v[i] < 0.0 ? (long long)0x8000000000000000ULL : 0LL;
    }
    H.lo = lo;
    H.n = n;
    return true;
}

static int warps_grid(int n) { return (n + 3) / 4; }

cudaError_t launch_xcopy(const Patch *p, int n, const double *sbuf, double *dbuf, BufGeo geo, int nc, cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    if (!p) return cudaErrorInvalidValue;
    xcopy_kernel<<<warps_grid(n), 128, 0, s>>>(p, n, sbuf, dbuf, geo, nc);
    return cudaGetLastError();
}

cudaError_t launch_hd_filter(int dim, const FilterEntry *ent, int n, const double *A, const double *T, BufGeo geo,
                             int Bx, int By, int Bz, int nc, const double *hd, int hd_lo, int hd_n, double *scratch,
                             cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    HdTaps H;
    if (!ent || !scratch || !make_hd_taps(hd, hd_lo, hd_n, H)) return cudaErrorInvalidValue;
    const int hi = hd_lo + hd_n - 1;
    if (-hd_lo > geo.gb || hi > geo.gb) return cudaErrorInvalidValue;
    const int hx = Bx / 2, hy = By / 2, ny = By + hi - hd_lo, nz = dim == 3 ? Bz + hi - hd_lo : 1;
    const size_t smem = sizeof(double) * ((size_t)hx * ny * nz + (size_t)hx * hy * nz);
    if (smem > 200 * 1024) return cudaErrorInvalidValue;
    auto go = [&](auto kern) -> cudaError_t {
        if (smem > 48 * 1024) {
            cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
            if (e != cudaSuccess) return e;
        }
        kern<<<n * nc, 256, smem, s>>>(H, ent, A, T, geo, Bx, By, Bz, nc, scratch);
        return cudaGetLastError();
    };
    return dim == 2 ? go(hd_filter_kernel<2>) : go(hd_filter_kernel<3>);
}

cudaError_t launch_scbox(const ScBox *b, int n, const FilterEntry *ent, const double *A, const double *T, BufGeo geo,
                         int hx, int hy, int hz, int nc, double *scratch, cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    if (!b || !ent) return cudaErrorInvalidValue;
    scbox_kernel<<<warps_grid(n), 128, 0, s>>>(b, n, ent, A, T, geo, hx, hy, hz, nc, scratch);
    return cudaGetLastError();
}

cudaError_t launch_restrict_scratch(const Patch *p, int n, const double *scratch, double *A, BufGeo geo, int hx,
                                    int hy, int hz, int nc, cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    if (!p || !scratch) return cudaErrorInvalidValue;
    restrict_scratch_kernel<<<warps_grid(n), 128, 0, s>>>(p, n, scratch, A, geo, hx, hy, hz, nc);
    return cudaGetLastError();
}

cudaError_t launch_boxop(const BoxOp *o, int n, double *A, const double *T, BufGeo geo, int nc, cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    if (!o) return cudaErrorInvalidValue;
    boxop_kernel<<<warps_grid(n), 128, 0, s>>>(o, n, A, T, geo, nc);
    return cudaGetLastError();
}

cudaError_t launch_blockcopy(const int *slots, int n, const double *src, double *dst, long long per_block,
                             cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    if (!slots) return cudaErrorInvalidValue;
    const long long work = (long long)n * ((per_block + 1023) / 1024);
    const int grid = (int)std::min<long long>(work, 152LL * 16);
    blockcopy_kernel<<<grid, 256, 0, s>>>(slots, n, src, dst, per_block);
    return cudaGetLastError();
}

cudaError_t launch_zone_detail(const void *items, int n, const double *A, BufGeo geo, int nc, int dim, double *det,
                               cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    if (!items || !det) return cudaErrorInvalidValue;
    zone_detail_kernel<<<n * nc, 128, 0, s>>>((const ZoneBox *)items, n, A, geo, nc, dim, det);
    return cudaGetLastError();
}

}  // namespace wg
