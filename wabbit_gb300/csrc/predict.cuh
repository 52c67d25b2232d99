// predict.cuh -- coarse-to-fine interpolation of the reference's prediction
// routine (LIB/WAVELETS/module_wavelets.f90:96-284), evaluated point-wise.
//
// For a coarse box of n points per direction the reference fills a fine array
// of 2n-1 points: even fine indices copy coarse values, odd ones are
// interpolated first along x (on coarse rows/planes), then along y, then z,
// with the order-X predictor c (e.g. (-1,9,9,-1)/16); fine points whose
// stencil would leave the box stay zero. pred_xyz() returns the value the
// reference's fine array holds at (fx,fy,fz), with every product and sum
// rounded separately in the reference's left-to-right order.
#pragma once
#include "common.cuh"

namespace wg {

// predictor coefficients for order 2, 4, 6, 8 (module_wavelets.f90:126-128
// and the order-2/6/8 rows): exact binary fractions, initialised with the
// module on every device that loads it; one copy per translation unit
static __constant__ double c_pred[4][8] = {
    {0.5, 0.5},
    {-1.0 / 16.0, 9.0 / 16.0, 9.0 / 16.0, -1.0 / 16.0},
    {3.0 / 256.0, -25.0 / 256.0, 150.0 / 256.0, 150.0 / 256.0, -25.0 / 256.0, 3.0 / 256.0},
    {-5.0 / 2048.0, 49.0 / 2048.0, -245.0 / 2048.0, 1225.0 / 2048.0, 1225.0 / 2048.0, -245.0 / 2048.0, 49.0 / 2048.0,
     -5.0 / 2048.0},
};

struct PredCtx {
    const double *src;
    int nx, ny;          // source buffer strides
    int sx, sy, sz;      // coarse box lower corner
    int Fx, Fy, Fz;      // fine extents (2n-1)
    int nc;              // number of coefficients
    const double *c;
};

static __device__ __forceinline__ double coarse_at(const PredCtx &p, int cx, int cy, int cz) {
    return p.src[((long long)(p.sz + cz) * p.ny + (p.sy + cy)) * p.nx + (p.sx + cx)];
}

// value after the x pass at (fx, fy, fz) with fy, fz even
static __device__ double pred_x(const PredCtx &p, int fx, int fy, int fz) {
    if (!(fx & 1)) return coarse_at(p, fx >> 1, fy >> 1, fz >> 1);
    const int h = p.nc - 1;
    if (fx < h || fx > p.Fx - 1 - h) return 0.0;
    double s = __dmul_rn(p.c[0], coarse_at(p, (fx - h) >> 1, fy >> 1, fz >> 1));
    for (int m = 1; m < p.nc; m++) s = __dadd_rn(s, __dmul_rn(p.c[m], coarse_at(p, (fx - h + 2 * m) >> 1, fy >> 1, fz >> 1)));
    return s;
}

// value after the y pass at (fx, fy, fz) with fz even
static __device__ double pred_xy(const PredCtx &p, int fx, int fy, int fz) {
    if (!(fy & 1)) return pred_x(p, fx, fy, fz);
    const int h = p.nc - 1;
    if (fy < h || fy > p.Fy - 1 - h) return 0.0;
    double s = __dmul_rn(p.c[0], pred_x(p, fx, fy - h, fz));
    for (int m = 1; m < p.nc; m++) s = __dadd_rn(s, __dmul_rn(p.c[m], pred_x(p, fx, fy - h + 2 * m, fz)));
    return s;
}

static __device__ double pred_xyz(const PredCtx &p, int fx, int fy, int fz) {
    if (!(fz & 1)) return pred_xy(p, fx, fy, fz);
    const int h = p.nc - 1;
    if (fz < h || fz > p.Fz - 1 - h) return 0.0;
    double s = __dmul_rn(p.c[0], pred_xy(p, fx, fy, fz - h));
    for (int m = 1; m < p.nc; m++) s = __dadd_rn(s, __dmul_rn(p.c[m], pred_xy(p, fx, fy, fz - h + 2 * m)));
    return s;
}


}  // namespace wg
