// geometry.cpp -- penalisation masks drawn from a tree's geometry.
//
// The reference builds hvy_mask in createMask_tree (LIB/MESH/
// createMask_tree.f90) through CREATE_MASK_meta (LIB/EQUATION/
// module_physics_metamodule.f90:38-83: mask = 0, colour = 1) and the ACM
// module's create_mask_2D_acm / create_mask_3D_acm (LIB/EQUATION/ACMnew/
// create_mask.f90:6-320, stage "all-parts"): the obstacle (draw_circle /
// draw_sphere, LIB/EQUATION/insects/module_geometry.f90:49-117,315-381) and
// the sponge (sponge_2D / sponge_3D, LIB/EQUATION/ACMnew/sponge.f90). Only
// interior points reach the RHS and the indicator, so only those are
// computed here, straight into the interior-only layout of the device mask
// pool. Every expression keeps the reference's operand order, and this
// unit is compiled without floating-point contraction, so the words equal
// the reference's on the same host libm.
#include "geometry.hpp"

#include <algorithm>
#include <cmath>

namespace wg {

namespace {

const double kPi = 4.0 * std::atan(1.0);   // module_globals.f90:51

// step_cosine3/4 (LIB/HELPER/module_helpers.f90:436-487): 1 below t-h, 0
// above t+h, a half cosine in between
double cos_step(double x, double t, double h) {
    const double r = x - t;
    if (r <= -h) return 1.0;
    if (r >= +h) return 0.0;
    return 0.5 * (1.0 + std::cos((r + h) * kPi / (2.0 * h)));
}

struct BlockGeo {
    int dim, g, n[3];          // interior extents (n[2] = 1 in 2-D)
    double x0[3], dx[3];
};

BlockGeo block_geo(const wg_config &c, int level, const int co[3]) {
    BlockGeo b;
    b.dim = c.dim;
    b.g = c.g;
    for (int d = 0; d < 3; d++) {
        b.n[d] = d < c.dim ? c.Bs[d] : 1;
        b.dx[d] = 0.0;
        b.x0[d] = 0.0;
    }
    // get_block_spacing_origin (LIB/TREE/module_treelib.f90:96-101)
    for (int d = 0; d < c.dim; d++) {
        b.dx[d] = std::pow(2.0, -level) * c.domain[d] / (double)c.Bs[d];
        b.x0[d] = (double)(co[d] * c.Bs[d]) * b.dx[d];
    }
    return b;
}

// chi of the obstacle on the interior (component 0 of out); colour stays 1
void draw_obstacle(const wg_config &c, const wg_geometry &G, const BlockGeo &b, double *chi) {
    if (G.kind != WG_GEOM_CYLINDER && G.kind != WG_GEOM_SPHERE) return;
    // smoothing width and safety of the cosine step (module_ACM.f90:457-471)
    double dx_min = 9e9;
    for (int d = 0; d < c.dim; d++) dx_min = std::min(dx_min, std::pow(2.0, -c.Jmax) * (c.domain[d] / (double)c.Bs[d]));
    const double h = dx_min * G.C_smooth, safety = 1.0 * h;
    double dmin = b.dx[0];
    for (int d = 1; d < b.dim; d++) dmin = std::min(dmin, b.dx[d]);
    const int Nsafety = (int)std::ceil(safety / dmin);
    // index box of the drawing (1-based array indices of the ghosted block),
    // clipped to the interior g+1 .. g+Bs
    int lo[3] = {0, 0, 0}, hi[3] = {0, 0, 0};
    for (int d = 0; d < b.dim; d++) {
        const int bmin = (int)((G.x_cntr[d] - G.R_cyl - b.x0[d]) / b.dx[d]) - Nsafety + (b.g + 1);
        const int bmax = (int)std::ceil((G.x_cntr[d] + G.R_cyl - b.x0[d]) / b.dx[d]) + Nsafety + (b.g + 1);
        lo[d] = std::max(bmin, b.g + 1) - (b.g + 1);
        hi[d] = std::min(bmax, b.g + b.n[d]) - (b.g + 1);
        if (lo[d] > hi[d]) return;
    }
    for (int k = lo[2]; k <= hi[2]; k++)
        for (int j = lo[1]; j <= hi[1]; j++)
            for (int i = lo[0]; i <= hi[0]; i++) {
                const double x = (double)i * b.dx[0] + b.x0[0];
                const double y = (double)j * b.dx[1] + b.x0[1];
                double dist;
                if (b.dim == 2) {   // signed_distance_circle_2D, norm2_2d
                    const double ax = x - G.x_cntr[0], ay = y - G.x_cntr[1];
                    dist = std::sqrt(ax * ax + ay * ay) - G.R_cyl;
                } else {            // signed_distance_sphere_3D, norm2_3d
                    const double z = (double)k * b.dx[2] + b.x0[2];
                    const double ax = x - G.x_cntr[0], ay = y - G.x_cntr[1], az = z - G.x_cntr[2];
                    dist = std::sqrt(ax * ax + ay * ay + az * az) - G.R_cyl;
                }
                const double v = cos_step(dist, 0.0, h);
                double &w = chi[((size_t)k * b.n[1] + j) * b.n[0] + i];
                if (v >= w) w = v;
            }
}

// sponge on the interior (component 5 of out)
void draw_sponge(const wg_config &c, const wg_geometry &G, const BlockGeo &b, double *spo) {
    const double Ls = G.L_sponge;
    const double off = 0.5 * c.domain[0];
    if (b.dim == 3) {
        // blocks that no sponge point can reach are left at zero
        if (G.sponge_type == WG_SPONGE_RECT) {
            double t = std::min(std::min(b.x0[0], b.x0[1]), b.x0[2]);
            for (int d = 0; d < 3; d++) t = std::min(t, c.domain[d] - (b.x0[d] + b.dx[d] * (double)c.Bs[d]));
            if (t > Ls) return;
        } else {
            const double pp = G.p_sponge, pinv = 1.0 / pp;
            double e[3];
            for (int d = 0; d < 3; d++)
                e[d] = std::pow(std::max(std::fabs(b.x0[d] - off), std::fabs(b.x0[d] + b.dx[d] * (double)c.Bs[d] - off)), pp);
            if (off - std::pow(e[0] + e[1] + e[2], pinv) > Ls) return;
        }
    }
    for (int k = 0; k < b.n[2]; k++)
        for (int j = 0; j < b.n[1]; j++)
            for (int i = 0; i < b.n[0]; i++) {
                double t;
                if (G.sponge_type == WG_SPONGE_RECT) {
                    // distance to the nearest domain face
                    const double x = (double)i * b.dx[0] + b.x0[0];
                    const double y = (double)j * b.dx[1] + b.x0[1];
                    if (b.dim == 2) {
                        t = std::min(std::min(x, y), std::min(-(x - c.domain[0]), -(y - c.domain[1])));
                    } else {
                        const double z = (double)k * b.dx[2] + b.x0[2];
                        const double v[6] = {x, y, z, -(x - c.domain[0]), -(y - c.domain[1]), -(z - c.domain[2])};
                        t = v[0];
                        for (int q = 1; q < 6; q++) t = std::min(t, v[q]);
                    }
                } else if (b.dim == 2) {
                    // p-norm distance to the centre, turned into distance to the boundary
                    const double y = (double)j * b.dx[1] + b.x0[1] - off;
                    const double x = (double)i * b.dx[0] + b.x0[0] - off;
                    t = -(std::pow(std::pow(x, G.p_sponge) + std::pow(y, G.p_sponge), 1.0 / G.p_sponge) - off);
                } else {
                    const double pp = G.p_sponge, pinv = 1.0 / pp;
                    const double z = std::pow((double)k * b.dx[2] + b.x0[2] - off, pp);
                    const double y = std::pow((double)j * b.dx[1] + b.x0[1] - off, pp);
                    const double x = std::pow((double)i * b.dx[0] + b.x0[0] - off, pp);
                    t = -(std::pow(x + y + z, pinv) - off);
                }
                spo[((size_t)k * b.n[1] + j) * b.n[0] + i] = cos_step(t, 0.5 * Ls, 0.5 * Ls);
            }
}

}  // namespace

const char *geometry_check(const wg_config &c, const wg_geometry &G) {
    if (G.kind != WG_GEOM_NONE && G.kind != WG_GEOM_CYLINDER && G.kind != WG_GEOM_SPHERE) return "unknown geometry kind";
    if (G.kind == WG_GEOM_CYLINDER && c.dim != 2) return "the cylinder geometry is 2-D";
    if (G.kind == WG_GEOM_SPHERE && c.dim != 3) return "the sphere geometry is 3-D";
    if (G.kind != WG_GEOM_NONE && !(G.R_cyl > 0.0 && G.C_smooth > 0.0)) return "R_cyl and C_smooth must be positive";
    if (c.use_sponge) {
        if (G.sponge_type != WG_SPONGE_RECT && G.sponge_type != WG_SPONGE_PNORM) return "unknown sponge type";
        if (!(G.L_sponge > 0.0)) return "L_sponge must be positive";
        if (G.sponge_type == WG_SPONGE_PNORM) {
            if (!(G.p_sponge > 0.0)) return "p_sponge must be positive";
            // sponge.f90: the p-norm sponge needs a cubic / square domain
            for (int d = 1; d < c.dim; d++)
                if (std::fabs(c.domain[d] - c.domain[0]) > 1.0e-10) return "the p-norm sponge needs equal domain sizes";
        }
    }
    return "";
}

bool geometry_mask_block(const wg_config &c, const wg_geometry &G, int level, const int co[3], double *out) {
    const BlockGeo b = block_geo(c, level, co);
    const size_t ni = (size_t)b.n[0] * b.n[1] * b.n[2];
    std::fill(out, out + 6 * ni, 0.0);
    std::fill(out + 4 * ni, out + 5 * ni, 1.0);
    if (!c.penalization) return false;
    draw_obstacle(c, G, b, out);
    if (c.use_sponge) draw_sponge(c, G, b, out + 5 * ni);
    for (size_t q = 0; q < ni; q++)
        if (out[q] != 0.0 || out[5 * ni + q] != 0.0) return true;
    return false;
}

int geometry_mask_status(const wg_config &c, const wg_geometry &G, int level, const int co[3]) {
    const BlockGeo b = block_geo(c, level, co);
    const size_t ni = (size_t)b.n[0] * b.n[1] * b.n[2];
    std::vector<double> chi(ni, 0.0);
    if (c.penalization) draw_obstacle(c, G, b, chi.data());
    double mx = chi[0], mn = chi[0];
    for (size_t q = 0; q < ni; q++) {
        if (chi[q] > 1.0e-12 && chi[q] < 1.0 - 1.0e-12) return 0;
        mx = std::max(mx, chi[q]);
        mn = std::min(mn, chi[q]);
    }
    return (mx - mn) > 1.0e-12 ? 0 : -1;
}

}  // namespace wg
