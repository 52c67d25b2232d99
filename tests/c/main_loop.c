/*
 * main_loop.c -- a plain C host of the C ABI (include/wabbit_gb300.h): the
 * time loop of the reference's main program (LIB/MAIN/main.f90:309-427) on
 * one tree -- sync_ghosts_tree, refine_tree("everywhere"), N_dt_per_grid
 * RK4 steps (timeStep_tree, LIB/TIME/timeStep_tree.f90:44), adapt_tree
 * (LIB/MESH/adapt_tree.f90:11) -- on a 2-D ACM run with two Gaussian
 * vortices, checking every status, the grid after each adaptation and the
 * state. Prints "main loop OK" and exits 0 on success.
 *
 * Build: cc -std=c99 -I include tests/c/main_loop.c -L wabbit_gb300/_lib
 *        -lwabbit_gb300 -lm
 */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "wabbit_gb300.h"

#define CHECK(call)                                                                                   \
    do {                                                                                              \
        int rc_ = (call);                                                                             \
        if (rc_ != WG_OK) {                                                                           \
            fprintf(stderr, "%s:%d: %s returned %d (%s)\n", __FILE__, __LINE__, #call, rc_,            \
                    wg_last_error());                                                                 \
            return 1;                                                                                 \
        }                                                                                             \
    } while (0)

#define EXPECT(cond)                                                                                  \
    do {                                                                                              \
        if (!(cond)) {                                                                                \
            fprintf(stderr, "%s:%d: expected %s\n", __FILE__, __LINE__, #cond);                       \
            return 1;                                                                                 \
        }                                                                                             \
    } while (0)

enum { BS = 16, NEQ = 3, JMIN = 2, JMAX = 4, JSTART = 3, MAXB = 4096, N_DT_PER_GRID = 2, ITERS = 3 };

static const double PI = 3.14159265358979323846;

/* velocity of a Gaussian vortex at (x0, y0) of radius r and strength s,
 * minimum-image distance on the periodic unit square */
static void vortex(double x, double y, double x0, double y0, double r, double s, double *u, double *v) {
    double dx = x - x0, dy = y - y0;
    dx -= floor(dx + 0.5);
    dy -= floor(dy + 0.5);
    const double e = s / (PI * r * r) * exp(-(dx * dx + dy * dy) / (r * r));
    *u += -dy * e;
    *v += dx * e;
}

/* interior initial state of the listed blocks, (nblk, NEQ, BS, BS) */
static void initial_state(int nblk, const int *level, const int *coords, double *u) {
    for (int b = 0; b < nblk; b++) {
        const double dx = ldexp(1.0, -level[b]) / BS;
        for (int j = 0; j < BS; j++)
            for (int i = 0; i < BS; i++) {
                const double x = (coords[3 * b] * BS + i) * dx, y = (coords[3 * b + 1] * BS + j) * dx;
                double vx = 0.0, vy = 0.0;
                vortex(x, y, 0.40, 0.50, 0.08, 1.0, &vx, &vy);
                vortex(x, y, 0.62, 0.50, 0.06, -0.8, &vx, &vy);
                const size_t o = (size_t)b * NEQ * BS * BS + (size_t)j * BS + i;
                u[o] = vx;
                u[o + BS * BS] = vy;
                u[o + 2 * BS * BS] = 0.0;
            }
    }
}

static int count_finite(const double *u, size_t n) {
    for (size_t i = 0; i < n; i++)
        if (!isfinite(u[i])) return 0;
    return 1;
}

int main(void) {
    wg_config cfg;
    CHECK(wg_config_defaults(&cfg, 2));
    cfg.Bs[0] = cfg.Bs[1] = BS;
    cfg.Jmin = JMIN;
    cfg.Jmax = JMAX;
    cfg.c0 = 20.0;
    cfg.nu = 1.0e-3;
    cfg.CFL = 0.5;
    cfg.penalization = 0;
    cfg.eps = 1.0e-3;
    cfg.eps_normalized = 1;
    cfg.time_max = 1.0e9;

    wg_ctx *ctx = NULL;
    CHECK(wg_ctx_create(&cfg, MAXB, &ctx));
    int tree = -1;
    CHECK(wg_tree_create(ctx, &cfg, &tree));

    /* equidistant start grid on level JSTART */
    const int n0 = 1 << (2 * JSTART);
    int *level = malloc(sizeof(int) * MAXB), *coords = malloc(sizeof(int) * 3 * MAXB);
    double *u = malloc(sizeof(double) * (size_t)MAXB * NEQ * BS * BS);
    if (!level || !coords || !u) return 1;
    for (int b = 0; b < n0; b++) {
        level[b] = JSTART;
        coords[3 * b] = b % (1 << JSTART);
        coords[3 * b + 1] = b / (1 << JSTART);
        coords[3 * b + 2] = 0;
    }
    CHECK(wg_set_grid(ctx, tree, n0, level, coords));
    initial_state(n0, level, coords, u);
    CHECK(wg_upload_interior(ctx, tree, u));
    CHECK(wg_set_time(ctx, tree, 0.0));

    /* an invalid call fails with a status and a message, and changes nothing */
    EXPECT(wg_set_grid(ctx, tree, -1, level, coords) == WG_EINVAL);
    EXPECT(strlen(wg_last_error()) > 0);

    double t_prev = 0.0;
    for (int it = 0; it < ITERS; it++) {
        int nblk = 0;
        CHECK(wg_sync_ghosts(ctx, tree, cfg.g, cfg.g));
        CHECK(wg_refine_everywhere(ctx, tree));
        CHECK(wg_get_nblocks(ctx, tree, &nblk));
        EXPECT(nblk > 0 && nblk <= MAXB);
        double dt = 0.0;
        CHECK(wg_compute_dt(ctx, tree, &dt));
        EXPECT(dt > 0.0 && isfinite(dt));
        CHECK(wg_run(ctx, 1, &tree, N_DT_PER_GRID - 1, 1));
        double t = 0.0, dt_last = 0.0;
        CHECK(wg_rk4_step(ctx, tree, &t, &dt_last));
        EXPECT(t > t_prev && dt_last > 0.0);
        t_prev = t;
        int nnew = 0;
        CHECK(wg_adapt(ctx, tree, NULL, WG_ADAPT_THRESHOLD, &nnew));
        CHECK(wg_get_nblocks(ctx, tree, &nblk));
        EXPECT(nnew == nblk && nblk > 0 && nblk <= MAXB);
        CHECK(wg_get_grid(ctx, tree, MAXB, level, coords));
        /* the adapted grid covers the unit square exactly once */
        long long area = 0;
        for (int b = 0; b < nblk; b++) {
            EXPECT(level[b] >= JMIN && level[b] <= JMAX);
            EXPECT(coords[3 * b] >= 0 && coords[3 * b] < (1 << level[b]));
            area += 1LL << (2 * (JMAX - level[b]));
        }
        EXPECT(area == 1LL << (2 * JMAX));
        CHECK(wg_download_interior(ctx, tree, u));
        EXPECT(count_finite(u, (size_t)nblk * NEQ * BS * BS));
        printf("iteration %d: t = %.6e, %d blocks\n", it, t, nblk);
    }
    CHECK(wg_synchronize(ctx));
    CHECK(wg_tree_destroy(ctx, tree));
    CHECK(wg_ctx_destroy(ctx));
    free(level);
    free(coords);
    free(u);
    printf("main loop OK\n");
    return 0;
}
