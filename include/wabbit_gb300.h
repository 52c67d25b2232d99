/*
 * wabbit_gb300.h -- C ABI of the GB300-native block-level time-step hot path
 * of WABBIT (artificial-compressibility (ACM) right-hand side with volume
 * penalisation, ghost-node synchronisation, RK4 stage update, CDF wavelet
 * coarsening indicator).
 *
 * Every entry point returns an int status (WG_OK == 0, negative on error) and
 * never aborts the calling process. Arguments are plain pointers and sizes;
 * host buffers are borrowed only for the duration of a call.
 *
 * Heavy-data layout (identical to the reference's per-block Fortran layout
 * hvy_block(1:Bs+2g, 1:Bs+2g, 1:Bs+2g|1, 1:neq, 1:Nblocks),
 * LIB/MESH/allocate_forest.f90:228-271): for one block, x is fastest, then y,
 * then z, then the component; blocks follow each other. A "block-major host
 * array" below means exactly that layout, nblk * neq * nz * ny * nx doubles
 * with nx = ny = Bs+2g and nz = Bs+2g (3-D) or 1 (2-D).
 *
 * Grid description: block i sits on refinement level level[i] and has the
 * 0-based integer block coordinates coords[3*i+0..2] on that level
 * (0 <= c < 2^level), i.e. its origin is x0 = c*Bs*dx with
 * dx = 2^-level * domain/Bs (LIB/TREE/module_treelib.f90:96-101).
 */
#ifndef WABBIT_GB300_H
#define WABBIT_GB300_H

#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* status codes (mirroring the reference's abort() sites as return values) */
#define WG_OK          0
#define WG_EINVAL     -1   /* invalid argument / configuration               */
#define WG_ENOMEM     -2   /* device allocation failed (HBM budget)          */
#define WG_ECUDA      -3   /* a CUDA runtime call failed                      */
#define WG_EDIVERGED  -4   /* |u| > 1e12 in the state (rhs_ACM.f90:133-146)  */
#define WG_ETIMEOUT   -5   /* a bounded device wait gave up                   */
#define WG_EGRID      -6   /* grid is not a valid graded periodic forest      */
#define WG_ENOTSUP    -7   /* configuration not supported by this build       */

/* RHS precision modes */
#define WG_RHS_FP64   0    /* FP64 stencils and state                         */
#define WG_RHS_FP32   1    /* FP32 stencils, FP64 RK state and penalisation   */

/*
 * Run configuration: the subset of the reference's .ini keys that the hot
 * path reads (LIB/MESH/ini_file_to_params.f90:2-647 and
 * LIB/EQUATION/ACMnew/module_ACM.f90:172-609). Defaults are applied by
 * wg_config_defaults(); key names are given in brackets.
 */
typedef struct wg_config {
    int    dim;                 /* [Domain] dim: 2 or 3                        */
    int    Bs[3];               /* [Blocks] number_block_nodes (even)          */
    int    g;                   /* [Blocks] number_ghost_nodes                 */
    int    g_rhs;               /* [Blocks] number_ghost_nodes_rhs             */
    int    neq;                 /* [Blocks] number_equations (dim+1)           */
    double domain[3];           /* [Domain] domain_size                        */
    int    Jmin, Jmax;          /* [Blocks] min_treelevel / max_treelevel      */
    char   wavelet[16];         /* [Wavelet] wavelet, e.g. "CDF40", "CDF44"    */
    /* ACM physics [ACM-new] */
    double c0, nu, gamma_p;
    int    skew_symmetry;
    /* volume penalisation [VPM] */
    int    penalization;
    double C_eta;
    /* sponge [Sponge] */
    int    use_sponge;
    double C_sponge;
    double u_mean_set[3];
    /* time stepping [Time] */
    double CFL, CFL_nu, CFL_eta;
    double dt_fixed, dt_max;
    double time_max;
    double write_time;          /* fixed_time output trigger (<=0: off)       */
    double tsave_stats;         /* [Statistics] tsave_stats (<=0: off)        */
    /* coarsening indicator [Blocks] */
    double eps;
    int    eps_normalized;
    int    threshold_state_vector_component[8];
    /* GB300 build options */
    int    rhs_precision;       /* WG_RHS_FP64 or WG_RHS_FP32                  */
    int    reserved[14];
} wg_config;

typedef struct wg_ctx wg_ctx;

/* Fill *cfg with the reference defaults for a 2-D/3-D ACM run. */
int wg_config_defaults(wg_config *cfg, int dim);

#ifdef __cplusplus
}
#endif

#endif /* WABBIT_GB300_H */
