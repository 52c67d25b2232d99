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
#define WG_ETIMEOUT   -5   /* a bounded device wait gave up; the context is
                              unusable from then on (every call but
                              wg_ctx_destroy returns WG_ETIMEOUT)           */
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
    /* [Blocks] threshold_mask: blocks whose penalisation mask has an
     * interface stay (coarseningIndicatorMask_tree,
     * LIB/MESH/coarseningIndicator_tree.f90:333-420); needs a geometry
     * (wg_set_geometry) */
    int    threshold_mask;
    /* [Blocks] force_maxlevel_dealiasing: blocks on Jmax are flagged for
     * coarsening (coarseningIndicator_tree.f90:287-293) */
    int    force_maxlevel_dealiasing;
    /* [Blocks] useCoarseExtension (with useSecurityZone): the adaptation
     * takes the coarse-extension path of the lifted wavelets also for an
     * unlifted wavelet (ini_file_to_params.f90:543-546: the default is on
     * for lifted wavelets only); lifted wavelets always take it */
    int    use_coarse_extension;
    int    reserved[11];
} wg_config;

/*
 * Penalisation geometry of a tree: what the physics module draws in
 * createMask_tree -> CREATE_MASK_meta -> create_mask_2D_acm /
 * create_mask_3D_acm (LIB/MESH/createMask_tree.f90,
 * LIB/EQUATION/module_physics_metamodule.f90:38-83,
 * LIB/EQUATION/ACMnew/create_mask.f90:6-320) with the "all-parts" stage:
 * mask = 0 and colour = 1 everywhere, then the obstacle's chi (cosine step of
 * the signed distance over h = C_smooth * dx_min at Jmax,
 * module_ACM.f90:468-471) with colour 1, then, with use_sponge, the sponge
 * (LIB/EQUATION/ACMnew/sponge.f90). Keys in brackets are the .ini keys.
 */
#define WG_GEOM_NONE     0
#define WG_GEOM_CYLINDER 1   /* 2-D 'cylinder'/'circle' (draw_circle)         */
#define WG_GEOM_SPHERE   2   /* 3-D 'sphere-fixed' (draw_sphere)              */
#define WG_SPONGE_RECT   0   /* [Sponge] sponge_type=rect                     */
#define WG_SPONGE_PNORM  1   /* [Sponge] sponge_type=p-norm                   */
typedef struct wg_geometry {
    int    kind;                /* WG_GEOM_*  ([VPM] geometry)                 */
    int    sponge_type;         /* WG_SPONGE_*                                  */
    double x_cntr[3];           /* [VPM] x_cntr                                 */
    double R_cyl;               /* [VPM] R_cyl                                  */
    double C_smooth;            /* [VPM] C_smooth (default 1.5)                 */
    double L_sponge;            /* [Sponge] L_sponge                            */
    double p_sponge;            /* [Sponge] p_sponge (default 20)               */
    int    reserved[8];
} wg_geometry;

typedef struct wg_ctx wg_ctx;

/* Fill *cfg with the reference defaults for a 2-D/3-D ACM run
 * (ini_file_to_params.f90, READ_PARAMETERS_ACM module_ACM.f90:172-609). */
int wg_config_defaults(wg_config *cfg, int dim);

/* Message of the last failing call on this thread. */
const char *wg_last_error(void);

/* Device bytes one block slot needs (state, two RK stage buffers with
 * g_rhs ghosts, interior RK accumulator, descriptor). Replaces the memory
 * estimate of allocate_forest (LIB/MESH/allocate_forest.f90:122-147). */
size_t wg_bytes_per_block(const wg_config *cfg);

/* ---- context: a device arena for one block geometry -------------------
 * Replaces allocate_forest / deallocate_forest
 * (LIB/MESH/allocate_forest.f90:1-381): all heavy data lives in HBM for the
 * lifetime of the context; max_blocks is the arena size. */
int wg_ctx_create(const wg_config *cfg, int max_blocks, wg_ctx **ctx);
int wg_ctx_destroy(wg_ctx *ctx);
/* 1: FMA stencil (default); 0: strict reference arithmetic (no FMA). */
int wg_set_variant(wg_ctx *ctx, int fast);
/* Form of the FP32-pipe stage kernel (no counterpart in the reference, whose
 * RHS is a per-block loop): WG_FORM_AUTO (default) times, for each of the
 * four RK stages, the forms that apply before the first step of a context
 * and keeps the fastest per stage; WG_FORM_DIRECT reads the stencil from
 * global memory; WG_FORM_TILE stages 4-plane slabs of a block in shared
 * memory by TMA (3-D, 16x16 planes, g_rhs = 2); WG_FORM_MARCH walks a whole
 * 16^3 block through a ring of 5 planes loaded by TMA; WG_FORM_PIPE is the
 * tile form as a persistent kernel (one CTA per SM walking its slabs with
 * two slab buffers, the next slab loading while one is computed);
 * WG_FORM_TILE2 / WG_FORM_TILE8 are the tile form with slabs of 2 / 8
 * planes. The forms compute the same bits. wg_get_stage_form
 * returns the form of stage 2, wg_get_stage_forms the forms of stages 1-4
 * (the autotuner's choices once it has run). */
#define WG_FORM_AUTO 0
#define WG_FORM_DIRECT 1
#define WG_FORM_TILE 2
#define WG_FORM_MARCH 3
#define WG_FORM_PIPE 4
#define WG_FORM_TILE2 5   /* the tile form with slabs of 2 interior planes  */
#define WG_FORM_TILE8 6   /* ... of 8 interior planes (Bs2 a multiple of 8)  */
int wg_set_stage_form(wg_ctx *ctx, int form);
int wg_get_stage_form(wg_ctx *ctx, int *form);
int wg_get_stage_forms(wg_ctx *ctx, int *forms);
/* Fixes the forms of RK stages 1-4 (each WG_FORM_DIRECT, _TILE, _MARCH, _PIPE, _TILE2 or _TILE8),
 * e.g. to reuse the autotuner's choice of one context in another. */
int wg_set_stage_forms(wg_ctx *ctx, const int *forms);
int wg_synchronize(wg_ctx *ctx);
/* the context's CUDA stream (cudaStream_t) */
void *wg_stream(wg_ctx *ctx);

/* ---- trees: independent solves in one arena (the reference's tree_ID) -- */
int wg_tree_create(wg_ctx *ctx, const wg_config *cfg, int *tree);
int wg_tree_destroy(wg_ctx *ctx, int tree);

/* Set the grid of a tree: level[nblk], coords[3*nblk] (see top of file).
 * Runs the neighbour search (find_neighbor, LIB/MESH/find_neighbors.f90:18)
 * and rejects grids that are not complete, periodic and graded. The state
 * of the new blocks is undefined until wg_upload_state. */
int wg_set_grid(wg_ctx *ctx, int tree, int nblk, const int *level, const int *coords);
int wg_get_nblocks(wg_ctx *ctx, int tree, int *nblk);
int wg_get_grid(wg_ctx *ctx, int tree, int cap, int *level, int *coords);

/* Heavy data in the reference block layout (hvy_block, see top of file). */
int wg_upload_state(wg_ctx *ctx, int tree, const double *host_blocks);
int wg_download_state(wg_ctx *ctx, int tree, double *host_blocks);
/* Interior points only, compact (nblk, neq, Bz, By, Bx) x fastest: one
 * contiguous copy each way; ghost nodes are refilled by the next sync. The
 * array may be host memory (pageable or pinned) or device memory of the
 * context's GPU (unified addressing picks the copy direction). */
int wg_upload_interior(wg_ctx *ctx, int tree, const double *host);
int wg_download_interior(wg_ctx *ctx, int tree, double *host);
/* nsteps RK4 steps with host buffers: for step k the interior state is set
 * from ins[k], one step is taken (as wg_rk4_step) and the interior result is
 * written to outs[k]. With page-locked buffers the copy of step k+1's input
 * and of step k's result run while step k / k+1 compute (five device
 * staging buffers of the interior size: three inputs, two results). Returns
 * after the last result is on the host; the context's state then holds the
 * last step's result. */
int wg_rk4_stream(wg_ctx *ctx, int tree, int nsteps, const double *const *ins, double *const *outs);
/* Penalisation mask in the layout of hvy_mask (..., 1:6, Nb): chi, usx,
 * usy, usz, colour, sponge (createMask_tree, LIB/MESH/createMask_tree.f90);
 * NULL removes it. Only blocks with a non-zero mask keep a device copy. */
int wg_set_mask(wg_ctx *ctx, int tree, const double *host_mask);
/* Same for the n listed blocks only (mask holds n*6*npts doubles); every
 * other block has chi = 0. */
int wg_set_mask_sparse(wg_ctx *ctx, int tree, int n, const int *blocks, const double *mask);
/* Mask of a fixed sphere (centre[3], radius) computed on the device for a
 * 3-D tree (create_mask_3D_acm 'sphere-fixed' -> draw_sphere,
 * LIB/EQUATION/ACMnew/create_mask.f90:58-61,
 * LIB/EQUATION/insects/module_geometry.f90:49-117): chi is the cosine step
 * of the signed distance over h = c_smooth * dx at Jmax, colour 1, u_s = 0;
 * only blocks with chi > 0 at an interior point keep a mask. */
int wg_set_mask_sphere(wg_ctx *ctx, int tree, const double *centre, double radius, double c_smooth);
/* Penalisation geometry of a tree (see wg_geometry); NULL removes it. The
 * tree then draws its masks itself, as the reference's createMask_tree does
 * in every RHS and adaptation: now, and after every grid change
 * (wg_set_grid, wg_refine_everywhere, wg_adapt), on the host from the
 * block geometry, keeping device copies only for blocks with a non-zero
 * chi or sponge word. The same geometry supplies wg_adapt's threshold_mask
 * test. wg_set_mask, wg_set_mask_sparse and wg_set_mask_sphere replace it
 * by the caller's masks. Replaces createMask_tree
 * (LIB/MESH/createMask_tree.f90:1-136) for 'cylinder' (2-D) and
 * 'sphere-fixed' (3-D) with the 'rect' and 'p-norm' sponges. */
int wg_set_geometry(wg_ctx *ctx, int tree, const wg_geometry *geo);
/* Interior mask of one block (6 * Bs^d doubles) for inspection: returns 1
 * and fills out if the block has a mask, 0 if it has none. */
int wg_get_mask_block(wg_ctx *ctx, int tree, int block, double *out);

int wg_set_time(wg_ctx *ctx, int tree, double time);
int wg_get_time(wg_ctx *ctx, int tree, double *time, double *dt);

/* adapt_tree (LIB/MESH/adapt_tree.f90:11-255): full tree with every
 * ancestor down to Jmin, mothers filled with their daughters' scaling
 * coefficients (sync_D2M), coarsening indicator on every block
 * (WG_ADAPT_THRESHOLD: threshold-state-vector with eps_use = eps * norm per
 * component; eps_use NULL takes cfg.eps, times the leaves' Linfty norm per
 * component with eps_normalized as componentWiseNorm_tree gives it;
 * WG_ADAPT_EVERYWHERE: every leaf), force_maxlevel_dealiasing and
 * threshold_mask as configured, respectJmaxJmin, completeness,
 * gradedness (ensureGradedness_tree with check_daughters), deletion and
 * pruning; the grid and the state are replaced, *nblk_out receives the new
 * block count (wg_get_grid returns the new grid). Masks are redrawn from the
 * tree's geometry (wg_set_geometry), else dropped. Needs
 * free arena slots for the mothers (about nblk/(2^d-1)).
 * Unlifted wavelets (CDF X0) without use_coarse_extension: the original
 * values are kept (decimation). Lifted wavelets (CDF XY), or any wavelet
 * with use_coarse_extension: the reference's coarse-extension algorithm --
 * filtered ghost sync, level-by-level FWT of the full tree
 * (wavelet_decompose_full_tree), coarse extension, the indicator on the
 * decomposition, the security zone (addSecurityZone_CE_tree), and the
 * reconstruction of the blocks at coarse/fine interfaces
 * (wavelet_reconstruct_full_tree_CEoptimized), then a filtered ghost sync of
 * the new grid. It allocates, on first use, a second block arena of the size
 * of the state (hvy_tmp). */
#define WG_ADAPT_THRESHOLD 0
#define WG_ADAPT_EVERYWHERE 1
int wg_adapt(wg_ctx *ctx, int tree, const double *eps_use, int indicator, int *nblk_out);
/* The refinement status the last adaptation left on the tree's blocks
 * (lgt_block(:, IDX_REFINE_STS) after adapt_tree): 0 for a block the
 * indicator (or the security zone) kept, 9 (REF_UNSIGNIFICANT_STAY,
 * LIB/MODULE/module_globals.f90:28) for a block kept only for completeness,
 * gradedness or Jmin. Writes min(cap, nblk) values in block order and
 * returns the block count; WG_EINVAL if the grid changed otherwise since. */
int wg_get_refinement_status(wg_ctx *ctx, int tree, int cap, int *status);
/* Sets that status for the tree's current blocks (nblk values in block
 * order), as a run restarted from a field file reads it with its grid
 * (readHDF5vct_tree(..., read_refinement_status), LIB/MESH/InputOutput.f90:
 * 322); each value must be 0 or 9. */
int wg_set_refinement_status(wg_ctx *ctx, int tree, int nblk, const int *status);
/* Phase times of the last lifted adaptation in ms: [0] host planning, [1]
 * ghost syncs, [2] FWT, [3] coarse extension and D2M copies, [4] indicator and
 * security zone, [5] IWT, [6] hvy_tmp block copies, [7] total. enable 1 / 0
 * switches timing on / off for later calls (it synchronises the stream at
 * every phase boundary), -1 leaves it; ms_out may be NULL. */
int wg_adapt_profile(wg_ctx *ctx, int enable, double *ms_out, int n);
/* One-level wavelet transforms of every block of the tree, in place on the
 * state (interior points; the ghost nodes must be synchronised first, for the
 * inverse with the decomposed data):
 *   wg_wavelet_decompose   -- waveletDecomposition_optimized_block
 *     (LIB/WAVELETS/wavelet_decomposition_reconstruction.f90:23-389), result
 *     in spaghetti order (SC at even interior offsets)
 *   wg_wavelet_reconstruct -- waveletReconstruction_optimized_block
 *     (wavelet_decomposition_reconstruction.f90:426-840)
 *   wg_wavelet_threshold   -- wc_threshold_tree (LIB/MESH/adapt_tree.f90:
 *     1091-1180) on decomposed data: thresh holds neq values */
int wg_wavelet_decompose(wg_ctx *ctx, int tree);
int wg_wavelet_reconstruct(wg_ctx *ctx, int tree);
int wg_wavelet_threshold(wg_ctx *ctx, int tree, const double *thresh);
/* ---- the hot path ------------------------------------------------------ */
/* sync_ghosts_RHS_tree / sync_ghosts_tree without the HD filter
 * (LIB/MPI/synchronize_ghosts_generic.f90:121-174): fill gminus/gplus ghost
 * layers of every block by copy, restriction and prediction. */
int wg_sync_ghosts(wg_ctx *ctx, int tree, int gminus, int gplus);
/* RHS_ACM "local_stage" of every block (LIB/EQUATION/ACMnew/rhs_ACM.f90:7;
 * plugin entry RHS_META, LIB/EQUATION/module_physics_metamodule.f90:268)
 * on the current synchronised state; host_rhs in the hvy_block layout. */
int wg_rhs(wg_ctx *ctx, int tree, double *host_rhs);
/* calculate_time_step + GET_DT_BLOCK_ACM (LIB/TIME/calculate_time_step.f90:2,
 * LIB/EQUATION/ACMnew/module_ACM.f90:617) at the tree's current time. */
int wg_compute_dt(wg_ctx *ctx, int tree, double *dt);
/* timeStep_tree -> RungeKuttaGeneric, default RK4 tableau
 * (LIB/TIME/timeStep_tree.f90:1, LIB/TIME/runge_kutta_generic.f90:1):
 * sync, dt, four stages; the tree's time advances on the device. */
int wg_rk4_step(wg_ctx *ctx, int tree, double *time, double *dt);
/* nsteps RK4 steps of each listed tree, asynchronous; use_graph captures the
 * launch sequence of one step of all trees in a CUDA graph and replays it. */
int wg_run(wg_ctx *ctx, int ntrees, const int *trees, int nsteps, int use_graph);
/* coarseningIndicator_tree -> coarseningIndicator_block -> threshold_block
 * (LIB/MESH/coarseningIndicator_tree.f90:4,
 *  LIB/INDICATORS/threshold_block.f90:1): one-level FWT of every block and
 * detail thresholding; flags[b] = -1 (may coarsen) or 0. eps_use holds the
 * per-component threshold (eps * norm). Ghosts must hold g synced layers. */
int wg_threshold_flags(wg_ctx *ctx, int tree, const double *eps_use, int *flags, double *details);
/* The same flags from a state that already holds the one-level decomposition
 * (wg_wavelet_decompose): coarseningIndicator_tree(..., input_is_WD=.true.)
 * (LIB/MESH/coarseningIndicator_tree.f90:4), no second transform. */
int wg_threshold_flags_wd(wg_ctx *ctx, int tree, const double *eps_use, int *flags, double *details);
/* Allocation-free variant of wg_threshold_flags, for callers that may not
 * allocate device memory while they run (e.g. a host code with its own
 * memory pool or an externally enforced device-memory budget). It has no
 * counterpart in the reference. It takes no context: d_blocks points to nblk
 * blocks on the device in the hvy_block layout with g synced ghost layers,
 * contiguous; eps_use (host, neq values) holds the per-component threshold;
 * d_flags (device, nblk ints) and d_details (device, nblk*neq doubles, or
 * NULL) receive the result on `stream` (a cudaStream_t, NULL = default).
 * Its scratch is a file-scope static device array sized for at most 16384
 * blocks and 8 components (~1.2 MB, held by every device that loads the
 * library until exit); larger calls are rejected with WG_EINVAL. The first
 * call on a device resolves the scratch address (cudaGetSymbolAddress) and
 * fills a block list, synchronising that stream once, so make it before any
 * stream capture. All calls share the scratch: calls whose work overlaps on
 * the GPU race. */
int wg_threshold_flags_noalloc(const wg_config *cfg, int nblk, const double *d_blocks, const double *eps_use,
                               int *d_flags, double *d_details, void *stream);
/* refine_tree(..., "everywhere") data part: refineBlock for every block
 * below Jmax (LIB/MESH/refinementExecute.f90:4-116; blocks on Jmax stay,
 * respectJmaxJmin_tree). In the new block order each refined block is
 * replaced, at its position, by its 2^d daughters (digit order y, x, z).
 * Ghosts must hold g synced layers. */
int wg_refine_everywhere(wg_ctx *ctx, int tree);
/* refine_tree(..., "significant") (LIB/MESH/refine_tree.f90:1-100): the
 * blocks whose status from the last adaptation is 0 refine (the status
 * translation of refinementIndicator_tree.f90:152-167), those on Jmax stay
 * (respectJmaxJmin_tree), and a block next to a finer block that refines
 * refines as well (ensureGradedness_tree.f90), then refineBlock for them;
 * the others keep their place. The new block order is that of
 * wg_refine_everywhere. WG_EINVAL if no adaptation set the status. */
int wg_refine_significant(wg_ctx *ctx, int tree);

/* ---- measurement -------------------------------------------------------- */
/* Mean device time (ms) of one launch over reps launches, CUDA events on the
 * context stream: which = 0 RK-stage kernel, 1 RHS ghost sync, 2 dt. */
int wg_time_kernel(wg_ctx *ctx, int tree, int which, int reps, double *ms_per_launch);
/* nsteps RK4 steps of the listed trees (the launches of wg_run without a
 * graph), one step at a time with CUDA events between the kernel groups;
 * ms[9] receives the mean device time (ms) per step of the ghost sync before
 * stages 1-4 (ms[0..3]), the dt reduction (ms[4]) and the stage kernels of
 * stages 1-4 (ms[5..8]). The state advances by nsteps steps. No counterpart
 * in the reference (its toc timers, LIB/TIMING/module_timing.f90:76-127,
 * time the same phases on the host). */
int wg_step_profile(wg_ctx *ctx, int ntrees, const int *trees, int nsteps, double *ms);
int wg_tree_stats(wg_ctx *ctx, int tree, int *nblocks, int *nmasked);
/* kernel nodes in the captured RK4-step graph of the last wg_run(.., 1) */
int wg_graph_kernels(wg_ctx *ctx);

/* ---- inspection (tests, tooling) --------------------------------------- */
/* ghost-patch table: returns the patch count; out receives 19 ints per
 * patch: src, dst, op, stage, rlo[3], rhi[3], slo[3], shi[3], blo[3] */
int wg_sync_table(wg_ctx *ctx, int tree, int gminus, int gplus, int thin, int cap, int *out);
int wg_block_slot(wg_ctx *ctx, int tree, int b);
/* the same table computed on the host alone (no device needed), with block
 * indices in place of arena slots; thin != 0 gives the g_rhs-ghost layout */
int wg_sync_table_host(const wg_config *cfg, int nblk, const int *level, const int *coords, int gminus,
                       int gplus, int thin, int cap, int *out);

#ifdef __cplusplus
}
#endif

#endif /* WABBIT_GB300_H */
