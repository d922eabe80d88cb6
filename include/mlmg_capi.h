/*
 * mlmg_capi.h -- C ABI of the GB300-native MLMG cell-centred solver.
 *
 * Drop-in boundary for AMReX's MLMG path (MLPoisson / MLABecLaplacian on
 * MultiFab data).  The entry points mirror the reference's own C ABI for
 * this path -- the Fortran-interface layer Src/F_Interfaces/ (files below are
 * relative to the AMReX source tree) -- with opaque handles, caller-owned
 * handle arrays, LinOpBCType codes (101 Dirichlet, 102 Neumann, 103
 * reflect_odd, 200 periodic) and an int status instead of amrex::Abort:
 *
 *    0  converged / ok            1  not converged within max_iter
 *   -1  bad argument or handle   -2  residual blew up (> 1e20 * norm)
 *   -3  CUDA error               -4  unsupported request
 *   -5  NaN/Inf in the residual  -6  internal error   -7  device wait timed out
 *
 * mlmg_last_error() returns the message of the last failing call on the
 * calling thread.  Handles are not thread-safe; distinct solver handles may
 * be used from distinct host threads.  Every call returns after its device
 * work has completed (like the reference, which synchronises its stream after
 * every Fsmooth/Fapply).
 *
 * Data layout of a MultiFab box (FAB): the box grown by ngrow (plus one cell
 * in the nodal direction of a face MultiFab), x fastest, then y, z, then
 * component -- the layout of amrex::BaseFab (Src/Base/AMReX_Array4.H:60-100).
 */
#ifndef MLMG_CAPI_H_
#define MLMG_CAPI_H_

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif
#if defined(__GNUC__)
#pragma GCC visibility push(default)
#endif

typedef struct mlmg_boxarray_s* mlmg_boxarray;
typedef struct mlmg_distromap_s* mlmg_distromap;
typedef struct mlmg_geometry_s* mlmg_geometry;
typedef struct mlmg_multifab_s* mlmg_multifab;
typedef struct mlmg_linop_s* mlmg_linop;
typedef struct mlmg_solver_s* mlmg_solver;

/* LPInfo (Src/LinearSolvers/MLMG/AMReX_MLLinOp.H:34-83).  agg/con grid size
 * <= 0 selects the reference's GPU-build default (32). */
typedef struct {
    int agglomeration;
    int consolidation;
    int agg_grid_size;
    int con_grid_size;
    int max_coarsening_level;
} mlmg_lpinfo;

/* ------------------------------------------------------------ library ---- */
const char* mlmg_last_error(void);
int mlmg_version(void);
/* the CUDA stream the library works on (a cudaStream_t) */
void* mlmg_stream(void);
/* number of kernels this library has launched since the last reset */
long long mlmg_kernel_launches(int reset);
/* the device's FP64 FMA throughput in TFLOP/s (2 FLOPs per FMA), measured by
 * one register-resident kernel (8 independent FMA chains per thread, eight
 * 256-thread blocks per SM) timed with CUDA events on the library stream after
 * a warm-up launch: the FP64 roofline of the outer residual.  Changes no
 * device setting. */
int mlmg_fp64_fma_rate(double* tflops);
/* the FP64-bound kernels convert FP32 <-> FP64 and take |x| by integer bit
 * assembly; this compares those results with the hardware's on n device cases
 * (edge values, random bit patterns, halfway points between floats,
 * subnormals): mismatches[0..2] = cases that differ for FP64 -> FP32, FP32 ->
 * FP64 and |x| (0 expected); first_bad (may be null) = an input of each kind
 * that differed (FP32 inputs with bit 32 set; 0 when none) */
int mlmg_check_bit_conversions(long long n, unsigned long long seed, long long mismatches[3],
                               unsigned long long first_bad[3]);

/* ----------------------------------------------------------- BoxArray ----
 * replaces amrex_fi_new_boxarray / amrex_fi_boxarray_maxsize / ..._get_box
 * (Src/F_Interfaces/Base/AMReX_boxarray_fi.cpp:10,16,44) */
int mlmg_boxarray_new(const int* boxes, int nbox, mlmg_boxarray* out);  /* boxes: lo[3],hi[3] per box */
int mlmg_boxarray_new_domain(const int lo[3], const int hi[3], mlmg_boxarray* out);  /* BoxArray(const Box&) */
int mlmg_boxarray_maxsize(mlmg_boxarray ba, const int chunk[3]);       /* BoxArray::maxSize */
int mlmg_boxarray_size(mlmg_boxarray ba);
int mlmg_boxarray_get(mlmg_boxarray ba, int i, int lo[3], int hi[3]);
int mlmg_boxarray_delete(mlmg_boxarray ba);

/* ------------------------------------------------ DistributionMapping ----
 * replaces amrex_fi_new_distromap (Src/F_Interfaces/Base/AMReX_distromap_fi.cpp:9,14);
 * one GPU: every box is local */
int mlmg_distromap_new(mlmg_boxarray ba, mlmg_distromap* out);
int mlmg_distromap_delete(mlmg_distromap dm);

/* ----------------------------------------------------------- Geometry ----
 * replaces amrex_fi_new_geometry (Src/F_Interfaces/Base/AMReX_geometry_fi.cpp:7) */
int mlmg_geometry_new(const int lo[3], const int hi[3], const double prob_lo[3], const double prob_hi[3],
                      const int is_periodic[3], mlmg_geometry* out);
int mlmg_geometry_delete(mlmg_geometry g);

/* ----------------------------------------------------------- MultiFab ----
 * replaces amrex_fi_new_multifab (Src/F_Interfaces/Base/AMReX_multifab_fi.cpp:10).
 * nodal_dir: -1 cell-centred, 0..2 face-centred; precision: 8 (double) or 4 (float) */
int mlmg_multifab_new(mlmg_boxarray ba, mlmg_distromap dm, int ncomp, int ngrow, int nodal_dir, int precision,
                      mlmg_multifab* out);
int mlmg_multifab_delete(mlmg_multifab mf);
/* FAB of box i: element count, device pointer */
int mlmg_multifab_fab_size(mlmg_multifab mf, int box, size_t* nelem);
int mlmg_multifab_fab_ptr(mlmg_multifab mf, int box, void** dptr);
/* copy one FAB (box grown by ngrow) from / to host memory */
int mlmg_multifab_upload(mlmg_multifab mf, int box, const void* host);
int mlmg_multifab_download(mlmg_multifab mf, int box, void* host);
/* copy a whole-domain host array (x fastest; lower corner glo, extents gn)
 * into every box's cells (ghosts included where the array covers them) or
 * out of every box's valid cells -- one host<->device copy and one kernel */
int mlmg_multifab_upload_global(mlmg_multifab mf, const void* host, const int glo[3], const int gn[3]);
int mlmg_multifab_download_global(mlmg_multifab mf, void* host, const int glo[3], const int gn[3]);
int mlmg_multifab_setval(mlmg_multifab mf, double v);                    /* FabArray::setVal, ghosts included;
                                                                          * stream-ordered, returns without waiting */
/* FabArray::FillBoundary (Src/Base/AMReX_FabArray.H:1000-1044), one rank */
int mlmg_multifab_fill_boundary(mlmg_multifab mf, mlmg_geometry geom, int cross);
int mlmg_multifab_norminf(mlmg_multifab mf, double* out);                /* valid cells */
/* Same result as mlmg_multifab_norminf, for callers that must not allocate
 * device memory: a caller whose device memory is already fully claimed by its
 * own allocator (a framework's caching allocator holding the HBM), or a time-
 * step loop where a cudaMalloc/cudaFree -- which can synchronise the whole
 * device -- is not acceptable.  No counterpart in the reference.  The call
 * allocates nothing: its scratch (box table and result word) is a static
 * device array of 131,584 bytes that every GPU loading the library keeps
 * until the process exits.  At most 4096 boxes (more returns -1 with a
 * message).  The MultiFab's device (the one current when it was made) must
 * be current (-1 otherwise); the library keeps one stream per device and
 * the call runs on that device's.  The first call on a device looks up that
 * array's device address with the device current; make that first call
 * before any stream capture.
 * Every call shares the array, which keeps the last call's contents; each
 * call clears the result word before use, and calls that overlap on the GPU
 * race (calls through this library are serialised by a lock). */
int mlmg_multifab_norminf_noalloc(mlmg_multifab mf, double* out);

/* ------------------------------------------------- linear operators -----
 * replace amrex_fi_new_poisson (Src/F_Interfaces/LinearSolvers/AMReX_poisson_fi.cpp:8-30)
 * and amrex_fi_new_abeclaplacian (AMReX_abeclaplacian_fi.cpp:8-49).  geom, ba
 * and dm hold nlev entries, one per AMR level (MLPoissonT(Vector<Geometry>,
 * Vector<BoxArray>, ...), AMReX_MLPoisson.H:21-40).  nlev > 1 (a composite
 * solve, up to 8 levels) is implemented for MLPoisson and MLABecLaplacian
 * with refinement ratio 2, periodic or not: level l's domain is level 0's
 * refined by 2^l (same periodicity), its boxes coarsen by 2 and nest properly
 * in level l-1 (a box coarsened and grown by one cell stays in level l-1, its
 * periodic images included, or outside the domain).  MLABecLaplacian takes a and b per AMR level (amrlev of the
 * coefficient setters); the solve averages each finer level's a and b onto
 * the next coarser level before restricting them to level 0's MG levels
 * (MLABecLaplacianT::averageDownCoeffs, AMReX_MLABecLaplacian.H:610-712). */
int mlmg_linop_new_poisson(int nlev, const mlmg_geometry* geom, const mlmg_boxarray* ba, const mlmg_distromap* dm,
                           const mlmg_lpinfo* info, mlmg_linop* out);
int mlmg_linop_new_abeclap(int nlev, const mlmg_geometry* geom, const mlmg_boxarray* ba, const mlmg_distromap* dm,
                           const mlmg_lpinfo* info, mlmg_linop* out);
int mlmg_linop_delete(mlmg_linop op);
/* amrex_fi_linop_set_domain_bc / _level_bc / _maxorder (AMReX_linop_fi.cpp:8-40) */
int mlmg_linop_set_domain_bc(mlmg_linop op, const int lobc[3], const int hibc[3]);
/* the Dirichlet values of AMR level amrlev in its ghost cells (taken at this
 * call); NULL: homogeneous */
int mlmg_linop_set_level_bc(mlmg_linop op, int amrlev, mlmg_multifab levelbc);
int mlmg_linop_set_maxorder(mlmg_linop op, int maxorder);
/* MLLinOpT::setCoarseFineBC(crse, crse_ratio) (AMReX_MLLinOp.H:200-211,
 * 1427-1441) and amrex_fi_linop_set_coarse_fine_bc (AMReX_linop_fi.cpp:31-34):
 * a single-level operator whose boxes do not cover its domain (a fine AMR
 * level solved on its own) takes, on its coarse/fine faces, Dirichlet values
 * at 0.5 * crse_ratio * dx interpolated (InterpBndryData, third order) from
 * crse, a cell-centred MultiFab over the domain coarsened by crse_ratio.  The
 * values are taken at this call (the reference reads them at setLevelBC,
 * which is called after this).  Without it such a level's coarse/fine values
 * are zero and located on the face itself, as in the reference.  crse_ratio
 * 2 only (-4 otherwise); crse NULL clears it; -4 on a composite operator. */
int mlmg_linop_set_coarse_fine_bc(mlmg_linop op, mlmg_multifab crse, int crse_ratio);
/* amrex_fi_abeclap_set_scalars / _acoeffs / _bcoeffs (AMReX_abeclaplacian_fi.cpp:20-49);
 * amrlev in 0..nlev-1, the MultiFabs on that level's BoxArray; a level whose
 * a or b is never set takes 1 */
int mlmg_abeclap_set_scalars(mlmg_linop op, double alpha, double beta);
int mlmg_abeclap_set_acoeffs(mlmg_linop op, int amrlev, mlmg_multifab a);
int mlmg_abeclap_set_acoeffs_const(mlmg_linop op, int amrlev, double a);
int mlmg_abeclap_set_bcoeffs(mlmg_linop op, int amrlev, const mlmg_multifab b[3]);
int mlmg_abeclap_set_bcoeffs_const(mlmg_linop op, int amrlev, double b);
/* number of MG levels of AMR level 0 (built from the LPInfo) */
int mlmg_linop_num_mg_levels(mlmg_linop op);
/* number of AMR levels (MLLinOpT::NAMRLevels, AMReX_MLLinOp.H:309) */
int mlmg_linop_num_amr_levels(mlmg_linop op);

/* ------------------------------------------------------------- solver ----
 * replace amrex_fi_new_multigrid / amrex_fi_multigrid_solve / setters
 * (Src/F_Interfaces/LinearSolvers/AMReX_multigrid_fi.cpp:8-112), with the
 * setters of MLMGT (Src/LinearSolvers/MLMG/AMReX_MLMG.H:116-142) */
int mlmg_new(mlmg_linop op, mlmg_solver* out);
int mlmg_delete(mlmg_solver s);
int mlmg_set_verbose(mlmg_solver s, int v);
int mlmg_set_max_iter(mlmg_solver s, int n);
int mlmg_set_max_fmg_iter(mlmg_solver s, int n);        /* F-cycles for the first n iterations */
int mlmg_set_fixed_iter(mlmg_solver s, int n);
int mlmg_set_pre_smooth(mlmg_solver s, int n);
int mlmg_set_post_smooth(mlmg_solver s, int n);
int mlmg_set_final_smooth(mlmg_solver s, int n);
int mlmg_set_bottom_smooth(mlmg_solver s, int n);
/* MLMG::BottomSolver codes (AMReX_MLLinOp.H:30-31; amrex_fi_multigrid_set_bottom_solver,
 * AMReX_multigrid_fi.cpp:82-97): 0 default (bicgstab), 1 smoother, 2 bicgstab, 3 cg,
 * 4 bicgcg, 5 cgbicg (the second solver runs when the first fails and, once it
 * succeeds, replaces it for later bottom solves, as MLMGT::actualBottomSolve
 * does); 6 hypre and 7 petsc return -4 */
int mlmg_set_bottom_solver(mlmg_solver s, int which);
int mlmg_set_bottom_max_iter(mlmg_solver s, int n);
int mlmg_set_bottom_tolerance(mlmg_solver s, double t);
int mlmg_set_bottom_tolerance_abs(mlmg_solver s, double t);
int mlmg_set_always_use_bnorm(mlmg_solver s, int flag);
/* MLMGT::setFinalFillBC (AMReX_MLMG.H:137, 515-524) and
 * amrex_fi_multigrid_set_final_fill_bc (AMReX_multigrid_fi.cpp:109-112): a
 * solution MultiFab with more than one ghost layer also receives the first
 * ghost layer the solve's last residual evaluation filled (neighbouring boxes'
 * values and boundary closures); a one-ghost solution always does. */
int mlmg_set_final_fill_bc(mlmg_solver s, int flag);
/* GB300 additions: 0 = FP64 throughout, 1 = FP32 V-cycles inside FP64
 * iterative refinement (residual, update, bottom solve and norms in FP64) */
int mlmg_set_precision(mlmg_solver s, int mode);
int mlmg_set_graph(mlmg_solver s, int on);               /* replay each iteration as a CUDA graph */
int mlmg_set_fused_smoother(mlmg_solver s, int on);      /* fused two-colour Gauss-Seidel sweeps */
/* engine tuning knobs by name: "coarse_block" (0/1: run the coarse levels of
 * each V-cycle in one thread block per solve), "coarse_cells" (a level is
 * coarse when every solve has at most this many cells on it),
 * "merge_boxes" (0/1), "march_sweep" (0/1: fused sweeps by the z-marching
 * kernel), "march_min_tiles" (levels with fewer marching tiles use the tiled
 * fused sweep), "march_tz" (planes per z-slab of the marching sweep),
 * "fused_tma" (0/1: the tiled fused sweep stages each tile by one TMA tensor
 * load, else by 16-byte cp.async copies; default 1), "fused_prefetch" (0/1:
 * ... and prefetches the tile's rhs and stencil boxes into L2, default 1),
 * "tma_wait_limit" (polls of the tiled TMA sweep's bounded wait for its tile;
 * -1 the default bound; 0 makes every wait expire -- a test of the failure
 * path: each block then waits, with the full bound, for its own copy, leaves,
 * and the solve returns -7; the next solve with the default works);
 * "pdl" (0/1: V-cycle and composite-path kernels as programmatic dependent
 * launches, default 1), "fused_fine" (0/1/2: AMR fine levels smoothed by
 * colour passes per level / fused sweeps where the tile allows them, the
 * default / colour passes on every tile), "fused_restrict" (0/1: the
 * correction residual and its restriction on TMA-swept levels in one tile
 * kernel, default 1); -4 for an unknown name */
int mlmg_set_option(mlmg_solver s, const char* name, double value);
/* time every finest-level smoother launch and every FP64 outer residual of
 * the mixed path with CUDA events on the library stream (graph replays
 * included); the stats accumulate until reset */
int mlmg_set_time_kernels(mlmg_solver s, int on);
int mlmg_get_smoother_stats(mlmg_solver s, double* total_ms, long long* launches, double* bytes_per_launch,
                            int reset);
/* the FP64 outer residual of the mixed path (with the correction update where
 * it is fused): total ms, launches, algorithmic bytes and FP64 operations
 * (an FMA counts 2) per launch */
int mlmg_get_residual_stats(mlmg_solver s, double* total_ms, long long* launches, double* bytes_per_launch,
                            double* flops_per_launch, int reset);

/* MLMGT::solve (AMReX_MLMG.H:44-51): sol holds the initial guess, rhs the
 * right-hand side; returns a status, final_resid gets the final max-norm */
int mlmg_solve(mlmg_solver s, mlmg_multifab sol, mlmg_multifab rhs, double tol_rel, double tol_abs,
               double* final_resid);
/* MLMGT::solve(Vector<MultiFab*>, Vector<MultiFab const*>, ...) (AMReX_MLMG.H:
 * 353-541) and amrex_fi_multigrid_solve (AMReX_multigrid_fi.cpp:40-50): sol
 * and rhs hold one MultiFab per AMR level of the operator, on the level's
 * BoxArray.  The composite solve iterates MLMGT::oneIter over the levels and
 * converges when the finest level's residual and then the masked residual of
 * the coarser levels reach the target; final_resid gets the composite
 * max-norm.  With one level this is mlmg_solve.  The single-level calls
 * (mlmg_solve, mlmg_apply, fluxes, adjoint, autotune, batching) return -4 on
 * a composite operator. */
int mlmg_solve_levels(mlmg_solver s, const mlmg_multifab* sol, const mlmg_multifab* rhs, double tol_rel,
                      double tol_abs, double* final_resid);
/* MLMGT::compResidual (AMReX_MLMG.H:790-856) and
 * amrex_fi_multigrid_comp_residual (AMReX_multigrid_fi.cpp:53-60): res, sol
 * and rhs hold one MultiFab per AMR level; res = rhs - L(sol) with the level
 * BC values (fine levels: coarse/fine values from the next coarser sol), the
 * finer level's fluxes refluxed and its residual averaged down onto the cells
 * it covers, in the reference's FP64 operation order.  Unlike the reference
 * (whose one-ghost sol is filled in place), sol is not modified. */
int mlmg_comp_residual(mlmg_solver s, const mlmg_multifab* res, const mlmg_multifab* sol, const mlmg_multifab* rhs);
/* MLMGT::apply (AMReX_MLMG.H:858-932): out = L(in) with the level BC values */
int mlmg_apply(mlmg_solver s, mlmg_multifab out, mlmg_multifab in);
/* MLMGT::getFluxes(a_flux, a_sol, loc) (AMReX_MLMG.H:627-655) and
 * MLMGT::getGradSolution (AMReX_MLMG.H:553-572): face-centred FP64 MultiFabs
 * flux[3] / grad[3] (entries may be NULL) of the solution sol, whose ghost
 * values come from the operator's boundary conditions and level BC values.
 * flux = -b dphi/dn (MLABecLaplacian, after the 1/beta scaling of
 * MLCellABecLapT::getFluxes) or -dphi/dn (MLPoisson); grad = dphi/dn.  The
 * reference's variants read the solver's internal solution; here the
 * solution is passed explicitly (the one given to mlmg_solve). */
int mlmg_get_fluxes(mlmg_solver s, mlmg_multifab sol, const mlmg_multifab* flux);
int mlmg_get_grad_solution(mlmg_solver s, mlmg_multifab sol, const mlmg_multifab* grad);
/* getters (AMReX_MLMG.H:220-228) and the device time of the last solve */
int mlmg_get_num_iters(mlmg_solver s);
int mlmg_get_residual_history(mlmg_solver s, double* out, int max);
int mlmg_get_num_cg_iters(mlmg_solver s, int* out, int max);
double mlmg_get_init_residual(mlmg_solver s);
double mlmg_get_final_residual(mlmg_solver s);
double mlmg_get_init_rhs(mlmg_solver s);
double mlmg_get_solve_time_ms(mlmg_solver s);
int mlmg_get_num_mg_levels(mlmg_solver s);

/* n independent solves (each with its own operator, solver settings taken
 * from solvers[0]) run together: every V-cycle stage is one launch over all
 * solves' patches.  Per-solve statuses go to status[] (may be NULL); the
 * return value is the worst status. */
int mlmg_solve_batched(int n, const mlmg_solver* solvers, const mlmg_multifab* sols, const mlmg_multifab* rhss,
                       double tol_rel, double tol_abs, int* status);

/* Autotuner (no counterpart in the reference): times `vcycles` fixed
 * iterations of this solver's problem (sol is the initial guess and is left
 * unchanged, rhs the right-hand side) under each candidate smoother layout --
 * two colour passes, the fused sweep on 32x8x8 tiles, the z-marching fused
 * sweep on 64x16 columns with z-slabs of 8, 16 or 32 planes, and the coarse
 * levels run in one block per solve -- keeps the fastest in the solver's
 * options and reports its time.  FP64 solvers have one layout.  The text of
 * the last report (one line per candidate) comes from mlmg_autotune_report. */
int mlmg_autotune(mlmg_solver s, mlmg_multifab sol, mlmg_multifab rhs, int vcycles, double* best_ms);
const char* mlmg_autotune_report(mlmg_solver s);

/* Adjoint gradients of J(phi) for the solution phi = sol of A phi = f (no
 * counterpart in the reference; the face-gradient contraction is the one of
 * MLMG::getGradSolution / compFlux, AMReX_MLMG.H:553-761).  Solves
 * A^T lambda = dJdphi (homogeneous BCs, same MLMG settings and precision as
 * s, to tol_rel/tol_abs) and writes dJ/df = lambda into out_dJdf.  For
 * MLABecLaplacian, out_dJdb[3] (face-centred MultiFabs, entries may be NULL,
 * or the pointer NULL) receive dJ/db = -beta dxinv^2 (phi_c - phi_{c-1})
 * (lambda_c - lambda_{c-1}) per face (lambda = 0 outside the domain, phi's
 * ghosts from the level BC), and out_dJda (may be NULL) dJ/da = -alpha
 * lambda phi.  Returns the adjoint solve's status; the solver's getters then
 * report the adjoint solve.  Singular operators are rejected (-4). */
int mlmg_adjoint_grad(mlmg_solver s, mlmg_multifab sol, mlmg_multifab dJdphi, double tol_rel, double tol_abs,
                      mlmg_multifab out_dJdf, const mlmg_multifab* out_dJdb, mlmg_multifab out_dJda);

#if defined(__GNUC__)
#pragma GCC visibility pop
#endif
#ifdef __cplusplus
}
#endif

#endif /* MLMG_CAPI_H_ */
