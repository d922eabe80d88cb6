/* C interface of the CPU oracle (test infrastructure only; see mlmg_oracle.c). */
#ifndef MLMG_ORACLE_H_
#define MLMG_ORACLE_H_
#ifdef __cplusplus
extern "C" {
#endif

#define ORACLE_MAX_HIST 256

typedef struct {
    int n[3];            /* domain cells, lower corner 0 */
    int periodic[3];
    double prob_lo[3], prob_hi[3];
    int lobc[3], hibc[3];  /* LinOpBCType codes */
    int max_grid_size;     /* used when nbox == 0 */
    int nbox;              /* explicit boxes (lo[3], hi[3]) when > 0 */
    const int* boxes;
    int is_abec;
    double alpha, beta;
    const double* sol;     /* (nz+2)(ny+2)(nx+2): initial guess + Dirichlet values in ghosts */
    const double* rhs;     /* nz*ny*nx */
    const double* a;       /* nz*ny*nx or NULL (= 1) */
    const double* bx;      /* nz*ny*(nx+1) or NULL (= 1) */
    const double* by;      /* nz*(ny+1)*nx */
    const double* bz;      /* (nz+1)*ny*nx */
} OracleProblem;

typedef struct {
    int agg, con, agg_grid_size, con_grid_size, max_coarsening_level;
    int maxorder, nu1, nu2, nuf, nub;
    int max_iter, fixed_iter, bottom_solver, bottom_maxiter;
    double bottom_reltol, tol_rel, tol_abs;
    int max_fmg_iter;      /* F-cycles for the first max_fmg_iter iterations */
} OracleOptions;

typedef struct {
    int status, niters, nlev;
    double init_resid, rhs_norm, final_resid;
    double iter_seconds;   /* wall time of the iteration loop (setup excluded) */
    double history[ORACLE_MAX_HIST];
    int cg_iters[ORACLE_MAX_HIST];   /* one entry per bottom solve (F-cycles make several per iteration) */
    int ncg;
} OracleResult;

void oracle_default_options(OracleOptions* o);
int oracle_max_size(const int* dom_lo, const int* dom_hi, int chunk, int* out, int max_out);
int oracle_hierarchy(const OracleProblem* P, const OracleOptions* o, int* nbox_per_level, int* boxes_out,
                     int max_boxes);
int oracle_fill_boundary(const OracleProblem* P, int cross, double* data);
int oracle_apply(const OracleProblem* P, const OracleOptions* o, double* out);
/* mode 0: getGradSolution, mode 1: getFluxes; global face arrays */
int oracle_fluxes(const OracleProblem* P, const OracleOptions* o, int mode, double* fx, double* fy, double* fz);
int oracle_solve(const OracleProblem* P, const OracleOptions* o, double* phi_out, OracleResult* R);
/* composite solve over nlev AMR levels (ratio 2, MLPoisson): P[l] is level l
 * (n = n_0 2^l, its boxes, rhs over its domain, initial guess + boundary
 * values over its grown domain); phi_out[l] gets level l's solution */
int oracle_solve_amr(int nlev, const OracleProblem* P, const OracleOptions* o, double** phi_out,
                     OracleResult* R);

#ifdef __cplusplus
}
#endif
#endif
