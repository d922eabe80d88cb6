// The GB300 MLMG engine: a batch of N >= 1 independent cell-centred
// MLPoisson / MLABecLaplacian solves (single AMR level each), run V-cycle
// stage by V-cycle stage with one launch per stage covering every patch of
// every solve.  A single MLMG::solve is a batch of one.
#pragma once

#include "devbuf.hpp"
#include "hierarchy.hpp"

#include <memory>

namespace mlmg {

// A user MultiFab as the engine sees it: per-box FABs (box grown by ngrow,
// x fastest) in one device allocation.
struct FabSet {
    const void* data = nullptr;
    int prec = 8;               // bytes per value
    int ngrow = 0;
    int nodal_dir = -1;         // -1 cell-centred, 0..2 face-centred in that direction
    std::vector<Box3> boxes;    // valid boxes, cell-centred index space
    std::vector<long long> off; // element offset of each FAB
};

struct EngineOptions {
    int max_iter = 200;
    int fixed_iter = 0;
    int nu1 = 2, nu2 = 2, nuf = 8, nub = 0;
    int bottom_solver = 2;      // 1 smoother, 2 bicgstab
    int bottom_maxiter = 200;
    double bottom_reltol = 1.e-4;
    double bottom_abstol = -1.0;
    int always_use_bnorm = 0;
    int verbose = 0;
    int precision = 0;          // 0: FP64 throughout; 1: FP32 V-cycle inside FP64 refinement
    int use_graph = 0;          // capture one iteration in a CUDA graph and replay it
    int fused_smoother = 0;     // fused two-colour sweeps where a level allows
    int merge_boxes = 1;        // merge a level's boxes into one patch where exact
    int time_kernels = 0;       // time every finest-level smoother launch with CUDA events
    int coarse_block = 0;       // run the coarse levels of each V-cycle in one thread block per solve
                                // (slower than graph-replayed grid-wide launches on GB300 at every
                                // threshold from 2^3 to 32^3 cells)
    int coarse_cells = 512;     // a level is coarse when every solve has at most this many cells on it
    int march_sweep = 0;        // fused sweeps marching along z on levels with enough columns
                                // (measured slower than the tiled fused sweep: 0.27 vs 0.18 ms at 256^3)
    int march_min_tiles = 304;  // ... at least this many (column, z-chunk) tiles
    int march_tz = 16;          // planes per z-slab of the marching sweep
    int fused_tma = 1;          // tiled fused sweeps stage each tile by one TMA tensor load (else 16-byte
                                // cp.async copies)
    int fused_prefetch = 1;     // TMA sweeps also prefetch each tile's rhs and stencil boxes into L2
    int max_fmg_iter = 0;       // F-cycles (MLMGT::mgFcycle) for the first max_fmg_iter iterations
    int transpose = 0;          // solve A^T x = rhs (homogeneous BCs): the outer residual uses A^T,
                                // the V-cycle of A is the correction operator (adjoint solves)
    long long tma_first_wait = -1;  // polls of a tiled sweep's wait for its tile (-1: the default bound);
                                // a test knob: 0 makes every wait expire, which the solve reports as -7
    int final_fill_bc = 0;      // MLMGT::setFinalFillBC: a solution with more than one ghost layer also
                                // gets its first ghost layer written back
    int pdl = 1;                // V-cycle kernels as programmatic dependent launches
    int fused_fine = 1;         // AMR fine levels (MLPoisson, mixed): fused sweeps on the tiles whose halo
                                // meets no face shared with another patch, colour passes on the rest
                                // (2: colour passes on every tile; 0: the per-level colour passes)
    int fused_restrict = 1;     // TMA-swept levels: the V-cycle's correction residual and its restriction
                                // in one tile kernel (the fine residual stays in shared memory)
};

// true when two option sets capture the same iteration graph
bool same_iteration (const EngineOptions& a, const EngineOptions& b);

// Live timing of the dominant kernel (the finest-level smoother).
struct KernelStats {
    double total_ms = 0;        // summed device time of the timed launches
    long long launches = 0;
    double bytes_per_launch = 0;  // algorithmic bytes moved by one launch
    double cells_per_launch = 0;
    double flops_per_launch = 0;  // algorithmic FP64 operations of one launch (an FMA counts 2)
};

struct SolveProblem {           // one solve of a batch
    SolveSpec spec;             // geometry, MG grids, BCs, scalars
    std::vector<Box3> boxes;    // level-0 user boxes
    const FabSet* acoef = nullptr;       // cell-centred a (ABec); null = 1
    const FabSet* bcoef[3] = {nullptr, nullptr, nullptr};  // face b (ABec); null = 1
    const FabSet* levelbc = nullptr;     // Dirichlet values in its ghost cells; null = 0
    const FabSet* crse_bc = nullptr;     // coarse data of the coarse/fine faces of a level that does not
                                         // cover its domain (ratio spec.crse_ratio); null = 0
};

struct SolveReport {
    int status = 0;
    int niters = 0;
    double init_resid = 0, rhs_norm = 0, final_resid = 0;
    std::vector<double> history;
    std::vector<int> cg_iters;
};

class Engine {
public:
    Engine (std::vector<SolveProblem> problems, const EngineOptions& opt, cudaStream_t stream);
    ~Engine ();
    Engine (const Engine&) = delete;
    Engine& operator= (const Engine&) = delete;

    // (Re)load coefficients and BC values from the problems' FabSets and
    // restrict them to every MG level.
    void set_coefficients ();
    // Restrict the level-0 a and b held on the device to every MG level and
    // rebuild the stencil form (the second half of set_coefficients; a
    // composite solve calls it after averaging finer AMR levels' coefficients
    // into level 0's).
    void restrict_coefficients ();

    // MLMGT::solve on every solve of the batch.  sol[s] (ngrow >= 0) holds the
    // initial guess and receives the solution; rhs[s] the right-hand side.
    void solve (const std::vector<const FabSet*>& sol_in, const std::vector<FabSet*>& sol_out,
                const std::vector<const FabSet*>& rhs, double tol_rel, double tol_abs);

    // out = L(in) with inhomogeneous BCs (MLMGT::apply)
    void apply (const FabSet& in, FabSet& out);

    // res = rhs - L(sol) with inhomogeneous BCs, in the reference's operation
    // order (MLMGT::compResidual on one AMR level, AMReX_MLMG.H:790-856)
    void comp_residual (const FabSet& sol, const FabSet& rhs, FabSet& res);

    // After a transposed solve (options().transpose) of a batch of one, whose
    // solution lambda solves A^T lambda = dJ/dphi: the face-gradient
    // contraction dJ/db[d] = -beta dxinv_d^2 (phi_c - phi_{c-1})(lam_c - lam_{c-1})
    // and dJ/da = -alpha lam phi for the forward solution phi (MLABecLaplacian).
    // Null outputs are skipped.
    void adjoint_gradient (const FabSet& phi, FabSet* const grad_b[3], FabSet* grad_a);

    // MLMG::getGradSolution (mode 0) / MLMG::getFluxes (mode 1) of the
    // solution phi of a batch of one: face arrays of every box, phi's ghosts
    // from applyBC with the level's boundary values.  Null outputs are skipped.
    void face_fluxes (const FabSet& phi, FabSet* const out[3], int mode);

    const std::vector<SolveReport>& reports () const { return m_reports; }
    int nlevels (int s) const { return (int)m_problems[s].spec.levels.size(); }
    const EngineOptions& options () const { return m_opt; }
    EngineOptions& options () { return m_opt; }
    double last_solve_ms () const { return m_last_ms; }
    int kernel_launches () const { return m_launches; }
    void reset_launch_count () { m_launches = 0; }
    const KernelStats& smoother_stats () const { return m_kstats; }
    void reset_smoother_stats () { m_kstats.total_ms = 0; m_kstats.launches = 0; }
    // the FP64 outer residual of the mixed path (with the correction update
    // where it is fused), timed with the smoother under time_kernels
    const KernelStats& residual_stats () const { return m_rstats; }
    void reset_residual_stats () { m_rstats.total_ms = 0; m_rstats.launches = 0; }

    struct Impl;
    Impl& impl () { return *m_impl; }   // engine internals (AMR composite driver)
private:
    std::vector<SolveProblem> m_problems;
    EngineOptions m_opt;
    cudaStream_t m_stream;
    std::vector<SolveReport> m_reports;
    double m_last_ms = 0;
    int m_launches = 0;
    KernelStats m_kstats, m_rstats;
    std::unique_ptr<Impl> m_impl;
};

} // namespace mlmg
