// The AMR composite MLMG solve: MLMGT::solve over several AMR levels
// (refinement ratio 2, MLPoisson or MLABecLaplacian, periodic or not).  AMR
// level 0 is a full single-level
// engine (its own MG hierarchy, bottom solve, graphs); each finer AMR level is
// an engine of one MG level that is only smoothed.  The coarse/fine coupling
// (boundary-value interpolation, flux-register reflux, average-down,
// correction interpolation, masked norms) runs in the kernels of
// amr_kernels.cuh, driven from amr.cu.
#pragma once

#include "solver.hpp"

#include <memory>

namespace mlmg {

struct AmrLevelProblem {
    std::vector<Box3> boxes;            // the AMR level's BoxArray (level-l index space)
    const FabSet* levelbc = nullptr;    // Dirichlet values in its ghost cells; null = 0
    const FabSet* acoef = nullptr;      // MLABecLaplacian: cell-centred a; null = 1
    const FabSet* bcoef[3] = {nullptr, nullptr, nullptr};  // face b; null = 1
};

struct AmrProblem {
    GeomC geom;                         // geometry of AMR level 0
    int lobc[3] = {BC_DIRICHLET, BC_DIRICHLET, BC_DIRICHLET};
    int hibc[3] = {BC_DIRICHLET, BC_DIRICHLET, BC_DIRICHLET};
    int maxorder = 3;
    int is_abec = 0;                    // MLABecLaplacian (alpha a - beta div b grad) or MLPoisson
    double alpha = 0.0, beta = 1.0;
    LPInfoC info;                       // MG coarsening of AMR level 0
    std::vector<AmrLevelProblem> levels;
};

class AmrEngine {
public:
    AmrEngine (const AmrProblem& prob, const EngineOptions& opt, cudaStream_t stream);
    ~AmrEngine ();
    AmrEngine (const AmrEngine&) = delete;
    AmrEngine& operator= (const AmrEngine&) = delete;

    // MLMGT::solve (AMReX_MLMG.H:353-541) with one sol and one rhs per AMR
    // level; sol_in[l] is the initial guess, sol_out[l] receives the solution.
    void solve (const std::vector<const FabSet*>& sol_in, const std::vector<FabSet*>& sol_out,
                const std::vector<const FabSet*>& rhs, double tol_rel, double tol_abs);

    // MLMGT::compResidual (AMReX_MLMG.H:790-856): from the finest level down,
    // res[l] = rhs[l] - L(sol[l]) with the coarse/fine values interpolated
    // from sol[l-1], then the reflux of level l+1's fluxes into res[l] and the
    // average-down of res[l+1] onto the cells of level l it covers
    void comp_residual (const std::vector<const FabSet*>& sol, const std::vector<const FabSet*>& rhs,
                        const std::vector<FabSet*>& res);

    const SolveReport& report () const { return m_report; }
    EngineOptions& options () { return m_opt; }
    const EngineOptions& options () const { return m_opt; }
    double last_solve_ms () const { return m_last_ms; }
    int kernel_launches () const;
    void reset_launch_count ();
    int namr () const;
    int num_mg_levels () const;         // MG levels of AMR level 0

    struct Impl;
private:
    EngineOptions m_opt;
    cudaStream_t m_stream;
    SolveReport m_report;
    double m_last_ms = 0;
    std::unique_ptr<Impl> m_impl;
};

} // namespace mlmg
