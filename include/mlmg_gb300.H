// mlmg_gb300.H -- C++ facade of the GB300 MLMG library, header only, over
// the C ABI in mlmg_capi.h.
//
// The classes keep the names and the signatures of the reference C++ API
// that callers of this path use (AMReX 24.10):
//   amrex::Box, IntVect, RealBox, BoxArray (Src/Base/AMReX_BoxArray.H),
//   DistributionMapping, Geometry, MultiFab (AMReX_MultiFab.H), LPInfo,
//   MLPoisson (AMReX_MLPoisson.H:25-36), MLABecLaplacian
//   (AMReX_MLABecLaplacian.H:25-145: setScalars, setACoeffs, setBCoeffs),
//   MLMG (AMReX_MLMG.H:44-228: solve, apply, getFluxes, getGradSolution,
//   setters, getters),
// in namespace amrex_gb300, so that a translation unit written against the
// reference switches with
//     #include <mlmg_gb300.H>
//     namespace amrex = amrex_gb300;
// A MultiFab lives in device memory: fabPtr(i) is the device pointer of FAB i
// (the layout of amrex::BaseFab: box grown by nGrow, x fastest), and
// copyFromHost / copyToHost move one FAB.  Failures throw MLMG::error
// (std::runtime_error), as the reference does with setThrowException(true);
// MLMG::solve also throws when the solve does not converge, as the
// reference's aborts or throws (AMReX_MLMG.H:478-509).
#pragma once

#include "mlmg_capi.h"

#include <algorithm>
#include <array>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

namespace amrex_gb300 {

using Real = double;
using Long = long long;
template <class T> using Vector = std::vector<T>;
template <class T, std::size_t N> using Array = std::array<T, N>;

namespace detail {
inline void check (int rc)
{
    if (rc < 0) { throw std::runtime_error("[" + std::to_string(rc) + "] " + mlmg_last_error()); }
}
} // namespace detail

// ------------------------------------------------------------- index space --
struct IntVect {
    int v[3] = {0, 0, 0};
    IntVect () = default;
    IntVect (int i, int j, int k) : v{i, j, k} {}
    explicit IntVect (int s) : v{s, s, s} {}
    int operator[] (int d) const { return v[d]; }
    int& operator[] (int d) { return v[d]; }
    bool operator== (const IntVect& o) const { return v[0] == o.v[0] && v[1] == o.v[1] && v[2] == o.v[2]; }
};

class Box {
public:
    Box () = default;
    Box (const IntVect& lo, const IntVect& hi) : m_lo(lo), m_hi(hi) {}
    const IntVect& smallEnd () const { return m_lo; }
    const IntVect& bigEnd () const { return m_hi; }
    int length (int d) const { return m_hi[d] - m_lo[d] + 1; }
    Long numPts () const { return (Long)length(0) * length(1) * length(2); }
    bool operator== (const Box& o) const { return m_lo == o.m_lo && m_hi == o.m_hi; }
private:
    IntVect m_lo, m_hi;
};

struct RealBox {
    Array<Real, 3> lo{0, 0, 0}, hi{1, 1, 1};
    RealBox () = default;
    RealBox (const Array<Real, 3>& l, const Array<Real, 3>& h) : lo(l), hi(h) {}
};

enum class LinOpBCType : int {
    interior = 0, Dirichlet = 101, Neumann = 102, reflectOdd = 103, Periodic = 200,
};

// -------------------------------------------------------------- BoxArray --
// Shared handle: copies refer to the same array, as amrex::BoxArray copies
// share their data.
class BoxArray {
public:
    BoxArray () = default;
    explicit BoxArray (const Box& domain)
    {
        const int lo[3] = {domain.smallEnd()[0], domain.smallEnd()[1], domain.smallEnd()[2]};
        const int hi[3] = {domain.bigEnd()[0], domain.bigEnd()[1], domain.bigEnd()[2]};
        mlmg_boxarray h = nullptr;
        detail::check(mlmg_boxarray_new_domain(lo, hi, &h));
        m_h.reset(h, [] (mlmg_boxarray p) { mlmg_boxarray_delete(p); });
    }
    explicit BoxArray (const Vector<Box>& boxes)
    {
        std::vector<int> flat;
        for (const Box& b : boxes) {
            for (int d = 0; d < 3; ++d) { flat.push_back(b.smallEnd()[d]); }
            for (int d = 0; d < 3; ++d) { flat.push_back(b.bigEnd()[d]); }
        }
        mlmg_boxarray h = nullptr;
        detail::check(mlmg_boxarray_new(flat.data(), (int)boxes.size(), &h));
        m_h.reset(h, [] (mlmg_boxarray p) { mlmg_boxarray_delete(p); });
    }
    BoxArray& maxSize (int chunk)
    {
        const int c[3] = {chunk, chunk, chunk};
        detail::check(mlmg_boxarray_maxsize(m_h.get(), c));
        return *this;
    }
    BoxArray& maxSize (const IntVect& chunk)
    {
        const int c[3] = {chunk[0], chunk[1], chunk[2]};
        detail::check(mlmg_boxarray_maxsize(m_h.get(), c));
        return *this;
    }
    Long size () const { return mlmg_boxarray_size(m_h.get()); }
    Box operator[] (int i) const
    {
        int lo[3], hi[3];
        detail::check(mlmg_boxarray_get(m_h.get(), i, lo, hi));
        return Box(IntVect(lo[0], lo[1], lo[2]), IntVect(hi[0], hi[1], hi[2]));
    }
    mlmg_boxarray handle () const { return m_h.get(); }
private:
    std::shared_ptr<mlmg_boxarray_s> m_h;
};

class DistributionMapping {
public:
    DistributionMapping () = default;
    explicit DistributionMapping (const BoxArray& ba)
    {
        mlmg_distromap h = nullptr;
        detail::check(mlmg_distromap_new(ba.handle(), &h));
        m_h.reset(h, [] (mlmg_distromap p) { mlmg_distromap_delete(p); });
    }
    mlmg_distromap handle () const { return m_h.get(); }
private:
    std::shared_ptr<mlmg_distromap_s> m_h;
};

class Geometry {
public:
    Geometry () = default;
    // Geometry(const Box& dom, const RealBox& rb, int coord, const Array<int,3>& is_per)
    Geometry (const Box& dom, const RealBox& rb = RealBox(), int /*coord: cartesian*/ = 0,
              const Array<int, 3>& is_periodic = {0, 0, 0})
        : m_domain(dom)
    {
        const int lo[3] = {dom.smallEnd()[0], dom.smallEnd()[1], dom.smallEnd()[2]};
        const int hi[3] = {dom.bigEnd()[0], dom.bigEnd()[1], dom.bigEnd()[2]};
        mlmg_geometry h = nullptr;
        detail::check(mlmg_geometry_new(lo, hi, rb.lo.data(), rb.hi.data(), is_periodic.data(), &h));
        m_h.reset(h, [] (mlmg_geometry p) { mlmg_geometry_delete(p); });
    }
    const Box& Domain () const { return m_domain; }
    mlmg_geometry handle () const { return m_h.get(); }
private:
    Box m_domain;
    std::shared_ptr<mlmg_geometry_s> m_h;
};

// -------------------------------------------------------------- MultiFab --
class MultiFab {
public:
    MultiFab () = default;
    MultiFab (const BoxArray& ba, const DistributionMapping& dm, int ncomp, int ngrow)
        : MultiFab(ba, dm, ncomp, ngrow, -1) {}
    // face-centred in direction nodal_dir (amrex::convert(ba, IntVect::TheDimensionVector(d)))
    MultiFab (const BoxArray& ba, const DistributionMapping& dm, int ncomp, int ngrow, int nodal_dir)
        : m_ba(ba), m_ncomp(ncomp), m_ngrow(ngrow)
    {
        mlmg_multifab h = nullptr;
        detail::check(mlmg_multifab_new(ba.handle(), dm.handle(), ncomp, ngrow, nodal_dir, 8, &h));
        m_h.reset(h, [] (mlmg_multifab p) { mlmg_multifab_delete(p); });
    }
    MultiFab (const MultiFab&) = delete;
    MultiFab& operator= (const MultiFab&) = delete;
    MultiFab (MultiFab&&) = default;
    MultiFab& operator= (MultiFab&&) = default;

    const BoxArray& boxArray () const { return m_ba; }
    int nComp () const { return m_ncomp; }
    int nGrow () const { return m_ngrow; }
    int size () const { return (int)m_ba.size(); }
    void setVal (Real v) { detail::check(mlmg_multifab_setval(m_h.get(), v)); }
    void FillBoundary (const Geometry& geom, bool cross = false)
    {
        detail::check(mlmg_multifab_fill_boundary(m_h.get(), geom.handle(), cross ? 1 : 0));
    }
    Real norminf () const
    {
        double v = 0;
        detail::check(mlmg_multifab_norminf(m_h.get(), &v));
        return v;
    }
    // FAB i: element count, device pointer, host transfers
    std::size_t fabSize (int i) const
    {
        std::size_t n = 0;
        detail::check(mlmg_multifab_fab_size(m_h.get(), i, &n));
        return n;
    }
    Real* fabPtr (int i)
    {
        void* p = nullptr;
        detail::check(mlmg_multifab_fab_ptr(m_h.get(), i, &p));
        return static_cast<Real*>(p);
    }
    void copyFromHost (int i, const Real* host) { detail::check(mlmg_multifab_upload(m_h.get(), i, host)); }
    void copyToHost (int i, Real* host) const { detail::check(mlmg_multifab_download(m_h.get(), i, host)); }
    mlmg_multifab handle () const { return m_h.get(); }
private:
    BoxArray m_ba;
    int m_ncomp = 0, m_ngrow = 0;
    std::shared_ptr<mlmg_multifab_s> m_h;
};

// ----------------------------------------------------------------- LPInfo --
struct LPInfo {
    bool do_agglomeration = true;
    bool do_consolidation = true;
    int agg_grid_size = -1;          // <= 0: the GPU-build default (32)
    int con_grid_size = -1;
    int max_coarsening_level = 30;
    LPInfo& setAgglomeration (bool x) { do_agglomeration = x; return *this; }
    LPInfo& setConsolidation (bool x) { do_consolidation = x; return *this; }
    LPInfo& setAgglomerationGridSize (int x) { agg_grid_size = x; return *this; }
    LPInfo& setConsolidationGridSize (int x) { con_grid_size = x; return *this; }
    LPInfo& setMaxCoarseningLevel (int n) { max_coarsening_level = n; return *this; }
    mlmg_lpinfo c () const
    {
        return mlmg_lpinfo{do_agglomeration ? 1 : 0, do_consolidation ? 1 : 0, agg_grid_size, con_grid_size,
                           max_coarsening_level};
    }
};

// ------------------------------------------------------ linear operators --
class MLLinOp {
public:
    virtual ~MLLinOp () = default;
    MLLinOp (const MLLinOp&) = delete;
    MLLinOp& operator= (const MLLinOp&) = delete;
    // MLLinOpT::setDomainBC (AMReX_MLLinOp.H:380-400)
    void setDomainBC (const Array<LinOpBCType, 3>& lobc, const Array<LinOpBCType, 3>& hibc)
    {
        const int lo[3] = {(int)lobc[0], (int)lobc[1], (int)lobc[2]};
        const int hi[3] = {(int)hibc[0], (int)hibc[1], (int)hibc[2]};
        detail::check(mlmg_linop_set_domain_bc(m_h.get(), lo, hi));
    }
    // MLCellLinOpT::setLevelBC (AMReX_MLCellLinOp.H:513): Dirichlet values in
    // the ghost cells of levelbcdata (nullptr: homogeneous)
    void setLevelBC (int amrlev, const MultiFab* levelbcdata)
    {
        detail::check(mlmg_linop_set_level_bc(m_h.get(), amrlev, levelbcdata ? levelbcdata->handle() : nullptr));
    }
    void setMaxOrder (int maxorder) { detail::check(mlmg_linop_set_maxorder(m_h.get(), maxorder)); }
    // MLLinOpT::setCoarseFineBC (AMReX_MLLinOp.H:200-211): coarse data for the
    // coarse/fine faces of a level that does not cover its domain (Dirichlet
    // only; the values are taken at this call)
    void setCoarseFineBC (const MultiFab* crse, int crse_ratio)
    {
        detail::check(mlmg_linop_set_coarse_fine_bc(m_h.get(), crse ? crse->handle() : nullptr, crse_ratio));
    }
    int NAMRLevels () const { return mlmg_linop_num_amr_levels(m_h.get()); }
    int NMGLevels (int /*amrlev*/) const { return mlmg_linop_num_mg_levels(m_h.get()); }
    mlmg_linop handle () const { return m_h.get(); }
protected:
    MLLinOp () = default;
    using Ctor = int (*)(int, const mlmg_geometry*, const mlmg_boxarray*, const mlmg_distromap*,
                         const mlmg_lpinfo*, mlmg_linop*);
    void define (Ctor ctor, const Vector<Geometry>& geom, const Vector<BoxArray>& grids,
                 const Vector<DistributionMapping>& dmap, const LPInfo& info)
    {
        const int n = (int)geom.size();
        std::vector<mlmg_geometry> g(n);
        std::vector<mlmg_boxarray> b(n);
        std::vector<mlmg_distromap> d(n);
        for (int l = 0; l < n; ++l) { g[l] = geom[l].handle(); b[l] = grids[l].handle(); d[l] = dmap[l].handle(); }
        const mlmg_lpinfo li = info.c();
        mlmg_linop h = nullptr;
        detail::check(ctor(n, g.data(), b.data(), d.data(), &li, &h));
        m_h.reset(h, [] (mlmg_linop p) { mlmg_linop_delete(p); });
    }
    std::shared_ptr<mlmg_linop_s> m_h;
};

// MLPoissonT(const Vector<Geometry>&, const Vector<BoxArray>&,
//            const Vector<DistributionMapping>&, const LPInfo&) (AMReX_MLPoisson.H:25-36)
class MLPoisson : public MLLinOp {
public:
    MLPoisson (const Vector<Geometry>& geom, const Vector<BoxArray>& grids, const Vector<DistributionMapping>& dmap,
               const LPInfo& info = LPInfo())
    {
        define(&mlmg_linop_new_poisson, geom, grids, dmap, info);
    }
};

// MLABecLaplacianT (AMReX_MLABecLaplacian.H:25-145): alpha a phi - beta div(b grad phi)
class MLABecLaplacian : public MLLinOp {
public:
    MLABecLaplacian (const Vector<Geometry>& geom, const Vector<BoxArray>& grids,
                     const Vector<DistributionMapping>& dmap, const LPInfo& info = LPInfo())
    {
        define(&mlmg_linop_new_abeclap, geom, grids, dmap, info);
    }
    void setScalars (Real a, Real b) { detail::check(mlmg_abeclap_set_scalars(m_h.get(), a, b)); }
    void setACoeffs (int amrlev, const MultiFab& alpha)
    {
        detail::check(mlmg_abeclap_set_acoeffs(m_h.get(), amrlev, alpha.handle()));
    }
    void setACoeffs (int amrlev, Real alpha) { detail::check(mlmg_abeclap_set_acoeffs_const(m_h.get(), amrlev, alpha)); }
    void setBCoeffs (int amrlev, const Array<MultiFab const*, 3>& beta)
    {
        const mlmg_multifab b[3] = {beta[0]->handle(), beta[1]->handle(), beta[2]->handle()};
        detail::check(mlmg_abeclap_set_bcoeffs(m_h.get(), amrlev, b));
    }
    void setBCoeffs (int amrlev, Real beta) { detail::check(mlmg_abeclap_set_bcoeffs_const(m_h.get(), amrlev, beta)); }
};

// ------------------------------------------------------------------- MLMG --
class MLMG {
public:
    struct error : std::runtime_error {
        using std::runtime_error::runtime_error;
    };
    enum class BottomSolver : int { Default = 0, smoother = 1, bicgstab = 2 };

    explicit MLMG (MLLinOp& linop) : m_linop(&linop)
    {
        mlmg_solver h = nullptr;
        guard(mlmg_new(linop.handle(), &h));
        m_h.reset(h, [] (mlmg_solver p) { mlmg_delete(p); });
    }
    MLMG (const MLMG&) = delete;
    MLMG& operator= (const MLMG&) = delete;

    // setters (AMReX_MLMG.H:116-142)
    void setVerbose (int v) { guard(mlmg_set_verbose(m_h.get(), v)); }
    void setMaxIter (int n) { guard(mlmg_set_max_iter(m_h.get(), n)); }
    void setMaxFmgIter (int n) { guard(mlmg_set_max_fmg_iter(m_h.get(), n)); }
    void setFixedIter (int n) { guard(mlmg_set_fixed_iter(m_h.get(), n)); m_fixed = n; }
    void setPreSmooth (int n) { guard(mlmg_set_pre_smooth(m_h.get(), n)); }
    void setPostSmooth (int n) { guard(mlmg_set_post_smooth(m_h.get(), n)); }
    void setFinalSmooth (int n) { guard(mlmg_set_final_smooth(m_h.get(), n)); }
    void setBottomSmooth (int n) { guard(mlmg_set_bottom_smooth(m_h.get(), n)); }
    void setBottomSolver (BottomSolver s) { guard(mlmg_set_bottom_solver(m_h.get(), (int)s)); }
    void setBottomMaxIter (int n) { guard(mlmg_set_bottom_max_iter(m_h.get(), n)); }
    void setBottomTolerance (Real t) { guard(mlmg_set_bottom_tolerance(m_h.get(), t)); }
    void setBottomToleranceAbs (Real t) { guard(mlmg_set_bottom_tolerance_abs(m_h.get(), t)); }
    void setAlwaysUseBNorm (int f) { guard(mlmg_set_always_use_bnorm(m_h.get(), f)); }
    void setFinalFillBC (int f) { guard(mlmg_set_final_fill_bc(m_h.get(), f)); }
    // GB300 additions: FP32 V-cycles in FP64 refinement, CUDA-graph iterations, fused sweeps
    void setMixedPrecision (bool on) { guard(mlmg_set_precision(m_h.get(), on ? 1 : 0)); }
    void setCudaGraph (bool on) { guard(mlmg_set_graph(m_h.get(), on ? 1 : 0)); }
    void setFusedSmoother (bool on) { guard(mlmg_set_fused_smoother(m_h.get(), on ? 1 : 0)); }

    // MLMGT::solve (AMReX_MLMG.H:44-51): one sol and one rhs per AMR level;
    // returns the final composite max-norm of the residual
    Real solve (const Vector<MultiFab*>& a_sol, const Vector<MultiFab const*>& a_rhs, Real a_tol_rel,
                Real a_tol_abs, const char* /*checkpoint_file*/ = nullptr)
    {
        std::vector<mlmg_multifab> s, r;
        for (MultiFab* m : a_sol) { s.push_back(m->handle()); }
        for (const MultiFab* m : a_rhs) { r.push_back(m->handle()); }
        double resid = 0;
        const int rc = mlmg_solve_levels(m_h.get(), s.data(), r.data(), a_tol_rel, a_tol_abs, &resid);
        if (rc < 0 || (rc > 0 && m_fixed == 0)) {
            throw error(std::string("MLMG: ") + mlmg_last_error());
        }
        return resid;
    }
    // MLMGT::compResidual (AMReX_MLMG.H:790-856): res = rhs - L(sol) on every AMR level
    void compResidual (const Vector<MultiFab*>& a_res, const Vector<MultiFab*>& a_sol,
                       const Vector<MultiFab const*>& a_rhs)
    {
        std::vector<mlmg_multifab> r, x, b;
        for (MultiFab* m : a_res) { r.push_back(m->handle()); }
        for (MultiFab* m : a_sol) { x.push_back(m->handle()); }
        for (const MultiFab* m : a_rhs) { b.push_back(m->handle()); }
        guard(mlmg_comp_residual(m_h.get(), r.data(), x.data(), b.data()));
    }
    // MLMGT::apply (AMReX_MLMG.H:858-932): out = L(in) with the level BC values
    void apply (const Vector<MultiFab*>& out, const Vector<MultiFab*>& in)
    {
        guard(mlmg_apply(m_h.get(), out[0]->handle(), in[0]->handle()));
    }
    // MLMGT::getFluxes / getGradSolution (AMReX_MLMG.H:553-655) of the
    // solution passed explicitly (the one given to solve)
    void getFluxes (const Vector<Array<MultiFab*, 3>>& a_flux, const Vector<MultiFab*>& a_sol)
    {
        const mlmg_multifab f[3] = {a_flux[0][0] ? a_flux[0][0]->handle() : nullptr,
                                    a_flux[0][1] ? a_flux[0][1]->handle() : nullptr,
                                    a_flux[0][2] ? a_flux[0][2]->handle() : nullptr};
        guard(mlmg_get_fluxes(m_h.get(), a_sol[0]->handle(), f));
    }
    void getGradSolution (const Vector<Array<MultiFab*, 3>>& a_grad, const Vector<MultiFab*>& a_sol)
    {
        const mlmg_multifab g[3] = {a_grad[0][0] ? a_grad[0][0]->handle() : nullptr,
                                    a_grad[0][1] ? a_grad[0][1]->handle() : nullptr,
                                    a_grad[0][2] ? a_grad[0][2]->handle() : nullptr};
        guard(mlmg_get_grad_solution(m_h.get(), a_sol[0]->handle(), g));
    }

    // getters (AMReX_MLMG.H:220-228)
    int getNumIters () const { return mlmg_get_num_iters(m_h.get()); }
    Vector<Real> getResidualHistory () const
    {
        std::vector<double> h(512);
        const int n = mlmg_get_residual_history(m_h.get(), h.data(), (int)h.size());
        h.resize(n > 0 ? std::min<std::size_t>((std::size_t)n, h.size()) : 0);
        return h;
    }
    Vector<int> getNumCGIters () const
    {
        std::vector<int> c(4096);
        const int n = mlmg_get_num_cg_iters(m_h.get(), c.data(), (int)c.size());
        c.resize(n > 0 ? std::min<std::size_t>((std::size_t)n, c.size()) : 0);
        return c;
    }
    Real getInitResidual () const { return mlmg_get_init_residual(m_h.get()); }
    Real getFinalResidual () const { return mlmg_get_final_residual(m_h.get()); }
    Real getInitRHS () const { return mlmg_get_init_rhs(m_h.get()); }
    double getSolveTimeMs () const { return mlmg_get_solve_time_ms(m_h.get()); }
    mlmg_solver handle () const { return m_h.get(); }

private:
    static void guard (int rc)
    {
        if (rc < 0) { throw error("[" + std::to_string(rc) + "] " + mlmg_last_error()); }
    }
    MLLinOp* m_linop;
    int m_fixed = 0;
    std::shared_ptr<mlmg_solver_s> m_h;
};

} // namespace amrex_gb300
