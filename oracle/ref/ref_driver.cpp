// Harness around the reference AMReX CPU MLMG, written against its public API
// (amrex::MLMG, MLPoisson, MLABecLaplacian, MultiFab, BoxArray,
// DistributionMapping, Geometry).  It reads a case directory written by
// tests/golden/make_golden.py and writes the reference's outputs back into it.
//
// Test infrastructure only: it is built by oracle/ref/Makefile into
// oracle/_ref/<machine>/ and used to generate golden fixtures and as the
// timed CPU baseline.
//
//   ref_driver <mode> <case_dir>
//     mode = hier   : MG hierarchy box lists (per MG level)       -> hier.txt
//            fb     : FillBoundary on a MultiFab with 1 ghost      -> fb_out.bin
//            apply  : MLMG::apply (out = L phi, inhomogeneous BC)  -> out.bin
//            solve  : MLMG::solve                                  -> phi.bin, result.txt
//                     (sol_ngrow != 1: also phi_fabs.bin, every grown FAB in box order)
//            flux   : solve, then getFluxes / getGradSolution    -> also f[xyz].bin, g[xyz].bin
//            resid  : MLMG::compResidual of the initial guess       -> res.bin
//            amrgrids : AmrMesh::MakeNewGrids tagging |rhs_l| > thresh_l -> grids.txt
//            amrsolve : composite multi-level MLPoisson / MLABecLaplacian solve -> phi_l<lev>.bin, result.txt
//            amrresid : MLMG::compResidual over the AMR levels of the initial guess -> res_l<lev>.bin
//
// Single-level keys beyond the operator's: crse_ratio / crse_file / crse_mgs
// (MLLinOp::setCoarseFineBC with a coarse MultiFab over the coarsened domain,
// BoxArray chopped to crse_mgs, filled from a whole-coarse-domain array),
// sol_ngrow (ghost cells of the solution MultiFab), final_fill_bc
// (MLMG::setFinalFillBC), bottom_solver (MLMG::BottomSolver code).
//
// case.txt holds "key value..." lines; binary inputs are little-endian
// float64 arrays over the whole domain, x fastest.
#include <AMReX.H>
#include <AMReX_MultiFab.H>
#include <AMReX_MLMG.H>
#include <AMReX_MLABecLaplacian.H>
#include <AMReX_MLPoisson.H>
#include <AMReX_ParmParse.H>
#include <AMReX_AmrMesh.H>
#include <AMReX_TagBox.H>

#include <omp.h>

#include <chrono>
#include <cstdio>
#include <fstream>
#include <map>
#include <sstream>
#include <string>
#include <vector>

using namespace amrex;

namespace {

std::map<std::string, std::vector<std::string>> read_case (const std::string& dir)
{
    std::map<std::string, std::vector<std::string>> kv;
    std::ifstream is(dir + "/case.txt");
    std::string line;
    while (std::getline(is, line)) {
        std::istringstream ls(line);
        std::string key, tok;
        if (!(ls >> key) || key[0] == '#') { continue; }
        std::vector<std::string> v;
        while (ls >> tok) { v.push_back(tok); }
        kv[key] = v;
    }
    return kv;
}

struct Case {
    std::map<std::string, std::vector<std::string>> kv;
    bool has (const std::string& k) const { return kv.count(k) > 0; }
    int geti (const std::string& k, int d, int i = 0) const {
        auto it = kv.find(k); return (it == kv.end() || (int)it->second.size() <= i) ? d : std::stoi(it->second[i]);
    }
    double getd (const std::string& k, double d, int i = 0) const {
        auto it = kv.find(k); return (it == kv.end() || (int)it->second.size() <= i) ? d : std::stod(it->second[i]);
    }
    std::string gets (const std::string& k, const std::string& d) const {
        auto it = kv.find(k); return (it == kv.end() || it->second.empty()) ? d : it->second[0];
    }
};

std::vector<double> read_bin (const std::string& path, size_t n)
{
    std::vector<double> v(n);
    std::FILE* f = std::fopen(path.c_str(), "rb");
    if (!f) { amrex::Abort("ref_driver: cannot open " + path); }
    size_t got = std::fread(v.data(), sizeof(double), n, f);
    std::fclose(f);
    if (got != n) { amrex::Abort("ref_driver: short read " + path); }
    return v;
}

void write_bin (const std::string& path, const std::vector<double>& v)
{
    std::FILE* f = std::fopen(path.c_str(), "wb");
    std::fwrite(v.data(), sizeof(double), v.size(), f);
    std::fclose(f);
}

// global array g with extents (nx,ny,nz) and index origin (ox,oy,oz)
struct Global {
    int nx, ny, nz, ox, oy, oz;
    std::vector<double> v;
    double& at (int i, int j, int k) {
        return v[((size_t)(k-oz)*ny + (j-oy))*nx + (i-ox)];
    }
};

void fill_from_global (MultiFab& mf, Global& g, int ngrow)
{
    for (MFIter mfi(mf); mfi.isValid(); ++mfi) {
        Box bx = amrex::grow(mfi.validbox(), ngrow);
        bx.setType(mf.boxArray().ixType());
        auto a = mf.array(mfi);
        const auto lo = lbound(bx), hi = ubound(bx);
        for (int k = lo.z; k <= hi.z; ++k)
        for (int j = lo.y; j <= hi.y; ++j)
        for (int i = lo.x; i <= hi.x; ++i) { a(i,j,k) = g.at(i,j,k); }
    }
}

void copy_to_global (const MultiFab& mf, Global& g)
{
    for (MFIter mfi(mf); mfi.isValid(); ++mfi) {
        const Box& bx = mfi.validbox();
        auto a = mf.const_array(mfi);
        const auto lo = lbound(bx), hi = ubound(bx);
        for (int k = lo.z; k <= hi.z; ++k)
        for (int j = lo.y; j <= hi.y; ++j)
        for (int i = lo.x; i <= hi.x; ++i) { g.at(i,j,k) = a(i,j,k); }
    }
}

// exposes the protected MG hierarchy of a linear operator
template <class Op>
struct HierProbe : Op {
    using Op::Op;
    const Vector<Vector<BoxArray>>& grids () const { return this->m_grids; }
};

BoxArray make_grids (const Case& c, const Box& domain)
{
    if (c.has("boxes")) {
        BoxList bl;
        const auto& v = c.kv.at("boxes");
        for (size_t m = 0; m + 5 < v.size(); m += 6) {
            bl.push_back(Box(IntVect(std::stoi(v[m]), std::stoi(v[m+1]), std::stoi(v[m+2])),
                             IntVect(std::stoi(v[m+3]), std::stoi(v[m+4]), std::stoi(v[m+5]))));
        }
        return BoxArray(bl);
    }
    BoxArray ba(domain);
    ba.maxSize(c.geti("max_grid_size", 32));
    return ba;
}

template <class Op>
void setup_op (Op& op, const Case& c)
{
    Array<LinOpBCType,3> lo, hi;
    for (int d = 0; d < 3; ++d) {
        lo[d] = static_cast<LinOpBCType>(c.geti("lobc", 101, d));
        hi[d] = static_cast<LinOpBCType>(c.geti("hibc", 101, d));
    }
    op.setDomainBC(lo, hi);
    op.setMaxOrder(c.geti("maxorder", 3));
}

LPInfo make_info (const Case& c)
{
    LPInfo info;
    info.setAgglomeration(c.geti("agg", 1) != 0);
    info.setConsolidation(c.geti("con", 1) != 0);
    info.setAgglomerationGridSize(c.geti("agg_grid_size", 32));
    info.setConsolidationGridSize(c.geti("con_grid_size", 32));
    info.setMaxCoarseningLevel(c.geti("max_coarsening_level", 30));
    return info;
}

// AmrMesh whose ErrorEst tags cells where |rhs_l| > thresh_l (rhs of each
// level given on the level's whole domain)
struct TagMesh : AmrMesh {
    std::vector<std::vector<double>> rhs;   // per level, x fastest
    std::vector<double> thresh;
    std::vector<Box> dom;
    TagMesh (Geometry const& g, AmrInfo const& info) : AmrMesh(g, info) {}
    void ErrorEst (int lev, TagBoxArray& tags, Real, int) override {
        const Box& d = dom[lev];
        const int nx = d.length(0), ny = d.length(1);
        for (MFIter mfi(tags); mfi.isValid(); ++mfi) {
            const Box& bx = mfi.validbox();
            auto t = tags.array(mfi);
            const auto lo = lbound(bx), hi = ubound(bx);
            for (int k = lo.z; k <= hi.z; ++k)
            for (int j = lo.y; j <= hi.y; ++j)
            for (int i = lo.x; i <= hi.x; ++i) {
                const double v = rhs[lev][((size_t)k * ny + j) * nx + i];
                if (std::abs(v) > thresh[lev]) { t(i,j,k) = TagBox::SET; }
            }
        }
    }
};

void read_boxes (const Case& c, const std::string& key, BoxList& bl)
{
    const auto& v = c.kv.at(key);
    for (size_t m = 0; m + 5 < v.size(); m += 6) {
        bl.push_back(Box(IntVect(std::stoi(v[m]), std::stoi(v[m+1]), std::stoi(v[m+2])),
                         IntVect(std::stoi(v[m+3]), std::stoi(v[m+4]), std::stoi(v[m+5]))));
    }
}

// amrgrids: AmrMesh::MakeNewGrids with |rhs| tagging -> grids.txt
// amrsolve: composite MLPoisson solve on the given per-level grids
//           -> phi_l<lev>.bin (level domain, cells of the level's boxes), result.txt
int run_amr (const std::string& mode, const std::string& dir)
{
    Case c{read_case(dir)};
    const int nlev = c.geti("nlev", 1);
    const int nx = c.geti("n", 32, 0), ny = c.geti("n", 32, 1), nz = c.geti("n", 32, 2);
    RealBox rb({0., 0., 0.}, {1., 1., 1.});
    Array<int,3> is_per{c.geti("periodic", 0, 0), c.geti("periodic", 0, 1), c.geti("periodic", 0, 2)};
    std::vector<Box> dom;
    Vector<Geometry> geom;
    for (int l = 0; l < nlev; ++l) {
        const int r = 1 << l;
        dom.emplace_back(IntVect(0), IntVect(nx*r-1, ny*r-1, nz*r-1));
        geom.emplace_back(dom.back(), rb, CoordSys::cartesian, is_per);
    }
    if (mode == "amrgrids") {
        AmrInfo info;
        info.max_level = nlev - 1;
        info.ref_ratio = Vector<IntVect>(nlev, IntVect(2));
        info.blocking_factor = Vector<IntVect>(nlev, IntVect(c.geti("blocking_factor", 8)));
        info.max_grid_size = Vector<IntVect>(nlev, IntVect(c.geti("max_grid_size", 64)));
        info.n_error_buf = Vector<IntVect>(nlev, IntVect(c.geti("n_error_buf", 1)));
        info.grid_eff = c.getd("grid_eff", 0.7);
        TagMesh mesh(geom[0], info);
        mesh.dom = dom;
        for (int l = 0; l < nlev; ++l) {
            mesh.rhs.push_back(read_bin(dir + "/rhs_l" + std::to_string(l) + ".bin", (size_t)dom[l].numPts()));
            mesh.thresh.push_back(c.getd("thresh", 0.0, l));
        }
        mesh.MakeNewGrids(0.0);
        std::ofstream gs(dir + "/grids.txt");
        for (int l = 0; l <= mesh.finestLevel(); ++l) {
            const BoxArray& g = mesh.boxArray(l);
            gs << "level " << l << " " << g.size() << "\n";
            for (int b = 0; b < g.size(); ++b) {
                gs << g[b].smallEnd(0) << " " << g[b].smallEnd(1) << " " << g[b].smallEnd(2) << " "
                   << g[b].bigEnd(0) << " " << g[b].bigEnd(1) << " " << g[b].bigEnd(2) << "\n";
            }
        }
        return 0;
    }
    // composite solve
    Vector<BoxArray> ba(nlev);
    Vector<DistributionMapping> dm(nlev);
    for (int l = 0; l < nlev; ++l) {
        BoxList bl;
        read_boxes(c, "boxes_l" + std::to_string(l), bl);
        ba[l] = BoxArray(bl);
        dm[l] = DistributionMapping(ba[l]);
    }
    LPInfo info = make_info(c);
    // MLPoisson, or (op abec) MLABecLaplacian with per-level a (a_l<lev>.bin)
    // and face b (b[xyz]_l<lev>.bin) over each level's whole domain
    const bool is_abec = c.gets("op", "poisson") == "abec";
    std::unique_ptr<MLCellLinOp> linop;
    if (is_abec) {
        auto* abec = new MLABecLaplacian(geom, ba, dm, info);
        setup_op(*abec, c);
        abec->setScalars(c.getd("alpha", 1.0), c.getd("beta", 1.0));
        for (int l = 0; l < nlev; ++l) {
            const int gx = dom[l].length(0), gy = dom[l].length(1), gz = dom[l].length(2);
            const std::string sl = "_l" + std::to_string(l) + ".bin";
            MultiFab acoef(ba[l], dm[l], 1, 0);
            Global ga{gx, gy, gz, 0, 0, 0, read_bin(dir + "/a" + sl, (size_t)gx*gy*gz)};
            fill_from_global(acoef, ga, 0);
            abec->setACoeffs(l, acoef);
            Array<MultiFab,3> face;
            for (int d = 0; d < 3; ++d) {
                face[d].define(amrex::convert(ba[l], IntVect::TheDimensionVector(d)), dm[l], 1, 0);
                Global gb{gx + (d==0), gy + (d==1), gz + (d==2), 0, 0, 0, {}};
                gb.v = read_bin(dir + "/b" + std::string(1, char('x'+d)) + sl, (size_t)gb.nx*gb.ny*gb.nz);
                fill_from_global(face[d], gb, 0);
            }
            abec->setBCoeffs(l, amrex::GetArrOfConstPtrs(face));
        }
        linop.reset(abec);
    } else {
        auto* p = new MLPoisson(geom, ba, dm, info);
        setup_op(*p, c);
        linop.reset(p);
    }
    MLCellLinOp& pois = *linop;
    Vector<MultiFab> sol(nlev), rhs(nlev);
    for (int l = 0; l < nlev; ++l) {
        sol[l].define(ba[l], dm[l], 1, 1);
        rhs[l].define(ba[l], dm[l], 1, 0);
        const int gx = dom[l].length(0), gy = dom[l].length(1), gz = dom[l].length(2);
        Global gs{gx+2, gy+2, gz+2, -1, -1, -1, std::vector<double>((size_t)(gx+2)*(gy+2)*(gz+2), 0.0)};
        // optional initial guess and Dirichlet values in the ghosts (grown level domain)
        const std::string bcf = dir + "/solbc_l" + std::to_string(l) + ".bin";
        if (std::FILE* tf = std::fopen(bcf.c_str(), "rb")) {
            std::fclose(tf);
            gs.v = read_bin(bcf, (size_t)(gx+2)*(gy+2)*(gz+2));
        }
        fill_from_global(sol[l], gs, 1);
        Global gr{gx, gy, gz, 0, 0, 0, read_bin(dir + "/rhs_l" + std::to_string(l) + ".bin", (size_t)gx*gy*gz)};
        fill_from_global(rhs[l], gr, 0);
        pois.setLevelBC(l, &sol[l]);
    }
    MLMG mlmg(pois);
    mlmg.setVerbose(c.geti("verbose", 0));
    mlmg.setMaxIter(c.geti("max_iter", 200));
    if (c.geti("fixed_iter", 0) > 0) { mlmg.setFixedIter(c.geti("fixed_iter", 0)); }
    if (c.geti("max_fmg_iter", 0) > 0) { mlmg.setMaxFmgIter(c.geti("max_fmg_iter", 0)); }
    if (mode == "amrresid") {
        Vector<MultiFab> res(nlev);
        for (int l = 0; l < nlev; ++l) { res[l].define(ba[l], dm[l], 1, 0); }
        mlmg.compResidual(GetVecOfPtrs(res), GetVecOfPtrs(sol), GetVecOfConstPtrs(rhs));
        for (int l = 0; l < nlev; ++l) {
            const int gx = dom[l].length(0), gy = dom[l].length(1), gz = dom[l].length(2);
            Global go{gx, gy, gz, 0, 0, 0, std::vector<double>((size_t)gx*gy*gz, 0.0)};
            copy_to_global(res[l], go);
            write_bin(dir + "/res_l" + std::to_string(l) + ".bin", go.v);
        }
        return 0;
    }
    auto t0 = std::chrono::steady_clock::now();
    const Real resid = mlmg.solve(GetVecOfPtrs(sol), GetVecOfConstPtrs(rhs), c.getd("tol_rel", 1e-10),
                                  c.getd("tol_abs", 0.0));
    auto t1 = std::chrono::steady_clock::now();
    for (int l = 0; l < nlev; ++l) {
        const int gx = dom[l].length(0), gy = dom[l].length(1), gz = dom[l].length(2);
        Global go{gx, gy, gz, 0, 0, 0, std::vector<double>((size_t)gx*gy*gz, 0.0)};
        copy_to_global(sol[l], go);
        write_bin(dir + "/phi_l" + std::to_string(l) + ".bin", go.v);
    }
    std::ofstream res(dir + "/result.txt");
    res.precision(17);
    res << "final_resid " << resid << "\n";
    res << "init_resid " << mlmg.getInitResidual() << "\n";
    res << "rhs_norm " << mlmg.getInitRHS() << "\n";
    res << "niters " << mlmg.getNumIters() << "\n";
    res << "history";
    for (auto h : mlmg.getResidualHistory()) { res << " " << h; }
    res << "\ncg_iters";
    for (auto h : mlmg.getNumCGIters()) { res << " " << h; }
    res << "\nsolve_seconds " << std::chrono::duration<double>(t1 - t0).count();
    res << "\nthreads " << omp_get_max_threads() << "\n";
    return 0;
}

} // namespace

int main (int argc, char* argv[])
{
    if (argc < 3) { std::fprintf(stderr, "usage: ref_driver mode case_dir\n"); return 2; }
    const std::string mode = argv[1];
    const std::string dir = argv[2];
    char* fake_argv[] = { argv[0], nullptr };
    int fake_argc = 1;
    char** fake = fake_argv;
    amrex::Initialize(fake_argc, fake, false, MPI_COMM_WORLD, [] () {
        ParmParse pp("amrex");
        pp.add("verbose", 0);
        pp.add("signal_handling", 0);
    });
    if (mode == "amrgrids" || mode == "amrsolve" || mode == "amrresid") {
        const int rc = run_amr(mode, dir);
        amrex::Finalize();
        return rc;
    }
    {
        Case c{read_case(dir)};
        const int nx = c.geti("n", 32, 0), ny = c.geti("n", 32, 1), nz = c.geti("n", 32, 2);
        const Box domain(IntVect(0), IntVect(nx-1, ny-1, nz-1));
        RealBox rb({c.getd("prob_lo", 0., 0), c.getd("prob_lo", 0., 1), c.getd("prob_lo", 0., 2)},
                   {c.getd("prob_hi", 1., 0), c.getd("prob_hi", 1., 1), c.getd("prob_hi", 1., 2)});
        Array<int,3> is_per{c.geti("periodic", 0, 0), c.geti("periodic", 0, 1), c.geti("periodic", 0, 2)};
        Geometry geom(domain, rb, CoordSys::cartesian, is_per);
        BoxArray ba = make_grids(c, domain);
        DistributionMapping dm(ba);
        const std::string op = c.gets("op", "poisson");
        std::ofstream res(dir + "/result.txt");
        res.precision(17);

        if (mode == "fb") {
            // per-box grown FAB data in box order, x fastest
            MultiFab mf(ba, dm, 1, 1);
            size_t total = 0;
            for (int b = 0; b < ba.size(); ++b) { total += amrex::grow(ba[b], 1).numPts(); }
            auto in = read_bin(dir + "/fb_in.bin", total);
            size_t off = 0;
            std::vector<size_t> offs(ba.size());
            for (int b = 0; b < ba.size(); ++b) { offs[b] = off; off += amrex::grow(ba[b], 1).numPts(); }
            for (MFIter mfi(mf); mfi.isValid(); ++mfi) {
                std::copy(in.begin() + offs[mfi.index()],
                          in.begin() + offs[mfi.index()] + mfi.fabbox().numPts(), mf[mfi].dataPtr());
            }
            mf.FillBoundary(geom.periodicity(), c.geti("cross", 1) != 0);
            std::vector<double> out(total);
            for (MFIter mfi(mf); mfi.isValid(); ++mfi) {
                std::copy(mf[mfi].dataPtr(), mf[mfi].dataPtr() + mfi.fabbox().numPts(),
                          out.begin() + offs[mfi.index()]);
            }
            write_bin(dir + "/fb_out.bin", out);
            res << "nboxes " << ba.size() << "\n";
        } else {
            LPInfo info = make_info(c);
            std::unique_ptr<MLLinOp> linop;
            HierProbe<MLPoisson>* pois = nullptr;
            HierProbe<MLABecLaplacian>* abec = nullptr;
            if (op == "poisson") {
                pois = new HierProbe<MLPoisson>({geom}, {ba}, {dm}, info);
                setup_op(*pois, c);
                linop.reset(pois);
            } else {
                abec = new HierProbe<MLABecLaplacian>({geom}, {ba}, {dm}, info);
                setup_op(*abec, c);
                linop.reset(abec);
            }
            const auto& grids = pois ? pois->grids() : abec->grids();

            if (mode == "hier") {
                std::ofstream hs(dir + "/hier.txt");
                for (int lev = 0; lev < (int)grids[0].size(); ++lev) {
                    const BoxArray& g = grids[0][lev];
                    hs << "level " << lev << " " << g.size() << "\n";
                    for (int b = 0; b < g.size(); ++b) {
                        const Box& bx = g[b];
                        hs << bx.smallEnd(0) << " " << bx.smallEnd(1) << " " << bx.smallEnd(2) << " "
                           << bx.bigEnd(0) << " " << bx.bigEnd(1) << " " << bx.bigEnd(2) << "\n";
                    }
                }
            } else {
                // sol holds the initial guess in its valid cells and the
                // Dirichlet boundary values in its ghost cells
                const int sol_ngrow = c.geti("sol_ngrow", 1);
                MultiFab sol(ba, dm, 1, sol_ngrow);
                MultiFab rhs(ba, dm, 1, 0);
                Global gs{nx+2, ny+2, nz+2, -1, -1, -1, {}};
                const size_t ngs = (size_t)(nx+2)*(ny+2)*(nz+2);
                gs.v = c.has("sol_file") ? read_bin(dir + "/" + c.gets("sol_file", ""), ngs)
                                         : std::vector<double>(ngs, 0.0);
                sol.setVal(0.0);
                fill_from_global(sol, gs, 1);
                Global gr{nx, ny, nz, 0, 0, 0, {}};
                gr.v = c.has("rhs_file") ? read_bin(dir + "/" + c.gets("rhs_file", ""), (size_t)nx*ny*nz)
                                         : std::vector<double>((size_t)nx*ny*nz, 0.0);
                fill_from_global(rhs, gr, 0);
                // coarse data for the coarse/fine faces of a level that does
                // not cover its domain (set before setLevelBC, which reads it)
                MultiFab crse;
                if (c.geti("crse_ratio", 0) > 0) {
                    const int r = c.geti("crse_ratio", 2);
                    const Box cdom = amrex::coarsen(domain, r);
                    BoxArray cba(cdom);
                    cba.maxSize(c.geti("crse_mgs", 32));
                    crse.define(cba, DistributionMapping(cba), 1, 0);
                    Global gc{cdom.length(0), cdom.length(1), cdom.length(2), 0, 0, 0,
                              read_bin(dir + "/" + c.gets("crse_file", "crse.bin"), (size_t)cdom.numPts())};
                    fill_from_global(crse, gc, 0);
                    linop->setCoarseFineBC(&crse, r);
                }
                linop->setLevelBC(0, &sol);
                if (abec) {
                    abec->setScalars(c.getd("alpha", 1.0), c.getd("beta", 1.0));
                    MultiFab acoef(ba, dm, 1, 0);
                    if (c.has("a_file")) {
                        Global ga{nx, ny, nz, 0, 0, 0, read_bin(dir + "/" + c.gets("a_file", ""), (size_t)nx*ny*nz)};
                        fill_from_global(acoef, ga, 0);
                    } else {
                        acoef.setVal(c.getd("a_const", 1.0));
                    }
                    abec->setACoeffs(0, acoef);
                    Array<MultiFab,3> face;
                    for (int d = 0; d < 3; ++d) {
                        face[d].define(amrex::convert(ba, IntVect::TheDimensionVector(d)), dm, 1, 0);
                        const std::string key = std::string("b") + char('x'+d) + "_file";
                        if (c.has(key)) {
                            Global gb{nx + (d==0), ny + (d==1), nz + (d==2), 0, 0, 0, {}};
                            gb.v = read_bin(dir + "/" + c.gets(key, ""), (size_t)gb.nx*gb.ny*gb.nz);
                            fill_from_global(face[d], gb, 0);
                        } else {
                            face[d].setVal(c.getd("b_const", 1.0));
                        }
                    }
                    abec->setBCoeffs(0, amrex::GetArrOfConstPtrs(face));
                }
                MLMG mlmg(*linop);
                mlmg.setVerbose(c.geti("verbose", 0));
                mlmg.setMaxIter(c.geti("max_iter", 200));
                mlmg.setMaxFmgIter(c.geti("max_fmg_iter", 0));
                if (c.geti("fixed_iter", 0) > 0) { mlmg.setFixedIter(c.geti("fixed_iter", 0)); }
                mlmg.setBottomSolver(static_cast<MLMG::BottomSolver>(c.geti("bottom_solver", 2)));
                mlmg.setBottomMaxIter(c.geti("bottom_maxiter", 200));
                mlmg.setBottomVerbose(0);
                mlmg.setFinalFillBC(c.geti("final_fill_bc", 0));
                if (mode == "resid") {
                    MultiFab res(ba, dm, 1, 0);
                    mlmg.compResidual({&res}, {&sol}, {&rhs});
                    Global go{nx, ny, nz, 0, 0, 0, std::vector<double>((size_t)nx*ny*nz)};
                    copy_to_global(res, go);
                    write_bin(dir + "/res.bin", go.v);
                } else if (mode == "apply") {
                    MultiFab out(ba, dm, 1, 0);
                    mlmg.apply({&out}, {&sol});
                    Global go{nx, ny, nz, 0, 0, 0, std::vector<double>((size_t)nx*ny*nz)};
                    copy_to_global(out, go);
                    write_bin(dir + "/out.bin", go.v);
                } else {
                    const int nrep = c.geti("repeat", 1);
                    std::vector<double> times;
                    MultiFab sol0(ba, dm, 1, sol_ngrow);
                    MultiFab::Copy(sol0, sol, 0, 0, 1, sol_ngrow);
                    Real resid = 0;
                    for (int r = 0; r < nrep; ++r) {
                        MultiFab::Copy(sol, sol0, 0, 0, 1, sol_ngrow);
                        auto t0 = std::chrono::steady_clock::now();
                        resid = mlmg.solve({&sol}, {&rhs}, c.getd("tol_rel", 1e-10), c.getd("tol_abs", 0.0));
                        auto t1 = std::chrono::steady_clock::now();
                        times.push_back(std::chrono::duration<double>(t1 - t0).count());
                    }
                    Global go{nx, ny, nz, 0, 0, 0, std::vector<double>((size_t)nx*ny*nz)};
                    copy_to_global(sol, go);
                    write_bin(dir + "/phi.bin", go.v);
                    if (sol_ngrow != 1) {
                        std::vector<double> fabs;
                        for (int b = 0; b < ba.size(); ++b) {
                            const FArrayBox& fab = sol[b];
                            fabs.insert(fabs.end(), fab.dataPtr(), fab.dataPtr() + fab.box().numPts());
                        }
                        write_bin(dir + "/phi_fabs.bin", fabs);
                    }
                    if (mode == "flux") {
                        // MLMG::getFluxes (with the solution passed explicitly) and
                        // MLMG::getGradSolution on face MultiFabs
                        Array<MultiFab,3> flux, grad;
                        for (int d = 0; d < 3; ++d) {
                            const BoxArray fba = amrex::convert(ba, IntVect::TheDimensionVector(d));
                            flux[d].define(fba, dm, 1, 0);
                            grad[d].define(fba, dm, 1, 0);
                        }
                        mlmg.getFluxes({amrex::GetArrOfPtrs(flux)}, {&sol}, MLMG::Location::FaceCenter);
                        mlmg.getGradSolution({amrex::GetArrOfPtrs(grad)});
                        for (int d = 0; d < 3; ++d) {
                            Global gf{nx + (d==0), ny + (d==1), nz + (d==2), 0, 0, 0, {}};
                            gf.v.assign((size_t)gf.nx*gf.ny*gf.nz, 0.0);
                            copy_to_global(flux[d], gf);
                            write_bin(dir + "/f" + char('x'+d) + ".bin", gf.v);
                            copy_to_global(grad[d], gf);
                            write_bin(dir + "/g" + char('x'+d) + ".bin", gf.v);
                        }
                    }
                    res << "final_resid " << resid << "\n";
                    res << "init_resid " << mlmg.getInitResidual() << "\n";
                    res << "rhs_norm " << mlmg.getInitRHS() << "\n";
                    res << "niters " << mlmg.getNumIters() << "\n";
                    res << "history";
                    for (auto h : mlmg.getResidualHistory()) { res << " " << h; }
                    res << "\ncg_iters";
                    for (auto h : mlmg.getNumCGIters()) { res << " " << h; }
                    res << "\nsolve_seconds";
                    for (auto t : times) { res << " " << t; }
                    res << "\nthreads " << omp_get_max_threads() << "\n";
                }
            }
        }
    }
    amrex::Finalize();
    return 0;
}
