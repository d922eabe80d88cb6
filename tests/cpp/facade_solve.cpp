// A solve written against the reference's C++ API (names and signatures of
// amrex::BoxArray, DistributionMapping, Geometry, MultiFab, MLPoisson /
// MLABecLaplacian, MLMG), compiled against the GB300 library's C++ facade.
//
//   facade_solve n max_grid_size rhs.bin phi_out.bin mixed
//
// rhs.bin: n^3 float64 values, x fastest; phi_out.bin receives the solution
// the same way.  Homogeneous Dirichlet on every face, tol_rel 1e-10.
#include <mlmg_gb300.H>

#include <cstdio>
#include <cstdlib>
#include <vector>

namespace amrex = amrex_gb300;

int main (int argc, char** argv)
{
    if (argc < 6) { std::fprintf(stderr, "usage: facade_solve n mgs rhs.bin phi.bin mixed\n"); return 2; }
    const int n = std::atoi(argv[1]), mgs = std::atoi(argv[2]);
    const bool mixed = std::atoi(argv[5]) != 0;
    std::vector<double> g((size_t)n * n * n);
    std::FILE* f = std::fopen(argv[3], "rb");
    if (!f || std::fread(g.data(), sizeof(double), g.size(), f) != g.size()) { std::fprintf(stderr, "bad rhs\n"); return 2; }
    std::fclose(f);
    try {
        const amrex::Box domain(amrex::IntVect(0), amrex::IntVect(n - 1));
        amrex::BoxArray ba(domain);
        ba.maxSize(mgs);
        amrex::DistributionMapping dm(ba);
        amrex::Geometry geom(domain, amrex::RealBox({0., 0., 0.}, {1., 1., 1.}), 0, {0, 0, 0});
        amrex::MultiFab sol(ba, dm, 1, 1);
        amrex::MultiFab rhs(ba, dm, 1, 0);
        auto at = [&] (int i, int j, int k) { return ((size_t)k * n + j) * n + i; };
        for (int b = 0; b < rhs.size(); ++b) {
            const amrex::Box bx = ba[b];
            std::vector<double> fab(rhs.fabSize(b));
            size_t q = 0;
            for (int k = bx.smallEnd()[2]; k <= bx.bigEnd()[2]; ++k)
            for (int j = bx.smallEnd()[1]; j <= bx.bigEnd()[1]; ++j)
            for (int i = bx.smallEnd()[0]; i <= bx.bigEnd()[0]; ++i) { fab[q++] = g[at(i, j, k)]; }
            rhs.copyFromHost(b, fab.data());
        }
        sol.setVal(0.0);

        amrex::MLPoisson op({geom}, {ba}, {dm});
        using BC = amrex::LinOpBCType;
        op.setDomainBC({BC::Dirichlet, BC::Dirichlet, BC::Dirichlet}, {BC::Dirichlet, BC::Dirichlet, BC::Dirichlet});
        op.setLevelBC(0, nullptr);
        amrex::MLMG mlmg(op);
        mlmg.setMaxIter(200);
        mlmg.setMixedPrecision(mixed);
        mlmg.setCudaGraph(mixed);
        const amrex::Real resid = mlmg.solve({&sol}, {&rhs}, 1e-10, 0.0);

        for (int b = 0; b < sol.size(); ++b) {
            const amrex::Box bx = ba[b];
            std::vector<double> fab(sol.fabSize(b));
            sol.copyToHost(b, fab.data());
            const int sx = bx.length(0) + 2, sy = bx.length(1) + 2;
            for (int k = bx.smallEnd()[2]; k <= bx.bigEnd()[2]; ++k)
            for (int j = bx.smallEnd()[1]; j <= bx.bigEnd()[1]; ++j)
            for (int i = bx.smallEnd()[0]; i <= bx.bigEnd()[0]; ++i) {
                const size_t q = ((size_t)(k - bx.smallEnd()[2] + 1) * sy + (j - bx.smallEnd()[1] + 1)) * sx
                               + (i - bx.smallEnd()[0] + 1);
                g[at(i, j, k)] = fab[q];
            }
        }
        std::FILE* o = std::fopen(argv[4], "wb");
        std::fwrite(g.data(), sizeof(double), g.size(), o);
        std::fclose(o);
        std::printf("iters %d resid %.6e init_rhs %.6e\n", mlmg.getNumIters(), resid, mlmg.getInitRHS());
    } catch (const std::exception& e) {
        std::fprintf(stderr, "error: %s\n", e.what());
        return 1;
    }
    return 0;
}
