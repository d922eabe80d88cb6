// AMR composite MLMG (MLMGT::solve over several AMR levels, refinement ratio
// 2, MLPoisson or MLABecLaplacian): host orchestration of MLMGT::oneIter (AMReX_MLMG.H:1227-1293)
// over one engine per AMR level, with the coarse/fine kernels of
// amr_kernels.cuh.  FP64 throughout, or (precision 1) FP32 corrections --
// the V-cycle of AMR level 0, the fine levels' smoothing sweeps and the
// correction residuals -- inside the FP64 composite residual, reflux,
// average-down, solution update and norms.
#include "amr.hpp"
#include "engine_impl.cuh"
#include "amr_kernels.cuh"

#include <array>
#include <climits>
#include <cmath>
#include <map>

namespace mlmg {

namespace {

template <typename T>
void upload_or_keep (DevBuf<T>& b, const std::vector<T>& v, cudaStream_t st)
{
    if (!v.empty()) { b.upload(v, st); }
}

unsigned blocks_for (long long n, int threads) { return (unsigned)((n + threads - 1) / threads); }

// wrap cell c into the level domain `dom` along the periodic directions;
// false if it lies outside along a non-periodic one
bool wrap_cell (const Box3& dom, const int* periodic, int* c)
{
    for (int d = 0; d < 3; ++d) {
        if (c[d] >= dom.lo[d] && c[d] <= dom.hi[d]) { continue; }
        if (!periodic[d]) { return false; }
        const int n = dom.len(d);
        c[d] = dom.lo[d] + (((c[d] - dom.lo[d]) % n) + n) % n;
    }
    return true;
}

// the periodic image shifts of a level domain (0 included): multiples -1, 0, 1
// of the domain length along each periodic direction
std::vector<std::array<int, 3>> image_shifts (const Box3& dom, const int* periodic)
{
    std::vector<std::array<int, 3>> out;
    for (int sz = -1; sz <= 1; ++sz)
    for (int sy = -1; sy <= 1; ++sy)
    for (int sx = -1; sx <= 1; ++sx) {
        const int sv[3] = {sx, sy, sz};
        bool ok = true;
        for (int d = 0; d < 3; ++d) { if (sv[d] != 0 && !periodic[d]) { ok = false; } }
        if (ok) { out.push_back({sx * dom.len(0), sy * dom.len(1), sz * dom.len(2)}); }
    }
    return out;
}

} // namespace

// One AMR level: its engine and, towards the next coarser level (l > 0) or
// the next finer one (l < finest), the coupling tables.
struct AmrLevelData {
    std::unique_ptr<Engine> eng;
    Engine::Impl* I = nullptr;
    // -- as the fine level of level l-1 --
    std::vector<PatchDesc> h_cfd;           // coarse buffer layout per fine patch (coarsened patch + 1 ghost)
    DevBuf<PatchDesc> cfd;
    long long cf_n = 0;
    DevBuf<double> cf64;
    DevBuf<float> cf32;
    DevBuf<CopyTag> gtags;                  // gather: dst fine patch, src coarse patch
    DevBuf<long long> gstart;
    int ngtag = 0;
    long long ngcell = 0;
    DevBuf<int2> cff;                       // coarse/fine (patch, face) pairs
    DevBuf<long long> cffstart;
    GhostWork cfw{};                        // face-cell walk over them (no copy tags)
    DevBuf<int8_t> bflags;                  // per Dirichlet-value slot: BF_* bits
    DevBuf<int4> bitems;                    // the coarse/fine ghost cells (k_amr_bndry_list)
    int nbitems = 0;
    DevBuf<double> bcor;                    // boundary values of the correction (physical slots 0)
    DevBuf<long long> nbr;                  // per Dirichlet-value slot: element of the covering patch's cell, or -1
                                            // (colour passes without ghost fills; empty if a closure has 4 points)
    // fused two-colour sweeps of the level (MLPoisson, FP32 corrections): the
    // fused-sweep tiles whose halo meets no face shared with another patch,
    // the others (colour passes), the sweeps' second buffer and tensor maps
    // (per patch, over the correction, the hold and the second buffer)
    DevBuf<int4> fz_safe, fz_rest;
    int nsafe = 0, nrest = 0;
    DevBuf<float> fz_buf;
    DevBuf<CUtensorMap> fz_maps;
    DevBuf<double> hold64;                  // cor_hold of the AMR level
    DevBuf<float> hold32;
    void* cor_p = nullptr;                  // the level's correction buffer (swapped with the hold)
    void* hold_p = nullptr;
    // -- as the coarse level of level l+1 --
    DevBuf<CopyTag> atags;                  // average-down: dst coarse patch, src fine patch
    DevBuf<long long> astart;
    int natag = 0;
    long long nacell = 0;
    DevBuf<int8_t> covered;                 // per element: 1 where the finer level covers the cell
    DevBuf<RefluxCell> rcells;
    DevBuf<RefluxFace> rfaces;
    int nrcell = 0;
    RefluxParams rprm{};
    // MLABecLaplacian: face average-down tags per direction (coarse faces of
    // the coarsened fine patches)
    DevBuf<CopyTag> ftags[3];
    DevBuf<long long> fstart[3];
    int nftag[3] = {0, 0, 0};
    long long nfcell[3] = {0, 0, 0};
};

struct AmrEngine::Impl {
    AmrEngine& A;
    AmrProblem prob;
    std::vector<AmrLevelData> lev;
    int nl = 0;
    int own_launches = 0;
    PinnedBuf<double> h_norm;
    cudaGraphExec_t graph_exec = nullptr;
    int graph_launches = 0;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;

    explicit Impl (AmrEngine& a) : A(a) {}
    ~Impl () {
        if (graph_exec) { cudaGraphExecDestroy(graph_exec); }
        if (ev0) { cudaEventDestroy(ev0); }
        if (ev1) { cudaEventDestroy(ev1); }
    }
    cudaStream_t st () const { return A.m_stream; }
    bool mixed () const { return A.m_opt.precision == 1; }
    void launched (int n = 1) { own_launches += n; }
    LevelData& L (int l) { return lev[l].I->lev[0]; }
    // a kernel on the engine's stream, as a programmatic dependent launch
    // unless the option is off (every kernel of the path starts with
    // griddepcontrol.wait before it touches the previous kernels' data)
    template <typename... KArgs, typename... Args>
    void launch (void (*kern)(KArgs...), dim3 grid, dim3 block, size_t smem, Args&&... args)
    {
        cudaLaunchConfig_t cfg{};
        cfg.gridDim = grid;
        cfg.blockDim = block;
        cfg.dynamicSmemBytes = smem;
        cfg.stream = st();
        cudaLaunchAttribute at[1];
        at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
        at[0].val.programmaticStreamSerializationAllowed = 1;
        cfg.attrs = at;
        cfg.numAttrs = A.m_opt.pdl ? 1 : 0;
        MLMG_CUDA_CHECK(cudaLaunchKernelEx(&cfg, kern, std::forward<Args>(args)...));
    }

    bool abec () const { return prob.is_abec != 0; }
    void build ();
    void build_fine_tables (int l);
    void build_coarse_tables (int c);
    void average_down_coefficients ();
    RefluxCoef reflux_coef (int c);

    // operations
    // exact: the reference's operation order (MLMGT::compResidual) even in
    // mixed precision
    void solution_residual (int l, bool update, bool want_norm = false, bool exact = false);
    void reflux (int c);
    void avgdown (int c, const double* fine, double* crse, float* crse32 = nullptr);
    template <typename T> void gather (int l, const T* crse);
    template <typename T> T* cor (int l);
    template <typename T> T* hold (int l);
    template <typename T> void mini_cycle (int l, const T* rhs);
    void build_fused_tiles (int l, const std::vector<long long>& nb);
    template <typename T, typename TB, typename TO> void cor_residual (int l, bool inhomog, const TB* b, TO* out);
    template <typename T> void one_iter (int iter);
    void norm_start (int l, const double* x, bool masked, int slot);
    void fine_residual_and_norm ();
};

template <> double* AmrEngine::Impl::cor<double> (int l) { return (double*)lev[l].cor_p; }
template <> float* AmrEngine::Impl::cor<float> (int l) { return (float*)lev[l].cor_p; }
template <> double* AmrEngine::Impl::hold<double> (int l) { return (double*)lev[l].hold_p; }
template <> float* AmrEngine::Impl::hold<float> (int l) { return (float*)lev[l].hold_p; }

// ------------------------------------------------------------------ build --
void AmrEngine::Impl::build ()
{
    nl = (int)prob.levels.size();
    MLMG_REQUIRE(nl >= 2 && nl <= 8, ERR_ARGS, "an AMR solve needs 2 to 8 levels");
    lev.resize(nl);
    for (int l = 0; l < nl; ++l) {
        SolveProblem pr;
        SolveSpec& S = pr.spec;
        S.geom = prob.geom;
        S.geom.domain = refine(prob.geom.domain, 1 << l);
        if (l == 0) {
            S.levels = define_grids(S.geom, prob.levels[0].boxes, prob.info);
        } else {
            LevelGrids G;
            G.geom = S.geom;
            G.boxes = prob.levels[l].boxes;
            G.derived = 1;
            S.levels.push_back(G);
            for (const auto& b : G.boxes) {
                MLMG_REQUIRE(S.geom.domain.contains(b.lo[0], b.lo[1], b.lo[2]) &&
                             S.geom.domain.contains(b.hi[0], b.hi[1], b.hi[2]), ERR_ARGS,
                             "AMR level box outside its domain");
                MLMG_REQUIRE(refine(coarsen(b, 2), 2) == b, ERR_ARGS,
                             "AMR level boxes must be coarsenable by the refinement ratio 2");
            }
        }
        for (int d = 0; d < 3; ++d) {
            S.lobc[d] = prob.lobc[d]; S.hibc[d] = prob.hibc[d];
            S.dx0[d] = (S.geom.prob_hi[d] - S.geom.prob_lo[d]) / (double)S.geom.domain.len(d);
        }
        S.maxorder = prob.maxorder;
        S.is_abec = prob.is_abec;
        S.alpha = prob.is_abec ? prob.alpha : 0.0;
        S.beta = prob.is_abec ? prob.beta : 1.0;
        S.crse_ratio = (l > 0) ? 2 : 1;
        S.amr_fine = (l > 0) ? 1 : 0;
        pr.boxes = prob.levels[l].boxes;
        pr.levelbc = prob.levels[l].levelbc;
        if (prob.is_abec) {
            pr.acoef = prob.levels[l].acoef;
            for (int d = 0; d < 3; ++d) { pr.bcoef[d] = prob.levels[l].bcoef[d]; }
        }
        EngineOptions o = A.m_opt;
        o.max_fmg_iter = 0;
        o.transpose = 0;
        std::vector<SolveProblem> probs{pr};
        lev[l].eng = std::make_unique<Engine>(std::move(probs), o, st());
        lev[l].I = &lev[l].eng->impl();
    }
    // proper nesting: a fine box coarsened and grown by one lies in the
    // coarser level (or outside the domain), which the coarse/fine
    // interpolation, the reflux and the correction interpolation rely on
    for (int l = 1; l < nl; ++l) {
        const BoxLocator cl(prob.levels[l - 1].boxes);
        const Box3 cdom = refine(prob.geom.domain, 1 << (l - 1));
        for (const auto& b : prob.levels[l].boxes) {
            const Box3 g = grow(coarsen(b, 2), 1);
            for (int k = g.lo[2]; k <= g.hi[2]; ++k)
            for (int j = g.lo[1]; j <= g.hi[1]; ++j)
            for (int i = g.lo[0]; i <= g.hi[0]; ++i) {
                int c[3] = {i, j, k};
                if (!wrap_cell(cdom, prob.geom.periodic, c)) { continue; }
                MLMG_REQUIRE(cl.find(c[0], c[1], c[2]) >= 0, ERR_ARGS,
                             "AMR levels are not properly nested (a coarsened fine box grown by one leaves the coarser level)");
            }
        }
    }
    for (int l = 0; l < nl; ++l) {
        AmrLevelData& D = lev[l];
        LevelData& Ld = L(l);
        const size_t n = (size_t)Ld.meta.nelem;
        if (mixed()) {
            D.cor_p = Ld.cor32.p;
            if (l > 0 && l < nl - 1) { D.hold32.alloc(n); D.hold32.zero(st()); D.hold_p = D.hold32.p; }
        } else {
            D.cor_p = Ld.cor.p;
            if (l > 0 && l < nl - 1) { D.hold64.alloc(n); D.hold64.zero(st()); D.hold_p = D.hold64.p; }
        }
        if (l > 0) { build_fine_tables(l); }
        if (l < nl - 1) { build_coarse_tables(l); }
    }
    if (abec()) { average_down_coefficients(); }
    h_norm.alloc(4 * (size_t)nl + 4);
    MLMG_CUDA_CHECK(cudaEventCreate(&ev0));
    MLMG_CUDA_CHECK(cudaEventCreate(&ev1));
    MLMG_CUDA_CHECK(cudaStreamSynchronize(st()));
}

void AmrEngine::Impl::build_fine_tables (int l)
{
    AmrLevelData& D = lev[l];
    const PatchLevel& Mf = L(l).meta;
    const PatchLevel& Mc = L(l - 1).meta;
    // coarse buffers: the coarsened fine patch and one ghost layer
    long long cursor = 0;
    D.h_cfd.clear();
    for (const PatchDesc& P : Mf.patches) {
        Box3 pb;
        for (int d = 0; d < 3; ++d) { pb.lo[d] = P.lo[d]; pb.hi[d] = P.hi[d]; }
        const Box3 cb = coarsen(pb, 2);
        PatchDesc G{};
        for (int d = 0; d < 3; ++d) { G.lo[d] = cb.lo[d]; G.hi[d] = cb.hi[d]; }
        G.sx = cb.len(0) + 2;
        G.sxy = (long long)G.sx * (cb.len(1) + 2);
        G.base = cursor + G.sxy + G.sx + 1;
        cursor += G.sxy * (cb.len(2) + 2);
        D.h_cfd.push_back(G);
    }
    D.cf_n = std::max<long long>(cursor, 1);
    D.cfd.upload(D.h_cfd, st());
    D.cf64.alloc((size_t)D.cf_n);
    if (mixed()) { D.cf32.alloc((size_t)D.cf_n); }
    // gather tags: every coarse patch's valid cells (and their periodic
    // images: source cell = buffer cell - shift) inside each grown buffer
    const Box3 cdom = refine(prob.geom.domain, 1 << (l - 1));
    const auto cshifts = image_shifts(cdom, prob.geom.periodic);
    std::vector<CopyTag> tags;
    std::vector<long long> start{0};
    for (int p = 0; p < (int)Mf.patches.size(); ++p) {
        Box3 g;
        for (int d = 0; d < 3; ++d) { g.lo[d] = D.h_cfd[p].lo[d] - 1; g.hi[d] = D.h_cfd[p].hi[d] + 1; }
        for (int cp = 0; cp < (int)Mc.patches.size(); ++cp) {
            Box3 cb;
            for (int d = 0; d < 3; ++d) { cb.lo[d] = Mc.patches[cp].lo[d]; cb.hi[d] = Mc.patches[cp].hi[d]; }
            for (const auto& sh : cshifts) {
                const Box3 is = intersect(g, shift(cb, sh.data()));
                if (!is.ok()) { continue; }
                CopyTag t{};
                t.dst = p; t.src = cp; t.box = is;
                for (int d = 0; d < 3; ++d) { t.shift[d] = sh[d]; }
                tags.push_back(t);
                start.push_back(start.back() + is.npts());
            }
        }
    }
    D.ngtag = (int)tags.size();
    D.ngcell = start.back();
    upload_or_keep(D.gtags, tags, st());
    D.gstart.upload(start, st());
    // coarse/fine faces and the neighbourhood flags of their ghost cells
    const Box3 fdom = refine(prob.geom.domain, 1 << l);
    const BoxLocator floc(prob.levels[l].boxes);
    auto notcov = [&] (int i, int j, int k) {
        int c[3] = {i, j, k};
        return wrap_cell(fdom, prob.geom.periodic, c) && floc.find(c[0], c[1], c[2]) < 0;
    };
    std::vector<int8_t> flags(L(l).bcval.n, 0);
    std::vector<int4> bitems;
    std::vector<int2> faces;
    std::vector<long long> fstart{0};
    for (int p = 0; p < (int)Mf.patches.size(); ++p) {
        const PatchDesc& P = Mf.patches[p];
        for (int f = 0; f < 6; ++f) {
            const FaceBC& F = P.face[f];
            const int d = f % 3;
            if (F.on_domain && !prob.geom.periodic[d]) { continue; }   // physical face: the level's own BC values
            const int t1 = (d == 0) ? 1 : 0, t2 = (d == 2) ? 1 : 2;
            const int g = (f >= 3) ? P.hi[d] + 1 : P.lo[d] - 1;
            const int n1 = P.hi[t1] - P.lo[t1] + 1, n2 = P.hi[t2] - P.lo[t2] + 1;
            faces.push_back(make_int2(p, f));
            fstart.push_back(fstart.back() + (long long)n1 * n2);
            for (int v2 = 0; v2 < n2; ++v2)
            for (int v1 = 0; v1 < n1; ++v1) {
                int c[3];
                c[d] = g; c[t1] = P.lo[t1] + v1; c[t2] = P.lo[t2] + v2;
                int fl = 0;
                if (notcov(c[0], c[1], c[2])) {
                    fl |= BF_SELF;
                    auto nc_at = [&] (int a1, int a2) {
                        int e[3] = {c[0], c[1], c[2]};
                        e[t1] += a1; e[t2] += a2;
                        return notcov(e[0], e[1], e[2]);
                    };
                    if (nc_at(-2, 0)) { fl |= BF_T1LO; }
                    if (nc_at(2, 0)) { fl |= BF_T1HI; }
                    if (nc_at(0, -2)) { fl |= BF_T2LO; }
                    if (nc_at(0, 2)) { fl |= BF_T2HI; }
                    if (nc_at(-2, -2) && nc_at(2, -2) && nc_at(-2, 2) && nc_at(2, 2)) { fl |= BF_CROSS; }
                    const long long slot = F.bcval_off + (long long)v2 * n1 + v1;
                    const long long q = cidx(D.h_cfd[p], c[0] >> 1, c[1] >> 1, c[2] >> 1);
                    MLMG_REQUIRE(slot < INT_MAX && q < INT_MAX, ERR_UNSUPPORTED, "coarse/fine tables above 2^31 entries");
                    bitems.push_back(make_int4((int)slot, (int)q, p,
                                               fl | ((c[t1] & 1) << 6) | ((c[t2] & 1) << 7) | (f << 8)));
                }
                flags[(size_t)(F.bcval_off + (long long)v2 * n1 + v1)] = (int8_t)fl;
            }
        }
    }
    upload_or_keep(D.cff, faces, st());
    D.cffstart.upload(fstart, st());
    D.cfw = GhostWork{D.cff.p, D.cffstart.p, (int)faces.size(), nullptr, nullptr, 0, fstart.back(), 0};
    D.bflags.upload(flags, st());
    D.nbitems = (int)bitems.size();
    upload_or_keep(D.bitems, bitems, st());
    D.bcor.alloc(L(l).bcval.n);
    D.bcor.zero(st());
    // neighbour table of the ghost-free colour passes: every copy-tag cell
    // (a ghost covered by another patch) points at its source cell
    bool short_closures = !abec();     // the ghost-free passes have MLPoisson's stencil
    for (const PatchDesc& P : Mf.patches) {
        for (int f = 0; f < 6; ++f) {
            if (P.face[f].type == BC_DIRICHLET && P.face[f].nx > 3) { short_closures = false; }
        }
    }
    if (short_closures) {
        std::vector<long long> nb(L(l).bcval.n, -1);
        for (const CopyTag& t : Mf.tags) {
            const PatchDesc& P = Mf.patches[t.dst];
            const PatchDesc& Q = Mf.patches[t.src];
            for (int k = t.box.lo[2]; k <= t.box.hi[2]; ++k)
            for (int j = t.box.lo[1]; j <= t.box.hi[1]; ++j)
            for (int i = t.box.lo[0]; i <= t.box.hi[0]; ++i) {
                int f;
                if (i < P.lo[0]) { f = 0; } else if (i > P.hi[0]) { f = 3; }
                else if (j < P.lo[1]) { f = 1; } else if (j > P.hi[1]) { f = 4; }
                else if (k < P.lo[2]) { f = 2; } else { f = 5; }
                const int nx = P.hi[0] - P.lo[0] + 1, ny = P.hi[1] - P.lo[1] + 1;
                const int d = f % 3;
                const long long u = (d == 0) ? (long long)(k - P.lo[2]) * ny + (j - P.lo[1])
                                  : (d == 1) ? (long long)(k - P.lo[2]) * nx + (i - P.lo[0])
                                             : (long long)(j - P.lo[1]) * nx + (i - P.lo[0]);
                nb[(size_t)(P.face[f].bcval_off + u)] = cidx(Q, i - t.shift[0], j - t.shift[1], k - t.shift[2]);
            }
        }
        D.nbr.upload(nb, st());
        if (mixed() && A.m_opt.fused_smoother && A.m_opt.fused_fine) { build_fused_tiles(l, nb); }
    }
}

// The fused-sweep tiles of fine level l: a tile is safe when no face of its
// patch that its halo (the tile grown by one) reaches has a ghost covered by
// another patch within that halo's extent; such a tile's two colours can run
// in one fused sweep.  The others get colour passes.
void AmrEngine::Impl::build_fused_tiles (int l, const std::vector<long long>& nb)
{
    AmrLevelData& D = lev[l];
    LevelData& Ld = L(l);
    const PatchLevel& M = Ld.meta;
    std::vector<int4> safe, rest;
    for (int p = 0; p < (int)M.patches.size(); ++p) {
        const PatchDesc& P = M.patches[p];
        const int nx = P.hi[0] - P.lo[0] + 1, ny = P.hi[1] - P.lo[1] + 1;
        const int tdim[3] = {FS_TX, FS_TY, FS_TZ};
        for (int z0 = P.lo[2]; z0 <= P.hi[2]; z0 += FS_TZ)
        for (int y0 = P.lo[1]; y0 <= P.hi[1]; y0 += FS_TY)
        for (int x0 = P.lo[0]; x0 <= P.hi[0]; x0 += FS_TX) {
            const int t0[3] = {x0, y0, z0};
            // the tile + 1 clipped to the patch
            int a[3], b[3];
            for (int d = 0; d < 3; ++d) {
                a[d] = std::max(P.lo[d], t0[d] - 1);
                b[d] = std::min(P.hi[d], t0[d] + tdim[d]);
            }
            bool ok = true;
            for (int f = 0; f < 6 && ok; ++f) {
                const int d = f % 3;
                const bool reach = (f < 3) ? (t0[d] == P.lo[d]) : (t0[d] + tdim[d] >= P.hi[d]);
                if (!reach) { continue; }
                const int e1 = (d == 0) ? 1 : 0, e2 = (d == 2) ? 1 : 2;
                const int n1 = (d == 0) ? ny : nx;
                for (int v = a[e2]; v <= b[e2] && ok; ++v) {
                    for (int w = a[e1]; w <= b[e1] && ok; ++w) {
                        const long long u = (long long)(v - P.lo[e2]) * n1 + (w - P.lo[e1]);
                        if (nb[(size_t)(P.face[f].bcval_off + u)] >= 0) { ok = false; }
                    }
                }
            }
            (ok && A.m_opt.fused_fine == 1 ? safe : rest).push_back(make_int4(p, x0, y0, z0));
        }
    }
    D.nsafe = (int)safe.size();
    D.nrest = (int)rest.size();
    D.fz_safe.upload(safe, st());
    D.fz_rest.upload(rest, st());
    D.fz_buf.alloc((size_t)M.nelem);
    D.fz_buf.zero(st());
    const size_t np = M.patches.size();
    std::vector<CUtensorMap> maps(3 * np);
    for (size_t p = 0; p < np; ++p) {
        maps[p] = patch_tensor_map(Ld.cor32.p, M.patches[p]);
        maps[np + p] = D.hold32.p ? patch_tensor_map(D.hold32.p, M.patches[p]) : maps[p];
        maps[2 * np + p] = patch_tensor_map(D.fz_buf.p, M.patches[p]);
    }
    D.fz_maps.upload(maps, st());
}

void AmrEngine::Impl::build_coarse_tables (int c)
{
    AmrLevelData& D = lev[c];
    const PatchLevel& Mc = L(c).meta;
    const PatchLevel& Mf = L(c + 1).meta;
    auto pbox = [] (const PatchDesc& P) {
        Box3 b;
        for (int d = 0; d < 3; ++d) { b.lo[d] = P.lo[d]; b.hi[d] = P.hi[d]; }
        return b;
    };
    // average-down tags and the covered mask
    std::vector<CopyTag> tags;
    std::vector<long long> start{0};
    std::vector<int8_t> cov((size_t)Mc.nelem, 0);
    std::vector<Box3> cfboxes;
    for (int fp = 0; fp < (int)Mf.patches.size(); ++fp) {
        const Box3 cb = coarsen(pbox(Mf.patches[fp]), 2);
        cfboxes.push_back(cb);
        for (int cp = 0; cp < (int)Mc.patches.size(); ++cp) {
            const Box3 is = intersect(cb, pbox(Mc.patches[cp]));
            if (!is.ok()) { continue; }
            CopyTag t{};
            t.dst = cp; t.src = fp; t.box = is;
            tags.push_back(t);
            start.push_back(start.back() + is.npts());
            const PatchDesc& C = Mc.patches[cp];
            for (int k = is.lo[2]; k <= is.hi[2]; ++k)
            for (int j = is.lo[1]; j <= is.hi[1]; ++j)
            for (int i = is.lo[0]; i <= is.hi[0]; ++i) { cov[(size_t)cidx(C, i, j, k)] = 1; }
        }
    }
    D.natag = (int)tags.size();
    D.nacell = start.back();
    upload_or_keep(D.atags, tags, st());
    D.astart.upload(start, st());
    D.covered.upload(cov, st());
    // reflux: every (uncovered coarse cell, face) pair next to a coarsened fine patch
    std::vector<Box3> cpboxes;
    for (const auto& P : Mc.patches) { cpboxes.push_back(pbox(P)); }
    const BoxLocator cfl(cfboxes), cpl(cpboxes);
    const Box3 cdom = refine(prob.geom.domain, 1 << c);
    auto cfl_find = [&] (const int* w) { return cfl.find(w[0], w[1], w[2]); };
    struct E { long long q; int key; RefluxFace f; };
    std::vector<E> ent;
    for (int fp = 0; fp < (int)Mf.patches.size(); ++fp) {
        const Box3& cb = cfboxes[fp];
        const PatchDesc& F = Mf.patches[fp];
        for (int f = 0; f < 6; ++f) {
            const int d = f % 3;
            Box3 ab = cb;
            if (f >= 3) { ab.lo[d] = ab.hi[d] = cb.hi[d] + 1; } else { ab.lo[d] = ab.hi[d] = cb.lo[d] - 1; }
            const int side = (f < 3) ? 1 : 0;     // the coarsened patch lies at +d of a cell below its low face
            for (int k = ab.lo[2]; k <= ab.hi[2]; ++k)
            for (int j = ab.lo[1]; j <= ab.hi[1]; ++j)
            for (int i = ab.lo[0]; i <= ab.hi[0]; ++i) {
                // the coarse cell taking the reflux: (i,j,k) or, past a
                // periodic face, its image inside the domain
                int w[3] = {i, j, k};
                if (!wrap_cell(cdom, prob.geom.periodic, w) || cfl_find(w) >= 0) { continue; }
                const int cp = cpl.find(w[0], w[1], w[2]);
                int n[3] = {i, j, k};
                n[d] += side ? 1 : -1;
                const int cpn = cpl.find(n[0], n[1], n[2]);
                MLMG_REQUIRE(cp >= 0 && cpn >= 0, ERR_ARGS, "AMR levels are not properly nested");
                int fi[3] = {2 * i, 2 * j, 2 * k};
                fi[d] = side ? 2 * n[d] : 2 * n[d] + 1;
                E e;
                e.q = cidx(Mc.patches[cp], w[0], w[1], w[2]);
                e.key = 2 * d + side;
                e.f.qn = cidx(Mc.patches[cpn], n[0], n[1], n[2]);
                int fc[3] = {w[0], w[1], w[2]};
                if (side) { fc[d] += 1; }
                e.f.qb = cidx(Mc.patches[cp], fc[0], fc[1], fc[2]);
                e.f.qf = cidx(F, fi[0], fi[1], fi[2]);
                e.f.fp = fp;
                e.f.dir = d;
                e.f.side = side;
                ent.push_back(e);
            }
        }
    }
    std::sort(ent.begin(), ent.end(), [] (const E& a, const E& b) { return a.q != b.q ? a.q < b.q : a.key < b.key; });
    std::vector<RefluxCell> cells;
    std::vector<RefluxFace> rf;
    for (size_t e = 0; e < ent.size(); ++e) {
        if (cells.empty() || cells.back().q != ent[e].q) { cells.push_back(RefluxCell{ent[e].q, (int)e, 0}); }
        cells.back().ne++;
        rf.push_back(ent[e].f);
    }
    D.nrcell = (int)cells.size();
    upload_or_keep(D.rcells, cells, st());
    upload_or_keep(D.rfaces, rf, st());
    for (int d = 0; d < 3; ++d) {
        D.rprm.dxinv_c[d] = Mc.patches[0].dxinv[d];
        D.rprm.dxinv_f[d] = Mf.patches[0].dxinv[d];
    }
    // face average-down tags: the faces of each coarsened fine patch (its
    // boundary faces included) within the faces of each coarse patch
    if (abec()) {
        // (box in the fine patch's frame; the coarse face is box - shift, so a
        // face on a periodic boundary also reaches its image, as the
        // reference's ParallelCopy with the coarse periodicity does)
        const auto cshifts = image_shifts(cdom, prob.geom.periodic);
        for (int d = 0; d < 3; ++d) {
            std::vector<CopyTag> ft;
            std::vector<long long> fs{0};
            for (int fp = 0; fp < (int)Mf.patches.size(); ++fp) {
                Box3 fb = cfboxes[fp];
                fb.hi[d] += 1;
                for (int cp = 0; cp < (int)Mc.patches.size(); ++cp) {
                    Box3 cb = pbox(Mc.patches[cp]);
                    cb.hi[d] += 1;
                    for (const auto& sh : cshifts) {
                        const Box3 is = intersect(fb, shift(cb, sh.data()));
                        if (!is.ok()) { continue; }
                        CopyTag t{};
                        t.dst = cp; t.src = fp; t.box = is;
                        for (int e = 0; e < 3; ++e) { t.shift[e] = sh[e]; }
                        ft.push_back(t);
                        fs.push_back(fs.back() + is.npts());
                    }
                }
            }
            D.nftag[d] = (int)ft.size();
            D.nfcell[d] = fs.back();
            upload_or_keep(D.ftags[d], ft, st());
            D.fstart[d].upload(fs, st());
        }
    }
}

// MLABecLaplacianT::averageDownCoeffs (AMReX_MLABecLaplacian.H:610-626): from
// the finest AMR level down, a (unless alpha is 0) onto the covered cells and
// b onto the faces of the coarsened fine patches of the next coarser level
// (averageDownCoeffsToCoarseAmrLevel, :693-712); then every level's own MG
// restriction and stencil form again from the averaged coefficients.
void AmrEngine::Impl::average_down_coefficients ()
{
    for (int c = nl - 2; c >= 0; --c) {
        AmrLevelData& D = lev[c];
        LevelData& Lc = L(c);
        LevelData& Lf = L(c + 1);
        if (prob.alpha != 0.0 && D.nacell > 0) {
            launch(k_amr_avgdown<double, double>, blocks_for(D.nacell, 256), 256, 0, Lc.dl, Lf.dl, D.atags.p,
                D.astart.p, D.natag, D.nacell, Lf.a.p, Lc.a.p, (float*)nullptr);
            launched();
        }
        const double* fb[3] = {Lf.bx.p, Lf.by.p, Lf.bz.p};
        double* cb[3] = {Lc.bx.p, Lc.by.p, Lc.bz.p};
        for (int d = 0; d < 3; ++d) {
            if (D.nfcell[d] == 0) { continue; }
            launch(k_amr_avgdown_faces, blocks_for(D.nfcell[d], 256), 256, 0, Lc.dl, Lf.dl, D.ftags[d].p,
                D.fstart[d].p, D.nftag[d], D.nfcell[d], d, fb[d], cb[d]);
            launched();
        }
    }
    MLMG_CUDA_CHECK(cudaGetLastError());
    for (int l = 0; l < nl - 1; ++l) { lev[l].eng->restrict_coefficients(); }
}

RefluxCoef AmrEngine::Impl::reflux_coef (int c)
{
    RefluxCoef co{};
    if (abec()) {
        LevelData& Lc = L(c);
        LevelData& Lf = L(c + 1);
        co.bc[0] = Lc.bx.p; co.bc[1] = Lc.by.p; co.bc[2] = Lc.bz.p;
        co.bf[0] = Lf.bx.p; co.bf[1] = Lf.by.p; co.bf[2] = Lf.bz.p;
        co.beta = prob.beta;
    }
    return co;
}

// ------------------------------------------------------------- operations --
template <> void AmrEngine::Impl::gather<double> (int l, const double* crse)
{
    AmrLevelData& D = lev[l];
    MLMG_CUDA_CHECK(cudaMemsetAsync(D.cf64.p, 0, sizeof(double) * (size_t)D.cf_n, st()));
    if (D.ngcell > 0) {
        launch(k_amr_gather<double>, blocks_for(D.ngcell, 256), 256, 0, L(l - 1).dl, D.cfd.p, D.gtags.p, D.gstart.p,
                                                                         D.ngtag, D.ngcell, crse, D.cf64.p);
        launched();
    }
}

template <> void AmrEngine::Impl::gather<float> (int l, const float* crse)
{
    AmrLevelData& D = lev[l];
    MLMG_CUDA_CHECK(cudaMemsetAsync(D.cf32.p, 0, sizeof(float) * (size_t)D.cf_n, st()));
    if (D.ngcell > 0) {
        launch(k_amr_gather<float>, blocks_for(D.ngcell, 256), 256, 0, L(l - 1).dl, D.cfd.p, D.gtags.p, D.gstart.p,
                                                                        D.ngtag, D.ngcell, crse, D.cf32.p);
        launched();
    }
}

// MLCellLinOpT::solutionResidual (AMReX_MLCellLinOp.H:1219-1236); on a fine
// level with update, the boundary values are first refreshed from the
// coarser level's solution (updateSolBC, :651-664)
void AmrEngine::Impl::solution_residual (int l, bool update, bool want_norm, bool exact)
{
    LevelData& Ld = L(l);
    AmrLevelData& D = lev[l];
    const double* bcv = nullptr;
    if (l > 0) {
        if (update) {
            gather<double>(l, L(l - 1).sol.p);
            if (D.nbitems > 0) {
                launch(k_amr_bndry_list<double>, blocks_for(D.nbitems, 256), 256, 0, (const int4*)D.bitems.p,
                       D.nbitems, (const PatchDesc*)D.cfd.p, (const double*)D.cf64.p, Ld.bcval.p);
                launched();
            }
        }
        bcv = Ld.bcval.p;
    }
    D.I->ghost<double>(0, Ld.sol.p, true, true, bcv);
    Engine::Impl& I = *D.I;
    if (mixed() && !exact) {
        // stencil form (D x - sum s x_nb: 8 FP64 operations per cell instead of
        // 14), with the level's max|r| by atomic max into red_out[0], and the
        // FP32 copy the level's correction solve starts from (the reflux and
        // the average-down that change res afterwards update it too)
        if (want_norm) { MLMG_CUDA_CHECK(cudaMemsetAsync(I.red_out.p, 0, sizeof(double), st())); }
        double* nrm = want_norm ? I.red_out.p : nullptr;
        float* r32 = Ld.res32.p;
        if (abec()) {
            launch(k_residual_s<double, double, true, false, false>, Ld.all.ntiles, kTileBlock, 0, Ld.dl,
                Ld.all.dev(), Ld.res.p, Ld.sol.p, Ld.rhs.p, I.stencil64(0), nullptr, nrm, r32);
        } else {
            launch(k_residual_s<double, double, false, false, false>, Ld.all.ntiles, kTileBlock, 0, Ld.dl,
                Ld.all.dev(), Ld.res.p, Ld.sol.p, Ld.rhs.p, StencilPtrs{}, nullptr, nrm, r32);
        }
        launched();
    } else {
        // the reference's operation order (MLPoissonT::Fapply / MLABecLaplacianT::Fapply),
        // block maxima for the norm
        if (abec()) {
            launch(k_residual<double, double, true>, Ld.all.ntiles, kTileBlock, 0, Ld.dl, Ld.all.dev(), Ld.res.p,
                Ld.sol.p, Ld.rhs.p, Ld.a.p, Ld.bx.p, Ld.by.p, Ld.bz.p, want_norm ? I.partial.p : nullptr);
        } else {
            launch(k_residual<double, double, false>, Ld.all.ntiles, kTileBlock, 0, Ld.dl, Ld.all.dev(), Ld.res.p,
                Ld.sol.p, Ld.rhs.p, nullptr, nullptr, nullptr, nullptr, want_norm ? I.partial.p : nullptr);
        }
        launched();
        if (want_norm) {
            launch(k_reduce_final, 1, 1024, 0, I.partial.p, Ld.all.solve_begin.p, RED_MAXABS, I.red_out.p);
            launched();
        }
    }
}

// MLCellLinOpT::reflux (AMReX_MLCellLinOp.H:1272-1346) into res of level c
void AmrEngine::Impl::reflux (int c)
{
    LevelData& Lf = L(c + 1);
    LevelData& Lc = L(c);
    AmrLevelData& D = lev[c];
    // the reflux reads the fine solution's ghosts across the coarse/fine faces
    // only: the face closures, no copies between the fine patches
    lev[c + 1].I->ghost<double>(0, Lf.sol.p, true, false, Lf.bcval.p);
    if (D.nrcell > 0) {
        if (abec()) {
            launch(k_amr_reflux<true>, blocks_for(D.nrcell, 128), 128, 0, Lf.dl, D.rcells.p, D.rfaces.p, D.nrcell,
                D.rprm, reflux_coef(c), Lc.sol.p, Lf.sol.p, Lc.res.p, mixed() ? Lc.res32.p : nullptr);
        } else {
            launch(k_amr_reflux<false>, blocks_for(D.nrcell, 128), 128, 0, Lf.dl, D.rcells.p, D.rfaces.p, D.nrcell,
                D.rprm, RefluxCoef{}, Lc.sol.p, Lf.sol.p, Lc.res.p, mixed() ? Lc.res32.p : nullptr);
        }
        launched();
    }
}

void AmrEngine::Impl::avgdown (int c, const double* fine, double* crse, float* crse32)
{
    AmrLevelData& D = lev[c];
    if (D.nacell == 0) { return; }
    launch(k_amr_avgdown<double, double>, blocks_for(D.nacell, 256), 256, 0, L(c).dl, L(c + 1).dl, D.atags.p,
        D.astart.p, D.natag, D.nacell, fine, crse, crse32);
    launched();
}

// the mini-cycle of a fine AMR level (mgVcycle with one MG level,
// AMReX_MLMG.H:1306-1415): nu1 smoothing sweeps from zero on right-hand side rhs
template <typename T>
void AmrEngine::Impl::mini_cycle (int l, const T* rhs)
{
    T* x = cor<T>(l);
    LevelData& Ld = L(l);
    AmrLevelData& D = lev[l];
    const bool fused = std::is_same_v<T, float> && D.nsafe + D.nrest > 0 && A.m_opt.nu1 > 0;
    // the correction starts at zero: the fused sweeps' first one takes that
    // as given, the other paths clear the array
    if (!fused) { MLMG_CUDA_CHECK(cudaMemsetAsync(x, 0, sizeof(T) * (size_t)Ld.meta.nelem, st())); }
    if constexpr (std::is_same_v<T, float>) {
        if (fused) {
            // fused two-colour sweeps on the safe tiles, colour passes on the
            // rest: both read the old buffer and write the new one, the
            // second colour of the rest then reads the new buffer
            const dim3 blk(FS_TX, FS_TY);
            const size_t np = Ld.meta.patches.size();
            int* err = lev[0].I->err_d.p;
            float* a = x;
            float* b = D.fz_buf.p;
            auto maps_of = [&] (const float* f) {
                const size_t w = (f == Ld.cor32.p) ? 0 : ((f == D.hold32.p) ? 1 : 2);
                return D.fz_maps.p + w * np;
            };
            for (int i = 0; i < A.m_opt.nu1; ++i) {
                const float* in = (i == 0) ? nullptr : a;      // the first sweep reads a zero correction
                if (D.nsafe > 0) {
                    launch(k_sweep_fused2<false, true>, D.nsafe, blk, 0, Ld.dl, Ld.mg.dev(), a, b, rhs, StencilPtrs{},
                        maps_of(a), err, tma::WAIT_LIMIT, nullptr, i == 0 ? 1 : 0, D.fz_safe.p);
                    launched();
                }
                if (D.nrest > 0) {
                    const float* bb = b;
                    if (in == nullptr) {
                        launch(k_gsrb_tiles<false, false>, D.nrest, blk, 0, Ld.dl, D.fz_rest.p, in, in, b, rhs,
                               D.nbr.p, 0);
                        launch(k_gsrb_tiles<false, true>, D.nrest, blk, 0, Ld.dl, D.fz_rest.p, in, bb, b, rhs,
                               D.nbr.p, 1);
                    } else {
                        launch(k_gsrb_tiles<true, true>, D.nrest, blk, 0, Ld.dl, D.fz_rest.p, in, in, b, rhs,
                               D.nbr.p, 0);
                        launch(k_gsrb_tiles<true, true>, D.nrest, blk, 0, Ld.dl, D.fz_rest.p, in, bb, b, rhs,
                               D.nbr.p, 1);
                    }
                    launched(2);
                }
                std::swap(a, b);
            }
            if (a != x) {
                MLMG_CUDA_CHECK(cudaMemcpyAsync(x, a, sizeof(float) * (size_t)Ld.meta.nelem, cudaMemcpyDeviceToDevice,
                                                st()));
            }
            return;
        }
    }
    if (lev[l].nbr.p != nullptr) {
        // colour passes reading covered neighbours directly: no ghost fills
        for (int i = 0; i < A.m_opt.nu1; ++i) {
            for (int rb = 0; rb < 2; ++rb) {
                launch(k_gsrb_nbr<T>, Ld.mg.ntiles, kTileBlock, 0, Ld.dl, Ld.mg.dev(), x, rhs, lev[l].nbr.p, rb);
                launched();
            }
        }
        return;
    }
    for (int i = 0; i < A.m_opt.nu1; ++i) { lev[l].I->smooth<T>(0, x, rhs, i == 0); }
}

// out = b - L(cor): homogeneous, or (inhomog) with the coarse/fine values of
// the coarser level's correction, which gather() has just loaded
// (MLCellLinOpT::correctionResidual with updateCorBC, AMReX_MLCellLinOp.H:
// 666-680, 1246-1270).  L(cor) in the correction's precision.
template <typename T, typename TB, typename TO>
void AmrEngine::Impl::cor_residual (int l, bool inhomog, const TB* b, TO* out)
{
    LevelData& Ld = L(l);
    AmrLevelData& D = lev[l];
    T* x = cor<T>(l);
    if (inhomog) {
        const T* cf;
        if constexpr (std::is_same_v<T, float>) { cf = D.cf32.p; } else { cf = D.cf64.p; }
        if (D.nbitems > 0) {
            launch(k_amr_bndry_list<T>, blocks_for(D.nbitems, 256), 256, 0, (const int4*)D.bitems.p, D.nbitems,
                   (const PatchDesc*)D.cfd.p, cf, D.bcor.p);
            launched();
        }
        D.I->ghost<T>(0, x, true, true, D.bcor.p);
    } else {
        D.I->ghost<T>(0, x, false, true);
    }
    if (abec()) {
        const StencilPtrs sp = std::is_same_v<T, float> ? D.I->stencil32(0) : StencilPtrs{};
        launch(k_amr_resid<T, TB, TO, true>, Ld.all.ntiles, kTileBlock, 0, Ld.dl, Ld.all.dev(), out, x, b, Ld.a.p,
            Ld.bx.p, Ld.by.p, Ld.bz.p, sp);
    } else {
        launch(k_amr_resid<T, TB, TO, false>, Ld.all.ntiles, kTileBlock, 0, Ld.dl, Ld.all.dev(), out, x, b, nullptr,
            nullptr, nullptr, nullptr, StencilPtrs{});
    }
    launched();
}

// max|x| of level l (masked: cells under the finer level excluded) into h_norm[slot]
void AmrEngine::Impl::norm_start (int l, const double* x, bool masked, int slot)
{
    LevelData& Ld = L(l);
    Engine::Impl& I = *lev[l].I;
    launch(k_amr_norm<double>, Ld.all.ntiles, kTileBlock, 0, Ld.dl, Ld.all.dev(), x,
        masked ? lev[l].covered.p : nullptr, I.partial.p);
    launch(k_reduce_final, 1, 1024, 0, I.partial.p, Ld.all.solve_begin.p, RED_MAXABS, I.red_out.p);
    launched(2);
    MLMG_CUDA_CHECK(cudaMemcpyAsync(h_norm.p + slot, I.red_out.p, sizeof(double), cudaMemcpyDeviceToHost, st()));
}

// MLMGT::computeResidual(finest) with its (unmasked) norm from the residual
// kernel's block maxima, into h_norm[0]
void AmrEngine::Impl::fine_residual_and_norm ()
{
    const int fin = nl - 1;
    Engine::Impl& I = *lev[fin].I;
    solution_residual(fin, true, true);
    MLMG_CUDA_CHECK(cudaMemcpyAsync(h_norm.p, I.red_out.p, sizeof(double), cudaMemcpyDeviceToHost, st()));
}

// MLMGT::oneIter (AMReX_MLMG.H:1227-1293) followed by the convergence
// residual of the finest level (:436-441).  The residual a fine level ends
// its down-sweep with (fine_res after computeResWithCrseSolFineCor) lives in
// `dres` until the up-sweep takes it as b; the up-sweep's residual goes to a
// second buffer, whose only reader is that level's mini-cycle.
template <typename T>
void AmrEngine::Impl::one_iter (int iter)
{
    const int fin = nl - 1;
    Engine::Impl& I0 = *lev[0].I;
    I0.bslot = 0;
    std::vector<double*> dres(nl, nullptr);
    for (int l = fin; l > 0; --l) {
        LevelData& Ld = L(l);
        const unsigned g = (unsigned)Ld.all.ntiles;
        const T* rhs;
        if constexpr (std::is_same_v<T, float>) {
            // res32 was written with res (residual, reflux, average-down)
            rhs = Ld.res32.p;
            dres[l] = Ld.res.p;
        } else {
            rhs = Ld.res.p;
            dres[l] = Ld.rescor.p;
        }
        mini_cycle<T>(l, rhs);
        launch(k_add_to<double, T>, g, kTileBlock, 0, Ld.dl, Ld.all.dev(), Ld.sol.p, cor<T>(l), nullptr, nullptr, 0);
        launched();
        // computeResWithCrseSolFineCor(l-1, l), AMReX_MLMG.H:1660-1690
        solution_residual(l - 1, l - 1 > 0);
        cor_residual<T, T, double>(l, false, rhs, dres[l]);
        reflux(l - 1);
        avgdown(l - 1, dres[l], L(l - 1).res.p, std::is_same_v<T, float> ? L(l - 1).res32.p : nullptr);
        if (l != fin) { std::swap(lev[l].cor_p, lev[l].hold_p); }
    }
    {
        LevelData& L0 = L(0);
        if (iter < A.m_opt.max_fmg_iter) { I0.fcycle<T>(); } else { I0.vcycle<T>(0); }
        launch(k_add_to<double, T>, L0.all.ntiles, kTileBlock, 0, L0.dl, L0.all.dev(), L0.sol.p, cor<T>(0), nullptr,
               nullptr, 0);
        launched();
    }
    for (int l = 1; l <= fin; ++l) {
        LevelData& Ld = L(l);
        AmrLevelData& D = lev[l];
        const unsigned g = (unsigned)Ld.all.ntiles;
        T* hold_l = (l != fin) ? hold<T>(l) : nullptr;
        // interpCorrection(l) (AMReX_MLMG.H:1719-1750), sol += cor, hold += cor
        gather<T>(l, cor<T>(l - 1));
        const T* cf;
        if constexpr (std::is_same_v<T, float>) { cf = D.cf32.p; } else { cf = D.cf64.p; }
        launch(k_amr_interp_add<T>, g, kTileBlock, 0, Ld.dl, Ld.all.dev(), D.cfd.p, cf, cor<T>(l), Ld.sol.p, hold_l);
        launched();
        // computeResWithCrseCorFineCor(l), AMReX_MLMG.H:1693-1715
        T* ures;
        if constexpr (std::is_same_v<T, float>) { ures = Ld.rescor32.p; } else { ures = Ld.res.p; }
        cor_residual<T, double, T>(l, true, dres[l], ures);
        mini_cycle<T>(l, ures);
        launch(k_amr_finish<T>, g, kTileBlock, 0, Ld.dl, Ld.all.dev(), Ld.sol.p, cor<T>(l), hold_l);
        launched();
    }
    // averageDownAndSync, AMReX_MLCellLinOp.H:2102-2122
    for (int l = fin; l > 0; --l) { avgdown(l - 1, L(l).sol.p, L(l - 1).sol.p); }
    fine_residual_and_norm();
    I0.fetch_bottom_counts();
}

// ----------------------------------------------------------------- AmrEngine --
AmrEngine::AmrEngine (const AmrProblem& prob, const EngineOptions& opt, cudaStream_t stream)
    : m_opt(opt), m_stream(stream)
{
    m_opt.time_kernels = 0;
    m_impl = std::make_unique<Impl>(*this);
    m_impl->prob = prob;
    m_impl->build();
}

AmrEngine::~AmrEngine () = default;

int AmrEngine::kernel_launches () const
{
    int n = m_impl->own_launches;
    for (const auto& D : m_impl->lev) { n += D.eng->kernel_launches(); }
    return n;
}

void AmrEngine::reset_launch_count ()
{
    m_impl->own_launches = 0;
    for (auto& D : m_impl->lev) { D.eng->reset_launch_count(); }
}

int AmrEngine::namr () const { return m_impl->nl; }
int AmrEngine::num_mg_levels () const { return m_impl->lev[0].eng->nlevels(0); }

void AmrEngine::solve (const std::vector<const FabSet*>& sol_in, const std::vector<FabSet*>& sol_out,
                       const std::vector<const FabSet*>& rhs, double tol_rel, double tol_abs)
{
    Impl& M = *m_impl;
    const int nl = M.nl, fin = nl - 1;
    MLMG_REQUIRE((int)sol_in.size() == nl && (int)sol_out.size() == nl && (int)rhs.size() == nl, ERR_ARGS,
                 "one sol and one rhs per AMR level");
    MLMG_REQUIRE(!M.lev[0].I->singular[0], ERR_UNSUPPORTED, "singular AMR composite solves are not supported");
    m_report = SolveReport{};
    // the valid cells of sol and rhs; their other elements (zero since the
    // fields were allocated) are written before they are read: the ghost
    // shells by the fills ahead of every stencil, the padding never
    for (int l = 0; l < nl; ++l) {
        LevelData& Ld = M.L(l);
        Engine::Impl& I = *M.lev[l].I;
        I.xfer(I.items_for(*sol_in[l], 0, 0, -1), *sol_in[l], Ld.sol.p, false, 0);
        I.xfer(I.items_for(*rhs[l], 0, 0, -1), *rhs[l], Ld.rhs.p, false, 0);
    }
    MLMG_CUDA_CHECK(cudaEventRecord(M.ev0, m_stream));
    // prepareForSolve: averageDownSolutionRHS (AMReX_MLMG.H:1025-1028)
    for (int l = fin; l > 0; --l) {
        M.avgdown(l - 1, M.L(l).sol.p, M.L(l - 1).sol.p);
        M.avgdown(l - 1, M.L(l).rhs.p, M.L(l - 1).rhs.p);
    }
    // computeMLResidual(finest) and the masked norms (AMReX_MLMG.H:391-396, 1632-1648)
    auto ml_residual = [&] (int lmax) {
        for (int l = lmax; l >= 0; --l) {
            M.solution_residual(l, l > 0);
            if (l < fin) { M.reflux(l); }
        }
    };
    ml_residual(fin);
    for (int l = 0; l < nl; ++l) {
        M.norm_start(l, M.L(l).res.p, l < fin, 1 + l);
        M.norm_start(l, M.L(l).rhs.p, l < fin, 1 + nl + l);
    }
    MLMG_CUDA_CHECK(cudaStreamSynchronize(m_stream));
    double resnorm0 = 0, rhsnorm0 = 0;
    for (int l = 0; l < nl; ++l) {
        resnorm0 = std::max(resnorm0, M.h_norm.p[1 + l]);
        rhsnorm0 = std::max(rhsnorm0, M.h_norm.p[1 + nl + l]);
    }
    SolveReport& R = m_report;
    R.init_resid = resnorm0;
    R.rhs_norm = rhsnorm0;
    const double max_norm = (m_opt.always_use_bnorm || rhsnorm0 >= resnorm0) ? rhsnorm0 : resnorm0;
    const double target = std::max(tol_abs, std::max(tol_rel, 1.e-16) * max_norm);
    R.final_resid = resnorm0;
    if (m_opt.verbose >= 1) {
        std::printf("MLMG: Initial rhs               = %.10g\nMLMG: Initial residual (resid0) = %.10g\n",
                    rhsnorm0, resnorm0);
    }
    // the first swap of every intermediate level's correction buffers
    // happens inside the iteration; their contents never carry over
    M.lev[0].I->bottom_mode_init();
    const int niters = m_opt.fixed_iter ? m_opt.fixed_iter : m_opt.max_iter;
    bool converged = false;
    int graph_bslots = 1;
    Engine::Impl& I0 = *M.lev[0].I;
    if (resnorm0 > target) {
        for (int iter = 0; iter < niters; ++iter) {
            const bool fmg = iter < m_opt.max_fmg_iter;
            if (!fmg && m_opt.use_graph) {
                if (M.graph_exec == nullptr) {
                    const int before = kernel_launches();
                    cudaGraph_t g;
                    MLMG_CUDA_CHECK(cudaStreamBeginCapture(m_stream, cudaStreamCaptureModeThreadLocal));
                    I0.capturing = true;
                    if (M.mixed()) { M.one_iter<float>(iter); } else { M.one_iter<double>(iter); }
                    I0.capturing = false;
                    graph_bslots = I0.bslot;
                    MLMG_CUDA_CHECK(cudaStreamEndCapture(m_stream, &g));
                    MLMG_CUDA_CHECK(cudaGraphInstantiate(&M.graph_exec, g, 0));
                    MLMG_CUDA_CHECK(cudaGraphDestroy(g));
                    M.graph_launches = kernel_launches() - before;
                    M.own_launches -= M.graph_launches;
                }
                MLMG_CUDA_CHECK(cudaGraphLaunch(M.graph_exec, m_stream));
                M.own_launches += M.graph_launches;
                I0.bslot = graph_bslots;
            } else {
                if (M.mixed()) { M.one_iter<float>(iter); } else { M.one_iter<double>(iter); }
            }
            MLMG_CUDA_CHECK(cudaGetLastError());
            MLMG_CUDA_CHECK(cudaStreamSynchronize(m_stream));
            const double fine = M.h_norm.p[0];
            R.history.push_back(fine);
            for (int q = 0; q < I0.bslot && q < I0.nlev_max + 2; ++q) {
                R.cg_iters.push_back(I0.h_iters.p[q]);
                if (I0.h_iters2.p[q] >= 0) { R.cg_iters.push_back(I0.h_iters2.p[q]); }
            }
            R.niters++;
            R.final_resid = fine;
            if (m_opt.verbose >= 2) {
                std::printf("MLMG: Iteration %3d Fine resid/%s = %.10g\n", iter + 1,
                            (max_norm == rhsnorm0) ? "bnorm" : "resid0", fine / max_norm);
            }
            if (!std::isfinite(fine)) { R.status = ERR_NONFINITE; break; }
            if (fine <= target) {
                // the finest level has converged: test the coarser levels (AMReX_MLMG.H:450-467)
                ml_residual(fin - 1);
                for (int l = 0; l < fin; ++l) { M.norm_start(l, M.L(l).res.p, true, 1 + l); }
                MLMG_CUDA_CHECK(cudaStreamSynchronize(m_stream));
                double crse = 0;
                for (int l = 0; l < fin; ++l) { crse = std::max(crse, M.h_norm.p[1 + l]); }
                R.final_resid = std::max(fine, crse);
                if (crse <= target) { converged = true; break; }
            }
            if (R.final_resid > 1.e20 * max_norm) { R.status = ERR_DIVERGED; break; }
        }
        if (!converged && R.status == OK && m_opt.fixed_iter == 0) { R.status = NOT_CONVERGED; }
    }
    MLMG_CUDA_CHECK(cudaEventRecord(M.ev1, m_stream));
    M.lev[0].I->check_device_error();
    if (m_opt.verbose >= 1) {
        std::printf("MLMG: Final Iter. %d resid, resid/bnorm = %.10g, %.10g\n", R.niters, R.final_resid,
                    R.final_resid / max_norm);
    }
    for (int l = 0; l < nl; ++l) {
        FabSet& out = *sol_out[l];
        Engine::Impl& I = *M.lev[l].I;
        I.xfer(I.items_for(out, 0, out.ngrow >= 1 ? 1 : 0, -1), out, M.L(l).sol.p, false, 1);
    }
    MLMG_CUDA_CHECK(cudaEventSynchronize(M.ev1));
    float ms = 0;
    MLMG_CUDA_CHECK(cudaEventElapsedTime(&ms, M.ev0, M.ev1));
    m_last_ms = ms;
}

void AmrEngine::comp_residual (const std::vector<const FabSet*>& sol, const std::vector<const FabSet*>& rhs,
                               const std::vector<FabSet*>& res)
{
    Impl& M = *m_impl;
    const int nl = M.nl, fin = nl - 1;
    MLMG_REQUIRE((int)sol.size() == nl && (int)rhs.size() == nl && (int)res.size() == nl, ERR_ARGS,
                 "one res, one sol and one rhs per AMR level");
    for (int l = 0; l < nl; ++l) {
        LevelData& Ld = M.L(l);
        Engine::Impl& I = *M.lev[l].I;
        MLMG_CUDA_CHECK(cudaMemsetAsync(Ld.sol.p, 0, Ld.sol.n * sizeof(double), m_stream));
        MLMG_CUDA_CHECK(cudaMemsetAsync(Ld.rhs.p, 0, Ld.rhs.n * sizeof(double), m_stream));
        I.xfer(I.items_for(*sol[l], 0, 0, -1), *sol[l], Ld.sol.p, false, 0);
        I.xfer(I.items_for(*rhs[l], 0, 0, -1), *rhs[l], Ld.rhs.p, false, 0);
    }
    // AMReX_MLMG.H:821-845: from the finest level down, the solution residual
    // (fine levels with the coarse/fine values of the next coarser solution),
    // the reflux of the finer level's fluxes and the average-down of its
    // residual onto the covered cells
    for (int l = fin; l >= 0; --l) {
        M.solution_residual(l, l > 0, false, true);
        if (l < fin) {
            M.reflux(l);
            M.avgdown(l, M.L(l + 1).res.p, M.L(l).res.p);
        }
    }
    for (int l = 0; l < nl; ++l) {
        Engine::Impl& I = *M.lev[l].I;
        I.xfer(I.items_for(*res[l], 0, 0, -1), *res[l], M.L(l).res.p, false, 1);
    }
    MLMG_CUDA_CHECK(cudaStreamSynchronize(m_stream));
}

// MLLinOpT::setCoarseFineBC (AMReX_MLLinOp.H:1427-1441) as
// MLCellLinOpT::setLevelBC applies it at AMR level 0 (AMReX_MLCellLinOp.H:
// 537-566): a level whose boxes do not cover its domain takes, on its
// coarse/fine faces, Dirichlet values interpolated from the coarse data
// (InterpBndryDataT::setBndryValues, o3, AMReX_InterpBndryData.H:158-244),
// after the coarse FABs' valid cells (and their periodic images) are copied
// into each fine patch's coarsened box grown by one cell
// (BndryRegisterT::copyFrom; cells no FAB reaches hold 0).  Refinement ratio 2.
void coarse_fine_bc_values (Engine::Impl& I, int s, const SolveSpec& S, const FabSet& crse)
{
    MLMG_REQUIRE(S.crse_ratio == 2, ERR_UNSUPPORTED, "coarse/fine boundary values need refinement ratio 2");
    MLMG_REQUIRE(crse.nodal_dir < 0, ERR_ARGS, "the coarse data must be cell-centred");
    cudaStream_t st = I.st();
    LevelData& L0 = I.lev[0];
    const PatchLevel& Mf = L0.meta;
    const int p0 = Mf.solve_first_patch[s], np = Mf.solve_npatch[s];
    const int npatch = (int)Mf.patches.size();
    // coarse buffers (indexed by level patch; patches of other solves get none)
    std::vector<PatchDesc> cfd(npatch);
    long long cursor = 0;
    for (int p = p0; p < p0 + np; ++p) {
        const PatchDesc& P = Mf.patches[p];
        Box3 pb;
        for (int d = 0; d < 3; ++d) { pb.lo[d] = P.lo[d]; pb.hi[d] = P.hi[d]; }
        const Box3 cb = coarsen(pb, 2);
        PatchDesc& G = cfd[p];
        for (int d = 0; d < 3; ++d) { G.lo[d] = cb.lo[d]; G.hi[d] = cb.hi[d]; }
        G.sx = cb.len(0) + 2;
        G.sxy = (long long)G.sx * (cb.len(1) + 2);
        G.base = cursor + G.sxy + G.sx + 1;
        cursor += G.sxy * (cb.len(2) + 2);
    }
    // the coarse FABs as patch descriptors (valid box; index of its lower
    // corner inside the grown FAB)
    const int nfab = (int)crse.boxes.size();
    std::vector<PatchDesc> cdesc(std::max(nfab, 1));
    for (int b = 0; b < nfab; ++b) {
        const Box3& vb = crse.boxes[b];
        const Box3 fb = grow(vb, crse.ngrow);
        PatchDesc& G = cdesc[b];
        for (int d = 0; d < 3; ++d) { G.lo[d] = vb.lo[d]; G.hi[d] = vb.hi[d]; }
        G.sx = fb.len(0);
        G.sxy = (long long)fb.len(0) * fb.len(1);
        G.base = crse.off[b] + (long long)crse.ngrow * (G.sxy + G.sx + 1);
    }
    // gather tags
    const Box3 cdom = coarsen(S.geom.domain, 2);
    const auto cshifts = image_shifts(cdom, S.geom.periodic);
    std::vector<CopyTag> tags;
    std::vector<long long> start{0};
    for (int p = p0; p < p0 + np; ++p) {
        Box3 g;
        for (int d = 0; d < 3; ++d) { g.lo[d] = cfd[p].lo[d] - 1; g.hi[d] = cfd[p].hi[d] + 1; }
        for (int b = 0; b < nfab; ++b) {
            for (const auto& sh : cshifts) {
                const Box3 is = intersect(g, shift(crse.boxes[b], sh.data()));
                if (!is.ok()) { continue; }
                CopyTag t{};
                t.dst = p; t.src = b; t.box = is;
                for (int d = 0; d < 3; ++d) { t.shift[d] = sh[d]; }
                tags.push_back(t);
                start.push_back(start.back() + is.npts());
            }
        }
    }
    // coarse/fine faces and the neighbourhood flags of their ghost cells
    const Box3 fdom = S.geom.domain;
    const BoxLocator floc(S.levels[0].boxes);
    auto notcov = [&] (int i, int j, int k) {
        int c[3] = {i, j, k};
        return wrap_cell(fdom, S.geom.periodic, c) && floc.find(c[0], c[1], c[2]) < 0;
    };
    std::vector<int8_t> flags(L0.bcval.n, 0);
    std::vector<int2> faces;
    std::vector<long long> fstart{0};
    for (int p = p0; p < p0 + np; ++p) {
        const PatchDesc& P = Mf.patches[p];
        for (int f = 0; f < 6; ++f) {
            const FaceBC& F = P.face[f];
            const int d = f % 3;
            if (F.on_domain && !S.geom.periodic[d]) { continue; }   // physical face: the level BC values
            const int t1 = (d == 0) ? 1 : 0, t2 = (d == 2) ? 1 : 2;
            const int g = (f >= 3) ? P.hi[d] + 1 : P.lo[d] - 1;
            const int n1 = P.hi[t1] - P.lo[t1] + 1, n2 = P.hi[t2] - P.lo[t2] + 1;
            faces.push_back(make_int2(p, f));
            fstart.push_back(fstart.back() + (long long)n1 * n2);
            for (int v2 = 0; v2 < n2; ++v2)
            for (int v1 = 0; v1 < n1; ++v1) {
                int c[3];
                c[d] = g; c[t1] = P.lo[t1] + v1; c[t2] = P.lo[t2] + v2;
                int fl = 0;
                if (notcov(c[0], c[1], c[2])) {
                    fl |= BF_SELF;
                    auto nc_at = [&] (int a1, int a2) {
                        int e[3] = {c[0], c[1], c[2]};
                        e[t1] += a1; e[t2] += a2;
                        return notcov(e[0], e[1], e[2]);
                    };
                    if (nc_at(-2, 0)) { fl |= BF_T1LO; }
                    if (nc_at(2, 0)) { fl |= BF_T1HI; }
                    if (nc_at(0, -2)) { fl |= BF_T2LO; }
                    if (nc_at(0, 2)) { fl |= BF_T2HI; }
                    if (nc_at(-2, -2) && nc_at(2, -2) && nc_at(-2, 2) && nc_at(2, 2)) { fl |= BF_CROSS; }
                }
                flags[(size_t)(F.bcval_off + (long long)v2 * n1 + v1)] = (int8_t)fl;
            }
        }
    }
    if (faces.empty()) { return; }
    DevBuf<PatchDesc> d_cfd, d_cdesc;
    DevBuf<CopyTag> d_tags;
    DevBuf<long long> d_start, d_fstart;
    DevBuf<int2> d_faces;
    DevBuf<int8_t> d_flags;
    d_cfd.upload(cfd, st);
    d_cdesc.upload(cdesc, st);
    d_start.upload(start, st);
    d_faces.upload(faces, st);
    d_fstart.upload(fstart, st);
    d_flags.upload(flags, st);
    if (!tags.empty()) { d_tags.upload(tags, st); }
    const DevLevel Lc{d_cdesc.p, nullptr, nullptr, nullptr, nfab};
    const GhostWork W{d_faces.p, d_fstart.p, (int)faces.size(), nullptr, nullptr, 0, fstart.back(), 0};
    auto run = [&] (auto tag) {
        using T = decltype(tag);
        DevBuf<T> cf;
        cf.alloc((size_t)std::max<long long>(cursor, 1));
        cf.zero(st);
        if (!tags.empty()) {
            k_amr_gather<T><<<blocks_for(start.back(), 256), 256, 0, st>>>(Lc, d_cfd.p, d_tags.p, d_start.p,
                (int)tags.size(), start.back(), static_cast<const T*>(crse.data), cf.p);
            I.launched();
        }
        k_amr_bndry<T><<<blocks_for(W.nfacecells, 256), 256, 0, st>>>(L0.dl, W, d_cfd.p, cf.p, d_flags.p,
                                                                      L0.bcval.p);
        I.launched();
        MLMG_CUDA_CHECK(cudaGetLastError());
        MLMG_CUDA_CHECK(cudaStreamSynchronize(st));
    };
    if (crse.prec == 8) { run(double{}); } else { run(float{}); }
}

} // namespace mlmg
