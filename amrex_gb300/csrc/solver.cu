// The batched MLMG engine: host orchestration of the V-cycle stages.
#include "engine_impl.cuh"

#include <cudaTypedefs.h>

#include <cmath>
#include <cstring>
#include <type_traits>

namespace mlmg {


// ------------------------------------------------------------ tensor maps --
namespace {

PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder ()
{
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    if (fn == nullptr) {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q{};
        MLMG_CUDA_CHECK(cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q));
        MLMG_REQUIRE(q == cudaDriverEntryPointSuccess && p != nullptr, ERR_CUDA, "cuTensorMapEncodeTiled is unavailable");
        fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    }
    return fn;
}


} // namespace

// 3-D tiled tensor map over the allocation of patch P inside an FP32 level
// field: x over the whole padded row (sx), y and z over the rows and planes
// with their ghost layers; box bx x by x bz floats (default: a fused sweep's
// 40 x 12 x 12 staging box)
CUtensorMap patch_tensor_map (const float* field, const PatchDesc& P, int by, int bz, int bx)
{
    const long long start = P.base - P.sxy - P.sx - XOFF;      // first element of the patch's allocation
    const int ny = P.hi[1] - P.lo[1] + 1, nz = P.hi[2] - P.lo[2] + 1;
    MLMG_REQUIRE(start % 4 == 0 && P.sx % 4 == 0 && P.sxy % 4 == 0, ERR_INTERNAL, "patch layout not 16-byte aligned");
    cuuint64_t dims[3] = {(cuuint64_t)P.sx, (cuuint64_t)(ny + 2), (cuuint64_t)(nz + 2)};
    cuuint64_t strides[2] = {(cuuint64_t)P.sx * sizeof(float), (cuuint64_t)P.sxy * sizeof(float)};
    cuuint32_t box[3] = {(cuuint32_t)bx, (cuuint32_t)by, (cuuint32_t)bz};
    cuuint32_t estride[3] = {1, 1, 1};
    CUtensorMap m;
    const CUresult r = tensor_map_encoder()(&m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3,
        const_cast<float*>(field + start), dims, strides, box, estride, CU_TENSOR_MAP_INTERLEAVE_NONE,
        CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    MLMG_REQUIRE(r == CUDA_SUCCESS, ERR_CUDA, "cuTensorMapEncodeTiled failed (" + std::to_string((int)r) + ")");
    return m;
}

// -------------------------------------------------------------- fields ----
template <> double* Engine::Impl::field_cor<double> (int l) { return lev[l].cor.p; }
template <> double* Engine::Impl::field_res<double> (int l) { return lev[l].res.p; }
template <> double* Engine::Impl::field_rescor<double> (int l) { return lev[l].rescor.p; }
template <> float* Engine::Impl::field_cor<float> (int l) { return lev[l].cor32.p; }
template <> float* Engine::Impl::field_res<float> (int l) { return lev[l].res32.p; }
template <> float* Engine::Impl::field_rescor<float> (int l) { return lev[l].rescor32.p; }
template <> const double* Engine::Impl::coef<double> (int l, int w)
{
    const LevelData& L = lev[l];
    return w == 0 ? L.a.p : (w == 1 ? L.bx.p : (w == 2 ? L.by.p : L.bz.p));
}

// --------------------------------------------------------------- build ----
void Engine::Impl::build ()
{
    nsolve = (int)E.m_problems.size();
    MLMG_REQUIRE(nsolve > 0, ERR_ARGS, "empty batch");
    abec = E.m_problems[0].spec.is_abec != 0;
    std::vector<const SolveSpec*> specs;
    for (auto& pr : E.m_problems) {
        MLMG_REQUIRE((pr.spec.is_abec != 0) == abec, ERR_UNSUPPORTED, "a batch must hold one operator type");
        specs.push_back(&pr.spec);
        nlev_max = std::max(nlev_max, (int)pr.spec.levels.size());
    }
    lev.resize(nlev_max);
    size_t max_tiles = 1;
    for (int l = 0; l < nlev_max; ++l) {
        LevelData& L = lev[l];
        L.meta = build_patch_level(specs, l, E.m_opt.merge_boxes != 0);
        PatchLevel& M = L.meta;
        // level-0 Dirichlet values: one slot per face cell of every level-0 patch face
        if (l == 0) {
            long long off = 0;
            for (auto& P : M.patches) {
                for (int f = 0; f < 6; ++f) {
                    const int d = f % 3;
                    const int e0 = (d == 0) ? 1 : 0, e1 = (d == 2) ? 1 : 2;
                    P.face[f].bcval_off = off;
                    off += (long long)(P.hi[e0] - P.lo[e0] + 1) * (P.hi[e1] - P.lo[e1] + 1);
                }
            }
            L.bcval.alloc((size_t)std::max<long long>(off, 1));
            L.bcval.zero(st());
        }
        L.P.upload(M.patches, st());
        if (!M.masks.empty()) { L.masks.upload(M.masks, st()); }
        std::vector<int> sfirst(nsolve), snp(nsolve);
        for (int s = 0; s < nsolve; ++s) { sfirst[s] = M.solve_first_patch[s]; snp[s] = M.solve_npatch[s]; }
        L.sfirst.upload(sfirst, st());
        L.snp.upload(snp, st());
        // tags grouped per solve (they are generated solve by solve)
        L.solve_tag_first.assign(nsolve, 0);
        L.solve_tag_n.assign(nsolve, 0);
        for (size_t t = 0; t < M.tags.size(); ++t) {
            const int s = M.patches[M.tags[t].dst].solve;
            if (L.solve_tag_n[s] == 0) { L.solve_tag_first[s] = (int)t; }
            L.solve_tag_n[s]++;
        }
        // ghost work
        std::vector<int2> faces;
        std::vector<long long> fstart{0}, tstart{0};
        for (int p = 0; p < (int)M.patches.size(); ++p) {
            const PatchDesc& P = M.patches[p];
            for (int f = 0; f < 6; ++f) {
                const int d = f % 3;
                const int e0 = (d == 0) ? 1 : 0, e1 = (d == 2) ? 1 : 2;
                faces.push_back(make_int2(p, f));
                fstart.push_back(fstart.back() + (long long)(P.hi[e0] - P.lo[e0] + 1) * (P.hi[e1] - P.lo[e1] + 1));
            }
        }
        for (const auto& t : M.tags) { tstart.push_back(tstart.back() + t.box.npts()); }
        L.faces.upload(faces, st());
        L.fstart.upload(fstart, st());
        if (!M.tags.empty()) { L.tags.upload(M.tags, st()); }
        L.tstart.upload(tstart, st());
        L.gw = GhostWork{L.faces.p, L.fstart.p, (int)faces.size(), L.tags.p, L.tstart.p, (int)M.tags.size(),
                         fstart.back(), tstart.back()};
        L.dl = DevLevel{L.P.p, L.masks.p, L.sfirst.p, L.snp.p, (int)M.patches.size()};
        std::vector<int> all(M.patches.size()), mg;
        std::iota(all.begin(), all.end(), 0);
        for (int p = 0; p < (int)M.patches.size(); ++p) {
            if (!M.patch_is_bottom[p]) { mg.push_back(p); } else { L.has_bottom = true; }
        }
        build_subset(L.all, M, all, nsolve, st());
        build_subset(L.mg, M, mg, nsolve, st());
        max_tiles = std::max(max_tiles, (size_t)L.all.ntiles);
        // inline ghost values: no intra-level copies, and every face closed by
        // a BC of at most two interior cells
        L.inline_bc = M.tags.empty();
        for (const auto& P : M.patches) {
            for (int f = 0; f < 6; ++f) {
                const FaceBC& F = P.face[f];
                const bool closure = (F.type == BC_DIRICHLET && F.nx <= 3) || F.type == BC_NEUMANN ||
                                     F.type == BC_REFLECT_ODD;
                if (F.mask_uniform < 1 || !closure) { L.inline_bc = false; }
            }
        }
        L.fused = E.m_opt.fused_smoother && mixed() && L.inline_bc && !mg.empty();
        if (L.fused) {
            // same patches as the mg subset, tiled for the fused sweep
            SubsetData& S = L.fz;
            S.h_plist = mg;
            S.n = (int)mg.size();
            S.h_tstart.assign(S.n + 1, 0);
            for (int q = 0; q < S.n; ++q) { S.h_tstart[q + 1] = S.h_tstart[q] + fused_tiles_of(M.patches[mg[q]]); }
            S.ntiles = S.h_tstart[S.n];
            S.plist.upload(S.h_plist, st());
            S.tstart.upload(S.h_tstart, st());
            // the z-marching sweep where the level has enough columns to fill the GPU
            SubsetData& Z = L.mz;
            Z.h_plist = mg;
            Z.n = (int)mg.size();
            Z.h_tstart.assign(Z.n + 1, 0);
            for (int q = 0; q < Z.n; ++q) { Z.h_tstart[q + 1] = Z.h_tstart[q] + march_tiles_of(M.patches[mg[q]], E.m_opt.march_tz); }
            Z.ntiles = Z.h_tstart[Z.n];
            L.march = E.m_opt.march_sweep && Z.ntiles >= E.m_opt.march_min_tiles;
            if (L.march) {
                Z.plist.upload(Z.h_plist, st());
                Z.tstart.upload(Z.h_tstart, st());
                static bool attr_set = false;
                if (!attr_set) {
                    MLMG_CUDA_CHECK(cudaFuncSetAttribute(k_sweep_march_tma<true>,
                        cudaFuncAttributeMaxDynamicSharedMemorySize, march_tma_smem_floats(true) * (int)sizeof(float)));
                    MLMG_CUDA_CHECK(cudaFuncSetAttribute(k_sweep_march_tma<false>,
                        cudaFuncAttributeMaxDynamicSharedMemorySize, march_tma_smem_floats(false) * (int)sizeof(float)));
                    attr_set = true;
                }
            }
        }
        // fields
        const size_t n = (size_t)M.nelem;
        auto alloc0 = [&] (DevBuf<double>& b) { b.alloc(n); b.zero(st()); };
        auto alloc0f = [&] (DevBuf<float>& b) { b.alloc(n); b.zero(st()); };
        if (abec) { alloc0(L.a); alloc0(L.bx); alloc0(L.by); alloc0(L.bz); }
        if (l == 0) { alloc0(L.sol); alloc0(L.rhs); alloc0(L.res); }
        if (mixed()) {
            alloc0f(L.cor32); alloc0f(L.res32); alloc0f(L.rescor32);
            if (L.fused) { alloc0f(L.cor32b); }
            if (abec) {
                alloc0(L.D); alloc0(L.sx); alloc0(L.sy); alloc0(L.sz);
                alloc0f(L.D32); alloc0f(L.sx32); alloc0f(L.sy32); alloc0f(L.sz32);
            }
        } else {
            alloc0(L.cor); if (l > 0) { alloc0(L.res); } alloc0(L.rescor);
        }
        if (L.has_bottom) { for (auto& b : L.bw) { alloc0(b); } }
        // tensor maps of the fused sweep's TMA staging, one per patch of the level
        if (L.fused && !L.march && E.m_opt.fused_tma) {
            std::vector<CUtensorMap> ta(M.patches.size()), tb(M.patches.size());
            for (size_t p = 0; p < M.patches.size(); ++p) {
                ta[p] = patch_tensor_map(L.cor32.p, M.patches[p]);
                tb[p] = patch_tensor_map(L.cor32b.p, M.patches[p]);
            }
            L.tm_a.upload(ta, st());
            L.tm_b.upload(tb, st());
            // L2-prefetch maps: the tile grown by one (40 x 10 x 10; the y / z
            // face arrays one row / plane more)
            std::vector<CUtensorMap> tp((size_t)FS_PF_NMAP * M.patches.size());
            std::memset(tp.data(), 0, tp.size() * sizeof(CUtensorMap));
            for (size_t p = 0; p < M.patches.size(); ++p) {
                CUtensorMap* m = &tp[p * FS_PF_NMAP];
                const PatchDesc& P = M.patches[p];
                m[FS_PF_RHS] = patch_tensor_map(L.res32.p, P, 10, 10);
                if (abec) {
                    m[FS_PF_D] = patch_tensor_map(L.D32.p, P, 10, 10);
                    m[FS_PF_SX] = patch_tensor_map(L.sx32.p, P, 10, 10);
                    m[FS_PF_SY] = patch_tensor_map(L.sy32.p, P, 11, 10);
                    m[FS_PF_SZ] = patch_tensor_map(L.sz32.p, P, 10, 11);
                }
            }
            L.tm_pf.upload(tp, st());
        }
        // the TMA z-march's maps: one plane (72 x 20 of phi, 72 x 19 of rhs and
        // the stencil arrays) per load, per patch
        if (L.march) {
            std::vector<CUtensorMap> tm((size_t)MT_NMAP * M.patches.size());
            std::memset(tm.data(), 0, tm.size() * sizeof(CUtensorMap));
            for (size_t p = 0; p < M.patches.size(); ++p) {
                CUtensorMap* m = &tm[p * MT_NMAP];
                const PatchDesc& P = M.patches[p];
                m[MT_PHI_A] = patch_tensor_map(L.cor32.p, P, MS_XR, 1, MS_RP);
                m[MT_PHI_B] = patch_tensor_map(L.cor32b.p, P, MS_XR, 1, MS_RP);
                m[MT_RHS] = patch_tensor_map(L.res32.p, P, MS_CR, 1, MS_RP);
                if (abec) {
                    m[MT_D] = patch_tensor_map(L.D32.p, P, MS_CR, 1, MS_RP);
                    m[MT_SX] = patch_tensor_map(L.sx32.p, P, MS_CR, 1, MS_RP);
                    m[MT_SY] = patch_tensor_map(L.sy32.p, P, MS_CR, 1, MS_RP);
                    m[MT_SZ] = patch_tensor_map(L.sz32.p, P, MS_CR, 1, MS_RP);
                }
            }
            L.tm_m.upload(tm, st());
        }
    }
    err_d.alloc(1);
    err_d.zero(st());
    partial.alloc(max_tiles + 1);
    red_out.alloc((size_t)nsolve * 4 + 4);
    h_red.alloc((size_t)nsolve * 4 + 4);
    h_iters.alloc((size_t)nsolve * (nlev_max + 2) + 2);
    // one slot of nsolve counts per bottom solve of an iteration
    bot_iters.alloc((size_t)nsolve * (nlev_max + 2));
    bot_ret.alloc((size_t)nsolve * (nlev_max + 2));
    bot_iters2.alloc((size_t)nsolve * (nlev_max + 2));
    bot_mode.alloc(nsolve);
    h_iters2.alloc((size_t)nsolve * (nlev_max + 2) + 2);
    active_d.alloc(nsolve);

    // singular operators (update_singular_flags, AMReX_MLABecLaplacian.H:714-773;
    // MLPoissonT::prepareForSolve, AMReX_MLPoisson.H:138-178) and the
    // solvability volumes (AMReX_MLCellLinOp.H:1941-1995)
    singular.assign(nsolve, 0);
    volinv0.assign(nsolve, 0.0);
    volinv_bottom.assign(nsolve, 0.0);
    for (int s = 0; s < nsolve; ++s) {
        const SolveSpec& S = E.m_problems[s].spec;
        bool dir = false;
        for (int d = 0; d < 3; ++d) { if (S.lobc[d] == BC_DIRICHLET || S.hibc[d] == BC_DIRICHLET) { dir = true; } }
        long long np = 0;
        for (const auto& b : S.levels[0].boxes) { np += b.npts(); }
        const bool covered = (np == S.levels[0].geom.domain.npts());
        singular[s] = (!dir && covered && (!abec || S.alpha == 0.0)) ? 1 : 0;
        // zero for a regular solve, so that the mean removal launched for the
        // singular solves of a batch leaves the other solves unchanged
        volinv0[s] = singular[s] ? 1.0 / (double)S.levels[0].geom.domain.npts() : 0.0;
        volinv_bottom[s] = 1.0 / (double)S.levels.back().geom.domain.npts();
    }
    volinv0_d.upload(volinv0, st());
    build_bottom_tables();
    // F-cycle interpolation tables: level l as the fine level of level l+1
    for (int l = 0; l < nlev_max; ++l) {
        LevelData& L = lev[l];
        if (!L.meta.rboxes.empty()) { L.rbox.upload(L.meta.rboxes, st()); }
        if (l + 1 >= nlev_max) { continue; }
        std::vector<FmgSolveInfo> info(nsolve);
        for (int s = 0; s < nsolve; ++s) {
            const SolveSpec& S = E.m_problems[s].spec;
            FmgSolveInfo I{};
            if (l + 1 < (int)S.levels.size()) {
                I.cdom = S.levels[l + 1].geom.domain;
                for (int d = 0; d < 3; ++d) { I.per[d] = S.geom.periodic[d]; }
                I.safe = (S.levels[l].derived && S.levels[l + 1].derived) ? 1 : 0;
                I.rbox0 = L.meta.solve_rbox_first[s];
                I.nrbox = L.meta.solve_rbox_n[s];
            }
            info[s] = I;
        }
        L.fmg.upload(info, st());
    }
    // algorithmic bytes of one finest-level smoother launch (one colour pass
    // reads phi, rhs and, for ABec, a, bX, bY, bZ over the whole level and
    // writes phi: 7 words per cell; Poisson: 3)
    {
        double cells = 0;
        for (int p : lev[0].mg.h_plist) {
            const PatchDesc& P = lev[0].meta.patches[p];
            cells += (double)(P.hi[0] - P.lo[0] + 1) * (P.hi[1] - P.lo[1] + 1) * (P.hi[2] - P.lo[2] + 1);
        }
        E.m_kstats.cells_per_launch = cells;
        E.m_kstats.bytes_per_launch = cells * (abec ? 7.0 : 3.0) * (mixed() ? 4.0 : 8.0);
    }
    outer_residual_stats();
    MLMG_CUDA_CHECK(cudaEventCreate(&ev0));
    MLMG_CUDA_CHECK(cudaEventCreate(&ev1));
}

void Engine::Impl::build_bottom_tables ()
{
    std::vector<BottomLevelPtrs> tab(nlev_max);
    std::vector<BottomJob> jobs;
    for (int l = 0; l < nlev_max; ++l) {
        LevelData& L = lev[l];
        BottomLevelPtrs& B = tab[l];
        B.L = L.dl;
        B.tags = L.tags.p;
        if (L.has_bottom) {
            B.x = L.bw[0].p; B.b = L.bw[1].p; B.p = L.bw[2].p; B.r = L.bw[3].p;
            B.rh = L.bw[4].p; B.v = L.bw[5].p; B.t = L.bw[6].p;
        }
        B.a = L.a.p; B.bx = L.bx.p; B.by = L.by.p; B.bz = L.bz.p;
        B.x_out = mixed() ? (void*)L.cor32.p : (void*)L.cor.p;
        B.b_in = mixed() ? (const void*)L.res32.p : (const void*)L.res.p;
    }
    for (int s = 0; s < nsolve; ++s) {
        if (E.m_problems[s].spec.amr_fine) { continue; }   // a finer AMR level has no bottom solve
        const int l = (int)E.m_problems[s].spec.levels.size() - 1;
        BottomJob J{};
        J.lev = l; J.solve = s;
        J.p0 = lev[l].meta.solve_first_patch[s];
        J.np = lev[l].meta.solve_npatch[s];
        J.t0 = lev[l].solve_tag_first[s];
        J.nt = lev[l].solve_tag_n[s];
        J.singular = singular[s];
        J.volinv = volinv_bottom[s];
        jobs.push_back(J);
    }
    njobs = (int)jobs.size();
    long long max_cells = 0;
    for (const auto& J : jobs) {
        long long c = 0;
        for (int p = J.p0; p < J.p0 + J.np; ++p) {
            const PatchDesc& P = lev[J.lev].meta.patches[p];
            c += (long long)(P.hi[0] - P.lo[0] + 1) * (P.hi[1] - P.lo[1] + 1) * (P.hi[2] - P.lo[2] + 1);
        }
        max_cells = std::max(max_cells, c);
    }
    bot_threads = (max_cells <= 512) ? 32 : BOTTOM_THREADS;
    bot_levels.upload(tab, st());
    // coarse levels: from the bottom up, every level on which each solve has
    // at most coarse_cells cells (mixed path)
    lc = -1;
    if (mixed() && E.m_opt.coarse_block) {
        for (int l = nlev_max - 1; l >= 0; --l) {
            const PatchLevel& M = lev[l].meta;
            bool small = true;
            for (int s = 0; s < nsolve; ++s) {
                long long c = 0;
                for (int p = M.solve_first_patch[s]; p >= 0 && p < M.solve_first_patch[s] + M.solve_npatch[s]; ++p) {
                    const PatchDesc& P = M.patches[p];
                    c += (long long)(P.hi[0] - P.lo[0] + 1) * (P.hi[1] - P.lo[1] + 1) * (P.hi[2] - P.lo[2] + 1);
                }
                if (c > E.m_opt.coarse_cells) { small = false; }
            }
            if (!small) { break; }
            lc = l;
        }
        std::vector<CoarseLevelPtrs> ct(nlev_max);
        for (int l = 0; l < nlev_max; ++l) {
            LevelData& L = lev[l];
            L.tfirst_d.upload(L.solve_tag_first, st());
            L.tn_d.upload(L.solve_tag_n, st());
            ct[l] = CoarseLevelPtrs{L.dl, L.tags.p, L.tfirst_d.p, L.tn_d.p, L.cor32.p, L.res32.p, L.rescor32.p,
                                    stencil32(l)};
        }
        coarse_lv.upload(ct, st());
    }
    bot_jobs.upload(jobs, st());
}

// ----------------------------------------------------- user data transfer --
std::vector<XferItem> Engine::Impl::items_for (const FabSet& fs, int s, int ghost_mode, int nodal_dir) const
{
    // ghost_mode 0: valid cells (nodal-extended for faces); 1: valid cells,
    // the first ghost layer where it lies inside the owning patch (values of
    // the neighbouring boxes, as FillBoundary leaves them) and the face-ghost
    // layers on the patch's boundary (its ghost shell: boundary closures and
    // copies from other patches)
    std::vector<XferItem> items;
    const PatchLevel& M = lev[0].meta;
    const int p0 = M.solve_first_patch[s], np = M.solve_npatch[s];
    if ((int)xfer_loc.size() < nsolve) { xfer_loc.resize(nsolve); }
    if (!xfer_loc[s]) {
        std::vector<Box3> pbs;
        for (int p = p0; p < p0 + np; ++p) {
            Box3 pb; for (int d = 0; d < 3; ++d) { pb.lo[d] = M.patches[p].lo[d]; pb.hi[d] = M.patches[p].hi[d]; }
            pbs.push_back(pb);
        }
        xfer_loc[s] = std::make_unique<BoxLocator>(pbs);
    }
    for (size_t b = 0; b < fs.boxes.size(); ++b) {
        const Box3& vb = fs.boxes[b];
        const int loc = xfer_loc[s]->find(vb.lo[0], vb.lo[1], vb.lo[2]);
        const int pid = (loc >= 0) ? p0 + loc : -1;
        MLMG_REQUIRE(pid >= 0, ERR_ARGS, "MultiFab box outside the operator's BoxArray");
        Box3 fab = grow(vb, fs.ngrow);
        if (fs.nodal_dir >= 0) { fab.hi[fs.nodal_dir] += 1; }
        XferItem X{};
        X.patch = pid;
        X.src_off = fs.off[b];
        for (int d = 0; d < 3; ++d) { X.flo[d] = fab.lo[d]; }
        X.fsx = fab.len(0);
        X.fsxy = (long long)fab.len(0) * fab.len(1);
        Box3 reg = vb;
        if (nodal_dir >= 0) { reg.hi[nodal_dir] += 1; }
        if (ghost_mode == 1 && fs.ngrow >= 1 && nodal_dir < 0) {
            const PatchDesc& P = M.patches[pid];
            Box3 pb;
            for (int d = 0; d < 3; ++d) { pb.lo[d] = P.lo[d]; pb.hi[d] = P.hi[d]; }
            reg = intersect(grow(vb, 1), pb);
        }
        X.region = reg;
        items.push_back(X);
        if (ghost_mode == 1 && fs.ngrow >= 1) {
            const PatchDesc& P = M.patches[pid];
            for (int f = 0; f < 6; ++f) {
                const int d = f % 3;
                Box3 g = vb;
                if (f >= 3) { g.lo[d] = g.hi[d] = vb.hi[d] + 1; } else { g.lo[d] = g.hi[d] = vb.lo[d] - 1; }
                // only ghost layers on the patch boundary (the rest are valid cells of the patch)
                const bool on_patch_face = (f >= 3) ? (vb.hi[d] == P.hi[d]) : (vb.lo[d] == P.lo[d]);
                if (!on_patch_face) { continue; }
                X.region = g;
                items.push_back(X);
            }
        }
    }
    return items;
}

namespace {
bool same_item (const XferItem& a, const XferItem& b)
{
    for (int d = 0; d < 3; ++d) {
        if (a.region.lo[d] != b.region.lo[d] || a.region.hi[d] != b.region.hi[d] || a.flo[d] != b.flo[d]) {
            return false;
        }
    }
    return a.patch == b.patch && a.src_off == b.src_off && a.fsx == b.fsx && a.fsxy == b.fsxy;
}
} // namespace

const Engine::Impl::XferTables& Engine::Impl::xfer_tables_for (const std::vector<XferItem>& items)
{
    XferTables* T = nullptr;
    for (auto& c : xfer_tables) {
        if (c->items.size() != items.size()) { continue; }
        bool same = true;
        for (size_t w = 0; w < items.size() && same; ++w) { same = same_item(c->items[w], items[w]); }
        if (same) { T = c.get(); break; }
    }
    if (T == nullptr) {
        if (xfer_tables.size() < XFER_TABLES) {
            xfer_tables.push_back(std::make_unique<XferTables>());
            T = xfer_tables.back().get();
        } else {
            T = xfer_tables[0].get();
            for (auto& c : xfer_tables) { if (c->used < T->used) { T = c.get(); } }
        }
        std::vector<long long> start{0};
        for (const auto& X : items) {
            MLMG_REQUIRE(X.region.npts() < (1ll << 32), ERR_UNSUPPORTED, "a FAB of 2^32 cells or more");
            start.push_back(start.back() + X.region.npts());
        }
        // stream order keeps the upload behind the kernels that read the
        // tables this one replaces
        T->items = items;
        T->d_items.upload(items, st());
        T->d_start.upload(start, st());
        T->n = start.back();
    }
    T->used = ++xfer_tick;
    return *T;
}

void Engine::Impl::xfer (const std::vector<XferItem>& items, const FabSet& fs, void* field, bool field_is_f32,
                         int dir)
{
    if (items.empty()) { return; }
    const XferTables& T = xfer_tables_for(items);
    const XferItem* d_items = T.d_items.p;
    const long long* d_start = T.d_start.p;
    const long long n = T.n;
    const int threads = 256;
    const unsigned blocks = (unsigned)((n + (long long)threads * XF_CELLS - 1) / ((long long)threads * XF_CELLS));
    const DevLevel& dl = lev[0].dl;
    if (fs.prec == 8 && !field_is_f32) {
        k_xfer<double, double><<<blocks, threads, 0, st()>>>(dl, d_items, d_start, (int)items.size(), n,
            (double*)const_cast<void*>(fs.data), (double*)field, dir);
    } else if (fs.prec == 4 && !field_is_f32) {
        k_xfer<float, double><<<blocks, threads, 0, st()>>>(dl, d_items, d_start, (int)items.size(), n,
            (float*)const_cast<void*>(fs.data), (double*)field, dir);
    } else {
        MLMG_REQUIRE(false, ERR_UNSUPPORTED, "unsupported transfer precision");
    }
    launched();
    MLMG_CUDA_CHECK(cudaGetLastError());
    MLMG_CUDA_CHECK(cudaStreamSynchronize(st()));
}

void Engine::Impl::load_level0_field (const FabSet* fs, double* field, double defval, int nodal_dir, int s)
{
    if (fs == nullptr) {
        // constant value over the solve's level-0 patches (valid + nodal layer)
        const PatchLevel& M = lev[0].meta;
        std::vector<double> h((size_t)M.nelem, 0.0);
        MLMG_CUDA_CHECK(cudaMemcpyAsync(h.data(), field, h.size() * sizeof(double), cudaMemcpyDeviceToHost, st()));
        MLMG_CUDA_CHECK(cudaStreamSynchronize(st()));
        for (int p = M.solve_first_patch[s]; p < M.solve_first_patch[s] + M.solve_npatch[s]; ++p) {
            const PatchDesc& P = M.patches[p];
            Box3 r; for (int d = 0; d < 3; ++d) { r.lo[d] = P.lo[d]; r.hi[d] = P.hi[d]; }
            if (nodal_dir >= 0) { r.hi[nodal_dir] += 1; }
            for (int k = r.lo[2]; k <= r.hi[2]; ++k)
            for (int j = r.lo[1]; j <= r.hi[1]; ++j)
            for (int i = r.lo[0]; i <= r.hi[0]; ++i) { h[(size_t)pidx(P, i, j, k)] = defval; }
        }
        MLMG_CUDA_CHECK(cudaMemcpyAsync(field, h.data(), h.size() * sizeof(double), cudaMemcpyHostToDevice, st()));
        MLMG_CUDA_CHECK(cudaStreamSynchronize(st()));
        return;
    }
    MLMG_REQUIRE(fs->nodal_dir == nodal_dir, ERR_ARGS, "coefficient MultiFab has the wrong index type");
    xfer(items_for(*fs, s, 0, nodal_dir), *fs, field, false, 0);
}

// ------------------------------------------------------------ operations --

template <typename T>
void Engine::Impl::ghost (int l, T* phi, bool inhomog, bool do_copy, const double* bcv)
{
    const LevelData& L = lev[l];
    const long long n = L.gw.nfacecells + (do_copy ? L.gw.ntagcells : 0);
    if (n == 0) { return; }
    const int threads = 256;
    launch(k_ghost<T>, (unsigned)((n + threads - 1) / threads), threads, 0, 
        L.dl, L.gw, phi, inhomog ? 1 : 0, bcv ? bcv : ((l == 0) ? L.bcval.p : nullptr), do_copy ? 1 : 0);
    launched();
}

StencilPtrs Engine::Impl::stencil32 (int l) const
{
    const LevelData& L = lev[l];
    return StencilPtrs{L.D32.p, L.sx32.p, L.sy32.p, L.sz32.p};
}

StencilPtrs Engine::Impl::stencil64 (int l) const
{
    const LevelData& L = lev[l];
    return StencilPtrs{L.D.p, L.sx.p, L.sy.p, L.sz.p};
}

// one FP32 colour pass in stencil form (mixed path)
void Engine::Impl::gsrb32 (int l, float* cor, const float* res, int rb)
{
    const LevelData& L = lev[l];
    const StencilPtrs S = stencil32(l);
    const unsigned g = (unsigned)L.mg.ntiles;
    if (abec) {
        if (L.inline_bc) { launch(k_gsrb_s<float, true, true>, g, kTileBlock, 0, L.dl, L.mg.dev(), cor, res, S, rb); }
        else { launch(k_gsrb_s<float, true, false>, g, kTileBlock, 0, L.dl, L.mg.dev(), cor, res, S, rb); }
    } else {
        if (L.inline_bc) { launch(k_gsrb_s<float, false, true>, g, kTileBlock, 0, L.dl, L.mg.dev(), cor, res, S, rb); }
        else { launch(k_gsrb_s<float, false, false>, g, kTileBlock, 0, L.dl, L.mg.dev(), cor, res, S, rb); }
    }
    launched();
}

// rescor = res - L(cor), homogeneous BCs, FP32 stencil form (mixed path)
void Engine::Impl::resid32 (int l, float* rescor, float* cor, const float* res)
{
    const LevelData& L = lev[l];
    if (!L.inline_bc) { ghost<float>(l, cor, false, true); }
    const StencilPtrs S = stencil32(l);
    const unsigned g = (unsigned)L.mg.ntiles;
    float* const none = nullptr;
    if (abec) {
        if (L.inline_bc) {
            launch(k_residual_s<float, float, true, true, false>, g, kTileBlock, 0, L.dl, L.mg.dev(), rescor, cor,
                   res, S, nullptr, nullptr, none);
        } else {
            launch(k_residual_s<float, float, true, false, false>, g, kTileBlock, 0, L.dl, L.mg.dev(), rescor, cor,
                   res, S, nullptr, nullptr, none);
        }
    } else {
        if (L.inline_bc) {
            launch(k_residual_s<float, float, false, true, false>, g, kTileBlock, 0, L.dl, L.mg.dev(), rescor, cor,
                   res, S, nullptr, nullptr, none);
        } else {
            launch(k_residual_s<float, float, false, false, false>, g, kTileBlock, 0, L.dl, L.mg.dev(), rescor, cor,
                   res, S, nullptr, nullptr, none);
        }
    }
    launched();
}

// n fused two-colour sweeps on level l (mixed path), ping-ponging between
// cor32 and cor32b and ending in cor32
void Engine::Impl::smooth_fused (int l, int n, bool from_zero)
{
    LevelData& L = lev[l];
    const bool timed = E.m_opt.time_kernels && l == 0;
    float* a = L.cor32.p;
    float* b = L.cor32b.p;
    const CUtensorMap* ma = L.tm_a.p;      // tensor maps over a and b (TMA staging)
    const CUtensorMap* mb = L.tm_b.p;
    const bool use_tma = ma != nullptr;
    const StencilPtrs S = stencil32(l);
    for (int i = 0; i < n; ++i) {
        const int zero = (from_zero && i == 0) ? 1 : 0;
        if (timed) { kev_record(); }
        if (L.march) {
            const dim3 blk(MS_TX / 2, MS_TY);
            const int pm = (a == L.cor32.p) ? MT_PHI_A : MT_PHI_B;
            if (abec) {
                k_sweep_march_tma<true><<<L.mz.ntiles, blk, march_tma_smem_floats(true) * sizeof(float), st()>>>(
                    L.dl, L.mz.dev(), b, L.tm_m.p, pm, E.m_opt.march_tz, err_d.p);
            } else {
                k_sweep_march_tma<false><<<L.mz.ntiles, blk, march_tma_smem_floats(false) * sizeof(float), st()>>>(
                    L.dl, L.mz.dev(), b, L.tm_m.p, pm, E.m_opt.march_tz, err_d.p);
            }
        } else if (use_tma) {
            const dim3 g(L.fz.ntiles), blk(FS_TX, FS_TY);
            const CUtensorMap* pf = E.m_opt.fused_prefetch ? L.tm_pf.p : nullptr;
            const long long fw = E.m_opt.tma_first_wait < 0 ? tma::WAIT_LIMIT : E.m_opt.tma_first_wait;
            if (abec) {
                launch(k_sweep_fused2<true, true>, g, blk, 0, L.dl, L.fz.dev(), a, b, L.res32.p, S, ma, err_d.p,
                                                                fw, pf, zero, nullptr);
            } else {
                launch(k_sweep_fused2<false, true>, g, blk, 0, L.dl, L.fz.dev(), a, b, L.res32.p, S, ma, err_d.p,
                                                                 fw, pf, zero, nullptr);
            }
        } else {
            const dim3 g(L.fz.ntiles), blk(FS_TX, FS_TY);
            if (abec) {
                launch(k_sweep_fused2<true>, g, blk, 0, L.dl, L.fz.dev(), a, b, L.res32.p, S, nullptr, err_d.p,
                                                          tma::WAIT_LIMIT, nullptr, zero, nullptr);
            } else {
                launch(k_sweep_fused2<false>, g, blk, 0, L.dl, L.fz.dev(), a, b, L.res32.p, S, nullptr, err_d.p,
                                                           tma::WAIT_LIMIT, nullptr, zero, nullptr);
            }
        }
        launched();
        if (timed) { kev_record(); }
        std::swap(a, b);
        std::swap(ma, mb);
    }
    if (a != L.cor32.p) {
        MLMG_CUDA_CHECK(cudaMemcpyAsync(L.cor32.p, a, sizeof(float) * (size_t)L.meta.nelem, cudaMemcpyDeviceToDevice,
                                        st()));
    }
}

// computeResOfCorrection and the restriction of the result to the next MG
// level in one launch over a TMA-swept level's tiles (the correction in
// cor32, as the fused sweeps leave it); false where the level has no tensor
// maps or the option is off
bool Engine::Impl::resid_restrict_fused (int l)
{
    LevelData& L = lev[l];
    if (!E.m_opt.fused_restrict || !L.fused || L.march || L.tm_a.p == nullptr) { return false; }
    LevelData& C = lev[l + 1];
    const dim3 g(L.fz.ntiles), blk(FS_TX, FS_TY);
    const StencilPtrs S = stencil32(l);
    // ABec: the first two planes' stencil loads before the copy's wait, five
    // blocks per SM; MLPoisson loads only rhs, all eight planes early
    if (abec) {
        launch(k_resid_restrict_tma<true, 2, 5>, g, blk, 0, L.dl, L.fz.dev(), C.dl, L.res32.p, S, L.tm_a.p,
               C.res32.p, err_d.p);
    } else {
        launch(k_resid_restrict_tma<false, 8, 5>, g, blk, 0, L.dl, L.fz.dev(), C.dl, L.res32.p, S, L.tm_a.p,
               C.res32.p, err_d.p);
    }
    launched();
    return true;
}

template <typename T>
void Engine::Impl::smooth (int l, T* cor, const T* res, bool skip_fb)
{
    // MLCellLinOpT::smooth (AMReX_MLCellLinOp.H:1204-1217): per colour, applyBC then Fsmooth
    const LevelData& L = lev[l];
    const bool timed = E.m_opt.time_kernels && l == 0;
    for (int rb = 0; rb < 2; ++rb) {
        if constexpr (std::is_same_v<T, float>) {
            if (!L.inline_bc) { ghost<T>(l, cor, false, !skip_fb); }
        } else {
            ghost<T>(l, cor, false, !skip_fb);
        }
        skip_fb = false;
        if (timed) { kev_record(); }
        if constexpr (std::is_same_v<T, float>) {
            gsrb32(l, cor, res, rb);
        } else {
            if (abec) {
                launch(k_gsrb<T, true>, L.mg.ntiles, kTileBlock, 0, L.dl, L.mg.dev(), cor, res, coef<T>(l, 0),
                    coef<T>(l, 1), coef<T>(l, 2), coef<T>(l, 3), rb);
            } else {
                launch(k_gsrb<T, false>, L.mg.ntiles, kTileBlock, 0, L.dl, L.mg.dev(), cor, res, nullptr, nullptr,
                    nullptr, nullptr, rb);
            }
            launched();
        }
        if (timed) { kev_record(); }
    }
}

// rescor = res - L(cor), homogeneous BCs (MLMGT::computeResOfCorrection,
// AMReX_MLMG.H:1796-1803)
template <typename T>
void Engine::Impl::correction_residual (int l)
{
    LevelData& L = lev[l];
    T* cor = field_cor<T>(l);
    T* res = field_res<T>(l);
    T* rescor = field_rescor<T>(l);
    if constexpr (std::is_same_v<T, float>) {
        resid32(l, rescor, cor, res);
    } else {
        ghost<T>(l, cor, false, true);
        if (abec) {
            launch(k_residual<T, T, true>, L.mg.ntiles, kTileBlock, 0, L.dl, L.mg.dev(), rescor, cor, res,
                coef<T>(l, 0), coef<T>(l, 1), coef<T>(l, 2), coef<T>(l, 3), nullptr);
        } else {
            launch(k_residual<T, T, false>, L.mg.ntiles, kTileBlock, 0, L.dl, L.mg.dev(), rescor, cor, res,
                nullptr, nullptr, nullptr, nullptr, nullptr);
        }
        launched();
    }
}

// the bottom solve's BiCGStab iteration counts of this iteration's bottom
// solve number bslot, to the host (MLMGT::m_niters_cg keeps one per solve)
void Engine::Impl::bottom_done ()
{
    ++bslot;
}

// the bottom iteration counts of the iteration's bottom solves to the host,
// once at the end of the iteration (a copy between the V-cycle's kernels
// would stall their dependent launches)
void Engine::Impl::fetch_bottom_counts ()
{
    const size_t n = (size_t)std::min(bslot, nlev_max + 2) * nsolve;
    if (n == 0) { return; }
    MLMG_CUDA_CHECK(cudaMemcpyAsync(h_iters.p, bot_iters.p, sizeof(int) * n, cudaMemcpyDeviceToHost, st()));
    MLMG_CUDA_CHECK(cudaMemcpyAsync(h_iters2.p, bot_iters2.p, sizeof(int) * n, cudaMemcpyDeviceToHost, st()));
}

// the per-solve bottom solver on the device: set from the option at the
// first solve and whenever the option changes (a bicgcg / cgbicg switch made
// by an earlier solve is kept otherwise, as MLMGT keeps its bottom_solver)
void Engine::Impl::bottom_mode_init ()
{
    if (bot_mode_set == E.m_opt.bottom_solver) { return; }
    std::vector<int> m(nsolve, E.m_opt.bottom_solver);
    MLMG_CUDA_CHECK(cudaMemcpyAsync(bot_mode.p, m.data(), sizeof(int) * nsolve, cudaMemcpyHostToDevice, st()));
    MLMG_CUDA_CHECK(cudaStreamSynchronize(st()));
    bot_mode_set = E.m_opt.bottom_solver;
}

BottomParams Engine::Impl::bottom_params () const
{
    const EngineOptions& o = E.m_opt;
    return BottomParams{o.bottom_maxiter, o.bottom_reltol, o.bottom_abstol, o.nub, o.nuf,
                        o.bottom_solver == BK_SMOOTHER ? 1 : 0, bot_mode.p,
                        bot_iters2.p + (size_t)bottom_slot() * nsolve};
}

// MLMGT::mgVcycle (AMReX_MLMG.H:1306-1415) from MG level `top`, one stage per
// launch for every patch of every solve at that level.
template <typename T>
void Engine::Impl::vcycle (int top)
{
    const EngineOptions& o = E.m_opt;
    // levels >= top_end run in the coarse-level kernel (mixed path)
    const bool coarse = std::is_same_v<T, float> && lc >= 0 && top <= lc;
    const int top_end = coarse ? lc : nlev_max - 1;
    for (int l = top; l < top_end; ++l) {
        LevelData& L = lev[l];
        if (L.mg.n == 0) { continue; }
        T* cor = field_cor<T>(l);
        T* res = field_res<T>(l);
        T* rescor = field_rescor<T>(l);
        // the correction starts at zero: a fused level's first sweep takes
        // that as given, every other level clears the array
        const bool zero_sweep = std::is_same_v<T, float> && L.fused && !L.march && o.nu1 > 0;
        if (!zero_sweep) { MLMG_CUDA_CHECK(cudaMemsetAsync(cor, 0, (size_t)L.meta.nelem * sizeof(T), st())); }
        if (std::is_same_v<T, float> && L.fused) {
            smooth_fused(l, o.nu1, zero_sweep);
        } else {
            for (int i = 0; i < o.nu1; ++i) { smooth<T>(l, cor, res, i == 0); }
        }
        if (std::is_same_v<T, float> && resid_restrict_fused(l)) { continue; }
        correction_residual<T>(l);
        LevelData& C = lev[l + 1];
        launch(k_restrict<T>, C.all.ntiles, kTileBlock, 0, L.dl, C.dl, C.all.dev(), rescor, field_res<T>(l + 1));
        launched();
    }
    const BottomParams prm = bottom_params();
    int* const iters_slot = bot_iters.p + (size_t)bottom_slot() * nsolve;
    int* const ret_slot = bot_ret.p + (size_t)bottom_slot() * nsolve;
    // the coarse levels' stages in one block per solve, down and up, with the
    // one-warp bottom solve launched between them
    auto coarse_part = [&] (int part) {
        if (abec) {
            launch(k_coarse_vcycle<true>, njobs, COARSE_THREADS, 0, (const CoarseLevelPtrs*)coarse_lv.p, lc,
                   (const BottomLevelPtrs*)bot_levels.p, (const BottomJob*)bot_jobs.p, prm, o.nu1, o.nu2, iters_slot,
                   ret_slot, part);
        } else {
            launch(k_coarse_vcycle<false>, njobs, COARSE_THREADS, 0, (const CoarseLevelPtrs*)coarse_lv.p, lc,
                   (const BottomLevelPtrs*)bot_levels.p, (const BottomJob*)bot_jobs.p, prm, o.nu1, o.nu2, iters_slot,
                   ret_slot, part);
        }
        launched();
    };
    if (coarse) { coarse_part(1); }
    if (abec) {
        launch(k_bottom<T, true>, njobs, bot_threads, 0, bot_levels.p, bot_jobs.p, prm, nullptr, iters_slot,
               ret_slot);
    } else {
        launch(k_bottom<T, false>, njobs, bot_threads, 0, bot_levels.p, bot_jobs.p, prm, nullptr, iters_slot,
               ret_slot);
    }
    launched();
    if (coarse) { coarse_part(2); }
    bottom_done();
    for (int l = top_end - 1; l >= top; --l) {
        LevelData& L = lev[l];
        if (L.mg.n == 0) { continue; }
        T* cor = field_cor<T>(l);
        launch(k_interp_add<T>, L.mg.ntiles, kTileBlock, 0, L.dl, L.mg.dev(), lev[l + 1].dl, field_cor<T>(l + 1), cor);
        launched();
        if (std::is_same_v<T, float> && L.fused) {
            smooth_fused(l, o.nu2);
        } else {
            for (int i = 0; i < o.nu2; ++i) { smooth<T>(l, cor, field_res<T>(l), false); }
        }
    }
}

// MLMGT::mgFcycle (AMReX_MLMG.H:1420-1457): restrict the residual to every
// level, solve the bottom, then on each level from the coarsest up: assign the
// trilinear prolongation of the coarser correction, take its residual as the
// level's right-hand side, run a V-cycle from that level and add the
// prolongation back.  All solves of the batch have the same number of levels.
template <typename T>
void Engine::Impl::fcycle ()
{
    const int nb = nlev_max - 1;
    for (int l = 1; l <= nb; ++l) {
        LevelData& C = lev[l];
        // avgDownResMG (AMReX_MLLinOp.H:1563-1584)
        launch(k_restrict<T>, C.all.ntiles, kTileBlock, 0, lev[l - 1].dl, C.dl, C.all.dev(), field_res<T>(l - 1),
                                                             field_res<T>(l));
        launched();
    }
    {
        const EngineOptions& o = E.m_opt;
        const BottomParams prm = bottom_params();
        if (abec) {
            launch(k_bottom<T, true>, njobs, bot_threads, 0, bot_levels.p, bot_jobs.p, prm, nullptr,
                                                                  bot_iters.p + (size_t)bottom_slot() * nsolve,
                   bot_ret.p + (size_t)bottom_slot() * nsolve);
        } else {
            launch(k_bottom<T, false>, njobs, bot_threads, 0, bot_levels.p, bot_jobs.p, prm, nullptr,
                                                                   bot_iters.p + (size_t)bottom_slot() * nsolve,
                   bot_ret.p + (size_t)bottom_slot() * nsolve);
        }
        launched();
        bottom_done();
    }
    for (int l = nb - 1; l >= 0; --l) {
        LevelData& L = lev[l];
        T* cor = field_cor<T>(l);
        const size_t bytes = (size_t)L.meta.nelem * sizeof(T);
        if constexpr (std::is_same_v<T, float>) {
            // inline-BC levels keep no ghost values: give the coarse
            // correction the ghosts applyBC would have left
            if (lev[l + 1].inline_bc) { ghost<float>(l + 1, field_cor<float>(l + 1), false, true); }
        }
        k_interp_assign<T><<<L.mg.ntiles, kTileBlock, 0, st()>>>(L.dl, L.mg.dev(), lev[l + 1].dl, L.fmg.p, L.rbox.p,
                                                                 field_cor<T>(l + 1), cor);
        launched();
        correction_residual<T>(l);
        k_copy_valid<T><<<L.mg.ntiles, kTileBlock, 0, st()>>>(L.dl, L.mg.dev(), field_res<T>(l), field_rescor<T>(l));
        launched();
        T* hold;
        if constexpr (std::is_same_v<T, float>) {
            if (L.cor_hold32.n != (size_t)L.meta.nelem) { L.cor_hold32.alloc((size_t)L.meta.nelem); }
            hold = L.cor_hold32.p;
        } else {
            if (L.cor_hold.n != (size_t)L.meta.nelem) { L.cor_hold.alloc((size_t)L.meta.nelem); }
            hold = L.cor_hold.p;
        }
        MLMG_CUDA_CHECK(cudaMemcpyAsync(hold, cor, bytes, cudaMemcpyDeviceToDevice, st()));
        vcycle<T>(l);
        launch(k_add_to<T, T>, L.mg.ntiles, kTileBlock, 0, L.dl, L.mg.dev(), cor, hold, nullptr, nullptr, 0);
        launched();
    }
}

void Engine::Impl::reduce_per_solve (int l, const SubsetData& S, int op, const double* x, const double* y)
{
    const LevelData& L = lev[l];
    launch(k_reduce<double>, S.ntiles, kTileBlock, 0, L.dl, S.dev(), x, y, op, partial.p);
    launch(k_reduce_final, nsolve, 256, 0, partial.p, S.solve_begin.p, op, red_out.p);
    launched(2);
}

// res[0] = rhs - L(sol) with the solution's BCs (solutionResidual,
// AMReX_MLCellLinOp.H:1219-1236) and per-solve max|res| into red_out
void Engine::Impl::residual0 (bool to32, bool norm_zeroed)
{
    LevelData& L = lev[0];
    if (E.m_opt.transpose) {
        // adjoint solve: r = rhs - A^T sol, FP64, homogeneous BCs
        MLMG_CUDA_CHECK(cudaMemsetAsync(red_out.p, 0, sizeof(double) * nsolve, st()));
        ghost<double>(0, L.sol.p, false, true);
        const unsigned g = (unsigned)L.all.ntiles;
        const double *a = L.a.p, *bx = L.bx.p, *by = L.by.p, *bz = L.bz.p;
        if (to32) {
            if (abec) {
                k_residual_transpose<float, true><<<g, kTileBlock, 0, st()>>>(L.dl, L.all.dev(), L.res32.p, L.sol.p,
                    L.rhs.p, a, bx, by, bz, L.partner.p, red_out.p);
            } else {
                k_residual_transpose<float, false><<<g, kTileBlock, 0, st()>>>(L.dl, L.all.dev(), L.res32.p, L.sol.p,
                    L.rhs.p, a, bx, by, bz, L.partner.p, red_out.p);
            }
        } else {
            if (abec) {
                k_residual_transpose<double, true><<<g, kTileBlock, 0, st()>>>(L.dl, L.all.dev(), L.res.p, L.sol.p,
                    L.rhs.p, a, bx, by, bz, L.partner.p, red_out.p);
            } else {
                k_residual_transpose<double, false><<<g, kTileBlock, 0, st()>>>(L.dl, L.all.dev(), L.res.p, L.sol.p,
                    L.rhs.p, a, bx, by, bz, L.partner.p, red_out.p);
            }
        }
        launched();
        return;
    }
    if (to32) {
        // mixed path: FP64 residual in stencil form, FP32 copy for the V-cycle,
        // per-solve max-norm by atomic max (zeroed first)
        if (!norm_zeroed) { MLMG_CUDA_CHECK(cudaMemsetAsync(red_out.p, 0, sizeof(double) * nsolve, st())); }
        if (!L.inline_bc) { ghost<double>(0, L.sol.p, true, true); }
        const StencilPtrs S = stencil64(0);
        const unsigned g = (unsigned)L.all.ntiles;
        if (abec) {
            if (L.inline_bc) {
                launch(k_residual_s<double, float, true, true, true>, g, kTileBlock, 0, L.dl, L.all.dev(), L.res32.p,
                    L.sol.p, L.rhs.p, S, L.bcval.p, red_out.p, (float*)nullptr);
            } else {
                launch(k_residual_s<double, float, true, false, true>, g, kTileBlock, 0, L.dl, L.all.dev(),
                    L.res32.p, L.sol.p, L.rhs.p, S, L.bcval.p, red_out.p, (float*)nullptr);
            }
        } else {
            if (L.inline_bc) {
                launch(k_residual_s<double, float, false, true, true>, g, kTileBlock, 0, L.dl, L.all.dev(),
                    L.res32.p, L.sol.p, L.rhs.p, S, L.bcval.p, red_out.p, (float*)nullptr);
            } else {
                launch(k_residual_s<double, float, false, false, true>, g, kTileBlock, 0, L.dl, L.all.dev(),
                    L.res32.p, L.sol.p, L.rhs.p, S, L.bcval.p, red_out.p, (float*)nullptr);
            }
        }
        launched();
        return;
    }
    ghost<double>(0, L.sol.p, true, true);
    const double *a = L.a.p, *bx = L.bx.p, *by = L.by.p, *bz = L.bz.p;
    if (abec) {
        launch(k_residual<double, double, true>, L.all.ntiles, kTileBlock, 0, L.dl, L.all.dev(), L.res.p,
            L.sol.p, L.rhs.p, a, bx, by, bz, partial.p);
    } else {
        launch(k_residual<double, double, false>, L.all.ntiles, kTileBlock, 0, L.dl, L.all.dev(), L.res.p,
            L.sol.p, L.rhs.p, a, bx, by, bz, partial.p);
    }
    launch(k_reduce_final, nsolve, 256, 0, partial.p, L.all.solve_begin.p, RED_MAXABS, red_out.p);
    launched(2);
}

// MLMGT::oneIter (AMReX_MLMG.H:1227-1293), single AMR level, followed by the
// convergence residual of MLMGT::solve (:436-441)
void Engine::Impl::one_iteration (bool fmg)
{
    LevelData& L0 = lev[0];
    kev_used[0] = kev_used[1] = 0;
    const bool timed = E.m_opt.time_kernels != 0;
    bslot = 0;
    bool any_singular = false;
    for (int s : singular) { if (s) { any_singular = true; } }
    if (mixed()) {
        if (any_singular) {
            // makeSolvable on the (FP32) residual: offsets from FP64 sums
            launch(k_reduce<float>, L0.all.ntiles, kTileBlock, 0, L0.dl, L0.all.dev(), L0.res32.p, nullptr,
                                                                    RED_SUM, partial.p);
            launch(k_reduce_final, nsolve, 256, 0, partial.p, L0.all.solve_begin.p, RED_SUM, red_out.p + nsolve);
            launch(k_minus_offset<float>, L0.all.ntiles, kTileBlock, 0, L0.dl, L0.all.dev(), L0.res32.p,
                                                                         red_out.p + nsolve, volinv0_d.p);
            launched(3);
        }
        if (fmg) { fcycle<float>(); } else { vcycle<float>(0); }
        // phi += cor, which also clears the norms the residual takes its maximum into
        launch(k_add_to<double, float>, L0.all.ntiles, kTileBlock, 0, L0.dl, L0.all.dev(), L0.sol.p, L0.cor32.p,
               active_d.p, red_out.p, nsolve);
        launched();
        if (timed) { kev_record(1); }
        residual0(true, true);
        if (timed) { kev_record(1); }
    } else {
        if (any_singular) {
            launch(k_reduce<double>, L0.all.ntiles, kTileBlock, 0, L0.dl, L0.all.dev(), L0.res.p, nullptr,
                                                                     RED_SUM, partial.p);
            launch(k_reduce_final, nsolve, 256, 0, partial.p, L0.all.solve_begin.p, RED_SUM, red_out.p + nsolve);
            launch(k_minus_offset<double>, L0.all.ntiles, kTileBlock, 0, L0.dl, L0.all.dev(), L0.res.p,
                                                                          red_out.p + nsolve, volinv0_d.p);
            launched(3);
        }
        if (fmg) { fcycle<double>(); } else { vcycle<double>(0); }
        launch(k_add_to<double, double>, L0.all.ntiles, kTileBlock, 0, L0.dl, L0.all.dev(), L0.sol.p, L0.cor.p,
                                                                         active_d.p, nullptr, 0);
        launched();
        residual0(false);
    }
    MLMG_CUDA_CHECK(cudaMemcpyAsync(h_red.p, red_out.p, sizeof(double) * nsolve, cudaMemcpyDeviceToHost, st()));
    fetch_bottom_counts();
}

// algorithmic bytes and FP64 operations of one outer residual launch of the
// mixed path over the whole finest level: phi (8 B), rhs (8 B), the FP64
// stencil D, sX, sY, sZ (ABec, 32 B) and the FP32 residual (4 B) per cell;
// FP64 operations: 7 FMAs (14 FLOPs) per cell
void Engine::Impl::outer_residual_stats ()
{
    double cells = 0;
    for (int p : lev[0].all.h_plist) {
        const PatchDesc& P = lev[0].meta.patches[p];
        cells += (double)(P.hi[0] - P.lo[0] + 1) * (P.hi[1] - P.lo[1] + 1) * (P.hi[2] - P.lo[2] + 1);
    }
    KernelStats& R = E.m_rstats;
    R.cells_per_launch = cells;
    R.bytes_per_launch = cells * (abec ? 52.0 : 20.0);
    R.flops_per_launch = cells * 14.0;
}

// ---------------------------------------------------------------- Engine ---
bool same_iteration (const EngineOptions& a, const EngineOptions& b)
{
    return a.max_iter == b.max_iter && a.fixed_iter == b.fixed_iter && a.nu1 == b.nu1 && a.nu2 == b.nu2 &&
           a.nuf == b.nuf && a.nub == b.nub && a.bottom_solver == b.bottom_solver &&
           a.bottom_maxiter == b.bottom_maxiter && a.bottom_reltol == b.bottom_reltol &&
           a.bottom_abstol == b.bottom_abstol && a.always_use_bnorm == b.always_use_bnorm &&
           a.verbose == b.verbose && a.precision == b.precision && a.use_graph == b.use_graph &&
           a.fused_smoother == b.fused_smoother && a.merge_boxes == b.merge_boxes &&
           a.time_kernels == b.time_kernels && a.coarse_block == b.coarse_block &&
           a.coarse_cells == b.coarse_cells && a.march_sweep == b.march_sweep &&
           a.march_min_tiles == b.march_min_tiles && a.march_tz == b.march_tz && a.fused_tma == b.fused_tma &&
           a.fused_prefetch == b.fused_prefetch && a.max_fmg_iter == b.max_fmg_iter &&
           a.transpose == b.transpose && a.tma_first_wait == b.tma_first_wait &&
           a.final_fill_bc == b.final_fill_bc && a.pdl == b.pdl && a.fused_fine == b.fused_fine &&
           a.fused_restrict == b.fused_restrict;
}

Engine::Engine (std::vector<SolveProblem> problems, const EngineOptions& opt, cudaStream_t stream)
    : m_problems(std::move(problems)), m_opt(opt), m_stream(stream)
{
    m_impl = std::make_unique<Impl>(*this);
    m_impl->build();
    set_coefficients();
}

Engine::~Engine () = default;

void Engine::set_coefficients ()
{
    Impl& I = *m_impl;
    LevelData& L0 = I.lev[0];
    for (int s = 0; s < I.nsolve; ++s) {
        const SolveProblem& pr = m_problems[s];
        if (I.abec) {
            I.load_level0_field(pr.acoef, L0.a.p, 1.0, -1, s);
            for (int d = 0; d < 3; ++d) {
                double* dst = d == 0 ? L0.bx.p : (d == 1 ? L0.by.p : L0.bz.p);
                I.load_level0_field(pr.bcoef[d], dst, 1.0, d, s);
            }
        }
        // Dirichlet values: ghost cells of the level-BC MultiFab on the
        // domain faces (MLCellLinOpT::setLevelBC, AMReX_MLCellLinOp.H:552-649)
        if (pr.levelbc != nullptr) {
            const FabSet& fs = *pr.levelbc;
            MLMG_REQUIRE(fs.ngrow >= 1, ERR_ARGS, "level BC MultiFab needs one ghost cell");
            const PatchLevel& M = L0.meta;
            std::vector<double> hb(L0.bcval.n, 0.0);
            MLMG_CUDA_CHECK(cudaMemcpyAsync(hb.data(), L0.bcval.p, hb.size() * sizeof(double), cudaMemcpyDeviceToHost, m_stream));
            // pull the whole BC MultiFab to the host (setup only)
            long long total = 0;
            for (size_t b = 0; b < fs.boxes.size(); ++b) { total = std::max(total, fs.off[b] + grow(fs.boxes[b], fs.ngrow).npts()); }
            std::vector<double> hm((size_t)total);
            if (fs.prec == 8) {
                MLMG_CUDA_CHECK(cudaMemcpyAsync(hm.data(), fs.data, (size_t)total * 8, cudaMemcpyDeviceToHost, m_stream));
                MLMG_CUDA_CHECK(cudaStreamSynchronize(m_stream));
            } else {
                std::vector<float> hf((size_t)total);
                MLMG_CUDA_CHECK(cudaMemcpyAsync(hf.data(), fs.data, (size_t)total * 4, cudaMemcpyDeviceToHost, m_stream));
                MLMG_CUDA_CHECK(cudaStreamSynchronize(m_stream));
                for (size_t q = 0; q < hf.size(); ++q) { hm[q] = hf[q]; }
            }
            const Box3 dom = pr.spec.levels[0].geom.domain;
            for (int p = M.solve_first_patch[s]; p < M.solve_first_patch[s] + M.solve_npatch[s]; ++p) {
                const PatchDesc& P = M.patches[p];
                for (int f = 0; f < 6; ++f) {
                    const int d = f % 3;
                    const bool hi = f >= 3;
                    const int e0 = (d == 0) ? 1 : 0, e1 = (d == 2) ? 1 : 2;
                    const int nx0 = P.hi[e0] - P.lo[e0] + 1;
                    const int g = hi ? P.hi[d] + 1 : P.lo[d] - 1;
                    if (g >= dom.lo[d] && g <= dom.hi[d]) { continue; }     // not a physical face
                    for (size_t b = 0; b < fs.boxes.size(); ++b) {
                        const Box3& vb = fs.boxes[b];
                        if ((hi ? vb.hi[d] : vb.lo[d]) != (hi ? P.hi[d] : P.lo[d])) { continue; }
                        // only the boxes of this patch (others may share the face plane)
                        bool inside = true;
                        for (int e = 0; e < 3; ++e) { if (vb.lo[e] < P.lo[e] || vb.hi[e] > P.hi[e]) { inside = false; } }
                        if (!inside) { continue; }
                        const Box3 fab = grow(vb, fs.ngrow);
                        for (int v1 = vb.lo[e1]; v1 <= vb.hi[e1]; ++v1)
                        for (int v0 = vb.lo[e0]; v0 <= vb.hi[e0]; ++v0) {
                            int c[3];
                            c[d] = g; c[e0] = v0; c[e1] = v1;
                            const long long qm = fs.off[b] + ((long long)(c[2] - fab.lo[2]) * fab.len(1)
                                               + (c[1] - fab.lo[1])) * fab.len(0) + (c[0] - fab.lo[0]);
                            const long long u = (long long)(v1 - P.lo[e1]) * nx0 + (v0 - P.lo[e0]);
                            hb[(size_t)(P.face[f].bcval_off + u)] = hm[(size_t)qm];
                        }
                    }
                }
            }
            MLMG_CUDA_CHECK(cudaMemcpyAsync(L0.bcval.p, hb.data(), hb.size() * sizeof(double), cudaMemcpyHostToDevice, m_stream));
            MLMG_CUDA_CHECK(cudaStreamSynchronize(m_stream));
        }
        // coarse/fine faces of a level that does not cover its domain
        if (pr.crse_bc != nullptr) { coarse_fine_bc_values(I, s, pr.spec, *pr.crse_bc); }
    }
    restrict_coefficients();
}

void Engine::restrict_coefficients ()
{
    Impl& I = *m_impl;
    LevelData& L0 = I.lev[0];
    // restrict a and b to every MG level (averageDownCoeffsSameAmrLevel)
    if (I.abec) {
        int a_zero = 1;
        for (auto& pr : m_problems) { if (pr.spec.alpha != 0.0) { a_zero = 0; } }
        if (a_zero) { MLMG_CUDA_CHECK(cudaMemsetAsync(L0.a.p, 0, L0.a.n * sizeof(double), m_stream)); }
        for (int l = 1; l < I.nlev_max; ++l) {
            LevelData& F = I.lev[l - 1];
            LevelData& C = I.lev[l];
            k_restrict_coef<double><<<C.all.ntiles, kTileBlock, 0, m_stream>>>(F.dl, C.dl, C.all.dev(), F.a.p, F.bx.p,
                F.by.p, F.bz.p, C.a.p, C.bx.p, C.by.p, C.bz.p, a_zero);
            I.launched();
        }
        if (I.mixed()) {
            // stencil form on every level: D, s in FP64 and FP32
            for (int l = 0; l < I.nlev_max; ++l) {
                LevelData& L = I.lev[l];
                k_build_stencil<<<L.all.ntiles, kTileBlock, 0, m_stream>>>(L.dl, L.all.dev(), L.a.p, L.bx.p, L.by.p,
                    L.bz.p, L.D.p, L.sx.p, L.sy.p, L.sz.p, L.D32.p, L.sx32.p, L.sy32.p, L.sz32.p);
                I.launched();
            }
        }
    }
    MLMG_CUDA_CHECK(cudaGetLastError());
    MLMG_CUDA_CHECK(cudaStreamSynchronize(m_stream));
}

void Engine::apply (const FabSet& in, FabSet& out)
{
    Impl& I = *m_impl;
    MLMG_REQUIRE(I.nsolve == 1, ERR_UNSUPPORTED, "apply works on a single solve");
    LevelData& L0 = I.lev[0];
    I.xfer(I.items_for(in, 0, 0, -1), in, L0.sol.p, false, 0);
    I.ghost<double>(0, L0.sol.p, true, true);
    if (I.abec) {
        k_residual<double, double, true><<<L0.all.ntiles, kTileBlock, 0, m_stream>>>(L0.dl, L0.all.dev(), L0.res.p,
            L0.sol.p, nullptr, L0.a.p, L0.bx.p, L0.by.p, L0.bz.p, nullptr);
    } else {
        k_residual<double, double, false><<<L0.all.ntiles, kTileBlock, 0, m_stream>>>(L0.dl, L0.all.dev(), L0.res.p,
            L0.sol.p, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr);
    }
    I.launched();
    I.xfer(I.items_for(out, 0, 0, -1), out, L0.res.p, false, 1);
}

void Engine::comp_residual (const FabSet& sol, const FabSet& rhs, FabSet& res)
{
    Impl& I = *m_impl;
    MLMG_REQUIRE(I.nsolve == 1, ERR_UNSUPPORTED, "compResidual works on a single solve");
    LevelData& L0 = I.lev[0];
    I.xfer(I.items_for(sol, 0, 0, -1), sol, L0.sol.p, false, 0);
    I.xfer(I.items_for(rhs, 0, 0, -1), rhs, L0.rhs.p, false, 0);
    // MLCellLinOpT::solutionResidual (AMReX_MLCellLinOp.H:1219-1236): applyBC
    // with the level's boundary values, Fapply, then Xpay
    I.ghost<double>(0, L0.sol.p, true, true);
    if (I.abec) {
        k_residual<double, double, true><<<L0.all.ntiles, kTileBlock, 0, m_stream>>>(L0.dl, L0.all.dev(), L0.res.p,
            L0.sol.p, L0.rhs.p, L0.a.p, L0.bx.p, L0.by.p, L0.bz.p, nullptr);
    } else {
        k_residual<double, double, false><<<L0.all.ntiles, kTileBlock, 0, m_stream>>>(L0.dl, L0.all.dev(), L0.res.p,
            L0.sol.p, L0.rhs.p, nullptr, nullptr, nullptr, nullptr, nullptr);
    }
    I.launched();
    I.xfer(I.items_for(res, 0, 0, -1), res, L0.res.p, false, 1);
}

void Engine::face_fluxes (const FabSet& phi, FabSet* const out[3], int mode)
{
    Impl& I = *m_impl;
    MLMG_REQUIRE(I.nsolve == 1, ERR_UNSUPPORTED, "fluxes are computed for a single solve");
    MLMG_REQUIRE(mode == 0 || mode == 1, ERR_ARGS, "mode must be 0 (gradient) or 1 (flux)");
    LevelData& L0 = I.lev[0];
    const size_t n = (size_t)L0.meta.nelem;
    if (L0.face_phi.n != n) {
        L0.face_phi.alloc(n);
        for (auto& g : L0.face_out) { g.alloc(n); }
    }
    L0.face_phi.zero(m_stream);
    I.xfer(I.items_for(phi, 0, 0, -1), phi, L0.face_phi.p, false, 0);
    I.ghost<double>(0, L0.face_phi.p, true, true);
    double* o[3] = {L0.face_out[0].p, L0.face_out[1].p, L0.face_out[2].p};
    const unsigned g = (unsigned)L0.all.ntiles;
    const double *bx = L0.bx.p, *by = L0.by.p, *bz = L0.bz.p;
    if (mode == 0) {
        k_face_flux<0, false><<<g, kTileBlock, 0, m_stream>>>(L0.dl, L0.all.dev(), L0.face_phi.p, bx, by, bz, o[0],
                                                              o[1], o[2]);
    } else if (I.abec) {
        k_face_flux<1, true><<<g, kTileBlock, 0, m_stream>>>(L0.dl, L0.all.dev(), L0.face_phi.p, bx, by, bz, o[0],
                                                             o[1], o[2]);
    } else {
        k_face_flux<1, false><<<g, kTileBlock, 0, m_stream>>>(L0.dl, L0.all.dev(), L0.face_phi.p, bx, by, bz, o[0],
                                                              o[1], o[2]);
    }
    I.launched();
    MLMG_CUDA_CHECK(cudaGetLastError());
    for (int d = 0; d < 3; ++d) {
        if (out[d]) {
            MLMG_REQUIRE(out[d]->nodal_dir == d, ERR_ARGS, "face MultiFabs must be face-centred in x, y, z");
            I.xfer(I.items_for(*out[d], 0, 0, d), *out[d], L0.face_out[d].p, false, 1);
        }
    }
}

void Engine::adjoint_gradient (const FabSet& phi, FabSet* const grad_b[3], FabSet* grad_a)
{
    Impl& I = *m_impl;
    MLMG_REQUIRE(I.nsolve == 1 && m_opt.transpose, ERR_INTERNAL, "adjoint_gradient needs a transposed engine of one solve");
    MLMG_REQUIRE(I.abec, ERR_UNSUPPORTED, "coefficient gradients need MLABecLaplacian");
    LevelData& L0 = I.lev[0];
    const size_t n = (size_t)L0.meta.nelem;
    if (L0.face_phi.n != n) {
        L0.face_phi.alloc(n);
        for (auto& g : L0.face_out) { g.alloc(n); }
    }
    // phi with the ghosts of the inhomogeneous applyBC; lambda (the last
    // transposed solution, valid cells) with copies between patches
    L0.face_phi.zero(m_stream);
    I.xfer(I.items_for(phi, 0, 0, -1), phi, L0.face_phi.p, false, 0);
    I.ghost<double>(0, L0.face_phi.p, true, true);
    I.ghost<double>(0, L0.sol.p, false, true);
    double* g[3];
    for (int d = 0; d < 3; ++d) { g[d] = grad_b[d] ? L0.face_out[d].p : nullptr; }
    k_face_grad<<<L0.all.ntiles, kTileBlock, 0, m_stream>>>(L0.dl, L0.all.dev(), L0.face_phi.p, L0.sol.p, g[0], g[1],
                                                            g[2], grad_a ? L0.face_out[3].p : nullptr);
    I.launched();
    MLMG_CUDA_CHECK(cudaGetLastError());
    for (int d = 0; d < 3; ++d) {
        if (grad_b[d]) {
            MLMG_REQUIRE(grad_b[d]->nodal_dir == d, ERR_ARGS, "dJ/db MultiFabs must be face-centred in x, y, z");
            I.xfer(I.items_for(*grad_b[d], 0, 0, d), *grad_b[d], L0.face_out[d].p, false, 1);
        }
    }
    if (grad_a) { I.xfer(I.items_for(*grad_a, 0, 0, -1), *grad_a, L0.face_out[3].p, false, 1); }
}

void Engine::solve (const std::vector<const FabSet*>& sol_in, const std::vector<FabSet*>& sol_out,
                    const std::vector<const FabSet*>& rhs, double tol_rel, double tol_abs)
{
    Impl& I = *m_impl;
    const int ns = I.nsolve;
    MLMG_REQUIRE((int)sol_in.size() == ns && (int)sol_out.size() == ns && (int)rhs.size() == ns, ERR_ARGS,
                 "one sol and one rhs per solve");
    LevelData& L0 = I.lev[0];
    m_reports.assign(ns, SolveReport{});
    // initial guess (valid cells) and rhs; the solution's ghosts come from BCs
    MLMG_CUDA_CHECK(cudaMemsetAsync(L0.sol.p, 0, L0.sol.n * sizeof(double), m_stream));
    MLMG_CUDA_CHECK(cudaMemsetAsync(L0.rhs.p, 0, L0.rhs.n * sizeof(double), m_stream));
    // a graph captured under other options is not this iteration
    if (I.graph_exec != nullptr && !same_iteration(I.graph_opt, m_opt)) { I.drop_graphs(); }
    for (int s = 0; s < ns; ++s) {
        I.xfer(I.items_for(*sol_in[s], s, 0, -1), *sol_in[s], L0.sol.p, false, 0);
        I.xfer(I.items_for(*rhs[s], s, 0, -1), *rhs[s], L0.rhs.p, false, 0);
    }
    MLMG_CUDA_CHECK(cudaEventRecord(I.ev0, m_stream));
    // enforce solvability of singular problems (MLMGT::makeSolvable, AMReX_MLMG.H:1844-1858)
    bool any_singular = false;
    for (int s : I.singular) { if (s) { any_singular = true; } }
    MLMG_REQUIRE(!(any_singular && m_opt.transpose), ERR_UNSUPPORTED,
                 "adjoint solves of singular operators are not supported");
    if (m_opt.transpose && I.abec && L0.gw.ntagcells > 0) {
        if (L0.partner.n != (size_t)L0.meta.nelem) { L0.partner.alloc((size_t)L0.meta.nelem); }
        L0.partner.zero(m_stream);
        k_partner_faces<<<(unsigned)((L0.gw.ntagcells + 255) / 256), 256, 0, m_stream>>>(L0.dl, L0.gw, L0.bx.p,
            L0.by.p, L0.bz.p, L0.partner.p);
        I.launched();
    }
    if (any_singular) {
        k_reduce<double><<<L0.all.ntiles, kTileBlock, 0, m_stream>>>(L0.dl, L0.all.dev(), L0.rhs.p, nullptr, RED_SUM,
                                                                    I.partial.p);
        k_reduce_final<<<ns, 256, 0, m_stream>>>(I.partial.p, L0.all.solve_begin.p, RED_SUM, I.red_out.p + ns);
        k_minus_offset<double><<<L0.all.ntiles, kTileBlock, 0, m_stream>>>(L0.dl, L0.all.dev(), L0.rhs.p,
                                                                          I.red_out.p + ns, I.volinv0_d.p);
        I.launched(3);
    }
    // initial residual and norms (AMReX_MLMG.H:391-420); the mixed forward
    // solve takes the norm from its stencil-form FP64 residual, which also
    // leaves the FP32 copy the first V-cycle reads (the FP64 path keeps the
    // reference's operation order)
    const bool fused_init = I.mixed() && !m_opt.transpose;
    I.residual0(fused_init);
    MLMG_CUDA_CHECK(cudaMemcpyAsync(I.h_red.p, I.red_out.p, sizeof(double) * ns, cudaMemcpyDeviceToHost, m_stream));
    I.reduce_per_solve(0, L0.all, RED_MAXABS, L0.rhs.p, nullptr);
    MLMG_CUDA_CHECK(cudaMemcpyAsync(I.h_red.p + ns, I.red_out.p, sizeof(double) * ns, cudaMemcpyDeviceToHost, m_stream));
    MLMG_CUDA_CHECK(cudaStreamSynchronize(m_stream));
    std::vector<double> target(ns), max_norm(ns);
    std::vector<int> active(ns, 1);
    for (int s = 0; s < ns; ++s) {
        SolveReport& R = m_reports[s];
        R.init_resid = I.h_red.p[s];
        R.rhs_norm = I.h_red.p[ns + s];
        max_norm[s] = (m_opt.always_use_bnorm || R.rhs_norm >= R.init_resid) ? R.rhs_norm : R.init_resid;
        target[s] = std::max(tol_abs, std::max(tol_rel, 1.e-16) * max_norm[s]);
        R.final_resid = R.init_resid;
        if (R.init_resid <= target[s]) { active[s] = 0; }
        if (m_opt.verbose >= 1) {
            std::printf("MLMG: Initial rhs               = %.10g\nMLMG: Initial residual (resid0) = %.10g\n",
                        R.rhs_norm, R.init_resid);
        }
    }
    // the transposed (adjoint) mixed solve takes its norm from the FP64
    // residual above and makes the FP32 copy for its first V-cycle here
    if (I.mixed() && !fused_init) { I.residual0(true); }
    MLMG_CUDA_CHECK(cudaMemcpyAsync(I.active_d.p, active.data(), sizeof(int) * ns, cudaMemcpyHostToDevice, m_stream));
    I.bottom_mode_init();
    const int niters = m_opt.fixed_iter ? m_opt.fixed_iter : m_opt.max_iter;
    bool any_active = false;
    for (int a : active) { if (a) { any_active = true; } }
    int& per_iter_launches = I.graph_launches;
    if (m_opt.max_fmg_iter > 0) {
        for (int s = 0; s < ns; ++s) {
            MLMG_REQUIRE((int)m_problems[s].spec.levels.size() == I.nlev_max, ERR_UNSUPPORTED,
                         "F-cycles need every solve of a batch to have the same number of MG levels");
        }
    }
    int graph_bslots = 1;
    for (int iter = 0; iter < niters && any_active; ++iter) {
        if (iter < m_opt.max_fmg_iter) {
            // F-cycles run eagerly: they differ from the replayed V-cycle iteration
            I.one_iteration(true);
        } else if (m_opt.use_graph) {
            if (I.graph_exec == nullptr) {
                const int before = m_launches;
                cudaGraph_t g;
                MLMG_CUDA_CHECK(cudaStreamBeginCapture(m_stream, cudaStreamCaptureModeThreadLocal));
                I.capturing = true;
                I.one_iteration(false);
                I.capturing = false;
                graph_bslots = I.bslot;
                MLMG_CUDA_CHECK(cudaStreamEndCapture(m_stream, &g));
                MLMG_CUDA_CHECK(cudaGraphInstantiate(&I.graph_exec, g, 0));
                MLMG_CUDA_CHECK(cudaGraphDestroy(g));
                I.graph_opt = m_opt;
                per_iter_launches = m_launches - before;
                m_launches = before;
            }
            MLMG_CUDA_CHECK(cudaGraphLaunch(I.graph_exec, m_stream));
            m_launches += per_iter_launches;
            I.bslot = graph_bslots;
        } else {
            I.one_iteration(false);
        }
        MLMG_CUDA_CHECK(cudaGetLastError());
        MLMG_CUDA_CHECK(cudaStreamSynchronize(m_stream));
        if (m_opt.time_kernels) { I.kev_harvest(); }
        bool changed = false;
        for (int s = 0; s < ns; ++s) {
            if (!active[s]) { continue; }
            SolveReport& R = m_reports[s];
            const double fine = I.h_red.p[s];
            R.history.push_back(fine);
            for (int q = 0; q < I.bslot && q < I.nlev_max + 2; ++q) {
                R.cg_iters.push_back(I.h_iters.p[(size_t)q * ns + s]);
                // a bicgcg / cgbicg bottom solve that ran its second solver
                // counts twice, as MLMGT::bottomSolveWithCG records each call
                const int second = I.h_iters2.p[(size_t)q * ns + s];
                if (second >= 0) { R.cg_iters.push_back(second); }
            }
            R.niters++;
            R.final_resid = fine;
            if (m_opt.verbose >= 2) {
                std::printf("MLMG: Iteration %3d Fine resid/%s = %.10g\n", iter + 1,
                            (max_norm[s] == R.rhs_norm) ? "bnorm" : "resid0", fine / max_norm[s]);
            }
            if (!std::isfinite(fine)) {
                R.status = ERR_NONFINITE; active[s] = 0; changed = true;
            } else if (fine <= target[s]) {
                R.status = OK; active[s] = 0; changed = true;
            } else if (fine > 1.e20 * max_norm[s]) {
                R.status = ERR_DIVERGED; active[s] = 0; changed = true;
            }
        }
        if (changed) {
            MLMG_CUDA_CHECK(cudaMemcpyAsync(I.active_d.p, active.data(), sizeof(int) * ns, cudaMemcpyHostToDevice,
                                            m_stream));
        }
        any_active = false;
        for (int a : active) { if (a) { any_active = true; } }
    }
    MLMG_CUDA_CHECK(cudaEventRecord(I.ev1, m_stream));
    I.check_device_error();
    for (int s = 0; s < ns; ++s) {
        if (active[s] && m_opt.fixed_iter == 0) { m_reports[s].status = NOT_CONVERGED; }
        if (m_opt.verbose >= 1) {
            std::printf("MLMG: Final Iter. %d resid, resid/bnorm = %.10g, %.10g\n", m_reports[s].niters,
                        m_reports[s].final_resid, m_reports[s].final_resid / max_norm[s]);
        }
    }
    // write back the solution: valid cells and, for one-ghost MultiFabs (the
    // reference's aliased solution) or with final_fill_bc (MLMGT::solve,
    // AMReX_MLMG.H:515-524), the ghost layer left by the last residual
    // evaluation
    bool any_ghosts = false;
    for (int s = 0; s < ns; ++s) {
        const FabSet& out = *sol_out[s];
        any_ghosts = any_ghosts || out.ngrow == 1 || (m_opt.final_fill_bc && out.ngrow >= 1);
    }
    // the ghost layer of the final solution: boundary closures with the level
    // BC values and copies between patches (kernels that evaluate the
    // closures in registers leave the stored layer behind)
    if (any_ghosts) { I.ghost<double>(0, L0.sol.p, true, true); }
    for (int s = 0; s < ns; ++s) {
        FabSet& out = *sol_out[s];
        const bool ghosts = out.ngrow == 1 || (m_opt.final_fill_bc && out.ngrow >= 1);
        I.xfer(I.items_for(out, s, ghosts ? 1 : 0, -1), out, L0.sol.p, false, 1);
    }
    MLMG_CUDA_CHECK(cudaEventSynchronize(I.ev1));
    float ms = 0;
    MLMG_CUDA_CHECK(cudaEventElapsedTime(&ms, I.ev0, I.ev1));
    m_last_ms = ms;
}

// the AMR composite driver (amr.cu) calls these on the engines of its levels
template void Engine::Impl::ghost<double> (int, double*, bool, bool, const double*);
template void Engine::Impl::ghost<float> (int, float*, bool, bool, const double*);
template void Engine::Impl::smooth<double> (int, double*, const double*, bool);
template void Engine::Impl::smooth<float> (int, float*, const float*, bool);
template void Engine::Impl::vcycle<double> (int);
template void Engine::Impl::vcycle<float> (int);
template void Engine::Impl::fcycle<double> ();
template void Engine::Impl::fcycle<float> ();
template void Engine::Impl::correction_residual<double> (int);
template void Engine::Impl::correction_residual<float> (int);

} // namespace mlmg
