// Internal state of the MLMG engine (Engine::Impl and its per-level data),
// shared by the single-level engine (solver.cu) and the AMR composite
// driver (amr.cu).  Not part of the public interface.
#pragma once

#include "solver.hpp"
#include "bottom.cuh"
#include "stencil_kernels.cuh"
#include "fused_sweep.cuh"
#include "fused_sweep2.cuh"
#include "march_sweep.cuh"
#include "coarse_vcycle.cuh"
#include "adjoint_kernels.cuh"
#include "flux_kernels.cuh"
#include "fmg_kernels.cuh"

#include <algorithm>
#include <numeric>

namespace mlmg {


struct SubsetData {
    DevBuf<int> plist, tstart, solve_begin;
    std::vector<int> h_plist, h_tstart, h_solve_begin;
    int n = 0, ntiles = 0;
    Subset dev () const { return Subset{plist.p, tstart.p, n, ntiles}; }
};

inline int tiles_of (const PatchDesc& P)
{
    const int nx = P.hi[0] - P.lo[0] + 1, ny = P.hi[1] - P.lo[1] + 1, nz = P.hi[2] - P.lo[2] + 1;
    return ((nx + TILE_X - 1) / TILE_X) * ((ny + TILE_Y - 1) / TILE_Y) * ((nz + TILE_Z - 1) / TILE_Z);
}

inline void build_subset (SubsetData& S, const PatchLevel& PL, const std::vector<int>& plist, int nsolve,
                   cudaStream_t st)
{
    S.h_plist = plist;
    S.n = (int)plist.size();
    S.h_tstart.assign(S.n + 1, 0);
    for (int q = 0; q < S.n; ++q) { S.h_tstart[q + 1] = S.h_tstart[q] + tiles_of(PL.patches[plist[q]]); }
    S.ntiles = S.h_tstart[S.n];
    S.h_solve_begin.assign(nsolve + 1, 0);
    // tiles of solve s are [begin[s], begin[s+1]) (patches are grouped by solve)
    int q = 0;
    for (int s = 0; s < nsolve; ++s) {
        S.h_solve_begin[s] = S.h_tstart[q];
        while (q < S.n && PL.patches[plist[q]].solve == s) { ++q; }
    }
    S.h_solve_begin[nsolve] = S.ntiles;
    if (S.n > 0) {
        S.plist.upload(S.h_plist, st);
        S.tstart.upload(S.h_tstart, st);
    }
    S.solve_begin.upload(S.h_solve_begin, st);
}


// 3-D tiled tensor map over the allocation of patch P inside an FP32 level
// field (the fused sweep's staging box by default)
CUtensorMap patch_tensor_map (const float* field, const PatchDesc& P, int by = FS_AY, int bz = FS_AZ,
                              int bx = FS_AX);

struct LevelData {
    PatchLevel meta;
    DevBuf<PatchDesc> P;
    DevBuf<int8_t> masks;
    DevBuf<int> sfirst, snp;
    DevBuf<CopyTag> tags;
    DevBuf<int2> faces;
    DevBuf<long long> fstart, tstart;
    GhostWork gw{};
    SubsetData all, mg;
    DevLevel dl{};
    // FP64 fields
    DevBuf<double> cor, res, rescor, a, bx, by, bz;
    DevBuf<double> sol, rhs, bcval;                 // level 0 only
    DevBuf<double> face_phi, face_out[4];           // level 0 scratch: a solution with ghosts and face outputs
                                                    // (adjoint gradients, fluxes), allocated on demand
    DevBuf<double> partner;                         // level 0, periodic image face coefficients (A^T)
    // FP32 fields (mixed precision)
    DevBuf<float> cor32, res32, rescor32;
    // stencil form of the ABec operator (mixed path): FP64 on every level,
    // FP32 copies for the FP32 V-cycle
    DevBuf<double> D, sx, sy, sz;
    DevBuf<float> D32, sx32, sy32, sz32;
    bool inline_bc = false;   // ghost values computed inside the stencil kernels
    // fused two-colour sweeps (mixed path): tile map and the second buffer
    bool fused = false;
    SubsetData fz;
    DevBuf<CUtensorMap> tm_a, tm_b;   // per patch: tensor maps of the 40x12x12 staging box over cor32 / cor32b
    DevBuf<CUtensorMap> tm_pf;        // per patch: FS_PF_NMAP L2-prefetch maps (rhs, D, sX, sY, sZ)
    DevBuf<CUtensorMap> tm_m;         // per patch: MT_NMAP plane maps of the TMA z-march
    bool march = false;           // fused sweeps by the z-marching kernel
    SubsetData mz;
    DevBuf<float> cor32b;
    DevBuf<int> tfirst_d, tn_d;    // per-solve tag ranges (coarse-level kernel)
    // F-cycles: the solves' own boxes of this level, interpolation data for
    // this level as the fine one, and the saved corrections (on demand)
    DevBuf<Box3> rbox;
    DevBuf<FmgSolveInfo> fmg;
    DevBuf<double> cor_hold;
    DevBuf<float> cor_hold32;
    // bottom work arrays
    DevBuf<double> bw[7];
    bool has_bottom = false;
    std::vector<int> solve_tag_first, solve_tag_n;  // tags grouped per solve
};

struct Engine::Impl {
    Engine& E;
    int nsolve = 0;
    int nlev_max = 0;
    bool abec = false;
    std::vector<LevelData> lev;
    std::vector<int> singular;
    std::vector<double> volinv0, volinv_bottom;
    DevBuf<double> partial, red_out, volinv0_d;
    DevBuf<int> active_d, bot_iters, bot_ret;
    DevBuf<int> bot_iters2, bot_mode;   // second bottom solver's iterations; per solve BottomKind
    int bot_mode_set = -1;       // the bottom_solver option bot_mode was last initialised from
    DevBuf<int> err_d;           // device-side error report of bounded waits (0: none)
    PinnedBuf<double> h_red;
    PinnedBuf<int> h_iters, h_iters2;
    DevBuf<BottomLevelPtrs> bot_levels;
    DevBuf<BottomJob> bot_jobs;
    int njobs = 0;
    // one warp when every bottom level is tiny (its block barriers are then
    // nearly free), else BOTTOM_THREADS
    int bot_threads = BOTTOM_THREADS;
    // levels >= lc run inside k_coarse_vcycle (one block per solve); -1: none
    int lc = -1;
    DevBuf<CoarseLevelPtrs> coarse_lv;
    cudaGraphExec_t graph_exec = nullptr;
    EngineOptions graph_opt{};   // the options the graph was captured with
    int graph_launches = 0;      // kernels in one replay of the iteration graph
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    // event pairs around the finest-level smoother launches (0) and the outer
    // residual (1) of one iteration
    std::vector<cudaEvent_t> kev[2];
    int kev_used[2] = {0, 0};
    bool capturing = false;
    int bslot = 0;               // bottom solves issued in the current iteration

    explicit Impl (Engine& e) : E(e) {}
    ~Impl () {
        drop_graphs();
        if (ev0) { cudaEventDestroy(ev0); }
        if (ev1) { cudaEventDestroy(ev1); }
        for (auto& v : kev) { for (auto e : v) { cudaEventDestroy(e); } }
    }

    void drop_graphs ()
    {
        if (graph_exec) { cudaGraphExecDestroy(graph_exec); }
        graph_exec = nullptr;
    }

    void kev_record (int t = 0)
    {
        std::vector<cudaEvent_t>& v = kev[t];
        if (kev_used[t] >= (int)v.size()) {
            cudaEvent_t e;
            MLMG_CUDA_CHECK(cudaEventCreate(&e));
            v.push_back(e);
        }
        cudaEvent_t e = v[kev_used[t]++];
        if (capturing) {
            MLMG_CUDA_CHECK(cudaEventRecordWithFlags(e, st(), cudaEventRecordExternal));
        } else {
            MLMG_CUDA_CHECK(cudaEventRecord(e, st()));
        }
    }

    void kev_harvest ()
    {
        KernelStats* out[2] = {&E.m_kstats, &E.m_rstats};
        for (int t = 0; t < 2; ++t) {
            for (int q = 0; q + 1 < kev_used[t]; q += 2) {
                float ms = 0;
                MLMG_CUDA_CHECK(cudaEventElapsedTime(&ms, kev[t][q], kev[t][q + 1]));
                out[t]->total_ms += ms;
                out[t]->launches += 1;
            }
        }
    }

    cudaStream_t st () const { return E.m_stream; }
    // a V-cycle kernel on the engine's stream, as a programmatic dependent
    // launch (the kernel calls pdl_wait before it reads what the previous
    // kernel wrote) unless the pdl option is off
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
        cfg.numAttrs = E.m_opt.pdl ? 1 : 0;
        MLMG_CUDA_CHECK(cudaLaunchKernelEx(&cfg, kern, std::forward<Args>(args)...));
    }
    bool mixed () const { return E.m_opt.precision == 1; }
    void launched (int n = 1) { E.m_launches += n; }

    // ------------------------------------------------------------ setup --
    void build ();
    void build_bottom_tables ();
    void outer_residual_stats ();
    void load_level0_field (const FabSet* fs, double* field, double defval, int nodal_dir, int s);
    void xfer (const std::vector<XferItem>& items, const FabSet& fs, void* field, bool field_is_f32, int dir);
    std::vector<XferItem> items_for (const FabSet& fs, int s, int ghost_mode, int nodal_dir) const;
    // transfer tables: device copies kept while a transfer's items recur (a
    // MultiFab and a level give the same items from call to call, and an
    // upload from pageable memory makes the host wait for the stream), least
    // recently used replaced; per solve a locator of its level-0 patches
    struct XferTables {
        std::vector<XferItem> items;
        DevBuf<XferItem> d_items;
        DevBuf<long long> d_start;
        long long n = 0;
        unsigned long long used = 0;
    };
    static constexpr size_t XFER_TABLES = 8;
    std::vector<std::unique_ptr<XferTables>> xfer_tables;
    unsigned long long xfer_tick = 0;
    const XferTables& xfer_tables_for (const std::vector<XferItem>& items);
    mutable std::vector<std::unique_ptr<BoxLocator>> xfer_loc;

    // ------------------------------------------------------- operations --
    // bcv: Dirichlet values of an inhomogeneous fill (null: the level-0 values)
    template <typename T> void ghost (int l, T* phi, bool inhomog, bool do_copy, const double* bcv = nullptr);
    template <typename T> void smooth (int l, T* cor, const T* res, bool skip_fb);
    template <typename T> void vcycle (int top);
    template <typename T> void fcycle ();
    template <typename T> void correction_residual (int l);
    void bottom_done ();
    void fetch_bottom_counts ();
    int bottom_slot () const { return std::min(bslot, nlev_max + 1); }
    BottomParams bottom_params () const;
    void bottom_mode_init ();
    template <typename T> T* field_cor (int l);
    template <typename T> T* field_res (int l);
    template <typename T> T* field_rescor (int l);
    template <typename T> const T* coef (int l, int which);
    void reduce_per_solve (int l, const SubsetData& S, int op, const double* x, const double* y);
    StencilPtrs stencil32 (int l) const;
    StencilPtrs stencil64 (int l) const;
    void gsrb32 (int l, float* cor, const float* res, int rb);
    void smooth_fused (int l, int n, bool from_zero = false);
    bool resid_restrict_fused (int l);
    void resid32 (int l, float* rescor, float* cor, const float* res);
    void residual0 (bool to32, bool norm_zeroed = false);   // res[0] (FP64, or FP32 in mixed) and its max-norm
    void one_iteration (bool fmg);
    // reads (and clears) the device-side error report of bounded waits; throws if set
    void check_device_error ()
    {
        int h = 0;
        MLMG_CUDA_CHECK(cudaMemcpyAsync(&h, err_d.p, sizeof(int), cudaMemcpyDeviceToHost, st()));
        MLMG_CUDA_CHECK(cudaStreamSynchronize(st()));
        if (h != 0) {
            MLMG_CUDA_CHECK(cudaMemsetAsync(err_d.p, 0, sizeof(int), st()));
            MLMG_REQUIRE(h != tma::ERR_TMA_TIMEOUT, ERR_TIMEOUT, "a fused-sweep tile's TMA copy did not complete");
            MLMG_REQUIRE(false, ERR_INTERNAL, "a fused-sweep tile's TMA box was not 16-byte aligned");
        }
    }
};

static const dim3 kTileBlock(32, TILE_Y);

// The Dirichlet values of the coarse/fine faces of solve s's level 0 when
// its boxes do not cover the domain, interpolated from the coarse data
// `crse` (refinement ratio 2; amr.cu)
void coarse_fine_bc_values (Engine::Impl& I, int s, const SolveSpec& S, const FabSet& crse);

} // namespace mlmg
