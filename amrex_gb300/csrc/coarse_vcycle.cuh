// The coarse part of the V-cycle (mixed path) in one thread block per solve.
//
// Below a few ten thousand cells per solve, every V-cycle stage of MLMGT::
// mgVcycle (AMReX_MLMG.H:1306-1415) -- smooth, correction residual,
// restriction, the bottom solve, interpolation, smooth -- is a handful of
// microseconds of work but a full kernel launch.  This kernel runs all the
// stages of levels lc..bottom of one solve inside one block, separated by
// block barriers, and ends with the correction of level lc ready for the
// grid-wide kernels above it.  Stage arithmetic is that of the grid-wide
// FP32 kernels (stencil form, ghost values filled as applyBC does); the
// bottom solve is the FP64 BiCGStab of bottom.cuh.  `part` selects the
// stages: 1 the levels down to the bottom, 2 the levels back up from it, 3
// all of them with the bottom solve inside this block (1 and 2 leave the
// bottom solve to the one-warp k_bottom launched between them).
#pragma once

#include "bottom.cuh"
#include "stencil_kernels.cuh"

namespace mlmg {

constexpr int COARSE_THREADS = 512;

struct CoarseLevelPtrs {
    DevLevel L;
    const CopyTag* tags;
    const int* tfirst;      // first ghost-copy tag of each solve at this level
    const int* tn;          // number of tags of each solve
    float *cor, *res, *rescor;
    StencilPtrs S;          // FP32 stencil form (null for MLPoisson)
};

template <bool ABEC>
__global__ void __launch_bounds__(COARSE_THREADS, 1)
k_coarse_vcycle (const CoarseLevelPtrs* __restrict__ lv, int lc, const BottomLevelPtrs* __restrict__ blev,
                 const BottomJob* __restrict__ jobs, BottomParams prm, int nu1, int nu2,
                 int* __restrict__ out_iters, int* __restrict__ out_ret, int part)
{
    using namespace bottom_detail;
    pdl_wait();
    pdl_trigger();
    const BottomJob J = jobs[blockIdx.x];
    const int s = J.solve, lb = J.lev;

    auto smooth_level = [&] (const CoarseLevelPtrs& C, int p0, int np, int t0, int nt) {
        for (int rb = 0; rb < 2; ++rb) {
            ghost_fill<float>(C.L, C.tags, p0, np, t0, nt, C.cor);
            for_cells(C.L, p0, np, [&] (const PatchDesc& P, int i, int j, int k, long long) {
                if (((i + j + k + rb) & 1) == 0) {
                    gsrb_s_cell<float, ABEC, false>(C.L, P, i, j, k, C.cor, C.res, C.S);
                }
            });
            __syncthreads();
        }
    };

    // ---- down
    for (int l = lc; l < lb && (part & 1); ++l) {
        const CoarseLevelPtrs& C = lv[l];
        const int p0 = C.L.sfirst[s], np = C.L.snp[s], t0 = C.tfirst[s], nt = C.tn[s];
        // cor = 0, ghosts included
        for (int p = p0; p < p0 + np; ++p) {
            const PatchDesc& P = C.L.P[p];
            const long long n0 = P.base - P.sxy - P.sx - XOFF;   // the patch's whole allocation
            const long long n = P.sxy * (P.hi[2] - P.lo[2] + 3);
            for (long long u = threadIdx.x; u < n; u += blockDim.x) { C.cor[n0 + u] = 0.0f; }
        }
        __syncthreads();
        for (int i = 0; i < nu1; ++i) { smooth_level(C, p0, np, t0, nt); }
        // rescor = res - L(cor)
        ghost_fill<float>(C.L, C.tags, p0, np, t0, nt, C.cor);
        for_cells(C.L, p0, np, [&] (const PatchDesc& P, int i, int j, int k, long long q) {
            const float xc = C.cor[q];
            float xm, xp, ym, yp, zm, zp;
            neighbours<float, false, false>(P, P, i, j, k, q, C.cor, xc, nullptr, xm, xp, ym, yp, zm, zp);
            const Coef7<float, ABEC> cf = load_coef<float, ABEC>(P, q, C.S);
            const float nb = cf.sxl * xm + cf.sxh * xp + cf.syl * ym + cf.syh * yp + cf.szl * zm + cf.szh * zp;
            C.rescor[q] = C.res[q] - (cf.d * xc - nb);
        });
        __syncthreads();
        // res(l+1) = average of rescor(l) (amrex_avgdown order)
        const CoarseLevelPtrs& Cc = lv[l + 1];
        for_cells(Cc.L, Cc.L.sfirst[s], Cc.L.snp[s], [&] (const PatchDesc& PC, int i, int j, int k, long long qc) {
            const PatchDesc& F = C.L.P[find_patch(C.L, s, 2 * i, 2 * j, 2 * k)];
            const long long qf = cidx(F, 2 * i, 2 * j, 2 * k);
            const long long sx = F.sx, sxy = F.sxy;
            float v = 0;
            v += C.rescor[qf];            v += C.rescor[qf + 1];
            v += C.rescor[qf + sx];       v += C.rescor[qf + sx + 1];
            v += C.rescor[qf + sxy];      v += C.rescor[qf + sxy + 1];
            v += C.rescor[qf + sxy + sx]; v += C.rescor[qf + sxy + sx + 1];
            Cc.res[qc] = (1.0f / 8.0f) * v;
        });
        __syncthreads();
    }

    // ---- bottom (FP64)
    if (part == 3) { bottom_solve_block<float, ABEC>(blev[lb], J, prm, out_iters, out_ret); }

    // ---- up
    for (int l = lb - 1; l >= lc && (part & 2); --l) {
        const CoarseLevelPtrs& C = lv[l];
        const CoarseLevelPtrs& Cc = lv[l + 1];
        const int p0 = C.L.sfirst[s], np = C.L.snp[s], t0 = C.tfirst[s], nt = C.tn[s];
        for_cells(C.L, p0, np, [&] (const PatchDesc&, int i, int j, int k, long long q) {
            const int ic = i >> 1, jc = j >> 1, kc = k >> 1;
            const PatchDesc& PC = Cc.L.P[find_patch(Cc.L, s, ic, jc, kc)];
            C.cor[q] += Cc.cor[cidx(PC, ic, jc, kc)];
        });
        __syncthreads();
        for (int i = 0; i < nu2; ++i) { smooth_level(C, p0, np, t0, nt); }
    }
}

} // namespace mlmg
