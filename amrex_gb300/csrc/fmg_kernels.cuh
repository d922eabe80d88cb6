// F-cycle prolongation: MLCellLinOpT::interpAssign (AMReX_MLCellLinOp.H:
// 1003-1100) with mlmg_lin_cc_interp_r2 (AMReX_MLMG_3D_K.H:7-37): the fine
// correction is assigned the trilinear interpolation of the coarse one,
// weights 27/64, 9/64, 3/64, 1/64 on the coarse cell and its neighbours
// towards the fine cell.
//
// Coarse values outside a coarse box come, as in the reference, from
// FillBoundary (neighbouring boxes and periodic images) when MFIter over the
// two levels is safe -- both levels' grids made by coarsening the level-0
// BoxArray -- and otherwise from a ParallelCopy into zeroed coarsened fine
// boxes.  Outside the domain the safe case keeps what the coarse FAB's ghost
// cell holds: on a face of the coarse box the value the last applyBC left
// there, on an edge or corner zero (setVal at the start of the V-cycle);
// the other case gives zero.  Patches merge boxes, so the "coarse box" of a
// fine cell is the coarsening of the solve's own fine box that contains it.
#pragma once

#include "kernels.cuh"
#include "stage_kernels.cuh"

namespace mlmg {

struct FmgSolveInfo {       // one solve, fine level l -> coarse level l+1
    Box3 cdom;              // coarse domain
    int per[3];             // periodic directions
    int safe;               // isMFIterSafe between the two levels
    int rbox0, nrbox;       // the solve's own fine boxes in the level's box list
};

// patch of solve s at level L containing (i,j,k), or -1
__device__ __forceinline__ int find_patch_or_none (const DevLevel& L, int s, int i, int j, int k)
{
    const int p0 = L.sfirst[s], np = L.snp[s];
    for (int p = p0; p < p0 + np; ++p) {
        const PatchDesc& P = L.P[p];
        if (i >= P.lo[0] && i <= P.hi[0] && j >= P.lo[1] && j <= P.hi[1] && k >= P.lo[2] && k <= P.hi[2]) {
            return p;
        }
    }
    return -1;
}

template <typename T>
__device__ __forceinline__ T coarse_at (const DevLevel& Lc, const FmgSolveInfo& I, const Box3* __restrict__ rbox,
                                        const T* __restrict__ crse, int s, int i, int j, int k, int ci, int cj,
                                        int ck)
{
    // a valid coarse cell, periodic images included (FillBoundary / ParallelCopy)
    int c[3] = {ci, cj, ck};
    bool in_domain = true;
    for (int d = 0; d < 3; ++d) {
        const int lo = I.cdom.lo[d], hi = I.cdom.hi[d];
        if (c[d] < lo || c[d] > hi) {
            if (I.per[d]) {
                const int n = hi - lo + 1;
                c[d] = lo + ((c[d] - lo) % n + n) % n;
            } else {
                in_domain = false;
            }
        }
    }
    if (in_domain) {
        const int p = find_patch_or_none(Lc, s, c[0], c[1], c[2]);
        if (p >= 0) { return crse[cidx(Lc.P[p], c[0], c[1], c[2])]; }
    }
    if (!I.safe) { return T(0); }
    // the coarse box of this fine cell
    Box3 cb{};
    bool found = false;
    for (int q = I.rbox0; q < I.rbox0 + I.nrbox && !found; ++q) {
        const Box3& b = rbox[q];
        if (b.contains(i, j, k)) {
            for (int d = 0; d < 3; ++d) { cb.lo[d] = b.lo[d] >> 1; cb.hi[d] = b.hi[d] >> 1; }
            found = true;
        }
    }
    if (!found) { return T(0); }
    const int u[3] = {ci, cj, ck};
    int nout = 0, dout = 0;
    for (int d = 0; d < 3; ++d) {
        if (u[d] < cb.lo[d] || u[d] > cb.hi[d]) { ++nout; dout = d; }
    }
    if (nout != 1) { return T(0); }
    // a face ghost of the coarse box: the ghost cell of the patch holding the box
    int v[3] = {u[0], u[1], u[2]};
    v[dout] = (u[dout] < cb.lo[dout]) ? cb.lo[dout] : cb.hi[dout];
    const int p = find_patch_or_none(Lc, s, v[0], v[1], v[2]);
    if (p < 0) { return T(0); }
    const PatchDesc& P = Lc.P[p];
    if (u[dout] < P.lo[dout] - 1 || u[dout] > P.hi[dout] + 1) { return T(0); }
    return crse[cidx(P, u[0], u[1], u[2])];
}

template <typename T>
__global__ void __launch_bounds__(TILE_THREADS)
k_interp_assign (DevLevel Lf, Subset S, DevLevel Lc, const FmgSolveInfo* __restrict__ info,
                 const Box3* __restrict__ rbox, const T* __restrict__ crse, T* __restrict__ fine)
{
    const TileCoord c = decode_tile(Lf, S, blockIdx.x);
    const PatchDesc& P = Lf.P[c.p];
    const int j = c.y0 + threadIdx.y;
    if (j > P.hi[1]) { return; }
    const int s = P.solve;
    const FmgSolveInfo I = info[s];
    for (int kk = 0; kk < TILE_Z; ++kk) {
        const int k = c.z0 + kk;
        if (k > P.hi[2]) { break; }
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const int i = c.x0 + threadIdx.x + 32 * h;
            if (i > P.hi[0]) { continue; }
            const int kc = k >> 1, koff = 2 * (k - kc * 2) - 1;
            const int jc = j >> 1, joff = 2 * (j - jc * 2) - 1;
            const int ic = i >> 1, ioff = 2 * (i - ic * 2) - 1;
            auto cc = [&] (int a, int b, int d) { return coarse_at<T>(Lc, I, rbox, crse, s, i, j, k, a, b, d); };
            const T v = T(0.421875) * cc(ic, jc, kc)
                      + T(0.140625) * cc(ic + ioff, jc, kc)
                      + T(0.140625) * cc(ic, jc + joff, kc)
                      + T(0.140625) * cc(ic, jc, kc + koff)
                      + T(0.046875) * cc(ic, jc + joff, kc + koff)
                      + T(0.046875) * cc(ic + ioff, jc, kc + koff)
                      + T(0.046875) * cc(ic + ioff, jc + joff, kc)
                      + T(0.015625) * cc(ic + ioff, jc + joff, kc + koff);
            fine[cidx(P, i, j, k)] = v;
        }
    }
}

// dst = src over the valid cells of a subset (the copy res = rescor of mgFcycle)
template <typename T>
__global__ void __launch_bounds__(TILE_THREADS)
k_copy_valid (DevLevel L, Subset S, T* __restrict__ dst, const T* __restrict__ src)
{
    const TileCoord c = decode_tile(L, S, blockIdx.x);
    const PatchDesc& P = L.P[c.p];
    const int j = c.y0 + threadIdx.y;
    if (j > P.hi[1]) { return; }
    for (int kk = 0; kk < TILE_Z; ++kk) {
        const int k = c.z0 + kk;
        if (k > P.hi[2]) { break; }
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const int i = c.x0 + threadIdx.x + 32 * h;
            if (i > P.hi[0]) { continue; }
            const long long q = cidx(P, i, j, k);
            dst[q] = src[q];
        }
    }
}

} // namespace mlmg
