// Fused two-colour red-black Gauss-Seidel sweep (FP32, stencil form): tile
// geometry, the tile map and the per-patch constants shared by the sweep
// kernels (k_sweep_fused2 in fused_sweep2.cuh, k_sweep_march_tma in
// march_sweep.cuh).
//
// One launch performs both colour passes of MLCellLinOpT::smooth
// (AMReX_MLCellLinOp.H:1204-1217) with the arithmetic of abec_gsrb /
// mlpoisson_gsrb, reading each array from HBM about once: ~7 words per cell
// per sweep instead of 7 words per colour pass.  Out of place
// (phi_in -> phi_out), so no block reads another block's output.  Ghost
// values at patch faces are computed inline from the two cells next to the
// face (Dirichlet closure of at most 3 points, Neumann, reflect_odd): for the
// first colour from phi_in, for the second from the first colour's new
// values -- what applyBC would store before each pass.
#pragma once

#include "stencil_kernels.cuh"

namespace mlmg {

constexpr int FS_TX = 32;       // output tile
constexpr int FS_TY = 8;
constexpr int FS_TZ = 8;
constexpr int FS_THREADS = FS_TX * FS_TY;
constexpr int FS_AX = FS_TX + 8;                       // staged row: x0-4 .. x0+FS_TX+3 (16-byte chunks)
constexpr int FS_AY = FS_TY + 4, FS_AZ = FS_TZ + 4;    // y0-2 .., z0-2 ..
constexpr int FS_NX = FS_TX + 2, FS_NY = FS_TY + 2, FS_NZ = FS_TZ + 2;   // first colour on tile + 1
constexpr int FS_RED_ROW = FS_NX / 2;                  // first-colour cells per row of the tile + 1

__device__ __forceinline__ TileCoord decode_fused_tile (const DevLevel& L, const Subset& S, int b)
{
    int lo = 0, hi = S.n - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (S.tstart[mid] <= b) { lo = mid; } else { hi = mid - 1; }
    }
    TileCoord c;
    c.p = S.plist[lo];
    const PatchDesc& P = L.P[c.p];
    const int t = b - S.tstart[lo];
    const int ntx = (P.hi[0] - P.lo[0] + FS_TX) / FS_TX;
    const int nty = (P.hi[1] - P.lo[1] + FS_TY) / FS_TY;
    c.x0 = P.lo[0] + (t % ntx) * FS_TX;
    c.y0 = P.lo[1] + ((t / ntx) % nty) * FS_TY;
    c.z0 = P.lo[2] + (t / (ntx * nty)) * FS_TZ;
    return c;
}

inline int fused_tiles_of (const PatchDesc& P)
{
    const int nx = P.hi[0] - P.lo[0] + 1, ny = P.hi[1] - P.lo[1] + 1, nz = P.hi[2] - P.lo[2] + 1;
    return ((nx + FS_TX - 1) / FS_TX) * ((ny + FS_TY - 1) / FS_TY) * ((nz + FS_TZ - 1) / FS_TZ);
}

struct FaceLite {
    int type, nx;
    float c1, c2, fco;
};

struct PatchLite {
    int lo[3], hi[3];
    int sx;
    long long sxy, base;
    float dhx, dhy, dhz;
    FaceLite f[6];
    __device__ __forceinline__ long long idx (int i, int j, int k) const {
        return base + (long long)(k - lo[2]) * sxy + (long long)(j - lo[1]) * sx + (i - lo[0]);
    }
    __device__ __forceinline__ bool inside (int i, int j, int k) const {
        return i >= lo[0] && i <= hi[0] && j >= lo[1] && j <= hi[1] && k >= lo[2] && k <= hi[2];
    }
    // homogeneous inline closure of face f from the cell itself and the next inner cell
    __device__ __forceinline__ float closure (int fi, float pc, float pin) const {
        const FaceLite& F = f[fi];
        if (F.type == BC_DIRICHLET) {
            float g = (F.nx >= 2) ? pc * F.c1 : 0.0f;
            if (F.nx >= 3) { g += pin * F.c2; }
            return g;
        }
        if (F.type == BC_NEUMANN) { return pc; }
        if (F.type == BC_REFLECT_ODD) { return -pc; }
        return 0.0f;
    }
};

__device__ __forceinline__ void cp_async16 (void* smem, const void* gmem)
{
    const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" :: "r"(s), "l"(gmem) : "memory");
}

__device__ __forceinline__ void cp_async_wait_all ()
{
    asm volatile("cp.async.commit_group;\ncp.async.wait_group 0;\n" ::: "memory");
}

} // namespace mlmg
