// Device kernels of the GB300 MLMG.  All stencils are memory-bound: no tensor
// cores.  Every kernel walks a *subset* of the patches of one level through a
// tile map (64 x 4 x TZ cells per 128-thread block; block -> patch by binary
// search over a prefix of tile counts), so one launch covers every box of a
// level and every solve of a batch.
#pragma once

#include "common.hpp"

namespace mlmg {

constexpr int TILE_X = 64;        // cells per tile along x (two per lane)
constexpr int TILE_Y = 4;         // rows per tile (one per warp)
constexpr int TILE_Z = 4;         // planes per tile
constexpr int TILE_THREADS = 128;

// Programmatic dependent launch: the V-cycle's kernels are launched so that a
// kernel's blocks may start while the previous kernel drains.  Each such
// kernel reads only static data (tile maps, patch descriptors) before
// pdl_wait(), which returns once the previous kernel has completed and its
// writes are visible; pdl_trigger() then lets the next kernel be launched.
// Both are no-ops for a kernel launched the ordinary way.
__device__ __forceinline__ void pdl_wait () { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void pdl_trigger () { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }

struct DevLevel {
    const PatchDesc* P;
    const int8_t* masks;
    const int* sfirst;    // first patch of each solve at this level (-1: none)
    const int* snp;       // number of patches of each solve at this level
    int npatch;
};

struct Subset {           // launch map over a subset of a level's patches
    const int* plist;     // patch ids, grouped by solve
    const int* tstart;    // prefix of tile counts, n+1 entries
    int n;
    int ntiles;
};

struct TileCoord { int p; int x0, y0, z0; };

__device__ __forceinline__ TileCoord decode_tile (const DevLevel& L, const Subset& S, int b)
{
    int lo = 0, hi = S.n - 1;
    while (lo < hi) {                       // last s with tstart[s] <= b
        const int mid = (lo + hi + 1) >> 1;
        if (S.tstart[mid] <= b) { lo = mid; } else { hi = mid - 1; }
    }
    TileCoord c;
    c.p = S.plist[lo];
    const PatchDesc& P = L.P[c.p];
    const int t = b - S.tstart[lo];
    const int ntx = (P.hi[0] - P.lo[0] + TILE_X) / TILE_X;
    const int nty = (P.hi[1] - P.lo[1] + TILE_Y) / TILE_Y;
    c.x0 = P.lo[0] + (t % ntx) * TILE_X;
    c.y0 = P.lo[1] + ((t / ntx) % nty) * TILE_Y;
    c.z0 = P.lo[2] + (t / (ntx * nty)) * TILE_Z;
    return c;
}

__host__ __device__ __forceinline__ long long cidx (const PatchDesc& P, int i, int j, int k)
{
    return P.base + (long long)(k - P.lo[2]) * P.sxy + (long long)(j - P.lo[1]) * P.sx + (i - P.lo[0]);
}

// the index geometry (and MLPoisson factors) of a patch, loaded once into
// registers by the streaming kernels instead of being read through the
// descriptor inside their cell loops
struct PatchGeom {
    int lo[3], hi[3];
    long long base, sxy;
    int sx, solve;
    double dha[3];
};

__device__ __forceinline__ PatchGeom geom_of (const PatchDesc& P)
{
    PatchGeom g;
#pragma unroll
    for (int d = 0; d < 3; ++d) { g.lo[d] = P.lo[d]; g.hi[d] = P.hi[d]; g.dha[d] = P.dha[d]; }
    g.base = P.base;
    g.sxy = P.sxy;
    g.sx = P.sx;
    g.solve = P.solve;
    return g;
}

__host__ __device__ __forceinline__ long long cidx (const PatchGeom& P, int i, int j, int k)
{
    return P.base + (long long)(k - P.lo[2]) * P.sxy + (long long)(j - P.lo[1]) * P.sx + (i - P.lo[0]);
}

__device__ __forceinline__ bool contains (const PatchGeom& P, int i, int j, int k)
{
    return i >= P.lo[0] && i <= P.hi[0] && j >= P.lo[1] && j <= P.hi[1] && k >= P.lo[2] && k <= P.hi[2];
}

// mask value of the outside cell (i,j,k) adjacent to face f of patch P
__device__ __forceinline__ int face_mask (const DevLevel& L, const PatchDesc& P, int f, int i, int j, int k)
{
    const FaceBC& F = P.face[f];
    if (F.mask_uniform >= 0) { return F.mask_uniform; }
    const int d = f % 3;
    const int nx = P.hi[0] - P.lo[0] + 1, ny = P.hi[1] - P.lo[1] + 1;
    long long q;
    if (d == 0) { q = (long long)(k - P.lo[2]) * ny + (j - P.lo[1]); }
    else if (d == 1) { q = (long long)(k - P.lo[2]) * nx + (i - P.lo[0]); }
    else { q = (long long)(j - P.lo[1]) * nx + (i - P.lo[0]); }
    return L.masks[F.mask_off + q];
}

// smoother coefficient of face f at boundary cell (i,j,k): f where mask > 0
__device__ __forceinline__ double face_cf (const DevLevel& L, const PatchDesc& P, int f, int i, int j, int k)
{
    const int d = f % 3;
    int oi = i, oj = j, ok = k;
    const int s = (f >= 3) ? 1 : -1;
    if (d == 0) { oi += s; } else if (d == 1) { oj += s; } else { ok += s; }
    return (face_mask(L, P, f, oi, oj, ok) > 0) ? P.face[f].fco : 0.0;
}

// ------------------------------------------------------- per-cell stencils --
// One red-black Gauss-Seidel update of cell (i,j,k): abec_gsrb
// (AMReX_MLABecLap_3D_K.H:208-264) and mlpoisson_gsrb (AMReX_MLPoisson_3D_K.H:153-196)
template <typename T, bool ABEC>
__device__ __forceinline__ void gsrb_cell (const DevLevel& L, const PatchDesc& P, int i, int j, int k,
                                           T* __restrict__ phi, const T* __restrict__ rhs,
                                           const T* __restrict__ a, const T* __restrict__ bx,
                                           const T* __restrict__ by, const T* __restrict__ bz)
{
    const long long q = cidx(P, i, j, k);
    const long long sx = P.sx, sxy = P.sxy;
    const T omega = T(1.15);
    const T dhx = T(P.dhs[0]), dhy = T(P.dhs[1]), dhz = T(P.dhs[2]);
    T cf0 = 0, cf1 = 0, cf2 = 0, cf3 = 0, cf4 = 0, cf5 = 0;
    if (i == P.lo[0]) { cf0 = T(face_cf(L, P, 0, i, j, k)); }
    if (j == P.lo[1]) { cf1 = T(face_cf(L, P, 1, i, j, k)); }
    if (k == P.lo[2]) { cf2 = T(face_cf(L, P, 2, i, j, k)); }
    if (i == P.hi[0]) { cf3 = T(face_cf(L, P, 3, i, j, k)); }
    if (j == P.hi[1]) { cf4 = T(face_cf(L, P, 4, i, j, k)); }
    if (k == P.hi[2]) { cf5 = T(face_cf(L, P, 5, i, j, k)); }
    const T pc = phi[q];
    if constexpr (ABEC) {
        const T bxl = bx[q], bxh = bx[q + 1];
        const T byl = by[q], byh = by[q + sx];
        const T bzl = bz[q], bzh = bz[q + sxy];
        const T gamma = T(P.alpha) * a[q] + dhx * (bxl + bxh) + dhy * (byl + byh) + dhz * (bzl + bzh);
        const T g_m_d = gamma - (dhx * (bxl * cf0 + bxh * cf3) + dhy * (byl * cf1 + byh * cf4)
                                 + dhz * (bzl * cf2 + bzh * cf5));
        const T rho = dhx * (bxl * phi[q - 1] + bxh * phi[q + 1])
                    + dhy * (byl * phi[q - sx] + byh * phi[q + sx])
                    + dhz * (bzl * phi[q - sxy] + bzh * phi[q + sxy]);
        const T res = rhs[q] - (gamma * pc - rho);
        phi[q] = pc + omega / g_m_d * res;
    } else {
        const T gamma = T(-2.0) * (dhx + dhy + dhz);
        const T g_m_d = gamma + dhx * (cf0 + cf3) + dhy * (cf1 + cf4) + dhz * (cf2 + cf5);
        const T res = rhs[q] - gamma * pc - dhx * (phi[q - 1] + phi[q + 1]) - dhy * (phi[q - sx] + phi[q + sx])
                    - dhz * (phi[q - sxy] + phi[q + sxy]);
        phi[q] = pc + omega / g_m_d * res;
    }
}

// y = A x at cell (i,j,k): mlabeclap_adotx (AMReX_MLABecLap_3D_K.H:7-28),
// mlpoisson_adotx (AMReX_MLPoisson_3D_K.H:7-16)
template <typename T, bool ABEC>
__device__ __forceinline__ T adotx_cell (const PatchDesc& P, long long q, const T* __restrict__ x,
                                         const T* __restrict__ a, const T* __restrict__ bx,
                                         const T* __restrict__ by, const T* __restrict__ bz)
{
    const long long sx = P.sx, sxy = P.sxy;
    const T dhx = T(P.dha[0]), dhy = T(P.dha[1]), dhz = T(P.dha[2]);
    const T xc = x[q];
    if constexpr (ABEC) {
        return T(P.alpha) * a[q] * xc
            - dhx * (bx[q + 1] * (x[q + 1] - xc) - bx[q] * (xc - x[q - 1]))
            - dhy * (by[q + sx] * (x[q + sx] - xc) - by[q] * (xc - x[q - sx]))
            - dhz * (bz[q + sxy] * (x[q + sxy] - xc) - bz[q] * (xc - x[q - sxy]));
    } else {
        return dhx * (x[q - 1] - T(2.0) * xc + x[q + 1])
             + dhy * (x[q - sx] - T(2.0) * xc + x[q + sx])
             + dhz * (x[q - sxy] - T(2.0) * xc + x[q + sxy]);
    }
}

// diagonal of the Jacobi-preconditioned BiCGStab: mlabeclap_normalize
// (AMReX_MLABecLap_3D_K.H:58-75); MLPoisson's normalize is a no-op in 3-D
template <typename T>
__device__ __forceinline__ T abec_diag (const PatchDesc& P, long long q, const T* __restrict__ a,
                                        const T* __restrict__ bx, const T* __restrict__ by,
                                        const T* __restrict__ bz)
{
    const T dhx = T(P.dha[0]), dhy = T(P.dha[1]), dhz = T(P.dha[2]);
    return T(P.alpha) * a[q] + dhx * (bx[q] + bx[q + 1]) + dhy * (by[q] + by[q + P.sx])
         + dhz * (bz[q] + bz[q + P.sxy]);
}

// Ghost value of boundary-face cell (i,j,k) of face f (mllinop_apply_bc_*,
// AMReX_MLLinOp_K.H:74-320); `s` steps from the ghost into the patch.
template <typename T>
__device__ __forceinline__ void bc_ghost (const PatchDesc& P, int f, long long qg, long long step, T* phi,
                                          int inhomog, const double* bcval, long long bq)
{
    const FaceBC& F = P.face[f];
    if (F.type == BC_NEUMANN) {
        phi[qg] = phi[qg + step];
    } else if (F.type == BC_REFLECT_ODD) {
        phi[qg] = -phi[qg + step];
    } else if (F.type == BC_DIRICHLET) {
        T tmp = T(0.0);
        for (int m = 1; m < F.nx; ++m) { tmp += phi[qg + m * step] * T(F.coef[m]); }
        phi[qg] = tmp;
        if (inhomog && bcval != nullptr && F.bcval_off >= 0) {
            phi[qg] += T(bcval[F.bcval_off + bq]) * T(F.coef[0]);
        }
    }
}

} // namespace mlmg
