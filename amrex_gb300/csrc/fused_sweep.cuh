// Fused two-colour red-black Gauss-Seidel sweep (FP32, stencil form).
//
// One launch performs both colour passes of MLCellLinOpT::smooth
// (AMReX_MLCellLinOp.H:1204-1217) with the arithmetic of abec_gsrb /
// mlpoisson_gsrb, reading each array once: ~7 words per cell per sweep
// instead of 7 words per colour pass.
//
// Out of place (phi_in -> phi_out), so no block reads another block's output:
// a block owns a TX x TY column tile and a chunk of CZ planes; it stages
// phi_in on the tile grown by two cells in a 3-plane shared-memory ring,
// computes the first colour on the tile grown by one cell (the redundant halo
// makes the second colour of the tile self-contained), then the second colour
// on the tile one plane behind, and writes both colours of the tile.  Ghost
// values at patch faces are computed inline from the two cells next to the
// face (Dirichlet closure of at most 3 points, Neumann, reflect_odd): for the
// first colour from phi_in, for the second from the first colour's new values
// -- exactly what applyBC would store before each colour pass.
#pragma once

#include "stencil_kernels.cuh"

namespace mlmg {

constexpr int FS_TX = 32;       // output tile (x)
constexpr int FS_TY = 8;        // output tile (y)
constexpr int FS_CZ = 32;       // planes per block
constexpr int FS_THREADS = FS_TX * FS_TY;
constexpr int FS_AX = FS_TX + 4, FS_AY = FS_TY + 4;   // phi_in plane, tile + 2
constexpr int FS_NX = FS_TX + 2, FS_NY = FS_TY + 2;   // first-colour plane, tile + 1

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
    c.z0 = P.lo[2] + (t / (ntx * nty)) * FS_CZ;
    return c;
}

inline int fused_tiles_of (const PatchDesc& P)
{
    const int nx = P.hi[0] - P.lo[0] + 1, ny = P.hi[1] - P.lo[1] + 1, nz = P.hi[2] - P.lo[2] + 1;
    return ((nx + FS_TX - 1) / FS_TX) * ((ny + FS_TY - 1) / FS_TY) * ((nz + FS_CZ - 1) / FS_CZ);
}

// homogeneous inline closure (a correction's BCs are homogeneous)
__device__ __forceinline__ float closure (const PatchDesc& P, int f, float pc, float pin)
{
    return inline_ghost<float, false>(P, f, pc, pin, nullptr, 0);
}

// the smoother's diagonal correction at patch faces (uniform masks > 0), in
// the same order as gsrb_s_cell so both smoothers round alike
template <bool VARC>
__device__ __forceinline__ float face_corr (const PatchDesc& P, const Coef7<float, VARC>& cf, int i, int j, int k)
{
    float corr = 0;
    if (i == P.lo[0]) { corr += cf.sxl * float(P.face[0].fco); }
    if (i == P.hi[0]) { corr += cf.sxh * float(P.face[3].fco); }
    if (j == P.lo[1]) { corr += cf.syl * float(P.face[1].fco); }
    if (j == P.hi[1]) { corr += cf.syh * float(P.face[4].fco); }
    if (k == P.lo[2]) { corr += cf.szl * float(P.face[2].fco); }
    if (k == P.hi[2]) { corr += cf.szh * float(P.face[5].fco); }
    return corr;
}

template <bool VARC>
__global__ void __launch_bounds__(FS_THREADS)
k_sweep_fused (DevLevel L, Subset S, const float* __restrict__ phi_in, float* __restrict__ phi_out,
               const float* __restrict__ rhs, StencilPtrs Sc)
{
    __shared__ float A[3][FS_AY][FS_AX];    // phi_in planes (tile + 2)
    __shared__ float N[3][FS_NY][FS_NX];    // after the first colour (tile + 1)

    const TileCoord c = decode_fused_tile(L, S, blockIdx.x);
    const PatchDesc& P = L.P[c.p];
    const int tid = threadIdx.y * FS_TX + threadIdx.x;
    const int x0 = c.x0, y0 = c.y0, z0 = c.z0;
    const int z1 = min(z0 + FS_CZ, P.hi[2] + 1);          // output planes [z0, z1)
    const float omega = 1.15f;

    auto valid = [&] (int i, int j, int k) {
        return i >= P.lo[0] && i <= P.hi[0] && j >= P.lo[1] && j <= P.hi[1] && k >= P.lo[2] && k <= P.hi[2];
    };
    auto slot = [&] (int k) { return (k - z0 + 3) % 3; };
    auto load_A = [&] (int k) {
        const int s = slot(k);
        for (int u = tid; u < FS_AX * FS_AY; u += FS_THREADS) {
            const int lx = u % FS_AX, ly = u / FS_AX;
            const int i = x0 - 2 + lx, j = y0 - 2 + ly;
            A[s][ly][lx] = valid(i, j, k) ? phi_in[cidx(P, i, j, k)] : 0.0f;
        }
    };

    load_A(z0 - 2);
    load_A(z0 - 1);
    for (int kr = z0 - 1; kr <= z1; ++kr) {
        load_A(kr + 1);
        __syncthreads();
        // ---- first colour on plane kr, tile + 1
        if (kr >= P.lo[2] && kr <= P.hi[2]) {
            const int sm = slot(kr - 1), s0 = slot(kr), sp = slot(kr + 1);
            for (int u = tid; u < FS_NX * FS_NY; u += FS_THREADS) {
                const int lx = u % FS_NX, ly = u / FS_NX;
                const int i = x0 - 1 + lx, j = y0 - 1 + ly, k = kr;
                float out = 0.0f;
                if (valid(i, j, k)) {
                    const float pc = A[s0][ly + 1][lx + 1];
                    if (((i + j + k) & 1) == 0) {
                        const long long q = cidx(P, i, j, k);
                        const float xm = (i == P.lo[0]) ? closure(P, 0, pc, A[s0][ly + 1][lx + 2]) : A[s0][ly + 1][lx];
                        const float xp = (i == P.hi[0]) ? closure(P, 3, pc, A[s0][ly + 1][lx]) : A[s0][ly + 1][lx + 2];
                        const float ym = (j == P.lo[1]) ? closure(P, 1, pc, A[s0][ly + 2][lx + 1]) : A[s0][ly][lx + 1];
                        const float yp = (j == P.hi[1]) ? closure(P, 4, pc, A[s0][ly][lx + 1]) : A[s0][ly + 2][lx + 1];
                        const float zm = (k == P.lo[2]) ? closure(P, 2, pc, A[sp][ly + 1][lx + 1]) : A[sm][ly + 1][lx + 1];
                        const float zp = (k == P.hi[2]) ? closure(P, 5, pc, A[sm][ly + 1][lx + 1]) : A[sp][ly + 1][lx + 1];
                        const Coef7<float, VARC> cf = load_coef<float, VARC>(P, q, Sc);
                        const float gmd = cf.d - face_corr(P, cf, i, j, k);
                        const float rho = cf.sxl * xm + cf.sxh * xp + cf.syl * ym + cf.syh * yp + cf.szl * zm + cf.szh * zp;
                        const float res = rhs[q] - (cf.d * pc - rho);
                        out = pc + omega / gmd * res;
                    } else {
                        out = pc;
                    }
                }
                N[s0][ly][lx] = out;
            }
        }
        __syncthreads();
        // ---- second colour on plane kb = kr - 1, tile
        const int kb = kr - 1;
        if (kb >= z0 && kb < z1) {
            const int i = x0 + threadIdx.x, j = y0 + threadIdx.y, k = kb;
            if (valid(i, j, k)) {
                const int sm = slot(kb - 1), s0 = slot(kb), sp = slot(kb + 1);
                const int lx = threadIdx.x + 1, ly = threadIdx.y + 1;
                const long long q = cidx(P, i, j, k);
                const float pc = N[s0][ly][lx];
                float out = pc;
                if (((i + j + k) & 1) == 1) {
                    const float xm = (i == P.lo[0]) ? closure(P, 0, pc, N[s0][ly][lx + 1]) : N[s0][ly][lx - 1];
                    const float xp = (i == P.hi[0]) ? closure(P, 3, pc, N[s0][ly][lx - 1]) : N[s0][ly][lx + 1];
                    const float ym = (j == P.lo[1]) ? closure(P, 1, pc, N[s0][ly + 1][lx]) : N[s0][ly - 1][lx];
                    const float yp = (j == P.hi[1]) ? closure(P, 4, pc, N[s0][ly - 1][lx]) : N[s0][ly + 1][lx];
                    const float zm = (k == P.lo[2]) ? closure(P, 2, pc, N[sp][ly][lx]) : N[sm][ly][lx];
                    const float zp = (k == P.hi[2]) ? closure(P, 5, pc, N[sm][ly][lx]) : N[sp][ly][lx];
                    const Coef7<float, VARC> cf = load_coef<float, VARC>(P, q, Sc);
                    const float gmd = cf.d - face_corr(P, cf, i, j, k);
                    const float rho = cf.sxl * xm + cf.sxh * xp + cf.syl * ym + cf.syh * yp + cf.szl * zm + cf.szh * zp;
                    const float res = rhs[q] - (cf.d * pc - rho);
                    out = pc + omega / gmd * res;
                }
                phi_out[q] = out;
            }
        }
    }
}

} // namespace mlmg
