// Fused two-colour red-black Gauss-Seidel sweep (FP32, stencil form).
//
// One launch performs both colour passes of MLCellLinOpT::smooth
// (AMReX_MLCellLinOp.H:1204-1217) with the arithmetic of abec_gsrb /
// mlpoisson_gsrb, reading each array from HBM about once: ~7 words per cell
// per sweep instead of 7 words per colour pass.
//
// Out of place (phi_in -> phi_out), so no block reads another block's output.
// A block owns a FS_TX x FS_TY x FS_TZ tile.  It stages phi_in on the tile
// grown by two cells into shared memory with 16-byte cp.async copies issued
// all at once (rows start 16-byte aligned: x from x0-4), waits once, computes
// the first colour on the tile grown by one cell (this redundant halo makes
// the second colour self-contained), then the second colour on the tile, and
// writes both colours.  Ghost values at patch faces are computed inline from
// the two cells next to the face (Dirichlet closure of at most 3 points,
// Neumann, reflect_odd): for the first colour from phi_in, for the second from
// the first colour's new values -- what applyBC would store before each pass.
// The patch's fields live in shared memory for the whole block, so stores to
// phi_out cannot force the compiler to reload them.
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

// one Gauss-Seidel update from the six neighbour values (ghosts already substituted)
template <bool VARC>
__device__ __forceinline__ float gs_update (const PatchLite& P, const StencilPtrs& Sc, const float* __restrict__ rhs,
                                            long long q, int i, int j, int k, float pc, float xm, float xp, float ym,
                                            float yp, float zm, float zp)
{
    float d, sxl, sxh, syl, syh, szl, szh;
    if constexpr (VARC) {
        const float* D = static_cast<const float*>(Sc.D);
        const float* sx = static_cast<const float*>(Sc.sx);
        const float* sy = static_cast<const float*>(Sc.sy);
        const float* sz = static_cast<const float*>(Sc.sz);
        d = __ldg(D + q);
        sxl = __ldg(sx + q); sxh = __ldg(sx + q + 1);
        syl = __ldg(sy + q); syh = __ldg(sy + q + P.sx);
        szl = __ldg(sz + q); szh = __ldg(sz + q + P.sxy);
    } else {
        d = -2.0f * (P.dhx + P.dhy + P.dhz);
        sxl = sxh = -P.dhx; syl = syh = -P.dhy; szl = szh = -P.dhz;
    }
    float corr = 0;
    if (i == P.lo[0]) { corr += sxl * P.f[0].fco; }
    if (i == P.hi[0]) { corr += sxh * P.f[3].fco; }
    if (j == P.lo[1]) { corr += syl * P.f[1].fco; }
    if (j == P.hi[1]) { corr += syh * P.f[4].fco; }
    if (k == P.lo[2]) { corr += szl * P.f[2].fco; }
    if (k == P.hi[2]) { corr += szh * P.f[5].fco; }
    const float gmd = d - corr;
    const float rho = sxl * xm + sxh * xp + syl * ym + syh * yp + szl * zm + szh * zp;
    const float res = __ldg(rhs + q) - (d * pc - rho);
    return pc + relax_factor(gmd) * res;
}

template <bool VARC>
__global__ void __launch_bounds__(FS_THREADS)
k_sweep_fused (DevLevel L, Subset S, const float* __restrict__ phi_in, float* __restrict__ phi_out,
               const float* __restrict__ rhs, StencilPtrs Sc)
{
    __shared__ __align__(16) float A[FS_AZ][FS_AY][FS_AX];   // phi_in, tile + 2 (x: tile + 4 | + 4)
    __shared__ float N[FS_NZ][FS_NY][FS_NX];                  // first colour's new values, tile + 1
    __shared__ PatchLite SP;

    const int tid = threadIdx.y * FS_TX + threadIdx.x;
    int x0, y0, z0;
    {
        const TileCoord c = decode_fused_tile(L, S, blockIdx.x);
        x0 = c.x0; y0 = c.y0; z0 = c.z0;
        if (tid == 0) {
            const PatchDesc& P = L.P[c.p];
            for (int d = 0; d < 3; ++d) { SP.lo[d] = P.lo[d]; SP.hi[d] = P.hi[d]; }
            SP.sx = P.sx; SP.sxy = P.sxy; SP.base = P.base;
            SP.dhx = float(P.dha[0]); SP.dhy = float(P.dha[1]); SP.dhz = float(P.dha[2]);
            for (int f = 0; f < 6; ++f) {
                SP.f[f].type = P.face[f].type;
                SP.f[f].nx = P.face[f].nx;
                SP.f[f].c1 = float(P.face[f].coef[1]);
                SP.f[f].c2 = float(P.face[f].coef[2]);
                SP.f[f].fco = float(P.face[f].fco);
            }
        }
    }
    __syncthreads();
    const PatchLite& P = SP;

    // ---- stage phi_in: rows of (z, y) in the tile + 2, 16-byte chunks of x
    constexpr int CH = FS_AX / 4;
    for (int u = tid; u < FS_AZ * FS_AY * CH; u += FS_THREADS) {
        const int ch = u % CH, row = u / CH;
        const int ly = row % FS_AY, lz = row / FS_AY;
        const int j = y0 - 2 + ly, k = z0 - 2 + lz, i = x0 - 4 + 4 * ch;
        float* dst = &A[lz][ly][4 * ch];
        const bool row_ok = j >= P.lo[1] && j <= P.hi[1] && k >= P.lo[2] && k <= P.hi[2];
        const bool x_ok = (i + 3 >= P.lo[0]) && (i <= P.hi[0]);
        if (row_ok && x_ok) {
            cp_async16(dst, phi_in + P.idx(i, j, k));
        } else {
            *reinterpret_cast<float4*>(dst) = make_float4(0.f, 0.f, 0.f, 0.f);
        }
    }
    cp_async_wait_all();
    __syncthreads();

    // ---- interior tiles: the tile + 1 touches no patch face, so no closure,
    // no boundary correction and no bounds checks; offsets are 32-bit from the
    // tile's first cell
    const bool interior = (x0 - 1 > P.lo[0]) && (x0 + FS_TX < P.hi[0]) && (y0 - 1 > P.lo[1]) &&
                          (y0 + FS_TY < P.hi[1]) && (z0 - 1 > P.lo[2]) && (z0 + FS_TZ < P.hi[2]);
    if (interior) {
        const long long q0 = P.idx(x0, y0, z0);
        const int sx = P.sx, sxy = (int)P.sxy;
        const float* __restrict__ rh = rhs + q0;
        const float *Dp = nullptr, *SXp = nullptr, *SYp = nullptr, *SZp = nullptr;
        if constexpr (VARC) {
            Dp = static_cast<const float*>(Sc.D) + q0;
            SXp = static_cast<const float*>(Sc.sx) + q0;
            SYp = static_cast<const float*>(Sc.sy) + q0;
            SZp = static_cast<const float*>(Sc.sz) + q0;
        }
        const float cdx = -P.dhx, cdy = -P.dhy, cdz = -P.dhz, cd = -2.0f * (P.dhx + P.dhy + P.dhz);
        auto update = [&] (int o, float pc, float xm, float xp, float ym, float yp, float zm, float zp) {
            float d, sxl, sxh, syl, syh, szl, szh;
            if constexpr (VARC) {
                d = __ldg(Dp + o);
                sxl = __ldg(SXp + o); sxh = __ldg(SXp + o + 1);
                syl = __ldg(SYp + o); syh = __ldg(SYp + o + sx);
                szl = __ldg(SZp + o); szh = __ldg(SZp + o + sxy);
            } else {
                d = cd; sxl = sxh = cdx; syl = syh = cdy; szl = szh = cdz;
            }
            const float rho = sxl * xm + sxh * xp + syl * ym + syh * yp + szl * zm + szh * zp;
            const float res = __ldg(rh + o) - (d * pc - rho);
            return pc + relax_factor(d) * res;
        };
        for (int u = tid; u < FS_NZ * FS_NY * FS_RED_ROW; u += FS_THREADS) {
            const int r = u % FS_RED_ROW, row = u / FS_RED_ROW;
            const int ly = row % FS_NY, lz = row / FS_NY;
            const int lx = 2 * r + ((x0 - 1 + y0 - 1 + ly + z0 - 1 + lz) & 1);
            const int ax = lx + 3, ay = ly + 1, az = lz + 1;
            const int o = (lz - 1) * sxy + (ly - 1) * sx + (lx - 1);     // offset from (x0, y0, z0)
            N[lz][ly][lx] = update(o, A[az][ay][ax], A[az][ay][ax - 1], A[az][ay][ax + 1], A[az][ay - 1][ax],
                                   A[az][ay + 1][ax], A[az - 1][ay][ax], A[az + 1][ay][ax]);
        }
        __syncthreads();
        // every lane takes cells of one colour, so warps do not diverge: the
        // tile holds FS_TX/2 cells of each colour per row
        constexpr int HALF = FS_TX / 2;
        constexpr int PER_PLANE = HALF * FS_TY;
#pragma unroll
        for (int u = tid; u < PER_PLANE * FS_TZ; u += FS_THREADS) {
            const int r = u % HALF, row = u / HALF;
            const int ty = row % FS_TY, lz0 = row / FS_TY;
            const int par = (x0 + y0 + ty + z0 + lz0) & 1;          // parity of (i+j+k) at tx = 0
            const int tx2 = 2 * r + (par ^ 1);                      // second colour: (i+j+k) odd
            const int tx1 = 2 * r + par;                            // first colour: (i+j+k) even
            const int lz = lz0 + 1, ly = ty + 1, az = lz + 1, ay = ly + 1;
            const int base = lz0 * sxy + ty * sx;
            {
                const int lx = tx2 + 1, ax = lx + 3;
                phi_out[q0 + base + tx2] =
                    update(base + tx2, A[az][ay][ax], N[lz][ly][lx - 1], N[lz][ly][lx + 1], N[lz][ly - 1][lx],
                           N[lz][ly + 1][lx], N[lz - 1][ly][lx], N[lz + 1][ly][lx]);
            }
            phi_out[q0 + base + tx1] = N[lz][ly][tx1 + 1];
        }
        return;
    }

    // ---- first colour ((i+j+k) even) on tile + 1
    for (int u = tid; u < FS_NZ * FS_NY * FS_RED_ROW; u += FS_THREADS) {
        const int r = u % FS_RED_ROW, row = u / FS_RED_ROW;
        const int ly = row % FS_NY, lz = row / FS_NY;
        const int j = y0 - 1 + ly, k = z0 - 1 + lz;
        // x of the r-th first-colour cell of this row: x0-1+lx with (x0-1+lx+j+k) even
        const int lx = 2 * r + ((x0 - 1 + j + k) & 1);
        const int i = x0 - 1 + lx;
        if (!P.inside(i, j, k)) { continue; }
        const int ax = lx + 3, ay = ly + 1, az = lz + 1;
        const float pc = A[az][ay][ax];
        const float xm = (i == P.lo[0]) ? P.closure(0, pc, A[az][ay][ax + 1]) : A[az][ay][ax - 1];
        const float xp = (i == P.hi[0]) ? P.closure(3, pc, A[az][ay][ax - 1]) : A[az][ay][ax + 1];
        const float ym = (j == P.lo[1]) ? P.closure(1, pc, A[az][ay + 1][ax]) : A[az][ay - 1][ax];
        const float yp = (j == P.hi[1]) ? P.closure(4, pc, A[az][ay - 1][ax]) : A[az][ay + 1][ax];
        const float zm = (k == P.lo[2]) ? P.closure(2, pc, A[az + 1][ay][ax]) : A[az - 1][ay][ax];
        const float zp = (k == P.hi[2]) ? P.closure(5, pc, A[az - 1][ay][ax]) : A[az + 1][ay][ax];
        N[lz][ly][lx] = gs_update<VARC>(P, Sc, rhs, P.idx(i, j, k), i, j, k, pc, xm, xp, ym, yp, zm, zp);
    }
    __syncthreads();

    // ---- second colour ((i+j+k) odd) on the tile; write both colours.
    // Second-colour cells read their own old value from A and their
    // (first-colour) neighbours' new values from N.
    const int i = x0 + threadIdx.x, j = y0 + threadIdx.y;
    const int lx = threadIdx.x + 1, ly = threadIdx.y + 1;
    const int ax = lx + 3, ay = ly + 1;
#pragma unroll 2
    for (int lz0 = 0; lz0 < FS_TZ; ++lz0) {
        const int k = z0 + lz0, lz = lz0 + 1, az = lz + 1;
        if (!P.inside(i, j, k)) { continue; }
        const long long q = P.idx(i, j, k);
        float out;
        if (((i + j + k) & 1) == 0) {
            out = N[lz][ly][lx];
        } else {
            const float pc = A[az][ay][ax];
            const float xm = (i == P.lo[0]) ? P.closure(0, pc, N[lz][ly][lx + 1]) : N[lz][ly][lx - 1];
            const float xp = (i == P.hi[0]) ? P.closure(3, pc, N[lz][ly][lx - 1]) : N[lz][ly][lx + 1];
            const float ym = (j == P.lo[1]) ? P.closure(1, pc, N[lz][ly + 1][lx]) : N[lz][ly - 1][lx];
            const float yp = (j == P.hi[1]) ? P.closure(4, pc, N[lz][ly - 1][lx]) : N[lz][ly + 1][lx];
            const float zm = (k == P.lo[2]) ? P.closure(2, pc, N[lz + 1][ly][lx]) : N[lz - 1][ly][lx];
            const float zp = (k == P.hi[2]) ? P.closure(5, pc, N[lz - 1][ly][lx]) : N[lz + 1][ly][lx];
            out = gs_update<VARC>(P, Sc, rhs, q, i, j, k, pc, xm, xp, ym, yp, zm, zp);
        }
        phi_out[q] = out;
    }
}

} // namespace mlmg
