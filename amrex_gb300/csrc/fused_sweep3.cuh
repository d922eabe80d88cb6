// Fused two-colour Gauss-Seidel sweep, third form: every input of a tile in
// shared memory.
//
// k_sweep_fused2 keeps phi in shared memory but reads the stencil arrays (D,
// sX, sY, sZ) and the right-hand side from global memory, cell by cell: each
// value is used by about one update per colour pass, so those loads mostly
// miss L1 and the kernel waits on L2.  Here one block stages, with six TMA
// tensor loads completing on one mbarrier,
//   phi_in on the tile grown by two cells   (40 x 12 x 12 floats, x from x0-4)
//   D, rhs, sX on the tile grown by one     (40 x 10 x 10, x from x0-4)
//   sY on the tile + 1 and one more row     (40 x 11 x 10)
//   sZ on the tile + 1 and one more plane   (40 x 10 x 11)
// and then runs both colours from shared memory.  The colours update phi in
// place in shared memory (a first-colour update reads only second-colour
// cells, and the reverse), as the reference's in-place smoother does; the
// ghost layers at patch faces are rewritten with the inline closure before
// each colour, as in k_sweep_fused2.  The tile is written out of place with
// 16-byte stores.  About 104 KB of shared memory: two blocks per SM.
//
// Every box's x coordinate is x0 - lo + 4 (a multiple of 4 floats: 16-byte
// aligned); y and z coordinates may be -1 (the loads fill outside the tensor).
// The wait is bounded as in k_sweep_fused2.
#pragma once

#include "fused_sweep2.cuh"

namespace mlmg {

constexpr int fs3_pad (int n) { return (n + 31) / 32 * 32; }   // floats, rounded to 128-byte multiples

// shared-memory plan of the third form (floats; each buffer starts on a
// 128-byte boundary relative to a 128-byte aligned base)
struct Fs3Plan {
    static constexpr int AX = 40;
    static constexpr int A_N = 12 * 12 * AX;          // phi: z -2..9, y -2..9, x -4..35
    static constexpr int C_N = 10 * 10 * AX;          // D, rhs, sX: z -1..8, y -1..8
    static constexpr int SY_N = 10 * 11 * AX;         // sY: z -1..8, y -1..9
    static constexpr int SZ_N = 11 * 10 * AX;         // sZ: z -1..9, y -1..8
    static constexpr int oA = 0;
    static constexpr int oR = oA + fs3_pad(A_N);
    static constexpr int oD = oR + fs3_pad(C_N);          // D, sX, sY, sZ: variable coefficients only
    static constexpr int oSX = oD + fs3_pad(C_N);
    static constexpr int oSY = oSX + fs3_pad(C_N);
    static constexpr int oSZ = oSY + fs3_pad(SY_N);
    static constexpr int total_var = oSZ + fs3_pad(SZ_N);
    static constexpr int total_const = oD;
    // dynamic shared memory of a block: the buffers plus room to align the base to 128 bytes
    static constexpr int bytes (bool varc) { return (varc ? total_var : total_const) * 4 + 128; }
};

// tensor maps of one patch for the third form, in this order
enum : int { F3_PHI_A = 0, F3_PHI_B, F3_RHS, F3_D, F3_SX, F3_SY, F3_SZ, F3_NMAP };

// Both colours and the write of one tile whose inputs sit in shared memory
// at `sm` (Fs3Plan layout), by NT threads that all call it (block barriers
// inside).
template <bool VARC, int NT>
__device__ __forceinline__ void fs3_tile (const PatchLite& P, int x0, int y0, int z0, float* __restrict__ sm,
                                          float* __restrict__ phi_out, int tid)
{
    static_assert(NT % ((FS_TX / 2) * FS_TY) == 0 && NT >= FS_RED_ROW, "thread count");
    using PL = Fs3Plan;
    float* const As = sm + PL::oA;
    float* const Ds = sm + PL::oD;
    float* const Rs = sm + PL::oR;
    float* const SXs = sm + PL::oSX;
    float* const SYs = sm + PL::oSY;
    float* const SZs = sm + PL::oSZ;
    const int pxl = P.lo[0] - x0, pxh = P.hi[0] - x0;
    const int pyl = P.lo[1] - y0, pyh = P.hi[1] - y0;
    const int pzl = P.lo[2] - z0, pzh = P.hi[2] - z0;
    const bool touches = (pxl >= -1) || (pxh <= FS_TX) || (pyl >= -1) || (pyh <= FS_TY) || (pzl >= -1) ||
                         (pzh <= FS_TZ);

    // local (lx, ly, lz) -> shared element
    auto a_at = [&] (int lx, int ly, int lz) -> float& { return As[((lz + 2) * 12 + (ly + 2)) * PL::AX + lx + 4]; };
    auto c_idx = [&] (int lx, int ly, int lz) { return ((lz + 1) * 10 + (ly + 1)) * PL::AX + lx + 4; };
    auto sy_idx = [&] (int lx, int ly, int lz) { return ((lz + 1) * 11 + (ly + 1)) * PL::AX + lx + 4; };

    // ghost layers of the patch faces inside the tile + 1 (as k_sweep_fused2)
    auto for_face_ghosts = [&] (auto&& fn) {
        const int lim[3] = {FS_TX, FS_TY, FS_TZ};
        const int plo[3] = {pxl, pyl, pzl}, phi[3] = {pxh, pyh, pzh};
        for (int f = 0; f < 6; ++f) {
            const int d = f % 3;
            const int g = (f < 3) ? plo[d] - 1 : phi[d] + 1;
            if (g < -1 || g > lim[d]) { continue; }
            const int s = (f < 3) ? 1 : -1;
            const int t1 = (d == 0) ? 1 : 0, t2 = (d == 2) ? 1 : 2;
            const int a1 = max(-1, plo[t1]), b1 = min(lim[t1], phi[t1]);
            const int a2 = max(-1, plo[t2]), b2 = min(lim[t2], phi[t2]);
            const int n1 = b1 - a1 + 1, n2 = b2 - a2 + 1;
            if (n1 <= 0 || n2 <= 0) { continue; }
            for (int u = tid; u < n1 * n2; u += NT) {
                int c[3];
                c[d] = g; c[t1] = a1 + u % n1; c[t2] = a2 + u / n1;
                int cf[3] = {c[0], c[1], c[2]}, ci[3] = {c[0], c[1], c[2]};
                cf[d] += s; ci[d] += 2 * s;
                fn(f, c, cf, ci);
            }
        }
    };
    auto closure_pass = [&] () {
        for_face_ghosts([&] (int f, const int* c, const int* cf, const int* ci) {
            a_at(c[0], c[1], c[2]) = P.closure(f, a_at(cf[0], cf[1], cf[2]), a_at(ci[0], ci[1], ci[2]));
        });
    };

    const float cdx = -P.dhx, cdy = -P.dhy, cdz = -P.dhz, cd = -2.0f * (P.dhx + P.dhy + P.dhz);
    const float fco0 = P.f[0].fco, fco1 = P.f[1].fco, fco2 = P.f[2].fco;
    const float fco3 = P.f[3].fco, fco4 = P.f[4].fco, fco5 = P.f[5].fco;
    // in-place Gauss-Seidel update of local cell (lx, ly, lz), all inputs in shared memory
    auto update = [&] (int lx, int ly, int lz) {
        float* ap = &a_at(lx, ly, lz);
        const int ci = c_idx(lx, ly, lz);
        float d, sxl, sxh, syl, syh, szl, szh;
        if constexpr (VARC) {
            d = Ds[ci];
            sxl = SXs[ci]; sxh = SXs[ci + 1];
            const int yi = sy_idx(lx, ly, lz);
            syl = SYs[yi]; syh = SYs[yi + PL::AX];
            szl = SZs[ci]; szh = SZs[ci + 10 * PL::AX];
        } else {
            d = cd; sxl = sxh = cdx; syl = syh = cdy; szl = szh = cdz;
        }
        float gmd = d;
        if (touches) {
            float corr = 0.0f;
            if (lx == pxl) { corr += sxl * fco0; }
            if (lx == pxh) { corr += sxh * fco3; }
            if (ly == pyl) { corr += syl * fco1; }
            if (ly == pyh) { corr += syh * fco4; }
            if (lz == pzl) { corr += szl * fco2; }
            if (lz == pzh) { corr += szh * fco5; }
            gmd = d - corr;
        }
        constexpr int SY = PL::AX, SZ = 12 * PL::AX;
        const float pc = ap[0];
        const float rho = sxl * ap[-1] + sxh * ap[1] + syl * ap[-SY] + syh * ap[SY] + szl * ap[-SZ] + szh * ap[SZ];
        const float res = Rs[ci] - (d * pc - rho);
        ap[0] = pc + relax_factor(gmd) * res;
    };

    if (touches) { closure_pass(); __syncthreads(); }

    // ---- first colour ((i+j+k) even) on the tile + 1, in place
    {
        constexpr int RS = NT / FS_RED_ROW;              // row streams x 17 columns
        const int par0 = (x0 - 1 + y0 - 1 + z0 - 1) & 1;
        if (tid < RS * FS_RED_ROW) {
            const int r = tid % FS_RED_ROW;
            int ry = (tid / FS_RED_ROW) % FS_NY, rz = (tid / FS_RED_ROW) / FS_NY;
#pragma unroll 2
            for (int row = tid / FS_RED_ROW; row < FS_NZ * FS_NY; row += RS) {
                const int ly = ry - 1, lz = rz - 1;
                const int lx = 2 * r - 1 + ((par0 + ry + rz) & 1);
                const bool in = !touches || (lx >= pxl && lx <= pxh && ly >= pyl && ly <= pyh && lz >= pzl &&
                                             lz <= pzh);
                if (in) { update(lx, ly, lz); }
                ry += RS % FS_NY; rz += RS / FS_NY;
                if (ry >= FS_NY) { ry -= FS_NY; rz += 1; }
            }
        }
    }
    __syncthreads();
    if (touches) { closure_pass(); __syncthreads(); }

    // ---- second colour on the tile, in place: 16 cells per row, 8 x 8 rows
    {
        constexpr int ZST = NT / ((FS_TX / 2) * FS_TY);   // z streams
        const int r = tid % (FS_TX / 2);
        const int ly = (tid / (FS_TX / 2)) % FS_TY;
        const int lzs = (tid / (FS_TX / 2)) / FS_TY;
        const int par0 = (x0 + y0 + z0) & 1;
#pragma unroll
        for (int lz = lzs; lz < FS_TZ; lz += ZST) {
            const int lx = 2 * r + (((par0 + ly + lz) & 1) ^ 1);   // (x+y+z) odd
            const bool in = !touches || (lx <= pxh && ly <= pyh && lz <= pzh);
            if (in) { update(lx, ly, lz); }
        }
    }
    __syncthreads();

    // ---- write the tile: 8 x 8 rows of 8 float4
    {
        const long long q0 = P.idx(x0, y0, z0);
        const int sx = P.sx, sxy = (int)P.sxy;
        const bool full = !touches || (pxh >= FS_TX - 1 && pyh >= FS_TY - 1 && pzh >= FS_TZ - 1);
        for (int u = tid; u < FS_TZ * FS_TY * (FS_TX / 4); u += NT) {
            const int c4 = u % (FS_TX / 4), row = u / (FS_TX / 4);
            const int ly = row % FS_TY, lz = row / FS_TY;
            const float* src = &a_at(4 * c4, ly, lz);
            float* dst = phi_out + q0 + (long long)(lz * sxy + ly * sx + 4 * c4);
            if (full) {
                *reinterpret_cast<float4*>(dst) = *reinterpret_cast<const float4*>(src);
            } else if (ly <= pyh && lz <= pzh) {
                for (int e = 0; e < 4; ++e) { if (4 * c4 + e <= pxh) { dst[e] = src[e]; } }
            }
        }
    }
}

template <bool VARC>
__global__ void __launch_bounds__(FS_THREADS, 2)
k_sweep_fused3 (DevLevel L, Subset S, const float* __restrict__ phi_in, float* __restrict__ phi_out,
                StencilPtrs Sc, const CUtensorMap* __restrict__ maps, int phi_map, int* err)
{
    extern __shared__ unsigned char fs3_raw[];
    __shared__ PatchLite SP;
    __shared__ unsigned long long bar;
    using PL = Fs3Plan;
    float* const sm = reinterpret_cast<float*>((reinterpret_cast<size_t>(fs3_raw) + 127) & ~size_t(127));
    float* const As = sm + PL::oA;
    float* const Ds = sm + PL::oD;
    float* const Rs = sm + PL::oR;
    float* const SXs = sm + PL::oSX;
    float* const SYs = sm + PL::oSY;
    float* const SZs = sm + PL::oSZ;

    const int tid = threadIdx.y * FS_TX + threadIdx.x;
    int x0, y0, z0, pid;
    {
        const TileCoord c = decode_fused_tile(L, S, blockIdx.x);
        x0 = c.x0; y0 = c.y0; z0 = c.z0; pid = c.p;
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
            tma::mbar_init(&bar, 1);
        }
    }
    __syncthreads();
    const PatchLite& P = SP;

    // ---- stage every input with TMA
    {
        const int cx = x0 - P.lo[0] + XOFF - 4;                 // tensor x of local x = -4
        const int cy1 = y0 - P.lo[1], cz1 = z0 - P.lo[2];       // tensor y, z of local -1
        if ((cx & 3) != 0) {
            if (tid == 0) { atomicExch(err, tma::ERR_TMA_ALIGN); }
            return;
        }
        if (tid == 0) {
            const CUtensorMap* M = maps + (size_t)pid * F3_NMAP;
            unsigned bytes = (unsigned)(PL::A_N + PL::C_N) * 4u;
            if constexpr (VARC) { bytes += (unsigned)(2 * PL::C_N + PL::SY_N + PL::SZ_N) * 4u; }
            tma::mbar_expect_tx(&bar, bytes);
            tma::load_3d(As, M + phi_map, &bar, cx, cy1 - 1, cz1 - 1);
            tma::load_3d(Rs, M + F3_RHS, &bar, cx, cy1, cz1);
            if constexpr (VARC) {
                tma::load_3d(Ds, M + F3_D, &bar, cx, cy1, cz1);
                tma::load_3d(SXs, M + F3_SX, &bar, cx, cy1, cz1);
                tma::load_3d(SYs, M + F3_SY, &bar, cx, cy1, cz1);
                tma::load_3d(SZs, M + F3_SZ, &bar, cx, cy1, cz1);
            }
        }
        const bool late = !tma::mbar_wait_bounded(&bar, 0, tma::WAIT_LIMIT);
        if (__syncthreads_or(late)) {
            if (tid == 0) { atomicExch(err, tma::ERR_TMA_TIMEOUT); }
            tma::mbar_wait_bounded(&bar, 0, tma::WAIT_LIMIT);
            return;
        }
    }

    fs3_tile<VARC, FS_THREADS>(P, x0, y0, z0, sm, phi_out, tid);
}

} // namespace mlmg
