// Fused two-colour Gauss-Seidel sweep that marches along z (FP32, stencil form).
//
// The same update as k_sweep_fused2 (both colour passes of
// MLCellLinOpT::smooth, AMReX_MLCellLinOp.H:1204-1217, with the arithmetic of
// abec_gsrb / mlpoisson_gsrb and the inline ghost closures), organised as a
// march instead of independent tiles:
//
// * a block owns an MS_TX x MS_TY column of cells and walks tz planes of
//   it; the first colour is recomputed only on a one-cell ring in x and y and
//   on one plane above and below the chunk, not on a halo around every tile;
// * every array (phi_in, rhs, D, sX, sY, sZ) is staged plane by plane into
//   shared-memory rings, so each value crosses HBM once and the arithmetic
//   reads shared memory;
// * thread (tx, ty) owns the cell pair x0+2tx, x0+2tx+1 of row y0+ty -- one
//   cell of each colour -- and writes it with one 8-byte store.
//
// Step kr of the march computes the first colour ((i+j+k) even) on plane kr
// over the column plus its ring, then the second colour on plane kr-1 from
// the first colour's planes kr-2, kr-1, kr, and writes plane kr-1.  It is an
// autotuner candidate (slower than the tiled sweep on the 256^3 benchmark).
#pragma once

#include "fused_sweep.cuh"
#include "tma.cuh"

namespace mlmg {

constexpr int MS_TX = 64;                  // column width in x (32 thread pairs)
constexpr int MS_TY = 16;                  // rows of the column
constexpr int MS_TZ = 16;                  // default planes per chunk (the slab depth tz is a launch parameter)
constexpr int MS_THREADS = (MS_TX / 2) * MS_TY;
constexpr int MS_RP = MS_TX + 8;           // shared row: x0-4 .. x0+MS_TX+3 (16-byte chunks)
constexpr int MS_CH = MS_RP / 4;           // 16-byte chunks per row
constexpr int MS_XR = MS_TY + 4;           // phi rows: y0-2 .. y0+MS_TY+1
constexpr int MS_CR = MS_TY + 3;           // coefficient rows: y0-1 .. y0+MS_TY+1
constexpr int MS_RR = MS_TY + 2;           // first-colour rows: y0-1 .. y0+MS_TY
constexpr int MS_XS = 4;                   // phi planes kr-1 .. kr+2
constexpr int MS_RS = 3;                   // first-colour planes kr-2 .. kr
constexpr int MS_CS = 3;                   // rhs / D / sX / sY planes kr-1 .. kr+1
constexpr int MS_ZS = 4;                   // sZ planes kr-1 .. kr+2
constexpr int MS_XPLANE = MS_XR * MS_RP;
constexpr int MS_RPLANE = MS_RR * MS_RP;
constexpr int MS_CPLANE = MS_CR * MS_RP;

inline int march_tiles_of (const PatchDesc& P, int tz)
{
    const int nx = P.hi[0] - P.lo[0] + 1, ny = P.hi[1] - P.lo[1] + 1, nz = P.hi[2] - P.lo[2] + 1;
    return ((nx + MS_TX - 1) / MS_TX) * ((ny + MS_TY - 1) / MS_TY) * ((nz + tz - 1) / tz);
}

__device__ __forceinline__ TileCoord decode_march_tile (const DevLevel& L, const Subset& S, int b, int tz)
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
    const int ntx = (P.hi[0] - P.lo[0] + MS_TX) / MS_TX;
    const int nty = (P.hi[1] - P.lo[1] + MS_TY) / MS_TY;
    c.x0 = P.lo[0] + (t % ntx) * MS_TX;
    c.y0 = P.lo[1] + ((t / ntx) % nty) * MS_TY;
    c.z0 = P.lo[2] + (t / (ntx * nty)) * tz;
    return c;
}

__device__ __forceinline__ int ring (int k, int n) { return ((k % n) + n) % n; }

// one Gauss-Seidel update with the boundary correction of the smoother's
// diagonal (abec_gsrb / mlpoisson_gsrb in stencil form)
__device__ __forceinline__ float ms_update (const PatchLite& P, int i, int j, int k, float pc, float xm, float xp,
                                            float ym, float yp, float zm, float zp, float d, float sxl, float sxh,
                                            float syl, float syh, float szl, float szh, float rh)
{
    float corr = 0;
    if (i == P.lo[0]) { corr += sxl * P.f[0].fco; }
    if (i == P.hi[0]) { corr += sxh * P.f[3].fco; }
    if (j == P.lo[1]) { corr += syl * P.f[1].fco; }
    if (j == P.hi[1]) { corr += syh * P.f[4].fco; }
    if (k == P.lo[2]) { corr += szl * P.f[2].fco; }
    if (k == P.hi[2]) { corr += szh * P.f[5].fco; }
    const float gmd = d - corr;
    const float rho = sxl * xm + sxh * xp + syl * ym + syh * yp + szl * zm + szh * zp;
    const float res = rh - (d * pc - rho);
    return pc + relax_factor(gmd) * res;
}

// ---------------------------------------------------------------------------
// Staging by the Tensor Memory Accelerator: each plane of phi_in (72 x 20
// floats from (x0-4, y0-2)) and of rhs, D, sX, sY, sZ (72 x 19 from
// (x0-4, y0-1)) arrives by one cp.async.bulk.tensor.3d
// load of a per-patch tensor map, issued by one thread, MT_LA steps ahead of
// the plane being computed, so that about MT_LA x 33 KB per SM are in flight
// while the block computes.  Group g = {phi plane g+1, rhs/D/sX/sY plane g,
// sZ plane g+1} completes on mbarrier slot (g - ks + 2) mod MT_NB; step kr
// needs groups up to kr.  Box x coordinates are (x0 - lo + 4), a multiple of
// 4 floats (the column width is 64); y and z coordinates may be negative (one
// ghost row / plane below the allocation), which TMA fills with zeros, as it
// fills everything past the tensor's end.  Values staged from outside the
// patch are never read: the colour loops skip cells outside the patch and
// use the inline closures on its faces.  Every wait is bounded: on expiry the
// block records ERR_TMA_TIMEOUT, waits (bounded) for the copies it issued and
// leaves.
constexpr int MT_LA = 2;                   // groups in flight ahead of the step being computed
constexpr int MT_NB = MT_LA + 1;           // mbarrier slots
constexpr int MT_XS = 3 + MT_LA;           // phi planes
constexpr int MT_CS = 2 + MT_LA;           // rhs / D / sX / sY planes
constexpr int MT_ZS = 3 + MT_LA;           // sZ planes
constexpr int MT_XPL = MS_XR * MS_RP;      // 1440 floats = 45 x 128 bytes
constexpr int MT_CPL = 1376;               // MS_CR * MS_RP = 1368 rounded up to 128 bytes
constexpr int MT_RPL = 1312;               // MS_RR * MS_RP = 1296 rounded up to 128 bytes
enum : int { MT_PHI_A = 0, MT_PHI_B = 1, MT_RHS = 2, MT_D = 3, MT_SX = 4, MT_SY = 5, MT_SZ = 6, MT_NMAP = 7 };

constexpr int march_tma_smem_floats (bool varc)
{
    return MT_XS * MT_XPL + MS_RS * MT_RPL + (varc ? 4 : 1) * MT_CS * MT_CPL + (varc ? MT_ZS * MT_CPL : 0);
}

template <bool VARC>
__global__ void __launch_bounds__(MS_THREADS, 1)
k_sweep_march_tma (DevLevel L, Subset S, float* __restrict__ phi_out, const CUtensorMap* __restrict__ maps,
                   int phi_map, int tz, int* err)
{
    extern __shared__ __align__(128) float mt_smem[];
    __shared__ PatchLite SP;
    __shared__ __align__(8) unsigned long long bars[MT_NB];
    constexpr int NC = VARC ? 4 : 1;
    float* const Xs = mt_smem;                                        // [MT_XS][MT_XPL] phi_in
    float* const Rs = Xs + MT_XS * MT_XPL;                            // [MS_RS][MT_RPL] first colour
    float* const Cs = Rs + MS_RS * MT_RPL;                            // [rhs, D, sX, sY][MT_CS][MT_CPL]
    float* const Zs = Cs + NC * MT_CS * MT_CPL;                       // [MT_ZS][MT_CPL] sZ
    const int tid = threadIdx.y * (MS_TX / 2) + threadIdx.x;
    int x0, y0, z0, pid;
    {
        const TileCoord c = decode_march_tile(L, S, blockIdx.x, tz);
        x0 = c.x0; y0 = c.y0; z0 = c.z0; pid = c.p;
        if (tid == 0) {
            const PatchDesc& Q = L.P[c.p];
            for (int d = 0; d < 3; ++d) { SP.lo[d] = Q.lo[d]; SP.hi[d] = Q.hi[d]; }
            SP.sx = Q.sx; SP.sxy = Q.sxy; SP.base = Q.base;
            SP.dhx = float(Q.dha[0]); SP.dhy = float(Q.dha[1]); SP.dhz = float(Q.dha[2]);
            for (int f = 0; f < 6; ++f) {
                SP.f[f].type = Q.face[f].type;
                SP.f[f].nx = Q.face[f].nx;
                SP.f[f].c1 = float(Q.face[f].coef[1]);
                SP.f[f].c2 = float(Q.face[f].coef[2]);
                SP.f[f].fco = float(Q.face[f].fco);
            }
            for (int b = 0; b < MT_NB; ++b) { tma::mbar_init(&bars[b], 1); }
        }
    }
    __syncthreads();
    const PatchLite& P = SP;
    const int lo0 = P.lo[0], lo1 = P.lo[1], lo2 = P.lo[2], hi0 = P.hi[0], hi1 = P.hi[1], hi2 = P.hi[2];
    const int ks = z0, ke = min(z0 + tz, hi2 + 1);                    // output planes [ks, ke)
    const CUtensorMap* const M = maps + (size_t)pid * MT_NMAP;
    const int mx = x0 - lo0 + XOFF - 4;                               // box x coordinate (16-byte aligned)
    const int myx = y0 - lo1 - 1, myc = y0 - lo1;                     // phi rows from y0-2, coefficient rows from y0-1
    if ((mx & 3) != 0) {
        if (tid == 0) { atomicExch(err, tma::ERR_TMA_ALIGN); }
        return;
    }
    constexpr unsigned XB = MS_XR * MS_RP * sizeof(float), CB = MS_CR * MS_RP * sizeof(float);
    // group g (planes as above) on slot (g - ks + 2) % MT_NB; group ks-2 also brings phi plane ks-2
    auto issue = [&] (int g) {
        const int gi = g - (ks - 2);
        unsigned long long* bar = &bars[gi % MT_NB];
        const bool first = gi == 0;
        tma::mbar_expect_tx(bar, XB * (first ? 2u : 1u) + CB * (unsigned)NC + (VARC ? CB : 0u));
        tma::load_3d(Xs + ring(g + 1, MT_XS) * MT_XPL, M + phi_map, bar, mx, myx, g + 1 - lo2 + 1);
        if (first) { tma::load_3d(Xs + ring(g, MT_XS) * MT_XPL, M + phi_map, bar, mx, myx, g - lo2 + 1); }
        const int cs = ring(g, MT_CS) * MT_CPL;
        tma::load_3d(Cs + cs, M + MT_RHS, bar, mx, myc, g - lo2 + 1);
        if constexpr (VARC) {
            tma::load_3d(Cs + 1 * MT_CS * MT_CPL + cs, M + MT_D, bar, mx, myc, g - lo2 + 1);
            tma::load_3d(Cs + 2 * MT_CS * MT_CPL + cs, M + MT_SX, bar, mx, myc, g - lo2 + 1);
            tma::load_3d(Cs + 3 * MT_CS * MT_CPL + cs, M + MT_SY, bar, mx, myc, g - lo2 + 1);
            tma::load_3d(Zs + ring(g + 1, MT_ZS) * MT_CPL, M + MT_SZ, bar, mx, myc, g + 1 - lo2 + 1);
        }
    };
    auto wait = [&] (int g) {
        const int gi = g - (ks - 2);
        return tma::mbar_wait_bounded(&bars[gi % MT_NB], (unsigned)((gi / MT_NB) & 1), tma::WAIT_LIMIT);
    };
    // leave after a timeout once the copies issued (groups up to `last`) have landed
    auto drain = [&] (int from, int last) {
        if (tid == 0) { atomicExch(err, tma::ERR_TMA_TIMEOUT); }
        for (int g = from; g <= last; ++g) { wait(g); }
    };

    // prologue: groups ks-2 .. ks-2+MT_LA (those up to ke)
    if (tid == 0) {
        for (int g = ks - 2; g <= min(ks - 2 + MT_LA, ke); ++g) { issue(g); }
    }
    if (__syncthreads_or(!wait(ks - 2))) { drain(ks - 2, min(ks - 2 + MT_LA, ke)); return; }

    const float cd = -2.0f * (P.dhx + P.dhy + P.dhz);
    constexpr int NRED = (MS_TX + 2) / 2;                             // first-colour cells per ring row
    for (int kr = ks - 1; kr <= ke; ++kr) {
        if (__syncthreads_or(!wait(kr))) { drain(kr, min(kr + MT_LA - 1, ke)); return; }
        if (tid == 0 && kr + MT_LA <= ke) { issue(kr + MT_LA); }

        // ---- first colour ((i+j+k) even) on plane kr, column + ring
        if (kr >= lo2 && kr <= hi2) {
            const float* const Xm = Xs + ring(kr - 1, MT_XS) * MT_XPL;
            const float* const Xc = Xs + ring(kr, MT_XS) * MT_XPL;
            const float* const Xp = Xs + ring(kr + 1, MT_XS) * MT_XPL;
            const int cs = ring(kr, MT_CS) * MT_CPL;
            const float* const Zc = Zs + ring(kr, MT_ZS) * MT_CPL;
            const float* const Zp = Zs + ring(kr + 1, MT_ZS) * MT_CPL;
            float* const Rw = Rs + ring(kr, MS_RS) * MT_RPL;
            for (int u = tid; u < MS_RR * NRED; u += MS_THREADS) {
                const int row = u / NRED, r = u - row * NRED;
                const int j = y0 - 1 + row;
                const int i = x0 - 1 + 2 * r + ((x0 - 1 + j + kr) & 1);
                if (i < lo0 || i > hi0 || j < lo1 || j > hi1) { continue; }
                const int cx = i - (x0 - 4);
                const int xo = (j - (y0 - 2)) * MS_RP + cx;
                const int co = row * MS_RP + cx;
                const float pc = Xc[xo];
                const float xm = (i == lo0) ? P.closure(0, pc, Xc[xo + 1]) : Xc[xo - 1];
                const float xp = (i == hi0) ? P.closure(3, pc, Xc[xo - 1]) : Xc[xo + 1];
                const float ym = (j == lo1) ? P.closure(1, pc, Xc[xo + MS_RP]) : Xc[xo - MS_RP];
                const float yp = (j == hi1) ? P.closure(4, pc, Xc[xo - MS_RP]) : Xc[xo + MS_RP];
                const float zm = (kr == lo2) ? P.closure(2, pc, Xp[xo]) : Xm[xo];
                const float zp = (kr == hi2) ? P.closure(5, pc, Xm[xo]) : Xp[xo];
                float d, sxl, sxh, syl, syh, szl, szh;
                if constexpr (VARC) {
                    d = Cs[1 * MT_CS * MT_CPL + cs + co];
                    sxl = Cs[2 * MT_CS * MT_CPL + cs + co]; sxh = Cs[2 * MT_CS * MT_CPL + cs + co + 1];
                    syl = Cs[3 * MT_CS * MT_CPL + cs + co]; syh = Cs[3 * MT_CS * MT_CPL + cs + co + MS_RP];
                    szl = Zc[co]; szh = Zp[co];
                } else {
                    d = cd; sxl = sxh = -P.dhx; syl = syh = -P.dhy; szl = szh = -P.dhz;
                }
                Rw[co] = ms_update(P, i, j, kr, pc, xm, xp, ym, yp, zm, zp, d, sxl, sxh, syl, syh, szl, szh,
                                   Cs[cs + co]);
            }
        }
        __syncthreads();

        // ---- second colour on plane kb = kr-1 and the output of that plane
        const int kb = kr - 1;
        if (kb >= ks && kb < ke) {
            const int j = y0 + threadIdx.y;
            const int i0 = x0 + 2 * threadIdx.x;
            if (j <= hi1 && i0 <= hi0) {
                const bool red0 = ((i0 + j + kb) & 1) == 0;
                const int ib = red0 ? i0 + 1 : i0;
                const int ir = red0 ? i0 : i0 + 1;
                const int row = j - (y0 - 1);
                const float* const Rc = Rs + ring(kb, MS_RS) * MT_RPL + row * MS_RP;
                float vb = 0.0f;
                if (ib <= hi0) {
                    const int cx = ib - (x0 - 4);
                    const int co = row * MS_RP + cx;
                    const float pc = Xs[ring(kb, MT_XS) * MT_XPL + (j - (y0 - 2)) * MS_RP + cx];
                    const float* const R0 = Rc + cx;
                    const float xm = (ib == lo0) ? P.closure(0, pc, R0[1]) : R0[-1];
                    const float xp = (ib == hi0) ? P.closure(3, pc, R0[-1]) : R0[1];
                    const float ym = (j == lo1) ? P.closure(1, pc, R0[MS_RP]) : R0[-MS_RP];
                    const float yp = (j == hi1) ? P.closure(4, pc, R0[-MS_RP]) : R0[MS_RP];
                    const float rm = Rs[ring(kb - 1, MS_RS) * MT_RPL + co];
                    const float rp = Rs[ring(kb + 1, MS_RS) * MT_RPL + co];
                    const float zm = (kb == lo2) ? P.closure(2, pc, rp) : rm;
                    const float zp = (kb == hi2) ? P.closure(5, pc, rm) : rp;
                    const int cs = ring(kb, MT_CS) * MT_CPL;
                    float d, sxl, sxh, syl, syh, szl, szh;
                    if constexpr (VARC) {
                        d = Cs[1 * MT_CS * MT_CPL + cs + co];
                        sxl = Cs[2 * MT_CS * MT_CPL + cs + co]; sxh = Cs[2 * MT_CS * MT_CPL + cs + co + 1];
                        syl = Cs[3 * MT_CS * MT_CPL + cs + co]; syh = Cs[3 * MT_CS * MT_CPL + cs + co + MS_RP];
                        szl = Zs[ring(kb, MT_ZS) * MT_CPL + co]; szh = Zs[ring(kb + 1, MT_ZS) * MT_CPL + co];
                    } else {
                        d = cd; sxl = sxh = -P.dhx; syl = syh = -P.dhy; szl = szh = -P.dhz;
                    }
                    vb = ms_update(P, ib, j, kb, pc, xm, xp, ym, yp, zm, zp, d, sxl, sxh, syl, syh, szl, szh,
                                   Cs[cs + co]);
                }
                const float vr = Rc[ir - (x0 - 4)];
                float* const out = phi_out + P.idx(i0, j, kb);
                if (i0 + 1 <= hi0) {
                    *reinterpret_cast<float2*>(out) = red0 ? make_float2(vr, vb) : make_float2(vb, vr);
                } else {
                    out[0] = red0 ? vr : vb;
                }
            }
        }
    }
}

} // namespace mlmg
