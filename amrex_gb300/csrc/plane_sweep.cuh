// Fused two-colour Gauss-Seidel sweep marching along z with the stencil
// coefficients in registers (FP32, stencil form).
//
// Both colour passes of MLCellLinOpT::smooth (AMReX_MLCellLinOp.H:1204-1217)
// with the arithmetic of abec_gsrb / mlpoisson_gsrb (AMReX_MLABecLap_3D_K.H:
// 208-264, AMReX_MLPoisson_3D_K.H:153-196) and the inline ghost closures of
// applyBC, out of place (phi_in -> phi_out).  The tiled sweep
// (fused_sweep2.cuh) reads each coefficient sector about three times from L2
// (first colour on the tile grown by one, second colour after the lines left
// L1); this form reads each once:
//
// * a block owns a PS_TX x PS_TY column of cells and walks a z-slab of it;
//   thread (m, jj) owns the cell pair (x0+2m, x0+2m+1) of row y0+jj -- one
//   cell of each colour -- in every plane;
// * step t updates the first colour ((i+j+k) even) on plane r = z0-1+t and
//   then the second colour on plane r-1, and writes plane r-1;
// * phi_in arrives plane by plane (72 x 12 floats from (x0-4, y0-2)) by one
//   TMA tensor load per plane into a ring of PS_NR planes, PS_LA planes ahead
//   of the step; first-colour values are written into the ring in place (a
//   first-colour update reads only second-colour cells and its own);
// * each thread loads its pair's rhs, D, sX, sY and sZ for plane r+1 as
//   8-byte pairs while plane r is computed (one plane of loads in flight),
//   uses the first-colour half in step t and keeps the second-colour half in
//   registers for the second colour of that plane in step t+1;
// * the first colour is also computed on the one-cell ring around the column
//   that the second colour reads (rows y0-1 and y0+PS_TY: warps 0 and 1; the
//   first-colour cell of x0-1 / x0+PS_TX in each row: warp 2; their stencils
//   are loaded at the top of the step, ahead of the plane wait), and on one
//   plane below and above the slab.
//
// Cells outside the patch are not updated; their values are replaced, for
// the cells next to a patch face, by the closure of the two cells next to the
// face (what applyBC stores before each colour pass), and those cells take
// the smoother's boundary correction of the diagonal.  Every wait is bounded:
// on expiry the block records ERR_TMA_TIMEOUT, waits (bounded) for the copies
// it issued and leaves.
#pragma once

#include "fused_sweep.cuh"
#include "tma.cuh"

namespace mlmg {

constexpr int PS_TX = 64;                       // column width in x (32 thread pairs)
constexpr int PS_TY = 8;                        // rows of the column
constexpr int PS_THREADS = (PS_TX / 2) * PS_TY;
constexpr int PS_RX = PS_TX + 8;                // staged row: x0-4 .. x0+PS_TX+3 (16-byte chunks)
constexpr int PS_RY = PS_TY + 4;                // staged rows: y0-2 .. y0+PS_TY+1
constexpr int PS_PL = PS_RX * PS_RY;            // floats of one staged plane (a multiple of 32)
constexpr int PS_LA = 2;                        // planes in flight beyond the step's last plane (r+1)
constexpr int PS_NR = PS_LA + 4;                // ring slots: planes r-2 .. r+1 in use, PS_LA landing

inline int plane_tiles_of (const PatchDesc& P, int tz)
{
    const int nx = P.hi[0] - P.lo[0] + 1, ny = P.hi[1] - P.lo[1] + 1, nz = P.hi[2] - P.lo[2] + 1;
    return ((nx + PS_TX - 1) / PS_TX) * ((ny + PS_TY - 1) / PS_TY) * ((nz + tz - 1) / tz);
}

__device__ __forceinline__ TileCoord decode_plane_tile (const DevLevel& L, const Subset& S, int b, int tz)
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
    const int ntx = (P.hi[0] - P.lo[0] + PS_TX) / PS_TX;
    const int nty = (P.hi[1] - P.lo[1] + PS_TY) / PS_TY;
    c.x0 = P.lo[0] + (t % ntx) * PS_TX;
    c.y0 = P.lo[1] + ((t / ntx) % nty) * PS_TY;
    c.z0 = P.lo[2] + (t / (ntx * nty)) * tz;
    return c;
}

// the stencil of one cell: diagonal, right-hand side, the six face coefficients
struct Cell8 {
    float d, rh, sxl, sxh, syl, syh, szl, szh;
};

// the stencil of a cell pair (x, x+1): pairs of D, rhs, sX (plus sX(x+2)),
// sY at rows j and j+1, sZ at planes k and k+1
struct Pair15 {
    float2 d, rh, sx, syl, syh, szl, szh;
    float sx2;
    __device__ __forceinline__ Cell8 cell (int e) const
    {
        Cell8 c;
        c.d = e ? d.y : d.x;
        c.rh = e ? rh.y : rh.x;
        c.sxl = e ? sx.y : sx.x;
        c.sxh = e ? sx2 : sx.y;
        c.syl = e ? syl.y : syl.x;
        c.syh = e ? syh.y : syh.x;
        c.szl = e ? szl.y : szl.x;
        c.szh = e ? szh.y : szh.x;
        return c;
    }
};

// Gauss-Seidel update of one cell from its six neighbours (ghosts already
// substituted), gmd = D less the boundary correction (abec_gsrb's g_m_d)
__device__ __forceinline__ float ps_update (const Cell8& c, float gmd, float pc, float xm, float xp, float ym,
                                            float yp, float zm, float zp)
{
    const float rho = c.sxl * xm + c.sxh * xp + c.syl * ym + c.syh * yp + c.szl * zm + c.szh * zp;
    const float res = c.rh - (c.d * pc - rho);
    return pc + relax_factor(gmd) * res;
}

template <bool VARC>
__global__ void __launch_bounds__(PS_THREADS, 3)
k_sweep_planes (DevLevel L, Subset S, float* __restrict__ phi_out, const float* __restrict__ rhs, StencilPtrs Sc,
                const CUtensorMap* __restrict__ maps, int phi_map, int tz, int* err)
{
    __shared__ __align__(128) float ring[PS_NR * PS_PL];
    __shared__ __align__(8) unsigned long long bars[PS_NR];
    __shared__ PatchLite SP;
    const int lane = threadIdx.x, jj = threadIdx.y;          // pair m = lane, row y0 + jj
    const int tid = jj * (PS_TX / 2) + lane;
    int x0, y0, z0, pid;
    {
        const TileCoord c = decode_plane_tile(L, S, blockIdx.x, tz);
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
            for (int b = 0; b < PS_NR; ++b) { tma::mbar_init(&bars[b], 1); }
        }
    }
    __syncthreads();
    const PatchLite& P = SP;
    const int lo0 = P.lo[0], lo1 = P.lo[1], lo2 = P.lo[2], hi0 = P.hi[0], hi1 = P.hi[1], hi2 = P.hi[2];
    const int ke = min(z0 + tz, hi2 + 1);                    // second-colour planes [z0, ke)
    const int pfirst = z0 - 2, plast = ke + 1;               // staged planes
    const int cx = x0 - lo0 + XOFF - 4;                      // box x coordinate (a multiple of 4 floats)
    const int cy = y0 - lo1 - 1;                             // rows from y0-2 (-1: TMA fills zeros)
    if ((cx & 3) != 0) {
        if (tid == 0) { atomicExch(err, tma::ERR_TMA_ALIGN); }
        return;
    }
    const CUtensorMap* const map = maps + (size_t)pid * 2 + phi_map;
    auto slot = [&] (int p) { return ((p - pfirst) % PS_NR) * PS_PL; };
    auto issue = [&] (int p) {
        unsigned long long* bar = &bars[(p - pfirst) % PS_NR];
        tma::mbar_expect_tx(bar, (unsigned)(PS_PL * sizeof(float)));
        tma::load_3d(ring + slot(p), map, bar, cx, cy, p - lo2 + 1);
    };
    auto wait = [&] (int p, long long limit) {
        const int g = p - pfirst;
        return tma::mbar_wait_bounded(&bars[g % PS_NR], (unsigned)((g / PS_NR) & 1), limit);
    };
    auto drain = [&] (int from, int last) {
        if (tid == 0) { atomicExch(err, tma::ERR_TMA_TIMEOUT); }
        for (int p = from; p <= last; ++p) { wait(p, tma::WAIT_LIMIT); }
    };
    // step r reads planes r-2 .. r+1 and issues plane r+3 into the slot of
    // r-3 (last read in step r-1); the prologue stages z0-2 .. z0+1
    int issued = min(pfirst + PS_LA + 1, plast);
    if (tid == 0) {
        for (int p = pfirst; p <= issued; ++p) { issue(p); }
    }

    // ---- coefficient loads
    const int sx = P.sx;
    const long long sxy = P.sxy;
    const float* const Dg = static_cast<const float*>(Sc.D);
    const float* const SXg = static_cast<const float*>(Sc.sx);
    const float* const SYg = static_cast<const float*>(Sc.sy);
    const float* const SZg = static_cast<const float*>(Sc.sz);
    const float cd = -2.0f * (P.dhx + P.dhy + P.dhz);
    const Cell8 cpois{cd, 0.0f, -P.dhx, -P.dhx, -P.dhy, -P.dhy, -P.dhz, -P.dhz};
    // this thread's pair
    const int i0 = x0 + 2 * lane, j = y0 + jj;
    const bool act = i0 <= hi0 && j <= hi1;
    // pairs that load: also the one after the patch's last cell (its sX is
    // the last cell's high face; the row's ghost column and padding are
    // allocated)
    const bool ld = i0 <= hi0 + 1 && j <= hi1;
    const long long q0 = P.idx(i0, j, 0);                    // plane offsets added per plane
    // called by every lane of the warp (the shuffle); loads where ld
    auto load_pair = [&] (Pair15& c, int k, bool with_szl) {
        const long long q = q0 + (long long)k * sxy;
        if (ld) { c.rh = __ldg(reinterpret_cast<const float2*>(rhs + q)); }
        if constexpr (VARC) {
            if (ld) {
                c.d = __ldg(reinterpret_cast<const float2*>(Dg + q));
                c.sx = __ldg(reinterpret_cast<const float2*>(SXg + q));
                c.syl = __ldg(reinterpret_cast<const float2*>(SYg + q));
                c.syh = __ldg(reinterpret_cast<const float2*>(SYg + q + sx));
                if (with_szl) { c.szl = __ldg(reinterpret_cast<const float2*>(SZg + q)); }
                c.szh = __ldg(reinterpret_cast<const float2*>(SZg + q + sxy));
            }
            c.sx2 = __shfl_down_sync(0xffffffffu, c.sx.x, 1);
            if (lane == 31 && ld) { c.sx2 = __ldg(SXg + q + 2); }
        }
    };
    // halo task: warps 0 / 1 the first-colour cell of each pair of rows y0-1 /
    // y0+PS_TY, warp 2 lanes 0..PS_TY-1 the first-colour cell of x0-1 or
    // x0+PS_TX in row y0+lane
    const int hkind = (jj <= 1) ? 1 : ((jj == 2 && lane < PS_TY) ? 2 : 0);
    const int hj = (hkind == 1) ? (jj == 0 ? y0 - 1 : y0 + PS_TY) : y0 + lane;
    auto halo_cell = [&] (int k, int& hi) {                  // x of the halo task's cell on plane k
        if (hkind == 1) { hi = i0 + (((i0 + hj + k) & 1) ? 1 : 0); }
        else { hi = (((x0 - 1 + hj + k) & 1) == 0) ? x0 - 1 : x0 + PS_TX; }
        return hkind != 0 && hi >= lo0 && hi <= hi0 && hj >= lo1 && hj <= hi1;
    };
    auto load_cell = [&] (Cell8& c, int i, int jc, int k) {
        const long long q = P.idx(i, jc, k);
        c.rh = __ldg(rhs + q);
        if constexpr (VARC) {
            c.d = __ldg(Dg + q);
            c.sxl = __ldg(SXg + q); c.sxh = __ldg(SXg + q + 1);
            c.syl = __ldg(SYg + q); c.syh = __ldg(SYg + q + sx);
            c.szl = __ldg(SZg + q); c.szh = __ldg(SZg + q + sxy);
        } else {
            c.d = cpois.d; c.sxl = cpois.sxl; c.sxh = cpois.sxh; c.syl = cpois.syl; c.syh = cpois.syh;
            c.szl = cpois.szl; c.szh = cpois.szh;
        }
    };

    // the block's patch faces (block-uniform)
    // (x0 - lo0 and y0 - lo1 are multiples of the column's extent, so only the
    // column's first cell can be a low face, but its ring can hold a high one)
    const bool fxl = x0 == lo0, fxh = x0 + PS_TX >= hi0, fyl = y0 == lo1, fyh = y0 + PS_TY >= hi1;
    const float fco0 = P.f[0].fco, fco1 = P.f[1].fco, fco2 = P.f[2].fco;
    const float fco3 = P.f[3].fco, fco4 = P.f[4].fco, fco5 = P.f[5].fco;

    // first cell of the staged plane at (i, jc)
    auto at = [&] (int i, int jc) { return (jc - (y0 - 2)) * PS_RX + (i - (x0 - 4)); };
    // update of cell (i, jc) on plane k (colour c: 0 first, 1 second) with
    // stencil cs, reading the staged planes km / kc / kp; faces of the patch
    // get the closures of the current values and the diagonal correction
    const bool touch = fxl || fxh || fyl || fyh;
    auto relax = [&] (const Cell8& cs, int i, int jc, int k, const float* Xm, const float* Xc, const float* Xp) {
        const int o = at(i, jc);
        const float pc = Xc[o];
        float xm = Xc[o - 1], xp = Xc[o + 1], ym = Xc[o - PS_RX], yp = Xc[o + PS_RX], zm = Xm[o], zp = Xp[o];
        float gmd = cs.d;
        const bool bxl = fxl && i == lo0, bxh = fxh && i == hi0, byl = fyl && jc == lo1, byh = fyh && jc == hi1;
        const bool bzl = k == lo2, bzh = k == hi2;
        if ((touch || bzl || bzh) && (bxl || bxh || byl || byh || bzl || bzh)) {
            float corr = 0.0f;
            if (bxl) { xm = P.closure(0, pc, xp); corr += cs.sxl * fco0; }
            if (bxh) { xp = P.closure(3, pc, xm); corr += cs.sxh * fco3; }
            if (byl) { ym = P.closure(1, pc, yp); corr += cs.syl * fco1; }
            if (byh) { yp = P.closure(4, pc, ym); corr += cs.syh * fco4; }
            if (bzl) { zm = P.closure(2, pc, zp); corr += cs.szl * fco2; }
            if (bzh) { zp = P.closure(5, pc, zm); corr += cs.szh * fco5; }
            gmd = cs.d - corr;
        }
        return ps_update(cs, gmd, pc, xm, xp, ym, yp, zm, zp);
    };

    // ---- prologue: the stencil of plane z0-1, and of the halo cells
    Pair15 cur{}, nxt{};
    Cell8 blk = cpois;                                       // second-colour cell of plane r-1
    {
        const int k = z0 - 1;
        if (k >= lo2 && k <= hi2) { load_pair(cur, k, true); }
    }
    if (__syncthreads_or(!(wait(pfirst, tma::WAIT_LIMIT) && wait(pfirst + 1, tma::WAIT_LIMIT)))) {
        drain(pfirst, issued);
        return;
    }

    for (int r = z0 - 1; r <= ke; ++r) {
        // the halo task's cell on plane r (loaded here, used after the wait)
        const bool rin = r >= lo2 && r <= hi2;
        int hi_cur = 0;
        Cell8 hcur;
        const bool hact = halo_cell(r, hi_cur) && rin;
        if (hact) { load_cell(hcur, hi_cur, hj, r); }
        // plane r+1 staged; the next plane's stencil in flight
        if (__syncthreads_or(!wait(r + 1, tma::WAIT_LIMIT))) { drain(r + 1, issued); return; }
        if (tid == 0 && issued < plast) { issue(++issued); }
        const int kn = r + 1;
        const bool knin = kn >= lo2 && kn <= hi2 && kn <= ke;
        if (knin) {                                          // block-uniform: the whole warp loads
            load_pair(nxt, kn, r < lo2);                     // plane r's high face is kn's low one
            if constexpr (VARC) { if (r >= lo2) { nxt.szl = cur.szh; } }
        }

        float* const Xm = ring + slot(r - 1);
        float* const Xc = ring + slot(r);
        float* const Xp = ring + slot(r + 1);
        // ---- first colour on plane r (the column and its ring)
        const int e = ((i0 + j + r) & 1) ? 1 : 0;           // first-colour cell of the pair: i0 + e
        if (rin) {
            if (act && i0 + e <= hi0) {
                Cell8 cs;
                if constexpr (VARC) { cs = cur.cell(e); } else { cs = cpois; cs.rh = e ? cur.rh.y : cur.rh.x; }
                Xc[at(i0 + e, j)] = relax(cs, i0 + e, j, r, Xm, Xc, Xp);
            }
            if (hact) { Xc[at(hi_cur, hj)] = relax(hcur, hi_cur, hj, r, Xm, Xc, Xp); }
            // the ring slots take TMA writes again after these generic ones
            asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
        }
        __syncthreads();

        // ---- second colour on plane b = r-1 and the output of that plane
        const int b = r - 1;
        if (b >= z0 && b < ke && act) {
            const int eb = ((i0 + j + b) & 1) ? 0 : 1;      // second-colour cell of the pair: i0 + eb
            const float* const Bm = ring + slot(b - 1);
            const float* const Bc = ring + slot(b);
            const float* const Bp = Xc;
            float vb = 0.0f;
            if (i0 + eb <= hi0) { vb = relax(blk, i0 + eb, j, b, Bm, Bc, Bp); }
            const float vr = Bc[at(i0 + (eb ^ 1), j)];
            float* const out = phi_out + q0 + (long long)b * sxy;
            if (i0 + 1 <= hi0) {
                *reinterpret_cast<float2*>(out) = eb ? make_float2(vr, vb) : make_float2(vb, vr);
            } else {
                out[0] = eb ? vr : vb;
            }
        }
        // the second-colour half of plane r's pair, for the next step (the
        // barrier at the top of the next step orders this step's ring reads
        // before the TMA write into the slot of plane r-2)
        if constexpr (VARC) { blk = cur.cell(e ^ 1); } else { blk = cpois; blk.rh = e ? cur.rh.x : cur.rh.y; }
        cur = nxt;
    }
}

} // namespace mlmg
