// Fused two-colour Gauss-Seidel sweep on 32x8x8 tiles: one code path for
// every tile, little integer work per cell.
//
// phi_in on the 32x8x8 tile grown by two cells in shared memory (A), the
// first colour ((i+j+k) even) on the tile grown by one (N), the second colour
// on the tile, both written out of place.  Measured choices:
//
// * Patch faces are handled by rewriting ghost values in shared memory
//   instead of testing every cell: after staging, the ghost layer next to each
//   patch face inside the tile gets the closure of the two cells next to the
//   face (what applyBC stores before the first colour pass); after the first
//   colour, the same layer of N gets the closure of the current values (what
//   applyBC stores before the second pass: new first-colour values, old
//   second-colour values).  Both colour loops then read neighbours without
//   branches.  Cells of the tile + 1 outside the patch are not updated.
// * Tiles that touch no patch face (block-uniform flag) skip the inside test
//   and the smoother's boundary correction, which every other tile evaluates
//   with six register comparisons in tile-local coordinates.
// * Thread -> cell maps advance incrementally (no division per cell); global
//   offsets are 32-bit from the tile's first cell; each thread writes one
//   8-byte pair (one cell of each colour).
#pragma once

#include "fused_sweep.cuh"
#include "tma.cuh"

namespace mlmg {

//
// With TMA, phi_in is staged by one Tensor Memory Accelerator load per tile
// (cp.async.bulk.tensor.3d) instead of 16-byte cp.async copies: a 3-D tensor
// map over the patch's allocation (x with its row padding, y and z with their
// ghost layers) delivers the 40 x 12 x 12 box into A and signals an mbarrier.
// The box's x coordinate (x0 - lo + 4) is a multiple of 4 floats, so the copy
// starts on a 16-byte boundary (checked; a violation is reported in *err and
// the copy is not issued).  Cells of the box outside the patch hold whatever
// the allocation holds there (zero past its end): the sweep reads them only
// through the ghost layers it rewrites.  The wait is bounded (first_wait
// polls); on expiry the block reports ERR_TMA_TIMEOUT, waits once more, with
// the full bound, for its own copy so that no copy outlives the block, and
// leaves.
//
// With `pf` (FS_PF_NMAP maps per patch over rhs, D, sX, sY, sZ), the block
// also asks the TMA unit to prefetch into L2 the boxes of those arrays that
// its colour passes read (the tile grown by one, x widened to the 16-byte
// aligned 40 columns of the phi box), so that their per-thread loads, issued
// once phi has arrived, find the lines in L2 rather than in DRAM.
enum : int { FS_PF_RHS = 0, FS_PF_D = 1, FS_PF_SX = 2, FS_PF_SY = 3, FS_PF_SZ = 4, FS_PF_NMAP = 5 };

// The first colour skips the cells of the tile + 1 with two or three
// coordinates outside the tile (its edges and corners): no second-colour cell
// of the tile has them as neighbours, so the tile's output is unchanged and
// their coefficient sectors are not loaded.
template <bool VARC, bool TMA = false>
__global__ void __launch_bounds__(FS_THREADS, 5)
k_sweep_fused2 (DevLevel L, Subset S, const float* __restrict__ phi_in, float* __restrict__ phi_out,
                const float* __restrict__ rhs, StencilPtrs Sc, const CUtensorMap* __restrict__ maps, int* err,
                long long first_wait, const CUtensorMap* __restrict__ pf = nullptr, int zero_in = 0,
                const int4* __restrict__ tiles = nullptr)
{
    __shared__ __align__(128) float A[FS_AZ][FS_AY][FS_AX];   // phi_in, local (x-4..x+35, y-2..y+9, z-2..z+9)
    __shared__ float N[FS_NZ][FS_NY][FS_NX];                    // first colour, local (x-1..x+32, y-1..y+8, z-1..z+8)
    __shared__ PatchLite SP;

    const int tid = threadIdx.y * FS_TX + threadIdx.x;
    int x0, y0, z0, pid;
    {
        // the tile: from the level's tile map, or (an AMR fine level) from a
        // list of the tiles whose halo meets no face shared with another patch
        const TileCoord c = (tiles != nullptr)
            ? TileCoord{tiles[blockIdx.x].x, tiles[blockIdx.x].y, tiles[blockIdx.x].z, tiles[blockIdx.x].w}
            : decode_fused_tile(L, S, blockIdx.x);
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
        }
    }
    __syncthreads();
    pdl_wait();
    pdl_trigger();
    const PatchLite& P = SP;
    // patch bounds in tile-local coordinates (lo <= 0 since tiles start inside the patch)
    const int pxl = P.lo[0] - x0, pxh = P.hi[0] - x0;
    const int pyl = P.lo[1] - y0, pyh = P.hi[1] - y0;
    const int pzl = P.lo[2] - z0, pzh = P.hi[2] - z0;
    // the tile + 1 holds a face cell of the patch (or reaches past it)
    const bool touches = (pxl >= -1) || (pxh <= FS_TX) || (pyl >= -1) || (pyh <= FS_TY) || (pzl >= -1) ||
                         (pzh <= FS_TZ);

    if constexpr (TMA) {
        __shared__ unsigned long long bar;
        const int cx = x0 - P.lo[0] + XOFF - 4, cy = y0 - P.lo[1] - 1, cz = z0 - P.lo[2] - 1;
        const bool aligned = (cx & 3) == 0;
        if (tid == 0) { tma::mbar_init(&bar, 1); }
        __syncthreads();
        if (!aligned) {
            if (tid == 0) { atomicExch(err, tma::ERR_TMA_ALIGN); }
            return;
        }
        if (tid == 0 && !zero_in) {
            tma::mbar_expect_tx(&bar, (unsigned)sizeof(A));
            tma::load_3d(&A[0][0][0], maps + pid, &bar, cx, cy, cz);
        }
        if (pf != nullptr && tid >= 32 && tid < 32 + (VARC ? FS_PF_NMAP : 1)) {
            // coordinates of the tile grown by one: never negative
            tma::prefetch_3d(pf + (size_t)pid * FS_PF_NMAP + (tid - 32), cx, cy + 1, cz + 1);
        }
        if (zero_in) {
            // the first sweep of a V-cycle level starts from a zero correction
            float* a = &A[0][0][0];
            for (int u = tid; u < FS_AZ * FS_AY * FS_AX; u += FS_THREADS) { a[u] = 0.f; }
            __syncthreads();
        } else {
            const bool late = !tma::mbar_wait_bounded(&bar, 0, first_wait);
            if (__syncthreads_or(late)) {
                if (tid == 0) { atomicExch(err, tma::ERR_TMA_TIMEOUT); }
                tma::mbar_wait_bounded(&bar, 0, tma::WAIT_LIMIT);
                return;
            }
        }
    } else {
    // ---- stage phi_in: 12 x 12 rows of 10 16-byte chunks; 250 threads, (ly, lz) advanced incrementally
    constexpr int CH = FS_AX / 4;                    // 10
    constexpr int RSTEP = (FS_THREADS / CH);         // 25 rows per round
    if (tid < RSTEP * CH) {
        const int ch = tid % CH;
        int ly = (tid / CH) % FS_AY, lz = (tid / CH) / FS_AY;
        const int i = x0 - 4 + 4 * ch;
        const bool x_ok = (i + 3 >= P.lo[0]) && (i <= P.hi[0]);
        for (int row = tid / CH; row < FS_AZ * FS_AY; row += RSTEP) {
            const int j = y0 - 2 + ly, k = z0 - 2 + lz;
            float* dst = &A[lz][ly][4 * ch];
            if (!zero_in && x_ok && j >= P.lo[1] && j <= P.hi[1] && k >= P.lo[2] && k <= P.hi[2]) {
                cp_async16(dst, phi_in + P.idx(i, j, k));
            } else {
                *reinterpret_cast<float4*>(dst) = make_float4(0.f, 0.f, 0.f, 0.f);
            }
            ly += RSTEP % FS_AY; lz += RSTEP / FS_AY;
            if (ly >= FS_AY) { ly -= FS_AY; lz += 1; }
        }
    }
    cp_async_wait_all();
    __syncthreads();
    }

    // local (lx, ly, lz) -> A / N element, and the patch-inside test
    auto aat = [&] (int lx, int ly, int lz) -> float& { return A[lz + 2][ly + 2][lx + 4]; };
    auto nat = [&] (int lx, int ly, int lz) -> float& { return N[lz + 1][ly + 1][lx + 1]; };

    // ghost layers of the patch faces inside the tile + 1 region (lx in -1..32,
    // ly, lz in -1..8), restricted to the patch's extent along the face.
    // fn(face, ghost, face cell, inner cell) with local coordinates.
    auto for_face_ghosts = [&] (auto&& fn) {
        const int lim[3] = {FS_TX, FS_TY, FS_TZ};
        const int plo[3] = {pxl, pyl, pzl}, phi[3] = {pxh, pyh, pzh};
        for (int f = 0; f < 6; ++f) {
            const int d = f % 3;
            const int g = (f < 3) ? plo[d] - 1 : phi[d] + 1;
            if (g < -1 || g > lim[d]) { continue; }
            const int s = (f < 3) ? 1 : -1;          // from the ghost into the patch
            const int t1 = (d == 0) ? 1 : 0, t2 = (d == 2) ? 1 : 2;
            const int a1 = max(-1, plo[t1]), b1 = min(lim[t1], phi[t1]);
            const int a2 = max(-1, plo[t2]), b2 = min(lim[t2], phi[t2]);
            const int n1 = b1 - a1 + 1, n2 = b2 - a2 + 1;
            if (n1 <= 0 || n2 <= 0) { continue; }
            for (int u = tid; u < n1 * n2; u += FS_THREADS) {
                int c[3];
                c[d] = g; c[t1] = a1 + u % n1; c[t2] = a2 + u / n1;
                int cf[3] = {c[0], c[1], c[2]}, ci[3] = {c[0], c[1], c[2]};
                cf[d] += s; ci[d] += 2 * s;
                fn(f, c, cf, ci);
            }
        }
    };

    // the rest of the sweep, compiled separately for tiles that touch a patch
    // face (ghost rewrites, inside tests, boundary correction) and for the others
    auto sweep = [&] (auto touch_tag) {
        constexpr bool TOUCH = decltype(touch_tag)::value;
        if constexpr (TOUCH) {
            // applyBC before the first colour: closure of the old values
            for_face_ghosts([&] (int f, const int* c, const int* cf, const int* ci) {
                aat(c[0], c[1], c[2]) = P.closure(f, aat(cf[0], cf[1], cf[2]), aat(ci[0], ci[1], ci[2]));
            });
            __syncthreads();
        }

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
        const float fco0 = P.f[0].fco, fco1 = P.f[1].fco, fco2 = P.f[2].fco;
        const float fco3 = P.f[3].fco, fco4 = P.f[4].fco, fco5 = P.f[5].fco;
        // Gauss-Seidel update of local cell (lx, ly, lz) at global offset o from q0
        auto update = [&] (int lx, int ly, int lz, int o, float pc, float xm, float xp, float ym, float yp, float zm,
                           float zp) {
            float d, sxl, sxh, syl, syh, szl, szh;
            if constexpr (VARC) {
                d = __ldg(Dp + o);
                sxl = __ldg(SXp + o); sxh = __ldg(SXp + o + 1);
                syl = __ldg(SYp + o); syh = __ldg(SYp + o + sx);
                szl = __ldg(SZp + o); szh = __ldg(SZp + o + sxy);
            } else {
                d = cd; sxl = sxh = cdx; syl = syh = cdy; szl = szh = cdz;
            }
            float gmd = d;
            if constexpr (TOUCH) {
                float corr = 0.0f;
                if (lx == pxl) { corr += sxl * fco0; }
                if (lx == pxh) { corr += sxh * fco3; }
                if (ly == pyl) { corr += syl * fco1; }
                if (ly == pyh) { corr += syh * fco4; }
                if (lz == pzl) { corr += szl * fco2; }
                if (lz == pzh) { corr += szh * fco5; }
                gmd = d - corr;
            }
            const float rho = sxl * xm + sxh * xp + syl * ym + syh * yp + szl * zm + szh * zp;
            const float res = __ldg(rh + o) - (d * pc - rho);
            return pc + relax_factor(gmd) * res;
        };

        // ---- first colour on the tile + 1: 17 cells per row, 10 x 10 rows;
        // 255 threads = 17 columns x 15 row streams
        {
            constexpr int RS = FS_THREADS / FS_RED_ROW;      // 15
            const int par0 = (x0 - 1 + y0 - 1 + z0 - 1) & 1;  // parity of local (-1, -1, -1)
            if (tid < RS * FS_RED_ROW) {
                const int r = tid % FS_RED_ROW;
                int ry = (tid / FS_RED_ROW) % FS_NY, rz = (tid / FS_RED_ROW) / FS_NY;
    #pragma unroll 2
                for (int row = tid / FS_RED_ROW; row < FS_NZ * FS_NY; row += RS) {
                    const int ly = ry - 1, lz = rz - 1;
                    // (x+y+z) even: local lx = 2r - 1 + ((par0 + ry + rz) & 1)
                    const int lx = 2 * r - 1 + ((par0 + ry + rz) & 1);
                    const int nout = int(lx < 0 || lx >= FS_TX) + int(ly < 0 || ly >= FS_TY) +
                                     int(lz < 0 || lz >= FS_TZ);
                    const bool in = nout <= 1 && (!TOUCH || (lx >= pxl && lx <= pxh && ly >= pyl && ly <= pyh &&
                                                              lz >= pzl && lz <= pzh));
                    if (in) {
                        const int o = lz * sxy + ly * sx + lx;
                        nat(lx, ly, lz) = update(lx, ly, lz, o, aat(lx, ly, lz), aat(lx - 1, ly, lz), aat(lx + 1, ly, lz),
                                                 aat(lx, ly - 1, lz), aat(lx, ly + 1, lz), aat(lx, ly, lz - 1),
                                                 aat(lx, ly, lz + 1));
                    }
                    ry += RS % FS_NY; rz += RS / FS_NY;
                    if (ry >= FS_NY) { ry -= FS_NY; rz += 1; }
                }
            }
        }
        __syncthreads();
        if constexpr (TOUCH) {
            // applyBC before the second colour: closure of the current values
            // (new first-colour values in N, old second-colour values in A)
            const int par0 = (x0 + y0 + z0) & 1;      // parity of local (0, 0, 0)
            auto cur = [&] (const int* c) -> float {
                return (((par0 + c[0] + c[1] + c[2]) & 1) == 0) ? nat(c[0], c[1], c[2]) : aat(c[0], c[1], c[2]);
            };
            for_face_ghosts([&] (int f, const int* c, const int* cf, const int* ci) {
                nat(c[0], c[1], c[2]) = P.closure(f, cur(cf), cur(ci));
            });
            __syncthreads();
        }

        // ---- second colour on the tile; each thread writes one (even x, odd x)
        // pair: 16 pairs per row, 8 x 8 rows, 4 rounds
        {
            const int r = tid % (FS_TX / 2);
            const int ly = (tid / (FS_TX / 2)) % FS_TY;
            const int lzs = (tid / (FS_TX / 2)) / FS_TY;     // 0..1
            const int par0 = (x0 + y0 + z0) & 1;
    #pragma unroll
            for (int lz = lzs; lz < FS_TZ; lz += 2) {
                const int lxe = 2 * r;                       // pair (lxe, lxe + 1)
                const bool first_at_even = ((par0 + lxe + ly + lz) & 1) == 0;
                const int lx2 = first_at_even ? lxe + 1 : lxe;   // the second-colour cell of the pair
                const int o = lz * sxy + ly * sx + lx2;
                const bool in2 = !TOUCH || (lx2 <= pxh && ly <= pyh && lz <= pzh);
                float v2 = 0.0f;
                if (in2) {
                    v2 = update(lx2, ly, lz, o, aat(lx2, ly, lz), nat(lx2 - 1, ly, lz), nat(lx2 + 1, ly, lz),
                                nat(lx2, ly - 1, lz), nat(lx2, ly + 1, lz), nat(lx2, ly, lz - 1), nat(lx2, ly, lz + 1));
                }
                const int lx1 = first_at_even ? lxe : lxe + 1;
                const float v1 = nat(lx1, ly, lz);
                const long long qp = q0 + (long long)(lz * sxy + ly * sx + lxe);
                if (!TOUCH || (lxe + 1 <= pxh && ly <= pyh && lz <= pzh)) {
                    *reinterpret_cast<float2*>(phi_out + qp) = first_at_even ? make_float2(v1, v2) : make_float2(v2, v1);
                } else if (lxe <= pxh && ly <= pyh && lz <= pzh) {
                    phi_out[qp] = first_at_even ? v1 : v2;
                }
            }
        }
    };
    if (touches) { sweep(std::true_type{}); } else { sweep(std::false_type{}); }
}

// The correction residual of a fused level and its restriction in one pass
// (MLMGT::mgVcycle's computeResOfCorrection then restriction,
// AMReX_MLMG.H:1306-1415; amrex_avgdown, AMReX_MultiFabUtil_3D_C.H:375-392):
// each 32x8x8 tile stages the correction over the tile grown by two by one
// TMA load (the box of the fused sweep), closes the patch faces in shared
// memory (homogeneous closures, as applyBC before the residual), computes
// r = res - A cor for its cells with the arithmetic of k_residual_s into
// shared memory, and writes the 16x4x4 coarse right-hand sides as the mean of
// each 2x2x2 group, summed in k_restrict's order.  The fine residual never
// goes to memory, and the restriction is no separate launch.  A level is
// coarsenable, so patches and tiles start on even cells and hold whole groups.
// Each thread computes the residuals of a column of 8 cells; the loads of the
// first NB planes' rhs and stencil values are issued before it waits for the
// copy, the rest after it.  Measured on the 256^3 solve (ABec): all 8 planes
// early (64 values in registers, 3 blocks per SM) 23.34 ms, 4 early at 4 / 5
// blocks 23.31 / 23.10 ms, 2 early at 5 blocks 22.98 ms, none early at 5 / 6
// blocks 23.14 / 23.10 ms; the separate residual and restriction launches
// 23.78 ms.
template <bool VARC, int NB = FS_TZ, int MINB = 3>
__global__ void __launch_bounds__(FS_THREADS, MINB)
k_resid_restrict_tma (DevLevel L, Subset S, DevLevel Lc, const float* __restrict__ rhs, StencilPtrs Sc,
                      const CUtensorMap* __restrict__ maps, float* __restrict__ crse, int* err)
{
    __shared__ __align__(128) float A[FS_AZ][FS_AY][FS_AX];   // cor, local (x-4..x+35, y-2..y+9, z-2..z+9)
    __shared__ float R[FS_TZ][FS_TY][FS_TX];                    // the tile's residuals
    __shared__ PatchLite SP;
    __shared__ unsigned long long bar;
    const int tid = threadIdx.y * FS_TX + threadIdx.x;
    const TileCoord c = decode_fused_tile(L, S, blockIdx.x);
    const int x0 = c.x0, y0 = c.y0, z0 = c.z0;
    const PatchDesc& PD = L.P[c.p];
    if (tid == 0) {
        for (int d = 0; d < 3; ++d) { SP.lo[d] = PD.lo[d]; SP.hi[d] = PD.hi[d]; }
        SP.sx = PD.sx; SP.sxy = PD.sxy; SP.base = PD.base;
        SP.dhx = float(PD.dha[0]); SP.dhy = float(PD.dha[1]); SP.dhz = float(PD.dha[2]);
        for (int f = 0; f < 6; ++f) {
            SP.f[f].type = PD.face[f].type;
            SP.f[f].nx = PD.face[f].nx;
            SP.f[f].c1 = float(PD.face[f].coef[1]);
            SP.f[f].c2 = float(PD.face[f].coef[2]);
            SP.f[f].fco = float(PD.face[f].fco);
        }
        tma::mbar_init(&bar, 1);
    }
    // the coarse patch under the tile's first and last cells; a tile that
    // lies over one coarse patch (nearly all) looks it up once
    const int pc = find_patch(Lc, PD.solve, x0 >> 1, y0 >> 1, z0 >> 1);
    const PatchGeom C = geom_of(Lc.P[pc]);
    const bool one = contains(C, min(x0 + FS_TX - 1, PD.hi[0]) >> 1, min(y0 + FS_TY - 1, PD.hi[1]) >> 1,
                              min(z0 + FS_TZ - 1, PD.hi[2]) >> 1);
    __syncthreads();
    pdl_wait();
    pdl_trigger();
    const PatchLite& P = SP;
    const int cx = x0 - P.lo[0] + XOFF - 4, cy = y0 - P.lo[1] - 1, cz = z0 - P.lo[2] - 1;
    if ((cx & 3) != 0) {
        if (tid == 0) { atomicExch(err, tma::ERR_TMA_ALIGN); }
        return;
    }
    if (tid == 0) {
        tma::mbar_expect_tx(&bar, (unsigned)sizeof(A));
        tma::load_3d(&A[0][0][0], maps + c.p, &bar, cx, cy, cz);
    }
    // patch bounds in tile-local coordinates
    const int pl[3] = {P.lo[0] - x0, P.lo[1] - y0, P.lo[2] - z0};
    const int ph[3] = {P.hi[0] - x0, P.hi[1] - y0, P.hi[2] - z0};
    // the rhs and stencil values of the thread's column of 8 cells, loaded
    // while the correction's copy is in flight
    const int lx = threadIdx.x, ly = threadIdx.y;
    const bool inxy = lx <= ph[0] && ly <= ph[1];
    const long long q0 = P.idx(x0, y0, z0);
    const int sx = P.sx, sxy = (int)P.sxy;
    // the stencil of plane lz of the thread's column (zeros outside the patch)
    struct Cell8 { float r, d, xl, xh, yl, yh, zl, zh; };
    auto load = [&] (int lz) {
        Cell8 c{};
        const bool in = inxy && lz <= ph[2];
        const int o = lz * sxy + ly * sx + lx;
        c.r = in ? __ldg(rhs + q0 + o) : 0.0f;
        if constexpr (VARC) {
            const float* Dp = static_cast<const float*>(Sc.D) + q0;
            const float* SXp = static_cast<const float*>(Sc.sx) + q0;
            const float* SYp = static_cast<const float*>(Sc.sy) + q0;
            const float* SZp = static_cast<const float*>(Sc.sz) + q0;
            c.d = in ? __ldg(Dp + o) : 0.0f;
            c.xl = in ? __ldg(SXp + o) : 0.0f; c.xh = in ? __ldg(SXp + o + 1) : 0.0f;
            c.yl = in ? __ldg(SYp + o) : 0.0f; c.yh = in ? __ldg(SYp + o + sx) : 0.0f;
            c.zl = in ? __ldg(SZp + o) : 0.0f; c.zh = in ? __ldg(SZp + o + sxy) : 0.0f;
        }
        return c;
    };
    // the first NB planes' loads are issued before the copy's wait
    Cell8 pre[NB > 0 ? NB : 1];
#pragma unroll
    for (int lz = 0; lz < NB; ++lz) { pre[lz] = load(lz); }
    const bool late = !tma::mbar_wait_bounded(&bar, 0, tma::WAIT_LIMIT);
    if (__syncthreads_or(late)) {
        if (tid == 0) { atomicExch(err, tma::ERR_TMA_TIMEOUT); }
        tma::mbar_wait_bounded(&bar, 0, tma::WAIT_LIMIT);
        return;
    }
    auto aat = [&] (int ax, int ay, int az) -> float& { return A[az + 2][ay + 2][ax + 4]; };
    const int lim[3] = {FS_TX - 1, FS_TY - 1, FS_TZ - 1};
    // ghost layers of the patch faces next to the tile's cells: the closure
    // of the face cell and the next inner cell
    for (int f = 0; f < 6; ++f) {
        const int d = f % 3;
        const int g = (f < 3) ? pl[d] - 1 : ph[d] + 1;
        if (g < -1 || g > lim[d] + 1) { continue; }
        const int s = (f < 3) ? 1 : -1;
        const int t1 = (d == 0) ? 1 : 0, t2 = (d == 2) ? 1 : 2;
        const int a1 = max(0, pl[t1]), b1 = min(lim[t1], ph[t1]);
        const int a2 = max(0, pl[t2]), b2 = min(lim[t2], ph[t2]);
        const int n1 = b1 - a1 + 1, n2 = b2 - a2 + 1;
        if (n1 <= 0 || n2 <= 0) { continue; }
        for (int u = tid; u < n1 * n2; u += FS_THREADS) {
            int cc[3];
            cc[d] = g; cc[t1] = a1 + u % n1; cc[t2] = a2 + u / n1;
            int cf[3] = {cc[0], cc[1], cc[2]}, ci[3] = {cc[0], cc[1], cc[2]};
            cf[d] += s; ci[d] += 2 * s;
            aat(cc[0], cc[1], cc[2]) = P.closure(f, aat(cf[0], cf[1], cf[2]), aat(ci[0], ci[1], ci[2]));
        }
    }
    __syncthreads();
    // r = res - A cor for the tile's cells (k_residual_s's arithmetic)
    {
        const float dhx = P.dhx, dhy = P.dhy, dhz = P.dhz;
        const float cdd = float(-2.0) * (dhx + dhy + dhz);
#pragma unroll
        for (int lz = 0; lz < FS_TZ; ++lz) {
            float v = 0.0f;
            const Cell8 c = (lz < NB) ? pre[lz < NB ? lz : 0] : load(lz);
            if (inxy && lz <= ph[2]) {
                float d, sxl, sxh, syl, syh, szl, szh;
                if constexpr (VARC) {
                    d = c.d; sxl = c.xl; sxh = c.xh; syl = c.yl; syh = c.yh; szl = c.zl; szh = c.zh;
                } else {
                    d = cdd; sxl = sxh = -dhx; syl = syh = -dhy; szl = szh = -dhz;
                }
                const float xc = aat(lx, ly, lz);
                const float nb = sxl * aat(lx - 1, ly, lz) + sxh * aat(lx + 1, ly, lz) + syl * aat(lx, ly - 1, lz) +
                                 syh * aat(lx, ly + 1, lz) + szl * aat(lx, ly, lz - 1) + szh * aat(lx, ly, lz + 1);
                v = c.r - (d * xc - nb);
            }
            R[lz][ly][lx] = v;
        }
    }
    __syncthreads();
    // the coarse cells of the tile: one per thread (16 x 4 x 4)
    {
        const int ux = tid % (FS_TX / 2), uy = (tid / (FS_TX / 2)) % (FS_TY / 2), uz = tid / ((FS_TX / 2) * (FS_TY / 2));
        const int fx = 2 * ux, fy = 2 * uy, fz = 2 * uz;
        if (fx <= ph[0] && fy <= ph[1] && fz <= ph[2]) {
            float v = 0;
            v += R[fz][fy][fx];         v += R[fz][fy][fx + 1];
            v += R[fz][fy + 1][fx];     v += R[fz][fy + 1][fx + 1];
            v += R[fz + 1][fy][fx];     v += R[fz + 1][fy][fx + 1];
            v += R[fz + 1][fy + 1][fx]; v += R[fz + 1][fy + 1][fx + 1];
            const int i = (x0 >> 1) + ux, j = (y0 >> 1) + uy, k = (z0 >> 1) + uz;
            const long long qc = one ? cidx(C, i, j, k) : cidx(Lc.P[find_patch(Lc, C.solve, i, j, k)], i, j, k);
            crse[qc] = (float(1.0) / float(8)) * v;
        }
    }
}

// One colour of MLPoisson's Gauss-Seidel sweep over a list of fused-sweep
// tiles of an AMR fine level (the tiles whose halo meets a face shared with
// another patch): old cell values from `old` (null: a zero correction),
// neighbours from `nb` (the old array for the first colour, the new one for
// the second; null: zeros), results into `out`.  A ghost covered by another patch is that
// patch's cell (nbr), any other ghost the homogeneous closure; the update is
// the fused sweep's arithmetic, so a cell gets the value the fused sweep gives
// it from the same neighbours.  Launched for the first colour over these tiles
// together with the fused sweep over the others (both read only the old
// array), then for the second colour.
template <bool OLD, bool NB>
static __global__ void __launch_bounds__(FS_THREADS)
k_gsrb_tiles (DevLevel L, const int4* __restrict__ tiles, const float* __restrict__ old, const float* __restrict__ nb,
              float* __restrict__ out, const float* __restrict__ rhs, const long long* __restrict__ nbr, int rb)
{
    const int4 t = tiles[blockIdx.x];
    const PatchDesc& P = L.P[t.x];
    // the patch's geometry in registers (as far as the compiler knows, the
    // stores below could change the descriptor, which it would then reload
    // for every cell); offsets inside the tile in 32 bits from its first cell
    const int lo0 = P.lo[0], lo1 = P.lo[1], lo2 = P.lo[2], hi0 = P.hi[0], hi1 = P.hi[1], hi2 = P.hi[2];
    const int sx = P.sx, sxy = (int)P.sxy;
    const float dhx = float(P.dha[0]), dhy = float(P.dha[1]), dhz = float(P.dha[2]);
    const float cdx = -dhx, cdy = -dhy, cdz = -dhz, cd = -2.0f * (dhx + dhy + dhz);
    const long long q00 = cidx(P, t.y, t.z, t.w);
    pdl_wait();
    pdl_trigger();
    // lanes 0..15 take the 16 cells of the colour in a row of plane lz, lanes
    // 16..31 those of plane lz + 1
    const int j = t.z + threadIdx.y;
    const int half = threadIdx.x >> 4, r = threadIdx.x & 15;
    if (j > hi1) { return; }
    // the ghost across face f: the covering patch's cell, or the closure
    // (which also adds the face's diagonal term, s_f * fco_f, to corr)
    auto ghost = [&] (int f, int i, int k, float pc, long long qin, float s, float& corr) -> float {
        const FaceBC& F = P.face[f];
        const long long v = nbr[F.bcval_off + face_local(P, f, i, j, k)];
        if (v >= 0) { return NB ? nb[v] : 0.0f; }
        const float pin = NB ? nb[qin] : 0.0f;
        float g = 0.0f;
        if (F.type == BC_DIRICHLET) {
            const float c1 = float(F.coef[1]), c2 = float(F.coef[2]);
            g = (F.nx >= 2) ? pc * c1 : 0.0f;
            if (F.nx >= 3) { g += pin * c2; }
        } else if (F.type == BC_NEUMANN) {
            g = pc;
        } else if (F.type == BC_REFLECT_ODD) {
            g = -pc;
        }
        corr += s * float(F.fco);
        return g;
    };
    for (int lz = half; lz < FS_TZ; lz += 2) {
        const int k = t.w + lz;
        if (k > hi2) { break; }
        const int i = t.y + 2 * r + ((t.y + j + k + rb) & 1);
        if (i > hi0) { continue; }
        const long long q = q00 + (lz * sxy + (int)threadIdx.y * sx + (i - t.y));
        const float pc = OLD ? old[q] : 0.0f;
        // the closures' diagonal terms accumulate in the fused sweep's order
        // (x-lo, x-hi, y-lo, y-hi, z-lo, z-hi)
        float corr = 0.0f;
        const float xm = (i == lo0) ? ghost(0, i, k, pc, q + 1, cdx, corr) : (NB ? nb[q - 1] : 0.0f);
        const float xp = (i == hi0) ? ghost(3, i, k, pc, q - 1, cdx, corr) : (NB ? nb[q + 1] : 0.0f);
        const float ym = (j == lo1) ? ghost(1, i, k, pc, q + sx, cdy, corr) : (NB ? nb[q - sx] : 0.0f);
        const float yp = (j == hi1) ? ghost(4, i, k, pc, q - sx, cdy, corr) : (NB ? nb[q + sx] : 0.0f);
        const float zm = (k == lo2) ? ghost(2, i, k, pc, q + sxy, cdz, corr) : (NB ? nb[q - sxy] : 0.0f);
        const float zp = (k == hi2) ? ghost(5, i, k, pc, q - sxy, cdz, corr) : (NB ? nb[q + sxy] : 0.0f);
        const bool face = (i == lo0) | (i == hi0) | (j == lo1) | (j == hi1) | (k == lo2) | (k == hi2);
        const float gmd = face ? cd - corr : cd;
        const float d = cd, sxl = cdx, sxh = cdx, syl = cdy, syh = cdy, szl = cdz, szh = cdz;
        const float rho = sxl * xm + sxh * xp + syl * ym + syh * yp + szl * zm + szh * zp;
        const float res = __ldg(rhs + q) - (d * pc - rho);
        out[q] = pc + relax_factor(gmd) * res;
    }
}

} // namespace mlmg
