// Coarse/fine coupling kernels of the AMR composite solve (refinement ratio
// 2, MLPoisson or MLABecLaplacian).  Every kernel reads index tables built on the host from the
// two levels' patch layouts, so a launch covers every box of a level.
#pragma once

#include "stencil_kernels.cuh"

namespace mlmg {

// One thread per cell of a list of boxes: prefix `start` over the boxes' cell
// counts, box w holds cells [start[w], start[w+1]).
__device__ __forceinline__ void tag_cell (const CopyTag* tags, const long long* start, int ntag, long long t,
                                          int& w, int& i, int& j, int& k)
{
    w = bsearch_ll<int>(start, ntag, t);
    const CopyTag& C = tags[w];
    // a box holds fewer than 2^32 cells: 32-bit index arithmetic
    const unsigned u = (unsigned)(t - start[w]);
    const unsigned nx = C.box.hi[0] - C.box.lo[0] + 1, ny = C.box.hi[1] - C.box.lo[1] + 1;
    const unsigned row = u / nx;
    i = C.box.lo[0] + (int)(u - row * nx);
    j = C.box.lo[1] + (int)(row % ny);
    k = C.box.lo[2] + (int)(row / ny);
}

// The coarse level's field (valid cells) into the per-fine-patch coarse
// buffers over the coarsened fine patch grown by one cell, which were zeroed
// first: BndryRegisterT::copyFrom and the ParallelCopy of
// MLMGT::interpCorrection (AMReX_MLMG.H:1719-1750).  Tag dst = fine patch
// (its coarse buffer descriptor), src = coarse patch, whose cell is the
// buffer cell minus the tag's periodic shift.
template <typename T>
__global__ void k_amr_gather (DevLevel Lc, const PatchDesc* __restrict__ cfd, const CopyTag* __restrict__ tags,
                              const long long* __restrict__ start, int ntag, long long ncell,
                              const T* __restrict__ crse, T* __restrict__ cf)
{
    pdl_wait();
    pdl_trigger();
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= ncell) { return; }
    int w, i, j, k;
    tag_cell(tags, start, ntag, t, w, i, j, k);
    const CopyTag& C = tags[w];
    cf[cidx(cfd[C.dst], i, j, k)] = crse[cidx(Lc.P[C.src], i - C.shift[0], j - C.shift[1], k - C.shift[2])];
}

// amrex::average_down onto the covered coarse cells (amrex_avgdown,
// Src/Base/AMReX_MultiFabUtil_3D_C.H:375-392).  Tag dst = coarse patch,
// src = fine patch, box in coarse index space.
template <typename TD, typename TS>
__global__ void k_amr_avgdown (DevLevel Lc, DevLevel Lf, const CopyTag* __restrict__ tags,
                               const long long* __restrict__ start, int ntag, long long ncell,
                               const TS* __restrict__ fine, TD* __restrict__ crse, float* __restrict__ crse32)
{
    pdl_wait();
    pdl_trigger();
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= ncell) { return; }
    int w, i, j, k;
    tag_cell(tags, start, ntag, t, w, i, j, k);
    const CopyTag& C = tags[w];
    const PatchDesc& F = Lf.P[C.src];
    const long long qf = cidx(F, 2 * i, 2 * j, 2 * k);
    const long long sx = F.sx, sxy = F.sxy;
    double v = 0;
    v += (double)fine[qf];            v += (double)fine[qf + 1];
    v += (double)fine[qf + sx];       v += (double)fine[qf + sx + 1];
    v += (double)fine[qf + sxy];      v += (double)fine[qf + sxy + 1];
    v += (double)fine[qf + sxy + sx]; v += (double)fine[qf + sxy + sx + 1];
    const long long qc = cidx(Lc.P[C.dst], i, j, k);
    crse[qc] = TD(0.125 * v);
    if (crse32 != nullptr) { crse32[qc] = d2f_bits(double(TD(0.125 * v))); }
}

// average_down_faces with the coarse geometry (Src/Base/AMReX_MultiFabUtil.H:
// 958-968; amrex_avgdown_faces, AMReX_MultiFabUtil_3D_C.H:170-225) of the face
// coefficient b_dir: every coarse face of a coarsened fine patch, its boundary
// faces included, takes the mean of the 2x2 fine faces on it, summed with the
// second tangential offset outermost.  Tag dst = coarse patch, src = fine
// patch, box = coarse faces in the fine patch's frame (face i stored at cell
// index i of a patch); the coarse patch's face is box - shift (periodic images).
__global__ void k_amr_avgdown_faces (DevLevel Lc, DevLevel Lf, const CopyTag* __restrict__ tags,
                                     const long long* __restrict__ start, int ntag, long long ncell, int dir,
                                     const double* __restrict__ fine, double* __restrict__ crse)
{
    pdl_wait();
    pdl_trigger();
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= ncell) { return; }
    int w, i, j, k;
    tag_cell(tags, start, ntag, t, w, i, j, k);
    const CopyTag& C = tags[w];
    const PatchDesc& F = Lf.P[C.src];
    const long long st[3] = {1, (long long)F.sx, F.sxy};
    const int t1 = (dir == 0) ? 1 : 0, t2 = (dir == 2) ? 1 : 2;
    const long long qf = cidx(F, 2 * i, 2 * j, 2 * k);
    double c = 0.0;
    c += fine[qf];
    c += fine[qf + st[t1]];
    c += fine[qf + st[t2]];
    c += fine[qf + st[t1] + st[t2]];
    crse[cidx(Lc.P[C.dst], i - C.shift[0], j - C.shift[1], k - C.shift[2])] = c * 0.25;
}

// bits of the per-face-cell neighbourhood flags of the boundary interpolation
enum : int {
    BF_SELF = 1,        // the ghost cell itself is not covered (a coarse/fine cell)
    BF_T1LO = 2,        // the ghost cell two fine cells down the first tangential direction is not covered
    BF_T1HI = 4,        // ... two cells up the first tangential direction
    BF_T2LO = 8,        // ... down the second tangential direction
    BF_T2HI = 16,       // ... up the second tangential direction
    BF_CROSS = 32,      // all four diagonal ghost cells (+-2, +-2) are not covered
};

// InterpBndryDataT::updateBndryValues (Src/Boundary/AMReX_InterpBndryData.H:
// 158-267) with interpbndrydata_{x,y,z}_o3 (AMReX_InterpBndryData_3D_K.H:20-120):
// the Dirichlet value of every not-covered ghost cell on the coarse/fine faces
// of the fine level, from the coarse buffer: the coarse value at the ghost
// cell's coarse cell plus tangential slopes and curvatures (one-sided where a
// neighbouring ghost cell is covered or outside) and the cross term.  Output
// slots are the faces' Dirichlet-value slots (FaceBC::bcval_off + u).
template <typename T>
__global__ void k_amr_bndry (DevLevel Lf, GhostWork W, const PatchDesc* __restrict__ cfd, const T* __restrict__ cf,
                             const int8_t* __restrict__ flags, double* __restrict__ bcval)
{
    pdl_wait();
    pdl_trigger();
    const long long tid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (tid >= W.nfacecells) { return; }
    const int w = bsearch_ll<int>(W.fstart, W.nface, tid);
    const int2 pf = W.faces[w];
    const PatchDesc& P = Lf.P[pf.x];
    const int f = pf.y;
    const long long u = tid - W.fstart[w];
    const long long slot = P.face[f].bcval_off + u;
    const int fl = flags[slot];
    if (!(fl & BF_SELF)) { return; }
    int c[3];
    face_cell(P, f, u, c[0], c[1], c[2]);
    const int d = f % 3;
    const int t1 = (d == 0) ? 1 : 0, t2 = (d == 2) ? 1 : 2;
    const PatchDesc& G = cfd[pf.x];
    const long long st[3] = {1, (long long)G.sx, G.sxy};
    const int cc[3] = {c[0] >> 1, c[1] >> 1, c[2] >> 1};
    const long long q = cidx(G, cc[0], cc[1], cc[2]);
    const double c0 = (double)cf[q];
    double slope[2], curv[2];
#pragma unroll
    for (int m = 0; m < 2; ++m) {
        const long long s = st[m == 0 ? t1 : t2];
        const bool lo_nc = fl & (m == 0 ? BF_T1LO : BF_T2LO);
        const bool hi_nc = fl & (m == 0 ? BF_T1HI : BF_T2HI);
        const double vm = (double)cf[q - s], vp = (double)cf[q + s];
        const double vlo = lo_nc ? vm : c0, vhi = hi_nc ? vp : c0;
        const double fac = (lo_nc != hi_nc) ? 1.0 : 0.5;
        slope[m] = fac * (vhi - vlo);
        curv[m] = (lo_nc && hi_nc) ? 0.5 * (vp - 2.0 * c0 + vm) : 0.0;
    }
    double cross = 0.0;
    if (fl & BF_CROSS) {
        const long long s1 = st[t1], s2 = st[t2];
        cross = 0.25 * ((double)cf[q + s1 + s2] - (double)cf[q - s1 + s2] + (double)cf[q - s1 - s2]
                        - (double)cf[q + s1 - s2]);
    }
    const double y = -0.5 + ((double)(c[t1] - 2 * cc[t1]) + 0.5) / 2.0;
    const double z = -0.5 + ((double)(c[t2] - 2 * cc[t2]) + 0.5) / 2.0;
    bcval[slot] = c0 + y * slope[0] + (y * y) * curv[0] + z * slope[1] + (z * z) * curv[1] + y * z * cross;
}

// The same boundary values over a list of the coarse/fine ghost cells only
// (built with the flags): x = Dirichlet-value slot, y = element of the ghost
// cell's coarse cell in the coarse buffer, z = fine patch, w = the BF_* flags
// | the ghost cell's parity along the first / second tangential direction
// (bits 6, 7) | the face (bits 8..10).  No search and no covered ghost cells;
// the arithmetic is k_amr_bndry's.
template <typename T>
__global__ void k_amr_bndry_list (const int4* __restrict__ items, int n, const PatchDesc* __restrict__ cfd,
                                  const T* __restrict__ cf, double* __restrict__ bcval)
{
    pdl_wait();
    pdl_trigger();
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) { return; }
    const int4 it = items[t];
    const int fl = it.w & 63, f = it.w >> 8;
    const int d = f % 3;
    const int t1 = (d == 0) ? 1 : 0, t2 = (d == 2) ? 1 : 2;
    const PatchDesc& G = cfd[it.z];
    const long long st[3] = {1, (long long)G.sx, G.sxy};
    const long long q = it.y;
    const double c0 = (double)cf[q];
    double slope[2], curv[2];
#pragma unroll
    for (int m = 0; m < 2; ++m) {
        const long long s = st[m == 0 ? t1 : t2];
        const bool lo_nc = fl & (m == 0 ? BF_T1LO : BF_T2LO);
        const bool hi_nc = fl & (m == 0 ? BF_T1HI : BF_T2HI);
        const double vm = (double)cf[q - s], vp = (double)cf[q + s];
        const double vlo = lo_nc ? vm : c0, vhi = hi_nc ? vp : c0;
        const double fac = (lo_nc != hi_nc) ? 1.0 : 0.5;
        slope[m] = fac * (vhi - vlo);
        curv[m] = (lo_nc && hi_nc) ? 0.5 * (vp - 2.0 * c0 + vm) : 0.0;
    }
    double cross = 0.0;
    if (fl & BF_CROSS) {
        const long long s1 = st[t1], s2 = st[t2];
        cross = 0.25 * ((double)cf[q + s1 + s2] - (double)cf[q - s1 + s2] + (double)cf[q - s1 - s2]
                        - (double)cf[q + s1 - s2]);
    }
    const double y = -0.5 + ((double)((it.w >> 6) & 1) + 0.5) / 2.0;
    const double z = -0.5 + ((double)((it.w >> 7) & 1) + 0.5) / 2.0;
    bcval[it.x] = c0 + y * slope[0] + (y * y) * curv[0] + z * slope[1] + (z * z) * curv[1] + y * z * cross;
}

// ----------------------------------------------------------------- reflux --
// One coarse cell next to the fine level and the faces it shares with it.
struct RefluxCell {
    long long q;        // element index of the coarse cell
    int e0, ne;         // its face entries [e0, e0+ne)
};
struct RefluxFace {
    long long qn;       // element index of the covered coarse neighbour (in its own patch)
    long long qf;       // element index of the fine cell inside the fine patch at sub-face (0,0)
    long long qb;       // element index of the coarse face in the cell's patch (face coefficients)
    int fp;             // fine patch
    int dir, side;      // face direction; side 1: the neighbour (and the fine level) lies at +dir
};
struct RefluxParams {
    double dxinv_c[3];  // coarse 1/dx
    double dxinv_f[3];  // fine 1/dx
};
struct RefluxCoef {     // MLABecLaplacian: beta and the face b of both levels
    const double* bc[3];
    const double* bf[3];
    double beta;
};

// MLCellLinOpT::reflux (AMReX_MLCellLinOp.H:1272-1346) through YAFluxRegister
// (Src/Boundary/AMReX_YAFluxRegister.H:343-560, AMReX_YAFluxRegister_3D_K.H):
// res += sum over the cell's coarse/fine faces of the coarse face flux minus
// the mean of the fine face fluxes, divided by the coarse dx, with MLPoisson's
// flux F = (phi_hi - phi_lo)/dx.  The fine solution's ghosts must hold the
// inhomogeneous applyBC values.  Coarse contributions are summed first, in
// face order, then the fine ones (the register adds its fine patches last).
// The face flux is MLPoisson's dxinv (phi_i - phi_i-1) (mlpoisson_flux_x,
// AMReX_MLPoisson_3D_K.H:36-50) or MLABecLaplacian's
// -beta dxinv b_i (phi_i - phi_i-1) (mlabeclap_flux_x, AMReX_MLABecLap_3D_K.H:79-95).
template <bool ABEC>
__global__ void k_amr_reflux (DevLevel Lf, const RefluxCell* __restrict__ cells, const RefluxFace* __restrict__ faces,
                              int ncell, RefluxParams prm, RefluxCoef co, const double* __restrict__ sol_c,
                              const double* __restrict__ sol_f, double* __restrict__ res_c,
                              float* __restrict__ res32_c)
{
    pdl_wait();
    pdl_trigger();
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= ncell) { return; }
    const RefluxCell C = cells[t];
    const double vc = sol_c[C.q];
    double dc = 0.0;
    for (int e = C.e0; e < C.e0 + C.ne; ++e) {
        const RefluxFace& R = faces[e];
        const double dtdx = prm.dxinv_c[R.dir];
        const double vn = sol_c[R.qn];
        double fac = prm.dxinv_c[R.dir];
        if constexpr (ABEC) { fac = -(co.beta * prm.dxinv_c[R.dir]) * co.bc[R.dir][R.qb]; }
        if (R.side) { dc += dtdx * (fac * (vn - vc)); }
        else { dc -= dtdx * (fac * (vc - vn)); }
    }
    double dfine = 0.0;
    for (int e = C.e0; e < C.e0 + C.ne; ++e) {
        const RefluxFace& R = faces[e];
        const PatchDesc& F = Lf.P[R.fp];
        const long long st[3] = {1, (long long)F.sx, F.sxy};
        const int t1 = (R.dir == 0) ? 1 : 0, t2 = (R.dir == 2) ? 1 : 2;
        const long long sd = st[R.dir];
        const double dtdx = prm.dxinv_f[R.dir] * 0.125;   // dt / (dx_f * rr^3)
        double acc = 0.0;
        for (int o2 = 0; o2 < 2; ++o2)
        for (int o1 = 0; o1 < 2; ++o1) {
            const long long qi = R.qf + o1 * st[t1] + o2 * st[t2];
            double fac = prm.dxinv_f[R.dir];
            if (R.side) {   // fine level above: the fine box's low face, ghost below
                if constexpr (ABEC) { fac = -(co.beta * prm.dxinv_f[R.dir]) * co.bf[R.dir][qi]; }
                acc += -dtdx * (fac * (sol_f[qi] - sol_f[qi - sd]));
            } else {        // fine level below: the fine box's high face, ghost above
                if constexpr (ABEC) { fac = -(co.beta * prm.dxinv_f[R.dir]) * co.bf[R.dir][qi + sd]; }
                acc += dtdx * (fac * (sol_f[qi + sd] - sol_f[qi]));
            }
        }
        dfine += acc;
    }
    const double nv = res_c[C.q] + (dc + dfine);
    res_c[C.q] = nv;
    if (res32_c != nullptr) { res32_c[C.q] = d2f_bits(nv); }
}

// per-block max|x| over the valid cells whose `covered` byte is 0 (the
// norms of a coarse AMR level, MLCellLinOpT::normInf, AMReX_MLCellLinOp.H:2006-2101)
template <typename T>
__global__ void __launch_bounds__(TILE_THREADS)
k_amr_norm (DevLevel L, Subset S, const T* __restrict__ x, const int8_t* __restrict__ covered,
            double* __restrict__ partial)
{
    pdl_wait();
    pdl_trigger();
    __shared__ double sm[32];
    const TileCoord c = decode_tile(L, S, blockIdx.x);
    const PatchDesc& P = L.P[c.p];
    const int j = c.y0 + threadIdx.y;
    double acc = 0.0;
    if (j <= P.hi[1]) {
        for (int kk = 0; kk < TILE_Z; ++kk) {
            const int k = c.z0 + kk;
            if (k > P.hi[2]) { break; }
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                const int i = c.x0 + threadIdx.x + 32 * h;
                if (i > P.hi[0]) { continue; }
                const long long q = cidx(P, i, j, k);
                if (covered == nullptr || covered[q] == 0) {
                    if constexpr (std::is_same_v<T, double>) {
                        // integer max of the |x| bit patterns (NaN orders above every number)
                        const unsigned long long ab = abs_bits(x[q]), cur = (unsigned long long)__double_as_longlong(acc);
                        acc = __longlong_as_double((long long)((ab > cur) ? ab : cur));
                    } else {
                        acc = max_nan(acc, fabs((double)x[q]));
                    }
                }
            }
        }
    }
    const double red = block_reduce(acc, RED_MAXABS, sm);
    if (threadIdx.x == 0 && threadIdx.y == 0) { partial[blockIdx.x] = red; }
}

// r = b - A x over valid cells (BCs already in x's ghosts), with A x evaluated
// in x's precision: the correction residuals of the composite iteration, b
// and r in either precision.  MLABecLaplacian reads a and b in FP64, or the
// FP32 stencil form for FP32 corrections.
template <typename TX, typename TB, typename TO, bool ABEC>
__global__ void __launch_bounds__(TILE_THREADS)
k_amr_resid (DevLevel L, Subset S, TO* __restrict__ r, const TX* __restrict__ x, const TB* __restrict__ b,
             const double* __restrict__ a, const double* __restrict__ bx, const double* __restrict__ by,
             const double* __restrict__ bz, StencilPtrs sp)
{
    pdl_wait();
    pdl_trigger();
    const TileCoord c = decode_tile(L, S, blockIdx.x);
    const PatchDesc& P = L.P[c.p];
    // the geometry in registers, one 64-bit row start per plane
    const PatchGeom G = geom_of(P);
    const int j = c.y0 + threadIdx.y;
    if (j > G.hi[1]) { return; }
    const TX pdhx = convert<TX>(G.dha[0]), pdhy = convert<TX>(G.dha[1]), pdhz = convert<TX>(G.dha[2]);
    for (int kk = 0; kk < TILE_Z; ++kk) {
        const int k = c.z0 + kk;
        if (k > G.hi[2]) { break; }
        const long long row = cidx(G, G.lo[0], j, k);
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const int i = c.x0 + threadIdx.x + 32 * h;
            if (i > G.hi[0]) { continue; }
            const long long q = row + (i - G.lo[0]);
            TX ax;
            if constexpr (!ABEC) {
                // adotx_cell's MLPoisson form with the factors converted once per block
                const int sx = G.sx, sxy = (int)G.sxy;
                const TX xc = x[q];
                ax = pdhx * (x[q - 1] - TX(2.0) * xc + x[q + 1])
                   + pdhy * (x[q - sx] - TX(2.0) * xc + x[q + sx])
                   + pdhz * (x[q - sxy] - TX(2.0) * xc + x[q + sxy]);
            } else if constexpr (std::is_same_v<TX, double>) {
                ax = adotx_cell<double, true>(P, q, x, a, bx, by, bz);
            } else {
                // FP32 corrections: the stencil form D x - sum s x_nb
                const Coef7<TX, true> cf = load_coef<TX, true>(P, q, sp);
                const long long sx = P.sx, sxy = P.sxy;
                ax = cf.d * x[q] - (cf.sxl * x[q - 1] + cf.sxh * x[q + 1] + cf.syl * x[q - sx] + cf.syh * x[q + sx]
                                    + cf.szl * x[q - sxy] + cf.szh * x[q + sxy]);
            }
            r[q] = convert<TO>(TX(convert<TX>(b[q])) - ax);
        }
    }
}

// fine = trilinear prolongation of the coarse buffer (mlmg_lin_cc_interp_r2,
// AMReX_MLMG_3D_K.H:7-37; MLCellLinOpT::interpolationAmr,
// AMReX_MLCellLinOp.H:1094-1181), then sol += fine and,
// for an intermediate level, hold += fine (MLMGT::oneIter's up-sweep,
// AMReX_MLMG.H:1266-1276)
template <typename T>
__global__ void __launch_bounds__(TILE_THREADS)
k_amr_interp_add (DevLevel Lf, Subset Sf, const PatchDesc* __restrict__ cfd, const T* __restrict__ cf,
                  T* __restrict__ fine, double* __restrict__ sol, T* __restrict__ hold)
{
    pdl_wait();
    pdl_trigger();
    const TileCoord c = decode_tile(Lf, Sf, blockIdx.x);
    // both layouts in registers; per plane one 64-bit row start in each, the
    // rest 32-bit offsets (a coarse buffer plane holds fewer than 2^31 cells)
    const PatchGeom F = geom_of(Lf.P[c.p]);
    const PatchGeom G = geom_of(cfd[c.p]);
    const int j = c.y0 + threadIdx.y;
    if (j > F.hi[1]) { return; }
    const int gy = G.sx, gz = (int)G.sxy;
    const int jc = j >> 1;
    const int dj = (j & 1) ? gy : -gy;
    for (int kk = 0; kk < TILE_Z; ++kk) {
        const int k = c.z0 + kk;
        if (k > F.hi[2]) { break; }
        const int kc = k >> 1;
        const int dk = (k & 1) ? gz : -gz;
        const long long grow = cidx(G, G.lo[0], jc, kc), frow = cidx(F, F.lo[0], j, k);
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const int i = c.x0 + threadIdx.x + 32 * h;
            if (i > F.hi[0]) { continue; }
            const int ic = i >> 1;
            const int di = (i & 1) ? 1 : -1;
            const long long q = grow + (ic - G.lo[0]);
            const T v = T(0.421875) * cf[q]
                      + T(0.140625) * cf[q + di]
                      + T(0.140625) * cf[q + dj]
                      + T(0.140625) * cf[q + dk]
                      + T(0.046875) * cf[q + dj + dk]
                      + T(0.046875) * cf[q + di + dk]
                      + T(0.046875) * cf[q + di + dj]
                      + T(0.015625) * cf[q + di + dj + dk];
            const long long qf = frow + (i - F.lo[0]);
            fine[qf] = v;
            sol[qf] += double(v);
            if (hold != nullptr) { hold[qf] += v; }
        }
    }
}

// sol += cor and, for an intermediate level, cor += hold (the end of the
// up-sweep at one level, AMReX_MLMG.H:1283-1289)
template <typename T>
__global__ void __launch_bounds__(TILE_THREADS)
k_amr_finish (DevLevel L, Subset S, double* __restrict__ sol, T* __restrict__ cor, const T* __restrict__ hold)
{
    pdl_wait();
    pdl_trigger();
    const TileCoord c = decode_tile(L, S, blockIdx.x);
    const PatchGeom P = geom_of(L.P[c.p]);
    const int j = c.y0 + threadIdx.y;
    if (j > P.hi[1]) { return; }
    for (int kk = 0; kk < TILE_Z; ++kk) {
        const int k = c.z0 + kk;
        if (k > P.hi[2]) { break; }
        const long long row = cidx(P, P.lo[0], j, k);
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const int i = c.x0 + threadIdx.x + 32 * h;
            if (i > P.hi[0]) { continue; }
            const long long q = row + (i - P.lo[0]);
            const T v = cor[q];
            sol[q] += double(v);
            if (hold != nullptr) { cor[q] = v + hold[q]; }
        }
    }
}

// ---------------------------------------------- colour pass without ghosts --
// Neighbour value across face f of patch cell (i,j,k) for a homogeneous colour
// pass of a level with several patches: where the ghost is covered by another
// patch (nbr >= 0, indexed like the face's Dirichlet slots) the neighbour's
// current value, else the inline closure of the cell and its inner neighbour.
// In a colour pass both are cells of the other colour or the cell itself, so
// this equals what a ghost fill before the pass would have stored.
template <typename T>
__device__ __forceinline__ T nbr_ghost (const PatchDesc& P, int f, int i, int j, int k, const T* phi, T pc, T pin,
                                        const long long* __restrict__ nbr)
{
    const long long v = nbr[P.face[f].bcval_off + face_local(P, f, i, j, k)];
    return (v >= 0) ? phi[v] : inline_ghost<T, false>(P, f, pc, pin, nullptr, 0);
}

// one colour pass of MLPoisson's Gauss-Seidel (mlpoisson_gsrb,
// AMReX_MLPoisson_3D_K.H:153-196) reading patch-face neighbours through nbr
// instead of a ghost fill.  Latency-bound on those dependent loads: capped at
// 40 registers for twelve 128-thread blocks per SM (48 warps)
template <typename T>
__global__ void __launch_bounds__(TILE_THREADS, 12)
k_gsrb_nbr (DevLevel L, Subset Sb, T* __restrict__ phi, const T* __restrict__ rhs, const long long* __restrict__ nbr,
            int rb)
{
    pdl_wait();
    pdl_trigger();
    const TileCoord c = decode_tile(L, Sb, blockIdx.x);
    const PatchDesc& P = L.P[c.p];
    const int j = c.y0 + threadIdx.y;
    if (j > P.hi[1]) { return; }
    const long long sx = P.sx, sxy = P.sxy;
    const T dhx = T(P.dhs[0]), dhy = T(P.dhs[1]), dhz = T(P.dhs[2]);
    const T gamma = T(-2.0) * (dhx + dhy + dhz);
    for (int kk = 0; kk < TILE_Z; ++kk) {
        const int k = c.z0 + kk;
        if (k > P.hi[2]) { break; }
        const int i = c.x0 + ((c.x0 + j + k + rb) & 1) + 2 * threadIdx.x;
        if (i > P.hi[0]) { continue; }
        const long long q = cidx(P, i, j, k);
        const T pc = phi[q];
        const T xm = (i == P.lo[0]) ? nbr_ghost<T>(P, 0, i, j, k, phi, pc, phi[q + 1], nbr) : phi[q - 1];
        const T xp = (i == P.hi[0]) ? nbr_ghost<T>(P, 3, i, j, k, phi, pc, phi[q - 1], nbr) : phi[q + 1];
        const T ym = (j == P.lo[1]) ? nbr_ghost<T>(P, 1, i, j, k, phi, pc, phi[q + sx], nbr) : phi[q - sx];
        const T yp = (j == P.hi[1]) ? nbr_ghost<T>(P, 4, i, j, k, phi, pc, phi[q - sx], nbr) : phi[q + sx];
        const T zm = (k == P.lo[2]) ? nbr_ghost<T>(P, 2, i, j, k, phi, pc, phi[q + sxy], nbr) : phi[q - sxy];
        const T zp = (k == P.hi[2]) ? nbr_ghost<T>(P, 5, i, j, k, phi, pc, phi[q - sxy], nbr) : phi[q + sxy];
        T cf0 = 0, cf1 = 0, cf2 = 0, cf3 = 0, cf4 = 0, cf5 = 0;
        if (i == P.lo[0]) { cf0 = T(face_cf(L, P, 0, i, j, k)); }
        if (j == P.lo[1]) { cf1 = T(face_cf(L, P, 1, i, j, k)); }
        if (k == P.lo[2]) { cf2 = T(face_cf(L, P, 2, i, j, k)); }
        if (i == P.hi[0]) { cf3 = T(face_cf(L, P, 3, i, j, k)); }
        if (j == P.hi[1]) { cf4 = T(face_cf(L, P, 4, i, j, k)); }
        if (k == P.hi[2]) { cf5 = T(face_cf(L, P, 5, i, j, k)); }
        const T g_m_d = gamma + dhx * (cf0 + cf3) + dhy * (cf1 + cf4) + dhz * (cf2 + cf5);
        const T res = rhs[q] - gamma * pc - dhx * (xm + xp) - dhy * (ym + yp) - dhz * (zm + zp);
        phi[q] = pc + relax_factor(g_m_d) * res;
    }
}

// dst = src over valid cells, with precision conversion
template <typename TD, typename TS>
__global__ void __launch_bounds__(TILE_THREADS)
k_amr_copy (DevLevel L, Subset S, TD* __restrict__ dst, const TS* __restrict__ src)
{
    pdl_wait();
    pdl_trigger();
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
            dst[q] = TD(src[q]);
        }
    }
}

} // namespace mlmg
