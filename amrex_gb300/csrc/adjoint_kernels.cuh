// Adjoint of the cell-centred operator (no counterpart in the reference).
//
// For J(phi) with A phi = f, the gradients are dJ/df = lambda and
// dJ/db = -lambda^T (dA/db) phi, where A^T lambda = dJ/dphi.
//
// A is symmetric except for the Dirichlet ghost closure of applyBC
// (mllinop_apply_bc_x, AMReX_MLLinOp_K.H:74-320): the ghost of boundary cell
// c0 is g = sum_{m>=1} coef[m] x(c0 + (m-1) step) (homogeneous part), so the
// row of c0 couples to the cells at distance 1..nx-2 from the face with
// weight w * coef[m], where w is the ghost's weight in the row
// (ABec: -beta*dxinv^2*b_face; Poisson: +dxinv^2).  A^T therefore differs
// from A only there: the row of c0 keeps only its coef[1] self term, and the
// row of the cell at distance t gains w * coef[t+1] * x(c0).
//
// The adjoint solve reuses the forward MLMG V-cycle as the correction
// operator and evaluates the outer residual g - A^T lambda with this kernel
// (iterative refinement on A^T with an A-preconditioner).
#pragma once

#include "stage_kernels.cuh"
#include "stencil_kernels.cuh"

namespace mlmg {

// weight of the ghost of face f in the row of boundary cell q0
template <bool ABEC>
__device__ __forceinline__ double ghost_weight (const PatchDesc& P, int f, long long q0, const double* __restrict__ bx,
                                                const double* __restrict__ by, const double* __restrict__ bz)
{
    const int d = f % 3;
    if constexpr (ABEC) {
        const double* b = (d == 0) ? bx : ((d == 1) ? by : bz);
        const long long st = (d == 0) ? 1 : ((d == 1) ? (long long)P.sx : P.sxy);
        const double bf = (f < 3) ? b[q0] : b[q0 + st];
        return -P.dha[d] * bf;
    } else {
        return P.dha[d];
    }
}

// Periodic domain faces: the two stored copies of a face on opposite sides
// of a periodic direction are separate entries (row 0 reads b[0], row n-1
// reads b[n]), so A couples cells 0 and n-1 unsymmetrically when they differ.
// For every periodic ghost cell (a copy tag with a non-zero shift) this puts
// the face coefficient that the image cell's row uses for the same coupling
// at the ghost's index.  ABec only.
static __global__ void k_partner_faces (DevLevel L, GhostWork W, const double* __restrict__ bx,
                                 const double* __restrict__ by, const double* __restrict__ bz,
                                 double* __restrict__ out)
{
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= W.ntagcells) { return; }
    const int w = bsearch_ll<int>(W.tstart, W.ntag, t);
    const CopyTag& C = W.tags[w];
    if (C.shift[0] == 0 && C.shift[1] == 0 && C.shift[2] == 0) { return; }
    const long long u = t - W.tstart[w];
    const int nx = C.box.hi[0] - C.box.lo[0] + 1, ny = C.box.hi[1] - C.box.lo[1] + 1;
    const int i = C.box.lo[0] + (int)(u % nx);
    const int j = C.box.lo[1] + (int)((u / nx) % ny);
    const int k = C.box.lo[2] + (int)(u / ((long long)nx * ny));
    const PatchDesc& D = L.P[C.dst];
    const PatchDesc& Sp = L.P[C.src];
    const long long qd = cidx(D, i, j, k);
    const long long qs = cidx(Sp, i - C.shift[0], j - C.shift[1], k - C.shift[2]);
    if (i < D.lo[0]) { out[qd] = bx[qs + 1]; }
    else if (i > D.hi[0]) { out[qd] = bx[qs]; }
    else if (j < D.lo[1]) { out[qd] = by[qs + Sp.sx]; }
    else if (j > D.hi[1]) { out[qd] = by[qs]; }
    else if (k < D.lo[2]) { out[qd] = bz[qs + Sp.sxy]; }
    else { out[qd] = bz[qs]; }
}

// r = g - A^T x (FP64, homogeneous BCs; x carries ghost values from the
// homogeneous applyBC, including copies between patches); max|r| per solve by
// atomicMax into norm[solve] (zeroed beforehand)
template <typename TO, bool ABEC>
__global__ void __launch_bounds__(TILE_THREADS)
k_residual_transpose (DevLevel L, Subset S, TO* __restrict__ r, const double* __restrict__ x,
                      const double* __restrict__ g, const double* __restrict__ a, const double* __restrict__ bx,
                      const double* __restrict__ by, const double* __restrict__ bz,
                      const double* __restrict__ partner, double* __restrict__ norm)
{
    __shared__ double sm[32];
    const TileCoord c = decode_tile(L, S, blockIdx.x);
    const PatchDesc& P = L.P[c.p];
    const int j = c.y0 + threadIdx.y;
    double mx = 0.0;
    if (j <= P.hi[1]) {
        for (int kk = 0; kk < TILE_Z; ++kk) {
            const int k = c.z0 + kk;
            if (k > P.hi[2]) { break; }
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                const int i = c.x0 + threadIdx.x + 32 * h;
                if (i > P.hi[0]) { continue; }
                const long long q = cidx(P, i, j, k);
                double row = adotx_cell<double, ABEC>(P, q, x, a, bx, by, bz);
                const int ijk[3] = {i, j, k};
                for (int f = 0; f < 6; ++f) {
                    const FaceBC& F = P.face[f];
                    const int d = f % 3;
                    if constexpr (ABEC) {
                        // periodic image across a domain face: the image row's coefficient
                        const bool at_face = (f < 3) ? ijk[d] == P.lo[d] : ijk[d] == P.hi[d];
                        if (partner != nullptr && at_face && F.on_domain) {
                            int gi = ijk[0], gj = ijk[1], gk = ijk[2];
                            const int gd = (f < 3) ? P.lo[d] - 1 : P.hi[d] + 1;
                            if (d == 0) { gi = gd; } else if (d == 1) { gj = gd; } else { gk = gd; }
                            if (face_mask(L, P, f, gi, gj, gk) == MASK_COVERED) {
                                const long long st = (d == 0) ? 1 : ((d == 1) ? (long long)P.sx : P.sxy);
                                const double* b = (d == 0) ? bx : ((d == 1) ? by : bz);
                                const long long qg = (f < 3) ? q - st : q + st;
                                const double own = (f < 3) ? b[q] : b[q + st];
                                row += -P.dha[d] * (partner[qg] - own) * x[qg];
                            }
                        }
                    }
                    if (F.type != BC_DIRICHLET || F.nx < 3) { continue; }
                    const int t = (f < 3) ? ijk[d] - P.lo[d] : P.hi[d] - ijk[d];   // distance from the face
                    if (t > F.nx - 2) { continue; }
                    const long long stride = (d == 0) ? 1 : ((d == 1) ? (long long)P.sx : P.sxy);
                    const long long step = (f < 3) ? stride : -stride;           // into the patch
                    const long long q0 = q - t * step;                           // boundary cell
                    int gi = ijk[0], gj = ijk[1], gk = ijk[2];                   // its ghost neighbour
                    const int gd = (f < 3) ? P.lo[d] - 1 : P.hi[d] + 1;
                    if (d == 0) { gi = gd; } else if (d == 1) { gj = gd; } else { gk = gd; }
                    if (face_mask(L, P, f, gi, gj, gk) <= 0) { continue; }
                    const double w = ghost_weight<ABEC>(P, f, q0, bx, by, bz);
                    if (t == 0) {
                        double off = 0.0;
                        for (int m = 2; m < F.nx; ++m) { off += F.coef[m] * x[q0 + (m - 1) * step]; }
                        row -= w * off;
                    } else {
                        row += w * F.coef[t + 1] * x[q0];
                    }
                }
                const double v = g[q] - row;
                r[q] = TO(v);
                mx = max_nan(mx, fabs(v));
            }
        }
    }
    if (norm != nullptr) {
        const double red = block_reduce(mx, RED_MAXABS, sm);
        if (threadIdx.x == 0 && threadIdx.y == 0) { atomic_max_nonneg(&norm[P.solve], red); }
    }
}

// Fused face-gradient contraction.  For the face between cells c-1 and c
// along d:  dJ/db = -beta*dxinv_d^2 * (phi_c - phi_{c-1}) * (lam_c - lam_{c-1})
// with phi's ghosts from the inhomogeneous applyBC (the forward solution's
// boundary values, periodic images) and lam = 0 outside the domain: a face on
// the domain boundary is read by the one row inside, so its term is
// -beta*dxinv^2 * lam_0 * (phi_0 - phi_ghost); the two stored faces of a
// periodic direction are separate entries, each read by one row.  Faces
// lo..hi+1 of every patch, stored at the low-side cell index like the b
// coefficients; a face shared by two boxes gets its full (two-row) value in
// both boxes' copies.
// dJ/da = -alpha * lam * phi per cell.  MLABecLaplacian only.
static __global__ void __launch_bounds__(TILE_THREADS)
k_face_grad (DevLevel L, Subset S, const double* __restrict__ phi, const double* __restrict__ lam,
             double* __restrict__ gx, double* __restrict__ gy, double* __restrict__ gz, double* __restrict__ ga)
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
            const int ijk[3] = {i, j, k};
            const double pc = phi[q], lc = lam[q];
            double* gout[3] = {gx, gy, gz};
            for (int d = 0; d < 3; ++d) {
                if (gout[d] == nullptr) { continue; }
                const long long st = (d == 0) ? 1 : ((d == 1) ? (long long)P.sx : P.sxy);
                const double fac = -P.beta * P.dxinv[d] * P.dxinv[d];
                // low face of the cell
                const double lm = (ijk[d] == P.lo[d] && P.face[d].on_domain) ? 0.0 : lam[q - st];
                gout[d][q] = fac * (pc - phi[q - st]) * (lc - lm);
                // high face of the last cell
                if (ijk[d] == P.hi[d]) {
                    const double lp = P.face[d + 3].on_domain ? 0.0 : lam[q + st];
                    gout[d][q + st] = fac * (phi[q + st] - pc) * (lp - lc);
                }
            }
            if (ga != nullptr) { ga[q] = -P.alpha * lc * pc; }
        }
    }
}

} // namespace mlmg
