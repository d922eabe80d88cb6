// Face gradients and fluxes of a solution, the step a caller runs right after
// MLMG::solve:
//   grad (mode 0): MLMG::getGradSolution -> MLCellLinOpT::compGrad
//                  (AMReX_MLCellLinOp.H:1392-1442): dxinv * (s_c - s_{c-1})
//   flux (mode 1): MLMG::getFluxes -> MLCellABecLapT::getFluxes
//                  (AMReX_MLCellABecLap.H:272-291): compFlux with
//                  mlabeclap_flux_x (AMReX_MLABecLap_3D_K.H:79-97),
//                  -(beta*dxinv) * b * (s_c - s_{c-1}), then scaled by
//                  1/beta unless that is 1; MLPoisson (mlpoisson_flux_x,
//                  AMReX_MLPoisson_3D_K.H:36-50) gives dxinv * (s_c - s_{c-1})
//                  scaled by 1/getBScalar() = -1.
// The solution's ghosts are those of applyBC with the level's boundary values.
// Every patch writes its faces lo..hi+1 (low-side cell index storage).
#pragma once

#include "kernels.cuh"

namespace mlmg {

template <int MODE, bool ABEC>
__device__ __forceinline__ double face_value (const PatchDesc& P, int d, double ds, const double* __restrict__ b,
                                              long long qf)
{
    const double dxi = P.dxinv[d];
    if constexpr (MODE == 0) {
        return dxi * ds;
    } else if constexpr (ABEC) {
        const double fac = P.beta * dxi;
        double v = -fac * b[qf] * ds;
        const double betainv = 1.0 / P.beta;
        if (betainv != 1.0) { v *= betainv; }
        return v;
    } else {
        double v = dxi * ds;
        v *= -1.0;
        return v;
    }
}

template <int MODE, bool ABEC>
__global__ void __launch_bounds__(TILE_THREADS)
k_face_flux (DevLevel L, Subset S, const double* __restrict__ phi, const double* __restrict__ bx,
             const double* __restrict__ by, const double* __restrict__ bz, double* __restrict__ fx,
             double* __restrict__ fy, double* __restrict__ fz)
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
            const double pc = phi[q];
            double* out[3] = {fx, fy, fz};
            const double* bc[3] = {bx, by, bz};
#pragma unroll
            for (int d = 0; d < 3; ++d) {
                const long long st = (d == 0) ? 1 : ((d == 1) ? (long long)P.sx : P.sxy);
                out[d][q] = face_value<MODE, ABEC>(P, d, pc - phi[q - st], bc[d], q);
                if (ijk[d] == P.hi[d]) {
                    out[d][q + st] = face_value<MODE, ABEC>(P, d, phi[q + st] - pc, bc[d], q + st);
                }
            }
        }
    }
}

} // namespace mlmg
