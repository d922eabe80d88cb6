// Kernels of the mixed-precision path in "stencil form".
//
// The ABec operator A x = alpha a x - sum_d dh_d [b(+)(x(+)-x) - b(-)(x-x(-))]
// is rewritten with precomputed per-level arrays
//     D  = alpha a + sum_d dh_d (b(-) + b(+))      (the smoother's gamma)
//     s_d = dh_d b_d                                (scaled face coefficients)
// as  A x = D x - sum (s(-) x(-) + s(+) x(+)).  The residual then costs
// 1 multiply + 6 FMAs + 1 subtraction per cell instead of ~18 FP64
// operations (GB300's FP64 rate is ~1.25 TFLOP/s, so the FP64 residual of the
// refinement loop is FP64-bound in the reference form), and the FP32 smoother
// reads 6 arrays instead of 7.  MLPoisson is the same with constant D and s.
//
// Where every face of a level's patches is a physical or coarse/fine face
// with a Dirichlet closure of at most 3 points (maxorder <= 3), Neumann or
// reflect_odd, the ghost value is a function of the two cells next to the
// face and is computed inline (INLINE_BC), so no separate ghost-fill launch
// is needed.  In a colour pass those two cells are the cell being updated and
// a cell of the other colour, neither of which another thread writes in the
// same pass, so the inline value equals the ghost applyBC would have stored.
#pragma once

#include "stage_kernels.cuh"

namespace mlmg {


// omega / g for the Gauss-Seidel update (omega = 1.15, abec_gsrb).  The FP32
// V-cycle is only a preconditioner of the FP64 refinement, so its division
// uses the fast single-precision intrinsic; FP64 keeps IEEE division.
__device__ __forceinline__ float relax_factor (float g) { return __fdividef(1.15f, g); }
__device__ __forceinline__ double relax_factor (double g) { return 1.15 / g; }

struct StencilPtrs {            // per-level stencil arrays (null for constant coefficients)
    const void* D;
    const void* sx;
    const void* sy;
    const void* sz;
};

// build D, s in FP64 from the FP64 a, bX, bY, bZ of a level; optional FP32 copies
static __global__ void __launch_bounds__(TILE_THREADS)
k_build_stencil (DevLevel L, Subset S, const double* __restrict__ a, const double* __restrict__ bx,
                 const double* __restrict__ by, const double* __restrict__ bz, double* __restrict__ D,
                 double* __restrict__ sx, double* __restrict__ sy, double* __restrict__ sz,
                 float* __restrict__ D32, float* __restrict__ sx32, float* __restrict__ sy32,
                 float* __restrict__ sz32)
{
    const TileCoord c = decode_tile(L, S, blockIdx.x);
    const PatchDesc& P = L.P[c.p];
    const int j = c.y0 + threadIdx.y;
    if (j > P.hi[1]) { return; }
    const double dhx = P.dha[0], dhy = P.dha[1], dhz = P.dha[2];
    for (int kk = 0; kk < TILE_Z; ++kk) {
        const int k = c.z0 + kk;
        if (k > P.hi[2]) { break; }
        for (int h = 0; h < 2; ++h) {
            const int i = c.x0 + threadIdx.x + 32 * h;
            if (i > P.hi[0]) { continue; }
            const long long q = cidx(P, i, j, k);
            const double d = P.alpha * a[q] + dhx * (bx[q] + bx[q + 1]) + dhy * (by[q] + by[q + P.sx])
                           + dhz * (bz[q] + bz[q + P.sxy]);
            D[q] = d;
            if (D32) { D32[q] = (float)d; }
            // faces: own low face, plus the high face at the patch's high end
            auto put = [&] (double* s, float* s32, long long qq, double v) {
                s[qq] = v;
                if (s32) { s32[qq] = (float)v; }
            };
            put(sx, sx32, q, dhx * bx[q]);
            put(sy, sy32, q, dhy * by[q]);
            put(sz, sz32, q, dhz * bz[q]);
            if (i == P.hi[0]) { put(sx, sx32, q + 1, dhx * bx[q + 1]); }
            if (j == P.hi[1]) { put(sy, sy32, q + P.sx, dhy * by[q + P.sx]); }
            if (k == P.hi[2]) { put(sz, sz32, q + P.sxy, dhz * bz[q + P.sxy]); }

        }
    }
}

// ghost value of the neighbour across face f of cell (i,j,k) on a patch face
// (the cell itself is pc, the next inner cell pin): Dirichlet closure with
// nx <= 3 points, Neumann, reflect_odd (mllinop_apply_bc_*,
// AMReX_MLLinOp_K.H:74-320); bq indexes the face's Dirichlet values
template <typename T, bool INHOMOG>
__device__ __forceinline__ T inline_ghost (const PatchDesc& P, int f, T pc, T pin, const double* bcval, long long bq)
{
    const FaceBC& F = P.face[f];
    if (F.type == BC_DIRICHLET) {
        T g = (F.nx >= 2) ? pc * T(F.coef[1]) : T(0);
        if (F.nx >= 3) { g += pin * T(F.coef[2]); }
        if constexpr (INHOMOG) {
            if (bcval != nullptr) { g += T(bcval[F.bcval_off + bq]) * T(F.coef[0]); }
        }
        return g;
    }
    if (F.type == BC_NEUMANN) { return pc; }
    if (F.type == BC_REFLECT_ODD) { return -pc; }
    return T(0);
}

// local index of the face cell of face f for the patch cell (i,j,k) next to it
template <typename Geo>
__device__ __forceinline__ long long face_local (const Geo& P, int f, int i, int j, int k)
{
    const int d = f % 3;
    const int nx = P.hi[0] - P.lo[0] + 1, ny = P.hi[1] - P.lo[1] + 1;
    if (d == 0) { return (long long)(k - P.lo[2]) * ny + (j - P.lo[1]); }
    if (d == 1) { return (long long)(k - P.lo[2]) * nx + (i - P.lo[0]); }
    return (long long)(j - P.lo[1]) * nx + (i - P.lo[0]);
}

// the six neighbours of cell q (ghosts inline at patch faces when INLINE_BC)
// (Geo: the patch's geometry, PatchDesc or PatchGeom; PD: its descriptor,
// whose face BCs the closures read)
template <typename T, bool INLINE_BC, bool INHOMOG, typename Geo>
__device__ __forceinline__ void neighbours (const Geo& P, const PatchDesc& PD, int i, int j, int k, long long q,
                                            const T* phi, T pc, const double* bcval,
                                            T& xm, T& xp, T& ym, T& yp, T& zm, T& zp)
{
    const long long sx = P.sx, sxy = P.sxy;
    if constexpr (!INLINE_BC) {
        xm = phi[q - 1]; xp = phi[q + 1]; ym = phi[q - sx]; yp = phi[q + sx]; zm = phi[q - sxy]; zp = phi[q + sxy];
    } else {
        xm = (i == P.lo[0]) ? inline_ghost<T, INHOMOG>(PD, 0, pc, phi[q + 1], bcval, face_local(P, 0, i, j, k)) : phi[q - 1];
        xp = (i == P.hi[0]) ? inline_ghost<T, INHOMOG>(PD, 3, pc, phi[q - 1], bcval, face_local(P, 3, i, j, k)) : phi[q + 1];
        ym = (j == P.lo[1]) ? inline_ghost<T, INHOMOG>(PD, 1, pc, phi[q + sx], bcval, face_local(P, 1, i, j, k)) : phi[q - sx];
        yp = (j == P.hi[1]) ? inline_ghost<T, INHOMOG>(PD, 4, pc, phi[q - sx], bcval, face_local(P, 4, i, j, k)) : phi[q + sx];
        zm = (k == P.lo[2]) ? inline_ghost<T, INHOMOG>(PD, 2, pc, phi[q + sxy], bcval, face_local(P, 2, i, j, k)) : phi[q - sxy];
        zp = (k == P.hi[2]) ? inline_ghost<T, INHOMOG>(PD, 5, pc, phi[q - sxy], bcval, face_local(P, 5, i, j, k)) : phi[q + sxy];
    }
}

template <typename T, bool VARC>
struct Coef7 {
    T d, sxl, sxh, syl, syh, szl, szh;
};

template <typename T, bool VARC, typename Geo>
__device__ __forceinline__ Coef7<T, VARC> load_coef (const Geo& P, long long q, const StencilPtrs& S)
{
    Coef7<T, VARC> c;
    if constexpr (VARC) {
        const T* D = static_cast<const T*>(S.D);
        const T* sx = static_cast<const T*>(S.sx);
        const T* sy = static_cast<const T*>(S.sy);
        const T* sz = static_cast<const T*>(S.sz);
        c.d = D[q];
        c.sxl = sx[q]; c.sxh = sx[q + 1];
        c.syl = sy[q]; c.syh = sy[q + P.sx];
        c.szl = sz[q]; c.szh = sz[q + P.sxy];
    } else {
        // MLPoisson: A x = sum dh (x(-) - 2x + x(+)) = D x - sum s x(+-) with
        // D = -2 sum dh, s = -dh
        const T dhx = T(P.dha[0]), dhy = T(P.dha[1]), dhz = T(P.dha[2]);
        c.d = T(-2.0) * (dhx + dhy + dhz);
        c.sxl = c.sxh = -dhx; c.syl = c.syh = -dhy; c.szl = c.szh = -dhz;
    }
    return c;
}

// red-black Gauss-Seidel update of one cell in stencil form
template <typename T, bool VARC, bool INLINE_BC>
__device__ __forceinline__ void gsrb_s_cell (const DevLevel& L, const PatchDesc& P, int i, int j, int k,
                                             T* __restrict__ phi, const T* __restrict__ rhs, const StencilPtrs& S)
{
    const long long q = cidx(P, i, j, k);
    const T pc = phi[q];
    T xm, xp, ym, yp, zm, zp;
    neighbours<T, INLINE_BC, false>(P, P, i, j, k, q, phi, pc, nullptr, xm, xp, ym, yp, zm, zp);
    const Coef7<T, VARC> c = load_coef<T, VARC>(P, q, S);
    T gmd = c.d;
    const bool face = (i == P.lo[0]) | (i == P.hi[0]) | (j == P.lo[1]) | (j == P.hi[1]) | (k == P.lo[2]) | (k == P.hi[2]);
    if (face) {
        T corr = 0;
        if (i == P.lo[0]) { corr += c.sxl * T(face_cf(L, P, 0, i, j, k)); }
        if (i == P.hi[0]) { corr += c.sxh * T(face_cf(L, P, 3, i, j, k)); }
        if (j == P.lo[1]) { corr += c.syl * T(face_cf(L, P, 1, i, j, k)); }
        if (j == P.hi[1]) { corr += c.syh * T(face_cf(L, P, 4, i, j, k)); }
        if (k == P.lo[2]) { corr += c.szl * T(face_cf(L, P, 2, i, j, k)); }
        if (k == P.hi[2]) { corr += c.szh * T(face_cf(L, P, 5, i, j, k)); }
        gmd -= corr;
    }
    const T rho = c.sxl * xm + c.sxh * xp + c.syl * ym + c.syh * yp + c.szl * zm + c.szh * zp;
    const T res = rhs[q] - (c.d * pc - rho);
    phi[q] = pc + relax_factor(gmd) * res;
}

template <typename T, bool VARC, bool INLINE_BC>
__global__ void __launch_bounds__(TILE_THREADS)
k_gsrb_s (DevLevel L, Subset Sb, T* __restrict__ phi, const T* __restrict__ rhs, StencilPtrs S, int rb)
{
    pdl_wait();
    pdl_trigger();
    const TileCoord c = decode_tile(L, Sb, blockIdx.x);
    const PatchDesc& P = L.P[c.p];
    const int j = c.y0 + threadIdx.y;
    if (j > P.hi[1]) { return; }
    for (int kk = 0; kk < TILE_Z; ++kk) {
        const int k = c.z0 + kk;
        if (k > P.hi[2]) { break; }
        const int i = c.x0 + ((c.x0 + j + k + rb) & 1) + 2 * threadIdx.x;
        if (i <= P.hi[0]) { gsrb_s_cell<T, VARC, INLINE_BC>(L, P, i, j, k, phi, rhs, S); }
    }
}

__device__ __forceinline__ void atomic_max_nonneg (double* addr, double v)
{
    // max of non-negative doubles == max of their bit patterns
    atomicMax(reinterpret_cast<unsigned long long*>(addr), (unsigned long long)__double_as_longlong(v));
}

// block maximum of non-negative doubles held as bit patterns (integer
// compares; a NaN pattern orders above every number), valid in thread 0
__device__ __forceinline__ unsigned long long block_max_bits (unsigned long long v, double* sm)
{
    unsigned long long* smb = reinterpret_cast<unsigned long long*>(sm);
    const int lane = (threadIdx.y * blockDim.x + threadIdx.x) & 31;
    const int warp = (threadIdx.y * blockDim.x + threadIdx.x) >> 5;
    const int nwarp = (blockDim.x * blockDim.y + 31) >> 5;
    for (int o = 16; o > 0; o >>= 1) {
        const unsigned long long w = __shfl_down_sync(0xffffffffu, v, o);
        v = (w > v) ? w : v;
    }
    __syncthreads();
    if (lane == 0) { smb[warp] = v; }
    __syncthreads();
    unsigned long long r = 0ull;
    if (warp == 0) {
        r = (lane < nwarp) ? smb[lane] : 0ull;
        for (int o = 16; o > 0; o >>= 1) {
            const unsigned long long w = __shfl_down_sync(0xffffffffu, r, o);
            r = (w > r) ? w : r;
        }
    }
    return r;
}

// r = b - A x in stencil form (the mixed-precision paths' residuals; the FP64
// path keeps the reference's operation order in k_residual); optional
// per-solve max|r| by atomicMax into norm[solve] (zeroed beforehand; a
// maximum does not depend on the order); optional FP32 copy of an FP64 r
// (r32, rounded on the integer pipe)
template <typename T, typename TO, bool VARC, bool INLINE_BC, bool INHOMOG>
__global__ void __launch_bounds__(TILE_THREADS)
k_residual_s (DevLevel L, Subset Sb, TO* __restrict__ r, const T* __restrict__ x, const T* __restrict__ b,
              StencilPtrs S, const double* __restrict__ bcval, double* __restrict__ norm,
              float* __restrict__ r32)
{
    __shared__ double sm[32];
    const TileCoord c = decode_tile(L, Sb, blockIdx.x);
    const PatchDesc& P = L.P[c.p];
    pdl_wait();
    pdl_trigger();
    const int j = c.y0 + threadIdx.y;
    // MLPoisson: the constant stencil, formed once (the cell loop would
    // otherwise repeat its FP64 arithmetic for every cell)
    Coef7<T, VARC> cc{};
    if constexpr (!VARC) { cc = load_coef<T, false>(P, 0, S); }
    float mxf = 0.f;                     // FP32: max |r|
    unsigned long long mxb = 0ull;       // FP64: max |r| as the max of the sign-cleared bit patterns
    if (j <= P.hi[1]) {
        for (int kk = 0; kk < TILE_Z; ++kk) {
            const int k = c.z0 + kk;
            if (k > P.hi[2]) { break; }
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                const int i = c.x0 + threadIdx.x + 32 * h;
                if (i > P.hi[0]) { continue; }
                const long long q = cidx(P, i, j, k);
                const T xc = x[q];
                T xm, xp, ym, yp, zm, zp;
                neighbours<T, INLINE_BC, INHOMOG>(P, P, i, j, k, q, x, xc, bcval, xm, xp, ym, yp, zm, zp);
                Coef7<T, VARC> cf;
                if constexpr (VARC) { cf = load_coef<T, true>(P, q, S); } else { cf = cc; }
                T v;
                if constexpr (std::is_same_v<T, double>) {
                    // seven FMAs (b - D x, then + s x_nb) and nothing else on
                    // the FP64 pipe, whose rate bounds this kernel on GB300:
                    // the FP32 copy and the max-norm are integer operations
                    v = fma(-cf.d, xc, b[q]);
                    v = fma(cf.sxl, xm, v); v = fma(cf.sxh, xp, v);
                    v = fma(cf.syl, ym, v); v = fma(cf.syh, yp, v);
                    v = fma(cf.szl, zm, v); v = fma(cf.szh, zp, v);
                } else {
                    const T nb = cf.sxl * xm + cf.sxh * xp + cf.syl * ym + cf.syh * yp + cf.szl * zm + cf.szh * zp;
                    v = b[q] - (cf.d * xc - nb);
                }
                if constexpr (std::is_same_v<T, double> && std::is_same_v<TO, float>) {
                    r[q] = d2f_bits(v);
                } else {
                    r[q] = TO(v);
                }
                if constexpr (std::is_same_v<TO, double>) {
                    if (r32 != nullptr) { r32[q] = d2f_bits(v); }
                }
                if constexpr (std::is_same_v<T, double>) {
                    // integer max on the bit patterns of |v| keeps the FP64 pipe
                    // free (non-negative doubles order like their bits; a NaN
                    // residual orders above every number and reaches the norm)
                    const unsigned long long ab = abs_bits(v);
                    mxb = (ab > mxb) ? ab : mxb;
                } else if (norm != nullptr) {
                    // FP32 max of |v| (NaN kept), widened once per block
                    const float av = fabsf(v);
                    mxf = (av > mxf || av != av) ? av : mxf;
                }
            }
        }
    }
    if (norm != nullptr) {
        double red;
        if constexpr (std::is_same_v<T, double>) {
            red = __longlong_as_double((long long)block_max_bits(mxb, sm));
        } else {
            red = block_reduce((double)mxf, RED_MAXABS, sm);
        }
        if (threadIdx.x == 0 && threadIdx.y == 0) { atomic_max_nonneg(&norm[P.solve], red); }
    }
}

} // namespace mlmg
