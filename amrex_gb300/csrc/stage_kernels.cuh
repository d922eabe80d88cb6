// Global kernels of the V-cycle stages, ghost fill, reductions, transfers.
#pragma once

#include "kernels.cuh"

namespace mlmg {

// FP32 <-> FP64 conversions and |x| of an FP64 value on the integer pipe.
// GB300's FP64 pipe completes 2 operations per clock per SM, and a hardware
// conversion (or the predicated-off conversion of a guarded fallback, or an
// FP64 absolute value) occupies it like arithmetic does, so the kernels that
// FP64 bounds (the outer residual, phi += cor) assemble these results from
// the IEEE 754 bit fields instead.  Each equals the hardware result for every
// finite input and for +-Inf (a NaN stays a quiet NaN with the top bits of
// its payload); mlmg_check_bit_conversions compares them on the device.

// binary32 -> binary64 (exact): rebias the exponent by 1023 - 127 and move the
// 23 fraction bits to the top of the 52; a subnormal is normalised first
__device__ __forceinline__ double f2d_bits (float c)
{
    const unsigned u = __float_as_uint(c);
    const unsigned sign = u & 0x80000000u;
    const unsigned e = (u >> 23) & 0xffu;
    unsigned m = u & 0x7fffffu;
    unsigned ed;
    if (e == 0u) {
        if (m == 0u) { return __hiloint2double((int)sign, 0); }
        const int p = 31 - __clz((int)m);              // leading one of the subnormal's fraction
        ed = (unsigned)(p + 1023 - 149);               // value = 1.f x 2^(p - 149)
        m = (m << (23 - p)) & 0x7fffffu;
    } else if (e == 255u) {
        ed = 2047u;
        if (m != 0u) { m |= 0x400000u; }               // quiet NaN
    } else {
        ed = e + 896u;
    }
    return __hiloint2double((int)(sign | (ed << 20) | (m >> 3)), (int)(m << 29));
}

// binary64 -> binary32, round to nearest even: keep the top 23 fraction bits
// and round on the 29 dropped ones (above half, or exactly half with an odd
// kept part); a carry moves into the exponent (the largest finite float
// rounds up to Inf).  Results below the normal range shift the 53-bit
// significand right by the subnormal distance and round the same way.
__device__ __forceinline__ float d2f_bits (double v)
{
    const unsigned hi = (unsigned)__double2hiint(v), lo = (unsigned)__double2loint(v);
    const unsigned sign = hi & 0x80000000u;
    const unsigned E = (hi >> 20) & 0x7ffu;
    const int e = (int)E - 896;                        // binary32 biased exponent
    unsigned f;
    if (e >= 1 && e <= 254) {
        f = ((unsigned)e << 23) | ((hi & 0xfffffu) << 3) | (lo >> 29);
        const unsigned rem = lo & 0x1fffffffu;
        f += (rem > 0x10000000u || (rem == 0x10000000u && (f & 1u))) ? 1u : 0u;
    } else if (E == 2047u) {
        f = (((hi & 0xfffffu) | lo) != 0u) ? (0x7fc00000u | ((hi & 0xfffffu) << 3) | (lo >> 29)) : 0x7f800000u;
    } else if (e > 254) {
        f = 0x7f800000u;                               // overflow
    } else {
        const int sh = 926 - (int)E;                   // value = M x 2^-sh in units of 2^-149
        if (sh >= 64) {
            f = 0u;
        } else {
            const unsigned long long M = (1ull << 52) | ((unsigned long long)(hi & 0xfffffu) << 32) | lo;
            const unsigned long long q = M >> sh;
            const unsigned long long rem = M & ((1ull << sh) - 1ull);
            const unsigned long long half = 1ull << (sh - 1);
            f = (unsigned)q + ((rem > half || (rem == half && (q & 1ull))) ? 1u : 0u);
        }
    }
    return __uint_as_float(sign | f);
}

// the bit pattern of |v| as an integer (non-negative doubles order like their
// bits; a NaN orders above every number), cleared on the high word so that
// it stays an integer operation rather than an FP64 absolute value
__device__ __forceinline__ unsigned long long abs_bits (double v)
{
    return ((unsigned long long)((unsigned)__double2hiint(v) & 0x7fffffffu) << 32) | (unsigned)__double2loint(v);
}

// TD(v) with the FP32 <-> FP64 cases on the integer pipe
template <typename TD, typename TS>
__device__ __forceinline__ TD convert (TS v)
{
    if constexpr (std::is_same_v<TD, double> && std::is_same_v<TS, float>) {
        return f2d_bits(v);
    } else if constexpr (std::is_same_v<TD, float> && std::is_same_v<TS, double>) {
        return d2f_bits(v);
    } else {
        return TD(v);
    }
}

// ------------------------------------------------------------ reductions --
enum RedOp : int { RED_MAXABS = 0, RED_DOT = 1, RED_SUM = 2 };

// maximum that keeps a NaN (fmax drops it), so that a NaN in a residual or a
// right-hand side reaches the norm and the solve reports it
__device__ __forceinline__ double max_nan (double a, double b) { return (a > b || a != a) ? a : b; }

__device__ __forceinline__ double red_combine (int op, double a, double b)
{
    return (op == RED_MAXABS) ? max_nan(a, b) : a + b;
}

// deterministic block reduction over TILE_THREADS (or any multiple of 32 up to 1024) threads
__device__ __forceinline__ double block_reduce (double v, int op, double* sm)
{
    const int lane = (threadIdx.y * blockDim.x + threadIdx.x) & 31;
    const int warp = (threadIdx.y * blockDim.x + threadIdx.x) >> 5;
    const int nwarp = (blockDim.x * blockDim.y + 31) >> 5;
    for (int o = 16; o > 0; o >>= 1) { v = red_combine(op, v, __shfl_down_sync(0xffffffffu, v, o)); }
    __syncthreads();
    if (lane == 0) { sm[warp] = v; }
    __syncthreads();
    double r = (op == RED_MAXABS) ? 0.0 : 0.0;
    if (warp == 0) {
        r = (lane < nwarp) ? sm[lane] : 0.0;
        for (int o = 16; o > 0; o >>= 1) { r = red_combine(op, r, __shfl_down_sync(0xffffffffu, r, o)); }
    }
    return r;   // valid in thread 0
}

// --------------------------------------------------------------- smoother --
template <typename T, bool ABEC>
__global__ void __launch_bounds__(TILE_THREADS)
k_gsrb (DevLevel L, Subset S, T* __restrict__ phi, const T* __restrict__ rhs, const T* __restrict__ a,
        const T* __restrict__ bx, const T* __restrict__ by, const T* __restrict__ bz, int rb)
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
        const int i = c.x0 + ((c.x0 + j + k + rb) & 1) + 2 * threadIdx.x;
        if (i <= P.hi[0]) { gsrb_cell<T, ABEC>(L, P, i, j, k, phi, rhs, a, bx, by, bz); }
    }
}

// r = b - A x (b != null) or r = A x (b == null); optional per-block max|r|
template <typename T, typename TO, bool ABEC>
__global__ void __launch_bounds__(TILE_THREADS)
k_residual (DevLevel L, Subset S, TO* __restrict__ r, const T* __restrict__ x, const T* __restrict__ b,
            const T* __restrict__ a, const T* __restrict__ bx, const T* __restrict__ by,
            const T* __restrict__ bz, double* __restrict__ partial)
{
    pdl_wait();
    pdl_trigger();
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
                const T ax = adotx_cell<T, ABEC>(P, q, x, a, bx, by, bz);
                // MF::Xpay(resid, -1, b): resid = b + (-1)*resid
                const T v = (b != nullptr) ? T(b[q] + T(-1.0) * ax) : ax;
                r[q] = TO(v);
                mx = max_nan(mx, fabs((double)v));
            }
        }
    }
    if (partial != nullptr) {
        const double red = block_reduce(mx, RED_MAXABS, sm);
        if (threadIdx.x == 0 && threadIdx.y == 0) { partial[blockIdx.x] = red; }
    }
}

// ------------------------------------------------------------- ghost fill --
struct GhostWork {
    const int2* faces;          // (patch, face)
    const long long* fstart;    // prefix over face cell counts (nface+1)
    int nface;
    const CopyTag* tags;
    const long long* tstart;    // prefix over tag cell counts (ntag+1)
    int ntag;
    long long nfacecells, ntagcells;
};

template <typename P_>
__device__ __forceinline__ int bsearch_ll (const long long* start, int n, long long v)
{
    int lo = 0, hi = n - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (start[mid] <= v) { lo = mid; } else { hi = mid - 1; }
    }
    return lo;
}

// face-cell coordinates of local index u on face f of patch P (the outside layer)
__device__ __forceinline__ void face_cell (const PatchDesc& P, int f, long long u, int& i, int& j, int& k)
{
    const int d = f % 3;
    const unsigned nx = P.hi[0] - P.lo[0] + 1, ny = P.hi[1] - P.lo[1] + 1;
    const int g = (f >= 3) ? P.hi[d] + 1 : P.lo[d] - 1;
    const unsigned uu = (unsigned)u;          // a face holds fewer than 2^32 cells
    if (d == 0) { i = g; j = P.lo[1] + (int)(uu % ny); k = P.lo[2] + (int)(uu / ny); }
    else if (d == 1) { j = g; i = P.lo[0] + (int)(uu % nx); k = P.lo[2] + (int)(uu / nx); }
    else { k = g; i = P.lo[0] + (int)(uu % nx); j = P.lo[1] + (int)(uu / nx); }
}

// FillBoundary (face ghosts) + physical/coarse-fine BC closure, one launch:
// MLCellLinOpT::applyBC (AMReX_MLCellLinOp.H:682-893).  The two parts write
// disjoint ghost cells (mask > 0 vs covered) and read only valid cells.
template <typename T>
__global__ void k_ghost (DevLevel L, GhostWork W, T* __restrict__ phi, int inhomog,
                         const double* __restrict__ bcval, int do_copy)
{
    pdl_wait();
    pdl_trigger();
    const long long tid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (tid < W.nfacecells) {
        const int w = bsearch_ll<int>(W.fstart, W.nface, tid);
        const int2 pf = W.faces[w];
        const PatchDesc& P = L.P[pf.x];
        const int f = pf.y;
        const long long u = tid - W.fstart[w];
        int i, j, k;
        face_cell(P, f, u, i, j, k);
        if (face_mask(L, P, f, i, j, k) > 0) {
            const int d = f % 3;
            const long long stride = (d == 0) ? 1 : ((d == 1) ? (long long)P.sx : P.sxy);
            const long long step = (f >= 3) ? -stride : stride;
            bc_ghost<T>(P, f, cidx(P, i, j, k), step, phi, inhomog, bcval, u);
        }
    } else if (do_copy) {
        const long long t = tid - W.nfacecells;
        if (t >= W.ntagcells) { return; }
        const int w = bsearch_ll<int>(W.tstart, W.ntag, t);
        const CopyTag& C = W.tags[w];
        const unsigned u = (unsigned)(t - W.tstart[w]);      // a tag box holds fewer than 2^32 cells
        const unsigned nx = C.box.hi[0] - C.box.lo[0] + 1, ny = C.box.hi[1] - C.box.lo[1] + 1;
        const unsigned row = u / nx;
        const int i = C.box.lo[0] + (int)(u - row * nx);
        const int j = C.box.lo[1] + (int)(row % ny);
        const int k = C.box.lo[2] + (int)(row / ny);
        const PatchDesc& D = L.P[C.dst];
        const PatchDesc& Sp = L.P[C.src];
        phi[cidx(D, i, j, k)] = phi[cidx(Sp, i - C.shift[0], j - C.shift[1], k - C.shift[2])];
    }
}

// ---------------------------------------------------- inter-level transfer --
// patch of solve s at level L containing cell (i,j,k) (linear search; levels
// are almost always a single patch per solve)
__device__ __forceinline__ int find_patch (const DevLevel& L, int s, int i, int j, int k)
{
    const int p0 = L.sfirst[s], np = L.snp[s];
    for (int p = p0; p < p0 + np; ++p) {
        const PatchDesc& P = L.P[p];
        if (i >= P.lo[0] && i <= P.hi[0] && j >= P.lo[1] && j <= P.hi[1] && k >= P.lo[2] && k <= P.hi[2]) {
            return p;
        }
    }
    return p0;
}

// crse = average of 2x2x2 fine: amrex_avgdown (Src/Base/AMReX_MultiFabUtil_3D_C.H:375-392)
template <typename T>
__global__ void __launch_bounds__(TILE_THREADS)
k_restrict (DevLevel Lf, DevLevel Lc, Subset Sc, const T* __restrict__ fine, T* __restrict__ crse)
{
    const TileCoord c = decode_tile(Lc, Sc, blockIdx.x);
    const PatchGeom C = geom_of(Lc.P[c.p]);
    const int s = C.solve;
    // the fine patch over the tile's first and last cells; a tile that lies
    // over one fine patch (nearly all) looks it up once
    const int xe = min(c.x0 + TILE_X - 1, C.hi[0]), ye = min(c.y0 + TILE_Y - 1, C.hi[1]);
    const int ze = min(c.z0 + TILE_Z - 1, C.hi[2]);
    const int pf = find_patch(Lf, s, 2 * c.x0, 2 * c.y0, 2 * c.z0);
    const PatchGeom F0 = geom_of(Lf.P[pf]);
    const bool one = contains(F0, 2 * xe + 1, 2 * ye + 1, 2 * ze + 1);
    pdl_wait();
    pdl_trigger();
    const int j = c.y0 + threadIdx.y;
    if (j > C.hi[1]) { return; }
    const T volfrac = T(1.0) / T(8);
    for (int kk = 0; kk < TILE_Z; ++kk) {
        const int k = c.z0 + kk;
        if (k > C.hi[2]) { break; }
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const int i = c.x0 + threadIdx.x + 32 * h;
            if (i > C.hi[0]) { continue; }
            long long qf, sx, sxy;
            if (one) {
                qf = cidx(F0, 2 * i, 2 * j, 2 * k); sx = F0.sx; sxy = F0.sxy;
            } else {
                const PatchDesc& F = Lf.P[find_patch(Lf, s, 2 * i, 2 * j, 2 * k)];
                qf = cidx(F, 2 * i, 2 * j, 2 * k); sx = F.sx; sxy = F.sxy;
            }
            T v = 0;
            v += fine[qf];           v += fine[qf + 1];
            v += fine[qf + sx];      v += fine[qf + sx + 1];
            v += fine[qf + sxy];     v += fine[qf + sxy + 1];
            v += fine[qf + sxy + sx]; v += fine[qf + sxy + sx + 1];
            crse[cidx(C, i, j, k)] = volfrac * v;
        }
    }
}

// fine += crse(i/2,j/2,k/2): MLCellLinOpT::interpolation (AMReX_MLCellLinOp.H:954-999)
template <typename T>
__global__ void __launch_bounds__(TILE_THREADS)
k_interp_add (DevLevel Lf, Subset Sf, DevLevel Lc, const T* __restrict__ crse, T* __restrict__ fine)
{
    const TileCoord c = decode_tile(Lf, Sf, blockIdx.x);
    const PatchGeom F = geom_of(Lf.P[c.p]);
    const int s = F.solve;
    // the coarse patch under the tile's first and last cells; a tile that
    // lies under one coarse patch (nearly all) looks it up once
    const int xe = min(c.x0 + TILE_X - 1, F.hi[0]), ye = min(c.y0 + TILE_Y - 1, F.hi[1]);
    const int ze = min(c.z0 + TILE_Z - 1, F.hi[2]);
    const int pc = find_patch(Lc, s, c.x0 >> 1, c.y0 >> 1, c.z0 >> 1);
    const PatchGeom C = geom_of(Lc.P[pc]);
    const bool one = contains(C, xe >> 1, ye >> 1, ze >> 1);
    pdl_wait();
    pdl_trigger();
    const int j = c.y0 + threadIdx.y;
    if (j > F.hi[1]) { return; }
    // all of the thread's loads first, then the sums and stores
    T f[TILE_Z][2], v[TILE_Z][2];
    bool ok[TILE_Z][2];
    long long qf[TILE_Z][2];
#pragma unroll
    for (int kk = 0; kk < TILE_Z; ++kk) {
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const int i = c.x0 + threadIdx.x + 32 * h, k = c.z0 + kk;
            ok[kk][h] = (k <= F.hi[2]) && (i <= F.hi[0]);
            qf[kk][h] = cidx(F, i, j, k);
            f[kk][h] = T(0); v[kk][h] = T(0);
            if (ok[kk][h]) {
                const int ic = i >> 1, jc = j >> 1, kc = k >> 1;
                const long long qc = one ? cidx(C, ic, jc, kc) : cidx(Lc.P[find_patch(Lc, s, ic, jc, kc)], ic, jc, kc);
                f[kk][h] = fine[qf[kk][h]];
                v[kk][h] = crse[qc];
            }
        }
    }
#pragma unroll
    for (int kk = 0; kk < TILE_Z; ++kk) {
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            if (ok[kk][h]) { fine[qf[kk][h]] = f[kk][h] + v[kk][h]; }
        }
    }
}

// dst += src over valid cells (LocalAdd), with precision conversion; solves
// whose `active` flag is 0 are left untouched
template <typename TD, typename TS>
__global__ void __launch_bounds__(TILE_THREADS)
k_add_to (DevLevel L, Subset S, TD* __restrict__ dst, const TS* __restrict__ src, const int* __restrict__ active,
          double* __restrict__ clear = nullptr, int nclear = 0)
{
    const TileCoord c = decode_tile(L, S, blockIdx.x);
    const PatchGeom P = geom_of(L.P[c.p]);
    pdl_wait();
    pdl_trigger();
    if (blockIdx.x == 0 && threadIdx.y == 0) {
        for (int t = threadIdx.x; t < nclear; t += 32) { clear[t] = 0.0; }
    }
    const int j = c.y0 + threadIdx.y;
    if (j > P.hi[1]) { return; }
    if (active != nullptr && !active[P.solve]) { return; }
    // all of the thread's loads first, then the sums and stores
    const long long q0 = cidx(P, c.x0 + threadIdx.x, j, c.z0);
    TD d[TILE_Z][2];
    TS v[TILE_Z][2];
    bool ok[TILE_Z][2];
#pragma unroll
    for (int kk = 0; kk < TILE_Z; ++kk) {
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            ok[kk][h] = (c.z0 + kk <= P.hi[2]) && (c.x0 + threadIdx.x + 32 * h <= P.hi[0]);
            const long long q = q0 + kk * P.sxy + 32 * h;
            d[kk][h] = ok[kk][h] ? dst[q] : TD(0);
            v[kk][h] = ok[kk][h] ? src[q] : TS(0);
        }
    }
#pragma unroll
    for (int kk = 0; kk < TILE_Z; ++kk) {
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            if (!ok[kk][h]) { continue; }
            const long long q = q0 + kk * P.sxy + 32 * h;
            if constexpr (std::is_same_v<TD, double> && std::is_same_v<TS, float>) {
                dst[q] = d[kk][h] + f2d_bits(v[kk][h]);
            } else {
                dst[q] = d[kk][h] + TD(v[kk][h]);
            }
        }
    }
}

// per-block partial of max|x|, sum x*y or sum x over valid cells
template <typename T>
__global__ void __launch_bounds__(TILE_THREADS)
k_reduce (DevLevel L, Subset S, const T* __restrict__ x, const T* __restrict__ y, int op,
          double* __restrict__ partial)
{
    pdl_wait();
    pdl_trigger();
    __shared__ double sm[32];
    const TileCoord c = decode_tile(L, S, blockIdx.x);
    const PatchGeom P = geom_of(L.P[c.p]);
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
                const double xv = (double)x[q];
                if (op == RED_MAXABS) { acc = max_nan(acc, fabs(xv)); }
                else if (op == RED_DOT) { acc += xv * (double)y[q]; }
                else { acc += xv; }
            }
        }
    }
    const double red = block_reduce(acc, op, sm);
    if (threadIdx.x == 0 && threadIdx.y == 0) { partial[blockIdx.x] = red; }
}

// one block per solve: combine the partials of blocks [begin[s], begin[s+1])
static __global__ void k_reduce_final (const double* __restrict__ partial, const int* __restrict__ begin, int op,
                                double* __restrict__ out)
{
    pdl_wait();
    pdl_trigger();
    __shared__ double sm[32];
    const int s = blockIdx.x;
    double acc = 0.0;
    for (int b = begin[s] + (int)threadIdx.x; b < begin[s + 1]; b += blockDim.x) {
        acc = red_combine(op, acc, partial[b]);
    }
    const double red = block_reduce(acc, op, sm);
    if (threadIdx.x == 0) { out[s] = red; }
}

// x -= offset[solve] * scale over valid cells (fixSolvabilityByOffset)
template <typename T>
__global__ void __launch_bounds__(TILE_THREADS)
k_minus_offset (DevLevel L, Subset S, T* __restrict__ x, const double* __restrict__ sums,
                const double* __restrict__ volinv)
{
    pdl_wait();
    pdl_trigger();
    const TileCoord c = decode_tile(L, S, blockIdx.x);
    const PatchGeom P = geom_of(L.P[c.p]);
    const int j = c.y0 + threadIdx.y;
    if (j > P.hi[1]) { return; }
    const T off = T(sums[P.solve] * volinv[P.solve]);
    for (int kk = 0; kk < TILE_Z; ++kk) {
        const int k = c.z0 + kk;
        if (k > P.hi[2]) { break; }
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const int i = c.x0 + threadIdx.x + 32 * h;
            if (i > P.hi[0]) { continue; }
            x[cidx(P, i, j, k)] += -off;
        }
    }
}

template <typename TD, typename TS>
__global__ void k_convert (long long n, TD* __restrict__ dst, const TS* __restrict__ src)
{
    for (long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x; q < n;
         q += (long long)gridDim.x * blockDim.x) {
        dst[q] = TD(src[q]);
    }
}

// ------------------------------------------- user MultiFab <-> patch field --
struct XferItem {
    int patch;
    Box3 region;          // cells (in the FAB's index space) to move
    long long src_off;    // FAB offset in the MultiFab allocation
    int flo[3];           // lower corner of the FAB box (grown, nodal-extended)
    int fsx;              // FAB x extent
    long long fsxy;       // FAB x*y extent
};

// dir 0: MultiFab -> patch field ; dir 1: patch field -> MultiFab.  Each
// thread moves XF_CELLS cells blockDim.x apart (coalesced per step): one
// search of the item list for the first, then a walk forward (items hold at
// least one cell, most of them thousands), all loads issued before the stores.
constexpr int XF_CELLS = 8;
template <typename TM, typename TP>
__global__ void k_xfer (DevLevel L, const XferItem* __restrict__ items, const long long* __restrict__ start,
                        int nitem, long long ncell, TM* __restrict__ mf, TP* __restrict__ field, int dir)
{
    const long long t0 = (long long)blockIdx.x * blockDim.x * XF_CELLS + threadIdx.x;
    if (t0 >= ncell) { return; }
    int w = bsearch_ll<int>(start, nitem, t0);
    long long qs[XF_CELLS], qd[XF_CELLS];
    int m_n = 0;
#pragma unroll
    for (int m = 0; m < XF_CELLS; ++m) {
        const long long t = t0 + (long long)m * blockDim.x;
        if (t < ncell) {
            while (w + 1 < nitem && start[w + 1] <= t) { ++w; }
            const XferItem& X = items[w];
            // a region holds fewer than 2^32 cells: 32-bit index arithmetic
            const unsigned u = (unsigned)(t - start[w]);
            const unsigned nx = X.region.hi[0] - X.region.lo[0] + 1, ny = X.region.hi[1] - X.region.lo[1] + 1;
            const unsigned row = u / nx;
            const int i = X.region.lo[0] + (int)(u - row * nx);
            const int j = X.region.lo[1] + (int)(row % ny);
            const int k = X.region.lo[2] + (int)(row / ny);
            const long long qm = X.src_off + (long long)(k - X.flo[2]) * X.fsxy + (long long)(j - X.flo[1]) * X.fsx
                               + (i - X.flo[0]);
            const long long qp = cidx(L.P[X.patch], i, j, k);
            qs[m] = (dir == 0) ? qm : qp;
            qd[m] = (dir == 0) ? qp : qm;
            m_n = m + 1;
        }
    }
    if (dir == 0) {
        TP v[XF_CELLS];
#pragma unroll
        for (int m = 0; m < XF_CELLS; ++m) { if (m < m_n) { v[m] = TP(mf[qs[m]]); } }
#pragma unroll
        for (int m = 0; m < XF_CELLS; ++m) { if (m < m_n) { field[qd[m]] = v[m]; } }
    } else {
        TM v[XF_CELLS];
#pragma unroll
        for (int m = 0; m < XF_CELLS; ++m) { if (m < m_n) { v[m] = TM(field[qs[m]]); } }
#pragma unroll
        for (int m = 0; m < XF_CELLS; ++m) { if (m < m_n) { mf[qd[m]] = v[m]; } }
    }
}

// ------------------------------------------------- coefficient restriction --
// patch of solve s holding face (i,j,k) of direction d: the one whose cells
// include (i,j,k) or, at a high face, (i,j,k) - e_d
__device__ __forceinline__ int find_face_patch (const DevLevel& L, int s, int d, int i, int j, int k)
{
    const int p0 = L.sfirst[s], np = L.snp[s];
    for (int p = p0; p < p0 + np; ++p) {
        const PatchDesc& P = L.P[p];
        const int c[3] = {i, j, k};
        bool in = true;
        for (int e = 0; e < 3; ++e) {
            const int hi = (e == d) ? P.hi[e] + 1 : P.hi[e];
            if (c[e] < P.lo[e] || c[e] > hi) { in = false; }
        }
        if (in) { return p; }
    }
    return p0;
}

template <typename T>
__device__ __forceinline__ void restrict_face (const DevLevel& Lf, const PatchDesc& C, int s, int d, int i, int j,
                                               int k, const T* __restrict__ bf, T* __restrict__ bc)
{
    const int fi = 2 * i, fj = 2 * j, fk = 2 * k;
    const PatchDesc& F = Lf.P[find_face_patch(Lf, s, d, fi, fj, fk)];
    const long long qf = cidx(F, fi, fj, fk);
    long long s0, s1;
    if (d == 0) { s0 = F.sx; s1 = F.sxy; } else if (d == 1) { s0 = 1; s1 = F.sxy; } else { s0 = 1; s1 = F.sx; }
    // amrex_avgdown_faces sums the outer index slowest: (r1, r0) = (k,j) / (k,i) / (j,i)
    T v = T(0.);
    v += bf[qf]; v += bf[qf + s0]; v += bf[qf + s1]; v += bf[qf + s1 + s0];
    bc[cidx(C, i, j, k)] = v * (T(1.0) / T(4));
}

// cell a: amrex_avgdown ; faces: amrex_avgdown_faces
// (Src/Base/AMReX_MultiFabUtil_3D_C.H:170-225, 375-392)
template <typename T>
__global__ void __launch_bounds__(TILE_THREADS)
k_restrict_coef (DevLevel Lf, DevLevel Lc, Subset Sc, const T* __restrict__ af, const T* __restrict__ bxf,
                 const T* __restrict__ byf, const T* __restrict__ bzf, T* __restrict__ ac, T* __restrict__ bxc,
                 T* __restrict__ byc, T* __restrict__ bzc, int a_zero)
{
    const TileCoord c = decode_tile(Lc, Sc, blockIdx.x);
    const PatchDesc& C = Lc.P[c.p];
    const int j = c.y0 + threadIdx.y;
    const int s = C.solve;
    if (j > C.hi[1]) { return; }
    for (int kk = 0; kk < TILE_Z; ++kk) {
        const int k = c.z0 + kk;
        if (k > C.hi[2]) { break; }
        for (int h = 0; h < 2; ++h) {
            const int i = c.x0 + threadIdx.x + 32 * h;
            if (i > C.hi[0]) { continue; }
            const long long qc = cidx(C, i, j, k);
            if (a_zero) {
                ac[qc] = T(0);
            } else {
                const PatchDesc& F = Lf.P[find_patch(Lf, s, 2 * i, 2 * j, 2 * k)];
                const long long qf = cidx(F, 2 * i, 2 * j, 2 * k);
                const long long sx = F.sx, sxy = F.sxy;
                T v = 0;
                v += af[qf]; v += af[qf + 1]; v += af[qf + sx]; v += af[qf + sx + 1];
                v += af[qf + sxy]; v += af[qf + sxy + 1]; v += af[qf + sxy + sx]; v += af[qf + sxy + sx + 1];
                ac[qc] = (T(1.0) / T(8)) * v;
            }
            restrict_face<T>(Lf, C, s, 0, i, j, k, bxf, bxc);
            restrict_face<T>(Lf, C, s, 1, i, j, k, byf, byc);
            restrict_face<T>(Lf, C, s, 2, i, j, k, bzf, bzc);
            if (i == C.hi[0]) { restrict_face<T>(Lf, C, s, 0, i + 1, j, k, bxf, bxc); }
            if (j == C.hi[1]) { restrict_face<T>(Lf, C, s, 1, i, j + 1, k, byf, byc); }
            if (k == C.hi[2]) { restrict_face<T>(Lf, C, s, 2, i, j, k + 1, bzf, bzc); }
        }
    }
}

} // namespace mlmg
