// Bottom solve: one thread block per solve runs the whole Krylov bottom
// solve -- the Jacobi-preconditioned BiCGStab of MLCGSolverT::solve_bicgstab
// (AMReX_MLCGSolver.H:96-273) or the CG of MLCGSolverT::solve_cg (:275-410),
// or one then the other (BottomSolver::bicgcg / cgbicg, with the switch to
// the second kept for later bottom solves once it succeeds) -- and the
// follow-up smoothing of MLMGT::actualBottomSolve (AMReX_MLMG.H:1500-1610) on
// the solve's coarsest level, with FP64 arithmetic, dot products and norms,
// and no host round trip.  The coarsest level is tiny (2^3..8^3 cells for the benchmark
// configurations), so one block is the right size.  The block-level helpers
// here are also used by the coarse-level V-cycle kernel.
#pragma once

#include "stage_kernels.cuh"

namespace mlmg {

constexpr int BOTTOM_THREADS = 128;

struct BottomLevelPtrs {       // one level that is the bottom of some solve
    DevLevel L;
    const CopyTag* tags;
    double *x, *b, *p, *r, *rh, *v, *t;    // FP64 work arrays (level layout)
    const double *a, *bx, *by, *bz;        // FP64 coefficients
    void* x_out;                           // working-precision cor of the level
    const void* b_in;                      // working-precision res of the level
};

struct BottomJob {
    int lev;                   // index into the BottomLevelPtrs table
    int solve;
    int p0, np;                // the solve's patches at that level
    int t0, nt;                // the solve's ghost-copy tags at that level
    int singular;
    double volinv;
};

// MLMG::BottomSolver codes (AMReX_MLLinOp.H:30-31)
enum BottomKind : int { BK_SMOOTHER = 1, BK_BICGSTAB = 2, BK_CG = 3, BK_BICGCG = 4, BK_CGBICG = 5 };

struct BottomParams {
    int maxiter;
    double eps_rel, eps_abs;
    int nub, nuf;
    int smoother_only;         // bottom_solver == smoother
    int* mode;                 // per solve: the current BottomKind (bicgcg / cgbicg become cg /
                               // bicgstab once their second solver succeeds); null: bicgstab
    int* iters2;               // per solve: the second solver's iterations, -1 if it did not run
};

namespace bottom_detail {

// flat loop over the valid cells of patches [p0, p0+np)
template <typename F>
__device__ __forceinline__ void for_cells (const DevLevel& L, int p0, int np, F&& f)
{
    for (int p = p0; p < p0 + np; ++p) {
        const PatchDesc& P = L.P[p];
        const int nx = P.hi[0] - P.lo[0] + 1, ny = P.hi[1] - P.lo[1] + 1, nz = P.hi[2] - P.lo[2] + 1;
        const int n = nx * ny * nz;
        for (int u = threadIdx.x; u < n; u += blockDim.x) {
            const int i = P.lo[0] + u % nx;
            const int j = P.lo[1] + (u / nx) % ny;
            const int k = P.lo[2] + u / (nx * ny);
            f(P, i, j, k, cidx(P, i, j, k));
        }
    }
}

// applyBC (homogeneous) for one solve's patches of a level: BC closures
// where the mask is > 0, then copies from neighbouring patches
template <typename T>
__device__ void ghost_fill (const DevLevel& L, const CopyTag* tags, int p0, int np, int t0, int nt, T* phi)
{
    __syncthreads();
    for (int p = p0; p < p0 + np; ++p) {
        const PatchDesc& P = L.P[p];
        for (int f = 0; f < 6; ++f) {
            const int d = f % 3;
            const int e0 = (d == 0) ? 1 : 0, e1 = (d == 2) ? 1 : 2;
            const int n = (P.hi[e0] - P.lo[e0] + 1) * (P.hi[e1] - P.lo[e1] + 1);
            for (int u = threadIdx.x; u < n; u += blockDim.x) {
                int i, j, k;
                face_cell(P, f, u, i, j, k);
                if (face_mask(L, P, f, i, j, k) > 0) {
                    const long long stride = (d == 0) ? 1 : ((d == 1) ? (long long)P.sx : P.sxy);
                    bc_ghost<T>(P, f, cidx(P, i, j, k), (f >= 3) ? -stride : stride, phi, 0, nullptr, u);
                }
            }
        }
    }
    for (int w = t0; w < t0 + nt; ++w) {
        const CopyTag& C = tags[w];
        const int nx = C.box.hi[0] - C.box.lo[0] + 1, ny = C.box.hi[1] - C.box.lo[1] + 1;
        const int n = nx * ny * (C.box.hi[2] - C.box.lo[2] + 1);
        for (int u = threadIdx.x; u < n; u += blockDim.x) {
            const int i = C.box.lo[0] + u % nx;
            const int j = C.box.lo[1] + (u / nx) % ny;
            const int k = C.box.lo[2] + u / (nx * ny);
            phi[cidx(L.P[C.dst], i, j, k)] = phi[cidx(L.P[C.src], i - C.shift[0], j - C.shift[1], k - C.shift[2])];
        }
    }
    __syncthreads();
}

// out = A in (homogeneous BCs), divided by the diagonal (MLABecLaplacianT::
// normalize, AMReX_MLABecLaplacian.H:1128-1168) when NORM
template <bool ABEC, bool NORM = true>
__device__ void apply_normalize (const BottomLevelPtrs& B, const BottomJob& J, double* out, double* in)
{
    ghost_fill<double>(B.L, B.tags, J.p0, J.np, J.t0, J.nt, in);
    for_cells(B.L, J.p0, J.np, [&] (const PatchDesc& P, int, int, int, long long q) {
        double v = adotx_cell<double, ABEC>(P, q, in, B.a, B.bx, B.by, B.bz);
        if constexpr (ABEC && NORM) { v /= abec_diag<double>(P, q, B.a, B.bx, B.by, B.bz); }
        out[q] = v;
    });
    __syncthreads();
}

__device__ inline double reduce (const DevLevel& L, int p0, int np, const double* x, const double* y, int op)
{
    __shared__ double sm[32];
    __shared__ double result;
    double acc = 0.0;
    for_cells(L, p0, np, [&] (const PatchDesc&, int, int, int, long long q) {
        if (op == RED_MAXABS) { acc = max_nan(acc, fabs(x[q])); }
        else if (op == RED_DOT) { acc += x[q] * y[q]; }
        else { acc += x[q]; }
    });
    const double r = block_reduce(acc, op, sm);
    if (threadIdx.x == 0) { result = r; }
    __syncthreads();
    const double out = result;
    __syncthreads();
    return out;
}

template <bool ABEC>
__device__ void smooth (const BottomLevelPtrs& B, const BottomJob& J, double* x, const double* b)
{
    for (int rb = 0; rb < 2; ++rb) {
        ghost_fill<double>(B.L, B.tags, J.p0, J.np, J.t0, J.nt, x);
        for_cells(B.L, J.p0, J.np, [&] (const PatchDesc& P, int i, int j, int k, long long) {
            if (((i + j + k + rb) & 1) == 0) {
                gsrb_cell<double, ABEC>(B.L, P, i, j, k, x, b, B.a, B.bx, B.by, B.bz);
            }
        });
        __syncthreads();
    }
}

// x = 0 and the solver's work vectors p, r = 0, ghosts included
__device__ inline void zero_work (const BottomLevelPtrs& B, const BottomJob& J)
{
    for (int pp = J.p0; pp < J.p0 + J.np; ++pp) {
        const PatchDesc& P = B.L.P[pp];
        const long long n0 = P.base - P.sxy - P.sx - XOFF;   // the patch's whole allocation
        const long long n = P.sxy * (P.hi[2] - P.lo[2] + 3);
        for (long long u = threadIdx.x; u < n; u += blockDim.x) {
            B.x[n0 + u] = 0.0; B.p[n0 + u] = 0.0; B.r[n0 + u] = 0.0;
        }
    }
    __syncthreads();
}

// MLCGSolverT::solve_bicgstab with a zero initial guess (AMReX_MLCGSolver.H:
// 96-273) on right-hand side bb; returns its code, the iterations in *iters
template <bool ABEC>
__device__ int bicgstab (const BottomLevelPtrs& B, const BottomJob& J, const BottomParams& prm, const double* bb,
                         int* iters)
{
    double *x = B.x, *p = B.p, *r = B.r, *rh = B.rh, *v = B.v, *t = B.t;
    zero_work(B, J);
    // r = b ; normalize ; rh = r
    for_cells(B.L, J.p0, J.np, [&] (const PatchDesc& P, int, int, int, long long q) {
        double val = bb[q];
        if constexpr (ABEC) { val /= abec_diag<double>(P, q, B.a, B.bx, B.by, B.bz); }
        r[q] = val;
    });
    __syncthreads();
    for_cells(B.L, J.p0, J.np, [&] (const PatchDesc&, int, int, int, long long q) { rh[q] = r[q]; });
    __syncthreads();
    double rnorm = reduce(B.L, J.p0, J.np, r, nullptr, RED_MAXABS);
    const double rnorm0 = rnorm;
    double rho_1 = 0, alpha = 0, omega = 0;
    int ret = 0, iter = 1;
    if (!(rnorm0 == 0 || rnorm0 < prm.eps_abs)) {
        for (; iter <= prm.maxiter; ++iter) {
            const double rho = reduce(B.L, J.p0, J.np, rh, r, RED_DOT);
            if (rho == 0) { ret = 1; break; }
            if (iter == 1) {
                for_cells(B.L, J.p0, J.np, [&] (const PatchDesc&, int, int, int, long long q) { p[q] = r[q]; });
            } else {
                const double beta = (rho / rho_1) * (alpha / omega);
                for_cells(B.L, J.p0, J.np, [&] (const PatchDesc&, int, int, int, long long q) {
                    double pv = p[q] + (-omega) * v[q];   // Saxpy
                    p[q] = r[q] + beta * pv;              // Xpay
                });
            }
            __syncthreads();
            apply_normalize<ABEC>(B, J, v, p);
            const double rhTv = reduce(B.L, J.p0, J.np, rh, v, RED_DOT);
            if (rhTv != 0.0) { alpha = rho / rhTv; } else { ret = 2; break; }
            for_cells(B.L, J.p0, J.np, [&] (const PatchDesc&, int, int, int, long long q) {
                x[q] += alpha * p[q];
                r[q] += (-alpha) * v[q];
            });
            __syncthreads();
            rnorm = reduce(B.L, J.p0, J.np, r, nullptr, RED_MAXABS);
            if (rnorm < prm.eps_rel * rnorm0 || rnorm < prm.eps_abs) { break; }
            apply_normalize<ABEC>(B, J, t, r);
            const double tt = reduce(B.L, J.p0, J.np, t, t, RED_DOT);
            const double tr = reduce(B.L, J.p0, J.np, t, r, RED_DOT);
            if (tt != 0.0) { omega = tr / tt; } else { ret = 3; break; }
            for_cells(B.L, J.p0, J.np, [&] (const PatchDesc&, int, int, int, long long q) {
                x[q] += omega * r[q];
                r[q] += (-omega) * t[q];
            });
            __syncthreads();
            rnorm = reduce(B.L, J.p0, J.np, r, nullptr, RED_MAXABS);
            if (rnorm < prm.eps_rel * rnorm0 || rnorm < prm.eps_abs) { break; }
            if (omega == 0) { ret = 4; break; }
            rho_1 = rho;
        }
        if (ret == 0 && rnorm > prm.eps_rel * rnorm0 && rnorm > prm.eps_abs) { ret = 8; }
        if ((ret == 0 || ret == 8) && (rnorm < rnorm0)) {
            if (ret == 8) { ret = 9; }
        } else {
            for_cells(B.L, J.p0, J.np, [&] (const PatchDesc&, int, int, int, long long q) { x[q] = 0.0; });
            __syncthreads();
        }
    }
    *iters = iter;
    return ret;
}

// MLCGSolverT::solve_cg with a zero initial guess (AMReX_MLCGSolver.H:
// 275-410): unpreconditioned CG, q = A p with homogeneous BCs; v holds q
template <bool ABEC>
__device__ int conj_grad (const BottomLevelPtrs& B, const BottomJob& J, const BottomParams& prm, const double* bb,
                          int* iters)
{
    double *x = B.x, *p = B.p, *r = B.r, *q = B.v;
    zero_work(B, J);
    for_cells(B.L, J.p0, J.np, [&] (const PatchDesc&, int, int, int, long long c) { r[c] = bb[c]; });
    __syncthreads();
    double rnorm = reduce(B.L, J.p0, J.np, r, nullptr, RED_MAXABS);
    const double rnorm0 = rnorm;
    double rho_1 = 0;
    int ret = 0, iter = 1;
    if (rnorm0 == 0 || rnorm0 < prm.eps_abs) {
        *iters = iter;
        return ret;
    }
    for (; iter <= prm.maxiter; ++iter) {
        const double rho = reduce(B.L, J.p0, J.np, r, r, RED_DOT);
        if (rho == 0) { ret = 1; break; }
        if (iter == 1) {
            for_cells(B.L, J.p0, J.np, [&] (const PatchDesc&, int, int, int, long long c) { p[c] = r[c]; });
        } else {
            const double beta = rho / rho_1;
            for_cells(B.L, J.p0, J.np, [&] (const PatchDesc&, int, int, int, long long c) {
                p[c] = r[c] + beta * p[c];        // Xpay
            });
        }
        __syncthreads();
        apply_normalize<ABEC, false>(B, J, q, p);
        const double pw = reduce(B.L, J.p0, J.np, p, q, RED_DOT);
        double alpha;
        if (pw != 0.0) { alpha = rho / pw; } else { ret = 1; break; }
        for_cells(B.L, J.p0, J.np, [&] (const PatchDesc&, int, int, int, long long c) {
            x[c] += alpha * p[c];                 // Saxpy
            r[c] += (-alpha) * q[c];
        });
        __syncthreads();
        rnorm = reduce(B.L, J.p0, J.np, r, nullptr, RED_MAXABS);
        if (rnorm < prm.eps_rel * rnorm0 || rnorm < prm.eps_abs) { break; }
        rho_1 = rho;
    }
    if (ret == 0 && rnorm > prm.eps_rel * rnorm0 && rnorm > prm.eps_abs) { ret = 8; }
    if ((ret == 0 || ret == 8) && (rnorm < rnorm0)) {
        if (ret == 8) { ret = 9; }
    } else {
        for_cells(B.L, J.p0, J.np, [&] (const PatchDesc&, int, int, int, long long c) { x[c] = 0.0; });
        __syncthreads();
    }
    *iters = iter;
    return ret;
}

} // namespace bottom_detail

// the bottom solve of one solve, executed by the calling block
template <typename T, bool ABEC>
__device__ void bottom_solve_block (const BottomLevelPtrs& B, const BottomJob& J, const BottomParams& prm,
                                    int* __restrict__ out_iters, int* __restrict__ out_ret)
{
    using namespace bottom_detail;
    double *x = B.x, *b = B.b;
    const T* bin = static_cast<const T*>(B.b_in);
    T* xout = static_cast<T*>(B.x_out);

    zero_work(B, J);
    for_cells(B.L, J.p0, J.np, [&] (const PatchDesc&, int, int, int, long long q) { b[q] = (double)bin[q]; });
    __syncthreads();

    int ret = 0, iter = 0, iter2 = -1;
    if (prm.smoother_only) {
        for (int i = 0; i < prm.nuf; ++i) { smooth<ABEC>(B, J, x, b); }
    } else {
        // the solve's b, made solvable for a singular operator (the Krylov
        // solvers' private copy: the smoothing after them takes the level's b)
        const double* bb = b;
        if (J.singular) {
            const double off = reduce(B.L, J.p0, J.np, b, nullptr, RED_SUM) * J.volinv;
            for_cells(B.L, J.p0, J.np, [&] (const PatchDesc&, int, int, int, long long q) { b[q] = b[q] + (-off); });
            __syncthreads();
        }
        const int kind = (prm.mode != nullptr) ? prm.mode[J.solve] : BK_BICGSTAB;
        const bool cg_first = (kind == BK_CG || kind == BK_CGBICG);
        ret = cg_first ? conj_grad<ABEC>(B, J, prm, bb, &iter) : bicgstab<ABEC>(B, J, prm, bb, &iter);
        if (ret != 0 && (kind == BK_BICGCG || kind == BK_CGBICG)) {
            // MLMGT::actualBottomSolve: the other solver from zero; once it
            // succeeds it is used from then on
            ret = cg_first ? bicgstab<ABEC>(B, J, prm, bb, &iter2) : conj_grad<ABEC>(B, J, prm, bb, &iter2);
            if (ret == 0 && threadIdx.x == 0) { prm.mode[J.solve] = cg_first ? BK_BICGSTAB : BK_CG; }
        }
        if (ret != 0 && ret != 9) {
            for_cells(B.L, J.p0, J.np, [&] (const PatchDesc&, int, int, int, long long q) { x[q] = 0.0; });
            __syncthreads();
        }
        if (J.singular) {
            // the smoother below takes the level's own b
            for_cells(B.L, J.p0, J.np, [&] (const PatchDesc&, int, int, int, long long q) { b[q] = (double)bin[q]; });
            __syncthreads();
        }
        const int n = (ret == 0) ? prm.nub : prm.nuf;
        for (int i = 0; i < n; ++i) { smooth<ABEC>(B, J, x, b); }
    }
    __syncthreads();
    for_cells(B.L, J.p0, J.np, [&] (const PatchDesc&, int, int, int, long long q) { xout[q] = T(x[q]); });
    if (threadIdx.x == 0) {
        out_iters[J.solve] = iter;
        out_ret[J.solve] = ret;
        if (prm.iters2 != nullptr) { prm.iters2[J.solve] = iter2; }
    }
    __syncthreads();
}

template <typename T, bool ABEC>
__global__ void __launch_bounds__(BOTTOM_THREADS)
k_bottom (const BottomLevelPtrs* __restrict__ levels, const BottomJob* __restrict__ jobs, BottomParams prm,
          const int* __restrict__ active, int* __restrict__ out_iters, int* __restrict__ out_ret)
{
    const BottomJob J = jobs[blockIdx.x];
    pdl_wait();
    pdl_trigger();
    if (active != nullptr && !active[J.solve]) { return; }
    bottom_solve_block<T, ABEC>(levels[J.lev], J, prm, out_iters, out_ret);
}

} // namespace mlmg
