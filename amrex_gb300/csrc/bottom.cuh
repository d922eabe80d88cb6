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

// Per-thread cache of a solve's bottom level, built once per bottom solve:
// the thread's cells (the same cells, in the same order, as for_cells gives
// it) and its face-ghost entries (as ghost_fill assigns them), so the Krylov
// loop's many passes skip the index divisions and face walks.  Used when the
// solve has one patch and every thread's share fits; uniform over the block.
constexpr int BC_CELLS = 2;
constexpr int BC_GHOSTS = 6;

struct BotCache {
    bool cells = false, ghosts = false;
    const PatchDesc* P = nullptr;
    int n = 0;
    long long q[BC_CELLS];
    int i[BC_CELLS], j[BC_CELLS], k[BC_CELLS];
    int ng = 0;
    int gf[BC_GHOSTS];               // the face of each ghost entry
    long long gq[BC_GHOSTS];         // its ghost cell
};

struct BottomJobK : BottomJob {
    BotCache K;
};

__device__ inline BottomJobK make_job (const BottomLevelPtrs& B, const BottomJob& J0)
{
    BottomJobK J;
    static_cast<BottomJob&>(J) = J0;
    if (J0.np != 1) { return J; }
    const PatchDesc& P = B.L.P[J0.p0];
    const int nx = P.hi[0] - P.lo[0] + 1, ny = P.hi[1] - P.lo[1] + 1, nz = P.hi[2] - P.lo[2] + 1;
    const int ncell = nx * ny * nz;
    BotCache& K = J.K;
    K.P = &P;
    if (ncell <= BC_CELLS * (int)blockDim.x) {
        K.cells = true;
#pragma unroll
        for (int c = 0; c < BC_CELLS; ++c) {
            const int u = (int)threadIdx.x + c * (int)blockDim.x;
            K.i[c] = K.j[c] = K.k[c] = 0;
            K.q[c] = 0;
            if (u < ncell) {
                K.n = c + 1;
                K.i[c] = P.lo[0] + u % nx;
                K.j[c] = P.lo[1] + (u / nx) % ny;
                K.k[c] = P.lo[2] + u / (nx * ny);
                K.q[c] = cidx(P, K.i[c], K.j[c], K.k[c]);
            }
        }
    }
    // the face walk of ghost_fill: face f's cells u = tid, tid + blockDim, ...
    int per_thread = 0;
    const int nf[6] = {ny * nz, nx * nz, nx * ny, ny * nz, nx * nz, nx * ny};
    for (int f = 0; f < 6; ++f) { per_thread += (nf[f] + (int)blockDim.x - 1) / (int)blockDim.x; }
    if (per_thread <= BC_GHOSTS) {
        // entries in the walk's order; with at most one cell per face per
        // thread (the common case) slot f holds face f's cell, or none
        K.ghosts = true;
        int g = 0;
#pragma unroll
        for (int s = 0; s < BC_GHOSTS; ++s) { K.gf[s] = -1; K.gq[s] = 0; }
        for (int f = 0; f < 6; ++f) {
            for (int u = threadIdx.x; u < nf[f]; u += blockDim.x) {
                int i, j, k;
                face_cell(P, f, u, i, j, k);
                if (face_mask(B.L, P, f, i, j, k) > 0) {
#pragma unroll
                    for (int s = 0; s < BC_GHOSTS; ++s) {
                        if (s == g) { K.gf[s] = f; K.gq[s] = cidx(P, i, j, k); }
                    }
                    ++g;
                }
            }
        }
        K.ng = g;
    }
    return J;
}

// for_cells over the solve's bottom patches, from the cache when it holds them
template <typename F>
__device__ __forceinline__ void cells (const BottomJobK& J, const DevLevel& L, F&& f)
{
    if (J.K.cells) {
#pragma unroll
        for (int c = 0; c < BC_CELLS; ++c) {
            if (c < J.K.n) { f(*J.K.P, J.K.i[c], J.K.j[c], J.K.k[c], J.K.q[c]); }
        }
    } else {
        for_cells(L, J.p0, J.np, f);
    }
}

// ghost_fill of the solve's bottom patches, the closures from the cache when
// it holds them (the copies between patches keep their walk)
__device__ inline void ghosts (const BottomJobK& J, const BottomLevelPtrs& B, double* phi)
{
    if (!J.K.ghosts) {
        ghost_fill<double>(B.L, B.tags, J.p0, J.np, J.t0, J.nt, phi);
        return;
    }
    __syncthreads();
    const PatchDesc& P = *J.K.P;
#pragma unroll
    for (int g = 0; g < BC_GHOSTS; ++g) {
        if (g < J.K.ng) {
            // homogeneous closures: the Dirichlet value slot index is not read
            const int f = J.K.gf[g], d = f % 3;
            const long long stride = (d == 0) ? 1 : ((d == 1) ? (long long)P.sx : P.sxy);
            bc_ghost<double>(P, f, J.K.gq[g], (f >= 3) ? -stride : stride, phi, 0, nullptr, 0);
        }
    }
    for (int w = J.t0; w < J.t0 + J.nt; ++w) {
        const CopyTag& C = B.tags[w];
        const int nx = C.box.hi[0] - C.box.lo[0] + 1, ny = C.box.hi[1] - C.box.lo[1] + 1;
        const int n = nx * ny * (C.box.hi[2] - C.box.lo[2] + 1);
        for (int u = threadIdx.x; u < n; u += blockDim.x) {
            const int i = C.box.lo[0] + u % nx;
            const int j = C.box.lo[1] + (u / nx) % ny;
            const int k = C.box.lo[2] + u / (nx * ny);
            phi[cidx(B.L.P[C.dst], i, j, k)] = phi[cidx(B.L.P[C.src], i - C.shift[0], j - C.shift[1], k - C.shift[2])];
        }
    }
    __syncthreads();
}

// out = A in (homogeneous BCs), divided by the diagonal (MLABecLaplacianT::
// normalize, AMReX_MLABecLaplacian.H:1128-1168) when NORM
template <bool ABEC, bool NORM = true>
__device__ void apply_normalize (const BottomLevelPtrs& B, const BottomJobK& J, double* out, double* in)
{
    ghosts(J, B, in);
    cells(J, B.L, [&] (const PatchDesc& P, int, int, int, long long q) {
        double v = adotx_cell<double, ABEC>(P, q, in, B.a, B.bx, B.by, B.bz);
        if constexpr (ABEC && NORM) { v /= abec_diag<double>(P, q, B.a, B.bx, B.by, B.bz); }
        out[q] = v;
    });
    __syncthreads();
}

__device__ inline double reduce (const BottomJobK& J, const DevLevel& L, const double* x, const double* y, int op)
{
    __shared__ double sm[32];
    __shared__ double result;
    double acc = 0.0;
    cells(J, L, [&] (const PatchDesc&, int, int, int, long long q) {
        if (op == RED_MAXABS) { acc = max_nan(acc, fabs(x[q])); }
        else if (op == RED_DOT) { acc += x[q] * y[q]; }
        else { acc += x[q]; }
    });
    if (blockDim.x == 32) {
        // one warp: block_reduce's two stages without its barriers (the
        // second stage combines lane 0's value with five zeros)
        double v = acc;
        for (int o = 16; o > 0; o >>= 1) { v = red_combine(op, v, __shfl_down_sync(0xffffffffu, v, o)); }
        for (int o = 16; o > 0; o >>= 1) { v = red_combine(op, v, 0.0); }
        return __shfl_sync(0xffffffffu, v, 0);
    }
    const double r = block_reduce(acc, op, sm);
    if (threadIdx.x == 0) { result = r; }
    __syncthreads();
    const double out = result;
    __syncthreads();
    return out;
}

template <bool ABEC>
__device__ void smooth (const BottomLevelPtrs& B, const BottomJobK& J, double* x, const double* b)
{
    for (int rb = 0; rb < 2; ++rb) {
        ghosts(J, B, x);
        cells(J, B.L, [&] (const PatchDesc& P, int i, int j, int k, long long) {
            if (((i + j + k + rb) & 1) == 0) {
                gsrb_cell<double, ABEC>(B.L, P, i, j, k, x, b, B.a, B.bx, B.by, B.bz);
            }
        });
        __syncthreads();
    }
}

// x = 0 and the solver's work vectors p, r = 0, ghosts included
__device__ inline void zero_work (const BottomLevelPtrs& B, const BottomJobK& J)
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
__device__ int bicgstab (const BottomLevelPtrs& B, const BottomJobK& J, const BottomParams& prm, const double* bb,
                         int* iters)
{
    double *x = B.x, *p = B.p, *r = B.r, *rh = B.rh, *v = B.v, *t = B.t;
    zero_work(B, J);
    // r = b ; normalize ; rh = r
    cells(J, B.L, [&] (const PatchDesc& P, int, int, int, long long q) {
        double val = bb[q];
        if constexpr (ABEC) { val /= abec_diag<double>(P, q, B.a, B.bx, B.by, B.bz); }
        r[q] = val;
    });
    __syncthreads();
    cells(J, B.L, [&] (const PatchDesc&, int, int, int, long long q) { rh[q] = r[q]; });
    __syncthreads();
    double rnorm = reduce(J, B.L, r, nullptr, RED_MAXABS);
    const double rnorm0 = rnorm;
    double rho_1 = 0, alpha = 0, omega = 0;
    int ret = 0, iter = 1;
    if (!(rnorm0 == 0 || rnorm0 < prm.eps_abs)) {
        for (; iter <= prm.maxiter; ++iter) {
            const double rho = reduce(J, B.L, rh, r, RED_DOT);
            if (rho == 0) { ret = 1; break; }
            if (iter == 1) {
                cells(J, B.L, [&] (const PatchDesc&, int, int, int, long long q) { p[q] = r[q]; });
            } else {
                const double beta = (rho / rho_1) * (alpha / omega);
                cells(J, B.L, [&] (const PatchDesc&, int, int, int, long long q) {
                    double pv = p[q] + (-omega) * v[q];   // Saxpy
                    p[q] = r[q] + beta * pv;              // Xpay
                });
            }
            __syncthreads();
            apply_normalize<ABEC>(B, J, v, p);
            const double rhTv = reduce(J, B.L, rh, v, RED_DOT);
            if (rhTv != 0.0) { alpha = rho / rhTv; } else { ret = 2; break; }
            cells(J, B.L, [&] (const PatchDesc&, int, int, int, long long q) {
                x[q] += alpha * p[q];
                r[q] += (-alpha) * v[q];
            });
            __syncthreads();
            rnorm = reduce(J, B.L, r, nullptr, RED_MAXABS);
            if (rnorm < prm.eps_rel * rnorm0 || rnorm < prm.eps_abs) { break; }
            apply_normalize<ABEC>(B, J, t, r);
            const double tt = reduce(J, B.L, t, t, RED_DOT);
            const double tr = reduce(J, B.L, t, r, RED_DOT);
            if (tt != 0.0) { omega = tr / tt; } else { ret = 3; break; }
            cells(J, B.L, [&] (const PatchDesc&, int, int, int, long long q) {
                x[q] += omega * r[q];
                r[q] += (-omega) * t[q];
            });
            __syncthreads();
            rnorm = reduce(J, B.L, r, nullptr, RED_MAXABS);
            if (rnorm < prm.eps_rel * rnorm0 || rnorm < prm.eps_abs) { break; }
            if (omega == 0) { ret = 4; break; }
            rho_1 = rho;
        }
        if (ret == 0 && rnorm > prm.eps_rel * rnorm0 && rnorm > prm.eps_abs) { ret = 8; }
        if ((ret == 0 || ret == 8) && (rnorm < rnorm0)) {
            if (ret == 8) { ret = 9; }
        } else {
            cells(J, B.L, [&] (const PatchDesc&, int, int, int, long long q) { x[q] = 0.0; });
            __syncthreads();
        }
    }
    *iters = iter;
    return ret;
}

// MLCGSolverT::solve_cg with a zero initial guess (AMReX_MLCGSolver.H:
// 275-410): unpreconditioned CG, q = A p with homogeneous BCs; v holds q
template <bool ABEC>
__device__ int conj_grad (const BottomLevelPtrs& B, const BottomJobK& J, const BottomParams& prm, const double* bb,
                          int* iters)
{
    double *x = B.x, *p = B.p, *r = B.r, *q = B.v;
    zero_work(B, J);
    cells(J, B.L, [&] (const PatchDesc&, int, int, int, long long c) { r[c] = bb[c]; });
    __syncthreads();
    double rnorm = reduce(J, B.L, r, nullptr, RED_MAXABS);
    const double rnorm0 = rnorm;
    double rho_1 = 0;
    int ret = 0, iter = 1;
    if (rnorm0 == 0 || rnorm0 < prm.eps_abs) {
        *iters = iter;
        return ret;
    }
    for (; iter <= prm.maxiter; ++iter) {
        const double rho = reduce(J, B.L, r, r, RED_DOT);
        if (rho == 0) { ret = 1; break; }
        if (iter == 1) {
            cells(J, B.L, [&] (const PatchDesc&, int, int, int, long long c) { p[c] = r[c]; });
        } else {
            const double beta = rho / rho_1;
            cells(J, B.L, [&] (const PatchDesc&, int, int, int, long long c) {
                p[c] = r[c] + beta * p[c];        // Xpay
            });
        }
        __syncthreads();
        apply_normalize<ABEC, false>(B, J, q, p);
        const double pw = reduce(J, B.L, p, q, RED_DOT);
        double alpha;
        if (pw != 0.0) { alpha = rho / pw; } else { ret = 1; break; }
        cells(J, B.L, [&] (const PatchDesc&, int, int, int, long long c) {
            x[c] += alpha * p[c];                 // Saxpy
            r[c] += (-alpha) * q[c];
        });
        __syncthreads();
        rnorm = reduce(J, B.L, r, nullptr, RED_MAXABS);
        if (rnorm < prm.eps_rel * rnorm0 || rnorm < prm.eps_abs) { break; }
        rho_1 = rho;
    }
    if (ret == 0 && rnorm > prm.eps_rel * rnorm0 && rnorm > prm.eps_abs) { ret = 8; }
    if ((ret == 0 || ret == 8) && (rnorm < rnorm0)) {
        if (ret == 8) { ret = 9; }
    } else {
        cells(J, B.L, [&] (const PatchDesc&, int, int, int, long long c) { x[c] = 0.0; });
        __syncthreads();
    }
    *iters = iter;
    return ret;
}

} // namespace bottom_detail

// the bottom solve of one solve, executed by the calling block
template <typename T, bool ABEC>
__device__ void bottom_solve_block (const BottomLevelPtrs& B, const BottomJob& J0, const BottomParams& prm,
                                    int* __restrict__ out_iters, int* __restrict__ out_ret)
{
    using namespace bottom_detail;
    const BottomJobK J = make_job(B, J0);
    double *x = B.x, *b = B.b;
    const T* bin = static_cast<const T*>(B.b_in);
    T* xout = static_cast<T*>(B.x_out);

    zero_work(B, J);
    cells(J, B.L, [&] (const PatchDesc&, int, int, int, long long q) { b[q] = (double)bin[q]; });
    __syncthreads();

    int ret = 0, iter = 0, iter2 = -1;
    if (prm.smoother_only) {
        for (int i = 0; i < prm.nuf; ++i) { smooth<ABEC>(B, J, x, b); }
    } else {
        // the solve's b, made solvable for a singular operator (the Krylov
        // solvers' private copy: the smoothing after them takes the level's b)
        const double* bb = b;
        if (J.singular) {
            const double off = reduce(J, B.L, b, nullptr, RED_SUM) * J.volinv;
            cells(J, B.L, [&] (const PatchDesc&, int, int, int, long long q) { b[q] = b[q] + (-off); });
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
            cells(J, B.L, [&] (const PatchDesc&, int, int, int, long long q) { x[q] = 0.0; });
            __syncthreads();
        }
        if (J.singular) {
            // the smoother below takes the level's own b
            cells(J, B.L, [&] (const PatchDesc&, int, int, int, long long q) { b[q] = (double)bin[q]; });
            __syncthreads();
        }
        const int n = (ret == 0) ? prm.nub : prm.nuf;
        for (int i = 0; i < n; ++i) { smooth<ABEC>(B, J, x, b); }
    }
    __syncthreads();
    cells(J, B.L, [&] (const PatchDesc&, int, int, int, long long q) { xout[q] = T(x[q]); });
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
