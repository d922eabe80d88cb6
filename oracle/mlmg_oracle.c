/*
 * mlmg_oracle.c -- CPU restatement of AMReX's cell-centred MLMG solve
 * (MLPoisson / MLABecLaplacian, single AMR level) in plain C.
 *
 * TEST INFRASTRUCTURE ONLY.  This is the oracle the GPU library is checked
 * against: only the tests, the smoke check and the CPU-baseline leg of the
 * benchmark load it.  It is pinned against golden fixtures produced by the
 * reference itself (the .npz files in tests/golden, made by
 * tests/golden/make_golden.py through oracle/ref/ref_driver.cpp).
 *
 * Every routine follows one reference routine; the file:line of the
 * reference (AMReX 24.10, paths relative to the AMReX source tree) is given
 * beside it.  Storage mirrors a MultiFab: one FAB per box, the box grown by
 * its ghost width, x fastest.  Faces are indexed by AMReX's Orientation
 * numbering: 0..2 = low x,y,z ; 3..5 = high x,y,z.
 *
 * All arithmetic is IEEE double, evaluated in the reference's order; build
 * with -ffp-contract=off so no FMA is introduced.
 */
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#include "mlmg_oracle.h"

#define LO_DIRICHLET 101
#define LO_NEUMANN 102
#define LO_REFLECT_ODD 103
#define LO_PERIODIC 200

/* mask values, Src/Boundary/AMReX_BndryData.H:44 */
#define MASK_COVERED 0
#define MASK_NOT_COVERED 1
#define MASK_OUTSIDE 2

typedef struct { int lo[3], hi[3]; } Box;

static int blen(const Box* b, int d) { return b->hi[d] - b->lo[d] + 1; }
static long long bnpts(const Box* b) { return (long long)blen(b, 0) * blen(b, 1) * blen(b, 2); }
static int floordiv(int a, int r) { return (a >= 0) ? a / r : -((-a + r - 1) / r); }
static Box bcoarsen(Box b, int r) {
    for (int d = 0; d < 3; ++d) { b.lo[d] = floordiv(b.lo[d], r); b.hi[d] = floordiv(b.hi[d], r); }
    return b;
}
static int bequal(const Box* a, const Box* b) { return memcmp(a, b, sizeof(Box)) == 0; }

/* Box::coarsenable(refrat, min_width), Src/Base/AMReX_Box.H:745-755 */
static int bcoarsenable(const Box* b, int r, int min_width) {
    for (int d = 0; d < 3; ++d) { if (blen(b, d) < r * min_width) return 0; }
    Box c = bcoarsen(*b, r);
    for (int d = 0; d < 3; ++d) { c.lo[d] *= r; c.hi[d] = (c.hi[d] + 1) * r - 1; }
    return bequal(&c, b);
}

/* ---------------------------------------------------------------- FAB ---- */
typedef struct {
    Box bx;      /* fab's box in its own index space (nodal boxes include hi+1) */
    int ng;      /* ghost width */
    int sx, sy, sz;
    double* p;
} Fab;

static void fab_define(Fab* f, Box bx, int ng) {
    f->bx = bx; f->ng = ng;
    f->sx = blen(&bx, 0) + 2 * ng; f->sy = blen(&bx, 1) + 2 * ng; f->sz = blen(&bx, 2) + 2 * ng;
    f->p = (double*)calloc((size_t)f->sx * f->sy * f->sz, sizeof(double));
}
static size_t fab_size(const Fab* f) { return (size_t)f->sx * f->sy * f->sz; }
static inline double* fab_at(const Fab* f, int i, int j, int k) {
    return f->p + (((size_t)(k - f->bx.lo[2] + f->ng)) * f->sy + (size_t)(j - f->bx.lo[1] + f->ng)) * f->sx
                + (size_t)(i - f->bx.lo[0] + f->ng);
}
#define A(f, i, j, k) (*fab_at((f), (i), (j), (k)))

typedef struct { int nbox; Fab* fab; } MF;

static void mf_define(MF* m, int nbox, const Box* boxes, int ng, int nodal_dir) {
    m->nbox = nbox;
    m->fab = (Fab*)calloc((size_t)nbox, sizeof(Fab));
    for (int b = 0; b < nbox; ++b) {
        Box bx = boxes[b];
        if (nodal_dir >= 0) bx.hi[nodal_dir] += 1;
        fab_define(&m->fab[b], bx, ng);
    }
}
static void mf_free(MF* m) {
    for (int b = 0; b < m->nbox; ++b) free(m->fab[b].p);
    free(m->fab); m->fab = NULL; m->nbox = 0;
}
static void mf_setval(MF* m, double v) {
    for (int b = 0; b < m->nbox; ++b) {
        size_t n = fab_size(&m->fab[b]);
        for (size_t q = 0; q < n; ++q) m->fab[b].p[q] = v;
    }
}
#define FOR_VALID(f, i, j, k) \
    for (int k = (f)->bx.lo[2]; k <= (f)->bx.hi[2]; ++k) \
    for (int j = (f)->bx.lo[1]; j <= (f)->bx.hi[1]; ++j) \
    for (int i = (f)->bx.lo[0]; i <= (f)->bx.hi[0]; ++i)

/* The same loop with the k planes spread over OpenMP threads.  Used only
 * where every iteration writes its own cell and reads cells nobody writes
 * in that loop, so results do not depend on the thread count. */
#define FOR_VALID_PAR(f, i, j, k) \
    _Pragma("omp parallel for schedule(static)") \
    for (int k = (f)->bx.lo[2]; k <= (f)->bx.hi[2]; ++k) \
    for (int j = (f)->bx.lo[1]; j <= (f)->bx.hi[1]; ++j) \
    for (int i = (f)->bx.lo[0]; i <= (f)->bx.hi[0]; ++i)

/* --------------------------------------------- BoxArray::maxSize ---------- */
/* BoxList::maxSize, Src/Base/AMReX_BoxList.cpp:765-824 */
static int max_size(const Box* in, int nin, int chunk, Box** out) {
    int cap = 64, n = 0;
    Box* res = (Box*)malloc(sizeof(Box) * cap);
    for (int q = 0; q < nin; ++q) {
        const Box* bx = &in[q];
        int ratio[3] = {1, 1, 1}, numblk[3] = {1, 1, 1}, extra[3] = {0, 0, 0}, sz[3];
        for (int d = 0; d < 3; ++d) {
            sz[d] = blen(bx, d);
            if (blen(bx, d) > chunk) {
                int bs = chunk, nlen = blen(bx, d);
                while ((bs % 2 == 0) && (nlen % 2 == 0)) { ratio[d] *= 2; bs /= 2; nlen /= 2; }
                numblk[d] = (nlen + bs - 1) / bs;
                sz[d] = nlen / numblk[d];
                extra[d] = nlen - sz[d] * numblk[d];
            }
        }
        for (int k = 0; k < numblk[2]; ++k)
        for (int j = 0; j < numblk[1]; ++j)
        for (int i = 0; i < numblk[0]; ++i) {
            int idx[3] = {i, j, k};
            Box nb;
            for (int d = 0; d < 3; ++d) {
                if (numblk[d] == 1) { nb.lo[d] = bx->lo[d]; nb.hi[d] = bx->hi[d]; continue; }
                int b = idx[d];
                int lo = (b < extra[d]) ? b * (sz[d] + 1) * ratio[d] : (b * sz[d] + extra[d]) * ratio[d];
                int hi = (b < extra[d]) ? lo + (sz[d] + 1) * ratio[d] - 1 : lo + sz[d] * ratio[d] - 1;
                nb.lo[d] = lo + bx->lo[d]; nb.hi[d] = hi + bx->lo[d];
            }
            if (n == cap) { cap *= 2; res = (Box*)realloc(res, sizeof(Box) * cap); }
            res[n++] = nb;
        }
    }
    *out = res;
    return n;
}

/* --------------------------------------------------- MG hierarchy ---------- */
typedef struct {
    Box domain;
    double dx[3], dxinv[3];
    int nbox;
    Box* boxes;
    int* boxmap;        /* domain cell -> box index, -1 if uncovered */
    int* bct_p;         /* per box, per face: BC type */
    double* bcl_p;      /* per box, per face: BC location */
    Fab* mask;          /* [nbox*6]: over the face-adjacent outside cells */
    Fab* fco;           /* [nbox*6]: f coefficient over the face-adjacent inside cells */
    int derived;        /* grids made by coarsening the level-0 BoxArray (they share its data,
                           so MFIter over two such levels is safe: amrex::isMFIterSafe) */
    MF acoef, bcoef[3];
} Level;

typedef struct {
    int nlev;
    Level lev[32];
    int n[3];
    int periodic[3];
    double prob_lo[3], prob_hi[3];
    int lobc[3], hibc[3];
    int maxorder;
    int is_abec;
    double alpha, beta;
    double dx0[3];
    int crse_ratio;     /* refinement ratio to the next coarser AMR level (1 at AMR level 0) */
} Hier;

static void level_geom(Level* L, const Box* dom, const Hier* H) {
    L->domain = *dom;
    for (int d = 0; d < 3; ++d) {
        /* Geometry cell size, Src/Base/AMReX_Geometry.H:406-407 */
        L->dx[d] = (H->prob_hi[d] - H->prob_lo[d]) / (double)blen(dom, d);
        L->dxinv[d] = 1.0 / L->dx[d];
    }
}

/* MLLinOpT::defineGrids, amrex level 0 only,
 * Src/LinearSolvers/MLMG/AMReX_MLLinOp.H:793-1165 (no semicoarsening, no
 * hidden direction).  Consolidation only changes the distribution map, so
 * with a single rank it leaves the box arrays as plain coarsenings. */
static int define_grids(Hier* H, const Box* ba, int nba, const OracleOptions* o) {
    Box dom = {{0, 0, 0}, {H->n[0] - 1, H->n[1] - 1, H->n[2] - 1}};
    long long npts0 = 0;
    for (int b = 0; b < nba; ++b) npts0 += bnpts(&ba[b]);
    const int domain_covered = (npts0 == bnpts(&dom));
    const int mg_box_min_width = 2, mg_domain_min_width = 2;
    int nlev = 0;
    Level* L0 = &H->lev[nlev++];
    L0->nbox = nba; L0->boxes = (Box*)malloc(sizeof(Box) * nba);
    memcpy(L0->boxes, ba, sizeof(Box) * nba);
    L0->derived = 1;
    level_geom(L0, &dom, H);

    Box aggbox; int aggable = 0;
    if (nba > 1 && o->agg) {
        if (domain_covered) { aggbox = dom; aggable = 1; }
        else {
            aggbox = ba[0];
            for (int b = 1; b < nba; ++b)
                for (int d = 0; d < 3; ++d) {
                    if (ba[b].lo[d] < aggbox.lo[d]) aggbox.lo[d] = ba[b].lo[d];
                    if (ba[b].hi[d] > aggbox.hi[d]) aggbox.hi[d] = ba[b].hi[d];
                }
            aggable = (bnpts(&aggbox) == npts0);
        }
    }
    int all_coarsenable(const Box* bs, int nb, int r, int mw);
    if (o->agg && aggable) {
        Box dbx = dom, bbx = aggbox;
        const double nbxs = (double)nba;
        const double threshold_npts = (double)o->agg_grid_size * o->agg_grid_size * o->agg_grid_size;
        Box domainboxes[64], boundboxes[64];
        int agg_flag[64], accum[64];
        int nd = 0;
        domainboxes[nd] = dbx; boundboxes[nd] = bbx; agg_flag[nd] = 0; accum[nd] = 1; nd++;
        for (int lev = 0; lev < o->max_coarsening_level; ++lev) {
            if (!(bcoarsenable(&dbx, 2, mg_domain_min_width) && bcoarsenable(&bbx, 2, mg_box_min_width))) break;
            accum[nd] = accum[nd - 1] * 2;
            dbx = bcoarsen(dbx, 2); bbx = bcoarsen(bbx, 2);
            domainboxes[nd] = dbx; boundboxes[nd] = bbx;
            agg_flag[nd] = ((double)bnpts(&bbx) / nbxs) < 0.999 * threshold_npts;
            nd++;
        }
        int agged = 0;
        for (int lev = 1; lev < nd; ++lev) {
            Level* Lp = &H->lev[nlev - 1];
            Level* L = &H->lev[nlev];
            if (!agged && !agg_flag[lev] && all_coarsenable(ba, nba, accum[lev], mg_box_min_width)) {
                L->nbox = nba; L->boxes = (Box*)malloc(sizeof(Box) * nba);
                for (int b = 0; b < nba; ++b) L->boxes[b] = bcoarsen(ba[b], accum[lev]);
                L->derived = 1;
            } else {
                int cr = blen(&domainboxes[lev - 1], 0) / blen(&domainboxes[lev], 0);
                if (!all_coarsenable(Lp->boxes, Lp->nbox, cr, 1)) break;
                Box* nb = NULL;
                L->nbox = max_size(&boundboxes[lev], 1, o->agg_grid_size, &nb);
                L->boxes = nb;
                L->derived = 0;
                agged = 1;
            }
            level_geom(L, &domainboxes[lev], H);
            nlev++;
        }
    } else {
        int rr = 1;
        for (int lev = 0; lev < o->max_coarsening_level; ++lev) {
            int r2 = rr * 2;
            if (!(bcoarsenable(&dom, r2, mg_domain_min_width) && all_coarsenable(ba, nba, r2, mg_box_min_width))) break;
            rr = r2;
            Level* L = &H->lev[nlev];
            Box cd = bcoarsen(dom, rr);
            L->nbox = nba; L->boxes = (Box*)malloc(sizeof(Box) * nba);
            for (int b = 0; b < nba; ++b) L->boxes[b] = bcoarsen(ba[b], rr);
            L->derived = 1;
            level_geom(L, &cd, H);
            nlev++;
        }
    }
    H->nlev = nlev;
    return nlev;
}

int all_coarsenable(const Box* bs, int nb, int r, int mw) {
    for (int b = 0; b < nb; ++b) if (!bcoarsenable(&bs[b], r, mw)) return 0;
    return 1;
}

static void build_boxmap(Level* L) {
    const Box* d = &L->domain;
    size_t n = (size_t)bnpts(d);
    L->boxmap = (int*)malloc(sizeof(int) * n);
    for (size_t q = 0; q < n; ++q) L->boxmap[q] = -1;
    int nx = blen(d, 0), ny = blen(d, 1);
    for (int b = 0; b < L->nbox; ++b) {
        const Box* bx = &L->boxes[b];
        for (int k = bx->lo[2]; k <= bx->hi[2]; ++k)
        for (int j = bx->lo[1]; j <= bx->hi[1]; ++j)
        for (int i = bx->lo[0]; i <= bx->hi[0]; ++i)
            L->boxmap[((size_t)(k - d->lo[2]) * ny + (j - d->lo[1])) * nx + (i - d->lo[0])] = b;
    }
}

/* box index covering cell (i,j,k) after periodic wrapping into the domain;
 * returns -1 if none; (*pi,*pj,*pk) get the wrapped index */
static int locate(const Level* L, const int* periodic, int i, int j, int k, int* pi, int* pj, int* pk) {
    int c[3] = {i, j, k};
    const Box* d = &L->domain;
    for (int q = 0; q < 3; ++q) {
        int n = blen(d, q);
        if (c[q] < d->lo[q] || c[q] > d->hi[q]) {
            if (!periodic[q]) return -1;
            c[q] = d->lo[q] + ((c[q] - d->lo[q]) % n + n) % n;
        }
    }
    *pi = c[0]; *pj = c[1]; *pk = c[2];
    int nx = blen(d, 0), ny = blen(d, 1);
    return L->boxmap[((size_t)(c[2] - d->lo[2]) * ny + (c[1] - d->lo[1])) * nx + (c[0] - d->lo[0])];
}

/* poly_interp_coeff, Src/Boundary/AMReX_LOUtil_K.H:22-37 */
static void poly_interp_coeff(double xInt, const double* x, int N, double* c) {
    for (int j = 0; j < N; ++j) {
        double num = 1.0, den = 1.0;
        for (int i = 0; i < N; ++i) {
            if (i != j) { num *= xInt - x[i]; den *= x[j] - x[i]; }
        }
        c[j] = num / den;
    }
}

/* face-adjacent outside cell box (amrex::adjCell) of face f of box b */
static Box adj_cell(const Box* b, int f) {
    int d = f % 3, hi = f >= 3;
    Box r = *b;
    if (hi) { r.lo[d] = b->hi[d] + 1; r.hi[d] = b->hi[d] + 1; }
    else { r.lo[d] = b->lo[d] - 1; r.hi[d] = b->lo[d] - 1; }
    return r;
}
static Box inside_layer(const Box* b, int f) {
    int d = f % 3, hi = f >= 3;
    Box r = *b;
    if (hi) r.lo[d] = b->hi[d]; else r.hi[d] = b->lo[d];
    return r;
}

/* MultiMask::define, Src/Boundary/AMReX_MultiMask.cpp:25-69 (cross stencil:
 * extent 0) ; MLMGBndryT::setBoxBC, AMReX_MLMGBndry.H:106-150 ;
 * mllinop_comp_interp_coef0_*, AMReX_MLLinOp_K.H:327-420 */
static void define_bc(Hier* H, Level* L, const OracleOptions* o) {
    int nb = L->nbox;
    L->bct_p = (int*)malloc(sizeof(int) * 6 * nb);
    L->bcl_p = (double*)malloc(sizeof(double) * 6 * nb);
    L->mask = (Fab*)calloc((size_t)6 * nb, sizeof(Fab));
    L->fco = (Fab*)calloc((size_t)6 * nb, sizeof(Fab));
    for (int b = 0; b < nb; ++b) {
        const Box* bx = &L->boxes[b];
        for (int f = 0; f < 6; ++f) {
            int d = f % 3, hi = f >= 3;
            int* bct = &L->bct_p[6 * b + f];
            double* bcl = &L->bcl_p[6 * b + f];
            int on_domain = hi ? (L->domain.hi[d] == bx->hi[d]) : (L->domain.lo[d] == bx->lo[d]);
            if (on_domain && !H->periodic[d]) {
                *bcl = 0.0;  /* default domain BC location */
                *bct = hi ? H->hibc[d] : H->lobc[d];
            } else {
                *bct = LO_DIRICHLET; /* default coarse/fine BC type */
                /* MLMGBndryT::setBoxBC (AMReX_MLMGBndry.H:106-150): 0.5 * ratio * dx of the
                   AMR level (ratio 1 at AMR level 0) */
                *bcl = 0.5 * (double)(H->crse_ratio > 0 ? H->crse_ratio : 1) * H->dx0[d];
            }
            Box ab = adj_cell(bx, f);
            Fab* m = &L->mask[6 * b + f];
            fab_define(m, ab, 0);
            FOR_VALID(m, i, j, k) {
                int c[3] = {i, j, k}, in_dom = 1;
                for (int q = 0; q < 3; ++q)
                    if (!H->periodic[q] && (c[q] < L->domain.lo[q] || c[q] > L->domain.hi[q])) in_dom = 0;
                double v;
                if (!in_dom) v = MASK_OUTSIDE;
                else {
                    int wi, wj, wk;
                    v = (locate(L, H->periodic, i, j, k, &wi, &wj, &wk) >= 0) ? MASK_COVERED : MASK_NOT_COVERED;
                }
                A(m, i, j, k) = v;
            }
            Fab* fc = &L->fco[6 * b + f];
            Box il = inside_layer(bx, f);
            fab_define(fc, il, 0);
            int nx_len = blen(bx, d);
            double coef[4] = {0, 0, 0, 0};
            if (*bct == LO_DIRICHLET) {
                int NX = (nx_len + 1 < H->maxorder) ? nx_len + 1 : H->maxorder;
                double x[4] = {-(*bcl) * L->dxinv[d], 0.5, 1.5, 2.5};
                poly_interp_coeff(-0.5, x, NX, coef);
            }
            int s = hi ? -1 : 1;
            FOR_VALID(fc, i, j, k) {
                int oi = i, oj = j, ok = k;
                if (d == 0) oi -= s; else if (d == 1) oj -= s; else ok -= s;
                double mk = A(m, oi, oj, ok);
                double v = 0.0;
                if (*bct == LO_NEUMANN) v = 1.0;
                else if (*bct == LO_REFLECT_ODD) v = (mk > 0) ? 1.0 : 0.0;
                else if (*bct == LO_DIRICHLET) v = (mk > 0) ? coef[1] : 0.0;
                A(fc, i, j, k) = v;
            }
            (void)o;
        }
    }
}

/* ------------------------------------------------ FillBoundary ------------ */
/* FabArray::FillBoundary (single rank): each ghost cell covered by the valid
 * region of a box (after periodic shifts) gets that cell's value.  The
 * ``cross`` flag only trims the MPI send/receive tags
 * (Src/Base/AMReX_FabArrayBase.cpp:814-870); the local-copy tags built at
 * :745-790 are not trimmed, so on one rank edge and corner ghosts are filled
 * too, whatever ``cross`` says.  Local copies: Src/Base/AMReX_FBI.H:209-334. */
static void fill_boundary(const Level* L, const int* periodic, MF* m, int cross) {
    (void)cross;
    for (int b = 0; b < m->nbox; ++b) {
        Fab* f = &m->fab[b];
        const Box* vb = &L->boxes[b];
        int ng = f->ng;
        for (int k = vb->lo[2] - ng; k <= vb->hi[2] + ng; ++k)
        for (int j = vb->lo[1] - ng; j <= vb->hi[1] + ng; ++j)
        for (int i = vb->lo[0] - ng; i <= vb->hi[0] + ng; ++i) {
            int out = (i < vb->lo[0] || i > vb->hi[0]) + (j < vb->lo[1] || j > vb->hi[1]) +
                      (k < vb->lo[2] || k > vb->hi[2]);
            if (out == 0) continue;
            int wi, wj, wk;
            int src = locate(L, periodic, i, j, k, &wi, &wj, &wk);
            if (src < 0) continue;
            A(f, i, j, k) = A(&m->fab[src], wi, wj, wk);
        }
    }
}

/* ------------------------------------------------------ applyBC ----------- */
/* MLCellLinOpT::applyBC, AMReX_MLCellLinOp.H:682-893 ; mllinop_apply_bc_*,
 * AMReX_MLLinOp_K.H:74-320.  bcval (may be NULL) holds the Dirichlet values
 * in the ghost cells of a grown-domain array. */
typedef struct { const double* v; int n[3]; } GrownGlobal;

static double gg_at(const GrownGlobal* g, int i, int j, int k) {
    return g->v[((size_t)(k + 1) * (g->n[1] + 2) + (j + 1)) * (g->n[0] + 2) + (i + 1)];
}

static void apply_bc(const Hier* H, const Level* L, MF* m, int inhomog, const GrownGlobal* bcval,
                     int skip_fillboundary, const Fab* bfab) {
    if (!skip_fillboundary) fill_boundary(L, H->periodic, m, 1);
    for (int b = 0; b < m->nbox; ++b) {
        Fab* phi = &m->fab[b];
        const Box* vb = &L->boxes[b];
        for (int f = 0; f < 6; ++f) {
            int d = f % 3, hi = f >= 3;
            int s = hi ? -1 : 1;
            int bct = L->bct_p[6 * b + f];
            double bcl = L->bcl_p[6 * b + f];
            const Fab* mk = &L->mask[6 * b + f];
            int bl = blen(vb, d);
            double coef[4] = {0, 0, 0, 0};
            int NX = 0;
            if (bct == LO_DIRICHLET) {
                NX = (bl + 1 < H->maxorder) ? bl + 1 : H->maxorder;
                double x[4] = {-bcl * L->dxinv[d], 0.5, 1.5, 2.5};
                poly_interp_coeff(-0.5, x, NX, coef);
            }
            FOR_VALID(mk, i, j, k) {
                if (!(A(mk, i, j, k) > 0)) continue;
                int di = (d == 0) ? s : 0, dj = (d == 1) ? s : 0, dk = (d == 2) ? s : 0;
                if (bct == LO_NEUMANN) {
                    A(phi, i, j, k) = A(phi, i + di, j + dj, k + dk);
                } else if (bct == LO_REFLECT_ODD) {
                    A(phi, i, j, k) = -A(phi, i + di, j + dj, k + dk);
                } else if (bct == LO_DIRICHLET) {
                    double tmp = 0.0;
                    for (int q = 1; q < NX; ++q) tmp += A(phi, i + q * di, j + q * dj, k + q * dk) * coef[q];
                    A(phi, i, j, k) = tmp;
                    if (inhomog) {
                        /* boundary values per box face (a fine AMR level: coarse/fine
                           values from InterpBndryData, physical values from the level BC),
                           or the level-0 values in the ghosts of a grown global array */
                        double bv = bfab ? A(&bfab[6 * b + f], i, j, k) : (bcval ? gg_at(bcval, i, j, k) : 0.0);
                        A(phi, i, j, k) += bv * coef[0];
                    }
                }
            }
        }
    }
}

/* ------------------------------------------------------ operators --------- */
/* mlabeclap_adotx, AMReX_MLABecLap_3D_K.H:7-28 ; MLABecLaplacianT::Fapply,
 * AMReX_MLABecLaplacian.H:775-854 ; mlpoisson_adotx,
 * AMReX_MLPoisson_3D_K.H:7-16 ; MLPoissonT::Fapply, AMReX_MLPoisson.H:180-310 */
static void fapply(const Hier* H, const Level* L, MF* out, const MF* in) {
    for (int b = 0; b < out->nbox; ++b) {
        Fab* y = &out->fab[b];
        const Fab* x = &in->fab[b];
        if (H->is_abec) {
            const double dhx = H->beta * L->dxinv[0] * L->dxinv[0];
            const double dhy = H->beta * L->dxinv[1] * L->dxinv[1];
            const double dhz = H->beta * L->dxinv[2] * L->dxinv[2];
            const Fab* a = &L->acoef.fab[b];
            const Fab* bX = &L->bcoef[0].fab[b];
            const Fab* bY = &L->bcoef[1].fab[b];
            const Fab* bZ = &L->bcoef[2].fab[b];
            FOR_VALID_PAR(y, i, j, k) {
                A(y, i, j, k) = H->alpha * A(a, i, j, k) * A(x, i, j, k)
                    - dhx * (A(bX, i + 1, j, k) * (A(x, i + 1, j, k) - A(x, i, j, k))
                           - A(bX, i, j, k) * (A(x, i, j, k) - A(x, i - 1, j, k)))
                    - dhy * (A(bY, i, j + 1, k) * (A(x, i, j + 1, k) - A(x, i, j, k))
                           - A(bY, i, j, k) * (A(x, i, j, k) - A(x, i, j - 1, k)))
                    - dhz * (A(bZ, i, j, k + 1) * (A(x, i, j, k + 1) - A(x, i, j, k))
                           - A(bZ, i, j, k) * (A(x, i, j, k) - A(x, i, j, k - 1)));
            }
        } else {
            const double dhx = L->dxinv[0] * L->dxinv[0];
            const double dhy = L->dxinv[1] * L->dxinv[1];
            const double dhz = L->dxinv[2] * L->dxinv[2];
            FOR_VALID_PAR(y, i, j, k) {
                A(y, i, j, k) = dhx * (A(x, i - 1, j, k) - 2.0 * A(x, i, j, k) + A(x, i + 1, j, k))
                    + dhy * (A(x, i, j - 1, k) - 2.0 * A(x, i, j, k) + A(x, i, j + 1, k))
                    + dhz * (A(x, i, j, k - 1) - 2.0 * A(x, i, j, k) + A(x, i, j, k + 1));
            }
        }
    }
}

/* abec_gsrb, AMReX_MLABecLap_3D_K.H:208-264 ; MLABecLaplacianT::Fsmooth,
 * AMReX_MLABecLaplacian.H:856-1126 ; mlpoisson_gsrb, AMReX_MLPoisson_3D_K.H:153-196 ;
 * MLPoissonT::Fsmooth, AMReX_MLPoisson.H:364-855 */
static void fsmooth(const Hier* H, const Level* L, MF* sol, const MF* rhs, int redblack) {
    const double omega = 1.15;
    for (int b = 0; b < sol->nbox; ++b) {
        Fab* phi = &sol->fab[b];
        const Fab* r = &rhs->fab[b];
        const Box* vb = &L->boxes[b];
        const Fab* m[6]; const Fab* fc[6];
        for (int f = 0; f < 6; ++f) { m[f] = &L->mask[6 * b + f]; fc[f] = &L->fco[6 * b + f]; }
        double dhx, dhy, dhz;
        if (H->is_abec) {
            dhx = H->beta / (L->dx[0] * L->dx[0]);
            dhy = H->beta / (L->dx[1] * L->dx[1]);
            dhz = H->beta / (L->dx[2] * L->dx[2]);
        } else {
            dhx = L->dxinv[0] * L->dxinv[0];
            dhy = L->dxinv[1] * L->dxinv[1];
            dhz = L->dxinv[2] * L->dxinv[2];
        }
        FOR_VALID_PAR(r, i, j, k) {
            if ((i + j + k + redblack) % 2 != 0) continue;
            double cf0 = (i == vb->lo[0] && A(m[0], vb->lo[0] - 1, j, k) > 0) ? A(fc[0], vb->lo[0], j, k) : 0.0;
            double cf1 = (j == vb->lo[1] && A(m[1], i, vb->lo[1] - 1, k) > 0) ? A(fc[1], i, vb->lo[1], k) : 0.0;
            double cf2 = (k == vb->lo[2] && A(m[2], i, j, vb->lo[2] - 1) > 0) ? A(fc[2], i, j, vb->lo[2]) : 0.0;
            double cf3 = (i == vb->hi[0] && A(m[3], vb->hi[0] + 1, j, k) > 0) ? A(fc[3], vb->hi[0], j, k) : 0.0;
            double cf4 = (j == vb->hi[1] && A(m[4], i, vb->hi[1] + 1, k) > 0) ? A(fc[4], i, vb->hi[1], k) : 0.0;
            double cf5 = (k == vb->hi[2] && A(m[5], i, j, vb->hi[2] + 1) > 0) ? A(fc[5], i, j, vb->hi[2]) : 0.0;
            if (H->is_abec) {
                const Fab* a = &L->acoef.fab[b];
                const Fab* bX = &L->bcoef[0].fab[b];
                const Fab* bY = &L->bcoef[1].fab[b];
                const Fab* bZ = &L->bcoef[2].fab[b];
                double gamma = H->alpha * A(a, i, j, k)
                    + dhx * (A(bX, i, j, k) + A(bX, i + 1, j, k))
                    + dhy * (A(bY, i, j, k) + A(bY, i, j + 1, k))
                    + dhz * (A(bZ, i, j, k) + A(bZ, i, j, k + 1));
                double g_m_d = gamma
                    - (dhx * (A(bX, i, j, k) * cf0 + A(bX, i + 1, j, k) * cf3)
                     + dhy * (A(bY, i, j, k) * cf1 + A(bY, i, j + 1, k) * cf4)
                     + dhz * (A(bZ, i, j, k) * cf2 + A(bZ, i, j, k + 1) * cf5));
                double rho = dhx * (A(bX, i, j, k) * A(phi, i - 1, j, k) + A(bX, i + 1, j, k) * A(phi, i + 1, j, k))
                           + dhy * (A(bY, i, j, k) * A(phi, i, j - 1, k) + A(bY, i, j + 1, k) * A(phi, i, j + 1, k))
                           + dhz * (A(bZ, i, j, k) * A(phi, i, j, k - 1) + A(bZ, i, j, k + 1) * A(phi, i, j, k + 1));
                double res = A(r, i, j, k) - (gamma * A(phi, i, j, k) - rho);
                A(phi, i, j, k) = A(phi, i, j, k) + omega / g_m_d * res;
            } else {
                const double gamma = -2.0 * (dhx + dhy + dhz);
                double g_m_d = gamma + dhx * (cf0 + cf3) + dhy * (cf1 + cf4) + dhz * (cf2 + cf5);
                double res = A(r, i, j, k) - gamma * A(phi, i, j, k)
                    - dhx * (A(phi, i - 1, j, k) + A(phi, i + 1, j, k))
                    - dhy * (A(phi, i, j - 1, k) + A(phi, i, j + 1, k))
                    - dhz * (A(phi, i, j, k - 1) + A(phi, i, j, k + 1));
                A(phi, i, j, k) = A(phi, i, j, k) + omega / g_m_d * res;
            }
        }
    }
}

/* mlabeclap_normalize, AMReX_MLABecLap_3D_K.H:58-75 (MLPoisson's normalize is a
 * no-op in 3-D, AMReX_MLPoisson.H:311-364) */
static void normalize(const Hier* H, const Level* L, MF* x) {
    if (!H->is_abec) return;
    const double dhx = H->beta * L->dxinv[0] * L->dxinv[0];
    const double dhy = H->beta * L->dxinv[1] * L->dxinv[1];
    const double dhz = H->beta * L->dxinv[2] * L->dxinv[2];
    for (int b = 0; b < x->nbox; ++b) {
        Fab* f = &x->fab[b];
        const Fab* a = &L->acoef.fab[b];
        const Fab* bX = &L->bcoef[0].fab[b];
        const Fab* bY = &L->bcoef[1].fab[b];
        const Fab* bZ = &L->bcoef[2].fab[b];
        Box vb = L->boxes[b];
#pragma omp parallel for schedule(static)
        for (int k = vb.lo[2]; k <= vb.hi[2]; ++k)
        for (int j = vb.lo[1]; j <= vb.hi[1]; ++j)
        for (int i = vb.lo[0]; i <= vb.hi[0]; ++i) {
            A(f, i, j, k) /= H->alpha * A(a, i, j, k)
                + dhx * (A(bX, i, j, k) + A(bX, i + 1, j, k))
                + dhy * (A(bY, i, j, k) + A(bY, i, j + 1, k))
                + dhz * (A(bZ, i, j, k) + A(bZ, i, j, k + 1));
        }
    }
}

/* ------------------------------------------------- BLAS-1 (valid cells) --- */
static double mf_norminf(const Level* L, const MF* m) {
    double r = 0.0;
    for (int b = 0; b < m->nbox; ++b) {
        Box vb = L->boxes[b];
        const Fab* f = &m->fab[b];
        for (int k = vb.lo[2]; k <= vb.hi[2]; ++k)
        for (int j = vb.lo[1]; j <= vb.hi[1]; ++j)
        for (int i = vb.lo[0]; i <= vb.hi[0]; ++i) { double v = fabs(A(f, i, j, k)); if (v > r) r = v; }
    }
    return r;
}
static double mf_dot(const Level* L, const MF* x, const MF* y) {
    double r = 0.0;
    for (int b = 0; b < x->nbox; ++b) {
        Box vb = L->boxes[b];
        for (int k = vb.lo[2]; k <= vb.hi[2]; ++k)
        for (int j = vb.lo[1]; j <= vb.hi[1]; ++j)
        for (int i = vb.lo[0]; i <= vb.hi[0]; ++i) r += A(&x->fab[b], i, j, k) * A(&y->fab[b], i, j, k);
    }
    return r;
}
static double mf_sum(const Level* L, const MF* x) {
    double r = 0.0;
    for (int b = 0; b < x->nbox; ++b) {
        Box vb = L->boxes[b];
        for (int k = vb.lo[2]; k <= vb.hi[2]; ++k)
        for (int j = vb.lo[1]; j <= vb.hi[1]; ++j)
        for (int i = vb.lo[0]; i <= vb.hi[0]; ++i) r += A(&x->fab[b], i, j, k);
    }
    return r;
}
/* dst = op(dst, src) over valid cells; op: 0 copy, 1 add, 2 dst+=a*src
 * (Saxpy), 3 dst = src + a*dst (Xpay) ; AMReX_FabArrayUtility.H:1630-1660 */
static void mf_axpy(const Level* L, MF* dst, double a, const MF* src, int op) {
    for (int b = 0; b < dst->nbox; ++b) {
        Box vb = L->boxes[b];
        Fab* d = &dst->fab[b];
        const Fab* s = &src->fab[b];
#pragma omp parallel for schedule(static)
        for (int k = vb.lo[2]; k <= vb.hi[2]; ++k)
        for (int j = vb.lo[1]; j <= vb.hi[1]; ++j)
        for (int i = vb.lo[0]; i <= vb.hi[0]; ++i) {
            double* p = fab_at(d, i, j, k);
            double v = A(s, i, j, k);
            if (op == 0) *p = v;
            else if (op == 1) *p += v;
            else if (op == 2) *p += a * v;
            else *p = v + a * *p;
        }
    }
}
static void mf_plus(const Level* L, MF* dst, double v) {
    for (int b = 0; b < dst->nbox; ++b) {
        Box vb = L->boxes[b];
        for (int k = vb.lo[2]; k <= vb.hi[2]; ++k)
        for (int j = vb.lo[1]; j <= vb.hi[1]; ++j)
        for (int i = vb.lo[0]; i <= vb.hi[0]; ++i) A(&dst->fab[b], i, j, k) += v;
    }
}

/* -------------------------------------------- inter-level transfers ------- */
/* average_down / amrex_avgdown, Src/Base/AMReX_MultiFabUtil_3D_C.H:375-392
 * (the BoxArrays may differ after agglomeration: the reference then averages
 * into a temporary on the coarsened fine layout and ParallelCopies, which
 * gives the same values as reading the fine level by global index). */
static void restriction(const Hier* H, const Level* Lf, const MF* fine, const Level* Lc, MF* crse) {
    for (int b = 0; b < crse->nbox; ++b) {
        Fab* c = &crse->fab[b];
        Box vb = Lc->boxes[b];
#pragma omp parallel for schedule(static)
        for (int k = vb.lo[2]; k <= vb.hi[2]; ++k)
        for (int j = vb.lo[1]; j <= vb.hi[1]; ++j)
        for (int i = vb.lo[0]; i <= vb.hi[0]; ++i) {
            double s = 0;
            for (int kr = 0; kr < 2; ++kr)
            for (int jr = 0; jr < 2; ++jr)
            for (int ir = 0; ir < 2; ++ir) {
                int wi, wj, wk;
                int fb = locate(Lf, H->periodic, 2 * i + ir, 2 * j + jr, 2 * k + kr, &wi, &wj, &wk);
                s += A(&fine->fab[fb], wi, wj, wk);
            }
            A(c, i, j, k) = (1.0 / 8.0) * s;
        }
    }
}

/* MLCellLinOpT::interpolation (piecewise constant, add),
 * AMReX_MLCellLinOp.H:954-999 */
static void interp_add(const Hier* H, const Level* Lc, const MF* crse, const Level* Lf, MF* fine) {
    for (int b = 0; b < fine->nbox; ++b) {
        Fab* f = &fine->fab[b];
        Box vb = Lf->boxes[b];
#pragma omp parallel for schedule(static)
        for (int k = vb.lo[2]; k <= vb.hi[2]; ++k)
        for (int j = vb.lo[1]; j <= vb.hi[1]; ++j)
        for (int i = vb.lo[0]; i <= vb.hi[0]; ++i) {
            int wi, wj, wk;
            int cb = locate(Lc, H->periodic, floordiv(i, 2), floordiv(j, 2), floordiv(k, 2), &wi, &wj, &wk);
            A(f, i, j, k) += A(&crse->fab[cb], wi, wj, wk);
        }
    }
}

/* average_down_faces / amrex_avgdown_faces, Src/Base/AMReX_MultiFabUtil_3D_C.H:170-225 */
static void restrict_coeffs(const Hier* H, Level* Lf, Level* Lc) {
    const int nbc = Lc->nbox;
    mf_define(&Lc->acoef, nbc, Lc->boxes, 0, -1);
    for (int d = 0; d < 3; ++d) mf_define(&Lc->bcoef[d], nbc, Lc->boxes, 0, d);
    /* cell a: same as restriction; a_scalar == 0 gives zero */
    if (H->alpha == 0.0) {
        mf_setval(&Lc->acoef, 0.0);
    } else {
        restriction(H, Lf, &Lf->acoef, Lc, &Lc->acoef);
    }
    /* faces: locate the fine face through the fine cell on its high side, or
     * the low side for the domain's high face */
    for (int d = 0; d < 3; ++d) {
        for (int b = 0; b < nbc; ++b) {
            Fab* c = &Lc->bcoef[d].fab[b];
            FOR_VALID(c, i, j, k) {
                int ii = 2 * i, jj = 2 * j, kk = 2 * k;
                double s = 0;
                for (int r1 = 0; r1 < 2; ++r1)
                for (int r0 = 0; r0 < 2; ++r0) {
                    int fi = ii, fj = jj, fk = kk;
                    if (d == 0) { fj += r0; fk += r1; }
                    else if (d == 1) { fi += r0; fk += r1; }
                    else { fi += r0; fj += r1; }
                    /* the fine box holding the cell on the face's high side
                     * (low side for the domain's high face) owns this face */
                    int ci = fi, cj = fj, ck = fk;
                    if (d == 0 && ci > Lf->domain.hi[0]) ci--;
                    if (d == 1 && cj > Lf->domain.hi[1]) cj--;
                    if (d == 2 && ck > Lf->domain.hi[2]) ck--;
                    int wi, wj, wk;
                    int zero_per[3] = {0, 0, 0};
                    int found = locate(Lf, zero_per, ci, cj, ck, &wi, &wj, &wk);
                    s += A(&Lf->bcoef[d].fab[found], fi, fj, fk);
                }
                A(c, i, j, k) = s * (1.0 / 4.0);
            }
        }
    }
}

/* ------------------------------------------------------ solver state ------ */
typedef struct {
    Hier H;
    OracleOptions o;
    MF cor[32], res[32], rescor[32], cor_hold[32];
    MF sol, rhs;
    int cg_log[ORACLE_MAX_HIST];   /* BiCGStab iterations of every bottom solve (MLMGT::m_niters_cg) */
    int ncg;
    GrownGlobal bcval;
    int bottom_cg_iters_total;
    int singular;
    double volinv0, volinv_bottom;
    int bottom_mode;               /* MLMGT::bottom_solver, switched by bicgcg / cgbicg */
} Solver;

static void smooth(Solver* S, int lev, MF* sol, const MF* rhs, int skip_fb) {
    /* MLCellLinOpT::smooth, AMReX_MLCellLinOp.H:1204-1217 */
    for (int rb = 0; rb < 2; ++rb) {
        apply_bc(&S->H, &S->H.lev[lev], sol, 0, NULL, skip_fb, NULL);
        fsmooth(&S->H, &S->H.lev[lev], sol, rhs, rb);
        skip_fb = 0;
    }
}

/* correctionResidual (homogeneous): r = b - A x, AMReX_MLCellLinOp.H:1246-1270 */
static void correction_residual(Solver* S, int lev, MF* r, MF* x, const MF* b) {
    apply_bc(&S->H, &S->H.lev[lev], x, 0, NULL, 0, NULL);
    fapply(&S->H, &S->H.lev[lev], r, x);
    mf_axpy(&S->H.lev[lev], r, -1.0, b, 3);
}

/* solutionResidual, AMReX_MLCellLinOp.H:1219-1236 */
static void solution_residual(Solver* S, MF* r, MF* x, const MF* b) {
    apply_bc(&S->H, &S->H.lev[0], x, 1, &S->bcval, 0, NULL);
    fapply(&S->H, &S->H.lev[0], r, x);
    mf_axpy(&S->H.lev[0], r, -1.0, b, 3);
}

static void make_solvable(Solver* S, int lev, MF* m) {
    /* getSolvabilityOffset / fixSolvabilityByOffset, AMReX_MLCellLinOp.H:1559-1611 */
    double vi = (lev == 0) ? S->volinv0 : S->volinv_bottom;
    double off = mf_sum(&S->H.lev[lev], m) * vi;
    mf_plus(&S->H.lev[lev], m, -off);
}

/* MLCGSolverT::solve_bicgstab, AMReX_MLCGSolver.H:96-273 (zero initial guess) */
static int bicgstab(Solver* S, int lev, MF* sol, const MF* rhs, double eps_rel, double eps_abs, int maxiter,
                    int* niter) {
    Level* L = &S->H.lev[lev];
    Hier* H = &S->H;
    MF p, r, rh, v, t;
    mf_define(&p, L->nbox, L->boxes, 1, -1);
    mf_define(&r, L->nbox, L->boxes, 1, -1);
    mf_define(&rh, L->nbox, L->boxes, 0, -1);
    mf_define(&v, L->nbox, L->boxes, 0, -1);
    mf_define(&t, L->nbox, L->boxes, 0, -1);
    mf_axpy(L, &r, 0, rhs, 0);
    normalize(H, L, &r);
    mf_axpy(L, &rh, 0, &r, 0);
    double rnorm = mf_norminf(L, &r);
    const double rnorm0 = rnorm;
    int ret = 0, iter = 1;
    double rho_1 = 0, alpha = 0, omega = 0;
    if (rnorm0 == 0 || rnorm0 < eps_abs) {
        *niter = iter;
        goto done;
    }
    for (; iter <= maxiter; ++iter) {
        const double rho = mf_dot(L, &rh, &r);
        if (rho == 0) { ret = 1; break; }
        if (iter == 1) {
            mf_axpy(L, &p, 0, &r, 0);
        } else {
            const double beta = (rho / rho_1) * (alpha / omega);
            mf_axpy(L, &p, -omega, &v, 2);
            mf_axpy(L, &p, beta, &r, 3);
        }
        apply_bc(H, L, &p, 0, NULL, 0, NULL);
        fapply(H, L, &v, &p);
        normalize(H, L, &v);
        double rhTv = mf_dot(L, &rh, &v);
        if (rhTv != 0.0) alpha = rho / rhTv;
        else { ret = 2; break; }
        mf_axpy(L, sol, alpha, &p, 2);
        mf_axpy(L, &r, -alpha, &v, 2);
        rnorm = mf_norminf(L, &r);
        if (rnorm < eps_rel * rnorm0 || rnorm < eps_abs) break;
        apply_bc(H, L, &r, 0, NULL, 0, NULL);
        fapply(H, L, &t, &r);
        normalize(H, L, &t);
        double tt = mf_dot(L, &t, &t), tr = mf_dot(L, &t, &r);
        if (tt != 0.0) omega = tr / tt;
        else { ret = 3; break; }
        mf_axpy(L, sol, omega, &r, 2);
        mf_axpy(L, &r, -omega, &t, 2);
        rnorm = mf_norminf(L, &r);
        if (rnorm < eps_rel * rnorm0 || rnorm < eps_abs) break;
        if (omega == 0) { ret = 4; break; }
        rho_1 = rho;
    }
    if (ret == 0 && rnorm > eps_rel * rnorm0 && rnorm > eps_abs) ret = 8;
    if ((ret == 0 || ret == 8) && (rnorm < rnorm0)) {
        if (ret == 8) ret = 9;
    } else {
        mf_setval(sol, 0.0);
    }
    *niter = iter;
done:
    mf_free(&p); mf_free(&r); mf_free(&rh); mf_free(&v); mf_free(&t);
    return ret;
}

/* MLCGSolverT::solve_cg, AMReX_MLCGSolver.H:275-410 (zero initial guess,
 * unpreconditioned) */
static int conj_grad(Solver* S, int lev, MF* sol, const MF* rhs, double eps_rel, double eps_abs, int maxiter,
                     int* niter) {
    Level* L = &S->H.lev[lev];
    Hier* H = &S->H;
    MF p, r, q;
    mf_define(&p, L->nbox, L->boxes, 1, -1);
    mf_define(&r, L->nbox, L->boxes, 0, -1);
    mf_define(&q, L->nbox, L->boxes, 0, -1);
    mf_axpy(L, &r, 0, rhs, 0);
    double rnorm = mf_norminf(L, &r);
    const double rnorm0 = rnorm;
    int ret = 0, iter = 1;
    double rho_1 = 0;
    if (rnorm0 == 0 || rnorm0 < eps_abs) {
        *niter = iter;
        goto done;
    }
    for (; iter <= maxiter; ++iter) {
        const double rho = mf_dot(L, &r, &r);
        if (rho == 0) { ret = 1; break; }
        if (iter == 1) {
            mf_axpy(L, &p, 0, &r, 0);
        } else {
            const double beta = rho / rho_1;
            mf_axpy(L, &p, beta, &r, 3);          /* Xpay: p = r + beta p */
        }
        apply_bc(H, L, &p, 0, NULL, 0, NULL);
        fapply(H, L, &q, &p);
        const double pw = mf_dot(L, &p, &q);
        double alpha;
        if (pw != 0.0) alpha = rho / pw;
        else { ret = 1; break; }
        mf_axpy(L, sol, alpha, &p, 2);
        mf_axpy(L, &r, -alpha, &q, 2);
        rnorm = mf_norminf(L, &r);
        if (rnorm < eps_rel * rnorm0 || rnorm < eps_abs) break;
        rho_1 = rho;
    }
    if (ret == 0 && rnorm > eps_rel * rnorm0 && rnorm > eps_abs) ret = 8;
    if ((ret == 0 || ret == 8) && (rnorm < rnorm0)) {
        if (ret == 8) ret = 9;
    } else {
        mf_setval(sol, 0.0);
    }
    *niter = iter;
done:
    mf_free(&p); mf_free(&r); mf_free(&q);
    return ret;
}

/* MLMGT::actualBottomSolve, AMReX_MLMG.H:1500-1610 */
static void bottom_solve(Solver* S) {
    int lev = S->H.nlev - 1;
    Level* L = &S->H.lev[lev];
    MF* x = &S->cor[lev];
    MF* b = &S->res[lev];
    mf_setval(x, 0.0);
    if (S->o.bottom_solver == 1) { /* smoother */
        int skip = 1;
        for (int i = 0; i < S->o.nuf; ++i) { smooth(S, lev, x, b, skip); skip = 0; }
        if (S->ncg < ORACLE_MAX_HIST) S->cg_log[S->ncg] = 0;
        S->ncg++;
        return;
    }
    MF bb; int own = 0;
    const MF* bottom_b = b;
    if (S->singular) {
        mf_define(&bb, L->nbox, L->boxes, 0, -1);
        mf_axpy(L, &bb, 0, b, 0);
        make_solvable(S, lev, &bb);
        bottom_b = &bb; own = 1;
    }
    /* BottomSolver: 2 bicgstab, 3 cg, 4 bicgcg, 5 cgbicg; the second solver of
     * bicgcg / cgbicg runs when the first fails, and replaces it for good once
     * it succeeds (AMReX_MLMG.H:1563-1597) */
    const int kind = S->bottom_mode;
    const int cg_first = (kind == 3 || kind == 5);
    int it = 0;
    int ret = cg_first ? conj_grad(S, lev, x, bottom_b, S->o.bottom_reltol, -1.0, S->o.bottom_maxiter, &it)
                       : bicgstab(S, lev, x, bottom_b, S->o.bottom_reltol, -1.0, S->o.bottom_maxiter, &it);
    if (S->ncg < ORACLE_MAX_HIST) S->cg_log[S->ncg] = it;
    S->ncg++;
    if (ret != 0 && (kind == 4 || kind == 5)) {
        mf_setval(x, 0.0);
        ret = cg_first ? bicgstab(S, lev, x, bottom_b, S->o.bottom_reltol, -1.0, S->o.bottom_maxiter, &it)
                       : conj_grad(S, lev, x, bottom_b, S->o.bottom_reltol, -1.0, S->o.bottom_maxiter, &it);
        if (S->ncg < ORACLE_MAX_HIST) S->cg_log[S->ncg] = it;
        S->ncg++;
        if (ret == 0) S->bottom_mode = cg_first ? 2 : 3;
    }
    if (ret != 0 && ret != 9) mf_setval(x, 0.0);
    int n = (ret == 0) ? S->o.nub : S->o.nuf;
    for (int i = 0; i < n; ++i) smooth(S, lev, x, b, 0);
    if (own) mf_free(&bb);
}

/* MLMGT::mgVcycle, AMReX_MLMG.H:1306-1415, from MG level `top` down */
static void vcycle(Solver* S, int top) {
    int bottom = S->H.nlev - 1;
    for (int lev = top; lev < bottom; ++lev) {
        mf_setval(&S->cor[lev], 0.0);
        int skip = 1;
        for (int i = 0; i < S->o.nu1; ++i) { smooth(S, lev, &S->cor[lev], &S->res[lev], skip); skip = 0; }
        correction_residual(S, lev, &S->rescor[lev], &S->cor[lev], &S->res[lev]);
        restriction(&S->H, &S->H.lev[lev], &S->rescor[lev], &S->H.lev[lev + 1], &S->res[lev + 1]);
    }
    bottom_solve(S);
    for (int lev = bottom - 1; lev >= top; --lev) {
        interp_add(&S->H, &S->H.lev[lev + 1], &S->cor[lev + 1], &S->H.lev[lev], &S->cor[lev]);
        for (int i = 0; i < S->o.nu2; ++i) smooth(S, lev, &S->cor[lev], &S->res[lev], 0);
    }
}

/* MLCellLinOpT::interpAssign, AMReX_MLCellLinOp.H:1003-1100, with
 * mlmg_lin_cc_interp_r2 (AMReX_MLMG_3D_K.H:7-37): cor[lev] = trilinear
 * prolongation of cor[lev+1] on every fine box.  When MFIter over both
 * levels is safe the coarse ghosts are refreshed by FillBoundary and the
 * ghosts outside the domain keep what the last applyBC (or setVal) left in
 * them; otherwise the coarse data is copied into zeroed FABs over the
 * coarsened fine boxes (ParallelCopy). */
static void interp_assign(Solver* S, int lev) {
    Hier* H = &S->H;
    const Level* Lf = &H->lev[lev];
    const Level* Lc = &H->lev[lev + 1];
    MF* crse = &S->cor[lev + 1];
    MF* fine = &S->cor[lev];
    MF tmp;
    const MF* cm = crse;
    int own = 0;
    /* isMFIterSafe(crse, fine): both levels' BoxArrays come from the level-0
     * BoxArray by BoxArray::coarsen (lazy, shared data), MLLinOpT::defineGrids
     * (AMReX_MLLinOp.H:995-1000, 1076-1077); agglomerated levels are new
     * BoxArrays (:1006) */
    if (Lf->derived && Lc->derived) {
        fill_boundary(Lc, H->periodic, crse, 0);
    } else {
        Box* cb = (Box*)malloc(sizeof(Box) * (size_t)Lf->nbox);
        for (int b = 0; b < Lf->nbox; ++b) cb[b] = bcoarsen(Lf->boxes[b], 2);
        mf_define(&tmp, Lf->nbox, cb, 1, -1);
        mf_setval(&tmp, 0.0);
        for (int b = 0; b < Lf->nbox; ++b) {
            Fab* t = &tmp.fab[b];
            for (int k = cb[b].lo[2] - 1; k <= cb[b].hi[2] + 1; ++k)
            for (int j = cb[b].lo[1] - 1; j <= cb[b].hi[1] + 1; ++j)
            for (int i = cb[b].lo[0] - 1; i <= cb[b].hi[0] + 1; ++i) {
                int wi, wj, wk;
                int src = locate(Lc, H->periodic, i, j, k, &wi, &wj, &wk);
                if (src >= 0) A(t, i, j, k) = A(&crse->fab[src], wi, wj, wk);
            }
        }
        free(cb);
        cm = &tmp; own = 1;
    }
    for (int b = 0; b < fine->nbox; ++b) {
        Fab* ff = &fine->fab[b];
        const Fab* cc = &cm->fab[b];
        FOR_VALID(ff, i, j, k) {
            const int kc = k / 2, koff = 2 * (k - kc * 2) - 1;
            const int jc = j / 2, joff = 2 * (j - jc * 2) - 1;
            const int ic = i / 2, ioff = 2 * (i - ic * 2) - 1;
            A(ff, i, j, k) = 0.421875 * A(cc, ic, jc, kc)
                + 0.140625 * A(cc, ic + ioff, jc, kc)
                + 0.140625 * A(cc, ic, jc + joff, kc)
                + 0.140625 * A(cc, ic, jc, kc + koff)
                + 0.046875 * A(cc, ic, jc + joff, kc + koff)
                + 0.046875 * A(cc, ic + ioff, jc, kc + koff)
                + 0.046875 * A(cc, ic + ioff, jc + joff, kc)
                + 0.015625 * A(cc, ic + ioff, jc + joff, kc + koff);
        }
    }
    if (own) mf_free(&tmp);
}

/* MLMGT::mgFcycle, AMReX_MLMG.H:1420-1457 */
static void fcycle(Solver* S) {
    Hier* H = &S->H;
    int bottom = H->nlev - 1;
    for (int lev = 1; lev <= bottom; ++lev) {
        /* avgDownResMG, AMReX_MLLinOp.H:1563-1584 */
        restriction(H, &H->lev[lev - 1], &S->res[lev - 1], &H->lev[lev], &S->res[lev]);
    }
    bottom_solve(S);
    for (int lev = bottom - 1; lev >= 0; --lev) {
        Level* L = &H->lev[lev];
        interp_assign(S, lev);
        correction_residual(S, lev, &S->rescor[lev], &S->cor[lev], &S->res[lev]);
        mf_axpy(L, &S->res[lev], 0, &S->rescor[lev], 0);
        MF t = S->cor[lev]; S->cor[lev] = S->cor_hold[lev]; S->cor_hold[lev] = t;
        vcycle(S, lev);
        mf_axpy(L, &S->cor[lev], 1.0, &S->cor_hold[lev], 1);
    }
}

static void copy_global_to_mf(const Level* L, MF* m, const double* g, int ngrow_src, int nodal_dir) {
    int n[3] = {blen(&L->domain, 0), blen(&L->domain, 1), blen(&L->domain, 2)};
    int e[3] = {n[0] + 2 * ngrow_src, n[1] + 2 * ngrow_src, n[2] + 2 * ngrow_src};
    if (nodal_dir >= 0) e[nodal_dir] += 1;
    for (int b = 0; b < m->nbox; ++b) {
        Fab* f = &m->fab[b];
        int ng = f->ng < ngrow_src ? f->ng : ngrow_src;
        for (int k = f->bx.lo[2] - ng; k <= f->bx.hi[2] + ng; ++k)
        for (int j = f->bx.lo[1] - ng; j <= f->bx.hi[1] + ng; ++j)
        for (int i = f->bx.lo[0] - ng; i <= f->bx.hi[0] + ng; ++i)
            A(f, i, j, k) = g[((size_t)(k + ngrow_src) * e[1] + (j + ngrow_src)) * e[0] + (i + ngrow_src)];
    }
}

static void copy_mf_to_global(const Level* L, const MF* m, double* g) {
    int n[3] = {blen(&L->domain, 0), blen(&L->domain, 1), blen(&L->domain, 2)};
    for (int b = 0; b < m->nbox; ++b) {
        Box vb = L->boxes[b];
        for (int k = vb.lo[2]; k <= vb.hi[2]; ++k)
        for (int j = vb.lo[1]; j <= vb.hi[1]; ++j)
        for (int i = vb.lo[0]; i <= vb.hi[0]; ++i)
            g[((size_t)k * n[1] + j) * n[0] + i] = A(&m->fab[b], i, j, k);
    }
}

static int setup_ratio(Solver* S, const OracleProblem* P, const OracleOptions* o, int crse_ratio);
static int setup(Solver* S, const OracleProblem* P, const OracleOptions* o) { return setup_ratio(S, P, o, 1); }
static int setup_ratio(Solver* S, const OracleProblem* P, const OracleOptions* o, int crse_ratio) {
    memset(S, 0, sizeof(*S));
    S->o = *o;
    S->bottom_mode = o->bottom_solver;
    Hier* H = &S->H;
    H->crse_ratio = crse_ratio;
    for (int d = 0; d < 3; ++d) {
        H->n[d] = P->n[d]; H->periodic[d] = P->periodic[d];
        H->prob_lo[d] = P->prob_lo[d]; H->prob_hi[d] = P->prob_hi[d];
        H->lobc[d] = P->lobc[d]; H->hibc[d] = P->hibc[d];
        H->dx0[d] = (P->prob_hi[d] - P->prob_lo[d]) / (double)P->n[d];
    }
    H->maxorder = o->maxorder;
    H->is_abec = P->is_abec;
    H->alpha = P->is_abec ? P->alpha : 0.0;
    H->beta = P->is_abec ? P->beta : 1.0;
    Box* ba = NULL; int nba;
    if (P->nbox > 0) {
        nba = P->nbox; ba = (Box*)malloc(sizeof(Box) * nba);
        for (int b = 0; b < nba; ++b)
            for (int d = 0; d < 3; ++d) { ba[b].lo[d] = P->boxes[6 * b + d]; ba[b].hi[d] = P->boxes[6 * b + 3 + d]; }
    } else {
        Box dom = {{0, 0, 0}, {P->n[0] - 1, P->n[1] - 1, P->n[2] - 1}};
        nba = max_size(&dom, 1, P->max_grid_size, &ba);
    }
    define_grids(H, ba, nba, o);
    free(ba);
    for (int l = 0; l < H->nlev; ++l) {
        build_boxmap(&H->lev[l]);
        define_bc(H, &H->lev[l], o);
    }
    return 0;
}

static void free_solver(Solver* S) {
    for (int l = 0; l < S->H.nlev; ++l) {
        Level* L = &S->H.lev[l];
        for (int q = 0; q < 6 * L->nbox; ++q) { free(L->mask[q].p); free(L->fco[q].p); }
        free(L->mask); free(L->fco); free(L->bct_p); free(L->bcl_p); free(L->boxmap); free(L->boxes);
        if (L->acoef.fab) mf_free(&L->acoef);
        for (int d = 0; d < 3; ++d) if (L->bcoef[d].fab) mf_free(&L->bcoef[d]);
        if (S->cor[l].fab) mf_free(&S->cor[l]);
        if (S->res[l].fab) mf_free(&S->res[l]);
        if (S->rescor[l].fab) mf_free(&S->rescor[l]);
        if (S->cor_hold[l].fab) mf_free(&S->cor_hold[l]);
    }
    if (S->sol.fab) mf_free(&S->sol);
    if (S->rhs.fab) mf_free(&S->rhs);
}

static void load_coeffs(Solver* S, const OracleProblem* P) {
    Hier* H = &S->H;
    Level* L0 = &H->lev[0];
    if (!H->is_abec) return;
    mf_define(&L0->acoef, L0->nbox, L0->boxes, 0, -1);
    for (int d = 0; d < 3; ++d) mf_define(&L0->bcoef[d], L0->nbox, L0->boxes, 0, d);
    if (P->a) copy_global_to_mf(L0, &L0->acoef, P->a, 0, -1); else mf_setval(&L0->acoef, 1.0);
    const double* bp[3] = {P->bx, P->by, P->bz};
    for (int d = 0; d < 3; ++d) {
        if (bp[d]) copy_global_to_mf(L0, &L0->bcoef[d], bp[d], 0, d); else mf_setval(&L0->bcoef[d], 1.0);
    }
    if (H->alpha == 0.0) mf_setval(&L0->acoef, 0.0);
}

/* averageDownCoeffsSameAmrLevel, AMReX_MLABecLaplacian.H:628-690 */
static void restrict_all_coeffs(Solver* S) {
    Hier* H = &S->H;
    if (!H->is_abec) return;
    for (int l = 1; l < H->nlev; ++l) restrict_coeffs(H, &H->lev[l - 1], &H->lev[l]);
}

static void set_coeffs(Solver* S, const OracleProblem* P) {
    load_coeffs(S, P);
    restrict_all_coeffs(S);
}

static int is_singular(const Solver* S) {
    /* update_singular_flags, AMReX_MLABecLaplacian.H:714-741 ;
     * MLPoissonT::prepareForSolve, AMReX_MLPoisson.H:138-178 */
    const Hier* H = &S->H;
    for (int d = 0; d < 3; ++d) if (H->lobc[d] == LO_DIRICHLET || H->hibc[d] == LO_DIRICHLET) return 0;
    const Level* L0 = &H->lev[0];
    long long np = 0;
    for (int b = 0; b < L0->nbox; ++b) np += bnpts(&L0->boxes[b]);
    if (np != bnpts(&L0->domain)) return 0;
    if (!H->is_abec || H->alpha == 0.0) return 1;
    const Level* Lb = &H->lev[H->nlev - 1];
    double asum = mf_sum(Lb, &Lb->acoef), amax = mf_norminf(Lb, &Lb->acoef);
    return fabs(asum) <= amax * 1.e-12;
}

/* ------------------------------------------------------ public API ------- */
int oracle_max_size(const int* dom_lo, const int* dom_hi, int chunk, int* out, int max_out) {
    Box d; Box* res = NULL;
    for (int q = 0; q < 3; ++q) { d.lo[q] = dom_lo[q]; d.hi[q] = dom_hi[q]; }
    int n = max_size(&d, 1, chunk, &res);
    for (int b = 0; b < n && b < max_out; ++b)
        for (int q = 0; q < 3; ++q) { out[6 * b + q] = res[b].lo[q]; out[6 * b + 3 + q] = res[b].hi[q]; }
    free(res);
    return n;
}

int oracle_hierarchy(const OracleProblem* P, const OracleOptions* o, int* nbox_per_level, int* boxes_out,
                     int max_boxes) {
    Solver* S = (Solver*)calloc(1, sizeof(Solver));
    setup(S, P, o);
    int q = 0;
    for (int l = 0; l < S->H.nlev; ++l) {
        nbox_per_level[l] = S->H.lev[l].nbox;
        for (int b = 0; b < S->H.lev[l].nbox; ++b, ++q) {
            if (q >= max_boxes) continue;
            for (int d = 0; d < 3; ++d) {
                boxes_out[6 * q + d] = S->H.lev[l].boxes[b].lo[d];
                boxes_out[6 * q + 3 + d] = S->H.lev[l].boxes[b].hi[d];
            }
        }
    }
    int nlev = S->H.nlev;
    free_solver(S);
    free(S);
    return nlev;
}

int oracle_fill_boundary(const OracleProblem* P, int cross, double* data) {
    OracleOptions o; oracle_default_options(&o); o.max_coarsening_level = 0;
    Solver* S = (Solver*)calloc(1, sizeof(Solver));
    setup(S, P, &o);
    Level* L = &S->H.lev[0];
    MF m; mf_define(&m, L->nbox, L->boxes, 1, -1);
    size_t off = 0;
    for (int b = 0; b < m.nbox; ++b) { memcpy(m.fab[b].p, data + off, sizeof(double) * fab_size(&m.fab[b])); off += fab_size(&m.fab[b]); }
    fill_boundary(L, S->H.periodic, &m, cross);
    off = 0;
    for (int b = 0; b < m.nbox; ++b) { memcpy(data + off, m.fab[b].p, sizeof(double) * fab_size(&m.fab[b])); off += fab_size(&m.fab[b]); }
    mf_free(&m);
    free_solver(S);
    free(S);
    return 0;
}

int oracle_apply(const OracleProblem* P, const OracleOptions* o, double* out) {
    Solver* S = (Solver*)calloc(1, sizeof(Solver));
    OracleOptions oo = *o; oo.max_coarsening_level = 0;
    setup(S, P, &oo);
    set_coeffs(S, P);
    Level* L = &S->H.lev[0];
    S->bcval.v = P->sol; for (int d = 0; d < 3; ++d) S->bcval.n[d] = P->n[d];
    MF x, y, z;
    mf_define(&x, L->nbox, L->boxes, 1, -1);
    mf_define(&y, L->nbox, L->boxes, 0, -1);
    mf_define(&z, L->nbox, L->boxes, 0, -1);
    copy_global_to_mf(L, &x, P->sol, 1, -1);
    mf_setval(&z, 0.0);
    solution_residual(S, &y, &x, &z);
    /* MLMGT::apply scales the residual of a zero rhs by -1, AMReX_MLMG.H:858-932 */
    for (int b = 0; b < y.nbox; ++b) FOR_VALID(&y.fab[b], i, j, k) A(&y.fab[b], i, j, k) *= -1.0;
    copy_mf_to_global(L, &y, out);
    mf_free(&x); mf_free(&y); mf_free(&z);
    free_solver(S);
    free(S);
    return 0;
}

/* MLMGT::getGradSolution -> MLCellLinOpT::compGrad (AMReX_MLCellLinOp.H:1392-1442)
 * for mode 0; MLMGT::getFluxes -> MLCellABecLapT::getFluxes
 * (AMReX_MLCellABecLap.H:272-291) -> compFlux (AMReX_MLCellLinOp.H:1348-1390)
 * -> FFlux (mlabeclap_flux_x, AMReX_MLABecLap_3D_K.H:79-97; mlpoisson_flux_x,
 * AMReX_MLPoisson_3D_K.H:36-50) then the 1/beta scaling for mode 1.  The
 * solution's ghosts come from applyBC with the level's Dirichlet values.
 * Outputs are global face arrays (n_d + 1 along d), written box by box over
 * each box's surrounding nodes. */
int oracle_fluxes(const OracleProblem* P, const OracleOptions* o, int mode, double* fx, double* fy, double* fz) {
    Solver* S = (Solver*)calloc(1, sizeof(Solver));
    OracleOptions oo = *o; oo.max_coarsening_level = 0;
    setup(S, P, &oo);
    set_coeffs(S, P);
    Hier* H = &S->H;
    Level* L = &H->lev[0];
    S->bcval.v = P->sol; for (int d = 0; d < 3; ++d) S->bcval.n[d] = P->n[d];
    MF x;
    mf_define(&x, L->nbox, L->boxes, 1, -1);
    copy_global_to_mf(L, &x, P->sol, 1, -1);
    apply_bc(H, L, &x, 1, &S->bcval, 0, NULL);
    double* out[3] = {fx, fy, fz};
    const double bscalar = H->is_abec ? H->beta : -1.0;   /* MLPoissonT::getBScalar is -1 */
    const double betainv = 1.0 / bscalar;
    for (int b = 0; b < L->nbox; ++b) {
        const Box* vb = &L->boxes[b];
        const Fab* s = &x.fab[b];
        for (int d = 0; d < 3; ++d) {
            int e[3] = {P->n[0], P->n[1], P->n[2]};
            e[d] += 1;
            const int di = (d == 0), dj = (d == 1), dk = (d == 2);
            const double dxi = L->dxinv[d];
            for (int k = vb->lo[2]; k <= vb->hi[2] + dk; ++k)
            for (int j = vb->lo[1]; j <= vb->hi[1] + dj; ++j)
            for (int i = vb->lo[0]; i <= vb->hi[0] + di; ++i) {
                const double ds = A(s, i, j, k) - A(s, i - di, j - dj, k - dk);
                double v;
                if (mode == 0) {
                    v = dxi * ds;
                } else if (H->is_abec) {
                    const double fac = H->beta * dxi;
                    v = -fac * A(&L->bcoef[d].fab[b], i, j, k) * ds;
                    if (betainv != 1.0) v *= betainv;
                } else {
                    v = dxi * ds;
                    v *= betainv;
                }
                out[d][((size_t)k * e[1] + j) * e[0] + i] = v;
            }
        }
    }
    mf_free(&x);
    free_solver(S);
    free(S);
    return 0;
}

void oracle_default_options(OracleOptions* o) {
    memset(o, 0, sizeof(*o));
    o->agg = 1; o->con = 1; o->agg_grid_size = 32; o->con_grid_size = 32; o->max_coarsening_level = 30;
    o->maxorder = 3; o->nu1 = 2; o->nu2 = 2; o->nuf = 8; o->nub = 0;
    o->max_iter = 200; o->fixed_iter = 0; o->bottom_solver = 2; o->bottom_maxiter = 200;
    o->bottom_reltol = 1.e-4; o->tol_rel = 1.e-10; o->tol_abs = 0.0;
    o->max_fmg_iter = 0;
}

/* MLMGT::solve, AMReX_MLMG.H:353-541, single AMR level */
int oracle_solve(const OracleProblem* P, const OracleOptions* o, double* phi_out, OracleResult* R) {
    Solver* S = (Solver*)calloc(1, sizeof(Solver));
    setup(S, P, o);
    set_coeffs(S, P);
    Hier* H = &S->H;
    Level* L0 = &H->lev[0];
    S->bcval.v = P->sol; for (int d = 0; d < 3; ++d) S->bcval.n[d] = P->n[d];
    mf_define(&S->sol, L0->nbox, L0->boxes, 1, -1);
    copy_global_to_mf(L0, &S->sol, P->sol, 1, -1);
    mf_define(&S->rhs, L0->nbox, L0->boxes, 0, -1);
    copy_global_to_mf(L0, &S->rhs, P->rhs, 0, -1);
    S->singular = is_singular(S);
    {
        long long np = bnpts(&L0->domain);
        S->volinv0 = 1.0 / (double)np;
        S->volinv_bottom = 1.0 / (double)bnpts(&H->lev[H->nlev - 1].domain);
    }
    for (int l = 0; l < H->nlev; ++l) {
        Level* L = &H->lev[l];
        mf_define(&S->cor[l], L->nbox, L->boxes, 1, -1);
        mf_define(&S->res[l], L->nbox, L->boxes, 0, -1);
        mf_define(&S->rescor[l], L->nbox, L->boxes, 0, -1);
        mf_define(&S->cor_hold[l], L->nbox, L->boxes, 1, -1);
        mf_setval(&S->cor_hold[l], 0.0);
    }
    if (S->singular) make_solvable(S, 0, &S->rhs);
    solution_residual(S, &S->res[0], &S->sol, &S->rhs);
    double resnorm0 = mf_norminf(L0, &S->res[0]);
    double rhsnorm0 = mf_norminf(L0, &S->rhs);
    double max_norm = (rhsnorm0 >= resnorm0) ? rhsnorm0 : resnorm0;
    double tr = o->tol_rel > 1.e-16 ? o->tol_rel : 1.e-16;
    double res_target = o->tol_abs > tr * max_norm ? o->tol_abs : tr * max_norm;
    R->init_resid = resnorm0; R->rhs_norm = rhsnorm0; R->niters = 0; R->status = 0;
    double composite = resnorm0;
    struct timespec t0, t1;
    clock_gettime(CLOCK_MONOTONIC, &t0);
    if (resnorm0 > res_target) {
        int converged = 0;
        int niters = o->fixed_iter ? o->fixed_iter : o->max_iter;
        for (int iter = 0; iter < niters; ++iter) {
            if (S->singular) make_solvable(S, 0, &S->res[0]);
            if (iter < o->max_fmg_iter) { fcycle(S); } else { vcycle(S, 0); }
            mf_axpy(L0, &S->sol, 1.0, &S->cor[0], 1);
            solution_residual(S, &S->res[0], &S->sol, &S->rhs);
            double fine = mf_norminf(L0, &S->res[0]);
            if (R->niters < ORACLE_MAX_HIST) { R->history[R->niters] = fine; }
            R->niters++;
            composite = fine;
            if (fine <= res_target) { converged = 1; break; }
            if (composite > 1.e20 * max_norm) { R->status = -2; break; }
        }
        if (!converged && o->fixed_iter == 0 && R->status == 0) R->status = 1;
    }
    clock_gettime(CLOCK_MONOTONIC, &t1);
    R->iter_seconds = (double)(t1.tv_sec - t0.tv_sec) + 1e-9 * (double)(t1.tv_nsec - t0.tv_nsec);
    R->final_resid = composite;
    R->nlev = H->nlev;
    R->ncg = S->ncg;
    for (int q = 0; q < S->ncg && q < ORACLE_MAX_HIST; ++q) R->cg_iters[q] = S->cg_log[q];
    copy_mf_to_global(L0, &S->sol, phi_out);
    free_solver(S);
    free(S);
    return R->status;
}


/* ======================================================================
 * AMR composite solve: MLMGT::solve over several AMR levels
 * (AMReX_MLMG.H:353-541, oneIter :1227-1293), MLPoisson or MLABecLaplacian,
 * refinement ratio 2, periodic or not.  AMR level 0 keeps its full MG hierarchy; each finer
 * AMR level has one MG level (MLLinOpT::defineGrids, AMReX_MLLinOp.H:843-880),
 * so its mini-cycle is nu1 smoothing sweeps from zero (mgVcycle,
 * AMReX_MLMG.H:1306-1415, amrlev > 0 branch).
 * ====================================================================== */
#define AMR_MAX 4

typedef struct {
    int nlev;
    Solver S[AMR_MAX];      /* S[l].sol/rhs/res[0]/rescor[0]/cor[0]/cor_hold[0] are the AMR level's data */
    Fab* bsol[AMR_MAX];     /* [6*nbox] boundary values of the solution (m_bndry_sol) */
    Fab* bcor[AMR_MAX];     /* [6*nbox] boundary values of the correction (m_bndry_cor) */
} Amr;

/* mask value (MultiMask, Src/Boundary/AMReX_MultiMask.cpp:25-69) of cell
 * (i,j,k) at a level: outside the domain, covered by a box of the level
 * (periodic images included) or not covered */
static int level_mask(const Hier* H, const Level* L, int i, int j, int k) {
    int c[3] = {i, j, k};
    for (int q = 0; q < 3; ++q)
        if (!H->periodic[q] && (c[q] < L->domain.lo[q] || c[q] > L->domain.hi[q])) return MASK_OUTSIDE;
    int wi, wj, wk;
    return (locate(L, H->periodic, i, j, k, &wi, &wj, &wk) >= 0) ? MASK_COVERED : MASK_NOT_COVERED;
}

/* value of a valid cell of MF m on level L (periodic images included), or 0
 * where no box holds it (ParallelCopy of valid cells into zeroed data) */
static double cell_value(const Hier* H, const Level* L, const MF* m, int i, int j, int k) {
    int wi, wj, wk;
    int b = locate(L, H->periodic, i, j, k, &wi, &wj, &wk);
    return (b >= 0) ? A(&m->fab[b], wi, wj, wk) : 0.0;
}

static int cdiv2(int a) { return (a >= 0) ? a / 2 : -((-a + 1) / 2); }

/* coarse cell (i,j,k) of AMR level l lies under a box of level l+1 (boxes of
 * a finer level are aligned to the refinement ratio) */
static int covered_by_fine(const Amr* M, int l, int i, int j, int k) {
    if (l + 1 >= M->nlev) return 0;
    const Hier* Hf = &M->S[l + 1].H;
    int wi, wj, wk;
    return locate(&Hf->lev[0], Hf->periodic, 2 * i, 2 * j, 2 * k, &wi, &wj, &wk) >= 0;
}

/* InterpBndryDataT::setBndryValues / updateBndryValues (Src/Boundary/
 * AMReX_InterpBndryData.H:158-267) with interpbndrydata_{x,y,z}_o3
 * (Src/Boundary/AMReX_InterpBndryData_3D_K.H:20-120), ratio 2: boundary
 * values of AMR level l on every box face.  A face off the non-periodic
 * domain boundary gets the coarse value (crse on level l-1, valid cells) at
 * the ghost cell's coarse cell plus tangential slopes and curvatures, one-sided
 * where a neighbouring fine ghost cell is not "not covered"; a face on it
 * keeps the level's BC values (phys != 0: the solution) or zero (the
 * correction, whose register is zeroed before the solve). */
static void interp_bndry(Amr* M, int l, const MF* crse, int phys, Fab* dst) {
    Solver* Sf = &M->S[l];
    const Hier* Hf = &Sf->H;
    const Level* Lf = &Hf->lev[0];
    const Hier* Hc = &M->S[l - 1].H;
    const Level* Lc = &Hc->lev[0];
    const int r = 2;
    for (int b = 0; b < Lf->nbox; ++b) {
        const Box* bx = &Lf->boxes[b];
        for (int f = 0; f < 6; ++f) {
            const int d = f % 3, hi = f >= 3;
            Fab* out = &dst[6 * b + f];
            if (out->p == NULL) fab_define(out, adj_cell(bx, f), 0);
            const int on_domain = hi ? (Lf->domain.hi[d] == bx->hi[d]) : (Lf->domain.lo[d] == bx->lo[d]);
            if (on_domain && !Hf->periodic[d]) {
                FOR_VALID(out, i, j, k) {
                    A(out, i, j, k) = (phys && Sf->bcval.v) ? gg_at(&Sf->bcval, i, j, k) : 0.0;
                }
                continue;
            }
            const int t1 = (d == 0) ? 1 : 0, t2 = (d == 2) ? 1 : 2;   /* tangential directions */
            FOR_VALID(out, i, j, k) {
                const int c[3] = {i, j, k};
                const int cc[3] = {cdiv2(i), cdiv2(j), cdiv2(k)};
#define CRS(v) cell_value(Hc, Lc, crse, (v)[0], (v)[1], (v)[2])
#define NOTCOV(v) (level_mask(Hf, Lf, (v)[0], (v)[1], (v)[2]) == MASK_NOT_COVERED)
                double slope[2], curv[2];
                const int tdir[2] = {t1, t2};
                for (int q = 0; q < 2; ++q) {
                    const int t = tdir[q];
                    int fm[3] = {c[0], c[1], c[2]}, fp[3] = {c[0], c[1], c[2]};
                    fm[t] -= r; fp[t] += r;
                    const int lo = NOTCOV(fm) ? cc[t] - 1 : cc[t];
                    const int hi2 = NOTCOV(fp) ? cc[t] + 1 : cc[t];
                    const double fac = (hi2 == lo + 1) ? 1.0 : 0.5;
                    int ch[3] = {cc[0], cc[1], cc[2]}, cl[3] = {cc[0], cc[1], cc[2]};
                    ch[t] = hi2; cl[t] = lo;
                    slope[q] = fac * (CRS(ch) - CRS(cl));
                    if (hi2 == lo + 2) {
                        int cp[3] = {cc[0], cc[1], cc[2]}, cm[3] = {cc[0], cc[1], cc[2]};
                        cp[t] += 1; cm[t] -= 1;
                        curv[q] = 0.5 * (CRS(cp) - 2.0 * CRS(cc) + CRS(cm));
                    } else {
                        curv[q] = 0.0;
                    }
                }
                /* cross term when the four diagonal fine ghost cells are not covered */
                int ok = 1;
                for (int s1 = -1; s1 <= 1; s1 += 2)
                    for (int s2 = -1; s2 <= 1; s2 += 2) {
                        int a[3] = {c[0], c[1], c[2]};
                        a[t1] += s1 * r; a[t2] += s2 * r;
                        if (!NOTCOV(a)) ok = 0;
                    }
                double cross = 0.0;
                if (ok) {
                    int pp[3] = {cc[0], cc[1], cc[2]}, mp[3] = {cc[0], cc[1], cc[2]};
                    int mm[3] = {cc[0], cc[1], cc[2]}, pm[3] = {cc[0], cc[1], cc[2]};
                    pp[t1] += 1; pp[t2] += 1;
                    mp[t1] -= 1; mp[t2] += 1;
                    mm[t1] -= 1; mm[t2] -= 1;
                    pm[t1] += 1; pm[t2] -= 1;
                    cross = 0.25 * (CRS(pp) - CRS(mp) + CRS(mm) - CRS(pm));
                }
                const double y = -0.5 + ((double)(c[t1] - cc[t1] * r) + 0.5) / (double)r;
                const double z = -0.5 + ((double)(c[t2] - cc[t2] * r) + 0.5) / (double)r;
                A(out, i, j, k) = CRS(cc) + y * slope[0] + (y * y) * curv[0]
                                  + z * slope[1] + (z * z) * curv[1] + y * z * cross;
#undef CRS
#undef NOTCOV
            }
        }
    }
}

/* MLCellLinOpT::solutionResidual (AMReX_MLCellLinOp.H:1219-1236): at a fine
 * AMR level the boundary values come from the coarser level's solution
 * (updateSolBC, :651-664) when update != 0 */
static void amr_solution_residual(Amr* M, int l, MF* r, MF* x, const MF* b, int update) {
    Solver* S = &M->S[l];
    if (l == 0) { solution_residual(S, r, x, b); return; }
    if (update) interp_bndry(M, l, &M->S[l - 1].sol, 1, M->bsol[l]);
    apply_bc(&S->H, &S->H.lev[0], x, 1, NULL, 0, M->bsol[l]);
    fapply(&S->H, &S->H.lev[0], r, x);
    mf_axpy(&S->H.lev[0], r, -1.0, b, 3);
}

/* MLCellLinOpT::correctionResidual, inhomogeneous with the coarser level's
 * correction as boundary data (updateCorBC, AMReX_MLCellLinOp.H:666-680,
 * 1246-1270) */
static void amr_correction_residual_inhomog(Amr* M, int l, MF* r, MF* x, const MF* b) {
    Solver* S = &M->S[l];
    interp_bndry(M, l, &M->S[l - 1].cor[0], 0, M->bcor[l]);
    apply_bc(&S->H, &S->H.lev[0], x, 1, NULL, 0, M->bcor[l]);
    fapply(&S->H, &S->H.lev[0], r, x);
    mf_axpy(&S->H.lev[0], r, -1.0, b, 3);
}

/* amrex::average_down of the valid fine cells onto the covered coarse cells
 * (amrex_avgdown, Src/Base/AMReX_MultiFabUtil_3D_C.H:375-392) */
static void amr_average_down(Amr* M, int c, const MF* fine, MF* crse) {
    const Hier* Hc = &M->S[c].H;
    const Level* Lc = &Hc->lev[0];
    const Level* Lf = &M->S[c + 1].H.lev[0];
    for (int b = 0; b < crse->nbox; ++b) {
        Fab* cf = &crse->fab[b];
        Box vb = Lc->boxes[b];
        for (int k = vb.lo[2]; k <= vb.hi[2]; ++k)
        for (int j = vb.lo[1]; j <= vb.hi[1]; ++j)
        for (int i = vb.lo[0]; i <= vb.hi[0]; ++i) {
            if (!covered_by_fine(M, c, i, j, k)) continue;
            double s = 0;
            for (int kr = 0; kr < 2; ++kr)
            for (int jr = 0; jr < 2; ++jr)
            for (int ir = 0; ir < 2; ++ir) {
                int wi, wj, wk;
                int fb = locate(Lf, Hc->periodic, 2 * i + ir, 2 * j + jr, 2 * k + kr, &wi, &wj, &wk);
                s += A(&fine->fab[fb], wi, wj, wk);
            }
            A(cf, i, j, k) = 0.125 * s;
        }
    }
}

/* averageDownCoeffsToCoarseAmrLevel (AMReX_MLABecLaplacian.H:693-712):
 * a (unless alpha is 0) by amr_average_down, and b by average_down_faces
 * with the crse geometry (Src/Base/AMReX_MultiFabUtil.H:958-968): every coarse
 * face of a coarsened fine box, its boundary faces included, takes the mean of
 * the rr^2 fine faces on it (amrex_avgdown_faces,
 * Src/Base/AMReX_MultiFabUtil_3D_C.H:170-225, same summation order). */
static void amr_average_down_coeffs(Amr* M, int c) {
    Hier* Hc = &M->S[c].H;
    Level* Lc = &Hc->lev[0];
    const Level* Lf = &M->S[c + 1].H.lev[0];
    if (Hc->alpha != 0.0) amr_average_down(M, c, &Lf->acoef, &Lc->acoef);
    for (int d = 0; d < 3; ++d) {
        for (int b = 0; b < Lc->nbox; ++b) {
            Fab* cf = &Lc->bcoef[d].fab[b];
            FOR_VALID(cf, i, j, k) {
                int lo[3] = {i, j, k};
                lo[d] -= 1;
                if (!covered_by_fine(M, c, i, j, k) && !covered_by_fine(M, c, lo[0], lo[1], lo[2])) continue;
                double s = 0;
                for (int r1 = 0; r1 < 2; ++r1)
                for (int r0 = 0; r0 < 2; ++r0) {
                    int f[3] = {2 * i, 2 * j, 2 * k};
                    if (d == 0) { f[1] += r0; f[2] += r1; }
                    else if (d == 1) { f[0] += r0; f[2] += r1; }
                    else { f[0] += r0; f[1] += r1; }
                    /* a fine box holding the cell on either side of the face
                     * holds the face: its image's index when the cell lies
                     * past a periodic face (the box stores the face at the
                     * wrapped cell, or one above the wrapped low-side cell) */
                    int w[3];
                    int fb = locate(Lf, Hc->periodic, f[0], f[1], f[2], &w[0], &w[1], &w[2]);
                    if (fb < 0) {
                        int g[3] = {f[0], f[1], f[2]};
                        g[d] -= 1;
                        fb = locate(Lf, Hc->periodic, g[0], g[1], g[2], &w[0], &w[1], &w[2]);
                        w[d] += 1;
                    }
                    s += A(&Lf->bcoef[d].fab[fb], w[0], w[1], w[2]);
                }
                A(cf, i, j, k) = s * (1.0 / 4.0);
            }
        }
    }
}

/* MLCellLinOpT::reflux (AMReX_MLCellLinOp.H:1272-1346) through YAFluxRegister
 * (Src/Boundary/AMReX_YAFluxRegister.H:125-335, 343-560; yafluxreg_crseadd /
 * yafluxreg_fineadd, AMReX_YAFluxRegister_3D_K.H): every coarse cell of level
 * c next to level c+1 trades its coarse face flux for the mean of the fine
 * face fluxes, res += (F_crse - <F_fine>) / dx_crse with MLPoisson's flux
 * F = (phi_hi - phi_lo) / dx.  The fine solution's ghosts come from applyBC
 * with the level's solution boundary values. */
static void amr_reflux(Amr* M, int c, MF* res) {
    Solver* Sc = &M->S[c];
    Solver* Sf = &M->S[c + 1];
    const Hier* Hc = &Sc->H;
    const Level* Lc = &Hc->lev[0];
    const Hier* Hf = &Sf->H;
    const Level* Lf = &Hf->lev[0];
    apply_bc(Hf, Lf, &Sf->sol, 1, NULL, 0, M->bsol[c + 1]);
    MF data;
    mf_define(&data, Lc->nbox, Lc->boxes, 0, -1);
    mf_setval(&data, 0.0);
    /* coarse side (CrseAdd, dt = 1) */
    for (int b = 0; b < Lc->nbox; ++b) {
        Fab* d = &data.fab[b];
        Box vb = Lc->boxes[b];
        for (int k = vb.lo[2]; k <= vb.hi[2]; ++k)
        for (int j = vb.lo[1]; j <= vb.hi[1]; ++j)
        for (int i = vb.lo[0]; i <= vb.hi[0]; ++i) {
            if (covered_by_fine(M, c, i, j, k)) continue;
            const int c0[3] = {i, j, k};
            for (int q = 0; q < 3; ++q) {
                const double dtdx = 1.0 / Lc->dx[q];
                for (int side = 0; side < 2; ++side) {
                    int n[3] = {c0[0], c0[1], c0[2]};
                    n[q] += side ? 1 : -1;
                    if (!covered_by_fine(M, c, n[0], n[1], n[2])) continue;
                    const double vc = cell_value(Hc, Lc, &Sc->sol, i, j, k);
                    const double vn = cell_value(Hc, Lc, &Sc->sol, n[0], n[1], n[2]);
                    /* face flux on the face between the cell and its neighbour:
                     * MLPoisson's dxinv (phi_i - phi_i-1) (mlpoisson_flux_x,
                     * AMReX_MLPoisson_3D_K.H:36-50), MLABecLaplacian's
                     * -beta dxinv b (phi_i - phi_i-1) (mlabeclap_flux_x,
                     * AMReX_MLABecLap_3D_K.H:79-95) */
                    double fx;
                    if (Hc->is_abec) {
                        int fc[3] = {i, j, k};
                        if (side) fc[q] += 1;
                        const double fac = Hc->beta * Lc->dxinv[q];
                        const double bf = A(&Lc->bcoef[q].fab[b], fc[0], fc[1], fc[2]);
                        fx = side ? -fac * bf * (vn - vc) : -fac * bf * (vc - vn);
                    } else {
                        fx = side ? Lc->dxinv[q] * (vn - vc) : Lc->dxinv[q] * (vc - vn);
                    }
                    if (side) A(d, i, j, k) += dtdx * fx; else A(d, i, j, k) -= dtdx * fx;
                }
            }
        }
    }
    /* fine side (FineAdd, one coarse/fine patch per fine box, then added) */
    for (int fb = 0; fb < Lf->nbox; ++fb) {
        const Box cb = bcoarsen(Lf->boxes[fb], 2);
        Box gb = cb;
        for (int q = 0; q < 3; ++q) { gb.lo[q] -= 1; gb.hi[q] += 1; }
        Fab patch;
        fab_define(&patch, gb, 0);
        memset(patch.p, 0, sizeof(double) * fab_size(&patch));
        const Fab* fs = &Sf->sol.fab[fb];
        for (int q = 0; q < 3; ++q) {
            const double dtdx = 1.0 / (Lf->dx[q] * 8.0);
            for (int side = 0; side < 2; ++side) {
                Box ab = adj_cell(&cb, q + 3 * side);
                for (int k = ab.lo[2]; k <= ab.hi[2]; ++k)
                for (int j = ab.lo[1]; j <= ab.hi[1]; ++j)
                for (int i = ab.lo[0]; i <= ab.hi[0]; ++i) {
                    const int cc3[3] = {i, j, k};
                    int indom = 1;   /* periodic directions wrap (covered_by_fine does) */
                    for (int e = 0; e < 3; ++e)
                        if (!Hc->periodic[e] && (cc3[e] < Lc->domain.lo[e] || cc3[e] > Lc->domain.hi[e])) indom = 0;
                    if (!indom || covered_by_fine(M, c, i, j, k)) continue;
                    /* the rr^2 fine faces on the coarse cell's face shared with the fine box */
                    const int t1 = (q == 0) ? 1 : 0, t2 = (q == 2) ? 1 : 2;
                    const int face = side ? 2 * cc3[q] : 2 * (cc3[q] + 1);
                    for (int o2 = 0; o2 < 2; ++o2)
                    for (int o1 = 0; o1 < 2; ++o1) {
                        int fi[3];
                        fi[q] = face;
                        fi[t1] = 2 * cc3[t1] + o1;
                        fi[t2] = 2 * cc3[t2] + o2;
                        int lo3[3] = {fi[0], fi[1], fi[2]};
                        lo3[q] -= 1;
                        double ff;
                        if (Hf->is_abec) {
                            const double fac = Hf->beta * Lf->dxinv[q];
                            const double bf = A(&Lf->bcoef[q].fab[fb], fi[0], fi[1], fi[2]);
                            ff = -fac * bf * (A(fs, fi[0], fi[1], fi[2]) - A(fs, lo3[0], lo3[1], lo3[2]));
                        } else {
                            ff = Lf->dxinv[q] * (A(fs, fi[0], fi[1], fi[2]) - A(fs, lo3[0], lo3[1], lo3[2]));
                        }
                        const double tmp = side ? dtdx * ff : -dtdx * ff;
                        A(&patch, i, j, k) += tmp;
                    }
                }
            }
        }
        /* add the patch into the register over the uncovered cells of grow(cb,1),
         * through the periodic images (the register's ParallelAdd with the
         * coarse geometry's periodicity) */
        FOR_VALID(&patch, i, j, k) {
            const int cc3[3] = {i, j, k};
            int indom = 1;
            for (int e = 0; e < 3; ++e)
                if (!Hc->periodic[e] && (cc3[e] < Lc->domain.lo[e] || cc3[e] > Lc->domain.hi[e])) indom = 0;
            if (!indom || covered_by_fine(M, c, i, j, k)) continue;
            int wi, wj, wk;
            int db = locate(Lc, Hc->periodic, i, j, k, &wi, &wj, &wk);
            if (db >= 0) A(&data.fab[db], wi, wj, wk) += A(&patch, i, j, k);
        }
        free(patch.p);
    }
    mf_axpy(Lc, res, 1.0, &data, 1);
    mf_free(&data);
}

/* MLMGT::interpCorrection(alev) (AMReX_MLMG.H:1719-1750) with
 * MLCellLinOpT::interpolationAmr (AMReX_MLCellLinOp.H:1094-1181) and
 * mlmg_lin_cc_interp_r2: the coarser level's correction is copied (valid
 * cells) into zeroed FABs over the coarsened fine boxes grown by one, then
 * interpolated trilinearly onto the fine level's valid cells. */
static void amr_interp_correction(Amr* M, int l) {
    const Hier* Hc = &M->S[l - 1].H;
    const Level* Lc = &Hc->lev[0];
    const Level* Lf = &M->S[l].H.lev[0];
    const MF* crse = &M->S[l - 1].cor[0];
    MF* fine = &M->S[l].cor[0];
    for (int b = 0; b < Lf->nbox; ++b) {
        Box cb = bcoarsen(Lf->boxes[b], 2);
        Fab t;
        fab_define(&t, cb, 1);
        for (int k = cb.lo[2] - 1; k <= cb.hi[2] + 1; ++k)
        for (int j = cb.lo[1] - 1; j <= cb.hi[1] + 1; ++j)
        for (int i = cb.lo[0] - 1; i <= cb.hi[0] + 1; ++i)
            A(&t, i, j, k) = cell_value(Hc, Lc, crse, i, j, k);
        Fab* ff = &fine->fab[b];
        FOR_VALID(ff, i, j, k) {
            const int kc = k / 2, koff = 2 * (k - kc * 2) - 1;
            const int jc = j / 2, joff = 2 * (j - jc * 2) - 1;
            const int ic = i / 2, ioff = 2 * (i - ic * 2) - 1;
            A(ff, i, j, k) = 0.421875 * A(&t, ic, jc, kc)
                + 0.140625 * A(&t, ic + ioff, jc, kc)
                + 0.140625 * A(&t, ic, jc + joff, kc)
                + 0.140625 * A(&t, ic, jc, kc + koff)
                + 0.046875 * A(&t, ic, jc + joff, kc + koff)
                + 0.046875 * A(&t, ic + ioff, jc, kc + koff)
                + 0.046875 * A(&t, ic + ioff, jc + joff, kc)
                + 0.015625 * A(&t, ic + ioff, jc + joff, kc + koff);
        }
        free(t.p);
    }
}

/* MLCellLinOpT::normInf (AMReX_MLCellLinOp.H:2006-2101): the finest level
 * counts every cell; a coarser level only the cells no finer box covers */
static double amr_norminf(const Amr* M, int l, const MF* m) {
    const Level* L = &M->S[l].H.lev[0];
    if (l == M->nlev - 1) return mf_norminf(L, m);
    double r = 0.0;
    for (int b = 0; b < m->nbox; ++b) {
        Box vb = L->boxes[b];
        const Fab* f = &m->fab[b];
        for (int k = vb.lo[2]; k <= vb.hi[2]; ++k)
        for (int j = vb.lo[1]; j <= vb.hi[1]; ++j)
        for (int i = vb.lo[0]; i <= vb.hi[0]; ++i) {
            if (covered_by_fine(M, l, i, j, k)) continue;
            double v = fabs(A(f, i, j, k));
            if (v > r) r = v;
        }
    }
    return r;
}

/* MLMGT::computeMLResidual, AMReX_MLMG.H:1632-1648 */
static void amr_compute_ml_residual(Amr* M, int lmax) {
    for (int l = lmax; l >= 0; --l) {
        Solver* S = &M->S[l];
        amr_solution_residual(M, l, &S->res[0], &S->sol, &S->rhs, 1);
        if (l < M->nlev - 1) amr_reflux(M, l, &S->res[0]);
    }
}

static double amr_ml_norminf(const Amr* M, int lmax, int rhs) {
    double r = 0.0;
    for (int l = 0; l <= lmax; ++l) {
        double v = amr_norminf(M, l, rhs ? &M->S[l].rhs : &M->S[l].res[0]);
        if (v > r) r = v;
    }
    return r;
}

/* nu1 smoothing sweeps from zero: the mini-cycle of a fine AMR level */
static void amr_mini_cycle(Amr* M, int l) {
    Solver* S = &M->S[l];
    mf_setval(&S->cor[0], 0.0);
    int skip = 1;
    for (int i = 0; i < S->o.nu1; ++i) { smooth(S, 0, &S->cor[0], &S->res[0], skip); skip = 0; }
}

/* MLMGT::oneIter, AMReX_MLMG.H:1227-1293 */
static void amr_one_iter(Amr* M, int iter) {
    const int finest = M->nlev - 1;
    for (int l = finest; l > 0; --l) {
        Solver* S = &M->S[l];
        Solver* C = &M->S[l - 1];
        amr_mini_cycle(M, l);
        mf_axpy(&S->H.lev[0], &S->sol, 1.0, &S->cor[0], 1);
        /* computeResWithCrseSolFineCor(l-1, l), AMReX_MLMG.H:1660-1690 */
        amr_solution_residual(M, l - 1, &C->res[0], &C->sol, &C->rhs, 1);
        correction_residual(S, 0, &S->rescor[0], &S->cor[0], &S->res[0]);
        mf_axpy(&S->H.lev[0], &S->res[0], 0, &S->rescor[0], 0);
        amr_reflux(M, l - 1, &C->res[0]);
        amr_average_down(M, l - 1, &S->res[0], &C->res[0]);
        if (l != finest) { MF t = S->cor_hold[0]; S->cor_hold[0] = S->cor[0]; S->cor[0] = t; }
    }
    {
        Solver* S = &M->S[0];
        if (iter < S->o.max_fmg_iter) fcycle(S); else vcycle(S, 0);
        mf_axpy(&S->H.lev[0], &S->sol, 1.0, &S->cor[0], 1);
    }
    for (int l = 1; l <= finest; ++l) {
        Solver* S = &M->S[l];
        const Level* L = &S->H.lev[0];
        amr_interp_correction(M, l);
        mf_axpy(L, &S->sol, 1.0, &S->cor[0], 1);
        if (l != finest) mf_axpy(L, &S->cor_hold[0], 1.0, &S->cor[0], 1);
        /* computeResWithCrseCorFineCor(l), AMReX_MLMG.H:1693-1715 */
        amr_correction_residual_inhomog(M, l, &S->rescor[0], &S->cor[0], &S->res[0]);
        mf_axpy(L, &S->res[0], 0, &S->rescor[0], 0);
        amr_mini_cycle(M, l);
        mf_axpy(L, &S->sol, 1.0, &S->cor[0], 1);
        if (l != finest) mf_axpy(L, &S->cor[0], 1.0, &S->cor_hold[0], 1);
    }
    /* averageDownAndSync, AMReX_MLCellLinOp.H:2102-2122 */
    for (int l = finest; l > 0; --l) amr_average_down(M, l - 1, &M->S[l].sol, &M->S[l - 1].sol);
}

/* MLMGT::solve, AMReX_MLMG.H:353-541, several AMR levels (refinement ratio 2,
 * MLPoisson or MLABecLaplacian, any periodicity shared by the levels).  P[l] describes AMR level l: its domain
 * (n = n_0 2^l), boxes, right-hand side over its domain and initial guess
 * with boundary values in the ghosts (grown domain).  phi_out[l] receives the
 * level's solution on its boxes' cells (level-domain array). */
int oracle_solve_amr(int nlev, const OracleProblem* P, const OracleOptions* o, double** phi_out,
                     OracleResult* R) {
    if (nlev < 1 || nlev > AMR_MAX) return -1;
    for (int l = 0; l < nlev; ++l) {
        if (P[l].is_abec != P[0].is_abec ||
            (P[0].is_abec && (P[l].alpha != P[0].alpha || P[l].beta != P[0].beta))) return -2;
        for (int d = 0; d < 3; ++d) if (P[l].periodic[d] != P[0].periodic[d]) return -3;
    }
    Amr* M = (Amr*)calloc(1, sizeof(Amr));
    M->nlev = nlev;
    for (int l = 0; l < nlev; ++l) {
        Solver* S = &M->S[l];
        OracleOptions ol = *o;
        if (l > 0) ol.max_coarsening_level = 0;
        setup_ratio(S, &P[l], &ol, l > 0 ? 2 : 1);
        load_coeffs(S, &P[l]);
        Hier* H = &S->H;
        Level* L0 = &H->lev[0];
        S->bcval.v = P[l].sol; for (int d = 0; d < 3; ++d) S->bcval.n[d] = P[l].n[d];
        mf_define(&S->sol, L0->nbox, L0->boxes, 1, -1);
        copy_global_to_mf(L0, &S->sol, P[l].sol, 1, -1);
        mf_define(&S->rhs, L0->nbox, L0->boxes, 0, -1);
        copy_global_to_mf(L0, &S->rhs, P[l].rhs, 0, -1);
        S->volinv0 = 1.0 / (double)bnpts(&L0->domain);
        S->volinv_bottom = 1.0 / (double)bnpts(&H->lev[H->nlev - 1].domain);
        for (int q = 0; q < H->nlev; ++q) {
            Level* L = &H->lev[q];
            mf_define(&S->cor[q], L->nbox, L->boxes, 1, -1);
            mf_define(&S->res[q], L->nbox, L->boxes, 0, -1);
            mf_define(&S->rescor[q], L->nbox, L->boxes, 0, -1);
            mf_define(&S->cor_hold[q], L->nbox, L->boxes, 1, -1);
            mf_setval(&S->cor[q], 0.0);
            mf_setval(&S->res[q], 0.0);
            mf_setval(&S->rescor[q], 0.0);
            mf_setval(&S->cor_hold[q], 0.0);
        }
        if (l > 0) {
            M->bsol[l] = (Fab*)calloc((size_t)6 * L0->nbox, sizeof(Fab));
            M->bcor[l] = (Fab*)calloc((size_t)6 * L0->nbox, sizeof(Fab));
        }
    }
    Solver* S0 = &M->S[0];
    const int finest = nlev - 1;
    /* MLABecLaplacianT::averageDownCoeffs (AMReX_MLABecLaplacian.H:610-626):
     * finest to coarsest across AMR levels, then the MG levels of level 0 */
    if (S0->H.is_abec) {
        for (int l = finest; l > 0; --l) amr_average_down_coeffs(M, l - 1);
        restrict_all_coeffs(S0);
    }
    S0->singular = is_singular(S0);
    /* prepareForSolve: averageDownSolutionRHS, AMReX_MLMG.H:1025-1028 */
    for (int l = finest; l > 0; --l) {
        amr_average_down(M, l - 1, &M->S[l].sol, &M->S[l - 1].sol);
        amr_average_down(M, l - 1, &M->S[l].rhs, &M->S[l - 1].rhs);
    }
    if (S0->singular) make_solvable(S0, 0, &S0->rhs);
    amr_compute_ml_residual(M, finest);
    const double resnorm0 = amr_ml_norminf(M, finest, 0);
    const double rhsnorm0 = amr_ml_norminf(M, finest, 1);
    const double max_norm = (rhsnorm0 >= resnorm0) ? rhsnorm0 : resnorm0;
    const double tr = o->tol_rel > 1.e-16 ? o->tol_rel : 1.e-16;
    const double res_target = o->tol_abs > tr * max_norm ? o->tol_abs : tr * max_norm;
    R->init_resid = resnorm0; R->rhs_norm = rhsnorm0; R->niters = 0; R->status = 0;
    double composite = resnorm0;
    struct timespec t0, t1;
    clock_gettime(CLOCK_MONOTONIC, &t0);
    if (resnorm0 > res_target) {
        int converged = 0;
        const int niters = o->fixed_iter ? o->fixed_iter : o->max_iter;
        for (int iter = 0; iter < niters; ++iter) {
            if (S0->singular) make_solvable(S0, 0, &S0->res[0]);
            amr_one_iter(M, iter);
            /* computeResidual(finest): no reflux, boundary data from the coarser solution */
            Solver* Sf = &M->S[finest];
            amr_solution_residual(M, finest, &Sf->res[0], &Sf->sol, &Sf->rhs, 1);
            const double fine = amr_norminf(M, finest, &Sf->res[0]);
            if (R->niters < ORACLE_MAX_HIST) R->history[R->niters] = fine;
            R->niters++;
            composite = fine;
            const int fine_converged = fine <= res_target;
            if (nlev == 1 && fine_converged) {
                converged = 1;
            } else if (fine_converged) {
                amr_compute_ml_residual(M, finest - 1);
                const double crse = amr_ml_norminf(M, finest - 1, 0);
                converged = crse <= res_target;
                composite = fine > crse ? fine : crse;
            }
            if (converged) break;
            if (composite > 1.e20 * max_norm) { R->status = -2; break; }
        }
        if (!converged && o->fixed_iter == 0 && R->status == 0) R->status = 1;
    }
    clock_gettime(CLOCK_MONOTONIC, &t1);
    R->iter_seconds = (double)(t1.tv_sec - t0.tv_sec) + 1e-9 * (double)(t1.tv_nsec - t0.tv_nsec);
    R->final_resid = composite;
    R->nlev = S0->H.nlev;
    R->ncg = S0->ncg;
    for (int q = 0; q < S0->ncg && q < ORACLE_MAX_HIST; ++q) R->cg_iters[q] = S0->cg_log[q];
    for (int l = 0; l < nlev; ++l) {
        copy_mf_to_global(&M->S[l].H.lev[0], &M->S[l].sol, phi_out[l]);
        if (l > 0) {
            const int nf = 6 * M->S[l].H.lev[0].nbox;
            for (int q = 0; q < nf; ++q) { free(M->bsol[l][q].p); free(M->bcor[l][q].p); }
            free(M->bsol[l]); free(M->bcor[l]);
        }
        free_solver(&M->S[l]);
    }
    free(M);
    return R->status;
}
