// Host-side grid metadata of the GB300 MLMG: BoxArray chopping, the MG
// hierarchy with agglomeration, patch merging, masks and BC records.
#include "hierarchy.hpp"

#include <algorithm>
#include <array>
#include <map>
#include <cmath>
#include <cstring>

namespace mlmg {

std::vector<Box3> max_size (const std::vector<Box3>& in, const int chunk[3])
{
    // BoxList::maxSize (Src/Base/AMReX_BoxList.cpp:765-824): per direction the
    // length is halved together with the chunk while both are even, then split
    // into ceil(len/chunk) blocks whose sizes differ by at most one (the first
    // `extra` blocks one larger); x varies fastest in the output.
    std::vector<Box3> out;
    for (const Box3& bx : in) {
        int ratio[3] = {1, 1, 1}, numblk[3] = {1, 1, 1}, extra[3] = {0, 0, 0}, sz[3];
        for (int d = 0; d < 3; ++d) {
            sz[d] = bx.len(d);
            if (bx.len(d) > chunk[d]) {
                int bs = chunk[d], nlen = bx.len(d);
                while ((bs % 2 == 0) && (nlen % 2 == 0)) { ratio[d] *= 2; bs /= 2; nlen /= 2; }
                numblk[d] = (nlen + bs - 1) / bs;
                sz[d] = nlen / numblk[d];
                extra[d] = nlen - sz[d] * numblk[d];
            }
        }
        for (int k = 0; k < numblk[2]; ++k)
        for (int j = 0; j < numblk[1]; ++j)
        for (int i = 0; i < numblk[0]; ++i) {
            const int idx[3] = {i, j, k};
            Box3 nb;
            for (int d = 0; d < 3; ++d) {
                if (numblk[d] == 1) { nb.lo[d] = bx.lo[d]; nb.hi[d] = bx.hi[d]; continue; }
                const int b = idx[d];
                const int lo = (b < extra[d]) ? b * (sz[d] + 1) * ratio[d] : (b * sz[d] + extra[d]) * ratio[d];
                const int hi = (b < extra[d]) ? lo + (sz[d] + 1) * ratio[d] - 1 : lo + sz[d] * ratio[d] - 1;
                nb.lo[d] = lo + bx.lo[d];
                nb.hi[d] = hi + bx.lo[d];
            }
            out.push_back(nb);
        }
    }
    return out;
}

void poly_interp_coeff (double xInt, const double* x, int N, double* c)
{
    for (int j = 0; j < N; ++j) {
        double num = 1.0, den = 1.0;
        for (int i = 0; i < N; ++i) {
            if (i != j) { num *= xInt - x[i]; den *= x[j] - x[i]; }
        }
        c[j] = num / den;
    }
}

static bool all_coarsenable (const std::vector<Box3>& bs, int r, int mw)
{
    for (const auto& b : bs) { if (!coarsenable(b, r, mw)) { return false; } }
    return true;
}

std::vector<LevelGrids> define_grids (const GeomC& geom, const std::vector<Box3>& ba, const LPInfoC& info)
{
    // MLLinOpT::defineGrids (Src/LinearSolvers/MLMG/AMReX_MLLinOp.H:793-1165),
    // AMR level 0, no semicoarsening, no hidden direction.  Consolidation only
    // changes the distribution map, so on one GPU it leaves plain coarsenings.
    const int mg_box_min_width = 2, mg_domain_min_width = 2;
    const Box3 dom = geom.domain;
    long long npts0 = 0;
    for (const auto& b : ba) { npts0 += b.npts(); }
    const bool domain_covered = (npts0 == dom.npts());

    std::vector<LevelGrids> out;
    out.push_back({geom, ba});

    auto make_geom = [&] (const Box3& d) { GeomC g = geom; g.domain = d; return g; };

    Box3 aggbox{};
    bool aggable = false;
    if (ba.size() > 1 && info.agg) {
        if (domain_covered) {
            aggbox = dom; aggable = true;
        } else {
            aggbox = ba[0];
            for (const auto& b : ba) {
                for (int d = 0; d < 3; ++d) {
                    aggbox.lo[d] = std::min(aggbox.lo[d], b.lo[d]);
                    aggbox.hi[d] = std::max(aggbox.hi[d], b.hi[d]);
                }
            }
            aggable = (aggbox.npts() == npts0);
        }
    }

    if (info.agg && aggable) {
        Box3 dbx = dom, bbx = aggbox;
        const double nbxs = (double)ba.size();
        const double threshold_npts = (double)info.agg_grid_size * info.agg_grid_size * info.agg_grid_size;
        std::vector<Box3> domainboxes{dbx}, boundboxes{bbx};
        std::vector<int> agg_flag{0}, accum{1};
        for (int lev = 0; lev < info.max_coarsening_level; ++lev) {
            if (!(coarsenable(dbx, 2, mg_domain_min_width) && coarsenable(bbx, 2, mg_box_min_width))) { break; }
            accum.push_back(accum.back() * 2);
            dbx = coarsen(dbx, 2);
            bbx = coarsen(bbx, 2);
            domainboxes.push_back(dbx);
            boundboxes.push_back(bbx);
            agg_flag.push_back(((double)bbx.npts() / nbxs) < 0.999 * threshold_npts);
        }
        bool agged = false;
        for (size_t lev = 1; lev < domainboxes.size(); ++lev) {
            LevelGrids L;
            if (!agged && !agg_flag[lev] && all_coarsenable(ba, accum[lev], mg_box_min_width)) {
                for (const auto& b : ba) { L.boxes.push_back(coarsen(b, accum[lev])); }
            } else {
                const int cr = domainboxes[lev - 1].len(0) / domainboxes[lev].len(0);
                if (!all_coarsenable(out.back().boxes, cr, 1)) { break; }
                const int chunk[3] = {info.agg_grid_size, info.agg_grid_size, info.agg_grid_size};
                L.boxes = max_size({boundboxes[lev]}, chunk);
                L.derived = 0;
                agged = true;
            }
            L.geom = make_geom(domainboxes[lev]);
            out.push_back(std::move(L));
        }
    } else {
        int rr = 1;
        for (int lev = 0; lev < info.max_coarsening_level; ++lev) {
            const int r2 = rr * 2;
            if (!(coarsenable(dom, r2, mg_domain_min_width) && all_coarsenable(ba, r2, mg_box_min_width))) { break; }
            rr = r2;
            LevelGrids L;
            L.geom = make_geom(coarsen(dom, rr));
            for (const auto& b : ba) { L.boxes.push_back(coarsen(b, rr)); }
            out.push_back(std::move(L));
        }
    }
    return out;
}

namespace {

// wrap a cell index into the domain along periodic directions; false if it
// lies outside along a non-periodic direction
bool wrap (const GeomC& g, int c[3])
{
    for (int d = 0; d < 3; ++d) {
        const int n = g.domain.len(d);
        if (c[d] < g.domain.lo[d] || c[d] > g.domain.hi[d]) {
            if (!g.periodic[d]) { return false; }
            c[d] = g.domain.lo[d] + ((c[d] - g.domain.lo[d]) % n + n) % n;
        }
    }
    return true;
}

Box3 adj_cell (const Box3& b, int f)
{
    const int d = f % 3;
    Box3 r = b;
    if (f >= 3) { r.lo[d] = r.hi[d] = b.hi[d] + 1; } else { r.lo[d] = r.hi[d] = b.lo[d] - 1; }
    return r;
}

} // namespace

BoxLocator::BoxLocator (const std::vector<Box3>& boxes) : m_boxes(boxes)
{
    if (boxes.empty()) { return; }
    m_bb = boxes[0];
    for (const auto& b : boxes) {
        for (int d = 0; d < 3; ++d) { m_bb.lo[d] = std::min(m_bb.lo[d], b.lo[d]); m_bb.hi[d] = std::max(m_bb.hi[d], b.hi[d]); }
    }
    for (int d = 0; d < 3; ++d) { m_nb[d] = (m_bb.len(d) + 7) / 8; }
    const size_t nbk = (size_t)m_nb[0] * m_nb[1] * m_nb[2];
    std::vector<int> cnt(nbk + 1, 0);
    auto each_bucket = [&] (const Box3& b, auto&& fn) {
        int lo[3], hi[3];
        for (int d = 0; d < 3; ++d) { lo[d] = (b.lo[d] - m_bb.lo[d]) / 8; hi[d] = (b.hi[d] - m_bb.lo[d]) / 8; }
        for (int z = lo[2]; z <= hi[2]; ++z)
        for (int y = lo[1]; y <= hi[1]; ++y)
        for (int x = lo[0]; x <= hi[0]; ++x) { fn(((size_t)z * m_nb[1] + y) * m_nb[0] + x); }
    };
    for (const auto& b : boxes) { each_bucket(b, [&] (size_t q) { cnt[q + 1]++; }); }
    for (size_t q = 0; q < nbk; ++q) { cnt[q + 1] += cnt[q]; }
    m_start = cnt;
    m_list.assign((size_t)cnt[nbk], 0);
    std::vector<int> fill(cnt.begin(), cnt.end() - 1);
    for (int bi = 0; bi < (int)boxes.size(); ++bi) {
        each_bucket(boxes[bi], [&] (size_t q) { m_list[(size_t)fill[q]++] = bi; });
    }
}

int BoxLocator::find (int i, int j, int k) const
{
    if (m_boxes.empty() || !m_bb.contains(i, j, k)) { return -1; }
    const size_t q = ((size_t)((k - m_bb.lo[2]) / 8) * m_nb[1] + (j - m_bb.lo[1]) / 8) * m_nb[0] + (i - m_bb.lo[0]) / 8;
    for (int t = m_start[q]; t < m_start[q + 1]; ++t) {
        if (m_boxes[(size_t)m_list[(size_t)t]].contains(i, j, k)) { return m_list[(size_t)t]; }
    }
    return -1;
}

std::vector<Box3> merge_face_neighbours (std::vector<Box3> b)
{
    std::vector<char> alive(b.size(), 1);
    bool changed = true;
    while (changed) {
        changed = false;
        for (int d = 0; d < 3; ++d) {
            const int t1 = (d == 0) ? 1 : 0, t2 = (d == 2) ? 1 : 2;
            auto key = [&] (const Box3& x, int pos) {
                return std::array<int, 5>{x.lo[t1], x.hi[t1], x.lo[t2], x.hi[t2], pos};
            };
            std::map<std::array<int, 5>, int> by_lo;
            for (int i = 0; i < (int)b.size(); ++i) { if (alive[i]) { by_lo[key(b[i], b[i].lo[d])] = i; } }
            for (int i = 0; i < (int)b.size(); ++i) {
                if (!alive[i]) { continue; }
                for (;;) {
                    auto it = by_lo.find(key(b[i], b[i].hi[d] + 1));
                    if (it == by_lo.end() || it->second == i) { break; }
                    const int j = it->second;
                    b[i].hi[d] = b[j].hi[d];
                    alive[j] = 0;
                    by_lo.erase(it);
                    changed = true;
                }
            }
        }
    }
    std::vector<Box3> out;
    for (size_t i = 0; i < b.size(); ++i) { if (alive[i]) { out.push_back(b[i]); } }
    return out;
}

PatchLevel build_patch_level (const std::vector<const SolveSpec*>& solves, int lev, bool allow_merge)
{
    PatchLevel PL;
    PL.lev = lev;
    PL.solve_first_patch.assign(solves.size(), -1);
    PL.solve_npatch.assign(solves.size(), 0);
    PL.solve_rbox_first.assign(solves.size(), 0);
    PL.solve_rbox_n.assign(solves.size(), 0);
    PL.solve_derived.assign(solves.size(), 0);
    long long cursor = 0;
    for (size_t s = 0; s < solves.size(); ++s) {
        const SolveSpec& S = *solves[s];
        if (lev >= (int)S.levels.size()) { continue; }
        const LevelGrids& LG = S.levels[lev];
        PL.solve_rbox_first[s] = (int)PL.rboxes.size();
        PL.solve_rbox_n[s] = (int)LG.boxes.size();
        PL.solve_derived[s] = LG.derived;
        PL.rboxes.insert(PL.rboxes.end(), LG.boxes.begin(), LG.boxes.end());
        const bool is_bottom = (lev == (int)S.levels.size() - 1) && !S.amr_fine;
        const BoxLocator loc(LG.boxes);
        double dx[3], dxinv[3];
        LG.geom.cell_size(dx, dxinv);

        // merge decision: boxes that share a whole face join one patch while
        // every box is at least maxorder-1 cells long, so that each Dirichlet
        // closure keeps its interpolation points
        std::vector<Box3> pboxes = LG.boxes;
        if (allow_merge && LG.boxes.size() > 1) {
            int minlen = 1 << 30;
            for (const auto& b : LG.boxes) {
                for (int d = 0; d < 3; ++d) { minlen = std::min(minlen, b.len(d)); }
            }
            if (minlen >= S.maxorder - 1) { pboxes = merge_face_neighbours(LG.boxes); }
        }

        PL.solve_first_patch[s] = (int)PL.patches.size();
        PL.solve_npatch[s] = (int)pboxes.size();
        for (const Box3& pb : pboxes) {
            PatchDesc P{};
            for (int d = 0; d < 3; ++d) { P.lo[d] = pb.lo[d]; P.hi[d] = pb.hi[d]; }
            const int nx = pb.len(0), ny = pb.len(1), nz = pb.len(2);
            // row: XOFF cells before lo, the patch, and at least 7 cells after
            // hi, so 16-byte staged copies of any row chunk touching the patch
            // stay inside the row
            P.sx = ((XOFF + nx + 8 + XALIGN - 1) / XALIGN) * XALIGN;
            P.sxy = (long long)P.sx * (ny + 2);
            cursor = ((cursor + XALIGN - 1) / XALIGN) * XALIGN;
            P.base = cursor + P.sxy + P.sx + XOFF;
            cursor += P.sxy * (nz + 2);
            P.solve = (int)s;
            for (int d = 0; d < 3; ++d) { P.dx[d] = dx[d]; P.dxinv[d] = dxinv[d]; }
            P.alpha = S.alpha;
            P.beta = S.beta;
            for (int d = 0; d < 3; ++d) {
                if (S.is_abec) {
                    // MLABecLaplacianT::Fapply / Fsmooth (AMReX_MLABecLaplacian.H:775-1126)
                    P.dha[d] = S.beta * dxinv[d] * dxinv[d];
                    P.dhs[d] = S.beta / (dx[d] * dx[d]);
                } else {
                    // MLPoissonT::Fapply / Fsmooth (AMReX_MLPoisson.H:180-420)
                    P.dha[d] = dxinv[d] * dxinv[d];
                    P.dhs[d] = dxinv[d] * dxinv[d];
                }
            }
            for (int f = 0; f < 6; ++f) {
                const int d = f % 3;
                const bool hi = f >= 3;
                FaceBC& F = P.face[f];
                const bool on_domain = hi ? (LG.geom.domain.hi[d] == pb.hi[d]) : (LG.geom.domain.lo[d] == pb.lo[d]);
                F.on_domain = on_domain ? 1 : 0;
                double bcl;
                // MLMGBndryT::setBoxBC (Src/LinearSolvers/MLMG/AMReX_MLMGBndry.H:106-150)
                if (on_domain && !LG.geom.periodic[d]) {
                    F.type = hi ? S.hibc[d] : S.lobc[d];
                    bcl = 0.0;
                } else {
                    F.type = BC_DIRICHLET;            // coarse/fine BC type
                    bcl = 0.5 * (double)S.crse_ratio * S.dx0[d];
                }
                F.coef[0] = F.coef[1] = F.coef[2] = F.coef[3] = 0.0;
                F.nx = 0;
                if (F.type == BC_DIRICHLET) {
                    const int blen = pb.len(d);
                    F.nx = std::min(blen + 1, S.maxorder);
                    const double x[4] = {-bcl * dxinv[d], 0.5, 1.5, 2.5};
                    poly_interp_coeff(-0.5, x, F.nx, F.coef);
                }
                // f coefficient (mllinop_comp_interp_coef0_*, AMReX_MLLinOp_K.H:327-420),
                // applied only where the mask is > 0
                F.fco = (F.type == BC_DIRICHLET) ? F.coef[1] : ((F.type == BC_NEUMANN || F.type == BC_REFLECT_ODD) ? 1.0 : 0.0);
                // mask of the outside layer (MultiMask::define, Src/Boundary/AMReX_MultiMask.cpp:25-69)
                const Box3 ab = adj_cell(pb, f);
                std::vector<int8_t> m;
                m.reserve((size_t)ab.npts());
                for (int k = ab.lo[2]; k <= ab.hi[2]; ++k)
                for (int j = ab.lo[1]; j <= ab.hi[1]; ++j)
                for (int i = ab.lo[0]; i <= ab.hi[0]; ++i) {
                    int c[3] = {i, j, k};
                    int v;
                    if (!wrap(LG.geom, c)) { v = MASK_OUTSIDE; }
                    else {
                        // covered by a box of the same level (original boxes, which
                        // cover the same cells as the patches)
                        v = (loc.find(c[0], c[1], c[2]) >= 0) ? MASK_COVERED : MASK_NOT_COVERED;
                    }
                    m.push_back((int8_t)v);
                }
                bool uniform = true;
                for (auto v : m) { if (v != m[0]) { uniform = false; break; } }
                if (uniform) {
                    F.mask_uniform = m.empty() ? 0 : m[0];
                    F.mask_off = -1;
                } else {
                    F.mask_uniform = -1;
                    F.mask_off = (long long)PL.masks.size();
                    PL.masks.insert(PL.masks.end(), m.begin(), m.end());
                }
                F.bcval_off = -1;
            }
            PL.patches.push_back(P);
            PL.patch_is_bottom.push_back(is_bottom ? 1 : 0);
        }

        // intra-level face-ghost copies (periodic images included)
        const int first = PL.solve_first_patch[s];
        for (size_t q = 0; q < pboxes.size(); ++q) {
            const Box3& vb = pboxes[q];
            for (int f = 0; f < 6; ++f) {
                const Box3 slab = adj_cell(vb, f);
                int sh[3];
                for (int sz = -1; sz <= 1; ++sz)
                for (int sy = -1; sy <= 1; ++sy)
                for (int sxx = -1; sxx <= 1; ++sxx) {
                    const int sv[3] = {sxx, sy, sz};
                    bool okp = true;
                    for (int d = 0; d < 3; ++d) {
                        if (sv[d] != 0 && !LG.geom.periodic[d]) { okp = false; }
                        sh[d] = sv[d] * LG.geom.domain.len(d);
                    }
                    if (!okp) { continue; }
                    for (size_t r = 0; r < pboxes.size(); ++r) {
                        const Box3 src = shift(pboxes[r], sh);
                        const Box3 isect = intersect(slab, src);
                        if (!isect.ok()) { continue; }
                        CopyTag t;
                        t.dst = first + (int)q;
                        t.src = first + (int)r;
                        for (int d = 0; d < 3; ++d) { t.shift[d] = sh[d]; }
                        t.box = isect;
                        PL.tags.push_back(t);
                    }
                }
            }
        }
    }
    PL.nelem = ((cursor + 63) / 64) * 64;
    return PL;
}

} // namespace mlmg
