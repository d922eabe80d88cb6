// Host-side grid metadata: MG hierarchy, patch levels, masks, BC records and
// ghost-copy tags.  No device code.
#pragma once

#include "common.hpp"

#include <array>
#include <memory>

namespace mlmg {

struct LPInfoC {
    int agg = 1, con = 1;
    int agg_grid_size = 32, con_grid_size = 32;   // the reference's GPU-build defaults
    int max_coarsening_level = 30;
};

struct GeomC {
    Box3 domain;
    double prob_lo[3] = {0, 0, 0}, prob_hi[3] = {1, 1, 1};
    int periodic[3] = {0, 0, 0};
    void cell_size (double dx[3], double dxinv[3]) const {
        for (int d = 0; d < 3; ++d) {
            // Geometry cell size (Src/Base/AMReX_Geometry.H:406-407)
            dx[d] = (prob_hi[d] - prob_lo[d]) / (double)domain.len(d);
            dxinv[d] = 1.0 / dx[d];
        }
    }
};

struct LevelGrids {
    GeomC geom;
    std::vector<Box3> boxes;
    // grids made by coarsening the level-0 BoxArray (BoxArray::coarsen shares
    // the data, so amrex::isMFIterSafe holds between two such levels);
    // agglomerated levels are new BoxArrays
    int derived = 1;
};

// MLLinOpT::defineGrids for AMR level 0 (Src/LinearSolvers/MLMG/AMReX_MLLinOp.H:793-1165)
std::vector<LevelGrids> define_grids (const GeomC& geom, const std::vector<Box3>& ba, const LPInfoC& info);

// Description of one solve's operator, as seen by the patch builder.
struct SolveSpec {
    GeomC geom;                       // level-0 geometry
    std::vector<LevelGrids> levels;   // MG levels
    int lobc[3], hibc[3];             // domain BC types
    int maxorder = 3;
    double alpha = 0.0, beta = 1.0;
    int is_abec = 0;
    double dx0[3];                    // level-0 cell size (BC location of internal faces)
    int crse_ratio = 1;               // refinement ratio to the next coarser AMR level (1 at AMR level 0;
                                      // at AMR level 0 of a domain it does not cover, the ratio of
                                      // setCoarseFineBC, or 0 without one): coarse/fine faces sit
                                      // 0.5 * crse_ratio * dx0 outside the box
    int amr_fine = 0;                 // a finer AMR level: one MG level that is smoothed, never bottom-solved
};

// Ghost-copy tag: copy region `box` (destination index space) of patch `dst`
// from patch `src`, whose source index is destination index - shift.
struct CopyTag {
    int dst, src;
    int shift[3];
    Box3 box;
};

// One joint level of a batch: the patches of MG level `lev` of every solve
// that has such a level.
struct PatchLevel {
    int lev = 0;
    std::vector<PatchDesc> patches;
    std::vector<int> patch_is_bottom;      // 1 if this level is the owning solve's bottom level
    std::vector<int8_t> masks;             // per-cell masks of faces whose mask is not uniform
    std::vector<CopyTag> tags;             // intra-level ghost copies (faces only)
    long long nelem = 0;                   // elements per field
    std::vector<int> solve_first_patch;    // first patch index of each solve at this level (-1 if absent)
    std::vector<int> solve_npatch;
    std::vector<Box3> rboxes;              // the solves' own (unmerged) boxes of this level, solve by solve
    std::vector<int> solve_rbox_first, solve_rbox_n;
    std::vector<int> solve_derived;        // LevelGrids::derived of each solve (0 if absent)
};

struct BoxToPatch {                        // level-0 user box -> patch location
    int patch;
};

// Which box of a BoxArray holds a cell: boxes bucketed on a coarse grid of
// 8^3-cell buckets over their bounding box, so a query checks only the few
// boxes that touch the cell's bucket.
class BoxLocator {
public:
    explicit BoxLocator (const std::vector<Box3>& boxes);
    int find (int i, int j, int k) const;   // box index, -1 if none
private:
    std::vector<Box3> m_boxes;
    Box3 m_bb;
    int m_nb[3] = {0, 0, 0};
    std::vector<int> m_start, m_list;
};

// Join boxes that share a whole face, repeatedly along x, y and z, into
// larger boxes covering the same cells (the patches of a level).
std::vector<Box3> merge_face_neighbours (std::vector<Box3> boxes);

// Build the patch layout of level `lev` for every solve in `solves`.
// Boxes of one solve's level that share whole faces are merged into larger
// patches when the merge leaves every Dirichlet closure unchanged.
PatchLevel build_patch_level (const std::vector<const SolveSpec*>& solves, int lev, bool allow_merge);

// index of cell (i,j,k) of patch p
inline long long pidx (const PatchDesc& p, int i, int j, int k)
{
    return p.base + (long long)(k - p.lo[2]) * p.sxy + (long long)(j - p.lo[1]) * p.sx + (i - p.lo[0]);
}

// poly_interp_coeff (Src/Boundary/AMReX_LOUtil_K.H:22-37)
void poly_interp_coeff (double xInt, const double* x, int N, double* c);

} // namespace mlmg
