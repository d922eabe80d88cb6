// Shared definitions of the GB300 MLMG library: error handling, boxes,
// patch descriptors.  Host and device.
#pragma once

#include <cstdint>
#include <cstdio>
#include <stdexcept>
#include <string>
#include <vector>

#include <cuda_runtime.h>

namespace mlmg {

// ---------------------------------------------------------------- errors ---
struct Error : std::runtime_error {
    int code;
    Error (int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

// status codes of the C ABI (negative = error)
enum Status : int {
    OK = 0,
    NOT_CONVERGED = 1,      // max iterations reached
    ERR_ARGS = -1,          // invalid argument / handle
    ERR_DIVERGED = -2,      // residual > 1e20 * norm ("MLMG blew up")
    ERR_CUDA = -3,          // a CUDA call failed
    ERR_UNSUPPORTED = -4,   // valid request outside what this build implements
    ERR_NONFINITE = -5,     // NaN/Inf in the residual
    ERR_INTERNAL = -6,
    ERR_TIMEOUT = -7,       // bounded device wait expired
};

#define MLMG_CUDA_CHECK(expr)                                                          \
    do {                                                                               \
        cudaError_t e_ = (expr);                                                       \
        if (e_ != cudaSuccess) {                                                       \
            throw ::mlmg::Error(::mlmg::ERR_CUDA, std::string(#expr " failed: ") +     \
                                cudaGetErrorString(e_) + " at " + __FILE__ + ":" +     \
                                std::to_string(__LINE__));                             \
        }                                                                              \
    } while (0)

#define MLMG_REQUIRE(cond, code, msg)                                                  \
    do { if (!(cond)) { throw ::mlmg::Error((code), (msg)); } } while (0)

// ----------------------------------------------------------------- boxes ---
struct Box3 {
    int lo[3], hi[3];
    __host__ __device__ int len (int d) const { return hi[d] - lo[d] + 1; }
    __host__ __device__ long long npts () const {
        return (long long)len(0) * len(1) * len(2);
    }
    __host__ __device__ bool ok () const { return hi[0] >= lo[0] && hi[1] >= lo[1] && hi[2] >= lo[2]; }
    __host__ __device__ bool contains (int i, int j, int k) const {
        return i >= lo[0] && i <= hi[0] && j >= lo[1] && j <= hi[1] && k >= lo[2] && k <= hi[2];
    }
    bool operator== (const Box3& o) const {
        for (int d = 0; d < 3; ++d) { if (lo[d] != o.lo[d] || hi[d] != o.hi[d]) { return false; } }
        return true;
    }
    bool operator!= (const Box3& o) const { return !(*this == o); }
};

inline int floordiv (int a, int r) { return (a >= 0) ? a / r : -((-a + r - 1) / r); }

inline Box3 coarsen (Box3 b, int r)
{
    for (int d = 0; d < 3; ++d) { b.lo[d] = floordiv(b.lo[d], r); b.hi[d] = floordiv(b.hi[d], r); }
    return b;
}
inline Box3 refine (Box3 b, int r)
{
    for (int d = 0; d < 3; ++d) { b.lo[d] *= r; b.hi[d] = (b.hi[d] + 1) * r - 1; }
    return b;
}
inline Box3 grow (Box3 b, int g)
{
    for (int d = 0; d < 3; ++d) { b.lo[d] -= g; b.hi[d] += g; }
    return b;
}
inline Box3 intersect (const Box3& a, const Box3& b)
{
    Box3 r;
    for (int d = 0; d < 3; ++d) {
        r.lo[d] = a.lo[d] > b.lo[d] ? a.lo[d] : b.lo[d];
        r.hi[d] = a.hi[d] < b.hi[d] ? a.hi[d] : b.hi[d];
    }
    return r;
}
inline Box3 shift (Box3 b, const int* s)
{
    for (int d = 0; d < 3; ++d) { b.lo[d] += s[d]; b.hi[d] += s[d]; }
    return b;
}

// Box::coarsenable(refrat, min_width) (Src/Base/AMReX_Box.H:745-755)
inline bool coarsenable (const Box3& b, int r, int min_width)
{
    for (int d = 0; d < 3; ++d) { if (b.len(d) < r * min_width) { return false; } }
    return refine(coarsen(b, r), r) == b;
}

// BoxList::maxSize (Src/Base/AMReX_BoxList.cpp:765-824)
std::vector<Box3> max_size (const std::vector<Box3>& in, const int chunk[3]);

// ---------------------------------------------------- LinOp BC codes ------
enum BCType : int { BC_INTERIOR = 0, BC_DIRICHLET = 101, BC_NEUMANN = 102, BC_REFLECT_ODD = 103,
                    BC_PERIODIC = 200 };

// mask values (Src/Boundary/AMReX_BndryData.H:44)
enum MaskVal : int { MASK_COVERED = 0, MASK_NOT_COVERED = 1, MASK_OUTSIDE = 2 };

// --------------------------------------------------------- patch layout ---
// A patch is one rectangular block of cells of one MG level of one solve,
// stored with a one-cell ghost layer; every field of the level uses the same
// layout, so one index serves all arrays.  Face-centred coefficients bX/bY/bZ
// live at the cell index of their low-side cell: bX(i) for i = lo..hi+1, the
// hi+1 entry sitting in the ghost column.
//
// index(i,j,k) = base + (k-lo2)*sxy + (j-lo1)*sx + (i-lo0)
struct FaceBC {
    int type;            // BC type code (only used where the mask is > 0)
    int nx;              // number of interpolation points of the Dirichlet closure
    int mask_uniform;    // uniform mask value of the face, or -1 if per-cell
    int on_domain;       // 1 if the patch face lies on the domain boundary (periodic or not)
    long long mask_off;  // offset of the per-cell mask (int8) in the level's mask array
    long long bcval_off; // offset of the face's Dirichlet values in the level's bcval array, -1 if none
    double coef[4];      // closure coefficients (coef[0] multiplies the boundary value)
    double fco;          // f coefficient of the smoother's diagonal correction
};

struct PatchDesc {
    int lo[3], hi[3];
    long long base;      // element offset of cell lo
    long long sxy;       // z stride (elements)
    int sx;              // y stride (elements)
    int solve;           // owning solve of a batch
    double dx[3], dxinv[3];
    double alpha, beta;  // ABec scalars of the owning solve (Poisson: 0, 1)
    double dha[3];       // operator/normalize factors: beta*dxinv*dxinv (Poisson: dxinv*dxinv)
    double dhs[3];       // smoother factors: beta/(dx*dx) (Poisson: dxinv*dxinv)
    FaceBC face[6];      // Orientation order: xlo, ylo, zlo, xhi, yhi, zhi
};

// x offset of the first valid cell within a row, and row pitch rounding, in
// elements; rows of every patch start 64-byte aligned for fp64 and fp32
constexpr int XOFF = 8;
constexpr int XALIGN = 8;

} // namespace mlmg
