"""Case definitions shared by the golden-fixture generator and the parity
tests.  A case is a plain dict; its inputs are rebuilt from seeds by
``inputs(case)`` so fixtures only need to store the reference's outputs.
"""
from __future__ import annotations

import os

import numpy as np

from amrex_gb300 import synth

DIRICHLET, NEUMANN, REFLECT_ODD, PERIODIC = 101, 102, 103, 200


def _c(**kw):
    base = dict(op="poisson", n=(32, 32, 32), max_grid_size=16, lobc=(101,) * 3, hibc=(101,) * 3,
                maxorder=3, agg=1, agg_grid_size=32, con=1, con_grid_size=32, periodic=(0, 0, 0),
                alpha=1.0, beta=1.0, tol_rel=1e-10, tol_abs=0.0, max_iter=200, fixed_iter=0)
    base.update(kw)
    return base


CASES = {
    # --- BoxArray::maxSize and the MG hierarchy (agglomeration) -------------
    "hier_c0_agg32": _c(mode="hier", n=(64, 64, 64), max_grid_size=32),
    "hier_c0_agg8": _c(mode="hier", n=(64, 64, 64), max_grid_size=32, agg_grid_size=8, con_grid_size=8),
    "hier_c1_agg32": _c(mode="hier", n=(256, 256, 256), max_grid_size=64),
    "hier_c1_agg8": _c(mode="hier", n=(256, 256, 256), max_grid_size=64, agg_grid_size=8, con_grid_size=8),
    "hier_48": _c(mode="hier", n=(48, 48, 48), max_grid_size=32),
    "hier_80": _c(mode="hier", n=(80, 80, 80), max_grid_size=32),
    "hier_112": _c(mode="hier", n=(112, 112, 112), max_grid_size=32),
    "hier_aniso": _c(mode="hier", n=(40, 24, 56), max_grid_size=16),
    "hier_noagg": _c(mode="hier", n=(64, 64, 64), max_grid_size=16, agg=0),
    "hier_noagg_nocon": _c(mode="hier", n=(64, 32, 32), max_grid_size=16, agg=0, con=0),
    "hier_irregular": _c(mode="hier", n=(32, 32, 32),
                         boxes=((0, 0, 0, 15, 15, 15), (16, 0, 0, 31, 15, 15), (0, 16, 0, 31, 31, 15),
                                (0, 0, 16, 31, 31, 31))),
    # --- FillBoundary ---------------------------------------------------------
    "fb_cross": _c(mode="fb", n=(16, 16, 16), max_grid_size=8, cross=1, seed=11),
    "fb_full": _c(mode="fb", n=(16, 16, 16), max_grid_size=8, cross=0, seed=12),
    "fb_periodic_cross": _c(mode="fb", n=(16, 12, 8), max_grid_size=8, periodic=(1, 1, 1), cross=1, seed=13),
    "fb_periodic_full": _c(mode="fb", n=(16, 12, 8), max_grid_size=8, periodic=(1, 0, 1), cross=0, seed=14),
    "fb_ragged": _c(mode="fb", n=(24, 20, 12), max_grid_size=8, cross=1, seed=15),
    # --- MLMG::apply (inhomogeneous Dirichlet / Neumann) ----------------------
    "apply_poisson": _c(mode="apply", n=(16, 16, 16), max_grid_size=8, sol_seed=21),
    "apply_abec": _c(mode="apply", op="abec", n=(16, 16, 16), max_grid_size=8, sol_seed=22, b_seed=23,
                     a_seed=24, alpha=0.5, beta=2.0),
    "apply_abec_mixed_bc": _c(mode="apply", op="abec", n=(24, 16, 20), max_grid_size=8, sol_seed=25,
                              b_seed=26, lobc=(101, 102, 102), hibc=(102, 101, 103)),
    "apply_abec_mo2": _c(mode="apply", op="abec", n=(16, 16, 16), max_grid_size=8, sol_seed=27, b_seed=28,
                         maxorder=2),
    # --- MLMG::solve -----------------------------------------------------------
    "solve_poisson_32": _c(mode="solve", n=(32, 32, 32), max_grid_size=16, rhs_seed=1000),
    "solve_poisson_c0": _c(mode="solve", n=(64, 64, 64), max_grid_size=32, rhs_seed=1000),
    "solve_abec_32": _c(mode="solve", op="abec", n=(32, 32, 32), max_grid_size=16, rhs_seed=1001,
                        b_seed=2001),
    "solve_abec_32_vcycle1": _c(mode="solve", op="abec", n=(32, 32, 32), max_grid_size=16, rhs_seed=1001,
                                b_seed=2001, fixed_iter=1),
    "solve_abec_48": _c(mode="solve", op="abec", n=(48, 48, 48), max_grid_size=32, rhs_seed=4001,
                        b_seed=5001),
    "solve_abec_mixed_bc": _c(mode="solve", op="abec", n=(32, 24, 16), max_grid_size=8, rhs_seed=1003,
                              b_seed=2003, a_seed=3003, alpha=1.0, beta=1.0,
                              lobc=(101, 102, 101), hibc=(102, 101, 101), sol_seed=3004),
    "solve_abec_agg8": _c(mode="solve", op="abec", n=(32, 32, 32), max_grid_size=8, rhs_seed=1005,
                          b_seed=2005, agg_grid_size=8, con_grid_size=8),
    # singular operators (solvability fix) and a 4-point Dirichlet closure
    "solve_poisson_periodic": _c(mode="solve", n=(32, 32, 32), max_grid_size=16, rhs_seed=1006,
                                 periodic=(1, 1, 1), lobc=(200,) * 3, hibc=(200,) * 3),
    "solve_abec_neumann_singular": _c(mode="solve", op="abec", n=(32, 32, 32), max_grid_size=16, rhs_seed=1007,
                                      b_seed=2007, alpha=0.0, lobc=(102,) * 3, hibc=(102,) * 3),
    "solve_abec_mo4": _c(mode="solve", op="abec", n=(32, 32, 32), max_grid_size=16, rhs_seed=1008, b_seed=2008,
                         maxorder=4),
    "solve_poisson_periodic_x": _c(mode="solve", n=(32, 24, 16), max_grid_size=8, rhs_seed=1009,
                                   periodic=(1, 0, 0), lobc=(200, 101, 102), hibc=(200, 102, 101)),
    # --- F-cycles (max_fmg_iter > 0): mgFcycle with trilinear interpAssign ---
    "solve_abec_32_fmg": _c(mode="solve", op="abec", n=(32, 32, 32), max_grid_size=16, rhs_seed=1001,
                            b_seed=2001, max_fmg_iter=200),
    "solve_poisson_c0_fmg": _c(mode="solve", n=(64, 64, 64), max_grid_size=32, rhs_seed=1000, max_fmg_iter=2),
    "solve_abec_mixed_bc_fmg": _c(mode="solve", op="abec", n=(32, 24, 16), max_grid_size=8, rhs_seed=1003,
                                  b_seed=2003, a_seed=3003, lobc=(101, 102, 101), hibc=(102, 101, 101),
                                  sol_seed=3004, max_fmg_iter=200),
    "solve_poisson_periodic_x_fmg": _c(mode="solve", n=(32, 24, 16), max_grid_size=8, rhs_seed=1009,
                                       periodic=(1, 0, 0), lobc=(200, 101, 102), hibc=(200, 102, 101),
                                       max_fmg_iter=200),
    "solve_abec_agg8_fmg": _c(mode="solve", op="abec", n=(32, 32, 32), max_grid_size=8, rhs_seed=1005,
                              b_seed=2005, agg_grid_size=8, con_grid_size=8, max_fmg_iter=200),
    # --- bottom solvers other than BiCGStab (MLMG::BottomSolver cg, bicgcg,
    # cgbicg): with a small bottom_maxiter the first solver of bicgcg / cgbicg
    # fails and the second runs (cgbicg then switches to BiCGStab for good)
    "solve_abec_cg": _c(mode="solve", op="abec", n=(32, 32, 32), max_grid_size=8, rhs_seed=1005, b_seed=2005,
                        bottom_solver=3),
    "solve_poisson_cg": _c(mode="solve", n=(32, 32, 32), max_grid_size=16, rhs_seed=1000, bottom_solver=3),
    "solve_abec_cgbicg": _c(mode="solve", op="abec", n=(32, 32, 32), max_grid_size=8, rhs_seed=1005, b_seed=2005,
                            bottom_solver=5, bottom_maxiter=4),
    "solve_abec_bicgcg": _c(mode="solve", op="abec", n=(32, 32, 32), max_grid_size=8, rhs_seed=1005, b_seed=2005,
                            bottom_solver=4, bottom_maxiter=3),
    "solve_poisson_bicgcg": _c(mode="solve", n=(32, 32, 32), max_grid_size=8, rhs_seed=1005, bottom_solver=4,
                               bottom_maxiter=2),
    # --- MLMG::getFluxes / getGradSolution after a solve ----------------------
    "flux_abec_32": _c(mode="flux", op="abec", n=(32, 32, 32), max_grid_size=16, rhs_seed=1011, b_seed=2011,
                       beta=2.0),
    "flux_abec_mixed_bc": _c(mode="flux", op="abec", n=(32, 24, 16), max_grid_size=8, rhs_seed=1012,
                             b_seed=2012, a_seed=3012, sol_seed=3013, alpha=1.0, beta=0.5,
                             lobc=(101, 102, 101), hibc=(102, 101, 101)),
    "flux_poisson_32": _c(mode="flux", n=(32, 32, 32), max_grid_size=16, rhs_seed=1013, sol_seed=3014),
    "flux_poisson_periodic_x": _c(mode="flux", n=(32, 24, 16), max_grid_size=8, rhs_seed=1014,
                                  periodic=(1, 0, 0), lobc=(200, 101, 102), hibc=(200, 102, 101)),
    # --- MLMG::compResidual of a random initial guess (inhomogeneous BCs) ----
    "resid_abec_32": _c(mode="resid", op="abec", n=(32, 32, 32), max_grid_size=16, rhs_seed=1001, b_seed=2001,
                        sol_seed=3021),
    "resid_abec_mixed_bc": _c(mode="resid", op="abec", n=(32, 24, 16), max_grid_size=8, rhs_seed=1003,
                              b_seed=2003, a_seed=3003, alpha=0.75, beta=1.5, lobc=(101, 102, 101),
                              hibc=(102, 101, 101), sol_seed=3022),
    "resid_poisson_periodic_x": _c(mode="resid", n=(32, 24, 16), max_grid_size=8, rhs_seed=1009,
                                   periodic=(1, 0, 0), lobc=(200, 101, 102), hibc=(200, 102, 101), sol_seed=3023),
    # --- a level that does not cover its domain: coarse/fine faces take
    # Dirichlet values interpolated from a coarse MultiFab
    # (MLLinOp::setCoarseFineBC, refinement ratio 2), or zero coarse values
    # at ratio 2 when none is given
    "cf_solve_poisson": _c(mode="solve", n=(32, 32, 32), boxes=((8, 8, 8, 23, 23, 23),), rhs_seed=1015,
                             crse_ratio=2, crse_seed=6001, crse_mgs=8),
    "cf_solve_abec": _c(mode="solve", op="abec", n=(32, 32, 32), rhs_seed=1016, b_seed=2016, sol_seed=3024,
                          boxes=((0, 8, 8, 15, 23, 23), (16, 8, 8, 31, 23, 23), (0, 24, 8, 15, 31, 23)),
                          crse_ratio=2, crse_seed=6002, crse_mgs=8),
    "cf_uncovered_poisson": _c(mode="solve", n=(32, 32, 32), boxes=((8, 8, 8, 23, 23, 23),), rhs_seed=1015),
    "cf_resid_abec": _c(mode="resid", op="abec", n=(32, 32, 32), rhs_seed=1016, b_seed=2016, sol_seed=3025,
                          boxes=((0, 8, 8, 15, 23, 23), (16, 8, 8, 31, 23, 23), (0, 24, 8, 15, 31, 23)),
                          crse_ratio=2, crse_seed=6002, crse_mgs=8),
    # --- MLMG::setFinalFillBC with a solution of two ghost cells ----------------
    "ffbc_solve_abec": _c(mode="solve", op="abec", n=(32, 24, 16), max_grid_size=8, rhs_seed=1003, b_seed=2003,
                          sol_seed=3026, lobc=(101, 102, 101), hibc=(102, 101, 101), sol_ngrow=2, final_fill_bc=1),
    "ffbc_off_solve_abec": _c(mode="solve", op="abec", n=(32, 24, 16), max_grid_size=8, rhs_seed=1003, b_seed=2003,
                            sol_seed=3026, lobc=(101, 102, 101), hibc=(102, 101, 101), sol_ngrow=2, final_fill_bc=0),
}


# --- full-size solves, kept as statistics and seeded samples of phi -------
# (make_large_golden.py): the 256^3 variable-coefficient benchmark (max grid
# size 64) and four solves of the 64-solve batch (cube edges from
# {32, 48, ..., 128}, max grid size 32, solve i with seeds 4001 + i: solves 0,
# 1, 5 and 7 are 128^3, 80^3, 48^3 and 112^3; 80, 48 and 112 chop into ragged
# boxes of 32 + 32 + 16, 32 + 16 and 32 + 32 + 32 + 16 cells)
LARGE_CASES = {
    "large_c1_256": _c(mode="solve", op="abec", n=(256, 256, 256), max_grid_size=64, rhs_seed=1001, b_seed=2001),
    "large_c4_128": _c(mode="solve", op="abec", n=(128, 128, 128), max_grid_size=32, rhs_seed=4001, b_seed=4001),
    "large_c4_80": _c(mode="solve", op="abec", n=(80, 80, 80), max_grid_size=32, rhs_seed=4002, b_seed=4002),
    "large_c4_48": _c(mode="solve", op="abec", n=(48, 48, 48), max_grid_size=32, rhs_seed=4006, b_seed=4006),
    "large_c4_112": _c(mode="solve", op="abec", n=(112, 112, 112), max_grid_size=32, rhs_seed=4008, b_seed=4008),
}


def large_sample_index(size, count=4096):
    """seeded sample of positions into a whole-domain phi (x fastest)"""
    rng = np.random.Generator(np.random.PCG64(7100))
    return np.sort(rng.choice(size, size=min(count, size), replace=False))


def sol_grown(case):
    """Initial guess (valid cells) and Dirichlet values (ghost cells) on the
    domain grown by one cell, shape (nz+2, ny+2, nx+2)."""
    nx, ny, nz = case["n"]
    if "sol_seed" not in case:
        return np.zeros((nz + 2, ny + 2, nx + 2))
    rng = np.random.Generator(np.random.PCG64(case["sol_seed"]))
    v = rng.uniform(-1.0, 1.0, size=(nz + 2, ny + 2, nx + 2))
    if case["mode"] in ("solve", "flux"):
        v[1:-1, 1:-1, 1:-1] = 0.0
    return v


def inputs(case):
    """All array inputs of a case, rebuilt from its seeds."""
    n = case["n"]
    nx, ny, nz = n
    d = {"sol": sol_grown(case)}
    d["rhs"] = synth.gaussian_rhs(n, case["rhs_seed"]) if "rhs_seed" in case else np.zeros((nz, ny, nx))
    if case["op"] == "abec":
        if "b_seed" in case:
            d["bx"], d["by"], d["bz"] = synth.lognormal_bcoef(n, case["b_seed"], sigma_cells=case.get("b_sigma", 5.0),
                                                               max_ratio=case.get("b_ratio", 1e3))
        else:
            d["bx"], d["by"], d["bz"] = (np.ones((nz, ny, nx + 1)), np.ones((nz, ny + 1, nx)),
                                        np.ones((nz + 1, ny, nx)))
        if "a_seed" in case:
            rng = np.random.Generator(np.random.PCG64(case["a_seed"]))
            d["a"] = rng.uniform(0.5, 1.5, size=(nz, ny, nx))
        else:
            d["a"] = np.ones((nz, ny, nx))
    if "crse_seed" in case:
        # coarse data for the coarse/fine faces over the coarsened domain
        r = case["crse_ratio"]
        d["crse"] = synth.gaussian_rhs((nx // r, ny // r, nz // r), case["crse_seed"])
    return d


def boxes_of(case):
    """Box list of the case as (lo, hi) tuples; max_grid_size chopping is done
    by the library under test, so this only returns explicit boxes."""
    return case.get("boxes")


def max_size_boxes(n, chunk):
    """BoxArray(domain).maxSize(chunk) for a domain with lower corner 0,
    restated from BoxList::maxSize (Src/Base/AMReX_BoxList.cpp:765-824):
    per direction the length is halved together with the chunk while both
    are even, split into ceil(len/chunk) blocks whose sizes differ by at most
    one (the first ``extra`` blocks one larger), then scaled back up.  Boxes
    are ordered with x fastest."""
    ranges = []
    for d in range(3):
        nlen, bs, ratio = n[d], chunk, 1
        if nlen <= chunk:
            ranges.append([(0, nlen - 1)])
            continue
        while bs % 2 == 0 and nlen % 2 == 0:
            ratio, bs, nlen = ratio * 2, bs // 2, nlen // 2
        nblk = (nlen + bs - 1) // bs
        sz = nlen // nblk
        extra = nlen - sz * nblk
        r = []
        for b in range(nblk):
            if b < extra:
                lo = b * (sz + 1) * ratio
                hi = lo + (sz + 1) * ratio - 1
            else:
                lo = (b * sz + extra) * ratio
                hi = lo + sz * ratio - 1
            r.append((lo, hi))
        ranges.append(r)
    return [((xr[0], yr[0], zr[0]), (xr[1], yr[1], zr[1]))
            for zr in ranges[2] for yr in ranges[1] for xr in ranges[0]]


def fb_input(case):
    """Per-box grown FAB data for the FillBoundary cases, in box order, x
    fastest.  The box list is the one the reference's BoxArray::maxSize makes;
    the values are a function of a seed and the total size only."""
    boxes = max_size_boxes(case["n"], case["max_grid_size"]) if "boxes" not in case else \
        [((b[0], b[1], b[2]), (b[3], b[4], b[5])) for b in case["boxes"]]
    total = 0
    for lo, hi in boxes:
        total += (hi[0] - lo[0] + 3) * (hi[1] - lo[1] + 3) * (hi[2] - lo[2] + 3)
    rng = np.random.Generator(np.random.PCG64(case["seed"]))
    return rng.uniform(-1.0, 1.0, size=total)


def write_inputs(case, d):
    """Write the binary inputs of ``case`` into directory ``d``; returns the
    case-file keys that name them."""
    files = {}
    if case["mode"] == "fb":
        fb_input(case).astype(np.float64).tofile(os.path.join(d, "fb_in.bin"))
        return files
    if case["mode"] == "hier":
        return files
    inp = inputs(case)
    inp["sol"].astype(np.float64).tofile(os.path.join(d, "sol.bin"))
    files["sol_file"] = "sol.bin"
    inp["rhs"].astype(np.float64).tofile(os.path.join(d, "rhs.bin"))
    files["rhs_file"] = "rhs.bin"
    if case["op"] == "abec":
        for k in ("a", "bx", "by", "bz"):
            inp[k].astype(np.float64).tofile(os.path.join(d, k + ".bin"))
            files[k + "_file"] = k + ".bin"
    if "crse" in inp:
        inp["crse"].astype(np.float64).tofile(os.path.join(d, "crse.bin"))
        files["crse_file"] = "crse.bin"
    return files


def case_text(case, files):
    lines = []
    for k in ("op", "n", "max_grid_size", "lobc", "hibc", "maxorder", "agg", "agg_grid_size", "con",
              "con_grid_size", "periodic", "alpha", "beta", "tol_rel", "tol_abs", "max_iter", "fixed_iter",
              "cross", "max_fmg_iter", "bottom_solver", "bottom_maxiter", "repeat", "verbose", "crse_ratio", "crse_mgs",
              "sol_ngrow", "final_fill_bc"):
        if k in case:
            v = case[k]
            lines.append(k + " " + (" ".join(str(x) for x in v) if isinstance(v, (tuple, list)) else str(v)))
    if "boxes" in case:
        lines.append("boxes " + " ".join(str(x) for b in case["boxes"] for x in b))
    for k, v in files.items():
        lines.append(f"{k} {v}")
    return "\n".join(lines) + "\n"
