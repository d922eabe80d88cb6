"""The oracle's AMR composite solve (MLMG over several AMR levels, refinement
ratio 2, MLPoisson and MLABecLaplacian) against the reference's own composite solves on
AmrMesh-generated grids (tests/golden/amrsolve_*.npz)."""
from __future__ import annotations

import numpy as np
import pytest

from oracle import oracle
from tests.golden import amr_cases as ac


def oracle_case(case):
    n = case["n"]
    out = dict(n=(n, n, n), tol_rel=case.get("tol_rel", 1e-10), tol_abs=0.0,
               agg_grid_size=case.get("agg_grid_size", 32), con_grid_size=case.get("con_grid_size", 32),
               max_fmg_iter=case.get("max_fmg_iter", 0))
    if case.get("abec"):
        out.update(op="abec", alpha=case["abec"][0], beta=case["abec"][1])
    if case.get("periodic"):
        per = tuple(case["periodic"])
        bc = tuple(200 if p else 101 for p in per)
        out.update(periodic=per, lobc=bc, hibc=bc)
    return out


def levels_of(case, grids):
    out = []
    for lev in range(len(grids)):
        L = dict(boxes=grids[lev], rhs=ac.level_rhs(case, lev))
        sb = ac.level_solbc(case, lev)
        if sb is not None:
            L["sol"] = sb
        co = ac.level_abec(case, lev)
        if co is not None:
            L.update(zip(("a", "bx", "by", "bz"), co[2:]))
        out.append(L)
    return out


@pytest.mark.parametrize("name", ["c2_n16_2lev", "c2_n32", "c2_n16_2lev_bc", "c2_n32_fmg", "c2_n16_2lev_abec",
                                  "c2_n32_abec", "c2_n16_2lev_per", "c2_n32_per", "c2_n16_2lev_per_abec",
                                  "c2_n16_4lev"])
def test_oracle_amr_matches_reference(name):
    """Iteration and bottom counts, norms, residual history and phi (every
    cell, or per-level statistics and seeded samples for summary fixtures);
    the cases cover 2, 3 and 4 levels, inhomogeneous Dirichlet values with a
    non-zero initial guess, F-cycles on AMR level 0, MLABecLaplacian with
    per-level coefficients (averaged down across levels before level 0's MG
    restriction), and domains periodic in x and y with fine boxes on the
    periodic faces."""
    g = ac.load("amrsolve", name)
    case, grids, ref = g["case"], g["grids"], g["result"]
    phis, info = oracle.solve_amr(oracle_case(case), levels_of(case, grids))
    assert info["status"] == 0
    assert info["niters"] == ref["niters"]
    assert info["cg_iters"] == ref["cg_iters"]
    assert info["init_resid"] == pytest.approx(ref["init_resid"], rel=1e-13)
    assert info["rhs_norm"] == pytest.approx(ref["rhs_norm"], rel=1e-13)
    # the convergence path to 1e-6 (it pins the coefficient average-down of the
    # MLABecLaplacian cases); residuals near 1e-10 carry roundoff from the
    # order of the flux-register sums
    ac.check_history(info["history"], ref)
    for lev in range(len(grids)):
        got = ac.pack_boxes(phis[lev], grids[lev])
        if f"phi_l{lev}" in g:
            want = g[f"phi_l{lev}"]
            np.testing.assert_allclose(got, want, rtol=0, atol=1e-12 * np.abs(want).max())
        else:
            st = g[f"phi_l{lev}_stats"]
            assert np.abs(got).max() == pytest.approx(st[0], rel=1e-12)
            want = g[f"phi_l{lev}_sample"]
            np.testing.assert_allclose(got[ac.sample_index(got.size, lev)], want, rtol=0, atol=1e-12 * st[0])


def test_amr_grids_are_properly_nested():
    """Every fixture's finer boxes sit inside the next coarser level grown by
    one coarse cell (AmrMesh proper nesting), the premise of the oracle's and
    the engine's coarse/fine boundary interpolation."""
    for name in ("c2", "c2_n32", "c2_n16_2lev", "c2_n16_2lev_abec", "c2_n32_abec"):
        g = ac.load("amrgrids", name)
        n = g["case"]["n"]
        grids = g["grids"]
        for lev in range(1, len(grids)):
            m = n << (lev - 1)
            cov = np.zeros((m + 2,) * 3, dtype=bool)
            for b in grids[lev - 1]:
                cov[b[2] + 1:b[5] + 2, b[1] + 1:b[4] + 2, b[0] + 1:b[3] + 2] = True
            # cells outside the domain count as covered
            cov[0, :, :] = cov[-1, :, :] = True
            cov[:, 0, :] = cov[:, -1, :] = True
            cov[:, :, 0] = cov[:, :, -1] = True
            for b in grids[lev]:
                lo = [v // 2 for v in b[:3]]
                hi = [v // 2 for v in b[3:]]
                assert all(v % 2 == 0 for v in b[:3]) and all(v % 2 == 1 for v in b[3:])
                blk = cov[lo[2]:hi[2] + 3, lo[1]:hi[1] + 3, lo[0]:hi[0] + 3]
                assert blk.all(), (name, lev, b)


def test_box_rhs_matches_whole_domain_rhs():
    """The box-restricted RHS generator the GPU workloads use gives the
    whole-domain generator's values bit for bit."""
    from amrex_gb300 import synth
    full = synth.gaussian_rhs(32, 1002)
    for b in [(0, 0, 0, 7, 7, 7), (8, 16, 4, 23, 31, 11), (5, 3, 30, 5, 9, 31)]:
        box = synth.gaussian_rhs_box(32, 1002, b)
        np.testing.assert_array_equal(box, full[b[2]:b[5] + 1, b[1]:b[4] + 1, b[0]:b[3] + 1])
