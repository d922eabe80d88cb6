"""GPU composite (multi-AMR-level) MLPoisson and MLABecLaplacian solves
through the C ABI against the reference's own composite solves on AmrMesh
grids (tests/golden/amrsolve_*.npz) and, at the configuration size, against
per-level statistics and sampled values of the reference solution."""
from __future__ import annotations

import numpy as np
import pytest

import amrex_gb300 as ag
from amrex_gb300 import workloads
from tests.golden import amr_cases as ac

pytestmark = pytest.mark.gpu

SMALL = ["c2_n16_2lev", "c2_n32", "c2_n16_2lev_bc", "c2_n16_2lev_abec", "c2_n16_2lev_per", "c2_n16_2lev_per_abec"]
SUMMARY = ["c2_n32_fmg", "c2_n32_abec", "c2_n32_per", "c2_n16_4lev"]


def _phi_error(g, lev, got):
    """max |phi - phi_ref| / max |phi_ref| over every cell, or over the
    seeded samples of a summary fixture"""
    if f"phi_l{lev}" in g:
        want = g[f"phi_l{lev}"]
        return np.abs(got - want).max() / np.abs(want).max()
    st = g[f"phi_l{lev}_stats"]
    return np.abs(got[ac.sample_index(got.size, lev)] - g[f"phi_l{lev}_sample"]).max() / st[0]


def _solve(name, precision=0, graph=False, tol_rel=None, fused=False, options=None):
    g = ac.load("amrsolve", name)
    case, grids = g["case"], g["grids"]
    solbc = [ac.level_solbc(case, lev) for lev in range(len(grids))]
    abec = [ac.level_abec(case, lev) for lev in range(len(grids))] if case.get("abec") else None
    P = workloads.amr_problem(case["n"], grids, case["rhs_seed"], precision=precision, graph=graph,
                              agg_grid_size=case.get("agg_grid_size", 32), con_grid_size=case.get("con_grid_size", 32),
                              fused=fused, solbc=solbc, max_fmg_iter=case.get("max_fmg_iter", 0), abec=abec,
                              periodic=case.get("periodic", (0, 0, 0)))
    for k, v in (options or {}).items():
        P["mlmg"].setOption(k, v)
    resid = P["mlmg"].solve(P["sols"], P["rhss"], tol_rel or case.get("tol_rel", 1e-10), 0.0)
    phis = []
    for lev, boxes in enumerate(grids):
        sol = P["sols"][lev]
        phis.append(np.concatenate([sol.get_fab(i)[1:-1, 1:-1, 1:-1].ravel() for i in range(len(boxes))]))
    return g, P, resid, phis


@pytest.mark.parametrize("name", SMALL + SUMMARY)
def test_amr_fp64_matches_reference(name):
    g, P, resid, phis = _solve(name, precision=0)
    ref = g["result"]
    m = P["mlmg"]
    assert m.getNumIters() == ref["niters"]
    assert m.getNumCGIters() == ref["cg_iters"]
    assert m.getInitResidual() == pytest.approx(ref["init_resid"], rel=1e-12)
    assert m.getInitRHS() == pytest.approx(ref["rhs_norm"], rel=1e-12)
    # fine residual history: the convergence path to 1e-6, the entries near
    # roundoff (1e-10 * |rhs|) to 1e-4
    ac.check_history(m.getResidualHistory(), ref)
    assert resid <= 1e-10 * max(ref["rhs_norm"], ref["init_resid"])
    for lev in range(len(phis)):
        err = _phi_error(g, lev, phis[lev])
        assert err < 1e-10, (lev, err)


@pytest.mark.parametrize("name", SMALL + SUMMARY)
@pytest.mark.parametrize("graph,fused", [(False, False), (True, False), (True, True)])
def test_amr_mixed_reaches_target(name, graph, fused):
    """FP32 corrections inside the FP64 composite residual reach the same
    1e-10 relative composite residual; the solution agrees with the
    reference's FP64 solution to within the discretisation-free tolerance
    that a 1e-10 residual allows."""
    g, P, resid, phis = _solve(name, precision=1, graph=graph, fused=fused)
    ref = g["result"]
    assert resid <= 1e-10 * max(ref["rhs_norm"], ref["init_resid"])
    assert P["mlmg"].getNumIters() <= ref["niters"] + 3
    for lev in range(len(phis)):
        err = _phi_error(g, lev, phis[lev])
        assert err < 1e-8, (lev, err)


@pytest.mark.parametrize("name", ["c2_n16_2lev", "c2_n32", "c2_n16_2lev_bc", "c2_n16_2lev_per", "c2_n32_fmg",
                                  "c2_n16_4lev"])
def test_amr_fused_fine_sweeps_bitwise(name):
    """On the fine AMR levels, fused two-colour sweeps on the tiles whose halo
    meets no face shared with another patch, with colour passes on the other
    tiles, give the solution of colour passes on every tile bit for bit."""
    _, P1, r1, phis1 = _solve(name, precision=1, graph=True, fused=True, options={"fused_fine": 1})
    _, P2, r2, phis2 = _solve(name, precision=1, graph=True, fused=True, options={"fused_fine": 2})
    assert P1["mlmg"].getNumIters() == P2["mlmg"].getNumIters()
    assert r1 == r2
    for a, b in zip(phis1, phis2):
        np.testing.assert_array_equal(a, b)


@pytest.mark.parametrize("name", ["c2_n32", "c2_n16_2lev_bc", "c2_n16_2lev_per", "c2_n16_2lev_abec", "c2_n16_4lev"])
@pytest.mark.parametrize("precision", [0, 1])
def test_amr_dependent_launches_bitwise(name, precision):
    """Programmatic dependent launches (every composite-path kernel waits on
    its predecessor with griddepcontrol.wait) change only when kernels start:
    the solutions with and without them are bit for bit the same."""
    _, P1, r1, phis1 = _solve(name, precision=precision, graph=True, fused=bool(precision), options={"pdl": 1})
    _, P0, r0, phis0 = _solve(name, precision=precision, graph=True, fused=bool(precision), options={"pdl": 0})
    assert P1["mlmg"].getNumIters() == P0["mlmg"].getNumIters()
    assert r1 == r0
    for a, b in zip(phis1, phis0):
        np.testing.assert_array_equal(a, b)


def test_amr_graph_replay_matches_eager_fp64():
    _, P0, r0, phis0 = _solve("c2_n32", precision=0, graph=False)
    _, P1, r1, phis1 = _solve("c2_n32", precision=0, graph=True)
    assert P0["mlmg"].getNumIters() == P1["mlmg"].getNumIters()
    for a, b in zip(phis0, phis1):
        np.testing.assert_array_equal(a, b)


def test_amr_config_size_against_reference_summary():
    """The 3-level composite configuration (base 128^3, 57 and 495 boxes on
    levels 1 and 2): FP64 iteration and bottom counts equal the reference's,
    per-level statistics and sampled solution values agree to 1e-9; the mixed
    solve reaches the same residual target and agrees to 1e-8."""
    g = ac.load("amrsolve", "c2")
    ref = g["result"]
    for precision, tol in ((0, 1e-9), (1, 1e-8)):
        _, P, resid, phis = _solve("c2", precision=precision, graph=True, fused=precision == 1)
        m = P["mlmg"]
        assert resid <= 1e-10 * max(ref["rhs_norm"], ref["init_resid"])
        if precision == 0:
            assert m.getNumIters() == ref["niters"]
            assert m.getNumCGIters() == ref["cg_iters"]
        for lev in range(len(phis)):
            st = g[f"phi_l{lev}_stats"]
            scale = st[0]
            assert np.abs(phis[lev]).max() == pytest.approx(st[0], rel=tol)
            idx = ac.sample_index(phis[lev].size, lev)
            err = np.abs(phis[lev][idx] - g[f"phi_l{lev}_sample"]).max() / scale
            assert err < tol, (precision, lev, err)


def test_amr_rejects_unsupported_and_bad_nesting():
    n = 16
    grids = ac.load("amrgrids", "c2_n16_2lev")["grids"]
    # a fine box whose coarsening grown by one leaves level 0
    bad = [[(0, 0, 0, 7, 7, 7)], [(0, 0, 0, 15, 15, 15)]]
    P = workloads.amr_problem(n, bad, 1012)
    with pytest.raises(ag.MLMGError) as e:
        P["mlmg"].solve(P["sols"], P["rhss"], 1e-10, 0.0)
    assert e.value.code == -1
    # single-level calls on a composite operator
    P = workloads.amr_problem(n, grids, 1012)
    with pytest.raises(ag.MLMGError) as e:
        P["mlmg"].solve(P["sols"][0], P["rhss"][0], 1e-10, 0.0)
    assert e.value.code in (-1, -4)


def test_amr_abec_coefficient_arguments():
    """Per-level coefficients of a composite MLABecLaplacian: a MultiFab on
    another level's BoxArray, or an AMR level out of range, is rejected (-1)
    before any solve."""
    g = ac.load("amrsolve", "c2_n16_2lev_abec")
    case, grids = g["case"], g["grids"]
    abec = [ac.level_abec(case, lev) for lev in range(len(grids))]
    P = workloads.amr_problem(case["n"], grids, case["rhs_seed"], abec=abec)
    op = P["op"]
    wrong = ag.MultiFab(P["bas"][0], P["dms"][0], 1, 0)      # level 0's BoxArray offered for level 1
    with pytest.raises(ag.MLMGError) as e:
        op.setACoeffs(1, wrong)
    assert e.value.code == -1
    with pytest.raises(ag.MLMGError) as e:
        op.setACoeffs(len(grids), 1.0)
    assert e.value.code == -1
    # the rejected calls left the operator as it was: the solve still matches the reference
    resid = P["mlmg"].solve(P["sols"], P["rhss"], 1e-10, 0.0)
    assert P["mlmg"].getNumIters() == g["result"]["niters"]
    assert resid <= 1e-10 * max(g["result"]["rhs_norm"], g["result"]["init_resid"])
