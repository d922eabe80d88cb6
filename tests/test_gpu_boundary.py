"""The C-ABI entries that complete the reference's Fortran-interface surface
for this path, against the reference's own outputs (tests/golden/):

* mlmg_comp_residual (MLMG::compResidual, amrex_fi_multigrid_comp_residual):
  one level (``resid_*``) and over AMR levels (``amrresid_*``);
* mlmg_linop_set_coarse_fine_bc (MLLinOp::setCoarseFineBC,
  amrex_fi_linop_set_coarse_fine_bc): single-level solves and a residual on a
  level that does not cover its domain (``cf_*``);
* mlmg_set_final_fill_bc (MLMG::setFinalFillBC,
  amrex_fi_multigrid_set_final_fill_bc): the ghost cells of a two-ghost
  solution after the solve (``ffbc_*``).

Needs a GPU."""
import numpy as np
import pytest

import amrex_gb300 as ag
from amrex_gb300 import workloads
from tests import helpers
from tests.golden import amr_cases as ac
from tests.golden import cases, load

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("name", load.names("resid_"))
def test_comp_residual_one_level(name, precision):
    g = load.load(name)
    c = g["case"]
    nx, ny, nz = c["n"]
    prob = helpers.make_problem(c, cases.inputs(c), precision=precision)
    res = ag.MultiFab(prob["ba"], prob["dm"], 1, 0)
    before = prob["sol"].get_global((nz + 2, ny + 2, nx + 2), lo=(-1, -1, -1))
    prob["mlmg"].compResidual(res, prob["sol"], prob["rhs"])
    got = res.get_global((nz, ny, nx))
    ref = g["res"].reshape(got.shape)
    np.testing.assert_allclose(got, ref, rtol=0, atol=1e-13 * np.abs(ref).max())
    assert np.array_equal(before, prob["sol"].get_global((nz + 2, ny + 2, nx + 2), lo=(-1, -1, -1)))


@pytest.mark.parametrize("precision", [0, 1])
@pytest.mark.parametrize("name", ["c2_n16_2lev_resid", "c2_n32_resid", "c2_n16_2lev_abec_resid",
                                  "c2_n16_2lev_per_resid"])
def test_comp_residual_amr_levels(name, precision):
    g = ac.load("amrresid", name)
    case, grids = g["case"], g["grids"]
    nl = len(grids)
    solbc = [ac.level_solbc(case, lev) for lev in range(nl)]
    abec = [ac.level_abec(case, lev) for lev in range(nl)] if case.get("abec") else None
    P = workloads.amr_problem(case["n"], grids, case["rhs_seed"], precision=precision, solbc=solbc, abec=abec,
                              periodic=case.get("periodic", (0, 0, 0)))
    res = [ag.MultiFab(P["bas"][lev], P["dms"][lev], 1, 0) for lev in range(nl)]
    P["mlmg"].compResidual(res, P["sols"], P["rhss"])
    for lev, boxes in enumerate(grids):
        got = np.concatenate([res[lev].get_fab(i).ravel() for i in range(len(boxes))])
        want = g[f"res_l{lev}"]
        np.testing.assert_allclose(got, want, rtol=0, atol=1e-12 * np.abs(want).max(), err_msg=f"level {lev}")


def _cf_problem(name, precision, graph=False, fused=False):
    g = load.load(name)
    c = g["case"]
    inp = cases.inputs(c)
    prob = helpers.make_problem(c, inp, precision=precision, graph=graph, fused=fused)
    crse = None
    if "crse_ratio" in c:
        nx, ny, nz = c["n"]
        r = c["crse_ratio"]
        cdom = ag.Box((0, 0, 0), (nx // r - 1, ny // r - 1, nz // r - 1))
        cba = ag.BoxArray(cdom).maxSize(c["crse_mgs"])
        crse = ag.MultiFab(cba, ag.DistributionMapping(cba), 1, 0)
        crse.set_global(inp["crse"])
        prob["op"].setCoarseFineBC(crse, r)
    prob["keep"].append(crse)
    return g, c, prob


@pytest.mark.parametrize("name", ["cf_solve_poisson", "cf_solve_abec", "cf_uncovered_poisson"])
def test_coarse_fine_bc_fp64_solve(name):
    """FP64 on a level that does not cover its domain: the reference's
    iteration and bottom counts, history and phi to 1e-10."""
    g, c, prob = _cf_problem(name, "fp64")
    prob["mlmg"].solve(prob["sol"], prob["rhs"], c["tol_rel"], c["tol_abs"])
    r = g["result"]
    assert prob["mlmg"].getNumIters() == r["niters"]
    assert prob["mlmg"].getNumCGIters() == r["cg_iters"]
    np.testing.assert_allclose(prob["mlmg"].getResidualHistory(), r["history"], rtol=1e-6,
                               atol=1e-13 * max(r["rhs_norm"], r["init_resid"]))
    nx, ny, nz = c["n"]
    phi = prob["sol"].get_global((nz, ny, nx))
    ref = g["phi"].reshape(phi.shape)
    mask = np.zeros(phi.shape, dtype=bool)
    for b in c["boxes"]:
        mask[b[2]:b[5] + 1, b[1]:b[4] + 1, b[0]:b[3] + 1] = True
    assert np.abs(phi - ref)[mask].max() <= 1e-10 * np.abs(ref[mask]).max()


@pytest.mark.parametrize("graph,fused", [(False, False), (True, True)])
@pytest.mark.parametrize("name", ["cf_solve_poisson", "cf_solve_abec"])
def test_coarse_fine_bc_mixed_reaches_target(name, graph, fused):
    g, c, prob = _cf_problem(name, "mixed", graph=graph, fused=fused)
    resid = prob["mlmg"].solve(prob["sol"], prob["rhs"], c["tol_rel"], c["tol_abs"])
    r = g["result"]
    assert resid <= c["tol_rel"] * max(r["rhs_norm"], r["init_resid"])
    nx, ny, nz = c["n"]
    phi = prob["sol"].get_global((nz, ny, nx))
    ref = g["phi"].reshape(phi.shape)
    mask = np.zeros(phi.shape, dtype=bool)
    for b in c["boxes"]:
        mask[b[2]:b[5] + 1, b[1]:b[4] + 1, b[0]:b[3] + 1] = True
    assert np.abs(phi - ref)[mask].max() <= 1e-8 * np.abs(ref[mask]).max()


def test_coarse_fine_bc_residual():
    g, c, prob = _cf_problem("cf_resid_abec", "fp64")
    nx, ny, nz = c["n"]
    res = ag.MultiFab(prob["ba"], prob["dm"], 1, 0)
    prob["mlmg"].compResidual(res, prob["sol"], prob["rhs"])
    got = res.get_global((nz, ny, nx))
    ref = g["res"].reshape(got.shape)
    mask = np.zeros(got.shape, dtype=bool)
    for b in c["boxes"]:
        mask[b[2]:b[5] + 1, b[1]:b[4] + 1, b[0]:b[3] + 1] = True
    np.testing.assert_allclose(got[mask], ref[mask], rtol=0, atol=1e-13 * np.abs(ref[mask]).max())


def test_coarse_fine_bc_arguments():
    g, c, prob = _cf_problem("cf_solve_poisson", "fp64")
    cba = ag.BoxArray(ag.Box((0, 0, 0), (7, 7, 7)))
    crse = ag.MultiFab(cba, ag.DistributionMapping(cba), 1, 0)
    with pytest.raises(ag.MLMGError) as e:
        prob["op"].setCoarseFineBC(crse, 4)
    assert e.value.code == -4
    prob["op"].setCoarseFineBC(None, 2)        # clears: zero coarse values at ratio 2


def _face_ghost_mask(shape, ng):
    """cells of a grown FAB (z, y, x) in its first ghost layer with exactly
    one coordinate outside the valid box"""
    nz, ny, nx = shape
    z, y, x = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    out = [(v < ng) | (v >= n - ng) for v, n in ((z, nz), (y, ny), (x, nx))]
    first = [(v == ng - 1) | (v == n - ng) for v, n in ((z, nz), (y, ny), (x, nx))]
    nout = out[0].astype(int) + out[1] + out[2]
    return (nout == 1) & (first[0] | first[1] | first[2])


@pytest.mark.parametrize("precision,graph,fused", [("fp64", False, False), ("mixed", True, True)])
@pytest.mark.parametrize("name", ["ffbc_solve_abec", "ffbc_off_solve_abec"])
def test_final_fill_bc_two_ghost_solution(name, precision, graph, fused):
    """With final_fill_bc the first ghost layer of a two-ghost solution gets
    the reference's values (boundary closures, neighbouring boxes); without
    it every ghost cell keeps its value."""
    g = load.load(name)
    c = g["case"]
    inp = cases.inputs(c)
    prob = helpers.make_problem(c, inp, precision=precision, graph=graph, fused=fused)
    sol2 = ag.MultiFab(prob["ba"], prob["dm"], 1, 2)
    sol2.setVal(0.0)
    sol2.set_global(inp["sol"], lo=(-1, -1, -1))
    before = [sol2.get_fab(b) for b in range(prob["ba"].size())]
    prob["mlmg"].setFinalFillBC(c["final_fill_bc"])
    prob["mlmg"].solve(sol2, prob["rhs"], c["tol_rel"], c["tol_abs"])
    off = 0
    tol = 1e-10 if precision == "fp64" else 1e-8
    scale = np.abs(g["phi"]).max()
    for b in range(prob["ba"].size()):
        got = sol2.get_fab(b)
        want = g["phi_fabs"][off:off + got.size].reshape(got.shape)
        off += got.size
        valid = np.zeros(got.shape, dtype=bool)
        valid[2:-2, 2:-2, 2:-2] = True
        assert np.abs(got - want)[valid].max() <= tol * scale
        ghosts = _face_ghost_mask(got.shape, 2)
        if c["final_fill_bc"]:
            assert np.abs(got - want)[ghosts].max() <= tol * scale, f"box {b}"
        else:
            assert np.array_equal(got[~valid], before[b][~valid]), f"box {b}"
