"""Failure paths of the solve, made on the host or by a wait bound of zero
(no GPU fault, trap or hang): a NaN planted in the host right-hand side, an
iteration limit that stops the solve early, an indefinite operator whose
residual grows past 1e20 times its starting norm (the oracle, which follows
the reference's test at AMReX_MLMG.H:478-509, diverges in the same
iteration), and a fused-sweep tile wait that expires.  Needs a GPU."""
import numpy as np
import pytest

import amrex_gb300 as ag
from oracle import oracle
from tests import helpers
from tests.golden import cases, load

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision,graph,fused", [("fp64", False, False), ("mixed", True, True)])
def test_nan_in_host_rhs_is_reported(precision, graph, fused):
    c = load.load("solve_abec_32")["case"]
    inp = cases.inputs(c)
    inp["rhs"] = inp["rhs"].copy()
    inp["rhs"][5, 7, 9] = np.nan                  # planted before the upload
    prob = helpers.make_problem(c, inp, precision=precision, graph=graph, fused=fused)
    rc, _ = prob["mlmg"].solve_status(prob["sol"], prob["rhs"], 1e-10, 0.0)
    assert rc == -5


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_iteration_limit_reports_not_converged(precision):
    c = load.load("solve_abec_32")["case"]
    prob = helpers.make_problem(c, cases.inputs(c), precision=precision)
    prob["mlmg"].setMaxIter(1)
    rc, resid = prob["mlmg"].solve_status(prob["sol"], prob["rhs"], 1e-10, 0.0)
    assert rc == 1
    assert prob["mlmg"].getNumIters() == 1
    hist = prob["mlmg"].getResidualHistory()
    assert len(hist) == 1 and hist[0] == resid
    assert resid > 1e-10 * max(prob["mlmg"].getInitRHS(), prob["mlmg"].getInitResidual())


def test_divergence_is_reported_in_the_oracle_iteration():
    """alpha = -50: an indefinite operator; the residual blows up and the
    solve stops with -2 in the iteration the oracle stops in."""
    c = cases._c(mode="solve", op="abec", n=(16, 16, 16), max_grid_size=8, rhs_seed=1001, alpha=-50.0, beta=1.0)
    inp = cases.inputs(c)
    _, info = oracle.solve(c, inp)
    assert info["status"] == -2
    prob = helpers.make_problem(c, inp, precision="fp64")
    rc, resid = prob["mlmg"].solve_status(prob["sol"], prob["rhs"], 1e-10, 0.0)
    assert rc == -2
    assert prob["mlmg"].getNumIters() == info["niters"]
    assert resid > 1e20 * max(prob["mlmg"].getInitRHS(), prob["mlmg"].getInitResidual())


def test_expired_tile_wait_is_reported_and_the_solver_recovers():
    """With a wait bound of zero polls every tile of the TMA fused sweep gives
    up on its staging copy, waits (with the full bound) for that copy to land
    and leaves; the solve returns -7.  The same solver with the default bound
    then solves to the reference's answer."""
    g = load.load("solve_abec_48")
    c = g["case"]
    prob = helpers.make_problem(c, cases.inputs(c), precision="mixed", graph=True, fused=True)
    m = prob["mlmg"]
    m.setMaxIter(3)
    m.setOption("tma_wait_limit", 0)
    rc, _ = m.solve_status(prob["sol"], prob["rhs"], 1e-10, 0.0)
    assert rc == -7
    assert "TMA" in ag.capi.lib().mlmg_last_error().decode()
    m.setOption("tma_wait_limit", -1)
    m.setMaxIter(200)
    prob["sol"].setVal(0.0)
    resid = m.solve(prob["sol"], prob["rhs"], c["tol_rel"], c["tol_abs"])
    r = g["result"]
    assert resid <= c["tol_rel"] * max(r["rhs_norm"], r["init_resid"])
    phi = helpers.solution(prob, c)
    ref = g["phi"].reshape(phi.shape)
    assert np.abs(phi - ref).max() <= 1e-8 * np.abs(ref).max()
