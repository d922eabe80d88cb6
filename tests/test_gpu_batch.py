"""Batched independent solves (one launch per V-cycle stage for all solves)
against the reference's golden answers and against the same solves run one
at a time.  Needs a CUDA GPU (GB300)."""
import numpy as np
import pytest

import amrex_gb300 as ag
from tests import helpers
from tests.golden import cases, load

pytestmark = pytest.mark.gpu

# uneven shapes, box sizes, BC types, maxorder 4, an inhomogeneous Dirichlet
# level BC, agglomeration grid size 8 and a singular (all-Neumann, alpha=0) one
ABEC_CASES = ["solve_abec_32", "solve_abec_48", "solve_abec_mixed_bc", "solve_abec_agg8",
              "solve_abec_neumann_singular", "solve_abec_mo4"]


def _batch(names, precision):
    probs, gold = [], []
    for nm in names:
        g = load.load(nm)
        c = g["case"]
        probs.append(helpers.make_problem(c, cases.inputs(c), precision=precision))
        gold.append(g)
    return probs, gold


def _tol(names):
    c = load.load(names[0])["case"]
    return c["tol_rel"], c["tol_abs"]


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_batched_golden_cases(precision):
    """Every solve of a heterogeneous batch matches the reference: FP64 with
    the reference's iteration count and phi to 1e-10; mixed reaching the same
    relative residual target."""
    probs, gold = _batch(ABEC_CASES, precision)
    tol_rel, tol_abs = _tol(ABEC_CASES)
    st = ag.solve_batched([p["mlmg"] for p in probs], [p["sol"] for p in probs], [p["rhs"] for p in probs],
                          tol_rel, tol_abs)
    assert st == [0] * len(probs)
    for nm, p, g in zip(ABEC_CASES, probs, gold):
        c, r = g["case"], g["result"]
        phi = helpers.solution(p, c)
        ref = g["phi"].reshape(phi.shape)
        if "singular" in nm:
            phi, ref = phi - phi.mean(), ref - ref.mean()
        if precision == "fp64":
            assert p["mlmg"].getNumIters() == r["niters"], nm
            assert np.abs(phi - ref).max() <= 1e-10 * np.abs(ref).max(), nm
        else:
            target = c["tol_rel"] * max(r["rhs_norm"], r["init_resid"])
            assert p["mlmg"].getFinalResidual() <= target, nm
            assert p["mlmg"].getNumIters() <= r["niters"] + 2, nm
            assert np.abs(phi - ref).max() <= 1e-8 * np.abs(ref).max(), nm


@pytest.mark.parametrize("precision,graph,fused", [("fp64", False, False), ("mixed", True, True)])
def test_batched_equals_sequential(precision, graph, fused):
    """A batch of uneven cubes (edges from {32, 48, 64}, max_grid_size 32,
    per-solve seeds) gives every solve the iteration count and phi of the same
    solve run alone."""
    from amrex_gb300 import workloads
    edges = [32, 48, 64, 48, 32]
    specs = [workloads.BatchSolveSpec(n, 4001 + i, 4001 + i) for i, n in enumerate(edges)]
    batch = [workloads.abec_problem(s.n, 32, s.rhs_seed, s.b_seed) for s in specs]
    alone = [workloads.abec_problem(s.n, 32, s.rhs_seed, s.b_seed) for s in specs]
    ms = []
    for p in batch:
        m = ag.MLMG(p["op"])
        m.setPrecision(precision)
        m.setGraph(graph)
        m.setFusedSmoother(fused)
        ms.append(m)
    st = ag.solve_batched(ms, [p["sol"] for p in batch], [p["rhs"] for p in batch], 1e-10, 0.0)
    assert st == [0] * len(batch)
    for p, q, mb in zip(batch, alone, ms):
        m = ag.MLMG(q["op"])
        m.setPrecision(precision)
        m.setGraph(graph)
        m.setFusedSmoother(fused)
        m.solve(q["sol"], q["rhs"], 1e-10, 0.0)
        assert mb.getNumIters() == m.getNumIters()
        n = p["n"]
        a, b = p["sol"].get_global((n, n, n)), q["sol"].get_global((n, n, n))
        assert np.abs(a - b).max() <= 1e-12 * np.abs(b).max()


def test_batched_repeat_reuses_engine():
    """A second batched call on the same solvers (new RHS values) reuses the
    engine and answers like a fresh one."""
    from amrex_gb300 import workloads
    ps = [workloads.abec_problem(n, 32, 4100 + n, 4200 + n) for n in (32, 48)]
    ms = [ag.MLMG(p["op"]) for p in ps]
    for m in ms:
        m.setPrecision("mixed")
    for rep in range(2):
        for p in ps:
            p["sol"].setVal(0.0)
        st = ag.solve_batched(ms, [p["sol"] for p in ps], [p["rhs"] for p in ps], 1e-10, 0.0)
        assert st == [0, 0]
        its = [m.getNumIters() for m in ms]
        if rep == 0:
            first = [p["sol"].get_global((p["n"],) * 3) for p in ps]
            its0 = its
    assert its == its0
    for p, f in zip(ps, first):
        assert np.array_equal(p["sol"].get_global((p["n"],) * 3), f)
