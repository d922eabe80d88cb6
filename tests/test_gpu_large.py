"""Full-size parity through the C ABI: the 256^3 variable-coefficient
MLABecLaplacian benchmark (max grid size 64) and four solves of the 64-solve
batch (128^3, 112^3, 80^3 and 48^3, max grid size 32, ragged boxes) against
the reference's own CPU solves of the same seeded inputs
(``tests/golden/large_*.npz``, made by ``make_large_golden.py``): iteration
and per-iteration bottom BiCGStab counts, residual history, and phi through
max|phi|, sum(phi), sum(phi^2) and 4096 seeded samples.  Needs a GPU."""
import numpy as np
import pytest

import amrex_gb300 as ag
from tests import helpers
from tests.golden import cases, load

pytestmark = pytest.mark.gpu

LARGE = list(cases.LARGE_CASES)
BATCH = [n for n in LARGE if n.startswith("large_c4_")]


def check_phi(phi, g, tol):
    """phi (whole domain, x fastest) against the fixture's statistics and
    samples, to ``tol`` of max|phi|"""
    flat = phi.ravel()
    mx, s1, s2 = (float(v) for v in g["phi_stats"])
    idx = cases.large_sample_index(flat.size)
    assert np.abs(flat[idx] - g["phi_sample"]).max() <= tol * mx
    assert abs(np.abs(flat).max() - mx) <= tol * mx
    assert abs(flat.sum() - s1) <= tol * mx * flat.size
    assert abs((flat * flat).sum() - s2) <= 2.0 * tol * mx * mx * flat.size


@pytest.mark.parametrize("name", LARGE)
def test_large_fp64_matches_reference(name):
    """FP64: the reference's iteration and bottom counts, its residual
    history, and phi to 1e-10 of max|phi|."""
    g = load.load(name)
    c, r = g["case"], g["result"]
    prob = helpers.make_problem(c, cases.inputs(c), precision="fp64")
    prob["mlmg"].solve(prob["sol"], prob["rhs"], c["tol_rel"], c["tol_abs"])
    assert prob["mlmg"].getNumIters() == r["niters"]
    assert prob["mlmg"].getNumCGIters() == r["cg_iters"]
    np.testing.assert_allclose(prob["mlmg"].getResidualHistory(), r["history"], rtol=1e-6,
                               atol=1e-13 * max(r["rhs_norm"], r["init_resid"]))
    check_phi(helpers.solution(prob, c), g, 1e-10)


@pytest.mark.parametrize("name", LARGE)
def test_large_mixed_reaches_reference_target(name):
    """Mixed precision (FP32 fused-sweep V-cycles in FP64 refinement, CUDA
    graph): the reference's 1e-10 relative residual target, at most two more
    iterations, phi to 1e-8 of max|phi|."""
    g = load.load(name)
    c, r = g["case"], g["result"]
    prob = helpers.make_problem(c, cases.inputs(c), precision="mixed", graph=True, fused=True)
    resid = prob["mlmg"].solve(prob["sol"], prob["rhs"], c["tol_rel"], c["tol_abs"])
    assert resid <= c["tol_rel"] * max(r["rhs_norm"], r["init_resid"])
    assert prob["mlmg"].getNumIters() <= r["niters"] + 2
    check_phi(helpers.solution(prob, c), g, 1e-8)


def test_large_batch_matches_reference():
    """The four batch solves in one batched mixed-precision call: every solve
    reaches its reference target and matches the reference's phi."""
    gs = [load.load(n) for n in BATCH]
    probs = [helpers.make_problem(g["case"], cases.inputs(g["case"]), precision="mixed", graph=True, fused=True)
             for g in gs]
    st = ag.solve_batched([p["mlmg"] for p in probs], [p["sol"] for p in probs], [p["rhs"] for p in probs],
                          1e-10, 0.0)
    assert all(v == 0 for v in st), st
    for g, p in zip(gs, probs):
        r = g["result"]
        assert p["mlmg"].getFinalResidual() <= 1e-10 * max(r["rhs_norm"], r["init_resid"])
        assert p["mlmg"].getNumIters() <= r["niters"] + 2
        check_phi(helpers.solution(p, g["case"]), g, 1e-8)
