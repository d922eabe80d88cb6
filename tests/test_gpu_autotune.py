"""mlmg_autotune: every candidate layout runs, the chosen one is kept and the
solve afterwards still meets the reference's answer.  Needs a CUDA GPU."""
import numpy as np
import pytest

from tests import helpers
from tests.golden import cases, load

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", ["solve_abec_48", "solve_poisson_c0"])
def test_autotune_then_solve(name):
    g = load.load(name)
    c = g["case"]
    prob = helpers.make_problem(c, cases.inputs(c), precision="mixed", graph=True)
    before = prob["sol"].get_global((c["n"][2] + 2, c["n"][1] + 2, c["n"][0] + 2), lo=(-1, -1, -1))
    ms, report = prob["mlmg"].autotune(prob["sol"], prob["rhs"], vcycles=2)
    after = prob["sol"].get_global((c["n"][2] + 2, c["n"][1] + 2, c["n"][0] + 2), lo=(-1, -1, -1))
    assert np.array_equal(before, after)            # the initial guess is not touched
    lines = [ln for ln in report.splitlines() if ln.strip()]
    assert len(lines) == 9 and lines[-1].startswith("chosen: ")
    assert ms > 0
    resid = prob["mlmg"].solve(prob["sol"], prob["rhs"], c["tol_rel"], c["tol_abs"])
    r = g["result"]
    assert resid <= c["tol_rel"] * max(r["rhs_norm"], r["init_resid"])
    phi = helpers.solution(prob, c)
    ref = g["phi"].reshape(phi.shape)
    assert np.abs(phi - ref).max() <= 1e-8 * np.abs(ref).max()
