"""MLMG::getFluxes / getGradSolution through the C ABI against the
reference's outputs (golden fixtures made by the reference itself).  Needs a
CUDA GPU (GB300)."""
import numpy as np
import pytest

from tests import helpers
from tests.golden import cases, load

pytestmark = pytest.mark.gpu

import amrex_gb300 as ag  # noqa: E402


def _shapes(c):
    nx, ny, nz = c["n"]
    return [(nz, ny, nx + 1), (nz, ny + 1, nx), (nz + 1, ny, nx)]


def _faces(prob):
    return [ag.MultiFab(prob["ba"], prob["dm"], 1, 0, nodal_dir=d) for d in range(3)]


@pytest.mark.parametrize("name", load.names("flux_"))
def test_fluxes_of_reference_solution(name):
    """Fluxes and gradients of the reference's own solution: the same
    arithmetic as the reference up to the rounding of the boundary closure."""
    g = load.load(name)
    c = g["case"]
    nx, ny, nz = c["n"]
    arr = cases.inputs(c)
    prob = helpers.make_problem(c, arr, precision="fp64")
    grown = arr["sol"].copy()
    grown[1:-1, 1:-1, 1:-1] = g["phi"].reshape(nz, ny, nx)
    prob["sol"].set_global(grown, lo=(-1, -1, -1))
    flux, grad = _faces(prob), _faces(prob)
    prob["mlmg"].getFluxes(flux, prob["sol"])
    prob["mlmg"].getGradSolution(grad, prob["sol"])
    for d, s in enumerate(_shapes(c)):
        for mf, k in ((flux[d], "f" + "xyz"[d]), (grad[d], "g" + "xyz"[d])):
            ref = g[k].reshape(s)
            got = mf.get_global(s)
            np.testing.assert_allclose(got, ref, rtol=0, atol=1e-13 * np.abs(ref).max(), err_msg=k)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("name", load.names("flux_"))
def test_fluxes_after_solve(name, precision):
    """Solve, then fluxes and gradients of the GPU solution, against the
    reference's (the solutions agree to the solve tolerance)."""
    g = load.load(name)
    c = g["case"]
    prob = helpers.make_problem(c, cases.inputs(c), precision=precision)
    prob["mlmg"].solve(prob["sol"], prob["rhs"], c["tol_rel"], c["tol_abs"])
    flux, grad = _faces(prob), _faces(prob)
    prob["mlmg"].getFluxes(flux, prob["sol"])
    prob["mlmg"].getGradSolution(grad, prob["sol"])
    for d, s in enumerate(_shapes(c)):
        for mf, k in ((flux[d], "f" + "xyz"[d]), (grad[d], "g" + "xyz"[d])):
            ref = g[k].reshape(s)
            np.testing.assert_allclose(mf.get_global(s), ref, rtol=0, atol=1e-8 * np.abs(ref).max(), err_msg=k)


def test_fluxes_reject_wrong_layout():
    g = load.load("flux_abec_32")
    c = g["case"]
    prob = helpers.make_problem(c, cases.inputs(c), precision="fp64")
    bad = [ag.MultiFab(prob["ba"], prob["dm"], 1, 0, nodal_dir=(d + 1) % 3) for d in range(3)]
    with pytest.raises(ag.MLMGError):
        prob["mlmg"].getFluxes(bad, prob["sol"])
