"""The CPU oracle (oracle/mlmg_oracle.c) against the golden fixtures made by
the reference AMReX CPU MLMG itself (tests/golden/make_golden.py)."""
import numpy as np
import pytest

from oracle import oracle
from tests.golden import cases, load


@pytest.mark.parametrize("name", load.names("hier_"))
def test_hierarchy_matches_reference(name):
    g = load.load(name)
    assert oracle.hierarchy(g["case"]) == g["hier"]


@pytest.mark.parametrize("name", load.names("hier_"))
def test_python_max_size_matches_reference(name):
    g = load.load(name)
    c = g["case"]
    if "boxes" in c:
        pytest.skip("explicit boxes")
    assert cases.max_size_boxes(c["n"], c["max_grid_size"]) == \
        [((b[0], b[1], b[2]), (b[3], b[4], b[5])) for b in g["hier"][0]]
    assert oracle.max_size(c["n"], c["max_grid_size"]) == g["hier"][0]


@pytest.mark.parametrize("name", load.names("fb_"))
def test_fill_boundary_bit_exact(name):
    g = load.load(name)
    out = oracle.fill_boundary(g["case"], g["fb_in"], g["case"]["cross"])
    assert np.array_equal(out, g["fb_out"])


@pytest.mark.parametrize("name", load.names("apply_"))
def test_apply_matches_reference(name):
    g = load.load(name)
    c = g["case"]
    out = oracle.apply(c, cases.inputs(c))
    ref = g["out"].reshape(out.shape)
    scale = np.abs(ref).max()
    np.testing.assert_allclose(out, ref, rtol=0, atol=1e-13 * scale)


@pytest.mark.parametrize("name", load.names("solve_"))
def test_solve_matches_reference(name):
    g = load.load(name)
    c = g["case"]
    phi, info = oracle.solve(c, cases.inputs(c))
    ref = g["phi"].reshape(phi.shape)
    r = g["result"]
    assert info["status"] == 0
    assert info["niters"] == r["niters"]
    assert info["cg_iters"] == r["cg_iters"]
    # near the rounding floor the residuals move with the summation order of
    # the reference's OpenMP reductions (solvability offsets, bottom dots)
    np.testing.assert_allclose(info["history"], r["history"], rtol=1e-6,
                               atol=1e-13 * max(r["rhs_norm"], r["init_resid"]))
    # phi agrees to 1e-10 relative (max norm)
    assert np.abs(phi - ref).max() <= 1e-10 * np.abs(ref).max()


@pytest.mark.parametrize("name", load.names("flux_"))
def test_oracle_fluxes_match_reference(name):
    """getFluxes / getGradSolution of the reference's own solution: the
    oracle's restatement reproduces the reference bit for bit."""
    g = load.load(name)
    c = g["case"]
    nx, ny, nz = c["n"]
    arr = cases.inputs(c)
    sol = arr["sol"].copy()
    sol[1:-1, 1:-1, 1:-1] = g["phi"].reshape(nz, ny, nx)
    arr["sol"] = sol
    shapes = [(nz, ny, nx + 1), (nz, ny + 1, nx), (nz + 1, ny, nx)]
    for mode, keys in (("flux", ("fx", "fy", "fz")), ("grad", ("gx", "gy", "gz"))):
        out = oracle.fluxes(c, arr, mode)
        for d, k in enumerate(keys):
            ref = g[k].reshape(shapes[d])
            assert np.array_equal(out[d], ref), (mode, d, np.abs(out[d] - ref).max())


@pytest.mark.parametrize("name", ["large_c4_48", "large_c4_80", "large_c4_112", "large_c4_128"])
def test_solve_matches_reference_batch_shapes(name):
    """The batch solves with ragged max-grid-size-32 boxes (48 -> 32+16,
    80 -> 32+32+16, 112 -> 32+32+32+16) at full size: the reference's
    iteration and bottom counts, its history, and its phi samples and
    statistics."""
    g = load.load(name)
    c, r = g["case"], g["result"]
    phi, info = oracle.solve(c, cases.inputs(c))
    assert info["status"] == 0
    assert info["niters"] == r["niters"]
    assert info["cg_iters"] == r["cg_iters"]
    np.testing.assert_allclose(info["history"], r["history"], rtol=1e-6,
                               atol=1e-13 * max(r["rhs_norm"], r["init_resid"]))
    flat = phi.ravel()
    mx = float(g["phi_stats"][0])
    assert np.abs(flat[cases.large_sample_index(flat.size)] - g["phi_sample"]).max() <= 1e-10 * mx
    assert abs(np.abs(flat).max() - mx) <= 1e-10 * mx


@pytest.mark.parametrize("name", load.names("resid_"))
def test_comp_residual_matches_reference(name):
    """MLMG::compResidual on one level is rhs - L(sol) with the level's
    inhomogeneous boundary values: the oracle's apply gives the reference's
    residual."""
    g = load.load(name)
    c = g["case"]
    inp = cases.inputs(c)
    out = oracle.apply(c, inp)
    ref = g["res"].reshape(out.shape)
    np.testing.assert_allclose(inp["rhs"] - out, ref, rtol=0, atol=1e-13 * np.abs(ref).max())
