"""GPU library vs the reference's golden fixtures and the CPU oracle, through
the C ABI.  Needs a CUDA GPU (GB300)."""
import numpy as np
import pytest

import amrex_gb300 as ag
from oracle import oracle
from tests import helpers
from tests.golden import cases, load

pytestmark = pytest.mark.gpu


def _fb_boxes(c):
    if c.get("boxes"):
        return [((b[0], b[1], b[2]), (b[3], b[4], b[5])) for b in c["boxes"]]
    return cases.max_size_boxes(c["n"], c["max_grid_size"])


@pytest.mark.parametrize("name", load.names("fb_"))
def test_fill_boundary_bit_exact(name):
    g = load.load(name)
    c = g["case"]
    nx, ny, nz = c["n"]
    domain = ag.Box((0, 0, 0), (nx - 1, ny - 1, nz - 1))
    ba = ag.BoxArray(domain).maxSize(c["max_grid_size"])
    dm = ag.DistributionMapping(ba)
    geom = ag.Geometry(domain, is_periodic=c["periodic"])
    mf = ag.MultiFab(ba, dm, 1, 1)
    off = 0
    shapes = []
    for b in range(ba.size()):
        shp = mf.fab_shape(b)
        n = int(np.prod(shp))
        mf.set_fab(b, g["fb_in"][off:off + n].reshape(shp))
        shapes.append((off, n, shp))
        off += n
    mf.FillBoundary(geom, cross=bool(c["cross"]))
    out = np.concatenate([mf.get_fab(b).ravel() for b in range(ba.size())])
    assert np.array_equal(out, g["fb_out"])


@pytest.mark.parametrize("name", load.names("apply_"))
def test_apply_matches_reference(name):
    g = load.load(name)
    c = g["case"]
    prob = helpers.make_problem(c, cases.inputs(c))
    nx, ny, nz = c["n"]
    out = ag.MultiFab(prob["ba"], prob["dm"], 1, 0)
    prob["mlmg"].apply(out, prob["sol"])
    got = out.get_global((nz, ny, nx))
    ref = g["out"].reshape(got.shape)
    np.testing.assert_allclose(got, ref, rtol=0, atol=1e-13 * np.abs(ref).max())


@pytest.mark.parametrize("name", load.names("solve_"))
def test_fp64_solve_matches_reference(name):
    """FP64 solves agree with the reference to 1e-10 relative in phi, with the
    same V-cycle and bottom iteration counts."""
    g = load.load(name)
    c = g["case"]
    prob = helpers.make_problem(c, cases.inputs(c), precision="fp64")
    prob["mlmg"].solve(prob["sol"], prob["rhs"], c["tol_rel"], c["tol_abs"])
    phi = helpers.solution(prob, c)
    ref = g["phi"].reshape(phi.shape)
    r = g["result"]
    assert prob["mlmg"].getNumIters() == r["niters"]
    assert prob["mlmg"].getNumCGIters() == r["cg_iters"]
    # the last residuals sit near the rounding floor; FMA contraction on the
    # GPU moves them by ~1e-15 of the initial norm
    np.testing.assert_allclose(prob["mlmg"].getResidualHistory(), r["history"], rtol=1e-6,
                               atol=1e-13 * max(r["rhs_norm"], r["init_resid"]))
    assert np.abs(phi - ref).max() <= 1e-10 * np.abs(ref).max()


MIXED_CASES = ["solve_poisson_32", "solve_abec_32", "solve_abec_48", "solve_abec_mixed_bc", "solve_abec_agg8",
               "solve_poisson_c0", "solve_poisson_periodic", "solve_abec_neumann_singular", "solve_abec_mo4",
               "solve_poisson_periodic_x", "solve_abec_32_fmg", "solve_abec_mixed_bc_fmg",
               "solve_poisson_periodic_x_fmg", "solve_poisson_c0_fmg", "solve_abec_cg", "solve_abec_cgbicg",
               "solve_abec_bicgcg"]


@pytest.mark.parametrize("name", MIXED_CASES)
@pytest.mark.parametrize("graph,fused,coarse,march", [(False, False, 1, 0), (True, False, 1, 0), (True, True, 1, 0),
                                                      (False, False, 0, 0), (True, True, 0, 0), (True, True, 0, 1)])
def test_mixed_solve_reaches_target(name, graph, fused, coarse, march):
    """FP32 V-cycles inside FP64 refinement reach the same 1e-10 relative
    residual (the residual is evaluated in FP64); phi agrees with the
    reference's FP64 answer to the accuracy that residual implies (up to the
    constant null-space component for singular problems)."""
    g = load.load(name)
    c = g["case"]
    opts = {"coarse_block": coarse}
    if march:
        # the z-marching sweep on every fused level
        opts.update(march_sweep=1, march_min_tiles=0)
    prob = helpers.make_problem(c, cases.inputs(c), precision="mixed", graph=graph, fused=fused, options=opts)
    resid = prob["mlmg"].solve(prob["sol"], prob["rhs"], c["tol_rel"], c["tol_abs"])
    r = g["result"]
    target = c["tol_rel"] * max(r["rhs_norm"], r["init_resid"])
    assert resid <= target
    assert prob["mlmg"].getNumIters() <= r["niters"] + 2
    phi = helpers.solution(prob, c)
    ref = g["phi"].reshape(phi.shape)
    if "periodic" in name and c["periodic"] == (1, 1, 1) or "singular" in name:
        phi, ref = phi - phi.mean(), ref - ref.mean()
    assert np.abs(phi - ref).max() <= 1e-8 * np.abs(ref).max()


@pytest.mark.parametrize("name", ["solve_abec_32", "solve_poisson_32", "solve_abec_mixed_bc", "solve_abec_48",
                                  "solve_poisson_periodic_x", "solve_abec_mo4"])
@pytest.mark.parametrize("variant", ["tiled", "tiled_noprefetch", "tiled_cpasync", "march"])
def test_fused_sweep_matches_colour_passes(name, variant):
    """The fused two-colour sweep (tiled, staged by TMA with or without the
    L2 prefetch of its coefficient boxes, or by cp.async; or marching along z
    with its planes staged by TMA) performs the same arithmetic as two colour
    passes with ghost refreshes in between."""
    c = load.load(name)["case"]
    inp = cases.inputs(c)
    march = variant.startswith("march")
    opts = {"march_sweep": int(march), "march_min_tiles": 0, "fused_tma": int(variant != "tiled_cpasync"),
            "fused_prefetch": int(variant != "tiled_noprefetch")}
    p1 = helpers.make_problem(c, inp, precision="mixed", fused=False)
    p2 = helpers.make_problem(c, inp, precision="mixed", fused=True, options=opts)
    p1["mlmg"].solve(p1["sol"], p1["rhs"], 1e-10, 0)
    p2["mlmg"].solve(p2["sol"], p2["rhs"], 1e-10, 0)
    assert p1["mlmg"].getNumIters() == p2["mlmg"].getNumIters()
    h1, h2 = np.array(p1["mlmg"].getResidualHistory()), np.array(p2["mlmg"].getResidualHistory())
    np.testing.assert_allclose(h2, h1, rtol=1e-5, atol=1e-13 * h1[0])
    a, b = helpers.solution(p1, c), helpers.solution(p2, c)
    assert np.abs(a - b).max() <= 1e-12 * np.abs(a).max()


def _one_sweep(c, inp, fused, opts=None):
    """phi after a single pre-smoothing sweep on the finest level: one MG
    level below it, one iteration, no post-smoothing, and a bottom
    'smoother' of zero sweeps (its correction stays 0)"""
    cc = dict(c, max_coarsening_level=1)
    p = helpers.make_problem(cc, inp, precision="mixed", fused=fused, options=opts)
    m = p["mlmg"]
    m.setFixedIter(1)
    m.setPreSmooth(1)
    m.setPostSmooth(0)
    m.setBottomSolver(1)
    m.setFinalSmooth(0)
    m.solve(p["sol"], p["rhs"], 1e-10, 0)
    return helpers.solution(p, cc)


@pytest.mark.parametrize("name", ["solve_abec_32", "solve_poisson_32", "solve_abec_mixed_bc", "solve_abec_48"])
@pytest.mark.parametrize("opts", [{}, {"fused_prefetch": 0}, {"fused_tma": 0}, {"march_sweep": 1, "march_min_tiles": 0}])
def test_fused_single_sweep_matches_colour_passes(name, opts):
    """One fused two-colour sweep on the finest level, isolated (one
    iteration, one pre-smoothing sweep, no post-smoothing, a bottom of zero
    sweeps), gives the two colour passes' values bit for bit."""
    c = load.load(name)["case"]
    inp = cases.inputs(c)
    assert np.array_equal(_one_sweep(c, inp, True, opts), _one_sweep(c, inp, False))


@pytest.mark.parametrize("name", ["solve_abec_32", "solve_abec_48", "solve_abec_mixed_bc", "solve_poisson_periodic_x"])
def test_fused_sweep_staging_bitwise(name):
    """Staging a tile by one TMA tensor load or by cp.async copies, with or
    without the L2 prefetch, changes no arithmetic: the solution is bit for
    bit the same."""
    c = load.load(name)["case"]
    inp = cases.inputs(c)
    p1 = helpers.make_problem(c, inp, precision="mixed", fused=True, options={"fused_tma": 0})
    p1["mlmg"].solve(p1["sol"], p1["rhs"], 1e-10, 0)
    for opts in ({"fused_tma": 1, "fused_prefetch": 0}, {"fused_tma": 1, "fused_prefetch": 1}):
        p2 = helpers.make_problem(c, inp, precision="mixed", fused=True, options=opts)
        p2["mlmg"].solve(p2["sol"], p2["rhs"], 1e-10, 0)
        assert p1["mlmg"].getNumIters() == p2["mlmg"].getNumIters()
        assert np.array_equal(helpers.solution(p1, c), helpers.solution(p2, c))


@pytest.mark.parametrize("name", ["solve_abec_32", "solve_poisson_32", "solve_abec_48", "solve_abec_mixed_bc",
                                  "solve_abec_agg8", "solve_poisson_periodic", "solve_poisson_periodic_x",
                                  "solve_abec_mo4"])
@pytest.mark.parametrize("merge", [1, 0])
def test_fused_residual_restriction_bitwise(name, merge):
    """The correction residual and its restriction computed in one TMA tile
    kernel (the fine residual kept in shared memory) give the separate
    residual and restriction launches' coarse right-hand sides bit for bit:
    the same iterations and the same solution, with merged or unmerged
    patches."""
    c = load.load(name)["case"]
    inp = cases.inputs(c)
    sols = []
    for fr in (0, 1):
        p = helpers.make_problem(c, inp, precision="mixed", fused=True,
                                 options={"fused_restrict": fr, "merge_boxes": merge})
        p["mlmg"].solve(p["sol"], p["rhs"], 1e-10, 0)
        sols.append((p["mlmg"].getNumIters(), list(p["mlmg"].getResidualHistory()), helpers.solution(p, c)))
    assert sols[0][0] == sols[1][0]
    assert sols[0][1] == sols[1][1]
    assert np.array_equal(sols[0][2], sols[1][2])


@pytest.mark.parametrize("name", ["solve_abec_32", "solve_poisson_32", "solve_abec_48", "solve_abec_mixed_bc",
                                  "solve_abec_agg8", "solve_poisson_periodic"])
@pytest.mark.parametrize("cells", [512, 32768])
def test_coarse_block_vcycle_matches_grid_kernels(name, cells):
    """Running the coarse levels inside one block per solve performs the same
    FP32 stage arithmetic as the grid-wide kernels: the same iteration count
    and residual history up to FP32 summation order."""
    c = load.load(name)["case"]
    inp = cases.inputs(c)
    p1 = helpers.make_problem(c, inp, precision="mixed", options={"coarse_block": 0})
    p2 = helpers.make_problem(c, inp, precision="mixed", options={"coarse_block": 1, "coarse_cells": cells})
    p1["mlmg"].solve(p1["sol"], p1["rhs"], 1e-10, 0)
    p2["mlmg"].solve(p2["sol"], p2["rhs"], 1e-10, 0)
    assert abs(p1["mlmg"].getNumIters() - p2["mlmg"].getNumIters()) <= 1
    h1, h2 = np.array(p1["mlmg"].getResidualHistory()), np.array(p2["mlmg"].getResidualHistory())
    n = min(len(h1), len(h2), 4)
    np.testing.assert_allclose(h2[:n], h1[:n], rtol=1e-3, atol=1e-12 * h1[0])
    a, b = helpers.solution(p1, c), helpers.solution(p2, c)
    assert np.abs(a - b).max() <= 1e-8 * np.abs(a).max()


def test_bit_assembled_conversions_match_hardware():
    """The FP32 <-> FP64 conversions and |x| that the FP64-bound kernels
    assemble on the integer pipe equal the hardware's on 2^26 device cases
    (edge values, random patterns, halfway points, subnormals)."""
    for n, seed in ((1 << 26, 2024), (1 << 20, 7)):
        bad, first = ag.check_bit_conversions(n, seed=seed)
        assert sum(bad.values()) == 0, (bad, first)


def test_global_transfers_from_pinned_host_memory():
    """Whole-array transfers from and to page-locked host memory (read and
    written by the scatter / gather kernel directly) give what the staged
    transfers of ordinary host memory give, and a download leaves the
    array's cells that no FAB's valid box covers untouched."""
    torch = pytest.importorskip("torch")
    n = 40
    ba = ag.BoxArray(ag.Box((0, 0, 0), (n - 1, n - 1, n - 1))).maxSize(16)
    dm = ag.DistributionMapping(ba)
    rng = np.random.default_rng(11)
    src = rng.standard_normal((n + 2, n + 2, n + 2))
    mf_a, mf_b = ag.MultiFab(ba, dm, 1, 1), ag.MultiFab(ba, dm, 1, 1)
    mf_a.set_global(src, lo=(-1, -1, -1))
    pin = torch.empty((n + 2, n + 2, n + 2), dtype=torch.float64, pin_memory=True).numpy()
    pin[...] = src
    mf_b.set_global(pin, lo=(-1, -1, -1))
    got_a = mf_a.get_global((n + 4, n + 4, n + 4), lo=(-2, -2, -2))
    out = torch.full((n + 4, n + 4, n + 4), 7.0, dtype=torch.float64, pin_memory=True).numpy()
    mf_b.get_global((n + 4, n + 4, n + 4), lo=(-2, -2, -2), out=out)
    # valid cells 0..n-1 sit at [2:-2]; the two outer layers are no FAB's valid cells
    assert np.array_equal(got_a[2:-2, 2:-2, 2:-2], out[2:-2, 2:-2, 2:-2])
    assert np.array_equal(got_a[2:-2, 2:-2, 2:-2], src[1:-1, 1:-1, 1:-1])
    assert np.all(out[:2] == 7.0) and np.all(out[:, :, -2:] == 7.0)


def test_graph_replay_is_bitwise_identical():
    c = load.load("solve_abec_32")["case"]
    inp = cases.inputs(c)
    p1 = helpers.make_problem(c, inp, precision="fp64", graph=False)
    p2 = helpers.make_problem(c, inp, precision="fp64", graph=True)
    p1["mlmg"].solve(p1["sol"], p1["rhs"], 1e-10, 0)
    p2["mlmg"].solve(p2["sol"], p2["rhs"], 1e-10, 0)
    assert np.array_equal(helpers.solution(p1, c), helpers.solution(p2, c))


@pytest.mark.parametrize("name", ["solve_abec_32", "solve_poisson_32", "solve_abec_mixed_bc", "solve_abec_agg8",
                                  "solve_poisson_periodic_x"])
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_dependent_launches_bitwise(name, precision):
    """Programmatic dependent launches change only when kernels start: the
    graph solves with and without them are bit for bit the same."""
    c = load.load(name)["case"]
    inp = cases.inputs(c)
    out = []
    for pdl in (1, 0):
        p = helpers.make_problem(c, inp, precision=precision, graph=True, fused=precision == "mixed",
                                 options={"pdl": pdl})
        p["mlmg"].solve(p["sol"], p["rhs"], 1e-10, 0)
        out.append((p["mlmg"].getNumIters(), list(p["mlmg"].getResidualHistory()), helpers.solution(p, c)))
    assert out[0][0] == out[1][0] and out[0][1] == out[1][1]
    assert np.array_equal(out[0][2], out[1][2])


def test_oracle_and_gpu_agree_on_unpinned_shape():
    """A shape with no golden fixture (anisotropic, ragged boxes, Neumann and
    reflect_odd faces): the GPU FP64 solve against the CPU oracle."""
    c = cases._c(mode="solve", op="abec", n=(40, 24, 28), max_grid_size=16, rhs_seed=77, b_seed=78, a_seed=79,
                 alpha=0.7, beta=1.3, lobc=(101, 102, 103), hibc=(102, 101, 101), sol_seed=80)
    inp = cases.inputs(c)
    phi_o, info = oracle.solve(c, inp)
    prob = helpers.make_problem(c, inp, precision="fp64")
    prob["mlmg"].solve(prob["sol"], prob["rhs"], c["tol_rel"], c["tol_abs"])
    phi = helpers.solution(prob, c)
    assert prob["mlmg"].getNumIters() == info["niters"]
    assert np.abs(phi - phi_o).max() <= 1e-10 * np.abs(phi_o).max()
