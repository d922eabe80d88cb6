"""AMR composite-solve cases: a base level of n^3 cells, refinement ratio 2,
levels tagged where |RHS| exceeds the 90th (or ``tag_pct``-th) percentile of
|RHS| on that level (RHS: the seeded sum of 16 Gaussian blobs sampled at each
level's cell centres), homogeneous Dirichlet on the domain (or, with ``bc``,
seeded Dirichlet values and initial guess; ``periodic`` makes directions
periodic), MLPoisson (or, with ``abec``, MLABecLaplacian).  Grids come from
the reference's AmrMesh (tests/golden/make_amr_golden.py)."""
from __future__ import annotations

import ast
import os

import numpy as np

from amrex_gb300 import synth

HERE = os.path.dirname(os.path.abspath(__file__))

CASES = {
    # the 3-level composite configuration: base 128^3, max_grid_size 64
    # (solution kept as per-level statistics and samples)
    "c2": dict(n=128, nlev=3, max_grid_size=64, rhs_seed=1002, solve="summary"),
    # small composite solves for parity
    "c2_n32": dict(n=32, nlev=3, max_grid_size=16, rhs_seed=1002),
    "c2_n16_2lev": dict(n=16, nlev=2, max_grid_size=8, rhs_seed=1012),
    # inhomogeneous Dirichlet values on every level and a non-zero initial guess
    "c2_n16_2lev_bc": dict(n=16, nlev=2, max_grid_size=8, rhs_seed=1012, bc=True),
    # F-cycles on AMR level 0 for the first two iterations
    "c2_n32_fmg": dict(n=32, nlev=3, max_grid_size=16, rhs_seed=1002, max_fmg_iter=2, solve="summary"),
    # MLABecLaplacian with per-level a and face b (level_abec): coefficients
    # averaged down across AMR levels, fluxes beta b grad(phi) in the reflux
    "c2_n16_2lev_abec": dict(n=16, nlev=2, max_grid_size=8, rhs_seed=1012, abec=(0.75, 1.25)),
    "c2_n32_abec": dict(n=32, nlev=3, max_grid_size=16, rhs_seed=1002, abec=(0.75, 1.25), bc=True,
                        solve="summary"),
    # periodic in x and y (Dirichlet in z): coarse/fine boundaries, reflux and
    # interpolation across the periodic faces
    "c2_n16_2lev_per": dict(n=16, nlev=2, max_grid_size=8, rhs_seed=1013, periodic=(1, 1, 0), tag_pct=98),
    "c2_n32_per": dict(n=32, nlev=3, max_grid_size=16, rhs_seed=1004, periodic=(1, 1, 0), tag_pct=97,
                       solve="summary"),
    "c2_n16_2lev_per_abec": dict(n=16, nlev=2, max_grid_size=8, rhs_seed=1013, periodic=(1, 1, 0), tag_pct=98,
                                 abec=(0.75, 1.25)),
    # four levels: two intermediate levels with their correction holds
    "c2_n16_4lev": dict(n=16, nlev=4, max_grid_size=16, rhs_seed=1002, tag_pct=95, solve="summary"),
    # MLMG::compResidual of a non-zero initial guess with inhomogeneous
    # Dirichlet values (no solve)
    "c2_n16_2lev_resid": dict(n=16, nlev=2, max_grid_size=8, rhs_seed=1012, bc=True, solve=False, resid=True),
    "c2_n32_resid": dict(n=32, nlev=3, max_grid_size=16, rhs_seed=1002, bc=True, solve=False, resid=True),
    "c2_n16_2lev_abec_resid": dict(n=16, nlev=2, max_grid_size=8, rhs_seed=1012, abec=(0.75, 1.25), bc=True,
                                   solve=False, resid=True),
    "c2_n16_2lev_per_resid": dict(n=16, nlev=2, max_grid_size=8, rhs_seed=1013, periodic=(1, 1, 0), tag_pct=98,
                                  bc=True, solve=False, resid=True),
}


def level_rhs(case, lev):
    """RHS on the whole domain of level lev, shape (m, m, m), m = n 2^lev."""
    return synth.gaussian_rhs(case["n"] << lev, case["rhs_seed"])


def sample_index(size, lev, count=4096):
    """seeded sample of positions into a level's box-packed phi"""
    rng = np.random.Generator(np.random.PCG64(7000 + lev))
    return np.sort(rng.choice(size, size=min(count, size), replace=False))


def level_solbc(case, lev):
    """Grown level-domain array (m+2)^3 of a case with ``bc``: the initial
    guess in the valid cells, the Dirichlet boundary values in the ghost
    cells, both from smooth functions of the cell centres; None otherwise."""
    if not case.get("bc"):
        return None
    m = case["n"] << lev
    c = (np.arange(-1, m + 1) + 0.5) / m
    z, y, x = np.meshgrid(c, c, c, indexing="ij")
    bc = np.sin(3.0 * x) + 0.5 * np.cos(2.0 * y) + z * z
    out = 0.01 * np.cos(x + y - z)
    ghost = np.ones(out.shape, dtype=bool)
    ghost[1:-1, 1:-1, 1:-1] = False
    out[ghost] = bc[ghost]
    return out


def level_abec(case, lev):
    """(alpha, beta, a, bx, by, bz) of a case with ``abec``: a at the cell
    centres, (m, m, m); b_d at the face centres normal to d, m+1 faces along
    d (arrays indexed z, y, x) -- smooth positive functions of position with
    an order-one variation, so that the coarse and fine samplings differ;
    None otherwise."""
    if not case.get("abec"):
        return None
    alpha, beta = case["abec"]
    m = case["n"] << lev
    cc = (np.arange(m) + 0.5) / m
    fc = np.arange(m + 1) / m
    z, y, x = np.meshgrid(cc, cc, cc, indexing="ij")
    a = 1.0 + 0.5 * np.sin(5.0 * x + 1.0) * np.cos(3.0 * y) + 0.25 * z

    def b(x, y, z):
        return 1.0 + 0.6 * np.cos(4.0 * x - 1.0) * np.sin(3.0 * y + z) + 0.3 * x * z

    if case.get("periodic"):
        # periodic along the periodic directions, so that the two stored
        # copies of a face on a periodic boundary hold the same b
        tp = 2.0 * np.pi
        a = 1.0 + 0.5 * np.sin(tp * x + 1.0) * np.cos(tp * y) + 0.25 * z

        def b(x, y, z):
            return 1.0 + 0.6 * np.cos(tp * x - 1.0) * np.sin(tp * y + z) + 0.3 * z * np.cos(tp * x)

    bx = b(*np.meshgrid(cc, cc, fc, indexing="ij")[::-1])
    by = b(*np.meshgrid(cc, fc, cc, indexing="ij")[::-1])
    bz = b(*np.meshgrid(fc, cc, cc, indexing="ij")[::-1])
    return alpha, beta, a, bx, by, bz


def check_history(got, ref, rtol_early=1e-6):
    """Residual history against the reference's: entries above 1e-7 of the
    residual scale (max of |rhs| and the initial residual) to ``rtol_early``
    -- they carry the convergence path, which is where the coefficient
    average-down across AMR levels shows (the converged phi hardly depends on
    it) -- and the rest, near roundoff, to 1e-4."""
    got = np.asarray(got, dtype=float)
    want = np.asarray(ref["history"], dtype=float)
    assert got.shape == want.shape, (got.shape, want.shape)
    scale = max(ref["rhs_norm"], ref["init_resid"])
    early = want >= 1e-7 * scale
    np.testing.assert_allclose(got[early], want[early], rtol=rtol_early, atol=0)
    np.testing.assert_allclose(got, want, rtol=1e-4, atol=1e-14 * ref["rhs_norm"])


def parse_grids(text):
    levels = []
    for line in text.strip().splitlines():
        p = line.split()
        if p[0] == "level":
            levels.append([])
        else:
            levels[-1].append(tuple(int(v) for v in p))
    return levels


def pack_boxes(arr, boxes):
    """values of a whole-domain array (z, y, x) on the cells of `boxes`, box by
    box, x fastest"""
    out = []
    for b in boxes:
        out.append(arr[b[2]:b[5] + 1, b[1]:b[4] + 1, b[0]:b[3] + 1].ravel())
    return np.concatenate(out)


def unpack_boxes(flat, boxes, m):
    arr = np.zeros((m, m, m))
    q = 0
    for b in boxes:
        shp = (b[5] - b[2] + 1, b[4] - b[1] + 1, b[3] - b[0] + 1)
        sz = shp[0] * shp[1] * shp[2]
        arr[b[2]:b[5] + 1, b[1]:b[4] + 1, b[0]:b[3] + 1] = flat[q:q + sz].reshape(shp)
        q += sz
    return arr


def load(kind, name):
    z = np.load(os.path.join(HERE, f"{kind}_{name}.npz"))
    out = {k: z[k] for k in z.files}
    out["case"] = ast.literal_eval(str(out["case"]))
    out["grids"] = parse_grids(str(out["grids"]))
    if "result" in out:
        from tests.golden.load import parse_result
        out["result"] = parse_result(str(out["result"]))
    return out
