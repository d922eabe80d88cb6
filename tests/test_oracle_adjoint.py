"""The adjoint's reference: exact derivatives of the oracle's discrete
operator (sparse direct solves, probing of the operator apply), checked by
central finite differences, and the closed-form face-gradient contraction the
library's kernel evaluates checked against them.  CPU only."""
import numpy as np
import pytest

from oracle import adjoint, oracle
from tests.golden import cases


def _small_cases():
    return {
        # Dirichlet everywhere, variable b
        "dirichlet": cases._c(mode="solve", op="abec", n=(12, 10, 8), max_grid_size=8, rhs_seed=1101, b_seed=2101,
                              b_sigma=2.0),
        # Neumann and Dirichlet faces, inhomogeneous Dirichlet values, variable a
        "mixed_bc": cases._c(mode="solve", op="abec", n=(12, 10, 8), max_grid_size=8, rhs_seed=1102, b_seed=2102,
                             a_seed=3102, sol_seed=3103, lobc=(101, 102, 101), hibc=(102, 101, 101), b_sigma=2.0),
        # periodic in x, maxorder 4 closures on the other faces
        "periodic_x_mo4": cases._c(mode="solve", op="abec", n=(12, 10, 8), max_grid_size=8, rhs_seed=1104,
                                   b_seed=2104, periodic=(1, 0, 0), lobc=(200, 101, 101), hibc=(200, 101, 101),
                                   maxorder=4, b_sigma=2.0),
    }


def _inputs(c):
    """Case inputs with the two stored copies of each periodic domain face
    made equal (as a face MultiFab synchronised across the periodic boundary
    holds them): the operator is then symmetric across that boundary."""
    arr = cases.inputs(c)
    per = c.get("periodic", (0, 0, 0))
    for d, k in enumerate(("bx", "by", "bz")):
        if per[d] and k in arr:
            ax = 2 - d
            b = arr[k].copy()
            last = [slice(None)] * 3
            last[ax] = slice(-1, None)
            first = [slice(None)] * 3
            first[ax] = slice(0, 1)
            b[tuple(last)] = b[tuple(first)]
            arr[k] = b
    return arr


@pytest.fixture(scope="module", autouse=True)
def _built():
    oracle.build()


def _target_and_region(c):
    nx, ny, nz = c["n"]
    rng = np.random.Generator(np.random.PCG64(7))
    tgt = rng.standard_normal((nz, ny, nx)) * 1e-3
    region = (slice(nz // 4, nz - nz // 4), slice(ny // 4, ny - ny // 4), slice(nx // 4, nx - nx // 4))
    return tgt, region


def _dJdphi(tgt, region):
    def f(phi):
        g = np.zeros_like(phi)
        g[region] = phi[region] - tgt[region]
        return g
    return f


@pytest.mark.parametrize("name", list(_small_cases()))
def test_operator_matrix_reproduces_apply(name):
    c = _small_cases()[name]
    arr = _inputs(c)
    A = adjoint.operator_matrix(c, arr)
    nx, ny, nz = c["n"]
    x = np.random.Generator(np.random.PCG64(3)).standard_normal((nz, ny, nx))
    g = arr["sol"].copy()
    g[:] = 0.0
    g[1:-1, 1:-1, 1:-1] = x
    ref = oracle.apply(c, dict(arr, sol=g))
    np.testing.assert_allclose((A @ x.ravel()).reshape(nz, ny, nx), ref, rtol=1e-12, atol=1e-12 * np.abs(ref).max())


@pytest.mark.parametrize("name", list(_small_cases()))
def test_reference_gradient_matches_finite_differences(name):
    """dJ/db and dJ/df from lambda = A^{-T} dJ/dphi agree with central
    differences (eps = 1e-6, relative perturbations of b) to 1e-6."""
    c = _small_cases()[name]
    arr = _inputs(c)
    tgt, region = _target_and_region(c)
    phi, lam, gb = adjoint.gradients(c, arr, _dJdphi(tgt, region))
    rng = np.random.Generator(np.random.PCG64(11))
    eps = 1e-6
    for _ in range(3):
        d = [rng.standard_normal(arr[k].shape) * arr[k] for k in ("bx", "by", "bz")]
        jp = adjoint.objective(c, dict(arr, bx=arr["bx"] + eps * d[0], by=arr["by"] + eps * d[1],
                                       bz=arr["bz"] + eps * d[2]), tgt, region)
        jm = adjoint.objective(c, dict(arr, bx=arr["bx"] - eps * d[0], by=arr["by"] - eps * d[1],
                                       bz=arr["bz"] - eps * d[2]), tgt, region)
        fd = (jp - jm) / (2 * eps)
        ad = sum(float(np.sum(g * dd)) for g, dd in zip(gb, d))
        assert abs(fd - ad) <= 1e-6 * abs(fd), (fd, ad)
    df = rng.standard_normal(arr["rhs"].shape)
    jp = adjoint.objective(c, dict(arr, rhs=arr["rhs"] + eps * df), tgt, region)
    jm = adjoint.objective(c, dict(arr, rhs=arr["rhs"] - eps * df), tgt, region)
    fd = (jp - jm) / (2 * eps)
    ad = float(np.sum(lam * df))
    assert abs(fd - ad) <= 1e-6 * abs(fd), (fd, ad)


@pytest.mark.parametrize("name", list(_small_cases()))
def test_face_gradient_closed_form(name):
    """-beta dxinv^2 (phi_c - phi_{c-1})(lam_c - lam_{c-1}) with lam = 0
    outside the domain equals -lam . (dA/db_face) phi on every face."""
    c = _small_cases()[name]
    arr = _inputs(c)
    tgt, region = _target_and_region(c)
    phi, lam, gb = adjoint.gradients(c, arr, _dJdphi(tgt, region))
    closed = adjoint.face_gradient_formula(c, arr, phi, lam)
    for g, h in zip(gb, closed):
        np.testing.assert_allclose(h, g, rtol=1e-9, atol=1e-11 * np.abs(g).max())


def test_transpose_differs_only_next_to_dirichlet_faces():
    """A - A^T is non-zero only in rows and columns within maxorder-2 cells of
    a Dirichlet face (the ghost closure), as the transposed residual kernel
    assumes."""
    c = _small_cases()["mixed_bc"]
    arr = _inputs(c)
    A = adjoint.operator_matrix(c, arr)
    D = (A - A.T).tocoo()
    D.eliminate_zeros()
    nx, ny, nz = c["n"]
    big = np.abs(D.data) > 1e-9 * np.abs(A.data).max()
    rows = D.row[big]
    k, j, i = np.unravel_index(rows, (nz, ny, nx))
    # Dirichlet faces of this case: x lo, y hi, z lo, z hi
    near = (i <= 1) | (j >= ny - 2) | (k <= 1) | (k >= nz - 2)
    assert big.any() and near.all()
