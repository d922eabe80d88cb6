"""Reference adjoint gradients for small cases, built from the oracle's
operator apply (TEST INFRASTRUCTURE ONLY: used by tests/, never by the
library).

The reference has no adjoint; what it pins is the discrete operator.  The
oracle's `apply` restates MLMG::apply (AMReX_MLMG.H:858-932: applyBC with the
level's Dirichlet values, then Fapply) and is itself checked against the
reference's golden apply outputs.  From it:

* ``operator_matrix``: the homogeneous-BC matrix A, column by column, by
  probing with unit vectors on cells 5 apart (a row couples to cells at most
  2 away: the 7-point stencil and the Dirichlet ghost closure of maxorder <= 4;
  periodic axes use a spacing that divides their length);
* ``bc_term``: the inhomogeneous part (apply of zero with the level BC);
* ``coef_derivative``: (dA/db_face) phi for every face, by probing with b
  equal to one on faces 3 apart (alpha = 0), which is exact because A phi is
  linear in b for a fixed phi (the ghost closure does not involve b);
* ``gradients``: phi = A^{-1}(f - bc), lambda = A^{-T} dJ/dphi with scipy's
  sparse LU, dJ/df = lambda and dJ/db_face = -lambda . (dA/db_face) phi.
"""
from __future__ import annotations

import numpy as np

from oracle import oracle


def _case_arrays(case, arrays, sol_interior=None, ghost=True, bx=None, by=None, bz=None, alpha=None):
    nx, ny, nz = case["n"]
    g = np.array(arrays["sol"], dtype=np.float64, copy=True)
    if not ghost:
        g[:] = 0.0
    g[1:-1, 1:-1, 1:-1] = 0.0 if sol_interior is None else sol_interior
    a = dict(arrays)
    a["sol"] = g
    if case.get("op", "poisson") == "abec":
        if bx is not None:
            a["bx"], a["by"], a["bz"] = bx, by, bz
    c = dict(case)
    if alpha is not None:
        c["alpha"] = alpha
    return c, a


def _strides(case, reach=2):
    """Probe spacing per axis (z, y, x): 2*reach+1, or for a periodic axis the
    smallest divisor of its length that is at least that (else the length)."""
    n = case["n"]
    per = case.get("periodic", (0, 0, 0))
    out = []
    for d in (2, 1, 0):
        s = 2 * reach + 1
        if per[d]:
            s = next((q for q in range(s, n[d] + 1) if n[d] % q == 0), n[d])
        out.append(s)
    return out


def _nearest(k, o, s, n, periodic):
    if periodic:
        delta = (k - o) % s
        c = np.where(delta <= s // 2, k - delta, k + (s - delta))
        return c % n
    return o + np.round((k - o) / s).astype(int) * s


def operator_matrix(case, arrays):
    """Sparse CSR matrix of the homogeneous-BC operator (rows and columns in
    z-major, x-fastest cell order)."""
    import scipy.sparse as sp
    nx, ny, nz = case["n"]
    per = case.get("periodic", (0, 0, 0))
    N = nx * ny * nz
    sz, sy, sx = _strides(case)
    rows, cols, vals = [], [], []
    idx = np.arange(N).reshape(nz, ny, nx)
    for oz in range(sz):
        for oy in range(sy):
            for ox in range(sx):
                e = np.zeros((nz, ny, nx))
                e[oz::sz, oy::sy, ox::sx] = 1.0
                if not e.any():
                    continue
                c, a = _case_arrays(case, arrays, e, ghost=False)
                y = oracle.apply(c, a)
                # the column of row r is the probed cell nearest to r
                kz, ky, kx = np.nonzero(y)
                cz = _nearest(kz, oz, sz, nz, per[2])
                cy = _nearest(ky, oy, sy, ny, per[1])
                cx = _nearest(kx, ox, sx, nx, per[0])
                rows.append(idx[kz, ky, kx])
                cols.append(idx[cz, cy, cx])
                vals.append(y[kz, ky, kx])
    return sp.csr_matrix((np.concatenate(vals), (np.concatenate(rows), np.concatenate(cols))), shape=(N, N))


def bc_term(case, arrays):
    """A applied to zero valid cells with the level's Dirichlet values."""
    c, a = _case_arrays(case, arrays, None, ghost=True)
    return oracle.apply(c, a)


def coef_derivative(case, arrays, phi, lam, stride=3):
    """-lam . (dA/db_face) phi for every face: arrays shaped like bx, by, bz."""
    nx, ny, nz = case["n"]
    shapes = [(nz, ny, nx + 1), (nz, ny + 1, nx), (nz + 1, ny, nx)]
    out = [np.zeros(s) for s in shapes]
    for d in range(3):
        for oz in range(stride):
            for oy in range(stride):
                for ox in range(stride):
                    unit = np.zeros(shapes[d])
                    unit[oz::stride, oy::stride, ox::stride] = 1.0
                    if not unit.any():
                        continue
                    b = [np.zeros(s) for s in shapes]
                    b[d] = unit
                    c, a = _case_arrays(case, arrays, phi, ghost=True, bx=b[0], by=b[1], bz=b[2], alpha=0.0)
                    y = oracle.apply(c, a) * lam        # per-row contribution
                    # each row touches at most one probed face; give it to that face
                    kz, ky, kx = np.nonzero(y)
                    f = [kz, ky, kx]
                    # the probed face of the row: its low face or its high face along d
                    ax = 2 - d                           # array axis of direction d
                    lo = [kz.copy(), ky.copy(), kx.copy()]
                    hi = [kz.copy(), ky.copy(), kx.copy()]
                    hi[ax] = hi[ax] + 1
                    lo_hit = unit[lo[0], lo[1], lo[2]] > 0
                    hz, hy, hx = hi
                    in_hi = hi[ax] < shapes[d][ax]
                    hi_hit = np.zeros_like(lo_hit)
                    hi_hit[in_hi] = unit[hz[in_hi], hy[in_hi], hx[in_hi]] > 0
                    assert not np.any(lo_hit & hi_hit)
                    np.add.at(out[d], (lo[0][lo_hit], lo[1][lo_hit], lo[2][lo_hit]), -y[f[0], f[1], f[2]][lo_hit])
                    np.add.at(out[d], (hz[hi_hit], hy[hi_hit], hx[hi_hit]), -y[f[0], f[1], f[2]][hi_hit])
    return out


def gradients(case, arrays, dJdphi_fn):
    """(phi, lam, [dJ/dbx, dJ/dby, dJ/dbz]) with dJ/dphi = dJdphi_fn(phi)."""
    import scipy.sparse.linalg as spla
    nx, ny, nz = case["n"]
    A = operator_matrix(case, arrays).tocsc()
    f = np.asarray(arrays["rhs"], dtype=np.float64) - bc_term(case, arrays)
    lu = spla.splu(A)
    phi = lu.solve(f.ravel()).reshape(nz, ny, nx)
    g = dJdphi_fn(phi)
    lam = lu.solve(g.ravel(), trans="T").reshape(nz, ny, nx)
    return phi, lam, coef_derivative(case, arrays, phi, lam)


def objective(case, arrays, target, region):
    """J = 0.5 sum over `region` (a tuple of slices, z-major) of (phi - target)^2
    with phi from a sparse direct solve."""
    import scipy.sparse.linalg as spla
    nx, ny, nz = case["n"]
    A = operator_matrix(case, arrays).tocsc()
    f = np.asarray(arrays["rhs"], dtype=np.float64) - bc_term(case, arrays)
    phi = spla.splu(A).solve(f.ravel()).reshape(nz, ny, nx)
    return 0.5 * float(np.sum((phi[region] - target[region]) ** 2))


def face_gradient_formula(case, arrays, phi, lam):
    """The closed form the library's contraction kernel evaluates:
    dJ/db = -beta dxinv^2 (phi_c - phi_{c-1}) (lam_c - lam_{c-1}) per face,
    phi's ghosts from the Dirichlet/Neumann closure of the level BC, lam = 0
    outside the domain.  Ghost values come from the oracle's applyBC through
    probing: ghost = phi_c - (A_b phi)_c / (beta dxinv^2) on a unit boundary
    face."""
    nx, ny, nz = case["n"]
    beta = case.get("beta", 1.0)
    dxinv = [case["n"][d] / (case.get("prob_hi", (1, 1, 1))[d] - case.get("prob_lo", (0, 0, 0))[d])
             for d in range(3)]
    shapes = [(nz, ny, nx + 1), (nz, ny + 1, nx), (nz + 1, ny, nx)]
    out = []
    for d in range(3):
        ax = 2 - d
        # boundary ghosts of phi along d from one probing apply per side
        b = [np.zeros(s) for s in shapes]
        sl_lo = [slice(None)] * 3
        sl_lo[ax] = slice(0, 1)
        sl_hi = [slice(None)] * 3
        sl_hi[ax] = slice(-1, None)
        b[d][tuple(sl_lo)] = 1.0
        b[d][tuple(sl_hi)] = 1.0
        c, a = _case_arrays(case, arrays, phi, ghost=True, bx=b[0], by=b[1], bz=b[2], alpha=0.0)
        y = oracle.apply(c, a)
        h = beta * dxinv[d] ** 2
        ext = [list(phi.shape) for _ in range(1)][0]
        ext[ax] += 2
        pe = np.zeros(ext)
        le = np.zeros(ext)
        inner = [slice(None)] * 3
        inner[ax] = slice(1, -1)
        pe[tuple(inner)] = phi
        le[tuple(inner)] = lam
        # (A_b phi)_0 = beta dxinv^2 (phi_0 - ghost) on the low side (one unit face per row)
        first = [slice(None)] * 3
        first[ax] = slice(0, 1)
        last = [slice(None)] * 3
        last[ax] = slice(-1, None)
        y_lo = y[tuple(first)]
        y_hi = y[tuple(last)]
        if phi.shape[ax] == 1:
            raise ValueError("boxes one cell wide are not supported here")
        g0 = [slice(None)] * 3
        g0[ax] = slice(0, 1)
        g1 = [slice(None)] * 3
        g1[ax] = slice(-1, None)
        pe[tuple(g0)] = phi[tuple(first)] - y_lo / h
        pe[tuple(g1)] = phi[tuple(last)] - y_hi / h
        lo_s = [slice(None)] * 3
        lo_s[ax] = slice(0, -1)
        hi_s = [slice(None)] * 3
        hi_s[ax] = slice(1, None)
        out.append(-h * (pe[tuple(hi_s)] - pe[tuple(lo_s)]) * (le[tuple(hi_s)] - le[tuple(lo_s)]))
    return out
