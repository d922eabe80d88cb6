"""Adjoint gradients through the C ABI (mlmg_adjoint_grad) on the GPU:
against the exact derivatives of the oracle's discrete operator on small
cases, and against central finite differences on the 128^3 variable-
coefficient ABecLaplacian, through a torch.autograd.Function that exists only
in this test harness.  Needs a CUDA GPU (GB300)."""
import math

import numpy as np
import pytest

import amrex_gb300 as ag
from oracle import adjoint, oracle
from tests import helpers
from tests.golden import cases
from tests.test_oracle_adjoint import _dJdphi, _inputs, _small_cases, _target_and_region

pytestmark = pytest.mark.gpu

TOL = 1e-12


def _mf_like(prob, nodal_dir=-1):
    return ag.MultiFab(prob["ba"], prob["dm"], 1, 0, nodal_dir=nodal_dir)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("name", list(_small_cases()))
def test_adjoint_matches_exact_derivatives(name, precision):
    """lambda (= dJ/df), dJ/db and dJ/da against sparse-direct derivatives of
    the oracle's operator."""
    oracle.build()
    c = _small_cases()[name]
    arr = _inputs(c)
    tgt, region = _target_and_region(c)
    phi_ref, lam_ref, gb_ref = adjoint.gradients(c, arr, _dJdphi(tgt, region))
    prob = helpers.make_problem(c, arr, precision=precision)
    m = prob["mlmg"]
    m.solve(prob["sol"], prob["rhs"], TOL, 0.0)
    phi = helpers.solution(prob, c)
    assert np.abs(phi - phi_ref).max() <= 1e-9 * np.abs(phi_ref).max()
    g = _mf_like(prob)
    g.set_global(_dJdphi(tgt, region)(phi))
    lam = _mf_like(prob)
    gb = [_mf_like(prob, d) for d in range(3)]
    ga = _mf_like(prob)
    m.adjointGrad(prob["sol"], g, TOL, 0.0, lam, gb, ga)
    nx, ny, nz = c["n"]
    lam_gpu = lam.get_global((nz, ny, nx))
    np.testing.assert_allclose(lam_gpu, lam_ref, rtol=0, atol=1e-8 * np.abs(lam_ref).max())
    shapes = [(nz, ny, nx + 1), (nz, ny + 1, nx), (nz + 1, ny, nx)]
    for d in range(3):
        got = gb[d].get_global(shapes[d])
        np.testing.assert_allclose(got, gb_ref[d], rtol=0, atol=1e-8 * np.abs(gb_ref[d]).max())
    ga_ref = -c.get("alpha", 1.0) * lam_ref * phi_ref
    np.testing.assert_allclose(ga.get_global((nz, ny, nx)), ga_ref, rtol=0, atol=1e-8 * np.abs(ga_ref).max())


def test_adjoint_rejects_singular_operator():
    from tests.golden import load
    c = load.load("solve_abec_neumann_singular")["case"]
    prob = helpers.make_problem(c, cases.inputs(c), precision="fp64")
    g, lam = _mf_like(prob), _mf_like(prob)
    with pytest.raises(ag.MLMGError):
        prob["mlmg"].adjointGrad(prob["sol"], g, 1e-10, 0.0, lam)


class _SolveFn:
    """phi(b, f) of one MLABecLaplacian as a torch.autograd.Function (test
    harness only): forward = MLMG solve, backward = mlmg_adjoint_grad."""

    def __init__(self, n, mgs, precision, tol, fixed_iter=0):
        import torch
        from amrex_gb300 import workloads
        self.p = workloads.abec_problem(n, mgs, 1003, 2003)
        self.n = n
        self.m = ag.MLMG(self.p["op"])
        self.m.setPrecision(precision)
        if fixed_iter:
            self.m.setFixedIter(fixed_iter)
        self.tol = tol
        self.shapes = [(n, n, n + 1), (n, n + 1, n), (n + 1, n, n)]
        outer = self

        class Fn(torch.autograd.Function):
            @staticmethod
            def forward(ctx, bx, by, bz, f):
                phi = outer.solve([bx, by, bz], f)
                return torch.from_numpy(phi)

            @staticmethod
            def backward(ctx, gphi):
                g = _mf_like(outer.p)
                g.set_global(gphi.detach().cpu().numpy().astype(np.float64))
                lam = _mf_like(outer.p)
                gb = [_mf_like(outer.p, d) for d in range(3)]
                outer.m.adjointGrad(outer.p["sol"], g, outer.tol, 0.0, lam, gb)
                out = [torch.from_numpy(gb[d].get_global(outer.shapes[d])) for d in range(3)]
                return out[0], out[1], out[2], torch.from_numpy(lam.get_global((n, n, n)))

        self.Fn = Fn

    def solve(self, b, f):
        n = self.n
        for d in range(3):
            self.p["faces"][d].set_global(np.ascontiguousarray(b[d].detach().cpu().numpy()))
        self.p["op"].setBCoeffs(0, self.p["faces"])
        self.p["rhs"].set_global(np.ascontiguousarray(f.detach().cpu().numpy()))
        self.p["sol"].setVal(0.0)
        self.m.solve(self.p["sol"], self.p["rhs"], self.tol, 0.0)
        return self.p["sol"].get_global((n, n, n))


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_adjoint_fd_128(precision):
    """128^3 variable-coefficient ABecLaplacian (log-normal b, contrast 1e3),
    J = 0.5 |phi - phi_t|^2 over the central 64^3: directional derivatives of
    the adjoint gradients dJ/db (all faces) and dJ/df match central finite
    differences (eps = 1e-6) along 20 seeded smooth random directions each
    (5-cell Gaussian fields; relative perturbations for b), to 1e-6
    relative.  The finite differences, the reference here, always come from
    the FP64 solver: a mixed-precision forward solve stagnates near the
    rounding floor of its FP64 residual (about 1e-10 relative at this size),
    and that noise, not the adjoint, would dominate a 1e-6 comparison."""
    import torch
    from amrex_gb300 import synth, workloads
    n = 128
    # a fixed count of 30 V-cycles (to the FP64 rounding floor) for every
    # forward and adjoint solve, so that the +eps and -eps solves run the same
    # iteration and their errors cancel in the difference
    S = _SolveFn(n, 64, precision, 1e-16, fixed_iter=30)
    FD = S if precision == "fp64" else _SolveFn(n, 64, "fp64", 1e-16, fixed_iter=30)
    b0 = [torch.from_numpy(np.ascontiguousarray(x)) for x in S.p["b_h"]]
    f0 = torch.from_numpy(np.ascontiguousarray(S.p["rhs_h"]))
    phi0 = S.solve(b0, f0)
    tgt, region = workloads.adjoint_objective(n, float(phi0.std()))
    tgt_t = torch.from_numpy(tgt)

    def J_of(b, f):
        phi = FD.solve(b, f)
        return 0.5 * math.fsum(((phi - tgt)[region] ** 2).ravel())

    bs = [x.clone().requires_grad_(True) for x in b0]
    f = f0.clone().requires_grad_(True)
    phi = S.Fn.apply(bs[0], bs[1], bs[2], f)
    J = 0.5 * ((phi - tgt_t)[region] ** 2).sum()
    J.backward()
    gb = [x.grad.numpy() for x in bs]
    gf = f.grad.numpy()
    eps = 1e-6
    worst_b = worst_f = 0.0
    for k in range(20):
        # a smooth random direction (5-cell Gaussian field), relative to b
        g = synth.lognormal_bcoef(n, 3100 + k, contrast=1.0)
        d = [np.log(gg) * x.numpy() for gg, x in zip(g, b0)]
        jp = J_of([torch.from_numpy(x.numpy() + eps * dd) for x, dd in zip(b0, d)], f0)
        jm = J_of([torch.from_numpy(x.numpy() - eps * dd) for x, dd in zip(b0, d)], f0)
        fd = (jp - jm) / (2 * eps)
        ad = sum(float(np.sum(gg * dd)) for gg, dd in zip(gb, d))
        worst_b = max(worst_b, abs(fd - ad) / abs(fd))
    for k in range(20):
        df = synth.smooth_field(n, 3200 + k) * float(np.abs(S.p["rhs_h"]).max())
        jp = J_of(b0, torch.from_numpy(f0.numpy() + eps * df))
        jm = J_of(b0, torch.from_numpy(f0.numpy() - eps * df))
        fd = (jp - jm) / (2 * eps)
        ad = float(np.sum(gf * df))
        worst_f = max(worst_f, abs(fd - ad) / abs(fd))
    print(f"adjoint vs FD ({precision}): worst relative error dJ/db {worst_b:.3e}, dJ/df {worst_f:.3e}")
    worst = max(worst_b, worst_f)
    assert worst <= 1e-6, worst
