"""Seeded benchmark workloads built through the public API.

* ``abec_problem(n, mgs, rhs_seed, b_seed)``: the variable-coefficient
  MLABecLaplacian on an n^3 unit cube (alpha = a = beta = 1, face b from a
  log-normal random field with max/min contrast 1e3, Gaussian-blob RHS,
  homogeneous Dirichlet on every face, boxes of at most ``mgs`` cells).
* ``batch_specs(nsolve, seed)``: the batch of independent solves of uneven
  sizes -- cube edges drawn uniformly from {32, 48, ..., 128}, solve i with
  RHS and b seeds ``seed + 1 + i``.
* ``amr_problem(n, grids, rhs_seed)``: the composite MLPoisson (or, given
  per-level coefficients, MLABecLaplacian) over AMR levels (base n^3 unit
  cube, refinement ratio 2, level l's boxes ``grids[l]``), Gaussian-blob RHS
  sampled at each level's cell centres, homogeneous Dirichlet and a zero
  initial guess unless given.
"""
from __future__ import annotations

from collections import namedtuple

import numpy as np

import amrex_gb300 as ag
from amrex_gb300 import synth

BatchSolveSpec = namedtuple("BatchSolveSpec", "n rhs_seed b_seed")

BATCH_EDGES = (32, 48, 64, 80, 96, 112, 128)


def batch_specs(nsolve=64, seed=4000):
    rng = np.random.default_rng(seed)
    edges = rng.choice(np.array(BATCH_EDGES), size=nsolve)
    return [BatchSolveSpec(int(e), seed + 1 + i, seed + 1 + i) for i, e in enumerate(edges)]


def abec_problem(n, mgs, rhs_seed, b_seed, rhs_host=None, bcoef_host=None):
    """Operator, solution (1 ghost) and RHS MultiFabs of one solve; the host
    inputs are returned too (``rhs_h``, ``b_h``)."""
    rhs_h = synth.gaussian_rhs(n, rhs_seed) if rhs_host is None else rhs_host
    b_h = synth.lognormal_bcoef(n, b_seed, sigma_cells=5.0, max_ratio=1e3) if bcoef_host is None else bcoef_host
    domain = ag.Box((0, 0, 0), (n - 1, n - 1, n - 1))
    ba = ag.BoxArray(domain).maxSize(mgs)
    dm = ag.DistributionMapping(ba)
    geom = ag.Geometry(domain)
    sol = ag.MultiFab(ba, dm, 1, 1)
    rhs = ag.MultiFab(ba, dm, 1, 0)
    rhs.set_global(rhs_h)
    op = ag.MLABecLaplacian(geom, ba, dm)
    op.setDomainBC((101,) * 3, (101,) * 3)
    op.setLevelBC(0, None)
    op.setScalars(1.0, 1.0)
    op.setACoeffs(0, 1.0)
    faces = []
    for d in range(3):
        f = ag.MultiFab(ba, dm, 1, 0, nodal_dir=d)
        f.set_global(b_h[d])
        faces.append(f)
    op.setBCoeffs(0, faces)
    return dict(n=n, ba=ba, dm=dm, geom=geom, sol=sol, rhs=rhs, op=op, faces=faces, rhs_h=rhs_h, b_h=b_h)


def adjoint_objective(n, phi_scale, target_seed=3003):
    """J = 0.5 * sum over the central half-width cube [n/4, 3n/4)^3 of
    (phi - phi_t)^2, phi_t = phi_scale * (a smooth random field, 5-cell
    Gaussian, unit variance).  Returns (phi_t, region slices z-major)."""
    tgt = phi_scale * synth.smooth_field(n, target_seed)
    q = n // 4
    region = (slice(q, n - q),) * 3
    return tgt, region


def amr_problem(n, grids, rhs_seed, precision=0, graph=False, max_iter=200, agg_grid_size=32, con_grid_size=32,
                fused=False, solbc=None, max_fmg_iter=0, abec=None, periodic=(0, 0, 0)):
    """Composite MLPoisson over len(grids) AMR levels: per-level geometry,
    BoxArray, DistributionMapping, solution (1 ghost, zero) and RHS
    MultiFabs, the operator and the MLMG solver.  ``grids[l]`` holds level l's
    boxes as (lo0, lo1, lo2, hi0, hi1, hi2); ``solbc[l]`` (optional) is a
    grown level-domain array with the initial guess in the valid cells and the
    Dirichlet values in the ghosts.  With ``abec[l] = (alpha, beta, a, bx, by,
    bz)`` (level-domain arrays, z-major) the operator is MLABecLaplacian with
    those per-level coefficients; ``periodic`` makes those directions periodic
    (Dirichlet on the others)."""
    geoms, bas, dms, sols, rhss = [], [], [], [], []
    for lev, g in enumerate(grids):
        m = n << lev
        dom = ag.Box((0, 0, 0), (m - 1, m - 1, m - 1))
        ba = ag.BoxArray([ag.Box(b[:3], b[3:]) for b in g])
        dm = ag.DistributionMapping(ba)
        sol = ag.MultiFab(ba, dm, 1, 1)
        sol.setVal(0.0)
        if solbc is not None and solbc[lev] is not None:
            sol.set_global(solbc[lev], lo=(-1, -1, -1))
        rhs = ag.MultiFab(ba, dm, 1, 0)
        for i, b in enumerate(g):
            rhs.set_fab(i, synth.gaussian_rhs_box(m, rhs_seed, b))
        geoms.append(ag.Geometry(dom, is_periodic=tuple(periodic)))
        bas.append(ba)
        dms.append(dm)
        sols.append(sol)
        rhss.append(rhs)
    info = ag.LPInfo().setAgglomerationGridSize(agg_grid_size).setConsolidationGridSize(con_grid_size)
    coefs = []
    if abec is not None:
        op = ag.MLABecLaplacian(geoms, bas, dms, info)
        op.setScalars(abec[0][0], abec[0][1])
    else:
        op = ag.MLPoisson(geoms, bas, dms, info)
    bc = tuple(ag.LinOpBCType.Periodic if p else ag.LinOpBCType.Dirichlet for p in periodic)
    op.setDomainBC(bc, bc)
    for lev in range(len(grids)):
        op.setLevelBC(lev, sols[lev])
        if abec is not None:
            a = ag.MultiFab(bas[lev], dms[lev], 1, 0)
            a.set_global(abec[lev][2])
            op.setACoeffs(lev, a)
            faces = []
            for d in range(3):
                f = ag.MultiFab(bas[lev], dms[lev], 1, 0, nodal_dir=d)
                f.set_global(abec[lev][3 + d])
                faces.append(f)
            op.setBCoeffs(lev, faces)
            coefs.append((a, faces))
    mlmg = ag.MLMG(op)
    mlmg.setMaxIter(max_iter)
    if max_fmg_iter:
        mlmg.setMaxFmgIter(max_fmg_iter)
    mlmg.setPrecision(precision)
    mlmg.setGraph(graph)
    mlmg.setFusedSmoother(fused)
    return dict(geoms=geoms, bas=bas, dms=dms, sols=sols, rhss=rhss, op=op, mlmg=mlmg, coefs=coefs)
