"""Build MultiFab-based problems for the GPU library from a case dict
(tests/golden/cases.py layout) -- the same inputs the reference driver and
the oracle read."""
from __future__ import annotations

import numpy as np

import amrex_gb300 as ag


def make_problem(case, arrays, precision=None, graph=False, fused=False, options=None):
    nx, ny, nz = case["n"]
    domain = ag.Box((0, 0, 0), (nx - 1, ny - 1, nz - 1))
    if case.get("boxes"):
        ba = ag.BoxArray([ag.Box(b[:3], b[3:]) for b in case["boxes"]])
    else:
        ba = ag.BoxArray(domain).maxSize(case.get("max_grid_size", 32))
    dm = ag.DistributionMapping(ba)
    geom = ag.Geometry(domain, case.get("prob_lo", (0, 0, 0)), case.get("prob_hi", (1, 1, 1)),
                       case.get("periodic", (0, 0, 0)))
    info = ag.LPInfo().setAgglomeration(case.get("agg", 1)).setConsolidation(case.get("con", 1)) \
        .setAgglomerationGridSize(case.get("agg_grid_size", 32)).setConsolidationGridSize(case.get("con_grid_size", 32)) \
        .setMaxCoarseningLevel(case.get("max_coarsening_level", 30))
    sol = ag.MultiFab(ba, dm, 1, 1)
    sol.set_global(arrays["sol"], lo=(-1, -1, -1))
    rhs = ag.MultiFab(ba, dm, 1, 0)
    rhs.set_global(arrays["rhs"])
    if case.get("op", "poisson") == "abec":
        op = ag.MLABecLaplacian(geom, ba, dm, info)
    else:
        op = ag.MLPoisson(geom, ba, dm, info)
    op.setDomainBC(case.get("lobc", (101,) * 3), case.get("hibc", (101,) * 3))
    op.setMaxOrder(case.get("maxorder", 3))
    op.setLevelBC(0, sol)
    keep = []
    if case.get("op", "poisson") == "abec":
        op.setScalars(case.get("alpha", 1.0), case.get("beta", 1.0))
        a = ag.MultiFab(ba, dm, 1, 0)
        a.set_global(arrays["a"])
        op.setACoeffs(0, a)
        faces = []
        for d, k in enumerate(("bx", "by", "bz")):
            f = ag.MultiFab(ba, dm, 1, 0, nodal_dir=d)
            f.set_global(arrays[k])
            faces.append(f)
        op.setBCoeffs(0, faces)
        keep += [a] + faces
    mlmg = ag.MLMG(op)
    mlmg.setMaxIter(case.get("max_iter", 200))
    if "bottom_solver" in case:
        mlmg.setBottomSolver(case["bottom_solver"])
    if "bottom_maxiter" in case:
        mlmg.setBottomMaxIter(case["bottom_maxiter"])
    if case.get("fixed_iter", 0):
        mlmg.setFixedIter(case["fixed_iter"])
    if case.get("max_fmg_iter", 0):
        mlmg.setMaxFmgIter(case["max_fmg_iter"])
    if precision is not None:
        mlmg.setPrecision(precision)
    mlmg.setGraph(graph)
    mlmg.setFusedSmoother(fused)
    for k, v in (options or {}).items():
        mlmg.setOption(k, v)
    return dict(ba=ba, dm=dm, geom=geom, sol=sol, rhs=rhs, op=op, mlmg=mlmg, keep=keep, domain=domain)


def solution(prob, case):
    nx, ny, nz = case["n"]
    return prob["sol"].get_global((nz, ny, nx))
