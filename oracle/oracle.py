"""ctypes front end of the CPU oracle (oracle/mlmg_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, by ``__graft_entry__.smoke()``
and by the CPU-baseline leg of ``bench.py`` -- never by the library itself.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "mlmg_oracle.c")
LIB = os.path.join(HERE, "liboracle.so")

MAX_HIST = 256


def build(force=False):
    """Compile the oracle with gcc (no FMA contraction, OpenMP off)."""
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= max(
            os.path.getmtime(SRC), os.path.getmtime(os.path.join(HERE, "mlmg_oracle.h"))):
        return LIB
    tmp = LIB + ".tmp.%d" % os.getpid()
    subprocess.run(["gcc", "-O2", "-std=gnu11", "-fopenmp", "-fPIC", "-shared", "-ffp-contract=off", "-o", tmp,
                    SRC, "-lm"], check=True)
    os.replace(tmp, LIB)
    return LIB


class Problem(ctypes.Structure):
    _fields_ = [("n", ctypes.c_int * 3), ("periodic", ctypes.c_int * 3),
                ("prob_lo", ctypes.c_double * 3), ("prob_hi", ctypes.c_double * 3),
                ("lobc", ctypes.c_int * 3), ("hibc", ctypes.c_int * 3),
                ("max_grid_size", ctypes.c_int), ("nbox", ctypes.c_int),
                ("boxes", ctypes.POINTER(ctypes.c_int)),
                ("is_abec", ctypes.c_int), ("alpha", ctypes.c_double), ("beta", ctypes.c_double),
                ("sol", ctypes.POINTER(ctypes.c_double)), ("rhs", ctypes.POINTER(ctypes.c_double)),
                ("a", ctypes.POINTER(ctypes.c_double)), ("bx", ctypes.POINTER(ctypes.c_double)),
                ("by", ctypes.POINTER(ctypes.c_double)), ("bz", ctypes.POINTER(ctypes.c_double))]


class Options(ctypes.Structure):
    _fields_ = [(k, ctypes.c_int) for k in ("agg", "con", "agg_grid_size", "con_grid_size",
                                            "max_coarsening_level", "maxorder", "nu1", "nu2", "nuf", "nub",
                                            "max_iter", "fixed_iter", "bottom_solver", "bottom_maxiter")] + \
               [(k, ctypes.c_double) for k in ("bottom_reltol", "tol_rel", "tol_abs")] + \
               [("max_fmg_iter", ctypes.c_int)]


class Result(ctypes.Structure):
    _fields_ = [("status", ctypes.c_int), ("niters", ctypes.c_int), ("nlev", ctypes.c_int),
                ("init_resid", ctypes.c_double), ("rhs_norm", ctypes.c_double), ("final_resid", ctypes.c_double),
                ("iter_seconds", ctypes.c_double),
                ("history", ctypes.c_double * MAX_HIST), ("cg_iters", ctypes.c_int * MAX_HIST),
                ("ncg", ctypes.c_int)]


_lib = None


def lib():
    global _lib
    if _lib is None:
        _lib = ctypes.CDLL(build())
        P = ctypes.POINTER
        _lib.oracle_default_options.argtypes = [P(Options)]
        _lib.oracle_max_size.argtypes = [P(ctypes.c_int), P(ctypes.c_int), ctypes.c_int, P(ctypes.c_int), ctypes.c_int]
        _lib.oracle_hierarchy.argtypes = [P(Problem), P(Options), P(ctypes.c_int), P(ctypes.c_int), ctypes.c_int]
        _lib.oracle_fill_boundary.argtypes = [P(Problem), ctypes.c_int, P(ctypes.c_double)]
        _lib.oracle_apply.argtypes = [P(Problem), P(Options), P(ctypes.c_double)]
        _lib.oracle_fluxes.argtypes = [P(Problem), P(Options), ctypes.c_int, P(ctypes.c_double), P(ctypes.c_double),
                                       P(ctypes.c_double)]
        _lib.oracle_solve.argtypes = [P(Problem), P(Options), P(ctypes.c_double), P(Result)]
        _lib.oracle_solve_amr.argtypes = [ctypes.c_int, P(Problem), P(Options), P(P(ctypes.c_double)), P(Result)]
    return _lib


def _dp(a):
    return None if a is None else a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _f64(a):
    return None if a is None else np.ascontiguousarray(a, dtype=np.float64)


def make_problem(case, arrays):
    """Problem struct from a case dict (tests/golden/cases.py layout) and the
    arrays returned by cases.inputs().  Returns (problem, keepalive)."""
    p = Problem()
    keep = []
    p.n[:] = list(case["n"])
    p.periodic[:] = list(case.get("periodic", (0, 0, 0)))
    p.prob_lo[:] = list(case.get("prob_lo", (0.0, 0.0, 0.0)))
    p.prob_hi[:] = list(case.get("prob_hi", (1.0, 1.0, 1.0)))
    p.lobc[:] = list(case.get("lobc", (101, 101, 101)))
    p.hibc[:] = list(case.get("hibc", (101, 101, 101)))
    p.max_grid_size = case.get("max_grid_size", 32)
    if case.get("boxes"):
        bx = np.ascontiguousarray(np.array(case["boxes"], dtype=np.int32).ravel())
        keep.append(bx)
        p.nbox = len(case["boxes"])
        p.boxes = bx.ctypes.data_as(ctypes.POINTER(ctypes.c_int))
    p.is_abec = 1 if case.get("op", "poisson") == "abec" else 0
    p.alpha = case.get("alpha", 1.0)
    p.beta = case.get("beta", 1.0)
    for k in ("sol", "rhs", "a", "bx", "by", "bz"):
        a = _f64(arrays.get(k))
        keep.append(a)
        setattr(p, k, _dp(a))
    return p, keep


def make_options(case):
    o = Options()
    lib().oracle_default_options(ctypes.byref(o))
    for k in ("agg", "con", "agg_grid_size", "con_grid_size", "maxorder", "max_iter", "fixed_iter",
              "max_coarsening_level", "max_fmg_iter", "bottom_solver", "bottom_maxiter"):
        if k in case:
            setattr(o, k, int(case[k]))
    for k in ("tol_rel", "tol_abs"):
        if k in case:
            setattr(o, k, float(case[k]))
    return o


def max_size(n, chunk, lo=(0, 0, 0)):
    lo_a = (ctypes.c_int * 3)(*lo)
    hi_a = (ctypes.c_int * 3)(*[lo[d] + n[d] - 1 for d in range(3)])
    out = (ctypes.c_int * (6 * 100000))()
    nb = lib().oracle_max_size(lo_a, hi_a, chunk, out, 100000)
    return [tuple(out[6 * b:6 * b + 6]) for b in range(nb)]


def hierarchy(case):
    p, keep = make_problem(case, {})
    o = make_options(case)
    nb = (ctypes.c_int * 64)()
    out = (ctypes.c_int * (6 * 200000))()
    nlev = lib().oracle_hierarchy(ctypes.byref(p), ctypes.byref(o), nb, out, 200000)
    levels, q = [], 0
    for lev in range(nlev):
        levels.append([tuple(out[6 * (q + b):6 * (q + b) + 6]) for b in range(nb[lev])])
        q += nb[lev]
    return levels


def fill_boundary(case, data, cross):
    p, keep = make_problem(case, {})
    d = np.ascontiguousarray(data, dtype=np.float64).copy()
    lib().oracle_fill_boundary(ctypes.byref(p), int(cross), _dp(d))
    return d


def apply(case, arrays):
    p, keep = make_problem(case, arrays)
    o = make_options(case)
    nx, ny, nz = case["n"]
    out = np.zeros((nz, ny, nx))
    lib().oracle_apply(ctypes.byref(p), ctypes.byref(o), _dp(out))
    return out


def fluxes(case, arrays, mode):
    """mode "grad" (MLMG::getGradSolution) or "flux" (MLMG::getFluxes) of the
    solution in arrays["sol"] (valid cells + level BC values in the ghosts);
    returns the three global face arrays, z-major."""
    p, keep = make_problem(case, arrays)
    o = make_options(case)
    nx, ny, nz = case["n"]
    out = [np.zeros((nz, ny, nx + 1)), np.zeros((nz, ny + 1, nx)), np.zeros((nz + 1, ny, nx))]
    lib().oracle_fluxes(ctypes.byref(p), ctypes.byref(o), 0 if mode == "grad" else 1, _dp(out[0]), _dp(out[1]),
                        _dp(out[2]))
    return out


def solve(case, arrays):
    """Returns (phi, info dict)."""
    p, keep = make_problem(case, arrays)
    o = make_options(case)
    nx, ny, nz = case["n"]
    phi = np.zeros((nz, ny, nx))
    r = Result()
    lib().oracle_solve(ctypes.byref(p), ctypes.byref(o), _dp(phi), ctypes.byref(r))
    info = dict(status=r.status, niters=r.niters, nlev=r.nlev, init_resid=r.init_resid, rhs_norm=r.rhs_norm,
                final_resid=r.final_resid, iter_seconds=r.iter_seconds,
                history=list(r.history[:min(r.niters, MAX_HIST)]),
                cg_iters=list(r.cg_iters[:min(r.ncg, MAX_HIST)]))
    return phi, info


def solve_amr(case, levels):
    """Composite solve over AMR levels (ratio 2, MLPoisson, or MLABecLaplacian
    with case["op"] == "abec" and its alpha, beta).  ``case`` holds the
    level-0 settings (n, bc, solver options); ``levels`` is a list of dicts
    with "boxes", "rhs" (level domain, z-major), optionally "sol" (grown level
    domain: initial guess + boundary values; zero by default) and, for
    MLABecLaplacian, "a", "bx", "by", "bz" over the level domain.
    Returns (list of level-domain phi arrays, info dict)."""
    nlev = len(levels)
    probs = (Problem * nlev)()
    keep = []
    phis = []
    for lev, L in enumerate(levels):
        n = [v << lev for v in case["n"]]
        c = dict(case, n=tuple(n), boxes=L["boxes"])
        sol = L.get("sol")
        if sol is None:
            sol = np.zeros((n[2] + 2, n[1] + 2, n[0] + 2))
        arrays = {"sol": sol, "rhs": L["rhs"]}
        for key in ("a", "bx", "by", "bz"):
            if L.get(key) is not None:
                arrays[key] = L[key]
        p, k = make_problem(c, arrays)
        keep.append(k)
        probs[lev] = p
        phis.append(np.zeros((n[2], n[1], n[0])))
    ptrs = (ctypes.POINTER(ctypes.c_double) * nlev)(*[_dp(a) for a in phis])
    o = make_options(case)
    r = Result()
    lib().oracle_solve_amr(nlev, probs, ctypes.byref(o), ptrs, ctypes.byref(r))
    info = dict(status=r.status, niters=r.niters, nlev=r.nlev, init_resid=r.init_resid, rhs_norm=r.rhs_norm,
                final_resid=r.final_resid, iter_seconds=r.iter_seconds,
                history=list(r.history[:min(r.niters, MAX_HIST)]),
                cg_iters=list(r.cg_iters[:min(r.ncg, MAX_HIST)]))
    return phis, info
