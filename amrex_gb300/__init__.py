"""GB300-native MLMG (cell-centred MLPoisson / MLABecLaplacian) -- Python host API.

A thin mirror of the reference's C++ interface for this path (amrex::BoxArray,
DistributionMapping, Geometry, MultiFab, LPInfo, MLPoisson, MLABecLaplacian,
MLMG), implemented over the C ABI of ``libamrex_gb300.so``
(include/mlmg_capi.h).  All compute runs in hand-written sm_103a kernels;
importing this package never falls back to a CPU path.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import capi
from .capi import MLMGError, check

__all__ = ["Box", "BoxArray", "DistributionMapping", "Geometry", "MultiFab", "LPInfo", "LinOpBCType",
           "MLPoisson", "MLABecLaplacian", "MLMG", "MLMGError", "solve_batched", "kernel_launches",
           "fp64_fma_rate", "check_bit_conversions"]


class LinOpBCType:
    """LinOpBCType codes (Src/Boundary/AMReX_LO_BCTYPES.H:5-35)."""
    interior = 0
    Dirichlet = 101
    Neumann = 102
    reflect_odd = 103
    Periodic = 200


def _i3(v):
    return capi.I3(*[int(x) for x in v])


def _d3(v):
    return capi.D3(*[float(x) for x in v])


class Box:
    def __init__(self, lo, hi):
        self.lo = tuple(int(x) for x in lo)
        self.hi = tuple(int(x) for x in hi)

    def length(self, d=None):
        ln = tuple(self.hi[i] - self.lo[i] + 1 for i in range(3))
        return ln if d is None else ln[d]

    def numPts(self):
        n = self.length()
        return n[0] * n[1] * n[2]

    def __eq__(self, o):
        return isinstance(o, Box) and self.lo == o.lo and self.hi == o.hi

    def __repr__(self):
        return f"Box({self.lo}, {self.hi})"


class BoxArray:
    """amrex::BoxArray: BoxArray(domain) or BoxArray(list_of_boxes); maxSize."""

    def __init__(self, boxes):
        h = ctypes.c_void_p()
        if isinstance(boxes, Box):
            check(capi.lib().mlmg_boxarray_new_domain(_i3(boxes.lo), _i3(boxes.hi), ctypes.byref(h)))
        else:
            flat = np.array([list(b.lo) + list(b.hi) for b in boxes], dtype=np.int32).ravel()
            check(capi.lib().mlmg_boxarray_new(flat.ctypes.data_as(ctypes.POINTER(ctypes.c_int)), len(boxes),
                                               ctypes.byref(h)))
        self._h = h

    def maxSize(self, chunk):
        if np.isscalar(chunk):
            chunk = (chunk, chunk, chunk)
        check(capi.lib().mlmg_boxarray_maxsize(self._h, _i3(chunk)))
        return self

    def size(self):
        return capi.lib().mlmg_boxarray_size(self._h)

    def __len__(self):
        return self.size()

    def __getitem__(self, i):
        lo, hi = capi.I3(), capi.I3()
        check(capi.lib().mlmg_boxarray_get(self._h, int(i), lo, hi))
        return Box(tuple(lo), tuple(hi))

    def boxes(self):
        return [self[i] for i in range(self.size())]

    def __del__(self):
        if getattr(self, "_h", None) and capi._lib is not None:
            capi.lib().mlmg_boxarray_delete(self._h)


class DistributionMapping:
    """amrex::DistributionMapping(const BoxArray&): one GPU owns every box."""

    def __init__(self, ba):
        h = ctypes.c_void_p()
        check(capi.lib().mlmg_distromap_new(ba._h, ctypes.byref(h)))
        self._h = h

    def __del__(self):
        if getattr(self, "_h", None) and capi._lib is not None:
            capi.lib().mlmg_distromap_delete(self._h)


class Geometry:
    """amrex::Geometry(domain, RealBox, coord=cartesian, is_periodic)."""

    def __init__(self, domain, prob_lo=(0.0, 0.0, 0.0), prob_hi=(1.0, 1.0, 1.0), is_periodic=(0, 0, 0)):
        h = ctypes.c_void_p()
        check(capi.lib().mlmg_geometry_new(_i3(domain.lo), _i3(domain.hi), _d3(prob_lo), _d3(prob_hi),
                                           _i3(is_periodic), ctypes.byref(h)))
        self._h = h
        self.domain = domain
        self.is_periodic = tuple(is_periodic)

    def __del__(self):
        if getattr(self, "_h", None) and capi._lib is not None:
            capi.lib().mlmg_geometry_delete(self._h)


class MultiFab:
    """amrex::MultiFab(ba, dm, ncomp, ngrow) on the GPU; ``nodal_dir`` makes a
    face-centred MultiFab (amrex::convert(ba, IntVect::TheDimensionVector(d))),
    ``precision`` 8 (double) or 4 (float)."""

    def __init__(self, ba, dm, ncomp=1, ngrow=0, nodal_dir=-1, precision=8):
        h = ctypes.c_void_p()
        check(capi.lib().mlmg_multifab_new(ba._h, dm._h, ncomp, ngrow, nodal_dir, precision, ctypes.byref(h)))
        self._h = h
        self.ba, self.ncomp, self.ngrow, self.nodal_dir, self.precision = ba, ncomp, ngrow, nodal_dir, precision
        self.dtype = np.float64 if precision == 8 else np.float32

    def __del__(self):
        if getattr(self, "_h", None) and capi._lib is not None:
            capi.lib().mlmg_multifab_delete(self._h)

    def fab_box(self, i):
        b = self.ba[i]
        lo = [x - self.ngrow for x in b.lo]
        hi = [x + self.ngrow for x in b.hi]
        if self.nodal_dir >= 0:
            hi[self.nodal_dir] += 1
        return Box(lo, hi)

    def fab_shape(self, i):
        n = self.fab_box(i).length()
        return (self.ncomp, n[2], n[1], n[0]) if self.ncomp > 1 else (n[2], n[1], n[0])

    def set_fab(self, i, arr):
        a = np.ascontiguousarray(arr, dtype=self.dtype)
        assert a.size == int(np.prod(self.fab_shape(i)))
        check(capi.lib().mlmg_multifab_upload(self._h, int(i), a.ctypes.data))

    def get_fab(self, i):
        a = np.empty(self.fab_shape(i), dtype=self.dtype)
        check(capi.lib().mlmg_multifab_download(self._h, int(i), a.ctypes.data))
        return a

    def set_global(self, arr, lo=(0, 0, 0)):
        """Fill every FAB from a whole-domain array (nz, ny, nx) whose lowest
        cell is ``lo`` (ghost cells are filled where the array covers them)."""
        a = np.ascontiguousarray(arr, dtype=self.dtype)
        n = (a.shape[2], a.shape[1], a.shape[0])
        check(capi.lib().mlmg_multifab_upload_global(self._h, a.ctypes.data, _i3(lo), _i3(n)))

    def get_global(self, shape_zyx, lo=(0, 0, 0), out=None):
        a = out if out is not None else np.zeros(shape_zyx, dtype=self.dtype)
        n = (a.shape[2], a.shape[1], a.shape[0])
        check(capi.lib().mlmg_multifab_download_global(self._h, a.ctypes.data, _i3(lo), _i3(n)))
        return a

    def setVal(self, v):
        check(capi.lib().mlmg_multifab_setval(self._h, float(v)))

    def FillBoundary(self, geom, cross=False):
        check(capi.lib().mlmg_multifab_fill_boundary(self._h, geom._h, int(bool(cross))))

    def norminf(self):
        v = ctypes.c_double()
        check(capi.lib().mlmg_multifab_norminf(self._h, ctypes.byref(v)))
        return v.value


class LPInfo:
    """amrex::LPInfo (Src/LinearSolvers/MLMG/AMReX_MLLinOp.H:34-83)."""

    def __init__(self):
        self.agglomeration, self.consolidation = True, True
        self.agg_grid_size, self.con_grid_size = -1, -1
        self.max_coarsening_level = 30

    def setAgglomeration(self, x):
        self.agglomeration = bool(x); return self

    def setConsolidation(self, x):
        self.consolidation = bool(x); return self

    def setAgglomerationGridSize(self, x):
        self.agg_grid_size = int(x); return self

    def setConsolidationGridSize(self, x):
        self.con_grid_size = int(x); return self

    def setMaxCoarseningLevel(self, n):
        self.max_coarsening_level = int(n); return self

    def _c(self):
        return capi.LPInfoC(int(self.agglomeration), int(self.consolidation), self.agg_grid_size,
                            self.con_grid_size, self.max_coarsening_level)


class _LinOp:
    _ctor = None

    def __init__(self, geom, ba, dm, info=None):
        geoms = geom if isinstance(geom, (list, tuple)) else [geom]
        bas = ba if isinstance(ba, (list, tuple)) else [ba]
        dms = dm if isinstance(dm, (list, tuple)) else [dm]
        n = len(geoms)
        G = (ctypes.c_void_p * n)(*[g._h for g in geoms])
        B = (ctypes.c_void_p * n)(*[b._h for b in bas])
        D = (ctypes.c_void_p * n)(*[d._h for d in dms])
        h = ctypes.c_void_p()
        inf = (info or LPInfo())._c()
        check(getattr(capi.lib(), self._ctor)(n, G, B, D, ctypes.byref(inf), ctypes.byref(h)))
        self._h = h
        self._keep = (geoms, bas, dms)

    def __del__(self):
        if getattr(self, "_h", None) and capi._lib is not None:
            capi.lib().mlmg_linop_delete(self._h)

    def setDomainBC(self, lobc, hibc):
        check(capi.lib().mlmg_linop_set_domain_bc(self._h, _i3(lobc), _i3(hibc)))

    def setLevelBC(self, amrlev, mf):
        check(capi.lib().mlmg_linop_set_level_bc(self._h, amrlev, None if mf is None else mf._h))

    def setMaxOrder(self, o):
        check(capi.lib().mlmg_linop_set_maxorder(self._h, int(o)))

    def setCoarseFineBC(self, crse, crse_ratio):
        """MLLinOp::setCoarseFineBC: coarse data for the coarse/fine faces of
        a level that does not cover its domain (values taken at this call)."""
        check(capi.lib().mlmg_linop_set_coarse_fine_bc(self._h, None if crse is None else crse._h, int(crse_ratio)))

    def NMGLevels(self, amrlev=0):
        return capi.lib().mlmg_linop_num_mg_levels(self._h)

    def NAMRLevels(self):
        return capi.lib().mlmg_linop_num_amr_levels(self._h)


class MLPoisson(_LinOp):
    _ctor = "mlmg_linop_new_poisson"


class MLABecLaplacian(_LinOp):
    """alpha a phi - beta div(b grad phi)."""
    _ctor = "mlmg_linop_new_abeclap"

    def setScalars(self, a, b):
        check(capi.lib().mlmg_abeclap_set_scalars(self._h, float(a), float(b)))

    def setACoeffs(self, amrlev, a):
        if isinstance(a, MultiFab):
            check(capi.lib().mlmg_abeclap_set_acoeffs(self._h, amrlev, a._h))
        else:
            check(capi.lib().mlmg_abeclap_set_acoeffs_const(self._h, amrlev, float(a)))

    def setBCoeffs(self, amrlev, b):
        if isinstance(b, (list, tuple)):
            arr = (ctypes.c_void_p * 3)(*[x._h for x in b])
            check(capi.lib().mlmg_abeclap_set_bcoeffs(self._h, amrlev, arr))
        else:
            check(capi.lib().mlmg_abeclap_set_bcoeffs_const(self._h, amrlev, float(b)))


class MLMG:
    """amrex::MLMG(linop): solve, apply, setters and getters."""

    def __init__(self, linop):
        h = ctypes.c_void_p()
        check(capi.lib().mlmg_new(linop._h, ctypes.byref(h)))
        self._h = h
        self.linop = linop

    def __del__(self):
        if getattr(self, "_h", None) and capi._lib is not None:
            capi.lib().mlmg_delete(self._h)

    def _set(self, name, v):
        check(getattr(capi.lib(), name)(self._h, v))

    def setVerbose(self, v): self._set("mlmg_set_verbose", int(v))
    def setMaxIter(self, n): self._set("mlmg_set_max_iter", int(n))
    def setMaxFmgIter(self, n): self._set("mlmg_set_max_fmg_iter", int(n))
    def setFixedIter(self, n): self._set("mlmg_set_fixed_iter", int(n))
    def setPreSmooth(self, n): self._set("mlmg_set_pre_smooth", int(n))
    def setPostSmooth(self, n): self._set("mlmg_set_post_smooth", int(n))
    def setFinalSmooth(self, n): self._set("mlmg_set_final_smooth", int(n))
    def setBottomSmooth(self, n): self._set("mlmg_set_bottom_smooth", int(n))
    def setBottomSolver(self, s): self._set("mlmg_set_bottom_solver", int(s))
    def setBottomMaxIter(self, n): self._set("mlmg_set_bottom_max_iter", int(n))
    def setBottomTolerance(self, t): self._set("mlmg_set_bottom_tolerance", float(t))
    def setBottomToleranceAbs(self, t): self._set("mlmg_set_bottom_tolerance_abs", float(t))
    def setAlwaysUseBNorm(self, f): self._set("mlmg_set_always_use_bnorm", int(f))
    def setFinalFillBC(self, f): self._set("mlmg_set_final_fill_bc", int(f))
    def setPrecision(self, mode): self._set("mlmg_set_precision", {"fp64": 0, "mixed": 1}.get(mode, mode))
    def setGraph(self, on): self._set("mlmg_set_graph", int(bool(on)))
    def setFusedSmoother(self, on): self._set("mlmg_set_fused_smoother", int(bool(on)))
    def setTimeKernels(self, on): self._set("mlmg_set_time_kernels", int(bool(on)))

    def setOption(self, name, value):
        """Engine tuning knob by name (coarse_block, coarse_cells, merge_boxes, march_sweep, ...)."""
        check(capi.lib().mlmg_set_option(self._h, name.encode(), float(value)))

    def smootherStats(self, reset=False):
        """(total ms, launches, algorithmic bytes per launch) of the
        finest-level smoother since the last reset."""
        ms, n, b = ctypes.c_double(), ctypes.c_longlong(), ctypes.c_double()
        check(capi.lib().mlmg_get_smoother_stats(self._h, ctypes.byref(ms), ctypes.byref(n), ctypes.byref(b),
                                                 int(bool(reset))))
        return ms.value, n.value, b.value

    def residualStats(self, reset=False):
        """(total ms, launches, algorithmic bytes, FP64 operations per launch)
        of the mixed path's FP64 outer residual since the last reset."""
        ms, n, b, f = ctypes.c_double(), ctypes.c_longlong(), ctypes.c_double(), ctypes.c_double()
        check(capi.lib().mlmg_get_residual_stats(self._h, ctypes.byref(ms), ctypes.byref(n), ctypes.byref(b),
                                                 ctypes.byref(f), int(bool(reset))))
        return ms.value, n.value, b.value, f.value

    def solve(self, sol, rhs, tol_rel, tol_abs):
        """Returns the final residual max-norm; raises MLMGError unless the
        solve converged (or ran its fixed iteration count)."""
        sols = sol if isinstance(sol, (list, tuple)) else [sol]
        rhss = rhs if isinstance(rhs, (list, tuple)) else [rhs]
        r = ctypes.c_double()
        if len(sols) > 1:
            # composite solve over the AMR levels (MLMG::solve with one MultiFab per level)
            S = (ctypes.c_void_p * len(sols))(*[m._h for m in sols])
            R = (ctypes.c_void_p * len(rhss))(*[m._h for m in rhss])
            rc = capi.lib().mlmg_solve_levels(self._h, S, R, float(tol_rel), float(tol_abs), ctypes.byref(r))
        else:
            rc = capi.lib().mlmg_solve(self._h, sols[0]._h, rhss[0]._h, float(tol_rel), float(tol_abs),
                                       ctypes.byref(r))
        if rc != 0:
            raise MLMGError(rc, capi.lib().mlmg_last_error().decode())
        return r.value

    def solve_status(self, sol, rhs, tol_rel, tol_abs):
        r = ctypes.c_double()
        rc = capi.lib().mlmg_solve(self._h, sol._h, rhs._h, float(tol_rel), float(tol_abs), ctypes.byref(r))
        return rc, r.value

    def autotune(self, sol, rhs, vcycles=2):
        """Time the candidate smoother layouts on this problem and keep the
        fastest.  Returns (best ms for `vcycles` V-cycles, report text)."""
        ms = ctypes.c_double()
        check(capi.lib().mlmg_autotune(self._h, sol._h, rhs._h, int(vcycles), ctypes.byref(ms)))
        return ms.value, capi.lib().mlmg_autotune_report(self._h).decode()

    def getFluxes(self, flux, sol):
        """MLMG::getFluxes of ``sol`` into three face-centred MultiFabs."""
        F = (ctypes.c_void_p * 3)(*[(m._h if m is not None else None) for m in flux])
        check(capi.lib().mlmg_get_fluxes(self._h, sol._h, F))

    def getGradSolution(self, grad, sol):
        """MLMG::getGradSolution of ``sol`` into three face-centred MultiFabs."""
        G = (ctypes.c_void_p * 3)(*[(m._h if m is not None else None) for m in grad])
        check(capi.lib().mlmg_get_grad_solution(self._h, sol._h, G))

    def adjointGrad(self, sol, dJdphi, tol_rel, tol_abs, dJdf, dJdb=None, dJda=None):
        """Adjoint gradients of J(phi) at the solution ``sol``: solves
        A^T lambda = dJdphi, writes dJ/df = lambda into ``dJdf`` and, for
        MLABecLaplacian, dJ/db into the three face MultiFabs ``dJdb`` and
        dJ/da into ``dJda``.  Returns the adjoint solve's final residual."""
        B = None
        if dJdb is not None:
            B = (ctypes.c_void_p * 3)(*[(m._h if m is not None else None) for m in dJdb])
        rc = capi.lib().mlmg_adjoint_grad(self._h, sol._h, dJdphi._h, float(tol_rel), float(tol_abs), dJdf._h, B,
                                          dJda._h if dJda is not None else None)
        if rc != 0:
            raise MLMGError(rc, capi.lib().mlmg_last_error().decode())
        return capi.lib().mlmg_get_final_residual(self._h)

    def compResidual(self, res, sol, rhs):
        """MLMG::compResidual: res = rhs - L(sol) on every AMR level (lists
        of one MultiFab per level, or single MultiFabs)."""
        lists = [x if isinstance(x, (list, tuple)) else [x] for x in (res, sol, rhs)]
        arrs = [(ctypes.c_void_p * len(v))(*[m._h for m in v]) for v in lists]
        check(capi.lib().mlmg_comp_residual(self._h, *arrs))

    def apply(self, out, inp):
        outs = out if isinstance(out, (list, tuple)) else [out]
        ins = inp if isinstance(inp, (list, tuple)) else [inp]
        check(capi.lib().mlmg_apply(self._h, outs[0]._h, ins[0]._h))

    def getNumIters(self):
        return capi.lib().mlmg_get_num_iters(self._h)

    def getResidualHistory(self):
        n = self.getNumIters()
        a = (ctypes.c_double * max(n, 1))()
        capi.lib().mlmg_get_residual_history(self._h, a, n)
        return list(a[:n])

    def getNumCGIters(self):
        """BiCGStab iterations of every bottom solve (F-cycles make several
        per MLMG iteration), as MLMG::getNumCGIters."""
        one = (ctypes.c_int * 1)()
        n = capi.lib().mlmg_get_num_cg_iters(self._h, one, 0)
        a = (ctypes.c_int * max(n, 1))()
        capi.lib().mlmg_get_num_cg_iters(self._h, a, n)
        return list(a[:n])

    def getInitResidual(self):
        return capi.lib().mlmg_get_init_residual(self._h)

    def getFinalResidual(self):
        return capi.lib().mlmg_get_final_residual(self._h)

    def getInitRHS(self):
        return capi.lib().mlmg_get_init_rhs(self._h)

    def solveTimeMs(self):
        return capi.lib().mlmg_get_solve_time_ms(self._h)


def solve_batched(solvers, sols, rhss, tol_rel, tol_abs):
    """Independent solves run together (one launch per V-cycle stage).
    Returns the per-solve statuses."""
    n = len(solvers)
    S = (ctypes.c_void_p * n)(*[s._h for s in solvers])
    X = (ctypes.c_void_p * n)(*[m._h for m in sols])
    B = (ctypes.c_void_p * n)(*[m._h for m in rhss])
    st = (ctypes.c_int * n)()
    rc = capi.lib().mlmg_solve_batched(n, S, X, B, float(tol_rel), float(tol_abs), st)
    if rc < 0 and rc != -2 and all(v == 0 for v in st):
        raise MLMGError(rc, capi.lib().mlmg_last_error().decode())
    return list(st)


def kernel_launches(reset=False):
    return capi.lib().mlmg_kernel_launches(int(bool(reset)))


def check_bit_conversions(n, seed=1):
    """({kind: mismatches}, {kind: first differing input}) over the device's
    n test cases of the integer-assembled FP64 -> FP32 and FP32 -> FP64
    conversions and |x| against the hardware's."""
    bad = (ctypes.c_longlong * 3)()
    first = (ctypes.c_ulonglong * 3)()
    check(capi.lib().mlmg_check_bit_conversions(int(n), int(seed), bad, first))
    kinds = ("f64_to_f32", "f32_to_f64", "abs")
    return dict(zip(kinds, list(bad))), {k: hex(v) for k, v in zip(kinds, list(first)) if v}


def fp64_fma_rate():
    """The GPU's FP64 FMA throughput in TFLOP/s, measured by one
    register-resident FMA kernel (the FP64 roofline of the outer residual)."""
    v = ctypes.c_double(0.0)
    rc = capi.lib().mlmg_fp64_fma_rate(ctypes.byref(v))
    if rc < 0:
        raise MLMGError(rc, capi.lib().mlmg_last_error().decode())
    return v.value
