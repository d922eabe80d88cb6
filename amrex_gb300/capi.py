"""ctypes binding of the C ABI in include/mlmg_capi.h.

The shared library is built in-tree (amrex_gb300/libamrex_gb300.so) by
``amrex_gb300.build``.  Loading fails loudly when it is missing: there is no
CPU fallback.
"""
from __future__ import annotations

import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libamrex_gb300.so")

c_int, c_double, c_void_p, c_size_t = ctypes.c_int, ctypes.c_double, ctypes.c_void_p, ctypes.c_size_t
P = ctypes.POINTER
I3 = ctypes.c_int * 3
D3 = ctypes.c_double * 3


class LPInfoC(ctypes.Structure):
    _fields_ = [("agglomeration", c_int), ("consolidation", c_int), ("agg_grid_size", c_int),
                ("con_grid_size", c_int), ("max_coarsening_level", c_int)]


# name -> (restype, argtypes)
SIGNATURES = {
    "mlmg_last_error": (ctypes.c_char_p, []),
    "mlmg_version": (c_int, []),
    "mlmg_stream": (c_void_p, []),
    "mlmg_kernel_launches": (ctypes.c_longlong, [c_int]),
    "mlmg_fp64_fma_rate": (c_int, [P(ctypes.c_double)]),
    "mlmg_check_bit_conversions": (c_int, [ctypes.c_longlong, ctypes.c_ulonglong, P(ctypes.c_longlong),
                                           P(ctypes.c_ulonglong)]),
    "mlmg_boxarray_new": (c_int, [P(c_int), c_int, P(c_void_p)]),
    "mlmg_boxarray_new_domain": (c_int, [I3, I3, P(c_void_p)]),
    "mlmg_boxarray_maxsize": (c_int, [c_void_p, I3]),
    "mlmg_boxarray_size": (c_int, [c_void_p]),
    "mlmg_boxarray_get": (c_int, [c_void_p, c_int, I3, I3]),
    "mlmg_boxarray_delete": (c_int, [c_void_p]),
    "mlmg_distromap_new": (c_int, [c_void_p, P(c_void_p)]),
    "mlmg_distromap_delete": (c_int, [c_void_p]),
    "mlmg_geometry_new": (c_int, [I3, I3, D3, D3, I3, P(c_void_p)]),
    "mlmg_geometry_delete": (c_int, [c_void_p]),
    "mlmg_multifab_new": (c_int, [c_void_p, c_void_p, c_int, c_int, c_int, c_int, P(c_void_p)]),
    "mlmg_multifab_delete": (c_int, [c_void_p]),
    "mlmg_multifab_fab_size": (c_int, [c_void_p, c_int, P(c_size_t)]),
    "mlmg_multifab_fab_ptr": (c_int, [c_void_p, c_int, P(c_void_p)]),
    "mlmg_multifab_upload": (c_int, [c_void_p, c_int, c_void_p]),
    "mlmg_multifab_download": (c_int, [c_void_p, c_int, c_void_p]),
    "mlmg_multifab_upload_global": (c_int, [c_void_p, c_void_p, I3, I3]),
    "mlmg_multifab_download_global": (c_int, [c_void_p, c_void_p, I3, I3]),
    "mlmg_multifab_setval": (c_int, [c_void_p, c_double]),
    "mlmg_multifab_fill_boundary": (c_int, [c_void_p, c_void_p, c_int]),
    "mlmg_multifab_norminf": (c_int, [c_void_p, P(c_double)]),
    "mlmg_multifab_norminf_noalloc": (c_int, [c_void_p, P(c_double)]),
    "mlmg_linop_new_poisson": (c_int, [c_int, P(c_void_p), P(c_void_p), P(c_void_p), P(LPInfoC), P(c_void_p)]),
    "mlmg_linop_new_abeclap": (c_int, [c_int, P(c_void_p), P(c_void_p), P(c_void_p), P(LPInfoC), P(c_void_p)]),
    "mlmg_linop_delete": (c_int, [c_void_p]),
    "mlmg_linop_set_domain_bc": (c_int, [c_void_p, I3, I3]),
    "mlmg_linop_set_level_bc": (c_int, [c_void_p, c_int, c_void_p]),
    "mlmg_linop_set_maxorder": (c_int, [c_void_p, c_int]),
    "mlmg_linop_set_coarse_fine_bc": (c_int, [c_void_p, c_void_p, c_int]),
    "mlmg_abeclap_set_scalars": (c_int, [c_void_p, c_double, c_double]),
    "mlmg_abeclap_set_acoeffs": (c_int, [c_void_p, c_int, c_void_p]),
    "mlmg_abeclap_set_acoeffs_const": (c_int, [c_void_p, c_int, c_double]),
    "mlmg_abeclap_set_bcoeffs": (c_int, [c_void_p, c_int, P(c_void_p)]),
    "mlmg_abeclap_set_bcoeffs_const": (c_int, [c_void_p, c_int, c_double]),
    "mlmg_linop_num_mg_levels": (c_int, [c_void_p]),
    "mlmg_linop_num_amr_levels": (c_int, [c_void_p]),
    "mlmg_new": (c_int, [c_void_p, P(c_void_p)]),
    "mlmg_delete": (c_int, [c_void_p]),
    "mlmg_set_verbose": (c_int, [c_void_p, c_int]),
    "mlmg_set_max_iter": (c_int, [c_void_p, c_int]),
    "mlmg_set_max_fmg_iter": (c_int, [c_void_p, c_int]),
    "mlmg_set_fixed_iter": (c_int, [c_void_p, c_int]),
    "mlmg_set_pre_smooth": (c_int, [c_void_p, c_int]),
    "mlmg_set_post_smooth": (c_int, [c_void_p, c_int]),
    "mlmg_set_final_smooth": (c_int, [c_void_p, c_int]),
    "mlmg_set_bottom_smooth": (c_int, [c_void_p, c_int]),
    "mlmg_set_bottom_solver": (c_int, [c_void_p, c_int]),
    "mlmg_set_bottom_max_iter": (c_int, [c_void_p, c_int]),
    "mlmg_set_bottom_tolerance": (c_int, [c_void_p, c_double]),
    "mlmg_set_bottom_tolerance_abs": (c_int, [c_void_p, c_double]),
    "mlmg_set_always_use_bnorm": (c_int, [c_void_p, c_int]),
    "mlmg_set_final_fill_bc": (c_int, [c_void_p, c_int]),
    "mlmg_set_precision": (c_int, [c_void_p, c_int]),
    "mlmg_set_graph": (c_int, [c_void_p, c_int]),
    "mlmg_set_fused_smoother": (c_int, [c_void_p, c_int]),
    "mlmg_set_time_kernels": (c_int, [c_void_p, c_int]),
    "mlmg_set_option": (c_int, [c_void_p, ctypes.c_char_p, c_double]),
    "mlmg_get_smoother_stats": (c_int, [c_void_p, P(c_double), P(ctypes.c_longlong), P(c_double), c_int]),
    "mlmg_get_residual_stats": (c_int, [c_void_p, P(ctypes.c_double), P(ctypes.c_longlong), P(ctypes.c_double),
                                        P(ctypes.c_double), c_int]),
    "mlmg_solve": (c_int, [c_void_p, c_void_p, c_void_p, c_double, c_double, P(c_double)]),
    "mlmg_solve_levels": (c_int, [c_void_p, P(c_void_p), P(c_void_p), c_double, c_double, P(c_double)]),
    "mlmg_apply": (c_int, [c_void_p, c_void_p, c_void_p]),
    "mlmg_comp_residual": (c_int, [c_void_p, c_void_p, c_void_p, c_void_p]),
    "mlmg_get_fluxes": (c_int, [c_void_p, c_void_p, P(c_void_p)]),
    "mlmg_get_grad_solution": (c_int, [c_void_p, c_void_p, P(c_void_p)]),
    "mlmg_get_num_iters": (c_int, [c_void_p]),
    "mlmg_get_residual_history": (c_int, [c_void_p, P(c_double), c_int]),
    "mlmg_get_num_cg_iters": (c_int, [c_void_p, P(c_int), c_int]),
    "mlmg_get_init_residual": (c_double, [c_void_p]),
    "mlmg_get_final_residual": (c_double, [c_void_p]),
    "mlmg_get_init_rhs": (c_double, [c_void_p]),
    "mlmg_get_solve_time_ms": (c_double, [c_void_p]),
    "mlmg_get_num_mg_levels": (c_int, [c_void_p]),
    "mlmg_solve_batched": (c_int, [c_int, P(c_void_p), P(c_void_p), P(c_void_p), c_double, c_double, P(c_int)]),
    "mlmg_autotune": (c_int, [c_void_p, c_void_p, c_void_p, c_int, P(c_double)]),
    "mlmg_autotune_report": (ctypes.c_char_p, [c_void_p]),
    "mlmg_adjoint_grad": (c_int, [c_void_p, c_void_p, c_void_p, c_double, c_double, c_void_p, P(c_void_p),
                                  c_void_p]),
}

_lib = None


class MLMGError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"[{code}] {msg}")
        self.code = code


def lib():
    """Load the library; raise if it was not built (no fallback)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"{LIB_PATH} is missing: run `python -m amrex_gb300.build` (nvcc, sm_103a)")
        L = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def check(rc, ok=(0,)):
    """Raise MLMGError for a negative (or not-OK) status."""
    if rc not in ok and rc < 0:
        raise MLMGError(rc, lib().mlmg_last_error().decode())
    return rc


def exported_symbols():
    return list(SIGNATURES)
