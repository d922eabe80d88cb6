"""CPU-side checks of the C ABI library: it loads, exports every entry point
declared in include/*.h, and its host logic (BoxArray::maxSize, the MG
hierarchy, argument checking) matches the reference.  No kernel runs here."""
import ctypes
import os
import re

import pytest

from amrex_gb300 import build as libbuild
from amrex_gb300 import capi
from tests.golden import load

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def lib():
    libbuild.build()
    return capi.lib()


def declared_symbols():
    names = set()
    inc = os.path.join(ROOT, "include")
    for f in os.listdir(inc):
        if f.endswith(".h"):
            text = open(os.path.join(inc, f)).read()
            names |= set(re.findall(r"\b(mlmg_[a-z0-9_]+)\s*\(", text))
    return sorted(names)


def test_every_declared_symbol_is_exported(lib):
    names = declared_symbols()
    assert len(names) > 50
    for n in names:
        assert hasattr(lib, n), n


def test_python_binding_covers_the_header():
    assert set(declared_symbols()) <= set(capi.exported_symbols())


@pytest.mark.parametrize("name", [n for n in load.names("hier_") if "irregular" not in n])
def test_boxarray_maxsize_matches_reference(lib, name):
    g = load.load(name)
    c = g["case"]
    h = ctypes.c_void_p()
    n = c["n"]
    capi.check(lib.mlmg_boxarray_new_domain(capi.I3(0, 0, 0), capi.I3(n[0] - 1, n[1] - 1, n[2] - 1), ctypes.byref(h)))
    m = c["max_grid_size"]
    capi.check(lib.mlmg_boxarray_maxsize(h, capi.I3(m, m, m)))
    boxes = []
    for i in range(lib.mlmg_boxarray_size(h)):
        lo, hi = capi.I3(), capi.I3()
        capi.check(lib.mlmg_boxarray_get(h, i, lo, hi))
        boxes.append(tuple(lo) + tuple(hi))
    lib.mlmg_boxarray_delete(h)
    assert boxes == g["hier"][0]


@pytest.mark.parametrize("name", load.names("hier_"))
def test_mg_level_count_matches_reference(lib, name):
    import amrex_gb300 as ag
    g = load.load(name)
    c = g["case"]
    n = c["n"]
    domain = ag.Box((0, 0, 0), (n[0] - 1, n[1] - 1, n[2] - 1))
    if c.get("boxes"):
        ba = ag.BoxArray([ag.Box(b[:3], b[3:]) for b in c["boxes"]])
    else:
        ba = ag.BoxArray(domain).maxSize(c["max_grid_size"])
    dm = ag.DistributionMapping(ba)
    geom = ag.Geometry(domain)
    info = ag.LPInfo().setAgglomeration(c["agg"]).setConsolidation(c["con"]) \
        .setAgglomerationGridSize(c["agg_grid_size"]).setConsolidationGridSize(c["con_grid_size"])
    op = ag.MLPoisson(geom, ba, dm, info)
    assert op.NMGLevels() == len(g["hier"])


def test_bad_arguments_return_errors(lib):
    h = ctypes.c_void_p()
    # overlapping boxes are rejected on the host
    boxes = (ctypes.c_int * 12)(0, 0, 0, 7, 7, 7, 4, 4, 4, 11, 11, 11)
    rc = lib.mlmg_boxarray_new(boxes, 2, ctypes.byref(h))
    assert rc == -1 and b"overlap" in lib.mlmg_last_error()
    assert lib.mlmg_boxarray_maxsize(None, capi.I3(8, 8, 8)) == -1
    # composite solves are refused, not faked
    import amrex_gb300 as ag
    d = ag.Box((0, 0, 0), (15, 15, 15))
    ba = ag.BoxArray(d)
    dm = ag.DistributionMapping(ba)
    geom = ag.Geometry(d)
    G = (ctypes.c_void_p * 2)(geom._h, geom._h)
    B = (ctypes.c_void_p * 2)(ba._h, ba._h)
    D = (ctypes.c_void_p * 2)(dm._h, dm._h)
    assert lib.mlmg_linop_new_poisson(2, G, B, D, None, ctypes.byref(h)) == -4
