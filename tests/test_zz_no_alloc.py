"""The allocation-free max-norm entry point (mlmg_multifab_norminf_noalloc)
against the allocating one (mlmg_multifab_norminf), through the C ABI.

It exists for callers that cannot allocate device memory -- a framework whose
caching allocator already holds the HBM, or a time-step loop where the device-
wide synchronisation of cudaMalloc/cudaFree is not acceptable.  Its scratch is
a static device array, so this file also checks that consecutive calls do not
see each other's results and that the box limit is enforced.  The file is
collected last so that a failure here leaves every other test already run."""
import ctypes

import numpy as np
import pytest

import amrex_gb300 as ag
from amrex_gb300 import capi

pytestmark = pytest.mark.gpu


def _noalloc(mf):
    v = ctypes.c_double(-1.0)
    rc = capi.lib().mlmg_multifab_norminf_noalloc(mf._h, ctypes.byref(v))
    return rc, v.value


def _ragged_multifab(precision):
    n = (40, 24, 32)
    domain = ag.Box((0, 0, 0), (n[0] - 1, n[1] - 1, n[2] - 1))
    ba = ag.BoxArray(domain).maxSize(16)
    dm = ag.DistributionMapping(ba)
    mf = ag.MultiFab(ba, dm, 1, 1, precision=precision)
    return mf, n


@pytest.mark.parametrize("precision", [8, 4])
def test_noalloc_norminf_equals_allocating_norminf_on_two_calls(precision):
    mf, n = _ragged_multifab(precision)
    rng = np.random.default_rng(7)
    grown = np.full((n[2] + 2, n[1] + 2, n[0] + 2), 1.0e6)   # domain ghosts: must not count
    grown[1:-1, 1:-1, 1:-1] = rng.uniform(-3.0, 3.0, size=(n[2], n[1], n[0]))
    for scale in (1.0, 0.25):   # the second call has a smaller maximum: the result word must be cleared
        mf.set_global(grown * np.where(np.abs(grown) < 1e5, scale, 1.0), lo=(-1, -1, -1))
        ref = mf.norminf()
        rc, got = _noalloc(mf)
        assert rc == 0, capi.lib().mlmg_last_error()
        assert got == ref            # a maximum is exact: no tolerance needed
        assert got < 1e5


def test_noalloc_norminf_rejects_more_boxes_than_its_scratch_holds():
    domain = ag.Box((0, 0, 0), (67, 63, 63))
    ba = ag.BoxArray(domain).maxSize(4)       # 17 * 16 * 16 = 4352 boxes
    assert ba.size() > 4096
    dm = ag.DistributionMapping(ba)
    mf = ag.MultiFab(ba, dm, 1, 0)
    rc, _ = _noalloc(mf)
    assert rc == -1
    assert b"4096" in capi.lib().mlmg_last_error()
