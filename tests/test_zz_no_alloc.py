"""The allocation-free StabilityTester reduction, hlbg_reduce_noalloc.

Callers that must not allocate device memory once their time loop runs (a host
framework that reserved its whole device budget up front, or one for which a
cudaMalloc inside the loop would synchronise the device) use this variant; its
scratch is a fixed static device array, so it rejects geometries above its slot
limit.  Checked through the C ABI against hlbg_reduce, the entry point that
allocates, on two calls in a row and again after more steps.  This file is
collected last so that a run stopping at the first failure has run every other
test already.
"""
import ctypes as C

import pytest

from hemelb_gb300 import capi, cases

pytestmark = pytest.mark.gpu

REL = 1e-12  # tolerance of the reduction checks in tests/test_gpu_parity.py


def _close(a, b):
    return abs(a - b) <= REL * max(abs(a), abs(b)) + 1e-15


def _both(lib, ctx):
    ref = capi.Stats()
    rc_ref = lib.hlbg_reduce(ctx, C.byref(ref))
    new = capi.Stats()
    rc_new = lib.hlbg_reduce_noalloc(ctx, C.byref(new))
    return rc_ref, ref, rc_new, new


@pytest.mark.parametrize("precision", [capi.FP64, capi.FP32DEV])
def test_noalloc_reduce_matches_reduce(precision):
    lib = capi.load()
    c = cases.pipe(radius=6.0, length=30)
    s = c.solver(precision)
    s.SetInitialConditions()
    s.DoTimeStep(25)
    assert s.n_slots <= capi.NOALLOC_MAX_SLOTS
    for _ in range(2):  # two calls in a row on the same state, then after more steps
        for _call in range(2):
            rc_ref, ref, rc_new, new = _both(lib, s.ctx)
            assert rc_ref == rc_new == capi.HLBG_OK, capi.load().hlbg_last_error(s.ctx)
            assert _close(new.mass, ref.mass)
            assert _close(new.max_du, ref.max_du)
            assert _close(new.min_f, ref.min_f)
            assert new.unstable_sites == ref.unstable_sites == 0
            assert new.time_step == ref.time_step
        s.DoTimeStep(9)


def test_noalloc_reduce_reports_instability_like_reduce():
    lib = capi.load()
    c = cases.pipe(radius=5.0, length=20)
    s = c.solver()
    s.SetInitialConditions()
    s.DoTimeStep(5)
    f = s.GetFOld()
    f[3, 7] = -1.0
    s.PutF(f, 0)
    rc_ref, ref, rc_new, new = _both(lib, s.ctx)
    assert rc_ref == rc_new == capi.HLBG_ERR_UNSTABLE
    assert new.unstable_sites == ref.unstable_sites == 1


def test_noalloc_reduce_rejects_geometries_above_its_limit():
    lib = capi.load()
    c = cases.tree(seed=7, box_sites=1280, n_roots=1, depth=7, root_radius=60.0, precision=capi.FP16)
    s = c.solver()
    assert s.n_slots > capi.NOALLOC_MAX_SLOTS
    s.SetInitialConditions()
    st = capi.Stats()
    rc = lib.hlbg_reduce_noalloc(s.ctx, C.byref(st))
    assert rc == capi.HLBG_ERR_INVAL
    assert b"exceed its limit" in lib.hlbg_last_error(s.ctx)
    s.close()
