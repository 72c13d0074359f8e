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
import json
import os
import subprocess
import sys

import pytest

from hemelb_gb300 import capi, cases

pytestmark = pytest.mark.gpu

REL = 1e-12  # tolerance of the reduction checks in tests/test_gpu_parity.py
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


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


_FREE_BYTES_SCRIPT = r"""
import ctypes as C, json, sys
sys.path.insert(0, sys.argv[1])
from hemelb_gb300 import capi, cases
lib = capi.load()
cu = C.CDLL("libcuda.so.1")
cu.cuMemGetInfo_v2.argtypes = [C.POINTER(C.c_size_t), C.POINTER(C.c_size_t)]

def free_bytes():
    f, t = C.c_size_t(), C.c_size_t()
    assert cu.cuMemGetInfo_v2(C.byref(f), C.byref(t)) == 0
    return f.value

c = cases.pipe(radius=6.0, length=30)
s = c.solver(capi.FP32DEV)
s.SetInitialConditions()
s.DoTimeStep(5)
before = free_bytes()
rcs = []
for _ in range(4):
    st = capi.Stats()
    rcs.append(lib.hlbg_reduce_noalloc(s.ctx, C.byref(st)))
    s.DoTimeStep(1)
after = free_bytes()
print(json.dumps({"before": before, "after": after, "rcs": rcs}))
"""


def test_noalloc_reduce_takes_no_device_memory_under_lazy_loading():
    """With lazy module loading the library's device code is placed on the GPU on
    first use; the context's creation must have done that for the static scratch
    array, so the first hlbg_reduce_noalloc call (and every later one) leaves the
    device's free memory unchanged.  Fresh process, CUDA_MODULE_LOADING=LAZY."""
    env = dict(os.environ, CUDA_MODULE_LOADING="LAZY")
    r = subprocess.run([sys.executable, "-c", _FREE_BYTES_SCRIPT, ROOT], env=env, capture_output=True,
                       text=True, timeout=300)
    assert r.returncode == 0, r.stderr[-2000:]
    out = json.loads(r.stdout.strip().splitlines()[-1])
    assert out["rcs"] == [capi.HLBG_OK] * 4
    assert out["after"] == out["before"], out
