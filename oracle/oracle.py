"""ctypes binding of the CPU oracle (oracle/liboracle.so) -- TEST INFRASTRUCTURE.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use this.
It mirrors the reference's own layout: AoS distributions of N*Q+1 doubles in
contiguous site order with the rubbish slot at N*Q.
"""
from __future__ import annotations

import ctypes as C
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))

from hemelb_gb300 import capi  # noqa: E402  (struct layouts of the shared header)

ORDER_SCALAR, ORDER_SSE3 = 0, 1


class Domain(C.Structure):
    _fields_ = [
        ("q", C.c_int32), ("n", C.c_int64), ("type_count", C.c_int64 * 6),
        ("nbr", C.POINTER(C.c_int64)), ("wall_mask", C.POINTER(C.c_uint32)),
        ("iolet_mask", C.POINTER(C.c_uint32)), ("iolet_id", C.POINTER(C.c_int32)),
        ("site_type", C.POINTER(C.c_int8)), ("cut", C.POINTER(C.c_double)),
        ("coords", C.POINTER(C.c_int64)), ("slot", C.POINTER(C.c_int64)),
    ]


class Params(C.Structure):
    _fields_ = [
        ("q", C.c_int32), ("kernel", C.c_int32), ("wall", C.c_int32), ("inlet", C.c_int32),
        ("outlet", C.c_int32), ("order", C.c_int32), ("tau", C.c_double),
        ("n_inlets", C.c_int32), ("n_outlets", C.c_int32),
        ("inlets", C.POINTER(capi.Iolet)), ("outlets", C.POINTER(capi.Iolet)),
    ]


_lib = None


def load():
    global _lib
    if _lib is None:
        from oracle.build import build
        lib = C.CDLL(build())
        P = C.POINTER
        lib.hlbo_domain_build.argtypes = [P(capi.Geometry), P(Domain)]
        lib.hlbo_domain_free.argtypes = [P(Domain)]
        lib.hlbo_domain_free.restype = None
        lib.hlbo_init_equilibrium.argtypes = [P(Domain), P(Params), C.c_double, C.c_double,
                                              C.c_double, C.c_double, P(C.c_double)]
        lib.hlbo_init_equilibrium.restype = None
        for nm in ("hlbo_step",):
            getattr(lib, nm).argtypes = [P(Domain), P(Params), P(C.c_double), P(C.c_double),
                                         C.c_uint64, C.c_int]
            getattr(lib, nm).restype = None
        lib.hlbo_stream_and_collide.argtypes = [P(Domain), P(Params), P(C.c_double), P(C.c_double),
                                                C.c_uint64, C.c_int64, C.c_int64, C.c_int]
        lib.hlbo_stream_and_collide.restype = None
        lib.hlbo_post_step.argtypes = [P(Domain), P(Params), P(C.c_double), C.c_int64, C.c_int64,
                                       C.c_int]
        lib.hlbo_post_step.restype = None
        lib.hlbo_macro.argtypes = [P(Domain), P(Params), P(C.c_double), P(C.c_double), P(C.c_double)]
        lib.hlbo_macro.restype = None
        lib.hlbo_collide_site.argtypes = [P(Params), P(C.c_double), P(C.c_double), P(C.c_double),
                                          P(C.c_double), P(C.c_double), P(C.c_double)]
        lib.hlbo_collide_site.restype = None
        lib.hlbo_feq.argtypes = [P(Params), C.c_double, P(C.c_double), P(C.c_double)]
        lib.hlbo_feq.restype = None
        lib.hlbo_cosine_density.argtypes = [P(capi.Iolet), C.c_uint64, C.c_double]
        lib.hlbo_cosine_density.restype = C.c_double
        lib.hlbo_min_density.argtypes = [P(Params)]
        lib.hlbo_min_density.restype = C.c_double
        lib.hlbo_iolet_velocity.argtypes = [P(capi.Iolet), P(C.c_double), C.c_uint64, P(C.c_double)]
        lib.hlbo_iolet_velocity.restype = None
        _lib = lib
    return _lib


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


class OracleLBM:
    """The reference's per-step sweep on the CPU, over the same sparse geometry."""

    def __init__(self, geom_view: capi.Geometry, params, inlets=(), outlets=(),
                 order: int = ORDER_SCALAR, q: int | None = None):
        self.lib = load()
        self.dom = Domain()
        rc = self.lib.hlbo_domain_build(C.byref(geom_view), C.byref(self.dom))
        if rc != 0:
            raise RuntimeError("oracle domain build failed: %d" % rc)
        self.q = self.dom.q
        self.n = self.dom.n
        self._in = (capi.Iolet * max(1, len(inlets)))(*inlets)
        self._out = (capi.Iolet * max(1, len(outlets)))(*outlets)
        self.p = Params()
        self.p.q = self.q
        self.p.kernel, self.p.wall = params.kernel, params.wall
        self.p.inlet, self.p.outlet = params.inlet, params.outlet
        self.p.order = order
        self.p.tau = params.tau
        self.p.n_inlets, self.p.n_outlets = len(inlets), len(outlets)
        self.p.inlets = C.cast(self._in, C.POINTER(capi.Iolet))
        self.p.outlets = C.cast(self._out, C.POINTER(capi.Iolet))
        self.f_old = np.zeros(self.n * self.q + 1)
        self.f_new = np.zeros(self.n * self.q + 1)
        self.t1 = 1
        self.type_count = tuple(self.dom.type_count)

    def close(self):
        if self.dom.nbr:
            self.lib.hlbo_domain_free(C.byref(self.dom))

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def arrays(self):
        n, q = self.n, self.q
        return {
            "nbr": np.ctypeslib.as_array(self.dom.nbr, (n * q,)),
            "wall_mask": np.ctypeslib.as_array(self.dom.wall_mask, (n,)),
            "iolet_mask": np.ctypeslib.as_array(self.dom.iolet_mask, (n,)),
            "iolet_id": np.ctypeslib.as_array(self.dom.iolet_id, (n,)),
            "cut": np.ctypeslib.as_array(self.dom.cut, (n * (q - 1),)),
            "coords": np.ctypeslib.as_array(self.dom.coords, (n * 3,)).reshape(n, 3),
            "slot": np.ctypeslib.as_array(self.dom.slot, (n,)),
        }

    def set_equilibrium(self, rho=1.0, u=(0.0, 0.0, 0.0)):
        self.lib.hlbo_init_equilibrium(C.byref(self.dom), C.byref(self.p), rho, *u, _dp(self.f_old))
        self.f_new[:] = self.f_old
        self.t1 = 1

    def step(self, n: int = 1, threads: int = 1):
        for _ in range(n):
            self.lib.hlbo_step(C.byref(self.dom), C.byref(self.p), _dp(self.f_old), _dp(self.f_new),
                               self.t1, threads)
            self.f_old, self.f_new = self.f_new, self.f_old
            self.t1 += 1

    def stream_and_collide(self, first, count, threads=1):
        self.lib.hlbo_stream_and_collide(C.byref(self.dom), C.byref(self.p), _dp(self.f_old),
                                         _dp(self.f_new), self.t1, first, count, threads)

    def post_step(self, first, count, threads=1):
        self.lib.hlbo_post_step(C.byref(self.dom), C.byref(self.p), _dp(self.f_new), first, count,
                                threads)

    def swap(self):
        self.f_old, self.f_new = self.f_new, self.f_old
        self.t1 += 1

    def fold(self):
        return self.f_old[: self.n * self.q].reshape(self.n, self.q)

    def fnew(self):
        return self.f_new[: self.n * self.q].reshape(self.n, self.q)

    def macro(self, f=None):
        f = self.f_old if f is None else f
        rho = np.empty(self.n)
        u = np.empty(self.n * 3)
        self.lib.hlbo_macro(C.byref(self.dom), C.byref(self.p), _dp(f), _dp(rho), _dp(u))
        return rho, u.reshape(self.n, 3)
