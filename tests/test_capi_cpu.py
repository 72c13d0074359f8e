"""CPU-side checks of the C ABI library: it loads, exports every entry point the
public header declares, and its seeded generators and host logic behave."""
import ctypes as C
import os
import re
import subprocess

import numpy as np
import pytest

from hemelb_gb300 import capi, cases
from hemelb_gb300.lbm import SyntheticGeometry
from oracle.oracle import OracleLBM
from tests.helpers import CX19, CY19, CZ19

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADERS = [os.path.join(ROOT, "include", h) for h in ("hemelb_gb300.h", "hemelb_gb300_nn.h")]


def declared_symbols():
    text = "".join(open(h).read() for h in HEADERS)
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(hlbg_[a-z0-9_]+)\s*\(", text)))


def test_library_exports_every_declared_symbol():
    syms = declared_symbols()
    assert len(syms) >= 30
    out = subprocess.run(["nm", "-D", "--defined-only", capi.LIB_PATH], capture_output=True,
                         text=True, check=True).stdout
    exported = set(re.findall(r"\bT (hlbg_[a-z0-9_]+)\b", out))
    missing = [s for s in syms if s not in exported]
    assert not missing, missing
    # and the ctypes binding declares each of them
    assert set(syms) <= set(capi.SIGNATURES), set(syms) - set(capi.SIGNATURES)


def test_library_loads_and_reports_version():
    lib = capi.load()
    assert b"sm_103a" in lib.hlbg_version()


def test_null_arguments_are_rejected_without_a_gpu():
    lib = capi.load()
    ctx = C.c_void_p()
    assert lib.hlbg_create(None, None, None, 0, None, 0, C.byref(ctx)) == capi.HLBG_ERR_INVAL
    assert lib.hlbg_step(None, 1, None) == capi.HLBG_ERR_INVAL
    assert lib.hlbg_reduce(None, None) == capi.HLBG_ERR_INVAL
    h = C.c_void_p()
    assert lib.hlbg_synth_pipe(-1.0, 10, 19, 1, C.byref(h)) == capi.HLBG_ERR_INVAL
    assert lib.hlbg_synth_pipe(5.0, 10, 27, 1, C.byref(h)) == capi.HLBG_ERR_INVAL


def test_pipe_geometry_matches_specification():
    """Radius 10, length 80: voxel centres strictly inside the radius, z in [0, 80]."""
    g = SyntheticGeometry.pipe(10.0, 80, 19, True)
    xs = np.arange(-12, 13)
    per_slice = int(((xs[:, None] ** 2 + xs[None, :] ** 2) < 100).sum())
    assert g.n_fluid == per_slice * 81 == 24705
    assert g.n_inlets == 1 and g.n_outlets == 1


def test_generators_are_deterministic():
    a = SyntheticGeometry.bifurcation(99, 8.0, 30.0, 1.0, 19, True)
    b = SyntheticGeometry.bifurcation(99, 8.0, 30.0, 1.0, 19, True)
    assert a.n_fluid == b.n_fluid
    assert np.array_equal(a.fluid_mask, b.fluid_mask)
    assert np.array_equal(a.cut_distance, b.cut_distance)
    c = SyntheticGeometry.bifurcation(100, 8.0, 30.0, 1.0, 19, True)
    assert c.n_fluid != a.n_fluid or not np.array_equal(c.fluid_mask, a.fluid_mask)


def test_link_records_are_consistent_with_fluid_map():
    """Every wall/iolet bit points at a non-fluid neighbour; every fluid site with
    a non-fluid neighbour has a record; cut distances lie in (0, 1]."""
    g = SyntheticGeometry.bifurcation(5, 7.0, 20.0, 1.0, 19, True)
    o = OracleLBM(g.view, cases.pipe(4.0, 4).params)  # domain arrays only
    a = o.arrays()
    n, q = o.n, o.q
    nbr = a["nbr"].reshape(n, q)
    rubbish = n * q
    for d in range(1, q):
        bit = np.uint32(1 << (d - 1))
        flagged = ((a["wall_mask"] & bit) | (a["iolet_mask"] & bit)) != 0
        assert np.all(nbr[flagged, d] == rubbish)
        assert np.all(flagged[nbr[:, d] == rubbish])
    cut = a["cut"].reshape(n, q - 1)
    flagged_any = (a["wall_mask"][:, None] >> np.arange(q - 1, dtype=np.uint32)) & 1
    vals = cut[flagged_any.astype(bool)]
    assert np.all((vals > 0) & (vals <= 1.0))


def test_site_order_is_reference_contiguous_order():
    """Contiguous ids are grouped by collision type 0..5 (Domain.cc:188-207)."""
    g = SyntheticGeometry.bifurcation(5, 7.0, 20.0, 1.0, 19, True)
    c = cases.pipe(4.0, 4)
    o = OracleLBM(g.view, c.params)
    a = o.arrays()
    counts = o.type_count
    assert sum(counts) == o.n == g.n_fluid
    wall = a["wall_mask"] != 0
    start = 0
    for t, cnt in enumerate(counts):
        seg = wall[start:start + cnt]
        assert np.all(seg) if t in (1, 4, 5) else not np.any(seg)
        start += cnt


def test_tree_generator_statistics():
    g = SyntheticGeometry.tree(7, 320, 1, 3, 20.0, 19, False, 0)
    assert g.n_fluid > 50_000
    assert g.n_inlets == 1 and g.n_outlets >= 2
    frac = g.n_link_sites / g.n_fluid
    assert 0.01 < frac < 0.5
    # blocks listed in Morton order
    bc = g.block_coords.astype(np.uint64)
    def morton(x, y, z):
        m = np.zeros_like(x)
        for k in range(16):
            m |= ((x >> np.uint64(k)) & np.uint64(1)) << np.uint64(3 * k + 2)
            m |= ((y >> np.uint64(k)) & np.uint64(1)) << np.uint64(3 * k + 1)
            m |= ((z >> np.uint64(k)) & np.uint64(1)) << np.uint64(3 * k)
        return m
    m = morton(bc[:, 0], bc[:, 1], bc[:, 2])
    assert np.all(np.diff(m.astype(np.int64)) > 0)


def test_d3q19_lattice_structure():
    """Vectors in {-1,0,1}, unique, inverse pairs, weights sum to one
    (Code/tests/lb/LatticeTests.cc:21)."""
    v = np.array([CX19, CY19, CZ19]).T
    assert len({tuple(r) for r in v}) == 19
    for i in range(19):
        assert (tuple(-v[i]) in {tuple(r) for r in v})
    inv = [0, 2, 1, 4, 3, 6, 5, 8, 7, 10, 9, 12, 11, 14, 13, 16, 15, 18, 17]
    assert all(np.array_equal(v[inv[i]], -v[i]) for i in range(19))
    w = np.array([1 / 3] + [1 / 18] * 6 + [1 / 36] * 12)
    assert abs(w.sum() - 1.0) < 1e-15


@pytest.mark.parametrize("kernel", [capi.KERNEL_LBGK, capi.KERNEL_TRT])
def test_collision_closed_form(kernel):
    """Oracle collide vs an independent numpy statement of the LBGK / TRT
    formulas (Code/tests/lb/LbTestsHelper.h:90-143 for LBGK)."""
    from oracle.oracle import Params, load
    lib = load()
    p = Params()
    p.q, p.kernel, p.tau = 19, kernel, 0.7
    rng = np.random.default_rng(1)
    v = np.array([CX19, CY19, CZ19], dtype=np.float64)
    w = np.array([1 / 3] + [1 / 18] * 6 + [1 / 36] * 12)
    for _ in range(20):
        f = w * (1.0 + 0.05 * rng.standard_normal(19))
        rho = np.zeros(1)
        mom = np.zeros(3)
        vel = np.zeros(3)
        feq = np.zeros(19)
        fpost = np.zeros(19)
        dp = lambda a: a.ctypes.data_as(C.POINTER(C.c_double))
        lib.hlbo_collide_site(C.byref(p), dp(f), dp(rho), dp(mom), dp(vel), dp(feq), dp(fpost))
        r = f.sum()
        m = v @ f
        cu = m @ v
        eq = w * (r - 1.5 * (m @ m) / r + 4.5 * cu ** 2 / r + 3 * cu)
        assert np.allclose(feq, eq, rtol=1e-13, atol=1e-15)
        neq = f - eq
        if kernel == capi.KERNEL_LBGK:
            expect = f - neq / 0.7
        else:
            inv = [0, 2, 1, 4, 3, 6, 5, 8, 7, 10, 9, 12, 11, 14, 13, 16, 15, 18, 17]
            tm = 0.5 + (3 / 16) / (0.7 - 0.5)
            sym = 0.5 * (neq + neq[inv])
            asym = 0.5 * (neq - neq[inv])
            expect = f - sym / 0.7 - asym / tm
        assert np.allclose(fpost, expect, rtol=1e-12, atol=1e-15)
        # mass and momentum are conserved by the collision
        assert abs(fpost.sum() - r) < 1e-14
        assert np.allclose(v @ fpost, m, atol=1e-15)
