"""Pin the CPU oracle to the reference.

1. Against the reference's own LB code compiled here from the HemeLB sources
   (oracle/refbuild): bit-exact in both of the reference's evaluation orders
   (scalar = aarch64 build, SSE3 = x86_64 build) on geometries that exercise
   every collision type, SBB and BFL walls (with PostStep), Nash and Ladd iolets,
   D3Q19 and D3Q15, LBGK and TRT (the reference's Code/lb/kernels/TRT.h with the
   recipe's build-time patch of its two compile defects).  Skipped where the
   reference sources are absent.
2. Against golden vectors the compiled reference produced (tests/golden/*.npz,
   made by tests/golden/make_golden.py), which travel with the repository.
"""
import os

import numpy as np
import pytest

from hemelb_gb300 import capi, cases
from hemelb_gb300.lbm import LbmParameters
from oracle.oracle import ORDER_SCALAR, ORDER_SSE3, OracleLBM
from tests import golden_cases
from tests.helpers import anisotropic, four_cube

HERE = os.path.dirname(os.path.abspath(__file__))


def _ref_available():
    try:
        from oracle.refbuild.build_ref import available, build
        return available() and bool(build())
    except Exception:
        return False


needs_ref = pytest.mark.skipif(not _ref_available(), reason="reference sources not present")


def _variants():
    from oracle.refbuild.build_ref import targets
    out = [("scalar", ORDER_SCALAR)]
    if "sse3" in targets():
        out.append(("sse3", ORDER_SSE3))
    return out


def _compare_with_reference(view, params, inlets, outlets, steps, variant, order, f0=None):
    from oracle.refbuild.run_ref import run_reference
    o = OracleLBM(view, params, inlets, outlets, order=order)
    o.set_equilibrium()
    if f0 is not None:
        o.f_old[: f0.size] = f0.reshape(-1)
        o.f_new[: f0.size] = f0.reshape(-1)
    tau_used, t_end, rf_old, rf_new = run_reference(o, steps, variant)
    assert tau_used == params.tau
    o.step(steps)
    assert t_end == o.t1
    assert np.array_equal(o.f_old[:-1], rf_old[:-1])
    assert np.array_equal(o.f_new[:-1], rf_new[:-1])
    return o


@needs_ref
def test_pipe_sbb_nash_matches_reference():
    c = cases.pipe(radius=6.0, length=30)
    for variant, order in _variants():
        _compare_with_reference(c.geometry.view, c.params, c.inlets, c.outlets, 60, variant, order)


@needs_ref
def test_bifurcation_bfl_ladd_nash_matches_reference():
    """BFL walls (StreamLink eq. 5b and PostStep eq. 5a), parabolic Ladd inlet with
    warm-up, Nash outlets, LBGK; all six collision types populated."""
    g, inl, outl, p = golden_cases.bifurcation_bfl_ladd()
    o = None
    for variant, order in _variants():
        o = _compare_with_reference(g.view, p, inl, outl, 60, variant, order)
    assert all(n > 0 for n in o.type_count)


@needs_ref
def test_cosine_pressure_iolets_with_warmup_match_reference():
    c = cases.pipe(radius=5.0, length=20)
    for k, io in enumerate(c.inlets + c.outlets):
        io.density_amp = 0.002
        io.period = 40.0
        io.phase = 0.4 * k
        io.warmup_steps = 15
    for variant, order in _variants():
        _compare_with_reference(c.geometry.view, c.params, c.inlets, c.outlets, 50, variant, order)


@needs_ref
@pytest.mark.parametrize("wall", [capi.WALL_SBB, capi.WALL_BFL])
def test_four_cube_d3q15_anisotropic_matches_reference(wall):
    """The reference's streamer-test setting: D3Q15, LBGK, the four-cube fixture
    with rand() cut distances and anisotropic f = (d+1)/10 + site/100."""
    g, inl, outl = four_cube(15)
    p = LbmParameters(tau=0.8, wall=wall)
    f0 = anisotropic(64, 15)
    for variant, order in _variants():
        _compare_with_reference(g.view, p, inl, outl, 3, variant, order, f0=f0)


@needs_ref
def test_trt_pipe_matches_reference():
    """TRT, magic parameter 3/16 (Code/lb/kernels/TRT.h:94-122), SBB walls, Nash
    iolets: the benchmark's physics on a small pipe."""
    c = cases.pipe(radius=6.0, length=30)
    c.params.kernel = capi.KERNEL_TRT
    for variant, order in _variants():
        _compare_with_reference(c.geometry.view, c.params, c.inlets, c.outlets, 60, variant, order)


@needs_ref
@pytest.mark.parametrize("tau", [0.51, 0.6, 1.0, 1.9])
def test_trt_bifurcation_bfl_ladd_matches_reference(tau):
    """TRT over all six collision types with BFL walls and a Ladd inlet, at τ near
    the stability limit, at τ = 1 (ω+ = −1) and far above it (τ− < τ+ and > τ+)."""
    g, inl, outl, p = golden_cases.bifurcation_bfl_ladd()
    p.kernel = capi.KERNEL_TRT
    p.tau = tau
    for variant, order in _variants():
        _compare_with_reference(g.view, p, inl, outl, 40, variant, order)


@needs_ref
@pytest.mark.parametrize("q", [15, 19])
def test_trt_four_cube_anisotropic_matches_reference(q):
    """TRT on the reference's streamer-test fixture with anisotropic f, where f_neq
    differs in every direction so a mis-paired (i, iBar) would show."""
    g, inl, outl = four_cube(q)
    p = LbmParameters(tau=0.7, kernel=capi.KERNEL_TRT, wall=capi.WALL_BFL)
    f0 = anisotropic(64, q)
    for variant, order in _variants():
        _compare_with_reference(g.view, p, inl, outl, 3, variant, order, f0=f0)


@pytest.mark.parametrize("name", golden_cases.NAMES)
def test_oracle_matches_golden_vectors(name):
    """Golden vectors written by the compiled reference (scalar order)."""
    path = os.path.join(HERE, "golden", name + ".npz")
    z = np.load(path)
    g, inl, outl, p, steps, f0 = golden_cases.build(name)
    o = OracleLBM(g.view, p, inl, outl, order=ORDER_SCALAR)
    assert o.n == int(z["n"])
    assert np.array_equal(np.ctypeslib.as_array(o.dom.nbr, (o.n * o.q,)), z["nbr"])
    o.set_equilibrium()
    if f0 is not None:
        o.f_old[: f0.size] = f0.reshape(-1)
        o.f_new[: f0.size] = f0.reshape(-1)
    o.step(steps)
    assert np.array_equal(o.f_old[:-1], z["f_old"])
    assert np.array_equal(o.f_new[:-1], z["f_new"])
