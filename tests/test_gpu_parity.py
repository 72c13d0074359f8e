"""Parity of the CUDA update with the CPU oracle, through the C ABI.

FP64 plain form: bit-exact against the oracle's scalar evaluation order (the
reference's aarch64 build) and within 1e-12 relative per distribution of the
SSE3 order (the reference's x86_64 build).  FP32-deviation / FP16-storage forms:
velocity and pressure error against the FP64 oracle within the stated bounds.
"""
import numpy as np
import pytest

from hemelb_gb300 import capi, cases
from hemelb_gb300.lbm import LBM, LbmParameters
from oracle.oracle import ORDER_SCALAR, ORDER_SSE3, OracleLBM

pytestmark = pytest.mark.gpu

THREADS = 8


def oracle_for(case, order=ORDER_SCALAR, params=None):
    o = OracleLBM(case.geometry.view, params or case.params, case.inlets, case.outlets, order=order)
    o.set_equilibrium()
    return o


def small_bifurcation(**kw):
    return cases.bifurcation(seed=kw.pop("seed", 11), parent_radius=kw.pop("parent_radius", 8.0),
                             parent_length=kw.pop("parent_length", 40.0),
                             daughter_length_factor=kw.pop("daughter_length_factor", 1.2),
                             period=kw.pop("period", 200.0), **kw)


def test_pipe_fp64_bit_exact_full_run():
    """Straight pipe, 2000 steps from rest: every distribution equal to the oracle."""
    c = cases.pipe()
    o = oracle_for(c)
    o.step(c.steps, THREADS)
    s = c.solver()
    s.SetInitialConditions()
    s.DoTimeStep(c.steps)
    f = s.GetFOld()
    assert f.shape == o.fold().shape
    assert np.array_equal(f, o.fold())
    assert np.array_equal(s.GetFNew(), o.fnew())


def test_pipe_fp64_within_1e12_of_sse3_order():
    c = cases.pipe()
    o = oracle_for(c, ORDER_SSE3)
    o.step(c.steps, THREADS)
    s = c.solver()
    s.SetInitialConditions()
    s.DoTimeStep(c.steps)
    f = s.GetFOld()
    rel = np.abs(f - o.fold()) / np.abs(o.fold())
    assert rel.max() <= 1e-12


@pytest.mark.parametrize("kernel", [capi.KERNEL_LBGK, capi.KERNEL_TRT])
def test_bifurcation_bfl_ladd_fp64_bit_exact(kernel):
    """BFL walls (with PostStep), pulsatile Ladd inlet, Nash outlets, all six types."""
    c = small_bifurcation()
    c.params.kernel = kernel
    counts = None
    o = oracle_for(c)
    o.step(400, THREADS)
    s = c.solver()
    counts = s.collision_counts
    assert counts == o.type_count
    assert all(n > 0 for n in counts), counts
    s.SetInitialConditions()
    s.DoTimeStep(400)
    assert np.array_equal(s.GetFOld(), o.fold())
    assert np.array_equal(s.GetFNew(), o.fnew())


def test_nash_cosine_iolets_with_warmup_bit_exact():
    """Pulsatile cosine pressure iolets with warm-up from the minimum density."""
    c = cases.pipe(radius=6.0, length=30)
    for k, io in enumerate(c.inlets + c.outlets):
        io.density_amp = 0.002
        io.period = 50.0
        io.phase = 0.3 * k
        io.warmup_steps = 20
    o = oracle_for(c)
    o.step(120, THREADS)
    s = c.solver()
    s.SetInitialConditions()
    s.DoTimeStep(120)
    assert np.array_equal(s.GetFOld(), o.fold())


def test_per_range_streamer_drop_in_matches_oracle():
    """StreamAndCollide / PostStep over each collision-type range, then swap."""
    c = small_bifurcation(seed=5)
    o = oracle_for(c)
    s = c.solver()
    s.SetInitialConditions()
    counts = s.collision_counts
    for _ in range(3):
        first = 0
        for t in range(6):
            s.StreamAndCollide(first, counts[t])
            o.stream_and_collide(first, counts[t])
            first += counts[t]
        first = 0
        for t in range(6):
            s.PostStep(first, counts[t])
            o.post_step(first, counts[t])
            first += counts[t]
        s.SwapOldAndNew()
        o.swap()
    assert np.array_equal(s.GetFOld(), o.fold())


def test_whole_step_equals_per_range_path():
    c = small_bifurcation(seed=6)
    a = c.solver()
    b = c.solver()
    a.SetInitialConditions()
    b.SetInitialConditions()
    a.DoTimeStep(5)
    counts = b.collision_counts
    n = sum(counts)
    for _ in range(5):
        b.StreamAndCollide(0, n)
        b.PostStep(0, n)
        b.SwapOldAndNew()
    assert np.array_equal(a.GetFOld(), b.GetFOld())


def test_put_get_round_trip_and_continue():
    """FieldData-layout put/get is exact, and stepping from a put state matches the oracle."""
    c = small_bifurcation(seed=3)
    o = oracle_for(c)
    o.step(7, THREADS)
    s = c.solver()
    s.PutF(o.fold(), 0)
    s.PutF(o.fnew(), 1)
    assert np.array_equal(s.GetFOld(), o.fold())
    assert np.array_equal(s.GetFNew(), o.fnew())
    # the device time step must follow the oracle's 1-indexed step for the iolets
    s2 = c.solver()
    s2.SetInitialConditions()
    s2.DoTimeStep(7)
    assert np.array_equal(s2.GetFOld(), o.fold())
    o.step(5, THREADS)
    s2.DoTimeStep(5)
    assert np.array_equal(s2.GetFOld(), o.fold())


def test_macro_density_velocity_match_oracle():
    c = cases.pipe(radius=6.0, length=30)
    o = oracle_for(c)
    o.step(50, THREADS)
    s = c.solver()
    s.SetInitialConditions()
    s.DoTimeStep(50)
    rho, u = s.macro()
    orho, ou = o.macro()
    assert np.array_equal(rho, orho)
    assert np.array_equal(u, ou)


def test_reduce_mass_residual_and_instability():
    c = cases.pipe(radius=6.0, length=30)
    o = oracle_for(c)
    o.step(30, THREADS)
    s = c.solver()
    s.SetInitialConditions()
    s.DoTimeStep(30)
    st = s.reduce()
    orho, ou = o.macro(o.f_old)
    prho, pu = o.macro(o.f_new)
    assert st.unstable_sites == 0
    assert abs(st.mass - orho.sum()) <= 1e-9 * orho.sum()
    du = np.sqrt(((ou - pu) ** 2).sum(axis=1)).max()
    assert abs(st.max_du - du) <= 1e-15 + 1e-12 * du
    f = s.GetFOld()
    f[17, 3] = -1.0e-3
    f[99, 0] = np.nan
    s.PutF(f, 0)
    st = s.reduce()
    assert st.unstable_sites == 2


@pytest.mark.parametrize("precision,u_tol,p_tol", [(capi.FP32DEV, 1e-4, 1e-6), (capi.FP16, 2e-2, 1e-4)])
def test_precision_forms_error_against_fp64(precision, u_tol, p_tol):
    """FP32-deviation and FP16-storage forms: relative L2 velocity error and max
    pressure error (p = rho c_s^2) against the FP64 oracle after 1000 steps."""
    c = cases.pipe(radius=8.0, length=48)
    o = oracle_for(c)
    o.step(1000, THREADS)
    s = c.solver(precision)
    s.SetInitialConditions()
    s.DoTimeStep(1000)
    rho, u = s.macro()
    orho, ou = o.macro()
    u_err = np.linalg.norm(u - ou) / np.linalg.norm(ou)
    p_err = np.abs(rho - orho).max() / 3.0
    assert u_err <= u_tol, u_err
    assert p_err <= p_tol, p_err


def test_warm_start_field_init_is_equilibrium():
    c = cases.pipe(radius=6.0, length=30)
    s = c.solver()
    n = s.n_sites
    rng = np.random.default_rng(0)
    rho = 1.0 + 1e-3 * rng.standard_normal(n)
    u = 1e-2 * rng.standard_normal((n, 3))
    s.SetInitialField(rho, u)
    f = s.GetFOld()
    o = oracle_for(c)
    import ctypes as C
    feq = np.empty(19)
    for i in (0, n // 2, n - 1):
        m = (C.c_double * 3)(*(rho[i] * u[i]))
        o.lib.hlbo_feq(C.byref(o.p), rho[i], m, feq.ctypes.data_as(C.POINTER(C.c_double)))
        assert np.array_equal(f[i], feq)


def test_invalid_arguments_fail_loudly():
    c = cases.pipe(radius=4.0, length=10)
    bad = LbmParameters(tau=0.4)
    with pytest.raises(capi.HlbgError):
        LBM(c.geometry, bad, c.inlets, c.outlets)
    # Ladd streamer with pressure iolets is inconsistent
    p = LbmParameters(tau=0.8, inlet=capi.IOLET_LADD)
    with pytest.raises(capi.HlbgError):
        LBM(c.geometry, p, c.inlets, c.outlets)
    s = c.solver()
    with pytest.raises(capi.HlbgError):
        s.DoTimeStep(1)  # no initial condition yet


def test_empty_and_malformed_geometries_fail_loudly():
    """No blocks, blocks without a fluid site, a block outside the block grid, a
    duplicate block and a link record on a solid site: each is refused at
    creation with a message, never run."""
    from tests.helpers import ArrayGeometry
    p = LbmParameters(tau=0.8)
    one = np.zeros((1, 8), dtype=np.uint64)
    one[0, 0] = 1  # local site 0 fluid
    none = np.zeros((0, 8), dtype=np.uint64)
    empty_rec = ([], [], [], [], [], np.zeros((0, 18)))
    cases_ = {
        "no blocks": ArrayGeometry(19, (1, 1, 1), np.zeros((0, 3)), none, *empty_rec),
        "no fluid sites": ArrayGeometry(19, (1, 1, 1), [[0, 0, 0]], np.zeros((1, 8), np.uint64), *empty_rec),
        "outside the block grid": ArrayGeometry(19, (1, 1, 1), [[1, 0, 0]], one, *empty_rec),
        "duplicate block": ArrayGeometry(19, (2, 1, 1), [[0, 0, 0], [0, 0, 0]], np.vstack([one, one]),
                                         *empty_rec),
        "solid site": ArrayGeometry(19, (1, 1, 1), [[0, 0, 0]], one, [1], [0], [0], [-1],
                                    [capi.SITE_FLUID], np.zeros((1, 18))),
    }
    for what, g in cases_.items():
        with pytest.raises(capi.HlbgError) as e:
            LBM(g.view, p, [], [])
        assert str(e.value), what


@pytest.mark.parametrize("kernel", [capi.KERNEL_LBGK, capi.KERNEL_TRT])
def test_fluid_list_launch_fp64_bit_exact(kernel):
    """The fluid-list launch (warps of fluid slots only, zero-fill warps for the
    sectors shared with solid slots): FP64 bit-exact against the oracle on the
    BFL/Ladd/Nash bifurcation."""
    c = small_bifurcation()
    c.params.kernel = kernel
    o = oracle_for(c)
    o.step(300, THREADS)
    s = c.solver()
    s.SetLaunchVariant(5)
    s.SetInitialConditions()
    s.DoTimeStep(300)
    assert np.array_equal(s.GetFOld(), o.fold())
    assert np.array_equal(s.GetFNew(), o.fnew())


@pytest.mark.parametrize("precision", [capi.FP32DEV, capi.FP16])
def test_every_launch_shape_gives_identical_distributions(precision):
    """Every launch shape of the stream-and-collide kernel (the autotuner's
    candidates) computes the same update: identical arrays after 200 steps."""
    c = small_bifurcation()
    ref = None
    for v in range(9):
        s = c.solver(precision)
        s.SetLaunchVariant(v)
        s.SetInitialConditions()
        s.DoTimeStep(200)
        f = (s.GetFOld(), s.GetFNew())
        s.close()
        if ref is None:
            ref = f
        else:
            assert np.array_equal(f[0], ref[0]) and np.array_equal(f[1], ref[1]), v


def _wss_reference(o, normals, tau, q=19):
    """Lattice::CalculateWallShearStressMagnitude (Code/lb/lattices/Lattice.h:652-726)
    restated step by step in FP64, on the oracle's state: moments and equilibrium
    from the oracle's collision of each site, f_neq = f - f_eq."""
    import ctypes as C
    from oracle.oracle import Params, load
    from tests.helpers import CX19, CY19, CZ19
    lib = load()
    p = Params()
    p.q, p.kernel, p.tau = q, capi.KERNEL_LBGK, tau
    V = list(zip(CX19, CY19, CZ19))
    param = (1.0 - 1.0 / (2.0 * tau)) / np.sqrt(2.0)
    f_all = o.fold()
    a = o.arrays()
    out = {}
    for i in np.nonzero(a["wall_mask"] != 0)[0]:
        f = np.ascontiguousarray(f_all[i])
        rho, mom, vel, feq, fpost = np.zeros(1), np.zeros(3), np.zeros(3), np.zeros(q), np.zeros(q)
        dp = lambda x: x.ctypes.data_as(C.POINTER(C.c_double))
        lib.hlbo_collide_site(C.byref(p), dp(f), dp(rho), dp(mom), dp(vel), dp(feq), dp(fpost))
        fneq = [float(f[l] - feq[l]) for l in range(q)]
        pi = [[0.0] * 3 for _ in range(3)]
        for ii in range(3):
            for jj in range(ii + 1):
                acc = 0.0
                for l in range(q):
                    acc += fneq[l] * V[l][ii] * V[l][jj]
                pi[ii][jj] = pi[jj][ii] = acc
        nor = [float(x) for x in normals[i]]
        temp = param * (-np.sqrt(2.0))
        sq = nrm = 0.0
        for ii in range(3):
            sv = 0.0
            for jj in range(3):
                sv += pi[ii][jj] * nor[jj] * temp
            sq += sv * sv
            nrm += sv * nor[ii]
        out[i] = np.sqrt(sq - nrm * nrm)
    return out


def test_wall_shear_stress_matches_reference_formula():
    """Wall shear stress of every wall site after 300 steps (FP64) against the
    reference's formula on the oracle's state, with the geometry's wall normals;
    float max (NO_VALUE) elsewhere."""
    c = small_bifurcation()
    o = oracle_for(c)
    o.step(300, THREADS)
    s = c.solver()
    s.SetInitialConditions()
    s.DoTimeStep(300)
    w = s.WallShearStress()
    g = c.geometry
    a = o.arrays()
    rec = {int(ls): k for k, ls in enumerate(g.link_site)}
    normals = np.zeros((o.n, 3))
    for i, slot in enumerate(a["slot"]):
        k = rec.get(int(slot))
        if k is not None:
            normals[i] = g.wall_normal[k]
    ref = _wss_reference(o, normals, c.params.tau)
    wall = a["wall_mask"] != 0
    assert len(ref) == wall.sum() > 100
    got = np.array([w[i] for i in ref])
    exp = np.array([ref[i] for i in ref])
    assert np.all(np.abs(got - exp) <= 1e-12 * np.abs(exp).max())
    assert np.all(w[~wall] == np.finfo(np.float64).max)
    assert exp.max() > 0


def _flux_reference(o, g, n_in, iolets):
    """Per-iolet sum over the sites with iolet links of their momentum along the
    iolet's normalised normal, from the oracle's state (FP64 numpy)."""
    from tests.helpers import CX19, CY19, CZ19
    a = o.arrays()
    f = o.fold()
    c = np.array([CX19, CY19, CZ19], dtype=np.float64)  # (3, 19)
    rec = {int(ls): k for k, ls in enumerate(g.link_site)}
    out = np.zeros(len(iolets))
    scale = np.zeros(len(iolets))
    for i in np.nonzero(a["iolet_mask"] != 0)[0]:
        k = rec[int(a["slot"][i])]
        gi = int(a["iolet_id"][i]) + (0 if g.site_type[k] == capi.SITE_INLET else n_in)
        nrm = np.array(iolets[gi].normal[:], dtype=np.float64)
        v = float((c @ f[i]) @ (nrm / np.sqrt(nrm @ nrm)))
        out[gi] += v
        scale[gi] += abs(v)
    return out, scale


@pytest.mark.parametrize("case", ["pipe", "bifurcation"])
def test_iolet_flux_matches_oracle_state(case):
    """Mass flux per iolet (momentum along the inward normal over the sites with
    links to it) of the FP64 state against the same sum on the oracle's state."""
    c = cases.pipe() if case == "pipe" else small_bifurcation(seed=4)
    o = oracle_for(c)
    o.step(200, THREADS)
    s = c.solver()
    s.SetInitialConditions()
    s.DoTimeStep(200)
    got = s.IoletFlux()
    exp, scale = _flux_reference(o, c.geometry, len(c.inlets), list(c.inlets) + list(c.outlets))
    assert len(got) == len(c.inlets) + len(c.outlets)
    assert np.all(scale > 0)
    assert np.all(np.abs(got - exp) <= 1e-12 * scale)
    import ctypes as C
    short = np.zeros(1)  # one value for two or more iolets
    assert s._lib.hlbg_iolet_flux(s.ctx, short.ctypes.data_as(C.POINTER(C.c_double)), 1) == capi.HLBG_ERR_INVAL


def test_iolet_flux_balances_at_steady_state():
    """Pipe run to the StabilityTester's steady state: the flux in at the inlet
    equals the flux out at the outlet (mass conservation) to 1e-4."""
    c = cases.pipe()
    s = c.solver()
    s.SetInitialConditions()
    first, run, du, rc = s.RunToSteady(1e-6, 0.01, max_steps=50000)
    assert rc == capi.HLBG_OK
    phi_in, phi_out = s.IoletFlux()
    assert phi_in > 0 and phi_out < 0
    assert abs(phi_in + phi_out) <= 1e-4 * phi_in


def test_set_iolets_is_creating_with_them():
    """hlbg_set_iolets: new iolet parameters on a context give the same run, bit for
    bit, as a context created with them, also when changed between steps (against a
    context created with the new ones and given the state at the change); the
    counts cannot change and the models must match the streamers."""
    from hemelb_gb300.lbm import InOutLetCosine
    old = small_bifurcation(seed=6)
    new = small_bifurcation(seed=6, peak=0.03, period=150.0)
    new_out = [InOutLetCosine(tuple(o.position), tuple(o.normal), density_mean=0.9995) for o in new.outlets]
    a = old.solver()
    a.SetIolets(new.inlets, new_out)
    a.SetInitialConditions()
    a.DoTimeStep(60)
    b = LBM(new.geometry, new.params, new.inlets, new_out)
    b.SetInitialConditions()
    b.DoTimeStep(60)
    assert np.array_equal(a.GetFOld(), b.GetFOld())
    # a change between steps: the state at the change, continued with the new iolets
    c = old.solver()
    c.SetInitialConditions()
    c.DoTimeStep(30)
    d = LBM(new.geometry, new.params, new.inlets, new_out)
    d.PutF(c.GetFOld(), 0)
    d.PutF(c.GetFNew(), 1)
    d.SetTimeStep(31)
    c.SetIolets(new.inlets, new_out)
    c.DoTimeStep(30)
    d.DoTimeStep(30)
    assert np.array_equal(c.GetFOld(), d.GetFOld())
    with pytest.raises(capi.HlbgError):
        c.SetIolets(new.inlets, new_out[:-1])
    with pytest.raises(capi.HlbgError):
        c.SetIolets(new_out[:1], new_out)  # pressure iolet on the Ladd inlet streamer


def test_tree_fp32_deviation_velocity_error_within_1e5_developed_flow():
    """The forest generator's workload (TRT, SBB, Nash 1.001 / 1.0) on a small tree
    (256^3 box, depth 5, root radius 12, about 0.46M sites), run until the flow has
    developed (3000 steps: several viscous times R^2 / nu of the root segment):
    the FP32-deviation velocity is within 1e-5 relative L2 of FP64, the bound the
    FP32-deviation form is held to."""
    c = cases.tree(seed=7, box_sites=256, n_roots=1, depth=5, root_radius=12.0, precision=capi.FP64)
    a = c.solver(capi.FP64)
    b = c.solver(capi.FP32DEV)
    for s in (a, b):
        s.SetInitialConditions()
        s.DoTimeStep(3000)
    _, ua = a.macro()
    _, ub = b.macro()
    assert np.linalg.norm(ua, axis=1).max() > 1e-4  # the flow is there
    rel = np.linalg.norm(ub - ua) / np.linalg.norm(ua)
    assert rel <= 1e-5, rel
