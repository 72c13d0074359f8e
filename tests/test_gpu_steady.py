"""Steady-state runs (StabilityTester's convergence test, evaluated on the device
after every step) and the time-level average, against the oracle in FP64."""
import numpy as np
import pytest

from hemelb_gb300 import capi
from hemelb_gb300.surrogate import Sample
from oracle.oracle import OracleLBM

pytestmark = pytest.mark.gpu


def _max_rel_du(o, u_ref):
    """Code/lb/StabilityTester.h:160-183: max over sites |u(fNew) - u(fOld)| / U_ref."""
    _, un = o.macro(o.f_old)  # after a step the oracle's f_old holds the new state
    _, uo = o.macro(o.f_new)
    return float(np.sqrt(((un - uo) ** 2).sum(axis=1)).max() / u_ref)


def _small_case(i):
    smp = Sample.draw(i, base_seed=11, box=32)
    g = smp.geometry()
    return g, smp.case(g), smp.u_ref(g)


@pytest.mark.parametrize("i", [0, 1])
def test_run_to_steady_matches_oracle(i):
    g, case, ur = _small_case(i)
    s = case.solver()
    s.SetInitialConditions()
    tol = 1e-4
    steps, run, du, rc = s.RunToSteady(tol, ur, 100000, 7)
    # the check of step k is made while step k + 1 collides
    assert rc == 0 and steps < run <= steps + 7
    o = OracleLBM(g.view, case.params, case.inlets, case.outlets)
    o.set_equilibrium()
    n = 0
    while True:
        o.step(1, 4)
        n += 1
        if _max_rel_du(o, ur) <= tol:
            break
        assert n < 100000
    assert n == steps
    o.step(run - 1 - n, 4)
    assert abs(du - _max_rel_du(o, ur)) <= 1e-12 * du  # the last check: step run - 1
    o.step(1, 4)
    assert np.array_equal(s.GetFOld(), o.fold())
    s.close()


def test_run_to_steady_reports_timeout():
    g, case, ur = _small_case(0)
    s = case.solver()
    s.SetInitialConditions()
    steps, run, du, rc = s.RunToSteady(1e-12, ur, 30, 8)
    assert rc == capi.HLBG_ERR_TIMEOUT and steps == -1 and run == 30 and du > 0
    s.close()


def test_average_time_levels_matches_oracle():
    g, case, ur = _small_case(1)
    s = case.solver()
    s.SetInitialConditions()
    s.DoTimeStep(5)
    s.AverageTimeLevels()
    o = OracleLBM(g.view, case.params, case.inlets, case.outlets)
    o.set_equilibrium()
    o.step(5)
    o.f_old[:-1] = (o.f_old[:-1] + o.f_new[:-1]) * 0.5
    assert np.array_equal(s.GetFOld(), o.fold())
    s.DoTimeStep(3)
    o.step(3)
    assert np.array_equal(s.GetFOld(), o.fold())
    s.close()


@pytest.mark.parametrize("prec", [capi.FP64, capi.FP32DEV])
def test_fused_monitor_matches_separate_reduction(prec):
    """hlbg_step_monitored's stats of step k against hlbg_step + hlbg_reduce after
    step k on a second context (the same StabilityTester quantities)."""
    g, case, ur = _small_case(0)
    a = case.solver(prec)
    b = case.solver(prec)
    a.SetInitialConditions()
    b.SetInitialConditions()
    assert a.StepMonitored(1).time_step == -1  # the first step only records
    for k in range(1, 40):
        sa = a.StepMonitored(1)  # stats of step k
        b.DoTimeStep(1)
        sb = b.reduce()  # stats after step k
        assert sa.time_step == sb.time_step == k + 1
        if prec == capi.FP64:
            assert sa.max_du == sb.max_du and sa.min_f == sb.min_f
            assert abs(sa.mass - sb.mass) <= 1e-12 * sb.mass
        else:
            assert abs(sa.max_du - sb.max_du) <= 1e-5 * sb.max_du + 1e-12
            assert abs(sa.min_f - sb.min_f) <= 1e-6 and abs(sa.mass - sb.mass) <= 1e-9 * sb.mass
        assert sa.unstable_sites == sb.unstable_sites == 0
    # the states themselves are the same (a made one step more: the first, recording one)
    b.DoTimeStep(1)
    assert np.array_equal(a.GetFOld(), b.GetFOld())
    # stepping outside a monitored step invalidates the record
    a.DoTimeStep(1)
    assert a.StepMonitored(1).time_step == -1
    a.close()
    b.close()


@pytest.mark.parametrize("prec", [capi.FP64, capi.FP32DEV])
def test_incompressibility_checker_of_the_monitored_state(prec):
    """IncompressibilityChecker's min / max density and max velocity magnitude
    (Code/lb/IncompressibilityChecker.hpp:157-199) of the state the last monitored
    step collided, against the macroscopic fields of that state."""
    g, case, ur = _small_case(1)
    a = case.solver(prec)
    b = case.solver(prec)
    a.SetInitialConditions()
    b.SetInitialConditions()
    a.StepMonitored(1)
    assert a.Incompressibility().time_step == -1
    for k in range(1, 30):
        a.StepMonitored(1)  # collides state k
        b.DoTimeStep(1)     # state k
        inc = a.Incompressibility()
        rho, u = b.macro()
        umag = np.sqrt((u * u).sum(axis=1))
        tol = 1e-14 if prec == capi.FP64 else 1e-6
        assert inc.time_step == k + 1
        assert abs(inc.min_density - rho.min()) <= tol and abs(inc.max_density - rho.max()) <= tol
        assert abs(inc.max_velocity - umag.max()) <= tol * max(1.0, umag.max()) + (0 if prec == capi.FP64 else 1e-7)
        assert abs(inc.max_relative_density_difference - (inc.max_density - inc.min_density)) <= 1e-15
    assert a.IsDensityDiffWithinRange() == (inc.max_relative_density_difference < 0.05)
    assert not a.IsDensityDiffWithinRange(allowed=0.0)
    assert abs(a.MaxMachNumber() - inc.max_velocity * np.sqrt(3.0)) <= 1e-15
    a.close()
    b.close()


@pytest.mark.parametrize("prec", [capi.FP64, capi.FP32DEV])
@pytest.mark.parametrize("interval", [3, 6])
def test_monitor_interval_checks_every_kth_step(prec, interval):
    """With a check interval K the StabilityTester checks the steps t with
    t % K == 0 (the step before records the velocities, the others run the plain
    update): the stats of each check equal the separate reduction after the same
    step, and the state equals plain stepping (monitoring changes no distribution)."""
    g, case, ur = _small_case(0)
    a = case.solver(prec)
    b = case.solver(prec)
    a.SetInitialConditions()
    b.SetInitialConditions()
    a.SetMonitorInterval(interval)
    last = -1
    for t in range(1, 5 * interval + 2):
        # step t collides the state after t - 1 steps, which b holds now
        sb = b.reduce() if t % interval == 0 else None
        sa = a.StepMonitored(1)
        b.DoTimeStep(1)
        if sb is not None:
            last = t
            assert sa.time_step == sb.time_step == t
            if prec == capi.FP64:
                assert sa.max_du == sb.max_du and sa.min_f == sb.min_f
            else:
                assert abs(sa.max_du - sb.max_du) <= 1e-5 * sb.max_du + 1e-12
        assert sa.time_step == last  # stats of the last check made
    assert np.array_equal(a.GetFOld(), b.GetFOld())
    a.close()
    b.close()
