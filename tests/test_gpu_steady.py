"""Steady-state runs (StabilityTester's convergence test, evaluated on the device
after every step) and the time-level average, against the oracle in FP64."""
import numpy as np
import pytest

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
    assert rc == 0 and steps <= run < steps + 7
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
    o.step(run - n, 4)
    assert np.array_equal(s.GetFOld(), o.fold())
    assert abs(du - _max_rel_du(o, ur)) <= 1e-12 * du
    s.close()


def test_run_to_steady_reports_timeout():
    g, case, ur = _small_case(0)
    s = case.solver()
    s.SetInitialConditions()
    steps, run, du, rc = s.RunToSteady(1e-12, ur, 30, 8)
    from hemelb_gb300 import capi
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
