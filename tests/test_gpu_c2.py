"""The bifurcation workload at its full size, FP64, against the oracle.

Seeded bifurcation (seed 1234): parent radius 24 and length 200, Murray
daughters, about 1.46M fluid sites; BFL walls with analytic cut distances, the
pulsatile Poiseuille Ladd inlet (peak 0.05, period 2000 steps), Nash outlets at
density 1, LBGK tau = 0.6; 10,000 steps from rest.  Every distribution of both
time levels equals the oracle's (the oracle is pinned bit for bit to the
reference's own LB code).  The oracle runs on all host cores.
"""
import os

import numpy as np
import pytest

from hemelb_gb300 import capi, cases
from oracle.oracle import OracleLBM

pytestmark = pytest.mark.gpu


def test_bifurcation_full_size_fp64_bit_exact_over_10k_steps():
    c = cases.bifurcation()
    p = c.params
    assert (p.tau, p.kernel, p.wall, p.inlet, p.outlet) == (0.6, capi.KERNEL_LBGK, capi.WALL_BFL,
                                                           capi.IOLET_LADD, capi.IOLET_NASH)
    assert c.steps == 10000
    s = c.solver()
    assert 1.3e6 < s.n_sites < 1.7e6
    assert all(n > 0 for n in s.collision_counts)
    s.SetInitialConditions()
    o = OracleLBM(c.geometry.view, p, c.inlets, c.outlets)
    o.set_equilibrium()
    threads = os.cpu_count() or 1
    done = 0
    for chunk in (1000, 9000):  # a checkpoint on the way narrows down any divergence
        s.DoTimeStep(chunk)
        o.step(chunk, threads)
        done += chunk
        assert np.array_equal(s.GetFOld(), o.fold()), "differs after %d steps" % done
    assert np.array_equal(s.GetFNew(), o.fnew())
    # the flow has developed: the inlet has completed most of a pulsatile period
    _, u = o.macro()
    assert np.abs(u).max() > 0.01
