"""Batched ensemble: many stenosed pipes with their own relaxation times in one
geometry and one launch per step (or one CUDA graph per batch of steps).  Each
member evolves exactly as it does alone (FP64, bit for bit against the oracle run
of the standalone member), and graph replay equals plain stepping."""
import numpy as np
import pytest

from hemelb_gb300 import capi, cases
from oracle.oracle import OracleLBM

pytestmark = pytest.mark.gpu


def _member_sites(ens_oracle, block_member, m):
    a = ens_oracle.arrays()
    member = block_member[a["slot"] >> 9]
    return np.nonzero(member == m)[0], a["coords"]


def test_ensemble_members_match_standalone_oracle_fp64():
    ens = cases.ensemble(n_members=4, seed=11, precision=capi.FP64, period=200.0)
    s = ens.solver(capi.FP64)
    s.SetInitialConditions()
    s.DoTimeStep(40)
    f = s.GetFOld()
    eo = OracleLBM(ens.geometry.view, ens.params, ens.inlets, ens.outlets)  # numbering and coordinates
    taus = ens.members["tau"]
    assert len(set(taus.tolist())) == 4
    for m in range(4):
        idx, coords = _member_sites(eo, ens.members["block_member"], m)
        mc = ens.member_case(m, precision=capi.FP64)
        o = OracleLBM(mc.geometry.view, mc.params, mc.inlets, mc.outlets)
        o.set_equilibrium()
        o.step(40, 8)
        oc = o.arrays()["coords"]
        shift = coords[idx].min(axis=0) - oc.min(axis=0)
        key_e = {tuple(c - shift): i for i, c in zip(idx, coords[idx])}
        order = np.array([key_e[tuple(c)] for c in oc])
        assert len(order) == o.n == ens.members["sites"][m]
        assert np.array_equal(f[order], o.fold()), m


def test_graph_replay_equals_plain_steps():
    ens = cases.ensemble(n_members=9, seed=5, precision=capi.FP32DEV, period=300.0)
    a = ens.solver()
    b = ens.solver()
    a.SetInitialConditions()
    b.SetInitialConditions()
    a.DoTimeStep(37)
    for n in (8, 8, 13, 8):  # repeated counts replay cached graphs, odd counts flip parity
        b.DoTimeStepGraph(n)
    assert np.array_equal(a.GetFOld(), b.GetFOld())
    assert np.array_equal(a.GetFNew(), b.GetFNew())
