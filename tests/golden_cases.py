"""Definitions of the golden-vector cases (inputs are regenerated from seeds;
tests/golden/<name>.npz holds what the compiled reference produced for them)."""
from __future__ import annotations

from hemelb_gb300 import capi, cases
from hemelb_gb300.lbm import InOutLetCosine, LbmParameters, SyntheticGeometry
from tests.helpers import anisotropic, four_cube, steady_parabolic_inlets

NAMES = ["pipe_sbb_nash_d3q19", "bifurcation_bfl_ladd_d3q19", "four_cube_d3q15_bfl_anisotropic",
         "four_cube_d3q19_sbb_anisotropic"]


def bifurcation_bfl_ladd(seed=21, parent_radius=5.0, parent_length=14.0, factor=1.0):
    g = SyntheticGeometry.bifurcation(seed, parent_radius, parent_length, factor, 19, True)
    inl = steady_parabolic_inlets(g)
    outl = []
    for k in range(g.n_outlets):
        pos, nrm, _ = g.iolet(True, k)
        outl.append(InOutLetCosine(pos, nrm, density_mean=1.0))
    p = LbmParameters(tau=0.6, kernel=capi.KERNEL_LBGK, wall=capi.WALL_BFL,
                      inlet=capi.IOLET_LADD, outlet=capi.IOLET_NASH)
    return g, inl, outl, p


def build(name):
    """-> (geometry with .view, inlets, outlets, params, steps, f0 or None)"""
    if name == "pipe_sbb_nash_d3q19":
        c = cases.pipe(radius=4.0, length=12)
        return c.geometry, c.inlets, c.outlets, c.params, 100, None
    if name == "bifurcation_bfl_ladd_d3q19":
        g, inl, outl, p = bifurcation_bfl_ladd()
        return g, inl, outl, p, 80, None
    if name == "four_cube_d3q15_bfl_anisotropic":
        g, inl, outl = four_cube(15)
        return g, inl, outl, LbmParameters(tau=0.8, wall=capi.WALL_BFL), 3, anisotropic(64, 15)
    if name == "four_cube_d3q19_sbb_anisotropic":
        g, inl, outl = four_cube(19)
        return g, inl, outl, LbmParameters(tau=0.8, wall=capi.WALL_SBB), 3, anisotropic(64, 19)
    raise KeyError(name)
