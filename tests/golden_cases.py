"""Definitions of the golden-vector cases (inputs are regenerated from seeds;
tests/golden/<name>.npz holds what the compiled reference produced for them)."""
from __future__ import annotations

import os

from hemelb_gb300 import capi, cases
from hemelb_gb300.lbm import InOutLetCosine, LbmParameters, SyntheticGeometry
from tests.helpers import anisotropic, four_cube, steady_parabolic_inlets

NAMES = ["pipe_sbb_nash_d3q19", "bifurcation_bfl_ladd_d3q19", "four_cube_d3q15_bfl_anisotropic",
         "four_cube_d3q19_sbb_anisotropic", "pipe_trt_sbb_nash_d3q19", "bifurcation_trt_bfl_ladd_d3q19",
         "four_cube_d3q19_trt_bfl_anisotropic"]


# The reference's large_cylinder.gmy (Code/tests/resources) re-written by this
# library's .gmy writer (tests/golden/make_gmy_golden.py); golden vectors from the
# compiled reference on it, per kernel.
GMY_FIXTURE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "large_cylinder_rw.gmy")
GMY_KERNELS = {capi.KERNEL_LBGK: "lbgk", capi.KERNEL_TRT: "trt"}


def gmy_case(path, kernel, steps=60):
    """-> (geometry, inlets, outlets, params, steps): Nash pressure iolets at the two
    ends of the cylinder (z = 0 inlet at 1.001, z = 40 outlet at 0.999), τ = 0.8."""
    g = SyntheticGeometry.from_gmy(path, 19) if path else None
    inl = [InOutLetCosine((8, 8, 0), (0, 0, 1), density_mean=1.001)]
    outl = [InOutLetCosine((8, 8, 40), (0, 0, -1), density_mean=0.999)]
    p = LbmParameters(tau=0.8, kernel=kernel)
    return g, inl, outl, p, steps


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
    # TRT (magic parameter 3/16): the reference's Code/lb/kernels/TRT.h, compiled
    # with the build-time patch of oracle/refbuild/build_ref.py
    if name == "pipe_trt_sbb_nash_d3q19":
        c = cases.pipe(radius=4.0, length=12)
        c.params.kernel = capi.KERNEL_TRT
        return c.geometry, c.inlets, c.outlets, c.params, 100, None
    if name == "bifurcation_trt_bfl_ladd_d3q19":
        g, inl, outl, p = bifurcation_bfl_ladd()
        p.kernel = capi.KERNEL_TRT
        return g, inl, outl, p, 80, None
    if name == "four_cube_d3q19_trt_bfl_anisotropic":
        g, inl, outl = four_cube(19)
        p = LbmParameters(tau=0.7, kernel=capi.KERNEL_TRT, wall=capi.WALL_BFL)
        return g, inl, outl, p, 3, anisotropic(64, 19)
    raise KeyError(name)
