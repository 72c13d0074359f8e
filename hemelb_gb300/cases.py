"""The synthetic workloads the update is measured and checked on.

* ``pipe``: straight pipe, radius 10, length 80 (about 25k fluid sites), D3Q19 LBGK
  tau = 0.8, simple bounce-back walls, Nash pressure iolets with lattice density
  1.001 / 0.999, rest start, 2000 steps.
* ``bifurcation``: seeded bifurcation, parent radius 24 and length 200, Murray
  daughters (split ratio in [0.3, 0.7], half-angle in [25, 60] degrees), about
  1.5M sites; BFL walls with analytic cut distances, pulsatile Poiseuille Ladd inlet
  (peak 0.05, period 2000), Nash outlets at density 1, LBGK tau = 0.6.
* ``tree``: seeded random vascular forest in a 1280^3 box of sparse 8^3 blocks,
  root radius 60, Murray radii, branch angles in [20, 70] degrees, segment length
  6-10 x radius; TRT (Lambda = 3/16), SBB walls, inlet density 1.001, outlets 1.0,
  FP32-deviation storage.
* ``stenosis``: pipe with a Gaussian stenosis (one member of the batched ensemble).
"""
from __future__ import annotations

from . import capi
from .lbm import (Case, InOutLetCosine, InOutLetParabolicVelocity, LbmParameters,
                  SyntheticGeometry)


def _pressure_iolets(geom: SyntheticGeometry, rho_in: float, rho_out: float):
    inl, outl = [], []
    for k in range(geom.n_inlets):
        pos, nrm, _ = geom.iolet(False, k)
        inl.append(InOutLetCosine(pos, nrm, density_mean=rho_in))
    for k in range(geom.n_outlets):
        pos, nrm, _ = geom.iolet(True, k)
        outl.append(InOutLetCosine(pos, nrm, density_mean=rho_out))
    return inl, outl


def pipe(radius: float = 10.0, length: int = 80, steps: int = 2000, precision=capi.FP64) -> Case:
    g = SyntheticGeometry.pipe(radius, length, 19, with_cuts=True)
    inl, outl = _pressure_iolets(g, 1.001, 0.999)
    p = LbmParameters(tau=0.8, kernel=capi.KERNEL_LBGK, wall=capi.WALL_SBB,
                      inlet=capi.IOLET_NASH, outlet=capi.IOLET_NASH, precision=precision)
    return Case("pipe_r%g_l%d" % (radius, length), g, p, inl, outl, steps)


def bifurcation(seed: int = 1234, parent_radius: float = 24.0, parent_length: float = 200.0,
                daughter_length_factor: float = 2.5, steps: int = 10000, precision=capi.FP64,
                peak: float = 0.05, period: float = 2000.0) -> Case:
    g = SyntheticGeometry.bifurcation(seed, parent_radius, parent_length, daughter_length_factor,
                                      19, with_cuts=True)
    inl = []
    for k in range(g.n_inlets):
        pos, nrm, r = g.iolet(False, k)
        inl.append(InOutLetParabolicVelocity(pos, nrm, radius=r, max_speed=peak,
                                             pulsatile_period=period))
    outl = []
    for k in range(g.n_outlets):
        pos, nrm, _ = g.iolet(True, k)
        outl.append(InOutLetCosine(pos, nrm, density_mean=1.0))
    p = LbmParameters(tau=0.6, kernel=capi.KERNEL_LBGK, wall=capi.WALL_BFL,
                      inlet=capi.IOLET_LADD, outlet=capi.IOLET_NASH, precision=precision)
    return Case("bifurcation_s%d_r%g" % (seed, parent_radius), g, p, inl, outl, steps)


def tree(seed: int = 7, box_sites: int = 1280, n_roots: int = 5, depth: int = 7,
         root_radius: float = 60.0, precision=capi.FP32DEV, n_threads: int = 0) -> Case:
    g = SyntheticGeometry.tree(seed, box_sites, n_roots, depth, root_radius, 19, with_cuts=False,
                               n_threads=n_threads)
    inl, outl = _pressure_iolets(g, 1.001, 1.0)
    p = LbmParameters(tau=0.8, kernel=capi.KERNEL_TRT, wall=capi.WALL_SBB,
                      inlet=capi.IOLET_NASH, outlet=capi.IOLET_NASH, precision=precision)
    return Case("tree_s%d_box%d_roots%d_depth%d" % (seed, box_sites, n_roots, depth), g, p, inl,
                outl, 0)


def stenosis(radius: float = 10.0, length: int = 80, depth: float = 0.5, tau: float = 0.8,
             precision=capi.FP32DEV, peak: float = 0.02, period: float = 1000.0) -> Case:
    g = SyntheticGeometry.stenosis(radius, length, depth, 19, with_cuts=True)
    inl = []
    for k in range(g.n_inlets):
        pos, nrm, r = g.iolet(False, k)
        inl.append(InOutLetParabolicVelocity(pos, nrm, radius=r, max_speed=peak,
                                             pulsatile_period=period))
    outl = []
    for k in range(g.n_outlets):
        pos, nrm, _ = g.iolet(True, k)
        outl.append(InOutLetCosine(pos, nrm, density_mean=1.0))
    p = LbmParameters(tau=tau, kernel=capi.KERNEL_LBGK, wall=capi.WALL_SBB,
                      inlet=capi.IOLET_LADD, outlet=capi.IOLET_NASH, precision=precision)
    return Case("stenosis_r%g_l%d_d%.2f" % (radius, length, depth), g, p, inl, outl, 0)


def ensemble(n_members: int = 512, seed: int = 2024, precision=capi.FP32DEV, peak: float = 0.02,
             period: float = 1000.0):
    """Batched ensemble of seeded stenosed pipes in one geometry (one cell per
    member), per-member tau, pulsatile Ladd inlets and Nash outlets.  Returns the
    Case (its solver() sets the per-block tau) and the member table."""
    g = SyntheticGeometry.ensemble(seed, n_members, 19)
    block_member, tau, shape, sites = g.members()
    inl, outl = [], []
    for k in range(g.n_inlets):
        pos, nrm, r = g.iolet(False, k)
        inl.append(InOutLetParabolicVelocity(pos, nrm, radius=r, max_speed=peak, pulsatile_period=period))
    for k in range(g.n_outlets):
        pos, nrm, _ = g.iolet(True, k)
        outl.append(InOutLetCosine(pos, nrm, density_mean=1.0))
    p = LbmParameters(tau=0.8, kernel=capi.KERNEL_LBGK, wall=capi.WALL_SBB,
                      inlet=capi.IOLET_LADD, outlet=capi.IOLET_NASH, precision=precision)
    case = EnsembleCase("ensemble_%d_s%d" % (n_members, seed), g, p, inl, outl, 0)
    case.block_tau = tau[block_member]
    case.members = {"tau": tau, "shape": shape, "sites": sites, "block_member": block_member,
                    "peak": peak, "period": period}
    return case


class EnsembleCase(Case):
    """A Case whose solver carries one relaxation time per member."""

    block_tau = None
    members = None

    def solver(self, precision=None):
        s = super().solver(precision)
        s.SetBlockTau(self.block_tau)
        return s

    def member_case(self, m: int, precision=capi.FP32DEV) -> Case:
        """Member m as a standalone geometry (same voxels up to a translation)."""
        R, L, depth = self.members["shape"][m]
        g = SyntheticGeometry.stenosis(R, int(L), depth, 19, with_cuts=True)
        inl, outl = [], []
        for k in range(g.n_inlets):
            pos, nrm, r = g.iolet(False, k)
            inl.append(InOutLetParabolicVelocity(pos, nrm, radius=r, max_speed=self.members["peak"],
                                                 pulsatile_period=self.members["period"]))
        for k in range(g.n_outlets):
            pos, nrm, _ = g.iolet(True, k)
            outl.append(InOutLetCosine(pos, nrm, density_mean=1.0))
        p = LbmParameters(tau=float(self.members["tau"][m]), kernel=capi.KERNEL_LBGK,
                          wall=capi.WALL_SBB, inlet=capi.IOLET_LADD, outlet=capi.IOLET_NASH,
                          precision=precision)
        return Case("member_%d" % m, g, p, inl, outl, 0)
