"""Host-side Python mirror of the reference's LB interface over the C ABI.

Names follow HemeLB's classes: ``InOutLetCosine`` / ``InOutLetParabolicVelocity``
(Code/lb/iolets), ``LbmParameters`` (Code/lb/LbmParameters.h) and ``LBM``
(Code/lb/lb.h) with ``SetInitialConditions``, the per-range streamer calls
``StreamAndCollide(first, count)`` / ``PostStep(first, count)`` and the whole-step
``DoTimeStep``.  Every call goes through libhemelb_gb300.so; nothing here computes
the update.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

import numpy as np

from . import capi
from .capi import check

_D = C.POINTER(C.c_double)


def _np(ptr, n, dtype):
    if n == 0 or not ptr:
        return np.zeros(0, dtype=dtype)
    return np.ctypeslib.as_array(ptr, shape=(n,)).view(dtype)


class SyntheticGeometry:
    """A seeded synthetic vessel geometry in sparse-block (GmyReadResult) form."""

    def __init__(self, handle: C.c_void_p, lib):
        self._lib = lib
        self._h = handle
        self.view = capi.Geometry()
        nf = C.c_int64()
        ni = C.c_int32()
        no = C.c_int32()
        check(lib.hlbg_synth_view(self._h, C.byref(self.view), C.byref(nf), C.byref(ni), C.byref(no)))
        self.n_fluid = nf.value
        self.n_inlets = ni.value
        self.n_outlets = no.value
        v = self.view
        self.q = v.q
        self.blocks = tuple(v.blocks)
        self.n_blocks = v.n_blocks
        self.block_coords = _np(v.block_coords, 3 * v.n_blocks, np.int32).reshape(-1, 3)
        self.fluid_mask = _np(v.fluid_mask, 8 * v.n_blocks, np.uint64).reshape(-1, 8)
        n = v.n_link_sites
        self.n_link_sites = n
        self.link_site = _np(v.link_site, n, np.int64)
        self.wall_mask = _np(v.wall_mask, n, np.uint32)
        self.iolet_mask = _np(v.iolet_mask, n, np.uint32)
        self.iolet_id = _np(v.iolet_id, n, np.int32)
        self.site_type = _np(v.site_type, n, np.int8)
        self.cut_distance = (_np(v.cut_distance, n * (v.q - 1), np.float32).reshape(n, v.q - 1)
                             if v.cut_distance else None)
        self.wall_normal = _np(v.wall_normal, n * 3, np.float32).reshape(n, 3) if v.wall_normal else None

    def write_gmy(self, path: str):
        """Write this geometry as a HemeLB .gmy file (readable by GeometryReader)."""
        check(self._lib.hlbg_write_gmy(C.byref(self.view), path.encode()), None, "hlbg_write_gmy")

    def iolet(self, is_outlet: bool, index: int):
        pos = (C.c_double * 3)()
        nrm = (C.c_double * 3)()
        r = C.c_double()
        check(self._lib.hlbg_synth_iolet(self._h, int(is_outlet), index, pos, nrm, C.byref(r)))
        return tuple(pos), tuple(nrm), r.value

    def close(self):
        if self._h:
            self._lib.hlbg_synth_free(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # ---- seeded generators ---------------------------------------------------
    @classmethod
    def pipe(cls, radius=10.0, length=80, q=19, with_cuts=True):
        lib = capi.load()
        h = C.c_void_p()
        check(lib.hlbg_synth_pipe(radius, length, q, int(with_cuts), C.byref(h)))
        return cls(h, lib)

    @classmethod
    def bifurcation(cls, seed=1234, parent_radius=24.0, parent_length=200.0,
                    daughter_length_factor=2.5, q=19, with_cuts=True):
        lib = capi.load()
        h = C.c_void_p()
        check(lib.hlbg_synth_bifurcation(seed, parent_radius, parent_length, daughter_length_factor,
                                         q, int(with_cuts), C.byref(h)))
        return cls(h, lib)

    @classmethod
    def stenosis(cls, radius=10.0, length=80, depth=0.5, q=19, with_cuts=True):
        lib = capi.load()
        h = C.c_void_p()
        check(lib.hlbg_synth_stenosis(radius, length, depth, q, int(with_cuts), C.byref(h)))
        return cls(h, lib)

    @classmethod
    def from_gmy(cls, path: str, q: int = 19):
        """A HemeLB .gmy file (GeometryReader's input) as a sparse block geometry."""
        lib = capi.load()
        h = C.c_void_p()
        check(lib.hlbg_read_gmy(path.encode(), q, C.byref(h)), None, "hlbg_read_gmy(%s)" % path)
        return cls(h, lib)

    @classmethod
    def ensemble(cls, seed=2024, n_members=512, q=19, n_threads=0):
        lib = capi.load()
        h = C.c_void_p()
        check(lib.hlbg_synth_ensemble(seed, n_members, q, n_threads, C.byref(h)))
        return cls(h, lib)

    def members(self):
        """(block_member[n_blocks], member_tau[m], member_shape[m,3], member_sites[m]) or None."""
        n = C.c_int32()
        bm = C.POINTER(C.c_int32)()
        tau = C.POINTER(C.c_double)()
        shape = C.POINTER(C.c_double)()
        sites = C.POINTER(C.c_int64)()
        check(self._lib.hlbg_synth_members(self._h, C.byref(n), C.byref(bm), C.byref(tau),
                                           C.byref(shape), C.byref(sites)))
        if n.value == 0:
            return None
        m = n.value
        return (_np(bm, self.n_blocks, np.int32).copy(), _np(tau, m, np.float64).copy(),
                _np(shape, 3 * m, np.float64).reshape(m, 3).copy(), _np(sites, m, np.int64).copy())

    @classmethod
    def vessel_box(cls, seed: int, box_sites: int = 96, kind: int = 0, q: int = 19):
        """Seeded stenosis (kind 0) or bifurcation (kind 1) in a fixed box."""
        lib = capi.load()
        h = C.c_void_p()
        check(lib.hlbg_synth_vessel_box(seed, box_sites, kind, q, C.byref(h)))
        return cls(h, lib)

    def box_shape(self):
        return tuple(int(b) * 8 for b in self.view.blocks)

    def signed_distance(self) -> np.ndarray:
        """Signed distance to the wall on the box grid, shape (X, Y, Z), positive inside."""
        out = np.empty(self.box_shape(), dtype=np.float32)
        check(self._lib.hlbg_synth_distance(self._h, out.ctypes.data_as(C.POINTER(C.c_float))))
        return out

    def fluid_grid(self) -> np.ndarray:
        """Fluid flags on the box grid, shape (X, Y, Z), from the block bitmaps."""
        X, Y, Z = self.box_shape()
        grid = np.zeros((X, Y, Z), dtype=bool)
        bc = self.block_coords.reshape(-1, 3)
        bits = np.unpackbits(self.fluid_mask.reshape(-1, 8).view(np.uint8), axis=1,
                             bitorder="little").astype(bool)  # [blocks, 512], local (x*8+y)*8+z
        loc = np.arange(512)
        lx, ly, lz = loc >> 6, (loc >> 3) & 7, loc & 7
        for b in range(bc.shape[0]):
            m = bits[b]
            grid[bc[b, 0] * 8 + lx[m], bc[b, 1] * 8 + ly[m], bc[b, 2] * 8 + lz[m]] = True
        return grid

    @classmethod
    def tree(cls, seed=7, box_sites=1280, n_roots=1, depth=7, root_radius=60.0, q=19,
             with_cuts=False, n_threads=0):
        lib = capi.load()
        h = C.c_void_p()
        check(lib.hlbg_synth_tree(seed, box_sites, n_roots, depth, root_radius, q, int(with_cuts),
                                  n_threads, C.byref(h)))
        return cls(h, lib)


def InOutLetCosine(position, normal, density_mean=1.0, density_amp=0.0, phase=0.0,
                   period=1.0, warmup_steps=0) -> capi.Iolet:
    """Pressure iolet (Code/lb/iolets/InOutLetCosine.cc:26-43)."""
    io = capi.Iolet()
    io.model = capi.IOLET_COSINE
    io.position[:] = position
    io.normal[:] = normal
    io.density_mean = density_mean
    io.density_amp = density_amp
    io.phase = phase
    io.period = period
    io.warmup_steps = warmup_steps
    return io


def InOutLetParabolicVelocity(position, normal, radius, max_speed, warmup_steps=0,
                              pulsatile_period=None) -> capi.Iolet:
    """Velocity iolet (Code/lb/iolets/InOutLetParabolicVelocity.cc:23-43); with
    ``pulsatile_period`` the peak follows max_speed * (1 - cos(2 pi t / T)) / 2."""
    io = capi.Iolet()
    io.model = capi.IOLET_PARABOLIC if pulsatile_period is None else capi.IOLET_PULSATILE
    io.position[:] = position
    io.normal[:] = normal
    io.radius = radius
    io.max_speed = max_speed
    io.vel_period = pulsatile_period or 0.0
    io.warmup_steps = warmup_steps
    return io


@dataclass
class LbmParameters:
    tau: float = 0.8
    kernel: int = capi.KERNEL_LBGK
    wall: int = capi.WALL_SBB
    inlet: int = capi.IOLET_NASH
    outlet: int = capi.IOLET_NASH
    precision: int = capi.FP64

    @property
    def omega(self) -> float:
        return -1.0 / self.tau

    def to_c(self) -> capi.Params:
        p = capi.Params()
        p.kernel, p.wall, p.inlet, p.outlet = self.kernel, self.wall, self.inlet, self.outlet
        p.precision = self.precision
        p.flags = 0
        p.tau = self.tau
        return p


class LBM:
    """The device LB update for one geometry (lb::LBM's role, Code/lb/lb.h:30-142)."""

    def __init__(self, geometry: SyntheticGeometry | capi.Geometry, params: LbmParameters,
                 inlets=(), outlets=()):
        self._lib = capi.load()
        self.params = params
        self._geom_keep = geometry
        gview = geometry.view if isinstance(geometry, SyntheticGeometry) else geometry
        ni, no = len(inlets), len(outlets)
        self._n_inlets, self._n_outlets = ni, no
        self._inl = (capi.Iolet * max(ni, 1))(*inlets)
        self._outl = (capi.Iolet * max(no, 1))(*outlets)
        pc = params.to_c()
        ctx = C.c_void_p()
        rc = self._lib.hlbg_create(C.byref(gview), C.byref(pc), self._inl, ni, self._outl, no,
                                   C.byref(ctx))
        self._ctx = ctx
        if rc != capi.HLBG_OK:
            msg = self._lib.hlbg_last_error(ctx).decode() if ctx else ""
            if ctx:
                self._lib.hlbg_destroy(ctx)
            self._ctx = None
            raise capi.HlbgError(rc, msg)
        self.n_sites = self._lib.hlbg_site_count(self._ctx)
        self.n_slots = self._lib.hlbg_slot_count(self._ctx)
        cnt = (C.c_int64 * 6)()
        check(self._lib.hlbg_collision_counts(self._ctx, cnt), self._ctx)
        self.collision_counts = tuple(cnt)

    def close(self):
        if getattr(self, "_ctx", None):
            self._lib.hlbg_destroy(self._ctx)
            self._ctx = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def ctx(self):
        return self._ctx

    def device_bytes(self) -> int:
        return int(self._lib.hlbg_device_bytes(self._ctx))

    def site_order(self) -> np.ndarray:
        out = np.empty(self.n_sites, dtype=np.int64)
        check(self._lib.hlbg_site_order(self._ctx, out.ctypes.data_as(C.POINTER(C.c_int64))), self._ctx)
        return out

    def site_coords(self) -> np.ndarray:
        out = np.empty((self.n_sites, 3), dtype=np.int32)
        check(self._lib.hlbg_site_coords(self._ctx, out.ctypes.data_as(C.POINTER(C.c_int32))), self._ctx)
        return out

    # ---- LBM::SetInitialConditions -------------------------------------------
    def SetInitialConditions(self, density=1.0, velocity=(0.0, 0.0, 0.0)):
        check(self._lib.hlbg_init_equilibrium(self._ctx, density, *velocity), self._ctx)

    def SetInitialField(self, rho: np.ndarray, u: np.ndarray):
        rho = np.ascontiguousarray(rho, dtype=np.float64)
        u = np.ascontiguousarray(u, dtype=np.float64)
        check(self._lib.hlbg_init_equilibrium_field(self._ctx, rho.ctypes.data_as(_D),
                                                    u.ctypes.data_as(_D)), self._ctx)

    # ---- stepping ---------------------------------------------------------------
    def DoTimeStep(self, n: int = 1, sync: bool = True):
        check(self._lib.hlbg_step(self._ctx, n, None), self._ctx)
        if sync:
            check(self._lib.hlbg_sync(self._ctx), self._ctx)

    def DoTimeStepGraph(self, n: int = 1, sync: bool = True):
        check(self._lib.hlbg_step_graph(self._ctx, n), self._ctx)
        if sync:
            check(self._lib.hlbg_sync(self._ctx), self._ctx)

    def RunToSteady(self, tol: float, u_ref: float, max_steps: int = 1_000_000,
                    check_batch: int = 25):
        """Step until max |u_new - u_old| / u_ref <= tol (checked after every step on
        the device).  Returns (steps_to_steady, steps_run, final_rel_du, status);
        status is 0 when converged, HLBG_ERR_TIMEOUT or HLBG_ERR_UNSTABLE otherwise."""
        a, b, d = C.c_int64(), C.c_int64(), C.c_double()
        rc = self._lib.hlbg_run_to_steady(self._ctx, tol, u_ref, max_steps, check_batch,
                                          C.byref(a), C.byref(b), C.byref(d))
        if rc not in (capi.HLBG_OK, capi.HLBG_ERR_TIMEOUT, capi.HLBG_ERR_UNSTABLE):
            check(rc, self._ctx)
        return a.value, b.value, d.value, rc

    def SetMonitorInterval(self, interval: int):
        """StabilityTester check every `interval` steps in StepMonitored (default 1)."""
        check(self._lib.hlbg_set_monitor_interval(self._ctx, interval), self._ctx)

    def StepMonitored(self, n: int = 1) -> capi.Stats:
        """n steps with the fused StabilityTester; the stats of the step before the last
        (time_step -1 when there is none yet)."""
        st = capi.Stats()
        rc = self._lib.hlbg_step_monitored(self._ctx, n, C.byref(st))
        if rc not in (capi.HLBG_OK, capi.HLBG_ERR_UNSTABLE):
            check(rc, self._ctx)
        return st

    def WriteCheckpoint(self, path: str, timestep: int, voxel_size: float = 1.0, origin=(0.0, 0.0, 0.0),
                        append: bool = False):
        """XTR (version 5) distribution checkpoint of the current state."""
        o = (C.c_double * 3)(*origin)
        check(self._lib.hlbg_write_checkpoint(self._ctx, path.encode(), timestep, voxel_size, o, int(append)),
              self._ctx)

    def ReadCheckpoint(self, path: str, timestep: int = -1) -> int:
        """Load a distribution checkpoint (its last record when timestep < 0) into both
        time levels; returns the record's timestep.  The step counter is left alone,
        as LocalDistributionInput leaves it to the initial condition's SetTime:
        SetTimeStep sets the step of the next update."""
        t = C.c_uint64()
        check(self._lib.hlbg_read_checkpoint(self._ctx, path.encode(), timestep, C.byref(t)), self._ctx)
        return int(t.value)

    def SetTimeStep(self, t1: int):
        """1-indexed time step of the next update (SimulationState::timeStep)."""
        check(self._lib.hlbg_set_time_step(self._ctx, t1), self._ctx)

    def WallShearStress(self) -> np.ndarray:
        """Wall shear stress magnitude per contiguous site (float max where no wall link)."""
        out = np.empty(self.n_sites, dtype=np.float64)
        check(self._lib.hlbg_wall_shear_stress(self._ctx, out.ctypes.data_as(_D)), self._ctx)
        return out

    def SetIolets(self, inlets, outlets):
        """New iolet parameters (same counts as at creation)."""
        ni, no = len(inlets), len(outlets)
        self._inl = (capi.Iolet * max(ni, 1))(*inlets)
        self._outl = (capi.Iolet * max(no, 1))(*outlets)
        check(self._lib.hlbg_set_iolets(self._ctx, self._inl, ni, self._outl, no), self._ctx)

    def IoletFlux(self) -> np.ndarray:
        """Mass flux through each iolet (inlets, then outlets) of the current state:
        momentum of the sites with links to it along its inward normal."""
        n = self._n_inlets + self._n_outlets
        out = np.zeros(n, dtype=np.float64)
        check(self._lib.hlbg_iolet_flux(self._ctx, out.ctypes.data_as(_D), n), self._ctx)
        return out

    def Incompressibility(self) -> capi.Incomp:
        """IncompressibilityChecker's quantities of the last monitored step."""
        out = capi.Incomp()
        check(self._lib.hlbg_incompressibility(self._ctx, C.byref(out)), self._ctx)
        return out

    def IsDensityDiffWithinRange(self, allowed: float = 0.05) -> bool:
        """IncompressibilityChecker::IsDensityDiffWithinRange with its default 5 %
        (Code/lb/IncompressibilityChecker.hpp:247-250)."""
        return self.Incompressibility().max_relative_density_difference < allowed

    def MaxMachNumber(self) -> float:
        """Largest velocity magnitude over the lattice sound speed 1/sqrt(3)."""
        return self.Incompressibility().max_velocity * 3.0 ** 0.5

    def AverageTimeLevels(self):
        """Current distributions <- mean of the two time levels (right after a step)."""
        check(self._lib.hlbg_average_time_levels(self._ctx), self._ctx)

    def SetLaunchVariant(self, variant: int):
        check(self._lib.hlbg_set_launch_variant(self._ctx, variant), self._ctx)

    def autotune(self, steps_per_trial: int = 5):
        v = C.c_int32()
        ms = C.c_float()
        check(self._lib.hlbg_autotune(self._ctx, steps_per_trial, C.byref(v), C.byref(ms)), self._ctx)
        return int(v.value), float(ms.value)

    def SetBlockTau(self, tau_per_block: np.ndarray):
        t = np.ascontiguousarray(tau_per_block, dtype=np.float64)
        check(self._lib.hlbg_set_block_tau(self._ctx, t.ctypes.data_as(_D)), self._ctx)

    def StreamAndCollide(self, first: int, count: int):
        check(self._lib.hlbg_stream_and_collide_range(self._ctx, first, count), self._ctx)

    def PostStep(self, first: int, count: int):
        check(self._lib.hlbg_post_step_range(self._ctx, first, count), self._ctx)

    def SwapOldAndNew(self):
        check(self._lib.hlbg_swap(self._ctx), self._ctx)

    def time_steps(self, n: int) -> float:
        ms = C.c_float()
        check(self._lib.hlbg_time_steps(self._ctx, n, C.byref(ms)), self._ctx)
        return float(ms.value)

    def time_kernels(self, n: int):
        c = C.c_float()
        p = C.c_float()
        check(self._lib.hlbg_time_kernels(self._ctx, n, C.byref(c), C.byref(p)), self._ctx)
        return float(c.value), float(p.value)

    # ---- FieldData access ------------------------------------------------------
    def GetFOld(self, out: np.ndarray | None = None) -> np.ndarray:
        return self._get_f(0, out)

    def GetFNew(self, out: np.ndarray | None = None) -> np.ndarray:
        return self._get_f(1, out)

    def _get_f(self, which, out):
        if out is None:
            out = np.empty((self.n_sites, 19), dtype=np.float64)
        check(self._lib.hlbg_get_f(self._ctx, out.ctypes.data_as(_D), which), self._ctx)
        return out

    def PutF(self, f: np.ndarray, which: int = 0):
        f = np.ascontiguousarray(f, dtype=np.float64)
        check(self._lib.hlbg_put_f(self._ctx, f.ctypes.data_as(_D), which), self._ctx)

    def macro(self):
        rho = np.empty(self.n_sites, dtype=np.float64)
        u = np.empty((self.n_sites, 3), dtype=np.float64)
        check(self._lib.hlbg_get_macro(self._ctx, rho.ctypes.data_as(_D), u.ctypes.data_as(_D)),
              self._ctx)
        return rho, u

    def reduce(self) -> capi.Stats:
        st = capi.Stats()
        rc = self._lib.hlbg_reduce(self._ctx, C.byref(st))
        if rc not in (capi.HLBG_OK, capi.HLBG_ERR_UNSTABLE):
            check(rc, self._ctx)
        return st

    def iolet_density(self, is_outlet: bool, index: int, t: int) -> float:
        d = C.c_double()
        check(self._lib.hlbg_iolet_density(self._ctx, int(is_outlet), index, t, C.byref(d)), self._ctx)
        return d.value


@dataclass
class Case:
    """A named workload: geometry, parameters and iolets."""

    name: str
    geometry: SyntheticGeometry
    params: LbmParameters
    inlets: list = field(default_factory=list)
    outlets: list = field(default_factory=list)
    steps: int = 0

    def solver(self, precision: int | None = None) -> LBM:
        p = self.params
        if precision is not None:
            p = LbmParameters(**{**p.__dict__, "precision": precision})
        return LBM(self.geometry, p, self.inlets, self.outlets)
