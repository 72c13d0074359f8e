"""Shared helpers for the tests: small geometries built directly in the sparse
block form, including a four-cube fixture in the style of the reference's
FourCubeLatticeData (Code/tests/helpers/FourCubeLatticeData.cc:53-170)."""
from __future__ import annotations

import ctypes as C

import numpy as np

from hemelb_gb300 import capi
from hemelb_gb300.lbm import InOutLetCosine, InOutLetParabolicVelocity

CX15 = [0, 1, -1, 0, 0, 0, 0, 1, -1, 1, -1, 1, -1, 1, -1]
CY15 = [0, 0, 0, 1, -1, 0, 0, 1, -1, 1, -1, -1, 1, -1, 1]
CZ15 = [0, 0, 0, 0, 0, 1, -1, 1, -1, -1, 1, 1, -1, -1, 1]
CX19 = [0, 1, -1, 0, 0, 0, 0, 1, -1, 1, -1, 1, -1, 1, -1, 0, 0, 0, 0]
CY19 = [0, 0, 0, 1, -1, 0, 0, 1, -1, -1, 1, 0, 0, 0, 0, 1, -1, 1, -1]
CZ19 = [0, 0, 0, 0, 0, 1, -1, 0, 0, 0, 0, 1, -1, -1, 1, 1, -1, -1, 1]


class ArrayGeometry:
    """Owns numpy arrays and exposes them as a capi.Geometry view."""

    def __init__(self, q, blocks, block_coords, fluid_mask, link_site, wall, iolet, ioid, stype, cuts):
        self.arrays = dict(
            block_coords=np.ascontiguousarray(block_coords, dtype=np.int32),
            fluid_mask=np.ascontiguousarray(fluid_mask, dtype=np.uint64),
            link_site=np.ascontiguousarray(link_site, dtype=np.int64),
            wall=np.ascontiguousarray(wall, dtype=np.uint32),
            iolet=np.ascontiguousarray(iolet, dtype=np.uint32),
            ioid=np.ascontiguousarray(ioid, dtype=np.int32),
            stype=np.ascontiguousarray(stype, dtype=np.int8),
            cuts=np.ascontiguousarray(cuts, dtype=np.float32),
        )
        a = self.arrays
        v = capi.Geometry()
        v.q, v.block_size = q, 8
        v.blocks[:] = blocks
        v.n_blocks = len(a["block_coords"])
        v.block_coords = a["block_coords"].ctypes.data_as(C.POINTER(C.c_int32))
        v.fluid_mask = a["fluid_mask"].ctypes.data_as(C.POINTER(C.c_uint64))
        v.n_link_sites = len(a["link_site"])
        v.link_site = a["link_site"].ctypes.data_as(C.POINTER(C.c_int64))
        v.wall_mask = a["wall"].ctypes.data_as(C.POINTER(C.c_uint32))
        v.iolet_mask = a["iolet"].ctypes.data_as(C.POINTER(C.c_uint32))
        v.iolet_id = a["ioid"].ctypes.data_as(C.POINTER(C.c_int32))
        v.site_type = a["stype"].ctypes.data_as(C.POINTER(C.c_int8))
        v.cut_distance = a["cuts"].ctypes.data_as(C.POINTER(C.c_float))
        self.view = v


def glibc_rand_sequence():
    """rand() from the C library with its default seed (as the four-cube fixture
    draws cut distances with an unseeded std::rand)."""
    libc = C.CDLL(None)
    libc.srand(1)
    while True:
        yield libc.rand()


def four_cube(q: int = 15, side: int = 4):
    """A side^3 fluid cube at coordinates 1..side of one 8^3 block: inlet below
    z=1 (iolet 0), outlet above z=side (iolet 0), walls on the x and y faces,
    cut distances rand() % 10000 / 1e4 for every link as the reference fixture
    draws them."""
    cx, cy, cz = (CX15, CY15, CZ15) if q == 15 else (CX19, CY19, CZ19)
    rnd = glibc_rand_sequence()
    mask = np.zeros(8, dtype=np.uint64)
    recs = []
    lo, hi = 1, side
    for i in range(8):
        for j in range(8):
            for k in range(8):
                if not (lo <= i <= hi and lo <= j <= hi and lo <= k <= hi):
                    continue
                l = (i * 8 + j) * 8 + k
                mask[l >> 6] |= np.uint64(1) << np.uint64(l & 63)
                wm = im = 0
                ioid = -1
                had_in = had_out = False
                cuts = np.full(q - 1, -1.0, dtype=np.float32)
                for d in range(1, q):
                    ni, nj, nk = i + cx[d], j + cy[d], k + cz[d]
                    rd = np.float32(float(next(rnd) % 10000) / 10000.0)
                    if nk < lo:
                        im |= 1 << (d - 1)
                        ioid = 0
                        had_in = True
                        cuts[d - 1] = rd
                    elif nk > hi:
                        im |= 1 << (d - 1)
                        ioid = 0
                        had_out = True
                        cuts[d - 1] = rd
                    elif ni < lo or nj < lo or ni > hi or nj > hi:
                        wm |= 1 << (d - 1)
                        cuts[d - 1] = rd
                if wm or im:
                    st = capi.SITE_INLET if had_in else (capi.SITE_OUTLET if had_out else capi.SITE_FLUID)
                    recs.append((l, wm, im, ioid, st, cuts))
    g = ArrayGeometry(q, (1, 1, 1), [[0, 0, 0]], mask.reshape(1, 8),
                      [r[0] for r in recs], [r[1] for r in recs], [r[2] for r in recs],
                      [r[3] for r in recs], [r[4] for r in recs],
                      np.array([r[5] for r in recs]).reshape(-1, q - 1))
    inl = [InOutLetCosine((2.5, 2.5, 0.5), (0, 0, 1), density_mean=1.001)]
    outl = [InOutLetCosine((2.5, 2.5, side + 0.5), (0, 0, -1), density_mean=0.999)]
    return g, inl, outl


def anisotropic(n: int, q: int) -> np.ndarray:
    """f[d] = (d+1)/10 + site/100 (Code/tests/lb/LbTestsHelper.h:165-183)."""
    d = np.arange(q, dtype=np.float64)
    s = np.arange(n, dtype=np.float64)
    return (d[None, :] + 1.0) / 10.0 + s[:, None] / 100.0


def steady_parabolic_inlets(geom):
    inl = []
    for k in range(geom.n_inlets):
        pos, nrm, r = geom.iolet(False, k)
        inl.append(InOutLetParabolicVelocity(pos, nrm, radius=r, max_speed=0.03, warmup_steps=40))
    return inl
