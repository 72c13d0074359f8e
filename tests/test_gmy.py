"""HemeLB .gmy geometry files: the reader on the reference's own geometry files,
and writer -> reader round trips of the synthetic geometries."""
import os

import numpy as np
import pytest

from hemelb_gb300 import capi
from hemelb_gb300.lbm import InOutLetCosine, LbmParameters, SyntheticGeometry
from oracle.oracle import OracleLBM
from oracle.refbuild.build_ref import REF as _REF_CODE
from tests import golden_cases

RES = _REF_CODE + "/tests/resources"
needs_ref = pytest.mark.skipif(not os.path.isdir(RES), reason="reference resources not present")


def _domain(g, q=19):
    o = OracleLBM(g.view, LbmParameters(), q=q)
    a = o.arrays()
    return o, a


@pytest.mark.parametrize("maker", [
    lambda: SyntheticGeometry.bifurcation(3, 7.0, 20.0, 1.0, 19, True),
    lambda: SyntheticGeometry.stenosis(6.0, 30, 0.4, 19, True),
    lambda: SyntheticGeometry.bifurcation(4, 6.0, 16.0, 1.0, 15, True),
])
def test_write_read_round_trip(tmp_path, maker):
    g = maker()
    path = str(tmp_path / "g.gmy")
    g.write_gmy(path)
    h = SyntheticGeometry.from_gmy(path, g.q)
    assert h.n_fluid == g.n_fluid
    o1, a1 = _domain(g, g.q)
    o2, a2 = _domain(h, g.q)
    # same reference numbering, push table, SiteData and cut distances
    assert o1.type_count == o2.type_count
    for k in ("nbr", "wall_mask", "iolet_mask", "iolet_id", "coords"):
        assert np.array_equal(a1[k], a2[k]), k
    flagged = (a1["wall_mask"][:, None] | a1["iolet_mask"][:, None]) >> np.arange(g.q - 1, dtype=np.uint32) & 1
    c1 = a1["cut"].reshape(o1.n, -1)[flagged.astype(bool)]
    c2 = a2["cut"].reshape(o2.n, -1)[flagged.astype(bool)]
    assert np.array_equal(c1, c2)
    # the wall normals travel with the file (the format stores one per wall site)
    assert np.array_equal(g.link_site, h.link_site)
    wall = g.wall_mask != 0
    assert g.wall_normal is not None and h.wall_normal is not None
    assert np.allclose(np.linalg.norm(g.wall_normal[wall], axis=1), 1.0, atol=1e-6)
    assert np.array_equal(g.wall_normal[wall], h.wall_normal[wall])


@needs_ref
def test_reads_reference_geometry_files():
    g = SyntheticGeometry.from_gmy(os.path.join(RES, "four_cube.gmy"), 19)
    assert g.n_fluid == 64  # a 4^3 cube (Code/tests/helpers/FourCubeLatticeData.cc)
    types = np.bincount(g.site_type.astype(int), minlength=4)
    assert types[capi.SITE_INLET] == 16 and types[capi.SITE_OUTLET] == 16
    assert g.n_link_sites == 64 - 8  # every site but the 2^3 interior touches a face
    for fn, n in (("large_cylinder.gmy", 5576), ("cyl_l100_r5.gmy", 212400)):
        h = SyntheticGeometry.from_gmy(os.path.join(RES, fn), 19)
        assert h.n_fluid == n


@needs_ref
def test_oracle_matches_reference_on_reference_geometry():
    """The compiled reference and the oracle agree bit for bit on a HemeLB
    geometry file (large_cylinder.gmy), Nash iolets along the cylinder axis."""
    from oracle.refbuild.build_ref import build
    from oracle.refbuild.run_ref import run_reference
    if not build():
        pytest.skip("reference build unavailable")
    g = SyntheticGeometry.from_gmy(os.path.join(RES, "large_cylinder.gmy"), 19)
    inl = [InOutLetCosine((8, 8, 0), (0, 0, 1), density_mean=1.001)]
    outl = [InOutLetCosine((8, 8, 40), (0, 0, -1), density_mean=0.999)]
    p = LbmParameters(tau=0.8)
    o = OracleLBM(g.view, p, inl, outl)
    o.set_equilibrium()
    tau_used, t_end, rf_old, rf_new = run_reference(o, 40, "scalar")
    o.step(40)
    assert np.array_equal(o.f_old[:-1], rf_old[:-1])
    assert np.array_equal(o.f_new[:-1], rf_new[:-1])


@pytest.mark.parametrize("kernel", sorted(golden_cases.GMY_KERNELS))
def test_oracle_on_committed_gmy_fixture_matches_reference_golden(kernel):
    """The committed fixture (the reference's large_cylinder.gmy re-written by this
    library's writer) read by hlbg_read_gmy: the oracle reproduces the compiled
    reference's distributions on it bit for bit.  Needs no reference tree."""
    z = np.load(os.path.join(os.path.dirname(golden_cases.GMY_FIXTURE),
                             "large_cylinder_%s.npz" % golden_cases.GMY_KERNELS[kernel]))
    g, inl, outl, p, steps = golden_cases.gmy_case(golden_cases.GMY_FIXTURE, kernel)
    assert g.n_fluid == int(z["n"]) == 5576
    o = OracleLBM(g.view, p, inl, outl)
    o.set_equilibrium()
    o.step(steps)
    assert np.array_equal(o.f_old[:-1], z["f_old"])
    assert np.array_equal(o.f_new[:-1], z["f_new"])
