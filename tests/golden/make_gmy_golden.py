"""Derive the .gmy fixture and its golden vectors from the reference's own test
geometry (Code/tests/resources/large_cylinder.gmy, a 5,576-site cylinder along z).

1. Read the reference file with this library's reader (hlbg_read_gmy) and write it
   back with this library's writer to tests/golden/large_cylinder_rw.gmy; check
   that the written file decodes to the same sites, push table, SiteData masks,
   iolet ids, cut distances and coordinates as the reference file.
2. Run the reference's own LB code compiled from its sources (oracle/refbuild,
   scalar order) on that geometry with Nash pressure iolets at both ends, LBGK
   and TRT, and store the distributions in tests/golden/large_cylinder_<kernel>.npz.

Run in a checkout that has the reference tree:
    python tests/golden/make_gmy_golden.py
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from hemelb_gb300.build import build as build_lib  # noqa: E402
from oracle.build import build as build_oracle  # noqa: E402
from oracle.oracle import ORDER_SCALAR, OracleLBM  # noqa: E402
from oracle.refbuild.build_ref import REF  # noqa: E402
from oracle.refbuild.run_ref import run_reference  # noqa: E402
from tests.golden_cases import GMY_FIXTURE, GMY_KERNELS, gmy_case  # noqa: E402


def _domain_arrays(geometry):
    o = OracleLBM(geometry.view, gmy_case(None, 0)[3])
    return o.type_count, {k: np.array(v, copy=True) for k, v in o.arrays().items()}


def main():
    build_lib()
    build_oracle()
    from hemelb_gb300.lbm import SyntheticGeometry
    src = os.path.join(REF, "tests", "resources", "large_cylinder.gmy")
    ref_geom = SyntheticGeometry.from_gmy(src, 19)
    ref_geom.write_gmy(GMY_FIXTURE)
    rw_geom = SyntheticGeometry.from_gmy(GMY_FIXTURE, 19)
    assert rw_geom.n_fluid == ref_geom.n_fluid
    c1, a1 = _domain_arrays(ref_geom)
    c2, a2 = _domain_arrays(rw_geom)
    assert c1 == c2
    for k in ("nbr", "wall_mask", "iolet_mask", "iolet_id", "coords", "cut"):
        assert np.array_equal(a1[k], a2[k]), k
    for kernel in GMY_KERNELS:
        g, inl, outl, p, steps = gmy_case(GMY_FIXTURE, kernel)
        o = OracleLBM(g.view, p, inl, outl, order=ORDER_SCALAR)
        o.set_equilibrium()
        tau_used, t_end, f_old, f_new = run_reference(o, steps, "scalar")
        assert tau_used == p.tau
        out = os.path.join(os.path.dirname(GMY_FIXTURE), "large_cylinder_%s.npz" % GMY_KERNELS[kernel])
        np.savez_compressed(out, n=o.n, q=o.q, steps=steps, t_end=t_end, f_old=f_old[:-1],
                            f_new=f_new[:-1])
        print(out, o.n, "sites", steps, "steps")


if __name__ == "__main__":
    main()
