"""Regenerate the golden vectors with the reference's own LB code compiled from
its sources (oracle/refbuild, scalar evaluation order; TRT from the reference's
TRT.h with the recipe's build-time patch).  Run in a checkout that has the
reference tree:  python tests/golden/make_golden.py [name ...]"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from hemelb_gb300.build import build as build_lib  # noqa: E402
from oracle.build import build as build_oracle  # noqa: E402
from oracle.oracle import ORDER_SCALAR, OracleLBM  # noqa: E402
from oracle.refbuild.run_ref import run_reference  # noqa: E402
from tests import golden_cases  # noqa: E402


def main():
    build_lib()
    build_oracle()
    out_dir = os.path.dirname(os.path.abspath(__file__))
    for name in (sys.argv[1:] or golden_cases.NAMES):
        g, inl, outl, p, steps, f0 = golden_cases.build(name)
        o = OracleLBM(g.view, p, inl, outl, order=ORDER_SCALAR)
        o.set_equilibrium()
        if f0 is not None:
            o.f_old[: f0.size] = f0.reshape(-1)
            o.f_new[: f0.size] = f0.reshape(-1)
        tau_used, t_end, f_old, f_new = run_reference(o, steps, "scalar")
        assert tau_used == p.tau
        nbr = np.ctypeslib.as_array(o.dom.nbr, (o.n * o.q,)).copy()
        np.savez_compressed(os.path.join(out_dir, name + ".npz"), n=o.n, q=o.q, steps=steps,
                            t_end=t_end, nbr=nbr, f_old=f_old[:-1], f_new=f_new[:-1])
        print(name, o.n, "sites", steps, "steps")


if __name__ == "__main__":
    main()
