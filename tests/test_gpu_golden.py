"""The CUDA update against the compiled reference's own outputs, through the C ABI.

Every D3Q19 golden vector in tests/golden (written by the reference's LB code
compiled from its sources: LBGK and TRT, SBB and BFL walls, Nash and Ladd iolets,
anisotropic four-cube states) is reproduced bit for bit by the FP64 device path,
and so is the reference run on a HemeLB .gmy geometry read by hlbg_read_gmy (the
reference's large_cylinder.gmy re-written by this library's writer).  These
tests need no reference tree: the fixtures travel with the repository.
"""
import os

import numpy as np
import pytest

from hemelb_gb300.lbm import LBM, SyntheticGeometry
from tests import golden_cases

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
D3Q19 = [n for n in golden_cases.NAMES if "d3q19" in n]


def _run(g, p, inl, outl, steps, f0=None):
    # ArrayGeometry (the four-cube fixture) exposes its C view; it stays alive here
    s = LBM(g if isinstance(g, SyntheticGeometry) else g.view, p, inl, outl)
    s.SetInitialConditions()
    if f0 is not None:
        s.PutF(f0, 0)
        s.PutF(f0, 1)
    s.DoTimeStep(steps)
    return s.GetFOld().reshape(-1), s.GetFNew().reshape(-1)


@pytest.mark.parametrize("name", D3Q19)
def test_device_update_equals_reference_golden(name):
    z = np.load(os.path.join(HERE, "golden", name + ".npz"))
    g, inl, outl, p, steps, f0 = golden_cases.build(name)
    f_old, f_new = _run(g, p, inl, outl, steps, f0)
    assert f_old.size == int(z["n"]) * 19
    assert np.array_equal(f_old, z["f_old"])
    assert np.array_equal(f_new, z["f_new"])


@pytest.mark.parametrize("kernel", sorted(golden_cases.GMY_KERNELS))
def test_device_update_on_gmy_geometry_equals_reference(kernel):
    """hlbg_read_gmy -> device layout -> FP64 update: equal to the reference's
    distributions on the same HemeLB geometry file after 60 steps."""
    z = np.load(os.path.join(HERE, "golden", "large_cylinder_%s.npz" % golden_cases.GMY_KERNELS[kernel]))
    g, inl, outl, p, steps = golden_cases.gmy_case(golden_cases.GMY_FIXTURE, kernel)
    f_old, f_new = _run(g, p, inl, outl, steps)
    assert f_old.size == int(z["n"]) * 19
    assert np.array_equal(f_old, z["f_old"])
    assert np.array_equal(f_new, z["f_new"])
