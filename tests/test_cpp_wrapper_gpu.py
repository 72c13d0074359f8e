"""The C++ host wrapper (include/hemelb_gb300.hpp: GeometryBuilder + Solver) drives
the CUDA update through the C ABI; its result equals the oracle's bit for bit, and
an XTR checkpoint written and read through it restarts the run bit for bit."""
import os
import struct
import subprocess

import numpy as np
import pytest

from hemelb_gb300 import capi
from hemelb_gb300.lbm import LbmParameters
from oracle.oracle import OracleLBM
from tests.helpers import four_cube

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_cpp_wrapper_matches_oracle(tmp_path):
    exe = tmp_path / "wrapper_run"
    r = subprocess.run(["g++", "-std=c++17", "-O2", "-I", os.path.join(ROOT, "include"),
                        os.path.join(ROOT, "tests", "cpp", "wrapper_run.cc"), capi.LIB_PATH,
                        "-Wl,-rpath," + os.path.dirname(capi.LIB_PATH), "-o", str(exe)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-2000:]
    g, inl, outl = four_cube(19, side=6)
    p = LbmParameters(tau=0.7, wall=capi.WALL_BFL)
    o = OracleLBM(g.view, p, inl, outl)
    a = o.arrays()
    n = o.n
    st = np.ctypeslib.as_array(o.dom.site_type, (n,))
    sites = tmp_path / "sites.bin"
    with open(sites, "wb") as fh:
        fh.write(struct.pack("<q", n))
        cut = a["cut"].reshape(n, 18).astype(np.float32)
        for i in range(n):
            x, y, z = a["coords"][i]
            fh.write(struct.pack("<3qIIii", x, y, z, int(a["wall_mask"][i]), int(a["iolet_mask"][i]),
                                 int(a["iolet_id"][i]), int(st[i])))
            fh.write(cut[i].tobytes())
        fh.write(struct.pack("<ii", len(inl), len(outl)))
        for io in inl + outl:
            fh.write(bytes(io))
        fh.write(bytes(p.to_c()))
    out = tmp_path / "f.bin"
    restart = tmp_path / "restart.bin"
    r = subprocess.run([str(exe), str(sites), "40", str(out), str(tmp_path / "state.xtr"), "15", str(restart)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    f = np.fromfile(out, dtype=np.float64).reshape(n, 19)
    o.set_equilibrium()
    o.step(40)
    assert np.array_equal(f, o.fold())
    # the checkpoint restart continues bit for bit, and the fluxes come back
    rr = np.fromfile(restart, dtype=np.float64)
    cont, rest, flux = rr[:n * 19], rr[n * 19:2 * n * 19], rr[2 * n * 19:]
    o.step(15)
    assert np.array_equal(cont.reshape(n, 19), o.fold())
    assert np.array_equal(rest, cont)
    assert flux.shape == (len(inl) + len(outl),) and np.all(np.isfinite(flux))
