"""The C++ plugin layer over the C ABI (include/hemelb_gb300_hemelb.hpp) compiles
against the reference's own headers and satisfies its lb::streamer concept
(Code/lb/concepts.h:91-102); skipped where the reference sources are absent."""
import os
import subprocess

import pytest

from hemelb_gb300 import capi
from oracle.refbuild.build_ref import REF

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.mark.skipif(not os.path.isdir(REF), reason="reference sources not present")
def test_plugin_types_satisfy_reference_concepts(tmp_path):
    exe = tmp_path / "adapter_concept"
    cmd = ["g++", "-std=c++20", "-O0", "-DNDEBUG", "-I", os.path.join(ROOT, "oracle", "refbuild", "shim"),
           "-I", REF, "-I", os.path.join(ROOT, "include"), os.path.join(ROOT, "tests", "cpp", "adapter_concept.cc"),
           os.path.join(REF, "lb", "iolets", "InOutLet.cc"), os.path.join(REF, "lb", "iolets", "InOutLetCosine.cc"),
           os.path.join(REF, "lb", "iolets", "InOutLetVelocity.cc"),
           os.path.join(REF, "lb", "iolets", "InOutLetParabolicVelocity.cc"),
           os.path.join(REF, "geometry", "SiteDataBare.cc"),
           capi.LIB_PATH, "-Wl,-rpath," + os.path.dirname(capi.LIB_PATH), "-o", str(exe)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    r = subprocess.run([str(exe)], capture_output=True, text=True)
    assert r.returncode == 0
