"""Recipe: compile the reference's LB code into oracle/_ref/ (test infrastructure).

Compiles HemeLB's own sources where they lie (lattices, LBGK kernel, Normal
collision, the BulkStreamer / StreamerTypeFactory / SimpleBounceBack / BFL / Nash /
Ladd link streamers, the cosine and parabolic iolets and SiteData) together with
ref_driver.cc and the serial shims in oracle/refbuild/shim (which stand in for the
MPI-bound Domain, FieldData, BoundaryValues, property cache and logger).  Two
binaries: the scalar Lattice path (what an aarch64 build compiles) and, on x86_64,
the SSE3 path (HEMELB_USE_SSE3, what an x86_64 build compiles by default).

The reference tree is only present on the development machine; without it the
recipe reports that and builds nothing.
"""
from __future__ import annotations

import os
import platform
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(os.path.dirname(HERE), "_ref")
REF = os.environ.get("HEMELB_REFERENCE", "/root/reference") + "/Code"
SOURCES = ["lb/iolets/InOutLet.cc", "lb/iolets/InOutLetCosine.cc", "lb/iolets/InOutLetVelocity.cc",
           "lb/iolets/InOutLetParabolicVelocity.cc", "geometry/SiteDataBare.cc"]


def available() -> bool:
    return os.path.isdir(REF)


def targets():
    t = {"scalar": []}
    if platform.machine() in ("x86_64", "AMD64"):
        t["sse3"] = ["-DHEMELB_USE_SSE3", "-msse3"]
    return t


def build(force: bool = False) -> dict:
    """Return {variant: path} of the built reference drivers (empty without the sources)."""
    if not available():
        return {}
    os.makedirs(OUT, exist_ok=True)
    deps = [os.path.join(HERE, "ref_driver.cc"), __file__]
    for root, _, files in os.walk(os.path.join(HERE, "shim")):
        deps += [os.path.join(root, f) for f in files]
    out = {}
    for name, flags in targets().items():
        exe = os.path.join(OUT, "ref_lbm_" + name)
        out[name] = exe
        if (not force and os.path.exists(exe)
                and all(os.path.getmtime(d) <= os.path.getmtime(exe) for d in deps)):
            continue
        cmd = (["g++", "-std=c++20", "-O2", "-ffp-contract=off", "-DNDEBUG"] + flags
               + ["-I", os.path.join(HERE, "shim"), "-I", REF, os.path.join(HERE, "ref_driver.cc")]
               + [os.path.join(REF, s) for s in SOURCES] + ["-o", exe + ".tmp"])
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("reference build failed:\n" + r.stderr[-4000:])
        os.replace(exe + ".tmp", exe)
    return out


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
