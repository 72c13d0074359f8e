"""Recipe: compile the reference's LB code into oracle/_ref/ (test infrastructure).

Compiles HemeLB's own sources where they lie (lattices, LBGK and TRT kernels,
Normal collision, the BulkStreamer / StreamerTypeFactory / SimpleBounceBack / BFL /
Nash / Ladd link streamers, the cosine and parabolic iolets and SiteData) together
with ref_driver.cc and the serial shims in oracle/refbuild/shim (which stand in for
the MPI-bound Domain, FieldData, BoundaryValues, property cache and logger).  Two
binaries: the scalar Lattice path (what an aarch64 build compiles) and, on x86_64,
the SSE3 path (HEMELB_USE_SSE3, what an x86_64 build compiles by default).

TRT: the reference's `Code/lb/kernels/TRT.h` does not compile in this revision.
The recipe copies it into oracle/_ref/patched/ (git-ignored, never committed),
applies the edits in TRT_PATCH there, and puts that directory ahead of the
reference on the include path.  The edits touch only the two defects:

* `MakeOpposites` (TRT.h:42-54) stores a pair for every i with iBar >= i, which
  counts the rest direction as a pair and writes NUMVECTORS/2 + 1 pairs into an
  array of NUMVECTORS/2 (a constant-expression overrun).  The patch keeps the
  pairs with iBar > i; the rest direction is relaxed separately at TRT.h:108-112.
* `CalculateDensityMomentumFeq` / `CalculateFeq` (TRT.h:62-92) call a 9- and a
  5-argument lattice overload on `.f` members that `Lattice.h` and `HydroVars.h`
  do not declare.  The patch routes them to the overloads `Lattice.h` does
  declare (CalculateDensityMomentumFEq(f, density, momentum, velocity, f_eq) at
  Lattice.h:471-483 and CalculateFeq(density, momentum, f_eq)), which are the
  ones LBGK.h:29-53 calls, and indexes f_eq / f_neq directly.

The collision itself (TRT.h:94-122) compiles unchanged.

The reference tree is found through HEMELB_REFERENCE (default: the checkout
beside this development machine's repository); without it the recipe reports that
and builds nothing.
"""
from __future__ import annotations

import os
import platform
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(os.path.dirname(HERE), "_ref")
PATCHED = os.path.join(OUT, "patched")
REF_ROOT = os.environ.get("HEMELB_REFERENCE", "/root/reference")
REF = REF_ROOT + "/Code"
SOURCES = ["lb/iolets/InOutLet.cc", "lb/iolets/InOutLetCosine.cc", "lb/iolets/InOutLetVelocity.cc",
           "lb/iolets/InOutLetParabolicVelocity.cc", "geometry/SiteDataBare.cc"]

# (file, [(old, new), ...]): each `old` must occur exactly once in the reference file.
TRT_PATCH = ("lb/kernels/TRT.h", [
    ("if (iBar >= i) {", "if (iBar > i) {"),
    ("""LatticeType::CalculateDensityMomentumFEq(hydroVars.f,
                                                     hydroVars.density,
                                                     hydroVars.momentum.x,
                                                     hydroVars.momentum.y,
                                                     hydroVars.momentum.z,
                                                     hydroVars.velocity.x,
                                                     hydroVars.velocity.y,
                                                     hydroVars.velocity.z,
                                                     hydroVars.f_eq.f);""",
     """LatticeType::CalculateDensityMomentumFEq(hydroVars.f,
                                                     hydroVars.density,
                                                     hydroVars.momentum,
                                                     hydroVars.velocity,
                                                     hydroVars.f_eq);"""),
    ("""LatticeType::CalculateFeq(hydroVars.density,
                                      hydroVars.momentum.x,
                                      hydroVars.momentum.y,
                                      hydroVars.momentum.z,
                                      hydroVars.f_eq.f);""",
     """LatticeType::CalculateFeq(hydroVars.density,
                                      hydroVars.momentum,
                                      hydroVars.f_eq);"""),
    ("hydroVars.f_neq.f[ii] = hydroVars.f[ii] - hydroVars.f_eq.f[ii];",
     "hydroVars.f_neq[ii] = hydroVars.f[ii] - hydroVars.f_eq[ii];"),
    ("hydroVars.f[iZero] + omega_plus * hydroVars.f_neq.f[iZero]",
     "hydroVars.f[iZero] + omega_plus * hydroVars.f_neq[iZero]"),
    ("(hydroVars.f_neq.f[i] + hydroVars.f_neq.f[iBar])", "(hydroVars.f_neq[i] + hydroVars.f_neq[iBar])"),
    ("(hydroVars.f_neq.f[i] - hydroVars.f_neq.f[iBar])", "(hydroVars.f_neq[i] - hydroVars.f_neq[iBar])"),
])


def available() -> bool:
    return os.path.isdir(REF)


def targets():
    t = {"scalar": []}
    if platform.machine() in ("x86_64", "AMD64"):
        t["sse3"] = ["-DHEMELB_USE_SSE3", "-msse3"]
    return t


def patch_trt() -> str:
    """Write the patched TRT.h under oracle/_ref/patched and return that include root.

    The replacement of f_neq lines may match more than once (CalculateDensityMomentumFeq
    and CalculateFeq hold the same statement); every other edit must match once."""
    rel, edits = TRT_PATCH
    src = open(os.path.join(REF, rel)).read()
    for old, new in edits:
        n = src.count(old)
        if n == 0 or (n > 1 and "f_neq.f[ii]" not in old):
            raise RuntimeError("TRT patch does not apply: %r found %d times" % (old[:40], n))
        src = src.replace(old, new)
    dst = os.path.join(PATCHED, rel)
    os.makedirs(os.path.dirname(dst), exist_ok=True)
    if not os.path.exists(dst) or open(dst).read() != src:
        with open(dst + ".tmp", "w") as fh:
            fh.write(src)
        os.replace(dst + ".tmp", dst)
    return PATCHED


def build(force: bool = False) -> dict:
    """Return {variant: path} of the built reference drivers (empty without the sources)."""
    if not available():
        return {}
    os.makedirs(OUT, exist_ok=True)
    inc = patch_trt()
    deps = [os.path.join(HERE, "ref_driver.cc"), __file__, os.path.join(REF, TRT_PATCH[0])]
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
               + ["-I", os.path.join(HERE, "shim"), "-I", inc, "-I", REF,
                  os.path.join(HERE, "ref_driver.cc")]
               + [os.path.join(REF, s) for s in SOURCES] + ["-o", exe + ".tmp"])
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("reference build failed:\n" + r.stderr[-4000:])
        os.replace(exe + ".tmp", exe)
    return out


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
