"""In-tree build of libhemelb_gb300.so (CUDA sm_103a + host C++).

The FP64 kernel translation unit is compiled with --fmad=false so that no
multiply-add is fused (the plain form reproduces the reference's arithmetic
operation by operation); host code is compiled with -ffp-contract=off for the
same reason (the iolet density and equilibrium values it computes feed the
kernels).
"""
from __future__ import annotations

import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libhemelb_gb300.so")

NVCC = os.environ.get("NVCC", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off",
          "-I", os.path.join(HERE, "..", "include")]

UNITS = [
    ("lb_fp64.cu", ["--fmad=false"]),
    ("lb_fp32.cu", []),
    ("capi.cu", ["--fmad=false"]),
    ("nn_kernels.cu", []),
    ("nn_tc.cu", []),
]
HOST_UNITS = ["synthgeo.cpp", "halo.cpp"]


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed: " + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return r.stdout + r.stderr


def _sources_newer(target, sources):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(s) > t for s in sources)


def build(force: bool = False, verbose: bool = False, defines=(), out: str | None = None,
          build_dir: str | None = None) -> str:
    """Compile the library (in-tree by default).  `defines` are extra -D flags for
    the CUDA units (launch-shape knobs); `out` / `build_dir` redirect the output."""
    lib = out or LIB
    bdir = build_dir or BUILD
    os.makedirs(bdir, exist_ok=True)
    deps = [os.path.join(SRC, f) for f in os.listdir(SRC)] + [
        os.path.join(HERE, "..", "include", "hemelb_gb300.h"),
        os.path.join(HERE, "..", "include", "hemelb_gb300_nn.h")]
    if not force and not _sources_newer(lib, deps + [__file__]):
        return lib
    jobs = []
    objs = []
    for unit, extra in UNITS:
        obj = os.path.join(bdir, unit + ".o")
        objs.append(obj)
        jobs.append([NVCC] + ARCH + COMMON + extra + ["-D" + d for d in defines]
                    + ["-c", os.path.join(SRC, unit), "-o", obj])
    zlib = os.path.exists("/usr/include/zlib.h")  # .gmy reader needs zlib
    for unit in HOST_UNITS:
        obj = os.path.join(bdir, unit + ".o")
        objs.append(obj)
        jobs.append(["g++", "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-pthread",
                     "-DHLBG_HAVE_ZLIB=%d" % int(zlib),
                     "-I", os.path.join(HERE, "..", "include"), "-c",
                     os.path.join(SRC, unit), "-o", obj])
    with ThreadPoolExecutor(max_workers=len(jobs)) as ex:
        outs = list(ex.map(_run, jobs))
    if verbose:
        for o in outs:
            sys.stdout.write(o)
    tmp = lib + ".tmp"
    _run([NVCC] + ARCH + ["-shared", "-o", tmp] + objs + ["-lpthread"] + (["-lz"] if zlib else []))
    os.replace(tmp, lib)
    return lib


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
