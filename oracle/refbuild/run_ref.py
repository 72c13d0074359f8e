"""Run the compiled reference LB code on an oracle-built domain (test infrastructure)."""
from __future__ import annotations

import os
import struct
import subprocess
import tempfile

import numpy as np

from oracle.refbuild.build_ref import build


def run_reference(orc, nsteps: int, variant: str = "scalar", mode: int = 0, t_start: int | None = None,
                  f0: np.ndarray | None = None, f1: np.ndarray | None = None):
    """Run `nsteps` of the reference's own streamers over oracle `orc`'s domain.

    Returns (tau_used, t_end, f_old, f_new) with f arrays of N*Q+1 doubles.
    mode=1 stops after the last StreamAndCollide/PostStep without the final swap.
    """
    exes = build()
    if variant not in exes:
        raise RuntimeError("reference variant %s not available" % variant)
    a = orc.arrays()
    n, q = orc.n, orc.q
    p = orc.p
    with tempfile.TemporaryDirectory() as td:
        fin = os.path.join(td, "in.bin")
        fout = os.path.join(td, "out.bin")
        with open(fin, "wb") as fh:
            fh.write(struct.pack("<iq", q, n))
            fh.write(struct.pack("<6q", *orc.type_count))
            fh.write(struct.pack("<4i", p.kernel, p.wall, p.inlet, p.outlet))
            fh.write(struct.pack("<d", p.tau))
            fh.write(struct.pack("<ii", nsteps, mode))
            fh.write(struct.pack("<Q", orc.t1 if t_start is None else t_start))
            fh.write(struct.pack("<ii", p.n_inlets, p.n_outlets))
            for k in range(p.n_inlets):
                fh.write(bytes(p.inlets[k]))
            for k in range(p.n_outlets):
                fh.write(bytes(p.outlets[k]))
            fh.write(a["nbr"].astype(np.int64).tobytes())
            fh.write(a["wall_mask"].astype(np.uint32).tobytes())
            fh.write(a["iolet_mask"].astype(np.uint32).tobytes())
            fh.write(a["iolet_id"].astype(np.int32).tobytes())
            fh.write(np.ctypeslib.as_array(orc.dom.site_type, (n,)).astype(np.int8).tobytes())
            fh.write(a["cut"].astype(np.float64).tobytes())
            fh.write(a["coords"].astype(np.int64).tobytes())
            fh.write((orc.f_old if f0 is None else f0).astype(np.float64).tobytes())
            fh.write((orc.f_new if f1 is None else f1).astype(np.float64).tobytes())
        r = subprocess.run([exes[variant], fin, fout], capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("reference run failed (%d): %s" % (r.returncode, r.stderr))
        raw = open(fout, "rb").read()
    tau_used, t_end = struct.unpack_from("<dQ", raw, 0)
    m = n * q + 1
    arr = np.frombuffer(raw, dtype=np.float64, offset=16)
    return tau_used, t_end, arr[:m].copy(), arr[m:2 * m].copy()
