#!/usr/bin/env python
"""Benchmark of the GB300 lattice-Boltzmann update (fluid MLUPS, % of HBM roofline).

Workload (default): seeded random vascular forest in a 1280^3 box of sparse 8^3
blocks (6 trees of depth 7, root radius 60, Murray radii, branch angles 20-70
degrees, segment length 6-10 x radius), 222,966,063 fluid sites; D3Q19 TRT
(Lambda = 3/16), simple bounce-back walls, Nash pressure inlets at density 1.001
and outlets at 1.0, distributions stored as FP32 deviations from the rest
weights.  A "step" is one full LB time step over every fluid site.  The
distribution arrays (tens of GB) are far larger than the 129 MB L2, so no flush
is needed between steps.

Arms:
  default           the CUDA update through libhemelb_gb300.so's C ABI
  --impl reference  the reference's CPU algorithm on this host's cores (the
                    oracle port, OpenMP over all cores), on a bounded Morton-
                    contiguous sample of the same geometry.
Under torchrun (--gpus N > 1) each rank runs an independent replica on its own
GPU ("replicas only": the single-device update has no data-path exchange).
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

RANK = int(os.environ.get("RANK", "0"))
WORLD = int(os.environ.get("WORLD_SIZE", "1"))
LOCAL_RANK = int(os.environ.get("LOCAL_RANK", "0"))
if WORLD > 1 and "CUDA_VISIBLE_DEVICES" not in os.environ:
    os.environ["CUDA_VISIBLE_DEVICES"] = str(LOCAL_RANK)

import numpy as np  # noqa: E402

B_ALG = {0: 304, 1: 152, 2: 76}  # algorithmic bytes per fluid-site update (2 * 19 * elem)
# the update kernel each launch shape runs (hlbg_set_launch_variant)
KERNEL_OF_VARIANT = {-1: "k_stream_collide<P, 128, 2>", 0: "k_stream_collide<P, 128, 10>",
                     1: "k_stream_collide<P, 128, 8>", 2: "k_stream_collide<P, 256, 4>",
                     3: "k_stream_collide<P, 512, 2>", 4: "k_stream_collide_block<P, 256, 4>",
                     5: "k_stream_collide_listed<P, 128, 9>", 6: "k_stream_collide_listed<P, 128, 8>",
                     7: "k_stream_collide_listed<P, 64, 16>", 8: "k_stream_collide_pipe<P, 31, S>"}
DTYPE = {0: "f64", 1: "f32", 2: "f16-storage/f32"}
METRIC = "fluid MLUPS (D3Q19 LB update)"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gpu", choices=["gpu", "reference"])
    ap.add_argument("--workload", default="tree", choices=["tree", "pipe", "bifurcation"])
    ap.add_argument("--roots", type=int, default=6)
    ap.add_argument("--box", type=int, default=1280)
    ap.add_argument("--depth", type=int, default=7)
    ap.add_argument("--root-radius", type=float, default=60.0)
    ap.add_argument("--variant", type=int, default=-1,
                    help="launch shape of the update (hlbg_set_launch_variant); -1: autotune")
    ap.add_argument("--precision", default="fp32dev", choices=["fp64", "fp32dev", "fp16"])
    ap.add_argument("--e2e-steps", type=int, default=20)
    ap.add_argument("--check-interval", type=int, default=6,
                    help="StabilityTester check interval of the e2e path (hlbg_set_monitor_interval): "
                         "the reference checks once per phased-broadcast round trip, 2 x tree depth "
                         "steps, i.e. 6 on a 1000-rank run (spread factor 10)")
    ap.add_argument("--ref-seconds", type=float, default=10.0,
                    help="target length of the reference arm's timed region")
    ap.add_argument("--cpu-sites", type=int, default=2_000_000,
                    help="fluid sites in the CPU sample (Morton-contiguous blocks)")
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--members", type=int, default=512)
    ap.add_argument("--checkpoints", default="",
                    help="tree_precision report: comma-separated steps at which to compare the forms")
    ap.add_argument("--report", default=None, choices=["precision", "steady", "ensemble", "tree_precision"],
                    help="print a report instead of the throughput line")
    return ap.parse_args()


def dist_init():
    if WORLD <= 1:
        return None
    import torch.distributed as dist
    dist.init_process_group("gloo")
    return dist


def barrier(dist):
    if dist is not None:
        dist.barrier()


def max_over_ranks(dist, v: float) -> float:
    if dist is None:
        return v
    import torch
    t = torch.tensor([v], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def make_case(args):
    from hemelb_gb300 import capi, cases
    prec = {"fp64": capi.FP64, "fp32dev": capi.FP32DEV, "fp16": capi.FP16}[args.precision]
    if args.workload == "tree":
        c = cases.tree(seed=7, box_sites=args.box, n_roots=args.roots, depth=args.depth,
                       root_radius=args.root_radius, precision=prec)
        cfg = {"workload": "random vascular forest, %d trees of depth %d (root radius %g) in a %d^3 box "
               "of 8^3 blocks" % (args.roots, args.depth, args.root_radius, args.box),
               "lattice": "D3Q19", "kernel": "TRT (Lambda=3/16)", "wall": "SimpleBounceBack",
               "iolets": "Nash pressure, inlet 1.001 / outlets 1.0", "storage": args.precision,
               "seed": 7}
    elif args.workload == "pipe":
        c = cases.pipe(precision=prec)
        cfg = {"workload": "straight pipe R=10 L=80", "lattice": "D3Q19", "kernel": "LBGK tau=0.8",
               "wall": "SimpleBounceBack", "iolets": "Nash 1.001/0.999", "storage": args.precision}
    else:
        c = cases.bifurcation(precision=prec)
        cfg = {"workload": "bifurcation R=24 L=200 seed 1234", "lattice": "D3Q19",
               "kernel": "LBGK tau=0.6", "wall": "BFL", "iolets": "Ladd pulsatile inlet, Nash outlets",
               "storage": args.precision}
    return c, prec, cfg


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 200 ms during a region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self):
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        self.p = None

    def start(self):
        try:
            self.p = subprocess.Popen(["nvidia-smi", "--query-gpu=" + self.Q,
                                       "--format=csv,noheader,nounits", "-lms", "200"],
                                      stdout=self.f, stderr=subprocess.DEVNULL)
        except OSError:
            self.p = None
        time.sleep(0.3)

    def stop(self):
        if self.p is None:
            return None
        time.sleep(0.25)
        self.p.terminate()
        try:
            self.p.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.p.kill()
        self.f.flush()
        rows = []
        with open(self.f.name) as fh:
            for line in fh:
                parts = [x.strip() for x in line.split(",")]
                if len(parts) >= 9:
                    rows.append(parts)
        os.unlink(self.f.name)
        dev = os.environ.get("CUDA_VISIBLE_DEVICES", "0").split(",")[0]
        mine = [r for r in rows if r[0] == dev] or rows
        if not mine:
            return None
        sm = [float(r[1]) for r in mine if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in mine if r[2].replace(".", "").isdigit()]
        pw = [float(r[3]) for r in mine if r[3].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in mine for k in range(4) if r[5 + k].lower() == "active"})
        load = [s for s, p in zip(sm, pw)] if sm else []
        return {"sm_mhz": statistics.median(load) if load else None,
                "sm_max_mhz": max(mx) if mx else None,
                "power_w_max": max(pw) if pw else None,
                "samples": len(mine), "reasons": reasons}


def measured_peak():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as fh:
            return float(json.load(fh)["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def profile_traffic(kernel_tag: str):
    """dram bytes per fluid-site update of the dominant kernel from the committed
    ncu summary (profiles/<tag>.md line `dram_bytes_per_site: X`), or None."""
    p = os.path.join(ROOT, "profiles", kernel_tag + ".md")
    try:
        for line in open(p):
            if line.strip().startswith("dram_bytes_per_site:"):
                return float(line.split(":", 1)[1].split()[0])
    except OSError:
        pass
    return None


# ---------------------------------------------------------------------------
# CPU sample: Morton-contiguous blocks of the same geometry through the oracle
# ---------------------------------------------------------------------------
def cpu_sample(case, n_sites: int, seconds: float, threads: int):
    from hemelb_gb300 import capi
    from oracle.oracle import ORDER_SCALAR, OracleLBM
    g = case.geometry
    bytes_ = np.ascontiguousarray(g.fluid_mask).view(np.uint8)
    table = np.array([bin(i).count("1") for i in range(256)], dtype=np.int64)
    per_block = table[bytes_].reshape(g.n_blocks, 64).sum(axis=1)
    nb = int(np.searchsorted(np.cumsum(per_block), n_sites) + 1)
    nb = min(nb, g.n_blocks)
    keep = g.link_site < nb * 512
    arrays = {
        "block_coords": np.ascontiguousarray(g.block_coords[:nb]),
        "fluid_mask": np.ascontiguousarray(g.fluid_mask[:nb]),
        "link_site": np.ascontiguousarray(g.link_site[keep]),
        "wall_mask": np.ascontiguousarray(g.wall_mask[keep]),
        "iolet_mask": np.ascontiguousarray(g.iolet_mask[keep]),
        "iolet_id": np.ascontiguousarray(g.iolet_id[keep]),
        "site_type": np.ascontiguousarray(g.site_type[keep]),
    }
    v = capi.Geometry()
    v.q, v.block_size = 19, 8
    v.blocks[:] = g.blocks
    v.n_blocks = nb
    v.block_coords = arrays["block_coords"].ctypes.data_as(C.POINTER(C.c_int32))
    v.fluid_mask = arrays["fluid_mask"].ctypes.data_as(C.POINTER(C.c_uint64))
    v.n_link_sites = int(keep.sum())
    v.link_site = arrays["link_site"].ctypes.data_as(C.POINTER(C.c_int64))
    v.wall_mask = arrays["wall_mask"].ctypes.data_as(C.POINTER(C.c_uint32))
    v.iolet_mask = arrays["iolet_mask"].ctypes.data_as(C.POINTER(C.c_uint32))
    v.iolet_id = arrays["iolet_id"].ctypes.data_as(C.POINTER(C.c_int32))
    v.site_type = arrays["site_type"].ctypes.data_as(C.POINTER(C.c_int8))
    o = OracleLBM(v, case.params, case.inlets, case.outlets, order=ORDER_SCALAR)
    o.set_equilibrium()
    o.step(1, threads)  # warm-up (page faults, thread pool)
    t0 = time.perf_counter()
    o.step(1, threads)
    one = time.perf_counter() - t0
    k = max(1, int(seconds / max(one, 1e-6)))
    t0 = time.perf_counter()
    o.step(k, threads)
    dt = time.perf_counter() - t0
    return o.n, k, dt, o


def run_reference_arm(args):
    threads = os.cpu_count() or 1
    case, prec, cfg = make_case(args)
    cfg["storage"] = "fp64"  # the reference's own distributions are doubles
    from oracle.oracle import ORDER_SCALAR, OracleLBM  # noqa: F401
    n, _, _, o = cpu_sample(case, args.cpu_sites, 0.0, threads)
    for _ in range(args.warmup):
        o.step(1, threads)
    # each bench step is m LB time steps over the sample, m chosen so that the
    # timed region lasts about --ref-seconds
    t0 = time.perf_counter()
    o.step(1, threads)
    one = time.perf_counter() - t0
    m = max(1, int(args.ref_seconds / max(one * args.steps, 1e-9)))
    t0 = time.perf_counter()
    for _ in range(args.steps):
        o.step(m, threads)
    dt = time.perf_counter() - t0
    mlups = n * m * args.steps / dt / 1e6
    sample = ("%d fluid sites (the first Morton-ordered blocks of the workload), %d LB steps per bench "
              "step, FP64, scalar (aarch64) evaluation order, OpenMP over %d threads" % (n, m, threads))
    cfg["lb_steps_per_bench_step"] = m
    line = {"impl": "reference", "metric": METRIC, "value": mlups, "unit": "MLUPS", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt / args.steps * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded generator)", "config": cfg,
            "cpu_baseline": {"value": mlups, "unit": "MLUPS", "cores": threads, "kind": "port",
                             "sample": sample},
            "e2e": {"value": mlups, "unit": "MLUPS", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def main():
    args = parse()
    if args.report:
        from hemelb_gb300 import cases, reports
        if args.report == "precision":
            print(json.dumps(reports.precision_report(steps=args.steps)), flush=True)
        elif args.report == "tree_precision":
            cps = [int(c) for c in args.checkpoints.split(",") if c] or None
            print(json.dumps(reports.tree_precision_report(steps=args.steps, roots=args.roots,
                                                           box=args.box, depth=args.depth,
                                                           root_radius=args.root_radius,
                                                           checkpoints=cps)), flush=True)
        elif args.report == "ensemble":
            print(json.dumps(reports.ensemble_report(args.members, steps=args.steps,
                                                     warmup=args.warmup)), flush=True)
        else:
            c = cases.pipe()
            # Poiseuille centre-line speed of the pipe's pressure drop, as U_ref
            print(json.dumps(reports.steady_report(c, u_ref=0.01)), flush=True)
        return
    if args.impl == "reference":
        if RANK == 0:
            run_reference_arm(args)
        return
    dist = dist_init()
    from hemelb_gb300 import capi
    from hemelb_gb300.lbm import LBM
    t_setup = time.perf_counter()
    case, prec, cfg = make_case(args)
    t_gen = time.perf_counter() - t_setup
    lbm = case.solver(prec)
    t_layout = time.perf_counter() - t_setup - t_gen
    n = lbm.n_sites
    lbm.SetInitialConditions()
    # launch shape picked by the library's autotuner (its trial steps are warm-up)
    if args.variant < 0:
        variant, tuned_ms = lbm.autotune(3)
    else:
        variant = args.variant
        lbm.SetLaunchVariant(variant)
    lbm.DoTimeStep(args.warmup)
    # ---- device-resident timed region ---------------------------------------
    sampler = ClockSampler()
    barrier(dist)
    lbm._lib.hlbg_sync(lbm.ctx)
    sampler.start()
    ms = lbm.time_steps(args.steps)
    clocks = sampler.stop()
    barrier(dist)
    ms = max_over_ranks(dist, ms)
    value = WORLD * n * args.steps / (ms / 1e3) / 1e6
    # ---- dominant kernel: per-launch device time -----------------------------
    kms, pms = lbm.time_kernels(args.steps)
    per_launch = kms / args.steps
    peak, peak_kind = measured_peak()
    achieved = B_ALG[prec] * n / (per_launch / 1e3) / 1e9
    if prec == 0:  # FP64 runs two CTAs per SM in every shape, the fluid list from index 4 up
        kname = ("k_stream_collide_listed<0, %d, 2>" % (64 if variant == 7 else 128)) if variant >= 4 \
            else "k_stream_collide<0, 128, 2>"
    else:
        kname = KERNEL_OF_VARIANT.get(variant, "k_stream_collide").replace("<P", "<%d" % prec)
        kname = kname.replace(", S>", ", %d>" % (4 if prec == 1 else 8))
    base = kname.split("<")[0]
    # DRAM bytes per site from the ncu capture of one launch of this kernel on a small
    # case of the same generator (one tree in a 512^3 box, root radius 50, depth 6:
    # 16.9M sites, 10.5% boundary sites against the forest's 9.6%), scaled by sites
    tps = profile_traffic("%s_%s_%s" % (base, args.precision, args.workload))
    roofline = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": achieved / peak, "peak_source": peak_kind,
                "traffic": (tps * n if tps is not None else None),
                "traffic_source": "ncu dram bytes per site of a small case of the same generator, x sites",
                "algorithmic_bytes_per_launch": B_ALG[prec] * n,
                "kernel": "hlbg::" + kname, "launch_ms": per_launch}
    # ---- end to end through the C ABI: per step, H2D of that step's iolet values,
    # the update with the StabilityTester fused into it on its check cadence, and the
    # D2H read-back of the stats (stability, mass, max |du| for the convergence
    # test), synchronous
    st = capi.Stats()
    ke = max(1, min(args.e2e_steps, args.steps))

    def e2e_rate(interval):
        capi.check(lbm._lib.hlbg_set_monitor_interval(lbm.ctx, interval), lbm.ctx)
        for _ in range(interval + 1):  # one full check cycle before the clock starts
            capi.check(lbm._lib.hlbg_step_monitored(lbm.ctx, 1, C.byref(st)), lbm.ctx)
        barrier(dist)
        lbm._lib.hlbg_sync(lbm.ctx)
        t0 = time.perf_counter()
        for _ in range(ke):
            rc = lbm._lib.hlbg_step_monitored(lbm.ctx, 1, C.byref(st))
            if rc not in (0, capi.HLBG_ERR_UNSTABLE):
                capi.check(rc, lbm.ctx)
        dt = time.perf_counter() - t0
        barrier(dist)
        return WORLD * n * ke / max_over_ranks(dist, dt) / 1e6

    every = e2e_rate(1)
    cadence = e2e_rate(args.check_interval)
    n_io = len(case.inlets) + len(case.outlets)
    e2e = {"value": cadence, "unit": "MLUPS", "steps": ke,
           "h2d_bytes_per_step": 2 * 8 * n_io, "d2h_bytes_per_step": 5 * 8,
           "check_interval": args.check_interval, "value_check_every_step": every,
           "path": "hlbg_step_monitored(1) per step: iolet values in, update with the fused "
                   "StabilityTester checking every %d steps, its stats (mass, max |du|, min f, "
                   "unstable count) out" % args.check_interval}
    stable = st.unstable_sites == 0 and st.time_step > 0
    # ---- CPU baseline ---------------------------------------------------------
    cpu = None
    if RANK == 0 and not args.no_cpu:
        threads = os.cpu_count() or 1
        cn, ck, cdt, _ = cpu_sample(case, args.cpu_sites, args.cpu_seconds, threads)
        cpu = {"value": cn * ck / cdt / 1e6, "unit": "MLUPS", "cores": threads, "kind": "port",
               "sample": "%d fluid sites (first Morton-ordered blocks of the same geometry), %d steps, "
                         "FP64 oracle, scalar order, OpenMP" % (cn, ck)}
    launches = args.steps * int(lbm._lib.hlbg_launches_per_step(lbm.ctx))
    cfg.update({"fluid_sites": int(n), "slots": int(lbm.n_slots), "launch_variant": int(variant),
                "collision_counts": list(lbm.collision_counts), "device_bytes": lbm.device_bytes(),
                "l2": "inputs (distribution arrays) far larger than L2; no flush",
                "setup_s": {"generate": round(t_gen, 2), "layout_upload": round(t_layout, 2)},
                "parallelism": "replicas" if WORLD > 1 else "single GPU"})
    line = {"metric": METRIC, "value": value, "unit": "MLUPS", "n_gpus": WORLD, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": DTYPE[prec],
            "data": "synthetic (seeded generator)", "config": cfg, "roofline": roofline,
            "cpu_baseline": cpu, "e2e": e2e, "clocks": clocks, "gpu_launches": launches,
            "stable": bool(stable)}
    if RANK == 0:
        print(json.dumps(line), flush=True)
    lbm.close()
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
