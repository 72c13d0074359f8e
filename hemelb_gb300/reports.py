"""Measurement reports beyond the throughput line of bench.py.

precision_report: the bifurcation workload (parent radius 24, length 200, Murray
daughters, BFL walls, pulsatile Ladd inlet, Nash outlets, LBGK tau 0.6) run in the
FP64 plain form (bit-identical to the CPU oracle, see tests/test_gpu_parity.py),
the FP32-deviation form and the FP16-storage form; the velocity and pressure of the
two reduced forms are compared with FP64 after the same number of steps.

steady_report: steps and device time to steady state, max_site |u_new - u_old| /
U_ref <= tol (the convergence test of Code/lb/StabilityTester.h:160-183), from rest.
"""
from __future__ import annotations

import time

import numpy as np

from . import capi, cases


def _errors(rho, u, rho_ref, u_ref):
    du = u - u_ref
    p_err = np.abs(rho - rho_ref) / 3.0  # lattice pressure p = rho c_s^2
    umag = np.linalg.norm(u_ref, axis=1)
    return {
        "u_rel_l2": float(np.linalg.norm(du) / np.linalg.norm(u_ref)),
        "u_max_abs": float(np.abs(du).max()),
        "u_max_over_peak": float(np.abs(du).max() / umag.max()),
        "p_max_abs": float(p_err.max()),
        "p_rel_l2_of_deviation": float(np.linalg.norm(rho - rho_ref) / np.linalg.norm(rho_ref - 1.0)),
    }


def precision_report(steps: int = 10000, seed: int = 1234, **kw) -> dict:
    case = cases.bifurcation(seed=seed, steps=steps, **kw)
    out = {"workload": "bifurcation seed %d, %d fluid sites, %d steps, LBGK tau 0.6, BFL, "
                       "pulsatile Ladd inlet (peak 0.05, period 2000), Nash outlets"
                       % (seed, case.geometry.n_fluid, steps), "forms": {}}
    ref = None
    for name, prec in (("fp64", capi.FP64), ("fp32dev", capi.FP32DEV), ("fp16", capi.FP16)):
        s = case.solver(prec)
        s.SetInitialConditions()
        t0 = time.perf_counter()
        s.DoTimeStep(steps)
        dt = time.perf_counter() - t0
        rho, u = s.macro()
        st = s.reduce()
        entry = {"seconds": dt, "mlups": s.n_sites * steps / dt / 1e6,
                 "stable": bool(st.unstable_sites == 0)}
        if ref is None:
            ref = (rho, u)
            entry["u_peak"] = float(np.linalg.norm(u, axis=1).max())
        else:
            entry.update(_errors(rho, u, *ref))
        out["forms"][name] = entry
        s.close()
    return out


def steady_report(case, u_ref: float, tol: float = 1e-6, check_every: int = 10,
                  max_steps: int = 200000, precision=None) -> dict:
    """Run from rest until max |du| / U_ref <= tol, checking every `check_every` steps
    with the StabilityTester reduction (the per-step change measured over the last
    step of each interval)."""
    s = case.solver(precision)
    s.SetInitialConditions()
    t0 = time.perf_counter()
    steps = 0
    du = float("inf")
    while steps < max_steps:
        s.DoTimeStep(check_every, sync=False)
        steps += check_every
        st = s.reduce()
        if st.unstable_sites:
            break
        du = st.max_du / u_ref
        if du <= tol:
            break
    dt = time.perf_counter() - t0
    s.close()
    return {"steps": steps, "seconds": dt, "final_rel_du": du, "u_ref": u_ref, "tol": tol,
            "converged": bool(du <= tol)}


def ensemble_report(n_members: int = 512, steps: int = 50, warmup: int = 5, seed: int = 2024) -> dict:
    """Batched ensemble of stenosed pipes (one context, autotuned launch variant,
    CUDA-graph steps) against the same pipes stepped one after another as
    single-geometry contexts (one launch sequence per pipe per step)."""
    import ctypes as C
    case = cases.ensemble(n_members=n_members, seed=seed)
    lib = capi.load()
    t0 = time.perf_counter()
    s = case.solver()
    t_setup = time.perf_counter() - t0
    s.SetInitialConditions()
    variant, tuned_ms = s.autotune(5)
    # every candidate's step time on this workload (the same update bit for bit)
    per_variant = {}
    for v in range(9):
        s.SetLaunchVariant(v)
        s.DoTimeStep(1)
        per_variant[v] = s.time_steps(10) / 10
    s.SetLaunchVariant(variant)
    s.DoTimeStepGraph(warmup)
    ms = C.c_float()
    capi.check(lib.hlbg_sync(s.ctx), s.ctx)
    ev0 = time.perf_counter()
    s.DoTimeStepGraph(steps)
    batched_s = time.perf_counter() - ev0
    st = s.reduce()
    n = s.n_sites
    s.close()
    # sequential: every member in its own context, stepped in turn, one hlbg_step each
    solvers = []
    for m in range(n_members):
        mc = case.member_case(m)
        ms_ = mc.solver()
        ms_.SetInitialConditions()
        ms_.DoTimeStep(warmup)
        solvers.append(ms_)
    for x in solvers:
        capi.check(lib.hlbg_sync(x.ctx), x.ctx)
    t0 = time.perf_counter()
    for _ in range(steps):
        for x in solvers:
            capi.check(lib.hlbg_step(x.ctx, 1, None), x.ctx)
    for x in solvers:
        capi.check(lib.hlbg_sync(x.ctx), x.ctx)
    seq_s = time.perf_counter() - t0
    seq_sites = sum(x.n_sites for x in solvers)
    for x in solvers:
        x.close()
    return {"workload": "%d stenosed pipes (radius 6-20, length 60-240, narrowing 0-70%%, tau 0.55-1.0), "
                        "LBGK, SBB, pulsatile Ladd inlets, Nash outlets, FP32 deviations" % n_members,
            "fluid_sites": int(n), "steps": steps,
            "batched": {"mlups": n * steps / batched_s / 1e6, "seconds": batched_s,
                        "autotuned_variant": variant, "tuned_ms_per_step": tuned_ms,
                        "ms_per_step_by_variant": per_variant,
                        "setup_s": t_setup, "stable": bool(st.unstable_sites == 0)},
            "sequential": {"mlups": seq_sites * steps / seq_s / 1e6, "seconds": seq_s},
            "speedup": (n * steps / batched_s) / (seq_sites * steps / seq_s)}


def tree_precision_report(steps: int = 10000, roots: int = 1, box: int = 1280, depth: int = 7,
                          root_radius: float = 60.0, checkpoints=None) -> dict:
    """The forest generator's workload (TRT, SBB, Nash) in FP64, FP32-deviation and
    FP16-storage forms from rest, stepped side by side; at each checkpoint the
    velocity / pressure error of the reduced forms against FP64 (FP64 is the
    oracle's arithmetic, bit-exact on the GPU).  The default is one tree of the
    benchmark's forest (a cropped forest: the same generator and parameters) run
    long enough for the flow to cross it."""
    case = cases.tree(n_roots=roots, box_sites=box, depth=depth, root_radius=root_radius,
                      precision=capi.FP64)
    cps = sorted({int(c) for c in (checkpoints or [steps // 10, steps // 2, steps]) if 0 < c <= steps})
    forms = (("fp64", capi.FP64), ("fp32dev", capi.FP32DEV), ("fp16", capi.FP16))
    solvers = {}
    for name, prec in forms:
        solvers[name] = case.solver(prec)
        solvers[name].SetInitialConditions()
    n = solvers["fp64"].n_sites
    out = {"workload": "forest of %d tree(s) depth %d (root radius %g) in %d^3, %d fluid sites, TRT, "
                       "SBB walls, Nash inlet 1.001 / outlets 1.0, from rest"
                       % (roots, depth, root_radius, box, n), "checkpoints": []}
    secs = {name: 0.0 for name, _ in forms}
    done = 0
    for cp in cps:
        for name, _ in forms:
            t0 = time.perf_counter()
            solvers[name].DoTimeStep(cp - done)
            secs[name] += time.perf_counter() - t0
        done = cp
        rho_ref, u_ref = solvers["fp64"].macro()
        umag = np.linalg.norm(u_ref, axis=1)
        entry = {"step": cp, "u_peak": float(umag.max()), "u_mean": float(umag.mean())}
        for name in ("fp32dev", "fp16"):
            rho, u = solvers[name].macro()
            entry[name] = _errors(rho, u, rho_ref, u_ref)
            del rho, u
        out["checkpoints"].append(entry)
        del rho_ref, u_ref
    out["mlups"] = {name: n * done / secs[name] / 1e6 for name, _ in forms}
    for s in solvers.values():
        s.close()
    return out
