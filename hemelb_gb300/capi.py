"""ctypes binding of include/hemelb_gb300.h (the library's C ABI).

The shared library is built in-tree by ``hemelb_gb300.build``.  Loading fails
loudly when it is missing: there is no fallback implementation.
"""
from __future__ import annotations

import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libhemelb_gb300.so")

HLBG_OK, HLBG_ERR_INVAL, HLBG_ERR_OOM, HLBG_ERR_CUDA = 0, 1, 2, 3
HLBG_ERR_UNSTABLE, HLBG_ERR_TIMEOUT, HLBG_ERR_STATE = 4, 5, 6
KERNEL_LBGK, KERNEL_TRT = 0, 1
WALL_SBB, WALL_BFL = 0, 1
IOLET_NASH, IOLET_LADD = 0, 1
FP64, FP32DEV, FP16 = 0, 1, 2
IOLET_COSINE, IOLET_PARABOLIC, IOLET_PULSATILE = 0, 1, 2
SITE_FLUID, SITE_INLET, SITE_OUTLET = 1, 2, 3

NOALLOC_MAX_SLOTS = 65536 * 256

ERRORS = {1: "INVAL", 2: "OOM", 3: "CUDA", 4: "UNSTABLE", 5: "TIMEOUT", 6: "STATE"}


class Geometry(C.Structure):
    _fields_ = [
        ("q", C.c_int32), ("block_size", C.c_int32), ("blocks", C.c_int32 * 3),
        ("n_blocks", C.c_int64), ("block_coords", C.POINTER(C.c_int32)),
        ("fluid_mask", C.POINTER(C.c_uint64)), ("n_link_sites", C.c_int64),
        ("link_site", C.POINTER(C.c_int64)), ("wall_mask", C.POINTER(C.c_uint32)),
        ("iolet_mask", C.POINTER(C.c_uint32)), ("iolet_id", C.POINTER(C.c_int32)),
        ("site_type", C.POINTER(C.c_int8)), ("cut_distance", C.POINTER(C.c_float)),
        ("wall_normal", C.POINTER(C.c_float)),
    ]


class Iolet(C.Structure):
    _fields_ = [
        ("model", C.c_int32), ("pad_", C.c_int32), ("position", C.c_double * 3),
        ("normal", C.c_double * 3), ("density_mean", C.c_double), ("density_amp", C.c_double),
        ("phase", C.c_double), ("period", C.c_double), ("radius", C.c_double),
        ("max_speed", C.c_double), ("vel_period", C.c_double), ("warmup_steps", C.c_uint64),
    ]


class Params(C.Structure):
    _fields_ = [
        ("kernel", C.c_int32), ("wall", C.c_int32), ("inlet", C.c_int32), ("outlet", C.c_int32),
        ("precision", C.c_int32), ("flags", C.c_int32), ("tau", C.c_double),
    ]


class Stats(C.Structure):
    _fields_ = [
        ("mass", C.c_double), ("max_du", C.c_double), ("min_f", C.c_double),
        ("unstable_sites", C.c_int64), ("time_step", C.c_int64),
    ]


class Incomp(C.Structure):
    _fields_ = [
        ("min_density", C.c_double), ("max_density", C.c_double), ("max_velocity", C.c_double),
        ("max_relative_density_difference", C.c_double), ("time_step", C.c_int64),
    ]


# name -> (restype, argtypes)
SIGNATURES = {
    "hlbg_synth_pipe": (C.c_int, [C.c_double, C.c_int32, C.c_int32, C.c_int32, C.POINTER(C.c_void_p)]),
    "hlbg_synth_bifurcation": (C.c_int, [C.c_uint64, C.c_double, C.c_double, C.c_double, C.c_int32,
                                         C.c_int32, C.POINTER(C.c_void_p)]),
    "hlbg_synth_stenosis": (C.c_int, [C.c_double, C.c_int32, C.c_double, C.c_int32, C.c_int32,
                                      C.POINTER(C.c_void_p)]),
    "hlbg_synth_tree": (C.c_int, [C.c_uint64, C.c_int32, C.c_int32, C.c_int32, C.c_double, C.c_int32,
                                  C.c_int32, C.c_int32, C.POINTER(C.c_void_p)]),
    "hlbg_synth_ensemble": (C.c_int, [C.c_uint64, C.c_int32, C.c_int32, C.c_int32, C.POINTER(C.c_void_p)]),
    "hlbg_synth_members": (C.c_int, [C.c_void_p, C.POINTER(C.c_int32), C.POINTER(C.POINTER(C.c_int32)),
                                     C.POINTER(C.POINTER(C.c_double)), C.POINTER(C.POINTER(C.c_double)),
                                     C.POINTER(C.POINTER(C.c_int64))]),
    "hlbg_synth_vessel_box": (C.c_int, [C.c_uint64, C.c_int32, C.c_int32, C.c_int32, C.POINTER(C.c_void_p)]),
    "hlbg_synth_distance": (C.c_int, [C.c_void_p, C.POINTER(C.c_float)]),
    "hlbg_write_gmy": (C.c_int, [C.POINTER(Geometry), C.c_char_p]),
    "hlbg_read_gmy": (C.c_int, [C.c_char_p, C.c_int32, C.POINTER(C.c_void_p)]),
    "hlbg_synth_view": (C.c_int, [C.c_void_p, C.POINTER(Geometry), C.POINTER(C.c_int64),
                                  C.POINTER(C.c_int32), C.POINTER(C.c_int32)]),
    "hlbg_synth_iolet": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32, C.c_double * 3, C.c_double * 3,
                                   C.POINTER(C.c_double)]),
    "hlbg_synth_free": (None, [C.c_void_p]),
    "hlbg_create": (C.c_int, [C.POINTER(Geometry), C.POINTER(Params), C.POINTER(Iolet), C.c_int32,
                              C.POINTER(Iolet), C.c_int32, C.POINTER(C.c_void_p)]),
    "hlbg_destroy": (None, [C.c_void_p]),
    "hlbg_last_error": (C.c_char_p, [C.c_void_p]),
    "hlbg_site_count": (C.c_int64, [C.c_void_p]),
    "hlbg_slot_count": (C.c_int64, [C.c_void_p]),
    "hlbg_launches_per_step": (C.c_int32, [C.c_void_p]),
    "hlbg_collision_counts": (C.c_int, [C.c_void_p, C.POINTER(C.c_int64)]),
    "hlbg_device_bytes": (C.c_size_t, [C.c_void_p]),
    "hlbg_site_order": (C.c_int, [C.c_void_p, C.POINTER(C.c_int64)]),
    "hlbg_site_coords": (C.c_int, [C.c_void_p, C.POINTER(C.c_int32)]),
    "hlbg_init_equilibrium": (C.c_int, [C.c_void_p, C.c_double, C.c_double, C.c_double, C.c_double]),
    "hlbg_init_equilibrium_field": (C.c_int, [C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_double)]),
    "hlbg_step": (C.c_int, [C.c_void_p, C.c_int32, C.c_void_p]),
    "hlbg_sync": (C.c_int, [C.c_void_p]),
    "hlbg_step_graph": (C.c_int, [C.c_void_p, C.c_int32]),
    "hlbg_autotune": (C.c_int, [C.c_void_p, C.c_int32, C.POINTER(C.c_int32), C.POINTER(C.c_float)]),
    "hlbg_run_to_steady": (C.c_int, [C.c_void_p, C.c_double, C.c_double, C.c_int64, C.c_int32,
                                     C.POINTER(C.c_int64), C.POINTER(C.c_int64), C.POINTER(C.c_double)]),
    "hlbg_average_time_levels": (C.c_int, [C.c_void_p]),
    "hlbg_set_launch_variant": (C.c_int, [C.c_void_p, C.c_int32]),
    "hlbg_step_monitored": (C.c_int, [C.c_void_p, C.c_int32, C.POINTER(Stats)]),
    "hlbg_set_monitor_interval": (C.c_int, [C.c_void_p, C.c_int32]),
    "hlbg_incompressibility": (C.c_int, [C.c_void_p, C.POINTER(Incomp)]),
    "hlbg_wall_shear_stress": (C.c_int, [C.c_void_p, C.POINTER(C.c_double)]),
    "hlbg_iolet_flux": (C.c_int, [C.c_void_p, C.POINTER(C.c_double), C.c_int32]),
    "hlbg_set_iolets": (C.c_int, [C.c_void_p, C.POINTER(Iolet), C.c_int32, C.POINTER(Iolet), C.c_int32]),
    "hlbg_write_checkpoint": (C.c_int, [C.c_void_p, C.c_char_p, C.c_uint64, C.c_double,
                                        C.POINTER(C.c_double), C.c_int32]),
    "hlbg_read_checkpoint": (C.c_int, [C.c_void_p, C.c_char_p, C.c_int64, C.POINTER(C.c_uint64)]),
    "hlbg_set_block_tau": (C.c_int, [C.c_void_p, C.POINTER(C.c_double)]),
    "hlbg_stream_and_collide_range": (C.c_int, [C.c_void_p, C.c_int64, C.c_int64]),
    "hlbg_post_step_range": (C.c_int, [C.c_void_p, C.c_int64, C.c_int64]),
    "hlbg_swap": (C.c_int, [C.c_void_p]),
    "hlbg_set_time_step": (C.c_int, [C.c_void_p, C.c_uint64]),
    "hlbg_get_f": (C.c_int, [C.c_void_p, C.POINTER(C.c_double), C.c_int32]),
    "hlbg_put_f": (C.c_int, [C.c_void_p, C.POINTER(C.c_double), C.c_int32]),
    "hlbg_get_f_device": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int32]),
    "hlbg_put_f_device": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int32]),
    "hlbg_get_macro": (C.c_int, [C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_double)]),
    "hlbg_reduce": (C.c_int, [C.c_void_p, C.POINTER(Stats)]),
    "hlbg_reduce_noalloc": (C.c_int, [C.c_void_p, C.POINTER(Stats)]),
    "hlbg_iolet_density": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32, C.c_uint64,
                                     C.POINTER(C.c_double)]),
    "hlbg_time_steps": (C.c_int, [C.c_void_p, C.c_int32, C.POINTER(C.c_float)]),
    "hlbg_time_kernels": (C.c_int, [C.c_void_p, C.c_int32, C.POINTER(C.c_float), C.POINTER(C.c_float)]),
    "hlbg_version": (C.c_char_p, []),
    # multi-rank halo: host-side index maps (no device work)
    "hlbg_halo_partition": (C.c_int, [C.POINTER(Geometry), C.c_int32, C.POINTER(C.c_int32)]),
    "hlbg_halo_create": (C.c_int, [C.POINTER(Geometry), C.POINTER(C.c_int32), C.c_int32, C.c_int32,
                                   C.POINTER(C.c_void_p)]),
    "hlbg_halo_destroy": (None, [C.c_void_p]),
    "hlbg_halo_last_error": (C.c_char_p, [C.c_void_p]),
    "hlbg_halo_local_geometry": (C.c_int, [C.c_void_p, C.POINTER(Geometry), C.POINTER(C.c_int64)]),
    "hlbg_halo_block_source": (C.c_int, [C.c_void_p, C.POINTER(C.c_int64)]),
    "hlbg_halo_edge_blocks": (C.c_int, [C.c_void_p, C.POINTER(C.c_uint8)]),
    "hlbg_halo_peer_count": (C.c_int32, [C.c_void_p]),
    "hlbg_halo_peer": (C.c_int, [C.c_void_p, C.c_int32, C.POINTER(C.c_int32), C.POINTER(C.c_int64),
                                 C.POINTER(C.c_int64)]),
    "hlbg_halo_offsets": (C.c_int, [C.c_void_p, C.POINTER(C.c_int32), C.POINTER(C.c_int8), C.POINTER(C.c_int16),
                                    C.c_int64, C.POINTER(C.c_int64)]),
    "hlbg_halo_pack_device": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p]),
    "hlbg_halo_unpack_device": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p]),
    "hlbg_halo_check": (C.c_int, [C.c_void_p]),
    "hlbg_storage_bytes": (C.c_int, [C.c_void_p]),
    "hlbg_halo_list": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32, C.POINTER(C.c_int32), C.POINTER(C.c_int8),
                                 C.POINTER(C.c_int16)]),
    # include/hemelb_gb300_nn.h: the surrogate's kernels (device pointers, stream last)
    "hlbg_nn_conv3d": (C.c_int, [C.c_void_p, C.c_int32, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                 C.c_int32, C.c_int32, C.c_int32, C.c_int32, C.c_int32, C.c_int32,
                                 C.c_int32, C.c_void_p]),
    "hlbg_nn_conv3d_tc": (C.c_int, [C.c_void_p, C.c_int32, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                    C.c_int32, C.c_int32, C.c_int32, C.c_int32, C.c_int32, C.c_int32,
                                    C.c_int32, C.c_void_p]),
    "hlbg_nn_tc_error": (C.c_int, [C.c_int32]),
    "hlbg_nn_conv3d_wgrad": (C.c_int, [C.c_void_p, C.c_int32, C.c_void_p, C.c_int32, C.c_void_p, C.c_int32,
                                       C.c_int32, C.c_int32, C.c_int32, C.c_int32, C.c_void_p]),
    "hlbg_nn_flip_transpose": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int32, C.c_int32, C.c_int32, C.c_void_p]),
    "hlbg_nn_relu_bwd": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p]),
    "hlbg_nn_bias_grad": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int64, C.c_int32, C.c_void_p]),
    "hlbg_nn_pool2": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int32, C.c_int32, C.c_int32, C.c_int32, C.c_int32,
                                C.c_int32, C.c_void_p]),
    "hlbg_nn_up2": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int32, C.c_int32, C.c_int32, C.c_int32, C.c_int32,
                              C.c_int32, C.c_void_p]),
    "hlbg_nn_concat": (C.c_int, [C.c_void_p, C.c_int32, C.c_void_p, C.c_int32, C.c_void_p, C.c_int64,
                                 C.c_void_p]),
    "hlbg_nn_split": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int32, C.c_void_p, C.c_int32, C.c_int64,
                                C.c_int32, C.c_void_p]),
    "hlbg_nn_add": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p]),
    "hlbg_nn_mse": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int64,
                              C.c_int32, C.c_float, C.c_void_p]),
    "hlbg_nn_adam": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int64,
                               C.c_float, C.c_float, C.c_float, C.c_float, C.c_int32, C.c_void_p]),
    "hlbg_nn_to_bf16": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p]),
}

_lib = None


def load(path: str | None = None) -> C.CDLL:
    """Load libhemelb_gb300.so and declare every exported entry point."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = path or os.environ.get("HEMELB_GB300_LIB") or LIB_PATH
    if not os.path.exists(p):
        raise RuntimeError(
            f"{p} is missing: build it with `python -m hemelb_gb300.build` "
            "(there is no CPU fallback for the LB update)")
    lib = C.CDLL(p)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if path is None:
        _lib = lib
    return lib


class HlbgError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"HLBG_ERR_{ERRORS.get(code, code)}: {msg}")
        self.code = code


def check(rc: int, ctx=None, what: str = "") -> None:
    if rc != HLBG_OK:
        lib = load()
        msg = lib.hlbg_last_error(ctx).decode() if ctx else what
        raise HlbgError(rc, msg or what)
