"""ctypes bindings of libfesom_tracer_gb300.so (include/fesom_tracer_gb300.h).

The library is built in-tree (``fesom2_tracer_dwarf_gb300/lib``). There is no
CPU fallback: if the library is missing or cannot be loaded, every entry point
raises.
"""
from __future__ import annotations

import ctypes
import os

from . import build as _build

HOR = {"UPW1": 0, "MUSCL": 1, "MFCT": 2}
VER = {"UPW1": 0, "QR4C": 1, "CDIFF": 2, "PPM": 3}
LIM = {"NONE": 0, "FCT": 1}
FP64, FP32, FP64_FAST = 0, 1, 2
NCFG = 12  # launch knobs of fgb_step_desc.cfg
STAGE_VFLUX, STAGE_HFLUX, STAGE_LO, STAGE_RATIO, STAGE_UPDATE = 1, 2, 4, 8, 16
STAGE_ALL = 31

_vp = ctypes.c_void_p
_ip = ctypes.POINTER(ctypes.c_int)
_dp = ctypes.POINTER(ctypes.c_double)
_llp = ctypes.POINTER(ctypes.c_longlong)


class StepDesc(ctypes.Structure):
    """fgb_step_desc of include/fesom_tracer_gb300.h."""

    _fields_ = [
        ("precision", ctypes.c_int),
        ("ntracers", ctypes.c_int),
        ("hor", ctypes.c_int),
        ("ver", ctypes.c_int),
        ("lim", ctypes.c_int),
        ("ph", ctypes.c_double),
        ("pv", ctypes.c_double),
        ("dt", ctypes.c_double),
        ("T", _vp),
        ("strideT", ctypes.c_longlong),
        ("TA", _vp),
        ("strideTA", ctypes.c_longlong),
        ("TAout", _vp),
        ("vel", _vp),
        ("w", _vp),
        ("we", _vp),
        ("del_", _vp),
        ("workspace", _vp),
        ("workspace_bytes", ctypes.c_longlong),
        ("tracer_vec", ctypes.c_int),
        ("cfg", ctypes.c_int * NCFG),
        ("wi", _vp),
        ("ab_order", ctypes.c_int),
        ("ab_eps", ctypes.c_double),
        ("fp32_plain_sums", ctypes.c_int),
        ("Tlo", _vp),
    ]


# Every extern "C" symbol the header declares (checked by the CPU tests).
REFERENCE_SYMBOLS = [
    "tracer_init_mpi", "tracer_finalize_mpi", "tracer_init", "tracer_advect_step", "tracer_get_stats",
    "tracer_get_size", "tracer_get_values", "tracer_finalize", "tracer_run_workflow", "tracer_cleanup",
    "tracer_set_mesh_dims", "tracer_set_levels", "tracer_set_thickness", "tracer_set_partition",
    "tracer_allocate_tracers", "tracer_set_values", "tracer_set_velocity_zero", "tracer_set_velocity",
    "tracer_init_complete", "tracer_load_mesh_partition", "tracer_load_mesh_from_files",
    "tracer_init_ale_arrays", "tracer_init_for_advection",
]
EXTENSION_SYMBOLS = ["tracer_generate_analytic_mesh", "tracer_set_schemes", "tracer_set_precision",
                     "tracer_set_input_checks"]
ENGINE_SYMBOLS = [
    "fgb_last_error", "fgb_version", "fgb_hmesh_analytic", "fgb_hmesh_from_files", "fgb_hmesh_from_arrays", "fgb_hmesh_union", "fgb_hmesh_free", "fgb_hmesh_sizes", "fgb_hmesh_get",
    "fgb_hmesh_set_vertical", "fgb_mesh_create", "fgb_mesh_free", "fgb_mesh_dims", "fgb_mesh_update_vertical",
    "fgb_workspace_bytes", "fgb_workspace_offsets", "fgb_adv_step", "fgb_adv_stages", "fgb_stats_scratch_bytes",
    "fgb_tracer_stats", "fgb_tracer_stats_grouped", "fgb_last_launch_count", "fgb_static_workspace_bytes", "fgb_adv_step_static",
    "fgb_probe_fp64", "fgb_check_inputs",
]

_lib = None


def load(build_if_missing: bool = True):
    """Load (building if needed) the shared library; raises if it is unavailable."""
    global _lib
    if _lib is not None:
        return _lib
    path = _build.LIB_PATH
    if build_if_missing:
        path = _build.build()
    if not os.path.exists(path):
        raise RuntimeError(f"{path} is missing: build it with fesom2_tracer_dwarf_gb300.build.build()")
    L = ctypes.CDLL(path, mode=ctypes.RTLD_GLOBAL)
    sig = {
        "fgb_last_error": (ctypes.c_char_p, []),
        "fgb_version": (ctypes.c_int, []),
        "fgb_last_launch_count": (ctypes.c_int, []),
        "fgb_hmesh_analytic": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_double,
                                              ctypes.c_double, ctypes.c_double, ctypes.c_int, ctypes.c_int,
                                              _dp, _ip, ctypes.POINTER(_vp)]),
        "fgb_hmesh_from_files": (ctypes.c_int, [ctypes.c_char_p, ctypes.c_int, ctypes.POINTER(_vp)]),
        "fgb_hmesh_from_arrays": (ctypes.c_int, [ctypes.c_int] * 5 + [_dp, _ip, _ip, _ip, _ip, _ip, _dp, ctypes.c_int,
                                                                     ctypes.POINTER(_vp)]),
        "fgb_hmesh_free": (None, [_vp]),
        "fgb_hmesh_sizes": (ctypes.c_int, [_vp, _llp]),
        "fgb_hmesh_get": (ctypes.c_longlong, [_vp, ctypes.c_char_p, _vp, _ip]),
        "fgb_hmesh_set_vertical": (ctypes.c_int, [_vp, _dp, _dp, _dp]),
        "fgb_hmesh_union": (ctypes.c_int, [ctypes.POINTER(_vp), ctypes.c_int, ctypes.POINTER(_vp)]),
        "fgb_mesh_create": (ctypes.c_int, [_vp, ctypes.POINTER(_vp)]),
        "fgb_mesh_free": (None, [_vp]),
        "fgb_mesh_dims": (ctypes.c_int, [_vp, _ip]),
        "fgb_mesh_update_vertical": (ctypes.c_int, [_vp, _vp]),
        "fgb_workspace_bytes": (ctypes.c_longlong, [_vp, ctypes.c_int, ctypes.c_int]),
        "fgb_workspace_offsets": (ctypes.c_int, [_vp, ctypes.c_int, ctypes.c_int, _llp]),
        "fgb_adv_step": (ctypes.c_int, [_vp, ctypes.POINTER(StepDesc), _vp]),
        "fgb_adv_stages": (ctypes.c_int, [_vp, ctypes.POINTER(StepDesc), ctypes.c_int, _vp]),
        "fgb_stats_scratch_bytes": (ctypes.c_longlong, [_vp, ctypes.c_int]),
        "fgb_static_workspace_bytes": (ctypes.c_longlong, []),
        "fgb_adv_step_static": (ctypes.c_int, [_vp, ctypes.POINTER(StepDesc), _vp]),
        "fgb_probe_fp64": (ctypes.c_int, [_dp, _vp]),
        "fgb_check_inputs": (ctypes.c_int, [_vp, ctypes.POINTER(StepDesc), _vp, _ip]),
        "fgb_tracer_stats": (ctypes.c_int, [_vp, ctypes.c_int, _vp, ctypes.c_longlong, ctypes.c_int, _vp, _vp,
                                            _vp]),
        "fgb_tracer_stats_grouped": (ctypes.c_int, [_vp, _vp, ctypes.c_longlong, ctypes.c_int, ctypes.c_int, _vp,
                                                    _vp, _vp]),
    }
    for name, (res, args) in sig.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    _lib = L
    return L


def last_error() -> str:
    return load().fgb_last_error().decode()


def probe_fp64(stream=None) -> dict:
    """The current device's FP64 rates (fgb_probe_fp64): fused multiply-add
    TFLOP/s and IEEE double divisions in G/s."""
    out = (ctypes.c_double * 3)()
    check(load().fgb_probe_fp64(out, stream), "fgb_probe_fp64")
    return {"fma_tflops": out[0], "div_g_per_s": out[1], "ms": out[2]}


def check(rc: int, what: str):
    if rc != 0:
        raise RuntimeError(f"{what} failed: {last_error()}")
