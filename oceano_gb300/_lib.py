"""ctypes binding of liboceano_gpu.so (the C ABI of include/oceano_gpu.h).

The library is built in-tree by :func:`oceano_gb300.build.build`; importing
this module never falls back to anything else: if the shared library is
missing or fails to load, :func:`lib` raises.
"""
from __future__ import annotations

import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboceano_gpu.so")
# bounds-checked variant (oceano_gb300.build.build(bounds_check=True)), loaded
# instead when the environment sets OCEANO_BOUNDS_CHECK=1
LIB_CHECKED_PATH = os.path.join(HERE, "liboceano_gpu_checked.so")

OC_OK, OC_ERR_INVALID_ARG, OC_ERR_UNKNOWN_BOUNDARY_ID, OC_ERR_NONFINITE, OC_ERR_TIMEOUT, \
    OC_ERR_CUDA, OC_ERR_UNSUPPORTED, OC_ERR_NOMEM, OC_ERR_BOUNDS = range(9)
OC_MEM_HOST, OC_MEM_DEVICE = 0, 1
OC_PREC_FP64, OC_PREC_MIXED = 0, 1
BC_KIND = {"none": 0, "wall": 1, "supercritical_inflow": 2, "supercritical_outflow": 3,
           "height_inflow": 4, "discharge_inflow": 5, "absorbing_outflow": 6}
LAUNCH_MODE = {"auto": 0, "per_group": 1, "one": 2}
CELL_RULE = {"default": 0, "p+1": 1}  # oc_params.cell_quadrature
SCHEME = {"forward_euler": 0, "ssp22": 1, "ssp33": 2, "rk4": 3, "stage3_order2": 4,
          "ark_stage3_order2": 5}


class MeshDesc(C.Structure):
    _fields_ = [("n_cells", C.c_int32), ("degree", C.c_void_p), ("vertices", C.c_void_p),
                ("n_inner_faces", C.c_int32), ("n_boundary_faces", C.c_int32),
                ("cell_m", C.c_void_p), ("cell_p", C.c_void_p), ("face_m", C.c_void_p),
                ("face_p", C.c_void_p), ("subface", C.c_void_p), ("orientation", C.c_void_p),
                ("boundary_id", C.c_void_p)]


class Params(C.Structure):
    _fields_ = [("g", C.c_double), ("threshold_wetdry", C.c_double),
                ("horizontal_viscosity", C.c_double), ("friction_model", C.c_int32),
                ("max_iteration_height", C.c_int32), ("batch_width", C.c_int32),
                ("precision", C.c_int32), ("zeta_reference", C.c_double),
                ("cell_quadrature", C.c_int32)]


class StageVectors(C.Structure):
    _fields_ = [("ri_height", C.c_void_p), ("ri_discharge", C.c_void_p),
                ("ri_velocity", C.c_void_p), ("ki_height", C.POINTER(C.c_void_p)),
                ("n_ki_height", C.c_int32), ("ki_discharge", C.POINTER(C.c_void_p)),
                ("n_ki_discharge", C.c_int32), ("solution_height", C.c_void_p),
                ("solution_discharge", C.c_void_p), ("next_height", C.c_void_p),
                ("next_discharge", C.c_void_p)]


EXPORTS = {
    "oc_create": (C.c_int, [C.POINTER(MeshDesc), C.POINTER(Params), C.POINTER(C.c_void_p)]),
    "oc_destroy": (None, [C.c_void_p]),
    "oc_last_error": (C.c_char_p, [C.c_void_p]),
    "oc_n_dofs": (C.c_int64, [C.c_void_p]),
    "oc_set_boundary": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32, C.c_int32, C.c_void_p]),
    "oc_set_vortex": (C.c_int, [C.c_void_p, C.c_void_p]),
    "oc_set_static_data": (C.c_int, [C.c_void_p] + [C.c_void_p] * 5),
    "oc_static_data_size": (C.c_int64, [C.c_void_p, C.c_int32]),
    "oc_quadrature_points": (C.c_int, [C.c_void_p, C.c_int32, C.c_void_p]),
    "oc_perform_stage_hydro": (C.c_int, [C.c_void_p, C.c_uint32, C.c_uint32, C.c_double,
                                         C.c_void_p, C.c_void_p, C.c_double,
                                         C.POINTER(StageVectors), C.c_int32]),
    "oc_perform_time_step": (C.c_int, [C.c_void_p, C.c_int32, C.c_double, C.c_double,
                                       C.c_void_p, C.c_void_p, C.c_int32]),
    "oc_transport_speed": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int32,
                                     C.POINTER(C.c_double)]),
    "oc_apply": (C.c_int, [C.c_void_p, C.c_double, C.c_void_p, C.c_void_p, C.c_void_p,
                           C.c_void_p, C.c_int32]),
    "oc_velocity_field": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int32]),
    "oc_vorticity_indicator": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int32, C.c_void_p,
                                         C.c_int32]),
    "oc_project_vortex": (C.c_int, [C.c_void_p, C.c_double, C.c_void_p, C.c_void_p, C.c_int32]),
    "oc_transport_speed_noalloc": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "oc_errors_vortex": (C.c_int, [C.c_void_p, C.c_double, C.c_void_p, C.c_void_p, C.c_int32,
                                   C.c_void_p]),
    "oc_conservative_coarsening": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int32]),
    "oc_indicator_features": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                        C.c_int32, C.c_float, C.c_void_p, C.c_void_p,
                                        C.c_void_p, C.c_int32]),
    "oc_mlp_create": (C.c_int, [C.c_uint64, C.POINTER(C.c_void_p)]),
    "oc_mlp_destroy": (None, [C.c_void_p]),
    "oc_mlp_last_error": (C.c_char_p, [C.c_void_p]),
    "oc_mlp_stream": (C.c_void_p, [C.c_void_p]),
    "oc_mlp_synchronize": (C.c_int, [C.c_void_p]),
    "oc_mlp_get_params": (C.c_int, [C.c_void_p, C.c_void_p]),
    "oc_mlp_set_params": (C.c_int, [C.c_void_p, C.c_void_p]),
    "oc_mlp_get_normalization": (C.c_int, [C.c_void_p, C.c_void_p]),
    "oc_mlp_set_normalization": (C.c_int, [C.c_void_p, C.c_void_p]),
    "oc_mlp_fit_normalization": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int64]),
    "oc_mlp_forward": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p]),
    "oc_mlp_gradient": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int64, C.c_float,
                                  C.c_void_p, C.POINTER(C.c_double)]),
    "oc_mlp_adam_step": (C.c_int, [C.c_void_p, C.c_float]),
    "oc_set_reference_state": (C.c_int, [C.c_void_p, C.c_double, C.c_double, C.c_double]),
    "oc_set_cell_time_scale": (C.c_int, [C.c_void_p, C.c_void_p]),
    "oc_set_timing": (C.c_int, [C.c_void_p, C.c_int32]),
    "oc_timer_summary": (C.c_int, [C.c_void_p, C.c_char_p, C.c_int64]),
    "oc_cell_transport_speed": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int32,
                                          C.c_void_p]),
    "oc_set_launch_mode": (C.c_int, [C.c_void_p, C.c_int32]),
    "oc_launch_config": (C.c_int, [C.c_void_p, C.c_void_p]),
    "oc_synchronize": (C.c_int, [C.c_void_p]),
    "oc_stream": (C.c_void_p, [C.c_void_p]),
    "oc_launch_count": (C.c_int64, [C.c_void_p]),
    "oc_bounds_checked": (C.c_int32, []),
    "oc_bounds_selftest": (C.c_int, [C.c_void_p]),
}

_lib = None


def default_path() -> str:
    """The bounds-checked library when OCEANO_BOUNDS_CHECK=1, else the regular one."""
    return LIB_CHECKED_PATH if os.environ.get("OCEANO_BOUNDS_CHECK") == "1" else LIB_PATH


def lib(path: str | None = None):
    """Load the library (raises if it is absent: there is no fallback path)."""
    global _lib
    if _lib is None:
        path = path or default_path()
        if not os.path.exists(path):
            raise RuntimeError(f"{path} is missing: run oceano_gb300.build.build() first")
        L = C.CDLL(path)
        for name, (res, args) in EXPORTS.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


class OceanoError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__(f"oceano_gpu status {status}: {msg}")
        self.status = status


def check(status, handle=None):
    if status != OC_OK:
        msg = lib().oc_last_error(handle).decode() if handle else ""
        raise OceanoError(status, msg)
