"""ctypes binding of libphx.so (include/phx.h).

The library is built in-tree by photon_gb300.build; loading fails loudly when
it is missing -- there is no CPU fallback for the GPU step.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libphx.so")

PHX_OK, PHX_ERR_INVALID, PHX_ERR_UNSUPPORTED, PHX_ERR_OOM, PHX_ERR_CUDA, PHX_ERR_TIMEOUT, PHX_ERR_BUDGET, PHX_ERR_STATE = range(8)
PREC_FP64, PREC_MIXED = 0, 1

FIELDS = ["u", "v", "w", "p", "S", "T", "Yo", "Yf", "Ys", "Ya", "Yp", "Yc", "Yw", "Yco", "Yai", "nu", "Pb", "Q", "Qr",
          "hrr", "massSrc", "lit", "zone", "rhs", "cgR", "cgZ", "zoneP"]
FIELD_ID = {n: i for i, n in enumerate(FIELDS)}
STAGES = ["begin", "combustion", "turbulence", "heat", "energy", "momentum", "leakage", "project", "advect", "end"]
STAGE_ID = {n: i for i, n in enumerate(STAGES)}

# exported symbols, as declared in include/phx.h
SYMBOLS = ["phx_create", "phx_destroy", "phx_last_error", "phx_last_global_error", "phx_abi_version", "phx_add_burner",
           "phx_add_ignition", "phx_step", "phx_run", "phx_stage", "phx_precondition", "phx_get_field",
           "phx_set_field", "phx_field_count", "phx_get_stats", "phx_set_scalars", "phx_set_stats", "phx_device_bytes", "phx_sync",
           "phx_time_steps", "phx_profile_step", "phx_last_step_launches", "phx_rad_trace", "phx_batch_rad_trace", "phx_rad_last_ms", "phx_vol_render", "phx_batch_vol_render", "phx_vol_last_ms", "phx_selftest_wait_timeout", "phx_select_device", "phx_alloc_host",
           "phx_free_host", "phx_create_batch", "phx_batch_add", "phx_batch_remove", "phx_batch_size",
           "phx_batch_scenario_bytes", "phx_batch_add_burner", "phx_batch_step", "phx_batch_get_field",
           "phx_batch_set_field", "phx_batch_field_count", "phx_batch_get_stats", "phx_batch_set_stats", "phx_batch_mg_info", "phx_batch_mg_nnz", "phx_batch_tune_vcycle", "phx_gather_stats_noalloc",
           "phx_server_create", "phx_server_destroy", "phx_server_last_error", "phx_server_submit", "phx_server_step",
           "phx_server_poll", "phx_server_get_field", "phx_server_release", "phx_server_counts"]

REQ_QUEUED, REQ_RUNNING, REQ_DONE, REQ_REJECTED = 0, 1, 2, 3


class PhxGrid(ctypes.Structure):
    _fields_ = [("nx", ctypes.c_int), ("ny", ctypes.c_int), ("nz", ctypes.c_int),
                ("dx", ctypes.c_double), ("ox", ctypes.c_double), ("oy", ctypes.c_double), ("oz", ctypes.c_double),
                ("cfl", ctypes.c_double), ("dt_max", ctypes.c_double), ("max_iters", ctypes.c_int),
                ("tol", ctypes.c_double), ("rel_tol", ctypes.c_double),
                ("radiation_on", ctypes.c_int), ("adiabatic_surfaces", ctypes.c_int),
                ("wind_speed", ctypes.c_double), ("wind_from_deg", ctypes.c_double), ("wind_exponent", ctypes.c_double),
                ("blocked", ctypes.c_void_p),
                ("fx", ctypes.c_void_p), ("fy", ctypes.c_void_p), ("fz", ctypes.c_void_p),
                ("ax", ctypes.c_void_p), ("ay", ctypes.c_void_p), ("az", ctypes.c_void_p),
                ("lx", ctypes.c_void_p), ("ly", ctypes.c_void_p), ("lz", ctypes.c_void_p)]


# phx_rad_elem and phx_rad_wall as numpy record types (same layout as the C structs)
RAD_ELEM_DTYPE = np.dtype([("o", "<f8", (3,)), ("n", "<f8", (3,)), ("area", "<f8"), ("emissivity", "<f8"),
                           ("temperature", "<f8"), ("sphere", "<i4"), ("skip_own_cell", "<i4")], align=True)
RAD_WALL_DTYPE = np.dtype([("axis", "<i4"), ("face", "<i4"), ("t_lower", "<f8"), ("t_upper", "<f8")], align=True)


def rad_elements(a) -> np.ndarray:
    """phx_rad_elem records from an (n, 11) array (o, n, area, emissivity,
    temperature, sphere, skip own cell) or records already."""
    if isinstance(a, np.ndarray) and a.dtype == RAD_ELEM_DTYPE:
        return np.ascontiguousarray(a)
    a = np.asarray(a, np.float64).reshape(-1, 11)
    r = np.zeros(len(a), RAD_ELEM_DTYPE)
    r["o"], r["n"] = a[:, 0:3], a[:, 3:6]
    r["area"], r["emissivity"], r["temperature"] = a[:, 6], a[:, 7], a[:, 8]
    r["sphere"], r["skip_own_cell"] = a[:, 9].astype(np.int32), a[:, 10].astype(np.int32)
    return r


def rad_walls(a) -> np.ndarray:
    """phx_rad_wall records from an (m, 4) array (axis, face, T from the lower
    cell, T from the upper cell) or records already."""
    if isinstance(a, np.ndarray) and a.dtype == RAD_WALL_DTYPE:
        return np.ascontiguousarray(a)
    a = np.asarray(a, np.float64).reshape(-1, 4)
    r = np.zeros(len(a), RAD_WALL_DTYPE)
    r["axis"], r["face"] = a[:, 0].astype(np.int32), a[:, 1].astype(np.int32)
    r["t_lower"], r["t_upper"] = a[:, 2], a[:, 3]
    return r


class PhxVolParams(ctypes.Structure):
    """phx_vol_params (include/phx.h): the volume shader's uniforms."""
    _fields_ = [("width", ctypes.c_int), ("height", ctypes.c_int), ("inv_vp", ctypes.c_float * 16),
                ("eye", ctypes.c_float * 3), ("step", ctypes.c_float), ("clip_z", ctypes.c_float),
                ("slice_z", ctypes.c_float), ("t_min", ctypes.c_float), ("t_max", ctypes.c_float),
                ("smoke", ctypes.c_int), ("slice", ctypes.c_int), ("fire", ctypes.c_int), ("time", ctypes.c_float),
                ("smoke_scale", ctypes.c_float), ("sun_dir", ctypes.c_float * 3), ("n_lights", ctypes.c_int),
                ("lights", (ctypes.c_float * 4) * 8), ("background", ctypes.c_float * 3)]


class PhxStats(ctypes.Structure):
    _fields_ = [("time", ctypes.c_double), ("dt", ctypes.c_double),
                ("max_vel", ctypes.c_double), ("max_nu", ctypes.c_double), ("max_div", ctypes.c_double),
                ("pressure_iters", ctypes.c_int), ("pressure_residual", ctypes.c_double),
                ("pressure_rel_residual", ctypes.c_double),
                ("hrr", ctypes.c_double), ("max_gas_t", ctypes.c_double), ("burning_cells", ctypes.c_int),
                ("fuel_in", ctypes.c_double), ("fuel_burned", ctypes.c_double), ("fuel_in_domain", ctypes.c_double),
                ("zones", ctypes.c_int), ("leak_faces", ctypes.c_int)]


class PhxRequestInfo(ctypes.Structure):
    _fields_ = [("state", ctypes.c_int), ("steps", ctypes.c_int),
                ("sim_time", ctypes.c_double), ("duration", ctypes.c_double),
                ("t_submit", ctypes.c_double), ("t_admit", ctypes.c_double), ("t_done", ctypes.c_double),
                ("device_bytes", ctypes.c_size_t), ("cells", ctypes.c_longlong), ("stats", PhxStats)]


class PhxKernelTime(ctypes.Structure):
    _fields_ = [("name", ctypes.c_char * 48), ("launches", ctypes.c_int), ("ms", ctypes.c_double)]


_L = None


def lib_path() -> str:
    return LIB_PATH


def load():
    """Load libphx.so; raises if it has not been built."""
    global _L
    if _L is not None:
        return _L
    if not os.path.exists(LIB_PATH):
        raise RuntimeError("libphx.so is not built (run python -m photon_gb300.build); the GPU step has no CPU fallback")
    L = ctypes.CDLL(LIB_PATH)
    vp, d, i, sz = ctypes.c_void_p, ctypes.c_double, ctypes.c_int, ctypes.c_size_t
    L.phx_create.argtypes = [ctypes.POINTER(PhxGrid), i, ctypes.POINTER(vp)]
    L.phx_destroy.argtypes = [vp]
    L.phx_last_error.restype = ctypes.c_char_p
    L.phx_last_error.argtypes = [vp]
    L.phx_last_global_error.restype = ctypes.c_char_p
    L.phx_add_burner.argtypes = [vp, d, d, d, d, d, d, d, d, d, ctypes.POINTER(i)]
    L.phx_add_ignition.argtypes = [vp, i, d, d]
    L.phx_step.argtypes = [vp, d, ctypes.POINTER(d)]
    L.phx_run.argtypes = [vp, i, d, vp]
    L.phx_stage.argtypes = [vp, i, d]
    L.phx_precondition.argtypes = [vp, vp, vp]
    L.phx_get_field.argtypes = [vp, i, vp, sz]
    L.phx_set_field.argtypes = [vp, i, vp, sz]
    L.phx_field_count.restype = sz
    L.phx_field_count.argtypes = [vp, i]
    L.phx_get_stats.argtypes = [vp, ctypes.POINTER(PhxStats)]
    L.phx_set_scalars.argtypes = [vp, d, d, d, d]
    L.phx_set_stats.argtypes = [vp, ctypes.POINTER(PhxStats)]
    L.phx_device_bytes.restype = sz
    L.phx_device_bytes.argtypes = [vp]
    L.phx_sync.argtypes = [vp]
    L.phx_time_steps.argtypes = [vp, i, d, i, ctypes.POINTER(d), ctypes.POINTER(i)]
    L.phx_profile_step.argtypes = [vp, d, i, ctypes.POINTER(PhxKernelTime), i, ctypes.POINTER(i)]
    L.phx_last_step_launches.argtypes = [vp]
    L.phx_gather_stats_noalloc.argtypes = [vp, i, ctypes.POINTER(PhxStats)]
    L.phx_server_create.argtypes = [i, sz, i, ctypes.POINTER(vp)]
    L.phx_server_destroy.argtypes = [vp]
    L.phx_server_destroy.restype = None
    L.phx_server_last_error.argtypes = [vp]
    L.phx_server_last_error.restype = ctypes.c_char_p
    L.phx_server_submit.argtypes = [vp, ctypes.POINTER(PhxGrid), vp, i, d, d, ctypes.POINTER(i)]
    L.phx_server_step.argtypes = [vp, ctypes.POINTER(i), ctypes.POINTER(i), ctypes.POINTER(i)]
    L.phx_server_poll.argtypes = [vp, i, ctypes.POINTER(PhxRequestInfo)]
    L.phx_server_get_field.argtypes = [vp, i, i, vp, sz]
    L.phx_server_release.argtypes = [vp, i]
    L.phx_server_counts.argtypes = [vp, ctypes.POINTER(i), ctypes.POINTER(i), ctypes.POINTER(sz),
                                    ctypes.POINTER(ctypes.c_longlong)]
    L.phx_select_device.argtypes = [i]
    L.phx_create_batch.argtypes = [ctypes.POINTER(PhxGrid), i, i, ctypes.POINTER(vp)]
    L.phx_batch_add.argtypes = [vp, ctypes.POINTER(PhxGrid), ctypes.POINTER(i)]
    L.phx_batch_remove.argtypes = [vp, i]
    L.phx_batch_size.argtypes = [vp]
    L.phx_batch_scenario_bytes.restype = sz
    L.phx_batch_scenario_bytes.argtypes = [vp, i]
    L.phx_batch_add_burner.argtypes = [vp, i, d, d, d, d, d, d, d, d, d, ctypes.POINTER(i)]
    L.phx_batch_step.argtypes = [vp, vp, d, vp]
    L.phx_batch_get_field.argtypes = [vp, i, i, vp, sz]
    L.phx_batch_set_field.argtypes = [vp, i, i, vp, sz]
    L.phx_batch_field_count.restype = sz
    L.phx_batch_field_count.argtypes = [vp, i, i]
    L.phx_batch_get_stats.argtypes = [vp, i, ctypes.POINTER(PhxStats)]
    L.phx_batch_set_stats.argtypes = [vp, i, ctypes.POINTER(PhxStats)]
    L.phx_batch_mg_info.argtypes = [vp, i, ctypes.POINTER(i), vp, i]
    L.phx_batch_mg_nnz.argtypes = [vp, i, vp, i]
    L.phx_batch_tune_vcycle.argtypes = [vp, i, d, vp, i]
    L.phx_rad_trace.argtypes = [vp, vp, i, vp, i, vp, vp, vp]
    L.phx_batch_rad_trace.argtypes = [vp, i, vp, i, vp, i, vp, vp, vp]
    L.phx_rad_last_ms.restype = d
    L.phx_rad_last_ms.argtypes = [vp]
    L.phx_vol_render.argtypes = [vp, ctypes.POINTER(PhxVolParams), vp, vp]
    L.phx_batch_vol_render.argtypes = [vp, i, ctypes.POINTER(PhxVolParams), vp, vp]
    L.phx_vol_last_ms.restype = d
    L.phx_vol_last_ms.argtypes = [vp]
    L.phx_selftest_wait_timeout.argtypes = [vp, d]
    L.phx_alloc_host.restype = vp
    L.phx_alloc_host.argtypes = [sz]
    L.phx_free_host.argtypes = [vp]
    _L = L
    return L


class PhxError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("phx error %d: %s" % (code, msg))
        self.code = code
