"""ctypes access to the FP64 C restatement (oracle/phx_oracle.c) -- test infrastructure.

`OracleSolver(case)` mirrors oracle.refpy.RefSolver so a test can drive the
restatement, the reference build and the CUDA path with the same calls.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libphx_oracle.so")
_L = None

U8_FIELDS = ("lx", "ly", "lz", "lit", "pilot", "blocked", "zoneOpen")
I32_FIELDS = ("zone",)
SCALARS = ("time", "maxVel", "maxNu", "maxDiv", "pressureIters", "pressureResidual", "hrr", "maxGasT",
           "burningCells", "fuelIn", "fuelBurned", "fuelInDomain", "leakFaces", "nZones")


def build(force: bool = False) -> str:
    """Compile phx_oracle.c with FP contraction off (so a*b+c is never fused)."""
    src = os.path.join(HERE, "phx_oracle.c")
    hdr = os.path.join(HERE, "phx_oracle.h")
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= max(os.path.getmtime(src), os.path.getmtime(hdr)):
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    tmp = LIB + ".tmp%d" % os.getpid()
    cmd = ["gcc", "-std=c11", "-O2", "-ffp-contract=off", "-fno-math-errno", "-fPIC", "-shared", "-o", tmp, src, "-lm"]
    subprocess.run(cmd, check=True)
    os.replace(tmp, LIB)
    return LIB


def load():
    global _L
    if _L is not None:
        return _L
    build()
    L = ctypes.CDLL(LIB)
    vp, d, i = ctypes.c_void_p, ctypes.c_double, ctypes.c_int
    L.orc_new.restype = vp
    L.orc_new.argtypes = [i, i, i, d, d, d, d]
    L.orc_free.argtypes = [vp]
    L.orc_set_profile.argtypes = [vp, d, d, i, d, d]
    L.orc_set_switches.argtypes = [vp, i, i]
    L.orc_set_wind.argtypes = [vp, d, d, d]
    L.orc_mark_geometry_dirty.argtypes = [vp]
    L.orc_add_burner.argtypes = [vp, d, d, d, d, d, d, d, d, d]
    L.orc_burner_cells.argtypes = [vp, i, ctypes.c_void_p, i]
    L.orc_add_ignition.argtypes = [vp, i, d, d]
    L.orc_set_coarse_mode.argtypes = [vp, i]
    L.orc_step.restype = d
    L.orc_step.argtypes = [vp, d]
    L.orc_stage.argtypes = [vp, ctypes.c_char_p, d]
    L.orc_stable_dt.restype = d
    L.orc_stable_dt.argtypes = [vp, d]
    L.orc_precondition.argtypes = [vp, ctypes.c_void_p, ctypes.c_void_p]
    L.orc_field_len.restype = ctypes.c_long
    L.orc_field_len.argtypes = [vp, ctypes.c_char_p]
    L.orc_field.argtypes = [vp, ctypes.c_char_p, i, ctypes.c_void_p, ctypes.c_long]
    L.orc_scalars.argtypes = [vp, ctypes.c_void_p]
    L.orc_set_scalars.argtypes = [vp, d, d, d, d]
    L.orc_mg_levels.argtypes = [vp]
    L.orc_mg_info.argtypes = [vp, i, ctypes.c_void_p]
    L.orc_mg_get.argtypes = [vp, i, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
    vpp = ctypes.c_void_p
    L.orc_rad_trace.argtypes = [i, i, i, d, d, d, d, vpp, vpp, vpp, vpp, vpp, vpp, vpp, i, vpp, i, vpp, vpp, vpp, vpp]
    L.orc_vol_render.argtypes = [i, i, i, ctypes.c_float, ctypes.c_float, ctypes.c_float, ctypes.c_float, vpp, vpp,
                                 vpp, vpp, i, i]
    _L = L
    return L


RAD_GAS_FIELDS = ("T", "Ys", "Yw", "Yc", "Pb", "hrr")


def rad_trace(dims, geo, blocked, gas: dict, elements, walls, solidT):
    """Solver::traceRadiation (src/sim/radiation.cpp:181-319) over flat inputs:
    dims (nx, ny, nz), geo (dx, ox, oy, oz), gas fields by name (T Ys Yw Yc Pb
    hrr), elements (n x 11), walls (m x 4), solidT (N). Returns (radAbs, radGas)."""
    L = load()
    nx, ny, nz = (int(v) for v in dims)
    dx, ox, oy, oz = (float(v) for v in geo)
    n = nx * ny * nz
    bl = np.ascontiguousarray(blocked, np.uint8)
    g = [np.ascontiguousarray(gas[f], np.float64) for f in RAD_GAS_FIELDS]
    el = np.ascontiguousarray(elements, np.float64).reshape(-1, 11)
    wl = np.ascontiguousarray(walls, np.float64).reshape(-1, 4)
    st = np.ascontiguousarray(solidT, np.float64)
    assert bl.size == n and st.size == n and all(a.size == n for a in g)
    ab = np.zeros(len(el), np.float64)
    gas_out = np.zeros(n, np.float64)
    L.orc_rad_trace(nx, ny, nz, dx, ox, oy, oz, _ptr(bl), *[_ptr(a) for a in g], len(el), _ptr(el), len(wl),
                    _ptr(wl), _ptr(st), _ptr(ab), _ptr(gas_out))
    return ab, gas_out


def vol_render(case, vol: np.ndarray, params, depth=None, rows=None) -> np.ndarray:
    """The viewer's volume shader restated in C (orc_vol_render) over vol
    (N x 4 float32: soot density, aerosol density, T, heat release) with the
    uniforms of a photon_gb300._lib.PhxVolParams. rows: (first, end) to render
    a band of rows (the rest stays 0). Returns (height, width, 3) float32."""
    L = load()
    v = np.ascontiguousarray(vol, np.float32).reshape(-1, 4)
    rgb = np.zeros((params.height, params.width, 3), np.float32)
    d = None if depth is None else np.ascontiguousarray(depth, np.float32)
    r0, r1 = rows if rows else (0, params.height)
    L.orc_vol_render(case.nx, case.ny, case.nz, float(case.dx), float(case.ox), float(case.oy), float(case.oz),
                     _ptr(v), ctypes.byref(params), None if d is None else _ptr(d), _ptr(rgb), int(r0), int(r1))
    return rgb


def pack_volume(blocked, T, Ys, Ya, Pb, hrr) -> np.ndarray:
    """Viewer::uploadVolume's packing (src/app/viewer.cpp:941-949) in FP32."""
    T32 = np.asarray(T).astype(np.float32)
    rho = np.asarray(Pb).astype(np.float32) / (np.float32(287.0) * T32)
    v = np.stack([np.asarray(Ys).astype(np.float32) * rho, np.asarray(Ya).astype(np.float32) * rho, T32,
                  np.asarray(hrr).astype(np.float32)], 1)
    v[np.asarray(blocked) != 0] = 0
    return v


def _ptr(a):
    return a.ctypes.data_as(ctypes.c_void_p)


class OracleSolver:
    def __init__(self, case=None):
        self.L = load()
        self.h = None
        if case is not None:
            self.setup(case)

    def __del__(self):
        try:
            if self.h:
                self.L.orc_free(self.h)
                self.h = None
        except Exception:
            pass

    def setup(self, case):
        L = self.L
        if self.h:
            L.orc_free(self.h)
        self.h = ctypes.c_void_p(L.orc_new(case.nx, case.ny, case.nz, case.dx, case.ox, case.oy, case.oz))
        pr = case.profile
        L.orc_set_profile(self.h, pr.cfl, pr.dtMax, pr.maxIters, pr.tol, pr.rel_tol)
        L.orc_set_switches(self.h, int(case.radiationOn), int(case.adiabatic))
        L.orc_set_wind(self.h, *case.wind)
        for n in ("fx", "fy", "fz", "ax", "ay", "az", "blocked", "lx", "ly", "lz"):
            self.set(n, getattr(case, n))
        L.orc_mark_geometry_dirty(self.h)
        self.burner_ids = [L.orc_add_burner(self.h, b.x0, b.y0, b.x1, b.y1, b.z, b.peakW, b.rampS, b.start, b.duration)
                           for b in case.burners]

    def burner_cells(self, b: int):
        buf = np.zeros(1 << 16, np.int32)
        n = self.L.orc_burner_cells(self.h, b, _ptr(buf), buf.size)
        return buf[:n].copy()

    def get(self, name: str) -> np.ndarray:
        n = self.L.orc_field_len(self.h, name.encode())
        if n < 0:
            raise KeyError(name)
        dt = np.uint8 if name in U8_FIELDS else np.int32 if name in I32_FIELDS else np.float64
        a = np.zeros(n, dt)
        if self.L.orc_field(self.h, name.encode(), 0, _ptr(a), n) < 0:
            raise KeyError(name)
        return a

    def set(self, name: str, arr):
        dt = np.uint8 if name in U8_FIELDS else np.int32 if name in I32_FIELDS else np.float64
        a = np.ascontiguousarray(arr, dtype=dt)
        if self.L.orc_field(self.h, name.encode(), 1, _ptr(a), a.size) < 0:
            raise KeyError(name)

    def step(self, dtMax: float) -> float:
        return self.L.orc_step(self.h, dtMax)

    def stage(self, name: str, dt: float = 0.0):
        if self.L.orc_stage(self.h, name.encode(), dt) != 0:
            raise KeyError(name)

    def stable_dt(self, dtMax: float) -> float:
        return self.L.orc_stable_dt(self.h, dtMax)

    def precondition(self, r):
        r = np.ascontiguousarray(r, np.float64)
        z = np.zeros_like(r)
        self.L.orc_precondition(self.h, _ptr(r), _ptr(z))
        return z

    def scalars(self) -> dict:
        o = (ctypes.c_double * len(SCALARS))()
        self.L.orc_scalars(self.h, o)
        return dict(zip(SCALARS, list(o)))

    def set_scalars(self, time, maxVel, maxNu, maxDiv):
        self.L.orc_set_scalars(self.h, time, maxVel, maxNu, maxDiv)

    def mg(self):
        out = []
        for l in range(self.L.orc_mg_levels(self.h)):
            info = (ctypes.c_int * 3)()
            self.L.orc_mg_info(self.h, l, info)
            n, nnz, nagg = list(info)
            agg = np.zeros(nagg, np.int32)
            rs = np.zeros(n + 1 if l > 0 else 0, np.int32)
            col = np.zeros(nnz, np.int32)
            val = np.zeros(nnz, np.float64)
            diag = np.zeros(n, np.float64)
            self.L.orc_mg_get(self.h, l, _ptr(agg), _ptr(rs), _ptr(col), _ptr(val), _ptr(diag))
            out.append(dict(n=n, agg=agg, rowStart=rs, col=col, val=val, diag=diag))
        return out
