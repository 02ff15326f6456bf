"""ctypes access to the reference solver builds in oracle/_ref (test infrastructure).

`RefSolver(case, bits=64)` fills a reference photon::Solver with the arrays of a
synthetic case (photon_gb300.casegen.Case) and steps it. bits=64 is the FP64
oracle build, bits=32 the reference as shipped.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
_LIBS = {}

REAL_FIELDS = ("u", "v", "w", "fx", "fy", "fz", "ax", "ay", "az", "p", "S", "T", "Yo", "Yf", "Ys", "Ya", "Yp", "Yc",
               "Yw", "Yco", "Yai", "nu", "Pb", "Q", "Qr", "hrr", "massSrc", "zoneP", "rhs", "diag", "cgR", "cgZ",
               "cgP", "cgQ", "zoneDP")
U8_FIELDS = ("lx", "ly", "lz", "lit", "pilot", "blocked", "zoneOpen")
I32_FIELDS = ("zone",)
SCALARS = ("time", "maxVel", "maxNu", "maxDiv", "pressureIters", "pressureResidual", "hrr", "maxGasT",
           "burningCells", "fuelIn", "fuelBurned", "fuelInDomain", "leakFaces", "nZones")


def lib_path(bits: int) -> str:
    return os.path.join(HERE, "_ref", "libphoton_ref%d.so" % bits)


def available(bits: int = 64) -> bool:
    return os.path.exists(lib_path(bits))


def load(bits: int = 64):
    if bits in _LIBS:
        return _LIBS[bits]
    L = ctypes.CDLL(lib_path(bits))
    vp, d, i = ctypes.c_void_p, ctypes.c_double, ctypes.c_int
    L.ref_new.restype = vp
    L.ref_new.argtypes = [i]
    L.ref_free.argtypes = [vp]
    L.ref_init_grid.argtypes = [vp, i, i, i, d, d, d, d]
    L.ref_load_scene.argtypes = [vp, ctypes.c_char_p, ctypes.c_char_p, i, i, i, i, ctypes.c_char_p, i]
    L.ref_toggle_opening.argtypes = [vp, ctypes.c_char_p]
    L.ref_grid_info.argtypes = [vp, ctypes.c_void_p, ctypes.c_void_p]
    L.ref_set_profile.argtypes = [vp, d, d, i, d]
    L.ref_set_switches.argtypes = [vp, i, i]
    L.ref_set_pressure_tol.argtypes = [vp, d]
    L.ref_rhs_max_abs.restype = d
    L.ref_rhs_max_abs.argtypes = [vp]
    L.ref_set_wind.argtypes = [vp, d, d, d]
    L.ref_mark_geometry_dirty.argtypes = [vp]
    L.ref_add_burner.argtypes = [vp, d, d, d, d, d, d, d, d, d]
    L.ref_burner_cells.argtypes = [vp, i, ctypes.c_void_p, i]
    L.ref_add_ignition.argtypes = [vp, i, d, d]
    L.ref_step.restype = d
    L.ref_step.argtypes = [vp, d]
    L.ref_stage.argtypes = [vp, ctypes.c_char_p, d]
    L.ref_stable_dt.restype = d
    L.ref_stable_dt.argtypes = [vp, d]
    L.ref_precondition.argtypes = [vp, ctypes.c_void_p, ctypes.c_void_p]
    L.ref_field_len.restype = ctypes.c_long
    L.ref_field_len.argtypes = [vp, ctypes.c_char_p]
    L.ref_field.argtypes = [vp, ctypes.c_char_p, i, ctypes.c_void_p, ctypes.c_long]
    L.ref_scalars.argtypes = [vp, ctypes.c_void_p]
    L.ref_set_scalars.argtypes = [vp, d, d, d, d]
    L.ref_mg_levels.argtypes = [vp]
    L.ref_mg_info.argtypes = [vp, i, ctypes.c_void_p]
    L.ref_mg_get.argtypes = [vp, i, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
    L.ref_phase_ms.restype = d
    L.ref_phase_ms.argtypes = [vp, i]
    L.ref_set_stats.argtypes = [vp, ctypes.c_void_p]
    L.ref_rad_counts.argtypes = [vp, ctypes.c_void_p]
    L.ref_sample_device.restype = d
    L.ref_sample_device.argtypes = [vp, i, d, d, d, d, d]
    L.ref_rad_export.argtypes = [vp, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
    L.ref_rad_trace.argtypes = [vp, ctypes.c_void_p, ctypes.c_void_p]
    L.ref_compute_zones.argtypes = [vp]
    L.ref_save_state.argtypes = [vp, ctypes.c_char_p, ctypes.c_char_p, i]
    L.ref_load_state.argtypes = [vp, ctypes.c_char_p, ctypes.c_char_p, i]
    _LIBS[bits] = L
    return L


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(ctypes.c_void_p)


class RefSolver:
    def __init__(self, case=None, bits: int = 64, threads: int = 4):
        self.L = load(bits)
        self.bits = bits
        self.h = ctypes.c_void_p(self.L.ref_new(threads))
        if case is not None:
            self.setup(case)

    def __del__(self):
        try:
            if self.h:
                self.L.ref_free(self.h)
                self.h = None
        except Exception:
            pass

    def setup(self, case):
        L, h = self.L, self.h
        if L.ref_init_grid(h, case.nx, case.ny, case.nz, case.dx, case.ox, case.oy, case.oz) != 0:
            raise ValueError("grid size out of range")
        pr = case.profile
        L.ref_set_profile(h, pr.cfl, pr.dtMax, pr.maxIters, pr.tol)
        L.ref_set_switches(h, int(case.radiationOn), int(case.adiabatic))
        L.ref_set_wind(h, *case.wind)
        for n in ("fx", "fy", "fz", "ax", "ay", "az", "blocked", "lx", "ly", "lz"):
            self.set(n, getattr(case, n))
        L.ref_mark_geometry_dirty(h)
        self.burner_ids = []
        for b in case.burners:
            r = L.ref_add_burner(h, b.x0, b.y0, b.x1, b.y1, b.z, b.peakW, b.rampS, b.start, b.duration)
            self.burner_ids.append(r)

    def load_scene(self, data_dir: str, scene: str, reference_profile=True, radiation=False, adiabatic=True,
                   no_leak=True):
        err = ctypes.create_string_buffer(512)
        r = self.L.ref_load_scene(self.h, data_dir.encode(), scene.encode(), int(reference_profile), int(radiation),
                                  int(adiabatic), int(no_leak), err, 512)
        if r != 0:
            raise RuntimeError(err.value.decode())

    def grid(self):
        dims = (ctypes.c_int * 4)()
        geo = (ctypes.c_double * 4)()
        self.L.ref_grid_info(self.h, dims, geo)
        return tuple(dims), tuple(geo)

    def burner_cells(self, b: int):
        buf = np.zeros(4096, np.int32)
        n = self.L.ref_burner_cells(self.h, b, _ptr(buf), buf.size)
        return buf[:n].copy()

    def get(self, name: str) -> np.ndarray:
        n = self.L.ref_field_len(self.h, name.encode())
        if n < 0:
            raise KeyError(name)
        if name in U8_FIELDS:
            a = np.zeros(n, np.uint8)
        elif name in I32_FIELDS:
            a = np.zeros(n, np.int32)
        else:
            a = np.zeros(n, np.float64)
        if self.L.ref_field(self.h, name.encode(), 0, _ptr(a), n) < 0:
            raise KeyError(name)
        return a

    def set(self, name: str, arr):
        if name in U8_FIELDS:
            a = np.ascontiguousarray(arr, dtype=np.uint8)
        elif name in I32_FIELDS:
            a = np.ascontiguousarray(arr, dtype=np.int32)
        else:
            a = np.ascontiguousarray(arr, dtype=np.float64)
        if self.L.ref_field(self.h, name.encode(), 1, _ptr(a), a.size) < 0:
            raise KeyError(name)

    def step(self, dtMax: float) -> float:
        return self.L.ref_step(self.h, dtMax)

    def set_pressure_tol(self, tol: float):
        self.L.ref_set_pressure_tol(self.h, tol)

    def rhs_max_abs(self) -> float:
        return self.L.ref_rhs_max_abs(self.h)

    def step_relative(self, dtMax: float, rel_tol: float) -> float:
        """One step, then the CG stop of the next step set to rel_tol times
        this step's max|b| in 1/s. The reference has only an absolute stop,
        max|r| dt/dx^2 <= pressureTol (src/sim/gasphase.cpp:594-605); with
        this it stops at about max|r| <= rel_tol max|b|, the GPU path's
        relative stop, with b taken one step behind (1e-8 1/s after a step
        whose b was zero)."""
        dt = self.step(dtMax)
        dx = self.grid()[1][0]
        bmax = self.rhs_max_abs()
        self.set_pressure_tol(rel_tol * bmax * dt / (dx * dx) if bmax > 0 else 1e-8)
        return dt

    def stage(self, name: str, dt: float = 0.0):
        if self.L.ref_stage(self.h, name.encode(), dt) != 0:
            raise KeyError(name)

    def stable_dt(self, dtMax: float) -> float:
        return self.L.ref_stable_dt(self.h, dtMax)

    def precondition(self, r: np.ndarray) -> np.ndarray:
        r = np.ascontiguousarray(r, np.float64)
        z = np.zeros_like(r)
        self.L.ref_precondition(self.h, _ptr(r), _ptr(z))
        return z

    def scalars(self) -> dict:
        o = (ctypes.c_double * len(SCALARS))()
        self.L.ref_scalars(self.h, o)
        return dict(zip(SCALARS, list(o)))

    def set_scalars(self, time, maxVel, maxNu, maxDiv):
        self.L.ref_set_scalars(self.h, time, maxVel, maxNu, maxDiv)

    # stats under the names of the GPU library's phx_stats
    _STATS = (("time", "time"), ("max_vel", "maxVel"), ("max_nu", "maxNu"), ("max_div", "maxDiv"), ("hrr", "hrr"),
              ("max_gas_t", "maxGasT"), ("burning_cells", "burningCells"), ("fuel_in", "fuelIn"),
              ("fuel_burned", "fuelBurned"), ("fuel_in_domain", "fuelInDomain"))

    def stats(self) -> dict:
        sc = self.scalars()
        return {k: int(sc[r]) if k == "burning_cells" else sc[r] for k, r in self._STATS}

    def set_stats(self, st: dict):
        v = (ctypes.c_double * len(self._STATS))(*[float(st[k]) for k, _ in self._STATS])
        self.L.ref_set_stats(self.h, v)

    def rad_inputs(self) -> dict:
        """The radiation trace's inputs in flat form: elements (n x 11: o, n,
        area, eps, temp, sphere, skip own cell), walls (m x 4: axis, face, T
        from the lower cell, T from the upper cell), solidT (N)."""
        cnt = (ctypes.c_int * 2)()
        self.L.ref_rad_counts(self.h, cnt)
        elem = np.zeros((cnt[0], 11), np.float64)
        wall = np.zeros((cnt[1], 4), np.float64)
        (nx, ny, nz, n), _ = self.grid()
        solid = np.zeros(n, np.float64)
        self.L.ref_rad_export(self.h, _ptr(elem), _ptr(wall), _ptr(solid))
        return {"elements": elem, "walls": wall, "solidT": solid}

    def rad_trace(self):
        """Run Solver::traceRadiation; returns (radAbs per element, radGas per cell)."""
        cnt = (ctypes.c_int * 2)()
        self.L.ref_rad_counts(self.h, cnt)
        (nx, ny, nz, n), _ = self.grid()
        ab = np.zeros(cnt[0], np.float64)
        gas = np.zeros(n, np.float64)
        self.L.ref_rad_trace(self.h, _ptr(ab), _ptr(gas))
        return ab, gas

    # photon::DeviceKind (src/sim/devices.h:11)
    DEVICE_KINDS = ("Temperature", "VelU", "VelV", "VelW", "LayerHeight", "UpperTemp", "LowerTemp", "O2", "CO2",
                    "CO", "Soot", "Pressure")

    def sample_device(self, kind: str, x: float, y: float, z: float, z0: float = 0.0, z1: float = 0.0) -> float:
        """photon::sampleDevice on this solver (src/sim/devices.h:61-96)."""
        return self.L.ref_sample_device(self.h, self.DEVICE_KINDS.index(kind), x, y, z, z0, z1)

    def compute_zones(self):
        self.L.ref_compute_zones(self.h)

    def save_state(self, path: str):
        err = ctypes.create_string_buffer(512)
        if self.L.ref_save_state(self.h, path.encode(), err, 512) != 0:
            raise RuntimeError(err.value.decode())

    def load_state(self, path: str):
        err = ctypes.create_string_buffer(512)
        if self.L.ref_load_state(self.h, path.encode(), err, 512) != 0:
            raise RuntimeError(err.value.decode())

    def mg(self):
        """Multigrid hierarchy: list of dicts (n, agg, rowStart, col, val, diag)."""
        out = []
        for l in range(self.L.ref_mg_levels(self.h)):
            info = (ctypes.c_int * 3)()
            self.L.ref_mg_info(self.h, l, info)
            n, nnz, nagg = list(info)
            agg = np.zeros(nagg, np.int32)
            rs = np.zeros(n + 1 if l > 0 else 0, np.int32)
            col = np.zeros(nnz, np.int32)
            val = np.zeros(nnz, np.float64)
            diag = np.zeros(n, np.float64)
            self.L.ref_mg_get(self.h, l, _ptr(agg), _ptr(rs), _ptr(col), _ptr(val), _ptr(diag))
            out.append(dict(n=n, agg=agg, rowStart=rs, col=col, val=val, diag=diag))
        return out

    def phase_ms(self):
        return [self.L.ref_phase_ms(self.h, i) for i in range(10)]
