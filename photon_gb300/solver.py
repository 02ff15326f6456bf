"""Python mirror of photon::Solver's step API over the GB300 C ABI.

`Solver(case, precision)` creates a device context for a synthetic case
(photon_gb300.casegen.Case) or any arrays with the reference's layout; the
methods follow photon::Solver (src/sim/solver.h:156-347): step(dtMax) -> dt,
add_burner -> index, add_ignition, fields by name, and stats. Everything runs
in libphx.so on the GPU.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib
from ._lib import FIELD_ID, STAGE_ID, PhxError, PhxGrid, PhxStats


def _ptr(a):
    return ctypes.c_void_p(a.ctypes.data) if a is not None else None


def make_grid(case):
    """phx_grid for a case; returns (grid, arrays kept alive for the call)."""
    g = PhxGrid()
    g.nx, g.ny, g.nz = case.nx, case.ny, case.nz
    g.dx, g.ox, g.oy, g.oz = case.dx, case.ox, case.oy, case.oz
    pr = case.profile
    g.cfl, g.dt_max, g.max_iters, g.tol, g.rel_tol = pr.cfl, pr.dtMax, pr.maxIters, pr.tol, pr.rel_tol
    g.radiation_on, g.adiabatic_surfaces = int(case.radiationOn), int(case.adiabatic)
    g.wind_speed, g.wind_from_deg, g.wind_exponent = case.wind
    keep = {}
    for n in ("blocked", "lx", "ly", "lz"):
        keep[n] = np.ascontiguousarray(getattr(case, n), dtype=np.uint8)
    for n in ("fx", "fy", "fz", "ax", "ay", "az"):
        keep[n] = np.ascontiguousarray(getattr(case, n), dtype=np.float64)
    for n, a in keep.items():
        setattr(g, n, a.ctypes.data)
    return g, keep


# the gas-phase fields of a checkpoint, in the order Solver::saveState writes
# them (src/sim/state.cpp:75-79); geometry and solid-phase state stay on the host
CHECKPOINT_FIELDS = ("u", "v", "w", "p", "S", "T", "Yo", "Yf", "Ys", "Ya", "Yp", "Yc", "Yw", "Yco", "Yai",
                     "nu", "Pb", "zoneP", "hrr", "lit")
# the stats a checkpoint restores (time, maxVel, maxNu and SimStats)
STAT_KEYS = ("time", "max_vel", "max_nu", "max_div", "hrr", "max_gas_t", "burning_cells", "fuel_in",
             "fuel_burned", "fuel_in_domain")


def _mg_rows(L, h, s):
    """unknowns per multigrid level of scenario s (phx_batch_mg_info)"""
    nl = ctypes.c_int()
    rows = (ctypes.c_int * 16)()
    r = L.phx_batch_mg_info(h, s, ctypes.byref(nl), ctypes.cast(rows, ctypes.c_void_p), 16)
    if r != 0:
        raise PhxError(r, L.phx_last_error(h).decode())
    return [rows[l] for l in range(min(nl.value, 16))]


class Solver:
    def __init__(self, case, precision: int = _lib.PREC_FP64, add_burners: bool = True):
        self.L = _lib.load()
        self.case = case
        self.h = ctypes.c_void_p()
        g, keep = make_grid(case)
        r = self.L.phx_create(ctypes.byref(g), precision, ctypes.byref(self.h))
        if r != 0:
            raise PhxError(r, self.L.phx_last_global_error().decode())
        self.precision = precision
        self.burner_ids = []
        if add_burners:
            for b in case.burners:
                self.burner_ids.append(self.add_burner(b.x0, b.y0, b.x1, b.y1, b.z, b.peakW, b.rampS, b.start, b.duration))

    def close(self):
        if self.h:
            self.L.phx_destroy(self.h)
            self.h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, r):
        if r != 0:
            raise PhxError(r, self.L.phx_last_error(self.h).decode())

    def add_burner(self, x0, y0, x1, y1, z, peakW, rampS=0.0, start=0.0, duration=1e9) -> int:
        idx = ctypes.c_int(-1)
        self._check(self.L.phx_add_burner(self.h, x0, y0, x1, y1, z, peakW, rampS, start, duration, ctypes.byref(idx)))
        return idx.value

    def add_ignition(self, cell, power, duration):
        self._check(self.L.phx_add_ignition(self.h, int(cell), float(power), float(duration)))

    def step(self, dtMax: float) -> float:
        dt = ctypes.c_double()
        self._check(self.L.phx_step(self.h, dtMax, ctypes.byref(dt)))
        return dt.value

    def run(self, n: int, dtMax: float) -> np.ndarray:
        out = np.zeros(n, np.float64)
        self._check(self.L.phx_run(self.h, n, dtMax, _ptr(out)))
        return out

    def stage(self, name: str, arg: float = 0.0):
        self._check(self.L.phx_stage(self.h, STAGE_ID[name], arg))

    def precondition(self, r: np.ndarray) -> np.ndarray:
        r = np.ascontiguousarray(r, np.float64)
        z = np.zeros_like(r)
        self._check(self.L.phx_precondition(self.h, _ptr(r), _ptr(z)))
        return z

    def _dtype(self, name):
        return np.uint8 if name == "lit" else np.int32 if name == "zone" else np.float64

    def get(self, name: str) -> np.ndarray:
        fid = FIELD_ID[name]
        n = self.L.phx_field_count(self.h, fid)
        a = np.zeros(n, self._dtype(name))
        self._check(self.L.phx_get_field(self.h, fid, _ptr(a), a.nbytes))
        return a

    def set(self, name: str, arr):
        a = np.ascontiguousarray(arr, dtype=self._dtype(name))
        self._check(self.L.phx_set_field(self.h, FIELD_ID[name], _ptr(a), a.nbytes))

    def stats(self) -> dict:
        s = PhxStats()
        self._check(self.L.phx_get_stats(self.h, ctypes.byref(s)))
        return {k: getattr(s, k) for k, _ in PhxStats._fields_}

    def set_scalars(self, time, maxVel, maxNu, maxDiv):
        self._check(self.L.phx_set_scalars(self.h, time, maxVel, maxNu, maxDiv))

    def set_stats(self, st: dict):
        """Restore the scalars a checkpoint holds (keys as stats() returns them)."""
        s = PhxStats()
        for k in STAT_KEYS:
            setattr(s, k, int(st[k]) if k == "burning_cells" else float(st[k]))
        self._check(self.L.phx_set_stats(self.h, ctypes.byref(s)))

    def export_state(self, host):
        """Copy the gas-phase state into `host` (get/set by field name,
        set_stats), e.g. a host solver about to write a checkpoint
        (Solver::saveState, src/sim/state.cpp:62-121). The host's zone tables
        must exist; zones depend on the geometry only."""
        for f in CHECKPOINT_FIELDS:
            host.set(f, self.get(f))
        host.set_stats(self.stats())

    def import_state(self, host):
        """The reverse of export_state, after `host` loaded a checkpoint
        (Solver::loadState, src/sim/state.cpp:123-195)."""
        if len(host.get("zoneP")) != len(self.get("zoneP")):
            raise PhxError(_lib.PHX_ERR_INVALID, "state zone count does not match")
        for f in CHECKPOINT_FIELDS:
            self.set(f, host.get(f))
        self.set_stats(host.stats())

    def rad_trace(self, elements, walls, solid_t=None, gas: bool = True):
        """Solver::traceRadiation (src/sim/radiation.cpp:181-319) on the GPU over
        this context's gas fields: elements (phx_rad_elem records or an (n, 11)
        array), walls (phx_rad_wall records or an (m, 4) array), solid_t (N, K,
        or None for ambient). Returns (radAbs per element, radGas per cell or
        None); rad_last_ms() is the device time of its kernels."""
        el, wl = _lib.rad_elements(elements), _lib.rad_walls(walls)
        n = len(self.get("T"))
        st = None if solid_t is None else np.ascontiguousarray(solid_t, np.float64)
        if st is not None and st.size != n:
            raise PhxError(_lib.PHX_ERR_INVALID, "solid_t needs one value per cell")
        ab = np.zeros(len(el), np.float64)
        g = np.zeros(n, np.float64) if gas else None
        self._check(self.L.phx_rad_trace(self.h, el.ctypes.data if len(el) else None, len(el),
                                         wl.ctypes.data if len(wl) else None, len(wl),
                                         None if st is None else st.ctypes.data, ab.ctypes.data,
                                         None if g is None else g.ctypes.data))
        return ab, g

    def rad_last_ms(self) -> float:
        return float(self.L.phx_rad_last_ms(self.h))

    def vol_render(self, params, depth=None) -> np.ndarray:
        """The viewer's smoke and flame volume render of this context's fields
        (src/render/renderer.cpp:119-283): params is a PhxVolParams
        (photon_gb300.render.camera builds one); returns an (height, width, 3)
        float image, rows from the bottom. vol_last_ms() is its device time."""
        rgb = np.zeros((params.height, params.width, 3), np.float32)
        d = None if depth is None else np.ascontiguousarray(depth, np.float32)
        if d is not None and d.size != params.width * params.height:
            raise PhxError(_lib.PHX_ERR_INVALID, "depth needs one value per pixel")
        self._check(self.L.phx_vol_render(self.h, ctypes.byref(params), None if d is None else d.ctypes.data,
                                          rgb.ctypes.data))
        return rgb

    def vol_last_ms(self) -> float:
        return float(self.L.phx_vol_last_ms(self.h))

    def selftest_wait_timeout(self, limit_ms: float = 20.0):
        """Make one bounded device wait run out (phx_selftest_wait_timeout);
        raises PhxError with PHX_ERR_TIMEOUT, after which the context is usable."""
        self._check(self.L.phx_selftest_wait_timeout(self.h, float(limit_ms)))

    def mg_levels(self) -> list:
        """unknowns of each level of the pressure multigrid"""
        return _mg_rows(self.L, self.h, 0)

    def device_bytes(self) -> int:
        return int(self.L.phx_device_bytes(self.h))

    def sync(self):
        self._check(self.L.phx_sync(self.h))

    def time_steps(self, n: int, dtMax: float, flush_l2: bool = False):
        """Device time (ms, CUDA events) of n steps and their kernel launches."""
        tot, nl = ctypes.c_double(), ctypes.c_int()
        self._check(self.L.phx_time_steps(self.h, n, dtMax, int(flush_l2), ctypes.byref(tot), ctypes.byref(nl)))
        return tot.value, nl.value

    def profile_step(self, dtMax: float, flush_l2: bool = True) -> list:
        """One step with events around every launch: [(kernel, launches, ms)]."""
        cap = 128
        arr = (_lib.PhxKernelTime * cap)()
        n = ctypes.c_int()
        self._check(self.L.phx_profile_step(self.h, dtMax, int(flush_l2), arr, cap, ctypes.byref(n)))
        return [(arr[i].name.decode(), arr[i].launches, arr[i].ms) for i in range(min(n.value, cap))]

    def last_launches(self) -> int:
        return int(self.L.phx_last_step_launches(self.h))


class Batch:
    """Several scenarios stepped together by the same kernel launches (one CUDA
    graph per step). Scenario indices are positions; removing one moves the
    later ones down."""

    def __init__(self, cases=(), precision: int = _lib.PREC_FP64, add_burners: bool = True):
        self.L = _lib.load()
        self.h = ctypes.c_void_p()
        self.precision = precision
        r = self.L.phx_create_batch(None, 0, precision, ctypes.byref(self.h))
        if r != 0:
            raise PhxError(r, self.L.phx_last_global_error().decode())
        self.cases = []
        for c in cases:
            self.add(c, add_burners)

    def close(self):
        if self.h:
            self.L.phx_destroy(self.h)
            self.h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, r):
        if r != 0:
            raise PhxError(r, self.L.phx_last_error(self.h).decode())

    def add(self, case, add_burners: bool = True) -> int:
        g, keep = make_grid(case)
        sid = ctypes.c_int(-1)
        self._check(self.L.phx_batch_add(self.h, ctypes.byref(g), ctypes.byref(sid)))
        self.cases.append(case)
        if add_burners:
            for b in case.burners:
                idx = ctypes.c_int(-1)
                self._check(self.L.phx_batch_add_burner(self.h, sid.value, b.x0, b.y0, b.x1, b.y1, b.z, b.peakW,
                                                        b.rampS, b.start, b.duration, ctypes.byref(idx)))
        return sid.value

    def remove(self, s: int):
        self._check(self.L.phx_batch_remove(self.h, s))
        del self.cases[s]

    def __len__(self):
        return self.L.phx_batch_size(self.h)

    def mg_levels(self, s: int) -> list:
        """unknowns of each level of scenario s's pressure multigrid"""
        return _mg_rows(self.L, self.h, s)

    def mg_nnz(self, s: int) -> list:
        """stored off-diagonal entries of each level's CSR rows (phx_batch_mg_nnz; 0 for level 0)"""
        n = len(self.mg_levels(s))
        out = (ctypes.c_int * 16)()
        self._check(self.L.phx_batch_mg_nnz(self.h, s, ctypes.cast(out, ctypes.c_void_p), 16))
        return [out[l] for l in range(min(n, 16))]

    def tune_vcycle(self, steps: int = 3, dtMax: float = 0.02) -> list:
        """phx_batch_tune_vcycle: the coarsening stop chosen per size bucket;
        the coarse levels' Jacobi sweeps per leg it chose go to self.coarse_sweeps"""
        out = (ctypes.c_int * 9)()
        self._check(self.L.phx_batch_tune_vcycle(self.h, steps, dtMax, ctypes.cast(out, ctypes.c_void_p), 9))
        self.coarse_sweeps = out[8]
        return list(out)[:8]

    def scenario_bytes(self, s: int) -> int:
        return int(self.L.phx_batch_scenario_bytes(self.h, s))

    def step(self, dtMax=None) -> np.ndarray:
        """One step of every scenario; dtMax: scalar or one per scenario (default:
        each scenario's profile dtMax). Returns each scenario's dt."""
        n = len(self)
        if dtMax is None:
            dtm = np.array([c.profile.dtMax for c in self.cases], np.float64)
        else:
            dtm = np.broadcast_to(np.asarray(dtMax, np.float64), (n,)).copy()
        out = np.zeros(n, np.float64)
        self._check(self.L.phx_batch_step(self.h, _ptr(dtm), 0.0, _ptr(out)))
        return out

    def run(self, n: int, dtMax: float):
        for _ in range(n):
            self.step_fast(dtMax)

    def step_fast(self, dtMax: float):
        """One step of every scenario with one dtMax and no read-back."""
        self._check(self.L.phx_batch_step(self.h, None, float(dtMax), None))

    def get(self, s: int, name: str) -> np.ndarray:
        fid = FIELD_ID[name]
        n = self.L.phx_batch_field_count(self.h, s, fid)
        dt = np.uint8 if name == "lit" else np.int32 if name == "zone" else np.float64
        a = np.zeros(n, dt)
        self._check(self.L.phx_batch_get_field(self.h, s, fid, _ptr(a), a.nbytes))
        return a

    def set(self, s: int, name: str, arr):
        dt = np.uint8 if name == "lit" else np.int32 if name == "zone" else np.float64
        a = np.ascontiguousarray(arr, dtype=dt)
        self._check(self.L.phx_batch_set_field(self.h, s, FIELD_ID[name], _ptr(a), a.nbytes))

    def stats(self, s: int) -> dict:
        st = PhxStats()
        self._check(self.L.phx_batch_get_stats(self.h, s, ctypes.byref(st)))
        return {k: getattr(st, k) for k, _ in PhxStats._fields_}

    def rad_trace(self, s: int, elements, walls, solid_t=None, gas: bool = True):
        """Solver.rad_trace for scenario s of the batch (phx_batch_rad_trace)."""
        el, wl = _lib.rad_elements(elements), _lib.rad_walls(walls)
        n = len(self.get(s, "T"))
        st = None if solid_t is None else np.ascontiguousarray(solid_t, np.float64)
        ab = np.zeros(len(el), np.float64)
        g = np.zeros(n, np.float64) if gas else None
        self._check(self.L.phx_batch_rad_trace(self.h, s, el.ctypes.data if len(el) else None, len(el),
                                               wl.ctypes.data if len(wl) else None, len(wl),
                                               None if st is None else st.ctypes.data, ab.ctypes.data,
                                               None if g is None else g.ctypes.data))
        return ab, g

    def vol_render(self, s: int, params, depth=None) -> np.ndarray:
        """Solver.vol_render for scenario s of the batch (phx_batch_vol_render)."""
        rgb = np.zeros((params.height, params.width, 3), np.float32)
        d = None if depth is None else np.ascontiguousarray(depth, np.float32)
        self._check(self.L.phx_batch_vol_render(self.h, s, ctypes.byref(params), None if d is None else d.ctypes.data,
                                                rgb.ctypes.data))
        return rgb

    def device_bytes(self) -> int:
        return int(self.L.phx_device_bytes(self.h))

    def sync(self):
        self._check(self.L.phx_sync(self.h))

    def time_steps(self, n: int, dtMax: float, flush_l2: bool = False):
        tot, nl = ctypes.c_double(), ctypes.c_int()
        self._check(self.L.phx_time_steps(self.h, n, dtMax, int(flush_l2), ctypes.byref(tot), ctypes.byref(nl)))
        return tot.value, nl.value

    def profile_step(self, dtMax: float, flush_l2: bool = False) -> list:
        cap = 128
        arr = (_lib.PhxKernelTime * cap)()
        n = ctypes.c_int()
        self._check(self.L.phx_profile_step(self.h, dtMax, int(flush_l2), arr, cap, ctypes.byref(n)))
        return [(arr[i].name.decode(), arr[i].launches, arr[i].ms) for i in range(min(n.value, cap))]
