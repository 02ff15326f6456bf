"""Python face of the serving loop (include/phx.h, phx_server_*).

A Server owns one batch on the GPU. Requests are submitted with their grid,
burners, simulated duration and dtMax; step() admits queued requests that fit
the HBM budget, steps every running request once in the same kernel launches
and retires the finished ones (their final fields stay readable on the host
until release()).
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib
from ._lib import FIELD_ID, PhxRequestInfo, PhxStats
from .solver import PhxError, make_grid

STATES = {_lib.REQ_QUEUED: "queued", _lib.REQ_RUNNING: "running", _lib.REQ_DONE: "done",
          _lib.REQ_REJECTED: "rejected"}


class Server:
    def __init__(self, precision: int = _lib.PREC_MIXED, hbm_budget_bytes: int = 150 << 30, max_scenarios: int = 1024):
        self.L = _lib.load()
        self.h = ctypes.c_void_p()
        r = self.L.phx_server_create(precision, int(hbm_budget_bytes), int(max_scenarios), ctypes.byref(self.h))
        if r != 0:
            raise PhxError(r, "phx_server_create failed")
        self.cases = {}

    def close(self):
        if self.h:
            self.L.phx_server_destroy(self.h)
            self.h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, r):
        if r != 0:
            raise PhxError(r, self.L.phx_server_last_error(self.h).decode())

    def submit(self, case, duration: float, dt_max: float | None = None) -> int:
        """Queue a request (host set-up runs in the calling thread); returns its id."""
        g, keep = make_grid(case)
        b = np.array([[x.x0, x.y0, x.x1, x.y1, x.z, x.peakW, x.rampS, x.start, x.duration] for x in case.burners],
                     dtype=np.float64).reshape(-1, 9)
        rid = ctypes.c_int()
        self._check(self.L.phx_server_submit(self.h, ctypes.byref(g), b.ctypes.data if len(b) else None, len(b),
                                             float(duration), float(dt_max or case.profile.dtMax), ctypes.byref(rid)))
        self.cases[rid.value] = case
        return rid.value

    def step(self):
        """Admit, step once, retire: returns (admitted, finished, running)."""
        a, f, n = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        self._check(self.L.phx_server_step(self.h, ctypes.byref(a), ctypes.byref(f), ctypes.byref(n)))
        return a.value, f.value, n.value

    def poll(self, rid: int) -> dict:
        info = PhxRequestInfo()
        self._check(self.L.phx_server_poll(self.h, rid, ctypes.byref(info)))
        out = {k: getattr(info, k) for k, _ in PhxRequestInfo._fields_ if k != "stats"}
        out["state"] = STATES.get(info.state, str(info.state))
        out["stats"] = {k: getattr(info.stats, k) for k, _ in PhxStats._fields_}
        return out

    def get(self, rid: int, name: str) -> np.ndarray:
        c = self.cases[rid]
        n = {"u": (c.nx + 1) * c.ny * c.nz, "v": c.nx * (c.ny + 1) * c.nz, "w": c.nx * c.ny * (c.nz + 1)}.get(name, c.N)
        a = np.zeros(n, np.float64)
        self._check(self.L.phx_server_get_field(self.h, rid, FIELD_ID[name], a.ctypes.data, a.nbytes))
        return a

    def release(self, rid: int):
        self._check(self.L.phx_server_release(self.h, rid))
        self.cases.pop(rid, None)

    def counts(self) -> dict:
        q, r, u, cu = ctypes.c_int(), ctypes.c_int(), ctypes.c_size_t(), ctypes.c_longlong()
        self._check(self.L.phx_server_counts(self.h, ctypes.byref(q), ctypes.byref(r), ctypes.byref(u), ctypes.byref(cu)))
        return {"queued": q.value, "running": r.value, "used_bytes": u.value, "cell_updates": cu.value}
