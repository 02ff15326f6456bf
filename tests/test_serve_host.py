"""Serving host logic without a GPU: request validation, the budget check at
submission and the queue (the host set-up runs on the CPU)."""
import ctypes

import pytest

from photon_gb300 import _lib, casegen
from photon_gb300.serve import Server
from photon_gb300.solver import PhxError, make_grid


def test_submit_validates_and_queues():
    srv = Server(_lib.PREC_MIXED, hbm_budget_bytes=1 << 30)
    rid = srv.submit(casegen.tiny_room(12, 10, 9, 0.2, 60e3), duration=1.0)
    info = srv.poll(rid)
    assert info["state"] == "queued" and info["device_bytes"] > 0 and info["cells"] == 12 * 10 * 9
    assert srv.counts() == {"queued": 1, "running": 0, "used_bytes": 0, "cell_updates": 0}
    with pytest.raises(PhxError):
        srv.submit(casegen.tiny_room(12, 10, 9, 0.2, 60e3), duration=-1.0)
    with pytest.raises(PhxError):
        srv.release(rid)              # still queued
    srv.close()


def test_request_larger_than_budget_is_refused():
    srv = Server(_lib.PREC_FP64, hbm_budget_bytes=1 << 20)
    with pytest.raises(PhxError) as e:
        srv.submit(casegen.tiny_room(40, 30, 20, 0.2, 60e3), duration=1.0)
    assert e.value.code == 6          # PHX_ERR_BUDGET
    srv.close()


def test_bad_grid_is_refused():
    srv = Server(_lib.PREC_MIXED, hbm_budget_bytes=1 << 30)
    c = casegen.tiny_room(12, 10, 9, 0.2, 60e3)
    g, keep = make_grid(c)
    g.nx = 0
    rid = ctypes.c_int()
    r = srv.L.phx_server_submit(srv.h, ctypes.byref(g), None, 0, 1.0, 0.02, ctypes.byref(rid))
    assert r == 1 and b"invalid grid" in srv.L.phx_server_last_error(srv.h)
    srv.close()
