"""Serving form: requests that arrive while others run are admitted between
steps as the HBM budget allows, share the kernel launches, and each result is
the same as the request run alone (bit for bit: every scenario's arithmetic
and reduction order is independent of the batch)."""
import numpy as np
import pytest

from photon_gb300 import _lib, casegen
from photon_gb300.serve import Server
from photon_gb300.solver import Solver

pytestmark = pytest.mark.gpu

FIELDS = ("u", "v", "w", "p", "T", "Yo", "Yf", "Ys", "nu", "hrr")


def requests():
    a = casegen.tiny_room(12, 10, 9, 0.2, 60e3)
    b = casegen.house(24, 20, 14, 0.2, 3)
    c = casegen.tiny_room(10, 8, 8, 0.2, 40e3, doorway=False)
    for x in (a, b, c):
        x.profile.tol = 0.0
        x.profile.rel_tol = 1e-8
    return [(a, 0.2, 0.02), (b, 0.15, 0.025), (c, 0.12, 0.02)]


def alone(case, duration, dt_max, precision):
    s = Solver(case, precision)
    while s.stats()["time"] < duration:
        s.step(dt_max)
    out = {f: s.get(f) for f in FIELDS}
    st = s.stats()
    s.close()
    return out, st


@pytest.mark.parametrize("precision", [_lib.PREC_FP64, _lib.PREC_MIXED])
def test_served_requests_equal_alone(precision):
    reqs = requests()
    srv = Server(precision, hbm_budget_bytes=8 << 30)
    ids = [srv.submit(reqs[0][0], reqs[0][1], reqs[0][2])]
    for _ in range(3):
        srv.step()
    ids.append(srv.submit(reqs[1][0], reqs[1][1], reqs[1][2]))   # arrives while the first runs
    srv.step()
    ids.append(srv.submit(reqs[2][0], reqs[2][1], reqs[2][2]))
    for _ in range(1000):
        srv.step()
        if all(srv.poll(i)["state"] == "done" for i in ids):
            break
    for rid, (case, duration, dt_max) in zip(ids, reqs):
        info = srv.poll(rid)
        assert info["state"] == "done" and info["sim_time"] >= duration
        ref, st = alone(case, duration, dt_max, precision)
        assert info["stats"]["time"] == st["time"]
        assert info["stats"]["pressure_iters"] == st["pressure_iters"]
        for f in FIELDS:
            a = srv.get(rid, f)
            assert np.array_equal(a, ref[f]), (rid, f, float(np.max(np.abs(a - ref[f]))))
        srv.release(rid)
    srv.close()


def test_budget_admits_in_order_as_memory_frees():
    reqs = requests()
    srv = Server(_lib.PREC_MIXED, hbm_budget_bytes=1 << 30)
    a = srv.submit(reqs[1][0], 0.1, 0.025)
    need = srv.poll(a)["device_bytes"]
    srv.close()
    # room for one request at a time
    srv = Server(_lib.PREC_MIXED, hbm_budget_bytes=int(need * 1.5))
    ids = [srv.submit(reqs[1][0], 0.1, 0.025), srv.submit(reqs[1][0], 0.05, 0.025)]
    peak = 0
    for _ in range(500):
        srv.step()
        c = srv.counts()
        assert c["used_bytes"] <= int(need * 1.5)
        peak = max(peak, c["running"])
        if all(srv.poll(i)["state"] == "done" for i in ids):
            break
    first, second = srv.poll(ids[0]), srv.poll(ids[1])
    assert peak == 1
    assert first["state"] == second["state"] == "done"
    assert second["t_admit"] >= first["t_done"]
    srv.close()
