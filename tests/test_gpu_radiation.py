"""The GPU radiation trace (phx_rad_trace; Solver::traceRadiation,
src/sim/radiation.cpp:181-319) against the reference's own trace recorded in
tests/golden/rad_sofa_room.npz, and against the oracle's restatement on a
larger seeded house.

FP64 context: radAbs and radGas within 1e-12 relative L2 of the reference (the
gas cells sum their rays' contributions by atomic adds, so only the order of
those sums and the last bit of exp differ). Mixed context: the trace runs in
FP32, the reference's own precision; within 1e-4 relative L2 of the FP64
reference."""
import numpy as np
import pytest

from oracle import oraclepy
from photon_gb300 import _lib, casegen
from photon_gb300.solver import PhxError, Solver

from gpu_util import rel_l2
from test_oracle_rad import load_fixture

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-12
FP32_TOL = 1e-4


def fixture_solver(fx, precision):
    nx, ny, nz = (int(v) for v in fx["dims"])
    dx, ox, oy, oz = (float(v) for v in fx["geo"])
    c = casegen.from_blocked("rad_sofa_room", fx["blocked"].reshape(nz, ny, nx), dx, (ox, oy, oz))
    g = Solver(c, precision)
    for f in oraclepy.RAD_GAS_FIELDS:
        g.set(f, fx[f].astype(np.float64))
    return g


@pytest.mark.parametrize("precision,tol", [(_lib.PREC_FP64, FP64_TOL), (_lib.PREC_MIXED, FP32_TOL)])
def test_trace_matches_reference(precision, tol):
    fx = load_fixture()
    g = fixture_solver(fx, precision)
    ab, gas = g.rad_trace(fx["elements"], fx["walls"], fx["solidT"])
    assert rel_l2(ab, fx["radAbs"]) <= tol
    assert rel_l2(gas, fx["radGas"]) <= tol
    assert g.rad_last_ms() > 0


def test_trace_fp64_elementwise():
    """Every element's absorbed power, not only the norm."""
    fx = load_fixture()
    g = fixture_solver(fx, _lib.PREC_FP64)
    ab, _ = g.rad_trace(fx["elements"], fx["walls"], fx["solidT"])
    ref = fx["radAbs"]
    assert np.all(np.abs(ab - ref) <= 1e-11 * np.maximum(np.abs(ref), 1.0))


def test_trace_wall_order_does_not_matter():
    fx = load_fixture()
    g = fixture_solver(fx, _lib.PREC_FP64)
    perm = np.random.default_rng(1).permutation(len(fx["walls"]))
    ab1, _ = g.rad_trace(fx["elements"], fx["walls"], fx["solidT"])
    ab2, _ = g.rad_trace(fx["elements"], fx["walls"][perm], fx["solidT"])
    np.testing.assert_array_equal(ab1, ab2)


@pytest.mark.parametrize("precision,tol", [(_lib.PREC_FP64, FP64_TOL), (_lib.PREC_MIXED, FP32_TOL)])
def test_trace_house_matches_oracle(precision, tol):
    """A seeded 72x52x44 house: 30 k elements, 9 k walls, hot plume and layer."""
    c = casegen.house_small(2)
    w = casegen.rad_workload(c)
    g = Solver(c, precision)
    for f, a in w["gas"].items():
        g.set(f, a)
    ab, gas = g.rad_trace(w["elements"], w["walls"], w["solidT"])
    oab, ogas = oraclepy.rad_trace((c.nx, c.ny, c.nz), (c.dx, c.ox, c.oy, c.oz), c.blocked, w["gas"], w["elements"],
                                   w["walls"], w["solidT"])
    assert rel_l2(ab, oab) <= tol
    assert rel_l2(gas, ogas) <= tol


def test_trace_ambient_room_exchanges_nothing():
    fx = load_fixture()
    g = fixture_solver(fx, _lib.PREC_FP64)
    n = fx["T"].size
    g.set("T", np.full(n, 293.15))
    g.set("hrr", np.zeros(n))
    el = fx["elements"].copy()
    el[:, 8] = 293.15
    wl = fx["walls"].copy()
    wl[:, 2:] = 293.15
    ab, gas = g.rad_trace(el, wl, np.full(n, 293.15))
    assert np.abs(ab).max() < 1e-9 and np.abs(gas).max() < 1e-9


def test_trace_without_elements_or_gas_output():
    fx = load_fixture()
    g = fixture_solver(fx, _lib.PREC_FP64)
    ab, gas = g.rad_trace(np.zeros((0, 11)), fx["walls"], None)
    assert ab.size == 0 and np.abs(gas).max() == 0
    ab, gas = g.rad_trace(fx["elements"][:10], np.zeros((0, 4)), None, gas=False)
    assert ab.size == 10 and gas is None


def test_trace_rejects_bad_walls():
    fx = load_fixture()
    g = fixture_solver(fx, _lib.PREC_FP64)
    two = np.concatenate([fx["walls"][:1], fx["walls"][:1]])
    with pytest.raises(PhxError, match="two radiation walls"):
        g.rad_trace(fx["elements"][:4], two, None)
    bad = fx["walls"][:1].copy()
    bad[0, 1] = 10 ** 8
    with pytest.raises(PhxError, match="out of range"):
        g.rad_trace(fx["elements"][:4], bad, None)
    bad[0, 0], bad[0, 1] = 3, 0
    with pytest.raises(PhxError, match="out of range"):
        g.rad_trace(fx["elements"][:4], bad, None)


def test_trace_and_render_of_a_batch_scenario():
    """phx_batch_rad_trace / phx_batch_vol_render on scenario 1 of a batch
    equal the single-context calls on the same case and fields."""
    from photon_gb300 import render
    from photon_gb300.solver import Batch
    c0, c1 = casegen.tiny_room(12, 10, 9, 0.2, 60e3), casegen.house_small(2)
    w = casegen.rad_workload(c1)
    B = Batch([c0, c1], _lib.PREC_FP64)
    g = Solver(c1, _lib.PREC_FP64)
    gas = dict(w["gas"])
    gas["Ys"] = gas["Ys"] * 0.01
    for f, a in gas.items():
        B.set(1, f, a)
        g.set(f, a)
    ab_b, gas_b = B.rad_trace(1, w["elements"], w["walls"], w["solidT"])
    ab_g, gas_g = g.rad_trace(w["elements"], w["walls"], w["solidT"])
    np.testing.assert_array_equal(ab_b, ab_g)                 # absorbed powers are summed in a fixed order
    assert rel_l2(gas_b, gas_g) <= 1e-13                      # gas cells gain by atomic adds
    cx, cy = c1.ox + c1.nx * c1.dx / 2, c1.oy + c1.ny * c1.dx / 2
    p = render.camera(c1, eye=(cx - 14, cy - 16, 9.0), target=(cx, cy, 2.0), width=96, height=54,
                      lights=render.fire_lights(c1, gas["hrr"]))
    np.testing.assert_array_equal(B.vol_render(1, p), g.vol_render(p))
