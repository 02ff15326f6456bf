"""Pin the FP64 oracle against the reference's own source built at FP64
(oracle/_ref/libphoton_ref64.so, made by oracle/make_ref.py where the
reference checkout exists). Skipped where that build is absent."""
import numpy as np
import pytest

from oracle import refpy
from oracle.oraclepy import OracleSolver
from photon_gb300 import casegen

pytestmark = pytest.mark.skipif(not refpy.available(64), reason="reference FP64 build not present")

FIELDS = ("u", "v", "w", "p", "S", "T", "Yo", "Yf", "Ys", "Ya", "Yp", "Yc", "Yw", "Yco", "Yai", "nu", "Pb", "Q",
          "Qr", "hrr", "massSrc", "zone", "lit")


def _compare(c, steps, dtMax):
    r = refpy.RefSolver(c, 64, 2)
    o = OracleSolver(c)
    assert list(r.burner_cells(0)) == list(o.burner_cells(0))
    for s in range(steps):
        assert r.step(dtMax) == o.step(dtMax)
        for f in FIELDS:
            a, b = r.get(f), o.get(f)
            assert np.array_equal(a, b), "step %d field %s" % (s, f)
        assert r.scalars() == o.scalars()
    for x, y in zip(r.mg(), o.mg()):
        for k in ("agg", "rowStart", "col", "val", "diag"):
            assert np.array_equal(x[k], y[k]), k
    return r.scalars()


def test_pin_single_room_36x24x24():
    sc = _compare(casegen.single_room(), 3, 0.02)
    assert sc["pressureIters"] > 0


def test_pin_house_blocked_cells():
    _compare(casegen.house(40, 30, 20, 0.2, 5), 3, 0.02)


def test_pin_precondition_single_vcycle():
    c = casegen.tiny_room()
    r = refpy.RefSolver(c, 64, 2)
    o = OracleSolver(c)
    r.step(0.02)
    o.step(0.02)
    rng = np.random.default_rng(0)
    vec = rng.standard_normal(c.N)
    assert np.array_equal(r.precondition(vec), o.precondition(vec))
