"""The reference arm's relative CG stop. RefSolver.step_relative sets the
reference's absolute stop (max|r| dt/dx^2 <= pressureTol,
src/sim/gasphase.cpp:594-605) before each step from the previous step's
max|b|, so that the reference stops at about the GPU path's relative residual
max|r| <= 1e-8 max|b|. Checked on the reference's FP32 build, the one the
bench times."""
import pytest

from oracle import refpy
from photon_gb300 import casegen

pytestmark = pytest.mark.skipif(not refpy.available(32), reason="reference FP32 build not present")

REL = 1e-8


def test_step_relative_stops_near_the_relative_residual():
    c = casegen.house(40, 30, 20, 0.2, 5)
    c.profile.tol = 1e-8
    c.profile.maxIters = 400
    s = refpy.RefSolver(c, 32, 2)
    rels = []
    for k in range(12):
        dt = s.step_relative(c.profile.dtMax, REL)
        if k < 4:
            continue
        sc = s.scalars()
        bmax = s.rhs_max_abs()
        assert bmax > 0
        assert 0 < sc["pressureIters"] < c.profile.maxIters
        rels.append(sc["pressureResidual"] * c.dx * c.dx / dt / bmax)
    assert max(rels) <= 2 * REL        # b is taken one step behind
    assert min(rels) >= 1e-3 * REL     # and the stop is not far stricter than asked


def test_step_relative_after_a_quiet_step_keeps_an_absolute_stop():
    c = casegen.tiny_room(12, 10, 9, 0.2, 0.0)     # no heat release: b stays zero
    s = refpy.RefSolver(c, 32, 2)
    for _ in range(3):
        s.step_relative(c.profile.dtMax, REL)
    assert s.rhs_max_abs() == 0
    assert s.scalars()["pressureIters"] == 0
