"""FP64 GPU parity with the oracle at the workloads' own grid sizes.

The small parity cases (tests/test_gpu_parity.py) have at most 6,720 cells,
so their pressure multigrid stops at level 1: the reference coarsens past a
level only while it has more than 2,000 rows (src/sim/pressure_mg.cpp:141).
The grids here are large enough for three or more levels, so the damped
Jacobi sweeps of the intermediate levels (k_jacobi, k_res_restrict_jac0;
pressure_mg.cpp:237-257, 285-297), the coarsening of levels 2 and up
(pressure_mg.cpp:141-184) and the dense coarsest operator of a deep hierarchy
are all compared with the oracle:

- the 36x24x24 single room at 0.1 m (20,736 cells, levels 20736/2592/324);
- a 40x32x24 seeded house at 0.2 m (30,720 cells);
- the 72x52x44 seeded house at 0.2 m (164,736 cells, four levels);
- the smallest and the largest scenario of the 64-scenario batch workload
  (19,456 and 391,230 cells).

Each test first checks that the GPU built the oracle's hierarchy, level by
level, with at least three levels. The pressure solve stops at the relative
residual the benchmark uses (max|r| <= 1e-8 max|b|). Bars: one V-cycle within
1e-12 relative L2; every step within 1e-9 relative L2 on pressure, velocity
and the scalars, with the same dt (1e-12) and the same CG iteration count as
the oracle on every step."""
import numpy as np
import pytest

from oracle.oraclepy import OracleSolver
from photon_gb300 import casegen
from photon_gb300.solver import Solver

from gpu_util import STATE, rel_l2

pytestmark = pytest.mark.gpu

STEP_TOL = 1e-9
STAGE_TOL = 1e-12


def rel_case(c):
    c.profile.tol = 0.0
    c.profile.rel_tol = 1e-8
    c.profile.maxIters = 400
    return c


def _batch_extreme(which):
    cs = casegen.batch_scenarios(64)
    c = min(cs, key=lambda c: c.N) if which == "min" else max(cs, key=lambda c: c.N)
    return c


CASES = {
    "single_room_36x24x24": lambda: rel_case(casegen.single_room()),
    "house_40x32x24": lambda: rel_case(casegen.house(40, 32, 24, 0.2, 5)),
    "house_72x52x44": lambda: rel_case(casegen.house_small(1)),
    "batch_smallest": lambda: rel_case(_batch_extreme("min")),
    "batch_largest": lambda: rel_case(_batch_extreme("max")),
}
# (oracle steps before the GPU takes over, steps compared)
RUNS = {
    "single_room_36x24x24": (60, 8),
    "house_40x32x24": (40, 6),
    "house_72x52x44": (30, 4),
    "batch_smallest": (30, 3),
    "batch_largest": (20, 3),
}


def check_hierarchy(o, g):
    rows_o = [l["n"] for l in o.mg()]
    rows_g = g.mg_levels()
    assert rows_g == rows_o, (rows_g, rows_o)
    assert len(rows_g) >= 3, rows_g
    return rows_g


def load_state(o, g):
    for f in STATE:
        g.set(f, o.get(f))
    g.set("lit", o.get("lit"))
    g.set("zoneP", o.get("zoneP"))
    sc = o.scalars()
    g.set_scalars(sc["time"], sc["maxVel"], sc["maxNu"], sc["maxDiv"])


def step_both(o, g, n, what):
    for s in range(n):
        dto = o.step(0.02)
        dtg = g.step(0.02)
        assert abs(dtg - dto) <= 1e-12 * dto, (what, s, dtg, dto)
        bad = {}
        for f in STATE:
            e = rel_l2(g.get(f), o.get(f))
            if not e <= STEP_TOL:
                bad[f] = e
        assert not bad, "%s step %d: %s" % (what, s, bad)
        it_o, it_g = int(o.scalars()["pressureIters"]), g.stats()["pressure_iters"]
        assert it_g == it_o, (what, s, it_g, it_o)
        assert g.stats()["pressure_rel_residual"] <= 1e-8


@pytest.mark.parametrize("name", list(CASES))
def test_hierarchy_and_vcycle_match_oracle(name):
    c = CASES[name]()
    o = OracleSolver(c)
    o.step(0.02)
    g = Solver(c)
    check_hierarchy(o, g)
    rng = np.random.default_rng(7)
    for _ in range(2):
        r = rng.standard_normal(c.N) * (1 - c.blocked)
        assert rel_l2(g.precondition(r), o.precondition(r)) <= STAGE_TOL


@pytest.mark.parametrize("name", list(CASES))
def test_steps_from_developed_state_match_oracle(name):
    """The oracle runs the fire up for a while; the GPU takes over its state
    and both step on, compared every step."""
    c = CASES[name]()
    spin, n = RUNS[name]
    o = OracleSolver(c)
    for _ in range(spin):
        o.step(0.02)
    g = Solver(c)
    check_hierarchy(o, g)
    load_state(o, g)
    step_both(o, g, n, name)


def test_single_room_steps_from_start_match_oracle():
    """The 36x24x24 room from its initial state, 24 steps, GPU and oracle
    side by side with no state exchanged."""
    c = CASES["single_room_36x24x24"]()
    o = OracleSolver(c)
    g = Solver(c)
    step_both(o, g, 24, "single room from start")
    so, sg = o.scalars(), g.stats()
    assert abs(sg["hrr"] - so["hrr"]) <= 1e-9 * max(1.0, so["hrr"])
    assert sg["burning_cells"] == so["burningCells"]
    assert abs(sg["fuel_in_domain"] - so["fuelInDomain"]) <= 1e-9 * max(1e-12, so["fuelInDomain"])
