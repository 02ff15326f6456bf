"""The V-cycle schedule autotuner of the mixed path (phx_batch_tune_vcycle):
per bucket of scenario size it picks the multigrid coarsening stop that steps
the batch fastest at the solve's relative residual, rebuilds the bucket's
hierarchies with it and restores the batch's state.

Checked here: the chosen stops are candidates; every field of the batch is
bit-identical before and after the call; each scenario's hierarchy is the one
its bucket's stop builds (a smaller stop never gives fewer levels); the tuned
batch keeps solving to the relative residual of 1e-8; an FP64 context keeps the
reference's schedule."""
import numpy as np
import pytest

from photon_gb300 import _lib, casegen
from photon_gb300.solver import Batch

pytestmark = pytest.mark.gpu

FIELDS = ("u", "v", "w", "p", "T", "Yo", "Yf", "Ys", "nu", "Pb", "S")


def rel_case(c):
    c.profile.tol = 0.0
    c.profile.rel_tol = 1e-8
    c.profile.maxIters = 400
    return c


def bucket(n):
    b, e = 0, 40000
    while n >= e and b < 7:
        e *= 2
        b += 1
    return b


def test_tuner_keeps_state_and_picks_candidates():
    cases = [rel_case(casegen.house(40, 32, 24, 0.2, 5)), rel_case(casegen.house_small(1)),
             rel_case(casegen.tiny_room(12, 10, 9, 0.2, 60e3))]
    B = Batch(cases, _lib.PREC_MIXED)
    for _ in range(10):
        B.step(0.02)
    B.sync()
    before = [{f: B.get(s, f) for f in FIELDS} for s in range(len(cases))]
    levels_ref = [B.mg_levels(s) for s in range(len(cases))]
    stops = B.tune_vcycle(2, 0.02)
    assert len(stops) == 8 and all(v in (2000, 1000, 500) for v in stops), stops
    assert B.coarse_sweeps in (1, 2)
    for s in range(len(cases)):
        for f in FIELDS:
            assert np.array_equal(B.get(s, f), before[s][f]), (s, f)
        lv = B.mg_levels(s)
        assert lv[:2] == levels_ref[s][:2]              # level 0 and level 1 do not depend on the stop
        assert len(lv) >= len(levels_ref[s]) if stops[bucket(cases[s].N)] < 2000 else lv == levels_ref[s]
    for _ in range(3):
        B.step(0.02)
        for s in range(len(cases)):
            assert B.stats(s)["pressure_rel_residual"] <= 1e-8
    B.close()


def test_tuner_leaves_fp64_schedule():
    c = rel_case(casegen.house(40, 32, 24, 0.2, 5))
    B = Batch([c], _lib.PREC_FP64)
    B.step(0.02)
    lv = B.mg_levels(0)
    assert B.tune_vcycle(2, 0.02) is not None
    assert B.mg_levels(0) == lv
    B.close()


def test_one_sweep_schedule_solves_to_the_bar(monkeypatch):
    """The mixed path's one-sweep coarse smoothing (one damped Jacobi sweep per
    level on each leg: the V-cycle stays symmetric) is a different
    preconditioner, not a different answer: forced through the tuner, the
    batch still meets the relative residual of 1e-8 on every step, and its
    pressure stays within the mixed path's bar of the two-sweep run's."""
    def run(sweeps):
        monkeypatch.setenv("PHX_COARSE_SWEEPS", str(sweeps))
        cases = [rel_case(casegen.house(40, 32, 24, 0.2, 5)), rel_case(casegen.house_small(1))]
        B = Batch(cases, _lib.PREC_MIXED)
        for _ in range(4):
            B.step(0.02)
        B.tune_vcycle(1, 0.02)
        assert B.coarse_sweeps == sweeps
        iters = []
        for _ in range(4):
            B.step(0.02)
            for s in range(len(cases)):
                assert B.stats(s)["pressure_rel_residual"] <= 1e-8
                iters.append(B.stats(s)["pressure_iters"])
        p = [B.get(s, "p") for s in range(len(cases))]
        B.close()
        return p, iters

    p1, it1 = run(1)
    p2, it2 = run(2)   # leaves the process-wide schedule at the reference's two sweeps
    for a, b in zip(p1, p2):
        assert np.linalg.norm(a - b) <= 1e-3 * np.linalg.norm(b)
    assert max(it1) <= 2 * max(it2)
