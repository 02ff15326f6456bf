"""Batching: scenarios of different grids stepped together by the same kernel
launches give the same results as each scenario alone (bit for bit in FP64:
every scenario's arithmetic and reduction order is independent of the batch),
including when a scenario joins or leaves between steps."""
import numpy as np
import pytest

from photon_gb300 import _lib, casegen
from photon_gb300.solver import Batch, PhxError, Solver

from gpu_util import STATE

pytestmark = pytest.mark.gpu


def cases():
    a = casegen.tiny_room(12, 10, 9, 0.2, 60e3)
    b = casegen.house(24, 20, 14, 0.2, 3)
    c = casegen.tiny_room(10, 8, 8, 0.2, 40e3, doorway=False)
    for x in (a, b, c):
        x.profile.tol = 0.0
        x.profile.rel_tol = 1e-8
    return [a, b, c]


@pytest.mark.parametrize("precision", [_lib.PREC_FP64, _lib.PREC_MIXED])
def test_batch_equals_alone(precision):
    cs = cases()
    B = Batch(cs, precision)
    alone = [Solver(c, precision) for c in cs]
    for step in range(8):
        dts = B.step(0.02)
        for s, g in enumerate(alone):
            assert g.step(0.02) == dts[s]
    for s, g in enumerate(alone):
        for f in STATE:
            a, b = B.get(s, f), g.get(f)
            assert np.array_equal(a, b), (precision, s, f, float(np.max(np.abs(a - b))))
        assert B.stats(s)["pressure_iters"] == g.stats()["pressure_iters"]


def test_batch_membership_change_keeps_results():
    cs = cases()
    B = Batch(cs[:2], _lib.PREC_FP64)
    ref = [Solver(c, _lib.PREC_FP64) for c in cs]
    for _ in range(3):
        B.step(0.02)
        ref[0].step(0.02)
        ref[1].step(0.02)
    B.add(cs[2])                 # joins mid-run
    B.remove(0)                  # scenario 0 leaves; 1 -> 0, the new one -> 1
    for _ in range(3):
        B.step(0.02)
        ref[1].step(0.02)
        ref[2].step(0.02)
    for f in ("p", "T", "u", "Yf"):
        assert np.array_equal(B.get(0, f), ref[1].get(f)), f
        assert np.array_equal(B.get(1, f), ref[2].get(f)), f


@pytest.mark.parametrize("precision", [_lib.PREC_FP64, _lib.PREC_MIXED])
def test_batch_equals_alone_with_many_tiles_per_cta(precision, monkeypatch):
    """Persistent grids capped at 3 CTAs: each CTA walks tiles of several
    scenarios of different row lengths and plane counts in turn, so every
    staging slot is reused across scenarios."""
    monkeypatch.setenv("PHX_PERSIST_CTAS", "3")
    cs = cases() + [casegen.house(30, 22, 34, 0.2, 5)]
    cs[-1].profile.tol = 0.0
    cs[-1].profile.rel_tol = 1e-8
    B = Batch(cs, precision)
    alone = [Solver(c, precision) for c in cs]
    for step in range(6):
        dts = B.step(0.02)
        for s, g in enumerate(alone):
            assert g.step(0.02) == dts[s]
    for s, g in enumerate(alone):
        for f in STATE:
            a, b = B.get(s, f), g.get(f)
            assert np.array_equal(a, b), (precision, s, f, float(np.max(np.abs(a - b))))
        assert B.stats(s)["pressure_iters"] == g.stats()["pressure_iters"]
        assert B.stats(s)["pressure_rel_residual"] <= 1e-8


@pytest.mark.parametrize("precision", [_lib.PREC_FP64, _lib.PREC_MIXED])
def test_bounded_wait_timeout_is_reported_and_context_stays_usable(precision):
    """One bounded device wait runs out on purpose (an mbarrier nothing arrives
    on, 20 ms limit): the call reports PHX_ERR_TIMEOUT, the error word is
    cleared, and the same context then steps exactly like a fresh one."""
    c = cases()[0]
    g, ref = Solver(c, precision), Solver(c, precision)
    g.step(0.02)
    ref.step(0.02)
    with pytest.raises(PhxError) as e:
        g.selftest_wait_timeout(20.0)
    assert e.value.code == _lib.PHX_ERR_TIMEOUT
    assert "ran out" in str(e.value)
    g.sync()                                   # the word was cleared: no error left
    for _ in range(3):
        assert g.step(0.02) == ref.step(0.02)
    for f in STATE:
        assert np.array_equal(g.get(f), ref.get(f)), f
