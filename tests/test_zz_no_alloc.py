"""phx_gather_stats_noalloc: gatherStats' sums recomputed with the reduction
scratch in a file-scope device array (no device allocation). Two calls in a
row must agree with the stats the step itself gathered (phx_batch_get_stats),
for both precisions and for every scenario of a batch; a scenario above the
scratch's size limit is refused with a clear message. This file is collected
last so that it also runs after every other GPU test in the same process."""
import ctypes

import pytest

from photon_gb300 import _lib, casegen
from photon_gb300.solver import Batch

pytestmark = pytest.mark.gpu

# the sums use the same tiling and reduction order as the step's gatherStats:
# they agree to rounding (in practice bit for bit)
REL = 1e-12


def _noalloc(B, s):
    st = _lib.PhxStats()
    r = B.L.phx_gather_stats_noalloc(B.h, s, ctypes.byref(st))
    assert r == 0, B.L.phx_last_error(B.h).decode()
    return st


def _close(a, b):
    return abs(a - b) <= REL * max(abs(a), abs(b), 1e-300)


@pytest.mark.parametrize("precision", [_lib.PREC_FP64, _lib.PREC_MIXED])
def test_noalloc_stats_match_step_stats_twice(precision):
    cases = [casegen.tiny_room(12, 10, 9, 0.2, 60e3), casegen.house(24, 20, 14, 0.2, 3)]
    B = Batch(cases, precision)
    for _ in range(6):
        B.step(0.02)
    B.sync()
    for s in range(len(cases)):
        ref = B.stats(s)
        assert ref["hrr"] > 0
        for _ in range(2):        # two calls in a row: the scratch is left ready for the next call
            st = _noalloc(B, s)
            assert _close(st.hrr, ref["hrr"]), (st.hrr, ref["hrr"])
            assert _close(st.fuel_in_domain, ref["fuel_in_domain"]), (st.fuel_in_domain, ref["fuel_in_domain"])
            assert _close(st.max_gas_t, ref["max_gas_t"]), (st.max_gas_t, ref["max_gas_t"])
            assert st.burning_cells == ref["burning_cells"]
            # the members the call does not compute are zero
            for name in ("time", "dt", "max_vel", "max_nu", "max_div", "pressure_iters", "pressure_residual",
                         "pressure_rel_residual", "fuel_in", "fuel_burned", "zones", "leak_faces"):
                assert getattr(st, name) == 0, name
        # the context's own stats are left as the step gathered them
        assert B.stats(s) == ref
    B.close()


def test_noalloc_refuses_unstepped_context_and_bad_scenario():
    B = Batch([casegen.tiny_room(10, 8, 8, 0.2, 40e3)], _lib.PREC_FP64)
    st = _lib.PhxStats()
    assert B.L.phx_gather_stats_noalloc(B.h, 0, ctypes.byref(st)) == 7          # PHX_ERR_STATE: not stepped yet
    assert b"step the context" in B.L.phx_last_error(B.h)
    B.step(0.02)
    assert B.L.phx_gather_stats_noalloc(B.h, 5, ctypes.byref(st)) != 0          # no such scenario
    assert B.L.phx_gather_stats_noalloc(B.h, 0, ctypes.byref(st)) == 0
    B.close()


def test_noalloc_refuses_scenario_above_limit():
    c = casegen.tiny_room(256, 128, 129, 0.2, 60e3)   # 4,227,072 cells > 4,194,304
    B = Batch([c], _lib.PREC_MIXED)
    B.step(0.02)
    st = _lib.PhxStats()
    assert B.L.phx_gather_stats_noalloc(B.h, 0, ctypes.byref(st)) == 1          # PHX_ERR_INVALID
    assert b"at most 4194304" in B.L.phx_last_error(B.h)
    B.close()
