"""Pin the oracle's radiation trace (orc_rad_trace in oracle/phx_oracle.c)
against the reference's own Solver::traceRadiation (src/sim/radiation.cpp:
181-319), recorded in tests/golden/rad_sofa_room.npz by
tests/golden/make_rad_golden.py from the reference built at FP64: a hot NIST
sofa room with walls, solid and porous fuel elements and flame cells."""
import os

import numpy as np
import pytest

from oracle import oraclepy

HERE = os.path.dirname(os.path.abspath(__file__))
FIXTURE = os.path.join(HERE, "golden", "rad_sofa_room.npz")


def load_fixture():
    z = np.load(FIXTURE)
    return {k: z[k] for k in z.files}


def oracle_trace(fx, **over):
    a = dict(fx, **over)
    gas = {f: a[f].astype(np.float64) for f in oraclepy.RAD_GAS_FIELDS}
    return oraclepy.rad_trace(a["dims"], a["geo"], a["blocked"], gas, a["elements"], a["walls"], a["solidT"])


def test_fixture_covers_every_branch():
    fx = load_fixture()
    el = fx["elements"]
    assert len(el) > 1000 and len(fx["walls"]) > 500
    assert (el[:, 9] == 1).any() and (el[:, 9] == 0).any()     # porous (sphere) and surface elements
    assert (el[:, 10] == 1).any()                              # porous fuel skips its own cell
    assert fx["hrr"].max() > 0 and fx["T"].max() > 1000         # flame cells
    assert fx["blocked"].any() and (fx["solidT"][fx["blocked"] == 1] > 293.2).any()
    assert (fx["radGas"] > 0).any() and (fx["radGas"] < 0).any()


def test_oracle_matches_reference_trace():
    fx = load_fixture()
    ab, gas = oracle_trace(fx)
    np.testing.assert_array_equal(ab, fx["radAbs"])
    np.testing.assert_array_equal(gas, fx["radGas"])


def test_oracle_cold_room_exchanges_nothing():
    """Everything at ambient: no element absorbs, no cell gains (the trace is
    written relative to ambient, src/sim/radiation.cpp:24-25)."""
    fx = load_fixture()
    n = fx["T"].size
    el = fx["elements"].copy()
    el[:, 8] = 293.15
    wl = fx["walls"].copy()
    wl[:, 2:] = 293.15
    ab, gas = oracle_trace(fx, T=np.full(n, 293.15), hrr=np.zeros(n), elements=el, walls=wl,
                           solidT=np.full(n, 293.15))
    assert np.abs(ab).max() < 1e-9 and np.abs(gas).max() < 1e-9
