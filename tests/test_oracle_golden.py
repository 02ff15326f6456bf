"""The FP64 oracle (oracle/phx_oracle.c) reproduces the reference's own FP64
step bit for bit on the golden fixtures made by tests/golden/make_golden.py."""
import glob
import os

import numpy as np
import pytest

from oracle.oraclepy import OracleSolver
from photon_gb300 import casegen

# the step fixtures (rad_*.npz hold the radiation trace's, tests/test_oracle_rad.py)
GOLDEN = sorted(p for p in glob.glob(os.path.join(os.path.dirname(__file__), "golden", "*.npz"))
                if not os.path.basename(p).startswith("rad_"))


def case_from_golden(g):
    nx, ny, nz = int(g["nx"]), int(g["ny"]), int(g["nz"])
    pr = g["profile"]
    burners = [casegen.Burner(*map(float, b)) for b in g["burners"]]
    c = casegen.Case(name="golden", nx=nx, ny=ny, nz=nz, dx=float(g["dx"]), ox=float(g["origin"][0]),
                     oy=float(g["origin"][1]), oz=float(g["origin"][2]),
                     blocked=g["geom_blocked"], fx=g["geom_fx"], fy=g["geom_fy"], fz=g["geom_fz"],
                     ax=g["geom_ax"], ay=g["geom_ay"], az=g["geom_az"], lx=g["geom_lx"], ly=g["geom_ly"],
                     lz=g["geom_lz"], burners=burners,
                     profile=casegen.Profile(float(pr[0]), float(pr[1]), int(pr[2]), float(pr[3]), 0.0),
                     radiationOn=bool(g["switches"][0]), adiabatic=bool(g["switches"][1]),
                     wind=tuple(float(x) for x in g["wind"]))
    return c


@pytest.mark.parametrize("path", GOLDEN, ids=[os.path.basename(p)[:-4] for p in GOLDEN])
def test_oracle_matches_reference_golden(path):
    g = np.load(path)
    c = case_from_golden(g)
    o = OracleSolver(c)
    dts = [o.step(float(g["dtMax"])) for _ in range(int(g["steps"]))]
    assert np.array_equal(np.array(dts), g["dts"])
    for key in g.files:
        if not key.startswith("out_"):
            continue
        name = key[4:]
        got = o.get(name)
        assert np.array_equal(got, g[key]), "%s differs in %d places (max %g)" % (
            name, int(np.sum(got != g[key])), float(np.max(np.abs(got.astype(float) - g[key]))))
    sc = o.scalars()
    for name, val in zip(g["scalar_names"], g["scalars"]):
        assert sc[str(name)] == val, name


def test_golden_fixtures_present():
    assert len(GOLDEN) >= 4
