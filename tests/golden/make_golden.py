"""Generate the golden fixtures in tests/golden/ from the reference's own solver.

The reference publishes no numeric goldens for the gas-phase step, so these
come from the reference itself: its src/ compiled at FP64 by oracle/make_ref.py
(oracle/_ref/libphoton_ref64.so), driven through oracle/ref_harness.cpp on
small synthetic cases. Each .npz holds the case geometry, the burners and
profile, and the solver fields and scalars after a few steps; the oracle tests
rebuild the case from the stored arrays and must reproduce every value bit for
bit.

Usage: python tests/golden/make_golden.py   (needs oracle/_ref built)
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from photon_gb300 import casegen  # noqa: E402
from oracle.refpy import RefSolver  # noqa: E402

OUT_FIELDS = ("u", "v", "w", "p", "S", "T", "Yo", "Yf", "Ys", "Ya", "Yp", "Yc", "Yw", "Yco", "Yai", "nu", "Pb", "Q",
              "hrr", "massSrc")
GEOM = ("blocked", "fx", "fy", "fz", "ax", "ay", "az", "lx", "ly", "lz")


def golden_cases():
    """Small cases covering every branch of the gas-only step."""
    cases = []
    c = casegen.tiny_room(12, 10, 9, 0.2, 60e3)
    c.name = "open_room"
    cases.append((c, 6, 0.02))
    c = casegen.tiny_room(10, 8, 8, 0.2, 40e3, doorway=False)
    c.name = "sealed_room"
    cases.append((c, 6, 0.02))
    c = casegen.house(24, 20, 14, 0.2, 3)
    c.wind = (5.0, 250.0, 0.25)
    c.name = "house_wind"
    cases.append((c, 4, 0.05))
    c = casegen.tiny_room(10, 8, 7, 0.2, 50e3, doorway=False)
    fx = c.fx.reshape(c.nz, c.ny, c.nx + 1)
    lx = c.lx.reshape(c.nz, c.ny, c.nx + 1)
    ax = c.ax.reshape(c.nz, c.ny, c.nx + 1)
    fx[1:4, 2:5, 0] = 0.01
    lx[1:4, 2:5, 0] = 1
    ax[1:4, 2:5, 0] = 0
    fx[:, :, 5] = 0.02
    lx[:, :, 5] = 1
    ax[:, :, 5] = 0
    c.name = "leaky_zones"
    cases.append((c, 6, 0.02))
    return cases


def main():
    for c, steps, dtMax in golden_cases():
        r = RefSolver(c, 64, 2)
        dts = [r.step(dtMax) for _ in range(steps)]
        sc = r.scalars()
        data = dict(nx=c.nx, ny=c.ny, nz=c.nz, dx=c.dx, origin=np.array([c.ox, c.oy, c.oz]),
                    profile=np.array([c.profile.cfl, c.profile.dtMax, c.profile.maxIters, c.profile.tol]),
                    switches=np.array([int(c.radiationOn), int(c.adiabatic)]), wind=np.array(c.wind),
                    burners=np.array([[b.x0, b.y0, b.x1, b.y1, b.z, b.peakW, b.rampS, b.start, b.duration]
                                      for b in c.burners]).reshape(-1, 9),
                    steps=steps, dtMax=dtMax, dts=np.array(dts),
                    scalars=np.array([sc[k] for k in sorted(sc)]), scalar_names=np.array(sorted(sc)))
        for g in GEOM:
            data["geom_" + g] = getattr(c, g)
        for f in OUT_FIELDS:
            data["out_" + f] = r.get(f)
        data["out_zone"] = r.get("zone")
        data["out_zoneP"] = r.get("zoneP")
        path = os.path.join(HERE, c.name + ".npz")
        np.savez_compressed(path, **data)
        print(path, os.path.getsize(path), "bytes", "iters", sc["pressureIters"], "zones", sc["nZones"])


if __name__ == "__main__":
    main()
