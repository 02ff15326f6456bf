"""Generate the radiation-trace golden fixture tests/golden/rad_sofa_room.npz from
the reference's own solver.

The reference's FP64 build (oracle/_ref/libphoton_ref64.so, made by
oracle/make_ref.py) loads the reference's NIST sofa-room scene with radiation on
and non-adiabatic surfaces, a 400 kW gas burner in the middle of the floor, and runs
150 steps so that gas, walls and fuel are hot. The fixture then holds the
inputs of Solver::traceRadiation (src/sim/radiation.cpp:181-319) in the flat
form the GPU trace takes -- the gas fields it reads, the radiating elements
with emissivity and temperature, the intact barriers as walls, the solid
temperatures -- and the reference's outputs radAbs (per element) and radGas
(per cell) for those inputs.

Usage: python tests/golden/make_rad_golden.py   (needs oracle/_ref built and
the reference checkout, located as oracle/make_ref.py locates it)
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import make_ref  # noqa: E402
from oracle.refpy import RefSolver  # noqa: E402

GAS = ("T", "Ys", "Yw", "Yc", "Pb", "hrr")


def generate(path: str, steps: int = 150) -> dict:
    r = RefSolver(None, 64, 8)
    r.load_scene(os.path.join(make_ref.REF, "data"), os.path.join(make_ref.REF, "scenes", "nist_sofa_room.txt"),
                 reference_profile=False, radiation=True, adiabatic=False, no_leak=True)
    (nx, ny, nz, n), (dx, ox, oy, oz) = r.grid()
    # 0.6 m square burner on the floor in the middle of the room (the first gas
    # layer above the raised floor is at z = 0.3 m)
    cx, cy = ox + 0.5 * nx * dx, oy + 0.5 * ny * dx
    if r.L.ref_add_burner(r.h, cx - 0.3, cy - 0.3, cx + 0.3, cy + 0.3, 0.3, 400e3, 5.0, 0.0, 1e9) < 0:
        raise RuntimeError("burner covers no gas cell")
    for _ in range(steps):
        r.step(0.05)
    # gas inputs rounded to FP32 (exact in the fixture at half the size)
    for f in GAS:
        r.set(f, r.get(f).astype(np.float32).astype(np.float64))
    inp = r.rad_inputs()
    rad_abs, rad_gas = r.rad_trace()
    out = {"dims": np.array([nx, ny, nz], np.int64), "geo": np.array([dx, ox, oy, oz], np.float64),
           "blocked": r.get("blocked")}
    for f in GAS:
        out[f] = r.get(f).astype(np.float32)
    out.update(inp)
    out["radAbs"] = rad_abs
    out["radGas"] = rad_gas
    out["time"] = np.array(r.scalars()["time"])
    np.savez_compressed(path, **out)
    return out


if __name__ == "__main__":
    p = os.path.join(HERE, "rad_sofa_room.npz")
    o = generate(p)
    print(p, os.path.getsize(p), "bytes;", len(o["elements"]), "elements,", len(o["walls"]), "walls, max T",
          o["T"].max(), "radGas range", o["radGas"].min(), o["radGas"].max())
