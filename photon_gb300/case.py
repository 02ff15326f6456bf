"""GPU-backed case runs: the stepping loop of `photon_cli --case` over the GPU
solver, with the host solver's own device probes and checkpoints.

The reference's case runner (src/app/cli_case.cpp:205-248) steps a
photon::Solver to a duration, landing steps exactly on output and checkpoint
times so that a resumed run samples the same instants; at every output time it
writes a row of device readings (photon::sampleDevice, src/sim/devices.h:65-96)
and of stats, and at every checkpoint time it writes the state with
Solver::saveState (src/sim/state.cpp:62-121). `run_case` runs the same loop
with the GPU solver stepping: at each output or checkpoint time the gas-phase
state moves to a host solver (the reference's own Solver, or anything with its
get/set, sample_device and save_state), whose probes and saveState do the
rest. A run resumes from a checkpoint the host loaded (`resume_from`).

Times follow the reference's float arithmetic (Solver::time is a float there).
"""
from __future__ import annotations

import math
import os
from dataclasses import dataclass, field

import numpy as np

f32 = np.float32

# photon_cli case-file device names -> photon::DeviceKind (src/app/cli_case.cpp:90-93)
DEVICE_KINDS = {"temp": "Temperature", "u": "VelU", "v": "VelV", "w": "VelW", "o2": "O2", "co2": "CO2",
                "co": "CO", "soot": "Soot", "pressure": "Pressure"}


@dataclass
class Device:
    """photon::Device (src/sim/devices.h:14-22): a probe at (x, y, z), or a
    layer measurement between z0 and z1 for the layer kinds."""
    kind: str
    id: str
    x: float
    y: float
    z: float = 0.0
    z0: float = 0.0
    z1: float = 0.0


@dataclass
class CaseSchedule:
    duration: float = 60.0           # s simulated
    output_interval: float = 1.0     # s between rows
    checkpoint: float = 0.0          # s between checkpoints (0: none)
    prefix: str = "case"             # checkpoint files: <prefix>_<t>s.state


@dataclass
class CaseResult:
    header: list = field(default_factory=list)
    rows: list = field(default_factory=list)       # one list per output time
    checkpoints: list = field(default_factory=list)
    steps: int = 0


HRR_COLUMNS = ["Time", "HRR_kW", "MaxGas_C", "MaxVel", "PressureIters", "PressureResidual", "Zones", "LeakFaces"]


def run_case(gpu, host, schedule: CaseSchedule, devices=(), resume_from: str | None = None) -> CaseResult:
    """Step `gpu` (photon_gb300.solver.Solver) through the case. `host` is the
    reference's Solver built on the same grid (oracle.refpy.RefSolver or a
    photon::Solver behind any binding with get/set, set_stats, sample_device,
    save_state, load_state). With `resume_from`, the host loads that
    checkpoint and the GPU continues from it; rows then start after it, as in
    the reference (src/app/cli_case.cpp:152-154, 228-233)."""
    res = CaseResult(header=["Time"] + [d.id for d in devices] + HRR_COLUMNS[1:])
    if resume_from:
        host.load_state(resume_from)
        gpu.import_state(host)
    out_dt, dur, ck = f32(schedule.output_interval), f32(schedule.duration), f32(schedule.checkpoint)

    def now():
        return f32(gpu.stats()["time"])

    def row():
        gpu.export_state(host)
        st = gpu.stats()
        t = f32(st["time"])
        vals = [float(t)] + [host.sample_device(DEVICE_KINDS.get(d.kind, d.kind), d.x, d.y, d.z, d.z0, d.z1)
                             for d in devices]
        vals += [st["hrr"] / 1000.0, st["max_gas_t"] - 273.15, st["max_vel"], st["pressure_iters"],
                 st["pressure_residual"], st["zones"], st["leak_faces"]]
        res.rows.append(vals)

    t = now()
    resumed = resume_from is not None
    next_out = f32(math.floor(t / out_dt + 0.5) * out_dt + out_dt) if resumed else f32(0.0)
    next_ck = f32(math.floor(t / ck + 0.5) * ck + ck) if ck > 0 else f32(1e30)
    if not resumed:
        row()
        next_out = out_dt
    while t < dur - f32(1e-5):
        # land exactly on output and checkpoint times (src/app/cli_case.cpp:238-240)
        target = min(next_out, dur, next_ck)
        gpu.step(float(max(f32(1e-4), f32(target - t))))
        res.steps += 1
        t = now()
        if t >= next_out - f32(1e-5):
            row()
            next_out = f32(next_out + out_dt)
        if t >= next_ck - f32(1e-5):
            path = "%s_%ds.state" % (schedule.prefix, int(round(float(t))))
            gpu.export_state(host)
            host.save_state(path)
            res.checkpoints.append(path)
            next_ck = f32(next_ck + ck)
    return res


def write_csv(res: CaseResult, path: str, append: bool = False):
    """The rows as the reference's _devc / _hrr CSV pair would hold them, in one file."""
    mode = "a" if append and os.path.exists(path) else "w"
    with open(path, mode) as f:
        if mode == "w":
            f.write(",".join(res.header) + "\n")
        for r in res.rows:
            f.write(",".join(repr(float(v)) for v in r) + "\n")
