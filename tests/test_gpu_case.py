"""GPU-backed case runs (photon_gb300.case.run_case): the loop of
`photon_cli --case` (src/app/cli_case.cpp:205-248) with the GPU stepping and
the reference's own Solver (the FP64 build, oracle/_ref) as the host that
samples the devices (photon::sampleDevice) and writes the checkpoints
(Solver::saveState).

- The GPU run lands on the same output times as the same loop run with the
  reference stepping on the CPU, and its device rows agree within 1e-7
  relative (both FP64; the per-step parity bar is 1e-9).
- The checkpoints are the host's own files: resuming the GPU from one gives
  the rows of the uninterrupted run (within 1e-9), as the reference's
  resume_matches_uninterrupted test requires of the CPU solver
  (src/tests/test_main.cpp:519-546)."""
import os

import numpy as np
import pytest

from oracle import refpy
from photon_gb300 import casegen
from photon_gb300.case import CaseSchedule, Device, run_case
from photon_gb300.solver import Solver

pytestmark = [pytest.mark.gpu, pytest.mark.skipif(not refpy.available(64), reason="reference FP64 build not present")]


class RefStepper:
    """The reference's Solver driven by the same loop (its own state is the host's)."""

    def __init__(self, ref):
        self.ref = ref

    def step(self, dt_max):
        return self.ref.step(dt_max)

    def stats(self):
        st = self.ref.stats()
        sc = self.ref.scalars()
        st.update(pressure_iters=int(sc["pressureIters"]), pressure_residual=sc["pressureResidual"],
                  zones=int(sc["nZones"]), leak_faces=int(sc["leakFaces"]))
        return st

    def export_state(self, host):
        assert host is self.ref

    def import_state(self, host):
        assert host is self.ref


def room():
    return casegen.tiny_room(12, 10, 9, 0.2, 60e3)


DEVICES = [Device("temp", "T_plume", 1.3, 1.1, 1.2), Device("temp", "T_ceiling", 1.9, 1.5, 1.7),
           Device("u", "U_door", 0.0, 1.0, 0.5), Device("o2", "O2_plume", 1.3, 1.1, 0.9),
           Device("co2", "CO2_upper", 0.5, 0.5, 1.6), Device("pressure", "P_floor", 1.0, 1.0, 0.1)]


def test_gpu_case_rows_match_reference_loop(tmp_path):
    c = room()
    sched = CaseSchedule(duration=0.6, output_interval=0.2, checkpoint=0.4, prefix=str(tmp_path / "gpu"))
    host = refpy.RefSolver(c, 64, 2)
    g = run_case(Solver(c), host, sched, DEVICES)
    ref = refpy.RefSolver(c, 64, 2)
    r = run_case(RefStepper(ref), ref, CaseSchedule(0.6, 0.2, 0.4, str(tmp_path / "ref")), DEVICES)
    assert len(g.rows) == len(r.rows) == 4
    # one checkpoint, at 0.4 s, named as the reference names it (std::lround of the time)
    assert len(g.checkpoints) == 1 and os.path.exists(g.checkpoints[0]) and g.checkpoints[0].endswith("gpu_0s.state")
    for a, b in zip(g.rows, r.rows):
        assert abs(a[0] - b[0]) <= 1e-6, (a[0], b[0])
        da, db = np.array(a[1:1 + len(DEVICES)]), np.array(b[1:1 + len(DEVICES)])
        assert np.all(np.abs(da - db) <= 1e-7 * np.maximum(np.abs(db), 1e-3)), (da, db)
    assert g.rows[-1][1 + len(DEVICES)] > 10.0    # the burner burns (HRR in kW)
    assert g.rows[-1][1] > 20.0                   # and the plume probe (deg C) has warmed


def test_gpu_case_resumes_from_host_checkpoint(tmp_path):
    c = room()
    full = run_case(Solver(c), refpy.RefSolver(c, 64, 2), CaseSchedule(0.6, 0.2, 0.4, str(tmp_path / "a")), DEVICES)
    ck = full.checkpoints[0]
    part = run_case(Solver(c), refpy.RefSolver(c, 64, 2), CaseSchedule(0.6, 0.2, 0.0, str(tmp_path / "b")), DEVICES,
                    resume_from=ck)
    assert len(part.rows) == 1 and abs(part.rows[0][0] - full.rows[-1][0]) <= 1e-6
    a, b = np.array(part.rows[0][1:1 + len(DEVICES)]), np.array(full.rows[-1][1:1 + len(DEVICES)])
    assert np.all(np.abs(a - b) <= 1e-9 * np.maximum(np.abs(b), 1e-3)), (a, b)
