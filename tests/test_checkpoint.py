"""Checkpoint interop: the gas-phase state moves between the GPU step and the
reference's own save/load (Solver::saveState / Solver::loadState,
src/sim/state.cpp:62-195) without loss, and a run resumed on either side from
a checkpoint written by the other continues as the uninterrupted run does.

The host solver is the reference built at FP64 (oracle/_ref/libphoton_ref64.so),
so FP64 GPU fields pass through the reference's file unrounded. Skipped where
that build is absent."""
import numpy as np
import pytest

from oracle import refpy
from photon_gb300 import casegen
from photon_gb300.solver import CHECKPOINT_FIELDS, PhxError, Solver

from gpu_util import rel_l2

pytestmark = pytest.mark.skipif(not refpy.available(64), reason="reference FP64 build not present")

RESUME_TOL = 1e-9
COMPARED = ("u", "v", "w", "p", "T", "Yo", "Yf", "Ys", "Yc", "Yw", "Yco", "Pb", "hrr", "zoneP")


def _cases():
    return {"room": casegen.tiny_room(12, 10, 9, 0.2, 60e3),
            "sealed": casegen.tiny_room(10, 8, 7, 0.2, 50e3, doorway=False)}


def test_reference_save_load_round_trip(tmp_path):
    """The reference's own round trip through the harness (host side only): a
    loaded solver continues bit for bit as the saved one does."""
    c = _cases()["room"]
    a = refpy.RefSolver(c, 64, 2)
    for _ in range(4):
        a.step(0.02)
    path = str(tmp_path / "a.state")
    a.save_state(path)
    b = refpy.RefSolver(c, 64, 2)
    b.load_state(path)
    for f in CHECKPOINT_FIELDS:
        assert np.array_equal(a.get(f), b.get(f)), f
    # maxDiv is not part of the file (src/sim/state.cpp:81 writes maxVel and
    # maxNu only): the loading solver keeps its own
    sa, sb = a.stats(), b.stats()
    sa.pop("max_div"), sb.pop("max_div")
    assert sa == sb
    for _ in range(2):
        assert a.step(0.02) == b.step(0.02)
    for f in CHECKPOINT_FIELDS:
        assert np.array_equal(a.get(f), b.get(f)), f


def test_reference_refuses_other_grid(tmp_path):
    """loadState refuses a state of another grid with its message
    (src/sim/state.cpp:148-149)."""
    a = refpy.RefSolver(_cases()["room"], 64, 2)
    a.step(0.02)
    path = str(tmp_path / "a.state")
    a.save_state(path)
    b = refpy.RefSolver(casegen.tiny_room(11, 10, 9, 0.2, 60e3), 64, 2)
    with pytest.raises(RuntimeError, match="grid"):
        b.load_state(path)


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["room", "sealed"])
def test_gpu_state_resumes_in_reference(name, tmp_path):
    """GPU run -> export into a host solver -> its saveState -> a fresh host
    solver's loadState: the fields arrive unchanged, and the reference resumed
    from that file tracks the GPU run within the step tolerance."""
    c = _cases()[name]
    g = Solver(c)
    for _ in range(5):
        g.step(0.02)
    host = refpy.RefSolver(c, 64, 2)
    host.compute_zones()
    g.export_state(host)
    path = str(tmp_path / "gpu.state")
    host.save_state(path)
    r = refpy.RefSolver(c, 64, 2)
    r.load_state(path)
    for f in CHECKPOINT_FIELDS:
        assert np.array_equal(r.get(f), g.get(f).astype(r.get(f).dtype)), f
    st_g, st_r = g.stats(), r.stats()
    for k in ("time", "fuel_in", "fuel_burned"):
        assert st_r[k] == pytest.approx(st_g[k], rel=1e-15, abs=0), k
    for s in range(3):
        dtr, dtg = r.step(0.02), g.step(0.02)
        assert abs(dtr - dtg) <= 1e-12
        bad = {f: e for f in COMPARED if not (e := rel_l2(g.get(f), r.get(f))) <= RESUME_TOL}
        assert not bad, "step %d after resume: %s" % (s, bad)


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["room", "sealed"])
def test_reference_checkpoint_resumes_on_gpu(name, tmp_path):
    """Reference run -> saveState -> loadState into a host solver -> import
    into a fresh GPU solver: the GPU continues as the host resumed from the
    same file does, and as the uninterrupted reference run does."""
    c = _cases()[name]
    a = refpy.RefSolver(c, 64, 2)
    for _ in range(5):
        a.step(0.02)
    path = str(tmp_path / "ref.state")
    a.save_state(path)
    host = refpy.RefSolver(c, 64, 2)
    host.load_state(path)
    g = Solver(c)
    g.import_state(host)
    for f in CHECKPOINT_FIELDS:
        assert np.array_equal(g.get(f), host.get(f).astype(g.get(f).dtype)), f
    for s in range(3):
        dta, dth, dtg = a.step(0.02), host.step(0.02), g.step(0.02)
        assert abs(dth - dtg) <= 1e-12 and abs(dta - dtg) <= 1e-12
        for ref in (host, a):
            bad = {f: e for f in COMPARED if not (e := rel_l2(g.get(f), ref.get(f))) <= RESUME_TOL}
            assert not bad, "step %d after resume: %s" % (s, bad)
    assert g.stats()["fuel_in"] == pytest.approx(a.stats()["fuel_in"], rel=1e-12)


@pytest.mark.gpu
def test_gpu_refuses_state_of_other_zones(tmp_path):
    """A host state with another zone count is refused before any field moves."""
    sealed = refpy.RefSolver(_cases()["sealed"], 64, 2)
    sealed.step(0.02)
    g = Solver(_cases()["room"])
    with pytest.raises(PhxError):
        g.import_state(sealed)


@pytest.mark.gpu
def test_reference_devices_read_gpu_state():
    """The reference's own device probes (photon::sampleDevice,
    src/sim/devices.h) on a host solver holding the GPU's exported state read
    what they read on the reference's own run of the same case (FP64 builds,
    8 steps): thermocouples, velocities, gas fractions, soot, pressure and the
    two-zone layer reduction."""
    c = _cases()["room"]
    g = Solver(c)
    r = refpy.RefSolver(c, 64, 2)
    for _ in range(8):
        g.step(0.02)
        r.step(0.02)
    host = refpy.RefSolver(c, 64, 2)
    host.compute_zones()
    g.export_state(host)
    x, y = c.ox + 0.45 * c.nx * c.dx, c.oy + 0.5 * c.ny * c.dx
    probes = [(k, x, y, z, 0.0, 0.0) for k in ("Temperature", "VelU", "VelV", "VelW", "O2", "CO2", "CO", "Soot",
                                                "Pressure") for z in (0.3, 0.9, 1.5)]
    probes += [(k, x, y, 0.0, 0.0, c.nz * c.dx) for k in ("LayerHeight", "UpperTemp", "LowerTemp")]
    for kind, px, py, pz, z0, z1 in probes:
        a, b = host.sample_device(kind, px, py, pz, z0, z1), r.sample_device(kind, px, py, pz, z0, z1)
        assert abs(a - b) <= 1e-7 * max(1.0, abs(b)), (kind, pz, a, b)
