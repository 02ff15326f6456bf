"""The C++ adapter (include/photon_gpu/solver.hpp) compiles against the C ABI,
and a Photon-style C++ caller runs on the GPU with the oracle's results: its
FP64 fields after 40 steps match the oracle's run of the same room within the
parity bar (1e-9 relative L2 read through the C ABI in double; the adapter's
own float vectors within the rounding of FP32, 1e-7)."""
import os
import subprocess
import tempfile

import numpy as np
import pytest

from photon_gb300 import build, casegen

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "cpp", "adapter_room.cpp")
EXE = os.path.join(ROOT, "photon_gb300", "_build", "adapter_room")


def compile_adapter():
    lib = build.build()
    cmd = ["g++", "-std=c++17", "-O2", "-I" + os.path.join(ROOT, "include"), SRC, "-o", EXE,
           "-L" + os.path.dirname(lib), "-lphx", "-Wl,-rpath," + os.path.dirname(lib)]
    subprocess.run(cmd, check=True)
    return EXE


def test_adapter_compiles_and_links():
    assert os.path.exists(compile_adapter())


@pytest.mark.gpu
@pytest.mark.parametrize("mode", ["fp64", "mixed"])
def test_adapter_runs_room(mode):
    exe = compile_adapter()
    out = subprocess.run([exe, mode], capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stdout + out.stderr
    vals = dict(zip(out.stdout.split()[0::2], out.stdout.split()[1::2]))
    assert float(vals["time"]) > 0.5
    assert float(vals["fuelIn"]) > 0
    assert float(vals["maxT"]) > 400          # the burner heats the room
    assert float(vals["hrr"]) > 10e3          # and burns
    assert int(vals["cells"]) == 18 * 12 * 12


def adapter_room_case():
    """The room tests/cpp/adapter_room.cpp builds through the adapter, with its
    float settings rounded exactly as the adapter passes them on"""
    f = lambda v: float(np.float32(v))
    nx, ny, nz = 18, 12, 12
    blocked = np.zeros((nz, ny, nx), np.uint8)
    fx, fy, fz = casegen.faces_from_blocked(blocked)
    fx[:, :, 0] = 0
    fx[:10, 4:8, 0] = 1.0        # doorway: j 4..7, k 0..9
    fx[:, :, nx] = 0
    fy[:, 0, :] = 0
    fy[:, ny, :] = 0
    fz[nz] = 0
    prof = casegen.Profile(f(0.8), f(0.05), 80, f(0.02), 0.0)
    burners = [casegen.Burner(f(2.4), f(1.0), f(2.8), f(1.4), 0.0, 100e3, 0.0, 0.0, 1e9)]
    c = casegen._finish("adapter_room", blocked, fx, fy, fz, f(0.2), (0.0, 0.0, 0.0), burners, prof, 10.0, 0,
                        radiationOn=False)
    c.adiabatic = True
    return c


@pytest.mark.gpu
def test_adapter_fields_match_oracle():
    from oracle.oraclepy import OracleSolver
    exe = compile_adapter()
    with tempfile.TemporaryDirectory() as d:
        prefix = os.path.join(d, "room")
        out = subprocess.run([exe, "fp64", "dump", prefix], capture_output=True, text=True, timeout=300)
        assert out.returncode == 0, out.stdout + out.stderr
        c = adapter_room_case()
        o = OracleSolver(c)
        for _ in range(40):
            o.step(float(np.float32(0.05)))
        for name in ("u", "v", "w", "p", "T", "Yo", "Yf", "Ys", "nu"):
            ref = o.get(name)
            nb = np.linalg.norm(ref)
            d64 = np.fromfile(prefix + "_" + name + ".f64", np.float64)
            d32 = np.fromfile(prefix + "_" + name + ".f32", np.float32).astype(np.float64)
            assert d64.shape == ref.shape and d32.shape == ref.shape, name
            assert np.linalg.norm(d64 - ref) <= 1e-9 * nb, (name, np.linalg.norm(d64 - ref) / nb)
            assert np.linalg.norm(d32 - ref) <= 1e-7 * nb, (name, np.linalg.norm(d32 - ref) / nb)


@pytest.mark.gpu
@pytest.mark.parametrize("mode", ["fp64", "mixed"])
def test_adapter_checkpoint_round_trip(mode):
    """exportTo / importFrom through a host object shaped like photon::Solver:
    the fields arrive unchanged, and the resumed solver tracks the original
    (the host holds FP32 fields, as the reference does, so the FP64 state is
    rounded once on the way)."""
    exe = compile_adapter()
    out = subprocess.run([exe, mode, "checkpoint"], capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stdout + out.stderr
    vals = dict(zip(out.stdout.split()[0::2], out.stdout.split()[1::2]))
    assert int(vals["ckpt_same"]) == 1
    assert float(vals["ckpt_dtime"]) < 1e-5
    assert float(vals["ckpt_maxrel"]) < 1e-3


@pytest.mark.gpu
def test_adapter_case_loop_lands_on_output_times():
    """photon_gpu::runCase (include/photon_gpu/case_loop.hpp): rows at 0, 0.5,
    1, 1.5 and 2 s exactly (in the float time of photon::Solver), and one
    checkpoint at 1 s and one at 2 s, written by the host's saveState."""
    exe = compile_adapter()
    with tempfile.TemporaryDirectory() as d:
        prefix = os.path.join(d, "room")
        out = subprocess.run([exe, "fp64", "case", prefix], capture_output=True, text=True, timeout=300)
        assert out.returncode == 0, out.stdout + out.stderr
        times = [float(l.split()[1]) for l in out.stdout.splitlines() if l.startswith("row ")]
        assert len(times) == 5, out.stdout
        for t, want in zip(times, (0.0, 0.5, 1.0, 1.5, 2.0)):
            assert abs(t - want) <= 1e-6, (t, want)
        assert sorted(os.listdir(d)) == ["room_1s.state", "room_2s.state"]
