"""The C++ adapter (include/photon_gpu/solver.hpp) compiles against the C ABI,
and a Photon-style C++ caller runs on the GPU with the same results as the
Python binding (same library, same inputs)."""
import os
import subprocess

import pytest

from photon_gb300 import build

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
