"""The mixed path's exact coarsest solve: phx::coarseInverse (dense blocked
Cholesky, photon_gb300/csrc/host_setup.cpp) compiled on the host with the
checks of tests/cpp/coarse_inverse.cpp (A inv = I within 1e-12 on random
definite levels up to 1700 unknowns, symmetry, rows without a diagonal,
failure on a singular level). No GPU needed."""
import os
import subprocess

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_coarse_inverse(tmp_path):
    exe = str(tmp_path / "coarse_inverse")
    csrc = os.path.join(ROOT, "photon_gb300", "csrc")
    subprocess.run(["g++", "-std=c++17", "-O2", "-pthread", "-I" + csrc, "-I" + os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "cpp", "coarse_inverse.cpp"), os.path.join(csrc, "host_setup.cpp"),
                    "-o", exe], check=True)
    out = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stdout + out.stderr
    assert out.stdout.strip().endswith("ok")
