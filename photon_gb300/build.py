"""Build libphx.so (the C-ABI library with the sm_103a kernels) in-tree.

    python -m photon_gb300.build [--verbose]

Compiles each translation unit with nvcc for sm_103a only, in parallel, and
links photon_gb300/_build/libphx.so (CUDA runtime linked statically).
"""
from __future__ import annotations

import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libphx.so")
NVCC = os.environ.get("NVCC", "/usr/local/cuda/bin/nvcc" if os.path.exists("/usr/local/cuda/bin/nvcc") else "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-I" + os.path.join(ROOT, "include"), "-I" + CSRC]

# translation unit -> extra flags. The FP64 path keeps every multiply and add
# separate (--fmad=false) so its rounding follows the reference's arithmetic.
UNITS = {
    "engine_fp64.cu": ["--fmad=false"],
    "engine_mixed.cu": [],
    "host_setup.cpp": [],
    "api.cpp": [],
    "noalloc.cu": ["--fmad=false"],
    "server.cpp": [],
}
HEADERS = ["phx_dev.cuh", "step_kernels.cuh", "pressure_kernels.cuh", "engine.cuh", "engine.h", "host_setup.h",
           "mixed_kernels.cuh", "rowblock.cuh", "level0.cuh", "fdiv.cuh", "radiation.cuh", "volume.cuh"]


def _newer(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.exists(d) and os.path.getmtime(d) > t for d in deps)


def build(verbose: bool = False, force: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    hdrs = [os.path.join(CSRC, h) for h in HEADERS] + [os.path.join(ROOT, "include", "phx.h")]

    def one(unit):
        src = os.path.join(CSRC, unit)
        obj = os.path.join(BUILD, unit + ".o")
        if not force and not _newer(obj, [src, __file__] + hdrs):
            return obj
        cmd = [NVCC] + ARCH + COMMON + UNITS[unit] + ["-c", src, "-o", obj + ".tmp"]
        if verbose and unit.endswith(".cu"):
            cmd += ["-Xptxas", "-v"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (unit, " ".join(cmd), r.stderr[-6000:]))
        if verbose:
            sys.stderr.write(r.stderr)
        os.replace(obj + ".tmp", obj)
        return obj

    with ThreadPoolExecutor(max_workers=len(UNITS)) as ex:
        objs = list(ex.map(one, list(UNITS)))
    if force or _newer(LIB, objs):
        tmp = LIB + ".tmp%d" % os.getpid()
        cmd = [NVCC] + ARCH + ["-shared", "-o", tmp] + objs + ["-Xcompiler", "-pthread", "-lpthread"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed:\n%s\n%s" % (" ".join(cmd), r.stderr[-4000:]))
        os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(verbose="--verbose" in sys.argv, force="--force" in sys.argv))
