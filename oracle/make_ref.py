"""Build the reference's own CPU solver into oracle/_ref/ (test infrastructure).

Two shared libraries are made from the reference's unmodified `src/` files,
each linked with oracle/ref_harness.cpp:

* ``libphoton_ref32.so`` -- the reference as shipped (FP32 fields, FP64
  accumulators). It is the timed CPU baseline.
* ``libphoton_ref64.so`` -- the same sources made FP64 mechanically: the ``f``
  suffix is dropped from floating literals outside strings and comments, and a
  prelude maps ``float`` to ``double``. It pins the C restatement in
  oracle/phx_oracle.c.

Both builds also map ``private`` to ``public`` in the prelude so the harness can
fill geometry and call single stages. The reference sources are copied into
oracle/_ref/src32 and oracle/_ref/src64 (git-ignored build copies, never
committed) so the libraries can be rebuilt on a machine without the reference
checkout. Only this script reads the reference checkout: PHX_REFERENCE, or a
directory named "reference" beside this repository.

Usage: python oracle/make_ref.py [--jobs N]
"""
from __future__ import annotations

import argparse
import os
import platform
import re
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")
# the reference checkout: PHX_REFERENCE, else a directory named "reference" beside this repository
REF = os.environ.get("PHX_REFERENCE", os.path.join(os.path.dirname(os.path.dirname(HERE)), "reference"))

# the solver and the scene/material loaders it links against
SOURCES = [
    "sim/solver.cpp", "sim/gasphase.cpp", "sim/pressure_mg.cpp", "sim/discretize.cpp",
    "sim/radiation.cpp", "sim/state.cpp",
    "scene/materials.cpp", "scene/scene.cpp", "scene/objects.cpp", "scene/textfile.cpp",
]
HEADERS = ["core/jobs.h", "core/vmath.h", "scene/materials.h", "scene/scene.h", "scene/textfile.h",
           "sim/solver.h", "sim/devices.h", "sim/structure.h", "sim/fds_export.h"]

STD_HEADERS = """#include <algorithm>
#include <array>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <deque>
#include <fstream>
#include <functional>
#include <limits>
#include <map>
#include <memory>
#include <mutex>
#include <numeric>
#include <set>
#include <sstream>
#include <string>
#include <thread>
#include <unordered_map>
#include <utility>
#include <vector>
#if defined(__x86_64__) || defined(_M_X64)
#include <immintrin.h>
#endif
"""

# floating literal with an f/F suffix: 1.5f, 2.f, .5f, 1e-3f, 25.0e6f
_FLIT = re.compile(r"(?<![\w.])((?:\d+\.\d*|\.\d+)(?:[eE][+-]?\d+)?|\d+[eE][+-]?\d+)[fF](?![\w.])")


def strip_float_suffix(src: str) -> str:
    """Drop the f suffix of floating literals in code (not in strings, chars or comments)."""
    out = []
    i, n = 0, len(src)
    code_start = 0

    def flush(upto):
        out.append(_FLIT.sub(r"\1", src[code_start:upto]))

    while i < n:
        c = src[i]
        if c == '"' or c == "'":
            flush(i)
            q = c
            j = i + 1
            while j < n and src[j] != q:
                j += 2 if src[j] == "\\" else 1
            out.append(src[i:j + 1])
            i = j + 1
            code_start = i
        elif src.startswith("//", i):
            flush(i)
            j = src.find("\n", i)
            j = n if j < 0 else j
            out.append(src[i:j])
            i = j
            code_start = i
        elif src.startswith("/*", i):
            flush(i)
            j = src.find("*/", i + 2)
            j = n if j < 0 else j + 2
            out.append(src[i:j])
            i = j
            code_start = i
        else:
            i += 1
    flush(n)
    return "".join(out)


def copy_sources():
    for variant in ("src32", "src64"):
        for rel in SOURCES + HEADERS:
            src = os.path.join(REF, "src", rel)
            dst = os.path.join(OUT, variant, rel)
            os.makedirs(os.path.dirname(dst), exist_ok=True)
            with open(src, "r", encoding="utf-8") as f:
                text = f.read()
            if variant == "src64":
                text = strip_float_suffix(text)
            _write_if_changed(dst, text)
    _write_if_changed(os.path.join(OUT, "prelude32.h"), STD_HEADERS + "#define private public\n")
    _write_if_changed(os.path.join(OUT, "prelude64.h"), STD_HEADERS + "#define private public\n#define float double\n")


def _write_if_changed(path: str, text: str):
    # keep mtimes (and so the incremental compile) stable when nothing changed
    if os.path.exists(path):
        with open(path, "r", encoding="utf-8") as f:
            if f.read() == text:
                return
    with open(path, "w", encoding="utf-8") as f:
        f.write(text)


def compile_variant(variant: str, jobs: int) -> str:
    src_root = os.path.join(OUT, "src" + variant)
    obj_root = os.path.join(OUT, "obj" + variant)
    os.makedirs(obj_root, exist_ok=True)
    prelude = os.path.join(OUT, "prelude%s.h" % variant)
    flags = ["-std=c++20", "-fPIC", "-pthread", "-fno-math-errno", "-I" + src_root, "-include", prelude]
    if variant == "32":
        # the reference's own optimisation flags (CMakeLists.txt:16-18); the AVX2/FMA
        # switches exist on x86 only
        flags += ["-O3"] + (["-mavx2", "-mfma"] if platform.machine() in ("x86_64", "AMD64") else [])
    else:
        flags += ["-O2", "-ffp-contract=off"]
    units = [os.path.join(src_root, s) for s in SOURCES] + [os.path.join(HERE, "ref_harness.cpp")]

    def one(u):
        o = os.path.join(obj_root, os.path.basename(u).replace(".cpp", ".o"))
        if os.path.exists(o) and os.path.getmtime(o) >= max(os.path.getmtime(u), os.path.getmtime(prelude)):
            return o
        cmd = ["g++"] + flags + ["-c", u, "-o", o]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("compile failed: %s\n%s" % (" ".join(cmd), r.stderr[-4000:]))
        return o

    with ThreadPoolExecutor(max_workers=jobs) as ex:
        objs = list(ex.map(one, units))
    lib = os.path.join(OUT, "libphoton_ref%s.so" % variant)
    cmd = ["g++", "-shared", "-pthread", "-o", lib] + objs
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed: %s\n%s" % (" ".join(cmd), r.stderr[-4000:]))
    return lib


def build(jobs: int | None = None, quiet: bool = False) -> list[str]:
    """Refresh the build copies when the reference checkout exists, then compile.

    Returns the built library paths; returns [] when neither the checkout nor
    earlier build copies exist."""
    jobs = jobs or max(1, min(16, os.cpu_count() or 1))
    os.makedirs(OUT, exist_ok=True)
    if os.path.isdir(os.path.join(REF, "src", "sim")):
        copy_sources()
    if not os.path.isdir(os.path.join(OUT, "src64", "sim")):
        if not quiet:
            print("make_ref: no reference sources; oracle/_ref not built", file=sys.stderr)
        return []
    libs = [compile_variant("64", jobs), compile_variant("32", jobs)]
    return libs


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("--jobs", type=int, default=None)
    a = ap.parse_args()
    for p in build(a.jobs):
        print(p)
