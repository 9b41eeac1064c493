"""Build recipe for libqtipgpu.so (the CUDA library behind include/qtip4pf_gb300.h).

Compiles every csrc/*.cu for sm_103a only, one translation unit per nvcc
process in parallel, and links them (cudart linked statically) into
qtip4pf_water_gb300/_build/libqtipgpu.so. Also builds the drop-in C++ shim
libqtip_compat.so that exports the reference's own function signatures.

    python -m qtip4pf_water_gb300.build [--force] [--verbose]
"""
from __future__ import annotations

import argparse
import concurrent.futures as cf
import glob
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libqtipgpu.so")
COMPAT = os.path.join(BUILD, "libqtip_compat.so")
DROPIN_BENCH = os.path.join(BUILD, "dropin_bench")
RUN_DRIVER = os.path.join(BUILD, "qtg_water")
E2E_BENCH = os.path.join(BUILD, "e2e_bench")
INCLUDE = os.path.join(ROOT, "include")
# boost::math::cubic_b_spline for drop-in builds without Boost (the reference's
# spline signatures name that type)
COMPAT_INCLUDE = os.path.join(CSRC, "compat", "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# host code: no floating-point contraction, so the host-side parameter derivations
# round like the reference's x86-64 build on every host architecture
NVFLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
           "--expt-relaxed-constexpr", "-Xptxas", "-warn-spills"]


def nvcc() -> str:
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found: the CUDA 13 toolkit is required to build libqtipgpu")


def _sources():
    return sorted(glob.glob(os.path.join(CSRC, "*.cu")) + glob.glob(os.path.join(CSRC, "*.cpp")))


def _headers():
    return sorted(glob.glob(os.path.join(CSRC, "*.h")) + glob.glob(os.path.join(INCLUDE, "*.h")))


def _stale(target: str, deps) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _run(cmd, verbose):
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"command failed ({r.returncode}): {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    if verbose and (r.stdout or r.stderr):
        print(r.stdout + r.stderr, flush=True)
    return r


def build(force: bool = False, verbose: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    nv = nvcc()
    srcs = _sources()
    hdrs = _headers()
    objs = []
    jobs = []
    cxx = shutil.which("g++") or "g++"
    for s in srcs:
        o = os.path.join(BUILD, os.path.splitext(os.path.basename(s))[0] + ".o")
        objs.append(o)
        if force or _stale(o, [s] + hdrs):
            if s.endswith(".cpp"):  # host-only C++
                jobs.append([cxx, "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-I", INCLUDE, "-c", s, "-o", o])
            else:
                jobs.append([nv] + ARCH + NVFLAGS + ["-I", INCLUDE, "-c", s, "-o", o])
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            for f in [ex.submit(_run, j, verbose) for j in jobs]:
                f.result()
    if force or jobs or _stale(LIB, objs):
        _run([nv] + ARCH + ["-shared", "-cudart", "static", "-o", LIB] + objs, verbose)
    compat_src = os.path.join(CSRC, "compat", "compat.cpp")
    compat_hdrs = glob.glob(os.path.join(COMPAT_INCLUDE, "**", "*.hpp"), recursive=True)
    if os.path.exists(compat_src) and (force or _stale(COMPAT, [compat_src, LIB] + hdrs + compat_hdrs)):
        cxx = shutil.which("g++") or "g++"
        # an installed Boost.Math takes precedence over the stand-in spline header
        _run([cxx, "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-shared", "-I", INCLUDE,
              "-idirafter", COMPAT_INCLUDE, compat_src, "-o", COMPAT,
              "-L", BUILD, "-lqtipgpu", "-Wl,-rpath,$ORIGIN"], verbose)
    # the drop-in's end-to-end timing driver (simulation.cpp's sampling loop)
    bench_src = os.path.join(CSRC, "compat", "dropin_bench.cpp")
    if os.path.exists(bench_src) and (force or _stale(DROPIN_BENCH, [bench_src, COMPAT])):
        cxx = shutil.which("g++") or "g++"
        _run([cxx, "-O2", "-std=c++17", bench_src, "-o", DROPIN_BENCH, "-L", BUILD, "-lqtip_compat", "-lqtipgpu",
              "-Wl,-rpath,$ORIGIN"], verbose)
    # the run driver: config.txt in, the reference's output files out (device-resident steps)
    drv_src = os.path.join(CSRC, "driver", "qtg_water.cpp")
    if os.path.exists(drv_src) and (force or _stale(RUN_DRIVER, [drv_src, LIB, os.path.join(CSRC, "lattice.h")] + hdrs)):
        cxx = shutil.which("g++") or "g++"
        _run([cxx, "-O2", "-std=c++17", "-ffp-contract=off", "-I", INCLUDE, drv_src, "-o", RUN_DRIVER, "-L", BUILD,
              "-lqtipgpu", "-Wl,-rpath,$ORIGIN"], verbose)
    # the per-call end-to-end timing driver (C ABI from host C++)
    e2e_src = os.path.join(CSRC, "driver", "e2e_bench.cpp")
    if os.path.exists(e2e_src) and (force or _stale(E2E_BENCH, [e2e_src, LIB] + hdrs)):
        cxx = shutil.which("g++") or "g++"
        _run([cxx, "-O2", "-std=c++17", "-I", INCLUDE, e2e_src, "-o", E2E_BENCH, "-L", BUILD, "-lqtipgpu",
              "-Wl,-rpath,$ORIGIN"], verbose)
    return LIB


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--force", action="store_true")
    ap.add_argument("--verbose", action="store_true")
    a = ap.parse_args(argv)
    print(build(force=a.force, verbose=a.verbose))


if __name__ == "__main__":
    sys.exit(main())
