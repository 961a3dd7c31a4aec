"""Build libark_gb300.so (and the ark_run driver) for sm_103a with nvcc, in-tree.

    python ark-cpp-mpi_gb300/ark_build.py            # build if sources changed
    python ark-cpp-mpi_gb300/ark_build.py --force    # rebuild

Translation units are compiled in parallel:
  ark_fp64.cu  FP64 kernels, --fmad=false (bit parity with the reference's FP64 rounding)
  ark_fp32.cu  FP32 kernels, also --fmad=false: every code path rounds alike, so the
               reference-order calls and the fused step agree bit for bit
  ark_api.cu   C ABI, context, CUDA-graph step
  ark_noalloc.cu  conservation sums over caller-owned device arrays, static scratch (--fmad=false)
  ark_ensemble.cu batched ensembles: persistent kernels over a member table (--fmad=false)
  ark_slabs.cu    one channel split along z into slabs with halo exchanges (host code)
  ark_output.cu   VTK packing, time averages, kinetic energy (--fmad=false: the averages and
                  the energy terms round as the reference's)
  ark_closure.cu  learned eddy-viscosity closure: training data, network kernels, inference
  ark_host.cpp host-only helpers (seeded channel init)
Outputs go to ark-cpp-mpi_gb300/lib/ (git-ignored).
"""
from __future__ import annotations

import argparse
import hashlib
import platform
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
SRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "lib")
OBJ = os.path.join(OUT, "obj")
LIB = os.path.join(OUT, "libark_gb300.so")
RUN = os.path.join(OUT, "ark_run")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.isfile(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _digest(extra=()):
    h = hashlib.sha256()
    for name in sorted(os.listdir(SRC)) + [os.path.join("..", "..", "include", "ark_gpu.h")]:
        p = os.path.join(SRC, name)
        if os.path.isfile(p):
            h.update(name.encode())
            with open(p, "rb") as f:
                h.update(f.read())
    with open(__file__, "rb") as f:
        h.update(f.read())
    for e in extra:
        h.update(str(e).encode())
    return h.hexdigest()


CHECK_OUT = os.path.join(HERE, "lib_check")
CHECK_LIB = os.path.join(CHECK_OUT, "libark_gb300.so")


def build(force=False, verbose=False, check=False):
    """Build lib/libark_gb300.so, or with check=True the bounds-checked variant (-DARK_CHECK,
    lib_check/libark_gb300.so: every checked kernel index is compared with its array's extent and
    violations are recorded for ark_bounds_check; slower, for tests)."""
    out = CHECK_OUT if check else OUT
    obj = os.path.join(out, "obj")
    lib = os.path.join(out, "libark_gb300.so")
    run = os.path.join(out, "ark_run")
    os.makedirs(obj, exist_ok=True)
    stamp = os.path.join(out, ".stamp")
    dig = _digest((platform.machine(), check))  # a build for another architecture never counts as current
    if not force and os.path.isfile(lib) and os.path.isfile(run) and os.path.isfile(stamp):
        with open(stamp) as f:
            if f.read().strip() == dig:
                return lib
    nv = nvcc()
    common = ARCH + ["-lineinfo", "-O3", "-std=c++17", "-Xcompiler", "-fPIC", "-I", os.path.join(ROOT, "include")]
    if check:
        common += ["-DARK_CHECK"]
    jobs = [
        [nv] + common + ["--fmad=false", "-c", os.path.join(SRC, "ark_fp64.cu"), "-o", os.path.join(obj, "ark_fp64.o")],
        [nv] + common + ["--fmad=false", "-c", os.path.join(SRC, "ark_fp32.cu"), "-o", os.path.join(obj, "ark_fp32.o")],
        [nv] + common + ["-c", os.path.join(SRC, "ark_api.cu"), "-o", os.path.join(obj, "ark_api.o")],
        [nv] + common + ["--fmad=false", "-c", os.path.join(SRC, "ark_noalloc.cu"), "-o",
                         os.path.join(obj, "ark_noalloc.o")],
        [nv] + common + ["--fmad=false", "-c", os.path.join(SRC, "ark_ensemble.cu"), "-o",
                         os.path.join(obj, "ark_ensemble.o")],
        [nv] + common + ["--fmad=false", "-c", os.path.join(SRC, "ark_output.cu"), "-o",
                         os.path.join(obj, "ark_output.o")],
        [nv] + common + ["-c", os.path.join(SRC, "ark_closure.cu"), "-o", os.path.join(obj, "ark_closure.o")],
        [nv] + common + ["-c", os.path.join(SRC, "ark_slabs.cu"), "-o", os.path.join(obj, "ark_slabs.o")],
        ["g++", "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-I", os.path.join(ROOT, "include"), "-c",
         os.path.join(SRC, "ark_host.cpp"), "-o", os.path.join(obj, "ark_host.o")],
        ["g++", "-O2", "-std=c++17", "-I", os.path.join(ROOT, "include"), "-c",
         os.path.join(SRC, "ark_run.cpp"), "-o", os.path.join(obj, "ark_run.o")],
    ]
    procs = []
    for cmd in jobs:
        if verbose:
            print(" ".join(cmd))
        procs.append((cmd, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)))
    failed = []
    for cmd, p in procs:
        log, _ = p.communicate()
        if p.returncode != 0:
            failed.append((cmd, log.decode(errors="replace")))
        elif verbose and log:
            print(log.decode(errors="replace"))
    if failed:
        msg = "\n".join(" ".join(c) + "\n" + o for c, o in failed)
        raise RuntimeError("build failed:\n" + msg)
    objs = [os.path.join(obj, n) for n in ("ark_fp64.o", "ark_fp32.o", "ark_api.o", "ark_noalloc.o", "ark_ensemble.o",
                                           "ark_output.o", "ark_closure.o", "ark_slabs.o", "ark_host.o")]
    subprocess.run([nv] + ARCH + ["-shared", "-o", lib] + objs + ["-cudart", "static"], check=True)
    subprocess.run(["g++", "-o", run, os.path.join(obj, "ark_run.o"), "-L", out, "-lark_gb300",
                    "-Wl,-rpath,$ORIGIN"], check=True)
    with open(stamp, "w") as f:
        f.write(dig)
    return lib


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("--force", action="store_true")
    ap.add_argument("-v", "--verbose", action="store_true")
    ap.add_argument("--check", action="store_true", help="the bounds-checked build (lib_check/)")
    a = ap.parse_args()
    print(build(force=a.force, verbose=a.verbose, check=a.check))
    sys.exit(0)
