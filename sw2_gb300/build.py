"""Builds, in-tree (sw2_gb300/_build/):
  libsw2g.so    the GPU step behind the C ABI, for sm_103a;
  libsw2host.so the case reader and forcing restatement (plain C, no CUDA);
  sw2g-run      the command-line runner of SW2 case files (host/swmain.c).

Translation units compile in parallel; the FP64 step is compiled with
-fmad=false (no contraction, for bit-identity with the reference) and host
code with -ffp-contract=off (gcc contracts by default on aarch64).

    python -m sw2_gb300.build
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libsw2g.so")
HOSTDIR = os.path.join(HERE, "host")
HOSTLIB = os.path.join(OUT, "libsw2host.so")
RUNNER = os.path.join(OUT, "sw2g-run")
HOST_SRC = ["swcase.c", "swforce.c"]
HOST_C = ["gcc", "-std=gnu11", "-O2", "-fPIC", "-ffp-contract=off", "-fno-fast-math", "-Wall"]

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
HOST = "-fPIC,-ffp-contract=off,-O2"

# (source, extra nvcc flags, object name); the FP32 form's limiter kernels are
# one source compiled once per limiter group
UNITS = [
    ("api.cu", [], "api.o"),
    ("step_fp64.cu", ["-fmad=false"], "step_fp64.o"),
    ("noalloc.cu", ["-fmad=false"], "noalloc.o"),
    ("step_fp32.cu", ["-fmad=false"], "step_fp32.o"),
    *[("step_fp32_limiters.cu", ["-fmad=false", f"-DSW2G_LIMITER_GROUP={g}"], f"step_fp32_limiters{g}.o")
      for g in range(4)],
    ("forcing.cu", ["-fmad=false"], "forcing.o"),
    ("geometry.cpp", None, "geometry.o"),  # plain host C++
]


def nvcc() -> str:
    p = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    return p


def _compile(src: str, extra, objname: str) -> str:
    obj = os.path.join(OUT, objname)
    path = os.path.join(CSRC, src)
    inc = ["-I", os.path.join(ROOT, "include"), "-I", CSRC]
    if extra is None:
        cuda_inc = os.path.join(os.path.dirname(os.path.dirname(nvcc())), "include")
        cmd = ["g++", "-std=c++17", "-O2", "-fPIC", "-ffp-contract=off", "-fno-fast-math", *inc, "-I", cuda_inc,
               "-c", path, "-o", obj]
    else:
        cmd = [nvcc(), *ARCH, "-std=c++17", "-O3", "-lineinfo", "-Xcompiler", HOST, "-Xptxas", "-v" if os.environ.get("SW2G_PTXAS_V") else "-O3",
               *extra, *inc, "-c", path, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    if os.environ.get("SW2G_PTXAS_V"):
        sys.stderr.write(r.stderr)
    return obj


def _stale() -> bool:
    outs = [LIB, HOSTLIB, RUNNER]
    if not all(os.path.exists(o) for o in outs):
        return True
    t = min(os.path.getmtime(o) for o in outs)
    srcs = [os.path.join(CSRC, f) for f in os.listdir(CSRC)] + [os.path.join(HOSTDIR, f) for f in os.listdir(HOSTDIR)]
    srcs += [os.path.join(ROOT, "include", "sw2g.h"), __file__]
    return any(os.path.getmtime(s) > t for s in srcs)


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"build step failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")


def build_host() -> None:
    """libsw2host.so and sw2g-run (the runner links libsw2g.so, found next to it)."""
    inc = ["-I", os.path.join(ROOT, "include"), "-I", HOSTDIR]
    srcs = [os.path.join(HOSTDIR, f) for f in HOST_SRC]
    _run([*HOST_C, "-shared", *inc, *srcs, "-o", HOSTLIB + ".tmp", "-lm"])
    os.replace(HOSTLIB + ".tmp", HOSTLIB)
    run_srcs = srcs + [os.path.join(HOSTDIR, "swrun.c"), os.path.join(HOSTDIR, "swmain.c")]
    _run([*HOST_C, *inc, *run_srcs, "-o", RUNNER + ".tmp", "-L", OUT, "-lsw2g", "-Wl,-rpath,$ORIGIN", "-lm",
          "-lpthread"])
    os.replace(RUNNER + ".tmp", RUNNER)


def build(force: bool = False) -> str:
    if not force and not _stale():
        return LIB
    os.makedirs(OUT, exist_ok=True)
    with ThreadPoolExecutor(max_workers=min(len(UNITS), os.cpu_count() or 4)) as ex:
        objs = list(ex.map(lambda u: _compile(*u), UNITS))
    tmp = LIB + ".tmp"
    cmd = [nvcc(), *ARCH, "-shared", "-o", tmp, *objs, "-Xcompiler", "-fPIC"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    build_host()
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
