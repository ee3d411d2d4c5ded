"""Builds libscaffold_gb300.so in-tree: CUDA kernels for sm_103a, host C++.

Translation units compile in parallel; the library links cudart statically
and OpenMP dynamically, so it loads on any box with the same CUDA driver.
Usage: python build.py [--force]
"""
from __future__ import annotations

import concurrent.futures as cf
import json
import os
import platform
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "scaffold_gb300", "libscaffold_gb300.so")
INCLUDE = os.path.normpath(os.path.join(HERE, "..", "include"))

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CUDA_HOME = os.environ.get("CUDA_HOME", "/usr/local/cuda")
NVCC = shutil.which("nvcc") or os.path.join(CUDA_HOME, "bin", "nvcc")
CXX = os.environ.get("CXX", "g++")

# Host code must give identical results on x86-64 and aarch64: no
# -march=native, no fused multiply-add contraction.
HOST_FLAGS = ["-O3", "-std=c++17", "-fPIC", "-fopenmp", "-ffp-contract=off", "-Wall",
              "-Wno-unused-function"]
NVCC_FLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
                     "-Xcompiler", "-ffp-contract=off", "-Xcompiler", "-fopenmp",
                     "--expt-relaxed-constexpr"]

SOURCES = [
    ("sgb_model.cpp", "cxx"),
    ("sgb_capi.cpp", "cxx"),
    ("sgb_compat.cpp", "cxx"),
    ("sgb_engine.cu", "nvcc"),
    ("sgb_kernels.cu", "nvcc"),
    ("sgb_ops.cu", "nvcc"),
]
HEADERS = ["sgb_philox.h", "sgb_model.h", "sgb_device.h", "sgb_engine.h"]


def _newer(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _compile(src: str, kind: str) -> tuple[str, bool]:
    """Object of one translation unit, and whether it was compiled now."""
    path = os.path.join(CSRC, src)
    obj = os.path.join(BUILD, src + ".o")
    deps = [path] + [os.path.join(CSRC, h) for h in HEADERS] + [
        os.path.join(INCLUDE, "scaffold_gb300.h"), os.path.join(INCLUDE, "scaffold_compat.h")]
    if not _newer(obj, deps):
        return obj, False
    if kind == "cxx":
        cmd = [CXX] + HOST_FLAGS + ["-I", os.path.join(CUDA_HOME, "include"), "-c", path, "-o", obj]
    else:
        cmd = [NVCC] + NVCC_FLAGS + ["-c", path, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return obj, True


def build(force: bool = False) -> str:
    """Builds the library if any source is newer than it; writes what was done
    (units compiled or up to date, whether the library was linked) to
    _build/build_record.json and prints it as one JSON line."""
    os.makedirs(BUILD, exist_ok=True)
    if force:
        for f in os.listdir(BUILD):
            if f.endswith(".o"):
                os.remove(os.path.join(BUILD, f))
    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        done = list(ex.map(lambda s: _compile(*s), SOURCES))
    objs = [o for o, _ in done]
    linked = force or _newer(LIB, objs)
    if linked:
        cmd = [NVCC] + ARCH + ["-shared", "-o", LIB] + objs + ["-Xcompiler", "-fopenmp", "-lgomp"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    record = {"lib": LIB, "arch": ARCH[1],
              "compiled": [src for (src, _), (_, c) in zip(SOURCES, done) if c],
              "up_to_date": [src for (src, _), (_, c) in zip(SOURCES, done) if not c],
              "linked": linked, "machine": platform.machine()}
    with open(os.path.join(BUILD, "build_record.json"), "w") as f:
        json.dump(record, f)
    print("build record: " + json.dumps(record), flush=True)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
