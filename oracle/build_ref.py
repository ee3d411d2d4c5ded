"""Builds oracle/_ref/libref_harness_s{1,10}.so from the reference's own sources.

TEST INFRASTRUCTURE ONLY.  Compiles the reference's Simulation_header.cu where
it lies (never copied) together with ref_harness.cu, oracle.c and refport.c.
The reference fixes its step in option.h (DT 0.1 ms, STEP_MAX 10); that header
is skipped through its own include guard (-DOPTION_H) and the same macros are
given on the command line, once with STEP_MAX=1 (0.1-ms exchange steps) and
once with STEP_MAX=10 (the reference's 1-ms steps).  Output goes to
oracle/_ref/ only.  Exits 0 with a message when the sources are absent.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")
# The reference's Scaffold directory: SGB_REFERENCE_DIR when set, else the
# read-only checkout this recipe is written for.
REF = os.environ.get("SGB_REFERENCE_DIR") or "/root/reference/SimulationModule/Scaffold"
NVCC = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode:
        raise RuntimeError(" ".join(cmd) + "\n" + r.stdout + r.stderr)


def build() -> list[str]:
    src = os.path.join(REF, "Simulation_header.cu")
    if not os.path.exists(src):
        print(f"reference sources not found at {REF}; oracle/_ref not built")
        return []
    os.makedirs(OUT, exist_ok=True)
    built = []
    for step_max in (1, 10):
        defs = ["-DOPTION_H", "-Dsec=(1000.)", "-DDT=(0.1)", "-DT_MAX=(1000)",
                f"-DSTEP_MAX={step_max}", "-DCUDA_CORES=(5000)"]
        lib = os.path.join(OUT, f"libref_harness_s{step_max}.so")
        deps = [src, os.path.join(HERE, "ref_harness.cu"), os.path.join(HERE, "refport.c"),
                os.path.join(HERE, "oracle.c")]
        if os.path.exists(lib) and all(os.path.getmtime(lib) > os.path.getmtime(d) for d in deps):
            built.append(lib)
            continue
        common = ARCH + ["-O3", "-Xcompiler", "-fPIC", "-Xcompiler", "-fopenmp",
                         "-Xcompiler", "-ffp-contract=off", "-I", REF, "-I", HERE] + defs
        o_ref = os.path.join(OUT, f"Simulation_header_s{step_max}.o")
        o_h = os.path.join(OUT, f"ref_harness_s{step_max}.o")
        o_c = os.path.join(OUT, "oracle.o")
        o_p = os.path.join(OUT, "refport.o")
        _run([NVCC] + common + ["-c", src, "-o", o_ref])
        _run([NVCC] + common + ["-c", os.path.join(HERE, "ref_harness.cu"), "-o", o_h])
        cflags = ["-O2", "-std=c99", "-fPIC", "-ffp-contract=off", "-fopenmp", "-I", HERE]
        _run(["gcc"] + cflags + ["-c", os.path.join(HERE, "oracle.c"), "-o", o_c])
        _run(["gcc"] + cflags + ["-c", os.path.join(HERE, "refport.c"), "-o", o_p])
        _run([NVCC] + ARCH + ["-shared", "-o", lib, o_ref, o_h, o_c, o_p,
                              "-Xcompiler", "-fopenmp", "-lgomp", "-lcurand"])
        built.append(lib)
    return built


if __name__ == "__main__":
    for p in build():
        print(p)
    sys.exit(0)
