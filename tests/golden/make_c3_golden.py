"""Generates tests/golden/c3_rates_s1.json: the oracle over config 3's 10 s.

Config 3 is the 92,550-cell config-2 scaffold (seed 1, the benchmark's
instance) run for 100,000 exchange steps of 0.1 ms with BF16 synapse tables
and compared against an FP64 run of the same equations.  This script runs the
CPU oracle three times over the full 10 s -- ORC_FP64 (FP32 weights, double
arithmetic), ORC_FP32 with FP32 tables and ORC_FP32 with BF16 tables (the
modes the GPU path reproduces bit for bit) -- and stores per population:

  * spike counts per 1,000-step chunk (100 chunks),
  * a SHA-256 of the complete per-step count array (steps x populations,
    uint32, C order), and
  * for the two FP32 modes, a SHA-256 of the final state (u, g, refractory
    counters as the oracle reports them, little-endian bytes).

The GPU test compares its own 10-s runs with these numbers without having to
rerun the FP64 oracle on the GPU machine.  The oracle is plain C compiled without
floating-point contraction, so the fixture is the same on x86-64 and aarch64.
Usage: python tests/golden/make_c3_golden.py   (about two minutes per mode)
"""
import hashlib
import json
import multiprocessing as mp
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))

SEED, STEPS, CHUNK = 1, 100_000, 1000
MODES = {"fp64": dict(mode=1, bf16=False), "fp32": dict(mode=0, bf16=False),
         "bf16": dict(mode=0, bf16=True)}


def state_digest(u, g, ref) -> str:
    h = hashlib.sha256()
    for a in (u, g, ref):
        h.update(np.ascontiguousarray(a).astype(a.dtype.newbyteorder("<")).tobytes())
    return h.hexdigest()


def run_mode(name: str, steps: int = STEPS):
    import oracle_py

    desc = oracle_py.scaffold_desc(2, 1.0, SEED)
    o = oracle_py.Oracle(desc, seed=SEED, **MODES[name])
    h = hashlib.sha256()
    chunks = []
    for _ in range(steps // CHUNK):
        c, _ = o.run(CHUNK, raster_cap=1 << 22)
        c = np.ascontiguousarray(c, dtype="<u4")
        h.update(c.tobytes())
        chunks.append(c.sum(0).astype(np.int64).tolist())
    out = {"chunk_counts": chunks, "counts_sha256": h.hexdigest()}
    if name != "fp64":
        out["state_sha256"] = state_digest(*o.state())
    return name, out


def main():
    with mp.get_context("spawn").Pool(len(MODES)) as pool:
        res = dict(pool.map(run_mode, list(MODES)))
    doc = {"config": 2, "scale": 1.0, "seed": SEED, "steps": STEPS, "chunk": CHUNK,
           "populations": ["mossy", "granule", "golgi", "stellate", "basket", "purkinje", "dcn"],
           **res}
    with open(os.path.join(HERE, f"c3_rates_s{SEED}.json"), "w") as f:
        json.dump(doc, f, separators=(",", ":"))
    for k in MODES:
        print(k, np.sum(res[k]["chunk_counts"], axis=0).tolist())


if __name__ == "__main__":
    main()
