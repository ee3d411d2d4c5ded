"""Generates tests/golden/ref_*.npz from the reference's own CPU functions.

Runs host_update_lif_ch / host_spike_propagation, compiled from the reference
sources by oracle/build_ref.py (needs the reference checkout, so this runs only
where it is mounted), over synthetic scaffolds drawn by the oracle's own
generator (oracle/netgen.c, which draws the library's networks exactly), and
stores per-step spike counts, the raster and the final state: quarter-scale
config 1, the full config 1 (9,256 cells) over its whole 10,000 steps, and
full config 2 (92,550 cells, 2.73M synapses) over 600 steps in FP32 and BF16.
Tests replay the same networks and compare without needing the reference.
Usage: python tests/golden/make_ref_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "cerebellar-scaffold-model-simulation-on-gpu_gb300"))
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import build_ref  # noqa: E402
import oracle_py  # noqa: E402

# (file, scaffold config, scale, seed, substeps, steps, bf16)
CASES = [
    ("ref_c1q_s11.npz", 1, 0.25, 11, 1, 2000, False),
    ("ref_c1q_s12_bf16.npz", 1, 0.25, 12, 1, 1500, True),
    ("ref_c1q_s4_sub10.npz", 1, 0.25, 4, 10, 300, False),
    ("ref_c1_s1_full.npz", 1, 1.0, 1, 1, 10000, False),
    ("ref_c2_s3.npz", 2, 1.0, 3, 1, 600, False),
    ("ref_c2_s3_bf16.npz", 2, 1.0, 3, 1, 600, True),
]


def main(only=None):
    if not build_ref.build():
        raise SystemExit("reference sources are required to generate these fixtures")
    for fname, cfg, scale, seed, sub, steps, bf16 in CASES:
        if only and fname not in only:
            continue
        desc = oracle_py.scaffold_desc(cfg, scale, seed)
        h = oracle_py.RefHarness(desc, seed=seed, substeps=sub, bf16=bf16)
        counts, (ids, offs) = h.run(steps, threads=0, raster_cap=1 << 24)
        u, g, ref = h.state()
        np.savez_compressed(os.path.join(HERE, fname), config=cfg, scale=scale, seed=seed,
                            substeps=sub, steps=steps, bf16=bf16, counts=counts, ids=ids,
                            offs=offs, u=u, g=g, ref=ref)
        print(fname, int(counts.sum()), "spikes")


if __name__ == "__main__":
    main(sys.argv[1:])
