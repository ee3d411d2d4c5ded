"""Generates tests/golden/ref_*.npz from the reference's own CPU functions.

Runs host_update_lif_ch / host_spike_propagation, compiled from the reference
sources by oracle/build_ref.py (needs the reference checkout, so this runs only
where it is mounted), over small synthetic scaffolds built with the library's
generator, and stores per-step spike counts, the raster and the final state.
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
import scaffold_gb300 as sg  # noqa: E402

# (file, scaffold config, scale, seed, substeps, steps, bf16)
CASES = [
    ("ref_c1q_s11.npz", 1, 0.25, 11, 1, 2000, False),
    ("ref_c1q_s12_bf16.npz", 1, 0.25, 12, 1, 1500, True),
    ("ref_c1q_s4_sub10.npz", 1, 0.25, 4, 10, 300, False),
]


def main():
    if not build_ref.build():
        raise SystemExit("reference sources are required to generate these fixtures")
    for fname, cfg, scale, seed, sub, steps, bf16 in CASES:
        net = sg.scaffold(cfg, scale, seed)
        h = oracle_py.RefHarness(oracle_py.describe(net), seed=seed, substeps=sub, bf16=bf16)
        counts, (ids, offs) = h.run(steps, threads=1)
        u, g, ref = h.state()
        np.savez_compressed(os.path.join(HERE, fname), config=cfg, scale=scale, seed=seed,
                            substeps=sub, steps=steps, bf16=bf16, counts=counts, ids=ids,
                            offs=offs, u=u, g=g, ref=ref)
        print(fname, int(counts.sum()), "spikes")


if __name__ == "__main__":
    main()
