"""Config 3 accuracy: BF16 synapse weights and FP32 state against the FP64 oracle.

On the 92,550-cell scaffold the GPU raster (FP32 and BF16 tables) is compared
with the FP64 oracle's: first step whose spike sets differ, fraction of the
oracle's spikes reproduced by the same cell within +-1 step, and the relative
firing-rate error of every population.  The FP32 path is additionally
bit-identical to the FP32 oracle.  Set SGB_ACCURACY_OUT to a path to record
the numbers as JSON.
"""
import json
import os

import numpy as np
import pytest

import oracle_py
import scaffold_gb300 as sg

pytestmark = pytest.mark.gpu

STEPS = 4000  # 0.4 s of biological time (includes the 260-300 ms mossy burst)


def _match_within_one(ids_a, off_a, ids_b, off_b, n_cells):
    """Fraction of b's spikes that a has at the same cell within +-1 step."""
    n = len(off_b) - 1
    sets = [set(ids_a[off_a[s]:off_a[s + 1]].tolist()) for s in range(n)]
    hit = tot = 0
    for s in range(n):
        for c in ids_b[off_b[s]:off_b[s + 1]].tolist():
            tot += 1
            if c in sets[s] or (s > 0 and c in sets[s - 1]) or (s + 1 < n and c in sets[s + 1]):
                hit += 1
    return hit / max(tot, 1)


def _first_div(ids_a, off_a, ids_b, off_b):
    for s in range(len(off_a) - 1):
        if not np.array_equal(ids_a[off_a[s]:off_a[s + 1]], ids_b[off_b[s]:off_b[s + 1]]):
            return s
    return len(off_a) - 1


def test_bf16_and_fp32_against_fp64_oracle():
    net = sg.scaffold(2, 1.0, 1)
    d = oracle_py.describe(net)
    nums = np.array([p["num"] for p in d["pops"]], float)
    ref64 = oracle_py.Oracle(d, seed=1, mode=oracle_py.FP64)
    c64, (i64, o64) = ref64.run(STEPS, raster_cap=1 << 24)
    out = {"steps": STEPS, "populations": [p.name for p in net.populations]}
    for name, wt in (("fp32", sg.WEIGHT_FP32), ("bf16", sg.WEIGHT_BF16)):
        sim = sg.Simulation([net], [1], weight_type=wt, raster=True)
        c, (ids, offs) = sim.loop_n_steps(STEPS, raster=True, raster_cap=1 << 24)
        tot, tot64 = c.sum(0).astype(np.int64), c64.sum(0).astype(np.int64)
        rate_err = (tot - tot64) / np.maximum(tot64, 1)
        out[name] = {
            "first_divergence_step": _first_div(ids, offs, i64, o64),
            "matched_within_1_step": _match_within_one(ids, offs, i64, o64, net.counts()["neurons"]),
            "rate_rel_error": rate_err.tolist(),
            "rates_hz": (c.sum(0) / nums / (STEPS * 1e-4)).tolist(),
        }
        sim.close()
    out["fp64_rates_hz"] = (c64.sum(0) / nums / (STEPS * 1e-4)).tolist()
    path = os.environ.get("SGB_ACCURACY_OUT")
    if path:
        with open(path, "w") as f:
            json.dump(out, f, indent=1)
    for name in ("fp32", "bf16"):
        # Populations with enough spikes for a rate to be meaningful.
        r = np.abs(np.array(out[name]["rate_rel_error"]))[c64.sum(0) > 500]
        assert (r < 0.05).all(), (name, out[name])
        assert out[name]["matched_within_1_step"] > 0.5, (name, out[name])
    assert out["fp32"]["first_divergence_step"] > 100
