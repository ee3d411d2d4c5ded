"""The oracle itself: pinned to independent implementations and closed forms.

* Philox4x32-10 against vectors from PyTorch's engine (tests/golden).
* Golden rasters produced by the reference's own compiled CPU functions
  (tests/golden/ref_*.npz): the restatement of those loops reproduces them bit
  for bit; the FP32 and FP64 oracles reproduce their spikes.
* The LIF arithmetic against closed-form solutions of the Euler recurrences.
"""
import json
import os

import numpy as np
import pytest

import oracle_py
import scaffold_gb300 as sg
from scaffold_gb300 import configs

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def test_philox_matches_pytorch_engine():
    d = json.load(open(os.path.join(GOLDEN, "philox4x32_10.json")))
    assert len(d["vectors"]) >= 8
    for v in d["vectors"]:
        assert oracle_py.philox(v["ctr"], v["key"]) == v["out"]
        assert configs._philox(v["ctr"], v["key"][0], v["key"][1]) == v["out"]


def _golden(name):
    z = np.load(os.path.join(GOLDEN, name))
    net = sg.scaffold(int(z["config"]), float(z["scale"]), int(z["seed"]))
    return z, net


def _first_divergence(ids_a, off_a, ids_b, off_b):
    n = len(off_a) - 1
    for s in range(n):
        if not np.array_equal(ids_a[off_a[s]:off_a[s + 1]], ids_b[off_b[s]:off_b[s + 1]]):
            return s
    return n


@pytest.mark.parametrize("name", ["ref_c1q_s11.npz", "ref_c1q_s12_bf16.npz",
                                  "ref_c1q_s4_sub10.npz"])
def test_reference_cpu_restatement_reproduces_golden(name):
    """rp_* (C restatement of host_update_lif_ch / host_spike_propagation) gives
    exactly the raster and state the reference's compiled functions gave."""
    z, net = _golden(name)
    rp = oracle_py.RefPort(oracle_py.describe(net), seed=int(z["seed"]),
                           substeps=int(z["substeps"]), bf16=bool(z["bf16"]))
    counts, (ids, offs) = rp.run(int(z["steps"]), threads=2)
    u, g, ref = rp.state()
    assert np.array_equal(counts, z["counts"])
    assert np.array_equal(ids, z["ids"]) and np.array_equal(offs, z["offs"])
    assert np.array_equal(u.view(np.uint32), z["u"].view(np.uint32))
    assert np.array_equal(g.view(np.uint32), z["g"].view(np.uint32))
    assert np.array_equal(ref, z["ref"])


@pytest.mark.parametrize("mode", [oracle_py.FP32, oracle_py.FP64])
@pytest.mark.parametrize("name", ["ref_c1q_s11.npz", "ref_c1q_s4_sub10.npz"])
def test_oracle_raster_equals_reference_until_divergence(name, mode):
    """The oracle's spikes equal the reference's over the fixture; membrane
    state within FP32 rounding of the reference's mixed precision."""
    z, net = _golden(name)
    o = oracle_py.Oracle(oracle_py.describe(net), seed=int(z["seed"]),
                         substeps=int(z["substeps"]), mode=mode)
    counts, (ids, offs) = o.run(int(z["steps"]))
    assert _first_divergence(ids, offs, z["ids"], z["offs"]) == int(z["steps"])
    assert np.array_equal(counts, z["counts"])
    u, g, ref = o.state()
    assert np.array_equal(ref, z["ref"])
    np.testing.assert_allclose(u, z["u"], rtol=0, atol=2e-3)
    np.testing.assert_allclose(g, z["g"], rtol=1e-3, atol=1e-4)


def test_bf16_golden_fp32_oracle():
    z, net = _golden("ref_c1q_s12_bf16.npz")
    o = oracle_py.Oracle(oracle_py.describe(net), seed=int(z["seed"]), bf16=True)
    counts, (ids, offs) = o.run(int(z["steps"]))
    assert _first_divergence(ids, offs, z["ids"], z["offs"]) == int(z["steps"])


# ---- benchmark-scale fixtures: full config 1 (10,000 steps), config 2 (600) ----
def _golden_desc(name):
    z = np.load(os.path.join(GOLDEN, name))
    return z, oracle_py.scaffold_desc(int(z["config"]), float(z["scale"]), int(z["seed"]))


@pytest.mark.parametrize("name", ["ref_c1_s1_full.npz", "ref_c2_s3.npz", "ref_c2_s3_bf16.npz"])
def test_reference_cpu_restatement_reproduces_benchmark_scale_golden(name):
    """rp_* reproduces the reference's compiled functions bit for bit on the
    full config 1 over its 10,000 steps and on config 2 (92,550 cells,
    2,731,520 synapses, in-degree up to 25,000) in FP32 and BF16."""
    z, desc = _golden_desc(name)
    rp = oracle_py.RefPort(desc, seed=int(z["seed"]), bf16=bool(z["bf16"]))
    counts, (ids, offs) = rp.run(int(z["steps"]), threads=4, raster_cap=1 << 22)
    u, g, ref = rp.state()
    assert np.array_equal(counts, z["counts"])
    assert np.array_equal(ids, z["ids"]) and np.array_equal(offs, z["offs"])
    assert np.array_equal(u.view(np.uint32), z["u"].view(np.uint32))
    assert np.array_equal(g.view(np.uint32), z["g"].view(np.uint32))
    assert np.array_equal(ref, z["ref"])


@pytest.mark.parametrize("name,mode", [("ref_c2_s3.npz", oracle_py.FP32),
                                       ("ref_c2_s3.npz", oracle_py.FP64),
                                       ("ref_c2_s3_bf16.npz", oracle_py.FP32)])
def test_oracle_equals_reference_on_config2(name, mode):
    """On config 2 the oracle's raster equals the reference's spike for spike
    over the whole fixture (600 steps), FP32 and BF16 tables (the FP64 mode
    always uses the unrounded weights, so it pairs with the FP32 fixture)."""
    z, desc = _golden_desc(name)
    o = oracle_py.Oracle(desc, seed=int(z["seed"]), bf16=bool(z["bf16"]), mode=mode)
    counts, (ids, offs) = o.run(int(z["steps"]), raster_cap=1 << 22)
    assert _first_divergence(ids, offs, z["ids"], z["offs"]) == int(z["steps"])
    assert np.array_equal(counts, z["counts"])
    u, g, ref = o.state()
    assert np.array_equal(ref, z["ref"])
    np.testing.assert_allclose(u, z["u"], rtol=0, atol=2e-3)
    np.testing.assert_allclose(g, z["g"], rtol=1e-3, atol=1e-4)


@pytest.mark.parametrize("mode", [oracle_py.FP32, oracle_py.FP64])
def test_oracle_against_reference_full_config1(mode):
    """Full config 1 over its 1 s (10,000 steps): the rasters are identical
    until step 2,703, where a cell at threshold crosses one step apart in the
    reference's mixed precision (FP32 state, double DT/Cm) and in the oracle;
    over the whole second every spike is matched by the same cell within one
    step and every population's spike total is identical."""
    z, desc = _golden_desc("ref_c1_s1_full.npz")
    o = oracle_py.Oracle(desc, seed=1, mode=mode)
    steps = int(z["steps"])
    counts, (ids, offs) = o.run(steps, raster_cap=1 << 22)
    assert _first_divergence(ids, offs, z["ids"], z["offs"]) >= 2000
    differing = []
    for s in range(steps):
        a = set(ids[offs[s]:offs[s + 1]].tolist())
        b = set(z["ids"][z["offs"][s]:z["offs"][s + 1]].tolist())
        if a != b:
            differing.append((s, a - b, b - a))
    assert len(differing) <= 8
    for s, extra, missing in differing:  # each difference is a spike moved by one step
        for c in extra | missing:
            near = set()
            for t in (s - 1, s + 1):
                near |= set(z["ids"][z["offs"][t]:z["offs"][t + 1]].tolist())
                near |= set(ids[offs[t]:offs[t + 1]].tolist())
            assert c in near
    assert np.array_equal(counts.sum(0), z["counts"].sum(0))


# ---- closed forms -------------------------------------------------------------
def _single(num=4, Ie=0.0, dt_ref=2.0, tau=(0.5, 10.0), Vth=-50.0):
    net = sg.Network()
    net.set_neuron_params("p", num, 3.0, -70.0, dt_ref, Ie, -70.0, Vth, 0.2, sg.NORMAL,
                          [(1.0, 0.0, 1.0, tau[0]), (1.0, -80.0, 1.0, tau[1])])
    return net


@pytest.mark.parametrize("mode,tol", [(oracle_py.FP64, 1e-5), (oracle_py.FP32, 2e-4)])
def test_subthreshold_relaxation(mode, tol):
    """u_{k+1} - u* = (1 - dt gL / C)(u_k - u*), u* = E_L + Ie / gL."""
    Ie = 2.0  # u* = -60 mV, below threshold
    net = _single(Ie=Ie)
    o = oracle_py.Oracle(oracle_py.describe(net), seed=3, mode=mode)
    u0, _, _ = o.state()
    n = 700
    o.run(n)
    u, g, ref = o.state()
    ustar = -70.0 + Ie / 0.2
    expect = ustar + (1 - 0.1 * 0.2 / 3.0) ** n * (u0.astype(np.float64) - ustar)
    np.testing.assert_allclose(u, expect, rtol=0, atol=tol)  # state is reported in FP32
    assert (ref == 0).all() and (g == 0).all()


@pytest.mark.parametrize("dt_ref,steps", [(1.5, 15), (0.8, 8), (1.6, 16), (2.0, 20), (3.7, 37)])
def test_refractory_length(dt_ref, steps):
    """ref_step = (int)(dt_ref / DT) in double (Simulation_header.cu:322); the
    cell stays at Vr for that many steps after a spike."""
    net = _single(num=1, dt_ref=dt_ref)
    for mode in (oracle_py.FP32, oracle_py.FP64):
        o = oracle_py.Oracle(oracle_py.describe(net), seed=1, mode=mode)
        o.set_state(np.array([-40.0], np.float32), np.zeros((1, 2), np.float32),
                    np.zeros(1, np.int32))
        c, _ = o.run(1)
        assert c[0, 0] == 1
        u, _, ref = o.state()
        assert ref[0] == steps and u[0] == -70.0
        for k in range(steps - 1):
            o.run(1)
            u, _, ref = o.state()
            assert u[0] == -70.0 and ref[0] == steps - 1 - k


def test_conductance_decay():
    """Without input g_c decays by (1 - dt / tau_c) per step."""
    net = _single(num=2)
    o = oracle_py.Oracle(oracle_py.describe(net), seed=1, mode=oracle_py.FP64)
    o.set_state(np.array([-70.0, -65.0], np.float32), np.full((2, 2), 1.0, np.float32),
                np.zeros(2, np.int32))
    o.run(25)
    _, g, _ = o.state()
    np.testing.assert_allclose(g[:, 0], (1 - 0.1 / 0.5) ** 25, rtol=1e-6)
    np.testing.assert_allclose(g[:, 1], (1 - 0.1 / 10.0) ** 25, rtol=1e-6)


def test_first_spike_time_constant_current():
    """Suprathreshold drive: the oracle fires on the step the Euler recurrence
    crosses threshold (the crossing is tested on the pre-update potential)."""
    Ie = 5.0  # u* = -45 mV > Vth
    net = _single(num=1, Ie=Ie)
    o = oracle_py.Oracle(oracle_py.describe(net), seed=1, mode=oracle_py.FP64)
    o.set_state(np.array([-70.0], np.float32), np.zeros((1, 2), np.float32),
                np.zeros(1, np.int32))
    c, _ = o.run(600)
    u, k = -70.0, 0
    while True:
        if u > -50.0:
            break
        u = u + 0.1 / 3.0 * (Ie - 0.2 * (u + 70.0))
        k += 1
    assert np.flatnonzero(c[:, 0])[0] == k


def test_fp32_fp64_rates_close():
    net = sg.scaffold(1, 0.5, 21)
    d = oracle_py.describe(net)
    c32, _ = oracle_py.Oracle(d, seed=21, mode=oracle_py.FP32).run(4000)
    c64, _ = oracle_py.Oracle(d, seed=21, mode=oracle_py.FP64).run(4000)
    r32, r64 = c32.sum(0).astype(float), c64.sum(0).astype(float)
    assert r64.min() > 0
    np.testing.assert_allclose(r32, r64, rtol=0.05)


def test_scale_bits_rule():
    """Largest S <= 30 with every post cell's sum of rint(w 2^S) <= INT32_MAX."""
    net = sg.scaffold(1, 0.25, 2)
    d = oracle_py.describe(net)
    o = oracle_py.Oracle(d, seed=2)
    for p, pop in enumerate(d["pops"]):
        for ch in (0, 1):
            s = o.scale_bits(p, ch)
            projs = [q for q in d["projs"] if q["post"] == p and q["channel"] == ch]
            if not projs:
                assert s == 30
                continue

            def worst(S):
                tot = np.zeros(pop["num"], np.int64)
                for q in projs:
                    np.add.at(tot, q["post_idx"].astype(np.int64),
                              np.rint(q["weight"].astype(np.float32) * np.float32(2.0 ** S))
                              .astype(np.int64))
                return tot.max()

            assert worst(s) <= 2**31 - 1
            assert s == 30 or worst(s + 1) > 2**31 - 1


def test_config3_fixture_matches_the_oracle():
    """tests/golden/c3_rates_s1.json (the oracle over config 3's 10 s, which
    the GPU accuracy test reads) agrees with a fresh oracle run over its
    first 1,000 steps in all three modes."""
    fx = json.load(open(os.path.join(GOLDEN, "c3_rates_s1.json")))
    desc = oracle_py.scaffold_desc(fx["config"], fx["scale"], fx["seed"])
    modes = {"fp64": dict(mode=oracle_py.FP64), "fp32": dict(mode=oracle_py.FP32),
             "bf16": dict(mode=oracle_py.FP32, bf16=True)}
    for name, kw in modes.items():
        o = oracle_py.Oracle(desc, seed=fx["seed"], **kw)
        c, _ = o.run(fx["chunk"], raster_cap=1 << 20)
        assert c.sum(0).tolist() == fx[name]["chunk_counts"][0], name
    assert len(fx["fp64"]["chunk_counts"]) * fx["chunk"] == fx["steps"] == 100_000
