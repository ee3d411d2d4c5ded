"""GPU parity: the CUDA path against the FP32 oracle, bit for bit.

The device kernels and the oracle's FP32 mode perform the same IEEE-rounded
operations and accumulate synaptic increments in exact fixed point, so spike
counts, rasters and the complete neuron state must be identical -- for every
propagation mode (event-driven CSR, dense ELL), weight type, step driver and
batch layout.
"""
import numpy as np
import pytest

import oracle_py
import scaffold_gb300 as sg

pytestmark = pytest.mark.gpu


def _oracle(net, seed, steps, bf16=False, substeps=1, rates=None, raster_cap=None):
    o = oracle_py.Oracle(oracle_py.describe(net), seed=seed, bf16=bf16, substeps=substeps,
                         mode=oracle_py.FP32)
    if rates is not None:
        o.set_rates(rates)
    counts, (ids, offs) = o.run(steps, raster_cap)
    u, g, ref = o.state()
    return counts, ids, offs, u, g, ref, o.events()


def _assert_same(sim, net_counts, net_state, exp):
    counts, ids, offs = net_counts
    u, g, ref = net_state
    ecounts, eids, eoffs, eu, eg, eref, _ = exp
    assert counts.sum() > 0
    assert np.array_equal(counts, ecounts)
    assert np.array_equal(offs, eoffs)
    assert np.array_equal(ids, eids)
    assert np.array_equal(u.view(np.uint32), eu.view(np.uint32))
    assert np.array_equal(g.view(np.uint32), eg.view(np.uint32))
    assert np.array_equal(ref, eref)


@pytest.mark.parametrize("prop", [sg.PROP_CSR, sg.PROP_ELL])
@pytest.mark.parametrize("weight", [sg.WEIGHT_FP32, sg.WEIGHT_BF16])
@pytest.mark.parametrize("exec_mode", [sg.EXEC_GRAPH, sg.EXEC_STREAM, sg.EXEC_PERSISTENT])
def test_c1_quarter_bit_exact(prop, weight, exec_mode):
    net = sg.scaffold(1, 0.25, 11)
    steps = 1200
    sim = sg.Simulation([net], [11], weight_type=weight, exec_mode=exec_mode, default_prop=prop,
                        raster=True, chunk_steps=500)
    if exec_mode == sg.EXEC_PERSISTENT and prop == sg.PROP_CSR:
        # the fused kernel's split-barrier timeline by default, 128-synapse items
        assert sim.info().step_kernel == 3 and sim.info().spike_ahead == 2
        assert sim.info().item_width == 128
    counts, (ids, offs) = sim.loop_n_steps(steps, raster=True)
    exp = _oracle(net, 11, steps, bf16=weight == sg.WEIGHT_BF16)
    _assert_same(sim, (counts, ids, offs), sim.state(), exp)
    sim.close()


@pytest.mark.parametrize("exec_mode", [sg.EXEC_GRAPH, sg.EXEC_PERSISTENT])
def test_c1_full_bit_exact_mixed_modes(exec_mode):
    """Full-size config 1 (9,256 cells, 196,960 synapses), projections split
    between ELL and CSR delivery, 3,000 steps."""
    net = sg.scaffold(1, 1.0, 3)
    steps = 3000
    sim = sg.Simulation([net], [3], raster=True, exec_mode=exec_mode)
    for j, pr in enumerate(net.projections):
        sim.set_propagation(0, j, sg.PROP_ELL if j % 2 else sg.PROP_CSR)
    counts, (ids, offs) = sim.loop_n_steps(steps, raster=True)
    exp = _oracle(net, 3, steps)
    _assert_same(sim, (counts, ids, offs), sim.state(), exp)


@pytest.mark.parametrize("prop", [sg.PROP_CSR, sg.PROP_ELL])
@pytest.mark.parametrize("exec_mode", [sg.EXEC_GRAPH, sg.EXEC_PERSISTENT])
def test_large_net_general_kernels(prop, exec_mode):
    """Config 1 at 20x population size (185k cells, more 32-cell words than a
    grid of resident warps): the general persistent kernel (two barriers a
    step) or, per step, k_update + k_pull + k_deliver with the staged spike
    summary; bit-exact either way."""
    net = sg.scaffold(1, 20.0, 21)
    steps = 240
    sim = sg.Simulation([net], [21], default_prop=prop, exec_mode=exec_mode, raster=True,
                        chunk_steps=120)
    if exec_mode == sg.EXEC_PERSISTENT:
        assert sim.info().step_kernel == 1  # SGB_KERNEL_GENERAL
    counts, (ids, offs) = sim.loop_n_steps(steps, raster=True)
    exp = _oracle(net, 21, steps)
    _assert_same(sim, (counts, ids, offs), sim.state(), exp)
    if prop == sg.PROP_ELL:
        assert sim.info().pulled > 0
    sim.close()


def test_batched_instances_match_standalone():
    """Three instances of different size and seed in one handle: each equals its own oracle."""
    seeds = [5, 6, 9]
    nets = [sg.scaffold(1, s, seed) for s, seed in zip((0.2, 0.35, 0.27), seeds)]
    steps = 800
    sim = sg.Simulation(nets, seeds, weight_type=sg.WEIGHT_BF16, raster=True, chunk_steps=256,
                        exec_mode=sg.EXEC_PERSISTENT, blocks_per_sm=2)
    counts, (ids, offs) = sim.loop_n_steps(steps, raster=True)
    u, g, ref = sim.state()
    segs = sim.segments()
    base = 0
    col = 0
    for k, (net, seed) in enumerate(zip(nets, seeds)):
        npop = net.counts()["populations"]
        ncell = net.counts()["neurons"]
        ec, eids, eoffs, eu, eg, eref, _ = _oracle(net, seed, steps, bf16=True)
        assert np.array_equal(counts[:, col:col + npop], ec)
        assert segs[col].first_id == base
        # raster of instance k: ids in [base, base + ncell)
        for s in range(steps):
            mine = ids[offs[s]:offs[s + 1]]
            mine = mine[(mine >= base) & (mine < base + ncell)] - base
            assert np.array_equal(mine, eids[eoffs[s]:eoffs[s + 1]])
        assert np.array_equal(u[base:base + ncell].view(np.uint32), eu.view(np.uint32))
        assert np.array_equal(g[base:base + ncell].view(np.uint32), eg.view(np.uint32))
        assert np.array_equal(ref[base:base + ncell], eref)
        base += ncell
        col += npop


@pytest.mark.parametrize("exec_mode", [sg.EXEC_GRAPH, sg.EXEC_PERSISTENT])
def test_ten_substeps_reference_structure(exec_mode):
    """1-ms exchange steps of 10 Euler substeps (the reference's STEP_MAX=10)."""
    net = sg.scaffold(1, 0.25, 4)
    steps = 300
    sim = sg.Simulation([net], [4], substeps=10, raster=True, exec_mode=exec_mode)
    counts, (ids, offs) = sim.loop_n_steps(steps, raster=True)
    exp = _oracle(net, 4, steps, substeps=10)
    _assert_same(sim, (counts, ids, offs), sim.state(), exp)


@pytest.mark.parametrize("exec_mode", [sg.EXEC_GRAPH, sg.EXEC_PERSISTENT])
def test_rates_reset_and_periodic_input(exec_mode):
    """Rate changes between chunks, a periodic source with a repeating window
    on a third of the cells (two sources each), reset; the persistent form
    draws each step's stimulus one step ahead."""
    net = sg.Network()
    ch = [(1.0, 0.0, 1.0, 0.5), (1.0, -80.0, 1.0, 10.0)]
    mf = net.set_neuron_params("mf", 300, 0, 0, 0, 0, 0, 0, 0, sg.INPUT)
    grc = net.set_neuron_params("grc", 500, 3.0, -70.0, 2.0, 0.0, -70.0, -50.0, 0.2, sg.NORMAL, ch)
    net.add_random_projection(mf, grc, 6, 2.0, sg.CH_EXC, seed=1)
    net.add_random_projection(grc, grc, 5, 0.5, sg.CH_INH, seed=2, d_min=1, d_max=7)
    net.set_input_stim(mf, None, rate_hz=5.0)
    net.set_input_stim(mf, np.arange(0, 300, 3), kind=sg.INPUT_PERIODIC, rate_hz=140.0,
                       phase_ms=2.3, win_period_ms=50.0, win_start_ms=10.0, win_end_ms=30.0)
    sim = sg.Simulation([net], [21], raster=True, chunk_steps=128, exec_mode=exec_mode)
    o = oracle_py.Oracle(oracle_py.describe(net), seed=21)
    for rates in ([5.0, 140.0], [40.0, 90.0], [0.0, 200.0]):
        sim.set_input_freq(0, rates)
        o.set_rates(rates)
        c, (ids, offs) = sim.loop_n_steps(700, raster=True)
        ec, (eids, eoffs) = o.run(700)
        assert c.sum() > 0 and np.array_equal(c, ec) and np.array_equal(ids, eids)
    u, g, ref = sim.state()
    eu, eg, eref = o.state()
    assert np.array_equal(u.view(np.uint32), eu.view(np.uint32))
    # reset: same seed gives the same trajectory as a fresh handle
    sim.reset([21])
    sim.set_input_freq(0, [5.0, 140.0])
    c1, _ = sim.loop_n_steps(500)
    fresh = sg.Simulation([net], [21], chunk_steps=128, exec_mode=exec_mode)
    c2, _ = fresh.loop_n_steps(500)
    assert np.array_equal(c1, c2)
    assert sim.info().step == 500


def test_state_roundtrip_and_totals():
    net = sg.scaffold(1, 0.25, 2)
    sim = sg.Simulation([net], [2], chunk_steps=200)
    c, _ = sim.loop_n_steps(700)
    tot = sim.spike_totals()
    assert np.array_equal(tot, c.sum(0).astype(np.float64))
    u, g, ref = sim.state()
    assert np.isfinite(u).all() and (ref >= 0).all()
    sim.set_state(u + 0.0, g * 0.5, ref)
    u2, g2, ref2 = sim.state()
    assert np.array_equal(u2, u) and np.array_equal(g2, g * 0.5) and np.array_equal(ref2, ref)
    o = oracle_py.Oracle(oracle_py.describe(net), seed=2)
    o.run(700)
    o.set_state(u, g * 0.5, ref)
    ec, _ = o.run(300)
    c2, _ = sim.loop_n_steps(300)
    assert np.array_equal(c2, ec)


def test_launch_count_and_events():
    net = sg.scaffold(1, 0.25, 8)
    sim = sg.Simulation([net], [8], chunk_steps=100)
    before = sim.launch_count()
    sim.run(300)
    assert sim.launch_count() - before == 3 * (2 + 2 * 100)
    o = oracle_py.Oracle(oracle_py.describe(net), seed=8)
    o.run(300)
    assert sim.info().events == o.events() > 0


def test_determinism_two_runs():
    net = sg.scaffold(1, 0.5, 13)
    a = sg.Simulation([net], [13], default_prop=sg.PROP_CSR)
    b = sg.Simulation([net], [13], default_prop=sg.PROP_CSR)
    ca, _ = a.loop_n_steps(1500)
    cb, _ = b.loop_n_steps(1500)
    assert np.array_equal(ca, cb)
    ua, ga, _ = a.state()
    ub, gb, _ = b.state()
    assert np.array_equal(ga.view(np.uint32), gb.view(np.uint32))


def test_autotune_keeps_state_and_caches(tmp_path):
    """The autotuner times candidates from a snapshot and restores it: after
    tuning, the simulation continues exactly as the oracle does."""
    net = sg.scaffold(1, 0.25, 19)
    sim = sg.Simulation([net], [19], chunk_steps=250)
    o = oracle_py.Oracle(oracle_py.describe(net), seed=19)
    c0, _ = sim.loop_n_steps(300)
    e0, _ = o.run(300)
    assert np.array_equal(c0, e0)
    cache = str(tmp_path / "tune.jsonl")
    sim.autotune(200, cache)
    assert sim.info().step == 300
    modes = [sim.get_propagation(0, j) for j in range(len(net.projections))]
    assert set(modes) <= {sg.PROP_CSR, sg.PROP_ELL}
    c1, _ = sim.loop_n_steps(500)
    e1, _ = o.run(500)
    assert np.array_equal(c1, e1)
    lines = open(cache).read().splitlines()
    assert len(lines) == 1 and '"signature"' in lines[0]
    other = sg.Simulation([net], [19], chunk_steps=250)
    other.autotune(200, cache)  # served from the cache: no new line
    assert [other.get_propagation(0, j) for j in range(len(net.projections))] == modes
    assert len(open(cache).read().splitlines()) == 1


@pytest.mark.parametrize("weight", [sg.WEIGHT_FP32, sg.WEIGHT_BF16])
def test_fused_kernel_rows_partly_in_shared_memory(weight):
    """The fused persistent kernel copies each block's push rows into shared
    memory while they fit: 4,864 Poisson cells (one 32-cell word per block)
    with 1,000 synapses each need 32,000 row entries per block, more than the
    capacity, so the first rows of a word are read from shared memory and the
    rest from global memory.  Bit-exact against the oracle either way."""
    rng = np.random.default_rng(17)
    net = sg.Network()
    ch = [(1.0, 0.0, 1.0, 0.5), (1.0, -80.0, 1.0, 10.0)]
    src = net.set_neuron_params("src", 4864, 0, 0, 0, 0, 0, 0, 0, sg.INPUT)
    dst = net.set_neuron_params("dst", 2048, 3.0, -70.0, 2.0, 0.0, -70.0, -50.0, 0.2, sg.NORMAL, ch)
    fan = 1000
    pre = np.repeat(np.arange(4864, dtype=np.uint32), fan)
    post = rng.integers(0, 2048, pre.size, dtype=np.uint32)
    w = rng.uniform(0.02, 0.2, pre.size).astype(np.float32)
    d = rng.integers(1, 5, pre.size).astype(np.uint8)
    net.add_projection(src, dst, pre, post, w, d, sg.CH_EXC, sg.PROP_CSR)
    net.set_input_stim(src, rate_hz=30.0)
    steps = 300
    sim = sg.Simulation([net], [5], weight_type=weight, exec_mode=sg.EXEC_PERSISTENT,
                        raster=True, chunk_steps=150)
    info = sim.info()
    assert info.step_kernel == 3  # SGB_KERNEL_FUSED
    assert 0 < info.push_smem_bytes < 32000 * 8
    assert info.shard_cells > 0   # ~500 synapses of delay >= 3 per cell
    counts, (ids, offs) = sim.loop_n_steps(steps, raster=True)
    exp = _oracle(net, 5, steps, bf16=weight == sg.WEIGHT_BF16)
    _assert_same(sim, (counts, ids, offs), sim.state(), exp)
    assert counts[:, 1].sum() > 0
    sim.close()


@pytest.mark.parametrize("chunk", [97, 1000])
def test_config2_fused_shards_bit_exact(chunk):
    """Config 2 (92,550 cells) in the fused persistent kernel: the Golgi cells'
    1,600-synapse rows keep their delay-1 and delay-2 synapses and hand the
    rest, as 256-synapse shards, to other blocks a step or two later; short
    chunks check that every launch pushes its last step's shards before it
    ends."""
    net = sg.scaffold(2, 1.0, 3)
    steps = 400
    sim = sg.Simulation([net], [3], exec_mode=sg.EXEC_PERSISTENT, raster=True, chunk_steps=chunk)
    info = sim.info()
    assert info.step_kernel == 3 and info.shard_cells >= 200
    assert info.spike_ahead == 2  # the split-barrier timeline by default
    counts, (ids, offs) = sim.loop_n_steps(steps, raster=True)
    exp = _oracle(net, 3, steps)
    _assert_same(sim, (counts, ids, offs), sim.state(), exp)
    assert sim.info().delivered == exp[6]
    sim.close()


@pytest.mark.parametrize("delay", [1, 2, 3])
def test_fused_kernel_item_list_overflow(delay):
    """Every one of 4,864 input cells fires every step with 5,000 synapses:
    with delay 1 or 2 each block's own push items exceed its shared-memory
    list (the overflow is pushed by the warps that made it); with delay 3 the
    rows are sharded until the shard capacity runs out and the shards' items
    overflow the list too.  Bit-exact against the oracle."""
    rng = np.random.default_rng(23)
    net = sg.Network()
    ch = [(1.0, 0.0, 1.0, 0.5), (1.0, -80.0, 1.0, 10.0)]
    src = net.set_neuron_params("src", 4864, 0, 0, 0, 0, 0, 0, 0, sg.INPUT)
    dst = net.set_neuron_params("dst", 2048, 3.0, -70.0, 2.0, 0.0, -70.0, -50.0, 0.2, sg.NORMAL, ch)
    fan = 5000
    pre = np.repeat(np.arange(4864, dtype=np.uint32), fan)
    post = rng.integers(0, 2048, pre.size, dtype=np.uint32)
    w = rng.uniform(0.0001, 0.0004, pre.size).astype(np.float32)
    net.add_projection(src, dst, pre, post, w, delay, sg.CH_EXC, sg.PROP_CSR)
    net.set_input_stim(src, rate_hz=10000.0)  # fires every 0.1-ms step
    steps = 40
    sim = sg.Simulation([net], [9], exec_mode=sg.EXEC_PERSISTENT, raster=True, chunk_steps=20)
    assert sim.info().step_kernel == 3  # SGB_KERNEL_FUSED
    if delay == 3:
        assert 0 < sim.info().shard_cells < 4864
    counts, (ids, offs) = sim.loop_n_steps(steps, raster=True)
    exp = _oracle(net, 9, steps, raster_cap=1 << 20)
    _assert_same(sim, (counts, ids, offs), sim.state(), exp)
    assert counts[:, 0].sum() == 4864 * steps
    assert sim.info().delivered == exp[6]
    sim.close()


@pytest.mark.parametrize("delay", [1, 3])
def test_general_kernel_block_item_overflow(delay):
    """163,840 input cells (more 32-cell words than the grid has warps: the
    general persistent kernel, in its one-barrier form since every projection
    is event-driven) fire every step with 8 synapses each: every block makes
    more push items a step than its shared-memory list holds, and the warps
    push the rest themselves.  Bit-exact against the oracle."""
    rng = np.random.default_rng(29)
    net = sg.Network()
    ch = [(1.0, 0.0, 1.0, 0.5), (1.0, -80.0, 1.0, 10.0)]
    n_src, n_dst, fan = 163840, 4096, 8
    src = net.set_neuron_params("src", n_src, 0, 0, 0, 0, 0, 0, 0, sg.INPUT)
    dst = net.set_neuron_params("dst", n_dst, 3.0, -70.0, 2.0, 0.0, -70.0, -50.0, 0.2, sg.NORMAL, ch)
    pre = np.repeat(np.arange(n_src, dtype=np.uint32), fan)
    post = rng.integers(0, n_dst, pre.size, dtype=np.uint32)
    w = rng.uniform(0.0002, 0.0008, pre.size).astype(np.float32)
    net.add_projection(src, dst, pre, post, w, delay, sg.CH_EXC, sg.PROP_CSR)
    net.set_input_stim(src, rate_hz=10000.0)  # fires every 0.1-ms step
    steps = 20
    sim = sg.Simulation([net], [4], exec_mode=sg.EXEC_PERSISTENT, raster=True, chunk_steps=10)
    assert sim.info().step_kernel == 1  # SGB_KERNEL_GENERAL
    counts, (ids, offs) = sim.loop_n_steps(steps, raster=True, raster_cap=1 << 22)
    exp = _oracle(net, 4, steps, raster_cap=1 << 22)
    _assert_same(sim, (counts, ids, offs), sim.state(), exp)
    assert counts[:, 0].sum() == n_src * steps and counts[:, 1].sum() > 0
    assert sim.info().delivered == exp[6]
    sim.close()


@pytest.mark.parametrize("exec_mode,prop,shape", [
    (sg.EXEC_PERSISTENT, sg.PROP_CSR, [6, 2, 1, 0]),  # fused, spikes in their own step
    (sg.EXEC_PERSISTENT, sg.PROP_CSR, [6, 2, 1, 1]),  # fused, late push, 64-synapse items
    (sg.EXEC_PERSISTENT, sg.PROP_CSR, [7, 2, 1, 1]),  # fused, late push, 128-synapse items
    (sg.EXEC_PERSISTENT, sg.PROP_CSR, [6, 2, 1, 2]),  # fused, late push, split barrier
    (sg.EXEC_PERSISTENT, sg.PROP_CSR, [7, 2, 1, 2]),  # the same, 128-synapse items
    (sg.EXEC_GRAPH, None, [6, 1, 0, 1]),              # per-step kernels: 1 delivery block per SM, no summary
    (sg.EXEC_GRAPH, None, [6, 4, 1, 1]),              # k_pull: summary, four-byte entry loads
    (sg.EXEC_GRAPH, sg.PROP_ELL, [6, 2, 2, 0]),       # k_pull_vec: 16-byte entry loads
    (sg.EXEC_PERSISTENT, sg.PROP_ELL, [6, 4, 0, 1]),  # resident kernel, pulls without the summary
])
def test_cached_launch_shapes_bit_exact(tmp_path, exec_mode, prop, shape):
    """The autotuner's decisions (driver, propagation modes, launch shapes)
    are cached as one JSON line and applied as they are by a later handle; every
    launch shape it may pick gives the same bit-exact run.  The line is written
    by a first tuning run and then edited to the combination under test."""
    import json

    net = sg.scaffold(2, 1.0, 3)
    cache = str(tmp_path / "tune.jsonl")
    first = sg.Simulation([net], [3], chunk_steps=100)
    first.autotune(20, cache)
    first.close()
    line = json.loads(open(cache).read().splitlines()[0])
    n = len(net.projections)
    line["exec_mode"] = exec_mode
    line["modes"] = [prop if prop is not None else (sg.PROP_ELL if j % 2 else sg.PROP_CSR)
                     for j in range(n)]
    line["shape"] = shape
    with open(cache, "w") as f:
        f.write(json.dumps(line) + "\n")
    sim = sg.Simulation([net], [3], raster=True, chunk_steps=100)
    sim.autotune(20, cache)  # served from the cache
    info = sim.info()
    assert info.exec_mode == exec_mode
    assert info.item_width == 1 << shape[0]
    assert info.deliver_blocks % shape[1] == 0 and info.pull_summary == shape[2]
    if exec_mode == sg.EXEC_PERSISTENT:
        assert info.step_kernel == (3 if prop == sg.PROP_CSR else 2)
        assert info.spike_ahead == (shape[3] if prop == sg.PROP_CSR else 0)
    steps = 300
    counts, (ids, offs) = sim.loop_n_steps(steps, raster=True)
    exp = _oracle(net, 3, steps)
    _assert_same(sim, (counts, ids, offs), sim.state(), exp)
    sim.close()


@pytest.mark.parametrize("shape", [None, [6, 2, 1, 1], [6, 2, 1, 0]])
def test_fused_timelines_hand_over_to_dense_pulls(tmp_path, shape):
    """Every fused-kernel timeline ends a launch in the state the other kernels
    expect: full config 1 runs 700 steps all event-driven (fused kernel;
    default timeline, late push, or spikes in their own step), then every
    other projection pulls densely for 600 steps (the resident kernel reads
    the spike history and summary rows the fused launches left), then all
    push again for 300 steps.  Counts, rasters and the final state against
    one 1,600-step oracle run."""
    import json

    net = sg.scaffold(1, 1.0, 5)
    n = len(net.projections)
    kw = dict(raster=True, chunk_steps=250, exec_mode=sg.EXEC_PERSISTENT,
              default_prop=sg.PROP_CSR)
    if shape is None:
        sim = sg.Simulation([net], [5], **kw)
    else:
        cache = str(tmp_path / "tune.jsonl")
        first = sg.Simulation([net], [5], chunk_steps=250, exec_mode=sg.EXEC_PERSISTENT)
        first.autotune(20, cache)
        first.close()
        line = json.loads(open(cache).read().splitlines()[0])
        line.update(exec_mode=sg.EXEC_PERSISTENT, modes=[sg.PROP_CSR] * n, shape=shape)
        with open(cache, "w") as f:
            f.write(json.dumps(line) + "\n")
        sim = sg.Simulation([net], [5], **kw)
        sim.autotune(20, cache)
    assert sim.info().step_kernel == 3
    assert sim.info().spike_ahead == (2 if shape is None else shape[3])
    exp = _oracle(net, 5, 1600)
    ecounts, eids, eoffs = exp[0], exp[1], exp[2]
    s0 = 0
    for steps, ell in ((700, False), (600, True), (300, False)):
        for j in range(n):
            sim.set_propagation(0, j, sg.PROP_ELL if ell and j % 2 else sg.PROP_CSR)
        assert sim.info().step_kernel == (2 if ell else 3)
        counts, (ids, offs) = sim.loop_n_steps(steps, raster=True)
        s1 = s0 + steps
        bad = np.nonzero((counts != ecounts[s0:s1]).any(1))[0]
        assert bad.size == 0, f"segment from step {s0}: first divergent step {s0 + bad[0]}"
        assert np.array_equal(offs, eoffs[s0:s1 + 1] - eoffs[s0])
        assert np.array_equal(ids, eids[eoffs[s0]:eoffs[s1]])
        s0 = s1
    u, g, ref = sim.state()
    assert np.array_equal(u.view(np.uint32), exp[3].view(np.uint32))
    assert np.array_equal(g.view(np.uint32), exp[4].view(np.uint32))
    assert np.array_equal(ref, exp[5])
    sim.close()
