"""GPU parity at the benchmark configurations, against the FP32 oracle.

The same bit-exact bar as tests/test_gpu_parity.py (spike counts, rasters,
complete neuron state), on the networks the benchmark times:

  * config 2 (92,550 cells) with every projection delivered by dense pull --
    the parallel-fibre -> Purkinje projection has in-degree 25,000, the regime
    of the reference's spike_propagation_PR (Simulation_header.cu:153-303) --
    in FP32 and BF16, through the persistent kernel and the per-step kernels;
  * config 2 with BF16 tables through the fused persistent kernel (config 3);
  * config 4: 64 instances of config 2 scaled U[0.25, 2.0], BF16, one
    persistent launch per chunk; a spread of instances (first, last,
    smallest, largest and four more) each against its own oracle run;
  * one config-5 instance (925,500 cells) after the autotuner has picked each
    projection's propagation mode;
  * 250 small batched instances whose segment descriptors exceed shared
    memory, a subset against the oracle.
"""
import numpy as np
import pytest

import oracle_py
import scaffold_gb300 as sg

pytestmark = pytest.mark.gpu


def _oracle(net, seed, steps, bf16=False, raster_cap=1 << 22):
    o = oracle_py.Oracle(oracle_py.describe(net), seed=seed, bf16=bf16, mode=oracle_py.FP32)
    counts, (ids, offs) = o.run(steps, raster_cap)
    u, g, ref = o.state()
    return counts, ids, offs, u, g, ref, o.events()


def _step_of(offs):
    return np.repeat(np.arange(len(offs) - 1), np.diff(offs))


def _assert_instance(k, nets, seeds, counts, ids, offs, state, steps, bf16):
    """Instance k of a batched run equals its own oracle run: its columns of
    the per-step counts, its part of the raster and its slice of the state."""
    base = sum(n.counts()["neurons"] for n in nets[:k])
    col = sum(n.counts()["populations"] for n in nets[:k])
    net = nets[k]
    npop, ncell = net.counts()["populations"], net.counts()["neurons"]
    ec, eids, eoffs, eu, eg, eref, _ = _oracle(net, seeds[k], steps, bf16=bf16)
    assert np.array_equal(counts[:, col:col + npop], ec), f"instance {k}: counts"
    sel = (ids >= base) & (ids < base + ncell)
    st = _step_of(offs)
    assert np.array_equal(st[sel], _step_of(eoffs)), f"instance {k}: raster steps"
    assert np.array_equal(ids[sel] - base, eids), f"instance {k}: raster ids"
    u, g, ref = state
    assert np.array_equal(u[base:base + ncell].view(np.uint32), eu.view(np.uint32))
    assert np.array_equal(g[base:base + ncell].view(np.uint32), eg.view(np.uint32))
    assert np.array_equal(ref[base:base + ncell], eref)
    return int(ec.sum())


def _with_shape(nets, seeds, shape, modes, exec_mode, tmp_path, **kw):
    """A handle whose driver, propagation modes and launch shape are the
    given ones: a first handle tunes briefly to write the cache line for
    this network, the line is edited, and a second handle serves from it."""
    import json

    cache = str(tmp_path / "tune.jsonl")
    first = sg.Simulation(nets, seeds, **kw)
    first.autotune(5, cache)
    first.close()
    line = json.loads(open(cache).read().splitlines()[0])
    line.update(exec_mode=exec_mode, modes=modes, shape=shape)
    with open(cache, "w") as f:
        f.write(json.dumps(line) + "\n")
    sim = sg.Simulation(nets, seeds, **kw)
    sim.autotune(5, cache)
    return sim


def _assert_same(counts, ids, offs, state, exp):
    ecounts, eids, eoffs, eu, eg, eref, _ = exp
    u, g, ref = state
    assert counts.sum() > 0
    assert np.array_equal(counts, ecounts)
    assert np.array_equal(offs, eoffs)
    assert np.array_equal(ids, eids)
    assert np.array_equal(u.view(np.uint32), eu.view(np.uint32))
    assert np.array_equal(g.view(np.uint32), eg.view(np.uint32))
    assert np.array_equal(ref, eref)


def test_config5x4_dense_pull_vec(tmp_path):
    """Config 5 with 4 seeds (3.7M cells, 109M synapses), every projection
    pulled densely by the per-step kernels with 16-byte entry loads
    (k_pull_vec): two instances against their own oracle runs."""
    seeds = [1, 2, 3, 4]
    nets = [sg.scaffold(5, 1.0, sd) for sd in seeds]
    steps = 60
    sim = _with_shape(nets, seeds, [6, 2, 2, 0, 2],
                      [sg.PROP_ELL] * sum(len(n.projections) for n in nets), sg.EXEC_GRAPH,
                      tmp_path, weight_type=sg.WEIGHT_BF16, raster=True, chunk_steps=60)
    assert sim.info().pull_summary == 2
    counts, (ids, offs) = sim.loop_n_steps(steps, raster=True, raster_cap=1 << 22)
    state = sim.state()
    spikes = sum(_assert_instance(k, nets, seeds, counts, ids, offs, state, steps, True)
                 for k in (0, 3))
    assert spikes > 0 and sim.info().pulled > 0
    sim.close()


@pytest.mark.parametrize("weight", [sg.WEIGHT_FP32, sg.WEIGHT_BF16])
@pytest.mark.parametrize("exec_mode", [sg.EXEC_PERSISTENT, sg.EXEC_GRAPH])
def test_config2_dense_pull_in_degree_25000(weight, exec_mode):
    net = sg.scaffold(2, 1.0, 3)
    pf_pc = [p for p in net.projections if p.name == "granule_to_purkinje"][0]
    assert pf_pc.max_in_degree == 25000
    steps = 320
    sim = sg.Simulation([net], [3], weight_type=weight, exec_mode=exec_mode,
                        default_prop=sg.PROP_ELL, raster=True, chunk_steps=160)
    assert all(sim.get_propagation(0, j) == sg.PROP_ELL for j in range(len(net.projections)))
    if exec_mode == sg.EXEC_PERSISTENT:
        assert sim.info().step_kernel == 2  # SGB_KERNEL_RESIDENT: dense pulls need two barriers
    counts, (ids, offs) = sim.loop_n_steps(steps, raster=True)
    exp = _oracle(net, 3, steps, bf16=weight == sg.WEIGHT_BF16)
    _assert_same(counts, ids, offs, sim.state(), exp)
    info = sim.info()
    assert info.pull_entries >= 2731520 and info.pulled > 0
    assert counts[:, 5].sum() > 0  # Purkinje cells fire from their 25,000-entry pulls
    sim.close()


def test_config3_bf16_push_fused():
    net = sg.scaffold(2, 1.0, 5)
    steps = 400
    sim = sg.Simulation([net], [5], weight_type=sg.WEIGHT_BF16, exec_mode=sg.EXEC_PERSISTENT,
                        raster=True, chunk_steps=1000)
    assert sim.info().step_kernel == 3  # SGB_KERNEL_FUSED
    counts, (ids, offs) = sim.loop_n_steps(steps, raster=True)
    exp = _oracle(net, 5, steps, bf16=True)
    _assert_same(counts, ids, offs, sim.state(), exp)
    assert sim.info().delivered == exp[6]
    sim.close()


@pytest.mark.parametrize("lane_cells", [1, 2])
def test_config4_batch_of_64_scaled_instances(tmp_path, lane_cells):
    """lane_cells 2: the general kernel's two-cells-per-lane update."""
    seeds = [1 + k for k in range(64)]
    scales = sg.batched_scales(seeds)
    nets = [sg.scaffold(2, sc, sd) for sc, sd in zip(scales, seeds)]
    steps = 200
    sim = _with_shape(nets, seeds, [6, 2, 1, 0, lane_cells],
                      [sg.PROP_CSR] * sum(len(n.projections) for n in nets), sg.EXEC_PERSISTENT,
                      tmp_path, weight_type=sg.WEIGHT_BF16, raster=True, chunk_steps=100)
    info = sim.info()
    assert info.step_kernel == 1  # SGB_KERNEL_GENERAL: more words than resident warps
    assert info.lane_cells == lane_cells
    assert info.n_synapses > 150_000_000
    counts, (ids, offs) = sim.loop_n_steps(steps, raster=True, raster_cap=1 << 24)
    state = sim.state()
    check = sorted({0, 63, int(np.argmin(scales)), int(np.argmax(scales)), 17, 31, 42, 50})
    spikes = 0
    for k in check:
        spikes += _assert_instance(k, nets, seeds, counts, ids, offs, state, steps, True)
    assert spikes > 0
    sim.close()


def test_config5_instance_after_autotune():
    net = sg.scaffold(5, 1.0, 2)
    steps = 200
    sim = sg.Simulation([net], [2], weight_type=sg.WEIGHT_BF16, exec_mode=sg.EXEC_PERSISTENT,
                        raster=True, chunk_steps=100)
    sim.autotune(100)
    assert sim.info().step == 0  # candidates are timed from a snapshot that is restored
    modes = [sim.get_propagation(0, j) for j in range(len(net.projections))]
    assert set(modes) <= {sg.PROP_CSR, sg.PROP_ELL}
    counts, (ids, offs) = sim.loop_n_steps(steps, raster=True, raster_cap=1 << 22)
    exp = _oracle(net, 2, steps, bf16=True)
    _assert_same(counts, ids, offs, sim.state(), exp)
    sim.close()


def test_config5_mixed_modes_general_kernel():
    """Config 5 with the parallel-fibre projections (in-degrees 25,000, 400 and
    100) pulled densely and the rest pushed: the general persistent kernel's
    two-barrier form at 925,500 cells."""
    net = sg.scaffold(5, 1.0, 4)
    steps = 120
    sim = sg.Simulation([net], [4], weight_type=sg.WEIGHT_BF16, exec_mode=sg.EXEC_PERSISTENT,
                        raster=True, chunk_steps=60)
    for j, p in enumerate(net.projections):
        sim.set_propagation(0, j, sg.PROP_ELL if p.pre == 1 else sg.PROP_CSR)
    assert sim.info().step_kernel == 1
    counts, (ids, offs) = sim.loop_n_steps(steps, raster=True, raster_cap=1 << 22)
    exp = _oracle(net, 4, steps, bf16=True)
    _assert_same(counts, ids, offs, sim.state(), exp)
    assert sim.info().pulled > 0
    sim.close()


def test_many_segments_against_the_oracle():
    """250 batched instances (1,750 segments): the persistent kernels' copy of
    the segment descriptors no longer fits in shared memory, so the general
    kernel reads them from global memory; instances spread over the batch
    each equal their own oracle run."""
    seeds = list(range(1, 251))
    nets = [sg.scaffold(1, 0.1, sd) for sd in seeds]
    steps = 120
    sim = sg.Simulation(nets, seeds, exec_mode=sg.EXEC_PERSISTENT, raster=True, chunk_steps=60)
    assert sim.info().step_kernel == 1  # SGB_KERNEL_GENERAL
    counts, (ids, offs) = sim.loop_n_steps(steps, raster=True, raster_cap=1 << 22)
    state = sim.state()
    spikes = 0
    for k in (0, 1, 77, 124, 125, 200, 248, 249):
        spikes += _assert_instance(k, nets, seeds, counts, ids, offs, state, steps, False)
    assert spikes > 0
    sim.close()


@pytest.mark.parametrize("weight,lane_cells", [(sg.WEIGHT_FP32, 2), (sg.WEIGHT_BF16, 2)])
def test_two_cells_per_lane_general_kernel(tmp_path, weight, lane_cells):
    """Config 1 at 20x (185,120 cells; its DCN segment is five words long, so
    pairs of words straddle segment ends and a warp's two halves run different
    segments, even an input and a LIF segment) plus a second, smaller
    instance, through the general kernel with two cells per lane."""
    nets = [sg.scaffold(1, 20.0, 21), sg.scaffold(1, 3.3, 22)]
    seeds = [21, 22]
    steps = 240
    sim = _with_shape(nets, seeds, [6, 2, 1, 0, lane_cells],
                      [sg.PROP_CSR] * sum(len(n.projections) for n in nets), sg.EXEC_PERSISTENT,
                      tmp_path, weight_type=weight, raster=True, chunk_steps=120)
    info = sim.info()
    assert info.step_kernel == 1 and info.lane_cells == lane_cells
    counts, (ids, offs) = sim.loop_n_steps(steps, raster=True, raster_cap=1 << 22)
    state = sim.state()
    spikes = 0
    for k in range(2):
        spikes += _assert_instance(k, nets, seeds, counts, ids, offs, state, steps,
                                   weight == sg.WEIGHT_BF16)
    assert spikes > 0
    assert sim.info().delivered > 0
    sim.close()
