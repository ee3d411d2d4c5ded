"""Synaptic plasticity (STDP): the reference's Hebb / Teacher rules
(SynapticPlasticity.cu:40-120), switched off in the reference and without a
test there, so the oracle's restatement is checked here against a hand
computation, and the CUDA path against the oracle bit for bit.
"""
import numpy as np
import pytest

import oracle_py
import scaffold_gb300 as sg

CH = [(1.0, 0.0, 1.0, 0.5), (1.0, -80.0, 1.0, 10.0)]


def _pair_net(delay=2, a1_j=-0.01, a2_ji=0.0, a1_i=0.0, window=0, post_silent=True):
    """4 Poisson cells -> 2 LIF cells, all-to-all, one delay, Hebb rule."""
    net = sg.Network()
    src = net.set_neuron_params("src", 4, 0, 0, 0, 0, 0, 0, 0, sg.INPUT)
    vth = 1e6 if post_silent else -50.0
    dst = net.set_neuron_params("dst", 2, 3.0, -70.0, 2.0, 0.0, -70.0, vth, 0.2, sg.NORMAL, CH)
    pre = np.repeat(np.arange(4), 2)
    post = np.tile(np.arange(2), 4)
    net.add_projection(src, dst, pre, post, np.full(8, 0.01 if post_silent else 3.0), delay,
                       sg.CH_EXC)
    net.set_input_stim(src, rate_hz=800.0)
    net.add_plasticity(0, sg.STDP_HEBB, window=window, a1_j=a1_j, a1_i=a1_i, a2_ji=a2_ji)
    return net


def test_oracle_hebb_pre_term_by_hand():
    """v_q = 1 + a1_j per spike of q's pre cell at t - d, summed in FP32 in step order."""
    net, d, steps = _pair_net(delay=2), 2, 300
    o = oracle_py.Oracle(oracle_py.describe(net), seed=5)
    counts, (ids, offs) = o.run(steps)
    v = o.plastic_values(0)
    spikes = np.zeros((steps, 4), bool)
    for t in range(steps):
        for g in ids[offs[t]:offs[t + 1]]:
            if g < 4:
                spikes[t, g] = True
    pre, _, _, _ = net.synapses(0)
    for q in range(8):
        x = np.float32(1.0)
        for t in range(steps):
            if t - d >= 0 and spikes[t - d, pre[q]]:
                dw = np.float32(np.float32(0.0) + np.float32(0.0)) + np.float32(-0.01)  # (0 + a0) + a1_j
                x = np.float32(max(np.float32(0.0), np.float32(x + dw)))
        assert v[q] == x
    assert (v < 1).all() and spikes.sum() > 20


def test_oracle_hebb_window_and_post_terms():
    """Post cells that spike: each post spike adds a1_i plus a2_ji per pre spike
    in the window; values stay within [0, v_max]."""
    net = _pair_net(delay=1, a1_j=0.0, a1_i=0.002, a2_ji=-0.003, window=6, post_silent=False)
    o = oracle_py.Oracle(oracle_py.describe(net), seed=9)
    counts, _ = o.run(400)
    v = o.plastic_values(0)
    assert counts[:, 1].sum() > 0          # the post cells fire
    assert (v >= 0).all() and (v <= 1).all() and (v != 1).any()


def test_plasticity_api_validation():
    net = sg.scaffold(1, 0.1, 3)
    with pytest.raises(sg.SgbError):
        net.add_plasticity(6, sg.STDP_HEBB, v_max=1.5)
    with pytest.raises(sg.SgbError):
        net.add_plasticity(6, sg.STDP_HEBB, window=65)
    with pytest.raises(sg.SgbError):     # teacher must target the same post population
        net.add_plasticity(6, sg.STDP_TEACHER, teacher=2)
    net.add_plasticity(6, sg.STDP_TEACHER, teacher=8, a2_ji=-0.01)
    q = net.plasticity(6)
    assert q["rule"] == sg.STDP_TEACHER and q["teacher"] == 8 and q["window"] == 50
    assert net.plasticity(5) is None
    assert net.projections[6].mode == sg.PROP_ELL
    with pytest.raises(sg.SgbError):
        net.add_plasticity(6, sg.STDP_HEBB)


def _plastic_c1(seed):
    net = sg.scaffold(1, 0.25, seed)
    net.add_plasticity(2, sg.STDP_HEBB, window=8, a0=-1e-5, a1_j=-0.002, a1_i=0.01,
                       a2_ji=0.001)
    net.add_plasticity(6, sg.STDP_TEACHER, teacher=8, window=20, a1_j=0.0005, a2_ji=-0.004)
    return net


@pytest.mark.gpu
@pytest.mark.parametrize("weight", [sg.WEIGHT_FP32, sg.WEIGHT_BF16])
@pytest.mark.parametrize("exec_mode", [sg.EXEC_GRAPH, sg.EXEC_STREAM, sg.EXEC_PERSISTENT])
def test_gpu_plasticity_bit_exact(weight, exec_mode):
    """Hebb on granule->Golgi, Teacher (basket cells as teachers) on
    granule->Purkinje: counts, rasters, cell state and every synapse's value
    equal the FP32 oracle's (per-step kernels, or the persistent kernel's
    plasticity phase between its update and delivery phases)."""
    net = _plastic_c1(11)
    steps = 800
    sim = sg.Simulation([net], [11], weight_type=weight, exec_mode=exec_mode, raster=True,
                        chunk_steps=200)
    counts, (ids, offs) = sim.loop_n_steps(steps, raster=True)
    o = oracle_py.Oracle(oracle_py.describe(net), seed=11, bf16=weight == sg.WEIGHT_BF16)
    ec, (eids, eoffs) = o.run(steps)
    assert np.array_equal(counts, ec) and np.array_equal(offs, eoffs)
    assert np.array_equal(ids, eids)
    u, g, ref = sim.state()
    eu, eg, eref = o.state()
    assert np.array_equal(u.view(np.uint32), eu.view(np.uint32))
    assert np.array_equal(g.view(np.uint32), eg.view(np.uint32))
    assert np.array_equal(ref, eref)
    for j in (2, 6):
        v, ev = sim.plastic_values(0, j), o.plastic_values(j)
        assert np.array_equal(v.view(np.uint32), ev.view(np.uint32))
        assert (v != 1).any()
    sim.close()


@pytest.mark.gpu
def test_gpu_plasticity_limits_and_reset():
    net = _plastic_c1(4)
    sim = sg.Simulation([net], [4])
    with pytest.raises(sg.SgbError):
        sim.set_propagation(0, 2, sg.PROP_CSR)
    with pytest.raises(sg.SgbError):
        sim.autotune(50)
    c1, _ = sim.loop_n_steps(300)
    assert (sim.plastic_values(0, 6) != 1).any()
    sim.reset()
    assert (sim.plastic_values(0, 6) == 1).all()
    c2, _ = sim.loop_n_steps(300)
    assert np.array_equal(c1, c2)
    sim.close()


@pytest.mark.gpu
def test_gpu_plasticity_general_persistent_kernel():
    """A network with more 32-cell words than the grid has warps runs the
    general persistent kernel (two grid barriers a step, three with the
    plasticity phase); plastic values and spikes match the oracle."""
    net = sg.scaffold(1, 20.0, 21)
    net.add_plasticity(6, sg.STDP_TEACHER, teacher=8, window=20, a1_j=0.0005, a2_ji=-0.004)
    sim = sg.Simulation([net], [21], exec_mode=sg.EXEC_PERSISTENT, chunk_steps=120)
    assert sim.info().step_kernel == 1  # SGB_KERNEL_GENERAL
    c, _ = sim.loop_n_steps(240)
    o = oracle_py.Oracle(oracle_py.describe(net), seed=21)
    ec, _ = o.run(240)
    assert np.array_equal(c, ec)
    v, ev = sim.plastic_values(0, 6), o.plastic_values(6)
    assert np.array_equal(v.view(np.uint32), ev.view(np.uint32))
    assert (v != 1).any()
    u, g, ref = sim.state()
    eu, eg, eref = o.state()
    assert np.array_equal(u.view(np.uint32), eu.view(np.uint32))
    sim.close()


@pytest.mark.gpu
@pytest.mark.parametrize("window", [40, 64])
def test_gpu_plasticity_window_sources(window):
    """Windows ending within 64 steps are counted from the per-cell spike
    registers, longer ones (window 64 with any delay) from the spike history;
    both agree with the oracle bit for bit."""
    net = sg.scaffold(1, 0.25, 7)
    net.add_plasticity(2, sg.STDP_HEBB, window=window, a1_i=0.001, a2_ji=-0.003)
    sim = sg.Simulation([net], [7], chunk_steps=150)
    c, _ = sim.loop_n_steps(450)
    o = oracle_py.Oracle(oracle_py.describe(net), seed=7)
    ec, _ = o.run(450)
    assert np.array_equal(c, ec)
    v, ev = sim.plastic_values(0, 2), o.plastic_values(2)
    assert np.array_equal(v.view(np.uint32), ev.view(np.uint32))
    assert (v != 1).any()
    sim.close()


@pytest.mark.gpu
@pytest.mark.parametrize("window", [40, 64])
@pytest.mark.parametrize("weight", [sg.WEIGHT_FP32, sg.WEIGHT_BF16])
@pytest.mark.parametrize("exec_mode", [sg.EXEC_PERSISTENT, sg.EXEC_GRAPH, sg.EXEC_STREAM])
def test_gpu_teacher_rule_in_update_phase(window, weight, exec_mode):
    """The Teacher rule reads only earlier steps' spikes (the teacher's at t -
    its delay, the pre cells' at t - d - j), so it runs beside the step's
    update: in the persistent kernels' update phase, and with the per-step
    drivers as k_stdp on a forked stream concurrent with k_update (reading the
    previous step's spike registers, window 40, or the history, window 64);
    bit-exact against the oracle."""
    net = sg.scaffold(1, 0.25, 13)
    net.add_plasticity(6, sg.STDP_TEACHER, teacher=8, window=window, a1_j=0.0007, a2_ji=-0.003)
    sim = sg.Simulation([net], [13], exec_mode=exec_mode, weight_type=weight,
                        raster=True, chunk_steps=170)
    counts, (ids, offs) = sim.loop_n_steps(600, raster=True)
    o = oracle_py.Oracle(oracle_py.describe(net), seed=13, bf16=weight == sg.WEIGHT_BF16)
    ec, (eids, eoffs) = o.run(600)
    assert np.array_equal(counts, ec) and np.array_equal(ids, eids)
    v, ev = sim.plastic_values(0, 6), o.plastic_values(6)
    assert np.array_equal(v.view(np.uint32), ev.view(np.uint32))
    assert (v != 1).any()
    u, g, ref = sim.state()
    eu, eg, eref = o.state()
    assert np.array_equal(u.view(np.uint32), eu.view(np.uint32))
    assert np.array_equal(g.view(np.uint32), eg.view(np.uint32))
    sim.close()


@pytest.mark.gpu
def test_gpu_plasticity_start_value_and_sparse_rule():
    """Values start at v_max; with a0 = a1_j = 0 (the reference's Teacher
    coefficients) only rows of posts whose teacher fired change, and the
    kernel's skipping of the rest is bit-exact."""
    net = sg.scaffold(1, 0.25, 4)
    net.add_plasticity(6, sg.STDP_TEACHER, teacher=8, window=20, a2_ji=-0.004, v_max=0.75)
    sim = sg.Simulation([net], [4])
    c, _ = sim.loop_n_steps(400)
    o = oracle_py.Oracle(oracle_py.describe(net), seed=4)
    ec, _ = o.run(400)
    assert np.array_equal(c, ec)
    v, ev = sim.plastic_values(0, 6), o.plastic_values(6)
    assert np.array_equal(v.view(np.uint32), ev.view(np.uint32))
    assert v.max() == np.float32(0.75) and v.min() < np.float32(0.75)
    sim.close()
