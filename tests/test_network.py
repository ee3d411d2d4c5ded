"""Host-side network description through the C ABI (no GPU needed).

Mirrors the reference's loaders: set_neuron_params (init_params.cu:255),
set_connectivity_params + LoadConnectivityFile_ELL (:304, :13) on the
"pre post" .dat format, setInputStim's one-id-per-line lists
(UserInputFunctions.cu:41), plus the synthetic fixed in-degree generator.
"""
import numpy as np
import pytest

import scaffold_gb300 as sg
from scaffold_gb300 import SgbError

CH = [(1.0, 0.0, 1.0, 0.5), (1.0, -80.0, 1.0, 10.0)]


def _two_pops(npre=50, npost=40):
    net = sg.Network()
    a = net.set_neuron_params("a", npre, 3.0, -70.0, 2.0, 0.0, -70.0, -50.0, 0.2, sg.NORMAL, CH)
    b = net.set_neuron_params("b", npost, 3.0, -70.0, 2.0, 0.0, -70.0, -50.0, 0.2, sg.OUTPUT, CH)
    return net, a, b


def test_population_validation():
    net = sg.Network()
    with pytest.raises(SgbError) as e:
        net.set_neuron_params("x", 10, 3.0, -70, 2, 0, -70, -50, 0.2, sg.NORMAL,
                              [(1, 0, 1, 0.5)] * 3)
    assert e.value.code == -10  # more than 2 channels
    with pytest.raises(SgbError):
        net.set_neuron_params("x", -1, 3.0, -70, 2, 0, -70, -50, 0.2, sg.NORMAL, CH)
    with pytest.raises(SgbError):
        net.set_neuron_params("x", 10, 0, 0, 0, 0, 0, 0, 0, sg.INPUT, CH)  # INPUT takes none
    with pytest.raises(SgbError):
        net.set_neuron_params("x", 10, 3.0, -70, 2, 0, -70, -50, 0.2, sg.NORMAL,
                              [(1, 0, 1, 0.0)])  # tau must be > 0
    p = net.set_neuron_params("mf", 7, 0, 0, 0, 0, 0, 0, 0, sg.INPUT)
    assert net.populations[p].dev_type == sg.INPUT and net.populations[p].num == 7


def test_dat_roundtrip(tmp_path):
    net, a, b = _two_pops()
    j = net.add_random_projection(a, b, 6, 1.0, sg.CH_EXC, seed=5, d_min=3, d_max=3)
    path = str(tmp_path / "a_to_b.dat")
    net.write_projection_dat(j, path)
    lines = open(path).read().splitlines()
    pairs = [tuple(map(int, l.split("\t"))) for l in lines]
    assert pairs == sorted(pairs, key=lambda x: (x[1], x[0]))  # by post, then pre
    k = net.set_connectivity_params(path, a, b, -2.5, 3)
    pre0, post0, _, _ = net.synapses(j)
    pre1, post1, w1, d1 = net.synapses(k)
    assert sorted(zip(pre0, post0)) == sorted(zip(pre1, post1))
    assert (w1 == 2.5).all() and (d1 == 3).all()
    assert net.projections[k].channel == sg.CH_INH  # negative weight -> dg_inh
    assert net.projections[k].name == "a_to_b"


def test_dat_errors(tmp_path):
    net, a, b = _two_pops(10, 10)
    with pytest.raises(SgbError) as e:
        net.set_connectivity_params(str(tmp_path / "missing.dat"), a, b, 1.0, 1)
    assert e.value.code == -2
    bad = tmp_path / "bad.dat"
    bad.write_text("1\t2\n3 x\n")
    with pytest.raises(SgbError) as e:
        net.set_connectivity_params(str(bad), a, b, 1.0, 1)
    assert e.value.code == -3 and ":2:" in str(e.value)
    rng = tmp_path / "range.dat"
    rng.write_text("1 2\n10 3\n")
    with pytest.raises(SgbError) as e:
        net.set_connectivity_params(str(rng), a, b, 1.0, 1)
    assert e.value.code == -4
    ok = tmp_path / "ok.dat"
    ok.write_text("1\t2\r\n\n  3 4\n")
    k = net.set_connectivity_params(str(ok), a, b, 1.0, 2)
    pre, post, _, _ = net.synapses(k)
    assert list(pre) == [1, 3] and list(post) == [2, 4]
    with pytest.raises(SgbError):
        net.set_connectivity_params(str(ok), a, b, 1.0, 16)  # delay beyond 15 steps
    empty = tmp_path / "empty.dat"
    empty.write_text("")
    k = net.set_connectivity_params(str(empty), a, b, 1.0, 1)
    assert net.projections[k].n_synapses == 0


def test_projection_arrays_validation():
    net, a, b = _two_pops(10, 10)
    with pytest.raises(SgbError) as e:
        net.add_projection(a, b, [0, 11], [0, 1], [1.0, 1.0], 1, sg.CH_EXC)
    assert e.value.code == -4
    with pytest.raises(SgbError):
        net.add_projection(a, b, [0], [0], [-1.0], 1, sg.CH_EXC)  # magnitudes only
    with pytest.raises(SgbError):
        net.add_projection(a, b, [0], [0], [1.0], [0], sg.CH_EXC)  # delay 0
    mf = net.set_neuron_params("mf", 5, 0, 0, 0, 0, 0, 0, 0, sg.INPUT)
    with pytest.raises(SgbError):
        net.add_projection(a, mf, [0], [0], [1.0], 1, sg.CH_EXC)  # onto an INPUT population
    k = net.add_projection(a, b, [1, 2, 3], [0, 0, 9], [0.5, 1.5, 2.0], [1, 2, 15], sg.CH_INH)
    info = net.projections[k]
    assert (info.min_delay, info.max_delay, info.max_in_degree) == (1, 15, 2)


def test_random_projection_properties():
    net, a, b = _two_pops(300, 200)
    k = net.add_random_projection(a, b, 25, 2.0, sg.CH_EXC, seed=9, d_min=1, d_max=4)
    pre, post, w, d = net.synapses(k)
    assert len(pre) == 25 * 200
    for p in range(200):
        sel = pre[post == p]
        assert len(sel) == 25 and len(np.unique(sel)) == 25  # distinct pres
    assert w.min() >= 1.0 and w.max() < 3.0  # [0.5, 1.5) x 2.0
    assert set(np.unique(d)) == {1, 2, 3, 4}
    k2 = net.add_random_projection(a, b, 25, 2.0, sg.CH_EXC, seed=9)
    assert all(np.array_equal(x, y) for x, y in zip(net.synapses(k), net.synapses(k2)))
    k3 = net.add_random_projection(a, b, 25, 2.0, sg.CH_EXC, seed=10)
    assert not np.array_equal(net.synapses(k)[0], net.synapses(k3)[0])
    # uniform pre choice: every pre is used about 25*200/300 ~ 16.7 times
    hist = np.bincount(pre, minlength=300)
    assert 8 < hist.mean() < 25 and hist.max() < 45
    with pytest.raises(SgbError):
        net.add_random_projection(a, b, 301, 1.0, sg.CH_EXC, seed=1)  # more than npre
    k4 = net.add_random_projection(a, b, 300, 1.0, sg.CH_EXC, seed=1)  # dense: all pres
    pre4, post4, _, _ = net.synapses(k4)
    assert all(np.array_equal(np.sort(pre4[post4 == p]), np.arange(300)) for p in (0, 77, 199))


def test_input_sources(tmp_path):
    net = sg.Network()
    mf = net.set_neuron_params("mf", 20, 0, 0, 0, 0, 0, 0, 0, sg.INPUT)
    s0 = net.set_input_stim(mf, None, rate_hz=4.0)
    f = tmp_path / "tone_stim.dat"
    f.write_text("3\n1\n3\n7\n")
    s1 = net.set_input_stim(mf, filename=str(f), kind=sg.INPUT_PERIODIC, rate_hz=140.0,
                            phase_ms=292.8, win_start_ms=300.0, win_end_ms=351.0)
    ins = net.inputs()
    assert list(ins[s0][2]) == list(range(20))
    assert list(ins[s1][2]) == [1, 3, 7]  # sorted, unique
    assert ins[s1][1]["kind"] == sg.INPUT_PERIODIC and ins[s1][1]["win_end_ms"] == 351.0
    with pytest.raises(SgbError):
        net.set_input_stim(mf, [20])
    g = net.set_neuron_params("g", 5, 3.0, -70, 2, 0, -70, -50, 0.2, sg.NORMAL, CH)
    with pytest.raises(SgbError):
        net.set_input_stim(g, None)  # not an INPUT population
    bad = tmp_path / "bad_ids.dat"
    bad.write_text("1\n-4\n")
    with pytest.raises(SgbError) as e:
        net.set_input_stim(mf, filename=str(bad))
    assert e.value.code == -3


@pytest.mark.parametrize("config,cells,synapses", [(1, 9256, 196960), (2, 92550, 2731520)])
def test_scaffold_sizes(config, cells, synapses):
    net = sg.scaffold(config, 1.0, 1)
    c = net.counts()
    assert (c["neurons"], c["synapses"], c["populations"], c["projections"]) == (
        cells, synapses, 7, 11)
    names = [p.name for p in net.populations]
    assert names == ["mossy", "granule", "golgi", "stellate", "basket", "purkinje", "dcn"]
    assert net.populations[0].dev_type == sg.INPUT and net.populations[6].dev_type == sg.OUTPUT
    assert len(net.inputs()) == (1 if config == 1 else 2)


def test_scaffold_deterministic_and_scaled():
    a = sg.scaffold(1, 0.3, 5)
    b = sg.scaffold(1, 0.3, 5)
    for j in range(len(a.projections)):
        assert all(np.array_equal(x, y) for x, y in zip(a.synapses(j), b.synapses(j)))
    assert a.populations[1].num == round(8192 * 0.3)
    scales = sg.batched_scales(range(1, 65))
    assert len(scales) == 64 and min(scales) >= 0.25 and max(scales) < 2.0
    assert len(set(scales)) == 64
    with pytest.raises(SgbError):
        sg.Network().build_scaffold(3)


@pytest.mark.parametrize("config,scale,seed", [(1, 1.0, 1), (2, 1.0, 1), (2, 0.41, 23),
                                               (1, 0.25, 7), (5, 0.05, 3)])
def test_oracle_generator_draws_the_library_networks(config, scale, seed):
    """The oracle's own generator (oracle/netgen.c), which the CPU arms of the
    benchmark use so that they load no library code, draws exactly the
    library's synthetic scaffolds: populations, every synapse array and the
    stimulus sources."""
    import oracle_py

    a = oracle_py.describe(sg.scaffold(config, scale, seed))
    b = oracle_py.scaffold_desc(config, scale, seed)
    assert a["pops"] == b["pops"]
    assert len(a["projs"]) == len(b["projs"]) == 11
    for pa, pb in zip(a["projs"], b["projs"]):
        assert (pa["pre"], pa["post"], pa["channel"]) == (pb["pre"], pb["post"], pb["channel"])
        for k in ("pre_idx", "post_idx", "weight", "delay"):
            assert pa[k].dtype == pb[k].dtype
            assert np.array_equal(pa[k].view(np.uint8), pb[k].view(np.uint8)), k
    assert len(a["srcs"]) == len(b["srcs"])
    for sa, sb in zip(a["srcs"], b["srcs"]):
        assert np.array_equal(sa["ids"], sb["ids"])
        assert {k: v for k, v in sa.items() if k != "ids"} == \
            {k: v for k, v in sb.items() if k != "ids"}
