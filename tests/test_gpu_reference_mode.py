"""Reference-structure mode: the reference's scaffold definition over .dat files
in its format, 1-ms exchange steps of 10 Euler substeps, its stimulus lists,
and a main.cu-style driver using the reference's six API calls."""
import os
import subprocess
import sys

import numpy as np
import pytest

import oracle_py
import scaffold_gb300 as sg

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "cerebellar-scaffold-model-simulation-on-gpu_gb300")


def test_reference_scaffold_structure(tmp_path):
    sizes = sg.write_reference_dat(str(tmp_path), 0.05, 2)
    net = sg.reference_scaffold(str(tmp_path), sizes)
    c = net.counts()
    assert (c["populations"], c["projections"], c["inputs"]) == (7, 16, 3)
    pops = net.populations
    assert [p.name for p in pops] == ["granule_cell", "purkinje_cell", "golgi_cell",
                                      "stellate_cell", "basket_cell", "dcn_cell", "glomerulus"]
    assert pops[1].Cm == 620.0 and pops[1].Ie == 600.0 and pops[5].dev_type == sg.OUTPUT
    projs = {p.name: p for p in net.projections}
    assert projs["golgi_to_granule"].channel == sg.CH_INH
    assert projs["golgi_to_granule"].min_delay == projs["golgi_to_granule"].max_delay == 2
    assert projs["parallel_fiber_to_purkinje"].max_delay == 5
    _, _, w, _ = net.synapses(list(projs).index("purkinje_to_dcn"))
    assert np.allclose(w, 0.0075)
    kinds = [x[1]["kind"] for x in net.inputs()]
    assert kinds == [sg.INPUT_POISSON, sg.INPUT_PERIODIC, sg.INPUT_POISSON]
    assert sg.lib().sgb_reference_type_id(6) == 1 and sg.lib().sgb_reference_type_id(1) == 2
    with pytest.raises(sg.SgbError) as e:
        sg.reference_scaffold(str(tmp_path / "missing"), sizes)
    assert e.value.code == -2


@pytest.mark.skipif(not oracle_py.have_ref_harness(10), reason="reference sources not built")
def test_reference_mode_oracle_matches_reference_cpu_functions(tmp_path):
    """10-substep steps: the FP64 oracle's raster equals the one produced by the
    reference's compiled host_update_lif_ch / host_spike_propagation."""
    sizes = sg.write_reference_dat(str(tmp_path), 0.05, 4)
    net = sg.reference_scaffold(str(tmp_path), sizes)
    d = oracle_py.describe(net)
    h = oracle_py.RefHarness(d, seed=4, substeps=10)
    hc, (hi, ho) = h.run(400, threads=2)
    o = oracle_py.Oracle(d, seed=4, substeps=10, mode=oracle_py.FP64)
    oc, (oi, oo) = o.run(400)
    assert hc.sum() > 0
    first = next((s for s in range(400) if not np.array_equal(hi[ho[s]:ho[s + 1]], oi[oo[s]:oo[s + 1]])), 400)
    assert first >= 100, first


@pytest.mark.gpu
def test_reference_mode_bit_exact(tmp_path):
    sizes = sg.write_reference_dat(str(tmp_path), 0.1, 3)
    net = sg.reference_scaffold(str(tmp_path), sizes)
    steps = 600  # 600 ms: covers the tone window [300, 351) ms
    sim = sg.Simulation([net], [3], substeps=10, raster=True, chunk_steps=200)
    c, (ids, offs) = sim.loop_n_steps(steps, raster=True)
    o = oracle_py.Oracle(oracle_py.describe(net), seed=3, substeps=10)
    ec, (eids, eoffs) = o.run(steps)
    assert c.sum() > 0 and np.array_equal(c, ec)
    assert np.array_equal(ids, eids) and np.array_equal(offs, eoffs)
    u, g, ref = sim.state()
    eu, eg, eref = o.state()
    assert np.array_equal(u.view(np.uint32), eu.view(np.uint32)) and np.array_equal(ref, eref)
    # Raster in the reference's text format: t, local id, NeuronType id.
    path = str(tmp_path / "raster.dat")
    tids = [sg.lib().sgb_reference_type_id(p) for p in range(7)]
    sim.write_raster(path, ids, offs, 0, tids)
    lines = open(path).read().splitlines()
    assert len(lines) == len(ids)
    t0, lid, tid = lines[0].split("\t")
    first_step = int(np.searchsorted(offs, 1, side="left")) - 1
    assert float(t0) == pytest.approx(float(first_step)) and int(tid) in tids


@pytest.mark.gpu
def test_main_driver_through_compat_api(tmp_path):
    """A C driver written like the reference's main.cu builds against
    scaffold_compat.h and runs one trial of 1,000 ms on the full-size scaffold."""
    data = tmp_path / "data"
    sg.write_reference_dat(str(data), 1.0, 5)
    exe = str(tmp_path / "driver")
    libdir = os.path.join(PKG, "scaffold_gb300")
    subprocess.run(["gcc", "-O2", os.path.join(ROOT, "tests", "compat", "main_driver.c"),
                    "-I", os.path.join(ROOT, "include"), "-L", libdir, "-lscaffold_gb300",
                    f"-Wl,-rpath,{libdir}", "-lm", "-o", exe], check=True)
    env = dict(os.environ, SGB_DAT_DIR=str(data))
    r = subprocess.run([exe, "1", "25", "50"], cwd=str(tmp_path), env=env, capture_output=True,
                       text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    assert "neuron_num = 96737" in r.stderr  # Env.Host_sim_val[0].Host.neuron_num
    assert r.stdout.startswith("dcn_spikes ")
    out = tmp_path / "spike_output" / "spike_result_trial0.dat"
    lines = out.read_text().splitlines()
    assert lines
    t, lid, tid = lines[-1].split("\t")
    assert 0.0 <= float(t) < 1000.0 and int(tid) in range(7)
