"""Checkpoint / resume: a handle restored from another's checkpoint continues
exactly as the saved one (counts, rasters, state, totals, plastic values)."""
import numpy as np
import pytest

import scaffold_gb300 as sg

pytestmark = pytest.mark.gpu


def _same_run(a, b, steps):
    ca, (ia, oa) = a.loop_n_steps(steps, raster=True)
    cb, (ib, ob) = b.loop_n_steps(steps, raster=True)
    assert ca.sum() > 0
    assert np.array_equal(ca, cb) and np.array_equal(oa, ob) and np.array_equal(ia, ib)
    for x, y in zip(a.state(), b.state()):
        assert np.array_equal(np.asarray(x).view(np.uint32), np.asarray(y).view(np.uint32))
    assert np.array_equal(a.spike_totals(), b.spike_totals())
    assert a.info().step == b.info().step and a.info().events == b.info().events


@pytest.mark.parametrize("exec_mode", [sg.EXEC_GRAPH, sg.EXEC_PERSISTENT])
def test_checkpoint_resume_bit_exact(exec_mode):
    net = sg.scaffold(2, 0.2, 6)
    kw = dict(exec_mode=exec_mode, chunk_steps=250, raster=True)
    a = sg.Simulation([net], [6], **kw)
    a.loop_n_steps(500)
    a.set_input_freq(0, [8.0, 60.0])  # changed rates travel with the checkpoint
    blob = a.save_checkpoint()
    b = sg.Simulation([net], [6], **kw)
    b.loop_n_steps(130)                # whatever b did before is overwritten
    b.load_checkpoint(blob)
    _same_run(a, b, 700)
    a.close()
    b.close()


@pytest.mark.parametrize("exec_mode", [sg.EXEC_GRAPH, sg.EXEC_PERSISTENT])
def test_checkpoint_with_plasticity_and_dense_pull(exec_mode):
    net = sg.scaffold(1, 0.25, 8)
    net.add_plasticity(6, sg.STDP_TEACHER, teacher=8, window=20, a1_j=0.0005, a2_ji=-0.004)
    a = sg.Simulation([net], [8], exec_mode=exec_mode, chunk_steps=200, raster=True)
    a.set_propagation(0, 0, sg.PROP_ELL)
    a.loop_n_steps(400)
    blob = a.save_checkpoint()
    b = sg.Simulation([net], [8], exec_mode=exec_mode, chunk_steps=200, raster=True)
    b.set_propagation(0, 0, sg.PROP_ELL)
    b.load_checkpoint(blob)
    assert np.array_equal(a.plastic_values(0, 6), b.plastic_values(0, 6))
    _same_run(a, b, 600)
    assert np.array_equal(a.plastic_values(0, 6).view(np.uint32),
                          b.plastic_values(0, 6).view(np.uint32))
    a.close()
    b.close()


def test_checkpoint_layout_mismatch_refused():
    a = sg.Simulation([sg.scaffold(1, 0.25, 1)], [1])
    b = sg.Simulation([sg.scaffold(1, 0.3, 1)], [1])
    blob = a.save_checkpoint()
    with pytest.raises(sg.SgbError):
        b.load_checkpoint(blob)
    with pytest.raises(sg.SgbError):
        a.load_checkpoint(blob[:-8])
    a.close()
    b.close()
