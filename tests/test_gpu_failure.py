"""Failure detection without a GPU fault: the persistent kernels' grid barrier
is the library's only device-side wait, and it gives up after 1 s.  The test
makes it wait for arrivals that no block makes (sgb_config.barrier_test_extra)
and checks that the run ends, the host sees SGB_ERR_DEVICE, and the context
stays usable."""
import time

import numpy as np
import pytest

import oracle_py
import scaffold_gb300 as sg

SGB_ERR_ARG, SGB_ERR_DEVICE = -1, -8


def test_barrier_test_extra_validation():
    net = sg.scaffold(1, 0.1, 2)
    with pytest.raises(sg.SgbError) as ei:
        sg.Simulation([net], [2], barrier_test_extra=-1)
    assert ei.value.code == SGB_ERR_ARG


@pytest.mark.gpu
@pytest.mark.parametrize("scale", [0.25, 20.0])  # fused / general persistent kernel
def test_grid_barrier_wait_runs_out_and_reports(scale):
    net = sg.scaffold(1, scale, 2)
    sim = sg.Simulation([net], [2], exec_mode=sg.EXEC_PERSISTENT, barrier_test_extra=1,
                        chunk_steps=50)
    t0 = time.time()
    with pytest.raises(sg.SgbError) as ei:
        sim.run(50)
    assert ei.value.code == SGB_ERR_DEVICE
    assert time.time() - t0 < 15.0
    sim.close()
    # The context is intact: a new handle runs and matches the oracle bit for bit.
    sim = sg.Simulation([net], [2], exec_mode=sg.EXEC_PERSISTENT)
    counts, _ = sim.loop_n_steps(200)
    o = oracle_py.Oracle(oracle_py.describe(net), seed=2)
    ec, _ = o.run(200)
    assert np.array_equal(counts, ec)
    sim.close()
