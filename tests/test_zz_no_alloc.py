"""sgb_deliver_spikes_static: spike delivery that allocates no device memory.

It exists for callers that cannot allocate device memory at the point of
delivery -- a real-time step loop in which a device allocation could
synchronise the device and miss the step deadline, or a process whose device
memory is owned by another allocator that must not be bypassed.  It must give
exactly what sgb_deliver_spikes (which draws its scratch from the stream-ordered
pool) gives.  Two calls in a row share the static scratch, so the second call
also checks that nothing of the first call's active list leaks into it.  This
file is collected last so that a failure here leaves every other test already
run.
"""
import os
import sys

import numpy as np
import pytest

import scaffold_gb300 as sg
from scaffold_gb300 import _lib as L

sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
from test_gpu_ops import bf16_bits, push_table  # noqa: E402

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("bf16,slots", [(False, 5), (True, 5), (False, 3)])
def test_static_scratch_matches_allocating_entry_point(bf16, slots):
    """slots 3 is below the table's largest delay (4): those synapses wrap
    around the ring in both entry points alike."""
    import torch

    net = sg.scaffold(1, 0.25, 23)
    n, row, syn, wsc = push_table(net, bf16)
    dev = torch.device("cuda")
    t_row = torch.from_numpy(row.view(np.int32)).to(dev)
    t_syn = torch.from_numpy(syn.view(np.int32)).to(dev)
    t_w = (torch.from_numpy(bf16_bits(wsc).view(np.int16)) if bf16
           else torch.from_numpy(wsc)).to(dev)
    ring_static = torch.zeros((slots, n, 2), dtype=torch.int32, device=dev)
    ring_pool = torch.zeros((slots, n, 2), dtype=torch.int32, device=dev)
    stream = torch.cuda.current_stream().cuda_stream
    rng = np.random.default_rng(29)
    # Two calls in a row with different spike sets: the second one has fewer
    # spikes, so a stale active list from the first call would show up.
    for step, p in ((4, 0.2), (9, 0.03)):
        spikes = torch.from_numpy((rng.random(n) < p).astype(np.uint8)).to(dev)
        wt = 1 if bf16 else 0
        L.check(L.lib().sgb_deliver_spikes_static(
            spikes.data_ptr(), n, t_row.data_ptr(), t_syn.data_ptr(), t_w.data_ptr(), wt,
            ring_static.data_ptr(), slots, step, stream))
        L.check(L.lib().sgb_deliver_spikes(
            spikes.data_ptr(), n, t_row.data_ptr(), t_syn.data_ptr(), t_w.data_ptr(), wt,
            ring_pool.data_ptr(), slots, step, stream))
        torch.cuda.synchronize()
        a, b = ring_static.cpu().numpy(), ring_pool.cpu().numpy()
        assert np.array_equal(a, b)  # integer fixed-point sums: exact
        assert a.any()


def test_static_scratch_rejects_oversized_input():
    # Beyond the stated maximum of 1,048,576 cells: rejected before any GPU work.
    rc = L.lib().sgb_deliver_spikes_static(None, (1 << 20) + 1, None, None, None, 0, None, 5, 0,
                                           None)
    assert rc == -4
    assert b"static scratch" in L.lib().sgb_last_error()
