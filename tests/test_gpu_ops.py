"""Standalone delivery operator (sgb_deliver_spikes) on caller-owned device buffers.

Checked against a numpy restatement of the operation: for each spiking cell,
every synapse of its push-table row adds rint(weight) to ring slot
(step + delay) % slots of its target's accumulator.  Integer sums: exact.
"""
import ctypes as C

import numpy as np
import pytest

import oracle_py
import scaffold_gb300 as sg
from scaffold_gb300 import _lib as L

gpu = pytest.mark.gpu


def bf16_bits(x: np.ndarray) -> np.ndarray:
    u = x.astype(np.float32).view(np.uint32).astype(np.uint64)
    return ((u + 0x7FFF + ((u >> 16) & 1)) >> 16).astype(np.uint16)


def push_table(net, bf16: bool):
    """Cell-major push table over every projection of `net` (unpadded ids)."""
    d = oracle_py.describe(net)
    o = oracle_py.Oracle(d, seed=1, bf16=bf16)
    base = np.cumsum([0] + [p["num"] for p in d["pops"]])
    n = int(base[-1])
    pre_g, word, wsc = [], [], []
    for pr in d["projs"]:
        s = o.scale_bits(pr["post"], pr["channel"])
        w = pr["weight"].astype(np.float32)
        if bf16:
            w = (bf16_bits(w).astype(np.uint32) << 16).view(np.float32)
        ws = (w * np.float32(2.0 ** s)).astype(np.float32)
        pre_g.append(np.int64(base[pr["pre"]]) + pr["pre_idx"].astype(np.int64))
        post_g = np.uint64(base[pr["post"]]) + pr["post_idx"].astype(np.uint64)
        word.append(post_g | (pr["delay"].astype(np.uint64) << np.uint64(27))
                    | (np.uint64(pr["channel"]) << np.uint64(31)))
        wsc.append(ws)
    pre_g, word, wsc = np.concatenate(pre_g), np.concatenate(word), np.concatenate(wsc)
    order = np.argsort(pre_g, kind="stable")
    row = np.zeros(n + 1, np.int64)
    np.add.at(row, pre_g + 1, 1)
    row = np.cumsum(row).astype(np.uint32)
    return n, row, word[order].astype(np.uint32), wsc[order]


def expected(ring, n, row, syn, wsc, spikes, step, slots):
    for j in np.flatnonzero(spikes):
        for q in range(int(row[j]), int(row[j + 1])):
            s = int(syn[q])
            post, dl, ch = s & ((1 << 27) - 1), (s >> 27) & 15, s >> 31
            ring[(step + dl) % slots, post, ch] += int(np.rint(wsc[q]))


def test_ring_wrap_restatement_cpu():
    """The restatement's slot rule for delays at or beyond the ring size: a
    delay-4 synapse on a 3-slot ring at step 1 lands in slot (1 + 4) % 3 = 2."""
    ring = np.zeros((3, 2, 2), np.int64)
    row = np.array([0, 1, 1], np.uint32)
    syn = np.array([1 | (4 << 27)], np.uint32)
    expected(ring, 2, row, syn, np.array([7.0], np.float32), np.array([1, 0], np.uint8), 1, 3)
    assert ring[2, 1, 0] == 7 and ring.sum() == 7


def test_push_table_helper_cpu():
    """The restatement used by the GPU checks covers every synapse once (no GPU)."""
    net = sg.scaffold(1, 0.25, 17)
    n, row, syn, wsc = push_table(net, False)
    assert row[-1] == net.counts()["synapses"] == len(syn) == len(wsc)
    ring = np.zeros((5, n, 2), np.int64)
    expected(ring, n, row, syn, wsc, np.ones(n, np.uint8), 0, 5)
    assert ring[0].sum() == 0 and ring[1:].sum() > 0


@gpu
@pytest.mark.parametrize("bf16,slots", [(False, 5), (True, 5), (False, 2), (True, 3)])
def test_deliver_spikes_matches_restatement(bf16, slots):
    """slots 2 and 3 are below the table's largest delay (4): those synapses
    wrap around the ring, (step + d) % slots, and stay inside it."""
    import torch

    net = sg.scaffold(1, 0.25, 17)
    n, row, syn, wsc = push_table(net, bf16)
    assert int(((syn >> 27) & 15).max()) == 4
    dev = torch.device("cuda")
    t_row = torch.from_numpy(row.view(np.int32)).to(dev)
    t_syn = torch.from_numpy(syn.view(np.int32)).to(dev)
    if bf16:
        t_w = torch.from_numpy(bf16_bits(wsc).view(np.int16)).to(dev)
    else:
        t_w = torch.from_numpy(wsc).to(dev)
    ring = torch.zeros((slots, n, 2), dtype=torch.int32, device=dev)
    exp = np.zeros((slots, n, 2), np.int64)
    rng = np.random.default_rng(5)
    stream = torch.cuda.current_stream().cuda_stream
    for step in (0, 3, 7):
        spikes = (rng.random(n) < 0.08).astype(np.uint8)
        t_sp = torch.from_numpy(spikes).to(dev)
        rc = L.lib().sgb_deliver_spikes(t_sp.data_ptr(), n, t_row.data_ptr(), t_syn.data_ptr(),
                                        t_w.data_ptr(), 1 if bf16 else 0, ring.data_ptr(),
                                        slots, step, stream)
        L.check(rc)
        expected(exp, n, row, syn, wsc, spikes, step, slots)
    torch.cuda.synchronize()
    assert np.array_equal(ring.cpu().numpy().astype(np.int64), exp)
    assert exp.any()


@gpu
def test_deliver_spikes_argument_errors():
    assert L.lib().sgb_deliver_spikes(None, 10, None, None, None, 0, None, 5, 0, None) == -1
    assert L.lib().sgb_deliver_spikes(None, 0, None, None, None, 0, None, 1, 0, None) == -1
    assert L.lib().sgb_deliver_spikes(None, 0, None, None, None, 0, None, 5, 0, None) == 0
