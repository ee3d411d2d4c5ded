"""Synthetic benchmark workloads.

  C1  9,256-cell net (512 mossy, 8,192 granule, ...), FP32, 10,000 steps of 0.1 ms
  C2  92,550-cell scaffold (2,400 mossy, 88,000 granule, ...), FP32, 100,000 steps
  C3  C2 with BF16 synapse tables
  C4  64 instances of the C2 architecture, sizes scaled by U[0.25, 2.0] drawn from
      each instance's seed, BF16, 20,000 steps
  C5  ~925k-cell scaffold (10x C2), BF16, 4 batched seeds, 10,000 steps
Connectivity, weights and delays are drawn by the library's generator
(sgb_net_build_scaffold); nothing here needs a dataset.
"""
from __future__ import annotations

from .network import Network

_M0, _M1, _W0, _W1 = 0xD2511F53, 0xCD9E8D57, 0x9E3779B9, 0xBB67AE85
_MASK = 0xFFFFFFFF
TAG_SCALE = 4  # Philox stream tag of the per-instance scale draw


def _philox(c, k0, k1):
    """Philox4x32-10 (Salmon et al., SC'11) for a single counter block."""
    c = list(c)
    for _ in range(10):
        p0, p1 = _M0 * c[0], _M1 * c[2]
        c = [((p1 >> 32) ^ c[1] ^ k0) & _MASK, p1 & _MASK, ((p0 >> 32) ^ c[3] ^ k1) & _MASK,
             p0 & _MASK]
        k0, k1 = (k0 + _W0) & _MASK, (k1 + _W1) & _MASK
    return c


def batched_scales(seeds, lo: float = 0.25, hi: float = 2.0):
    """Population-size factor of each batched instance, U[lo, hi) from its seed."""
    out = []
    for s in seeds:
        x = _philox([0, 0, 0, TAG_SCALE], s & _MASK, (s >> 32) & _MASK)[0]
        out.append(lo + (hi - lo) * ((x >> 8) / 16777216.0))
    return out


def scaffold(config: int, scale: float = 1.0, seed: int = 1) -> Network:
    """Network of scaffold config 1, 2 or 5 (C3/C4 reuse config 2's architecture)."""
    return Network().build_scaffold(config, scale, seed)


WORKLOADS = {
    "c1": dict(config=1, instances=1, steps=10_000, bf16=False),
    "c2": dict(config=2, instances=1, steps=100_000, bf16=False),
    "c3": dict(config=2, instances=1, steps=100_000, bf16=True),
    "c4": dict(config=2, instances=64, steps=20_000, bf16=True, scaled=True),
    "c5": dict(config=5, instances=4, steps=10_000, bf16=True),
}
