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


# Reference-structure mode ---------------------------------------------------
# Populations of the reference scaffold in its array order and its .dat names
# (init_params.cu:367-766).  The reference's connectivity files are not
# available, so write_reference_dat draws a stand-in with fixed in-degrees.
REFERENCE_SIZES = [88158, 69, 219, 603, 603, 12, 7073]  # grc, pc, goc, sc, bc, dcn, glom
_GRC, _PC, _GOC, _SC, _BC, _DCN, _GLOM = range(7)
REFERENCE_PROJECTIONS = [  # file, pre, post, in-degree of the synthetic stand-in
    ("parallel_fiber_to_purkinje.dat", _GRC, _PC, 5000),
    ("parallel_fiber_to_golgi.dat", _GRC, _GOC, 400),
    ("parallel_fiber_to_stellate.dat", _GRC, _SC, 100),
    ("parallel_fiber_to_basket.dat", _GRC, _BC, 100),
    ("ascending_axon_to_golgi.dat", _GRC, _GOC, 20),
    ("ascending_axon_to_purkinje.dat", _GRC, _PC, 50),
    ("golgi_to_golgi.dat", _GOC, _GOC, 10),
    ("stellate_to_stellate.dat", _SC, _SC, 10),
    ("basket_to_basket.dat", _BC, _BC, 10),
    ("glomerulus_to_dcn.dat", _GLOM, _DCN, 50),
    ("purkinje_to_dcn.dat", _PC, _DCN, 12),
    ("basket_to_purkinje.dat", _BC, _PC, 10),
    ("stellate_to_purkinje.dat", _SC, _PC, 10),
    ("glomerulus_to_granule.dat", _GLOM, _GRC, 4),
    ("glomerulus_to_golgi.dat", _GLOM, _GOC, 20),
    ("golgi_to_granule.dat", _GOC, _GRC, 4),
]


def reference_sizes(scale: float = 1.0):
    return [max(1, int(round(n * scale))) for n in REFERENCE_SIZES]


def write_reference_dat(directory: str, scale: float = 1.0, seed: int = 1,
                        tone_fraction: float = 0.1):
    """Writes the reference scaffold's 16 projection files and its two stimulus
    id lists (background_noise.dat: every glomerulus; tone_stim.dat: the first
    `tone_fraction` of them) in the reference's format; returns the sizes."""
    import os

    import numpy as np

    from . import _lib as L

    sizes = reference_sizes(scale)
    net = Network()
    ch = [(1.0, 0.0, 1.0, 0.5), (1.0, -80.0, 1.0, 10.0)]
    for k, n in enumerate(sizes):
        if k == _GLOM:
            net.set_neuron_params(f"p{k}", n, 0, 0, 0, 0, 0, 0, 0, L.INPUT)
        else:
            net.set_neuron_params(f"p{k}", n, 3.0, -70.0, 2.0, 0.0, -70.0, -50.0, 0.2, L.NORMAL, ch)
    os.makedirs(directory, exist_ok=True)
    for j, (fname, pre, post, k) in enumerate(REFERENCE_PROJECTIONS):
        p = net.add_random_projection(pre, post, min(k, sizes[pre]), 1.0, L.CH_EXC,
                                      seed=seed * 7919 + j)
        net.write_projection_dat(p, os.path.join(directory, fname))
    glom = np.arange(sizes[_GLOM])
    np.savetxt(os.path.join(directory, "background_noise.dat"), glom, fmt="%d")
    np.savetxt(os.path.join(directory, "tone_stim.dat"),
               glom[: max(1, int(sizes[_GLOM] * tone_fraction))], fmt="%d")
    return sizes


def reference_scaffold(directory: str, sizes=None) -> Network:
    """The reference scaffold over the .dat files in `directory`."""
    import ctypes as C

    from . import _lib as L

    net = Network()
    arr = (C.c_int32 * 7)(*sizes) if sizes is not None else None
    L.check(L.lib().sgb_net_build_reference_scaffold(net.handle, directory.encode(), arr))
    return net
