"""Generates tests/golden/philox4x32_10.json from PyTorch's Philox engine.

PyTorch ships an independent host implementation of Philox4x32-10
(ATen/core/PhiloxRNGEngine.h, philox_engine(seed, subsequence, offset)); its
first four outputs for (seed, subsequence, offset) are the block of counter
{offset lo, offset hi, subsequence lo, subsequence hi} under key {seed lo,
seed hi}.  This script compiles a few lines against that header and records
the blocks for a fixed list of counters and keys, so the library's and the
oracle's Philox can be checked without PyTorch present.
Usage: python tests/golden/make_philox_golden.py
"""
import json
import os
import subprocess
import tempfile

from torch.utils.cpp_extension import include_paths

CASES = [
    ((0, 0, 0, 0), (0, 0)),
    ((0xFFFFFFFF,) * 4, (0xFFFFFFFF, 0xFFFFFFFF)),
    ((0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344), (0xA4093822, 0x299F31D0)),
    ((1, 0, 0, 0), (1, 0)),
    ((123, 456, 0, 1), (7, 0)),          # neuron 123, step 456, input draw, seed 7
    ((5000, 99999, 0, 2), (11, 0)),      # initial-potential draw
    ((88157, 1000000, 0, 1 | (2 << 8)), (0xDEADBEEF, 0x12345678)),
    ((0, 0x89ABCDEF, 0x1, 3), (1000004, 0)),
]

SRC = r"""
#include <ATen/core/PhiloxRNGEngine.h>
#include <cstdio>
#include <cstdint>
int main() {
  unsigned long long c0, c1, c2, c3, k0, k1;
  while (std::scanf("%llu %llu %llu %llu %llu %llu", &c0, &c1, &c2, &c3, &k0, &k1) == 6) {
    const uint64_t seed = k0 | (k1 << 32), sub = c2 | (c3 << 32), off = c0 | (c1 << 32);
    at::Philox4_32 e(seed, sub, off);
    unsigned a = e(), b = e(), c = e(), d = e();
    std::printf("%u %u %u %u\n", a, b, c, d);
  }
  return 0;
}
"""


def main():
    here = os.path.dirname(os.path.abspath(__file__))
    with tempfile.TemporaryDirectory() as td:
        src = os.path.join(td, "p.cpp")
        exe = os.path.join(td, "p")
        open(src, "w").write(SRC)
        inc = sum((["-I", p] for p in include_paths()), [])
        subprocess.run(["g++", "-std=c++17", "-O1", src, "-o", exe] + inc, check=True)
        inp = "\n".join(" ".join(str(x) for x in c + k) for c, k in CASES) + "\n"
        out = subprocess.run([exe], input=inp, capture_output=True, text=True, check=True).stdout
    rows = [list(map(int, l.split())) for l in out.strip().splitlines()]
    data = [{"ctr": list(c), "key": list(k), "out": r} for (c, k), r in zip(CASES, rows)]
    with open(os.path.join(here, "philox4x32_10.json"), "w") as f:
        json.dump({"source": "PyTorch ATen/core/PhiloxRNGEngine.h (philox_engine)",
                   "vectors": data}, f, indent=1)


if __name__ == "__main__":
    main()
