"""bench.py's reference arm on the CPU: one JSON line with the benchmark's keys.

The reference arm times the reference's own CPU implementation of the step
(its compiled host functions where the sources are present, else their
bit-exact restatement) on the host cores, so it runs without a GPU; the GPU
arm's line carries the same metric, unit and config.
"""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_json_line():
    out = subprocess.run(
        [sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "2",
         "--warmup", "0", "--chunk", "3"],
        cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [x for x in out.stdout.splitlines() if x.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference"
    assert d["metric"].startswith("realtime factor")
    assert d["unit"] == "x realtime" and d["higher_is_better"] is True
    assert d["steps"] == 2 and d["warmup"] == 0 and d["n_gpus"] == 1
    assert d["value"] > 0 and d["ms_per_step"] > 0
    assert d["config"]["workload"].startswith("config 2")
    assert d["config"]["steps_per_bench_step"] == 3
    cb = d["cpu_baseline"]
    assert cb["value"] == d["value"] and cb["unit"] == d["unit"]
    assert cb["kind"] in ("reference", "port") and cb["cores"] >= 1
    assert cb["sample"].startswith("2 bench steps of 3 exchange steps")
    assert d["config"]["cells"] == 92550 and d["config"]["synapses"] == 2731520
    e2e = d["e2e"]
    assert e2e["value"] == d["value"] and e2e["unit"] == d["unit"]
    assert e2e["h2d_bytes_per_step"] == 0 and e2e["d2h_bytes_per_step"] == 0


def test_reference_arm_under_torchrun_prints_once():
    """Launched like the GPU arm for N > 1 (one process per rank), rank 0
    alone runs the reference and prints; the other rank exits 0 without work."""
    import socket

    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    out = subprocess.run(
        [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
         "--master-addr", "127.0.0.1", "--master-port", str(port),
         os.path.join(ROOT, "bench.py"), "--impl", "reference", "--gpus", "2", "--steps", "1",
         "--warmup", "0", "--chunk", "2"],
        cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [x for x in out.stdout.splitlines() if x.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["value"] > 0


def test_reference_arm_maps_no_library_code():
    """The reference arm builds its network with the oracle's generator and
    runs only oracle code: the library's shared object is never mapped."""
    code = (
        "import sys; sys.argv = ['bench.py', '--impl', 'reference', '--steps', '1', "
        "'--warmup', '0', '--chunk', '2']\n"
        "import bench; bench.main()\n"
        "maps = open('/proc/self/maps').read()\n"
        "print('LIBSCAFFOLD_MAPPED' if 'libscaffold_gb300' in maps else 'LIBSCAFFOLD_ABSENT')\n"
        "print('PRODUCT_IMPORTED' if 'scaffold_gb300' in sys.modules else 'PRODUCT_NOT_IMPORTED')\n")
    out = subprocess.run([sys.executable, "-c", code], cwd=ROOT, capture_output=True, text=True,
                         timeout=600)
    assert out.returncode == 0, out.stderr[-2000:]
    assert "LIBSCAFFOLD_ABSENT" in out.stdout and "PRODUCT_NOT_IMPORTED" in out.stdout


def test_both_arms_share_one_config():
    """The GPU arm and the reference arm describe the same workload with the
    same config object (the GPU arm's implementation details live apart)."""
    sys.path.insert(0, ROOT)
    import bench

    wl = bench.WORKLOADS["c2"]
    a = bench.workload_config(wl, 92550, 2731520, 1, 1000, 1)
    assert a == bench.workload_config(wl, 92550, 2731520, 1, 1000, 1)
    assert set(a) == {"workload", "cells", "synapses", "instances_per_gpu", "dt_ms",
                      "steps_per_bench_step", "bio_s_per_bench_step", "weights", "l2",
                      "parallelism"}
