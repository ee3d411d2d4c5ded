#!/usr/bin/env python3
"""Benchmark of the scaffold simulation hot path: realtime factor (RTF).

One bench step = one chunk of 1,000 exchange steps of 0.1 ms (0.1 s of
biological time) of the configured workload, replayed as one CUDA graph.
Rank 0 prints one JSON line.  `--impl reference` times the reference's own
CPU path (its compiled functions where built, else their C restatement) on
the host cores instead.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "cerebellar-scaffold-model-simulation-on-gpu_gb300"))
sys.path.insert(0, os.path.join(ROOT, "oracle"))

FALLBACK_HBM_GBS = 6800.0
METRIC = "realtime factor (biological s per wall s), 100k-cell scaffold"
DATA = "synthetic: seeded fixed in-degree connectivity, Philox Poisson mossy input"
WORKLOADS = {
    "c2": dict(config=2, scale=1.0, instances=1, bf16=False,
               desc="config 2: 92,550-cell scaffold, 2,731,520 synapses, FP32 weights, 1 instance"),
    "c3": dict(config=2, scale=1.0, instances=1, bf16=True,
               desc="config 3: config-2 scaffold with BF16 synapse weights, 1 instance"),
    "c4": dict(config=2, scale=None, instances=64, bf16=True,
               desc="config 4: 64 config-2 instances scaled U[0.25,2.0], BF16, batched"),
    "c1": dict(config=1, scale=1.0, instances=1, bf16=False,
               desc="config 1: 9,256-cell net, 196,960 synapses, FP32"),
    "c5": dict(config=5, scale=1.0, instances=4, bf16=True, autotune=True,
               desc="config 5: 4 seeds of the ~925k-cell scaffold (10x config 2), BF16, "
                    "batched, propagation mode per projection from the autotuner"),
}


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="c2", choices=sorted(WORKLOADS))
    ap.add_argument("--chunk", type=int, default=1000, help="exchange steps per bench step")
    ap.add_argument("--cpu-sample", type=int, default=20000,
                    help="exchange steps of the CPU-baseline sample")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--exec", default="persistent", choices=["persistent", "graph"])
    ap.add_argument("--no-ell-roofline", action="store_true",
                    help="skip the dense-pull and plasticity side measurements")
    ap.add_argument("--blocks-per-sm", type=int, default=1)
    ap.add_argument("--no-l2-persist", action="store_true",
                    help="plain L2 caching of the cell state (no persisting window)")
    ap.add_argument("--autotune", action="store_true",
                    help="run the propagation/driver autotuner before timing (default for c5)")
    return ap.parse_args()


def dist_env():
    return (int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")),
            int(os.environ.get("LOCAL_RANK", "0")))


def aggregate(pg, device, ms: float, events: float):
    """Whole-job numbers of one timed region: max wall time over ranks (the job
    finishes with its slowest replica) and the sum of events over ranks."""
    import torch

    if pg is None:
        return ms, events
    tm = torch.tensor([ms], dtype=torch.float64, device=device)
    te = torch.tensor([events], dtype=torch.float64, device=device)
    pg.all_reduce(tm, op=pg.ReduceOp.MAX)
    pg.all_reduce(te, op=pg.ReduceOp.SUM)
    return float(tm[0]), float(te[0])


def realtime_factor(world: int, bench_steps: int, bio_s_per_step: float, ms: float) -> float:
    """Biological seconds simulated by all replicas per wall second."""
    return world * bench_steps * bio_s_per_step / (ms / 1000.0)


def build_nets(wl: dict, rank: int):
    import scaffold_gb300 as sg

    n = wl["instances"]
    seeds = [1 + rank * 1000 + k for k in range(n)]
    scales = sg.batched_scales(seeds) if wl["scale"] is None else [wl["scale"]] * n
    nets = [sg.scaffold(wl["config"], sc, sd) for sc, sd in zip(scales, seeds)]
    return nets, seeds


class Clocks:
    """nvidia-smi sampler running during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None

    def stop(self):
        if not self.proc:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, mx, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = max(mx, float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        os.unlink(self.path)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def measured_hbm():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        d = json.load(open(p))
        for k in ("hbm_gbs", "hbm_GBs", "hbm_copy_gbs"):
            if k in d and d[k]:
                return float(d[k]), "measured"
    except (OSError, ValueError):
        pass
    return FALLBACK_HBM_GBS, "fallback"


def cpu_baseline(wl: dict, sample_steps: int):
    """Reference CPU path on a bounded sample of the workload, all host threads."""
    import oracle_py

    desc = oracle_py.scaffold_desc(wl["config"], wl["scale"] or 1.0, 1)
    threads = os.cpu_count() or 1
    if oracle_py.have_ref_harness(1):
        ref, kind = oracle_py.RefHarness(desc, seed=1, bf16=wl["bf16"]), "reference"
    else:
        ref, kind = oracle_py.RefPort(desc, seed=1, bf16=wl["bf16"]), "port"
    ref.run(20, threads=threads)  # warm caches and thread pool
    t0 = time.perf_counter()
    ref.run(sample_steps, threads=threads)
    dt = time.perf_counter() - t0
    rtf = sample_steps * 0.1e-3 / dt
    return {"value": rtf, "unit": "x realtime", "cores": threads, "kind": kind,
            "sample": f"{sample_steps} exchange steps (0.1 ms) of {wl['desc']}; dense per-delay "
                      f"ELL pull + LIF update as in host_spike_propagation/host_update_lif_ch, "
                      f"OpenMP over post cells"}


def config1_leg(steps: int = 10_000):
    """Config 1 (9,256 cells, 196,960 synapses, FP32) over its full 1 s of
    biological time (10,000 exchange steps): the GPU path (one persistent
    launch per 1,000 steps, CUDA events) and the reference CPU path on all
    host cores, both over the whole run."""
    import torch

    import oracle_py
    import scaffold_gb300 as sg

    net = sg.scaffold(1, 1.0, 1)
    sim = sg.Simulation([net], [1], exec_mode=sg.EXEC_PERSISTENT, chunk_steps=1000)
    stream = torch.cuda.Stream()
    sim.set_stream(stream.cuda_stream)
    sim.run(1000)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(stream)
    sim.enqueue(steps)
    e1.record(stream)
    sim.sync()
    torch.cuda.synchronize()
    gpu_rtf = steps * 1e-4 / (e0.elapsed_time(e1) * 1e-3)
    sim.close()
    desc = oracle_py.scaffold_desc(1, 1.0, 1)
    threads = os.cpu_count() or 1
    if oracle_py.have_ref_harness(1):
        ref, kind = oracle_py.RefHarness(desc, seed=1), "reference"
    else:
        ref, kind = oracle_py.RefPort(desc, seed=1), "port"
    t0 = time.perf_counter()
    ref.run(steps, threads=threads)
    cpu_rtf = steps * 1e-4 / (time.perf_counter() - t0)
    return {"workload": "config 1: 9,256 cells, 196,960 synapses, FP32, 10,000 steps",
            "gpu_realtime_factor": gpu_rtf, "cpu_realtime_factor": cpu_rtf, "cpu_kind": kind,
            "cpu_cores": threads}


def stream_copy_gbs(nbytes: int, reps: int = 20) -> float:
    """Bandwidth (read + write bytes) of a plain device copy of a buffer of
    `nbytes`: the measured-peak method at this launch size."""
    import torch

    x = torch.ones(nbytes // 4, dtype=torch.int32, device="cuda")
    y = torch.empty_like(x)
    for _ in range(3):
        y.copy_(x)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record()
    for _ in range(reps):
        y.copy_(x)
    e1.record()
    torch.cuda.synchronize()
    gbs = 2 * nbytes * reps / (e0.elapsed_time(e1) * 1e-3) / 1e9
    del x, y
    return gbs


def plasticity_leg(peak: float, bench_steps: int = 5, chunk: int = 1000):
    """Config 2 with STDP on the parallel-fibre -> Purkinje projection (1.75M
    synapses): the Teacher rule with the reference's depressing coefficient
    (-0.01 per pre spike in a 50-step window before a teacher spike,
    SynapticPlasticity.cu:13-18), basket cells standing in for the climbing
    fibre (config 2 has no inferior olive); plastic projections are delivered
    by dense pull.  Realtime factor over `bench_steps` chunks with the
    persistent kernel (update, plasticity, deliveries as phases between grid
    barriers) and with the per-step kernels in a CUDA graph, and the STDP
    kernel's per-launch time and algorithmic bytes (per updated plastic
    synapse 16 B + W; with this rule only the rows of Purkinje cells whose
    teacher fired are updated)."""
    import torch

    import scaffold_gb300 as sg

    net = sg.scaffold(2, 1.0, 1)
    names = {p.name: p.index for p in net.projections}
    net.add_plasticity(names["granule_to_purkinje"], sg.STDP_TEACHER,
                       teacher=names["basket_to_purkinje"], window=50, a2_ji=-0.01)

    def timed(exec_mode):
        sim = sg.Simulation([net], [1], chunk_steps=chunk, exec_mode=exec_mode)
        stream = torch.cuda.Stream()
        sim.set_stream(stream.cuda_stream)
        sim.run(chunk)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record(stream)
        for _ in range(bench_steps):
            sim.enqueue(chunk)
        e1.record(stream)
        sim.sync()
        torch.cuda.synchronize()
        return sim, e0.elapsed_time(e1)

    sim, ms_g = timed(sg.EXEC_GRAPH)
    mean_us, bytes_pl, nl = sim.profile(200)
    sim.close()
    sim, ms = timed(sg.EXEC_PERSISTENT)
    kern = {1: "k_persistent", 2: "k_persistent_resident", 3: "k_persistent_fused"}.get(
        sim.info().step_kernel, "graph")
    sim.close()
    gbs = bytes_pl[3] / (mean_us[3] * 1e-6) / 1e9 if mean_us[3] > 0 else 0.0
    return {"workload": "config 2, FP32, Teacher STDP on granule_to_purkinje (1,750,000 synapses)",
            "realtime_factor": bench_steps * chunk * 1e-4 / (ms * 1e-3),
            "us_per_step": 1000.0 * ms / (bench_steps * chunk), "exec_kernel": kern,
            "graph_realtime_factor": bench_steps * chunk * 1e-4 / (ms_g * 1e-3),
            "graph_us_per_step": 1000.0 * ms_g / (bench_steps * chunk),
            "k_stdp_us": mean_us[3], "k_stdp_bytes": bytes_pl[3], "k_stdp_gbs": gbs,
            "k_stdp_frac": gbs / peak, "k_pull_us": mean_us[2], "k_update_us": mean_us[0],
            "k_deliver_us": mean_us[1]}


def step_bytes(sim, pull_entries: int) -> int:
    """Algorithmic bytes of one exchange step's update phase: per LIF cell
    12 B state read + 12 B write + 8 B ring slot; per input cell 4 B source
    mask; 8 B per 32-cell bitmap word (two history copies); 4 B per dense
    entry streamed."""
    import scaffold_gb300 as sg

    segs = sim.segments()
    n_lif = sum(x.count for x in segs if x.dev_type != sg.INPUT)
    n_in = sum(x.count for x in segs if x.dev_type == sg.INPUT)
    n_words = sum((x.count + 31) // 32 for x in segs)
    return 32 * n_lif + 4 * n_in + 8 * n_words + 4 * pull_entries


def traffic_of(workload: str, kernel: str):
    """ncu DRAM bytes per launch (profiles/traffic.json) or None."""
    tp = os.path.join(ROOT, "profiles", "traffic.json")
    try:
        return json.load(open(tp)).get(workload, {}).get(kernel)
    except (OSError, ValueError):
        return None


def config4_leg(peak: float, bench_steps: int = 5, chunk: int = 1000):
    """Config 4, the batched form: 64 instances of the config-2 architecture,
    sizes scaled U[0.25, 2.0) from each instance's seed, BF16 tables, one
    persistent launch per 1,000-step chunk, L2 flushed before every timed
    launch.  Realtime factor over all instances, and the roofline of the
    launch twice: on algorithmic bytes (which count the cell state that the
    persisting L2 window serves) and on the DRAM bytes one ncu capture
    measured (profiles/traffic.json), which do not."""
    import torch

    import scaffold_gb300 as sg

    seeds = [1 + k for k in range(64)]
    nets = [sg.scaffold(2, sc, sd) for sc, sd in zip(sg.batched_scales(seeds), seeds)]
    sim = sg.Simulation(nets, seeds, weight_type=sg.WEIGHT_BF16, chunk_steps=chunk,
                        exec_mode=sg.EXEC_PERSISTENT)
    stream = torch.cuda.Stream()
    sim.set_stream(stream.cuda_stream)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    for _ in range(3):
        sim.enqueue(chunk)
    sim.sync()
    info0 = sim.info()
    evs = []
    for i in range(bench_steps):
        with torch.cuda.stream(stream):
            flush.fill_(i & 0xFF)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        sim.enqueue(chunk)
        e1.record(stream)
        evs.append((e0, e1))
    torch.cuda.synchronize()
    sim.sync()
    ms = sum(a.elapsed_time(b) for a, b in evs)
    info = sim.info()
    kname = sg._lib.KERNEL_NAMES.get(info.step_kernel, "?")
    alg = (bench_steps * chunk * step_bytes(sim, info.pull_entries) +
           (info.delivered - info0.delivered) * (12 + 2) + (info.pulled - info0.pulled) * (8 + 2))
    launch_s = ms / 1000.0 / bench_steps
    achieved = alg / bench_steps / launch_s / 1e9
    dram = traffic_of("c4", kname)
    dram_gbs = dram / launch_s / 1e9 if dram else None
    out = {"workload": f"config 4: 64 instances, {info.n_neurons} cells, {info.n_synapses} "
                       f"synapses, BF16, sizes scaled U[0.25, 2.0)",
           "exec_kernel": kname, "realtime_factor": len(nets) * bench_steps * chunk * 1e-4 /
           (ms * 1e-3), "us_per_step": 1000.0 * ms / (bench_steps * chunk),
           "synaptic_events_per_s": (info.events - info0.events) / (ms * 1e-3),
           "launches_timed": bench_steps, "steps_per_launch": chunk,
           "roofline_algorithmic": {"achieved": achieved, "peak": peak, "unit": "GB/s",
                                    "frac": achieved / peak,
                                    "bytes_per_launch": alg / bench_steps},
           "roofline_dram": {"achieved": dram_gbs, "peak": peak, "unit": "GB/s",
                             "frac": dram_gbs / peak if dram_gbs else None,
                             "bytes_per_launch": dram,
                             "source": "ncu dram__bytes_read.sum + dram__bytes_write.sum of one "
                                       "launch (profiles/traffic.json)"},
           "l2": "flushed (256 MiB write) before every timed launch; the cell state in the "
                 "persisting L2 window is exempt"}
    sim.close()
    return out


def ell_roofline(peak: float):
    """Dense ELL pull at HBM scale: config 5 (4 batched seeds of the ~925k-cell
    scaffold, 109M synapses, 437 MB of ELL entries, larger than L2) with every
    projection forced to dense pull; the per-step pull kernel's time from CUDA
    events per launch over 100 steps after a 1,000-step warm-up.
    Algorithmic bytes: 4 B per stored entry, plus W + 8 B per entry whose pre
    cell spiked (weight and ring atomic)."""
    import scaffold_gb300 as sg

    seeds = [1, 2, 3, 4]
    nets = [sg.scaffold(5, 1.0, sd) for sd in seeds]
    sim = sg.Simulation(nets, seeds, weight_type=sg.WEIGHT_BF16, chunk_steps=100,
                        exec_mode=sg.EXEC_GRAPH)
    for k, net in enumerate(nets):
        for j in range(len(net.projections)):
            sim.set_propagation(k, j, sg.PROP_ELL)
    # Past the start-up transient (every cell starts between reset and
    # threshold, so many fire together in the first milliseconds), as the
    # other legs are: 1,000 steps (0.1 s) before the timed launches.
    sim.run(1000)
    mean_us, bytes_pl, nl = sim.profile(100)
    info = sim.info()
    sim.close()
    gbs = bytes_pl[2] / (mean_us[2] * 1e-6) / 1e9
    ceiling = stream_copy_gbs(int(info.pull_entries) * 4)
    traffic = traffic_of("dense_ell", "k_pull")
    return {"kernel": "k_pull (dense ELL pull, every projection)", "traffic": traffic, "workload":
            f"config 5: 4 seeds, {info.n_neurons} cells, {info.n_synapses} synapses, BF16",
            "mean_us": mean_us[2], "bytes_per_launch": bytes_pl[2], "achieved": gbs,
            "unit": "GB/s", "peak": peak, "frac": gbs / peak,
            "copy_gbs_same_bytes": ceiling,
            "l2": "entries 437 MB per launch (not L2-resident); no flush between launches"}


def workload_config(wl: dict, cells: int, synapses: int, instances: int, chunk: int,
                    world: int) -> dict:
    """The `config` object of both arms' JSON lines: the workload and the
    measurement protocol, nothing that depends on the implementation."""
    return {"workload": wl["desc"], "cells": cells, "synapses": synapses,
            "instances_per_gpu": instances, "dt_ms": 0.1, "steps_per_bench_step": chunk,
            "bio_s_per_bench_step": chunk * 0.1e-3 * instances,
            "weights": "bf16" if wl["bf16"] else "fp32",
            "l2": "GPU arm: L2 flushed (256 MiB write) before every timed bench step; the cell "
                  "state kept in a persisting L2 window is exempt by design",
            "parallelism": f"replicas x{world}"}


def reference_desc(wl: dict):
    """Network of the reference arm, drawn by the oracle's generator (no
    library code): the same synapse arrays as the GPU arm's instance 0."""
    import oracle_py

    return oracle_py.scaffold_desc(wl["config"], wl["scale"] or 1.0, 1)


def run_reference(a):
    """The reference's CPU loops (host_update_lif_ch / host_spike_propagation,
    its compiled functions where they are built, else their restatement) on
    all host cores, over the GPU arm's workload: one bench step = `--chunk`
    exchange steps of one instance."""
    rank, world, _ = dist_env()
    if rank != 0:
        return
    import oracle_py

    wl = WORKLOADS[a.workload]
    desc = reference_desc(wl)
    cells, synapses = oracle_py.desc_counts(desc)
    threads = os.cpu_count() or 1
    if oracle_py.have_ref_harness(1):
        ref, kind = oracle_py.RefHarness(desc, seed=1, bf16=wl["bf16"]), "reference"
    else:
        ref, kind = oracle_py.RefPort(desc, seed=1, bf16=wl["bf16"]), "port"
    for _ in range(a.warmup):
        ref.run(a.chunk, threads=threads)
    t0 = time.perf_counter()
    for _ in range(a.steps):
        ref.run(a.chunk, threads=threads)
    dt = time.perf_counter() - t0
    bio = a.steps * a.chunk * 0.1e-3
    rtf = bio / dt
    line = {
        "impl": "reference", "metric": METRIC, "value": rtf, "unit": "x realtime",
        "n_gpus": world, "steps": a.steps, "warmup": a.warmup,
        "ms_per_step": 1000.0 * dt / a.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": DATA,
        "config": workload_config(wl, cells, synapses, 1, a.chunk, world),
        "engine": {"kind": kind, "threads": threads,
                   "path": "dense per-delay ELL pull + LIF update (host_spike_propagation / "
                           "host_update_lif_ch), OpenMP over post cells"},
        "cpu_baseline": {"value": rtf, "unit": "x realtime", "cores": threads, "kind": kind,
                         "sample": f"{a.steps} bench steps of {a.chunk} exchange steps "
                                   f"(0.1 ms) of instance 0"},
        "e2e": {"value": rtf, "unit": "x realtime", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def run_gb300(a):
    import torch

    import scaffold_gb300 as sg

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    pg = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
        pg = dist
    wl = WORKLOADS[a.workload]
    nets, seeds = build_nets(wl, rank)
    exec_mode = sg.EXEC_PERSISTENT if a.exec == "persistent" else sg.EXEC_GRAPH
    sim = sg.Simulation(nets, seeds, weight_type=sg.WEIGHT_BF16 if wl["bf16"] else sg.WEIGHT_FP32,
                        chunk_steps=a.chunk, device=local, exec_mode=exec_mode,
                        blocks_per_sm=a.blocks_per_sm, l2_persist=not a.no_l2_persist)
    stream = torch.cuda.Stream()
    sim.set_stream(stream.cuda_stream)
    tuned = None
    if a.autotune or wl.get("autotune"):
        sim.autotune(100)
        modes = [sim.get_propagation(0, j) for j in range(len(nets[0].projections))]
        tuned = {"ell": sum(m == sg.PROP_ELL for m in modes), "csr": sum(m == sg.PROP_CSR
                                                                     for m in modes)}
    info = sim.info()
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    bio_per_step = a.chunk * 0.1e-3 * len(nets)

    for _ in range(a.warmup):
        sim.enqueue(a.chunk)
    sim.sync()
    ev0 = sim.info().events
    dlv0 = sim.info().delivered
    pull0 = sim.info().pulled
    l0 = sim.launch_count()
    clocks = Clocks(local)
    clocks.start()
    if pg:
        pg.barrier()
    torch.cuda.synchronize()
    evs = []
    for i in range(a.steps):
        with torch.cuda.stream(stream):
            flush.fill_(i & 0xFF)  # > L2: every timed step starts from a cold L2
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        sim.enqueue(a.chunk)
        e1.record(stream)
        evs.append((e0, e1))
    torch.cuda.synchronize()
    sim.sync()
    if pg:
        pg.barrier()
    clk = clocks.stop()
    ms = sum(e0.elapsed_time(e1) for e0, e1 in evs)
    info_t = sim.info()
    events = info_t.events - ev0
    dlv1 = info_t.delivered
    launches = sim.launch_count() - l0
    ms_max, events_all = aggregate(pg, "cuda", ms, float(events))
    value = realtime_factor(world, a.steps, bio_per_step, ms_max)

    # End to end through the C ABI: new input rates from host memory before
    # each step, per-step spike counts of every population back to the host.
    rates = [4.0, 100.0] if wl["config"] != 1 else [4.0]
    n_src = len(nets[0].inputs())
    rates = rates[:n_src]
    e2e_steps = max(3, min(a.steps, 20))
    sim.loop_n_steps(a.chunk, counts=True)
    if pg:
        pg.barrier()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        for k in range(len(nets)):
            sim.set_input_freq(k, rates)
        counts, _ = sim.loop_n_steps(a.chunk, counts=True)
    e2e_s, _ = aggregate(pg, "cuda", time.perf_counter() - t0, 0.0)
    e2e = {"value": realtime_factor(world, e2e_steps, bio_per_step, e2e_s * 1000.0),
           "unit": "x realtime",
           "h2d_bytes_per_step": 56 * n_src * len(nets),
           "d2h_bytes_per_step": 4 * a.chunk * info.n_segments + 4}

    if rank != 0:
        if pg:
            pg.destroy_process_group()
        return
    # Roofline of the kernel that ran the timed region.  Algorithmic bytes:
    # per LIF cell and step 12 B state read + 12 B write + 8 B ring slot; per
    # input cell 4 B source mask; 8 B per 32-cell bitmap word (two history
    # copies); per delivered push synapse 4 B word + W B weight + 8 B atomic
    # read-modify-write; per dense entry and step 4 B, plus W + 8 B per entry
    # whose pre cell spiked.
    wbytes = 2 if wl["bf16"] else 4
    info1 = sim.info()
    upd_step = step_bytes(sim, info_t.pull_entries)
    alg_bytes = (a.steps * a.chunk * upd_step + (dlv1 - dlv0) * (12 + wbytes) +
                 (info_t.pulled - pull0) * (8 + wbytes))
    peak, peak_kind = measured_hbm()
    achieved = alg_bytes / (ms / 1000.0) / 1e9
    kname = sg._lib.KERNEL_NAMES.get(info1.step_kernel, "?")
    traffic = traffic_of(a.workload, kname)
    roof = {"bound": "hbm", "kernel": kname, "achieved": achieved, "peak": peak,
            "peak_source": peak_kind, "unit": "GB/s", "frac": achieved / peak,
            "traffic": traffic, "algorithmic_bytes_per_launch": alg_bytes / a.steps,
            "mean_us_per_launch": 1000.0 * ms / a.steps,
            "launches_timed": a.steps, "steps_per_launch": a.chunk}
    if kname in ("k_persistent_fused", "k_persistent_resident"):
        # Resident networks live in L2: the step is bounded by its chain of L2
        # round trips and the grid barrier, not by HBM bandwidth.
        roof["limiter"] = ("latency: L2-resident network; per 0.1-ms step the ring-slot read, the "
                           "cell update and the grid barrier's arrival and propagation are "
                           "dependent L2 round trips (the step's pushes overlap the barrier)")
    # Per-phase view from an instrumented run of the per-step kernels (CUDA
    # events on the handle's stream around every launch).
    mean_us, bytes_pl, nl = sim.profile(1000)
    phases = {n: {"mean_us": m, "bytes_per_launch": b,
                  "achieved_gbs": (b / (m * 1e-6) / 1e9) if m > 0 else 0.0}
              for n, m, b, c in zip(["k_update", "k_deliver", "k_pull", "k_stdp"], mean_us, bytes_pl,
                                    nl)
              if c > 0}
    ell = None if a.no_ell_roofline else ell_roofline(peak)
    plast = None if a.no_ell_roofline else plasticity_leg(peak)
    c4 = None if (a.no_ell_roofline or a.workload != "c2") else config4_leg(peak)
    cpu = None
    c1 = None
    if not a.no_cpu_baseline:
        try:
            cpu = cpu_baseline(wl, a.cpu_sample)
            if a.workload == "c2":
                c1 = config1_leg()
        except Exception as ex:  # report, do not fail the GPU number
            cpu = {"value": None, "error": str(ex)}
    line = {
        "metric": METRIC, "value": value, "unit": "x realtime", "n_gpus": world,
        "steps": a.steps, "warmup": a.warmup, "ms_per_step": ms_max / a.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": DATA,
        "config": workload_config(wl, info.n_neurons, info.n_synapses, len(nets), a.chunk,
                                  world),
        "engine": {"exec": {sg.EXEC_PERSISTENT: "one persistent cooperative kernel per chunk",
                            sg.EXEC_GRAPH: "cuda graph of 2 kernels per step"}.get(
                                info.exec_mode, "per-step launches"),
                   "propagation": ("event-driven CSR push" if tuned is None else
                                   f"autotuned: {tuned['ell']} projections dense ELL pull, "
                                   f"{tuned['csr']} event-driven CSR push (instance 0)"),
                   "exec_kernel": sg._lib.KERNEL_NAMES.get(info.step_kernel, "?"),
                   "l2_persist_bytes": info.l2_persist_bytes},
        "synaptic_events_per_s": events_all / (ms_max / 1000.0),
        "gpu_launches": launches,
        "e2e": e2e,
        "roofline": roof,
        "phase_profile": phases,
        "dense_ell_roofline": ell,
        "plasticity": plast,
        "config4": c4,
        "config1": c1,
        "cpu_baseline": cpu,
        "clocks": clk,
    }
    print(json.dumps(line), flush=True)
    if pg:
        pg.destroy_process_group()


def main():
    a = parse()
    if a.impl == "reference":
        run_reference(a)
    else:
        run_gb300(a)


if __name__ == "__main__":
    main()
