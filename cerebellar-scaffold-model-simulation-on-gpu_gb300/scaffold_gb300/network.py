"""Python mirror of the reference's population / projection / stimulus API.

Method names follow the reference (set_neuron_params, set_connectivity_params,
setInputStim in init_params.cu:255-332 and UserInputFunctions.cu:41-70;
loop_n_steps, SetInputFreq, ResetNetworkEnv in GPUScaffoldSimulation.cu);
every call goes through the C ABI of libscaffold_gb300.so.  Errors raise
SgbError carrying the library's status code instead of exiting.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass
from typing import Iterable, Sequence

import numpy as np

from . import _lib as L


def _ptr(a: np.ndarray, ctype):
    return a.ctypes.data_as(C.POINTER(ctype))


@dataclass
class Population:
    index: int
    name: str
    num: int
    dev_type: int
    c_num: int
    Cm: float
    El: float
    dt_ref: float
    Ie: float
    Vr: float
    Vth: float
    gL: float
    channels: list


@dataclass
class Projection:
    index: int
    name: str
    pre: int
    post: int
    channel: int
    mode: int
    n_synapses: int
    max_in_degree: int
    max_out_degree: int
    min_delay: int
    max_delay: int


class Network:
    """One scaffold instance (host description; no GPU needed)."""

    def __init__(self):
        h = C.c_void_p()
        L.check(L.lib().sgb_net_create(C.byref(h)))
        self._h = h

    @property
    def handle(self) -> C.c_void_p:
        return self._h

    def close(self):
        if self._h:
            L.lib().sgb_net_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # ---- reference-named builders --------------------------------------
    def set_neuron_params(self, name: str, num: int, Cm: float, El: float, dt_ref: float,
                          Ie: float, Vr: float, Vth: float, gL: float,
                          dev_type: int = L.NORMAL,
                          channels: Sequence[Sequence[float]] = ()) -> int:
        """set_neuron_params (init_params.cu:255): channels = [(w, E, g_bar, tau), ...]."""
        ch = np.ascontiguousarray(np.asarray(channels, dtype=np.float32).reshape(-1))
        pid = C.c_int32()
        L.check(L.lib().sgb_net_add_population(
            self._h, name.encode(), int(num), Cm, El, dt_ref, Ie, Vr, Vth, gL, dev_type,
            len(channels), _ptr(ch, C.c_float) if ch.size else None, C.byref(pid)))
        return pid.value

    def set_connectivity_params(self, filename: str, pre: int, post: int, initial_weight: float,
                                delay: int, mode: int = L.PROP_AUTO) -> int:
        """set_connectivity_params (init_params.cu:304): load a .dat projection."""
        pid = C.c_int32()
        L.check(L.lib().sgb_net_add_projection_dat(self._h, filename.encode(), pre, post,
                                                   initial_weight, int(delay), mode,
                                                   C.byref(pid)))
        return pid.value

    def add_projection(self, pre: int, post: int, pre_idx, post_idx, weight, delay,
                       channel: int, mode: int = L.PROP_AUTO) -> int:
        pre_idx = np.ascontiguousarray(pre_idx, dtype=np.uint32)
        post_idx = np.ascontiguousarray(post_idx, dtype=np.uint32)
        weight = np.ascontiguousarray(weight, dtype=np.float32)
        n = len(pre_idx)
        pid = C.c_int32()
        if np.isscalar(delay):
            dptr, dall = None, int(delay)
        else:
            delay = np.ascontiguousarray(delay, dtype=np.uint8)
            dptr, dall = _ptr(delay, C.c_uint8), 0
        L.check(L.lib().sgb_net_add_projection_arrays(
            self._h, pre, post, n, _ptr(pre_idx, C.c_uint32), _ptr(post_idx, C.c_uint32),
            _ptr(weight, C.c_float), dptr, dall, channel, mode, C.byref(pid)))
        return pid.value

    def add_random_projection(self, pre: int, post: int, in_degree: int, w_mean: float,
                              channel: int, seed: int, w_lo: float = 0.5, w_hi: float = 1.5,
                              d_min: int = 1, d_max: int = 4, mode: int = L.PROP_AUTO) -> int:
        pid = C.c_int32()
        L.check(L.lib().sgb_net_add_projection_random(self._h, pre, post, in_degree, w_mean, w_lo,
                                                      w_hi, d_min, d_max, channel, seed, mode,
                                                      C.byref(pid)))
        return pid.value

    def set_input_stim(self, pop: int, ids: Iterable[int] | None = None, *,
                       kind: int = L.INPUT_POISSON, rate_hz: float = 1.0, phase_ms: float = 0.0,
                       win_period_ms: float = 0.0, win_start_ms: float = 0.0,
                       win_end_ms: float = 0.0, filename: str | None = None) -> int:
        """setInputStim (UserInputFunctions.cu:41): a stimulus source over `ids` (all cells
        when None) or over the ids listed in `filename`."""
        p = L.InputParams(kind, rate_hz, phase_ms, win_period_ms, win_start_ms, win_end_ms)
        sid = C.c_int32()
        if filename is not None:
            L.check(L.lib().sgb_net_add_input_dat(self._h, filename.encode(), pop, C.byref(p),
                                                  C.byref(sid)))
        elif ids is None:
            L.check(L.lib().sgb_net_add_input(self._h, pop, -1, None, C.byref(p), C.byref(sid)))
        else:
            arr = np.ascontiguousarray(np.fromiter(ids, dtype=np.uint32) if not isinstance(ids, np.ndarray) else ids, dtype=np.uint32)
            L.check(L.lib().sgb_net_add_input(self._h, pop, len(arr), _ptr(arr, C.c_uint32),
                                              C.byref(p), C.byref(sid)))
        return sid.value

    def build_scaffold(self, config: int, scale: float = 1.0, seed: int = 1) -> "Network":
        L.check(L.lib().sgb_net_build_scaffold(self._h, config, scale, seed))
        return self

    # ---- introspection ---------------------------------------------------
    def counts(self):
        a, b, c = C.c_int32(), C.c_int32(), C.c_int32()
        n, s = C.c_int64(), C.c_int64()
        L.check(L.lib().sgb_net_counts(self._h, C.byref(a), C.byref(b), C.byref(c), C.byref(n),
                                       C.byref(s)))
        return dict(populations=a.value, projections=b.value, inputs=c.value,
                    neurons=n.value, synapses=s.value)

    @property
    def populations(self) -> list[Population]:
        out = []
        for i in range(self.counts()["populations"]):
            info = L.PopulationInfo()
            L.check(L.lib().sgb_net_population_info(self._h, i, C.byref(info)))
            ch = [(info.ch_w[c], info.ch_E[c], info.ch_gbar[c], info.ch_tau[c])
                  for c in range(info.c_num)]
            out.append(Population(i, info.name.decode(), info.num, info.dev_type, info.c_num,
                                  info.Cm, info.El, info.dt_ref, info.Ie, info.Vr, info.Vth,
                                  info.gL, ch))
        return out

    @property
    def projections(self) -> list[Projection]:
        out = []
        for i in range(self.counts()["projections"]):
            info = L.ProjectionInfo()
            L.check(L.lib().sgb_net_projection_info(self._h, i, C.byref(info)))
            out.append(Projection(i, info.name.decode(), info.pre_pop, info.post_pop,
                                  info.channel, info.mode, info.n_synapses, info.max_in_degree,
                                  info.max_out_degree, info.min_delay, info.max_delay))
        return out

    def synapses(self, proj: int):
        """(pre, post, weight, delay) numpy arrays of projection `proj`."""
        info = L.ProjectionInfo()
        L.check(L.lib().sgb_net_projection_info(self._h, proj, C.byref(info)))
        n = info.n_synapses
        pre = np.empty(n, np.uint32)
        post = np.empty(n, np.uint32)
        w = np.empty(n, np.float32)
        d = np.empty(n, np.uint8)
        L.check(L.lib().sgb_net_projection_synapses(self._h, proj, _ptr(pre, C.c_uint32),
                                                    _ptr(post, C.c_uint32), _ptr(w, C.c_float),
                                                    _ptr(d, C.c_uint8)))
        return pre, post, w, d

    def inputs(self):
        """[(pop, params dict, ids array)] for every stimulus source."""
        out = []
        for i in range(self.counts()["inputs"]):
            info = L.InputInfo()
            L.check(L.lib().sgb_net_input_info(self._h, i, C.byref(info)))
            ids = np.empty(info.n_ids, np.uint32)
            if info.n_ids:
                L.check(L.lib().sgb_net_input_ids(self._h, i, _ptr(ids, C.c_uint32)))
            p = info.params
            out.append((info.pop, dict(kind=p.kind, rate_hz=p.rate_hz, phase_ms=p.phase_ms,
                                       win_period_ms=p.win_period_ms,
                                       win_start_ms=p.win_start_ms, win_end_ms=p.win_end_ms),
                        ids))
        return out

    def write_projection_dat(self, proj: int, path: str) -> None:
        L.check(L.lib().sgb_net_write_projection_dat(self._h, proj, path.encode()))

    def add_plasticity(self, proj: int, rule: int = L.STDP_HEBB, *, teacher: int = -1,
                       window: int = 50, a0: float = 0.0, a1_i: float = 0.0, a1_j: float = 0.0,
                       a2_ji: float = 0.0, v_max: float = 1.0) -> None:
        """STDP on projection `proj` (the reference's Hebb / Teacher rules,
        SynapticPlasticity.cu:40-120, with constant coefficients)."""
        p = L.PlasticityParams(rule, teacher, window, a0, a1_i, a1_j, a2_ji, v_max)
        L.check(L.lib().sgb_net_add_plasticity(self._h, proj, C.byref(p)))

    def plasticity(self, proj: int):
        """Plasticity parameters of projection `proj` as a dict, or None."""
        flag = C.c_int32()
        p = L.PlasticityParams()
        L.check(L.lib().sgb_net_plasticity_info(self._h, proj, C.byref(flag), C.byref(p)))
        if not flag.value:
            return None
        return dict(rule=p.rule, teacher=p.teacher_proj, window=p.window_steps, a0=p.a0,
                    a1_i=p.a1_i, a1_j=p.a1_j, a2_ji=p.a2_ji, v_max=p.v_max)


class Simulation:
    """Device simulation of one or more independent networks (instances)."""

    def __init__(self, nets: Sequence[Network], seeds: Sequence[int] | None = None, *,
                 dt_ms: float = 0.1, substeps: int = 1, weight_type: int = L.WEIGHT_FP32,
                 exec_mode: int = L.EXEC_GRAPH, chunk_steps: int = 1000, device: int = 0,
                 default_prop: int = L.PROP_AUTO, raster: bool = False, blocks_per_sm: int = 0,
                 l2_persist: bool = True, barrier_test_extra: int = 0):
        cfg = L.Config()
        L.lib().sgb_config_init(C.byref(cfg))
        cfg.dt_ms = dt_ms
        cfg.substeps = substeps
        cfg.weight_type = weight_type
        cfg.exec_mode = exec_mode
        cfg.chunk_steps = chunk_steps
        cfg.device = device
        cfg.default_prop = default_prop
        cfg.raster = 1 if raster else 0
        cfg.blocks_per_sm = blocks_per_sm
        cfg.l2_persist = 1 if l2_persist else 0
        cfg.barrier_test_extra = barrier_test_extra
        self.nets = list(nets)
        n = len(self.nets)
        arr = (C.c_void_p * n)(*[x.handle.value for x in self.nets])
        seeds = list(seeds) if seeds is not None else list(range(1, n + 1))
        sarr = (C.c_uint64 * n)(*seeds)
        h = C.c_void_p()
        L.check(L.lib().sgb_sim_create(C.byref(cfg), arr, sarr, n, C.byref(h)))
        self._h = h
        self.raster_enabled = raster
        info = self.info()
        self.n_segments = info.n_segments
        self.n_neurons = info.n_neurons

    @property
    def handle(self) -> C.c_void_p:
        return self._h

    def close(self):
        if getattr(self, "_h", None):
            L.lib().sgb_sim_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def info(self) -> L.SimInfo:
        info = L.SimInfo()
        L.check(L.lib().sgb_sim_get_info(self._h, C.byref(info)))
        return info

    def segments(self) -> list[L.SegmentInfo]:
        out = []
        for i in range(self.info().n_segments):
            s = L.SegmentInfo()
            L.check(L.lib().sgb_sim_segment_info(self._h, i, C.byref(s)))
            out.append(s)
        return out

    def set_stream(self, stream_ptr: int | None) -> None:
        L.check(L.lib().sgb_sim_set_stream(self._h, C.c_void_p(stream_ptr or 0)))

    def set_input_freq(self, net: int, rates: Sequence[float]) -> None:
        """SetInputFreq (GPUScaffoldSimulation.cu:883)."""
        r = np.ascontiguousarray(rates, dtype=np.float32)
        L.check(L.lib().sgb_sim_set_input_rates(self._h, net, len(r), _ptr(r, C.c_float)))

    def loop_n_steps(self, n_steps: int, counts: bool = True, raster: bool = False,
                     raster_cap: int | None = None):
        """loop_n_steps (GPUScaffoldSimulation.cu:693).  Returns (counts[n, segments] or None,
        (ids, offsets) or None)."""
        cnt = np.zeros((n_steps, self.n_segments), np.uint32) if counts else None
        ids = offs = None
        if raster:
            cap = raster_cap if raster_cap is not None else max(1 << 20, n_steps * 64)
            ids = np.zeros(cap, np.uint32)
            offs = np.zeros(n_steps + 1, np.int64)
        L.check(L.lib().sgb_sim_run(
            self._h, n_steps, _ptr(cnt, C.c_uint32) if cnt is not None else None,
            _ptr(ids, C.c_uint32) if ids is not None else None,
            len(ids) if ids is not None else 0,
            _ptr(offs, C.c_int64) if offs is not None else None))
        r = None
        if raster:
            r = (ids[: offs[-1]].copy(), offs)
        return cnt, r

    def write_raster(self, path: str, ids, offsets, first_step: int = 0, type_ids=None,
                     append: bool = False) -> None:
        """Raster in the reference's text format ("t\tlocal_id\ttype_id" lines)."""
        ids = np.ascontiguousarray(ids, dtype=np.uint32)
        offsets = np.ascontiguousarray(offsets, dtype=np.int64)
        tids = None
        if type_ids is not None:
            tids = np.ascontiguousarray(type_ids, dtype=np.int32)
        L.check(L.lib().sgb_sim_write_raster(
            self._h, path.encode(), _ptr(ids, C.c_uint32), _ptr(offsets, C.c_int64),
            len(offsets) - 1, first_step, _ptr(tids, C.c_int32) if tids is not None else None,
            1 if append else 0))

    def run(self, n_steps: int) -> None:
        """Advances without host outputs (device-resident run)."""
        L.check(L.lib().sgb_sim_run(self._h, n_steps, None, None, 0, None))

    def enqueue(self, n_steps: int) -> None:
        """Enqueues n_steps on the handle's stream without waiting."""
        L.check(L.lib().sgb_sim_enqueue(self._h, n_steps))

    def sync(self) -> None:
        """Waits for the handle's stream; raises on device-side error flags."""
        L.check(L.lib().sgb_sim_sync(self._h))

    def reset(self, seeds: Sequence[int] | None = None) -> None:
        """ResetNetworkEnv (GPUScaffoldSimulation.cu:802)."""
        if seeds is None:
            L.check(L.lib().sgb_sim_reset(self._h, None))
        else:
            s = (C.c_uint64 * len(seeds))(*seeds)
            L.check(L.lib().sgb_sim_reset(self._h, s))

    def state(self):
        n = self.n_neurons
        u = np.empty(n, np.float32)
        g = np.empty((n, 2), np.float32)
        ref = np.empty(n, np.int32)
        L.check(L.lib().sgb_sim_get_state(self._h, _ptr(u, C.c_float), _ptr(g, C.c_float),
                                          _ptr(ref, C.c_int32)))
        return u, g, ref

    def set_state(self, u=None, g=None, ref=None) -> None:
        args = []
        for a, t, ct in ((u, np.float32, C.c_float), (g, np.float32, C.c_float),
                         (ref, np.int32, C.c_int32)):
            if a is None:
                args.append(None)
            else:
                a = np.ascontiguousarray(a, dtype=t)
                args.append(_ptr(a, ct))
                setattr(self, f"_keep_{len(args)}", a)
        L.check(L.lib().sgb_sim_set_state(self._h, *args))

    def spike_totals(self) -> np.ndarray:
        t = np.zeros(self.n_segments, np.float64)
        L.check(L.lib().sgb_sim_spike_totals(self._h, _ptr(t, C.c_double)))
        return t

    def save_checkpoint(self) -> bytes:
        """The handle's whole evolving state as bytes (at a chunk boundary)."""
        n = C.c_int64()
        L.check(L.lib().sgb_sim_checkpoint_size(self._h, C.byref(n)))
        buf = (C.c_char * n.value)()
        L.check(L.lib().sgb_sim_save_checkpoint(self._h, buf, n.value))
        return bytes(buf)

    def load_checkpoint(self, data: bytes) -> None:
        """Restores a checkpoint of a handle with the same networks and configuration."""
        buf = (C.c_char * len(data)).from_buffer_copy(data)
        L.check(L.lib().sgb_sim_load_checkpoint(self._h, buf, len(data)))

    def plastic_values(self, net: int, proj: int) -> np.ndarray:
        """Plasticity values of a plastic projection's synapses (synapse order)."""
        n = self.nets[net].synapses(proj)[0].size
        v = np.empty(max(n, 1), np.float32)
        L.check(L.lib().sgb_sim_plastic_values(self._h, net, proj, _ptr(v, C.c_float)))
        return v[:n]

    def set_propagation(self, net: int, proj: int, mode: int) -> None:
        L.check(L.lib().sgb_sim_set_propagation(self._h, net, proj, mode))

    def get_propagation(self, net: int, proj: int) -> int:
        m = C.c_int32()
        L.check(L.lib().sgb_sim_get_propagation(self._h, net, proj, C.byref(m)))
        return m.value

    def autotune(self, n_steps: int = 200, cache_path: str | None = None) -> None:
        L.check(L.lib().sgb_sim_autotune(self._h, n_steps,
                                         cache_path.encode() if cache_path else None))

    def launch_count(self) -> int:
        v = C.c_int64()
        L.check(L.lib().sgb_sim_launch_count(self._h, C.byref(v)))
        return v.value

    def profile(self, n_steps: int):
        mean = np.zeros(L.KCLASS_COUNT, np.float64)
        byts = np.zeros(L.KCLASS_COUNT, np.float64)
        n = np.zeros(L.KCLASS_COUNT, np.int64)
        L.check(L.lib().sgb_sim_profile(self._h, n_steps, _ptr(mean, C.c_double),
                                        _ptr(byts, C.c_double), _ptr(n, C.c_int64)))
        return mean, byts, n
