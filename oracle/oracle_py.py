"""ctypes wrapper of the CPU oracle -- TEST INFRASTRUCTURE ONLY.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg import
this module; the product never does.  The oracle receives a network's raw
description (population parameters, per-synapse arrays, stimulus sources)
and none of the product's device tables.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_build", "liboracle.so")
FP32, FP64 = 0, 1


class Pop(C.Structure):
    _fields_ = [("num", C.c_int32), ("is_input", C.c_int32), ("Cm", C.c_float),
                ("El", C.c_float), ("dt_ref", C.c_float), ("Ie", C.c_float), ("Vr", C.c_float),
                ("Vth", C.c_float), ("gL", C.c_float), ("c_num", C.c_int32),
                ("w", C.c_float * 2), ("E", C.c_float * 2), ("gbar", C.c_float * 2),
                ("tau", C.c_float * 2)]


class Proj(C.Structure):
    _fields_ = [("pre", C.c_int32), ("post", C.c_int32), ("channel", C.c_int32),
                ("pad_", C.c_int32), ("n", C.c_int64), ("pre_idx", C.POINTER(C.c_uint32)),
                ("post_idx", C.POINTER(C.c_uint32)), ("weight", C.POINTER(C.c_float)),
                ("delay", C.POINTER(C.c_uint8))]


class Src(C.Structure):
    _fields_ = [("pop", C.c_int32), ("kind", C.c_int32), ("rate_hz", C.c_float),
                ("pad_", C.c_float), ("phase_ms", C.c_double), ("win_period_ms", C.c_double),
                ("win_start_ms", C.c_double), ("win_end_ms", C.c_double),
                ("n_ids", C.c_int64), ("ids", C.POINTER(C.c_uint32))]


class Plast(C.Structure):
    _fields_ = [("proj", C.c_int32), ("rule", C.c_int32), ("teacher_proj", C.c_int32),
                ("window", C.c_int32), ("a0", C.c_float), ("a1_i", C.c_float),
                ("a1_j", C.c_float), ("a2_ji", C.c_float), ("v_max", C.c_float),
                ("pad_", C.c_float)]


class Net(C.Structure):
    _fields_ = [("n_pops", C.c_int32), ("n_projs", C.c_int32), ("n_srcs", C.c_int32),
                ("substeps", C.c_int32), ("pops", C.POINTER(Pop)), ("projs", C.POINTER(Proj)),
                ("srcs", C.POINTER(Src)), ("dt_ms", C.c_double), ("seed", C.c_uint64),
                ("bf16", C.c_int32), ("mode", C.c_int32), ("n_plast", C.c_int32),
                ("pad_", C.c_int32), ("plast", C.POINTER(Plast))]


_lib = None


def build() -> str:
    subprocess.run(["make", "-s", "-C", HERE], check=True)
    return LIB


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            build()
        L = C.CDLL(LIB)
        L.orc_philox4x32_10.argtypes = [C.POINTER(C.c_uint32)] * 3
        L.orc_philox4x32_10.restype = None
        L.orc_scale_bits.argtypes = [C.POINTER(Net), C.c_int32, C.c_int32]
        L.orc_scale_bits.restype = C.c_int32
        L.orc_create.argtypes = [C.POINTER(Net), C.POINTER(C.c_void_p)]
        L.orc_create.restype = C.c_int
        L.orc_destroy.argtypes = [C.c_void_p]
        L.orc_destroy.restype = None
        L.orc_set_rates.argtypes = [C.c_void_p, C.POINTER(C.c_float)]
        L.orc_run.argtypes = [C.c_void_p, C.c_int64, C.POINTER(C.c_uint32),
                              C.POINTER(C.c_uint32), C.c_int64, C.POINTER(C.c_int64)]
        L.orc_run.restype = C.c_int
        L.orc_get_state.argtypes = [C.c_void_p, C.POINTER(C.c_float), C.POINTER(C.c_float),
                                    C.POINTER(C.c_int32)]
        L.orc_set_state.argtypes = [C.c_void_p, C.POINTER(C.c_float), C.POINTER(C.c_float),
                                    C.POINTER(C.c_int32)]
        L.orc_events.argtypes = [C.c_void_p]
        L.orc_events.restype = C.c_int64
        L.orc_plastic_values.argtypes = [C.c_void_p, C.c_int32, C.POINTER(C.c_float)]
        L.orc_plastic_values.restype = C.c_int
        _lib = L
    return _lib


def philox(ctr, key):
    c = (C.c_uint32 * 4)(*ctr)
    k = (C.c_uint32 * 2)(*key)
    o = (C.c_uint32 * 4)()
    lib().orc_philox4x32_10(c, k, o)
    return list(o)


def _p(a, t):
    return a.ctypes.data_as(C.POINTER(t))


class Oracle:
    """Oracle simulation of one network description.

    `desc` is a dict: pops [dict(num, is_input, Cm, El, dt_ref, Ie, Vr, Vth, gL, channels)],
    projs [dict(pre, post, channel, pre_idx, post_idx, weight, delay)],
    srcs [dict(pop, kind, rate_hz, phase_ms, win_period_ms, win_start_ms, win_end_ms, ids)].
    """

    def __init__(self, desc: dict, *, dt_ms=0.1, substeps=1, seed=1, bf16=False, mode=FP32):
        self._keep = []
        pops = (Pop * max(1, len(desc["pops"])))()
        for i, p in enumerate(desc["pops"]):
            q = pops[i]
            q.num, q.is_input = p["num"], int(p["is_input"])
            for k in ("Cm", "El", "dt_ref", "Ie", "Vr", "Vth", "gL"):
                setattr(q, k, p[k])
            q.c_num = len(p["channels"])
            for c, (w, E, gb, tau) in enumerate(p["channels"]):
                q.w[c], q.E[c], q.gbar[c], q.tau[c] = w, E, gb, tau
        projs = (Proj * max(1, len(desc["projs"])))()
        for i, p in enumerate(desc["projs"]):
            arrs = [np.ascontiguousarray(p["pre_idx"], np.uint32),
                    np.ascontiguousarray(p["post_idx"], np.uint32),
                    np.ascontiguousarray(p["weight"], np.float32),
                    np.ascontiguousarray(p["delay"], np.uint8)]
            self._keep += arrs
            q = projs[i]
            q.pre, q.post, q.channel, q.n = p["pre"], p["post"], p["channel"], len(arrs[0])
            q.pre_idx, q.post_idx = _p(arrs[0], C.c_uint32), _p(arrs[1], C.c_uint32)
            q.weight, q.delay = _p(arrs[2], C.c_float), _p(arrs[3], C.c_uint8)
        srcs = (Src * max(1, len(desc["srcs"])))()
        for i, s in enumerate(desc["srcs"]):
            ids = np.ascontiguousarray(s["ids"], np.uint32)
            self._keep.append(ids)
            q = srcs[i]
            q.pop, q.kind, q.rate_hz = s["pop"], s["kind"], s["rate_hz"]
            q.phase_ms, q.win_period_ms = s["phase_ms"], s["win_period_ms"]
            q.win_start_ms, q.win_end_ms = s["win_start_ms"], s["win_end_ms"]
            q.n_ids, q.ids = len(ids), _p(ids, C.c_uint32)
        plast_list = desc.get("plast", [])
        plast = (Plast * max(1, len(plast_list)))()
        for i, q in enumerate(plast_list):
            plast[i] = Plast(q["proj"], q["rule"], q["teacher"], q["window"], q["a0"], q["a1_i"],
                             q["a1_j"], q["a2_ji"], q["v_max"], 0.0)
        self._keep += [pops, projs, srcs, plast]
        self.n_syn = [len(p["pre_idx"]) for p in desc["projs"]]
        self.net = Net(len(desc["pops"]), len(desc["projs"]), len(desc["srcs"]), substeps, pops,
                       projs, srcs, dt_ms, seed, int(bf16), mode, len(plast_list), 0, plast)
        self.n_pops = len(desc["pops"])
        self.n_cells = sum(p["num"] for p in desc["pops"])
        h = C.c_void_p()
        rc = lib().orc_create(C.byref(self.net), C.byref(h))
        if rc:
            raise RuntimeError(f"orc_create failed ({rc})")
        self._h = h

    def close(self):
        if getattr(self, "_h", None):
            lib().orc_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def scale_bits(self, pop, ch):
        return lib().orc_scale_bits(C.byref(self.net), pop, ch)

    def set_rates(self, rates):
        r = np.ascontiguousarray(rates, np.float32)
        self._keep.append(r)
        lib().orc_set_rates(self._h, _p(r, C.c_float))

    def run(self, n_steps, raster_cap=None):
        counts = np.zeros((n_steps, self.n_pops), np.uint32)
        cap = raster_cap if raster_cap is not None else max(1 << 16, n_steps * 64)
        ras = np.zeros(cap, np.uint32)
        off = np.zeros(n_steps + 1, np.int64)
        rc = lib().orc_run(self._h, n_steps, _p(counts, C.c_uint32), _p(ras, C.c_uint32), cap,
                           _p(off, C.c_int64))
        if rc:
            raise RuntimeError(f"orc_run failed ({rc}): raster capacity {cap} too small")
        return counts, (ras[: off[-1]].copy(), off)

    def state(self):
        u = np.empty(self.n_cells, np.float32)
        g = np.empty((self.n_cells, 2), np.float32)
        ref = np.empty(self.n_cells, np.int32)
        lib().orc_get_state(self._h, _p(u, C.c_float), _p(g, C.c_float), _p(ref, C.c_int32))
        return u, g, ref

    def set_state(self, u, g, ref):
        u = np.ascontiguousarray(u, np.float32)
        g = np.ascontiguousarray(g, np.float32)
        ref = np.ascontiguousarray(ref, np.int32)
        lib().orc_set_state(self._h, _p(u, C.c_float), _p(g, C.c_float), _p(ref, C.c_int32))

    def events(self):
        return lib().orc_events(self._h)

    def plastic_values(self, proj):
        v = np.empty(max(self.n_syn[proj], 1), np.float32)
        if lib().orc_plastic_values(self._h, proj, _p(v, C.c_float)):
            raise RuntimeError(f"projection {proj} is not plastic")
        return v[: self.n_syn[proj]]


def describe(net) -> dict:
    """Raw description of a scaffold_gb300.Network for the oracle."""
    pops = []
    for p in net.populations:
        pops.append(dict(num=p.num, is_input=p.dev_type == 1, Cm=p.Cm, El=p.El, dt_ref=p.dt_ref,
                         Ie=p.Ie, Vr=p.Vr, Vth=p.Vth, gL=p.gL, channels=p.channels))
    projs = []
    for pr in net.projections:
        pre, post, w, d = net.synapses(pr.index)
        projs.append(dict(pre=pr.pre, post=pr.post, channel=pr.channel, pre_idx=pre,
                          post_idx=post, weight=w, delay=d))
    srcs = []
    for pop, prm, ids in net.inputs():
        srcs.append(dict(pop=pop, ids=ids, **prm))
    plast = []
    for pr in net.projections:
        q = net.plasticity(pr.index)
        if q is not None:
            plast.append(dict(proj=pr.index, **q))
    return dict(pops=pops, projs=projs, srcs=srcs, plast=plast)


_LIF = dict(Cm=3.0, El=-70.0, dt_ref=2.0, Ie=0.0, Vr=-70.0, Vth=-50.0,
            gL=float(np.float32(0.2)), channels=[(1.0, 0.0, 1.0, 0.5), (1.0, -80.0, 1.0, 10.0)])
_INPUT = dict(Cm=0.0, El=0.0, dt_ref=0.0, Ie=0.0, Vr=0.0, Vth=0.0, gL=0.0, channels=[])


def random_projection(npre, npost, in_degree, w_mean, seed, w_lo=0.5, w_hi=1.5, d_min=1,
                      d_max=4):
    """Fixed in-degree projection drawn by the oracle's generator (netgen.c):
    (pre_idx, post_idx, weight, delay) arrays, post-major, pre ids ascending."""
    L = lib()
    L.orc_random_projection.argtypes = [C.c_int64, C.c_int64, C.c_int32, C.c_float, C.c_float,
                                        C.c_float, C.c_int32, C.c_int32, C.c_uint64,
                                        C.POINTER(C.c_uint32), C.POINTER(C.c_uint32),
                                        C.POINTER(C.c_float), C.POINTER(C.c_uint8)]
    n = int(npost) * int(in_degree)
    pre = np.empty(n, np.uint32)
    post = np.empty(n, np.uint32)
    w = np.empty(n, np.float32)
    d = np.empty(n, np.uint8)
    rc = L.orc_random_projection(npre, npost, in_degree, w_mean, w_lo, w_hi, d_min, d_max,
                                 seed & 0xFFFFFFFFFFFFFFFF, _p(pre, C.c_uint32),
                                 _p(post, C.c_uint32), _p(w, C.c_float), _p(d, C.c_uint8))
    if rc:
        raise RuntimeError(f"orc_random_projection failed ({rc})")
    return pre, post, w, d


def scaffold_desc(config: int, scale: float = 1.0, seed: int = 1) -> dict:
    """Description (as `describe`) of benchmark scaffold `config` (1, 2 or 5)
    at population scale `scale`, drawn from `seed` by the oracle's own
    generator: the same network the library builds for these arguments,
    without loading the library."""
    L = lib()
    L.orc_scaffold_spec.argtypes = [C.c_int32, C.c_double, C.POINTER(C.c_int32),
                                    C.POINTER(C.c_int32), C.POINTER(C.c_float),
                                    C.POINTER(C.c_int32)]
    sizes = np.zeros(7, np.int32)
    proj = np.zeros(44, np.int32)
    drive = np.zeros(11, np.float32)
    burst = C.c_int32()
    if L.orc_scaffold_spec(config, scale, _p(sizes, C.c_int32), _p(proj, C.c_int32),
                           _p(drive, C.c_float), C.byref(burst)):
        raise ValueError(f"unknown scaffold config {config} or scale {scale}")
    pops = [dict(num=int(sizes[0]), is_input=True, **_INPUT)]
    pops += [dict(num=int(n), is_input=False, **_LIF) for n in sizes[1:]]
    projs = []
    for j in range(11):
        pre, post, k, ch = (int(x) for x in proj[4 * j: 4 * j + 4])
        mean = float(drive[j] / np.float32(k)) if k > 0 else 0.0
        pj_seed = (seed * 1000003 + j + 1) & 0xFFFFFFFFFFFFFFFF
        a, b, w, d = random_projection(int(sizes[pre]), int(sizes[post]), k, mean, pj_seed)
        projs.append(dict(pre=pre, post=post, channel=ch, pre_idx=a, post_idx=b, weight=w,
                          delay=d))
    srcs = [dict(pop=0, ids=np.arange(sizes[0], dtype=np.uint32), kind=0, rate_hz=4.0,
                 phase_ms=0.0, win_period_ms=0.0, win_start_ms=0.0, win_end_ms=0.0)]
    if burst.value:
        srcs.append(dict(pop=0, ids=np.arange(burst.value, dtype=np.uint32), kind=0,
                         rate_hz=100.0, phase_ms=0.0, win_period_ms=1000.0, win_start_ms=260.0,
                         win_end_ms=300.0))
    return dict(pops=pops, projs=projs, srcs=srcs, plast=[])


def desc_counts(desc: dict):
    """(cells, synapses) of a description."""
    return (sum(p["num"] for p in desc["pops"]), sum(len(p["pre_idx"]) for p in desc["projs"]))


REF_DIR = os.path.join(HERE, "_ref")


class _CpuRef:
    """Shared wrapper of the reference-CPU-path restatement (rp_*) and of the
    harness around the reference's compiled functions (rh_*)."""

    prefix = "rp"

    def __init__(self, desc: dict, lib_, *, dt_ms=0.1, substeps=1, seed=1, bf16=False):
        self._o = Oracle(desc, dt_ms=dt_ms, substeps=substeps, seed=seed, bf16=bf16)
        self._o.close()  # only its ctypes description is reused
        self.L = lib_
        p = self.prefix
        getattr(self.L, f"{p}_create").argtypes = [C.POINTER(Net), C.POINTER(C.c_void_p)]
        getattr(self.L, f"{p}_run").argtypes = [C.c_void_p, C.c_int64, C.c_int32,
                                                C.POINTER(C.c_uint32), C.POINTER(C.c_uint32),
                                                C.c_int64, C.POINTER(C.c_int64)]
        getattr(self.L, f"{p}_get_state").argtypes = [C.c_void_p, C.POINTER(C.c_float),
                                                      C.POINTER(C.c_float), C.POINTER(C.c_int32)]
        getattr(self.L, f"{p}_destroy").argtypes = [C.c_void_p]
        self.n_pops, self.n_cells = self._o.n_pops, self._o.n_cells
        h = C.c_void_p()
        rc = getattr(self.L, f"{p}_create")(C.byref(self._o.net), C.byref(h))
        if rc:
            raise RuntimeError(f"{p}_create failed ({rc})")
        self._h = h

    def run(self, n_steps, threads=0, raster_cap=None):
        counts = np.zeros((n_steps, self.n_pops), np.uint32)
        cap = raster_cap if raster_cap is not None else max(1 << 16, n_steps * 64)
        ras = np.zeros(cap, np.uint32)
        off = np.zeros(n_steps + 1, np.int64)
        rc = getattr(self.L, f"{self.prefix}_run")(self._h, n_steps, threads,
                                                   _p(counts, C.c_uint32), _p(ras, C.c_uint32),
                                                   cap, _p(off, C.c_int64))
        if rc:
            raise RuntimeError(f"{self.prefix}_run failed ({rc})")
        return counts, (ras[: off[-1]].copy(), off)

    def state(self):
        u = np.empty(self.n_cells, np.float32)
        g = np.empty((self.n_cells, 2), np.float32)
        ref = np.empty(self.n_cells, np.int32)
        getattr(self.L, f"{self.prefix}_get_state")(self._h, _p(u, C.c_float), _p(g, C.c_float),
                                                    _p(ref, C.c_int32))
        return u, g, ref

    def close(self):
        if getattr(self, "_h", None):
            getattr(self.L, f"{self.prefix}_destroy")(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class RefPort(_CpuRef):
    """C restatement of the reference's CPU loops (liboracle.so)."""

    prefix = "rp"

    def __init__(self, desc, **kw):
        super().__init__(desc, lib(), **kw)


def ref_harness_path(substeps: int = 1) -> str:
    return os.path.join(REF_DIR, f"libref_harness_s{substeps}.so")


def have_ref_harness(substeps: int = 1) -> bool:
    return os.path.exists(ref_harness_path(substeps))


class RefHarness(_CpuRef):
    """The reference's own compiled CPU functions (oracle/_ref, built here only)."""

    prefix = "rh"

    def __init__(self, desc, **kw):
        path = ref_harness_path(kw.get("substeps", 1))
        if not os.path.exists(path):
            raise RuntimeError(f"{path} is not built (reference sources absent)")
        super().__init__(desc, C.CDLL(path), **kw)
