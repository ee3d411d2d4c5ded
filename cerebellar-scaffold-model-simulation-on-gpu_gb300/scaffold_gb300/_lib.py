"""ctypes binding of libscaffold_gb300.so (declarations: include/scaffold_gb300.h).

The library is loaded from this package directory only; there is no fallback:
if it is missing, every call raises immediately.
"""
from __future__ import annotations

import ctypes as C
import os

LIB_PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "libscaffold_gb300.so")

SGB_OK = 0
ERRORS = {
    -1: "SGB_ERR_ARG", -2: "SGB_ERR_IO", -3: "SGB_ERR_FORMAT", -4: "SGB_ERR_RANGE",
    -5: "SGB_ERR_CUDA", -6: "SGB_ERR_STATE", -7: "SGB_ERR_OVERFLOW", -8: "SGB_ERR_DEVICE",
    -9: "SGB_ERR_NOMEM", -10: "SGB_ERR_UNSUPPORTED",
}
NORMAL, INPUT, OUTPUT = 0, 1, 2
CH_EXC, CH_INH = 0, 1
PROP_AUTO, PROP_CSR, PROP_ELL = 0, 1, 2
STDP_HEBB, STDP_TEACHER = 0, 1
WEIGHT_FP32, WEIGHT_BF16 = 0, 1
EXEC_GRAPH, EXEC_PERSISTENT, EXEC_STREAM = 0, 1, 2
INPUT_POISSON, INPUT_PERIODIC = 0, 1
KCLASS_COUNT = 4
KERNEL_NAMES = {0: "k_update+k_deliver", 1: "k_persistent", 2: "k_persistent_resident",
                3: "k_persistent_fused"}


class SgbError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{ERRORS.get(code, code)}: {msg}")
        self.code = code


class Config(C.Structure):
    _fields_ = [("dt_ms", C.c_double), ("substeps", C.c_int32), ("weight_type", C.c_int32),
                ("exec_mode", C.c_int32), ("chunk_steps", C.c_int32), ("device", C.c_int32),
                ("default_prop", C.c_int32), ("raster", C.c_int32), ("blocks_per_sm", C.c_int32),
                ("l2_persist", C.c_int32), ("barrier_test_extra", C.c_int32),
                ("reserved", C.c_int32 * 6)]


class InputParams(C.Structure):
    _fields_ = [("kind", C.c_int32), ("rate_hz", C.c_float), ("phase_ms", C.c_double),
                ("win_period_ms", C.c_double), ("win_start_ms", C.c_double),
                ("win_end_ms", C.c_double)]


class PlasticityParams(C.Structure):
    _fields_ = [("rule", C.c_int32), ("teacher_proj", C.c_int32), ("window_steps", C.c_int32),
                ("a0", C.c_float), ("a1_i", C.c_float), ("a1_j", C.c_float), ("a2_ji", C.c_float),
                ("v_max", C.c_float)]


class PopulationInfo(C.Structure):
    _fields_ = [("num", C.c_int32), ("dev_type", C.c_int32), ("c_num", C.c_int32),
                ("n_in_projections", C.c_int32), ("Cm", C.c_float), ("El", C.c_float),
                ("dt_ref", C.c_float), ("Ie", C.c_float), ("Vr", C.c_float), ("Vth", C.c_float),
                ("gL", C.c_float), ("ch_w", C.c_float * 2), ("ch_E", C.c_float * 2),
                ("ch_gbar", C.c_float * 2), ("ch_tau", C.c_float * 2), ("name", C.c_char * 32)]


class ProjectionInfo(C.Structure):
    _fields_ = [("pre_pop", C.c_int32), ("post_pop", C.c_int32), ("channel", C.c_int32),
                ("mode", C.c_int32), ("n_synapses", C.c_int64), ("max_in_degree", C.c_int32),
                ("max_out_degree", C.c_int32), ("min_delay", C.c_int32),
                ("max_delay", C.c_int32), ("name", C.c_char * 32)]


class InputInfo(C.Structure):
    _fields_ = [("pop", C.c_int32), ("n_ids", C.c_int32), ("params", InputParams)]


class SegmentInfo(C.Structure):
    _fields_ = [("net", C.c_int32), ("pop", C.c_int32), ("dev_type", C.c_int32),
                ("count", C.c_int32), ("first_id", C.c_int64), ("scale_bits", C.c_int32 * 2)]


class SimInfo(C.Structure):
    _fields_ = [("n_nets", C.c_int32), ("n_segments", C.c_int32), ("n_projections", C.c_int32),
                ("ring_slots", C.c_int32), ("n_neurons", C.c_int64), ("n_synapses", C.c_int64),
                ("step", C.c_int64), ("device_bytes", C.c_int64), ("exec_mode", C.c_int32),
                ("weight_type", C.c_int32), ("substeps", C.c_int32), ("chunk_steps", C.c_int32),
                ("dt_ms", C.c_double), ("events", C.c_int64), ("delivered", C.c_int64),
                ("step_kernel", C.c_int32), ("push_smem_bytes", C.c_int32), ("pulled", C.c_int64),
                ("pull_entries", C.c_int64), ("l2_persist_bytes", C.c_int64),
                ("shard_cells", C.c_int64), ("item_width", C.c_int32),
                ("deliver_blocks", C.c_int32), ("pull_summary", C.c_int32),
                ("spike_ahead", C.c_int32), ("lane_cells", C.c_int32),
                ("reserved_", C.c_int32)]


P = C.POINTER
vp = C.c_void_p
i32, i64, u64, f32, f64 = C.c_int32, C.c_int64, C.c_uint64, C.c_float, C.c_double
u8p, u32p, i32p, i64p, f32p, f64p = P(C.c_uint8), P(C.c_uint32), P(C.c_int32), P(C.c_int64), P(C.c_float), P(C.c_double)

# name -> (restype, argtypes); the complete exported surface of the header.
PROTOTYPES = {
    "sgb_config_init": (None, [P(Config)]),
    "sgb_last_error": (C.c_char_p, []),
    "sgb_abi_version": (i32, []),
    "sgb_net_create": (C.c_int, [P(vp)]),
    "sgb_net_destroy": (None, [vp]),
    "sgb_net_add_population": (C.c_int, [vp, C.c_char_p, i32, f32, f32, f32, f32, f32, f32, f32,
                                          i32, i32, f32p, i32p]),
    "sgb_net_add_projection_dat": (C.c_int, [vp, C.c_char_p, i32, i32, f32, i32, i32, i32p]),
    "sgb_net_add_projection_arrays": (C.c_int, [vp, i32, i32, i64, u32p, u32p, f32p, u8p, i32,
                                                i32, i32, i32p]),
    "sgb_net_add_projection_random": (C.c_int, [vp, i32, i32, i32, f32, f32, f32, i32, i32, i32,
                                                u64, i32, i32p]),
    "sgb_net_add_input": (C.c_int, [vp, i32, i64, u32p, P(InputParams), i32p]),
    "sgb_net_add_input_dat": (C.c_int, [vp, C.c_char_p, i32, P(InputParams), i32p]),
    "sgb_net_build_scaffold": (C.c_int, [vp, i32, f64, u64]),
    "sgb_net_build_reference_scaffold": (C.c_int, [vp, C.c_char_p, i32p]),
    "sgb_reference_type_id": (i32, [i32]),
    "sgb_sim_write_raster": (C.c_int, [vp, C.c_char_p, u32p, i64p, i64, i64, i32p, i32]),
    "sgb_net_counts": (C.c_int, [vp, i32p, i32p, i32p, i64p, i64p]),
    "sgb_net_population_info": (C.c_int, [vp, i32, P(PopulationInfo)]),
    "sgb_net_projection_info": (C.c_int, [vp, i32, P(ProjectionInfo)]),
    "sgb_net_projection_synapses": (C.c_int, [vp, i32, u32p, u32p, f32p, u8p]),
    "sgb_net_input_info": (C.c_int, [vp, i32, P(InputInfo)]),
    "sgb_net_input_ids": (C.c_int, [vp, i32, u32p]),
    "sgb_net_write_projection_dat": (C.c_int, [vp, i32, C.c_char_p]),
    "sgb_net_add_plasticity": (C.c_int, [vp, i32, P(PlasticityParams)]),
    "sgb_net_plasticity_info": (C.c_int, [vp, i32, i32p, P(PlasticityParams)]),
    "sgb_sim_plastic_values": (C.c_int, [vp, i32, i32, f32p]),
    "sgb_sim_checkpoint_size": (C.c_int, [vp, i64p]),
    "sgb_sim_save_checkpoint": (C.c_int, [vp, vp, i64]),
    "sgb_sim_load_checkpoint": (C.c_int, [vp, vp, i64]),
    "sgb_sim_create": (C.c_int, [P(Config), P(vp), P(C.c_uint64), i32, P(vp)]),
    "sgb_sim_destroy": (None, [vp]),
    "sgb_sim_set_stream": (C.c_int, [vp, vp]),
    "sgb_sim_set_input_rates": (C.c_int, [vp, i32, i32, f32p]),
    "sgb_sim_run": (C.c_int, [vp, i64, u32p, u32p, i64, i64p]),
    "sgb_sim_enqueue": (C.c_int, [vp, i64]),
    "sgb_sim_sync": (C.c_int, [vp]),
    "sgb_sim_reset": (C.c_int, [vp, P(C.c_uint64)]),
    "sgb_sim_get_info": (C.c_int, [vp, P(SimInfo)]),
    "sgb_sim_segment_info": (C.c_int, [vp, i32, P(SegmentInfo)]),
    "sgb_sim_get_state": (C.c_int, [vp, f32p, f32p, i32p]),
    "sgb_sim_set_state": (C.c_int, [vp, f32p, f32p, i32p]),
    "sgb_sim_spike_totals": (C.c_int, [vp, f64p]),
    "sgb_sim_set_propagation": (C.c_int, [vp, i32, i32, i32]),
    "sgb_sim_get_propagation": (C.c_int, [vp, i32, i32, i32p]),
    "sgb_sim_autotune": (C.c_int, [vp, i32, C.c_char_p]),
    "sgb_sim_launch_count": (C.c_int, [vp, i64p]),
    "sgb_sim_profile": (C.c_int, [vp, i32, f64p, f64p, i64p]),
    "sgb_deliver_spikes": (C.c_int, [vp, i32, vp, vp, vp, i32, vp, i32, i64, vp]),
    "sgb_deliver_spikes_static": (C.c_int, [vp, i32, vp, vp, vp, i32, vp, i32, i64, vp]),
}

_lib = None


def lib() -> C.CDLL:
    """Loads the in-tree library (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"{LIB_PATH} is missing: build it with build.py first")
        L = C.CDLL(LIB_PATH)
        for name, (res, args) in PROTOTYPES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def check(rc: int) -> None:
    if rc != SGB_OK:
        raise SgbError(rc, (lib().sgb_last_error() or b"").decode(errors="replace"))
