"""GB300 cerebellar-scaffold simulation hot path (C ABI in libscaffold_gb300.so)."""
from ._lib import (CH_EXC, CH_INH, EXEC_GRAPH, EXEC_PERSISTENT, EXEC_STREAM, INPUT,
                   INPUT_PERIODIC, INPUT_POISSON, NORMAL, OUTPUT, PROP_AUTO, PROP_CSR, PROP_ELL,
                   STDP_HEBB, STDP_TEACHER, WEIGHT_BF16, WEIGHT_FP32, SgbError, lib)
from .network import Network, Simulation
from .configs import (batched_scales, reference_scaffold, reference_sizes, scaffold,
                      write_reference_dat)

__all__ = [
    "CH_EXC", "CH_INH", "EXEC_GRAPH", "EXEC_PERSISTENT", "EXEC_STREAM", "INPUT", "INPUT_PERIODIC",
    "INPUT_POISSON", "NORMAL", "OUTPUT", "PROP_AUTO", "PROP_CSR", "PROP_ELL", "STDP_HEBB",
    "STDP_TEACHER", "WEIGHT_BF16",
    "WEIGHT_FP32", "SgbError", "lib", "Network", "Simulation", "scaffold", "batched_scales",
    "reference_scaffold", "reference_sizes", "write_reference_dat",
]
