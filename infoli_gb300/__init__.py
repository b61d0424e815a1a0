"""GB300-native InfOli per-timestep network update.

The compute path is libinfoli_gpu.so (hand-written CUDA for sm_103a behind a
C ABI, include/infoli_gpu.h).  This package only binds it (capi) and builds
it (build); there is no CPU implementation of the step here.
"""
from . import capi  # noqa: F401
from .capi import (  # noqa: F401
    Batch, InfoliError, Server, Simulation, S, STATE_NAMES, TRACE_AXON, TRACE_DEND, TRACE_SOMA, batch_tune_sample,
    bitmask_to_csr,
    device_count, format_f8, format_row, gen_bitmask, gen_bitmask_csr, gen_fixed_degree, gen_grid_gaussian, gen_uniform,
    random_init, read_conn_dense, read_conn_triples, read_gcal, read_parameters, read_stim_file,
)

__all__ = [
    "capi", "Batch", "batch_tune_sample", "InfoliError", "Server", "Simulation", "gen_bitmask", "gen_bitmask_csr", "S", "STATE_NAMES", "TRACE_AXON", "TRACE_SOMA",
    "TRACE_DEND", "bitmask_to_csr", "device_count", "format_f8", "format_row", "gen_fixed_degree",
    "gen_grid_gaussian", "gen_uniform", "random_init", "read_conn_dense", "read_conn_triples", "read_gcal",
    "read_parameters", "read_stim_file",
]
