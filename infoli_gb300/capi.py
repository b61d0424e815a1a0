"""ctypes binding of libinfoli_gpu.so (include/infoli_gpu.h).

This is the Python side of the drop-in boundary: it calls exactly the C entry
points a C host (infoli.x) or any other FFI would call.  There is no CPU
fallback: if the shared library is missing the import fails loudly, and every
GPU entry point reports the CUDA error of the box it runs on.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_build", "libinfoli_gpu.so")

NPARAM = 23
NSTATE = 19
NCONF = 42
TRACE_AXON, TRACE_SOMA, TRACE_DEND = 1, 2, 4
F_KAHAN = 1

OK = 0
ERR_ARG, ERR_CUDA, ERR_NOMEM, ERR_TIMEOUT = -1, -2, -3, -4
ERR_FILE, ERR_CONFIG, ERR_CAPACITY, ERR_STATE = -5, -6, -7, -8

STATE_NAMES = [
    "V_dend", "Calcium_r", "Potassium_s", "Hcurrent_q", "Ca2Plus", "I_CaH", "g_CaL",
    "V_soma", "Sodium_m", "Sodium_h", "Potassium_n", "Potassium_p", "Potassium_x_s",
    "Calcium_k", "Calcium_l", "V_axon", "Sodium_m_a", "Sodium_h_a", "Potassium_x_a",
]
S = {name: i for i, name in enumerate(STATE_NAMES)}

# Every symbol the header declares; tests check the library exports all of them.
EXPORTED = [
    "infoli_last_error", "infoli_version", "infoli_build_info", "infoli_device_count",
    "infoli_read_parameters", "infoli_read_gcal", "infoli_gen_uniform", "infoli_gen_grid_gaussian",
    "infoli_gen_fixed_degree", "infoli_bitmask_to_csr", "infoli_sim_create",
    "infoli_sim_set_stimulus_pulse", "infoli_sim_set_stimulus_cells", "infoli_sim_run",
    "infoli_sim_run_into", "infoli_sim_get_state", "infoli_sim_set_state", "infoli_sim_step",
    "infoli_sim_last_run_stats", "infoli_sim_plan_info", "infoli_sim_destroy", "infoli_format_f8",
    "infoli_format_row", "infoli_sim_set_profiling", "infoli_sim_get_profile", "infoli_plan_emulate", "infoli_plan_locality_order",
    "infoli_run_noalloc", "infoli_sim_launch", "infoli_sim_query", "infoli_sim_sync",
    "infoli_sim_memory", "infoli_gen_bitmask_csr",
    "infoli_read_conn_dense", "infoli_read_conn_triples", "infoli_read_stim_file", "infoli_random_init",
    "infoli_sim_set_stimulus_table", "infoli_gen_bitmask", "infoli_batch_create", "infoli_batch_set_stimulus_pulse",
    "infoli_batch_run", "infoli_batch_get_state", "infoli_batch_set_state", "infoli_batch_info",
    "infoli_batch_cta_info",
    "infoli_batch_destroy", "infoli_batch_autotune", "infoli_batch_tune_sample", "infoli_server_create", "infoli_server_submit", "infoli_server_poll",
    "infoli_server_wait", "infoli_server_status", "infoli_server_destroy",
]


class InfoliError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"infoli error {code}: {msg}")
        self.code = code


class SimDesc(C.Structure):
    _fields_ = [
        ("n_cells", C.c_int),
        ("params", C.c_void_p),
        ("init_state", C.c_void_p),
        ("init_values", C.c_void_p),
        ("row_ptr", C.c_void_p),
        ("col", C.c_void_p),
        ("g", C.c_void_p),
        ("g_uniform", C.c_float),
        ("flags", C.c_int),
        ("device", C.c_int),
        ("grid", C.c_int),
    ]


class BatchDesc(C.Structure):
    _fields_ = [
        ("n_nets", C.c_int),
        ("n_cells", C.c_void_p),
        ("params", C.c_void_p),
        ("init_state", C.c_void_p),
        ("init_values", C.c_void_p),
        ("bits", C.c_void_p),
        ("g", C.c_void_p),
        ("flags", C.c_int),
        ("device", C.c_int),
        ("block", C.c_int),
        ("residency", C.c_int),
    ]


RES_FIT, RES_OCC, RES_NONE = 0, 1, 2
RES_NAMES = {RES_FIT: "fit", RES_OCC: "occupancy", RES_NONE: "none"}
TUNE_CANDIDATES = 5


class BatchTune(C.Structure):
    _fields_ = [
        ("block", C.c_int),
        ("residency", C.c_int),
        ("sample_nets", C.c_int),
        ("sample_cells", C.c_int64),
        ("cand_block", C.c_int * TUNE_CANDIDATES),
        ("cand_residency", C.c_int * TUNE_CANDIDATES),
        ("cand_ms_per_step", C.c_float * TUNE_CANDIDATES),
    ]


class ServerDesc(C.Structure):
    _fields_ = [
        ("params", C.c_void_p),
        ("device", C.c_int),
        ("hbm_budget", C.c_int64),
        ("max_active", C.c_int),
        ("work_per_cta", C.c_int64),
        ("backfill_ms", C.c_int),
        ("prep_threads", C.c_int),
        ("flags", C.c_int),
        ("age_ms", C.c_int),
        ("lane_sms", C.c_int),
        ("lane_chunk_steps", C.c_int),
        ("lane_edges_per_cta", C.c_int),
    ]


class RequestDesc(C.Structure):
    _fields_ = [
        ("n_cells", C.c_int),
        ("row_ptr", C.c_void_p),
        ("col", C.c_void_p),
        ("g", C.c_void_p),
        ("g_uniform", C.c_float),
        ("init_state", C.c_void_p),
        ("init_values", C.c_void_p),
        ("n_steps", C.c_int),
        ("pulse_start", C.c_int),
        ("pulse_end", C.c_int),
        ("pulse_amp", C.c_float),
    ]


class RequestInfo(C.Structure):
    _fields_ = [
        ("id", C.c_int64),
        ("n_cells", C.c_int),
        ("n_steps", C.c_int),
        ("grid", C.c_int),
        ("device_bytes", C.c_int64),
        ("admitted_bytes", C.c_int64),
        ("submit_s", C.c_double),
        ("admit_s", C.c_double),
        ("prepared_s", C.c_double),
        ("start_s", C.c_double),
        ("done_s", C.c_double),
        ("status", C.c_int),
        ("prep_start_s", C.c_double),
        ("lane", C.c_int),
        ("lane_launches", C.c_int),
    ]


TRACE_CB = C.CFUNCTYPE(None, C.c_void_p, C.c_int, C.c_int, C.POINTER(C.c_float), C.c_int)

_lib = None


def load():
    """Load libinfoli_gpu.so (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise ImportError(f"{LIB_PATH} is missing: build it with `python -m infoli_gb300.build`")
    L = C.CDLL(LIB_PATH)
    P, I, I64, F, U = C.c_void_p, C.c_int, C.c_int64, C.c_float, C.c_uint
    sig = {
        "infoli_last_error": ([], C.c_char_p),
        "infoli_version": ([], I),
        "infoli_build_info": ([], C.c_char_p),
        "infoli_device_count": ([], I),
        "infoli_read_parameters": ([C.c_char_p, P], I),
        "infoli_read_gcal": ([C.c_char_p, I, P], I),
        "infoli_gen_uniform": ([I, F, U, P, P, I64, P], I),
        "infoli_gen_grid_gaussian": ([I, I, F, F, C.c_uint64, P, P, I64, P], I),
        "infoli_gen_fixed_degree": ([I, I, F, F, C.c_uint64, P, P, P, I64], I),
        "infoli_bitmask_to_csr": ([I, P, P, P, I64, P], I),
        "infoli_sim_create": ([C.POINTER(SimDesc), C.POINTER(C.c_void_p)], I),
        "infoli_sim_set_stimulus_pulse": ([P, I, I, F], I),
        "infoli_sim_set_stimulus_cells": ([P, P, P, I], I),
        "infoli_sim_run": ([P, I, I, I, TRACE_CB, P], I),
        "infoli_sim_run_into": ([P, I, I, I, P, I64, P], I),
        "infoli_sim_get_state": ([P, P], I),
        "infoli_sim_set_state": ([P, P], I),
        "infoli_sim_step": ([P, P], I),
        "infoli_sim_last_run_stats": ([P, P, P], I),
        "infoli_sim_plan_info": ([P, P, P, P, P, P], I),
        "infoli_sim_destroy": ([P], I),
        "infoli_sim_launch": ([P, I], I),
        "infoli_sim_query": ([P], I),
        "infoli_sim_sync": ([P], I),
        "infoli_sim_memory": ([P, P], I),
        "infoli_plan_emulate": ([I, P, P, P, F, I, I, I, I64, I, P, P, P], I),
        "infoli_plan_locality_order": ([I, P, P, I, I, P, P], I),
        "infoli_run_noalloc": ([P, I, P, P, P, F, I, I, F, P, I, I, P, P], I),
        "infoli_sim_set_profiling": ([P, I], I),
        "infoli_sim_get_profile": ([P, P, P], I),
        "infoli_gen_bitmask": ([I, F, C.c_uint64, P], I),
        "infoli_gen_bitmask_csr": ([I, F, C.c_uint64, P, P, I64, P], I),
        "infoli_read_conn_dense": ([C.c_char_p, I, P, P, P, I64, P], I),
        "infoli_read_conn_triples": ([C.c_char_p, I, P, P, P, I64, P], I),
        "infoli_read_stim_file": ([C.c_char_p, I, P, I64, P], I),
        "infoli_random_init": ([P, I, U, P, I], I),
        "infoli_sim_set_stimulus_table": ([P, P, I, I], I),
        "infoli_batch_create": ([C.POINTER(BatchDesc), C.POINTER(C.c_void_p)], I),
        "infoli_batch_set_stimulus_pulse": ([P, I, I, F], I),
        "infoli_batch_run": ([P, I], I),
        "infoli_batch_get_state": ([P, P], I),
        "infoli_batch_set_state": ([P, P], I),
        "infoli_batch_info": ([P, P, P, P, P, P], I),
        "infoli_batch_cta_info": ([P, P, P, P, P], I),
        "infoli_batch_destroy": ([P], I),
        "infoli_batch_autotune": ([C.POINTER(BatchDesc), I, I, C.POINTER(BatchTune)], I),
        "infoli_batch_tune_sample": ([I, P, I, I64, P], I),
        "infoli_server_create": ([C.POINTER(ServerDesc), C.POINTER(C.c_void_p)], I),
        "infoli_server_submit": ([P, C.POINTER(RequestDesc), P], I),
        "infoli_server_poll": ([P, I64], I),
        "infoli_server_wait": ([P, I64, P, C.POINTER(RequestInfo)], I),
        "infoli_server_status": ([P, P, P, P, P], I),
        "infoli_server_destroy": ([P], I),
        "infoli_format_f8": ([C.c_char_p, F], I),
        "infoli_format_row": ([C.c_char_p, I64, P, I, I, I], I64),
    }
    for name, (args, res) in sig.items():
        fn = getattr(L, name)
        fn.argtypes = args
        fn.restype = res
    _lib = L
    return L


def _p(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def _check(rc):
    if rc < 0:
        raise InfoliError(rc, load().infoli_last_error().decode(errors="replace"))
    return rc


# ---------------------------------------------------------------- host side --

def read_parameters(path: str) -> np.ndarray:
    v = np.zeros(NCONF, dtype=np.float32)
    _check(load().infoli_read_parameters(os.fsencode(path), _p(v)))
    return v


def read_gcal(path: str, g_cal: np.ndarray) -> int:
    assert g_cal.dtype == np.float32 and g_cal.flags.c_contiguous
    return _check(load().infoli_read_gcal(os.fsencode(path), g_cal.size, _p(g_cal)))


def _csr_call(fn, n, *args, cap_hint):
    row_ptr = np.zeros(n + 1, dtype=np.int64)
    cap = max(16, int(cap_hint))
    ne = C.c_int64(0)
    while True:
        col = np.zeros(cap, dtype=np.int32)
        rc = fn(*args, _p(row_ptr), _p(col), cap, C.byref(ne))
        if rc == ERR_CAPACITY:
            cap = int(ne.value)
            continue
        _check(rc)
        return row_ptr, col[: ne.value].copy()


def gen_uniform(n: int, p: float, seed: int):
    """The reference's built-in generator (src/openmp/infoli.c:337-375)."""
    L = load()
    return _csr_call(L.infoli_gen_uniform, n, n, float(np.float32(p)), int(seed) & 0xFFFFFFFF,
                     cap_hint=n * (n - 1) * min(1.0, float(p) * 1.1 + 0.01) + 64)


def gen_grid_gaussian(rows: int, cols: int, sigma: float, radius: float, seed: int):
    L = load()
    cand = rows * cols * (3.2 * radius * radius + 8)
    return _csr_call(L.infoli_gen_grid_gaussian, rows * cols, rows, cols, float(sigma), float(radius),
                     int(seed) & (2**64 - 1), cap_hint=cand)


def gen_fixed_degree(n: int, k: int, seed: int, g_range=None):
    row_ptr = np.zeros(n + 1, dtype=np.int64)
    col = np.zeros(n * k, dtype=np.int32)
    g = np.zeros(n * k, dtype=np.float32) if g_range is not None else None
    lo, hi = g_range if g_range is not None else (0.0, 0.0)
    _check(load().infoli_gen_fixed_degree(n, k, float(lo), float(hi), int(seed) & (2**64 - 1),
                                          _p(row_ptr), _p(col), _p(g), n * k))
    return row_ptr, col, g


def bitmask_to_csr(n: int, bits: np.ndarray):
    bits = np.ascontiguousarray(bits, dtype=np.uint32)
    assert bits.size == n * ((n + 31) // 32)
    L = load()
    return _csr_call(L.infoli_bitmask_to_csr, n, n, _p(bits), cap_hint=int(np.unpackbits(
        bits.view(np.uint8)).sum()) + 16)


def _read_conn(fn, path, n):
    row_ptr = np.zeros(n + 1, dtype=np.int64)
    ne = C.c_int64(0)
    cap = 0
    while True:
        col = np.zeros(max(cap, 1), dtype=np.int32)
        g = np.zeros(max(cap, 1), dtype=np.float32)
        rc = fn(os.fsencode(path), n, _p(row_ptr), _p(col), _p(g), cap, C.byref(ne))
        if rc == ERR_CAPACITY and cap < ne.value:
            cap = int(ne.value)
            continue
        _check(rc)
        return row_ptr, col[: ne.value].copy(), g[: ne.value].copy()


def read_conn_dense(path: str, n: int):
    """(row_ptr, col, g) from an n x n conductance matrix file (row = sender)."""
    return _read_conn(load().infoli_read_conn_dense, path, n)


def read_conn_triples(path: str, n: int):
    """(row_ptr, col, g) from a "send rec g" triples file."""
    return _read_conn(load().infoli_read_conn_triples, path, n)


def read_stim_file(path: str, n: int) -> np.ndarray:
    """[rows, n] float32 per-step stimulus table."""
    L = load()
    rows = C.c_int64(0)
    rc = L.infoli_read_stim_file(os.fsencode(path), n, None, 0, C.byref(rows))
    if rc != ERR_CAPACITY:
        _check(rc)
    tab = np.zeros((rows.value, n), dtype=np.float32)
    _check(L.infoli_read_stim_file(os.fsencode(path), n, _p(tab), rows.value, C.byref(rows)))
    return tab


def random_init(params, state: np.ndarray, seed: int, device: int = 0) -> np.ndarray:
    """Randomised initial state (infoli_random_init); returns a new [19, n] array."""
    st = np.ascontiguousarray(state, dtype=np.float32).copy()
    prm = np.ascontiguousarray(params, dtype=np.float32)[:NPARAM].copy()
    _check(load().infoli_random_init(_p(prm), st.shape[1], int(seed) & 0xFFFFFFFF, _p(st), int(device)))
    return st


def format_f8(v: float) -> str:
    buf = C.create_string_buffer(64)
    k = load().infoli_format_f8(buf, float(v))
    return buf.raw[:k].decode()


def format_row(values: np.ndarray, tagged: bool, nthreads: int = 0) -> str:
    v = np.ascontiguousarray(values, dtype=np.float32)
    cap = 40 * v.size + 64
    buf = C.create_string_buffer(cap)
    k = _check(load().infoli_format_row(buf, cap, _p(v), v.size, int(bool(tagged)), nthreads))
    return buf.raw[:k].decode()


def plan_emulate(n, row_ptr, col, vdend, g=None, g_uniform=0.04, grid=0, grid_max=152, threads=1024,
                 smem_budget=232448 - 1024, sync_mode=0):
    """Host walk of the planner's tables (infoli_plan_emulate): (I_c[n], info dict)."""
    row_ptr = np.ascontiguousarray(row_ptr, dtype=np.int64)
    col = np.ascontiguousarray(col, dtype=np.int32)
    g = None if g is None else np.ascontiguousarray(g, dtype=np.float32)
    v = np.ascontiguousarray(vdend, dtype=np.float32)
    out = np.zeros(n, dtype=np.float32)
    info = np.zeros(10, dtype=np.int64)
    rc = load().infoli_plan_emulate(n, _p(row_ptr), _p(col) if col.size else None, _p(g), float(g_uniform),
                                    grid, grid_max, threads, int(smem_budget), sync_mode, _p(v), _p(out),
                                    _p(info))
    if rc != 0:
        raise InfoliError(rc, f"plan emulation failed with code {rc}")
    keys = ("ctas", "stamped", "tiles", "chunks", "max_slots", "smem_bytes", "probes", "resident",
            "gather_wavefronts", "gathers")
    d = dict(zip(keys, info.tolist()))
    if d["stamped"] == 1:
        d["relabelled"] = bool(d.pop("tiles"))
    return out, d


def plan_locality_order(n, row_ptr, col, parts, threads=512):
    """The planner's locality-preserving cell order (infoli_plan_locality_order):
    (order[new] = old cell, starts[parts + 1]) or None when no order exists."""
    row_ptr = np.ascontiguousarray(row_ptr, dtype=np.int64)
    col = np.ascontiguousarray(col, dtype=np.int32)
    order = np.zeros(n, dtype=np.int32)
    starts = np.zeros(parts + 1, dtype=np.int32)
    rc = load().infoli_plan_locality_order(int(n), _p(row_ptr), _p(col) if col.size else None, int(parts),
                                           int(threads), _p(order), _p(starts))
    return None if rc != 0 else (order, starts)


def device_count() -> int:
    return _check(load().infoli_device_count())


# --------------------------------------------------------------- simulation --

class Simulation:
    """One network on the GPU (infoli_sim_* handle)."""

    def __init__(self, n, params, row_ptr, col, g=None, g_uniform=None, init_state=None,
                 init_values=None, kahan=False, device=0, grid=0):
        L = load()
        self._L = L
        params = np.ascontiguousarray(params, dtype=np.float32)
        assert params.size >= NPARAM
        self.params = params[:NPARAM].copy()
        self.n = int(n)
        self.row_ptr = np.ascontiguousarray(row_ptr, dtype=np.int64)
        self.col = np.ascontiguousarray(col, dtype=np.int32)
        self.g = None if g is None else np.ascontiguousarray(g, dtype=np.float32)
        d = SimDesc()
        d.n_cells = self.n
        d.params = _p(self.params)
        st = None
        iv = None
        if init_state is not None:
            st = np.ascontiguousarray(init_state, dtype=np.float32).reshape(NSTATE, self.n)
            d.init_state = _p(st)
        else:
            iv = np.ascontiguousarray(init_values, dtype=np.float32)
            assert iv.size == NSTATE
            d.init_values = _p(iv)
        d.row_ptr = _p(self.row_ptr)
        d.col = _p(self.col) if self.col.size else None
        d.g = _p(self.g)
        d.g_uniform = float(self.params[1] if g_uniform is None else g_uniform)
        d.flags = F_KAHAN if kahan else 0
        d.device = int(device)
        d.grid = int(grid)
        h = C.c_void_p()
        _check(L.infoli_sim_create(C.byref(d), C.byref(h)))
        self._h = h

    def close(self):
        if getattr(self, "_h", None):
            self._L.infoli_sim_destroy(self._h)
            self._h = None

    __del__ = close

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def set_stimulus_pulse(self, start, end, amp):
        _check(self._L.infoli_sim_set_stimulus_pulse(self._h, int(start), int(end), float(amp)))

    def set_stimulus_table(self, table, first_step=0):
        self._tab = np.ascontiguousarray(table, dtype=np.float32)
        assert self._tab.ndim == 2 and self._tab.shape[1] == self.n
        _check(self._L.infoli_sim_set_stimulus_table(self._h, _p(self._tab), self._tab.shape[0], int(first_step)))

    def set_stimulus_cells(self, amp, onset, duration):
        self._amp = np.ascontiguousarray(amp, dtype=np.float32)
        self._onset = np.ascontiguousarray(onset, dtype=np.int32)
        _check(self._L.infoli_sim_set_stimulus_cells(self._h, _p(self._amp), _p(self._onset),
                                                     int(duration)))

    @property
    def step(self) -> int:
        v = C.c_int(0)
        _check(self._L.infoli_sim_step(self._h, C.byref(v)))
        return v.value

    def run(self, n_steps, trace_every=0, what=TRACE_AXON):
        """Advance n_steps; returns {"axon"/"soma"/"dend": [rows, n]} for the selected quantities."""
        names = [nm for bit, nm in ((TRACE_AXON, "axon"), (TRACE_SOMA, "soma"), (TRACE_DEND, "dend"))
                 if what & bit]
        if trace_every <= 0:
            _check(self._L.infoli_sim_run_into(self._h, int(n_steps), 0, 0, None, 0, None))
            return {}
        s0 = self.step
        rows = sum(1 for t in range(s0, s0 + n_steps) if t % trace_every == 0)
        out = np.zeros((max(rows, 1), len(names), self.n), dtype=np.float32)
        got = C.c_int(0)
        _check(self._L.infoli_sim_run_into(self._h, int(n_steps), int(trace_every), int(what), _p(out),
                                           out.size, C.byref(got)))
        assert got.value == rows
        return {nm: out[:rows, i, :].copy() for i, nm in enumerate(names)}

    def launch(self, n_steps):
        """Enqueue n_steps (no trace) and return at once."""
        _check(self._L.infoli_sim_launch(self._h, int(n_steps)))

    def query(self) -> bool:
        return bool(_check(self._L.infoli_sim_query(self._h)))

    def sync(self):
        _check(self._L.infoli_sim_sync(self._h))

    def device_bytes(self) -> int:
        v = C.c_int64()
        _check(self._L.infoli_sim_memory(self._h, C.byref(v)))
        return v.value

    def run_with_callback(self, n_steps, trace_every, what, fn):
        """fn(step, what_bit, values[n]) per recorded quantity, in step order."""
        def _cb(user, step, w, values, n):
            fn(step, w, np.ctypeslib.as_array(values, shape=(n,)))
        cb = TRACE_CB(_cb)
        _check(self._L.infoli_sim_run(self._h, int(n_steps), int(trace_every), int(what), cb, None))

    def get_state(self, out=None) -> np.ndarray:
        """The 19 state arrays [19, n]; written into `out` (float32, C-contiguous,
        e.g. a pinned buffer) when given."""
        if out is None:
            out = np.empty((NSTATE, self.n), dtype=np.float32)
        assert out.dtype == np.float32 and out.flags.c_contiguous and out.size == NSTATE * self.n
        _check(self._L.infoli_sim_get_state(self._h, _p(out)))
        return out

    def set_state(self, st):
        st = np.ascontiguousarray(st, dtype=np.float32).reshape(NSTATE, self.n)
        _check(self._L.infoli_sim_set_state(self._h, _p(st)))

    def last_run_stats(self):
        ms = C.c_float(0)
        nl = C.c_int(0)
        _check(self._L.infoli_sim_last_run_stats(self._h, C.byref(ms), C.byref(nl)))
        return ms.value, nl.value

    def set_profiling(self, on=True):
        _check(self._L.infoli_sim_set_profiling(self._h, int(bool(on))))

    def get_profile(self):
        """{"mean"/"max": {"wait","couple","update","barrier","units"}: ns per step}."""
        mean = np.zeros(5)
        mx = np.zeros(5)
        _check(self._L.infoli_sim_get_profile(self._h, _p(mean), _p(mx)))
        keys = ("wait", "couple", "update", "barrier", "units")
        return {"mean": dict(zip(keys, mean.tolist())), "max": dict(zip(keys, mx.tolist()))}

    def plan_info(self):
        g, t, ti, ch = C.c_int(), C.c_int(), C.c_int(), C.c_int()
        sm = C.c_int64()
        _check(self._L.infoli_sim_plan_info(self._h, C.byref(g), C.byref(t), C.byref(ti), C.byref(ch),
                                            C.byref(sm)))
        return {"grid": g.value, "threads": t.value, "tiles": ti.value, "chunks": ch.value,
                "smem_bytes": sm.value}


def gen_bitmask(n: int, p: float, seed: int) -> np.ndarray:
    """Receiver bitmask [n, ceil(n/32)] uint32 (include/infoli_gpu.h: infoli_gen_bitmask)."""
    bits = np.zeros((n, (n + 31) // 32), dtype=np.uint32)
    _check(load().infoli_gen_bitmask(int(n), float(p), int(seed) & (2**64 - 1), _p(bits)))
    return bits


def gen_bitmask_csr(n: int, p: float, seed: int):
    """CSR of gen_bitmask(n, p, seed) (include/infoli_gpu.h: infoli_gen_bitmask_csr)."""
    L = load()
    return _csr_call(L.infoli_gen_bitmask_csr, n, n, float(p), int(seed) & (2**64 - 1),
                     cap_hint=n * (n - 1) * min(1.0, float(p) * 1.05 + 0.002) + 1024)


def batch_tune_sample(n_cells, max_sample=0, target_cells=2 * 152 * 1024) -> np.ndarray:
    """Indices of the networks the batch autotuner times (host only; include/
    infoli_gpu.h: infoli_batch_tune_sample)."""
    sizes = np.ascontiguousarray(n_cells, dtype=np.int32)
    out = np.zeros(sizes.size, dtype=np.int32)
    m = load().infoli_batch_tune_sample(int(sizes.size), _p(sizes), int(max_sample), int(target_cells), _p(out))
    _check(min(m, 0))
    return out[:m].copy()


class Batch:
    """Many independent networks in one launch (infoli_batch_* handle).

    nets: list of (n_cells, bits[n, ceil(n/32)] uint32, g) per network.
    init_state: [NSTATE, total] over the networks' cells end to end, or None
    (then init_values is broadcast)."""

    def __init__(self, params, nets, init_state=None, init_values=None, kahan=False, device=0, shape=0,
                 tune_steps=200, tune_max_sample=0, residency=RES_FIT):
        """shape: cells per CTA, 1024 or 512; 0 = the library's default;
        "auto" = infoli_batch_autotune's pick of the shape and the residency
        together (every candidate timed on a sample of the networks,
        tune_steps steps each), kept in self.tune.  residency: RES_FIT,
        RES_OCC or RES_NONE (ignored with shape="auto")."""
        L = load()
        self._L = L
        params = np.ascontiguousarray(params, dtype=np.float32)
        assert params.size >= NPARAM
        self.params = params[:NPARAM].copy()
        self.sizes = np.array([int(n) for n, _, _ in nets], dtype=np.int32)
        self.offsets = np.concatenate([[0], np.cumsum(self.sizes, dtype=np.int64)])
        self.total = int(self.offsets[-1])
        self._bits = np.concatenate([np.ascontiguousarray(b, dtype=np.uint32).ravel() for _, b, _ in nets])
        self._g = np.array([float(g) for _, _, g in nets], dtype=np.float32)
        d = BatchDesc()
        d.n_nets = len(nets)
        d.n_cells = _p(self.sizes)
        d.params = _p(self.params)
        if init_state is not None:
            self._st = np.ascontiguousarray(init_state, dtype=np.float32).reshape(NSTATE, self.total)
            d.init_state = _p(self._st)
        else:
            self._iv = np.ascontiguousarray(init_values, dtype=np.float32)
            assert self._iv.size == NSTATE
            d.init_values = _p(self._iv)
        d.bits = _p(self._bits)
        d.g = _p(self._g)
        d.flags = F_KAHAN if kahan else 0
        d.device = int(device)
        self.tune = None
        if shape == "auto":
            t = BatchTune()
            _check(L.infoli_batch_autotune(C.byref(d), int(tune_max_sample), int(tune_steps), C.byref(t)))
            self.tune = {"block": t.block, "residency": RES_NAMES[t.residency], "sample_nets": t.sample_nets,
                         "sample_cells": t.sample_cells,
                         "ms_per_step": {f"{t.cand_block[k]}/{RES_NAMES[t.cand_residency[k]]}": t.cand_ms_per_step[k]
                                         for k in range(TUNE_CANDIDATES)}}
            d.block = t.block
            d.residency = t.residency
        else:
            d.block = int(shape)
            d.residency = int(residency)
        self.residency = int(d.residency)
        h = C.c_void_p()
        _check(L.infoli_batch_create(C.byref(d), C.byref(h)))
        self._h = h

    def close(self):
        if getattr(self, "_h", None):
            self._L.infoli_batch_destroy(self._h)
            self._h = None

    __del__ = close

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def set_stimulus_pulse(self, start, end, amp):
        _check(self._L.infoli_batch_set_stimulus_pulse(self._h, int(start), int(end), float(amp)))

    def run(self, n_steps):
        _check(self._L.infoli_batch_run(self._h, int(n_steps)))

    def get_state(self) -> np.ndarray:
        out = np.zeros((NSTATE, self.total), dtype=np.float32)
        _check(self._L.infoli_batch_get_state(self._h, _p(out)))
        return out

    def set_state(self, st):
        st = np.ascontiguousarray(st, dtype=np.float32).reshape(NSTATE, self.total)
        _check(self._L.infoli_batch_set_state(self._h, _p(st)))

    def net_state(self, st: np.ndarray, i: int) -> np.ndarray:
        return st[:, self.offsets[i]:self.offsets[i + 1]]

    def info(self):
        ctas, cl, blk = C.c_int(), C.c_int(), C.c_int()
        cells = C.c_int64()
        ms = C.c_float()
        _check(self._L.infoli_batch_info(self._h, C.byref(ctas), C.byref(cl), C.byref(blk), C.byref(cells),
                                         C.byref(ms)))
        return {"ctas": ctas.value, "cluster": cl.value, "block": blk.value, "cells": cells.value,
                "last_ms": ms.value}

    def cta_info(self):
        """{"max_active_clusters", "net"[ctas], "start_ns"[ctas], "end_ns"[ctas]} of the last run."""
        k = self.info()["ctas"]
        mac = C.c_int()
        net = np.zeros(k, np.int32)
        t0 = np.zeros(k, np.int64)
        t1 = np.zeros(k, np.int64)
        _check(self._L.infoli_batch_cta_info(self._h, C.byref(mac), _p(net), _p(t0), _p(t1)))
        return {"max_active_clusters": mac.value, "net": net, "start_ns": t0, "end_ns": t1}


class Server:
    """Request loop over many simulations on one GPU (infoli_server_* handle)."""

    def __init__(self, params, device=0, hbm_budget=0, max_active=0, work_per_cta=0, backfill_ms=0,
                 prep_threads=0, kahan=False, age_ms=0, lane_sms=0, lane_chunk_steps=0, lane_edges_per_cta=0):
        """age_ms: prepared requests launch shortest estimated work first, except
        those submitted more than age_ms ago (oldest first); 0 = 10 s, < 0 =
        arrival order.  lane_sms: SMs persistent requests leave to the lane of
        small requests (0 = none, < 0 = no lane); lane_chunk_steps: steps per
        lane launch (0 = 2000); lane_edges_per_cta: lane eligibility, edges
        per CTA of a request's cluster (0 = 24576, < 0 = any)."""
        L = load()
        self._L = L
        self.params = np.ascontiguousarray(params, dtype=np.float32)[:NPARAM].copy()
        d = ServerDesc()
        d.params = _p(self.params)
        d.device = int(device)
        d.hbm_budget = int(hbm_budget)
        d.max_active = int(max_active)
        d.work_per_cta = int(work_per_cta)
        d.backfill_ms = int(backfill_ms)
        d.prep_threads = int(prep_threads)
        d.flags = F_KAHAN if kahan else 0
        d.age_ms = int(age_ms)
        d.lane_sms = int(lane_sms)
        d.lane_chunk_steps = int(lane_chunk_steps)
        d.lane_edges_per_cta = int(lane_edges_per_cta)
        h = C.c_void_p()
        _check(L.infoli_server_create(C.byref(d), C.byref(h)))
        self._h = h
        self._n = {}

    def close(self):
        if getattr(self, "_h", None):
            self._L.infoli_server_destroy(self._h)
            self._h = None

    __del__ = close

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def submit(self, n, row_ptr, col, n_steps, g=None, g_uniform=0.04, init_state=None, init_values=None,
               pulse=(20000, 20499, 6.0)) -> int:
        rp = np.ascontiguousarray(row_ptr, dtype=np.int64)
        cl = np.ascontiguousarray(col, dtype=np.int32)
        gg = None if g is None else np.ascontiguousarray(g, dtype=np.float32)
        q = RequestDesc()
        q.n_cells = int(n)
        q.row_ptr = _p(rp)
        q.col = _p(cl) if cl.size else None
        q.g = _p(gg)
        q.g_uniform = float(g_uniform)
        if init_state is not None:
            st = np.ascontiguousarray(init_state, dtype=np.float32).reshape(NSTATE, int(n))
            q.init_state = _p(st)
        else:
            iv = np.ascontiguousarray(init_values, dtype=np.float32)
            q.init_values = _p(iv)
        q.n_steps = int(n_steps)
        q.pulse_start, q.pulse_end, q.pulse_amp = int(pulse[0]), int(pulse[1]), float(pulse[2])
        rid = C.c_int64()
        _check(self._L.infoli_server_submit(self._h, C.byref(q), C.byref(rid)))
        self._n[rid.value] = int(n)
        return rid.value

    def poll(self, rid) -> int:
        return _check(self._L.infoli_server_poll(self._h, int(rid)))

    def wait(self, rid, want_state=True):
        """Returns (state [19, n] or None, info dict)."""
        n = self._n.pop(int(rid))
        out = np.zeros((NSTATE, n), dtype=np.float32) if want_state else None
        info = RequestInfo()
        _check(self._L.infoli_server_wait(self._h, int(rid), _p(out), C.byref(info)))
        return out, {k: getattr(info, k) for k, _ in RequestInfo._fields_}

    def status(self):
        q, a = C.c_int(), C.c_int()
        c, m = C.c_int64(), C.c_int64()
        _check(self._L.infoli_server_status(self._h, C.byref(q), C.byref(a), C.byref(c), C.byref(m)))
        return {"queued": q.value, "active": a.value, "completed": c.value, "hbm_in_use": m.value}
