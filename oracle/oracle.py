"""ctypes front-end of the CPU oracle (oracle/infoli_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
CPU-baseline leg of bench.py, as the checker.  The product never imports it.

State layout used everywhere: a (19, n) array in bin/default.conf order
(lines 24-42 of the reference's default.conf: V_dend, Calcium_r, Potassium_s,
Hcurrent_q, Ca2Plus, I_CaH, g_CaL, V_soma, Sodium_m, Sodium_h, Potassium_n,
Potassium_p, Potassium_x_s, Calcium_k, Calcium_l, V_axon, Sodium_m_a,
Sodium_h_a, Potassium_x_a).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "liboracle.so")
_lib = None

STATE_NAMES = [
    "V_dend", "Calcium_r", "Potassium_s", "Hcurrent_q", "Ca2Plus", "I_CaH", "g_CaL",
    "V_soma", "Sodium_m", "Sodium_h", "Potassium_n", "Potassium_p", "Potassium_x_s",
    "Calcium_k", "Calcium_l", "V_axon", "Sodium_m_a", "Sodium_h_a", "Potassium_x_a",
]
S = {name: i for i, name in enumerate(STATE_NAMES)}


def build() -> str:
    """Compile liboracle.so (make -C oracle)."""
    subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return _LIB_PATH


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(_LIB_PATH):
            build()
        L = C.CDLL(_LIB_PATH)
        P = C.c_void_p
        L.orc_read_parameters.argtypes = [C.c_char_p, P]
        L.orc_read_parameters.restype = C.c_int
        L.orc_gen_uniform.argtypes = [C.c_int, C.c_float, C.c_uint, P, P, C.c_longlong]
        L.orc_gen_uniform.restype = C.c_longlong
        run_args = [C.c_int, P, P, P, P, P, None, C.c_int, P, P, P, P,
                    C.c_int, C.c_int, C.c_int, P, P, P, C.c_int]
        a32 = list(run_args)
        a32[6] = C.c_float
        a64 = list(run_args)
        a64[6] = C.c_double
        L.orc_run_f32.argtypes = a32
        L.orc_run_f32.restype = C.c_int
        L.orc_run_f64.argtypes = a64
        L.orc_run_f64.restype = C.c_int
        L.orc_max_threads.restype = C.c_int
        L.orc_random_init.argtypes = [C.c_int, P, P, C.c_uint, P]
        L.orc_random_init.restype = None
        L.orc_random_init_f64.argtypes = [C.c_int, P, P, C.c_uint, P]
        L.orc_random_init_f64.restype = None
        _lib = L
    return _lib


def _ptr(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def read_parameters(path: str) -> np.ndarray:
    """read_parameters (src/utils/utils.c:137-160): 42 floats, positional."""
    v = np.zeros(42, dtype=np.float32)
    rc = lib().orc_read_parameters(path.encode(), _ptr(v))
    if rc == -1000:
        raise FileNotFoundError(path)
    if rc != 0:
        raise ValueError(f"improper parameter at line {-rc} of {path}")
    return v


def gen_uniform(n: int, p: float, seed: int):
    """The reference's built-in Bernoulli(p) generator (src/openmp/infoli.c:337-375)."""
    row_ptr = np.zeros(n + 1, dtype=np.int64)
    cap = max(1, int(n * (n - 1) * min(1.0, float(p) * 1.2 + 0.01)) + 64)
    while True:
        col = np.zeros(cap, dtype=np.int32)
        e = lib().orc_gen_uniform(n, C.c_float(p), seed, _ptr(row_ptr), _ptr(col), cap)
        if e >= 0:
            return row_ptr, col[:e].copy()
        cap = int(row_ptr[-1])


def default_state(n: int, init42: np.ndarray, dtype=np.float32) -> np.ndarray:
    """Per-cell initial state from the 19 trailing conf values (src/openmp/infoli.c:267-292)."""
    st = np.empty((19, n), dtype=dtype)
    st[:] = np.asarray(init42[23:42], dtype=dtype)[:, None]
    return st


def _stim_args(stim, n):
    """stim = ('pulse', start, end, amp), ('cell', amp[n], onset[n], dur) or
    ('table', rows[k, n], first_step)."""
    if stim is None:
        stim = ("pulse", 20000, 20499, 6.0)
    if stim[0] == "pulse":
        si = np.array([stim[1], stim[2]], dtype=np.int32)
        sf = np.array([stim[3]], dtype=np.float32)
        return 0, si, sf, None, None
    if stim[0] == "table":
        tab = np.ascontiguousarray(stim[1], dtype=np.float32)
        assert tab.ndim == 2 and tab.shape[1] == n
        si = np.array([stim[2], tab.shape[0]], dtype=np.int32)
        return 2, si, np.zeros(1, dtype=np.float32), tab, None
    amp = np.ascontiguousarray(stim[1], dtype=np.float32)
    onset = np.ascontiguousarray(stim[2], dtype=np.int32)
    assert amp.shape == (n,) and onset.shape == (n,)
    si = np.array([stim[3], 0], dtype=np.int32)
    sf = np.zeros(1, dtype=np.float32)
    return 1, si, sf, amp, onset


def run(n, params, state, row_ptr, col, g=None, g_uniform=0.04, stim=None,
        step0=0, nsteps=1, trace_every=1, traces=("axon", "soma", "dend"),
        nthreads=1, fp64=False):
    """Advance `state` (19, n) in place by nsteps; return {name: [rows, n]} traces."""
    dt = np.float64 if fp64 else np.float32
    assert state.dtype == dt and state.shape == (19, n) and state.flags.c_contiguous
    params = np.ascontiguousarray(params, dtype=dt)
    assert params.shape[0] >= 23
    row_ptr = np.ascontiguousarray(row_ptr, dtype=np.int64)
    col = np.ascontiguousarray(col, dtype=np.int32)
    if g is not None:
        g = np.ascontiguousarray(g, dtype=np.float32)
        assert g.shape == col.shape
    kind, si, sf, amp, onset = _stim_args(stim, n)
    if trace_every > 0:
        rows = sum(1 for t in range(nsteps) if (step0 + t) % trace_every == 0)
    else:
        rows = 0
    out = {k: (np.zeros((max(rows, 1), n), dtype=dt) if k in traces else None)
           for k in ("axon", "soma", "dend")}
    fn = lib().orc_run_f64 if fp64 else lib().orc_run_f32
    got = fn(n, _ptr(params), _ptr(state), _ptr(row_ptr), _ptr(col), _ptr(g),
             float(g_uniform), kind, _ptr(si), _ptr(sf), _ptr(amp), _ptr(onset),
             step0, nsteps, trace_every, _ptr(out["axon"]), _ptr(out["soma"]),
             _ptr(out["dend"]), int(nthreads))
    assert got == rows
    return {k: v[:rows] for k, v in out.items() if v is not None}


def random_init(n, params, state, seed):
    """Randomised initial state (orc_random_init, or orc_random_init_f64 for a
    float64 state); state (19, n) is updated in place; returns the step count
    drawn for every cell (the state is the one after that count minus one)."""
    assert state.dtype in (np.float32, np.float64) and state.shape == (19, n) and state.flags.c_contiguous
    params = np.ascontiguousarray(params, dtype=state.dtype)
    steps = np.zeros(n, dtype=np.int32)
    fn = lib().orc_random_init_f64 if state.dtype == np.float64 else lib().orc_random_init
    fn(n, _ptr(params), _ptr(state), int(seed) & 0xFFFFFFFF, _ptr(steps))
    return steps


def max_threads() -> int:
    return lib().orc_max_threads()
