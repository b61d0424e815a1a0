"""Shared helpers for the test suite (fixtures, topologies, comparisons)."""
from __future__ import annotations

import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = os.path.join(HERE, "golden")
ROOT = os.path.dirname(HERE)
CONF = os.path.join(ROOT, "infoli_gb300", "host", "default.conf")

# Tolerances of the path (V in mV): max |dV_soma| over the first 2000 steps,
# and soma/axon spike steps equal within one step.
TOL_VSOMA_MV = 1e-3
TOL_SPIKE_STEPS = 1


def golden(name):
    return np.load(os.path.join(GOLDEN, name))


def kat_topology():
    """The reference regression fixture (src/regression_test/cellConnections.txt,
    gcal_file.txt): dense conductance matrix, row = sender, column = receiver
    (stable_version.c reads neighId[i] = line index).  Returns CSR + g + g_CaL."""
    z = golden("kat_stable_version.npz")
    G = z["cond_sender_by_receiver"]
    n = G.shape[0]
    rp, col, g = [0], [], []
    for r in range(n):
        for s in range(n):
            if G[s, r] >= 1e-7:
                col.append(s)
                g.append(G[s, r])
        rp.append(len(col))
    return (n, np.array(rp, np.int64), np.array(col, np.int32), np.array(g, np.float32),
            z["gcal"].astype(np.float32))


def hetero_state(conf, n, seed, dv=1.0):
    """Default state with V_dend + U(-dv, dv) and g_CaL ~ U(0.6, 0.8)."""
    from oracle import oracle as O

    st = O.default_state(n, conf)
    rng = np.random.default_rng(seed)
    st[O.S["V_dend"]] += rng.uniform(-dv, dv, n).astype(np.float32)
    st[O.S["g_CaL"]] = rng.uniform(0.6, 0.8, n).astype(np.float32)
    return st


def spike_steps(v: np.ndarray, step0: int = 0, thr: float = 0.0):
    """Per column, the steps at which v crosses thr upwards (row r = step0 + r)."""
    return [step0 + np.nonzero((v[:-1, c] < thr) & (v[1:, c] >= thr))[0] + 1 for c in range(v.shape[1])]


def spikes_match(a, b, tol=TOL_SPIKE_STEPS):
    """Same number of spikes per cell and each within tol steps."""
    for x, y in zip(a, b):
        if len(x) != len(y):
            return False
        if len(x) and np.max(np.abs(np.asarray(x) - np.asarray(y))) > tol:
            return False
    return True
