"""Seeded synthetic workloads with the shapes of the benchmark configurations.

There is no dataset behind any of them: topologies come from the library's
own generators (include/infoli_gpu.h) and initial states from numpy draws, so
every run with the same seed sees the same inputs.
"""
from __future__ import annotations

import numpy as np

from . import capi


def popcount(bits: np.ndarray) -> int:
    """Set bits of a uint32 array."""
    if hasattr(np, "bitwise_count"):
        return int(np.bitwise_count(bits).sum(dtype=np.int64))
    return int(np.unpackbits(np.ascontiguousarray(bits).view(np.uint8)).sum(dtype=np.int64))


def default_state(conf, n):
    """[19, n] float32 with the default.conf initial values (lines 24-42)."""
    st = np.empty((capi.NSTATE, n), dtype=np.float32)
    st[:] = np.asarray(conf[23:42], dtype=np.float32)[:, None]
    return st


def perturbed_state(conf, n, rng, dv=1.0):
    """Default state with V_dend = -60 + U(-dv, dv) mV and g_CaL ~ U(0.6, 0.8)."""
    st = default_state(conf, n)
    st[capi.S["V_dend"]] += rng.uniform(-dv, dv, n).astype(np.float32)
    st[capi.S["g_CaL"]] = rng.uniform(0.6, 0.8, n).astype(np.float32)
    return st


def batched(conf, n_nets=512, lo=256, hi=8192, dens=(0.05, 0.5), g=(0.02, 0.06), seed=1):
    """Independent networks: sizes log-uniform in [lo, hi], density U(dens),
    one conductance U(g) per network, bitmask topology from seed b for network
    b (infoli_gen_bitmask).  Returns (nets, init_state, meta) with nets a list
    of (n, bits, g) and init_state [19, sum n]."""
    rng = np.random.default_rng(seed)
    sizes = np.exp(rng.uniform(np.log(lo), np.log(hi), n_nets)).astype(np.int64)
    sizes = np.clip(sizes, lo, hi)
    p = rng.uniform(dens[0], dens[1], n_nets)
    gs = rng.uniform(g[0], g[1], n_nets).astype(np.float32)
    nets = [(int(n), capi.gen_bitmask(int(n), float(d), b), float(gg)) for b, (n, d, gg) in enumerate(zip(sizes, p, gs))]
    st = perturbed_state(conf, int(sizes.sum()), rng)
    edges = np.array([popcount(b) for _, b, _ in nets], dtype=np.int64)
    meta = {"sizes": sizes, "density": p, "g": gs, "edges": edges}
    return nets, st, meta
