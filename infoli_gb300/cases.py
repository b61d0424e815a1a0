"""Small named runs of the library's paths, for profilers and quick checks.

    python -m infoli_gb300.cases <case> [--steps K]

Cases (seeded synthetic inputs):
  grid10k  10,000 cells on a 100x100 grid, Gaussian distance (sigma 10, radius
           18), stamped plan (the bench's headline workload)
  uniform1k  1,000 cells, the reference generator at p = 0.1
  sparse100k 100,000 cells, 100 senders each, per-edge g U(0.02, 0.06):
           gather plan
  dense10k 10,000 cells, bitmask generator at p = 0.2 (2,000 senders per
           cell): stamped plan dominated by the coupling
  batch64  the first 64 networks of the batched workload (sizes log-uniform
           256-8,192, density U(0.05, 0.5)), one graph launch
Each case builds its inputs, runs K steps once and prints the device time.
"""
from __future__ import annotations

import argparse
import os

import numpy as np

from . import capi, workloads

_CONF = os.path.join(os.path.dirname(os.path.abspath(__file__)), "host", "default.conf")


def _sim_case(name, steps):
    conf = capi.read_parameters(_CONF)
    rng = np.random.default_rng(1)
    g = None
    if name == "grid10k":
        rp, col = capi.gen_grid_gaussian(100, 100, 10.0, 18.0, 1)
        n = 10000
    elif name == "uniform1k":
        n = 1000
        rp, col = capi.gen_uniform(n, 0.1, 1)
    elif name == "dense10k":
        n = 10000
        rp, col = capi.gen_bitmask_csr(n, 0.2, 5)
    elif name == "sparse100k":
        n = 100000
        rp, col, g = capi.gen_fixed_degree(n, 100, 3, (0.02, 0.06))
    else:
        raise SystemExit(f"unknown case {name}")
    st = workloads.perturbed_state(conf, n, rng)
    with capi.Simulation(n, conf, rp, col, g=g, init_state=st) as sim:
        sim.run(steps)
        ms, launches = sim.last_run_stats()
        print(f"{name}: {n} cells, {len(col)} edges, plan {sim.plan_info()}, {steps} steps in {ms:.3f} ms "
              f"({launches} launches)")


def _batch_case(steps):
    conf = capi.read_parameters(_CONF)
    nets, st, meta = workloads.batched(conf, n_nets=64, seed=1)
    with capi.Batch(conf, nets, init_state=st, kahan=True) as bt:
        bt.run(steps)
        print(f"batch64: {int(meta['sizes'].sum())} cells, {int(meta['edges'].sum())} edges, {bt.info()}")


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("case", choices=["grid10k", "uniform1k", "dense10k", "sparse100k", "batch64"])
    ap.add_argument("--steps", type=int, default=100)
    a = ap.parse_args()
    if a.case == "batch64":
        _batch_case(a.steps)
    else:
        _sim_case(a.case, a.steps)


if __name__ == "__main__":
    main()
