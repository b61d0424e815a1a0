"""Benchmark: cell-steps/s of the InfOli network update on one GB300 (or N
replicas), with the batched and served forms measured in the same run.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]
                  [--workload all|grid10k|batched|serving] [--case NAME]

Default line (--workload all), one JSON line with three parts:

* headline (top-level keys): 10,000 cells on a 100x100 grid, Gaussian-distance
  connectivity (sigma = 10 cells, candidates within radius 18 = ~1,000 cells
  per receiver, mean degree ~439), uniform g = 0.04, initial V_dend = -60 +
  U(-1,1) mV and g_CaL ~ U(0.6, 0.8) from seed 1, the reference's 6 uA pulse
  schedule.  One bench step = one infoli_sim_run call advancing 1,000
  explicit-Euler timesteps (50 ms simulated) with the V_axon trace streamed to
  the host every 100 timesteps, as the reference prints it.  `value`: cells x
  timesteps / device time (CUDA events on the simulation's stream, state and
  topology resident in HBM, L2 flushed between steps).  `e2e`: the same work
  through the C ABI from pinned host buffers (set_state H2D, run with the
  trace D2H, get_state D2H), wall clock.  The line carries the coupling sum's
  precision mode, the FP64-oracle error, the roofline of the step kernel and
  the CPU baseline: the reference's own OpenMP build (untouched sources,
  compiled on this host by oracle/build_ref.sh) timed by its own clock at the
  same cell count and mean degree, all host cores.
* "batched": 512 independent networks (sizes log-uniform 256-8,192, density
  U(0.05, 0.5), g U(0.02, 0.06) per network), the full 10,000 timesteps of
  every network as 10 graph launches of 1,000 timesteps, launch shape picked by
  the library's autotuner; against sequential plain runs of every network
  (infoli_sim, one after another, 1,000 timesteps each) on the same GPU.
* "serving": a fixed trace of 24 requests arriving as a Poisson stream (mean
  50/s), sizes log-uniform 500-50,000 cells, durations U(100, 2,000) ms,
  density U(0.01, 0.30), through the library's request loop; against the same
  requests run alone one after another (first in, first out) on the same GPU.

--impl reference times the reference's own OpenMP build (or, where it could
not be built, the oracle's restatement of its loop) on the host cores.
--case NAME runs one named small case once and prints its device time (the
commands in profiles/ use these under ncu).
"""
from __future__ import annotations

import argparse
import json
import os
import re
import shutil
import statistics
import subprocess
import sys
import tempfile
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

ROWS, COLS, SIGMA, RADIUS, SEED = 100, 100, 10.0, 18.0, 1
STEPS_PER_ITER = 1000
TRACE_EVERY = 100
CPU_SAMPLE_STEPS = 2000  # timesteps of the oracle port, reported beside the reference build
N_SM_FALLBACK = 152
SFU_EX2_PER_CLK_SM = 16  # MUFU.EX2 results per clock per SM

CONF_PATH = os.path.join(ROOT, "infoli_gb300", "host", "default.conf")
REF_DIR = os.path.join(ROOT, "oracle", "_ref")


def ncu_traffic(kahan=True):
    """DRAM bytes (read + write) of one step-kernel launch of this workload, from
    the committed ncu summary of the kernel the headline runs."""
    name = "step_kernel_grid10k_kahan.md" if kahan else "step_kernel_grid10k_stamped.md"
    try:
        with open(os.path.join(ROOT, "profiles", name)) as f:
            m = re.search(r"traffic \(read \+ write\) per launch \| ([\d,]+) B", f.read())
        return int(m.group(1).replace(",", "")) if m else None
    except OSError:
        return None


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def workload():
    import numpy as np

    import infoli_gb300 as ig

    conf = ig.read_parameters(CONF_PATH)
    rp, col = ig.gen_grid_gaussian(ROWS, COLS, SIGMA, RADIUS, SEED)
    n = ROWS * COLS
    st = np.empty((19, n), dtype=np.float32)
    st[:] = conf[23:42][:, None]
    rng = np.random.default_rng(SEED)
    st[0] += rng.uniform(-1, 1, n).astype(np.float32)
    st[6] = rng.uniform(0.6, 0.8, n).astype(np.float32)
    return conf, n, rp, col, st


GRID_EDGES = 4391308  # edges of workload()'s grid (the C2 network), checked by the GPU arm


def workload_name():
    """The network both arms run (the same string in both JSON lines)."""
    return f"grid {ROWS}x{COLS} gaussian sigma={SIGMA} radius={RADIUS} g=0.04 seed=1"


class ClockSampler:
    """nvidia-smi clocks/throttle reasons sampled during the timed region."""

    def __init__(self, index):
        self.index = index
        self.rows = []
        self.proc = None

    def __enter__(self):
        q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={q}",
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
            # nvidia-smi's own start-up touches the GPU: let it finish before
            # the timed region (first sample, or 3 s at most)
            t0 = time.time()
            while not self.rows and time.time() - t0 < 3.0:
                time.sleep(0.02)
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) == 7:
                self.rows.append(parts)

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        sm = [float(r[0]) for r in self.rows if r[0].replace(".", "").isdigit()]
        mx = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in self.rows for i in range(4) if r[3 + i].lower().startswith("active")})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.rows)}


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("gloo")
    return world, rank, local


def dist_max(x, world):
    if world == 1:
        return x
    import torch
    import torch.distributed as dist

    t = torch.tensor([float(x)], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def dist_barrier(world):
    if world > 1:
        import torch.distributed as dist

        dist.barrier()


def host_cpu():
    """(logical cores, CPU model) of this host."""
    model = None
    try:
        with open("/proc/cpuinfo") as f:
            txt = f.read()
        m = re.search(r"model name\s*:\s*(.+)", txt)
        if m:
            model = m.group(1).strip()
    except OSError:
        pass
    if model is None:
        try:
            out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
            m = re.search(r"Model name:\s*(.+)", out)
            model = m.group(1).strip() if m else None
        except Exception:
            model = None
    return os.cpu_count() or 1, model


ACC_STEPS = 2000  # window of the accuracy criterion: max |dV_soma| <= 1e-3 mV over the first 2000 steps
ACC_TOL_MV = 1e-3


def soma_error_vs_fp64(conf, n, rp, col, st, gpu_soma, g_uniform, threads, final_only=False, step0=0):
    """max |V_soma(GPU) - V_soma(FP64 oracle)| in mV over ACC_STEPS steps from the
    initial state `st` (every step, or only the state after the last step),
    the GPU run's first step being step index `step0` (the stimulus schedule
    depends on it)."""
    import numpy as np
    from oracle import oracle as O

    s64 = np.ascontiguousarray(st, dtype=np.float64)
    ref = O.run(n, np.asarray(conf[:23], dtype=np.float64), s64, rp, col, g_uniform=g_uniform, step0=step0,
                nsteps=ACC_STEPS, trace_every=0 if final_only else 1, traces=() if final_only else ("soma",),
                nthreads=threads, fp64=True)
    want = s64[O.S["V_soma"]] if final_only else ref["soma"]
    return float(np.max(np.abs(np.asarray(gpu_soma, dtype=np.float64) - want)))


# ------------------------------------------------------- CPU baselines --
def reference_binary():
    """The reference's OpenMP build compiled on this host (oracle/_ref), or None."""
    exe = os.path.join(REF_DIR, "infoli_omp_perf.x")
    conf = os.path.join(REF_DIR, "default.conf")
    if os.access(exe, os.X_OK) and os.path.exists(conf):
        return exe, conf
    script = os.path.join(ROOT, "oracle", "build_ref.sh")
    try:
        subprocess.run(["bash", script], check=True, capture_output=True, timeout=300)
    except Exception:
        return None
    return (exe, conf) if os.access(exe, os.X_OK) else None


def reference_sim_steps(sim_ms):
    """The reference's step count (int)(simTime / DELTA), FP32 (src/openmp/infoli.c:478)."""
    import numpy as np

    return int(np.float32(sim_ms) / np.float32(0.05))


def run_reference_binary(n, p, sim_ms, threads, g=None):
    """One run of the untouched reference OpenMP build: -n n -p p -t sim_ms
    (with CONDUCTANCE = g in a copy of its default.conf when g is given).
    Returns (cell-steps/s by its own 'Execution Time for Simulation' clock,
    src/openmp/infoli.c:428,702,721; that time in s)."""
    found = reference_binary()
    if found is None:
        return None
    exe, conf = found
    env = dict(os.environ, OMP_NUM_THREADS=str(threads))
    d = tempfile.mkdtemp(prefix="infoli_ref_")
    try:
        if g is not None:
            # the parameter file is read by position: line 2 is CONDUCTANCE
            with open(conf) as f:
                lines = f.read().splitlines()
            lines[1] = f"CONDUCTANCE = {g:.6f}"
            conf = os.path.join(d, "default.conf")
            with open(conf, "w") as f:
                f.write("\n".join(lines) + "\n")
        r = subprocess.run([exe, "-n", str(n), "-p", f"{p:.6f}", "-t", str(sim_ms), "-c", conf, "-o",
                            os.path.join(d, "out.txt")], capture_output=True, text=True, env=env, cwd=d,
                           timeout=900)
    finally:
        shutil.rmtree(d, ignore_errors=True)
    m = re.search(r"Execution Time for Simulation: ([\d.]+) ms", r.stdout)
    if r.returncode != 0 or not m:
        return None
    t = float(m.group(1)) * 1e-3
    return n * reference_sim_steps(sim_ms) / t, t


def reference_median(n, p, sim_ms, threads, runs=3):
    """(median cell-steps/s, every run's time in s) of `runs` reference runs, or None."""
    got = []
    for _ in range(runs):
        r = run_reference_binary(n, p, sim_ms, threads)
        if r is None:
            return None
        got.append(r)
    return statistics.median(x[0] for x in got), [x[1] for x in got]


def cpu_port_rate(conf, n, rp, col, st, steps, threads):
    """Oracle restatement of the reference OpenMP loop on the host cores: cell-steps/s."""
    from oracle import oracle as O

    s = st.copy()
    t0 = time.perf_counter()
    O.run(n, conf[:23], s, rp, col, g_uniform=conf[1], nsteps=steps, trace_every=TRACE_EVERY,
          traces=("axon",), nthreads=threads)
    dt = time.perf_counter() - t0
    return n * steps / dt, dt


def grid_stand_in_p(n=ROWS * COLS, edges=GRID_EDGES):
    """Bernoulli p giving the reference generator the grid's mean degree."""
    return edges / (n * (n - 1.0))


def run_reference(args, world, rank):
    """Reference arm: the reference's own OpenMP build at the headline's cell
    count and mean degree (its CLI generates a uniform random network; it cannot
    express the Gaussian grid), 1,000 timesteps per bench step, timed by its own
    clock; the oracle port of its loop when the build is unavailable."""
    if rank != 0:
        return 0
    n = ROWS * COLS
    p = grid_stand_in_p()
    threads, model = host_cpu()
    sim_ms = STEPS_PER_ITER * 0.05
    kind = "reference"
    if reference_binary() is not None:
        for _ in range(args.warmup):
            run_reference_binary(n, p, sim_ms, threads)
        total = 0.0
        for _ in range(args.steps):
            r = run_reference_binary(n, p, sim_ms, threads)
            if r is None:
                kind = None
                break
            total += r[1]
        steps_per = reference_sim_steps(sim_ms)
        sample = (f"per bench step one run of the untouched reference OpenMP build (src/openmp/infoli.c + "
                  f"src/utils/utils.c, gcc -O3 -fopenmp): -n {n} -p {p:.6f} -t {sim_ms:g} = {steps_per} "
                  f"timesteps, uniform random network with the grid's mean degree, trace every 100 steps, "
                  f"its own execution-time clock")
    else:
        kind = None
    if kind is None:
        from oracle import oracle as O

        O.build()
        import numpy as np

        kind = "port"
        rp, col = O.gen_uniform(n, p, SEED)
        conf = O.read_parameters(CONF_PATH)
        st = O.default_state(n, conf)
        st[0] += np.random.default_rng(SEED).uniform(-1, 1, n).astype(np.float32)
        for _ in range(args.warmup):
            cpu_port_rate(conf, n, rp, col, st, 10, threads)
        total = 0.0
        steps_per = 100
        for _ in range(args.steps):
            total += cpu_port_rate(conf, n, rp, col, st, steps_per, threads)[1]
        sample = (f"reference build unavailable on this host; the oracle's restatement of its loop "
                  f"(oracle/, C + OpenMP), {steps_per} timesteps per bench step, uniform network at p={p:.6f}")
    value = n * steps_per * args.steps / total
    line = {
        "impl": "reference", "metric": "cell-steps/s", "value": value, "unit": "cell-steps/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * total / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": workload_name(), "cells": n, "mean_degree": GRID_EDGES / n,
                   "timesteps_per_step": steps_per, "trace": f"V_axon every {TRACE_EVERY} timesteps",
                   "topology": "uniform random at the same cell count and mean degree (the reference's "
                               "generator, src/openmp/infoli.c:337-375)"},
        "cpu_baseline": {"value": value, "unit": "cell-steps/s", "cores": threads, "cpu": model, "kind": kind,
                         "sample": sample},
        "e2e": {"value": value, "unit": "cell-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))
    return 0


def flush_l2():
    import torch

    if not hasattr(flush_l2, "buf"):
        flush_l2.buf = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    flush_l2.buf.zero_()
    torch.cuda.synchronize()


def sm_count(local):
    try:
        import torch

        return torch.cuda.get_device_properties(local).multi_processor_count
    except Exception:
        return N_SM_FALLBACK


# ------------------------------------------------------------- headline --
def time_grid(ig, sim, steps, warmup, local, on_row):
    """Device-timed bench steps of one Simulation: (per-step ms, launches, clocks, wall)."""
    import torch

    for _ in range(warmup):
        sim.run_with_callback(STEPS_PER_ITER, TRACE_EVERY, ig.TRACE_AXON, on_row)
    dev_ms, launches = [], 0
    torch.cuda.synchronize()
    t_wall0 = time.perf_counter()
    with ClockSampler(local) as clk:
        for _ in range(steps):
            flush_l2()
            sim.run_with_callback(STEPS_PER_ITER, TRACE_EVERY, ig.TRACE_AXON, on_row)
            ms, nl = sim.last_run_stats()
            dev_ms.append(ms)
            launches += nl
    torch.cuda.synchronize()
    return dev_ms, launches, clk.summary(), time.perf_counter() - t_wall0


def run_gpu(args, world, rank, local):
    import numpy as np
    import torch

    import infoli_gb300 as ig
    from infoli_gb300 import build

    torch.cuda.set_device(local)
    build.build()
    conf, n, rp, col, st = workload()
    assert len(col) == GRID_EDGES, len(col)
    threads, model = host_cpu()
    kahan = not args.no_kahan
    sim = ig.Simulation(n, conf, rp, col, init_state=st, device=local, kahan=kahan)
    plan = sim.plan_info()

    def on_row(step, what, v):
        pass

    # ---- device-resident throughput (CUDA events on the simulation stream)
    dist_barrier(world)
    dev_ms, launches, clocks, wall = time_grid(ig, sim, args.steps, args.warmup, local, on_row)
    dist_barrier(world)
    total_dev_ms = dist_max(sum(dev_ms), world)

    # ---- e2e through the C ABI from host buffers
    host_state = torch.from_numpy(st).pin_memory().numpy()
    out_state = torch.empty(st.shape, dtype=torch.float32).pin_memory().numpy()
    dist_barrier(world)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        sim.set_state(host_state)
        sim.run_with_callback(STEPS_PER_ITER, TRACE_EVERY, ig.TRACE_AXON, on_row)
        sim.get_state(out=out_state)
    e2e_s = dist_max(time.perf_counter() - t0, world)
    rows_per_iter = STEPS_PER_ITER // TRACE_EVERY
    h2d = 19 * 4 * n
    d2h = 19 * 4 * n + rows_per_iter * 4 * n

    # ---- phase profile of the kernel (separate pass, not part of the timing)
    sim.set_profiling(True)
    sim.run(STEPS_PER_ITER)
    prof = sim.get_profile()
    sim.set_profiling(False)
    # ---- accuracy: the same initial state, ACC_STEPS steps, V_soma every step
    # (from the simulation's current step index; the oracle starts there too)
    sim.set_state(st)
    acc_step0 = sim.step
    gpu_soma = sim.run(ACC_STEPS, 1, ig.TRACE_SOMA)["soma"]
    sim.close()

    # ---- the other summation mode, timed the same way (its cost and error)
    other = None
    if world == 1:
        with ig.Simulation(n, conf, rp, col, init_state=st, device=local, kahan=not kahan) as s2:
            o_ms, o_l, o_clk, _ = time_grid(ig, s2, min(args.steps, 10), min(args.warmup, 3), local, on_row)
            s2.set_state(st)
            o_step0 = s2.step
            o_soma = s2.run(ACC_STEPS, 1, ig.TRACE_SOMA)["soma"]
        other = (o_ms, o_clk, o_soma, o_step0)

    cell_steps = n * STEPS_PER_ITER * args.steps * world
    value = cell_steps / (total_dev_ms * 1e-3)
    e2e_value = cell_steps / e2e_s

    # roofline of the dominant kernel (the persistent step kernel): algorithmic
    # bytes per cell-step = 132 B of state + ceil(N/8) B of uniform-g adjacency bits
    alg_bytes_per_launch = (132 + (n + 7) // 8) * n * STEPS_PER_ITER
    launch_ms = sum(dev_ms) / max(1, launches)
    achieved = alg_bytes_per_launch / (launch_ms * 1e-3) / 1e9
    peak, peak_kind = peaks()
    # the bound that applies: the SFU exp2 rate (one exp per edge + 22 per cell)
    nsm = sm_count(local)
    mhz = clocks.get("sm_mhz") or 2070.0
    exps = (len(col) + 22 * n) * STEPS_PER_ITER
    sfu_ach = exps / (launch_ms * 1e-3)
    sfu_peak = SFU_EX2_PER_CLK_SM * nsm * mhz * 1e6

    if rank != 0:
        return None
    cpu = None
    ref = reference_median(n, grid_stand_in_p(), STEPS_PER_ITER * 0.05, threads)
    port_rate, port_dt = cpu_port_rate(conf, n, rp, col, st, CPU_SAMPLE_STEPS, threads)
    if ref is not None:
        cpu = {"value": ref[0], "unit": "cell-steps/s", "cores": threads, "cpu": model, "kind": "reference",
               "sample": f"the median of three runs of the untouched reference OpenMP build (gcc -O3 -fopenmp, "
                         f"all host threads) at the same cell count and mean degree (-n {n} -p "
                         f"{grid_stand_in_p():.6f} -t 50 = 1,000 timesteps, uniform random network), its own "
                         f"execution-time clock: {', '.join(f'{x:.2f}' for x in ref[1])} s",
               "port": {"value": port_rate, "sample": f"oracle restatement on the grid itself, "
                                                      f"{CPU_SAMPLE_STEPS} timesteps ({port_dt:.1f} s)"}}
    else:
        cpu = {"value": port_rate, "unit": "cell-steps/s", "cores": threads, "cpu": model, "kind": "port",
               "sample": f"{CPU_SAMPLE_STEPS} timesteps of the same workload ({port_dt:.1f} s); the reference "
                         f"build could not be made on this host"}
    acc = soma_error_vs_fp64(conf, n, rp, col, st, gpu_soma, conf[1], threads, step0=acc_step0)
    mode = ("kahan: each lane's two FP32 accumulators (paired f32x2) Kahan-add the lane-chunk's terms in "
            "two-term block sums, the lanes' partial sums and compensations are combined per receiver with "
            "TwoSum" if kahan else
            "fp32: two FP32 accumulators per lane (paired f32x2), partial sums per receiver in FP32")
    result = {
        "metric": "cell-steps/s", "value": value, "unit": "cell-steps/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": total_dev_ms / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic",
        "config": {
            "workload": workload_name(), "cells": n, "edges": int(len(col)), "mean_degree": float(len(col) / n),
            "timesteps_per_step": STEPS_PER_ITER, "trace": f"V_axon every {TRACE_EVERY} timesteps",
            "l2": "flushed between timed steps (256 MB memset)",
            "parallelism": f"replicas x{world}" if world > 1 else "single GPU",
            "plan": plan,
            "coupling_path": "stamped sender-list plan (topology resident in shared memory as 16-bit "
                             "window offsets; the planner prefers it to the dense bitmask because every "
                             "CTA's window fits on chip)",
        },
        "precision": {"coupling_sum": mode, "exp": "ex2.approx on the SFU (coupling), expf (gates)",
                      "ca2plus": "fp64"},
        "e2e": {"value": e2e_value, "unit": "cell-steps/s", "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h},
        "gpu_launches": launches,
        "wall_s": wall,
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": ncu_traffic(kahan),
                     "note": f"achieved = algorithmic bytes (132 + N/8 per cell-step) x cells x "
                             f"{STEPS_PER_ITER} timesteps over the step kernel's mean launch time "
                             f"(CUDA events); peak {peak_kind} HBM copy bandwidth; traffic = ncu "
                             f"DRAM read+write of one launch of this workload (profiles/): the "
                             f"topology and V_dend windows stay on chip, so HBM does not bound the step",
                     "sfu": {"achieved": sfu_ach, "peak": sfu_peak, "unit": "exp2/s", "frac": sfu_ach / sfu_peak,
                             "note": f"one ex2 per edge + 22 exps per cell per timestep; peak = "
                                     f"{SFU_EX2_PER_CLK_SM} per clock per SM x {nsm} SMs x the median SM "
                                     f"clock sampled ({mhz:.0f} MHz)"}},
        "phase_ns_per_timestep": prof["max"],
        "accuracy": {"max_abs_dV_soma_mV": acc, "steps": ACC_STEPS, "vs": "FP64 oracle (oracle/, same "
                     "initial state and topology)", "tolerance_mV": ACC_TOL_MV, "pass": acc <= ACC_TOL_MV},
        "clocks": clocks,
        "cpu_baseline": cpu,
    }
    if other is not None:
        o_ms, o_clk, o_soma, o_step0 = other
        o_acc = soma_error_vs_fp64(conf, n, rp, col, st, o_soma, conf[1], threads, step0=o_step0)
        result["precision"]["other_mode"] = {
            "coupling_sum": "fp32" if kahan else "kahan",
            "value": n * STEPS_PER_ITER * len(o_ms) / (sum(o_ms) * 1e-3), "unit": "cell-steps/s",
            "ms_per_step": sum(o_ms) / len(o_ms), "steps": len(o_ms),
            "max_abs_dV_soma_mV": o_acc, "clocks": o_clk}
    return result


# ------------------------------------------------------- C1 and C3 lines --
def run_gpu_config(args, world, rank, local, which):
    """The other single-network configurations, each a sub-object of the
    default line (one replica per GPU; rank 0's own):
      c1  1,000 cells, the reference generator at p = 0.1 (seed 1), g = 0.04,
          the default initial state (all cells alike: the reference's plain
          run), 20,000 timesteps = 1 s as one bench step; CPU baseline: the
          reference's own build on exactly this configuration (-n 1000 -p 0.1
          -t 1000);
      c3  100,000 cells x 100 senders drawn uniformly, per-edge g U(0.02,
          0.06), per-cell pulses of amplitude U(0, 8) uA/cm2 at onsets U(0,
          500) ms lasting 5 ms, 1,000 timesteps per bench step; CPU baseline:
          the oracle's restatement on the same network (the reference's
          generator takes minutes at this size and cannot draw per-edge g)."""
    import numpy as np
    import torch

    import infoli_gb300 as ig
    from infoli_gb300 import build

    torch.cuda.set_device(local)
    build.build()
    conf = ig.read_parameters(CONF_PATH)
    g = None
    stim = None
    if which == "c1":
        n, steps_per, iters = 1000, 20000, 3
        rp, col = ig.gen_uniform(n, 0.1, SEED)
        st = np.empty((19, n), dtype=np.float32)
        st[:] = conf[23:42][:, None]
        name = "1000 cells, reference generator p=0.1 seed=1, g=0.04, default initial state, 20000 timesteps"
    else:
        n, steps_per, iters = 100000, 1000, 10
        rp, col, g = ig.gen_fixed_degree(n, 100, 3, (0.02, 0.06))
        rng = np.random.default_rng(3)
        amp = rng.uniform(0.0, 8.0, n).astype(np.float32)
        onset = rng.integers(0, 10000, n).astype(np.int32)
        stim = ("cell", amp, onset, 100)
        from infoli_gb300 import workloads

        st = workloads.perturbed_state(conf, n, np.random.default_rng(3))
        name = ("100000 cells x 100 uniform senders, g U(0.02,0.06) per edge, per-cell pulses U(0,8) uA/cm2 at "
                "U(0,500) ms for 5 ms, 1000 timesteps per bench step")
    sim = ig.Simulation(n, conf, rp, col, g=g, init_state=st, device=local, kahan=True)
    if stim is not None:
        sim.set_stimulus_cells(stim[1], stim[2], stim[3])
    plan = sim.plan_info()
    warm = min(args.warmup, 3)
    for _ in range(warm):
        sim.run(min(steps_per, 1000))
    sim.set_state(st)
    dev_ms = []
    with ClockSampler(local) as clk:
        for _ in range(iters):
            flush_l2()
            sim.run(steps_per)
            dev_ms.append(sim.last_run_stats()[0])
    host_state = torch.from_numpy(st).pin_memory().numpy()
    out_state = torch.empty(st.shape, dtype=torch.float32).pin_memory().numpy()
    t0 = time.perf_counter()
    for _ in range(iters):
        sim.set_state(host_state)
        sim.run(steps_per)
        sim.get_state(out=out_state)
    e2e_s = time.perf_counter() - t0
    # accuracy: V_soma every step from the initial state against the FP64
    # oracle (C3 over fewer steps: the FP64 oracle is slow at 1e7 edges)
    acc_steps = ACC_STEPS if which == "c1" else 200
    sim.close()
    # a fresh simulation, so the window is the configuration's first steps
    # (C3's early pulse onsets fall inside it)
    with ig.Simulation(n, conf, rp, col, g=g, init_state=st, device=local, kahan=True) as sim:
        if stim is not None:
            sim.set_stimulus_cells(stim[1], stim[2], stim[3])
        acc_step0 = sim.step
        gpu_soma = sim.run(acc_steps, 1, ig.TRACE_SOMA)["soma"]
    if rank != 0:
        return None
    threads, model = host_cpu()
    from oracle import oracle as O

    s64 = np.ascontiguousarray(st, dtype=np.float64)
    ref64 = O.run(n, np.asarray(conf[:23], dtype=np.float64), s64, rp, col, g=g, g_uniform=conf[1], stim=stim,
                  step0=acc_step0, nsteps=acc_steps, trace_every=1, traces=("soma",), nthreads=threads,
                  fp64=True)["soma"]
    acc = float(np.max(np.abs(gpu_soma.astype(np.float64) - ref64)))
    cell_steps = n * steps_per * iters
    value = cell_steps / (sum(dev_ms) * 1e-3)
    if which == "c1":
        ref = reference_median(n, 0.1, steps_per * 0.05, threads)
        cpu = None if ref is None else {
            "value": ref[0], "unit": "cell-steps/s", "cores": threads, "cpu": model, "kind": "reference",
            "sample": f"the median of three runs of the untouched reference OpenMP build on this configuration "
                      f"(-n 1000 -p 0.1 -t 1000 = 20,000 timesteps), its own execution-time clock: "
                      f"{', '.join(f'{x:.2f}' for x in ref[1])} s"}
    else:
        cpu = None
    if cpu is None:
        from oracle import oracle as O

        s2 = st.copy()
        ps = 100 if which == "c3" else 2000
        t0 = time.perf_counter()
        O.run(n, conf[:23], s2, rp, col, g=g, g_uniform=conf[1], stim=stim, nsteps=ps, trace_every=0, traces=(),
              nthreads=threads)
        dt = time.perf_counter() - t0
        cpu = {"value": n * ps / dt, "unit": "cell-steps/s", "cores": threads, "cpu": model, "kind": "port",
               "sample": f"the oracle's restatement of the reference loop (C + OpenMP) on the same network, {ps} "
                         f"timesteps ({dt:.1f} s)"}
    return {
        "metric": "cell-steps/s", "value": value, "unit": "cell-steps/s", "steps": iters, "warmup": warm,
        "ms_per_step": sum(dev_ms) / iters, "higher_is_better": True,
        "config": {"workload": name, "cells": n, "edges": int(len(col)), "timesteps_per_step": steps_per,
                   "plan": plan, "kahan": True, "l2": "flushed between timed steps (256 MB memset)"},
        "e2e": {"value": cell_steps / e2e_s, "unit": "cell-steps/s", "h2d_bytes_per_step": int(st.nbytes),
                "d2h_bytes_per_step": int(st.nbytes)},
        "clocks": clk.summary(),
        "cpu_baseline": cpu,
        "accuracy": {"max_abs_dV_soma_mV": acc, "steps": acc_steps, "vs": "FP64 oracle (oracle/, same initial "
                     "state, topology and stimulus), V_soma every step", "tolerance_mV": ACC_TOL_MV,
                     "pass": acc <= ACC_TOL_MV,
                     "at_size": "tests/test_gpu_configs.py checks the configuration against the float oracle over "
                                "1-2 s of simulated time, spike steps included"},
    }


# ---------------------------------------------------------------- batched --
BATCH_NETS, BATCH_TIMESTEPS, BATCH_STEP = 512, 10000, 1000


def batched_workload():
    import infoli_gb300 as ig
    from infoli_gb300 import workloads

    conf = ig.read_parameters(CONF_PATH)
    nets, st, meta = workloads.batched(conf, n_nets=BATCH_NETS, seed=SEED)
    return conf, nets, st, meta


def batched_draws(n_nets=BATCH_NETS, lo=256, hi=8192, dens=(0.05, 0.5), g=(0.02, 0.06), seed=SEED):
    """The batched workload's per-network sizes, densities and conductances:
    the first draws of infoli_gb300.workloads.batched (a CPU test checks they
    agree), restated here so the reference arm loads nothing from the
    product.  Edge counts are the expected ones."""
    import numpy as np

    rng = np.random.default_rng(seed)
    sizes = np.clip(np.exp(rng.uniform(np.log(lo), np.log(hi), n_nets)).astype(np.int64), lo, hi)
    p = rng.uniform(dens[0], dens[1], n_nets)
    gs = rng.uniform(g[0], g[1], n_nets).astype(np.float32)
    return {"sizes": sizes, "density": p, "g": gs, "edges": (sizes * (sizes - 1) * p).astype(np.int64)}


def batched_config(meta, extra=None):
    cfg = {
        "workload": f"{BATCH_NETS} independent networks, sizes log-uniform 256-8192, density U(0.05,0.5), "
                    f"g U(0.02,0.06) per network, bitmask topology seeded per network, "
                    f"{BATCH_TIMESTEPS} timesteps per simulation, {BATCH_STEP} timesteps per bench step",
        "networks": BATCH_NETS, "cells": int(meta["sizes"].sum()), "edges": int(meta["edges"].sum()),
        "timesteps_per_step": BATCH_STEP,
        "l2": "inputs larger than L2 (bitmasks %.0f MB)" % (sum(int(n) * ((int(n) + 31) // 32) * 4
                                                                for n in meta["sizes"]) / 1e6),
    }
    if extra:
        cfg.update(extra)
    return cfg


def sample_nets(meta, k):
    """k networks spread evenly over the size order (a stratified sample)."""
    import numpy as np

    order = np.argsort(meta["sizes"], kind="stable")
    return [int(order[int((i + 0.5) * len(order) / k)]) for i in range(k)]


def cpu_batched_rate(conf, nets, st, meta, threads, steps=40, k=8):
    """Oracle restatement on a stratified sample of the networks: sims/s
    (10,000-timestep simulations) extrapolated to the whole batch."""
    import numpy as np

    import infoli_gb300 as ig
    from oracle import oracle as O

    off = np.concatenate([[0], np.cumsum(meta["sizes"])])
    picks = sample_nets(meta, k)
    t_sample = 0.0
    for i in picks:
        n, bits, g = nets[i]
        rp, col = ig.bitmask_to_csr(n, bits)
        s = np.ascontiguousarray(st[:, off[i]:off[i + 1]])
        t0 = time.perf_counter()
        O.run(n, conf[:23], s, rp, col, g_uniform=g, nsteps=steps, trace_every=0, traces=(), nthreads=threads)
        t_sample += time.perf_counter() - t0
    est_batch_s = t_sample * (len(nets) / k) * (BATCH_TIMESTEPS / steps)
    return len(nets) / est_batch_s, t_sample, picks


def reference_batched_rate(nets, meta, threads, k=8, sim_ms=5.0):
    """The reference's own OpenMP build on a stratified sample of the
    networks, each at its own cell count, density and conductance (its
    generator draws a uniform random network of that density), sim_ms of
    simulated time each, timed by its own clock: sims/s (10,000-timestep
    simulations) extrapolated to the whole batch, or None."""
    picks = sample_nets(meta, k)
    t_sample = 0.0
    for i in picks:
        r = run_reference_binary(int(meta["sizes"][i]), float(meta["density"][i]), sim_ms, threads,
                                 g=float(meta["g"][i]))
        if r is None:
            return None
        t_sample += r[1]
    steps = reference_sim_steps(sim_ms)
    est_batch_s = t_sample * (len(nets) / k) * (BATCH_TIMESTEPS / steps)
    return len(nets) / est_batch_s, t_sample, picks


def run_gpu_batched(args, world, rank, local, warmup=None):
    """The batched form (C4): returns its result dict on rank 0."""
    import numpy as np
    import torch

    import infoli_gb300 as ig
    from infoli_gb300 import build

    torch.cuda.set_device(local)
    build.build()
    steps = BATCH_TIMESTEPS // BATCH_STEP  # the whole 10,000-timestep simulation of every network
    warmup = min(args.warmup, 3) if warmup is None else warmup
    conf, nets, st, meta = batched_workload()
    # cells per CTA and bitmask-row residency picked together by the library's
    # autotuner (every candidate timed on a stratified sample of the networks,
    # before the timed region)
    t_tune = time.perf_counter()
    bt = ig.Batch(conf, nets, init_state=st, kahan=True, device=local, shape="auto")
    t_tune = time.perf_counter() - t_tune
    info = bt.info()
    residency = bt.residency
    for _ in range(warmup):
        bt.run(BATCH_STEP)
    bt.set_state(st)
    dist_barrier(world)
    torch.cuda.synchronize()
    dev_ms = []
    t_wall0 = time.perf_counter()
    with ClockSampler(local) as clk:
        for _ in range(steps):
            bt.run(BATCH_STEP)  # one graph launch; inputs (588 MB of bitmasks) exceed L2
            dev_ms.append(bt.info()["last_ms"])
    torch.cuda.synchronize()
    dist_barrier(world)
    wall = time.perf_counter() - t_wall0
    total_dev_ms = dist_max(sum(dev_ms), world)
    cta = bt.cta_info()

    # e2e: state from pinned host memory in, state out, through the C ABI
    host_state = torch.from_numpy(st).pin_memory().numpy()
    out_state = torch.empty(st.shape, dtype=torch.float32).pin_memory().numpy()
    dist_barrier(world)
    t0 = time.perf_counter()
    for _ in range(steps):
        bt.set_state(host_state)
        bt.run(BATCH_STEP)
        out_state[:] = bt.get_state()
    e2e_s = dist_max(time.perf_counter() - t0, world)
    finite = float(np.mean([np.isfinite(bt.net_state(out_state, i)).all() for i in range(len(nets))]))
    bt.close()

    sims = len(nets) * world * (BATCH_STEP * steps / BATCH_TIMESTEPS)
    value = sims / (total_dev_ms * 1e-3)
    e2e_value = sims / e2e_s
    edges = int(meta["edges"].sum())

    # sequential plain runs: every network alone through infoli_sim (the
    # single-network path, each on its auto-selected plan), one after another,
    # BATCH_STEP timesteps each, the same summation mode
    off = np.concatenate([[0], np.cumsum(meta["sizes"])])
    plain_dev_s, plain_create_s = 0.0, 0.0
    t_plain0 = time.perf_counter()
    for i in range(len(nets)):
        n, bits, g = nets[i]
        rp, col = ig.bitmask_to_csr(n, bits)
        tc = time.perf_counter()
        with ig.Simulation(n, conf, rp, col, g_uniform=g, init_state=st[:, off[i]:off[i + 1]], kahan=True,
                           device=local) as sim:
            plain_create_s += time.perf_counter() - tc
            sim.run(BATCH_STEP)
            plain_dev_s += sim.last_run_stats()[0] * 1e-3
            sim.get_state()
    plain_wall_s = time.perf_counter() - t_plain0
    sims_per_plain_pass = len(nets) * BATCH_STEP / BATCH_TIMESTEPS
    plain_rate = sims_per_plain_pass / plain_dev_s
    plain_rate_wall = sims_per_plain_pass / (plain_wall_s - plain_create_s)

    # accuracy: the three smallest networks as a batch of their own, ACC_STEPS
    # steps, final V_soma against the FP64 oracle
    acc_ids = [int(i) for i in np.argsort(meta["sizes"])[:3]]
    acc_nets = [nets[i] for i in acc_ids]
    acc_st = np.concatenate([st[:, off[i]:off[i + 1]] for i in acc_ids], axis=1)
    with ig.Batch(conf, acc_nets, init_state=acc_st, kahan=True, device=local, shape=info["block"],
                  residency=residency) as ab:
        ab.run(ACC_STEPS)
        acc_out = ab.get_state()
        acc_soma = [ab.net_state(acc_out, k)[7] for k in range(len(acc_ids))]

    if rank != 0:
        return None
    threads, model = host_cpu()
    acc = 0.0
    for k, i in enumerate(acc_ids):
        n_i, bits_i, g_i = nets[i]
        rp_i, col_i = ig.bitmask_to_csr(n_i, bits_i)
        acc = max(acc, soma_error_vs_fp64(conf, n_i, rp_i, col_i, st[:, off[i]:off[i + 1]], acc_soma[k], g_i,
                                          threads, final_only=True))
    cpu_rate, cpu_t, cpu_picks = cpu_batched_rate(conf, nets, st, meta, threads)
    ref_b = reference_batched_rate(nets, meta, threads)
    if ref_b is not None:
        cpu = {"value": ref_b[0], "unit": "sims/s", "cores": threads, "cpu": model, "kind": "reference",
               "sample": f"the untouched reference OpenMP build on networks {ref_b[2]} (each -n size -p density, "
                         f"CONDUCTANCE = its g, -t 5 = 100 timesteps; its own execution-time clock, "
                         f"{ref_b[1]:.1f} s in all), extrapolated to {len(nets)} networks x {BATCH_TIMESTEPS} "
                         f"timesteps",
               "port": {"value": cpu_rate, "sample": f"oracle restatement on networks {cpu_picks} x 40 timesteps "
                                                     f"({cpu_t:.1f} s), extrapolated"}}
    else:
        cpu = {"value": cpu_rate, "unit": "sims/s", "cores": threads, "cpu": model, "kind": "port",
               "sample": f"networks {cpu_picks} x 40 timesteps ({cpu_t:.1f} s), extrapolated"}
    # algorithmic bytes of one launch: the bitmask rows once per timestep
    # (networks whose rows stay in shared memory are still counted) and 132 B
    # of state per cell-step
    bits_bytes = sum(int(n) * ((int(n) + 31) // 32) * 4 for n in meta["sizes"])
    alg = (bits_bytes + 132 * int(meta["sizes"].sum())) * BATCH_STEP
    launch_ms = sum(dev_ms) / len(dev_ms)
    achieved = alg / (launch_ms * 1e-3) / 1e9
    peak, peak_kind = peaks()
    nsm = sm_count(local)
    busy = float((cta["end_ns"] - cta["start_ns"]).sum()) / (nsm * float(cta["end_ns"].max()))
    return {
        "metric": "sims/s", "value": value, "unit": "sims/s (10,000-timestep simulations)",
        "steps": steps, "warmup": warmup, "ms_per_step": total_dev_ms / steps, "higher_is_better": True,
        "config": batched_config(meta, {"layout": info, "kahan": True, "autotune": bt.tune,
                                        "autotune_s": t_tune}),
        "cell_steps_per_s": int(meta["sizes"].sum()) * BATCH_STEP * steps * world / (total_dev_ms * 1e-3),
        "edge_evals_per_s": edges * BATCH_STEP * steps * world / (total_dev_ms * 1e-3),
        "finite_fraction": finite,
        "accuracy": {"max_abs_dV_soma_mV": acc, "steps": ACC_STEPS, "networks": acc_ids,
                     "vs": "FP64 oracle, V_soma after the last step (the batch's three smallest networks run "
                           "as a batch of their own)", "tolerance_mV": ACC_TOL_MV, "pass": acc <= ACC_TOL_MV},
        "sequential_plain": {
            "value": plain_rate, "unit": "sims/s", "value_wall": plain_rate_wall,
            "sample": f"all {len(nets)} networks, one after another through infoli_sim (Kahan, each on its "
                      f"auto-selected plan), {BATCH_STEP} timesteps each: device time {plain_dev_s:.2f} s "
                      f"(value), wall time without creation {plain_wall_s - plain_create_s:.2f} s "
                      f"(value_wall), creation {plain_create_s:.2f} s; the batched bench step is the same "
                      f"{BATCH_STEP} timesteps of every network",
            "speedup_batched_vs_plain": value / plain_rate},
        "e2e": {"value": e2e_value, "unit": "sims/s", "h2d_bytes_per_step": int(st.nbytes),
                "d2h_bytes_per_step": int(st.nbytes)},
        # per bench step: one launch per cluster-size group + the step-index advance
        "gpu_launches": steps * (len({(int(n) + info["block"] - 1) // info["block"]
                                      for n in meta["sizes"]}) + 1),
        "wall_s": wall,
        "sm_busy_fraction": busy,
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": None,
                     "note": f"achieved = bitmask bytes + 132 B per cell-step per timestep over the mean "
                             f"launch time; peak {peak_kind} HBM copy bandwidth; the batched kernel is "
                             f"issue-bound (bit extraction + SFU exp per edge), not HBM-bound"},
        "clocks": clk.summary(),
        "cpu_baseline": cpu,
    }


def run_reference_batched(args, world, rank):
    if rank != 0:
        return 0
    from oracle import oracle as O

    O.build()
    conf = O.read_parameters(CONF_PATH)
    threads, model = host_cpu()
    # the networks' sizes, densities and conductances (the same draws as the
    # GPU arm's workload), without building the bitmasks or loading the product
    meta = batched_draws()
    nets = [None] * BATCH_NETS
    rates = []
    kind = "reference"
    if reference_batched_rate(nets, meta, threads, k=2) is None:
        kind = None
    t_total = 0.0
    picks = []
    if kind == "reference":
        for _ in range(args.warmup):
            reference_batched_rate(nets, meta, threads, k=2)
        for _ in range(args.steps):
            r, t, picks = reference_batched_rate(nets, meta, threads, k=4)
            rates.append(r)
            t_total += t
        sample = (f"per bench step the untouched reference OpenMP build on networks {picks} (-n size -p density, "
                  f"CONDUCTANCE = its g, 100 timesteps, its own clock), extrapolated")
    else:
        kind = "port"
        conf, nets, st, meta = batched_workload()
        for _ in range(args.warmup):
            cpu_batched_rate(conf, nets, st, meta, threads, steps=2, k=2)
        for _ in range(args.steps):
            r, t, picks = cpu_batched_rate(conf, nets, st, meta, threads, steps=5, k=4)
            rates.append(r)
            t_total += t
        sample = f"per bench step networks {picks} x 5 timesteps of the oracle port, extrapolated"
    value = statistics.mean(rates)
    line = {
        "impl": "reference", "metric": "sims/s", "value": value, "unit": "sims/s (10,000-timestep simulations)",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * t_total / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic", "config": batched_config(meta),
        "cpu_baseline": {"value": value, "unit": "sims/s", "cores": threads, "cpu": model, "kind": kind,
                         "sample": sample},
        "e2e": {"value": value, "unit": "sims/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))
    return 0


# ---------------------------------------------------------------- serving --
SERVE_RATE, SERVE_REQUESTS = 50.0, 24


def serving_requests(conf, count, seed=SEED):
    """Poisson arrivals (mean SERVE_RATE per s); sizes log-uniform 500-50,000
    cells; durations U(100, 2000) ms = 2,000-40,000 steps of 0.05 ms; density
    U(0.01, 0.30); g = 0.04; topology from seed 1000 + k."""
    import numpy as np

    import infoli_gb300 as ig
    from infoli_gb300 import workloads

    rng = np.random.default_rng(seed)
    t = np.cumsum(rng.exponential(1.0 / SERVE_RATE, count))
    t -= t[0]
    sizes = np.exp(rng.uniform(np.log(500), np.log(50000), count)).astype(np.int64)
    steps = np.round(rng.uniform(100, 2000, count) / 0.05).astype(np.int64)
    dens = rng.uniform(0.01, 0.30, count)
    reqs = []
    for k in range(count):
        n = int(sizes[k])
        rp, col = ig.gen_bitmask_csr(n, float(dens[k]), 1000 + k)
        reqs.append(dict(n=n, row_ptr=rp, col=col, n_steps=int(steps[k]), g_uniform=0.04,
                         init_state=workloads.perturbed_state(conf, n, rng)))
    return t, reqs


def run_gpu_serving(args, world, rank, local, count=SERVE_REQUESTS, warmup=None):
    """The served form (C5): returns its result dict on rank 0."""
    import numpy as np
    import torch

    import infoli_gb300 as ig
    from infoli_gb300 import build

    torch.cuda.set_device(local)
    build.build()
    warmup = min(args.warmup, 3) if warmup is None else warmup
    conf = ig.read_parameters(CONF_PATH)
    arrivals, reqs = serving_requests(conf, count)
    work = np.array([len(r["col"]) * r["n_steps"] for r in reqs], dtype=np.float64)
    with ig.Server(conf, device=local, kahan=True, lane_sms=args.lane_sms) as sv:
        # warm-up: small requests through the same server
        wu = [sv.submit(n=r["n"], row_ptr=r["row_ptr"], col=r["col"], n_steps=200, g_uniform=0.04,
                        init_state=r["init_state"]) for r in sorted(reqs, key=lambda r: r["n"])[:warmup]]
        for i in wu:
            sv.wait(i, want_state=False)
        dist_barrier(world)
        t0 = time.perf_counter()
        ids = []
        with ClockSampler(local) as clk:
            for k, r in enumerate(reqs):
                delay = arrivals[k] - (time.perf_counter() - t0)
                if delay > 0:
                    time.sleep(delay)
                ids.append((sv.submit(**r), time.perf_counter() - t0))
            infos = [sv.wait(i, want_state=False)[1] for i, _ in ids]
        makespan = time.perf_counter() - t0
    lat = np.array([i["done_s"] - i["submit_s"] for i in infos])
    served = count / makespan

    # sequential plain runs: each request alone through infoli_sim (create +
    # run + state read back, the whole GPU), then a first-in-first-out
    # schedule with the same arrival times
    service, plain_create = [], []
    for r in reqs:
        ts = time.perf_counter()
        with ig.Simulation(r["n"], conf, r["row_ptr"], r["col"], g_uniform=0.04, init_state=r["init_state"],
                           kahan=True, device=local) as sim:
            plain_create.append(time.perf_counter() - ts)
            sim.run(r["n_steps"])
            sim.get_state()
        service.append(time.perf_counter() - ts)
    finish, seq_lat = 0.0, []
    for a, sdur in zip(arrivals, service):
        finish = max(finish, a) + sdur
        seq_lat.append(finish - a)
    seq_lat = np.array(seq_lat)
    seq_rate = count / finish

    if rank != 0:
        return None
    in_bytes = sum(r["row_ptr"].nbytes + r["col"].nbytes + r["init_state"].nbytes for r in reqs)
    return {
        "metric": "served sims/s", "value": served, "unit": "sims/s", "steps": count,
        "warmup": warmup, "ms_per_step": 1e3 * makespan / count, "higher_is_better": True,
        "config": {"workload": f"Poisson request stream, mean {SERVE_RATE:g}/s, {count} requests (one per "
                               f"bench step), sizes log-uniform 500-50000 cells, durations U(100,2000) ms, "
                               f"density U(0.01,0.30), g=0.04, admitted by HBM budget (80% of free memory)",
                   "requests": count, "cells": [r["n"] for r in reqs], "timesteps": [r["n_steps"] for r in reqs],
                   "edges": [int(len(r["col"])) for r in reqs],
                   "arrivals_s": [round(float(a), 4) for a in arrivals],
                   "timing": "host wall clock from the first arrival to the last result (serving is end to end)",
                   "paths": ("no lane: every request runs its own persistent launch" if args.lane_sms < 0 else
                             "requests of at most 8192 cells with one conductance and at most 24576 edges per "
                             "CTA of their cluster run in the lane (the batched cluster kernel relaunched every "
                             "2000 steps over all of them, joining between launches); the others each run their "
                             f"own persistent launch, leaving {args.lane_sms} SMs to the lane"),
                   "l2": "inputs larger than L2"},
        "latency_s": {"p50": float(np.percentile(lat, 50)), "p99": float(np.percentile(lat, 99)),
                      "max": float(lat.max())},
        "sequential_plain": {"value": seq_rate, "unit": "sims/s",
                             "latency_s": {"p50": float(np.percentile(seq_lat, 50)),
                                           "p99": float(np.percentile(seq_lat, 99))},
                             "sample": "every request alone through infoli_sim (create+run+read), measured one "
                                       "after another; first-in-first-out schedule on the same arrivals"},
        "offered_edge_evals_per_s": float(work.sum() / max(arrivals[-1], 1e-9)),
        "sustained_edge_evals_per_s": float(work.sum() / makespan),
        "e2e": {"value": served, "unit": "sims/s", "h2d_bytes_per_step": int(in_bytes / count),
                "d2h_bytes_per_step": int(sum(19 * 4 * r["n"] for r in reqs) / count)},
        "placement_per_request": [i["grid"] for i in infos],
        "lane_per_request": [i["lane"] for i in infos],
        "lane_launches_per_request": [i["lane_launches"] for i in infos],
        "prepare_s_per_request": [round(i["prepared_s"] - i["prep_start_s"], 3) for i in infos],
        "launch_wait_s_per_request": [round(i["start_s"] - i["prepared_s"], 3) for i in infos],
        "run_s_per_request": [round(i["done_s"] - i["start_s"], 3) for i in infos],
        "plain_service_s_per_request": [round(x, 3) for x in service],
        "gpu_launches": int(sum((r["n_steps"] + 8191) // 8192 for r in reqs)),
        "clocks": clk.summary(),
    }


# ------------------------------------------------------------------ cases --
CASES = ("grid10k", "uniform1k", "dense10k", "sparse100k", "batch64", "serve43k")


def run_case(name, steps):
    """One named small case, run once; prints its device time.  Seeded inputs:
      grid10k    the headline workload (10,000-cell Gaussian grid), stamped plan
      uniform1k  1,000 cells, the reference generator at p = 0.1
      dense10k   10,000 cells, bitmask generator at p = 0.2 (coupling-dominated)
      sparse100k 100,000 cells, 100 senders each, per-edge g U(0.02, 0.06)
      batch64    the first 64 networks of the batched workload, one graph launch
      serve43k   the serving stream's largest request (43,533 cells, density
                 0.28, g = 0.04), bitmask plan"""
    import numpy as np

    import infoli_gb300 as ig
    from infoli_gb300 import build, workloads

    build.build()
    conf = ig.read_parameters(CONF_PATH)
    if name == "batch64":
        nets, st, meta = workloads.batched(conf, n_nets=64, seed=1)
        with ig.Batch(conf, nets, init_state=st, kahan=True) as bt:
            bt.run(steps)
            print(f"batch64: {int(meta['sizes'].sum())} cells, {int(meta['edges'].sum())} edges, {bt.info()}")
        return 0
    rng = np.random.default_rng(1)
    g = None
    if name == "grid10k":
        _, n, rp, col, st = workload()
    elif name == "serve43k":
        _, reqs = serving_requests(conf, SERVE_REQUESTS)
        r = reqs[4]
        n, rp, col, st = r["n"], r["row_ptr"], r["col"], r["init_state"]
    else:
        if name == "uniform1k":
            n = 1000
            rp, col = ig.gen_uniform(n, 0.1, 1)
        elif name == "dense10k":
            n = 10000
            rp, col = ig.gen_bitmask_csr(n, 0.2, 5)
        else:
            n = 100000
            rp, col, g = ig.gen_fixed_degree(n, 100, 3, (0.02, 0.06))
        st = workloads.perturbed_state(conf, n, rng)
    with ig.Simulation(n, conf, rp, col, g=g, init_state=st, kahan=True) as sim:
        sim.run(steps)
        ms, launches = sim.last_run_stats()
        print(f"{name}: {n} cells, {len(col)} edges, plan {sim.plan_info()}, {steps} steps in {ms:.3f} ms "
              f"({launches} launches)")
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=None)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="all", choices=["all", "grid10k", "batched", "serving", "c1", "c3"])
    ap.add_argument("--case", choices=CASES, default=None)
    ap.add_argument("--no-kahan", action="store_true", help="headline with the uncompensated coupling sum")
    ap.add_argument("--lane-sms", type=int, default=0,
                    help="serving: SMs larger requests leave to the lane of small ones (0 = the library's "
                         "default, < 0 = no lane)")
    args = ap.parse_args()
    if args.case:
        return run_case(args.case, args.steps or 100)
    if args.steps is None:
        args.steps = {"all": 20, "grid10k": 20, "batched": 10, "serving": SERVE_REQUESTS, "c1": 3, "c3": 10}[
            args.workload]
    world, rank, local = dist_setup()
    if args.impl == "reference":
        if args.workload == "serving":
            print(json.dumps({"impl": "reference", "unavailable": "the reference has no serving mode; its "
                              "per-request CPU cost is the headline reference arm"}))
            return 0
        if args.workload == "batched":
            return run_reference_batched(args, world, rank)
        return run_reference(args, world, rank)
    if args.workload == "batched":
        res = run_gpu_batched(args, world, rank, local, warmup=args.warmup)
        if res is not None:
            res.update({"n_gpus": world, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic"})
            print(json.dumps(res))
        return 0
    if args.workload in ("c1", "c3"):
        res = run_gpu_config(args, world, rank, local, args.workload)
        if res is not None:
            res.update({"n_gpus": world, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic"})
            print(json.dumps(res))
        return 0
    if args.workload == "serving":
        res = run_gpu_serving(args, world, rank, local, count=args.steps, warmup=args.warmup)
        if res is not None:
            res.update({"n_gpus": world, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic"})
            print(json.dumps(res))
        return 0
    line = run_gpu(args, world, rank, local)
    if args.workload == "all":
        # the batched and served forms on the same GPU, in the same run (one
        # replica per GPU under torchrun: the sub-objects are rank 0's own)
        bres = run_gpu_batched(args, world, rank, local)
        sres = run_gpu_serving(args, world, rank, local)
        c1 = run_gpu_config(args, world, rank, local, "c1")
        c3 = run_gpu_config(args, world, rank, local, "c3")
        if line is not None:
            line["batched"] = bres
            line["serving"] = sres
            line["c1"] = c1
            line["c3"] = c3
    if line is not None:
        print(json.dumps(line))
    return 0


if __name__ == "__main__":
    sys.exit(main())
