"""The multi-GPU row of the path is "replicas only": bench.py --gpus N runs N
independent simulations, one per rank, joined only by a barrier and a MAX of
the timings (no data-path collective).  These tests run that host logic as
two gloo ranks on the CPU, launched the way the driver launches bench.py."""
import json
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _torchrun(args, timeout=600):
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(_port()), *args]
    env = dict(os.environ, OMP_NUM_THREADS="2")
    return subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=timeout, env=env)


def test_two_ranks_barrier_and_max_over_ranks():
    r = _torchrun([os.path.join("tests", "dist_probe.py")])
    assert r.returncode == 0, r.stdout + r.stderr
    lines = [json.loads(l) for l in r.stdout.splitlines() if l.startswith("{")]
    assert sorted(d["rank"] for d in lines) == [0, 1]
    assert all(d["world"] == 2 and d["max"] == 20.0 for d in lines)


def test_reference_arm_under_two_ranks_prints_one_line(built):
    r = _torchrun(["bench.py", "--impl", "reference", "--gpus", "2", "--steps", "1", "--warmup", "0"])
    assert r.returncode == 0, r.stdout + r.stderr
    lines = [json.loads(l) for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1  # rank 0 alone prints; rank 1 exits without work
    d = lines[0]
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["value"] > 0
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["cpu_baseline"]["kind"] in ("reference", "port")


def test_reference_arm_loads_nothing_from_the_product(built):
    """The reference arm times the reference's own build (or the oracle port)
    and must not load the GPU library or import the product package."""
    code = ("import runpy, sys\n"
            "sys.argv = ['bench.py', '--impl', 'reference', '--steps', '1', '--warmup', '0']\n"
            "try:\n    runpy.run_path('bench.py', run_name='__main__')\nexcept SystemExit:\n    pass\n"
            "maps = open('/proc/self/maps').read()\n"
            "print('PRODUCT', 'infoli_gb300' in sys.modules, 'libinfoli_gpu' in maps)\n")
    r = subprocess.run([sys.executable, "-c", code], cwd=ROOT, capture_output=True, text=True, timeout=600,
                       env=dict(os.environ, OMP_NUM_THREADS="2"))
    assert r.returncode == 0, r.stdout + r.stderr
    assert "PRODUCT False False" in r.stdout, r.stdout


def test_reference_arm_batched_draws_match_the_workload():
    """The batched reference arm draws the networks' sizes, densities and
    conductances itself (it loads nothing from the product); they are the
    GPU arm's."""
    sys.path.insert(0, ROOT)
    import numpy as np

    import bench
    import infoli_gb300 as ig
    from infoli_gb300 import workloads

    conf = ig.read_parameters(bench.CONF_PATH)
    _, _, meta = workloads.batched(conf, n_nets=40, seed=3)
    d = bench.batched_draws(n_nets=40, seed=3)
    assert np.array_equal(d["sizes"], meta["sizes"]) and np.array_equal(d["density"], meta["density"])
    assert np.array_equal(d["g"], meta["g"])
