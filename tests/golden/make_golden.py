"""Regenerate the golden fixtures in tests/golden/ from the UNTOUCHED reference
binaries built by oracle/build_ref.sh (oracle/_ref/).  Needs the reference
tree (only present where it is mounted); the tests themselves only read the
committed fixtures.

Fixtures
  omp_test_n50_p0.3_t25.npz   reference OpenMP build, -DG_CAL_FROM_FILE
                              (make target omp_test), seed 1,
                              -n 50 -p 0.3 -t 25: V_axon every step (500 x 50)
                              plus the g_CaL values it read; exercises the
                              built-in generator + coupling + update
  omp_test_n20_p0.5_t1100.npz same, -n 20 -p 0.5 -t 1100 (22000 steps, the
                              6 uA pulse at steps 20000-20498 makes the cells
                              spike): every 10th row + per-cell spike steps
  omp_n200_p0.1_t30.txt       reference OpenMP build (normal trace format,
                              tagged, every 100th step), seed 1,
                              -n 200 -p 0.1 -t 30, header line 1 blanked
  omp_test_n1000_p0.1_t5.npz  reference OpenMP build, -DG_CAL_FROM_FILE, seed
                              1, -n 1000 -p 0.1 -t 5 (the C1 configuration's
                              network with per-cell g_CaL, so the cells differ
                              and the coupling acts; 100 steps): V_axon of every
                              10th step plus the g_CaL values it read
  kat_stable_version.npz      the reference's regression golden generator
                              (src/regression_test/stable_version.c) on its
                              own fixtures (10 cells, cellConnections.txt,
                              gcal_file.txt), SIMTIME 2000 ms: V_axon rows for
                              the first 10000 steps (the 'standard' 500 ms
                              check) + every 100th row + spike steps; also the
                              fixture conductance matrix and g_CaL values
  single_rand_init.npz        src/single_threaded/infoli.c with its RAND_INIT
                              switch at 1 (oracle/_ref/single_rand.x, seed 1):
                              randomised initial states (g_CaL and isolated
                              steps drawn by rand()), then its SIMTIME of 10 ms
                              (200 steps) in FP64, V_axon every step; on 10
                              cells coupled by the regression fixture's
                              conductance matrix and on 64 uncoupled cells;
                              and on 16 cells (30 % density, conductances
                              1/32, 3/64, 1/16: exact in binary, so float32 and
                              double agree) driven by a 400-line stimulus file
                              (the program's input-file mode, V_axon printed
                              with 16 decimals)
Usage: python tests/golden/make_golden.py
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
REF = os.environ.get("INFOLI_REFERENCE_DIR", "/root/reference")
BIN = os.path.join(ROOT, "oracle", "_ref")


def spikes(v: np.ndarray) -> list:
    """Steps (row index) at which each column crosses 0 mV upwards."""
    out = []
    for c in range(v.shape[1]):
        x = v[:, c]
        out.append((np.nonzero((x[:-1] < 0) & (x[1:] >= 0))[0] + 1).astype(np.int32))
    return out


def run(exe, args, cwd):
    env = dict(os.environ, OMP_NUM_THREADS="1")
    subprocess.run([exe, *args], cwd=cwd, env=env, check=True, stdout=subprocess.DEVNULL)


def omp_test_case(n, p, t, gcal_seed):
    rng = np.random.RandomState(gcal_seed)
    gcal_txt = " ".join("%.4f" % x for x in (0.6 + 0.2 * rng.rand(n)))
    with tempfile.TemporaryDirectory() as d:
        with open(os.path.join(d, "gcal_file.txt"), "w") as f:
            f.write(gcal_txt)
        run(os.path.join(BIN, "infoli_omp_test.x"),
            ["-n", str(n), "-p", str(p), "-t", str(t), "-c", os.path.join(BIN, "default.conf"), "-o", "out.txt"], d)
        rows = [np.array(l.split(), dtype=np.float64) for l in open(os.path.join(d, "out.txt"))]
    v = np.array(rows, dtype=np.float64)  # exact parse of the 8-decimal text
    gcal = np.array([float(x) for x in gcal_txt.split()], dtype=np.float32)
    return v, gcal, gcal_txt


def main():
    if not os.path.exists(os.path.join(BIN, "infoli_omp.x")):
        subprocess.run([os.path.join(ROOT, "oracle", "build_ref.sh")], check=True)

    v, gcal, txt = omp_test_case(50, 0.3, 25, 3)
    np.savez_compressed(os.path.join(HERE, "omp_test_n50_p0.3_t25.npz"), v_axon=v, gcal=gcal,
                        gcal_text=np.array(txt), n=50, p=np.float32(0.3), t=np.float32(25), seed=1)

    v, gcal, txt = omp_test_case(20, 0.5, 1100, 5)
    sp = spikes(v)
    np.savez_compressed(os.path.join(HERE, "omp_test_n20_p0.5_t1100.npz"), v_axon_every10=v[::10],
                        gcal=gcal, gcal_text=np.array(txt), n=20, p=np.float32(0.5), t=np.float32(1100),
                        seed=1, n_steps=v.shape[0],
                        **{f"spikes_{c}": s for c, s in enumerate(sp)})

    with tempfile.TemporaryDirectory() as d:
        run(os.path.join(BIN, "infoli_omp.x"),
            ["-n", "200", "-p", "0.1", "-t", "30", "-c", os.path.join(BIN, "default.conf"), "-o", "out.txt"], d)
        lines = open(os.path.join(d, "out.txt")).read().split("\n")
    lines[0] = "Execution Time for Simulation in ms: <timing>"
    with open(os.path.join(HERE, "omp_n200_p0.1_t30.txt"), "w") as f:
        f.write("\n".join(lines))

    v, gcal, txt = omp_test_case(1000, 0.1, 5, 11)
    assert v.shape == (100, 1000)
    np.savez_compressed(os.path.join(HERE, "omp_test_n1000_p0.1_t5.npz"), v_axon_every10=v[9::10], gcal=gcal,
                        gcal_text=np.array(txt), n=1000, p=np.float32(0.1), t=np.float32(5), seed=1)

    src = os.path.join(REF, "src", "regression_test")
    with tempfile.TemporaryDirectory() as d:
        shutil.copy(os.path.join(src, "cellConnections.txt"), d)
        shutil.copy(os.path.join(src, "gcal_file.txt"), d)
        run(os.path.join(BIN, "stable_version.x"), ["10"], d)
        v = np.array([np.array(l.split(), dtype=np.float64) for l in
                      open(os.path.join(d, "InferiorOlive_Output_Baseline.txt"))], dtype=np.float64)
        g = np.loadtxt(os.path.join(src, "cellConnections.txt"), dtype=np.float32)
        gcal = np.loadtxt(os.path.join(src, "gcal_file.txt"), dtype=np.float32)
    sp = spikes(v)
    np.savez_compressed(os.path.join(HERE, "kat_stable_version.npz"), v_axon_first10000=v[:10000],
                        v_axon_every100=v[::100], n_steps=v.shape[0], cond_sender_by_receiver=g,
                        gcal=gcal, **{f"spikes_{c}": s for c, s in enumerate(sp)})
    out = {}
    for tag, n, cond in (("coupled10", 10, np.loadtxt(os.path.join(src, "cellConnections.txt"))),
                         ("isolated64", 64, np.zeros((64, 64)))):
        with tempfile.TemporaryDirectory() as d:
            with open(os.path.join(d, "cellConnections.txt"), "w") as f:
                for row in cond:
                    f.write(" ".join(repr(float(x)) for x in row) + "\n")
            run(os.path.join(BIN, "single_rand.x"), [str(n)], d)
            lines = open(os.path.join(d, "InferiorOlive_Output.txt")).read().splitlines()[1:]
        # rows: " step iApp 1 : v1 2 : v2 ..."; the values are every third token from the fourth
        v = np.array([[float(t) for t in l.split()[4::3]] for l in lines], dtype=np.float64)
        assert v.shape == (200, n)
        out[f"v_axon_{tag}"] = v
        out[f"cond_sender_by_receiver_{tag}"] = cond.astype(np.float32)
    rng = np.random.default_rng(7)
    n = 16
    cond = np.where(rng.random((n, n)) < 0.3, rng.choice([0.03125, 0.046875, 0.0625], (n, n)), 0.0)
    np.fill_diagonal(cond, 0.0)
    amp = rng.choice([0.0, 2.5, 5.0, 7.25], n)
    onset = rng.integers(0, 300, n)
    stim = np.array([[amp[c] if onset[c] <= t < onset[c] + 100 else 0.0 for c in range(n)] for t in range(400)])
    with tempfile.TemporaryDirectory() as d:
        with open(os.path.join(d, "cellConnections.txt"), "w") as f:
            for row in cond:
                f.write(" ".join(repr(float(x)) for x in row) + "\n")
        with open(os.path.join(d, "stim.txt"), "w") as f:
            for row in stim:
                f.write(" ".join("%.4f" % x for x in row) + "\n")
        run(os.path.join(BIN, "single_rand.x"), [str(n), "stim.txt"], d)
        lines = open(os.path.join(d, "InferiorOlive_Output.txt")).read().splitlines()[1:]
    # input-file mode rows: "step time v1 v2 ..."
    v = np.array([[float(t) for t in l.split()[2:]] for l in lines], dtype=np.float64)
    assert v.shape == (400, n)
    out["v_axon_stim16"] = v
    out["cond_sender_by_receiver_stim16"] = cond.astype(np.float32)
    out["stim_stim16"] = stim.astype(np.float32)
    np.savez_compressed(os.path.join(HERE, "single_rand_init.npz"), seed=1, **out)
    print("fixtures written to", HERE)


if __name__ == "__main__":
    sys.exit(main())
