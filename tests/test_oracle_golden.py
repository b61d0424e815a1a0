"""The CPU oracle is pinned to the untouched reference (golden fixtures made by
tests/golden/make_golden.py from oracle/build_ref.sh's binaries)."""
import numpy as np
import pytest

from helpers import CONF, golden, kat_topology, spike_steps
from oracle import oracle as O


@pytest.fixture(scope="module")
def conf(built):
    return O.read_parameters(CONF)


def _fmt8(a):
    return np.array([float("%.8f" % float(x)) for x in a.ravel()]).reshape(a.shape)


def test_read_parameters_matches_reference_defaults(conf):
    assert conf.shape == (42,)
    assert conf[0] == np.float32(0.05) and conf[1] == np.float32(0.04)
    assert conf[23] == -60 and conf[41] == np.float32(0.2369847)


def test_generator_known_answer(built):
    # seed-1 draws of the reference generator on 50 cells at p=0.3 (742 edges)
    rp, col = O.gen_uniform(50, np.float32(0.3), 1)
    assert rp[-1] == 742
    for r in range(50):
        row = col[rp[r]:rp[r + 1]]
        assert np.all(np.diff(row) > 0) and r not in row


def test_oracle_bit_exact_vs_reference_omp_test(conf):
    """Generator + coupling + update, 50 cells, 500 steps: byte-identical trace text."""
    z = golden("omp_test_n50_p0.3_t25.npz")
    n = int(z["n"])
    rp, col = O.gen_uniform(n, np.float32(z["p"]), int(z["seed"]))
    st = O.default_state(n, conf)
    st[O.S["g_CaL"]] = z["gcal"]
    steps = int(np.float32(z["t"]) / conf[0])
    tr = O.run(n, conf[:23], st, rp, col, g_uniform=conf[1], nsteps=steps, trace_every=1,
               traces=("axon",))["axon"]
    assert np.array_equal(_fmt8(tr), z["v_axon"])


def test_oracle_bit_exact_vs_reference_at_the_c1_size(conf):
    """The C1 configuration's network (1,000 cells, the reference generator at
    p = 0.1, seed 1) with per-cell g_CaL (the plain run's identical cells
    would leave the coupling at zero), 100 steps against the reference's
    omp_test build: every 10th row byte-identical."""
    z = golden("omp_test_n1000_p0.1_t5.npz")
    n = int(z["n"])
    rp, col = O.gen_uniform(n, np.float32(z["p"]), int(z["seed"]))
    st = O.default_state(n, conf)
    st[O.S["g_CaL"]] = z["gcal"]
    steps = int(np.float32(z["t"]) / conf[0])
    tr = O.run(n, conf[:23], st, rp, col, g_uniform=conf[1], nsteps=steps, trace_every=1,
               traces=("axon",), nthreads=O.max_threads())["axon"]
    assert np.array_equal(_fmt8(tr[9::10]), z["v_axon_every10"])
    assert np.std(z["v_axon_every10"][-1]) > 1e-4  # the cells differ


def test_oracle_bit_exact_through_spikes(conf):
    """20 cells, 22000 steps with the 6 uA pulse: same rows and spike steps."""
    z = golden("omp_test_n20_p0.5_t1100.npz")
    n = int(z["n"])
    rp, col = O.gen_uniform(n, np.float32(z["p"]), int(z["seed"]))
    st = O.default_state(n, conf)
    st[O.S["g_CaL"]] = z["gcal"]
    steps = int(z["n_steps"])
    tr = O.run(n, conf[:23], st, rp, col, g_uniform=conf[1], nsteps=steps, trace_every=1,
               traces=("axon",))["axon"]
    assert np.array_equal(_fmt8(tr[::10]), z["v_axon_every10"])
    sp = spike_steps(tr)
    for c in range(n):
        assert np.array_equal(sp[c], z[f"spikes_{c}"])


def test_oracle_trace_format_vs_reference_output(conf):
    """Normal build output file (src/openmp/infoli.c:383-396,682-696): header, then
    every 100th step ' %d %.2f ' + '%d : %.8f ' per cell; byte-identical rows."""
    lines = open(__import__("os").path.join(__import__("helpers").GOLDEN, "omp_n200_p0.1_t30.txt")).read().split("\n")
    n = 200
    assert lines[2] == "#simSteps Input(Iapp) Output(V_axon)" + "".join("%d " % c for c in range(n))
    st = O.default_state(n, conf)
    rp, col = O.gen_uniform(n, np.float32(0.1), 1)
    tr = O.run(n, conf[:23], st, rp, col, g_uniform=conf[1], nsteps=600, trace_every=100,
               traces=("axon",))["axon"]
    assert len(tr) == 6 and lines[9] == ""
    for k, row in enumerate(tr):
        want = " %d %.2f " % (100 * k + 1, 0.0) + "".join("%d : %.8f " % (c + 1, float(v)) for c, v in enumerate(row))
        assert lines[3 + k] == want


def test_kat_regression_checker_criterion(conf):
    """The reference's own regression check (src/regression_test/regression_checker.c:41-65):
    max relative error <= 1% over the 'standard' 500 ms, against stable_version.c's
    golden; plus identical spike steps over the 'full' 2000 ms."""
    n, rp, col, g, gcal = kat_topology()
    z = golden("kat_stable_version.npz")
    st = O.default_state(n, conf)
    st[O.S["g_CaL"]] = gcal
    steps = int(z["n_steps"])
    tr = O.run(n, conf[:23], st, rp, col, g=g, nsteps=steps, trace_every=1, traces=("axon",))["axon"]
    base = z["v_axon_first10000"]
    assert np.max(np.abs(tr[:10000] - base) / np.abs(base)) <= 0.01
    sp = spike_steps(tr)
    for c in range(n):
        assert np.array_equal(sp[c], z[f"spikes_{c}"])


def test_fp64_twin_close_to_fp32(conf):
    n, rp, col, g, gcal = kat_topology()
    st32 = O.default_state(n, conf)
    st32[O.S["g_CaL"]] = gcal
    st64 = st32.astype(np.float64)
    a = O.run(n, conf[:23], st32, rp, col, g=g, nsteps=2000, trace_every=1, traces=("soma",))["soma"]
    b = O.run(n, conf[:23].astype(np.float64), st64, rp, col, g=g, nsteps=2000, trace_every=1,
              traces=("soma",), fp64=True)["soma"]
    assert np.max(np.abs(a - b)) < 1e-3


def test_removable_singularities_take_their_limits():
    """V_dend = -8.5, V_soma = -25 and V_axon = -25 make three rate
    expressions 0/0 in the reference's arithmetic (src/openmp/infoli.c:574,
    :627, :656); one such cell would turn the whole network to NaN through the
    coupling.  The oracle (and the GPU path) use the limits there."""
    conf = O.read_parameters(CONF)
    n = 3
    st = O.default_state(n, conf)
    st[O.S["V_dend"]] = [-8.5, -60.0, -8.5]
    st[O.S["V_soma"]] = [-25.0, -25.0, -60.0]
    st[O.S["V_axon"]] = [-25.0, -60.0, -25.0]
    rp = np.array([0, 1, 2, 3], dtype=np.int64)
    col = np.array([1, 2, 0], dtype=np.int32)
    # one step: the crafted states are far from equilibrium (later steps
    # would run away for that reason alone)
    O.run(n, conf[:23], st, rp, col, g_uniform=0.04, nsteps=1, trace_every=0, traces=())
    assert np.isfinite(st).all()
    s64 = O.default_state(n, conf).astype(np.float64)
    s64[O.S["V_soma"]] = -25.0
    s64[O.S["V_axon"]] = -25.0
    s64[O.S["V_dend"]] = -8.5
    O.run(n, conf[:23].astype(np.float64), s64, rp, col, g_uniform=0.04, nsteps=1, trace_every=0, traces=(),
          fp64=True)
    assert np.isfinite(s64).all()


def _dense_to_csr(G):
    """Conductance matrix, row = sender, column = receiver (the single-threaded
    reference reads neighId = row index; a zero means no connection)."""
    n = G.shape[0]
    rp, col, g = [0], [], []
    for r in range(n):
        for s in range(n):
            if G[s, r] != 0:
                col.append(s)
                g.append(G[s, r])
        rp.append(len(col))
    return np.array(rp, np.int64), np.array(col, np.int32), np.array(g, np.float32)


@pytest.mark.parametrize("tag", ["coupled10", "isolated64"])
def test_random_init_vs_reference_single_threaded(conf, tag):
    """Randomised initial states (RAND_INIT) against the reference's own
    single-threaded build with the switch at 1 (src/single_threaded/
    infoli.c:206-236, seed 1): the oracle's draws and isolated steps, then 200
    FP64 steps, follow the reference's V_axon to within the FP32 rounding of the
    isolated steps.  The reference starts its simulation from the state after
    k - 1 of the k isolated steps it draws (the last one lands in the buffer the
    simulation does not read first); with k steps the trajectories differ by
    about 5e-2 mV, so the tolerance separates the two by two orders of
    magnitude."""
    z = golden("single_rand_init.npz")
    G, ref = z[f"cond_sender_by_receiver_{tag}"], z[f"v_axon_{tag}"]
    n = G.shape[0]
    rp, col, g = _dense_to_csr(G)
    st = O.default_state(n, conf)
    ks = O.random_init(n, conf, st, int(z["seed"]))
    assert np.all(ks % 2 == 1) and np.all(ks < 2000)
    st64 = st.astype(np.float64)
    got = O.run(n, conf[:23].astype(np.float64), st64, rp, col, g=g, nsteps=200, trace_every=1,
                traces=("axon",), fp64=True)["axon"]
    assert got.shape == ref.shape
    assert np.max(np.abs(got - ref)) < 5e-4


def _conf_f64():
    """default.conf parsed as doubles: the same decimals as the single-threaded
    reference's constants and initial state (src/single_threaded/infoli.h:33-66,
    infoli.c:862-889)."""
    vals = np.array([float(l.split("=")[1]) for l in open(CONF) if "=" in l], dtype=np.float64)
    assert vals.shape == (42,)
    return vals


@pytest.mark.parametrize("tag", ["coupled10", "isolated64"])
def test_fp64_twin_vs_reference_single_threaded(built, tag):
    """The FP64 twin (the FP64 oracle that every accuracy figure of the bench
    is quoted against) on the single-threaded reference's own FP64 run: its
    randomised initial state in double, then 200 steps, V_axon every step.  The
    reference prints 8 decimals (5e-9 mV of rounding); the oracle takes the
    conductances as float32 (the reference reads them as double)."""
    z = golden("single_rand_init.npz")
    G, ref = z[f"cond_sender_by_receiver_{tag}"], z[f"v_axon_{tag}"]
    n = G.shape[0]
    rp, col, g = _dense_to_csr(G)
    vals = _conf_f64()
    st = np.empty((19, n), dtype=np.float64)
    st[:] = vals[23:42, None]
    O.random_init(n, vals[:23], st, int(z["seed"]))
    got = O.run(n, vals[:23], st, rp, col, g=g, nsteps=200, trace_every=1, traces=("axon",), fp64=True)["axon"]
    assert np.max(np.abs(got - ref)) < 5e-8


def test_fp64_twin_stimulus_file_vs_reference_single_threaded(built):
    """The single-threaded reference in its input-file mode (one line of
    per-cell currents per step, V_axon printed with 16 decimals) on 16 cells
    whose conductances are exact in binary, after its randomised initial
    state: the FP64 oracle follows it through the spikes (V_axon up to 48 mV)
    to 1e-11 mV over 400 steps.  This pins the stimulus table's step alignment
    (row t drives step t; a shift by one step gives 34 mV), the randomised
    state and the FP64 cell update together."""
    z = golden("single_rand_init.npz")
    G, ref, tab = z["cond_sender_by_receiver_stim16"], z["v_axon_stim16"], z["stim_stim16"]
    n = G.shape[0]
    rp, col, g = _dense_to_csr(G)
    vals = _conf_f64()
    st = np.empty((19, n), dtype=np.float64)
    st[:] = vals[23:42, None]
    O.random_init(n, vals[:23], st, int(z["seed"]))
    got = O.run(n, vals[:23], st, rp, col, g=g, stim=("table", tab, 0), nsteps=tab.shape[0], trace_every=1,
                traces=("axon",), fp64=True)["axon"]
    assert ref.max() > 30.0  # the pulses make cells spike
    assert np.max(np.abs(got - ref)) < 1e-9
