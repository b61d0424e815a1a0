"""Batched path (infoli_batch_*: many independent networks in one clustered
launch) against the CPU oracle, network by network.

Each network of a batch must evolve exactly as the same network simulated on
its own: max |dV_soma| <= 1e-3 mV against the oracle's float build over the
first 2000 steps, spike steps equal within one step; the FP64 oracle gives
the reported precision of the compensated (Kahan) sums.
"""
import os

import numpy as np
import pytest

from helpers import CONF, TOL_VSOMA_MV, hetero_state, spike_steps, spikes_match
from oracle import oracle as O

pytestmark = pytest.mark.gpu

# sizes cover single-CTA networks, partial CTAs and networks over 2 to 5 CTAs
SIZES = [256, 300, 777, 1024, 1100, 2100, 4500]
DENS = [0.5, 0.05, 0.3, 0.2, 0.45, 0.12, 0.06]
GS = [0.04, 0.02, 0.06, 0.035, 0.05, 0.045, 0.025]


@pytest.fixture(scope="module")
def ig(built):
    import infoli_gb300

    assert infoli_gb300.device_count() >= 1
    return infoli_gb300


@pytest.fixture(scope="module")
def conf(built):
    return O.read_parameters(CONF)


def _batch_inputs(ig, conf, sizes, dens, gs, seed0=1):
    nets, states, csr = [], [], []
    for b, (n, p, g) in enumerate(zip(sizes, dens, gs)):
        bits = ig.gen_bitmask(n, p, seed0 + b)
        nets.append((n, bits, g))
        states.append(hetero_state(conf, n, 100 + b))
        csr.append(ig.bitmask_to_csr(n, bits))
    return nets, np.concatenate(states, axis=1), states, csr


def _oracle(conf, n, st, rp, col, g, steps, fp64=False, stim=None, traces=("soma",), every=0):
    s = st.astype(np.float64 if fp64 else np.float32).copy()
    out = O.run(n, conf[:23], s, rp, col, g_uniform=g, stim=stim, nsteps=steps, trace_every=every,
                traces=traces, nthreads=O.max_threads(), fp64=fp64)
    return s, out


@pytest.mark.parametrize("shape", ["1024x8", "512x16"])
def test_batch_each_network_matches_oracle(ig, conf, shape, monkeypatch):
    if shape == "512x16":
        monkeypatch.setenv("INFOLI_BATCH_SHAPE", "512")
    nets, st0, states, csr = _batch_inputs(ig, conf, SIZES, DENS, GS)
    steps = 1000
    with ig.Batch(conf, nets, init_state=st0) as bt:
        info = bt.info()
        assert info["block"] == int(shape.split("x")[0])
        bt.run(steps)
        got = bt.get_state()
        for i, (n, _, g) in enumerate(nets):
            ref, _ = _oracle(conf, n, states[i], *csr[i], g, steps)
            mine = bt.net_state(got, i)
            dvs = np.max(np.abs(mine[O.S["V_soma"]] - ref[O.S["V_soma"]]))
            dvd = np.max(np.abs(mine[O.S["V_dend"]] - ref[O.S["V_dend"]]))
            assert dvs <= TOL_VSOMA_MV, (i, n, dvs)
            assert dvd <= TOL_VSOMA_MV, (i, n, dvd)
            assert np.allclose(mine[O.S["Ca2Plus"]], ref[O.S["Ca2Plus"]], rtol=1e-5, atol=1e-7)


def test_batch_split_runs_equal_one_run(ig, conf):
    """Two launches of 300 + 700 steps give the state of one 1000-step launch
    (FP64 Ca2+ is carried between launches, the step index advances)."""
    nets, st0, _, _ = _batch_inputs(ig, conf, SIZES[:5], DENS[:5], GS[:5], seed0=7)
    with ig.Batch(conf, nets, init_state=st0) as a, ig.Batch(conf, nets, init_state=st0) as b:
        a.set_stimulus_pulse(500, 700, 2.0)
        b.set_stimulus_pulse(500, 700, 2.0)
        a.run(1000)
        b.run(300)
        b.run(700)
        assert np.array_equal(a.get_state(), b.get_state())


def test_batch_kahan_vs_fp64_oracle(ig, conf, capsys):
    """Compensated sums, subthreshold: within 1e-3 mV of the float oracle and
    of the FP64 oracle over the first 2000 steps (sampled every 100 steps)."""
    sizes, dens, gs = [600, 2500, 1300], [0.4, 0.1, 0.25], [0.04, 0.05, 0.03]
    nets, st0, states, csr = _batch_inputs(ig, conf, sizes, dens, gs, seed0=11)
    steps = 2000
    with ig.Batch(conf, nets, init_state=st0, kahan=True) as bt:
        soma = []
        for _ in range(steps // 100):
            bt.run(100)
            soma.append(bt.get_state()[O.S["V_soma"]].copy())
        soma = np.stack(soma)
    rows = np.arange(99, steps, 100)  # oracle row t = state after step t
    for i, (n, _, g) in enumerate(nets):
        _, r64 = _oracle(conf, n, states[i], *csr[i], g, steps, fp64=True, every=1)
        _, r32 = _oracle(conf, n, states[i], *csr[i], g, steps, fp64=False, every=1)
        mine = soma[:, bt.offsets[i]:bt.offsets[i + 1]]
        e32 = np.max(np.abs(mine - r32["soma"][rows]))
        e64 = np.max(np.abs(mine - r64["soma"][rows]))
        f64 = np.max(np.abs(r32["soma"][rows] - r64["soma"][rows]))
        with capsys.disabled():
            print(f"\n  net {i} n={n}: |dV_soma| vs float oracle {e32:.2e} mV, vs FP64 oracle {e64:.2e} mV "
                  f"(float oracle vs FP64: {f64:.2e})")
        assert e32 <= TOL_VSOMA_MV, (i, e32)
        assert e64 <= TOL_VSOMA_MV, (i, e64, f64)


def test_batch_spike_steps_match_oracle(ig, conf):
    """Soma spike steps within one step of the oracle, with a dendritic pulse;
    the batch is sampled after every step through 1-step launches."""
    sizes, dens, gs = [256, 700, 1500], [0.3, 0.2, 0.1], [0.04, 0.04, 0.04]
    nets, st0, states, csr = _batch_inputs(ig, conf, sizes, dens, gs, seed0=21)
    steps = 1500
    stim = ("pulse", 100, 400, 6.0)
    with ig.Batch(conf, nets, init_state=st0) as bt:
        bt.set_stimulus_pulse(*stim[1:])
        rows = []
        for _ in range(steps):
            bt.run(1)
            rows.append(bt.get_state()[O.S["V_soma"]].copy())
        rows = np.stack(rows)
    for i, (n, _, g) in enumerate(nets):
        _, ref = _oracle(conf, n, states[i], *csr[i], g, steps, stim=stim, every=1)
        mine = rows[:, bt.offsets[i]:bt.offsets[i + 1]]
        sm, sr = spike_steps(mine), spike_steps(ref["soma"])
        assert sum(len(x) for x in sr) > 0
        assert spikes_match(sm, sr)


def test_batch_rejects_bad_input(ig, conf):
    bits = ig.gen_bitmask(100, 0.1, 1)
    with pytest.raises(ig.InfoliError):
        ig.Batch(conf, [(9000, np.zeros((9000, 282), np.uint32), 0.04)],
                 init_values=O.default_state(1, conf)[:, 0])
    with pytest.raises(ig.InfoliError):
        ig.Batch(conf, [(0, bits, 0.04)], init_values=O.default_state(1, conf)[:, 0])


def test_batch_autotune_picks_the_faster_shape(ig, conf):
    """infoli_batch_autotune times every (cells per CTA, row residency)
    candidate on a sample of the networks (on a GB300 every network: they hold
    fewer cells than the sample target); the batch built with its pick equals
    the batch built with that layout explicitly, bit for bit, and the oracle;
    the layout does not change the results."""
    nets, st0, states, csr = _batch_inputs(ig, conf, SIZES, DENS, GS, seed0=31)
    steps = 500
    with ig.Batch(conf, nets, init_state=st0, shape="auto", tune_steps=50) as bt:
        t = bt.tune
        ms = t["ms_per_step"]
        assert set(ms) == {"1024/fit", "1024/none", "512/fit", "512/occupancy", "512/none"}
        assert all(v > 0 for v in ms.values())
        assert t["block"] in (512, 1024)
        # the pick is within the tuner's 2% margin of the fastest candidate
        assert ms[f"{t['block']}/{t['residency']}"] * 0.98 <= min(ms.values())
        import torch

        sms = torch.cuda.get_device_properties(0).multi_processor_count
        expect = ig.batch_tune_sample(SIZES, target_cells=2 * sms * 1024)
        assert t["sample_nets"] == len(expect) and t["sample_cells"] == sum(SIZES[i] for i in expect)
        assert bt.info()["block"] == t["block"]
        bt.run(steps)
        got = bt.get_state()
        offsets = bt.offsets
    res = {"fit": ig.capi.RES_FIT, "occupancy": ig.capi.RES_OCC, "none": ig.capi.RES_NONE}
    with ig.Batch(conf, nets, init_state=st0, shape=t["block"], residency=res[t["residency"]]) as same:
        same.run(steps)
        assert np.array_equal(got, same.get_state())
    # another layout: same arithmetic per network, so the same bits
    other = ig.capi.RES_NONE if t["residency"] != "none" else ig.capi.RES_FIT
    with ig.Batch(conf, nets, init_state=st0, shape=512 if t["block"] == 1024 else 1024,
                  residency=other) as alt:
        alt.run(steps)
        assert np.array_equal(got, alt.get_state())
    for i, (n, _, g) in enumerate(nets):
        ref, _ = _oracle(conf, n, states[i], *csr[i], g, steps)
        dvs = np.max(np.abs(got[O.S["V_soma"], offsets[i]:offsets[i + 1]] - ref[O.S["V_soma"]]))
        assert dvs <= TOL_VSOMA_MV, (i, n, dvs)
