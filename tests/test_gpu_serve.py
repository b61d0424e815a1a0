"""Serving loop (infoli_server_*): many simulations admitted by device-memory
budget and run side by side.  A request's result must be the same alone and
in a mix (bit for bit: its path, plan and launches depend only on itself),
agree with the oracle within the path's tolerance, and the admission rules
must hold: concurrent requests overlap on the device, a tight budget
serialises them, a request larger than the budget is refused.  Each rule is
checked on both paths: the lane (small requests relaunched together through
the batched cluster kernel, joining between launches) and the persistent
per-request launches (the lane switched off).  Requests submitted while
others are on the GPU join them and still give their alone results.
"""
import time

import numpy as np
import pytest

from helpers import CONF, TOL_VSOMA_MV, hetero_state
from oracle import oracle as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ig(built):
    import infoli_gb300

    assert infoli_gb300.device_count() >= 1
    return infoli_gb300


@pytest.fixture(scope="module")
def conf(built):
    return O.read_parameters(CONF)


# (cells, density, steps, seed)
MIX = [(400, 0.2, 1500, 1), (2500, 0.05, 800, 2), (900, 0.3, 1200, 3), (6000, 0.02, 600, 4),
       (1500, 0.1, 1000, 5), (300, 0.5, 2000, 6)]


def _requests(ig, conf):
    reqs = []
    for n, p, steps, seed in MIX:
        rp, col = ig.gen_uniform(n, p, seed)
        reqs.append(dict(n=n, row_ptr=rp, col=col, n_steps=steps, init_state=hetero_state(conf, n, seed),
                         pulse=(200, 400, 3.0), g_uniform=0.04))
    return reqs


def _serve(ig, conf, reqs, **kw):
    with ig.Server(conf, **kw) as sv:
        ids = [sv.submit(**r) for r in reqs]
        return [sv.wait(i) for i in ids]


# the lane forced for every request of the mix (by default only light ones take it)
PATHS = {"lane": {"lane_edges_per_cta": -1}, "persistent": {"lane_sms": -1}}


@pytest.mark.parametrize("path", list(PATHS))
def test_alone_equals_mixed_and_oracle(ig, conf, path):
    kw = PATHS[path]
    reqs = _requests(ig, conf)
    mixed = _serve(ig, conf, reqs, **kw)
    assert all(info["lane"] == (path == "lane") for _, info in mixed)
    for k in (0, 2, 5):
        alone = _serve(ig, conf, [reqs[k]], **kw)[0]
        assert np.array_equal(alone[0], mixed[k][0]), k
    # oracle (float build) for the small ones
    for k in (0, 5):
        r = reqs[k]
        st = r["init_state"].copy()
        O.run(r["n"], conf[:23], st, r["row_ptr"], r["col"], g_uniform=0.04,
              stim=("pulse",) + tuple(r["pulse"]), nsteps=r["n_steps"], trace_every=0, traces=(),
              nthreads=O.max_threads())
        assert np.max(np.abs(mixed[k][0][O.S["V_soma"]] - st[O.S["V_soma"]])) <= TOL_VSOMA_MV
    for _, info in mixed:
        assert info["status"] == 0
        assert info["submit_s"] <= info["admit_s"] <= info["start_s"] <= info["done_s"]


@pytest.mark.parametrize("path", list(PATHS))
def test_requests_overlap_on_the_device(ig, conf, path):
    reqs = _requests(ig, conf)
    out = _serve(ig, conf, reqs, **PATHS[path])
    iv = [(i["start_s"], i["done_s"]) for _, i in out]
    overlaps = sum(1 for a in range(len(iv)) for b in range(a + 1, len(iv))
                   if iv[a][0] < iv[b][1] and iv[b][0] < iv[a][1])
    assert overlaps >= 1
    assert sum(i["grid"] for _, i in out) <= 152 * len(out)


@pytest.mark.parametrize("path", list(PATHS))
def test_budget_serialises_and_refuses(ig, conf, path):
    """Three requests of one size under a budget that holds one admission
    reservation plus half of one prepared request: admissions never overlap."""
    kw = PATHS[path]
    n, p, steps = 2000, 0.1, 600
    rp, col = ig.gen_uniform(n, p, 9)
    reqs = [dict(n=n, row_ptr=rp, col=col, n_steps=steps, init_state=hetero_state(conf, n, 20 + k),
                 g_uniform=0.04) for k in range(3)]
    first = _serve(ig, conf, reqs, **kw)
    est = first[0][1]["admitted_bytes"]
    held = first[0][1]["device_bytes"]
    assert 0 < held <= est
    out = _serve(ig, conf, reqs, hbm_budget=est + held // 2, **kw)
    iv = sorted((i["admit_s"], i["done_s"]) for _, i in out)
    for (a0, a1), (b0, b1) in zip(iv, iv[1:]):
        assert b0 >= a1 - 1e-6  # the next one is admitted only after the previous one is done
    for (s0, _), (s1, _) in zip(first, out):
        assert np.array_equal(s0, s1)
    with ig.Server(conf, hbm_budget=1 << 20) as sv:
        with pytest.raises(ig.InfoliError):
            sv.submit(**reqs[0])


def test_requests_join_while_others_run(ig, conf):
    """Continuous admission: a long small request A (lane) and a large request
    P (its own persistent launch: per-edge conductances) start first; small
    requests B and C are submitted while both are on the GPU.  B and C join
    the lane at its next launch, finish while A and P still run, and every
    result is bit-for-bit its result alone and within tolerance of the
    oracle."""
    def small(n, p, steps, seed):
        rp, col = ig.gen_uniform(n, p, seed)
        return dict(n=n, row_ptr=rp, col=col, n_steps=steps, init_state=hetero_state(conf, n, seed),
                    pulse=(100, 300, 3.0), g_uniform=0.04)

    a = small(3000, 0.05, 100000, 41)
    n_p = 12000
    rp_p, col_p, g_p = ig.gen_fixed_degree(n_p, 40, 42, (0.02, 0.06))
    big = dict(n=n_p, row_ptr=rp_p, col=col_p, g=g_p, n_steps=60000, init_state=hetero_state(conf, n_p, 42),
               pulse=(100, 300, 3.0))
    b, c = small(700, 0.2, 600, 43), small(1200, 0.1, 900, 44)
    with ig.Server(conf, lane_chunk_steps=500, lane_edges_per_cta=-1) as sv:
        ia, ip = sv.submit(**a), sv.submit(**big)
        time.sleep(0.05)
        assert sv.poll(ia) == 1 and sv.poll(ip) == 1  # both admitted and on their way
        t_join = time.perf_counter()
        ib, ic = sv.submit(**b), sv.submit(**c)
        rb, rc_, ra, rp = sv.wait(ib), sv.wait(ic), sv.wait(ia), sv.wait(ip)
        wall = time.perf_counter() - t_join
    ib_, ic_, ia_, ip_ = rb[1], rc_[1], ra[1], rp[1]
    assert ia_["lane"] == 1 and ib_["lane"] == 1 and ic_["lane"] == 1 and ip_["lane"] == 0
    # B and C started after A was already running, and finished before A and P
    assert ib_["start_s"] > ia_["start_s"] and ic_["start_s"] > ia_["start_s"]
    assert max(ib_["done_s"], ic_["done_s"]) < min(ia_["done_s"], ip_["done_s"])
    assert ib_["start_s"] < ip_["done_s"]  # they ran while P was on the GPU
    assert ia_["lane_launches"] >= 100000 // 500 and ib_["lane_launches"] >= 2
    assert wall > 0
    for req, got in ((a, ra), (b, rb), (c, rc_), (big, rp)):
        alone = _serve(ig, conf, [req], lane_chunk_steps=500, lane_edges_per_cta=-1)[0]
        assert np.array_equal(alone[0], got[0]), req["n"]
    for req, got in ((b, rb), (c, rc_)):
        st = req["init_state"].copy()
        O.run(req["n"], conf[:23], st, req["row_ptr"], req["col"], g_uniform=0.04,
              stim=("pulse",) + tuple(req["pulse"]), nsteps=req["n_steps"], trace_every=0, traces=(),
              nthreads=O.max_threads())
        assert np.max(np.abs(got[0][O.S["V_soma"]] - st[O.S["V_soma"]])) <= TOL_VSOMA_MV


def test_lane_join_interval_does_not_change_results(ig, conf):
    """A lane request relaunched every 300 or every 5,000 steps ends in the
    same state (launch boundaries carry the whole state, Ca2+ in FP64)."""
    rp, col = ig.gen_uniform(1500, 0.1, 51)
    req = dict(n=1500, row_ptr=rp, col=col, n_steps=2100, init_state=hetero_state(conf, 1500, 51),
               pulse=(200, 500, 3.0), g_uniform=0.04)
    short = _serve(ig, conf, [req], lane_chunk_steps=300, lane_edges_per_cta=-1)[0]
    long_ = _serve(ig, conf, [req], lane_chunk_steps=5000, lane_edges_per_cta=-1)[0]
    assert short[1]["lane_launches"] == 7 and long_[1]["lane_launches"] == 1
    assert np.array_equal(short[0], long_[0])


def test_lane_takes_only_light_requests_by_default(ig, conf):
    """Default eligibility: a sparse small request takes the lane, a dense one
    of the same size its own persistent launch (decided from the request
    alone), each with its alone result."""
    def req(p, seed):
        rp, col = ig.gen_uniform(2000, p, seed)
        return dict(n=2000, row_ptr=rp, col=col, n_steps=400, init_state=hetero_state(conf, 2000, seed),
                    g_uniform=0.04)

    light, dense = req(0.005, 61), req(0.2, 62)  # ~10 and ~400 senders per cell
    out = _serve(ig, conf, [light, dense])
    assert out[0][1]["lane"] == 1 and out[1][1]["lane"] == 0
    assert np.array_equal(out[0][0], _serve(ig, conf, [light])[0][0])
    assert np.array_equal(out[1][0], _serve(ig, conf, [dense])[0][0])
