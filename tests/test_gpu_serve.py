"""Serving loop (infoli_server_*): many simulations admitted by device-memory
budget and run side by side.  A request's result must be the same alone and
in a mix (bit for bit: its plan and launches depend only on itself), agree
with the oracle within the path's tolerance, and the admission rules must
hold: concurrent requests overlap on the device, a tight budget serialises
them, a request larger than the budget is refused.
"""
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


def test_alone_equals_mixed_and_oracle(ig, conf):
    reqs = _requests(ig, conf)
    mixed = _serve(ig, conf, reqs)
    for k in (0, 2, 5):
        alone = _serve(ig, conf, [reqs[k]])[0]
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


def test_requests_overlap_on_the_device(ig, conf):
    reqs = _requests(ig, conf)
    out = _serve(ig, conf, reqs)
    iv = [(i["start_s"], i["done_s"]) for _, i in out]
    overlaps = sum(1 for a in range(len(iv)) for b in range(a + 1, len(iv))
                   if iv[a][0] < iv[b][1] and iv[b][0] < iv[a][1])
    assert overlaps >= 1
    assert sum(i["grid"] for _, i in out) <= 152 * len(out)


def test_budget_serialises_and_refuses(ig, conf):
    """Three requests of one size under a budget that holds one admission
    reservation plus half of one prepared request: admissions never overlap."""
    n, p, steps = 2000, 0.1, 600
    rp, col = ig.gen_uniform(n, p, 9)
    reqs = [dict(n=n, row_ptr=rp, col=col, n_steps=steps, init_state=hetero_state(conf, n, 20 + k),
                 g_uniform=0.04) for k in range(3)]
    first = _serve(ig, conf, reqs)
    est = first[0][1]["admitted_bytes"]
    held = first[0][1]["device_bytes"]
    assert 0 < held <= est
    out = _serve(ig, conf, reqs, hbm_budget=est + held // 2)
    iv = sorted((i["admit_s"], i["done_s"]) for _, i in out)
    for (a0, a1), (b0, b1) in zip(iv, iv[1:]):
        assert b0 >= a1 - 1e-6  # the next one is admitted only after the previous one is done
    for (s0, _), (s1, _) in zip(first, out):
        assert np.array_equal(s0, s1)
    with ig.Server(conf, hbm_budget=1 << 20) as sv:
        with pytest.raises(ig.InfoliError):
            sv.submit(**reqs[0])
