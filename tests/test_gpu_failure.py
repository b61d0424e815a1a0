"""Failure detection without a GPU fault: every device-side wait of the step
kernels is bounded.  A test hook (INFOLI_STALL_CTA) makes one CTA skip its
grid-barrier arrivals and its stamped-word publications, so the other CTAs'
waits run out; the call must return INFOLI_ERR_TIMEOUT within the configured
limit, and the same handle (and the CUDA context) must keep working once the
hook is cleared."""
import time

import numpy as np
import pytest

from helpers import CONF, hetero_state
from oracle import oracle as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ig(built):
    import infoli_gb300

    assert infoli_gb300.device_count() >= 1
    return infoli_gb300


@pytest.mark.parametrize("mode", ["stamped", "barrier", "tgather"])
def test_stalled_cta_times_out_and_recovers(ig, mode, monkeypatch):
    conf = O.read_parameters(CONF)
    monkeypatch.setenv("INFOLI_SYNC", mode)
    monkeypatch.setenv("INFOLI_WAIT_TIMEOUT_MS", "300")
    rp, col = ig.gen_grid_gaussian(40, 50, 6.0, 10.0, 3)
    n = 2000
    st0 = hetero_state(conf, n, 2)
    with ig.Simulation(n, conf, rp, col, init_state=st0) as sim, \
            ig.Simulation(n, conf, rp, col, init_state=st0) as ref:
        assert sim.plan_info()["grid"] > 2
        monkeypatch.setenv("INFOLI_STALL_CTA", "1")
        t0 = time.time()
        with pytest.raises(ig.InfoliError) as e:
            sim.run(50)
        assert e.value.code == ig.capi.ERR_TIMEOUT
        assert time.time() - t0 < 30
        monkeypatch.delenv("INFOLI_STALL_CTA")
        # the context is usable and a fresh state runs normally
        sim.set_state(st0)
        ref_tr = ref.run(200, 1, 2)["soma"]
        assert np.isfinite(ref_tr).all()
        sim2_tr = sim.run(200, 1, 2)["soma"]
        assert np.array_equal(sim2_tr, ref_tr)  # same steps, same inputs: same bits
