"""infoli_run_noalloc: the allocation-free entry point, for callers that may not
allocate device memory (a fixed device-memory arena, a binding whose allocator
owns all device buffers, loops that cannot take cudaFree's device-wide sync).

It is checked through the C ABI against the regular entry point
(infoli_sim_create / infoli_sim_run) on the same network and state, for two
calls in a row (the second continues from the state the first left), within
the tolerance the parity tests use.  The file sorts last so a run that stops at
the first failure has already run every other test; it also passes alone.
"""
import ctypes as C

import numpy as np
import pytest

from helpers import CONF, TOL_VSOMA_MV, hetero_state

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def env(built):
    import torch

    import infoli_gb300 as ig

    assert ig.device_count() >= 1
    return ig, torch, ig.read_parameters(CONF)


def _dev(torch, a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def _ptr(t):
    return None if t is None else C.c_void_p(t.data_ptr())


@pytest.mark.parametrize("per_edge_g", [False, True])
def test_noalloc_matches_regular_entry_point_two_calls(env, per_edge_g):
    ig, torch, conf = env
    n, steps = 1500, 400
    if per_edge_g:
        rp, col, g = ig.gen_fixed_degree(n, 40, 7, (0.02, 0.06))
    else:
        rp, col = ig.gen_uniform(n, 0.05, 3)
        g = None
    st0 = hetero_state(conf, n, 4)
    params = np.ascontiguousarray(conf[:23], dtype=np.float32)

    # regular entry point: two runs of `steps`
    sim = ig.Simulation(n, conf, rp, col, g=g, init_state=st0)
    sim.set_stimulus_pulse(150, 450, 1.0)  # subthreshold: no spikes to amplify differences
    ref1 = sim.run(steps, 1, ig.TRACE_AXON)["axon"]
    ref2 = sim.run(steps, 1, ig.TRACE_AXON)["axon"]
    ref_state = sim.get_state()
    sim.close()

    # allocation-free entry point on caller-owned device buffers
    d_rp, d_col = _dev(torch, rp), _dev(torch, col)
    d_g = _dev(torch, g) if g is not None else None
    d_state = _dev(torch, st0.reshape(-1))
    d_tr = torch.zeros(steps * n, dtype=torch.float32, device="cuda")
    lib = ig.capi.load()
    got, free_before, free_after = [], None, None
    torch.cuda.synchronize()
    for call in range(2):
        if call == 1:
            # the second call must leave the device's free memory unchanged
            # (the first may still be the library's first use on this device)
            free_before = torch.cuda.mem_get_info()[0]
        rc = lib.infoli_run_noalloc(params.ctypes.data_as(C.c_void_p), n, _ptr(d_rp), _ptr(d_col), _ptr(d_g),
                                    float(conf[1]), 150, 450, 1.0, _ptr(d_state), call * steps, steps,
                                    _ptr(d_tr), None)
        if call == 1:
            free_after = torch.cuda.mem_get_info()[0]
        assert rc == 0, lib.infoli_last_error()
        got.append(d_tr.cpu().numpy().reshape(steps, n).copy())
    state = d_state.cpu().numpy().reshape(19, n)
    assert free_after == free_before, (free_before, free_after)

    d1, d2 = np.max(np.abs(got[0] - ref1)), np.max(np.abs(got[1] - ref2))
    assert d1 <= 10 * TOL_VSOMA_MV and d2 <= 10 * TOL_VSOMA_MV, (d1, d2)
    vs = ig.S["V_soma"]
    ds = np.max(np.abs(state[vs] - ref_state[vs]))
    assert ds <= TOL_VSOMA_MV, ds
    assert np.allclose(state, ref_state, rtol=1e-3, atol=1e-3)


def test_noalloc_rejects_networks_beyond_the_static_limit(env):
    ig, torch, conf = env
    n = 65537
    params = np.ascontiguousarray(conf[:23], dtype=np.float32)
    d_rp = torch.zeros(n + 1, dtype=torch.int64, device="cuda")
    d_state = torch.zeros(19 * n, dtype=torch.float32, device="cuda")
    lib = ig.capi.load()
    rc = lib.infoli_run_noalloc(params.ctypes.data_as(C.c_void_p), n, _ptr(d_rp), None, None, 0.04, 0, 0, 0.0,
                                _ptr(d_state), 0, 1, None, None)
    assert rc == ig.capi.ERR_CAPACITY
    assert b"65536" in lib.infoli_last_error()


def test_noalloc_reports_malformed_topology_then_runs_clean(env):
    """A sender id outside [0, n) and a decreasing row_ptr are caught on the
    device (the bad read is skipped) and returned as INFOLI_ERR_ARG; the next
    call on the same buffers, with the topology repaired, succeeds."""
    ig, torch, conf = env
    n, steps = 64, 20
    rp, col = ig.gen_uniform(n, 0.2, 5)
    st0 = hetero_state(conf, n, 6)
    params = np.ascontiguousarray(conf[:23], dtype=np.float32)
    lib = ig.capi.load()
    d_rp, d_col = _dev(torch, rp), _dev(torch, col)
    d_state = _dev(torch, st0.reshape(-1))

    def call():
        return lib.infoli_run_noalloc(params.ctypes.data_as(C.c_void_p), n, _ptr(d_rp), _ptr(d_col), None,
                                      float(conf[1]), 0, 0, 0.0, _ptr(d_state), 0, steps, None, None)

    bad_col = col.copy()
    bad_col[len(col) // 2] = n
    d_col.copy_(torch.from_numpy(bad_col))
    assert call() == ig.capi.ERR_ARG
    assert b"sender id" in lib.infoli_last_error()

    d_col.copy_(torch.from_numpy(col))
    bad_rp = rp.copy()
    bad_rp[n // 2] = bad_rp[n // 2 + 1] + 1  # row n/2 - 1 grows, row n/2 runs backwards
    d_rp.copy_(torch.from_numpy(bad_rp))
    assert call() == ig.capi.ERR_ARG
    assert b"row_ptr" in lib.infoli_last_error()

    d_rp.copy_(torch.from_numpy(rp))
    d_state.copy_(torch.from_numpy(st0.reshape(-1)))
    assert call() == 0, lib.infoli_last_error()
    assert np.isfinite(d_state.cpu().numpy()).all()
