"""The work planner, checked on the CPU: every plan the step kernel would run
is walked with the kernel's addressing (infoli_plan_emulate) and must give the
gap-junction currents of the CSR network, for both V_dend exchange modes."""
import numpy as np
import pytest

from helpers import kat_topology


@pytest.fixture(scope="module")
def capi(built):
    from infoli_gb300 import capi

    return capi


def direct_ic(n, rp, col, v, g=None, g_uniform=0.04):
    v = v.astype(np.float64)
    out = np.zeros(n)
    for r in range(n):
        s = col[rp[r]:rp[r + 1]]
        V = v[r] - v[s]
        w = g[rp[r]:rp[r + 1]].astype(np.float64) if g is not None else g_uniform
        out[r] = np.sum(w * (0.8 * np.exp(-V * V / 100) + 0.2) * V)
    return out


def check(capi, n, rp, col, g=None, sync_mode=0, seed=0, **kw):
    rng = np.random.default_rng(seed)
    v = (-60 + rng.uniform(-15, 15, n)).astype(np.float32)
    ic, info = capi.plan_emulate(n, rp, col, v, g=g, sync_mode=sync_mode, **kw)
    ref = direct_ic(n, rp, col, v, g)
    scale = np.maximum(1.0, np.abs(ref))
    assert np.max(np.abs(ic - ref) / scale) < 2e-4, info
    return info


@pytest.mark.parametrize("mode", [1, 2])
def test_kat_network(capi, mode):
    n, rp, col, g, _ = kat_topology()
    info = check(capi, n, rp, col, g=g, sync_mode=mode)
    assert info["stamped"] == (mode == 2)


@pytest.mark.parametrize("mode", [1, 2])
@pytest.mark.parametrize("n,p", [(1, 0.5), (33, 1.0), (1000, 0.1), (3000, 0.02)])
def test_reference_generator_networks(capi, n, p, mode):
    rp, col = capi.gen_uniform(n, p, 1)
    info = check(capi, n, rp, col, sync_mode=mode)
    assert info["ctas"] >= 1


@pytest.mark.parametrize("n,p,ctas", [(500, 0.1, 50), (1000, 0.1, 100), (2000, 0.02, 100), (2000, 0.1, 100),
                                      (64, 0.5, 7)])
def test_small_networks_get_the_grid_floor(capi, n, p, ctas):
    """Small networks get at least min(n / 10, 100) CTAs (the chunk count
    alone gave 1,000 cells at p = 0.1 25 CTAs: 2.53 against 1.95 us per step
    with 100), and their plans still give the network's currents."""
    rp, col = capi.gen_uniform(n, p, 1)
    info = check(capi, n, rp, col, threads=512)
    assert info["ctas"] == ctas and info["stamped"] == 1


def test_grid_network_10k_stamped(capi):
    rp, col = capi.gen_grid_gaussian(100, 100, 10.0, 18.0, 1)
    info = check(capi, 10000, rp, col, sync_mode=0)
    assert info["stamped"] == 1 and info["resident"] == 1 and info["ctas"] == 152


def test_grid_network_barrier_and_small_grids(capi):
    rp, col = capi.gen_grid_gaussian(40, 50, 6.0, 10.0, 3)
    for grid in (2, 7, 64):
        check(capi, 2000, rp, col, sync_mode=1, grid=grid)
        check(capi, 2000, rp, col, sync_mode=0 if grid < 7 else 2, grid=grid)


def test_per_edge_g_stamped_and_barrier(capi):
    rp, col, g = capi.gen_fixed_degree(5000, 40, 3, (0.02, 0.06))
    a = check(capi, 5000, rp, col, g=g, sync_mode=2)
    b = check(capi, 5000, rp, col, g=g, sync_mode=1)
    assert a["stamped"] == 1 and b["stamped"] == 0


def test_large_window_sparse_rows_gather_else_barrier_tiles(capi):
    rp, col, g = capi.gen_fixed_degree(90000, 6, 12, (0.02, 0.06))
    info = check(capi, 90000, rp, col, g=g)
    assert info["stamped"] == 3  # auto: short rows over a large window: tiled gather
    info = check(capi, 90000, rp, col, g=g, sync_mode=1)
    assert info["stamped"] == 0 and info["tiles"] > info["ctas"]


@pytest.mark.parametrize("mode,code", [(3, 2), (4, 3)])
def test_gather_plans(capi, mode, code):
    # ragged rows (uniform generator), per-edge g, empty rows, several grids
    rp, col = capi.gen_uniform(3000, 0.02, 5)
    for grid in (1, 5, 152):
        info = check(capi, 3000, rp, col, sync_mode=mode, grid=grid)
        assert info["stamped"] == code and (mode == 4 or info["smem_bytes"] == 0)
    rp, col, g = capi.gen_fixed_degree(4000, 25, 6, (0.02, 0.06))
    check(capi, 4000, rp, col, g=g, sync_mode=mode)
    n = 500
    rp, col = capi.gen_uniform(n, 0.05, 7)
    keep = np.ones(col.size, bool)
    keep[: rp[200]] = False
    rp2 = np.concatenate([[0] * 201, rp[201:] - rp[200]]).astype(np.int64)
    check(capi, n, rp2, col[keep], sync_mode=mode)


def test_tiled_gather_many_tiles_and_small_budget(capi):
    # a window of 90,000 floats: two buffers and several tiles per CTA; then a
    # small budget forcing many small tiles
    rp, col, g = capi.gen_fixed_degree(90000, 6, 12, (0.02, 0.06))
    info = check(capi, 90000, rp, col, g=g, sync_mode=4)
    assert info["tiles"] > 2 * info["ctas"]
    rp, col = capi.gen_uniform(2000, 0.05, 8)
    info = check(capi, 2000, rp, col, sync_mode=4, smem_budget=4096)
    assert info["tiles"] > info["ctas"]


def test_isolated_cells_and_empty_rows(capi):
    n = 300
    rp, col = capi.gen_uniform(n, 0.05, 4)
    # drop every edge of the first 100 receivers
    keep = np.ones(col.size, bool)
    keep[: rp[100]] = False
    col2 = col[keep]
    rp2 = np.concatenate([[0] * 101, rp[101:] - rp[100]]).astype(np.int64)
    for mode in (1, 2):
        check(capi, n, rp2, col2, sync_mode=mode)


def test_stamped_request_that_cannot_fit_is_rejected(capi):
    rp, col, g = capi.gen_fixed_degree(90000, 6, 12, (0.02, 0.06))
    with pytest.raises(capi.InfoliError):
        capi.plan_emulate(90000, rp, col, np.zeros(90000, np.float32), g=g, sync_mode=2)


def test_bitmask_plans(capi):
    """Bitmask plans (uniform g): one tile, several tiles (small budget) and
    ragged CTAs; the emulation walks the bit rows with the kernel's layout."""
    rp, col = capi.gen_bitmask_csr(3000, 0.2, 5)
    for grid in (1, 7, 152):
        info = check(capi, 3000, rp, col, sync_mode=5, grid=grid)
        assert info["stamped"] == 4
    info = check(capi, 3000, rp, col, sync_mode=5, smem_budget=8 * 1024)
    assert info["tiles"] > info["ctas"]
    # auto picks it for dense rows over a window larger than shared memory
    rp, col = capi.gen_bitmask_csr(60000, 0.08, 6)
    info = check(capi, 60000, rp, col)
    assert info["stamped"] == 4 and info["tiles"] >= 2 * info["ctas"]
    with pytest.raises(capi.InfoliError):
        capi.plan_emulate(100, *capi.gen_fixed_degree(100, 5, 1, (0.02, 0.06))[:2], np.zeros(100, np.float32),
                          g=np.full(500, 0.04, np.float32), sync_mode=5)


def _windows(rp, col, order, starts):
    """Unique senders of each block of cells order[starts[b]:starts[b+1]]."""
    out = []
    for b in range(len(starts) - 1):
        cells = order[starts[b]:starts[b + 1]]
        idx = np.concatenate([np.arange(rp[c], rp[c + 1]) for c in cells]) if len(cells) else np.zeros(0, int)
        out.append(len(np.unique(col[idx])))
    return np.array(out)


def test_locality_order_compacts_grid_windows(capi):
    """Spectral order + recursive bisection on a 60 x 60 Gaussian grid: a valid
    permutation into 152 blocks of at most 512 cells whose sender windows are
    far narrower than those of contiguous ranges of the caller's order."""
    n, parts = 3600, 152
    rp, col = capi.gen_grid_gaussian(60, 60, 6.0, 11.0, 4)
    rp, col = np.asarray(rp), np.asarray(col)
    order, starts = capi.plan_locality_order(n, rp, col, parts, 512)
    assert np.array_equal(np.sort(order), np.arange(n))
    assert starts[0] == 0 and starts[-1] == n and np.all(np.diff(starts) >= 1) and np.all(np.diff(starts) <= 512)
    w_new = _windows(rp, col, order, starts)
    w_old = _windows(rp, col, np.arange(n), np.linspace(0, n, parts + 1).astype(int))
    assert w_new.max() * 1.5 < w_old.max() and w_new.mean() * 1.5 < w_old.mean()
    assert capi.plan_locality_order(4, rp[:5] * 0, col[:0], 8, 512) is None  # fewer cells than needed


@pytest.mark.parametrize("per_edge_g", [False, True])
def test_relabelled_stamped_plan_emulates_exactly(capi, per_edge_g):
    """The planner relabels a wide-window grid network; the emulated currents,
    reported in the caller's order, match the direct CSR computation."""
    n = 3600
    rp, col = capi.gen_grid_gaussian(60, 60, 6.0, 11.0, 4)
    rp, col = np.asarray(rp), np.asarray(col)
    g = np.random.default_rng(3).uniform(0.02, 0.06, len(col)).astype(np.float32) if per_edge_g else None
    info = check(capi, n, rp, col, g=g, threads=512)
    assert info["stamped"] == 1 and info["relabelled"]


def test_random_graph_keeps_caller_order(capi):
    """No spatial structure: the relabelled plan would not narrow the windows,
    so the plan keeps the caller's cell order."""
    rp, col = capi.gen_uniform(3000, 0.02, 1)
    info = check(capi, 3000, rp, col, threads=512)
    assert info["stamped"] == 1 and not info["relabelled"]
