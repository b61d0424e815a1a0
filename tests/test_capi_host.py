"""C-ABI host-side behaviour (no GPU needed): the library loads, exports every
symbol include/infoli_gpu.h declares, and its host functions follow the
reference (parameter reader, g_CaL reader, generator, trace text)."""
import ctypes
import os
import re

import numpy as np
import pytest

from helpers import CONF, ROOT
from oracle import oracle as O


@pytest.fixture(scope="module")
def capi(built):
    from infoli_gb300 import capi

    capi.load()
    return capi


def _header_functions():
    text = open(os.path.join(ROOT, "include", "infoli_gpu.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(infoli_[a-z0-9_]+)\s*\(", text)))


def test_library_exports_every_declared_symbol(capi):
    lib = ctypes.CDLL(capi.LIB_PATH)
    declared = _header_functions()
    assert len(declared) >= 20
    for name in declared:
        assert hasattr(lib, name), name
    assert sorted(capi.EXPORTED) == declared


def test_version_and_build_info(capi):
    assert capi.load().infoli_version() == 1
    assert b"sm_103a" in capi.load().infoli_build_info()


def test_read_parameters(capi):
    v = capi.read_parameters(CONF)
    assert np.array_equal(v, O.read_parameters(CONF))


def test_read_parameters_errors(capi, tmp_path):
    with pytest.raises(capi.InfoliError) as e:
        capi.read_parameters(str(tmp_path / "missing.conf"))
    assert e.value.code == capi.ERR_FILE
    bad = tmp_path / "bad.conf"
    bad.write_text("DELTA = 0.05\nCONDUCTANCE = oops\n")
    with pytest.raises(capi.InfoliError) as e:
        capi.read_parameters(str(bad))
    assert e.value.code == capi.ERR_CONFIG and "line 2" in str(e.value)


def test_read_gcal_partial_file_keeps_defaults(capi, tmp_path):
    f = tmp_path / "gcal_file.txt"
    f.write_text("0.68 0.76 0.689")
    g = np.full(5, 0.5, dtype=np.float32)
    assert capi.read_gcal(str(f), g) == 3
    assert np.allclose(g, [0.68, 0.76, 0.689, 0.5, 0.5])


@pytest.mark.parametrize("n,p,seed", [(1, 0.5, 1), (2, 1.0, 3), (57, 0.25, 1), (300, 0.05, 9), (40, 0.0, 2)])
def test_generator_matches_oracle(capi, n, p, seed):
    a = capi.gen_uniform(n, p, seed)
    b = O.gen_uniform(n, np.float32(p), seed)
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])


def test_generator_full_density_is_all_to_all(capi):
    rp, col = capi.gen_uniform(10, 1.0, 123)
    assert rp[-1] == 90
    for r in range(10):
        assert list(col[rp[r]:rp[r + 1]]) == [s for s in range(10) if s != r]


def test_grid_gaussian_generator(capi):
    rp, col = capi.gen_grid_gaussian(30, 40, 5.0, 9.0, 7)
    n = 1200
    assert rp.shape == (n + 1,) and rp[-1] == col.size
    for r in (0, 17, 615, 1199):
        row = col[rp[r]:rp[r + 1]]
        assert np.all(np.diff(row) > 0) and r not in row
        dy = row // 40 - r // 40
        dx = row % 40 - r % 40
        assert np.all(dy * dy + dx * dx <= 81)
    again = capi.gen_grid_gaussian(30, 40, 5.0, 9.0, 7)
    assert np.array_equal(again[1], col)


def test_fixed_degree_generator(capi):
    rp, col, g = capi.gen_fixed_degree(500, 20, 11, (0.02, 0.06))
    assert np.all(np.diff(rp) == 20)
    for r in range(500):
        row = col[rp[r]:rp[r + 1]]
        assert np.all(np.diff(row) > 0) and r not in row
    assert g.min() >= 0.02 and g.max() < 0.06


def test_bitmask_round_trip(capi):
    rp, col = capi.gen_uniform(70, 0.3, 5)
    words = (70 + 31) // 32
    bits = np.zeros((70, words), dtype=np.uint32)
    for r in range(70):
        for s in col[rp[r]:rp[r + 1]]:
            bits[r, s // 32] |= np.uint32(1 << (s % 32))
    rp2, col2 = capi.bitmask_to_csr(70, bits)
    assert np.array_equal(rp, rp2) and np.array_equal(col, col2)


def test_format_f8_matches_printf(capi):
    rng = np.random.default_rng(0)
    vals = np.concatenate([
        rng.normal(-60, 25, 20000).astype(np.float32),
        rng.uniform(-1e-7, 1e-7, 2000).astype(np.float32),
        np.array([0.0, -0.0, 5e-9, -5e-9, 1.5e-8, 2.5e-8, 1e30, -3e9, np.inf, -np.inf], dtype=np.float32),
        rng.integers(0, 2**32, 20000, dtype=np.uint64).astype(np.uint32).view(np.float32),
    ])
    libc = ctypes.CDLL(None)
    buf = ctypes.create_string_buffer(512)
    for v in vals:
        libc.snprintf(buf, 512, b"%.8f", ctypes.c_double(float(v)))
        assert capi.format_f8(v) == buf.value.decode(), repr(v)


@pytest.mark.parametrize("tagged", [True, False])
def test_format_row_matches_reference_text(capi, tagged):
    v = np.random.default_rng(1).normal(-60, 10, 9000).astype(np.float32)
    want = "".join(("%d : %.8f " % (i + 1, float(x))) if tagged else ("%.8f " % float(x)) for i, x in enumerate(v))
    assert capi.format_row(v, tagged) == want + "\n"
    assert capi.format_row(v[:7], tagged, 1) == want[: len(capi.format_row(v[:7], tagged, 1)) - 1] + "\n"


def test_sim_create_rejects_bad_arguments_without_crashing(capi):
    conf = capi.read_parameters(CONF)
    rp = np.array([0, 1, 2], dtype=np.int64)
    col = np.array([1, 5], dtype=np.int32)  # sender 5 out of range for 2 cells
    with pytest.raises(capi.InfoliError) as e:
        capi.Simulation(2, conf, rp, col, init_values=conf[23:])
    # on a machine without a GPU the device check fails first
    assert e.value.code in (capi.ERR_ARG, capi.ERR_CUDA)


def test_bitmask_generator_csr_form_matches(built):
    from infoli_gb300 import capi

    for n, p, seed in [(100, 0.1, 3), (777, 0.3, 5), (33, 1.0, 1), (64, 0.0, 2)]:
        bits = capi.gen_bitmask(n, p, seed)
        rp, col = capi.bitmask_to_csr(n, bits)
        rp2, col2 = capi.gen_bitmask_csr(n, p, seed)
        assert np.array_equal(rp, rp2) and np.array_equal(col, col2)
        assert not any(r in col[rp[r]:rp[r + 1]] for r in range(n))  # no self edges
        if n > 100:
            assert abs(len(col) / (n * (n - 1)) - p) < 0.01


def _tune_sample_py(sizes, max_sample, target):
    """The batch autotuner's sample, restated: sizes sorted (stable), m evenly
    spaced picks (2k + 1) N / (2m), m the smallest count reaching target."""
    n = len(sizes)
    order = sorted(range(n), key=lambda i: sizes[i])
    cap = min(max_sample if max_sample > 0 else 4096, n)
    for m in range(1, cap + 1):
        pick = [order[(2 * k + 1) * n // (2 * m)] for k in range(m)]
        if sum(sizes[i] for i in pick) >= target:
            break
    return sorted(pick)


def test_batch_tune_sample_is_stratified(capi):
    rng = np.random.default_rng(3)
    sizes = np.exp(rng.uniform(np.log(256), np.log(8192), 512)).astype(np.int32)
    target = 2 * 152 * 1024
    idx = capi.batch_tune_sample(sizes, target_cells=target)
    assert list(idx) == _tune_sample_py(list(sizes), 0, target)
    assert np.all(np.diff(idx) > 0) and idx[0] >= 0 and idx[-1] < sizes.size
    assert sizes[idx].sum() >= target
    # the sample spans the size range
    assert sizes[idx].min() <= np.quantile(sizes, 0.1) and sizes[idx].max() >= np.quantile(sizes, 0.9)
    # a target no sample reaches takes every network; a zero target the median one
    assert list(capi.batch_tune_sample(sizes, target_cells=1 << 40)) == list(range(sizes.size))
    one = capi.batch_tune_sample(sizes, target_cells=0)
    assert len(one) == 1 and sizes[one[0]] == np.sort(sizes, kind="stable")[sizes.size // 2]
    capped = capi.batch_tune_sample(sizes, max_sample=10, target_cells=1 << 40)
    assert list(capped) == _tune_sample_py(list(sizes), 10, 1 << 40) and len(capped) == 10
    # many small networks: the default cap bounds the sample (and the search)
    tiny = np.full(100000, 3, dtype=np.int32)
    assert len(capi.batch_tune_sample(tiny, target_cells=target)) == 4096
    mixed = np.concatenate([tiny, [8192]]).astype(np.int32)
    assert list(capi.batch_tune_sample(mixed, max_sample=300, target_cells=target)) == \
        _tune_sample_py(list(mixed), 300, target)


def test_batch_shape_arguments_rejected_without_crashing(capi):
    conf = capi.read_parameters(CONF)
    bits = capi.gen_bitmask(100, 0.1, 1)
    iv = np.ascontiguousarray(conf[23:], dtype=np.float32)
    with pytest.raises(capi.InfoliError) as e:
        capi.Batch(conf, [(100, bits, 0.04)], init_values=iv, shape=7)
    assert e.value.code == capi.ERR_ARG
    with pytest.raises(capi.InfoliError) as e:
        capi.Batch(conf, [(100, bits, 0.04)], init_values=iv, shape="auto", tune_steps=0)
    assert e.value.code == capi.ERR_ARG
    big = np.zeros((9000, 282), np.uint32)
    with pytest.raises(capi.InfoliError) as e:
        capi.Batch(conf, [(9000, big, 0.04)], init_values=iv, shape="auto")
    assert e.value.code == capi.ERR_ARG
    # the row-residency policy is FIT, OCC or NONE
    for bad in (-1, 3):
        with pytest.raises(capi.InfoliError) as e:
            capi.Batch(conf, [(100, bits, 0.04)], init_values=iv, shape=1024, residency=bad)
        assert e.value.code == capi.ERR_ARG
