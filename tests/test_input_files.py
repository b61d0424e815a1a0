"""Connectivity and stimulus file readers (host side, no GPU): the formats of
the reference's older simulator (src/truncated/openmp-oldAPI/infoli.c:262-350)
and stimulus file (src/utils/utils.c:70-122), with the reference's
regression topology as the dense fixture."""
import numpy as np
import pytest

from helpers import golden, kat_topology


@pytest.fixture(scope="module")
def capi(built):
    from infoli_gb300 import capi

    return capi


def test_dense_matrix_reads_the_regression_topology(capi, tmp_path):
    n, rp, col, g, _ = kat_topology()
    G = golden("kat_stable_version.npz")["cond_sender_by_receiver"]
    f = tmp_path / "cellConnections.txt"
    # the writers' format (tools/connectivity/*: "%0.2f " / "%f " per value, a row per sender)
    f.write_text("".join("".join(f"{v:f} " for v in row) + "\n" for row in G))
    rp2, col2, g2 = capi.read_conn_dense(str(f), n)
    assert np.array_equal(rp, rp2) and np.array_equal(col, col2)
    assert np.allclose(g, g2, rtol=1e-6)


def test_dense_matrix_threshold_and_errors(capi, tmp_path):
    f = tmp_path / "m.txt"
    f.write_text("0 0.00000005 0.04\n0.03 0 0\n0 0.5 0\n")
    rp, col, g = capi.read_conn_dense(str(f), 3)
    # receiver 0 <- sender 1 (0.03); receiver 1 <- sender 2 (0.5; 5e-8 is below 1e-7); receiver 2 <- sender 0
    assert rp.tolist() == [0, 1, 2, 3] and col.tolist() == [1, 2, 0]
    assert np.allclose(g, [0.03, 0.5, 0.04])
    f.write_text("0 1\n1 0\n")
    with pytest.raises(capi.InfoliError) as e:
        capi.read_conn_dense(str(f), 3)
    assert e.value.code == capi.ERR_CONFIG
    with pytest.raises(capi.InfoliError) as e:
        capi.read_conn_dense(str(tmp_path / "missing.txt"), 3)
    assert e.value.code == capi.ERR_FILE


def test_triples_keep_file_order_per_receiver(capi, tmp_path):
    rng = np.random.default_rng(3)
    n = 40
    trip = [(int(rng.integers(n)), int(rng.integers(n)), float(f"{rng.uniform(0.02, 0.06):f}"))
            for _ in range(300)]
    trip += [(1, 2, 0.0), (3, 4, 5e-8)]  # not connections
    f = tmp_path / "t.txt"
    f.write_text("".join(f"{s} {r} {g:f}\n" for s, r, g in trip))
    rp, col, g = capi.read_conn_triples(str(f), n)
    for r in range(n):
        want = [(s, gg) for s, rr, gg in trip if rr == r and gg >= 1e-7]
        got = list(zip(col[rp[r]:rp[r + 1]].tolist(), g[rp[r]:rp[r + 1]].tolist()))
        assert [s for s, _ in got] == [s for s, _ in want]
        assert np.allclose([x for _, x in got], [x for _, x in want], rtol=1e-6)
    f.write_text("1 2 0.04\n5 99 0.04\n")
    with pytest.raises(capi.InfoliError) as e:
        capi.read_conn_triples(str(f), n)
    assert e.value.code == capi.ERR_CONFIG


def test_stimulus_file(capi, tmp_path):
    n, rows = 7, 5
    tab = np.round(np.random.default_rng(1).uniform(0, 8, (rows, n)), 3).astype(np.float32)
    f = tmp_path / "stim.txt"
    # extra values beyond n are ignored, as in the reference
    f.write_text("".join(" ".join(f"{v}" for v in row) + " 9.5 9.5\n" for row in tab))
    got = capi.read_stim_file(str(f), n)
    assert got.shape == (rows, n) and np.array_equal(got, tab)
    f.write_text("1 2 3\n")
    with pytest.raises(capi.InfoliError) as e:
        capi.read_stim_file(str(f), 5)
    assert e.value.code == capi.ERR_CONFIG and "only 3" in str(e.value)


def test_stimulus_file_of_the_single_threaded_fixture(capi, tmp_path):
    """The stimulus file the single-threaded reference ran on (tests/golden/
    single_rand_init.npz, written with "%.4f " per value as there) reads back
    as the table the GPU path is given."""
    tab = golden("single_rand_init.npz")["stim_stim16"]
    f = tmp_path / "stim.txt"
    f.write_text("".join(" ".join("%.4f" % x for x in row) + "\n" for row in tab))
    got = capi.read_stim_file(str(f), tab.shape[1])
    assert np.array_equal(got, tab)
