"""The FP64 oracle against the golden vectors written by the reference's own code.

Bit-exact: the restatement must round exactly as cpp/algo/algo.hpp does.
"""
import glob
import os

import numpy as np
import pytest

import oracle


def _runs(golden_dir):
    return sorted(glob.glob(os.path.join(golden_dir, "run_*.npz")))


def test_golden_files_present(golden_dir):
    assert len(_runs(golden_dir)) >= 5


@pytest.mark.parametrize("idx", range(5))
def test_oracle_run_bitexact(golden_dir, idx):
    path = _runs(golden_dir)[idx]
    g = np.load(path)
    x1, _ = oracle.run(g["rowptr"], g["col"], g["x0"], int(g["epochs"]), int(g["batch"]), int(g["ns"]),
                       g["lr"], quirks=True)
    assert np.array_equal(x1, g["x1"]), os.path.basename(path)


def test_oracle_batch_grad_bitexact(golden_dir):
    g = np.load(os.path.join(golden_dir, "grad_knn300_d64.npz"))
    n_keys = 0
    for key in g.files:
        if not (key.startswith("b") and key.count("_") == 2):
            continue
        b, s, c = (int(t[1:]) for t in key.split("_"))
        prev, _ = oracle.batch_grad(g["rowptr"], g["col"], g["x"], int(g["batch"]), int(g["ns"]), float(g["lr"]),
                                    b, s, c, quirks=True)
        assert np.array_equal(prev, g[key]), key
        n_keys += 1
    assert n_keys == 4


def test_oracle_negatives_bitexact(golden_dir):
    g = np.load(os.path.join(golden_dir, "negatives.npz"))
    assert np.array_equal(oracle.negatives(60000, 1234, 10), g["u60000_s1234_k10"].astype(np.int64))
    for key in g.files:
        if key.count("_") != 1:
            continue
        upper, ns = int(key.split("_")[0][1:]), int(key.split("_")[1][1:])
        want = g[key].astype(np.int64)
        got = np.stack([oracle.negatives(upper, s, ns) for s in range(want.shape[0])])
        assert np.array_equal(got, want), key


def test_negatives_inclusive_upper_bound(golden_dir):
    # uniform_int_distribution<int>(0, n) includes n (cpp/core/common.cpp:44)
    g = np.load(os.path.join(golden_dir, "negatives.npz"))
    assert g["u1_k8"].max() == 1 and g["u0_k4"].max() == 0


def test_csr_builder_order(golden_dir):
    from distembed_gb300 import graphgen as gg
    g = np.load(os.path.join(golden_dir, "csr_small.npz"))
    rp, col = gg.coo_to_csr(4, g["coo_row"], g["coo_col"])
    assert np.array_equal(rp, g["rowptr"]) and np.array_equal(col, g["col"])


def test_rep_rows_quirk():
    # F8: from the second epoch of a call every batch repulses only last_batch_size rows
    assert oracle.rep_rows(300, 64, 0, 0, True) == 64
    assert oracle.rep_rows(300, 64, 0, 4, True) == 300 - 4 * 64
    assert oracle.rep_rows(300, 64, 1, 0, True) == 300 - 4 * 64
    assert oracle.rep_rows(300, 64, 1, 0, False) == 64
    assert oracle.rep_rows(256, 64, 3, 1, True) == 64


@pytest.mark.skipif(not oracle.ref_available(), reason="reference harness is only buildable where its sources are")
def test_oracle_matches_reference_live():
    from distembed_gb300 import graphgen as gg
    n, rp, col = gg.rmat_csr(10, 6, seed=11)
    x0 = gg.init_embedding(n, 32, 12)
    for driver in (True, False):
        lr = 0.03 if driver else np.array([0.03, 0.02, 0.01])
        xr = oracle.ref_run(rp, col, x0, 3, 200, 6, lr, driver_loop=driver)
        if xr is None:
            pytest.skip("draw hits the reference's undefined path")
        xo, _ = oracle.run(rp, col, x0, 3, 200, 6, lr, quirks=True)
        assert np.array_equal(xr, xo)


@pytest.mark.parametrize("name", ["spmm_hand18_d32", "spmm_rmat9_d16"])
def test_oracle_spmm_bitexact(golden_dir, name):
    # the reference's SpMM step (SpMMAlgo::algo_spmm, cpp/algo/spmm.hpp:54-159):
    # the hand graph has edges into its last vertex, which the reference skips
    g = np.load(os.path.join(golden_dir, f"{name}.npz"))
    y = oracle.spmm(g["rowptr"], g["col"], g["x"], float(g["lr"]), quirks=True)
    assert np.array_equal(y, g["y"])
    assert not np.array_equal(oracle.spmm(g["rowptr"], g["col"], g["x"], float(g["lr"]), quirks=False), g["y"]) \
        or name != "spmm_hand18_d32"


@pytest.mark.skipif(not oracle.ref_available(), reason="reference harness is only buildable where its sources are")
def test_oracle_spmm_matches_reference_live():
    from distembed_gb300 import graphgen as gg
    n, rp, col = gg.rmat_csr(10, 6, seed=13)
    x = gg.init_embedding(n, 64, 14)
    for batch in (64, 300, n):
        assert np.array_equal(oracle.ref_spmm(rp, col, x, batch, 0.05), oracle.spmm(rp, col, x, 0.05))


@pytest.mark.parametrize("name", ["sparse_hand18_d16_q", "sparse_rmat9_d16_m"])
def test_oracle_sparse_embedding_bitexact(golden_dir, name):
    # the reference's sparse embedding at one rank (cpp/algo/sparse_embedding.hpp:78-194):
    # embedding values and batch collector equal to the reference's, bit for bit
    g = np.load(os.path.join(golden_dir, f"{name}.npz"))
    x, coll = oracle.sparse_embedding(g["rowptr"], g["col"], g["x"], int(g["iterations"]), int(g["batch"]),
                                      int(g["ns"]), float(g["lr"]), float(g["density"]), bool(g["merge"]))
    assert np.array_equal(x, g["x_out"]) and np.array_equal(coll, g["coll"])
    if bool(g["merge"]):
        # the repulsive row count of the multi-rank branch (F8) matters here
        x2, _ = oracle.sparse_embedding(g["rowptr"], g["col"], g["x"], int(g["iterations"]), int(g["batch"]),
                                        int(g["ns"]), float(g["lr"]), float(g["density"]), True, quirks=False)
        assert not np.array_equal(x2, g["x_out"])
    else:
        # the one-rank branch never merges its collector: the values are the
        # input's with the dim - k smallest of every row set to zero
        k = int(g["x"].shape[1] * float(g["density"]))
        kept = (g["x_out"] != 0).sum(1)
        assert np.all(kept == k) and np.all(np.isin(g["x_out"][g["x_out"] != 0], g["x"]))


@pytest.mark.skipif(not oracle.ref_available(), reason="reference harness is only buildable where its sources are")
@pytest.mark.parametrize("merge", [False, True])
def test_oracle_sparse_embedding_matches_reference_live(merge):
    from distembed_gb300 import graphgen as gg
    cases = [(gg.rmat_csr(10, 8, seed=21), 32, 3, 97, 0.3), (gg.knn_csr(1200, 8, 8, 4, seed=22), 64, 3, 256, 0.5),
             (gg.rmat_csr(9, 4, seed=23), 16, 2, 512, 1.0), (gg.rmat_csr(9, 4, seed=24), 16, 3, 50, 0.0)]
    for (n, rp, col), dim, iters, batch, density in cases:
        x = gg.init_embedding(n, dim, 25)
        try:
            want = oracle.ref_sparse_embedding(rp, col, x, iters, batch, 5, 0.05, density, merge)
        except ValueError:  # a draw equal to n: the reference's out-of-range path
            continue
        got = oracle.sparse_embedding(rp, col, x, iters, batch, 5, 0.05, density, merge)
        assert np.array_equal(got[0], want[0]) and np.array_equal(got[1], want[1])


@pytest.mark.skipif(not oracle.ref_available(), reason="reference harness is only buildable where its sources are")
def test_col_major_reads_the_transposed_csr():
    # with col_major the reference's loop reads the receiver matrix's CSR, the
    # transpose of the native one (cpp/algo/algo.hpp:131-133), and runs the row-major
    # pass on it (:184-186): on a directed graph, the oracle on the transposed CSR
    from distembed_gb300 import graphgen as gg
    n = 600
    rng = np.random.default_rng(41)
    src, dst = rng.integers(0, n, 5000), rng.integers(0, n, 5000)
    keep = src != dst
    rp, col = gg.coo_to_csr(n, src[keep], dst[keep])
    trp, tcol = gg.transpose_csr(rp, col)
    x0 = gg.init_embedding(n, 32, 42)
    for driver in (True, False):
        xr = oracle.ref_run(rp, col, x0, 3, 128, 5, 0.03, driver_loop=driver, col_major=True)
        if xr is None:
            pytest.skip("draw hits the reference's undefined path")
        xo, _ = oracle.run(trp, tcol, x0, 3, 128, 5, 0.03, quirks=True)
        assert np.array_equal(xr, xo)
        assert not np.array_equal(xr, oracle.ref_run(rp, col, x0, 3, 128, 5, 0.03, driver_loop=driver))
