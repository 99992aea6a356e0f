"""The host driver end to end on the GPU: MatrixMarket in, the reference's
initial embedding (U[-1, 1) from the C library's unseeded rand(),
cpp/core/dense_mat.hpp:55-63), the epochs through GpuEmbeddingAlgo, the
reference's embedding file out.

Tolerance: the file holds 5 decimals, so every value must be within 6e-6 of the
same run through the Python API (identical GPU arithmetic), and the embedding
within the FP32 plain run tolerance of the FP64 oracle
(||x - x_oracle|| / ||x_oracle|| <= 1e-4).
"""
import ctypes
import os
import subprocess

import numpy as np
import pytest

import distembed_gb300 as de
import oracle
from distembed_gb300 import graphgen as gg

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _built():
    from distembed_gb300 import build
    build.build()


def reference_init(n, dim):
    """DenseMat's initial values: -1 + 2 rand() / (RAND_MAX + 1), row-major, glibc
    rand() from its default seed."""
    libc = ctypes.CDLL(None)
    libc.srand(1)
    vals = np.array([libc.rand() for _ in range(n * dim)], dtype=np.float64)
    return (-1.0 + 2.0 * vals / (2147483647 + 1.0)).reshape(n, dim)


def read_embedding(path, dim):
    rows = [line.split() for line in open(path)]
    ids = np.array([int(r[0]) for r in rows])
    x = np.array([[float(v) for v in r[1:]] for r in rows])
    assert x.shape[1] == dim
    return ids, x


@pytest.mark.parametrize("dim", [64, 128])
def test_driver_matches_api_and_oracle(tmp_path, dim):
    n, rp, col = gg.knn_csr(1500, 16, 8, 5, seed=90 + dim)
    mtx = str(tmp_path / "g.mtx")
    gg.write_mtx(mtx, n, rp, col)
    out = tmp_path / "out"
    out.mkdir()
    E, B, ns, lr = 4, 256, 5, 0.02
    r = subprocess.run([de.DRIVER_PATH, "-input", mtx, "-output", str(out), "-iter", str(E), "-batch", str(B),
                        "-nsamples", str(ns), "-lr", str(lr), "-dim", str(dim)], capture_output=True, text=True,
                       cwd=str(tmp_path))
    assert r.returncode == 0, r.stderr
    ids, x = read_embedding(str(out / "embedding.txt"), dim)
    assert np.array_equal(ids, np.arange(1, n + 1))
    x0 = reference_init(n, dim)
    with de.Handle(rp, col, dim) as h:
        h.set_embeddings(x0)
        h.run(E, B, ns, lr)
        xa = h.get_embeddings()
    assert np.max(np.abs(x - xa)) <= 6e-6
    xo, _ = oracle.run(rp, col, x0, E, B, ns, lr, quirks=True)
    assert np.linalg.norm(xa - xo) / np.linalg.norm(xo) <= 1e-4
    assert os.path.exists(tmp_path / "perf_output")


def test_driver_col_major_flag_is_the_one_rank_row_major_pass(tmp_path):
    """-col_major 1 writes the same file: the reference's one-rank branch calls the
    attractive pass with col_major = false (cpp/algo/algo.hpp:184-186)."""
    n, rp, col = gg.knn_csr(800, 16, 8, 4, seed=7)
    mtx = str(tmp_path / "g.mtx")
    gg.write_mtx(mtx, n, rp, col)
    texts = []
    for cm in ("0", "1"):
        out = tmp_path / f"out{cm}"
        out.mkdir()
        r = subprocess.run([de.DRIVER_PATH, "-input", mtx, "-output", str(out), "-iter", "3", "-batch", "128",
                            "-dim", "64", "-col_major", cm], capture_output=True, text=True, cwd=str(tmp_path))
        assert r.returncode == 0, r.stderr
        texts.append((out / "embedding.txt").read_text())
    assert texts[0] == texts[1]


def test_driver_col_major_on_a_directed_graph_reads_the_transpose(tmp_path):
    """-col_major 1 on an asymmetric (general) file: the passes read the receiver
    matrix's CSR, the transpose (cpp/algo/algo.hpp:131-133), so each row takes its
    attractive forces from its in-neighbours; the file matches the API run on the
    transposed CSR and differs from -col_major 0."""
    n = 700
    rng = np.random.default_rng(43)
    src, dst = rng.integers(0, n, 6000), rng.integers(0, n, 6000)
    keep = src != dst
    rp, col = gg.coo_to_csr(n, src[keep], dst[keep])
    mtx = str(tmp_path / "g.mtx")
    gg.write_mtx(mtx, n, rp, col)
    files = {}
    for cm in ("0", "1"):
        out = tmp_path / f"out{cm}"
        out.mkdir()
        r = subprocess.run([de.DRIVER_PATH, "-input", mtx, "-output", str(out), "-iter", "3", "-batch", "128",
                            "-dim", "64", "-col_major", cm], capture_output=True, text=True, cwd=str(tmp_path))
        assert r.returncode == 0, r.stderr
        files[cm] = read_embedding(str(out / "embedding.txt"), 64)[1]
    x0 = reference_init(n, 64)
    trp, tcol = gg.transpose_csr(rp, col)
    want = {}
    for cm, (a, b) in (("0", (rp, col)), ("1", (trp, tcol))):
        with de.Handle(a, b, 64) as h:
            h.set_embeddings(x0)
            h.run(3, 128, 5, 0.02)
            want[cm] = h.get_embeddings()
        assert np.max(np.abs(files[cm] - want[cm])) <= 6e-6
    assert np.max(np.abs(files["0"] - files["1"])) > 1e-3
    # the Python mirror of the reference class takes the same flag
    dense = x0.copy()
    de.EmbeddingAlgo(rp, col, dense, col_major=True).algo_force2_vec_ns(3, 128, 5, 0.02)
    assert np.array_equal(dense, want["1"])
    xo, _ = oracle.run(trp, tcol, x0, 3, 128, 5, 0.02, quirks=True)
    assert np.linalg.norm(dense - xo) / np.linalg.norm(xo) <= 1e-4


def test_driver_spmm_baseline(tmp_path):
    """-spmm 1: the reference's SpMM baseline (BaselineSpMM::execute,
    cpp/algo/baseline_spmm.hpp:52-90), one timed SpMM step per iteration."""
    n, rp, col = gg.knn_csr(700, 8, 6, 3, seed=8)
    mtx = str(tmp_path / "g.mtx")
    gg.write_mtx(mtx, n, rp, col)
    r = subprocess.run([de.DRIVER_PATH, "-input", mtx, "-spmm", "1", "-iter", "3", "-batch", "128", "-dim", "64",
                        "-lr", "0.02"], capture_output=True, text=True, cwd=str(tmp_path))
    assert r.returncode == 0, r.stderr
    assert r.stdout.count("SpMM iteration") == 3
    line = [ln for ln in open(tmp_path / "perf_output") if '"SpMM"' in ln][-1]
    import json
    assert len(json.loads(line)["iteration_time_s"]) == 3


@pytest.mark.parametrize("merge", ["0", "1"])
def test_driver_sparse_embedding(tmp_path, merge):
    """-sparse_embedding 1: the reference's sparse embedding branch
    (cpp/dist_embed.cpp:317-330): rand() rows, algo_sparse_embedding, embedding.txt."""
    n, rp, col = gg.knn_csr(900, 8, 6, 3, seed=9)
    mtx = str(tmp_path / "g.mtx")
    gg.write_mtx(mtx, n, rp, col)
    out = tmp_path / "out"
    out.mkdir()
    r = subprocess.run([de.DRIVER_PATH, "-input", mtx, "-output", str(out), "-sparse_embedding", "1", "-iter", "3",
                        "-batch", "128", "-dim", "64", "-lr", "0.02", "-density", "0.5", "-sparse_merge", merge],
                       capture_output=True, text=True, cwd=str(tmp_path))
    assert r.returncode == 0, r.stderr
    ids, x = read_embedding(str(out / "embedding.txt"), 64)
    assert np.array_equal(ids, np.arange(1, n + 1))
    xo, _ = oracle.sparse_embedding(rp, col, reference_init(n, 64), 3, 128, 5, 0.02, 0.5, merge=merge == "1")
    assert np.max(np.abs(x - xo)) <= 6e-6 + (1e-4 if merge == "1" else 0.0)
    if merge == "0":
        assert np.all((x != 0).sum(1) == 32)
    line = [ln for ln in open(tmp_path / "perf_output") if '"SparseEmbedding"' in ln][-1]
    assert '"iterations":3' in line
