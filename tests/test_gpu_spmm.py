"""The SpMM step (de_spmm: SpMMAlgo::algo_spmm at one rank, cpp/algo/spmm.hpp:54-159)
on the GPU against the FP64 oracle (oracle.spmm, pinned to the reference's own
SpMM by tests/test_oracle_golden.py) and the reference's golden output.

Tolerance (FP32 accumulation against FP64): elementwise
|y_gpu - y_oracle| <= 1e-5 * (|y_oracle| + rms(y_oracle)).
"""
import os

import numpy as np
import pytest

import distembed_gb300 as de
import oracle
from distembed_gb300 import graphgen as gg

pytestmark = pytest.mark.gpu

RTOL = 1e-5


def close(got, want):
    tol = RTOL * (np.abs(want) + np.sqrt(np.mean(want ** 2)))
    return bool(np.all(np.abs(got - want) <= tol))


def f32(x):
    return np.asarray(x, dtype=np.float32).astype(np.float64)


@pytest.fixture(scope="module", autouse=True)
def _built():
    from distembed_gb300 import build
    build.build()


def test_spmm_matches_reference_golden(golden_dir):
    g = np.load(os.path.join(golden_dir, "spmm_hand18_d32.npz"))
    with de.Handle(g["rowptr"], g["col"], 32) as h:
        h.set_embeddings(f32(g["x"]))
        y = h.spmm(int(g["batch"]), float(g["lr"]))
    want = oracle.spmm(g["rowptr"], g["col"], f32(g["x"]), float(g["lr"]))
    assert close(y, want)
    assert close(y, g["y"]) or np.allclose(y, g["y"], rtol=1e-6, atol=1e-7)


@pytest.mark.parametrize("dim", [32, 64, 128, 256])
@pytest.mark.parametrize("quirks", [True, False])
@pytest.mark.parametrize("graph", ["rmat", "knn"])
def test_spmm_matches_oracle(dim, quirks, graph):
    if graph == "rmat":
        n, rp, col = gg.rmat_csr(12, 8, seed=dim)  # hub rows longer than the edge cap
    else:
        n, rp, col = gg.knn_csr(3000, 8, 10, 5, seed=dim)
    x = f32(gg.init_embedding(n, dim, seed=3))
    with de.Handle(rp, col, dim, quirks=quirks) as h:
        h.set_embeddings(x)
        y = h.spmm(512, 0.05)
        x_after = h.get_embeddings()
    assert close(y, oracle.spmm(rp, col, x, 0.05, quirks=quirks))
    assert np.array_equal(x_after, x)  # the input is not changed


@pytest.mark.parametrize("batch,edge_cap", [(1, 0), (97, 8), (4096, 0), (100000, 4)])
def test_spmm_any_minibatch_size_and_split_rows(batch, edge_cap):
    n, rp, col = gg.rmat_csr(11, 16, seed=4)
    x = f32(gg.init_embedding(n, 64, seed=4))
    with de.Handle(rp, col, 64, edge_cap=edge_cap) as h:
        h.set_embeddings(x)
        y = h.spmm(batch, 0.02)
        y32 = h.spmm(batch, 0.02, dtype=np.float32)
    assert close(y, oracle.spmm(rp, col, x, 0.02))
    assert np.array_equal(y32.astype(np.float64), y)  # the same FP32 values either way


def test_spmm_on_a_bf16_handle_reads_the_fp32_master():
    n, rp, col = gg.knn_csr(2000, 8, 8, 4, seed=6)
    x = f32(gg.init_embedding(n, 128, seed=6))
    with de.Handle(rp, col, 128, precision="bf16") as h:
        h.set_embeddings(x)
        y = h.spmm(256, 0.1)
    assert close(y, oracle.spmm(rp, col, x, 0.1))
