"""The sparse embedding (de_sparse_embedding: SparseEmbedding::algo_sparse_embedding at
one rank, cpp/algo/sparse_embedding.hpp:78-194) on the GPU against the FP64 oracle
(oracle.sparse_embedding, pinned to the reference's own SparseEmbedding by
tests/test_oracle_golden.py).

merge=False (the reference's one-rank branch): the rows change only by the top-k
pruning, which compares the FP64 values, so the rows must be bitwise equal; the
batch collector is accumulated in FP32 per row and in FP64 across minibatches:
elementwise |c_gpu - c_oracle| <= 1e-4 * (|c_oracle| + rms(c_oracle)) + a, with
a = 1e-5 * lr * iterations * sqrt(minibatches) for the slots whose sum over many
rows cancels (attractive forces cancel in pairs on a symmetric graph).
merge=True: the rows are trained in FP32 (the plain minibatch step on the rows'
FP32 mirror): |x_gpu - x_oracle| <= 1e-4 * (|x_oracle| + rms(x_oracle)).
"""
import numpy as np
import pytest

import distembed_gb300 as de
import oracle
from distembed_gb300 import graphgen as gg

pytestmark = pytest.mark.gpu

RTOL = 1e-4
ABSENT = de.Handle.ABSENT


def close(got, want, atol=0.0):
    tol = RTOL * (np.abs(want) + np.sqrt(np.mean(want ** 2)) + 1e-30) + atol
    return bool(np.all(np.abs(got - want) <= tol))


def coll_atol(n, batch, iterations, lr):
    return 1e-5 * lr * iterations * np.sqrt(-(-n // batch))


def f32(x):
    return np.asarray(x, dtype=np.float32).astype(np.float64)


@pytest.fixture(scope="module", autouse=True)
def _built():
    from distembed_gb300 import build
    build.build()


def graph(kind, seed):
    if kind == "rmat":
        return gg.rmat_csr(11, 8, seed=seed)  # hub rows longer than the edge cap
    return gg.knn_csr(2500, 8, 10, 5, seed=seed)


@pytest.mark.parametrize("dim", [32, 64, 128, 256])
@pytest.mark.parametrize("kind", ["rmat", "knn"])
@pytest.mark.parametrize("iterations,density", [(1, 0.5), (3, 0.5), (3, 0.25)])
def test_one_rank_branch_matches_oracle(dim, kind, iterations, density):
    n, rp, col = graph(kind, dim)
    x = f32(gg.init_embedding(n, dim, seed=dim + 1))
    with de.Handle(rp, col, dim) as h:
        got_x, got_c = h.sparse_embedding(x, iterations, 300, 5, 0.05, density)
    want_x, want_c = oracle.sparse_embedding(rp, col, x, iterations, 300, 5, 0.05, density)
    assert np.array_equal(got_x, want_x)
    assert close(got_c, want_c, coll_atol(n, 300, iterations, 0.05))
    if iterations > 1:
        assert np.all((got_x != 0).sum(1) == int(dim * density))


@pytest.mark.parametrize("dim", [32, 64, 128, 256])
@pytest.mark.parametrize("kind", ["rmat", "knn"])
@pytest.mark.parametrize("quirks", [True, False])
def test_merge_matches_oracle(dim, kind, quirks):
    n, rp, col = graph(kind, dim + 7)
    x = f32(gg.init_embedding(n, dim, seed=dim + 2))
    with de.Handle(rp, col, dim, quirks=quirks) as h:
        got_x, got_c = h.sparse_embedding(x, 3, 256, 5, 0.05, 0.5, merge=True)
    want_x, want_c = oracle.sparse_embedding(rp, col, x, 3, 256, 5, 0.05, 0.5, merge=True, quirks=quirks)
    assert close(got_x, want_x)
    assert np.array_equal(got_c, np.zeros_like(got_c)) and np.array_equal(want_c, np.zeros_like(want_c))


@pytest.mark.parametrize("merge", [False, True])
def test_sparse_input_and_edge_cases(merge):
    # rows that already have absent entries; a minibatch size that does not divide
    # n; split rows (edge cap 8); zero iterations; density 0 and 1
    n, rp, col = gg.rmat_csr(10, 16, seed=31)
    dim = 64
    x = f32(gg.init_embedding(n, dim, seed=32))
    rng = np.random.default_rng(33)
    x[rng.random(x.shape) < 0.3] = ABSENT
    for iterations, batch, density in [(0, 97, 0.5), (2, 97, 0.5), (3, 1000, 0.0), (2, 5000, 1.0), (2, 1, 0.3)]:
        with de.Handle(rp, col, dim, edge_cap=8) as h:
            got_x, got_c = h.sparse_embedding(x, iterations, batch, 4, 0.1, density, merge=merge)
        want_x, want_c = oracle.sparse_embedding(rp, col, x, iterations, batch, 4, 0.1, density, merge=merge)
        if merge:
            assert close(got_x, want_x), (iterations, batch, density)
        else:
            assert np.array_equal(got_x, want_x), (iterations, batch, density)
            assert close(got_c, want_c, coll_atol(n, batch, iterations, 0.1)), (iterations, batch, density)
        if iterations == 0:
            assert np.array_equal(got_x, x)  # no iteration, no final clear: absent entries stay INT_MIN


def test_three_step_api_equals_one_call():
    n, rp, col = graph("knn", 5)
    x = f32(gg.init_embedding(n, 128, seed=6))
    with de.Handle(rp, col, 128) as h:
        one_x, one_c = h.sparse_embedding(x, 3, 512, 5, 0.05, 0.5)
        h.sparse_set(x)
        h.sparse_run(3, 512, 5, 0.05, 0.5)
        three_x, three_c = h.sparse_get()
    assert np.array_equal(one_x, three_x) and np.array_equal(one_c, three_c)


def test_unsupported_handles_refuse():
    n, rp, col = graph("knn", 7)
    with de.Handle(rp, col, 128, precision="bf16") as h:
        with pytest.raises(de.DEError):
            h.sparse_embedding(np.zeros((n, 128)), 1, 256, 5, 0.05, 0.5)
    with de.Handle(rp, col, 64) as h:
        with pytest.raises(de.DEError):
            h.sparse_run(1, 256, 5, 0.05, 0.5)  # no rows uploaded


@pytest.mark.parametrize("merge", [False, True])
def test_pinned_and_device_rows_equal_pageable(merge):
    # pinned host rows and device rows are read and written by kernels, pageable
    # rows by copies: the same results either way
    torch = pytest.importorskip("torch")
    n, rp, col = graph("rmat", 51)
    x = f32(gg.init_embedding(n, 64, seed=52))
    x[::7, 3] = ABSENT
    with de.Handle(rp, col, 64) as h:
        want_x, want_c = h.sparse_embedding(x, 3, 200, 5, 0.05, 0.5, merge=merge)
        pinned = torch.empty((n, 64), dtype=torch.float64, pin_memory=True).numpy()
        pinned[:] = x
        coll = torch.empty((200, 64), dtype=torch.float64, pin_memory=True).numpy()
        h.sparse_embedding(pinned, 3, 200, 5, 0.05, 0.5, merge=merge, inplace=True, coll=coll)
        h.sparse_set(torch.from_numpy(x).to("cuda"))
        h.sparse_run(3, 200, 5, 0.05, 0.5, merge=merge)
        dev_x, dev_c = h.sparse_get()
    assert np.array_equal(pinned, want_x) and np.array_equal(coll, want_c)
    assert np.array_equal(dev_x, want_x) and np.array_equal(dev_c, want_c)
