"""The oracle's many-graph entry (oracle_run_many) against its one-graph loop.

run_many trains each graph on one host thread; a graph's arithmetic is the same
as oracle.run's, so embeddings and per-epoch losses must be bitwise equal.  The
-O3 build (the timed CPU baseline) fuses multiply-adds and is held to 1e-10.
"""
import numpy as np
import pytest

import oracle
from distembed_gb300 import graphgen as gg


@pytest.fixture(scope="module")
def suite():
    gs = gg.graph_suite(10, 300, 3000, 7, knn_k=6, knn_dim=8, rmat_ef=4)
    xs = [gg.init_embedding(n, 32, seed=50 + i) for i, (_, n, _, _) in enumerate(gs)]
    return [(rp, c) for _, _, rp, c in gs], xs


@pytest.mark.parametrize("quirks", [True, False])
def test_run_many_equals_run(suite, quirks):
    csr, xs = suite
    lr = [0.03, 0.02, 0.01, 0.02]
    many = [x.copy() for x in xs]
    u, loss = oracle.run_many(csr, many, 4, 128, 5, lr, quirks=quirks, threads=4)
    total = 0
    for i, (rp, c) in enumerate(csr):
        x1, l1 = oracle.run(rp, c, xs[i], 4, 128, 5, lr, quirks=quirks, threads=1)
        assert np.array_equal(x1, many[i]), i
        assert np.array_equal(l1, loss[i]), i
        n = len(rp) - 1
        for e in range(4):
            total += oracle.run_batches(rp, c, xs[i].copy(), e, 128, 5, 0.0, list(range((n + 127) // 128)),
                                        quirks=quirks)
    assert u == total


def test_run_many_resume_and_no_loss(suite):
    csr, xs = suite
    a = [x.copy() for x in xs]
    b = [x.copy() for x in xs]
    oracle.run_many(csr, a, 5, 256, 7, 0.02)
    oracle.run_many(csr, b, 2, 256, 7, 0.02, want_loss=False)
    _, tail = oracle.run_many(csr, b, 3, 256, 7, 0.02, first_epoch=2)
    assert all(np.array_equal(p, q) for p, q in zip(a, b))
    _, full = oracle.run_many(csr, [x.copy() for x in xs], 5, 256, 7, 0.02)
    assert np.array_equal(full[:, 2:], tail)


def test_fast_build_close(suite):
    csr, xs = suite
    a = [x.copy() for x in xs]
    b = [x.copy() for x in xs]
    ua, _ = oracle.run_many(csr, a, 3, 128, 5, 0.02, want_loss=False)
    ub, _ = oracle.run_many(csr, b, 3, 128, 5, 0.02, want_loss=False, fast=True)
    assert ua == ub
    for p, q in zip(a, b):
        assert np.linalg.norm(p - q) <= 1e-10 * np.linalg.norm(p)
