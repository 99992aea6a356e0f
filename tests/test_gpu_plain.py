"""FP32 plain GPU path against the FP64 oracle, through the C ABI.

Tolerances (FP32 arithmetic against FP64, same FP32-rounded starting point):
  one minibatch     ||gpu - oracle||_2 / ||oracle||_2 <= 1e-5 (relative, over the whole
                    minibatch) and |gpu - oracle| <= 1e-5 * (|oracle| + rms(oracle))
                    elementwise, for the update itself and for the updated embedding
  several epochs    ||gpu - oracle||_2 / ||oracle||_2 <= 1e-4 for the embedding,
                    |loss_gpu - loss_oracle| / loss_oracle <= 1e-3 for every epoch
  indices, CSR order and traversal order are exact by construction (same sampler,
  same CSR), and results are bitwise reproducible run to run.
"""
import glob
import os

import numpy as np
import pytest

import distembed_gb300 as de
import oracle
from distembed_gb300 import graphgen as gg

pytestmark = pytest.mark.gpu

ONE_STEP_RTOL = 1e-5
RUN_REL_L2 = 1e-4
LOSS_RTOL = 1e-3


def f32(x):
    return np.asarray(x, dtype=np.float32).astype(np.float64)


def close_one_step(got, want):
    tol = ONE_STEP_RTOL * (np.abs(want) + np.sqrt(np.mean(want ** 2)))
    bad = np.abs(got - want) > tol
    return not bad.any(), float(np.max(np.abs(got - want) / (tol / ONE_STEP_RTOL)))


def rel_l2(got, want):
    return float(np.linalg.norm(got - want) / np.linalg.norm(want))


def gpu_run(rp, col, x0, epochs, batch, ns, lr, quirks=True, edge_cap=0, dim=None):
    with de.Handle(rp, col, x0.shape[1], quirks=quirks, edge_cap=edge_cap) as h:
        h.set_embeddings(x0)
        loss = h.run(epochs, batch, ns, lr)
        return h.get_embeddings(), loss


@pytest.fixture(scope="module", autouse=True)
def _built():
    from distembed_gb300 import build
    build.build()


# ---------------------------------------------------------------- one step

@pytest.mark.parametrize("dim", [32, 64, 128, 256])
@pytest.mark.parametrize("quirks", [True, False])
def test_one_minibatch_matches_oracle(dim, quirks):
    n, rp, col = gg.knn_csr(700, 8, 7, 5, seed=dim)
    x0 = f32(gg.init_embedding(n, dim, seed=3))
    # one minibatch covering every row: the update is exactly one step
    prev, _ = oracle.batch_grad(rp, col, x0, n, 5, 0.02, 0, 0, n, quirks=quirks)
    x1, _ = gpu_run(rp, col, x0, 1, n, 5, 0.02, quirks=quirks)
    assert rel_l2(x1 - x0, prev) <= ONE_STEP_RTOL, rel_l2(x1 - x0, prev)
    assert rel_l2(x1, x0 + prev) <= ONE_STEP_RTOL
    ok, worst = close_one_step(x1 - x0, prev)
    assert ok, f"update off by {worst:.2e} (relative units)"
    ok, worst = close_one_step(x1, x0 + prev)
    assert ok, f"embedding off by {worst:.2e}"


def test_one_minibatch_split_rows_match_oracle():
    # a star: vertex 0 adjacent to everyone, so its row is split into many parts
    n = 3000
    s = np.concatenate([np.zeros(n - 1, np.int64), np.arange(1, n)])
    d = np.concatenate([np.arange(1, n), np.zeros(n - 1, np.int64)])
    rp, col = gg.coo_to_csr(n, s, d)
    x0 = f32(gg.init_embedding(n, 128, seed=4))
    prev, _ = oracle.batch_grad(rp, col, x0, n, 5, 0.01, 0, 0, n, quirks=True)
    for cap in (8, 64, 4096):
        x1, _ = gpu_run(rp, col, x0, 1, n, 5, 0.01, edge_cap=cap)
        ok, worst = close_one_step(x1 - x0, prev)
        assert ok, f"cap {cap}: off by {worst:.2e}"


# ------------------------------------------------------------ full runs

def _golden_cases():
    d = os.path.join(os.path.dirname(__file__), "golden")
    for path in sorted(glob.glob(os.path.join(d, "run_*.npz"))):
        g = np.load(path)
        if g["x0"].shape[1] in (32, 64, 128, 256):
            yield os.path.basename(path)


@pytest.mark.parametrize("name", list(_golden_cases()))
def test_golden_runs(name):
    g = np.load(os.path.join(os.path.dirname(__file__), "golden", name))
    x1, _ = gpu_run(g["rowptr"], g["col"], g["x0"], int(g["epochs"]), int(g["batch"]), int(g["ns"]), g["lr"])
    assert rel_l2(x1, g["x1"]) <= RUN_REL_L2


@pytest.mark.parametrize("quirks", [True, False])
def test_multi_epoch_rmat_matches_oracle(quirks):
    n, rp, col = gg.rmat_csr(11, 8, seed=21)
    x0 = f32(gg.init_embedding(n, 64, seed=5))
    E, B, ns = 5, 300, 5          # 2048 % 300 != 0: the last-batch quirk is active
    lr = 0.02 * (1 - np.arange(E) / E)
    xo, lo = oracle.run(rp, col, x0, E, B, ns, lr, quirks=quirks)
    xg, lg = gpu_run(rp, col, x0, E, B, ns, lr, quirks=quirks, edge_cap=16)
    assert rel_l2(xg, xo) <= RUN_REL_L2
    assert np.all(np.abs(lg - lo) <= LOSS_RTOL * lo), (lg, lo)


def test_quirk_edges_into_last_vertex():
    # only difference between the modes on one minibatch: edges into n-1 and
    # nothing else (ns = 0)
    n, rp, col = gg.knn_csr(400, 8, 6, 3, seed=9)
    x0 = f32(gg.init_embedding(n, 32, seed=6))
    on, _ = gpu_run(rp, col, x0, 1, n, 0, 0.05, quirks=True)
    off, _ = gpu_run(rp, col, x0, 1, n, 0, 0.05, quirks=False)
    src = np.repeat(np.arange(n), np.diff(rp))
    touched = np.unique(src[col == n - 1])
    assert len(touched) > 0
    diff_rows = np.where(np.any(on != off, axis=1))[0]
    assert set(diff_rows) == set(touched)


def test_draw_equal_to_n_is_skipped():
    # small n: some minibatch draws the value n (the sampler's bound is inclusive)
    n, rp, col = gg.knn_csr(12, 4, 3, 2, seed=12)
    hits = [(i, j) for i in range(6) for j in range(3) if (oracle.negatives(n, i + j, 5) == n).any()]
    assert hits, "pick parameters where a draw equals n"
    x0 = f32(gg.init_embedding(n, 32, seed=7))
    xo, lo = oracle.run(rp, col, x0, 6, 4, 5, 0.05, quirks=True)
    xg, lg = gpu_run(rp, col, x0, 6, 4, 5, 0.05)
    assert rel_l2(xg, xo) <= RUN_REL_L2
    assert np.allclose(lg, lo, rtol=LOSS_RTOL)


@pytest.mark.parametrize("n,batch", [(50, 64), (64, 64), (65, 64), (1, 8), (33, 1)])
def test_batch_edge_cases(n, batch):
    if n > 1:
        _, rp, col = gg.knn_csr(n, 4, min(3, n - 1), 2, seed=n)
    else:
        rp, col = np.array([0, 0]), np.zeros(0, np.int64)
    x0 = f32(gg.init_embedding(n, 64, seed=8))
    E = 3
    xo, lo = oracle.run(rp, col, x0, E, batch, 3, 0.03, quirks=True)
    xg, lg = gpu_run(rp, col, x0, E, batch, 3, 0.03)
    assert rel_l2(xg, xo) <= RUN_REL_L2
    assert np.allclose(lg, lo, rtol=LOSS_RTOL, atol=1e-9)


def test_bitwise_reproducible_and_handle_reuse():
    n, rp, col = gg.rmat_csr(12, 8, seed=22)
    x0 = f32(gg.init_embedding(n, 128, seed=9))
    a, la = gpu_run(rp, col, x0, 3, 512, 5, 0.02, edge_cap=16)
    b, lb = gpu_run(rp, col, x0, 3, 512, 5, 0.02, edge_cap=16)
    assert np.array_equal(a, b) and np.array_equal(la, lb)
    # one handle, changing minibatch size and ns between calls, FP32 round trip
    with de.Handle(rp, col, 128, edge_cap=16) as h:
        h.set_embeddings(x0.astype(np.float32))
        h.run(3, 512, 5, 0.02)
        assert np.array_equal(h.get_embeddings(dtype=np.float32).astype(np.float64), a)
        h.set_embeddings(x0)
        h.run(1, 1000, 7, 0.02)
        h.set_embeddings(x0)
        h.run(3, 512, 5, 0.02)
        assert np.array_equal(h.get_embeddings(), a)


@pytest.mark.parametrize("precision", ["fp32", "bf16"])
def test_pinned_host_buffers_equal_pageable(precision):
    # pinned host memory is converted in place by the GPU, pageable memory through
    # a staging copy: the same values either way
    import torch
    n, rp, col = gg.rmat_csr(11, 8, seed=25)
    x0 = f32(gg.init_embedding(n, 128, seed=10))
    pinned_in = torch.empty((n, 128), dtype=torch.float64, pin_memory=True).numpy()
    pinned_in[:] = x0
    pinned_out = torch.empty((n, 128), dtype=torch.float64, pin_memory=True).numpy()
    out = []
    for src in (x0, pinned_in):
        with de.Handle(rp, col, 128, precision=precision) as h:
            h.set_embeddings(src)
            loss = h.run(2, 300, 5, 0.02)
            y = h.get_embeddings(out=pinned_out) if src is pinned_in else h.get_embeddings()
            out.append((np.array(y), loss))
    assert np.array_equal(out[0][0], out[1][0]) and np.array_equal(out[0][1], out[1][1])
    with de.Handle(rp, col, 128) as h:
        h.set_embeddings(pinned_in)
        assert np.array_equal(h.get_embeddings(), x0)
        assert np.array_equal(h.spmm(256, 0.1, out=pinned_out), h.spmm(256, 0.1))


@pytest.mark.parametrize("dim", [64, 128])
def test_overlapped_launches_bitwise_equal_to_serial(dim):
    # launch j+1 starts before launch j completes; its early phase must only
    # read final rows, so the result may not depend on the overlap
    n, rp, col = gg.rmat_csr(13, 8, seed=24)
    x0 = f32(gg.init_embedding(n, dim, seed=12))
    out = []
    for pdl in (True, False):
        with de.Handle(rp, col, dim, pdl=pdl, edge_cap=16) as h:
            h.set_embeddings(x0)
            loss = h.run(4, 256, 7, 0.03)
            out.append((h.get_embeddings(), loss))
    assert np.array_equal(out[0][0], out[1][0]) and np.array_equal(out[0][1], out[1][1])
    xo, lo = oracle.run(rp, col, x0, 4, 256, 7, 0.03, quirks=True)
    assert rel_l2(out[0][0], xo) <= RUN_REL_L2


def test_resume_equals_one_call():
    n, rp, col = gg.rmat_csr(11, 8, seed=23)
    x0 = f32(gg.init_embedding(n, 64, seed=11))
    E, B, ns = 5, 300, 5
    lr = 0.02 * (1 - np.arange(E) / E)
    with de.Handle(rp, col, 64, edge_cap=16) as h:
        h.set_embeddings(x0)
        l_all = h.run(E, B, ns, lr)
        x_all = h.get_embeddings()
        h.set_embeddings(x0)
        l_a = h.run(2, B, ns, lr[:2])
        l_b = h.run(3, B, ns, lr[2:], first_epoch=2)
        x_split = h.get_embeddings()
        assert h.edge_updates(2, B, ns) + h.edge_updates(3, B, ns, first_epoch=2) == h.edge_updates(E, B, ns)
    assert np.array_equal(x_all, x_split)
    assert np.array_equal(l_all, np.concatenate([l_a, l_b]))


def test_edge_update_count():
    n, rp, col = gg.knn_csr(500, 8, 5, 3, seed=10)
    E, B, ns = 4, 96, 5
    want = 0
    for i in range(E):
        for j in range((n + B - 1) // B):
            rows = oracle.rep_rows(n, B, i, j, True)
            valid = int(np.sum(oracle.negatives(n, i + j, ns) < n))
            want += rows * valid
    want += E * (len(col) - int(np.sum(col == n - 1)))
    with de.Handle(rp, col, 32) as h:
        assert h.edge_updates(E, B, ns) == want


def test_reference_interface_updates_in_place():
    n, rp, col = gg.knn_csr(300, 8, 5, 4, seed=300)
    dense = f32(gg.init_embedding(n, 32, seed=1))
    want, _ = oracle.run(rp, col, dense, 2, 64, 5, 0.02, quirks=True)
    algo = de.EmbeddingAlgo(rp, col, dense, 0.0, 0.25, 5, -5, False, False)
    loss = algo.algo_force2_vec_ns(2, 64, 5, 0.02)
    assert loss.shape == (2,)
    assert rel_l2(dense, want) <= RUN_REL_L2


@pytest.mark.parametrize("dim,ns", [(32, 5), (64, 8), (128, 5), (256, 7)])
def test_staged_negatives_bitwise_equal(dim, ns):
    # negatives copied into shared memory (bulk asynchronous copies) or read from
    # L1/L2: the same pairs in the same order, so the same bits
    n, rp, col = gg.rmat_csr(12, 8, seed=27)
    x0 = f32(gg.init_embedding(n, dim, seed=15))
    out = []
    for stage in (False, True):
        with de.Handle(rp, col, dim, stage_negatives=stage, edge_cap=16) as h:
            h.set_embeddings(x0)
            loss = h.run(3, 300, ns, 0.03)
            out.append((h.get_embeddings(), loss))
    assert np.array_equal(out[0][0], out[1][0]) and np.array_equal(out[0][1], out[1][1])
