"""Batched form (many graphs in one persistent launch) against the FP64 oracle,
through the C ABI.

Each graph of a batch must train exactly as if it ran alone through the
reference's one-rank step (its own sampler seeds, its own minibatch order).

Tolerances:
  FP32 storage   ||x_gpu - x_oracle||_2 / ||x_oracle||_2 <= 1e-4 per graph after
                 several epochs; per-epoch loss within 1e-3 (relative)
  BF16 storage   per-epoch loss within 1% of the FP64 oracle's (FP32 master and
                 accumulation, every read BF16)
  alone vs mix   bitwise equal, for one team shape: a graph's arithmetic does not
                 depend on which team runs it or what else is in the batch
"""
import numpy as np
import pytest

import distembed_gb300 as de
import oracle
from distembed_gb300 import graphgen as gg

pytestmark = pytest.mark.gpu

RUN_REL_L2 = 1e-4
LOSS_RTOL = 1e-3
BF16_LOSS_GAP = 1e-2


@pytest.fixture(scope="module", autouse=True)
def _built():
    from distembed_gb300 import build
    build.build()


def f32(x):
    return np.asarray(x, dtype=np.float32).astype(np.float64)


def rel_l2(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def suite():
    """Small graphs of both kinds: sizes below, at and above the minibatch, a
    partial last minibatch, hub rows longer than every edge cap tried."""
    gs = [(k, n, rp, c) for k, n, rp, c in gg.graph_suite(6, 150, 2500, seed=11)]
    n, rp, c = gg.rmat_csr_n(97, 8, seed=5)        # smaller than one minibatch
    gs.append(("rmat", n, rp, c))
    n, rp, c = gg.rmat_csr(10, 16, seed=6)         # hubs of several hundred entries
    gs.append(("rmat", n, rp, c))
    return gs


GRAPHS = suite()


def x_init(i, n, dim):
    return f32(gg.init_embedding(n, dim, seed=100 + i))


REG = dict(kernel="register", vertices_per_warp=4, team_warps=8, edge_cap=32)
STAGED = dict(kernel="staged", team_warps=8, edge_cap=32, pairs=2, stages=3)
ROWS = dict(kernel="rows", team_warps=4, edge_cap=16, pairs=2, stages=3)
CLUSTER = dict(kernel="staged", team_warps=8, edge_cap=16, pairs=2, stages=3, team_ctas=2)


def run_batch(graphs, dim, epochs, batch, ns, lr, precision="fp32", shape=None, ids=None):
    ids = list(range(len(graphs))) if ids is None else ids
    with de.Batch([(rp, c) for _, _, rp, c in graphs], dim, precision=precision) as b:
        if shape:
            b.set_shape(**shape)
        for j, (i, (_, n, _, _)) in enumerate(zip(ids, graphs)):
            b.set_embeddings(j, x_init(i, n, dim))
        loss = b.run(epochs, batch, ns, lr)
        return [b.get_embeddings(j).astype(np.float64) for j in range(len(graphs))], loss


@pytest.mark.parametrize("kernel", ["register", "staged", "rows"])
@pytest.mark.parametrize("dim", [32, 64, 128])
def test_fp32_batch_matches_oracle_per_graph(dim, kernel):
    E, B, ns = 3, 256, 5
    lr = [0.02 * (1 - e / E) for e in range(E)]
    if kernel == "register":
        shape = REG
    elif kernel == "staged":
        shape = STAGED if dim < 128 else dict(STAGED, team_warps=4, edge_cap=16)
    else:
        shape = ROWS if dim < 128 else dict(ROWS, team_warps=2, edge_cap=16)
    xs, loss = run_batch(GRAPHS, dim, E, B, ns, lr, shape=shape)
    for i, (kind, n, rp, c) in enumerate(GRAPHS):
        xo, lo = oracle.run(rp, c, x_init(i, n, dim), E, B, ns, lr, quirks=True)
        assert rel_l2(xs[i], xo) <= RUN_REL_L2, (i, kind, n)
        assert np.all(np.abs(loss[i] - lo) <= LOSS_RTOL * lo), (i, loss[i], lo)


SHAPES = [dict(kernel="register", vertices_per_warp=1, team_warps=4, edge_cap=32),
          dict(kernel="register", vertices_per_warp=2, team_warps=8, edge_cap=8),
          dict(kernel="register", vertices_per_warp=4, team_warps=16, edge_cap=64),
          dict(kernel="register", vertices_per_warp=4, team_warps=8, edge_cap=4096),
          dict(kernel="register", vertices_per_warp=2, team_warps=32, edge_cap=128),
          dict(kernel="staged", team_warps=4, edge_cap=8, pairs=1, stages=3),
          dict(kernel="staged", team_warps=16, edge_cap=8, pairs=2, stages=3),
          dict(kernel="staged", team_warps=8, edge_cap=16, pairs=2, stages=4),
          dict(kernel="staged", team_warps=8, edge_cap=32, pairs=2, stages=3),
          dict(kernel="staged", team_warps=2, edge_cap=1, pairs=1, stages=4),
          dict(kernel="rows", team_warps=4, edge_cap=16, pairs=1, stages=3),
          dict(kernel="rows", team_warps=4, edge_cap=8, pairs=2, stages=4),
          dict(kernel="rows", team_warps=2, edge_cap=32, pairs=2, stages=3),
          dict(kernel="rows", team_warps=3, edge_cap=1, pairs=1, stages=4),
          CLUSTER, dict(CLUSTER, team_warps=4, edge_cap=8, pairs=1, stages=4), dict(CLUSTER, team_ctas=4)]


@pytest.mark.parametrize("shape", SHAPES, ids=lambda s: "-".join(str(v) for v in s.values()))
def test_every_team_shape_matches_oracle(shape):
    dim, E, B, ns = 64, 2, 128, 7
    xs, loss = run_batch(GRAPHS, dim, E, B, ns, 0.03, shape=shape)
    for i, (kind, n, rp, c) in enumerate(GRAPHS):
        xo, lo = oracle.run(rp, c, x_init(i, n, dim), E, B, ns, 0.03, quirks=True)
        assert rel_l2(xs[i], xo) <= RUN_REL_L2, (shape, i, kind, n)
        assert np.all(np.abs(loss[i] - lo) <= LOSS_RTOL * lo), (shape, i)


@pytest.mark.parametrize("shape", [REG, STAGED, ROWS, CLUSTER], ids=["register", "staged", "rows", "cluster"])
@pytest.mark.parametrize("precision", ["fp32", "bf16"])
def test_alone_equals_mix_bitwise(precision, shape):
    dim, E, B, ns = 64, 3, 256, 5
    xs, loss = run_batch(GRAPHS, dim, E, B, ns, 0.02, precision=precision, shape=shape)
    for i in (0, 3, len(GRAPHS) - 1):
        xa, la = run_batch([GRAPHS[i]], dim, E, B, ns, 0.02, precision=precision, shape=shape, ids=[i])
        assert np.array_equal(xa[0], xs[i]), i
        assert np.array_equal(la[0], loss[i]), i
    # the mix in another order gives the same per-graph results
    perm = [5, 2, 7, 0, 6, 1, 4, 3]
    xp, lp = run_batch([GRAPHS[i] for i in perm], dim, E, B, ns, 0.02, precision=precision, shape=shape,
                       ids=perm)
    for j, i in enumerate(perm):
        assert np.array_equal(xp[j], xs[i]) and np.array_equal(lp[j], loss[i]), i


@pytest.mark.parametrize("shape", [REG, STAGED, ROWS], ids=["register", "staged", "rows"])
def test_bf16_batch_loss_within_one_percent(shape):
    dim, E, B, ns = 64, 4, 256, 5
    _, loss = run_batch(GRAPHS, dim, E, B, ns, 0.02, precision="bf16", shape=shape)
    for i, (kind, n, rp, c) in enumerate(GRAPHS):
        x0 = x_init(i, n, dim)
        # the BF16 form starts from the BF16 rounding of the FP32 embedding
        u = np.asarray(x0, dtype=np.float32).view(np.uint32).astype(np.uint64)
        x0b = ((u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000).astype(np.uint32).view(np.float32)
        _, lo = oracle.run(rp, c, x0b.astype(np.float64), E, B, ns, 0.02, quirks=True)
        gap = np.abs(loss[i] - lo) / lo
        assert np.all(gap <= BF16_LOSS_GAP), (i, kind, loss[i], lo)


def test_autotune_keeps_embeddings_and_picks_a_valid_shape():
    dim, B, ns = 64, 256, 5
    graphs = GRAPHS[:4]
    with de.Batch([(rp, c) for _, _, rp, c in graphs], dim) as b:
        for i, (_, n, _, _) in enumerate(graphs):
            b.set_embeddings(i, x_init(i, n, dim))
        best, tried = b.autotune(1, B, ns, 0.02)
        assert len(tried) >= 36 and all(ms > 0 for _, ms in tried)
        assert any(sh["team_ctas"] == 2 for sh, _ in tried)
        assert {sh["kernel"] for sh, _ in tried} == {0, 1, 2}
        assert best == min(tried, key=lambda t: t[1])[0] == b.shape()
        for i, (_, n, _, _) in enumerate(graphs):
            assert np.array_equal(b.get_embeddings(i).astype(np.float64), x_init(i, n, dim))
        loss = b.run(2, B, ns, 0.02)
        got = [b.get_embeddings(i).astype(np.float64) for i in range(len(graphs))]
    shape = dict(best)
    shape["kernel"] = int(shape["kernel"])
    xs, ls = run_batch(graphs, dim, 2, B, ns, 0.02, shape=shape)
    for i in range(len(graphs)):
        assert np.array_equal(got[i], xs[i]) and np.array_equal(loss[i], ls[i])


def test_autotune_with_more_negatives_than_the_staged_kernels_take():
    # ns > 32: only the register kernel's shapes are timed
    dim, B, ns = 32, 128, 40
    graphs = GRAPHS[:3]
    with de.Batch([(rp, c) for _, _, rp, c in graphs], dim) as b:
        for i, (_, n, _, _) in enumerate(graphs):
            b.set_embeddings(i, x_init(i, n, dim))
        best, tried = b.autotune(1, B, ns, 0.02)
        assert tried and {sh["kernel"] for sh, _ in tried} == {0} and best["kernel"] == 0


def test_edge_updates_is_the_sum_over_graphs():
    dim, E, B, ns = 32, 3, 256, 5
    with de.Batch([(rp, c) for _, _, rp, c in GRAPHS], dim) as b:
        total = b.edge_updates(E, B, ns)
    want = 0
    for _, n, rp, c in GRAPHS:
        with de.Handle(rp, c, dim) as h:
            want += h.edge_updates(E, B, ns)
    assert total == want


def test_run_twice_continues_from_the_first():
    # two calls of one epoch each = the oracle's two separate one-epoch calls
    dim, B, ns = 64, 256, 5
    graphs = GRAPHS[:3]
    with de.Batch([(rp, c) for _, _, rp, c in graphs], dim) as b:
        for i, (_, n, _, _) in enumerate(graphs):
            b.set_embeddings(i, x_init(i, n, dim))
        b.run(1, B, ns, 0.02)
        b.run(1, B, ns, 0.02)
        got = [b.get_embeddings(i).astype(np.float64) for i in range(len(graphs))]
    for i, (_, n, rp, c) in enumerate(graphs):
        x1, _ = oracle.run(rp, c, x_init(i, n, dim), 1, B, ns, 0.02, quirks=True)
        x2, _ = oracle.run(rp, c, x1, 1, B, ns, 0.02, quirks=True)
        assert rel_l2(got[i], x2) <= RUN_REL_L2


def test_prepared_launch_replays_the_same_run():
    dim, B, ns = 64, 256, 5
    graphs = GRAPHS[:3]
    with de.Batch([(rp, c) for _, _, rp, c in graphs], dim) as b:
        for i, (_, n, _, _) in enumerate(graphs):
            b.set_embeddings(i, x_init(i, n, dim))
        b.prepare(1, B, ns, 0.02)
        b.launch()
        b.launch()
        b.wait()
        got = [b.get_embeddings(i).astype(np.float64) for i in range(len(graphs))]
        b.run(1, B, ns, 0.02)
        again = [b.get_embeddings(i).astype(np.float64) for i in range(len(graphs))]
    for i, (_, n, rp, c) in enumerate(graphs):
        x1, _ = oracle.run(rp, c, x_init(i, n, dim), 1, B, ns, 0.02, quirks=True)
        x2, _ = oracle.run(rp, c, x1, 1, B, ns, 0.02, quirks=True)
        x3, _ = oracle.run(rp, c, x2, 1, B, ns, 0.02, quirks=True)
        assert rel_l2(got[i], x2) <= RUN_REL_L2
        assert rel_l2(again[i], x3) <= RUN_REL_L2


def test_staged_rejects_more_than_32_negatives():
    with de.Batch([(rp, c) for _, _, rp, c in GRAPHS[:2]], 64) as b:
        b.set_shape(**STAGED)
        with pytest.raises(de.DEError) as ei:
            b.run(1, 256, 33, 0.02)
        assert ei.value.code == de.DE_ERR_UNSUPPORTED


@pytest.mark.parametrize("shape", [REG, STAGED, ROWS, CLUSTER], ids=["register", "staged", "rows", "cluster"])
def test_hub_rows_and_many_chunks_per_warp(shape):
    # one graph whose minibatches hold far more than 32 chunks per warp (hub rows
    # split into cap-sized pieces), so the staged pipeline restarts within a minibatch
    n, rp, c = gg.rmat_csr(11, 32, seed=9)
    g = [("rmat", n, rp, c)]
    sh = dict(shape, edge_cap=4, team_warps=2) if shape["kernel"] != "register" else dict(shape, edge_cap=4)
    xs, loss = run_batch(g, 32, 2, 512, 6, 0.02, shape=sh, ids=[50])
    xo, lo = oracle.run(rp, c, x_init(50, n, 32), 2, 512, 6, 0.02, quirks=True)
    assert rel_l2(xs[0], xo) <= RUN_REL_L2
    assert np.all(np.abs(loss[0] - lo) <= LOSS_RTOL * lo)


@pytest.mark.parametrize("ctas", [2, 4])
def test_cluster_teams_match_single_cta_teams_bitwise(ctas):
    # the largest graphs of a mix go to teams of two or four CTAs of a cluster;
    # every graph's result is the same as with one CTA per graph (same items, same
    # order of every sum)
    dim, E, B, ns = 64, 3, 256, 5
    one = dict(CLUSTER, team_ctas=1)
    xs1, l1 = run_batch(GRAPHS, dim, E, B, ns, 0.02, precision="bf16", shape=one)
    xs2, l2 = run_batch(GRAPHS, dim, E, B, ns, 0.02, precision="bf16", shape=dict(CLUSTER, team_ctas=ctas))
    for i in range(len(GRAPHS)):
        assert np.array_equal(xs1[i], xs2[i]) and np.array_equal(l1[i], l2[i]), i
