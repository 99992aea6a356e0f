"""Writes tests/golden/*.npz from the reference's own code.

Run here, where the reference sources exist:
    make -C oracle ref && python tests/golden/make_golden.py

Every output comes from oracle/_ref/libderef.so, i.e. the reference's
EmbeddingAlgo (cpp/algo/algo.hpp), SpMMAlgo (cpp/algo/spmm.hpp), sampler (cpp/core/common.cpp:37-53) and CSR
builder (cpp/core/csr_local.hpp) compiled unmodified against single-rank
stand-ins for MPI/MKL/Eigen.  The FP64 restatement in oracle/ is then checked
against these files bit for bit (tests/test_oracle_golden.py).
"""
from __future__ import annotations

import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402
from distembed_gb300 import graphgen as gg  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))


def hand_graph():
    """18 vertices: a hub, a chain, an isolated vertex (7), duplicate-free,
    several edges into the last vertex (17), one self-loop (5)."""
    e = [(0, j) for j in range(1, 12)] + [(12, 13), (13, 14), (14, 15), (15, 16), (16, 17),
                                          (3, 17), (9, 17), (5, 5), (2, 4)]
    s = [a for a, b in e] + [b for a, b in e if a != b]
    d = [b for a, b in e] + [a for a, b in e if a != b]
    return 18, *gg.coo_to_csr(18, np.array(s), np.array(d))


def cases():
    n, rp, col = gg.knn_csr(300, 8, 5, 4, seed=300)
    yield "knn300_d16_driver", rp, col, gg.init_embedding(n, 16, 1), dict(E=3, B=64, ns=5, lr=[0.02] * 3, driver=True)
    n, rp, col = gg.knn_csr(517, 8, 6, 4, seed=517)
    yield "knn517_d32_decay", rp, col, gg.init_embedding(n, 32, 2), dict(E=3, B=100, ns=7, lr=[0.02 * (1 - e / 3) for e in range(3)], driver=False)
    n, rp, col = gg.rmat_csr(9, 8, seed=5)
    yield "rmat9_d64_driver", rp, col, gg.init_embedding(n, 64, 3), dict(E=2, B=96, ns=5, lr=[0.05] * 2, driver=True)
    n, rp, col = hand_graph()
    yield "hand18_d32", rp, col, gg.init_embedding(n, 32, 4), dict(E=4, B=5, ns=3, lr=[0.1] * 4, driver=True)
    n, rp, col = gg.knn_csr(50, 4, 3, 2, seed=50)
    yield "single_batch_d128", rp, col, gg.init_embedding(n, 128, 5), dict(E=2, B=64, ns=5, lr=[0.02, 0.01], driver=False)


def main():
    assert oracle.ref_available(), "build the reference harness first: make -C oracle ref"
    for name, rp, col, x0, p in cases():
        n = len(rp) - 1
        x1 = oracle.ref_run(rp, col, x0, p["E"], p["B"], p["ns"], np.array(p["lr"]), driver_loop=p["driver"])
        assert x1 is not None, f"{name}: a negative draw hits the reference's undefined path"
        np.savez_compressed(os.path.join(OUT, f"run_{name}.npz"), rowptr=rp, col=col, x0=x0, x1=x1,
                            epochs=p["E"], batch=p["B"], ns=p["ns"], lr=np.array(p["lr"]))
        print(name, n, len(col), x0.shape)
    # one minibatch's update before it is applied (prevCoordinates)
    n, rp, col = gg.knn_csr(300, 8, 5, 4, seed=300)
    x = gg.init_embedding(n, 64, 6)
    grads = {}
    for (b, seed, cons) in [(0, 0, 64), (2, 7, 64), (4, 9, 44), (1, 11, 44)]:
        g = oracle.ref_batch_grad(rp, col, x, 64, 5, 0.02, b, seed, cons)
        assert g is not None
        grads[f"b{b}_s{seed}_c{cons}"] = g
    np.savez_compressed(os.path.join(OUT, "grad_knn300_d64.npz"), rowptr=rp, col=col, x=x, batch=64, ns=5,
                        lr=0.02, **grads)
    # the sampler
    rng = {}
    rng["u60000_s1234_k10"] = oracle.ref_negatives(0, 60000, 1234, 10)
    for upper, ns in [(20000, 5), (1 << 20, 5), (1 << 22, 1024), (17, 3), (1, 8), (0, 4)]:
        rng[f"u{upper}_k{ns}"] = np.stack([oracle.ref_negatives(0, upper, s, ns) for s in range(0, 40)])
    np.savez_compressed(os.path.join(OUT, "negatives.npz"), **rng)
    # the CSR builder: unsorted COO in, CSR out
    r = np.array([3, 0, 2, 0, 3, 1, 0, 3], dtype=np.int64)
    c = np.array([1, 2, 0, 1, 0, 3, 3, 2], dtype=np.int64)
    rp, cc = oracle.ref_csr(4, r, c)
    np.savez_compressed(os.path.join(OUT, "csr_small.npz"), coo_row=r, coo_col=c, rowptr=rp, col=cc)
    write_spmm()
    write_sparse()
    print("done")


def write_spmm():
    """The reference's SpMM step (SpMMAlgo::algo_spmm, cpp/algo/spmm.hpp:54-159)."""
    n, rp, col = hand_graph()
    x = gg.init_embedding(n, 32, 7)
    np.savez_compressed(os.path.join(OUT, "spmm_hand18_d32.npz"), rowptr=rp, col=col, x=x, batch=5, lr=0.1,
                        y=oracle.ref_spmm(rp, col, x, 5, 0.1))
    n, rp, col = gg.rmat_csr(9, 8, seed=5)
    x = gg.init_embedding(n, 16, 8)
    np.savez_compressed(os.path.join(OUT, "spmm_rmat9_d16.npz"), rowptr=rp, col=col, x=x, batch=96, lr=0.02,
                        y=oracle.ref_spmm(rp, col, x, 96, 0.02))



def write_sparse():
    """The reference's sparse embedding at one rank (SparseEmbedding::algo_sparse_embedding,
    cpp/algo/sparse_embedding.hpp:78-194): the one-rank branch (merge 0) and the
    local steps of the multi-rank branch (merge 1)."""
    cases = [("sparse_hand18_d16_q", hand_graph(), 16, dict(iterations=3, batch=5, ns=3, lr=0.1, density=0.5,
                                                                merge=0)),
             ("sparse_rmat9_d16_m", gg.rmat_csr(9, 8, seed=6), 16, dict(iterations=4, batch=100, ns=5, lr=0.1,
                                                                          density=0.5, merge=1))]
    for name, (n, rp, col), dim, kw in cases:
        x = gg.init_embedding(n, dim, 9)
        xo, coll = oracle.ref_sparse_embedding(rp, col, x, kw["iterations"], kw["batch"], kw["ns"], kw["lr"],
                                               kw["density"], bool(kw["merge"]))
        np.savez_compressed(os.path.join(OUT, f"{name}.npz"), rowptr=rp, col=col, x=x, x_out=xo, coll=coll, **kw)


if __name__ == "__main__":
    main()
