"""The FP64 GPU restatement (oracle/de_oracle_gpu.cu) against the CPU oracle.

The GPU restatement is the checker for the BF16 precision form at R-MAT scale 22
(dim 256, 1024 negatives per minibatch), a size the CPU oracle cannot finish.  It
does the CPU oracle's arithmetic in the same order without fused multiply-adds,
so the embeddings must be bitwise equal; the loss uses the GPU's FP64 log and is
held to 1e-12 relative.
"""
import numpy as np
import pytest

import oracle
from distembed_gb300 import graphgen as gg

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("dim,ns,batch,quirks", [(32, 5, 100, True), (256, 64, 256, True), (128, 7, 300, False),
                                                 (256, 1024, 512, True)])
def test_gpu_fp64_oracle_bitwise(dim, ns, batch, quirks):
    n, rp, col = gg.rmat_csr_n(1500, 8, seed=41)     # 1500 vertices: ragged last minibatch
    x0 = gg.init_embedding(n, dim, seed=42)
    lr = [0.03, 0.02, 0.01]
    xc, lc = oracle.run(rp, col, x0, 3, batch, ns, lr, quirks=quirks)
    xg, lg = oracle.gpu_run(rp, col, x0, 3, batch, ns, lr, quirks=quirks)
    assert np.array_equal(xc, xg)
    assert np.all(np.abs(lg - lc) <= 1e-12 * lc), (lg, lc)


def test_gpu_fp64_oracle_knn_with_edges_into_last_vertex():
    n, rp, col = gg.knn_csr(700, 8, 6, 4, seed=43)
    x0 = gg.init_embedding(n, 64, seed=44)
    assert np.any(col == n - 1)
    xc, lc = oracle.run(rp, col, x0, 2, 128, 5, 0.02, quirks=True)
    xg, lg = oracle.gpu_run(rp, col, x0, 2, 128, 5, 0.02, quirks=True)
    assert np.array_equal(xc, xg)
    assert np.all(np.abs(lg - lc) <= 1e-12 * lc)
