"""The CPU-runnable workload at full size against the FP64 oracle, every epoch.

20,000 points of a 10-component isotropic Gaussian mixture in 64-D (seed 0,
component means ~N(0, 4I), unit variance), symmetrised exact kNN (k=15);
dim 128, U[-0.5, 0.5] start (seed 0), minibatch 256, 5 negatives, learning rate
0.02 (1 - e/30), 30 epochs.

Tolerances (FP32 GPU against FP64 oracle from the same FP32-rounded start):
per-epoch loss within 1e-3 (relative) over the whole run; the final embedding
within 1e-3 relative L2.
"""
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


def test_knn20k_thirty_epochs_against_oracle():
    n, rp, col = gg.knn_csr(20000, 64, 15, 10, seed=0)
    x0 = gg.init_embedding(n, 128, seed=0).astype(np.float32).astype(np.float64)
    E, B, ns = 30, 256, 5
    lr = [0.02 * (1 - e / E) for e in range(E)]
    with de.Handle(rp, col, 128) as h:
        h.set_embeddings(x0)
        lg = h.run(E, B, ns, lr)
        xg = h.get_embeddings()
        updates = h.edge_updates(E, B, ns)
    xo, lo = oracle.run(rp, col, x0, E, B, ns, lr, quirks=True)
    gap = np.abs(lg - lo) / lo
    assert np.all(gap <= 1e-3), gap
    assert np.linalg.norm(xg - xo) / np.linalg.norm(xo) <= 1e-3
    assert updates > 30 * len(col)
