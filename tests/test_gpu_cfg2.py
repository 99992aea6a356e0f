"""The plain form's at-scale workload, whole job, against the FP64 oracle.

R-MAT scale 20 (1,048,576 vertices, edge factor 16, a=.57 b=.19 c=.19, seed 1,
symmetrised, duplicates and self-loops removed), dim 128, minibatch 4096, 5
shared negatives per minibatch, lr 0.02, 10 epochs, U[-0.5, 0.5] start (seed 0)
rounded to FP32 for both sides.

Tolerances (FP32 GPU against the FP64 oracle):
  after the first epoch (256 minibatches) the embedding within 1e-5 relative L2;
  every epoch's loss within 1e-3 relative over the whole run;
  the embedding after 10 epochs within 1e-3 relative L2: FP32 and FP64 runs part
  slowly on this graph (1.8e-4 after 10 epochs, the loss within 3e-6), as they
  do on the 30-epoch kNN workload, which holds the same 1e-3.
"""
import os

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


def test_rmat20_ten_epochs_against_oracle():
    n, rp, col = gg.rmat_csr(20, 16, seed=1)
    x0 = gg.init_embedding(n, 128, seed=0).astype(np.float32).astype(np.float64)
    E, B, ns, lr = 10, 4096, 5, 0.02
    threads = os.cpu_count() or 1
    with de.Handle(rp, col, 128) as h:
        h.set_embeddings(x0)
        h.run(1, B, ns, lr)
        x1 = h.get_embeddings()
        h.set_embeddings(x0)
        lg = h.run(E, B, ns, lr)
        xg = h.get_embeddings()
    xo1, _ = oracle.run(rp, col, x0, 1, B, ns, lr, quirks=True, threads=threads)
    err1 = np.linalg.norm(x1 - xo1) / np.linalg.norm(xo1)
    assert err1 <= 1e-5, err1
    xo, lo = oracle.run(rp, col, x0, E, B, ns, lr, quirks=True, threads=threads)
    gap = np.abs(lg - lo) / lo
    assert np.all(gap <= 1e-3), gap
    err = np.linalg.norm(xg - xo) / np.linalg.norm(xo)
    assert err <= 1e-3, err
