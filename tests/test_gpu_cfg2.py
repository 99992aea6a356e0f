"""The plain form's at-scale workload, whole job, against the FP64 oracle.

R-MAT scale 20 (1,048,576 vertices, edge factor 16, a=.57 b=.19 c=.19, seed 1,
symmetrised, duplicates and self-loops removed), dim 128, minibatch 4096, 5
shared negatives per minibatch, lr 0.02, 10 epochs, U[-0.5, 0.5] start (seed 0)
rounded to FP32 for both sides.

Tolerances (FP32 GPU against the FP64 oracle): every epoch's loss within 1e-3
relative, the final embedding within 1e-4 relative L2.
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
    with de.Handle(rp, col, 128) as h:
        h.set_embeddings(x0)
        lg = h.run(E, B, ns, lr)
        xg = h.get_embeddings()
    xo, lo = oracle.run(rp, col, x0, E, B, ns, lr, quirks=True, threads=os.cpu_count() or 1)
    gap = np.abs(lg - lo) / lo
    assert np.all(gap <= 1e-3), gap
    err = np.linalg.norm(xg - xo) / np.linalg.norm(xo)
    assert err <= 1e-4, err
