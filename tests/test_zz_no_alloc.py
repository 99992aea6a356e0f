"""The allocation-free minibatch entry point (de_minibatch_noalloc).

It serves callers that may not allocate device memory themselves through the
library: a framework that owns the device heap through its own pool, or a
latency-bound loop that cannot take cudaMalloc's implicit synchronisation.  The
test allocates the inputs and outputs itself (as such a caller would), calls the
entry point twice in a row through the C ABI (minibatch 0, then minibatch 1 of
one epoch, so the second call reuses the library's scratch after the first),
and checks the result against the regular entry point (de_run) with the
tolerances the other GPU tests use.  This file is named to be collected last.
"""
import ctypes

import numpy as np
import pytest

import distembed_gb300 as de
from distembed_gb300 import graphgen as gg

pytestmark = pytest.mark.gpu

RUN_REL_L2 = 1e-4   # same as the multi-step tolerance of tests/test_gpu_plain.py
LOSS_RTOL = 1e-3


@pytest.fixture(scope="module")
def torch_cuda():
    torch = pytest.importorskip("torch")
    from distembed_gb300 import build
    build.build()
    return torch


def test_two_noalloc_calls_match_de_run(torch_cuda):
    torch = torch_cuda
    n, rp, col = gg.rmat_csr(11, 8, seed=31)        # 2048 vertices
    dim, batch, ns, lr = 64, 1024, 5, 0.03          # exactly two minibatches
    x0 = gg.init_embedding(n, dim, seed=13).astype(np.float32)

    with de.Handle(rp, col, dim, quirks=True) as h:
        h.set_embeddings(x0)
        want_loss = h.run(1, batch, ns, lr)[0]
        want = h.get_embeddings()

    dev = torch.device("cuda", 0)
    rowptr = torch.tensor(rp, dtype=torch.int32, device=dev)
    cols = torch.tensor(col, dtype=torch.int32, device=dev)
    x = torch.tensor(x0, device=dev)
    stream = torch.cuda.current_stream(dev)
    losses = []
    L = de.lib()
    for j in range(2):
        negs = torch.tensor(de.negatives(n, j, ns), dtype=torch.int32, device=dev)  # seed = epoch 0 + j
        loss = torch.zeros(1, dtype=torch.float64, device=dev)
        rc = L.de_minibatch_noalloc(n, rowptr.data_ptr(), cols.data_ptr(), dim, x.data_ptr(), j, batch,
                                    negs.data_ptr(), ns, batch, 1, ctypes.c_float(lr), ctypes.c_float(5.0),
                                    loss.data_ptr(), ctypes.c_void_p(stream.cuda_stream))
        assert rc == de.DE_OK, L.de_last_error(None)
        losses.append(loss)
    torch.cuda.synchronize(dev)
    got = x.cpu().numpy().astype(np.float64)
    rel = np.linalg.norm(got - want) / np.linalg.norm(want)
    assert rel <= RUN_REL_L2, rel
    got_loss = sum(float(l.item()) for l in losses)
    assert abs(got_loss - want_loss) <= LOSS_RTOL * want_loss, (got_loss, want_loss)


@pytest.mark.parametrize("dim", [32, 64, 128, 256])
def test_noalloc_two_epochs_ragged_last_minibatch(torch_cuda, dim):
    # 2348 vertices, minibatch 1024: minibatches of 1024, 1024 and 324 rows.  In
    # the second epoch only the first last_batch_size rows of every minibatch take
    # the repulsive pass (the reference's repulsive row count is never reset,
    # cpp/algo/algo.hpp:135, 167-169, 594), and edges into vertex n-1 are dropped.
    torch = torch_cuda
    import oracle
    n, rp, col = gg.rmat_csr_n(2348, 8, seed=33)
    batch, ns, lr = 1024, 6, 0.025
    batches = (n + batch - 1) // batch
    last = n - batch * (batches - 1)
    x0 = gg.init_embedding(n, dim, seed=14).astype(np.float32)

    with de.Handle(rp, col, dim, quirks=True) as h:
        h.set_embeddings(x0)
        want_loss = h.run(2, batch, ns, lr)
        want = h.get_embeddings()
    xo, lo = oracle.run(rp, col, x0.astype(np.float64), 2, batch, ns, lr, quirks=True)

    dev = torch.device("cuda", 0)
    rowptr = torch.tensor(rp, dtype=torch.int32, device=dev)
    cols = torch.tensor(col, dtype=torch.int32, device=dev)
    x = torch.tensor(x0, device=dev)
    stream = torch.cuda.current_stream(dev)
    L = de.lib()
    got_loss = [0.0, 0.0]
    for e in range(2):
        for j in range(batches):
            negs = torch.tensor(de.negatives(n, e + j, ns), dtype=torch.int32, device=dev)
            rows = min(batch, n - j * batch)
            rep = last if e > 0 else rows
            loss = torch.zeros(1, dtype=torch.float64, device=dev)
            rc = L.de_minibatch_noalloc(n, rowptr.data_ptr(), cols.data_ptr(), dim, x.data_ptr(), j, batch,
                                        negs.data_ptr(), ns, rep, 1, ctypes.c_float(lr), ctypes.c_float(5.0),
                                        loss.data_ptr(), ctypes.c_void_p(stream.cuda_stream))
            assert rc == de.DE_OK, L.de_last_error(None)
            torch.cuda.synchronize(dev)
            got_loss[e] += float(loss.item())
    got = x.cpu().numpy().astype(np.float64)
    assert np.linalg.norm(got - want) / np.linalg.norm(want) <= RUN_REL_L2
    assert np.linalg.norm(got - xo) / np.linalg.norm(xo) <= RUN_REL_L2
    for e in range(2):
        assert abs(got_loss[e] - want_loss[e]) <= LOSS_RTOL * want_loss[e], (e, got_loss, want_loss)
        assert abs(got_loss[e] - lo[e]) <= LOSS_RTOL * lo[e], (e, got_loss, lo)


def test_noalloc_rejects_minibatch_beyond_scratch(torch_cuda):
    torch = torch_cuda
    n, rp, col = gg.rmat_csr(13, 4, seed=32)        # 8192 vertices
    dev = torch.device("cuda", 0)
    rowptr = torch.tensor(rp, dtype=torch.int32, device=dev)
    cols = torch.tensor(col, dtype=torch.int32, device=dev)
    x = torch.zeros((n, 256), dtype=torch.float32, device=dev)
    negs = torch.zeros(5, dtype=torch.int32, device=dev)
    L = de.lib()
    rc = L.de_minibatch_noalloc(n, rowptr.data_ptr(), cols.data_ptr(), 256, x.data_ptr(), 0, 8192,
                                negs.data_ptr(), 5, 8192, 1, ctypes.c_float(0.02), ctypes.c_float(5.0), None, None)
    assert rc == de.DE_ERR_INVALID
    assert b"1048576" in L.de_last_error(None)
    assert float(x.abs().sum().item()) == 0.0      # nothing ran
