"""Served form (de_server_*): concurrent jobs, admission by memory and slots,
and every job's result identical to the same job run alone.

Tolerances: a served job runs the same kernels as a resident handle, so its
embedding and loss are compared bitwise with the job run alone through
de_create/de_run (FP32 plain and BF16 forms); against the FP64 oracle the FP32
plain tolerance applies (||x - x_oracle|| / ||x_oracle|| <= 1e-4).
"""
import time

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


def make_jobs():
    jobs = []
    specs = [("knn", 700, 32, 4, "fp32"), ("rmat", 1500, 64, 3, "fp32"), ("rmat", 4096, 128, 2, "fp32"),
             ("knn", 2500, 64, 5, "bf16"), ("rmat", 900, 32, 6, "fp32"), ("knn", 1200, 128, 3, "bf16"),
             ("rmat", 3000, 64, 4, "fp32"), ("knn", 400, 64, 2, "fp32")]
    for i, (kind, n, dim, epochs, prec) in enumerate(specs):
        if kind == "knn":
            n, rp, col = gg.knn_csr(n, 16, 8, 5, seed=60 + i)
        else:
            n, rp, col = gg.rmat_csr_n(n, 8, seed=60 + i)
        x0 = gg.init_embedding(n, dim, seed=70 + i).astype(np.float32)
        batch = 128 if n < 1000 else 512
        jobs.append(dict(rowptr=rp, col=col, x0=x0, epochs=epochs, batch=batch, ns=5 if prec == "fp32" else 64,
                         lr=[0.02 * (1 - e / (epochs + 1)) for e in range(epochs)], precision=prec))
    return jobs


JOBS = make_jobs()


def alone(j):
    with de.Handle(j["rowptr"], j["col"], j["x0"].shape[1], precision=j["precision"]) as h:
        h.set_embeddings(j["x0"])
        loss = h.run(j["epochs"], j["batch"], j["ns"], j["lr"])
        return h.get_embeddings(dtype=np.float32), loss


def submit(srv, j):
    return srv.submit(j["rowptr"], j["col"], j["x0"], j["epochs"], j["batch"], j["ns"], j["lr"], j["precision"])


def test_every_job_in_the_mix_equals_the_job_alone():
    with de.Server(slots=8, hbm_bytes=2 << 30) as srv:
        ids = [submit(srv, j) for j in JOBS]
        got = [srv.wait(i) for i in ids]
        st = srv.stats()
    assert st["done"] == len(JOBS) and st["failed"] == 0 and st["peak_running"] >= 2
    for j, (x, loss, info) in zip(JOBS, got):
        xa, la = alone(j)
        assert np.array_equal(x, xa), j["precision"]
        assert np.array_equal(loss, la)
        assert info["state"] == "done" and info["submit_s"] <= info["start_s"] <= info["end_s"]


def test_served_job_matches_oracle():
    j = JOBS[1]
    with de.Server(slots=2, hbm_bytes=1 << 30) as srv:
        x, loss, info = srv.wait(submit(srv, j))
    xo, lo = oracle.run(j["rowptr"], j["col"], j["x0"].astype(np.float64), j["epochs"], j["batch"], j["ns"], j["lr"])
    assert np.linalg.norm(x - xo) / np.linalg.norm(xo) <= 1e-4
    assert np.all(np.abs(loss - lo) <= 1e-3 * lo)
    with de.Handle(j["rowptr"], j["col"], 64) as h:
        assert info["edge_updates"] == h.edge_updates(j["epochs"], j["batch"], j["ns"])


def test_admission_respects_memory_budget_and_slots():
    budget = 48 << 20
    with de.Server(slots=6, hbm_bytes=budget) as srv:
        ids = [submit(srv, JOBS[i % len(JOBS)]) for i in range(16)]
        infos = [srv.wait(i)[2] for i in ids]
        st = srv.stats()
    assert st["done"] == 16 and st["peak_reserved_bytes"] <= budget and st["peak_running"] <= 6
    big = max(infos, key=lambda d: d["device_bytes"])["device_bytes"]
    assert big < budget
    # a job larger than the whole budget is refused at submission
    n, rp, col = gg.rmat_csr(14, 8, seed=3)
    with de.Server(slots=2, hbm_bytes=4 << 20) as srv:
        with pytest.raises(de.DEError) as ei:
            srv.submit(rp, col, np.zeros((n, 128), np.float32), 2, 1024, 5, 0.02)
        assert ei.value.code == de.DE_ERR_UNSUPPORTED


def test_job_arriving_while_another_runs_overlaps_it():
    n, rp, col = gg.rmat_csr(16, 16, seed=8)
    long_job = dict(rowptr=rp, col=col, x0=gg.init_embedding(n, 128, seed=1).astype(np.float32), epochs=30,
                    batch=256, ns=5, lr=0.02, precision="fp32")
    with de.Server(slots=4, hbm_bytes=2 << 30) as srv:
        a = submit(srv, long_job)
        time.sleep(0.02)
        later = [submit(srv, JOBS[i]) for i in (0, 4, 7)]
        res_later = [srv.wait(i)[2] for i in later]
        res_a = srv.wait(a)[2]
    # the short jobs were admitted and finished while the long one was running
    assert all(r["start_s"] < res_a["end_s"] and r["end_s"] < res_a["end_s"] for r in res_later), (res_a, res_later)
