"""CPU oracle for the force-model SGD embedding step.

TEST INFRASTRUCTURE ONLY: imported by tests/, by __graft_entry__.smoke() as the
checker and by bench.py's CPU legs.  The product (distembed_gb300) never
imports it.

Three libraries live here:
  liboracle.so       the FP64 restatement (de_oracle.cpp), built anywhere g++ exists;
                     bit-exact with the reference (no fused multiply-add)
  liboracle_fast.so  the same source built -O3 with contraction: the timed CPU
                     baseline (FP64, not bit-exact)
  _ref/libderef.so   the reference's own code compiled against oracle/shim/; it can
                     only be built where the reference sources are (see Makefile)
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = None
_FAST = None
_REF = None

_i64p = ctypes.POINTER(ctypes.c_int64)
_f64p = ctypes.POINTER(ctypes.c_double)


def _p(a, t=ctypes.c_void_p):
    return ctypes.cast(a.ctypes.data, t) if a is not None else None


def build(ref: bool = False) -> None:
    """Compile liboracle.so (and the reference harness when ref=True)."""
    subprocess.check_call(["make", "-s", "-C", HERE] + (["all", "ref"] if ref else ["all"]))


def lib():
    global _LIB
    if _LIB is None:
        _LIB = _load("liboracle.so")
    return _LIB


def lib_fast():
    """The -O3 build of the same restatement (the timed CPU baseline)."""
    global _FAST
    if _FAST is None:
        _FAST = _load("liboracle_fast.so")
    return _FAST


def _load(name):
    path = os.path.join(HERE, name)
    src = os.path.join(HERE, "de_oracle.cpp")
    if not os.path.exists(path) or os.path.getmtime(src) > os.path.getmtime(path):
        build()
    L = ctypes.CDLL(path)
    L.oracle_negatives.argtypes = [ctypes.c_int64, ctypes.c_int, ctypes.c_int, _i64p]
    L.oracle_rep_rows.argtypes = [ctypes.c_int64, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int]
    L.oracle_batch_grad.argtypes = [ctypes.c_int64, _i64p, _i64p, ctypes.c_int, _f64p, ctypes.c_int,
                                    ctypes.c_int, ctypes.c_double, ctypes.c_int, ctypes.c_int,
                                    ctypes.c_int, ctypes.c_int, _f64p, _f64p]
    L.oracle_run.argtypes = [ctypes.c_int64, _i64p, _i64p, ctypes.c_int, _f64p, ctypes.c_int,
                             ctypes.c_int, ctypes.c_int, _f64p, ctypes.c_int, _f64p, ctypes.c_int]
    L.oracle_run_batches.argtypes = [ctypes.c_int64, _i64p, _i64p, ctypes.c_int, _f64p, ctypes.c_int,
                                     ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_int,
                                     ctypes.POINTER(ctypes.c_int32), ctypes.c_int, ctypes.c_int]
    L.oracle_run_batches.restype = ctypes.c_int64
    L.oracle_spmm.argtypes = [ctypes.c_int64, _i64p, _i64p, ctypes.c_int, _f64p, ctypes.c_double, ctypes.c_int,
                              _f64p]
    L.oracle_sparse_embedding.argtypes = [ctypes.c_int, ctypes.c_int64, _i64p, _i64p, _f64p, ctypes.c_int,
                                          ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_double,
                                          ctypes.c_int, ctypes.c_int, _f64p]
    L.oracle_run_many.argtypes = [ctypes.c_int, _i64p, ctypes.POINTER(_i64p), ctypes.POINTER(_i64p), ctypes.c_int,
                                  ctypes.POINTER(_f64p), ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                  _f64p, ctypes.c_int, _f64p, ctypes.c_int]
    L.oracle_run_many.restype = ctypes.c_int64
    return L


_GPU = None


def lib_gpu():
    """The FP64 GPU restatement (liboracle_gpu.so, built by `make -C oracle gpu`)."""
    global _GPU
    if _GPU is None:
        path = os.path.join(HERE, "liboracle_gpu.so")
        src = os.path.join(HERE, "de_oracle_gpu.cu")
        if not os.path.exists(path) or os.path.getmtime(src) > os.path.getmtime(path):
            subprocess.check_call(["make", "-s", "-C", HERE, "gpu"])
        L = ctypes.CDLL(path)
        L.oracle_gpu_run.argtypes = [ctypes.c_int64, _i64p, _i64p, ctypes.c_int, _f64p, ctypes.c_int, ctypes.c_int,
                                     ctypes.c_int, _f64p, ctypes.c_int, _f64p, ctypes.c_int]
        _GPU = L
    return _GPU


def gpu_run(rowptr, col, x, epochs, batch, ns, lr, quirks=True, device=0):
    """oracle.run on the GPU in FP64 (the same arithmetic in the same order, so
    the embedding is bitwise oracle.run's): returns (x_new, loss_per_epoch)."""
    rowptr, col = _csr(rowptr, col)
    x = np.array(x, dtype=np.float64, order="C", copy=True)
    n, dim = x.shape
    lrs = np.ascontiguousarray(np.broadcast_to(np.asarray(lr, dtype=np.float64), (max(epochs, 1),)))
    loss = np.zeros(max(epochs, 1), dtype=np.float64)
    rc = lib_gpu().oracle_gpu_run(n, _p(rowptr, _i64p), _p(col, _i64p), dim, _p(x, _f64p), epochs, batch, ns,
                                  _p(lrs, _f64p), int(quirks), _p(loss, _f64p), device)
    if rc != 0:
        raise ValueError(f"oracle_gpu_run failed ({rc})")
    return x, loss[:epochs]


def ref_path() -> str:
    return os.path.join(HERE, "_ref", "libderef.so")


def ref_available() -> bool:
    return os.path.exists(ref_path())


def ref():
    """The reference's own code (shim-compiled); raises if it was not built here."""
    global _REF
    if _REF is None:
        L = ctypes.CDLL(ref_path())
        L.deref_run.argtypes = [ctypes.c_int, ctypes.c_int64, ctypes.c_int64, _i64p, _i64p, _f64p,
                                ctypes.c_int, ctypes.c_int, ctypes.c_int, _f64p, ctypes.c_int, ctypes.c_int]
        L.deref_batch_grad.argtypes = [ctypes.c_int, ctypes.c_int64, ctypes.c_int64, _i64p, _i64p, _f64p,
                                       ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_int,
                                       ctypes.c_int, ctypes.c_int, _f64p]
        L.deref_negatives.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                      ctypes.POINTER(ctypes.c_uint64)]
        L.deref_csr.argtypes = [ctypes.c_int64, ctypes.c_int64, _i64p, _i64p, _i64p, _i64p]
        L.deref_spmm.argtypes = [ctypes.c_int, ctypes.c_int64, ctypes.c_int64, _i64p, _i64p, _f64p, ctypes.c_int,
                                 ctypes.c_double, _f64p]
        L.deref_sparse_embedding.argtypes = [ctypes.c_int, ctypes.c_int64, ctypes.c_int64, _i64p, _i64p, _f64p,
                                             ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_double,
                                             ctypes.c_double, ctypes.c_int, _f64p]
        _REF = L
    return _REF


def _csr(rowptr, col):
    return (np.ascontiguousarray(rowptr, dtype=np.int64), np.ascontiguousarray(col, dtype=np.int64))


# ---------------------------------------------------------------- restatement

def negatives(n: int, seed: int, ns: int) -> np.ndarray:
    out = np.zeros(max(ns, 1), dtype=np.int64)
    lib().oracle_negatives(n, seed, ns, _p(out, _i64p))
    return out[:ns]


def rep_rows(n: int, batch: int, epoch_in_call: int, batch_id: int, quirks: bool) -> int:
    return lib().oracle_rep_rows(n, batch, epoch_in_call, batch_id, int(quirks))


def batch_grad(rowptr, col, x, batch, ns, lr, batch_id, seed, rep, quirks=True):
    """One minibatch's update before it is applied; returns (prev[batch, dim], row_loss[batch])."""
    rowptr, col = _csr(rowptr, col)
    x = np.ascontiguousarray(x, dtype=np.float64)
    n, dim = x.shape
    prev = np.zeros((batch, dim), dtype=np.float64)
    rl = np.zeros(batch, dtype=np.float64)
    rc = lib().oracle_batch_grad(n, _p(rowptr, _i64p), _p(col, _i64p), dim, _p(x, _f64p), batch, ns, lr,
                                 batch_id, seed, rep, int(quirks), _p(prev, _f64p), _p(rl, _f64p))
    if rc != 0:
        raise ValueError(f"oracle_batch_grad failed ({rc})")
    return prev, rl


def run(rowptr, col, x, epochs, batch, ns, lr, quirks=True, threads=0, want_loss=True, fast=False):
    """Runs `epochs` epochs; returns (x_new, loss_per_epoch or None).  lr: scalar or
    per-epoch array.  fast: the -O3 build (the timed CPU baseline)."""
    rowptr, col = _csr(rowptr, col)
    x = np.array(x, dtype=np.float64, order="C", copy=True)
    n, dim = x.shape
    lrs = np.ascontiguousarray(np.broadcast_to(np.asarray(lr, dtype=np.float64), (max(epochs, 1),)))
    loss = np.zeros(max(epochs, 1), dtype=np.float64) if want_loss else None
    rc = (lib_fast() if fast else lib()).oracle_run(n, _p(rowptr, _i64p), _p(col, _i64p), dim, _p(x, _f64p), epochs,
                                                    batch, ns, _p(lrs, _f64p), int(quirks), _p(loss, _f64p), threads)
    if rc != 0:
        raise ValueError(f"oracle_run failed ({rc})")
    return x, (loss[:epochs] if want_loss else None)


def run_many(graphs, xs, epochs, batch, ns, lr, first_epoch=0, quirks=True, want_loss=True, threads=0,
             fast=False):
    """Many independent graphs, each one job of the one-rank step, spread over
    `threads` host threads (one graph per thread at a time).  graphs: a list of
    (rowptr, col); xs: their FP64 embeddings (n x dim, C-contiguous), updated in
    place; epochs [first_epoch, first_epoch + epochs) with one lr per epoch.
    Returns (edge-updates, loss [graphs, epochs] or None).  fast: the -O3 build
    (the timed baseline) instead of the bit-exact one."""
    L = lib_fast() if fast else lib()
    csr = [_csr(rp, c) for rp, c in graphs]
    for x in xs:
        assert x.dtype == np.float64 and x.flags.c_contiguous
    G = len(graphs)
    dim = xs[0].shape[1]
    n = np.array([len(rp) - 1 for rp, _ in csr], dtype=np.int64)
    rps = (_i64p * G)(*[_p(rp, _i64p) for rp, _ in csr])
    cols = (_i64p * G)(*[_p(c, _i64p) for _, c in csr])
    xps = (_f64p * G)(*[_p(x, _f64p) for x in xs])
    lrs = np.ascontiguousarray(np.broadcast_to(np.asarray(lr, dtype=np.float64), (max(epochs, 1),)))
    loss = np.zeros((G, max(epochs, 1)), dtype=np.float64) if want_loss else None
    u = L.oracle_run_many(G, _p(n, _i64p), rps, cols, dim, xps, first_epoch, epochs, batch, ns, _p(lrs, _f64p),
                          int(quirks), _p(loss, _f64p), threads)
    if u < 0:
        raise ValueError("oracle_run_many failed")
    return int(u), (loss[:, :epochs] if want_loss else None)


def spmm(rowptr, col, x, lr, quirks=True):
    """The reference's SpMM step (cpp/algo/spmm.hpp:54-159): y = lr * A x, FP64."""
    rowptr, col = _csr(rowptr, col)
    x = np.ascontiguousarray(x, dtype=np.float64)
    n, dim = x.shape
    y = np.zeros((n, dim), dtype=np.float64)
    rc = lib().oracle_spmm(n, _p(rowptr, _i64p), _p(col, _i64p), dim, _p(x, _f64p), lr, int(quirks), _p(y, _f64p))
    if rc != 0:
        raise ValueError(f"oracle_spmm failed ({rc})")
    return y


def run_batches(rowptr, col, x, epoch_in_call, batch, ns, lr, batch_ids, quirks=True, threads=0, fast=False):
    """Runs the listed minibatches of one epoch in place on x (FP64, C-contiguous);
    returns the edge-updates performed.  Used for bounded CPU timing samples
    (fast: the -O3 build)."""
    ids = np.ascontiguousarray(batch_ids, dtype=np.int32)
    n, dim = x.shape
    assert x.dtype == np.float64 and x.flags.c_contiguous
    u = (lib_fast() if fast else lib()).oracle_run_batches(n, _p(rowptr, _i64p), _p(col, _i64p), dim, _p(x, _f64p), epoch_in_call, batch,
                                 ns, lr, int(quirks), _p(ids, ctypes.POINTER(ctypes.c_int32)), len(ids), threads)
    if u < 0:
        raise ValueError("oracle_run_batches failed")
    return int(u)


# ------------------------------------------------------ the reference's code

def ref_negatives(lower: int, upper: int, seed: int, ns: int) -> np.ndarray:
    out = np.zeros(max(ns, 1), dtype=np.uint64)
    ref().deref_negatives(lower, upper, seed, ns, _p(out, ctypes.POINTER(ctypes.c_uint64)))
    return out[:ns]


def ref_run(rowptr, col, x, epochs, batch, ns, lr, driver_loop=False, col_major=False):
    """The reference's EmbeddingAlgo (FP64, its quirks included; col_major as its
    constructor flag).  Returns x_new, or None when a negative draw would hit the
    reference's undefined path."""
    rowptr, col = _csr(rowptr, col)
    x = np.array(x, dtype=np.float64, order="C", copy=True)
    n, dim = x.shape
    lrs = np.ascontiguousarray(np.broadcast_to(np.asarray(lr, dtype=np.float64), (max(epochs, 1),)))
    rc = ref().deref_run(dim, n, len(col), _p(rowptr, _i64p), _p(col, _i64p), _p(x, _f64p), epochs,
                         batch, ns, _p(lrs, _f64p), int(driver_loop), int(col_major))
    if rc == -2:
        return None
    if rc != 0:
        raise ValueError(f"deref_run failed ({rc})")
    return x


ABSENT = float(-2 ** 31)  # INT_MIN: an absent entry of a sparse embedding row


def sparse_embedding(rowptr, col, x, iterations, batch, ns, lr, density, merge=False, quirks=True):
    """The reference's sparse embedding at one rank (cpp/algo/sparse_embedding.hpp:
    78-194), FP64: returns (x after the run, batch collector [batch, dim])."""
    rowptr, col = _csr(rowptr, col)
    x = np.array(x, dtype=np.float64, order="C")
    n, dim = x.shape
    coll = np.zeros((batch, dim), dtype=np.float64)
    rc = lib().oracle_sparse_embedding(dim, n, _p(rowptr, _i64p), _p(col, _i64p), _p(x, _f64p), iterations, batch,
                                       ns, lr, density, int(merge), int(quirks), _p(coll, _f64p))
    if rc != 0:
        raise ValueError(f"oracle_sparse_embedding failed ({rc})")
    return x, coll


def ref_sparse_embedding(rowptr, col, x, iterations, batch, ns, lr, density, merge=False):
    """The reference's own SparseEmbedding at one rank (FP64): (x, batch collector)."""
    rowptr, col = _csr(rowptr, col)
    x = np.array(x, dtype=np.float64, order="C")
    n, dim = x.shape
    coll = np.zeros((batch, dim), dtype=np.float64)
    rc = ref().deref_sparse_embedding(dim, n, len(col), _p(rowptr, _i64p), _p(col, _i64p), _p(x, _f64p), iterations,
                                      batch, ns, lr, density, int(merge), _p(coll, _f64p))
    if rc != 0:
        raise ValueError(f"deref_sparse_embedding failed ({rc})")
    return x, coll


def ref_spmm(rowptr, col, x, batch, lr):
    """The reference's own SpMMAlgo::algo_spmm(1, batch, lr) (FP64): y."""
    rowptr, col = _csr(rowptr, col)
    x = np.ascontiguousarray(x, dtype=np.float64)
    n, dim = x.shape
    y = np.zeros((n, dim), dtype=np.float64)
    rc = ref().deref_spmm(dim, n, len(col), _p(rowptr, _i64p), _p(col, _i64p), _p(x, _f64p), batch, lr,
                          _p(y, _f64p))
    if rc != 0:
        raise ValueError(f"deref_spmm failed ({rc})")
    return y


def ref_batch_grad(rowptr, col, x, batch, ns, lr, batch_id, seed, considering):
    rowptr, col = _csr(rowptr, col)
    x = np.ascontiguousarray(x, dtype=np.float64)
    n, dim = x.shape
    prev = np.zeros((batch, dim), dtype=np.float64)
    rc = ref().deref_batch_grad(dim, n, len(col), _p(rowptr, _i64p), _p(col, _i64p), _p(x, _f64p), batch,
                                ns, lr, batch_id, seed, considering, _p(prev, _f64p))
    if rc == -2:
        return None
    if rc != 0:
        raise ValueError(f"deref_batch_grad failed ({rc})")
    return prev


def ref_csr(n, coo_row, coo_col):
    coo_row = np.ascontiguousarray(coo_row, dtype=np.int64)
    coo_col = np.ascontiguousarray(coo_col, dtype=np.int64)
    rowptr = np.zeros(n + 1, dtype=np.int64)
    col = np.zeros(max(len(coo_col), 1), dtype=np.int64)
    ref().deref_csr(n, len(coo_col), _p(coo_row, _i64p), _p(coo_col, _i64p), _p(rowptr, _i64p), _p(col, _i64p))
    return rowptr, col[:len(coo_col)]
