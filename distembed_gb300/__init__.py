"""distembed_gb300 — GB300 (sm_103a) force-model SGD graph embedding.

Python mirror of DistEmbed's embedding interface over the C ABI in
include/distembed_gb300.h (libdistembed_gb300.so, built in-tree by
distembed_gb300.build).  Nothing here computes: every call goes to the CUDA
library, and a missing library is an error, never a fallback.

    EmbeddingAlgo   the reference's algo class (cpp/algo/algo.hpp:54-74):
                    construct on a CSR and a dense FP64 embedding, then
                    algo_force2_vec_ns(iterations, batch_size, ns, lr)
                    updates the embedding in place
    Handle          the resident-graph handle (de_create / de_run / ...)
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libdistembed_gb300.so")

DE_OK = 0
DE_ERR_INVALID = -1
DE_ERR_OOM = -2
DE_ERR_CUDA = -3
DE_ERR_STATE = -4
DE_ERR_UNSUPPORTED = -5
PRECISION = {"fp32": 0, "bf16": 1}

# Every entry point include/distembed_gb300.h declares.
EXPORTS = ("de_default_options", "de_create", "de_destroy", "de_set_embeddings", "de_get_embeddings",
           "de_set_embeddings_f32", "de_get_embeddings_f32", "de_run", "de_run_from", "de_profile_epoch", "de_sync",
           "de_edge_updates",
           "de_negatives", "de_minibatch_noalloc", "de_stream", "de_last_error", "de_version",
           "de_batch_create", "de_batch_destroy", "de_batch_set_embeddings_f32", "de_batch_get_embeddings_f32",
           "de_batch_set_shape", "de_batch_get_shape", "de_batch_prepare", "de_batch_launch", "de_batch_wait", "de_batch_run", "de_batch_autotune", "de_batch_edge_updates", "de_batch_set_near_distance", "de_batch_set_loss", "de_batch_trace", "de_batch_stream",
           "de_batch_last_error", "de_server_create", "de_server_submit", "de_server_info", "de_server_wait",
           "de_server_drain", "de_server_get_stats", "de_server_clock", "de_server_destroy", "de_server_last_error",
           "de_mm_read", "de_embedding_write", "de_mm_read_gpu", "de_coo_to_csr", "de_csr_info", "de_csr_copy",
           "de_csr_free", "de_spmm", "de_spmm_f32", "de_sparse_embedding", "de_sparse_set", "de_sparse_run",
           "de_sparse_get")


class BatchShape(ctypes.Structure):
    _fields_ = [("kernel", ctypes.c_int32), ("vertices_per_warp", ctypes.c_int32), ("team_warps", ctypes.c_int32),
                ("edge_cap", ctypes.c_int32), ("pairs", ctypes.c_int32), ("stages", ctypes.c_int32),
                ("team_ctas", ctypes.c_int32)]

    def as_dict(self):
        return {k: int(getattr(self, k)) for k, _ in self._fields_}


BATCH_KERNEL = {"register": 0, "staged": 1, "rows": 2}


class JobSpec(ctypes.Structure):
    _fields_ = [("n", ctypes.c_int64), ("rowptr", ctypes.c_void_p), ("col", ctypes.c_void_p), ("nnz", ctypes.c_int64),
                ("dim", ctypes.c_int32), ("precision", ctypes.c_int32), ("epochs", ctypes.c_int32),
                ("batch_size", ctypes.c_int32), ("ns", ctypes.c_int32), ("pad", ctypes.c_int32),
                ("lr_per_epoch", ctypes.c_void_p), ("x0", ctypes.c_void_p), ("x_out", ctypes.c_void_p),
                ("loss_out", ctypes.c_void_p)]


class JobInfo(ctypes.Structure):
    _fields_ = [("state", ctypes.c_int32), ("pad", ctypes.c_int32), ("submit_s", ctypes.c_double),
                ("start_s", ctypes.c_double), ("end_s", ctypes.c_double), ("device_bytes", ctypes.c_int64),
                ("edge_updates", ctypes.c_int64)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_ if k != "pad"}


class ServerStats(ctypes.Structure):
    _fields_ = [(k, ctypes.c_int64) for k in ("submitted", "done", "failed", "queued", "running", "peak_running",
                                              "budget_bytes", "reserved_bytes", "peak_reserved_bytes")]

    def as_dict(self):
        return {k: int(getattr(self, k)) for k, _ in self._fields_}


JOB_STATE = {0: "queued", 1: "running", 2: "done", 3: "failed"}


class DEError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"[{code}] {msg}")
        self.code = code


class Options(ctypes.Structure):
    _fields_ = [("precision", ctypes.c_int32), ("ref_quirks", ctypes.c_int32), ("compute_loss", ctypes.c_int32),
                ("device", ctypes.c_int32), ("stream", ctypes.c_void_p), ("max_bound", ctypes.c_double),
                ("edge_cap", ctypes.c_int32), ("pdl", ctypes.c_int32), ("stage_negatives", ctypes.c_int32),
                ("reserved", ctypes.c_int32 * 5)]


_lib = None
_vp = ctypes.c_void_p
_i32, _i64 = ctypes.c_int32, ctypes.c_int64


def lib():
    """The loaded CUDA library.  Raises if it has not been built."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(f"{LIB_PATH} is missing: run `python -m distembed_gb300.build`")
        L = ctypes.CDLL(LIB_PATH)
        L.de_default_options.argtypes = [ctypes.POINTER(Options)]
        L.de_default_options.restype = None
        L.de_create.argtypes = [_i64, _vp, _vp, _i64, _i32, ctypes.POINTER(Options), ctypes.POINTER(_vp)]
        L.de_destroy.argtypes = [_vp]
        L.de_set_embeddings.argtypes = [_vp, _vp]
        L.de_get_embeddings.argtypes = [_vp, _vp]
        L.de_set_embeddings_f32.argtypes = [_vp, _vp, _i32]
        L.de_get_embeddings_f32.argtypes = [_vp, _vp, _i32]
        L.de_run.argtypes = [_vp, _i32, _i32, _i32, _vp, _vp]
        L.de_run_from.argtypes = [_vp, _i32, _i32, _i32, _i32, _vp, _vp]
        L.de_profile_epoch.argtypes = [_vp, _i32, _i32, _i32, ctypes.c_double, _vp, _vp, _i32, _vp]
        L.de_sync.argtypes = [_vp]
        L.de_edge_updates.argtypes = [_vp, _i32, _i32, _i32, _i32]
        L.de_edge_updates.restype = _i64
        L.de_negatives.argtypes = [_i64, _i32, _i32, _vp]
        L.de_negatives.restype = None
        L.de_minibatch_noalloc.argtypes = [_i64, _vp, _vp, _i32, _vp, _i32, _i32, _vp, _i32, _i32, _i32,
                                           ctypes.c_float, ctypes.c_float, _vp, _vp]
        L.de_stream.argtypes = [_vp]
        L.de_stream.restype = _vp
        L.de_last_error.argtypes = [_vp]
        L.de_last_error.restype = ctypes.c_char_p
        L.de_version.restype = ctypes.c_char_p
        L.de_batch_create.argtypes = [_i32, _vp, _vp, _vp, _i32, ctypes.POINTER(Options), ctypes.POINTER(_vp)]
        L.de_batch_destroy.argtypes = [_vp]
        L.de_batch_set_embeddings_f32.argtypes = [_vp, _i32, _vp]
        L.de_batch_get_embeddings_f32.argtypes = [_vp, _i32, _vp]
        L.de_batch_set_shape.argtypes = [_vp, ctypes.POINTER(BatchShape)]
        L.de_batch_get_shape.argtypes = [_vp, ctypes.POINTER(BatchShape)]
        L.de_batch_run.argtypes = [_vp, _i32, _i32, _i32, _vp, _vp]
        L.de_batch_prepare.argtypes = [_vp, _i32, _i32, _i32, _vp]
        L.de_batch_launch.argtypes = [_vp]
        L.de_batch_wait.argtypes = [_vp, _vp]
        L.de_batch_autotune.argtypes = [_vp, _i32, _i32, _i32, ctypes.c_double, _vp, _vp, _i32, _vp,
                                        ctypes.POINTER(BatchShape)]
        L.de_batch_edge_updates.argtypes = [_vp, _i32, _i32, _i32]
        L.de_batch_edge_updates.restype = _i64
        L.de_batch_set_near_distance.argtypes = [_vp, ctypes.c_float]
        L.de_batch_set_loss.argtypes = [_vp, _i32]
        L.de_batch_trace.argtypes = [_vp, _vp]
        L.de_batch_stream.argtypes = [_vp]
        L.de_batch_stream.restype = _vp
        L.de_batch_last_error.argtypes = [_vp]
        L.de_batch_last_error.restype = ctypes.c_char_p
        L.de_server_create.argtypes = [_i32, _i32, _i64, ctypes.c_double, _i32, ctypes.POINTER(_vp)]
        L.de_server_submit.argtypes = [_vp, ctypes.POINTER(JobSpec), ctypes.POINTER(_i64)]
        L.de_server_info.argtypes = [_vp, _i64, ctypes.POINTER(JobInfo)]
        L.de_server_wait.argtypes = [_vp, _i64, ctypes.POINTER(JobInfo)]
        L.de_server_drain.argtypes = [_vp]
        L.de_server_get_stats.argtypes = [_vp, ctypes.POINTER(ServerStats)]
        L.de_server_clock.argtypes = [_vp]
        L.de_server_clock.restype = ctypes.c_double
        L.de_server_destroy.argtypes = [_vp]
        L.de_server_last_error.argtypes = [_vp]
        L.de_server_last_error.restype = ctypes.c_char_p
        L.de_mm_read.argtypes = [ctypes.c_char_p, _vp, _vp, _vp, _vp, _vp, _i64]
        L.de_embedding_write.argtypes = [ctypes.c_char_p, _vp, _i64, _i32]
        L.de_mm_read_gpu.argtypes = [ctypes.c_char_p, _i32, _vp]
        L.de_spmm.argtypes = [_vp, _i32, ctypes.c_double, _vp]
        L.de_spmm_f32.argtypes = [_vp, _i32, ctypes.c_float, _vp, _i32]
        L.de_sparse_embedding.argtypes = [_vp, _vp, _i32, _i32, _i32, ctypes.c_double, ctypes.c_double, _i32, _vp]
        L.de_sparse_set.argtypes = [_vp, _vp]
        L.de_sparse_run.argtypes = [_vp, _i32, _i32, _i32, ctypes.c_double, ctypes.c_double, _i32]
        L.de_sparse_get.argtypes = [_vp, _vp, _vp]
        L.de_coo_to_csr.argtypes = [_i64, _i64, _vp, _vp, _i64, _i32, _i32, _vp]
        L.de_csr_info.argtypes = [_vp, _vp, _vp, _vp]
        L.de_csr_copy.argtypes = [_vp, _vp, _vp]
        L.de_csr_free.argtypes = [_vp]
        L.de_csr_free.restype = None
        _lib = L
    return _lib


def _ptr(a) -> int:
    if hasattr(a, "data_ptr"):
        return a.data_ptr()
    return a.ctypes.data


DRIVER_PATH = os.path.join(HERE, "dist_embed_gb300")


def _take_csr(L, rc, h):
    if rc != DE_OK:
        raise DEError(rc, L.de_last_error(None).decode())
    try:
        r, c, z = _i64(0), _i64(0), _i64(0)
        L.de_csr_info(h, ctypes.byref(r), ctypes.byref(c), ctypes.byref(z))
        rowptr = np.zeros(r.value + 1, dtype=np.int64)
        col = np.zeros(max(z.value, 1), dtype=np.int64)
        L.de_csr_copy(h, rowptr.ctypes.data, col.ctypes.data)
        return r.value, c.value, rowptr, col[: z.value]
    finally:
        L.de_csr_free(h)


def coo_to_csr(rows: int, cols: int, row_idx, col_idx, mirror: bool = False, device: int = 0):
    """COO -> (rows, cols, rowptr, col) int64 CSR on the GPU: duplicates merged,
    columns ascending, mirrored off-diagonal entries added when mirror."""
    L = lib()
    ri = np.ascontiguousarray(row_idx, dtype=np.int64)
    ci = np.ascontiguousarray(col_idx, dtype=np.int64)
    h = _vp()
    rc = L.de_coo_to_csr(rows, cols, ri.ctypes.data, ci.ctypes.data, len(ri), int(mirror), device, ctypes.byref(h))
    return _take_csr(L, rc, h)


def read_mtx(path: str, gpu: bool = False, device: int = 0):
    """MatrixMarket -> (rows, cols, rowptr, col) int64 CSR, by the library's
    reader (cpp/io/parrallel_IO.hpp:31-88 semantics at one rank); gpu: the
    COO -> CSR on GPU `device`."""
    L = lib()
    if gpu:
        h = _vp()
        rc = L.de_mm_read_gpu(path.encode(), device, ctypes.byref(h))
        return _take_csr(L, rc, h)
    r, c, z = _i64(0), _i64(0), _i64(0)
    rc = L.de_mm_read(path.encode(), ctypes.byref(r), ctypes.byref(c), ctypes.byref(z), None, None, 0)
    if rc != DE_OK:
        raise DEError(rc, L.de_last_error(None).decode())
    rowptr = np.zeros(r.value + 1, dtype=np.int64)
    col = np.zeros(max(z.value, 1), dtype=np.int64)
    rc = L.de_mm_read(path.encode(), ctypes.byref(r), ctypes.byref(c), ctypes.byref(z), rowptr.ctypes.data,
                      col.ctypes.data, len(col))
    if rc != DE_OK:
        raise DEError(rc, L.de_last_error(None).decode())
    return r.value, c.value, rowptr, col[: z.value]


def write_embedding(path: str, x) -> None:
    """The reference's embedding file (cpp/io/parrallel_IO.hpp:90-146)."""
    x = np.ascontiguousarray(x, dtype=np.float64)
    rc = lib().de_embedding_write(path.encode(), x.ctypes.data, x.shape[0], x.shape[1])
    if rc != DE_OK:
        raise DEError(rc, lib().de_last_error(None).decode())


def negatives(n: int, seed: int, ns: int) -> np.ndarray:
    """The reference's sampler (cpp/core/common.cpp:37-53), computed by the library."""
    out = np.zeros(max(ns, 1), dtype=np.int64)
    lib().de_negatives(n, seed, ns, out.ctypes.data)
    return out[:ns]


class Handle:
    """One graph resident on one GPU, with its embedding."""

    def __init__(self, rowptr, col, dim: int, precision: str = "fp32", quirks: bool = True,
                 compute_loss: bool = True, device: int = 0, stream: int | None = None,
                 max_bound: float = 5.0, edge_cap: int = 0, pdl: bool = True, stage_negatives: bool = False):
        L = lib()
        self._rowptr = np.ascontiguousarray(rowptr, dtype=np.int64)
        self._col = np.ascontiguousarray(col, dtype=np.int64)
        self.n = len(self._rowptr) - 1
        self.nnz = len(self._col)
        self.dim = dim
        o = Options()
        L.de_default_options(ctypes.byref(o))
        o.precision = PRECISION[precision]
        o.ref_quirks = int(quirks)
        o.compute_loss = int(compute_loss)
        o.device = device
        o.stream = stream
        o.max_bound = max_bound
        o.edge_cap = edge_cap
        o.pdl = int(pdl)
        o.stage_negatives = int(stage_negatives)
        h = _vp()
        rc = L.de_create(self.n, self._rowptr.ctypes.data, self._col.ctypes.data if self.nnz else None, self.nnz,
                         dim, ctypes.byref(o), ctypes.byref(h))
        if rc != DE_OK:
            raise DEError(rc, L.de_last_error(None).decode())
        self._h = h

    def _check(self, rc: int):
        if rc != DE_OK:
            raise DEError(rc, lib().de_last_error(self._h).decode())

    @property
    def stream(self) -> int:
        return lib().de_stream(self._h)

    def set_embeddings(self, x):
        """x: host FP64 (n, dim) array, host FP32 array, or a CUDA FP32 tensor."""
        if hasattr(x, "is_cuda") and x.is_cuda:
            assert x.dtype.__str__() == "torch.float32" and x.is_contiguous()
            self._check(lib().de_set_embeddings_f32(self._h, x.data_ptr(), 1))
        elif hasattr(x, "dtype") and str(x.dtype) in ("float32", "torch.float32"):
            x = x if hasattr(x, "data_ptr") else np.ascontiguousarray(x)
            self._check(lib().de_set_embeddings_f32(self._h, _ptr(x), 0))
        else:
            x = x if hasattr(x, "data_ptr") else np.ascontiguousarray(x, dtype=np.float64)
            self._check(lib().de_set_embeddings(self._h, _ptr(x)))

    def get_embeddings(self, out=None, dtype=np.float64):
        if out is None:
            out = np.empty((self.n, self.dim), dtype=dtype)
        if hasattr(out, "is_cuda") and out.is_cuda:
            self._check(lib().de_get_embeddings_f32(self._h, out.data_ptr(), 1))
        elif str(out.dtype) in ("float32", "torch.float32"):
            self._check(lib().de_get_embeddings_f32(self._h, _ptr(out), 0))
        else:
            self._check(lib().de_get_embeddings(self._h, _ptr(out)))
        return out

    def run(self, epochs: int, batch_size: int, ns: int, lr, want_loss: bool = True, first_epoch: int = 0):
        """Runs `epochs` epochs (resumed at `first_epoch` of a call); lr is a scalar or
        one rate per epoch run.  Returns the FP64 per-epoch loss (waits for the GPU),
        or None when want_loss is False (returns once the work is queued on the
        handle's stream)."""
        lrs = np.ascontiguousarray(np.broadcast_to(np.asarray(lr, dtype=np.float64), (max(epochs, 1),)))
        loss = np.zeros(max(epochs, 1), dtype=np.float64) if want_loss else None
        self._check(lib().de_run_from(self._h, first_epoch, epochs, batch_size, ns, lrs.ctypes.data,
                                      loss.ctypes.data if want_loss else None))
        return loss[:epochs] if want_loss else None

    def sync(self):
        self._check(lib().de_sync(self._h))

    def profile_epoch(self, batch_size: int, ns: int, lr: float, first_epoch: int = 0):
        """One epoch with a CUDA event around every launch; returns (ms[], kind[])
        (kinds: 0 minibatch/attractive kernel, 1 repulsion GEMM, 2 update with exact
        pairs, 3 flush, 4 negative gather)."""
        count = ctypes.c_int32(0)
        cap = 4 * (self.n // max(batch_size, 1) + 2) + 8
        ms = np.zeros(cap, dtype=np.float32)
        kind = np.zeros(cap, dtype=np.int32)
        self._check(lib().de_profile_epoch(self._h, first_epoch, batch_size, ns, lr, ms.ctypes.data,
                                           kind.ctypes.data, cap, ctypes.byref(count)))
        return ms[:count.value], kind[:count.value]

    def edge_updates(self, epochs: int, batch_size: int, ns: int, first_epoch: int = 0) -> int:
        return int(lib().de_edge_updates(self._h, first_epoch, epochs, batch_size, ns))

    def spmm(self, batch_size: int, lr: float, out=None, dtype=np.float64):
        """The reference's SpMM step (cpp/algo/spmm.hpp:54-159): y = lr * A x from
        the current embedding x, which does not change.  out: host FP64 or FP32
        array, or a CUDA FP32 tensor."""
        if out is None:
            out = np.empty((self.n, self.dim), dtype=dtype)
        if hasattr(out, "is_cuda") and out.is_cuda:
            self._check(lib().de_spmm_f32(self._h, batch_size, lr, out.data_ptr(), 1))
        elif str(out.dtype) in ("float32", "torch.float32"):
            self._check(lib().de_spmm_f32(self._h, batch_size, lr, _ptr(out), 0))
        else:
            self._check(lib().de_spmm(self._h, batch_size, lr, out.ctypes.data))
        return out

    # INT_MIN: an absent entry of a sparse embedding row (the reference's marker)
    ABSENT = float(-2 ** 31)

    def sparse_embedding(self, x, iterations: int, batch_size: int, ns: int, lr: float, density: float,
                         merge: bool = False, inplace: bool = False, coll=None):
        """The reference's sparse embedding at one rank (SparseEmbedding::algo_sparse_embedding,
        cpp/algo/sparse_embedding.hpp:78-194) on the handle's graph.  x: FP64 n x dim rows,
        Handle.ABSENT marking an absent entry.  Returns (rows after the run with absent
        entries as 0, batch collector [batch_size, dim]).  merge=False is the reference's
        one-rank branch (the collector is never merged; the rows change only by the top-k
        pruning); merge=True merges the collector into the rows after every minibatch,
        with the repulsive pass first, as the multi-rank branch does.  inplace=True
        overwrites x (a C-contiguous FP64 array, e.g. pinned) instead of a copy; coll:
        an FP64 [batch_size, dim] array to receive the collector."""
        if inplace:
            if not (isinstance(x, np.ndarray) and x.dtype == np.float64 and x.flags.c_contiguous):
                raise ValueError("inplace needs a C-contiguous FP64 array")
            out = x
        else:
            out = np.array(x, dtype=np.float64, order="C")
        if out.shape != (self.n, self.dim):
            raise ValueError(f"x must be {self.n} x {self.dim}")
        if coll is None:
            coll = np.zeros((batch_size, self.dim), dtype=np.float64)
        elif coll.shape != (batch_size, self.dim) or coll.dtype != np.float64 or not coll.flags.c_contiguous:
            raise ValueError(f"coll must be a C-contiguous FP64 {batch_size} x {self.dim} array")
        self._check(lib().de_sparse_embedding(self._h, out.ctypes.data, iterations, batch_size, ns, lr, density,
                                              int(merge), coll.ctypes.data))
        self._sparse_batch = batch_size
        return out, coll

    def sparse_set(self, x):
        """Copy sparse embedding rows (FP64 n x dim, Handle.ABSENT = absent) in: a host
        array, or a contiguous CUDA FP64 tensor (a device-to-device copy)."""
        if hasattr(x, "is_cuda") and x.is_cuda:
            if tuple(x.shape) != (self.n, self.dim) or str(x.dtype) != "torch.float64" or not x.is_contiguous():
                raise ValueError(f"x must be a contiguous FP64 {self.n} x {self.dim} tensor")
            self._check(lib().de_sparse_set(self._h, x.data_ptr()))
            return
        x = np.ascontiguousarray(x, dtype=np.float64)
        if x.shape != (self.n, self.dim):
            raise ValueError(f"x must be {self.n} x {self.dim}")
        self._check(lib().de_sparse_set(self._h, x.ctypes.data))

    def sparse_run(self, iterations: int, batch_size: int, ns: int, lr: float, density: float,
                   merge: bool = False):
        """Enqueue a sparse embedding run on the device-resident rows (returns at once)."""
        self._check(lib().de_sparse_run(self._h, iterations, batch_size, ns, lr, density, int(merge)))
        self._sparse_batch = batch_size

    def sparse_get(self, collector: bool = True):
        """Wait for the run and return (rows, batch collector of the last run, or None)."""
        x = np.empty((self.n, self.dim), dtype=np.float64)
        batch = getattr(self, "_sparse_batch", 0)
        if collector and batch <= 0:
            raise DEError(DE_ERR_INVALID, "no batch collector: run first")
        coll = np.empty((batch, self.dim), dtype=np.float64) if collector else None
        self._check(lib().de_sparse_get(self._h, x.ctypes.data, coll.ctypes.data if coll is not None else None))
        return x, coll

    def close(self):
        if getattr(self, "_h", None):
            lib().de_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


class EmbeddingAlgo:
    """The reference's EmbeddingAlgo (cpp/algo/algo.hpp:54-74) on one GPU.

    `dense` is the FP64 (n, dim) embedding, DenseMat::nCoordinates; like the
    reference, algo_force2_vec_ns updates it in place.  The CSR is the native
    matrix's (rowStart, col_idx).  alpha, beta and sync_comm steer the
    multi-rank exchange, which a single resident partition does not have; they
    are accepted and ignored.  col_major makes the passes read the receiver
    matrix's CSR, the transpose of the native one, as the reference's loop does
    (cpp/algo/algo.hpp:131-133; at one rank it then runs the row-major pass,
    :184-186): on an asymmetric graph each row takes its attractive forces from
    its in-neighbours.
    """

    def __init__(self, rowptr, col, dense: np.ndarray, alpha: float = 0.0, beta: float = 0.25,
                 max_bound: float = 5.0, min_bound: float = -5.0, col_major: bool = False,
                 sync_comm: bool = False, *, quirks: bool = True, precision: str = "fp32",
                 device: int = 0, stream: int | None = None, compute_loss: bool = True):
        if col_major:
            from .graphgen import transpose_csr
            rowptr, col = transpose_csr(rowptr, col, dense.shape[0])
        if min_bound != -max_bound:
            raise DEError(DE_ERR_INVALID, "the reference clips to [-MAX_BOUND, MAX_BOUND]")
        if dense.dtype != np.float64 or dense.ndim != 2 or not dense.flags.c_contiguous:
            raise DEError(DE_ERR_INVALID, "dense must be a C-contiguous FP64 (n, dim) array")
        self.dense = dense
        self.handle = Handle(rowptr, col, dense.shape[1], precision=precision, quirks=quirks,
                             compute_loss=compute_loss, device=device, stream=stream, max_bound=max_bound)
        self.last_loss = None

    def algo_force2_vec_ns(self, iterations: int, batch_size: int, ns: int, lr) -> np.ndarray:
        self.handle.set_embeddings(self.dense)
        self.last_loss = self.handle.run(iterations, batch_size, ns, lr, want_loss=True)
        self.handle.get_embeddings(out=self.dense)
        return self.last_loss


class Batch:
    """Many independent graphs trained in one persistent launch (de_batch_*).

    graphs: a list of (rowptr, col) CSR pairs with local vertex ids.  Every graph
    follows the reference's one-rank step on its own, with its own sampler seeds,
    so its result does not depend on the other graphs of the batch."""

    def __init__(self, graphs, dim: int, precision: str = "fp32", quirks: bool = True, device: int = 0,
                 stream: int | None = None, max_bound: float = 5.0, edge_cap: int = 0):
        L = lib()
        self._rp = [np.ascontiguousarray(rp, dtype=np.int64) for rp, _ in graphs]
        self._col = [np.ascontiguousarray(c, dtype=np.int64) if len(c) else np.zeros(1, np.int64)
                     for _, c in graphs]
        self.n = np.array([len(rp) - 1 for rp in self._rp], dtype=np.int64)
        self.dim = dim
        o = Options()
        L.de_default_options(ctypes.byref(o))
        o.precision = PRECISION[precision]
        o.ref_quirks = int(quirks)
        o.device = device
        o.stream = stream
        o.max_bound = max_bound
        o.edge_cap = edge_cap
        rps = (ctypes.c_void_p * len(graphs))(*[a.ctypes.data for a in self._rp])
        cols = (ctypes.c_void_p * len(graphs))(*[a.ctypes.data for a in self._col])
        h = _vp()
        rc = L.de_batch_create(len(graphs), self.n.ctypes.data, rps, cols, dim, ctypes.byref(o), ctypes.byref(h))
        if rc != DE_OK:
            raise DEError(rc, L.de_batch_last_error(None).decode())
        self._h = h

    def _check(self, rc: int):
        if rc != DE_OK:
            raise DEError(rc, lib().de_batch_last_error(self._h).decode())

    @property
    def stream(self) -> int:
        return lib().de_batch_stream(self._h)

    def _rows(self, g: int) -> int:
        return int(self.n.sum()) if g < 0 else int(self.n[g])

    def set_embeddings(self, g: int, x):
        """Graph g's FP32 (n[g], dim) embedding; g = -1: all graphs concatenated."""
        x = np.ascontiguousarray(x, dtype=np.float32)
        assert x.shape == (self._rows(g), self.dim)
        self._check(lib().de_batch_set_embeddings_f32(self._h, g, x.ctypes.data))

    def get_embeddings(self, g: int, out=None) -> np.ndarray:
        if out is None:
            out = np.empty((self._rows(g), self.dim), dtype=np.float32)
        assert out.dtype == np.float32 and out.flags.c_contiguous and out.shape == (self._rows(g), self.dim)
        self._check(lib().de_batch_get_embeddings_f32(self._h, g, out.ctypes.data))
        return out

    def set_shape(self, kernel="register", vertices_per_warp=0, team_warps=8, edge_cap=32, pairs=0, stages=0,
                  team_ctas=1):
        """Team shape (see de_batch_shape); kernel "register", "staged" or "rows" (or 0 / 1 / 2)."""
        k = BATCH_KERNEL.get(kernel, kernel)
        sh = BatchShape(k, vertices_per_warp, team_warps, edge_cap, pairs, stages, team_ctas)
        self._check(lib().de_batch_set_shape(self._h, ctypes.byref(sh)))

    def shape(self) -> dict:
        sh = BatchShape()
        self._check(lib().de_batch_get_shape(self._h, ctypes.byref(sh)))
        return sh.as_dict()

    def run(self, epochs: int, batch_size: int, ns: int, lr) -> np.ndarray:
        """Trains every graph; returns the FP64 loss, shape (graphs, epochs)."""
        lrs = np.ascontiguousarray(np.broadcast_to(np.asarray(lr, dtype=np.float64), (max(epochs, 1),)))
        loss = np.zeros((len(self.n), max(epochs, 1)), dtype=np.float64)
        self._check(lib().de_batch_run(self._h, epochs, batch_size, ns, lrs.ctypes.data, loss.ctypes.data))
        return loss[:, :epochs]

    def prepare(self, epochs: int, batch_size: int, ns: int, lr):
        """Host preparation and CUDA-graph capture of one run (nothing runs)."""
        self._epochs = epochs
        lrs = np.ascontiguousarray(np.broadcast_to(np.asarray(lr, dtype=np.float64), (max(epochs, 1),)))
        self._check(lib().de_batch_prepare(self._h, epochs, batch_size, ns, lrs.ctypes.data))

    def launch(self):
        """Replays the prepared run on the batch's stream; returns at once."""
        self._check(lib().de_batch_launch(self._h))

    def wait(self) -> np.ndarray:
        """Waits; returns the (graphs, epochs) FP64 loss of the last launch."""
        loss = np.zeros((len(self.n), max(self._epochs, 1)), dtype=np.float64)
        self._check(lib().de_batch_wait(self._h, loss.ctypes.data))
        return loss[:, :self._epochs]

    def autotune(self, epochs: int, batch_size: int, ns: int, lr: float):
        """Times every team shape on `epochs` real epochs (embeddings restored) and
        keeps the fastest.  Returns (best shape dict, [(shape dict, ms), ...])."""
        cap = 256
        ms = np.zeros(cap, dtype=np.float32)
        shapes = (BatchShape * cap)()
        cnt = ctypes.c_int32(0)
        best = BatchShape()
        self._check(lib().de_batch_autotune(self._h, epochs, batch_size, ns, lr, ms.ctypes.data, shapes, cap,
                                            ctypes.byref(cnt), ctypes.byref(best)))
        return best.as_dict(), [(shapes[i].as_dict(), float(ms[i])) for i in range(cnt.value)]

    def edge_updates(self, epochs: int, batch_size: int, ns: int) -> int:
        return int(lib().de_batch_edge_updates(self._h, epochs, batch_size, ns))

    def set_near_distance(self, near_r: float):
        self._check(lib().de_batch_set_near_distance(self._h, near_r))

    def set_loss(self, mode: str):
        """"every" (default), "last" (the last epoch of each run only) or "none"."""
        self._check(lib().de_batch_set_loss(self._h, {"none": 0, "every": 1, "last": 2}[mode]))

    def trace(self) -> np.ndarray:
        """(graphs, 3): start and end (ns, from the earliest start) and team of each graph."""
        out = np.zeros((len(self.n), 3), dtype=np.int64)
        self._check(lib().de_batch_trace(self._h, out.ctypes.data))
        out[:, :2] -= out[:, 0].min()
        return out

    def close(self):
        if getattr(self, "_h", None):
            lib().de_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


class Server:
    """The served form (de_server_*): a request loop training many jobs at once.

    submit() queues a job and returns its id at once; wait(id) blocks until it is
    done and returns (embedding, per-epoch loss, info).  The arrays of a job are
    kept alive here until it has been waited for."""

    def __init__(self, slots: int = 16, hbm_bytes: int = 0, hbm_fraction: float = 0.0, device: int = 0,
                 quirks: bool = True):
        L = lib()
        h = _vp()
        rc = L.de_server_create(device, slots, hbm_bytes, hbm_fraction, int(quirks), ctypes.byref(h))
        if rc != DE_OK:
            raise DEError(rc, L.de_server_last_error(None).decode())
        self._h = h
        self._jobs = {}

    def _check(self, rc: int):
        if rc != DE_OK:
            raise DEError(rc, lib().de_server_last_error(self._h).decode())

    def clock(self) -> float:
        return lib().de_server_clock(self._h)

    def submit(self, rowptr, col, x0, epochs: int, batch_size: int, ns: int, lr, precision: str = "fp32",
               out=None) -> int:
        rowptr = np.ascontiguousarray(rowptr, dtype=np.int64)
        col = np.ascontiguousarray(col, dtype=np.int64) if len(col) else np.zeros(1, np.int64)
        x0 = np.ascontiguousarray(x0, dtype=np.float32)
        n, dim = x0.shape
        out = np.empty((n, dim), dtype=np.float32) if out is None else out
        loss = np.zeros(epochs, dtype=np.float64)
        lrs = np.ascontiguousarray(np.broadcast_to(np.asarray(lr, dtype=np.float64), (epochs,)))
        spec = JobSpec(n, rowptr.ctypes.data, col.ctypes.data, int(rowptr[-1]), dim, PRECISION[precision], epochs,
                       batch_size, ns, 0, lrs.ctypes.data, x0.ctypes.data, out.ctypes.data, loss.ctypes.data)
        jid = _i64(0)
        self._check(lib().de_server_submit(self._h, ctypes.byref(spec), ctypes.byref(jid)))
        self._jobs[jid.value] = (rowptr, col, x0, out, loss, lrs)
        return jid.value

    def info(self, jid: int) -> dict:
        inf = JobInfo()
        self._check(lib().de_server_info(self._h, jid, ctypes.byref(inf)))
        d = inf.as_dict()
        d["state"] = JOB_STATE[d["state"]]
        return d

    def wait(self, jid: int):
        inf = JobInfo()
        rc = lib().de_server_wait(self._h, jid, ctypes.byref(inf))
        arrays = self._jobs.pop(jid, None)
        self._check(rc)
        d = inf.as_dict()
        d["state"] = JOB_STATE[d["state"]]
        return arrays[3], arrays[4], d

    def drain(self):
        self._check(lib().de_server_drain(self._h))

    def stats(self) -> dict:
        st = ServerStats()
        self._check(lib().de_server_get_stats(self._h, ctypes.byref(st)))
        return st.as_dict()

    def close(self):
        if getattr(self, "_h", None):
            lib().de_server_destroy(self._h)
            self._h = None
            self._jobs.clear()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()
