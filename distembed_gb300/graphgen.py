"""Synthetic input graphs for the embedding step, and MatrixMarket text I/O.

The reference reads a MatrixMarket file through CombBLAS
(cpp/io/parrallel_IO.hpp:31-88): coordinates are 1-based, duplicate entries are
merged (by `maximum`), and the values are replaced by the column id
(copy_col_to_value, cpp/dist_embed.cpp:168).  The CSR it then builds
(cpp/core/csr_local.hpp:37-125) has rows in order; within a row this package
fixes the order to ascending column.

Generators (seeded, numpy only):
  rmat_edges / rmat_csr        R-MAT (a, b, c, d = 1-a-b-c), edge factor ef,
                               symmetrised, duplicates and self-loops removed
  gaussian_mixture / knn_csr   points from an isotropic Gaussian mixture, exact
                               Euclidean k-nearest-neighbour graph, symmetrised (union)
"""
from __future__ import annotations

import numpy as np


# ------------------------------------------------------------------- CSR

def coo_to_csr(n: int, src: np.ndarray, dst: np.ndarray, dedup: bool = True):
    """int64 CSR (rowptr[n+1], col[nnz]) with ascending columns in each row."""
    src = np.asarray(src, dtype=np.int64)
    dst = np.asarray(dst, dtype=np.int64)
    key = np.sort(src * np.int64(n) + dst)
    if dedup and len(key) > 1:
        key = key[np.concatenate(([True], key[1:] != key[:-1]))]
    rows = key // n
    col = (key - rows * n).astype(np.int64)
    rowptr = np.zeros(n + 1, dtype=np.int64)
    np.cumsum(np.bincount(rows, minlength=n), out=rowptr[1:])
    return rowptr, col


def transpose_csr(rowptr, col, n: int | None = None):
    """The CSR of the transposed matrix (columns ascending in each row): the
    receiver matrix's CSR, which the reference's col_major flag selects
    (cpp/algo/algo.hpp:131-133, built with transpose = true, cpp/dist_embed.cpp:197-200)."""
    rowptr = np.asarray(rowptr, dtype=np.int64)
    col = np.asarray(col, dtype=np.int64)
    n = len(rowptr) - 1 if n is None else n
    src = np.repeat(np.arange(len(rowptr) - 1, dtype=np.int64), np.diff(rowptr))
    return coo_to_csr(n, col, src, dedup=False)


def symmetrise(src, dst, drop_self_loops: bool = True):
    s = np.concatenate([src, dst])
    d = np.concatenate([dst, src])
    if drop_self_loops:
        keep = s != d
        s, d = s[keep], d[keep]
    return s, d


# ------------------------------------------------------------------- R-MAT

def rmat_edges(scale: int, edge_factor: int, a=0.57, b=0.19, c=0.19, seed: int = 1,
               chunk: int = 1 << 24):
    """edge_factor * 2**scale directed R-MAT edges (src, dst), int64.  At each of
    the `scale` levels a quadrant is drawn: a -> (0,0), b -> (0,1), c -> (1,0),
    d -> (1,1); the first level sets the most significant bit."""
    m = edge_factor << scale
    rng = np.random.Generator(np.random.PCG64(seed))
    src = np.zeros(m, dtype=np.int64)
    dst = np.zeros(m, dtype=np.int64)
    ab, abc = a + b, a + b + c
    for lo in range(0, m, chunk):
        hi = min(m, lo + chunk)
        s = np.zeros(hi - lo, dtype=np.int64)
        t = np.zeros(hi - lo, dtype=np.int64)
        for _ in range(scale):
            u = rng.random(hi - lo, dtype=np.float32)
            sb = u >= ab
            tb = ((u >= a) & (u < ab)) | (u >= abc)
            s = (s << 1) | sb
            t = (t << 1) | tb
        src[lo:hi] = s
        dst[lo:hi] = t
    return src, dst


def rmat_csr(scale: int, edge_factor: int, seed: int, a=0.57, b=0.19, c=0.19):
    n = 1 << scale
    s, d = rmat_edges(scale, edge_factor, a, b, c, seed)
    s, d = symmetrise(s, d)
    return n, *coo_to_csr(n, s, d)


def rmat_csr_n(n: int, edge_factor: int, seed: int, a=0.57, b=0.19, c=0.19):
    """R-MAT on n vertices (n need not be a power of two): edge_factor * 2**scale
    edges are drawn at scale = ceil(log2 n) and those with an endpoint >= n are
    dropped."""
    scale = max(1, int(np.ceil(np.log2(max(n, 2)))))
    s, d = rmat_edges(scale, edge_factor, a, b, c, seed)
    keep = (s < n) & (d < n)
    s, d = symmetrise(s[keep], d[keep])
    return n, *coo_to_csr(n, s, d)


def rmat_csr_torch(n: int, edge_factor: int, seed: int, device, a=0.57, b=0.19, c=0.19):
    """rmat_csr_n drawn with torch on `device` (input preparation for large
    suites; its own random stream, so the graph differs from rmat_csr_n's)."""
    import torch
    scale = max(1, int(np.ceil(np.log2(max(n, 2)))))
    m = edge_factor << scale
    g = torch.Generator(device=device)
    g.manual_seed(int(seed))
    s = torch.zeros(m, dtype=torch.int64, device=device)
    t = torch.zeros(m, dtype=torch.int64, device=device)
    ab, abc = a + b, a + b + c
    for _ in range(scale):
        u = torch.rand(m, generator=g, device=device)
        s = (s << 1) | (u >= ab).long()
        t = (t << 1) | (((u >= a) & (u < ab)) | (u >= abc)).long()
    keep = (s < n) & (t < n) & (s != t)
    s, t = s[keep], t[keep]
    key = torch.unique(torch.cat([s * n + t, t * n + s]))
    rows = key // n
    col = key - rows * n
    rowptr = torch.zeros(n + 1, dtype=torch.int64, device=device)
    rowptr[1:] = torch.cumsum(torch.bincount(rows, minlength=n), 0)
    return n, rowptr.cpu().numpy(), col.cpu().numpy()


# ------------------------------------------------------- Gaussian-mixture kNN

def gaussian_mixture(n: int, dim: int, components: int, seed: int, mean_std: float = 2.0):
    """n points; component means ~ N(0, mean_std^2 I), unit-variance clusters,
    components drawn uniformly per point."""
    rng = np.random.Generator(np.random.PCG64(seed))
    means = rng.normal(0.0, mean_std, size=(components, dim))
    comp = rng.integers(0, components, size=n)
    pts = means[comp] + rng.normal(0.0, 1.0, size=(n, dim))
    return pts, comp


def knn_edges(pts: np.ndarray, k: int, block: int = 2048):
    """Exact Euclidean k nearest neighbours (self excluded), FP64, ties by index."""
    pts = np.asarray(pts, dtype=np.float64)
    n = pts.shape[0]
    k = min(k, n - 1)
    sq = np.einsum("ij,ij->i", pts, pts)
    src = np.repeat(np.arange(n, dtype=np.int64), k)
    dst = np.empty(n * k, dtype=np.int64)
    for lo in range(0, n, block):
        hi = min(n, lo + block)
        d2 = sq[lo:hi, None] + sq[None, :] - 2.0 * (pts[lo:hi] @ pts.T)
        d2[np.arange(hi - lo), np.arange(lo, hi)] = np.inf
        part = np.argpartition(d2, k, axis=1)[:, : k + 1]
        pd = np.take_along_axis(d2, part, axis=1)
        order = np.lexsort((part, pd), axis=1)[:, :k]
        dst[lo * k: hi * k] = np.take_along_axis(part, order, axis=1).reshape(-1)
    return src, dst


def knn_edges_torch(pts: np.ndarray, k: int, device, block: int = 2048):
    """k nearest neighbours on a torch device in FP32 (input preparation for large
    suites; the FP64 knn_edges is the exact reference).  Self excluded."""
    import torch
    x = torch.as_tensor(np.asarray(pts, dtype=np.float32), device=device)
    n = x.shape[0]
    k = min(k, n - 1)
    sq = (x * x).sum(1)
    dst = torch.empty(n * k, dtype=torch.int64, device=device)
    for lo in range(0, n, block):
        hi = min(n, lo + block)
        d2 = sq[lo:hi, None] + sq[None, :] - 2.0 * (x[lo:hi] @ x.T)
        d2[torch.arange(hi - lo, device=device), torch.arange(lo, hi, device=device)] = float("inf")
        dst[lo * k: hi * k] = torch.topk(d2, k, dim=1, largest=False).indices.reshape(-1)
    src = np.repeat(np.arange(n, dtype=np.int64), k)
    return src, dst.cpu().numpy()


def knn_csr(n: int, dim: int, k: int, components: int, seed: int, device=None):
    """Symmetrised kNN graph of a Gaussian mixture; device: compute the neighbours
    with torch on that device (FP32) instead of numpy (FP64)."""
    pts, _ = gaussian_mixture(n, dim, components, seed)
    s, d = knn_edges(pts, k) if device is None else knn_edges_torch(pts, k, device)
    s, d = symmetrise(s, d)
    return n, *coo_to_csr(n, s, d)


def graph_suite(count: int, n_lo: int, n_hi: int, seed: int, knn_k: int = 10, knn_dim: int = 32,
                knn_components: int = 10, rmat_ef: int = 8, device=None):
    """`count` independent graphs, vertex counts log-uniform in [n_lo, n_hi]
    (PCG64(seed)); even positions are kNN graphs (knn_k neighbours of knn_dim-D
    mixtures), odd positions R-MAT graphs (edge factor rmat_ef).  Graph i is
    seeded with seed * 100003 + i.  Returns a list of (kind, n, rowptr, col)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    ns = np.rint(np.exp(rng.uniform(np.log(n_lo), np.log(n_hi), size=count))).astype(np.int64)
    out = []
    for i, n in enumerate(ns):
        gs = seed * 100003 + i
        if i % 2 == 0:
            out.append(("knn", *knn_csr(int(n), knn_dim, knn_k, knn_components, gs, device=device)))
        else:
            out.append(("rmat", *rmat_csr_n(int(n), rmat_ef, gs)))
    return out


# ------------------------------------------------------------ embeddings

def init_embedding(n: int, dim: int, seed: int, lo: float = -0.5, hi: float = 0.5):
    """Seeded U[lo, hi) FP64 initial embedding (n x dim, row-major)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    return rng.uniform(lo, hi, size=(n, dim))


# ------------------------------------------------------------ MatrixMarket

def write_mtx(path: str, n: int, rowptr: np.ndarray, col: np.ndarray) -> None:
    """`coordinate pattern general`, both directions explicit, 1-based."""
    rows = np.repeat(np.arange(n, dtype=np.int64), np.diff(rowptr))
    with open(path, "w") as f:
        f.write("%%MatrixMarket matrix coordinate pattern general\n")
        f.write(f"{n} {n} {len(col)}\n")
        np.savetxt(f, np.stack([rows + 1, np.asarray(col) + 1], axis=1), fmt="%d")


def read_mtx(path: str):
    """(n_rows, n_cols, rowptr, col) with duplicates merged, 1-based input."""
    with open(path) as f:
        header = f.readline()
        if not header.startswith("%%MatrixMarket"):
            raise ValueError("not a MatrixMarket file")
        symmetric = "symmetric" in header.lower()
        line = f.readline()
        while line.startswith("%"):
            line = f.readline()
        nr, nc, nnz = (int(t) for t in line.split()[:3])
        data = np.loadtxt(f, dtype=np.float64, ndmin=2, max_rows=nnz)
    r = data[:, 0].astype(np.int64) - 1 if nnz else np.zeros(0, np.int64)
    c = data[:, 1].astype(np.int64) - 1 if nnz else np.zeros(0, np.int64)
    if symmetric:
        off = r != c
        r, c = np.concatenate([r, c[off]]), np.concatenate([c, r[off]])
    rowptr, col = coo_to_csr(max(nr, nc), r, c, dedup=True)
    return nr, nc, rowptr, col
