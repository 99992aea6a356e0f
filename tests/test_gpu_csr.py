"""COO -> CSR on the GPU (de_coo_to_csr, de_mm_read_gpu) against the host reader
(de_mm_read) and a NumPy restatement: merge of duplicate entries, mirrored
off-diagonal entries under a symmetric header, columns ascending within a row
(cpp/io/parrallel_IO.hpp:31-88, cpp/core/csr_local.hpp:37-125 at one rank).
Integer work: bitwise equal."""
import time

import numpy as np
import pytest

import distembed_gb300 as de
from distembed_gb300 import graphgen as gg

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _built():
    from distembed_gb300 import build
    build.build()


def numpy_csr(rows, cols, r, c, mirror):
    r, c = np.asarray(r, np.int64), np.asarray(c, np.int64)
    if mirror:
        off = r != c
        r, c = np.concatenate([r, c[off]]), np.concatenate([c, r[off]])
    key = np.unique(r * cols + c)
    rr, cc = key // cols, key % cols
    rowptr = np.zeros(rows + 1, np.int64)
    np.add.at(rowptr, rr + 1, 1)
    return np.cumsum(rowptr), cc


@pytest.mark.parametrize("mirror", [False, True])
@pytest.mark.parametrize("rows,cols,nnz", [(1000, 1000, 20000), (5000, 300, 60000), (7, 7, 40), (300000, 300000, 1000)])
def test_coo_to_csr_matches_numpy(rows, cols, nnz, mirror):
    if mirror and rows != cols:
        pytest.skip("a mirrored matrix is square here")
    rng = np.random.default_rng(rows + nnz)
    r = rng.integers(0, rows, nnz)
    c = rng.integers(0, cols, nnz)
    r[: nnz // 10] = r[nnz // 10: 2 * (nnz // 10)]  # duplicate entries
    c[: nnz // 10] = c[nnz // 10: 2 * (nnz // 10)]
    r[-5:] = c[-5:]                                  # self-loops
    got = de.coo_to_csr(rows, cols, r, c, mirror=mirror)
    rp, cc = numpy_csr(rows, cols, r, c, mirror)
    assert got[0] == rows and got[1] == cols
    assert np.array_equal(got[2], rp) and np.array_equal(got[3], cc)


def test_empty_and_bad_input():
    r, c, rp, col = de.coo_to_csr(10, 10, [], [])
    assert np.array_equal(rp, np.zeros(11, np.int64)) and len(col) == 0
    with pytest.raises(de.DEError):
        de.coo_to_csr(10, 10, [3, 10], [1, 2])
    with pytest.raises(de.DEError):
        de.coo_to_csr(10, 5, [7], [1], mirror=True)   # mirrored entry (1, 7) outside 10 x 5


def write_mm(path, rows, cols, r, c, symmetric):
    with open(path, "w") as f:
        f.write(f"%%MatrixMarket matrix coordinate pattern {'symmetric' if symmetric else 'general'}\n")
        f.write("% comment line\n")
        f.write(f"{rows} {cols} {len(r)}\n")
        for i, j in zip(r, c):
            f.write(f"{i + 1} {j + 1}\n")


@pytest.mark.parametrize("symmetric", [False, True])
def test_mm_read_gpu_equals_host_reader(tmp_path, symmetric):
    rng = np.random.default_rng(5)
    n, m = 4000, 30000
    r, c = rng.integers(0, n, m), rng.integers(0, n, m)
    if symmetric:  # a symmetric file holds one triangle
        r, c = np.maximum(r, c), np.minimum(r, c)
    r[:100], c[:100] = r[100:200], c[100:200]
    path = str(tmp_path / "g.mtx")
    write_mm(path, n, n, r, c, symmetric)
    host = de.read_mtx(path)
    gpu = de.read_mtx(path, gpu=True)
    assert host[0] == gpu[0] and host[1] == gpu[1]
    assert np.array_equal(host[2], gpu[2]) and np.array_equal(host[3], gpu[3])


def test_rmat_file_equals_host_reader_and_generator(tmp_path):
    # a generated R-MAT graph written as a general file: both readers give back
    # the generator's CSR; the GPU build's share of the read is printed
    n, rp, col = gg.rmat_csr(17, 16, seed=3)
    path = str(tmp_path / "rmat.mtx")
    gg.write_mtx(path, n, rp, col)
    t0 = time.perf_counter()
    host = de.read_mtx(path)
    t1 = time.perf_counter()
    gpu = de.read_mtx(path, gpu=True)
    t2 = time.perf_counter()
    for got in (host, gpu):
        assert np.array_equal(got[2], rp) and np.array_equal(got[3], col)
    print(f"\nR-MAT s17 ({len(col)} entries): host reader {t1 - t0:.2f} s, GPU CSR reader {t2 - t1:.2f} s")
