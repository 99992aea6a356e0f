"""MatrixMarket reader, embedding writer and the host driver, without a GPU.

The reader follows ParallelIO::parallel_read_MM at one rank
(cpp/io/parrallel_IO.hpp:31-88): 1-based coordinates, duplicates merged, values
ignored, a symmetric header mirrors off-diagonal entries.  The writer follows
ParallelIO::parallel_write (cpp/io/parrallel_IO.hpp:90-146).
"""
import os
import subprocess

import numpy as np
import pytest

import distembed_gb300 as de
from distembed_gb300 import graphgen as gg

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module", autouse=True)
def _built():
    from distembed_gb300 import build
    build.build()


def test_reader_round_trips_the_generators_files(tmp_path):
    n, rp, col = gg.knn_csr(300, 8, 6, 3, seed=2)
    p = str(tmp_path / "g.mtx")
    gg.write_mtx(p, n, rp, col)
    r, c, rp2, col2 = de.read_mtx(p)
    assert (r, c) == (n, n)
    assert np.array_equal(rp2, rp) and np.array_equal(col2, col)
    # the Python reader agrees
    n3, m3, rp3, col3 = gg.read_mtx(p)
    assert n3 == m3 == n and np.array_equal(rp3, rp) and np.array_equal(col3, col)


def test_reader_mirrors_symmetric_files_and_merges_duplicates(tmp_path):
    p = str(tmp_path / "s.mtx")
    with open(p, "w") as f:
        f.write("%%MatrixMarket matrix coordinate real symmetric\n% a comment\n5 5 6\n"
                "2 1 1.0\n3 1 2.5\n3 3 1.0\n5 4 7\n2 1 9.0\n4 2 0.5\n")
    r, c, rp, col = de.read_mtx(p)
    want = {(1, 0), (0, 1), (2, 0), (0, 2), (2, 2), (4, 3), (3, 4), (3, 1), (1, 3)}
    got = {(i, int(col[e])) for i in range(r) for e in range(rp[i], rp[i + 1])}
    assert (r, c) == (5, 5) and got == want
    for i in range(r):  # ascending columns within a row
        assert np.all(np.diff(col[rp[i]:rp[i + 1]]) > 0)


def test_reader_rejects_bad_files(tmp_path):
    bad = tmp_path / "b.mtx"
    bad.write_text("%%MatrixMarket matrix array real general\n2 2\n1\n2\n3\n4\n")
    with pytest.raises(de.DEError):
        de.read_mtx(str(bad))
    bad.write_text("%%MatrixMarket matrix coordinate pattern general\n3 3 2\n1 2\n4 1\n")
    with pytest.raises(de.DEError):
        de.read_mtx(str(bad))
    with pytest.raises(de.DEError):
        de.read_mtx(str(tmp_path / "missing.mtx"))


def test_writer_format(tmp_path):
    x = np.array([[0.5, -1.25, 3.0], [1e-7, 2.0 / 3.0, -0.000004]])
    p = str(tmp_path / "e.txt")
    de.write_embedding(p, x)
    want = "".join(f"{i + 1}" + "".join(f" {v:.5f}" for v in row) + "\n" for i, row in enumerate(x))
    assert open(p).read() == want


def test_driver_usage_and_missing_input_without_a_gpu(tmp_path):
    exe = de.DRIVER_PATH
    assert os.access(exe, os.X_OK)
    r = subprocess.run([exe], capture_output=True, text=True)
    assert r.returncode == 2 and "usage" in r.stderr
    r = subprocess.run([exe, "-input", str(tmp_path / "none.mtx")], capture_output=True, text=True)
    assert r.returncode == 1 and "cannot open" in r.stderr
    r = subprocess.run([exe, "-input", "x.mtx", "-spgemm", "1"], capture_output=True, text=True)
    assert r.returncode == 2
    r = subprocess.run([exe, "-input", str(tmp_path / "none.mtx"), "-spmm", "1"], capture_output=True, text=True)
    assert r.returncode == 1 and "cannot open" in r.stderr
    r = subprocess.run([exe, "-input", str(tmp_path / "none.mtx"), "-sparse_embedding", "1"], capture_output=True,
                       text=True)
    assert r.returncode == 1 and "cannot open" in r.stderr


def test_cpp_header_compiles_against_reference_shaped_types(tmp_path):
    src = tmp_path / "t.cpp"
    src.write_text('''
#include <memory>
#include <vector>
#include "distembed_gb300.hpp"
struct CSRHandle { std::vector<long long> rowStart, col_idx; };
struct CSRLocal { std::unique_ptr<CSRHandle> handler; };
struct SpMat { std::unique_ptr<CSRLocal> csr_local_data; };
struct DenseMat { unsigned long rows; double *nCoordinates; };
struct Grid {};
using Algo = distembed_gb300::GpuEmbeddingAlgo<long long, double, 128>;
void f(SpMat *s, DenseMat *d, Grid *g) {
  Algo a(s, s, s, d, g, 0.0, 0.25, 5.0, -5.0, false, false);
  a.algo_force2_vec_ns(30, 16384, 5, 0.02);
}
''')
    r = subprocess.run(["g++", "-std=c++17", "-fsyntax-only", "-I" + os.path.join(ROOT, "include"), str(src)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def _ref_root():
    return os.environ.get("DE_REF_ROOT") or os.path.abspath(os.path.join(ROOT, "..", "reference"))


def test_cpp_header_compiles_against_the_reference_headers(tmp_path):
    # the binding as the reference driver's embedding branch would use it
    # (cpp/dist_embed.cpp:331-346, only the class name changed), compiled against
    # the reference's own SpMat / DenseMat / Process3DGrid headers where they lie,
    # with oracle/shim/ standing in for MPI, MKL and Eigen (the include path of
    # oracle/Makefile's `ref` target)
    ref = _ref_root()
    if not os.path.exists(os.path.join(ref, "cpp", "core", "sparse_mat.hpp")):
        pytest.skip("reference sources not present")
    subprocess.check_call(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "ref", f"REF_ROOT={ref}"],
                          stderr=subprocess.DEVNULL)
    src = tmp_path / "embedding_branch.cpp"
    src.write_text('''
#include "algo/algo.hpp"
#include "core/dense_mat.hpp"
#include "core/sparse_mat.hpp"
#include "net/process_3D_grid.hpp"
#include "distembed_gb300.hpp"
#include <memory>
using namespace std;
using namespace distblas::core;
using namespace distblas::net;
void embedding_branch(Process3DGrid *grid, shared_ptr<SpMat<VALUE_TYPE>> shared_sparseMat,
                      shared_ptr<SpMat<VALUE_TYPE>> shared_sparseMat_receiver,
                      shared_ptr<SpMat<VALUE_TYPE>> shared_sparseMat_sender, INDEX_TYPE localARows, double alpha,
                      double beta, bool col_major, bool sync_comm, int iterations, int batch_size, int ns,
                      VALUE_TYPE lr) {
  const int dimension = 128;
  auto dense_mat = shared_ptr<DenseMat<INDEX_TYPE, VALUE_TYPE, dimension>>(
      new DenseMat<INDEX_TYPE, VALUE_TYPE, dimension>(grid, localARows));
  unique_ptr<distembed_gb300::GpuEmbeddingAlgo<INDEX_TYPE, VALUE_TYPE, dimension>> embedding_algo =
      make_unique<distembed_gb300::GpuEmbeddingAlgo<INDEX_TYPE, VALUE_TYPE, dimension>>(
          shared_sparseMat.get(), shared_sparseMat_receiver.get(), shared_sparseMat_sender.get(),
          dense_mat.get(), grid, alpha, beta, 5, -5, col_major, sync_comm);
  embedding_algo->algo_force2_vec_ns(iterations, batch_size, ns, lr);
}
''')
    ovl = os.path.join(ROOT, "oracle", "_ref", "overlay")
    gxx = subprocess.run(["g++", "-dumpversion"], capture_output=True, text=True).stdout.strip().split(".")[0]
    cmd = ["g++", "-std=c++17", "-fsyntax-only", "-fopenmp", "-w", "-fpermissive", "-include", "climits", "-I-",
           "-I" + os.path.join(ROOT, "oracle", "shim"), "-I" + os.path.join(ovl, "algo"),
           "-I" + os.path.join(ref, "cpp", "algo"), "-I" + os.path.join(ovl, "core"),
           "-I" + os.path.join(ref, "cpp", "core"), "-I" + os.path.join(ref, "cpp"),
           "-I" + os.path.join(ref, "cpp", "net"), f"-I/usr/include/c++/{gxx}/pstl",
           "-I" + os.path.join(ROOT, "include"), str(src)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-4000:]


def _big_file(path, n, m, seed, bad_at=None, extra=0):
    """A general file of m random entries over n vertices, comment lines every
    1000 entries, optionally a malformed entry line at index bad_at and `extra`
    entries past the declared count."""
    rng = np.random.default_rng(seed)
    r, c = rng.integers(1, n + 1, m + extra), rng.integers(1, n + 1, m + extra)
    with open(path, "w") as f:
        f.write("%%MatrixMarket matrix coordinate real general\n% generated\n")
        f.write(f"{n} {n} {m}\n")
        for e in range(m + extra):
            if e % 1000 == 0:
                f.write("% a comment between entries\n")
            if e == bad_at:
                f.write(f"{r[e]} x\n")
            else:
                f.write(f"  {r[e]}\t{c[e]} 0.5\n")
    return r[:m] - 1, c[:m] - 1


def test_reader_large_file_in_chunks(tmp_path):
    # a file of several MB is parsed by several host threads; entries past the
    # declared count are not read (as the one-line-at-a-time reference reader)
    p = str(tmp_path / "big.mtx")
    r, c = _big_file(p, 5000, 200000, 3, extra=500)
    rows, cols, rp, col = de.read_mtx(p)
    key = np.unique(r * 5000 + c)
    want_rp = np.zeros(5001, np.int64)
    np.add.at(want_rp, key // 5000 + 1, 1)
    assert rows == cols == 5000
    assert np.array_equal(rp, np.cumsum(want_rp)) and np.array_equal(col, key % 5000)


def test_reader_reports_the_first_bad_entry_by_number(tmp_path):
    p = str(tmp_path / "bad.mtx")
    _big_file(p, 5000, 200000, 4, bad_at=171234)
    with pytest.raises(de.DEError, match="bad MatrixMarket entry 171235"):
        de.read_mtx(p)
    # a malformed line after the declared entries is never read
    q = str(tmp_path / "late.mtx")
    _big_file(q, 5000, 200000, 4, bad_at=200100, extra=200)
    assert de.read_mtx(q)[0] == 5000
    # fewer entries than declared
    t = str(tmp_path / "short.mtx")
    with open(t, "w") as f:
        f.write("%%MatrixMarket matrix coordinate pattern general\n3 3 4\n1 2\n2 3\n")
    with pytest.raises(de.DEError, match="ends early"):
        de.read_mtx(t)


def test_transpose_csr_is_the_receiver_matrix():
    # the CSR the reference's col_major flag selects: entries (j, i) for every (i, j),
    # columns ascending in each row; transposing twice gives the input back
    from distembed_gb300 import graphgen as gg
    rng = np.random.default_rng(61)
    n = 300
    src, dst = rng.integers(0, n, 2000), rng.integers(0, n, 2000)
    rp, col = gg.coo_to_csr(n, src, dst)
    trp, tcol = gg.transpose_csr(rp, col)
    rows = np.repeat(np.arange(n), np.diff(rp))
    trows = np.repeat(np.arange(n), np.diff(trp))
    assert set(zip(rows.tolist(), col.tolist())) == set(zip(tcol.tolist(), trows.tolist()))
    assert all(np.all(np.diff(tcol[trp[i]:trp[i + 1]]) > 0) for i in range(n))
    back = gg.transpose_csr(trp, tcol)
    assert np.array_equal(back[0], rp) and np.array_equal(back[1], col)
