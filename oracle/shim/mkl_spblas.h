/*
 * Stand-in for Intel MKL's sparse BLAS (<mkl_spblas.h>).  TEST INFRASTRUCTURE ONLY.
 *
 * The reference builds its CSR with MKL's COO->CSR conversion
 * (cpp/core/csr_local.hpp:59-121) under -DMKL_ILP64 (CMakeLists.txt:73), so
 * MKL_INT is 64-bit.  MKL is not available here, and the order MKL leaves the
 * columns in within one row is not documented.  This stand-in fixes that
 * order: ascending column, ties kept in input order (a stable sort).  The GPU
 * path and the oracle use the same convention.
 */
#pragma once
#include <algorithm>
#include <cstdint>
#include <numeric>
#include <vector>

typedef int64_t MKL_INT;

typedef enum { SPARSE_STATUS_SUCCESS = 0, SPARSE_STATUS_NOT_SUPPORTED = 6 } sparse_status_t;
typedef enum {
  SPARSE_OPERATION_NON_TRANSPOSE = 10,
  SPARSE_OPERATION_TRANSPOSE = 11,
  SPARSE_OPERATION_CONJUGATE_TRANSPOSE = 12
} sparse_operation_t;
typedef enum { SPARSE_INDEX_BASE_ZERO = 0, SPARSE_INDEX_BASE_ONE = 1 } sparse_index_base_t;

struct shim_sparse_matrix {
  MKL_INT rows = 0, cols = 0;
  bool is_csr = false;
  std::vector<MKL_INT> r, c;  // COO (owned)
  std::vector<double> v;
  std::vector<MKL_INT> rs, ci;  // CSR (owned when produced by convert)
  std::vector<double> cv;
};
typedef shim_sparse_matrix *sparse_matrix_t;

inline sparse_status_t mkl_sparse_d_create_coo(sparse_matrix_t *A, sparse_index_base_t base,
                                               MKL_INT rows, MKL_INT cols, MKL_INT nnz,
                                               const MKL_INT *ri, const MKL_INT *ci,
                                               const double *v) {
  if (base != SPARSE_INDEX_BASE_ZERO) return SPARSE_STATUS_NOT_SUPPORTED;
  auto *m = new shim_sparse_matrix;
  m->rows = rows;
  m->cols = cols;
  m->r.assign(ri, ri + nnz);
  m->c.assign(ci, ci + nnz);
  m->v.assign(v, v + nnz);
  *A = m;
  return SPARSE_STATUS_SUCCESS;
}

inline sparse_status_t mkl_sparse_convert_csr(sparse_matrix_t A, sparse_operation_t op,
                                              sparse_matrix_t *B) {
  const bool tr = (op != SPARSE_OPERATION_NON_TRANSPOSE);
  auto *m = new shim_sparse_matrix;
  m->is_csr = true;
  m->rows = tr ? A->cols : A->rows;
  m->cols = tr ? A->rows : A->cols;
  const size_t nnz = A->r.size();
  const std::vector<MKL_INT> &R = tr ? A->c : A->r;
  const std::vector<MKL_INT> &C = tr ? A->r : A->c;
  std::vector<size_t> order(nnz);
  std::iota(order.begin(), order.end(), size_t(0));
  std::stable_sort(order.begin(), order.end(), [&](size_t a, size_t b) {
    return R[a] != R[b] ? R[a] < R[b] : C[a] < C[b];
  });
  m->rs.assign(size_t(m->rows) + 1, 0);
  m->ci.resize(nnz);
  m->cv.resize(nnz);
  for (size_t k = 0; k < nnz; ++k) {
    m->ci[k] = C[order[k]];
    m->cv[k] = A->v[order[k]];
    m->rs[size_t(R[order[k]]) + 1]++;
  }
  for (MKL_INT i = 0; i < m->rows; ++i) m->rs[i + 1] += m->rs[i];
  *B = m;
  return SPARSE_STATUS_SUCCESS;
}

inline sparse_status_t mkl_sparse_d_export_csr(sparse_matrix_t A, sparse_index_base_t *base,
                                               MKL_INT *rows, MKL_INT *cols,
                                               MKL_INT **rows_start, MKL_INT **rows_end,
                                               MKL_INT **col_idx, double **values) {
  *base = SPARSE_INDEX_BASE_ZERO;
  *rows = A->rows;
  *cols = A->cols;
  *rows_start = A->rs.data();
  *rows_end = A->rs.data() + 1;
  *col_idx = A->ci.data();
  *values = A->cv.data();
  return SPARSE_STATUS_SUCCESS;
}

inline sparse_status_t mkl_sparse_d_create_csr(sparse_matrix_t *A, sparse_index_base_t,
                                               MKL_INT rows, MKL_INT cols, MKL_INT *,
                                               MKL_INT *, MKL_INT *, double *) {
  auto *m = new shim_sparse_matrix;  // borrowed arrays; never read back by the path
  m->rows = rows;
  m->cols = cols;
  m->is_csr = true;
  *A = m;
  return SPARSE_STATUS_SUCCESS;
}

inline sparse_status_t mkl_sparse_destroy(sparse_matrix_t A) {
  delete A;
  return SPARSE_STATUS_SUCCESS;
}
