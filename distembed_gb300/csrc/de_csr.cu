// COO -> CSR on the GPU: the CSR the host reader builds (cpp/io/parrallel_IO.hpp:31-88
// and the COO -> CSR of cpp/core/csr_local.hpp:37-125 at one rank, with columns
// ascending within a row), from keys row * cols + col: radix sort of the keys,
// merge of equal keys, then per row the first key of the row by binary search
// (row pointers) and per key its column.  The parse of a MatrixMarket file stays
// on the host (de_io.cpp); the sort, which dominates the host reader on large
// graphs, runs here.
#include <cub/device/device_radix_sort.cuh>
#include <cub/device/device_select.cuh>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/distembed_gb300.h"

struct de_csr {
  int64_t rows = 0, cols = 0;
  std::vector<int64_t> rowptr, col;
};

namespace de {

void set_thread_error(const std::string &msg);  // de_runtime.cpp
int parse_mm(const char *path, int64_t *rows, int64_t *cols, std::vector<int64_t> &key);  // de_io.cpp

namespace {

int csr_fail(int rc, const std::string &m) {
  set_thread_error(m);
  return rc;
}

// rowptr[r] = first position of a key >= r * cols (r = 0 .. rows).
__global__ void row_pointers_kernel(const uint64_t *__restrict__ key, int64_t m, int64_t rows, int64_t cols,
                                    int64_t *__restrict__ rowptr) {
  for (int64_t r = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; r <= rows; r += int64_t(gridDim.x) * blockDim.x) {
    const uint64_t target = uint64_t(r) * uint64_t(cols);
    int64_t lo = 0, hi = m;
    while (lo < hi) {
      const int64_t mid = (lo + hi) >> 1;
      if (key[mid] < target) lo = mid + 1;
      else hi = mid;
    }
    rowptr[r] = lo;
  }
}

__global__ void columns_kernel(const uint64_t *__restrict__ key, int64_t m, int64_t cols, int64_t *__restrict__ col) {
  for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < m; i += int64_t(gridDim.x) * blockDim.x)
    col[i] = int64_t(key[i] % uint64_t(cols));
}

int grid_for(int64_t n) { return int(std::min<int64_t>((n + 255) / 256 + 1, 152 * 16)); }

struct DeviceBuffers {
  void *p[6] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
  cudaStream_t st = nullptr;
  ~DeviceBuffers() {
    if (st) cudaStreamSynchronize(st);
    for (void *q : p)
      if (q) cudaFree(q);
    if (st) cudaStreamDestroy(st);
  }
};

#define CSR_CUDA(call)                                                              \
  do {                                                                              \
    const cudaError_t e_ = (call);                                                  \
    if (e_ != cudaSuccess) return csr_fail(DE_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
  } while (0)

// Sorted, merged keys -> CSR in `out`.
int build_on_gpu(int32_t device, int64_t rows, int64_t cols, const std::vector<int64_t> &keys, de_csr *out) {
  out->rows = rows;
  out->cols = cols;
  const int64_t n = int64_t(keys.size());
  out->rowptr.assign(size_t(rows) + 1, 0);
  out->col.clear();
  if (n == 0) return DE_OK;
  if (n >= (int64_t(1) << 31)) return csr_fail(DE_ERR_UNSUPPORTED, "at most 2^31 - 1 entries");
  CSR_CUDA(cudaSetDevice(device));
  DeviceBuffers b;
  CSR_CUDA(cudaStreamCreateWithFlags(&b.st, cudaStreamNonBlocking));
  uint64_t *d_in = nullptr, *d_sorted = nullptr, *d_uniq = nullptr;
  int64_t *d_num = nullptr, *d_rowptr = nullptr, *d_col = nullptr;
  CSR_CUDA(cudaMalloc(&b.p[0], size_t(n) * sizeof(uint64_t)));
  CSR_CUDA(cudaMalloc(&b.p[1], size_t(n) * sizeof(uint64_t)));
  CSR_CUDA(cudaMalloc(&b.p[2], size_t(n) * sizeof(uint64_t)));
  CSR_CUDA(cudaMalloc(&b.p[3], sizeof(int64_t)));
  d_in = static_cast<uint64_t *>(b.p[0]);
  d_sorted = static_cast<uint64_t *>(b.p[1]);
  d_uniq = static_cast<uint64_t *>(b.p[2]);
  d_num = static_cast<int64_t *>(b.p[3]);
  // bits of the largest key rows * cols - 1
  const uint64_t top = uint64_t(rows) * uint64_t(cols) - 1;
  int end_bit = 1;
  while (end_bit < 64 && (top >> end_bit) != 0) ++end_bit;
  size_t sort_bytes = 0, uniq_bytes = 0;
  CSR_CUDA(cub::DeviceRadixSort::SortKeys(nullptr, sort_bytes, d_in, d_sorted, n, 0, end_bit, b.st));
  CSR_CUDA(cub::DeviceSelect::Unique(nullptr, uniq_bytes, d_sorted, d_uniq, d_num, n, b.st));
  CSR_CUDA(cudaMalloc(&b.p[4], std::max(sort_bytes, uniq_bytes)));
  void *temp = b.p[4];
  CSR_CUDA(cudaMemcpyAsync(d_in, keys.data(), size_t(n) * sizeof(uint64_t), cudaMemcpyHostToDevice, b.st));
  CSR_CUDA(cub::DeviceRadixSort::SortKeys(temp, sort_bytes, d_in, d_sorted, n, 0, end_bit, b.st));
  CSR_CUDA(cub::DeviceSelect::Unique(temp, uniq_bytes, d_sorted, d_uniq, d_num, n, b.st));
  int64_t m = 0;
  CSR_CUDA(cudaMemcpyAsync(&m, d_num, sizeof(int64_t), cudaMemcpyDeviceToHost, b.st));
  CSR_CUDA(cudaStreamSynchronize(b.st));
  // the merged keys' CSR; d_in is free again and holds rowptr, then col reuses d_sorted
  d_rowptr = reinterpret_cast<int64_t *>(d_in);
  if (size_t(rows) + 1 > size_t(n)) {
    CSR_CUDA(cudaMalloc(&b.p[5], (size_t(rows) + 1) * sizeof(int64_t)));
    d_rowptr = static_cast<int64_t *>(b.p[5]);
  }
  d_col = reinterpret_cast<int64_t *>(d_sorted);
  row_pointers_kernel<<<grid_for(rows + 1), 256, 0, b.st>>>(d_uniq, m, rows, cols, d_rowptr);
  CSR_CUDA(cudaGetLastError());
  columns_kernel<<<grid_for(m), 256, 0, b.st>>>(d_uniq, m, cols, d_col);
  CSR_CUDA(cudaGetLastError());
  out->col.resize(size_t(m));
  CSR_CUDA(cudaMemcpyAsync(out->rowptr.data(), d_rowptr, (size_t(rows) + 1) * sizeof(int64_t), cudaMemcpyDeviceToHost,
                           b.st));
  CSR_CUDA(cudaMemcpyAsync(out->col.data(), d_col, size_t(m) * sizeof(int64_t), cudaMemcpyDeviceToHost, b.st));
  CSR_CUDA(cudaStreamSynchronize(b.st));
  return DE_OK;
}

}  // namespace
}  // namespace de

extern "C" {

int de_coo_to_csr(int64_t rows, int64_t cols, const int64_t *row_idx, const int64_t *col_idx, int64_t nnz,
                  int32_t mirror, int32_t device, de_csr **out) {
  if (!out) return de::csr_fail(DE_ERR_INVALID, "out is NULL");
  *out = nullptr;
  if (rows <= 0 || cols <= 0 || nnz < 0 || (nnz > 0 && (!row_idx || !col_idx)) || rows >= (int64_t(1) << 31) ||
      cols >= (int64_t(1) << 31))
    return de::csr_fail(DE_ERR_INVALID, "bad COO arguments");
  std::vector<int64_t> keys;
  keys.reserve(size_t(mirror ? 2 : 1) * size_t(nnz));
  for (int64_t e = 0; e < nnz; ++e) {
    const int64_t i = row_idx[e], j = col_idx[e];
    if (i < 0 || j < 0 || i >= rows || j >= cols) return de::csr_fail(DE_ERR_INVALID, "COO entry outside the matrix");
    keys.push_back(i * cols + j);
    if (mirror && i != j) {
      if (j >= rows || i >= cols) return de::csr_fail(DE_ERR_INVALID, "mirrored entry outside the matrix");
      keys.push_back(j * cols + i);
    }
  }
  auto c = new de_csr;
  if (int rc = de::build_on_gpu(device, rows, cols, keys, c)) {
    delete c;
    return rc;
  }
  *out = c;
  return DE_OK;
}

int de_mm_read_gpu(const char *path, int32_t device, de_csr **out) {
  if (!path || !out) return de::csr_fail(DE_ERR_INVALID, "NULL argument");
  *out = nullptr;
  int64_t rows = 0, cols = 0;
  std::vector<int64_t> keys;
  if (int rc = de::parse_mm(path, &rows, &cols, keys)) return rc;
  auto c = new de_csr;
  if (int rc = de::build_on_gpu(device, rows, cols, keys, c)) {
    delete c;
    return rc;
  }
  *out = c;
  return DE_OK;
}

int de_csr_info(const de_csr *c, int64_t *rows, int64_t *cols, int64_t *nnz) {
  if (!c || !rows || !cols || !nnz) return DE_ERR_INVALID;
  *rows = c->rows;
  *cols = c->cols;
  *nnz = int64_t(c->col.size());
  return DE_OK;
}

int de_csr_copy(const de_csr *c, int64_t *rowptr, int64_t *col) {
  if (!c || !rowptr || (!col && !c->col.empty())) return DE_ERR_INVALID;
  std::memcpy(rowptr, c->rowptr.data(), c->rowptr.size() * sizeof(int64_t));
  if (!c->col.empty()) std::memcpy(col, c->col.data(), c->col.size() * sizeof(int64_t));
  return DE_OK;
}

void de_csr_free(de_csr *c) { delete c; }

}  // extern "C"
