// MatrixMarket input and embedding output of the driver (host code).
//
// Reader: the semantics of ParallelIO::parallel_read_MM
// (cpp/io/parrallel_IO.hpp:31-88) at one rank: `coordinate` matrices, 1-based
// indices, duplicate entries merged into one, values not used by the embedding
// (the reference replaces them by the column id, cpp/dist_embed.cpp:168).  A
// `symmetric` (or skew/hermitian) header adds the mirrored entry of every
// off-diagonal one.  The CSR has columns ascending within a row.
//
// Writer: ParallelIO::parallel_write (cpp/io/parrallel_IO.hpp:90-146): per row
// the 1-based row id ("%lu"), then " %.5f" per component, then "\n"; no header.
#include <algorithm>
#include <cctype>
#include <cinttypes>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/distembed_gb300.h"

namespace de {
void set_thread_error(const std::string &msg);  // de_runtime.cpp
}

namespace {

struct MM {
  int64_t rows = 0, cols = 0;
  std::vector<int64_t> rowptr, col;
};

int io_fail(const std::string &m) {
  de::set_thread_error(m);
  return DE_ERR_INVALID;
}

std::string lower(std::string s) {
  for (char &c : s) c = char(std::tolower(static_cast<unsigned char>(c)));
  return s;
}

int read_mm(const char *path, MM &m) {
  FILE *f = std::fopen(path, "r");
  if (!f) return io_fail(std::string("cannot open ") + path);
  char line[4096];
  if (!std::fgets(line, sizeof line, f)) {
    std::fclose(f);
    return io_fail("empty MatrixMarket file");
  }
  char banner[64] = {0}, object[64] = {0}, format[64] = {0}, field[64] = {0}, symmetry[64] = {0};
  const int got = std::sscanf(line, "%63s %63s %63s %63s %63s", banner, object, format, field, symmetry);
  if (got < 4 || lower(banner) != "%%matrixmarket" || lower(object) != "matrix" || lower(format) != "coordinate") {
    std::fclose(f);
    return io_fail("not a MatrixMarket coordinate matrix");
  }
  const std::string sym = got >= 5 ? lower(symmetry) : "general";
  const bool mirror = sym == "symmetric" || sym == "skew-symmetric" || sym == "hermitian";
  int64_t nnz_decl = -1;
  while (std::fgets(line, sizeof line, f)) {
    if (line[0] == '%' || line[0] == '\n' || line[0] == '\r') continue;
    if (std::sscanf(line, "%" SCNd64 " %" SCNd64 " %" SCNd64, &m.rows, &m.cols, &nnz_decl) != 3) {
      std::fclose(f);
      return io_fail("bad MatrixMarket size line");
    }
    break;
  }
  if (nnz_decl < 0 || m.rows <= 0 || m.cols <= 0) {
    std::fclose(f);
    return io_fail("missing MatrixMarket size line");
  }
  std::vector<int64_t> key;
  key.reserve(size_t(mirror ? 2 : 1) * size_t(nnz_decl));
  int64_t read = 0;
  while (read < nnz_decl && std::fgets(line, sizeof line, f)) {
    if (line[0] == '%' || line[0] == '\n' || line[0] == '\r') continue;
    int64_t i = 0, j = 0;
    if (std::sscanf(line, "%" SCNd64 " %" SCNd64, &i, &j) != 2 || i < 1 || j < 1 || i > m.rows || j > m.cols) {
      std::fclose(f);
      return io_fail("bad MatrixMarket entry " + std::to_string(read + 1));
    }
    key.push_back((i - 1) * m.cols + (j - 1));
    if (mirror && i != j) {
      if (j > m.rows || i > m.cols) {
        std::fclose(f);
        return io_fail("symmetric entry outside the matrix");
      }
      key.push_back((j - 1) * m.cols + (i - 1));
    }
    ++read;
  }
  std::fclose(f);
  if (read != nnz_decl) return io_fail("MatrixMarket file ends early");
  std::sort(key.begin(), key.end());
  key.erase(std::unique(key.begin(), key.end()), key.end());  // duplicates merged
  m.rowptr.assign(size_t(m.rows) + 1, 0);
  m.col.resize(key.size());
  for (size_t e = 0; e < key.size(); ++e) {
    const int64_t r = key[e] / m.cols;
    m.col[e] = key[e] - r * m.cols;
    ++m.rowptr[size_t(r) + 1];
  }
  for (int64_t r = 0; r < m.rows; ++r) m.rowptr[r + 1] += m.rowptr[r];
  return DE_OK;
}

}  // namespace

extern "C" {

int de_mm_read(const char *path, int64_t *rows, int64_t *cols, int64_t *nnz, int64_t *rowptr, int64_t *col,
               int64_t capacity) {
  if (!path || !rows || !cols || !nnz) return io_fail("NULL argument");
  MM m;
  if (int rc = read_mm(path, m)) return rc;
  *rows = m.rows;
  *cols = m.cols;
  *nnz = int64_t(m.col.size());
  if (!rowptr && !col) return DE_OK;  // sizes only
  if (!rowptr || !col || capacity < int64_t(m.col.size())) return io_fail("rowptr/col missing or capacity below nnz");
  std::memcpy(rowptr, m.rowptr.data(), m.rowptr.size() * sizeof(int64_t));
  if (!m.col.empty()) std::memcpy(col, m.col.data(), m.col.size() * sizeof(int64_t));
  return DE_OK;
}

int de_embedding_write(const char *path, const double *x, int64_t rows, int32_t dim) {
  if (!path || !x || rows < 0 || dim <= 0) return io_fail("bad argument");
  FILE *f = std::fopen(path, "w");
  if (!f) return io_fail(std::string("cannot create ") + path);
  std::vector<char> buf(size_t(dim) * 24 + 32);
  for (int64_t i = 0; i < rows; ++i) {
    size_t k = size_t(std::snprintf(buf.data(), buf.size(), "%lu", static_cast<unsigned long>(i + 1)));
    for (int32_t d = 0; d < dim; ++d)
      k += size_t(std::snprintf(buf.data() + k, buf.size() - k, " %.5f", x[size_t(i) * dim + d]));
    buf[k++] = '\n';
    if (std::fwrite(buf.data(), 1, k, f) != k) {
      std::fclose(f);
      return io_fail(std::string("write failed: ") + path);
    }
  }
  if (std::fclose(f) != 0) return io_fail(std::string("close failed: ") + path);
  return DE_OK;
}

}  // extern "C"
