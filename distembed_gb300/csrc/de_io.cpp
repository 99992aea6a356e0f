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
#include <thread>
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

int parse_mm_keys(const char *path, MM &m, std::vector<int64_t> &key);

std::string lower(std::string s) {
  for (char &c : s) c = char(std::tolower(static_cast<unsigned char>(c)));
  return s;
}

}  // namespace

namespace de {

// Parses a MatrixMarket coordinate file into COO keys row * cols + col (0-based),
// the mirrored key of every off-diagonal entry added under a symmetric header;
// neither sorted nor merged.
int parse_mm(const char *path, int64_t *rows_out, int64_t *cols_out, std::vector<int64_t> &key) {
  MM m;
  const int rc = parse_mm_keys(path, m, key);
  *rows_out = m.rows;
  *cols_out = m.cols;
  return rc;
}

}  // namespace de

namespace {

// Decimal integer at p (leading blanks skipped, optional sign), as sscanf's %ld
// reads one; false when there is none or it does not fit.
bool scan_int(const char *&p, const char *end, int64_t &v) {
  while (p < end && (*p == ' ' || *p == '\t' || *p == '\r' || *p == '\v' || *p == '\f')) ++p;
  bool neg = false;
  if (p < end && (*p == '+' || *p == '-')) neg = *p++ == '-';
  const char *d0 = p;
  int64_t x = 0;
  while (p < end && *p >= '0' && *p <= '9') {
    if (p - d0 >= 18) return false;
    x = x * 10 + (*p++ - '0');
  }
  if (p == d0) return false;
  v = neg ? -x : x;
  return true;
}

// Entries of the lines in [b, e): (i, j) pairs in file order, up to the first line
// that is not an entry (err_at = the number of entries before it, else -1).
struct Chunk {
  std::vector<int64_t> ij;
  int64_t err_at = -1;
};

void parse_entries(const char *b, const char *e, int64_t rows, int64_t cols, Chunk &c) {
  for (const char *p = b; p < e;) {
    const char *nl = static_cast<const char *>(std::memchr(p, '\n', size_t(e - p)));
    const char *le = nl ? nl : e;
    if (p < le && *p != '%' && *p != '\r') {
      int64_t i = 0, j = 0;
      const char *q = p;
      if (!scan_int(q, le, i) || !scan_int(q, le, j) || i < 1 || j < 1 || i > rows || j > cols) {
        c.err_at = int64_t(c.ij.size() / 2);
        return;
      }
      c.ij.push_back(i);
      c.ij.push_back(j);
    }
    p = nl ? nl + 1 : e;
  }
}

int parse_mm_keys(const char *path, MM &m, std::vector<int64_t> &key) {
  FILE *f = std::fopen(path, "rb");
  if (!f) return io_fail(std::string("cannot open ") + path);
  std::vector<char> buf;
  if (std::fseek(f, 0, SEEK_END) == 0) {
    const long size = std::ftell(f);
    if (size > 0) {
      buf.resize(size_t(size));
      std::rewind(f);
      buf.resize(std::fread(buf.data(), 1, buf.size(), f));
    }
  }
  std::fclose(f);
  const char *p = buf.data(), *end = buf.data() + buf.size();
  auto next_line = [&](std::string &line) {
    if (p >= end) return false;
    const char *nl = static_cast<const char *>(std::memchr(p, '\n', size_t(end - p)));
    const char *le = nl ? nl : end;
    line.assign(p, le);
    p = nl ? nl + 1 : end;
    return true;
  };
  std::string line;
  if (!next_line(line)) return io_fail("empty MatrixMarket file");
  char banner[64] = {0}, object[64] = {0}, format[64] = {0}, field[64] = {0}, symmetry[64] = {0};
  const int got = std::sscanf(line.c_str(), "%63s %63s %63s %63s %63s", banner, object, format, field, symmetry);
  if (got < 4 || lower(banner) != "%%matrixmarket" || lower(object) != "matrix" || lower(format) != "coordinate")
    return io_fail("not a MatrixMarket coordinate matrix");
  const std::string sym = got >= 5 ? lower(symmetry) : "general";
  const bool mirror = sym == "symmetric" || sym == "skew-symmetric" || sym == "hermitian";
  int64_t nnz_decl = -1;
  while (next_line(line)) {
    if (line.empty() || line[0] == '%' || line[0] == '\r') continue;
    if (std::sscanf(line.c_str(), "%" SCNd64 " %" SCNd64 " %" SCNd64, &m.rows, &m.cols, &nnz_decl) != 3)
      return io_fail("bad MatrixMarket size line");
    break;
  }
  if (nnz_decl < 0 || m.rows <= 0 || m.cols <= 0) return io_fail("missing MatrixMarket size line");
  // entry lines in newline-aligned chunks, parsed by host threads
  const size_t bytes = size_t(end - p);
  const unsigned hw = std::max(1u, std::min(32u, std::thread::hardware_concurrency()));
  const int nchunks = bytes < (size_t(1) << 20) ? 1 : int(hw);
  std::vector<const char *> cut(size_t(nchunks) + 1, end);
  cut[0] = p;
  for (int c = 1; c < nchunks; ++c) {
    const char *q = std::max(cut[c - 1], p + bytes * size_t(c) / size_t(nchunks));
    const char *nl = q < end ? static_cast<const char *>(std::memchr(q, '\n', size_t(end - q))) : nullptr;
    cut[c] = nl ? nl + 1 : end;
  }
  std::vector<Chunk> chunks(static_cast<size_t>(nchunks));
  {
    std::vector<std::thread> pool;
    for (int c = 1; c < nchunks; ++c)
      pool.emplace_back(parse_entries, cut[c], cut[c + 1], m.rows, m.cols, std::ref(chunks[size_t(c)]));
    parse_entries(cut[0], cut[1], m.rows, m.cols, chunks[0]);
    for (auto &t : pool) t.join();
  }
  // entries in file order up to the declared count or the first bad line
  key.clear();
  key.reserve(size_t(mirror ? 2 : 1) * size_t(nnz_decl));
  int64_t read = 0;
  for (const Chunk &c : chunks) {
    const int64_t have = int64_t(c.ij.size() / 2);
    for (int64_t e = 0; e < have && read < nnz_decl; ++e, ++read) {
      const int64_t i = c.ij[size_t(2 * e)], j = c.ij[size_t(2 * e + 1)];
      key.push_back((i - 1) * m.cols + (j - 1));
      if (mirror && i != j) {
        if (j > m.rows || i > m.cols) return io_fail("symmetric entry outside the matrix");
        key.push_back((j - 1) * m.cols + (i - 1));
      }
    }
    if (read == nnz_decl) break;
    if (c.err_at >= 0) return io_fail("bad MatrixMarket entry " + std::to_string(read + 1));
  }
  if (read != nnz_decl) return io_fail("MatrixMarket file ends early");
  return DE_OK;
}

int read_mm(const char *path, MM &m) {
  std::vector<int64_t> key;
  if (int rc = parse_mm_keys(path, m, key)) return rc;
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
