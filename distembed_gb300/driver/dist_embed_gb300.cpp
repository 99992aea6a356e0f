// dist_embed_gb300 — the reference's host driver (cpp/dist_embed.cpp) for the
// force-model embedding branch (cpp/dist_embed.cpp:330-347), on one GB300.
//
// Same flags, same input (MatrixMarket, cpp/io/parrallel_IO.hpp:31-88), same
// initial embedding (DenseMat, cpp/core/dense_mat.hpp:55-63: U[-1, 1) from the
// C library's rand(), unseeded), same entry (EmbeddingAlgo::algo_force2_vec_ns
// through GpuEmbeddingAlgo) and same output file (<output>/embedding.txt,
// cpp/io/parrallel_IO.hpp:90-146).  Extra flags: -dim (the reference fixes 128
// at compile time), -precision fp32|bf16, -device, -csr gpu|host.  -spmm 1 runs
// the reference's SpMM baseline instead (BaselineSpMM::execute,
// cpp/algo/baseline_spmm.hpp:52-90: per iteration a fresh DenseMat and one
// SpMMAlgo::algo_spmm step, timed).  -sparse_embedding 1 runs the reference's
// sparse embedding (cpp/dist_embed.cpp:317-330: an SpMat of rand() rows,
// SparseEmbedding::algo_sparse_embedding(iterations, batch, ns, lr, density), its
// rows written as embedding.txt) with -density (default 0.5) and the extra flag
// -sparse_merge 1 (merge the batch collector after every minibatch).  Flags that
// select the other algorithms of the reference (-spgemm, -msbfs) are refused;
// flags of the multi-rank exchange are accepted and not used.
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include "distembed_gb300.hpp"

namespace {

// The one-rank shapes the reference's EmbeddingAlgo constructor reads.
struct CSRHandle {
  std::vector<int64_t> rowStart, col_idx;
};
struct CSRLocal {
  std::unique_ptr<CSRHandle> handler = std::make_unique<CSRHandle>();
};
struct SpMat {
  std::unique_ptr<CSRLocal> csr_local_data = std::make_unique<CSRLocal>();
  int64_t gRows = 0, gCols = 0, gNNz = 0;
};
struct DenseMat {
  uint64_t rows = 0;
  double *nCoordinates = nullptr;
};
struct Grid {};

struct Flags {
  std::string input, output = "embedding.txt", dataset;
  int batch_size = 16384, iterations = 30, ns = 5, dim = 128, device = 0;
  double alpha = 0, beta = 0.25, lr = 0.02;
  bool col_major = false, sync_comm = false;
  bool gpu_csr = true;  // -csr gpu|host: where the input's COO -> CSR runs
  bool spmm = false;    // -spmm 1: the SpMM baseline (cpp/dist_embed.cpp:255-268)
  bool sparse = false;  // -sparse_embedding 1 (cpp/dist_embed.cpp:317-330)
  bool sparse_merge = false;
  double density = 0.5;  // cpp/dist_embed.cpp:62
  int precision = DE_PRECISION_FP32;
};

// The receiver matrix's CSR: the transpose of the native one (cpp/dist_embed.cpp:197-200,
// CSRLocal with transpose = true), columns ascending in each row; it has `cols` rows.
void transpose_csr(const CSRHandle &a, int64_t rows, int64_t cols, CSRHandle &t) {
  const int64_t nnz = a.rowStart[size_t(rows)];
  t.rowStart.assign(size_t(cols) + 1, 0);
  t.col_idx.assign(size_t(nnz > 0 ? nnz : 1), 0);
  for (int64_t e = 0; e < nnz; ++e) t.rowStart[size_t(a.col_idx[size_t(e)]) + 1]++;
  for (int64_t c = 0; c < cols; ++c) t.rowStart[size_t(c) + 1] += t.rowStart[size_t(c)];
  std::vector<int64_t> fill(t.rowStart.begin(), t.rowStart.end() - 1);
  for (int64_t r = 0; r < rows; ++r)
    for (int64_t e = a.rowStart[size_t(r)]; e < a.rowStart[size_t(r) + 1]; ++e)
      t.col_idx[size_t(fill[size_t(a.col_idx[size_t(e)])]++)] = r;
}

template <size_t D>
double run(const Flags &f, SpMat &sp, SpMat &receiver, DenseMat &dense, std::vector<double> &loss) {
  Grid grid;
  // with -col_major 1 the passes read the receiver's CSR (cpp/algo/algo.hpp:131-133)
  distembed_gb300::GpuEmbeddingAlgo<int64_t, double, D> algo(&sp, &receiver, &sp, &dense, &grid, f.alpha, f.beta,
                                                             5.0, -5.0, f.col_major, f.sync_comm, f.precision,
                                                             f.device);
  const auto t0 = std::chrono::steady_clock::now();
  algo.algo_force2_vec_ns(f.iterations, f.batch_size, f.ns, f.lr);
  const double s = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  loss = algo.last_loss();
  return s;
}

// BaselineSpMM::execute (cpp/algo/baseline_spmm.hpp:52-90) at one rank: per
// iteration a fresh input DenseMat (U[-1, 1) from rand(), dense_mat.hpp:55-63) and
// one SpMMAlgo::algo_spmm(1, batch, lr) step into an output DenseMat, timed; the
// timings are appended to perf_output.
int run_spmm(const Flags &f, const CSRHandle &csr, int64_t rows, int64_t nnz) {
  de_options o;
  de_default_options(&o);
  o.device = f.device;
  de_handle *h = nullptr;
  if (de_create(rows, csr.rowStart.data(), csr.col_idx.data(), nnz, f.dim, &o, &h) != DE_OK) {
    std::fprintf(stderr, "spmm: %s\n", de_last_error(nullptr));
    return 1;
  }
  std::vector<double> x(size_t(rows) * size_t(f.dim)), y(x.size());
  std::vector<double> secs;
  for (int it = 0; it < f.iterations; ++it) {
    for (double &v : x) v = -1.0 + 2.0 * std::rand() / (RAND_MAX + 1.0);
    const auto t0 = std::chrono::steady_clock::now();
    if (de_set_embeddings(h, x.data()) != DE_OK || de_spmm(h, f.batch_size, f.lr, y.data()) != DE_OK) {
      std::fprintf(stderr, "spmm: %s\n", de_last_error(h));
      de_destroy(h);
      return 1;
    }
    secs.push_back(std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count());
    std::printf(" rank 0 SpMM iteration %d completed in %.4f s\n", it, secs.back());
  }
  de_destroy(h);
  if (FILE *pf = std::fopen("perf_output", "a")) {
    std::fprintf(pf, "{\"algo\":\"SpMM\",\"p\":1,\"data_set\":\"%s\",\"device\":\"GB300\",\"batch\":%d,"
                     "\"iteration_time_s\":[", f.dataset.c_str(), f.batch_size);
    for (size_t i = 0; i < secs.size(); ++i) std::fprintf(pf, "%s%.6f", i ? "," : "", secs[i]);
    std::fprintf(pf, "]}\n");
    std::fclose(pf);
  }
  return 0;
}

// The -sparse_embedding branch at one rank (cpp/dist_embed.cpp:317-330): the
// output SpMat's rows from rand() (sparse_mat.hpp:367-377, row-major, the same
// draws as DenseMat's), the sparse embedding, its rows written by parallel_write.
int run_sparse(const Flags &f, const CSRHandle &csr, int64_t rows, int64_t nnz) {
  de_options o;
  de_default_options(&o);
  o.device = f.device;
  de_handle *h = nullptr;
  if (de_create(rows, csr.rowStart.data(), csr.col_idx.data(), nnz, f.dim, &o, &h) != DE_OK) {
    std::fprintf(stderr, "sparse_embedding: %s\n", de_last_error(nullptr));
    return 1;
  }
  std::vector<double> x(size_t(rows) * size_t(f.dim));
  for (double &v : x) v = -1.0 + 2.0 * std::rand() / (RAND_MAX + 1.0);
  const auto t0 = std::chrono::steady_clock::now();
  const int rc = de_sparse_embedding(h, x.data(), f.iterations, f.batch_size, f.ns, f.lr, f.density,
                                     f.sparse_merge ? 1 : 0, nullptr);
  const double secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  if (rc != DE_OK) {
    std::fprintf(stderr, "sparse_embedding: %s\n", de_last_error(h));
    de_destroy(h);
    return 1;
  }
  de_destroy(h);
  std::printf(" rank 0 sparse embedding completed in %.3f s\n", secs);
  const std::string out = f.output + "/embedding.txt";
  if (de_embedding_write(out.c_str(), x.data(), rows, f.dim) != DE_OK) {
    std::fprintf(stderr, "writing %s: %s\n", out.c_str(), de_last_error(nullptr));
    return 1;
  }
  if (FILE *pf = std::fopen("perf_output", "a")) {
    std::fprintf(pf, "{\"algo\":\"SparseEmbedding\",\"p\":1,\"data_set\":\"%s\",\"device\":\"GB300\","
                     "\"total_time_s\":%.6f,\"iterations\":%d,\"batch\":%d,\"density\":%g,\"merge\":%d}\n",
                 f.dataset.c_str(), secs, f.iterations, f.batch_size, f.density, f.sparse_merge ? 1 : 0);
    std::fclose(pf);
  }
  return 0;
}

}  // namespace

int main(int argc, char **argv) {
  Flags f;
  for (int p = 0; p + 1 < argc; p++) {
    const char *a = argv[p], *v = argv[p + 1];
    if (!std::strcmp(a, "-input")) f.input = v;
    else if (!std::strcmp(a, "-output")) f.output = v;
    else if (!std::strcmp(a, "-batch")) f.batch_size = std::atoi(v);
    else if (!std::strcmp(a, "-iter")) f.iterations = std::atoi(v);
    else if (!std::strcmp(a, "-alpha")) f.alpha = std::atof(v);
    else if (!std::strcmp(a, "-lr")) f.lr = std::atof(v);
    else if (!std::strcmp(a, "-nsamples")) f.ns = std::atoi(v);
    else if (!std::strcmp(a, "-beta")) f.beta = std::atof(v);
    else if (!std::strcmp(a, "-dataset")) f.dataset = v;
    else if (!std::strcmp(a, "-col_major")) f.col_major = std::atoi(v) != 0;
    else if (!std::strcmp(a, "-sync_comm")) f.sync_comm = std::atoi(v) != 0;
    else if (!std::strcmp(a, "-dim")) f.dim = std::atoi(v);
    else if (!std::strcmp(a, "-device")) f.device = std::atoi(v);
    else if (!std::strcmp(a, "-csr")) f.gpu_csr = std::strcmp(v, "host") != 0;
    else if (!std::strcmp(a, "-precision")) f.precision = std::strcmp(v, "bf16") ? DE_PRECISION_FP32 : DE_PRECISION_BF16;
    else if (!std::strcmp(a, "-spmm")) f.spmm = std::atoi(v) == 1;
    else if (!std::strcmp(a, "-sparse_embedding")) f.sparse = std::atoi(v) == 1;
    else if (!std::strcmp(a, "-sparse_merge")) f.sparse_merge = std::atoi(v) == 1;
    else if (!std::strcmp(a, "-density")) f.density = std::atof(v);
    else if ((!std::strcmp(a, "-spgemm") || !std::strcmp(a, "-msbfs")) && std::atoi(v) == 1) {
      std::fprintf(stderr, "%s: only the force-model embedding, the SpMM baseline and the sparse embedding are "
                           "provided by this build\n", a);
      return 2;
    }
  }
  if (f.input.empty()) {
    std::fprintf(stderr, "usage: %s -input graph.mtx [-output dir] [-iter 30] [-batch 16384] [-nsamples 5] "
                         "[-lr 0.02] [-dim 128] [-precision fp32|bf16] [-device 0] [-csr gpu|host]\n", argv[0]);
    return 2;
  }
  // ---- input (cpp/dist_embed.cpp:165): parsed on the host, COO -> CSR on the GPU
  // (or on the host with -csr host)
  SpMat sp;
  int64_t rows = 0, cols = 0, nnz = 0;
  CSRHandle &csr = *sp.csr_local_data->handler;
  const auto t_read = std::chrono::steady_clock::now();
  if (f.gpu_csr) {
    de_csr *c = nullptr;
    if (de_mm_read_gpu(f.input.c_str(), f.device, &c) != DE_OK) {
      std::fprintf(stderr, "reading %s: %s\n", f.input.c_str(), de_last_error(nullptr));
      return 1;
    }
    de_csr_info(c, &rows, &cols, &nnz);
    csr.rowStart.resize(size_t(rows) + 1);
    csr.col_idx.resize(size_t(nnz > 0 ? nnz : 1));
    de_csr_copy(c, csr.rowStart.data(), csr.col_idx.data());
    de_csr_free(c);
  } else {
    if (de_mm_read(f.input.c_str(), &rows, &cols, &nnz, nullptr, nullptr, 0) != DE_OK) {
      std::fprintf(stderr, "reading %s: %s\n", f.input.c_str(), de_last_error(nullptr));
      return 1;
    }
    csr.rowStart.resize(size_t(rows) + 1);
    csr.col_idx.resize(size_t(nnz > 0 ? nnz : 1));
    if (de_mm_read(f.input.c_str(), &rows, &cols, &nnz, csr.rowStart.data(), csr.col_idx.data(),
                   int64_t(csr.col_idx.size())) != DE_OK) {
      std::fprintf(stderr, "reading %s: %s\n", f.input.c_str(), de_last_error(nullptr));
      return 1;
    }
  }
  const double read_s = std::chrono::duration<double>(std::chrono::steady_clock::now() - t_read).count();
  if (cols > rows) {
    std::fprintf(stderr, "the graph has more columns (%lld) than rows (%lld)\n", (long long)cols, (long long)rows);
    return 1;
  }
  sp.gRows = rows;
  sp.gCols = cols;
  sp.gNNz = nnz;
  std::printf(" rank 0 gROWs  %lld gCols %lld nnz %lld\n", (long long)rows, (long long)cols, (long long)nnz);
  if (f.spmm) return run_spmm(f, csr, rows, nnz);
  if (f.sparse) return run_sparse(f, csr, rows, nnz);
  // ---- initial embedding (cpp/core/dense_mat.hpp:55-63)
  std::vector<double> coords(size_t(rows) * size_t(f.dim));
  for (size_t i = 0; i < coords.size(); ++i) coords[i] = -1.0 + 2.0 * std::rand() / (RAND_MAX + 1.0);
  DenseMat dense;
  dense.rows = uint64_t(rows);
  dense.nCoordinates = coords.data();
  // ---- the algorithm (cpp/dist_embed.cpp:331-344)
  SpMat receiver;
  if (f.col_major) transpose_csr(csr, rows, cols, *receiver.csr_local_data->handler);
  SpMat &rec = f.col_major ? receiver : sp;
  std::vector<double> loss;
  double secs = 0;
  try {
    switch (f.dim) {
      case 32: secs = run<32>(f, sp, rec, dense, loss); break;
      case 64: secs = run<64>(f, sp, rec, dense, loss); break;
      case 128: secs = run<128>(f, sp, rec, dense, loss); break;
      case 256: secs = run<256>(f, sp, rec, dense, loss); break;
      default: std::fprintf(stderr, "-dim must be 32, 64, 128 or 256\n"); return 2;
    }
  } catch (const distembed_gb300::Error &e) {
    std::fprintf(stderr, "embedding failed: %s\n", e.what());
    return 1;
  }
  std::printf(" rank 0 algo completed in %.3f s, final loss %.6e\n", secs, loss.empty() ? 0.0 : loss.back());
  // ---- output (cpp/dist_embed.cpp:346)
  const std::string out = f.output + "/embedding.txt";
  if (de_embedding_write(out.c_str(), coords.data(), rows, f.dim) != DE_OK) {
    std::fprintf(stderr, "writing %s: %s\n", out.c_str(), de_last_error(nullptr));
    return 1;
  }
  // ---- timing record (the reference appends its perf JSON to "perf_output")
  if (FILE *pf = std::fopen("perf_output", "a")) {
    std::fprintf(pf, "{\"alpha\":%g,\"beta\":%g,\"algo\":\"Embedding\",\"p\":1,\"data_set\":\"%s\",\"device\":\"GB300\","
                     "\"total_time_s\":%.6f,\"iterations\":%d,\"batch\":%d,\"ns\":%d,\"read_s\":%.6f,"
                     "\"csr\":\"%s\"}\n",
                 f.alpha, f.beta, f.dataset.c_str(), secs, f.iterations, f.batch_size, f.ns, read_s,
                 f.gpu_csr ? "gpu" : "host");
    std::fclose(pf);
  }
  return 0;
}
