/*
 * TEST INFRASTRUCTURE ONLY — never linked into the product.
 *
 * Drives the reference's own embedding step, SpMM step and sparse embedding,
 * compiled unmodified from their sources (cpp/algo/algo.hpp, cpp/algo/spmm.hpp,
 * cpp/algo/sparse_embedding.hpp, cpp/core/common.cpp, cpp/net/process_3D_grid.cpp)
 * against the single-rank stand-ins in oracle/shim/.  It exposes a small C ABI
 * used to (1) pin the FP64 restatement in oracle/de_oracle.cpp bit-for-bit and
 * (2) write the golden vectors under tests/golden/.
 *
 * The objects are set up the way the reference's driver sets them up for one
 * rank (cpp/dist_embed.cpp:168-200, 237-241, 331-341): three SpMat copies of
 * the COO list (native, receiver = transpose, sender = column partitioned),
 * CSR blocks built through CSRLocal, a DenseMat whose coordinates are then
 * overwritten with the caller's initial embedding, and an EmbeddingAlgo with
 * alpha 0, beta 0.25, bounds +-5, row-major, async comm (the driver defaults).
 */
#include "algo/algo.hpp"
#include "algo/sparse_embedding.hpp"
#include "algo/spmm.hpp"

#include <cstring>
#include <memory>

using namespace distblas::core;
using namespace distblas::net;

namespace {

struct RefGraph {
  Process3DGrid grid{1, 1, 1, 1};
  std::unique_ptr<SpMat<double>> native, receiver, sender;
  INDEX_TYPE gRows = 0, gCols = 0, gNNz = 0;
  int batch = 0, prw = 0, pcw = 0;

  RefGraph(int64_t n, int64_t nnz, const int64_t *rowptr, const int64_t *col, int batch_size) {
    // COO list as the MatrixMarket reader leaves it: value = column id
    // (copy_col_to_value = true, cpp/dist_embed.cpp:168; parrallel_IO.hpp:62-64).
    vector<Tuple<double>> coords(nnz);
    for (int64_t i = 0; i < n; ++i)
      for (int64_t e = rowptr[i]; e < rowptr[i + 1]; ++e)
        coords[e] = Tuple<double>{i, col[e], double(col[e])};
    gRows = gCols = INDEX_TYPE(n);
    gNNz = INDEX_TYPE(nnz);
    batch = batch_size;
    prw = int(n);  // divide_and_round_up(gRows, 1)
    pcw = int(n);
    native = std::make_unique<SpMat<double>>(&grid, coords, gRows, gCols, gNNz, batch, prw, pcw,
                                             false, false);
    receiver = std::make_unique<SpMat<double>>(&grid, coords, gRows, gCols, gNNz, batch, prw,
                                               pcw, true, false);
    sender = std::make_unique<SpMat<double>>(&grid, coords, gRows, gCols, gNNz, batch, prw, pcw,
                                             false, true);
    native->initialize_CSR_blocks(true);
    receiver->initialize_CSR_blocks(true);
    sender->initialize_CSR_blocks(true);
  }
};

bool draws_in_range(int64_t n, int epochs, int batches, int ns) {
  for (int i = 0; i < epochs; ++i)
    for (int j = 0; j < batches; ++j) {
      vector<INDEX_TYPE> v = generate_random_numbers(0, int(n), i + j, ns);
      for (INDEX_TYPE x : v)
        if (x >= INDEX_TYPE(n)) return false;
    }
  return true;
}

template <size_t D>
int run_dim(int64_t n, int64_t nnz, const int64_t *rowptr, const int64_t *col, double *emb,
            int epochs, int batch, int ns, const double *lr, int use_driver_loop, int col_major) {
  int batches = int(n / batch) + (n % batch ? 1 : 0);
  // A draw equal to gRows makes the reference index a one-element cache
  // vector out of range (cpp/algo/algo.hpp:605-617 at one rank): undefined
  // behaviour, so such runs are refused rather than executed.
  if (!draws_in_range(n, epochs, batches, ns)) return -2;
  RefGraph g(n, nnz, rowptr, col, batch);
  DenseMat<INDEX_TYPE, double, D> dense(&g.grid, INDEX_TYPE(n));
  std::memcpy(dense.nCoordinates, emb, sizeof(double) * size_t(n) * D);
  distblas::algo::EmbeddingAlgo<INDEX_TYPE, double, D> algo(
      g.native.get(), g.receiver.get(), g.sender.get(), &dense, &g.grid, 0.0, 0.25, 5, -5,
      col_major != 0, false);
  if (use_driver_loop) {
    // The reference's own epoch/minibatch loop (cpp/algo/algo.hpp:74-262);
    // it takes one constant learning rate.
    reset_performance_timers();
    algo.algo_force2_vec_ns(epochs, batch, ns, lr[0]);
  } else {
    // The one-rank branch of that loop (cpp/algo/algo.hpp:164-192) with a
    // learning rate per epoch.
    int last_batch_size = (n % batch) ? int(n - int64_t(batch) * (batches - 1)) : batch;
    // the CSR the loop reads: the receiver's (transposed) one with col_major
    // (cpp/algo/algo.hpp:131-133)
    CSRLocal<double> *csr_block = col_major ? g.receiver->csr_local_data.get() : g.native->csr_local_data.get();
    vector<double> prev(size_t(batch) * D);
    int considering_batch_size = batch;
    for (int i = 0; i < epochs; ++i) {
      for (int j = 0; j < batches; ++j) {
        int seed = j + i;
        if (j == batches - 1) considering_batch_size = last_batch_size;
        vector<INDEX_TYPE> negs = generate_random_numbers(0, int(g.gRows), seed, ns);
        std::fill(prev.begin(), prev.end(), 0.0);
        algo.calc_t_dist_grad_rowptr(csr_block, prev.data(), lr[i], j, batch,
                                     considering_batch_size, true, false, 0, 0, false);
        algo.calc_t_dist_replus_rowptr(prev.data(), negs, lr[i], j, batch,
                                       considering_batch_size);
        algo.update_data_matrix_rowptr(prev.data(), j, batch);
      }
    }
  }
  std::memcpy(emb, dense.nCoordinates, sizeof(double) * size_t(n) * D);
  ::operator delete(dense.nCoordinates);
  return 0;
}

template <size_t D>
int grad_dim(int64_t n, int64_t nnz, const int64_t *rowptr, const int64_t *col,
             const double *emb, int batch, int ns, double lr, int batch_id, int seed,
             int considering_batch_size, double *prev_out) {
  vector<INDEX_TYPE> negs = generate_random_numbers(0, int(n), seed, ns);
  for (INDEX_TYPE x : negs)
    if (x >= INDEX_TYPE(n)) return -2;
  RefGraph g(n, nnz, rowptr, col, batch);
  DenseMat<INDEX_TYPE, double, D> dense(&g.grid, INDEX_TYPE(n));
  std::memcpy(dense.nCoordinates, emb, sizeof(double) * size_t(n) * D);
  distblas::algo::EmbeddingAlgo<INDEX_TYPE, double, D> algo(
      g.native.get(), g.receiver.get(), g.sender.get(), &dense, &g.grid, 0.0, 0.25, 5, -5,
      false, false);
  std::fill(prev_out, prev_out + size_t(batch) * D, 0.0);
  algo.calc_t_dist_grad_rowptr(g.native->csr_local_data.get(), prev_out, lr, batch_id, batch,
                               considering_batch_size, true, false, 0, 0, false);
  algo.calc_t_dist_replus_rowptr(prev_out, negs, lr, batch_id, batch, considering_batch_size);
  ::operator delete(dense.nCoordinates);
  return 0;
}

template <size_t D>
int spmm_dim(int64_t n, int64_t nnz, const int64_t *rowptr, const int64_t *col, const double *x, int batch,
             double lr, double *y) {
  RefGraph g(n, nnz, rowptr, col, batch);
  DenseMat<INDEX_TYPE, double, D> dense(&g.grid, INDEX_TYPE(n)), out(&g.grid, INDEX_TYPE(n));
  std::memcpy(dense.nCoordinates, x, sizeof(double) * size_t(n) * D);
  distblas::algo::SpMMAlgo<INDEX_TYPE, double, D> algo(g.native.get(), g.receiver.get(), g.sender.get(), &dense,
                                                       &out, &g.grid, 0.0, 0.25, false, false);
  reset_performance_timers();
  algo.algo_spmm(1, batch, lr);
  std::memcpy(y, out.nCoordinates, sizeof(double) * size_t(n) * D);
  ::operator delete(dense.nCoordinates);
  ::operator delete(out.nCoordinates);
  return 0;
}

template <size_t D>
int sparse_dim(int64_t n, int64_t nnz, const int64_t *rowptr, const int64_t *col, double *x, int iterations,
               int batch, int ns, double lr, double density, int merge, double *coll) {
  const int batches = int(n / batch + (n % batch ? 1 : 0));
  // merge = 1 runs the repulsive pass, whose draw equal to gRows reads another
  // rank's cache out of range (cpp/algo/sparse_embedding.hpp:516-537)
  if (merge && !draws_in_range(n, iterations, batches, ns)) return -2;
  RefGraph g(n, nnz, rowptr, col, batch);
  // the output matrix as the driver makes it (cpp/dist_embed.cpp:318), holding
  // the caller's values instead of rand() ones
  SpMat<double> out(&g.grid, INDEX_TYPE(n), INDEX_TYPE(D), false, false);
  for (int64_t i = 0; i < n; ++i)
    for (size_t d = 0; d < D; ++d) (*out.dense_collector)[i][d] = x[i * int64_t(D) + int64_t(d)];
  distblas::algo::SparseEmbedding<INDEX_TYPE, double, D> se(g.native.get(), g.receiver.get(), g.sender.get(), &out,
                                                           &g.grid, 0.0, 0.25, false, true, 0.5, false);
  // algo_sparse_embedding's one-rank loop (cpp/algo/sparse_embedding.hpp:78-194)
  // without the tile communicator, which the one-rank branch does not use; with
  // merge = 1 the local steps of the multi-rank branch (lines 145-168)
  const int expected_nnz_per_row = static_cast<int>(D * density);
  out.initialize_CSR_blocks(false, nullptr, static_cast<double>(INT_MIN), false);
  const int last_batch_size = (n % batch) ? int(n - int64_t(batch) * (batches - 1)) : batch;
  out.initialize_batch_collector(batch);
  CSRLocal<double> *csr_block = g.native->csr_local_data.get();
  int considering_batch_size = batch;
  for (int i = 0; i < iterations; ++i) {
    for (int j = 0; j < batches; ++j) {
      if (j == batches - 1) considering_batch_size = last_batch_size;
      vector<INDEX_TYPE> negs = generate_random_numbers(0, int(g.gRows), j + i, ns);
      if (merge) se.calc_t_dist_replus_rowptr(negs, lr, j, batch, considering_batch_size, &out);
      se.calc_t_dist_grad_rowptr(csr_block, lr, i, j, batch, considering_batch_size, 0, 0, 0, false, nullptr, &out);
      if (merge) out.merge_batch_collector(j, batch);
    }
    if (i < iterations - 1) {
      out.initialize_CSR_blocks(false, nullptr, static_cast<double>(INT_MIN), false);
      size_t size_r = out.csr_local_data->handler->rowStart.size();
      double output_nnz = out.csr_local_data->handler->rowStart[size_r - 1];
      auto output_nnz_per_row = static_cast<int>(output_nnz / g.receiver->proc_row_width);
      if (output_nnz_per_row > expected_nnz_per_row)
        se.preserveHighestK(out.dense_collector.get(), expected_nnz_per_row, static_cast<double>(INT_MIN));
    } else {
      out.initialize_CSR_blocks(false, nullptr, static_cast<double>(INT_MIN), true);
    }
  }
  for (int64_t i = 0; i < n; ++i)
    for (size_t d = 0; d < D; ++d) x[i * int64_t(D) + int64_t(d)] = (*out.dense_collector)[i][d];
  if (coll)
    for (int r = 0; r < batch; ++r)
      for (size_t d = 0; d < D; ++d) coll[size_t(r) * D + d] = (*out.batch_collector)[r][d];
  return 0;
}

}  // namespace

extern "C" {

/* The reference's sparse embedding at one rank (cpp/algo/sparse_embedding.hpp:
 * 78-194): x (n x dim, INT_MIN = absent) in place; coll (batch x dim, may be
 * NULL) receives the batch collector.  Returns 0, -1 for an unsupported dim, -2
 * when merge = 1 and a negative draw would hit the out-of-range path. */
int deref_sparse_embedding(int dim, int64_t n, int64_t nnz, const int64_t *rowptr, const int64_t *col, double *x,
                           int iterations, int batch, int ns, double lr, double density, int merge, double *coll) {
  switch (dim) {
    case 16: return sparse_dim<16>(n, nnz, rowptr, col, x, iterations, batch, ns, lr, density, merge, coll);
    case 32: return sparse_dim<32>(n, nnz, rowptr, col, x, iterations, batch, ns, lr, density, merge, coll);
    case 64: return sparse_dim<64>(n, nnz, rowptr, col, x, iterations, batch, ns, lr, density, merge, coll);
    case 128: return sparse_dim<128>(n, nnz, rowptr, col, x, iterations, batch, ns, lr, density, merge, coll);
  }
  return -1;
}

/* The reference's SpMM step, SpMMAlgo::algo_spmm(1, batch, lr)
 * (cpp/algo/spmm.hpp:54-159) as BaselineSpMM::execute runs it
 * (cpp/algo/baseline_spmm.hpp:63-88): y (n x dim) from x. */
int deref_spmm(int dim, int64_t n, int64_t nnz, const int64_t *rowptr, const int64_t *col, const double *x,
               int batch, double lr, double *y) {
  switch (dim) {
    case 16: return spmm_dim<16>(n, nnz, rowptr, col, x, batch, lr, y);
    case 32: return spmm_dim<32>(n, nnz, rowptr, col, x, batch, lr, y);
    case 64: return spmm_dim<64>(n, nnz, rowptr, col, x, batch, lr, y);
    case 128: return spmm_dim<128>(n, nnz, rowptr, col, x, batch, lr, y);
  }
  return -1;
}

/* Runs `epochs` epochs of the reference embedding step in place on emb (n x dim,
 * row-major FP64).  lr holds one rate per epoch; use_driver_loop = 1 calls
 * algo_force2_vec_ns itself (lr[0] only); col_major is the constructor's flag.
 * Returns 0, -1 for an unsupported dim, -2 when a negative draw would hit the
 * reference's out-of-range path. */
int deref_run(int dim, int64_t n, int64_t nnz, const int64_t *rowptr, const int64_t *col,
              double *emb, int epochs, int batch, int ns, const double *lr,
              int use_driver_loop, int col_major) {
  switch (dim) {
    case 16: return run_dim<16>(n, nnz, rowptr, col, emb, epochs, batch, ns, lr, use_driver_loop, col_major);
    case 32: return run_dim<32>(n, nnz, rowptr, col, emb, epochs, batch, ns, lr, use_driver_loop, col_major);
    case 64: return run_dim<64>(n, nnz, rowptr, col, emb, epochs, batch, ns, lr, use_driver_loop, col_major);
    case 128: return run_dim<128>(n, nnz, rowptr, col, emb, epochs, batch, ns, lr, use_driver_loop, col_major);
    case 256: return run_dim<256>(n, nnz, rowptr, col, emb, epochs, batch, ns, lr, use_driver_loop, col_major);
  }
  return -1;
}

/* One minibatch's accumulated update (prevCoordinates, batch x dim) before it
 * is applied: attractive pass then repulsive pass (cpp/algo/algo.hpp:177-190). */
int deref_batch_grad(int dim, int64_t n, int64_t nnz, const int64_t *rowptr, const int64_t *col,
                     const double *emb, int batch, int ns, double lr, int batch_id, int seed,
                     int considering_batch_size, double *prev_out) {
  switch (dim) {
    case 16: return grad_dim<16>(n, nnz, rowptr, col, emb, batch, ns, lr, batch_id, seed, considering_batch_size, prev_out);
    case 32: return grad_dim<32>(n, nnz, rowptr, col, emb, batch, ns, lr, batch_id, seed, considering_batch_size, prev_out);
    case 64: return grad_dim<64>(n, nnz, rowptr, col, emb, batch, ns, lr, batch_id, seed, considering_batch_size, prev_out);
    case 128: return grad_dim<128>(n, nnz, rowptr, col, emb, batch, ns, lr, batch_id, seed, considering_batch_size, prev_out);
    case 256: return grad_dim<256>(n, nnz, rowptr, col, emb, batch, ns, lr, batch_id, seed, considering_batch_size, prev_out);
  }
  return -1;
}

/* The reference's negative sampler (cpp/core/common.cpp:37-53). */
void deref_negatives(int lower, int upper, int seed, int ns, uint64_t *out) {
  vector<INDEX_TYPE> v = generate_random_numbers(lower, upper, seed, ns);
  for (int i = 0; i < ns; ++i) out[i] = v[i];
}

/* The CSR the reference's CSRLocal builds from a COO list for the native
 * (row-major, non-transposed) matrix.  rowptr_out has n+1 entries. */
int deref_csr(int64_t n, int64_t nnz, const int64_t *coo_row, const int64_t *coo_col,
              int64_t *rowptr_out, int64_t *col_out) {
  Process3DGrid grid(1, 1, 1, 1);
  vector<Tuple<double>> coords(nnz);
  for (int64_t k = 0; k < nnz; ++k) coords[k] = Tuple<double>{coo_row[k], coo_col[k], double(coo_col[k])};
  INDEX_TYPE gRows = n, gCols = n, gNNz = nnz;
  int batch = int(n), prw = int(n), pcw = int(n);
  SpMat<double> native(&grid, coords, gRows, gCols, gNNz, batch, prw, pcw, false, false);
  native.initialize_CSR_blocks(true);
  CSRHandle *h = native.csr_local_data->handler.get();
  for (int64_t i = 0; i <= n; ++i) rowptr_out[i] = h->rowStart[i];
  for (int64_t k = 0; k < nnz; ++k) col_out[k] = h->col_idx[k];
  return 0;
}

}  // extern "C"
