/*
 * FP64 CPU restatement of DistEmbed's one-rank force-model SGD embedding step.
 *
 * TEST INFRASTRUCTURE ONLY.  Only tests/, __graft_entry__.smoke() and the CPU
 * legs of bench.py load this library, and only as the checker or the timed CPU
 * baseline; the product path never calls it.
 *
 * Parity is pinned bit-for-bit against the reference's own code (compiled by
 * `make -C oracle ref`) through the golden vectors in tests/golden/.
 *
 * Follows, line for line in arithmetic order:
 *   epoch/minibatch loop      cpp/algo/algo.hpp:74-88, 135, 164-192
 *   negative sampler          cpp/core/common.cpp:37-53
 *   attractive pass           cpp/algo/algo.hpp:389-417 (dispatch), 521-584 (body)
 *   repulsive pass            cpp/algo/algo.hpp:586-649
 *   update                    cpp/algo/algo.hpp:651-666
 *   clip                      cpp/algo/algo.hpp:65-72, bounds +-5 from cpp/dist_embed.cpp:341
 * with the reference's one-rank quirks switchable (quirks = 1 reproduces them):
 *   F7  edges into vertex n-1 are skipped: the destination filter is
 *       `dst_id < dst_end_index` with dst_end_index = gCols - 1 (algo.hpp:399-405, 538)
 *   F8  the repulsive row count becomes last_batch_size on the last batch of the
 *       first epoch and is never reset (algo.hpp:135, 167-169, 188-190, 594)
 * and one defined choice where the reference is undefined:
 *   F9  a negative draw equal to n (the sampler's upper bound is inclusive) makes
 *       the reference index a one-element vector out of range (algo.hpp:605-617).
 *       Such draws contribute nothing here, in both modes.
 * Also: the reference's SpMM step (oracle_spmm, cpp/algo/spmm.hpp:54-159, 358-412)
 * and its sparse embedding at one rank (oracle_sparse_embedding,
 * cpp/algo/sparse_embedding.hpp:78-194, 338-503, 505-659, 745-767).
 * The loss (absent from the reference) is the t-distribution objective whose
 * negative gradient is the force before clipping:
 *   attractive pair  log(1 + r)
 *   repulsive pair   log((1 + r) / (r + 1e-6))
 * with r the squared distance at the values the minibatch reads, summed in FP64.
 */
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <random>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

const double kBound = 5.0;  // MAX_BOUND, cpp/dist_embed.cpp:341

inline double clip(double v) {  // EmbeddingAlgo::scale, algo.hpp:65-72
  if (v > kBound) return kBound;
  if (v < -kBound) return -kBound;
  return v;
}

void negatives(int64_t n, int seed, int ns, int64_t *out) {
  std::minstd_rand gen(seed);
  std::uniform_int_distribution<int> dist(0, int(n));
  for (int k = 0; k < ns; ++k) out[k] = int64_t(dist(gen));
}

struct Batch {
  int64_t n;
  const int64_t *rowptr, *col;
  int dim;
  const double *x;     // embeddings, read only during the pass
  int batch, batch_id;
  double lr;
  bool quirks;
};

// Attractive pass for one source row (algo.hpp:531-582).  Returns the FP64
// attractive loss of the row.
inline double attract_row(const Batch &b, int64_t i, double *prev_row, double *fd, bool want_loss) {
  const int D = b.dim;
  const int64_t dst_end = b.quirks ? b.n - 1 : b.n;  // F7
  double loss = 0.0;
  for (int64_t e = b.rowptr[i]; e < b.rowptr[i + 1]; ++e) {
    const int64_t dst = b.col[e];
    if (!(dst >= 0 && dst < dst_end)) continue;
    double attrc = 0;
    for (int d = 0; d < D; ++d) {
      fd[d] = b.x[i * D + d] - b.x[dst * D + d];
      attrc += fd[d] * fd[d];
    }
    double d1 = -2.0 / (1.0 + attrc);
    for (int d = 0; d < D; ++d) {
      double l = clip(fd[d] * d1);
      prev_row[d] = prev_row[d] + (b.lr) * l;
    }
    if (want_loss) loss += std::log1p(attrc);
  }
  return loss;
}

// Repulsive pass for one row (algo.hpp:594-647).
inline double repulse_row(const Batch &b, int64_t row, const int64_t *negs, int ns,
                          double *prev_row, double *fd, bool want_loss) {
  const int D = b.dim;
  double loss = 0.0;
  for (int k = 0; k < ns; ++k) {
    const int64_t c = negs[k];
    if (c < 0 || c >= b.n) continue;  // F9
    double repuls = 0;
    for (int d = 0; d < D; ++d) {
      fd[d] = b.x[row * D + d] - b.x[c * D + d];
      repuls += fd[d] * fd[d];
    }
    double d1 = 2.0 / ((repuls + 0.000001) * (1.0 + repuls));
    for (int d = 0; d < D; ++d) {
      fd[d] = clip(fd[d] * d1);
      prev_row[d] += (b.lr) * fd[d];
    }
    if (want_loss) loss += std::log((1.0 + repuls) / (repuls + 0.000001));
  }
  return loss;
}

// One minibatch: prev = attractive + repulsive (rows < rep_rows), FP64 loss
// per row into row_loss.  Three parallel passes, as the reference runs them.
void batch_grad(const Batch &b, const int64_t *negs, int ns, int rep_rows, double *prev,
                double *row_loss) {
  const int D = b.dim;
  const int64_t src_begin = int64_t(b.batch_id) * b.batch;
  const int64_t src_end = std::min<int64_t>(src_begin + b.batch, b.n);  // exclusive
  const int64_t rows = src_end - src_begin;
  std::memset(prev, 0, sizeof(double) * size_t(b.batch) * D);
#pragma omp parallel
  {
    std::vector<double> fd(D);
#pragma omp for schedule(static)
    for (int64_t i = src_begin; i < src_end; ++i) {
      double l = attract_row(b, i, prev + (i - src_begin) * D, fd.data(), row_loss != nullptr);
      if (row_loss) row_loss[i - src_begin] = l;
    }
#pragma omp for schedule(static)
    for (int64_t i = 0; i < rep_rows; ++i) {
      double l = repulse_row(b, src_begin + i, negs, ns, prev + i * D, fd.data(), row_loss != nullptr);
      if (row_loss && i < rows) row_loss[i] += l;
    }
  }
}

// Rows of minibatch j that receive the repulsive pass in epoch `epoch` (F8:
// from the second epoch on, last_batch_size; algo.hpp:135, 167-169, 594).
int rep_rows_of(int64_t n, int batch, int epoch, int batch_id, bool quirks) {
  const int batches = int(n / batch) + (n % batch ? 1 : 0);
  const int last = (n % batch) ? int(n - int64_t(batch) * (batches - 1)) : batch;
  if (batch_id == batches - 1) return last;
  if (quirks && epoch > 0) return last;
  return batch;
}

// One graph's epochs [first_epoch, first_epoch + epochs) on one thread: the
// same minibatch loop as oracle_run (seed = epoch + batch, attractive pass,
// repulsive pass, update), the passes run row after row.  loss (nullable) gets
// each epoch's FP64 loss; returns the edge-updates performed.
int64_t run_graph_serial(int64_t n, const int64_t *rowptr, const int64_t *col, int dim, double *x,
                         int first_epoch, int epochs, int batch, int ns, const double *lr_per_epoch,
                         bool quirks, double *loss) {
  const int batches = int(n / batch) + (n % batch ? 1 : 0);
  std::vector<double> prev(static_cast<size_t>(batch) * dim);
  std::vector<double> fd(static_cast<size_t>(dim)), row_loss(static_cast<size_t>(batch));
  std::vector<int64_t> negs(size_t(std::max(ns, 1)));
  const int64_t dst_end = quirks ? n - 1 : n;
  int64_t updates = 0;
  for (int i = 0; i < epochs; ++i) {
    const int epoch = first_epoch + i;
    double epoch_loss = 0.0;
    for (int j = 0; j < batches; ++j) {
      negatives(n, epoch + j, ns, negs.data());
      Batch b{n, rowptr, col, dim, x, batch, j, lr_per_epoch[i], quirks};
      const int rep_rows = rep_rows_of(n, batch, epoch, j, quirks);
      const int64_t base = int64_t(j) * batch;
      const int64_t rows = std::min<int64_t>(base + batch, n) - base;
      std::fill(prev.begin(), prev.end(), 0.0);
      for (int64_t r = 0; r < rows; ++r) {
        row_loss[r] = attract_row(b, base + r, prev.data() + r * dim, fd.data(), loss != nullptr);
        for (int64_t e = rowptr[base + r]; e < rowptr[base + r + 1]; ++e) updates += (col[e] >= 0 && col[e] < dst_end);
      }
      int valid = 0;
      for (int k = 0; k < ns; ++k) valid += (negs[k] >= 0 && negs[k] < n);
      for (int64_t r = 0; r < rep_rows; ++r) {
        const double l = repulse_row(b, base + r, negs.data(), ns, prev.data() + r * dim, fd.data(), loss != nullptr);
        if (r < rows) row_loss[r] += l;
      }
      updates += int64_t(rep_rows) * valid;
      for (int64_t r = 0; r < rows; ++r)
        for (int d = 0; d < dim; ++d) x[(base + r) * dim + d] += prev[r * dim + d];
      if (loss)  // row by row, as oracle_run sums it
        for (int64_t r = 0; r < rows; ++r) epoch_loss += row_loss[r];
    }
    if (loss) loss[i] = epoch_loss;
  }
  return updates;
}

}  // namespace

extern "C" {

/* The reference's negative sampler: ns draws of
 * uniform_int_distribution<int>(0, n) from minstd_rand(seed). */
void oracle_negatives(int64_t n, int seed, int ns, int64_t *out) { negatives(n, seed, ns, out); }

/* Rows of minibatch j that receive the repulsive pass, in epoch i of one call. */
int oracle_rep_rows(int64_t n, int batch, int epoch_in_call, int batch_id, int quirks) {
  const int batches = int(n / batch) + (n % batch ? 1 : 0);
  const int last = (n % batch) ? int(n - int64_t(batch) * (batches - 1)) : batch;
  if (batch_id == batches - 1) return last;
  if (quirks && epoch_in_call > 0) return last;  // F8
  return batch;
}

/* One minibatch's accumulated update, before it is applied (batch x dim, FP64),
 * for batch `batch_id` drawn with `seed`; row_loss (nullable) gets each row's
 * FP64 loss.  Returns 0, or -1 on a bad argument. */
int oracle_batch_grad(int64_t n, const int64_t *rowptr, const int64_t *col, int dim,
                      const double *x, int batch, int ns, double lr, int batch_id, int seed,
                      int rep_rows, int quirks, double *prev_out, double *row_loss) {
  if (n <= 0 || dim <= 0 || batch <= 0 || ns < 0) return -1;
  std::vector<int64_t> negs(size_t(std::max(ns, 1)));
  negatives(n, seed, ns, negs.data());
  Batch b{n, rowptr, col, dim, x, batch, batch_id, lr, quirks != 0};
  batch_grad(b, negs.data(), ns, rep_rows, prev_out, row_loss);
  return 0;
}

/* `epochs` epochs of the one-rank embedding step in place on x (n x dim, FP64),
 * one learning rate per epoch; loss_per_epoch (nullable) gets the FP64 loss of
 * each epoch.  threads <= 0 keeps the OpenMP default.  Returns 0 or -1. */
int oracle_run(int64_t n, const int64_t *rowptr, const int64_t *col, int dim, double *x,
               int epochs, int batch, int ns, const double *lr_per_epoch, int quirks,
               double *loss_per_epoch, int threads) {
  if (n <= 0 || dim <= 0 || batch <= 0 || ns < 0 || epochs < 0) return -1;
#ifdef _OPENMP
  if (threads > 0) omp_set_num_threads(threads);
#endif
  const int batches = int(n / batch) + (n % batch ? 1 : 0);
  std::vector<double> prev(size_t(batch) * dim);
  std::vector<double> row_loss(static_cast<size_t>(batch));
  std::vector<int64_t> negs(size_t(std::max(ns, 1)));
  for (int i = 0; i < epochs; ++i) {
    double epoch_loss = 0.0;
    for (int j = 0; j < batches; ++j) {
      negatives(n, i + j, ns, negs.data());
      Batch b{n, rowptr, col, dim, x, batch, j, lr_per_epoch[i], quirks != 0};
      const int rep_rows = oracle_rep_rows(n, batch, i, j, quirks);
      batch_grad(b, negs.data(), ns, rep_rows, prev.data(), loss_per_epoch ? row_loss.data() : nullptr);
      const int64_t base = int64_t(j) * batch;
      const int64_t rows = std::min<int64_t>(base + batch, n) - base;
#pragma omp parallel for schedule(static)
      for (int64_t r = 0; r < rows; ++r)
        for (int d = 0; d < dim; ++d) x[(base + r) * dim + d] += prev[r * dim + d];
      if (loss_per_epoch)
        for (int64_t r = 0; r < rows; ++r) epoch_loss += row_loss[r];
    }
    if (loss_per_epoch) loss_per_epoch[i] = epoch_loss;
  }
  return 0;
}

/* A bounded sample of one epoch for timing: runs only the minibatches listed in
 * batch_ids (ascending), each exactly as oracle_run would in epoch
 * `epoch_in_call`, updating x in place.  Returns the number of edge-updates
 * performed (attractive entries plus repulsive (row, valid negative) pairs),
 * or -1 on a bad argument. */
int64_t oracle_run_batches(int64_t n, const int64_t *rowptr, const int64_t *col, int dim,
                           double *x, int epoch_in_call, int batch, int ns, double lr, int quirks,
                           const int32_t *batch_ids, int n_ids, int threads) {
  if (n <= 0 || dim <= 0 || batch <= 0 || ns < 0) return -1;
#ifdef _OPENMP
  if (threads > 0) omp_set_num_threads(threads);
#endif
  std::vector<double> prev(size_t(batch) * dim);
  std::vector<int64_t> negs(size_t(std::max(ns, 1)));
  int64_t updates = 0;
  for (int t = 0; t < n_ids; ++t) {
    const int j = batch_ids[t];
    negatives(n, epoch_in_call + j, ns, negs.data());
    Batch b{n, rowptr, col, dim, x, batch, j, lr, quirks != 0};
    const int rep_rows = oracle_rep_rows(n, batch, epoch_in_call, j, quirks);
    batch_grad(b, negs.data(), ns, rep_rows, prev.data(), nullptr);
    const int64_t base = int64_t(j) * batch;
    const int64_t rows = std::min<int64_t>(base + batch, n) - base;
#pragma omp parallel for schedule(static)
    for (int64_t r = 0; r < rows; ++r)
      for (int d = 0; d < dim; ++d) x[(base + r) * dim + d] += prev[r * dim + d];
    for (int64_t i = base; i < base + rows; ++i)
      for (int64_t e = rowptr[i]; e < rowptr[i + 1]; ++e) updates += (!quirks || col[e] < n - 1);
    int valid = 0;
    for (int k = 0; k < ns; ++k) valid += (negs[k] >= 0 && negs[k] < n);
    updates += int64_t(rep_rows) * valid;
  }
  return updates;
}

/* Many independent graphs, each one job of the one-rank step (the loop of
 * oracle_run, epochs [first_epoch, first_epoch + epochs) with the seeds and
 * repulsive row counts of those epochs), the graphs spread over `threads`
 * threads (largest first; a graph runs on one thread, its minibatches in
 * order).  x[g] is graph g's embedding (n[g] x dim, FP64), updated in place;
 * loss (nullable) gets [n_graphs x epochs] FP64 losses, and with loss NULL no
 * logarithm is taken.  Returns the edge-updates performed, or -1. */
int64_t oracle_run_many(int n_graphs, const int64_t *n, const int64_t *const *rowptr, const int64_t *const *col,
                        int dim, double *const *x, int first_epoch, int epochs, int batch, int ns,
                        const double *lr_per_epoch, int quirks, double *loss, int threads) {
  if (n_graphs < 0 || dim <= 0 || batch <= 0 || ns < 0 || epochs < 0 || first_epoch < 0) return -1;
  for (int g = 0; g < n_graphs; ++g)
    if (n[g] <= 0) return -1;
  std::vector<int> order(static_cast<size_t>(n_graphs));
  for (int g = 0; g < n_graphs; ++g) order[g] = g;
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) {
    return n[a] + rowptr[a][n[a]] > n[b] + rowptr[b][n[b]];
  });
  int64_t total = 0;
#ifdef _OPENMP
  const int nt = threads > 0 ? threads : omp_get_max_threads();
#pragma omp parallel for schedule(dynamic, 1) num_threads(nt) reduction(+ : total)
#endif
  for (int t = 0; t < n_graphs; ++t) {
    const int g = order[t];
    total += run_graph_serial(n[g], rowptr[g], col[g], dim, x[g], first_epoch, epochs, batch, ns, lr_per_epoch,
                              quirks != 0, loss ? loss + size_t(g) * epochs : nullptr);
  }
  return total;
}

/* SpMMAlgo::algo_spmm at one rank (cpp/algo/spmm.hpp:54-159): for every row i,
 * y[i] = sum over the CSR entries e of row i, in CSR order, of lr * x[col[e]]
 * (spmm.hpp:358-392, accumulated from zero as prevCoordinates, spmm.hpp:116-121,
 * then stored into the output matrix, spmm.hpp:397-412).  x is not changed; the
 * minibatch size only orders the rows, which do not depend on one another.  With
 * quirks, edges into vertex n-1 are skipped (the destination filter
 * `dst_id < dst_end_index`, dst_end_index = gCols - 1, spmm.hpp:260-265, 365). */
int oracle_spmm(int64_t n, const int64_t *rowptr, const int64_t *col, int dim, const double *x, double lr,
                int quirks, double *y) {
  const int64_t skip = quirks ? n - 1 : -1;
#pragma omp parallel for schedule(dynamic, 256)
  for (int64_t i = 0; i < n; ++i) {
    double *yi = y + i * dim;
    for (int d = 0; d < dim; ++d) yi[d] = 0.0;
    for (int64_t e = rowptr[i]; e < rowptr[i + 1]; ++e) {
      const int64_t c = col[e];
      if (c == skip) continue;
      const double *xc = x + c * dim;
      for (int d = 0; d < dim; ++d) yi[d] = yi[d] + lr * xc[d];
    }
  }
  return 0;
}

/* SparseEmbedding::algo_sparse_embedding at one rank (col_world_size == 1,
 * cpp/algo/sparse_embedding.hpp:78-194).  Embedding rows are dense FP64 vectors in
 * which the value INT_MIN marks an absent entry (the dense collector,
 * cpp/core/sparse_mat.hpp:367-377, 492-505).  Per iteration i and minibatch j
 * (rows [jB, min(jB + B, n))):
 *   merge = 0 (the reference's one-rank branch, lines 138-144): the attractive pass
 *     only.  Its updates go into the batch collector coll [B, dim], slot r for row
 *     jB + r, which that branch never merges nor clears: coll accumulates over all
 *     minibatches and iterations and the embedding values do not change.
 *   merge = 1 (the steps of the multi-rank branch that touch the local partition,
 *     lines 145-168): the repulsive pass on the minibatch's negatives (seed i + j),
 *     the attractive pass, then merge_batch_collector (sparse_mat.hpp:385-400):
 *     x = (x != INT_MIN ? x + coll : coll), coll = 0, for every entry of the rows.
 * Pair term (both passes, lines 380-427 and 548-598): the union of the two rows'
 * present entries in ascending dim order; value = x_i - x_j where both are
 * present, x_i or -x_j where one is; r = sum of value^2 in that order;
 * attractive d1 = -2 / (1 + r), repulsive d1 = 2 / ((r + 1e-6)(1 + r)); each union
 * entry k gets coll[k] += lr * clip(value_k * d1), clip at +-5 (lines 737-743).
 * After every iteration but the last, when floor(present entries / n) > k with
 * k = (int)(dim * density) (lines 172-181), every row keeps its k largest values
 * and the other dim - k become INT_MIN (preserveHighestK, lines 745-767; at equal
 * values the lower index is nullified first, which the reference leaves to its
 * heap's order).  After the last iteration absent entries become 0 (the final
 * CSR build with clear_dense_collector, lines 183-186,
 * cpp/core/distributed_mat.hpp:63-91).  A negative draw equal to n (the reference
 * would read another rank's cache out of range, lines 516-537) contributes
 * nothing.  With quirks, F8 holds for the repulsive pass of merge = 1: its row
 * count (block_size = considering_batch_size, lines 132-137, 146, 510-511) stays
 * last_batch_size from the last minibatch of the first iteration on.  coll (may
 * be NULL) receives the batch collector after the run.
 * Returns 0, or -1 for bad arguments. */
int oracle_sparse_embedding(int dim, int64_t n, const int64_t *rowptr, const int64_t *col, double *x,
                            int iterations, int batch, int ns, double lr, double density, int merge, int quirks,
                            double *coll_out) {
  if (dim <= 0 || n <= 0 || batch <= 0 || iterations < 0 || ns < 0) return -1;
  const double kAbsent = double(INT32_MIN);
  const int k_keep = static_cast<int>(dim * density);
  const int batches = int(n / batch + (n % batch ? 1 : 0));
  const int64_t last_batch_size = (n % batch) ? n - int64_t(batch) * (batches - 1) : batch;
  std::vector<double> coll(size_t(batch) * dim, 0.0);
  std::vector<int64_t> negs(size_t(std::max(ns, 1)));
  // one pair of rows: the union walk and the update of coll row `slot`
  auto pair = [&](int64_t i, int64_t j, bool attract, double *c) {
    const double *xi = x + i * dim, *xj = x + j * dim;
    double r = 0.0;
    for (int d = 0; d < dim; ++d) {
      const bool pi = xi[d] != kAbsent, pj = xj[d] != kAbsent;
      if (!pi && !pj) continue;
      const double v = (pi && pj) ? xi[d] - xj[d] : (pi ? xi[d] : -1 * xj[d]);
      r += v * v;
    }
    const double d1 = attract ? -2.0 / (1.0 + r) : 2.0 / ((r + 0.000001) * (1.0 + r));
    for (int d = 0; d < dim; ++d) {
      const bool pi = xi[d] != kAbsent, pj = xj[d] != kAbsent;
      if (!pi && !pj) continue;
      const double v = (pi && pj) ? xi[d] - xj[d] : (pi ? xi[d] : -1 * xj[d]);
      c[d] += lr * clip(v * d1);
    }
  };
  for (int it = 0; it < iterations; ++it) {
    for (int j = 0; j < batches; ++j) {
      const int64_t base = int64_t(j) * batch;
      const int64_t rows = (j == batches - 1) ? last_batch_size : batch;
      if (merge) {
        negatives(n, j + it, ns, negs.data());
        const int64_t rep_rows = (quirks && it > 0) ? last_batch_size : rows;
#pragma omp parallel for schedule(dynamic, 64)
        for (int64_t r = 0; r < rep_rows; ++r)
          for (int q = 0; q < ns; ++q)
            if (negs[q] >= 0 && negs[q] < n) pair(base + r, negs[q], false, coll.data() + r * dim);
      }
#pragma omp parallel for schedule(dynamic, 64)
      for (int64_t r = 0; r < rows; ++r)
        for (int64_t e = rowptr[base + r]; e < rowptr[base + r + 1]; ++e)
          pair(base + r, col[e], true, coll.data() + r * dim);
      if (merge) {
        for (int64_t r = 0; r < rows; ++r)
          for (int d = 0; d < dim; ++d) {
            double &xv = x[(base + r) * dim + d];
            double &cv = coll[size_t(r) * dim + d];
            xv = (xv != kAbsent) ? xv + cv : cv;
            cv = 0.0;
          }
      }
    }
    if (it < iterations - 1) {
      int64_t present = 0;
      for (int64_t e = 0; e < n * dim; ++e) present += x[e] != kAbsent;
      const int per_row = static_cast<int>(double(present) / double(n));
      if (per_row > k_keep) {
        const int nullify = dim - k_keep;
        std::vector<int> idx(dim);
        for (int64_t i = 0; i < n; ++i) {
          double *xi = x + i * dim;
          for (int d = 0; d < dim; ++d) idx[d] = d;
          std::stable_sort(idx.begin(), idx.end(), [&](int a, int b) { return xi[a] < xi[b]; });
          for (int q = 0; q < nullify && q < dim; ++q) xi[idx[q]] = kAbsent;
        }
      }
    } else {
      for (int64_t e = 0; e < n * dim; ++e)
        if (x[e] == kAbsent) x[e] = 0.0;
    }
  }
  if (coll_out) std::memcpy(coll_out, coll.data(), coll.size() * sizeof(double));
  return 0;
}

}  // extern "C"
