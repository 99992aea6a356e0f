/*
 * distembed_gb300.hpp — C++ drop-in for DistEmbed's EmbeddingAlgo on one GB300.
 *
 *   distblas::algo::EmbeddingAlgo<INDEX_TYPE, VALUE_TYPE, embedding_dim>   (cpp/algo/algo.hpp:54-74)
 *   distembed_gb300::GpuEmbeddingAlgo<INDEX_TYPE, VALUE_TYPE, embedding_dim>
 *
 * Same constructor arguments and the same algo_force2_vec_ns(iterations,
 * batch_size, ns, lr) entry (cpp/algo/algo.hpp:74): the caller's driver
 * (cpp/dist_embed.cpp:331-346) changes only the class name.  The constructor
 * reads the one-rank CSR of the native matrix
 * (native->csr_local_data->handler->rowStart / col_idx, cpp/core/common.h:127-131)
 * and keeps it resident on the GPU; algo_force2_vec_ns uploads
 * dense->nCoordinates (cpp/core/dense_mat.hpp:34), runs the epochs on the GPU
 * and writes the embedding back in place, as the reference does.  receiver,
 * sender, grid, alpha, beta and sync_comm steer the multi-rank exchange, which
 * one resident partition does not have: they are accepted and not used.
 * col_major selects the CSR the passes read, as the reference's loop does
 * (cpp/algo/algo.hpp:131-133): the receiver matrix's, built with transpose = true
 * (cpp/dist_embed.cpp:197-200), so on an asymmetric graph a row takes its
 * attractive forces from its in-neighbours.  The traversal stays the row-major
 * one: the one-rank branch calls the attractive pass with col_major = false
 * whatever the flag (algo.hpp:184-186); the transposed traversal (algo.hpp:450-518,
 * racy in the reference) runs only in the multi-rank exchange.
 *
 * Errors throw distembed_gb300::Error (a std::runtime_error) with the library's
 * message, where the reference prints and exits.
 */
#ifndef DISTEMBED_GB300_HPP
#define DISTEMBED_GB300_HPP

#include <algorithm>
#include <cstddef>
#include <cstdint>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <vector>

#include "distembed_gb300.h"

namespace distembed_gb300 {

class Error : public std::runtime_error {
 public:
  Error(int code, const std::string &msg) : std::runtime_error(msg), code_(code) {}
  int code() const { return code_; }

 private:
  int code_;
};

inline void check(int rc, const de_handle *h) {
  if (rc != DE_OK) throw Error(rc, de_last_error(h));
}

template <typename INDEX_TYPE, typename VALUE_TYPE, size_t embedding_dim>
class GpuEmbeddingAlgo {
  static_assert(std::is_same<VALUE_TYPE, double>::value || std::is_same<VALUE_TYPE, float>::value,
                "VALUE_TYPE must be double or float");

 public:
  /* The reference constructor (cpp/algo/algo.hpp:54-63). */
  template <class SpMat, class DenseMat, class Grid>
  GpuEmbeddingAlgo(SpMat *native, SpMat *receiver, SpMat * /*sender*/, DenseMat *dense, Grid * /*grid*/,
                   double /*alpha*/, double /*beta*/, VALUE_TYPE MAX_BOUND, VALUE_TYPE MIN_BOUND, bool col_major,
                   bool /*sync_comm*/, int precision = DE_PRECISION_FP32, int device = 0) {
    const auto &csr = col_major ? *receiver->csr_local_data->handler : *native->csr_local_data->handler;
    const int64_t n = int64_t(dense->rows);
    // a transposed CSR of a matrix with fewer columns than rows has fewer row
    // pointers: the rows past them have no entries
    const int64_t have = std::min<int64_t>(int64_t(csr.rowStart.size()), n + 1);
    std::vector<int64_t> rowptr(csr.rowStart.begin(), csr.rowStart.begin() + have);
    rowptr.resize(size_t(n + 1), have > 0 ? rowptr[size_t(have - 1)] : 0);
    std::vector<int64_t> col(csr.col_idx.begin(), csr.col_idx.begin() + rowptr[n]);
    init(n, rowptr.data(), col.data(), dense->nCoordinates, MAX_BOUND, MIN_BOUND, col_major, precision, device);
  }

  /* The same on plain arrays: n vertices, CSR rowptr[n+1] / col[rowptr[n]],
   * coordinates n x embedding_dim row-major (updated in place by each call). */
  GpuEmbeddingAlgo(int64_t n, const int64_t *rowptr, const int64_t *col, VALUE_TYPE *coordinates,
                   VALUE_TYPE MAX_BOUND = 5, VALUE_TYPE MIN_BOUND = -5, bool col_major = false,
                   int precision = DE_PRECISION_FP32, int device = 0) {
    init(n, rowptr, col, coordinates, MAX_BOUND, MIN_BOUND, col_major, precision, device);
  }

  GpuEmbeddingAlgo(const GpuEmbeddingAlgo &) = delete;
  GpuEmbeddingAlgo &operator=(const GpuEmbeddingAlgo &) = delete;
  ~GpuEmbeddingAlgo() { de_destroy(h_); }

  /* cpp/algo/algo.hpp:74: `iterations` epochs of minibatch force-model SGD. */
  void algo_force2_vec_ns(int iterations, int batch_size, int ns, VALUE_TYPE lr) {
    set();
    std::vector<double> lrs(size_t(iterations > 0 ? iterations : 1), double(lr));
    loss_.assign(size_t(iterations > 0 ? iterations : 0), 0.0);
    check(de_run(h_, iterations, batch_size, ns, lrs.data(), iterations > 0 ? loss_.data() : nullptr), h_);
    get();
  }

  /* One learning rate per epoch (the reference takes one constant rate). */
  void algo_force2_vec_ns(int iterations, int batch_size, int ns, const std::vector<double> &lr_per_epoch) {
    if (lr_per_epoch.size() < size_t(iterations)) throw Error(DE_ERR_INVALID, "lr_per_epoch is too short");
    set();
    loss_.assign(size_t(iterations > 0 ? iterations : 0), 0.0);
    check(de_run(h_, iterations, batch_size, ns, lr_per_epoch.data(), iterations > 0 ? loss_.data() : nullptr), h_);
    get();
  }

  /* FP64 loss of each epoch of the last call. */
  const std::vector<double> &last_loss() const { return loss_; }
  de_handle *handle() { return h_; }

 private:
  void init(int64_t n, const int64_t *rowptr, const int64_t *col, VALUE_TYPE *coordinates, VALUE_TYPE max_bound,
            VALUE_TYPE min_bound, bool col_major, int precision, int device) {
    (void)col_major;  // the CSR was chosen by the caller; the pass is row-major (algo.hpp:184-186)
    if (min_bound != -max_bound) throw Error(DE_ERR_INVALID, "the bounds must be [-MAX_BOUND, MAX_BOUND]");
    de_options o;
    de_default_options(&o);
    o.precision = precision;
    o.device = device;
    o.max_bound = double(max_bound);
    n_ = n;
    x_ = coordinates;
    check(de_create(n, rowptr, col, rowptr[n], int32_t(embedding_dim), &o, &h_), nullptr);
  }
  void set() {
    if (std::is_same<VALUE_TYPE, double>::value)
      check(de_set_embeddings(h_, reinterpret_cast<const double *>(x_)), h_);
    else
      check(de_set_embeddings_f32(h_, reinterpret_cast<const float *>(x_), 0), h_);
  }
  void get() {
    if (std::is_same<VALUE_TYPE, double>::value)
      check(de_get_embeddings(h_, reinterpret_cast<double *>(x_)), h_);
    else
      check(de_get_embeddings_f32(h_, reinterpret_cast<float *>(x_), 0), h_);
  }

  de_handle *h_ = nullptr;
  int64_t n_ = 0;
  VALUE_TYPE *x_ = nullptr;
  std::vector<double> loss_;
};

}  // namespace distembed_gb300

#endif /* DISTEMBED_GB300_HPP */
