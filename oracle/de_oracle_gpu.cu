/*
 * FP64 GPU restatement of DistEmbed's one-rank force-model SGD embedding step.
 *
 * TEST INFRASTRUCTURE ONLY: the checker for sizes the CPU restatement
 * (oracle/de_oracle.cpp) cannot finish in reasonable time (R-MAT scale 22,
 * dim 256, 1024 shared negatives: ~4e12 FP64 operations per epoch).  Only
 * tests/ and bench.py's oracle-gap legs load it; the product never does.
 *
 * It performs the arithmetic of oracle/de_oracle.cpp (which is pinned bit for
 * bit to the reference's cpp/algo/algo.hpp:74-262, 521-666) in the same order
 * and without fused multiply-adds (every product and sum through __dmul_rn /
 * __dadd_rn / __dsub_rn, divisions IEEE-rounded), so the embeddings it returns
 * are bitwise those of the CPU restatement:
 *   pass 1  one thread per (row, other row) pair: the squared distance summed over
 *           the dims in order (attrc / repuls, algo.hpp:540-558, 605-625), then
 *           the coefficient d1 = -2/(1 + r) (attractive) or 2/((r + 1e-6)(1 + r))
 *           (repulsive) and the pair's loss term;
 *   pass 2  one warp per row, lanes over the dims: prev[d] += lr * clip(diff[d] * d1)
 *           over the row's CSR entries in order, then over the negatives in draw
 *           order (algo.hpp:559-580, 626-647);
 *   pass 3  x[row] += prev (algo.hpp:651-666).
 * The negatives come from the same host sampler (std::minstd_rand(epoch + batch)
 * and std::uniform_int_distribution<int>(0, n), cpp/core/common.cpp:37-53), the
 * quirks F7 / F8 / F9 are those of oracle_run.  The loss uses the GPU's FP64 log
 * (within an ulp of the host's), summed per row and then over rows in order on
 * the host, as oracle_run sums it.
 */
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <random>
#include <vector>

namespace {

struct PassArgs {
  const double *x;
  const int64_t *rowptr, *col;
  const int64_t *negs;   // this minibatch's draws
  int64_t n, base;       // minibatch rows [base, base + rows)
  int rows, rep_rows, ns, dim, quirks;
  const int64_t *pair_off;  // [rows + 1]: first pair of each row (attractive, then repulsive)
  double *d1;            // [pairs] coefficient, 0 for pairs that do not count
  double *ploss;         // [pairs] loss term, 0 for pairs that do not count
  double *prev;          // [rows, dim]
  double *row_loss;      // [rows]
  double lr;
};

__device__ __forceinline__ double clip5(double v) { return v > 5.0 ? 5.0 : (v < -5.0 ? -5.0 : v); }

// The other row of pair p of row i (local r), or -1 when the pair does not count.
__device__ __forceinline__ int64_t pair_other(const PassArgs &a, int r, int64_t p, bool &attract) {
  const int64_t i = a.base + r;
  const int64_t e0 = a.rowptr[i], e1 = a.rowptr[i + 1];
  const int64_t k = p - a.pair_off[r];
  if (k < e1 - e0) {
    attract = true;
    const int64_t dst = a.col[e0 + k];
    const int64_t dst_end = a.quirks ? a.n - 1 : a.n;  // F7: edges into n-1 skipped
    return (dst >= 0 && dst < dst_end) ? dst : -1;
  }
  attract = false;
  const int64_t c = a.negs[k - (e1 - e0)];
  return (c >= 0 && c < a.n) ? c : -1;  // F9: a draw equal to n counts nothing
}

__global__ void pass1_kernel(PassArgs a, int64_t total) {
  const int64_t p = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
  if (p >= total) return;
  // row of pair p: binary search in pair_off
  int lo = 0, hi = a.rows;
  while (hi - lo > 1) {
    const int mid = (lo + hi) / 2;
    if (a.pair_off[mid] <= p) lo = mid; else hi = mid;
  }
  bool attract = false;
  const int64_t o = pair_other(a, lo, p, attract);
  if (o < 0) {
    a.d1[p] = 0.0;
    a.ploss[p] = 0.0;
    return;
  }
  const double *xi = a.x + (a.base + lo) * a.dim, *xo = a.x + o * a.dim;
  double r = 0.0;
  for (int d = 0; d < a.dim; ++d) {
    const double t = __dsub_rn(xi[d], xo[d]);
    r = __dadd_rn(r, __dmul_rn(t, t));
  }
  if (attract) {
    a.d1[p] = -2.0 / __dadd_rn(1.0, r);
    a.ploss[p] = log1p(r);
  } else {
    a.d1[p] = 2.0 / __dmul_rn(__dadd_rn(r, 0.000001), __dadd_rn(1.0, r));
    a.ploss[p] = log(__dadd_rn(1.0, r) / __dadd_rn(r, 0.000001));
  }
}

// One warp per row: lanes over the dims, pairs in order.
__global__ void pass2_kernel(PassArgs a) {
  const int r = blockIdx.x * (blockDim.x / 32) + threadIdx.x / 32;
  const int lane = threadIdx.x & 31;
  if (r >= a.rows) return;
  const int64_t i = a.base + r;
  const double *xi = a.x + i * a.dim;
  double *pv = a.prev + int64_t(r) * a.dim;
  for (int d = lane; d < a.dim; d += 32) pv[d] = 0.0;
  const int64_t p0 = a.pair_off[r], p1 = a.pair_off[r + 1];
  const int64_t na = a.rowptr[i + 1] - a.rowptr[i];
  double la = 0.0, lrp = 0.0;
  for (int64_t p = p0; p < p1; ++p) {
    bool attract = false;
    const int64_t o = pair_other(a, r, p, attract);
    if (o < 0) continue;
    if (!attract && p - p0 - na >= a.ns) break;
    const double c = a.d1[p];
    const double *xo = a.x + o * a.dim;
    for (int d = lane; d < a.dim; d += 32) {
      const double l = clip5(__dmul_rn(__dsub_rn(xi[d], xo[d]), c));
      pv[d] = __dadd_rn(pv[d], __dmul_rn(a.lr, l));
    }
    if (lane == 0) {
      if (attract) la = __dadd_rn(la, a.ploss[p]);
      else lrp = __dadd_rn(lrp, a.ploss[p]);
    }
  }
  if (lane == 0) a.row_loss[r] = __dadd_rn(la, lrp);
}

__global__ void pass3_kernel(double *x, const double *prev, int64_t base, int64_t count) {
  const int64_t t = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
  if (t < count) x[base + t] = __dadd_rn(x[base + t], prev[t]);
}

#define OCHK(call)                       \
  do {                                   \
    if ((call) != cudaSuccess) {         \
      rc = -2;                           \
      goto done;                         \
    }                                    \
  } while (0)

}  // namespace

extern "C" {

/* `epochs` epochs of the one-rank step on the GPU in FP64, x (n x dim, host FP64)
 * updated in place, one learning rate per epoch, loss_per_epoch (nullable).
 * Returns 0, -1 for bad arguments, -2 for a CUDA error. */
int oracle_gpu_run(int64_t n, const int64_t *rowptr, const int64_t *col, int dim, double *x, int epochs, int batch,
                   int ns, const double *lr_per_epoch, int quirks, double *loss_per_epoch, int device) {
  if (n <= 0 || dim <= 0 || batch <= 0 || ns < 0 || epochs < 0) return -1;
  int rc = 0;
  const int64_t nnz = rowptr[n];
  const int batches = int(n / batch) + (n % batch ? 1 : 0);
  const int last = (n % batch) ? int(n - int64_t(batch) * (batches - 1)) : batch;
  double *dx = nullptr, *d1 = nullptr, *ploss = nullptr, *prev = nullptr, *rloss = nullptr;
  int64_t *drp = nullptr, *dcol = nullptr, *dnegs = nullptr, *doff = nullptr;
  int64_t max_pairs = 0;
  std::vector<int64_t> off(size_t(batch) + 1), negs(size_t(std::max(ns, 1)));
  std::vector<double> hloss(static_cast<size_t>(batch));
  for (int j = 0; j < batches; ++j) {
    const int64_t b0 = int64_t(j) * batch, rows = std::min<int64_t>(batch, n - b0);
    max_pairs = std::max(max_pairs, rowptr[b0 + rows] - rowptr[b0] + rows * ns);
  }
  OCHK(cudaSetDevice(device));
  OCHK(cudaMalloc(&dx, size_t(n) * dim * sizeof(double)));
  OCHK(cudaMalloc(&drp, size_t(n + 1) * sizeof(int64_t)));
  OCHK(cudaMalloc(&dcol, size_t(std::max<int64_t>(nnz, 1)) * sizeof(int64_t)));
  OCHK(cudaMalloc(&dnegs, negs.size() * sizeof(int64_t)));
  OCHK(cudaMalloc(&doff, off.size() * sizeof(int64_t)));
  OCHK(cudaMalloc(&d1, size_t(std::max<int64_t>(max_pairs, 1)) * sizeof(double)));
  OCHK(cudaMalloc(&ploss, size_t(std::max<int64_t>(max_pairs, 1)) * sizeof(double)));
  OCHK(cudaMalloc(&prev, size_t(batch) * dim * sizeof(double)));
  OCHK(cudaMalloc(&rloss, size_t(batch) * sizeof(double)));
  OCHK(cudaMemcpy(dx, x, size_t(n) * dim * sizeof(double), cudaMemcpyHostToDevice));
  OCHK(cudaMemcpy(drp, rowptr, size_t(n + 1) * sizeof(int64_t), cudaMemcpyHostToDevice));
  if (nnz > 0) OCHK(cudaMemcpy(dcol, col, size_t(nnz) * sizeof(int64_t), cudaMemcpyHostToDevice));
  for (int e = 0; e < epochs; ++e) {
    double epoch_loss = 0.0;
    for (int j = 0; j < batches; ++j) {
      std::minstd_rand gen(e + j);
      std::uniform_int_distribution<int> dist(0, int(n));
      for (int k = 0; k < ns; ++k) negs[k] = int64_t(dist(gen));
      const int64_t b0 = int64_t(j) * batch;
      const int rows = int(std::min<int64_t>(batch, n - b0));
      const int rep_rows = (j == batches - 1 || (quirks && e > 0)) ? last : batch;  // F8
      off[0] = 0;
      for (int r = 0; r < rows; ++r)
        off[r + 1] = off[r] + (rowptr[b0 + r + 1] - rowptr[b0 + r]) + (r < rep_rows ? ns : 0);
      OCHK(cudaMemcpy(dnegs, negs.data(), negs.size() * sizeof(int64_t), cudaMemcpyHostToDevice));
      OCHK(cudaMemcpy(doff, off.data(), size_t(rows + 1) * sizeof(int64_t), cudaMemcpyHostToDevice));
      PassArgs a{dx, drp, dcol, dnegs, n, b0, rows, rep_rows, ns, dim, quirks, doff, d1, ploss, prev, rloss,
                 lr_per_epoch[e]};
      const int64_t total = off[rows];
      if (total > 0) pass1_kernel<<<unsigned((total + 255) / 256), 256>>>(a, total);
      pass2_kernel<<<unsigned((rows + 7) / 8), 256>>>(a);
      pass3_kernel<<<unsigned((int64_t(rows) * dim + 255) / 256), 256>>>(dx, prev, b0 * dim, int64_t(rows) * dim);
      OCHK(cudaGetLastError());
      if (loss_per_epoch) {
        OCHK(cudaMemcpy(hloss.data(), rloss, size_t(rows) * sizeof(double), cudaMemcpyDeviceToHost));
        for (int r = 0; r < rows; ++r) epoch_loss += hloss[r];
      }
    }
    if (loss_per_epoch) loss_per_epoch[e] = epoch_loss;
  }
  OCHK(cudaMemcpy(x, dx, size_t(n) * dim * sizeof(double), cudaMemcpyDeviceToHost));
done:
  for (void *p : {static_cast<void *>(dx), static_cast<void *>(d1), static_cast<void *>(ploss),
                  static_cast<void *>(prev), static_cast<void *>(rloss), static_cast<void *>(drp),
                  static_cast<void *>(dcol), static_cast<void *>(dnegs), static_cast<void *>(doff)})
    if (p) cudaFree(p);
  return rc;
}

}  // extern "C"
