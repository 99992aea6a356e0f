// Internal types shared by the host runtime and the kernels.
#pragma once
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/distembed_gb300.h"

#include <algorithm>
#include <string>
#include <thread>
#include <vector>

namespace de {

// f(i) for i in [0, count), on host threads when count * cost_per_item is large
// (contiguous index ranges, one per thread; f must write only what index i owns,
// so the result does not depend on the split).
template <class F>
void parallel_indices(int64_t count, int64_t cost_per_item, F &&f) {
  int threads = 1;
  if (count * cost_per_item >= (int64_t(1) << 18))
    threads = int(std::min<int64_t>({int64_t(std::max(1u, std::thread::hardware_concurrency())), 32, count}));
  if (threads <= 1) {
    for (int64_t i = 0; i < count; ++i) f(i);
    return;
  }
  std::vector<std::thread> pool;
  const int64_t per = (count + threads - 1) / threads;
  for (int t = 0; t < threads; ++t) {
    const int64_t lo = t * per, hi = std::min(count, lo + per);
    if (lo >= hi) break;
    pool.emplace_back([&f, lo, hi] {
      for (int64_t i = lo; i < hi; ++i) f(i);
    });
  }
  for (auto &th : pool) th.join();
}

// One unit of attractive work: row `row` (index within its minibatch) over CSR
// entries [e_begin, e_end).  Rows whose degree exceeds the edge cap are split
// into P = `nparts` items, combined in two fixed-order levels so the result does
// not depend on timing:
//   part p writes its partial to slot first_slot + p; parts form groups of
//   kCombineGroup; the last part of group g to arrive (counters[counter + g])
//   sums the group's slots in order.  With NG = ceil(P / kCombineGroup) > 1
//   groups, that sum goes to slot first_slot + P + g and the last group to
//   arrive (counters[counter + NG]) sums the NG group slots in order.
// A split row uses P + (NG > 1 ? NG : 0) slots and NG + (NG > 1) counters.
constexpr int kCombineGroup = 16;
struct WorkItem {
  int32_t row;
  int32_t e_begin;
  int32_t e_end;
  int32_t nparts;      // 1 = whole row
  int32_t first_slot;  // split rows: first slot of the row
  int32_t part;        // split rows: index of this part
  int32_t counter;     // split rows: first counter of the row
  int32_t batch;       // minibatch of the item (the one-launch SpMM)
};
static_assert(sizeof(WorkItem) == 32, "WorkItem layout");

// Work list of one minibatch size over the whole graph.
struct Schedule {
  int batch = 0;          // minibatch size B
  int batches = 0;        // ceil(n / B)
  int last_batch_size = 0;
  int edge_cap = 0;
  std::vector<int64_t> item_off;   // [batches + 1] into the item array
  std::vector<int32_t> n_parts;    // partial slots used by batch j
  std::vector<int32_t> n_split;    // arrival counters used by batch j
  int max_parts = 0, max_split = 0;
  std::vector<int64_t> cta_off;    // [batches + 1] CTA counts (prefix) of the minibatch launches
  WorkItem *d_items = nullptr;
  int64_t n_items = 0;
};

// Kernel arguments of one minibatch of the FP32 plain path.
struct PlainBatchArgs {
  float *X;                 // [n, dim] embedding; rows of batch prev are written here
  const float *S_prev2;     // staged new rows of minibatch j-2 (read)
  const float *S_prev;      // staged new rows of minibatch j-1 (read)
  float *S_cur;             // staged new rows of this minibatch (write)
  const int32_t *rowptr;    // [n + 1]
  const int32_t *col;       // [nnz]
  const WorkItem *items;    // this batch's work items
  int32_t n_items;
  int32_t base, rows;       // first row and row count of this batch
  int32_t prev_base, prev_rows;    // minibatch j-1 (prev_rows = 0: none)
  int32_t prev2_base, prev2_rows;  // minibatch j-2 (prev2_rows = 0: none)
  int32_t batch_id, batches, last_batch_size;
  int32_t n;
  int32_t quirks, compute_loss;
  int32_t skip_last;        // F7: edges into vertex n-1 are dropped
  float bound;
  const int32_t *negs;      // [epochs, batches, ns]
  int32_t ns;
  const float *lr;          // [epochs]
  float *P;                 // partial slots [max_parts, dim]
  int32_t *counters;        // [max counters of a minibatch], zero between uses
  double *loss_partial;     // one per work item of the epoch
  int64_t loss_off;         // first item of this minibatch in the epoch
  const int32_t *epoch;     // device [2]: epoch index within this call, first epoch of the call
  int32_t stage_negs;       // 1: the minibatch's final negative rows are copied into every CTA's
                            // shared memory (cp.async.bulk) before the repulsive pass; ns <= kStageNegMax
  int32_t *err;             // set when a bounded device wait gives up
};

constexpr int kStageNegMax = 8;  // negatives per minibatch the shared-memory staging takes

struct FlushArgs {
  float *X;
  const float *S_last;
  int32_t last_base, last_rows;
  const double *loss_partial;
  int64_t n_partials;
  double *block_sums;       // [kFlushBlocks]
  int32_t *done;            // CTA arrival counter, zero between uses
  double *loss;             // [epochs] per-epoch loss
  int32_t *epoch;           // device [2]; [0] incremented once per epoch
  int32_t compute_loss;
};

constexpr int kFlushBlocks = 152;

// The SpMM step (spmm_kernel): every work item of every minibatch in one launch,
// y rows from the unchanged input x; a minibatch's split rows use partial slots
// from slot_off[j] and counters from counter_off[j] (WorkItem::batch = j).
struct SpmmArgs {
  const float *X;
  float *Y;
  const int32_t *col;
  const WorkItem *items;
  int64_t n_items;
  int32_t batch, skip;
  const int32_t *slot_off, *counter_off;
  float lr;
  float *P;
  int32_t *counters;
  float bound;  // sparse embedding: clip bound of the attractive force
};

// Kernel arguments of one minibatch of the BF16 precision form.
struct BF16BatchArgs {
  float *xm;                // [n, dim] FP32 master copy
  __nv_bfloat16 *xb;        // [n, dim] BF16 copy, read by every force
  const int32_t *rowptr, *col;
  const WorkItem *items;
  int32_t n_items;
  int32_t base, rows, last_batch_size;  // minibatch rows; see rep_rows in the kernels
  int32_t batch_id, batches;
  int32_t n, quirks, compute_loss;
  float bound;
  const int32_t *negs;      // [epochs, batches, ns]
  int32_t ns, kpad;         // kpad = ns rounded up to a multiple of 64 (>= 64)
  const float *lr;          // [epochs]
  const int32_t *epoch;     // device [2]
  float *P;                 // partial slots of split rows
  int32_t *counters;
  float *abuf;              // [B, dim] attractive update of the minibatch (lr applied)
  float *rbuf;              // [B, dim] repulsive (GEMM) update of the minibatch (lr applied)
  __nv_bfloat16 *nb;        // [kpad, dim] gathered negatives
  float *nn;                // [kpad] squared norms of the gathered negatives
  int32_t *nid;             // [kpad] vertex id of each negative, -1 = none
  uint32_t *near_bits;      // [B, kpad / 32] bit k: pair (row, negative k) takes the exact
                            // path; zero between minibatches
  double *loss_item;        // attractive loss per work item of the epoch
  int64_t loss_off;
  double *loss_row;         // [n] repulsive loss per vertex of the epoch
  int32_t *err;             // set when a bounded device wait gives up
};

struct BF16FlushArgs {
  const double *loss_item;
  const double *loss_row;
  int64_t n_items, n_rows;
  double *block_sums;
  int32_t *done;
  double *loss;
  int32_t *epoch;
  int32_t compute_loss;
};

// BF16 launchers (de_bf16.cu).
int bf16_repulse_smem_bytes(int dim);
cudaError_t bf16_prepare(int dim);
// One minibatch: gather of the negatives, then the attractive pass (on s) and the
// repulsion GEMMs (on s2, forked and joined with the two events), then the
// update with the exact close pairs.  ev (nullable): four events recorded before
// the gather, attractive, GEMM and update launches, all on s one after another
// (so is everything when s2 is null).
cudaError_t launch_bf16_batch(int dim, const BF16BatchArgs &a, const CUtensorMap &mx, const CUtensorMap &mn,
                              cudaStream_t s, cudaEvent_t *ev, cudaStream_t s2,
                              cudaEvent_t fork, cudaEvent_t join);
cudaError_t launch_bf16_flush(const BF16FlushArgs &a, cudaStream_t s);
cudaError_t launch_f32_to_bf16(const float *src, __nv_bfloat16 *dst, int64_t count, cudaStream_t s);

// Where a handle's buffers come from.  With dalloc set, device buffers come from
// dalloc/dfree (a caller-owned arena; no implicit device synchronisation) and
// host staging buffers from malloc; otherwise cudaMalloc and pinned cudaHostAlloc.
struct MemHooks {
  void *(*dalloc)(void *ctx, size_t bytes) = nullptr;
  void (*dfree)(void *ctx, void *p) = nullptr;
  void *ctx = nullptr;
};

// de_create with memory hooks (nullable) (de_runtime.cpp).
int create_handle(int64_t n, const int64_t *rowptr, const int64_t *col, int64_t nnz, int32_t dim,
                  const de_options *opts, const MemHooks *hooks, de_handle **out);
// The FP64 per-epoch loss of the last de_run_from of `epochs` epochs; waits for
// the handle's stream.
int copy_loss(de_handle *h, double *out, int32_t epochs);

// Launchers (de_plain.cu).  pdl: launch with a programmatic dependency on the
// previous kernel in the stream.
cudaError_t launch_plain_batch(int dim, const PlainBatchArgs &a, int grid, bool pdl, cudaStream_t s);
cudaError_t launch_flush(int dim, const FlushArgs &a, bool pdl, cudaStream_t s);
cudaError_t launch_spmm(int dim, const SpmmArgs &a, cudaStream_t s);

// Sparse embedding (de_sparse.cu).  Rows are FP64 vectors with INT_MIN marking
// an absent entry; their FP32 mirror holds 0 there.
cudaError_t launch_sparse_attract(int dim, const SpmmArgs &a, cudaStream_t s);
cudaError_t launch_sparse_collect(const float *y, double *coll, int64_t n, int32_t batch, int32_t dim,
                                  cudaStream_t s);
cudaError_t launch_sparse_mirror(const double *x64, float *x32, int64_t count, cudaStream_t s);
// src / dst: device or mapped pinned host memory, 16-byte aligned; count even
cudaError_t launch_sparse_load(const double *src, double *x64, float *x32, int64_t count, cudaStream_t s);
cudaError_t launch_sparse_store(const double *src, double *dst, int64_t count, cudaStream_t s);
cudaError_t launch_sparse_count(const double *x64, int64_t count, unsigned long long *present, cudaStream_t s);
cudaError_t launch_sparse_prune_f64(int dim, double *x64, float *x32, int64_t n, int32_t keep,
                                    const unsigned long long *present, cudaStream_t s);
cudaError_t launch_sparse_prune_f32(int dim, float *x32, int64_t n, int32_t keep, cudaStream_t s);
cudaError_t launch_sparse_finalize(double *x64, int64_t count, cudaStream_t s);
cudaError_t launch_f64_to_f32(const double *src, float *dst, int64_t count, cudaStream_t s);
cudaError_t launch_f32_to_f64(const float *src, double *dst, int64_t count, cudaStream_t s);
constexpr int kPlainWarps = 4;      // warps per CTA of the plain batch kernel
constexpr int kPlainMinBlocks = 8;  // resident CTAs per SM the register budget targets (one wave of
                                    // work items at minibatch 4096: 152 x 8 x 4 warps)
constexpr int kMaxEdgeCap = 32;     // CSR entries per work item: one per lane

}  // namespace de
