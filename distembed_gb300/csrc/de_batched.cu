// Batched form: many independent graphs in one persistent launch (sm_103a).
//
// Each graph is owned by one CTA (a "team") for all its epochs, so the
// reference's minibatch order (cpp/algo/algo.hpp:164-192: batch b+1 reads the
// update of batch b, rows of one batch read pre-batch values) needs nothing but
// __syncthreads: no grid-wide barrier and no waiting on other CTAs.  Teams take
// graphs largest first from an atomic counter.  Per minibatch:
//   1. work items (a row, or a <= cap-edge piece of a high-degree row) are spread
//      over the team's warps; a warp runs VPW items at once, each on 32/VPW lanes;
//      whole rows write their update to the team's staging rows, pieces write
//      partials (part 0 of a row also carries its repulsive pass);
//   2. split rows add their pieces in piece order into the staging rows;
//   3. the rows are updated (FP32 master, and the BF16 copy in the BF16 form).
// The arithmetic of a graph does not depend on which team runs it or when, so a
// graph's result is bitwise the same alone or in any mix (for one team shape).
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <memory>
#include <random>
#include <string>
#include <vector>

#include "de_batched.cuh"

namespace de {
void set_thread_error(const std::string &msg);  // de_runtime.cpp
}

using namespace de::batched;

namespace {

// Largest dynamic shared memory a staged team may use (the static part is small).
constexpr size_t kStagedSmemMax = 227 * 1024 - 1024;

// Dynamic shared memory of a staged team with (ids = 1) or without its column-id
// buffers.
template <int D, bool kBF16>
size_t staged_smem(const de_batch_shape &s, int ns, int ids) {
  return StagedLayout<D, kBF16>::bytes(s.team_warps, s.stages, s.edge_cap, ns, ids);
}

template <int D, bool kBF16>
size_t rows_smem(const de_batch_shape &s, int ns) {
  return RowsLayout<D, kBF16>::bytes(s.team_warps, s.stages, s.edge_cap, ns);
}

// The kernel, its block size and dynamic shared memory for a team shape; fn is
// null when the shape does not exist.
struct KernelPick {
  BatchedKernel fn = nullptr;
  int block = 0;
  size_t smem = 0;
  int ctas = 1;  // CTAs per cluster the kernel is launched with
  int stage_ids = 0;  // staged kernel: the column-id buffers fit in shared memory
};

KernelPick pick_kernel(int dim, bool bf16, const de_batch_shape &s, int ns = 0) {
  KernelPick k;
  if ((s.team_ctas > 1 && s.team_ctas != 2 && s.team_ctas != 4) ||
      (s.team_ctas > 1 && s.kernel != DE_BATCH_STAGED))
    return k;
  k.ctas = s.team_ctas > 1 ? s.team_ctas : 1;
  if (s.kernel == DE_BATCH_REGISTER) {
    if (s.edge_cap < 1 || s.edge_cap > 4096) return k;
    k.fn = pick_register(dim, bf16, s.vertices_per_warp, s.team_warps);
    k.block = 32 * s.team_warps;
    return k;
  }
  if ((s.kernel != DE_BATCH_STAGED && s.kernel != DE_BATCH_ROWS) || s.team_warps < 2 || s.team_warps > 16 ||
      s.edge_cap < 1 || s.edge_cap > 32)
    return k;
  if (s.kernel == DE_BATCH_ROWS) {
    switch (dim) {
      case 32:
        k.fn = pick_rows(32, bf16, s.pairs, s.stages);
        k.smem = bf16 ? rows_smem<32, true>(s, ns) : rows_smem<32, false>(s, ns);
        break;
      case 64:
        k.fn = pick_rows(64, bf16, s.pairs, s.stages);
        k.smem = bf16 ? rows_smem<64, true>(s, ns) : rows_smem<64, false>(s, ns);
        break;
      case 128:
        k.fn = pick_rows(128, bf16, s.pairs, s.stages);
        k.smem = bf16 ? rows_smem<128, true>(s, ns) : rows_smem<128, false>(s, ns);
        break;
    }
    if (k.smem > kStagedSmemMax) k.fn = nullptr;
    k.block = 32 * s.team_warps;
    return k;
  }
  auto smem_of = [&](int ids) -> size_t {
    switch (dim) {
      case 32: return bf16 ? staged_smem<32, true>(s, ns, ids) : staged_smem<32, false>(s, ns, ids);
      case 64: return bf16 ? staged_smem<64, true>(s, ns, ids) : staged_smem<64, false>(s, ns, ids);
      case 128: return bf16 ? staged_smem<128, true>(s, ns, ids) : staged_smem<128, false>(s, ns, ids);
    }
    return 0;
  };
  k.fn = pick_staged(dim, bf16, s.pairs, s.stages, k.ctas);
  // the column-id buffers where they fit; without them the kernel reads the ids
  // from global memory one chunk ahead
  k.stage_ids = smem_of(1) <= kStagedSmemMax ? 1 : 0;
  k.smem = smem_of(k.stage_ids);
  if (k.smem > kStagedSmemMax) k.fn = nullptr;
  k.block = 32 * s.team_warps;
  return k;
}

}  // namespace

// ---------------------------------------------------------------- host side

struct de_batch {
  int n_graphs = 0, dim = 0;
  de_options opt{};
  int device = 0;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  std::string err;
  std::vector<int64_t> n, nnz, voff, eoff;
  std::vector<std::vector<int64_t>> rowptr;  // host copies for schedules
  std::vector<int64_t> edges_into_last;
  int64_t total_n = 0, total_nnz = 0;
  int32_t *d_col = nullptr;
  float *d_xm = nullptr;
  __nv_bfloat16 *d_xb = nullptr;
  // per (batch size, edge cap) schedule
  int sched_batch = 0, sched_cap = 0;
  std::vector<GraphInfo> ginfo;
  std::vector<int32_t> order;
  GraphInfo *d_graphs = nullptr;
  int32_t *d_order = nullptr, *d_next = nullptr;
  WorkItem *d_items = nullptr;
  int64_t *d_bitem = nullptr;
  int32_t *d_bsplit = nullptr;
  SplitRow *d_splits = nullptr;
  int max_slots = 0;
  // per run
  int32_t *d_negs = nullptr;
  size_t negs_cap = 0;
  float *d_lr = nullptr;
  size_t lr_cap = 0;
  double *d_loss = nullptr;
  size_t loss_cap = 0;
  float *d_stage = nullptr, *d_slots = nullptr;
  size_t stage_cap = 0, slots_cap = 0;
  de_batch_shape shape{DE_BATCH_REGISTER, 4, 8, 32, 0, 0, 1};
  int teams = 0, block = 0, ctas = 1, n_big = 0;
  size_t smem = 0;
  float *d_item_loss = nullptr;
  size_t item_loss_cap = 0;
  int32_t *d_cluster_slot = nullptr;
  size_t cluster_slot_cap = 0;
  int max_batch_items = 1;
  int32_t *d_err = nullptr;
  BatchedKernel kernel = nullptr;
  BatchedArgs args{};
  cudaGraphExec_t exec = nullptr;  // the prepared run
  int prepared_epochs = 0;
  float near_r = 0.02f;            // BF16 form: squared distance below which a pair is recomputed in FP32
  int loss_mode = DE_LOSS_EVERY_EPOCH;
  long long *d_trace = nullptr;    // [n_graphs x 3] of the last launch
};

namespace {

int bfail(de_batch *b, int code, const std::string &m) {
  if (b) b->err = m; else de::set_thread_error(m);
  return code;
}

#define BCUDA(b, call)                                                                              \
  do {                                                                                              \
    cudaError_t e_ = (call);                                                                        \
    if (e_ != cudaSuccess)                                                                          \
      return bfail(b, e_ == cudaErrorMemoryAllocation ? DE_ERR_OOM : DE_ERR_CUDA,                   \
                   std::string(#call) + ": " + cudaGetErrorString(e_));                             \
  } while (0)

template <typename T>
int bgrow(de_batch *b, T **p, size_t *cap, size_t need) {
  if (need <= *cap && *p) return DE_OK;
  if (*p) cudaFree(*p);
  *p = nullptr;
  *cap = 0;
  BCUDA(b, cudaMalloc(reinterpret_cast<void **>(p), std::max<size_t>(need, 1) * sizeof(T)));
  *cap = std::max<size_t>(need, 1);
  return DE_OK;
}

// Work items and split rows of every minibatch of every graph (edge cap `cap`).
int build_batched_schedule(de_batch *b, int B, int cap) {
  std::vector<WorkItem> items;
  std::vector<int64_t> bitem{0};
  std::vector<int32_t> bsplit{0};
  std::vector<SplitRow> splits;
  b->ginfo.assign(b->n_graphs, GraphInfo{});
  int max_slots = 1;
  int64_t max_items = 1;
  int64_t batch_off = 0;
  for (int g = 0; g < b->n_graphs; ++g) {
    GraphInfo &G = b->ginfo[g];
    const int64_t n = b->n[g];
    G.voff = b->voff[g];
    G.eoff = b->eoff[g];
    G.n = int32_t(n);
    G.batches = int32_t(n / B + (n % B ? 1 : 0));
    G.last_batch_size = (n % B) ? int32_t(n - int64_t(B) * (G.batches - 1)) : B;
    G.batch_off = batch_off;
    const std::vector<int64_t> &rp = b->rowptr[g];
    for (int j = 0; j < G.batches; ++j) {
      const int64_t base = int64_t(j) * B;
      const int rows = int(std::min<int64_t>(B, n - base));
      const size_t first = items.size();
      int slot = 0;
      for (int r = 0; r < rows; ++r) {
        const int64_t e0 = rp[base + r], e1 = rp[base + r + 1];
        if (e1 - e0 <= cap) {
          items.push_back(WorkItem{r, int32_t(e0), int32_t(e1), 1, 0, 0, 0, 0});
        } else {
          const int np = int((e1 - e0 + cap - 1) / cap);
          for (int p = 0; p < np; ++p) {
            const int64_t x = e0 + int64_t(p) * cap, y = std::min<int64_t>(e1, x + cap);
            items.push_back(WorkItem{r, int32_t(x), int32_t(y), np, slot, p, 0, 0});
          }
          splits.push_back(SplitRow{r, slot, np, 0});
          slot += np;
        }
      }
      std::stable_sort(items.begin() + first, items.end(), [](const WorkItem &x, const WorkItem &y) {
        return (x.e_end - x.e_begin) > (y.e_end - y.e_begin);
      });
      max_slots = std::max(max_slots, slot);
      bitem.push_back(int64_t(items.size()));
      max_items = std::max<int64_t>(max_items, bitem.back() - bitem[bitem.size() - 2]);
      bsplit.push_back(int32_t(splits.size()));
    }
    batch_off += G.batches;
  }
  b->sched_batch = B;
  b->sched_cap = cap;
  b->max_slots = max_slots;
  b->max_batch_items = int(max_items);
  // graphs largest first (LPT): by total work n + nnz
  b->order.resize(b->n_graphs);
  for (int g = 0; g < b->n_graphs; ++g) b->order[g] = g;
  std::stable_sort(b->order.begin(), b->order.end(), [&](int x, int y) {
    return b->n[x] + b->nnz[x] > b->n[y] + b->nnz[y];
  });
  for (void *p : {static_cast<void *>(b->d_graphs), static_cast<void *>(b->d_order), static_cast<void *>(b->d_items),
                  static_cast<void *>(b->d_bitem), static_cast<void *>(b->d_bsplit), static_cast<void *>(b->d_splits)})
    if (p) cudaFree(p);
  b->d_graphs = nullptr; b->d_order = nullptr; b->d_items = nullptr; b->d_bitem = nullptr; b->d_bsplit = nullptr;
  b->d_splits = nullptr;
  BCUDA(b, cudaMalloc(&b->d_graphs, b->ginfo.size() * sizeof(GraphInfo)));
  BCUDA(b, cudaMalloc(&b->d_order, b->order.size() * sizeof(int32_t)));
  BCUDA(b, cudaMalloc(&b->d_items, std::max<size_t>(items.size(), 1) * sizeof(WorkItem)));
  BCUDA(b, cudaMalloc(&b->d_bitem, bitem.size() * sizeof(int64_t)));
  BCUDA(b, cudaMalloc(&b->d_bsplit, bsplit.size() * sizeof(int32_t)));
  BCUDA(b, cudaMalloc(&b->d_splits, std::max<size_t>(splits.size(), 1) * sizeof(SplitRow)));
  BCUDA(b, cudaMemcpyAsync(b->d_graphs, b->ginfo.data(), b->ginfo.size() * sizeof(GraphInfo), cudaMemcpyHostToDevice, b->stream));
  BCUDA(b, cudaMemcpyAsync(b->d_order, b->order.data(), b->order.size() * sizeof(int32_t), cudaMemcpyHostToDevice, b->stream));
  if (!items.empty())
    BCUDA(b, cudaMemcpyAsync(b->d_items, items.data(), items.size() * sizeof(WorkItem), cudaMemcpyHostToDevice, b->stream));
  BCUDA(b, cudaMemcpyAsync(b->d_bitem, bitem.data(), bitem.size() * sizeof(int64_t), cudaMemcpyHostToDevice, b->stream));
  BCUDA(b, cudaMemcpyAsync(b->d_bsplit, bsplit.data(), bsplit.size() * sizeof(int32_t), cudaMemcpyHostToDevice, b->stream));
  if (!splits.empty())
    BCUDA(b, cudaMemcpyAsync(b->d_splits, splits.data(), splits.size() * sizeof(SplitRow), cudaMemcpyHostToDevice, b->stream));
  BCUDA(b, cudaStreamSynchronize(b->stream));  // the host vectors go away on return
  return DE_OK;
}

int teams_for(de_batch *b, const KernelPick &k) {
  int per_sm = 0, sms = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k.fn, k.block, k.smem) != cudaSuccess || per_sm < 1)
    per_sm = 1;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, b->device) != cudaSuccess || sms < 1) sms = 1;
  if (k.ctas == 1) return std::min(per_sm * sms, b->n_graphs);
  // clusters of k.ctas CTAs: as many as can be resident at once (a cluster sits in one GPC)
  cudaLaunchConfig_t cfg{};
  cfg.gridDim = dim3(k.ctas * per_sm * sms);
  cfg.blockDim = dim3(k.block);
  cfg.dynamicSmemBytes = k.smem;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = k.ctas;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  int clusters = 0;
  if (cudaOccupancyMaxActiveClusters(&clusters, k.fn, &cfg) != cudaSuccess || clusters < 1) {
    cudaGetLastError();
    clusters = std::max(1, per_sm * sms / k.ctas);
  }
  return k.ctas * std::min(clusters, (b->n_graphs + k.ctas - 1) / k.ctas);
}

// Everything of a run except the launch: schedule, negatives, rates, team staging
// areas and the kernel arguments (kept in b->args, b->kernel, b->teams).  Nothing
// here may run inside a stream capture: it allocates and copies synchronously.
int prepare_batched(de_batch *b, int epochs, int B, int ns, const double *lr, const de_batch_shape &shape) {
  BCUDA(b, cudaSetDevice(b->device));
  if (shape.kernel != DE_BATCH_REGISTER && ns > kStagedMaxNs)
    return bfail(b, DE_ERR_UNSUPPORTED, "the staged kernel takes at most 32 negatives per minibatch");
  const KernelPick k = pick_kernel(b->dim, b->opt.precision == DE_PRECISION_BF16, shape, ns);
  if (!k.fn) return bfail(b, DE_ERR_UNSUPPORTED, "no kernel for this dim and team shape (or its shared memory is too large)");
  if (k.smem) BCUDA(b, cudaFuncSetAttribute(k.fn, cudaFuncAttributeMaxDynamicSharedMemorySize, int(k.smem)));
  const int cap = shape.edge_cap;
  if (b->sched_batch != B || b->sched_cap != cap)
    if (int rc = build_batched_schedule(b, B, cap)) return rc;
  // negatives: the reference's sampler per graph and minibatch (seed = epoch + batch)
  size_t total = 0;
  for (int g = 0; g < b->n_graphs; ++g) {
    b->ginfo[g].neg_off = int64_t(total);
    total += size_t(epochs) * b->ginfo[g].batches * ns;
  }
  std::vector<int32_t> negs(std::max<size_t>(total, 1));
  // minibatch q of the run (graphs in order, then epochs, then minibatches) owns
  // negs[q * ns, (q + 1) * ns); its draws depend only on its graph and seed, so
  // they are made on host threads
  std::vector<int64_t> mb_end(b->n_graphs);  // minibatches up to and including graph g
  int64_t mbs = 0;
  for (int g = 0; g < b->n_graphs; ++g) mb_end[g] = (mbs += int64_t(epochs) * b->ginfo[g].batches);
  if (ns > 0)
    de::parallel_indices(mbs, ns, [&](int64_t q) {
      const int g = int(std::upper_bound(mb_end.begin(), mb_end.end(), q) - mb_end.begin());
      const GraphInfo &G = b->ginfo[g];
      const int64_t local = q - (mb_end[g] - int64_t(epochs) * G.batches);
      const int e = int(local / G.batches), j = int(local % G.batches);
      std::minstd_rand gen(e + j);  // the sampler of de_negatives (seed = epoch + batch)
      std::uniform_int_distribution<int> dist(0, int(G.n));
      int32_t *o = negs.data() + size_t(q) * ns;
      for (int k = 0; k < ns; ++k) o[k] = dist(gen);
    });
  std::vector<float> lrf(epochs);
  for (int e = 0; e < epochs; ++e) lrf[e] = float(lr[e]);
  if (int rc = bgrow(b, &b->d_negs, &b->negs_cap, negs.size())) return rc;
  if (int rc = bgrow(b, &b->d_lr, &b->lr_cap, size_t(epochs))) return rc;
  if (int rc = bgrow(b, &b->d_loss, &b->loss_cap, size_t(epochs) * b->n_graphs)) return rc;
  BCUDA(b, cudaMemcpyAsync(b->d_negs, negs.data(), negs.size() * sizeof(int32_t), cudaMemcpyHostToDevice, b->stream));
  BCUDA(b, cudaMemcpyAsync(b->d_lr, lrf.data(), epochs * sizeof(float), cudaMemcpyHostToDevice, b->stream));
  BCUDA(b, cudaMemcpyAsync(b->d_graphs, b->ginfo.data(), b->ginfo.size() * sizeof(GraphInfo), cudaMemcpyHostToDevice,
                           b->stream));
  BCUDA(b, cudaStreamSynchronize(b->stream));
  const int teams = teams_for(b, k);
  if (int rc = bgrow(b, &b->d_stage, &b->stage_cap, size_t(teams) * B * b->dim)) return rc;
  if (int rc = bgrow(b, &b->d_slots, &b->slots_cap, size_t(teams) * b->max_slots * b->dim)) return rc;
  if (int rc = bgrow(b, &b->d_item_loss, &b->item_loss_cap, size_t(teams) * b->max_batch_items)) return rc;
  if (int rc = bgrow(b, &b->d_cluster_slot, &b->cluster_slot_cap, size_t(teams / std::max(k.ctas, 1) + 1)))
    return rc;
  // graphs largest first by work (CSR entries, repulsive pairs and a fixed cost per
  // minibatch, all per epoch); with two-CTA teams the graphs above 0.6 of the
  // balanced share of one CTA are trained by a whole cluster
  {
    std::vector<double> w(b->n_graphs);
    double total_w = 0;
    for (int g = 0; g < b->n_graphs; ++g) {
      w[g] = double(b->nnz[g]) + double(ns) * double(b->n[g]) + 900.0 * b->ginfo[g].batches;
      total_w += w[g];
    }
    std::stable_sort(b->order.begin(), b->order.end(), [&](int x, int y) { return w[x] > w[y]; });
    b->n_big = 0;
    if (k.ctas > 1)
      while (b->n_big < b->n_graphs && w[b->order[b->n_big]] > 0.6 * total_w / teams) ++b->n_big;
    BCUDA(b, cudaMemcpyAsync(b->d_order, b->order.data(), b->order.size() * sizeof(int32_t), cudaMemcpyHostToDevice,
                             b->stream));
    BCUDA(b, cudaStreamSynchronize(b->stream));
  }
  BatchedArgs &a = b->args;
  a = BatchedArgs{};
  a.graphs = b->d_graphs;
  a.order = b->d_order;
  a.n_graphs = b->n_graphs;
  a.next_graph = b->d_next;
  a.col = b->d_col;
  a.items = b->d_items;
  a.batch_item_off = b->d_bitem;
  a.batch_split_off = b->d_bsplit;
  a.splits = b->d_splits;
  a.xm = b->d_xm;
  a.xb = b->d_xb;
  a.negs = b->d_negs;
  a.lr = b->d_lr;
  a.epochs = epochs;
  a.batch = B;
  a.ns = ns;
  a.quirks = b->opt.ref_quirks;
  a.compute_loss = b->loss_mode != DE_LOSS_NONE;
  a.loss_from = b->loss_mode == DE_LOSS_LAST_EPOCH ? epochs - 1 : 0;
  a.bound = float(b->opt.max_bound);
  a.stage = b->d_stage;
  a.slots = b->d_slots;
  a.slot_stride = b->max_slots;
  a.loss = b->d_loss;
  a.near_r = b->near_r;
  a.trace = b->d_trace;
  a.cap = cap;
  a.err = b->d_err;
  a.n_big = b->n_big;
  a.next_big = b->d_next + 1;
  a.cluster_slot = b->d_cluster_slot;
  a.item_loss = b->d_item_loss;
  a.item_stride = b->max_batch_items;
  a.stage_ids = k.stage_ids;
  b->ctas = k.ctas;
  b->kernel = k.fn;
  b->teams = teams;
  b->block = k.block;
  b->smem = k.smem;
  return DE_OK;
}

// The whole run: reset the team work counter, then one persistent launch.
int launch_batched(de_batch *b, cudaStream_t st) {
  BCUDA(b, cudaMemsetAsync(b->d_next, 0, 2 * sizeof(int32_t), st));
  if (b->ctas == 1) {
    b->kernel<<<b->teams, b->block, b->smem, st>>>(b->args);
  } else {
    cudaLaunchConfig_t cfg{};
    cfg.gridDim = dim3(b->teams);
    cfg.blockDim = dim3(b->block);
    cfg.dynamicSmemBytes = b->smem;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = b->ctas;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    BCUDA(b, cudaLaunchKernelEx(&cfg, b->kernel, b->args));
  }
  BCUDA(b, cudaGetLastError());
  return DE_OK;
}

}  // namespace

extern "C" {

int de_batch_create(int32_t n_graphs, const int64_t *n, const int64_t *const *rowptr, const int64_t *const *col,
                    int32_t dim, const de_options *opts, de_batch **out) {
  if (!out) return bfail(nullptr, DE_ERR_INVALID, "out is NULL");
  *out = nullptr;
  if (n_graphs <= 0 || !n || !rowptr || !col) return bfail(nullptr, DE_ERR_INVALID, "bad graph arguments");
  if (dim != 32 && dim != 64 && dim != 128) return bfail(nullptr, DE_ERR_INVALID, "the batched form takes dim 32, 64 or 128");
  auto b = std::make_unique<de_batch>();
  if (opts) b->opt = *opts; else de_default_options(&b->opt);
  if (b->opt.precision != DE_PRECISION_FP32 && b->opt.precision != DE_PRECISION_BF16)
    return bfail(nullptr, DE_ERR_INVALID, "unknown precision");
  b->n_graphs = n_graphs;
  b->dim = dim;
  if (b->opt.edge_cap > 0) b->shape.edge_cap = b->opt.edge_cap;
  b->device = b->opt.device;
  b->n.resize(n_graphs);
  b->nnz.resize(n_graphs);
  b->voff.resize(n_graphs);
  b->eoff.resize(n_graphs);
  b->rowptr.resize(n_graphs);
  b->edges_into_last.assign(n_graphs, 0);
  std::vector<int32_t> rp32, col32;
  for (int g = 0; g < n_graphs; ++g) {
    const int64_t ng = n[g];
    if (ng <= 0 || !rowptr[g]) return bfail(nullptr, DE_ERR_INVALID, "graph " + std::to_string(g) + ": empty");
    const int64_t nnz = rowptr[g][ng];
    if (rowptr[g][0] != 0 || nnz < 0 || nnz >= (int64_t(1) << 31)) return bfail(nullptr, DE_ERR_INVALID, "graph " + std::to_string(g) + ": bad rowptr");
    for (int64_t i = 0; i < ng; ++i)
      if (rowptr[g][i + 1] < rowptr[g][i]) return bfail(nullptr, DE_ERR_INVALID, "graph " + std::to_string(g) + ": rowptr decreases");
    for (int64_t e = 0; e < nnz; ++e) {
      if (col[g][e] < 0 || col[g][e] >= ng) return bfail(nullptr, DE_ERR_INVALID, "graph " + std::to_string(g) + ": column out of range");
      b->edges_into_last[g] += col[g][e] == ng - 1;
    }
    b->n[g] = ng;
    b->nnz[g] = nnz;
    b->voff[g] = b->total_n;
    b->eoff[g] = b->total_nnz;
    b->rowptr[g].assign(rowptr[g], rowptr[g] + ng + 1);
    for (int64_t e = 0; e < nnz; ++e) col32.push_back(int32_t(col[g][e]));
    b->total_n += ng;
    b->total_nnz += nnz;
  }
  de_batch *raw = b.get();
  auto bail = [&](int rc) {
    std::string m = raw->err;
    de_batch_destroy(b.release());
    return bfail(nullptr, rc, m);
  };
  cudaError_t e = cudaSetDevice(b->device);
  if (e != cudaSuccess) return bail(bfail(raw, DE_ERR_CUDA, cudaGetErrorString(e)));
  if (b->opt.stream) {
    b->stream = static_cast<cudaStream_t>(b->opt.stream);
  } else {
    if ((e = cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking)) != cudaSuccess)
      return bail(bfail(raw, DE_ERR_CUDA, cudaGetErrorString(e)));
    b->own_stream = true;
  }
  const size_t xn = size_t(b->total_n) * dim;
  if ((e = cudaMalloc(&b->d_col, std::max<size_t>(col32.size(), 1) * sizeof(int32_t))) != cudaSuccess ||
      (e = cudaMalloc(&b->d_xm, xn * sizeof(float))) != cudaSuccess ||
      (e = cudaMalloc(&b->d_next, 2 * sizeof(int32_t))) != cudaSuccess ||
      (e = cudaMalloc(&b->d_trace, size_t(n_graphs) * 3 * sizeof(long long))) != cudaSuccess ||
      (e = cudaMalloc(&b->d_err, sizeof(int32_t))) != cudaSuccess ||
      (e = cudaMemsetAsync(b->d_err, 0, sizeof(int32_t), b->stream)) != cudaSuccess ||
      (e = cudaMemsetAsync(b->d_xm, 0, xn * sizeof(float), b->stream)) != cudaSuccess ||
      (!col32.empty() && (e = cudaMemcpyAsync(b->d_col, col32.data(), col32.size() * sizeof(int32_t),
                                              cudaMemcpyHostToDevice, b->stream)) != cudaSuccess) ||
      (e = cudaStreamSynchronize(b->stream)) != cudaSuccess)
    return bail(bfail(raw, e == cudaErrorMemoryAllocation ? DE_ERR_OOM : DE_ERR_CUDA, cudaGetErrorString(e)));
  if (b->opt.precision == DE_PRECISION_BF16) {
    if ((e = cudaMalloc(&b->d_xb, xn * sizeof(__nv_bfloat16))) != cudaSuccess ||
        (e = cudaMemsetAsync(b->d_xb, 0, xn * sizeof(__nv_bfloat16), b->stream)) != cudaSuccess ||
        (e = cudaStreamSynchronize(b->stream)) != cudaSuccess)
      return bail(bfail(raw, e == cudaErrorMemoryAllocation ? DE_ERR_OOM : DE_ERR_CUDA, cudaGetErrorString(e)));
  }
  *out = b.release();
  return DE_OK;
}

int de_batch_destroy(de_batch *b) {
  if (!b) return DE_OK;
  cudaSetDevice(b->device);
  if (b->stream) cudaStreamSynchronize(b->stream);
  if (b->exec) cudaGraphExecDestroy(b->exec);
  for (void *p : {static_cast<void *>(b->d_col), static_cast<void *>(b->d_xm),
                  static_cast<void *>(b->d_xb), static_cast<void *>(b->d_graphs), static_cast<void *>(b->d_order),
                  static_cast<void *>(b->d_next), static_cast<void *>(b->d_items), static_cast<void *>(b->d_bitem),
                  static_cast<void *>(b->d_bsplit), static_cast<void *>(b->d_splits), static_cast<void *>(b->d_negs),
                  static_cast<void *>(b->d_lr), static_cast<void *>(b->d_loss), static_cast<void *>(b->d_stage),
                  static_cast<void *>(b->d_slots), static_cast<void *>(b->d_trace),
                  static_cast<void *>(b->d_err), static_cast<void *>(b->d_item_loss),
                  static_cast<void *>(b->d_cluster_slot)})
    if (p) cudaFree(p);
  if (b->own_stream && b->stream) cudaStreamDestroy(b->stream);
  delete b;
  return DE_OK;
}

int de_batch_set_embeddings_f32(de_batch *b, int32_t graph, const float *x) {
  if (!b || !x || graph < -1 || graph >= b->n_graphs) return bfail(b, DE_ERR_INVALID, "bad argument");
  BCUDA(b, cudaSetDevice(b->device));
  const size_t cnt = size_t(graph < 0 ? b->total_n : b->n[graph]) * b->dim;
  const size_t off = graph < 0 ? 0 : size_t(b->voff[graph]) * b->dim;
  BCUDA(b, cudaMemcpyAsync(b->d_xm + off, x, cnt * sizeof(float), cudaMemcpyHostToDevice, b->stream));
  if (b->d_xb) BCUDA(b, de::launch_f32_to_bf16(b->d_xm + off, b->d_xb + off, int64_t(cnt), b->stream));
  BCUDA(b, cudaStreamSynchronize(b->stream));
  return DE_OK;
}

int de_batch_get_embeddings_f32(de_batch *b, int32_t graph, float *x) {
  if (!b || !x || graph < -1 || graph >= b->n_graphs) return bfail(b, DE_ERR_INVALID, "bad argument");
  BCUDA(b, cudaSetDevice(b->device));
  const size_t cnt = size_t(graph < 0 ? b->total_n : b->n[graph]) * b->dim;
  const size_t off = graph < 0 ? 0 : size_t(b->voff[graph]) * b->dim;
  BCUDA(b, cudaMemcpyAsync(x, b->d_xm + off, cnt * sizeof(float), cudaMemcpyDeviceToHost, b->stream));
  BCUDA(b, cudaStreamSynchronize(b->stream));
  return DE_OK;
}

int de_batch_set_shape(de_batch *b, const de_batch_shape *shape) {
  if (!b || !shape) return DE_ERR_INVALID;
  if (!pick_kernel(b->dim, b->opt.precision == DE_PRECISION_BF16, *shape).fn)
    return bfail(b, DE_ERR_UNSUPPORTED, "no kernel for this dim and team shape");
  b->shape = *shape;
  if (b->exec) cudaGraphExecDestroy(b->exec);
  b->exec = nullptr;
  b->prepared_epochs = 0;
  return DE_OK;
}

int de_batch_get_shape(const de_batch *b, de_batch_shape *shape) {
  if (!b || !shape) return DE_ERR_INVALID;
  *shape = b->shape;
  return DE_OK;
}

int de_batch_prepare(de_batch *b, int32_t epochs, int32_t batch_size, int32_t ns, const double *lr_per_epoch) {
  if (!b) return DE_ERR_INVALID;
  if (epochs <= 0 || batch_size <= 0 || ns < 0 || !lr_per_epoch)
    return bfail(b, DE_ERR_INVALID, "epochs > 0, batch_size > 0, ns >= 0, lr given");
  if (b->exec) cudaGraphExecDestroy(b->exec);
  b->exec = nullptr;
  b->prepared_epochs = 0;
  if (int rc = prepare_batched(b, epochs, batch_size, ns, lr_per_epoch, b->shape)) return rc;
  // one launch for every graph and epoch, captured once and replayed as a CUDA graph
  cudaGraph_t graph = nullptr;
  BCUDA(b, cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
  const int rc = launch_batched(b, b->stream);
  cudaError_t e = cudaStreamEndCapture(b->stream, &graph);
  if (rc) {
    if (graph) cudaGraphDestroy(graph);
    return rc;
  }
  BCUDA(b, e);
  e = cudaGraphInstantiate(&b->exec, graph, 0);
  cudaGraphDestroy(graph);
  BCUDA(b, e);
  b->prepared_epochs = epochs;
  return DE_OK;
}

int de_batch_launch(de_batch *b) {
  if (!b) return DE_ERR_INVALID;
  if (!b->exec) return bfail(b, DE_ERR_STATE, "de_batch_launch before de_batch_prepare");
  BCUDA(b, cudaSetDevice(b->device));
  BCUDA(b, cudaGraphLaunch(b->exec, b->stream));
  return DE_OK;
}

int de_batch_wait(de_batch *b, double *loss) {
  if (!b) return DE_ERR_INVALID;
  BCUDA(b, cudaSetDevice(b->device));
  BCUDA(b, cudaStreamSynchronize(b->stream));
  int32_t derr = 0;
  BCUDA(b, cudaMemcpyAsync(&derr, b->d_err, sizeof(int32_t), cudaMemcpyDeviceToHost, b->stream));
  BCUDA(b, cudaStreamSynchronize(b->stream));
  if (derr) {
    BCUDA(b, cudaMemsetAsync(b->d_err, 0, sizeof(int32_t), b->stream));
    return bfail(b, DE_ERR_CUDA, "a bounded wait in the staged kernel gave up; results of this launch are invalid");
  }
  if (loss && b->prepared_epochs > 0)
    BCUDA(b, cudaMemcpyAsync(loss, b->d_loss, size_t(b->prepared_epochs) * b->n_graphs * sizeof(double),
                             cudaMemcpyDeviceToHost, b->stream));
  BCUDA(b, cudaStreamSynchronize(b->stream));
  return DE_OK;
}

int de_batch_run(de_batch *b, int32_t epochs, int32_t batch_size, int32_t ns, const double *lr_per_epoch,
                 double *loss) {
  if (!b) return DE_ERR_INVALID;
  if (epochs < 0 || batch_size <= 0 || ns < 0 || (epochs > 0 && !lr_per_epoch))
    return bfail(b, DE_ERR_INVALID, "epochs >= 0, batch_size > 0, ns >= 0, lr given");
  if (epochs == 0) return DE_OK;
  if (int rc = de_batch_prepare(b, epochs, batch_size, ns, lr_per_epoch)) return rc;
  if (int rc = de_batch_launch(b)) return rc;
  return de_batch_wait(b, loss);
}

int64_t de_batch_edge_updates(de_batch *b, int32_t epochs, int32_t batch_size, int32_t ns) {
  if (!b || epochs < 0 || batch_size <= 0 || ns < 0) return -1;
  int64_t total = 0;
  std::vector<int64_t> draw(std::max(ns, 1));
  for (int g = 0; g < b->n_graphs; ++g) {
    const int64_t n = b->n[g];
    const int batches = int(n / batch_size + (n % batch_size ? 1 : 0));
    const int last = (n % batch_size) ? int(n - int64_t(batch_size) * (batches - 1)) : batch_size;
    total += (b->nnz[g] - (b->opt.ref_quirks ? b->edges_into_last[g] : 0)) * epochs;
    for (int e = 0; e < epochs; ++e)
      for (int j = 0; j < batches; ++j) {
        de_negatives(n, e + j, ns, draw.data());
        int valid = 0;
        for (int q = 0; q < ns; ++q) valid += draw[q] < n;
        const int rows = (j == batches - 1) ? last : batch_size;
        total += int64_t((b->opt.ref_quirks && e > 0) ? last : rows) * valid;
      }
  }
  return total;
}

int de_batch_autotune(de_batch *b, int32_t epochs, int32_t batch_size, int32_t ns, double lr, float *ms,
                      de_batch_shape *shapes, int32_t capacity, int32_t *count, de_batch_shape *best) {
  if (!b) return DE_ERR_INVALID;
  if (epochs <= 0 || batch_size <= 0 || ns < 0) return bfail(b, DE_ERR_INVALID, "epochs > 0, batch_size > 0, ns >= 0");
  BCUDA(b, cudaSetDevice(b->device));
  // the tuning runs are real training steps: keep the embeddings and put them back
  const size_t xn = size_t(b->total_n) * b->dim;
  float *save_m = nullptr;
  __nv_bfloat16 *save_b = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  auto cleanup = [&]() {
    if (save_m) cudaFree(save_m);
    if (save_b) cudaFree(save_b);
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
  };
  cudaError_t e = cudaMalloc(&save_m, xn * sizeof(float));
  if (e == cudaSuccess && b->d_xb) e = cudaMalloc(&save_b, xn * sizeof(__nv_bfloat16));
  if (e == cudaSuccess) e = cudaMemcpyAsync(save_m, b->d_xm, xn * sizeof(float), cudaMemcpyDeviceToDevice, b->stream);
  if (e == cudaSuccess && b->d_xb)
    e = cudaMemcpyAsync(save_b, b->d_xb, xn * sizeof(__nv_bfloat16), cudaMemcpyDeviceToDevice, b->stream);
  if (e == cudaSuccess) e = cudaEventCreate(&e0);
  if (e == cudaSuccess) e = cudaEventCreate(&e1);
  if (e != cudaSuccess) {
    cleanup();
    return bfail(b, e == cudaErrorMemoryAllocation ? DE_ERR_OOM : DE_ERR_CUDA, cudaGetErrorString(e));
  }
  // candidate shapes: the register kernel over vertices per warp x team warps x
  // edge cap, the staged kernel over team warps x edge cap x pairs x stages
  std::vector<de_batch_shape> cand;
  for (int v : {1, 2, 4})
    for (int w : {4, 8, 16, 32})
      for (int c : {32, 64, 128}) cand.push_back(de_batch_shape{DE_BATCH_REGISTER, v, w, c, 0, 0, 1});
  if (ns <= kStagedMaxNs) {  // the staged kernels take at most 32 negatives
    for (int fam : {DE_BATCH_STAGED, DE_BATCH_ROWS})
      for (int w : {4, 8, 12, 16})
        for (int c : {8, 16, 32})
          for (int u : {1, 2})
            for (int st : {3, 4}) cand.push_back(de_batch_shape{fam, 0, w, c, u, st, 1});
    for (int ct : {2, 4})
      for (int w : {8, 16})
        for (int c : {16, 32})
          for (int u : {1, 2})
            for (int st : {3, 4}) cand.push_back(de_batch_shape{DE_BATCH_STAGED, 0, w, c, u, st, ct});
  }
  const bool bf16 = b->opt.precision == DE_PRECISION_BF16;
  std::vector<double> lrs(epochs, lr);
  float best_ms = -1.f;
  de_batch_shape best_shape = b->shape;
  int tried = 0, rc = DE_OK;
  for (const de_batch_shape &sh : cand) {
    if (!pick_kernel(b->dim, bf16, sh, ns).fn) continue;
    rc = prepare_batched(b, epochs, batch_size, ns, lrs.data(), sh);
    if (rc) break;
    b->args.compute_loss = 0;  // shapes are timed on the training work alone
    e = cudaMemcpyAsync(b->d_xm, save_m, xn * sizeof(float), cudaMemcpyDeviceToDevice, b->stream);
    if (e == cudaSuccess && b->d_xb)
      e = cudaMemcpyAsync(b->d_xb, save_b, xn * sizeof(__nv_bfloat16), cudaMemcpyDeviceToDevice, b->stream);
    if (e == cudaSuccess) e = cudaEventRecord(e0, b->stream);
    if (e == cudaSuccess) rc = launch_batched(b, b->stream);
    if (e == cudaSuccess && !rc) e = cudaEventRecord(e1, b->stream);
    if (e == cudaSuccess && !rc) e = cudaEventSynchronize(e1);
    float t = 0.f;
    if (e == cudaSuccess && !rc) e = cudaEventElapsedTime(&t, e0, e1);
    int32_t derr = 0;
    if (e == cudaSuccess && !rc) e = cudaMemcpyAsync(&derr, b->d_err, sizeof(int32_t), cudaMemcpyDeviceToHost, b->stream);
    if (e == cudaSuccess && !rc) e = cudaStreamSynchronize(b->stream);
    if (e != cudaSuccess && !rc) rc = bfail(b, DE_ERR_CUDA, cudaGetErrorString(e));
    if (!rc && derr) rc = bfail(b, DE_ERR_CUDA, "a bounded wait in the staged kernel gave up during tuning");
    if (rc) break;
    if (ms && tried < capacity) ms[tried] = t;
    if (shapes && tried < capacity) shapes[tried] = sh;
    ++tried;
    if (best_ms < 0.f || t < best_ms) best_ms = t, best_shape = sh;
  }
  if (!rc) {
    e = cudaMemcpyAsync(b->d_xm, save_m, xn * sizeof(float), cudaMemcpyDeviceToDevice, b->stream);
    if (e == cudaSuccess && b->d_xb)
      e = cudaMemcpyAsync(b->d_xb, save_b, xn * sizeof(__nv_bfloat16), cudaMemcpyDeviceToDevice, b->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(b->stream);
    if (e != cudaSuccess) rc = bfail(b, DE_ERR_CUDA, cudaGetErrorString(e));
  } else {
    cudaStreamSynchronize(b->stream);
  }
  cleanup();
  if (b->exec) cudaGraphExecDestroy(b->exec);
  b->exec = nullptr;
  b->prepared_epochs = 0;
  if (rc) return rc;
  b->shape = best_shape;
  if (count) *count = tried;
  if (best) *best = best_shape;
  return DE_OK;
}

int de_batch_set_loss(de_batch *b, int32_t mode) {
  if (!b || (mode != DE_LOSS_NONE && mode != DE_LOSS_EVERY_EPOCH && mode != DE_LOSS_LAST_EPOCH))
    return bfail(b, DE_ERR_INVALID, "loss mode must be DE_LOSS_NONE, DE_LOSS_EVERY_EPOCH or DE_LOSS_LAST_EPOCH");
  b->loss_mode = mode;
  if (b->exec) cudaGraphExecDestroy(b->exec);
  b->exec = nullptr;
  b->prepared_epochs = 0;
  return DE_OK;
}

int de_batch_set_near_distance(de_batch *b, float near_r) {
  if (!b || !(near_r >= 0.f)) return bfail(b, DE_ERR_INVALID, "near_r must be >= 0");
  b->near_r = near_r;
  if (b->exec) cudaGraphExecDestroy(b->exec);
  b->exec = nullptr;
  b->prepared_epochs = 0;
  return DE_OK;
}

int de_batch_trace(de_batch *b, int64_t *out) {
  if (!b || !out) return DE_ERR_INVALID;
  BCUDA(b, cudaSetDevice(b->device));
  BCUDA(b, cudaStreamSynchronize(b->stream));
  BCUDA(b, cudaMemcpyAsync(out, b->d_trace, size_t(b->n_graphs) * 3 * sizeof(long long), cudaMemcpyDeviceToHost,
                           b->stream));
  BCUDA(b, cudaStreamSynchronize(b->stream));
  return DE_OK;
}

void *de_batch_stream(de_batch *b) { return b ? static_cast<void *>(b->stream) : nullptr; }

const char *de_batch_last_error(const de_batch *b) { return b ? b->err.c_str() : de_last_error(nullptr); }

}  // extern "C"
