// Host runtime of the C ABI declared in include/distembed_gb300.h.
//
// A handle owns one resident graph (int32 CSR on the device) and its embedding.
// de_run mirrors EmbeddingAlgo::algo_force2_vec_ns at one rank
// (cpp/algo/algo.hpp:74-262): batches = ceil(n / B), last_batch_size, seed =
// epoch + batch, attractive -> repulsive -> update per minibatch, minibatches
// strictly in order.  The minibatch sequence of one epoch is captured once per
// (B, ns) into a CUDA graph and replayed per epoch; the epoch index, learning
// rate and negatives are read from device memory so the same graph serves
// every epoch.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <random>
#include <string>
#include <vector>

#include "../../include/distembed_gb300.h"
#include "de_internal.h"

using namespace de;

namespace {
thread_local std::string g_create_error;
}

namespace de {
// Error text for entry points without a handle (read by de_last_error(NULL)).
void set_thread_error(const std::string &msg) { g_create_error = msg; }
}  // namespace de

struct de_handle {
  int64_t n = 0, nnz = 0;
  int dim = 0;
  de_options opt{};
  int device = 0;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  std::string err;

  // resident graph and embedding
  int32_t *d_rowptr = nullptr, *d_col = nullptr;
  float *d_x = nullptr;
  std::vector<int64_t> rowptr;  // host copy for schedule building
  int64_t edges_into_last = 0;  // CSR entries whose column is n-1

  // per-minibatch-size state
  Schedule sched;
  float *d_stage = nullptr;  // three minibatch staging buffers
  float *d_y = nullptr;      // SpMM output [n, dim]
  int32_t *d_spmm_off = nullptr;  // SpMM: per-minibatch first partial slot, then first counter
  int spmm_batch = 0, spmm_cap = 0;
  // sparse embedding: FP64 rows (INT_MIN = absent; d_x holds their FP32 mirror),
  // the batch collector [B, dim] and the present-entry count
  double *d_sx = nullptr;
  double *d_coll = nullptr;
  size_t coll_cap = 0;
  unsigned long long *d_present = nullptr;
  int sparse_batch = 0;
  bool sparse_in_mirror = false;  // the last run's result is in d_x (merge = 1)
  bool keep_last_edges = false;   // F7 off for the plain pass (the sparse embedding's merge = 1)
  int64_t spmm_parts = 0, spmm_split = 0;
  size_t stage_cap = 0;
  float *d_parts = nullptr;
  size_t parts_cap = 0;
  int32_t *d_counters = nullptr;
  size_t counters_cap = 0;
  double *d_loss_partial = nullptr;
  size_t loss_partial_cap = 0;
  double *d_block_sums = nullptr;  // [kFlushBlocks]
  int32_t *d_done = nullptr;       // flush arrival counter

  // per-call state
  int32_t *d_epoch = nullptr;
  double *d_loss = nullptr;
  size_t loss_cap = 0;
  int32_t *d_negs = nullptr;
  size_t negs_cap = 0;
  float *d_lr = nullptr;
  size_t lr_cap = 0;
  int32_t *h_negs = nullptr;  // pinned
  size_t h_negs_cap = 0;
  float *h_lr = nullptr;      // pinned
  size_t h_lr_cap = 0;
  double *h_loss = nullptr;   // pinned
  size_t h_loss_cap = 0;
  int32_t *h_epoch = nullptr;  // pinned [2]: epoch within call, first epoch
  cudaEvent_t upload_done = nullptr;

  // captured epoch
  cudaGraphExec_t graph = nullptr;
  int graph_batch = 0, graph_ns = -1;

  // FP64 <-> FP32 staging for the host embedding copies
  double *d_stage64 = nullptr;
  size_t stage64_cap = 0;

  // BF16 precision form: BF16 copy of the embedding (d_x is the FP32 master),
  // per-minibatch buffers and the tensor maps of the GEMM operands
  __nv_bfloat16 *d_xb = nullptr;
  float *d_abuf = nullptr;
  size_t abuf_cap = 0;
  float *d_rbuf = nullptr;
  size_t rbuf_cap = 0;
  cudaStream_t stream2 = nullptr;  // the repulsion GEMMs, forked from and joined to `stream`
  cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
  __nv_bfloat16 *d_nb = nullptr;
  size_t nb_cap = 0;
  float *d_nn = nullptr;
  int32_t *d_nid = nullptr;
  size_t kpad_cap = 0;
  uint32_t *d_near_bits = nullptr;  // [B, 32], zero between minibatches
  size_t near_cap = 0;
  double *d_loss_row = nullptr;
  int32_t *d_err = nullptr;
  int kpad = 0;
  CUtensorMap map_x{}, map_n{};

  // where device and host buffers come from (default: cudaMalloc / cudaHostAlloc)
  MemHooks hooks{};
};

namespace {

int fail(de_handle *h, int code, const std::string &msg) {
  if (h) h->err = msg; else g_create_error = msg;
  return code;
}

int cuda_fail(de_handle *h, cudaError_t e, const char *what) {
  return fail(h, e == cudaErrorMemoryAllocation ? DE_ERR_OOM : DE_ERR_CUDA,
              std::string(what) + ": " + cudaGetErrorString(e));
}

#define DE_CUDA(h, call)                                  \
  do {                                                    \
    cudaError_t e_ = (call);                              \
    if (e_ != cudaSuccess) return cuda_fail(h, e_, #call); \
  } while (0)

// Device and host buffers of a handle: from its memory hooks when it has them
// (a caller-owned arena: no implicit device synchronisation on free), else from
// cudaMalloc / cudaHostAlloc (pinned).
template <class H>
cudaError_t dev_alloc(const H &h, void **p, size_t bytes) {
  if (h->hooks.dalloc) {
    *p = h->hooks.dalloc(h->hooks.ctx, bytes);
    return *p ? cudaSuccess : cudaErrorMemoryAllocation;
  }
  return cudaMalloc(p, bytes);
}

template <class H>
void dev_free(const H &h, void *p) {
  if (!p) return;
  if (h->hooks.dalloc) {
    // an arena block may be handed out again at once: no kernel of this
    // handle may still be using it
    if (h->stream) cudaStreamSynchronize(h->stream);
    h->hooks.dfree(h->hooks.ctx, p);
  } else {
    cudaFree(p);
  }
}

template <class H>
cudaError_t host_alloc(const H &h, void **p, size_t bytes) {
  if (h->hooks.dalloc) {
    *p = std::malloc(bytes);
    return *p ? cudaSuccess : cudaErrorMemoryAllocation;
  }
  return cudaHostAlloc(p, bytes, cudaHostAllocDefault);
}

template <class H>
void host_free(const H &h, void *p) {
  if (!p) return;
  if (h->hooks.dalloc) std::free(p);
  else cudaFreeHost(p);
}

template <typename T>
int grow(de_handle *h, T **p, size_t *cap, size_t need, bool *moved = nullptr) {
  if (need <= *cap && *p) return DE_OK;
  size_t want = std::max(need, size_t(1));
  if (*p) dev_free(h, *p);
  *p = nullptr;
  *cap = 0;
  DE_CUDA(h, dev_alloc(h, reinterpret_cast<void **>(p), want * sizeof(T)));
  *cap = want;
  if (moved) *moved = true;
  return DE_OK;
}

template <typename T>
int grow_pinned(de_handle *h, T **p, size_t *cap, size_t need) {
  if (need <= *cap && *p) return DE_OK;
  if (*p) host_free(h, *p);
  *p = nullptr;
  *cap = 0;
  DE_CUDA(h, host_alloc(h, reinterpret_cast<void **>(p), std::max(need, size_t(1)) * sizeof(T)));
  *cap = std::max(need, size_t(1));
  return DE_OK;
}

int default_edge_cap(int) { return kMaxEdgeCap; }

// Work items of minibatch size B: each row of each minibatch becomes one item,
// or ceil(deg / cap) items when its degree exceeds the cap.
void build_schedule(const de_handle *h, int B, int cap, Schedule &s, std::vector<WorkItem> &items) {
  s.batch = B;
  s.batches = int(h->n / B + (h->n % B ? 1 : 0));
  s.last_batch_size = (h->n % B) ? int(h->n - int64_t(B) * (s.batches - 1)) : B;
  s.edge_cap = cap;
  s.item_off.assign(s.batches + 1, 0);
  s.n_parts.assign(s.batches, 0);
  s.n_split.assign(s.batches, 0);
  s.cta_off.assign(s.batches + 1, 0);
  s.max_parts = s.max_split = 0;
  items.clear();
  for (int j = 0; j < s.batches; ++j) {
    const int64_t base = int64_t(j) * B;
    const int rows = int(std::min<int64_t>(B, h->n - base));
    int parts = 0, split = 0;
    for (int r = 0; r < rows; ++r) {
      const int64_t e0 = h->rowptr[base + r], e1 = h->rowptr[base + r + 1];
      const int64_t deg = e1 - e0;
      if (deg <= cap) {
        items.push_back(WorkItem{r, int32_t(e0), int32_t(e1), 1, 0, 0, 0, j});
      } else {
        const int np = int((deg + cap - 1) / cap);
        const int ng = (np + kCombineGroup - 1) / kCombineGroup;
        for (int p = 0; p < np; ++p) {
          const int64_t a = e0 + int64_t(p) * cap, b = std::min<int64_t>(e1, a + cap);
          items.push_back(WorkItem{r, int32_t(a), int32_t(b), np, parts, p, split, j});
        }
        parts += np + (ng > 1 ? ng : 0);
        split += ng + (ng > 1 ? 1 : 0);
      }
    }
    // longest items first: the block scheduler then starts them first
    std::stable_sort(items.begin() + s.item_off[j], items.end(), [](const WorkItem &x, const WorkItem &y) {
      return (x.e_end - x.e_begin) > (y.e_end - y.e_begin);
    });
    s.item_off[j + 1] = int64_t(items.size());
    s.n_parts[j] = parts;
    s.n_split[j] = split;
    s.max_parts = std::max(s.max_parts, parts);
    s.max_split = std::max(s.max_split, split);
    const int64_t n_items = s.item_off[j + 1] - s.item_off[j];
    s.cta_off[j + 1] = s.cta_off[j] + (n_items + kPlainWarps - 1) / kPlainWarps;
  }
  s.n_items = int64_t(items.size());
}

void drop_graph(de_handle *h) {
  if (h->graph) cudaGraphExecDestroy(h->graph);
  h->graph = nullptr;
  h->graph_batch = 0;
  h->graph_ns = -1;
}

int ensure_schedule(de_handle *h, int B) {
  const int cap = h->opt.edge_cap > 0 ? std::min(h->opt.edge_cap, kMaxEdgeCap) : default_edge_cap(h->dim);
  if (h->sched.batch == B && h->sched.edge_cap == cap && h->sched.d_items) return DE_OK;
  drop_graph(h);
  if (h->sched.d_items) dev_free(h, h->sched.d_items);
  h->sched = Schedule{};
  std::vector<WorkItem> items;
  build_schedule(h, B, cap, h->sched, items);
  DE_CUDA(h, dev_alloc(h, reinterpret_cast<void **>(&h->sched.d_items), std::max<size_t>(items.size(), 1) * sizeof(WorkItem)));
  // on the handle's stream (its kernels do not wait for the legacy stream), and
  // finished before `items` goes away
  DE_CUDA(h, cudaMemcpyAsync(h->sched.d_items, items.data(), items.size() * sizeof(WorkItem),
                             cudaMemcpyHostToDevice, h->stream));
  DE_CUDA(h, cudaStreamSynchronize(h->stream));
  return DE_OK;
}

void draw_negatives(int64_t n, int seed, int ns, int32_t *out) {
  std::minstd_rand gen(seed);
  std::uniform_int_distribution<int> dist(0, int(n));
  for (int k = 0; k < ns; ++k) out[k] = dist(gen);
}

typedef CUresult (*EncodeTiledFn)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                  const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

// 2-D BF16 tensor map over a row-major [rows, cols] array, box [box_rows, 64],
// 128-byte swizzle (the layout the tcgen05 operand descriptors expect).
int encode_map(de_handle *h, CUtensorMap *m, void *base, uint64_t rows, uint64_t cols, uint32_t box_rows) {
  static EncodeTiledFn enc = nullptr;
  if (!enc) {
    cudaDriverEntryPointQueryResult q;
    void *fn = nullptr;
    DE_CUDA(h, cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q));
    if (!fn) return fail(h, DE_ERR_UNSUPPORTED, "cuTensorMapEncodeTiled is not available");
    enc = reinterpret_cast<EncodeTiledFn>(fn);
  }
  cuuint64_t dims[2] = {cols, rows};
  cuuint64_t strides[1] = {cols * 2};
  cuuint32_t box[2] = {64, box_rows};
  cuuint32_t es[2] = {1, 1};
  CUresult r = enc(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, base, dims, strides, box, es, CU_TENSOR_MAP_INTERLEAVE_NONE,
                   CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) return fail(h, DE_ERR_CUDA, "cuTensorMapEncodeTiled failed");
  return DE_OK;
}

// Enqueues one epoch of the BF16 form on st.  ev (nullable): 3 events per
// minibatch (before each of its launches) and one before the flush.
cudaError_t enqueue_epoch_bf16(de_handle *h, int ns, cudaStream_t st, cudaEvent_t *ev) {
  const Schedule &s = h->sched;
  cudaError_t err = cudaSuccess;
  for (int j = 0; j < s.batches && err == cudaSuccess; ++j) {
    BF16BatchArgs a{};
    a.xm = h->d_x;
    a.xb = h->d_xb;
    a.rowptr = h->d_rowptr;
    a.col = h->d_col;
    a.items = s.d_items + s.item_off[j];
    a.n_items = int32_t(s.item_off[j + 1] - s.item_off[j]);
    a.base = int32_t(int64_t(j) * s.batch);
    a.rows = int32_t(std::min<int64_t>(s.batch, h->n - a.base));
    a.last_batch_size = s.last_batch_size;
    a.batch_id = j;
    a.batches = s.batches;
    a.n = int32_t(h->n);
    a.quirks = h->opt.ref_quirks;
    a.compute_loss = h->opt.compute_loss;
    a.bound = float(h->opt.max_bound);
    a.negs = h->d_negs;
    a.ns = ns;
    a.kpad = h->kpad;
    a.lr = h->d_lr;
    a.epoch = h->d_epoch;
    a.P = h->d_parts;
    a.counters = h->d_counters;
    a.abuf = h->d_abuf;
    a.rbuf = h->d_rbuf;
    a.nb = h->d_nb;
    a.nn = h->d_nn;
    a.nid = h->d_nid;
    a.near_bits = h->d_near_bits;
    a.loss_item = h->d_loss_partial;
    a.loss_off = s.item_off[j];
    a.loss_row = h->d_loss_row;
    a.err = h->d_err;
    err = launch_bf16_batch(h->dim, a, h->map_x, h->map_n, st, ev ? ev + 4 * j : nullptr, h->stream2,
                            h->ev_fork, h->ev_join);
  }
  if (err == cudaSuccess) {
    BF16FlushArgs f{};
    f.loss_item = h->d_loss_partial;
    f.loss_row = h->d_loss_row;
    f.n_items = s.n_items;
    f.n_rows = h->n;
    f.block_sums = h->d_block_sums;
    f.done = h->d_done;
    f.loss = h->d_loss;
    f.epoch = h->d_epoch;
    f.compute_loss = h->opt.compute_loss;
    if (ev) cudaEventRecord(ev[4 * s.batches], st);
    err = launch_bf16_flush(f, st);
  }
  return err;
}

// Buffers of the BF16 form for minibatch size B and ns negatives.
int ensure_bf16_buffers(de_handle *h, int ns, bool *moved) {
  const Schedule &s = h->sched;
  const int kpad = std::max(64, (ns + 63) / 64 * 64);
  if (kpad > 1024) return fail(h, DE_ERR_UNSUPPORTED, "the BF16 form takes at most 1024 negatives per minibatch");
  bool m = false, near_moved = false;
  int rc = DE_OK;
  if ((rc = grow(h, &h->d_abuf, &h->abuf_cap, size_t(s.batch) * h->dim, &m)) ||
      (rc = grow(h, &h->d_rbuf, &h->rbuf_cap, size_t(s.batch) * h->dim, &m)) ||
      (rc = grow(h, &h->d_near_bits, &h->near_cap, size_t(s.batch) * 32, &near_moved)))
    return rc;
  if (near_moved) {
    DE_CUDA(h, cudaMemsetAsync(h->d_near_bits, 0, h->near_cap * sizeof(uint32_t), h->stream));
    m = true;
  }
  if (size_t(kpad) > h->kpad_cap || !h->d_nn) {
    for (void *p : {static_cast<void *>(h->d_nn), static_cast<void *>(h->d_nid), static_cast<void *>(h->d_nb)})
      if (p) dev_free(h, p);
    h->d_nn = nullptr; h->d_nid = nullptr; h->d_nb = nullptr;
    DE_CUDA(h, dev_alloc(h, reinterpret_cast<void **>(&h->d_nn), kpad * sizeof(float)));
    DE_CUDA(h, dev_alloc(h, reinterpret_cast<void **>(&h->d_nid), kpad * sizeof(int32_t)));
    DE_CUDA(h, dev_alloc(h, reinterpret_cast<void **>(&h->d_nb), size_t(kpad) * h->dim * sizeof(__nv_bfloat16)));
    h->kpad_cap = kpad;
    m = true;
  }
  if (kpad != h->kpad || m) {
    h->kpad = kpad;
    if ((rc = encode_map(h, &h->map_x, h->d_xb, uint64_t(h->n), uint64_t(h->dim), 128)) ||
        (rc = encode_map(h, &h->map_n, h->d_nb, uint64_t(kpad), uint64_t(h->dim), 64)))
      return rc;
    m = true;
  }
  if (m) *moved = true;
  return DE_OK;
}

// Enqueues one epoch of the FP32 plain form on st.  ev (nullable): one event
// before each minibatch launch and one before the flush (the events also stop
// launches from overlapping).
cudaError_t enqueue_epoch_plain(de_handle *h, int ns, cudaStream_t st, cudaEvent_t *ev) {
  const Schedule &s = h->sched;
  cudaError_t err = cudaSuccess;
  for (int j = 0; j < s.batches && err == cudaSuccess; ++j) {
    PlainBatchArgs a{};
    a.X = h->d_x;
    const size_t slice = size_t(s.batch) * h->dim;
    a.S_cur = h->d_stage + slice * (j % 3);
    a.S_prev = h->d_stage + slice * ((j + 2) % 3);
    a.S_prev2 = h->d_stage + slice * ((j + 1) % 3);
    a.rowptr = h->d_rowptr;
    a.col = h->d_col;
    a.items = s.d_items + s.item_off[j];
    a.n_items = int32_t(s.item_off[j + 1] - s.item_off[j]);
    a.base = int32_t(int64_t(j) * s.batch);
    a.rows = int32_t(std::min<int64_t>(s.batch, h->n - a.base));
    a.prev_base = j > 0 ? int32_t(int64_t(j - 1) * s.batch) : 0;
    a.prev_rows = j > 0 ? s.batch : 0;
    a.prev2_base = j > 1 ? int32_t(int64_t(j - 2) * s.batch) : 0;
    a.prev2_rows = j > 1 ? s.batch : 0;
    a.batch_id = j;
    a.batches = s.batches;
    a.last_batch_size = s.last_batch_size;
    a.n = int32_t(h->n);
    a.quirks = h->opt.ref_quirks;
    a.skip_last = h->opt.ref_quirks && !h->keep_last_edges;
    a.compute_loss = h->opt.compute_loss;
    a.bound = float(h->opt.max_bound);
    a.negs = h->d_negs;
    a.ns = ns;
    a.lr = h->d_lr;
    a.P = h->d_parts;
    a.counters = h->d_counters;
    a.loss_partial = h->d_loss_partial;
    a.loss_off = s.item_off[j];
    a.epoch = h->d_epoch;
    a.stage_negs = h->opt.stage_negatives && ns > 0 && ns <= kStageNegMax;
    a.err = h->d_err;
    const int grid = int(s.cta_off[j + 1] - s.cta_off[j]);
    if (ev) cudaEventRecord(ev[j], st);
    err = launch_plain_batch(h->dim, a, grid, h->opt.pdl && j > 0 && !ev, st);
  }
  if (err == cudaSuccess) {
    FlushArgs f{};
    f.X = h->d_x;
    f.S_last = h->d_stage + size_t(s.batch) * h->dim * ((s.batches - 1) % 3);
    f.last_base = int32_t(int64_t(s.batches - 1) * s.batch);
    f.last_rows = s.last_batch_size;
    f.loss_partial = h->d_loss_partial;
    f.n_partials = s.n_items;
    f.block_sums = h->d_block_sums;
    f.done = h->d_done;
    f.loss = h->d_loss;
    f.epoch = h->d_epoch;
    f.compute_loss = h->opt.compute_loss;
    if (ev) cudaEventRecord(ev[s.batches], st);
    err = launch_flush(h->dim, f, h->opt.pdl != 0 && !ev, st);
  }
  return err;
}

// Launches of one epoch and the kind of each: 0 minibatch kernel (FP32) or
// attractive kernel (BF16), 1 repulsive GEMM kernel, 2 exact-row kernel, 3 flush.
std::vector<int> epoch_launch_kinds(const de_handle *h) {
  std::vector<int> k;
  if (h->opt.precision == DE_PRECISION_BF16)
    for (int j = 0; j < h->sched.batches; ++j) k.insert(k.end(), {4, 0, 1, 2});
  else
    k.assign(h->sched.batches, 0);
  k.push_back(3);
  return k;
}

cudaError_t enqueue_epoch(de_handle *h, int ns, cudaStream_t st, cudaEvent_t *ev) {
  return h->opt.precision == DE_PRECISION_BF16 ? enqueue_epoch_bf16(h, ns, st, ev)
                                               : enqueue_epoch_plain(h, ns, st, ev);
}

int capture_epoch(de_handle *h, int ns) {
  const Schedule &s = h->sched;
  cudaStream_t st = h->stream;
  DE_CUDA(h, cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
  const cudaError_t err = enqueue_epoch(h, ns, st, nullptr);
  cudaGraph_t g = nullptr;
  cudaError_t e2 = cudaStreamEndCapture(st, &g);
  if (err != cudaSuccess) {
    if (g) cudaGraphDestroy(g);
    return cuda_fail(h, err, "kernel launch during capture");
  }
  if (e2 != cudaSuccess) return cuda_fail(h, e2, "cudaStreamEndCapture");
  cudaError_t e3 = cudaGraphInstantiate(&h->graph, g, 0);
  cudaGraphDestroy(g);
  if (e3 != cudaSuccess) {
    h->graph = nullptr;
    return cuda_fail(h, e3, "cudaGraphInstantiate");
  }
  h->graph_batch = s.batch;
  h->graph_ns = ns;
  return DE_OK;
}

// A kernel whose bounded wait gave up records it in d_err; report and re-arm.
int check_device_error(de_handle *h) {
  int32_t e = 0;
  DE_CUDA(h, cudaMemcpyAsync(&e, h->d_err, sizeof(int32_t), cudaMemcpyDeviceToHost, h->stream));
  DE_CUDA(h, cudaStreamSynchronize(h->stream));
  if (e) {
    DE_CUDA(h, cudaMemsetAsync(h->d_err, 0, sizeof(int32_t), h->stream));
    if (h->d_near_bits) DE_CUDA(h, cudaMemsetAsync(h->d_near_bits, 0, h->near_cap * sizeof(uint32_t), h->stream));
    DE_CUDA(h, cudaStreamSynchronize(h->stream));
    return fail(h, DE_ERR_CUDA, "a device-side wait timed out; results of this call are not valid");
  }
  return DE_OK;
}

int check_csr(de_handle *h, int64_t n, const int64_t *rowptr, const int64_t *col, int64_t nnz) {
  if (rowptr[0] != 0 || rowptr[n] != nnz) return fail(h, DE_ERR_INVALID, "rowptr must start at 0 and end at nnz");
  for (int64_t i = 0; i < n; ++i)
    if (rowptr[i + 1] < rowptr[i]) return fail(h, DE_ERR_INVALID, "rowptr must be non-decreasing");
  for (int64_t e = 0; e < nnz; ++e)
    if (col[e] < 0 || col[e] >= n) return fail(h, DE_ERR_INVALID, "column index out of range");
  return DE_OK;
}

}  // namespace

extern "C" {

void de_default_options(de_options *o) {
  std::memset(o, 0, sizeof(*o));
  o->precision = DE_PRECISION_FP32;
  o->ref_quirks = 1;
  o->compute_loss = 1;
  o->device = 0;
  o->stream = nullptr;
  o->max_bound = 5.0;
  o->edge_cap = 0;
  o->pdl = 1;
}

int de_create(int64_t n, const int64_t *rowptr, const int64_t *col, int64_t nnz, int32_t dim,
              const de_options *opts, de_handle **out) {
  return de::create_handle(n, rowptr, col, nnz, dim, opts, nullptr, out);
}

}  // extern "C"

namespace de {

int create_handle(int64_t n, const int64_t *rowptr, const int64_t *col, int64_t nnz, int32_t dim,
                  const de_options *opts, const MemHooks *hooks, de_handle **out) {
  if (!out) return fail(nullptr, DE_ERR_INVALID, "out is NULL");
  *out = nullptr;
  if (n <= 0 || nnz < 0 || !rowptr || (nnz > 0 && !col)) return fail(nullptr, DE_ERR_INVALID, "bad graph arguments");
  if (dim != 32 && dim != 64 && dim != 128 && dim != 256)
    return fail(nullptr, DE_ERR_INVALID, "dim must be 32, 64, 128 or 256");
  if (n >= (int64_t(1) << 31) - 1 || nnz >= (int64_t(1) << 31) - 1)
    return fail(nullptr, DE_ERR_UNSUPPORTED, "n and nnz must be below 2^31 - 1");
  auto h = std::make_unique<de_handle>();
  if (opts) h->opt = *opts; else de_default_options(&h->opt);
  if (hooks) h->hooks = *hooks;
  if (h->opt.precision != DE_PRECISION_FP32 && h->opt.precision != DE_PRECISION_BF16)
    return fail(nullptr, DE_ERR_INVALID, "unknown precision");
  if (h->opt.precision == DE_PRECISION_BF16 && dim < 64)
    return fail(nullptr, DE_ERR_UNSUPPORTED, "the BF16 form needs dim 64, 128 or 256");
  if (!(h->opt.max_bound > 0)) return fail(nullptr, DE_ERR_INVALID, "max_bound must be positive");
  if (int rc = check_csr(h.get(), n, rowptr, col, nnz)) return fail(nullptr, rc, h->err);
  h->n = n;
  h->nnz = nnz;
  h->dim = dim;
  h->device = h->opt.device;
  h->rowptr.assign(rowptr, rowptr + n + 1);
  for (int64_t e = 0; e < nnz; ++e) h->edges_into_last += (col[e] == n - 1);

  auto bail = [&](int rc) {
    std::string m = h->err;
    de_destroy(h.release());
    return fail(nullptr, rc, m);
  };
  cudaError_t e = cudaSetDevice(h->device);
  if (e != cudaSuccess) return bail(cuda_fail(h.get(), e, "cudaSetDevice"));
  if (h->opt.stream) {
    h->stream = static_cast<cudaStream_t>(h->opt.stream);
  } else {
    e = cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) return bail(cuda_fail(h.get(), e, "cudaStreamCreate"));
    h->own_stream = true;
  }
  std::vector<int32_t> rp32(rowptr, rowptr + n + 1), col32(col, col + nnz);
  if ((e = dev_alloc(h, reinterpret_cast<void **>(&h->d_rowptr), (n + 1) * sizeof(int32_t))) != cudaSuccess ||
      (e = dev_alloc(h, reinterpret_cast<void **>(&h->d_col), std::max<int64_t>(nnz, 1) * sizeof(int32_t))) != cudaSuccess ||
      (e = dev_alloc(h, reinterpret_cast<void **>(&h->d_x), size_t(n) * dim * sizeof(float))) != cudaSuccess ||
      (e = dev_alloc(h, reinterpret_cast<void **>(&h->d_epoch), 2 * sizeof(int32_t))) != cudaSuccess ||
      (e = dev_alloc(h, reinterpret_cast<void **>(&h->d_block_sums), kFlushBlocks * sizeof(double))) != cudaSuccess ||
      (e = dev_alloc(h, reinterpret_cast<void **>(&h->d_done), sizeof(int32_t))) != cudaSuccess ||
      (e = dev_alloc(h, reinterpret_cast<void **>(&h->d_err), sizeof(int32_t))) != cudaSuccess ||
      (e = host_alloc(h, reinterpret_cast<void **>(&h->h_epoch), 2 * sizeof(int32_t))) != cudaSuccess ||
      (e = cudaEventCreateWithFlags(&h->upload_done, cudaEventDisableTiming)) != cudaSuccess)
    return bail(cuda_fail(h.get(), e, "allocation"));
  // uploads and clears on the handle's stream: its kernels do not wait for the
  // legacy stream, and a synchronous cudaMemcpy from pageable memory may return
  // before its DMA has landed
  cudaStream_t st = h->stream;
  if ((e = cudaMemcpyAsync(h->d_rowptr, rp32.data(), (n + 1) * sizeof(int32_t), cudaMemcpyHostToDevice, st)) != cudaSuccess ||
      (nnz > 0 && (e = cudaMemcpyAsync(h->d_col, col32.data(), nnz * sizeof(int32_t), cudaMemcpyHostToDevice, st)) != cudaSuccess) ||
      (e = cudaMemsetAsync(h->d_x, 0, size_t(n) * dim * sizeof(float), st)) != cudaSuccess ||
      (e = cudaMemsetAsync(h->d_done, 0, sizeof(int32_t), st)) != cudaSuccess ||
      (e = cudaMemsetAsync(h->d_err, 0, sizeof(int32_t), st)) != cudaSuccess ||
      (e = cudaStreamSynchronize(st)) != cudaSuccess)
    return bail(cuda_fail(h.get(), e, "upload"));
  if (h->opt.precision == DE_PRECISION_BF16) {
    if ((e = dev_alloc(h, reinterpret_cast<void **>(&h->d_xb), size_t(n) * dim * sizeof(__nv_bfloat16))) != cudaSuccess ||
        (e = dev_alloc(h, reinterpret_cast<void **>(&h->d_loss_row), size_t(n) * sizeof(double))) != cudaSuccess ||
        (e = cudaMemsetAsync(h->d_xb, 0, size_t(n) * dim * sizeof(__nv_bfloat16), h->stream)) != cudaSuccess ||
        (e = cudaMemsetAsync(h->d_loss_row, 0, size_t(n) * sizeof(double), h->stream)) != cudaSuccess ||
        (e = cudaStreamSynchronize(h->stream)) != cudaSuccess ||
        (e = bf16_prepare(dim)) != cudaSuccess ||
        (e = cudaStreamCreateWithFlags(&h->stream2, cudaStreamNonBlocking)) != cudaSuccess ||
        (e = cudaEventCreateWithFlags(&h->ev_fork, cudaEventDisableTiming)) != cudaSuccess ||
        (e = cudaEventCreateWithFlags(&h->ev_join, cudaEventDisableTiming)) != cudaSuccess)
      return bail(cuda_fail(h.get(), e, "BF16 form set-up"));
  }
  *out = h.release();
  return DE_OK;
}

int copy_loss(de_handle *h, double *out, int32_t epochs) {
  if (!h || !out || epochs <= 0) return DE_ERR_INVALID;
  if (size_t(epochs) > h->loss_cap || !h->d_loss) return fail(h, DE_ERR_STATE, "no loss of that many epochs");
  DE_CUDA(h, cudaMemcpyAsync(out, h->d_loss, epochs * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
  DE_CUDA(h, cudaStreamSynchronize(h->stream));
  return check_device_error(h);
}

}  // namespace de

extern "C" {

int de_destroy(de_handle *h) {
  if (!h) return DE_OK;
  cudaSetDevice(h->device);
  if (h->stream) cudaStreamSynchronize(h->stream);
  drop_graph(h);
  dev_free(h, h->d_rowptr);
  dev_free(h, h->d_col);
  dev_free(h, h->d_x);
  dev_free(h, h->sched.d_items);
  dev_free(h, h->d_stage);
  dev_free(h, h->d_y);
  dev_free(h, h->d_sx);
  dev_free(h, h->d_coll);
  dev_free(h, h->d_present);
  dev_free(h, h->d_spmm_off);
  dev_free(h, h->d_parts);
  dev_free(h, h->d_counters);
  dev_free(h, h->d_loss_partial);
  dev_free(h, h->d_block_sums);
  dev_free(h, h->d_done);
  dev_free(h, h->d_err);
  dev_free(h, h->d_xb);
  dev_free(h, h->d_abuf);
  dev_free(h, h->d_rbuf);
  dev_free(h, h->d_nb);
  dev_free(h, h->d_nn);
  dev_free(h, h->d_nid);
  dev_free(h, h->d_near_bits);
  dev_free(h, h->d_loss_row);
  dev_free(h, h->d_epoch);
  dev_free(h, h->d_loss);
  dev_free(h, h->d_negs);
  dev_free(h, h->d_lr);
  dev_free(h, h->d_stage64);
  if (h->h_negs) host_free(h, h->h_negs);
  if (h->h_lr) host_free(h, h->h_lr);
  if (h->h_loss) host_free(h, h->h_loss);
  if (h->h_epoch) host_free(h, h->h_epoch);
  if (h->upload_done) cudaEventDestroy(h->upload_done);
  if (h->stream2) {
    cudaStreamSynchronize(h->stream2);
    cudaStreamDestroy(h->stream2);
  }
  if (h->ev_fork) cudaEventDestroy(h->ev_fork);
  if (h->ev_join) cudaEventDestroy(h->ev_join);
  if (h->own_stream && h->stream) cudaStreamDestroy(h->stream);
  delete h;
  return DE_OK;
}

// Device address of host memory the GPU can read and write in place (pinned and
// mapped, e.g. from cudaHostAlloc), or nullptr.
static void *mapped_host(const void *p) {
  cudaPointerAttributes at{};
  if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  return at.type == cudaMemoryTypeHost ? at.devicePointer : nullptr;
}

// A pointer kernels can read: device memory as it is, pinned host memory through
// its device alias; nullptr for pageable host memory.
static const double *device_view(const double *p) {
  cudaPointerAttributes at{};
  if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  if (at.type == cudaMemoryTypeDevice || at.type == cudaMemoryTypeManaged) return p;
  if (at.type == cudaMemoryTypeHost) return static_cast<const double *>(at.devicePointer);
  return nullptr;
}

static int copy_embeddings_f64(de_handle *h, double *host, bool to_device, float *dev = nullptr) {
  if (!h || !host) return fail(h, DE_ERR_INVALID, "NULL argument");
  DE_CUDA(h, cudaSetDevice(h->device));
  if (!dev) dev = h->d_x;
  const int64_t total = h->n * h->dim;
  if (double *mapped = static_cast<double *>(mapped_host(host))) {
    // pinned host memory: the conversion kernel reads or writes it in place, one
    // pass over the link instead of a copy to a staging buffer and a second pass
    if (to_device) {
      DE_CUDA(h, launch_f64_to_f32(mapped, dev, total, h->stream));
      if (h->d_xb) DE_CUDA(h, launch_f32_to_bf16(dev, h->d_xb, total, h->stream));
    } else {
      DE_CUDA(h, launch_f32_to_f64(dev, mapped, total, h->stream));
    }
    DE_CUDA(h, cudaStreamSynchronize(h->stream));
    return DE_OK;
  }
  const int64_t chunk = std::min<int64_t>(total, int64_t(8) << 20);  // 64 MiB of FP64
  if (int rc = grow(h, &h->d_stage64, &h->stage64_cap, size_t(chunk))) return rc;
  for (int64_t off = 0; off < total; off += chunk) {
    const int64_t cnt = std::min(chunk, total - off);
    if (to_device) {
      DE_CUDA(h, cudaMemcpyAsync(h->d_stage64, host + off, cnt * sizeof(double), cudaMemcpyHostToDevice, h->stream));
      DE_CUDA(h, launch_f64_to_f32(h->d_stage64, dev + off, cnt, h->stream));
      if (h->d_xb) DE_CUDA(h, launch_f32_to_bf16(dev + off, h->d_xb + off, cnt, h->stream));
    } else {
      DE_CUDA(h, launch_f32_to_f64(dev + off, h->d_stage64, cnt, h->stream));
      DE_CUDA(h, cudaMemcpyAsync(host + off, h->d_stage64, cnt * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    }
  }
  DE_CUDA(h, cudaStreamSynchronize(h->stream));
  return DE_OK;
}

int de_set_embeddings(de_handle *h, const double *x) { return copy_embeddings_f64(h, const_cast<double *>(x), true); }
int de_get_embeddings(de_handle *h, double *x) { return copy_embeddings_f64(h, x, false); }

int de_set_embeddings_f32(de_handle *h, const float *x, int32_t on_device) {
  if (!h || !x) return fail(h, DE_ERR_INVALID, "NULL argument");
  DE_CUDA(h, cudaSetDevice(h->device));
  DE_CUDA(h, cudaMemcpyAsync(h->d_x, x, size_t(h->n) * h->dim * sizeof(float),
                             on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, h->stream));
  if (h->d_xb) DE_CUDA(h, launch_f32_to_bf16(h->d_x, h->d_xb, h->n * h->dim, h->stream));
  DE_CUDA(h, cudaStreamSynchronize(h->stream));
  return DE_OK;
}

int de_get_embeddings_f32(de_handle *h, float *x, int32_t on_device) {
  if (!h || !x) return fail(h, DE_ERR_INVALID, "NULL argument");
  DE_CUDA(h, cudaSetDevice(h->device));
  DE_CUDA(h, cudaMemcpyAsync(x, h->d_x, size_t(h->n) * h->dim * sizeof(float),
                             on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, h->stream));
  DE_CUDA(h, cudaStreamSynchronize(h->stream));
  return DE_OK;
}

int de_run(de_handle *h, int32_t epochs, int32_t batch_size, int32_t ns, const double *lr_per_epoch,
           double *loss_per_epoch) {
  return de_run_from(h, 0, epochs, batch_size, ns, lr_per_epoch, loss_per_epoch);
}

// Schedule, buffers and per-call uploads (negatives, learning rates, epoch
// counter) for `epochs` epochs starting at first_epoch; arguments already checked.
static int prepare_run(de_handle *h, int32_t first_epoch, int32_t epochs, int32_t batch_size, int32_t ns,
                       const double *lr_per_epoch) {
  DE_CUDA(h, cudaSetDevice(h->device));
  if (int rc = ensure_schedule(h, batch_size)) return rc;
  const Schedule &s = h->sched;
  bool moved = false;
  int rc = DE_OK;
  const bool bf16 = h->opt.precision == DE_PRECISION_BF16;
  if (!bf16 && (rc = grow(h, &h->d_stage, &h->stage_cap, size_t(3) * s.batch * h->dim, &moved)) != DE_OK) return rc;
  if (bf16 && (rc = ensure_bf16_buffers(h, ns, &moved)) != DE_OK) return rc;
  bool counters_moved = false;
  if ((rc = grow(h, &h->d_parts, &h->parts_cap, size_t(std::max(s.max_parts, 1)) * h->dim, &moved)) ||
      (rc = grow(h, &h->d_counters, &h->counters_cap, size_t(std::max(s.max_split, 1)), &counters_moved)) ||
      (rc = grow(h, &h->d_loss_partial, &h->loss_partial_cap, size_t(s.n_items), &moved)))
    return rc;
  if (counters_moved) {
    DE_CUDA(h, cudaMemsetAsync(h->d_counters, 0, h->counters_cap * sizeof(int32_t), h->stream));
    moved = true;
  }
  const size_t ecap = std::max<size_t>(size_t(epochs), 64);
  if (size_t(epochs) > h->loss_cap || !h->d_loss)
    if ((rc = grow(h, &h->d_loss, &h->loss_cap, ecap, &moved))) return rc;
  if (size_t(epochs) > h->lr_cap || !h->d_lr)
    if ((rc = grow(h, &h->d_lr, &h->lr_cap, ecap, &moved))) return rc;
  const size_t nneg = size_t(epochs) * s.batches * std::max(ns, 1);
  if (nneg > h->negs_cap || !h->d_negs)
    if ((rc = grow(h, &h->d_negs, &h->negs_cap, std::max(nneg, ecap * s.batches * std::max(ns, 1)), &moved)))
      return rc;
  if (moved) drop_graph(h);

  // Host side of the upload: wait until the previous call's copies have read
  // the pinned buffers before overwriting them.
  DE_CUDA(h, cudaEventSynchronize(h->upload_done));
  if ((rc = grow_pinned(h, &h->h_negs, &h->h_negs_cap, nneg)) ||
      (rc = grow_pinned(h, &h->h_lr, &h->h_lr_cap, size_t(epochs))) ||
      (rc = grow_pinned(h, &h->h_loss, &h->h_loss_cap, size_t(epochs))))
    return rc;
  // the draws of minibatch j of epoch i at (i * batches + j) * ns; many runs'
  // worth (e.g. 10 epochs x 512 minibatches x 1024 draws) on host threads
  const int64_t batches = s.batches;
  parallel_indices(int64_t(epochs) * batches, std::max(ns, 1), [&](int64_t q) {
    const int i = int(q / batches), j = int(q % batches);
    draw_negatives(h->n, first_epoch + i + j, ns, h->h_negs + size_t(q) * ns);
  });
  for (int i = 0; i < epochs; ++i) h->h_lr[i] = float(lr_per_epoch[i]);
  DE_CUDA(h, cudaMemcpyAsync(h->d_negs, h->h_negs, nneg * sizeof(int32_t), cudaMemcpyHostToDevice, h->stream));
  DE_CUDA(h, cudaMemcpyAsync(h->d_lr, h->h_lr, epochs * sizeof(float), cudaMemcpyHostToDevice, h->stream));
  h->h_epoch[0] = 0;
  h->h_epoch[1] = first_epoch;
  DE_CUDA(h, cudaMemcpyAsync(h->d_epoch, h->h_epoch, 2 * sizeof(int32_t), cudaMemcpyHostToDevice, h->stream));
  // after every copy from the pinned buffers: the next call waits on it before
  // writing them again
  DE_CUDA(h, cudaEventRecord(h->upload_done, h->stream));
  return DE_OK;
}

int de_run_from(de_handle *h, int32_t first_epoch, int32_t epochs, int32_t batch_size, int32_t ns,
                const double *lr_per_epoch, double *loss_per_epoch) {
  if (!h) return DE_ERR_INVALID;
  if (first_epoch < 0 || epochs < 0 || batch_size <= 0 || ns < 0)
    return fail(h, DE_ERR_INVALID, "first_epoch >= 0, epochs >= 0, batch_size > 0, ns >= 0");
  if (epochs > 0 && !lr_per_epoch) return fail(h, DE_ERR_INVALID, "lr_per_epoch is NULL");
  if (epochs == 0) return DE_OK;
  int rc = prepare_run(h, first_epoch, epochs, batch_size, ns, lr_per_epoch);
  if (rc) return rc;
  const Schedule &s = h->sched;
  if (!h->graph || h->graph_batch != s.batch || h->graph_ns != ns) {
    drop_graph(h);
    if ((rc = capture_epoch(h, ns))) return rc;
  }
  for (int i = 0; i < epochs; ++i) DE_CUDA(h, cudaGraphLaunch(h->graph, h->stream));
  if (loss_per_epoch) {
    DE_CUDA(h, cudaMemcpyAsync(h->h_loss, h->d_loss, epochs * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    DE_CUDA(h, cudaStreamSynchronize(h->stream));
    std::memcpy(loss_per_epoch, h->h_loss, epochs * sizeof(double));
    if ((rc = check_device_error(h))) return rc;
  }
  DE_CUDA(h, cudaGetLastError());
  return DE_OK;
}

// Work list, partial slots, counters and output rows of a one-launch pass over
// every minibatch (the SpMM step and the sparse embedding's attractive pass).
static int spmm_layout(de_handle *h, int32_t batch_size) {
  if (batch_size <= 0) return fail(h, DE_ERR_INVALID, "batch_size > 0");
  DE_CUDA(h, cudaSetDevice(h->device));
  if (int rc = ensure_schedule(h, batch_size)) return rc;
  const Schedule &s = h->sched;
  // the minibatches do not depend on one another: every item in one launch, each
  // minibatch with its own partial slots and counters
  if (h->spmm_batch != s.batch || h->spmm_cap != s.edge_cap) {
    std::vector<int32_t> off(2 * size_t(s.batches) + 2, 0);
    for (int j = 0; j < s.batches; ++j) {
      off[j + 1] = off[j] + s.n_parts[j];
      off[s.batches + 1 + j + 1] = off[s.batches + 1 + j] + s.n_split[j];
    }
    h->spmm_parts = off[s.batches];
    h->spmm_split = off[2 * size_t(s.batches) + 1];
    if (h->d_spmm_off) dev_free(h, h->d_spmm_off);
    h->d_spmm_off = nullptr;
    DE_CUDA(h, dev_alloc(h, reinterpret_cast<void **>(&h->d_spmm_off), off.size() * sizeof(int32_t)));
    DE_CUDA(h, cudaMemcpyAsync(h->d_spmm_off, off.data(), off.size() * sizeof(int32_t), cudaMemcpyHostToDevice,
                               h->stream));
    DE_CUDA(h, cudaStreamSynchronize(h->stream));
    h->spmm_batch = s.batch;
    h->spmm_cap = s.edge_cap;
  }
  bool moved = false, counters_moved = false;
  int rc = DE_OK;
  if ((rc = grow(h, &h->d_parts, &h->parts_cap, size_t(std::max<int64_t>(h->spmm_parts, 1)) * h->dim, &moved)) ||
      (rc = grow(h, &h->d_counters, &h->counters_cap, size_t(std::max<int64_t>(h->spmm_split, 1)), &counters_moved)))
    return rc;
  if (counters_moved) DE_CUDA(h, cudaMemsetAsync(h->d_counters, 0, h->counters_cap * sizeof(int32_t), h->stream));
  if (moved || counters_moved) drop_graph(h);
  if (!h->d_y) DE_CUDA(h, dev_alloc(h, reinterpret_cast<void **>(&h->d_y), size_t(h->n) * h->dim * sizeof(float)));
  return DE_OK;
}

// SpMMAlgo::algo_spmm(1, batch_size, lr) at one rank (cpp/algo/spmm.hpp:54-159):
// the rows of each minibatch into d_y from the current embedding.
static int spmm_run(de_handle *h, int32_t batch_size, double lr) {
  if (int rc = spmm_layout(h, batch_size)) return rc;
  const Schedule &s = h->sched;
  SpmmArgs a{};
  a.X = h->d_x;
  a.Y = h->d_y;
  a.col = h->d_col;
  a.items = s.d_items;
  a.n_items = s.n_items;
  a.batch = s.batch;
  a.slot_off = h->d_spmm_off;
  a.counter_off = h->d_spmm_off + s.batches + 1;
  a.skip = h->opt.ref_quirks ? int32_t(h->n - 1) : -1;
  a.lr = float(lr);
  a.P = h->d_parts;
  a.counters = h->d_counters;
  DE_CUDA(h, launch_spmm(h->dim, a, h->stream));
  return DE_OK;
}

int de_spmm(de_handle *h, int32_t batch_size, double lr, double *y) {
  if (!h || !y) return DE_ERR_INVALID;
  if (int rc = spmm_run(h, batch_size, lr)) return rc;
  return copy_embeddings_f64(h, y, false, h->d_y);
}

int de_spmm_f32(de_handle *h, int32_t batch_size, float lr, float *y, int32_t on_device) {
  if (!h || !y) return DE_ERR_INVALID;
  if (int rc = spmm_run(h, batch_size, lr)) return rc;
  DE_CUDA(h, cudaMemcpyAsync(y, h->d_y, size_t(h->n) * h->dim * sizeof(float),
                             on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, h->stream));
  DE_CUDA(h, cudaStreamSynchronize(h->stream));
  return DE_OK;
}

// ---------------------------------------------------------------- sparse embedding
// SparseEmbedding::algo_sparse_embedding at one rank (cpp/algo/sparse_embedding.hpp:
// 78-194).  merge = 0: the one-rank branch, whose attractive updates go into the
// batch collector and are never merged (the values change only by the top-k
// pruning after the first iteration); merge = 1: per minibatch the repulsive
// pass, the attractive pass and the merge of the collector into the rows (the
// steps of the multi-rank branch that touch the local partition), which is the
// FP32 plain minibatch step on the mirror with edges into n - 1 kept.

int de_sparse_set(de_handle *h, const double *x) {
  if (!h || !x) return DE_ERR_INVALID;
  if (h->opt.precision != DE_PRECISION_FP32)
    return fail(h, DE_ERR_UNSUPPORTED, "the sparse embedding runs on an FP32 handle");
  if (h->dim != 32 && h->dim != 64 && h->dim != 128 && h->dim != 256)
    return fail(h, DE_ERR_UNSUPPORTED, "the sparse embedding supports dim 32, 64, 128 or 256");
  DE_CUDA(h, cudaSetDevice(h->device));
  const size_t count = size_t(h->n) * h->dim;
  if (!h->d_sx) DE_CUDA(h, dev_alloc(h, reinterpret_cast<void **>(&h->d_sx), count * sizeof(double)));
  if (!h->d_present) DE_CUDA(h, dev_alloc(h, reinterpret_cast<void **>(&h->d_present), sizeof(unsigned long long)));
  // Device memory or pinned host memory: one kernel reads it once and writes
  // the rows and their mirror; pageable host memory: a copy, then the mirror.
  const double *src = device_view(x);
  if (src && (reinterpret_cast<uintptr_t>(src) & 15) == 0) {
    DE_CUDA(h, launch_sparse_load(src, h->d_sx, h->d_x, int64_t(count), h->stream));
  } else {
    DE_CUDA(h, cudaMemcpyAsync(h->d_sx, x, count * sizeof(double), cudaMemcpyDefault, h->stream));
    DE_CUDA(h, launch_sparse_mirror(h->d_sx, h->d_x, int64_t(count), h->stream));
  }
  h->sparse_in_mirror = false;
  return DE_OK;
}

int de_sparse_run(de_handle *h, int32_t iterations, int32_t batch_size, int32_t ns, double lr, double density,
                  int32_t merge) {
  if (!h) return DE_ERR_INVALID;
  if (!h->d_sx) return fail(h, DE_ERR_INVALID, "no sparse embedding rows: call de_sparse_set first");
  if (iterations < 0 || batch_size <= 0 || ns < 0 || !std::isfinite(density))
    return fail(h, DE_ERR_INVALID, "iterations >= 0, batch_size > 0, ns >= 0, finite density");
  DE_CUDA(h, cudaSetDevice(h->device));
  // expected_nnz_per_row = static_cast<int>(embedding_dim * density) (line 86)
  const double kd = double(h->dim) * density;
  const int32_t keep = int32_t(std::max(-1.0, std::min(kd, double(h->dim) + 1.0)));
  const int64_t count = h->n * int64_t(h->dim);
  int rc = DE_OK;
  // the batch collector starts at zero (initialize_batch_collector, line 95)
  bool moved = false;
  if ((rc = grow(h, &h->d_coll, &h->coll_cap, size_t(batch_size) * h->dim, &moved))) return rc;
  DE_CUDA(h, cudaMemsetAsync(h->d_coll, 0, size_t(batch_size) * h->dim * sizeof(double), h->stream));
  h->sparse_batch = batch_size;
  h->sparse_in_mirror = false;
  if (iterations == 0) return DE_OK;
  if (!merge) {
    if ((rc = spmm_layout(h, batch_size))) return rc;
    const Schedule &s = h->sched;
    SpmmArgs a{};
    a.X = h->d_x;
    a.Y = h->d_y;
    a.col = h->d_col;
    a.items = s.d_items;
    a.n_items = s.n_items;
    a.batch = s.batch;
    a.slot_off = h->d_spmm_off;
    a.counter_off = h->d_spmm_off + s.batches + 1;
    a.skip = -1;
    a.lr = float(lr);
    a.P = h->d_parts;
    a.counters = h->d_counters;
    a.bound = float(h->opt.max_bound);
    // The rows change only by the pruning, so only the check after the first
    // iteration can prune: after it floor(present / n) <= k, and the rows, hence
    // the count, stay as they are.  The later checks are left out.
    for (int it = 0; it < iterations; ++it) {
      DE_CUDA(h, launch_sparse_attract(h->dim, a, h->stream));
      DE_CUDA(h, launch_sparse_collect(h->d_y, h->d_coll, h->n, batch_size, h->dim, h->stream));
      if (it == 0 && iterations > 1) {
        DE_CUDA(h, cudaMemsetAsync(h->d_present, 0, sizeof(unsigned long long), h->stream));
        DE_CUDA(h, launch_sparse_count(h->d_sx, count, h->d_present, h->stream));
        DE_CUDA(h, launch_sparse_prune_f64(h->dim, h->d_sx, h->d_x, h->n, keep, h->d_present, h->stream));
      } else if (it == iterations - 1) {
        DE_CUDA(h, launch_sparse_finalize(h->d_sx, count, h->stream));
      }
    }
    return DE_OK;
  }
  // merge = 1: every entry of a row is present after its minibatch's merge
  // (merge_batch_collector writes all of them, cpp/core/sparse_mat.hpp:385-400),
  // so at the end of an iteration floor(present / n) = dim and the rows are
  // pruned whenever keep < dim; the pruned entries read as 0 in the mirror.
  h->keep_last_edges = true;
  drop_graph(h);
  for (int it = 0; it < iterations && rc == DE_OK; ++it) {
    rc = de_run_from(h, it, 1, batch_size, ns, &lr, nullptr);
    if (rc == DE_OK && it < iterations - 1 && keep < h->dim) {
      const cudaError_t e = launch_sparse_prune_f32(h->dim, h->d_x, h->n, keep, h->stream);
      if (e != cudaSuccess) rc = cuda_fail(h, e, "launch_sparse_prune_f32");
    }
  }
  drop_graph(h);
  h->keep_last_edges = false;
  if (rc) return rc;
  h->sparse_in_mirror = true;
  return DE_OK;
}

int de_sparse_get(de_handle *h, double *x, double *coll) {
  if (!h || (!x && !coll)) return DE_ERR_INVALID;
  if (!h->d_sx) return fail(h, DE_ERR_INVALID, "no sparse embedding rows: call de_sparse_set first");
  DE_CUDA(h, cudaSetDevice(h->device));
  const size_t count = size_t(h->n) * h->dim;
  if (h->sparse_in_mirror) {
    DE_CUDA(h, launch_f32_to_f64(h->d_x, h->d_sx, int64_t(count), h->stream));
    h->sparse_in_mirror = false;
  }
  if (x) {
    // pinned host memory is written by a kernel over the host link
    double *dst = static_cast<double *>(mapped_host(x));
    if (dst && (reinterpret_cast<uintptr_t>(dst) & 15) == 0)
      DE_CUDA(h, launch_sparse_store(h->d_sx, dst, int64_t(count), h->stream));
    else
      DE_CUDA(h, cudaMemcpyAsync(x, h->d_sx, count * sizeof(double), cudaMemcpyDefault, h->stream));
  }
  if (coll) {
    if (!h->d_coll || h->sparse_batch <= 0) return fail(h, DE_ERR_INVALID, "no batch collector: run first");
    DE_CUDA(h, cudaMemcpyAsync(coll, h->d_coll, size_t(h->sparse_batch) * h->dim * sizeof(double),
                               cudaMemcpyDeviceToHost, h->stream));
  }
  DE_CUDA(h, cudaStreamSynchronize(h->stream));
  return check_device_error(h);
}

int de_sparse_embedding(de_handle *h, double *x, int32_t iterations, int32_t batch_size, int32_t ns, double lr,
                        double density, int32_t merge, double *coll) {
  if (!h || !x) return DE_ERR_INVALID;
  int rc = de_sparse_set(h, x);
  if (!rc) rc = de_sparse_run(h, iterations, batch_size, ns, lr, density, merge);
  if (!rc) rc = de_sparse_get(h, x, coll);
  return rc;
}

int de_sync(de_handle *h) {
  if (!h) return DE_ERR_INVALID;
  DE_CUDA(h, cudaSetDevice(h->device));
  DE_CUDA(h, cudaStreamSynchronize(h->stream));
  return check_device_error(h);
}

int de_profile_epoch(de_handle *h, int32_t first_epoch, int32_t batch_size, int32_t ns, double lr,
                     float *launch_ms, int32_t *launch_kind, int32_t capacity, int32_t *count) {
  if (!h || !count) return DE_ERR_INVALID;
  if (first_epoch < 0 || batch_size <= 0 || ns < 0) return fail(h, DE_ERR_INVALID, "bad epoch, batch_size or ns");
  int rc = prepare_run(h, first_epoch, 1, batch_size, ns, &lr);
  if (rc) return rc;
  const std::vector<int> kinds = epoch_launch_kinds(h);
  const int n = int(kinds.size());
  *count = n;
  if (!launch_ms || !launch_kind || capacity < n) return fail(h, DE_ERR_INVALID, "capacity below the launch count");
  std::vector<cudaEvent_t> ev(n + 1, nullptr);
  for (auto &e : ev) DE_CUDA(h, cudaEventCreate(&e));
  cudaError_t err = enqueue_epoch(h, ns, h->stream, ev.data());
  if (err == cudaSuccess) err = cudaEventRecord(ev[n], h->stream);
  if (err == cudaSuccess) err = cudaStreamSynchronize(h->stream);
  for (int i = 0; err == cudaSuccess && i < n; ++i) {
    err = cudaEventElapsedTime(&launch_ms[i], ev[i], ev[i + 1]);
    launch_kind[i] = kinds[i];
  }
  for (auto &e : ev) cudaEventDestroy(e);
  if (err != cudaSuccess) return cuda_fail(h, err, "profiled epoch");
  return check_device_error(h);
}

int64_t de_edge_updates(de_handle *h, int32_t first_epoch, int32_t epochs, int32_t batch_size,
                        int32_t ns) {
  if (!h || first_epoch < 0 || epochs < 0 || batch_size <= 0 || ns < 0) return -1;
  const int batches = int(h->n / batch_size + (h->n % batch_size ? 1 : 0));
  const int last = (h->n % batch_size) ? int(h->n - int64_t(batch_size) * (batches - 1)) : batch_size;
  const int64_t attract = h->nnz - (h->opt.ref_quirks ? h->edges_into_last : 0);
  int64_t total = attract * epochs;
  std::vector<int32_t> negs(std::max(ns, 1));
  for (int i = first_epoch; i < first_epoch + epochs; ++i)
    for (int j = 0; j < batches; ++j) {
      draw_negatives(h->n, i + j, ns, negs.data());
      int valid = 0;
      for (int k = 0; k < ns; ++k) valid += (negs[k] >= 0 && negs[k] < h->n);
      const int rows = (j == batches - 1) ? last : batch_size;
      const int rep = (h->opt.ref_quirks && i > 0) ? last : rows;
      total += int64_t(rep) * valid;
    }
  return total;
}

void de_negatives(int64_t n, int32_t seed, int32_t ns, int64_t *out) {
  std::minstd_rand gen(seed);
  std::uniform_int_distribution<int> dist(0, int(n));
  for (int k = 0; k < ns; ++k) out[k] = dist(gen);
}

void *de_stream(de_handle *h) { return h ? static_cast<void *>(h->stream) : nullptr; }

const char *de_last_error(const de_handle *h) { return h ? h->err.c_str() : g_create_error.c_str(); }

const char *de_version(void) { return "distembed_gb300 0.1 (sm_103a)"; }

}  // extern "C"
