// Served form: a request loop that trains many embedding jobs on one GPU.
//
// No counterpart in the reference, which runs one job per process
// (cpp/dist_embed.cpp:156-347).  Each job is that same one-rank step
// (cpp/algo/algo.hpp:164-192) on its own resident handle, so a job's result does
// not depend on what else runs.
//
//   admission   jobs wait in FIFO order until a worker slot is free and the
//               job's device footprint fits in the server's memory budget (a
//               share of the GPU's free HBM, taken once as an arena)
//   overlap     every slot is a host thread with its own CUDA stream: the
//               kernels of all running jobs share the GPU, and a job that
//               arrives while others run starts as soon as a slot and memory
//               free up (no batch boundary to wait for)
//   state       a job's CSR and embedding stay on the device for all its
//               epochs; the arena hands out and takes back device memory
//               without the device-wide synchronisation of cudaFree
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "../../include/distembed_gb300.h"
#include "de_internal.h"

namespace de {
void set_thread_error(const std::string &msg);  // de_runtime.cpp
}

namespace {

// Best-fit arena over one device allocation; free blocks are coalesced.
class Arena {
 public:
  cudaError_t init(size_t bytes) {
    size_ = bytes & ~size_t(255);
    cudaError_t e = cudaMalloc(&base_, size_);
    if (e == cudaSuccess) free_[0] = size_;
    return e;
  }
  void release() {
    if (base_) cudaFree(base_);
    base_ = nullptr;
  }
  void *alloc(size_t bytes) {
    bytes = (std::max<size_t>(bytes, 1) + 255) & ~size_t(255);
    std::lock_guard<std::mutex> lk(mu_);
    auto best = free_.end();
    for (auto it = free_.begin(); it != free_.end(); ++it)
      if (it->second >= bytes && (best == free_.end() || it->second < best->second)) best = it;
    if (best == free_.end()) return nullptr;
    const size_t off = best->first, len = best->second;
    free_.erase(best);
    if (len > bytes) free_[off + bytes] = len - bytes;
    used_[off] = bytes;
    in_use_ += bytes;
    return static_cast<char *>(base_) + off;
  }
  void free(void *p) {
    std::lock_guard<std::mutex> lk(mu_);
    const size_t off = static_cast<char *>(p) - static_cast<char *>(base_);
    auto u = used_.find(off);
    if (u == used_.end()) return;
    size_t start = off, len = u->second;
    in_use_ -= len;
    used_.erase(u);
    auto next = free_.lower_bound(start);
    if (next != free_.end() && next->first == start + len) {
      len += next->second;
      next = free_.erase(next);
    }
    if (next != free_.begin()) {
      auto prev = std::prev(next);
      if (prev->first + prev->second == start) {
        start = prev->first;
        len += prev->second;
        free_.erase(prev);
      }
    }
    free_[start] = len;
  }
  size_t size() const { return size_; }

 private:
  void *base_ = nullptr;
  size_t size_ = 0, in_use_ = 0;
  std::map<size_t, size_t> free_;  // offset -> length
  std::map<size_t, size_t> used_;
  std::mutex mu_;
};

void *arena_alloc(void *ctx, size_t bytes) { return static_cast<Arena *>(ctx)->alloc(bytes); }
void arena_free(void *ctx, void *p) { static_cast<Arena *>(ctx)->free(p); }

struct Job {
  int64_t id = 0;
  de_job_spec spec{};
  std::vector<double> lr;
  int64_t bytes = 0;
  de_job_info info{};
  std::string err;
};

// Device bytes a job's handle allocates (an upper bound of the runtime's own
// buffers: graph, embedding, work lists, staging, per-call arrays, BF16 form).
int64_t job_bytes(const de_job_spec &s) {
  const int64_t n = s.n, nnz = s.nnz, D = s.dim, B = s.batch_size;
  const int64_t batches = (n + B - 1) / B;
  constexpr int64_t cap = 32;
  // work items: one per row plus one per further cap-sized piece of a long row
  int64_t items = 0, max_items = 0;
  for (int64_t j = 0; j < batches; ++j) {
    int64_t bi = 0;
    const int64_t r1 = std::min(n, (j + 1) * B);
    for (int64_t r = j * B; r < r1; ++r) {
      const int64_t deg = s.rowptr[r + 1] - s.rowptr[r];
      bi += deg <= cap ? 1 : (deg + cap - 1) / cap + (deg + cap - 1) / cap / 16 + 1;
    }
    items += bi;
    max_items = std::max(max_items, bi);
  }
  int64_t b = 4 * (n + 1) + 4 * std::max<int64_t>(nnz, 1) + 4 * n * D;  // CSR, embedding
  b += 32 * items;                                                      // work items
  b += 3 * B * D * 4 + max_items * D * 4 + max_items * 4;               // staging, partial slots, counters
  b += 8 * items;                                                       // per-item loss partials
  b += int64_t(s.epochs) * (batches * s.ns * 4 + 16);                   // negatives, rates, losses
  b += 8 * 2048;                                                        // small fixed buffers
  if (s.precision == DE_PRECISION_BF16) {
    const int64_t kpad = std::max<int64_t>(64, (s.ns + 63) / 64 * 64);
    b += 2 * n * D + 8 * n + 2 * B * D * 4 + 2 * kpad * D * 2 + kpad * 8 + B * 32 * 4;  // + update rows
  }
  return b + b / 16 + (1 << 20);  // allocator rounding and slack
}

double now_s(std::chrono::steady_clock::time_point t0) {
  return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
}

}  // namespace

struct de_server {
  int device = 0;
  int slots = 0;
  int ref_quirks = 1;
  Arena arena;
  std::chrono::steady_clock::time_point t0;
  std::mutex mu;
  std::condition_variable cv;
  std::deque<Job *> queue;
  std::map<int64_t, std::unique_ptr<Job>> jobs;
  std::vector<std::thread> workers;
  bool stopping = false;
  int64_t next_id = 1, reserved = 0, peak_reserved = 0, completions = 0, head_blocked_until = 0;
  int running = 0, peak_running = 0;
  de_server_stats stats{};
  std::string err;
};

namespace {

int sfail(de_server *s, int code, const std::string &m) {
  if (s) s->err = m; else de::set_thread_error(m);
  return code;
}

// One job on the worker's stream: resident handle, embedding in, the epochs,
// embedding and loss out.  Returns a DE_* code; err gets the text.
int run_job(de_server *s, Job *j, cudaStream_t stream, std::string &err) {
  const de_job_spec &sp = j->spec;
  de_options o;
  de_default_options(&o);
  o.precision = sp.precision;
  o.ref_quirks = s->ref_quirks;
  o.compute_loss = 1;
  o.device = s->device;
  o.stream = stream;
  de::MemHooks hooks;
  hooks.dalloc = arena_alloc;
  hooks.dfree = arena_free;
  hooks.ctx = &s->arena;
  de_handle *h = nullptr;
  int rc = de::create_handle(sp.n, sp.rowptr, sp.col, sp.nnz, sp.dim, &o, &hooks, &h);
  if (rc) {
    err = de_last_error(nullptr);
    return rc;
  }
  j->info.edge_updates = de_edge_updates(h, 0, sp.epochs, sp.batch_size, sp.ns);
  if (!rc) rc = de_set_embeddings_f32(h, sp.x0, 0);
  if (!rc) rc = de_run_from(h, 0, sp.epochs, sp.batch_size, sp.ns, j->lr.data(), nullptr);
  if (!rc) rc = de_sync(h);
  if (!rc && sp.loss_out) rc = de::copy_loss(h, sp.loss_out, sp.epochs);
  if (!rc) rc = de_get_embeddings_f32(h, sp.x_out, 0);
  if (rc) err = de_last_error(h);
  de_destroy(h);
  return rc;
}

bool head_admissible(de_server *s) {
  if (s->queue.empty() || s->running >= s->slots) return false;
  if (s->completions < s->head_blocked_until) return false;
  return s->reserved + s->queue.front()->bytes <= int64_t(s->arena.size());
}

void worker_main(de_server *s) {
  cudaSetDevice(s->device);
  cudaStream_t stream = nullptr;
  cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking);
  for (;;) {
    Job *j = nullptr;
    {
      std::unique_lock<std::mutex> lk(s->mu);
      s->cv.wait(lk, [&] { return (s->stopping && s->queue.empty()) || head_admissible(s); });
      if (s->queue.empty()) break;
      j = s->queue.front();
      s->queue.pop_front();
      s->reserved += j->bytes;
      s->peak_reserved = std::max(s->peak_reserved, s->reserved);
      ++s->running;
      s->peak_running = std::max(s->peak_running, s->running);
      j->info.state = DE_JOB_RUNNING;
      j->info.start_s = now_s(s->t0);
    }
    std::string err;
    const int rc = run_job(s, j, stream, err);
    {
      std::lock_guard<std::mutex> lk(s->mu);
      s->reserved -= j->bytes;
      --s->running;
      if (rc == DE_ERR_OOM && s->running > 0) {
        // the arena is fragmented: retry this job first, after the next completion
        j->info.state = DE_JOB_QUEUED;
        s->queue.push_front(j);
        s->head_blocked_until = s->completions + 1;
      } else {
        ++s->completions;
        j->info.state = rc ? DE_JOB_FAILED : DE_JOB_DONE;
        j->info.end_s = now_s(s->t0);
        j->err = err;
        if (rc) ++s->stats.failed; else ++s->stats.done;
      }
    }
    s->cv.notify_all();
  }
  if (stream) cudaStreamDestroy(stream);
}

}  // namespace

extern "C" {

int de_server_create(int32_t device, int32_t slots, int64_t hbm_bytes, double hbm_fraction, int32_t ref_quirks,
                     de_server **out) {
  if (!out) return sfail(nullptr, DE_ERR_INVALID, "out is NULL");
  *out = nullptr;
  if (slots < 1 || slots > 256) return sfail(nullptr, DE_ERR_INVALID, "slots must be in [1, 256]");
  cudaError_t e = cudaSetDevice(device);
  if (e != cudaSuccess) return sfail(nullptr, DE_ERR_CUDA, cudaGetErrorString(e));
  size_t free_b = 0, total_b = 0;
  if ((e = cudaMemGetInfo(&free_b, &total_b)) != cudaSuccess) return sfail(nullptr, DE_ERR_CUDA, cudaGetErrorString(e));
  size_t budget = hbm_bytes > 0 ? size_t(hbm_bytes) : size_t(double(free_b) * (hbm_fraction > 0 ? hbm_fraction : 0.8));
  if (budget > free_b) return sfail(nullptr, DE_ERR_OOM, "the memory budget exceeds the GPU's free memory");
  auto s = std::make_unique<de_server>();
  s->device = device;
  s->slots = slots;
  s->ref_quirks = ref_quirks;
  s->t0 = std::chrono::steady_clock::now();
  if ((e = s->arena.init(budget)) != cudaSuccess)
    return sfail(nullptr, DE_ERR_OOM, std::string("arena: ") + cudaGetErrorString(e));
  for (int i = 0; i < slots; ++i) s->workers.emplace_back(worker_main, s.get());
  *out = s.release();
  return DE_OK;
}

int de_server_submit(de_server *s, const de_job_spec *spec, int64_t *id) {
  if (!s || !spec || !id) return DE_ERR_INVALID;
  const de_job_spec &sp = *spec;
  if (sp.n <= 0 || !sp.rowptr || (sp.nnz > 0 && !sp.col) || !sp.x0 || !sp.x_out || sp.epochs <= 0 ||
      sp.batch_size <= 0 || sp.ns < 0 || !sp.lr_per_epoch)
    return sfail(s, DE_ERR_INVALID, "bad job: n, rowptr, col, x0, x_out, epochs, batch_size, ns and lr are required");
  if (sp.rowptr[0] != 0 || sp.rowptr[sp.n] != sp.nnz) return sfail(s, DE_ERR_INVALID, "bad job: rowptr");
  auto j = std::make_unique<Job>();
  j->spec = sp;
  j->lr.assign(sp.lr_per_epoch, sp.lr_per_epoch + sp.epochs);
  j->bytes = job_bytes(sp);
  if (j->bytes > int64_t(s->arena.size()))
    return sfail(s, DE_ERR_UNSUPPORTED, "job needs " + std::to_string(j->bytes) + " bytes, more than the server's budget");
  {
    std::lock_guard<std::mutex> lk(s->mu);
    j->id = s->next_id++;
    j->info.state = DE_JOB_QUEUED;
    j->info.submit_s = now_s(s->t0);
    j->info.device_bytes = j->bytes;
    *id = j->id;
    s->queue.push_back(j.get());
    s->jobs[j->id] = std::move(j);
    ++s->stats.submitted;
  }
  s->cv.notify_all();
  return DE_OK;
}

int de_server_info(de_server *s, int64_t id, de_job_info *info) {
  if (!s || !info) return DE_ERR_INVALID;
  std::lock_guard<std::mutex> lk(s->mu);
  auto it = s->jobs.find(id);
  if (it == s->jobs.end()) return sfail(s, DE_ERR_INVALID, "unknown job id");
  *info = it->second->info;
  return DE_OK;
}

int de_server_wait(de_server *s, int64_t id, de_job_info *info) {
  if (!s) return DE_ERR_INVALID;
  std::unique_lock<std::mutex> lk(s->mu);
  auto it = s->jobs.find(id);
  if (it == s->jobs.end()) return sfail(s, DE_ERR_INVALID, "unknown job id");
  Job *j = it->second.get();
  s->cv.wait(lk, [&] { return j->info.state == DE_JOB_DONE || j->info.state == DE_JOB_FAILED; });
  if (info) *info = j->info;
  const bool failed = j->info.state == DE_JOB_FAILED;
  const std::string err = j->err;
  s->jobs.erase(it);
  if (failed) return sfail(s, DE_ERR_CUDA, "job " + std::to_string(id) + " failed: " + err);
  return DE_OK;
}

int de_server_drain(de_server *s) {
  if (!s) return DE_ERR_INVALID;
  std::unique_lock<std::mutex> lk(s->mu);
  s->cv.wait(lk, [&] { return s->queue.empty() && s->running == 0; });
  return DE_OK;
}

int de_server_get_stats(de_server *s, de_server_stats *st) {
  if (!s || !st) return DE_ERR_INVALID;
  std::lock_guard<std::mutex> lk(s->mu);
  *st = s->stats;
  st->queued = int64_t(s->queue.size());
  st->running = s->running;
  st->peak_running = s->peak_running;
  st->budget_bytes = int64_t(s->arena.size());
  st->reserved_bytes = s->reserved;
  st->peak_reserved_bytes = s->peak_reserved;
  return DE_OK;
}

double de_server_clock(const de_server *s) { return s ? now_s(s->t0) : 0.0; }

int de_server_destroy(de_server *s) {
  if (!s) return DE_OK;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    s->stopping = true;
  }
  s->cv.notify_all();
  for (std::thread &t : s->workers) t.join();
  cudaSetDevice(s->device);
  s->arena.release();
  delete s;
  return DE_OK;
}

const char *de_server_last_error(const de_server *s) { return s ? s->err.c_str() : de_last_error(nullptr); }

}  // extern "C"
