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
#include <string>
#include <vector>

#include "../../include/distembed_gb300.h"
#include "de_async.cuh"
#include "de_device.cuh"
#include "de_internal.h"

namespace de {
void set_thread_error(const std::string &msg);  // de_runtime.cpp
}

namespace {

using de::WorkItem;
namespace dev = de::dev;

constexpr unsigned kAll = 0xffffffffu;

struct GraphInfo {
  int64_t voff;      // first vertex of the graph in the concatenated embedding
  int64_t eoff;      // first CSR entry of the graph in the concatenated col array
  int64_t batch_off; // first minibatch of the graph in the per-minibatch tables
  int64_t neg_off;   // first negative of the graph (per run: [epochs, batches, ns])
  int32_t n, batches, last_batch_size;
  int32_t pad;
};

struct SplitRow {
  int32_t row, first_slot, nparts, pad;
};

struct BatchedArgs {
  const GraphInfo *graphs;
  const int32_t *order;      // graphs, largest first
  int32_t n_graphs;
  int32_t *next_graph;       // team work counter, zeroed before the launch
  const int32_t *col;        // every graph's CSR columns, concatenated (graph g from eoff)
  const WorkItem *items;     // rows are local to the minibatch, edges local to the graph
  const int64_t *batch_item_off;
  const int32_t *batch_split_off;
  const SplitRow *splits;
  float *xm;                 // FP32 master [sum n, dim]
  __nv_bfloat16 *xb;         // BF16 copy (BF16 form) or nullptr
  const int32_t *negs;       // [graph][epoch][batch][ns]
  const float *lr;           // [epochs]
  int32_t epochs, batch, ns, quirks, compute_loss;
  float bound;
  float *stage;              // [teams, batch, dim] staged updates
  float *slots;              // [teams, max slots, dim] partials of split rows
  int32_t slot_stride;       // slots per team
  double *loss;              // [n_graphs, epochs]
  float near_r;              // BF16 form: pairs closer than this are recomputed in FP32
  long long *trace;          // nullable: per graph {start ns, end ns, team}
  int32_t cap;               // staged kernel: CSR entries per chunk (<= 32)
  int32_t *err;              // staged kernel: set when a bounded wait gives up
};

// One group of L = 32 / VPW lanes works on one item; lane j of the group holds
// components [j*P, j*P + P) of a row, P = D / L.
template <int D, int VPW>
struct Row {
  static constexpr int L = 32 / VPW;
  static constexpr int P = D / L;
  float v[P];
};

template <int D, int VPW, bool kBF16>
__device__ __forceinline__ void load_row(Row<D, VPW> &r, const BatchedArgs &a, int64_t vertex, int gl) {
  constexpr int P = Row<D, VPW>::P;
  const int64_t base = vertex * D + int64_t(gl) * P;
  if constexpr (kBF16) {
    const __nv_bfloat162 *p = reinterpret_cast<const __nv_bfloat162 *>(a.xb + base);
#pragma unroll
    for (int i = 0; i < P / 2; ++i) {
      float2 f = __bfloat1622float2(p[i]);
      r.v[2 * i] = f.x;
      r.v[2 * i + 1] = f.y;
    }
  } else {
    const float2 *p = reinterpret_cast<const float2 *>(a.xm + base);
#pragma unroll
    for (int i = 0; i < P / 2; ++i) {
      float2 f = __ldcg(p + i);
      r.v[2 * i] = f.x;
      r.v[2 * i + 1] = f.y;
    }
  }
}

template <int L>
__device__ __forceinline__ float group_sum(float v) {
#pragma unroll
  for (int m = L / 2; m >= 1; m >>= 1) v += __shfl_xor_sync(kAll, v, m);
  return v;
}

__device__ __forceinline__ long long globaltimer() {
  long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ float bclip(float v, float b) { return v > b ? b : (v < -b ? -b : v); }

// Forces of up to 4 rows named by lanes [k, k+4) of the group (ids < 0: none),
// all groups of the warp in step (the caller keeps the warp converged).  xi is the
// row's FP32 master value.  In the BF16 form the rows are read as BF16; a pair
// whose squared distance from those reads is below a.near_r is read again from
// the FP32 master and recomputed, so that the rounding of the copy does not bias
// close pairs (their distance is then comparable with the BF16 rounding step).
template <int D, int VPW, bool kBF16, bool kAttract>
__device__ __forceinline__ void group_forces(const BatchedArgs &a, Row<D, VPW> &acc, const Row<D, VPW> &xi,
                                             int64_t voff, int ids, int k, int gbase, int gl, float lr,
                                             float &loss) {
  constexpr int L = Row<D, VPW>::L, P = Row<D, VPW>::P;
  constexpr int U = L >= 4 ? 4 : L;
  Row<D, VPW> xn[U];
  int nid[U];
  float r[U];
#pragma unroll
  for (int u = 0; u < U; ++u) {
    int n = __shfl_sync(kAll, ids, gbase + k + u);
    nid[u] = n;
    if (n >= 0) load_row<D, VPW, kBF16>(xn[u], a, voff + n, gl);
    else xn[u] = xi;
  }
#pragma unroll
  for (int u = 0; u < U; ++u) {
    float p = 0.f;
#pragma unroll
    for (int t = 0; t < P; ++t) {
      const float d = xi.v[t] - xn[u].v[t];
      p = fmaf(d, d, p);
    }
    r[u] = group_sum<L>(p);
  }
  if constexpr (kBF16) {
    bool near[U], any = false;
#pragma unroll
    for (int u = 0; u < U; ++u) {
      near[u] = nid[u] >= 0 && r[u] < a.near_r;
      any |= near[u];
    }
    if (__any_sync(kAll, any)) {
#pragma unroll
      for (int u = 0; u < U; ++u)
        if (near[u]) load_row<D, VPW, false>(xn[u], a, voff + nid[u], gl);
#pragma unroll
      for (int u = 0; u < U; ++u) {
        float p = 0.f;
#pragma unroll
        for (int t = 0; t < P; ++t) {
          const float d = xi.v[t] - xn[u].v[t];
          p = fmaf(d, d, p);
        }
        p = group_sum<L>(p);
        if (near[u]) r[u] = p;
      }
    }
  }
#pragma unroll
  for (int u = 0; u < U; ++u) {
    float c = kAttract ? -2.0f / (1.0f + r[u]) : 2.0f / ((r[u] + 1e-6f) * (1.0f + r[u]));
    if (nid[u] < 0) c = 0.f;
#pragma unroll
    for (int t = 0; t < P; ++t) acc.v[t] = fmaf(lr, bclip((xi.v[t] - xn[u].v[t]) * c, a.bound), acc.v[t]);
    if (nid[u] >= 0 && gl == 0) loss += kAttract ? log1pf(r[u]) : logf((1.0f + r[u]) / (r[u] + 1e-6f));
  }
}

// x[row0 + i] += stage[i] for i < count (and the BF16 copy), every thread's
// loads issued before its stores.
template <bool kBF16>
__device__ __forceinline__ void update_rows(float *xm, __nv_bfloat16 *xb, const float *stage, int64_t row0, int count,
                                            int tid, int nthreads) {
  constexpr int K = 4;
  for (int b0 = tid * 4; b0 < count; b0 += nthreads * 4 * K) {
    float4 m[K], st[K];
#pragma unroll
    for (int k = 0; k < K; ++k) {
      const int idx = b0 + k * nthreads * 4;
      if (idx < count) {
        m[k] = __ldcg(reinterpret_cast<const float4 *>(xm + row0 + idx));
        st[k] = __ldcg(reinterpret_cast<const float4 *>(stage + idx));
      }
    }
#pragma unroll
    for (int k = 0; k < K; ++k) {
      const int idx = b0 + k * nthreads * 4;
      if (idx < count) {
        m[k].x += st[k].x;
        m[k].y += st[k].y;
        m[k].z += st[k].z;
        m[k].w += st[k].w;
        *reinterpret_cast<float4 *>(xm + row0 + idx) = m[k];
        if constexpr (kBF16) {
          __nv_bfloat162 *o = reinterpret_cast<__nv_bfloat162 *>(xb + row0 + idx);
          o[0] = __floats2bfloat162_rn(m[k].x, m[k].y);
          o[1] = __floats2bfloat162_rn(m[k].z, m[k].w);
        }
      }
    }
  }
}

// Split rows of a minibatch: the pieces of each row summed in piece order.
template <int D>
__device__ __forceinline__ void combine_split_rows(const BatchedArgs &a, const float *slots, float *stage, int s0, int s1,
                                                   int warp, int nwarps, int lane) {
  for (int i = s0 + warp; i < s1; i += nwarps) {
    const SplitRow sr = a.splits[i];
    dev::Frag<D> acc;
    dev::sum_slots<D>(acc, slots + size_t(sr.first_slot) * D, sr.nparts, lane);
    dev::store<D, false>(acc, stage + size_t(sr.row) * D, lane);
  }
}

template <int D, int VPW, int WARPS, bool kBF16>
__global__ void __launch_bounds__(WARPS * 32) batched_kernel(const BatchedArgs a) {
  constexpr int L = Row<D, VPW>::L, P = Row<D, VPW>::P;
  static_assert(P % 2 == 0, "components per lane must be even");
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int grp = lane / L, gl = lane % L, gbase = grp * L;
  __shared__ int sh_graph;
  __shared__ double sh_loss[WARPS];
  float *stage = a.stage + size_t(blockIdx.x) * a.batch * D;
  float *slots = a.slots + size_t(blockIdx.x) * a.slot_stride * D;
  const int skip_last = a.quirks;

  for (;;) {
    if (threadIdx.x == 0) {
      const int i = atomicAdd(a.next_graph, 1);
      sh_graph = i < a.n_graphs ? a.order[i] : -1;
    }
    __syncthreads();
    const int g = sh_graph;
    __syncthreads();
    if (g < 0) return;
    if (a.trace && threadIdx.x == 0) {
      a.trace[3 * g] = globaltimer();
      a.trace[3 * g + 2] = blockIdx.x;
    }
    const GraphInfo G = a.graphs[g];
    const int skip = skip_last ? G.n - 1 : -1;  // edges into n-1 are dropped (algo.hpp:399-405, 538)
    for (int e = 0; e < a.epochs; ++e) {
      const float lr = a.lr[e];
      double wloss = 0.0;  // this warp's share of the epoch loss, in item order
      for (int j = 0; j < G.batches; ++j) {
        const int64_t bi = G.batch_off + j;
        const int64_t it0 = a.batch_item_off[bi];
        const int n_items = int(a.batch_item_off[bi + 1] - a.batch_item_off[bi]);
        const int base = j * a.batch;
        const int rows = min(a.batch, G.n - base);
        const int rep_rows = (a.quirks && e > 0) ? G.last_batch_size : rows;  // algo.hpp:167-169, 594
        const int32_t *negs = a.negs + G.neg_off + (size_t(e) * G.batches + j) * a.ns;
        // ---- 1. items, VPW per warp at a time
        for (int i0 = warp * VPW; i0 < n_items; i0 += WARPS * VPW) {
          const int my = i0 + grp;
          const bool has = my < n_items;
          WorkItem it{};
          if (has) it = a.items[it0 + my];
          Row<D, VPW> xi, acc;
#pragma unroll
          for (int t = 0; t < P; ++t) acc.v[t] = 0.f;
          if (has) load_row<D, VPW, false>(xi, a, G.voff + base + it.row, gl);
          else
#pragma unroll
            for (int t = 0; t < P; ++t) xi.v[t] = 0.f;
          float loss = 0.f;
          const int cnt = has ? it.e_end - it.e_begin : 0;
          int maxcnt = cnt;
#pragma unroll
          for (int m = 16; m >= L; m >>= 1) maxcnt = max(maxcnt, __shfl_xor_sync(kAll, maxcnt, m));
          for (int c0 = 0; c0 < maxcnt; c0 += L) {
            int ids = -1;
            if (gl < cnt - c0) {
              ids = __ldg(a.col + G.eoff + it.e_begin + c0 + gl);
              if (ids == skip) ids = -1;
            }
            for (int k = 0; k < L && c0 + k < maxcnt; k += (L >= 4 ? 4 : L))
              group_forces<D, VPW, kBF16, true>(a, acc, xi, G.voff, ids, k, gbase, gl, lr, loss);
          }
          const bool repulse = has && it.part == 0 && it.row < rep_rows;
          const bool any_rep = __any_sync(kAll, repulse);
          for (int k0 = 0; any_rep && k0 < a.ns; k0 += L) {
            int ids = -1;
            if (repulse && gl < a.ns - k0) {
              ids = __ldg(negs + k0 + gl);
              if (ids >= G.n) ids = -1;  // a draw equal to n contributes nothing
            }
            for (int k = 0; k < L && k0 + k < a.ns; k += (L >= 4 ? 4 : L))
              group_forces<D, VPW, kBF16, false>(a, acc, xi, G.voff, ids, k, gbase, gl, lr, loss);
          }
          if (has) {
            float *dst = it.nparts > 1 ? slots + size_t(it.first_slot + it.part) * D : stage + size_t(it.row) * D;
#pragma unroll
            for (int t = 0; t < P; t += 2) *reinterpret_cast<float2 *>(dst + gl * P + t) = make_float2(acc.v[t], acc.v[t + 1]);
          }
          // item loss, fixed order: groups of the warp in order
#pragma unroll
          for (int q = 0; q < VPW; ++q) wloss += double(__shfl_sync(kAll, loss, q * L));
        }
        __syncthreads();
        // ---- 2. split rows: pieces in piece order
        combine_split_rows<D>(a, slots, stage, a.batch_split_off[bi], a.batch_split_off[bi + 1], warp, WARPS, lane);
        __syncthreads();
        // ---- 3. update (algo.hpp:651-666)
        update_rows<kBF16>(a.xm, a.xb, stage, (G.voff + base) * D, rows * D, threadIdx.x, WARPS * 32);
        __syncthreads();
      }
      if (lane == 0) sh_loss[warp] = wloss;
      __syncthreads();
      if (threadIdx.x == 0 && a.compute_loss) {
        double s = 0.0;
        for (int w = 0; w < WARPS; ++w) s += sh_loss[w];
        a.loss[size_t(g) * a.epochs + e] = s;
      }
      __syncthreads();
    }
    if (a.trace && threadIdx.x == 0) a.trace[3 * g + 1] = globaltimer();
  }
}


// ---------------------------------------------------------------- staged kernel
//
// The same per-graph step with the rows a warp reads staged in shared memory by
// 16-byte asynchronous copies (cp.async, through L2) instead of loaded into
// registers, so the bytes in flight per SM are bounded by shared memory, not by
// registers, and the copies of later chunks overlap the arithmetic of the current
// one.  Every warp runs its own pipeline over its chunks (work items i = warp,
// warp + W, ... of the minibatch; a chunk is at most cap <= 32 CSR entries):
//   column ids of chunk k+S are loaded while the rows of chunk k+S-1 are copied
//   (own row from the FP32 master, neighbours from the BF16 copy or the FP32
//   master) into ring slot (k+S-1) mod S, and chunk k is computed from slot k mod S
//   once its copy group has landed (cp.async.wait_group S-1).
// Each warp also copies the minibatch's ns negatives into its own area (with its
// first chunk).  A pair is computed by dim/8 lanes (8 components each),
// 32/(dim/8) pairs per warp step and NS steps in flight.  Results go to the
// team's staging rows as in the register kernel; the minibatch ends with the same
// combine and update.  No wait spins: every wait is a hardware wait on this
// thread's own copies or a CTA barrier.

constexpr int kStagedMaxNs = 32;

template <int D, bool kBF16>
struct StagedLayout {
  static constexpr int kRowB = kBF16 ? 2 * D : 4 * D;  // a neighbour row in shared memory
  static constexpr int kXiB = 4 * D;                   // the chunk's own row (FP32 master)
  __host__ __device__ static constexpr int slot_bytes(int cap) { return kXiB + cap * kRowB; }
  // per warp: S slots, the negatives (ns rows), 32 work items
  __host__ __device__ static size_t warp_bytes(int S, int cap, int ns) {
    return size_t(S) * slot_bytes(cap) + size_t(ns) * kRowB + 32 * sizeof(WorkItem);
  }
  __host__ __device__ static size_t bytes(int W, int S, int cap, int ns) { return size_t(W) * warp_bytes(S, cap, ns); }
};

// Copies `rows` rows (ids: lane j holds row j's vertex, local to voff) of
// kRowB bytes from `base` into consecutive rows at `dst`, 16 bytes per lane per
// instruction.
template <int kRowB>
__device__ __forceinline__ void copy_rows(uint32_t dst, const unsigned char *base, int64_t voff, int id, int rows,
                                          int lane) {
  constexpr int PR = kRowB / 16;  // pieces per row
  const int total = rows * PR;
  for (int p0 = 0; p0 < total; p0 += 32) {
    const int p = p0 + lane;
    const int row = p / PR;
    const int rid = __shfl_sync(kAll, id, row & 31);
    if (p < total) dev::cp_async16(dst + row * kRowB + (p % PR) * 16, base + (voff + rid) * kRowB + (p % PR) * 16);
  }
}

// Pair layout of the staged kernel: a pair is computed by LP = dim/8 lanes, each
// holding 8 components (16 bytes of a BF16 row), so one warp step covers
// G = 32/LP pairs: lane l works on pair l / LP of the step, components
// [8 (l % LP), 8 (l % LP) + 8).  A row's pairs are spread over the G groups and
// the groups' accumulators are summed (fixed order) when the row is done.
template <int D>
struct PairLanes {
  static constexpr int LP = D / 8;
  static constexpr int G = 32 / LP;
};

// 8 components of a row in shared memory (BF16 or FP32) for lane-in-pair gl.
template <bool kBF16>
__device__ __forceinline__ void ld8(float (&v)[8], const unsigned char *row, int gl) {
  if constexpr (kBF16) {
    const uint4 u = *reinterpret_cast<const uint4 *>(row + gl * 16);
    const uint32_t w[4] = {u.x, u.y, u.z, u.w};
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      v[2 * i] = __uint_as_float(w[i] << 16);
      v[2 * i + 1] = __uint_as_float(w[i] & 0xffff0000u);
    }
  } else {
    const float4 x = *reinterpret_cast<const float4 *>(row + gl * 32);
    const float4 y = *reinterpret_cast<const float4 *>(row + gl * 32 + 16);
    v[0] = x.x; v[1] = x.y; v[2] = x.z; v[3] = x.w;
    v[4] = y.x; v[5] = y.y; v[6] = y.z; v[7] = y.w;
  }
}

// NS warp steps of pairs (xi, rows[kb .. kb + NS*G)), rows past `count` skipped;
// valid bit k of vmask: pair k counts (rows of pairs that do not count hold real
// data, so they only need c = 0).
//
// Clip: |c * diff_k| <= |c| sqrt(r) for every component k, so when
// c^2 r <= bound^2 no component reaches the bound and the clip of
// algo.hpp:643 is the identity.  That always holds for the attractive force at
// bound >= 1 (|c| sqrt(r) = 2 sqrt(r) / (1 + r) <= 1) and for repulsion at
// r >= 0.25; a step in which some pair may clip takes the clipped path.
//
// BF16 form: a pair whose distance from the BF16 rows is below a.near_r is
// recomputed from the FP32 master row (global id: lane k of `ids`).
template <int D, int NS, bool kBF16, bool kAttract>
__device__ __forceinline__ void pair_steps(const BatchedArgs &a, float (&acc)[8], const float (&xi)[8],
                                           const unsigned char *rows, int row_bytes, int kb, int count, unsigned vmask,
                                           int ids, int64_t voff, float lr, float &loss, int lane) {
  constexpr int LP = PairLanes<D>::LP, G = PairLanes<D>::G;
  const int q = lane / LP, gl = lane % LP;
  float d[NS][8], r[NS];
  int k[NS];
  bool ok[NS];
#pragma unroll
  for (int st = 0; st < NS; ++st) {
    k[st] = kb + st * G + q;
    float xn[8];
    if (k[st] < count) {
      ld8<kBF16>(xn, rows + k[st] * row_bytes, gl);
    } else {
#pragma unroll
      for (int t = 0; t < 8; ++t) xn[t] = xi[t];
    }
    float p = 0.f;
#pragma unroll
    for (int t = 0; t < 8; ++t) {
      d[st][t] = xi[t] - xn[t];
      p = fmaf(d[st][t], d[st][t], p);
    }
    r[st] = p;
    ok[st] = k[st] < count && ((vmask >> k[st]) & 1u);
  }
#pragma unroll
  for (int m = LP / 2; m >= 1; m >>= 1)
#pragma unroll
    for (int st = 0; st < NS; ++st) r[st] += __shfl_xor_sync(kAll, r[st], m);
  if constexpr (kBF16) {
    bool near[NS], any = false;
#pragma unroll
    for (int st = 0; st < NS; ++st) {
      near[st] = ok[st] && r[st] < a.near_r;
      any |= near[st];
    }
    if (__any_sync(kAll, any)) {
#pragma unroll
      for (int st = 0; st < NS; ++st) {
        const int gid = __shfl_sync(kAll, ids, k[st] & 31);
        float p = 0.f;
        if (near[st]) {
          const float4 *src = reinterpret_cast<const float4 *>(a.xm + (voff + gid) * D + gl * 8);
          const float4 x = __ldcg(src), y = __ldcg(src + 1);
          const float f[8] = {x.x, x.y, x.z, x.w, y.x, y.y, y.z, y.w};
#pragma unroll
          for (int t = 0; t < 8; ++t) {
            d[st][t] = xi[t] - f[t];
            p = fmaf(d[st][t], d[st][t], p);
          }
        }
#pragma unroll
        for (int m = LP / 2; m >= 1; m >>= 1) p += __shfl_xor_sync(kAll, p, m);
        if (near[st]) r[st] = p;
      }
    }
  }
  float c[NS];
  bool may_clip = false;
#pragma unroll
  for (int st = 0; st < NS; ++st) {
    c[st] = kAttract ? __fdividef(-2.0f, 1.0f + r[st]) : __fdividef(2.0f, (r[st] + 1e-6f) * (1.0f + r[st]));
    if (!ok[st]) c[st] = 0.f;
    if (ok[st] && gl == 0) loss += kAttract ? __logf(1.0f + r[st]) : __logf(1.0f + r[st]) - __logf(r[st] + 1e-6f);
    may_clip |= c[st] * c[st] * r[st] > 0.98f * a.bound * a.bound;
  }
  if (!__any_sync(kAll, may_clip)) {
#pragma unroll
    for (int st = 0; st < NS; ++st) {
      const float lc = lr * c[st];
#pragma unroll
      for (int t = 0; t < 8; ++t) acc[t] = fmaf(lc, d[st][t], acc[t]);
    }
  } else {
#pragma unroll
    for (int st = 0; st < NS; ++st)
#pragma unroll
      for (int t = 0; t < 8; ++t) acc[t] = fmaf(lr, bclip(d[st][t] * c[st], a.bound), acc[t]);
  }
}

// All pairs of xi with rows [0, count).
template <int D, int NS, bool kBF16, bool kAttract>
__device__ __forceinline__ void staged_pairs(const BatchedArgs &a, float (&acc)[8], const float (&xi)[8],
                                             const unsigned char *rows, int row_bytes, int count, unsigned vmask,
                                             int ids, int64_t voff, float lr, float &loss, int lane) {
  constexpr int G = PairLanes<D>::G;
  int kb = 0;
  for (; kb + NS * G <= count; kb += NS * G)
    pair_steps<D, NS, kBF16, kAttract>(a, acc, xi, rows, row_bytes, kb, count, vmask, ids, voff, lr, loss, lane);
  if constexpr (NS > 1) {
    for (; kb < count; kb += G)
      pair_steps<D, 1, kBF16, kAttract>(a, acc, xi, rows, row_bytes, kb, count, vmask, ids, voff, lr, loss, lane);
  } else {
    if (kb < count)
      pair_steps<D, 1, kBF16, kAttract>(a, acc, xi, rows, row_bytes, kb, count, vmask, ids, voff, lr, loss, lane);
  }
}


template <int D, int NS, int S, bool kBF16>
__global__ void __launch_bounds__(512, 1) staged_kernel(const BatchedArgs a) {
  using Lay = StagedLayout<D, kBF16>;
  constexpr int kRowB = Lay::kRowB, kXiB = Lay::kXiB;
  constexpr int LP = PairLanes<D>::LP;
  extern __shared__ __align__(128) unsigned char smem[];
  const int W = blockDim.x >> 5, lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int gl = lane % LP;
  const int cap = a.cap, slotB = Lay::slot_bytes(cap);
  unsigned char *ring = smem + size_t(warp) * Lay::warp_bytes(S, cap, a.ns);
  unsigned char *negrows = ring + size_t(S) * slotB;
  WorkItem *my_items = reinterpret_cast<WorkItem *>(negrows + size_t(a.ns) * kRowB);
  const uint32_t ring_s = dev::smem_u32(ring), neg_s = dev::smem_u32(negrows);
  __shared__ int sh_graph;
  __shared__ double sh_loss[16];
  float *stage = a.stage + size_t(blockIdx.x) * a.batch * D;
  float *slots = a.slots + size_t(blockIdx.x) * a.slot_stride * D;
  const unsigned char *src = kBF16 ? reinterpret_cast<const unsigned char *>(a.xb)
                                   : reinterpret_cast<const unsigned char *>(a.xm);
  const unsigned char *srcm = reinterpret_cast<const unsigned char *>(a.xm);

  for (;;) {
    if (threadIdx.x == 0) {
      const int i = atomicAdd(a.next_graph, 1);
      sh_graph = i < a.n_graphs ? a.order[i] : -1;
    }
    __syncthreads();
    const int g = sh_graph;
    __syncthreads();
    if (g < 0) break;
    if (a.trace && threadIdx.x == 0) {
      a.trace[3 * g] = globaltimer();
      a.trace[3 * g + 2] = blockIdx.x;
    }
    const GraphInfo G = a.graphs[g];
    const int skip = a.quirks ? G.n - 1 : -1;  // edges into n-1 are dropped (algo.hpp:399-405, 538)
    for (int e = 0; e < a.epochs; ++e) {
      const float lr = a.lr[e];
      double wloss = 0.0;
      for (int j = 0; j < G.batches; ++j) {
        const int64_t bi = G.batch_off + j;
        const int64_t it0 = a.batch_item_off[bi];
        const int n_items = int(a.batch_item_off[bi + 1] - it0);
        const int base = j * a.batch;
        const int rows = min(a.batch, G.n - base);
        const int rep_rows = (a.quirks && e > 0) ? G.last_batch_size : rows;  // algo.hpp:167-169, 594
        const int32_t *negs = a.negs + G.neg_off + (size_t(e) * G.batches + j) * a.ns;
        // this minibatch's negatives: lane k holds draw k; a draw equal to n
        // contributes nothing (its slot copies row 0 so that it holds real data)
        const int nraw = lane < a.ns ? __ldg(negs + lane) : -1;
        const int nid = nraw < G.n ? nraw : 0;
        const unsigned neg_valid = __ballot_sync(kAll, lane < a.ns && nraw < G.n);
        const int nmine = n_items > warp ? (n_items - warp + W - 1) / W : 0;
        for (int r0 = 0; r0 < nmine; r0 += 32) {
          const int nr = min(32, nmine - r0);
          if (lane < nr) my_items[lane] = a.items[it0 + warp + int64_t(r0 + lane) * W];
          __syncwarp();
          // lane l: column id of CSR entry l of chunk k (-1 past its end)
          auto load_cols = [&](int k) -> int {
            const WorkItem &it = my_items[k];
            return lane < it.e_end - it.e_begin ? __ldg(a.col + G.eoff + it.e_begin + lane) : -1;
          };
          int issued = 0;  // chunks of this round whose copies were committed
          auto issue = [&](int k, int id) {
            const uint32_t slot = ring_s + uint32_t((k % S) * slotB);
            const int cnt = __popc(__ballot_sync(kAll, id >= 0));
            const int64_t own = G.voff + base + my_items[k].row;
            for (int p = lane; p < kXiB / 16; p += 32) dev::cp_async16(slot + p * 16, srcm + own * kXiB + p * 16);
            copy_rows<kRowB>(slot + kXiB, src, G.voff, id, cnt, lane);
            if (k == 0 && r0 == 0) copy_rows<kRowB>(neg_s, src, G.voff, nid, a.ns, lane);
            dev::cp_async_commit();
            ++issued;
          };
          int idq[S - 1];
#pragma unroll
          for (int i = 0; i < S - 1; ++i) idq[i] = i < nr ? load_cols(i) : -1;
#pragma unroll
          for (int i = 0; i < S - 1; ++i) {
            if (i < nr) issue(i, idq[i]);
            else dev::cp_async_commit();
          }
          int next = S - 1 < nr ? load_cols(S - 1) : -1;
          for (int k = 0; k < nr; ++k) {
            int nxt = -1;
            if (k + S - 1 < nr) {
              issue(k + S - 1, next);
              nxt = next;
            } else {
              dev::cp_async_commit();  // an empty group keeps "S-1 groups after chunk k"
            }
            next = k + S < nr ? load_cols(k + S) : -1;
            const int ids = idq[0];
#pragma unroll
            for (int i = 0; i + 1 < S - 1; ++i) idq[i] = idq[i + 1];
            idq[S - 2] = nxt;
            // ---- chunk k: its group is the oldest of the S in flight
            dev::cp_async_wait<S - 1>();
            __syncwarp();
            const WorkItem it = my_items[k];
            const unsigned char *slot = ring + size_t(k % S) * slotB;
            float xi[8], acc[8];
            ld8<false>(xi, slot, gl);
#pragma unroll
            for (int t = 0; t < 8; ++t) acc[t] = 0.f;
            float loss = 0.f;
            const int cnt = it.e_end - it.e_begin;
            const unsigned vmask = __ballot_sync(kAll, ids >= 0 && ids != skip);
            staged_pairs<D, NS, kBF16, true>(a, acc, xi, slot + kXiB, kRowB, cnt, vmask, ids, G.voff, lr, loss, lane);
            if (it.part == 0 && it.row < rep_rows && a.ns > 0)
              staged_pairs<D, NS, kBF16, false>(a, acc, xi, negrows, kRowB, a.ns, neg_valid, nid, G.voff, lr, loss,
                                                lane);
            // the groups' accumulators, summed; lanes of group 0 store the row
#pragma unroll
            for (int m = 16; m >= LP; m >>= 1)
#pragma unroll
              for (int t = 0; t < 8; ++t) acc[t] += __shfl_xor_sync(kAll, acc[t], m);
            float *dst = it.nparts > 1 ? slots + size_t(it.first_slot + it.part) * D : stage + size_t(it.row) * D;
            if (lane < LP) {
              reinterpret_cast<float4 *>(dst + gl * 8)[0] = make_float4(acc[0], acc[1], acc[2], acc[3]);
              reinterpret_cast<float4 *>(dst + gl * 8)[1] = make_float4(acc[4], acc[5], acc[6], acc[7]);
            }
#pragma unroll
            for (int m = 16; m >= 1; m >>= 1) loss += __shfl_xor_sync(kAll, loss, m);
            wloss += double(loss);
            __syncwarp();
          }
        }
        dev::cp_async_wait<0>();
        __syncthreads();
        combine_split_rows<D>(a, slots, stage, a.batch_split_off[bi], a.batch_split_off[bi + 1], warp, W, lane);
        __syncthreads();
        update_rows<kBF16>(a.xm, a.xb, stage, (G.voff + base) * D, rows * D, threadIdx.x, blockDim.x);  // algo.hpp:651-666
        __syncthreads();
      }
      if (lane == 0) sh_loss[warp] = wloss;
      __syncthreads();
      if (threadIdx.x == 0 && a.compute_loss) {
        double t = 0.0;
        for (int w = 0; w < W; ++w) t += sh_loss[w];
        a.loss[size_t(g) * a.epochs + e] = t;
      }
      __syncthreads();
    }
    if (a.trace && threadIdx.x == 0) a.trace[3 * g + 1] = globaltimer();
  }
}

// ---------------------------------------------------------------- dispatch

typedef void (*BatchedKernel)(BatchedArgs);

// A team shape exists when every lane of a group holds an even number of components.
template <int D, int V>
constexpr bool kShapeOk = (D / (32 / V)) % 2 == 0;

template <int D, bool kBF16, int V>
BatchedKernel pick_warps(int warps) {
  if constexpr (kShapeOk<D, V>) {
    switch (warps) {
      case 4: return batched_kernel<D, V, 4, kBF16>;
      case 8: return batched_kernel<D, V, 8, kBF16>;
      case 16: return batched_kernel<D, V, 16, kBF16>;
      case 32: return batched_kernel<D, V, 32, kBF16>;
    }
  }
  return nullptr;
}

template <int D, bool kBF16>
BatchedKernel pick(int vpw, int warps) {
  switch (vpw) {
    case 1: return pick_warps<D, kBF16, 1>(warps);
    case 2: return pick_warps<D, kBF16, 2>(warps);
    case 4: return pick_warps<D, kBF16, 4>(warps);
  }
  return nullptr;
}

BatchedKernel pick_register(int dim, bool bf16, int vpw, int warps) {
  switch (dim) {
    case 32: return bf16 ? pick<32, true>(vpw, warps) : pick<32, false>(vpw, warps);
    case 64: return bf16 ? pick<64, true>(vpw, warps) : pick<64, false>(vpw, warps);
    case 128: return bf16 ? pick<128, true>(vpw, warps) : pick<128, false>(vpw, warps);
  }
  return nullptr;
}

template <int D, bool kBF16>
BatchedKernel pick_staged_fn(int steps, int stages) {
  if (steps == 1 && stages == 3) return staged_kernel<D, 1, 3, kBF16>;
  if (steps == 1 && stages == 4) return staged_kernel<D, 1, 4, kBF16>;
  if (steps == 2 && stages == 3) return staged_kernel<D, 2, 3, kBF16>;
  if (steps == 2 && stages == 4) return staged_kernel<D, 2, 4, kBF16>;
  return nullptr;
}

// Largest dynamic shared memory a staged team may use (the static part is small).
constexpr size_t kStagedSmemMax = 227 * 1024 - 1024;

template <int D, bool kBF16>
size_t staged_smem(const de_batch_shape &s, int ns) {
  return StagedLayout<D, kBF16>::bytes(s.team_warps, s.stages, s.edge_cap, ns);
}

// The kernel, its block size and dynamic shared memory for a team shape; fn is
// null when the shape does not exist.
struct KernelPick {
  BatchedKernel fn = nullptr;
  int block = 0;
  size_t smem = 0;
};

KernelPick pick_kernel(int dim, bool bf16, const de_batch_shape &s, int ns = 0) {
  KernelPick k;
  if (s.kernel == DE_BATCH_REGISTER) {
    if (s.edge_cap < 1 || s.edge_cap > 4096) return k;
    k.fn = pick_register(dim, bf16, s.vertices_per_warp, s.team_warps);
    k.block = 32 * s.team_warps;
    return k;
  }
  if (s.kernel != DE_BATCH_STAGED || s.team_warps < 2 || s.team_warps > 16 || s.edge_cap < 1 || s.edge_cap > 32)
    return k;
  switch (dim) {
    case 32:
      k.fn = bf16 ? pick_staged_fn<32, true>(s.pairs, s.stages) : pick_staged_fn<32, false>(s.pairs, s.stages);
      k.smem = bf16 ? staged_smem<32, true>(s, ns) : staged_smem<32, false>(s, ns);
      break;
    case 64:
      k.fn = bf16 ? pick_staged_fn<64, true>(s.pairs, s.stages) : pick_staged_fn<64, false>(s.pairs, s.stages);
      k.smem = bf16 ? staged_smem<64, true>(s, ns) : staged_smem<64, false>(s, ns);
      break;
    case 128:
      k.fn = bf16 ? pick_staged_fn<128, true>(s.pairs, s.stages) : pick_staged_fn<128, false>(s.pairs, s.stages);
      k.smem = bf16 ? staged_smem<128, true>(s, ns) : staged_smem<128, false>(s, ns);
      break;
  }
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
  de_batch_shape shape{DE_BATCH_REGISTER, 4, 8, 32, 0, 0};
  int teams = 0, block = 0;
  size_t smem = 0;
  int32_t *d_err = nullptr;
  BatchedKernel kernel = nullptr;
  BatchedArgs args{};
  cudaGraphExec_t exec = nullptr;  // the prepared run
  int prepared_epochs = 0;
  float near_r = 0.02f;            // BF16 form: squared distance below which a pair is recomputed in FP32
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
      bsplit.push_back(int32_t(splits.size()));
    }
    batch_off += G.batches;
  }
  b->sched_batch = B;
  b->sched_cap = cap;
  b->max_slots = max_slots;
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
  return std::min(per_sm * sms, b->n_graphs);
}

// Everything of a run except the launch: schedule, negatives, rates, team staging
// areas and the kernel arguments (kept in b->args, b->kernel, b->teams).  Nothing
// here may run inside a stream capture: it allocates and copies synchronously.
int prepare_batched(de_batch *b, int epochs, int B, int ns, const double *lr, const de_batch_shape &shape) {
  BCUDA(b, cudaSetDevice(b->device));
  if (shape.kernel == DE_BATCH_STAGED && ns > kStagedMaxNs)
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
  std::vector<int64_t> draw(std::max(ns, 1));
  for (int g = 0; g < b->n_graphs; ++g) {
    const GraphInfo &G = b->ginfo[g];
    for (int e = 0; e < epochs; ++e)
      for (int j = 0; j < G.batches; ++j) {
        de_negatives(G.n, e + j, ns, draw.data());
        int32_t *o = negs.data() + G.neg_off + (size_t(e) * G.batches + j) * ns;
        for (int q = 0; q < ns; ++q) o[q] = int32_t(draw[q]);
      }
  }
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
  a.compute_loss = 1;
  a.bound = float(b->opt.max_bound);
  a.stage = b->d_stage;
  a.slots = b->d_slots;
  a.slot_stride = b->max_slots;
  a.loss = b->d_loss;
  a.near_r = b->near_r;
  a.trace = b->d_trace;
  a.cap = cap;
  a.err = b->d_err;
  b->kernel = k.fn;
  b->teams = teams;
  b->block = k.block;
  b->smem = k.smem;
  return DE_OK;
}

// The whole run: reset the team work counter, then one persistent launch.
int launch_batched(de_batch *b, cudaStream_t st) {
  BCUDA(b, cudaMemsetAsync(b->d_next, 0, sizeof(int32_t), st));
  b->kernel<<<b->teams, b->block, b->smem, st>>>(b->args);
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
      (e = cudaMalloc(&b->d_next, sizeof(int32_t))) != cudaSuccess ||
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
                  static_cast<void *>(b->d_err)})
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
      for (int c : {32, 64, 128}) cand.push_back(de_batch_shape{DE_BATCH_REGISTER, v, w, c, 0, 0});
  if (ns <= kStagedMaxNs)
    for (int w : {4, 8, 12, 16})
      for (int c : {8, 16, 32})
        for (int u : {1, 2})
          for (int st : {3, 4}) cand.push_back(de_batch_shape{DE_BATCH_STAGED, 0, w, c, u, st});
  const bool bf16 = b->opt.precision == DE_PRECISION_BF16;
  std::vector<double> lrs(epochs, lr);
  float best_ms = -1.f;
  de_batch_shape best_shape = b->shape;
  int tried = 0, rc = DE_OK;
  for (const de_batch_shape &sh : cand) {
    if (!pick_kernel(b->dim, bf16, sh, ns).fn) continue;
    rc = prepare_batched(b, epochs, batch_size, ns, lrs.data(), sh);
    if (rc) break;
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
