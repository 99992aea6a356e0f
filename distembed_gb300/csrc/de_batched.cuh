// Shared pieces of the batched form: arguments, per-graph tables, the update and
// split-row combine every kernel family ends a minibatch with, shared-memory
// layouts of the staged kernels (de_batched*.cu).
#pragma once
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include "../../include/distembed_gb300.h"
#include "de_async.cuh"
#include "de_device.cuh"
#include "de_internal.h"

namespace de {
namespace batched {

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
  // staged kernel with two-CTA teams: the first n_big graphs of `order` are trained
  // by both CTAs of a cluster together (next_big counts them out), the rest by
  // single CTAs (next_graph counts from order[n_big])
  int32_t n_big;
  int32_t *next_big;
  int32_t *cluster_slot;     // [clusters] graph handed from CTA rank 0 to rank 1
  float *item_loss;          // [teams, max items of a minibatch] loss of every work item
  int32_t item_stride;
  int32_t loss_from;         // epochs e >= loss_from (of this run) compute their loss; the others write 0
  int32_t stage_ids;         // staged kernel: 1 = a round's column ids are prefetched into shared memory
};

static __device__ __forceinline__ long long globaltimer() {
  long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

static __device__ __forceinline__ float bclip(float v, float b) { return v > b ? b : (v < -b ? -b : v); }

// d = x - y over 8 components with packed f32x2 arithmetic; returns |d|^2 (two
// interleaved partial sums, then their sum).
static __device__ __forceinline__ float diff8(float (&d)[8], const float (&x)[8], const float (&y)[8]) {
  float2 q = make_float2(0.f, 0.f);
#pragma unroll
  for (int t = 0; t < 8; t += 2) {
    const float2 v = dev::sub2(make_float2(x[t], x[t + 1]), make_float2(y[t], y[t + 1]));
    d[t] = v.x;
    d[t + 1] = v.y;
    q = __ffma2_rn(v, v, q);
  }
  return q.x + q.y;
}

// acc += s * d over 8 components (packed f32x2 FMA).
static __device__ __forceinline__ void axpy8(float (&acc)[8], float s, const float (&d)[8]) {
#pragma unroll
  for (int t = 0; t < 8; t += 2) {
    const float2 o = __ffma2_rn(make_float2(s, s), make_float2(d[t], d[t + 1]), make_float2(acc[t], acc[t + 1]));
    acc[t] = o.x;
    acc[t + 1] = o.y;
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

constexpr int kStagedMaxNs = 32;

template <int D, bool kBF16>
struct StagedLayout {
  static constexpr int kRowB = kBF16 ? 2 * D : 4 * D;  // a neighbour row in shared memory
  static constexpr int kXiB = 4 * D;                   // the chunk's own row (FP32 master)
  __host__ __device__ static constexpr int slot_bytes(int cap) { return kXiB + cap * kRowB; }
  // per warp: S slots, the negatives (ns rows), 32 work items and, with ids = 1,
  // their column ids (cap per item, 16-byte aligned)
  __host__ __device__ static size_t warp_bytes(int S, int cap, int ns, int ids = 1) {
    return size_t(S) * slot_bytes(cap) + size_t(ns) * kRowB + 32 * sizeof(WorkItem) +
           (ids ? ((size_t(32) * cap * 4 + 15) & ~size_t(15)) : 0);
  }
  __host__ __device__ static size_t bytes(int W, int S, int cap, int ns, int ids = 1) {
    return size_t(W) * warp_bytes(S, cap, ns, ids);
  }
};

// Copies `rows` rows (ids: lane j holds row j's vertex, local to voff) of
// kRowB bytes from `base` into consecutive rows at `dst`, 16 bytes per lane per
// instruction.
template <int kRowB>
static __device__ __forceinline__ void copy_rows(uint32_t dst, const unsigned char *base, int64_t voff, int id, int rows,
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
static __device__ __forceinline__ void ld8(float (&v)[8], const unsigned char *row, int gl) {
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

template <int D, bool kBF16>
struct RowsLayout {
  static constexpr int LP = D / 8, G = 32 / LP;
  static constexpr int kRowB = kBF16 ? 2 * D : 4 * D, kXiB = 4 * D;
  __host__ __device__ static constexpr int ids_bytes(int cap) { return (cap * 4 + 15) & ~15; }
  __host__ __device__ static constexpr int sub_bytes(int cap) { return kXiB + cap * kRowB + ids_bytes(cap); }
  __host__ __device__ static constexpr int slot_bytes(int cap) { return G * sub_bytes(cap); }
  __host__ __device__ static size_t warp_bytes(int S, int cap, int ns) {
    return size_t(S) * slot_bytes(cap) + size_t(ns) * kRowB + 32 * sizeof(WorkItem);
  }
  __host__ __device__ static size_t bytes(int W, int S, int cap, int ns) { return size_t(W) * warp_bytes(S, cap, ns); }
};

typedef void (*BatchedKernel)(BatchedArgs);

// Kernel of each family for a dim, precision and shape; nullptr when none.
BatchedKernel pick_register(int dim, bool bf16, int vpw, int warps);  // de_batched_reg.cu
BatchedKernel pick_staged(int dim, bool bf16, int steps, int stages, int ctas);  // de_batched_staged.cu
BatchedKernel pick_rows(int dim, bool bf16, int steps, int stages);    // de_batched_rows.cu

}  // namespace batched
}  // namespace de
