// FP32 plain form of the force-model SGD minibatch step (sm_103a).
//
// One launch per minibatch.  A warp owns one work item (a row, or an edge-capped
// piece of a high-degree row); items are sorted by decreasing cost so the block
// scheduler hands out the long ones first.  Each lane holds dim/32 components of
// a row, so a neighbour row is one coalesced 128-bit load per lane at dim 128.
// Eight neighbour rows are in flight per warp; their eight squared distances are
// reduced together (9 shuffles), each lane turns one of them into the
// t-distribution coefficient and the coefficients are broadcast back (8
// shuffles), then every lane clips and accumulates its components
// (cpp/algo/algo.hpp:531-582).  The repulsive pass over the minibatch's shared
// negatives (algo.hpp:594-647) and the update (algo.hpp:651-666) are fused into
// the same pass.
//
// Within a minibatch the reference reads only pre-minibatch values (the update
// is applied after both passes), and minibatch j+1 must see minibatch j's update
// (algo.hpp:164-192).  Here the new rows of minibatch j go to a staging buffer
// S[j % 3]; launch j+1 copies them back into X, and until that copy is known to
// be complete (two launches later) readers take those rows from S.  Launch j
// runs in two phases around griddepcontrol.wait (programmatic dependent launch):
// before the wait it does every force whose other row is not in minibatch j-1
// (those rows are final), overlapping launch j-1; after the wait it does the
// few forces into minibatch j-1, combines split rows and stores.  Launch j
// releases launch j+1 right after its own wait, so at most two minibatches are
// in flight and launch j+1's early phase only ever reads rows that are final.
#include <cuda_runtime.h>

#include "de_internal.h"

namespace de {
namespace {

constexpr unsigned kFull = 0xffffffffu;

// dim/32 components per lane.  Lane l holds, for dim 32: {l}; 64: {2l, 2l+1};
// 128: {4l..4l+3}; 256: {4l..4l+3, 128+4l..128+4l+3}.
template <int D>
struct Frag {
  static constexpr int N = D / 32;
  float v[N];
  __device__ __forceinline__ void zero() {
#pragma unroll
    for (int i = 0; i < N; ++i) v[i] = 0.f;
  }
};

template <int D>
__device__ __forceinline__ void load_nc(Frag<D> &f, const float *__restrict__ row, int lane) {
  if constexpr (D == 32) {
    f.v[0] = __ldg(row + lane);
  } else if constexpr (D == 64) {
    float2 t = __ldg(reinterpret_cast<const float2 *>(row) + lane);
    f.v[0] = t.x; f.v[1] = t.y;
  } else if constexpr (D == 128) {
    float4 t = __ldg(reinterpret_cast<const float4 *>(row) + lane);
    f.v[0] = t.x; f.v[1] = t.y; f.v[2] = t.z; f.v[3] = t.w;
  } else {
    float4 t = __ldg(reinterpret_cast<const float4 *>(row) + lane);
    float4 u = __ldg(reinterpret_cast<const float4 *>(row) + 32 + lane);
    f.v[0] = t.x; f.v[1] = t.y; f.v[2] = t.z; f.v[3] = t.w;
    f.v[4] = u.x; f.v[5] = u.y; f.v[6] = u.z; f.v[7] = u.w;
  }
}

// L2-coherent load (bypasses L1): partial slots written by other SMs in this launch.
template <int D>
__device__ __forceinline__ void load_cg(Frag<D> &f, const float *row, int lane) {
  if constexpr (D == 32) {
    f.v[0] = __ldcg(row + lane);
  } else if constexpr (D == 64) {
    float2 t = __ldcg(reinterpret_cast<const float2 *>(row) + lane);
    f.v[0] = t.x; f.v[1] = t.y;
  } else if constexpr (D == 128) {
    float4 t = __ldcg(reinterpret_cast<const float4 *>(row) + lane);
    f.v[0] = t.x; f.v[1] = t.y; f.v[2] = t.z; f.v[3] = t.w;
  } else {
    float4 t = __ldcg(reinterpret_cast<const float4 *>(row) + lane);
    float4 u = __ldcg(reinterpret_cast<const float4 *>(row) + 32 + lane);
    f.v[0] = t.x; f.v[1] = t.y; f.v[2] = t.z; f.v[3] = t.w;
    f.v[4] = u.x; f.v[5] = u.y; f.v[6] = u.z; f.v[7] = u.w;
  }
}

template <int D, bool kCg>
__device__ __forceinline__ void store(const Frag<D> &f, float *row, int lane) {
  if constexpr (D == 32) {
    if constexpr (kCg) __stcg(row + lane, f.v[0]); else row[lane] = f.v[0];
  } else if constexpr (D == 64) {
    float2 t = make_float2(f.v[0], f.v[1]);
    if constexpr (kCg) __stcg(reinterpret_cast<float2 *>(row) + lane, t);
    else reinterpret_cast<float2 *>(row)[lane] = t;
  } else if constexpr (D == 128) {
    float4 t = make_float4(f.v[0], f.v[1], f.v[2], f.v[3]);
    if constexpr (kCg) __stcg(reinterpret_cast<float4 *>(row) + lane, t);
    else reinterpret_cast<float4 *>(row)[lane] = t;
  } else {
    float4 t = make_float4(f.v[0], f.v[1], f.v[2], f.v[3]);
    float4 u = make_float4(f.v[4], f.v[5], f.v[6], f.v[7]);
    if constexpr (kCg) {
      __stcg(reinterpret_cast<float4 *>(row) + lane, t);
      __stcg(reinterpret_cast<float4 *>(row) + 32 + lane, u);
    } else {
      reinterpret_cast<float4 *>(row)[lane] = t;
      reinterpret_cast<float4 *>(row)[32 + lane] = u;
    }
  }
}

// Programmatic dependent launch: allow the next kernel in the stream to start
// scheduling, and wait for the previous one to complete with its memory visible.
// Both are no-ops when the launch carries no programmatic dependency.
__device__ __forceinline__ void pdl_trigger() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }

// EmbeddingAlgo::scale (cpp/algo/algo.hpp:65-72).
__device__ __forceinline__ float clip(float v, float b) { return v > b ? b : (v < -b ? -b : v); }

__device__ __forceinline__ bool in_prev(const PlainBatchArgs &a, int n) {
  return unsigned(n - a.prev_base) < unsigned(a.prev_rows);
}

// Row n before the wait (n is not in minibatch j-1): minibatch j-2's rows are
// read from their staging buffer (their copy-back may be in flight), every
// other row is final in X.  After the wait only rows of minibatch j-1 are read,
// from their staging buffer.
template <bool kAfterWait>
__device__ __forceinline__ const float *row_ptr(const PlainBatchArgs &a, int n, int D) {
  if (kAfterWait) return a.S_prev + size_t(n - a.prev_base) * D;
  const unsigned off = unsigned(n - a.prev2_base);
  return off < unsigned(a.prev2_rows) ? a.S_prev2 + size_t(off) * D : a.X + size_t(n) * D;
}

// log2 of the number of values reduced together.
template <int U>
struct Log2 {
  static constexpr int value = U == 8 ? 3 : U == 4 ? 2 : U == 2 ? 1 : 0;
  static_assert((1 << value) == U, "U must be 1, 2, 4 or 8");
};

// Sums U per-lane values over the warp at once.  Level s exchanges half of the
// remaining values across lane bit (4 - s), so after log2(U) levels lane l holds
// a partial of value v(l) (bits 4, 3, ... of l, most significant first); the
// last 5 - log2(U) levels finish that sum.  Lane (u << (5 - log2 U)) ends up
// holding the full sum of value u.
template <int U>
__device__ __forceinline__ float multi_warp_sum(float (&p)[U], int lane) {
  constexpr int L = Log2<U>::value;
#pragma unroll
  for (int s = 0; s < L; ++s) {
    const int m = 16 >> s;
    const int h = U >> (s + 1);
    const bool hi = (lane & m) != 0;
#pragma unroll
    for (int i = 0; i < h; ++i) {
      const float send = hi ? p[i] : p[i + h];
      const float keep = hi ? p[i + h] : p[i];
      p[i] = keep + __shfl_xor_sync(kFull, send, m);
    }
  }
  float r = p[0];
#pragma unroll
  for (int m = 16 >> L; m >= 1; m >>= 1) r += __shfl_xor_sync(kFull, r, m);
  return r;
}

// U pair forces between x_i and rows xn[0..U): valid_mask bit u says whether
// pair u counts (invalid pairs must carry xn[u] == xi).  Attractive:
// c = -2/(1+r); repulsive: c = 2/((r+1e-6)(1+r)) (algo.hpp:573, 626/641).
// Each component is clipped and accumulated in pair order.  The loss term of a
// pair is added on the lane that holds its full sum.
template <int D, int U, bool kAttract>
__device__ __forceinline__ void pair_forces(Frag<D> &acc, const Frag<D> &xi, const Frag<D> (&xn)[U],
                                            unsigned valid_mask, float lr, float bound, bool want_loss,
                                            double &loss, int lane) {
  constexpr int L = Log2<U>::value;
  float diff[U][Frag<D>::N];
  float p[U];
#pragma unroll
  for (int u = 0; u < U; ++u) {
    p[u] = 0.f;
#pragma unroll
    for (int t = 0; t < Frag<D>::N; ++t) {
      diff[u][t] = xi.v[t] - xn[u].v[t];
      p[u] = fmaf(diff[u][t], diff[u][t], p[u]);
    }
  }
  const float r = multi_warp_sum<U>(p, lane);
  const int v = (lane >> (5 - L)) & (U - 1);
  const bool valid = (valid_mask >> v) & 1u;
  float c = kAttract ? -2.0f / (1.0f + r) : 2.0f / ((r + 1e-6f) * (1.0f + r));
  if (!valid) c = 0.f;
  if (want_loss && valid && (lane & ((32 >> L) - 1)) == 0)
    loss += double(kAttract ? log1pf(r) : logf((1.0f + r) / (r + 1e-6f)));
#pragma unroll
  for (int u = 0; u < U; ++u) {
    const float cu = __shfl_sync(kFull, c, u << (5 - L));
#pragma unroll
    for (int t = 0; t < Frag<D>::N; ++t) acc.v[t] = fmaf(lr, clip(diff[u][t] * cu, bound), acc.v[t]);
  }
}

// acc = slot[0] + slot[1] + ... + slot[count-1], in that order; eight loads in flight.
template <int D>
__device__ __forceinline__ void sum_slots(Frag<D> &acc, const float *slot, int count, int lane) {
  acc.zero();
  for (int q0 = 0; q0 < count; q0 += 8) {
    Frag<D> t[8];
#pragma unroll
    for (int u = 0; u < 8; ++u)
      if (q0 + u < count) load_cg(t[u], slot + size_t(q0 + u) * D, lane);
#pragma unroll
    for (int u = 0; u < 8; ++u)
      if (q0 + u < count) {
#pragma unroll
        for (int q = 0; q < Frag<D>::N; ++q) acc.v[q] += t[u].v[q];
      }
  }
}

// Arrival on a split-row counter; true for the last of `expected` arrivals,
// which also re-arms the counter.  The fences order the partial written
// before the arrival against the reads of the last arriver.
__device__ __forceinline__ bool arrive_last(int32_t *counter, int expected, int lane) {
  __threadfence();
  int old = 0;
  if (lane == 0) old = atomicAdd(counter, 1);
  old = __shfl_sync(kFull, old, 0);
  if (old != expected - 1) return false;
  __threadfence();
  if (lane == 0) *counter = 0;
  return true;
}

// Gathers up to U rows named by lanes [k, k+U) of `ids` (one id per lane, -1 =
// none) and applies their forces.  Missing rows get xi (zero force).
template <int D, int U, bool kAttract, bool kAfterWait>
__device__ __forceinline__ void force_group(const PlainBatchArgs &a, Frag<D> &acc, const Frag<D> &xi, int ids,
                                            int k, float lr, float bound, bool want_loss, double &loss,
                                            int lane) {
  Frag<D> xn[U];
  unsigned mask = 0;
#pragma unroll
  for (int u = 0; u < U; ++u) {
    const int n = __shfl_sync(kFull, ids, k + u);
    if (n >= 0) {
      if (kAfterWait) load_cg(xn[u], row_ptr<true>(a, n, D), lane);
      else load_nc(xn[u], row_ptr<false>(a, n, D), lane);
      mask |= 1u << u;
    } else {
      xn[u] = xi;
    }
  }
  if (mask) pair_forces<D, U, kAttract>(acc, xi, xn, mask, lr, bound, want_loss, loss, lane);
}

// Forces of the ids held by the warp's lanes (-1 = none), U at a time.
template <int D, int U, bool kAttract, bool kAfterWait>
__device__ __forceinline__ void force_lanes(const PlainBatchArgs &a, Frag<D> &acc, const Frag<D> &xi, int ids,
                                            int cnt, float lr, float bound, bool want_loss, double &loss,
                                            int lane) {
  for (int k = 0; k < cnt; k += U)
    force_group<D, U, kAttract, kAfterWait>(a, acc, xi, ids, k, lr, bound, want_loss, loss, lane);
}

template <int D, int U>
__global__ void __launch_bounds__(kPlainWarps * 32, D >= 256 ? 4 : kPlainMinBlocks)
    plain_batch_kernel(const PlainBatchArgs a) {
  const int lane = threadIdx.x & 31;
  const int gw = blockIdx.x * kPlainWarps + (threadIdx.x >> 5);
  const int total_w = gridDim.x * kPlainWarps;
  const bool want_loss = a.compute_loss != 0;

  const bool has_item = gw < a.n_items;
  WorkItem it{};
  if (has_item) it = a.items[gw];
  const int epoch = a.epoch[0];
  const float lr = a.lr[epoch];
  const float bound = a.bound;
  const int skip = a.quirks ? a.n - 1 : -1;  // edges into n-1 are dropped (algo.hpp:399-405, 538)
  // this item's CSR entries, one per lane (at most 32)
  const int cnt = has_item ? it.e_end - it.e_begin : 0;
  int ids = -1;
  if (lane < cnt) {
    ids = __ldg(a.col + it.e_begin + lane);
    if (ids == skip) ids = -1;
  }
  const bool defer = ids >= 0 && in_prev(a, ids);
  // the repulsive pass of a row is done by its part 0
  const int rep_rows = (a.quirks && epoch + a.epoch[1] > 0) ? a.last_batch_size : a.rows;
  const bool repulse = has_item && it.part == 0 && it.row < rep_rows;
  const int32_t *negs = a.negs + (size_t(epoch) * a.batches + a.batch_id) * a.ns;

  double loss = 0.0;
  Frag<D> xi, acc;
  acc.zero();
  if (has_item) {
    load_nc(xi, a.X + size_t(a.base + it.row) * D, lane);
    // ---- before the wait: forces whose other row is final (CSR order, then draw order)
    force_lanes<D, U, true, false>(a, acc, xi, defer ? -1 : ids, cnt, lr, bound, want_loss, loss, lane);
    if (repulse)
      for (int k0 = 0; k0 < a.ns; k0 += 32) {
        const int kc = min(32, a.ns - k0);
        int nid = lane < kc ? __ldg(negs + k0 + lane) : -1;
        if (nid >= a.n || (nid >= 0 && in_prev(a, nid))) nid = -1;  // a draw equal to n contributes nothing
        force_lanes<D, U, false, false>(a, acc, xi, nid, kc, lr, bound, want_loss, loss, lane);
      }
  }

  pdl_wait();
  pdl_trigger();

  if (has_item) {
    // ---- after the wait: forces into minibatch j-1
    if (__any_sync(kFull, defer))
      force_lanes<D, U, true, true>(a, acc, xi, defer ? ids : -1, cnt, lr, bound, want_loss, loss, lane);
    if (repulse && a.prev_rows > 0)
      for (int k0 = 0; k0 < a.ns; k0 += 32) {
        const int kc = min(32, a.ns - k0);
        int nid = lane < kc ? __ldg(negs + k0 + lane) : -1;
        if (!(nid >= 0 && nid < a.n && in_prev(a, nid))) nid = -1;
        if (__any_sync(kFull, nid >= 0))
          force_lanes<D, U, false, true>(a, acc, xi, nid, kc, lr, bound, want_loss, loss, lane);
      }

    // ---- split rows: two-level, fixed-order combine of the parts
    bool owner = true;
    if (it.nparts > 1) {
      const int P = it.nparts;
      const int g = it.part / kCombineGroup;
      const int ng = (P + kCombineGroup - 1) / kCombineGroup;
      const int gsize = min(kCombineGroup, P - g * kCombineGroup);
      store<D, true>(acc, a.P + size_t(it.first_slot + it.part) * D, lane);
      owner = arrive_last(a.counters + it.counter + g, gsize, lane);
      if (owner) {
        sum_slots(acc, a.P + size_t(it.first_slot + g * kCombineGroup) * D, gsize, lane);
        if (ng > 1) {
          store<D, true>(acc, a.P + size_t(it.first_slot + P + g) * D, lane);
          owner = arrive_last(a.counters + it.counter + ng, ng, lane);
          if (owner) sum_slots(acc, a.P + size_t(it.first_slot + P) * D, ng, lane);
        }
      }
    }
    // ---- update, staged (algo.hpp:651-666)
    if (owner) {
      Frag<D> out;
#pragma unroll
      for (int t = 0; t < Frag<D>::N; ++t) out.v[t] = xi.v[t] + acc.v[t];
      store<D, false>(out, a.S_cur + size_t(it.row) * D, lane);
    }
  }

  // Rows of minibatch j-1: staging buffer -> X.  Until the next launch passes
  // its wait, every reader takes these rows from the staging buffer.
  for (int r = gw; r < a.prev_rows; r += total_w) {
    Frag<D> t;
    load_cg(t, a.S_prev + size_t(r) * D, lane);
    store<D, false>(t, a.X + size_t(a.prev_base + r) * D, lane);
  }

  if (want_loss && has_item) {
#pragma unroll
    for (int m = 16; m >= 1; m >>= 1) loss += __shfl_xor_sync(kFull, loss, m);
    if (lane == 0) a.loss_partial[a.loss_off + gw] = loss;
  }
}

// End of an epoch: write back the last minibatch, reduce the epoch's loss
// partials in a fixed order (each CTA a fixed chunk, then the last CTA to
// finish sums the chunk sums in order), advance the epoch counter.
template <int D>
__global__ void __launch_bounds__(256) flush_kernel(const FlushArgs a) {
  const int lane = threadIdx.x & 31;
  const int gw = blockIdx.x * 8 + (threadIdx.x >> 5);
  const int total_w = gridDim.x * 8;
  pdl_wait();
  for (int r = gw; r < a.last_rows; r += total_w) {
    Frag<D> t;
    load_nc(t, a.S_last + size_t(r) * D, lane);
    store<D, false>(t, a.X + size_t(a.last_base + r) * D, lane);
  }
  __shared__ double red[256];
  __shared__ bool last;
  double s = 0.0;
  if (a.compute_loss) {
    const int64_t chunk = (a.n_partials + gridDim.x - 1) / gridDim.x;
    const int64_t lo = blockIdx.x * chunk, hi = min(a.n_partials, lo + chunk);
    for (int64_t i = lo + threadIdx.x; i < hi; i += 256) s += a.loss_partial[i];
  }
  red[threadIdx.x] = s;
  __syncthreads();
  for (int w = 128; w > 0; w >>= 1) {
    if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    a.block_sums[blockIdx.x] = red[0];
    __threadfence();
    last = atomicAdd(a.done, 1) == int(gridDim.x) - 1;
  }
  __syncthreads();
  if (!last) return;
  __threadfence();
  s = 0.0;
  for (int b = threadIdx.x; b < int(gridDim.x); b += 256) s += __ldcg(a.block_sums + b);
  red[threadIdx.x] = s;
  __syncthreads();
  for (int w = 128; w > 0; w >>= 1) {
    if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    const int e = a.epoch[0];
    if (a.compute_loss) a.loss[e] = red[0];
    a.epoch[0] = e + 1;
    *a.done = 0;
  }
}

__global__ void f64_to_f32_kernel(const double *__restrict__ s, float *__restrict__ d, int64_t n) {
  for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x)
    d[i] = float(s[i]);
}

__global__ void f32_to_f64_kernel(const float *__restrict__ s, double *__restrict__ d, int64_t n) {
  for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x)
    d[i] = double(s[i]);
}

template <typename Args>
cudaError_t launch(void (*k)(Args), int grid, int block, const Args &a, bool pdl, cudaStream_t s) {
  cudaLaunchConfig_t cfg{};
  cfg.gridDim = dim3(grid);
  cfg.blockDim = dim3(block);
  cfg.dynamicSmemBytes = 0;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = pdl ? 1 : 0;
  return cudaLaunchKernelEx(&cfg, k, a);
}

}  // namespace

cudaError_t launch_plain_batch(int dim, const PlainBatchArgs &a, int grid, bool pdl, cudaStream_t s) {
  const int block = kPlainWarps * 32;
  switch (dim) {
    case 32: return launch(plain_batch_kernel<32, 8>, grid, block, a, pdl, s);
    case 64: return launch(plain_batch_kernel<64, 8>, grid, block, a, pdl, s);
    case 128: return launch(plain_batch_kernel<128, 8>, grid, block, a, pdl, s);
    case 256: return launch(plain_batch_kernel<256, 4>, grid, block, a, pdl, s);
    default: return cudaErrorInvalidValue;
  }
}

cudaError_t launch_flush(int dim, const FlushArgs &a, bool pdl, cudaStream_t s) {
  switch (dim) {
    case 32: return launch(flush_kernel<32>, kFlushBlocks, 256, a, pdl, s);
    case 64: return launch(flush_kernel<64>, kFlushBlocks, 256, a, pdl, s);
    case 128: return launch(flush_kernel<128>, kFlushBlocks, 256, a, pdl, s);
    case 256: return launch(flush_kernel<256>, kFlushBlocks, 256, a, pdl, s);
    default: return cudaErrorInvalidValue;
  }
}

cudaError_t launch_f64_to_f32(const double *src, float *dst, int64_t count, cudaStream_t s) {
  if (count <= 0) return cudaSuccess;
  const int grid = int(count / 256 + 1 < 152 * 8 ? count / 256 + 1 : 152 * 8);
  f64_to_f32_kernel<<<grid, 256, 0, s>>>(src, dst, count);
  return cudaGetLastError();
}

cudaError_t launch_f32_to_f64(const float *src, double *dst, int64_t count, cudaStream_t s) {
  if (count <= 0) return cudaSuccess;
  const int grid = int(count / 256 + 1 < 152 * 8 ? count / 256 + 1 : 152 * 8);
  f32_to_f64_kernel<<<grid, 256, 0, s>>>(src, dst, count);
  return cudaGetLastError();
}

}  // namespace de
