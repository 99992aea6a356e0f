// FP32 plain form of the force-model SGD minibatch step (sm_103a).
//
// One launch per minibatch.  A warp owns one work item (a row, or an edge-capped
// piece of a high-degree row).  Each lane holds dim/32 consecutive-ish components
// of a row, so a neighbour row is one coalesced 128-bit load per lane at dim 128.
// Per CSR entry the warp computes the squared distance with a shuffle reduction,
// the t-distribution coefficient and the clipped, scaled force, and accumulates
// it in registers (cpp/algo/algo.hpp:531-582).  The repulsive pass over the
// minibatch's shared negatives (algo.hpp:594-647) and the update
// (algo.hpp:651-666) are fused into the same pass.
//
// Within a minibatch the reference reads only pre-minibatch values (the update
// is applied after both passes).  Here the new rows of minibatch j go to a
// staging buffer S[j % 2]; the launch of minibatch j+1 reads rows of minibatch j
// from that buffer and copies them back into X, so one kernel boundary per
// minibatch is the only synchronisation.
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

__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(kFull, v, o);
  return v;
}

// EmbeddingAlgo::scale (cpp/algo/algo.hpp:65-72).
__device__ __forceinline__ float clip(float v, float b) { return v > b ? b : (v < -b ? -b : v); }

// Row n as the minibatch sees it: rows of the previous minibatch still sit in
// the staging buffer; every other row is current in X.
__device__ __forceinline__ const float *row_ptr(const PlainBatchArgs &a, int n, int D) {
  const unsigned off = unsigned(n - a.prev_base);
  return off < unsigned(a.prev_rows) ? a.S_prev + size_t(off) * D : a.X + size_t(n) * D;
}

template <int D, int U>
__global__ void __launch_bounds__(kPlainWarps * 32) plain_batch_kernel(const PlainBatchArgs a) {
  const int lane = threadIdx.x & 31;
  const int wib = threadIdx.x >> 5;
  const int gw = blockIdx.x * kPlainWarps + wib;
  const int total_w = gridDim.x * kPlainWarps;
  const int epoch = *a.epoch;
  const float lr = a.lr[epoch];
  const float bound = a.bound;

  // Rows of the previous minibatch: staging buffer -> X.  Nothing in this
  // launch reads those rows from X.
  for (int r = gw; r < a.prev_rows; r += total_w) {
    Frag<D> t;
    load_nc(t, a.S_prev + size_t(r) * D, lane);
    store<D, false>(t, a.X + size_t(a.prev_base + r) * D, lane);
  }

  double loss = 0.0;
  if (gw < a.n_items) {
    const WorkItem it = a.items[gw];
    const int row = a.base + it.row;
    Frag<D> xi, acc;
    load_nc(xi, a.X + size_t(row) * D, lane);
    acc.zero();
    const int skip = a.quirks ? a.n - 1 : -1;  // edges into n-1 are dropped (algo.hpp:399-405, 538)

    // ---- attractive pass over this item's CSR entries, in CSR order
    for (int e0 = it.e_begin; e0 < it.e_end; e0 += 32) {
      const int cnt = min(32, it.e_end - e0);
      const int my_col = lane < cnt ? __ldg(a.col + e0 + lane) : -1;
      for (int k = 0; k < cnt; k += U) {
        Frag<D> xn[U];
        int nn[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
          int n = __shfl_sync(kFull, my_col, k + u);
          if (n == skip) n = -1;
          nn[u] = n;
          if (n >= 0) load_nc(xn[u], row_ptr(a, n, D), lane);
        }
#pragma unroll
        for (int u = 0; u < U; ++u) {
          if (nn[u] < 0) continue;  // warp-uniform
          float diff[Frag<D>::N];
          float part = 0.f;
#pragma unroll
          for (int t = 0; t < Frag<D>::N; ++t) {
            diff[t] = xi.v[t] - xn[u].v[t];
            part = fmaf(diff[t], diff[t], part);
          }
          const float r = warp_sum(part);
          const float c = -2.0f / (1.0f + r);
#pragma unroll
          for (int t = 0; t < Frag<D>::N; ++t) acc.v[t] = fmaf(lr, clip(diff[t] * c, bound), acc.v[t]);
          if (a.compute_loss && lane == 0) loss += double(log1pf(r));
        }
      }
    }

    // ---- split rows: the last part to arrive sums all parts in slot order
    bool owner = true;
    if (it.nparts > 1) {
      store<D, true>(acc, a.P + size_t(it.first_slot + it.part) * D, lane);
      __threadfence();
      int old = 0;
      if (lane == 0) old = atomicAdd(a.counters + it.counter, 1);
      old = __shfl_sync(kFull, old, 0);
      owner = (old == it.nparts - 1);
      if (owner) {
        __threadfence();
        acc.zero();
        for (int p = 0; p < it.nparts; ++p) {
          Frag<D> t;
          load_cg(t, a.P + size_t(it.first_slot + p) * D, lane);
#pragma unroll
          for (int q = 0; q < Frag<D>::N; ++q) acc.v[q] += t.v[q];
        }
        if (lane == 0) a.counters[it.counter] = 0;  // ready for the next minibatch
      }
    }

    if (owner) {
      // ---- repulsive pass over the minibatch's shared negatives, in draw order
      const int rep_rows = (a.quirks && epoch + a.epoch[1] > 0) ? a.last_batch_size : a.rows;
      if (it.row < rep_rows) {
        const int32_t *negs = a.negs + (size_t(epoch) * a.batches + a.batch_id) * a.ns;
        for (int k = 0; k < a.ns; ++k) {
          const int n = __ldg(negs + k);
          if (n < 0 || n >= a.n) continue;  // a draw equal to n contributes nothing
          Frag<D> xn;
          load_nc(xn, row_ptr(a, n, D), lane);
          float diff[Frag<D>::N];
          float part = 0.f;
#pragma unroll
          for (int t = 0; t < Frag<D>::N; ++t) {
            diff[t] = xi.v[t] - xn.v[t];
            part = fmaf(diff[t], diff[t], part);
          }
          const float r = warp_sum(part);
          const float c = 2.0f / ((r + 1e-6f) * (1.0f + r));
#pragma unroll
          for (int t = 0; t < Frag<D>::N; ++t) acc.v[t] = fmaf(lr, clip(diff[t] * c, bound), acc.v[t]);
          if (a.compute_loss && lane == 0) loss += double(logf((1.0f + r) / (r + 1e-6f)));
        }
      }
      // ---- update, staged (algo.hpp:651-666)
      Frag<D> out;
#pragma unroll
      for (int t = 0; t < Frag<D>::N; ++t) out.v[t] = xi.v[t] + acc.v[t];
      store<D, false>(out, a.S_cur + size_t(it.row) * D, lane);
    }
  }

  if (a.compute_loss) {
    __shared__ double part_loss[kPlainWarps];
    if (lane == 0) part_loss[wib] = loss;
    __syncthreads();
    if (threadIdx.x == 0) {
      double s = 0.0;
      for (int w = 0; w < kPlainWarps; ++w) s += part_loss[w];
      a.loss_partial[a.loss_off + blockIdx.x] = s;
    }
  }
}

// End of an epoch: write back the last minibatch, reduce the epoch's loss in a
// fixed order, advance the epoch counter.
template <int D>
__global__ void __launch_bounds__(256) flush_kernel(const FlushArgs a) {
  const int lane = threadIdx.x & 31;
  const int gw = blockIdx.x * 8 + (threadIdx.x >> 5);
  const int total_w = gridDim.x * 8;
  for (int r = gw; r < a.last_rows; r += total_w) {
    Frag<D> t;
    load_nc(t, a.S_last + size_t(r) * D, lane);
    store<D, false>(t, a.X + size_t(a.last_base + r) * D, lane);
  }
  if (blockIdx.x != 0) return;
  __shared__ double red[256];
  double s = 0.0;
  if (a.compute_loss)
    for (int64_t i = threadIdx.x; i < a.n_partials; i += 256) s += a.loss_partial[i];
  red[threadIdx.x] = s;
  __syncthreads();
  for (int w = 128; w > 0; w >>= 1) {
    if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    const int e = *a.epoch;
    if (a.compute_loss) a.loss[e] = red[0];
    *a.epoch = e + 1;
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

}  // namespace

cudaError_t launch_plain_batch(int dim, const PlainBatchArgs &a, int grid, cudaStream_t s) {
  const dim3 block(kPlainWarps * 32);
  switch (dim) {
    case 32: plain_batch_kernel<32, 8><<<grid, block, 0, s>>>(a); break;
    case 64: plain_batch_kernel<64, 8><<<grid, block, 0, s>>>(a); break;
    case 128: plain_batch_kernel<128, 8><<<grid, block, 0, s>>>(a); break;
    case 256: plain_batch_kernel<256, 4><<<grid, block, 0, s>>>(a); break;
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

cudaError_t launch_flush(int dim, const FlushArgs &a, cudaStream_t s) {
  const int grid = 152;
  switch (dim) {
    case 32: flush_kernel<32><<<grid, 256, 0, s>>>(a); break;
    case 64: flush_kernel<64><<<grid, 256, 0, s>>>(a); break;
    case 128: flush_kernel<128><<<grid, 256, 0, s>>>(a); break;
    case 256: flush_kernel<256><<<grid, 256, 0, s>>>(a); break;
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
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
