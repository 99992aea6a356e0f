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

#include "de_async.cuh"
#include "de_device.cuh"
#include "de_internal.h"

namespace de {
namespace {

using namespace dev;

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

// Gathers up to U rows named by lanes [k, k+U) of `ids` (one id per lane, -1 =
// none) and applies their forces.  Missing rows get xi (zero force).
template <int D, int U, bool kAttract, bool kAfterWait>
__device__ __forceinline__ void force_group(const PlainBatchArgs &a, Frag<D> &acc, const Frag<D> &xi, int ids,
                                            int k, float lr, float bound, bool want_loss, float &loss,
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

// Forces of the ids held by the warp's lanes (-1 = none), U at a time; a last
// group of at most U/2 entries runs as a group of U/2.
template <int D, int U, bool kAttract, bool kAfterWait>
__device__ __forceinline__ void force_lanes(const PlainBatchArgs &a, Frag<D> &acc, const Frag<D> &xi, int ids,
                                            int cnt, float lr, float bound, bool want_loss, float &loss,
                                            int lane) {
  int k = 0;
  for (; k + U / 2 < cnt; k += U)
    force_group<D, U, kAttract, kAfterWait>(a, acc, xi, ids, k, lr, bound, want_loss, loss, lane);
  if (k < cnt) force_group<D, U / 2, kAttract, kAfterWait>(a, acc, xi, ids, k, lr, bound, want_loss, loss, lane);
}

// A row held in shared memory, in the Frag layout.
template <int D>
__device__ __forceinline__ void load_smem(Frag<D> &f, const float *row, int lane) {
  if constexpr (D == 32) {
    f.v[0] = row[lane];
  } else if constexpr (D == 64) {
    const float2 t = reinterpret_cast<const float2 *>(row)[lane];
    f.v[0] = t.x; f.v[1] = t.y;
  } else {
    const float4 t = reinterpret_cast<const float4 *>(row)[lane];
    f.v[0] = t.x; f.v[1] = t.y; f.v[2] = t.z; f.v[3] = t.w;
    if constexpr (D == 256) {
      const float4 u = reinterpret_cast<const float4 *>(row)[32 + lane];
      f.v[4] = u.x; f.v[5] = u.y; f.v[6] = u.z; f.v[7] = u.w;
    }
  }
}

// Repulsive forces of staged negatives k0 .. k0+V-1 (rows in shared memory;
// draws whose bit in `staged` is clear are left out).
template <int D, int V>
__device__ __forceinline__ void staged_group(Frag<D> &acc, const Frag<D> &xi, const float *negsm, unsigned staged,
                                             int k0, int ns, float lr, float bound, bool want_loss, float &loss,
                                             int lane) {
  Frag<D> xn[V];
  unsigned mask = 0;
#pragma unroll
  for (int u = 0; u < V; ++u) {
    const int k = k0 + u;
    if (k < ns && ((staged >> k) & 1u)) {
      load_smem(xn[u], negsm + k * D, lane);
      mask |= 1u << u;
    } else {
      xn[u] = xi;
    }
  }
  if (mask) pair_forces<D, V, false>(acc, xi, xn, mask, lr, bound, want_loss, loss, lane);
}

template <int D, int U>
__global__ void __launch_bounds__(kPlainWarps * 32, D >= 256 ? 4 : kPlainMinBlocks)
    plain_batch_kernel(const PlainBatchArgs a) {
  extern __shared__ __align__(16) float negsm[];  // stage_negs: [ns, D] rows of the minibatch's draws
  __shared__ __align__(8) uint64_t negbar;
  __shared__ int negerr;
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
  const int skip = a.skip_last ? a.n - 1 : -1;  // edges into n-1 are dropped (algo.hpp:399-405, 538)
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

  // Staged negatives: bit k of `staged`: draw k is a vertex outside minibatch j-1
  // (final before the wait), copied by one thread of the CTA into row k of negsm
  // with bulk asynchronous copies; the CTA waits (bounded) on one barrier.
  unsigned staged = 0;
  if (a.stage_negs) {
    for (int k = 0; k < a.ns; ++k) {
      const int nid = __ldg(negs + k);
      if (nid >= 0 && nid < a.n && !in_prev(a, nid)) staged |= 1u << k;
    }
    const uint32_t bar = smem_u32(&negbar);
    if (threadIdx.x == 0) {
      negerr = 0;
      mbar_init(bar, 1);
      asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
      mbar_expect_tx(bar, uint32_t(__popc(staged)) * D * 4u);
      for (int k = 0; k < a.ns; ++k)
        if ((staged >> k) & 1u)
          bulk_g2s(smem_u32(negsm + k * D), row_ptr<false>(a, __ldg(negs + k), D), D * 4u, bar);
    }
    __syncthreads();
    if (!mbar_wait(bar, 0, &negerr)) {
      if (lane == 0) atomicExch(a.err, 1);
      staged = 0;  // results of this launch are invalid; the host reports the error
    }
  }

  float loss = 0.f;  // this item's loss terms (FP32); the epoch sum is FP64
  Frag<D> xi, acc;
  acc.zero();
  if (has_item) {
    load_nc(xi, a.X + size_t(a.base + it.row) * D, lane);
    // ---- before the wait: forces whose other row is final (CSR order, then draw order)
    force_lanes<D, U, true, false>(a, acc, xi, defer ? -1 : ids, cnt, lr, bound, want_loss, loss, lane);
    if (repulse && a.stage_negs) {
      // the staged rows in draw order, grouped as force_lanes groups them (so the
      // arithmetic, and the result, equal the unstaged path's)
      int k0 = 0;
      for (; k0 + U / 2 < a.ns; k0 += U)
        staged_group<D, U>(acc, xi, negsm, staged, k0, a.ns, lr, bound, want_loss, loss, lane);
      if (k0 < a.ns) staged_group<D, U / 2>(acc, xi, negsm, staged, k0, a.ns, lr, bound, want_loss, loss, lane);
    } else if (repulse)
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
    if (lane == 0) a.loss_partial[a.loss_off + gw] = double(loss);
  }
}

// SpMMAlgo::algo_spmm's step at one rank (cpp/algo/spmm.hpp:54-159):
// y[i] = sum over the CSR entries of row i, in CSR order, of lr * x[col]
// (spmm.hpp:358-392), from the unchanged input x into the output y
// (spmm.hpp:397-412).  The reference goes minibatch by minibatch; the rows do not
// depend on one another, so every work item runs in one launch.  One warp per
// work item, U rows in flight; split rows are combined in piece order as in
// plain_batch_kernel.
template <int D, int U>
__global__ void __launch_bounds__(kPlainWarps * 32, D >= 256 ? 4 : (D == 128 ? 10 : kPlainMinBlocks))
    spmm_kernel(const SpmmArgs a) {
  const int lane = threadIdx.x & 31;
  const int64_t gw = blockIdx.x * int64_t(kPlainWarps) + (threadIdx.x >> 5);
  if (gw >= a.n_items) return;
  const WorkItem it = a.items[gw];
  const int j = it.batch;
  float *const P = a.P + size_t(__ldg(a.slot_off + j)) * D;
  int32_t *const counters = a.counters + __ldg(a.counter_off + j);
  const int cnt = it.e_end - it.e_begin;
  int ids = -1;
  if (lane < cnt) {
    ids = __ldg(a.col + it.e_begin + lane);
    if (ids == a.skip) ids = -1;  // edges into n-1 (spmm.hpp:260-265, 365)
  }
  Frag<D> acc;
  acc.zero();
  for (int k = 0; k < cnt; k += U) {
    Frag<D> xn[U];
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const int n = __shfl_sync(kFull, ids, (k + u) & 31);
      if (k + u < cnt && n >= 0) load_nc(xn[u], a.X + size_t(n) * D, lane);
      else xn[u].zero();
    }
#pragma unroll
    for (int u = 0; u < U; ++u)
#pragma unroll
      for (int t = 0; t < Frag<D>::N; ++t) acc.v[t] = fmaf(a.lr, xn[u].v[t], acc.v[t]);
  }
  bool owner = true;
  if (it.nparts > 1) {
    const int NP = it.nparts;
    const int g = it.part / kCombineGroup;
    const int ng = (NP + kCombineGroup - 1) / kCombineGroup;
    const int gsize = min(kCombineGroup, NP - g * kCombineGroup);
    store<D, true>(acc, P + size_t(it.first_slot + it.part) * D, lane);
    owner = arrive_last(counters + it.counter + g, gsize, lane);
    if (owner) {
      sum_slots(acc, P + size_t(it.first_slot + g * kCombineGroup) * D, gsize, lane);
      if (ng > 1) {
        store<D, true>(acc, P + size_t(it.first_slot + NP + g) * D, lane);
        owner = arrive_last(counters + it.counter + ng, ng, lane);
        if (owner) sum_slots(acc, P + size_t(it.first_slot + NP) * D, ng, lane);
      }
    }
  }
  if (owner) store<D, false>(acc, a.Y + (size_t(j) * a.batch + it.row) * D, lane);
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
cudaError_t launch(void (*k)(Args), int grid, int block, const Args &a, bool pdl, cudaStream_t s, size_t smem = 0) {
  cudaLaunchConfig_t cfg{};
  cfg.gridDim = dim3(grid);
  cfg.blockDim = dim3(block);
  cfg.dynamicSmemBytes = smem;
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
  if (a.stage_negs && a.ns > kStageNegMax) return cudaErrorInvalidValue;
  const size_t smem = a.stage_negs ? size_t(a.ns) * dim * sizeof(float) : 0;
  switch (dim) {
    case 32: return launch(plain_batch_kernel<32, 8>, grid, block, a, pdl, s, smem);
    case 64: return launch(plain_batch_kernel<64, 8>, grid, block, a, pdl, s, smem);
    case 128: return launch(plain_batch_kernel<128, 8>, grid, block, a, pdl, s, smem);
    case 256: return launch(plain_batch_kernel<256, 4>, grid, block, a, pdl, s, smem);
    default: return cudaErrorInvalidValue;
  }
}

cudaError_t launch_spmm(int dim, const SpmmArgs &a, cudaStream_t s) {
  const int64_t grid = (a.n_items + kPlainWarps - 1) / kPlainWarps;
  if (grid == 0) return cudaSuccess;
  if (grid >= (int64_t(1) << 31)) return cudaErrorInvalidValue;
  switch (dim) {
    case 32: spmm_kernel<32, 8><<<unsigned(grid), kPlainWarps * 32, 0, s>>>(a); break;
    case 64: spmm_kernel<64, 8><<<unsigned(grid), kPlainWarps * 32, 0, s>>>(a); break;
    case 128: spmm_kernel<128, 8><<<unsigned(grid), kPlainWarps * 32, 0, s>>>(a); break;
    case 256: spmm_kernel<256, 4><<<unsigned(grid), kPlainWarps * 32, 0, s>>>(a); break;
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
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
