// Sparse embedding (SparseEmbedding::algo_sparse_embedding at one rank,
// cpp/algo/sparse_embedding.hpp:78-194).  An embedding row is a dense FP64
// vector in which INT_MIN marks an absent entry (the reference's dense
// collector, cpp/core/sparse_mat.hpp:367-377, 492-505).  The pair term walks
// the union of the two rows' present entries (sparse_embedding.hpp:380-427,
// 548-598): value x_i - x_j, x_i or -x_j, r = sum of value^2, an update on
// every union entry.  With absent entries read as 0 this is the dense pair
// term: a dim absent from both rows adds 0 to r and 0 to the update.  So the
// kernels read an FP32 mirror of the rows that holds 0 for absent entries and
// reuse the dense pair arithmetic (dev::pair_forces); the FP64 rows keep the
// reference's values, and the top-k pruning compares them exactly.
#include <cuda_runtime.h>

#include <cstdint>

#include "de_device.cuh"
#include "de_internal.h"

namespace de {
namespace {

using dev::Frag;
using dev::kFull;

constexpr uint64_t kAbsent64 = 0xC1E0000000000000ull;  // bits of (double)INT_MIN
constexpr int kWarps = 8;

int elementwise_grid(int64_t count) { return int(count / 256 + 1 < 152 * 8 ? count / 256 + 1 : 152 * 8); }

// The attractive pass of every minibatch of one iteration in one launch (the
// one-rank branch never merges its updates, so no row changes during the
// iteration): one warp per work item, U neighbours in flight, split rows
// combined in piece order.  Row i's update goes to Y[i] (FP32, from zero).  The
// launch is hundreds of thousands of warps, so resident warps hide the gather's
// latency: at dim 128 the kernel is held to 48 registers for five CTAs per SM.
template <int D, int U>
__global__ void __launch_bounds__(kWarps * 32, D == 128 ? 5 : 1) sparse_attract_kernel(const SpmmArgs a) {
  const int lane = threadIdx.x & 31;
  const int64_t gw = blockIdx.x * int64_t(kWarps) + (threadIdx.x >> 5);
  if (gw >= a.n_items) return;
  const WorkItem it = a.items[gw];
  const int j = it.batch;
  float *const P = a.P + size_t(__ldg(a.slot_off + j)) * D;
  int32_t *const counters = a.counters + __ldg(a.counter_off + j);
  const int64_t row = int64_t(j) * a.batch + it.row;
  Frag<D> xi, acc;
  dev::load_nc(xi, a.X + size_t(row) * D, lane);
  acc.zero();
  float unused_loss = 0.f;
  const int cnt = it.e_end - it.e_begin;
  for (int k0 = 0; k0 < cnt; k0 += 32) {
    const int ids = k0 + lane < cnt ? __ldg(a.col + it.e_begin + k0 + lane) : -1;
    const int kn = min(32, cnt - k0);
    for (int k = 0; k < kn; k += U) {
      Frag<D> xn[U];
      unsigned valid = 0;
#pragma unroll
      for (int u = 0; u < U; ++u) {
        const int nb = __shfl_sync(kFull, ids, (k + u) & 31);
        if (k + u < kn) {
          dev::load_nc(xn[u], a.X + size_t(nb) * D, lane);
          valid |= 1u << u;
        } else {
          xn[u] = xi;
        }
      }
      dev::pair_forces<D, U, true>(acc, xi, xn, valid, a.lr, a.bound, false, unused_loss, lane);
    }
  }
  bool owner = true;
  if (it.nparts > 1) {
    const int NP = it.nparts;
    const int g = it.part / kCombineGroup;
    const int ng = (NP + kCombineGroup - 1) / kCombineGroup;
    const int gsize = min(kCombineGroup, NP - g * kCombineGroup);
    dev::store<D, true>(acc, P + size_t(it.first_slot + it.part) * D, lane);
    owner = dev::arrive_last(counters + it.counter + g, gsize, lane);
    if (owner) {
      dev::sum_slots(acc, P + size_t(it.first_slot + g * kCombineGroup) * D, gsize, lane);
      if (ng > 1) {
        dev::store<D, true>(acc, P + size_t(it.first_slot + NP + g) * D, lane);
        owner = dev::arrive_last(counters + it.counter + ng, ng, lane);
        if (owner) dev::sum_slots(acc, P + size_t(it.first_slot + NP) * D, ng, lane);
      }
    }
  }
  if (owner) dev::store<D, false>(acc, a.Y + size_t(row) * D, lane);
}

// Batch collector: slot r of minibatch j holds row jB + r, and the one-rank
// branch adds every minibatch into the same slots without clearing them
// (sparse_embedding.hpp:452-455, 380-386): coll[r] += Y[r] + Y[B + r] + ..., in
// minibatch order.  The terms are FP32 (the rows' updates); their running sum is
// kept as an unevaluated FP32 pair hi + lo (Knuth's TwoSum adds each term with
// its rounding error carried in lo, about 44 bits of precision), then added to
// the FP64 collector once: two FP64 operations per slot instead of two per term
// on the GPU's narrow FP64 pipe.
__global__ void __launch_bounds__(256)
    sparse_collect_kernel(const float *__restrict__ y, double *__restrict__ coll, int64_t n, int32_t batch,
                          int32_t dim) {
  const int64_t slots = int64_t(batch) * dim;
  for (int64_t e = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; e < slots; e += int64_t(gridDim.x) * blockDim.x) {
    const int64_t r = e / dim;
    const float *yp = y + r * dim + (e - r * dim);
    const int64_t stride = int64_t(batch) * dim;
    const int64_t rows = (n - r + batch - 1) / batch;  // rows r, r + B, ... below n
    float hi = 0.f, lo = 0.f;
    auto add = [&](float v) {
      const float s = __fadd_rn(hi, v);
      const float bv = __fsub_rn(s, hi);
      const float err = __fadd_rn(__fsub_rn(hi, __fsub_rn(s, bv)), __fsub_rn(v, bv));
      hi = s;
      lo = __fadd_rn(lo, err);
    };
    int64_t q = 0;
    for (; q + 8 <= rows; q += 8) {  // eight loads in flight, added in order
      float v[8];
#pragma unroll
      for (int u = 0; u < 8; ++u) v[u] = __ldg(yp + (q + u) * stride);
#pragma unroll
      for (int u = 0; u < 8; ++u) add(v[u]);
    }
    for (; q < rows; ++q) add(__ldg(yp + q * stride));
    coll[e] = coll[e] + (double(hi) + double(lo));
  }
}

// FP32 mirror: 0 for an absent entry, the value rounded to FP32 otherwise.
__global__ void __launch_bounds__(256) sparse_mirror_kernel(const double *__restrict__ x64, float *__restrict__ x32,
                                                            int64_t count) {
  for (int64_t e = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; e < count; e += int64_t(gridDim.x) * blockDim.x) {
    const double v = x64[e];
    x32[e] = __double_as_longlong(v) == int64_t(kAbsent64) ? 0.f : float(v);
  }
}

// Rows in: x64 = src and its mirror x32 in one pass over src (device memory, or
// pinned host memory read over the host link); two entries per thread step.
__global__ void __launch_bounds__(256) sparse_load_kernel(const double2 *__restrict__ src, double2 *__restrict__ x64,
                                                          float2 *__restrict__ x32, int64_t pairs) {
  for (int64_t e = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; e < pairs; e += int64_t(gridDim.x) * blockDim.x) {
    const double2 v = src[e];
    x64[e] = v;
    x32[e] = make_float2(__double_as_longlong(v.x) == int64_t(kAbsent64) ? 0.f : float(v.x),
                         __double_as_longlong(v.y) == int64_t(kAbsent64) ? 0.f : float(v.y));
  }
}

// Rows out: dst = src, two entries per thread step (dst: pinned host memory).
__global__ void __launch_bounds__(256) sparse_store_kernel(const double2 *__restrict__ src, double2 *__restrict__ dst,
                                                           int64_t pairs) {
  for (int64_t e = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; e < pairs; e += int64_t(gridDim.x) * blockDim.x)
    dst[e] = src[e];
}

// Present entries (value != INT_MIN) of the FP64 rows, added to *present.
__global__ void __launch_bounds__(256) sparse_count_kernel(const double *__restrict__ x64, int64_t count,
                                                           unsigned long long *present) {
  unsigned long long c = 0;
  for (int64_t e = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; e < count; e += int64_t(gridDim.x) * blockDim.x)
    c += __double_as_longlong(x64[e]) != int64_t(kAbsent64);
  for (int m = 16; m >= 1; m >>= 1) c += __shfl_xor_sync(kFull, c, m);
  __shared__ unsigned long long part[8];
  if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = c;
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned long long t = 0;
    for (int w = 0; w < int(blockDim.x >> 5); ++w) t += part[w];
    atomicAdd(present, t);
  }
}

// Order-preserving integer keys: a < b as floating-point values (with -0 = +0)
// iff key(a) < key(b).  INT_MIN, the absent marker, orders below every value
// of an embedding.
__device__ __forceinline__ uint64_t order_key(double v) {
  uint64_t b = uint64_t(__double_as_longlong(v));
  if (b == 0x8000000000000000ull) b = 0;  // -0 -> +0
  return (b >> 63) ? ~b : (b | 0x8000000000000000ull);
}
__device__ __forceinline__ uint64_t order_key(float v) {
  uint32_t b = __float_as_uint(v);
  if (b == 0x80000000u) b = 0;
  return (b >> 31) ? uint64_t(~b) : uint64_t(b | 0x80000000u);
}

// Top-k pruning (preserveHighestK, sparse_embedding.hpp:745-767): in every row
// the dim - keep smallest values become absent; at equal values the lower dim
// goes first.  One warp per row, lane l holding dims [lN, lN + N): a bitonic
// sort of the row's (key, dim) pairs in registers (partners across lanes by
// shuffle, within a lane directly), after which sorted position p < dim - keep
// names a dim to drop.  When half the row is dropped (density 0.5) the first
// step of the last merge already puts the D/2 smallest pairs below position
// D/2, and the remaining steps, which only order the halves, are skipped.
// T = double: the FP64 rows (absent = INT_MIN) and their mirror; T = float: the
// mirror alone.  With `present` set the rows are pruned only when
// floor(present / n) > keep (sparse_embedding.hpp:172-181), decided
// here so that the host need not wait.
template <int D, typename T>
__global__ void __launch_bounds__(256) sparse_prune_kernel(T *xs, float *x32, int64_t n, int32_t keep,
                                                           const unsigned long long *present) {
  constexpr int N = D / 32;
  if (present && static_cast<int>(double(*present) / double(n)) <= keep) return;
  const int lane = threadIdx.x & 31;
  const int nullify = D - keep;
  for (int64_t row = blockIdx.x * int64_t(blockDim.x >> 5) + (threadIdx.x >> 5); row < n;
       row += int64_t(gridDim.x) * (blockDim.x >> 5)) {
    T *xr = xs + row * D;
    uint64_t key[N];
    int idx[N];
#pragma unroll
    for (int t = 0; t < N; ++t) {
      idx[t] = lane * N + t;
      key[t] = order_key(xr[idx[t]]);
    }
#pragma unroll
    for (int k = 2; k <= D; k <<= 1) {
#pragma unroll
      for (int j = k >> 1; j > 0; j >>= 1) {
        uint64_t pk[N];
        int pi[N];
#pragma unroll
        for (int t = 0; t < N; ++t) {
          if (j >= N) {
            pk[t] = __shfl_xor_sync(kFull, key[t], j / N);
            pi[t] = __shfl_xor_sync(kFull, idx[t], j / N);
          } else {
            pk[t] = key[t ^ j];
            pi[t] = idx[t ^ j];
          }
        }
#pragma unroll
        for (int t = 0; t < N; ++t) {
          const int i = lane * N + t;
          const bool keep_min = ((i & j) == 0) == ((i & k) == 0);
          const bool p_less = pk[t] < key[t] || (pk[t] == key[t] && pi[t] < idx[t]);
          if (keep_min == p_less) {
            key[t] = pk[t];
            idx[t] = pi[t];
          }
        }
        if (k == D && j == D / 2 && nullify == D / 2) break;
      }
    }
#pragma unroll
    for (int t = 0; t < N; ++t)
      if (lane * N + t < nullify) {
        if constexpr (sizeof(T) == 8) {
          xr[idx[t]] = __longlong_as_double(int64_t(kAbsent64));
          x32[row * D + idx[t]] = 0.f;
        } else {
          xr[idx[t]] = 0.f;  // xs is the mirror itself
        }
      }
  }
}

// After the last iteration absent entries become 0 (the final CSR build with
// clear_dense_collector, cpp/core/distributed_mat.hpp:63-91).
// Two entries per thread step; a pair is written back only when it held one.
__global__ void __launch_bounds__(256) sparse_finalize_kernel(double2 *__restrict__ x64, int64_t pairs) {
  for (int64_t e = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; e < pairs; e += int64_t(gridDim.x) * blockDim.x) {
    double2 v = x64[e];
    const bool ax = __double_as_longlong(v.x) == int64_t(kAbsent64);
    const bool ay = __double_as_longlong(v.y) == int64_t(kAbsent64);
    if (ax) v.x = 0.0;
    if (ay) v.y = 0.0;
    if (ax || ay) x64[e] = v;
  }
}

template <typename T>
cudaError_t prune_dispatch(int dim, T *xs, float *x32, int64_t n, int32_t keep, const unsigned long long *present,
                           cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  const int grid = int(n / 8 + 1 < 152 * 16 ? n / 8 + 1 : 152 * 16);
  switch (dim) {
    case 32: sparse_prune_kernel<32, T><<<grid, 256, 0, s>>>(xs, x32, n, keep, present); break;
    case 64: sparse_prune_kernel<64, T><<<grid, 256, 0, s>>>(xs, x32, n, keep, present); break;
    case 128: sparse_prune_kernel<128, T><<<grid, 256, 0, s>>>(xs, x32, n, keep, present); break;
    case 256: sparse_prune_kernel<256, T><<<grid, 256, 0, s>>>(xs, x32, n, keep, present); break;
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

}  // namespace

cudaError_t launch_sparse_attract(int dim, const SpmmArgs &a, cudaStream_t s) {
  const int64_t grid = (a.n_items + kWarps - 1) / kWarps;
  if (grid == 0) return cudaSuccess;
  if (grid >= (int64_t(1) << 31)) return cudaErrorInvalidValue;
  switch (dim) {
    case 32: sparse_attract_kernel<32, 8><<<unsigned(grid), kWarps * 32, 0, s>>>(a); break;
    case 64: sparse_attract_kernel<64, 8><<<unsigned(grid), kWarps * 32, 0, s>>>(a); break;
    case 128: sparse_attract_kernel<128, 4><<<unsigned(grid), kWarps * 32, 0, s>>>(a); break;
    case 256: sparse_attract_kernel<256, 2><<<unsigned(grid), kWarps * 32, 0, s>>>(a); break;
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

cudaError_t launch_sparse_collect(const float *y, double *coll, int64_t n, int32_t batch, int32_t dim,
                                  cudaStream_t s) {
  const int64_t slots = int64_t(batch) * dim;
  if (slots <= 0) return cudaSuccess;
  sparse_collect_kernel<<<elementwise_grid(slots), 256, 0, s>>>(y, coll, n, batch, dim);
  return cudaGetLastError();
}

cudaError_t launch_sparse_mirror(const double *x64, float *x32, int64_t count, cudaStream_t s) {
  if (count <= 0) return cudaSuccess;
  sparse_mirror_kernel<<<elementwise_grid(count), 256, 0, s>>>(x64, x32, count);
  return cudaGetLastError();
}

cudaError_t launch_sparse_load(const double *src, double *x64, float *x32, int64_t count, cudaStream_t s) {
  if (count <= 0) return cudaSuccess;
  if ((count & 1) || (reinterpret_cast<uintptr_t>(src) & 15)) return cudaErrorInvalidValue;
  sparse_load_kernel<<<elementwise_grid(count / 2), 256, 0, s>>>(
      reinterpret_cast<const double2 *>(src), reinterpret_cast<double2 *>(x64), reinterpret_cast<float2 *>(x32),
      count / 2);
  return cudaGetLastError();
}

cudaError_t launch_sparse_store(const double *src, double *dst, int64_t count, cudaStream_t s) {
  if (count <= 0) return cudaSuccess;
  if ((count & 1) || (reinterpret_cast<uintptr_t>(dst) & 15)) return cudaErrorInvalidValue;
  sparse_store_kernel<<<elementwise_grid(count / 2), 256, 0, s>>>(reinterpret_cast<const double2 *>(src),
                                                                  reinterpret_cast<double2 *>(dst), count / 2);
  return cudaGetLastError();
}

cudaError_t launch_sparse_count(const double *x64, int64_t count, unsigned long long *present, cudaStream_t s) {
  if (count <= 0) return cudaSuccess;
  sparse_count_kernel<<<elementwise_grid(count), 256, 0, s>>>(x64, count, present);
  return cudaGetLastError();
}

cudaError_t launch_sparse_prune_f64(int dim, double *x64, float *x32, int64_t n, int32_t keep,
                                    const unsigned long long *present, cudaStream_t s) {
  return prune_dispatch<double>(dim, x64, x32, n, keep, present, s);
}

cudaError_t launch_sparse_prune_f32(int dim, float *x32, int64_t n, int32_t keep, cudaStream_t s) {
  return prune_dispatch<float>(dim, x32, x32, n, keep, nullptr, s);
}

cudaError_t launch_sparse_finalize(double *x64, int64_t count, cudaStream_t s) {
  if (count <= 0) return cudaSuccess;
  if (count & 1) return cudaErrorInvalidValue;  // n x dim with dim a multiple of 32
  sparse_finalize_kernel<<<elementwise_grid(count / 2), 256, 0, s>>>(reinterpret_cast<double2 *>(x64), count / 2);
  return cudaGetLastError();
}

}  // namespace de
