// One minibatch of the FP32 plain embedding step on caller-owned device memory,
// with no device allocation at all.
//
// Who needs this: code that is not allowed to call cudaMalloc / cudaFree.  A host
// framework that owns the whole device heap through its own pool allocator
// (an inference server, another training framework calling this as a plug-in
// operator) cannot let a library allocate behind its back: the memory would be
// invisible to its accounting and fragment its pool.  A latency-bound request
// loop cannot afford the implicit device-wide synchronisation that cudaMalloc
// and cudaFree bring.  Those callers allocate every input and output themselves
// and call this entry point, which only launches kernels.
//
// The only working memory is the file-scope device array below, of a fixed size
// that every GPU loading the library holds until the process exits.  It keeps the
// staged rows of one minibatch (at most kNoAllocMaxRowFloats floats, i.e.
// batch_size * dim <= 1,048,576) and one FP64 loss partial per row.  Both are
// fully rewritten by every call before they are read, so nothing has to start at
// zero; every call shares them, so two calls that overlap on the GPU (different
// streams, or different host threads without ordering) race and corrupt each
// other.
//
// The kernels are the one-warp-per-row form of the plain minibatch kernel:
// attractive pass in CSR order, repulsive pass over the minibatch's negatives
// (cpp/algo/algo.hpp:521-584, 586-649), result staged, then committed to x by a
// second launch (algo.hpp:651-666), so every read in the first launch sees the
// pre-minibatch values as the reference's does.
#include <cuda_runtime.h>

#include <string>

#include "../../include/distembed_gb300.h"

namespace de {
void set_thread_error(const std::string &msg);  // de_runtime.cpp
}

namespace {

constexpr int64_t kNoAllocMaxRowFloats = int64_t(1) << 20;  // 4 MiB of staged rows
constexpr int64_t kNoAllocMaxRows = 65536;                  // loss partials (FP64)
constexpr size_t kNoAllocBytes = size_t(kNoAllocMaxRowFloats) * sizeof(float) + size_t(kNoAllocMaxRows) * sizeof(double);

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocBytes];

constexpr unsigned kFullMask = 0xffffffffu;

struct NoAllocArgs {
  int32_t n;
  const int32_t *rowptr;
  const int32_t *col;
  float *x;
  int32_t base, rows, rep_rows;
  const int32_t *negs;
  int32_t ns;
  int32_t skip;  // column to drop (n - 1 when reproducing the reference), else -1
  float lr, bound;
  float *staged;    // [rows, dim] inside the scratch array
  double *partial;  // [rows] inside the scratch array
  double *loss;     // nullable: this minibatch's loss
};

__device__ __forceinline__ float nclip(float v, float b) { return v > b ? b : (v < -b ? -b : v); }

__device__ __forceinline__ float nwarp_sum(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(kFullMask, v, o);
  return v;
}

// One row per warp; lane l holds components l, l+32, ... of the row.
template <int D, bool kAttract>
__device__ __forceinline__ double nforce(float (&acc)[D / 32], const float (&xi)[D / 32], const float *xn_row,
                                         float lr, float bound, int lane) {
  constexpr int N = D / 32;
  float diff[N];
  float part = 0.f;
#pragma unroll
  for (int t = 0; t < N; ++t) {
    diff[t] = xi[t] - __ldg(xn_row + lane + 32 * t);
    part = fmaf(diff[t], diff[t], part);
  }
  const float r = nwarp_sum(part);
  const float c = kAttract ? -2.0f / (1.0f + r) : 2.0f / ((r + 1e-6f) * (1.0f + r));
#pragma unroll
  for (int t = 0; t < N; ++t) acc[t] = fmaf(lr, nclip(diff[t] * c, bound), acc[t]);
  return kAttract ? double(log1pf(r)) : double(logf((1.0f + r) / (r + 1e-6f)));
}

template <int D>
__global__ void __launch_bounds__(256) noalloc_rows_kernel(const NoAllocArgs a) {
  constexpr int N = D / 32;
  const int lane = threadIdx.x & 31;
  const int r = blockIdx.x * 8 + (threadIdx.x >> 5);
  if (r >= a.rows) return;
  const int row = a.base + r;
  float xi[N], acc[N];
#pragma unroll
  for (int t = 0; t < N; ++t) {
    xi[t] = __ldg(a.x + size_t(row) * D + lane + 32 * t);
    acc[t] = 0.f;
  }
  double loss = 0.0;
  for (int e = __ldg(a.rowptr + row), e1 = __ldg(a.rowptr + row + 1); e < e1; ++e) {
    const int nb = __ldg(a.col + e);
    if (nb == a.skip) continue;
    loss += nforce<D, true>(acc, xi, a.x + size_t(nb) * D, a.lr, a.bound, lane);
  }
  if (r < a.rep_rows)
    for (int k = 0; k < a.ns; ++k) {
      const int nb = __ldg(a.negs + k);
      if (nb < 0 || nb >= a.n) continue;  // a draw equal to n contributes nothing
      loss += nforce<D, false>(acc, xi, a.x + size_t(nb) * D, a.lr, a.bound, lane);
    }
#pragma unroll
  for (int t = 0; t < N; ++t) a.staged[size_t(r) * D + lane + 32 * t] = xi[t] + acc[t];
  if (lane == 0) a.partial[r] = loss;
}

template <int D>
__global__ void __launch_bounds__(256) noalloc_commit_kernel(const NoAllocArgs a) {
  const int64_t total = int64_t(a.rows) * D;
  for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < total; i += int64_t(gridDim.x) * blockDim.x)
    a.x[size_t(a.base) * D + i] = a.staged[i];
  if (blockIdx.x != 0 || a.loss == nullptr) return;
  __shared__ double red[256];
  double s = 0.0;
  for (int i = threadIdx.x; i < a.rows; i += 256) s += a.partial[i];
  red[threadIdx.x] = s;
  __syncthreads();
  for (int w = 128; w > 0; w >>= 1) {
    if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) *a.loss = red[0];
}

// Device address of the scratch array in the current device's context.  It is
// looked up on every call (a lookup allocates nothing): after a device reset, or
// under another context on the same device, the module is loaded again at a new
// address, and a cached address would point at memory of the old context.
int scratch_for_current_device(void **out) {
  void *ptr = nullptr;
  const cudaError_t e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
  if (e != cudaSuccess) {
    de::set_thread_error(std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
    return DE_ERR_CUDA;
  }
  *out = ptr;
  return DE_OK;
}

}  // namespace

extern "C" int de_minibatch_noalloc(int64_t n, const int32_t *rowptr, const int32_t *col, int32_t dim, float *x,
                                    int32_t batch_id, int32_t batch_size, const int32_t *negs, int32_t ns,
                                    int32_t rep_rows, int32_t skip_last_vertex, float lr, float max_bound,
                                    double *loss, void *stream) {
  if (n <= 0 || n >= (int64_t(1) << 31) - 1 || !rowptr || !col || !x || batch_size <= 0 || batch_id < 0 ||
      ns < 0 || (ns > 0 && !negs) || !(max_bound > 0)) {
    de::set_thread_error("de_minibatch_noalloc: bad argument");
    return DE_ERR_INVALID;
  }
  if (dim != 32 && dim != 64 && dim != 128 && dim != 256) {
    de::set_thread_error("de_minibatch_noalloc: dim must be 32, 64, 128 or 256");
    return DE_ERR_INVALID;
  }
  const int64_t base = int64_t(batch_id) * batch_size;
  if (base >= n) {
    de::set_thread_error("de_minibatch_noalloc: batch_id beyond the last minibatch");
    return DE_ERR_INVALID;
  }
  const int64_t rows = (n - base < batch_size) ? n - base : batch_size;
  if (rows * dim > kNoAllocMaxRowFloats || rows > kNoAllocMaxRows) {
    de::set_thread_error("de_minibatch_noalloc: minibatch too large for the fixed scratch: rows * dim must be "
                         "<= 1048576 (e.g. 8192 rows at dim 128)");
    return DE_ERR_INVALID;
  }
  void *scratch = nullptr;
  if (int rc = scratch_for_current_device(&scratch)) return rc;
  NoAllocArgs a{};
  a.n = int32_t(n);
  a.rowptr = rowptr;
  a.col = col;
  a.x = x;
  a.base = int32_t(base);
  a.rows = int32_t(rows);
  a.rep_rows = rep_rows < 0 ? 0 : (rep_rows > rows ? int32_t(rows) : rep_rows);
  a.negs = negs;
  a.ns = ns;
  a.skip = skip_last_vertex ? int32_t(n - 1) : -1;
  a.lr = lr;
  a.bound = max_bound;
  a.staged = static_cast<float *>(scratch);
  a.partial = reinterpret_cast<double *>(static_cast<unsigned char *>(scratch) + kNoAllocMaxRowFloats * sizeof(float));
  a.loss = loss;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const int grid_rows = int((rows + 7) / 8);
  const int grid_commit = int((rows * dim + 255) / 256 < 152 * 4 ? (rows * dim + 255) / 256 : 152 * 4);
  switch (dim) {
    case 32: noalloc_rows_kernel<32><<<grid_rows, 256, 0, s>>>(a); noalloc_commit_kernel<32><<<grid_commit, 256, 0, s>>>(a); break;
    case 64: noalloc_rows_kernel<64><<<grid_rows, 256, 0, s>>>(a); noalloc_commit_kernel<64><<<grid_commit, 256, 0, s>>>(a); break;
    case 128: noalloc_rows_kernel<128><<<grid_rows, 256, 0, s>>>(a); noalloc_commit_kernel<128><<<grid_commit, 256, 0, s>>>(a); break;
    default: noalloc_rows_kernel<256><<<grid_rows, 256, 0, s>>>(a); noalloc_commit_kernel<256><<<grid_commit, 256, 0, s>>>(a); break;
  }
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    de::set_thread_error(std::string("de_minibatch_noalloc launch: ") + cudaGetErrorString(e));
    return DE_ERR_CUDA;
  }
  return DE_OK;
}
