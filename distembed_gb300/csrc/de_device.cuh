// Device helpers shared by the embedding kernels (FP32 plain and BF16 forms).
#pragma once
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include "de_internal.h"

namespace de {
namespace dev {

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

// Packed FP32 pair arithmetic (Blackwell f32x2 FMA: two lanes of work per
// instruction).  sub2(a, b) = a - b exactly as a scalar subtraction rounds it.
__device__ __forceinline__ float2 sub2(float2 a, float2 b) { return __ffma2_rn(b, make_float2(-1.f, -1.f), a); }

// U pair forces between x_i and rows xn[0..U): valid_mask bit u says whether
// pair u counts (invalid pairs must carry xn[u] == xi).  Attractive:
// c = -2/(1+r); repulsive: c = 2/((r+1e-6)(1+r)) (algo.hpp:573, 626/641).
// Each component is clipped (algo.hpp:65-72) and accumulated in pair order.
// Clip-free fast path: |c (x_d - n_d)| <= |c| sqrt(r), so no component can reach
// the bound when c^2 r <= bound^2 and the clip is the identity.  For the
// attractive force |c| sqrt(r) = 2 sqrt(r) / (1 + r) <= 1, so any bound >= 1
// never clips; for repulsion the warp takes the clipped path when any of its
// pairs has c^2 r above 0.98 bound^2.  The loss term of a pair is added on the
// lane that holds its full sum (FP32 within one work item; the caller folds it
// into the FP64 epoch sum).
template <int D, int U, bool kAttract>
__device__ __forceinline__ void pair_forces(Frag<D> &acc, const Frag<D> &xi, const Frag<D> (&xn)[U],
                                            unsigned valid_mask, float lr, float bound, bool want_loss,
                                            float &loss, int lane) {
  constexpr int L = Log2<U>::value;
  constexpr int N = Frag<D>::N;
  float diff[U][N];
  float p[U];
#pragma unroll
  for (int u = 0; u < U; ++u) {
    if constexpr (N >= 2) {
      float2 q = make_float2(0.f, 0.f);
#pragma unroll
      for (int t = 0; t < N; t += 2) {
        const float2 d = sub2(make_float2(xi.v[t], xi.v[t + 1]), make_float2(xn[u].v[t], xn[u].v[t + 1]));
        diff[u][t] = d.x;
        diff[u][t + 1] = d.y;
        q = __ffma2_rn(d, d, q);
      }
      p[u] = q.x + q.y;
    } else {
      diff[u][0] = xi.v[0] - xn[u].v[0];
      p[u] = diff[u][0] * diff[u][0];
    }
  }
  const float r = multi_warp_sum<U>(p, lane);
  const int v = (lane >> (5 - L)) & (U - 1);
  const bool valid = (valid_mask >> v) & 1u;
  float c = kAttract ? __fdividef(-2.0f, 1.0f + r) : __fdividef(2.0f, (r + 1e-6f) * (1.0f + r));
  if (!valid) c = 0.f;
  if (want_loss && valid && (lane & ((32 >> L) - 1)) == 0)
    loss += kAttract ? log1pf(r) : logf((1.0f + r) / (r + 1e-6f));
  const bool no_clip = kAttract ? bound >= 1.0f : !__any_sync(kFull, c * c * r > 0.98f * bound * bound);
  if (no_clip) {
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const float lc = lr * __shfl_sync(kFull, c, u << (5 - L));
      if constexpr (N >= 2) {
#pragma unroll
        for (int t = 0; t < N; t += 2) {
          const float2 o = __ffma2_rn(make_float2(lc, lc), make_float2(diff[u][t], diff[u][t + 1]),
                                      make_float2(acc.v[t], acc.v[t + 1]));
          acc.v[t] = o.x;
          acc.v[t + 1] = o.y;
        }
      } else {
        acc.v[0] = fmaf(lc, diff[u][0], acc.v[0]);
      }
    }
  } else {
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const float cu = __shfl_sync(kFull, c, u << (5 - L));
#pragma unroll
      for (int t = 0; t < N; ++t) acc.v[t] = fmaf(lr, clip(diff[u][t] * cu, bound), acc.v[t]);
    }
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

}  // namespace dev
}  // namespace de
