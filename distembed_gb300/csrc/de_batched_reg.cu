// Batched form, register kernel: a warp runs vertices_per_warp work items at once
// on 32 / vertices_per_warp lanes each, neighbour rows loaded into registers.
#include "de_batched.cuh"

namespace de {
namespace batched {
namespace {

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

// Forces of up to 4 rows named by lanes [k, k+4) of the group (ids < 0: none),
// all groups of the warp in step (the caller keeps the warp converged).  xi is the
// row's FP32 master value.  In the BF16 form the rows are read as BF16; a pair
// whose squared distance from those reads is below a.near_r is read again from
// the FP32 master and recomputed, so that the rounding of the copy does not bias
// close pairs (their distance is then comparable with the BF16 rounding step).
template <int D, int VPW, bool kBF16, bool kAttract>
__device__ __forceinline__ void group_forces(const BatchedArgs &a, Row<D, VPW> &acc, const Row<D, VPW> &xi,
                                             int64_t voff, int ids, int k, int gbase, int gl, float lr,
                                             float &loss, bool want) {
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
    if (want && nid[u] >= 0 && gl == 0) loss += kAttract ? log1pf(r[u]) : logf((1.0f + r[u]) / (r[u] + 1e-6f));
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
      const bool want = a.compute_loss && e >= a.loss_from;
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
              group_forces<D, VPW, kBF16, true>(a, acc, xi, G.voff, ids, k, gbase, gl, lr, loss, want);
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
              group_forces<D, VPW, kBF16, false>(a, acc, xi, G.voff, ids, k, gbase, gl, lr, loss, want);
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

}  // namespace

BatchedKernel pick_register(int dim, bool bf16, int vpw, int warps) {
  switch (dim) {
    case 32: return bf16 ? pick<32, true>(vpw, warps) : pick<32, false>(vpw, warps);
    case 64: return bf16 ? pick<64, true>(vpw, warps) : pick<64, false>(vpw, warps);
    case 128: return bf16 ? pick<128, true>(vpw, warps) : pick<128, false>(vpw, warps);
  }
  return nullptr;
}


}  // namespace batched
}  // namespace de
