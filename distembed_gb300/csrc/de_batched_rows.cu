#include "de_batched.cuh"

namespace de {
namespace batched {
namespace {

// ---------------------------------------------------------------- staged rows kernel
//
// The staged pipeline with a work item per lane group: the D/8 lanes of group q
// own item q of the warp's chunk (G = 32/(D/8) items per chunk) and step through
// its CSR entries, then its negatives, one pair per group per warp step.  A row
// is accumulated inside its group (no cross-group sum), no pair slot is computed
// for nothing beyond the differences in length of the G items (they are adjacent
// in cost order), and the per-chunk costs are shared by G items.  Shared memory
// per warp: S ring slots of G sub-slots (own row FP32, cap neighbour rows, their
// ids), the minibatch's negatives, 32 work items.

// NS warp steps s0 .. s0+NS-1 of every group: group q pairs its xi with row s of
// `rows` (stride row_bytes) when s < cnt; valid(s) says whether the pair counts;
// gid(s) is the pair's global row (close-pair recompute in the BF16 form).
template <int D, int NS, bool kBF16, bool kAttract, class Valid, class Gid>
__device__ __forceinline__ void rows_steps(const BatchedArgs &a, float (&acc)[8], const float (&xi)[8],
                                           const unsigned char *rows, int row_bytes, int s0, int cnt, Valid valid,
                                           Gid gid, int64_t voff, float lr, float &loss, bool want, int gl) {
  constexpr int LP = D / 8;
  float d[NS][8], r[NS];
  bool ok[NS];
#pragma unroll
  for (int st = 0; st < NS; ++st) {
    const int sidx = s0 + st;
    const bool in = sidx < cnt;
    float xn[8];
    if (in) {
      ld8<kBF16>(xn, rows + sidx * row_bytes, gl);
    } else {
#pragma unroll
      for (int t = 0; t < 8; ++t) xn[t] = xi[t];
    }
    r[st] = diff8(d[st], xi, xn);
    ok[st] = in && valid(sidx);
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
        float p = 0.f;
        const int gv = gid(s0 + st);  // every lane: gid may shuffle
        if (near[st]) {
          const float4 *srcp = reinterpret_cast<const float4 *>(a.xm + (voff + gv) * D + gl * 8);
          const float4 x = __ldcg(srcp), y = __ldcg(srcp + 1);
          const float f[8] = {x.x, x.y, x.z, x.w, y.x, y.y, y.z, y.w};
          p = diff8(d[st], xi, f);
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
    if (want && ok[st] && gl == 0)
      loss += kAttract ? __logf(1.0f + r[st]) : __logf(1.0f + r[st]) - __logf(r[st] + 1e-6f);
    may_clip |= c[st] * c[st] * r[st] > 0.98f * a.bound * a.bound;
  }
  if (!__any_sync(kAll, may_clip)) {
#pragma unroll
    for (int st = 0; st < NS; ++st) {
      axpy8(acc, lr * c[st], d[st]);
    }
  } else {
#pragma unroll
    for (int st = 0; st < NS; ++st)
#pragma unroll
      for (int t = 0; t < 8; ++t) acc[t] = fmaf(lr, bclip(d[st][t] * c[st], a.bound), acc[t]);
  }
}

template <int D, int NS, int S, bool kBF16>
__global__ void __launch_bounds__(512, 1) staged_rows_kernel(const BatchedArgs a) {
  using Lay = RowsLayout<D, kBF16>;
  constexpr int LP = Lay::LP, G = Lay::G, kRowB = Lay::kRowB, kXiB = Lay::kXiB;
  constexpr int PR = kRowB / 16;   // 16-byte pieces of a neighbour row
  constexpr int MAXE = 32 / LP;    // CSR entries a lane loads for its group (cap <= 32)
  extern __shared__ __align__(128) unsigned char smem[];
  const int W = blockDim.x >> 5, lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int q = lane / LP, gl = lane % LP;
  const int cap = a.cap, subB = Lay::sub_bytes(cap), slotB = Lay::slot_bytes(cap);
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
    const GraphInfo Gi = a.graphs[g];
    const int skip = a.quirks ? Gi.n - 1 : -1;  // edges into n-1 are dropped (algo.hpp:399-405, 538)
    for (int e = 0; e < a.epochs; ++e) {
      const float lr = a.lr[e];
      const bool want = a.compute_loss && e >= a.loss_from;
      double wloss = 0.0;
      for (int j = 0; j < Gi.batches; ++j) {
        const int64_t bi = Gi.batch_off + j;
        const int64_t it0 = a.batch_item_off[bi];
        const int n_items = int(a.batch_item_off[bi + 1] - it0);
        const int base = j * a.batch;
        const int rows = min(a.batch, Gi.n - base);
        const int rep_rows = (a.quirks && e > 0) ? Gi.last_batch_size : rows;  // algo.hpp:167-169, 594
        const int32_t *negs = a.negs + Gi.neg_off + (size_t(e) * Gi.batches + j) * a.ns;
        // negatives: lane k holds draw k; a draw equal to n counts nothing (copies row 0)
        const int nraw = lane < a.ns ? __ldg(negs + lane) : -1;
        const int nid = nraw < Gi.n ? nraw : 0;
        const unsigned neg_valid = __ballot_sync(kAll, lane < a.ns && nraw < Gi.n);
        const int nmine = n_items > warp ? (n_items - warp + W - 1) / W : 0;
        for (int r0 = 0; r0 < nmine; r0 += 32) {
          const int nr = min(32, nmine - r0);
          if (lane < nr) my_items[lane] = a.items[it0 + warp + int64_t(r0 + lane) * W];
          __syncwarp();
          const int nch = (nr + G - 1) / G;  // chunks of G items
          // this lane's column ids of its group's item in chunk c (entries gl, gl+LP, ...)
          auto load_ids = [&](int c, int (&ids)[MAXE]) {
            const int m = c * G + q;
            const WorkItem &it = my_items[m < nr ? m : 0];
            const int cnt = m < nr ? it.e_end - it.e_begin : 0;
#pragma unroll
            for (int t = 0; t < MAXE; ++t) {
              const int en = gl + t * LP;
              ids[t] = en < cnt ? __ldg(a.col + Gi.eoff + it.e_begin + en) : -1;
            }
          };
          auto issue = [&](int c, const int (&ids)[MAXE]) {
            const int m = c * G + q;
            const bool has = m < nr;
            const uint32_t sub = ring_s + uint32_t((c % S) * slotB + q * subB);
            int *sid = reinterpret_cast<int *>(ring + size_t(c % S) * slotB + q * subB + kXiB + cap * kRowB);
#pragma unroll
            for (int t = 0; t < MAXE; ++t)
              if (gl + t * LP < cap) sid[gl + t * LP] = ids[t];
            __syncwarp();
            if (has) {
              const WorkItem &it = my_items[m];
              const int64_t own = Gi.voff + base + it.row;
              for (int p = gl; p < kXiB / 16; p += LP) dev::cp_async16(sub + p * 16, srcm + own * kXiB + p * 16);
              const int total = (it.e_end - it.e_begin) * PR;
              for (int p = gl; p < total; p += LP) {
                const int en = p / PR;
                dev::cp_async16(sub + kXiB + en * kRowB + (p % PR) * 16, src + (Gi.voff + sid[en]) * kRowB + (p % PR) * 16);
              }
            }
            if (c == 0 && r0 == 0) copy_rows<kRowB>(neg_s, src, Gi.voff, nid, a.ns, lane);
            dev::cp_async_commit();
          };
          {
            int pre[S - 1][MAXE];
#pragma unroll
            for (int i = 0; i < S - 1; ++i) {
              if (i < nch) load_ids(i, pre[i]);
              else
#pragma unroll
                for (int t = 0; t < MAXE; ++t) pre[i][t] = -1;
            }
#pragma unroll
            for (int i = 0; i < S - 1; ++i) {
              if (i < nch) issue(i, pre[i]);
              else dev::cp_async_commit();
            }
          }
          int next[MAXE];
          if (S - 1 < nch) load_ids(S - 1, next);
          for (int c = 0; c < nch; ++c) {
            if (c + S - 1 < nch) issue(c + S - 1, next);
            else dev::cp_async_commit();  // an empty group keeps "S-1 groups after chunk c"
            if (c + S < nch) load_ids(c + S, next);
            dev::cp_async_wait<S - 1>();
            __syncwarp();
            // ---- chunk c: group q trains item c*G + q
            const int m = c * G + q;
            const bool has = m < nr;
            WorkItem it{};
            if (has) it = my_items[m];
            const unsigned char *sub = ring + size_t(c % S) * slotB + q * subB;
            const int *sid = reinterpret_cast<const int *>(sub + kXiB + cap * kRowB);
            float xi[8], acc[8];
            if (has) {
              ld8<false>(xi, sub, gl);
            } else {
#pragma unroll
              for (int t = 0; t < 8; ++t) xi[t] = 0.f;
            }
#pragma unroll
            for (int t = 0; t < 8; ++t) acc[t] = 0.f;
            float loss = 0.f;
            const int cnt = has ? it.e_end - it.e_begin : 0;
            int maxcnt = cnt;
#pragma unroll
            for (int mm = 16; mm >= LP; mm >>= 1) maxcnt = max(maxcnt, __shfl_xor_sync(kAll, maxcnt, mm));
            auto att_valid = [&](int sidx) { const int v = sid[sidx]; return v >= 0 && v != skip; };
            auto att_gid = [&](int sidx) { return sid[sidx]; };
            int s0 = 0;
            for (; s0 + NS <= maxcnt; s0 += NS)
              rows_steps<D, NS, kBF16, true>(a, acc, xi, sub + kXiB, kRowB, s0, cnt, att_valid, att_gid, Gi.voff, lr,
                                             loss, want, gl);
            for (; s0 < maxcnt; ++s0)
              rows_steps<D, 1, kBF16, true>(a, acc, xi, sub + kXiB, kRowB, s0, cnt, att_valid, att_gid, Gi.voff, lr,
                                            loss, want, gl);
            const bool rep = has && it.part == 0 && it.row < rep_rows;
            if (__any_sync(kAll, rep) && a.ns > 0) {
              const int ncnt = rep ? a.ns : 0;
              auto neg_ok = [&](int sidx) { return ((neg_valid >> sidx) & 1u) != 0; };
              auto neg_gid = [&](int sidx) { return __shfl_sync(kAll, nid, sidx); };
              int k0 = 0;
              for (; k0 + NS <= a.ns; k0 += NS)
                rows_steps<D, NS, kBF16, false>(a, acc, xi, negrows, kRowB, k0, ncnt, neg_ok, neg_gid, Gi.voff, lr,
                                                loss, want, gl);
              for (; k0 < a.ns; ++k0)
                rows_steps<D, 1, kBF16, false>(a, acc, xi, negrows, kRowB, k0, ncnt, neg_ok, neg_gid, Gi.voff, lr,
                                               loss, want, gl);
            }
            if (has) {
              float *dst = it.nparts > 1 ? slots + size_t(it.first_slot + it.part) * D : stage + size_t(it.row) * D;
              reinterpret_cast<float4 *>(dst + gl * 8)[0] = make_float4(acc[0], acc[1], acc[2], acc[3]);
              reinterpret_cast<float4 *>(dst + gl * 8)[1] = make_float4(acc[4], acc[5], acc[6], acc[7]);
            }
#pragma unroll
            for (int mm = 16; mm >= 1; mm >>= 1) loss += __shfl_xor_sync(kAll, loss, mm);
            wloss += double(loss);
            __syncwarp();
          }
        }
        dev::cp_async_wait<0>();
        __syncthreads();
        combine_split_rows<D>(a, slots, stage, a.batch_split_off[bi], a.batch_split_off[bi + 1], warp, W, lane);
        __syncthreads();
        update_rows<kBF16>(a.xm, a.xb, stage, (Gi.voff + base) * D, rows * D, threadIdx.x, blockDim.x);  // algo.hpp:651-666
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

template <int D, bool kBF16>
BatchedKernel pick_rows_fn(int steps, int stages) {
  if (steps == 1 && stages == 3) return staged_rows_kernel<D, 1, 3, kBF16>;
  if (steps == 1 && stages == 4) return staged_rows_kernel<D, 1, 4, kBF16>;
  if (steps == 2 && stages == 3) return staged_rows_kernel<D, 2, 3, kBF16>;
  if (steps == 2 && stages == 4) return staged_rows_kernel<D, 2, 4, kBF16>;
  return nullptr;
}

}  // namespace

BatchedKernel pick_rows(int dim, bool bf16, int steps, int stages) {
  switch (dim) {
    case 32: return bf16 ? pick_rows_fn<32, true>(steps, stages) : pick_rows_fn<32, false>(steps, stages);
    case 64: return bf16 ? pick_rows_fn<64, true>(steps, stages) : pick_rows_fn<64, false>(steps, stages);
    case 128: return bf16 ? pick_rows_fn<128, true>(steps, stages) : pick_rows_fn<128, false>(steps, stages);
  }
  return nullptr;
}

}  // namespace batched
}  // namespace de
