#include "de_batched.cuh"

namespace de {
namespace batched {
namespace {

// ---------------------------------------------------------------- staged kernel
//
// The same per-graph step with the rows a warp reads staged in shared memory by
// 16-byte asynchronous copies (cp.async, through L2) instead of loaded into
// registers, so the bytes in flight per SM are bounded by shared memory, not by
// registers, and the copies of later chunks overlap the arithmetic of the current
// one.  Every warp runs its own pipeline over its chunks (work items i = warp,
// warp + W, ... of the minibatch; a chunk is at most cap <= 32 CSR entries):
//   a round of up to 32 items starts by fetching all their column ids into shared
//   memory (4-byte cp.async; where that buffer does not fit, chunk k+S's ids are
//   loaded from global memory one chunk ahead instead), then the rows of chunk
//   k+S-1 are copied (own row from the FP32 master, neighbours from the BF16 copy
//   or the FP32 master) into ring slot (k+S-1) mod S while chunk k is computed from
//   slot k mod S once its copy group has landed (cp.async.wait_group S-1).
// Each warp also copies the minibatch's ns negatives into its own area (with its
// first chunk).  A pair is computed by dim/8 lanes (8 components each),
// 32/(dim/8) pairs per warp step and NS steps in flight.  Results go to the
// team's staging rows as in the register kernel; the minibatch ends with the same
// combine and update.  No wait spins: every wait is a hardware wait on this
// thread's own copies or a CTA barrier.

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
                                           int ids, int64_t voff, float lr, float &loss, bool want, int lane) {
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
    r[st] = diff8(d[st], xi, xn);
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
  // attractive pairs never clip at bound >= 1 (2 sqrt(r) / (1 + r) <= 1): no vote
  if ((kAttract && a.bound >= 1.0f) || !__any_sync(kAll, may_clip)) {
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

// All pairs of xi with rows [0, count).
template <int D, int NS, bool kBF16, bool kAttract>
__device__ __forceinline__ void staged_pairs(const BatchedArgs &a, float (&acc)[8], const float (&xi)[8],
                                             const unsigned char *rows, int row_bytes, int count, unsigned vmask,
                                             int ids, int64_t voff, float lr, float &loss, bool want, int lane) {
  constexpr int G = PairLanes<D>::G;
  int kb = 0;
  for (; kb + NS * G <= count; kb += NS * G)
    pair_steps<D, NS, kBF16, kAttract>(a, acc, xi, rows, row_bytes, kb, count, vmask, ids, voff, lr, loss, want,
                                       lane);
  if constexpr (NS > 1) {
    for (; kb < count; kb += G)
      pair_steps<D, 1, kBF16, kAttract>(a, acc, xi, rows, row_bytes, kb, count, vmask, ids, voff, lr, loss, want,
                                        lane);
  } else {
    if (kb < count)
      pair_steps<D, 1, kBF16, kAttract>(a, acc, xi, rows, row_bytes, kb, count, vmask, ids, voff, lr, loss, want,
                                        lane);
  }
}


__device__ __forceinline__ int cluster_rank() {
  int r;
  asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
  return r;
}

// Every CTA of the cluster: every thread arrives (release) and waits (acquire),
// so each CTA's global writes before the barrier are visible to the others after it.
__device__ __forceinline__ void cluster_sync() {
  asm volatile("barrier.cluster.arrive.release.aligned;\nbarrier.cluster.wait.acquire.aligned;" ::: "memory");
}

// A team is one CTA or, with CT = 2 or 4, the CTAs of a cluster working on one
// graph: team warp tw = rank * W + warp of TW = nct * W, one shared staging area
// (that of rank 0), barriers across the cluster.  With CT > 1 a cluster first
// takes the big graphs (order[0, n_big)) as one team; when they are gone its CTAs
// take the remaining graphs one each.  The loss of an epoch is summed from the
// per-item losses in item order, so it does not depend on the team's make-up.
template <int D, int NS, int S, bool kBF16, int CT>
__global__ void __launch_bounds__(512, 1) staged_kernel(const BatchedArgs a) {
  using Lay = StagedLayout<D, kBF16>;
  constexpr int kRowB = Lay::kRowB, kXiB = Lay::kXiB;
  constexpr int LP = PairLanes<D>::LP;
  extern __shared__ __align__(128) unsigned char smem[];
  const int W = blockDim.x >> 5, lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int gl = lane % LP;
  const int cap = a.cap, slotB = Lay::slot_bytes(cap);
  unsigned char *ring = smem + size_t(warp) * Lay::warp_bytes(S, cap, a.ns, a.stage_ids);
  unsigned char *negrows = ring + size_t(S) * slotB;
  WorkItem *my_items = reinterpret_cast<WorkItem *>(negrows + size_t(a.ns) * kRowB);
  const int *colbuf = reinterpret_cast<const int *>(my_items + 32);  // [32][cap] column ids of the round
  const uint32_t colbuf_s = dev::smem_u32(colbuf);
  const uint32_t ring_s = dev::smem_u32(ring), neg_s = dev::smem_u32(negrows);
  __shared__ int sh_graph;
  const unsigned char *src = kBF16 ? reinterpret_cast<const unsigned char *>(a.xb)
                                   : reinterpret_cast<const unsigned char *>(a.xm);
  const unsigned char *srcm = reinterpret_cast<const unsigned char *>(a.xm);
  const int rank = CT > 1 ? cluster_rank() : 0;
  bool coop = CT > 1;

  for (;;) {
    int g;
    if (coop) {
      if (threadIdx.x == 0 && rank == 0) {
        const int i = atomicAdd(a.next_big, 1);
        *reinterpret_cast<volatile int *>(a.cluster_slot + blockIdx.x / CT) = i < a.n_big ? a.order[i] : -1;
        __threadfence();
      }
      cluster_sync();
      g = __ldcg(a.cluster_slot + blockIdx.x / CT);
      cluster_sync();  // rank 0 rewrites the slot only after every rank has read it
      if (g < 0) {
        coop = false;
        continue;
      }
    } else {
      if (threadIdx.x == 0) {
        const int i = atomicAdd(a.next_graph, 1);
        sh_graph = i < a.n_graphs - a.n_big ? a.order[a.n_big + i] : -1;
      }
      __syncthreads();
      g = sh_graph;
      __syncthreads();
      if (g < 0) break;
    }
    const int nct = coop ? CT : 1, trank = coop ? rank : 0;
    const int tw = trank * W + warp, TW = nct * W;
    const int team_blk = blockIdx.x - trank;
    float *stage = a.stage + size_t(team_blk) * a.batch * D;
    float *slots = a.slots + size_t(team_blk) * a.slot_stride * D;
    float *item_loss = a.item_loss + size_t(team_blk) * a.item_stride;
    auto team_sync = [&]() {
      if (nct > 1) cluster_sync();
      else __syncthreads();
    };
    if (a.trace && threadIdx.x == 0 && trank == 0) {
      a.trace[3 * g] = globaltimer();
      a.trace[3 * g + 2] = blockIdx.x;
    }
    const GraphInfo G = a.graphs[g];
    const int skip = a.quirks ? G.n - 1 : -1;  // edges into n-1 are dropped (algo.hpp:399-405, 538)
    for (int e = 0; e < a.epochs; ++e) {
      const float lr = a.lr[e];
      const bool want = a.compute_loss && e >= a.loss_from;
      double eloss = 0.0;  // rank 0, thread 0: the epoch's loss, minibatch by minibatch
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
        const int nmine = n_items > tw ? (n_items - tw + TW - 1) / TW : 0;
        for (int r0 = 0; r0 < nmine; r0 += 32) {
          const int nr = min(32, nmine - r0);
          // the round's work items, and every column id they read, fetched at once
          // (row l of colbuf: item l's CSR entries, 4-byte asynchronous copies), so
          // that no chunk waits on its column ids
          if (lane < nr) {
            const WorkItem mine = a.items[it0 + tw + int64_t(r0 + lane) * TW];
            my_items[lane] = mine;
            if (a.stage_ids) {
              const int32_t *cs = a.col + G.eoff + mine.e_begin;
              const uint32_t dst = colbuf_s + uint32_t(lane * cap * 4);
              for (int i = 0; i < mine.e_end - mine.e_begin; ++i) dev::cp_async4(dst + 4u * i, cs + i);
            }
          }
          if (a.stage_ids) {
            dev::cp_async_commit();
            dev::cp_async_wait<0>();
          }
          __syncwarp();
          // lane l: column id of CSR entry l of chunk k (-1 past its end)
          auto load_cols = [&](int k) -> int {
            const WorkItem &it = my_items[k];
            if (lane >= it.e_end - it.e_begin) return -1;
            return a.stage_ids ? colbuf[k * cap + lane] : __ldg(a.col + G.eoff + it.e_begin + lane);
          };
          auto issue = [&](int k, int id) {
            const uint32_t slot = ring_s + uint32_t((k % S) * slotB);
            const int cnt = __popc(__ballot_sync(kAll, id >= 0));
            const int64_t own = G.voff + base + my_items[k].row;
            for (int p = lane; p < kXiB / 16; p += 32) dev::cp_async16(slot + p * 16, srcm + own * kXiB + p * 16);
            copy_rows<kRowB>(slot + kXiB, src, G.voff, id, cnt, lane);
            if (k == 0 && r0 == 0) copy_rows<kRowB>(neg_s, src, G.voff, nid, a.ns, lane);
            dev::cp_async_commit();
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
            staged_pairs<D, NS, kBF16, true>(a, acc, xi, slot + kXiB, kRowB, cnt, vmask, ids, G.voff, lr, loss, want,
                                             lane);
            if (it.part == 0 && it.row < rep_rows && a.ns > 0)
              staged_pairs<D, NS, kBF16, false>(a, acc, xi, negrows, kRowB, a.ns, neg_valid, nid, G.voff, lr, loss,
                                                want, lane);
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
            if (want) {
#pragma unroll
              for (int m = 16; m >= 1; m >>= 1) loss += __shfl_xor_sync(kAll, loss, m);
              if (lane == 0) item_loss[tw + (r0 + k) * TW] = loss;
            }
            __syncwarp();
          }
        }
        dev::cp_async_wait<0>();
        team_sync();
        const int s0 = a.batch_split_off[bi], s1 = a.batch_split_off[bi + 1];
        combine_split_rows<D>(a, slots, stage, s0, s1, tw, TW, lane);
        // the minibatch's loss in item order (rank 0, warp 0), whatever team made it
        if (want && trank == 0 && warp == 0) {
          double l = 0.0;
          for (int i = lane; i < n_items; i += 32) l += double(__ldcg(item_loss + i));
#pragma unroll
          for (int m = 16; m >= 1; m >>= 1) l += __shfl_xor_sync(kAll, l, m);
          eloss += l;
        }
        if (s1 > s0) team_sync();  // combined split rows are staged before the update reads them
        update_rows<kBF16>(a.xm, a.xb, stage, (G.voff + base) * D, rows * D, trank * blockDim.x + threadIdx.x,
                           nct * blockDim.x);  // algo.hpp:651-666
        team_sync();
      }
      if (threadIdx.x == 0 && trank == 0 && a.compute_loss) a.loss[size_t(g) * a.epochs + e] = eloss;
    }
    if (a.trace && threadIdx.x == 0 && trank == 0) a.trace[3 * g + 1] = globaltimer();
  }
}

template <int D, bool kBF16, int CT>
BatchedKernel pick_staged_ct(int steps, int stages) {
  if (steps == 1 && stages == 3) return staged_kernel<D, 1, 3, kBF16, CT>;
  if (steps == 1 && stages == 4) return staged_kernel<D, 1, 4, kBF16, CT>;
  if (steps == 2 && stages == 3) return staged_kernel<D, 2, 3, kBF16, CT>;
  if (steps == 2 && stages == 4) return staged_kernel<D, 2, 4, kBF16, CT>;
  return nullptr;
}

template <int D, bool kBF16>
BatchedKernel pick_staged_fn(int steps, int stages, int ctas) {
  if (ctas == 1) return pick_staged_ct<D, kBF16, 1>(steps, stages);
  if (ctas == 2) return pick_staged_ct<D, kBF16, 2>(steps, stages);
  if (ctas == 4) return pick_staged_ct<D, kBF16, 4>(steps, stages);
  return nullptr;
}

}  // namespace

BatchedKernel pick_staged(int dim, bool bf16, int steps, int stages, int ctas) {
  switch (dim) {
    case 32: return bf16 ? pick_staged_fn<32, true>(steps, stages, ctas) : pick_staged_fn<32, false>(steps, stages, ctas);
    case 64: return bf16 ? pick_staged_fn<64, true>(steps, stages, ctas) : pick_staged_fn<64, false>(steps, stages, ctas);
    case 128:
      return bf16 ? pick_staged_fn<128, true>(steps, stages, ctas) : pick_staged_fn<128, false>(steps, stages, ctas);
  }
  return nullptr;
}

}  // namespace batched
}  // namespace de
