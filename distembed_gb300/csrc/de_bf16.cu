// BF16 precision form of the force-model SGD minibatch step (sm_103a).
//
// Storage: FP32 master copy Xm and a BF16 copy Xb of the embedding.  Every read
// inside a minibatch uses Xb (FP32 arithmetic on BF16 values); the update goes to
// Xm and is rounded back into Xb.  The minibatch's shared negatives (ns draws,
// cpp/algo/algo.hpp:172-173) make the repulsive pass (algo.hpp:586-649) a dense
// B x ns problem, done as two BF16 tcgen05 GEMMs per 128-row tile:
//
//   S  = X_tile . N^T                       (TMEM, FP32)
//   r  = |x|^2 + |n|^2 - 2 S,  c = 2 / ((r + 1e-6)(1 + r))  -> C (BF16, SMEM)
//   F += C . N                              (TMEM, FP32)
//   repulsive force of row i = (sum_k c_ik) x_i - F_i
//
// The factorisation drops the per-component clip of algo.hpp:643, which is exact
// when no component can reach the bound: |c (x_d - n_d)| <= c sqrt(r) < 5 for
// r >= 0.25.  A pair with r < 0.25 (other than a row drawn as its own negative,
// whose force is exactly zero) is left out of the GEMMs and recorded in a
// per-row bitmask; the update kernel adds those pairs one by one in FP32 with
// the clip.
//
// Per minibatch: bf16_gather_kernel (the negatives into N, |n|^2), then
// bf16_attract_kernel (attractive pass, warp per work item) and
// bf16_repulse_kernel (the GEMMs), which are independent and run on two
// streams, then bf16_apply_kernel (exact close pairs and the update of every
// row of the minibatch).
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include "de_async.cuh"
#include "de_device.cuh"
#include "de_internal.h"

namespace de {
namespace {

using namespace dev;

constexpr float kNearR = 0.25f;   // below this squared distance a component may clip
constexpr int kTileRows = 128;    // rows per tcgen05 tile (M)
constexpr int kChunk = 64;        // negatives per GEMM chunk (one 128-B swizzle atom)
constexpr int kMaxKpad = 1024;    // negatives per minibatch in the BF16 form (bitmask words: 32)
constexpr int kNearWords = kMaxKpad / 32;

// 1/x by the hardware approximation (rcp.approx.ftz.f32, the reciprocal
// __fdividef uses); 1/inf = 0.
__device__ __forceinline__ float rcp_approx(float x) {
  float y;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}

// ------------------------------------------------------------ BF16 rows
// Lane l holds components [l*N, l*N + N) of a row, N = dim / 32.

template <int D>
__device__ __forceinline__ void load_bf16_row(Frag<D> &f, const __nv_bfloat16 *row, int lane) {
  constexpr int N = D / 32;
  const __nv_bfloat16 *p = row + lane * N;
  if constexpr (N == 8) {
    uint4 u = __ldg(reinterpret_cast<const uint4 *>(p));
    const __nv_bfloat162 *h = reinterpret_cast<const __nv_bfloat162 *>(&u);
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      float2 t = __bfloat1622float2(h[i]);
      f.v[2 * i] = t.x;
      f.v[2 * i + 1] = t.y;
    }
  } else if constexpr (N == 4) {
    uint2 u = __ldg(reinterpret_cast<const uint2 *>(p));
    const __nv_bfloat162 *h = reinterpret_cast<const __nv_bfloat162 *>(&u);
#pragma unroll
    for (int i = 0; i < 2; ++i) {
      float2 t = __bfloat1622float2(h[i]);
      f.v[2 * i] = t.x;
      f.v[2 * i + 1] = t.y;
    }
  } else {
    static_assert(N == 2, "dim 64, 128 or 256");
    unsigned u = __ldg(reinterpret_cast<const unsigned *>(p));
    float2 t = __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162 *>(&u));
    f.v[0] = t.x;
    f.v[1] = t.y;
  }
}

template <int D>
__device__ __forceinline__ void store_f32_contig(const Frag<D> &f, float *row, int lane) {
  constexpr int N = D / 32;
  float *p = row + lane * N;
  if constexpr (N % 4 == 0) {
#pragma unroll
    for (int i = 0; i < N; i += 4) *reinterpret_cast<float4 *>(p + i) = make_float4(f.v[i], f.v[i + 1], f.v[i + 2], f.v[i + 3]);
  } else {
#pragma unroll
    for (int i = 0; i < N; i += 2) *reinterpret_cast<float2 *>(p + i) = make_float2(f.v[i], f.v[i + 1]);
  }
}

// ------------------------------------------------------------ attractive + gather

// A lane's D/32 BF16 components of a row as loaded (16, 8 or 4 bytes), unpacked
// to FP32 only when used, so that rows in flight cost half the registers.
template <int D>
struct RawRow {
  static constexpr int W = D / 64;  // 32-bit words per lane
  uint32_t w[W];
};

template <int D>
__device__ __forceinline__ void load_raw(RawRow<D> &r, const __nv_bfloat16 *row, int lane) {
  constexpr int W = RawRow<D>::W;
  const __nv_bfloat16 *p = row + lane * (D / 32);
  if constexpr (W == 4) {
    const uint4 u = __ldg(reinterpret_cast<const uint4 *>(p));
    r.w[0] = u.x, r.w[1] = u.y, r.w[2] = u.z, r.w[3] = u.w;
  } else if constexpr (W == 2) {
    const uint2 u = __ldg(reinterpret_cast<const uint2 *>(p));
    r.w[0] = u.x, r.w[1] = u.y;
  } else {
    static_assert(W == 1, "dim 64, 128 or 256");
    r.w[0] = __ldg(reinterpret_cast<const unsigned *>(p));
  }
}

// The same values load_bf16_row produces.
template <int D>
__device__ __forceinline__ void unpack_row(Frag<D> &f, const RawRow<D> &r) {
#pragma unroll
  for (int i = 0; i < RawRow<D>::W; ++i) {
    const float2 t = __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162 *>(&r.w[i]));
    f.v[2 * i] = t.x;
    f.v[2 * i + 1] = t.y;
  }
}

// The rows of CSR entries k .. k+U-1 (lane j of `ids`: the column of entry j,
// -1 for none) as raw BF16; bit u of the result: entry k+u is a row.
template <int D, int U>
__device__ __forceinline__ unsigned fetch_group(const BF16BatchArgs &a, RawRow<D> (&raw)[U], int ids, int k, int lane) {
  unsigned mask = 0;
#pragma unroll
  for (int u = 0; u < U; ++u) {
    const int n = __shfl_sync(kFull, ids, k + u);
    if (n >= 0) {
      load_raw<D>(raw[u], a.xb + size_t(n) * D, lane);
      mask |= 1u << u;
    }
  }
  return mask;
}

template <int D, int U>
__device__ __forceinline__ void bf16_force_group(const BF16BatchArgs &a, Frag<D> &acc, const Frag<D> &xi, int ids,
                                                 int k, float lr, float bound, bool want_loss, float &loss,
                                                 int lane) {
  Frag<D> xn[U];
  unsigned mask = 0;
#pragma unroll
  for (int u = 0; u < U; ++u) {
    const int n = __shfl_sync(kFull, ids, k + u);
    if (n >= 0) {
      load_bf16_row(xn[u], a.xb + size_t(n) * D, lane);
      mask |= 1u << u;
    } else {
      xn[u] = xi;
    }
  }
  if (mask) pair_forces<D, U, true>(acc, xi, xn, mask, lr, bound, want_loss, loss, lane);
}

// The minibatch's negatives gathered once: N (k x dim, zero rows for padding),
// |n|^2 and ids.  A CTA takes 32 consecutive negatives, one warp each: the warp
// copies its row into N (D/32 components per lane) and reduces |n|^2.
constexpr int kGatherTile = 32;
template <int D>
__global__ void __launch_bounds__(kGatherTile * 32) bf16_gather_kernel(const BF16BatchArgs a) {
  constexpr int N = D / 32;  // components per lane
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int epoch = a.epoch[0];
  const int32_t *negs = a.negs + (size_t(epoch) * a.batches + a.batch_id) * a.ns;
  const int k0 = blockIdx.x * kGatherTile;
  {
    const int kk = warp, k = k0 + kk;
    int n = k < a.ns ? __ldg(negs + k) : -1;
    if (n >= a.n) n = -1;  // a draw equal to n contributes nothing
    float sq = 0.f;
    if constexpr (N == 8) {
      uint4 u = n >= 0 ? __ldg(reinterpret_cast<const uint4 *>(a.xb + size_t(n) * D) + lane) : make_uint4(0, 0, 0, 0);
      reinterpret_cast<uint4 *>(a.nb + size_t(k) * D)[lane] = u;
      const uint32_t w[4] = {u.x, u.y, u.z, u.w};
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        const float lo = __uint_as_float(w[i] << 16), hi = __uint_as_float(w[i] & 0xffff0000u);
        sq = fmaf(lo, lo, fmaf(hi, hi, sq));
      }
    } else if constexpr (N == 4) {
      uint2 u = n >= 0 ? __ldg(reinterpret_cast<const uint2 *>(a.xb + size_t(n) * D) + lane) : make_uint2(0, 0);
      reinterpret_cast<uint2 *>(a.nb + size_t(k) * D)[lane] = u;
      const uint32_t w[2] = {u.x, u.y};
#pragma unroll
      for (int i = 0; i < 2; ++i) {
        const float lo = __uint_as_float(w[i] << 16), hi = __uint_as_float(w[i] & 0xffff0000u);
        sq = fmaf(lo, lo, fmaf(hi, hi, sq));
      }
    } else {
      static_assert(N == 2, "dim 64, 128 or 256");
      uint32_t u = n >= 0 ? __ldg(reinterpret_cast<const uint32_t *>(a.xb + size_t(n) * D) + lane) : 0u;
      reinterpret_cast<uint32_t *>(a.nb + size_t(k) * D)[lane] = u;
      const float lo = __uint_as_float(u << 16), hi = __uint_as_float(u & 0xffff0000u);
      sq = fmaf(lo, lo, hi * hi);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) sq += __shfl_xor_sync(kFull, sq, o);
    if (lane == 0) {
      a.nn[k] = n >= 0 ? sq : __int_as_float(0x7f800000);  // no draw: |n|^2 = +inf, so c = 0
      a.nid[k] = n;
    }
  }
}

template <int D, int U>
__global__ void __launch_bounds__(kPlainWarps * 32, 6) bf16_attract_kernel(const BF16BatchArgs a) {
  const int lane = threadIdx.x & 31;
  const int wib = threadIdx.x >> 5;
  const bool want_loss = a.compute_loss != 0;
  const int epoch = a.epoch[0];
  const float lr = a.lr[epoch];

  const int gw = blockIdx.x * kPlainWarps + wib;
  if (gw >= a.n_items) return;
  const WorkItem it = a.items[gw];
  const int skip = a.quirks ? a.n - 1 : -1;  // edges into n-1 are dropped (algo.hpp:399-405, 538)
  const int cnt = it.e_end - it.e_begin;
  if (cnt == 0) {  // a row without CSR entries: no attractive update (the update kernel reads none)
    if (want_loss && lane == 0) a.loss_item[a.loss_off + gw] = 0.0;
    return;
  }
  int ids = -1;
  if (lane < cnt) {
    ids = __ldg(a.col + it.e_begin + lane);
    if (ids == skip) ids = -1;
  }
  Frag<D> xi, acc;
  load_bf16_row(xi, a.xb + size_t(a.base + it.row) * D, lane);
  acc.zero();
  float loss = 0.f;  // this item's loss terms (FP32); the epoch sum is FP64
  // groups of U, software-pipelined: the next group's rows are in flight (as
  // raw BF16) while this group's forces are computed; a last group of at most
  // U/2 entries runs as a group of U/2
  int k = 0;
  if (U / 2 < cnt) {
    RawRow<D> cur[U];
    unsigned mcur = fetch_group<D, U>(a, cur, ids, 0, lane);
    for (; k + U / 2 < cnt; k += U) {
      RawRow<D> nxt[U];
      unsigned mnxt = 0;
      if (k + U + U / 2 < cnt) mnxt = fetch_group<D, U>(a, nxt, ids, k + U, lane);
      Frag<D> xn[U];
#pragma unroll
      for (int u = 0; u < U; ++u) {
        if ((mcur >> u) & 1u) unpack_row<D>(xn[u], cur[u]);
        else xn[u] = xi;
      }
      if (mcur) pair_forces<D, U, true>(acc, xi, xn, mcur, lr, a.bound, want_loss, loss, lane);
#pragma unroll
      for (int u = 0; u < U; ++u) cur[u] = nxt[u];
      mcur = mnxt;
    }
  }
  if (k < cnt) bf16_force_group<D, U / 2>(a, acc, xi, ids, k, lr, a.bound, want_loss, loss, lane);

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
  if (owner) store_f32_contig(acc, a.abuf + size_t(it.row) * D, lane);
  if (want_loss) {
#pragma unroll
    for (int m = 16; m >= 1; m >>= 1) loss += __shfl_xor_sync(kFull, loss, m);
    if (lane == 0) a.loss_item[a.loss_off + gw] = double(loss);
  }
}

// ------------------------------------------------------------ tcgen05 plumbing

// Shared-memory matrix descriptor: K-major operand in 128-byte swizzled atoms of
// 8 rows x 128 B (stride between 8-row groups 1024 B), sm_100 descriptor version.
__device__ __forceinline__ uint64_t umma_desc(uint32_t addr) {
  return uint64_t((addr & 0x3FFFF) >> 4) | (uint64_t(1) << 16) | (uint64_t(1024 >> 4) << 32) | (uint64_t(1) << 46) |
         (uint64_t(2) << 61);
}

// The same swizzled atoms read as an MN-major operand (B of the second GEMM: the
// rows of a chunk of N are its K index, their 64-dim atoms its N index): lbo =
// bytes between 64-element atoms along N, sbo = bytes between 8-row groups along K.
__device__ __forceinline__ uint64_t umma_desc_mn(uint32_t addr, uint32_t lbo, uint32_t sbo) {
  return uint64_t((addr & 0x3FFFF) >> 4) | (uint64_t(lbo >> 4) << 16) | (uint64_t(sbo >> 4) << 32) |
         (uint64_t(1) << 46) | (uint64_t(2) << 61);
}

// Instruction descriptor: BF16 x BF16 -> FP32, M x N, A K-major, B K-major or
// (b_mn) MN-major.
__host__ __device__ constexpr uint32_t umma_idesc(int m, int n, bool b_mn = false) {
  return (1u << 4) | (1u << 7) | (1u << 10) | (b_mn ? (1u << 16) : 0u) | (uint32_t(n >> 3) << 17) |
         (uint32_t(m >> 4) << 24);
}

__device__ __forceinline__ void tma_load_2d(uint32_t dst, const CUtensorMap *map, int x, int y, uint32_t bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(dst),
      "l"(map), "r"(x), "r"(y), "r"(bar)
      : "memory");
}

// One tcgen05 MMA (BF16 x BF16 -> FP32 in tensor memory) with A in tensor memory
// (M lanes, K packed two BF16 per column) and B from a shared-memory descriptor.
__device__ __forceinline__ void umma_ta(uint32_t tmem_d, uint32_t a_tmem, uint64_t b, uint32_t idesc, uint32_t accumulate) {
  asm volatile(
      "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\ntcgen05.mma.cta_group::1.kind::f16 [%0], [%1], %2, %3, p;\n}\n" ::"r"(tmem_d),
      "r"(a_tmem), "l"(b), "r"(idesc), "r"(accumulate)
      : "memory");
}

__device__ __forceinline__ void umma_commit(uint32_t bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar) : "memory");
}

__device__ __forceinline__ void tmem_ld32(uint32_t taddr, uint32_t (&r)[32]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16,%17,%18,%19,%20,"
      "%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]),
        "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]),
        "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr)
      : "memory");
}

__device__ __forceinline__ void tmem_ld16(uint32_t taddr, uint32_t (&r)[16]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr)
      : "memory");
}

__device__ __forceinline__ void tmem_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

// 16 consecutive columns of this warp's 32 lanes from registers.
__device__ __forceinline__ void tmem_st16(uint32_t taddr, const uint32_t (&r)[16]) {
  asm volatile(
      "tcgen05.st.sync.aligned.32x32b.x16.b32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16};" ::"r"(taddr),
      "r"(r[0]), "r"(r[1]), "r"(r[2]), "r"(r[3]), "r"(r[4]), "r"(r[5]), "r"(r[6]), "r"(r[7]), "r"(r[8]), "r"(r[9]),
      "r"(r[10]), "r"(r[11]), "r"(r[12]), "r"(r[13]), "r"(r[14]), "r"(r[15])
      : "memory");
}
__device__ __forceinline__ void tmem_wait_st() { asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// ------------------------------------------------------------ repulsion GEMMs

// Shared-memory plan of bf16_repulse_kernel (offsets from a 1024-aligned base).
template <int D>
struct RepulseSmem {
  static constexpr int kAtoms = D / 64;                  // 128-B column atoms of a dim-wide row
  static constexpr int kStages = 6;                      // chunks of N in flight
  static constexpr int kX = kAtoms * kTileRows * 128;    // X tile
  static constexpr int kN = kAtoms * kChunk * 128;       // one chunk of N (B operand of both GEMMs)
  static_assert(kX == 2 * kN, "the X tile takes two stages");
  static constexpr int kMisc = 16384;                    // per-row exchanges, flags and losses
  static constexpr int offN = 0;
  static constexpr int offX = offN + (kStages - 2) * kN;  // first over the last two stages
  static constexpr int offMisc = offN + kStages * kN;
  static constexpr int bytes = offMisc + kMisc;
  static constexpr int dynamic = bytes + 1024;           // + alignment slack
};

// Warp roles: 0-7 epilogue, 8 TMA producer, 9 MMA issuer and TMEM owner.
// Epilogue warp w serves TMEM lane quadrant w % 4 (tile rows 32(w%4) .. +31) and
// column half w / 4: 32 of the 64 coefficients of each chunk, and half of the
// dims in the final update.  TMEM: S chunks in columns [0, 128) (double
// buffered; the epilogue overwrites a chunk's S with its BF16 coefficients C,
// packed two per column, which the second GEMM reads as its A operand), the
// BF16 X tile in columns [128, 128 + dim / 2) (the first GEMM's A operand,
// written once by the epilogue warps from the TMA copy), F in columns
// [256, 256 + dim).  Both A operands live in tensor memory, so the shared-memory
// traffic of a chunk is its N (the B operand of both GEMMs: K-major for
// S = X N^T, MN-major for F += C N, so no transposed copy exists) streaming
// through a ring of six stages, the last two of which first hold the TMA copy
// of the X tile (until it is in tensor memory).
//
// KS = 2: the negatives of a tile are split between the two CTAs of a cluster
// (rank 0: the first ceil(chunks / 2) chunks, rank 1 the rest), so twice as
// many SMs work on a minibatch.  Rank r owns tile rows [64 r, 64 r + 64).  Each
// CTA stages its partial force (its row sums) x - (its F) of all 128 rows in its
// shared memory; once the peer has signalled (a release arrive on this CTA's
// PEER_FREE barrier) that its incoming area is free, one warp pushes the peer's
// 64 rows, their flags and losses with bulk copies into the peer's shared memory,
// completing on the peer's INCOMING barrier; each CTA then adds the two partials
// of its rows and stores them, and waits (PEER_GOT) until the peer has received
// its rows before its shared memory ends.  Partial sums are combined as own +
// peer, the same value on either rank.  Every wait is bounded.
constexpr int kEpiThreads = 256;
constexpr int kRepulseThreads = kEpiThreads + 64;

__device__ __forceinline__ int cta_rank_in_cluster() {
  int r;
  asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
  return r;
}
// Release arrive on a barrier of the peer CTA (address from peer_addr).
__device__ __forceinline__ void mbar_arrive_remote(uint32_t bar) {
  asm volatile("mbarrier.arrive.release.cluster.shared::cluster.b64 _, [%0];" ::"r"(bar) : "memory");
}
// mbar_wait for threads that may wait long and share their SM sub-partition
// with the MMA-issuing thread: each poll may suspend the thread (up to 2 us,
// woken early when the phase completes) instead of spinning on the issue slots;
// bounded like mbar_wait.
constexpr long kSleepPolls = 1L << 20;
__device__ __forceinline__ bool mbar_wait_sleep(uint32_t bar, uint32_t parity, int *err_shared) {
  for (long it = 0; it < kSleepPolls; ++it) {
    uint32_t ok;
    asm volatile(
        "{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\nselp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(bar), "r"(parity), "r"(2000)
        : "memory");
    if (ok) return true;
    if (*reinterpret_cast<volatile int *>(err_shared)) return false;
  }
  *reinterpret_cast<volatile int *>(err_shared) = 1;
  return false;
}
// mbar_wait with cluster-scope acquire (the phase was completed by the peer CTA).
__device__ __forceinline__ bool mbar_wait_cluster(uint32_t bar, uint32_t parity, int *err_shared) {
  for (long it = 0; it < kSpinLimit; ++it) {
    uint32_t ok;
    asm volatile(
        "{\n.reg .pred p;\nmbarrier.try_wait.parity.acquire.cluster.shared::cta.b64 p, [%1], %2;\nselp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(bar), "r"(parity)
        : "memory");
    if (ok) return true;
    if (*reinterpret_cast<volatile int *>(err_shared)) return false;
  }
  *reinterpret_cast<volatile int *>(err_shared) = 1;
  return false;
}
__device__ __forceinline__ uint32_t peer_addr(uint32_t local, int peer) {
  uint32_t r;
  asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(local), "r"(peer));
  return r;
}
// Bulk copy of `bytes` (a multiple of 16, both addresses 16-byte aligned) from
// this CTA's shared memory into the peer CTA's (dst, bar: peer_addr addresses),
// completing on the peer's barrier.
__device__ __forceinline__ void bulk_s2peer(uint32_t dst, uint32_t src, uint32_t bytes, uint32_t bar) {
  asm volatile("cp.async.bulk.shared::cluster.shared::cta.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
               "r"(src), "r"(bytes), "r"(bar)
               : "memory");
}

template <int D, int KS>
__global__ void __launch_bounds__(kRepulseThreads, 1) bf16_repulse_kernel(const __grid_constant__ CUtensorMap map_x,
                                                               const __grid_constant__ CUtensorMap map_n,
                                                               const BF16BatchArgs a) {
  using L = RepulseSmem<D>;
  extern __shared__ unsigned char smem_raw[];
  unsigned char *sm = reinterpret_cast<unsigned char *>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  __shared__ __align__(8) uint64_t bar[24];
  __shared__ uint32_t tmem_holder;
  __shared__ int err;
  __shared__ float2 negmeta[2][kChunk];  // (|n|^2, vertex id) of a chunk's negatives
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int nchunks = a.kpad / kChunk;
  const int ks = KS == 2 ? cta_rank_in_cluster() : 0;
  const int peer = ks ^ 1;  // KS = 2: the other CTA of the cluster
  const int tile_base = (blockIdx.x / KS) * kTileRows;  // row offset within the minibatch
  // this CTA's chunks [c_begin, c_end) (KS = 2 needs at least two chunks)
  const int c_begin = ks == 0 ? 0 : (nchunks + 1) / 2;
  const int c_end = (KS == 1 || ks == 1) ? nchunks : (nchunks + 1) / 2;
  const int nloc = c_end - c_begin;

  // barrier ids
  constexpr int NST = L::kStages;
  const uint32_t b0 = smem_u32(&bar[0]);
  auto B = [&](int i) { return b0 + 8u * uint32_t(i); };
  const int FULL_X = 0, FULL_N = 1, FREE_N = FULL_N + NST, X_TMEM = FREE_N + NST, S_FULL = X_TMEM + 1,
            C_FULL = S_FULL + 2, F_DONE = C_FULL + 2, INCOMING = F_DONE + 1, PEER_FREE = INCOMING + 1,
            PEER_GOT = PEER_FREE + 1;
  static_assert(1 + 2 * NST + 1 + 4 + 4 <= 24, "barrier slots");
  constexpr uint32_t kColX = 128, kColF = 256;  // tensor-memory columns of X and F
  auto failed = [&]() { return *reinterpret_cast<volatile int *>(&err) != 0; };

  if (tid == 0) {
    err = 0;
    mbar_init(B(FULL_X), 1);
    for (int i = 0; i < NST; ++i) {
      mbar_init(B(FULL_N + i), 1);
      mbar_init(B(FREE_N + i), 1);
    }
    mbar_init(B(X_TMEM), kEpiThreads);
    for (int i = 0; i < 2; ++i) {
      mbar_init(B(S_FULL + i), 1);
      mbar_init(B(C_FULL + i), kEpiThreads);
    }
    mbar_init(B(F_DONE), 1);
    mbar_init(B(INCOMING), 1);
    mbar_init(B(PEER_FREE), 1);
    mbar_init(B(PEER_GOT), 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 9) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_holder)),
                 "r"(512)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  // KS = 2: every thread arrives once here, after the barrier initialisation,
  // and waits once before this CTA first touches the peer's shared memory
  if constexpr (KS == 2) asm volatile("barrier.cluster.arrive.release.aligned;" ::: "memory");
  const uint32_t tmem = tmem_holder;
  const uint32_t sX = smem_u32(sm + L::offX);
  auto sN = [&](int st) { return smem_u32(sm + L::offN + st * L::kN); };
  // the misc area: per-row exchanges between the two column halves ([0, 4096),
  // used before the staging), then per tile row a flag (nonzero: the row's
  // force is final) and, with KS = 2, its loss, then the peer's flags and losses
  unsigned char *const misc = sm + L::offMisc;
  float *const xx_part = reinterpret_cast<float *>(misc);
  float *const rs_part = reinterpret_cast<float *>(misc + 1024);
  double *const loss_part = reinterpret_cast<double *>(misc + 2048);
  int *const row_flags = reinterpret_cast<int *>(misc + 4096);
  double *const row_loss = reinterpret_cast<double *>(misc + 5120);
  int *const in_flags = reinterpret_cast<int *>(misc + 8192);
  double *const in_loss = reinterpret_cast<double *>(misc + 8448);
  // after the GEMMs: the staged force rows (pitch D + 4 floats) over the N
  // stages; KS = 2: after them the peer's partials of this CTA's 64 rows (the
  // same pitch: one contiguous block, reaching into the then dead half-row
  // exchange area of misc, before the row flags), their 64 flags and 64 losses
  // in the misc area
  constexpr int kPitch = D + 4;
  constexpr int kStageBytes = kTileRows * kPitch * 4;
  constexpr uint32_t kHalfRowsBytes = 64 * kPitch * 4;
  float *const stage = reinterpret_cast<float *>(sm + L::offN);
  float *const in_rows = reinterpret_cast<float *>(sm + L::offN + kStageBytes);
  static_assert(kStageBytes + kHalfRowsBytes <= L::offMisc - L::offN + 4096, "incoming rows end before the row flags");
  constexpr uint32_t kInBytes = kHalfRowsBytes + 64 * 4 + 64 * 8;

  if (warp == 8) {
    // ---------------- TMA producer
    if (lane == 0) {
      int issued_n[NST] = {};
      mbar_expect_tx(B(FULL_X), L::kX);
      for (int ka = 0; ka < L::kAtoms; ++ka)
        tma_load_2d(sX + ka * kTileRows * 128, &map_x, ka * 64, a.base + tile_base, B(FULL_X));
      // chunk lc into stage lc % NST once the second GEMM of chunk lc - NST has
      // read that stage; the last two stages are first free once the epilogue
      // warps have copied the X tile into tensor memory
      for (int lc = 0; lc < nloc && !failed(); ++lc) {
        const int c = c_begin + lc, st = lc % NST, use = lc / NST;
        if (use > 0) {
          if (!mbar_wait_sleep(B(FREE_N + st), (use - 1) & 1, &err)) break;
        } else if (st >= NST - 2) {
          if (!mbar_wait_sleep(B(X_TMEM), 0, &err)) break;
        }
        mbar_expect_tx(B(FULL_N + st), L::kN);
        for (int ka = 0; ka < L::kAtoms; ++ka)
          tma_load_2d(sN(st) + ka * kChunk * 128, &map_n, ka * 64, c * kChunk, B(FULL_N + st));
        ++issued_n[st];
      }
      if (failed()) {
        // bounded wait for every copy this thread started before the CTA leaves
        int dummy = 0;
        for (int st = 0; st < NST; ++st)
          if (issued_n[st]) mbar_wait(B(FULL_N + st), (issued_n[st] - 1) & 1, &dummy);
        mbar_wait(B(FULL_X), 0, &dummy);
      }
    }
  } else if (warp == 9) {
    // ---------------- MMA issuer
    if (lane == 0) {
      constexpr uint32_t idesc1 = umma_idesc(kTileRows, kChunk);
      constexpr uint32_t idesc2 = umma_idesc(kTileRows, D, true);
      const uint32_t tmem_f = tmem + kColF;
      bool ok = mbar_wait(B(X_TMEM), 0, &err);  // X in tensor memory (stored by the epilogue warps)
      // F += C N: A = the chunk's coefficients in tensor memory (over its S), B =
      // the chunk of N itself, read MN-major; one instruction takes 16 negatives
      // (8 columns of C, two 8-row groups of 1024 B of N)
      auto gemm2 = [&](int lc) {  // lc: chunk index within this CTA's range
        const int b = lc & 1, st = lc % NST;
        if (!mbar_wait(B(C_FULL + b), (lc >> 1) & 1, &err)) return false;
        tc_fence_after();
        const uint64_t dn = umma_desc_mn(sN(st), kChunk * 128, 1024);
#pragma unroll
        for (int k = 0; k < kChunk / 16; ++k)  // descriptor address fields step by bytes / 16
          umma_ta(tmem_f, tmem + uint32_t(b * kChunk + 8 * k), dn + uint64_t(k * 2048 / 16), idesc2,
                  (lc > 0 || k > 0) ? 1u : 0u);
        umma_commit(B(FREE_N + st));
        return true;
      };
      for (int lc = 0; ok && lc < nloc; ++lc) {
        const int b = lc & 1, st = lc % NST;
        // S buffer b last held the coefficients of chunk lc - 2, read by that
        // chunk's second GEMM, which this thread issued before this first GEMM:
        // tcgen05.mma instructions of one thread are performed in issue order,
        // so no wait is needed before overwriting it
        ok = mbar_wait(B(FULL_N + st), (lc / NST) & 1, &err);
        if (!ok) break;
        tc_fence_after();
        const uint32_t tmem_s = tmem + uint32_t(b * kChunk);
        const uint64_t dn = umma_desc(sN(st));
#pragma unroll
        for (int kk = 0; kk < D / 16; ++kk)  // 16 dims per step: 8 columns of X, 32 B of an N atom row
          umma_ta(tmem_s, tmem + kColX + uint32_t(8 * kk),
                  dn + uint64_t(((kk >> 2) * kChunk * 128 + (kk & 3) * 32) / 16), idesc1, kk ? 1u : 0u);
        umma_commit(B(S_FULL + b));
        if (lc >= 1) ok = gemm2(lc - 1);
      }
      if (ok) ok = gemm2(nloc - 1);
      umma_commit(B(F_DONE));  // also fires after a failure, once issued MMAs finish
      int dummy = 0;
      mbar_wait(B(F_DONE), 0, &dummy);  // no tensor-core work may outlive the CTA
    }
  } else {
    // ---------------- epilogue
    const int q4 = warp & 3, hf = warp >> 2;  // lane quadrant, column half
    const int t = q4 * 32 + lane;             // tile row = TMEM lane
    const int epoch = a.epoch[0];
    // rows that take the repulsive pass (algo.hpp:167-169, 594)
    const int rep_rows = (a.quirks && epoch + a.epoch[1] > 0) ? a.last_batch_size : a.rows;
    const int row_local = tile_base + t;
    const bool row_valid = row_local < a.rows;
    const bool rep_active = row_valid && row_local < rep_rows;
    const int row_global = a.base + row_local;
    const float lr = a.lr[epoch];
    auto epi_sync = []() { asm volatile("bar.sync 1, 256;" ::: "memory"); };

    const uint32_t lane_base = uint32_t(q4 * 32) << 16;
    // The row's BF16 values from the X tile (the TMA copy of the rows, 128-byte
    // swizzled atoms), each half its D/2 dims: into tensor memory as the first
    // GEMM's A operand (column kColX + j holds dims 2j, 2j+1), and |x|^2 summed
    // in dim order
    float xx = 0.f;
    const bool x_ok = __all_sync(kFull, mbar_wait_sleep(B(FULL_X), 0, &err));
    {
      const unsigned char *xrow = sm + L::offX + (t >> 3) * 1024 + (t & 7) * 128;
#pragma unroll
      for (int g = 0; g < D / 64; ++g) {  // 16 columns (32 dims) at a time
        uint32_t w[16];
#pragma unroll
        for (int i = 0; i < 4; ++i) {
          const int chunk = hf * (D / 16) + g * 4 + i;  // 16-byte chunk of the row: dims 8 chunk .. 8 chunk + 7
          const uint4 u = x_ok ? *reinterpret_cast<const uint4 *>(xrow + (chunk >> 3) * (kTileRows * 128) +
                                                                  (((chunk & 7) ^ (t & 7)) << 4))
                               : make_uint4(0u, 0u, 0u, 0u);
          w[4 * i] = u.x, w[4 * i + 1] = u.y, w[4 * i + 2] = u.z, w[4 * i + 3] = u.w;
          const __nv_bfloat162 *h = reinterpret_cast<const __nv_bfloat162 *>(&u);
#pragma unroll
          for (int q = 0; q < 4; ++q) {
            const float2 f = __bfloat1622float2(h[q]);
            xx = fmaf(f.x, f.x, fmaf(f.y, f.y, xx));
          }
        }
        tmem_st16(tmem + lane_base + kColX + uint32_t(hf * (D / 4) + g * 16), w);
      }
      if (!row_valid) xx = 0.f;
    }
    tmem_wait_st();
    tc_fence_before();
    mbar_arrive(B(X_TMEM));
    // per-row exchange between the two column halves
    xx_part[hf * kTileRows + t] = xx;
    // |n|^2 and vertex id of the chunk's negatives, staged once per chunk; this
    // CTA's chunks start at c_begin (metadata, and the row's bitmask words)
    const float *nn_loc = a.nn + c_begin * kChunk;
    const int32_t *nid_loc = a.nid + c_begin * kChunk;
    uint32_t *near_loc = a.near_bits + size_t(row_local) * kNearWords + c_begin * 2 + hf;
    const int et = hf * 128 + t;  // 0..255
    if (et < kChunk)
      negmeta[0][et] = make_float2(__ldg(nn_loc + et), __int_as_float(__ldg(nid_loc + et)));
    epi_sync();
    xx = xx_part[t] + xx_part[kTileRows + t];

    float rowsum = 0.f;
    double loss = 0.0;
    for (int lc = 0; lc < nloc; ++lc) {
      const int b = lc & 1;
      // next chunk's metadata: loads issued now, stored before this chunk's barrier
      const bool pre = lc + 1 < nloc && et < kChunk;
      float pre_nn = 0.f;
      int pre_id = -1;
      if (pre) {
        pre_nn = __ldg(nn_loc + (lc + 1) * kChunk + et);
        pre_id = __ldg(nid_loc + (lc + 1) * kChunk + et);
      }
      uint32_t s_raw[32] = {};
      const bool got = __all_sync(kFull, mbar_wait_sleep(B(S_FULL + b), (lc >> 1) & 1, &err));
      tc_fence_after();
      if (got) {
        tmem_ld32(tmem + lane_base + uint32_t(b * kChunk + hf * 32), s_raw);
        tmem_wait_ld();
      }
      // Coefficients without branches, so the 32 pairs' chains interleave.  A
      // negative that is no draw (padding, or a draw equal to n) has |n|^2 = +inf,
      // so its r is +inf and its coefficient 0.  A pair with r < kNearR takes the
      // exact path (bit in near_word, coefficient 0 here); that includes a row
      // drawn as its own negative (r ~ 0), whose exact force is 0.
      uint32_t packed[16];
      uint32_t near_word = 0;  // bit i: column hf*32 + i of this chunk takes the exact path
      if (!rep_active) {
#pragma unroll
        for (int i = 0; i < 16; ++i) packed[i] = 0u;
      } else if (a.compute_loss) {
        // with the loss: the log of a product of eight ratios (each
        // (1+r)/(r+1e-6) in [1, 5] for the pairs taken), summed in FP32, folded
        // into FP64 once per chunk
        float loss_c = 0.f;
#pragma unroll
        for (int j = 0; j < 32; j += 8) {
          float prod = 1.f;
          float cv[8];
#pragma unroll
          for (int q = 0; q < 8; ++q) {
            const float2 m = negmeta[b][hf * 32 + j + q];
            const float r = xx + m.x - 2.0f * __uint_as_float(s_raw[j + q]);
            const bool nearp = r < kNearR;
            // one reciprocal: q = 1/((r+1e-6)(1+r)), c = 2q, (1+r)/(r+1e-6) = (1+r)^2 q
            const float r1 = 1.0f + r;
            const float qr = rcp_approx((r + 1e-6f) * r1);
            const float cc = __bfloat162float(__float2bfloat16(2.0f * qr));
            cv[q] = nearp ? 0.f : cc;
            prod *= (nearp || qr == 0.f) ? 1.0f : r1 * r1 * qr;
            near_word |= nearp ? (1u << (j + q)) : 0u;
            rowsum += cv[q];
          }
#pragma unroll
          for (int q = 0; q < 8; q += 2) {
            __nv_bfloat162 p2 = __floats2bfloat162_rn(cv[q], cv[q + 1]);
            packed[(j + q) / 2] = *reinterpret_cast<uint32_t *>(&p2);
          }
          loss_c += __logf(prod);
        }
        loss += double(loss_c);
      } else {
        // no loss: two pairs per packed f32x2 instruction; the row sum adds the
        // BF16-rounded coefficients the second GEMM multiplies with
        const float2 xx2 = make_float2(xx, xx);
        float2 rs2 = make_float2(0.f, 0.f);
#pragma unroll
        for (int j = 0; j < 32; j += 2) {
          const float4 m = *reinterpret_cast<const float4 *>(&negmeta[b][hf * 32 + j]);  // (nn, id) x 2
          const float2 s2 = make_float2(__uint_as_float(s_raw[j]), __uint_as_float(s_raw[j + 1]));
          const float2 r2 = __ffma2_rn(make_float2(-2.f, -2.f), s2, __fadd2_rn(xx2, make_float2(m.x, m.z)));
          const float2 den = __fmul2_rn(__fadd2_rn(r2, make_float2(1e-6f, 1e-6f)), __fadd2_rn(r2, make_float2(1.f, 1.f)));
          const bool n0 = r2.x < kNearR, n1 = r2.y < kNearR;
          const float2 c2 = __fmul2_rn(make_float2(2.f, 2.f), make_float2(rcp_approx(den.x), rcp_approx(den.y)));
          __nv_bfloat162 p2 = __floats2bfloat162_rn(n0 ? 0.f : c2.x, n1 ? 0.f : c2.y);
          const uint32_t pw = *reinterpret_cast<uint32_t *>(&p2);
          packed[j / 2] = pw;
          near_word |= (n0 ? (1u << j) : 0u) | (n1 ? (2u << j) : 0u);
          rs2 = __fadd2_rn(rs2, make_float2(__uint_as_float(pw << 16), __uint_as_float(pw & 0xffff0000u)));
        }
        rowsum += rs2.x + rs2.y;
      }
      if (near_word) near_loc[lc * 2] = near_word;
      if (pre) negmeta[b ^ 1][et] = make_float2(pre_nn, __int_as_float(pre_id));
      // every thread has read this chunk's S (which C overwrites: the row's other
      // half reads columns this half writes) and metadata; the next chunk's
      // metadata is visible after this barrier
      epi_sync();
      // C of this half (coefficients hf*32 .. +31, two per column) over S
      if (got) tmem_st16(tmem + lane_base + uint32_t(b * kChunk + hf * 16), packed);
      tmem_wait_st();
      tc_fence_before();
      mbar_arrive(B(C_FULL + b));
    }
    // every lane of a warp takes the same branch around the (warp-wide) TMEM loads
    const bool done = __all_sync(kFull, mbar_wait_sleep(B(F_DONE), 0, &err) && !failed());
    tc_fence_after();
    // combine the two column halves of each row
    rs_part[hf * kTileRows + t] = rowsum;
    loss_part[hf * kTileRows + t] = loss;
    epi_sync();
    rowsum = rs_part[t] + rs_part[kTileRows + t];
    loss = loss_part[t] + loss_part[kTileRows + t];
    if (KS == 1 && hf == 0 && row_valid && done) a.loss_row[row_global] = loss;
    epi_sync();  // the staging below may overwrite the combine area

    // Repulsive force rowsum * x - F of every tile row, staged as FP32 rows; x
    // comes from the BF16 X tile in tensor memory.  Thread (row t, half hf)
    // writes dims [hf D/2, (hf+1) D/2).
    float *const dst_row = stage + t * kPitch;
    for (int d0 = 0; done && d0 < D / 2; d0 += 32) {
      const int dg = hf * (D / 2) + d0;  // first dim of this group of 32
      uint32_t f[32], xw[16];
      tmem_ld32(tmem + lane_base + kColF + uint32_t(dg), f);
      tmem_ld16(tmem + lane_base + kColX + uint32_t(dg / 2), xw);  // word i: dims dg + 2i, dg + 2i + 1
      tmem_wait_ld();
#pragma unroll
      for (int d = 0; d < 32; d += 4) {
        const float2 x0 = __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162 *>(&xw[d / 2]));
        const float2 x1 = __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162 *>(&xw[d / 2 + 1]));
        *reinterpret_cast<float4 *>(dst_row + dg + d) =
            make_float4(rowsum * x0.x - __uint_as_float(f[d]), rowsum * x0.y - __uint_as_float(f[d + 1]),
                        rowsum * x1.x - __uint_as_float(f[d + 2]), rowsum * x1.y - __uint_as_float(f[d + 3]));
      }
    }
    if (hf == 0) {
      row_flags[t] = (row_valid && done) ? 1 : 0;
      if (KS == 2) row_loss[t] = loss;
    }
    if constexpr (KS == 2) {
      // the staged rows are read next by the bulk copy engine (async proxy)
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      epi_sync();
      asm volatile("barrier.cluster.wait.acquire.aligned;" ::: "memory");
      if (tid == 0) {
        // this CTA's incoming area is free and its INCOMING barrier expects the rows:
        // tell the peer (a release arrive on the peer's PEER_FREE barrier)
        mbar_expect_tx(B(INCOMING), kInBytes);
        mbar_arrive_remote(peer_addr(B(PEER_FREE), peer));
      }
      // warp 0 pushes the partials of the peer's 64 rows (one contiguous block
      // of staged rows), their flags and losses into the peer's shared memory
      // once the peer has staged its own rows, completing on the peer's
      // INCOMING barrier
      if (warp == 0 && __all_sync(kFull, mbar_wait_cluster(B(PEER_FREE), 0, &err))) {
        const int pr0 = peer * 64;
        const uint32_t pbar = peer_addr(B(INCOMING), peer);
        if (lane == 0) {
          bulk_s2peer(peer_addr(smem_u32(in_rows), peer), smem_u32(stage + pr0 * kPitch), kHalfRowsBytes, pbar);
          bulk_s2peer(peer_addr(smem_u32(in_flags), peer), smem_u32(&row_flags[pr0]), 64 * 4, pbar);
          bulk_s2peer(peer_addr(smem_u32(in_loss), peer), smem_u32(&row_loss[pr0]), 64 * 8, pbar);
        }
      }
    } else {
      epi_sync();
    }

    // Coalesced store of lr * force, one warp per row, lane l the 16-byte
    // vectors l, l + 32, ... (every store instruction writes whole 32-byte
    // sectors), into rbuf; bf16_apply_kernel adds it to the row together with
    // the attractive update (which runs concurrently into abuf).
    for (int rr = warp; KS == 1 && rr < kTileRows; rr += kEpiThreads / 32) {
      if (row_flags[rr] == 0) continue;
      const float4 *src = reinterpret_cast<const float4 *>(stage + rr * kPitch);
      float4 *rbp = reinterpret_cast<float4 *>(a.rbuf + size_t(tile_base + rr) * D);
#pragma unroll
      for (int v = lane; v < D / 4; v += 32) {
        const float4 f = src[v];
        rbp[v] = make_float4(lr * f.x, lr * f.y, lr * f.z, lr * f.w);
      }
    }
    if constexpr (KS == 2) {
      // this CTA's rows [64 ks, 64 ks + 64): own partial + the peer's
      const bool in_ok = __all_sync(kFull, mbar_wait_cluster(B(INCOMING), 0, &err));
      // the peer's copies into this CTA have landed, so the peer's staged rows
      // are no longer read: tell the peer at once
      if (tid == 0 && in_ok) mbar_arrive_remote(peer_addr(B(PEER_GOT), peer));
      const int r0 = ks * 64;
      for (int i = warp; in_ok && i < 64; i += kEpiThreads / 32) {
        if (row_flags[r0 + i] == 0 || in_flags[i] == 0) continue;
        const float4 *own = reinterpret_cast<const float4 *>(stage + (r0 + i) * kPitch);
        const float4 *oth = reinterpret_cast<const float4 *>(in_rows + i * kPitch);
        float4 *rbp = reinterpret_cast<float4 *>(a.rbuf + size_t(tile_base + r0 + i) * D);
#pragma unroll
        for (int v = lane; v < D / 4; v += 32) {
          const float4 p = own[v], q = oth[v];
          rbp[v] = make_float4(lr * (p.x + q.x), lr * (p.y + q.y), lr * (p.z + q.z), lr * (p.w + q.w));
        }
      }
      if (in_ok && tid < 64 && row_flags[r0 + tid] != 0 && in_flags[tid] != 0)
        a.loss_row[a.base + tile_base + r0 + tid] = row_loss[r0 + tid] + in_loss[tid];
      // the CTA (and its shared memory) ends only after the peer has received
      // this CTA's rows
      if (tid == 0) mbar_wait_cluster(B(PEER_GOT), 0, &err);
    }
  }
  if constexpr (KS == 2) {
    __syncwarp();
    if (warp >= kEpiThreads / 32) asm volatile("barrier.cluster.wait.acquire.aligned;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  if (failed() && tid == 0) atomicExch(a.err, 1);
  if (warp == 9) {
    __syncwarp();
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(512) : "memory");
  }
}

// ------------------------------------------------------------ update

// N consecutive floats through L2 (written by other kernels of this minibatch),
// in 16-byte vectors where N allows.
template <int N>
__device__ __forceinline__ void ld_contig(float (&v)[N], const float *p) {
  if constexpr (N % 4 == 0) {
#pragma unroll
    for (int i = 0; i < N; i += 4) {
      const float4 t = __ldcg(reinterpret_cast<const float4 *>(p + i));
      v[i] = t.x; v[i + 1] = t.y; v[i + 2] = t.z; v[i + 3] = t.w;
    }
  } else {
#pragma unroll
    for (int i = 0; i < N; i += 2) {
      const float2 t = __ldcg(reinterpret_cast<const float2 *>(p + i));
      v[i] = t.x; v[i + 1] = t.y;
    }
  }
}

template <int N>
__device__ __forceinline__ void st_contig(float *p, const float (&v)[N]) {
  if constexpr (N % 4 == 0) {
#pragma unroll
    for (int i = 0; i < N; i += 4) *reinterpret_cast<float4 *>(p + i) = make_float4(v[i], v[i + 1], v[i + 2], v[i + 3]);
  } else {
#pragma unroll
    for (int i = 0; i < N; i += 2) *reinterpret_cast<float2 *>(p + i) = make_float2(v[i], v[i + 1]);
  }
}

// One warp per row of the minibatch: x += abuf + rbuf (attractive and GEMM
// repulsive updates, algo.hpp:651-666), plus, for a row with exact-path pairs
// (bitmask bits), those pairs added in FP32 on the BF16 values with the
// per-component clip (algo.hpp:633-645), in negative order; the bits are cleared.
template <int D>
__global__ void __launch_bounds__(256) bf16_apply_kernel(const BF16BatchArgs a) {
  const int lane = threadIdx.x & 31;
  const int gw = blockIdx.x * 8 + (threadIdx.x >> 5);
  const int epoch = a.epoch[0];
  const float lr = a.lr[epoch];
  constexpr int N = D / 32;
  for (int row_local = gw; row_local < a.rows; row_local += gridDim.x * 8) {
    const int row = a.base + row_local;
    uint32_t *bits_row = a.near_bits + size_t(row_local) * kNearWords;
    // every load of the row at once: the bitmask, the row's CSR extent, the master
    // row and both updates (the attractive one is used only for rows with CSR
    // entries: other rows' slots hold an earlier minibatch's values)
    const uint32_t my_word = lane < kNearWords ? bits_row[lane] : 0u;
    const bool has_attr = __ldg(a.rowptr + row + 1) > __ldg(a.rowptr + row);
    float *xm = a.xm + size_t(row) * D + lane * N;
    __nv_bfloat16 *xb = a.xb + size_t(row) * D + lane * N;
    float mv[N], av[N], rv[N];
    ld_contig<N>(mv, xm);
    ld_contig<N>(av, a.abuf + size_t(row_local) * D + lane * N);
    ld_contig<N>(rv, a.rbuf + size_t(row_local) * D + lane * N);
    Frag<D> acc;
    acc.zero();
    const bool exact = __any_sync(kFull, my_word != 0u);
    if (exact) {
      Frag<D> xi;
      load_bf16_row(xi, a.xb + size_t(row) * D, lane);
      float loss = 0.f;
      for (int w = 0; w < kNearWords; ++w) {
        uint32_t bits = __shfl_sync(kFull, my_word, w);
        while (bits) {
          const int i = __ffs(bits) - 1;
          bits &= bits - 1;
          const int k = (w >> 1) * kChunk + (w & 1) * 32 + i;  // word w = 2 * chunk + half
          Frag<D> xn;
          load_bf16_row(xn, a.nb + size_t(k) * D, lane);
          float diff[N];
          float p = 0.f;
#pragma unroll
          for (int t = 0; t < N; ++t) {
            diff[t] = xi.v[t] - xn.v[t];
            p = fmaf(diff[t], diff[t], p);
          }
#pragma unroll
          for (int o = 16; o > 0; o >>= 1) p += __shfl_xor_sync(kFull, p, o);
          const float c = 2.0f / ((p + 1e-6f) * (1.0f + p));
#pragma unroll
          for (int t = 0; t < N; ++t) acc.v[t] = fmaf(lr, clip(diff[t] * c, a.bound), acc.v[t]);
          loss += logf((1.0f + p) / (p + 1e-6f));
        }
      }
      if (lane < kNearWords) bits_row[lane] = 0u;
      if (lane == 0) a.loss_row[row] += double(loss);
    }
    // lane: N consecutive components, moved as 16-byte vectors (8-byte at dim 64)
#pragma unroll
    for (int t = 0; t < N; ++t) {
      mv[t] = mv[t] + ((has_attr ? av[t] : 0.f) + rv[t]);
      if (exact) mv[t] = mv[t] + acc.v[t];
    }
    st_contig<N>(xm, mv);
    uint32_t hb[N / 2];
#pragma unroll
    for (int t = 0; t < N; t += 2) {
      const __nv_bfloat162 h2 = __floats2bfloat162_rn(mv[t], mv[t + 1]);
      hb[t / 2] = *reinterpret_cast<const uint32_t *>(&h2);
    }
    if constexpr (N == 8) *reinterpret_cast<uint4 *>(xb) = make_uint4(hb[0], hb[1], hb[2], hb[3]);
    else if constexpr (N == 4) *reinterpret_cast<uint2 *>(xb) = make_uint2(hb[0], hb[1]);
    else *reinterpret_cast<uint32_t *>(xb) = hb[0];
  }
}

// ------------------------------------------------------------ epoch end

__global__ void __launch_bounds__(256) bf16_flush_kernel(const BF16FlushArgs a) {
  __shared__ double red[256];
  __shared__ bool last;
  double s = 0.0;
  if (a.compute_loss) {
    const int64_t total = a.n_items + a.n_rows;
    const int64_t chunk = (total + gridDim.x - 1) / gridDim.x;
    const int64_t lo = blockIdx.x * chunk, hi = min(total, lo + chunk);
    for (int64_t i = lo + threadIdx.x; i < hi; i += 256) s += i < a.n_items ? a.loss_item[i] : a.loss_row[i - a.n_items];
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

__global__ void f32_to_bf16_kernel(const float *__restrict__ s, __nv_bfloat16 *__restrict__ d, int64_t n) {
  for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x)
    d[i] = __float2bfloat16(s[i]);
}

}  // namespace

int bf16_repulse_smem_bytes(int dim) {
  switch (dim) {
    case 64: return RepulseSmem<64>::dynamic;
    case 128: return RepulseSmem<128>::dynamic;
    case 256: return RepulseSmem<256>::dynamic;
  }
  return -1;
}

namespace {
template <int D>
cudaError_t prepare_d() {
  cudaError_t e = cudaFuncSetAttribute(bf16_repulse_kernel<D, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       RepulseSmem<D>::dynamic);
  if (e != cudaSuccess) return e;
  return cudaFuncSetAttribute(bf16_repulse_kernel<D, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              RepulseSmem<D>::dynamic);
}
}  // namespace

cudaError_t bf16_prepare(int dim) {
  switch (dim) {
    case 64: return prepare_d<64>();
    case 128: return prepare_d<128>();
    case 256: return prepare_d<256>();
  }
  return cudaErrorInvalidValue;
}

namespace {

// The repulsion GEMMs of a minibatch: one CTA per 128-row tile, or, with at
// least two chunks of negatives, a cluster of two CTAs per tile that split them.
template <int D>
cudaError_t launch_repulse(const BF16BatchArgs &a, const CUtensorMap &mx, const CUtensorMap &mn, int tiles,
                           cudaStream_t s) {
  if (a.kpad / kChunk < 2) {
    bf16_repulse_kernel<D, 1><<<tiles, kRepulseThreads, RepulseSmem<D>::dynamic, s>>>(mx, mn, a);
    return cudaGetLastError();
  }
  cudaLaunchConfig_t cfg{};
  cfg.gridDim = dim3(2 * tiles);
  cfg.blockDim = dim3(kRepulseThreads);
  cfg.dynamicSmemBytes = RepulseSmem<D>::dynamic;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = 2;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, bf16_repulse_kernel<D, 2>, mx, mn, a);
}

template <int D, int U>
cudaError_t launch_bf16_batch_d(const BF16BatchArgs &a, const CUtensorMap &mx, const CUtensorMap &mn,
                                cudaStream_t s, cudaEvent_t *ev, cudaStream_t s2,
                                cudaEvent_t fork, cudaEvent_t join) {
  const int item_ctas = (a.n_items + kPlainWarps - 1) / kPlainWarps;
  const int gather_ctas = a.kpad / kGatherTile;  // kpad: a multiple of 64
  const int tiles = (a.rows + kTileRows - 1) / kTileRows;
  const int apply_ctas = (a.rows + 7) / 8;
  cudaError_t e = cudaSuccess;
  if (ev || !s2) {  // one after another (per-kernel timing)
    if (ev) cudaEventRecord(ev[0], s);
    bf16_gather_kernel<D><<<gather_ctas, kGatherTile * 32, 0, s>>>(a);
    if (ev) cudaEventRecord(ev[1], s);
    bf16_attract_kernel<D, U><<<item_ctas, kPlainWarps * 32, 0, s>>>(a);
    if (ev) cudaEventRecord(ev[2], s);
    if ((e = launch_repulse<D>(a, mx, mn, tiles, s)) != cudaSuccess) return e;
    if (ev) cudaEventRecord(ev[3], s);
    bf16_apply_kernel<D><<<apply_ctas, 256, 0, s>>>(a);
    return cudaGetLastError();
  }
  // the attractive pass and the negatives' path (gather, repulsion GEMMs) are
  // independent within a minibatch: they run on two streams, forked after the
  // previous minibatch's update and joined before this one's
  if ((e = cudaEventRecord(fork, s)) != cudaSuccess || (e = cudaStreamWaitEvent(s2, fork, 0)) != cudaSuccess) return e;
  bf16_gather_kernel<D><<<gather_ctas, kGatherTile * 32, 0, s2>>>(a);
  if ((e = launch_repulse<D>(a, mx, mn, tiles, s2)) != cudaSuccess) return e;
  bf16_attract_kernel<D, U><<<item_ctas, kPlainWarps * 32, 0, s>>>(a);
  if ((e = cudaEventRecord(join, s2)) != cudaSuccess || (e = cudaStreamWaitEvent(s, join, 0)) != cudaSuccess) return e;
  bf16_apply_kernel<D><<<apply_ctas, 256, 0, s>>>(a);
  return cudaGetLastError();
}

}  // namespace

cudaError_t launch_bf16_batch(int dim, const BF16BatchArgs &a, const CUtensorMap &mx, const CUtensorMap &mn,
                              cudaStream_t s, cudaEvent_t *ev, cudaStream_t s2,
                              cudaEvent_t fork, cudaEvent_t join) {
  switch (dim) {
    case 64: return launch_bf16_batch_d<64, 8>(a, mx, mn, s, ev, s2, fork, join);
    case 128: return launch_bf16_batch_d<128, 8>(a, mx, mn, s, ev, s2, fork, join);
    case 256: return launch_bf16_batch_d<256, 4>(a, mx, mn, s, ev, s2, fork, join);
  }
  return cudaErrorInvalidValue;
}

cudaError_t launch_bf16_flush(const BF16FlushArgs &a, cudaStream_t s) {
  bf16_flush_kernel<<<kFlushBlocks, 256, 0, s>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_f32_to_bf16(const float *src, __nv_bfloat16 *dst, int64_t count, cudaStream_t s) {
  if (count <= 0) return cudaSuccess;
  const int grid = int(count / 256 + 1 < 152 * 8 ? count / 256 + 1 : 152 * 8);
  f32_to_bf16_kernel<<<grid, 256, 0, s>>>(src, dst, count);
  return cudaGetLastError();
}

}  // namespace de
