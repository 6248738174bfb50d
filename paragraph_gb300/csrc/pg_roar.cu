// pg_roar.cu -- ParaGraph's CPU RoarGraph path (MatchSup rounds, FusionNN) and the final fusion
// (FusionFinal) as GPU kernels (sm_103a).
//
// Reference: tests/test_t2iend.cu, the CPU code its driver runs beside the GPU build --
// compare :31-80, RNGPrune :99-177, MatchSup :365-488, FusionNN :490-537, FusionFinal :539-613.
// Results equal the reference's one-thread run id for id:
//   * distances follow compare()'s AVX-512 FP32 order: 16 FMA lanes over 16-wide chunks, folded
//     8+8, an 8-wide FMA step, folded 4+4, a 4-wide step, then ((s0+s1)+(s2+s3)) -- each lane of
//     a warp computes whole distances in that order;
//   * candidate lists are sorted by (distance, id), SimpleNeighbor's order (:82-91), with one warp
//     bitonic sort of 64-bit keys (ordered distance << 32 | id);
//   * RNGPrune's scan is sequential over the sorted list; the lanes test one candidate against all
//     kept entries at once (ballot).  Its second "double check" scan (:142-165) is not run: every
//     candidate it revisits was kept already or is occluded by the same kept entry as before;
//   * MatchSup's reverse appends keep, per base, the first 128 - M_nn sources in ascending query
//     order (the reference's one-thread order), through the same count/scan/scatter/sort CSR as
//     the link rounds; a merged list too short to be pruned is written in ascending id order (the
//     reference writes std::unordered_set order, which no consumer depends on).
// One warp per node or query, eight warps per block, per-warp lists in shared memory.
#include "pg_device.cuh"
#include "pg_kernels.h"

namespace pg {

namespace {

constexpr int kRoarWarps = 8;
constexpr uint32_t kRoarCap = 256;  // candidates per node
constexpr uint32_t kRoarRes = 128;  // kept entries per node

struct RoarSmem {
  uint32_t cand[kRoarCap];
  uint32_t sid[kRoarCap];
  float sdist[kRoarCap];
  uint32_t res[kRoarRes];
  uint32_t fin[kRoarCap + kRoarRes];
};

__device__ __forceinline__ const float* row_of(const float* base, uint32_t d, uint32_t id) {
  return base + static_cast<uint64_t>(id) * d;
}

// compare() (tests/test_t2iend.cu:31-80), the negated inner product in its exact FP32 order --
// 16 accumulators over 16-wide chunks, folded 8+8, an 8-wide FMA step, folded 4+4, a 4-wide
// step, then ((s0 + s1) + (s2 + s3)) -- computed by a group of 8 lanes: lane l of the group holds
// the accumulators of elements 16c + l and 16c + 8 + l, so the 8+8 fold happens in the lane, the
// 4+4 fold and the two horizontal adds by shuffles inside the group.  Every lane of the warp
// calls it (the shuffles are warp-wide); the distance is valid in lane 0 of each group; the
// group's loads are contiguous.
__device__ __forceinline__ float dist_avx8(const float* __restrict__ a,
                                           const float* __restrict__ b, uint32_t d, uint32_t l8) {
  float lo = 0.0f, hi = 0.0f;
  uint32_t i = 0;
#pragma unroll 4
  for (; i + 16 <= d; i += 16) {
    lo = fmaf(__ldg(a + i + l8), __ldg(b + i + l8), lo);
    hi = fmaf(__ldg(a + i + 8 + l8), __ldg(b + i + 8 + l8), hi);
  }
  float s8 = hi + lo;
  if (d - i >= 8) {
    s8 = fmaf(__ldg(a + i + l8), __ldg(b + i + l8), s8);
    i += 8;
  }
  float s4 = __shfl_down_sync(kFull, s8, 4, 8) + s8;
  if (d - i >= 4 && l8 < 4) s4 = fmaf(__ldg(a + i + l8), __ldg(b + i + l8), s4);
  const float pr = s4 + __shfl_down_sync(kFull, s4, 1, 8);
  return -(pr + __shfl_down_sync(kFull, pr, 2, 8));
}

// Two dist_avx8 at once (a against b0 and against b1), for twice the loads in flight.
__device__ __forceinline__ void dist_avx8x2(const float* __restrict__ a,
                                            const float* __restrict__ b0,
                                            const float* __restrict__ b1, uint32_t d, uint32_t l8,
                                            float& r0, float& r1) {
  float lo0 = 0.0f, hi0 = 0.0f, lo1 = 0.0f, hi1 = 0.0f;
  uint32_t i = 0;
#pragma unroll 2
  for (; i + 16 <= d; i += 16) {
    const float x0 = __ldg(a + i + l8), x1 = __ldg(a + i + 8 + l8);
    lo0 = fmaf(x0, __ldg(b0 + i + l8), lo0);
    hi0 = fmaf(x1, __ldg(b0 + i + 8 + l8), hi0);
    lo1 = fmaf(x0, __ldg(b1 + i + l8), lo1);
    hi1 = fmaf(x1, __ldg(b1 + i + 8 + l8), hi1);
  }
  float s0 = hi0 + lo0, s1 = hi1 + lo1;
  if (d - i >= 8) {
    const float x = __ldg(a + i + l8);
    s0 = fmaf(x, __ldg(b0 + i + l8), s0);
    s1 = fmaf(x, __ldg(b1 + i + l8), s1);
    i += 8;
  }
  float t0 = __shfl_down_sync(kFull, s0, 4, 8) + s0;
  float t1 = __shfl_down_sync(kFull, s1, 4, 8) + s1;
  if (d - i >= 4 && l8 < 4) {
    const float x = __ldg(a + i + l8);
    t0 = fmaf(x, __ldg(b0 + i + l8), t0);
    t1 = fmaf(x, __ldg(b1 + i + l8), t1);
  }
  const float p0 = t0 + __shfl_down_sync(kFull, t0, 1, 8);
  const float p1 = t1 + __shfl_down_sync(kFull, t1, 1, 8);
  r0 = -(p0 + __shfl_down_sync(kFull, p0, 2, 8));
  r1 = -(p1 + __shfl_down_sync(kFull, p1, 2, 8));
}

// Replaces every repeat of an earlier id in cand[0..len) by tomb (first occurrences stay): a sort
// of (id << 32 | position) keys puts the repeats of an id right after its first occurrence.
template <int E>
__device__ void dedupe_first(uint32_t* cand, uint32_t len) {
  const uint32_t lane = lane_id();
  uint64_t key[E];
  uint32_t val[E];
#pragma unroll
  for (int s = 0; s < E; s++) {
    const uint32_t i = static_cast<uint32_t>(s) * 32u + lane;
    const uint32_t x = i < len ? cand[i] : kTomb;
    key[s] = x != kTomb ? ((static_cast<uint64_t>(x) << 32) | i) : ~0ull;
    val[s] = i;
  }
  warp_sort_kv<E>(key, val);
  __syncwarp();
#pragma unroll
  for (int s = 0; s < E; s++) {
    const uint64_t up = __shfl_up_sync(kFull, key[s], 1);
    const uint64_t wrap = s > 0 ? __shfl_sync(kFull, key[s > 0 ? s - 1 : 0], 31) : ~0ull;
    const uint64_t prev = lane == 0 ? wrap : up;
    if (key[s] != ~0ull && prev != ~0ull && (prev >> 32) == (key[s] >> 32))
      cand[static_cast<uint32_t>(key[s])] = kTomb;
  }
  __syncwarp();
}

// Distances from `node` to the non-tomb ids of cand[0..len), sorted by (distance, id) into
// sid/sdist; returns their number.  With `unique`, repeats of an id are dropped (they carry the
// same distance, so they sit next to each other after the sort).
template <int E>
__device__ uint32_t sort_by_dist(const float* base, uint32_t d, uint32_t node,
                                 const uint32_t* cand, uint32_t len, uint32_t* sid, float* sdist,
                                 bool unique) {
  const uint32_t lane = lane_id(), g = lane >> 3, l8 = lane & 7u;
  const float* nrow = row_of(base, d, node);
  for (uint32_t i0 = 0; i0 < len; i0 += 8) {  // eight distances per pass, two per 8-lane group
    const uint32_t i = i0 + g, j = i0 + 4 + g;
    const uint32_t x = i < len ? cand[i] : kTomb;
    const uint32_t y = j < len ? cand[j] : kTomb;
    float dx, dy;
    dist_avx8x2(nrow, row_of(base, d, x != kTomb ? x : node), row_of(base, d, y != kTomb ? y : node),
                d, l8, dx, dy);
    if (l8 == 0 && x != kTomb) sdist[i] = dx;
    if (l8 == 0 && y != kTomb) sdist[j] = dy;
  }
  __syncwarp();
  uint64_t key[E];
  uint32_t val[E];
#pragma unroll
  for (int s = 0; s < E; s++) {
    const uint32_t i = static_cast<uint32_t>(s) * 32u + lane;
    const uint32_t x = i < len ? cand[i] : kTomb;
    key[s] = ~0ull;
    val[s] = 0;
    if (x != kTomb) {
      const float dist = sdist[i];
      key[s] = (static_cast<uint64_t>(order_key(dist)) << 32) | x;
      val[s] = __float_as_uint(dist);
    }
  }
  __syncwarp();
  warp_sort_kv<E>(key, val);
  uint32_t cnt = 0;
#pragma unroll
  for (int s = 0; s < E; s++) {
    const uint64_t up = __shfl_up_sync(kFull, key[s], 1);
    const uint64_t wrap = s > 0 ? __shfl_sync(kFull, key[s > 0 ? s - 1 : 0], 31) : ~0ull;
    const uint64_t prev = lane == 0 ? wrap : up;
    const bool keep = key[s] != ~0ull && !(unique && prev == key[s]);
    const unsigned m = __ballot_sync(kFull, keep);
    if (keep) {
      const uint32_t pos = cnt + __popc(m & ((1u << lane) - 1u));
      sid[pos] = static_cast<uint32_t>(key[s]);
      sdist[pos] = __uint_as_float(val[s]);
    }
    cnt += __popc(m);
  }
  __syncwarp();
  return cnt;
}

template <int E>
__device__ __forceinline__ uint32_t sort_by_dist_any(const float* base, uint32_t d, uint32_t node,
                                                     const uint32_t* cand, uint32_t len,
                                                     uint32_t* sid, float* sdist,
                                                     bool unique = false) {
  if (len <= 32) return sort_by_dist<1>(base, d, node, cand, len, sid, sdist, unique);
  if (len <= 64) return sort_by_dist<2>(base, d, node, cand, len, sid, sdist, unique);
  if (len <= 128) return sort_by_dist<4>(base, d, node, cand, len, sid, sdist, unique);
  return sort_by_dist<E>(base, d, node, cand, len, sid, sdist, unique);
}

__device__ __forceinline__ void dedupe_any(uint32_t* cand, uint32_t len) {
  if (len <= 32)
    dedupe_first<1>(cand, len);
  else if (len <= 64)
    dedupe_first<2>(cand, len);
  else if (len <= 128)
    dedupe_first<4>(cand, len);
  else
    dedupe_first<8>(cand, len);
}

__device__ __forceinline__ bool warp_contains(const uint32_t* a, uint32_t k, uint32_t x) {
  bool in = false;
  for (uint32_t t = lane_id(); t < k; t += 32) in |= a[t] == x;
  return __ballot_sync(kFull, in) != 0;
}

// RNGPrune (tests/test_t2iend.cu:99-177) over sid/sdist[0..c); kept ids in res, returns their
// number (M <= kRoarRes).
__device__ uint32_t rng_prune_warp(const float* base, uint32_t d, uint64_t n, uint32_t M,
                                   const uint32_t* sid, const float* sdist, uint32_t c,
                                   uint32_t target, bool strict, uint32_t* res) {
  const uint32_t lane = lane_id();
  uint32_t start = 0;
  while (start < c && sid[start] == target) start++;
  if (start == c) return 0;
  if (lane == 0) res[0] = sid[start];
  __syncwarp();
  uint32_t k = 1;
  const uint32_t g = lane >> 3, l8 = lane & 7u;
  // The scan decides the candidates in order; four of them (a window, one per 8-lane group) are
  // tested at once against the kept entries each has not been tested against yet.  The first
  // candidate of the window that no kept entry occludes is kept; the ones before it are dropped,
  // the ones after it stay in the window and are next tested against the new entry only.
  uint32_t w[4], tested[4];
  uint32_t wn = 0, next = start + 1;
  while (k < M) {
#pragma unroll
    for (int e = 0; e < 4; e++)
      if (static_cast<uint32_t>(e) == wn && next < c) {
        w[e] = next++;
        tested[e] = 0;
        wn++;
      }
    if (wn == 0) break;
    uint32_t my_w = w[0], my_t = tested[0], span = 0;
#pragma unroll
    for (int e = 0; e < 4; e++) {
      if (static_cast<uint32_t>(e) < wn) span = max(span, k - tested[e]);
      if (static_cast<uint32_t>(e) == g) {
        my_w = w[e];
        my_t = tested[e];
      }
    }
    const bool mine = g < wn;
    const uint32_t p = sid[mine ? my_w : w[0]];
    const float pd = sdist[mine ? my_w : w[0]];
    const float* prow = row_of(base, d, p);
    bool occ = false;
    for (uint32_t u = 0; u < span; u++) {
      const uint32_t t = my_t + u;
      const bool act = mine && t < k;
      const uint32_t r = act ? res[t] : res[0];
      const float dist = dist_avx8(prow, row_of(base, d, r), d, l8);
      occ |= act && l8 == 0 && (r == p || dist < pd);
    }
    const unsigned bits = __ballot_sync(kFull, occ);
    const uint32_t k_old = k;
    int kept = -1;
#pragma unroll
    for (int e = 0; e < 4; e++) {
      if (kept < 0 && static_cast<uint32_t>(e) < wn && ((bits >> (8 * e)) & 1u) == 0) {
        const uint32_t x = sid[w[e]];
        if (x != target) {  // not occluded: kept (the node itself never is, :133-137)
          if (lane == 0) res[k] = x;
          k++;
          kept = e;
        }
      }
    }
    __syncwarp();
    // the window keeps the entries after the kept one that nothing occludes yet, tested against
    // res[0 .. k_old); the occluded ones are decided
    uint32_t nw = 0;
    uint32_t w2[4], t2[4];
#pragma unroll
    for (int e = 0; e < 4; e++) {
      w2[e] = 0;
      t2[e] = 0;
    }
#pragma unroll
    for (int e = 0; e < 4; e++) {
      if (kept >= 0 && e > kept && static_cast<uint32_t>(e) < wn &&
          ((bits >> (8 * e)) & 1u) == 0) {
#pragma unroll
        for (int f = 0; f < 4; f++)
          if (static_cast<uint32_t>(f) == nw) {
            w2[f] = w[e];
            t2[f] = k_old;
          }
        nw++;
      }
    }
#pragma unroll
    for (int e = 0; e < 4; e++) {
      w[e] = w2[e];
      tested[e] = t2[e];
    }
    wn = nw;
  }
  if (!strict) {  // :168-176
    for (uint32_t i = 1; i < c && k < M; i++) {
      const uint32_t x = sid[i];
      if (!warp_contains(res, k, x) && x < n && x != target) {
        if (lane == 0) res[k] = x;
        k++;
        __syncwarp();
      }
    }
  }
  __syncwarp();
  return k;
}

// The u non-tomb ids of cand[0..len) in ascending order into out.
template <int E>
__device__ __forceinline__ void write_ascending(const uint32_t* cand, uint32_t len, uint32_t u,
                                                uint32_t* out) {
  const uint32_t lane = lane_id();
  uint32_t v[E];
#pragma unroll
  for (int s = 0; s < E; s++) {
    const uint32_t i = static_cast<uint32_t>(s) * 32u + lane;
    v[s] = i < len ? cand[i] : kTomb;
  }
  warp_sort_u32<E>(v);
#pragma unroll
  for (int s = 0; s < E; s++) {
    const uint32_t i = static_cast<uint32_t>(s) * 32u + lane;
    if (i < u) out[i] = v[s];
  }
}

__device__ __forceinline__ RoarSmem* warp_smem(RoarSmem* all) {
  return all + (threadIdx.x >> 5);
}

__device__ __forceinline__ uint64_t warp_global() {
  return blockIdx.x * static_cast<uint64_t>(kRoarWarps) + (threadIdx.x >> 5);
}

__device__ __forceinline__ uint64_t warp_count() {
  return static_cast<uint64_t>(gridDim.x) * kRoarWarps;
}

// ---- MatchSup (:365-488) ------------------------------------------------------------------

// :378-392: query q claims base gt[q][topn] when no lower query did (the one-thread order).
__global__ void k_sup_claim(const uint32_t* __restrict__ gt, uint64_t q, uint32_t gt_k,
                            uint32_t topn, uint64_t n, uint32_t* __restrict__ claim) {
  const uint64_t stride = static_cast<uint64_t>(gridDim.x) * blockDim.x;
  for (uint64_t i = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x; i < q;
       i += stride) {
    const uint32_t nn = gt[i * gt_k + topn];
    if (nn < n) atomicMin(claim + nn, static_cast<uint32_t>(i));
  }
}

// :407-441: each matched query prunes its ground-truth list around its base (non-strict).
__global__ void __launch_bounds__(kRoarWarps * 32) k_sup_prune(SupArgs a) {
  __shared__ RoarSmem sm_all[kRoarWarps];
  RoarSmem* sm = warp_smem(sm_all);
  const uint32_t lane = lane_id();
  for (uint64_t qi = warp_global(); qi < a.q; qi += warp_count()) {
    const uint32_t* row = a.gt + qi * a.gt_k;
    const uint32_t nn = row[a.topn];
    const bool matched = nn < a.n && a.claim[nn] == static_cast<uint32_t>(qi);
    if (!matched) {
      if (lane == 0) a.pcnt[qi] = 0;
      continue;
    }
    // candidates: the row up to its first id >= n, without the base itself
    uint32_t stop = a.gt_k;
    for (uint32_t c0 = 0; c0 < a.gt_k; c0 += 32) {
      const uint32_t i = c0 + lane;
      const unsigned bad = __ballot_sync(kFull, i < a.gt_k && row[i] >= a.n);
      if (bad) {
        stop = c0 + static_cast<uint32_t>(__ffs(static_cast<int>(bad)) - 1);
        break;
      }
    }
    for (uint32_t i = lane; i < a.gt_k; i += 32) {
      const uint32_t x = row[i];
      sm->cand[i] = (i < stop && x != nn) ? x : kTomb;
    }
    __syncwarp();
    const uint32_t c =
        sort_by_dist_any<8>(a.base, a.d, nn, sm->cand, a.gt_k, sm->sid, sm->sdist, true);
    const uint32_t k =
        rng_prune_warp(a.base, a.d, a.n, a.m_nn, sm->sid, sm->sdist, c, nn, false, sm->res);
    for (uint32_t i = lane; i < k; i += 32) {
      const uint32_t x = sm->res[i];
      a.plist[qi * a.m_nn + i] = x;
      atomicAdd(a.indeg + x, 1u);
    }
    if (lane == 0) a.pcnt[qi] = k;
    __syncwarp();
  }
}

// :449-475: a base's own pruned list joined with its first 128 - M_nn reverse sources; pruned
// (strict) when longer than M_nn.
__global__ void __launch_bounds__(kRoarWarps * 32) k_sup_merge(SupArgs a) {
  __shared__ RoarSmem sm_all[kRoarWarps];
  RoarSmem* sm = warp_smem(sm_all);
  const uint32_t lane = lane_id();
  for (uint64_t b = warp_global(); b < a.n; b += warp_count()) {
    const uint32_t owner = a.claim[b];
    const uint32_t k1 = owner < a.q ? a.pcnt[owner] : 0u;
    const uint32_t r = a.rnum[b];
    for (uint32_t i = lane; i < k1; i += 32)
      sm->cand[i] = a.plist[static_cast<uint64_t>(owner) * a.m_nn + i];
    for (uint32_t i = lane; i < r; i += 32) {
      const uint64_t src = a.rev[b * a.maxdeg + i];
      sm->cand[k1 + i] = a.gt[src * a.gt_k + a.topn];
    }
    const uint32_t len = k1 + r;
    if (len == 0) {
      if (lane == 0) a.cnt[b] = 0;
      continue;
    }
    __syncwarp();
    dedupe_any(sm->cand, len);
    uint32_t u = 0;
    for (uint32_t c0 = 0; c0 < len; c0 += 32)
      u += __popc(__ballot_sync(kFull, c0 + lane < len && sm->cand[c0 + lane] != kTomb));
    uint32_t* out = a.out + b * a.m_nn;
    if (u > a.m_nn) {
      const uint32_t c = sort_by_dist_any<8>(a.base, a.d, static_cast<uint32_t>(b), sm->cand, len,
                                             sm->sid, sm->sdist);
      const uint32_t k = rng_prune_warp(a.base, a.d, a.n, a.m_nn, sm->sid, sm->sdist, c,
                                        static_cast<uint32_t>(b), true, sm->res);
      for (uint32_t i = lane; i < k; i += 32) out[i] = sm->res[i];
      if (lane == 0) a.cnt[b] = k;
    } else {  // at most M_nn ids: ascending
      if (len <= 32)
        write_ascending<1>(sm->cand, len, u, out);
      else if (len <= 64)
        write_ascending<2>(sm->cand, len, u, out);
      else
        write_ascending<4>(sm->cand, len, u, out);
      if (lane == 0) a.cnt[b] = u;
    }
    __syncwarp();
  }
}

// ---- FusionNN (:490-537) ------------------------------------------------------------------

__global__ void __launch_bounds__(kRoarWarps * 32) k_fusion_nn(FusionArgs a) {
  __shared__ RoarSmem sm_all[kRoarWarps];
  RoarSmem* sm = warp_smem(sm_all);
  const uint32_t lane = lane_id();
  for (uint64_t b = warp_global(); b < a.n; b += warp_count()) {
    uint32_t len = 0;
    for (uint32_t r = 0; r < a.rounds; r++) {
      const uint64_t rb = static_cast<uint64_t>(r) * a.n + b;
      const uint32_t k = min(a.sup_cnt[rb], a.sup_stride);
      const uint32_t* row = a.sup + rb * a.sup_stride;
      for (uint32_t i = lane; i < k; i += 32) {
        const uint32_t x = row[i];
        sm->cand[len + i] = (x < a.n && x != static_cast<uint32_t>(b)) ? x : kTomb;
      }
      len += k;
    }
    __syncwarp();
    const uint32_t c = sort_by_dist_any<8>(a.base, a.d, static_cast<uint32_t>(b), sm->cand, len,
                                           sm->sid, sm->sdist, true);
    const uint32_t k = rng_prune_warp(a.base, a.d, a.n, a.m_out, sm->sid, sm->sdist, c,
                                      static_cast<uint32_t>(b), true, sm->res);
    for (uint32_t i = lane; i < k; i += 32) a.out[b * a.out_stride + i] = sm->res[i];
    if (lane == 0) a.cnt[b] = k;
    __syncwarp();
  }
}

// ---- FusionFinal (:539-613) ---------------------------------------------------------------

__global__ void __launch_bounds__(kRoarWarps * 32) k_fusion_final(FusionArgs a) {
  __shared__ RoarSmem sm_all[kRoarWarps];
  RoarSmem* sm = warp_smem(sm_all);
  const uint32_t lane = lane_id();
  for (uint64_t b = warp_global(); b < a.n; b += warp_count()) {
    const uint32_t self = static_cast<uint32_t>(b);
    const uint32_t* brow;
    uint32_t blen;
    if (a.bip_off) {
      brow = a.bip + a.bip_off[b];
      blen = static_cast<uint32_t>(a.bip_off[b + 1] - a.bip_off[b]);
    } else {
      brow = a.bip + b * a.bip_stride;
      blen = min(a.bip_cnt[b], a.bip_stride);
    }
    const uint32_t len = blen + a.m_link + a.m_supply;
    if (len > kRoarCap) {  // more candidates than the kernel holds: flag and leave the row empty
      if (lane == 0) {
        raise_error(a.status, kErrCapacity);
        a.cnt[b] = 0;
      }
      continue;
    }
    // the bipartite ids (not the node, < n), then the link ids (< n; the node itself is not
    // skipped, :568-576), then the projection ids (not the node, < n); repeats of any earlier id
    // dropped
    for (uint32_t i = lane; i < blen; i += 32) {
      const uint32_t x = brow[i];
      sm->cand[i] = (x < a.n && x != self) ? x : kTomb;
    }
    for (uint32_t i = lane; i < a.m_link; i += 32) {
      const uint32_t x = a.link[b * a.m_link + i];
      sm->cand[blen + i] = x < a.n ? x : kTomb;
    }
    for (uint32_t i = lane; i < a.m_supply; i += 32) {
      const uint32_t x = a.supply[b * a.m_supply + i];
      sm->cand[blen + a.m_link + i] = (x < a.n && x != self) ? x : kTomb;
    }
    __syncwarp();
    dedupe_any(sm->cand, len);
    // the final list starts with the surviving bipartite ids, in order
    uint32_t nbip = 0;
    for (uint32_t c0 = 0; c0 < blen; c0 += 32) {
      const uint32_t i = c0 + lane;
      const bool keep = i < blen && sm->cand[i] != kTomb;
      const unsigned m = __ballot_sync(kFull, keep);
      if (keep) sm->fin[nbip + __popc(m & ((1u << lane) - 1u))] = sm->cand[i];
      nbip += __popc(m);
    }
    __syncwarp();
    const uint32_t c = sort_by_dist_any<8>(a.base, a.d, self, sm->cand, len, sm->sid, sm->sdist);
    const uint32_t k =
        rng_prune_warp(a.base, a.d, a.n, a.m_out, sm->sid, sm->sdist, c, self, true, sm->res);
    // then the pruned ids not listed yet, up to m_final - nbip of them (an unsigned difference:
    // unlimited when the bipartite ids outnumber m_final, :599-606)
    const uint32_t slots = a.m_out >= nbip ? a.m_out - nbip : 0xFFFFFFFFu;
    uint32_t nf = nbip, added = 0;
    for (uint32_t i = 0; i < k && added < slots; i++) {
      const uint32_t x = sm->res[i];
      if (!warp_contains(sm->fin, nbip, x)) {
        if (lane == 0) sm->fin[nf] = x;
        nf++;
        added++;
        __syncwarp();
      }
    }
    __syncwarp();
    if (nf > a.out_stride) {
      if (lane == 0) {
        raise_error(a.status, kErrCapacity);
        a.cnt[b] = 0;
      }
      continue;
    }
    for (uint32_t i = lane; i < nf; i += 32) a.out[b * a.out_stride + i] = sm->fin[i];
    if (lane == 0) a.cnt[b] = nf;
    __syncwarp();
  }
}

int roar_grid(uint64_t items, int num_sms) {
  uint64_t blocks = (items + kRoarWarps - 1) / kRoarWarps;
  const uint64_t cap = static_cast<uint64_t>(num_sms) * 8;
  if (blocks > cap) blocks = cap;
  return static_cast<int>(blocks ? blocks : 1);
}

}  // namespace

bool roar_supported(uint32_t d, uint32_t m) { return d > 0 && d % 4 == 0 && m >= 1 && m <= kRoarRes; }

uint32_t roar_capacity() { return kRoarCap; }

cudaError_t launch_sup_claim(const uint32_t* gt, uint64_t q, uint32_t gt_k, uint32_t topn,
                             uint64_t n, uint32_t* claim, int num_sms, cudaStream_t st) {
  cudaError_t e = cudaMemsetAsync(claim, 0xFF, n * sizeof(uint32_t), st);
  if (e != cudaSuccess) return e;
  uint64_t blocks = (q + 255) / 256;
  if (blocks > static_cast<uint64_t>(num_sms) * 8) blocks = static_cast<uint64_t>(num_sms) * 8;
  k_sup_claim<<<static_cast<unsigned>(blocks ? blocks : 1), 256, 0, st>>>(gt, q, gt_k, topn, n,
                                                                          claim);
  return cudaGetLastError();
}

cudaError_t launch_sup_prune(const SupArgs& a, int num_sms, cudaStream_t st) {
  k_sup_prune<<<roar_grid(a.q, num_sms), kRoarWarps * 32, 0, st>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_sup_merge(const SupArgs& a, int num_sms, cudaStream_t st) {
  k_sup_merge<<<roar_grid(a.n, num_sms), kRoarWarps * 32, 0, st>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_fusion_nn(const FusionArgs& a, int num_sms, cudaStream_t st) {
  k_fusion_nn<<<roar_grid(a.n, num_sms), kRoarWarps * 32, 0, st>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_fusion_final(const FusionArgs& a, int num_sms, cudaStream_t st) {
  k_fusion_final<<<roar_grid(a.n, num_sms), kRoarWarps * 32, 0, st>>>(a);
  return cudaGetLastError();
}

}  // namespace pg
