// pg_graph.cu -- projection (K0), prune + reverse edges (K1/K2), reverse lists, merge (K3).
//
// Layout in HBM (all row-major, 64-bit row offsets):
//   base      n x d f32               the vectors (read-only)
//   winner    n u32                   projection winner key per base (K0)
//   pruned    n x P u32 + n counts    RNG-pruned out-lists (K2)
//   indeg     n u32 -> offs n+1       reverse-edge counts -> CSR offsets
//   edges     sum(pruned counts) u32  reverse sources grouped by destination (CSR)
//   reverse   n x R u32 + n counts    first R sources per destination, ascending (K2's add_reverse)
//   graph     n x degree u32          merged + pruned out-lists, tomb padded (K3)
// One warp owns one node in K2, the reverse-list finish and K3; lanes split candidates for the
// distance pass and kept entries for the occlusion tests.  Every distance is one FMA chain in
// d order (dist_seq), the reference's distance_between, so ids are bit-identical to it.
#include "pg_device.cuh"
#include "pg_kernels.h"

namespace pg {

// ------------------------------------------------------------------ K0: projection winners
// Winner key of query q for its top-1 base: queries whose gt[q][1] is a real id compete by
// lowest id; a query whose gt[q][1] is tomb leaves the CAS slot of match_top1_kernel_v0
// (Gbuilder.cuh:122) at tomb, so a later query overwrites its row: among those the highest id
// is the last writer.  Real-id queries always win over tomb ones.
__device__ __forceinline__ uint32_t winner_key(uint32_t q, bool real_first) {
  return real_first ? q : 0x80000000u + (0x7FFFFFFEu - q);
}
__device__ __forceinline__ uint32_t winner_query(uint32_t key) {
  if (key == kTomb) return kTomb;
  return key < 0x80000000u ? key : 0x7FFFFFFEu - (key - 0x80000000u);
}

__global__ void k_match_winner(const uint32_t* __restrict__ gt, uint64_t q, uint32_t gt_k,
                               uint64_t n, uint32_t* __restrict__ winner, uint32_t* status,
                               const uint64_t* __restrict__ seg_off,
                               const uint64_t* __restrict__ qseg_off, uint32_t seg_count) {
  const uint64_t stride = static_cast<uint64_t>(gridDim.x) * blockDim.x;
  for (uint64_t qi = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x; qi < q;
       qi += stride) {
    uint64_t off = 0, ns = n;  // the query's sub-index: its ground-truth ids are local to it
    if (seg_count) {
      const uint32_t sg = segment_of(qseg_off, seg_count, qi);
      off = seg_off[sg];
      ns = seg_off[sg + 1] - off;
    }
    const uint32_t bl = gt[qi * gt_k];
    if (bl == kTomb) continue;
    if (bl >= ns) {
      raise_error(status, kErrBadId);
      continue;
    }
    const uint64_t b = bl + off;
    const bool real = gt[qi * gt_k + 1] != kTomb;
    atomicMin(winner + b, winner_key(static_cast<uint32_t>(qi), real));
  }
}

// Materialises the n x gt_k projection rows of match_top1_kernel_v0 (stage API only; the build
// reads gt through `winner` directly): row b = gt[w][1..gt_k-2] followed by two tombs.
__global__ void k_match_rows(const uint32_t* __restrict__ gt, uint32_t gt_k, uint64_t n,
                             const uint32_t* __restrict__ winner, uint32_t* __restrict__ out) {
  const uint64_t total = n * gt_k;
  const uint64_t stride = static_cast<uint64_t>(gridDim.x) * blockDim.x;
  for (uint64_t i = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x; i < total;
       i += stride) {
    const uint64_t b = i / gt_k;
    const uint32_t j = static_cast<uint32_t>(i - b * gt_k);
    const uint32_t w = winner_query(winner[b]);
    out[i] = (w != kTomb && j + 2 < gt_k) ? gt[static_cast<uint64_t>(w) * gt_k + j + 1] : kTomb;
  }
}

__global__ void k_validate_ids(const uint32_t* __restrict__ ids, uint64_t count, uint64_t n,
                               uint32_t* status) {
  const uint64_t stride = static_cast<uint64_t>(gridDim.x) * blockDim.x;
  bool bad = false;
  for (uint64_t i = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x; i < count;
       i += stride) {
    const uint32_t v = ids[i];
    bad |= (v != kTomb && v >= n);
  }
  if (__any_sync(kFull, bad) && lane_id() == 0) raise_error(status, kErrBadId);
}

// ------------------------------------------------------------------ distances, E per lane
// E independent FMA chains (one per candidate slot of this lane), interleaved for ILP.  Slots
// with valid[s] == false are skipped and return FLT_MAX.
template <int E, bool WIDE>
__device__ __forceinline__ void dist_seq_multi(const float* __restrict__ brow,
                                               const float* __restrict__ base, uint32_t d,
                                               const uint32_t (&id)[E], const bool (&valid)[E],
                                               float (&out)[E]) {
  float s[E];
  const float4* rows[E];
#pragma unroll
  for (int e = 0; e < E; e++) {
    s[e] = 0.0f;
    rows[e] = reinterpret_cast<const float4*>(valid[e] ? base + static_cast<uint64_t>(id[e]) * d
                                                       : brow);
  }
  const float4* b4 = reinterpret_cast<const float4*>(brow);
  const uint32_t n4 = d >> 2;
  if (WIDE && (d & 7u) == 0 &&
      ((reinterpret_cast<uintptr_t>(base) | reinterpret_cast<uintptr_t>(brow)) & 31u) == 0) {
    // 32-byte aligned rows: 256-bit loads, one sector each (half the requests of float4)
#pragma unroll 2
    for (uint32_t i = 0; i < (d >> 3); i++) {
      float u[8];
      ld8(brow + 8 * i, u);
#pragma unroll
      for (int e = 0; e < E; e++) {
        float v[8];
        ld8(reinterpret_cast<const float*>(rows[e]) + 8 * i, v);
#pragma unroll
        for (int t = 0; t < 8; t++) s[e] = fmaf(u[t], v[t], s[e]);
      }
    }
#pragma unroll
    for (int e = 0; e < E; e++) out[e] = valid[e] ? -s[e] : FLT_MAX;
    return;
  }
  // four steps per pass keep (1 + E) * 4 row loads in flight: the rows come from L2, and the
  // chain's order leaves no other parallelism
#pragma unroll 4
  for (uint32_t i = 0; i < n4; i++) {
    const float4 u = __ldg(b4 + i);
#pragma unroll
    for (int e = 0; e < E; e++) {
      const float4 v = __ldg(rows[e] + i);
      s[e] = fmaf(u.x, v.x, s[e]);
      s[e] = fmaf(u.y, v.y, s[e]);
      s[e] = fmaf(u.z, v.z, s[e]);
      s[e] = fmaf(u.w, v.w, s[e]);
    }
  }
#pragma unroll
  for (int e = 0; e < E; e++) out[e] = valid[e] ? -s[e] : FLT_MAX;
}

// The occlusion scan of fusion_prune_reverse_kernel_v0 (Gbuilder.cuh:1150-1199) and
// fusion_merge_sort_prune_kernel over the sorted candidates ids_s/dist_s[j0 .. c): in order, a
// candidate is kept when no kept entry lies closer to it than the node does (exact FP32 chain),
// until `limit` are kept.  Many candidates are tested at once: the lanes take (candidate, kept
// entry) pairs of a window of consecutive undecided candidates, each candidate against the kept
// entries it has not been tested against yet.  Candidates are decided from the front of the
// window -- occluded ones dropped, the first unoccluded one kept, which sends the later ones back
// for one more test against it.  Kept entries and the evaluation count (the reference's count of
// tests: up to and including the first occluder, in kept order) equal the one-candidate-at-a-time
// scan (Gbuilder.cuh:1163-1181).  kept_s[0 .. K)
// on entry; returns where that scan stops: the candidate that filled the list, the first tomb
// (stop_at_tomb), or c.  Ids >= n count as occluded without a test.  win: 96 words per warp.
constexpr uint32_t kWinNone = 0xFFFFFFFFu, kWinInvalid = 0xFFFFFFFEu;

template <bool WIDE>
__device__ uint32_t scan_kept(const float* __restrict__ base, uint64_t n, uint32_t d,
                              const uint32_t* ids_s, const float* dist_s, uint32_t j0, uint32_t c,
                              uint32_t* kept_s, uint32_t& K, uint32_t limit, bool stop_at_tomb,
                              uint32_t* win, uint64_t* checks) {
  const uint32_t lane = lane_id();
  uint32_t* wj = win;        // candidate position
  uint32_t* wt = win + 32;   // kept entries tested so far without an occluder
  uint32_t* wo = win + 64;   // first occluder, kWinNone, or kWinInvalid
  uint32_t next = j0, wn = 0;
  for (;;) {
    while (wn < 32 && next < c) {
      const uint32_t x = ids_s[next];
      if (stop_at_tomb && (x == kTomb || x == kMaskedTomb)) break;
      if (lane == 0) {
        wj[wn] = next;
        wt[wn] = 0;
        wo[wn] = x >= n ? kWinInvalid : kWinNone;
      }
      wn++;
      next++;
    }
    __syncwarp();
    if (wn == 0) return next;
    // lanes -> (candidate, kept entry) pairs, front of the window first
    uint32_t my_w = kWinNone, my_t = 0, acc = 0;
    for (uint32_t w = 0; w < wn && acc < 32; w++) {
      if (wo[w] != kWinNone) continue;
      const uint32_t need = K - wt[w];
      if (lane >= acc && lane < acc + need) {
        my_w = w;
        my_t = wt[w] + (lane - acc);
      }
      acc += need;
    }
    bool o = false;
    if (my_w != kWinNone) {
      const uint32_t pos = wj[my_w];
      o = dist_seq<WIDE>(base + static_cast<uint64_t>(ids_s[pos]) * d,
                   base + static_cast<uint64_t>(kept_s[my_t]) * d, d) < dist_s[pos];
    }
    const unsigned mask = __ballot_sync(kFull, o);
    acc = 0;
    for (uint32_t w = 0; w < wn && acc < 32; w++) {
      if (wo[w] != kWinNone) continue;
      const uint32_t take = min(K - wt[w], 32u - acc);
      const unsigned range = (take >= 32 ? kFull : ((1u << take) - 1u)) << acc;
      const unsigned m = mask & range;
      if (lane == 0) {
        if (m)
          wo[w] = wt[w] + (static_cast<uint32_t>(__ffs(static_cast<int>(m)) - 1) - acc);
        else
          wt[w] += take;
      }
      acc += take;
    }
    __syncwarp();
    uint32_t dec = 0;
    for (uint32_t w = 0; w < wn; w++) {
      const uint32_t oc = wo[w];
      if (oc == kWinInvalid) {
        dec++;
        continue;
      }
      if (oc != kWinNone) {
        *checks += oc + 1;
        dec++;
        continue;
      }
      if (wt[w] != K) break;  // undecided: later candidates wait for it
      *checks += K;
      if (lane == 0) kept_s[K] = ids_s[wj[w]];
      K++;
      dec++;
      if (K == limit) {
        __syncwarp();
        return wj[w];
      }
    }
    __syncwarp();
    if (dec) {  // drop the decided front of the window
      uint32_t a = 0, b = 0, e = 0;
      if (lane + dec < wn) {
        a = wj[lane + dec];
        b = wt[lane + dec];
        e = wo[lane + dec];
      }
      __syncwarp();
      if (lane + dec < wn) {
        wj[lane] = a;
        wt[lane] = b;
        wo[lane] = e;
      }
      wn -= dec;
      __syncwarp();
    }
  }
}

__device__ __forceinline__ float key_dist(uint64_t key) {
  const uint32_t o = static_cast<uint32_t>(key >> 32);
  const uint32_t u = (o & 0x80000000u) ? (o & 0x7FFFFFFFu) : ~o;
  return __uint_as_float(u);
}

// ------------------------------------------------------------------ K2: prune + reverse
// fusion_prune_reverse_kernel_v0 (Gbuilder.cuh:1093-1244).  PHASE1 reads the candidate row of
// node b straight from the winner's ground truth (the K0 row) instead of a materialised graph.
template <int E, bool PHASE1, bool WIDE>
__global__ void __launch_bounds__(256) k_prune_reverse(PruneArgs a) {
  constexpr int C_MAX = 32 * E;
  extern __shared__ uint32_t smem_u32[];
  const uint32_t lane = lane_id();
  const uint32_t warp = threadIdx.x >> 5;
  uint32_t* ids_s = smem_u32 + warp * (3 * C_MAX + 96);
  float* dist_s = reinterpret_cast<float*>(ids_s + C_MAX);
  uint32_t* kept_s = ids_s + 2 * C_MAX;
  uint32_t* win_s = ids_s + 3 * C_MAX;
  const uint64_t nwarps = static_cast<uint64_t>(gridDim.x) * (blockDim.x >> 5);
  uint64_t ev = 0;
  for (uint64_t b = blockIdx.x * static_cast<uint64_t>(blockDim.x >> 5) + warp; b < a.n;
       b += nwarps) {
    uint32_t id[E];
    bool valid[E];
    uint32_t w = kTomb;
    uint64_t goff = 0, gn = a.n;  // phase 1: ground-truth ids are local to b's sub-index
    if (PHASE1) {
      w = winner_query(a.winner[b]);
      if (a.seg_count) {
        const uint32_t sg = segment_of(a.seg_off, a.seg_count, b);
        goff = a.seg_off[sg];
        gn = a.seg_off[sg + 1] - goff;
      }
    }
    if (PHASE1 && w == kTomb) {  // nobody's top-1: an all-tomb row, nothing kept
      if (lane == 0) a.pruned_num[b] = 0;
      if (a.sorted)
        for (uint32_t j = lane; j < a.c; j += 32) a.sorted[b * a.c + j] = kTomb;
      continue;
    }
#pragma unroll
    for (int s = 0; s < E; s++) {
      const uint32_t j = static_cast<uint32_t>(s) * 32u + lane;
      uint32_t x = kTomb;
      if (j < a.c) {
        if (PHASE1) {
          x = (j + 2 < a.gt_k) ? a.gt[static_cast<uint64_t>(w) * a.gt_k + j + 1] : kTomb;
          if (x != kTomb) {
            if (x >= gn) {  // out-of-range input id
              raise_error(a.status, kErrBadId);
              x = kTomb;
            } else {
              x = static_cast<uint32_t>(x + goff);
            }
          }
        } else {
          x = a.graph[b * a.c + j];
        }
      }
      if (x >= a.n && x != kTomb && x != kMaskedTomb) {  // out-of-range input id
        raise_error(a.status, kErrBadId);
        x = kTomb;
      }
      id[s] = x;
      valid[s] = (x != kTomb && x != static_cast<uint32_t>(b) && x != kMaskedTomb);
    }
    float dist[E];
    dist_seq_multi<E, WIDE>(a.base + b * a.d, a.base, a.d, id, valid, dist);
    uint64_t key[E];
#pragma unroll
    for (int s = 0; s < E; s++) {
      const uint32_t j = static_cast<uint32_t>(s) * 32u + lane;
      ev += __popc(__ballot_sync(kFull, valid[s])) * (lane == 0);
      key[s] = (j < a.c) ? pack_key(dist[s], j) : ~0ull;
    }
    warp_sort_kv<E>(key, id);
#pragma unroll
    for (int s = 0; s < E; s++) {
      const uint32_t i = static_cast<uint32_t>(s) * 32u + lane;
      if (i < a.c) {
        ids_s[i] = id[s];
        dist_s[i] = key_dist(key[s]);
        if (a.sorted) a.sorted[b * a.c + i] = id[s];
      }
    }
    __syncwarp();
    const uint32_t first = ids_s[0];
    if (first == kTomb || first == kMaskedTomb) {
      if (lane == 0) a.pruned_num[b] = 0;
      __syncwarp();
      continue;
    }
    if (lane == 0) kept_s[0] = first;
    __syncwarp();
    uint64_t checks = 0;
    uint32_t kc = 1;
    uint32_t j = a.p > 1 ? scan_kept<WIDE>(a.base, a.n, a.d, ids_s, dist_s, 1, a.c, kept_s, kc, a.p, true,
                                     win_s, &checks)
                         : 1;
    uint32_t k = kc - 1;
    if (!a.strict && k < a.p - 1) {  // non-strict fill (Gbuilder.cuh:1201-1239)
      for (uint32_t j2 = j; j2 < a.c && k < a.p - 1; j2++) {
        const uint32_t x = ids_s[j2];
        if (x == kTomb || x == static_cast<uint32_t>(b) || x == kMaskedTomb) continue;
        bool dup = false;
        for (uint32_t t0 = 0; t0 <= k; t0 += 32) {
          const uint32_t t = t0 + lane;
          dup |= __any_sync(kFull, t <= k && kept_s[t] == x);
        }
        if (!dup) {
          k++;
          if (lane == 0) kept_s[k] = x;
          __syncwarp();
        }
      }
    }
    ev += (lane == 0) ? checks : 0;
    const uint32_t cnt = k + 1;
    if (lane == 0) a.pruned_num[b] = cnt;
    for (uint32_t t = lane; t < cnt; t += 32) {
      const uint32_t dst = kept_s[t];
      a.pruned[b * a.p + t] = dst;
      atomicAdd(a.indeg + dst, 1u);
    }
    __syncwarp();
  }
  if (lane == 0 && ev) atomicAdd(a.evals, static_cast<unsigned long long>(ev));
}

// ------------------------------------------------------------------ reverse edges (CSR)
// Exclusive scan of n counts into offs[0..n] (offs[n] = total).  Three passes: per-block sums,
// one block scanning the block sums, per-block scan plus offset.
constexpr int kScanThreads = 1024;
constexpr int kScanItems = 4;
constexpr int kScanTile = kScanThreads * kScanItems;
// callers size the tile-sum buffers by kScanTileElems (pg_kernels.h)
static_assert(kScanTile == kScanTileElems, "scan tile size must match kScanTileElems");

__device__ __forceinline__ uint32_t block_exclusive_scan(uint32_t v, uint32_t* warp_sums,
                                                         uint32_t* total) {
  const uint32_t lane = lane_id(), warp = threadIdx.x >> 5;
  uint32_t x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t y = __shfl_up_sync(kFull, x, o);
    if (lane >= static_cast<uint32_t>(o)) x += y;
  }
  if (lane == 31) warp_sums[warp] = x;
  __syncthreads();
  if (warp == 0) {
    uint32_t w = (lane < (blockDim.x >> 5)) ? warp_sums[lane] : 0;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t y = __shfl_up_sync(kFull, w, o);
      if (lane >= static_cast<uint32_t>(o)) w += y;
    }
    warp_sums[lane] = w;
  }
  __syncthreads();
  const uint32_t before = (warp ? warp_sums[warp - 1] : 0) + x - v;
  if (total) *total = warp_sums[(blockDim.x >> 5) - 1];
  __syncthreads();
  return before;
}

__global__ void __launch_bounds__(kScanThreads) k_scan_tiles(const uint32_t* __restrict__ in,
                                                             uint64_t n,
                                                             uint32_t* __restrict__ tile_sums) {
  __shared__ uint32_t ws[32];
  const uint64_t base = static_cast<uint64_t>(blockIdx.x) * kScanTile + threadIdx.x * kScanItems;
  uint32_t s = 0;
#pragma unroll
  for (int i = 0; i < kScanItems; i++) s += (base + i < n) ? in[base + i] : 0u;
  uint32_t total;
  block_exclusive_scan(s, ws, &total);
  if (threadIdx.x == 0) tile_sums[blockIdx.x] = total;
}

__global__ void __launch_bounds__(kScanThreads) k_scan_tile_sums(uint32_t* __restrict__ sums,
                                                                 uint32_t tiles,
                                                                 uint32_t* __restrict__ total_out) {
  __shared__ uint32_t ws[32];
  uint32_t carry = 0;
  for (uint32_t t0 = 0; t0 < tiles; t0 += kScanThreads) {
    const uint32_t i = t0 + threadIdx.x;
    const uint32_t v = (i < tiles) ? sums[i] : 0u;
    uint32_t total;
    const uint32_t ex = block_exclusive_scan(v, ws, &total);
    if (i < tiles) sums[i] = carry + ex;
    carry += total;
  }
  if (threadIdx.x == 0) *total_out = carry;
}

__global__ void __launch_bounds__(kScanThreads) k_scan_apply(const uint32_t* __restrict__ in,
                                                             uint64_t n,
                                                             const uint32_t* __restrict__ tile_off,
                                                             uint32_t* __restrict__ out) {
  __shared__ uint32_t ws[32];
  const uint64_t base = static_cast<uint64_t>(blockIdx.x) * kScanTile + threadIdx.x * kScanItems;
  uint32_t v[kScanItems];
  uint32_t s = 0;
#pragma unroll
  for (int i = 0; i < kScanItems; i++) {
    v[i] = (base + i < n) ? in[base + i] : 0u;
    s += v[i];
  }
  uint32_t run = tile_off[blockIdx.x] + block_exclusive_scan(s, ws, nullptr);
#pragma unroll
  for (int i = 0; i < kScanItems; i++) {
    if (base + i < n) out[base + i] = run;
    run += v[i];
  }
}

// Every kept edge b -> p becomes the entry b in p's CSR segment (order fixed later by sorting).
__global__ void k_scatter_reverse(const uint32_t* __restrict__ pruned,
                                  const uint32_t* __restrict__ pruned_num, uint32_t p_len,
                                  uint64_t rows, const uint32_t* __restrict__ offs,
                                  uint32_t* __restrict__ cursor, uint32_t* __restrict__ edges) {
  const uint64_t stride = static_cast<uint64_t>(gridDim.x) * blockDim.x;
  for (uint64_t b = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x; b < rows;
       b += stride) {
    const uint32_t cnt = pruned_num[b];
    for (uint32_t t = 0; t < cnt; t++) {
      const uint32_t dst = pruned[b * p_len + t];
      const uint32_t pos = atomicAdd(cursor + dst, 1u);
      edges[offs[dst] + pos] = static_cast<uint32_t>(b);
    }
  }
}

// Reverse list of node p: the R smallest sources of its segment in ascending order, which is
// what add_reverse (Gbuilder.cuh:1020-1038) stores when sources run in ascending order; the
// count is min(in-degree, R).  Segments longer than 128 keep a running 128-smallest set.
__global__ void __launch_bounds__(256) k_reverse_lists(const uint32_t* __restrict__ offs,
                                                       const uint32_t* __restrict__ edges,
                                                       uint64_t n, uint32_t r,
                                                       uint32_t* __restrict__ rev,
                                                       uint32_t* __restrict__ rev_num) {
  const uint32_t lane = lane_id();
  const uint64_t nwarps = static_cast<uint64_t>(gridDim.x) * (blockDim.x >> 5);
  for (uint64_t p = blockIdx.x * static_cast<uint64_t>(blockDim.x >> 5) + (threadIdx.x >> 5);
       p < n; p += nwarps) {
    const uint32_t o0 = offs[p];
    const uint32_t deg = offs[p + 1] - o0;
    const uint32_t cnt = min(deg, r);
    if (deg == 0) {
      if (lane == 0) rev_num[p] = 0;
      continue;
    }
    uint32_t best[4];
    for (uint32_t c0 = 0; c0 < deg; c0 += 128) {
      uint32_t chunk[4];
#pragma unroll
      for (int s = 0; s < 4; s++) {
        const uint32_t i = c0 + static_cast<uint32_t>(s) * 32u + lane;
        chunk[s] = (i < deg) ? edges[o0 + i] : 0xFFFFFFFFu;
      }
      warp_sort_u32<4>(chunk);
      if (c0 == 0) {
#pragma unroll
        for (int s = 0; s < 4; s++) best[s] = chunk[s];
      } else {
        // best (ascending) against chunk reversed: the element-wise minimum holds the 128
        // smallest as a bitonic sequence, which one merge pass sorts.
#pragma unroll
        for (int s = 0; s < 4; s++) {
          const uint32_t rv = __shfl_sync(kFull, chunk[3 - s], 31 - lane);
          best[s] = min(best[s], rv);
        }
        warp_bitonic_merge_u32<4>(best);
      }
    }
#pragma unroll
    for (int s = 0; s < 4; s++) {
      const uint32_t i = static_cast<uint32_t>(s) * 32u + lane;
      if (i < cnt) rev[p * r + i] = best[s];
    }
    if (lane == 0) rev_num[p] = cnt;
  }
}

// One node's merged list (reverse entries, then pruned entries) with exact distances to the node,
// sorted by (distance, position) into ids_s / dist_s[0 .. nn); E = slots per lane (nn <= 32 E).
template <int E, bool WIDE>
__device__ __forceinline__ void merge_gather_sort(const MergeArgs& a, uint64_t b, uint32_t rn,
                                                  uint32_t nn, uint32_t* ids_s, float* dist_s) {
  const uint32_t lane = lane_id();
  uint32_t id[E];
  bool valid[E];
#pragma unroll
  for (int s = 0; s < E; s++) {
    const uint32_t j = static_cast<uint32_t>(s) * 32u + lane;
    uint32_t x = kTomb;
    if (j < rn)
      x = a.reverse[b * a.r + j];
    else if (j < nn)
      x = a.pruned[b * a.p + (j - rn)];
    if (j < nn && x >= a.n) {  // out-of-range input id
      raise_error(a.status, kErrBadId);
      x = kTomb;
    }
    id[s] = x;
    valid[s] = j < nn && x != kTomb;
  }
  float dist[E];
  dist_seq_multi<E, WIDE>(a.base + b * a.d, a.base, a.d, id, valid, dist);
  uint64_t key[E];
#pragma unroll
  for (int s = 0; s < E; s++) {
    const uint32_t j = static_cast<uint32_t>(s) * 32u + lane;
    key[s] = (j < nn) ? pack_key(dist[s], j) : ~0ull;
  }
  warp_sort_kv<E>(key, id);
#pragma unroll
  for (int s = 0; s < E; s++) {
    const uint32_t i = static_cast<uint32_t>(s) * 32u + lane;
    if (i < nn) {
      ids_s[i] = id[s];
      dist_s[i] = key_dist(key[s]);
    }
  }
}

// ------------------------------------------------------------------ K3: merge + prune
// fusion_merge_sort_prune_kernel (Gbuilder.cuh:1467-1601): merged list = reverse entries then
// pruned entries (pr_sort_list view); sort by distance keeping that order on ties; RNG prune
// into the out row; non-strict fill with first-occurrence marking; tomb padding.
template <int E, bool WIDE>
__global__ void __launch_bounds__(256) k_merge_prune(MergeArgs a) {
  constexpr int C_MAX = 32 * E;
  extern __shared__ uint32_t smem_u32[];
  const uint32_t lane = lane_id();
  const uint32_t warp = threadIdx.x >> 5;
  uint32_t* ids_s = smem_u32 + warp * (3 * C_MAX + C_MAX / 4 + 96);
  float* dist_s = reinterpret_cast<float*>(ids_s + C_MAX);
  uint32_t* out_s = ids_s + 2 * C_MAX;
  uint8_t* added_s = reinterpret_cast<uint8_t*>(ids_s + 3 * C_MAX);
  uint32_t* win_s = ids_s + 3 * C_MAX + C_MAX / 4;
  const uint64_t nwarps = static_cast<uint64_t>(gridDim.x) * (blockDim.x >> 5);
  uint64_t ev = 0;
  for (uint64_t b = blockIdx.x * static_cast<uint64_t>(blockDim.x >> 5) + warp; b < a.n;
       b += nwarps) {
    const uint32_t rn = min(a.reverse_num[b], a.r);
    const uint32_t pn = min(a.pruned_num[b], a.p);
    const uint32_t nn = rn + pn;
    uint32_t* orow = a.out + b * a.degree;
    if (nn == 0) {
      for (uint32_t t = lane; t < a.degree; t += 32) orow[t] = kTomb;
      continue;
    }
    if (lane == 0) ev += nn;
    // the merged lists are mostly short: size the distance slots and the sort to this one
    if (nn <= 32)
      merge_gather_sort<1, WIDE>(a, b, rn, nn, ids_s, dist_s);
    else if (E >= 2 && nn <= 64)
      merge_gather_sort<(E >= 2 ? 2 : 1), WIDE>(a, b, rn, nn, ids_s, dist_s);
    else
      merge_gather_sort<E, WIDE>(a, b, rn, nn, ids_s, dist_s);
    __syncwarp();
    if (lane == 0) out_s[0] = ids_s[0];
    __syncwarp();
    uint64_t checks = 0;
    uint32_t kc = 1;
    if (a.degree > 1)
      scan_kept<WIDE>(a.base, a.n, a.d, ids_s, dist_s, 1, nn, out_s, kc, a.degree, false, win_s,
                      &checks);
    uint32_t k = kc - 1;
    if (!a.strict && k < a.degree - 1) {
      for (uint32_t i = lane; i < nn; i += 32) added_s[i] = 0;
      __syncwarp();
      for (uint32_t i = 0; i <= k; i++) {  // first occurrence of each kept id
        const uint32_t x = out_s[i];
        for (uint32_t j0 = 0; j0 < nn; j0 += 32) {
          const uint32_t j = j0 + lane;
          const unsigned m = __ballot_sync(kFull, j < nn && ids_s[j] == x);
          if (m) {
            if (lane == 0) added_s[j0 + __ffs(static_cast<int>(m)) - 1] = 1;
            break;
          }
        }
        __syncwarp();
      }
      for (uint32_t i = 0; i < nn && k < a.degree - 1; i++) {
        if (added_s[i]) continue;
        const uint32_t x = ids_s[i];
        if (x != kTomb && x != static_cast<uint32_t>(b) && x < a.n) {
          k++;
          if (lane == 0) out_s[k] = x;
          __syncwarp();
        }
      }
    }
    ev += (lane == 0) ? checks : 0;
    for (uint32_t t = lane; t < a.degree; t += 32) orow[t] = (t <= k) ? out_s[t] : kTomb;
    __syncwarp();
  }
  if (lane == 0 && ev) atomicAdd(a.evals, static_cast<unsigned long long>(ev));
}

// ------------------------------------------------------------------ launchers
static int grid_for(uint64_t items, int per_block, int num_sms, int max_per_sm) {
  uint64_t blocks = (items + per_block - 1) / per_block;
  uint64_t cap = static_cast<uint64_t>(num_sms) * max_per_sm;
  if (blocks > cap) blocks = cap;
  if (blocks == 0) blocks = 1;
  return static_cast<int>(blocks);
}

cudaError_t launch_match_winner(const uint32_t* gt, uint64_t q, uint32_t gt_k, uint64_t n,
                                uint32_t* winner, uint32_t* status, int num_sms, cudaStream_t st,
                                const uint64_t* seg_off, const uint64_t* qseg_off,
                                uint32_t seg_count) {
  cudaError_t e = cudaMemsetAsync(winner, 0xFF, n * sizeof(uint32_t), st);
  if (e != cudaSuccess) return e;
  k_match_winner<<<grid_for(q, 256, num_sms, 8), 256, 0, st>>>(gt, q, gt_k, n, winner, status,
                                                               seg_off, qseg_off, seg_count);
  return cudaGetLastError();
}

__global__ void k_localize(uint32_t* __restrict__ rows, uint64_t n, uint32_t deg,
                           const uint64_t* __restrict__ seg_off, uint32_t seg_count) {
  const uint64_t stride = static_cast<uint64_t>(gridDim.x) * blockDim.x;
  for (uint64_t i = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x; i < n * deg;
       i += stride) {
    const uint32_t v = rows[i];
    if (v != kTomb) rows[i] = static_cast<uint32_t>(v - seg_off[segment_of(seg_off, seg_count, i / deg)]);
  }
}

cudaError_t launch_localize(uint32_t* rows, uint64_t n, uint32_t deg, const uint64_t* seg_off,
                            uint32_t seg_count, int num_sms, cudaStream_t st) {
  k_localize<<<grid_for(n * deg, 256, num_sms, 8), 256, 0, st>>>(rows, n, deg, seg_off, seg_count);
  return cudaGetLastError();
}

cudaError_t launch_match_rows(const uint32_t* gt, uint32_t gt_k, uint64_t n,
                              const uint32_t* winner, uint32_t* out, int num_sms,
                              cudaStream_t st) {
  k_match_rows<<<grid_for(n * gt_k, 256, num_sms, 8), 256, 0, st>>>(gt, gt_k, n, winner, out);
  return cudaGetLastError();
}

cudaError_t launch_validate_ids(const uint32_t* ids, uint64_t count, uint64_t n,
                                uint32_t* status, int num_sms, cudaStream_t st) {
  k_validate_ids<<<grid_for(count, 256, num_sms, 8), 256, 0, st>>>(ids, count, n, status);
  return cudaGetLastError();
}

// The 256-bit-load kernels for rows of kWideRowFloats or more on a 32-byte aligned base.
static bool wide_rows(const float* base, uint32_t d) {
  return d >= kWideRowFloats && (d % 8) == 0 && (reinterpret_cast<uintptr_t>(base) % 32) == 0;
}

template <int E, bool P1>
static cudaError_t launch_prune_e(const PruneArgs& a, int num_sms, cudaStream_t st) {
  const int threads = 256;
  const size_t smem = (threads / 32) * (3 * 32 * E + 96) * sizeof(uint32_t);
  const unsigned grid = grid_for(a.n, threads / 32, num_sms, 8);
  if (wide_rows(a.base, a.d))
    k_prune_reverse<E, P1, true><<<grid, threads, smem, st>>>(a);
  else
    k_prune_reverse<E, P1, false><<<grid, threads, smem, st>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_prune_reverse(const PruneArgs& a, bool phase1, int num_sms, cudaStream_t st) {
  if (a.c <= 32) return phase1 ? launch_prune_e<1, true>(a, num_sms, st)
                               : launch_prune_e<1, false>(a, num_sms, st);
  if (a.c <= 64) return phase1 ? launch_prune_e<2, true>(a, num_sms, st)
                               : launch_prune_e<2, false>(a, num_sms, st);
  return phase1 ? launch_prune_e<4, true>(a, num_sms, st)
                : launch_prune_e<4, false>(a, num_sms, st);
}

cudaError_t launch_reverse_csr(const uint32_t* pruned, const uint32_t* pruned_num, uint32_t p_len,
                               uint64_t n, const uint32_t* indeg, uint32_t* offs,
                               uint32_t* tile_sums, uint32_t* cursor, uint32_t* edges,
                               int num_sms, cudaStream_t st, uint64_t rows) {
  if (rows == 0) rows = n;
  const uint32_t tiles = static_cast<uint32_t>((n + kScanTile - 1) / kScanTile);
  k_scan_tiles<<<tiles, kScanThreads, 0, st>>>(indeg, n, tile_sums);
  k_scan_tile_sums<<<1, kScanThreads, 0, st>>>(tile_sums, tiles, offs + n);
  k_scan_apply<<<tiles, kScanThreads, 0, st>>>(indeg, n, tile_sums, offs);
  cudaError_t e = cudaMemsetAsync(cursor, 0, n * sizeof(uint32_t), st);
  if (e != cudaSuccess) return e;
  k_scatter_reverse<<<grid_for(rows, 256, num_sms, 8), 256, 0, st>>>(pruned, pruned_num, p_len,
                                                                      rows, offs, cursor, edges);
  return cudaGetLastError();
}

cudaError_t launch_reverse_lists(const uint32_t* offs, const uint32_t* edges, uint64_t n,
                                 uint32_t r, uint32_t* rev, uint32_t* rev_num, int num_sms,
                                 cudaStream_t st) {
  k_reverse_lists<<<grid_for(n, 8, num_sms, 8), 256, 0, st>>>(offs, edges, n, r, rev, rev_num);
  return cudaGetLastError();
}

template <int E>
static cudaError_t launch_merge_e(const MergeArgs& a, int num_sms, cudaStream_t st) {
  const int threads = 256;
  const size_t smem = (threads / 32) * (3 * 32 * E + 8 * E + 96) * sizeof(uint32_t);
  const unsigned grid = grid_for(a.n, threads / 32, num_sms, 8);
  if (wide_rows(a.base, a.d))
    k_merge_prune<E, true><<<grid, threads, smem, st>>>(a);
  else
    k_merge_prune<E, false><<<grid, threads, smem, st>>>(a);
  return cudaGetLastError();
}

// 16-byte words from src to dst by the SMs (host memory mapped into the device address space
// on one side): each thread moves four words per pass, so that every SM keeps many requests in
// flight over the CPU-GPU link.
__global__ void __launch_bounds__(256) k_copy16(uint4* __restrict__ dst,
                                                const uint4* __restrict__ src, uint64_t words) {
  const uint64_t stride = static_cast<uint64_t>(gridDim.x) * blockDim.x;
  uint64_t i = static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  for (; i + 3 * stride < words; i += 4 * stride) {
    const uint4 v0 = src[i], v1 = src[i + stride], v2 = src[i + 2 * stride],
                v3 = src[i + 3 * stride];
    dst[i] = v0;
    dst[i + stride] = v1;
    dst[i + 2 * stride] = v2;
    dst[i + 3 * stride] = v3;
  }
  for (; i < words; i += stride) dst[i] = src[i];
}

cudaError_t launch_copy16(void* dst, const void* src, uint64_t bytes, int num_sms,
                          cudaStream_t st) {
  if (bytes == 0) return cudaSuccess;
  if ((bytes % 16) != 0 || (reinterpret_cast<uintptr_t>(dst) % 16) != 0 ||
      (reinterpret_cast<uintptr_t>(src) % 16) != 0)
    return cudaErrorInvalidValue;
  k_copy16<<<static_cast<unsigned>(num_sms) * 4, 256, 0, st>>>(
      static_cast<uint4*>(dst), static_cast<const uint4*>(src), bytes / 16);
  return cudaGetLastError();
}

cudaError_t launch_merge_prune(const MergeArgs& a, int num_sms, cudaStream_t st) {
  const uint32_t cmax = a.r + a.p;
  if (cmax <= 32) return launch_merge_e<1>(a, num_sms, st);
  if (cmax <= 64) return launch_merge_e<2>(a, num_sms, st);
  return launch_merge_e<4>(a, num_sms, st);
}

}  // namespace pg
