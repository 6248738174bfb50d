// pg_search.cu -- beam search with every base point as the query (K4/K8).
//
// Semantics of link_process_v0_store_base_data (Gsearcher.cuh:890-1066): list of L = Km + Kp*Kd
// (distance, id); seeds (seed_base + i) % n in slots Km.., Km slots at FLT_MAX; sort; visited set
// = the top Km; loop { pick the first Kp unexplored of the top Km (collect_top_p_normal,
// Gsearcher.cuh:75-106) and mark them; read their first Kd graph neighbours; score each new id
// (visited or repeated ids get FLT_MAX); sort; every reset_iter iterations rebuild the visited set
// from the top Km }.  Output: all L ids with the parent bit cleared.
//
// GB300 design, one warp per query, persistent warps pulling queries from a work counter:
//   * the list lives in registers (32*E slots, element i = lane i%32, slot i/32) and is sorted with
//     a warp bitonic network on (distance, position) keys = the stable order of the reference;
//   * the visited set is an exact open-addressing table in shared memory (Ghashtable semantics);
//   * the candidate rows of one iteration are staged into shared memory with one cp.async.bulk
//     per new candidate (16-byte aligned 4*D-byte rows) completing on an mbarrier;
//   * distances keep the reference's FP32 order exactly: residue r = i mod 32 accumulates
//     q[i]*x[i] in i order, then the shuffle-down tree 16,8,4,2,1.  Eight lanes cover one row
//     (lane m owns residues 4m..4m+3 via 128-bit shared loads), four rows per pass, and a
//     transposed butterfly (xor 4, 2, 1 + two in-register adds) forms exactly that tree.
#include "pg_device.cuh"
#include "pg_kernels.h"

namespace pg {

namespace {

__device__ __forceinline__ uint32_t smem_addr(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count)
               : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile(
      "{\n\t.reg .b64 st;\n\t"
      "mbarrier.arrive.expect_tx.shared::cta.b64 st, [%0], %1;\n\t}" ::"r"(smem_addr(bar)),
      "r"(bytes)
      : "memory");
}

// try_wait with a suspend-time hint: a waiting warp sleeps until the phase completes (or the
// hint, in ns, runs out) instead of spinning on the issue slots the other warps need.
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  constexpr uint32_t kSuspendNs = 100000;
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_addr(bar)), "r"(parity), "r"(kSuspendNs)
      : "memory");
  return ok != 0;
}

__device__ __forceinline__ uint64_t global_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %globaltimer;" : "=l"(t));
  return t;
}

// Bounded wait: false if the phase did not complete within one second of wall time.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity) {
  if (mbar_try_wait(bar, parity)) return true;
  const uint64_t t0 = global_ns();
  while (!mbar_try_wait(bar, parity))
    if (global_ns() - t0 > 1000000000ull) return false;
  return true;
}

__device__ __forceinline__ void bulk_row_to_smem(float* dst, const float* src, uint32_t bytes,
                                                 uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::
          "r"(smem_addr(dst)),
      "l"(src), "r"(bytes), "r"(smem_addr(bar))
      : "memory");
}

__device__ __forceinline__ void fence_proxy_async() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ uint32_t hslot(uint32_t key, uint32_t mask) {
  uint32_t h = key * 0x9E3779B1u;
  h ^= h >> 16;
  return h & mask;
}

__device__ __forceinline__ void hash_insert(uint32_t* t, uint32_t mask, uint32_t key) {
  uint32_t s = hslot(key, mask);
  for (uint32_t probe = 0; probe <= mask; probe++) {
    const uint32_t old = atomicCAS(t + s, 0u, key + 1);
    if (old == 0 || old == key + 1) return;
    s = (s + 1) & mask;
  }
}

// Inserts key unless present, in one probe sequence; true when it was absent
// (warp_level_test_and_set, Ghashtable.cuh:39-64).  The lanes of a warp insert distinct keys, so
// a concurrent claim of a slot by another lane only moves the probe on.
__device__ __forceinline__ bool hash_test_and_set(uint32_t* t, uint32_t mask, uint32_t key) {
  uint32_t s = hslot(key, mask);
  for (uint32_t probe = 0; probe <= mask; probe++) {
    const uint32_t old = atomicCAS(t + s, 0u, key + 1);
    if (old == 0) return true;
    if (old == key + 1) return false;
    s = (s + 1) & mask;
  }
  return false;  // cannot happen: the table has twice the slots of the ids it ever holds
}

__device__ __forceinline__ void hash_clear(uint32_t* t, uint32_t slots) {
  uint4* t4 = reinterpret_cast<uint4*>(t);
  for (uint32_t i = lane_id(); i < (slots >> 2); i += 32) t4[i] = make_uint4(0, 0, 0, 0);
}

template <int NS>
struct Q4 {
  float4 v[NS];
};

}  // namespace

// ---------------------------------------------------------------------------------------------
// The search kernels (k_search_m32 for Km = 32, k_search_mk for Km = 64, 96):
//   * candidate rows are staged ROWS at a time (ROWS*D*4 bytes of shared memory), so many warps
//     stay resident;
//   * the sorted top Km is kept in registers and the new candidates are merged into it by rank
//     (ballot/popc against unique (distance, position) keys) -- the same total order as sorting
//     the whole list, without a sorting network every iteration;
//   * the full L-entry list (top before the last merge + the last candidates) is sorted once,
//     when the query ends, for the output.
namespace {

// Scores the lanes whose `newc` is set, ROWS rows per pass.  Lane (g, m) = (lane / 8, lane % 8)
// accumulates residues 4m..4m+3 of candidate rows 4r + g (the reference's lane-strided FMA
// chains, one 16-byte shared load per 32 elements).  ROUNDS = ROWS/4 candidates per 8-lane group; the first log2(ROUNDS) butterfly levels
// are transposed (each lane keeps one candidate), the remaining ones are plain xor reductions.
template <int KSTEPS, int ROWS>
__device__ __forceinline__ float score_passes(const SearchArgs& a, const Q4<KSTEPS>& q,
                                              uint32_t node, bool newc, float* rows,
                                              uint64_t* mbar, uint32_t& phase, bool& ok) {
  constexpr int ROUNDS = ROWS / 4;
  static_assert(ROUNDS == 2 || ROUNDS == 4 || ROUNDS == 8, "ROWS must be 8, 16 or 32");
  const uint32_t lane = lane_id();
  const unsigned newmask = __ballot_sync(kFull, newc);
  const uint32_t nnew = __popc(newmask);
  const uint32_t d = a.d;
  const uint32_t ci = __popc(newmask & ((1u << lane) - 1u));
  const uint32_t g = lane >> 3, m = lane & 7u;
  const bool bA = (m & 4u) != 0, bB = (m & 2u) != 0, bC = (m & 1u) != 0;
  float result = FLT_MAX;
  for (uint32_t c0 = 0; c0 < nnew; c0 += ROWS) {
    const uint32_t cnt = min(static_cast<uint32_t>(ROWS), nnew - c0);
    const bool mine = newc && ci >= c0 && ci < c0 + ROWS;
    fence_proxy_async();
    if (lane == 0) mbar_arrive_expect_tx(mbar, cnt * d * 4u);
    __syncwarp();
    if (mine)
      bulk_row_to_smem(rows + static_cast<size_t>(ci - c0) * d,
                       a.base + static_cast<uint64_t>(node) * d, d * 4u, mbar);
    ok = mbar_wait_bounded(mbar, phase);
    phase ^= 1u;
    if (!ok) return FLT_MAX;
    float p[ROUNDS][4];
#pragma unroll
    for (int r = 0; r < ROUNDS; r++) {
#pragma unroll
      for (int i = 0; i < 4; i++) p[r][i] = 0.0f;
      const uint32_t c = 4u * r + g;
      if (c < cnt) {
        const float* row = rows + static_cast<size_t>(c) * d;
#pragma unroll
        for (int k = 0; k < KSTEPS; k++) {
          const uint32_t off = 32u * k + 4u * m;
          if (off < d) {
            const float4 x = *reinterpret_cast<const float4*>(row + off);
            p[r][0] = fmaf(q.v[k].x, x.x, p[r][0]);
            p[r][1] = fmaf(q.v[k].y, x.y, p[r][1]);
            p[r][2] = fmaf(q.v[k].z, x.z, p[r][2]);
            p[r][3] = fmaf(q.v[k].w, x.w, p[r][3]);
          }
        }
      }
    }
    // level xor 4 (residues +16): transposed, keeps ROUNDS/2 rounds
    float v4[ROUNDS / 2][4];
#pragma unroll
    for (int i = 0; i < ROUNDS / 2; i++)
#pragma unroll
      for (int j = 0; j < 4; j++) {
        const float send = bA ? p[i][j] : p[i + ROUNDS / 2][j];
        const float keep = bA ? p[i + ROUNDS / 2][j] : p[i][j];
        v4[i][j] = keep + __shfl_xor_sync(kFull, send, 4);
      }
    float v[4];
    uint32_t r_of_lane;
    if constexpr (ROUNDS == 2) {
#pragma unroll
      for (int j = 0; j < 4; j++) {
        float t = v4[0][j];
        t = t + __shfl_xor_sync(kFull, t, 2);  // residues +8
        t = t + __shfl_xor_sync(kFull, t, 1);  // residues +4
        v[j] = t;
      }
      r_of_lane = bA ? 1u : 0u;
    } else if constexpr (ROUNDS == 4) {
      float v2[4];
#pragma unroll
      for (int j = 0; j < 4; j++) {
        const float send = bB ? v4[0][j] : v4[1][j];
        const float keep = bB ? v4[1][j] : v4[0][j];
        v2[j] = keep + __shfl_xor_sync(kFull, send, 2);
      }
#pragma unroll
      for (int j = 0; j < 4; j++) v[j] = v2[j] + __shfl_xor_sync(kFull, v2[j], 1);
      r_of_lane = (bA ? 2u : 0u) + (bB ? 1u : 0u);
    } else {
      float v2[2][4];
#pragma unroll
      for (int i = 0; i < 2; i++)
#pragma unroll
        for (int j = 0; j < 4; j++) {
          const float send = bB ? v4[i][j] : v4[i + 2][j];
          const float keep = bB ? v4[i + 2][j] : v4[i][j];
          v2[i][j] = keep + __shfl_xor_sync(kFull, send, 2);
        }
#pragma unroll
      for (int j = 0; j < 4; j++) {
        const float send = bC ? v2[0][j] : v2[1][j];
        const float keep = bC ? v2[1][j] : v2[0][j];
        v[j] = keep + __shfl_xor_sync(kFull, send, 1);
      }
      r_of_lane = m;
    }
    (void)r_of_lane;
    const float total = (v[0] + v[2]) + (v[1] + v[3]);
    // candidate lc = 4r + g sits in lane 8g + m(r): m(r) spreads r over the transposed bits
    const uint32_t lc = mine ? ci - c0 : 0u;
    const uint32_t r = lc >> 2;
    uint32_t msrc;
    if constexpr (ROUNDS == 2)
      msrc = r << 2;
    else if constexpr (ROUNDS == 4)
      msrc = ((r >> 1) << 2) | ((r & 1u) << 1);
    else
      msrc = r;
    const float dd = __shfl_sync(kFull, total, ((lc & 3u) << 3) | msrc);
    if (mine) result = -dd;
  }
  return result;
}

}  // namespace

template <int KSTEPS, int ROWS>
__global__ void __launch_bounds__(32, KSTEPS <= 8 ? 20 : 12) k_search_m32(SearchArgs a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const uint32_t lane = lane_id();
  uint64_t* mbar = reinterpret_cast<uint64_t*>(smem_raw);
  uint64_t* mkey = reinterpret_cast<uint64_t*>(smem_raw + 16);   // 32 merge keys
  uint32_t* mid = reinterpret_cast<uint32_t*>(smem_raw + 16 + 256);  // 32 merge ids
  uint32_t* hash = reinterpret_cast<uint32_t*>(smem_raw + 16 + 256 + 128);
  float* rows = reinterpret_cast<float*>(smem_raw + 16 + 256 + 128 + 4u * a.hash_slots);
  const uint32_t hmask = a.hash_slots - 1u;
  const uint32_t kp = a.kp, kd = a.kd;
  if (lane == 0) mbar_init(mbar, 1);
  __syncwarp();
  uint32_t phase = 0;
  unsigned long long ev = 0, it_all = 0;
  bool ok = true;
  const uint32_t m = lane & 7u;
  const uint32_t e_of_lane = lane / kd, nb_of_lane = lane % kd;

  for (;;) {
    uint32_t qi = 0;
    if (lane == 0) qi = atomicAdd(a.work, 1u);
    qi = __shfl_sync(kFull, qi, 0);
    if (qi >= (a.queries ? a.nq : a.n)) break;
    const uint32_t qid = a.order ? a.order[qi] : qi;
    const float* qrow = (a.queries ? a.queries : a.base) + static_cast<uint64_t>(qid) * a.d;
    Q4<KSTEPS> q;
#pragma unroll
    for (int k = 0; k < KSTEPS; k++) {
      const uint32_t off = 32u * k + 4u * m;
      q.v[k] = (off < a.d) ? __ldg(reinterpret_cast<const float4*>(qrow + off))
                           : make_float4(0.f, 0.f, 0.f, 0.f);
    }
    // list before the last merge (top) and the last candidates (cand): the full 64-entry list
    // is their sorted union
    uint64_t top_key = pack_key(FLT_MAX, lane);
    uint32_t top_id = kTomb;
    uint64_t cand_key;
    uint32_t cand_id;
    {  // seeds: every slot is scored (Gsearcher.cuh:958-976 has no visited test)
      uint64_t soff = 0, sn = a.n;  // entry points are drawn inside the query's sub-index
      if (a.seg_count) {
        const uint32_t sg = segment_of(a.seg_off, a.seg_count, qid);
        soff = a.seg_off[sg];
        sn = a.seg_off[sg + 1] - soff;
      }
      const uint32_t node =
          static_cast<uint32_t>((a.seed_base + static_cast<uint64_t>(lane)) % sn + soff);
      float dist;
      if (a.seed_dist) {  // scored for every query at once by k_seed_dists
        dist = a.seed_dist[static_cast<uint64_t>(qid) * 32u + lane];
      } else {
        dist = score_passes<KSTEPS, ROWS>(a, q, node, true, rows, mbar, phase, ok);
        if (!ok) break;
      }
      cand_key = pack_key(dist, 32u + lane);
      cand_id = node;
      ev += (lane == 0) ? 32u : 0u;
    }
    // current sorted top 32 after merging the seeds
    uint64_t cur_key;
    uint32_t cur_id;
    {
      uint64_t k2[2] = {top_key, cand_key};
      uint32_t i2[2] = {top_id, cand_id};
      warp_sort_kv<2>(k2, i2);
      cur_key = k2[0];
      cur_id = i2[0];
    }
    hash_clear(hash, a.hash_slots);
    __syncwarp();
    hash_insert(hash, hmask, cur_id & kMaskedTomb);
    __syncwarp();

    uint32_t iter = 0, total = 0;
    for (;;) {
      // collect_top_p_normal: first kp unexplored of the top 32, marked explored
      const bool unexp = (cur_id & kParent) == 0;
      const unsigned umask = __ballot_sync(kFull, unexp);
      const uint32_t found = __popc(umask);
      if (found == 0) break;
      const uint32_t rank = __popc(umask & ((1u << lane) - 1u));
      uint32_t src = 0;
      const bool want = lane < kp && lane < found;
      if (want) {
        unsigned mm = umask;
        for (uint32_t i = 0; i < lane; i++) mm &= mm - 1u;
        src = static_cast<uint32_t>(__ffs(static_cast<int>(mm)) - 1);
      }
      const uint32_t got = __shfl_sync(kFull, cur_id, src);
      const uint32_t ex_lane = want ? got : kTomb;
      if (unexp && rank < kp) cur_id |= kParent;
      if (++total > a.max_iters) {
        if (lane == 0) raise_error(a.status, kErrIterCap);
        // the output is the list of the last completed merge
        break;
      }
      const uint32_t ex = __shfl_sync(kFull, ex_lane, e_of_lane);
      uint32_t node = kTomb;
      if (ex < a.n)
        node = a.graph[static_cast<uint64_t>(ex) * a.graph_degree + nb_of_lane];
      else if (ex != kTomb)
        raise_error(a.status, kErrCapacity);
      if (node >= a.n && node != kTomb) {
        raise_error(a.status, kErrBadId);
        node = kTomb;
      }
      const bool valid = node != kTomb;
      const unsigned same = __match_any_sync(kFull, node);
      const bool first = lane == static_cast<uint32_t>(__ffs(static_cast<int>(same)) - 1);
      const bool newc = valid && first && hash_test_and_set(hash, hmask, node);
      __syncwarp();
      const float dist = score_passes<KSTEPS, ROWS>(a, q, node, newc, rows, mbar, phase, ok);
      if (!ok) break;
      const unsigned scored = __ballot_sync(kFull, newc);
      ev += (lane == 0) ? __popc(scored) : 0u;
      // the list that this merge sorts: top (positions 0..31) + candidates (32..63)
      top_key = (cur_key & 0xFFFFFFFF00000000ull) | lane;
      top_id = cur_id;
      cand_key = pack_key(newc ? dist : FLT_MAX, 32u + lane);
      cand_id = node;
      // merge by rank: only scored candidates can enter the top (the others carry FLT_MAX and
      // positions after every retained entry), and of those only the ones below the current
      // 32nd key: a candidate above it displaces nothing and lands at rank >= 32, and every
      // candidate below an entering one enters too, so the ranks come out the same
      const uint64_t worst = __shfl_sync(kFull, top_key, 31);
      uint32_t shift = 0, cpos = 0xFFFFFFFFu;
      unsigned rem = __ballot_sync(kFull, newc && cand_key < worst);
      while (rem) {
        const uint32_t c = static_cast<uint32_t>(__ffs(static_cast<int>(rem)) - 1);
        rem &= rem - 1u;
        const uint64_t kc = __shfl_sync(kFull, cand_key, c);
        const uint32_t below_top = __popc(__ballot_sync(kFull, top_key < kc));
        const uint32_t below_cand = __popc(__ballot_sync(kFull, newc && cand_key < kc));
        if (lane == c) cpos = below_top + below_cand;
        shift += (top_key > kc) ? 1u : 0u;
      }
      const uint32_t tpos = lane + shift;
      if (tpos < 32) {
        mkey[tpos] = top_key;
        mid[tpos] = top_id;
      }
      if (cpos < 32) {
        mkey[cpos] = cand_key;
        mid[cpos] = cand_id;
      }
      __syncwarp();
      cur_key = mkey[lane];
      cur_id = mid[lane];
      __syncwarp();
      if (++iter == a.reset_iter) {
        hash_clear(hash, a.hash_slots);
        __syncwarp();
        hash_insert(hash, hmask, cur_id & kMaskedTomb);
        __syncwarp();
        iter = 0;
      }
    }
    if (!ok) break;
    it_all += (lane == 0) ? total : 0u;
    uint64_t k2[2] = {top_key, cand_key};
    uint32_t i2[2] = {top_id, cand_id};
    warp_sort_kv<2>(k2, i2);
    uint32_t* orow = a.out + static_cast<uint64_t>(qid) * a.out_width;
    if (lane < a.out_width) orow[lane] = i2[0] & kMaskedTomb;
    if (32 + lane < a.out_width) orow[32 + lane] = i2[1] & kMaskedTomb;
  }
  if (!ok) {
    if (lane == 0) raise_error(a.status, kErrWait);
    mbar_wait_bounded(mbar, phase ^ 1u);
  }
  if (lane == 0) {
    if (ev) atomicAdd(a.evals, ev);
    if (it_all) atomicAdd(a.iters, it_all);
  }
}

// k_search_m32 generalised to Km = 32 * KM_S (64, 96): the top-Km list in KM_S register slots
// (element i in lane i % 32, slot i / 32), the same candidate staging and FP32 order, the rank
// merge of the scored candidates over all slots, one bitonic sort of the final list.
template <int KM_S, int KSTEPS, int ROWS>
__global__ void __launch_bounds__(32, KSTEPS <= 8 ? 16 : 8) k_search_mk(SearchArgs a) {
  constexpr int EF = (KM_S + 1 <= 2) ? 2 : 4;  // final sort: KM_S + 1 slots, padded to 2^k
  constexpr uint32_t KM = 32u * KM_S;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const uint32_t lane = lane_id();
  uint64_t* mbar = reinterpret_cast<uint64_t*>(smem_raw);
  uint64_t* mkey = reinterpret_cast<uint64_t*>(smem_raw + 16);      // KM merge keys
  uint32_t* mid = reinterpret_cast<uint32_t*>(smem_raw + 16 + 8 * KM);  // KM merge ids
  uint32_t* hash = reinterpret_cast<uint32_t*>(smem_raw + 16 + 12 * KM);
  float* rows = reinterpret_cast<float*>(smem_raw + 16 + 12 * KM + 4u * a.hash_slots);
  const uint32_t hmask = a.hash_slots - 1u;
  const uint32_t kp = a.kp, kd = a.kd;
  if (lane == 0) mbar_init(mbar, 1);
  __syncwarp();
  uint32_t phase = 0;
  unsigned long long ev = 0, it_all = 0;
  bool ok = true;
  const uint32_t m = lane & 7u;
  const uint32_t e_of_lane = lane / kd, nb_of_lane = lane % kd;
  const unsigned lt_mask = (1u << lane) - 1u;

  for (;;) {
    uint32_t qi = 0;
    if (lane == 0) qi = atomicAdd(a.work, 1u);
    qi = __shfl_sync(kFull, qi, 0);
    if (qi >= (a.queries ? a.nq : a.n)) break;
    const uint32_t qid = a.order ? a.order[qi] : qi;
    const float* qrow = (a.queries ? a.queries : a.base) + static_cast<uint64_t>(qid) * a.d;
    Q4<KSTEPS> q;
#pragma unroll
    for (int k = 0; k < KSTEPS; k++) {
      const uint32_t off = 32u * k + 4u * m;
      q.v[k] = (off < a.d) ? __ldg(reinterpret_cast<const float4*>(qrow + off))
                           : make_float4(0.f, 0.f, 0.f, 0.f);
    }
    uint64_t top_key[KM_S];
    uint32_t top_id[KM_S];
#pragma unroll
    for (int s = 0; s < KM_S; s++) {
      top_key[s] = pack_key(FLT_MAX, static_cast<uint32_t>(s) * 32u + lane);
      top_id[s] = kTomb;
    }
    uint64_t cand_key;
    uint32_t cand_id;
    {  // seeds (Gsearcher.cuh:958-976 has no visited test)
      uint64_t soff = 0, sn = a.n;
      if (a.seg_count) {
        const uint32_t sg = segment_of(a.seg_off, a.seg_count, qid);
        soff = a.seg_off[sg];
        sn = a.seg_off[sg + 1] - soff;
      }
      const uint32_t node =
          static_cast<uint32_t>((a.seed_base + static_cast<uint64_t>(lane)) % sn + soff);
      float dist;
      if (a.seed_dist) {
        dist = a.seed_dist[static_cast<uint64_t>(qid) * 32u + lane];
      } else {
        dist = score_passes<KSTEPS, ROWS>(a, q, node, true, rows, mbar, phase, ok);
        if (!ok) break;
      }
      cand_key = pack_key(dist, KM + lane);
      cand_id = node;
      ev += (lane == 0) ? 32u : 0u;
    }
    uint64_t cur_key[KM_S];
    uint32_t cur_id[KM_S];
    {
      uint64_t k2[EF];
      uint32_t i2[EF];
#pragma unroll
      for (int s = 0; s < EF; s++) {
        k2[s] = s < KM_S ? top_key[s < KM_S ? s : 0] : (s == KM_S ? cand_key : ~0ull);
        i2[s] = s < KM_S ? top_id[s < KM_S ? s : 0] : (s == KM_S ? cand_id : kTomb);
      }
      warp_sort_kv<EF>(k2, i2);
#pragma unroll
      for (int s = 0; s < KM_S; s++) {
        cur_key[s] = k2[s];
        cur_id[s] = i2[s];
      }
    }
    hash_clear(hash, a.hash_slots);
    __syncwarp();
#pragma unroll
    for (int s = 0; s < KM_S; s++) hash_insert(hash, hmask, cur_id[s] & kMaskedTomb);
    __syncwarp();

    uint32_t iter = 0, total = 0;
    for (;;) {
      // collect_top_p_normal: the first kp unexplored of the top Km, marked explored
      unsigned um[KM_S];
      uint32_t found = 0;
#pragma unroll
      for (int s = 0; s < KM_S; s++) {
        um[s] = __ballot_sync(kFull, (cur_id[s] & kParent) == 0);
        found += __popc(um[s]);
      }
      if (found == 0) break;
      int want_slot = -1;
      uint32_t want_src = 0;
      if (lane < kp && lane < found) {
        uint32_t r = lane;
#pragma unroll
        for (int s = 0; s < KM_S; s++) {
          const uint32_t c = __popc(um[s]);
          if (want_slot < 0) {
            if (r < c) {
              unsigned mm = um[s];
              for (uint32_t i = 0; i < r; i++) mm &= mm - 1u;
              want_src = static_cast<uint32_t>(__ffs(static_cast<int>(mm)) - 1);
              want_slot = s;
            } else {
              r -= c;
            }
          }
        }
      }
      uint32_t ex_lane = kTomb;
#pragma unroll
      for (int s = 0; s < KM_S; s++) {
        const uint32_t v = __shfl_sync(kFull, cur_id[s], want_src);
        if (want_slot == s) ex_lane = v;
      }
      {
        uint32_t before = 0;
#pragma unroll
        for (int s = 0; s < KM_S; s++) {
          const uint32_t rank = before + __popc(um[s] & lt_mask);
          if ((cur_id[s] & kParent) == 0 && rank < kp) cur_id[s] |= kParent;
          before += __popc(um[s]);
        }
      }
      if (++total > a.max_iters) {
        if (lane == 0) raise_error(a.status, kErrIterCap);
        break;  // the output is the list of the last completed merge
      }
      const uint32_t ex = __shfl_sync(kFull, ex_lane, e_of_lane);
      uint32_t node = kTomb;
      if (ex < a.n)
        node = a.graph[static_cast<uint64_t>(ex) * a.graph_degree + nb_of_lane];
      else if (ex != kTomb)
        raise_error(a.status, kErrCapacity);
      if (node >= a.n && node != kTomb) {
        raise_error(a.status, kErrBadId);
        node = kTomb;
      }
      const bool valid = node != kTomb;
      const unsigned same = __match_any_sync(kFull, node);
      const bool first = lane == static_cast<uint32_t>(__ffs(static_cast<int>(same)) - 1);
      const bool newc = valid && first && hash_test_and_set(hash, hmask, node);
      __syncwarp();
      const float dist = score_passes<KSTEPS, ROWS>(a, q, node, newc, rows, mbar, phase, ok);
      if (!ok) break;
      const unsigned scored = __ballot_sync(kFull, newc);
      ev += (lane == 0) ? __popc(scored) : 0u;
      // the list this merge sorts: top (positions 0..Km-1) + candidates (Km..Km+31)
#pragma unroll
      for (int s = 0; s < KM_S; s++) {
        top_key[s] = (cur_key[s] & 0xFFFFFFFF00000000ull) | (static_cast<uint32_t>(s) * 32u + lane);
        top_id[s] = cur_id[s];
      }
      cand_key = pack_key(newc ? dist : FLT_MAX, KM + lane);
      cand_id = node;
      // rank merge of the candidates below the current Km-th key (see k_search_m32)
      const uint64_t worst = __shfl_sync(kFull, top_key[KM_S - 1], 31);
      uint32_t shift[KM_S];
#pragma unroll
      for (int s = 0; s < KM_S; s++) shift[s] = 0;
      uint32_t cpos = 0xFFFFFFFFu;
      unsigned rem = __ballot_sync(kFull, newc && cand_key < worst);
      while (rem) {
        const uint32_t c = static_cast<uint32_t>(__ffs(static_cast<int>(rem)) - 1);
        rem &= rem - 1u;
        const uint64_t kc = __shfl_sync(kFull, cand_key, c);
        uint32_t below_top = 0;
#pragma unroll
        for (int s = 0; s < KM_S; s++) {
          below_top += __popc(__ballot_sync(kFull, top_key[s] < kc));
          shift[s] += (top_key[s] > kc) ? 1u : 0u;
        }
        const uint32_t below_cand = __popc(__ballot_sync(kFull, newc && cand_key < kc));
        if (lane == c) cpos = below_top + below_cand;
      }
#pragma unroll
      for (int s = 0; s < KM_S; s++) {
        const uint32_t tpos = static_cast<uint32_t>(s) * 32u + lane + shift[s];
        if (tpos < KM) {
          mkey[tpos] = top_key[s];
          mid[tpos] = top_id[s];
        }
      }
      if (cpos < KM) {
        mkey[cpos] = cand_key;
        mid[cpos] = cand_id;
      }
      __syncwarp();
#pragma unroll
      for (int s = 0; s < KM_S; s++) {
        cur_key[s] = mkey[static_cast<uint32_t>(s) * 32u + lane];
        cur_id[s] = mid[static_cast<uint32_t>(s) * 32u + lane];
      }
      __syncwarp();
      if (++iter == a.reset_iter) {
        hash_clear(hash, a.hash_slots);
        __syncwarp();
#pragma unroll
        for (int s = 0; s < KM_S; s++) hash_insert(hash, hmask, cur_id[s] & kMaskedTomb);
        __syncwarp();
        iter = 0;
      }
    }
    if (!ok) break;
    it_all += (lane == 0) ? total : 0u;
    uint64_t k2[EF];
    uint32_t i2[EF];
#pragma unroll
    for (int s = 0; s < EF; s++) {
      k2[s] = s < KM_S ? top_key[s < KM_S ? s : 0] : (s == KM_S ? cand_key : ~0ull);
      i2[s] = s < KM_S ? top_id[s < KM_S ? s : 0] : (s == KM_S ? cand_id : kTomb);
    }
    warp_sort_kv<EF>(k2, i2);
    uint32_t* orow = a.out + static_cast<uint64_t>(qid) * a.out_width;
#pragma unroll
    for (int s = 0; s < EF; s++) {
      const uint32_t pos = static_cast<uint32_t>(s) * 32u + lane;
      if (pos < KM + 32u && pos < a.out_width) orow[pos] = i2[s] & kMaskedTomb;
    }
  }
  if (!ok) {
    if (lane == 0) raise_error(a.status, kErrWait);
    mbar_wait_bounded(mbar, phase ^ 1u);
  }
  if (lane == 0) {
    if (ev) atomicAdd(a.evals, ev);
    if (it_all) atomicAdd(a.iters, it_all);
  }
}

size_t search_mk_smem(uint32_t d, uint32_t hash_slots, uint32_t rows, uint32_t km) {
  return 16 + 12 * static_cast<size_t>(km) + 4 * static_cast<size_t>(hash_slots) +
         static_cast<size_t>(rows) * 4 * d;
}

template <int KM_S, int KS>
static cudaError_t launch_search_mk(const SearchArgs& a, int num_sms, size_t smem_optin,
                                    cudaStream_t st) {
  constexpr int ROWS = 8;
  const size_t smem = search_mk_smem(a.d, a.hash_slots, ROWS, 32u * KM_S);
  if (smem > smem_optin) return cudaErrorInvalidValue;
  auto kern = k_search_mk<KM_S, KS, ROWS>;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       static_cast<int>(smem));
  if (e != cudaSuccess) return e;
  int per_sm = 0;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, 32, smem);
  if (e != cudaSuccess) return e;
  if (a.max_blocks_per_sm && per_sm > static_cast<int>(a.max_blocks_per_sm))
    per_sm = static_cast<int>(a.max_blocks_per_sm);
  if (per_sm < 1) per_sm = 1;
  uint64_t blocks = static_cast<uint64_t>(num_sms) * per_sm;
  const uint64_t nq = a.queries ? a.nq : a.n;
  if (blocks > nq) blocks = nq;
  kern<<<static_cast<unsigned>(blocks), 32, smem, st>>>(a);
  return cudaGetLastError();
}

size_t search_m32_smem(uint32_t d, uint32_t hash_slots, uint32_t rows) {
  return 16 + 256 + 128 + 4 * static_cast<size_t>(hash_slots) + static_cast<size_t>(rows) * 4 * d;
}

template <int KS, int ROWS>
static cudaError_t launch_search_m32(const SearchArgs& a, int num_sms, size_t smem_optin,
                                     cudaStream_t st) {
  const size_t smem = search_m32_smem(a.d, a.hash_slots, ROWS);
  if (smem > smem_optin) return cudaErrorInvalidValue;
  auto kern = k_search_m32<KS, ROWS>;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       static_cast<int>(smem));
  if (e != cudaSuccess) return e;
  int per_sm = 0;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, 32, smem);
  if (e != cudaSuccess) return e;
  if (a.max_blocks_per_sm && per_sm > static_cast<int>(a.max_blocks_per_sm))
    per_sm = static_cast<int>(a.max_blocks_per_sm);
  if (per_sm < 1) per_sm = 1;
  uint64_t blocks = static_cast<uint64_t>(num_sms) * per_sm;
  const uint64_t nq = a.queries ? a.nq : a.n;
  if (blocks > nq) blocks = nq;
  kern<<<static_cast<unsigned>(blocks), 32, smem, st>>>(a);
  return cudaGetLastError();
}

// The distances of every query to its 32 seeds ((seed_base + s) % n_sub + offset), in the
// search's FP32 order (Gsearcher.cuh:958-976): residue r = i mod 32 accumulates q[i]*x[i] in i
// order, then the shuffle-down tree 16, 8, 4, 2, 1.  Lane s holds seed s's 32 residue chains in
// registers and folds them in the tree's pairs.  The seeds of one (sub-)index are the same 32
// rows for every query, so they stay in L1; this pass replaces the four staging passes per query
// and round that scoring the seeds inside the search takes.  One warp per query.
__global__ void __launch_bounds__(256) k_seed_dists(SearchArgs a, float* __restrict__ out) {
  const uint32_t lane = lane_id();
  const uint64_t nq = a.queries ? a.nq : a.n;
  const uint64_t nw = static_cast<uint64_t>(gridDim.x) * (blockDim.x >> 5);
  const uint32_t d = a.d;
  for (uint64_t qid = blockIdx.x * static_cast<uint64_t>(blockDim.x >> 5) + (threadIdx.x >> 5);
       qid < nq; qid += nw) {
    uint64_t soff = 0, sn = a.n;
    if (a.seg_count) {
      const uint32_t sg = segment_of(a.seg_off, a.seg_count, qid);
      soff = a.seg_off[sg];
      sn = a.seg_off[sg + 1] - soff;
    }
    const uint64_t node = (a.seed_base + static_cast<uint64_t>(lane)) % sn + soff;
    const float4* q4 =
        reinterpret_cast<const float4*>((a.queries ? a.queries : a.base) + qid * d);
    const float4* x4 = reinterpret_cast<const float4*>(a.base + node * d);
    float s[32];
#pragma unroll
    for (int r = 0; r < 32; r++) s[r] = 0.f;
    for (uint32_t b = 0; b < d; b += 32) {
#pragma unroll
      for (int j = 0; j < 8; j++) {
        if (b + 4u * j < d) {
          const float4 q = __ldg(q4 + (b >> 2) + j);
          const float4 x = __ldg(x4 + (b >> 2) + j);
          s[4 * j] = fmaf(q.x, x.x, s[4 * j]);
          s[4 * j + 1] = fmaf(q.y, x.y, s[4 * j + 1]);
          s[4 * j + 2] = fmaf(q.z, x.z, s[4 * j + 2]);
          s[4 * j + 3] = fmaf(q.w, x.w, s[4 * j + 3]);
        }
      }
    }
#pragma unroll
    for (int w = 16; w >= 1; w >>= 1)
#pragma unroll
      for (int r = 0; r < w; r++) s[r] = s[r] + s[r + w];
    out[qid * 32u + lane] = -s[0];
  }
}

cudaError_t launch_seed_dists(const SearchArgs& a, float* out, int num_sms, cudaStream_t st) {
  if (a.d == 0 || (a.d % 4) != 0 || !out) return cudaErrorInvalidValue;
  const uint64_t nq = a.queries ? a.nq : a.n;
  if (nq == 0) return cudaSuccess;
  uint64_t blocks = (nq + 7) / 8;
  const uint64_t cap = static_cast<uint64_t>(num_sms) * 8;
  if (blocks > cap) blocks = cap;
  k_seed_dists<<<static_cast<unsigned>(blocks), 256, 0, st>>>(a, out);
  return cudaGetLastError();
}

bool search_supported(uint32_t d, uint32_t km, uint32_t kp, uint32_t kd) {
  return d > 0 && d <= 512 && (d % 4) == 0 && kp * kd == 32 && kp >= 1 && km >= 32 &&
         km <= 96 && (km % 32) == 0;
}

cudaError_t launch_search(const SearchArgs& a, int num_sms, size_t smem_optin, cudaStream_t st) {
  if (!search_supported(a.d, a.km, a.kp, a.kd)) return cudaErrorInvalidValue;
  const int km_s = static_cast<int>(a.km / 32);
  const bool small = a.d <= 256;
  if (a.rows != 0 && a.rows != 8 && a.rows != 16) return cudaErrorInvalidValue;
  const bool r16 = a.rows == 16;
  switch (km_s) {
    case 1:
      if (a.d <= 224)
        return r16 ? launch_search_m32<7, 16>(a, num_sms, smem_optin, st)
                   : launch_search_m32<7, 8>(a, num_sms, smem_optin, st);
      if (small)
        return r16 ? launch_search_m32<8, 16>(a, num_sms, smem_optin, st)
                   : launch_search_m32<8, 8>(a, num_sms, smem_optin, st);
      return r16 ? launch_search_m32<16, 16>(a, num_sms, smem_optin, st)
                 : launch_search_m32<16, 8>(a, num_sms, smem_optin, st);
    case 2:
      if (a.d <= 224) return launch_search_mk<2, 7>(a, num_sms, smem_optin, st);
      return small ? launch_search_mk<2, 8>(a, num_sms, smem_optin, st)
                   : launch_search_mk<2, 16>(a, num_sms, smem_optin, st);
    default:
      if (a.d <= 224) return launch_search_mk<3, 7>(a, num_sms, smem_optin, st);
      return small ? launch_search_mk<3, 8>(a, num_sms, smem_optin, st)
                   : launch_search_mk<3, 16>(a, num_sms, smem_optin, st);
  }
}

}  // namespace pg
