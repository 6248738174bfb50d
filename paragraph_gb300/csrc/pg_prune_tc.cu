// pg_prune_tc.cu -- screened prune + reverse (K6/K10) with the candidate Gram on the tcgen05
// tensor cores.
//
// Same result as k_prune_reverse (strict rounds), bit for bit: the RNG occlusion scan of
// fusion_prune_reverse_kernel_v0 (Gbuilder.cuh:1093-1244, scan at :1150-1199), each occlusion
// test dist(p, r) < d_p decided from a screened 16-bit inner product when that lies farther than
// a proven error bound from d_p, and re-scored with the reference's FP32 chain otherwise.
//
// One CTA works on tiles of 128 candidate rows -- two nodes of up to 64 candidates (c <= 64) or
// one node of up to 128 -- with one thread per tile row (four warps):
//   1. each warp streams its 32 candidate rows, 32 FP32 columns per chunk, into a ring of S
//      chunk stages with 16-byte cp.async copies, eight lanes per row segment (coalesced; no
//      registers held while the copies are in flight; S - 1 chunks run ahead, across tiles),
//      the 16-byte pieces XOR-swizzled by row so that the 32 threads, one per row, read their
//      rows without bank conflicts; the node rows come with a tile's first chunk;
//   2. each thread runs the exact FP32 chain dist(b, x) = -(b . x) of its candidate x against
//      the node b (distance_between's order, Gbuilder.cuh:785-797) over the chunk, and rounds
//      the chunk to FP16 (or BF16) into the MMA operand (K-major 8-row x 16-byte core matrices,
//      no swizzle);
//   3. one thread issues tcgen05.mma (M = N = 128, K = 16 per instruction, FP32 accumulation)
//      for the chunk: the Gram G = A A^T of the tile's 16-bit rows accumulates in 128 TMEM
//      columns, and each node's block of G lies in the node's own TMEM lanes and columns;
//   4. the node's threads rank their candidates by (exact distance, slot) -- the stable order of
//      bubble_sort (Gbuilder.cuh:890-902) -- and run the kept-major scan: for each kept entry r
//      every undecided candidate p reads G[p][r] from its own TMEM lane (one tcgen05.ld column),
//      decides dist(p, r) < d_p from it outside the bound, or re-scores with the exact chain.
//      A candidate's recorded occluder is thus the first kept entry, in kept order, that
//      occludes it, and the kept list equals the reference's one-candidate-at-a-time scan.
// Error bound (x, y = FP32 rows, x^ = the 16-bit x, e_x = x - x^, Cauchy-Schwarz throughout;
// the two norms per point come from launch_screen_norms, once per build):
//   |sum x^y^ - sum xy| <= |e_x|(|y| + |e_y|) + |x||e_y|
//   |MMA(x^, y^) - sum x^y^| <= c_acc (|x| + |e_x|)(|y| + |e_y|)   (FP32 accumulation of Dp terms)
//   |chain(x, y) - sum xy| <= c_seq |x||y|                          (the reference's FP32 chain)
// with c_acc = (Dp + 32) 2^-21 (eight times the sequential-summation bound, covering the tensor
// core's accumulation) and c_seq = (D + 2) 2^-23, plus a 2^-20 relative guard on the comparison.
// Values beyond FP16's range give infinite norms, which send every test of that node to the
// exact chain.  Every mbarrier wait is bounded (one second); a thread that gives up makes the
// whole CTA stop at its next barrier and raises kErrWait.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include "pg_device.cuh"
#include "pg_kernels.h"
#include "pg_tc.cuh"

namespace pg {

namespace {

using namespace tcu;

constexpr uint32_t kTile = 128;                 // tile rows = MMA M = N = TMEM columns = threads
constexpr uint32_t kWarps = kTile / 32;
constexpr uint32_t kCk = 32;                    // FP32 columns per chunk
constexpr uint32_t kRowBytes = kCk * 4;         // bytes per row and chunk (eight 16-byte pieces)
constexpr uint32_t kStageBytes = kTile * kRowBytes;
constexpr uint32_t kOpBytes = kTile * kCk * 2;  // one 16-bit chunk of the tile
constexpr uint32_t kLbo = 128;                  // core matrices along K
constexpr uint32_t kSbo = 512;                  // core matrices along M / N (8-row groups)
constexpr uint32_t kBarAll = 1, kBarNode = 2;   // named barriers: all threads; node 0 (+ node)
constexpr uint32_t kNone = 0xFFFFFFFFu;

struct TcShape {
  uint32_t cap;    // candidate slots per node: 64 (two nodes per tile) or 128 (one)
  uint32_t nk;     // chunks per row
  uint32_t nbuf;   // node-row buffers (tiles whose node rows are in flight or in use)
  uint32_t dpad;   // floats per staged node row: D rounded up to the chunk
  uint64_t tiles;  // ceil(n / nodes per tile)
};

// Shared-memory layout, offsets from a 1024-byte aligned base.
struct Layout {
  uint32_t op, stage, nrow, key, id, nrm, err, xch, bars, words, total;
};
__host__ __device__ constexpr Layout layout(uint32_t stages, uint32_t nbuf, uint32_t dpad) {
  Layout l{};
  l.op = 0;
  l.stage = l.op + 2 * kOpBytes;
  l.nrow = l.stage + stages * kStageBytes;
  l.key = l.nrow + nbuf * 2 * dpad * 4;  // multiple of 16
  l.id = l.key + kTile * 8;
  l.nrm = l.id + kTile * 4;
  l.err = l.nrm + kTile * 4;
  l.xch = l.err + kTile * 4;
  l.bars = l.xch + 2 * kWarps * 4;  // opfree[2], acc, drained
  l.words = l.bars + 4 * 8;         // TMEM address
  l.total = l.words + 16;
  return l;
}
// Stages of the copy ring (chunks in flight per thread + the one consumed); the default can be
// set at build time with -DPG_PRUNE_TC_STAGES.
#ifndef PG_PRUNE_TC_STAGES
#define PG_PRUNE_TC_STAGES 2
#endif
constexpr uint32_t kMinStages = 2, kMaxStages = 4, kDefaultStages = PG_PRUNE_TC_STAGES;
size_t smem_bytes(uint32_t stages, const TcShape& sh) {
  return layout(stages, sh.nbuf, sh.dpad).total + 1024;
}

// Two floats rounded to the screening type (FP16 when HALF, else BF16), packed.
template <bool HALF>
__device__ __forceinline__ uint32_t pack2(float lo, float hi) {
  if constexpr (HALF) {
    const __half2 h = __floats2half2_rn(lo, hi);
    return *reinterpret_cast<const uint32_t*>(&h);
  } else {
    const __nv_bfloat162 h = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<const uint32_t*>(&h);
  }
}

// 16 bytes global -> shared, cached in L2 only, completing with the thread's copy groups.
__device__ __forceinline__ void cp16(void* dst, const void* src) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(saddr(dst)), "l"(src)
               : "memory");
}
__device__ __forceinline__ void cp_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <uint32_t N>
__device__ __forceinline__ void cp_wait() {
  asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}

// Bounded wait (one second) on the phase of parity `parity`, sleeping between tries: try_wait
// with a suspend-time hint returns as soon as the phase completes.
__device__ __forceinline__ bool bar_wait_hint(uint64_t* b, uint32_t parity) {
  constexpr uint32_t kHintNs = 100000;
  const uint64_t t0 = now_ns();
  for (;;) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(saddr(b)), "r"(parity), "r"(kHintNs)
        : "memory");
    if (ok) return true;
    if (now_ns() - t0 > 1000000000ull) return false;
  }
}

__device__ __forceinline__ void named_sync(uint32_t id, uint32_t threads) {
  asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(threads) : "memory");
}
// Named barrier that also returns the AND of `v` over the participating threads.
__device__ __forceinline__ bool named_and(uint32_t id, uint32_t threads, bool v) {
  uint32_t r;
  asm volatile(
      "{\n\t.reg .pred p, q;\n\tsetp.ne.u32 q, %3, 0;\n\t"
      "bar.red.and.pred p, %1, %2, q;\n\tselp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(r)
      : "r"(id), "r"(threads), "r"(v ? 1u : 0u)
      : "memory");
  return r != 0;
}

// Minimum of v over the threads of one node (warps col0 / 32 .. + nw - 1, named barrier
// bar_node); every thread of the node makes the same sequence of calls, numbered by q.
__device__ __forceinline__ uint32_t node_min(uint32_t v, uint32_t* xch, uint32_t& q,
                                             uint32_t col0, uint32_t nw, uint32_t bar_node,
                                             uint32_t threads) {
  v = __reduce_min_sync(kFull, v);
  uint32_t* xb = xch + (q & 1u) * kWarps;
  if ((threadIdx.x & 31u) == 0) xb[threadIdx.x >> 5] = v;
  __syncwarp();
  named_sync(bar_node, threads);
  uint32_t m = kNone;
  for (uint32_t w = 0; w < nw; w++) m = min(m, xb[col0 / 32u + w]);
  q++;
  return m;
}

// This thread's candidate id in tile t, or kNone when the slot holds no row to stage (past the
// end, a tomb, an out-of-range id or the node itself).
__device__ __forceinline__ uint32_t cand_id(const PruneArgs& a, uint64_t t, uint32_t P,
                                            uint32_t node, uint32_t slot) {
  const uint64_t b = t * P + node;
  if (b >= a.n || slot >= a.c) return kNone;
  const uint32_t x = a.graph[b * a.c + slot];
  return (x >= a.n || x == static_cast<uint32_t>(b)) ? kNone : x;
}

// The copy stream of one thread: the chunks of its warp's rows in the CTA's tile order, S - 1
// chunks ahead of the one being consumed, one cp.async group per chunk (empty past the last
// tile).
struct Feed {
  uint64_t t;  // tile of the next chunk to issue
  uint32_t kc;  // the chunk
  uint32_t lt;  // the tile's index among this CTA's tiles (selects the node-row buffer)
  uint32_t x;   // this thread's candidate id in tile t (kNone: nothing to stage)
};

// Issues chunk f.kc of tile f.t into stage gi % S.  The warp copies its 32 rows four at a time:
// eight lanes per row, one 16-byte piece each, so that each copy instruction reads whole row
// segments (coalesced) rather than one piece of 32 rows.
template <uint32_t S>
__device__ __forceinline__ void feed_issue(Feed& f, const PruneArgs& a, const TcShape& sh,
                                           uint8_t* stage, float* nrow, uint32_t gi, uint32_t P,
                                           uint32_t node, uint32_t slot) {
  const uint32_t R = threadIdx.x, lane = R & 31u;
  if (f.t < sh.tiles) {
    const uint32_t pieces = min(kCk, a.d - f.kc * kCk) / 4;
    const uint32_t j = lane & 7u;
    uint8_t* st = stage + (gi % S) * kStageBytes;
#pragma unroll
    for (uint32_t i = 0; i < 8; i++) {
      const uint32_t rr = (R & ~31u) + 4u * i + (lane >> 3);  // tile row copied by this lane
      const uint32_t xr = __shfl_sync(kFull, f.x, 4u * i + (lane >> 3));
      if (xr != kNone && j < pieces)
        cp16(st + rr * kRowBytes + ((j ^ (rr & 7u)) << 4),
             reinterpret_cast<const char*>(a.base + static_cast<uint64_t>(xr) * a.d) +
                 f.kc * kRowBytes + 16u * j);
    }
    if (f.kc == 0) {  // the node rows of the tile, 16-byte pieces spread over the node's threads
      const uint64_t b = f.t * P + node;
      if (b < a.n) {
        const char* nsrc = reinterpret_cast<const char*>(a.base + b * a.d);
        float* nb = nrow + ((f.lt % sh.nbuf) * 2 + node) * sh.dpad;
        for (uint32_t i = slot; i < a.d / 4; i += sh.cap) cp16(nb + 4 * i, nsrc + 16u * i);
      }
    }
    if (++f.kc == sh.nk) {
      f.kc = 0;
      f.t += gridDim.x;
      f.lt++;
      f.x = f.t < sh.tiles ? cand_id(a, f.t, P, node, slot) : kNone;
    }
  }
  cp_commit();
}

template <bool HALF, uint32_t S>
__global__ void __launch_bounds__(kTile, S == 2 ? 4 : 3) k_prune_tc(const PruneArgs a, const TcShape sh) {
  extern __shared__ __align__(16) uint8_t smem_raw[];
  uint8_t* sm = smem_raw + ((1024u - (saddr(smem_raw) & 1023u)) & 1023u);
  const Layout L = layout(S, sh.nbuf, sh.dpad);
  uint8_t* op = sm + L.op;
  uint8_t* stage = sm + L.stage;
  float* nrow = reinterpret_cast<float*>(sm + L.nrow);
  uint64_t* skey = reinterpret_cast<uint64_t*>(sm + L.key);
  uint32_t* sid = reinterpret_cast<uint32_t*>(sm + L.id);
  float* snrm = reinterpret_cast<float*>(sm + L.nrm);
  float* serr = reinterpret_cast<float*>(sm + L.err);
  uint32_t* xch = reinterpret_cast<uint32_t*>(sm + L.xch);
  uint64_t* opfree = reinterpret_cast<uint64_t*>(sm + L.bars);  // [2]
  uint64_t* accfull = opfree + 2;
  uint64_t* drained = accfull + 1;
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(sm + L.words);

  const uint32_t R = threadIdx.x, warp = R >> 5, lane = R & 31u;
  const uint32_t cap = sh.cap, P = kTile / cap;
  const uint32_t node = R / cap, slot = R - node * cap, col0 = node * cap;
  const uint32_t bar_node = kBarNode + node, nw = cap / 32u;

  if (R == 0) {
    bar_init(opfree, 1);
    bar_init(opfree + 1, 1);
    bar_init(accfull, 1);
    bar_init(drained, 1);
    fence_barrier_init();
  }
  if (warp == 0) tmem_alloc(tmem_slot, kTile);
  fence_before();
  __syncthreads();
  fence_after();
  const uint32_t tmem = *tmem_slot;
  const uint32_t taddr = tmem + ((warp * 32u) << 16);

  const uint32_t d = a.d;
  const float c_acc = static_cast<float>((d + 15u) / 16u * 16u + 32u) * 4.76837158e-07f;  // 2^-21
  const float c_seq = static_cast<float>(d + 2u) * 1.19209290e-07f;                   // 2^-23
  // A and B FP16 (format 0) or BF16 (format 1, bits 7-9 and 10-12)
  constexpr uint32_t kIdesc = idesc_f16(kTile, kTile) | (HALF ? 0u : ((1u << 7) | (1u << 10)));
  uint64_t ev = 0, resc = 0;
  uint32_t g = 0, q = 0, it = 0;
  bool ok = true;

  Feed f{blockIdx.x, 0, 0, kNone};
  if (f.t < sh.tiles) f.x = cand_id(a, f.t, P, node, slot);
  for (uint32_t i = 0; i + 1 < S; i++) feed_issue<S>(f, a, sh, stage, nrow, i, P, node, slot);

  for (uint64_t t = blockIdx.x; t < sh.tiles; t += gridDim.x, it++) {
    const uint64_t b = t * P + node;
    const bool bval = b < a.n;
    uint32_t x = kTomb;
    if (bval && slot < a.c) {
      x = a.graph[b * a.c + slot];
      if (x >= a.n && x != kTomb && x != kMaskedTomb) {
        raise_error(a.status, kErrBadId);
        x = kTomb;
      }
    }
    const bool valid = bval && x != kTomb && x != kMaskedTomb && x != static_cast<uint32_t>(b);
    const float* nb = nrow + ((it % sh.nbuf) * 2 + node) * sh.dpad;
    float acc = 0.f;
    for (uint32_t kc = 0; kc < sh.nk; kc++, g++) {
      feed_issue<S>(f, a, sh, stage, nrow, g + S - 1, P, node, slot);
      cp_wait<S - 1>();  // this thread's copies of chunk g have landed; after the warp
      __syncwarp();      // barrier, so have the copies of this thread's row by the others
      if (kc == 0) named_sync(kBarAll, kTile);  // and the node-row pieces, for a first chunk
      const uint32_t kn = min(kCk, d - kc * kCk);  // columns in this chunk, a multiple of 4
      const uint8_t* rp = stage + (g % S) * kStageBytes + R * kRowBytes;
      const float* np = nb + kc * kCk;
      uint32_t h[16];
#pragma unroll
      for (uint32_t j = 0; j < 8; j++) {
        float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
        if (valid && 4u * j < kn) {
          v = *reinterpret_cast<const float4*>(rp + ((j ^ (R & 7u)) << 4));
          const float4 u = *reinterpret_cast<const float4*>(np + 4u * j);
          acc = fmaf(u.x, v.x, acc);
          acc = fmaf(u.y, v.y, acc);
          acc = fmaf(u.z, v.z, acc);
          acc = fmaf(u.w, v.w, acc);
        }
        h[2 * j] = pack2<HALF>(v.x, v.y);
        h[2 * j + 1] = pack2<HALF>(v.z, v.w);
      }
      const uint32_t o = g & 1u;
      bool w = true;
      if (g >= 2) w = bar_wait_hint(opfree + o, ((g >> 1) + 1u) & 1u);  // MMAs of chunk g - 2
      if (w) {
        uint8_t* dst = op + o * kOpBytes + (R >> 3) * kSbo + (R & 7u) * 16u;
#pragma unroll
        for (uint32_t j = 0; j < 4; j++)
          *reinterpret_cast<uint4*>(dst + j * kLbo) =
              make_uint4(h[4 * j], h[4 * j + 1], h[4 * j + 2], h[4 * j + 3]);
      }
      fence_proxy_async();
      __syncwarp();
      ok = named_and(kBarAll, kTile, w);
      if (!ok) break;
      if (R == 0) {
        fence_after();
        const uint32_t a0 = saddr(op + o * kOpBytes);
        const uint32_t steps = (kn + 15u) >> 4;
        for (uint32_t k = 0; k < steps; k++) {
          const uint64_t dsc = plain_desc(a0 + k * 2u * kLbo, kLbo, kSbo);
          mma_f16(tmem, dsc, dsc, kIdesc, (kc | k) != 0);
        }
        commit(opfree + o);  // the operand buffer is free once these MMAs have read it
        if (kc + 1 == sh.nk) commit(accfull);
      }
    }
    if (!ok) break;
    __syncwarp();
    ok = named_and(kBarAll, kTile, bar_wait_hint(accfull, it & 1u));
    if (!ok) break;
    fence_after();

    // ---- the node's scan
    const bool in = slot < a.c;
    const float dist = valid ? -acc : FLT_MAX;
    const float2 ne = valid ? __ldg(a.norms + x) : make_float2(0.f, 0.f);
    skey[R] = in ? pack_key(dist, slot) : ~0ull;
    sid[R] = x;
    snrm[R] = ne.x;
    serr[R] = ne.y;
    const uint32_t nv = __popc(__ballot_sync(kFull, valid));
    if (lane == 0) ev += nv;
    __syncwarp();
    named_sync(bar_node, cap);
    uint32_t pos = kNone;
    if (in) {
      const uint64_t my = skey[R];
      uint32_t r = 0;
      for (uint32_t j = 0; j < a.c; j++) r += skey[col0 + j] < my ? 1u : 0u;
      pos = r;
    }
    const bool tomb = in && (x == kTomb || x == kMaskedTomb);
    // the first tomb in sorted order, and the slot at sorted position 0
    const uint32_t tend = node_min(tomb ? pos : a.c, xch, q, col0, nw, bar_node, cap);
    const uint32_t k0 = node_min(in ? (pos << 8) | slot : kNone, xch, q, col0, nw, bar_node, cap);
    uint32_t K = 0, my_kept = kNone;
    if (tend != 0 && k0 != kNone) {
      K = 1;
      uint32_t ro = k0 & 0xFFu, last = 0, jend = 1, nres = 0, fo = kNone;
      if (slot == ro) my_kept = 0;
      while (a.p > 1) {
        const uint32_t t_k = K - 1;
        const uint32_t ri = sid[col0 + ro];
        const float nr = snrm[col0 + ro], er = serr[col0 + ro];
        const float gv = __uint_as_float(tmem_ld1(taddr + col0 + ro));
        tmem_wait_ld();
        if (in && pos > last && pos < tend && fo == kNone) {
          const float dhat = -gv;
          const float np2 = ne.x, ep = ne.y;
          const float bound = ep * (nr + er) + np2 * er + c_acc * (np2 + ep) * (nr + er) +
                              c_seq * np2 * nr + fabsf(dhat) * 9.5367431640625e-07f + 1e-30f;
          bool yes = dhat + bound < dist;
          if (!yes && !(dhat - bound >= dist)) {  // inside the margin (or NaN): exact chain
            // a re-score holds up the node's scan: 256-bit loads whatever the row length
            yes = dist_seq<true>(a.base + static_cast<uint64_t>(x) * d,
                                 a.base + static_cast<uint64_t>(ri) * d, d) < dist;
            nres++;
          }
          if (yes) fo = t_k;
        }
        const uint32_t nk = node_min(
            (in && pos > last && pos < tend && fo == kNone) ? (pos << 8) | slot : kNone, xch, q,
            col0, nw, bar_node, cap);
        if (nk == kNone) {  // no undecided candidate before the first tomb
          jend = tend;
          break;
        }
        ro = nk & 0xFFu;
        if (slot == ro) my_kept = K;
        K++;
        last = nk >> 8;
        if (K == a.p) {
          jend = last + 1;
          break;
        }
      }
      const uint32_t ch = (in && pos >= 1 && pos < jend && fo != kNone) ? fo + 1 : 0u;
      const uint32_t chs = __reduce_add_sync(kFull, ch);
      const uint32_t rs = __reduce_add_sync(kFull, nres);
      if (lane == 0) {
        ev += chs;
        resc += rs;
      }
    }
    if (bval) {
      if (R == col0) {
        a.pruned_num[b] = K;
        if (K > 1) ev += static_cast<uint64_t>(K) * (K - 1) / 2;  // kept entry m made m tests
      }
      if (my_kept != kNone) {
        a.pruned[b * a.p + my_kept] = x;
        atomicAdd(a.indeg + x, 1u);
      }
    }
    fence_before();  // the TMEM reads above precede the next tile's first MMA
  }
  cp_wait<0>();  // no copy lands after the CTA exits
  if (lane == 0) {
    if (ev) atomicAdd(a.evals, static_cast<unsigned long long>(ev));
    if (resc && a.rescored) atomicAdd(a.rescored, static_cast<unsigned long long>(resc));
  }
  if (R == 0) {
    if (!ok) raise_error(a.status, kErrWait);
    commit(drained);  // arrives once every MMA issued above has completed
    bar_wait(drained, 0, nullptr);
  }
  fence_before();
  __syncthreads();
  if (warp == 0) {
    fence_after();
    tmem_dealloc(tmem, kTile);
  }
}

}  // namespace

template <bool HALF, uint32_t S>
cudaError_t launch_s(const PruneArgs& a, const TcShape& sh, int num_sms, cudaStream_t st) {
  const size_t smem = smem_bytes(S, sh);
  auto kern = k_prune_tc<HALF, S>;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       static_cast<int>(smem));
  if (e != cudaSuccess) return e;
  // the largest shared-memory carveout, so that several CTAs fit on an SM (the driver otherwise
  // picks the smallest carveout that holds one)
  e = cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
  if (e != cudaSuccess) return e;
  // CTAs per SM from the kernel's registers and shared memory (at most 4: 4 x 128 TMEM columns)
  cudaFuncAttributes fa{};
  e = cudaFuncGetAttributes(&fa, kern);
  if (e != cudaSuccess) return e;
  int dev = 0, smem_sm = 0, regs_sm = 0;
  if ((e = cudaGetDevice(&dev)) != cudaSuccess) return e;
  if ((e = cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev)) !=
      cudaSuccess)
    return e;
  if ((e = cudaDeviceGetAttribute(&regs_sm, cudaDevAttrMaxRegistersPerMultiprocessor, dev)) !=
      cudaSuccess)
    return e;
  const int regs_cta = ((fa.numRegs + 7) / 8 * 8) * static_cast<int>(kTile);
  int per_sm = smem_sm / static_cast<int>(smem + fa.sharedSizeBytes + 1024);  // + reserved 1 KB
  if (regs_cta > 0 && regs_sm / regs_cta < per_sm) per_sm = regs_sm / regs_cta;
  if (per_sm < 1) per_sm = 1;
  if (per_sm > 4) per_sm = 4;
  uint64_t blocks = static_cast<uint64_t>(num_sms) * per_sm;
  if (blocks > sh.tiles) blocks = sh.tiles;
  kern<<<static_cast<unsigned>(blocks), kTile, smem, st>>>(a, sh);
  return cudaGetLastError();
}

cudaError_t launch_prune_screen(const PruneArgs& a, int num_sms, size_t smem_optin,
                                cudaStream_t st) {
  if (!screen_supported(a.c, a.d, a.strict) || !a.norms ||
      (reinterpret_cast<uintptr_t>(a.base) % 16) != 0)
    return cudaErrorInvalidValue;
  if (a.n == 0) return cudaSuccess;
  if (a.n > 0x7FFFFFFFull) return cudaErrorInvalidValue;
  TcShape sh{};
  sh.cap = a.c <= 64 ? 64u : 128u;
  sh.nk = (a.d + kCk - 1) / kCk;
  sh.dpad = sh.nk * kCk;
  const uint32_t per_tile = kTile / sh.cap;
  sh.tiles = (a.n + per_tile - 1) / per_tile;
  uint32_t s = a.stages ? a.stages : kDefaultStages;
  if (s < kMinStages) s = kMinStages;
  if (s > kMaxStages) s = kMaxStages;
  auto fit = [&](uint32_t k) {
    sh.nbuf = (k - 1 + sh.nk - 1) / sh.nk + 1;  // tiles the copies run ahead, plus the current
    return smem_bytes(k, sh) <= smem_optin;
  };
  while (s > kMinStages && !fit(s)) s--;
  if (!fit(s)) return cudaErrorInvalidValue;
  const bool half = a.screen_half != 0;
  switch (s) {
    case 2: return half ? launch_s<true, 2>(a, sh, num_sms, st) : launch_s<false, 2>(a, sh, num_sms, st);
    case 3: return half ? launch_s<true, 3>(a, sh, num_sms, st) : launch_s<false, 3>(a, sh, num_sms, st);
    default: return half ? launch_s<true, 4>(a, sh, num_sms, st) : launch_s<false, 4>(a, sh, num_sms, st);
  }
}

}  // namespace pg
