// pg_screen.cu -- screened prune + reverse (K6/K10) with a BF16 or FP16 tensor-core Gram.
//
// Same result as k_prune_reverse (strict rounds), bit for bit.  Per node (one warp, up to 64
// candidates; up to 96 in the three-slot variant, whose Gram is built in two passes):
//   1. one pass over the candidate rows: each lane runs the exact FP32 chain dist(b, c) for its
//      candidates (distance_between's order, Gbuilder.cuh:785-797) and, from the same loads,
//      rounds the row to the 16-bit type; the two norms per point, |x| and |x - x^|, come from a
//      pre-pass over the base (k_screen_norms, once per build).  The 32 lanes read 32 different
//      rows, so each load instruction costs one L1 wavefront per row: with 32-byte aligned rows
//      (D % 8 == 0) the pass reads 32 bytes per lane per load (ld.global.v8), half the wavefronts
//      of float4 loads (measured at 1M x 200: 16 ms per prune round against 18.5);
//   2. the candidate Gram G = A A^T (A = the 16-bit rows, C x Dp, Dp = D rounded up to 16) on
//      the tensor cores (m16n8k16 MMA, FP32 accumulation), streamed: each 16-wide K chunk of the
//      rows goes through a 3 KB shared buffer straight into the MMAs, and the 20 m16n8 tiles of
//      the lower triangle accumulate in registers; G is kept packed (strictly lower);
//   3. the RNG scan of the plain kernel, kept-major: each entry, once kept, is tested against
//      every later undecided candidate at once, each occlusion test dist(p, r) < d_p decided from
//      -G[p][r] when it lies farther than the error bound E(p, r) from d_p, and re-scored with the
//      exact FP32 chain otherwise.
// Error bound (x, y = FP32 rows, x^ = bf16(x) or fp16(x), e_x = x - x^; Cauchy-Schwarz
// throughout; FP16's 11-bit significand makes |e_x| about 8x smaller than BF16's, so far fewer
// tests fall inside the margin -- values beyond FP16's range give infinite norms, which send
// every test of that node to the exact chain):
//   |sum x^y^ - sum xy| <= |e_x|(|y| + |e_y|) + |x||e_y|
//   |MMA(x^, y^) - sum x^y^| <= c_acc (|x| + |e_x|)(|y| + |e_y|)   (FP32 accumulation of Dp terms)
//   |chain(x, y) - sum xy| <= c_seq |x||y|                          (the reference's FP32 chain)
// with c_acc = (Dp + 32) * 2^-21 and c_seq = (D + 2) * 2^-23 (both several times the textbook
// gamma_n), plus a 2^-20 relative guard on the comparison itself.  |e_x| also carries the norm of
// x^'s subnormal part, so the bound holds whether the tensor core flushes subnormal inputs or not.
#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include "pg_device.cuh"
#include "pg_kernels.h"

namespace pg {

namespace {

// Two floats rounded to the screening type (FP16 when HALF, else BF16), packed; the rounding
// errors in elo / ehi.
template <bool HALF>
__device__ __forceinline__ uint32_t pack2(float lo, float hi, float& elo, float& ehi) {
  if constexpr (HALF) {
    const __half2 h = __floats2half2_rn(lo, hi);
    elo = lo - __low2float(h);
    ehi = hi - __high2float(h);
    return *reinterpret_cast<const uint32_t*>(&h);
  } else {
    const __nv_bfloat162 h = __floats2bfloat162_rn(lo, hi);
    elo = lo - __low2float(h);
    ehi = hi - __high2float(h);
    return *reinterpret_cast<const uint32_t*>(&h);
  }
}

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

__device__ __forceinline__ void ldsm_x4(uint32_t (&r)[4], const void* p) {
  const uint32_t a = static_cast<uint32_t>(__cvta_generic_to_shared(p));
  asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
               : "r"(a));
}

template <bool HALF>
__device__ __forceinline__ void mma16(float (&c)[4], const uint32_t (&a)[4],
                                      const uint32_t (&b)[2]) {
  if constexpr (HALF) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.f16.f16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, "
        "{%8,%9}, {%0,%1,%2,%3};"
        : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
  } else {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, "
        "{%8,%9}, {%0,%1,%2,%3};"
        : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
  }
}

__device__ __forceinline__ float key_to_dist(uint64_t key) {
  const uint32_t o = static_cast<uint32_t>(key >> 32);
  const uint32_t u = (o & 0x80000000u) ? (o & 0x7FFFFFFFu) : ~o;
  return __uint_as_float(u);
}

__host__ __device__ inline uint32_t screen_dp(uint32_t d) { return (d + 15u) / 16u * 16u; }

}  // namespace

namespace {

constexpr uint32_t kChunkStride = 24;  // 16-bit values per chunk row: 48 B keeps ldmatrix rows conflict-free

template <int NS>
struct ScreenShape {
  static constexpr uint32_t kC = 32u * NS;                 // candidates per node
  static constexpr uint32_t kTri = kC * (kC - 1) / 2;      // packed strictly-lower Gram entries
};

// Per-warp shared memory of the screened kernels.
struct ScreenSmem {
  uint16_t* chunk;       // C x kChunkStride: one K chunk of the rows in the screening type
  float* G;              // C(C-1)/2: packed strictly-lower Gram
  uint32_t* ids;         // sorted ids
  float* dist;           // sorted exact distances to the node
  float* nrm;            // |x| per original slot
  float* err;            // |x - round(x)| per original slot (BF16 or FP16 rounding)
  uint32_t* orig;        // sorted position -> original slot
  uint32_t* kept_o;      // kept entries: original slot
  uint32_t* kept_i;      // kept entries: id
};

template <int NS>
__device__ __forceinline__ ScreenSmem screen_smem(unsigned char* raw) {
  constexpr uint32_t C = ScreenShape<NS>::kC;
  ScreenSmem m;
  m.chunk = reinterpret_cast<uint16_t*>(raw);
  m.G = reinterpret_cast<float*>(raw + static_cast<size_t>(C) * kChunkStride * 2);
  m.ids = reinterpret_cast<uint32_t*>(m.G + ScreenShape<NS>::kTri);
  m.dist = reinterpret_cast<float*>(m.ids + C);
  m.nrm = m.dist + C;
  m.err = m.nrm + C;
  m.orig = reinterpret_cast<uint32_t*>(m.err + C);
  m.kept_o = m.orig + C;
  m.kept_i = m.kept_o + C;
  return m;
}

__device__ __forceinline__ uint32_t tri_index(uint32_t r, uint32_t c) {  // r > c
  return r * (r - 1) / 2 + c;
}

// One streamed pass over the candidate rows, 16-wide K chunks through sm.chunk, accumulating the
// lower-triangle m16n8 Gram tiles of row blocks [MT_LO, MT_HI) (row block mt covers column tiles
// 0 .. 2 mt + 1) in registers and storing them packed into sm.G.  The FIRST pass also runs the
// exact chains dist(b, id[s]) (FLT_MAX where !valid[s]) and reads the two norms per row.  Lane l
// owns slots l, 32 + l, ...  V8: rows read 32 bytes per load (base 32-byte aligned, D % 8 == 0).
template <int NS, int MT_LO, int MT_HI, bool FIRST, bool HALF, bool V8>
__device__ __forceinline__ void screen_pass(const float* __restrict__ base, uint32_t d,
                                            const float2* __restrict__ norms,
                                            const float* __restrict__ brow,
                                            const uint32_t (&id)[NS], const bool (&valid)[NS],
                                            const ScreenSmem& sm, float (&dist)[NS]) {
  constexpr int kTiles = (MT_HI * (MT_HI + 1)) - (MT_LO * (MT_LO + 1));  // sum of 2 mt + 2
  const uint32_t lane = lane_id();
  const uint32_t dp = screen_dp(d);
  const uint32_t g = lane >> 2, t4 = lane & 3u;
  const float4* b4 = reinterpret_cast<const float4*>(brow);
  const float4* r4[NS];
#pragma unroll
  for (int s = 0; s < NS; s++)
    r4[s] = reinterpret_cast<const float4*>(valid[s] ? base + static_cast<uint64_t>(id[s]) * d
                                                     : brow);
  float acc[NS];
#pragma unroll
  for (int s = 0; s < NS; s++) acc[s] = 0.f;
  float gm[kTiles][4];  // tile (mt, nt) at mt*(mt+1) - MT_LO*(MT_LO+1) + nt
#pragma unroll
  for (int i = 0; i < kTiles; i++)
#pragma unroll
    for (int j = 0; j < 4; j++) gm[i][j] = 0.f;
  const uint32_t n4 = d >> 2;
  for (uint32_t k0 = 0; k0 < dp; k0 += 16) {
    if constexpr (V8) {
#pragma unroll
      for (uint32_t h = 0; h < 2; h++) {
        const uint32_t i = (k0 >> 3) + h;  // 8-float index
        const bool in = i < (d >> 3);
        float u[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
        if (FIRST && in) ld8(brow + 8 * i, u);
#pragma unroll
        for (int s = 0; s < NS; s++) {
          uint4 packed = make_uint4(0u, 0u, 0u, 0u);
          if (in) {
            float v[8];
            ld8(reinterpret_cast<const float*>(r4[s]) + 8 * i, v);
            packed.x = pack2<HALF>(v[0], v[1]);
            packed.y = pack2<HALF>(v[2], v[3]);
            packed.z = pack2<HALF>(v[4], v[5]);
            packed.w = pack2<HALF>(v[6], v[7]);
            if (FIRST) {
#pragma unroll
              for (int t = 0; t < 8; t++) acc[s] = fmaf(u[t], v[t], acc[s]);
            }
          }
          const uint32_t j = static_cast<uint32_t>(s) * 32u + lane;
          *reinterpret_cast<uint4*>(sm.chunk + j * kChunkStride + 8 * h) =
              valid[s] ? packed : make_uint4(0u, 0u, 0u, 0u);
        }
      }
    } else {
#pragma unroll
    for (uint32_t q = 0; q < 4; q++) {
      const uint32_t i = (k0 >> 2) + q;  // float4 index
      const bool in = i < n4;
      float4 u = make_float4(0.f, 0.f, 0.f, 0.f);
      if (FIRST && in) u = __ldg(b4 + i);
#pragma unroll
      for (int s = 0; s < NS; s++) {
        const float4 v = in ? __ldg(r4[s] + i) : make_float4(0.f, 0.f, 0.f, 0.f);
        uint2 packed = make_uint2(0u, 0u);
        if (in) {
          packed.x = pack2<HALF>(v.x, v.y);
          packed.y = pack2<HALF>(v.z, v.w);
          if (FIRST) {
            acc[s] = fmaf(u.x, v.x, acc[s]);
            acc[s] = fmaf(u.y, v.y, acc[s]);
            acc[s] = fmaf(u.z, v.z, acc[s]);
            acc[s] = fmaf(u.w, v.w, acc[s]);
          }
        }
        const uint32_t j = static_cast<uint32_t>(s) * 32u + lane;
        *reinterpret_cast<uint2*>(sm.chunk + j * kChunkStride + 4 * q) =
            valid[s] ? packed : make_uint2(0u, 0u);
      }
    }
    }
    __syncwarp();
    // A fragments of row blocks 0 .. MT_HI-1.  G = A A^T, so the B fragment of column tile nt
    // (rows 8 nt .. 8 nt + 7 as the n index) is half of an A fragment already held: (a0, a2) of
    // block nt / 2 for even nt, (a1, a3) for odd nt -- one ldmatrix.x4 per row block and chunk.
    uint32_t af[MT_HI][4];
#pragma unroll
    for (int mt = 0; mt < MT_HI; mt++)
      ldsm_x4(af[mt], sm.chunk + (16 * mt + (lane & 15u)) * kChunkStride + (lane >> 4) * 8);
#pragma unroll
    for (int mt = MT_LO; mt < MT_HI; mt++) {
#pragma unroll
      for (int nt = 0; nt <= 2 * mt + 1; nt++) {
        const uint32_t bf[2] = {af[nt >> 1][nt & 1], af[nt >> 1][(nt & 1) + 2]};
        mma16<HALF>(gm[mt * (mt + 1) - MT_LO * (MT_LO + 1) + nt], af[mt], bf);
      }
    }
    __syncwarp();
  }
#pragma unroll
  for (int mt = MT_LO; mt < MT_HI; mt++)
#pragma unroll
    for (int nt = 0; nt <= 2 * mt + 1; nt++) {
      const float* c = gm[mt * (mt + 1) - MT_LO * (MT_LO + 1) + nt];
      const uint32_t r0 = 16 * mt + g, c0 = 8 * nt + 2 * t4;
      if (r0 > c0) sm.G[tri_index(r0, c0)] = c[0];
      if (r0 > c0 + 1) sm.G[tri_index(r0, c0 + 1)] = c[1];
      if (r0 + 8 > c0) sm.G[tri_index(r0 + 8, c0)] = c[2];
      if (r0 + 8 > c0 + 1) sm.G[tri_index(r0 + 8, c0 + 1)] = c[3];
    }
  if (FIRST) {
#pragma unroll
    for (int s = 0; s < NS; s++) {
      const uint32_t j = static_cast<uint32_t>(s) * 32u + lane;
      const float2 ne = valid[s] ? __ldg(norms + id[s]) : make_float2(0.f, 0.f);
      sm.nrm[j] = ne.x;
      sm.err[j] = ne.y;
      dist[s] = valid[s] ? -acc[s] : FLT_MAX;
    }
  }
}

// Steps 1 and 2: exact chains, norms and the whole lower-triangle Gram of the 32 NS slots (two
// register passes for 96 candidates: row blocks 0-3, then 4-5).
template <int NS, bool HALF, bool V8>
__device__ __forceinline__ void screen_rows_and_gram(const float* __restrict__ base, uint32_t d,
                                                     const float2* __restrict__ norms,
                                                     const float* __restrict__ brow,
                                                     const uint32_t (&id)[NS],
                                                     const bool (&valid)[NS],
                                                     const ScreenSmem& sm, float (&dist)[NS]) {
  if constexpr (NS == 2) {
    screen_pass<2, 0, 4, true, HALF, V8>(base, d, norms, brow, id, valid, sm, dist);
  } else {
    screen_pass<3, 0, 4, true, HALF, V8>(base, d, norms, brow, id, valid, sm, dist);
    screen_pass<3, 4, 6, false, HALF, V8>(base, d, norms, brow, id, valid, sm, dist);
  }
}

// Sorts the slots by (exact distance, slot) into sm.ids / sm.dist / sm.orig (first c).
template <int NS>
__device__ __forceinline__ void screen_sort(const uint32_t (&idin)[NS], const float (&dist)[NS],
                                            uint32_t c, const ScreenSmem& sm) {
  constexpr int E = NS <= 2 ? 2 : 4;  // the bitonic network wants a power of two
  const uint32_t lane = lane_id();
  uint64_t key[E];
  uint32_t id[E];
#pragma unroll
  for (int s = 0; s < E; s++) {
    const uint32_t j = static_cast<uint32_t>(s) * 32u + lane;
    key[s] = (s < NS && j < c) ? pack_key(dist[s < NS ? s : 0], j) : ~0ull;
    id[s] = s < NS ? idin[s < NS ? s : 0] : kTomb;
  }
  warp_sort_kv<E>(key, id);
#pragma unroll
  for (int s = 0; s < E; s++) {
    const uint32_t i = static_cast<uint32_t>(s) * 32u + lane;
    if (i < c) {
      sm.ids[i] = id[s];
      sm.dist[i] = key_to_dist(key[s]);
      sm.orig[i] = key_pos(key[s]);
    }
  }
  __syncwarp();
}

// The occlusion scan of fusion_prune_reverse_kernel_v0 (Gbuilder.cuh:1150-1199), kept-major:
// lane l holds sorted positions l, 32 + l, ...; each entry, once kept, is tested against every
// later undecided candidate at once (Gbuilder.cuh:1163-1181's test dist(p, r) < d_p, decided
// from the screened Gram outside the error bound, re-scored with the exact FP32 chain inside
// it), and the next kept entry is the first candidate after it that no kept entry occludes.  A
// candidate's recorded occluder is thus the first kept entry, in kept order, that occludes it --
// the one the reference's one-candidate-at-a-time scan stops at -- and the kept list equals that
// scan's.  The scan ends at the first tomb or when `limit` entries are kept.  sm.kept_o/kept_i[0]
// hold sorted position 0 on entry.  Returns the kept count; *checks gets the reference's count
// of tests (up to the first occluder, for every candidate that scan reaches), *resc the exact
// re-scores.
template <int NS>
__device__ __forceinline__ uint32_t screen_scan(const float* __restrict__ base, uint32_t d,
                                                uint32_t c, uint32_t limit, float c_acc,
                                                float c_seq, const ScreenSmem& sm,
                                                uint64_t* checks, uint64_t* resc) {
  constexpr uint32_t kNone = 0xFFFFFFFFu;
  const uint32_t lane = lane_id();
  uint32_t tend = c;  // first tomb
  uint32_t pid[NS], po[NS], fo[NS];
  float np[NS], ep[NS], dp[NS];
#pragma unroll
  for (int s = 0; s < NS; s++) {
    const uint32_t pos = static_cast<uint32_t>(s) * 32u + lane;
    const bool in = pos < c;
    const uint32_t x = in ? sm.ids[pos] : kTomb;
    const unsigned m = __ballot_sync(kFull, in && (x == kTomb || x == kMaskedTomb));
    if (m && tend == c) tend = static_cast<uint32_t>(s) * 32u + __ffs(static_cast<int>(m)) - 1;
    pid[s] = x;
    po[s] = in ? sm.orig[pos] : 0u;
    np[s] = in ? sm.nrm[po[s]] : 0.f;
    ep[s] = in ? sm.err[po[s]] : 0.f;
    dp[s] = in ? sm.dist[pos] : 0.f;
    fo[s] = kNone;
  }
  uint32_t K = 1, last = 0, jend = 1, nres = 0;
  while (limit > 1) {
    const uint32_t t = K - 1;
    const uint32_t ro = sm.kept_o[t];
    const uint32_t ri = sm.kept_i[t];
    const float nr = sm.nrm[ro], er = sm.err[ro];
#pragma unroll
    for (int s = 0; s < NS; s++) {
      const uint32_t pos = static_cast<uint32_t>(s) * 32u + lane;
      if (pos > last && pos < tend && fo[s] == kNone) {
        const uint32_t a = po[s];
        const float dhat = -sm.G[a > ro ? tri_index(a, ro) : tri_index(ro, a)];
        const float bound = ep[s] * (nr + er) + np[s] * er + c_acc * (np[s] + ep[s]) * (nr + er) +
                            c_seq * np[s] * nr + fabsf(dhat) * 9.5367431640625e-07f + 1e-30f;
        bool yes = dhat + bound < dp[s];
        if (!yes && !(dhat - bound >= dp[s])) {  // inside the margin (or NaN): exact chain
          yes = dist_seq(base + static_cast<uint64_t>(pid[s]) * d,
                         base + static_cast<uint64_t>(ri) * d, d) < dp[s];
          nres++;
        }
        if (yes) fo[s] = t;
      }
    }
    uint32_t nxt = tend;
#pragma unroll
    for (int s = 0; s < NS; s++) {
      const uint32_t pos = static_cast<uint32_t>(s) * 32u + lane;
      const unsigned m = __ballot_sync(kFull, pos > last && pos < tend && fo[s] == kNone);
      if (m && nxt == tend) nxt = static_cast<uint32_t>(s) * 32u + __ffs(static_cast<int>(m)) - 1;
    }
    if (nxt >= tend) {
      jend = tend;
      break;
    }
    if (lane == 0) {
      sm.kept_o[K] = sm.orig[nxt];
      sm.kept_i[K] = sm.ids[nxt];
    }
    __syncwarp();
    K++;
    last = nxt;
    if (K == limit) {
      jend = nxt + 1;
      break;
    }
  }
  uint32_t ch = 0;
#pragma unroll
  for (int s = 0; s < NS; s++) {
    const uint32_t pos = static_cast<uint32_t>(s) * 32u + lane;
    if (pos >= 1 && pos < jend && fo[s] != kNone) ch += fo[s] + 1;
  }
  *checks += __reduce_add_sync(kFull, ch) + K * (K - 1) / 2;  // kept entry m made m tests
  *resc += __reduce_add_sync(kFull, nres);
  return K;
}

}  // namespace

// bytes of shared memory per warp
template <int NS>
size_t screen_smem_ns() {
  constexpr size_t C = ScreenShape<NS>::kC;
  return C * kChunkStride * 2                          // one K chunk of the 16-bit rows
         + static_cast<size_t>(ScreenShape<NS>::kTri) * 4  // G, strictly lower triangle
         + C * 4 * 7;                                  // ids, dist, |x|, |e|, slot, kept x2
}

bool screen_supported(uint32_t c, uint32_t d, int strict) {
  return strict && c <= ScreenShape<3>::kC && d >= 4 && d <= 1024 && (d % 4) == 0;
}

template <int NS, bool HALF, bool V8>
__global__ void __launch_bounds__(32, NS == 2 ? (V8 ? 12 : 16) : 8) k_prune_screen(PruneArgs a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const ScreenSmem sm = screen_smem<NS>(smem_raw);
  const uint32_t lane = lane_id();
  const uint32_t d = a.d;
  const float c_acc = static_cast<float>(screen_dp(d) + 32) * 4.76837158e-07f;  // 2^-21
  const float c_seq = static_cast<float>(d + 2) * 1.19209290e-07f;              // 2^-23
  uint64_t ev = 0, resc = 0;
  for (uint64_t b = blockIdx.x; b < a.n; b += gridDim.x) {
    uint32_t id[NS];
    bool valid[NS];
#pragma unroll
    for (int s = 0; s < NS; s++) {
      const uint32_t j = static_cast<uint32_t>(s) * 32u + lane;
      uint32_t x = (j < a.c) ? a.graph[b * a.c + j] : kTomb;
      if (x >= a.n && x != kTomb && x != kMaskedTomb) {
        raise_error(a.status, kErrBadId);
        x = kTomb;
      }
      id[s] = x;
      valid[s] = (x != kTomb && x != static_cast<uint32_t>(b) && x != kMaskedTomb);
    }
    float dist[NS];
    screen_rows_and_gram<NS, HALF, V8>(a.base, d, a.norms, a.base + b * d, id, valid, sm, dist);
    uint32_t nv = 0;
#pragma unroll
    for (int s = 0; s < NS; s++) nv += __popc(__ballot_sync(kFull, valid[s]));  // all lanes
    ev += (lane == 0) ? nv : 0u;
    screen_sort<NS>(id, dist, a.c, sm);

    const uint32_t first = sm.ids[0];
    if (first == kTomb || first == kMaskedTomb) {
      if (lane == 0) a.pruned_num[b] = 0;
      __syncwarp();
      continue;
    }
    if (lane == 0) {
      sm.kept_o[0] = sm.orig[0];
      sm.kept_i[0] = first;
    }
    __syncwarp();
    uint64_t checks = 0;
    const uint32_t cnt = screen_scan<NS>(a.base, d, a.c, a.p, c_acc, c_seq, sm, &checks, &resc);
    ev += (lane == 0) ? checks : 0;
    if (lane == 0) a.pruned_num[b] = cnt;
    for (uint32_t t = lane; t < cnt; t += 32) {
      const uint32_t dst = sm.kept_i[t];
      a.pruned[b * a.p + t] = dst;
      atomicAdd(a.indeg + dst, 1u);
    }
    __syncwarp();
  }
  if (lane == 0) {
    if (ev) atomicAdd(a.evals, static_cast<unsigned long long>(ev));
    if (resc && a.rescored) atomicAdd(a.rescored, static_cast<unsigned long long>(resc));
  }
}

// Per point: upper bounds of |x| and of |x - x^| + |x^_sub| (x^ = the 16-bit copy the screened
// prune packs, x^_sub its subnormal part), read by k_prune_screen in place of per-candidate sums.
// One warp per point.  The 1.0001 factor covers the FP32 sums' rounding for D <= 1024 and the
// 1e-21 term their underflow (at most D * 2^-150 absolute, whose square root is below 1e-21).
template <bool HALF>
__global__ void __launch_bounds__(256) k_screen_norms(const float* __restrict__ base, uint64_t n,
                                                      uint32_t d, float2* __restrict__ out) {
  const float min_normal = HALF ? 6.103515625e-05f : 1.17549435e-38f;  // 2^-14, 2^-126
  const uint32_t lane = lane_id();
  const uint64_t nw = static_cast<uint64_t>(gridDim.x) * (blockDim.x >> 5);
  for (uint64_t i = blockIdx.x * static_cast<uint64_t>(blockDim.x >> 5) + (threadIdx.x >> 5);
       i < n; i += nw) {
    const float4* r = reinterpret_cast<const float4*>(base + i * d);
    float nn = 0.f, ee = 0.f, ss = 0.f;
    for (uint32_t k = lane; k < (d >> 2); k += 32) {
      const float4 v = __ldg(r + k);
      const float x[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
      for (int t = 0; t < 4; t += 2) {
        float e0, e1;
        pack2<HALF>(x[t], x[t + 1], e0, e1);
        const float r0 = x[t] - e0, r1 = x[t + 1] - e1;  // the rounded values
        nn = fmaf(x[t], x[t], fmaf(x[t + 1], x[t + 1], nn));
        ee = fmaf(e0, e0, fmaf(e1, e1, ee));
        if (fabsf(r0) < min_normal) ss = fmaf(r0, r0, ss);
        if (fabsf(r1) < min_normal) ss = fmaf(r1, r1, ss);
      }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      nn += __shfl_xor_sync(kFull, nn, o);
      ee += __shfl_xor_sync(kFull, ee, o);
      ss += __shfl_xor_sync(kFull, ss, o);
    }
    if (lane == 0)
      out[i] = make_float2(sqrtf(nn) * 1.0001f + 1e-21f,
                           (sqrtf(ee) + sqrtf(ss)) * 1.0001f + 1e-21f);
  }
}

cudaError_t launch_screen_norms(const float* base, uint64_t n, uint32_t d, uint32_t half,
                                float2* out, int num_sms, cudaStream_t st) {
  if (n == 0) return cudaSuccess;
  if (d == 0 || (d % 4) != 0 || !out) return cudaErrorInvalidValue;
  uint64_t blocks = (n + 7) / 8;
  const uint64_t cap = static_cast<uint64_t>(num_sms) * 8;
  if (blocks > cap) blocks = cap;
  if (half)
    k_screen_norms<true><<<static_cast<unsigned>(blocks), 256, 0, st>>>(base, n, d, out);
  else
    k_screen_norms<false><<<static_cast<unsigned>(blocks), 256, 0, st>>>(base, n, d, out);
  return cudaGetLastError();
}

template <typename Args>
static cudaError_t launch_screen_kernel(void (*kern)(Args), const Args& a, uint64_t n,
                                        size_t smem, uint32_t carveout, int num_sms,
                                        size_t smem_optin, cudaStream_t st) {
  if (smem > smem_optin) return cudaErrorInvalidValue;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       static_cast<int>(smem));
  if (e != cudaSuccess) return e;
  // Hub rows recur across many nodes' candidate lists, so L1 hits matter more than resident
  // warps: keep about a quarter of the unified L1/shared capacity as L1 (measured on GB300 at
  // 1M x 200: 22 ms per prune round with this split against 35 ms with the largest shared
  // carveout).  A screened merge (K7/K11) built the same way was slower than the plain merge at
  // every list-length split tried: most merged lists hold 32 entries or fewer.  The autotuner
  // may pick another split (`carveout`).
  e = cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout,
                           carveout ? static_cast<int>(carveout) : 76);
  if (e != cudaSuccess) return e;
  int per_sm = 0;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, 32, smem);
  if (e != cudaSuccess) return e;
  if (per_sm < 1) per_sm = 1;
  uint64_t blocks = static_cast<uint64_t>(num_sms) * per_sm;
  if (blocks > n) blocks = n;
  kern<<<static_cast<unsigned>(blocks), 32, smem, st>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_prune_screen(const PruneArgs& a, int num_sms, size_t smem_optin,
                                cudaStream_t st) {
  if (!screen_supported(a.c, a.d, a.strict)) return cudaErrorInvalidValue;
  if (a.carveout > 100 || !a.norms) return cudaErrorInvalidValue;
  const bool half = a.screen_half != 0;
  const bool v8 = (reinterpret_cast<uintptr_t>(a.base) % 32) == 0 && (a.d % 8) == 0;
  const int sel = (a.c <= ScreenShape<2>::kC ? 0 : 4) + (half ? 2 : 0) + (v8 ? 1 : 0);
  using K = void (*)(PruneArgs);
  static const K kerns[8] = {k_prune_screen<2, false, false>, k_prune_screen<2, false, true>,
                             k_prune_screen<2, true, false>,  k_prune_screen<2, true, true>,
                             k_prune_screen<3, false, false>, k_prune_screen<3, false, true>,
                             k_prune_screen<3, true, false>,  k_prune_screen<3, true, true>};
  const size_t smem = sel < 4 ? screen_smem_ns<2>() : screen_smem_ns<3>();
  return launch_screen_kernel(kerns[sel], a, a.n, smem, a.carveout, num_sms, smem_optin, st);
}

}  // namespace pg
