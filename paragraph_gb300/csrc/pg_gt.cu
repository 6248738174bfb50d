// pg_gt.cu -- exact inner-product top-k ground truth on the GPU (sm_103a).
//
// The reference's build reads each training query's top-128 base ids from a file made outside it
// (README.md:25-31, notebooks); here they are computed on the GPU.  Result: for every query q the
// k base ids with the largest FP64 inner product q.x, ties to the lower id -- exact, whatever the
// arithmetic used to find them.
//
//   1. FP16 copies of base and queries, rows zero-padded to a multiple of 16 elements, with
//      per-row norms |x^| and |x - x^| (k_half_rows);
//   2. screening scores s^ = q^.x^ on the tensor cores: k_gt_tc, a persistent tcgen05 GEMM
//      (TMA-loaded 128-byte-swizzled tiles, FP32 accumulators in TMEM) whose epilogue consumes
//      each tile of scores in registers -- no score matrix is ever stored;
//   3. a rigorous bound: |q.x - s^| <= E_q = (|q^| + |e_q|) max|e_x| + |e_q| max|x^|
//      + g (|q^| max|x^|), with g covering the FP32 accumulation (d' * 2^-22, four times the
//      IEEE unit roundoff, for the tensor core's accumulation);
//   4. pass 1 (k_gt_tc<kMax>): the maximum screened score of every group of base rows per query
//      (disjoint groups, about 4096 or more of them); the k-th largest group maximum theta_q is
//      the score of k distinct base rows, so theta_q <= t_k, the k-th largest screened score of
//      the row (k_gt_theta);
//   5. pass 2 (k_gt_tc<kFilter>): every base row with s^ >= theta_q - 2 E_q is a candidate --
//      a superset of {s^ >= t_k - 2 E_q}, which holds the true top k (a true top-k member has
//      s^ >= s_k - E_q and s_k >= t_k - E_q);
//   6. k_gt_final: the candidates with s^ >= t_k - 2 E_q, exact FP64 inner products, sorted by
//      (score desc, id asc).
// With groups many enough that the top k fall in nearly distinct groups, theta_q sits just
// below t_k and a query keeps about 1.1 k candidates.
#include <cuda.h>
#include <cuda_fp16.h>

#include <cmath>

#include "pg_device.cuh"
#include "pg_kernels.h"
#include "pg_tc.cuh"

namespace pg {

namespace {

constexpr uint32_t kGtCap = 1024;          // candidates per query
constexpr uint32_t kGtErrRange = 1u << 4;  // a value beyond the FP16 range
constexpr uint32_t kGtErrFinal = 1u << 6;  // a query kept more candidates than kGtCap
constexpr int kFinalWarps = 2;

__device__ __forceinline__ float key_value(uint64_t key) {  // inverse of desc_key's value part
  const uint32_t o = ~static_cast<uint32_t>(key >> 32);
  const uint32_t u = (o & 0x80000000u) ? (o & 0x7FFFFFFFu) : ~o;
  return __uint_as_float(u);
}

// descending value, then ascending id, as an ascending 64-bit key
__device__ __forceinline__ uint64_t desc_key(float v, uint32_t id) {
  return (static_cast<uint64_t>(~order_key(v)) << 32) | id;
}

__device__ __forceinline__ uint64_t desc_key64(double v) {  // descending double
  const uint64_t u = static_cast<uint64_t>(__double_as_longlong(v + 0.0));
  const uint64_t o = (u >> 63) ? ~u : (u | 0x8000000000000000ull);
  return ~o;
}

// FP16 copy of rows x d FP32 values with row stride dp >= d (zeros in the padding), and per row
// upper bounds of |x^| and |x - x^| (FP64 sums rounded up).
__global__ void k_half_rows(const float* __restrict__ x, uint64_t rows, uint32_t d, uint32_t dp,
                            __half* __restrict__ h, float* __restrict__ nrm,
                            float* __restrict__ enrm, uint32_t* __restrict__ status) {
  const uint32_t lane = lane_id();
  const uint64_t nw = static_cast<uint64_t>(gridDim.x) * (blockDim.x >> 5);
  for (uint64_t r = blockIdx.x * static_cast<uint64_t>(blockDim.x >> 5) + (threadIdx.x >> 5);
       r < rows; r += nw) {
    double a = 0.0, e = 0.0;
    bool big = false;
    for (uint32_t i = lane; i < dp; i += 32) {
      if (i >= d) {
        h[r * dp + i] = __float2half_rn(0.0f);
        continue;
      }
      const float v = x[r * d + i];
      big |= !(fabsf(v) <= 65000.0f);  // beyond FP16 range (or NaN)
      const __half hv = __float2half_rn(v);
      h[r * dp + i] = hv;
      const double fv = static_cast<double>(__half2float(hv));
      a = fma(fv, fv, a);
      const double ev = static_cast<double>(v) - fv;
      e = fma(ev, ev, e);
    }
    for (int o = 16; o > 0; o >>= 1) {
      a += __shfl_xor_sync(kFull, a, o);
      e += __shfl_xor_sync(kFull, e, o);
    }
    if (__any_sync(kFull, big) && lane == 0) raise_error(status, kGtErrRange);
    if (lane == 0) {
      nrm[r] = __double2float_ru(sqrt(a) * (1.0 + 1e-12));
      enrm[r] = __double2float_ru(sqrt(e) * (1.0 + 1e-12));
    }
  }
}

__global__ void k_max2(const float* __restrict__ a, const float* __restrict__ b, uint64_t n,
                       uint32_t* __restrict__ out) {  // out[0] = max a, out[1] = max b (>= 0)
  float ma = 0.0f, mb = 0.0f;
  const uint64_t stride = static_cast<uint64_t>(gridDim.x) * blockDim.x;
  for (uint64_t i = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x; i < n;
       i += stride) {
    ma = fmaxf(ma, a[i]);
    mb = fmaxf(mb, b[i]);
  }
  for (int o = 16; o > 0; o >>= 1) {
    ma = fmaxf(ma, __shfl_xor_sync(kFull, ma, o));
    mb = fmaxf(mb, __shfl_xor_sync(kFull, mb, o));
  }
  if (lane_id() == 0) {  // non-negative floats order like their bit patterns
    atomicMax(out, __float_as_uint(ma));
    atomicMax(out + 1, __float_as_uint(mb));
  }
}

// Per query of the chunk: 2 E_q plus a relative slack for the FP32 arithmetic of the threshold.
// The tensor core accumulates over dp (d plus zero padding) products.
__global__ void k_gt_band(const float* __restrict__ qn, const float* __restrict__ qe,
                          const uint32_t* __restrict__ xmax, uint32_t rows, uint32_t dp,
                          float* __restrict__ band) {
  const uint32_t r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= rows) return;
  const double xn = __uint_as_float(xmax[0]), xe = __uint_as_float(xmax[1]);
  const double dd = dp + 16.0, u = 1.0 / 4194304.0;  // 2^-22
  const double g = dd * u / (1.0 - dd * u);
  const double q = qn[r], e = qe[r];
  const double E = (q + e) * xe + e * xn + g * q * xn;
  band[r] = __double2float_ru(2.0 * E * (1.0 + 1e-6) + 1e-30);
}

// ---------------------------------------------------------------- selection helpers

// Sorts buf[0 .. cnt) (desc value, asc id); returns the k-th largest value (or -inf when
// cnt < k) and keeps in buf the prefix with value >= that - band; *cnt updated.
template <int E>
__device__ float compact_sorted(uint64_t* buf, uint32_t& cnt, uint32_t k, float band) {
  const uint32_t lane = lane_id();
  uint64_t key[E];
#pragma unroll
  for (int s = 0; s < E; s++) {
    const uint32_t i = static_cast<uint32_t>(s) * 32u + lane;
    key[s] = i < cnt ? buf[i] : ~0ull;
  }
  __syncwarp();
  warp_sort_u64<E>(key);
  float theta = -INFINITY;
  if (cnt >= k) {
    const int s = static_cast<int>((k - 1) / 32);
    uint64_t kk = 0;
#pragma unroll
    for (int t = 0; t < E; t++)
      if (t == s) kk = __shfl_sync(kFull, key[t], (k - 1) & 31u);
    theta = key_value(kk);
  }
  const float lo = theta - band;
  uint32_t keep = 0;
#pragma unroll
  for (int s = 0; s < E; s++) {
    const uint32_t i = static_cast<uint32_t>(s) * 32u + lane;
    const bool ok = i < cnt && key_value(key[s]) >= lo;
    keep += __popc(__ballot_sync(kFull, ok));
    if (ok) buf[i] = key[s];
  }
  __syncwarp();
  cnt = keep;
  return theta;
}

__device__ float compact_any(uint64_t* buf, uint32_t& cnt, uint32_t k, float band) {
  if (cnt <= 128) return compact_sorted<4>(buf, cnt, k, band);
  if (cnt <= 256) return compact_sorted<8>(buf, cnt, k, band);
  if (cnt <= 512) return compact_sorted<16>(buf, cnt, k, band);
  return compact_sorted<32>(buf, cnt, k, band);
}

// The k-th smallest of key(0 .. cnt-1) (32-bit keys), by a four-pass 8-bit radix select with a
// 256-bin histogram in shared memory.  Requires cnt >= k.  One warp.
template <class Key>
__device__ uint32_t radix_kth(Key key, uint32_t cnt, uint32_t k, uint32_t* hist) {
  const uint32_t lane = lane_id();
  uint32_t prefix = 0, mask = 0, rem = k;
  for (int shift = 24; shift >= 0; shift -= 8) {
    for (uint32_t b = lane; b < 256; b += 32) hist[b] = 0;
    __syncwarp();
    for (uint32_t i = lane; i < cnt; i += 32) {
      const uint32_t vk = key(i);
      if ((vk & mask) == prefix) atomicAdd(hist + ((vk >> shift) & 255u), 1u);
    }
    __syncwarp();
    uint32_t local[8], sum = 0;
#pragma unroll
    for (int t = 0; t < 8; t++) {
      local[t] = hist[lane * 8 + t];
      sum += local[t];
    }
    uint32_t incl = sum;  // inclusive scan of the lanes' sums
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t y = __shfl_up_sync(kFull, incl, o);
      if (lane >= static_cast<uint32_t>(o)) incl += y;
    }
    const uint32_t excl = incl - sum;
    const unsigned owner = __ballot_sync(kFull, excl < rem && rem <= incl);
    const uint32_t src = static_cast<uint32_t>(__ffs(static_cast<int>(owner)) - 1);
    uint32_t bin = 0, before = 0;
    if (lane == src) {
      uint32_t c = excl;
#pragma unroll
      for (int t = 0; t < 8; t++) {
        if (c + local[t] >= rem) {
          bin = lane * 8 + t;
          before = c;
          break;
        }
        c += local[t];
      }
    }
    bin = __shfl_sync(kFull, bin, src);
    before = __shfl_sync(kFull, before, src);
    prefix |= bin << shift;
    mask |= 255u << shift;
    rem -= before;
    __syncwarp();
  }
  return prefix;
}

struct GtArgs {
  const float* base;     // n x d (FP32)
  const float* queries;  // rows x d (FP32, this chunk)
  uint32_t d, k;
  uint32_t rows;
  const uint64_t* cand;      // rows x kGtCap keys (desc_key), two halves of kGtCap / 2
  const uint32_t* cand_cnt;  // rows x 2
  const float* band;         // rows
  uint32_t* out;             // rows x k
  uint32_t* status;
};

// Exact FP64 scores of the candidates c = buf[0 .. cnt), sorted by (score desc, id asc); the
// first k ids go to out (tomb past cnt).
template <int E>
__device__ void rescore_write(const GtArgs& a, uint64_t row, const uint64_t* buf, uint32_t cnt,
                              uint32_t* ids_s) {
  const uint32_t lane = lane_id();
  const float* q = a.queries + row * a.d;
  uint64_t key[E];
  uint32_t id[E];
#pragma unroll
  for (int s = 0; s < E; s++) {
    const uint32_t i = static_cast<uint32_t>(s) * 32u + lane;
    key[s] = ~0ull;
    id[s] = kTomb;
    if (i < cnt) {
      const uint32_t x = static_cast<uint32_t>(buf[i]);
      const float* xr = a.base + static_cast<uint64_t>(x) * a.d;
      double acc = 0.0;
      for (uint32_t j = 0; j < a.d; j++)
        acc = fma(static_cast<double>(q[j]), static_cast<double>(xr[j]), acc);
      key[s] = desc_key64(acc);
      id[s] = x;
    }
  }
  warp_sort_kv<E>(key, id);
  // equal FP64 scores (duplicate vectors): ascending id inside each run
#pragma unroll
  for (int s = 0; s < E; s++) {
    const uint32_t i = static_cast<uint32_t>(s) * 32u + lane;
    if (i < cnt) ids_s[i] = id[s];
  }
  bool tie = false;
#pragma unroll
  for (int s = 0; s < E; s++) {
    const uint64_t up = __shfl_up_sync(kFull, key[s], 1);
    const uint64_t wrap = s > 0 ? __shfl_sync(kFull, key[s > 0 ? s - 1 : 0], 31) : ~0ull;
    const uint64_t prev = lane == 0 ? wrap : up;
    const uint32_t i = static_cast<uint32_t>(s) * 32u + lane;
    tie |= i > 0 && i < cnt && prev == key[s];
  }
  __syncwarp();
  if (__any_sync(kFull, tie)) {
    uint64_t* ks = const_cast<uint64_t*>(buf);  // reuse as keys
#pragma unroll
    for (int s = 0; s < E; s++) {
      const uint32_t i = static_cast<uint32_t>(s) * 32u + lane;
      if (i < cnt) ks[i] = key[s];
    }
    __syncwarp();
    if (lane == 0) {  // insertion sort by id inside runs of equal keys
      for (uint32_t i = 1; i < cnt; i++) {
        uint32_t j = i;
        while (j > 0 && ks[j - 1] == ks[j] && ids_s[j - 1] > ids_s[j]) {
          const uint32_t t = ids_s[j];
          ids_s[j] = ids_s[j - 1];
          ids_s[j - 1] = t;
          j--;
        }
      }
    }
    __syncwarp();
  }
  uint32_t* o = a.out + row * a.k;
  for (uint32_t i = lane; i < a.k; i += 32) o[i] = i < cnt ? ids_s[i] : kTomb;
  __syncwarp();
}

// One warp per query: its candidates (those with s^ >= theta - 2 E_q), then the ones with
// s^ >= t_k - 2 E_q, re-scored in FP64 and sorted.
__global__ void __launch_bounds__(kFinalWarps * 32) k_gt_final(GtArgs a) {
  __shared__ uint64_t buf_all[kFinalWarps][kGtCap];
  __shared__ uint32_t ids_all[kFinalWarps][kGtCap];
  uint64_t* buf = buf_all[threadIdx.x >> 5];
  uint32_t* ids_s = ids_all[threadIdx.x >> 5];
  const uint32_t lane = lane_id();
  const uint64_t nw = static_cast<uint64_t>(gridDim.x) * kFinalWarps;
  for (uint64_t row = blockIdx.x * static_cast<uint64_t>(kFinalWarps) + (threadIdx.x >> 5);
       row < a.rows; row += nw) {
    // the row's list is two halves of kGtCap / 2, one per half of the columns
    const uint32_t c0 = min(a.cand_cnt[2 * row], kGtCap / 2);
    const uint32_t c1 = min(a.cand_cnt[2 * row + 1], kGtCap / 2);
    const uint64_t* src = a.cand + row * kGtCap;
    for (uint32_t i = lane; i < c0; i += 32) buf[i] = src[i];
    for (uint32_t i = lane; i < c1; i += 32) buf[c0 + i] = src[kGtCap / 2 + i];
    uint32_t cnt = c0 + c1;
    __syncwarp();
    compact_any(buf, cnt, a.k, a.band[row]);  // candidates >= t_k - band, sorted
    if (cnt <= 128)
      rescore_write<4>(a, row, buf, cnt, ids_s);
    else if (cnt <= 256)
      rescore_write<8>(a, row, buf, cnt, ids_s);
    else if (cnt <= 512)
      rescore_write<16>(a, row, buf, cnt, ids_s);
    else
      rescore_write<32>(a, row, buf, cnt, ids_s);
  }
}

// One warp per query: lo = theta - 2 E_q, theta the k-th largest of the row's group maxima
// (-inf when there are fewer than k groups: every base row is then a candidate).
__global__ void __launch_bounds__(256) k_gt_theta(const float* __restrict__ maxima,
                                                  uint32_t rows, uint32_t groups, uint32_t k,
                                                  const float* __restrict__ band,
                                                  float* __restrict__ lo) {
  __shared__ uint32_t hist_all[8][256];
  uint32_t* hist = hist_all[threadIdx.x >> 5];
  const uint64_t nw = static_cast<uint64_t>(gridDim.x) * 8;
  for (uint64_t row = blockIdx.x * 8ull + (threadIdx.x >> 5); row < rows; row += nw) {
    if (groups < k) {
      if (lane_id() == 0) lo[row] = -INFINITY;
      continue;
    }
    const float* m = maxima + row * groups;
    const uint32_t kv =
        radix_kth([m](uint32_t i) { return ~order_key(m[i]); }, groups, k, hist);
    const float theta = key_value(static_cast<uint64_t>(kv) << 32);
    if (lane_id() == 0) lo[row] = theta - band[row];
  }
}

// ---------------------------------------------------------------- tcgen05 screening GEMM
//
// D (128 queries x BN base rows, FP32 in TMEM) = A (queries, FP16, K-major) . B (base rows,
// FP16, K-major)^T, K = dp in boxes of 64 elements (one 128-byte swizzled row per box row; the
// last box's columns past dp are read as zeros and its MMA K steps past dp are not issued).
// One CTA per SM, persistent over query tiles of 128 * MT rows (MT = 256 / BN M tiles sharing
// each B tile); for each query tile it sweeps every base tile in order:
//   warp 0      TMA producer: A tiles once per query tile, B boxes through a ring of stages;
//   warp 1      TMEM owner and MMA issuer (one thread): 4 MMAs (K = 16) per K box per M tile,
//               into one of two accumulator buffers per M tile;
//   warps 2..9  epilogue: warp w reads TMEM lanes 32 (w % 4) .. + 31 (one thread per query row)
//               and half of each tile's columns; each thread takes 128 scores per tile (4 chunks
//               of 32) with one TMEM wait, does the mode's work in straight-line code, then
//               releases the buffer.
// Every wait is bounded (1 s); a wait that gives up raises kErrWait, the CTA's roles stop, the
// issued MMAs are drained and the TMEM is freed before the CTA exits.
namespace tc {

using namespace tcu;

constexpr uint32_t kRows = 128;  // rows of an A tile (queries) and of a TMA box
constexpr uint32_t kChunk = 64;  // K elements per TMA box
constexpr uint32_t kBox = kRows * kChunk * 2;  // 16 KB
constexpr uint32_t kEpiWarps = 8;
constexpr uint32_t kThreads = 64 + 32 * kEpiWarps;
constexpr uint32_t kMaxKc = 8;  // dp <= 512
constexpr uint32_t kMinStages = 3, kMaxStages = 6;
constexpr uint32_t kHalfCap = kGtCap / 2;  // candidates per (query row, half of the columns)

// kind::f16 instruction descriptor: FP32 accumulator (bits 4-5 = 1), A and B FP16 (0), both
// K-major (bits 15, 16 = 0), N >> 3 at bits 17-22, M >> 4 at bits 24-28.
template <uint32_t BN>
constexpr uint32_t idesc() {
  return (1u << 4) | ((BN >> 3) << 17) | ((kRows >> 4) << 24);
}

enum Mode : int { kMax = 0, kFilter = 1, kDump = 2 };

struct Args {
  uint32_t q0;      // first row of this chunk in the query tensor map
  uint32_t nq;      // query rows of this chunk
  uint32_t n;       // base rows
  uint32_t kc;      // K boxes per row: ceil(dp / 64)
  uint32_t klast;   // MMA K steps (of 16) in the last box: 1 .. 4
  uint32_t stages;  // B ring stages
  // kMax: groups of base rows whose maxima are stored (groups per query row).  span > 0: a
  // group is `span` consecutive 32-column chunks of one thread (one half of each tile); span
  // == 0: a group is gs consecutive columns (gs < 32, for small n).
  uint32_t span, gs, groups;
  float* maxima;    // kMax: nq x groups
  const float* lo;  // kFilter: nq thresholds
  uint64_t* cand;   // kFilter: nq x kGtCap keys, two halves of kGtCap / 2
  uint32_t* cand_cnt;  // kFilter: nq x 2 (one count per half)
  float* dump;      // kDump: nq x n scores
  uint32_t* status;
};

template <uint32_t BN>
__device__ __forceinline__ void mma(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t acc) {
  mma_f16(d_tmem, a, b, idesc<BN>(), acc);
}

__device__ __forceinline__ float max32(const uint32_t* v) {  // pairwise tree, 31 FMNMX
  float m[16];
#pragma unroll
  for (int j = 0; j < 16; j++) m[j] = fmaxf(__uint_as_float(v[j]), __uint_as_float(v[j + 16]));
#pragma unroll
  for (int w = 8; w >= 1; w >>= 1)
#pragma unroll
    for (int j = 0; j < w; j++) m[j] = fmaxf(m[j], m[j + w]);
  return m[0];
}

// Bits j of the 32 columns col0 + j that are < n.
__device__ __forceinline__ uint32_t in_range(uint32_t col0, uint32_t n) {
  if (col0 + 32 <= n) return 0xFFFFFFFFu;
  return col0 >= n ? 0u : ((1u << (n - col0)) - 1u);
}

template <uint32_t BN>
size_t smem_bytes(uint32_t kc, uint32_t stages) {
  constexpr uint32_t MT = 256 / BN;
  return 1024 + static_cast<size_t>(MT) * kc * kBox + static_cast<size_t>(stages) * BN * 128 + 256;
}

template <int MODE, uint32_t BN>
__global__ void __launch_bounds__(kThreads, 1)
    k_gt_tc(const __grid_constant__ CUtensorMap ta, const __grid_constant__ CUtensorMap tb,
            const Args a) {
  constexpr uint32_t MT = 256 / BN;           // M tiles per query tile
  constexpr uint32_t kStageBytes = BN * 128;  // BN rows x 64 K x 2 bytes
  constexpr uint32_t kHalf = BN / 2;          // columns per epilogue thread per tile
  constexpr uint32_t kCpt = kHalf / 32;       // chunks per thread per tile and M tile
  static_assert(MT * kCpt == 4, "four 32-column chunks per thread per tile");
  extern __shared__ __align__(16) uint8_t smem_raw[];
  uint8_t* sm = smem_raw + ((1024u - (saddr(smem_raw) & 1023u)) & 1023u);
  uint8_t* sA = sm;                                       // MT x kc boxes
  uint8_t* sB = sA + static_cast<size_t>(MT) * a.kc * kBox;  // stages x (BN rows x 128 bytes)
  uint64_t* full = reinterpret_cast<uint64_t*>(sB + static_cast<size_t>(a.stages) * kStageBytes);
  uint64_t* empty = full + a.stages;
  uint64_t* a_full = empty + a.stages;
  uint64_t* a_empty = a_full + 1;
  uint64_t* t_full = a_empty + 1;   // [2]
  uint64_t* t_empty = t_full + 2;   // [2]
  uint64_t* drained = t_empty + 2;
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(drained + 1);
  volatile uint32_t* stop = tmem_slot + 1;

  const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31u;
  constexpr uint32_t rows_per_tile = kRows * MT;
  const uint32_t q_tiles = (a.nq + rows_per_tile - 1) / rows_per_tile;
  const uint32_t n_tiles = (a.n + BN - 1) / BN;
  constexpr uint32_t ncols = 2 * BN * MT;  // two accumulator buffers per M tile (512)

  if (threadIdx.x == 0) {
    for (uint32_t s = 0; s < a.stages; s++) {
      bar_init(full + s, 1);
      bar_init(empty + s, 1);
    }
    bar_init(a_full, 1);
    bar_init(a_empty, 1);
    for (int b = 0; b < 2; b++) {
      bar_init(t_full + b, 1);
      bar_init(t_empty + b, 32 * kEpiWarps);
    }
    bar_init(drained, 1);
    *stop = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     saddr(tmem_slot)),
                 "r"(ncols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  fence_before();
  __syncthreads();
  fence_after();
  const uint32_t tmem = *tmem_slot;

  if (warp == 0) {
    // ---- TMA producer
    if (lane == 0) {
      bool ok = true;
      uint32_t it = 0, sti = 0;
      for (uint32_t st = blockIdx.x; ok && st < q_tiles; st += gridDim.x, sti++) {
        if (!bar_wait(a_empty, (sti & 1u) ^ 1u, stop)) {
          ok = false;
          break;
        }
        bar_expect_tx(a_full, MT * a.kc * kBox);
        for (uint32_t m = 0; m < MT; m++)
          for (uint32_t c = 0; c < a.kc; c++)
            tma_load(sA + (m * a.kc + c) * kBox, &ta, c * kChunk,
                     a.q0 + st * rows_per_tile + m * kRows, a_full);
        for (uint32_t bt = 0; ok && bt < n_tiles; bt++)
          for (uint32_t c = 0; c < a.kc; c++, it++) {
            const uint32_t s = it % a.stages, ph = (it / a.stages) & 1u;
            if (!bar_wait(empty + s, ph ^ 1u, stop)) {
              ok = false;
              break;
            }
            bar_expect_tx(full + s, kStageBytes);
#pragma unroll
            for (uint32_t r = 0; r < BN / kRows; r++)
              tma_load(sB + s * kStageBytes + r * kBox, &tb, c * kChunk, bt * BN + r * kRows,
                       full + s);
          }
      }
      if (!ok) {
        raise_error(a.status, kErrWait);
        *stop = 1;
      }
      // the loads still in flight land before the CTA exits: each stage's last issued load
      for (uint32_t j = 0; j < a.stages && j < it; j++) {
        const uint32_t i = it - 1 - j;
        bar_wait(full + (i % a.stages), (i / a.stages) & 1u, nullptr);
      }
    }
  } else if (warp == 1) {
    // ---- MMA issuer
    if (lane == 0) {
      bool ok = true;
      uint32_t it = 0, t = 0, sti = 0;
      const uint32_t a0 = saddr(sA), b0 = saddr(sB);
      for (uint32_t st = blockIdx.x; ok && st < q_tiles; st += gridDim.x, sti++) {
        if (!bar_wait(a_full, sti & 1u, stop)) {
          ok = false;
          break;
        }
        fence_after();
        for (uint32_t bt = 0; ok && bt < n_tiles; bt++, t++) {
          const uint32_t buf = t & 1u, use = t >> 1;
          if (!bar_wait(t_empty + buf, (use & 1u) ^ 1u, stop)) {
            ok = false;
            break;
          }
          fence_after();
          for (uint32_t c = 0; c < a.kc; c++, it++) {
            const uint32_t s = it % a.stages, ph = (it / a.stages) & 1u;
            if (!bar_wait(full + s, ph, stop)) {
              ok = false;
              break;
            }
            fence_after();
            const uint32_t ks = c + 1 == a.kc ? a.klast : 4u;  // zero columns past dp skipped
#pragma unroll
            for (uint32_t m = 0; m < MT; m++)
#pragma unroll
              for (uint32_t k = 0; k < 4; k++)
                if (k < ks)
                  mma<BN>(tmem + (m * 2 + buf) * BN,
                          sw128_desc(a0 + (m * a.kc + c) * kBox + k * 32),
                          sw128_desc(b0 + s * kStageBytes + k * 32), (c | k) != 0);
            commit(empty + s);  // the stage is free once these MMAs have read it
          }
          if (ok) commit(t_full + buf);
        }
        if (ok) commit(a_empty);
      }
      if (!ok) {
        raise_error(a.status, kErrWait);
        *stop = 1;
      }
      commit(drained);  // arrives when every MMA issued above has completed
      bar_wait(drained, 0, nullptr);
    }
  } else {
    // ---- epilogue: one thread per (query row, half of the tile's columns)
    const uint32_t quarter = warp & 3u;
    const uint32_t half = (warp - 2) >> 2;
    const uint32_t row = quarter * 32u + lane;
    const uint32_t lane_base = (quarter * 32u) << 16;
    bool ok = true;
    uint32_t t = 0;
    const uint32_t chunks = n_tiles * kCpt;  // this thread's 32-column chunks per M tile
    for (uint32_t st = blockIdx.x; ok && st < q_tiles; st += gridDim.x) {
      uint32_t qrow[MT], cnt[MT];
      bool valid[MT];
      float lo[MT], run[MT];
#pragma unroll
      for (uint32_t m = 0; m < MT; m++) {
        qrow[m] = st * rows_per_tile + m * kRows + row;
        valid[m] = qrow[m] < a.nq;
        lo[m] = (MODE == kFilter && valid[m]) ? a.lo[qrow[m]] : INFINITY;
        run[m] = -INFINITY;
        cnt[m] = 0;
      }
      for (uint32_t bt = 0; bt < n_tiles; bt++, t++) {
        const uint32_t buf = t & 1u, use = t >> 1;
        ok = __all_sync(kFull, bar_wait(t_full + buf, use & 1u, stop));
        if (!ok) break;
        fence_after();
        uint32_t v[4][32];
#pragma unroll
        for (uint32_t i = 0; i < 4; i++) {
          const uint32_t m = i / kCpt, ch = i % kCpt;
          tmem_ld32(tmem + lane_base + (m * 2 + buf) * BN + half * kHalf + ch * 32, v[i]);
        }
        tmem_wait_ld();
        fence_before();
        bar_arrive(t_empty + buf);  // the scores are in registers: the buffer is free
#pragma unroll
        for (uint32_t i = 0; i < 4; i++) {
          const uint32_t m = i / kCpt, ch = i % kCpt;
          if (!valid[m]) continue;
          const uint32_t col0 = bt * BN + half * kHalf + ch * 32;
          const uint32_t inr = in_range(col0, a.n);
          if (MODE == kMax) {
            if (a.span) {
              float mx = max32(v[i]);
              if (inr != 0xFFFFFFFFu) {  // the last tile: only columns < n count
                mx = -INFINITY;
#pragma unroll
                for (uint32_t j = 0; j < 32; j++)
                  if ((inr >> j) & 1u) mx = fmaxf(mx, __uint_as_float(v[i][j]));
              }
              run[m] = fmaxf(run[m], mx);
              const uint32_t u = bt * kCpt + ch;  // this thread's chunk index
              if (((u + 1) & (a.span - 1)) == 0 || u + 1 == chunks) {
                a.maxima[static_cast<uint64_t>(qrow[m]) * a.groups + (u / a.span) * 2 + half] =
                    run[m];
                run[m] = -INFINITY;
              }
            } else {  // small n: groups of gs < 32 columns
#pragma unroll
              for (uint32_t j = 0; j < 32; j++) {
                const uint32_t c = col0 + j;
                if ((inr >> j) & 1u) {
                  run[m] = fmaxf(run[m], __uint_as_float(v[i][j]));
                  if (((c + 1) & (a.gs - 1)) == 0 || c + 1 == a.n) {
                    a.maxima[static_cast<uint64_t>(qrow[m]) * a.groups + c / a.gs] = run[m];
                    run[m] = -INFINITY;
                  }
                }
              }
            }
          } else if (MODE == kFilter) {
            uint32_t hit = 0;
#pragma unroll
            for (uint32_t j = 0; j < 32; j++)
              hit |= (__uint_as_float(v[i][j]) >= lo[m]) ? (1u << j) : 0u;
            hit &= inr;
            if (hit) {  // rare (about 1.1 k hits per row): a short loop over a local copy, so the
                        // unrolled common path stays small in the instruction cache
              float tmp[32];
#pragma unroll
              for (uint32_t j = 0; j < 32; j++) tmp[j] = __uint_as_float(v[i][j]);
              uint64_t* dst = a.cand + static_cast<uint64_t>(qrow[m]) * kGtCap + half * kHalfCap;
#pragma unroll 1
              while (hit) {
                const uint32_t j = static_cast<uint32_t>(__ffs(static_cast<int>(hit)) - 1);
                hit &= hit - 1u;
                if (cnt[m] < kHalfCap) dst[cnt[m]] = desc_key(tmp[j], col0 + j);
                cnt[m]++;
              }
            }
          } else {
            float* o = a.dump + static_cast<uint64_t>(qrow[m]) * a.n;
#pragma unroll
            for (uint32_t j = 0; j < 32; j++)
              if ((inr >> j) & 1u) o[col0 + j] = __uint_as_float(v[i][j]);
          }
        }
      }
      if (MODE == kFilter && ok) {
        // each half of a row keeps its candidates in its own half of the row's list
#pragma unroll
        for (uint32_t m = 0; m < MT; m++)
          if (valid[m]) {
            a.cand_cnt[static_cast<uint64_t>(qrow[m]) * 2 + half] = min(cnt[m], kHalfCap);
            if (cnt[m] > kHalfCap) raise_error(a.status, kGtErrFinal);
          }
      }
    }
    if (!ok && lane == 0) {
      raise_error(a.status, kErrWait);
      *stop = 1;
    }
  }
  fence_before();
  __syncthreads();
  if (warp == 1) {
    fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                 "r"(ncols)
                 : "memory");
  }
}

// A rows x dp FP16 matrix (row stride dp * 2 bytes, a multiple of 32) as TMA boxes of
// 64 x 128 with 128-byte swizzling; rows and columns past the end read as zeros.
bool make_map(CUtensorMap* m, const __half* p, uint64_t rows, uint32_t dp) {
  EncodeTiled enc = encoder();
  if (!enc) return false;
  const cuuint64_t dims[2] = {dp, rows};
  const cuuint64_t strides[1] = {static_cast<cuuint64_t>(dp) * 2};
  const cuuint32_t box[2] = {kChunk, kRows};
  const cuuint32_t elem[2] = {1, 1};
  return enc(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT16, 2, const_cast<__half*>(p), dims, strides, box,
             elem, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
             CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

template <uint32_t BN>
uint32_t stages_for(uint32_t kc, size_t smem_optin) {
  uint32_t s = kMaxStages;
  while (s > kMinStages && smem_bytes<BN>(kc, s) > smem_optin) s--;
  return smem_bytes<BN>(kc, s) <= smem_optin ? s : 0;
}

template <int MODE, uint32_t BN>
cudaError_t launch_bn(const CUtensorMap& ta, const CUtensorMap& tb, const Args& a, int num_sms,
                      cudaStream_t st) {
  const size_t smem = smem_bytes<BN>(a.kc, a.stages);
  auto kern = k_gt_tc<MODE, BN>;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       static_cast<int>(smem));
  if (e != cudaSuccess) return e;
  constexpr uint32_t rows_per_tile = kRows * (256 / BN);
  const uint32_t q_tiles = (a.nq + rows_per_tile - 1) / rows_per_tile;
  const uint32_t grid = q_tiles < static_cast<uint32_t>(num_sms) ? q_tiles
                                                                  : static_cast<uint32_t>(num_sms);
  kern<<<grid ? grid : 1, kThreads, smem, st>>>(ta, tb, a);
  return cudaGetLastError();
}

// The launched shape: 256 base rows per tile against one 128-row query tile (measured faster
// than 128 base rows against two query tiles: 1.12 s against 1.28 s for 1M x 1M x 200).
constexpr uint32_t kBN = 256;

template <int MODE>
cudaError_t launch(const CUtensorMap& ta, const CUtensorMap& tb, const Args& a, int num_sms,
                   cudaStream_t st) {
  return launch_bn<MODE, kBN>(ta, tb, a, num_sms, st);
}

}  // namespace tc

int blocks_for(uint64_t warps, int per_block, int num_sms, int per_sm) {
  uint64_t b = (warps + per_block - 1) / per_block;
  const uint64_t cap = static_cast<uint64_t>(num_sms) * per_sm;
  if (b > cap) b = cap;
  return static_cast<int>(b ? b : 1);
}

// FP16 rows are zero-padded to a multiple of 16 elements (one MMA K step); TMA reads the last
// 64-element box past the row end as zeros.
uint32_t padded_dim(uint32_t d) { return (d + 15) / 16 * 16; }
uint32_t k_boxes(uint32_t dp) { return (dp + tc::kChunk - 1) / tc::kChunk; }
uint32_t k_last(uint32_t dp) { return (dp - (k_boxes(dp) - 1) * tc::kChunk) / 16; }

}  // namespace

uint32_t gt_max_k() { return 256; }

uint32_t gt_max_dim() { return tc::kChunk * tc::kMaxKc; }

GtPlan gt_plan(uint64_t n, uint64_t nq, uint32_t d, int num_sms, size_t smem_optin) {
  GtPlan p{};
  p.dp = padded_dim(d);
  p.kc = k_boxes(p.dp);
  p.bn = tc::kBN;
  p.stages = tc::stages_for<tc::kBN>(p.kc, smem_optin);
  // groups of base rows for the threshold pass, about 4096 or more per query where n allows:
  // each epilogue thread's chunks (32 columns of one half of each tile), `span` at a time, or
  // for small n groups of gs < 32 columns
  const uint64_t n_tiles = (n + p.bn - 1) / p.bn;
  const uint64_t chunks = n_tiles * (p.bn / 64);  // per thread
  if (2 * chunks >= 4096) {
    p.span = 1;
    while (2 * ((chunks + 2 * p.span - 1) / (2 * p.span)) >= 4096) p.span *= 2;
    p.gs = 0;
    p.groups = static_cast<uint32_t>(2 * ((chunks + p.span - 1) / p.span));
  } else {
    p.span = 0;
    p.gs = 1;
    while (p.gs < 16 && n / (2ull * p.gs) >= 4096) p.gs *= 2;
    p.groups = static_cast<uint32_t>((n + p.gs - 1) / p.gs);
  }
  // queries per chunk: whole waves of query tiles, the chunk's maxima and candidate lists
  // within 4 GB
  const uint64_t wave = 256ull * static_cast<uint64_t>(num_sms);
  const uint64_t per_q = static_cast<uint64_t>(p.groups) * 4 + kGtCap * 8 + 16;
  uint64_t cq = (4ull << 30) / per_q / wave * wave;
  if (cq < 256) cq = 256;
  if (cq > nq) cq = nq;
  p.cq = cq;
  return p;
}

size_t gt_workspace_bytes(const GtPlan& p, uint64_t n, uint64_t nq) {
  auto al = [](uint64_t b) { return (b + 1023) & ~1023ull; };
  return al(n * p.dp * 2) + al(nq * p.dp * 2) + 2 * al(n * 4) + 2 * al(nq * 4) + al(8) +
         2 * al(p.cq * 4) + al(p.cq * p.groups * 4) + al(p.cq * kGtCap * 8) + al(p.cq * 8);
}

int ground_truth(const GtPlan& plan, const float* base, uint64_t n, uint32_t d,
                 const float* queries, uint64_t nq, uint32_t k, uint32_t* out, char* ws,
                 uint32_t* status, int num_sms, cudaStream_t st, float* diag) {
  const uint32_t dp = plan.dp;
  const uint64_t cq = plan.cq;
  auto al = [](uint64_t b) { return (b + 1023) & ~1023ull; };
  char* p = ws;
  auto take = [&](uint64_t bytes) {
    char* r = p;
    p += al(bytes);
    return r;
  };
  __half* b16 = reinterpret_cast<__half*>(take(n * dp * 2));
  __half* q16 = reinterpret_cast<__half*>(take(nq * dp * 2));
  float* bn = reinterpret_cast<float*>(take(n * 4));
  float* be = reinterpret_cast<float*>(take(n * 4));
  float* qn = reinterpret_cast<float*>(take(nq * 4));
  float* qe = reinterpret_cast<float*>(take(nq * 4));
  uint32_t* xmax = reinterpret_cast<uint32_t*>(take(8));
  float* band = reinterpret_cast<float*>(take(cq * 4));
  float* lo = reinterpret_cast<float*>(take(cq * 4));
  float* maxima = reinterpret_cast<float*>(take(cq * plan.groups * 4));
  uint64_t* cand = reinterpret_cast<uint64_t*>(take(cq * kGtCap * 8));
  uint32_t* cand_cnt = reinterpret_cast<uint32_t*>(take(cq * 8));

  cudaError_t e;
  k_half_rows<<<blocks_for(n, 8, num_sms, 8), 256, 0, st>>>(base, n, d, dp, b16, bn, be, status);
  k_half_rows<<<blocks_for(nq, 8, num_sms, 8), 256, 0, st>>>(queries, nq, d, dp, q16, qn, qe,
                                                               status);
  if ((e = cudaMemsetAsync(xmax, 0, 8, st)) != cudaSuccess) return -static_cast<int>(e);
  {
    uint64_t g = (n + 255) / 256;
    if (g > static_cast<uint64_t>(num_sms) * 4) g = static_cast<uint64_t>(num_sms) * 4;
    k_max2<<<static_cast<unsigned>(g ? g : 1), 256, 0, st>>>(bn, be, n, xmax);
  }
  if ((e = cudaGetLastError()) != cudaSuccess) return -static_cast<int>(e);
  CUtensorMap ta, tb;
  if (!tc::make_map(&ta, q16, nq, dp) || !tc::make_map(&tb, b16, n, dp)) return 1;
  for (uint64_t q0 = 0; q0 < nq; q0 += cq) {
    const uint32_t rows = static_cast<uint32_t>(min(cq, nq - q0));
    k_gt_band<<<(rows + 255) / 256, 256, 0, st>>>(qn + q0, qe + q0, xmax, rows, dp, band);
    tc::Args a{};
    a.q0 = static_cast<uint32_t>(q0);
    a.nq = rows;
    a.n = static_cast<uint32_t>(n);
    a.kc = plan.kc;
    a.klast = k_last(dp);
    a.stages = plan.stages;
    a.span = plan.span;
    a.gs = plan.gs;
    a.groups = plan.groups;
    a.maxima = maxima;
    a.lo = lo;
    a.cand = cand;
    a.cand_cnt = cand_cnt;
    a.status = status;
    if ((e = tc::launch<tc::kMax>(ta, tb, a, num_sms, st)) != cudaSuccess)
      return -static_cast<int>(e);
    k_gt_theta<<<blocks_for(rows, 8, num_sms, 8), 256, 0, st>>>(maxima, rows, plan.groups, k,
                                                                band, lo);
    if ((e = tc::launch<tc::kFilter>(ta, tb, a, num_sms, st)) != cudaSuccess)
      return -static_cast<int>(e);
    GtArgs f{};
    f.base = base;
    f.queries = queries + q0 * d;
    f.d = d;
    f.k = k;
    f.rows = rows;
    f.cand = cand;
    f.cand_cnt = cand_cnt;
    f.band = band;
    f.out = out + q0 * k;
    f.status = status;
    k_gt_final<<<blocks_for(rows, kFinalWarps, num_sms, 16), kFinalWarps * 32, 0, st>>>(f);
    if ((e = cudaGetLastError()) != cudaSuccess) return -static_cast<int>(e);
    if (diag && q0 == 0) {  // the first query's margin and the base's largest norms
      if ((e = cudaMemcpyAsync(diag, band, 4, cudaMemcpyDeviceToDevice, st)) != cudaSuccess)
        return -static_cast<int>(e);
      if ((e = cudaMemcpyAsync(diag + 1, xmax, 8, cudaMemcpyDeviceToDevice, st)) != cudaSuccess)
        return -static_cast<int>(e);
    }
  }
  return 0;
}

size_t screen_scores_workspace(uint64_t na, uint64_t nb, uint32_t d) {
  auto al = [](uint64_t b) { return (b + 1023) & ~1023ull; };
  const uint32_t dp = padded_dim(d);
  return al(na * dp * 2) + al(nb * dp * 2) + 2 * al(na * 4) + 2 * al(nb * 4);
}

int screen_scores(const float* a, uint64_t na, const float* b, uint64_t nb, uint32_t d,
                  float* out, char* ws, uint32_t* status, int num_sms, size_t smem_optin,
                  cudaStream_t st) {
  const uint32_t dp = padded_dim(d);
  auto al = [](uint64_t x) { return (x + 1023) & ~1023ull; };
  char* p = ws;
  auto take = [&](uint64_t bytes) {
    char* r = p;
    p += al(bytes);
    return r;
  };
  __half* a16 = reinterpret_cast<__half*>(take(na * dp * 2));
  __half* b16 = reinterpret_cast<__half*>(take(nb * dp * 2));
  float* an = reinterpret_cast<float*>(take(na * 4));
  float* ae = reinterpret_cast<float*>(take(na * 4));
  float* bn = reinterpret_cast<float*>(take(nb * 4));
  float* be = reinterpret_cast<float*>(take(nb * 4));
  k_half_rows<<<blocks_for(na, 8, num_sms, 8), 256, 0, st>>>(a, na, d, dp, a16, an, ae, status);
  k_half_rows<<<blocks_for(nb, 8, num_sms, 8), 256, 0, st>>>(b, nb, d, dp, b16, bn, be, status);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return -static_cast<int>(e);
  CUtensorMap ta, tb;
  if (!tc::make_map(&ta, a16, na, dp) || !tc::make_map(&tb, b16, nb, dp)) return 1;
  tc::Args x{};
  x.q0 = 0;
  x.nq = static_cast<uint32_t>(na);
  x.n = static_cast<uint32_t>(nb);
  x.kc = k_boxes(dp);
  x.klast = k_last(dp);
  x.stages = tc::stages_for<tc::kBN>(x.kc, smem_optin);
  x.span = 1;
  x.groups = 1;
  x.dump = out;
  x.status = status;
  e = tc::launch<tc::kDump>(ta, tb, x, num_sms, st);
  return e == cudaSuccess ? 0 : -static_cast<int>(e);
}

}  // namespace pg
