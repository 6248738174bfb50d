// pg_gt.cu -- exact inner-product top-k ground truth on the GPU (sm_103a).
//
// The reference's build reads each training query's top-128 base ids from a file made outside it
// (README.md:25-31, notebooks); here they are computed on the GPU.  Result: for every query q the
// k base ids with the largest FP64 inner product q.x, ties to the lower id -- exact, whatever the
// arithmetic used to find them.
//
//   1. FP16 copies of base and queries with per-row norms |x^| and |x - x^| (k_half_rows);
//   2. screening scores s^ = q^.x^ by a cuBLAS FP16 GEMM with FP32 accumulation (tensor cores),
//      a chunk of queries against all base rows at a time;
//   3. a rigorous bound: |q.x - s^| <= E_q = (|q^| + |e_q|) max|e_x| + |e_q| max|x^|
//      + g (|q^| max|x^|), with g covering the FP32 accumulation (d' * 2^-22, four times the
//      IEEE unit roundoff, for the tensor core's accumulation);
//   4. selection (k_gt_scan, eight warps per query row, one per row segment): a candidate
//      buffer that keeps every score >= (running k-th largest) - 2 E_q, compacted by a warp
//      radix select when full; then (k_gt_final) the row's k-th largest screened score t_k
//      over the segments' lists (radix select again), and the candidates with
//      s^ >= t_k - 2 E_q, a superset of the true top-k;
//   5. exact FP64 inner products of the candidates and a sort by (score desc, id asc).
// On the benchmark's data a query keeps about 1.1 k candidates.
#include <cublas_v2.h>
#include <cuda_fp16.h>

#include <cmath>

#include "pg_device.cuh"
#include "pg_kernels.h"

namespace pg {

namespace {

constexpr uint32_t kGtCap = 1024;  // candidate buffer per warp
constexpr uint32_t kGtErrRange = 1u << 4;  // a value beyond the FP16 range
constexpr uint32_t kGtErrScan = 1u << 5;   // a row segment kept more candidates than kGtCap
constexpr uint32_t kGtErrFinal = 1u << 6;  // a row kept more candidates than kGtCap
constexpr int kScanWarps = 4;
constexpr int kFinalWarps = 2;

__device__ __forceinline__ float key_value(uint64_t key) {  // inverse of the key below
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

__global__ void k_half_rows(const float* __restrict__ x, uint64_t rows, uint32_t d,
                            __half* __restrict__ h, float* __restrict__ nrm,
                            float* __restrict__ enrm, uint32_t* __restrict__ status) {
  const uint32_t lane = lane_id();
  const uint64_t nw = static_cast<uint64_t>(gridDim.x) * (blockDim.x >> 5);
  for (uint64_t r = blockIdx.x * static_cast<uint64_t>(blockDim.x >> 5) + (threadIdx.x >> 5);
       r < rows; r += nw) {
    double a = 0.0, e = 0.0;
    bool big = false;
    for (uint32_t i = lane; i < d; i += 32) {
      const float v = x[r * d + i];
      big |= !(fabsf(v) <= 65000.0f);  // beyond FP16 range (or NaN)
      const __half hv = __float2half_rn(v);
      h[r * d + i] = hv;
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
__global__ void k_gt_band(const float* __restrict__ qn, const float* __restrict__ qe,
                          const uint32_t* __restrict__ xmax, uint32_t rows, uint32_t d,
                          float* __restrict__ band) {
  const uint32_t r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= rows) return;
  const double xn = __uint_as_float(xmax[0]), xe = __uint_as_float(xmax[1]);
  const double dd = d + 16.0, u = 1.0 / 4194304.0;  // 2^-22
  const double g = dd * u / (1.0 - dd * u);
  const double q = qn[r], e = qe[r];
  const double E = (q + e) * xe + e * xn + g * q * xn;
  band[r] = __double2float_ru(2.0 * E * (1.0 + 1e-6) + 1e-30);
}

struct GtArgs {
  const float* scores;  // rows x n
  uint64_t n;
  uint32_t rows, k, segs;
  const float* band;     // rows
  uint64_t* seg_keys;    // rows x segs x kGtCap
  uint32_t* seg_cnt;     // rows x segs
  float* seg_theta;      // rows x segs (k-th largest of the segment, or -inf)
  const float* base;     // n x d (FP32)
  const float* queries;  // rows x d (FP32, this chunk)
  uint32_t d;
  uint32_t* out;  // rows x k
  uint32_t* status;
};

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

// The k-th smallest of the keys' upper 32 bits (the k-th largest value) among buf[0 .. cnt),
// by a four-pass 8-bit radix select with a 256-bin histogram in shared memory; loops, not an
// unrolled network, so the scan kernel stays small.  Requires cnt >= k.
__device__ uint32_t radix_kth(const uint64_t* buf, uint32_t cnt, uint32_t k, uint32_t* hist) {
  const uint32_t lane = lane_id();
  uint32_t prefix = 0, mask = 0, rem = k;
  for (int shift = 24; shift >= 0; shift -= 8) {
    for (uint32_t b = lane; b < 256; b += 32) hist[b] = 0;
    __syncwarp();
    for (uint32_t i = lane; i < cnt; i += 32) {
      const uint32_t vk = static_cast<uint32_t>(buf[i] >> 32);
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

// radix_kth over the union of a row's segment lists in global memory (seg_keys / seg_cnt).
__device__ uint32_t radix_kth_segs(const uint64_t* keys, const uint32_t* cnts, uint32_t segs,
                                   uint32_t k, uint32_t* hist) {
  const uint32_t lane = lane_id();
  uint32_t prefix = 0, mask = 0, rem = k;
  for (int shift = 24; shift >= 0; shift -= 8) {
    for (uint32_t b = lane; b < 256; b += 32) hist[b] = 0;
    __syncwarp();
    for (uint32_t sg = 0; sg < segs; sg++) {
      const uint64_t* src = keys + static_cast<uint64_t>(sg) * kGtCap;
      const uint32_t c = cnts[sg];
      for (uint32_t i = lane; i < c; i += 32) {
        const uint32_t vk = static_cast<uint32_t>(src[i] >> 32);
        if ((vk & mask) == prefix) atomicAdd(hist + ((vk >> shift) & 255u), 1u);
      }
    }
    __syncwarp();
    uint32_t local[8], sum = 0;
#pragma unroll
    for (int t = 0; t < 8; t++) {
      local[t] = hist[lane * 8 + t];
      sum += local[t];
    }
    uint32_t incl = sum;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t y = __shfl_up_sync(kFull, incl, o);
      if (lane >= static_cast<uint32_t>(o)) incl += y;
    }
    const uint32_t excl = incl - sum;
    const unsigned owner = __ballot_sync(kFull, excl < rem && rem <= incl);
    const uint32_t src_lane = static_cast<uint32_t>(__ffs(static_cast<int>(owner)) - 1);
    uint32_t bin = 0, before = 0;
    if (lane == src_lane) {
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
    bin = __shfl_sync(kFull, bin, src_lane);
    before = __shfl_sync(kFull, before, src_lane);
    prefix |= bin << shift;
    mask |= 255u << shift;
    rem -= before;
    __syncwarp();
  }
  return prefix;
}

// Keeps (in place, order not kept) the entries of buf[0 .. cnt) whose value is >= the k-th
// largest value minus band; returns that k-th largest value (-inf when cnt < k).
__device__ float compact_select(uint64_t* buf, uint32_t& cnt, uint32_t k, float band,
                                uint32_t* hist) {
  const uint32_t lane = lane_id();
  if (cnt < k) return -INFINITY;
  const uint32_t kv = radix_kth(buf, cnt, k, hist);
  const float theta = key_value(static_cast<uint64_t>(kv) << 32);
  const float lo = theta - band;
  uint32_t out = 0;
  for (uint32_t i0 = 0; i0 < cnt; i0 += 32) {
    const uint32_t i = i0 + lane;
    const uint64_t key = i < cnt ? buf[i] : ~0ull;
    const bool ok = i < cnt && key_value(key) >= lo;
    const unsigned m = __ballot_sync(kFull, ok);
    __syncwarp();
    if (ok) buf[out + __popc(m & ((1u << lane) - 1u))] = key;
    out += __popc(m);
    __syncwarp();
  }
  cnt = out;
  return theta;
}

__device__ float compact_any(uint64_t* buf, uint32_t& cnt, uint32_t k, float band) {
  if (cnt <= 128) return compact_sorted<4>(buf, cnt, k, band);
  if (cnt <= 256) return compact_sorted<8>(buf, cnt, k, band);
  if (cnt <= 512) return compact_sorted<16>(buf, cnt, k, band);
  return compact_sorted<32>(buf, cnt, k, band);
}

// One warp per (query row, row segment): every screened score that may be in the top k.
__global__ void __launch_bounds__(kScanWarps * 32) k_gt_scan(GtArgs a) {
  __shared__ uint64_t buf_all[kScanWarps][kGtCap];
  __shared__ uint32_t hist_all[kScanWarps][256];
  uint64_t* buf = buf_all[threadIdx.x >> 5];
  uint32_t* hist = hist_all[threadIdx.x >> 5];
  const uint32_t lane = lane_id();
  const uint64_t nw = static_cast<uint64_t>(gridDim.x) * kScanWarps;
  // segments start on 512-value boundaries: one pass of the loop below reads 512 values per
  // warp, 16 per lane as four 16-byte loads (when rows are 16-byte aligned, n % 4 == 0)
  const uint64_t seglen = ((a.n + a.segs - 1) / a.segs + 511) & ~511ull;
  const bool vec = (a.n & 3u) == 0;
  for (uint64_t w = blockIdx.x * static_cast<uint64_t>(kScanWarps) + (threadIdx.x >> 5);
       w < static_cast<uint64_t>(a.rows) * a.segs; w += nw) {
    const uint64_t row = w / a.segs, seg = w % a.segs;
    const uint64_t x0 = min(a.n, seg * seglen), x1 = min(a.n, x0 + seglen);
    const float band = a.band[row];
    const float* srow = a.scores + row * a.n;
    uint32_t cnt = 0;
    float theta = -INFINITY;
    bool over = false;
    for (uint64_t xb = x0; xb < x1 && !over; xb += 512) {
      float v[16];
#pragma unroll
      for (int j = 0; j < 4; j++) {
        const uint64_t p = xb + 128u * j + 4u * lane;
        if (vec && p + 3 < x1) {
          const float4 f = __ldg(reinterpret_cast<const float4*>(srow + p));
          v[4 * j] = f.x;
          v[4 * j + 1] = f.y;
          v[4 * j + 2] = f.z;
          v[4 * j + 3] = f.w;
        } else {
#pragma unroll
          for (int t = 0; t < 4; t++) v[4 * j + t] = p + t < x1 ? srow[p + t] : -INFINITY;
        }
      }
      float mx = v[0];
#pragma unroll
      for (int j = 1; j < 16; j++) mx = fmaxf(mx, v[j]);
      if (!__any_sync(kFull, mx >= theta - band)) continue;  // the common case once warm
#pragma unroll
      for (int j = 0; j < 16; j++) {
        const uint64_t xi = xb + 128u * (j >> 2) + 4u * lane + (j & 3);
        bool pass = xi < x1 && v[j] >= theta - band;
        unsigned m = __ballot_sync(kFull, pass);
        if (!m) continue;
        if (cnt + __popc(m) > kGtCap) {
          theta = compact_select(buf, cnt, a.k, band, hist);
          pass = xi < x1 && v[j] >= theta - band;
          m = __ballot_sync(kFull, pass);
          if (cnt + __popc(m) > kGtCap) {
            over = true;
            break;
          }
        }
        if (pass)
          buf[cnt + __popc(m & ((1u << lane) - 1u))] = desc_key(v[j], static_cast<uint32_t>(xi));
        cnt += __popc(m);
        __syncwarp();
      }
    }
    if (over) {
      if (lane == 0) {
        raise_error(a.status, kGtErrScan);
        a.seg_cnt[w] = 0;
        a.seg_theta[w] = -INFINITY;
      }
      continue;
    }
    theta = compact_select(buf, cnt, a.k, band, hist);
    uint64_t* dst = a.seg_keys + w * kGtCap;
    for (uint32_t i = lane; i < cnt; i += 32) dst[i] = buf[i];
    if (lane == 0) {
      a.seg_cnt[w] = cnt;
      a.seg_theta[w] = theta;
    }
    __syncwarp();
  }
}

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
    uint64_t* ks = reinterpret_cast<uint64_t*>(const_cast<uint64_t*>(buf));  // reuse as keys
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

__global__ void __launch_bounds__(kFinalWarps * 32) k_gt_final(GtArgs a) {
  __shared__ uint64_t buf_all[kFinalWarps][kGtCap];
  __shared__ uint32_t ids_all[kFinalWarps][kGtCap];
  __shared__ uint32_t hist_all[kFinalWarps][256];
  uint32_t* hist = hist_all[threadIdx.x >> 5];
  uint64_t* buf = buf_all[threadIdx.x >> 5];
  uint32_t* ids_s = ids_all[threadIdx.x >> 5];
  const uint32_t lane = lane_id();
  const uint64_t nw = static_cast<uint64_t>(gridDim.x) * kFinalWarps;
  for (uint64_t row = blockIdx.x * static_cast<uint64_t>(kFinalWarps) + (threadIdx.x >> 5);
       row < a.rows; row += nw) {
    const float band = a.band[row];
    // pass 1: the row's k-th largest screened score t_k over the union of the segment lists
    // (each holds its own segment's top k)
    uint32_t total = 0;
    for (uint32_t s = 0; s < a.segs; s++) total += a.seg_cnt[row * a.segs + s];
    const float tk = total >= a.k
                         ? key_value(static_cast<uint64_t>(radix_kth_segs(
                                         a.seg_keys + row * a.segs * kGtCap,
                                         a.seg_cnt + row * a.segs, a.segs, a.k, hist))
                                     << 32)
                         : -INFINITY;
    // pass 2: every screened score >= t_k - band, from the whole segment lists
    const float lo = tk - band;
    uint32_t cnt = 0;
    bool over = false;
    for (uint32_t s = 0; s < a.segs && !over; s++) {
      const uint64_t w = row * a.segs + s;
      const uint32_t c = a.seg_cnt[w];
      const uint64_t* src = a.seg_keys + w * kGtCap;
      for (uint32_t i0 = 0; i0 < c; i0 += 32) {
        const uint32_t i = i0 + lane;
        const uint64_t key = i < c ? src[i] : ~0ull;
        const bool ok = i < c && key_value(key) >= lo;
        const unsigned m = __ballot_sync(kFull, ok);
        if (cnt + __popc(m) > kGtCap) {
          over = true;
          break;
        }
        if (ok) buf[cnt + __popc(m & ((1u << lane) - 1u))] = key;
        cnt += __popc(m);
      }
    }
    __syncwarp();
    if (over) {
      if (lane == 0) raise_error(a.status, kGtErrFinal);
      for (uint32_t i = lane; i < a.k; i += 32) a.out[row * a.k + i] = kTomb;
      continue;
    }
    compact_any(buf, cnt, a.k, band);  // candidates >= t_k - band, sorted
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

int blocks_for(uint64_t warps, int per_block, int num_sms, int per_sm) {
  uint64_t b = (warps + per_block - 1) / per_block;
  const uint64_t cap = static_cast<uint64_t>(num_sms) * per_sm;
  if (b > cap) b = cap;
  return static_cast<int>(b ? b : 1);
}

}  // namespace

uint32_t gt_max_k() { return 256; }

size_t gt_chunk_rows(uint64_t n, uint64_t nq) {
  // an 8 GB score block: 2048 query rows per chunk at n = 1M (each chunk's GEMM re-reads the
  // FP16 base, so larger chunks read it fewer times and give the GEMM a wider N)
  uint64_t cq = (8ull << 30) / (4 * n);
  if (cq < 1) cq = 1;
  if (cq > 4096) cq = 4096;
  if (cq > nq) cq = nq;
  return cq;
}

size_t gt_workspace_bytes(uint64_t n, uint64_t nq, uint32_t d, uint32_t segs) {
  const uint64_t cq = gt_chunk_rows(n, nq);
  auto al = [](uint64_t b) { return (b + 255) & ~255ull; };
  return al(n * d * 2) + al(nq * d * 2) + 2 * al(n * 4) + 2 * al(nq * 4) + al(8) + al(cq * 4) +
         al(cq * n * 4) + al(cq * segs * kGtCap * 8) + al(cq * segs * 4) + al(cq * segs * 4);
}

int ground_truth(cublasContext* blas, const float* base, uint64_t n, uint32_t d,
                 const float* queries, uint64_t nq, uint32_t k, uint32_t* out, char* ws,
                 uint32_t* status, int num_sms, cudaStream_t st, float* diag) {
  // segments per row (each keeps its own top k plus the margin in a kGtCap buffer)
  const uint32_t kSegs = 8;
  const uint64_t cq = gt_chunk_rows(n, nq);
  auto al = [](uint64_t b) { return (b + 255) & ~255ull; };
  char* p = ws;
  auto take = [&](uint64_t bytes) {
    char* r = p;
    p += al(bytes);
    return r;
  };
  __half* b16 = reinterpret_cast<__half*>(take(n * d * 2));
  __half* q16 = reinterpret_cast<__half*>(take(nq * d * 2));
  float* bn = reinterpret_cast<float*>(take(n * 4));
  float* be = reinterpret_cast<float*>(take(n * 4));
  float* qn = reinterpret_cast<float*>(take(nq * 4));
  float* qe = reinterpret_cast<float*>(take(nq * 4));
  uint32_t* xmax = reinterpret_cast<uint32_t*>(take(8));
  float* band = reinterpret_cast<float*>(take(cq * 4));
  float* scores = reinterpret_cast<float*>(take(cq * n * 4));
  uint64_t* seg_keys = reinterpret_cast<uint64_t*>(take(cq * kSegs * kGtCap * 8));
  uint32_t* seg_cnt = reinterpret_cast<uint32_t*>(take(cq * kSegs * 4));
  float* seg_theta = reinterpret_cast<float*>(take(cq * kSegs * 4));

  cudaError_t e;
  k_half_rows<<<blocks_for(n, 8, num_sms, 8), 256, 0, st>>>(base, n, d, b16, bn, be, status);
  k_half_rows<<<blocks_for(nq, 8, num_sms, 8), 256, 0, st>>>(queries, nq, d, q16, qn, qe, status);
  if ((e = cudaMemsetAsync(xmax, 0, 8, st)) != cudaSuccess) return -static_cast<int>(e);
  {
    uint64_t g = (n + 255) / 256;
    if (g > static_cast<uint64_t>(num_sms) * 4) g = static_cast<uint64_t>(num_sms) * 4;
    k_max2<<<static_cast<unsigned>(g ? g : 1), 256, 0, st>>>(bn, be, n, xmax);
  }
  if ((e = cudaGetLastError()) != cudaSuccess) return -static_cast<int>(e);
  if (cublasSetStream(blas, st) != CUBLAS_STATUS_SUCCESS) return 1;
  const float one = 1.0f, zero = 0.0f;
  for (uint64_t q0 = 0; q0 < nq; q0 += cq) {
    const uint32_t rows = static_cast<uint32_t>(min(cq, nq - q0));
    k_gt_band<<<(rows + 255) / 256, 256, 0, st>>>(qn + q0, qe + q0, xmax, rows, d, band);
    // scores (column-major n x rows) = base16^T (n x d) . q16 (d x rows)
    const cublasStatus_t bs = cublasGemmEx(
        blas, CUBLAS_OP_T, CUBLAS_OP_N, static_cast<int>(n), static_cast<int>(rows),
        static_cast<int>(d), &one, b16, CUDA_R_16F, static_cast<int>(d), q16 + q0 * d,
        CUDA_R_16F, static_cast<int>(d), &zero, scores, CUDA_R_32F, static_cast<int>(n),
        CUBLAS_COMPUTE_32F, CUBLAS_GEMM_DEFAULT);
    if (bs != CUBLAS_STATUS_SUCCESS) return 2;
    GtArgs a{};
    a.scores = scores;
    a.n = n;
    a.rows = rows;
    a.k = k;
    a.segs = kSegs;
    a.band = band;
    a.seg_keys = seg_keys;
    a.seg_cnt = seg_cnt;
    a.seg_theta = seg_theta;
    a.base = base;
    a.queries = queries + q0 * d;
    a.d = d;
    a.out = out + q0 * k;
    a.status = status;
    k_gt_scan<<<blocks_for(static_cast<uint64_t>(rows) * kSegs, kScanWarps, num_sms, 16),
                kScanWarps * 32, 0, st>>>(a);
    k_gt_final<<<blocks_for(rows, kFinalWarps, num_sms, 16), kFinalWarps * 32, 0, st>>>(a);
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

}  // namespace pg
