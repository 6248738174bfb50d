// pg_device.cuh -- device helpers shared by the build kernels (sm_103a).
#pragma once
#include <cfloat>
#include <cstdint>
#include <cuda_runtime.h>

namespace pg {

constexpr uint32_t kTomb = 0xFFFFFFFFu;
constexpr uint32_t kMaskedTomb = 0x7FFFFFFFu;  // a tomb after `& 0x7FFFFFFF` (Gsearcher.cuh:1063)
constexpr uint32_t kParent = 0x80000000u;      // "explored" bit (Gsearcher.cuh:30-35)
constexpr unsigned kFull = 0xFFFFFFFFu;

// Device-side error codes, written into the handle's status word with atomicOr.
enum : uint32_t {
  kErrNone = 0,
  kErrIterCap = 1u << 0,   // a search ran past max_search_iters
  kErrWait = 1u << 1,      // a bounded mbarrier wait gave up
  kErrBadId = 1u << 2,     // an input id was >= n and not tomb
  kErrCapacity = 1u << 3,  // a list exceeded the capacity a kernel was built for
};

// 32 bytes of read-only global memory in one 256-bit load (p 32-byte aligned): one L1 wavefront
// per sector where two 16-byte loads take two.
__device__ __forceinline__ void ld8(const float* p, float (&v)[8]) {
  asm("ld.global.nc.v8.f32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
      : "=f"(v[0]), "=f"(v[1]), "=f"(v[2]), "=f"(v[3]), "=f"(v[4]), "=f"(v[5]), "=f"(v[6]),
        "=f"(v[7])
      : "l"(p));
}

// Rows of at least this many floats (1 KB) are read with 256-bit loads by the exact chains of the
// plain prune and the merges when 32-byte aligned (their launchers pick the WIDE kernels): such
// rows mostly come from DRAM, where half the load requests pay (measured at 1M x 512: merges
// 251 -> 190 ms per build); the shorter rows of the L2-resident 1M x 200 workload were measured
// faster with the float4 kernels.
constexpr uint32_t kWideRowFloats = 256;

// One FMA chain over d = 0..D-1: distance_between (Gbuilder.cuh:785-797), -(sum x[d]*y[d]).
// Rows are 16-byte aligned when D % 4 == 0 (the library checks), so float4 loads keep the order;
// with WIDE, 32-byte aligned rows (D % 8 == 0 on a 32-byte aligned base) take 256-bit loads, one
// sector each, half the load requests of float4.
template <bool WIDE = false>
__device__ __forceinline__ float dist_seq(const float* __restrict__ x, const float* __restrict__ y,
                                          uint32_t d) {
  float s = 0.0f;
  if (WIDE && (d & 7u) == 0 &&
      ((reinterpret_cast<uintptr_t>(x) | reinterpret_cast<uintptr_t>(y)) & 31u) == 0) {
    const uint32_t n8 = d >> 3;
#pragma unroll 5
    for (uint32_t i = 0; i < n8; i++) {
      float u[8], v[8];
      ld8(x + 8 * i, u);
      ld8(y + 8 * i, v);
#pragma unroll
      for (int t = 0; t < 8; t++) s = fmaf(u[t], v[t], s);
    }
  } else if ((d & 3u) == 0) {
    const float4* a = reinterpret_cast<const float4*>(x);
    const float4* b = reinterpret_cast<const float4*>(y);
    const uint32_t n4 = d >> 2;
#pragma unroll 10
    for (uint32_t i = 0; i < n4; i++) {
      float4 u = __ldg(a + i);
      float4 v = __ldg(b + i);
      s = fmaf(u.x, v.x, s);
      s = fmaf(u.y, v.y, s);
      s = fmaf(u.z, v.z, s);
      s = fmaf(u.w, v.w, s);
    }
  } else {
    for (uint32_t i = 0; i < d; i++) s = fmaf(__ldg(x + i), __ldg(y + i), s);
  }
  return -s;
}

// Monotone map float -> uint32 (ascending), -0.0 folded onto +0.0 so that equal floats give
// equal keys, as the reference's float comparisons treat them.
__device__ __forceinline__ uint32_t order_key(float f) {
  uint32_t u = __float_as_uint(f + 0.0f);
  return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}

// (distance, position) -> 64-bit key: sorting these ascending is the stable sort by distance
// that bubble_sort performs (Gbuilder.cuh:890-902).
__device__ __forceinline__ uint64_t pack_key(float dist, uint32_t pos) {
  return (static_cast<uint64_t>(order_key(dist)) << 32) | pos;
}
__device__ __forceinline__ uint32_t key_pos(uint64_t k) { return static_cast<uint32_t>(k); }

// Warp bitonic sort of 32*E (key, value) pairs, ascending.  Element i lives in lane i % 32,
// register slot i / 32.  Keys must be unique for a deterministic result (pack_key makes them so).
template <int E>
__device__ __forceinline__ void warp_sort_kv(uint64_t (&key)[E], uint32_t (&val)[E]) {
  const uint32_t lane = threadIdx.x & 31u;
  constexpr uint32_t n = 32u * E;
#pragma unroll
  for (uint32_t k = 2; k <= n; k <<= 1) {
#pragma unroll
    for (uint32_t j = k >> 1; j > 0; j >>= 1) {
      if (j >= 32) {
        const uint32_t js = j >> 5;
#pragma unroll
        for (int s = 0; s < E; s++) {
          const int s2 = s ^ static_cast<int>(js);
          if (s2 > s) {
            const uint32_t i = static_cast<uint32_t>(s) * 32u + lane;
            const bool asc = (i & k) == 0;
            const bool sw = asc ? (key[s] > key[s2]) : (key[s] < key[s2]);
            if (sw) {
              uint64_t tk = key[s];
              key[s] = key[s2];
              key[s2] = tk;
              uint32_t tv = val[s];
              val[s] = val[s2];
              val[s2] = tv;
            }
          }
        }
      } else {
        const bool lower = (lane & j) == 0;
#pragma unroll
        for (int s = 0; s < E; s++) {
          const uint32_t i = static_cast<uint32_t>(s) * 32u + lane;
          const bool asc = (i & k) == 0;
          const uint64_t ok = __shfl_xor_sync(kFull, key[s], j);
          const uint32_t ov = __shfl_xor_sync(kFull, val[s], j);
          const bool keep_min = (lower == asc);
          const bool take = keep_min ? (ok < key[s]) : (ok > key[s]);
          if (take) {
            key[s] = ok;
            val[s] = ov;
          }
        }
      }
    }
  }
}

// Sort 32*E uint32 keys ascending (duplicates allowed: equal values are interchangeable).
template <int E>
__device__ __forceinline__ void warp_sort_u32(uint32_t (&key)[E]) {
  const uint32_t lane = threadIdx.x & 31u;
  constexpr uint32_t n = 32u * E;
#pragma unroll
  for (uint32_t k = 2; k <= n; k <<= 1) {
#pragma unroll
    for (uint32_t j = k >> 1; j > 0; j >>= 1) {
      if (j >= 32) {
        const uint32_t js = j >> 5;
#pragma unroll
        for (int s = 0; s < E; s++) {
          const int s2 = s ^ static_cast<int>(js);
          if (s2 > s) {
            const uint32_t i = static_cast<uint32_t>(s) * 32u + lane;
            const bool asc = (i & k) == 0;
            const uint32_t a = key[s], b = key[s2];
            key[s] = asc ? min(a, b) : max(a, b);
            key[s2] = asc ? max(a, b) : min(a, b);
          }
        }
      } else {
        const bool lower = (lane & j) == 0;
#pragma unroll
        for (int s = 0; s < E; s++) {
          const uint32_t i = static_cast<uint32_t>(s) * 32u + lane;
          const bool asc = (i & k) == 0;
          const uint32_t o = __shfl_xor_sync(kFull, key[s], j);
          key[s] = (lower == asc) ? min(key[s], o) : max(key[s], o);
        }
      }
    }
  }
}

// Sort 32*E uint64 keys ascending (same layout as warp_sort_kv).
template <int E>
__device__ __forceinline__ void warp_sort_u64(uint64_t (&key)[E]) {
  const uint32_t lane = threadIdx.x & 31u;
  constexpr uint32_t n = 32u * E;
#pragma unroll
  for (uint32_t k = 2; k <= n; k <<= 1) {
#pragma unroll
    for (uint32_t j = k >> 1; j > 0; j >>= 1) {
      if (j >= 32) {
        const uint32_t js = j >> 5;
#pragma unroll
        for (int s = 0; s < E; s++) {
          const int s2 = s ^ static_cast<int>(js);
          if (s2 > s) {
            const uint32_t i = static_cast<uint32_t>(s) * 32u + lane;
            const bool asc = (i & k) == 0;
            const uint64_t a = key[s], b = key[s2];
            const bool sw = asc ? (a > b) : (a < b);
            key[s] = sw ? b : a;
            key[s2] = sw ? a : b;
          }
        }
      } else {
        const bool lower = (lane & j) == 0;
#pragma unroll
        for (int s = 0; s < E; s++) {
          const uint32_t i = static_cast<uint32_t>(s) * 32u + lane;
          const bool asc = (i & k) == 0;
          const uint64_t o = __shfl_xor_sync(kFull, key[s], j);
          key[s] = (lower == asc) ? (o < key[s] ? o : key[s]) : (o > key[s] ? o : key[s]);
        }
      }
    }
  }
}

// Merge stages only (the input is bitonic): sorts ascending in log2(32E) steps.
template <int E>
__device__ __forceinline__ void warp_bitonic_merge_u32(uint32_t (&key)[E]) {
  const uint32_t lane = threadIdx.x & 31u;
  constexpr uint32_t n = 32u * E;
#pragma unroll
  for (uint32_t j = n >> 1; j > 0; j >>= 1) {
    if (j >= 32) {
      const uint32_t js = j >> 5;
#pragma unroll
      for (int s = 0; s < E; s++) {
        const int s2 = s ^ static_cast<int>(js);
        if (s2 > s) {
          const uint32_t a = key[s], b = key[s2];
          key[s] = min(a, b);
          key[s2] = max(a, b);
        }
      }
    } else {
      const bool lower = (lane & j) == 0;
#pragma unroll
      for (int s = 0; s < E; s++) {
        const uint32_t o = __shfl_xor_sync(kFull, key[s], j);
        key[s] = lower ? min(key[s], o) : max(key[s], o);
      }
    }
  }
}

__device__ __forceinline__ void raise_error(uint32_t* status, uint32_t code) {
  if (status) atomicOr(status, code);
}

__device__ __forceinline__ uint32_t lane_id() { return threadIdx.x & 31u; }

// Sub-index of global id x in a batched build: the last s with off[s] <= x (off has count + 1
// ascending entries, off[0] = 0).  count == 0 means a single index.
__device__ __forceinline__ uint32_t segment_of(const uint64_t* off, uint32_t count, uint64_t x) {
  if (count == 0) return 0;
  uint32_t lo = 0, hi = count - 1;
  while (lo < hi) {
    const uint32_t mid = (lo + hi + 1) >> 1;
    if (off[mid] <= x) lo = mid; else hi = mid - 1;
  }
  return lo;
}

}  // namespace pg
