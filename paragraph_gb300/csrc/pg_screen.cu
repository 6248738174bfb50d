// pg_screen.cu -- the per-point norms of the screened prune (K6/K10, pg_prune_tc.cu).
//
// The screened prune bounds the error of a 16-bit inner product from two norms per point, |x| and
// |x - x^| (x^ = the FP16 or BF16 copy of x), computed here once per build instead of per
// candidate.  |x - x^| also carries the norm of x^'s subnormal part, so that the bound holds
// whether the tensor cores flush subnormal inputs or not; values beyond FP16's range give an
// infinite |x - x^|, which sends every test involving x to the exact chain.
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

}  // namespace

bool screen_supported(uint32_t c, uint32_t d, int strict) {
  return strict && c >= 1 && c <= 128 && d >= 4 && d <= 1024 && (d % 4) == 0;
}

// Per point: upper bounds of |x| and of |x - x^| + |x^_sub| (x^ = the 16-bit copy the screened
// prune packs, x^_sub its subnormal part), read by k_prune_tc in place of per-candidate sums.
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

}  // namespace pg
