/*
 * ref_shim.h -- CUDA built-ins for compiling the reference's device headers with g++
 * (TEST INFRASTRUCTURE ONLY; used by oracle/ref_harness.cpp).
 *
 * The reference's thread-per-node kernels (match_top1_kernel_v0, init_pr_lists,
 * fusion_prune_reverse_kernel_v0, fusion_merge_sort_prune_kernel in include/Gbuilder.cuh) use
 * only threadIdx/blockIdx, atomicCAS and atomicAdd.  Launched with grid_size = block_size = 1
 * they run every node on one thread in ascending id order, which is the canonical resolution
 * of their races.  Under g++ the __global__/__device__ qualifiers expand to nothing
 * (crt/host_defines.h), so a kernel becomes an ordinary function that this harness calls.
 */
#pragma once
#include <cuda_runtime.h>
#include <cstdint>

#ifndef __launch_bounds__
#define __launch_bounds__(...)
#endif

/* one-thread launch: every thread/block index is zero */
static const uint3 threadIdx = {0u, 0u, 0u};
static const uint3 blockIdx = {0u, 0u, 0u};
static const dim3 blockDim(1u, 1u, 1u);
static const dim3 gridDim(1u, 1u, 1u);

/* Declarations for the warp-level kernels that the header also defines; the harness never
 * launches those, so these are only parsed. */
static inline void __syncwarp(unsigned = 0xFFFFFFFFu) {}
static inline unsigned __ballot_sync(unsigned, int pred) { return pred ? 1u : 0u; }
static inline int __popc(unsigned x) { return __builtin_popcount(x); }
static inline int __ffs(unsigned x) { return __builtin_ffs((int)x); }

static inline unsigned int atomicCAS(unsigned int* addr, unsigned int cmp, unsigned int val) {
  unsigned int old = *addr;
  if (old == cmp) *addr = val;
  return old;
}

static inline unsigned int atomicAdd(unsigned int* addr, unsigned int val) {
  unsigned int old = *addr;
  *addr = old + val;
  return old;
}

/* Single-lane warp: a shuffle returns the caller's own value. */
template <class T>
static inline T __shfl_sync(unsigned, T v, int, int = 32) {
  return v;
}
template <class T>
static inline T __shfl_xor_sync(unsigned, T v, int, int = 32) {
  return v;
}
template <class T>
static inline T __shfl_down_sync(unsigned, T v, unsigned, int = 32) {
  return v;
}
