/*
 * ref_harness.cpp -- runs the reference's own thread-per-node kernels on the CPU
 * (TEST INFRASTRUCTURE ONLY; the fixture generator tests/golden/make_golden.py is its only user).
 *
 * Built by oracle/build_ref.sh with g++ from include/Gbuilder.cuh where it lies in the reference
 * tree, with oracle/ref_shim.h supplying the CUDA built-ins.  Each exported function launches a
 * reference kernel template with grid_size = block_size = 1, i.e. all nodes on one thread in
 * ascending id order, at the compile-time sizes REF_N x REF_D:
 *   ref_match_top1      match_top1_kernel_v0        Gbuilder.cuh:104-135  (test_t2iend.cu:976)
 *   ref_prune_*         init_pr_lists + fusion_prune_reverse_kernel_v0
 *                                                   Gbuilder.cuh:1066-1244 (test_t2iend.cu:987-1001)
 *   ref_merge_*         fusion_merge_sort_prune_kernel Gbuilder.cuh:1467-1601 (test_t2iend.cu:1010)
 *   ref_hash_*          HashTable visited set        Ghashtable.cuh:13-93
 * Parameter sets: phase 1 (C=128, P=15, R=111, degree 16, non-strict, test_t2iend.cu:671-677);
 * link rounds at M=32 (C=64, P=32, R=94, degree 32, strict) and at the reference's own M=55
 * (C=64, P=55, R=71, degree 55, strict, test_t2iend.cu:703-727).
 */
#include "Gbuilder.cuh"
#include "Ghashtable.cuh"

#include <cstring>
#include <vector>

#ifndef REF_N
#define REF_N 1000
#endif
#ifndef REF_D
#define REF_D 200
#endif

using namespace Gbuilder::Gpu;

namespace {
constexpr uint32_t kN = REF_N;
constexpr uint32_t kD = REF_D;
constexpr uint32_t kTomb = 0xFFFFFFFFu;
constexpr uint32_t kGt = 128;

template <uint32_t C, uint32_t P, uint32_t R, bool strict>
void prune(const float* base, uint32_t* graph, uint32_t* lists) {
  using list_t = pr_neighbor_list<uint32_t, R, P>;
  static_assert(sizeof(list_t) == 128 * sizeof(uint32_t), "pr list is 512 B");
  init_pr_lists<1, 1, kN, kGt, P, R, kTomb, kD, true, float, uint32_t>(
      reinterpret_cast<list_t*>(lists));
  fusion_prune_reverse_kernel_v0<1, 1, kN, C, P, R, kTomb, kD, strict, float, uint32_t>(
      base, graph, reinterpret_cast<list_t*>(lists));
}

template <uint32_t P, uint32_t R, uint32_t F, bool strict>
void merge(const float* base, uint32_t* lists, uint32_t* out) {
  using list_t = pr_neighbor_list<uint32_t, R, P>;
  fusion_merge_sort_prune_kernel<1, 1, kN, P, R, F, kTomb, kD, strict, float, uint32_t>(
      base, reinterpret_cast<list_t*>(lists), out);
}
}  // namespace

extern "C" {

uint32_t ref_n(void) { return kN; }
uint32_t ref_d(void) { return kD; }

/* gt: kN x 128; out: kN x 128 (preset to tomb here, as test_t2iend.cu:866-870 does) */
void ref_match_top1(const uint32_t* gt, uint32_t* out) {
  std::vector<uint32_t> g(gt, gt + (size_t)kN * kGt);
  for (size_t i = 0; i < (size_t)kN * kGt; i++) out[i] = kTomb;
  match_top1_kernel_v0<1, 1, kN, kGt, kGt, 127, kTomb, float, uint32_t>(g.data(), out);
}

/* graph: kN x C, sorted in place; lists: kN x 128 pr_neighbor_list records */
void ref_prune_phase1(const float* base, uint32_t* graph, uint32_t* lists) {
  prune<128, 15, 111, false>(base, graph, lists);
}
void ref_merge_phase1(const float* base, uint32_t* lists, uint32_t* out) {
  merge<15, 111, 16, false>(base, lists, out);
}
void ref_prune_link32(const float* base, uint32_t* graph, uint32_t* lists) {
  prune<64, 32, 94, true>(base, graph, lists);
}
void ref_merge_link32(const float* base, uint32_t* lists, uint32_t* out) {
  merge<32, 94, 32, true>(base, lists, out);
}
void ref_prune_link55(const float* base, uint32_t* graph, uint32_t* lists) {
  prune<64, 55, 71, true>(base, graph, lists);
}
void ref_merge_link55(const float* base, uint32_t* lists, uint32_t* out) {
  merge<55, 71, 55, true>(base, lists, out);
}

/* Visited-set pin: apply warp_level_test_and_set (lane 0) to keys in order, emptying the
 * table before key i whenever reset_before[i] is non-zero.  new_flags[i] = 1 when the key was
 * inserted.  The reset writes Kempty into every slot, which is what reset_sync's 32 lanes do
 * together; reset_sync itself is not called because it is declared bool and returns nothing
 * (Ghashtable.cuh:80-86), undefined behaviour that g++ compiles into a crash. */
void ref_hash_sequence(const uint32_t* keys, const uint8_t* reset_before, uint32_t count,
                       uint8_t* new_flags) {
  static HashTable<uint32_t, 1 << 12> table;
  std::memset(table.list_, 0, sizeof(table.list_));
  for (uint32_t i = 0; i < count; i++) {
    if (reset_before[i]) std::memset(table.list_, 0, sizeof(table.list_));
    new_flags[i] = table.warp_level_test_and_set(keys[i], 0) ? 1 : 0;
  }
}
}
