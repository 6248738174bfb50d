/*
 * ref_warp_emu.h -- a 32-lane warp emulator for compiling the reference's warp-synchronous
 * device code with g++ (TEST INFRASTRUCTURE ONLY; used by oracle/ref_search_harness.cpp).
 *
 * The reference's beam search (include/Gsearcher.cuh) is written for one warp per query: lanes
 * exchange values with __shfl_down_sync / __shfl_sync / __ballot_sync and meet at __syncwarp.
 * Here each lane of a warp is a fiber (a stack of its own) on one host thread.  A lane runs until
 * it reaches a warp-wide operation, deposits its operand there and yields; when all 32 lanes have
 * arrived, the operation completes for every lane at once (each sees every lane's operand, as the
 * hardware's exchange does) and the lanes resume in lane order.  Lanes that reach different kinds
 * of warp operation, or a warp operation that some lanes never reach because they exited, are
 * reported as an error instead of being guessed at.
 *
 * The context switch saves the six callee-saved registers and the stack pointer of the x86-64
 * System V ABI, so the emulator builds only for x86-64 (where the fixtures are generated).
 */
#pragma once
#if !defined(__x86_64__)
#error "ref_warp_emu.h: the fiber switch is written for x86-64"
#endif

#include <cuda_runtime.h>

#include <cstdint>
#include <cstdlib>
#include <cstring>

#ifndef __launch_bounds__
#define __launch_bounds__(...)
#endif

extern "C" void pg_emu_swap(void** save_sp, void* load_sp);

// pg_emu_swap(save, load): push the callee-saved registers, store the stack pointer in *save,
// switch to `load` and pop the registers saved there.
asm(".text\n"
    ".p2align 4\n"
    ".globl pg_emu_swap\n"
    ".hidden pg_emu_swap\n"
    ".type pg_emu_swap,@function\n"
    "pg_emu_swap:\n"
    "  pushq %rbp\n"
    "  pushq %rbx\n"
    "  pushq %r12\n"
    "  pushq %r13\n"
    "  pushq %r14\n"
    "  pushq %r15\n"
    "  movq %rsp, (%rdi)\n"
    "  movq %rsi, %rsp\n"
    "  popq %r15\n"
    "  popq %r14\n"
    "  popq %r13\n"
    "  popq %r12\n"
    "  popq %rbx\n"
    "  popq %rbp\n"
    "  ret\n"
    ".size pg_emu_swap, .-pg_emu_swap\n");

namespace emu {

constexpr int kLanes = 32;
constexpr size_t kStackBytes = 256 * 1024;

enum Op : int { kNoOp = 0, kSync, kShfl, kShflDown, kShflXor, kBallot };
enum State : int { kRunnable = 0, kWaiting, kDone };

struct Lane {
  void* sp = nullptr;
  State state = kDone;
  Op op = kNoOp;
  uint64_t val = 0;
  int arg = 0;
  uint64_t res = 0;
};

struct Warp {
  Lane lane[kLanes];
  void* sched_sp = nullptr;
  int cur = -1;  // lane running now; -1 outside an emulated warp
  uint32_t block = 0;
  void (*body)(void*) = nullptr;
  void* ctx = nullptr;
  char* stacks = nullptr;
};

inline Warp& warp() {
  static Warp w;
  return w;
}

inline int lane() { return warp().cur; }

[[noreturn]] inline void fiber_entry() {
  Warp& w = warp();
  const int l = w.cur;
  w.body(w.ctx);
  w.lane[l].state = kDone;
  pg_emu_swap(&w.lane[l].sp, w.sched_sp);
  std::abort();  // a finished lane is never resumed
}

// A warp-wide operation of the calling lane: returns what the hardware exchange gives it.
inline uint64_t warp_op(Op op, uint64_t val, int arg) {
  Warp& w = warp();
  const int l = w.cur;
  if (l < 0) {  // outside an emulated warp (host code of the harness): a lone lane
    if (op == kBallot) return val ? 1u : 0u;
    return val;
  }
  Lane& me = w.lane[l];
  me.op = op;
  me.val = val;
  me.arg = arg;
  me.state = kWaiting;
  pg_emu_swap(&me.sp, w.sched_sp);
  return me.res;
}

inline void complete(Op op) {
  Warp& w = warp();
  uint64_t ballot = 0;
  for (int l = 0; l < kLanes; l++)
    if (w.lane[l].val != 0) ballot |= 1ull << l;
  for (int l = 0; l < kLanes; l++) {
    Lane& me = w.lane[l];
    switch (op) {
      case kShfl:
        me.res = w.lane[me.arg & (kLanes - 1)].val;
        break;
      case kShflDown: {
        const int src = l + me.arg;
        me.res = src < kLanes ? w.lane[src].val : me.val;
        break;
      }
      case kShflXor:
        me.res = w.lane[l ^ (me.arg & (kLanes - 1))].val;
        break;
      case kBallot:
        me.res = ballot;
        break;
      default:
        me.res = 0;
        break;
    }
  }
}

// Runs `body(ctx)` on the 32 lanes of block `block` (blockDim.x = 32).  Returns nullptr, or the
// reason the warp could not be emulated.
inline const char* run_block(uint32_t block, void (*body)(void*), void* ctx) {
  Warp& w = warp();
  if (!w.stacks) {
    w.stacks = static_cast<char*>(std::aligned_alloc(64, kLanes * kStackBytes));
    if (!w.stacks) return "cannot allocate lane stacks";
  }
  w.block = block;
  w.body = body;
  w.ctx = ctx;
  for (int l = 0; l < kLanes; l++) {
    const uintptr_t top =
        reinterpret_cast<uintptr_t>(w.stacks + (l + 1) * kStackBytes) & ~uintptr_t(15);
    void** sp = reinterpret_cast<void**>(top);
    *--sp = nullptr;  // after the `ret` into fiber_entry the stack pointer is 8 mod 16
    *--sp = reinterpret_cast<void*>(&fiber_entry);
    for (int r = 0; r < 6; r++) *--sp = nullptr;  // rbp rbx r12 r13 r14 r15
    w.lane[l].sp = sp;
    w.lane[l].state = kRunnable;
    w.lane[l].op = kNoOp;
  }
  for (;;) {
    for (int l = 0; l < kLanes; l++) {
      if (w.lane[l].state != kRunnable) continue;
      w.cur = l;
      pg_emu_swap(&w.sched_sp, w.lane[l].sp);
      w.cur = -1;
    }
    int done = 0;
    for (int l = 0; l < kLanes; l++) done += w.lane[l].state == kDone ? 1 : 0;
    if (done == kLanes) return nullptr;
    if (done != 0) return "a warp operation was reached by some lanes after others exited";
    const Op op = w.lane[0].op;
    for (int l = 1; l < kLanes; l++)
      if (w.lane[l].op != op) return "lanes reached different warp operations";
    complete(op);
    for (int l = 0; l < kLanes; l++) w.lane[l].state = kRunnable;
  }
}

template <class T>
inline uint64_t bits(T v) {
  static_assert(sizeof(T) <= 8, "operand wider than 64 bits");
  uint64_t u = 0;
  std::memcpy(&u, &v, sizeof(T));
  return u;
}
template <class T>
inline T unbits(uint64_t u) {
  T v;
  std::memcpy(&v, &u, sizeof(T));
  return v;
}

inline uint3 thread_idx() { return make_uint3(static_cast<unsigned>(lane() < 0 ? 0 : lane()), 0, 0); }
inline uint3 block_idx() { return make_uint3(warp().block, 0, 0); }
inline uint3 block_dim() { return make_uint3(kLanes, 1, 1); }

}  // namespace emu

#define threadIdx (::emu::thread_idx())
#define blockIdx (::emu::block_idx())
#define blockDim (::emu::block_dim())

inline void __syncwarp(unsigned = 0xFFFFFFFFu) { emu::warp_op(emu::kSync, 0, 0); }
inline unsigned __ballot_sync(unsigned, int pred) {
  return static_cast<unsigned>(emu::warp_op(emu::kBallot, pred ? 1u : 0u, 0));
}
template <class T>
inline T __shfl_sync(unsigned, T v, int src, int = 32) {
  return emu::unbits<T>(emu::warp_op(emu::kShfl, emu::bits(v), src));
}
template <class T>
inline T __shfl_down_sync(unsigned, T v, unsigned delta, int = 32) {
  return emu::unbits<T>(emu::warp_op(emu::kShflDown, emu::bits(v), static_cast<int>(delta)));
}
template <class T>
inline T __shfl_xor_sync(unsigned, T v, int lane_mask, int = 32) {
  return emu::unbits<T>(emu::warp_op(emu::kShflXor, emu::bits(v), lane_mask));
}
inline int __popc(unsigned x) { return __builtin_popcount(x); }
inline int __ffs(int x) { return __builtin_ffs(x); }

// The lanes of one warp run one at a time, so the atomics are plain read-modify-writes.
inline unsigned int atomicCAS(unsigned int* addr, unsigned int cmp, unsigned int val) {
  const unsigned int old = *addr;
  if (old == cmp) *addr = val;
  return old;
}
inline unsigned int atomicAdd(unsigned int* addr, unsigned int val) {
  const unsigned int old = *addr;
  *addr = old + val;
  return old;
}
