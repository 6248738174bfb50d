// pg_noalloc.cu -- prune + reverse edges with no device allocation at all.
//
// Some callers cannot call cudaMalloc: a host application that owns the whole GPU through its
// own memory pool and forbids plugins from allocating behind its back, or a latency-bound caller
// that cannot afford cudaMalloc/cudaFree, which may synchronise the whole device, in the middle
// of its work.  pg_prune_reverse_noalloc serves them.  It computes exactly what
// pg_prune_reverse computes, but the reverse-edge workspace (in-degree counts, CSR offsets and
// cursors, the edge list) and the evaluation/status counters live in g_noalloc_scratch below, a
// fixed array in the library's own device image that every GPU loading the library holds until
// the process exits.  The caller still owns every input and output buffer.
//
// Limits: n <= kNoAllocMaxNodes and n * pruned <= kNoAllocMaxEdges (about 4.6 MB in total).
// Larger calls are rejected with PG_EINVAL before anything is launched.
// Every call shares the one array, which keeps the previous call's contents: each call clears
// the parts that must start at zero.  Calls whose work overlaps on the GPU (different streams or
// threads at the same time) race on the array and must be serialised by the caller.
// The first call on a device -- and the first after the device's context was reset -- looks up
// the array's device address there (see scratch_ptr); that first call should come before any
// stream capture on the device.  `stream` must belong to the current device.
#include <cuda.h>

#include <cstring>
#include <mutex>

#include "../../include/paragraph_gb300.h"
#include "pg_kernels.h"

namespace {

constexpr uint64_t kNoAllocMaxNodes = 32768;
constexpr uint64_t kNoAllocMaxEdges = kNoAllocMaxNodes * 32;
constexpr uint64_t kTiles = (kNoAllocMaxNodes + pg::kScanTileElems - 1) / pg::kScanTileElems + 1;
constexpr uint64_t align64(uint64_t w) { return (w + 63) / 64 * 64; }
// word offsets inside the array (64-word = 256-byte aligned regions)
constexpr uint64_t kWCounters = 0;  // [0..1] evals (u64), [2] status
constexpr uint64_t kWIndeg = 64;
constexpr uint64_t kWOffs = kWIndeg + align64(kNoAllocMaxNodes);
constexpr uint64_t kWTiles = kWOffs + align64(kNoAllocMaxNodes + 1);
constexpr uint64_t kWCursor = kWTiles + align64(kTiles);
constexpr uint64_t kWEdges = kWCursor + align64(kNoAllocMaxNodes);
constexpr uint64_t kWords = kWEdges + align64(kNoAllocMaxEdges);

// errors are reported through pg_last_error(), like every other entry point
int fail_na(int code, const char* msg) { return pg::set_last_error(code, msg); }

}  // namespace

// The workspace.  In host code this name is only a host-side stand-in for the symbol; kernels
// get the device address that scratch_ptr obtains from cudaGetSymbolAddress.
static __device__ __align__(256) uint32_t g_noalloc_scratch[kWords];

namespace {

constexpr int kMaxDevices = 64;
std::mutex g_ptr_mu;
uint32_t* g_ptr[kMaxDevices] = {};
unsigned long long g_ctx_id[kMaxDevices] = {};  // context the cached address belongs to

using CtxGetCurrentFn = CUresult (*)(CUcontext*);
using CtxGetIdFn = CUresult (*)(CUcontext, unsigned long long*);

// Unique id of the current device's context (cuCtxGetId, reached through the runtime's driver
// entry points, so the library needs no link to the driver library).  A reset device gets a new
// context and so a new id.  Called with g_ptr_mu held.
cudaError_t current_ctx_id(unsigned long long* id) {
  static CtxGetCurrentFn get_current = nullptr;
  static CtxGetIdFn get_id = nullptr;
  if (!get_current || !get_id) {
    void* f1 = nullptr;
    void* f2 = nullptr;
    cudaDriverEntryPointQueryResult q1, q2;
    cudaError_t e = cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f1, 12000,
                                                     cudaEnableDefault, &q1);
    if (e != cudaSuccess) return e;
    e = cudaGetDriverEntryPointByVersion("cuCtxGetId", &f2, 12000, cudaEnableDefault, &q2);
    if (e != cudaSuccess) return e;
    if (q1 != cudaDriverEntryPointSuccess || q2 != cudaDriverEntryPointSuccess || !f1 || !f2)
      return cudaErrorSymbolNotFound;
    get_current = reinterpret_cast<CtxGetCurrentFn>(f1);
    get_id = reinterpret_cast<CtxGetIdFn>(f2);
  }
  CUcontext ctx = nullptr;
  if (get_current(&ctx) != CUDA_SUCCESS || !ctx) return cudaErrorDeviceUninitialized;
  if (get_id(ctx, id) != CUDA_SUCCESS) return cudaErrorDeviceUninitialized;
  return cudaSuccess;
}

// Device address of g_noalloc_scratch on the current device.  The lookup runs once per device
// and again whenever the device's context has changed (a cudaDeviceReset reloads the module, and
// the array may then sit at another address).
cudaError_t scratch_ptr(uint32_t** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
  e = cudaSetDevice(dev);  // makes the device's primary context current (initialising it)
  if (e != cudaSuccess) return e;
  std::lock_guard<std::mutex> lk(g_ptr_mu);  // guards the cache and the entry-point lookup
  unsigned long long ctx = 0;
  e = current_ctx_id(&ctx);
  if (e != cudaSuccess) return e;
  if (!g_ptr[dev] || g_ctx_id[dev] != ctx) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return e;
    g_ptr[dev] = static_cast<uint32_t*>(p);
    g_ctx_id[dev] = ctx;
  }
  *out = g_ptr[dev];
  return cudaSuccess;
}

}  // namespace

extern "C" int pg_prune_reverse_noalloc(void* stream, const float* d_base, uint64_t n, uint32_t d,
                                        const uint32_t* d_graph, uint32_t c, uint32_t pruned,
                                        uint32_t reverse, int strict, uint32_t* d_pruned,
                                        uint32_t* d_pruned_num, uint32_t* d_reverse,
                                        uint32_t* d_reverse_num, uint64_t* evals) {
  if (!d_base || !d_graph || !d_pruned || !d_pruned_num || !d_reverse || !d_reverse_num)
    return fail_na(PG_EINVAL, "NULL argument");
  if (n == 0 || d == 0) return fail_na(PG_EINVAL, "n and d must be positive");
  if (n > kNoAllocMaxNodes)
    return fail_na(PG_EINVAL, "n exceeds the no-allocation limit of 32768 nodes");
  if (c < 1 || c > 128) return fail_na(PG_EINVAL, "c must be in [1, 128]");
  if (pruned < 2 || pruned > c) return fail_na(PG_EINVAL, "pruned must be in [2, c]");
  if (n * pruned > kNoAllocMaxEdges)
    return fail_na(PG_EINVAL, "n * pruned exceeds the no-allocation limit of 1048576 edges");
  if (reverse > 128) return fail_na(PG_EINVAL, "reverse must be <= 128");
  if (d % 4 != 0 || (reinterpret_cast<uintptr_t>(d_base) & 15u) != 0)
    return fail_na(PG_EUNSUPPORTED, "rows must be 16-byte aligned multiples of 4 floats");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  uint32_t* w = nullptr;
  cudaError_t e = scratch_ptr(&w);
  if (e != cudaSuccess) return fail_na(PG_ECUDA, cudaGetErrorString(e));
  int dev = 0, sdev = 0, sms = 0;
  if ((e = cudaGetDevice(&dev)) != cudaSuccess ||
      (e = cudaStreamGetDevice(s, &sdev)) != cudaSuccess ||
      (e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess)
    return fail_na(PG_ECUDA, cudaGetErrorString(e));
  if (sdev != dev)
    return fail_na(PG_EINVAL, "stream belongs to another device than the current one");
  unsigned long long* d_evals = reinterpret_cast<unsigned long long*>(w + kWCounters);
  uint32_t* d_status = w + kWCounters + 2;
  uint32_t* indeg = w + kWIndeg;
  // what must start at zero: the counters and the in-degree counts (the cursors are cleared by
  // launch_reverse_csr itself; offsets, tile sums and edges are fully rewritten)
  if ((e = cudaMemsetAsync(w + kWCounters, 0, 64 * sizeof(uint32_t), s)) != cudaSuccess ||
      (e = cudaMemsetAsync(indeg, 0, n * sizeof(uint32_t), s)) != cudaSuccess)
    return fail_na(PG_ECUDA, cudaGetErrorString(e));
  pg::PruneArgs a{};
  a.base = d_base;
  a.n = n;
  a.d = d;
  a.graph = d_graph;
  a.c = c;
  a.p = pruned;
  a.strict = strict;
  a.pruned = d_pruned;
  a.pruned_num = d_pruned_num;
  a.indeg = indeg;
  a.sorted = nullptr;
  a.evals = d_evals;
  a.status = d_status;
  if ((e = pg::launch_prune_reverse(a, false, sms, s)) != cudaSuccess ||
      (e = pg::launch_reverse_csr(d_pruned, d_pruned_num, pruned, n, indeg, w + kWOffs,
                                  w + kWTiles, w + kWCursor, w + kWEdges, sms, s)) != cudaSuccess ||
      (e = pg::launch_reverse_lists(w + kWOffs, w + kWEdges, n, reverse, d_reverse, d_reverse_num,
                                    sms, s)) != cudaSuccess)
    return fail_na(PG_ECUDA, cudaGetErrorString(e));
  uint32_t host[4] = {0, 0, 0, 0};  // evals (2 words) + status, read back after the stream drains
  if ((e = cudaMemcpyAsync(host, w + kWCounters, sizeof(host), cudaMemcpyDeviceToHost, s)) !=
          cudaSuccess ||
      (e = cudaStreamSynchronize(s)) != cudaSuccess)
    return fail_na(PG_ECUDA, cudaGetErrorString(e));
  uint64_t ev = 0;
  std::memcpy(&ev, host, sizeof(ev));
  if (evals) *evals = ev;
  return pg::status_error(host[2]);
}
