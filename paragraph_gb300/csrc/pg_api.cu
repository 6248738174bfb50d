// pg_api.cu -- C ABI (include/paragraph_gb300.h): handle, device workspace, the K0..K11
// pipeline of tests/test_t2iend.cu:974-1139 on one stream, stage entry points, file formats.
#include <algorithm>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <numeric>
#include <string>
#include <vector>


#include "../../include/paragraph_gb300.h"
#include "pg_kernels.h"

namespace {

thread_local std::string g_err;

int fail(int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_err = buf;
  return code;
}

#define PG_CUDA(call)                                                                    \
  do {                                                                                   \
    cudaError_t e_ = (call);                                                             \
    if (e_ != cudaSuccess)                                                               \
      return fail(PG_ECUDA, "%s failed: %s (%s:%d)", #call, cudaGetErrorString(e_), __FILE__, \
                  __LINE__);                                                             \
  } while (0)

constexpr int kMaxRounds = 4;
constexpr uint32_t kTomb = 0xFFFFFFFFu;

// counters block (device): evals and iterations per stage
enum Counter {
  C_PROJ_PRUNE = 0,
  C_PROJ_MERGE = 1,
  C_SEARCH = 2,   // + round
  C_PRUNE = 6,    // + round
  C_MERGE = 10,   // + round
  C_ITERS = 14,   // + round
  C_RESCORED = 18,  // + round
  C_COUNT = 22
};

struct Workspace {
  uint32_t* winner = nullptr;
  uint32_t* pruned = nullptr;
  uint32_t* pruned_num = nullptr;
  uint32_t* indeg = nullptr;
  uint32_t* offs = nullptr;
  uint32_t* tile_sums = nullptr;
  uint32_t* cursor = nullptr;
  uint32_t* edges = nullptr;
  uint32_t* rev = nullptr;
  uint32_t* rev_num = nullptr;
  uint32_t* sres = nullptr;
  uint32_t* proj = nullptr;
  uint32_t* graph = nullptr;
};

size_t align_up(size_t x, size_t a = 256) { return (x + a - 1) / a * a; }

struct Layout {
  size_t winner, pruned, pruned_num, indeg, offs, tile_sums, cursor, edges, rev, rev_num, sres,
      proj, graph, segs, norms, seeds, total;
};

Layout make_layout(uint64_t n, uint32_t pmax, uint32_t rmax, uint32_t L, uint32_t proj_deg,
                   uint32_t degree, uint32_t seg_count = 0) {
  Layout l{};
  size_t o = 0;
  auto take = [&](size_t bytes) {
    size_t at = o;
    o += align_up(bytes);
    return at;
  };
  l.winner = take(n * 4);
  l.pruned = take(n * pmax * 4);
  l.pruned_num = take(n * 4);
  l.indeg = take(n * 4);
  l.offs = take((n + 1) * 4);
  l.tile_sums = take(((n + pg::kScanTileElems - 1) / pg::kScanTileElems + 1) * 4);
  l.cursor = take(n * 4);
  l.edges = take(n * pmax * 4);
  l.rev = take(n * rmax * 4);
  l.rev_num = take(n * 4);
  l.sres = take(n * L * 4);
  l.proj = take(n * proj_deg * 4);
  l.graph = take(n * degree * 4);
  l.segs = take(2 * (static_cast<size_t>(seg_count) + 1) * 8);
  l.norms = take(n * 8);  // screened prune: per-point norm bounds
  l.seeds = take(n * 32 * 4);  // link-round searches: every query's 32 seed distances
  l.total = o;
  return l;
}

// What a captured build depends on: replaying it is valid only for the same parameters, buffers
// and sub-index table.
struct GraphKey {
  pg_params p{};
  const void* ptrs[5] = {};
  uint64_t n = 0, q = 0;
  uint32_t d = 0;
  std::vector<uint64_t> segs;
  bool operator==(const GraphKey& o) const {
    return std::memcmp(&p, &o.p, sizeof(p)) == 0 && std::memcmp(ptrs, o.ptrs, sizeof(ptrs)) == 0 &&
           n == o.n && q == o.q && d == o.d && segs == o.segs;
  }
};

}  // namespace

int pg::set_last_error(int code, const char* msg) { return fail(code, "%s", msg); }

struct pg_handle_s {
  int device = 0;
  cudaStream_t stream = nullptr;
  int num_sms = 0;
  size_t smem_optin = 0;
  char* ws = nullptr;
  size_t ws_bytes = 0;
  char* inbuf = nullptr;  // device copies of host inputs (pg_build_host)
  size_t in_bytes = 0;
  uint32_t* d_status = nullptr;
  unsigned long long* d_counters = nullptr;
  uint32_t* d_work = nullptr;
  uint32_t* h_status = nullptr;  // pinned
  unsigned long long* h_counters = nullptr;
  cudaEvent_t ev[16] = {};
  uint64_t* h_segs = nullptr;  // pinned copy of a batched build's sub-index table
  size_t segs_cap = 0;
  cudaGraphExec_t gexec = nullptr;  // captured build (PG_FLAG_CUDA_GRAPH) and what it was built for
  GraphKey gkey;
  pg_tuning tune{};  // launch shapes of later builds (zero = defaults)
  char* ws2 = nullptr;  // pg_build_index: graphs that outlive one stage (projection, link, rounds)
  size_t ws2_bytes = 0;
  cudaStream_t copy_stream = nullptr;  // pg_build_host: second host->device copy beside `stream`
  cudaEvent_t copy_done = nullptr;
  cudaEvent_t host_ev[4] = {};  // pg_build_host: H2D start/end, D2H start/end (made once)
  std::mutex mu;
};

namespace {

int ensure_ws(pg_handle h, size_t bytes) {
  if (bytes <= h->ws_bytes) return PG_OK;
  if (h->gexec) {  // a captured build refers to the old workspace
    cudaGraphExecDestroy(h->gexec);
    h->gexec = nullptr;
  }
  if (h->ws) cudaFree(h->ws);
  h->ws = nullptr;
  h->ws_bytes = 0;
  cudaError_t e = cudaMalloc(&h->ws, bytes);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return fail(PG_ENOMEM, "cudaMalloc of %zu workspace bytes failed: %s", bytes,
                cudaGetErrorString(e));
  }
  h->ws_bytes = bytes;
  return PG_OK;
}

int ensure_segs(pg_handle h, size_t words) {
  if (words <= h->segs_cap) return PG_OK;
  if (h->h_segs) cudaFreeHost(h->h_segs);
  h->h_segs = nullptr;
  h->segs_cap = 0;
  cudaError_t e = cudaMallocHost(&h->h_segs, words * 8);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return fail(PG_ENOMEM, "pinned allocation of the sub-index table failed");
  }
  h->segs_cap = words;
  return PG_OK;
}

int ensure_in(pg_handle h, size_t bytes) {
  if (bytes <= h->in_bytes) return PG_OK;
  if (h->inbuf) cudaFree(h->inbuf);
  h->inbuf = nullptr;
  h->in_bytes = 0;
  cudaError_t e = cudaMalloc(&h->inbuf, bytes);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return fail(PG_ENOMEM, "cudaMalloc of %zu input bytes failed: %s", bytes,
                cudaGetErrorString(e));
  }
  h->in_bytes = bytes;
  return PG_OK;
}

uint32_t pow2_at_least(uint32_t x) {
  uint32_t p = 1;
  while (p < x) p <<= 1;
  return p;
}

// Visited-set capacity: at most km + reset_iter * kp*kd ids live between rebuilds; twice that
// (a power of two) keeps the open-addressing table at most half full, so the set stays exact.
uint32_t hash_slots_for(uint32_t km, uint32_t reset_iter, uint32_t batch) {
  return pow2_at_least(2 * (km + reset_iter * batch));
}

int check_params(const pg_params* p, uint64_t n, uint32_t d, uint64_t q) {
  if (!p) return fail(PG_EINVAL, "params is NULL");
  if (n == 0 || n >= 0x7FFFFFFFull) return fail(PG_EINVAL, "n=%llu must be in [1, 2^31-1)", (unsigned long long)n);
  if (q == 0 || q >= 0x7FFFFFFFull) return fail(PG_EINVAL, "q=%llu must be in [1, 2^31-1)", (unsigned long long)q);
  if (d == 0) return fail(PG_EINVAL, "d must be positive");
  if (d % 4 != 0) return fail(PG_EUNSUPPORTED, "d=%u: rows must be a multiple of 4 floats", d);
  if (p->gt_k < 3 || p->gt_k > 128) return fail(PG_EINVAL, "gt_k=%u must be in [3, 128]", p->gt_k);
  if (p->proj_pruned < 2 || p->proj_pruned > p->gt_k)
    return fail(PG_EINVAL, "proj_pruned=%u must be in [2, gt_k]", p->proj_pruned);
  if (p->proj_pruned + p->proj_reverse > 128)
    return fail(PG_EINVAL, "proj_pruned + proj_reverse must be <= 128");
  if (p->proj_degree < 2) return fail(PG_EINVAL, "proj_degree must be >= 2");
  if (p->link_rounds > kMaxRounds) return fail(PG_EINVAL, "link_rounds must be <= %d", kMaxRounds);
  const uint32_t L = p->km + p->kp * p->kd;
  if (p->degree < 2 || p->degree > L) return fail(PG_EINVAL, "degree=%u must be in [2, L=%u]", p->degree, L);
  if (p->degree + p->link_reverse > 128) return fail(PG_EINVAL, "degree + link_reverse must be <= 128");
  if (p->reset_iter < 1) return fail(PG_EINVAL, "reset_iter must be positive");
  if (p->link_rounds > 0) {
    if (!pg::search_supported(d, p->km, p->kp, p->kd))
      return fail(PG_EUNSUPPORTED,
                  "search supports kp*kd == 32, km in {32,64,96}, d <= 512 and d %% 4 == 0 "
                  "(got km=%u kp=%u kd=%u d=%u)", p->km, p->kp, p->kd, d);
    if (p->kd > p->proj_degree || p->kd > p->degree)
      return fail(PG_EINVAL, "kd=%u exceeds a graph degree", p->kd);
  }
  if (p->screen != PG_SCREEN_NONE && p->screen != PG_SCREEN_BF16 && p->screen != PG_SCREEN_FP16)
    return fail(PG_EUNSUPPORTED,
                "screen=%u: PG_SCREEN_NONE, PG_SCREEN_BF16 and PG_SCREEN_FP16 are built",
                p->screen);
  return PG_OK;
}

bool aligned16(const void* p) { return (reinterpret_cast<uintptr_t>(p) & 15u) == 0; }

// The device address of host memory p (bytes long) when it is pinned memory that the device can
// address and the copy kernel can move (16-byte aligned, a multiple of 16 bytes); else nullptr.
// cudaHostGetDevicePointer fails, without a sticky error, for memory that CUDA did not pin.
const void* mapped_host(const void* p, size_t bytes) {
  if (!p || !aligned16(p) || (bytes % 16) != 0) return nullptr;
  void* dptr = nullptr;
  if (cudaHostGetDevicePointer(&dptr, const_cast<void*>(p), 0) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  return aligned16(dptr) ? dptr : nullptr;
}
void* mapped_host(void* p, size_t bytes) {
  return const_cast<void*>(mapped_host(static_cast<const void*>(p), bytes));
}

int status_to_error(uint32_t s) {
  if (s & 4u) return fail(PG_EINVAL, "input holds an id >= n that is not tomb (status 0x%x)", s);
  if (s & 1u) return fail(PG_ETIMEOUT, "a search exceeded max_search_iters (status 0x%x)", s);
  if (s & 2u) return fail(PG_ETIMEOUT, "a bounded device wait gave up (status 0x%x)", s);
  if (s & 8u) return fail(PG_EUNSUPPORTED, "a list exceeded the capacity of a kernel (status 0x%x)", s);
  if (s) return fail(PG_ECUDA, "device status 0x%x", s);
  return PG_OK;
}

}  // namespace

int pg::status_error(uint32_t status) { return status_to_error(status); }

namespace {

// seg_off / qseg_off (host arrays, seg_count + 1 entries each): batched builds only.
int run_build(pg_handle h, const pg_params* p, const float* base, uint64_t n, uint32_t d,
              const uint32_t* gt, uint64_t q, uint32_t* graph_out, uint32_t* proj_out,
              pg_stats* st, const uint64_t* seg_off = nullptr, const uint64_t* qseg_off = nullptr,
              uint32_t seg_count = 0) {
  cudaStream_t s = h->stream;
  const uint32_t L = p->km + p->kp * p->kd;
  const uint32_t pmax = std::max(p->proj_pruned, p->degree);
  const uint32_t rmax = std::max(p->proj_reverse, p->link_reverse);
  Layout lay = make_layout(n, pmax, rmax, L, p->proj_degree, p->degree, seg_count);
  int rc = ensure_ws(h, lay.total);
  if (rc) return rc;
  char* w = h->ws;
  uint32_t* winner = reinterpret_cast<uint32_t*>(w + lay.winner);
  uint32_t* pruned = reinterpret_cast<uint32_t*>(w + lay.pruned);
  uint32_t* pnum = reinterpret_cast<uint32_t*>(w + lay.pruned_num);
  uint32_t* indeg = reinterpret_cast<uint32_t*>(w + lay.indeg);
  uint32_t* offs = reinterpret_cast<uint32_t*>(w + lay.offs);
  uint32_t* tsum = reinterpret_cast<uint32_t*>(w + lay.tile_sums);
  uint32_t* cursor = reinterpret_cast<uint32_t*>(w + lay.cursor);
  uint32_t* edges = reinterpret_cast<uint32_t*>(w + lay.edges);
  uint32_t* rev = reinterpret_cast<uint32_t*>(w + lay.rev);
  uint32_t* rnum = reinterpret_cast<uint32_t*>(w + lay.rev_num);
  uint32_t* sres = reinterpret_cast<uint32_t*>(w + lay.sres);
  uint32_t* proj = proj_out ? proj_out : reinterpret_cast<uint32_t*>(w + lay.proj);
  float2* norms = reinterpret_cast<float2*>(w + lay.norms);
  float* seeds = reinterpret_cast<float*>(w + lay.seeds);
  const bool screened = p->screen != PG_SCREEN_NONE && pg::screen_supported(L, d, 1);
  unsigned long long* cnt = h->d_counters;
  const int sms = h->num_sms;
  uint64_t* d_seg = nullptr;
  uint64_t* d_qseg = nullptr;
  if (seg_count) {
    d_seg = reinterpret_cast<uint64_t*>(w + lay.segs);
    d_qseg = d_seg + seg_count + 1;
  }
  if (seg_count) {  // the sub-index table, staged in pinned memory owned by the handle
    rc = ensure_segs(h, 2 * (static_cast<size_t>(seg_count) + 1));
    if (rc) return rc;
    std::memcpy(h->h_segs, seg_off, (seg_count + 1) * 8);
    std::memcpy(h->h_segs + seg_count + 1, qseg_off, (seg_count + 1) * 8);
  }
  // everything the build puts on the stream, up to the read-back of status and counters; the
  // per-stage events are left out of a captured graph (it is timed as a whole)
  const bool use_graph = (p->flags & PG_FLAG_CUDA_GRAPH) && s != nullptr;
  const bool stage_events = !use_graph;
  auto enqueue = [&]() -> int {
    if (seg_count) {
      PG_CUDA(cudaMemcpyAsync(d_seg, h->h_segs, 2 * (seg_count + 1) * 8, cudaMemcpyHostToDevice,
                              s));
    }

    PG_CUDA(cudaMemsetAsync(h->d_status, 0, sizeof(uint32_t), s));
    PG_CUDA(cudaMemsetAsync(cnt, 0, C_COUNT * sizeof(unsigned long long), s));
    PG_CUDA(cudaMemsetAsync(h->d_work, 0, 8 * sizeof(uint32_t), s));
    if (stage_events) PG_CUDA(cudaEventRecord(h->ev[0], s));

    // K0 projection winners; K1+K2 phase-1 prune (rows read from gt through the winner)
    PG_CUDA(pg::launch_match_winner(gt, q, p->gt_k, n, winner, h->d_status, sms, s, d_seg, d_qseg,
                                    seg_count));
    PG_CUDA(cudaMemsetAsync(indeg, 0, n * 4, s));
    pg::PruneArgs pa{};
    pa.base = base;
    pa.n = n;
    pa.d = d;
    pa.graph = nullptr;
    pa.c = p->gt_k;
    pa.gt = gt;
    pa.winner = winner;
    pa.gt_k = p->gt_k;
    pa.p = p->proj_pruned;
    pa.strict = 0;
    pa.pruned = pruned;
    pa.pruned_num = pnum;
    pa.indeg = indeg;
    pa.sorted = nullptr;
    pa.evals = cnt + C_PROJ_PRUNE;
    pa.status = h->d_status;
    pa.seg_off = d_seg;
    pa.qseg_off = d_qseg;
    pa.seg_count = seg_count;
    PG_CUDA(pg::launch_prune_reverse(pa, true, sms, s));
    PG_CUDA(pg::launch_reverse_csr(pruned, pnum, p->proj_pruned, n, indeg, offs, tsum, cursor, edges,
                                   sms, s));
    PG_CUDA(pg::launch_reverse_lists(offs, edges, n, p->proj_reverse, rev, rnum, sms, s));
    // K3 phase-1 merge -> projection graph
    pg::MergeArgs ma{};
    ma.base = base;
    ma.n = n;
    ma.d = d;
    ma.pruned = pruned;
    ma.pruned_num = pnum;
    ma.p = p->proj_pruned;
    ma.reverse = rev;
    ma.reverse_num = rnum;
    ma.r = p->proj_reverse;
    ma.degree = p->proj_degree;
    ma.strict = 0;
    ma.out = proj;
    ma.evals = cnt + C_PROJ_MERGE;
    ma.status = h->d_status;
    PG_CUDA(pg::launch_merge_prune(ma, sms, s));
    if (stage_events) PG_CUDA(cudaEventRecord(h->ev[1], s));

    const uint32_t* g = proj;
    uint32_t gdeg = p->proj_degree;
    const uint32_t hslots = hash_slots_for(p->km, p->reset_iter, p->kp * p->kd) *
                            std::max(1u, h->tune.hash_factor);
    for (uint32_t r = 0; r < p->link_rounds; r++) {
      pg::SearchArgs sa{};
      sa.base = base;
      sa.n = n;
      sa.d = d;
      sa.graph = g;
      sa.graph_degree = gdeg;
      sa.km = p->km;
      sa.kp = p->kp;
      sa.kd = p->kd;
      sa.reset_iter = p->reset_iter;
      sa.seed_base = p->seed_base;
      sa.max_iters = p->max_search_iters;
      sa.order = nullptr;
      sa.out = sres;
      sa.out_width = L;
      sa.evals = cnt + C_SEARCH + r;
      sa.iters = cnt + C_ITERS + r;
      sa.work = h->d_work + r;
      sa.status = h->d_status;
      sa.hash_slots = hslots;
      sa.seg_off = d_seg;
      sa.seg_count = seg_count;
      sa.rows = h->tune.search_rows;
      sa.max_blocks_per_sm = h->tune.search_warps_per_sm;
      // the queries (the base points) and their seeds are the same in every round
      if (r == 0) PG_CUDA(pg::launch_seed_dists(sa, seeds, sms, s));
      sa.seed_dist = seeds;
      PG_CUDA(pg::launch_search(sa, sms, h->smem_optin, s));
      if (stage_events) PG_CUDA(cudaEventRecord(h->ev[2 + 3 * r], s));
      PG_CUDA(cudaMemsetAsync(indeg, 0, n * 4, s));
      pg::PruneArgs pr{};
      pr.base = base;
      pr.n = n;
      pr.d = d;
      pr.graph = sres;
      pr.c = L;
      pr.p = p->degree;
      pr.strict = 1;
      pr.pruned = pruned;
      pr.pruned_num = pnum;
      pr.indeg = indeg;
      pr.sorted = nullptr;
      pr.evals = cnt + C_PRUNE + r;
      pr.status = h->d_status;
      pr.rescored = cnt + C_RESCORED + r;
      pr.stages = h->tune.screen_stages;
      pr.screen_half = p->screen == PG_SCREEN_FP16;
      pr.norms = norms;
      if (screened) {
        if (r == 0)
          PG_CUDA(pg::launch_screen_norms(base, n, d, pr.screen_half, norms, sms, s));
        PG_CUDA(pg::launch_prune_screen(pr, sms, h->smem_optin, s));
      } else
        PG_CUDA(pg::launch_prune_reverse(pr, false, sms, s));
      PG_CUDA(pg::launch_reverse_csr(pruned, pnum, p->degree, n, indeg, offs, tsum, cursor, edges,
                                     sms, s));
      PG_CUDA(pg::launch_reverse_lists(offs, edges, n, p->link_reverse, rev, rnum, sms, s));
      if (stage_events) PG_CUDA(cudaEventRecord(h->ev[3 + 3 * r], s));
      pg::MergeArgs mr{};
      mr.base = base;
      mr.n = n;
      mr.d = d;
      mr.pruned = pruned;
      mr.pruned_num = pnum;
      mr.p = p->degree;
      mr.reverse = rev;
      mr.reverse_num = rnum;
      mr.r = p->link_reverse;
      mr.degree = p->degree;
      mr.strict = 1;
      mr.out = graph_out;
      mr.evals = cnt + C_MERGE + r;
      mr.status = h->d_status;
      PG_CUDA(pg::launch_merge_prune(mr, sms, s));
      if (stage_events) PG_CUDA(cudaEventRecord(h->ev[4 + 3 * r], s));
      g = graph_out;
      gdeg = p->degree;
    }
    if (p->link_rounds == 0 && graph_out) {
      // no link rounds: the projection is the graph (degree columns, tomb padded)
      PG_CUDA(cudaMemset2DAsync(graph_out, p->degree * 4, 0xFF, p->degree * 4, n, s));
      PG_CUDA(cudaMemcpy2DAsync(graph_out, p->degree * 4, proj, p->proj_degree * 4,
                                std::min(p->degree, p->proj_degree) * 4, n,
                                cudaMemcpyDeviceToDevice, s));
    }
    if (seg_count) {  // global ids -> ids local to each sub-index
      if (graph_out && p->link_rounds > 0)
        PG_CUDA(pg::launch_localize(graph_out, n, p->degree, d_seg, seg_count, sms, s));
      PG_CUDA(pg::launch_localize(proj, n, p->proj_degree, d_seg, seg_count, sms, s));
    }
    PG_CUDA(cudaMemcpyAsync(h->h_status, h->d_status, 4, cudaMemcpyDeviceToHost, s));
    PG_CUDA(cudaMemcpyAsync(h->h_counters, cnt, C_COUNT * 8, cudaMemcpyDeviceToHost, s));
    return PG_OK;
  };
  if (!use_graph) {
    rc = enqueue();
    if (rc) return rc;
  } else {
    GraphKey key;
    key.p = *p;
    key.ptrs[0] = base;
    key.ptrs[1] = gt;
    key.ptrs[2] = graph_out;
    key.ptrs[3] = proj_out;
    key.ptrs[4] = h->ws;
    key.n = n;
    key.q = q;
    key.d = d;
    key.segs.assign(h->h_segs ? h->h_segs : nullptr,
                    h->h_segs ? h->h_segs + (seg_count ? 2 * (seg_count + 1) : 0) : nullptr);
    if (!h->gexec || !(h->gkey == key)) {
      if (h->gexec) cudaGraphExecDestroy(h->gexec);
      h->gexec = nullptr;
      cudaGraph_t graph = nullptr;
      PG_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
      rc = enqueue();
      cudaError_t ce = cudaStreamEndCapture(s, &graph);
      if (rc) {
        if (graph) cudaGraphDestroy(graph);
        return rc;
      }
      if (ce != cudaSuccess) return fail(PG_ECUDA, "stream capture: %s", cudaGetErrorString(ce));
      ce = cudaGraphInstantiate(&h->gexec, graph, 0);
      cudaGraphDestroy(graph);
      if (ce != cudaSuccess) {
        h->gexec = nullptr;
        return fail(PG_ECUDA, "graph instantiate: %s", cudaGetErrorString(ce));
      }
      h->gkey = key;
    }
    PG_CUDA(cudaEventRecord(h->ev[14], s));
    PG_CUDA(cudaGraphLaunch(h->gexec, s));
    PG_CUDA(cudaEventRecord(h->ev[15], s));
  }
  PG_CUDA(cudaStreamSynchronize(s));
  rc = status_to_error(*h->h_status);
  if (rc) return rc;
  if (st) {
    const unsigned long long* c = h->h_counters;
    st->evals_proj_prune = c[C_PROJ_PRUNE];
    st->evals_proj_merge = c[C_PROJ_MERGE];
    st->evals_total = c[C_PROJ_PRUNE] + c[C_PROJ_MERGE];
    for (int r = 0; r < kMaxRounds; r++) {
      st->evals_search[r] = c[C_SEARCH + r];
      st->evals_prune[r] = c[C_PRUNE + r];
      st->evals_merge[r] = c[C_MERGE + r];
      st->search_iters[r] = c[C_ITERS + r];
      st->rescored[r] = c[C_RESCORED + r];
      st->evals_total += c[C_SEARCH + r] + c[C_PRUNE + r] + c[C_MERGE + r];
    }
    if (use_graph) {  // one replay, timed as a whole
      PG_CUDA(cudaEventElapsedTime(&st->ms_total, h->ev[14], h->ev[15]));
    } else {
      PG_CUDA(cudaEventElapsedTime(&st->ms_proj, h->ev[0], h->ev[1]));
      cudaEvent_t prev = h->ev[1];
      for (uint32_t r = 0; r < p->link_rounds; r++) {
        PG_CUDA(cudaEventElapsedTime(&st->ms_search[r], prev, h->ev[2 + 3 * r]));
        PG_CUDA(cudaEventElapsedTime(&st->ms_prune[r], h->ev[2 + 3 * r], h->ev[3 + 3 * r]));
        PG_CUDA(cudaEventElapsedTime(&st->ms_merge[r], h->ev[3 + 3 * r], h->ev[4 + 3 * r]));
        prev = h->ev[4 + 3 * r];
      }
      PG_CUDA(cudaEventElapsedTime(&st->ms_total, h->ev[0], prev));
    }
  }
  return PG_OK;
}


// ---- CPU RoarGraph path (pg_roar.cu) ------------------------------------------------------

int ensure_ws2(pg_handle h, size_t bytes) {
  if (bytes <= h->ws2_bytes) return PG_OK;
  if (h->ws2) cudaFree(h->ws2);
  h->ws2 = nullptr;
  h->ws2_bytes = 0;
  cudaError_t e = cudaMalloc(&h->ws2, bytes);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return fail(PG_ENOMEM, "cudaMalloc of %zu bytes failed: %s", bytes, cudaGetErrorString(e));
  }
  h->ws2_bytes = bytes;
  return PG_OK;
}

struct SupLayout {
  size_t claim, plist, pcnt, indeg, offs, tiles, cursor, edges, rev, rnum, total;
};

SupLayout sup_layout(uint64_t n, uint64_t q, uint32_t m_nn) {
  SupLayout l{};
  size_t o = 0;
  auto take = [&](size_t bytes) {
    size_t at = o;
    o += align_up(bytes);
    return at;
  };
  const uint32_t maxdeg = 128 - m_nn;
  l.claim = take(n * 4);
  l.plist = take(q * m_nn * 4);
  l.pcnt = take(q * 4);
  l.indeg = take(n * 4);
  l.offs = take((n + 1) * 4);
  l.tiles = take(((n + pg::kScanTileElems - 1) / pg::kScanTileElems + 1) * 4);
  l.cursor = take(n * 4);
  l.edges = take(q * m_nn * 4);
  l.rev = take(n * maxdeg * 4);
  l.rnum = take(n * 4);
  l.total = o;
  return l;
}

int check_sup(uint64_t n, uint32_t d, uint64_t q, uint32_t gt_k, uint32_t topn, uint32_t m_nn) {
  if (n == 0 || n >= 0x7FFFFFFFull || q == 0 || q >= 0x7FFFFFFFull)
    return fail(PG_EINVAL, "n and q must be in [1, 2^31-1)");
  if (d == 0 || d % 4 != 0) return fail(PG_EUNSUPPORTED, "d=%u must be a positive multiple of 4", d);
  if (gt_k == 0 || gt_k > pg::roar_capacity()) return fail(PG_EINVAL, "gt_k must be in [1, 256]");
  if (topn >= gt_k) return fail(PG_EINVAL, "topn=%u must be < gt_k=%u", topn, gt_k);
  if (m_nn < 1 || m_nn > 64) return fail(PG_EINVAL, "m_nn=%u must be in [1, 64]", m_nn);
  return PG_OK;
}

// One MatchSup round on the handle's stream (caller holds the lock; no synchronisation).
int enqueue_match_sup(pg_handle h, const float* base, uint64_t n, uint32_t d, const uint32_t* gt,
                      uint64_t q, uint32_t gt_k, uint32_t topn, uint32_t m_nn, uint32_t* out,
                      uint32_t* cnt) {
  const SupLayout lay = sup_layout(n, q, m_nn);
  int rc = ensure_ws(h, lay.total);
  if (rc) return rc;
  cudaStream_t s = h->stream;
  char* w = h->ws;
  pg::SupArgs a{};
  a.base = base;
  a.n = n;
  a.d = d;
  a.gt = gt;
  a.q = q;
  a.gt_k = gt_k;
  a.topn = topn;
  a.m_nn = m_nn;
  a.maxdeg = 128 - m_nn;
  uint32_t* claim = reinterpret_cast<uint32_t*>(w + lay.claim);
  a.claim = claim;
  a.plist = reinterpret_cast<uint32_t*>(w + lay.plist);
  a.pcnt = reinterpret_cast<uint32_t*>(w + lay.pcnt);
  a.indeg = reinterpret_cast<uint32_t*>(w + lay.indeg);
  uint32_t* offs = reinterpret_cast<uint32_t*>(w + lay.offs);
  uint32_t* rev = reinterpret_cast<uint32_t*>(w + lay.rev);
  uint32_t* rnum = reinterpret_cast<uint32_t*>(w + lay.rnum);
  a.rev = rev;
  a.rnum = rnum;
  a.out = out;
  a.cnt = cnt;
  a.status = h->d_status;
  PG_CUDA(pg::launch_sup_claim(gt, q, gt_k, topn, n, claim, h->num_sms, s));
  PG_CUDA(cudaMemsetAsync(a.indeg, 0, n * 4, s));
  PG_CUDA(pg::launch_sup_prune(a, h->num_sms, s));
  PG_CUDA(pg::launch_reverse_csr(a.plist, a.pcnt, m_nn, n, a.indeg, offs,
                                 reinterpret_cast<uint32_t*>(w + lay.tiles),
                                 reinterpret_cast<uint32_t*>(w + lay.cursor),
                                 reinterpret_cast<uint32_t*>(w + lay.edges), h->num_sms, s, q));
  PG_CUDA(pg::launch_reverse_lists(offs, reinterpret_cast<uint32_t*>(w + lay.edges), n, a.maxdeg,
                                   rev, rnum, h->num_sms, s));
  PG_CUDA(pg::launch_sup_merge(a, h->num_sms, s));
  return PG_OK;
}

int finish(pg_handle h) {
  PG_CUDA(cudaMemcpyAsync(h->h_status, h->d_status, 4, cudaMemcpyDeviceToHost, h->stream));
  PG_CUDA(cudaStreamSynchronize(h->stream));
  return status_to_error(*h->h_status);
}

pg::FusionArgs fusion_args(pg_handle h, const float* base, uint64_t n, uint32_t d) {
  pg::FusionArgs a{};
  a.base = base;
  a.n = n;
  a.d = d;
  a.status = h->d_status;
  return a;
}

// pg_query_search without taking the handle's lock (callers hold it).
int query_search_locked(pg_handle h, const float* d_base, uint64_t n, uint32_t d,
                        const uint32_t* d_graph, uint32_t graph_degree, const float* d_queries,
                        uint64_t nq, uint32_t km, uint32_t kp, uint32_t kd, uint32_t reset_iter,
                        uint32_t seed_base, uint32_t max_iters, uint32_t topk, uint32_t* d_out,
                        uint64_t* evals, uint64_t* iters) {
  if (n == 0 || n >= 0x7FFFFFFFull || nq == 0 || nq >= 0x7FFFFFFFull)
    return fail(PG_EINVAL, "bad n or nq");
  if (!pg::search_supported(d, km, kp, kd))
    return fail(PG_EUNSUPPORTED, "search supports kp*kd == 32, km in {32,64,96}, d <= 512, d %% 4 == 0");
  if (kd > graph_degree) return fail(PG_EINVAL, "kd exceeds graph_degree");
  if (reset_iter < 1) return fail(PG_EINVAL, "reset_iter must be positive");
  if (topk < 1 || topk > km + kp * kd) return fail(PG_EINVAL, "topk must be in [1, km + kp*kd]");
  if (!aligned16(d_base) || !aligned16(d_queries))
    return fail(PG_EINVAL, "base and queries must be 16-byte aligned");
  PG_CUDA(cudaSetDevice(h->device));
  cudaStream_t s = h->stream;
  PG_CUDA(cudaMemsetAsync(h->d_status, 0, 4, s));
  PG_CUDA(cudaMemsetAsync(h->d_counters, 0, 16, s));
  PG_CUDA(cudaMemsetAsync(h->d_work, 0, 4, s));
  pg::SearchArgs a{};
  a.base = d_base;
  a.n = n;
  a.d = d;
  a.graph = d_graph;
  a.graph_degree = graph_degree;
  a.km = km;
  a.kp = kp;
  a.kd = kd;
  a.reset_iter = reset_iter;
  a.seed_base = seed_base;
  a.max_iters = max_iters;
  a.out = d_out;
  a.evals = h->d_counters;
  a.iters = h->d_counters + 1;
  a.work = h->d_work;
  a.status = h->d_status;
  a.hash_slots = hash_slots_for(km, reset_iter, kp * kd);
  a.queries = d_queries;
  a.nq = nq;
  a.out_width = topk;
  a.rows = h->tune.search_rows;
  a.max_blocks_per_sm = h->tune.search_warps_per_sm;
  PG_CUDA(pg::launch_search(a, h->num_sms, h->smem_optin, s));
  PG_CUDA(cudaMemcpyAsync(h->h_status, h->d_status, 4, cudaMemcpyDeviceToHost, s));
  PG_CUDA(cudaMemcpyAsync(h->h_counters, h->d_counters, 16, cudaMemcpyDeviceToHost, s));
  PG_CUDA(cudaStreamSynchronize(s));
  if (evals) *evals = h->h_counters[0];
  if (iters) *iters = h->h_counters[1];
  return status_to_error(*h->h_status);
}

}  // namespace

extern "C" {

const char* pg_last_error(void) { return g_err.c_str(); }

uint32_t pg_abi_version(void) { return PG_ABI_VERSION; }

int pg_params_default(pg_params* p, uint32_t degree, uint32_t beam) {
  if (!p) return fail(PG_EINVAL, "params is NULL");
  if (degree < 2 || degree > 126) return fail(PG_EINVAL, "degree=%u must be in [2, 126]", degree);
  const uint32_t kp = 2, kd = 16;
  if (beam <= kp * kd) return fail(PG_EINVAL, "beam=%u must exceed kp*kd=%u", beam, kp * kd);
  std::memset(p, 0, sizeof(*p));
  p->gt_k = 128;
  p->proj_degree = 16;
  p->proj_pruned = 15;
  p->proj_reverse = 111;
  p->degree = degree;
  p->link_reverse = 128 - 2 - degree;
  p->link_rounds = 2;
  p->km = beam - kp * kd;
  p->kp = kp;
  p->kd = kd;
  p->reset_iter = 15;
  p->seed_base = 3030517;
  p->max_search_iters = 1u << 20;
  p->screen = PG_SCREEN_NONE;
  p->flags = 0;
  return PG_OK;
}

int pg_create(pg_handle* out, int device, void* stream) {
  if (!out) return fail(PG_EINVAL, "out is NULL");
  *out = nullptr;
  int count = 0;
  PG_CUDA(cudaGetDeviceCount(&count));
  if (device < 0 || device >= count) return fail(PG_EINVAL, "device %d of %d", device, count);
  PG_CUDA(cudaSetDevice(device));
  pg_handle h = new (std::nothrow) pg_handle_s();
  if (!h) return fail(PG_ENOMEM, "host allocation failed");
  h->device = device;
  h->stream = static_cast<cudaStream_t>(stream);
  cudaDeviceProp prop;
  cudaError_t e = cudaGetDeviceProperties(&prop, device);
  if (e == cudaSuccess) e = cudaMalloc(&h->d_status, 64);
  if (e == cudaSuccess) e = cudaMalloc(&h->d_counters, 64 * sizeof(unsigned long long));
  if (e == cudaSuccess) e = cudaMalloc(&h->d_work, 64);
  if (e == cudaSuccess) e = cudaMallocHost(&h->h_status, 64);
  if (e == cudaSuccess) e = cudaMallocHost(&h->h_counters, 64 * sizeof(unsigned long long));
  for (int i = 0; i < 16 && e == cudaSuccess; i++) e = cudaEventCreate(&h->ev[i]);
  if (e != cudaSuccess) {
    pg_destroy(h);
    return fail(PG_ECUDA, "pg_create: %s", cudaGetErrorString(e));
  }
  h->num_sms = prop.multiProcessorCount;
  h->smem_optin = prop.sharedMemPerBlockOptin;
  *out = h;
  return PG_OK;
}

int pg_destroy(pg_handle h) {
  if (!h) return PG_OK;
  cudaSetDevice(h->device);
  if (h->stream) cudaStreamSynchronize(h->stream);
  cudaFree(h->ws);
  cudaFree(h->ws2);
  cudaFree(h->inbuf);
  cudaFree(h->d_status);
  cudaFree(h->d_counters);
  cudaFree(h->d_work);
  cudaFreeHost(h->h_status);
  cudaFreeHost(h->h_counters);
  if (h->h_segs) cudaFreeHost(h->h_segs);
  if (h->gexec) cudaGraphExecDestroy(h->gexec);
  for (int i = 0; i < 16; i++)
    if (h->ev[i]) cudaEventDestroy(h->ev[i]);
  if (h->copy_done) cudaEventDestroy(h->copy_done);
  for (cudaEvent_t& e : h->host_ev)
    if (e) cudaEventDestroy(e);
  if (h->copy_stream) cudaStreamDestroy(h->copy_stream);
  delete h;
  return PG_OK;
}

int pg_workspace_bytes(const pg_params* p, uint64_t n, uint32_t d, uint64_t q, uint64_t* bytes) {
  int rc = check_params(p, n, d, q);
  if (rc) return rc;
  if (!bytes) return fail(PG_EINVAL, "bytes is NULL");
  const uint32_t L = p->km + p->kp * p->kd;
  Layout l = make_layout(n, std::max(p->proj_pruned, p->degree),
                         std::max(p->proj_reverse, p->link_reverse), L, p->proj_degree, p->degree);
  *bytes = l.total;
  return PG_OK;
}

int pg_build_device(pg_handle h, const pg_params* p, const float* d_base, uint64_t n, uint32_t d,
                    const uint32_t* d_gt, uint64_t q, uint32_t* d_graph, uint32_t* d_proj,
                    pg_stats* st) {
  if (!h) return fail(PG_EINVAL, "handle is NULL");
  int rc = check_params(p, n, d, q);
  if (rc) return rc;
  if (!d_base || !d_gt) return fail(PG_EINVAL, "base and gt must be device pointers");
  if (p->link_rounds > 0 && !d_graph) return fail(PG_EINVAL, "graph output is NULL");
  if (!aligned16(d_base)) return fail(PG_EINVAL, "base must be 16-byte aligned");
  std::lock_guard<std::mutex> lk(h->mu);
  PG_CUDA(cudaSetDevice(h->device));
  if (st) std::memset(st, 0, sizeof(*st));
  return run_build(h, p, d_base, n, d, d_gt, q, d_graph, d_proj, st);
}

int pg_build_host(pg_handle h, const pg_params* p, const float* base, uint64_t n, uint32_t d,
                  const uint32_t* gt, uint64_t q, uint32_t* graph, uint32_t* proj, pg_stats* st) {
  if (!h) return fail(PG_EINVAL, "handle is NULL");
  int rc = check_params(p, n, d, q);
  if (rc) return rc;
  if (!base || !gt) return fail(PG_EINVAL, "base and gt are NULL");
  std::lock_guard<std::mutex> lk(h->mu);
  PG_CUDA(cudaSetDevice(h->device));
  const size_t bb = align_up(n * d * 4), gb = align_up(q * p->gt_k * 4);
  const size_t ob = align_up(n * p->degree * 4), pb = align_up(n * p->proj_degree * 4);
  rc = ensure_in(h, bb + gb + ob + pb);
  if (rc) return rc;
  float* d_base = reinterpret_cast<float*>(h->inbuf);
  uint32_t* d_gt = reinterpret_cast<uint32_t*>(h->inbuf + bb);
  uint32_t* d_graph = reinterpret_cast<uint32_t*>(h->inbuf + bb + gb);
  uint32_t* d_proj = reinterpret_cast<uint32_t*>(h->inbuf + bb + gb + ob);
  cudaStream_t s = h->stream;
  for (cudaEvent_t& e : h->host_ev)
    if (!e) PG_CUDA(cudaEventCreate(&e));
  cudaEvent_t t0 = h->host_ev[0], t1 = h->host_ev[1], t2 = h->host_ev[2], t3 = h->host_ev[3];
  if (!h->copy_stream) {
    PG_CUDA(cudaStreamCreateWithFlags(&h->copy_stream, cudaStreamNonBlocking));
    PG_CUDA(cudaEventCreateWithFlags(&h->copy_done, cudaEventDisableTiming));
  }
  const size_t hb = n * d * 4, hg = q * p->gt_k * 4;
  PG_CUDA(cudaEventRecord(t0, s));
  // Pinned host memory that the device can address (cudaHostGetDevicePointer succeeds) is read
  // by a copy kernel: the SMs keep more requests in flight over the CPU-GPU link than the copy
  // engines.  Other host memory goes through cudaMemcpyAsync, split over two streams so that two
  // copy engines share it.
  const void* mb = mapped_host(base, hb);
  const void* mg = mapped_host(gt, hg);
  if (mb && mg) {
    PG_CUDA(pg::launch_copy16(d_base, mb, hb, h->num_sms, s));
    PG_CUDA(pg::launch_copy16(d_gt, mg, hg, h->num_sms, s));
  } else {
    const size_t b1 = std::min(hb, ((hb + hg) / 2) & ~static_cast<size_t>(4095));
    PG_CUDA(cudaStreamWaitEvent(h->copy_stream, t0, 0));
    PG_CUDA(cudaMemcpyAsync(d_base, base, b1, cudaMemcpyHostToDevice, s));
    if (hb > b1)
      PG_CUDA(cudaMemcpyAsync(reinterpret_cast<char*>(d_base) + b1,
                              reinterpret_cast<const char*>(base) + b1, hb - b1,
                              cudaMemcpyHostToDevice, h->copy_stream));
    PG_CUDA(cudaMemcpyAsync(d_gt, gt, hg, cudaMemcpyHostToDevice, h->copy_stream));
    PG_CUDA(cudaEventRecord(h->copy_done, h->copy_stream));
    PG_CUDA(cudaStreamWaitEvent(s, h->copy_done, 0));
  }
  PG_CUDA(cudaEventRecord(t1, s));
  if (st) std::memset(st, 0, sizeof(*st));
  rc = run_build(h, p, d_base, n, d, d_gt, q, d_graph, d_proj, st);
  if (rc) return rc;
  PG_CUDA(cudaEventRecord(t2, s));
  uint64_t d2h = 0;
  auto to_host = [&](uint32_t* dst, const uint32_t* src, size_t bytes) -> cudaError_t {
    void* md = mapped_host(dst, bytes);
    if (md) return pg::launch_copy16(md, src, bytes, h->num_sms, s);
    return cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, s);
  };
  if (graph && p->link_rounds > 0) {
    PG_CUDA(to_host(graph, d_graph, n * p->degree * 4));
    d2h += n * p->degree * 4;
  }
  if (proj) {
    PG_CUDA(to_host(proj, d_proj, n * p->proj_degree * 4));
    d2h += n * p->proj_degree * 4;
  }
  PG_CUDA(cudaEventRecord(t3, s));
  PG_CUDA(cudaStreamSynchronize(s));
  if (st) {
    cudaEventElapsedTime(&st->ms_h2d, t0, t1);
    cudaEventElapsedTime(&st->ms_d2h, t2, t3);
    st->h2d_bytes = n * d * 4 + q * p->gt_k * 4;
    st->d2h_bytes = d2h;
  }
  return PG_OK;
}

int pg_build_batched_device(pg_handle h, const pg_params* p, const float* d_base, uint32_t d,
                            const uint32_t* d_gt, const uint64_t* node_off,
                            const uint64_t* query_off, uint32_t count, uint32_t* d_graph,
                            uint32_t* d_proj, pg_stats* st) {
  if (!h) return fail(PG_EINVAL, "handle is NULL");
  if (!node_off || !query_off || count == 0) return fail(PG_EINVAL, "empty sub-index table");
  if (node_off[0] != 0 || query_off[0] != 0) return fail(PG_EINVAL, "offsets must start at 0");
  for (uint32_t i = 0; i < count; i++) {
    if (node_off[i + 1] <= node_off[i]) return fail(PG_EINVAL, "sub-index %u is empty", i);
    if (query_off[i + 1] < query_off[i]) return fail(PG_EINVAL, "query offsets must ascend");
  }
  const uint64_t n = node_off[count], q = query_off[count];
  int rc = check_params(p, n, d, q);
  if (rc) return rc;
  if (!d_base || !d_gt || (p->link_rounds > 0 && !d_graph))
    return fail(PG_EINVAL, "base, gt and graph must be device pointers");
  if (!aligned16(d_base)) return fail(PG_EINVAL, "base must be 16-byte aligned");
  std::lock_guard<std::mutex> lk(h->mu);
  PG_CUDA(cudaSetDevice(h->device));
  if (st) std::memset(st, 0, sizeof(*st));
  return run_build(h, p, d_base, n, d, d_gt, q, d_graph, d_proj, st, node_off, query_off, count);
}

// ---------------------------------------------------------------- stage entry points

int pg_match_top1(pg_handle h, const uint32_t* d_gt, uint64_t q, uint32_t gt_k, uint64_t n,
                  uint32_t* d_out) {
  if (!h || !d_gt || !d_out) return fail(PG_EINVAL, "NULL argument");
  if (gt_k < 3 || n == 0 || n >= 0x7FFFFFFFull || q >= 0x7FFFFFFFull)
    return fail(PG_EINVAL, "bad sizes");
  std::lock_guard<std::mutex> lk(h->mu);
  PG_CUDA(cudaSetDevice(h->device));
  int rc = ensure_ws(h, align_up(n * 4));
  if (rc) return rc;
  uint32_t* winner = reinterpret_cast<uint32_t*>(h->ws);
  cudaStream_t s = h->stream;
  PG_CUDA(cudaMemsetAsync(h->d_status, 0, 4, s));
  PG_CUDA(pg::launch_match_winner(d_gt, q, gt_k, n, winner, h->d_status, h->num_sms, s));
  PG_CUDA(pg::launch_match_rows(d_gt, gt_k, n, winner, d_out, h->num_sms, s));
  PG_CUDA(cudaMemcpyAsync(h->h_status, h->d_status, 4, cudaMemcpyDeviceToHost, s));
  PG_CUDA(cudaStreamSynchronize(s));
  return status_to_error(*h->h_status);
}

int pg_prune_reverse(pg_handle h, const float* d_base, uint64_t n, uint32_t d,
                     const uint32_t* d_graph, uint32_t c, uint32_t pruned, uint32_t reverse,
                     int strict, uint32_t* d_pruned, uint32_t* d_pruned_num, uint32_t* d_reverse,
                     uint32_t* d_reverse_num, uint32_t* d_sorted, uint64_t* evals) {
  if (!h || !d_base || !d_graph || !d_pruned || !d_pruned_num || !d_reverse || !d_reverse_num)
    return fail(PG_EINVAL, "NULL argument");
  if (n == 0 || n >= 0x7FFFFFFFull || d == 0) return fail(PG_EINVAL, "bad sizes");
  if (d % 4 != 0 || !aligned16(d_base)) return fail(PG_EUNSUPPORTED, "d %% 4 != 0 or unaligned base");
  if (c < 1 || c > 128) return fail(PG_EINVAL, "c=%u must be in [1, 128]", c);
  if (pruned < 2 || pruned > c) return fail(PG_EINVAL, "pruned=%u must be in [2, c]", pruned);
  if (reverse > 128) return fail(PG_EINVAL, "reverse must be <= 128");
  std::lock_guard<std::mutex> lk(h->mu);
  PG_CUDA(cudaSetDevice(h->device));
  const size_t tiles = (n + pg::kScanTileElems - 1) / pg::kScanTileElems + 1;
  const size_t b_indeg = align_up(n * 4), b_offs = align_up((n + 1) * 4),
               b_tiles = align_up(tiles * 4), b_cursor = align_up(n * 4),
               b_edges = align_up(n * pruned * 4);
  int rc = ensure_ws(h, b_indeg + b_offs + b_tiles + b_cursor + b_edges);
  if (rc) return rc;
  char* w = h->ws;
  uint32_t* indeg = reinterpret_cast<uint32_t*>(w);
  uint32_t* offs = reinterpret_cast<uint32_t*>(w + b_indeg);
  uint32_t* tsum = reinterpret_cast<uint32_t*>(w + b_indeg + b_offs);
  uint32_t* cursor = reinterpret_cast<uint32_t*>(w + b_indeg + b_offs + b_tiles);
  uint32_t* edges = reinterpret_cast<uint32_t*>(w + b_indeg + b_offs + b_tiles + b_cursor);
  cudaStream_t s = h->stream;
  PG_CUDA(cudaMemsetAsync(h->d_counters, 0, 8, s));
  PG_CUDA(cudaMemsetAsync(indeg, 0, n * 4, s));
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
  a.sorted = d_sorted;
  a.evals = h->d_counters;
  a.status = h->d_status;
  PG_CUDA(cudaMemsetAsync(h->d_status, 0, 4, s));
  PG_CUDA(pg::launch_prune_reverse(a, false, h->num_sms, s));
  PG_CUDA(pg::launch_reverse_csr(d_pruned, d_pruned_num, pruned, n, indeg, offs, tsum, cursor,
                                 edges, h->num_sms, s));
  PG_CUDA(pg::launch_reverse_lists(offs, edges, n, reverse, d_reverse, d_reverse_num, h->num_sms, s));
  PG_CUDA(cudaMemcpyAsync(h->h_counters, h->d_counters, 8, cudaMemcpyDeviceToHost, s));
  PG_CUDA(cudaMemcpyAsync(h->h_status, h->d_status, 4, cudaMemcpyDeviceToHost, s));
  PG_CUDA(cudaStreamSynchronize(s));
  if (evals) *evals = h->h_counters[0];
  return status_to_error(*h->h_status);
}

int pg_merge_prune(pg_handle h, const float* d_base, uint64_t n, uint32_t d,
                   const uint32_t* d_pruned, const uint32_t* d_pruned_num, uint32_t pruned,
                   const uint32_t* d_reverse, const uint32_t* d_reverse_num, uint32_t reverse,
                   uint32_t degree, int strict, uint32_t* d_out, uint64_t* evals) {
  if (!h || !d_base || !d_pruned || !d_pruned_num || !d_reverse || !d_reverse_num || !d_out)
    return fail(PG_EINVAL, "NULL argument");
  if (n == 0 || n >= 0x7FFFFFFFull || d == 0) return fail(PG_EINVAL, "bad sizes");
  if (d % 4 != 0 || !aligned16(d_base)) return fail(PG_EUNSUPPORTED, "d %% 4 != 0 or unaligned base");
  if (pruned + reverse > 128 || degree < 2)
    return fail(PG_EINVAL, "pruned + reverse must be <= 128 and degree >= 2");
  std::lock_guard<std::mutex> lk(h->mu);
  PG_CUDA(cudaSetDevice(h->device));
  cudaStream_t s = h->stream;
  PG_CUDA(cudaMemsetAsync(h->d_counters, 0, 8, s));
  pg::MergeArgs a{};
  a.base = d_base;
  a.n = n;
  a.d = d;
  a.pruned = d_pruned;
  a.pruned_num = d_pruned_num;
  a.p = pruned;
  a.reverse = d_reverse;
  a.reverse_num = d_reverse_num;
  a.r = reverse;
  a.degree = degree;
  a.strict = strict;
  a.out = d_out;
  a.evals = h->d_counters;
  a.status = h->d_status;
  PG_CUDA(cudaMemsetAsync(h->d_status, 0, 4, s));
  PG_CUDA(pg::launch_merge_prune(a, h->num_sms, s));
  PG_CUDA(cudaMemcpyAsync(h->h_counters, h->d_counters, 8, cudaMemcpyDeviceToHost, s));
  PG_CUDA(cudaMemcpyAsync(h->h_status, h->d_status, 4, cudaMemcpyDeviceToHost, s));
  PG_CUDA(cudaStreamSynchronize(s));
  if (evals) *evals = h->h_counters[0];
  return status_to_error(*h->h_status);
}

int pg_search(pg_handle h, const float* d_base, uint64_t n, uint32_t d, const uint32_t* d_graph,
              uint32_t graph_degree, uint32_t km, uint32_t kp, uint32_t kd, uint32_t reset_iter,
              uint32_t seed_base, uint32_t max_iters, uint32_t* d_out, uint64_t* evals,
              uint64_t* iters) {
  if (!h || !d_base || !d_graph || !d_out) return fail(PG_EINVAL, "NULL argument");
  if (n == 0 || n >= 0x7FFFFFFFull) return fail(PG_EINVAL, "bad n");
  if (!pg::search_supported(d, km, kp, kd))
    return fail(PG_EUNSUPPORTED, "search supports kp*kd == 32, km in {32,64,96}, d <= 512, d %% 4 == 0");
  if (kd > graph_degree) return fail(PG_EINVAL, "kd exceeds graph_degree");
  if (reset_iter < 1) return fail(PG_EINVAL, "reset_iter must be positive");
  if (!aligned16(d_base)) return fail(PG_EINVAL, "base must be 16-byte aligned");
  std::lock_guard<std::mutex> lk(h->mu);
  PG_CUDA(cudaSetDevice(h->device));
  cudaStream_t s = h->stream;
  PG_CUDA(cudaMemsetAsync(h->d_status, 0, 4, s));
  PG_CUDA(cudaMemsetAsync(h->d_counters, 0, 16, s));
  PG_CUDA(cudaMemsetAsync(h->d_work, 0, 4, s));
  pg::SearchArgs a{};
  a.base = d_base;
  a.n = n;
  a.d = d;
  a.graph = d_graph;
  a.graph_degree = graph_degree;
  a.km = km;
  a.kp = kp;
  a.kd = kd;
  a.reset_iter = reset_iter;
  a.seed_base = seed_base;
  a.max_iters = max_iters;
  a.order = nullptr;
  a.out = d_out;
  a.evals = h->d_counters;
  a.iters = h->d_counters + 1;
  a.work = h->d_work;
  a.status = h->d_status;
  a.hash_slots = hash_slots_for(km, reset_iter, kp * kd);
  a.out_width = km + kp * kd;
  PG_CUDA(pg::launch_search(a, h->num_sms, h->smem_optin, s));
  PG_CUDA(cudaMemcpyAsync(h->h_status, h->d_status, 4, cudaMemcpyDeviceToHost, s));
  PG_CUDA(cudaMemcpyAsync(h->h_counters, h->d_counters, 16, cudaMemcpyDeviceToHost, s));
  PG_CUDA(cudaStreamSynchronize(s));
  if (evals) *evals = h->h_counters[0];
  if (iters) *iters = h->h_counters[1];
  return status_to_error(*h->h_status);
}

int pg_query_search(pg_handle h, const float* d_base, uint64_t n, uint32_t d,
                    const uint32_t* d_graph, uint32_t graph_degree, const float* d_queries,
                    uint64_t nq, uint32_t km, uint32_t kp, uint32_t kd, uint32_t reset_iter,
                    uint32_t seed_base, uint32_t max_iters, uint32_t topk, uint32_t* d_out,
                    uint64_t* evals, uint64_t* iters) {
  if (!h || !d_base || !d_graph || !d_queries || !d_out) return fail(PG_EINVAL, "NULL argument");
  std::lock_guard<std::mutex> lk(h->mu);
  return query_search_locked(h, d_base, n, d, d_graph, graph_degree, d_queries, nq, km, kp, kd,
                             reset_iter, seed_base, max_iters, topk, d_out, evals, iters);
}

// ---------------------------------------------------------------- autotuning

int pg_set_tuning(pg_handle h, const pg_tuning* t) {
  if (!h || !t) return fail(PG_EINVAL, "NULL argument");
  if (t->search_rows != 0 && t->search_rows != 8 && t->search_rows != 16)
    return fail(PG_EINVAL, "search_rows=%u must be 0, 8 or 16", t->search_rows);
  if (t->search_warps_per_sm > 64) return fail(PG_EINVAL, "search_warps_per_sm must be <= 64");
  if (t->hash_factor > 4 || t->hash_factor == 3)
    return fail(PG_EINVAL, "hash_factor=%u must be 0, 1, 2 or 4", t->hash_factor);
  if (t->screen_stages == 1 || t->screen_stages > 4)
    return fail(PG_EINVAL, "screen_stages must be 0, 2, 3 or 4");
  std::lock_guard<std::mutex> lk(h->mu);
  h->tune = *t;
  if (h->gexec) {  // a captured build holds the old launch shapes
    cudaGraphExecDestroy(h->gexec);
    h->gexec = nullptr;
  }
  return PG_OK;
}

int pg_get_tuning(pg_handle h, pg_tuning* t) {
  if (!h || !t) return fail(PG_EINVAL, "NULL argument");
  std::lock_guard<std::mutex> lk(h->mu);
  *t = h->tune;
  return PG_OK;
}

int pg_autotune(pg_handle h, pg_params* p, const float* d_base, uint32_t d, const uint32_t* d_gt,
                const uint64_t* node_off, const uint64_t* query_off, uint32_t count,
                const float* d_queries, float target_recall, pg_tuning* out) {
  if (!h || !p) return fail(PG_EINVAL, "NULL argument");
  if (!node_off || !query_off || count == 0) return fail(PG_EINVAL, "empty sub-index table");
  if (node_off[0] != 0 || query_off[0] != 0) return fail(PG_EINVAL, "offsets must start at 0");
  for (uint32_t i = 0; i < count; i++) {
    if (node_off[i + 1] <= node_off[i]) return fail(PG_EINVAL, "sub-index %u is empty", i);
    if (query_off[i + 1] < query_off[i]) return fail(PG_EINVAL, "query offsets must ascend");
  }
  const uint64_t n = node_off[count], q = query_off[count];
  int rc = check_params(p, n, d, q);
  if (rc) return rc;
  if (!d_base || !d_gt) return fail(PG_EINVAL, "base and gt must be device pointers");
  if (!aligned16(d_base) || (d_queries && !aligned16(d_queries)))
    return fail(PG_EINVAL, "base and queries must be 16-byte aligned");
  std::lock_guard<std::mutex> lk(h->mu);
  PG_CUDA(cudaSetDevice(h->device));
  pg_params tp = *p;
  tp.flags &= ~PG_FLAG_CUDA_GRAPH;  // per-stage timing
  uint32_t* g = nullptr;
  uint32_t* pj = nullptr;
  uint32_t* qout = nullptr;
  const pg_tuning saved = h->tune;
  struct Cleanup {
    uint32_t** bufs[3];
    ~Cleanup() {
      for (auto b : bufs)
        if (*b) cudaFree(*b);
    }
  } cleanup{{&g, &pj, &qout}};
  PG_CUDA(cudaMalloc(&g, n * tp.degree * 4));
  PG_CUDA(cudaMalloc(&pj, n * tp.proj_degree * 4));
  auto build = [&](const pg_params& bp, pg_stats* st) -> int {
    std::memset(st, 0, sizeof(*st));
    if (count > 1)
      return run_build(h, &bp, d_base, n, d, d_gt, q, g, pj, st, node_off, query_off, count);
    return run_build(h, &bp, d_base, n, d, d_gt, q, g, pj, st);
  };
  auto restore = [&](int code) {
    h->tune = saved;
    return code;
  };
  pg_tuning best{};
  best.search_rows = 8;
  best.hash_factor = 1;
  best.screen_stages = 2;
  h->tune = best;
  pg_stats st;

  // 1) beam: the smallest L reaching the recall target on training queries of the largest
  //    sub-index (their exact top-10 is the first ten ground-truth ids)
  if (d_queries && target_recall > 0.0f && tp.kp * tp.kd == 32 && tp.link_rounds > 0) {
    uint32_t big = 0;
    for (uint32_t i = 1; i < count; i++)
      if (node_off[i + 1] - node_off[i] > node_off[big + 1] - node_off[big]) big = i;
    const uint64_t ni = node_off[big + 1] - node_off[big];
    const uint64_t ns = std::min<uint64_t>(query_off[big + 1] - query_off[big], 1000);
    if (ns > 0) {
      constexpr uint32_t kTop = 10;
      std::vector<uint32_t> truth(ns * tp.gt_k), got(ns * kTop);
      PG_CUDA(cudaMemcpy(truth.data(), d_gt + query_off[big] * tp.gt_k, truth.size() * 4,
                         cudaMemcpyDeviceToHost));
      PG_CUDA(cudaMalloc(&qout, ns * kTop * 4));
      float best_rec = -1.0f, chosen_rec = -1.0f;
      uint32_t best_beam = 0, chosen = 0;
      for (uint32_t beam : {64u, 96u, 128u}) {
        pg_params bp = tp;
        bp.km = beam - bp.kp * bp.kd;
        if (check_params(&bp, n, d, q) != PG_OK) continue;
        rc = build(bp, &st);
        if (rc) return restore(rc);
        rc = query_search_locked(h, d_base + node_off[big] * d, ni, d,
                                 g + node_off[big] * bp.degree, bp.degree,
                                 d_queries + query_off[big] * d, ns, bp.km, bp.kp, bp.kd,
                                 bp.reset_iter, bp.seed_base, bp.max_search_iters, kTop, qout,
                                 nullptr, nullptr);
        if (rc) return restore(rc);
        PG_CUDA(cudaMemcpy(got.data(), qout, got.size() * 4, cudaMemcpyDeviceToHost));
        double hit = 0, tot = 0;
        for (uint64_t i = 0; i < ns; i++) {
          const uint32_t* tr = truth.data() + i * tp.gt_k;
          const uint32_t* gg = got.data() + i * kTop;
          for (uint32_t a = 0; a < kTop; a++) {
            if (tr[a] == PG_TOMB) continue;
            tot += 1;
            for (uint32_t b = 0; b < kTop; b++)
              if (gg[b] == tr[a]) {
                hit += 1;
                break;
              }
          }
        }
        const float rec = tot > 0 ? static_cast<float>(hit / tot) : 0.0f;
        if (rec > best_rec) {
          best_rec = rec;
          best_beam = beam;
        }
        if (rec >= target_recall) {
          chosen = beam;
          chosen_rec = rec;
          break;
        }
      }
      if (!chosen) {
        chosen = best_beam;
        chosen_rec = best_rec;
      }
      if (chosen) {
        tp.km = chosen - tp.kp * tp.kd;
        best.beam = chosen;
        best.recall = chosen_rec;
      }
    }
  }

  // 2) launch shapes: coordinate search from the defaults, best of two builds per candidate
  auto measure = [&](const pg_tuning& t, float* ms) -> int {
    h->tune = t;
    float m = 1e30f;
    for (int rep = 0; rep < 2; rep++) {
      const int r = build(tp, &st);
      if (r) return r;
      m = std::min(m, st.ms_total);
    }
    *ms = m;
    return PG_OK;
  };
  rc = build(tp, &st);  // warm-up (workspace, first launches)
  if (rc) return restore(rc);
  float cur = 0.0f;
  rc = measure(best, &cur);
  if (rc) return restore(rc);
  best.ms_default = cur;
  auto try_value = [&](uint32_t pg_tuning::*field, uint32_t value) -> int {
    pg_tuning t = best;
    t.*field = value;
    float ms = 0.0f;
    const int r = measure(t, &ms);
    if (r == PG_ECUDA && g_err.find("invalid argument") != std::string::npos)
      return PG_OK;  // a shape this device cannot launch (e.g. shared memory): skip it
    if (r) return r;
    if (ms < cur * 0.99f) {
      best = t;
      cur = ms;
    }
    return PG_OK;
  };
  if (tp.link_rounds > 0) {
    if (tp.km == 32) {
      rc = try_value(&pg_tuning::search_rows, 16);
      if (rc) return restore(rc);
    }
    for (uint32_t w : {16u, 12u, 8u}) {
      rc = try_value(&pg_tuning::search_warps_per_sm, w);
      if (rc) return restore(rc);
    }
    for (uint32_t f : {2u, 4u}) {
      rc = try_value(&pg_tuning::hash_factor, f);
      if (rc) return restore(rc);
    }
    if (tp.screen != PG_SCREEN_NONE) {
      for (uint32_t c : {3u, 4u}) {
        rc = try_value(&pg_tuning::screen_stages, c);
        if (rc) return restore(rc);
      }
    }
  }
  best.ms_build = cur;
  h->tune = best;
  if (h->gexec) {
    cudaGraphExecDestroy(h->gexec);
    h->gexec = nullptr;
  }
  p->km = tp.km;
  if (out) *out = best;
  return PG_OK;
}

// ---------------------------------------------------------------- CPU RoarGraph path

int pg_match_sup(pg_handle h, const float* d_base, uint64_t n, uint32_t d, const uint32_t* d_gt,
                 uint64_t q, uint32_t gt_k, uint32_t topn, uint32_t m_nn, uint32_t* d_out,
                 uint32_t* d_cnt) {
  if (!h || !d_base || !d_gt || !d_out || !d_cnt) return fail(PG_EINVAL, "NULL argument");
  int rc = check_sup(n, d, q, gt_k, topn, m_nn);
  if (rc) return rc;
  if (!aligned16(d_base)) return fail(PG_EINVAL, "base must be 16-byte aligned");
  std::lock_guard<std::mutex> lk(h->mu);
  PG_CUDA(cudaSetDevice(h->device));
  PG_CUDA(cudaMemsetAsync(h->d_status, 0, 4, h->stream));
  rc = enqueue_match_sup(h, d_base, n, d, d_gt, q, gt_k, topn, m_nn, d_out, d_cnt);
  if (rc) return rc;
  return finish(h);
}

int pg_fusion_nn(pg_handle h, const float* d_base, uint64_t n, uint32_t d, uint32_t rounds,
                 const uint32_t* d_sup, const uint32_t* d_sup_cnt, uint32_t m_nn,
                 uint32_t* d_out, uint32_t* d_cnt) {
  if (!h || !d_base || !d_sup || !d_sup_cnt || !d_out || !d_cnt)
    return fail(PG_EINVAL, "NULL argument");
  if (n == 0 || n >= 0x7FFFFFFFull) return fail(PG_EINVAL, "bad n");
  if (d == 0 || d % 4 != 0) return fail(PG_EUNSUPPORTED, "d must be a positive multiple of 4");
  if (m_nn < 1 || m_nn > 64) return fail(PG_EINVAL, "m_nn must be in [1, 64]");
  if (rounds < 1 || rounds * m_nn > pg::roar_capacity())
    return fail(PG_EUNSUPPORTED, "rounds * m_nn must be in [1, %u]", pg::roar_capacity());
  if (!aligned16(d_base)) return fail(PG_EINVAL, "base must be 16-byte aligned");
  std::lock_guard<std::mutex> lk(h->mu);
  PG_CUDA(cudaSetDevice(h->device));
  PG_CUDA(cudaMemsetAsync(h->d_status, 0, 4, h->stream));
  pg::FusionArgs a = fusion_args(h, d_base, n, d);
  a.sup = d_sup;
  a.sup_cnt = d_sup_cnt;
  a.sup_stride = m_nn;
  a.rounds = rounds;
  a.m_out = 2 * m_nn;
  a.out = d_out;
  a.cnt = d_cnt;
  a.out_stride = 2 * m_nn;
  PG_CUDA(pg::launch_fusion_nn(a, h->num_sms, h->stream));
  return finish(h);
}

int pg_fusion_final(pg_handle h, const float* d_base, uint64_t n, uint32_t d,
                    const uint64_t* d_bip_off, const uint32_t* d_bip_ids,
                    const uint32_t* d_bip_cnt, uint32_t bip_stride, const uint32_t* d_supply,
                    uint32_t m_supply, const uint32_t* d_link, uint32_t m_link, uint32_t m_final,
                    uint32_t out_stride, uint32_t* d_out, uint32_t* d_cnt) {
  if (!h || !d_base || !d_bip_ids || !d_supply || !d_link || !d_out || !d_cnt)
    return fail(PG_EINVAL, "NULL argument");
  if (!d_bip_off && !d_bip_cnt) return fail(PG_EINVAL, "bipartite lists need offsets or counts");
  if (n == 0 || n >= 0x7FFFFFFFull) return fail(PG_EINVAL, "bad n");
  if (d == 0 || d % 4 != 0) return fail(PG_EUNSUPPORTED, "d must be a positive multiple of 4");
  if (m_final < 1 || m_final > 128) return fail(PG_EINVAL, "m_final must be in [1, 128]");
  if (m_link + m_supply > pg::roar_capacity())
    return fail(PG_EUNSUPPORTED, "m_link + m_supply must be <= %u", pg::roar_capacity());
  if (!aligned16(d_base)) return fail(PG_EINVAL, "base must be 16-byte aligned");
  std::lock_guard<std::mutex> lk(h->mu);
  PG_CUDA(cudaSetDevice(h->device));
  PG_CUDA(cudaMemsetAsync(h->d_status, 0, 4, h->stream));
  pg::FusionArgs a = fusion_args(h, d_base, n, d);
  a.bip = d_bip_ids;
  a.bip_off = d_bip_off;
  a.bip_cnt = d_bip_cnt;
  a.bip_stride = bip_stride;
  a.supply = d_supply;
  a.m_supply = m_supply;
  a.link = d_link;
  a.m_link = m_link;
  a.m_out = m_final;
  a.out = d_out;
  a.cnt = d_cnt;
  a.out_stride = out_stride;
  PG_CUDA(pg::launch_fusion_final(a, h->num_sms, h->stream));
  return finish(h);
}

namespace {

// Argument checks shared by pg_build_index and pg_build_index_host.
int check_index(pg_handle h, const pg_params* p, uint64_t n, uint32_t d, uint64_t q,
                uint32_t match_rounds, uint32_t m_nn, uint32_t m_final, uint32_t out_stride) {
  if (!h) return fail(PG_EINVAL, "handle is NULL");
  int rc = check_params(p, n, d, q);
  if (rc) return rc;
  if (p->link_rounds == 0) return fail(PG_EINVAL, "the index needs the link graph (link_rounds > 0)");
  if (match_rounds < 1 || match_rounds >= p->gt_k)
    return fail(PG_EINVAL, "match_rounds must be in [1, gt_k)");
  rc = check_sup(n, d, q, p->gt_k, match_rounds, m_nn);
  if (rc) return rc;
  if (match_rounds * m_nn > pg::roar_capacity() || 2 * m_nn + p->degree + p->proj_degree >
                                                          pg::roar_capacity())
    return fail(PG_EUNSUPPORTED, "match_rounds * m_nn and 2*m_nn + degree + 16 must be <= %u",
                pg::roar_capacity());
  if (m_final < 1 || m_final > 128) return fail(PG_EINVAL, "m_final must be in [1, 128]");
  if (out_stride < 2 * m_nn + m_final)
    return fail(PG_EINVAL, "out_stride must be >= 2*m_nn + m_final = %u", 2 * m_nn + m_final);
  return PG_OK;
}

// The whole index on device buffers; the caller holds h->mu with h->device current.
int build_index_locked(pg_handle h, const pg_params* p, const float* d_base, uint64_t n,
                       uint32_t d, const uint32_t* d_gt, uint64_t q, uint32_t match_rounds,
                       uint32_t m_nn, uint32_t m_final, uint32_t out_stride, uint32_t* d_out,
                       uint32_t* d_cnt, pg_stats* st) {
  int rc = PG_OK;
  if (st) std::memset(st, 0, sizeof(*st));
  // graphs that outlive a stage: link graph, projection, the rounds' lists, FusionNN's lists
  const size_t b_link = align_up(n * p->degree * 4), b_proj = align_up(n * p->proj_degree * 4);
  const size_t b_sup = align_up(static_cast<size_t>(match_rounds) * n * m_nn * 4);
  const size_t b_supc = align_up(static_cast<size_t>(match_rounds) * n * 4);
  const size_t b_fnn = align_up(n * 2 * m_nn * 4), b_fnnc = align_up(n * 4);
  rc = ensure_ws2(h, b_link + b_proj + b_sup + b_supc + b_fnn + b_fnnc);
  if (rc) return rc;
  uint32_t* link = reinterpret_cast<uint32_t*>(h->ws2);
  uint32_t* proj = reinterpret_cast<uint32_t*>(h->ws2 + b_link);
  uint32_t* sup = reinterpret_cast<uint32_t*>(h->ws2 + b_link + b_proj);
  uint32_t* supc = reinterpret_cast<uint32_t*>(h->ws2 + b_link + b_proj + b_sup);
  uint32_t* fnn = reinterpret_cast<uint32_t*>(h->ws2 + b_link + b_proj + b_sup + b_supc);
  uint32_t* fnnc = reinterpret_cast<uint32_t*>(h->ws2 + b_link + b_proj + b_sup + b_supc + b_fnn);
  pg_params bp = *p;
  bp.flags &= ~PG_FLAG_CUDA_GRAPH;
  rc = run_build(h, &bp, d_base, n, d, d_gt, q, link, proj, st);  // K0..K11 (synchronises)
  if (rc) return rc;
  cudaStream_t s = h->stream;
  PG_CUDA(cudaEventRecord(h->ev[10], s));
  PG_CUDA(cudaMemsetAsync(h->d_status, 0, 4, s));
  for (uint32_t r = 0; r < match_rounds; r++) {  // MatchSup rounds topn = 1 .. match_rounds
    rc = enqueue_match_sup(h, d_base, n, d, d_gt, q, p->gt_k, r + 1, m_nn,
                           sup + static_cast<size_t>(r) * n * m_nn, supc + static_cast<size_t>(r) * n);
    if (rc) return rc;
  }
  PG_CUDA(cudaEventRecord(h->ev[11], s));
  pg::FusionArgs a = fusion_args(h, d_base, n, d);
  a.sup = sup;
  a.sup_cnt = supc;
  a.sup_stride = m_nn;
  a.rounds = match_rounds;
  a.m_out = 2 * m_nn;
  a.out = fnn;
  a.cnt = fnnc;
  a.out_stride = 2 * m_nn;
  PG_CUDA(pg::launch_fusion_nn(a, h->num_sms, s));
  PG_CUDA(cudaEventRecord(h->ev[12], s));
  pg::FusionArgs f = fusion_args(h, d_base, n, d);
  f.bip = fnn;
  f.bip_cnt = fnnc;
  f.bip_stride = 2 * m_nn;
  f.supply = proj;
  f.m_supply = p->proj_degree;
  f.link = link;
  f.m_link = p->degree;
  f.m_out = m_final;
  f.out = d_out;
  f.cnt = d_cnt;
  f.out_stride = out_stride;
  PG_CUDA(pg::launch_fusion_final(f, h->num_sms, s));
  PG_CUDA(cudaEventRecord(h->ev[13], s));
  rc = finish(h);
  if (rc) return rc;
  if (st) {
    PG_CUDA(cudaEventElapsedTime(&st->ms_match_sup, h->ev[10], h->ev[11]));
    PG_CUDA(cudaEventElapsedTime(&st->ms_fusion_nn, h->ev[11], h->ev[12]));
    PG_CUDA(cudaEventElapsedTime(&st->ms_fusion_final, h->ev[12], h->ev[13]));
    st->ms_total += st->ms_match_sup + st->ms_fusion_nn + st->ms_fusion_final;
  }
  return PG_OK;
}

}  // namespace

int pg_build_index(pg_handle h, const pg_params* p, const float* d_base, uint64_t n, uint32_t d,
                   const uint32_t* d_gt, uint64_t q, uint32_t match_rounds, uint32_t m_nn,
                   uint32_t m_final, uint32_t out_stride, uint32_t* d_out, uint32_t* d_cnt,
                   pg_stats* st) {
  int rc = check_index(h, p, n, d, q, match_rounds, m_nn, m_final, out_stride);
  if (rc) return rc;
  if (!d_base || !d_gt || !d_out || !d_cnt) return fail(PG_EINVAL, "NULL argument");
  if (!aligned16(d_base)) return fail(PG_EINVAL, "base must be 16-byte aligned");
  std::lock_guard<std::mutex> lk(h->mu);
  PG_CUDA(cudaSetDevice(h->device));
  return build_index_locked(h, p, d_base, n, d, d_gt, q, match_rounds, m_nn, m_final, out_stride,
                            d_out, d_cnt, st);
}

int pg_build_index_host(pg_handle h, const pg_params* p, const float* base, uint64_t n,
                        uint32_t d, const uint32_t* gt, uint64_t q, uint32_t match_rounds,
                        uint32_t m_nn, uint32_t m_final, uint32_t out_stride, uint32_t* out,
                        uint32_t* cnt, pg_stats* st) {
  int rc = check_index(h, p, n, d, q, match_rounds, m_nn, m_final, out_stride);
  if (rc) return rc;
  if (!base || !gt || !out || !cnt) return fail(PG_EINVAL, "NULL argument");
  std::lock_guard<std::mutex> lk(h->mu);
  PG_CUDA(cudaSetDevice(h->device));
  const size_t bb = align_up(n * d * 4), gb = align_up(q * p->gt_k * 4);
  const size_t ob = align_up(n * out_stride * 4), cb = align_up(n * 4);
  rc = ensure_in(h, bb + gb + ob + cb);
  if (rc) return rc;
  float* d_base = reinterpret_cast<float*>(h->inbuf);
  uint32_t* d_gt = reinterpret_cast<uint32_t*>(h->inbuf + bb);
  uint32_t* d_out = reinterpret_cast<uint32_t*>(h->inbuf + bb + gb);
  uint32_t* d_cnt = reinterpret_cast<uint32_t*>(h->inbuf + bb + gb + ob);
  cudaStream_t s = h->stream;
  PG_CUDA(cudaMemcpyAsync(d_base, base, n * d * 4, cudaMemcpyHostToDevice, s));
  PG_CUDA(cudaMemcpyAsync(d_gt, gt, q * p->gt_k * 4, cudaMemcpyHostToDevice, s));
  rc = build_index_locked(h, p, d_base, n, d, d_gt, q, match_rounds, m_nn, m_final, out_stride,
                          d_out, d_cnt, st);
  if (rc) return rc;
  PG_CUDA(cudaMemcpyAsync(out, d_out, n * out_stride * 4, cudaMemcpyDeviceToHost, s));
  PG_CUDA(cudaMemcpyAsync(cnt, d_cnt, n * 4, cudaMemcpyDeviceToHost, s));
  PG_CUDA(cudaStreamSynchronize(s));
  return PG_OK;
}


// ---------------------------------------------------------------- ground truth

int pg_ground_truth(pg_handle h, const float* d_base, uint64_t n, uint32_t d,
                    const float* d_queries, uint64_t nq, uint32_t k, uint32_t* d_out) {
  if (!h || !d_base || !d_queries || !d_out) return fail(PG_EINVAL, "NULL argument");
  if (n == 0 || n >= 0x7FFFFFFFull || nq == 0 || nq >= 0x7FFFFFFFull)
    return fail(PG_EINVAL, "n and nq must be in [1, 2^31-1)");
  if (d == 0 || d % 4 != 0 || d > pg::gt_max_dim())
    return fail(PG_EUNSUPPORTED, "d=%u must be a positive multiple of 4, at most %u", d,
                pg::gt_max_dim());
  if (k < 1 || k > pg::gt_max_k()) return fail(PG_EINVAL, "k=%u must be in [1, %u]", k, pg::gt_max_k());
  std::lock_guard<std::mutex> lk(h->mu);
  PG_CUDA(cudaSetDevice(h->device));
  const pg::GtPlan plan = pg::gt_plan(n, nq, d, h->num_sms, h->smem_optin);
  int rc = ensure_ws(h, pg::gt_workspace_bytes(plan, n, nq));
  if (rc) return rc;
  PG_CUDA(cudaMemsetAsync(h->d_status, 0, 4, h->stream));
  // diagnostics in the counters' spare words: the first query's margin, max |x^|, max |x - x^|
  float* diag = reinterpret_cast<float*>(h->d_counters + 60);
  const int r = pg::ground_truth(plan, d_base, n, d, d_queries, nq, k, d_out, h->ws,
                                 h->d_status, h->num_sms, h->stream, diag);
  if (r < 0) return fail(PG_ECUDA, "ground truth: %s", cudaGetErrorString(static_cast<cudaError_t>(-r)));
  if (r > 0) return fail(PG_ECUDA, "ground truth: cannot encode a TMA tensor map");
  PG_CUDA(cudaMemcpyAsync(h->h_status, h->d_status, 4, cudaMemcpyDeviceToHost, h->stream));
  PG_CUDA(cudaMemcpyAsync(h->h_counters + 60, diag, 12, cudaMemcpyDeviceToHost, h->stream));
  PG_CUDA(cudaStreamSynchronize(h->stream));
  const uint32_t st = *h->h_status;
  const float* dg = reinterpret_cast<const float*>(h->h_counters + 60);
  if (st & (1u << 4)) return fail(PG_EUNSUPPORTED, "ground truth: a value beyond the FP16 range");
  if (st & (1u << 6))
    return fail(PG_EUNSUPPORTED,
                "ground truth: more candidates within the screening margin than the selection "
                "holds (status 0x%x; first query's margin %g, max |x| %g, max |x - fp16(x)| %g)",
                st, dg[0], dg[1], dg[2]);
  return status_to_error(st);
}

int pg_screen_scores(pg_handle h, const float* d_a, uint64_t na, const float* d_b, uint64_t nb,
                     uint32_t d, float* d_out) {
  if (!h || !d_a || !d_b || !d_out) return fail(PG_EINVAL, "NULL argument");
  if (na == 0 || na >= 0x7FFFFFFFull || nb == 0 || nb >= 0x7FFFFFFFull)
    return fail(PG_EINVAL, "na and nb must be in [1, 2^31-1)");
  if (d == 0 || d % 4 != 0 || d > pg::gt_max_dim())
    return fail(PG_EUNSUPPORTED, "d=%u must be a positive multiple of 4, at most %u", d,
                pg::gt_max_dim());
  std::lock_guard<std::mutex> lk(h->mu);
  PG_CUDA(cudaSetDevice(h->device));
  int rc = ensure_ws(h, pg::screen_scores_workspace(na, nb, d));
  if (rc) return rc;
  PG_CUDA(cudaMemsetAsync(h->d_status, 0, 4, h->stream));
  const int r = pg::screen_scores(d_a, na, d_b, nb, d, d_out, h->ws, h->d_status, h->num_sms,
                                  h->smem_optin, h->stream);
  if (r < 0) return fail(PG_ECUDA, "screen scores: %s", cudaGetErrorString(static_cast<cudaError_t>(-r)));
  if (r > 0) return fail(PG_ECUDA, "screen scores: cannot encode a TMA tensor map");
  PG_CUDA(cudaMemcpyAsync(h->h_status, h->d_status, 4, cudaMemcpyDeviceToHost, h->stream));
  PG_CUDA(cudaStreamSynchronize(h->stream));
  const uint32_t st = *h->h_status;
  if (st & (1u << 4)) return fail(PG_EUNSUPPORTED, "screen scores: a value beyond the FP16 range");
  return status_to_error(st);
}

// ---------------------------------------------------------------- file formats

int pg_read_file(const char* path, int headered, void* dst, uint64_t bytes, uint32_t* rows,
                 uint32_t* cols) {
  if (!path || (!dst && bytes)) return fail(PG_EINVAL, "NULL argument");
  FILE* f = std::fopen(path, "rb");
  if (!f) return fail(PG_EIO, "cannot open %s", path);
  if (headered) {
    uint32_t hdr[2];
    if (std::fread(hdr, 4, 2, f) != 2) {
      std::fclose(f);
      return fail(PG_EIO, "%s: short header", path);
    }
    if (rows) *rows = hdr[0];
    if (cols) *cols = hdr[1];
  }
  size_t got = bytes ? std::fread(dst, 1, bytes, f) : 0;
  std::fclose(f);
  if (got != bytes)
    return fail(PG_EIO, "%s: read %zu of %llu bytes", path, got, (unsigned long long)bytes);
  return PG_OK;
}

int pg_save_graph(const char* path, const uint32_t* graph, uint64_t n, uint32_t degree,
                  uint32_t ep) {
  if (!path || (!graph && n)) return fail(PG_EINVAL, "NULL argument");
  if (n > 0xFFFFFFFFull) return fail(PG_EINVAL, "n does not fit the u32 header");
  FILE* f = std::fopen(path, "wb");
  if (!f) return fail(PG_EIO, "cannot open %s for writing", path);
  uint32_t hdr[2] = {ep, static_cast<uint32_t>(n)};
  bool ok = std::fwrite(hdr, 4, 2, f) == 2;
  std::vector<uint32_t> row(static_cast<size_t>(degree) + 1);
  for (uint64_t i = 0; ok && i < n; i++) {
    uint32_t k = 0;
    for (uint32_t j = 0; j < degree; j++) {
      const uint32_t v = graph[i * degree + j];
      if (v != kTomb) row[1 + k++] = v;
    }
    row[0] = k;
    ok = std::fwrite(row.data(), 4, k + 1, f) == k + 1;
  }
  ok = (std::fclose(f) == 0) && ok;
  return ok ? PG_OK : fail(PG_EIO, "write to %s failed", path);
}

int pg_entry_point(const uint32_t* gt, uint64_t q, uint32_t gt_k, uint64_t n, uint32_t* ep) {
  if (!gt || !ep || n == 0) return fail(PG_EINVAL, "NULL argument");
  std::vector<uint32_t> freq(n, 0);
  std::vector<bool> vis(n, false);
  for (uint64_t qi = 0; qi < q; qi++) {
    bool matched = false;
    for (uint32_t j = 0; j < gt_k; j++) {
      const uint32_t nn = gt[qi * gt_k + j];
      if (nn >= n || matched) break;
      ++freq[nn];
      if (vis[nn]) continue;
      vis[nn] = true;
      matched = true;
    }
  }
  std::vector<uint32_t> order(n);
  std::iota(order.begin(), order.end(), 0u);
  std::sort(order.begin(), order.end(),
            [&](uint32_t a, uint32_t b) { return freq[a] > freq[b]; });
  *ep = order[0];
  return PG_OK;
}

}  // extern "C"
