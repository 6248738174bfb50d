/*
 * ref_search_harness.cpp -- runs the reference's own beam-search kernels on the CPU under a
 * 32-lane warp emulator (TEST INFRASTRUCTURE ONLY; tests/golden/make_golden.py is its only user).
 *
 * Built by oracle/build_ref_search.sh with g++ from include/Gsearcher.cuh, GBitonicSort.cuh and
 * Ghashtable.cuh where they lie in the reference tree; oracle/ref_warp_emu.h supplies the warp
 * (fibers, shuffles, ballots, __syncwarp).  Exported:
 *   ref_link_search    link_process_v0_store_base_data  Gsearcher.cuh:890-1066
 *                      (launched tests/test_t2iend.cu:1051,1096: Km=32, Kp=2, Kd=16, L=64,
 *                      reset_iter=15, HashTable<u32, 4096>), over graphs of degree 16, 32, 55
 *   ref_query_search   search_shared_hashtable          Gsearcher.cuh:108-296
 *                      (Km=32, Kp=2, Kd=16, reset_iter=4, topk=10, HashTable<u32, 4096>)
 * Both run with grid = one block of one warp per query, so every query starts from a fresh warp
 * state, and collect_top_p_normal (Gsearcher.cuh:75-106) runs as the reference wrote it.
 *
 * What the emulator supplies beyond the CUDA built-ins, each the behaviour of a converged warp:
 *   * Converged reads of the id list.  The kernels read a list id into a local (`auto x =
 *     list[i]`) with all 32 lanes converged and rely on every lane's read completing before any
 *     lane goes on (lane 0 then overwrites the explore slot all lanes just read, Gsearcher.cuh:
 *     1003-1013; the scoring loop reads ids the lanes wrote just before, :1016).  The harness
 *     instantiates the kernels with id_type = EmuId, a 32-bit id whose copy is such a warp-wide
 *     read: the lanes meet before and after it.  Every other use of an id (comparisons,
 *     arithmetic, stores) is the plain uint32_t operation.
 *   * warp_sort<float, EmuId, 64, 32> (GBitonicSort.cuh:237-244) is replaced by the canonical
 *     order: ascending distance, ties in list order (stable).  The kernels apply warp_sort to one
 *     shared array from all 32 lanes at once (Gsearcher.cuh:980,1045), where the lanes of a real
 *     warp race; the stable order is the resolution the whole build uses.
 *   * HashTable<u32, 4096>::reset_sync (Ghashtable.cuh:80-86) is declared bool and returns
 *     nothing, which g++ compiles into a crash; the specialisation below empties the lane's slots
 *     like the reference loop, returns, and lets the 32 lanes finish the loop together (they run
 *     it in lockstep on the GPU) before the inserts that follow.
 *   * Never-initialised list slots (Gsearcher.cuh:953-956 sets only their distances) hold tomb.
 * Evaluations are counted as the scored (finite-distance) entries of the candidate part of the
 * list at each sort, iterations as the sorts after the first.
 */
#include "ref_warp_emu.h"

#include <cfloat>
#include <cstdint>
#include <cstring>
#include <vector>

// A list id: plain uint32_t arithmetic; copying one is a converged read by the whole warp.
struct EmuId {
  uint32_t v;
  EmuId() = default;
  EmuId(uint32_t x) : v(x) {}
  EmuId(const EmuId& o) {
    __syncwarp();
    v = o.v;
    __syncwarp();
  }
  EmuId& operator=(const EmuId& o) {
    v = o.v;
    return *this;
  }
  EmuId& operator=(uint32_t x) {
    v = x;
    return *this;
  }
  operator uint32_t&() { return v; }
  operator uint32_t() const { return v; }
};
static_assert(sizeof(EmuId) == 4, "EmuId is a 32-bit id");

#include "GBitonicSort.cuh"
#include "Ghashtable.cuh"

namespace {
constexpr uint32_t kTomb = 0xFFFFFFFFu;
constexpr uint32_t kKm = 32, kKp = 2, kKd = 16, kL = kKm + kKp * kKd;
constexpr uint32_t kHash = 1u << 12;

// per-query counts, indexed by the emulated block (= query)
uint64_t* g_evals = nullptr;
uint64_t* g_iters = nullptr;
}  // namespace

namespace Gbuilder {
namespace Gpu {

template <>
inline void warp_sort<float, EmuId, kL, 32>(float* k, EmuId* v, bool const asc) {
  (void)asc;
  __syncwarp();  // every lane's writes to the list are complete
  if (emu::lane() == 0) {
    const uint32_t q = emu::warp().block;
    uint64_t scored = 0;
    for (uint32_t i = kKm; i < kL; i++) scored += k[i] != FLT_MAX ? 1u : 0u;
    if (g_evals) {
      g_evals[q] += scored;
      g_iters[q] += 1;
    }
    for (uint32_t i = 1; i < kL; i++) {  // stable insertion sort, ascending
      const float key = k[i];
      const uint32_t id = v[i].v;
      uint32_t j = i;
      while (j > 0 && k[j - 1] > key) {
        k[j] = k[j - 1];
        v[j].v = v[j - 1].v;
        j--;
      }
      k[j] = key;
      v[j].v = id;
    }
  }
  __syncwarp();
}

template <>
inline bool HashTable<uint32_t, kHash>::reset_sync(uint32_t const& lane_id) {
  for (uint32_t i = lane_id; i < kHash; i += 32) list_[i] = Kempty;
  __syncwarp();
  return true;
}

}  // namespace Gpu
}  // namespace Gbuilder

#include "Gsearcher.cuh"

#ifndef REF_N
#define REF_N 1000
#endif
#ifndef REF_D
#define REF_D 200
#endif
#ifndef REF_QN
#define REF_QN 2000
#endif
#ifndef REF_QD
#define REF_QD 64
#endif
#ifndef REF_QNQ
#define REF_QNQ 300
#endif
#ifndef REF_QDEG
#define REF_QDEG 32
#endif
#ifndef REF_QTOPK
#define REF_QTOPK 10
#endif

using namespace Gbuilder::Gpu;

namespace {
constexpr uint32_t kN = REF_N, kD = REF_D;
constexpr uint32_t kQN = REF_QN, kQD = REF_QD, kQNQ = REF_QNQ, kQDeg = REF_QDEG,
                   kQTopk = REF_QTOPK;
using LinkState = search_warp_state_store_base_data<EmuId, float, kD, kKm, kKp, kKd>;
using QueryState = search_warp_state<EmuId, float, kQD, kKm, kKp, kKd, kHash>;
const char* g_error = nullptr;
}  // namespace

// The kernels' `extern __shared__` arrays (one warp per block).
namespace Gbuilder {
namespace Gpu {
LinkState ssss_warp_states[1];
QueryState warp_states[1];
}  // namespace Gpu
}  // namespace Gbuilder

namespace {

template <class State>
void fresh_state(State& s) {
  std::memset(&s, 0, sizeof(s));
  for (auto& id : s.node_id_list_) id.v = kTomb;
  for (auto& dd : s.node_distance_list_) dd = FLT_MAX;
}

struct LinkArgs {
  float* base;
  HashTable<uint32_t, kHash>* tables;
  EmuId* graph;
  EmuId* out;
};

template <uint32_t DEG>
void link_body(void* p) {
  auto* a = static_cast<LinkArgs*>(p);
  link_process_v0_store_base_data<kN, 32, kN, kN, kD, DEG, sizeof(LinkState), kKm, kKp, kKd, kL,
                                  kTomb, kHash, 15, EmuId, float>(a->base, a->tables, a->graph,
                                                                  a->out);
}

struct QueryArgs {
  float* base;
  float* queries;
  EmuId* graph;
  EmuId* out;
};

void query_body(void* p) {
  auto* a = static_cast<QueryArgs*>(p);
  search_shared_hashtable<kQNQ, 32, kQN, kQNQ, kQD, kQDeg, sizeof(QueryState), kKm, kKp, kKd,
                          kQTopk, kTomb, kHash, 4, EmuId, float>(a->base, a->queries, a->graph,
                                                                 a->out);
}

template <uint32_t DEG>
int link_search(const float* base, const uint32_t* graph, uint32_t* out, uint64_t* evals,
                uint64_t* iters) {
  std::vector<float> b(base, base + static_cast<size_t>(kN) * kD);
  std::vector<EmuId> g(static_cast<size_t>(kN) * DEG), o(static_cast<size_t>(kN) * kL);
  for (size_t i = 0; i < g.size(); i++) g[i].v = graph[i];
  std::vector<HashTable<uint32_t, kHash>> tables(kN);
  std::memset(evals, 0, sizeof(uint64_t) * kN);
  std::memset(iters, 0, sizeof(uint64_t) * kN);
  g_evals = evals;
  g_iters = iters;
  LinkArgs a{b.data(), tables.data(), g.data(), o.data()};
  for (uint32_t q = 0; q < kN; q++) {
    fresh_state(ssss_warp_states[0]);
    std::memset(tables[q].list_, 0, sizeof(tables[q].list_));
    g_error = emu::run_block(q, &link_body<DEG>, &a);
    if (g_error) break;
    iters[q] -= 1;  // the first sort orders the seeds
  }
  g_evals = g_iters = nullptr;
  if (g_error) return -1;
  for (size_t i = 0; i < o.size(); i++) out[i] = o[i].v;
  return 0;
}

}  // namespace

extern "C" {

uint32_t ref_search_n(void) { return kN; }
uint32_t ref_search_d(void) { return kD; }
const char* ref_search_error(void) { return g_error ? g_error : ""; }

/* base kN x kD, graph kN x degree (degree 16, 32 or 55); out kN x 64 ids (parent bit cleared),
 * evals and iters per query.  Returns 0, -1 when the warp could not be emulated, -2 for an
 * unsupported degree. */
int ref_link_search(uint32_t degree, const float* base, const uint32_t* graph, uint32_t* out,
                    uint64_t* evals, uint64_t* iters) {
  switch (degree) {
    case 16:
      return link_search<16>(base, graph, out, evals, iters);
    case 32:
      return link_search<32>(base, graph, out, evals, iters);
    case 55:
      return link_search<55>(base, graph, out, evals, iters);
    default:
      return -2;
  }
}

void ref_query_shape(uint32_t* shape /* n, d, nq, degree, topk */) {
  shape[0] = kQN;
  shape[1] = kQD;
  shape[2] = kQNQ;
  shape[3] = kQDeg;
  shape[4] = kQTopk;
}

/* base kQN x kQD, graph kQN x kQDeg, queries kQNQ x kQD; out kQNQ x kQTopk, evals and iters
 * per query.  Returns 0 or -1. */
int ref_query_search(const float* base, const uint32_t* graph, const float* queries,
                     uint32_t* out, uint64_t* evals, uint64_t* iters) {
  std::vector<float> b(base, base + static_cast<size_t>(kQN) * kQD);
  std::vector<float> qv(queries, queries + static_cast<size_t>(kQNQ) * kQD);
  std::vector<EmuId> g(static_cast<size_t>(kQN) * kQDeg), o(static_cast<size_t>(kQNQ) * kQTopk);
  for (size_t i = 0; i < g.size(); i++) g[i].v = graph[i];
  std::memset(evals, 0, sizeof(uint64_t) * kQNQ);
  std::memset(iters, 0, sizeof(uint64_t) * kQNQ);
  g_evals = evals;
  g_iters = iters;
  QueryArgs a{b.data(), qv.data(), g.data(), o.data()};
  for (uint32_t q = 0; q < kQNQ; q++) {
    fresh_state(warp_states[0]);
    g_error = emu::run_block(q, &query_body, &a);
    if (g_error) break;
    iters[q] -= 1;
  }
  g_evals = g_iters = nullptr;
  if (g_error) return -1;
  for (size_t i = 0; i < o.size(); i++) out[i] = o[i].v;
  return 0;
}
}
