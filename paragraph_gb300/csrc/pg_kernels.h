// pg_kernels.h -- kernel argument blocks and launchers (host-visible, no device code).
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace pg {

struct PruneArgs {
  const float* base;
  uint64_t n;
  uint32_t d;
  const uint32_t* graph;   // n x c candidate rows (link rounds)
  uint32_t c;              // candidates per node
  const uint32_t* gt;      // phase 1: ground truth q x gt_k
  const uint32_t* winner;  // phase 1: winner key per base
  uint32_t gt_k;
  uint32_t p;              // pruned list length
  int strict;
  uint32_t* pruned;        // n x p
  uint32_t* pruned_num;    // n
  uint32_t* indeg;         // n, incremented per kept edge (reverse in-degree)
  uint32_t* sorted;        // optional n x c: candidate rows after the sort
  unsigned long long* evals;
  uint32_t* status;        // error flags (kErr*)
  unsigned long long* rescored;  // screened kernel: occlusion tests re-scored exactly (nullable)
  // batched builds: node-id offsets of the sub-indexes (seg_count + 1 entries, device) and the
  // query offsets of their ground-truth rows; seg_count == 0 means one index of n nodes
  const uint64_t* seg_off;
  const uint64_t* qseg_off;
  uint32_t seg_count;
  // screened kernel: depth of its row-copy ring (0 = default, else 2..4); results do not
  // depend on it
  uint32_t stages;
  uint32_t screen_half;  // screened kernel: FP16 operands instead of BF16
  // screened kernel: per point (|x|, |x - x^| + |x^_sub|) upper bounds from launch_screen_norms
  // with the same screen_half
  const float2* norms;
};

struct MergeArgs {
  const float* base;
  uint64_t n;
  uint32_t d;
  const uint32_t* pruned;
  const uint32_t* pruned_num;
  uint32_t p;
  const uint32_t* reverse;
  const uint32_t* reverse_num;
  uint32_t r;
  uint32_t degree;
  int strict;
  uint32_t* out;  // n x degree
  unsigned long long* evals;
  uint32_t* status;
};

struct SearchArgs {
  const float* base;
  uint64_t n;
  uint32_t d;
  const uint32_t* graph;  // n x graph_degree
  uint32_t graph_degree;
  uint32_t km, kp, kd, reset_iter, seed_base;
  uint32_t max_iters;
  const uint32_t* order;  // optional query order (permutation of 0..n-1), NULL = identity
  uint32_t* out;          // n x (km + kp*kd)
  unsigned long long* evals;
  unsigned long long* iters;
  uint32_t* work;         // work counter, zeroed before the launch
  uint32_t* status;
  uint32_t hash_slots;    // visited-set capacity per warp (power of two)
  const uint64_t* seg_off;  // batched builds: sub-index node offsets (seg_count + 1), else NULL
  uint32_t seg_count;
  // query search (search_shared_hashtable): nq external query vectors (nq x d) instead of the
  // base points; NULL for the build's link rounds
  const float* queries;
  uint64_t nq;
  uint32_t out_width;  // ids written per query: L for link rounds, top-k for a query search
  // launch shape (results do not depend on it): candidate rows staged per pass (8 or 16, Km = 32
  // kernel) and a cap on resident search warps per SM; 0 = defaults
  uint32_t rows;
  uint32_t max_blocks_per_sm;
  // optional (n or nq) x 32: each query's distances to its 32 seeds from launch_seed_dists (the
  // same values the search would compute); NULL = the search scores the seeds itself
  const float* seed_dist;
};

// CPU RoarGraph path on the GPU (tests/test_t2iend.cu:365-613), pg_roar.cu.
struct SupArgs {  // one MatchSup round
  const float* base;
  uint64_t n;
  uint32_t d;
  const uint32_t* gt;  // q x gt_k
  uint64_t q;
  uint32_t gt_k, topn, m_nn, maxdeg;  // maxdeg = 128 - m_nn reverse sources kept per base
  const uint32_t* claim;  // n: lowest query whose gt[topn] is the base, or tomb
  uint32_t* plist;        // q x m_nn: a matched query's pruned list
  uint32_t* pcnt;         // q
  uint32_t* indeg;        // n: reverse in-degree
  const uint32_t* rev;    // n x maxdeg: first reverse sources (query indices, ascending)
  const uint32_t* rnum;   // n
  uint32_t* out;          // n x m_nn
  uint32_t* cnt;          // n
  uint32_t* status;
};

struct FusionArgs {
  const float* base;
  uint64_t n;
  uint32_t d;
  // FusionNN: `rounds` supply graphs, rounds x n x sup_stride ids + rounds x n counts
  const uint32_t* sup;
  const uint32_t* sup_cnt;
  uint32_t sup_stride, rounds;
  // FusionFinal: bipartite lists as CSR (bip_off != NULL) or rows of bip_stride with counts
  const uint32_t* bip;
  const uint64_t* bip_off;
  const uint32_t* bip_cnt;
  uint32_t bip_stride;
  const uint32_t* supply;  // n x m_supply (projection)
  uint32_t m_supply;
  const uint32_t* link;  // n x m_link (link graph)
  uint32_t m_link;
  uint32_t m_out;  // prune width: 2*M_nn (FusionNN) or M_final
  uint32_t* out;   // n x out_stride
  uint32_t* cnt;   // n
  uint32_t out_stride;
  uint32_t* status;
};

bool roar_supported(uint32_t d, uint32_t m);
uint32_t roar_capacity();
cudaError_t launch_sup_claim(const uint32_t* gt, uint64_t q, uint32_t gt_k, uint32_t topn,
                             uint64_t n, uint32_t* claim, int num_sms, cudaStream_t st);
cudaError_t launch_sup_prune(const SupArgs& a, int num_sms, cudaStream_t st);
cudaError_t launch_sup_merge(const SupArgs& a, int num_sms, cudaStream_t st);
cudaError_t launch_fusion_nn(const FusionArgs& a, int num_sms, cudaStream_t st);
cudaError_t launch_fusion_final(const FusionArgs& a, int num_sms, cudaStream_t st);

// Exact inner-product top-k ground truth (pg_gt.cu): FP16 screening on the tensor cores
// (tcgen05) with a rigorous margin, FP64 re-ranking.  gt_plan picks the padded dimension, the
// M tiles per CTA, the group size of the threshold pass and the queries per chunk.  The entry
// points return 0, a negative cudaError_t, or 1 when a TMA tensor map cannot be encoded;
// device-side problems set bits in *status (1 << 4: a value beyond the FP16 range, 1 << 6: a
// query with more candidates than the selection holds, kErrWait: a bounded wait gave up).
struct GtPlan {
  uint32_t dp;      // d rounded up to a multiple of 16 (FP16 rows zero-padded)
  uint32_t kc;      // 64-element K boxes per row: ceil(dp / 64)
  uint32_t bn;      // base rows per tile (256, against one 128-row query tile)
  uint32_t stages;  // B ring stages
  uint32_t span;    // threshold pass: chunks of 32 columns per group (0: groups of gs columns)
  uint32_t gs;      // threshold pass, small n: columns per group
  uint32_t groups;  // groups per query
  uint64_t cq;      // queries per chunk
};
uint32_t gt_max_k();
uint32_t gt_max_dim();
GtPlan gt_plan(uint64_t n, uint64_t nq, uint32_t d, int num_sms, size_t smem_optin);
size_t gt_workspace_bytes(const GtPlan& p, uint64_t n, uint64_t nq);
int ground_truth(const GtPlan& plan, const float* base, uint64_t n, uint32_t d,
                 const float* queries, uint64_t nq, uint32_t k, uint32_t* out, char* ws,
                 uint32_t* status, int num_sms, cudaStream_t st, float* diag = nullptr);
// out (na x nb, FP32) = fp16(a) . fp16(b)^T accumulated in FP32 on the tensor cores: the
// screening product of ground_truth on its own.
size_t screen_scores_workspace(uint64_t na, uint64_t nb, uint32_t d);
int screen_scores(const float* a, uint64_t na, const float* b, uint64_t nb, uint32_t d,
                  float* out, char* ws, uint32_t* status, int num_sms, size_t smem_optin,
                  cudaStream_t st);

cudaError_t launch_match_winner(const uint32_t* gt, uint64_t q, uint32_t gt_k, uint64_t n,
                                uint32_t* winner, uint32_t* status, int num_sms, cudaStream_t st,
                                const uint64_t* seg_off = nullptr,
                                const uint64_t* qseg_off = nullptr, uint32_t seg_count = 0);
// Rewrites global ids of a batched build's rows (n x deg) to ids local to each row's sub-index.
cudaError_t launch_localize(uint32_t* rows, uint64_t n, uint32_t deg, const uint64_t* seg_off,
                            uint32_t seg_count, int num_sms, cudaStream_t st);
cudaError_t launch_match_rows(const uint32_t* gt, uint32_t gt_k, uint64_t n,
                              const uint32_t* winner, uint32_t* out, int num_sms,
                              cudaStream_t st);
cudaError_t launch_validate_ids(const uint32_t* ids, uint64_t count, uint64_t n,
                                uint32_t* status, int num_sms, cudaStream_t st, float* diag = nullptr);
cudaError_t launch_prune_reverse(const PruneArgs& a, bool phase1, int num_sms, cudaStream_t st);
// Reverse edges as CSR over n destinations: offs = exclusive scan of indeg, edges grouped by
// destination holding the source row index.  `rows` pruned rows are scanned (0 = n).
cudaError_t launch_reverse_csr(const uint32_t* pruned, const uint32_t* pruned_num, uint32_t p_len,
                               uint64_t n, const uint32_t* indeg, uint32_t* offs,
                               uint32_t* tile_sums, uint32_t* cursor, uint32_t* edges,
                               int num_sms, cudaStream_t st, uint64_t rows = 0);
cudaError_t launch_reverse_lists(const uint32_t* offs, const uint32_t* edges, uint64_t n,
                                 uint32_t r, uint32_t* rev, uint32_t* rev_num, int num_sms,
                                 cudaStream_t st);
cudaError_t launch_merge_prune(const MergeArgs& a, int num_sms, cudaStream_t st);
// bytes (a multiple of 16, both pointers 16-byte aligned) from src to dst by a kernel: used with
// pinned host memory mapped into the device address space (cudaHostGetDevicePointer).
cudaError_t launch_copy16(void* dst, const void* src, uint64_t bytes, int num_sms,
                          cudaStream_t st);
// Returns cudaErrorInvalidValue for parameter combinations the search kernel was not built for
// (see search_supported).
cudaError_t launch_search(const SearchArgs& a, int num_sms, size_t smem_optin, cudaStream_t st);
// Every query's 32 seed distances in the search's FP32 order into out (queries x 32).
cudaError_t launch_seed_dists(const SearchArgs& a, float* out, int num_sms, cudaStream_t st);
bool search_supported(uint32_t d, uint32_t km, uint32_t kp, uint32_t kd);
// Screened prune for strict rounds (pg_prune_tc.cu): FP16 or BF16 candidate Gram on the tcgen05
// tensor cores + exact re-scoring, 1 <= c <= 128, 4 <= d <= 1024, d % 4 == 0; the launch also
// wants a 16-byte aligned base.
bool screen_supported(uint32_t c, uint32_t d, int strict);
cudaError_t launch_prune_screen(const PruneArgs& a, int num_sms, size_t smem_optin,
                                cudaStream_t st);
// Per-point norm bounds for the screened prune (FP16 rounding when half, else BF16): n float2.
cudaError_t launch_screen_norms(const float* base, uint64_t n, uint32_t d, uint32_t half,
                                float2* out, int num_sms, cudaStream_t st);

constexpr uint32_t kScanTileElems = 4096;

// Records `msg` as the calling thread's pg_last_error() text and returns `code`.
int set_last_error(int code, const char* msg);
// Maps a device status word (kErr* bits) to the pg_status and pg_last_error() message every
// entry point reports.
int status_error(uint32_t status);

}  // namespace pg
