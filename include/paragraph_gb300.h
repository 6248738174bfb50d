/*
 * paragraph_gb300.h -- C ABI of the GB300 (sm_103a) ParaGraph graph-index builder.
 *
 * Drop-in for the GPU build path of ParaGraph (9p6p/ParaGraph): the twelve kernel launches
 * K0..K11 of tests/test_t2iend.cu:974-1139 that turn base vectors plus each training query's
 * top-128 ground-truth ids into a RoarGraph-style proximity graph.  The reference exposes that
 * path only as kernel templates driven by a gtest body; its intended library shell
 * (include/Builder.hpp:15-35, Gbuilder::Builder<T>) is commented out.  This ABI provides:
 *   - pg_build_host / pg_build_device: the whole pipeline (Builder::LaunchBuild);
 *   - one entry point per reference kernel, for callers that drive the stages themselves;
 *   - readers/writers for the reference's on-disk formats.
 * Every function returns a pg_status; pg_last_error() gives the message of the calling thread's
 * last failure.  No function calls exit().  Sizes are runtime values (the reference fixes
 * N, D and every degree as template parameters).
 *
 * Ids are uint32; PG_TOMB (0xFFFFFFFF) marks an empty slot as in the reference
 * (tests/test_t2iend.cu:674).  Graph outputs are row-major n x degree, tomb padded.
 */
#ifndef PARAGRAPH_GB300_H_
#define PARAGRAPH_GB300_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define PG_TOMB 0xFFFFFFFFu
#define PG_ABI_VERSION 1

typedef enum pg_status {
  PG_OK = 0,
  PG_EINVAL = 1,       /* bad argument: sizes, ids >= n, misaligned or null pointer */
  PG_ECUDA = 2,        /* a CUDA call failed */
  PG_ENOMEM = 3,       /* device or host allocation failed */
  PG_ETIMEOUT = 4,     /* a search exceeded max_search_iters, or a bounded device wait gave up */
  PG_EUNSUPPORTED = 5, /* parameter combination outside what the kernels implement */
  PG_EIO = 6           /* file could not be opened, read or written */
} pg_status;

typedef enum pg_screen {
  PG_SCREEN_NONE = 0, /* plain FP32: every distance in the reference's own FP32 order */
  PG_SCREEN_BF16 = 1, /* BF16 tensor-core screening + exact FP32 re-scoring inside a margin */
  PG_SCREEN_FP8 = 2,  /* FP8 E4M3 per-vector-scaled screening (not built: see the error study) */
  PG_SCREEN_FP16 = 3  /* FP16 tensor-core screening (11-bit significands: a margin about 8x
                         tighter than BF16's) + exact FP32 re-scoring; values beyond FP16's range
                         only make every test of their node exact */
} pg_screen;

/* Build parameters.  pg_params_default() maps (M, L) onto the reference driver's constants
 * (tests/test_t2iend.cu:671-727): phase 1 keeps gt_k=128, proj_degree=16, proj_pruned=15,
 * proj_reverse=111; link rounds use pruned = final degree = M and reverse = 128 - 2 - M; the
 * beam is Km = L - Kp*Kd with Kp=2, Kd=16; reset_iter=15; entry points seed_base + i. */
typedef struct pg_params {
  uint32_t gt_k;             /* ground-truth ids per query (columns of gt) */
  uint32_t proj_degree;      /* out-degree of the projection graph (K3) */
  uint32_t proj_pruned;      /* phase-1 pruned list length (K2) */
  uint32_t proj_reverse;     /* phase-1 reverse list length (K2) */
  uint32_t degree;           /* final out-degree M = link-round pruned length */
  uint32_t link_reverse;     /* link-round reverse list length */
  uint32_t link_rounds;      /* search + prune + merge rounds after the projection (2) */
  uint32_t km;               /* beam: retained list length (Km) */
  uint32_t kp;               /* beam: nodes expanded per iteration (Kp) */
  uint32_t kd;               /* beam: neighbours read per expanded node (Kd) */
  uint32_t reset_iter;       /* the visited set is rebuilt every reset_iter iterations */
  uint32_t seed_base;        /* search entry points are (seed_base + i) % n, i < Kp*Kd */
  uint32_t max_search_iters; /* per-query iteration cap; exceeding it returns PG_ETIMEOUT */
  uint32_t screen;           /* pg_screen */
  uint32_t flags;            /* PG_FLAG_* */
  uint32_t reserved[5];
} pg_params;

/* Ids are always range-checked on the device: an id >= n that is not tomb is replaced by tomb,
 * never read, and the call returns PG_EINVAL.  The flag is accepted for compatibility. */
#define PG_FLAG_VALIDATE_INPUT 1u
/* Capture the whole build (every launch, memset and copy) in a CUDA graph on the handle's stream
 * the first time, and replay that graph on later builds with identical parameters, buffers and
 * sub-index table.  Needs a handle created with a non-default stream; ignored otherwise. */
#define PG_FLAG_CUDA_GRAPH 2u

/* Per-build statistics.  A distance evaluation is one call of the reference's
 * distance_between (Gbuilder.cuh:785-797) or one search distance (Gsearcher.cuh:1016-1036),
 * counted as the reference would count it; tomb and visited slots cost nothing. */
typedef struct pg_stats {
  uint64_t evals_total;
  uint64_t evals_proj_prune, evals_proj_merge;
  uint64_t evals_search[4], evals_prune[4], evals_merge[4];
  uint64_t search_iters[4];
  uint64_t rescored[4];      /* screened path: candidates re-scored exactly in FP32 */
  float ms_total;            /* device time of the whole build (CUDA events) */
  float ms_proj;             /* K0..K3 */
  float ms_search[4], ms_prune[4], ms_merge[4];
  float ms_h2d, ms_d2h;      /* pg_build_host only */
  uint64_t h2d_bytes, d2h_bytes;
  uint32_t ep;               /* entry point (most frequent ground-truth id, MatchNN rule) */
  float ms_match_sup;        /* pg_build_index: the MatchSup rounds */
  float ms_fusion_nn;        /* pg_build_index: FusionNN */
  float ms_fusion_final;     /* pg_build_index: FusionFinal */
  uint32_t reserved[4];
} pg_stats;

typedef struct pg_handle_s* pg_handle;

/* Launch-shape choices of a handle.  None of them changes a result: every choice builds the same
 * graph bit for bit; they only move time.  Zero fields mean the library's defaults. */
typedef struct pg_tuning {
  uint32_t search_rows;         /* candidate rows staged per pass in the Km=32 search: 8 or 16 */
  uint32_t search_warps_per_sm; /* cap on resident search warps per SM (0 = occupancy maximum) */
  uint32_t hash_factor;         /* visited-set capacity multiplier over the exact minimum: 1, 2, 4 */
  uint32_t screen_stages;       /* row-copy ring depth of the screened prune: 0 (= 2), 2, 3, 4 */
  uint32_t beam;                /* L chosen by pg_autotune's recall target (0 = not tuned) */
  float recall;                 /* recall@10 measured for `beam` (when tuned) */
  float ms_build;               /* build time measured with this tuning */
  float ms_default;             /* build time measured with the defaults */
  uint32_t reserved[8];
} pg_tuning;

/* ---- library ---------------------------------------------------------------------------- */
const char* pg_last_error(void);
uint32_t pg_abi_version(void);
int pg_params_default(pg_params* p, uint32_t degree, uint32_t beam);

/* A handle owns the device workspace and runs everything on one CUDA stream.  `stream` is a
 * cudaStream_t (NULL = the legacy default stream).  One build in flight per handle. */
int pg_create(pg_handle* out, int device, void* stream);
int pg_destroy(pg_handle h);
/* Device bytes the handle allocates for a build of n points (the caller can check headroom). */
int pg_workspace_bytes(const pg_params* p, uint64_t n, uint32_t d, uint64_t q, uint64_t* bytes);

/* ---- whole build (Gbuilder::Builder<float>::LaunchBuild, include/Builder.hpp:15-35) ------- */
/* Host buffers: copies base (n x d f32) and gt (q x gt_k u32) to the device, builds, copies
 * the n x degree graph and the n x proj_degree projection back (either may be NULL). */
int pg_build_host(pg_handle h, const pg_params* p, const float* base, uint64_t n, uint32_t d,
                  const uint32_t* gt, uint64_t q, uint32_t* graph, uint32_t* proj, pg_stats* st);
/* Device buffers (resident inputs); outputs are device pointers too (proj may be NULL). */
int pg_build_device(pg_handle h, const pg_params* p, const float* d_base, uint64_t n,
                    uint32_t d, const uint32_t* d_gt, uint64_t q, uint32_t* d_graph,
                    uint32_t* d_proj, pg_stats* st);

/* Batched build of `count` independent sub-indexes (uneven sizes) in one pass of the pipeline:
 * every stage is one launch over all sub-indexes' points, and the beam search's work queue spans
 * them all.  Sub-index i owns points [node_off[i], node_off[i+1]) of d_base (all vectors
 * concatenated) and ground-truth rows [query_off[i], query_off[i+1]) of d_gt, whose ids are local
 * to it (0 .. n_i - 1); entry points are drawn inside each sub-index.  Outputs (concatenated like
 * the inputs, ids local to their sub-index) equal building each sub-index alone.  node_off and
 * query_off are host arrays of count + 1 ascending offsets starting at 0.  This is the batched
 * form of pg_build_device; the reference builds one index per driver run. */
int pg_build_batched_device(pg_handle h, const pg_params* p, const float* d_base, uint32_t d,
                            const uint32_t* d_gt, const uint64_t* node_off,
                            const uint64_t* query_off, uint32_t count, uint32_t* d_graph,
                            uint32_t* d_proj, pg_stats* st);

/* ---- CPU RoarGraph path and final fusion (tests/test_t2iend.cu:365-613), on the GPU --------
 * The reference runs these on the host beside its GPU build.  Results equal its one-thread run
 * (distances in compare()'s AVX-512 FP32 order, lists sorted by (distance, id)), with MatchSup's
 * reverse appends in ascending query order and short merged MatchSup lists in ascending id
 * order (the reference writes std::unordered_set order there).  Lists are rows of a fixed stride
 * with a count per row; D must be a multiple of 4.
 *
 * pg_match_sup: MatchSup (:365-488) round `topn` (1-based rank of the matched ground-truth id):
 *   out n x m_nn, cnt n.  gt: q x gt_k, ids >= n end a row (the reference's padding).
 * pg_fusion_nn: FusionNN (:490-537) over `rounds` MatchSup outputs (rounds x n x m_nn ids and
 *   rounds x n counts, round order as the reference driver's :912-921); MatchNN's own graph is
 *   empty in the reference (its graph-building loop is commented out, :234-306).  out
 *   n x 2*m_nn.
 * pg_fusion_final: FusionFinal (:539-613).  Bipartite lists (the FusionNN graph) as CSR
 *   (d_bip_off, n + 1 offsets) or as rows of bip_stride with counts (d_bip_off NULL); supply =
 *   the projection (n x m_supply), link = the link graph (n x m_link).  Row i of out (stride
 *   out_stride) holds the node's bipartite ids then its pruned ids; a row that does not fit makes
 *   the call return PG_EUNSUPPORTED.
 * pg_build_index: the reference driver's whole index (test_t2iend.cu:974-1229): the GPU build
 *   (K0..K11), `match_rounds` MatchSup rounds (topn 1..match_rounds), FusionNN(m_nn) and
 *   FusionFinal(m_supply = proj_degree, m_link = degree, m_final).  The reference driver's
 *   values are match_rounds 6, m_nn 40, m_final 70; out_stride >= 2*m_nn + m_final.  The entry point is
 *   pg_entry_point of the host ground truth. */
int pg_match_sup(pg_handle h, const float* d_base, uint64_t n, uint32_t d, const uint32_t* d_gt,
                 uint64_t q, uint32_t gt_k, uint32_t topn, uint32_t m_nn, uint32_t* d_out,
                 uint32_t* d_cnt);
int pg_fusion_nn(pg_handle h, const float* d_base, uint64_t n, uint32_t d, uint32_t rounds,
                 const uint32_t* d_sup, const uint32_t* d_sup_cnt, uint32_t m_nn,
                 uint32_t* d_out, uint32_t* d_cnt);
int pg_fusion_final(pg_handle h, const float* d_base, uint64_t n, uint32_t d,
                    const uint64_t* d_bip_off, const uint32_t* d_bip_ids,
                    const uint32_t* d_bip_cnt, uint32_t bip_stride, const uint32_t* d_supply,
                    uint32_t m_supply, const uint32_t* d_link, uint32_t m_link, uint32_t m_final,
                    uint32_t out_stride, uint32_t* d_out, uint32_t* d_cnt);
int pg_build_index(pg_handle h, const pg_params* p, const float* d_base, uint64_t n, uint32_t d,
                   const uint32_t* d_gt, uint64_t q, uint32_t match_rounds, uint32_t m_nn,
                   uint32_t m_final, uint32_t out_stride, uint32_t* d_out, uint32_t* d_cnt,
                   pg_stats* st);
/* pg_build_index with host buffers (base n x d f32, gt q x gt_k u32 in; out n x out_stride and
 * cnt n out): the inputs are copied to the device, the index is built there and copied back
 * (the reference driver's host-side flow, tests/test_t2iend.cu:850-873,1228-1258).  Row i holds
 * cnt[i] ids; the slots after them are unspecified. */
int pg_build_index_host(pg_handle h, const pg_params* p, const float* base, uint64_t n,
                        uint32_t d, const uint32_t* gt, uint64_t q, uint32_t match_rounds,
                        uint32_t m_nn, uint32_t m_final, uint32_t out_stride, uint32_t* out,
                        uint32_t* cnt, pg_stats* st);

/* ---- ground truth (the reference reads it from files made outside its build, README.md:25-31)
 * pg_ground_truth: for each of nq queries (nq x d, device) the k ids of the base rows (n x d)
 * with the largest inner product, best first -- exact: ranked by FP64 inner products, ties to the
 * lower id.  Candidates are screened on the tensor cores (FP16 operands, FP32 accumulation, a
 * tcgen05 GEMM whose epilogue selects: no score matrix is stored) with a rigorous error margin,
 * and every candidate inside the margin is re-scored in FP64.  k <= 256, d <= 512; rows past n
 * are tomb.  PG_EUNSUPPORTED when a value exceeds the FP16 range (|x| > 65000) or the margin
 * holds more candidates than the selection can keep (1024 per query).
 * pg_screen_scores: the screening product on its own, out (na x nb, FP32, device) =
 * fp16(a) . fp16(b)^T with FP32 accumulation (a: na x d, b: nb x d, device, row-major). */
int pg_ground_truth(pg_handle h, const float* d_base, uint64_t n, uint32_t d,
                    const float* d_queries, uint64_t nq, uint32_t k, uint32_t* d_out);
int pg_screen_scores(pg_handle h, const float* d_a, uint64_t na, const float* d_b, uint64_t nb,
                     uint32_t d, float* d_out);

/* ---- autotuning (no counterpart in the reference: its launch shapes, beam width and hash
 * capacity are compile-time constants, tests/test_t2iend.cu:671-727) --------------------------
 * pg_set_tuning / pg_get_tuning: the tuning later builds on this handle use.
 * pg_autotune: times trial builds of the given data and keeps the fastest choice of search
 * staging rows, resident search warps, visited-set capacity and screened-prune copy-ring depth
 * (coordinate search from the defaults, each candidate timed twice, kept only when it wins by
 * more than 1%).  When d_queries (the training queries behind d_gt, q_i x d per sub-index) and
 * target_recall > 0 are given, it first picks the beam: the smallest L in {64, 96, 128} whose
 * graph reaches target_recall recall@10 (pg_query_search of up to 1000 training queries of the
 * largest sub-index against their exact top-10 in d_gt), else the L with the best recall; p->km
 * is updated.  The tuning is stored in the handle and returned in *out.  A single index is
 * count = 1, node_off = {0, n}, query_off = {0, q}. */
int pg_set_tuning(pg_handle h, const pg_tuning* t);
int pg_get_tuning(pg_handle h, pg_tuning* t);
int pg_autotune(pg_handle h, pg_params* p, const float* d_base, uint32_t d, const uint32_t* d_gt,
                const uint64_t* node_off, const uint64_t* query_off, uint32_t count,
                const float* d_queries, float target_recall, pg_tuning* out);

/* ---- stages: one entry point per reference kernel, device pointers, handle's stream ------ */
/* K0 match_top1_kernel_v0 (Gbuilder.cuh:104-135, launched tests/test_t2iend.cu:976): for each
 * base b that is some query's top-1, row b = gt[w][1..gt_k-2] + 2 tombs where w is the winning
 * query (the lowest id; canonical form of the atomicCAS race); other rows all tomb.
 * out: n x gt_k. */
int pg_match_top1(pg_handle h, const uint32_t* d_gt, uint64_t q, uint32_t gt_k, uint64_t n,
                  uint32_t* d_out);

/* K1+K2 init_pr_lists + fusion_prune_reverse_kernel_v0 (Gbuilder.cuh:1066-1244, launched
 * tests/test_t2iend.cu:987-1001,1062-1077): per node, sort its c candidates by distance,
 * RNG-prune to `pruned`, append reverse edges (ascending source order, first `reverse` kept).
 * Outputs: pruned list n x pruned + counts n; reverse list n x reverse + counts n (clamped).
 * d_sorted (optional, n x c) receives each candidate row after the sort, as the reference
 * sorts the row in place.  evals (optional, host) receives the evaluation count. */
int pg_prune_reverse(pg_handle h, const float* d_base, uint64_t n, uint32_t d,
                     const uint32_t* d_graph, uint32_t c, uint32_t pruned, uint32_t reverse,
                     int strict, uint32_t* d_pruned, uint32_t* d_pruned_num, uint32_t* d_reverse,
                     uint32_t* d_reverse_num, uint32_t* d_sorted, uint64_t* evals);

/* K3 fusion_merge_sort_prune_kernel (Gbuilder.cuh:1467-1601, launched
 * tests/test_t2iend.cu:1010,1083,1130): merge reverse + pruned lists, sort, RNG-prune to
 * `degree`, non-strict fill, tomb padding.  out: n x degree. */
int pg_merge_prune(pg_handle h, const float* d_base, uint64_t n, uint32_t d,
                   const uint32_t* d_pruned, const uint32_t* d_pruned_num, uint32_t pruned,
                   const uint32_t* d_reverse, const uint32_t* d_reverse_num, uint32_t reverse,
                   uint32_t degree, int strict, uint32_t* d_out, uint64_t* evals);

/* K4 link_process_v0_store_base_data (Gsearcher.cuh:890-1066, launched
 * tests/test_t2iend.cu:1051,1096): beam search with every base point as the query over the
 * graph (n x graph_degree).  out: n x (km + kp*kd) ids, parent bit cleared. */
int pg_search(pg_handle h, const float* d_base, uint64_t n, uint32_t d, const uint32_t* d_graph,
              uint32_t graph_degree, uint32_t km, uint32_t kp, uint32_t kd, uint32_t reset_iter,
              uint32_t seed_base, uint32_t max_iters, uint32_t* d_out, uint64_t* evals,
              uint64_t* iters);

/* Same computation as pg_prune_reverse, for callers that cannot allocate device memory: a host
 * application that owns the GPU through its own memory pool and forbids plugins to allocate, or
 * a latency-bound caller that cannot take cudaMalloc's possible device-wide synchronisation.
 * Needs no handle and allocates nothing: the reverse-edge workspace and counters live in a fixed
 * array inside the library's device image (about 4.6 MB, held by every GPU that loads the
 * library until the process exits).  Limits: n <= 32768 and n * pruned <= 1048576, else
 * PG_EINVAL.  Runs on `stream` (a cudaStream_t of the current device), copies the evaluation
 * count and status to the host and synchronises `stream` before returning.  All calls share the
 * array: calls that overlap on the GPU race and must be serialised by the caller.  The first call
 * on a device, and the first after that device's context was reset, looks up the array's device
 * address there; that first call should come before any stream capture on the device.
 * This entry point has no counterpart in the reference. */
int pg_prune_reverse_noalloc(void* stream, const float* d_base, uint64_t n, uint32_t d,
                             const uint32_t* d_graph, uint32_t c, uint32_t pruned,
                             uint32_t reverse, int strict, uint32_t* d_pruned,
                             uint32_t* d_pruned_num, uint32_t* d_reverse, uint32_t* d_reverse_num,
                             uint64_t* evals);

/* Query-time search, search_shared_hashtable (Gsearcher.cuh:108-296): the same beam search over a
 * built graph (n x graph_degree) for nq external query vectors (nq x d, e.g. the other modality),
 * writing the best topk ids of each query's final list (out: nq x topk).  The reference never
 * empties its shared visited set between the queries one warp handles, so its result depends on
 * scheduling; here every query starts from an empty set. */
int pg_query_search(pg_handle h, const float* d_base, uint64_t n, uint32_t d,
                    const uint32_t* d_graph, uint32_t graph_degree, const float* d_queries,
                    uint64_t nq, uint32_t km, uint32_t kp, uint32_t kd, uint32_t reset_iter,
                    uint32_t seed_base, uint32_t max_iters, uint32_t topk, uint32_t* d_out,
                    uint64_t* evals, uint64_t* iters);

/* ---- on-disk formats ----------------------------------------------------------------------- */
/* Raw vectors as read by read_vec_from_file (include/utils.hpp:17-35): headerless, exactly
 * count*elem_size bytes, or with the Big-ANN [u32 n][u32 d] header (README.md:13-21) when
 * `headered` is non-zero (then rows and cols receive the header). */
int pg_read_file(const char* path, int headered, void* dst, uint64_t bytes, uint32_t* rows,
                 uint32_t* cols);
/* SaveGraph (tests/test_t2iend.cu:615-633): [u32 ep][u32 n] then per node [u32 deg][ids],
 * deg = number of non-tomb ids of the row, in row order. */
int pg_save_graph(const char* path, const uint32_t* graph, uint64_t n, uint32_t degree,
                  uint32_t ep);
/* ep of MatchNN (tests/test_t2iend.cu:188-221): per query in order, count gt ids up to and
 * including the first not yet matched one; ep = first id after std::sort by count desc. */
int pg_entry_point(const uint32_t* gt, uint64_t q, uint32_t gt_k, uint64_t n, uint32_t* ep);

#ifdef __cplusplus
}
#endif
#endif /* PARAGRAPH_GB300_H_ */
