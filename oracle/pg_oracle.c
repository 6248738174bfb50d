/*
 * pg_oracle.c -- CPU restatement of ParaGraph's GPU build path (TEST INFRASTRUCTURE ONLY).
 *
 * This file is the correctness oracle for the CUDA kernels in paragraph_gb300/csrc.  It is
 * imported only by tests/, by __graft_entry__.smoke() and by bench.py's CPU-baseline and
 * reference legs.  The product never links it and never falls back to it.
 *
 * It restates, loop for loop, the twelve kernel launches of the reference driver
 * (tests/test_t2iend.cu:974-1139) with these canonical resolutions of the reference's races:
 *   - projection slot winner (Gbuilder.cuh:122 atomicCAS): queries are applied in ascending id
 *     order, i.e. the result of a one-thread launch;
 *   - reverse edges (Gbuilder.cuh:1020-1038 add_reverse): appended in ascending source-node
 *     order, the first R kept, the count clamped to R;
 *   - the shared-memory warp sort (GBitonicSort.cuh:237 used at Gsearcher.cuh:980,1045):
 *     ascending distance, equal distances keep list order (a stable sort);
 *   - the search's never-initialised top-Km slots (Gsearcher.cuh:953-956): id = tomb.
 * Floating-point reduction orders are the reference's two device orders, reproduced with fmaf:
 *   - dist_seq: distance_between (Gbuilder.cuh:785-797), one FMA chain over d = 0..D-1;
 *   - dist_lane: the warp dot product (Gsearcher.cuh:958-976, 1021-1036), 32 lane-strided FMA
 *     chains then a shuffle-down tree 16, 8, 4, 2, 1.
 * Every function counts distance evaluations the way the reference calls them.
 */
#include <float.h>
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define TOMB 0xFFFFFFFFu
#define MASKED_TOMB 0x7FFFFFFFu
#define PARENT_BIT 0x80000000u

/* ---------------------------------------------------------------- distances */

/* distance_between, Gbuilder.cuh:785-797: -(sum_d x[d]*y[d]), one FMA chain in d order. */
static inline float dist_seq(const float* base, uint64_t d, uint32_t x, uint32_t y) {
  const float* a = base + (uint64_t)x * d;
  const float* b = base + (uint64_t)y * d;
  float s = 0.0f;
  for (uint64_t i = 0; i < d; i++) s = fmaf(a[i], b[i], s);
  return -s;
}

/* Warp dot product, Gsearcher.cuh:1021-1036: lane l accumulates q[i]*x[i] for i = l, l+32, ...,
 * then sum += __shfl_down_sync(sum, 16..1); lane 0's value, negated. */
static inline float dist_lane(const float* q, const float* x, uint64_t d) {
  float s[32];
  for (int l = 0; l < 32; l++) s[l] = 0.0f;
  uint64_t full = d / 32;
  for (uint64_t k = 0; k < full; k++) {
    const float* qk = q + k * 32;
    const float* xk = x + k * 32;
    for (int l = 0; l < 32; l++) s[l] = fmaf(qk[l], xk[l], s[l]);
  }
  for (uint64_t i = full * 32; i < d; i++) s[i - full * 32] = fmaf(q[i], x[i], s[i - full * 32]);
  for (int off = 16; off > 0; off >>= 1)
    for (int l = 0; l < off; l++) s[l] = s[l] + s[l + off];
  return -s[0];
}

/* Stable ascending sort of (key, id) pairs: the result of bubble_sort (Gbuilder.cuh:890-902),
 * strict '>' so equal keys keep their order.  Insertion sort has the same result. */
static void stable_sort(float* key, uint32_t* id, uint32_t n) {
  for (uint32_t i = 1; i < n; i++) {
    float k = key[i];
    uint32_t v = id[i];
    uint32_t j = i;
    while (j > 0 && key[j - 1] > k) {
      key[j] = key[j - 1];
      id[j] = id[j - 1];
      j--;
    }
    key[j] = k;
    id[j] = v;
  }
}

/* ---------------------------------------------------------------- K0: projection */

/* match_top1_kernel_v0 (Gbuilder.cuh:104-135) with queries applied in ascending order.
 * For query q with top-1 base b = gt[q][0]: if slot proj[b][0] is still tomb, the query writes
 * gt[q][1..gt_k-1] into slots 0..gt_k-2 and then tomb into slots gt_k-2 and gt_k-1
 * (match_real_degree = gt_k - 1, as launched at tests/test_t2iend.cu:976-979).
 * Queries whose top-1 is tomb are skipped (the reference writes out of bounds there).
 * out: n x gt_k, must be preset to tomb by the caller (tests/test_t2iend.cu:866-870). */
void pgo_match_top1(const uint32_t* gt, uint64_t q, uint32_t gt_k, uint64_t n, uint32_t* out) {
  for (uint64_t i = 0; i < n * gt_k; i++) out[i] = TOMB;
  for (uint64_t qi = 0; qi < q; qi++) {
    const uint32_t* g = gt + qi * gt_k;
    uint32_t b = g[0];
    if (b == TOMB || b >= n) continue;
    uint32_t* row = out + (uint64_t)b * gt_k;
    if (row[0] != TOMB) continue; /* atomicCAS(tomb -> gt[q][1]) fails */
    row[0] = g[1];
    for (uint32_t j = 2; j < gt_k; j++) row[j - 1] = g[j];
    for (uint32_t j = gt_k - 2; j < gt_k; j++) row[j] = TOMB;
  }
}

/* ---------------------------------------------------------------- K2: prune + reverse */

/* fusion_prune_reverse_kernel_v0 (Gbuilder.cuh:1093-1244) for one node b over its candidate
 * row cand[0..c).  Writes the kept list into kept[0..p) and returns the kept count (the value
 * set_prune_number stores; 0 when the sorted first entry is tomb, Gbuilder.cuh:1142-1144).
 * sorted_out (optional) receives the row after the in-place bubble sort (Gbuilder.cuh:1135). */
static uint32_t prune_one(const float* base, uint64_t d, uint32_t b, const uint32_t* cand,
                          uint32_t c, uint32_t p, int strict, uint32_t* kept, uint32_t* sorted_out,
                          uint64_t* evals) {
  float dist[256];
  uint32_t ids[256];
  uint64_t ev = 0;
  for (uint32_t j = 0; j < c; j++) {
    uint32_t id = cand[j];
    ids[j] = id;
    if (id == TOMB || id == b || id == MASKED_TOMB) {
      dist[j] = FLT_MAX;
    } else {
      dist[j] = dist_seq(base, d, b, id);
      ev++;
    }
  }
  stable_sort(dist, ids, c);
  if (sorted_out) memcpy(sorted_out, ids, sizeof(uint32_t) * c);
  uint32_t first = ids[0];
  if (first == TOMB || first == MASKED_TOMB) {
    *evals += ev;
    return 0;
  }
  uint32_t k = 0; /* index of the last kept entry (pruned_graph_neighbor_idx) */
  kept[0] = first;
  uint32_t j = 1;
  int explore = 1;
  for (; explore && j < c; j++) {
    uint32_t cand_id = ids[j];
    if (cand_id == TOMB || cand_id == MASKED_TOMB) break;
    uint32_t ci = 0;
    for (; ci <= k; ci++) {
      ev++;
      if (dist_seq(base, d, cand_id, kept[ci]) < dist[j]) break;
    }
    if (ci > k) {
      k++;
      kept[k] = cand_id;
      if (k == p - 1) {
        explore = 0;
        break;
      }
    }
  }
  /* non-strict fill (Gbuilder.cuh:1201-1239): continue from where the scan stopped */
  if (!strict && k < p - 1) {
    for (uint32_t j2 = j; j2 < c && k < p - 1; j2++) {
      uint32_t x = ids[j2];
      if (x == TOMB || x == b || x == MASKED_TOMB) continue;
      int dup = 0;
      for (uint32_t t = 0; t <= k; t++)
        if (kept[t] == x) {
          dup = 1;
          break;
        }
      if (!dup) {
        k++;
        kept[k] = x;
      }
    }
  }
  *evals += ev;
  return k + 1;
}

/* K1 + K2 over all nodes.  graph: n x c candidate rows (may be NULL when `winner`/`gt` give
 * the phase-1 rows directly).  Outputs: pruned (n x p) + pruned_num (n); reverse (n x r) +
 * reverse_num (n), reverse edges appended in ascending source order (the canonical form of
 * add_reverse, Gbuilder.cuh:1020-1038), count clamped to r.  sorted (optional, n x c) gets
 * each row after the in-place sort.  Returns the number of distance evaluations. */
uint64_t pgo_prune_reverse(const float* base, uint64_t n, uint32_t d, const uint32_t* graph,
                           uint32_t c, uint32_t p, uint32_t r, int strict, uint32_t* pruned,
                           uint32_t* pruned_num, uint32_t* reverse, uint32_t* reverse_num,
                           uint32_t* sorted) {
  uint64_t total = 0;
#pragma omp parallel for schedule(dynamic, 64) reduction(+ : total)
  for (int64_t bi = 0; bi < (int64_t)n; bi++) {
    uint64_t ev = 0;
    uint32_t kept[256];
    uint32_t cnt = prune_one(base, d, (uint32_t)bi, graph + (uint64_t)bi * c, c, p, strict, kept,
                             sorted ? sorted + (uint64_t)bi * c : NULL, &ev);
    pruned_num[bi] = cnt;
    for (uint32_t t = 0; t < cnt; t++) pruned[(uint64_t)bi * p + t] = kept[t];
    total += ev;
  }
  for (uint64_t i = 0; i < n; i++) reverse_num[i] = 0;
  for (uint64_t b = 0; b < n; b++) {
    for (uint32_t t = 0; t < pruned_num[b]; t++) {
      uint32_t dst = pruned[b * p + t];
      uint32_t slot = reverse_num[dst];
      if (slot < r) {
        reverse[(uint64_t)dst * r + slot] = (uint32_t)b;
        reverse_num[dst] = slot + 1;
      }
    }
  }
  return total;
}

/* ---------------------------------------------------------------- K3: merge + prune */

/* fusion_merge_sort_prune_kernel (Gbuilder.cuh:1467-1601) for one node.  The merged list is the
 * reverse list followed by the pruned list (pr_sort_list view, Gbuilder.cuh:1433-1465); the
 * stable sort keeps reverse entries before pruned ones on equal distance. */
static void merge_one(const float* base, uint64_t n, uint64_t d, uint32_t b, const uint32_t* rev,
                      uint32_t rn, const uint32_t* pr, uint32_t pn, uint32_t deg, int strict,
                      uint32_t* out, uint64_t* evals) {
  uint32_t nn = rn + pn;
  if (nn == 0) {
    for (uint32_t i = 0; i < deg; i++) out[i] = TOMB;
    return;
  }
  float dist[256];
  uint32_t ids[256];
  uint64_t ev = 0;
  for (uint32_t i = 0; i < rn; i++) ids[i] = rev[i];
  for (uint32_t i = 0; i < pn; i++) ids[rn + i] = pr[i];
  for (uint32_t i = 0; i < nn; i++) {
    dist[i] = dist_seq(base, d, b, ids[i]);
    ev++;
  }
  stable_sort(dist, ids, nn);
  uint32_t k = 0;
  out[0] = ids[0];
  int explore = 1;
  for (uint32_t j = 1; explore && j < nn; j++) {
    uint32_t x = ids[j];
    uint32_t ci = 0;
    for (; ci <= k; ci++) {
      ev++;
      if (dist_seq(base, d, x, out[ci]) < dist[j]) break;
    }
    if (ci > k) {
      k++;
      out[k] = x;
      if (k == deg - 1) {
        explore = 0;
        break;
      }
    }
  }
  for (uint32_t i = k + 1; i < deg; i++) out[i] = TOMB;
  if (!strict && k < deg - 1) {
    unsigned char added[256];
    memset(added, 0, sizeof(added));
    for (uint32_t i = 0; i <= k; i++) {
      for (uint32_t j = 0; j < nn; j++) {
        if (ids[j] == out[i]) {
          added[j] = 1;
          break;
        }
      }
    }
    for (uint32_t i = 0; i < nn && k < deg - 1; i++) {
      if (added[i]) continue;
      uint32_t x = ids[i];
      if (x != TOMB && x != b && x < n) {
        k++;
        out[k] = x;
      }
    }
    for (uint32_t i = k + 1; i < deg; i++) out[i] = TOMB;
  }
  *evals += ev;
}

uint64_t pgo_merge_prune(const float* base, uint64_t n, uint32_t d, const uint32_t* pruned,
                         const uint32_t* pruned_num, uint32_t p, const uint32_t* reverse,
                         const uint32_t* reverse_num, uint32_t r, uint32_t deg, int strict,
                         uint32_t* out) {
  uint64_t total = 0;
#pragma omp parallel for schedule(dynamic, 64) reduction(+ : total)
  for (int64_t bi = 0; bi < (int64_t)n; bi++) {
    uint64_t ev = 0;
    uint32_t rn = reverse_num[bi] < r ? reverse_num[bi] : r;
    merge_one(base, n, d, (uint32_t)bi, reverse + (uint64_t)bi * r, rn, pruned + (uint64_t)bi * p,
              pruned_num[bi], deg, strict, out + (uint64_t)bi * deg, &ev);
    total += ev;
  }
  return total;
}

/* ---------------------------------------------------------------- K4: beam search */

/* Exact visited set with the semantics of HashTable (Ghashtable.cuh:13-93): key+1 stored,
 * 0 = empty, slot = key & (size-1), linear probing. */
typedef struct {
  uint32_t* slot;
  uint32_t mask;
} vset;

static void vset_clear(vset* v) { memset(v->slot, 0, sizeof(uint32_t) * (v->mask + 1)); }

/* returns 1 when key was absent (and inserts it) */
static int vset_insert(vset* v, uint32_t key) {
  uint32_t s = key & v->mask;
  for (uint32_t probe = 0; probe <= v->mask; probe++) {
    uint32_t cur = v->slot[s];
    if (cur == 0) {
      v->slot[s] = key + 1;
      return 1;
    }
    if (cur == key + 1) return 0;
    s = (s + 1) & v->mask;
  }
  return 0; /* full: cannot happen with the capacity chosen by the caller */
}

typedef struct {
  uint64_t evals;
  uint64_t iters;
  uint32_t max_iters_hit;
} search_stats;

/* link_process_v0_store_base_data (Gsearcher.cuh:890-1066) for one base point used as query.
 * out receives the km + kp*kd ids with the parent bit cleared. */
static void search_one(const float* base, uint64_t n, uint64_t d, const uint32_t* graph,
                       uint32_t deg, uint32_t km, uint32_t kp, uint32_t kd, uint32_t reset_iter,
                       uint32_t seed_base, uint64_t max_iters, const float* q, uint32_t out_width,
                       vset* vs, float* dist, uint32_t* ids, uint32_t* out, search_stats* st) {
  const uint32_t L = km + kp * kd;
  for (uint32_t i = 0; i < kp * kd; i++) ids[km + i] = (uint32_t)((seed_base + (uint64_t)i) % n);
  for (uint32_t i = 0; i < km; i++) {
    dist[i] = FLT_MAX;
    ids[i] = TOMB;
  }
  for (uint32_t i = km; i < L; i++) {
    dist[i] = dist_lane(q, base + (uint64_t)ids[i] * d, d);
    st->evals++;
  }
  stable_sort(dist, ids, L);
  vset_clear(vs);
  for (uint32_t i = 0; i < km; i++) vset_insert(vs, ids[i] & MASKED_TOMB);
  uint32_t iter = 0;
  uint64_t total_iters = 0;
  uint32_t explore[64];
  for (;;) {
    /* collect_top_p_normal (Gsearcher.cuh:75-106): first kp unexplored of the top km */
    uint32_t found = 0;
    for (uint32_t i = 0; i < km && found < kp; i++) {
      if ((ids[i] & PARENT_BIT) == 0) {
        explore[found++] = ids[i];
        ids[i] |= PARENT_BIT;
      }
    }
    if (found == 0) break;
    for (uint32_t e = found; e < kp; e++) explore[e] = TOMB;
    if (++total_iters > max_iters) {
      st->max_iters_hit = 1;
      break;
    }
    for (uint32_t e = 0; e < kp; e++) {
      for (uint32_t nb = 0; nb < kd; nb++) {
        ids[km + e * kd + nb] =
            explore[e] != TOMB ? graph[(uint64_t)explore[e] * deg + nb] : TOMB;
      }
    }
    for (uint32_t j = 0; j < kp * kd; j++) {
      uint32_t node = ids[km + j];
      if (node != TOMB && vset_insert(vs, node)) {
        dist[km + j] = dist_lane(q, base + (uint64_t)node * d, d);
        st->evals++;
      } else {
        dist[km + j] = FLT_MAX;
      }
    }
    stable_sort(dist, ids, L);
    iter++;
    if (iter == reset_iter) {
      vset_clear(vs);
      for (uint32_t i = 0; i < km; i++) vset_insert(vs, ids[i] & MASKED_TOMB);
      iter = 0;
    }
  }
  st->iters += total_iters;
  for (uint32_t i = 0; i < L && i < out_width; i++) out[i] = ids[i] & MASKED_TOMB;
}

static uint32_t pow2_at_least(uint32_t x) {
  uint32_t p = 1;
  while (p < x) p <<= 1;
  return p;
}

/* Returns evaluations; *iters_out (optional) gets the total number of loop iterations and
 * *cap_hit is set when any query reached max_iters. */
uint64_t pgo_search(const float* base, uint64_t n, uint32_t d, const uint32_t* graph,
                    uint32_t deg, uint32_t km, uint32_t kp, uint32_t kd, uint32_t reset_iter,
                    uint32_t seed_base, uint64_t max_iters, uint64_t q_begin, uint64_t q_end,
                    uint32_t* out, uint64_t* iters_out, uint32_t* cap_hit) {
  const uint32_t L = km + kp * kd;
  const uint32_t cap = pow2_at_least(2 * (km + (reset_iter + 1) * kp * kd) + 64);
  uint64_t ev_total = 0, it_total = 0;
  uint32_t hit = 0;
#pragma omp parallel reduction(+ : ev_total, it_total) reduction(| : hit)
  {
    vset vs;
    vs.slot = (uint32_t*)malloc(sizeof(uint32_t) * cap);
    vs.mask = cap - 1;
    float* dist = (float*)malloc(sizeof(float) * L);
    uint32_t* ids = (uint32_t*)malloc(sizeof(uint32_t) * L);
    search_stats st = {0, 0, 0};
#pragma omp for schedule(dynamic, 16)
    for (int64_t qi = (int64_t)q_begin; qi < (int64_t)q_end; qi++) {
      search_one(base, n, d, graph, deg, km, kp, kd, reset_iter, seed_base, max_iters,
                 base + (uint64_t)qi * d, L, &vs, dist, ids,
                 out + (uint64_t)(qi - (int64_t)q_begin) * L, &st);
    }
    ev_total += st.evals;
    it_total += st.iters;
    hit |= st.max_iters_hit;
    free(vs.slot);
    free(dist);
    free(ids);
  }
  if (iters_out) *iters_out = it_total;
  if (cap_hit) *cap_hit = hit;
  return ev_total;
}

/* search_shared_hashtable (Gsearcher.cuh:108-296): the same search for external query vectors,
 * writing the first topk ids of each final list; the visited set starts empty for every query. */
uint64_t pgo_query_search(const float* base, uint64_t n, uint32_t d, const uint32_t* graph,
                          uint32_t deg, const float* queries, uint64_t nq, uint32_t km,
                          uint32_t kp, uint32_t kd, uint32_t reset_iter, uint32_t seed_base,
                          uint64_t max_iters, uint32_t topk, uint32_t* out, uint64_t* iters_out) {
  const uint32_t L = km + kp * kd;
  const uint32_t cap = pow2_at_least(2 * (km + (reset_iter + 1) * kp * kd) + 64);
  uint64_t ev_total = 0, it_total = 0;
#pragma omp parallel reduction(+ : ev_total, it_total)
  {
    vset vs;
    vs.slot = (uint32_t*)malloc(sizeof(uint32_t) * cap);
    vs.mask = cap - 1;
    float* dist = (float*)malloc(sizeof(float) * L);
    uint32_t* ids = (uint32_t*)malloc(sizeof(uint32_t) * L);
    search_stats st = {0, 0, 0};
#pragma omp for schedule(dynamic, 16)
    for (int64_t qi = 0; qi < (int64_t)nq; qi++) {
      search_one(base, n, d, graph, deg, km, kp, kd, reset_iter, seed_base, max_iters,
                 queries + (uint64_t)qi * d, topk, &vs, dist, ids, out + (uint64_t)qi * topk,
                 &st);
    }
    ev_total += st.evals;
    it_total += st.iters;
    free(vs.slot);
    free(dist);
    free(ids);
  }
  if (iters_out) *iters_out = it_total;
  return ev_total;
}

/* ---------------------------------------------------------------- whole build */

typedef struct {
  uint32_t gt_k, proj_degree, proj_pruned, proj_reverse;
  uint32_t degree, link_reverse, link_rounds;
  uint32_t km, kp, kd, reset_iter, seed_base;
  uint64_t max_iters;
} pgo_params;

typedef struct {
  uint64_t evals_proj_prune, evals_proj_merge;
  uint64_t evals_search[4], evals_prune[4], evals_merge[4];
  uint64_t iters_search[4];
  uint64_t evals_total;
  uint32_t cap_hit;
} pgo_stats;

/* The K0..K11 sequence of tests/test_t2iend.cu:974-1139 with runtime sizes.
 * proj_out: n x proj_degree.  graph_out: n x degree.  search_out (optional): n x L of the
 * last link round's search. */
int pgo_build(const pgo_params* P, const float* base, uint64_t n, uint32_t d, const uint32_t* gt,
              uint64_t q, uint32_t* proj_out, uint32_t* graph_out, uint32_t* search_out,
              pgo_stats* st) {
  memset(st, 0, sizeof(*st));
  const uint32_t gk = P->gt_k;
  const uint32_t L = P->km + P->kp * P->kd;
  uint32_t* cand = (uint32_t*)malloc(sizeof(uint32_t) * n * gk);
  uint32_t pmax = P->proj_pruned > P->degree ? P->proj_pruned : P->degree;
  uint32_t rmax = P->proj_reverse > P->link_reverse ? P->proj_reverse : P->link_reverse;
  uint32_t* pruned = (uint32_t*)malloc(sizeof(uint32_t) * n * pmax);
  uint32_t* pnum = (uint32_t*)malloc(sizeof(uint32_t) * n);
  uint32_t* rev = (uint32_t*)malloc(sizeof(uint32_t) * n * rmax);
  uint32_t* rnum = (uint32_t*)malloc(sizeof(uint32_t) * n);
  uint32_t* sres = (uint32_t*)malloc(sizeof(uint32_t) * n * L);
  uint32_t* cur = (uint32_t*)malloc(sizeof(uint32_t) * n * P->degree);
  if (!cand || !pruned || !pnum || !rev || !rnum || !sres || !cur) return -1;

  pgo_match_top1(gt, q, gk, n, cand);
  st->evals_proj_prune = pgo_prune_reverse(base, n, d, cand, gk, P->proj_pruned, P->proj_reverse,
                                           0, pruned, pnum, rev, rnum, NULL);
  st->evals_proj_merge = pgo_merge_prune(base, n, d, pruned, pnum, P->proj_pruned, rev, rnum,
                                         P->proj_reverse, P->proj_degree, 0, proj_out);
  const uint32_t* g = proj_out;
  uint32_t gdeg = P->proj_degree;
  for (uint32_t round = 0; round < P->link_rounds && round < 4; round++) {
    uint64_t it = 0;
    uint32_t hit = 0;
    st->evals_search[round] = pgo_search(base, n, d, g, gdeg, P->km, P->kp, P->kd, P->reset_iter,
                                         P->seed_base, P->max_iters, 0, n, sres, &it, &hit);
    st->iters_search[round] = it;
    st->cap_hit |= hit;
    st->evals_prune[round] = pgo_prune_reverse(base, n, d, sres, L, P->degree, P->link_reverse, 1,
                                               pruned, pnum, rev, rnum, NULL);
    st->evals_merge[round] = pgo_merge_prune(base, n, d, pruned, pnum, P->degree, rev, rnum,
                                             P->link_reverse, P->degree, 1, cur);
    memcpy(graph_out, cur, sizeof(uint32_t) * n * P->degree);
    g = graph_out;
    gdeg = P->degree;
  }
  if (search_out) memcpy(search_out, sres, sizeof(uint32_t) * n * L);
  st->evals_total = st->evals_proj_prune + st->evals_proj_merge;
  for (int r = 0; r < 4; r++) st->evals_total += st->evals_search[r] + st->evals_prune[r] + st->evals_merge[r];
  free(cand);
  free(pruned);
  free(pnum);
  free(rev);
  free(rnum);
  free(sres);
  free(cur);
  return 0;
}

/* Distance helpers exported for tests of the two reduction orders. */
float pgo_dist_seq(const float* base, uint64_t d, uint32_t x, uint32_t y) {
  return dist_seq(base, d, x, y);
}
float pgo_dist_lane(const float* q, const float* x, uint64_t d) { return dist_lane(q, x, d); }

int pgo_num_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}
