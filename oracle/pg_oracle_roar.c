/*
 * pg_oracle_roar.c -- CPU restatement of ParaGraph's CPU RoarGraph path and final fusion
 * (TEST INFRASTRUCTURE ONLY; part of libpg_oracle.so, imported by tests/ only).
 *
 * Follows tests/test_t2iend.cu:
 *   compare      :31-80    AVX-512 inner product, restated in its exact FP32 order (dist_avx);
 *   RNGPrune     :99-177   occlusion prune over a (distance, id)-sorted list;
 *   MatchSup     :365-488  one supplementary bipartite round (query -> its topn-th base);
 *   FusionNN     :490-537  union of the rounds, strict prune to 2*M_nn;
 *   FusionFinal  :539-613  union with the GPU projection and link graph, strict prune to M_final.
 * Canonical resolutions of the reference's races and unordered containers:
 *   - MatchSup's reverse appends (degrees[].fetch_add under OpenMP) happen in ascending query
 *     order: a base keeps the first 128 - M_nn sources in that order;
 *   - a merged MatchSup list short enough to skip the final prune is written in ascending id
 *     order (the reference writes std::unordered_set iteration order; every consumer of the list
 *     sorts or de-duplicates it, so the order carries no information).
 * Graphs are CSR: off[n + 1] (uint64) and ids.  D must be a multiple of 4 (the reference's
 * 4-wide masked tail, :66-72, is only reached otherwise).
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

/* compare (tests/test_t2iend.cu:31-80): 16 FMA lanes over 16-wide chunks, lanes folded 8+8, an
 * 8-wide FMA step, folded 4+4, a 4-wide FMA step, then the two horizontal adds:
 * ((s0 + s1) + (s2 + s3)); negated. */
static float dist_avx(const float* a, const float* b, uint64_t d) {
  float s16[16], s8[8], s4[4];
  for (int l = 0; l < 16; l++) s16[l] = 0.0f;
  uint64_t i = 0;
  for (; i + 16 <= d; i += 16)
    for (int l = 0; l < 16; l++) s16[l] = fmaf(a[i + l], b[i + l], s16[l]);
  for (int l = 0; l < 8; l++) s8[l] = s16[8 + l] + s16[l];
  if (d - i >= 8) {
    for (int l = 0; l < 8; l++) s8[l] = fmaf(a[i + l], b[i + l], s8[l]);
    i += 8;
  }
  for (int l = 0; l < 4; l++) s4[l] = s8[4 + l] + s8[l];
  if (d - i >= 4) {
    for (int l = 0; l < 4; l++) s4[l] = fmaf(a[i + l], b[i + l], s4[l]);
    i += 4;
  }
  return -((s4[0] + s4[1]) + (s4[2] + s4[3]));
}

float pgo_dist_avx(const float* a, const float* b, uint64_t d) { return dist_avx(a, b, d); }

/* SimpleNeighbor order (:82-91): distance, then id. */
static int nb_less(float da, uint32_t ia, float db, uint32_t ib) {
  return da < db || (da == db && ia < ib);
}

static void sort_nb(float* dist, uint32_t* id, uint32_t c) {
  for (uint32_t i = 1; i < c; i++) {
    const float k = dist[i];
    const uint32_t v = id[i];
    uint32_t j = i;
    while (j > 0 && nb_less(k, v, dist[j - 1], id[j - 1])) {
      dist[j] = dist[j - 1];
      id[j] = id[j - 1];
      j--;
    }
    dist[j] = k;
    id[j] = v;
  }
}

static int contains(const uint32_t* a, uint32_t k, uint32_t x) {
  for (uint32_t i = 0; i < k; i++)
    if (a[i] == x) return 1;
  return 0;
}

/* one scan of RNGPrune's occlusion loop (:115-139 and :142-165) from the first non-target */
static void rng_scan(const float* base, uint64_t d, uint32_t M, const float* dist,
                     const uint32_t* id, uint32_t c, uint32_t target, uint32_t* res,
                     uint32_t* k) {
  uint32_t start = 0;
  while (start < c && id[start] == target) start++;
  while (*k < M && ++start < c) {
    const uint32_t p = id[start];
    int occl = 0;
    for (uint32_t i = 0; i < *k; i++) {
      if (p == res[i]) {
        occl = 1;
        break;
      }
      if (dist_avx(base + (uint64_t)p * d, base + (uint64_t)res[i] * d, d) < dist[start]) {
        occl = 1;
        break;
      }
    }
    if (!occl && p != target && !contains(res, *k, p)) res[(*k)++] = p;
  }
}

/* RNGPrune (:99-177) over the sorted list (dist, id)[0..c); returns the kept count. */
static uint32_t rng_prune(const float* base, uint64_t d, uint64_t n, uint32_t M,
                          const float* dist, const uint32_t* id, uint32_t c, uint32_t target,
                          int strict, uint32_t* res) {
  uint32_t start = 0;
  while (start < c && id[start] == target) start++;
  if (start == c) return 0;
  uint32_t k = 0;
  res[k++] = id[start];
  rng_scan(base, d, M, dist, id, c, target, res, &k);
  rng_scan(base, d, M, dist, id, c, target, res, &k); /* the "double check" pass */
  if (!strict) {
    for (uint32_t i = 1; i < c && k < M; i++) {
      const uint32_t x = id[i];
      if (!contains(res, k, x) && x < n && x != target) res[k++] = x;
    }
  }
  return k;
}

static int cmp_u32(const void* a, const void* b) {
  const uint32_t x = *(const uint32_t*)a, y = *(const uint32_t*)b;
  return x < y ? -1 : x > y;
}

/* Rows (stride, counts) -> CSR; returns the id count or -1 when cap is too small. */
static long long compact_rows(const uint32_t* rows, const uint32_t* cnt, uint64_t stride,
                              uint64_t n, uint64_t* off, uint32_t* ids, uint64_t cap) {
  uint64_t o = 0;
  for (uint64_t b = 0; b < n; b++) {
    off[b] = o;
    if (o + cnt[b] > cap) return -1;
    memcpy(ids + o, rows + b * stride, sizeof(uint32_t) * cnt[b]);
    o += cnt[b];
  }
  off[n] = o;
  return (long long)o;
}

/* MatchSup (:365-488) for round topn.  gt: q x n_ctr.  Output CSR (off: n + 1; ids: capacity
 * cap).  Returns the number of ids written, or -1 when cap is too small.  The per-query prunes
 * and per-base merges run in parallel; the reverse appends run in ascending query order. */
long long pgo_match_sup(const float* base, uint64_t n, uint32_t d, const uint32_t* gt,
                        uint64_t q, uint32_t n_ctr, uint32_t topn, uint32_t m_nn, uint64_t* off,
                        uint32_t* ids, uint64_t cap) {
  const uint32_t maxdeg = 128 - m_nn;
  uint32_t* match = (uint32_t*)malloc(sizeof(uint32_t) * q);
  uint8_t* claimed = (uint8_t*)calloc(n, 1);
  for (uint64_t qi = 0; qi < q; qi++) { /* :378-392 */
    match[qi] = TOMB;
    if (topn >= n_ctr) continue;
    const uint32_t nn = gt[qi * n_ctr + topn];
    if (nn >= n || claimed[nn]) continue;
    claimed[nn] = 1;
    match[qi] = nn;
  }
  uint32_t* qlist = (uint32_t*)malloc(sizeof(uint32_t) * q * m_nn); /* per query */
  uint32_t* qcnt = (uint32_t*)calloc(q, sizeof(uint32_t));
#pragma omp parallel
  {
    float dist[256];
    uint32_t cid[256];
#pragma omp for schedule(dynamic, 64)
    for (int64_t qi = 0; qi < (int64_t)q; qi++) { /* :407-430 */
      const uint32_t cur = match[qi];
      if (cur >= n) continue;
      uint32_t c = 0;
      for (uint32_t j = 0; j < n_ctr; j++) {
        const uint32_t b = gt[(uint64_t)qi * n_ctr + j];
        if (b >= n) break;
        if (b == cur || contains(cid, c, b)) continue;
        cid[c] = b;
        dist[c] = dist_avx(base + (uint64_t)b * d, base + (uint64_t)cur * d, d);
        c++;
      }
      sort_nb(dist, cid, c);
      qcnt[qi] = rng_prune(base, d, n, m_nn, dist, cid, c, cur, 0,
                           qlist + (uint64_t)qi * m_nn);
    }
  }
  uint32_t* plist = (uint32_t*)malloc(sizeof(uint32_t) * n * m_nn); /* match_graph rows */
  uint32_t* pcnt = (uint32_t*)calloc(n, sizeof(uint32_t));
  uint32_t* tmp = (uint32_t*)malloc(sizeof(uint32_t) * n * maxdeg);
  uint32_t* deg = (uint32_t*)calloc(n, sizeof(uint32_t));
  uint8_t* full = (uint8_t*)calloc(n, 1);
  for (uint64_t qi = 0; qi < q; qi++) { /* :431-440, ascending query order */
    const uint32_t cur = match[qi];
    if (cur >= n) continue;
    const uint32_t* res = qlist + qi * m_nn;
    for (uint32_t i = 0; i < qcnt[qi]; i++) {
      const uint32_t des = res[i];
      if (full[des]) continue;
      const uint32_t cd = deg[des]++;
      if (cd < maxdeg)
        tmp[(uint64_t)des * maxdeg + cd] = cur;
      else if (cd == maxdeg)
        full[des] = 1;
    }
    memcpy(plist + (uint64_t)cur * m_nn, res, sizeof(uint32_t) * qcnt[qi]);
    pcnt[cur] = qcnt[qi];
  }
  uint32_t* rows = (uint32_t*)malloc(sizeof(uint32_t) * n * m_nn);
  uint32_t* rcnt = (uint32_t*)calloc(n, sizeof(uint32_t));
#pragma omp parallel
  {
    float dist[256];
    uint32_t cid[256];
    uint32_t merged[128];
#pragma omp for schedule(dynamic, 64)
    for (int64_t b = 0; b < (int64_t)n; b++) { /* :449-475 */
      uint32_t c = 0;
      for (uint32_t i = 0; i < pcnt[b]; i++) {
        const uint32_t x = plist[(uint64_t)b * m_nn + i];
        if (!contains(merged, c, x)) merged[c++] = x;
      }
      const uint32_t a = deg[b] < maxdeg ? deg[b] : maxdeg;
      for (uint32_t i = 0; i < a; i++) {
        const uint32_t x = tmp[(uint64_t)b * maxdeg + i];
        if (!contains(merged, c, x)) merged[c++] = x;
      }
      uint32_t* out = rows + (uint64_t)b * m_nn;
      if (c > m_nn) {
        for (uint32_t i = 0; i < c; i++) {
          cid[i] = merged[i];
          dist[i] = dist_avx(base + (uint64_t)merged[i] * d, base + (uint64_t)b * d, d);
        }
        sort_nb(dist, cid, c);
        rcnt[b] = rng_prune(base, d, n, m_nn, dist, cid, c, (uint32_t)b, 1, out);
      } else {
        qsort(merged, c, sizeof(uint32_t), cmp_u32);
        memcpy(out, merged, sizeof(uint32_t) * c);
        rcnt[b] = c;
      }
    }
  }
  const long long ret = compact_rows(rows, rcnt, m_nn, n, off, ids, cap);
  free(match);
  free(claimed);
  free(qlist);
  free(qcnt);
  free(plist);
  free(pcnt);
  free(tmp);
  free(deg);
  free(full);
  free(rows);
  free(rcnt);
  return ret;
}

/* Candidates of one node: the listed ids in order, skipping repeats, ids >= n and (when
 * skip_self) the node itself; returns the new count. */
static uint32_t gather(const uint32_t* src, uint64_t len, uint64_t n, uint32_t self, int skip_self,
                       uint32_t* cid, uint32_t c) {
  for (uint64_t i = 0; i < len; i++) {
    const uint32_t x = src[i];
    if (x >= n || (skip_self && x == self) || contains(cid, c, x)) continue;
    cid[c++] = x;
  }
  return c;
}

/* FusionNN (:490-537) with an empty top-NN graph (MatchNN's graph-building loop is commented out
 * in the reference, :234-306, so it returns empty lists): union of the `rounds` supply graphs
 * (CSR each; round r's offsets at sup_off + r*(n+1), ids at sup_ids + sup_base[r]), strict
 * RNGPrune to 2*m_nn.  Output CSR as for pgo_match_sup. */
long long pgo_fusion_nn(const float* base, uint64_t n, uint32_t d, uint32_t m_nn,
                        uint32_t rounds, const uint64_t* sup_off, const uint32_t* sup_ids,
                        const uint64_t* sup_base, uint64_t* off, uint32_t* ids, uint64_t cap) {
  const uint32_t M = 2 * m_nn;
  uint64_t ccap = 0;
  for (uint64_t b = 0; b < n; b++) {
    uint64_t t = 0;
    for (uint32_t r = 0; r < rounds; r++)
      t += sup_off[r * (n + 1) + b + 1] - sup_off[r * (n + 1) + b];
    if (t > ccap) ccap = t;
  }
  uint32_t* rows = (uint32_t*)malloc(sizeof(uint32_t) * n * M);
  uint32_t* rcnt = (uint32_t*)calloc(n, sizeof(uint32_t));
#pragma omp parallel
  {
    float* dist = (float*)malloc(sizeof(float) * (ccap + 1));
    uint32_t* cid = (uint32_t*)malloc(sizeof(uint32_t) * (ccap + 1));
#pragma omp for schedule(dynamic, 64)
    for (int64_t b = 0; b < (int64_t)n; b++) {
      uint32_t c = 0;
      for (uint32_t r = 0; r < rounds; r++) {
        const uint64_t* so = sup_off + r * (n + 1);
        c = gather(sup_ids + sup_base[r] + so[b], so[b + 1] - so[b], n, (uint32_t)b, 1, cid, c);
      }
      for (uint32_t i = 0; i < c; i++)
        dist[i] = dist_avx(base + (uint64_t)b * d, base + (uint64_t)cid[i] * d, d);
      sort_nb(dist, cid, c);
      rcnt[b] = rng_prune(base, d, n, M, dist, cid, c, (uint32_t)b, 1, rows + (uint64_t)b * M);
    }
    free(dist);
    free(cid);
  }
  const long long ret = compact_rows(rows, rcnt, M, n, off, ids, cap);
  free(rows);
  free(rcnt);
  return ret;
}

/* FusionFinal (:539-613).  bip: the FusionNN graph (CSR); supply: n x m_supply (the GPU
 * projection); link: n x m_link (the GPU graph).  A node's final list is its bipartite ids (first
 * occurrences, not itself, < n) followed by the strict RNGPrune (to m_final) of the union
 * bipartite + link + supply that are not already listed, up to m_final - |bipartite| of them --
 * an unsigned difference: when the bipartite ids outnumber m_final it wraps, and every pruned id
 * not already listed is appended (:599-606). */
long long pgo_fusion_final(const float* base, uint64_t n, uint32_t d, uint32_t m_supply,
                           uint32_t m_link, uint32_t m_final, const uint32_t* supply,
                           const uint64_t* bip_off, const uint32_t* bip_ids,
                           const uint32_t* link, uint64_t* off, uint32_t* ids, uint64_t cap) {
  uint64_t bmax = 0;
  for (uint64_t b = 0; b < n; b++)
    if (bip_off[b + 1] - bip_off[b] > bmax) bmax = bip_off[b + 1] - bip_off[b];
  const uint64_t ccap = bmax + m_link + m_supply + 1;
  const uint64_t stride = bmax + m_final;
  uint32_t* rows = (uint32_t*)malloc(sizeof(uint32_t) * n * stride);
  uint32_t* rcnt = (uint32_t*)calloc(n, sizeof(uint32_t));
#pragma omp parallel
  {
    float* dist = (float*)malloc(sizeof(float) * ccap);
    uint32_t* cid = (uint32_t*)malloc(sizeof(uint32_t) * ccap);
    uint32_t* res = (uint32_t*)malloc(sizeof(uint32_t) * (m_final + 1));
#pragma omp for schedule(dynamic, 64)
    for (int64_t bi = 0; bi < (int64_t)n; bi++) {
      const uint64_t b = (uint64_t)bi;
      uint32_t* fin = rows + b * stride;
      uint32_t c = gather(bip_ids + bip_off[b], bip_off[b + 1] - bip_off[b], n, (uint32_t)b, 1,
                          cid, 0);
      const uint32_t nbip = c;
      memcpy(fin, cid, sizeof(uint32_t) * nbip);
      c = gather(link + b * m_link, m_link, n, (uint32_t)b, 0, cid, c); /* self not skipped */
      c = gather(supply + b * m_supply, m_supply, n, (uint32_t)b, 1, cid, c);
      for (uint32_t i = 0; i < c; i++)
        dist[i] = dist_avx(base + b * d, base + (uint64_t)cid[i] * d, d);
      sort_nb(dist, cid, c);
      const uint32_t k = rng_prune(base, d, n, m_final, dist, cid, c, (uint32_t)b, 1, res);
      const uint64_t slots = m_final >= nbip ? (uint64_t)(m_final - nbip) : UINT64_MAX;
      uint32_t nf = nbip, added = 0;
      for (uint32_t i = 0; i < k; i++) {
        if (added >= slots) break;
        if (!contains(fin, nbip, res[i])) {
          fin[nf++] = res[i];
          added++;
        }
      }
      rcnt[b] = nf;
    }
    free(dist);
    free(cid);
    free(res);
  }
  const long long ret = compact_rows(rows, rcnt, stride, n, off, ids, cap);
  free(rows);
  free(rcnt);
  return ret;
}

/* ---------------------------------------------------------------- ground truth */

static int gt_better(double a, uint32_t ia, double b, uint32_t ib) {
  return a > b || (a == b && ia < ib);
}

/* Exact inner-product top-k (the definition pg_ground_truth implements): for each query the k
 * base ids with the largest FP64 inner product (sequential FMA over d), ties to the lower id,
 * best first; tomb past n. */
void pgo_ground_truth(const float* base, uint64_t n, uint32_t d, const float* queries,
                      uint64_t nq, uint32_t k, uint32_t* out) {
#pragma omp parallel
  {
    double* hs = (double*)malloc(sizeof(double) * (k + 1));
    uint32_t* hi = (uint32_t*)malloc(sizeof(uint32_t) * (k + 1));
#pragma omp for schedule(dynamic, 4)
    for (int64_t qi = 0; qi < (int64_t)nq; qi++) {
      const float* q = queries + (uint64_t)qi * d;
      uint32_t cnt = 0; /* sorted best-first list of the best k so far */
      for (uint64_t x = 0; x < n; x++) {
        const float* r = base + x * d;
        double s = 0.0;
        for (uint32_t j = 0; j < d; j++) s = fma((double)q[j], (double)r[j], s);
        if (cnt == k && !gt_better(s, (uint32_t)x, hs[k - 1], hi[k - 1])) continue;
        uint32_t pos = cnt < k ? cnt : k - 1;
        while (pos > 0 && gt_better(s, (uint32_t)x, hs[pos - 1], hi[pos - 1])) {
          hs[pos] = hs[pos - 1];
          hi[pos] = hi[pos - 1];
          pos--;
        }
        hs[pos] = s;
        hi[pos] = (uint32_t)x;
        if (cnt < k) cnt++;
      }
      for (uint32_t i = 0; i < k; i++) out[(uint64_t)qi * k + i] = i < cnt ? hi[i] : TOMB;
    }
    free(hs);
    free(hi);
  }
}
