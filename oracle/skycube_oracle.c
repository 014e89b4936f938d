/*
 * CPU oracle for the skycube hot path -- TEST INFRASTRUCTURE ONLY.
 *
 * Only tests/, the smoke check and the CPU-baseline leg of the benchmark may
 * load this library, and only to check or time against the CUDA path; the
 * product never calls it.
 *
 * It restates, in plain C with OpenMP, the skycube semantics of the suite's
 * STSC algorithm (the "-c" ground truth, src/main.h:125-146):
 *
 *   - lattice order: cuboids by descending popcount (get_tds_list,
 *     src/utilities/lattice_utilities.cpp:10-18), levels above max_d skipped
 *     (src/stsc/HybridCube.cpp:145-148);
 *   - candidate set of a cuboid = skyline + extended skyline of its parent
 *     with the fewest such points, or of the full space when the first parent
 *     was not computed (src/stsc/HybridCube.cpp:154-166, findMinParent
 *     :242-253; parents listed as in generate_lattice,
 *     src/utilities/lattice_utilities.cpp:52-79);
 *   - dominance on subspace S (DominateLeft_array, src/utilities/dt_avx2.h:
 *     550-640): q dominates p iff q[k] <= p[k] for all k in S and q[k] < p[k]
 *     for some k in S; q strictly dominates p iff q[k] < p[k] for all k in S.
 *     Skyline = not dominated; extended skyline = dominated but not strictly
 *     dominated (MommyQ::Execute, src/hybrid/mommyq.cpp:50-61).
 *
 * Pruning devices kept from the reference's Hybrid skyline (MommyQ,
 * src/hybrid/mommyq.cpp): a block-wise sort-filter order by median-partition
 * level and Manhattan norm, and median-partition masks that skip points
 * worse than the median where the tested point is not (canskip_partition,
 * src/utilities/SubTuple.h:69-73). Two deliberate differences: no priority-
 * queue prefilter (src/utilities/pq_filter.h:418-505; it only prunes work),
 * and no early stop at a peer with an EQUAL float norm (mommyq.cpp:104):
 * float rounding can make a dominator's norm equal to the dominated point's,
 * so equal-norm peers are compared in both directions, which is exact for
 * every input.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef struct {
  uint32_t *ids;
  uint64_t n;
} idlist;

typedef struct {
  int d;
  idlist *sky; /* indexed by cuboid mask, 1 .. 2^d-1 */
  idlist *ext;
} oracle_result;

static int cmp_float(const void *a, const void *b) {
  float x = *(const float *)a, y = *(const float *)b;
  return (x < y) ? -1 : (x > y);
}

/*
 * Skyline and extended skyline of the candidates cand[0..m) on subspace S.
 * status[i] = 0 skyline, 1 extended skyline, 2 strictly dominated.
 *
 * Block-wise sort-filter skyline as in MommyQ::skyline
 * (src/hybrid/mommyq.cpp:227-282): points sorted by (median-partition
 * level, partition mask, Manhattan norm) are processed in blocks of
 * ALPHA; each point of a block is compared with every confirmed point
 * (skyline or extended skyline of earlier blocks) whose partition can
 * dominate it (compare_to_skyline_points, :126-177), then with its peers in
 * the block (compare_to_peers, :63-116). Comparing with confirmed points is
 * enough: if a pruned q dominates p, the confirmed point that strictly
 * dominates q strictly dominates p. Exactness against float rounding of the
 * norm: a block never splits a run of equal (mask, norm) and such peers are
 * compared in both directions.
 */
#define ALPHA 1024

typedef struct {
  uint32_t level_mask; /* popcount << 16 | mask */
  float f;
  uint32_t pos;
} sort_key;

static int cmp_sort_key(const void *a, const void *b) {
  const sort_key *x = (const sort_key *)a, *y = (const sort_key *)b;
  if (x->level_mask != y->level_mask) return x->level_mask < y->level_mask ? -1 : 1;
  if (x->f < y->f) return -1;
  if (x->f > y->f) return 1;
  return (x->pos < y->pos) ? -1 : (x->pos > y->pos);
}

static inline int dominates_packed(const float *q, const float *p, int k) {
  int lt = 0, le = 0;
  for (int j = 0; j < k; ++j) {
    le += (q[j] <= p[j]);
    lt += (q[j] < p[j]);
  }
  if (le != k || lt == 0) return 0;
  return (lt == k) ? 2 : 1;
}

static void skyline_ext(const float *rows, int d, const uint32_t *cand,
                        uint64_t m, uint32_t S, int threads, uint8_t *status) {
  int dims[32], k = 0;
  for (int j = 0; j < d; ++j)
    if (S & (1u << j)) dims[k++] = j;
  if (m == 0) return;

  /* Median of every active dimension over the candidates
   * (MommyQ::PartitionMedian, src/hybrid/mommyq.cpp:284-321). */
  float med[32];
  float *col = (float *)malloc(sizeof(float) * m);
  for (int j = 0; j < k; ++j) {
    for (uint64_t i = 0; i < m; ++i) col[i] = rows[(size_t)cand[i] * d + dims[j]];
    qsort(col, m, sizeof(float), cmp_float);
    med[j] = col[m / 2];
  }
  free(col);

  sort_key *ord = (sort_key *)malloc(sizeof(sort_key) * m);
  for (uint64_t i = 0; i < m; ++i) {
    const float *r = rows + (size_t)cand[i] * d;
    float s = 0.0f;
    uint32_t mk = 0;
    for (int j = 0; j < k; ++j) {
      s += r[dims[j]];
      if (med[j] < r[dims[j]]) mk |= 1u << j; /* worse than the median */
    }
    ord[i].level_mask = ((uint32_t)__builtin_popcount(mk) << 16) | mk;
    ord[i].f = s;
    ord[i].pos = (uint32_t)i;
  }
  qsort(ord, m, sizeof(sort_key), cmp_sort_key);

  /* Coordinates of the active dimensions, packed in sorted order. */
  float *P = (float *)malloc(sizeof(float) * m * (size_t)k);
  uint32_t *mk = (uint32_t *)malloc(sizeof(uint32_t) * m);
  for (uint64_t j = 0; j < m; ++j) {
    const float *r = rows + (size_t)cand[ord[j].pos] * d;
    for (int t = 0; t < k; ++t) P[j * k + t] = r[dims[t]];
    mk[j] = ord[j].level_mask & 0xffffu;
  }
  uint8_t *st = (uint8_t *)calloc(m, 1);
  uint8_t *st1 = (uint8_t *)malloc(m);
  uint32_t *conf = (uint32_t *)malloc(sizeof(uint32_t) * m);
  uint64_t nconf = 0;

  for (uint64_t b0 = 0, b1; b0 < m; b0 = b1) {
    b1 = b0 + ALPHA < m ? b0 + ALPHA : m;
    while (b1 < m && ord[b1].level_mask == ord[b1 - 1].level_mask &&
           ord[b1].f == ord[b1 - 1].f)
      ++b1;
    /* Phase 1: against confirmed points of earlier blocks. */
#pragma omp parallel for schedule(dynamic, 16) num_threads(threads) if (threads > 1)
    for (int64_t j = (int64_t)b0; j < (int64_t)b1; ++j) {
      uint8_t s_ = 0;
      for (uint64_t t = 0; t < nconf; ++t) {
        const uint32_t q = conf[t];
        if (mk[q] & ~mk[j]) continue;
        const int r = dominates_packed(P + (size_t)q * k, P + (size_t)j * k, k);
        if (r == 2) { s_ = 2; break; }
        if (r == 1) s_ = 1;
      }
      st[j] = s_;
    }
    memcpy(st1 + b0, st + b0, b1 - b0);
    /* Phase 2: against peers of the block that can precede p. */
#pragma omp parallel for schedule(dynamic, 16) num_threads(threads) if (threads > 1)
    for (int64_t j = (int64_t)b0; j < (int64_t)b1; ++j) {
      if (st1[j] == 2) continue;
      uint8_t s_ = st1[j];
      for (uint64_t q = b0; q < b1; ++q) {
        if (q == (uint64_t)j || st1[q] == 2) continue;
        if (q > (uint64_t)j && !(ord[q].level_mask == ord[j].level_mask && ord[q].f == ord[j].f))
          continue;
        if (mk[q] & ~mk[j]) continue;
        const int r = dominates_packed(P + q * k, P + (size_t)j * k, k);
        if (r == 2) { s_ = 2; break; }
        if (r == 1) s_ = 1;
      }
      st[j] = s_;
    }
    for (uint64_t j = b0; j < b1; ++j)
      if (st[j] != 2) conf[nconf++] = (uint32_t)j;
  }
  for (uint64_t j = 0; j < m; ++j) status[ord[j].pos] = st[j];
  free(ord);
  free(P);
  free(mk);
  free(st);
  free(st1);
  free(conf);
}

static void emit(const uint32_t *cand, uint64_t m, const uint8_t *status,
                 idlist *sky, idlist *ext) {
  uint64_t ns = 0, ne = 0;
  for (uint64_t i = 0; i < m; ++i) {
    ns += status[i] == 0;
    ne += status[i] == 1;
  }
  sky->ids = (uint32_t *)malloc(sizeof(uint32_t) * (ns ? ns : 1));
  ext->ids = (uint32_t *)malloc(sizeof(uint32_t) * (ne ? ne : 1));
  sky->n = ns;
  ext->n = ne;
  ns = ne = 0;
  for (uint64_t i = 0; i < m; ++i) {
    if (status[i] == 0) sky->ids[ns++] = cand[i];
    else if (status[i] == 1) ext->ids[ne++] = cand[i];
  }
}

/* Parents of a cuboid in the order generate_lattice records them:
 * descending cuboid index (src/utilities/lattice_utilities.cpp:58-75). */
static int parents_of(uint32_t c, int d, uint32_t *out) {
  int np = 0;
  for (int j = d - 1; j >= 0; --j) {
    /* parent = c | bit j for a bit j not in c; descending parent index means
     * descending j. */
    if (!(c & (1u << j))) out[np++] = c | (1u << j);
  }
  return np;
}

static int popc(uint32_t x) { return __builtin_popcount(x); }

static void cuboid(const float *rows, int d, oracle_result *res, uint32_t c,
                   uint32_t full, int threads) {
  uint32_t par[32];
  int np = parents_of(c, d, par);
  uint32_t src = full;
  if (res->sky[par[0]].n != 0) {
    uint64_t best = res->sky[par[0]].n + res->ext[par[0]].n;
    src = par[0];
    for (int i = 1; i < np; ++i) {
      uint64_t s = res->sky[par[i]].n + res->ext[par[i]].n;
      if (s < best) { best = s; src = par[i]; }
    }
  }
  uint64_t m = res->sky[src].n + res->ext[src].n;
  uint32_t *cand = (uint32_t *)malloc(sizeof(uint32_t) * (m ? m : 1));
  memcpy(cand, res->sky[src].ids, sizeof(uint32_t) * res->sky[src].n);
  memcpy(cand + res->sky[src].n, res->ext[src].ids,
         sizeof(uint32_t) * res->ext[src].n);
  uint8_t *st = (uint8_t *)malloc(m ? m : 1);
  skyline_ext(rows, d, cand, m, c, threads, st);
  emit(cand, m, st, &res->sky[c], &res->ext[c]);
  free(st);
  free(cand);
}

/* Runs the restated STSC skycube. rows: n x d row-major float32. Cuboids
 * with popcount > max_d are left empty (max_d <= 0 means all). */
void *oracle_stsc_run(const float *rows, uint32_t n, int d, int max_d,
                      int threads) {
  if (d < 1 || d > 16) return NULL;
  if (max_d <= 0 || max_d > d) max_d = d;
  if (threads < 1) threads = 1;
  oracle_result *res = (oracle_result *)calloc(1, sizeof(oracle_result));
  res->d = d;
  const uint32_t nc = 1u << d, full = nc - 1;
  res->sky = (idlist *)calloc(nc, sizeof(idlist));
  res->ext = (idlist *)calloc(nc, sizeof(idlist));

  uint32_t *all = (uint32_t *)malloc(sizeof(uint32_t) * (n ? n : 1));
  for (uint32_t i = 0; i < n; ++i) all[i] = i;
  uint8_t *st = (uint8_t *)malloc(n ? n : 1);
  skyline_ext(rows, d, all, n, full, threads, st);
  emit(all, n, st, &res->sky[full], &res->ext[full]);
  free(st);
  free(all);

  for (int lev = d - 1; lev >= 1; --lev) {
    if (lev > max_d) continue;
    uint32_t *list = (uint32_t *)malloc(sizeof(uint32_t) * nc);
    int cnt = 0;
    for (uint32_t c = 1; c < full; ++c)
      if (popc(c) == lev) list[cnt++] = c;
    /* Large candidate sets: one cuboid at a time, parallel inside.
     * Small ones: cuboids in parallel. */
    uint64_t biggest = 0;
    for (int i = 0; i < cnt; ++i) {
      uint32_t par[32];
      int np = parents_of(list[i], d, par);
      for (int j = 0; j < np; ++j) {
        uint64_t s = res->sky[par[j]].n + res->ext[par[j]].n;
        if (s > biggest) biggest = s;
      }
    }
    if (biggest > 20000 || threads == 1) {
      for (int i = 0; i < cnt; ++i) cuboid(rows, d, res, list[i], full, threads);
    } else {
#pragma omp parallel for schedule(dynamic, 1) num_threads(threads)
      for (int i = 0; i < cnt; ++i) cuboid(rows, d, res, list[i], full, 1);
    }
    free(list);
  }
  return res;
}

uint64_t oracle_stsc_count(void *h, uint32_t c, int ext) {
  oracle_result *r = (oracle_result *)h;
  if (c == 0 || c >= (1u << r->d)) return 0;
  return ext ? r->ext[c].n : r->sky[c].n;
}

void oracle_stsc_ids(void *h, uint32_t c, int ext, uint32_t *out) {
  oracle_result *r = (oracle_result *)h;
  if (c == 0 || c >= (1u << r->d)) return;
  idlist *l = ext ? &r->ext[c] : &r->sky[c];
  memcpy(out, l->ids, sizeof(uint32_t) * l->n);
}

void oracle_stsc_free(void *h) {
  oracle_result *r = (oracle_result *)h;
  if (!r) return;
  for (uint32_t c = 0; c < (1u << r->d); ++c) {
    free(r->sky[c].ids);
    free(r->ext[c].ids);
  }
  free(r->sky);
  free(r->ext);
  free(r);
}

/*
 * Brute force by definition, for tiny inputs: for every cuboid S and point p,
 * p is in sky(S) iff no other point dominates it on S. out_bits[p * words + w]
 * gets bit (S % 32) of word S / 32 SET when p is dominated in S (the
 * dominated-subspace bitmap of the MDMC kernel,
 * src/utilities/kernels.cuh:415-908, bit = 1 means pruned as in
 * src/skycube/Hashcube.h:275-283). Bit 0 (the empty subspace) is left clear.
 */
void oracle_bruteforce_bitmaps(const float *rows, uint32_t n, int d,
                               uint32_t *out_bits) {
  const uint32_t nc = 1u << d;
  const uint32_t words = nc / 32 ? nc / 32 : 1;
  memset(out_bits, 0, sizeof(uint32_t) * (size_t)words * n);
  for (uint32_t p = 0; p < n; ++p) {
    for (uint32_t q = 0; q < n; ++q) {
      if (q == p) continue;
      uint32_t le = 0, lt = 0;
      for (int j = 0; j < d; ++j) {
        float a = rows[(size_t)q * d + j], b = rows[(size_t)p * d + j];
        if (a <= b) le |= 1u << j;
        if (a < b) lt |= 1u << j;
      }
      /* dominated in every S subset of le that meets lt */
      for (uint32_t S = le; S; S = (S - 1) & le)
        if (S & lt) out_bits[(size_t)p * words + S / 32] |= 1u << (S % 32);
    }
  }
}
