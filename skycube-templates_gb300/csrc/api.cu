// C ABI of the skycube engine (include/skycube_gb300.h) and the host-side
// orchestration of the device pipelines.
//
// Pipelines (all on the context's stream, device memory from the stream-
// ordered pool):
//
//  full space   grid pivots + cells of all points, Manhattan-norm bucket
//               order, skyline kernel on the full space, compaction into the
//               full-space skyline, extended skyline and their union, the
//               candidate set (ascending ids). Replaces gpu_extended_skyline
//               + run_skyalign (src/mdmc/MDMC.cu:504-522).
//
//  BATCHED      candidate SoA copy, grid cells over the candidates, q order
//               by median-mask lattice level, block minima, ONE persistent
//               bitmap launch covering every cuboid, then device compaction
//               of the bitmaps into per-cuboid id lists. No host round trip
//               between the candidate count and the final size read.
//
//  PLAIN/SDSC   the suite's per-cuboid schedule (SDSC<D>::Execute,
//               src/sdsc/SDSC.cu:248-335): lattice levels top-down, each
//               cuboid's candidates are the skyline + extended skyline of its
//               smallest computed parent (findMinParent, :366-376; full space
//               when the first parent was skipped by max_d, :84-93); one
//               launch sequence and one host synchronisation per cuboid.
//
//  PLAIN/MDMC   the bitmap kernel launched on batches of 5,600 points with a
//               synchronisation after each batch, the shape of
//               tombstoning_hearting_gpu (src/mdmc/MDMC.cu:752-857).
#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <map>
#include <memory>
#include <thread>
#include <cstdarg>
#include <cstdlib>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "kernels.cuh"

namespace skc {

static thread_local std::string g_err;

int set_error(int code, const char* fmt, ...) {
  char buf[1024];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_err = buf;
  return code;
}

void clear_error() { g_err.clear(); }

int check_device_pointer(const void* p, int device, const char* what) {
  cudaPointerAttributes a{};
  cudaError_t e = cudaPointerGetAttributes(&a, p);
  if (e != cudaSuccess) {
    cudaGetLastError();  // not sticky: clear it
    return set_error(SKC_ERR_INVALID, "%s is not a CUDA pointer (%s)", what, cudaGetErrorString(e));
  }
  if (a.type != cudaMemoryTypeDevice && a.type != cudaMemoryTypeManaged)
    return set_error(SKC_ERR_INVALID, "%s is not device memory (pointer type %d)", what, (int)a.type);
  if (a.type == cudaMemoryTypeDevice && a.device != device)
    return set_error(SKC_ERR_INVALID, "%s lives on device %d, not on the current device %d", what,
                     a.device, device);
  return SKC_OK;
}

static std::atomic<uint64_t> g_launches{0};
// Launches recorded into a CUDA graph are counted when the graph runs.
static thread_local bool t_capturing = false;
void count_launch() {
  if (!t_capturing) g_launches.fetch_add(1, std::memory_order_relaxed);
}

// Execution state of one pipeline run: the stream it is issued on and the
// per-phase device times (CUDA events on that stream). skc_skycube runs on
// the context's stream; each serving slot has its own.
// Capacities of a plan's buffers (skc_plan): candidates and skyline /
// extended-skyline ids. In plan mode the pipeline reads no count back to the
// host; it sizes everything by these and leaves the true values in `stats`
// (device): [0] candidates, [1] skyline ids, [2] extended-skyline ids.
struct PlanCaps {
  uint64_t m_cap = 0;
  uint64_t ids_cap[2] = {0, 0};
  uint64_t* stats = nullptr;
};

struct Exec {
  skc_context* ctx = nullptr;
  cudaStream_t stream = nullptr;
  std::vector<std::pair<std::string, float>> phases;
  float ms = 0.f;
  const PlanCaps* plan = nullptr;  // plan mode (no host synchronisation)
};

// Records phase marks on the Exec's stream; fills Exec::phases when it goes
// out of scope and prints them to stderr when SKC_TRACE=1.
struct Tracer {
  Exec& E;
  bool print;
  std::vector<std::pair<const char*, cudaEvent_t>> marks;
  explicit Tracer(Exec& e) : E(e) {
    const char* v = getenv("SKC_TRACE");
    print = v && *v && *v != '0';
    mark("start");
  }
  void mark(const char* name) {
    if (E.plan) return;  // plan mode: the graph is timed as a whole
    cudaEvent_t ev;
    if (cudaEventCreate(&ev) != cudaSuccess) return;
    cudaEventRecord(ev, E.stream);
    marks.push_back({name, ev});
  }
  ~Tracer() {
    E.phases.clear();
    E.ms = 0.f;
    if (marks.size() > 1 && cudaEventSynchronize(marks.back().second) == cudaSuccess) {
      for (size_t i = 1; i < marks.size(); ++i) {
        float ms = 0.f;
        cudaEventElapsedTime(&ms, marks[i - 1].second, marks[i].second);
        E.phases.push_back({marks[i].first, ms});
        if (print) fprintf(stderr, "[skc] %-24s %9.3f ms\n", marks[i].first, ms);
      }
      cudaEventElapsedTime(&E.ms, marks.front().second, marks.back().second);
    }
    for (auto& m : marks) cudaEventDestroy(m.second);
  }
};

// Owns the temporary device buffers of one call; frees them stream-ordered.
// For a plan (skc_plan) it runs in one of two other modes: RECORD allocates
// with cudaMalloc and keeps every buffer in *bufs (the plan owns them);
// REPLAY hands the recorded buffers out again in the same order, so the
// launch sequence captured into the graph allocates nothing.
struct Arena {
  enum Mode { STREAM, RECORD, REPLAY };
  cudaStream_t s;
  std::vector<void*> ptrs;
  Mode mode = STREAM;
  std::vector<std::pair<void*, size_t>>* bufs = nullptr;
  size_t next = 0;
  explicit Arena(cudaStream_t st) : s(st) {}
  Arena(cudaStream_t st, Mode m, std::vector<std::pair<void*, size_t>>* b)
      : s(st), mode(m), bufs(b) {}
  ~Arena() {
    if (mode == STREAM)
      for (void* p : ptrs) cudaFreeAsync(p, s);
  }
  template <typename T>
  int alloc(T** p, uint64_t count) {
    const size_t bytes = (size_t)std::max<uint64_t>(count, 1) * sizeof(T);
    if (mode == REPLAY) {
      if (next >= bufs->size() || (*bufs)[next].second != bytes)
        return set_error(SKC_ERR_INVALID, "plan replay does not match its recording (buffer %zu)", next);
      *p = (T*)(*bufs)[next++].first;
      return SKC_OK;
    }
    if (mode == RECORD) {
      cudaError_t e = cudaMalloc((void**)p, bytes);
      if (e != cudaSuccess)
        return set_error(e == cudaErrorMemoryAllocation ? SKC_ERR_OOM : SKC_ERR_CUDA,
                         "plan allocation of %zu bytes failed: %s", bytes, cudaGetErrorString(e));
      bufs->push_back({(void*)*p, bytes});
      return SKC_OK;
    }
    cudaError_t e = cudaMallocAsync((void**)p, bytes, s);
    if (e != cudaSuccess)
      return set_error(e == cudaErrorMemoryAllocation ? SKC_ERR_OOM : SKC_ERR_CUDA,
                       "device allocation of %zu bytes failed: %s", bytes,
                       cudaGetErrorString(e));
    ptrs.push_back((void*)*p);
    return SKC_OK;
  }
  // Hands a buffer over to the caller (it is no longer freed here).
  void release(void* p) {
    auto it = std::find(ptrs.begin(), ptrs.end(), p);
    if (it != ptrs.end()) ptrs.erase(it);
  }
};

static inline uint64_t round_up(uint64_t v, uint64_t a) { return (v + a - 1) / a * a; }

// Host <-> device copies of the pipelines. Pageable host memory is copied
// directly: a warm 65 MB device-to-host copy into an already-touched buffer
// takes 0.37 ms over the Grace C2C link, and staging it through a pinned
// double buffer (measured) cost 4.7 ms of host memcpy per 1M x 10 skycube.
static int copy_h2d(void* dst, const void* src, size_t bytes, cudaStream_t s) {
  if (bytes) SKC_CUDA(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, s));
  return SKC_OK;
}

// Device -> host on stream s; returns once `dst` holds the data (after the
// work queued before it on s).
static int copy_d2h(void* dst, const void* src, size_t bytes, cudaStream_t s) {
  if (bytes) SKC_CUDA(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, s));
  SKC_CUDA(cudaStreamSynchronize(s));
  return SKC_OK;
}

// Partition tables over B-bit masks, built once per context (partition.cu):
// one device buffer [rank | unrank | sub_off | sub_list].
static int level_tables(skc_context* ctx, int B, LevelTables* out) {
  const uint32_t ns = 1u << B;
  std::lock_guard<std::mutex> lock(ctx->mu);
  if (!ctx->d_level_tables[B]) {
    std::vector<uint32_t> order(ns), rank(ns);
    for (uint32_t i = 0; i < ns; ++i) order[i] = i;
    std::stable_sort(order.begin(), order.end(), [](uint32_t a, uint32_t b) {
      return __builtin_popcount(a) < __builtin_popcount(b);
    });
    for (uint32_t i = 0; i < ns; ++i) rank[order[i]] = i;
    std::vector<uint32_t> sub_off(ns + 1, 0), sub_list;
    for (uint32_t mk = 0; mk < ns; ++mk) {
      sub_off[mk] = (uint32_t)sub_list.size();
      for (uint32_t r = 0; r < ns; ++r)
        if ((order[r] & ~mk) == 0) sub_list.push_back(r);
    }
    sub_off[ns] = (uint32_t)sub_list.size();
    std::vector<uint32_t> all;
    all.insert(all.end(), rank.begin(), rank.end());
    all.insert(all.end(), order.begin(), order.end());
    all.insert(all.end(), sub_off.begin(), sub_off.end());
    all.insert(all.end(), sub_list.begin(), sub_list.end());
    uint32_t* p = nullptr;
    SKC_CUDA(cudaMalloc(&p, all.size() * sizeof(uint32_t)));
    SKC_CUDA(cudaMemcpy(p, all.data(), all.size() * sizeof(uint32_t), cudaMemcpyHostToDevice));
    ctx->d_level_tables[B] = p;
  }
  uint32_t* p = ctx->d_level_tables[B];
  out->B = B;
  out->rank = p;
  out->unrank = p + ns;
  out->sub_off = p + 2 * ns;
  out->sub_list = p + 3 * ns + 1;
  return SKC_OK;
}

static int partition_dims(uint32_t S) {
  const int k = __builtin_popcount(S);
  return k < kMaxPartitionDims ? k : kMaxPartitionDims;
}

// Partition width of the bitmap kernel's q order: as many attributes as
// keep partitions at >= tile_points points on average (at most 10, at
// least 1).
static int bitmap_partition_dims(int d, uint64_t m, int tile_points) {
  int B = 1;
  while (B < kMaxPartitionDims && B < d && (m >> (B + 1)) >= (uint64_t)tile_points) ++B;
  return B;
}

// Work parameters of one run, after defaults and stored tunings apply.
struct RunParams {
  int depth = kMaxDepth;
  int pq_size = 0;        // prefilter pruners; 0: no prefilter
  int tile_points = 256;  // bitmap kernel: mean q's per median partition
  int chunk = 1;          // bitmap kernel: candidates per queue grab
  int blocks_per_sm = 0;  // bitmap kernel: 0 = occupancy limit
};
constexpr int kDefaultChunk = 1;

// Device-side result of the full-space step.
struct FullSpace {
  uint4* cells = nullptr;    // by point id (depth of the call)
  uint32_t* sky = nullptr;   // full-space skyline ids, ascending
  uint32_t* ext = nullptr;   // full-space extended skyline ids, ascending
  uint32_t* cand = nullptr;  // union, ascending
  uint32_t* counts = nullptr;  // device [0]=|sky| [1]=|ext| [2]=|cand|
  uint32_t h_counts[3] = {0, 0, 0};
};

static int run_full_space(Exec& E, skc_dataset* ds, const RunParams& P, Arena& A,
                          FullSpace& F, Tracer& T) {
  skc_context* ctx = E.ctx;
  cudaStream_t s = E.stream;
  const uint64_t n = ds->n;
  const int d = ds->d;
  const int depth = P.depth;
  const uint32_t full = (1u << d) - 1;
  uint32_t* d_n;
  SKC_TRY(A.alloc(&d_n, 1));
  SKC_TRY(launch_set_u32(s, d_n, (uint32_t)n));
  float* pivots;
  SKC_TRY(A.alloc(&pivots, (uint64_t)kMaxDims * kMaxPivots));
  SKC_TRY(A.alloc(&F.cells, n));
  // The cells kernel also sums the points' cell sums and their squares: the
  // spread that picks the skyline kernel's order (partition.cu, gray_order).
  unsigned long long* spread;
  SKC_TRY(A.alloc(&spread, 3));
  SKC_TRY(launch_pivots_cells(s, ds->x, ds->n_pad, d, nullptr, d_n, n, depth, pivots, F.cells,
                              spread));
  T.mark("full: pivots+cells");

  // Pruner prefilter: the skyline kernel then runs over the survivors only
  // (as point ids, ascending; their count stays on the device).
  const uint32_t* list = nullptr;
  const uint32_t* m_list = d_n;
  if (P.pq_size > 0) {
    const uint32_t Kq = (uint32_t)P.pq_size;
    const uint64_t nb = (n + 1023) / 1024 + 1;
    PrefilterScratch pf;
    SKC_TRY(A.alloc(&pf.hist, prefilter_sum_bins()));
    SKC_TRY(A.alloc(&pf.sel, 8));
    SKC_TRY(A.alloc(&pf.pr_ids, Kq));
    SKC_TRY(A.alloc(&pf.pr_key, Kq));
    SKC_TRY(A.alloc(&pf.pr_cells, Kq));
    SKC_TRY(A.alloc(&pf.pr_x, (uint64_t)d * Kq));
    SKC_TRY(A.alloc(&pf.st, n));
    SKC_TRY(A.alloc(&pf.blk0, nb));
    SKC_TRY(A.alloc(&pf.blk1, nb));
    SKC_TRY(A.alloc(&pf.mid_ids, n));
    SKC_TRY(A.alloc(&pf.mid_count, 1));
    uint32_t *surv, *d_ns;
    SKC_TRY(A.alloc(&surv, n));
    SKC_TRY(A.alloc(&d_ns, 1));
    PrefilterArgs pfa{F.cells, ds->x, ds->n_pad, nullptr, d_n, n, full, Kq, pf};
    SKC_TRY(launch_prefilter(s, d, ctx->num_sms, pfa, surv, d_ns));
    list = surv;
    m_list = d_ns;
    T.mark("full: prefilter");
  }

  LevelTables LT;
  SKC_TRY(level_tables(ctx, partition_dims(full), &LT));
  const uint32_t K = 1u << LT.B;
  PartScratch ps;
  SKC_TRY(A.alloc(&ps.keys, n));
  SKC_TRY(A.alloc(&ps.sorted, n));
  SKC_TRY(A.alloc(&ps.ccells, n));
  SKC_TRY(A.alloc(&ps.cx, (uint64_t)d * round_up(n, 128)));
  if (n >= kConfirmedMinPoints) {
    SKC_TRY(A.alloc(&ps.conf_cells, n));
    SKC_TRY(A.alloc(&ps.conf_x, (uint64_t)d * round_up(n, 128)));
    SKC_TRY(A.alloc(&ps.ccount, K));
    SKC_TRY(A.alloc(&ps.pdone, K));
  }
  SKC_TRY(A.alloc(&ps.counts, K + 1));
  SKC_TRY(A.alloc(&ps.cursor, kMaxSortBuckets + 1));
  SKC_TRY(A.alloc(&ps.fine, kMaxSortBuckets + 1));
  SKC_TRY(A.alloc(&ps.items, K + 1));
  ps.spread = spread;
  uint8_t* status;
  SKC_TRY(A.alloc(&status, round_up(n, 4)));
  PartitionSkylineArgs pa{list, F.cells, ds->x, ds->n_pad, m_list, n, full, status};
  // Slices pay on candidate-dense lists (the survivors); on lists full of
  // dominated points the slices after the strongest partitions would run to
  // their end for points the first slice already settles.
  if (list) {
    pa.split_target = (uint32_t)ctx->num_sms * kSplitCtasPerSm;
    pa.spread_ready = true;  // the spread of all n points picks the order
  }
  SKC_TRY(launch_partition_skyline(s, d, depth, LT, pa, ps));
  T.mark("full: skyline kernel");

  const uint64_t nblk = (n + 1023) / 1024 + 1;
  uint32_t *blk0, *blk1;
  SKC_TRY(A.alloc(&blk0, nblk));
  SKC_TRY(A.alloc(&blk1, nblk));
  SKC_TRY(A.alloc(&F.counts, 3));
  SKC_TRY(A.alloc(&F.sky, n));
  SKC_TRY(A.alloc(&F.ext, n));
  SKC_TRY(A.alloc(&F.cand, n));
  SKC_TRY(launch_status_compact(s, status, list, m_list, n, 0, blk0, blk1, F.sky, F.ext,
                                F.counts + 0, F.counts + 1));
  SKC_TRY(launch_status_compact(s, status, list, m_list, n, 1, blk0, blk1, F.cand, nullptr,
                                F.counts + 2, nullptr));
  if (E.plan) {
    // Plan mode: candidates sized by the plan's capacity (no read-back).
    const uint64_t cap = std::min<uint64_t>(E.plan->m_cap, n);
    SKC_TRY(launch_cap_count(s, F.counts + 2, (uint32_t)cap, E.plan->stats, 0));
    F.h_counts[0] = F.h_counts[1] = 0;
    F.h_counts[2] = (uint32_t)cap;
    return SKC_OK;
  }
  SKC_TRY(copy_d2h(F.h_counts, F.counts, 3 * sizeof(uint32_t), s));
  T.mark("full: compaction");
  return SKC_OK;
}

// Bitmaps of every candidate, then CSR compaction (BATCHED and PLAIN/MDMC).
static int run_bitmaps(Exec& E, skc_dataset* ds, const skc_options& o,
                       const RunParams& P, int max_d, Arena& A, FullSpace& F,
                       skc_result* R, Tracer& T) {
  skc_context* ctx = E.ctx;
  cudaStream_t s = E.stream;
  const int d = ds->d;
  const int depth = P.depth;
  const uint32_t nsub = 1u << d;
  const uint32_t W = nsub >= 32 ? nsub / 32 : 1;
  const uint64_t m = F.h_counts[2];
  const uint64_t m_pad = round_up(m, 128);
  uint32_t* m_ptr = F.counts + 2;
  const bool want_ext = o.want_extended || o.algo == SKC_ALGO_SDSC;

  float *xc, *xq;
  SKC_TRY(A.alloc(&xc, (uint64_t)d * m_pad));
  SKC_TRY(A.alloc(&xq, (uint64_t)d * m_pad));
  SKC_TRY(launch_gather_soa(s, ds->x, ds->n_pad, d, F.cand, m_ptr, m, m_pad, xc));
  float* pivots;
  uint4 *cc, *qc, *bmin, *smin, *hmin;
  SKC_TRY(A.alloc(&pivots, (uint64_t)kMaxDims * kMaxPivots));
  SKC_TRY(A.alloc(&cc, m));
  SKC_TRY(A.alloc(&qc, round_up(m, 32)));  // padded to whole blocks (k_pad_q)
  SKC_TRY(A.alloc(&bmin, (m + 31) / 32));
  SKC_TRY(A.alloc(&smin, (m + 31) / 32 * 4));
  SKC_TRY(A.alloc(&hmin, (m + 31) / 32 * 8));
  SKC_TRY(launch_pivots_cells(s, ds->x, ds->n_pad, d, F.cand, m_ptr, m, depth, pivots, cc));

  // q list: the full-space skyline only. If a point q' weakly dominates q
  // (q' <= q on every attribute), then for every p, LT(q, p) and LE(q, p)
  // are subsets of LT(q', p) and LE(q', p), so q's strict and tie sets are
  // inside q''s; following such q' ends at a skyline point. The
  // extended-skyline candidates are therefore p's only (on tie-heavy data
  // they are nearly all candidates: 581k x 10 ties has 9 skyline points
  // among 24,446 candidates). q's are kept as positions in candidate order;
  // their count stays on the device.
  uint32_t *qpos, *mq_ptr;
  SKC_TRY(A.alloc(&qpos, m));
  SKC_TRY(A.alloc(&mq_ptr, 1));
  uint8_t* qst;  // per candidate: 0 full-space skyline, 2 dominated there
  SKC_TRY(A.alloc(&qst, m));
  {
    const uint64_t nb = (m + 1023) / 1024 + 1;
    uint32_t *b0, *b1;
    SKC_TRY(A.alloc(&b0, nb));
    SKC_TRY(A.alloc(&b1, nb));
    SKC_TRY(launch_member_flags(s, F.cand, m_ptr, m, F.sky, F.counts + 0, qst));
    SKC_TRY(launch_status_compact(s, qst, nullptr, m_ptr, m, 1, b0, b1, qpos, nullptr, mq_ptr,
                                  nullptr));
  }
  // Host-side size of the q list (plans know only the candidate capacity).
  const uint64_t mq_host = E.plan ? m : F.h_counts[0];

  // q order: partitions by median mask over the first B attributes, in
  // lattice-level order (strongest partitions first).
  LevelTables LT;
  SKC_TRY(level_tables(ctx, bitmap_partition_dims(d, mq_host, P.tile_points), &LT));
  // Inside a partition, q's are ordered by the quartile-cell bits of the
  // first 8 attributes in Gray-code order, so consecutive q's share their
  // quartile on most attributes and the 32-q blocks' minimum-cell boxes stay
  // tight. On anticorrelated data every point has about the same cell sum,
  // so the strength order used before grouped far-apart points: 1M x 10
  // anticorrelated, bitmap kernel 29.6 -> 23.2 ms (binary pattern order)
  // -> 21.6 ms (Gray order).
  const uint32_t K = 1u << LT.B;
  int sub_bits = 0;
  while (sub_bits < 8 && ((uint64_t)K << (sub_bits + 1)) <= kMaxSortBuckets) ++sub_bits;
  const uint32_t KB = K << sub_bits;
  BucketScratch b;
  uint32_t* boff;
  SKC_TRY(A.alloc(&b.keys, m));
  SKC_TRY(A.alloc(&b.counts, KB + 1));
  SKC_TRY(A.alloc(&b.cursor, KB + 1));
  SKC_TRY(A.alloc(&boff, K + 1));
  uint32_t *qperm, *qidx, *qids;
  SKC_TRY(A.alloc(&qperm, m));
  SKC_TRY(A.alloc(&qidx, m));
  SKC_TRY(A.alloc(&qids, m));
  SKC_TRY(launch_mask_keys(s, cc, qpos, mq_ptr, m, nsub - 1, d, LT.B, depth, sub_bits,
                           depth >= 2 ? 1 : 0,
                           LT.rank, b.keys));
  SKC_TRY(launch_counting_sort(s, b.keys, mq_ptr, m, KB, b, qperm, nullptr));
  SKC_TRY(launch_partition_offsets(s, b.counts, K, sub_bits, boff));
  SKC_TRY(launch_gather_u32(s, qpos, qperm, mq_ptr, m, qidx));  // q order -> candidate position
  SKC_TRY(launch_gather_u32(s, F.cand, qidx, mq_ptr, m, qids));
  SKC_TRY(launch_gather_soa(s, ds->x, ds->n_pad, d, qids, mq_ptr, m, m_pad, xq));
  SKC_TRY(launch_gather_u4(s, cc, qidx, mq_ptr, m, qc));
  SKC_TRY(launch_pad_q(s, mq_ptr, d, qc, xq, m_pad));
  SKC_TRY(launch_block_min(s, qc, mq_ptr, m, bmin, smin, hmin));

  T.mark("cand: cells+q order");
  uint32_t *dom, *ext = nullptr, *work;
  SKC_TRY(A.alloc(&dom, m * W));
  if (want_ext) SKC_TRY(A.alloc(&ext, m * W));
  SKC_TRY(A.alloc(&work, 1));

  uint64_t slab_words = 0;
  uint32_t* slab = nullptr;
  SKC_TRY(bitmap_tie_slab_words(d, ctx->num_sms, &slab_words));
  if (slab_words) SKC_TRY(A.alloc(&slab, slab_words));
  BitmapArgs ba{cc, xc, m_pad, qc, xq, bmin, smin, hmin, boff, LT.unrank, K, LT.B, depth,
                m_ptr, work, (uint32_t)P.chunk, 0xffffffffu, dom, ext,
                P.blocks_per_sm * ctx->num_sms, slab};
  // A cap below d - 1 lets the kernel skip q's that only reach subspaces
  // above it; the bits there are then not computed, so per-point bitmaps
  // (want_bitmaps) keep the full computation.
  if (max_d <= d - 2 && !o.want_bitmaps) {
    ba.cap = max_d;
    ba.full_dom = qst;
  }
  if (o.mode == SKC_MODE_BATCHED) {
    SKC_CUDA(cudaMemsetAsync(work, 0, sizeof(uint32_t), s));
    SKC_TRY(launch_bitmaps(s, d, ctx->num_sms, ba));
  } else {
    // One launch per batch of points with a host round trip after each
    // (bitmaps of the batch copied to pinned host memory).
    const uint32_t batch = d >= 16 ? 2300 : 5600;
    // (host memory: the thread's staging, chunk by chunk; a pinned block
    // allocated and freed per call would wait for the whole device on free)
    std::vector<uint32_t> h_stage((size_t)batch * W);
    int st = SKC_OK;
    for (uint64_t p0 = 0; p0 < m && st == SKC_OK; p0 += batch) {
      const uint32_t p1 = (uint32_t)std::min<uint64_t>(m, p0 + batch);
      st = launch_set_u32(s, work, (uint32_t)p0);
      if (st != SKC_OK) break;
      ba.p_end = p1;
      st = launch_bitmaps(s, d, ctx->num_sms, ba);
      if (st != SKC_OK) break;
      st = copy_d2h(h_stage.data(), dom + p0 * W, (size_t)(p1 - p0) * W * sizeof(uint32_t), s);
    }
    SKC_TRY(st);
  }
  T.mark("bitmap kernel");

  // Compaction of skylines (bit clear) and extended skylines (bit set).
  const uint32_t tiles = compact_tiles(m);
  const uint64_t C = 32ull * W;
  for (int pass = 0; pass < (want_ext ? 2 : 1); ++pass) {
    CompactArgs ca{};
    ca.bits = pass == 0 ? dom : ext;
    ca.words = W;
    ca.m_ptr = m_ptr;
    ca.m_max = m;
    ca.count_set = pass;
    ca.nsub = nsub;
    ca.max_d = max_d;
    ca.cand = F.cand;
    SKC_TRY(A.alloc(&ca.counts, C * tiles));
    SKC_TRY(A.alloc(&ca.offs, C * tiles + 1));
    SKC_TRY(A.alloc(&ca.bsum, scan_bsum_entries(C * tiles)));
    uint64_t* csr;
    SKC_TRY(A.alloc(&csr, nsub + 1));
    ca.csr_off = csr;
    SKC_TRY(launch_bits_count(s, ca));
    uint64_t total = 0;
    if (E.plan) {
      // Plan mode: ids sized by the plan's capacity; the true total goes to
      // the stats and writes past the capacity are skipped.
      total = E.plan->ids_cap[pass];
      SKC_TRY(launch_stat_u64(s, csr + nsub, E.plan->stats, 1 + pass));
    } else {
      SKC_TRY(copy_d2h(&total, csr + nsub, sizeof(uint64_t), s));
    }
    uint32_t* ids;
    SKC_TRY(A.alloc(&ids, total));
    ca.out = ids;
    ca.out_cap = total;
    SKC_TRY(launch_bits_write(s, ca));
    T.mark(pass == 0 ? "compaction: skylines" : "compaction: extended");
    A.release(csr);
    A.release(ids);
    if (pass == 0) {
      R->d_off = csr;
      R->d_ids = ids;
      R->total_ids = total;
    } else {
      R->d_eoff = csr;
      R->d_eids = ids;
      R->total_ext = total;
    }
  }
  if (o.want_bitmaps) {
    A.release(dom);
    A.release(F.cand);
    R->d_bits = dom;
    R->d_cand = F.cand;
    R->words = W;
  }
  return SKC_OK;
}

// The suite's per-cuboid schedule (PLAIN/SDSC).
// Scratch of the single-cuboid pipeline for lists of up to mmax entries.
struct CuboidScratch {
  PartScratch ps;
  uint32_t *cand = nullptr, *d_m = nullptr, *blk0 = nullptr, *blk1 = nullptr, *cnt = nullptr;
  uint8_t* status = nullptr;
  // Counts read back per cuboid. Pageable on purpose: freeing pinned host
  // memory (cudaFreeHost) waits for the whole device, which stalled a
  // serving request for as long as another request's kernels ran.
  uint32_t h_cnt[2] = {0, 0};
};

static int cuboid_scratch(Arena& A, int d, uint64_t mmax, CuboidScratch* cs) {
  PartScratch& ps = cs->ps;
  const uint32_t Kmax = 1u << kMaxPartitionDims;
  SKC_TRY(A.alloc(&ps.keys, mmax));
  SKC_TRY(A.alloc(&ps.sorted, mmax));
  SKC_TRY(A.alloc(&ps.ccells, mmax));
  SKC_TRY(A.alloc(&ps.cx, (uint64_t)d * round_up(mmax, 128)));
  if (mmax >= kConfirmedMinPoints) {
    SKC_TRY(A.alloc(&ps.conf_cells, mmax));
    SKC_TRY(A.alloc(&ps.conf_x, (uint64_t)d * round_up(mmax, 128)));
    SKC_TRY(A.alloc(&ps.ccount, Kmax));
    SKC_TRY(A.alloc(&ps.pdone, Kmax));
  }
  SKC_TRY(A.alloc(&ps.counts, Kmax + 1));
  SKC_TRY(A.alloc(&ps.cursor, kMaxSortBuckets + 1));
  SKC_TRY(A.alloc(&ps.fine, kMaxSortBuckets + 1));
  SKC_TRY(A.alloc(&ps.items, Kmax + 1));
  SKC_TRY(A.alloc(&cs->cand, mmax));
  SKC_TRY(A.alloc(&cs->status, round_up(mmax, 4)));
  SKC_TRY(A.alloc(&cs->d_m, 1));
  const uint64_t nblk = (mmax + 1023) / 1024 + 1;
  SKC_TRY(A.alloc(&cs->blk0, nblk));
  SKC_TRY(A.alloc(&cs->blk1, nblk));
  SKC_TRY(A.alloc(&cs->cnt, 2));
  return SKC_OK;
}

// Skyline and extended skyline of cuboid c over an ascending candidate list
// (both outputs ascending), with the median-partition pipeline; one host
// round trip for the counts.
static int cuboid_lists(Exec& E, skc_dataset* ds, FullSpace& F, int depth, Arena& A,
                        CuboidScratch& cs, uint32_t c, const uint32_t* cand, uint64_t mc,
                        uint32_t** osky, uint32_t** oext, uint64_t* nsky, uint64_t* next) {
  cudaStream_t s = E.stream;
  SKC_TRY(launch_set_u32(s, cs.d_m, (uint32_t)mc));
  LevelTables LT;
  SKC_TRY(level_tables(E.ctx, partition_dims(c), &LT));
  PartitionSkylineArgs pa{cand, F.cells, ds->x, ds->n_pad, cs.d_m, mc, c, cs.status};
  SKC_TRY(launch_partition_skyline(s, ds->d, depth, LT, pa, cs.ps));
  SKC_TRY(A.alloc(osky, mc));
  SKC_TRY(A.alloc(oext, mc));
  SKC_TRY(launch_status_compact(s, cs.status, cand, cs.d_m, mc, 0, cs.blk0, cs.blk1, *osky,
                                *oext, cs.cnt, cs.cnt + 1));
  SKC_TRY(copy_d2h(cs.h_cnt, cs.cnt, 2 * sizeof(uint32_t), s));
  *nsky = cs.h_cnt[0];
  *next = cs.h_cnt[1];
  return SKC_OK;
}

// Cuboid-indexed CSRs of skylines (and extended skylines when want_ext) from
// per-cuboid device lists; cuboids above max_d (except the full space) are
// left empty.
static int assemble_csr(Exec& E, Arena& A, int d, int max_d, bool want_ext,
                        const std::vector<uint32_t*>& sky, const std::vector<uint64_t>& nsky,
                        const std::vector<uint32_t*>& ext, const std::vector<uint64_t>& next,
                        skc_result* R) {
  cudaStream_t s = E.stream;
  const uint32_t nsub = 1u << d, full = nsub - 1;
  for (int pass = 0; pass < (want_ext ? 2 : 1); ++pass) {
    std::vector<uint64_t> off(nsub + 1, 0);
    const auto& cntv = pass == 0 ? nsky : next;
    const auto& srcv = pass == 0 ? sky : ext;
    for (uint32_t c = 0; c < nsub; ++c) {
      const bool want = c >= 1 && (__builtin_popcount(c) <= max_d || c == full);
      off[c + 1] = off[c] + (want ? cntv[c] : 0);
    }
    uint64_t* d_off;
    uint32_t* ids;
    const uint32_t** d_srcs;
    SKC_TRY(A.alloc(&d_off, nsub + 1));
    SKC_TRY(A.alloc(&ids, off[nsub]));
    SKC_TRY(A.alloc(&d_srcs, nsub));
    std::vector<const uint32_t*> srcs(nsub, nullptr);
    for (uint32_t c = 0; c < nsub; ++c)
      if (off[c + 1] > off[c]) srcs[c] = srcv[c];
    SKC_TRY(copy_h2d(d_off, off.data(), (nsub + 1) * sizeof(uint64_t), s));
    SKC_TRY(copy_h2d(d_srcs, srcs.data(), nsub * sizeof(void*), s));
    SKC_TRY(launch_csr_gather(s, d_srcs, d_off, nsub, ids));
    SKC_CUDA(cudaStreamSynchronize(s));  // host vectors above must outlive the copies
    A.release(d_off);
    A.release(ids);
    if (pass == 0) {
      R->d_off = d_off;
      R->d_ids = ids;
      R->total_ids = off[nsub];
    } else {
      R->d_eoff = d_off;
      R->d_eids = ids;
      R->total_ext = off[nsub];
    }
  }
  return SKC_OK;
}

// Smallest computed parent of c (the full space when none of its parents
// was computed), as the suite's findMinParent picks it.
static uint32_t min_parent(uint32_t c, int d, const std::vector<uint64_t>& nsky,
                           const std::vector<uint64_t>& next, const std::vector<char>& done) {
  const uint32_t full = (1u << d) - 1;
  uint32_t src = full;
  uint64_t best = ~0ull;
  for (int j = d - 1; j >= 0; --j) {  // parents in generate_lattice's order
    if (c & (1u << j)) continue;
    const uint32_t p = c | (1u << j);
    if (p == full || !done[p]) continue;
    const uint64_t v = nsky[p] + next[p];
    if (v < best) {
      best = v;
      src = p;
    }
  }
  return src;
}

static int run_sdsc_plain(Exec& E, skc_dataset* ds, int max_d,
                          int depth_of_call, Arena& A, FullSpace& F,
                          skc_result* R, Tracer& T) {
  const int d = ds->d;
  const uint32_t nsub = 1u << d, full = nsub - 1;
  std::vector<uint32_t*> sky(nsub, nullptr), ext(nsub, nullptr);
  std::vector<uint64_t> nsky(nsub, 0), next(nsub, 0);
  std::vector<char> done(nsub, 0);
  sky[full] = F.sky;
  ext[full] = F.ext;
  nsky[full] = F.h_counts[0];
  next[full] = F.h_counts[1];
  done[full] = 1;

  CuboidScratch cs;
  SKC_TRY(cuboid_scratch(A, d, nsky[full] + next[full], &cs));
  for (int lev = d - 1; lev >= 1; --lev) {
    if (lev > max_d) continue;
    for (uint32_t c = 1; c < full; ++c) {
      if (__builtin_popcount(c) != lev) continue;
      const uint32_t src = min_parent(c, d, nsky, next, done);
      const uint64_t mc = nsky[src] + next[src];
      done[c] = 1;
      if (mc == 0) continue;
      // Candidates = parent skyline + extended skyline, merged ascending so
      // every output list stays ascending (compaction keeps list order).
      SKC_TRY(launch_merge_disjoint(E.stream, sky[src], (uint32_t)nsky[src], ext[src],
                                    (uint32_t)next[src], cs.cand));
      SKC_TRY(cuboid_lists(E, ds, F, depth_of_call, A, cs, c, cs.cand, mc, &sky[c], &ext[c],
                           &nsky[c], &next[c]));
    }
  }
  T.mark("per-cuboid skylines");
  return assemble_csr(E, A, d, max_d, true, sky, nsky, ext, next, R);
}

// Capped skycubes (max_d <= kLvMaxDims) in the lattice form (levels.cu):
// every wanted cuboid of every job in ONE persistent launch whose device
// work queue runs the lattice levels top down, each cuboid from its
// smallest computed parent's skyline + extended skyline (or the full
// space's candidates). Cuboids over the kernel's capacities are computed
// afterwards with the single-cuboid pipeline.
// Survivor scratch per launch: at most this, and at most a quarter of the
// free device memory. A level whose cuboids do not all fit is cut into
// groups, each one more P/F/S phase triple; 8 GB holds the 1,820 cuboids
// of a 16-d first level at cap 4 in one group (2 GB took three: 500k x 16
// -m 4 53.1 -> 48.6 ms).
constexpr uint64_t kLvScratchBytes = 8192ull << 20;
constexpr uint32_t kLvMaxSurvivors = 262144;         // per cuboid
// More cuboids over the capacities than this on a job's first level (heavy
// exact ties: the per-cuboid fallback would dominate) and the bitmap form
// takes over; the job's status is then kLvGiveUp with its result untouched.
constexpr int kLvMaxFallbacks = 16;
constexpr int kLvGiveUp = 1000;

struct LatticeJob {
  skc_dataset* ds = nullptr;
  int max_d = 0;
  int depth = kMaxDepth;
  bool want_ext = false;
  FullSpace* F = nullptr;
  skc_result* R = nullptr;
  int status = SKC_OK;  // per job: SKC_OK or kLvGiveUp
  // filled by run_lattice
  uint4* lv_cells = nullptr;
  uint32_t* d_index = nullptr;
  uint32_t cub0 = 0;
  std::vector<uint32_t> masks;
};

static int run_lattice(Exec& E, std::vector<LatticeJob>& jobs, Arena& A, Tracer& T) {
  skc_context* ctx = E.ctx;
  cudaStream_t s = E.stream;
  const uint32_t nj = (uint32_t)jobs.size();
  // 1. Per job: cells on a grid of the candidates' own quantiles, by point id
  // (on the full-space grid most candidates of correlated data share one
  // cell on every attribute, which leaves the cell sums no order to give),
  // and its cuboid table (levels top down, masks ascending).
  std::vector<LtJob> hjobs(nj);
  std::vector<uint32_t> c_mask, c_job;
  std::vector<int> c_level;
  std::vector<std::vector<uint32_t>> index(nj);
  uint64_t max_cand = 1;
  int top = 0;
  for (uint32_t j = 0; j < nj; ++j) {
    LatticeJob& J = jobs[j];
    skc_dataset* ds = J.ds;
    const int d = ds->d;
    const uint64_t m = J.F->h_counts[2];
    float* pivots;
    uint4* cc;
    SKC_TRY(A.alloc(&pivots, (uint64_t)kMaxDims * kMaxPivots));
    SKC_TRY(A.alloc(&cc, std::max<uint64_t>(1, m)));
    SKC_TRY(A.alloc(&J.lv_cells, ds->n));
    SKC_TRY(launch_pivots_cells(s, ds->x, ds->n_pad, d, J.F->cand, J.F->counts + 2, m, J.depth,
                                pivots, cc));
    SKC_TRY(launch_scatter_u4(s, cc, J.F->cand, J.F->counts + 2, m, J.lv_cells));
    J.cub0 = (uint32_t)c_mask.size();
    const uint32_t full = (1u << d) - 1;
    index[j].assign(1u << d, 0xffffffffu);
    for (int lev = J.max_d; lev >= 1; --lev)
      for (uint32_t c = 1; c < full; ++c)
        if (__builtin_popcount(c) == lev) {
          index[j][c] = (uint32_t)c_mask.size();
          c_mask.push_back(c);
          c_job.push_back(j);
          c_level.push_back(lev);
        }
    J.masks.assign(c_mask.begin() + J.cub0, c_mask.end());
    SKC_TRY(A.alloc(&J.d_index, 1u << d));
    SKC_TRY(copy_h2d(J.d_index, index[j].data(), sizeof(uint32_t) << d, s));
    hjobs[j] = LtJob{ds->x, ds->n_pad, J.lv_cells, J.F->cand, (uint32_t)m, J.d_index, d, J.max_d};
    max_cand = std::max<uint64_t>(max_cand, m);
    top = std::max(top, J.max_d);
  }
  const uint32_t ncub = (uint32_t)c_mask.size();

  // 2. Work queue: per level (top down) groups of cuboids that fit the
  // survivor scratch, each as phases P, F and S.
  int grid = 0;
  SKC_TRY(lattice_grid(ctx->num_sms, &grid));
  const uint32_t cap = (uint32_t)std::min<uint64_t>(max_cand, kLvMaxSurvivors);
  uint64_t scratch = kLvScratchBytes;
  {
    size_t free_b = 0, total_b = 0;
    if (cudaMemGetInfo(&free_b, &total_b) == cudaSuccess)
      scratch = std::min<uint64_t>(scratch, std::max<uint64_t>(free_b / 4, 256ull << 20));
  }
  const uint32_t G = (uint32_t)std::max<uint64_t>(1, scratch / ((uint64_t)cap * 10));
  std::vector<uint32_t> c_scr(ncub, 0), it_cub, it_arg, it_phase, ph_size;
  std::vector<uint8_t> ph_kind;
  uint32_t g_used = 1;
  for (int lev = top; lev >= 1; --lev) {
    std::vector<uint32_t> cubs;
    for (uint32_t c = 0; c < ncub; ++c)
      if (c_level[c] == lev) cubs.push_back(c);
    for (size_t g0 = 0; g0 < cubs.size(); g0 += G) {
      const uint32_t ng = (uint32_t)std::min<size_t>(G, cubs.size() - g0);
      g_used = std::max(g_used, ng);
      for (int kind = 0; kind < 3; ++kind) {
        const uint32_t ph = (uint32_t)ph_size.size();
        uint32_t count = 0;
        for (uint32_t i = 0; i < ng; ++i) {
          const uint32_t c = cubs[g0 + i];
          c_scr[c] = i;
          uint32_t nsl = 1;
          if (kind == 1) {
            // a job's first level filters its full candidate list; lower
            // levels their parent's slot (at most kLvSlot entries)
            const bool first = c_level[c] == jobs[c_job[c]].max_d;
            const uint64_t len = first ? jobs[c_job[c]].F->h_counts[2] : kLvSlot;
            const uint64_t chunks = std::max<uint64_t>(1, (len + kLvChunk - 1) / kLvChunk);
            nsl = (uint32_t)std::min<uint64_t>(
                std::min<uint64_t>(chunks, 0xffffu), std::max<uint64_t>(1, (2ull * grid + ng - 1) / ng));
          }
          for (uint32_t sl = 0; sl < nsl; ++sl) {
            it_cub.push_back(c);
            it_arg.push_back(sl | (nsl << 16));
            it_phase.push_back(ph);
            ++count;
          }
        }
        ph_size.push_back(count);
        ph_kind.push_back((uint8_t)kind);
      }
    }
  }
  const uint32_t n_items = (uint32_t)it_cub.size(), n_ph = (uint32_t)ph_size.size();
  // Fault injection for the tests (SKC_FAULT_LATTICE_WAIT=1): the first
  // phase counts one item more than exists, so the second phase's waits run
  // out and the launch ends with SKC_ERR_TIMEOUT. Nothing faults or hangs.
  if (const char* f = getenv("SKC_FAULT_LATTICE_WAIT"))
    if (*f == '1' && n_ph > 1) ph_size[0] += 1;

  // 3. Device tables and scratch.
  LtArgs a{};
  LtJob* d_jobs;
  uint32_t *d_mask, *d_job, *d_scr, *d_list_n, *d_nsky, *d_next, *d_flag, *d_slot;
  const uint32_t** d_list;
  SKC_TRY(A.alloc(&d_jobs, nj));
  SKC_TRY(A.alloc(&d_mask, ncub));
  SKC_TRY(A.alloc(&d_job, ncub));
  SKC_TRY(A.alloc(&d_scr, ncub));
  SKC_TRY(A.alloc(&d_list, ncub));
  SKC_TRY(A.alloc(&d_list_n, ncub));
  SKC_TRY(A.alloc(&d_nsky, ncub));
  SKC_TRY(A.alloc(&d_next, ncub));
  SKC_TRY(A.alloc(&d_flag, ncub));
  SKC_TRY(A.alloc(&d_slot, (uint64_t)ncub * kLvSlot));
  SKC_TRY(A.alloc(&a.pr_c, (uint64_t)g_used * kLvPruners));
  SKC_TRY(A.alloc(&a.pr_v, (uint64_t)g_used * kLvMaxDims * kLvPruners));
  SKC_TRY(A.alloc(&a.pr_n, g_used));
  SKC_TRY(A.alloc(&a.cnt, g_used));
  SKC_TRY(A.alloc(&a.surv_id, (uint64_t)g_used * cap));
  SKC_TRY(A.alloc(&a.surv_key, (uint64_t)g_used * cap));
  SKC_TRY(A.alloc(&a.srt, (uint64_t)g_used * cap));
  uint32_t *d_it_cub, *d_it_arg, *d_it_phase, *d_ph_size, *d_counters;
  uint8_t* d_ph_kind;
  SKC_TRY(A.alloc(&d_it_cub, n_items));
  SKC_TRY(A.alloc(&d_it_arg, n_items));
  SKC_TRY(A.alloc(&d_it_phase, n_items));
  SKC_TRY(A.alloc(&d_ph_size, n_ph));
  SKC_TRY(A.alloc(&d_ph_kind, n_ph));
  // counters: [0, n_ph) phase done, n_ph next item, n_ph + 1 status,
  // then per job the first-level overflows
  SKC_TRY(A.alloc(&d_counters, n_ph + 2 + nj));
  SKC_TRY(copy_h2d(d_jobs, hjobs.data(), nj * sizeof(LtJob), s));
  SKC_TRY(copy_h2d(d_mask, c_mask.data(), ncub * 4, s));
  SKC_TRY(copy_h2d(d_job, c_job.data(), ncub * 4, s));
  SKC_TRY(copy_h2d(d_scr, c_scr.data(), ncub * 4, s));
  SKC_TRY(copy_h2d(d_it_cub, it_cub.data(), (size_t)n_items * 4, s));
  SKC_TRY(copy_h2d(d_it_arg, it_arg.data(), (size_t)n_items * 4, s));
  SKC_TRY(copy_h2d(d_it_phase, it_phase.data(), (size_t)n_items * 4, s));
  SKC_TRY(copy_h2d(d_ph_size, ph_size.data(), n_ph * 4, s));
  SKC_TRY(copy_h2d(d_ph_kind, ph_kind.data(), n_ph, s));
  SKC_CUDA(cudaMemsetAsync(d_counters, 0, (n_ph + 2 + nj) * 4, s));
  SKC_CUDA(cudaMemsetAsync(d_flag, 0, ncub * 4, s));
  a.jobs = d_jobs;
  a.c_mask = d_mask;
  a.c_job = d_job;
  a.c_scr = d_scr;
  a.c_list = d_list;
  a.c_list_n = d_list_n;
  a.c_nsky = d_nsky;
  a.c_next = d_next;
  a.c_flag = d_flag;
  a.slot = d_slot;
  a.cap = cap;
  a.n_items = n_items;
  a.it_cub = d_it_cub;
  a.it_arg = d_it_arg;
  a.it_phase = d_it_phase;
  a.ph_size = d_ph_size;
  a.ph_kind = d_ph_kind;
  a.ph_done = d_counters;
  a.next_item = d_counters + n_ph;
  a.status = d_counters + n_ph + 1;
  a.job_over = d_counters + n_ph + 2;
  a.max_fallbacks = kLvMaxFallbacks;
  SKC_TRY(launch_lattice(s, ctx->num_sms, a));

  std::vector<uint32_t> h_nsky(ncub), h_next(ncub), h_flag(ncub), h_tail(2 + nj);
  SKC_TRY(copy_d2h(h_nsky.data(), d_nsky, ncub * 4, s));
  SKC_TRY(copy_d2h(h_next.data(), d_next, ncub * 4, s));
  SKC_TRY(copy_d2h(h_flag.data(), d_flag, ncub * 4, s));
  SKC_TRY(copy_d2h(h_tail.data(), d_counters + n_ph, (2 + nj) * 4, s));
  if (h_tail[1]) return set_error(SKC_ERR_TIMEOUT, "lattice kernel: a phase wait ran out");
  T.mark("lattice kernel");

  // 4. Per job: host fallbacks for cuboids over a capacity, then the CSRs.
  for (uint32_t j = 0; j < nj; ++j) {
    LatticeJob& J = jobs[j];
    if (h_tail[2 + j] > (uint32_t)kLvMaxFallbacks) {
      J.status = kLvGiveUp;
      continue;
    }
    skc_dataset* ds = J.ds;
    const int d = ds->d;
    const uint32_t nsub = 1u << d, full = nsub - 1;
    FullSpace& F = *J.F;
    std::vector<uint32_t*> sky(nsub, nullptr), ext(nsub, nullptr);
    std::vector<uint64_t> nsky(nsub, 0), next(nsub, 0);
    sky[full] = F.sky;
    ext[full] = F.ext;
    nsky[full] = F.h_counts[0];
    next[full] = F.h_counts[1];
    CuboidScratch cs;
    bool cs_ready = false;
    int fallbacks = 0;
    for (uint32_t i = 0; i < (uint32_t)J.masks.size(); ++i) {
      const uint32_t c = J.masks[i], t = J.cub0 + i;
      if (h_flag[t] == 0) {
        sky[c] = d_slot + (uint64_t)t * kLvSlot;
        nsky[c] = h_nsky[t];
        ext[c] = sky[c] + nsky[c];
        next[c] = h_next[t];
        continue;
      }
      // Over a capacity: the single-cuboid pipeline on the full-space
      // candidates (ascending, a superset of every cuboid's lists).
      if (!cs_ready) {
        SKC_TRY(cuboid_scratch(A, d, F.h_counts[2], &cs));
        cs_ready = true;
      }
      ++fallbacks;
      SKC_TRY(cuboid_lists(E, ds, F, J.depth, A, cs, c, F.cand, F.h_counts[2], &sky[c], &ext[c],
                           &nsky[c], &next[c]));
    }
    if (fallbacks) T.mark("lattice fallbacks");
    J.R->level_fallbacks = fallbacks;
    SKC_TRY(assemble_csr(E, A, d, J.max_d, J.want_ext, sky, nsky, ext, next, J.R));
  }
  return SKC_OK;
}

static int run_levels(Exec& E, skc_dataset* ds, const skc_options& o, int max_d, int depth,
                      Arena& A, FullSpace& F, skc_result* R, Tracer& T) {
  std::vector<LatticeJob> jobs(1);
  jobs[0].ds = ds;
  jobs[0].max_d = max_d;
  jobs[0].depth = depth;
  jobs[0].want_ext = o.want_extended || o.algo == SKC_ALGO_SDSC;
  jobs[0].F = &F;
  jobs[0].R = R;
  SKC_TRY(run_lattice(E, jobs, A, T));
  return jobs[0].status;
}

// The level form can replace the bitmaps for batched capped skycubes of
// small caps, when no per-point bitmaps are wanted and no plan is being
// recorded (the level form syncs per level). Auto takes it where it was
// faster on one GB300 (device ms, level / bitmap form, cap 4 unless noted):
//   16 attributes: anticorrelated 500k 48.3 / 83.5, 396k 36.7 / 64.1;
//     uniform 937k 69.4 / 84.8, 200k 16.0 / 17.2
//   14-15 attributes: anticorrelated 799k x 14 (737k candidates) 51.9 /
//     58.8; but anticorrelated 150k x 14 9.7 / 9.1 and uniform 951k x 15
//     (503k candidates) 49.2 / 39.9
//   12 attributes and fewer, cap 4: anticorrelated 500k x 12 17.7 / 17.7,
//     1M x 10 15.3 / 11.5
//   caps under 4: anticorrelated 1M x 8 cap 3 4.55 / 4.69, uniform
//     400k x 11 cap 2 2.3 / 2.8
// Below 65,536 candidates the bitmap kernel is as fast or faster, and
// tie-heavy data (whose small cuboids have skylines over the level kernels'
// capacities) has few candidates.
constexpr uint64_t kLvMinCandidates = 65536;
constexpr uint64_t kLvMinCandidatesMidD = 600000;  // 14 and 15 attributes
static bool levels_by_default(int d, int max_d, uint64_t candidates) {
  if (candidates < kLvMinCandidates) return false;
  return max_d <= 3 || d >= 16 || (d >= 14 && candidates >= kLvMinCandidatesMidD);
}
static bool use_levels(const Exec& E, const skc_dataset* ds, const skc_options& o, int max_d,
                       const FullSpace& F) {
  if (o.form == SKC_FORM_BITMAPS) return false;
  const bool can = !E.plan && o.mode == SKC_MODE_BATCHED && !o.want_bitmaps &&
                   max_d <= kLvMaxDims && max_d <= ds->d - 2 && ds->n < (1ull << 31);
  return can && (o.form == SKC_FORM_LEVELS || levels_by_default(ds->d, max_d, F.h_counts[2]));
}

static int auto_depth(uint64_t n, int d) {
  (void)n;
  (void)d;
  return kMaxDepth;
}

// Defaults of the work parameters (used when neither the options nor a
// stored tuning set them).
// Pruners: 512 in two passes (32 on every point, the rest on the survivors
// when at least a quarter survive; prefilter.cu). The suite's -q default is
// 128 (one pass).
constexpr int kDefaultPruners = 512;
constexpr uint64_t kPrefilterMinPoints = 32768;  // below: launch-bound anyway
constexpr int kDefaultTilePoints = 256;

// The dataset's sample signature (computed once, on stream s).
static int dataset_signature(skc_dataset* ds, cudaStream_t s, uint32_t sig[3]) {
  skc_context* ctx = ds->ctx;
  {
    std::lock_guard<std::mutex> lock(ctx->mu);
    if (ds->sig_ready) {
      sig[0] = ds->sig_samples;
      sig[1] = ds->sig_sky;
      sig[2] = ds->sig_tied;
      return SKC_OK;
    }
  }
  uint32_t h[3] = {0, 0, 0};
  {
    Arena A(s);
    uint32_t* out;
    SKC_TRY(A.alloc(&out, 3));
    SKC_TRY(launch_sample_signature(s, ds->x, ds->n_pad, ds->n, ds->d, out));
    SKC_TRY(copy_d2h(h, out, sizeof(h), s));
  }
  std::lock_guard<std::mutex> lock(ctx->mu);
  ds->sig_samples = h[2];
  ds->sig_sky = h[0];
  ds->sig_tied = h[1];
  ds->sig_ready = true;
  sig[0] = h[2];
  sig[1] = h[0];
  sig[2] = h[1];
  return SKC_OK;
}

// floor(log2(1 + 1000 * f)) for f in [0, 1]: 0..9.
static int log_class(double f) {
  int c = 0;
  while (c < 9 && (double)(2u << c) <= 1.0 + 1000.0 * f) ++c;
  return c;
}

// Classes of a signature: size = floor(log2 n); sky = a two-sided log scale
// of the sample skyline fraction f, fine near 0 (correlated data) and near 1
// (anticorrelated or high-d data): log_class(f) for f <= 1/2, else
// 17 - log_class(1 - f), so 0..17; ties = at least 1/8 of the sample shares
// a value with another sample point.
static void signature_classes(const skc_dataset* ds, const uint32_t sig[3], int* size_class,
                              int* sky_class, int* ties) {
  int sc = 0;
  while (sc < 63 && (ds->n >> (sc + 1))) ++sc;
  const double f = sig[0] ? (double)sig[1] / sig[0] : 0.0;
  *size_class = sc;
  *sky_class = f <= 0.5 ? log_class(f) : 17 - log_class(1.0 - f);
  *ties = sig[0] && sig[2] * 8 >= sig[0];
}

// Tuning-table key: the dataset's classes, d, and the options that shape
// the pipeline (algorithm, form, cuboid cap, skyline query or skycube).
static uint64_t tuning_key(const skc_dataset* ds, const uint32_t sig[3], const skc_options& o,
                           int max_d) {
  int sc, kc, ties;
  signature_classes(ds, sig, &sc, &kc, &ties);
  uint64_t k = (uint64_t)sc;           // bits 0-5
  k |= (uint64_t)ds->d << 6;           // bits 6-10
  k |= (uint64_t)kc << 11;             // bits 11-15
  k |= (uint64_t)ties << 16;
  k |= (uint64_t)(o.algo & 1) << 17;
  k |= (uint64_t)(o.mode & 1) << 18;
  k |= (uint64_t)max_d << 19;          // bits 19-23
  k |= (uint64_t)(o.subspace != 0) << 24;
  return k;
}

// Work parameters of a run: explicit options first, then the stored tuning
// for the dataset's signature (looked up only when some field is automatic
// and the table is not empty), then the defaults.
static int resolve_params(skc_dataset* ds, cudaStream_t s, const skc_options& o, int max_d,
                          RunParams* out) {
  skc_context* ctx = ds->ctx;
  const uint64_t n = ds->n;
  const bool any_auto = !o.depth || !o.pq_size || !o.tile_points || !o.chunk || !o.blocks_per_sm;
  bool have = false;
  skc_context::Tuned tv{};
  bool table = false;
  {
    std::lock_guard<std::mutex> lock(ctx->mu);
    table = !ctx->tunings.empty();
  }
  if (any_auto && table) {
    uint32_t sig[3];
    SKC_TRY(dataset_signature(ds, s, sig));
    const uint64_t key = tuning_key(ds, sig, o, max_d);
    std::lock_guard<std::mutex> lock(ctx->mu);
    auto it = ctx->tunings.find(key);
    if (it != ctx->tunings.end()) {
      tv = it->second;
      have = true;
    }
  }
  RunParams P;
  P.depth = o.depth ? o.depth : have ? tv.depth : auto_depth(n, ds->d);
  int pq = 0;
  if (o.pq_size > 0) pq = o.pq_size;
  else if (o.pq_size == 0) pq = have ? tv.pq_size : (n >= kPrefilterMinPoints ? kDefaultPruners : 0);
  P.pq_size = (pq > 0 && n > 2ull * (uint64_t)pq) ? pq : 0;
  P.tile_points = o.tile_points ? o.tile_points : have ? tv.tile_points : kDefaultTilePoints;
  P.chunk = o.chunk ? o.chunk : have ? tv.chunk : kDefaultChunk;
  P.blocks_per_sm = o.blocks_per_sm ? o.blocks_per_sm : have ? tv.blocks_per_sm : 0;
  *out = P;
  return SKC_OK;
}

}  // namespace skc

using namespace skc;

// Frees an object's device memory and detaches it from its context; the host
// struct stays valid until the caller frees it.
// A captured batched pipeline (skc_plan_*): the plan owns every buffer of the
// pipeline (Arena RECORD mode) and a CUDA graph of its launch sequence.
struct skc_plan {
  skc_context* ctx = nullptr;
  skc_dataset* ds = nullptr;  // nullptr once the dataset was freed
  skc_options opt{};
  RunParams P;
  int max_d = 0;
  PlanCaps caps;
  std::vector<std::pair<void*, size_t>> bufs;
  skc_result outs;              // device views of the graph's outputs
  uint64_t* h_stats = nullptr;  // pinned copy of caps.stats
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  uint64_t kernels = 0;  // kernel nodes of the graph
  uint64_t replans = 0;
};

static void plan_release_device(skc_plan* p) {
  if (p->exec) cudaGraphExecDestroy(p->exec);
  if (p->graph) cudaGraphDestroy(p->graph);
  p->exec = nullptr;
  p->graph = nullptr;
  for (auto& b : p->bufs) cudaFree(b.first);
  p->bufs.clear();
  p->caps.stats = nullptr;
  p->kernels = 0;
  p->outs.d_off = p->outs.d_eoff = nullptr;
  p->outs.d_ids = p->outs.d_eids = p->outs.d_bits = p->outs.d_cand = nullptr;
}

// Frees a plan's device state and unregisters it (the object stays).
static void release_plan_memory(skc_plan* p) {
  if (!p->ctx) return;
  plan_release_device(p);
  if (p->h_stats) cudaFreeHost(p->h_stats);
  p->h_stats = nullptr;
  {
    std::lock_guard<std::mutex> lock(p->ctx->mu);
    p->ctx->plans.erase(p);
  }
  p->ctx = nullptr;
  p->ds = nullptr;
}

static void release_result_memory(skc_result* r) {
  if (!r->ctx) return;
  cudaStream_t s = r->stream ? r->stream : r->ctx->stream;
  for (void* p : {(void*)r->d_off, (void*)r->d_ids, (void*)r->d_eoff, (void*)r->d_eids,
                  (void*)r->d_bits, (void*)r->d_cand})
    if (p) cudaFreeAsync(p, s);
  r->d_off = nullptr;
  r->d_ids = nullptr;
  r->d_eoff = nullptr;
  r->d_eids = nullptr;
  r->d_bits = nullptr;
  r->d_cand = nullptr;
  {
    std::lock_guard<std::mutex> lock(r->ctx->mu);
    r->ctx->results.erase(r);
  }
  r->ctx = nullptr;
}

static void release_dataset_memory(skc_dataset* ds) {
  if (!ds->ctx) return;
  if (ds->x) cudaFreeAsync(ds->x, ds->stream ? ds->stream : ds->ctx->stream);
  ds->x = nullptr;
  {
    std::lock_guard<std::mutex> lock(ds->ctx->mu);
    ds->ctx->datasets.erase(ds);
    for (skc_plan* p : ds->ctx->plans)
      if (p->ds == ds) p->ds = nullptr;  // its graph reads ds->x: never again
  }
  ds->ctx = nullptr;
}

// ==========================================================================
// C ABI
extern "C" {

const char* skc_last_error(void) { return g_err.c_str(); }

uint64_t skc_kernel_launches(void) { return g_launches.load(); }

int skc_last_phase(skc_context* ctx, int index, const char** name, float* ms) {
  clear_error();
  if (!ctx || !name || !ms) return set_error(SKC_ERR_INVALID, "NULL argument");
  if (index < 0 || index >= (int)ctx->phases.size())
    return set_error(SKC_ERR_INVALID, "phase %d out of range (%d phases)", index, (int)ctx->phases.size());
  *name = ctx->phases[index].first.c_str();
  *ms = ctx->phases[index].second;
  return SKC_OK;
}

void skc_options_init(skc_options* o) {
  if (!o) return;
  o->algo = SKC_ALGO_MDMC;
  o->mode = SKC_MODE_BATCHED;
  o->max_d = 0;
  o->depth = 0;
  o->want_extended = 0;
  o->want_bitmaps = 0;
  o->subspace = 0;
  o->pq_size = 0;
  o->tile_points = 0;
  o->chunk = 0;
  o->blocks_per_sm = 0;
  o->form = 0;
}

int skc_context_create(int device, skc_context** out) {
  clear_error();
  if (!out) return set_error(SKC_ERR_INVALID, "out is NULL");
  *out = nullptr;
  int count = 0;
  cudaError_t e = cudaGetDeviceCount(&count);
  if (e != cudaSuccess) return set_error(SKC_ERR_CUDA, "no CUDA device: %s", cudaGetErrorString(e));
  if (device < 0 || device >= count)
    return set_error(SKC_ERR_INVALID, "device %d out of range (%d devices)", device, count);
  SKC_CUDA(cudaSetDevice(device));
  SKC_CUDA(cudaFree(0));
  auto* ctx = new skc_context;
  ctx->device = device;
  if (cudaDeviceGetAttribute(&ctx->num_sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess ||
      cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreate(&ctx->ev_start) != cudaSuccess || cudaEventCreate(&ctx->ev_stop) != cudaSuccess ||
      cudaDeviceGetDefaultMemPool(&ctx->pool, device) != cudaSuccess) {
    delete ctx;
    return set_error(SKC_ERR_CUDA, "context setup failed: %s", cudaGetErrorString(cudaGetLastError()));
  }
  uint64_t thr = UINT64_MAX;
  cudaMemPoolSetAttribute(ctx->pool, cudaMemPoolAttrReleaseThreshold, &thr);
  upload_submask_table();
  *out = ctx;
  return SKC_OK;
}

int skc_context_destroy(skc_context* ctx) {
  clear_error();
  if (!ctx) return SKC_OK;
  cudaSetDevice(ctx->device);
  cudaStreamSynchronize(ctx->stream);
  for (skc_plan* p : std::vector<skc_plan*>(ctx->plans.begin(), ctx->plans.end()))
    release_plan_memory(p);
  for (skc_result* r : std::vector<skc_result*>(ctx->results.begin(), ctx->results.end()))
    release_result_memory(r);
  for (skc_dataset* ds : std::vector<skc_dataset*>(ctx->datasets.begin(), ctx->datasets.end()))
    release_dataset_memory(ds);
  cudaStreamSynchronize(ctx->stream);
  for (auto* p : ctx->d_level_tables)
    if (p) cudaFree(p);
  cudaEventDestroy(ctx->ev_start);
  cudaEventDestroy(ctx->ev_stop);
  cudaStreamDestroy(ctx->stream);
  delete ctx;
  return SKC_OK;
}

static int upload_on(skc_context* ctx, cudaStream_t s, const float* rows, uint64_t n,
                     int d, bool from_host, skc_dataset** out);

static int upload_common(skc_context* ctx, const float* rows, uint64_t n, int d,
                         bool from_host, skc_dataset** out) {
  clear_error();
  if (!ctx || !rows || !out) return set_error(SKC_ERR_INVALID, "NULL argument");
  if (!from_host) {
    SKC_CUDA(cudaSetDevice(ctx->device));
    SKC_TRY(check_device_pointer(rows, ctx->device, "d_rows"));
  }
  return upload_on(ctx, ctx->stream, rows, n, d, from_host, out);
}

// Uploads on stream s (the context's stream, or a serving slot's).
static int upload_on(skc_context* ctx, cudaStream_t s, const float* rows, uint64_t n,
                     int d, bool from_host, skc_dataset** out) {
  *out = nullptr;
  if (d < SKC_MIN_DIMS || d > SKC_MAX_DIMS)
    return set_error(SKC_ERR_INVALID, "d=%d outside [%d,%d]", d, SKC_MIN_DIMS, SKC_MAX_DIMS);
  if (n == 0) return set_error(SKC_ERR_INVALID, "empty dataset (n=0)");
  if (n > 0xffffff00ull) return set_error(SKC_ERR_UNSUPPORTED, "n=%llu exceeds 32-bit point ids", (unsigned long long)n);
  SKC_CUDA(cudaSetDevice(ctx->device));
  auto* ds = new skc_dataset;
  ds->ctx = ctx;
  ds->stream = s;
  ds->n = n;
  ds->d = d;
  ds->n_pad = round_up(n, 128);
  Arena A(s);
  int st = SKC_OK;
  const float* d_rows = rows;
  uint32_t* bad = nullptr;
  uint32_t h_bad = 0;
  do {
    cudaError_t e = cudaMallocAsync((void**)&ds->x, (size_t)d * ds->n_pad * sizeof(float), s);
    if (e != cudaSuccess) { st = set_error(SKC_ERR_OOM, "dataset allocation failed: %s", cudaGetErrorString(e)); break; }
    if (from_host) {
      float* tmp;
      if ((st = A.alloc(&tmp, n * d)) != SKC_OK) break;
      if ((st = copy_h2d(tmp, rows, n * d * sizeof(float), s)) != SKC_OK) break;
      d_rows = tmp;
    }
    if ((st = A.alloc(&bad, 1)) != SKC_OK) break;
    if (cudaMemsetAsync(bad, 0, sizeof(uint32_t), s) != cudaSuccess) { st = set_error(SKC_ERR_CUDA, "memset"); break; }
    if ((st = launch_rows_to_soa(s, d_rows, n, d, ds->n_pad, ds->x, bad)) != SKC_OK) break;
    if ((st = copy_d2h(&h_bad, bad, sizeof(uint32_t), s)) != SKC_OK) break;
    if (h_bad) st = set_error(SKC_ERR_INVALID, "%u non-finite attribute values (NaN/inf) rejected", h_bad);
  } while (0);
  if (st != SKC_OK) {
    if (ds->x) cudaFreeAsync(ds->x, s);
    delete ds;
    return st;
  }
  {
    std::lock_guard<std::mutex> lock(ctx->mu);
    ctx->datasets.insert(ds);
  }
  *out = ds;
  return SKC_OK;
}

int skc_dataset_upload(skc_context* ctx, const float* rows, uint64_t n, int d, skc_dataset** out) {
  return upload_common(ctx, rows, n, d, true, out);
}

int skc_dataset_upload_device(skc_context* ctx, const float* d_rows, uint64_t n, int d,
                              skc_dataset** out) {
  return upload_common(ctx, d_rows, n, d, false, out);
}

int skc_dataset_free(skc_dataset* ds) {
  clear_error();
  if (!ds) return SKC_OK;
  if (ds->ctx) {
    skc_context* ctx = ds->ctx;
    cudaStream_t s = ds->stream ? ds->stream : ctx->stream;
    cudaSetDevice(ctx->device);
    release_dataset_memory(ds);
    cudaStreamSynchronize(s);
  }
  delete ds;
  return SKC_OK;
}

// Validates options against a dataset; fills *o with defaults where unset.
static int check_options(skc_dataset* ds, const skc_options* opt, skc_options* o) {
  skc_options_init(o);
  if (opt) *o = *opt;
  if (o->algo != SKC_ALGO_MDMC && o->algo != SKC_ALGO_SDSC)
    return set_error(SKC_ERR_INVALID, "unknown algorithm %d", o->algo);
  if (o->mode != SKC_MODE_PLAIN && o->mode != SKC_MODE_BATCHED)
    return set_error(SKC_ERR_INVALID, "unknown mode %d", o->mode);
  if (o->depth < 0 || o->depth > kMaxDepth)
    return set_error(SKC_ERR_INVALID, "depth %d outside [1,%d] (0 = auto)", o->depth, kMaxDepth);
  if (o->subspace >= (1u << ds->d))
    return set_error(SKC_ERR_INVALID, "subspace 0x%x has attributes beyond d=%d", o->subspace, ds->d);
  if (o->pq_size > kMaxPruners)
    return set_error(SKC_ERR_INVALID, "pq_size %d above %d", o->pq_size, kMaxPruners);
  if (o->tile_points != 0 &&
      (o->tile_points < 32 || o->tile_points > 65536 || (o->tile_points & (o->tile_points - 1))))
    return set_error(SKC_ERR_INVALID, "tile_points %d is not a power of two in [32, 65536]",
                     o->tile_points);
  if (o->chunk < 0 || o->chunk > 64)
    return set_error(SKC_ERR_INVALID, "chunk %d outside [1, 64] (0 = auto)", o->chunk);
  if (o->blocks_per_sm < 0 || o->blocks_per_sm > 32)
    return set_error(SKC_ERR_INVALID, "blocks_per_sm %d outside [1, 32] (0 = auto)",
                     o->blocks_per_sm);
  if (o->form != 0 && o->form != SKC_FORM_BITMAPS && o->form != SKC_FORM_LEVELS)
    return set_error(SKC_ERR_INVALID, "form %d is not 0, SKC_FORM_BITMAPS or SKC_FORM_LEVELS",
                     o->form);
  return SKC_OK;
}

// Skyline query: one cuboid S only. The full-space skyline plus extended
// skyline holds every point that can be in S's skyline or extended skyline
// (a point strictly dominated in the full space is strictly dominated in S),
// so S is computed over those candidates.
static int run_single_cuboid(Exec& E, skc_dataset* ds, uint32_t S, const RunParams& P,
                             Arena& A, FullSpace& F, skc_result* R, Tracer& T) {
  const int depth = P.depth;
  cudaStream_t s = E.stream;
  const int d = ds->d;
  const uint32_t nsub = 1u << d, full = nsub - 1;
  uint32_t *sky = F.sky, *ext = F.ext;
  uint64_t nsky = F.h_counts[0], next = F.h_counts[1];
  if (S != full) {
    const uint64_t m = F.h_counts[2];
    LevelTables LT;
    SKC_TRY(level_tables(E.ctx, partition_dims(S), &LT));
    const uint32_t K = 1u << LT.B;
    PartScratch ps;
    SKC_TRY(A.alloc(&ps.keys, m));
    SKC_TRY(A.alloc(&ps.sorted, m));
    SKC_TRY(A.alloc(&ps.ccells, m));
    SKC_TRY(A.alloc(&ps.cx, (uint64_t)d * round_up(m, 128)));
    SKC_TRY(A.alloc(&ps.counts, K + 1));
    SKC_TRY(A.alloc(&ps.cursor, kMaxSortBuckets + 1));
    SKC_TRY(A.alloc(&ps.fine, kMaxSortBuckets + 1));
    SKC_TRY(A.alloc(&ps.items, K + 1));
    SKC_TRY(A.alloc(&ps.spread, 3));
    if (m >= kConfirmedMinPoints) {
      SKC_TRY(A.alloc(&ps.conf_cells, m));
      SKC_TRY(A.alloc(&ps.conf_x, (uint64_t)d * round_up(m, 128)));
      SKC_TRY(A.alloc(&ps.ccount, K));
      SKC_TRY(A.alloc(&ps.pdone, K));
    }
    uint8_t* status;
    uint32_t *blk0, *blk1, *cnt;
    SKC_TRY(A.alloc(&status, round_up(m, 4)));
    const uint64_t nblk = (m + 1023) / 1024 + 1;
    SKC_TRY(A.alloc(&blk0, nblk));
    SKC_TRY(A.alloc(&blk1, nblk));
    SKC_TRY(A.alloc(&cnt, 2));
    SKC_TRY(A.alloc(&sky, m));
    SKC_TRY(A.alloc(&ext, m));
    const uint32_t* list = F.cand;
    const uint32_t* m_ptr = F.counts + 2;
    const bool filter = P.pq_size > 0 && m > 2ull * (uint64_t)P.pq_size;
    if (filter) {
      // The prefilter on S over the full-space candidates (same argument as
      // in the full space: every dominator of a survivor on S survives).
      const uint32_t Kq = (uint32_t)P.pq_size;
      PrefilterScratch pf;
      SKC_TRY(A.alloc(&pf.hist, prefilter_sum_bins()));
      SKC_TRY(A.alloc(&pf.sel, 8));
      SKC_TRY(A.alloc(&pf.pr_ids, Kq));
      SKC_TRY(A.alloc(&pf.pr_key, Kq));
      SKC_TRY(A.alloc(&pf.pr_cells, Kq));
      SKC_TRY(A.alloc(&pf.pr_x, (uint64_t)d * Kq));
      SKC_TRY(A.alloc(&pf.st, m));
      SKC_TRY(A.alloc(&pf.blk0, nblk));
      SKC_TRY(A.alloc(&pf.blk1, nblk));
      SKC_TRY(A.alloc(&pf.mid_ids, m));
      SKC_TRY(A.alloc(&pf.mid_count, 1));
      uint32_t *surv, *d_ns;
      SKC_TRY(A.alloc(&surv, m));
      SKC_TRY(A.alloc(&d_ns, 1));
      PrefilterArgs pfa{F.cells, ds->x, ds->n_pad, F.cand, m_ptr, m, S, Kq, pf};
      SKC_TRY(launch_prefilter(s, d, E.ctx->num_sms, pfa, surv, d_ns));
      list = surv;
      m_ptr = d_ns;
    }
    PartitionSkylineArgs pa{list, F.cells, ds->x, ds->n_pad, m_ptr, m, S, status};
    if (filter) {
      pa.split_target = (uint32_t)E.ctx->num_sms * kSplitCtasPerSm;
      pa.spread_ids = F.cand;  // the spread of the candidates on S picks the order
      pa.spread_m = F.counts + 2;
    }
    SKC_TRY(launch_partition_skyline(s, d, depth, LT, pa, ps));
    SKC_TRY(launch_status_compact(s, status, list, m_ptr, m, 0, blk0, blk1, sky, ext, cnt, cnt + 1));
    uint32_t h[2] = {0, 0};
    SKC_TRY(copy_d2h(h, cnt, sizeof(h), s));
    nsky = h[0];
    next = h[1];
    T.mark("subspace skyline");
  }
  for (int pass = 0; pass < 2; ++pass) {
    std::vector<uint64_t> off(nsub + 1, 0);
    const uint64_t cntc = pass == 0 ? nsky : next;
    for (uint32_t c = 0; c < nsub; ++c) off[c + 1] = off[c] + (c == S ? cntc : 0);
    uint64_t* d_off;
    SKC_TRY(A.alloc(&d_off, nsub + 1));
    SKC_TRY(copy_h2d(d_off, off.data(), (nsub + 1) * sizeof(uint64_t), s));
    SKC_CUDA(cudaStreamSynchronize(s));  // `off` is a host temporary
    uint32_t* ids = pass == 0 ? sky : ext;
    A.release(d_off);
    A.release(ids);
    if (pass == 0) {
      R->d_off = d_off;
      R->d_ids = ids;
      R->total_ids = cntc;
    } else {
      R->d_eoff = d_off;
      R->d_eids = ids;
      R->total_ext = cntc;
    }
  }
  return SKC_OK;
}

// Runs one skycube (or skyline query) on E's stream; on success *out is a
// new result registered with the context.
// `forced`, when given, replaces the resolution of the work parameters (the
// autotuner's trials).
static int skycube_exec(Exec& E, skc_dataset* ds, const skc_options* opt, skc_result** out,
                        const RunParams* forced = nullptr) {
  skc_context* ctx = E.ctx;
  skc_options o;
  SKC_TRY(check_options(ds, opt, &o));
  const int d = ds->d;
  const int max_d = (o.max_d <= 0 || o.max_d > d) ? d : o.max_d;
  SKC_CUDA(cudaSetDevice(ctx->device));
  cudaStream_t s = E.stream;
  RunParams P;
  if (forced) P = *forced;
  else SKC_TRY(resolve_params(ds, s, o, max_d, &P));
  const int depth = P.depth;

  auto* R = new skc_result;
  R->ctx = ctx;
  R->stream = s;
  R->d = d;
  R->max_d = o.subspace ? __builtin_popcount(o.subspace) : max_d;
  R->algo = o.algo;
  int st = SKC_OK;
  {
    Arena A(s);
    FullSpace F;
    Tracer T(E);
    st = run_full_space(E, ds, P, A, F, T);
    if (st == SKC_OK) {
      R->n_cand = F.h_counts[2];
      if (o.subspace) {
        R->form = SKC_FORM_SKYLINE;
        st = run_single_cuboid(E, ds, o.subspace, P, A, F, R, T);
      } else if (o.algo == SKC_ALGO_SDSC && o.mode == SKC_MODE_PLAIN) {
        R->form = SKC_FORM_CUBOIDS;
        st = run_sdsc_plain(E, ds, max_d, depth, A, F, R, T);
      } else if (use_levels(E, ds, o, max_d, F)) {
        R->form = SKC_FORM_LEVELS;
        st = run_levels(E, ds, o, max_d, depth, A, F, R, T);
        if (st == kLvGiveUp) {
          R->form = SKC_FORM_BITMAPS;
          st = run_bitmaps(E, ds, o, P, max_d, A, F, R, T);
        }
      } else {
        R->form = SKC_FORM_BITMAPS;
        st = run_bitmaps(E, ds, o, P, max_d, A, F, R, T);
      }
    }
    T.mark("end");
  }
  if (st == SKC_OK) {
    cudaError_t e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) st = set_error(SKC_ERR_CUDA, "skycube failed: %s", cudaGetErrorString(e));
  }
  if (st != SKC_OK) {
    std::string msg = g_err;
    skc_result_free(R);
    g_err = msg;
    return st;
  }
  {
    std::lock_guard<std::mutex> lock(ctx->mu);
    ctx->results.insert(R);
  }
  *out = R;
  return SKC_OK;
}

// Several skycubes in one pass: every dataset's full-space step, then ONE
// lattice launch shared by all the datasets whose skycube takes the lattice
// form, the other forms dataset by dataset. results[i] equals what
// skycube_exec gives for dataset i alone.
static int skycube_exec_batch(Exec& E, const std::vector<skc_dataset*>& dss,
                              const std::vector<skc_options>& opts,
                              std::vector<skc_result*>* out) {
  skc_context* ctx = E.ctx;
  const size_t nb = dss.size();
  out->assign(nb, nullptr);
  SKC_CUDA(cudaSetDevice(ctx->device));
  cudaStream_t s = E.stream;
  std::vector<skc_options> o(nb);
  std::vector<int> max_d(nb);
  std::vector<RunParams> P(nb);
  for (size_t i = 0; i < nb; ++i) {
    SKC_TRY(check_options(dss[i], &opts[i], &o[i]));
    const int d = dss[i]->d;
    max_d[i] = (o[i].max_d <= 0 || o[i].max_d > d) ? d : o[i].max_d;
    SKC_TRY(resolve_params(dss[i], s, o[i], max_d[i], &P[i]));
  }
  std::vector<skc_result*> R(nb, nullptr);
  for (size_t i = 0; i < nb; ++i) {
    R[i] = new skc_result;
    R[i]->ctx = ctx;
    R[i]->stream = s;
    R[i]->d = dss[i]->d;
    R[i]->max_d = o[i].subspace ? __builtin_popcount(o[i].subspace) : max_d[i];
    R[i]->algo = o[i].algo;
  }
  int st = SKC_OK;
  {
    Arena A(s);
    Tracer T(E);
    std::vector<FullSpace> F(nb);  // referenced by the lattice jobs: no reallocation
    std::vector<LatticeJob> jobs;
    std::vector<size_t> job_of;
    for (size_t i = 0; i < nb && st == SKC_OK; ++i) {
      skc_dataset* ds = dss[i];
      st = run_full_space(E, ds, P[i], A, F[i], T);
      if (st != SKC_OK) break;
      R[i]->n_cand = F[i].h_counts[2];
      if (o[i].subspace) {
        R[i]->form = SKC_FORM_SKYLINE;
        st = run_single_cuboid(E, ds, o[i].subspace, P[i], A, F[i], R[i], T);
      } else if (o[i].algo == SKC_ALGO_SDSC && o[i].mode == SKC_MODE_PLAIN) {
        R[i]->form = SKC_FORM_CUBOIDS;
        st = run_sdsc_plain(E, ds, max_d[i], P[i].depth, A, F[i], R[i], T);
      } else if (use_levels(E, ds, o[i], max_d[i], F[i])) {
        LatticeJob J;
        J.ds = ds;
        J.max_d = max_d[i];
        J.depth = P[i].depth;
        J.want_ext = o[i].want_extended || o[i].algo == SKC_ALGO_SDSC;
        J.F = &F[i];
        J.R = R[i];
        jobs.push_back(std::move(J));
        job_of.push_back(i);
      } else {
        R[i]->form = SKC_FORM_BITMAPS;
        st = run_bitmaps(E, ds, o[i], P[i], max_d[i], A, F[i], R[i], T);
      }
    }
    if (st == SKC_OK && !jobs.empty()) {
      st = run_lattice(E, jobs, A, T);
      for (size_t k = 0; k < jobs.size() && st == SKC_OK; ++k) {
        const size_t i = job_of[k];
        R[i]->form = SKC_FORM_LEVELS;
        if (jobs[k].status == kLvGiveUp) {
          R[i]->form = SKC_FORM_BITMAPS;
          st = run_bitmaps(E, dss[i], o[i], P[i], max_d[i], A, F[i], R[i], T);
        }
      }
    }
    T.mark("end");
  }
  if (st == SKC_OK) {
    cudaError_t e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) st = set_error(SKC_ERR_CUDA, "skycube batch failed: %s", cudaGetErrorString(e));
  }
  if (st != SKC_OK) {
    std::string msg = g_err;
    for (auto* r : R) skc_result_free(r);
    g_err = msg;
    return st;
  }
  {
    std::lock_guard<std::mutex> lock(ctx->mu);
    for (auto* r : R) ctx->results.insert(r);
  }
  *out = R;
  return SKC_OK;
}

int skc_skycube_batch(skc_context* ctx, skc_dataset* const* datasets, const skc_options* opts,
                      int count, skc_result** results) {
  clear_error();
  if (!ctx || !datasets || !results || count < 0) return set_error(SKC_ERR_INVALID, "NULL argument");
  std::vector<skc_dataset*> dss(count);
  std::vector<skc_options> o(count);
  for (int i = 0; i < count; ++i) {
    results[i] = nullptr;
    if (!datasets[i]) return set_error(SKC_ERR_INVALID, "dataset %d is NULL", i);
    if (datasets[i]->ctx != ctx)
      return set_error(SKC_ERR_INVALID, "dataset %d belongs to another (or a destroyed) context", i);
    dss[i] = datasets[i];
    if (opts) o[i] = opts[i];
    else skc_options_init(&o[i]);
  }
  Exec E;
  E.ctx = ctx;
  E.stream = ctx->stream;
  std::vector<skc_result*> R;
  const int st = skycube_exec_batch(E, dss, o, &R);
  ctx->phases = E.phases;
  ctx->last_ms = E.ms;
  if (st == SKC_OK)
    for (int i = 0; i < count; ++i) results[i] = R[i];
  return st;
}

int skc_skycube(skc_context* ctx, skc_dataset* ds, const skc_options* opt, skc_result** out) {
  clear_error();
  if (!ctx || !ds || !out) return set_error(SKC_ERR_INVALID, "NULL argument");
  *out = nullptr;
  if (ds->ctx != ctx) return set_error(SKC_ERR_INVALID, "dataset belongs to another (or a destroyed) context");
  Exec E;
  E.ctx = ctx;
  E.stream = ctx->stream;
  const int st = skycube_exec(E, ds, opt, out);
  ctx->phases = E.phases;
  ctx->last_ms = E.ms;
  return st;
}

}  // extern "C"

// The batched pipeline in plan mode on stream s: RECORD runs it eagerly and
// allocates the plan's buffers, REPLAY re-issues the identical launch
// sequence on those buffers (inside a stream capture).
static int plan_pipeline(skc_plan* p, Arena::Mode mode, cudaStream_t s) {
  Exec E;
  E.ctx = p->ctx;
  E.stream = s;
  E.plan = &p->caps;
  Arena A(s, mode, &p->bufs);
  SKC_TRY(A.alloc(&p->caps.stats, 4));
  FullSpace F;
  Tracer T(E);
  skc_result& R = p->outs;
  R.d = p->ds->d;
  R.max_d = p->max_d;
  R.algo = p->opt.algo;
  SKC_TRY(run_full_space(E, p->ds, p->P, A, F, T));
  SKC_TRY(run_bitmaps(E, p->ds, p->opt, p->P, p->max_d, A, F, &R, T));
  SKC_CUDA(cudaMemcpyAsync(p->h_stats, p->caps.stats, 3 * sizeof(uint64_t),
                           cudaMemcpyDeviceToHost, s));
  return SKC_OK;
}

static bool plan_fits(const skc_plan* p) {
  const bool ext = p->outs.d_eids != nullptr;
  return p->h_stats[0] <= p->caps.m_cap && p->h_stats[1] <= p->caps.ids_cap[0] &&
         (!ext || p->h_stats[2] <= p->caps.ids_cap[1]);
}

static uint64_t with_slack(uint64_t v) { return v + v / 4 + 1024; }

// Sizes the plan's buffers, records them with an eager run (growing the
// capacities until that run fits), then captures the launch sequence.
static int plan_build(skc_plan* p, uint64_t m_cap, uint64_t ids0, uint64_t ids1) {
  cudaStream_t s = p->ctx->stream;
  for (int tries = 0;; ++tries) {
    plan_release_device(p);
    p->caps.m_cap = std::min<uint64_t>(m_cap, p->ds->n);
    p->caps.ids_cap[0] = ids0;
    p->caps.ids_cap[1] = ids1;
    SKC_TRY(plan_pipeline(p, Arena::RECORD, s));
    SKC_CUDA(cudaStreamSynchronize(s));
    if (plan_fits(p)) break;
    if (tries == 3) return set_error(SKC_ERR_INVALID, "plan capacities do not settle");
    // A clamped candidate count also clamped the totals: grow them more.
    const bool m_over = p->h_stats[0] > p->caps.m_cap;
    m_cap = std::max(m_cap, with_slack(p->h_stats[0]));
    ids0 = std::max(ids0 * (m_over ? 2 : 1), with_slack(p->h_stats[1]));
    ids1 = std::max(ids1 * (m_over ? 2 : 1), with_slack(p->h_stats[2]));
  }
  t_capturing = true;
  cudaError_t e = cudaStreamBeginCapture(s, cudaStreamCaptureModeRelaxed);
  int st = e == cudaSuccess
               ? plan_pipeline(p, Arena::REPLAY, s)
               : set_error(SKC_ERR_CUDA, "stream capture failed: %s", cudaGetErrorString(e));
  cudaGraph_t g = nullptr;
  const cudaError_t e2 = e == cudaSuccess ? cudaStreamEndCapture(s, &g) : cudaSuccess;
  t_capturing = false;
  if (st != SKC_OK) {
    if (g) cudaGraphDestroy(g);
    return st;
  }
  if (e2 != cudaSuccess || !g)
    return set_error(SKC_ERR_CUDA, "stream capture failed: %s", cudaGetErrorString(e2));
  p->graph = g;
  SKC_CUDA(cudaGraphInstantiate(&p->exec, g, 0));
  size_t nn = 0;
  SKC_CUDA(cudaGraphGetNodes(g, nullptr, &nn));
  std::vector<cudaGraphNode_t> nodes(nn);
  SKC_CUDA(cudaGraphGetNodes(g, nodes.data(), &nn));
  p->kernels = 0;
  for (cudaGraphNode_t node : nodes) {
    cudaGraphNodeType t;
    SKC_CUDA(cudaGraphNodeGetType(node, &t));
    if (t == cudaGraphNodeTypeKernel) ++p->kernels;
  }
  return SKC_OK;
}

// Device copy of a plan output into memory the result owns.
template <typename T>
static int copy_out(cudaStream_t s, const T* src, uint64_t count, T** dst) {
  *dst = nullptr;
  if (!src) return SKC_OK;
  SKC_CUDA(cudaMallocAsync((void**)dst, std::max<uint64_t>(count, 1) * sizeof(T), s));
  if (count) SKC_CUDA(cudaMemcpyAsync(*dst, src, count * sizeof(T), cudaMemcpyDeviceToDevice, s));
  return SKC_OK;
}

extern "C" {

int skc_plan_create(skc_context* ctx, skc_dataset* ds, const skc_options* opt, skc_plan** out) {
  clear_error();
  if (!ctx || !ds || !out) return set_error(SKC_ERR_INVALID, "NULL argument");
  *out = nullptr;
  if (ds->ctx != ctx) return set_error(SKC_ERR_INVALID, "dataset belongs to another (or a destroyed) context");
  skc_options o;
  SKC_TRY(check_options(ds, opt, &o));
  if (o.mode != SKC_MODE_BATCHED || o.subspace)
    return set_error(SKC_ERR_UNSUPPORTED, "plans capture the BATCHED skycube only");
  SKC_CUDA(cudaSetDevice(ctx->device));
  auto* p = new skc_plan;
  p->ctx = ctx;
  p->ds = ds;
  p->opt = o;
  p->max_d = (o.max_d <= 0 || o.max_d > ds->d) ? ds->d : o.max_d;
  int st = resolve_params(ds, ctx->stream, o, p->max_d, &p->P);
  // One ordinary run gives the sizes the capacities start from.
  skc_result* R = nullptr;
  if (st == SKC_OK) {
    Exec E;
    E.ctx = ctx;
    E.stream = ctx->stream;
    st = skycube_exec(E, ds, &o, &R, &p->P);
  }
  if (st == SKC_OK && cudaMallocHost(&p->h_stats, 4 * sizeof(uint64_t)) != cudaSuccess)
    st = set_error(SKC_ERR_OOM, "pinned host allocation failed");
  if (st == SKC_OK) {
    {
      std::lock_guard<std::mutex> lock(ctx->mu);
      ctx->plans.insert(p);
    }
    st = plan_build(p, with_slack(R->n_cand), with_slack(R->total_ids), with_slack(R->total_ext));
  }
  if (R) skc_result_free(R);
  if (st != SKC_OK) {
    std::string msg = g_err;
    release_plan_memory(p);
    if (p->h_stats) cudaFreeHost(p->h_stats);
    delete p;
    g_err = msg;
    return st;
  }
  *out = p;
  return SKC_OK;
}

int skc_plan_execute(skc_plan* p, skc_result** out) {
  clear_error();
  if (!p) return set_error(SKC_ERR_INVALID, "NULL plan");
  if (out) *out = nullptr;
  if (!p->ctx) return set_error(SKC_ERR_INVALID, "plan's context was destroyed");
  if (!p->ds) return set_error(SKC_ERR_INVALID, "plan's dataset was freed");
  skc_context* ctx = p->ctx;
  cudaStream_t s = ctx->stream;
  SKC_CUDA(cudaSetDevice(ctx->device));
  for (int attempt = 0;; ++attempt) {
    SKC_CUDA(cudaEventRecord(ctx->ev_start, s));
    SKC_CUDA(cudaGraphLaunch(p->exec, s));
    SKC_CUDA(cudaEventRecord(ctx->ev_stop, s));
    g_launches.fetch_add(p->kernels, std::memory_order_relaxed);
    SKC_CUDA(cudaStreamSynchronize(s));
    if (plan_fits(p)) break;
    if (attempt == 1) return set_error(SKC_ERR_INVALID, "plan capacities do not settle");
    // The points changed (skc_dataset_update): re-size and capture again.
    ++p->replans;
    const bool m_over = p->h_stats[0] > p->caps.m_cap;
    SKC_TRY(plan_build(p, std::max(p->caps.m_cap, with_slack(p->h_stats[0])),
                       std::max(p->caps.ids_cap[0] * (m_over ? 2 : 1), with_slack(p->h_stats[1])),
                       std::max(p->caps.ids_cap[1] * (m_over ? 2 : 1), with_slack(p->h_stats[2]))));
  }
  float ms = 0.f;
  SKC_CUDA(cudaEventElapsedTime(&ms, ctx->ev_start, ctx->ev_stop));
  ctx->last_ms = ms;
  ctx->phases.assign(1, {std::string("plan graph"), ms});
  if (!out) return SKC_OK;
  const uint64_t m = p->h_stats[0];
  const uint32_t nsub = 1u << p->ds->d;
  auto* R = new skc_result;
  R->ctx = ctx;
  R->stream = s;
  R->d = p->outs.d;
  R->max_d = p->outs.max_d;
  R->form = SKC_FORM_BITMAPS;
  R->algo = p->outs.algo;
  R->n_cand = m;
  R->total_ids = p->h_stats[1];
  R->total_ext = p->outs.d_eids ? p->h_stats[2] : 0;
  R->words = p->outs.words;
  int st = copy_out(s, p->outs.d_off, nsub + 1, &R->d_off);
  if (st == SKC_OK) st = copy_out(s, p->outs.d_ids, R->total_ids, &R->d_ids);
  if (st == SKC_OK) st = copy_out(s, p->outs.d_eoff, nsub + 1, &R->d_eoff);
  if (st == SKC_OK) st = copy_out(s, p->outs.d_eids, R->total_ext, &R->d_eids);
  if (st == SKC_OK) st = copy_out(s, p->outs.d_bits, m * p->outs.words, &R->d_bits);
  if (st == SKC_OK) st = copy_out(s, p->outs.d_cand, m, &R->d_cand);
  if (st == SKC_OK && cudaStreamSynchronize(s) != cudaSuccess)
    st = set_error(SKC_ERR_CUDA, "plan result copy failed");
  {
    std::lock_guard<std::mutex> lock(ctx->mu);
    ctx->results.insert(R);
  }
  if (st != SKC_OK) {
    std::string msg = g_err;
    skc_result_free(R);
    g_err = msg;
    return st;
  }
  *out = R;
  return SKC_OK;
}

int skc_plan_info(skc_plan* p, uint64_t* kernels, uint64_t* replans, uint64_t* cand_capacity,
                  uint64_t* ids_capacity) {
  clear_error();
  if (!p) return set_error(SKC_ERR_INVALID, "NULL plan");
  if (kernels) *kernels = p->kernels;
  if (replans) *replans = p->replans;
  if (cand_capacity) *cand_capacity = p->caps.m_cap;
  if (ids_capacity) *ids_capacity = p->caps.ids_cap[0];
  return SKC_OK;
}

int skc_plan_destroy(skc_plan* p) {
  if (!p) return SKC_OK;
  if (p->ctx) {
    cudaSetDevice(p->ctx->device);
    cudaStreamSynchronize(p->ctx->stream);
    release_plan_memory(p);
  }
  delete p;
  return SKC_OK;
}

int skc_dataset_update(skc_dataset* ds, const float* rows) {
  clear_error();
  if (!ds || !rows) return set_error(SKC_ERR_INVALID, "NULL argument");
  skc_context* ctx = ds->ctx;
  if (!ctx) return set_error(SKC_ERR_INVALID, "dataset's context was destroyed");
  SKC_CUDA(cudaSetDevice(ctx->device));
  cudaStream_t s = ctx->stream;
  const uint64_t n = ds->n;
  const int d = ds->d;
  uint32_t h_bad = 0;
  {
    Arena A(s);
    float *tmp, *soa;
    uint32_t* bad;
    SKC_TRY(A.alloc(&tmp, n * d));
    SKC_TRY(A.alloc(&soa, (uint64_t)d * ds->n_pad));
    SKC_TRY(A.alloc(&bad, 1));
    SKC_TRY(copy_h2d(tmp, rows, n * d * sizeof(float), s));
    SKC_CUDA(cudaMemsetAsync(bad, 0, sizeof(uint32_t), s));
    SKC_TRY(launch_rows_to_soa(s, tmp, n, d, ds->n_pad, soa, bad));
    SKC_TRY(copy_d2h(&h_bad, bad, sizeof(uint32_t), s));
    if (!h_bad) {
      // The dataset may live on another stream: order the copy after it.
      if (ds->stream && ds->stream != s) SKC_CUDA(cudaStreamSynchronize(ds->stream));
      SKC_CUDA(cudaMemcpyAsync(ds->x, soa, (size_t)d * ds->n_pad * sizeof(float),
                               cudaMemcpyDeviceToDevice, s));
      SKC_CUDA(cudaStreamSynchronize(s));
    }
  }
  if (h_bad) return set_error(SKC_ERR_INVALID, "%u non-finite attribute values (NaN/inf) rejected", h_bad);
  std::lock_guard<std::mutex> lock(ctx->mu);
  ds->sig_ready = false;
  return SKC_OK;
}

int skc_autotune(skc_context* ctx, skc_dataset* ds, const skc_options* base, int repeats,
                 skc_options* best, float* best_ms) {
  clear_error();
  if (!ctx || !ds) return set_error(SKC_ERR_INVALID, "NULL argument");
  if (ds->ctx != ctx) return set_error(SKC_ERR_INVALID, "dataset belongs to another (or a destroyed) context");
  skc_options o;
  SKC_TRY(check_options(ds, base, &o));
  if (repeats <= 0) repeats = 2;
  if (repeats > 16) repeats = 16;
  const int d = ds->d;
  const int max_d = (o.max_d <= 0 || o.max_d > d) ? d : o.max_d;
  const uint64_t n = ds->n;
  Exec E;
  E.ctx = ctx;
  E.stream = ctx->stream;
  SKC_CUDA(cudaSetDevice(ctx->device));
  uint32_t sig[3];
  SKC_TRY(dataset_signature(ds, E.stream, sig));

  // Start from the explicit options and the defaults (not from the table).
  RunParams cur;
  cur.depth = o.depth ? o.depth : auto_depth(n, d);
  const int pq0 = o.pq_size > 0 ? o.pq_size
                  : o.pq_size < 0 ? 0
                                  : (n >= kPrefilterMinPoints ? kDefaultPruners : 0);
  cur.pq_size = (pq0 > 0 && n > 2ull * (uint64_t)pq0) ? pq0 : 0;
  cur.tile_points = o.tile_points ? o.tile_points : kDefaultTilePoints;
  cur.chunk = o.chunk ? o.chunk : kDefaultChunk;
  cur.blocks_per_sm = o.blocks_per_sm;

  auto time_run = [&](const RunParams& P, float* ms) -> int {
    float bestv = 3.0e38f;
    for (int r = 0; r < repeats; ++r) {
      skc_result* R = nullptr;
      SKC_TRY(skycube_exec(E, ds, &o, &R, &P));
      bestv = std::min(bestv, E.ms);
      skc_result_free(R);
    }
    *ms = bestv;
    return SKC_OK;
  };
  float cur_ms = 0.f;
  SKC_TRY(time_run(cur, &cur_ms));

  // One pass of coordinate search over the parameters the options leave
  // automatic; a change is kept when it is at least 2% faster.
  const bool bitmap_stage = !o.subspace && !(o.algo == SKC_ALGO_SDSC && o.mode == SKC_MODE_PLAIN);
  auto try_values = [&](int RunParams::*field, const std::vector<int>& values) -> int {
    for (int v : values) {
      if (cur.*field == v) continue;
      RunParams P = cur;
      P.*field = v;
      float ms = 0.f;
      SKC_TRY(time_run(P, &ms));
      if (ms < 0.98f * cur_ms) {
        cur = P;
        cur_ms = ms;
      }
    }
    return SKC_OK;
  };
  if (!o.depth) SKC_TRY(try_values(&RunParams::depth, {7, 6, 5, 4, 3, 2}));
  if (!o.pq_size) {
    std::vector<int> pqs;
    for (int v : {0, 32, 128, 512, kMaxPruners})
      if (v == 0 || n > 2ull * (uint64_t)v) pqs.push_back(v);
    SKC_TRY(try_values(&RunParams::pq_size, pqs));
  }
  if (bitmap_stage) {
    if (!o.tile_points) SKC_TRY(try_values(&RunParams::tile_points, {64, 256, 1024}));
    if (!o.chunk) SKC_TRY(try_values(&RunParams::chunk, {1, 4, 16}));
    if (!o.blocks_per_sm) SKC_TRY(try_values(&RunParams::blocks_per_sm, {0, 1, 2}));
  }
  {
    std::lock_guard<std::mutex> lock(ctx->mu);
    ctx->tunings[tuning_key(ds, sig, o, max_d)] =
        skc_context::Tuned{cur.depth, cur.pq_size, cur.tile_points, cur.chunk, cur.blocks_per_sm,
                           cur_ms};
  }
  if (best) {
    *best = o;
    best->depth = cur.depth;
    best->pq_size = cur.pq_size > 0 ? cur.pq_size : -1;
    best->tile_points = cur.tile_points;
    best->chunk = cur.chunk;
    best->blocks_per_sm = cur.blocks_per_sm;
  }
  if (best_ms) *best_ms = cur_ms;
  ctx->phases = E.phases;
  ctx->last_ms = E.ms;
  return SKC_OK;
}

int skc_dataset_signature(skc_dataset* ds, int* size_class, int* sky_class, int* ties) {
  clear_error();
  if (!ds) return set_error(SKC_ERR_INVALID, "NULL dataset");
  if (!ds->ctx) return set_error(SKC_ERR_INVALID, "dataset's context was destroyed");
  SKC_CUDA(cudaSetDevice(ds->ctx->device));
  uint32_t sig[3];
  SKC_TRY(dataset_signature(ds, ds->ctx->stream, sig));
  int sc, kc, t;
  signature_classes(ds, sig, &sc, &kc, &t);
  if (size_class) *size_class = sc;
  if (sky_class) *sky_class = kc;
  if (ties) *ties = t;
  return SKC_OK;
}

int skc_tuning_count(skc_context* ctx, uint64_t* count) {
  clear_error();
  if (!ctx || !count) return set_error(SKC_ERR_INVALID, "NULL argument");
  std::lock_guard<std::mutex> lock(ctx->mu);
  *count = ctx->tunings.size();
  return SKC_OK;
}

int skc_tuning_clear(skc_context* ctx) {
  clear_error();
  if (!ctx) return set_error(SKC_ERR_INVALID, "NULL context");
  std::lock_guard<std::mutex> lock(ctx->mu);
  ctx->tunings.clear();
  return SKC_OK;
}

int skc_result_form(skc_result* r, int* form, int* fallbacks) {
  clear_error();
  if (!r) return set_error(SKC_ERR_INVALID, "NULL result");
  if (form) *form = r->form;
  if (fallbacks) *fallbacks = r->level_fallbacks;
  return SKC_OK;
}

int skc_result_info(skc_result* r, int* d, uint64_t* n_cand, uint64_t* total) {
  clear_error();
  if (!r) return set_error(SKC_ERR_INVALID, "NULL result");
  if (d) *d = r->d;
  if (n_cand) *n_cand = r->n_cand;
  if (total) *total = r->total_ids;
  return SKC_OK;
}

// Gives `v` at least n entries, from the context's pool of recycled host
// buffers when one is large enough (its contents are overwritten by the
// copy; entries past n are unused, views index through the offsets).
static void take_host_buffer(skc_context* ctx, std::vector<uint32_t>& v, size_t n) {
  if (v.size() >= n) return;
  {
    std::lock_guard<std::mutex> lock(ctx->mu);
    auto& pool = ctx->host_id_pool;
    size_t best = pool.size();
    for (size_t i = 0; i < pool.size(); ++i)
      if (pool[i].size() >= n && (best == pool.size() || pool[i].size() < pool[best].size())) best = i;
    if (best < pool.size()) {
      v.swap(pool[best]);
      pool.erase(pool.begin() + best);
      return;
    }
  }
  v.resize(n);
}

constexpr size_t kHostPoolBuffers = 4;

// Returns a result's host id buffers to its context's pool.
static void recycle_host_buffers(skc_context* ctx, skc_result* r) {
  std::lock_guard<std::mutex> lock(ctx->mu);
  for (auto* v : {&r->h_ids, &r->h_eids}) {
    if (v->empty()) continue;
    if (ctx->host_id_pool.size() < kHostPoolBuffers) ctx->host_id_pool.push_back(std::move(*v));
    v->clear();
  }
}

static int download_csr(skc_result* r, bool ext) {
  bool& done = ext ? r->ext_downloaded : r->downloaded;
  if (done) return SKC_OK;
  if (!r->ctx) return set_error(SKC_ERR_INVALID, "result's context was destroyed");
  const uint64_t* d_off = ext ? r->d_eoff : r->d_off;
  const uint32_t* d_ids = ext ? r->d_eids : r->d_ids;
  if (!d_off) return set_error(SKC_ERR_INVALID, ext ? "extended skylines were not requested" : "no skylines");
  auto& off = ext ? r->h_eoff : r->h_off;
  auto& ids = ext ? r->h_eids : r->h_ids;
  const uint32_t nsub = 1u << r->d;
  cudaStream_t s = r->stream;
  SKC_CUDA(cudaSetDevice(r->ctx->device));
  off.resize(nsub + 1);
  SKC_TRY(copy_d2h(off.data(), d_off, (nsub + 1) * sizeof(uint64_t), s));
  take_host_buffer(r->ctx, ids, off[nsub]);
  SKC_TRY(copy_d2h(ids.data(), d_ids, off[nsub] * sizeof(uint32_t), s));
  done = true;
  return SKC_OK;
}

int skc_result_download(skc_result* r) {
  clear_error();
  if (!r) return set_error(SKC_ERR_INVALID, "NULL result");
  return download_csr(r, false);
}

static int cuboid_view(skc_result* r, uint32_t c, bool ext, const uint32_t** ids, uint64_t* count) {
  clear_error();
  if (!r || !ids || !count) return set_error(SKC_ERR_INVALID, "NULL argument");
  if (c == 0 || c >= (1u << r->d)) return set_error(SKC_ERR_INVALID, "cuboid %u outside [1, 2^%d)", c, r->d);
  SKC_TRY(download_csr(r, ext));
  const auto& off = ext ? r->h_eoff : r->h_off;
  const auto& v = ext ? r->h_eids : r->h_ids;
  *count = off[c + 1] - off[c];
  *ids = v.data() + off[c];
  return SKC_OK;
}

int skc_result_cuboid(skc_result* r, uint32_t c, const uint32_t** ids, uint64_t* count) {
  return cuboid_view(r, c, false, ids, count);
}

int skc_result_extended(skc_result* r, uint32_t c, const uint32_t** ids, uint64_t* count) {
  return cuboid_view(r, c, true, ids, count);
}

int skc_result_device_csr(skc_result* r, const uint64_t** d_off, const uint32_t** d_ids) {
  clear_error();
  if (!r || !d_off || !d_ids) return set_error(SKC_ERR_INVALID, "NULL argument");
  *d_off = r->d_off;
  *d_ids = r->d_ids;
  return SKC_OK;
}

int skc_result_bitmaps(skc_result* r, const uint32_t** bits, const uint32_t** pids,
                       uint64_t* n_points, uint32_t* words) {
  clear_error();
  if (!r || !bits || !pids || !n_points || !words) return set_error(SKC_ERR_INVALID, "NULL argument");
  if (!r->bits_downloaded && !r->ctx) return set_error(SKC_ERR_INVALID, "result's context was destroyed");
  if (!r->bits_downloaded && !r->d_bits) return set_error(SKC_ERR_INVALID, "bitmaps were not requested (want_bitmaps)");
  if (!r->bits_downloaded) {
    SKC_CUDA(cudaSetDevice(r->ctx->device));
    cudaStream_t s = r->stream;
    r->h_bits.resize(r->n_cand * r->words);
    r->h_cand.resize(r->n_cand);
    if (r->n_cand) {
      SKC_TRY(copy_d2h(r->h_bits.data(), r->d_bits, r->h_bits.size() * sizeof(uint32_t), s));
      SKC_TRY(copy_d2h(r->h_cand.data(), r->d_cand, r->n_cand * sizeof(uint32_t), s));
    }
    SKC_CUDA(cudaStreamSynchronize(s));
    r->bits_downloaded = true;
  }
  *bits = r->h_bits.data();
  *pids = r->h_cand.data();
  *n_points = r->n_cand;
  *words = r->words;
  return SKC_OK;
}

int skc_result_free(skc_result* r) {
  if (!r) return SKC_OK;
  if (r->ctx) {
    skc_context* ctx = r->ctx;
    cudaStream_t s = r->stream ? r->stream : ctx->stream;
    cudaSetDevice(ctx->device);
    recycle_host_buffers(ctx, r);
    release_result_memory(r);
    cudaStreamSynchronize(s);
  }
  delete r;
  return SKC_OK;
}

int skc_last_device_ms(skc_context* ctx, float* ms) {
  clear_error();
  if (!ctx || !ms) return set_error(SKC_ERR_INVALID, "NULL argument");
  *ms = ctx->last_ms;
  return SKC_OK;
}

}  // extern "C"

// ==========================================================================
// Serving loop (continuous batching). Requests wait in a FIFO queue; each of
// `slots` workers owns a CUDA stream and host thread. The head request is
// admitted as soon as a worker is free and its estimated device-memory
// footprint fits the budget left by the requests in flight, so requests that
// arrive while others run start as slots and memory free up, and their
// kernels overlap on the device (one stream per slot). A worker uploads the
// points (when the request brought host rows), runs the skycube or skyline
// query, copies the result to host memory and releases the device memory.
namespace {

struct Request {
  uint64_t ticket = 0;
  const float* rows = nullptr;  // host rows to upload, or
  skc_dataset* ds = nullptr;    // a resident dataset
  uint64_t n = 0;
  int d = 0;
  skc_options opt{};
  uint64_t footprint = 0;
  bool heavy = false;  // runs on the slot's low-priority stream
  std::chrono::steady_clock::time_point t_submit, t_start, t_end;
  bool done = false;
  bool claimed = false;  // a skc_server_wait has taken this ticket
  int status = SKC_OK;
  std::string err;
  skc_result* result = nullptr;
  float device_ms = 0.f;
};

double ms_between(std::chrono::steady_clock::time_point a, std::chrono::steady_clock::time_point b) {
  return std::chrono::duration<double, std::milli>(b - a).count();
}

}  // namespace

struct skc_server {
  skc_context* ctx = nullptr;
  uint64_t budget = 0;
  uint64_t in_use = 0;
  int slots = 0;
  std::vector<std::thread> workers;
  // Per slot: a high-priority stream for light requests and a low-priority
  // one for heavy requests, so a light request's kernels are dispatched
  // ahead of a heavy one's pending work.
  std::vector<cudaStream_t> streams, streams_lo;
  std::deque<std::shared_ptr<Request>> queue;
  std::map<uint64_t, std::shared_ptr<Request>> tickets;
  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  bool stopping = false;
  uint64_t next_ticket = 1;
  uint64_t admitted = 0, peak_in_flight = 0, in_flight = 0;
  uint64_t batches = 0, batched_requests = 0, largest_batch = 0;
};

// Requests that may share one lattice launch: batched capped skycubes the
// lattice form takes (max_d <= kLvMaxDims and <= d - 2, no bitmaps; forced,
// or by the automatic rule with n for the candidate count, its upper
// bound). A request bound for the bitmap form keeps a slot of its own, as
// it would run alone inside a batch's pass anyway.
static bool batchable(const Request& q) {
  const skc_options& o = q.opt;
  const int md = (o.max_d <= 0 || o.max_d > q.d) ? q.d : o.max_d;
  if (o.subspace || o.mode != SKC_MODE_BATCHED || o.want_bitmaps ||
      o.form == SKC_FORM_BITMAPS || md > kLvMaxDims || md > q.d - 2)
    return false;
  return o.form == SKC_FORM_LEVELS || levels_by_default(q.d, md, q.n);
}
constexpr size_t kMaxServerBatch = 8;

// Estimated device memory of one request: the resident points, the full-space
// pipeline, and the bitmap or per-cuboid stage with every point a candidate
// (an upper bound of the candidates), plus room for the id lists.
static uint64_t footprint_estimate(uint64_t n, int d, const skc_options& o, bool upload) {
  const uint64_t np = round_up(n, 128);
  const uint64_t W = d >= 5 ? (1ull << d) / 32 : 1;
  uint64_t b = (uint64_t)d * np * 4;          // resident points
  if (upload) b += n * (uint64_t)d * 4;        // staging copy
  b += n * (16 * 3 + 4 * 8) + 2 * (uint64_t)d * np * 4;  // full space
  if (o.subspace) {
    b += n * (16 * 2 + 4 * 6) + 2 * (uint64_t)d * np * 4;
  } else if (o.algo == SKC_ALGO_SDSC && o.mode == SKC_MODE_PLAIN) {
    b += n * (16 * 2 + 4 * 6) + 2 * (uint64_t)d * np * 4;
    b += 2 * n * 4 * std::min<uint64_t>(1ull << d, 64);  // per-cuboid lists
  } else {
    const bool ext = o.want_extended || o.algo == SKC_ALGO_SDSC;
    b += 2 * (uint64_t)d * np * 4 + n * (16 * 3 + 4 * 3);
    b += n * W * 4 * (ext ? 3 : 2);  // bitmaps + compaction
    b += n * 4 * std::min<uint64_t>(1ull << d, 64);  // id lists
    const int md = (o.max_d <= 0 || o.max_d > d) ? d : o.max_d;
    if (md <= kLvMaxDims && md <= d - 2) {  // the level form may run instead
      uint64_t cub = 1;  // cuboids of the widest level, C(d, md)
      for (int k = 0; k < md; ++k) cub = cub * (uint64_t)(d - k) / (uint64_t)(k + 1);
      b += std::min<uint64_t>(kLvScratchBytes, cub * std::min<uint64_t>(n, kLvMaxSurvivors) * 10);
      b += (uint64_t)md * cub * kLvSlot * 4 + n * (16 * 2 + 4 * 6) + 2 * (uint64_t)d * np * 4;
    }
  }
  return b;
}

// Copies a result's lists (and bitmaps) to host memory and frees its device
// memory, so later accessors are host lookups.
static int result_to_host(skc_result* r) {
  SKC_TRY(download_csr(r, false));
  if (r->d_eoff) SKC_TRY(download_csr(r, true));
  if (r->d_bits) {
    const uint32_t* b;
    const uint32_t* p;
    uint64_t n;
    uint32_t w;
    SKC_TRY(skc_result_bitmaps(r, &b, &p, &n, &w));
  }
  cudaStream_t s = r->stream;
  release_result_memory(r);
  SKC_CUDA(cudaStreamSynchronize(s));
  return SKC_OK;
}

// Heavy requests: the per-point bitmaps of many candidates over many
// subspaces (about n * 2^d >= 2^29: 8k points at d = 16, 512k at d = 10).
static bool heavy_request(uint64_t n, int d, const skc_options& o) {
  if (o.subspace) return false;
  return (n << d) >= (1ull << 29);
}

static void serve_one(skc_server* S, cudaStream_t stream, Request& q) {
  clear_error();
  Exec E;
  E.ctx = S->ctx;
  E.stream = stream;
  skc_dataset* ds = q.ds;
  int st = SKC_OK;
  if (!ds) st = upload_on(S->ctx, stream, q.rows, q.n, q.d, true, &ds);
  if (st == SKC_OK) st = skycube_exec(E, ds, &q.opt, &q.result);
  if (st == SKC_OK) st = result_to_host(q.result);
  if (!q.ds && ds) skc_dataset_free(ds);
  q.device_ms = E.ms;
  q.status = st;
  if (st != SKC_OK) {
    q.err = g_err;
    if (q.result) {
      skc_result_free(q.result);
      q.result = nullptr;
    }
  }
}

// Several batchable requests in one pass (skycube_exec_batch): their
// uploads, one lattice launch for all, their copies out.
static void serve_batch(skc_server* S, cudaStream_t stream,
                        std::vector<std::shared_ptr<Request>>& qs) {
  clear_error();
  Exec E;
  E.ctx = S->ctx;
  E.stream = stream;
  const size_t nb = qs.size();
  std::vector<skc_dataset*> dss(nb, nullptr);
  std::vector<skc_options> opts(nb);
  std::vector<bool> own(nb, false);
  int st = SKC_OK;
  for (size_t i = 0; i < nb && st == SKC_OK; ++i) {
    Request& q = *qs[i];
    opts[i] = q.opt;
    if (q.ds) {
      dss[i] = q.ds;
    } else {
      st = upload_on(S->ctx, stream, q.rows, q.n, q.d, true, &dss[i]);
      own[i] = st == SKC_OK;
    }
  }
  std::vector<skc_result*> R;
  if (st == SKC_OK) st = skycube_exec_batch(E, dss, opts, &R);
  for (size_t i = 0; i < nb; ++i) {
    Request& q = *qs[i];
    q.device_ms = E.ms;
    q.status = st;
    if (st == SKC_OK) {
      q.result = R[i];
      q.status = result_to_host(q.result);
    }
    if (q.status != SKC_OK) {
      q.err = g_err;
      if (q.result) {
        skc_result_free(q.result);
        q.result = nullptr;
      }
    }
    if (own[i] && dss[i]) skc_dataset_free(dss[i]);
  }
}

static void worker_loop(skc_server* S, int slot) {
  cudaSetDevice(S->ctx->device);
  for (;;) {
    std::vector<std::shared_ptr<Request>> batch;
    bool heavy = false;
    {
      std::unique_lock<std::mutex> lk(S->mu);
      S->cv_work.wait(lk, [&] {
        return S->stopping || (!S->queue.empty() &&
                               S->queue.front()->footprint <= S->budget - S->in_use);
      });
      if (S->stopping) return;
      // The head of the queue, and when it is a batchable request the
      // batchable requests right behind it that fit the budget.
      const auto now = std::chrono::steady_clock::now();
      do {
        auto q = S->queue.front();
        S->queue.pop_front();
        S->in_use += q->footprint;
        ++S->admitted;
        ++S->in_flight;
        q->t_start = now;
        heavy = heavy || q->heavy;
        batch.push_back(q);
      } while (batchable(*batch[0]) && batch.size() < kMaxServerBatch && !S->queue.empty() &&
               batchable(*S->queue.front()) &&
               S->queue.front()->footprint <= S->budget - S->in_use);
      S->peak_in_flight = std::max(S->peak_in_flight, S->in_flight);
      if (batch.size() > 1) {
        ++S->batches;
        S->batched_requests += batch.size();
        S->largest_batch = std::max<uint64_t>(S->largest_batch, batch.size());
      }
    }
    cudaStream_t stream = heavy ? S->streams_lo[slot] : S->streams[slot];
    if (batch.size() == 1) serve_one(S, stream, *batch[0]);
    else serve_batch(S, stream, batch);
    {
      std::lock_guard<std::mutex> lk(S->mu);
      const auto now = std::chrono::steady_clock::now();
      for (auto& q : batch) {
        S->in_use -= q->footprint;
        --S->in_flight;
        q->t_end = now;
        q->done = true;
      }
    }
    S->cv_done.notify_all();
    S->cv_work.notify_all();
  }
}

extern "C" {

int skc_server_create(skc_context* ctx, int slots, uint64_t budget, skc_server** out) {
  clear_error();
  if (!ctx || !out) return set_error(SKC_ERR_INVALID, "NULL argument");
  *out = nullptr;
  if (slots < 1 || slots > 64) return set_error(SKC_ERR_INVALID, "slots=%d outside [1,64]", slots);
  SKC_CUDA(cudaSetDevice(ctx->device));
  if (budget == 0) {
    size_t free_b = 0, total_b = 0;
    SKC_CUDA(cudaMemGetInfo(&free_b, &total_b));
    budget = (uint64_t)(free_b * 0.8);
  }
  auto* S = new skc_server;
  S->ctx = ctx;
  S->budget = budget;
  S->slots = slots;
  int prio_lo = 0, prio_hi = 0;
  SKC_CUDA(cudaDeviceGetStreamPriorityRange(&prio_lo, &prio_hi));
  for (int i = 0; i < slots; ++i) {
    cudaStream_t hi = nullptr, lo = nullptr;
    if (cudaStreamCreateWithPriority(&hi, cudaStreamNonBlocking, prio_hi) != cudaSuccess ||
        cudaStreamCreateWithPriority(&lo, cudaStreamNonBlocking, prio_lo) != cudaSuccess) {
      if (hi) cudaStreamDestroy(hi);
      for (auto x : S->streams) cudaStreamDestroy(x);
      for (auto x : S->streams_lo) cudaStreamDestroy(x);
      delete S;
      return set_error(SKC_ERR_CUDA, "stream creation failed");
    }
    S->streams.push_back(hi);
    S->streams_lo.push_back(lo);
  }
  for (int i = 0; i < slots; ++i) S->workers.emplace_back(worker_loop, S, i);
  *out = S;
  return SKC_OK;
}

static int submit_common(skc_server* S, std::shared_ptr<Request> q, uint64_t* ticket) {
  if (q->footprint > S->budget)
    return set_error(SKC_ERR_REJECTED,
                     "request needs about %.1f MiB of device memory, above the serving budget of %.1f MiB",
                     q->footprint / 1048576.0, S->budget / 1048576.0);
  {
    std::lock_guard<std::mutex> lk(S->mu);
    if (S->stopping) return set_error(SKC_ERR_INVALID, "server is shutting down");
    q->ticket = S->next_ticket++;
    q->t_submit = std::chrono::steady_clock::now();
    S->tickets[q->ticket] = q;
    S->queue.push_back(q);
  }
  S->cv_work.notify_all();
  *ticket = q->ticket;
  return SKC_OK;
}

int skc_server_submit(skc_server* S, const float* rows, uint64_t n, int d, const skc_options* opt,
                      uint64_t* ticket) {
  clear_error();
  if (!S || !rows || !ticket) return set_error(SKC_ERR_INVALID, "NULL argument");
  if (d < SKC_MIN_DIMS || d > SKC_MAX_DIMS)
    return set_error(SKC_ERR_INVALID, "d=%d outside [%d,%d]", d, SKC_MIN_DIMS, SKC_MAX_DIMS);
  if (n == 0) return set_error(SKC_ERR_INVALID, "empty dataset (n=0)");
  auto q = std::make_shared<Request>();
  q->rows = rows;
  q->n = n;
  q->d = d;
  skc_options_init(&q->opt);
  if (opt) q->opt = *opt;
  if (q->opt.subspace >= (1u << d))
    return set_error(SKC_ERR_INVALID, "subspace 0x%x has attributes beyond d=%d", q->opt.subspace, d);
  q->footprint = footprint_estimate(n, d, q->opt, true);
  q->heavy = heavy_request(n, d, q->opt);
  return submit_common(S, q, ticket);
}

int skc_server_submit_dataset(skc_server* S, skc_dataset* ds, const skc_options* opt,
                              uint64_t* ticket) {
  clear_error();
  if (!S || !ds || !ticket) return set_error(SKC_ERR_INVALID, "NULL argument");
  if (ds->ctx != S->ctx) return set_error(SKC_ERR_INVALID, "dataset belongs to another context");
  auto q = std::make_shared<Request>();
  q->ds = ds;
  q->n = ds->n;
  q->d = ds->d;
  skc_options_init(&q->opt);
  if (opt) q->opt = *opt;
  q->footprint = footprint_estimate(ds->n, ds->d, q->opt, false);
  q->heavy = heavy_request(ds->n, ds->d, q->opt);
  return submit_common(S, q, ticket);
}

int skc_server_wait(skc_server* S, uint64_t ticket, skc_result** out, skc_server_timing* t) {
  clear_error();
  if (!S || !out) return set_error(SKC_ERR_INVALID, "NULL argument");
  *out = nullptr;
  std::shared_ptr<Request> q;
  {
    std::unique_lock<std::mutex> lk(S->mu);
    auto it = S->tickets.find(ticket);
    if (it == S->tickets.end()) return set_error(SKC_ERR_INVALID, "unknown ticket %llu", (unsigned long long)ticket);
    q = it->second;
    // One waiter per ticket: a second one is refused at once instead of
    // sharing (and later double-freeing) the first one's result.
    if (q->claimed)
      return set_error(SKC_ERR_INVALID, "ticket %llu is already being waited on",
                       (unsigned long long)ticket);
    q->claimed = true;
    S->cv_done.wait(lk, [&] { return q->done; });
    S->tickets.erase(ticket);  // by key: other waits may have changed the map
  }
  if (t) {
    t->queued_ms = ms_between(q->t_submit, q->t_start);
    t->run_ms = ms_between(q->t_start, q->t_end);
    t->total_ms = ms_between(q->t_submit, q->t_end);
    t->device_ms = q->device_ms;
  }
  if (q->status != SKC_OK) {
    g_err = q->err;
    return q->status;
  }
  *out = q->result;
  return SKC_OK;
}

int skc_server_stats(skc_server* S, uint64_t* admitted, uint64_t* peak_in_flight,
                     uint64_t* budget) {
  clear_error();
  if (!S) return set_error(SKC_ERR_INVALID, "NULL server");
  std::lock_guard<std::mutex> lk(S->mu);
  if (admitted) *admitted = S->admitted;
  if (peak_in_flight) *peak_in_flight = S->peak_in_flight;
  if (budget) *budget = S->budget;
  return SKC_OK;
}

int skc_server_batch_stats(skc_server* S, uint64_t* batches, uint64_t* batched_requests,
                           uint64_t* largest) {
  clear_error();
  if (!S) return set_error(SKC_ERR_INVALID, "NULL server");
  std::lock_guard<std::mutex> lk(S->mu);
  if (batches) *batches = S->batches;
  if (batched_requests) *batched_requests = S->batched_requests;
  if (largest) *largest = S->largest_batch;
  return SKC_OK;
}

int skc_server_destroy(skc_server* S) {
  clear_error();
  if (!S) return SKC_OK;
  {
    // Let queued and running requests finish first.
    std::unique_lock<std::mutex> lk(S->mu);
    S->cv_done.wait(lk, [&] { return S->queue.empty() && S->in_flight == 0; });
    S->stopping = true;
  }
  S->cv_work.notify_all();
  for (auto& w : S->workers) w.join();
  for (auto& kv : S->tickets)
    if (kv.second->result) skc_result_free(kv.second->result);
  for (auto st : S->streams) cudaStreamDestroy(st);
  for (auto st : S->streams_lo) cudaStreamDestroy(st);
  delete S;
  return SKC_OK;
}

}  // extern "C"
