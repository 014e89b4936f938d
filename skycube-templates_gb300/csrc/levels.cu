// Capped skycubes by lattice level: the skyline and extended skyline of
// every cuboid of one level, all cuboids of the level in one launch pair.
// This is the per-cuboid computation of the suite's SDSC (each cuboid from
// its smallest computed parent's skyline + extended skyline, or from the
// full space's when the parents lie above the cap: findMinParent and
// gpu_processing_thread, src/sdsc/SDSC.cu:76-137,366-376), batched over a
// level instead of one SkyAlign call per cuboid, for cuboids of at most
// kLvMaxDims attributes.
//
// Per cuboid S and candidate list L:
//  1. k_lv_pruners: 32 pruners = the lowest cell sums over S of a
//     1,024-entry strided sample of L. k_lv_filter: every entry of L that a
//     pruner strictly dominates on S is dropped (exact float test on equal
//     cells). If a dropped q dominated a kept p, the pruner that drops q
//     would strictly dominate p, so the kept entries (survivors) decide each
//     other's status alone.
//  2. k_lv_sfs: the survivors, counting-sorted by cell sum over S (a
//     dominator's sum is never larger), go through a sort-filter skyline in
//     batches of 1,024: each entry is tested against the window of skyline
//     points found so far (strict domination drops it), the batch's
//     remaining entries against each other, and the batch's new skyline
//     points join the window. An entry can only be dominated by an entry of
//     equal cell sum that comes later if all their cells on S are equal; a
//     last pass tests each skyline and extended entry against the survivors
//     of its cell-sum bucket with equal cells. Output: [skyline | extended
//     skyline] ids, each ascending, in the cuboid's slot.
// Cells are those of a grid over the candidates' own quantiles (the caller
// passes them by point id). A cuboid whose survivors, skyline or extended
// skyline exceed the capacities is flagged; the host then computes it with
// the single-cuboid pipeline.
#include "kernels.cuh"

namespace skc {

namespace {

constexpr uint32_t kWarpAll = 0xffffffffu;

struct CubAttrs {
  int na;
  int att[kLvMaxDims];
  uint32_t gm;  // guard bits of bytes 0 .. na-1
};

__device__ __forceinline__ CubAttrs cub_attrs(uint32_t S) {
  CubAttrs A;
  A.na = min(__popc(S), kLvMaxDims);
#pragma unroll
  for (int a = 0; a < kLvMaxDims; ++a)  // index of the (a+1)-th set bit of S
    A.att[a] = a < A.na ? (int)__fns(S, 0, a + 1) : 0;
  A.gm = 0;
#pragma unroll
  for (int a = 0; a < kLvMaxDims; ++a)
    if (a < A.na) A.gm |= 0x80u << (8 * a);
  return A;
}

// Byte a = the cell of attribute att[a] (cells are < 128).
__device__ __forceinline__ uint32_t lv_pack(const uint4& c, const CubAttrs& A) {
  uint32_t r = 0;
#pragma unroll
  for (int a = 0; a < kLvMaxDims; ++a)
    if (a < A.na) {
      const int k = A.att[a];
      r |= ((word_of(c, k >> 2) >> (8 * (k & 3))) & 0x7fu) << (8 * a);
    }
  return r;
}

__device__ __forceinline__ uint32_t lv_key(uint32_t pc) {
  return (pc & 0xffu) + ((pc >> 8) & 0xffu) + ((pc >> 16) & 0xffu) + (pc >> 24);
}

__device__ __forceinline__ void lv_load(const float* __restrict__ x, uint64_t n_pad, uint32_t id,
                                        const CubAttrs& A, float* v) {
#pragma unroll
  for (int a = 0; a < kLvMaxDims; ++a)
    v[a] = a < A.na ? x[(uint64_t)A.att[a] * n_pad + id] : 0.f;
}

// 0: q does not dominate p on S; 1: dominates; 2: strictly dominates.
__device__ __forceinline__ int lv_dom(uint32_t qc, const float* qv, uint32_t pc, const float* pv,
                                      const CubAttrs& A) {
  if ((ge_bytes(pc | kGuard, qc) & A.gm) != A.gm) return 0;  // a cell of q above p's
  const uint32_t eq = ge_bytes(qc | kGuard, pc) & A.gm;       // equal cells
  if (!eq) return 2;
  bool any_lt = eq != A.gm, all_lt = true;
#pragma unroll
  for (int a = 0; a < kLvMaxDims; ++a) {
    if (eq & (0x80u << (8 * a))) {
      if (qv[a] > pv[a]) return 0;
      if (qv[a] < pv[a]) any_lt = true;
      else all_lt = false;
    }
  }
  if (!any_lt) return 0;
  return all_lt ? 2 : 1;
}

}  // namespace

// The first kLvFirstPruners pruners are tested on every entry; the entries
// they leave are staged and tested densely against the others, so a warp
// runs the long pruner loop only on entries that need it.
constexpr uint32_t kLvFirstPruners = 4;

// True when one of the pruners [j0, j1) strictly dominates p on S.
__device__ __forceinline__ bool lv_pruned(uint32_t pc, uint32_t id, uint32_t j0, uint32_t j1,
                                          const uint32_t* pr_c, const float (*pr_v)[kLvPruners],
                                          const float* __restrict__ x, uint64_t n_pad,
                                          const CubAttrs& A) {
  float pv[kLvMaxDims];
  bool have_v = false;
  for (uint32_t j = j0; j < j1; ++j) {
    const uint32_t qc = pr_c[j];
    if ((ge_bytes(pc | kGuard, qc) & A.gm) != A.gm) continue;
    const uint32_t eq = ge_bytes(qc | kGuard, pc) & A.gm;
    if (!eq) return true;
    if (!have_v) {
      lv_load(x, n_pad, id, A, pv);
      have_v = true;
    }
    bool strict = true;
#pragma unroll
    for (int a = 0; a < kLvMaxDims; ++a)
      if ((eq & (0x80u << (8 * a))) && !(pr_v[a][j] < pv[a])) strict = false;
    if (strict) return true;
  }
  return false;
}

// Data written inside the persistent kernel by other CTAs (pruners, lists,
// survivors, parent slots, counts) is read through L2 (ld.global.cg), never
// through the read-only or L1 paths, which are not coherent across SMs.
__device__ __forceinline__ uint32_t ld_l2(const uint32_t* p) { return __ldcg(p); }
__device__ __forceinline__ float ld_l2(const float* p) { return __ldcg(p); }
__device__ __forceinline__ uint16_t ld_l2(const uint16_t* p) {
  return __ldcg(reinterpret_cast<const unsigned short*>(p));
}

// Pruners of cuboid S over its list L[0, n): the lowest cell sums over S of a
// strided kLvSample-entry sample, into pr_c/pr_v/pr_n at scratch index g.
// One CTA of kLvThreads threads (kLvSample / kLvThreads entries each).
__device__ void lv_pruners_cta(const CubAttrs& A, const uint32_t* L, uint32_t n,
                               const uint4* __restrict__ cells, const float* __restrict__ x,
                               uint64_t n_pad, uint32_t g, uint32_t* pr_c_g, float* pr_v_g,
                               uint32_t* pr_n_g, uint32_t* hist) {
  __shared__ uint32_t s_thr, s_np;
  const int tid = threadIdx.x;
  if (n == 0) {  // uniform over the CTA
    if (tid == 0) pr_n_g[g] = 0;
    return;
  }
  const uint32_t ns = min(n, kLvSample);
  for (uint32_t i = tid; i < kLvKeyBins; i += blockDim.x) hist[i] = 0;
  __syncthreads();
  constexpr int kPer = (kLvSample + kLvThreads - 1) / kLvThreads;
  uint32_t sid[kPer], skey[kPer];
#pragma unroll
  for (int r = 0; r < kPer; ++r) {
    const uint32_t i = tid + kLvThreads * r;
    sid[r] = 0;
    skey[r] = 0xffffffffu;
    if (i < ns) {
      sid[r] = ld_l2(L + (uint64_t)i * n / ns);
      skey[r] = lv_key(lv_pack(cells[sid[r]], A));
      atomicAdd(&hist[skey[r]], 1u);
    }
  }
  __syncthreads();
  if (tid == 0) {
    uint32_t acc = 0, t = kLvKeyBins - 1;
    for (uint32_t k = 0; k < kLvKeyBins; ++k) {
      if (acc + hist[k] >= kLvPruners) {
        t = k;
        break;
      }
      acc += hist[k];
    }
    s_thr = t;
    s_np = 0;
  }
  __syncthreads();
  const uint32_t thr = s_thr;
  for (int pass = 0; pass < 2; ++pass) {  // sums below the threshold, then at it
#pragma unroll
    for (int r = 0; r < kPer; ++r) {
      const bool take = pass == 0 ? skey[r] < thr : skey[r] == thr;
      if (take) {
        const uint32_t k = atomicAdd(&s_np, 1u);
        if (k < kLvPruners) {
          pr_c_g[(uint64_t)g * kLvPruners + k] = lv_pack(cells[sid[r]], A);
          float v[kLvMaxDims];
          lv_load(x, n_pad, sid[r], A, v);
#pragma unroll
          for (int a = 0; a < kLvMaxDims; ++a)
            pr_v_g[((uint64_t)g * kLvMaxDims + a) * kLvPruners + k] = v[a];
        }
      }
    }
    __syncthreads();
  }
  if (tid == 0) pr_n_g[g] = min(s_np, kLvPruners);
}

// Shared memory of one filter chunk, in bytes.
static constexpr size_t kLvFilterSmem = (size_t)kLvChunk * (4 + 4 + 4 + 2);

// The pruner filter of list entries [beg, end) of cuboid S (scratch index g):
// every entry meets the first kLvFirstPruners pruners, the ones left are
// staged and meet the others densely; survivors are appended to g's scratch
// (one atomic per CTA). `sm` holds kLvFilterSmem bytes.
__device__ void lv_filter_chunk(const CubAttrs& A, const uint32_t* L, uint32_t beg, uint32_t end,
                                const uint4* __restrict__ cells, const float* __restrict__ x,
                                uint64_t n_pad, uint32_t g, const uint32_t* pr_c_g,
                                const float* pr_v_g, const uint32_t* pr_n_g, uint32_t cap,
                                uint32_t* cnt, uint32_t* surv_id, uint16_t* surv_key,
                                unsigned char* sm) {
  __shared__ uint32_t s_n1, s_n, s_base;
  __shared__ uint32_t pr_c[kLvPruners];
  __shared__ float pr_v[kLvMaxDims][kLvPruners];
  uint32_t* s1_id = reinterpret_cast<uint32_t*>(sm);          // [kLvChunk] staged entries
  uint32_t* s1_pc = s1_id + kLvChunk;                          // [kLvChunk]
  uint32_t* st_id = s1_pc + kLvChunk;                          // [kLvChunk] survivors
  uint16_t* st_key = reinterpret_cast<uint16_t*>(st_id + kLvChunk);  // [kLvChunk]
  const int tid = threadIdx.x, lane = tid & 31;
  if (tid < (int)kLvPruners) {
    pr_c[tid] = ld_l2(pr_c_g + (uint64_t)g * kLvPruners + tid);
#pragma unroll
    for (int a = 0; a < kLvMaxDims; ++a)
      pr_v[a][tid] = ld_l2(pr_v_g + ((uint64_t)g * kLvMaxDims + a) * kLvPruners + tid);
  }
  if (tid == 0) {
    s_n1 = 0;
    s_n = 0;
  }
  __syncthreads();
  const uint32_t np = ld_l2(pr_n_g + g);
  const uint32_t np1 = min(np, kLvFirstPruners);

  // Phase 1: every entry against the first pruners; the rest are staged.
  const uint32_t lt_mask = (1u << lane) - 1u;
  for (uint32_t base = beg; base < end; base += blockDim.x) {
    const uint32_t i = base + tid;
    const bool valid = i < end;
    uint32_t id = 0, pc = 0;
    bool keep = false;
    if (valid) {
      id = ld_l2(L + i);
      pc = lv_pack(cells[id], A);
      keep = !lv_pruned(pc, id, 0, np1, pr_c, pr_v, x, n_pad, A);
    }
    const uint32_t live = __ballot_sync(kWarpAll, keep);
    uint32_t pos0 = 0;
    if (lane == 0 && live) pos0 = atomicAdd(&s_n1, (uint32_t)__popc(live));
    pos0 = __shfl_sync(kWarpAll, pos0, 0);
    if (keep) {
      const uint32_t pos = pos0 + __popc(live & lt_mask);  // < kLvChunk
      s1_id[pos] = id;
      s1_pc[pos] = pc;
    }
  }
  __syncthreads();
  // Phase 2: the staged entries against the other pruners.
  const uint32_t n1 = s_n1;
  for (uint32_t k = tid; k < n1; k += blockDim.x) {
    const uint32_t id = s1_id[k], pc = s1_pc[k];
    if (!lv_pruned(pc, id, np1, np, pr_c, pr_v, x, n_pad, A)) {
      const uint32_t pos = atomicAdd(&s_n, 1u);  // < kLvChunk
      st_id[pos] = id;
      st_key[pos] = (uint16_t)lv_key(pc);
    }
  }
  __syncthreads();
  const uint32_t ns_kept = s_n;
  if (tid == 0) s_base = ns_kept ? atomicAdd(&cnt[g], ns_kept) : 0u;
  __syncthreads();
  const uint32_t b0 = s_base;
  for (uint32_t k = tid; k < ns_kept; k += blockDim.x) {
    const uint32_t pos = b0 + k;
    if (pos < cap) {
      surv_id[(uint64_t)g * cap + pos] = st_id[k];
      surv_key[(uint64_t)g * cap + pos] = st_key[k];
    }
  }
  __syncthreads();  // the staging arrays are reused by the next chunk
}

// Shared memory of the sort-filter skyline of one cuboid, in bytes.
static constexpr size_t kLvSfsSmem =
    (2 * (kLvKeyBins + 1)) * 4 +                                   // bucket offsets, cursors
    kLvWin * (4 + 4 * kLvMaxDims + 4 + 1) +                        // window
    kLvExt * (4 + 1) +                                             // extended entries
    kLvThreads * (4 + 4 * kLvMaxDims + 4 + 2 + 1) +                // batch
    kLvSortCap * 4 + 64;                                           // sort buffer, counters

// The skyline and extended skyline of cuboid c over the survivors in
// scratch index g, into c's slot (skyline ids, then extended ids, each
// ascending) and o_nsky/o_next/o_flag[c]; o_flag[c] = 1 when a capacity is
// exceeded (nothing computed: the host takes the cuboid). One CTA of
// kLvThreads threads; `lv_smem` holds kLvSfsSmem bytes. Returns the flag.
__device__ uint32_t lv_sfs_cta(const CubAttrs& A, uint32_t c, uint32_t g,
                               const uint4* __restrict__ cells, const float* __restrict__ x,
                               uint64_t n_pad, uint32_t cap, const uint32_t* cnt,
                               const uint32_t* surv_id, const uint16_t* surv_key, uint32_t* srt,
                               uint32_t* slot, uint32_t* o_nsky, uint32_t* o_next,
                               uint32_t* o_flag, unsigned char* lv_smem) {
  const int tid = threadIdx.x;
  const uint32_t n = ld_l2(cnt + g);
  if (n > cap) {  // survivors beyond the scratch: the host takes this cuboid
    if (tid == 0) {
      o_flag[c] = 1;
      o_nsky[c] = 0;
      o_next[c] = 0;
    }
    return 1;
  }
  const uint64_t off = (uint64_t)g * cap;

  uint32_t* kb = reinterpret_cast<uint32_t*>(lv_smem);   // [kLvKeyBins + 1]
  uint32_t* cur = kb + kLvKeyBins + 1;                    // [kLvKeyBins + 1]
  uint32_t* w_c = cur + kLvKeyBins + 1;                   // [kLvWin]
  float* w_v = reinterpret_cast<float*>(w_c + kLvWin);    // [kLvMaxDims][kLvWin]
  uint32_t* w_pos = reinterpret_cast<uint32_t*>(w_v + kLvMaxDims * kLvWin);
  uint32_t* e_pos = w_pos + kLvWin;                       // [kLvExt]
  uint32_t* b_c = e_pos + kLvExt;                         // [kLvThreads]
  float* b_v = reinterpret_cast<float*>(b_c + kLvThreads);  // [kLvMaxDims][kLvThreads]
  uint32_t* b_pos = reinterpret_cast<uint32_t*>(b_v + kLvMaxDims * kLvThreads);
  uint32_t* sb = b_pos + kLvThreads;                      // [kLvSortCap]
  uint16_t* b_key = reinterpret_cast<uint16_t*>(sb + kLvSortCap);  // [kLvThreads]
  uint8_t* b_st = reinterpret_cast<uint8_t*>(b_key + kLvThreads);  // [kLvThreads]
  uint8_t* w_st = b_st + kLvThreads;                      // [kLvWin]
  uint8_t* e_st = w_st + kLvWin;                          // [kLvExt]
  uint32_t* ctr = reinterpret_cast<uint32_t*>(
      (reinterpret_cast<uintptr_t>(e_st + kLvExt) + 15) & ~uintptr_t(15));
  // ctr: 0 window size, 1 extended size, 2 batch size, 3 overflow, 4 kept,
  // 5 skyline kept, 6 end of the current batch

  // 1. Counting sort of the survivors by cell sum.
  for (uint32_t k = tid; k <= kLvKeyBins; k += blockDim.x) cur[k] = 0;
  if (tid < 8) ctr[tid] = 0;
  __syncthreads();
  for (uint32_t i = tid; i < n; i += blockDim.x) atomicAdd(&cur[ld_l2(surv_key + off + i)], 1u);
  __syncthreads();
  if (tid == 0) {
    uint32_t acc = 0;
    for (uint32_t k = 0; k < kLvKeyBins; ++k) {
      kb[k] = acc;
      acc += cur[k];
    }
    kb[kLvKeyBins] = acc;
  }
  __syncthreads();
  for (uint32_t k = tid; k < kLvKeyBins; k += blockDim.x) cur[k] = kb[k];
  __syncthreads();
  for (uint32_t i = tid; i < n; i += blockDim.x) {
    const uint32_t p = atomicAdd(&cur[ld_l2(surv_key + off + i)], 1u);
    srt[off + p] = ld_l2(surv_id + off + i);
  }
  __syncthreads();

  // 2. Sort-filter skyline in batches of kLvThreads entries. The tests are
  // warp-cooperative: a warp takes one entry at a time and its lanes test
  // 32 window (or batch) entries per step, so no warp waits for its slowest
  // lane's scan.
  // A batch ends on a cell-sum bucket boundary when one lies in its range,
  // so entries of equal sum (which may dominate each other in either order)
  // meet in the same batch; only buckets larger than a batch are split.
  const int lane = tid & 31, wid = tid >> 5;
  constexpr uint32_t kWarps = kLvThreads / 32;
  for (uint32_t base = 0, bend = 0; base < n; base = bend) {
    if (tid == 0) {
      const uint32_t target = base + kLvThreads;
      uint32_t e = n;
      if (target < n) {
        uint32_t lo = 0, hi = kLvKeyBins;  // largest k with kb[k] <= target
        while (lo < hi) {
          const uint32_t mid = (lo + hi + 1) >> 1;
          if (kb[mid] <= target) lo = mid; else hi = mid - 1;
        }
        e = kb[lo] > base ? kb[lo] : target;
      }
      ctr[6] = e;
    }
    __syncthreads();
    bend = ctr[6];
    const uint32_t i = base + tid;
    const bool valid = i < bend;
    uint32_t pc = 0, key = 0;
    float pv[kLvMaxDims];
#pragma unroll
    for (int a = 0; a < kLvMaxDims; ++a) pv[a] = 0.f;
    if (valid) {
      const uint32_t id = srt[off + i];
      pc = lv_pack(cells[id], A);
      key = lv_key(pc);
      lv_load(x, n_pad, id, A, pv);
    }
    // Window test of the warp's 32 entries, one entry per step.
    const uint32_t wn = min(ctr[0], kLvWin);
    int my_st = valid ? 0 : 2;
    for (int e = 0; e < 32; ++e) {
      if (!__shfl_sync(kWarpAll, (int)valid, e)) continue;
      const uint32_t qpc = __shfl_sync(kWarpAll, pc, e);
      float qpv[kLvMaxDims];
#pragma unroll
      for (int a = 0; a < kLvMaxDims; ++a) qpv[a] = __shfl_sync(kWarpAll, pv[a], e);
      int st = 0;
      for (uint32_t j0 = 0; j0 < wn; j0 += 32) {
        const uint32_t j = j0 + lane;
        int r = 0;
        if (j < wn) {
          float wv[kLvMaxDims];
#pragma unroll
          for (int a = 0; a < kLvMaxDims; ++a) wv[a] = w_v[a * kLvWin + j];
          r = lv_dom(w_c[j], wv, qpc, qpv, A);
        }
        // one warp OR of the statuses (r: 0 none, 1 dominates, 2 strictly):
        // bit 1 some lane strictly dominates, bit 0 some lane dominates
        const uint32_t any = __reduce_or_sync(kWarpAll, (uint32_t)r);
        if (any & 2u) {
          st = 2;
          break;
        }
        if (any & 1u) st = 1;
      }
      if (lane == e) my_st = st;
    }
    __syncthreads();  // every thread has read ctr[0]
    if (tid == 0) ctr[2] = 0;
    __syncthreads();
    if (my_st < 2) {
      const uint32_t k = atomicAdd(&ctr[2], 1u);
      b_c[k] = pc;
#pragma unroll
      for (int a = 0; a < kLvMaxDims; ++a) b_v[a * kLvThreads + k] = pv[a];
      b_pos[k] = i;
      b_key[k] = (uint16_t)key;
      b_st[k] = (uint8_t)my_st;
    }
    __syncthreads();
    // The batch's remaining entries against each other (only entries of a
    // cell sum <= p's can dominate p); warp w takes entries w, w + 32, ...
    const uint32_t nb = ctr[2];
    for (uint32_t p = wid; p < nb; p += kWarps) {
      const uint32_t ppc = b_c[p];
      const uint32_t pkey = b_key[p];
      float ppv[kLvMaxDims];
#pragma unroll
      for (int a = 0; a < kLvMaxDims; ++a) ppv[a] = b_v[a * kLvThreads + p];
      int st = b_st[p];
      for (uint32_t q0 = 0; q0 < nb; q0 += 32) {
        const uint32_t q = q0 + lane;
        int r = 0;
        if (q < nb && q != p && b_key[q] <= pkey) {
          float qv[kLvMaxDims];
#pragma unroll
          for (int a = 0; a < kLvMaxDims; ++a) qv[a] = b_v[a * kLvThreads + q];
          r = lv_dom(b_c[q], qv, ppc, ppv, A);
        }
        // one warp OR of the statuses: bit 1 some lane strictly dominates,
        // bit 0 some lane dominates
        const uint32_t any = __reduce_or_sync(kWarpAll, (uint32_t)r);
        if (any & 2u) {
          st = 2;
          break;
        }
        if (any & 1u) st = 1;
      }
      __syncwarp();
      if (lane == 0) b_st[p] = (uint8_t)st;  // only this warp reads b_st[p]
    }
    __syncthreads();
    if ((uint32_t)tid < nb) {
      const int st2 = b_st[tid];
      if (st2 == 0) {
        const uint32_t k = atomicAdd(&ctr[0], 1u);
        if (k < kLvWin) {
          w_c[k] = b_c[tid];
#pragma unroll
          for (int a = 0; a < kLvMaxDims; ++a) w_v[a * kLvWin + k] = b_v[a * kLvThreads + tid];
          w_pos[k] = b_pos[tid];
          w_st[k] = 0;
        } else {
          ctr[3] = 1;
        }
      } else if (st2 == 1) {
        const uint32_t k = atomicAdd(&ctr[1], 1u);
        if (k < kLvExt) {
          e_pos[k] = b_pos[tid];
          e_st[k] = 1;
        } else {
          ctr[3] = 1;
        }
      }
    }
    __syncthreads();
    if (ctr[3]) break;  // uniform: read after the barrier
  }
  if (ctr[3]) {
    if (tid == 0) {
      o_flag[c] = 1;
      o_nsky[c] = 0;
      o_next[c] = 0;
    }
    __syncthreads();  // ctr is reused by the CTA's next item
    return 1;
  }

  // 3. Later entries of the same cell sum with equal cells on S; a warp per
  // skyline or extended entry, its lanes over the bucket.
  const uint32_t wn = ctr[0], en = ctr[1], tot = wn + en;
  for (uint32_t e = wid; e < tot; e += kWarps) {
    const uint32_t pos = e < wn ? w_pos[e] : e_pos[e - wn];
    int st = e < wn ? 0 : 1;
    const uint32_t id = srt[off + pos];
    const uint32_t pc = lv_pack(cells[id], A);
    const uint32_t key = lv_key(pc);
    float pv[kLvMaxDims];
    lv_load(x, n_pad, id, A, pv);
    const uint32_t j1 = kb[key + 1];
    for (uint32_t j0 = kb[key]; j0 < j1; j0 += 32) {
      const uint32_t j = j0 + lane;
      int r = 0;
      if (j < j1 && j != pos) {
        const uint32_t qid = srt[off + j];
        if (lv_pack(cells[qid], A) == pc) {
          float qv[kLvMaxDims];
          lv_load(x, n_pad, qid, A, qv);
          r = lv_dom(pc, qv, pc, pv, A);
        }
      }
      const uint32_t any = __reduce_or_sync(kWarpAll, (uint32_t)r);
      if (any & 2u) {
        st = 2;
        break;
      }
      if (any & 1u) st = 1;
    }
    if (lane == 0) {
      if (e < wn) w_st[e] = (uint8_t)st;
      else e_st[e - wn] = (uint8_t)st;
    }
  }
  __syncthreads();

  // 4. Output: (status << 31 | id) sorted, so skyline ids come first, each
  // part ascending.
  for (uint32_t e = tid; e < tot; e += blockDim.x) {
    const uint32_t pos = e < wn ? w_pos[e] : e_pos[e - wn];
    const uint32_t st = e < wn ? w_st[e] : e_st[e - wn];
    if (st < 2) {
      const uint32_t k = atomicAdd(&ctr[4], 1u);
      sb[k] = (st << 31) | srt[off + pos];
      if (st == 0) atomicAdd(&ctr[5], 1u);
    }
  }
  __syncthreads();
  const uint32_t kept = ctr[4];
  uint32_t p2 = 1;
  while (p2 < kept) p2 <<= 1;
  for (uint32_t k = kept + tid; k < p2; k += blockDim.x) sb[k] = 0xffffffffu;
  __syncthreads();
  for (uint32_t k = 2; k <= p2; k <<= 1) {
    for (uint32_t j = k >> 1; j > 0; j >>= 1) {
      for (uint32_t i = tid; i < p2; i += blockDim.x) {
        const uint32_t ixj = i ^ j;
        if (ixj > i) {
          const uint32_t a = sb[i], b = sb[ixj];
          const bool up = (i & k) == 0;
          if ((a > b) == up) {
            sb[i] = b;
            sb[ixj] = a;
          }
        }
      }
      __syncthreads();
    }
  }
  const uint64_t so = (uint64_t)c * kLvSlot;
  for (uint32_t k = tid; k < kept; k += blockDim.x) slot[so + k] = sb[k] & 0x7fffffffu;
  if (tid == 0) {
    o_nsky[c] = ctr[5];
    o_next[c] = kept - ctr[5];
    o_flag[c] = 0;
  }
  __syncthreads();  // shared memory is reused by the CTA's next item
  return 0;
}

// out[idx[i]] = in[i] for i < *m_ptr.
__global__ void k_scatter_u4(const uint4* __restrict__ in, const uint32_t* __restrict__ idx,
                             const uint32_t* __restrict__ m_ptr, uint4* __restrict__ out) {
  const uint32_t m = *m_ptr;
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < m; i += gridDim.x * blockDim.x)
    out[idx[i]] = in[i];
}

int launch_scatter_u4(cudaStream_t s, const uint4* in, const uint32_t* idx, const uint32_t* m_ptr,
                      uint64_t m_max, uint4* out) {
  uint64_t b = (m_max + 255) / 256;
  if (b < 1) b = 1;
  if (b > 152 * 8) b = 152 * 8;
  k_scatter_u4<<<(unsigned)b, 256, 0, s>>>(in, idx, m_ptr, out);
  SKC_LAUNCH_CHECK();
  return SKC_OK;
}

// ---------------------------------------------------------------------------
// The lattice work queue: one persistent launch computes every wanted cuboid
// of every job (dataset). Items sit in lattice-level order: for each level,
// top down, and each group of cuboids that fits the survivor scratch, a
// phase P (per cuboid: its smallest computed parent's skyline + extended
// skyline as the candidate list, then its pruners), a phase F (per cuboid
// and slice: the pruner filter of the slice's chunks) and a phase S (per
// cuboid: the sort-filter skyline). A CTA pops the next item from a device
// counter and, before running it, waits until every item of the previous
// phase is done. Items are popped in order, so the items waited for are
// running on resident CTAs (the launch is cooperative: every CTA is
// resident); the waits are bounded and set status[0] when they run out.
// After that no item runs: a skipped item still counts, so a later phase's
// counter can fill up, and its items must not run on inputs the skipped
// ones never wrote (a candidate-list pointer, a survivor count).
constexpr uint32_t kLtWaitLimit = 1u << 23;  // about 2 s of 256 ns sleeps

__device__ __forceinline__ uint32_t ld_acquire(const uint32_t* p) {
  uint32_t v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

// True when the phase before is done and no wait has run out. The status is
// read after the counter, both with acquire order: a skipped item set (or
// saw) the status before its count, so a full counter that includes it
// shows the status too.
__device__ __forceinline__ bool lt_wait_phase(const uint32_t* done, uint32_t want,
                                              uint32_t* status) {
  for (uint32_t it = 0; it < kLtWaitLimit; ++it) {
    if (ld_acquire(done) >= want) return ld_acquire(status) == 0;
    if (ld_acquire(status) != 0) return false;
    __nanosleep(256);
  }
  atomicExch(status, 1u);
  return false;
}

// Candidate list of cuboid c: the computed parent (one more attribute,
// within the job's cap, not the full space, not over a capacity) with the
// smallest skyline + extended skyline, as findMinParent picks it, else the
// job's full-space candidates. Any parent's list holds every point of c's
// skyline and extended skyline and its dominators among them, so the choice
// changes the work only.
__device__ void lt_choose_list(const LtArgs& a, uint32_t c, const uint32_t** list,
                               uint32_t* n) {
  const LtJob& J = a.jobs[a.c_job[c]];
  const uint32_t S = a.c_mask[c];
  const uint32_t full = (1u << J.d) - 1u;
  uint32_t best = 0xffffffffu, best_n = 0xffffffffu;
  for (int k = J.d - 1; k >= 0; --k) {  // parents in generate_lattice's order
    if (S & (1u << k)) continue;
    const uint32_t P = S | (1u << k);
    if (P == full || __popc(P) > J.max_d) continue;
    const uint32_t pi = J.cub_index[P];
    if (pi == 0xffffffffu || ld_l2(a.c_flag + pi) != 0) continue;
    const uint32_t pn = ld_l2(a.c_nsky + pi) + ld_l2(a.c_next + pi);
    if (pn < best_n) {
      best_n = pn;
      best = pi;
    }
  }
  if (best == 0xffffffffu) {
    *list = J.cand;
    *n = J.n_cand;
  } else {
    *list = a.slot + (uint64_t)best * kLvSlot;
    *n = best_n;
  }
}

__global__ void __launch_bounds__(kLvThreads, 1) k_lattice(LtArgs a) {
  extern __shared__ __align__(16) unsigned char lt_smem[];
  __shared__ uint32_t s_item, s_run;
  __shared__ const uint32_t* s_list;
  __shared__ uint32_t s_n;
  const int tid = threadIdx.x;
  for (;;) {
    if (tid == 0) {
      const uint32_t it = atomicAdd(a.next_item, 1u);
      uint32_t run = 0;
      if (it < a.n_items) {
        const uint32_t ph = a.it_phase[it];
        run = (ph == 0 || lt_wait_phase(a.ph_done + ph - 1, a.ph_size[ph - 1], a.status)) ? 1u : 0u;
        if (run) {
          // a job whose first level overflowed too often goes to the bitmap
          // form: the host recomputes it, its remaining items only count
          const uint32_t c = a.it_cub[it];
          const uint32_t j = a.c_job[c];
          if (ld_l2(a.job_over + j) > a.max_fallbacks) run = 2;
        }
      }
      s_item = it;
      s_run = run;
    }
    __syncthreads();
    const uint32_t it = s_item;
    if (it >= a.n_items) return;
    const uint32_t ph = a.it_phase[it];
    if (s_run == 1) {
      const uint32_t c = a.it_cub[it];
      const uint32_t g = a.c_scr[c];
      const LtJob& J = a.jobs[a.c_job[c]];
      const CubAttrs A = cub_attrs(a.c_mask[c]);
      const uint32_t kind = a.ph_kind[ph];
      if (kind == 0) {  // P: candidate list and pruners
        if (tid == 0) {
          const uint32_t* L;
          uint32_t n;
          lt_choose_list(a, c, &L, &n);
          a.c_list[c] = L;
          a.c_list_n[c] = n;
          a.cnt[g] = 0;
          s_list = L;
          s_n = n;
        }
        __syncthreads();
        lv_pruners_cta(A, s_list, s_n, J.cells, J.x, J.n_pad, g, a.pr_c, a.pr_v, a.pr_n,
                       reinterpret_cast<uint32_t*>(lt_smem));
      } else if (kind == 1) {  // F: chunks slice, slice + nslices, ... of the list
        const uint32_t slice = a.it_arg[it] & 0xffffu, nsl = a.it_arg[it] >> 16;
        const uint32_t* L = reinterpret_cast<const uint32_t*>(
            __ldcg(reinterpret_cast<const unsigned long long*>(a.c_list + c)));
        const uint32_t n = ld_l2(a.c_list_n + c);
        for (uint32_t k = slice; (uint64_t)k * kLvChunk < n; k += nsl)
          lv_filter_chunk(A, L, k * kLvChunk, min(n, (k + 1) * kLvChunk), J.cells, J.x, J.n_pad,
                          g, a.pr_c, a.pr_v, a.pr_n, a.cap, a.cnt, a.surv_id, a.surv_key, lt_smem);
      } else {  // S: the sort-filter skyline
        const uint32_t over = lv_sfs_cta(A, c, g, J.cells, J.x, J.n_pad, a.cap, a.cnt, a.surv_id,
                                         a.surv_key, a.srt, a.slot, a.c_nsky, a.c_next,
                                         a.c_flag, lt_smem);
        if (over && tid == 0 && __popc(a.c_mask[c]) == J.max_d)
          atomicAdd(a.job_over + a.c_job[c], 1u);
      }
    } else if (s_run == 2 && a.ph_kind[ph] == 2 && tid == 0) {
      const uint32_t c = a.it_cub[it];  // skipped: flagged for the host
      a.c_flag[c] = 2;
      a.c_nsky[c] = 0;
      a.c_next[c] = 0;
    }
    // Publish: every thread's writes reach L2 before the phase counter moves.
    __threadfence();
    __syncthreads();
    if (tid == 0) atomicAdd(a.ph_done + ph, 1u);
  }
}

static size_t lattice_smem() {
  return kLvSfsSmem > kLvFilterSmem ? kLvSfsSmem : kLvFilterSmem;
}

// Persistent CTAs of the lattice kernel on `num_sms` SMs (one per SM).
int lattice_grid(int num_sms, int* grid) {
  SKC_CUDA(cudaFuncSetAttribute(k_lattice, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)lattice_smem()));
  int per_sm = 0;
  SKC_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_lattice, kLvThreads,
                                                         lattice_smem()));
  if (per_sm < 1) return set_error(SKC_ERR_UNSUPPORTED, "the lattice kernel does not fit an SM");
  *grid = per_sm * num_sms;
  return SKC_OK;
}

int launch_lattice(cudaStream_t s, int num_sms, const LtArgs& a) {
  if (a.n_items == 0) return SKC_OK;
  int grid = 0;
  SKC_TRY(lattice_grid(num_sms, &grid));
  LtArgs args = a;
  void* params[] = {&args};
  SKC_CUDA(cudaLaunchCooperativeKernel((const void*)k_lattice, dim3(grid), dim3(kLvThreads),
                                       params, lattice_smem(), s));
  SKC_LAUNCH_CHECK();
  return SKC_OK;
}

}  // namespace skc
