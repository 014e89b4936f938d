// Median-partition skyline of a point list on one subspace S.
//
// Points are grouped by their median mask over the first B = min(|S|, 10)
// attributes of S (bit j set when the point is worse than the median on that
// attribute: the top bit of its grid cell). A point q can only dominate p
// when q's mask is a subset of p's: on an attribute where q is above the
// median and p is not, q is strictly worse. This is the partition test of
// the suite's SkyAlign and Hybrid skylines (distribute_pitch_two_level_median,
// src/utilities/kernels.cu:99-125; canskip_partition, src/utilities/
// SubTuple.h:69-73), applied here to whole partitions at once.
//
// Layout. A counting sort groups the list by the lattice-level rank of the
// mask (popcount, then value), so partitions of stronger points come first.
// One CTA owns up to 256 points of ONE partition (a work item); it visits
// only the partitions whose mask is a subset of its own, in level order, and
// streams their points through shared memory 256 at a time. Each thread
// tests its point against every staged point with the grid-cell SWAR test
// and, when cells tie, exact float32 comparisons (see skyline.cu). A
// strictly dominated point stops; the CTA stops when all its points have.
#include <algorithm>

#include "kernels.cuh"

namespace skc {

// Order inside the partitions of a sliced skyline list. The strength order
// (cell sum) lets a dominated point meet a dominator early; the Gray order
// keeps q tiles' minimum-cell boxes tight, so whole tiles are skipped. Which
// wins follows the spread of the points' cell sums: where they are
// concentrated (anticorrelated data, points near a hyperplane) the strength
// order carries little and the Gray order wins; where they spread as much
// as independent attributes would, or more, the strength order wins.
// Measured (skyline kernel, strength -> Gray + tile boxes): anticorrelated
// 1M x 10 7.03 -> 5.99 ms, 400k x 12 3.77 -> 3.48 ms, 200k x 8 0.50 -> 0.44
// ms (spread 0.51-0.62 of the independent value); uniform 1M x 10 1.74 ->
// 1.80 ms, 500k x 16 6.38 -> 6.57 ms (1.01); correlated 1M x 10 2.47 ->
// 3.61 ms, quantised 566k x 15 1.31 -> 1.93 ms (3.1-3.8). Only the
// partition part of the key matters for correctness. With the choice made
// on the device (both skyline instantiations launched, one returning at
// once): anticorrelated 1M x 10 6.90 -> 5.93 ms, 400k x 12 3.74 -> 3.47 ms,
// 500k x 16 8.48 -> 8.14 ms; the others within 1 %.
constexpr double kGraySpread = 0.8;  // limit, as a fraction of the independent spread
// Below this many points the choice is not made (strength order): the
// second skyline launch it needs costs about 13 us, more than the Gray
// order gains on such lists.
constexpr uint64_t kSpreadMinPoints = 1u << 17;

// spread[0] += sum over list entries of the cell sum over S, spread[1] += its
// square, spread[2] = the count. Cell sums are at most 16 * 127, so both
// sums fit 64 bits for any list of 32-bit length.
__global__ void k_cell_spread(const uint4* __restrict__ cells, const uint32_t* __restrict__ ids,
                              const uint32_t* __restrict__ m_ptr, uint32_t S, int d,
                              unsigned long long* __restrict__ spread) {
  const uint32_t m = *m_ptr;
  unsigned long long s1 = 0, s2 = 0;
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < m;
       i += gridDim.x * blockDim.x) {
    const uint4 c = cells[ids ? ids[i] : i];
    uint32_t sum = 0;
    for (int k = 0; k < d; ++k)
      if (S & (1u << k)) sum += (word_of(c, k >> 2) >> (8 * (k & 3))) & 0x7fu;
    s1 += sum;
    s2 += (unsigned long long)sum * sum;
  }
  for (int o = 16; o; o >>= 1) {
    s1 += __shfl_xor_sync(0xffffffffu, s1, o);
    s2 += __shfl_xor_sync(0xffffffffu, s2, o);
  }
  if ((threadIdx.x & 31) == 0 && s1) {
    atomicAdd(&spread[0], s1);
    atomicAdd(&spread[1], s2);
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) spread[2] = m;
}

// Gray order when the variance of the cell sums is below `limit`
// (kGraySpread^2 times the variance of a sum of |S| independent uniform
// cells). Every thread of the sort and skyline kernels evaluates it, so it
// is single precision (FP64 is a slow pipe here: in double it cost 80 us on
// 100k points); the variance is in the thousands and its rounding error
// below 0.1.
__device__ __forceinline__ bool gray_order(const unsigned long long* spread, float limit) {
  const unsigned long long n = spread[2];
  if (n < 2) return false;
  const float inv = 1.0f / (float)n;
  const float mean = (float)spread[0] * inv;
  const float var = (float)spread[1] * inv - mean * mean;
  return var < limit;
}

// key[i] = rank of the median mask of list entry i over the first B
// attributes of S, times 2^sub_bits, plus (when sub_bits > 0) the sum of its
// grid cells over S scaled to sub_bits bits. Sorting by the key groups
// points by partition and, inside a partition, from strong to weak, so
// points that survive long share warps. With sub_mode 1 the sub-key orders
// points by the quartile-cell bits (the cell bit below the median bit) of
// the first sub_bits attributes of S, as a Gray code: a point's pattern is
// ranked by its position in the reflected binary sequence (the prefix XOR of
// its bits, attribute 0 most significant), so consecutive patterns differ in
// one attribute and any run of them varies in few. Consecutive points then
// share their quartile on most attributes, which keeps the minimum-cell
// boxes of 32-point blocks tight. Only the partition part matters for
// correctness. Sub_mode 2 takes the Gray order when the list's cell sums
// are concentrated (gray_order below) and the strength order otherwise.
__global__ void k_mask_keys(const uint4* __restrict__ cells,
                            const uint32_t* __restrict__ ids,
                            const uint32_t* __restrict__ m_ptr, uint32_t S,
                            int d, int B, int depth, int sub_bits, int sub_mode,
                            const uint32_t* __restrict__ rank,
                            uint32_t* __restrict__ keys,
                            const unsigned long long* __restrict__ spread,
                            float spread_limit) {
  const uint32_t m = *m_ptr;
  if (sub_mode == 2) sub_mode = gray_order(spread, spread_limit) ? 1 : 0;
  const int sh = depth - 1;
  const uint32_t cmax = (1u << depth) - 1;
  const uint32_t span = cmax * (uint32_t)__popc(S);
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < m;
       i += gridDim.x * blockDim.x) {
    const uint32_t id = ids ? ids[i] : i;
    const uint4 c = cells[id];
    uint32_t cm = 0, csum = 0, qpat = 0;
    int j = 0;
    for (int k = 0; k < d; ++k) {
      if (!(S & (1u << k))) continue;
      const uint32_t cell = (word_of(c, k >> 2) >> (8 * (k & 3))) & 0x7fu;
      if (j < B) cm |= ((cell >> sh) & 1u) << j;
      if (j < sub_bits && sh >= 1) qpat |= ((cell >> (sh - 1)) & 1u) << (sub_bits - 1 - j);
      csum += cell;
      ++j;
    }
    uint32_t key = rank[cm] << sub_bits;
    if (sub_mode == 1) {
      uint32_t g = qpat;  // rank of qpat in the Gray sequence
      for (int s2 = 1; s2 < 32; s2 <<= 1) g ^= g >> s2;
      key |= g;
    }
    else if (sub_bits && span) key |= (csum * ((1u << sub_bits) - 1)) / span;
    keys[i] = key;
  }
}

// boff[b] = offsets[b << sub_bits] for b in [0, K]: partition offsets out of
// the finer counting-sort offsets.
__global__ void k_partition_offsets(const uint32_t* __restrict__ offsets, uint32_t K,
                                    int sub_bits, uint32_t* __restrict__ boff) {
  for (uint32_t b = blockIdx.x * blockDim.x + threadIdx.x; b <= K;
       b += gridDim.x * blockDim.x)
    boff[b] = offsets[(uint64_t)b << sub_bits];
}

// items[b] = number of 256-point work items of partition b.
__global__ void k_chunk_counts(const uint32_t* __restrict__ boff, uint32_t K,
                               uint32_t* __restrict__ items) {
  for (uint32_t b = blockIdx.x * blockDim.x + threadIdx.x; b < K;
       b += gridDim.x * blockDim.x)
    items[b] = (boff[b + 1] - boff[b] + 255) / 256;
}

// Compact copy of a list in partition order, restricted to the k attributes
// of S: cells repacked so attribute t of S sits in byte t % 4 of word t / 4,
// and attribute-major floats xs[t * pitch + j].
__global__ void k_gather_compact(const uint4* __restrict__ cells,
                                 const float* __restrict__ x, uint64_t n_pad,
                                 const uint32_t* __restrict__ ids,
                                 const uint32_t* __restrict__ sorted,
                                 const uint32_t* __restrict__ m_ptr, uint32_t S,
                                 int d, uint64_t pitch,
                                 uint4* __restrict__ out_cells,
                                 float* __restrict__ out_x) {
  const uint32_t m = *m_ptr;
  for (uint32_t j = blockIdx.x * blockDim.x + threadIdx.x; j < m;
       j += gridDim.x * blockDim.x) {
    const uint32_t pos = sorted[j];
    const uint32_t id = ids ? ids[pos] : pos;
    const uint4 c = cells[id];
    uint32_t w[4] = {0, 0, 0, 0};
    int t = 0;
    for (int k = 0; k < d; ++k) {
      if (!(S & (1u << k))) continue;
      const uint32_t cell = (word_of(c, k >> 2) >> (8 * (k & 3))) & 0x7fu;
      w[t >> 2] |= cell << (8 * (t & 3));
      out_x[(uint64_t)t * pitch + j] = x[(uint64_t)k * n_pad + id];
      ++t;
    }
    out_cells[j] = make_uint4(w[0], w[1], w[2], w[3]);
  }
}

struct PartKernelArgs {
  // Confirmed lists (optional, see k_skyline_part): the points of partition b
  // that are not strictly dominated, conf_*[boff[b] + k] for k < ccount[b],
  // complete once pdone[b] equals b's number of work items.
  uint4* conf_cells;
  float* conf_x;
  uint32_t* ccount;
  uint32_t* pdone;
  const uint32_t* sorted;   // sorted index -> list position (for the output)
  const uint4* cells;       // compact cells in sorted order
  const float* xs;          // compact floats in sorted order, pitch `pitch`
  uint64_t pitch;
  const uint32_t* boff;     // partition offsets in sorted order [K + 1]
  const uint32_t* items;    // work item prefix per partition [K + 1]
  const uint32_t* unrank;   // rank -> mask
  const uint32_t* sub_off;  // mask -> range in sub_list
  const uint32_t* sub_list; // ranks of submasks, level order
  uint32_t K;
  uint8_t* status;          // list position -> status (zeroed, 4-byte padded)
  const uint32_t* splits;   // slices per work item of partition b [K]
  const uint32_t* cta_off;  // first CTA of partition b [K + 1]
  uint32_t lvl_mul;         // strength level = cell sum * lvl_mul / lvl_span
  uint32_t lvl_span;        //   (the sort's sub-key, k_mask_keys); 0: no cut
  // Sliced lists: the cell-sum spread and its limit (gray_order); when the
  // partitions are in Gray order, q tiles are box-tested (nullptr: never).
  const unsigned long long* spread;
  float spread_limit;
};

// Cell sum of compact cells over NA attributes (the sort's strength level
// is sum * lvl_mul / lvl_span, k_mask_keys).
template <int NA>
__device__ __forceinline__ uint32_t cell_sum_na(const uint4& c) {
  uint32_t sum = 0;
#pragma unroll
  for (int k = 0; k < NA; ++k) sum += (word_of(c, k >> 2) >> (8 * (k & 3))) & 0x7fu;
  return sum;
}

constexpr uint32_t kMaxSplits = 64;
constexpr uint64_t kMinSliceWork = 256;  // q's (one tile): below this a slice is not worth a CTA

// Work-proportional slicing of the skyline kernel's items (one CTA of 1024
// threads, thread b = partition rank b). An item of partition b scans the
// points of every partition under b's mask, so its cost is work[b] = their
// count, the same for all of b's items. With W = max(total work / target,
// kMinSliceWork), each item of b gets ceil(work[b] / W) slices (at most
// kMaxSplits), so the heavy items of high-mask partitions no longer set the
// kernel's duration. cta_off is the exclusive prefix of CTAs per partition.
__global__ void __launch_bounds__(1024) k_split_plan(const uint32_t* __restrict__ boff,
                                                     const uint32_t* __restrict__ items,
                                                     const uint32_t* __restrict__ unrank,
                                                     const uint32_t* __restrict__ sub_off,
                                                     const uint32_t* __restrict__ sub_list,
                                                     uint32_t K, uint32_t target,
                                                     uint32_t* __restrict__ splits,
                                                     uint32_t* __restrict__ cta_off) {
  __shared__ unsigned long long s_total;
  __shared__ uint32_t wsum[32];
  const uint32_t b = threadIdx.x;
  const int lane = b & 31, wid = b >> 5;
  if (b == 0) s_total = 0;
  __syncthreads();
  unsigned long long work = 0;
  uint32_t chunks = 0;
  if (b < K) {
    const uint32_t mb = unrank[b];
    for (uint32_t si = sub_off[mb]; si < sub_off[mb + 1]; ++si) {
      const uint32_t qb = sub_list[si];
      work += boff[qb + 1] - boff[qb];
    }
    chunks = items[b + 1] - items[b];
    if (chunks) atomicAdd(&s_total, work * chunks);
  }
  __syncthreads();
  const unsigned long long total = s_total;
  unsigned long long W = target ? (total + target - 1) / target : ~0ull;
  if (W < kMinSliceWork) W = kMinSliceWork;
  uint32_t sb = 1;
  if (b < K && target) {
    const unsigned long long q = (work + W - 1) / W;
    sb = (uint32_t)(q < 1 ? 1 : (q > kMaxSplits ? kMaxSplits : q));
  }
  if (b < K) splits[b] = sb;
  const uint32_t c = b < K ? chunks * sb : 0u;
  uint32_t inc = c;
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t u = __shfl_up_sync(0xffffffffu, inc, o);
    if (lane >= o) inc += u;
  }
  if (lane == 31) wsum[wid] = inc;
  __syncthreads();
  if (wid == 0) {
    const uint32_t v = wsum[lane];
    uint32_t vi = v;
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t u = __shfl_up_sync(0xffffffffu, vi, o);
      if (lane >= o) vi += u;
    }
    wsum[lane] = vi - v;
  }
  __syncthreads();
  const uint32_t excl = wsum[wid] + inc - c;
  if (b < K) cta_off[b] = excl;
  if (b == K - 1) cta_off[K] = excl + c;
}

// NA = number of attributes of the subspace (all of them are compared).
//
// Confirmed lists. Work items start in lattice-level order, so the lower
// partitions under a CTA's mask have often finished by the time it reaches
// them. A finished partition is read through its confirmed list (its points
// that are not strictly dominated) instead of all its points. That is exact:
// if a strictly dominated q dominates p, the confirmed point that strictly
// dominates q lies in a partition under p's mask as well and strictly
// dominates p. Nothing waits: an unfinished partition is read in full. A CTA
// publishes its confirmed points, fences, then counts itself in pdone.
//
// Slices (k_split_plan). An item of partition b is cut into splits[b] CTAs,
// each taking an equal slice of the concatenated submask partitions; the
// slices' statuses combine by a byte-wise atomic OR of bit flags (1
// dominated, 2 strictly dominated; 3 reads as strictly dominated). A sliced
// partition neither publishes nor uses confirmed lists (no CTA knows its
// points' final status); the others still do.
//
// LV (level cutoffs, used on unsliced lists): a thread stops scanning a
// sorted partition at the first q above its own strength level.
constexpr uint32_t kFullMask = 0xffffffffu;

// Up to 10 attributes the sliced variant holds 6 CTAs per SM (40 registers,
// no spill; it had taken 48 and 5 CTAs): 1M x 10 anticorrelated full
// skycube 28.4 -> 27.7 ms. Above 10 attributes the bound would spill, and
// the unsliced level-cutoff variant (LV) keeps the free register budget.
// BOX (sliced lists only): q tiles are box-tested. Both instantiations are
// launched for a sliced list whose order follows the spread, and the one
// that does not match the device's choice (gray_order) returns at once: a
// runtime switch kept both paths' registers live and spilled at 40.
template <int NA, bool LV, bool BOX>
__global__ void __launch_bounds__(256, (!LV && NA <= 10) ? 6 : 1) k_skyline_part(PartKernelArgs a) {
  constexpr int NW = (NA + 3) / 4;
  if (a.spread != nullptr && gray_order(a.spread, a.spread_limit) != BOX) return;
  constexpr int TQ = 256;
  __shared__ uint4 q_cells[TQ];
  __shared__ float q_x[NA][TQ];
  __shared__ uint16_t q_sum[LV ? TQ : 1];

  __shared__ uint32_t s_conf_end;
  __shared__ unsigned long long s_total;
  // CTAs go in partition rank order (lattice level: lower partitions first).
  if (blockIdx.x >= a.cta_off[a.K]) return;
  uint32_t lo = 0, hi = a.K;
  while (hi - lo > 1) {
    const uint32_t mid = (lo + hi) >> 1;
    if (a.cta_off[mid] <= blockIdx.x) lo = mid; else hi = mid;
  }
  const uint32_t b = lo;
  const uint32_t splits = a.splits[b];
  const uint32_t local = blockIdx.x - a.cta_off[b];
  const uint32_t chunk = local / splits;
  const uint32_t sp = local - chunk * splits;
  const bool use_conf = a.conf_cells != nullptr && splits == 1;
  const uint32_t pbeg = a.boff[b] + chunk * TQ;
  const uint32_t pend = min(a.boff[b + 1], pbeg + TQ);
  const uint32_t i = pbeg + threadIdx.x;
  const bool valid = i < pend;

  uint32_t hS[NW];
#pragma unroll
  for (int w = 0; w < NW; ++w) hS[w] = guard_mask((1u << NA) - 1, w);
  uint32_t pc[NW], pH[NW];
  float pv[NA];
#pragma unroll
  for (int w = 0; w < NW; ++w) pc[w] = pH[w] = 0;
#pragma unroll
  for (int k = 0; k < NA; ++k) pv[k] = 0.f;
  uint4 my_cells = make_uint4(0, 0, 0, 0);
  if (valid) {
    my_cells = a.cells[i];
#pragma unroll
    for (int w = 0; w < NW; ++w) {
      pc[w] = word_of(my_cells, w);
      pH[w] = pc[w] | kGuard;
    }
#pragma unroll
    for (int k = 0; k < NA; ++k) pv[k] = a.xs[(uint64_t)k * a.pitch + i];
  }

  uint8_t st = 0;
  bool done = !valid;
  // Sort-filter bound: a q that dominates p, even weakly, has every cell
  // <= p's, so its cell sum and strength level are <= p's. Inside a
  // partition q's ascend in level, so a thread is finished with the
  // partition at the first q above its own level. level(q) > level(p)
  // exactly when cellsum(q) >= sum_cut, the smallest sum of a higher level.
  uint32_t sum_cut = 0xffffffffu;  // no cut without strength levels
  if (LV && a.lvl_mul) {
    const uint32_t plv = cell_sum_na<NA>(my_cells) * a.lvl_mul / a.lvl_span;
    sum_cut = ((plv + 1) * a.lvl_span + a.lvl_mul - 1) / a.lvl_mul;
  }
  const uint32_t mb = a.unrank[b];
  const uint32_t s0 = a.sub_off[mb], s1 = a.sub_off[mb + 1];
  // This CTA's slice [s_lo, s_hi) of the concatenated submask partitions.
  uint64_t s_lo = 0, s_hi = ~0ull;
  if (splits > 1) {
    if (threadIdx.x == 0) s_total = 0;
    __syncthreads();
    unsigned long long part = 0;
    for (uint32_t si = s0 + threadIdx.x; si < s1; si += blockDim.x) {
      const uint32_t qb = a.sub_list[si];
      part += a.boff[qb + 1] - a.boff[qb];
    }
    if (part) atomicAdd(&s_total, part);
    __syncthreads();
    const uint64_t total = s_total;
    s_lo = total * sp / splits;
    s_hi = total * (sp + 1) / splits;
  }
  // Unsliced lists with level cutoffs stream q tiles per CTA (a thread stops
  // at its level, so the CTA's tiles stay short); sliced lists stream them
  // per warp. Measured both ways: the per-warp loop cost the per-cuboid
  // form 800 -> 954 ms on 1M x 10, the per-CTA loop cost sliced lists up to
  // 34 % (581k x 10 ties).
  if constexpr (LV) {
  bool all_done = false;
  uint64_t acc = 0;  // q's of the partitions before si (uniform over the CTA)
  for (uint32_t si = s0; si < s1 && !all_done && acc < s_hi; ++si) {
    const uint32_t qb = a.sub_list[si];
    uint32_t qbeg = a.boff[qb];
    uint32_t qend = a.boff[qb + 1];
    if (splits > 1) {
      const uint64_t start = acc, sz = qend - qbeg;
      acc += sz;
      const uint64_t c0 = max(s_lo, start), c1 = min(s_hi, start + sz);
      if (c0 >= c1) continue;
      qend = qbeg + (uint32_t)(c1 - start);
      qbeg = qbeg + (uint32_t)(c0 - start);
    }
    bool beyond = false;  // past this thread's level in this partition
    bool conf = false;
    if (use_conf && qb != b) {
      if (threadIdx.x == 0) {
        uint32_t e = 0xffffffffu;
        const uint32_t need = a.items[qb + 1] - a.items[qb];
        if (atomicAdd(&a.pdone[qb], 0u) == need) {
          __threadfence();
          e = qbeg + atomicAdd(&a.ccount[qb], 0u);
        }
        s_conf_end = e;
      }
      __syncthreads();
      if (s_conf_end != 0xffffffffu) {
        conf = true;
        qend = s_conf_end;
      }
    }
    const uint4* qc = conf ? a.conf_cells : a.cells;
    const float* qxs = conf ? a.conf_x : a.xs;
    bool first = true;
    for (uint32_t base = qbeg; base < qend; base += TQ) {
      // Without level cutoffs, or on a partition's first tile (nobody is
      // beyond yet), the vote is "every point of the CTA is strictly
      // dominated": the CTA is finished.
      if (__syncthreads_and(done || (LV && beyond))) {
        if (!LV || first) all_done = true;
        break;
      }
      first = false;
      const uint32_t j = base + threadIdx.x;
      if (j < qend) {
        // Confirmed lists are written during this launch by other SMs: read
        // them through L2 (ld.cg), never from a possibly stale L1 line.
        uint4 qcl;
        if (conf) {
          qcl = __ldcg(qc + j);
#pragma unroll
          for (int k = 0; k < NA; ++k) q_x[k][threadIdx.x] = __ldcg(qxs + (uint64_t)k * a.pitch + j);
        } else {
          qcl = qc[j];
#pragma unroll
          for (int k = 0; k < NA; ++k) q_x[k][threadIdx.x] = qxs[(uint64_t)k * a.pitch + j];
        }
        q_cells[threadIdx.x] = qcl;
        if constexpr (LV) q_sum[threadIdx.x] = (uint16_t)cell_sum_na<NA>(qcl);
      }
      __syncthreads();
      if (!done && !(LV && beyond)) {
        uint32_t lim = min((uint32_t)TQ, qend - base);
        if (LV && !conf && sum_cut != 0xffffffffu) {
          // First q of the tile above p's level (levels ascend in a sorted
          // partition; confirmed lists are unordered and fully scanned).
          uint32_t lo = 0, hi = lim;
          while (lo < hi) {
            const uint32_t mid = (lo + hi) >> 1;
            if (q_sum[mid] >= sum_cut) hi = mid; else lo = mid + 1;
          }
          if (lo < lim) {
            lim = lo;
            beyond = true;
          }
        }
        for (uint32_t t = 0; t < lim; ++t) {
          const uint4 q = q_cells[t];
          uint32_t worse = 0;  // guard bits where cell(q) > cell(p)
#pragma unroll
          for (int w = 0; w < NW; ++w) worse |= ~(pH[w] - word_of(q, w)) & hS[w];
          if (worse) continue;
          uint32_t not_less = 0;  // guard bits where cell(q) >= cell(p)
#pragma unroll
          for (int w = 0; w < NW; ++w)
            not_less |= ge_bytes(word_of(q, w) | kGuard, pc[w]) & hS[w];
          if (!not_less) {  // a smaller cell on every attribute: strict
            st = 2;
            done = true;
            break;
          }
          bool le = true, lt_any = false, lt_all = true;
#pragma unroll
          for (int k = 0; k < NA; ++k) {
            const float v = q_x[k][t];
            le &= (v <= pv[k]);
            lt_any |= (v < pv[k]);
            lt_all &= (v < pv[k]);
          }
          if (le && lt_any) {
            if (lt_all) {
              st = 2;
              done = true;
              break;
            }
            st = 1;
          }
        }
      }
      __syncthreads();
    }
  }
  } else {
  uint64_t acc = 0;  // q's of the partitions before si
  // Each warp streams the q's through its own 32-entry slice of the tile
  // arrays and stops on its own: no CTA barrier inside the loop, so a warp
  // whose points are all settled does not wait for the slowest warp.
  const int lane = threadIdx.x & 31;
  // In Gray order a tile's q's share their quartile on most attributes, so
  // its byte-wise minimum cells often lie above a point's cell somewhere;
  // a point below the minimum on some attribute is dominated by no q of the
  // tile, and a tile no point of the warp can be dominated by is skipped.
  // In strength order the boxes are loose and the test only costs
  // (1M x 10 anticorrelated: 6.9 -> 8.3 ms).
  constexpr bool box = BOX;
  // With tile boxes a tile's floats are fetched only when some lane of the
  // warp walks it (after the box test, so a tile every lane's box rejects is
  // never read past its cells). Measured on anticorrelated data, full-space
  // skyline, before -> after: 1M x 6 0.81 -> 0.77 ms, x 8 2.67 -> 2.48, x 9
  // 4.60 -> 4.39, x 10 5.95 -> 5.83, 600k x 11 4.87 -> 4.37, 400k x 14
  // 5.18 -> 4.80; slower at 400k x 12 (3.57 -> 3.63) and 300k x 16 (3.85
  // -> 3.91), which load the floats with the cells as before.
  constexpr bool defer_x = box && NA != 12 && NA != 16;
  const uint32_t wbase = threadIdx.x & ~31u;  // this warp's slice
  bool wdone = false;  // every point of the warp is settled
  for (uint32_t si = s0; si < s1 && !wdone && acc < s_hi; ++si) {
    const uint32_t qb = a.sub_list[si];
    uint32_t qbeg = a.boff[qb];
    uint32_t qend = a.boff[qb + 1];
    if (splits > 1) {
      const uint64_t start = acc, sz = qend - qbeg;
      acc += sz;
      const uint64_t c0 = max(s_lo, start), c1 = min(s_hi, start + sz);
      if (c0 >= c1) continue;
      qend = qbeg + (uint32_t)(c1 - start);
      qbeg = qbeg + (uint32_t)(c0 - start);
    }
    bool beyond = false;  // past this thread's level in this partition
    bool conf = false;
    if (use_conf && qb != b) {
      uint32_t e = 0xffffffffu;
      if (lane == 0) {
        const uint32_t need = a.items[qb + 1] - a.items[qb];
        if (atomicAdd(&a.pdone[qb], 0u) == need) {
          __threadfence();
          e = qbeg + atomicAdd(&a.ccount[qb], 0u);
        }
      }
      e = __shfl_sync(kFullMask, e, 0);
      if (e != 0xffffffffu) {
        __threadfence();  // the list's entries are read after its count
        conf = true;
        qend = e;
      }
    }
    const uint4* qc = conf ? a.conf_cells : a.cells;
    const float* qxs = conf ? a.conf_x : a.xs;
    bool first = true;
    for (uint32_t base = qbeg; base < qend; base += 32) {
      // Without level cutoffs, or on a partition's first tile (nobody is
      // beyond yet), the vote is "every point of the warp is strictly
      // dominated": the warp is finished.
      if (__all_sync(kFullMask, done || (LV && beyond))) {
        if (!LV || first) wdone = true;
        break;
      }
      first = false;
      const uint32_t j = base + lane;
      uint4 qcl = make_uint4(0x7f7f7f7fu, 0x7f7f7f7fu, 0x7f7f7f7fu, 0x7f7f7f7fu);
      if (j < qend) {
        // Confirmed lists are written during this launch by other SMs: read
        // them through L2 (ld.cg), never from a possibly stale L1 line.
        if constexpr (defer_x) {
          qcl = conf ? __ldcg(qc + j) : qc[j];
        } else if (conf) {
          qcl = __ldcg(qc + j);
#pragma unroll
          for (int k = 0; k < NA; ++k) q_x[k][threadIdx.x] = __ldcg(qxs + (uint64_t)k * a.pitch + j);
        } else {
          qcl = qc[j];
#pragma unroll
          for (int k = 0; k < NA; ++k) q_x[k][threadIdx.x] = qxs[(uint64_t)k * a.pitch + j];
        }
        q_cells[threadIdx.x] = qcl;
        if constexpr (LV) q_sum[threadIdx.x] = (uint16_t)cell_sum_na<NA>(qcl);
      }
      bool box_out = false;  // no q of the tile dominates this point
      if constexpr (box) {
        uint32_t worse = 0;  // guard bits where the minimum cell is above p's
#pragma unroll
        for (int w = 0; w < NW; ++w) {  // one word at a time: few live registers
          uint32_t mn = word_of(qcl, w);
#pragma unroll
          for (int o = 1; o < 32; o <<= 1) mn = __vminu4(mn, __shfl_xor_sync(kFullMask, mn, o));
          worse |= ~(pH[w] - mn) & hS[w];
        }
        box_out = worse != 0;
      }
      const bool walk = !done && !(LV && beyond) && !box_out;
      if constexpr (defer_x) {
        if (__any_sync(kFullMask, walk) && j < qend) {
          if (conf) {
#pragma unroll
            for (int k = 0; k < NA; ++k) q_x[k][threadIdx.x] = __ldcg(qxs + (uint64_t)k * a.pitch + j);
          } else {
#pragma unroll
            for (int k = 0; k < NA; ++k) q_x[k][threadIdx.x] = qxs[(uint64_t)k * a.pitch + j];
          }
        }
      }
      __syncwarp();
      if (walk) {
        uint32_t lim = min(32u, qend - base);
        if (LV && !conf && sum_cut != 0xffffffffu) {
          // First q of the tile above p's level (levels ascend in a sorted
          // partition; confirmed lists are unordered and fully scanned).
          uint32_t lo = 0, hi = lim;
          while (lo < hi) {
            const uint32_t mid = (lo + hi) >> 1;
            if (q_sum[wbase + mid] >= sum_cut) hi = mid; else lo = mid + 1;
          }
          if (lo < lim) {
            lim = lo;
            beyond = true;
          }
        }
        for (uint32_t t = 0; t < lim; ++t) {
          const uint4 q = q_cells[wbase + t];
          uint32_t worse = 0;  // guard bits where cell(q) > cell(p)
#pragma unroll
          for (int w = 0; w < NW; ++w) worse |= ~(pH[w] - word_of(q, w)) & hS[w];
          if (worse) continue;
          uint32_t not_less = 0;  // guard bits where cell(q) >= cell(p)
#pragma unroll
          for (int w = 0; w < NW; ++w)
            not_less |= ge_bytes(word_of(q, w) | kGuard, pc[w]) & hS[w];
          if (!not_less) {  // a smaller cell on every attribute: strict
            st = 2;
            done = true;
            break;
          }
          bool le = true, lt_any = false, lt_all = true;
#pragma unroll
          for (int k = 0; k < NA; ++k) {
            const float v = q_x[k][wbase + t];
            le &= (v <= pv[k]);
            lt_any |= (v < pv[k]);
            lt_all &= (v < pv[k]);
          }
          if (le && lt_any) {
            if (lt_all) {
              st = 2;
              done = true;
              break;
            }
            st = 1;
          }
        }
      }
      __syncwarp();
    }
  }
  }
  if (valid) {
    const uint32_t pos = a.sorted[i];
    if (splits == 1)
      a.status[pos] = st;
    else if (st)
      atomicOr(reinterpret_cast<unsigned int*>(a.status + (pos & ~3u)),
               (unsigned int)st << (8 * (pos & 3u)));
  }
  if (use_conf) {
    if (valid && st != 2) {
      const uint32_t slot = a.boff[b] + atomicAdd(&a.ccount[b], 1u);
      a.conf_cells[slot] = my_cells;
#pragma unroll
      for (int k = 0; k < NA; ++k) a.conf_x[(uint64_t)k * a.pitch + slot] = pv[k];
    }
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) atomicAdd(&a.pdone[b], 1u);
  }
}

static inline unsigned blocks_for(uint64_t items, int threads, int cap);

int launch_mask_keys(cudaStream_t s, const uint4* cells, const uint32_t* ids,
                     const uint32_t* m_ptr, uint64_t m_max, uint32_t S, int d,
                     int B, int depth, int sub_bits, int sub_mode, const uint32_t* rank,
                     uint32_t* keys) {
  k_mask_keys<<<blocks_for(m_max, 256, 152 * 8), 256, 0, s>>>(cells, ids, m_ptr, S, d, B, depth,
                                                               sub_bits, sub_mode, rank, keys,
                                                               nullptr, 0.0f);
  SKC_LAUNCH_CHECK();
  return SKC_OK;
}

int launch_partition_offsets(cudaStream_t s, const uint32_t* fine, uint32_t K, int sub_bits,
                             uint32_t* boff) {
  k_partition_offsets<<<blocks_for(K + 1, 256, 64), 256, 0, s>>>(fine, K, sub_bits, boff);
  SKC_LAUNCH_CHECK();
  return SKC_OK;
}

static inline unsigned blocks_for(uint64_t items, int threads, int cap) {
  uint64_t b = (items + threads - 1) / threads;
  if (b < 1) b = 1;
  if (b > (uint64_t)cap) b = cap;
  return (unsigned)b;
}

int launch_partition_skyline(cudaStream_t s, int d, int depth,
                             const LevelTables& T, const PartitionSkylineArgs& a,
                             const PartScratch& ps) {
  const uint32_t K = 1u << T.B;
  const int na = __builtin_popcount(a.S);
  // Strength order inside partitions: as many cell-sum levels as keep the
  // counting sort at <= kMaxSortBuckets buckets.
  int sub_bits = 0;
  while (sub_bits < 8 && ((uint64_t)K << (sub_bits + 1)) <= kMaxSortBuckets) ++sub_bits;
  const uint32_t KB = K << sub_bits;
  BucketScratch bs;
  bs.keys = ps.keys;
  bs.counts = ps.fine;
  bs.cursor = ps.cursor;
  // Sliced lists: the order inside the partitions by the spread of the
  // cell sums over the list before the prefilter (gray_order).
  const bool by_spread = a.split_target && depth >= 2 && ps.spread &&
                         (a.spread_m || a.spread_ready) && a.m_max >= kSpreadMinPoints;
  const uint32_t c1 = 1u << depth;  // cells per attribute
  const float spread_limit =
      (float)(kGraySpread * kGraySpread * (double)na * ((double)c1 * c1 - 1.0) / 12.0);
  if (by_spread && !a.spread_ready) {
    SKC_CUDA(cudaMemsetAsync(ps.spread, 0, 3 * sizeof(unsigned long long), s));
    k_cell_spread<<<blocks_for(a.m_max, 256, 152 * 4), 256, 0, s>>>(
        a.cells, a.spread_ids, a.spread_m, a.S, d, ps.spread);
    SKC_LAUNCH_CHECK();
  }
  k_mask_keys<<<blocks_for(a.m_max, 256, 152 * 8), 256, 0, s>>>(
      a.cells, a.ids, a.m_ptr, a.S, d, T.B, depth, sub_bits, by_spread ? 2 : 0, T.rank, ps.keys,
      ps.spread, spread_limit);
  SKC_LAUNCH_CHECK();
  SKC_TRY(launch_counting_sort(s, ps.keys, a.m_ptr, a.m_max, KB, bs, ps.sorted, nullptr));
  k_partition_offsets<<<blocks_for(K + 1, 256, 64), 256, 0, s>>>(ps.fine, K, sub_bits, ps.counts);
  SKC_LAUNCH_CHECK();
  const uint64_t pitch = (a.m_max + 127) / 128 * 128;
  k_gather_compact<<<blocks_for(a.m_max, 256, 152 * 8), 256, 0, s>>>(
      a.cells, a.x, a.n_pad, a.ids, ps.sorted, a.m_ptr, a.S, d, pitch, ps.ccells, ps.cx);
  SKC_LAUNCH_CHECK();
  k_chunk_counts<<<blocks_for(K, 256, 64), 256, 0, s>>>(ps.counts, K, ps.items);
  SKC_LAUNCH_CHECK();
  SKC_TRY(launch_scan_single_u32(s, ps.items, K));
  // Slices per item and CTA offsets, in the counting sort's cursor scratch
  // (free once the partition offsets are extracted): [0, K) and [K, 2K + 1).
  uint32_t* splits = ps.cursor;
  uint32_t* cta_off = ps.cursor + K;
  k_split_plan<<<1, 1024, 0, s>>>(ps.counts, ps.items, T.unrank, T.sub_off, T.sub_list, K,
                                  a.split_target, splits, cta_off);
  SKC_LAUNCH_CHECK();
  PartKernelArgs k{ps.conf_cells, ps.conf_x, ps.ccount, ps.pdone, ps.sorted, ps.ccells, ps.cx,
                   pitch, ps.counts, ps.items, T.unrank, T.sub_off, T.sub_list, K, a.status,
                   splits, cta_off,
                   // Level cutoffs pay on lists full of dominated points (no
                   // prefilter); on candidate-dense, sliced lists they only
                   // cost (581k x 10 ties survivors: 3.05 -> 3.43 ms).
                   a.split_target ? 0u : (1u << sub_bits) - 1u,
                   ((1u << depth) - 1u) * (uint32_t)na,
                   by_spread ? ps.spread : nullptr, spread_limit};
  // Split CTAs OR their statuses in: start from zero (the buffer is padded
  // to a multiple of 4 bytes).
  SKC_CUDA(cudaMemsetAsync(a.status, 0, (a.m_max + 3) & ~3ull, s));
  if (ps.conf_cells) {
    SKC_CUDA(cudaMemsetAsync(ps.ccount, 0, K * sizeof(uint32_t), s));
    SKC_CUDA(cudaMemsetAsync(ps.pdone, 0, K * sizeof(uint32_t), s));
  }
  // Upper bound of the CTAs k_split_plan hands out: sum over items of
  // ceil(work / W) <= target + items.
  const unsigned grid = (unsigned)((a.m_max + 255) / 256 + K + a.split_target);
#define SKC_PART_CASE(N)                                           \
  case N:                                                          \
    if (k.lvl_mul) {                                               \
      k_skyline_part<N, true, false><<<grid, 256, 0, s>>>(k);      \
    } else {                                                       \
      if (by_spread) k_skyline_part<N, false, true><<<grid, 256, 0, s>>>(k); \
      k_skyline_part<N, false, false><<<grid, 256, 0, s>>>(k);     \
    }                                                              \
    break;
  switch (na) {
    SKC_PART_CASE(1) SKC_PART_CASE(2) SKC_PART_CASE(3) SKC_PART_CASE(4)
    SKC_PART_CASE(5) SKC_PART_CASE(6) SKC_PART_CASE(7) SKC_PART_CASE(8)
    SKC_PART_CASE(9) SKC_PART_CASE(10) SKC_PART_CASE(11) SKC_PART_CASE(12)
    SKC_PART_CASE(13) SKC_PART_CASE(14) SKC_PART_CASE(15) SKC_PART_CASE(16)
    default:
      return set_error(SKC_ERR_INVALID, "subspace with %d attributes", na);
  }
#undef SKC_PART_CASE
  SKC_LAUNCH_CHECK();
  return SKC_OK;
}

}  // namespace skc
