// Pruner prefilter ahead of the full-space skyline: the suite's priority-queue
// filter (PQFilter::ExecuteExtended, src/utilities/pq_filter.h:140-231,
// applied by MDMC<D>::Init when n > 2 * pq_size, src/mdmc/MDMC.cu:251-252).
// The pq_size points of smallest norm become pruners and every point that a
// pruner strictly dominates is dropped.
//
// Why it is exact: if r is dropped (a pruner t is < r on every attribute)
// and r dominates a point s (<= everywhere), then t is < s everywhere and s
// is dropped as well. So every point that dominates or strictly dominates a
// survivor is a survivor, and the skyline / extended-skyline status of each
// survivor over the survivors equals its status over all points; dropped
// points are strictly dominated, status 2.
//
// GB300 form. The norm is the cell sum over S (rank space, so attributes of
// different scales weigh alike; the suite sums raw values). The K smallest
// are picked without a sort: a 2048-bin histogram of cell sums (127 * 16 <
// 2048), a one-block scan for the threshold bin, a collection pass, and a
// one-block rank by (sum, id) so the strongest pruners are tried first.
// The filter holds the ranked pruners (cells + floats) in shared memory;
// one thread per point walks them until one strictly dominates it: a SWAR
// cell test decides most pairs, floats are read only on equal cells.
#include <algorithm>

#include "kernels.cuh"

namespace skc {

constexpr uint32_t kSumBins = 2048;

__device__ __forceinline__ uint32_t cell_sum(const uint4& c, uint32_t S, int d) {
  uint32_t s = 0;
  for (int k = 0; k < d; ++k)
    if ((S >> k) & 1u) s += (word_of(c, k >> 2) >> (8 * (k & 3))) & 0x7fu;
  return s;
}

__global__ void __launch_bounds__(256) k_pruner_hist(const uint4* __restrict__ cells,
                                                     const uint32_t* __restrict__ ids,
                                                     const uint32_t* __restrict__ m_ptr,
                                                     uint32_t S, int d,
                                                     uint32_t* __restrict__ hist) {
  __shared__ uint32_t h[kSumBins];
  for (uint32_t b = threadIdx.x; b < kSumBins; b += blockDim.x) h[b] = 0;
  __syncthreads();
  const uint32_t m = *m_ptr;
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < m; i += gridDim.x * blockDim.x) {
    const uint32_t id = ids ? ids[i] : i;
    atomicAdd(&h[cell_sum(cells[id], S, d)], 1u);
  }
  __syncthreads();
  for (uint32_t b = threadIdx.x; b < kSumBins; b += blockDim.x)
    if (h[b]) atomicAdd(&hist[b], h[b]);
}

// sel[0] = threshold sum, sel[1] = points below it, sel[2] = pruner count
// Kp = min(K, m), sel[3] / sel[4] = collection cursors (zeroed here).
__global__ void __launch_bounds__(1024) k_pruner_select(const uint32_t* __restrict__ hist,
                                                        const uint32_t* __restrict__ m_ptr,
                                                        uint32_t K, uint32_t* __restrict__ sel) {
  __shared__ uint32_t wsum[32];
  const uint32_t m = *m_ptr;
  const uint32_t Kp = min(K, m);
  const int t = threadIdx.x, lane = t & 31, wid = t >> 5;
  if (t == 0) {
    sel[0] = 0;
    sel[1] = 0;
    sel[2] = Kp;
    sel[3] = 0;
    sel[4] = 0;
  }
  const uint32_t h0 = hist[2 * t], h1 = hist[2 * t + 1];
  const uint32_t c = h0 + h1;
  uint32_t inc = c;  // inclusive scan over the warp
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t u = __shfl_up_sync(0xffffffffu, inc, o);
    if (lane >= o) inc += u;
  }
  if (lane == 31) wsum[wid] = inc;
  __syncthreads();
  if (wid == 0) {
    uint32_t v = wsum[lane], vi = v;
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t u = __shfl_up_sync(0xffffffffu, vi, o);
      if (lane >= o) vi += u;
    }
    wsum[lane] = vi - v;  // exclusive prefix of the warps
  }
  __syncthreads();
  const uint32_t e0 = wsum[wid] + inc - c;  // points with sum < 2t
  const uint32_t e1 = e0 + h0;              // points with sum < 2t + 1
  // The threshold bin is the first whose inclusive count reaches Kp.
  if (Kp > 0) {
    if (e0 < Kp && e0 + h0 >= Kp) {
      sel[0] = 2 * t;
      sel[1] = e0;
    } else if (e1 < Kp && e1 + h1 >= Kp) {
      sel[0] = 2 * t + 1;
      sel[1] = e1;
    }
  }
}

__global__ void __launch_bounds__(256) k_pruner_collect(const uint4* __restrict__ cells,
                                                        const uint32_t* __restrict__ ids,
                                                        const uint32_t* __restrict__ m_ptr,
                                                        uint32_t S, int d,
                                                        uint32_t* __restrict__ sel,
                                                        uint32_t* __restrict__ pr_ids,
                                                        uint32_t* __restrict__ pr_key) {
  const uint32_t m = *m_ptr;
  const uint32_t thr = sel[0], below = sel[1], Kp = sel[2];
  if (Kp == 0) return;
  const int lane = threadIdx.x & 31;
  const uint32_t warp0 = (blockIdx.x * blockDim.x + threadIdx.x) & ~31u;
  const uint32_t stride = gridDim.x * blockDim.x;
  for (uint32_t base = warp0; base < m; base += stride) {
    const uint32_t i = base + lane;
    uint32_t id = 0, s = 0xffffffffu;
    if (i < m) {
      id = ids ? ids[i] : i;
      s = cell_sum(cells[id], S, d);
    }
    // Warp-aggregated cursors: one atomic per warp and class.
    const uint32_t lo = __ballot_sync(0xffffffffu, s < thr);
    const uint32_t eq = __ballot_sync(0xffffffffu, s == thr);
    uint32_t lo_base = 0, eq_base = 0;
    if (lane == 0) {
      if (lo) lo_base = atomicAdd(&sel[3], (uint32_t)__popc(lo));
      if (eq) eq_base = atomicAdd(&sel[4], (uint32_t)__popc(eq));
    }
    lo_base = __shfl_sync(0xffffffffu, lo_base, 0);
    eq_base = __shfl_sync(0xffffffffu, eq_base, 0);
    const uint32_t before = (1u << lane) - 1u;
    uint32_t slot = 0xffffffffu;
    if (s < thr) {
      slot = lo_base + __popc(lo & before);
    } else if (s == thr) {
      const uint32_t t = eq_base + __popc(eq & before);
      if (t < Kp - below) slot = below + t;
    }
    if (slot < Kp) {
      pr_ids[slot] = id;
      pr_key[slot] = s;
    }
  }
}

// Ranks the Kp pruners by (sum, id) and stores their cells and floats in
// rank order: out_x[k * K + r] for attribute k.
__global__ void __launch_bounds__(1024) k_pruner_order(const uint32_t* __restrict__ pr_ids,
                                                       const uint32_t* __restrict__ pr_key,
                                                       const uint32_t* __restrict__ sel,
                                                       const uint4* __restrict__ cells,
                                                       const float* __restrict__ x,
                                                       uint64_t n_pad, int d, uint32_t K,
                                                       uint4* __restrict__ out_cells,
                                                       float* __restrict__ out_x) {
  __shared__ unsigned long long key[kMaxPruners];
  const uint32_t Kp = sel[2];
  for (uint32_t t = threadIdx.x; t < Kp; t += blockDim.x)
    key[t] = ((unsigned long long)pr_key[t] << 32) | pr_ids[t];
  __syncthreads();
  for (uint32_t t = threadIdx.x; t < Kp; t += blockDim.x) {
    const unsigned long long me = key[t];
    uint32_t r = 0;
    for (uint32_t j = 0; j < Kp; ++j) r += key[j] < me;
    const uint32_t id = (uint32_t)me;
    out_cells[r] = cells[id];
    for (int k = 0; k < d; ++k) out_x[(uint64_t)k * K + r] = x[(uint64_t)k * n_pad + id];
  }
}

// st[i] = 2 when one of the pruners of rank [r0, r1) strictly dominates
// list entry i on S, else 0. With gate_m set, the pass runs only when the
// list holds at least *gate_m / 4 entries (otherwise every entry is kept).
template <int D>
__global__ void __launch_bounds__(256) k_prefilter(const uint4* __restrict__ cells,
                                                   const float* __restrict__ x, uint64_t n_pad,
                                                   const uint32_t* __restrict__ ids,
                                                   const uint32_t* __restrict__ m_ptr, uint32_t S,
                                                   const uint32_t* __restrict__ sel,
                                                   const uint4* __restrict__ pr_cells,
                                                   const float* __restrict__ pr_x, uint32_t K,
                                                   uint32_t r0, uint32_t r1,
                                                   const uint32_t* __restrict__ gate_m,
                                                   uint8_t* __restrict__ st) {
  constexpr int NW = (D + 3) / 4;
  extern __shared__ uint4 sm4[];
  const uint32_t R = r1 - r0;                      // smem rows
  uint4* s_cells = sm4;                            // [R]
  float* s_x = reinterpret_cast<float*>(sm4 + R);  // [D][R]
  const uint32_t m = *m_ptr;
  if (gate_m && 4ull * m < *gate_m) {  // few survivors: this pass would not pay
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < m; i += gridDim.x * blockDim.x)
      st[i] = 0;
    return;
  }
  const uint32_t Kp = min(sel[2], r1) > r0 ? min(sel[2], r1) - r0 : 0u;
  for (uint32_t t = threadIdx.x; t < Kp; t += blockDim.x) {
    s_cells[t] = pr_cells[r0 + t];
#pragma unroll
    for (int k = 0; k < D; ++k) s_x[k * R + t] = pr_x[(uint64_t)k * K + r0 + t];
  }
  __syncthreads();
  uint32_t hS[NW];
#pragma unroll
  for (int w = 0; w < NW; ++w) hS[w] = guard_mask(S, w);
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < m; i += gridDim.x * blockDim.x) {
    const uint32_t id = ids ? ids[i] : i;
    const uint4 c4 = cells[id];
    uint32_t pc[NW], pH[NW];
#pragma unroll
    for (int w = 0; w < NW; ++w) {
      pc[w] = word_of(c4, w);
      pH[w] = pc[w] | kGuard;
    }
    float pv[D];
#pragma unroll
    for (int k = 0; k < D; ++k) pv[k] = ((S >> k) & 1u) ? x[(uint64_t)k * n_pad + id] : 0.f;
    bool pruned = false;
    for (uint32_t t = 0; t < Kp && !pruned; ++t) {
      const uint4 q = s_cells[t];
      uint32_t worse = 0;  // guard bits where cell(q) > cell(p)
#pragma unroll
      for (int w = 0; w < NW; ++w) worse |= ~(pH[w] - word_of(q, w)) & hS[w];
      if (worse) continue;
      uint32_t Z = 0;  // attributes of S with equal cells
#pragma unroll
      for (int w = 0; w < NW; ++w)
        Z |= pack_guards(ge_bytes(word_of(q, w) | kGuard, pc[w]) & hS[w]) << (4 * w);
      bool strict = true;
#pragma unroll
      for (int k = 0; k < D; ++k)
        if ((Z >> k) & 1u) strict &= s_x[k * R + t] < pv[k];
      pruned = strict;
    }
    st[i] = pruned ? 2 : 0;
  }
}

size_t prefilter_smem(int d, uint32_t K) {
  return (size_t)K * sizeof(uint4) + (size_t)d * K * sizeof(float);
}

template <int D>
static int launch_prefilter_d(cudaStream_t s, const PrefilterArgs& a, unsigned grid,
                              const uint32_t* ids, const uint32_t* m_ptr, uint32_t r0,
                              uint32_t r1, const uint32_t* gate_m) {
  const size_t smem = prefilter_smem(D, r1 - r0);
  if (smem > 48 * 1024)
    SKC_CUDA(cudaFuncSetAttribute(k_prefilter<D>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)smem));
  k_prefilter<D><<<grid, 256, smem, s>>>(a.cells, a.x, a.n_pad, ids, m_ptr, a.S, a.ps.sel,
                                         a.ps.pr_cells, a.ps.pr_x, a.K, r0, r1, gate_m, a.ps.st);
  SKC_LAUNCH_CHECK();
  return SKC_OK;
}

static int launch_prefilter_pass(cudaStream_t s, int d, const PrefilterArgs& a, unsigned grid,
                                 const uint32_t* ids, const uint32_t* m_ptr, uint32_t r0,
                                 uint32_t r1, const uint32_t* gate_m) {
  switch (d) {
#define SKC_PF_CASE(D) \
  case D: return launch_prefilter_d<D>(s, a, grid, ids, m_ptr, r0, r1, gate_m);
    SKC_PF_CASE(2) SKC_PF_CASE(3) SKC_PF_CASE(4) SKC_PF_CASE(5) SKC_PF_CASE(6)
    SKC_PF_CASE(7) SKC_PF_CASE(8) SKC_PF_CASE(9) SKC_PF_CASE(10) SKC_PF_CASE(11)
    SKC_PF_CASE(12) SKC_PF_CASE(13) SKC_PF_CASE(14) SKC_PF_CASE(15) SKC_PF_CASE(16)
#undef SKC_PF_CASE
    default:
      return set_error(SKC_ERR_INVALID, "unsupported d=%d", d);
  }
}

int launch_prefilter(cudaStream_t s, int d, int num_sms, const PrefilterArgs& a,
                     uint32_t* out_ids, uint32_t* out_count) {
  if (a.K < 1 || a.K > (uint32_t)kMaxPruners)
    return set_error(SKC_ERR_INVALID, "pruner count %u outside [1, %d]", a.K, kMaxPruners);
  const PrefilterScratch& p = a.ps;
  const uint64_t want = (a.m_max + 255) / 256;
  const unsigned grid =
      (unsigned)std::max<uint64_t>(1, std::min<uint64_t>(want, (uint64_t)num_sms * 8));
  SKC_CUDA(cudaMemsetAsync(p.hist, 0, kSumBins * sizeof(uint32_t), s));
  k_pruner_hist<<<grid, 256, 0, s>>>(a.cells, a.ids, a.m_ptr, a.S, d, p.hist);
  SKC_LAUNCH_CHECK();
  k_pruner_select<<<1, 1024, 0, s>>>(p.hist, a.m_ptr, a.K, p.sel);
  SKC_LAUNCH_CHECK();
  k_pruner_collect<<<grid, 256, 0, s>>>(a.cells, a.ids, a.m_ptr, a.S, d, p.sel, p.pr_ids,
                                        p.pr_key);
  SKC_LAUNCH_CHECK();
  k_pruner_order<<<1, 1024, 0, s>>>(p.pr_ids, p.pr_key, p.sel, a.cells, a.x, a.n_pad, d, a.K,
                                    p.pr_cells, p.pr_x);
  SKC_LAUNCH_CHECK();
  // Two passes: the strongest K1 = K / 16 pruners on every entry, then, only
  // when at least a quarter of the entries survived, the other pruners on
  // the survivors. Tie-heavy and correlated data lose nearly everything to
  // the first pass (more pruners only cost there: survivors that nothing can
  // strictly dominate walk every pruner); anticorrelated data keeps most
  // points, and the second pass removes a good part of them.
  const uint32_t K1 = std::max<uint32_t>(1, a.K / 16);
  SKC_TRY(launch_prefilter_pass(s, d, a, grid, a.ids, a.m_ptr, 0, K1, nullptr));
  if (K1 >= a.K) {
    return launch_status_compact(s, p.st, a.ids, a.m_ptr, a.m_max, 1, p.blk0, p.blk1, out_ids,
                                 nullptr, out_count, nullptr);
  }
  SKC_TRY(launch_status_compact(s, p.st, a.ids, a.m_ptr, a.m_max, 1, p.blk0, p.blk1, p.mid_ids,
                                nullptr, p.mid_count, nullptr));
  SKC_TRY(launch_prefilter_pass(s, d, a, grid, p.mid_ids, p.mid_count, K1, a.K, a.m_ptr));
  // Survivors (status 0) in list order, as point ids.
  return launch_status_compact(s, p.st, p.mid_ids, p.mid_count, a.m_max, 1, p.blk0, p.blk1,
                               out_ids, nullptr, out_count, nullptr);
}

uint32_t prefilter_sum_bins() { return kSumBins; }

}  // namespace skc
