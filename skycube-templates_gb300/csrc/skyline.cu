// Skyline and extended skyline of a point list on one subspace S.
//
// Replaces one call of the suite's SkyAlign pipeline (skyalign<dims>,
// src/sdsc/skyAlign.cuh:27-318, with its pruning rounds in
// total_pruning_moved_data_templated_pitch_two_level_full_warps,
// src/utilities/kernels.cuh:36-411): same output sets, different method.
//
// Method. The list is ordered by buckets of the Manhattan norm on S (a
// counting sort, prep.cu). Because the norm is monotone, a point can only be
// dominated by points whose bucket is not after its own, so point p scans the
// prefix [0, hi(p)) of that order. One thread owns one p; the CTA stages the
// grid cells of 256 q's at a time in shared memory and every thread tests its
// p against them:
//   - a q with a larger cell than p on any attribute of S cannot dominate p
//     (one subtract and one mask per 4 attributes, SWAR on the guard bits);
//   - a q with smaller cells on every attribute of S strictly dominates p;
//   - otherwise the exact float32 comparisons decide (q <= p on S and q < p
//     somewhere: dominated; q < p everywhere: strictly dominated).
// A strictly dominated p stops; the CTA stops when every p has stopped or
// passed its range. The heaviest tiles (end of the order) start first.
#include "kernels.cuh"

namespace skc {

template <int D>
__global__ void __launch_bounds__(256) k_skyline(
    const uint32_t* __restrict__ sorted, const uint32_t* __restrict__ hi,
    const uint32_t* __restrict__ ids, const uint4* __restrict__ cells,
    const float* __restrict__ x, uint64_t n_pad,
    const uint32_t* __restrict__ m_ptr, uint32_t S,
    uint8_t* __restrict__ status) {
  constexpr int NW = (D + 3) / 4;
  constexpr int TQ = 256;
  __shared__ uint4 q_cells[TQ];
  __shared__ uint32_t q_ids[TQ];

  const uint32_t m = *m_ptr;
  const uint32_t ntiles = (m + TQ - 1) / TQ;
  if (blockIdx.x >= ntiles) return;
  const uint32_t tile = ntiles - 1 - blockIdx.x;
  const uint32_t i = tile * TQ + threadIdx.x;
  const bool valid = i < m;

  uint32_t hS[NW];
#pragma unroll
  for (int w = 0; w < NW; ++w) hS[w] = guard_mask(S, w);

  uint32_t my_pos = 0, my_hi = 0;
  uint32_t pc[NW], pH[NW];
  float pv[D];
#pragma unroll
  for (int w = 0; w < NW; ++w) pc[w] = pH[w] = 0;
#pragma unroll
  for (int k = 0; k < D; ++k) pv[k] = 0.f;
  if (valid) {
    my_pos = sorted[i];
    my_hi = hi[i];
    const uint32_t id = ids ? ids[my_pos] : my_pos;
    const uint4 c = cells[id];
#pragma unroll
    for (int w = 0; w < NW; ++w) {
      pc[w] = word_of(c, w);
      pH[w] = pc[w] | kGuard;
    }
#pragma unroll
    for (int k = 0; k < D; ++k)
      if (S & (1u << k)) pv[k] = x[(uint64_t)k * n_pad + id];
  }
  const uint32_t last = min(tile * TQ + TQ, m) - 1;
  const uint32_t qlimit = hi[last];  // hi is non-decreasing in sorted order

  uint8_t st = 0;
  bool done = !valid;
  for (uint32_t base = 0; base < qlimit; base += TQ) {
    if (__syncthreads_and(done || my_hi <= base)) break;
    const uint32_t j = base + threadIdx.x;
    if (j < qlimit) {
      const uint32_t pos = sorted[j];
      const uint32_t id = ids ? ids[pos] : pos;
      q_cells[threadIdx.x] = cells[id];
      q_ids[threadIdx.x] = id;
    }
    __syncthreads();
    if (!done && my_hi > base) {
      const uint32_t lim = min((uint32_t)TQ, my_hi - base);
      for (uint32_t t = 0; t < lim; ++t) {
        const uint4 q = q_cells[t];
        uint32_t worse = 0;  // guard bits where cell(q) > cell(p) on S
#pragma unroll
        for (int w = 0; w < NW; ++w) worse |= ~(pH[w] - word_of(q, w)) & hS[w];
        if (worse) continue;
        uint32_t not_less = 0;  // guard bits where cell(q) >= cell(p) on S
#pragma unroll
        for (int w = 0; w < NW; ++w)
          not_less |= ge_bytes(word_of(q, w) | kGuard, pc[w]) & hS[w];
        if (!not_less) {  // smaller cell on every attribute: strict
          st = 2;
          done = true;
          break;
        }
        const uint32_t qid = q_ids[t];
        bool le = true, lt_any = false, lt_all = true;
#pragma unroll
        for (int k = 0; k < D; ++k) {
          if (S & (1u << k)) {
            const float a = x[(uint64_t)k * n_pad + qid];
            le &= (a <= pv[k]);
            lt_any |= (a < pv[k]);
            lt_all &= (a < pv[k]);
          }
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
  if (valid) status[my_pos] = st;
}

int launch_skyline(cudaStream_t s, int d, const SkylineArgs& a) {
  const unsigned grid = (unsigned)((a.m_max + 255) / 256);
  if (grid == 0) return SKC_OK;
#define SKC_SKY_CASE(D)                                                        \
  case D:                                                                      \
    k_skyline<D><<<grid, 256, 0, s>>>(a.sorted, a.hi, a.ids, a.cells, a.x,     \
                                      a.n_pad, a.m_ptr, a.S, a.status);        \
    break;
  switch (d) {
    SKC_SKY_CASE(2) SKC_SKY_CASE(3) SKC_SKY_CASE(4) SKC_SKY_CASE(5)
    SKC_SKY_CASE(6) SKC_SKY_CASE(7) SKC_SKY_CASE(8) SKC_SKY_CASE(9)
    SKC_SKY_CASE(10) SKC_SKY_CASE(11) SKC_SKY_CASE(12) SKC_SKY_CASE(13)
    SKC_SKY_CASE(14) SKC_SKY_CASE(15) SKC_SKY_CASE(16)
    default:
      return set_error(SKC_ERR_INVALID, "unsupported d=%d", d);
  }
#undef SKC_SKY_CASE
  SKC_LAUNCH_CHECK();
  return SKC_OK;
}

}  // namespace skc
