// Data-preparation kernels of the skycube engine: upload into attribute-major
// layout, Manhattan-norm scores and bucket keys, a counting sort by bucket,
// grid pivots and cells, order-preserving compaction and scans.
//
// Every kernel that works on a point list reads the list length from device
// memory (m_ptr), so a whole pipeline can be enqueued, or captured in a CUDA
// graph, before any length is known on the host.
#include <cfloat>
#include <cstdio>

#include "kernels.cuh"

namespace skc {

// --------------------------------------------------------------------------
// Upload: row-major n x d -> attribute-major x[k * n_pad + i]. Counts
// non-finite values into *bad (NaN would break every ordering below).
__global__ void k_rows_to_soa(const float* __restrict__ rows, uint64_t n, int d,
                              uint64_t n_pad, float* __restrict__ x,
                              uint32_t* __restrict__ bad) {
  const uint64_t total = n * (uint64_t)d;
  uint32_t nbad = 0;
  for (uint64_t t = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; t < total;
       t += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t i = t / d;
    const int k = (int)(t - i * d);
    const float v = rows[t];
    nbad += !isfinite(v);
    x[(uint64_t)k * n_pad + i] = v;
  }
  if (nbad) atomicAdd(bad, nbad);
}

__global__ void k_iota(uint32_t* __restrict__ out, uint64_t n) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n;
       i += (uint64_t)gridDim.x * blockDim.x)
    out[i] = (uint32_t)i;
}

// Order-preserving map of a float to uint32 (for atomic min/max).
__device__ __forceinline__ uint32_t f2u_ordered(float f) {
  uint32_t u = __float_as_uint(f);
  return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float u2f_ordered(uint32_t u) {
  return __uint_as_float((u & 0x80000000u) ? (u & 0x7fffffffu) : ~u);
}

// f[i] = sum of the attributes in S of point ids[i], in increasing attribute
// order. Summing in a fixed order makes f monotone: q <= p on S implies
// f(q) <= f(p) (float addition is monotone in each operand).
// minmax[0] / minmax[1] receive the ordered-uint min / max of f.
__global__ void k_score(const float* __restrict__ x, uint64_t n_pad,
                        const uint32_t* __restrict__ ids,
                        const uint32_t* __restrict__ m_ptr, uint32_t S, int d,
                        float* __restrict__ f, uint32_t* __restrict__ minmax) {
  const uint32_t m = *m_ptr;
  uint32_t lo = 0xffffffffu, hi = 0;
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < m;
       i += gridDim.x * blockDim.x) {
    const uint32_t id = ids ? ids[i] : i;
    float s = 0.f;
    for (int k = 0; k < d; ++k)
      if (S & (1u << k)) s += x[(uint64_t)k * n_pad + id];
    f[i] = s;
    const uint32_t u = f2u_ordered(s);
    lo = min(lo, u);
    hi = max(hi, u);
  }
  for (int o = 16; o; o >>= 1) {
    lo = min(lo, __shfl_xor_sync(0xffffffffu, lo, o));
    hi = max(hi, __shfl_xor_sync(0xffffffffu, hi, o));
  }
  if ((threadIdx.x & 31) == 0) {
    atomicMin(&minmax[0], lo);
    atomicMax(&minmax[1], hi);
  }
}

// key = floor((f - fmin) * (K - 1) / (fmax - fmin)), clamped to [0, K-1].
// Each step is monotone in f, so f(q) <= f(p) implies key(q) <= key(p).
__global__ void k_fkeys(const float* __restrict__ f,
                        const uint32_t* __restrict__ m_ptr,
                        const uint32_t* __restrict__ minmax, uint32_t K,
                        uint32_t* __restrict__ keys) {
  const uint32_t m = *m_ptr;
  const float fmin = u2f_ordered(minmax[0]), fmax = u2f_ordered(minmax[1]);
  const float range = fmax - fmin;
  const float scale = (range > 0.f && isfinite(range)) ? (float)(K - 1) / range : 0.f;
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < m;
       i += gridDim.x * blockDim.x) {
    float t = (f[i] - fmin) * scale;
    uint32_t k = t <= 0.f ? 0u : (t >= (float)(K - 1) ? K - 1 : (uint32_t)t);
    keys[i] = k;
  }
}

__global__ void k_hist(const uint32_t* __restrict__ keys,
                       const uint32_t* __restrict__ m_ptr,
                       uint32_t* __restrict__ counts) {
  const uint32_t m = *m_ptr;
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < m;
       i += gridDim.x * blockDim.x)
    atomicAdd(&counts[keys[i]], 1u);
}

// In-place exclusive scan of a[0 .. len) with one CTA of 1024 threads;
// a[len] receives the total. len + 1 entries must be allocated. The array is
// walked in tiles of 4096 (4 consecutive entries per thread, so each warp
// reads and writes 512 contiguous bytes), each tile scanned in the block and
// offset by the running total of the tiles before it.
template <typename T>
__global__ void __launch_bounds__(1024) k_scan_single(T* __restrict__ a,
                                                      uint32_t len) {
  __shared__ T warp_excl[32];
  __shared__ T tile_tot;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  T carry = 0;  // total of the tiles before this one (same in every thread)
  for (uint32_t base = 0; base < len; base += 4096) {
    T v[4];
    T local = 0;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const uint32_t i = base + 4 * threadIdx.x + j;
      v[j] = i < len ? a[i] : T(0);
      local += v[j];
    }
    T incl = local;
    for (int o = 1; o < 32; o <<= 1) {
      const T u = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= o) incl += u;
    }
    if (lane == 31) warp_excl[wid] = incl;  // warp totals for now
    __syncthreads();
    if (wid == 0) {
      const T w = warp_excl[lane];
      T sw = w;
      for (int o = 1; o < 32; o <<= 1) {
        const T u = __shfl_up_sync(0xffffffffu, sw, o);
        if (lane >= o) sw += u;
      }
      warp_excl[lane] = sw - w;
      if (lane == 31) tile_tot = sw;
    }
    __syncthreads();
    T run = carry + warp_excl[wid] + incl - local;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const uint32_t i = base + 4 * threadIdx.x + j;
      if (i < len) a[i] = run;
      run += v[j];
    }
    carry += tile_tot;
    __syncthreads();  // warp_excl and tile_tot are reused by the next tile
  }
  if (threadIdx.x == 0) a[len] = carry;
}

// Scatters item i to its bucket. sorted[pos] = i; hi[pos] = end of i's
// bucket in sorted order. Order inside a bucket is unspecified; every user
// of the order is insensitive to it.
__global__ void k_scatter(const uint32_t* __restrict__ keys,
                          const uint32_t* __restrict__ m_ptr,
                          const uint32_t* __restrict__ offsets,
                          uint32_t* __restrict__ cursor,
                          uint32_t* __restrict__ sorted,
                          uint32_t* __restrict__ hi) {
  const uint32_t m = *m_ptr;
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < m;
       i += gridDim.x * blockDim.x) {
    const uint32_t k = keys[i];
    const uint32_t pos = offsets[k] + atomicAdd(&cursor[k], 1u);
    sorted[pos] = i;
    if (hi) hi[pos] = offsets[k + 1];
  }
}

// --------------------------------------------------------------------------
// Pivots: one CTA per attribute samples up to kPivotSample values of the
// list (evenly strided), sorts them in shared memory and keeps
// 2^depth - 1 evenly spaced order statistics. Any pivot set is correct;
// quantiles only make the cells informative.
constexpr int kPivotSample = 4096;

__global__ void __launch_bounds__(1024) k_pivots(
    const float* __restrict__ x, uint64_t n_pad, const uint32_t* __restrict__ ids,
    const uint32_t* __restrict__ m_ptr, int depth, float* __restrict__ pivots,
    unsigned long long* __restrict__ spread) {
  __shared__ float s[kPivotSample];
  const int k = blockIdx.x;
  if (spread && k == 0 && threadIdx.x < 3) spread[threadIdx.x] = 0;  // k_cells adds to it
  const uint32_t m = *m_ptr;
  const uint32_t cnt = m < kPivotSample ? m : kPivotSample;
  for (int t = threadIdx.x; t < kPivotSample; t += blockDim.x) {
    float v = FLT_MAX;
    if ((uint32_t)t < cnt) {
      const uint32_t i = (uint32_t)(((uint64_t)t * m) / cnt);
      const uint32_t id = ids ? ids[i] : i;
      v = x[(uint64_t)k * n_pad + id];
    }
    s[t] = v;
  }
  __syncthreads();
  // bitonic sort, ascending
  for (int size = 2; size <= kPivotSample; size <<= 1) {
    for (int stride = size >> 1; stride > 0; stride >>= 1) {
      for (int t = threadIdx.x; t < kPivotSample / 2; t += blockDim.x) {
        const int lo = 2 * t - (t & (stride - 1));
        const int hi = lo + stride;
        const bool up = (lo & size) == 0;
        const float a = s[lo], b = s[hi];
        if ((a > b) == up) {
          s[lo] = b;
          s[hi] = a;
        }
      }
      __syncthreads();
    }
  }
  const int P = (1 << depth) - 1;
  for (int r = threadIdx.x; r < kMaxPivots; r += blockDim.x) {
    float v = FLT_MAX;
    if (r < P && cnt > 0) v = s[((uint64_t)(r + 1) * cnt) / (P + 1)];
    pivots[k * kMaxPivots + r] = v;
  }
}

// cells[i] = grid cells of point ids[i] (see common.cuh).
// With `spread`, also the sum and the sum of squares of the points' cell
// sums and their count (k_cell_spread's layout, every attribute).
__global__ void k_cells(const float* __restrict__ x, uint64_t n_pad,
                        const uint32_t* __restrict__ ids,
                        const uint32_t* __restrict__ m_ptr, int d, int depth,
                        const float* __restrict__ pivots,
                        uint4* __restrict__ cells,
                        unsigned long long* __restrict__ spread) {
  __shared__ float piv[kMaxDims * kMaxPivots];
  for (int t = threadIdx.x; t < d * kMaxPivots; t += blockDim.x) piv[t] = pivots[t];
  __syncthreads();
  const uint32_t m = *m_ptr;
  const int P = (1 << depth) - 1;
  unsigned long long s1 = 0, s2 = 0;
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < m;
       i += gridDim.x * blockDim.x) {
    const uint32_t id = ids ? ids[i] : i;
    uint32_t w[4] = {0, 0, 0, 0};
    uint32_t sum = 0;
    for (int k = 0; k < d; ++k) {
      const float v = x[(uint64_t)k * n_pad + id];
      const float* pk = piv + k * kMaxPivots;
      int lo = 0, hi = P;
      while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (pk[mid] < v) lo = mid + 1; else hi = mid;
      }
      w[k >> 2] |= (uint32_t)lo << (8 * (k & 3));
      sum += (uint32_t)lo;
    }
    cells[i] = make_uint4(w[0], w[1], w[2], w[3]);
    s1 += sum;
    s2 += (unsigned long long)sum * sum;
  }
  if (spread) {
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
}

// --------------------------------------------------------------------------
// Order-preserving two-way compaction of a status array: ids of entries
// with status 0 go to out0, with status 1 to out1 (status 2 is dropped).
// Works in blocks of 1024 items: count, scan of block counts, write.
__global__ void __launch_bounds__(1024) k_status_count(
    const uint8_t* __restrict__ st, const uint32_t* __restrict__ m_ptr,
    int merge01, uint32_t* __restrict__ c0, uint32_t* __restrict__ c1) {
  __shared__ uint32_t s0[32], s1[32];
  const uint32_t m = *m_ptr;
  const uint32_t nblk = (m + 1023) / 1024;
  if (blockIdx.x >= nblk) {
    if (threadIdx.x == 0 && blockIdx.x < gridDim.x) { c0[blockIdx.x] = 0; c1[blockIdx.x] = 0; }
    return;
  }
  const uint32_t i = blockIdx.x * 1024 + threadIdx.x;
  uint8_t v = i < m ? st[i] : 2;
  if (merge01 && v == 1) v = 0;
  const uint32_t b0 = __ballot_sync(0xffffffffu, v == 0);
  const uint32_t b1 = __ballot_sync(0xffffffffu, v == 1);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0) { s0[wid] = __popc(b0); s1[wid] = __popc(b1); }
  __syncthreads();
  if (wid == 0) {
    uint32_t a = s0[lane], b = s1[lane];
    for (int o = 16; o; o >>= 1) {
      a += __shfl_xor_sync(0xffffffffu, a, o);
      b += __shfl_xor_sync(0xffffffffu, b, o);
    }
    if (lane == 0) { c0[blockIdx.x] = a; c1[blockIdx.x] = b; }
  }
}

__global__ void __launch_bounds__(1024) k_status_write(
    const uint8_t* __restrict__ st, const uint32_t* __restrict__ ids,
    const uint32_t* __restrict__ m_ptr, int merge01,
    const uint32_t* __restrict__ o0, const uint32_t* __restrict__ o1,
    uint32_t nblk_alloc,
    uint32_t* __restrict__ out0, uint32_t* __restrict__ out1,
    uint32_t* __restrict__ n0, uint32_t* __restrict__ n1) {
  __shared__ uint32_t s0[32], s1[32];
  const uint32_t m = *m_ptr;
  const uint32_t nblk = (m + 1023) / 1024;
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    if (n0) *n0 = o0[nblk_alloc];
    if (n1) *n1 = o1[nblk_alloc];
  }
  if (blockIdx.x >= nblk) return;
  const uint32_t i = blockIdx.x * 1024 + threadIdx.x;
  uint8_t v = i < m ? st[i] : 2;
  if (merge01 && v == 1) v = 0;
  const uint32_t b0 = __ballot_sync(0xffffffffu, v == 0);
  const uint32_t b1 = __ballot_sync(0xffffffffu, v == 1);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0) { s0[wid] = __popc(b0); s1[wid] = __popc(b1); }
  __syncthreads();
  if (wid == 0) {
    uint32_t a = s0[lane], b = s1[lane];
    uint32_t ia = a, ib = b;
    for (int o = 1; o < 32; o <<= 1) {
      uint32_t u = __shfl_up_sync(0xffffffffu, ia, o);
      uint32_t w = __shfl_up_sync(0xffffffffu, ib, o);
      if (lane >= o) { ia += u; ib += w; }
    }
    s0[lane] = ia - a;
    s1[lane] = ib - b;
  }
  __syncthreads();
  const uint32_t lt = (1u << lane) - 1u;
  const uint32_t id = i < m ? (ids ? ids[i] : i) : 0;
  if (v == 0) out0[o0[blockIdx.x] + s0[wid] + __popc(b0 & lt)] = id;
  else if (v == 1 && out1) out1[o1[blockIdx.x] + s1[wid] + __popc(b1 & lt)] = id;
}

// --------------------------------------------------------------------------
// Multi-block exclusive scan of uint32 counts into uint64 offsets:
// out[i] = sum(in[0..i)), out[len] = total. Three phases.
constexpr int kScanBlock = 4096;

__global__ void __launch_bounds__(1024) k_scan_partials(
    const uint32_t* __restrict__ in, uint64_t len, uint64_t* __restrict__ bsum) {
  __shared__ uint64_t red[32];
  const uint64_t beg = (uint64_t)blockIdx.x * kScanBlock;
  uint64_t s = 0;
  for (int t = threadIdx.x; t < kScanBlock; t += 1024) {
    const uint64_t i = beg + t;
    if (i < len) s += in[i];
  }
  for (int o = 16; o; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x < 32) {
    s = red[threadIdx.x];
    for (int o = 16; o; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (threadIdx.x == 0) bsum[blockIdx.x] = s;
  }
}

__global__ void __launch_bounds__(1024) k_scan_apply(
    const uint32_t* __restrict__ in, uint64_t len,
    const uint64_t* __restrict__ bsum_scanned, uint64_t* __restrict__ out) {
  __shared__ uint64_t wt[32];
  const uint64_t beg = (uint64_t)blockIdx.x * kScanBlock;
  constexpr int per = kScanBlock / 1024;  // 4 consecutive items per thread
  uint32_t v[per];
  uint64_t local = 0;
  for (int j = 0; j < per; ++j) {
    const uint64_t i = beg + threadIdx.x * per + j;
    v[j] = i < len ? in[i] : 0;
    local += v[j];
  }
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  uint64_t incl = local;
  for (int o = 1; o < 32; o <<= 1) {
    uint64_t u = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += u;
  }
  if (lane == 31) wt[wid] = incl;
  __syncthreads();
  if (wid == 0) {
    uint64_t a = wt[lane], s = a;
    for (int o = 1; o < 32; o <<= 1) {
      uint64_t u = __shfl_up_sync(0xffffffffu, s, o);
      if (lane >= o) s += u;
    }
    wt[lane] = s - a;
  }
  __syncthreads();
  uint64_t run = bsum_scanned[blockIdx.x] + wt[wid] + incl - local;
  for (int j = 0; j < per; ++j) {
    const uint64_t i = beg + threadIdx.x * per + j;
    if (i < len) out[i] = run;
    run += v[j];
  }
  if (blockIdx.x == gridDim.x - 1 && threadIdx.x == 1023) out[len] = run;
}

// --------------------------------------------------------------------------
// Gathers.
__global__ void k_gather_soa(const float* __restrict__ x, uint64_t n_pad, int d,
                             const uint32_t* __restrict__ ids,
                             const uint32_t* __restrict__ m_ptr,
                             uint64_t out_pad, float* __restrict__ out) {
  const uint32_t m = *m_ptr;
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < m;
       i += gridDim.x * blockDim.x) {
    const uint32_t id = ids[i];
    for (int k = 0; k < d; ++k) out[(uint64_t)k * out_pad + i] = x[(uint64_t)k * n_pad + id];
  }
}

__global__ void k_gather_u4(const uint4* __restrict__ in,
                            const uint32_t* __restrict__ perm,
                            const uint32_t* __restrict__ m_ptr,
                            uint4* __restrict__ out) {
  const uint32_t m = *m_ptr;
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < m;
       i += gridDim.x * blockDim.x)
    out[i] = in[perm[i]];
}

// Per block of 32 consecutive q's, per 8-q quarter and per 4-q half of a
// quarter: byte-wise
// minimum of their cells. Padding entries (index >= m) get cell 127 so they
// never lower the minimum.
__global__ void k_block_min(const uint4* __restrict__ cells,
                            const uint32_t* __restrict__ m_ptr,
                            uint4* __restrict__ bmin, uint4* __restrict__ smin,
                            uint4* __restrict__ hmin) {
  const uint32_t m = *m_ptr;
  const uint32_t nblk = (m + 31) / 32;
  const int lane = threadIdx.x & 31;
  for (uint32_t b = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; b < nblk;
       b += (gridDim.x * blockDim.x) >> 5) {
    const uint32_t i = b * 32 + lane;
    uint4 c = i < m ? cells[i] : make_uint4(0x7f7f7f7fu, 0x7f7f7f7fu, 0x7f7f7f7fu, 0x7f7f7f7fu);
    for (int o = 1; o < 32; o <<= 1) {
      c.x = __vminu4(c.x, __shfl_xor_sync(0xffffffffu, c.x, o));
      c.y = __vminu4(c.y, __shfl_xor_sync(0xffffffffu, c.y, o));
      c.z = __vminu4(c.z, __shfl_xor_sync(0xffffffffu, c.z, o));
      c.w = __vminu4(c.w, __shfl_xor_sync(0xffffffffu, c.w, o));
      if (o == 2 && (lane & 3) == 0) hmin[(uint64_t)b * 8 + (lane >> 2)] = c;
      if (o == 4 && (lane & 7) == 0) smin[(uint64_t)b * 4 + (lane >> 3)] = c;
    }
    if (lane == 0) bmin[b] = c;
  }
}

// Copies one cuboid's list into a CSR slot: used to assemble per-cuboid
// outputs of the per-cuboid form into one cuboid-indexed CSR.
__global__ void k_csr_assemble(const uint32_t* __restrict__ src,
                               const uint64_t* __restrict__ src_off,
                               const uint64_t* __restrict__ dst_off,
                               uint32_t* __restrict__ dst) {
  const uint32_t c = blockIdx.x;
  const uint64_t n = dst_off[c + 1] - dst_off[c];
  const uint64_t s = src_off[c], o = dst_off[c];
  for (uint64_t i = threadIdx.x; i < n; i += blockDim.x) dst[o + i] = src[s + i];
}

// Gathers per-cuboid lists held in separate buffers into one CSR:
// cuboid c's list srcs[c] goes to dst[dst_off[c] .. dst_off[c+1]).
__global__ void k_csr_gather(const uint32_t* const* __restrict__ srcs,
                             const uint64_t* __restrict__ dst_off,
                             uint32_t* __restrict__ dst) {
  const uint32_t c = blockIdx.x;
  const uint32_t* src = srcs[c];
  const uint64_t n = dst_off[c + 1] - dst_off[c];
  if (!src) return;
  const uint64_t o = dst_off[c];
  for (uint64_t i = threadIdx.x; i < n; i += blockDim.x) dst[o + i] = src[i];
}

__global__ void k_set_u32(uint32_t* p, uint32_t v) { *p = v; }

// Merges two ascending, disjoint id lists a[0..na) and b[0..nb) into
// out[0..na+nb) (ascending): every element finds its rank in the other list
// by binary search.
__global__ void k_merge_disjoint(const uint32_t* __restrict__ a, uint32_t na,
                                 const uint32_t* __restrict__ b, uint32_t nb,
                                 uint32_t* __restrict__ out) {
  const uint32_t total = na + nb;
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < total;
       i += gridDim.x * blockDim.x) {
    const bool from_a = i < na;
    const uint32_t v = from_a ? a[i] : b[i - na];
    const uint32_t* o = from_a ? b : a;
    uint32_t lo = 0, hi = from_a ? nb : na;
    while (lo < hi) {
      const uint32_t mid = (lo + hi) >> 1;
      if (o[mid] < v) lo = mid + 1; else hi = mid;
    }
    out[(from_a ? i : i - na) + lo] = v;
  }
}

__global__ void k_gather_u32(const uint32_t* __restrict__ in,
                             const uint32_t* __restrict__ perm,
                             const uint32_t* __restrict__ m_ptr,
                             uint32_t* __restrict__ out) {
  const uint32_t m = *m_ptr;
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < m;
       i += gridDim.x * blockDim.x)
    out[i] = in[perm[i]];
}

// ==========================================================================
// Host-side launch helpers.
static inline unsigned grid_for(uint64_t items, int threads, int max_blocks) {
  uint64_t b = (items + threads - 1) / threads;
  if (b < 1) b = 1;
  if (b > (uint64_t)max_blocks) b = max_blocks;
  return (unsigned)b;
}

int launch_rows_to_soa(cudaStream_t s, const float* rows, uint64_t n, int d,
                       uint64_t n_pad, float* x, uint32_t* bad) {
  k_rows_to_soa<<<grid_for(n * d, 256, 152 * 32), 256, 0, s>>>(rows, n, d, n_pad, x, bad);
  SKC_LAUNCH_CHECK();
  return SKC_OK;
}

int launch_iota(cudaStream_t s, uint32_t* out, uint64_t n) {
  k_iota<<<grid_for(n, 256, 152 * 16), 256, 0, s>>>(out, n);
  SKC_LAUNCH_CHECK();
  return SKC_OK;
}

int launch_bucket_order(cudaStream_t s, const float* x, uint64_t n_pad, int d,
                        const uint32_t* ids, const uint32_t* m_ptr,
                        uint64_t m_max, uint32_t S, uint32_t K,
                        const BucketScratch& b, uint32_t* sorted, uint32_t* hi) {
  SKC_CUDA(cudaMemsetAsync(b.minmax, 0, 2 * sizeof(uint32_t), s));
  SKC_CUDA(cudaMemsetAsync(b.minmax, 0xff, sizeof(uint32_t), s));
  const unsigned g = grid_for(m_max, 256, 152 * 8);
  k_score<<<g, 256, 0, s>>>(x, n_pad, ids, m_ptr, S, d, b.f, b.minmax);
  SKC_LAUNCH_CHECK();
  k_fkeys<<<g, 256, 0, s>>>(b.f, m_ptr, b.minmax, K, b.keys);
  SKC_LAUNCH_CHECK();
  return launch_counting_sort(s, b.keys, m_ptr, m_max, K, b, sorted, hi);
}

int launch_counting_sort(cudaStream_t s, const uint32_t* keys,
                         const uint32_t* m_ptr, uint64_t m_max, uint32_t K,
                         const BucketScratch& b, uint32_t* sorted, uint32_t* hi) {
  SKC_CUDA(cudaMemsetAsync(b.counts, 0, (K + 1) * sizeof(uint32_t), s));
  SKC_CUDA(cudaMemsetAsync(b.cursor, 0, (K + 1) * sizeof(uint32_t), s));
  const unsigned g = grid_for(m_max, 256, 152 * 8);
  k_hist<<<g, 256, 0, s>>>(keys, m_ptr, b.counts);
  SKC_LAUNCH_CHECK();
  k_scan_single<uint32_t><<<1, 1024, 0, s>>>(b.counts, K);
  SKC_LAUNCH_CHECK();
  k_scatter<<<g, 256, 0, s>>>(keys, m_ptr, b.counts, b.cursor, sorted, hi);
  SKC_LAUNCH_CHECK();
  return SKC_OK;
}

int launch_pivots_cells(cudaStream_t s, const float* x, uint64_t n_pad, int d,
                        const uint32_t* ids, const uint32_t* m_ptr,
                        uint64_t m_max, int depth, float* pivots, uint4* cells,
                        unsigned long long* spread) {
  k_pivots<<<d, 1024, 0, s>>>(x, n_pad, ids, m_ptr, depth, pivots, spread);
  SKC_LAUNCH_CHECK();
  k_cells<<<grid_for(m_max, 256, 152 * 8), 256, 0, s>>>(x, n_pad, ids, m_ptr, d, depth, pivots,
                                                         cells, spread);
  SKC_LAUNCH_CHECK();
  return SKC_OK;
}

int launch_status_compact(cudaStream_t s, const uint8_t* st, const uint32_t* ids,
                          const uint32_t* m_ptr, uint64_t m_max, int merge01,
                          uint32_t* blk0, uint32_t* blk1, uint32_t* out0,
                          uint32_t* out1, uint32_t* n0, uint32_t* n1) {
  const uint32_t nblk = (uint32_t)((m_max + 1023) / 1024);
  const uint32_t g = nblk ? nblk : 1;
  k_status_count<<<g, 1024, 0, s>>>(st, m_ptr, merge01, blk0, blk1);
  SKC_LAUNCH_CHECK();
  k_scan_single<uint32_t><<<1, 1024, 0, s>>>(blk0, g);
  SKC_LAUNCH_CHECK();
  k_scan_single<uint32_t><<<1, 1024, 0, s>>>(blk1, g);
  SKC_LAUNCH_CHECK();
  k_status_write<<<g, 1024, 0, s>>>(st, ids, m_ptr, merge01, blk0, blk1, g, out0, out1, n0, n1);
  SKC_LAUNCH_CHECK();
  return SKC_OK;
}

int launch_scan_u32_to_u64(cudaStream_t s, const uint32_t* in, uint64_t len,
                           uint64_t* bsum, uint64_t* out) {
  const uint32_t nb = (uint32_t)((len + kScanBlock - 1) / kScanBlock);
  const uint32_t g = nb ? nb : 1;
  k_scan_partials<<<g, 1024, 0, s>>>(in, len, bsum);
  SKC_LAUNCH_CHECK();
  k_scan_single<uint64_t><<<1, 1024, 0, s>>>(bsum, g);
  SKC_LAUNCH_CHECK();
  k_scan_apply<<<g, 1024, 0, s>>>(in, len, bsum, out);
  SKC_LAUNCH_CHECK();
  return SKC_OK;
}

int launch_scan_single_u32(cudaStream_t s, uint32_t* a, uint32_t len) {
  k_scan_single<uint32_t><<<1, 1024, 0, s>>>(a, len);
  SKC_LAUNCH_CHECK();
  return SKC_OK;
}

uint64_t scan_bsum_entries(uint64_t len) {
  return (len + kScanBlock - 1) / kScanBlock + 1;
}

int launch_gather_soa(cudaStream_t s, const float* x, uint64_t n_pad, int d,
                      const uint32_t* ids, const uint32_t* m_ptr, uint64_t m_max,
                      uint64_t out_pad, float* out) {
  k_gather_soa<<<grid_for(m_max, 256, 152 * 8), 256, 0, s>>>(x, n_pad, d, ids, m_ptr, out_pad, out);
  SKC_LAUNCH_CHECK();
  return SKC_OK;
}

int launch_gather_u4(cudaStream_t s, const uint4* in, const uint32_t* perm,
                     const uint32_t* m_ptr, uint64_t m_max, uint4* out) {
  k_gather_u4<<<grid_for(m_max, 256, 152 * 8), 256, 0, s>>>(in, perm, m_ptr, out);
  SKC_LAUNCH_CHECK();
  return SKC_OK;
}

int launch_block_min(cudaStream_t s, const uint4* cells, const uint32_t* m_ptr,
                     uint64_t m_max, uint4* bmin, uint4* smin, uint4* hmin) {
  k_block_min<<<grid_for(m_max, 256, 152 * 8), 256, 0, s>>>(cells, m_ptr, bmin, smin, hmin);
  SKC_LAUNCH_CHECK();
  return SKC_OK;
}

int launch_csr_assemble(cudaStream_t s, const uint32_t* src,
                        const uint64_t* src_off, const uint64_t* dst_off,
                        uint32_t ncub, uint32_t* dst) {
  if (ncub == 0) return SKC_OK;
  k_csr_assemble<<<ncub, 256, 0, s>>>(src, src_off, dst_off, dst);
  SKC_LAUNCH_CHECK();
  return SKC_OK;
}

int launch_csr_gather(cudaStream_t s, const uint32_t* const* srcs,
                      const uint64_t* dst_off, uint32_t ncub, uint32_t* dst) {
  if (ncub == 0) return SKC_OK;
  k_csr_gather<<<ncub, 256, 0, s>>>(srcs, dst_off, dst);
  SKC_LAUNCH_CHECK();
  return SKC_OK;
}

int launch_merge_disjoint(cudaStream_t s, const uint32_t* a, uint32_t na,
                          const uint32_t* b, uint32_t nb, uint32_t* out) {
  if (na + nb == 0) return SKC_OK;
  k_merge_disjoint<<<grid_for((uint64_t)na + nb, 256, 152 * 8), 256, 0, s>>>(a, na, b, nb, out);
  SKC_LAUNCH_CHECK();
  return SKC_OK;
}

int launch_set_u32(cudaStream_t s, uint32_t* p, uint32_t v) {
  k_set_u32<<<1, 1, 0, s>>>(p, v);
  SKC_LAUNCH_CHECK();
  return SKC_OK;
}

int launch_gather_u32(cudaStream_t s, const uint32_t* in, const uint32_t* perm,
                      const uint32_t* m_ptr, uint64_t m_max, uint32_t* out) {
  k_gather_u32<<<grid_for(m_max, 256, 152 * 8), 256, 0, s>>>(in, perm, m_ptr, out);
  SKC_LAUNCH_CHECK();
  return SKC_OK;
}

// Distribution signature of a dataset from a strided sample of up to
// kSignatureSamples points: out[0] = sample points on the sample's own
// full-space skyline, out[1] = sample points that share an attribute value
// with another sample point, out[2] = sample size. It keys the autotuner's
// table (correlated, independent and anticorrelated data differ by orders
// of magnitude in the first; tie-heavy data shows in the second).
constexpr uint32_t kSignatureSamples = 512;

__global__ void __launch_bounds__(kSignatureSamples) k_sample_signature(
    const float* __restrict__ x, uint64_t n_pad, uint64_t n, int d,
    uint32_t* __restrict__ out) {
  __shared__ float xs[kMaxDims][kSignatureSamples];
  __shared__ uint32_t cnt[2];
  const uint32_t ns = (uint32_t)(n < kSignatureSamples ? n : kSignatureSamples);
  const uint32_t t = threadIdx.x;
  if (t < 2) cnt[t] = 0;
  if (t < ns) {
    const uint64_t id = (uint64_t)t * n / ns;
    for (int k = 0; k < d; ++k) xs[k][t] = x[(uint64_t)k * n_pad + id];
  }
  __syncthreads();
  if (t < ns) {
    bool dominated = false, tied = false;
    for (uint32_t j = 0; j < ns; ++j) {
      if (j == t) continue;
      bool le = true, lt = false;
      for (int k = 0; k < d; ++k) {
        const float a = xs[k][j], b = xs[k][t];
        le &= a <= b;
        lt |= a < b;
        tied |= a == b;
      }
      dominated |= le && lt;
    }
    if (!dominated) atomicAdd(&cnt[0], 1u);
    if (tied) atomicAdd(&cnt[1], 1u);
  }
  __syncthreads();
  if (t == 0) {
    out[0] = cnt[0];
    out[1] = cnt[1];
    out[2] = ns;
  }
}

int launch_sample_signature(cudaStream_t s, const float* x, uint64_t n_pad, uint64_t n, int d,
                            uint32_t* out) {
  if (d < 1 || d > kMaxDims) return set_error(SKC_ERR_INVALID, "unsupported d=%d", d);
  k_sample_signature<<<1, kSignatureSamples, 0, s>>>(x, n_pad, n, d, out);
  SKC_LAUNCH_CHECK();
  return SKC_OK;
}

// Plan helpers (graph-captured launch sequences, api.cu). k_cap_count
// records the true list length in stats[slot] and clamps the device count to
// the plan's capacity, so every later kernel stays inside the buffers; the
// host sees the overflow and re-plans. k_stat_u64 copies one device total.
__global__ void k_cap_count(uint32_t* m_ptr, uint32_t cap, uint64_t* stats, int slot) {
  const uint32_t m = *m_ptr;
  stats[slot] = m;
  if (m > cap) *m_ptr = cap;
}

__global__ void k_stat_u64(const uint64_t* src, uint64_t* stats, int slot) {
  stats[slot] = *src;
}

int launch_cap_count(cudaStream_t s, uint32_t* m_ptr, uint32_t cap, uint64_t* stats, int slot) {
  k_cap_count<<<1, 1, 0, s>>>(m_ptr, cap, stats, slot);
  SKC_LAUNCH_CHECK();
  return SKC_OK;
}

int launch_stat_u64(cudaStream_t s, const uint64_t* src, uint64_t* stats, int slot) {
  k_stat_u64<<<1, 1, 0, s>>>(src, stats, slot);
  SKC_LAUNCH_CHECK();
  return SKC_OK;
}

// st[i] = 0 when list[i] occurs in sorted_set[0 .. *nset_ptr) (ascending),
// else 2: status-compaction input that keeps the members.
__global__ void k_member_flags(const uint32_t* __restrict__ list,
                               const uint32_t* __restrict__ m_ptr,
                               const uint32_t* __restrict__ sorted_set,
                               const uint32_t* __restrict__ nset_ptr,
                               uint8_t* __restrict__ st) {
  const uint32_t m = *m_ptr, ns = *nset_ptr;
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < m; i += gridDim.x * blockDim.x) {
    const uint32_t v = list[i];
    uint32_t lo = 0, hi = ns;  // first position with sorted_set[pos] >= v
    while (lo < hi) {
      const uint32_t mid = (lo + hi) >> 1;
      if (sorted_set[mid] < v) lo = mid + 1; else hi = mid;
    }
    st[i] = (lo < ns && sorted_set[lo] == v) ? 0 : 2;
  }
}

int launch_member_flags(cudaStream_t s, const uint32_t* list, const uint32_t* m_ptr,
                        uint64_t m_max, const uint32_t* sorted_set, const uint32_t* nset_ptr,
                        uint8_t* st) {
  k_member_flags<<<grid_for(m_max, 256, 152 * 8), 256, 0, s>>>(list, m_ptr, sorted_set, nset_ptr, st);
  SKC_LAUNCH_CHECK();
  return SKC_OK;
}

// Pads the q list to a whole number of 32-q blocks with entries that add
// nothing, so the bitmap kernel can test every lane of a block without a
// bounds check: cells 127 (the top cell) and floats +inf. Such a q is worse
// than p on every attribute where p's cell is below 127, and where p's cell
// is 127 too the float test +inf <= p fails (inputs are finite), so LE = LT
// = {} for every p: no strict update and no tie pair.
__global__ void k_pad_q(const uint32_t* __restrict__ mq_ptr, int d, uint4* __restrict__ qc,
                        float* __restrict__ qx, uint64_t pitch) {
  const uint32_t mq = *mq_ptr;
  const uint32_t i = mq + threadIdx.x;
  if (i >= ((mq + 31) & ~31u)) return;
  qc[i] = make_uint4(0x7f7f7f7fu, 0x7f7f7f7fu, 0x7f7f7f7fu, 0x7f7f7f7fu);
  for (int k = 0; k < d; ++k) qx[(uint64_t)k * pitch + i] = __int_as_float(0x7f800000);
}

int launch_pad_q(cudaStream_t s, const uint32_t* mq_ptr, int d, uint4* qc, float* qx,
                 uint64_t pitch) {
  k_pad_q<<<1, 32, 0, s>>>(mq_ptr, d, qc, qx, pitch);
  SKC_LAUNCH_CHECK();
  return SKC_OK;
}

}  // namespace skc
