// Per-point dominated-subspace bitmaps over the candidate set (the MDMC
// computation of the suite: produce_bitmap_iterative_multi_partition_
// templated_async, src/utilities/kernels.cuh:415-908, driven by
// tombstoning_hearting_gpu, src/mdmc/MDMC.cu:752-857), and their compaction
// into per-cuboid id lists (HashCube decode, src/utilities/utilities.h:
// 253-267, done on the device).
//
// For a point p and another point q let LE = {k : q[k] <= p[k]} and
// LT = {k : q[k] < p[k]}. q dominates p exactly on the subspaces S with
// S subset of LE and S meeting LT, and strictly dominates p on the non-empty
// subsets of LT. Two bitmaps over all 2^d subspaces are kept per p:
//   STRICT = union over q of down(LT)      (down-closed)
//   TIE    = union over q with LE != LT of {S subset of LE, S not subset of
//            EQ}, EQ = LE \ LT            (only exact float ties feed it)
// Then p is dominated on S iff S in STRICT or TIE, and p is in the extended
// skyline of S iff S in TIE and not in STRICT.
//
// Pruning. Grid cells (common.cuh) give, without touching floats, the set U
// of attributes where q may be <= p (LE subset of U). If U is in STRICT, the
// down-closure of U is already strict and q adds nothing. The same test on
// the byte-wise minimum cells of a block of 32 consecutive q's skips the
// whole block (the box's U is the union of its q's U's); an open block's
// four 8-q quarters and an open quarter's two 4-q halves are box-tested the
// same way before their q's are walked (1M x 10 anticorrelated: 89 % of the
// 32-q blocks that passed their box test held no q that added anything,
// while 79 % of their 8-q quarter boxes were already strict). q's are ordered
// by the lattice level of their median mask so STRICT fills early.
//
// Mapping. One warp owns one p at a time (a persistent grid pulls p's from a
// device counter) and its 32 lanes test 32 q's per step. For d <= 10 the
// 2^d-bit STRICT and TIE bitmaps live in registers, one 32-bit word per lane
// (word w in lane w); a membership test is one shuffle. For d >= 11 they
// live in shared memory, one pair per warp. A new (LE, LT) pair is applied
// word-parallel: word w of down(L) is submask(L & 31) if w is a subset of
// L >> 5, else empty.
#include "kernels.cuh"

#ifndef SKC_BITMAP_COUNTERS
#define SKC_BITMAP_COUNTERS 0
#endif

namespace skc {

// c_submask[x] = bit b set iff b is a subset of x (5-bit masks).
__constant__ uint32_t c_submask[32];
// c_popabove[c] = bit b set iff b has more than c set bits (c = 0 .. 4).
__constant__ uint32_t c_popabove[5];

void upload_submask_table() {
  uint32_t t[32];
  for (uint32_t x = 0; x < 32; ++x) {
    uint32_t m = 0;
    for (uint32_t b = 0; b < 32; ++b)
      if ((b & ~x) == 0) m |= 1u << b;
    t[x] = m;
  }
  cudaMemcpyToSymbol(c_submask, t, sizeof(t));
  uint32_t a[5];
  for (int c = 0; c < 5; ++c) {
    uint32_t m = 0;
    for (uint32_t b = 0; b < 32; ++b)
      if (__builtin_popcount(b) > c) m |= 1u << b;
    a[c] = m;
  }
  cudaMemcpyToSymbol(c_popabove, a, sizeof(a));
}

constexpr uint32_t kFull = 0xffffffffu;

// Work counters of the bitmap kernel, compiled only into the counters build
// (SKC_BITMAP_COUNTERS=1, skycube_gb300.build(counters=True)); the normal
// build has none of this code. Per launch, summed over candidates:
// [0] candidates, [1] partition ballots, [2] partitions visited, [3] box-test
// steps, [4] block boxes tested, [5] walk steps (32 q's), [6] walk steps whose
// q's were all covered already, [7] STRICT updates, [8] tie pairs, [9] q's
// tested that were not covered, [10] 8-q sub-boxes tested, [11] sub-blocks
// opened; SM cycles (clock64, per warp, summed) spent in [12] partition
// ballots, [13] box tests, [14] quarter- and half-box tests, [15] walks,
// [16] the whole candidate and [17] its output; [18] 4-q half boxes tested,
// [19] halves opened.
[[maybe_unused]] constexpr int kBitmapCounters = 20;
#if SKC_BITMAP_COUNTERS
__device__ unsigned long long g_bitmap_counters[kBitmapCounters];
#define SKC_COUNT(i, v) (cnt_[i] += (v))
#define SKC_T0(v) const long long v = clock64()
#define SKC_TADD(i, v) (cnt_[i] += (unsigned long long)(clock64() - (v)))
// Adds the cycles from its construction to the end of its scope.
struct CycleScope {
  unsigned long long* acc;
  long long t0 = 0;
  __device__ explicit CycleScope(unsigned long long* a) : acc(a) {
#ifdef __CUDA_ARCH__
    t0 = clock64();
#endif
  }
  __device__ ~CycleScope() {
#ifdef __CUDA_ARCH__
    *acc += (unsigned long long)(clock64() - t0);
#endif
  }
};
#define SKC_SCOPE(name, i) CycleScope name(&cnt_[i])
#else
#define SKC_COUNT(i, v) ((void)0)
#define SKC_T0(v) ((void)0)
#define SKC_TADD(i, v) ((void)0)
#define SKC_SCOPE(name, i) ((void)0)
#endif

template <int D>
struct BitState {
  static constexpr uint32_t NSUB = 1u << D;
  static constexpr uint32_t W = NSUB >= 32 ? NSUB / 32 : 1;  // bitmap words
  static constexpr bool REG = (W <= 32);   // STRICT in registers
  static constexpr uint32_t AW = NSUB / 2;  // tie-map words (2 entries each)
  static constexpr bool A_SMEM = (D <= 12);  // tie map in shared memory
  // Above, the map lives in a global slab and is closed chunk by chunk
  // through a 512-word shared scratch (tie_global_output).
  static constexpr uint32_t CHUNK_WORDS = A_SMEM ? 0 : 512;
  // Also above: the first LIST_WORDS tie pairs of a candidate are kept as a
  // list (E | L << 16) and applied directly when no more come; the global
  // map is used only when a candidate has more.
  static constexpr uint32_t LIST_WORDS = A_SMEM ? 0 : 32;
  // The walk's queues, last: open blocks (up to 7 waiting + 32 from a
  // box-test step), open 8-q quarters (up to 15 + 32 from a quarter step)
  // and open 4-q halves (up to 7 + 32 from a half step).
  static constexpr uint32_t BQ_WORDS = 40, WQ_WORDS = 48, HQ_WORDS = 40;
  static constexpr uint32_t WALK_WORDS = BQ_WORDS + WQ_WORDS + HQ_WORDS;
  // shared memory per warp, in words
  static constexpr uint32_t SMEM_WORDS =
      (REG ? 0 : W) + (A_SMEM ? AW : 0) + CHUNK_WORDS + LIST_WORDS + WALK_WORDS;
};

// Splits the subsets of h over 32 lanes: `low` = the lowest five set bits of
// h, `rest` = the others. Lane j < 2^popc(low) gets base = the j-th subset
// of low and walks every subset of rest; other lanes get nothing (false).
__device__ __forceinline__ uint32_t pdep_bits(uint32_t t, uint32_t mask) {
  uint32_t w = 0;
  while (mask) {
    const uint32_t low = mask & (0u - mask);
    if (t & 1u) w |= low;
    t >>= 1;
    mask &= mask - 1;
  }
  return w;
}

__device__ __forceinline__ bool split_words(uint32_t h, int lane, uint32_t* base,
                                            uint32_t* rest) {
  uint32_t low = 0, t = h;
#pragma unroll
  for (int j = 0; j < 5; ++j) {
    low |= t & (0u - t);
    t &= t - 1;
  }
  if ((uint32_t)lane >= (1u << __popc(low))) return false;
  *base = pdep_bits((uint32_t)lane, low);
  *rest = h ^ low;
  return true;
}

// Tie map. A pair whose LE differs from LT (an exact float tie on some
// attribute) dominates p on {S subset of LE : S meets LT}. Instead of
// applying each such set, the warp keeps A[E] = union of LT over its tie
// pairs with LE == E (16-bit entries, two per word). At the end one
// superset-OR pass gives T[S] = union of A[E] over E containing S, and p is
// dominated through ties on S exactly when S meets T[S].
template <int D>
__device__ void tie_closure(uint32_t* A, int lane) {
  constexpr uint32_t AW = BitState<D>::AW;
  for (uint32_t w = lane; w < AW; w += 32) {  // attribute 0: inside a word
    const uint32_t x = A[w];
    A[w] = x | (x >> 16);
  }
  __syncwarp();
  for (int j = 1; j < D; ++j) {  // attribute j: words w and w + 2^(j-1)
    const uint32_t st = 1u << (j - 1);
    for (uint32_t t = lane; t < AW / 2; t += 32) {
      const uint32_t w = ((t >> (j - 1)) << j) | (t & (st - 1));
      A[w] |= A[w + st];
    }
    __syncwarp();
  }
}

// The same closure for a map in the global slab (d >= 13), blocked so that
// a warp makes tens of memory round trips per candidate instead of one per
// pass and word. Entries are grouped in chunks of 1024 (512 words): entry
// bits 0..9 lie inside a chunk, bits 10..d-1 index the chunk.
//
// Phase 1: the chunk-index bits, in groups of up to four. For one group a
// lane holds, in registers, the same word of the 2^GB chunks that differ
// only in the group's bits (coalesced over the warp: word 32i + lane), ORs
// each into its subsets (a butterfly), and stores them back.
template <int GB>
__device__ __forceinline__ void closure_chunk_bits(uint32_t* A, int lane, int g0, uint32_t nc) {
  constexpr uint32_t NX = 1u << GB;
  const uint32_t gmask = (NX - 1) << g0;
  for (uint32_t base = 0; base < nc; ++base) {
    if (base & gmask) continue;
    for (uint32_t i = 0; i < 16; ++i) {
      uint32_t v[NX];
#pragma unroll
      for (uint32_t x = 0; x < NX; ++x) v[x] = A[((base | (x << g0)) << 9) + 32 * i + lane];
#pragma unroll
      for (int bit = 0; bit < GB; ++bit)
#pragma unroll
        for (uint32_t x = 0; x < NX; ++x)
          if (!(x & (1u << bit))) v[x] |= v[x | (1u << bit)];
#pragma unroll
      for (uint32_t x = 0; x < NX; ++x) A[((base | (x << g0)) << 9) + 32 * i + lane] = v[x];
    }
  }
}

// Spreads the 16 bits of x to the even bit positions.
__device__ __forceinline__ uint32_t spread_even(uint32_t x) {
  x = (x | (x << 8)) & 0x00ff00ffu;
  x = (x | (x << 4)) & 0x0f0f0f0fu;
  x = (x | (x << 2)) & 0x33333333u;
  x = (x | (x << 1)) & 0x55555555u;
  return x;
}

// Output word t with the full-space bit (word W - 1) replaced, capped mode.
struct FullFix {
  uint32_t word = 0xffffffffu;  // no word
  uint32_t set = 0, clr = 0;
  __device__ __forceinline__ void apply(uint32_t t, uint32_t& dom, uint32_t& ext) const {
    if (t == word) {
      dom = (dom & ~clr) | set;
      ext = (ext & ~clr) | set;
    }
  }
};

// Phase 2, per chunk: load it into the scratch Cs, close its ten low entry
// bits there, and turn it straight into the chunk's 32 output words (entry
// S is tie-dominated iff S meets T[S]): word j of the chunk gives the bits
// of entries 2j and 2j+1, two ballots over j = 32i + lane give output words
// 2i (lanes 0..15) and 2i+1 (lanes 16..31) after an even/odd interleave.
// Lane l ends with output word 32c + l and writes dom and ext for it.
template <int D>
__device__ void tie_global_output(uint32_t* A, uint32_t* Cs, const uint32_t* sat_s, int lane,
                                  uint32_t p, uint32_t* __restrict__ out_dom,
                                  uint32_t* __restrict__ out_ext, const FullFix& fix) {
  constexpr int HB = D - 10;
  constexpr uint32_t NC = 1u << HB;
  constexpr uint32_t W = (1u << D) / 32;
  closure_chunk_bits<(HB < 4 ? HB : 4)>(A, lane, 0, NC);
  if constexpr (HB > 4) closure_chunk_bits<HB - 4>(A, lane, 4, NC);
  __syncwarp();
  for (uint32_t c = 0; c < NC; ++c) {
#pragma unroll
    for (uint32_t k = 0; k < 16; ++k) {
      const uint32_t x = A[(c << 9) + 32 * k + lane];
      Cs[32 * k + lane] = x | (x >> 16);  // entry bit 0 (inside the word)
    }
    __syncwarp();
    for (int j = 1; j <= 9; ++j) {  // entry bit j: words w and w + 2^(j-1)
      const uint32_t st = 1u << (j - 1);
#pragma unroll
      for (uint32_t t = lane; t < 256; t += 32) {
        const uint32_t w = ((t >> (j - 1)) << j) | (t & (st - 1));
        Cs[w] |= Cs[w + st];
      }
      __syncwarp();
    }
    uint32_t mine = 0;
#pragma unroll
    for (uint32_t i = 0; i < 16; ++i) {
      const uint32_t j = 32 * i + lane;
      const uint32_t x = Cs[j];
      const uint32_t e0 = (c << 10) + 2 * j;
      const uint32_t ev = __ballot_sync(kFull, (e0 & x & 0xffffu) != 0u);
      const uint32_t od = __ballot_sync(kFull, ((e0 + 1) & (x >> 16)) != 0u);
      const uint32_t lo = spread_even(ev & 0xffffu) | (spread_even(od & 0xffffu) << 1);
      const uint32_t hi = spread_even(ev >> 16) | (spread_even(od >> 16) << 1);
      if ((uint32_t)lane == 2 * i) mine = lo;
      if ((uint32_t)lane == 2 * i + 1) mine = hi;
    }
    const uint32_t t = 32 * c + lane;
    const uint32_t s_ = sat_s[t];
    uint32_t dom = s_ | mine, ext = mine & ~s_;
    if (t == 0) {
      dom &= ~1u;
      ext &= ~1u;
    }
    fix.apply(t, dom, ext);
    out_dom[(uint64_t)p * W + t] = dom;
    if (out_ext) out_ext[(uint64_t)p * W + t] = ext;
    __syncwarp();  // Cs is reused by the next chunk
  }
}

// Word t of the tie-dominated bitmap: bit b set iff S = 32t + b meets T[S].
template <int D>
__device__ __forceinline__ uint32_t tie_word(const uint32_t* A, uint32_t t) {
  constexpr uint32_t NSUB = BitState<D>::NSUB;
  uint32_t bits = 0;
  const uint32_t nb = NSUB < 32 ? NSUB : 32;
  for (uint32_t b = 0; b < nb; b += 2) {
    const uint32_t S = 32 * t + b;
    const uint32_t x = A[S >> 1];
    if (S & (x & 0xffffu)) bits |= 1u << b;
    if ((S + 1) & (x >> 16)) bits |= 2u << b;
  }
  return bits;
}

// Capped skycubes (only cuboids of at most `cap` attributes and the full
// space are output). A q whose U has every subspace of at most `cap`
// attributes in STRICT changes no output bit below the cap, so the
// membership test may use the larger down-closed set
//   NR = {U : every S subset of U with |S| <= cap is in STRICT}
// instead of STRICT. The bitmap then holds STRICT on the levels <= cap and
// a subset of NR above (the updates keep it so); a closure turns the levels
// above the cap into exactly NR: set them to 1, then AND every entry with
// its subsets, one attribute at a time. The full-space bit is not derived
// from the q's in this mode; it is the candidate's known full-space status.
__device__ __forceinline__ uint32_t pop_above(int c) {
  return c < 0 ? kFull : (c >= 5 ? 0u : c_popabove[c]);
}

// Entries b of a word (5-bit masks): b &= b minus each of its bits.
__device__ __forceinline__ uint32_t subset_and_in_word(uint32_t x) {
  x &= (x << 1) | 0x55555555u;
  x &= (x << 2) | 0x33333333u;
  x &= (x << 4) | 0x0f0f0f0fu;
  x &= (x << 8) | 0x00ff00ffu;
  x &= (x << 16) | 0x0000ffffu;
  return x;
}

// Registers (d <= 10): lane holds word wi (W words, W a power of two).
template <int D>
__device__ __forceinline__ uint32_t nr_close_reg(uint32_t x, uint32_t wi, int cap) {
  constexpr uint32_t W = BitState<D>::W;
  x = subset_and_in_word(x | pop_above(cap - __popc(wi)));
#pragma unroll
  for (int j = 0; (1u << j) < W; ++j) {
    const uint32_t y = __shfl_xor_sync(kFull, x, 1 << j);
    if (wi & (1u << j)) x &= y;
  }
  return x;
}

// Shared memory (d >= 11): lane owns words 32i + lane. Word bits 0..4 are
// exchanged by shuffles, the row bits i stay inside the lane's column.
template <int D>
__device__ void nr_close_smem(uint32_t* sat_s, int lane, int cap) {
  constexpr uint32_t R = BitState<D>::W / 32;
  __syncwarp();
  for (uint32_t i = 0; i < R; ++i) {
    const uint32_t w = 32 * i + lane;
    uint32_t x = subset_and_in_word(sat_s[w] | pop_above(cap - __popc(w)));
#pragma unroll
    for (int j = 0; j < 5; ++j) {
      const uint32_t y = __shfl_xor_sync(kFull, x, 1 << j);
      if (lane & (1 << j)) x &= y;
    }
    sat_s[w] = x;
  }
  for (uint32_t j = 0; (1u << j) < R; ++j) {
    const uint32_t st = 1u << j;
    for (uint32_t t = 0; t < R / 2; ++t) {
      const uint32_t i = ((t >> j) << (j + 1)) | st | (t & (st - 1));
      sat_s[32 * i + lane] &= sat_s[32 * (i ^ st) + lane];
    }
  }
  __syncwarp();
}

// Register budgets: d <= 10 (STRICT in registers) 8 CTAs per SM uncapped
// (32 registers, no spill), 6 capped; d >= 11, 4 CTAs (64 registers).
// Unbounded, the allocator took 48 registers at d = 10 (40 warps per SM
// instead of 64) and up to 136 at d = 16.
template <int D, bool CAP>
__global__ void __launch_bounds__(256, (D <= 10 ? (CAP ? 6 : 8) : 4)) k_bitmaps(
    const uint4* __restrict__ pcells, const float* __restrict__ px,
    uint64_t p_pad, const uint4* __restrict__ qcells,
    const float* __restrict__ qx, const uint4* __restrict__ bmin,
    const uint4* __restrict__ smin, const uint4* __restrict__ hmin,
    const uint32_t* __restrict__ boff, const uint32_t* __restrict__ unrank,
    uint32_t K, int B, int depth,
    const uint32_t* __restrict__ m_ptr, uint32_t* __restrict__ work, uint32_t chunk,
    uint32_t p_end_cap, uint32_t* __restrict__ out_dom,
    uint32_t* __restrict__ out_ext, uint32_t* __restrict__ tie_slab, int cap,
    const uint8_t* __restrict__ full_dom) {
  using BS = BitState<D>;
  constexpr int NW = (D + 3) / 4;
  constexpr uint32_t NSUB = BS::NSUB;
  constexpr uint32_t W = BS::W;
  constexpr bool REG = BS::REG;
  constexpr uint32_t AW = BS::AW;
  extern __shared__ uint32_t smem[];

  const int lane = threadIdx.x & 31;
  const int wib = threadIdx.x >> 5;
  uint32_t* wsm = smem + (size_t)wib * BS::SMEM_WORDS;
  uint32_t* bq = wsm + BS::SMEM_WORDS - BS::WALK_WORDS;  // open blocks, waiting
  uint32_t* wq = bq + BS::BQ_WORDS;                      // open quarters, waiting
  uint32_t* hq = wq + BS::WQ_WORDS;                      // open halves, waiting
  const uint32_t lt_mask = (1u << lane) - 1u;
  uint32_t* sat_s = REG ? nullptr : wsm;
  uint32_t* A = BS::A_SMEM
                    ? wsm + (REG ? 0 : W)
                    : tie_slab + ((size_t)blockIdx.x * (blockDim.x / 32) + wib) * AW;
  const uint32_t m = *m_ptr;
  const uint32_t pend = min(m, p_end_cap);
  const uint32_t wi = REG ? (uint32_t)lane % W : 0;
  const int sh = depth - 1;
  // Capped mode, d >= 11: blocks walked between closures (a closure costs
  // about as much as walking W / 32 blocks).
  constexpr uint32_t kCloseBlocks = W / 32;

#if SKC_BITMAP_COUNTERS
  unsigned long long cnt_[kBitmapCounters] = {};
#endif
  for (;;) {
    // The warp takes `chunk` consecutive candidates per grab.
    uint32_t p0 = 0;
    if (lane == 0) p0 = atomicAdd(work, chunk);
    p0 = __shfl_sync(kFull, p0, 0);
    if (p0 >= pend) {
#if SKC_BITMAP_COUNTERS
      if (lane == 0)
        for (int i = 0; i < kBitmapCounters; ++i) atomicAdd(&g_bitmap_counters[i], cnt_[i]);
#endif
      break;
    }
    const uint32_t p1 = min(pend, p0 + chunk);
    for (uint32_t p = p0; p < p1; ++p) {
    const uint4 pc4 = pcells[p];
    uint32_t pH[NW];  // p's cells with the guard bits set (cells are < 128)
#pragma unroll
    for (int w = 0; w < NW; ++w) pH[w] = word_of(pc4, w) | kGuard;
    // p's median mask over the partitioning attributes 0 .. B-1
    uint32_t pmask = 0;
#pragma unroll
    for (int k = 0; k < D; ++k)
      if (k < B) pmask |= ((word_of(pc4, k >> 2) >> (8 * (k & 3) + sh)) & 1u) << k;
    // p's floats are read where a cell ties (rare; cached), not held in
    // registers.
    const float* pxp = px + p;

    // STRICT starts with the empty subspace so that q's worse on every
    // attribute (U == 0) test as "nothing new".
    SKC_COUNT(0, 1);
    SKC_SCOPE(cs_cand, 16);
    uint32_t sat = 0;
    if (REG) {
      sat = (wi == 0) ? 1u : 0u;
    } else {
      for (uint32_t w = lane; w < W; w += 32) sat_s[w] = (w == 0) ? 1u : 0u;
      __syncwarp();
    }
    FullFix fix;
    bool dirty = false;   // capped: STRICT grew since the last closure
    uint32_t since = 0;   // capped, d >= 11: blocks walked since then
    if constexpr (CAP) {
      fix.word = W - 1;
      const uint32_t fb = 1u << ((NSUB - 1) & 31);
      if (full_dom[p]) fix.set = fb; else fix.clr = fb;
    }
    // Capped, d >= 11: close when STRICT grew and enough blocks were walked.
    auto maybe_close = [&]() {
      if constexpr (CAP && !REG) {
        if (dirty && since >= kCloseBlocks) {
          nr_close_smem<D>(sat_s, lane, cap);
          dirty = false;
          since = 0;
        }
      }
    };
    bool touched = false;  // tie map in use for this p
    // d >= 13: 0 no tie pair, 1 pairs in the list, 2 pairs in the global map
    int tmode = 0;
    uint32_t tcount = 0;  // pairs in the list (same in every lane)
    auto in_strict = [&](uint32_t S) -> bool {
      uint32_t word;
      if (REG) word = __shfl_sync(kFull, sat, S >> 5);
      else word = sat_s[S >> 5];
      return (word >> (S & 31)) & 1u;
    };

    // Tests the q's of one block (position qi in lane t) against p and
    // applies their strict and tie sets.
    auto test_q = [&](uint32_t qi) {
      const uint4 q4 = qcells[qi];
      uint32_t U = 0;
#pragma unroll
      for (int w = 0; w < NW; ++w)
        U |= pack_guards(ge_bytes(pH[w], word_of(q4, w))) << (4 * w);
      U &= NSUB - 1;
      const bool hit = in_strict(U);
      SKC_COUNT(5, 1);
      if (__all_sync(kFull, hit)) {
        SKC_COUNT(6, 1);
        return;
      }
      SKC_COUNT(9, __popc(__ballot_sync(kFull, !hit)));

      uint32_t le = 0, lt = 0;
      if (!hit) {
        uint32_t G = 0;  // cell(q) >= cell(p)
#pragma unroll
        for (int w = 0; w < NW; ++w)
          G |= pack_guards(ge_bytes(word_of(q4, w) | kGuard, pH[w] ^ kGuard)) << (4 * w);
        G &= NSUB - 1;
        const uint32_t Y = U & ~G;  // certainly q < p
        const uint32_t Z = U & G;   // equal cells: compare the floats
        le = Y;
        lt = Y;
        // The warp runs the union of its lanes' work: the unrolled form
        // costs all D predicated steps whenever any lane has a cell tie, the
        // loop only as many as the lane with the most ties. Measured on one
        // box (bitmap kernel, identical outputs): 1M x 10 13.53 -> 11.65 ms,
        // 400k x 12 33.7 -> 31.9 ms, 400k x 12 -m 6 23.06 -> 21.73 ms, 300k x
        // 14 51.2 -> 49.0 ms; capped above 12 attributes the loop lost
        // (500k x 16 -m 6 242.7 -> 249.0 ms, -m 8 434 -> 450 ms), and those
        // keep the unrolled form.
        if constexpr (!CAP || D <= 12) {
          for (uint32_t z = Z; z; z &= z - 1) {
            const int k = __ffs(z) - 1;
            const float a = qx[(uint64_t)k * p_pad + qi];
            const float b = pxp[(uint64_t)k * p_pad];
            const uint32_t bit = 1u << k;
            if (a <= b) le |= bit;
            if (a < b) lt |= bit;
          }
        } else if (Z) {
#pragma unroll
          for (int k = 0; k < D; ++k) {
            if (Z & (1u << k)) {
              const float a = qx[(uint64_t)k * p_pad + qi];
              const float b = pxp[(uint64_t)k * p_pad];
              if (a <= b) le |= 1u << k;
              if (a < b) lt |= 1u << k;
            }
          }
        }
      }
      const bool t_lt = in_strict(lt);
      const bool t_le = in_strict(le);
      // Tie pairs go to the tie map (one atomic per lane); a tie set
      // inside STRICT changes nothing.
      const bool tie_lane = !hit && le != lt && !t_le;
      const uint32_t tb = __ballot_sync(kFull, tie_lane);
      SKC_COUNT(8, __popc(tb));
      if (tb) {
        if constexpr (BS::A_SMEM) {
          if (!touched) {
            for (uint32_t w = lane; w < AW; w += 32) A[w] = 0;
            __syncwarp();
            touched = true;
          }
          if (tie_lane) atomicOr(&A[le >> 1], lt << (16 * (le & 1)));
        } else {
          uint32_t* tlist = wsm + W + BS::CHUNK_WORDS;
          const uint32_t nt = __popc(tb);
          if (tmode != 2 && tcount + nt <= BS::LIST_WORDS) {
            if (tie_lane) tlist[tcount + __popc(tb & ((1u << lane) - 1u))] = le | (lt << 16);
            tcount += nt;
            tmode = 1;
            __syncwarp();
          } else {
            if (tmode != 2) {
              // Too many pairs: move to the global map (zeroed, then
              // the listed pairs OR-ed in).
              for (uint32_t w = lane; w < AW; w += 32) A[w] = 0;
              __syncwarp();
              if ((uint32_t)lane < tcount) {
                const uint32_t e = tlist[lane];
                atomicOr(&A[(e & 0xffffu) >> 1], (e >> 16) << (16 * (e & 1u)));
              }
              tmode = 2;
            }
            if (tie_lane) atomicOr(&A[le >> 1], lt << (16 * (le & 1)));
          }
        }
      }
      // Strict updates: down(LT) into STRICT, one pair at a time.
      uint32_t todo = __ballot_sync(kFull, !hit && !t_lt);
      while (todo) {
        const int src = __ffs(todo) - 1;
        todo &= todo - 1;
        const uint32_t L = __shfl_sync(kFull, lt, src);
        if (in_strict(L)) continue;  // covered by an earlier update
        SKC_COUNT(7, 1);
        if constexpr (CAP) dirty = true;
        if (REG) {
          if ((wi & ~(L >> 5)) == 0) sat |= c_submask[L & 31];
        } else {
          // Only the words under L: the subsets of L >> 5. Lane j
          // takes the j-th subset of the lowest five bits of L >> 5
          // and walks all subsets of the remaining bits.
          const uint32_t sl = c_submask[L & 31];
          uint32_t base, rest;
          if (split_words(L >> 5, lane, &base, &rest)) {
            uint32_t sub = 0;
            do {
              sat_s[base | sub] |= sl;
              sub = (sub - rest) & rest;
            } while (sub);
          }
          __syncwarp();
        }
      }
      if constexpr (CAP && REG) {
        if (dirty) {
          sat = nr_close_reg<D>(sat, wi, cap);
          dirty = false;
        }
      }
    };

    // Open blocks, 8-q quarters and 4-q halves wait in per-warp stacks
    // until a full step's worth is there (8 blocks' quarters per quarter
    // step, 16 quarters' halves per half step, 8 halves per walk step), so
    // steps stay full across box-test steps; the order they are taken in
    // does not matter for the result.
    uint32_t bq_n = 0, wq_n = 0, hq_n = 0;
    // Walk step over the top c waiting halves (c <= 8: lane t on q t % 4 of
    // half t / 4) or, with `quarters`, quarters (c <= 4: lane t on q t % 8
    // of quarter t / 8); lanes past the last one repeat it (a q tested twice
    // changes nothing). The q arrays are padded to whole blocks with
    // entries that add nothing (k_pad_q). One call site of test_q: a second
    // one spilled the capped 15-attribute kernel.
    auto walk = [&](bool quarters, uint32_t c) {
      SKC_T0(t_walk);
      const int lg = quarters ? 3 : 2;  // log2 of the q's per entry
      uint32_t* st = quarters ? wq : hq;
      uint32_t& n = quarters ? wq_n : hq_n;
      const uint32_t jj = min((uint32_t)lane >> lg, c - 1);
      const uint32_t qi = (st[n - c + jj] << lg) + ((uint32_t)lane & ((1u << lg) - 1u));
      n -= c;
      __syncwarp();  // read before a later push overwrites the entry
      test_q(qi);
      SKC_TADD(15, t_walk);
      if constexpr (CAP && !REG) since += 1;
    };
    auto walk_step = [&](uint32_t c) { walk(false, c); };
    // Half step over the top c (<= 16) waiting quarters: lane t tests 4-q
    // half t % 2 of quarter t / 2; the open halves are pushed and walked
    // eight at a time.
    auto half_step = [&](uint32_t c) {
      SKC_T0(t_half);
      const uint32_t slot = lane >> 1;
      const bool valid = slot < c;
      const uint32_t hid = wq[wq_n - c + (valid ? slot : c - 1)] * 2 + (lane & 1);
      wq_n -= c;
      uint32_t Uh = 0;
      if (valid) {
        const uint4 hm = hmin[hid];
#pragma unroll
        for (int w = 0; w < NW; ++w)
          Uh |= pack_guards(ge_bytes(pH[w], word_of(hm, w))) << (4 * w);
        Uh &= NSUB - 1;
      }
      const bool uh_strict = in_strict(Uh);  // every lane (shuffle)
      const uint32_t open = __ballot_sync(kFull, valid && !uh_strict);
      SKC_COUNT(18, c * 2);
      SKC_COUNT(19, __popc(open));
      if constexpr (CAP && !REG) since += 1;
      __syncwarp();
      if ((open >> lane) & 1u) hq[hq_n + __popc(open & lt_mask)] = hid;
      hq_n += __popc(open);
      __syncwarp();
      SKC_TADD(14, t_half);
      while (hq_n >= 8) walk_step(8);
    };
    // Quarter step over the top c (<= 8) waiting blocks: lane t tests 8-q
    // quarter t % 4 of block t / 4 against STRICT as the walks so far left
    // it; the open quarters are pushed and their halves tested sixteen
    // quarters at a time.
    auto sub_step = [&](uint32_t c) {
      SKC_T0(t_sub);
      const uint32_t slot = lane >> 2;
      const bool valid = slot < c;
      const uint32_t sid = bq[bq_n - c + (valid ? slot : c - 1)] * 4 + (lane & 3);
      bq_n -= c;
      uint32_t Us = 0;
      if (valid) {
        const uint4 sm = smin[sid];
#pragma unroll
        for (int w = 0; w < NW; ++w)
          Us |= pack_guards(ge_bytes(pH[w], word_of(sm, w))) << (4 * w);
        Us &= NSUB - 1;
      }
      const bool us_strict = in_strict(Us);  // every lane (shuffle)
      const uint32_t open = __ballot_sync(kFull, valid && !us_strict);
      SKC_COUNT(10, c * 4);
      SKC_COUNT(11, __popc(open));
      if constexpr (CAP && !REG) since += 1;
      __syncwarp();
      if ((open >> lane) & 1u) wq[wq_n + __popc(open & lt_mask)] = sid;
      wq_n += __popc(open);
      __syncwarp();
      SKC_TADD(14, t_sub);
      while (wq_n >= 16) half_step(16);
    };

    uint32_t next_blk = 0;  // blocks below this one were already visited
    // Partitions are tested 32 at a time (lane t tests partition b0 + t):
    // a partition is skipped when the attributes its points may win on
    // (all but those where the partition is above the median and p is not)
    // already form a strictly dominated subspace.
    for (uint32_t b0 = 0; b0 < K; b0 += 32) {
      SKC_T0(t_part);
      maybe_close();
      if constexpr (CAP) {  // every subspace within the cap is strict
        if (in_strict(NSUB - 1)) break;
      }
      const uint32_t bl = b0 + lane;
      uint32_t qbeg_l = 0, qend_l = 0, Sb = 0;
      if (bl < K) {
        qbeg_l = boff[bl];
        qend_l = boff[bl + 1];
        Sb = (NSUB - 1) & ~(unrank[bl] & ~pmask);
      }
      // in_strict shuffles across the warp: every lane must evaluate it.
      const bool sb_strict = in_strict(Sb);
      const bool sel = (qbeg_l != qend_l) && !sb_strict;
      const uint32_t parts = __ballot_sync(kFull, sel);
      SKC_COUNT(1, 1);
      SKC_COUNT(2, __popc(parts));
      if (!parts) {
        SKC_TADD(12, t_part);
        continue;
      }
      // The blocks of all selected partitions form one list, so their box
      // tests fill the 32 lanes: lane t's partition owns blocks [bf, be).
      // A block shared with the previous selected partition (or visited
      // under an earlier ballot) is visited once; its q's from a skipped
      // partition are tested too (any q's update is valid).
      const uint32_t be = (qend_l + 31) / 32;
      const uint32_t lower = parts & ((1u << lane) - 1u);
      const int prev = lower ? 31 - __clz(lower) : 0;
      const uint32_t prev_be = __shfl_sync(kFull, be, prev);
      const uint32_t bf = max(qbeg_l / 32, lower ? prev_be : next_blk);
      const uint32_t cnt = (sel && be > bf) ? be - bf : 0u;
      uint32_t incl = cnt;  // inclusive prefix sum of the block counts
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(kFull, incl, o);
        if (lane >= o) incl += y;
      }
      const uint32_t total = __shfl_sync(kFull, incl, 31);
      next_blk = max(next_blk, __shfl_sync(kFull, be, 31 - __clz(parts)));
      // list entry g of lane t's partition is block g + base (mod 2^32)
      const uint32_t base = bf - (incl - cnt);
      SKC_TADD(12, t_part);
      for (uint32_t t0 = 0; t0 < total; t0 += 32) {
        SKC_T0(t_box);
        maybe_close();
        const uint32_t g = t0 + lane;
        // owner of list entry g: the first lane whose inclusive sum is > g
        int j = 0;
#pragma unroll
        for (int step = 16; step; step >>= 1) {
          const uint32_t v = __shfl_sync(kFull, incl, j + step - 1);
          if (v <= g) j += step;
        }
        const uint32_t kb = g + __shfl_sync(kFull, base, j);
        const bool in_list = g < total;
        // Blocks are tested against their byte-wise minimum cells; the
        // surviving ones wait for their quarters' tests (sub_step).
        uint32_t Ub = 0;
        if (in_list) {
          const uint4 bm = bmin[kb];
#pragma unroll
          for (int w = 0; w < NW; ++w)
            Ub |= pack_guards(ge_bytes(pH[w], word_of(bm, w))) << (4 * w);
          Ub &= NSUB - 1;
        }
        const bool ub_strict = in_strict(Ub);  // every lane (shuffle)
        const uint32_t blocks = __ballot_sync(kFull, in_list && !ub_strict);
        SKC_COUNT(3, 1);
        SKC_COUNT(4, min(32u, total - t0));
        if constexpr (CAP && !REG) since += 1;
        if (!blocks) {
          SKC_TADD(13, t_box);
          continue;
        }
        // The open blocks go on the warp's stack (earlier readers of those
        // entries are past the fence).
        __syncwarp();
        if ((blocks >> lane) & 1u) bq[bq_n + __popc(blocks & lt_mask)] = kb;
        bq_n += __popc(blocks);
        __syncwarp();
        SKC_TADD(13, t_box);
        while (bq_n >= 8) sub_step(8);
      }
    }
    // What still waits: one short step of each kind, except that at most
    // four waiting quarters are walked whole (one step instead of a half
    // step and a walk step: candidates with a single open block, as on
    // correlated data, mostly end here).
    if (bq_n) sub_step(bq_n);
    if (wq_n > 4) half_step(wq_n);
    else if (wq_n) walk(true, wq_n);
    if (hq_n) walk_step(hq_n);

    // Output: dominated = STRICT | TIE, extended = TIE \ STRICT, with TIE
    // from the closed tie map. Bit 0 (the empty subspace) is cleared.
    SKC_SCOPE(cs_out, 17);
    if constexpr (!BS::A_SMEM) {
      if (tmode == 2) {
        __syncwarp();
        tie_global_output<D>(A, wsm + W, sat_s, lane, p, out_dom, out_ext, fix);
        __syncwarp();
        continue;
      }
      if (tmode == 1) {
        // Few pairs: word w of each pair's tie set down(E) \ down(E \ L)
        // is submask(E & 31) when w is a subset of E >> 5, minus
        // submask(F & 31) when w is also a subset of F >> 5, F = E \ L.
        const uint32_t* tlist = wsm + W + BS::CHUNK_WORDS;
        for (uint32_t w = lane; w < W; w += 32) {
          uint32_t t_ = 0;
          for (uint32_t j = 0; j < tcount; ++j) {
            const uint32_t e = tlist[j];
            const uint32_t E = e & 0xffffu, F = E & ~(e >> 16);
            if ((w & ~(E >> 5)) == 0u)
              t_ |= c_submask[E & 31] & (((w & ~(F >> 5)) == 0u) ? ~c_submask[F & 31] : ~0u);
          }
          const uint32_t s_ = sat_s[w];
          uint32_t dom = s_ | t_, ext = t_ & ~s_;
          if (w == 0) {
            dom &= ~1u;
            ext &= ~1u;
          }
          if constexpr (CAP) fix.apply(w, dom, ext);
          out_dom[(uint64_t)p * W + w] = dom;
          if (out_ext) out_ext[(uint64_t)p * W + w] = ext;
        }
        __syncwarp();
        continue;
      }
    }
    if (touched) {
      __syncwarp();
      tie_closure<D>(A, lane);
    }
    if (REG) {
      uint32_t tie = 0;
      if (touched && (uint32_t)lane < W) tie = tie_word<D>(A, lane);
      if ((uint32_t)lane < W) {
        uint32_t dom = sat | tie, ext = tie & ~sat;
        if (lane == 0) {
          dom &= ~1u;
          ext &= ~1u;
        }
        if constexpr (CAP) fix.apply(lane, dom, ext);
        out_dom[(uint64_t)p * W + lane] = dom;
        if (out_ext) out_ext[(uint64_t)p * W + lane] = ext;
      }
    } else {
      for (uint32_t w = lane; w < W; w += 32) {
        const uint32_t s_ = sat_s[w];
        const uint32_t t_ = touched ? tie_word<D>(A, w) : 0u;
        uint32_t dom = s_ | t_, ext = t_ & ~s_;
        if (w == 0) {
          dom &= ~1u;
          ext &= ~1u;
        }
        if constexpr (CAP) fix.apply(w, dom, ext);
        out_dom[(uint64_t)p * W + w] = dom;
        if (out_ext) out_ext[(uint64_t)p * W + w] = ext;
      }
    }
    __syncwarp();
    }
  }
}

// Capped kernels exist for d >= 6 (below, a cap under d - 1 leaves too few
// cuboids to matter and the uncapped kernel serves).
constexpr int kMinCapDims = 6;

template <int D, bool CAP>
static int bitmap_grid_dc(int num_sms, int* grid, size_t* smem) {
  using BS = BitState<D>;
  constexpr int threads = 256;
  *smem = (size_t)(threads / 32) * BS::SMEM_WORDS * sizeof(uint32_t);
  if (*smem > 48 * 1024)
    SKC_CUDA(cudaFuncSetAttribute(k_bitmaps<D, CAP>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)*smem));
  int per_sm = 0;
  SKC_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_bitmaps<D, CAP>, threads, *smem));
  if (per_sm < 1) per_sm = 1;
  if (!BS::A_SMEM && per_sm > 4) per_sm = 4;  // bounds the global tie-map slab
  *grid = per_sm * num_sms;
  return SKC_OK;
}

// Persistent grid of the bitmap kernel: the larger of the two variants' (the
// tie-map slab is sized by it).
template <int D>
static int bitmap_grid_d(int num_sms, int* grid, size_t* smem) {
  SKC_TRY((bitmap_grid_dc<D, false>(num_sms, grid, smem)));
  if constexpr (D >= kMinCapDims) {
    int g2 = 0;
    size_t s2 = 0;
    SKC_TRY((bitmap_grid_dc<D, true>(num_sms, &g2, &s2)));
    if (g2 > *grid) *grid = g2;
  }
  return SKC_OK;
}

template <int D, bool CAP>
static int launch_bitmaps_dc(cudaStream_t s, int num_sms, const BitmapArgs& a) {
  int grid = 0;
  size_t smem = 0;
  SKC_TRY((bitmap_grid_dc<D, CAP>(num_sms, &grid, &smem)));
  if (a.grid_blocks > 0 && a.grid_blocks < grid) grid = a.grid_blocks;
  k_bitmaps<D, CAP><<<grid, 256, smem, s>>>(a.pcells, a.px, a.p_pad, a.qcells, a.qx,
                                             a.bmin, a.smin, a.hmin, a.boff, a.unrank, a.K, a.B, a.depth,
                                             a.m_ptr, a.work, a.chunk ? a.chunk : 1u, a.p_end,
                                             a.out_dom, a.out_ext,
                                             a.tie_slab, a.cap, a.full_dom);
  SKC_LAUNCH_CHECK();
  return SKC_OK;
}

template <int D>
static int launch_bitmaps_d(cudaStream_t s, int num_sms, const BitmapArgs& a) {
  if (a.cap > 0) {
    if (a.cap > D - 2 || !a.full_dom)
      return set_error(SKC_ERR_INVALID, "bitmap cap %d needs 1 <= cap <= d - 2 and full-space flags", a.cap);
    if constexpr (D >= kMinCapDims) return launch_bitmaps_dc<D, true>(s, num_sms, a);
  }
  return launch_bitmaps_dc<D, false>(s, num_sms, a);
}

#define SKC_BITMAP_DISPATCH(fn, ...)                    \
  switch (d) {                                          \
    case 2: return fn<2>(__VA_ARGS__);                  \
    case 3: return fn<3>(__VA_ARGS__);                  \
    case 4: return fn<4>(__VA_ARGS__);                  \
    case 5: return fn<5>(__VA_ARGS__);                  \
    case 6: return fn<6>(__VA_ARGS__);                  \
    case 7: return fn<7>(__VA_ARGS__);                  \
    case 8: return fn<8>(__VA_ARGS__);                  \
    case 9: return fn<9>(__VA_ARGS__);                  \
    case 10: return fn<10>(__VA_ARGS__);                \
    case 11: return fn<11>(__VA_ARGS__);                \
    case 12: return fn<12>(__VA_ARGS__);                \
    case 13: return fn<13>(__VA_ARGS__);                \
    case 14: return fn<14>(__VA_ARGS__);                \
    case 15: return fn<15>(__VA_ARGS__);                \
    case 16: return fn<16>(__VA_ARGS__);                \
    default: return set_error(SKC_ERR_INVALID, "unsupported d=%d", d); \
  }

#if SKC_BITMAP_COUNTERS
// Counters build only: copies the kBitmapCounters (20) summed counters out
// (`out` holds at least that many) and, when reset is nonzero, zeroes them.
extern "C" int skc_debug_bitmap_counters(unsigned long long* out, int reset) {
  if (cudaMemcpyFromSymbol(out, g_bitmap_counters, sizeof(g_bitmap_counters)) != cudaSuccess)
    return SKC_ERR_CUDA;
  if (reset) {
    unsigned long long z[kBitmapCounters] = {};
    if (cudaMemcpyToSymbol(g_bitmap_counters, z, sizeof(z)) != cudaSuccess) return SKC_ERR_CUDA;
  }
  return SKC_OK;
}
#endif

int launch_bitmaps(cudaStream_t s, int d, int num_sms, const BitmapArgs& a) {
  SKC_BITMAP_DISPATCH(launch_bitmaps_d, s, num_sms, a)
}

template <int D>
static int slab_words_d(int num_sms, uint64_t* words) {
  using BS = BitState<D>;
  if (BS::A_SMEM) {
    *words = 0;
    return SKC_OK;
  }
  int grid = 0;
  size_t smem = 0;
  SKC_TRY(bitmap_grid_d<D>(num_sms, &grid, &smem));
  *words = (uint64_t)grid * 8 * BS::AW;
  return SKC_OK;
}

// Words of global memory the bitmap kernel needs for its tie maps (0 when
// they fit in shared memory).
int bitmap_tie_slab_words(int d, int num_sms, uint64_t* words) {
  SKC_BITMAP_DISPATCH(slab_words_d, num_sms, words)
}

// --------------------------------------------------------------------------
// Compaction of bitmaps into per-cuboid id lists. Rows are cut in tiles of
// kTileRows; a CTA handles one (tile, word) pair with 8 warps, warp k owning
// rows [k*256, k*256+256) of the tile, so ids come out ascending per cuboid.
constexpr uint32_t kTileRows = 2048;

uint32_t compact_tiles(uint64_t m_max) {
  uint64_t t = (m_max + kTileRows - 1) / kTileRows;
  return (uint32_t)(t ? t : 1);
}

// Cuboids within max_d, plus the full space, which is always computed (the
// suite computes it first in both algorithms).
__device__ __forceinline__ bool cuboid_wanted(uint32_t c, uint32_t nsub, int max_d) {
  return c >= 1 && c < nsub && (__popc(c) <= max_d || c == nsub - 1);
}

// Bits of row r's word w that count (1 = counted).
__device__ __forceinline__ uint32_t counted_bits(const uint32_t* bits, uint32_t W,
                                                 uint32_t r, uint32_t m, uint32_t w,
                                                 int count_set) {
  if (r >= m) return 0u;
  const uint32_t v = bits[(uint64_t)r * W + w];
  return count_set ? v : ~v;
}

__global__ void __launch_bounds__(256) k_bits_count(
    const uint32_t* __restrict__ bits, uint32_t W,
    const uint32_t* __restrict__ m_ptr, uint32_t T, int count_set,
    uint32_t nsub, int max_d, uint32_t* __restrict__ counts) {
  __shared__ uint32_t wc[8][32];
  const uint32_t t = blockIdx.x, w = blockIdx.y;
  const int lane = threadIdx.x & 31, k = threadIdx.x >> 5;
  const uint32_t m = *m_ptr;
  // Cuboids of this word that are computed (all but the empty one without a
  // cap; under -m a word may hold none): only their bit columns are counted.
  const uint32_t wanted = __ballot_sync(kFull, cuboid_wanted(w * 32 + lane, nsub, max_d));
  uint32_t cnt = 0;
  const uint32_t row0 = t * kTileRows + k * 256;
  if (t * kTileRows < m && wanted) {
    const bool dense = __popc(wanted) > 16;  // then all 32 columns, unrolled
    for (int s = 0; s < 8; ++s) {
      const uint32_t v = counted_bits(bits, W, row0 + s * 32 + lane, m, w, count_set) & wanted;
      if (dense) {
#pragma unroll
        for (int b = 0; b < 32; ++b) {  // one warp reduction per bit column
          const uint32_t tot = __reduce_add_sync(kFull, (v >> b) & 1u);
          if (lane == b) cnt += tot;
        }
      } else {
        for (uint32_t mm = wanted; mm; mm &= mm - 1) {
          const int b = __ffs(mm) - 1;
          const uint32_t tot = __reduce_add_sync(kFull, (v >> b) & 1u);
          if (lane == b) cnt += tot;
        }
      }
    }
  }
  wc[k][lane] = cnt;
  __syncthreads();
  if (threadIdx.x < 32) {
    uint32_t sum = 0;
    for (int j = 0; j < 8; ++j) sum += wc[j][threadIdx.x];
    const uint32_t c = w * 32 + threadIdx.x;
    counts[(uint64_t)c * T + t] = cuboid_wanted(c, nsub, max_d) ? sum : 0u;
  }
}

__global__ void __launch_bounds__(256) k_bits_write(
    const uint32_t* __restrict__ bits, uint32_t W,
    const uint32_t* __restrict__ m_ptr, uint32_t T, int count_set,
    uint32_t nsub, int max_d, const uint64_t* __restrict__ offs,
    const uint32_t* __restrict__ cand, uint32_t* __restrict__ out, uint64_t out_cap) {
  __shared__ uint32_t wc[8][32];
  __shared__ uint32_t run[8][32];
  const uint32_t t = blockIdx.x, w = blockIdx.y;
  const int lane = threadIdx.x & 31, k = threadIdx.x >> 5;
  const uint32_t m = *m_ptr;
  const uint32_t wanted = __ballot_sync(kFull, cuboid_wanted(w * 32 + lane, nsub, max_d));
  if (t * kTileRows >= m || !wanted) return;  // uniform over the CTA
  const uint32_t row0 = t * kTileRows + k * 256;
  const bool dense = __popc(wanted) > 16;  // then all 32 columns, unrolled
  // pass 1: per-warp counts
  uint32_t cnt = 0;
  for (int s = 0; s < 8; ++s) {
    const uint32_t v = counted_bits(bits, W, row0 + s * 32 + lane, m, w, count_set) & wanted;
    if (dense) {
#pragma unroll
      for (int b = 0; b < 32; ++b) {
        const uint32_t bal = __ballot_sync(kFull, (v >> b) & 1u);
        if (lane == b) cnt += __popc(bal);
      }
    } else {
      for (uint32_t mm = wanted; mm; mm &= mm - 1) {
        const int b = __ffs(mm) - 1;
        const uint32_t bal = __ballot_sync(kFull, (v >> b) & 1u);
        if (lane == b) cnt += __popc(bal);
      }
    }
  }
  wc[k][lane] = cnt;
  __syncthreads();
  // exclusive prefix over warps, per bit
  if (threadIdx.x < 32) {
    uint32_t acc = 0;
    for (int j = 0; j < 8; ++j) {
      const uint32_t v = wc[j][threadIdx.x];
      run[j][threadIdx.x] = acc;
      acc += v;
    }
  }
  __syncthreads();
  // pass 2: write ids
  const uint32_t lt_mask = (1u << lane) - 1u;
  for (int s = 0; s < 8; ++s) {
    const uint32_t r = row0 + s * 32 + lane;
    const uint32_t v = counted_bits(bits, W, r, m, w, count_set) & wanted;
    const uint32_t id = r < m ? cand[r] : 0u;
    // Dense words walk all 32 columns (unwanted ones are masked to zero).
    const uint32_t cols = dense ? kFull : wanted;
#pragma unroll 4
    for (uint32_t mm = cols; mm; mm &= mm - 1) {
      const int b = __ffs(mm) - 1;
      const uint32_t bal = __ballot_sync(kFull, (v >> b) & 1u);
      if (!bal) continue;
      const uint32_t c = w * 32 + b;
      const uint32_t base = run[k][b];
      if ((v >> b) & 1u) {
        const uint64_t pos = offs[(uint64_t)c * T + t] + base + __popc(bal & lt_mask);
        if (pos < out_cap) out[pos] = id;
      }
      __syncwarp();
      if (lane == 0) run[k][b] = base + __popc(bal);
      __syncwarp();
    }
  }
}

// csr_off[c] = offs[c * T] for c in [0, nsub]; offs[32*W*T] is the total.
__global__ void k_extract_csr(const uint64_t* __restrict__ offs, uint32_t T,
                              uint32_t nsub, uint64_t* __restrict__ csr_off) {
  for (uint32_t c = blockIdx.x * blockDim.x + threadIdx.x; c <= nsub;
       c += gridDim.x * blockDim.x)
    csr_off[c] = offs[(uint64_t)c * T];
}

int launch_bits_count(cudaStream_t s, const CompactArgs& a) {
  const uint32_t T = compact_tiles(a.m_max);
  const uint64_t C = 32ull * a.words;
  k_bits_count<<<dim3(T, a.words), 256, 0, s>>>(a.bits, a.words, a.m_ptr, T, a.count_set,
                                                 a.nsub, a.max_d, a.counts);
  SKC_LAUNCH_CHECK();
  SKC_TRY(launch_scan_u32_to_u64(s, a.counts, C * T, a.bsum, a.offs));
  k_extract_csr<<<(a.nsub + 256) / 256, 256, 0, s>>>(a.offs, T, a.nsub, a.csr_off);
  SKC_LAUNCH_CHECK();
  return SKC_OK;
}

int launch_bits_write(cudaStream_t s, const CompactArgs& a) {
  const uint32_t T = compact_tiles(a.m_max);
  k_bits_write<<<dim3(T, a.words), 256, 0, s>>>(a.bits, a.words, a.m_ptr, T, a.count_set,
                                                 a.nsub, a.max_d, a.offs, a.cand, a.out,
                                                 a.out_cap);
  SKC_LAUNCH_CHECK();
  return SKC_OK;
}

}  // namespace skc
