// Portable stand-in for <immintrin.h>, used only to compile the reference's
// STSC sources (test infrastructure) on hosts without x86 AVX, such as the
// aarch64 GPU hosts. The reference selects its dominance tests by `#if
// __AVX__` (src/utilities/common2.h:276) and its non-AVX branch lacks the
// array forms STSC calls (DominateLeft_array, DT_bitmap_array,
// DT_bitmap_dvc_array), so the build defines __AVX__ and puts this header on
// the include path ahead of the system's.
//
// It covers exactly what src/utilities/dt_avx2.h uses: the 128- and 256-bit
// float vector types, aligned and unaligned loads, compares with the
// predicates EQ_OS (0), LT_OS (1), LE_OS (2) and LT_OQ (17), and movemask.
// Each compare is the ordered IEEE comparison of that predicate, lane by
// lane, giving an all-ones or all-zeros lane; movemask gathers bit 31 of
// every lane, lane 0 into bit 0. Signalling and quiet forms differ only in
// floating-point exceptions, which nothing here observes, and the inputs
// hold no NaN.
#ifndef SKC_REF_SHIM_IMMINTRIN_H_
#define SKC_REF_SHIM_IMMINTRIN_H_

#include <stdint.h>
#include <string.h>

#define _CMP_EQ_OQ 0x00
#define _CMP_LT_OS 0x01
#define _CMP_LE_OS 0x02
#define _CMP_EQ_OS 0x10
#define _CMP_LT_OQ 0x11
#define _CMP_LE_OQ 0x12

struct skc_shim_m128 {
  uint32_t u[4];
};
struct skc_shim_m256 {
  uint32_t u[8];
};
typedef skc_shim_m128 __m128;
typedef skc_shim_m256 __m256;

template <int L, typename V>
static inline V skc_shim_load(const float* p) {
  V v;
  memcpy(v.u, p, sizeof(float) * L);
  return v;
}

static inline float skc_shim_f(uint32_t bits) {
  float f;
  memcpy(&f, &bits, sizeof f);
  return f;
}

// Predicate imm on one lane: the ordered relation of a to b. The low four
// bits select the relation (the fifth bit only chooses signalling or quiet).
static inline uint32_t skc_shim_cmp1(uint32_t a_bits, uint32_t b_bits, int imm) {
  const float a = skc_shim_f(a_bits), b = skc_shim_f(b_bits);
  bool r;
  switch (imm & 0x0f) {
    case 0x00: r = (a == b); break;
    case 0x01: r = (a < b); break;
    case 0x02: r = (a <= b); break;
    default: r = false; break;  // not used by the reference
  }
  return r ? 0xffffffffu : 0u;
}

template <int L, typename V>
static inline V skc_shim_cmp(const V& a, const V& b, int imm) {
  V r;
  for (int i = 0; i < L; ++i) r.u[i] = skc_shim_cmp1(a.u[i], b.u[i], imm);
  return r;
}

template <int L, typename V>
static inline int skc_shim_movemask(const V& a) {
  int m = 0;
  for (int i = 0; i < L; ++i) m |= (int)((a.u[i] >> 31) & 1u) << i;
  return m;
}

static inline __m128 _mm_load_ps(const float* p) { return skc_shim_load<4, __m128>(p); }
static inline __m128 _mm_loadu_ps(const float* p) { return skc_shim_load<4, __m128>(p); }
static inline __m256 _mm256_load_ps(const float* p) { return skc_shim_load<8, __m256>(p); }
static inline __m256 _mm256_loadu_ps(const float* p) { return skc_shim_load<8, __m256>(p); }
static inline __m128 _mm_cmp_ps(__m128 a, __m128 b, int imm) { return skc_shim_cmp<4>(a, b, imm); }
static inline __m256 _mm256_cmp_ps(__m256 a, __m256 b, int imm) { return skc_shim_cmp<8>(a, b, imm); }
static inline int _mm_movemask_ps(__m128 a) { return skc_shim_movemask<4>(a); }
static inline int _mm256_movemask_ps(__m256 a) { return skc_shim_movemask<8>(a); }

#endif  // SKC_REF_SHIM_IMMINTRIN_H_
