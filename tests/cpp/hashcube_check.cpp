// Host-side result layout of the suite-shaped interface, checked without a
// GPU: HashCube<D> filled from per-point dominated-subspace bitmaps, its
// per-cuboid decode (HashCube::getSubspace and the free getsubspace over
// getMaps()), and the lattice helpers (generate_lattice, get_tds_list).
//
// Usage: hashcube_check BITS_FILE D N
//   BITS_FILE: N points x W words of little-endian uint32 bitmaps
//   (W = max(1, 2^D / 32); bit c of a point set = dominated on cuboid c),
//   followed by N uint32 point ids.
// Prints "C c id id ..." (ascending ids) for every cuboid c, "W j count"
// (ids listed under bitmap word j) for every map, "P c parents..." and
// "K c children..." for every lattice node, then "T" and the top-down
// cuboid order. Exits 1 if the two decodes disagree.
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "skycube_templates.h"

template <int D>
static int run(const std::vector<uint32_t>& bits, const std::vector<uint32_t>& pids, uint64_t n,
               uint32_t words) {
  HashCube<D> hc;
  hc.populateFromBitmaps(bits.data(), pids.data(), n, words);
  const unsigned m = 1u << D;
  for (unsigned c = 1; c < m; ++c) {
    std::vector<int> a = hc.getSubspace(c);
    std::vector<int> b = getsubspace(c, hc.getMaps());
    std::sort(a.begin(), a.end());
    std::sort(b.begin(), b.end());
    if (a != b) {
      std::fprintf(stderr, "cuboid %u: getSubspace and getsubspace differ\n", c);
      return 1;
    }
    std::printf("C %u", c);
    for (int id : a) std::printf(" %d", id);
    std::printf("\n");
  }
  for (uint32_t j = 0; j < HashCube<D>::bitvector_num_words_; ++j) {
    size_t listed = 0;
    for (const auto& kv : hc.getMaps()[j]) listed += kv.second.size();
    std::printf("W %u %zu\n", j, listed);
  }
  lattice_node* lat = generate_lattice((int)m);
  for (unsigned c = 1; c < m; ++c) {
    std::printf("P %u", c);
    for (unsigned p : lat[c].parents) std::printf(" %u", p);
    std::printf("\nK %u", c);
    for (unsigned k : lat[c].children) std::printf(" %u", k);
    std::printf("\n");
  }
  delete[] lat;
  std::printf("T");
  for (unsigned c : get_tds_list((int)m)) std::printf(" %u", c);
  std::printf("\n");
  return 0;
}

int main(int argc, char** argv) {
  if (argc != 4) {
    std::fprintf(stderr, "usage: %s BITS_FILE D N\n", argv[0]);
    return 2;
  }
  const int d = std::atoi(argv[2]);
  const uint64_t n = std::strtoull(argv[3], nullptr, 10);
  const uint32_t words = d >= 5 ? (1u << d) / 32 : 1u;
  std::vector<uint32_t> bits(n * words), pids(n);
  FILE* f = std::fopen(argv[1], "rb");
  if (!f || std::fread(bits.data(), 4, bits.size(), f) != bits.size() ||
      std::fread(pids.data(), 4, n, f) != n) {
    std::fprintf(stderr, "cannot read %s\n", argv[1]);
    return 2;
  }
  std::fclose(f);
  switch (d) {
#define CASE(D) case D: return run<D>(bits, pids, n, words);
    CASE(2) CASE(3) CASE(4) CASE(5) CASE(6) CASE(7) CASE(8) CASE(9) CASE(10)
#undef CASE
    default:
      std::fprintf(stderr, "d=%d outside 2..10\n", d);
      return 2;
  }
}
