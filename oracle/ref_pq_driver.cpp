// C entry points around the reference's PQSkycube (ExecuteQSkycubeGLPMR<D>,
// src/qskycube/QSkycubeG.h:223-303), the suite's parallel QSkycube: a CPU
// skycube algorithm independent of STSC (sky trees, not sort-filter
// blocks). Compiled from the reference sources by oracle/build_ref.sh --pq
// (staged copy or checkout); the result is
// test infrastructure only (a second, independent check of the skylines the
// oracle and the reference's STSC give; QSkycube has no extended skylines).
//
// Input rows become the suite's Point layout (src/utilities/utilities.h:
// 198-206: p[0] holds the row id as a float, p[1..d] the attributes).
// QSkycube indexes cuboids by the attributes it leaves OUT
// (src/qskycube/Common.h:85-99: slot k lists the attributes whose bit in k
// is clear), so slot k holds the skyline of the cuboid mask (2^d - 1) ^ k.
#include <cstdint>
#include <cstring>
#include <vector>
#include "qskycube/QSkycubeG.h"

namespace {

struct PqResult {
  int d;
  std::vector<std::vector<uint32_t>> sky;  // indexed by cuboid mask
};

template <int D>
PqResult* run(const float* rows, uint32_t n, int max_d, int threads) {
  std::vector<Point> pts;
  pts.reserve(n);
  for (uint32_t i = 0; i < n; ++i) {
    Point p = new float[D + 1];
    p[0] = static_cast<float>(i);
    std::memcpy(p + 1, rows + (size_t)i * D, sizeof(float) * D);
    pts.push_back(p);
  }
  const uint32_t full = (1u << D) - 1;
  auto* cube = new std::vector<Point>[full];
  ExecuteQSkycubeGLPMR<D>(D, pts, cube, threads, max_d);
  auto* res = new PqResult;
  res->d = D;
  res->sky.resize(1u << D);
  for (uint32_t k = 0; k < full; ++k) {
    auto& out = res->sky[full ^ k];
    out.reserve(cube[k].size());
    for (Point p : cube[k]) out.push_back(static_cast<uint32_t>(p[0]));
  }
  delete[] cube;
  for (Point p : pts) delete[] p;
  return res;
}

}  // namespace

extern "C" {

// Returns an opaque handle, or nullptr for an unsupported d or n above the
// ids a float holds exactly (2^24).
void* ref_pq_run(const float* rows, uint32_t n, int d, int max_d, int threads) {
  if (n > (1u << 24)) return nullptr;
  if (max_d <= 0 || max_d > d) max_d = d;
  if (threads <= 0) threads = 1;
  switch (d) {
#define CASE(D) case D: return run<D>(rows, n, max_d, threads);
    CASE(2) CASE(3) CASE(4) CASE(5) CASE(6) CASE(7) CASE(8) CASE(9)
    CASE(10) CASE(11) CASE(12) CASE(13) CASE(14) CASE(15) CASE(16)
#undef CASE
    default: return nullptr;
  }
}

// ext is accepted for the oracle module's common binding; QSkycube computes
// skylines only, so ext=1 lists are empty.
uint64_t ref_pq_count(void* h, uint32_t cuboid, int ext) {
  auto* r = static_cast<PqResult*>(h);
  if (ext || cuboid == 0 || cuboid >= (1u << r->d)) return 0;
  return r->sky[cuboid].size();
}

void ref_pq_ids(void* h, uint32_t cuboid, int ext, uint32_t* out) {
  auto* r = static_cast<PqResult*>(h);
  if (ext || cuboid == 0 || cuboid >= (1u << r->d)) return;
  const auto& v = r->sky[cuboid];
  std::memcpy(out, v.data(), v.size() * sizeof(uint32_t));
}

void ref_pq_free(void* h) { delete static_cast<PqResult*>(h); }

}  // extern "C"
