// C entry points around the reference's own STSC skycube (HybridCube<D>,
// src/stsc/HybridCube.cpp:108-214), the suite's "-c" ground truth
// (src/main.h:125-146). Compiled against the reference sources in place by
// oracle/build_ref.sh; the result is test infrastructure only.
#include <cstdint>
#include <cstring>
#include <vector>
#include "stsc/HybridCube.h"

namespace {

struct RefResult {
  int d;
  std::vector<std::vector<unsigned>> sky;  // indexed by cuboid mask
  std::vector<std::vector<unsigned>> ext;
};

template <int D>
RefResult* run(const float* rows, uint32_t n, int max_d, int threads,
               int alpha, int pq) {
  float** data = new float*[n];
  for (uint32_t i = 0; i < n; ++i) {
    data[i] = new float[D];
    std::memcpy(data[i], rows + (size_t)i * D, sizeof(float) * D);
  }
  auto* cube = new HybridCube<D>(n, threads, alpha, pq, max_d);
  cube->Init(data);
  cube->Execute();
  auto* res = new RefResult;
  res->d = D;
  res->sky.resize(1u << D);
  res->ext.resize(1u << D);
  lattice_node* lat = cube->getLattice();
  for (uint32_t s = 1; s < (1u << D); ++s) {
    res->sky[s] = lat[s].skyline;
    res->ext[s] = lat[s].extended_sky;
  }
  delete cube;
  for (uint32_t i = 0; i < n; ++i) delete[] data[i];
  delete[] data;
  return res;
}

}  // namespace

extern "C" {

// Runs STSC with the suite's defaults for alpha (1024) and pq (128) when the
// caller passes 0. Returns an opaque handle or nullptr for an unsupported d.
void* ref_stsc_run(const float* rows, uint32_t n, int d, int max_d,
                   int threads, int alpha, int pq) {
  if (alpha <= 0) alpha = 1024;
  if (pq <= 0) pq = 128;
  if (max_d <= 0) max_d = d;
  switch (d) {
#define CASE(D) case D: return run<D>(rows, n, max_d, threads, alpha, pq);
    CASE(2) CASE(3) CASE(4) CASE(5) CASE(6) CASE(7) CASE(8) CASE(9)
    CASE(10) CASE(11) CASE(12) CASE(13) CASE(14) CASE(15) CASE(16)
#undef CASE
    default: return nullptr;
  }
}

uint64_t ref_stsc_count(void* h, uint32_t cuboid, int ext) {
  auto* r = static_cast<RefResult*>(h);
  if (cuboid == 0 || cuboid >= (1u << r->d)) return 0;
  return ext ? r->ext[cuboid].size() : r->sky[cuboid].size();
}

// Copies the ids of one cuboid's skyline (ext=0) or extended skyline (ext=1).
void ref_stsc_ids(void* h, uint32_t cuboid, int ext, uint32_t* out) {
  auto* r = static_cast<RefResult*>(h);
  if (cuboid == 0 || cuboid >= (1u << r->d)) return;
  const auto& v = ext ? r->ext[cuboid] : r->sky[cuboid];
  std::memcpy(out, v.data(), v.size() * sizeof(uint32_t));
}

void ref_stsc_free(void* h) { delete static_cast<RefResult*>(h); }

}  // extern "C"
