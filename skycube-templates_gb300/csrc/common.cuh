// Internal declarations shared by the CUDA translation units of the skycube
// engine. Nothing here is part of the C ABI (include/skycube_gb300.h).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <map>
#include <mutex>
#include <set>
#include <string>
#include <vector>

#include "skycube_gb300.h"

namespace skc {

// ---------------------------------------------------------------------------
// Errors: every internal function returns an int status and records a
// message for skc_last_error().
int set_error(int code, const char* fmt, ...);
void clear_error();
// SKC_ERR_INVALID unless p is device (or managed) memory that kernels on
// `device` can read: host memory passed by mistake fails here, not as an
// illegal address inside a kernel. Allocates nothing.
int check_device_pointer(const void* p, int device, const char* what);

#define SKC_TRY(expr)                   \
  do {                                  \
    int st_ = (expr);                   \
    if (st_ != SKC_OK) return st_;      \
  } while (0)

#define SKC_CUDA(call)                                                      \
  do {                                                                      \
    cudaError_t e_ = (call);                                                \
    if (e_ != cudaSuccess) {                                                \
      return ::skc::set_error(e_ == cudaErrorMemoryAllocation ? SKC_ERR_OOM \
                                                              : SKC_ERR_CUDA, \
                              "%s failed: %s (%s:%d)", #call,              \
                              cudaGetErrorString(e_), __FILE__, __LINE__);  \
    }                                                                       \
  } while (0)

// Every kernel launch of the library is followed by SKC_LAUNCH_CHECK, which
// also counts it (skc_kernel_launches).
void count_launch();
#define SKC_LAUNCH_CHECK()       \
  do {                           \
    ::skc::count_launch();       \
    SKC_CUDA(cudaGetLastError()); \
  } while (0)

// ---------------------------------------------------------------------------
// Grid cells. Every attribute value v is mapped to cell(v) = number of
// pivots strictly below v, with 2^depth - 1 pivots (depth <= 7, so a cell
// fits in 7 bits). cell is monotone: cell(a) < cell(b) implies a < b and
// cell(a) > cell(b) implies a > b; equal cells decide nothing. The cells of
// one point are packed four per 32-bit word, attribute k in byte k % 4 of
// word k / 4, so d <= 16 attributes fit one uint4.
constexpr uint32_t kGuard = 0x80808080u;  // bit 7 of every byte
constexpr int kMaxDepth = 7;

// Bytes of `a` (each < 128) compared with bytes of `b`: bit 7 of byte j of
// the result is set iff a_j >= b_j. `a_or_guard` must be a | kGuard.
__host__ __device__ __forceinline__ uint32_t ge_bytes(uint32_t a_or_guard,
                                                      uint32_t b) {
  return (a_or_guard - b) & kGuard;
}

// Compresses the guard bits (7, 15, 23, 31) of g into bits 0..3.
__host__ __device__ __forceinline__ uint32_t pack_guards(uint32_t g) {
  return (g * 0x00204081u) >> 28;
}

// Guard-bit mask of the attributes of subspace S that live in word w.
__host__ __device__ __forceinline__ uint32_t guard_mask(uint32_t S, int w) {
  uint32_t m = 0;
  for (int j = 0; j < 4; ++j)
    if (S & (1u << (4 * w + j))) m |= 0x80u << (8 * j);
  return m;
}

__host__ __device__ __forceinline__ uint32_t word_of(const uint4& v, int w) {
  return w == 0 ? v.x : (w == 1 ? v.y : (w == 2 ? v.z : v.w));
}

}  // namespace skc

// Opaque handle types of the C ABI.
struct skc_context {
  int device = 0;
  int num_sms = 0;
  cudaStream_t stream = nullptr;
  cudaEvent_t ev_start = nullptr, ev_stop = nullptr;
  float last_ms = 0.f;
  cudaMemPool_t pool = nullptr;
  uint32_t* d_level_tables[11] = {};  // partition tables per B (see partition.cu)
  // Live objects created from this context; destroying the context frees
  // their device memory and detaches them (ctx = nullptr).
  std::set<skc_dataset*> datasets;
  std::set<skc_result*> results;
  std::set<skc_plan*> plans;
  // Per-phase device times of the last skc_skycube.
  std::vector<std::pair<std::string, float>> phases;
  // Host id buffers of freed results, reused by later downloads: a fresh
  // buffer costs its zero fill and first-touch page faults (about 3 ms for
  // the 65 MB of a 1M x 10 skycube, eight times the copy itself).
  std::vector<std::vector<uint32_t>> host_id_pool;
  // Work parameters chosen by skc_autotune, by signature key (api.cu).
  struct Tuned {
    int depth, pq_size, tile_points, chunk, blocks_per_sm;
    float ms;
  };
  std::map<uint64_t, Tuned> tunings;
  // Guards the table caches and the object registries (the serving loop
  // runs pipelines from several host threads).
  std::mutex mu;
};

struct skc_dataset {
  skc_context* ctx = nullptr;
  cudaStream_t stream = nullptr;  // stream its memory was allocated on
  uint64_t n = 0;
  uint64_t n_pad = 0;  // n rounded up to a multiple of 128
  int d = 0;
  float* x = nullptr;  // attribute-major (SoA): x[k * n_pad + i]
  // Distribution signature from a point sample, computed on first use
  // (guarded by the context's mutex): sample size, sample points on the
  // sample's own skyline, sample points sharing a value with another.
  bool sig_ready = false;
  uint32_t sig_samples = 0, sig_sky = 0, sig_tied = 0;
};

struct skc_result {
  skc_context* ctx = nullptr;
  cudaStream_t stream = nullptr;  // stream later device work on it goes to
  int d = 0;
  int max_d = 0;
  int algo = 0;
  uint64_t n_cand = 0;
  uint64_t total_ids = 0;
  int form = 0;             // SKC_FORM_*
  int level_fallbacks = 0;  // SKC_FORM_LEVELS: cuboids over the kernel's capacities
  // Device CSR of skylines and (optionally) extended skylines, indexed by
  // cuboid mask: ids of c are ids[off[c] .. off[c+1]).
  uint64_t* d_off = nullptr;
  uint32_t* d_ids = nullptr;
  uint64_t* d_eoff = nullptr;
  uint32_t* d_eids = nullptr;
  uint64_t total_ext = 0;
  // Per-point bitmaps (MDMC) and the candidate ids they belong to.
  uint32_t* d_bits = nullptr;
  uint32_t* d_cand = nullptr;
  uint32_t words = 0;
  // Host mirrors, filled on demand.
  bool downloaded = false, ext_downloaded = false, bits_downloaded = false;
  std::vector<uint64_t> h_off, h_eoff;
  std::vector<uint32_t> h_ids, h_eids, h_bits, h_cand;
};
