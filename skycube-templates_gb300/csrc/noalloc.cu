// Allocation-free skyline of one subspace: skc_skyline_noalloc.
//
// Some callers cannot allocate device memory at all: code running inside a
// memory budget that another runtime owns (a database or serving process
// whose allocator has claimed the GPU's memory up front), plugins that must
// not touch the device heap, or tools that run where cudaMalloc is forbidden
// after start-up. This entry point serves them. The caller passes device
// buffers for the points and for the per-point result; every temporary the
// computation needs lives in one file-scope device array that is part of the
// library image, so the call itself allocates nothing.
//
// The scratch array is sized for at most kNoAllocMaxPoints points of up to
// 16 attributes (about 6.3 MiB). Every GPU that loads this library holds that
// array until the process exits.
//
// Host code cannot use the array's name as a device address: on the host the
// symbol is only a stand-in. Every call therefore asks the runtime for the
// array's address in the current device's context (cudaGetSymbolAddress,
// which allocates nothing) before it launches anything, so a context that
// was reset or replaced since an earlier call never leaves a stale address.
// The first call on a device also loads this library's kernels there; make
// that first call before any stream capture. All calls share the one array,
// which keeps whatever the previous call left in it: the pipeline clears the
// counters it needs before use, and calls whose work overlaps on the GPU
// (different streams, or different host threads on one device) race on the
// array and must be serialised by the caller. The call is synchronous: it
// waits on its stream and returns once the statuses are in d_status.
#include "kernels.cuh"

namespace skc {

constexpr uint32_t kNoAllocMaxPoints = 65536;
constexpr uint32_t kNoAllocMaxBuckets = kNoAllocMaxPoints / 4;

// Byte layout of the scratch array (every piece 256-byte aligned).
constexpr size_t al256(size_t b) { return (b + 255) / 256 * 256; }
constexpr size_t kOffX = 0;  // attribute-major points: 16 x max floats
constexpr size_t kOffCells = kOffX + al256(sizeof(float) * kMaxDims * kNoAllocMaxPoints);
constexpr size_t kOffF = kOffCells + al256(sizeof(uint4) * kNoAllocMaxPoints);
constexpr size_t kOffKeys = kOffF + al256(sizeof(float) * kNoAllocMaxPoints);
constexpr size_t kOffSorted = kOffKeys + al256(sizeof(uint32_t) * kNoAllocMaxPoints);
constexpr size_t kOffHi = kOffSorted + al256(sizeof(uint32_t) * kNoAllocMaxPoints);
constexpr size_t kOffCounts = kOffHi + al256(sizeof(uint32_t) * kNoAllocMaxPoints);
constexpr size_t kOffCursor = kOffCounts + al256(sizeof(uint32_t) * (kNoAllocMaxBuckets + 1));
constexpr size_t kOffPivots = kOffCursor + al256(sizeof(uint32_t) * (kNoAllocMaxBuckets + 1));
constexpr size_t kOffSmall = kOffPivots + al256(sizeof(float) * kMaxDims * kMaxPivots);
constexpr size_t kNoAllocScratchBytes = kOffSmall + 256;  // minmax[2], n, bad

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

// Device address of g_noalloc_scratch in the current context.
static int noalloc_scratch(unsigned char** out) {
  void* p = nullptr;
  cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
  if (e != cudaSuccess || !p)
    return set_error(SKC_ERR_CUDA, "cudaGetSymbolAddress of the scratch array failed: %s",
                     cudaGetErrorString(e));
  *out = static_cast<unsigned char*>(p);
  return SKC_OK;
}

}  // namespace skc

using namespace skc;

extern "C" int skc_skyline_noalloc(const float* d_rows, uint32_t n, int d,
                                   uint32_t subspace, int depth,
                                   uint8_t* d_status, void* stream) {
  clear_error();
  if (!d_rows || !d_status) return set_error(SKC_ERR_INVALID, "NULL device buffer");
  if (d < SKC_MIN_DIMS || d > SKC_MAX_DIMS)
    return set_error(SKC_ERR_INVALID, "d=%d outside [%d,%d]", d, SKC_MIN_DIMS, SKC_MAX_DIMS);
  if (n == 0) return set_error(SKC_ERR_INVALID, "empty point set (n=0)");
  if (n > kNoAllocMaxPoints)
    return set_error(SKC_ERR_UNSUPPORTED,
                     "n=%u exceeds the allocation-free limit of %u points; use skc_skycube",
                     n, kNoAllocMaxPoints);
  if (subspace == 0 || (d < 32 && subspace >= (1u << d)))
    return set_error(SKC_ERR_INVALID, "subspace 0x%x is not a non-empty subset of %d attributes",
                     subspace, d);
  if (depth == 0) depth = kMaxDepth;
  if (depth < 1 || depth > kMaxDepth)
    return set_error(SKC_ERR_INVALID, "depth %d outside [1,%d] (0 = default)", depth, kMaxDepth);

  int device = 0;
  SKC_CUDA(cudaGetDevice(&device));
  SKC_TRY(check_device_pointer(d_rows, device, "d_rows"));
  SKC_TRY(check_device_pointer(d_status, device, "d_status"));
  unsigned char* base = nullptr;
  SKC_TRY(noalloc_scratch(&base));
  cudaStream_t s = static_cast<cudaStream_t>(stream);

  const uint64_t n_pad = (n + 127) / 128 * 128;
  float* x = reinterpret_cast<float*>(base + kOffX);
  uint4* cells = reinterpret_cast<uint4*>(base + kOffCells);
  BucketScratch b;
  b.f = reinterpret_cast<float*>(base + kOffF);
  b.keys = reinterpret_cast<uint32_t*>(base + kOffKeys);
  b.counts = reinterpret_cast<uint32_t*>(base + kOffCounts);
  b.cursor = reinterpret_cast<uint32_t*>(base + kOffCursor);
  uint32_t* small = reinterpret_cast<uint32_t*>(base + kOffSmall);
  b.minmax = small;  // [0], [1]
  uint32_t* d_n = small + 2;
  uint32_t* bad = small + 3;
  uint32_t* sorted = reinterpret_cast<uint32_t*>(base + kOffSorted);
  uint32_t* hi = reinterpret_cast<uint32_t*>(base + kOffHi);
  float* pivots = reinterpret_cast<float*>(base + kOffPivots);

  uint32_t K = n / 4;
  if (K < 64) K = 64;
  if (K > kNoAllocMaxBuckets) K = kNoAllocMaxBuckets;

  SKC_CUDA(cudaMemsetAsync(bad, 0, sizeof(uint32_t), s));
  SKC_TRY(launch_set_u32(s, d_n, n));
  SKC_TRY(launch_rows_to_soa(s, d_rows, n, d, n_pad, x, bad));
  SKC_TRY(launch_pivots_cells(s, x, n_pad, d, nullptr, d_n, n, depth, pivots, cells));
  SKC_TRY(launch_bucket_order(s, x, n_pad, d, nullptr, d_n, n, subspace, K, b, sorted, hi));
  SkylineArgs a{sorted, hi, nullptr, cells, x, n_pad, d_n, n, subspace, d_status};
  SKC_TRY(launch_skyline(s, d, a));

  uint32_t h_bad = 0;
  SKC_CUDA(cudaMemcpyAsync(&h_bad, bad, sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
  SKC_CUDA(cudaStreamSynchronize(s));
  if (h_bad)
    return set_error(SKC_ERR_INVALID, "%u non-finite attribute values (NaN/inf) rejected; statuses are undefined", h_bad);
  return SKC_OK;
}
