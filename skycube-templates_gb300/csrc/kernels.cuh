// Launch helpers of the skycube engine's kernels (internal).
#pragma once

#include "common.cuh"

namespace skc {

constexpr int kMaxDims = 16;
constexpr int kMaxPivots = 127;  // 2^kMaxDepth - 1

// Scratch of the counting sort by bucket (all device pointers).
struct BucketScratch {
  float* f = nullptr;        // [m_max] scores
  uint32_t* keys = nullptr;  // [m_max]
  uint32_t* counts = nullptr;  // [K + 1]
  uint32_t* cursor = nullptr;  // [K + 1]
  uint32_t* minmax = nullptr;  // [2]
};

// prep.cu
int launch_rows_to_soa(cudaStream_t s, const float* rows, uint64_t n, int d,
                       uint64_t n_pad, float* x, uint32_t* bad);
int launch_iota(cudaStream_t s, uint32_t* out, uint64_t n);
int launch_bucket_order(cudaStream_t s, const float* x, uint64_t n_pad, int d,
                        const uint32_t* ids, const uint32_t* m_ptr,
                        uint64_t m_max, uint32_t S, uint32_t K,
                        const BucketScratch& b, uint32_t* sorted, uint32_t* hi);
int launch_counting_sort(cudaStream_t s, const uint32_t* keys,
                         const uint32_t* m_ptr, uint64_t m_max, uint32_t K,
                         const BucketScratch& b, uint32_t* sorted, uint32_t* hi);
int launch_pivots_cells(cudaStream_t s, const float* x, uint64_t n_pad, int d,
                        const uint32_t* ids, const uint32_t* m_ptr,
                        uint64_t m_max, int depth, float* pivots, uint4* cells,
                        unsigned long long* spread = nullptr);
int launch_status_compact(cudaStream_t s, const uint8_t* st, const uint32_t* ids,
                          const uint32_t* m_ptr, uint64_t m_max, int merge01,
                          uint32_t* blk0, uint32_t* blk1, uint32_t* out0,
                          uint32_t* out1, uint32_t* n0, uint32_t* n1);
int launch_scan_single_u32(cudaStream_t s, uint32_t* a, uint32_t len);
int launch_scan_u32_to_u64(cudaStream_t s, const uint32_t* in, uint64_t len,
                           uint64_t* bsum, uint64_t* out);
uint64_t scan_bsum_entries(uint64_t len);
int launch_gather_soa(cudaStream_t s, const float* x, uint64_t n_pad, int d,
                      const uint32_t* ids, const uint32_t* m_ptr, uint64_t m_max,
                      uint64_t out_pad, float* out);
int launch_gather_u4(cudaStream_t s, const uint4* in, const uint32_t* perm,
                     const uint32_t* m_ptr, uint64_t m_max, uint4* out);
int launch_block_min(cudaStream_t s, const uint4* cells, const uint32_t* m_ptr,
                     uint64_t m_max, uint4* bmin, uint4* smin, uint4* hmin);
int launch_csr_gather(cudaStream_t s, const uint32_t* const* srcs,
                      const uint64_t* dst_off, uint32_t ncub, uint32_t* dst);
int launch_set_u32(cudaStream_t s, uint32_t* p, uint32_t v);
int launch_merge_disjoint(cudaStream_t s, const uint32_t* a, uint32_t na,
                          const uint32_t* b, uint32_t nb, uint32_t* out);
int launch_gather_u32(cudaStream_t s, const uint32_t* in, const uint32_t* perm,
                      const uint32_t* m_ptr, uint64_t m_max, uint32_t* out);
int launch_member_flags(cudaStream_t s, const uint32_t* list, const uint32_t* m_ptr,
                        uint64_t m_max, const uint32_t* sorted_set, const uint32_t* nset_ptr,
                        uint8_t* st);
int launch_pad_q(cudaStream_t s, const uint32_t* mq_ptr, int d, uint4* qc, float* qx,
                 uint64_t pitch);
int launch_sample_signature(cudaStream_t s, const float* x, uint64_t n_pad, uint64_t n, int d,
                            uint32_t* out);
int launch_cap_count(cudaStream_t s, uint32_t* m_ptr, uint32_t cap, uint64_t* stats, int slot);
int launch_stat_u64(cudaStream_t s, const uint64_t* src, uint64_t* stats, int slot);
int launch_csr_assemble(cudaStream_t s, const uint32_t* src,
                        const uint64_t* src_off, const uint64_t* dst_off,
                        uint32_t ncub, uint32_t* dst);

// skyline.cu: status of every list entry on subspace S (0 skyline,
// 1 extended skyline, 2 strictly dominated).
struct SkylineArgs {
  const uint32_t* sorted;  // sorted index -> list position (bucket order)
  const uint32_t* hi;      // sorted index -> end of its bucket
  const uint32_t* ids;     // list position -> point id (nullptr: identity)
  const uint4* cells;      // point id -> grid cells
  const float* x;          // attribute-major points
  uint64_t n_pad;
  const uint32_t* m_ptr;   // list length (device)
  uint64_t m_max;          // upper bound of the list length (host)
  uint32_t S;              // subspace mask
  uint8_t* status;         // list position -> status
};
int launch_skyline(cudaStream_t s, int d, const SkylineArgs& a);

// partition.cu: median-partition skyline (status as above).
// Lattice-level tables over B-bit masks (B <= 10): rank (popcount, then
// value), its inverse, and for every mask the ranks of its submasks in
// level order.
constexpr int kMaxPartitionDims = 10;
constexpr uint64_t kConfirmedMinPoints = 32768;
constexpr uint64_t kMaxSortBuckets = 1u << 18;  // partition x strength buckets
struct LevelTables {
  int B = 0;
  const uint32_t* rank = nullptr;      // [2^B]
  const uint32_t* unrank = nullptr;    // [2^B]
  const uint32_t* sub_off = nullptr;   // [2^B + 1]
  const uint32_t* sub_list = nullptr;  // [3^B]
};
struct PartScratch {
  uint32_t* keys;    // [m_max]
  uint32_t* sorted;  // [m_max]
  uint4* ccells;     // [m_max] compact cells in partition order
  float* cx;         // [|S| * round_up(m_max, 128)] compact floats
  // Confirmed lists (partition.cu), used for lists of at least
  // kConfirmedMinPoints points; nullptr disables them.
  uint4* conf_cells = nullptr;  // [m_max]
  float* conf_x = nullptr;      // [|S| * round_up(m_max, 128)]
  uint32_t* ccount = nullptr;   // [2^B]
  uint32_t* pdone = nullptr;    // [2^B]
  uint32_t* counts;  // [2^B + 1] partition offsets after the sort
  uint32_t* fine;    // [kMaxSortBuckets + 1] counting-sort offsets
  uint32_t* cursor;  // [kMaxSortBuckets + 1]
  uint32_t* items;   // [2^B + 1]
  // Spread of the cell sums of the list before the prefilter (sum, sum of
  // squares, count), for sliced lists; nullptr: strength order, no tile box.
  // Zeroed by k_pivots and filled by k_cells when launch_pivots_cells is
  // given it.
  unsigned long long* spread = nullptr;  // [3]
};
struct PartitionSkylineArgs {
  const uint32_t* ids;  // list position -> point id (nullptr: identity)
  const uint4* cells;   // point id -> grid cells
  const float* x;
  uint64_t n_pad;
  const uint32_t* m_ptr;
  uint64_t m_max;
  uint32_t S;
  uint8_t* status;      // list position -> status; m_max rounded up to 4 bytes
  uint32_t split_target = 0;  // CTAs the skyline kernel's work is cut into (0: no slicing)
  // Sliced lists: the list whose cell-sum spread picks the order inside the
  // partitions (point ids, nullptr: 0 .. count - 1; count on the device).
  const uint32_t* spread_ids = nullptr;
  const uint32_t* spread_m = nullptr;
  bool spread_ready = false;  // PartScratch::spread already holds the spread
};
// Skyline kernel: CTAs per SM the work is balanced over (split_target).
constexpr uint32_t kSplitCtasPerSm = 32;
int launch_mask_keys(cudaStream_t s, const uint4* cells, const uint32_t* ids,
                     const uint32_t* m_ptr, uint64_t m_max, uint32_t S, int d,
                     int B, int depth, int sub_bits, int sub_mode, const uint32_t* rank,
                     uint32_t* keys);
int launch_partition_offsets(cudaStream_t s, const uint32_t* fine, uint32_t K, int sub_bits,
                             uint32_t* boff);
int launch_partition_skyline(cudaStream_t s, int d, int depth,
                             const LevelTables& T, const PartitionSkylineArgs& a,
                             const PartScratch& ps);

// prefilter.cu: pruner prefilter of a list on subspace S. Survivors (the
// entries no pruner strictly dominates) come out as point ids in list order.
constexpr int kMaxPruners = 1024;
struct PrefilterScratch {
  uint32_t* hist;      // [prefilter_sum_bins()]
  uint32_t* sel;       // [8]
  uint32_t* pr_ids;    // [K]
  uint32_t* pr_key;    // [K]
  uint4* pr_cells;     // [K] pruner cells, rank order
  float* pr_x;         // [d * K] pruner floats, rank order
  uint8_t* st;         // [m_max]
  uint32_t* blk0;      // [m_max / 1024 + 1]
  uint32_t* blk1;      // [m_max / 1024 + 1]
  uint32_t* mid_ids;   // [m_max] survivors of the first pass
  uint32_t* mid_count; // [1]
};
struct PrefilterArgs {
  const uint4* cells;    // point id -> grid cells
  const float* x;        // attribute-major points, pitch n_pad
  uint64_t n_pad;
  const uint32_t* ids;   // list position -> point id (nullptr: identity)
  const uint32_t* m_ptr;
  uint64_t m_max;
  uint32_t S;
  uint32_t K;            // pruners, 1 .. kMaxPruners
  PrefilterScratch ps;
};
int launch_prefilter(cudaStream_t s, int d, int num_sms, const PrefilterArgs& a,
                     uint32_t* out_ids, uint32_t* out_count);
uint32_t prefilter_sum_bins();
size_t prefilter_smem(int d, uint32_t K);

// mdmc.cu: per-point dominated-subspace bitmaps over the candidate set.
struct BitmapArgs {
  const uint4* pcells;   // candidate order
  const float* px;       // candidate order, attribute-major, pitch p_pad
  uint64_t p_pad;
  const uint4* qcells;   // q order (level-sorted), padded to whole 32-q blocks
  const float* qx;       // q order, attribute-major, pitch p_pad
  const uint4* bmin;     // per block of 32 q's: byte-wise minimum cells
  const uint4* smin;     // the same per 8-q sub-block (4 per block)
  const uint4* hmin;     // the same per 4-q half of a sub-block (8 per block)
  const uint32_t* boff;  // q partitions: offsets in q order [K + 1]
  const uint32_t* unrank;  // partition rank -> median mask over B attributes
  uint32_t K;
  int B;
  int depth;
  const uint32_t* m_ptr;   // candidates (p's)
  uint32_t* work;        // work counter, must hold p_begin
  uint32_t chunk;        // candidates per work-counter grab (0: 1)
  uint32_t p_end;        // stop at min(m, p_end)
  uint32_t* out_dom;     // [m][words] dominated bitmaps
  uint32_t* out_ext;     // [m][words] extended-skyline bitmaps, or nullptr
  int grid_blocks;       // persistent grid (0: from occupancy)
  uint32_t* tie_slab;    // global tie maps (bitmap_tie_slab_words), or nullptr
  // Capped skycubes: only the bits of subspaces with at most `cap`
  // attributes and of the full space are exact (1 <= cap <= d - 2; 0: all
  // bits). The full-space bits then come from full_dom (per candidate,
  // nonzero when it is dominated on the full space).
  int cap = 0;
  const uint8_t* full_dom = nullptr;
};
int launch_bitmaps(cudaStream_t s, int d, int num_sms, const BitmapArgs& a);
int bitmap_tie_slab_words(int d, int num_sms, uint64_t* words);

struct CompactArgs {
  const uint32_t* bits;  // [m][words]
  uint32_t words;
  const uint32_t* m_ptr;
  uint64_t m_max;
  int count_set;         // 0: rows with the bit CLEAR (skyline); 1: SET
  uint32_t nsub;         // 2^d
  int max_d;
  const uint32_t* cand;  // row -> point id
  uint32_t* counts;      // [32*words * tiles]
  uint64_t* offs;        // [32*words * tiles + 1]
  uint64_t* bsum;        // scan scratch
  uint64_t* csr_off;     // [nsub + 1] output offsets per cuboid
  uint32_t* out;         // ids (sized by the caller after the count pass)
  uint64_t out_cap;      // entries of `out`; ids past it are not written
};
uint32_t compact_tiles(uint64_t m_max);
int launch_bits_count(cudaStream_t s, const CompactArgs& a);
int launch_bits_write(cudaStream_t s, const CompactArgs& a);

// levels.cu: capped skycubes by lattice level (cuboids of at most
// kLvMaxDims attributes), one CTA per cuboid for the sort-filter skyline.
constexpr int kLvMaxDims = 4;
constexpr uint32_t kLvPruners = 32;    // per cuboid, from a strided sample
constexpr uint32_t kLvSample = 1024;   // sampled list entries
constexpr uint32_t kLvChunk = 8192;    // list entries per filter item (staged in shared memory)
constexpr uint32_t kLvThreads = 1024;  // sort-filter CTA, one batch per pass
constexpr uint32_t kLvWin = 2048;      // skyline points per cuboid
constexpr uint32_t kLvExt = 4096;      // extended-skyline points per cuboid
constexpr uint32_t kLvSlot = kLvWin + kLvExt;  // output ids per cuboid
constexpr uint32_t kLvSortCap = 8192;  // power of two >= kLvSlot
constexpr uint32_t kLvKeyBins = 127 * kLvMaxDims + 1;  // cell sums
// One dataset of a lattice launch.
struct LtJob {
  const float* x;            // attribute-major points, pitch n_pad
  uint64_t n_pad;
  const uint4* cells;        // point id -> cells on the candidates' quantile grid
  const uint32_t* cand;      // full-space skyline + extended skyline ids
  uint32_t n_cand;
  const uint32_t* cub_index; // [2^d] mask -> cuboid table index (0xffffffff: none)
  int d, max_d;
};
// A lattice launch (levels.cu, k_lattice): every wanted cuboid of every job
// (cuboid table index c) from a device work queue in lattice-level order.
struct LtArgs {
  const LtJob* jobs;
  const uint32_t* c_mask;    // [ncub]
  const uint32_t* c_job;     // [ncub]
  const uint32_t* c_scr;     // [ncub] scratch index in the cuboid's group
  const uint32_t** c_list;   // [ncub] candidate list (set by phase P)
  uint32_t* c_list_n;        // [ncub]
  uint32_t* c_nsky;          // [ncub] outputs of phase S
  uint32_t* c_next;          // [ncub]
  uint32_t* c_flag;          // [ncub] 1: over a capacity; 2: skipped (job handed over)
  uint32_t* slot;            // [ncub * kLvSlot]: skyline ids, then extended
  uint32_t* pr_c;            // [G * kLvPruners] per scratch index
  float* pr_v;               // [G * kLvMaxDims * kLvPruners]
  uint32_t* pr_n;            // [G]
  uint32_t cap;              // survivors kept per cuboid
  uint32_t* cnt;             // [G]
  uint32_t* surv_id;         // [G * cap]
  uint16_t* surv_key;        // [G * cap]
  uint32_t* srt;             // [G * cap]
  uint32_t n_items;
  const uint32_t* it_cub;    // [n_items]
  const uint32_t* it_arg;    // [n_items] phase F: slice | slices << 16
  const uint32_t* it_phase;  // [n_items]
  const uint32_t* ph_size;   // [n_phases] items per phase
  const uint8_t* ph_kind;    // [n_phases] 0 P, 1 F, 2 S
  uint32_t* ph_done;         // [n_phases] zeroed before the launch
  uint32_t* next_item;       // zeroed before the launch
  uint32_t* job_over;        // [jobs] first-level cuboids over a capacity (zeroed)
  uint32_t max_fallbacks;    // more than this on a job's first level: job handed over
  uint32_t* status;          // 0, or 1 when a wait ran out (zeroed)
};
// One cooperative launch of the lattice kernel on `num_sms` SMs.
int launch_lattice(cudaStream_t s, int num_sms, const LtArgs& a);
int lattice_grid(int num_sms, int* grid);
int launch_scatter_u4(cudaStream_t s, const uint4* in, const uint32_t* idx, const uint32_t* m_ptr,
                      uint64_t m_max, uint4* out);

void upload_submask_table();

}  // namespace skc
