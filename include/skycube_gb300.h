/*
 * skycube_gb300.h -- C ABI of the GB300 skycube engine.
 *
 * A skycube is the skyline of every non-empty subspace ("cuboid") S of an
 * n x d float32 point set, smaller being better on every attribute. Point q
 * dominates p on S iff q[k] <= p[k] for all k in S and q[k] < p[k] for some
 * k in S; q strictly dominates p iff q[k] < p[k] for all k in S. The skyline
 * of S holds the points nobody dominates on S; the extended skyline holds the
 * dominated points nobody strictly dominates. Point ids are row indices of
 * the input, cuboid ids are bitmasks (bit k = attribute k).
 *
 * The entry points replace the suite's single-GPU MDMC and SDSC paths:
 *   skc_dataset_upload  -> MDMC<D>::Init / SDSC<D>::Init
 *                          (src/mdmc/MDMC.cu:183-236, src/sdsc/SDSC.cu:28-58)
 *                          plus initializeGpu's H2D copy
 *                          (src/mdmc/MDMC.cu:1060-1084, src/sdsc/SDSC.cu:208-227)
 *   skc_skycube         -> MDMC<D>::Execute (src/mdmc/MDMC.cu:524-616) and
 *                          SDSC<D>::Execute (src/sdsc/SDSC.cu:248-335), with
 *                          run_skyalign (src/sdsc/skyAlign.cu:9-53) inside
 *   skc_result_cuboid   -> lattice_node::skyline of SDSC<D>::getLattice
 *                          (src/sdsc/SDSC.h:39, src/utilities/
 *                          lattice_utilities.h:21-31) and getsubspace over
 *                          MDMC<D>::getHashCubeStructure (src/mdmc/MDMC.h:62,
 *                          src/utilities/utilities.h:253-267)
 *   skc_result_extended -> lattice_node::extended_sky
 *   skc_result_bitmaps  -> the per-point dominated-subspace bitmaps that
 *                          feed HashCube<D>::populateFromSingleNodeAux
 *                          (src/skycube/Hashcube.h:107-115)
 *
 * Conventions: every call returns an int status (SKC_OK == 0) and never
 * exits the process; skc_last_error() gives a one-line message for the
 * calling thread. Objects created from one context must be used from one
 * host thread at a time.
 */
#ifndef SKYCUBE_GB300_H_
#define SKYCUBE_GB300_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Status codes. */
#define SKC_OK 0
#define SKC_ERR_INVALID 1     /* bad argument: d out of range, NULL, non-finite value */
#define SKC_ERR_CUDA 2        /* a CUDA runtime call failed */
#define SKC_ERR_OOM 3         /* device or host allocation failed */
#define SKC_ERR_TIMEOUT 4     /* a device-side wait ran out of iterations */
#define SKC_ERR_UNSUPPORTED 5 /* request outside what this build supports */
#define SKC_ERR_REJECTED 6    /* admission refused the request (memory budget) */

/* Limits. */
#define SKC_MIN_DIMS 2
#define SKC_MAX_DIMS 16

/* Algorithms (the suite's -s values "mdmc" and "sdsc"). Both return the
 * per-cuboid skylines; MDMC also exposes per-point bitmaps, SDSC also
 * exposes per-cuboid extended skylines. */
#define SKC_ALGO_MDMC 0
#define SKC_ALGO_SDSC 1

/* Execution forms. PLAIN issues one launch sequence per cuboid with a host
 * round trip after each (the suite's SDSC shape; for MDMC, one bitmap launch
 * per batch of points as in tombstoning_hearting_gpu). BATCHED computes all
 * cuboids in one persistent launch with no host synchronisation until the
 * result is read. */
#define SKC_MODE_PLAIN 0
#define SKC_MODE_BATCHED 1

typedef struct skc_context skc_context;
typedef struct skc_dataset skc_dataset;
typedef struct skc_result skc_result;
typedef struct skc_plan skc_plan;

typedef struct skc_options {
  int algo;        /* SKC_ALGO_* */
  int mode;        /* SKC_MODE_* */
  int max_d;       /* only cuboids with <= max_d attributes (-m); <= 0: all */
  int depth;       /* grid depth: 2^depth cells per attribute, 1..7; 0: auto (-d) */
  int want_extended; /* also produce per-cuboid extended skylines */
  int want_bitmaps;  /* keep per-point bitmaps for skc_result_bitmaps */
  uint32_t subspace; /* 0: the skycube; a cuboid mask: only that cuboid's
                        skyline and extended skyline (a skyline query) */
  /* Work parameters: they change the work done, never the result. 0 means
   * automatic: the value skc_autotune stored for datasets like this one
   * (same size class, d and distribution signature), else the default. */
  int pq_size;       /* pruners of the prefilter ahead of the full-space
                        skyline (-q; Config::pq_size, src/utilities/config.h:20):
                        > 0 that many, applied when n > 2 * pq_size as the
                        suite does (src/mdmc/MDMC.cu:251); < 0 off; 0 auto
                        (default 512 when n >= 32768). Applied in two
                        passes: the strongest pq_size / 16 on every point,
                        the rest on the survivors when at least a quarter
                        of the points survive */
  int tile_points;   /* bitmap kernel: mean q points per median partition
                        (a power of two, 32..65536); 0 auto (256) */
  int chunk;         /* bitmap kernel: candidates a warp takes per work-queue
                        grab, 1..64; 0 auto (1) */
  int blocks_per_sm; /* bitmap kernel: persistent CTAs per SM, 1..32 (capped
                        by occupancy); 0 auto (the occupancy limit) */
  int form;          /* computation of a batched skycube (SKC_FORM_*): 0 auto
                        (the level form from 65,536 candidates at caps under
                        4, at 16 attributes, or at 14-15 attributes from
                        600,000 candidates; else the bitmaps);
                        SKC_FORM_BITMAPS; SKC_FORM_LEVELS where it applies
                        (max_d <= 4 and <= d - 2, no per-point bitmaps; it
                        hands over to the bitmaps when too many cuboids
                        exceed its capacities). Never changes the result */
} skc_options;

/* Fills *opt with defaults: MDMC, BATCHED, all cuboids, automatic work
 * parameters. */
void skc_options_init(skc_options* opt);

/* Creates a context on CUDA device `device` (the -g value). */
int skc_context_create(int device, skc_context** out);
int skc_context_destroy(skc_context* ctx);

/* Copies n x d row-major float32 points from HOST memory to the device and
 * keeps them resident. Rejects d outside [2,16], n == 0 and non-finite
 * values. The caller keeps ownership of `rows`. */
int skc_dataset_upload(skc_context* ctx, const float* rows, uint64_t n, int d,
                       skc_dataset** out);
/* Same, from a DEVICE pointer on the context's device (no host copy). */
int skc_dataset_upload_device(skc_context* ctx, const float* d_rows,
                              uint64_t n, int d, skc_dataset** out);
int skc_dataset_free(skc_dataset* ds);

/* Computes the skycube of `ds`. Results stay on the device until a
 * skc_result_* accessor asks for host data. */
int skc_skycube(skc_context* ctx, skc_dataset* ds, const skc_options* opt,
                skc_result** out);

/* Skycubes of `count` resident datasets in one call; results[i] equals
 * skc_skycube(ctx, datasets[i], &opts[i]) (opts NULL: defaults). Every
 * dataset's full-space step runs first; then ONE persistent lattice launch
 * (SKC_FORM_LEVELS) carries the cuboids of all the datasets whose skycube
 * takes that form, and the other datasets take their own launches. The
 * serving loop batches waiting requests through it. No reference
 * counterpart (the suite computes one dataset per run). On error no result
 * is returned. */
int skc_skycube_batch(skc_context* ctx, skc_dataset* const* datasets,
                      const skc_options* opts, int count, skc_result** results);

/* Number of attributes of the result's dataset and number of candidate
 * points (full-space skyline plus extended skyline). */
/* Which computation produced the result (SKC_FORM_*), and for
 * SKC_FORM_LEVELS how many cuboids exceeded the level kernels' capacities
 * and went through the per-cuboid pipeline instead. No reference
 * counterpart (the suite's algorithm is chosen by -s). */
enum {
  SKC_FORM_BITMAPS = 1, /* per-point dominated-subspace bitmaps, one launch */
  SKC_FORM_CUBOIDS = 2, /* per cuboid, one launch sequence each (plain SDSC) */
  SKC_FORM_LEVELS = 3,  /* per cuboid, one lattice level per launch pair:
                           batched capped skycubes, max_d <= 4 and <= d - 2 */
  SKC_FORM_SKYLINE = 4  /* a single-subspace skyline query */
};
int skc_result_form(skc_result* res, int* form, int* fallbacks);

int skc_result_info(skc_result* res, int* d, uint64_t* n_candidates,
                    uint64_t* total_skyline_ids);

/* Host view of one cuboid's skyline ids (ascending). The pointer stays valid
 * until skc_result_free. Cuboids above max_d report count 0, except the full
 * space, which is always computed (as the suite does). */
int skc_result_cuboid(skc_result* res, uint32_t cuboid, const uint32_t** ids,
                      uint64_t* count);
/* Host view of one cuboid's extended skyline ids (needs want_extended). */
int skc_result_extended(skc_result* res, uint32_t cuboid,
                        const uint32_t** ids, uint64_t* count);
/* Device view of all skylines: ids of cuboid c are d_ids[d_offsets[c] ..
 * d_offsets[c+1]); offsets has 2^d + 1 entries. */
int skc_result_device_csr(skc_result* res, const uint64_t** d_offsets,
                          const uint32_t** d_ids);
/* Copies every cuboid's skyline to host memory in one go (CSR layout as
 * above); afterwards skc_result_cuboid is a pure host lookup. */
int skc_result_download(skc_result* res);
/* Host copy of the per-point dominated-subspace bitmaps (needs
 * want_bitmaps): point pids[i]'s bitmap is bits[i*words .. (i+1)*words),
 * bit (s % 32) of word s / 32 set iff the point is dominated in cuboid s.
 * words = max(1, 2^d / 32). */
int skc_result_bitmaps(skc_result* res, const uint32_t** bits,
                       const uint32_t** pids, uint64_t* n_points,
                       uint32_t* words);
int skc_result_free(skc_result* res);

/* ---- Serving loop (continuous batching) ---------------------------------
 * A server owns `slots` worker threads, each with a high- and a
 * low-priority CUDA stream (requests with n * 2^d >= 2^29 take the low
 * one). Submitted requests wait in FIFO order; the first one starts as soon
 * as a slot is free and its estimated device-memory footprint fits what the
 * requests in flight leave of `budget` (bytes; 0: 80% of the free device
 * memory). A capped skycube request that the level form takes (batched
 * form, max_d <= 4 and <= d - 2, no bitmaps; SKC_FORM_LEVELS, or the
 * automatic rule of skc_options.form with n for the candidate count) takes
 * such requests right behind it in the queue (up to 8, within the budget)
 * into the same pass (skc_skycube_batch), where those the level form takes
 * share one persistent lattice launch. Requests whose estimate exceeds the
 * whole budget are rejected
 * with SKC_ERR_REJECTED at submission. Requests that run at the same time
 * overlap on the device. Results come back in host memory (their device
 * views are empty). Host rows passed to skc_server_submit must stay valid
 * until skc_server_wait returns for that ticket. A server and its requests
 * may be used from several host threads. */
typedef struct skc_server skc_server;
typedef struct skc_server_timing {
  double queued_ms;  /* submission to admission */
  double run_ms;     /* admission to completion (upload, compute, copy out) */
  double total_ms;   /* submission to completion: the request's latency */
  float device_ms;   /* device time of the computation (CUDA events) */
} skc_server_timing;

int skc_server_create(skc_context* ctx, int slots, uint64_t budget,
                      skc_server** out);
/* Request on host rows (n x d row-major float32), uploaded by the server. */
int skc_server_submit(skc_server* srv, const float* rows, uint64_t n, int d,
                      const skc_options* opt, uint64_t* ticket);
/* Request on a dataset already resident on the server's context. */
int skc_server_submit_dataset(skc_server* srv, skc_dataset* ds,
                              const skc_options* opt, uint64_t* ticket);
/* Blocks until the request is done; hands its result to the caller. Each
 * ticket has one waiter: a second skc_server_wait on a ticket that is being
 * waited on, or was already collected, fails with SKC_ERR_INVALID. */
int skc_server_wait(skc_server* srv, uint64_t ticket, skc_result** out,
                    skc_server_timing* timing);
int skc_server_stats(skc_server* srv, uint64_t* admitted,
                     uint64_t* peak_in_flight, uint64_t* budget);
/* Batches the server ran (groups of requests that shared one lattice
 * launch: batched capped skycubes, SKC_FORM_LEVELS candidates, taken
 * together from the head of the queue when they arrive while the slots are
 * busy), requests served in them, and the largest batch. */
int skc_server_batch_stats(skc_server* srv, uint64_t* batches,
                           uint64_t* batched_requests, uint64_t* largest);
/* Waits for queued and running requests, then stops the workers. */
int skc_server_destroy(skc_server* srv);

/* ---- Plans: the batched launch sequence as one CUDA graph ----------------
 * skc_plan_create runs skc_skycube(ctx, ds, opt) once to learn the
 * candidate count and the id totals, allocates every buffer of the batched
 * pipeline once (25% above those sizes), and captures the whole launch
 * sequence (prefilter, full-space skyline, bitmap kernel, compaction, and
 * the copy of the totals to pinned host memory) into a CUDA graph with no
 * host synchronisation inside. skc_plan_execute replays it: one graph
 * launch and one host synchronisation, on the dataset's current points
 * (skc_dataset_update replaces them in place). When the points changed so
 * much that a capacity overflows, the plan re-sizes itself, captures again
 * and re-runs (counted by skc_plan_info). Only the BATCHED form of the
 * skycube is planned (opt->mode must be SKC_MODE_BATCHED, opt->subspace 0).
 * The result owns copies of the plan's outputs. A plan whose dataset was
 * freed fails with SKC_ERR_INVALID. */
int skc_plan_create(skc_context* ctx, skc_dataset* ds, const skc_options* opt,
                    skc_plan** out);
int skc_plan_execute(skc_plan* plan, skc_result** out);
/* Kernels per replay, re-plans so far, and the capacities in use. */
int skc_plan_info(skc_plan* plan, uint64_t* kernels, uint64_t* replans,
                  uint64_t* cand_capacity, uint64_t* ids_capacity);
int skc_plan_destroy(skc_plan* plan);

/* Replaces the points of a resident dataset in place from HOST rows (same
 * n and d, row-major float32); plans on it stay valid. Rows with non-finite
 * values are rejected (SKC_ERR_INVALID) and the dataset keeps its points. */
int skc_dataset_update(skc_dataset* ds, const float* rows);

/* ---- Autotuner -----------------------------------------------------------
 * Picks the work parameters (grid depth, prefilter pruners, bitmap tile,
 * queue chunk, CTAs per SM) for `ds` under the options in `base`: starting
 * from the defaults it times full runs on the device (CUDA events, the
 * minimum of `repeats` runs, 0: 2) in one pass of coordinate search over
 * the fields `base` leaves at 0, keeping a change when it is at least 2%
 * faster. The winner is stored in the context under the dataset's
 * signature key: its size class (floor(log2 n)), d, its distribution class
 * (skc_dataset_signature) and the options' algorithm, form, cuboid cap and
 * query kind. Later skc_skycube calls (and server requests) on datasets
 * with the same key use it for the fields they leave at 0. *best receives
 * `base` with every work field set to the chosen value (pq_size -1 when the
 * prefilter lost), *best_ms its device time. The suite picks its
 * partitioning depth by hand (-d); nothing there times alternatives. */
int skc_autotune(skc_context* ctx, skc_dataset* ds, const skc_options* base,
                 int repeats, skc_options* best, float* best_ms);
/* Distribution classes of a dataset, measured once on a strided sample of
 * up to 512 points: size_class = floor(log2 n); sky_class from the fraction
 * f of the sample on its own skyline on a two-sided log scale,
 * L(f) = floor(log2(1 + 1000 f)) for f <= 1/2 and 17 - L(1 - f) above, so
 * 0..17 (at d = 8: correlated ~4, independent ~9, anticorrelated ~13; at
 * high d independent and anticorrelated data both reach 17, and both have
 * nearly every point as a candidate); ties = 1 when at least 1/8 of the
 * sample shares an attribute value with another sample point. */
int skc_dataset_signature(skc_dataset* ds, int* size_class, int* sky_class,
                          int* ties);
/* Number of stored tunings; forgets them all. */
int skc_tuning_count(skc_context* ctx, uint64_t* count);
int skc_tuning_clear(skc_context* ctx);

/* Milliseconds of device time of the last skc_skycube on this context,
 * measured with CUDA events on the context's stream. */
int skc_last_device_ms(skc_context* ctx, float* ms);

/* Device time of one phase of the last skc_skycube on this context (CUDA
 * events on the context's stream): index 0, 1, ... until SKC_ERR_INVALID.
 * Phase names are stable strings such as "bitmap kernel". */
int skc_last_phase(skc_context* ctx, int index, const char** name, float* ms);

/* Number of kernels this library has launched in this process so far (all
 * contexts). A caller brackets a region with two reads to count launches. */
uint64_t skc_kernel_launches(void);

/* Allocation-free skyline of one subspace, for callers that cannot allocate
 * device memory (for example a host process whose own allocator already owns
 * the GPU's memory, or a plugin that may not touch the device heap). No
 * counterpart in the reference: it is an addition of this library.
 *
 * d_rows: n x d row-major float32 points in DEVICE memory; d_status: n bytes
 * of DEVICE memory that receive, per point, 0 (skyline of `subspace`),
 * 1 (extended skyline: dominated, never strictly) or 2 (strictly dominated).
 * depth: grid depth 1..7, 0 for the default. stream: a cudaStream_t (NULL for
 * the default stream); the call returns after the statuses are written.
 *
 * Limits: n <= 65536 points, 2 <= d <= 16. Larger inputs are rejected with
 * SKC_ERR_UNSUPPORTED before any device work. All temporaries live in one
 * static device array of about 6.3 MiB inside the library, held by every GPU
 * that loads it until the process exits; the call makes no allocation. The
 * first call on a device resolves that array's address (make it before any
 * stream capture). Calls share the array, so calls that overlap on the GPU
 * race and must be serialised by the caller. */
int skc_skyline_noalloc(const float* d_rows, uint32_t n, int d,
                        uint32_t subspace, int depth, uint8_t* d_status,
                        void* stream);

/* Message of the last failed call on this thread ("" if none). */
const char* skc_last_error(void);

#ifdef __cplusplus
}
#endif
#endif /* SKYCUBE_GB300_H_ */
