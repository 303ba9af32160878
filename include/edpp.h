/*
 * edpp.h — C ABI of the GB300 (sm_103a) data-parallel primitives.
 *
 * Every entry point is a drop-in for one primitive of Efficient-DPP's
 * primitive API (opencl/primitives.h:12-49) or of its CUDA/OpenMP test
 * programs, with the reference's argument order kept: input, output, length,
 * index array, pass count, bucket count.  Differences from the reference:
 *
 *   - buffers are caller-owned CUDA device pointers (the reference takes
 *     cl_mem handles); AOS key/value tuples are int32 pairs {key, value}
 *     (the reference's cl_int2 tuple_t, opencl/types.h:47);
 *   - calls are stream-ordered and asynchronous: they enqueue work on
 *     `stream` (a cudaStream_t passed as void*, NULL = legacy default stream)
 *     and return at once.  The reference calls clFinish after every launch
 *     and returns elapsed milliseconds; edpp_primitives.hpp restores that
 *     synchronous, time-returning form on top of this ABI;
 *   - errors are returned as an edpp_status code, never by exit()
 *     (the reference exits in checkErr, opencl/util/utility.cpp:85-90);
 *   - temporaries the reference allocates per call (d_inter, d_reduction,
 *     d_his: opencl/primitives/scanImpl.cpp:39,98, splitImpl.cpp:76,224) are
 *     a caller-provided workspace sized by the *_workspace_size queries, so
 *     nothing on the call path allocates;
 *   - device-side waits (look-back, work queues) are bounded.  A wait that
 *     runs out records EDPP_FAULT_TIMEOUT in a device fault word, the kernel
 *     returns, and edpp_sync_status() reports EDPP_ETIMEOUT.
 *
 * Thread safety: calls on distinct streams with distinct workspaces may be
 * issued from several host threads at once.  Two calls that share a
 * workspace must be ordered on one stream.
 */
#ifndef EDPP_H_
#define EDPP_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------- */
typedef enum {
    EDPP_OK = 0,
    EDPP_EINVAL = 1,   /* bad argument (reference: return -1 / 1)             */
    EDPP_ENOMEM = 2,   /* workspace too small or allocation failed            */
    EDPP_ETIMEOUT = 3, /* a bounded device-side wait expired                  */
    EDPP_ECUDA = 4     /* CUDA runtime error (launch, copy, sticky error)     */
} edpp_status;

/* Bits of the device fault word (edpp_device_fault). */
#define EDPP_FAULT_TIMEOUT 0x1u   /* look-back / dependency wait ran out    */
#define EDPP_FAULT_TMA     0x2u   /* a TMA transaction wait ran out         */
#define EDPP_FAULT_PLAN    0x4u   /* a batch task named a segment or tile
                                     outside the uploaded plan's tables     */

/* ---- enums mirroring the reference's types (opencl/types.h:8-47) -------- */

/* Global scan scheme.  LOOKBACK replaces the reference's chained
 * (adjacent-synchronisation) scan, RTS its reduce-scan-scan (RSS) scan and
 * SSA the scan-scan-add scheme of its OpenMP scan (openmp/test_scan_CPU.cpp). */
typedef enum {
    EDPP_SCAN_LOOKBACK = 0,
    EDPP_SCAN_RTS = 1,
    EDPP_SCAN_SSA = 2
} edpp_scan_algo;

/* Element types a scan accepts. */
typedef enum {
    EDPP_I32 = 0,
    EDPP_I64 = 1,
    EDPP_F32 = 2
} edpp_dtype;

/* Split data layout, same order as the reference's DataStruc
 * {KO, KVS_AOS, KVS_SOA} (opencl/types.h:29-31). */
typedef enum {
    EDPP_KO = 0,       /* keys only                                        */
    EDPP_KVS_AOS = 1,  /* int32 {key,value} pairs in one array             */
    EDPP_KVS_SOA = 2   /* keys and values in two arrays                    */
} edpp_layout;

/* ---- library ------------------------------------------------------------ */

/* Human-readable name of a status code. */
const char *edpp_status_string(int status);

/* Library version, as major*10000 + minor*100 + patch. */
int edpp_version(void);

/* Wait for `stream`, then report the first error: a CUDA error, or, if a
 * kernel recorded a fault since the last clear, EDPP_EINVAL for
 * EDPP_FAULT_PLAN and EDPP_ETIMEOUT otherwise.  clear != 0 resets the fault
 * word afterwards. */
int edpp_sync_status(void *stream, int clear);

/* Read (and optionally clear) the device fault word of the current device.
 * Synchronises the device. */
int edpp_device_fault(unsigned int *fault_bits, int clear);

/* ---- multi-pass gather / scatter --------------------------------------- */

/* out[i] = in[loc[i]] for i in [0,length).  Replaces
 *   double gather(cl_mem d_in, cl_mem d_out, int length, cl_mem d_loc,
 *                 int localSize, int gridSize, int pass)
 * (opencl/primitives.h:12-14, opencl/primitives/gatherImpl.cpp:7-55,
 *  opencl/kernels/gather_kernel.cl:6-21) and cuda/test_gather.cu:12-18.
 * `pass` windows the source index: pass k serves loc[i] in
 * [k*ceil(length/pass), (k+1)*ceil(length/pass)) and every pass reads all of
 * loc, as in gatherImpl.cpp:38-53.  Entries with loc[i] outside [0,length)
 * are skipped (out[i] keeps its value).  pass >= 1. */
int edpp_gather_i32(const int32_t *in, int32_t *out, int64_t length,
                    const int32_t *loc, int pass, void *stream);

/* out[loc[i]] = in[i], windowed on the destination index.  Replaces
 *   double scatter(cl_mem d_in, cl_mem d_out, int length, cl_mem d_loc,
 *                  int localSize, int gridSize, int pass)
 * (opencl/primitives.h:17-19, opencl/primitives/scatterImpl.cpp:9-54,
 *  opencl/kernels/scatter_kernel.cl:6-22) and cuda/test_scatter.cu:12-18. */
int edpp_scatter_i32(const int32_t *in, int32_t *out, int64_t length,
                     const int32_t *loc, int pass, void *stream);

/* Partitioned multi-pass gather / scatter: identical results to
 * edpp_gather_i32 / edpp_scatter_i32 for every pass count, with the pass
 * windows realised as partitions.  Requests are grouped by window into a
 * caller workspace (edpp_*_workspace_size), then each window's random side is
 * served while that window of the array sits in L2.  pass >= 2: windows of
 * the next power of two >= ceil(length/pass) elements; pass == 0: windows
 * sized to half of this GPU's L2; pass == 1: the direct single sweep (no
 * workspace).  A scatter with repeated destinations keeps one of the
 * colliding values. */
size_t edpp_gather_workspace_size(int64_t length, int pass);
size_t edpp_scatter_workspace_size(int64_t length, int pass);
int edpp_gather_i32_ws(const int32_t *in, int32_t *out, int64_t length,
                       const int32_t *loc, int pass, void *ws, size_t ws_bytes,
                       void *stream);
int edpp_scatter_i32_ws(const int32_t *in, int32_t *out, int64_t length,
                        const int32_t *loc, int pass, void *ws, size_t ws_bytes,
                        void *stream);

/* Shared-memory-window gather / scatter: the same results again, for every
 * pass count (pass >= 0 is accepted for the same signature; the windows are
 * fixed by shared memory, 2^14 or 2^15 elements).  Requests are partitioned
 * twice by window (128 coarse windows, then fine windows) and one block per
 * fine window serves them inside a shared-memory copy of that window, so no
 * global access is random.  length <= 2^29; longer arrays take the
 * L2-window path (pass 0) with the workspace sized for it. */
size_t edpp_gather_tiled_workspace_size(int64_t length);
size_t edpp_scatter_tiled_workspace_size(int64_t length);
int edpp_gather_i32_tiled(const int32_t *in, int32_t *out, int64_t length,
                          const int32_t *loc, int pass, void *ws, size_t ws_bytes,
                          void *stream);
int edpp_scatter_i32_tiled(const int32_t *in, int32_t *out, int64_t length,
                           const int32_t *loc, int pass, void *ws, size_t ws_bytes,
                           void *stream);
/* 1 when a gather of `length` elements is faster as the direct single sweep
 * (edpp_gather_i32, pass 1) than in the tiled form on the current device.
 * The tuning table's choice for this size class when it has one
 * (EDPP_TUNE_GATHER), else the rule that the source is small enough (about
 * 2.5x L2) to stay largely in L2.  Scatter always favours the tiled form. */
int edpp_gather_prefers_direct(int64_t length);

/* ---- global scan -------------------------------------------------------- */

/* Bytes of workspace a scan of `length` elements of `dtype` with `algo`
 * needs (0 is a valid answer only for length 0). */
size_t edpp_scan_workspace_size(int64_t length, int dtype, int algo);

/* Exclusive / inclusive prefix sums.  Integer sums wrap (two's complement),
 * as the reference's int scans do on its platforms; f32 sums in f32.
 * in == out (in-place) is allowed, as split uses it at
 * opencl/primitives/splitImpl.cpp:97.  Replaces
 *   double scan_chained(cl_mem d_in, cl_mem d_out, int length, int localSize,
 *                       int gridSize, int R, int L)   (LOOKBACK)
 *   double scan_RSS(cl_mem d_in, cl_mem d_out, unsigned length,
 *                   int local_size, int grid_size)     (RTS)
 * (opencl/primitives.h:22-29, opencl/primitives/scanImpl.cpp:15-160),
 * scan_SSA_omp / scan_RTS_omp (openmp/test_scan_CPU.cpp:85-163) and the CUB
 * ExclusiveSum call of cuda/test_scan.cu:45-47. */
int edpp_scan_exclusive_i32(const int32_t *in, int32_t *out, int64_t length,
                            int algo, void *ws, size_t ws_bytes, void *stream);
int edpp_scan_inclusive_i32(const int32_t *in, int32_t *out, int64_t length,
                            int algo, void *ws, size_t ws_bytes, void *stream);
int edpp_scan_exclusive_i64(const int64_t *in, int64_t *out, int64_t length,
                            int algo, void *ws, size_t ws_bytes, void *stream);
int edpp_scan_inclusive_i64(const int64_t *in, int64_t *out, int64_t length,
                            int algo, void *ws, size_t ws_bytes, void *stream);
int edpp_scan_exclusive_f32(const float *in, float *out, int64_t length,
                            int algo, void *ws, size_t ws_bytes, void *stream);
int edpp_scan_inclusive_f32(const float *in, float *out, int64_t length,
                            int algo, void *ws, size_t ws_bytes, void *stream);

/* ---- stable multi-split ------------------------------------------------- */

/* Bytes of workspace a split needs. */
size_t edpp_split_workspace_size(int64_t length, int buckets, int layout);

/* Stable multi-split by bucket = key & (buckets-1): the output holds the
 * input's elements grouped by bucket in ascending bucket order, in input
 * order within a bucket.  buckets is a power of two in [1, 8192] (from 2048
 * buckets the split runs as two stable passes, low 8 bits then the rest).
 * bucket_start (optional, int32[buckets]) receives the first output index of
 * every bucket, as gatherStartPos does (opencl/kernels/split_kernel.cl:320-332).
 * KO: keys_in/keys_out hold keys, vals_* are ignored.  KVS_SOA: keys and
 * values in separate arrays.  KVS_AOS: keys_in/keys_out point at
 * int32 {key,value} pairs (length pairs), vals_* are ignored.
 * Replaces WI_split / WG_split / single_split (opencl/primitives.h:32-49,
 * opencl/primitives/splitImpl.cpp:21-498) and the warp-ballot split of
 * cuda/test_split.cu:18-88.  The stable order is the one the reference's
 * single_split, WG_split(FIXED_REORDER) and the CUDA split produce. */
int edpp_split_i32(const int32_t *keys_in, int32_t *keys_out,
                   int32_t *bucket_start, int64_t length, int buckets,
                   int layout, const int32_t *vals_in, int32_t *vals_out,
                   void *ws, size_t ws_bytes, void *stream);

/* WI_split's own output order (bit-exact with the reference's WI_split for
 * the given local_size / grid_size; opencl/primitives/splitImpl.cpp:21-142,
 * split_kernel.cl:335-412): elements by bucket, then by work-item, then in
 * each work-item's lane-strided visiting order.  Equals the stable order when
 * length <= local_size * grid_size.  (The reference's d_start output of
 * WI_split indexes its per-work-item histogram with the per-group stride, so
 * it has no bucket-start meaning; use edpp_split_i32's bucket_start.) */
size_t edpp_split_wi_workspace_size(int64_t length, int buckets, int layout);
int edpp_split_i32_wi(const int32_t *keys_in, int32_t *keys_out, int64_t length,
                      int buckets, int layout, const int32_t *vals_in, int32_t *vals_out,
                      int local_size, int grid_size, void *ws, size_t ws_bytes,
                      void *stream);

/* ---- radix sort on the stable split -------------------------------------- */

/* LSD radix sort of int32 keys (with optional int32 values) by the key's bit
 * pattern (unsigned order) over bits [begin_bit, end_bit), 8 bits per pass,
 * each pass one stable split; stable.  keys_in != keys_out.  vals_in NULL:
 * keys only.  Counterpart of the reference's LSD radix sort
 * (obsolete/CUDA/kernels/radixSort.cu:29-370), the main consumer of split. */
size_t edpp_radix_sort_workspace_size(int64_t length, int with_values);
int edpp_radix_sort_i32(const int32_t *keys_in, int32_t *keys_out,
                        const int32_t *vals_in, int32_t *vals_out, int64_t length,
                        int begin_bit, int end_bit, void *ws, size_t ws_bytes,
                        void *stream);

/* ---- partitioned hash join (match count) --------------------------------- */

/* Number of pairs (r, s) with r_keys[r] == s_keys[s], written to *d_count
 * (device memory).  Both relations are split into `buckets` partitions by
 * key & (buckets-1) (power of two <= 8192; 0 = chosen from s_len), then one
 * block per partition pair builds a shared-memory hash table from S and
 * probes it with R.  Counterpart of the reference's partitioned hash join,
 * which also returns only the match count (obsolete/OpenCL/phjImpl.cpp:14-129,
 * hj_partitioned_kernel.cl:8-107). */
size_t edpp_hash_join_workspace_size(int64_t r_len, int64_t s_len, int buckets);
int edpp_hash_join_count(const int32_t *r_keys, int64_t r_len, const int32_t *s_keys,
                         int64_t s_len, int buckets, unsigned long long *d_count, void *ws,
                         size_t ws_bytes, void *stream);

/* Non-partitioned form: one open-addressing table of 2^k >= 2*build_len
 * slots (8 bytes each) in the workspace, built from build_keys and probed
 * with probe_keys; same count.  Counterpart of the reference's
 * non-partitioned hash join (obsolete/OpenCL/nphjImpl.cpp:15-144,
 * hj_non_partitioned_kernel.cl:9-77). */
size_t edpp_hash_join_np_workspace_size(int64_t build_len);
int edpp_hash_join_np_count(const int32_t *build_keys, int64_t build_len,
                            const int32_t *probe_keys, int64_t probe_len,
                            unsigned long long *d_count, void *ws, size_t ws_bytes, void *stream);

/* ---- access-pattern and single-block scan microbenchmarks --------------- */

/* Scale out[i] = 3 * in[i] over i in [0, local_size*grid_size*repeat) with
 * the reference's three thread-to-element maps (opencl/kernels/mem_kernel.cl:
 * 33-69, driven by opencl/test/test_access.cpp): COLUMN, thread g touches
 * g + k*G; ROW, g*repeat + k; MIXED, warp-contiguous chunks with lanes
 * stepping by 32.  VEC is the 16-byte grid-stride form the STREAM kernels use
 * (local_size/grid_size only set the element count). */
typedef enum {
  EDPP_ACCESS_COLUMN = 0,
  EDPP_ACCESS_ROW = 1,
  EDPP_ACCESS_MIXED = 2,
  EDPP_ACCESS_VEC = 3
} edpp_access_pattern;
int edpp_access_scale_i32(const int32_t *in, int32_t *out, int repeat, int pattern,
                          int local_size, int grid_size, void *stream);
/* Block-order sweep (mem_kernel.cl:71-87, opencl/test/test_access_wg.cpp):
 * grid_size blocks of local_size threads; the block holding ticket t sums
 * the low bits of chunk order[t] (len / grid_size elements) into out[order[t]].
 * *ticket (device word) is zeroed on the stream first. */
int edpp_access_wg_i32(const int32_t *in, int64_t len, const int32_t *order, int grid_size,
                       int local_size, unsigned *ticket, long long *out, void *stream);
/* Write-only warm-up data[c] = c in warp-contiguous chunks (mem_kernel.cl:89-107). */
int edpp_cache_heat_i32(int32_t *data, int64_t length, int local_size, int grid_size,
                        void *stream);
/* Exclusive scan of 512*tile_size int32 by one block of 512 threads, launched
 * `repeat` times (opencl/kernels/scan_local_kernel.cl:530-695, driven by
 * opencl/test/test_scan_local.cpp).  tile_size 1..49; in != out. */
typedef enum {
  EDPP_LOCAL_SCAN_LM = 0,     /* tile in shared memory, serial row scans */
  EDPP_LOCAL_SCAN_REG = 1,    /* rows loaded straight into registers */
  EDPP_LOCAL_SCAN_LM_REG = 2, /* coalesced via shared memory, rows in registers */
  EDPP_LOCAL_SCAN_WARP = 3    /* LM_REG with a warp-shuffle block scan */
} edpp_local_scan_scheme;
int edpp_local_scan_i32(const int32_t *in, int32_t *out, int tile_size, int scheme, int repeat,
                        void *stream);

/* ---- STREAM ------------------------------------------------------------- */

/* copy c=a, scale c=s*a, add c=a+b, triad c=a+s*b.  Replace the kernels of
 * cuda/test_bandwidth.cu:14-44 and opencl/kernels/mem_kernel.cl:9-31
 * (int32, SCALAR=3) and copy_omp/scale_omp of
 * openmp/test_bandwidth_CPU.cpp:39-56.  Integer arithmetic wraps. */
int edpp_stream_copy_f32(const float *a, float *c, int64_t n, void *stream);
int edpp_stream_scale_f32(const float *a, float *c, float s, int64_t n,
                          void *stream);
int edpp_stream_add_f32(const float *a, const float *b, float *c, int64_t n,
                        void *stream);
int edpp_stream_triad_f32(const float *a, const float *b, float *c, float s,
                          int64_t n, void *stream);
int edpp_stream_copy_i32(const int32_t *a, int32_t *c, int64_t n,
                         void *stream);
int edpp_stream_scale_i32(const int32_t *a, int32_t *c, int32_t s, int64_t n,
                          void *stream);
int edpp_stream_add_i32(const int32_t *a, const int32_t *b, int32_t *c,
                        int64_t n, void *stream);
int edpp_stream_triad_i32(const int32_t *a, const int32_t *b, int32_t *c,
                          int32_t s, int64_t n, void *stream);

/* ---- allocation-free scan ------------------------------------------------ */

/* Exclusive int32 look-back scan that allocates nothing and takes no
 * workspace.  It has no counterpart in the reference; it exists for callers
 * that cannot allocate device memory at the point of the call (a host thread
 * that must not enter the device allocator, such as a real-time loop, or a
 * plugin whose host owns all device allocations).  Its scratch is one 1 MiB array in device
 * global memory that every GPU loading the library holds until exit, so
 * length is limited to edpp_scan_exclusive_i32_noalloc_max_length()
 * (536,739,840 elements); longer inputs return EDPP_EINVAL.  The first call on
 * a device looks up the array's device address (once per device; make that
 * first call before any stream capture).  All calls share the one array:
 * calls whose work overlaps on the GPU (different streams, or several host
 * threads without ordering) race and give wrong results; order them on one
 * stream.  Results equal edpp_scan_exclusive_i32 with EDPP_SCAN_LOOKBACK. */
int edpp_scan_exclusive_i32_noalloc(const int32_t *in, int32_t *out, int64_t length,
                                    void *stream);
int64_t edpp_scan_exclusive_i32_noalloc_max_length(void);

/* ---- batched segments (one plan, a handful of launches) ----------------- */

/* Operations a batch segment can run.  Results equal the plain calls:
 *   SCAN    out0 = exclusive int32 scan of in0            (edpp_scan_exclusive_i32)
 *   SPLIT   (out0, out1) = stable split of keys in0 / values in1 by
 *           key & (buckets-1), buckets a power of two <= 256  (edpp_split_i32, SOA)
 *   GATHER  out0[i] = in0[off + in1[i]] with segment-local indices in1
 *           (entries outside [0, length) skipped)       (edpp_gather_i32)
 * No reference counterpart: the reference runs one primitive per call. */
typedef enum {
    EDPP_BATCH_SCAN = 0,
    EDPP_BATCH_SPLIT = 1,
    EDPP_BATCH_GATHER = 2
} edpp_batch_op;

/* One segment: elements [offset, offset+length) of the batch arrays. */
typedef struct {
    int64_t offset;
    int32_t length;
    int32_t op;       /* edpp_batch_op */
    int32_t buckets;  /* SPLIT only */
    int32_t reserved;
} edpp_segment;

/* How a batch runs on the GPU:
 *   KINDS  one launch per kind of tile over every segment of that kind (scan
 *          tiles; gather tiles; split histogram tiles, the per-segment
 *          histogram scans, split scatter tiles), each sized for its kind
 *   QUEUE  one persistent launch whose blocks take all tiles from one work
 *          queue (blocks_per_sm, split_defer_segments, largest_first apply) */
typedef enum {
    EDPP_BATCH_SCHEDULE_KINDS = 0,
    EDPP_BATCH_SCHEDULE_QUEUE = 1
} edpp_batch_schedule;

/* Scheduling knobs (chosen per size class by the project's autotuner,
 * edpp_batch_autotune).  Zero-initialised = defaults. */
typedef struct {
    int32_t blocks_per_sm;         /* QUEUE: blocks per SM (default 4)            */
    int32_t split_defer_segments;  /* QUEUE: SPLIT tiles queued this many segments
                                      after their HIST tiles (default 1)         */
    int32_t largest_first;         /* QUEUE: segments by descending length        */
    int32_t schedule;              /* edpp_batch_schedule (default KINDS)         */
} edpp_batch_tuning;

typedef struct edpp_batch_plan edpp_batch_plan;  /* opaque, host side */

/* Build the task queue for `num_segs` segments (host only, no GPU work). */
int edpp_batch_plan_create(const edpp_segment *segs, int num_segs,
                           const edpp_batch_tuning *tuning, edpp_batch_plan **plan);
void edpp_batch_plan_destroy(edpp_batch_plan *plan);
size_t edpp_batch_plan_workspace_size(const edpp_batch_plan *plan);
/* Tile tasks of the batch (a split tile counts twice: histogram and scatter). */
int edpp_batch_plan_num_tasks(const edpp_batch_plan *plan);
/* Copy the plan's tables into the workspace (synchronises `stream`). */
int edpp_batch_plan_upload(const edpp_batch_plan *plan, void *ws, size_t ws_bytes,
                           void *stream);
/* Run every segment: one launch per tile kind (KINDS) or one persistent
 * launch (QUEUE), plus two memsets.  The workspace must hold an uploaded
 * plan.  Stream-ordered; may be captured in a CUDA graph and replayed while
 * the plan and arrays stay the same. */
int edpp_batch_launch(const edpp_batch_plan *plan, const int32_t *in0,
                      const int32_t *in1, int32_t *out0, int32_t *out1, void *ws,
                      size_t ws_bytes, void *stream);

/* Autotuner: times every candidate edpp_batch_tuning on this GPU for these
 * segments and writes the fastest to *best (its mean ms to *best_ms).
 * Synchronises `stream`; overwrites out0/out1. */
int edpp_batch_autotune(const edpp_segment *segs, int num_segs, const int32_t *in0,
                        const int32_t *in1, int32_t *out0, int32_t *out1, void *ws,
                        size_t ws_bytes, void *stream, int reps, edpp_batch_tuning *best,
                        float *best_ms);

/* The same segments as one plain C-ABI call each, back to back on `stream`
 * (the per-array baseline of the batch).  Workspace: the largest any one
 * call needs. */
size_t edpp_batch_plain_workspace_size(const edpp_segment *segs, int num_segs);
int edpp_batch_run_plain(const edpp_segment *segs, int num_segs, const int32_t *in0,
                         const int32_t *in1, int32_t *out0, int32_t *out1, void *ws,
                         size_t ws_bytes, void *stream);

/* ---- serving: continuous batching of requests --------------------------- */

/* A request: one scan / split / gather (edpp_batch_op) on HOST arrays of
 * `length` int32 (pinned memory gives asynchronous copies).  in1: split
 * values or segment-local gather indices; out1: split values. */
typedef struct {
    int32_t op;
    int32_t buckets;
    int64_t length;
    const int32_t *in0;
    const int32_t *in1;
    int32_t *out0;
    int32_t *out1;
} edpp_request;

typedef struct {
    size_t pool_bytes;           /* device memory for request buffers (admission cap) */
    int32_t slots;               /* batches in flight at once (streams), 1..16         */
    int32_t max_batch_requests;  /* per batch (default 1024)                          */
    int64_t max_batch_elements;  /* per batch (default: the whole pool)               */
    edpp_batch_tuning tuning;    /* schedule of the batch kernel                      */
} edpp_server_config;

typedef struct {
    double queue_ms;    /* submit -> admitted into a batch                     */
    double latency_ms;  /* submit -> outputs back in host memory               */
} edpp_request_timing;

typedef struct {
    int64_t submitted, completed, batches, elements_done;
    int64_t max_requests_per_batch, max_pool_bytes_used, max_batches_in_flight;
} edpp_server_stats;

typedef struct edpp_server edpp_server;  /* opaque */

/* Start a server on the current device: allocates the request pool (four
 * arenas of pool_bytes/4), per-slot streams and workspaces, and a scheduler
 * thread.  One scheduler loop retires finished batches, admits waiting
 * requests in arrival order while pool memory and a slot are free, and
 * launches each batch (config->tuning's schedule) between its copies.  No
 * reference counterpart. */
int edpp_server_create(const edpp_server_config *cfg, edpp_server **server);
/* Thread-safe, non-blocking.  EDPP_EINVAL for a malformed request or one
 * larger than the whole pool. */
int edpp_server_submit(edpp_server *server, const edpp_request *req, uint64_t *id);
/* Block until request `id` completes (outputs written); returns its status. */
int edpp_server_wait(edpp_server *server, uint64_t id, double timeout_s,
                     edpp_request_timing *timing);
int edpp_server_get_stats(edpp_server *server, edpp_server_stats *stats);
/* Finish all submitted work, stop the scheduler, free everything. */
void edpp_server_destroy(edpp_server *server);

/* ---- per-size-class tuning of the plain primitives ---------------------- */

/* Choices the primitives read at call time, per primitive, element size and
 * size class (log2 of the length); a length takes the entry of the nearest
 * recorded class, else the default (variant 0).  The reference fixes its
 * tunables per device by hand (R, L, local and grid sizes of scan_chained,
 * opencl/test/test_scan_global.cpp:87-94); here they are measured.
 *   EDPP_TUNE_SCAN_LOOKBACK  look-back tile shape (threads x 16-byte chunks):
 *                            0 128x8 (16 KB), 1 256x8 (32 KB), 2 512x4 (32 KB),
 *                            3 512x8 (64 KB)
 *   EDPP_TUNE_SCAN_RTS       slice of the chunked reduce-then-scan (inputs
 *                            larger than 60% of L2): 0 two tiles, 1 one,
 *                            2 four, 3 two with L2 eviction hints (first read
 *                            kept, second read demoted), 4 two tiles and the
 *                            chunked form also below 60% of L2
 *   EDPP_TUNE_GATHER         0 tiled form, 1 direct single sweep (the choice
 *                            edpp_gather_prefers_direct reports)
 * The table is read from efficient-dpp_gb300/tuning/plain_gb300.tsv (beside
 * the library's lib/ directory) on first use; edpp_tune_load replaces it.
 * All functions here are host-only and thread-safe. */
typedef enum {
    EDPP_TUNE_SCAN_LOOKBACK = 0,
    EDPP_TUNE_SCAN_RTS = 1,
    EDPP_TUNE_GATHER = 2
} edpp_tune_primitive;

/* Number of variants of a primitive (0: not tunable). */
int edpp_tune_variants(int primitive);
/* Record `variant` (measured at `ms`, informational) for the class. */
int edpp_tune_set(int primitive, int elem_bytes, int log2_length, int variant, float ms);
/* The variant a call of `length` elements takes now (EDPP_OK), or the
 * default with EDPP_EINVAL when the table has no entry for the primitive. */
int edpp_tune_get(int primitive, int elem_bytes, int64_t length, int *variant);
/* Replace the table with a file's entries (NULL: the default file); a
 * missing file leaves the table empty.  Lines: "name elem_bytes log2_length
 * variant ms", '#' starts a comment. */
int edpp_tune_load(const char *path);
/* Write the table to `path` in the same format. */
int edpp_tune_save(const char *path);
/* Empty the table (every primitive takes its default). */
void edpp_tune_clear(void);
/* The autotuner: times every variant of `primitive` at `length` on the
 * caller's arrays (scan: `in` / `out` of elem_bytes = 4 (int32) or 8
 * (int64) elements, exclusive, ws of edpp_scan_workspace_size for its
 * algorithm; gather: int32 in / out / loc, ws of
 * edpp_gather_tiled_workspace_size), CUDA events around each of `reps`
 * calls after one warm-up, and records the fastest in the table
 * (*best_variant, *best_ms; variant_ms, if not NULL, gets every variant's
 * mean ms).  With `flush` (a caller buffer of flush_bytes, larger than L2)
 * the buffer is overwritten before every timed call, outside the timed
 * span, so variants are timed with the input out of L2, as a first touch
 * of the data finds it.  Another variant replaces the default (0) only when
 * it is more than 1% faster.  Synchronises `stream`; overwrites out and
 * flush. */
int edpp_autotune_plain(int primitive, const void *in, void *out, const int32_t *loc,
                        int64_t length, int elem_bytes, void *ws, size_t ws_bytes,
                        void *stream, int reps, void *flush, size_t flush_bytes,
                        int *best_variant, float *best_ms, float *variant_ms);

/* ---- bounded-wait self-test --------------------------------------------- */

/* Runs a look-back scan over `length` int32 elements whose first tile is
 * never published, with every wait limited to `timeout_ns`, so that each
 * waiting tile gives up, records EDPP_FAULT_TIMEOUT and returns.  Exists to
 * test failure detection without faulting the GPU; the reference's chained
 * scan spins without a limit (opencl/kernels/scan_global_chain_kernel.cl:21).
 * Returns the launch status; read the outcome with edpp_sync_status. */
int edpp_selftest_lookback_timeout(const int32_t *in, int32_t *out,
                                   int64_t length, uint64_t timeout_ns,
                                   void *ws, size_t ws_bytes, void *stream);

#ifdef __cplusplus
}
#endif

#endif /* EDPP_H_ */
