/*
 * edpp_oracle.h — CPU oracle for the data-parallel primitives.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain-C restatement of
 * Efficient-DPP's algorithms, used as the checker by tests/, by
 * __graft_entry__.smoke() and by the cpu_baseline leg of bench.py.  Nothing
 * in the product (efficient-dpp_gb300/) may link, load or call it.
 *
 * Each function cites the reference file:line it follows.
 */
#ifndef EDPP_ORACLE_H_
#define EDPP_ORACLE_H_

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- multi-pass gather / scatter (opencl/primitives/gatherImpl.cpp:38-53,
 *      opencl/kernels/gather_kernel.cl:15-20, scatter_kernel.cl:16-21) ---- */
void orc_gather_i32(const int32_t *in, int32_t *out, int64_t n, const int32_t *loc, int pass);
void orc_scatter_i32(const int32_t *in, int32_t *out, int64_t n, const int32_t *loc, int pass);

/* ---- sequential scans (scan_check, openmp/test_scan_CPU.cpp:39-49) ---- */
void orc_scan_excl_i32(const int32_t *in, int32_t *out, int64_t n);
void orc_scan_incl_i32(const int32_t *in, int32_t *out, int64_t n);
void orc_scan_excl_i64(const int64_t *in, int64_t *out, int64_t n);
void orc_scan_incl_i64(const int64_t *in, int64_t *out, int64_t n);
/* f32 inputs accumulated in f64 (the oracle for f32 scans). */
void orc_scan_f32_in_f64(const float *in, double *out, int64_t n, int inclusive);

/* ---- OpenMP ports of the reference CPU scans; return elapsed ms.
 *      nthreads <= 0: OpenMP default.  (openmp/test_scan_CPU.cpp:85-163) ---- */
double orc_scan_ssa_omp_i32(const int32_t *in, int32_t *out, int64_t n, int nthreads);
double orc_scan_rts_omp_i32(const int32_t *in, int32_t *out, int64_t n, int nthreads);

/* ---- OpenMP ports of the reference CPU gather/scatter; elapsed ms
 *      (openmp/test_gather_scatter_CPU.cpp:24-41) ---- */
double orc_gather_omp_i32(const int32_t *in, int32_t *out, const int32_t *idx, int64_t n,
                          int nthreads);
double orc_scatter_omp_i32(const int32_t *in, int32_t *out, const int32_t *idx, int64_t n,
                           int nthreads);

/* ---- STREAM (cuda/test_bandwidth.cu:14-44, openmp/test_bandwidth_CPU.cpp:39-56);
 *      op: 0 copy, 1 scale, 2 add, 3 triad; elapsed ms ---- */
double orc_stream_f32(int op, const float *a, const float *b, float *c, float s, int64_t n,
                      int nthreads);
double orc_stream_i32(int op, const int32_t *a, const int32_t *b, int32_t *c, int32_t s,
                      int64_t n, int nthreads);

/* ---- multi-split ---- */
/* Stable split by key & (buckets-1) (counting sort).  layout: 0 KO,
 * 1 KVS_AOS (keys = int32 pairs), 2 KVS_SOA.  start (optional) gets the
 * first output index of every bucket (gatherStartPos). */
void orc_split_stable(const int32_t *keys, const int32_t *vals, int64_t n, int buckets,
                      int layout, int32_t *keys_out, int32_t *vals_out, int32_t *start);
/* Literal restatement of the CUDA warp-ballot split: pre_scan / warp_histogram,
 * exclusive sum of the bucket-major histogram, post_scan / warp_offset
 * (cuda/test_split.cu:18-88,149-186).  Keys must already be < 2^bucket_bits,
 * n a multiple of 32, bucket_bits <= 8 (the reference's limits). */
void orc_split_cuda_ballot(const int32_t *keys, int64_t n, int bucket_bits, int32_t *keys_out);
/* Literal restatement of the OpenCL single_split, KO and AOS layouts:
 * single_histogram, scan of his[b*G+g], single_shuffle
 * (opencl/primitives/splitImpl.cpp:366-498, split_kernel.cl:676-736),
 * with G groups (the reference uses 39). */
void orc_split_single(const int32_t *in, int64_t n, int buckets, int aos, int groups,
                      int32_t *out);
/* Literal restatement of the OpenCL WI_split order (per-work-item histograms,
 * lane-strided visiting; opencl/kernels/split_kernel.cl:335-412).  vals may
 * be NULL (KO); aos != 0: int32 pairs in `in`/`out`. */
void orc_split_wi(const int32_t *in, const int32_t *vals, int64_t n, int buckets, int aos,
                  int local_size, int grid_size, int32_t *out, int32_t *vals_out);
/* Elapsed-ms timing of the stable split restatement (CPU baseline). */
double orc_split_stable_timed(const int32_t *keys, const int32_t *vals, int64_t n, int buckets,
                              int layout, int32_t *keys_out, int32_t *vals_out);

/* ---- join: number of equal-key (r, s) pairs (phjImpl.cpp:14-129 res_len) ---- */
uint64_t orc_join_count(const int32_t *r, int64_t r_len, const int32_t *s, int64_t s_len);

/* ---- measurement helpers (openmp/util/utility.cpp:23-71) ---- */
double orc_compute_bandwidth(uint64_t num, int word_size, double ms);
double orc_average_hampel(const double *x, int n);

int orc_max_threads(void);

/* ---- seeded Fisher-Yates permutation of [0, n) (splitmix64 draws), the
 *      benchmark's gather/scatter index array; replaces the reference's
 *      time()-seeded random_generator_int_unique (openmp/util/utility.cpp:90-104) ---- */
void orc_gen_permutation_i32(int32_t *out, int64_t n, uint64_t seed);

#ifdef __cplusplus
}
#endif

#endif /* EDPP_ORACLE_H_ */
