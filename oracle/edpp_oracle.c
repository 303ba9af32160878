/*
 * edpp_oracle.c — CPU oracle for the data-parallel primitives.
 *
 * TEST INFRASTRUCTURE ONLY: the checker for tests/, __graft_entry__.smoke()
 * and the cpu_baseline leg of bench.py.  The product never links it.
 *
 * A plain-C restatement of Efficient-DPP's algorithms; each function cites
 * the reference file:line it follows.  Integer sums use unsigned arithmetic,
 * i.e. two's-complement wrapping, which is what the reference's signed int
 * sums do on its platforms (it relies on signed overflow wrapping).
 */
#include "edpp_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

#ifdef _OPENMP
#include <omp.h>
#endif

static double now_ms(void) {
#ifdef _OPENMP
  return omp_get_wtime() * 1000.0;
#else
  return 0.0;
#endif
}

int orc_max_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

static int pick_threads(int nthreads) {
  int t = nthreads > 0 ? nthreads : orc_max_threads();
  if (t > 256) t = 256; /* MAX_THREAD_NUM, openmp/test_scan_CPU.cpp:36 */
  return t < 1 ? 1 : t;
}

/* ---- multi-pass gather / scatter ----------------------------------------
 * Pass k serves positions pos in [from, to) with len_per_run = ceil(n/pass),
 * from = k*len_per_run, to = (k+1)*len_per_run (gatherImpl.cpp:38-44); the
 * kernels test `pos >= from && pos < to` (gather_kernel.cl:15-20,
 * scatter_kernel.cl:16-21).  The extra `pos < n` keeps an invalid index from
 * reading or writing past the array (the reference has no such guard). */
void orc_gather_i32(const int32_t *in, int32_t *out, int64_t n, const int32_t *loc, int pass) {
  const int64_t len_per_run = (n + pass - 1) / pass;
  for (int k = 0; k < pass; ++k) {
    const int64_t from = (int64_t)k * len_per_run, to = (int64_t)(k + 1) * len_per_run;
    for (int64_t i = 0; i < n; ++i) {
      const int64_t pos = loc[i];
      if (pos >= from && pos < to && pos < n) out[i] = in[pos];
    }
  }
}

void orc_scatter_i32(const int32_t *in, int32_t *out, int64_t n, const int32_t *loc, int pass) {
  const int64_t len_per_run = (n + pass - 1) / pass;
  for (int k = 0; k < pass; ++k) {
    const int64_t from = (int64_t)k * len_per_run, to = (int64_t)(k + 1) * len_per_run;
    for (int64_t i = 0; i < n; ++i) {
      const int64_t pos = loc[i];
      if (pos >= from && pos < to && pos < n) out[pos] = in[i];
    }
  }
}

/* ---- sequential scans ------------------------------------------------------
 * The exclusive prefix `acc` of scan_check (openmp/test_scan_CPU.cpp:39-49);
 * inclusive = exclusive + input (obsolete/CUDA/kernels/scan.cu:400-460). */
void orc_scan_excl_i32(const int32_t *in, int32_t *out, int64_t n) {
  uint32_t acc = 0;
  for (int64_t i = 0; i < n; ++i) {
    const uint32_t v = (uint32_t)in[i];
    out[i] = (int32_t)acc;
    acc += v;
  }
}

void orc_scan_incl_i32(const int32_t *in, int32_t *out, int64_t n) {
  uint32_t acc = 0;
  for (int64_t i = 0; i < n; ++i) {
    acc += (uint32_t)in[i];
    out[i] = (int32_t)acc;
  }
}

void orc_scan_excl_i64(const int64_t *in, int64_t *out, int64_t n) {
  uint64_t acc = 0;
  for (int64_t i = 0; i < n; ++i) {
    const uint64_t v = (uint64_t)in[i];
    out[i] = (int64_t)acc;
    acc += v;
  }
}

void orc_scan_incl_i64(const int64_t *in, int64_t *out, int64_t n) {
  uint64_t acc = 0;
  for (int64_t i = 0; i < n; ++i) {
    acc += (uint64_t)in[i];
    out[i] = (int64_t)acc;
  }
}

void orc_scan_f32_in_f64(const float *in, double *out, int64_t n, int inclusive) {
  double acc = 0.0;
  for (int64_t i = 0; i < n; ++i) {
    if (inclusive) {
      acc += (double)in[i];
      out[i] = acc;
    } else {
      out[i] = acc;
      acc += (double)in[i];
    }
  }
}

/* ---- OpenMP scan ports -------------------------------------------------------
 * scan_SSA_omp (openmp/test_scan_CPU.cpp:85-122): static-schedule local scan
 * per thread, serial exclusive scan of the thread sums, add pass. */
double orc_scan_ssa_omp_i32(const int32_t *in, int32_t *out, int64_t n, int nthreads) {
  const int nt = pick_threads(nthreads);
  uint32_t reduce_sum[256];
  memset(reduce_sum, 0, sizeof(reduce_sum));
  const double t0 = now_ms();
#pragma omp parallel num_threads(nt)
  {
    int tid = 0, nth = 1;
#ifdef _OPENMP
    tid = omp_get_thread_num();
    nth = omp_get_num_threads();
#endif
    uint32_t local_sum = 0;
#pragma omp for schedule(static) nowait
    for (int64_t i = 0; i < n; ++i) {
      out[i] = (int32_t)local_sum;
      local_sum += (uint32_t)in[i];
    }
    reduce_sum[tid] = local_sum;
#pragma omp barrier
#pragma omp single
    {
      uint32_t acc = 0;
      for (int i = 0; i < nth; ++i) {
        const uint32_t t = reduce_sum[i];
        reduce_sum[i] = acc;
        acc += t;
      }
    }
#pragma omp for schedule(static) nowait
    for (int64_t i = 0; i < n; ++i) out[i] = (int32_t)((uint32_t)out[i] + reduce_sum[tid]);
  }
  return now_ms() - t0;
}

/* scan_RTS_omp (openmp/test_scan_CPU.cpp:125-163): static-schedule reduce per
 * thread, serial exclusive scan of the sums, scan pass from each offset. */
double orc_scan_rts_omp_i32(const int32_t *in, int32_t *out, int64_t n, int nthreads) {
  const int nt = pick_threads(nthreads);
  uint32_t reduce_sum[256];
  memset(reduce_sum, 0, sizeof(reduce_sum));
  const double t0 = now_ms();
#pragma omp parallel num_threads(nt)
  {
    int tid = 0, nth = 1;
#ifdef _OPENMP
    tid = omp_get_thread_num();
    nth = omp_get_num_threads();
#endif
    uint32_t local_sum = 0;
#pragma omp for schedule(static) nowait
    for (int64_t i = 0; i < n; ++i) local_sum += (uint32_t)in[i];
    reduce_sum[tid] = local_sum;
#pragma omp barrier
#pragma omp single
    {
      uint32_t acc = 0;
      for (int i = 0; i < nth; ++i) {
        const uint32_t t = reduce_sum[i];
        reduce_sum[i] = acc;
        acc += t;
      }
    }
    local_sum = reduce_sum[tid];
#pragma omp for schedule(static) nowait
    for (int64_t i = 0; i < n; ++i) {
      out[i] = (int32_t)local_sum;
      local_sum += (uint32_t)in[i];
    }
  }
  return now_ms() - t0;
}

/* ---- OpenMP gather / scatter ports (openmp/test_gather_scatter_CPU.cpp:24-41) -- */
double orc_gather_omp_i32(const int32_t *in, int32_t *out, const int32_t *idx, int64_t n,
                          int nthreads) {
  const int nt = pick_threads(nthreads);
  const double t0 = now_ms();
#pragma omp parallel for schedule(auto) num_threads(nt)
  for (int64_t i = 0; i < n; ++i) out[i] = in[idx[i]];
  return now_ms() - t0;
}

double orc_scatter_omp_i32(const int32_t *in, int32_t *out, const int32_t *idx, int64_t n,
                           int nthreads) {
  const int nt = pick_threads(nthreads);
  const double t0 = now_ms();
#pragma omp parallel for schedule(auto) num_threads(nt)
  for (int64_t i = 0; i < n; ++i) out[idx[i]] = in[i];
  return now_ms() - t0;
}

/* ---- STREAM: copy c=a, scale c=s*a, add c=a+b, triad c=a+s*b
 * (cuda/test_bandwidth.cu:14-44; copy_omp/scale_omp at
 * openmp/test_bandwidth_CPU.cpp:39-56; add/triad restated) ---- */
double orc_stream_f32(int op, const float *a, const float *b, float *c, float s, int64_t n,
                      int nthreads) {
  const int nt = pick_threads(nthreads);
  const double t0 = now_ms();
#pragma omp parallel for schedule(static) num_threads(nt)
  for (int64_t i = 0; i < n; ++i) {
    switch (op) {
      case 0: c[i] = a[i]; break;
      case 1: c[i] = s * a[i]; break;
      case 2: c[i] = a[i] + b[i]; break;
      default: c[i] = a[i] + s * b[i]; break;
    }
  }
  return now_ms() - t0;
}

double orc_stream_i32(int op, const int32_t *a, const int32_t *b, int32_t *c, int32_t s,
                      int64_t n, int nthreads) {
  const int nt = pick_threads(nthreads);
  const uint32_t us = (uint32_t)s;
  const double t0 = now_ms();
#pragma omp parallel for schedule(static) num_threads(nt)
  for (int64_t i = 0; i < n; ++i) {
    const uint32_t x = (uint32_t)a[i];
    switch (op) {
      case 0: c[i] = (int32_t)x; break;
      case 1: c[i] = (int32_t)(x * us); break;
      case 2: c[i] = (int32_t)(x + (uint32_t)b[i]); break;
      default: c[i] = (int32_t)(x + us * (uint32_t)b[i]); break;
    }
  }
  return now_ms() - t0;
}

/* ---- stable multi-split (counting sort) --------------------------------------
 * The unique stable partition by key & (buckets-1): what single_split
 * (split_kernel.cl:676-736), WG_shuffle_fixed with one work-item per group
 * (split_kernel.cl:574-665) and the CUDA split (cuda/test_split.cu:56-88)
 * produce.  start[b] as gatherStartPos (split_kernel.cl:320-332). */
void orc_split_stable(const int32_t *keys, const int32_t *vals, int64_t n, int buckets,
                      int layout, int32_t *keys_out, int32_t *vals_out, int32_t *start) {
  const uint32_t mask = (uint32_t)buckets - 1u;
  int64_t *pos = (int64_t *)calloc((size_t)buckets, sizeof(int64_t));
  if (!pos) return;
  for (int64_t i = 0; i < n; ++i) {
    const int32_t k = (layout == 1) ? keys[2 * i] : keys[i];
    pos[(uint32_t)k & mask]++;
  }
  int64_t acc = 0;
  for (int b = 0; b < buckets; ++b) {
    const int64_t c = pos[b];
    pos[b] = acc;
    if (start) start[b] = (int32_t)acc;
    acc += c;
  }
  for (int64_t i = 0; i < n; ++i) {
    if (layout == 1) {
      const int32_t k = keys[2 * i];
      const int64_t p = pos[(uint32_t)k & mask]++;
      keys_out[2 * p] = k;
      keys_out[2 * p + 1] = keys[2 * i + 1];
    } else {
      const int32_t k = keys[i];
      const int64_t p = pos[(uint32_t)k & mask]++;
      keys_out[p] = k;
      if (layout == 2) vals_out[p] = vals[i];
    }
  }
  free(pos);
}

double orc_split_stable_timed(const int32_t *keys, const int32_t *vals, int64_t n, int buckets,
                              int layout, int32_t *keys_out, int32_t *vals_out) {
  const double t0 = now_ms();
  orc_split_stable(keys, vals, n, buckets, layout, keys_out, vals_out, NULL);
  return now_ms() - t0;
}

/* ---- literal restatement of the CUDA warp-ballot split ------------------------
 * cuda/test_split.cu: pre_scan -> warp_histogram (:19-54) builds
 * histo[b*warpNum + warpId] from bucket_bits ballots; ExclusiveSum over
 * buckets*warpNum entries (:165-167); post_scan -> warp_offset (:56-76)
 * ranks a lane by popc(same-bucket lanes <= lane) - 1.  Ballots are emulated
 * over the 32 lanes of each warp. */
static uint32_t ballot_bit(const int32_t *warp_bucket, int k) {
  uint32_t m = 0;
  for (int l = 0; l < 32; ++l)
    if (((uint32_t)warp_bucket[l] >> k) & 1u) m |= 1u << l;
  return m;
}

void orc_split_cuda_ballot(const int32_t *keys, int64_t n, int bucket_bits, int32_t *keys_out) {
  const int buckets = 1 << bucket_bits;
  const int64_t warp_num = n / 32;
  const int rounds = (buckets + 31) / 32;
  uint32_t *histo = (uint32_t *)calloc((size_t)(buckets * warp_num), sizeof(uint32_t));
  if (!histo) return;
  /* pre_scan / warp_histogram */
  for (int64_t w = 0; w < warp_num; ++w) {
    const int32_t *kb = keys + w * 32;
    uint32_t ballots[12];
    for (int k = 0; k < bucket_bits; ++k) ballots[k] = ballot_bit(kb, k);
    for (int lane = 0; lane < 32; ++lane) {
      for (int j = 0; j < rounds; ++j) {
        uint32_t bmp = 0xffffffffu;
        for (int k = 0; k < bucket_bits; ++k) {
          if ((((uint32_t)(j * 32 + lane)) >> k) & 1u) bmp &= ballots[k];
          else bmp &= (0xffffffffu ^ ballots[k]);
        }
        const int idx = j * 32 + lane;
        if (idx < buckets) histo[(int64_t)idx * warp_num + w] = (uint32_t)__builtin_popcount(bmp);
      }
    }
  }
  /* cub::DeviceScan::ExclusiveSum over buckets*warp_num entries */
  uint32_t acc = 0;
  for (int64_t i = 0; i < (int64_t)buckets * warp_num; ++i) {
    const uint32_t v = histo[i];
    histo[i] = acc;
    acc += v;
  }
  /* post_scan / warp_offset */
  for (int64_t w = 0; w < warp_num; ++w) {
    const int32_t *kb = keys + w * 32;
    uint32_t ballots[12];
    for (int k = 0; k < bucket_bits; ++k) ballots[k] = ballot_bit(kb, k);
    for (int lane = 0; lane < 32; ++lane) {
      const uint32_t bucket = (uint32_t)kb[lane];
      uint32_t bmp = 0xffffffffu;
      for (int k = 0; k < bucket_bits; ++k) {
        if ((bucket >> k) & 1u) bmp &= ballots[k];
        else bmp &= (0xffffffffu ^ ballots[k]);
      }
      const int offset = __builtin_popcount(bmp & (0xffffffffu >> (31 - lane))) - 1;
      const int64_t pos = (int64_t)histo[(int64_t)bucket * warp_num + w] + offset;
      keys_out[pos] = kb[lane];
    }
  }
  free(histo);
}

/* ---- literal restatement of the OpenCL single_split ---------------------------
 * single_histogram (split_kernel.cl:676-705): group g counts its contiguous
 * range [g*L, min((g+1)*L, n)), L = ceil(n/G), into his[b*G + g];
 * scan_chained exclusive over his (splitImpl.cpp:438); single_shuffle
 * (split_kernel.cl:708-736): d_out[local_buc[b]++] = d_in[i] in input order.
 * aos != 0: elements are int32 pairs keyed on the first. */
void orc_split_single(const int32_t *in, int64_t n, int buckets, int aos, int groups,
                      int32_t *out) {
  const uint32_t mask = (uint32_t)buckets - 1u;
  const int64_t len_per_group = (n + groups - 1) / groups;
  const int64_t his_len = (int64_t)buckets * groups;
  int64_t *his = (int64_t *)calloc((size_t)his_len, sizeof(int64_t));
  if (!his) return;
  for (int g = 0; g < groups; ++g) {
    int64_t s = len_per_group * g, e = len_per_group * (g + 1);
    if (e > n) e = n;
    for (int64_t i = s; i < e; ++i) {
      const uint32_t off = (uint32_t)(aos ? in[2 * i] : in[i]) & mask;
      his[(int64_t)off * groups + g]++;
    }
  }
  int64_t acc = 0;
  for (int64_t i = 0; i < his_len; ++i) {
    const int64_t v = his[i];
    his[i] = acc;
    acc += v;
  }
  for (int g = 0; g < groups; ++g) {
    int64_t s = len_per_group * g, e = len_per_group * (g + 1);
    if (e > n) e = n;
    for (int64_t i = s; i < e; ++i) {
      const uint32_t off = (uint32_t)(aos ? in[2 * i] : in[i]) & mask;
      const int64_t addr = his[(int64_t)off * groups + g]++;
      if (aos) {
        out[2 * addr] = in[2 * i];
        out[2 * addr + 1] = in[2 * i + 1];
      } else {
        out[addr] = in[i];
      }
    }
  }
  free(his);
}

/* ---- measurement helpers -------------------------------------------------------
 * compute_bandwidth (openmp/util/utility.cpp:23-25): GiB/s of num words. */
double orc_compute_bandwidth(uint64_t num, int word_size, double ms) {
  return 1.0 * (double)num / 1024 / 1024 / 1024 * word_size / ms * 1000;
}

static int cmp_double(const void *a, const void *b) {
  const double x = *(const double *)a, y = *(const double *)b;
  return (x > y) - (x < y);
}

/* average_Hampel (openmp/util/utility.cpp:27-71): mean of the samples whose
 * distance from the median is within 3.5 scaled MADs (MAD / 0.6745); if the
 * MAD is 0, the mean of the samples equal to the median. */
double orc_average_hampel(const double *x, int n) {
  if (n <= 0) return 0.0;
  double *s = (double *)malloc(sizeof(double) * (size_t)n);
  double *d = (double *)malloc(sizeof(double) * (size_t)n);
  if (!s || !d) {
    free(s);
    free(d);
    return 0.0;
  }
  memcpy(s, x, sizeof(double) * (size_t)n);
  qsort(s, (size_t)n, sizeof(double), cmp_double);
  const double med = (n % 2 == 0) ? 0.5 * (s[n / 2 - 1] + s[n / 2]) : s[(n - 1) / 2];
  for (int i = 0; i < n; ++i) d[i] = fabs(s[i] - med);
  double *ds = (double *)malloc(sizeof(double) * (size_t)n);
  if (!ds) {
    free(s);
    free(d);
    return 0.0;
  }
  memcpy(ds, d, sizeof(double) * (size_t)n);
  qsort(ds, (size_t)n, sizeof(double), cmp_double);
  double mad = (n % 2 == 0) ? 0.5 * (ds[n / 2 - 1] + ds[n / 2]) : ds[(n - 1) / 2];
  mad /= 0.6745;
  double total = 0.0;
  int valid = 0;
  for (int i = 0; i < n; ++i) {
    if (mad == 0.0) {
      if (d[i] == 0.0) {
        total += s[i];
        valid++;
      }
    } else if (d[i] / mad <= 3.5) {
      total += s[i];
      valid++;
    }
  }
  free(s);
  free(d);
  free(ds);
  return valid ? total / valid : 0.0;
}

/* ---- literal restatement of the OpenCL WI_split order --------------------------
 * WI_histogram / WI_shuffle (opencl/kernels/split_kernel.cl:335-412) with
 * compute_mixed_access (scan_global_RSS_kernel.cl:37-48): work-item g of G =
 * local_size * grid_size, step = min(local_size, 32), tile = ceil(n / G),
 * warp = g / step, begin = warp*step*tile + g%step, end = min((warp+1)*step*tile, n);
 * g visits i = begin, begin+step, ... < end.  Histogram his[b*G + g], exclusive
 * scan over (b, g), then each g writes its elements at his[b*G + g]++ in
 * visiting order.  aos != 0: int32 pairs keyed on the first. */
void orc_split_wi(const int32_t *in, const int32_t *vals, int64_t n, int buckets, int aos,
                  int local_size, int grid_size, int32_t *out, int32_t *vals_out) {
  const uint32_t mask = (uint32_t)buckets - 1u;
  const int64_t G = (int64_t)local_size * grid_size;
  const int64_t step = local_size < 32 ? local_size : 32;
  const int64_t tile = (n + G - 1) / G;
  int64_t *his = (int64_t *)calloc((size_t)(buckets * G), sizeof(int64_t));
  if (!his) return;
  for (int64_t g = 0; g < G; ++g) {
    const int64_t warp = g / step;
    const int64_t begin = warp * step * tile + (g % step);
    int64_t end = (warp + 1) * step * tile;
    if (end > n) end = n;
    for (int64_t i = begin; i < end; i += step) {
      const uint32_t b = (uint32_t)(aos ? in[2 * i] : in[i]) & mask;
      his[(int64_t)b * G + g]++;
    }
  }
  int64_t acc = 0;
  for (int64_t k = 0; k < (int64_t)buckets * G; ++k) {
    const int64_t v = his[k];
    his[k] = acc;
    acc += v;
  }
  for (int64_t g = 0; g < G; ++g) {
    const int64_t warp = g / step;
    const int64_t begin = warp * step * tile + (g % step);
    int64_t end = (warp + 1) * step * tile;
    if (end > n) end = n;
    for (int64_t i = begin; i < end; i += step) {
      const uint32_t b = (uint32_t)(aos ? in[2 * i] : in[i]) & mask;
      const int64_t p = his[(int64_t)b * G + g]++;
      if (aos) {
        out[2 * p] = in[2 * i];
        out[2 * p + 1] = in[2 * i + 1];
      } else {
        out[p] = in[i];
        if (vals) vals_out[p] = vals[i];
      }
    }
  }
  free(his);
}

/* ---- join match count ----------------------------------------------------------
 * The number of (r, s) pairs with equal keys, the res_len of the reference's
 * partitioned hash join (obsolete/OpenCL/phjImpl.cpp:14-129): sort both key
 * lists and merge runs of equal keys. */
static int cmp_i32(const void *a, const void *b) {
  const int32_t x = *(const int32_t *)a, y = *(const int32_t *)b;
  return (x > y) - (x < y);
}

uint64_t orc_join_count(const int32_t *r, int64_t r_len, const int32_t *s, int64_t s_len) {
  int32_t *a = (int32_t *)malloc(sizeof(int32_t) * (size_t)(r_len ? r_len : 1));
  int32_t *b = (int32_t *)malloc(sizeof(int32_t) * (size_t)(s_len ? s_len : 1));
  if (!a || !b) {
    free(a);
    free(b);
    return 0;
  }
  memcpy(a, r, sizeof(int32_t) * (size_t)r_len);
  memcpy(b, s, sizeof(int32_t) * (size_t)s_len);
  qsort(a, (size_t)r_len, sizeof(int32_t), cmp_i32);
  qsort(b, (size_t)s_len, sizeof(int32_t), cmp_i32);
  uint64_t total = 0;
  int64_t i = 0, j = 0;
  while (i < r_len && j < s_len) {
    if (a[i] < b[j]) ++i;
    else if (a[i] > b[j]) ++j;
    else {
      const int32_t k = a[i];
      int64_t ci = 0, cj = 0;
      while (i < r_len && a[i] == k) ++i, ++ci;
      while (j < s_len && b[j] == k) ++j, ++cj;
      total += (uint64_t)ci * (uint64_t)cj;
    }
  }
  free(a);
  free(b);
  return total;
}

/* ---- seeded inputs for the CPU side of the benchmark ----------------------
 * Draw i of stream `seed` is splitmix64's output function (Steele, Lea, Flood,
 * OOPSLA 2014) applied to seed + (i+1)*golden-gamma; a draw bounded to [0, r)
 * is Lemire's multiply-shift on its high 32 bits.  The permutation is
 * Durstenfeld's Fisher-Yates: for i = n-1 .. 1, swap a[i] with a[j],
 * j = bounded(draw k, i+1), k = n-1-i.  The reference's own generator
 * (random_generator_int_unique, openmp/util/utility.cpp:90-104) seeds from
 * time() and is not reproducible, so both sides of a comparison are fed this
 * one; it gives the same array as the library's data generator, which a CPU
 * test checks. */
static uint64_t orc_mix64(uint64_t z) {
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

void orc_gen_permutation_i32(int32_t *out, int64_t n, uint64_t seed) {
  for (int64_t i = 0; i < n; ++i) out[i] = (int32_t)i;
  for (int64_t i = n - 1; i > 0; --i) {
    const uint64_t x = orc_mix64(seed + (uint64_t)(n - i) * 0x9E3779B97F4A7C15ull);
    const int64_t j = (int64_t)(((x >> 32) * (uint64_t)(i + 1)) >> 32);
    const int32_t t = out[i];
    out[i] = out[j];
    out[j] = t;
  }
}
