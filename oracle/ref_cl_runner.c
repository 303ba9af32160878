/*
 * ref_cl_runner.c — runs the reference's WI_split kernels on the CPU.
 *
 * TEST INFRASTRUCTURE ONLY.  Built by oracle/build.py once per data layout
 * (-DKO, -DKVS_SOA, -DKVS_AOS, the flags the reference's host code passes to
 * its kernel compiler, opencl/primitives/splitImpl.cpp:61-64), with
 * ref_cl_shim.h force-included and REF_SPLIT_CL naming the reference's
 * opencl/kernels/split_kernel.cl, which is included below unchanged.
 *
 * ref_wi_split replays WI_split's host sequence
 * (opencl/primitives/splitImpl.cpp:21-142): WI_histogram over
 * grid_size x local_size work-items, an exclusive scan of the histogram in
 * place, WI_shuffle.  The reference scans with scan_chained (an exclusive
 * prefix sum, pinned by its own tests); a sequential exclusive scan gives
 * the same array.  Work-groups run one after another; the work-items of a
 * group run as local_size threads that meet at every barrier().
 */
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include REF_SPLIT_CL

__thread size_t edpp_cl_local_id, edpp_cl_global_id, edpp_cl_group_id;
size_t edpp_cl_local_size, edpp_cl_global_size, edpp_cl_num_groups;

static pthread_barrier_t g_bar;

void edpp_cl_barrier(void) { pthread_barrier_wait(&g_bar); }

enum { K_HIST = 0, K_SHUFFLE = 1 };

typedef struct {
  int which;
  const Tuple *in;
  Tuple *out;
  const Tuple *in_values;
  Tuple *out_values;
  int len;
  int *his;
  int buckets;
  int *local_buf;
} launch_t;

typedef struct {
  const launch_t *L;
  size_t lid;
} worker_t;

static void *work_item(void *p) {
  const worker_t *w = (const worker_t *)p;
  const launch_t *L = w->L;
  edpp_cl_local_id = w->lid;
  for (size_t g = 0; g < edpp_cl_num_groups; ++g) {
    edpp_cl_group_id = g;
    edpp_cl_global_id = g * edpp_cl_local_size + w->lid;
    if (L->which == K_HIST) {
      WI_histogram(L->in, L->len, L->his, L->buckets, L->local_buf);
    } else {
#ifdef KVS_SOA
      WI_shuffle(L->in, L->out, L->in_values, L->out_values, L->len, L->his, L->buckets,
                 L->local_buf);
#else
      WI_shuffle(L->in, L->out, L->len, L->his, L->buckets, L->local_buf);
#endif
    }
    /* the group's work-items finish before the next group reuses local memory */
    pthread_barrier_wait(&g_bar);
  }
  return NULL;
}

static int nd_range(const launch_t *L, int local_size, int grid_size) {
  edpp_cl_local_size = (size_t)local_size;
  edpp_cl_num_groups = (size_t)grid_size;
  edpp_cl_global_size = (size_t)local_size * (size_t)grid_size;
  if (pthread_barrier_init(&g_bar, NULL, (unsigned)local_size) != 0) return 1;
  pthread_t *th = (pthread_t *)calloc((size_t)local_size, sizeof(pthread_t));
  worker_t *ws = (worker_t *)calloc((size_t)local_size, sizeof(worker_t));
  int rc = (th && ws) ? 0 : 1;
  int started = 0;
  for (int i = 0; i < local_size && rc == 0; ++i) {
    ws[i].L = L;
    ws[i].lid = (size_t)i;
    if (pthread_create(&th[i], NULL, work_item, &ws[i]) != 0) rc = 1;
    else ++started;
  }
  for (int i = 0; i < started; ++i) pthread_join(th[i], NULL);
  pthread_barrier_destroy(&g_bar);
  free(th);
  free(ws);
  return started == local_size ? rc : 1;
}

/* in / out: keys (KO, SOA) or int32 pairs (AOS); vals / vals_out: SOA only.
 * Returns 0, or 1 on a parameter the reference cannot run (its histogram
 * index buckets*global_size must fit an int) or an allocation failure. */
int ref_wi_split(const int32_t *in, const int32_t *vals, int length, int buckets,
                 int local_size, int grid_size, int32_t *out, int32_t *vals_out) {
  const int64_t his_len = (int64_t)buckets * local_size * grid_size;
  if (length < 0 || buckets < 1 || local_size < 1 || grid_size < 1 || his_len >= INT32_MAX)
    return 1;
  int *his = (int *)calloc((size_t)his_len, sizeof(int));
  int *local_buf = (int *)calloc((size_t)local_size * (size_t)buckets, sizeof(int));
  if (!his || !local_buf) {
    free(his);
    free(local_buf);
    return 1;
  }
  launch_t L;
  memset(&L, 0, sizeof(L));
  L.in = (const Tuple *)in;
  L.out = (Tuple *)out;
  L.in_values = (const Tuple *)vals;
  L.out_values = (Tuple *)vals_out;
  L.len = length;
  L.his = his;
  L.buckets = buckets;
  L.local_buf = local_buf;
  L.which = K_HIST;
  int rc = nd_range(&L, local_size, grid_size);
  if (rc == 0) {
    int acc = 0;
    for (int64_t i = 0; i < his_len; ++i) {
      const int v = his[i];
      his[i] = acc;
      acc += v;
    }
    L.which = K_SHUFFLE;
    rc = nd_range(&L, local_size, grid_size);
  }
  free(his);
  free(local_buf);
  return rc;
}
