/*
 * ref_cl_shim.h — lets the reference's OpenCL C kernel source compile as C.
 *
 * TEST INFRASTRUCTURE ONLY.  Force-included (gcc -include) before
 * oracle/ref_cl_runner.c, which includes the reference's
 * opencl/kernels/split_kernel.cl from where it lies.  The address-space
 * qualifiers become nothing, the work-item functions read per-thread
 * variables that the runner sets, and barrier() is a barrier across the
 * threads that run one work-group's work-items (one POSIX thread each), so
 * the kernels run with their OpenCL semantics on the CPU.  OpenCL is not
 * installed anywhere this project runs; this is how the oracle gets outputs of
 * the reference's own kernels.
 */
#ifndef EDPP_REF_CL_SHIM_H_
#define EDPP_REF_CL_SHIM_H_

#include <stddef.h>

#define kernel
#define __kernel
#define global
#define __global
#define local
#define __local
#define constant const
#define __constant const
#define CLK_LOCAL_MEM_FENCE 1
#define CLK_GLOBAL_MEM_FENCE 2

typedef struct {
  int x, y;
} int2;

extern __thread size_t edpp_cl_local_id, edpp_cl_global_id, edpp_cl_group_id;
extern size_t edpp_cl_local_size, edpp_cl_global_size, edpp_cl_num_groups;

static inline size_t get_local_id(unsigned d) { return d == 0 ? edpp_cl_local_id : 0; }
static inline size_t get_global_id(unsigned d) { return d == 0 ? edpp_cl_global_id : 0; }
static inline size_t get_group_id(unsigned d) { return d == 0 ? edpp_cl_group_id : 0; }
static inline size_t get_local_size(unsigned d) { return d == 0 ? edpp_cl_local_size : 1; }
static inline size_t get_global_size(unsigned d) { return d == 0 ? edpp_cl_global_size : 1; }
static inline size_t get_num_groups(unsigned d) { return d == 0 ? edpp_cl_num_groups : 1; }

void edpp_cl_barrier(void);
#define barrier(flags) edpp_cl_barrier()
#define mem_fence(flags) __atomic_thread_fence(__ATOMIC_SEQ_CST)

static inline int atomic_inc(volatile int *p) { return __atomic_fetch_add(p, 1, __ATOMIC_SEQ_CST); }
static inline int atomic_add(volatile int *p, int v) {
  return __atomic_fetch_add(p, v, __ATOMIC_SEQ_CST);
}

#endif /* EDPP_REF_CL_SHIM_H_ */
