// edpp_primitives.hpp — the reference's primitive API, on GB300.
//
// Same function names, argument order and return convention as
// Efficient-DPP's opencl/primitives.h:12-49 (types from opencl/types.h:8-47),
// so the reference's test drivers port by swapping cl_mem for device
// pointers:
//   - every call is synchronous and returns the elapsed device time in
//     milliseconds, as the reference sums clEventTime over its launches;
//   - parameter errors return -1 (WI_split / WG_split / single_split,
//     opencl/primitives/splitImpl.cpp:32,43,378,388) or 1 (scan_chained with
//     R == L == 0, opencl/primitives/scanImpl.cpp:19-22), as the reference
//     does; a CUDA error or an expired device wait also returns -1 where the
//     reference would exit() the process;
//   - temporaries are allocated per call from CUDA's stream-ordered pool, as
//     the reference creates and releases d_inter / d_reduction / d_his per call;
//   - work is issued on the legacy default stream.
// Tuning knobs the reference exposes (localSize, gridSize, R, L, local_size,
// grid_size) are validated the way the reference validates them and otherwise
// ignored: the GB300 kernels choose their own launch shapes.
//
// Split order: every split here returns the stable order (elements grouped by
// bucket = key & (buckets-1), input order kept inside a bucket).  That is
// exactly the output of the reference's single_split and WG_split with
// FIXED_REORDER; for WG_split with NO_REORDER / VARIED_REORDER the reference's
// order is non-deterministic (local atomics) and the stable order is one of
// its possible outputs; WI_split's reference order interleaves work-items and
// differs from the stable order within a bucket.
#ifndef EDPP_PRIMITIVES_HPP_
#define EDPP_PRIMITIVES_HPP_

#include <cstdint>

namespace edpp {
namespace primitives {

// opencl/types.h:8-47
enum SCAN_GLOBAL_TYPE { RSS, RSS_SINGLE_THREAD, CHAINED };
enum DataStruc { KO, KVS_AOS, KVS_SOA };
enum SPLIT_ALGO { WI, WG, WG_fixed_reorder, WG_varied_reorder, Single, Single_reorder };
enum ReorderType { NO_REORDER, FIXED_REORDER, VARIED_REORDER };

// opencl/primitives.h:12-19
double gather(const int *d_in, int *d_out, int length, const int *d_loc, int localSize,
              int gridSize, int pass);
double scatter(const int *d_in, int *d_out, int length, const int *d_loc, int localSize,
               int gridSize, int pass);

// opencl/primitives.h:22-29 (exclusive int32 scans; in-place allowed)
double scan_chained(const int *d_in, int *d_out, int length, int localSize, int gridSize, int R,
                    int L);
double scan_RSS(const int *d_in, int *d_out, unsigned length, int local_size, int grid_size);
double scan_RSS_single(const int *d_in, int *d_out, unsigned length);

// opencl/primitives.h:32-49.  For KVS_AOS, d_in / d_out hold `length` int32
// {key,value} pairs and the value arguments must be null.
double WI_split(const int *d_in, int *d_out, int *d_start, int length, int buckets,
                DataStruc structure, const int *d_in_values = nullptr, int *d_out_values = nullptr,
                int local_size = 256, int grid_size = 32768);
double WG_split(const int *d_in, int *d_out, int *d_start, int length, int buckets,
                ReorderType reorder_type, DataStruc structure, const int *d_in_values = nullptr,
                int *d_out_values = nullptr, int local_size = 256, int grid_size = 32768);
double single_split(const int *d_in, int *d_out, int length, int buckets, bool reorder,
                    DataStruc structure);

// CPU-path names of the reference's OpenMP programs, run on the GPU:
// openmp/test_gather_scatter_CPU.cpp:24,34 and openmp/test_scan_CPU.cpp:85,125.
// Arguments are device pointers; the result is elapsed device milliseconds.
double scan_SSA(const int *d_in, int *d_out, uint64_t len);
double scan_RTS(const int *d_in, int *d_out, uint64_t len);

}  // namespace primitives
}  // namespace edpp

#endif  // EDPP_PRIMITIVES_HPP_
