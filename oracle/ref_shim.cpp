// ref_shim.cpp — C entry points onto the reference's own OpenMP functions.
//
// TEST INFRASTRUCTURE ONLY.  Linked (by oracle/build.py) with the reference's
// openmp/test_gather_scatter_CPU.cpp, openmp/test_scan_CPU.cpp,
// openmp/test_bandwidth_CPU.cpp and openmp/util/utility.cpp, compiled from
// where they lie with their main() renamed, into oracle/_ref/libref_omp.so.
// It lets the tests check the oracle's restatement against the real
// reference on the same seeded arrays, and generate golden vectors.
#include <cstdint>

// Signatures as declared in the reference sources.
double gather(int *input, int *output, int *idx, uint64_t len);    // test_gather_scatter_CPU.cpp:24
double scatter(int *input, int *output, int *idx, uint64_t len);   // test_gather_scatter_CPU.cpp:34
double scan_SSA_omp(int *input, int *output, uint64_t len);        // test_scan_CPU.cpp:85
double scan_RTS_omp(int *input, int *output, uint64_t len);        // test_scan_CPU.cpp:125
double scan_tbb(int *input, int *output, uint64_t len);            // test_scan_CPU.cpp:77
double copy_omp(int *input, int *output, uint64_t len);            // test_bandwidth_CPU.cpp:39
double scale_omp(int *input, int *output, uint64_t len);           // test_bandwidth_CPU.cpp:49
double average_Hampel(double *input, int num);                     // util/utility.cpp:27
double compute_bandwidth(uint64_t num, int wordSize, double kernel_time);  // util/utility.cpp:23

extern "C" {
double ref_gather(int *in, int *out, int *idx, uint64_t n) { return gather(in, out, idx, n); }
double ref_scatter(int *in, int *out, int *idx, uint64_t n) { return scatter(in, out, idx, n); }
double ref_scan_ssa(int *in, int *out, uint64_t n) { return scan_SSA_omp(in, out, n); }
double ref_scan_rts(int *in, int *out, uint64_t n) { return scan_RTS_omp(in, out, n); }
double ref_scan_tbb(int *in, int *out, uint64_t n) { return scan_tbb(in, out, n); }
double ref_copy(int *in, int *out, uint64_t n) { return copy_omp(in, out, n); }
double ref_scale(int *in, int *out, uint64_t n) { return scale_omp(in, out, n); }
double ref_average_hampel(double *x, int n) { return average_Hampel(x, n); }
double ref_compute_bandwidth(uint64_t num, int w, double ms) { return compute_bandwidth(num, w, ms); }
}
