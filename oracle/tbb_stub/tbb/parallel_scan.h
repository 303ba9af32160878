// Serial stand-in for tbb::parallel_scan: the whole range goes to the body
// in one final-scan call, which is a valid (one-chunk) execution of
// parallel_scan's contract.  Used only to build the reference's
// openmp/test_scan_CPU.cpp as an oracle.  Test infrastructure only.
#pragma once
namespace tbb {
struct split {};
struct pre_scan_tag {
  static bool is_final_scan() { return false; }
};
struct final_scan_tag {
  static bool is_final_scan() { return true; }
};
class auto_partitioner {};
template <typename Range, typename Body>
void parallel_scan(const Range &range, Body &body, const auto_partitioner &) {
  body(range, final_scan_tag());
}
}  // namespace tbb
