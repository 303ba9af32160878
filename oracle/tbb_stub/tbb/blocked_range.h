// Serial stand-in for tbb::blocked_range as used by openmp/test_scan_CPU.cpp:52-82.
// Test infrastructure only.
#pragma once
namespace tbb {
template <typename Value> class blocked_range {
 public:
  blocked_range(Value b, Value e) : b_(b), e_(e) {}
  Value begin() const { return b_; }
  Value end() const { return e_; }

 private:
  Value b_, e_;
};
}  // namespace tbb
