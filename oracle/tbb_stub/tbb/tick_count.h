// Serial stand-in for a TBB header included by openmp/test_scan_CPU.cpp.
// Test infrastructure only.
#pragma once
namespace tbb {
class tick_count {};
}  // namespace tbb
