// Serial stand-in for the TBB header the reference's openmp/test_scan_CPU.cpp
// includes (TBB is not installed here).  Test infrastructure only.
#pragma once
namespace tbb {
class task_scheduler_init {};
}  // namespace tbb
