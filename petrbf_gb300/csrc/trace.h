// trace.h -- phase ranges for profilers. The reference brackets its phases with PETSc
// log events (2d/rbf_interpolation.cxx:47-52: InitVec, InitCluster, InitIS, InitGhost,
// InitMat, Post Processing); the library marks the same phases as NVTX ranges, so an
// Nsight or ncu timeline shows them around the kernels. NVTX is header-only: with no tool
// attached a range costs a few host instructions.
#pragma once
#include <nvtx3/nvToolsExt.h>

namespace prbf {

// A range from construction to end() or destruction, whichever comes first.
struct TraceRange {
  explicit TraceRange(const char* name) { nvtxRangePushA(name); }
  void end() {
    if (open_) nvtxRangePop();
    open_ = false;
  }
  ~TraceRange() { end(); }
  TraceRange(const TraceRange&) = delete;
  TraceRange& operator=(const TraceRange&) = delete;

 private:
  bool open_ = true;
};

}  // namespace prbf
