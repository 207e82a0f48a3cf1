// solve.cu -- rbf_interpolation on the GPU: RASM set-up and GMRES (filled in next).
#include "context.h"

namespace prbf {
struct SolveState {};
Ctx::~Ctx() {
  delete solve;
  solve = nullptr;
  ctx_stream_release(*this);
}
}  // namespace prbf
