// rasm.h -- restricted additive Schwarz preconditioner (rasm.cu).
#pragma once
#include "context.h"

namespace prbf {

struct RasmPlan {
  bool fp32 = false;
  int ncell = 0, nblocks = 0;
  int max_nb = 0, max_nc = 0;
  int nfallback = 0;          // blocks that needed a diagonal-shift retry
  DevBuf<long long> boff;     // buffer-list offsets per cell (ncell + 1)
  DevBuf<int> idx;            // buffer lists (sorted positions), centre first
  DevBuf<long long> soff;     // S_c offsets per cell (n_c * n_b each)
  bool factor = false;        // apply by triangular solves with the kept factor (FP64 form)
  DevBuf<long long> loff;     // packed-factor offsets per cell (n_b (n_b + 1) / 2 each)
  DevBuf<double> L64;         // packed Cholesky factors (FP64 form), rows in block order
  DevBuf<float> S32;          // S_c (FP32 form)
};

// Buffer lists, blocks, factorisations and S_c for every non-empty cell of P.
// ws_budget_bytes bounds the per-batch workspace (blocks are processed in batches).
void rasm_build(RasmPlan& R, const PointSet& P, bool fp32, Workspace& ws, unsigned* err, cudaStream_t s,
                double ws_budget_bytes);
// Sets the dynamic shared memory limit of the apply kernel for this plan.
void rasm_set_apply_smem(const RasmPlan& R);
// out[centre(c)] = S_c r[buffer(c)] for every cell (sorted order, n entries).
void rasm_apply(const RasmPlan& R, const int* cs, const double* r, double* out, cudaStream_t s,
                const int* skip = nullptr);

}  // namespace prbf
