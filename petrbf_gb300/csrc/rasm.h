// rasm.h -- restricted additive Schwarz preconditioner (rasm.cu).
#pragma once
#include <vector>

#include "context.h"

namespace prbf {

struct RasmPlan {
  bool fp32 = false;
  bool basic = false;         // basic Schwarz (whole block solutions added) instead of restricted
  int n = 0;                  // points
  int ncell = 0, nblocks = 0;
  int max_nb = 0, max_nc = 0;
  int nfallback = 0;          // blocks that needed a diagonal-shift retry
  std::vector<int> retried;   // their cells (host)
  DevBuf<long long> boff;     // buffer-list offsets per cell (ncell + 1)
  DevBuf<int> idx;            // buffer lists (sorted positions), centre first
  DevBuf<long long> soff;     // S_c offsets per cell (n_c * n_b each)
  bool factor = false;        // apply by triangular solves with the kept factor (FP64 form)
  DevBuf<long long> loff;     // packed-factor offsets per cell (rows padded to 32 bytes FP32, 16 FP64)
  DevBuf<double> L64;         // packed Cholesky factors (FP64 factor form), rows in block order
  DevBuf<float> L32;          // packed Cholesky factors (FP32 factor form)
  DevBuf<float> S32;          // S_c (FP32 inverse-rows form)
  DevBuf<double> Y;           // basic form: block solutions, one slot per buffer-list entry
  DevBuf<long long> inv_off;  // basic form: per point, its slots (n + 1 offsets)
  DevBuf<long long> inv_slot; // basic form: the slots, ascending
  SegSkip seg;                // batches: skip the blocks of stopped problems (when seg.done set)
  int max_nv = 1;             // right-hand sides per apply launch (1..4; set before the build)
  long long nslot = 0;        // basic form: buffer-list entries (slot stride of Y)
  // FP64 form, set before the build: a block whose Cholesky meets a non-positive pivot is
  // factored by LU with partial pivoting (the reference's PETSc LU) instead of shifted
  bool lu_fallback = false;
  int nlu = 0;                     // blocks factored by LU
  std::vector<int> lu_cells;       // their cells, ascending (host)
  DevBuf<int> lucell;              // their cells (device)
  DevBuf<long long> lukoff;        // per LU block: offset of its nb x nb factor in LU64
  DevBuf<long long> lupoff;        // per LU block: offset of its nb pivot rows in lupiv
  DevBuf<int> lu_of_cell;          // per cell: its LU block, or -1 (ncell)
  DevBuf<double> LU64;             // the LU factors (row-major, unit lower L below U)
  DevBuf<int> lupiv;               // their pivot rows
  double lu_scale = 0.0;           // 2 pi sigma^2 (A^-1 = 2 pi sigma^2 K^-1)
  const double* lu_cell_sigma = nullptr;  // batches: per-cell sigma (device), else null
};

// Buffer lists, blocks, factorisations and S_c for every non-empty cell of P.
// ws_budget_bytes bounds the per-batch workspace (blocks are processed in batches).
// factor: keep the packed factors and apply by triangular solves (always for FP64 and for
// basic Schwarz; for restricted FP32 the alternative is S_c, one GEMV per apply).
// basic: PETSc's -pc_asm_type basic, z = sum_c R_c^T A_c^-1 R_c r (symmetric); otherwise
// the restricted form, z[centre(c)] = (A_c^-1 R_c r)[centre].
void rasm_build(RasmPlan& R, const PointSet& P, bool fp32, Workspace& ws, unsigned* err, cudaStream_t s,
                double ws_budget_bytes, bool factor = false, bool basic = false);
// Geometry of the blocks: cell-sorted points and cell starts (device, global indices),
// with one sigma (single problem) or one per cell (a batch of problems).
struct BlockGeom {
  int dim = 2, n = 0, ncell = 0;
  const double *x = nullptr, *y = nullptr, *z = nullptr;
  const int* cs = nullptr;
  double sigma = 0.0;
  const double* cell_sigma = nullptr;
};
// Buffer lists of one grid (get_buffer): counts per cell when boff_dev is null, else the
// lists at boff_dev (sorted positions of P, centre first).
void rasm_buffer_lists(const PointSet& P, int* counts_dev, const long long* boff_dev, int* idx_dev, cudaStream_t s);
// Factorisation of every non-empty block, with R.boff / R.idx already in place (global
// indices) and their host sizes: hcnt[c] block sizes, hcs the cell starts.
void rasm_factor(RasmPlan& R, const BlockGeom& G, const std::vector<int>& hcnt, const std::vector<int>& hcs, bool fp32,
                 Workspace& ws, unsigned* err, cudaStream_t s, double ws_budget_bytes, bool factor, bool basic);
// K = 2 pi sigma^2 A_c of one block of a single-problem plan, as the FP64 factorisation
// assembles it (rows neighbours first, lower triangle, no diagonal shift), into K_dev
// (nb x nb, zeroed first). Synchronises the stream.
void rasm_block_K(const RasmPlan& R, const PointSet& P, int cell, int nb, double* K_dev, Workspace& ws,
                  cudaStream_t s);
// The FP64 factor of one block as stored (row i: L_A[i][0..i-1] then 1/L_A[i][i]), the
// rows' padding removed, into out (host, nb (nb + 1) / 2 entries). PRBF_ERR_STATE for a
// block factored by LU.
void rasm_factor_rows(const RasmPlan& R, int cell, int nb, double* out, cudaStream_t s);
// Sets the dynamic shared memory limit of the apply kernel for this plan.
void rasm_set_apply_smem(const RasmPlan& R);
// Restricted: out[centre(c)] = (A_c^-1 r[buffer(c)])[centre] for every cell; basic:
// out = sum_c R_c^T A_c^-1 R_c r (sorted order, n entries).
// nv vectors at stride vstride (applied up to min(4, R.max_nv) at a time; the factor is
// read once per launch for all of them).
void rasm_apply(const RasmPlan& R, const int* cs, const double* r, double* out, cudaStream_t s,
                const int* skip = nullptr, int nv = 1, long long vstride = 0);

}  // namespace prbf
