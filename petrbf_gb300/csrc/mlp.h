// mlp.h -- the learned initial guess (mlp.cu).
#pragma once
#include <cuda_bf16.h>

#include "context.h"

namespace prbf {

constexpr int MLP_PTS = 64;               // particles per patch
constexpr int MLP_IN = 4 * MLP_PTS;       // (dx/sigma, dy/sigma, f/s, present) per particle
constexpr int MLP_HID = 256;              // width of the three hidden layers
constexpr int MLP_OUT = 16;               // centre-cell weights predicted
constexpr int MLP_LAYERS = 4;
constexpr int MLP_NBOX = 2;               // fine cell edge in sigma

extern const int kLayerIn[MLP_LAYERS];
extern const int kLayerOut[MLP_LAYERS];
size_t mlp_param_count();

// Network state: FP32 master weights (per layer: W[out][in] row-major, then b[out]), their
// BF16 copy W and its transpose W^T (same offsets, [in][out]) used by the tensor-core
// GEMMs, Adam moments, gradients, the FP32 activations of the last forward pass and their
// BF16 copies (the GEMM operands), and the device error word of the GEMMs.
struct Mlp {
  DevBuf<float> w, grad, m1, m2;
  DevBuf<__nv_bfloat16> wb, wbT;
  DevBuf<float> acts[MLP_LAYERS];
  DevBuf<float> dact[2];
  DevBuf<__nv_bfloat16> xb, actb[MLP_LAYERS - 1], dzb, dzT, hT;
  DevBuf<unsigned> err;
  int step = 0;
  bool ready = false;
  void init(uint64_t seed, cudaStream_t s);
  void set_weights(const float* host, cudaStream_t s);
  size_t woff(int l) const;
  void forward(const float* X, int n, cudaStream_t s);
  void backward(const float* X, const float* T, const float* Msk, int n, float inv_cnt, float* dloss, cudaStream_t s);
  void adam(float lr, cudaStream_t s);
  // raises PRBF_ERR_TIMEOUT if a GEMM's bounded wait gave up since the last check (syncs s)
  void check(cudaStream_t s);
  const float* out() const { return acts[MLP_LAYERS - 1].get(); }

 private:
  void refresh_bf16(cudaStream_t s);  // wb and wbT from w
};

// C[M][N] = A[M][K] B[N][K]^T (+ bias, ReLU) on the tensor cores (gemm_tc.cu): A and B
// BF16 row-major with K contiguous (leading dimensions lda, ldb multiples of 8, 16-byte
// aligned bases), FP32 accumulation; C (FP32, ldc) and/or Cb (BF16, ldcb) may be null.
// N <= 256; entries past the matrix edges read as zero.
void gemm_bf16_tc(int M, int N, int K, const __nv_bfloat16* A, int lda, const __nv_bfloat16* B, int ldb, float* C,
                  int ldc, __nv_bfloat16* Cb, int ldcb, const float* bias, bool relu, unsigned* err, cudaStream_t s);

// Non-empty fine cells of P (compacted list), returns their count.
int fine_cells(Ctx& c, PointSet& P, Workspace& ws, DevBuf<int>& cells);
// Patch features (and training targets when g_sorted/T are given) of the listed cells.
void patches_dev(Ctx& c, const PointSet& P, const double* f_sorted, const double* g_sorted, const int* cells,
                 int ncells, float* X, float* scale, float* T, float* Msk);
// g (fine-sorted order) from the network output of the listed cells.
void unpatch_dev(Ctx& c, const PointSet& P, const int* cells, int ncells, const float* Y, const float* scale,
                 double* g_sorted);

// Learned guess for n points on the device in any order; g written in the same order.
void guess_compute(Ctx& c, Mlp& net, int n, const double* x, const double* y, const double* f, double* g);

}  // namespace prbf
