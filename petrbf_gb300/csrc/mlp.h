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
// BF16 copy used by the GEMMs, Adam moments, gradients and the activations of the last
// forward pass.
struct Mlp {
  DevBuf<float> w, grad, m1, m2;
  DevBuf<__nv_bfloat16> wb;
  DevBuf<float> acts[MLP_LAYERS];
  DevBuf<float> dact[2];
  int step = 0;
  bool ready = false;
  void init(uint64_t seed, cudaStream_t s);
  void set_weights(const float* host, cudaStream_t s);
  size_t woff(int l) const;
  void forward(const float* X, int n, cudaStream_t s);
  void backward(const float* X, const float* T, const float* Msk, int n, float inv_cnt, float* dloss, cudaStream_t s);
  void adam(float lr, cudaStream_t s);
  const float* out() const { return acts[MLP_LAYERS - 1].get(); }
};

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
