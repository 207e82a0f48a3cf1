// mlp.cu -- the learned initial guess: a per-cell MLP that maps the particles of a 3 x 3
// neighbourhood of fine cells to the weights of the centre cell, and its training.
//
// Fine cells: the same grid construction as the solver's cells with a 2-sigma edge (about
// 6 points per cell at h = 0.8 sigma), so a 3 x 3 neighbourhood holds at most ~64 points.
// Patch features, per slot k < 64 (centre cell first, then the neighbour cells in column
// order): (dx/sigma, dy/sigma, f/s, 1), zeros for empty slots, where s = max |f| over the
// whole problem. Outputs: the first 16 points of the centre
// cell, as t = g * rho / s with rho the patch's point density, so the map is independent
// of the lattice spacing and of the field's amplitude; g = t * s / rho. (A per-patch s
// would make t unbounded where the local field is small but the weights still carry the
// tail of A^-1 applied to the field nearby.)
// Network: 256 -> 256 -> 256 -> 256 -> 16, ReLU after the three hidden layers; BF16
// weights (an FP32 master copy for Adam). Every GEMM of the forward and backward passes runs
// on the tensor cores (gemm_bf16_tc, tcgen05.mma kind::f16: BF16 operands, FP32
// accumulation): the features, activations and output gradients are rounded to BF16 as
// GEMM operands; the activations, biases, loss, bias gradients and weight gradients stay
// FP32. The weight gradient dW = dZ^T H and the input gradient dH = dZ W take K-major
// operands, so dZ, H and W are also kept transposed (BF16).
#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "mlp.h"

namespace prbf {
namespace {

// dY = 2 mask (Y - T) / sum(mask); loss partial sums
__global__ void k_mse(int n, const float* __restrict__ Y, const float* __restrict__ T, const float* __restrict__ Msk,
                      float inv_cnt, float* __restrict__ dY, float* __restrict__ loss) {
  float l = 0.f;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    float d = (Y[i] - T[i]) * Msk[i];
    dY[i] = 2.f * d * inv_cnt;
    l += d * d;
  }
  l = warp_sum(l);
  if ((threadIdx.x & 31) == 0) atomicAdd(loss, l * inv_cnt);
}

// dZ = dH * (H > 0)
__global__ void k_relu_back(int n, const float* __restrict__ H, float* __restrict__ dH) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    if (!(H[i] > 0.f)) dH[i] = 0.f;
}

// db[j] = sum_m dZ[m][j]
__global__ void k_colsum(int M, int N, const float* __restrict__ dZ, float* __restrict__ db) {
  int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= N) return;
  float s = 0.f;
  for (int m = 0; m < M; m++) s += dZ[(long long)m * N + j];
  db[j] = s;
}

__global__ void k_adam(int n, float* __restrict__ w, const float* __restrict__ g, float* __restrict__ m1,
                       float* __restrict__ m2, __nv_bfloat16* __restrict__ wb, float lr, float b1, float b2, float c1,
                       float c2, float eps) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    float gi = g[i];
    float a = b1 * m1[i] + (1.f - b1) * gi;
    float b = b2 * m2[i] + (1.f - b2) * gi * gi;
    m1[i] = a;
    m2[i] = b;
    float wi = w[i] - lr * (a * c1) / (sqrtf(b * c2) + eps);
    w[i] = wi;
    if (wb) wb[i] = __float2bfloat16_rn(wi);
  }
}

__global__ void k_to_bf16(long long n, const float* __restrict__ w, __nv_bfloat16* __restrict__ wb) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    wb[i] = __float2bfloat16_rn(w[i]);
}

// dst[c][r] = src[r][c] for a rows x cols BF16 matrix (leading dimensions lds, ldd); 32 x 32
// tiles through shared memory, 32 x 8 threads.
__global__ void k_transpose_bf16(int rows, int cols, const __nv_bfloat16* __restrict__ src, int lds,
                                 __nv_bfloat16* __restrict__ dst, int ldd) {
  __shared__ __nv_bfloat16 t[32][33];
  const int c0 = blockIdx.x * 32, r0 = blockIdx.y * 32;
  for (int k = threadIdx.y; k < 32; k += 8) {
    const int r = r0 + k, c = c0 + threadIdx.x;
    if (r < rows && c < cols) t[k][threadIdx.x] = src[(long long)r * lds + c];
  }
  __syncthreads();
  for (int k = threadIdx.y; k < 32; k += 8) {
    const int c = c0 + k, r = r0 + threadIdx.x;
    if (r < rows && c < cols) dst[(long long)c * ldd + r] = t[threadIdx.x][k];
  }
}

void transpose_bf16(int rows, int cols, const __nv_bfloat16* src, int lds, __nv_bfloat16* dst, int ldd,
                    cudaStream_t s) {
  dim3 grid((cols + 31) / 32, (rows + 31) / 32);
  k_transpose_bf16<<<grid, dim3(32, 8), 0, s>>>(rows, cols, src, lds, dst, ldd);
  PRBF_CHECK_LAUNCH();
}

void to_bf16(long long n, const float* src, __nv_bfloat16* dst, cudaStream_t s) {
  k_to_bf16<<<(int)std::min<long long>((n + 255) / 256, 4 * 152), 256, 0, s>>>(n, src, dst);
  PRBF_CHECK_LAUNCH();
}

// ---- patches ----------------------------------------------------------------------------
// One warp per fine cell. X[c][4k .. 4k+3] = (dx/sigma, dy/sigma, f/s, 1) for patch slot k,
// scale[c] = s / rho, T[c][j] = g_j rho / s and Msk[c][j] = 1 for the centre's first 16 points.
__global__ void k_patches(Grid g, const double* __restrict__ x, const double* __restrict__ y,
                          const double* __restrict__ f, const double* __restrict__ gw, const int* __restrict__ cs,
                          const int* __restrict__ cells, int ncells, double s, float* __restrict__ X,
                          float* __restrict__ scale, float* __restrict__ T, float* __restrict__ Msk) {
  int wc = blockIdx.x * (blockDim.x / 32) + (threadIdx.x >> 5);
  int lane = threadIdx.x & 31;
  if (wc >= ncells) return;
  int c = cells[wc];
  int ix, iy, iz;
  cell_xyz(g, c, ix, iy, iz);
  double xc = centre_coord(g.xmin, ix, g.box), yc = centre_coord(g.ymin, iy, g.box);
  double inv_s = 1.0 / g.sigma;
  int jx0 = max(0, ix - 1), jx1 = min(g.nx - 1, ix + 1), jy0 = max(0, iy - 1), jy1 = min(g.ny - 1, iy + 1);
  float* Xc = X + (long long)wc * MLP_IN;
  for (int k = lane; k < MLP_IN; k += 32) Xc[k] = 0.f;
  __syncwarp();
  // point density of the window
  int total = 0;
  for (int jx = jx0; jx <= jx1; jx++) total += cs[cell_of(g, jx, jy1, 0) + 1] - cs[cell_of(g, jx, jy0, 0)];
  double area = (double)((jx1 - jx0 + 1) * (jy1 - jy0 + 1)) * g.box * g.box;
  double rho = total / area;
  if (lane == 0) scale[wc] = (float)(s / rho);
  // pass 2: slots, centre cell first
  int c0 = cs[c], c1 = cs[c + 1];
  int slot = 0;
  auto put = [&](int j, int k) {
    if (k >= MLP_PTS) return;
    Xc[4 * k + 0] = (float)((x[j] - xc) * inv_s);
    Xc[4 * k + 1] = (float)((y[j] - yc) * inv_s);
    Xc[4 * k + 2] = (float)(f[j] / s);
    Xc[4 * k + 3] = 1.f;
  };
  for (int j = c0 + lane; j < c1; j += 32) put(j, j - c0);
  slot = c1 - c0;
  for (int jx = jx0; jx <= jx1; jx++) {
    int a = cs[cell_of(g, jx, jy0, 0)], b = cs[cell_of(g, jx, jy1, 0) + 1];
    for (int j0 = a; j0 < b; j0 += 32) {
      int j = j0 + lane;
      bool in = j < b && !(j >= c0 && j < c1);
      unsigned bal = __ballot_sync(0xffffffffu, in);
      if (in) put(j, slot + __popc(bal & ((1u << lane) - 1u)));
      slot += __popc(bal);
    }
  }
  if (T) {
    for (int q = lane; q < MLP_OUT; q += 32) {
      int j = c0 + q;
      bool has = j < c1;
      T[(long long)wc * MLP_OUT + q] = has ? (float)(gw[j] * rho / s) : 0.f;
      Msk[(long long)wc * MLP_OUT + q] = has ? 1.f : 0.f;
    }
  }
}

// g[cs[c] + j] = Y[c][j] * scale[c] for the centre points (fine-sorted order)
__global__ void k_unpatch(const int* __restrict__ cs, const int* __restrict__ cells, int ncells,
                          const float* __restrict__ Y, const float* __restrict__ scale, double* __restrict__ gout) {
  int wc = blockIdx.x;
  if (wc >= ncells) return;
  int c = cells[wc];
  int c0 = cs[c], c1 = cs[c + 1];
  for (int q = threadIdx.x; q < c1 - c0; q += blockDim.x)
    gout[c0 + q] = q < MLP_OUT ? (double)Y[(long long)wc * MLP_OUT + q] * (double)scale[wc] : 0.0;
}

__global__ void k_maxabs(int n, const double* __restrict__ f, double* __restrict__ part) {
  double m = 0.0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) m = fmax(m, fabs(f[i]));
  for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
  __shared__ double sh[8];
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = m;
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int k = 1; k < (int)(blockDim.x >> 5); k++) m = fmax(m, sh[k]);
    part[blockIdx.x] = m;
  }
}

__global__ void k_nonempty(int ncell, const int* __restrict__ cs, int* __restrict__ flag) {
  int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c < ncell) flag[c] = cs[c + 1] > cs[c] ? 1 : 0;
}

__global__ void k_compact(int ncell, const int* __restrict__ cs, const int* __restrict__ pos, int* __restrict__ cells) {
  int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c < ncell && cs[c + 1] > cs[c]) cells[pos[c]] = c;
}

uint64_t splitmix(uint64_t& s) {
  uint64_t z = (s += 0x9E3779B97F4A7C15ull);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

}  // namespace

const int kLayerIn[MLP_LAYERS] = {MLP_IN, MLP_HID, MLP_HID, MLP_HID};
const int kLayerOut[MLP_LAYERS] = {MLP_HID, MLP_HID, MLP_HID, MLP_OUT};

size_t mlp_param_count() {
  size_t n = 0;
  for (int l = 0; l < MLP_LAYERS; l++) n += (size_t)kLayerIn[l] * kLayerOut[l] + kLayerOut[l];
  return n;
}

void Mlp::init(uint64_t seed, cudaStream_t s) {
  size_t np = mlp_param_count();
  w.reserve(np);
  wb.reserve(np);
  grad.reserve(np);
  m1.reserve(np);
  m2.reserve(np);
  std::vector<float> h(np);
  size_t o = 0;
  uint64_t st = seed;
  for (int l = 0; l < MLP_LAYERS; l++) {
    float bound = std::sqrt(6.0f / (float)kLayerIn[l]);  // He-uniform for ReLU layers
    if (l == MLP_LAYERS - 1) bound = std::sqrt(3.0f / (float)kLayerIn[l]);
    for (int i = 0; i < kLayerIn[l] * kLayerOut[l]; i++) {
      double u = (double)(splitmix(st) >> 11) * (1.0 / 9007199254740992.0);
      h[o++] = (float)((2.0 * u - 1.0) * bound);
    }
    for (int i = 0; i < kLayerOut[l]; i++) h[o++] = 0.f;
  }
  set_weights(h.data(), s);
  PRBF_CUDA(cudaMemsetAsync(m1.get(), 0, sizeof(float) * np, s));
  PRBF_CUDA(cudaMemsetAsync(m2.get(), 0, sizeof(float) * np, s));
  step = 0;
}

void Mlp::set_weights(const float* host, cudaStream_t s) {
  size_t np = mlp_param_count();
  w.reserve(np);
  PRBF_CUDA(cudaMemcpyAsync(w.get(), host, sizeof(float) * np, cudaMemcpyHostToDevice, s));
  refresh_bf16(s);
  if (!err.get()) {
    err.reserve(4);
    PRBF_CUDA(cudaMemsetAsync(err.get(), 0, 16, s));
  }
  ready = true;
}

void Mlp::refresh_bf16(cudaStream_t s) {
  const size_t np = mlp_param_count();
  wb.reserve(np);
  wbT.reserve(np);
  to_bf16((long long)np, w.get(), wb.get(), s);
  for (int l = 0; l < MLP_LAYERS; l++)
    transpose_bf16(kLayerOut[l], kLayerIn[l], wb.get() + woff(l), kLayerIn[l], wbT.get() + woff(l), kLayerOut[l], s);
}

void Mlp::check(cudaStream_t s) {
  unsigned h = 0;
  PRBF_CUDA(cudaMemcpyAsync(&h, err.get(), sizeof(unsigned), cudaMemcpyDeviceToHost, s));
  PRBF_CUDA(cudaStreamSynchronize(s));
  if (h) {
    PRBF_CUDA(cudaMemsetAsync(err.get(), 0, sizeof(unsigned), s));
    throw Error(PRBF_ERR_TIMEOUT, "network GEMM: bounded device wait gave up");
  }
}

size_t Mlp::woff(int l) const {
  size_t o = 0;
  for (int k = 0; k < l; k++) o += (size_t)kLayerIn[k] * kLayerOut[k] + kLayerOut[k];
  return o;
}

// Forward for n rows of X (device); the activations (FP32, and BF16 as the next GEMM's
// operand) are kept for the backward pass.
void Mlp::forward(const float* X, int n, cudaStream_t s) {
  xb.reserve((size_t)n * MLP_IN);
  to_bf16((long long)n * MLP_IN, X, xb.get(), s);
  const __nv_bfloat16* in = xb.get();
  for (int l = 0; l < MLP_LAYERS; l++) {
    acts[l].reserve((size_t)n * kLayerOut[l]);
    const bool hidden = l < MLP_LAYERS - 1;
    if (hidden) actb[l].reserve((size_t)n * kLayerOut[l]);
    const size_t o = woff(l);
    const float* b = w.get() + o + (size_t)kLayerIn[l] * kLayerOut[l];
    gemm_bf16_tc(n, kLayerOut[l], kLayerIn[l], in, kLayerIn[l], wb.get() + o, kLayerIn[l], acts[l].get(),
                 kLayerOut[l], hidden ? actb[l].get() : nullptr, kLayerOut[l], b, hidden, err.get(), s);
    if (hidden) in = actb[l].get();
  }
}

// Loss and gradients (into grad) for n rows; returns nothing, loss accumulated on device.
void Mlp::backward(const float* X, const float* T, const float* Msk, int n, float inv_cnt, float* dloss,
                   cudaStream_t s) {
  size_t np = mlp_param_count();
  dact[0].reserve((size_t)n * MLP_HID);
  dact[1].reserve((size_t)n * MLP_HID);
  float* dY = dact[0].get();
  k_mse<<<256, 256, 0, s>>>(n * MLP_OUT, acts[MLP_LAYERS - 1].get(), T, Msk, inv_cnt, dY, dloss);
  PRBF_CHECK_LAUNCH();
  (void)np;
  (void)X;  // its BF16 copy from the forward pass is the first layer's operand
  const int ldn = (n + 7) / 8 * 8;  // transposed operands: rows padded to 16 bytes
  dzb.reserve((size_t)n * MLP_HID);
  dzT.reserve((size_t)MLP_HID * ldn);
  hT.reserve((size_t)MLP_HID * ldn);
  float* dcur = dY;
  for (int l = MLP_LAYERS - 1; l >= 0; l--) {
    const int K = kLayerIn[l], N = kLayerOut[l];
    const __nv_bfloat16* Hin = l > 0 ? actb[l - 1].get() : xb.get();
    size_t o = woff(l);
    to_bf16((long long)n * N, dcur, dzb.get(), s);
    transpose_bf16(n, N, dzb.get(), N, dzT.get(), ldn, s);
    transpose_bf16(n, K, Hin, K, hT.get(), ldn, s);
    // dW[N][K] = dZ^T Hin (the batch is the inner dimension) ; db = colsum dZ (FP32)
    gemm_bf16_tc(N, K, n, dzT.get(), ldn, hT.get(), ldn, grad.get() + o, K, nullptr, 0, nullptr, false, err.get(), s);
    k_colsum<<<(N + 127) / 128, 128, 0, s>>>(n, N, dcur, grad.get() + o + (size_t)K * N);
    PRBF_CHECK_LAUNCH();
    if (l > 0) {
      float* dprev = dact[(MLP_LAYERS - l) & 1].get();
      // dH[n][K] = dZ W, W^T [K][N] as the K-major operand
      gemm_bf16_tc(n, K, N, dzb.get(), N, wbT.get() + o, N, dprev, K, nullptr, 0, nullptr, false, err.get(), s);
      k_relu_back<<<256, 256, 0, s>>>(n * K, acts[l - 1].get(), dprev);
      PRBF_CHECK_LAUNCH();
      dcur = dprev;
    }
  }
}

void Mlp::adam(float lr, cudaStream_t s) {
  step++;
  const float b1 = 0.9f, b2 = 0.999f;
  float c1 = 1.f / (1.f - std::pow(b1, (float)step)), c2 = 1.f / (1.f - std::pow(b2, (float)step));
  k_adam<<<256, 256, 0, s>>>((int)mlp_param_count(), w.get(), grad.get(), m1.get(), m2.get(), nullptr, lr, b1, b2, c1,
                             c2, 1e-8f);
  PRBF_CHECK_LAUNCH();
  refresh_bf16(s);
}

int fine_cells(Ctx& c, PointSet& P, Workspace& ws, DevBuf<int>& cells) {
  const Grid& g = P.g;
  int* flag = (int*)ws.get(60, sizeof(int) * ((size_t)g.ncell + 1));
  k_nonempty<<<ceil_div(g.ncell, 256), 256, 0, c.stream>>>(g.ncell, P.cs.get(), flag);
  PRBF_CUDA(cudaMemsetAsync(flag + g.ncell, 0, sizeof(int), c.stream));
  scan_exclusive_dev(flag, flag, (long long)g.ncell + 1, ws, 61, c.stream);
  int nne = 0;
  PRBF_CUDA(cudaMemcpyAsync(&nne, flag + g.ncell, sizeof(int), cudaMemcpyDeviceToHost, c.stream));
  PRBF_CUDA(cudaStreamSynchronize(c.stream));
  cells.reserve(std::max(nne, 1));
  k_compact<<<ceil_div(g.ncell, 256), 256, 0, c.stream>>>(g.ncell, P.cs.get(), flag, cells.get());
  PRBF_CHECK_LAUNCH();
  return nne;
}

double max_abs_dev(Ctx& c, int n, const double* f) {
  double* part = (double*)c.ws.get(62, sizeof(double) * 256);
  k_maxabs<<<256, 256, 0, c.stream>>>(n, f, part);
  PRBF_CHECK_LAUNCH();
  double h[256];
  PRBF_CUDA(cudaMemcpyAsync(h, part, sizeof(h), cudaMemcpyDeviceToHost, c.stream));
  PRBF_CUDA(cudaStreamSynchronize(c.stream));
  double m = 0.0;
  for (double v : h) m = std::max(m, v);
  return m;
}

void patches_dev(Ctx& c, const PointSet& P, const double* f_sorted, const double* g_sorted, const int* cells,
                 int ncells, float* X, float* scale, float* T, float* Msk) {
  double s = max_abs_dev(c, P.n, f_sorted);
  if (!(s > 0)) s = 1.0;
  k_patches<<<ceil_div(ncells, 8), 256, 0, c.stream>>>(P.g, P.x.get(), P.y.get(), f_sorted, g_sorted, P.cs.get(), cells,
                                                      ncells, s, X, scale, T, Msk);
  PRBF_CHECK_LAUNCH();
}

void unpatch_dev(Ctx& c, const PointSet& P, const int* cells, int ncells, const float* Y, const float* scale,
                 double* g_sorted) {
  PRBF_CUDA(cudaMemsetAsync(g_sorted, 0, sizeof(double) * P.n, c.stream));
  k_unpatch<<<ncells, 32, 0, c.stream>>>(P.cs.get(), cells, ncells, Y, scale, g_sorted);
  PRBF_CHECK_LAUNCH();
}

}  // namespace prbf
