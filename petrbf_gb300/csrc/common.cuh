// common.cuh -- shared types and device helpers of the GB300 PetRBF kernels (sm_103a).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <cstdio>
#include <stdexcept>
#include <string>

#include "../../include/petrbf_gb300.h"

namespace prbf {

// Absolute slack added to box widths and domain bounds (2d/par.h:153).
constexpr double kEpsf = 1e-6;

// Error words a kernel can raise in the context's device status word (bit flags).
enum : unsigned {
  DEV_ERR_RANGE = 1u,     // a point fell outside the cell grid
  DEV_ERR_TIMEOUT = 2u,   // a bounded mbarrier wait gave up
  DEV_ERR_CAPACITY = 4u,  // a per-CTA capacity was exceeded
  DEV_ERR_FACTOR = 8u,    // a block factorisation met a non-positive pivot
  DEV_ERR_INDEX = 16u,    // a kernel's own bounds check caught an index out of range (skipped)
};

// Host-side exception carrying a status code; converted to an int at the C ABI.
struct Error : std::runtime_error {
  int status;
  Error(int s, const std::string& m) : std::runtime_error(m), status(s) {}
};

#define PRBF_CUDA(call)                                                                  \
  do {                                                                                   \
    cudaError_t e__ = (call);                                                            \
    if (e__ != cudaSuccess)                                                              \
      throw ::prbf::Error(PRBF_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e__)); \
  } while (0)

#define PRBF_CHECK_LAUNCH() PRBF_CUDA(cudaGetLastError())

// Cell grid (2d/get_cluster.h:176-190, 3d/get_cluster.h:21-44). Passed by value.
struct Grid {
  int dim;
  int nx, ny, nz, ncell;
  int cbase;                // global index of the first cell (batches of grids; else 0)
  int nb_trunc, nb_buffer;
  double sigma;
  double xmin, ymin, zmin;  // particle minimum - epsf
  double box;               // nsigma_box*sigma + epsf
  double trunc_len;         // sigma_trunc*sigma/2 + epsf
  double buffer_len;        // sigma_buffer*sigma/2 + epsf
};

// Work of stopped systems in a batch: cell -> problem, and the problems' stop flags
// (done[prob * stride], e.g. inside the Krylov per-system state); inactive when done is null.
struct SegSkip {
  const int* cprob = nullptr;
  const int* done = nullptr;
  int stride = 0;
  __device__ bool cell_done(int c) const { return done && done[(long long)cprob[c] * stride]; }
};

__host__ __device__ inline int cell_of(const Grid& g, int ix, int iy, int iz) {
  return g.dim == 2 ? ix * g.ny + iy : (iz * g.nx + ix) * g.ny + iy;
}

__host__ __device__ inline void cell_xyz(const Grid& g, int ic, int& ix, int& iy, int& iz) {
  if (g.dim == 2) {
    ix = ic / g.ny;
    iy = ic - ix * g.ny;
    iz = 0;
  } else {
    int nxy = g.nx * g.ny;
    iz = ic / nxy;
    int r = ic - iz * nxy;
    ix = r / g.ny;
    iy = r - ix * g.ny;
  }
}

#ifdef __CUDACC__
// Cell centre xmin + (ix+0.5)*box, rounded as written (no fused multiply-add), so it is
// bit-identical to the unfused host/CPU evaluation (2d/get_cluster.h:217-218).
__device__ __forceinline__ double centre_coord(double lo, int i, double box) {
  return __dadd_rn(lo, __dmul_rn((double)i + 0.5, box));
}

// ---- TMA bulk copies (cp.async.bulk, non-tensor) and mbarriers -------------------------
__device__ __forceinline__ uint32_t smem_addr(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count));
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)),
               "r"(bytes)
               : "memory");
}

// Orders earlier generic-proxy accesses of shared memory before later async-proxy ones.
__device__ __forceinline__ void fence_proxy_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// dst (shared) <- src (global), bytes a multiple of 16, both 16-byte aligned.
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, unsigned bytes, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          smem_addr(dst)),
      "l"(src), "r"(bytes), "r"(smem_addr(bar))
      : "memory");
}

// Bounded wait on an mbarrier phase. Returns false (and the caller raises
// DEV_ERR_TIMEOUT) if the phase has not completed after max_tries polls.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, unsigned phase, unsigned max_tries = 1u << 22) {
  uint32_t addr = smem_addr(bar);
  for (unsigned t = 0; t < max_tries; ++t) {
    uint32_t done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
        : "=r"(done)
        : "r"(addr), "r"(phase)
        : "memory");
    if (done) return true;
  }
  return false;
}

// 1024 / (2 sigma^2 ln2): the exponent factor of exp_neg_tab (the host computes the same
// expression for single problems; products and a division only, so nothing is fused).
__host__ __device__ __forceinline__ double kexp_of_sigma(double sigma) {
  return 1024.0 / (2.0 * sigma * sigma * 0.6931471805599453);
}

// v * 2^-m for a normal v whose exponent stays normal (m20 = m << 20): the exponent field
// is lowered by m, exactly.
__device__ __forceinline__ double pow2_lower(double v, int m20) {
  return __hiloint2double(__double2hiint(v) - m20, __double2loint(v));
}

// exp(-d2 / (2 sigma^2)) from the sums' FP64 table (exp_table_dev: n = 1024, tab[4j + i] =
// 2^(-j/n) c_i, c_i the cubic through e^(L r) at the Chebyshev nodes of [-1/2, 1/2], L =
// ln2/n), with kexp = n / (2 sigma^2 ln2): k = rint(kexp d2), r = k - kexp d2 (one rounding),
// k = n m + j, result 2^-m (T[j] p(r)) by Horner with every operation written out, so a CPU
// restatement with the same table reproduces it bit for bit. m is capped at 900 (2^-900 ~
// 1e-271) so the scaled coefficients stay normal; the blocks never reach the cap.
__device__ __forceinline__ double exp_neg_tab(double d2, double kexp, const double* __restrict__ tab) {
  const double magic = 6755399441055744.0;  // 1.5 * 2^52: rint by addition
  const double kd = __fma_rn(d2, kexp, magic);
  const int kk = __double2loint(kd);
  const double r = __fma_rn(-d2, kexp, __dsub_rn(kd, magic));
  const int m20 = min(kk >> 10, 900) << 20;
  const double* c = tab + 4 * (kk & 1023);
  double q = pow2_lower(c[3], m20);
  q = __fma_rn(r, q, pow2_lower(c[2], m20));
  q = __fma_rn(r, q, pow2_lower(c[1], m20));
  q = __fma_rn(r, q, pow2_lower(c[0], m20));
  return q;
}

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
#endif

inline int ceil_div(long long a, long long b) { return (int)((a + b - 1) / b); }

}  // namespace prbf
