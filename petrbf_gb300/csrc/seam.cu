// seam.cu -- the reference's own C++ -> CUDA seam, gpumatmult (2d/gpumatmult.cu:65-119,
// 3d/gpumatmult.cu:73-133), with the same packed-array meaning, for callers that keep the
// reference's host packer (2d/matmultgpu.cxx:9-97, 3d/matmultgpu.cxx:9-105):
//   * iblok blocks of 128 FP32 target slots each (tX, tY[, tZ]; the packer zero-pads the
//     slots past a cell's points, 2d/matmultgpu.cxx:48-57), and
//   * the blocks' truncation sets packed one after the other (sX, sY[, sZ], sG), block b's
//     at [offset[b], offset[b+1]) (2d/matmultgpu.cxx:58-67),
//   tW[128 b + i] = sum_j sG_j exp(-|t_i - s_j|^2 / (2 sigma^2)) / (2 pi sigma^2)
// for every slot of every block (padding slots included, as the reference computes them;
// the 3D form keeps the reference's 2D normalisation, 3d/gpumatmult.cu:37, 70).
//
// One CTA per block, one thread per slot; the block's sources stream through shared memory
// in chunks of kChunk, double-buffered with TMA bulk copies (cp.async.bulk + mbarrier) and
// read as float4 broadcasts. A chunk is copied from its 16-byte-aligned start; the
// entries outside [offset[b], offset[b+1]) get a zero weight in shared memory, so the pair
// loop has no bounds test. The differences are taken in FP32 on the caller's coordinates
// as the reference does; exp is ex2.approx on -d2 log2(e) / (2 sigma^2).
//
// Device buffers are grow-only and held for the life of the process, one set per device,
// as the reference's file statics are (2d/gpumatmult.cu:7-18); calls are serialised.
#include <cmath>
#include <cstring>
#include <mutex>
#include <new>

#include "device.h"

namespace prbf {

namespace {

constexpr int kSlots = 128;   // target slots per block (the reference's threadsPerBlock)
constexpr int kChunk = 1024;  // sources per staged chunk
constexpr int kRow = kChunk + 8;  // floats per staged array (aligned start, rounded end)

__device__ __forceinline__ float ex2_fast(float x) {
  float y;
  asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}

template <int DIM>
__global__ void __launch_bounds__(kSlots) k_seam(const int* __restrict__ offset, const float* __restrict__ tx,
                                                 const float* __restrict__ ty, const float* __restrict__ tz,
                                                 float* __restrict__ tw, float c2, double norm,
                                                 const float* __restrict__ sx, const float* __restrict__ sy,
                                                 const float* __restrict__ sz, const float* __restrict__ sg,
                                                 unsigned* err) {
  constexpr int NA = DIM + 1;  // staged arrays: coordinates + weight
  __shared__ __align__(16) float buf[2][NA][kRow];
  __shared__ __align__(8) uint64_t bar[2];
  __shared__ int s_abort;
  const int b = blockIdx.x, t = threadIdx.x;
  const long long i = (long long)b * kSlots + t;
  const float x = tx[i], y = ty[i], z = DIM == 3 ? tz[i] : 0.f;
  const int j0 = offset[b], j1 = offset[b + 1];
  const int nchunk = j1 > j0 ? (j1 - j0 + kChunk - 1) / kChunk : 0;
  if (t == 0) {
    mbar_init(&bar[0], 1);
    mbar_init(&bar[1], 1);
    s_abort = 0;
  }
  __syncthreads();
  // chunk k: sources [a, e), copied from a & ~3 to (e + 3) & ~3 (<= kChunk + 6 floats)
  auto issue = [&](int k) {
    const int a = j0 + k * kChunk, e = min(j1, a + kChunk);
    const int a_al = a & ~3, e_al = (e + 3) & ~3;
    const unsigned bytes = (unsigned)(e_al - a_al) * 4u;
    uint64_t* bk = &bar[k & 1];
    fence_proxy_async_smem();
    mbar_expect_tx(bk, bytes * NA);
    bulk_g2s(buf[k & 1][0], sx + a_al, bytes, bk);
    bulk_g2s(buf[k & 1][1], sy + a_al, bytes, bk);
    if (DIM == 3) bulk_g2s(buf[k & 1][2], sz + a_al, bytes, bk);
    bulk_g2s(buf[k & 1][DIM], sg + a_al, bytes, bk);
  };
  if (t == 0 && nchunk > 0) issue(0);
  float acc = 0.f;
  for (int k = 0; k < nchunk; k++) {
    __syncthreads();  // every thread is done with chunk k - 1 (its buffer is refilled next)
    if (t == 0 && k + 1 < nchunk) issue(k + 1);
    if (!mbar_wait(&bar[k & 1], (unsigned)(k >> 1) & 1u)) {
      atomicOr(err, DEV_ERR_TIMEOUT);
      s_abort = 1;
    }
    __syncthreads();
    if (s_abort) {
      // let the copies in flight (chunks k and k + 1) land before the CTA exits
      if (t == 0) {
        mbar_wait(&bar[k & 1], (unsigned)(k >> 1) & 1u, 1u << 20);
        if (k + 1 < nchunk) mbar_wait(&bar[(k + 1) & 1], (unsigned)((k + 1) >> 1) & 1u, 1u << 20);
      }
      return;
    }
    const int a = j0 + k * kChunk, e = min(j1, a + kChunk);
    const int a_al = a & ~3, e_al = (e + 3) & ~3;
    float* g = buf[k & 1][DIM];
    // the aligned copy's entries outside [a, e) carry no weight
    if (t < a - a_al) g[t] = 0.f;
    if (t < e_al - e) g[e - a_al + t] = 0.f;
    __syncthreads();
    const float4* X = (const float4*)buf[k & 1][0];
    const float4* Y = (const float4*)buf[k & 1][1];
    const float4* Z = (const float4*)buf[k & 1][DIM == 3 ? 2 : 0];
    const float4* Gw = (const float4*)g;
    const int n4 = (e_al - a_al) >> 2;
#pragma unroll 4
    for (int q = 0; q < n4; q++) {
      const float4 sx4 = X[q], sy4 = Y[q], g4 = Gw[q];
      float4 sz4 = make_float4(0.f, 0.f, 0.f, 0.f);
      if (DIM == 3) sz4 = Z[q];
      const float xs[4] = {sx4.x, sx4.y, sx4.z, sx4.w}, ys[4] = {sy4.x, sy4.y, sy4.z, sy4.w};
      const float zs[4] = {sz4.x, sz4.y, sz4.z, sz4.w}, gs[4] = {g4.x, g4.y, g4.z, g4.w};
#pragma unroll
      for (int u = 0; u < 4; u++) {
        const float dx = x - xs[u], dy = y - ys[u];
        float d2 = fmaf(dy, dy, dx * dx);
        if (DIM == 3) {
          const float dz = z - zs[u];
          d2 = fmaf(dz, dz, d2);
        }
        acc = fmaf(gs[u], ex2_fast(-d2 * c2), acc);
      }
    }
  }
  tw[i] = (float)((double)acc * norm);
}

struct SeamBufs {
  std::mutex m;
  cudaStream_t s = nullptr;
  DevBuf<int> off;
  DevBuf<float> t[4], src[4];
  DevBuf<unsigned> err;
};

// One set per device, created on first use and kept (never destroyed: freeing device
// memory from a static destructor would run after the runtime has shut down).
SeamBufs& seam_bufs(int dev) {
  static std::mutex gm;
  static SeamBufs* sets[64] = {nullptr};
  std::lock_guard<std::mutex> lk(gm);
  if (dev < 0 || dev >= 64) throw Error(PRBF_ERR_ARG, "device ordinal out of range");
  if (!sets[dev]) sets[dev] = new SeamBufs();
  return *sets[dev];
}

template <int DIM>
int seam(const float* tX, const float* tY, const float* tZ, float* tW, const float* sX, const float* sY,
         const float* sZ, const float* sG, const int* offset, int iblok, float sigma, int numCluster, int numTrunc) {
  try {
    if (!tX || !tY || (DIM == 3 && !tZ) || !tW || !sX || !sY || (DIM == 3 && !sZ) || !sG || !offset)
      return PRBF_ERR_ARG;
    if (iblok < 0 || numCluster < 0 || numTrunc < 0 || iblok > numCluster) return PRBF_ERR_ARG;
    if (!(sigma > 0.f) || !std::isfinite(sigma)) return PRBF_ERR_ARG;
    if (iblok == 0) return PRBF_OK;
    if (offset[0] < 0) return PRBF_ERR_ARG;
    for (int b = 0; b < iblok; b++)
      if (offset[b + 1] < offset[b]) return PRBF_ERR_ARG;
    const long long nsrc = offset[iblok];
    // the caller's capacity (2d/gpumatmult.cu:71); the offsets index a buffer of that size
    if (nsrc > (long long)numCluster * numTrunc) return PRBF_ERR_CAPACITY;
    if (nsrc > 0x7ffffff0LL) return PRBF_ERR_CAPACITY;
    int dev = 0;
    PRBF_CUDA(cudaGetDevice(&dev));
    SeamBufs& S = seam_bufs(dev);
    std::lock_guard<std::mutex> lk(S.m);
    if (!S.s) PRBF_CUDA(cudaStreamCreateWithFlags(&S.s, cudaStreamNonBlocking));
    const long long nt = (long long)iblok * kSlots;
    S.off.reserve((size_t)iblok + 1);
    for (int a = 0; a < (DIM == 3 ? 4 : 3); a++) S.t[a].reserve((size_t)nt);
    // sources padded: a chunk's copy ends up to 3 floats past the last source
    const size_t ns_alloc = (size_t)nsrc + 8;
    for (int a = 0; a < (DIM == 3 ? 4 : 3); a++) S.src[a].reserve(ns_alloc);
    S.err.reserve(1);
    PRBF_CUDA(cudaMemsetAsync(S.err.get(), 0, sizeof(unsigned), S.s));
    PRBF_CUDA(cudaMemcpyAsync(S.off.get(), offset, sizeof(int) * ((size_t)iblok + 1), cudaMemcpyHostToDevice, S.s));
    const float* th[3] = {tX, tY, tZ};
    for (int a = 0; a < DIM; a++)
      PRBF_CUDA(cudaMemcpyAsync(S.t[a].get(), th[a], sizeof(float) * nt, cudaMemcpyHostToDevice, S.s));
    const float* sh[4] = {sX, sY, DIM == 3 ? sZ : sG, sG};
    for (int a = 0; a <= DIM; a++) {
      float* d = S.src[a].get();
      if (nsrc > 0) PRBF_CUDA(cudaMemcpyAsync(d, sh[a], sizeof(float) * nsrc, cudaMemcpyHostToDevice, S.s));
      PRBF_CUDA(cudaMemsetAsync(d + nsrc, 0, sizeof(float) * 8, S.s));
    }
    // coef = 0.5 / sigma^2 (2d/gpumatmult.cu:33); exp(-d2 coef) = 2^(-d2 coef log2 e)
    const double coef = 0.5 / ((double)sigma * (double)sigma);
    const float c2 = (float)(coef * 1.4426950408889634);
    const double norm = coef / 3.141592653589793;
    float* tw_dev = S.t[DIM].get();
    k_seam<DIM><<<iblok, kSlots, 0, S.s>>>(S.off.get(), S.t[0].get(), S.t[1].get(), DIM == 3 ? S.t[2].get() : nullptr,
                                           tw_dev, c2, norm, S.src[0].get(), S.src[1].get(),
                                           DIM == 3 ? S.src[2].get() : nullptr, S.src[DIM].get(), S.err.get());
    PRBF_CHECK_LAUNCH();
    unsigned herr = 0;
    PRBF_CUDA(cudaMemcpyAsync(tW, tw_dev, sizeof(float) * nt, cudaMemcpyDeviceToHost, S.s));
    PRBF_CUDA(cudaMemcpyAsync(&herr, S.err.get(), sizeof(unsigned), cudaMemcpyDeviceToHost, S.s));
    PRBF_CUDA(cudaStreamSynchronize(S.s));
    if (herr) return PRBF_ERR_TIMEOUT;
    return PRBF_OK;
  } catch (const Error& e) {
    return e.status;
  } catch (const std::bad_alloc&) {
    return PRBF_ERR_CAPACITY;
  } catch (const std::exception&) {
    return PRBF_ERR_CUDA;
  }
}

}  // namespace
}  // namespace prbf

extern "C" {

int prbf_gpumatmult_2d(const float* tX, const float* tY, float* tW, const float* sX, const float* sY,
                       const float* sG, const int* offset, int iblok, float sigma, int numCluster, int numTrunc) {
  return prbf::seam<2>(tX, tY, nullptr, tW, sX, sY, nullptr, sG, offset, iblok, sigma, numCluster, numTrunc);
}

int prbf_gpumatmult_3d(const float* tX, const float* tY, const float* tZ, float* tW, const float* sX,
                       const float* sY, const float* sZ, const float* sG, const int* offset, int iblok, float sigma,
                       int numCluster, int numTrunc) {
  return prbf::seam<3>(tX, tY, tZ, tW, sX, sY, sZ, sG, offset, iblok, sigma, numCluster, numTrunc);
}

}  // extern "C"
