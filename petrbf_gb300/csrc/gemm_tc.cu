// gemm_tc.cu -- the learned-guess network's GEMMs on the tensor cores (sm_103a):
//
//   C[M][N] = A[M][K] B[N][K]^T  (+ bias[n], ReLU)   A, B BF16 row-major (K contiguous),
//                                                    FP32 accumulation, FP32 and/or BF16 out
//
// One CTA computes a 128-row tile with the whole N (<= 256) as one tcgen05.mma.kind::f16
// accumulator in TMEM. The K dimension runs in chunks of 64 BF16 (128 bytes): warp 0
// stages each chunk of A (128 x 64) and B (BN x 64) with two tiled TMA copies
// (cp.async.bulk.tensor, 128-byte swizzle, zero fill past the matrix edges) into a ring of
// shared-memory stages that complete on mbarriers; warp 1 issues the four K = 16 MMAs of a
// chunk and commits them to the stage's "empty" mbarrier, so the next copy into that stage
// waits for the tensor cores to have read it; the last commit releases the epilogue, where
// the four warps read their 32 TMEM lanes (rows) with tcgen05.ld and apply bias and ReLU.
// Every wait is bounded: a wait that gives up raises DEV_ERR_TIMEOUT and the CTA stops.
#include <cuda.h>  // CUtensorMap and its enums (the encoder comes from the runtime's entry point)
#include <cuda_bf16.h>

#include <mutex>

#include "device.h"
#include "mlp.h"

namespace prbf {
namespace {

constexpr int GM = 128;     // rows per CTA (TMEM lanes)
constexpr int GKC = 64;     // K per stage: 64 BF16 = 128 bytes, one swizzle row
constexpr int GSTAGES = 2;  // ring depth (two CTAs share an SM at N = 256)
constexpr int GTHREADS = 128;

typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                  const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiledFn encode_tiled() {
  static EncodeTiledFn fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = (EncodeTiledFn)p;
    else
      cudaGetLastError();
  });
  if (!fn) throw Error(PRBF_ERR_CUDA, "cuTensorMapEncodeTiled is not available from the driver");
  return fn;
}

// Tiled map of a row-major BF16 matrix [rows][cols] with leading dimension ld (elements):
// boxes of 64 columns x box_rows rows, 128-byte swizzle, zeros outside the matrix.
CUtensorMap tile_map(const void* base, long long rows, long long cols, long long ld, int box_rows) {
  if (((uintptr_t)base & 15) || (ld * 2) % 16) throw Error(PRBF_ERR_ARG, "GEMM operand not 16-byte aligned");
  CUtensorMap m;
  const cuuint64_t dims[2] = {(cuuint64_t)cols, (cuuint64_t)rows};
  const cuuint64_t strides[1] = {(cuuint64_t)ld * 2};
  const cuuint32_t box[2] = {(cuuint32_t)GKC, (cuuint32_t)box_rows};
  const cuuint32_t es[2] = {1, 1};
  const CUresult r = encode_tiled()(&m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void*>(base), dims, strides,
                                    box, es, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                                    CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) throw Error(PRBF_ERR_ARG, "GEMM tensor map rejected by the driver");
  return m;
}

__device__ __forceinline__ uint32_t s_addr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// K-major operand in the 128-byte-swizzled layout the TMA copy writes: 8-row x 128-byte
// atoms (SBO 1024 bytes), descriptor version 1, base 1024-aligned; a K = 16 step inside the
// 128-byte row advances the start address by 32 bytes.
__device__ __forceinline__ uint64_t sw128_desc(uint32_t saddr) {
  uint64_t d = (uint64_t)((saddr & 0x3FFFF) >> 4);
  d |= (uint64_t)1 << 16;               // leading byte offset (unused for swizzled K-major)
  d |= (uint64_t)(1024 >> 4) << 32;     // stride byte offset: 8 rows of 128 bytes
  d |= (uint64_t)1 << 46;               // tcgen05 descriptor version
  d |= (uint64_t)2 << 61;               // 128-byte swizzle
  return d;
}

__device__ __forceinline__ void tma_2d(void* dst, const CUtensorMap* map, int x, int y, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
          s_addr(dst)),
      "l"((uint64_t)map), "r"(x), "r"(y), "r"(s_addr(bar))
      : "memory");
}

__device__ __forceinline__ void umma_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(s_addr(bar))
               : "memory");
}

template <int BN>
__global__ void __launch_bounds__(GTHREADS, 1)
    k_gemm_tc(const __grid_constant__ CUtensorMap ta, const __grid_constant__ CUtensorMap tb, int M, int N, int K,
              float* __restrict__ C, int ldc, __nv_bfloat16* __restrict__ Cb, int ldcb,
              const float* __restrict__ bias, int relu, unsigned* __restrict__ err) {
  static_assert(BN % 16 == 0 && BN >= 16 && BN <= 256, "tcgen05 M = 128 takes N = 16 .. 256 in steps of 16");
  constexpr int TCOLS = BN < 32 ? 32 : BN;  // TMEM allocation: a power of two >= 32
  constexpr uint32_t A_BYTES = GM * GKC * 2, B_BYTES = BN * GKC * 2, STAGE = A_BYTES + B_BYTES;
  // D F32, A BF16, B BF16, both K-major, N >> 3 at bit 17, M >> 4 at bit 24
  constexpr uint32_t IDESC = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(BN >> 3) << 17) |
                             ((uint32_t)(GM >> 4) << 24);
  extern __shared__ unsigned char smem_raw[];
  unsigned char* sm = (unsigned char*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  __shared__ __align__(8) uint64_t full[GSTAGES], empty[GSTAGES], done;
  __shared__ uint32_t tmem_base;
  __shared__ int s_abort;
  const int tid = threadIdx.x, w = tid >> 5, lane = tid & 31;
  const int m0 = blockIdx.x * GM;
  const int nk = (K + GKC - 1) / GKC;
  if (tid == 0) {
    for (int s = 0; s < GSTAGES; s++) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    mbar_init(&done, 1);
    s_abort = 0;
    asm volatile("prefetch.tensormap [%0];" ::"l"((uint64_t)&ta) : "memory");
    asm volatile("prefetch.tensormap [%0];" ::"l"((uint64_t)&tb) : "memory");
  }
  if (w == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(s_addr(&tmem_base)),
                 "r"(TCOLS));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = tmem_base;

  if (w == 0 && lane == 0) {
    // producer: chunk kc into stage kc % GSTAGES once the MMAs of chunk kc - GSTAGES are done
    for (int kc = 0; kc < nk; kc++) {
      const int s = kc % GSTAGES;
      if (kc >= GSTAGES && !mbar_wait(&empty[s], ((kc / GSTAGES) + 1) & 1)) {
        atomicOr(err, DEV_ERR_TIMEOUT);
        s_abort = 1;
        break;
      }
      if (s_abort) break;
      unsigned char* a = sm + s * STAGE;
      mbar_expect_tx(&full[s], STAGE);
      tma_2d(a, &ta, kc * GKC, m0, &full[s]);
      tma_2d(a + A_BYTES, &tb, kc * GKC, 0, &full[s]);
    }
  } else if (w == 1 && lane == 0) {
    // MMA issuer
    int kc = 0;
    for (; kc < nk; kc++) {
      const int s = kc % GSTAGES;
      if (!mbar_wait(&full[s], (kc / GSTAGES) & 1)) {
        atomicOr(err, DEV_ERR_TIMEOUT);
        s_abort = 1;
        break;
      }
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      const uint32_t a = s_addr(sm + s * STAGE), b = a + A_BYTES;
#pragma unroll
      for (int ks = 0; ks < GKC / 16; ks++) {
        const uint64_t da = sw128_desc(a + ks * 32), db = sw128_desc(b + ks * 32);
        const uint32_t acc = (kc > 0 || ks > 0) ? 1u : 0u;
        asm volatile(
            "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}" ::"r"(
                tmem),
            "l"(da), "l"(db), "r"(IDESC), "r"(acc));
      }
      umma_commit(&empty[s]);
    }
    umma_commit(&done);  // tracks every MMA issued above (none after an abort)
  }
  // epilogue: warp w holds rows m0 + 32 w + lane in its TMEM lanes
  __syncwarp();
  const bool ok = mbar_wait(&done, 0);
  if (!ok && lane == 0) atomicOr(err, DEV_ERR_TIMEOUT);
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  // Each 16-column slice of the warp's 32 rows goes through shared memory (the ring is idle
  // once the last MMA has completed), so that a store instruction writes two rows of 16
  // consecutive columns instead of one column of 32 rows.
  float* stg = (float*)(sm + w * (32 * 17 * 4));
  const int half = lane >> 4, cl = lane & 15;
  // tcgen05.ld is warp-collective: the whole warp takes the same branch
  if (__all_sync(0xffffffffu, ok && !s_abort)) {
#pragma unroll 1
    for (int c0 = 0; c0 < BN; c0 += 16) {
      uint32_t r[16];
      const uint32_t addr = tmem + ((uint32_t)(32 * w) << 16) + (uint32_t)c0;
      asm volatile(
          "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
          : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
            "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
          : "r"(addr));
      asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
      for (int j = 0; j < 16; j++) stg[lane * 17 + j] = __uint_as_float(r[j]);
      __syncwarp();
      const int n = c0 + cl;
      const float bn = (bias && n < N) ? bias[n] : 0.f;
#pragma unroll 4
      for (int rr = 0; rr < 32; rr += 2) {
        const int rloc = rr + half;
        const long long row = m0 + 32 * w + rloc;
        if (row < M && n < N) {
          float v = stg[rloc * 17 + cl] + bn;
          if (relu) v = fmaxf(v, 0.f);
          if (C) C[row * ldc + n] = v;
          if (Cb) Cb[row * ldcb + n] = __float2bfloat16_rn(v);
        }
      }
      __syncwarp();
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (w == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TCOLS));
}

template <int BN>
void launch_gemm(const CUtensorMap& ta, const CUtensorMap& tb, int M, int N, int K, float* C, int ldc,
                 __nv_bfloat16* Cb, int ldcb, const float* bias, bool relu, unsigned* err, cudaStream_t s) {
  const size_t smem = (size_t)GSTAGES * (GM + BN) * GKC * 2 + 1024;
  static bool attr[64] = {false};
  int dev = 0;
  PRBF_CUDA(cudaGetDevice(&dev));
  if (dev >= 0 && dev < 64 && !attr[dev]) {
    PRBF_CUDA(cudaFuncSetAttribute(k_gemm_tc<BN>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    attr[dev] = true;
  }
  k_gemm_tc<BN><<<(M + GM - 1) / GM, GTHREADS, smem, s>>>(ta, tb, M, N, K, C, ldc, Cb, ldcb, bias, relu ? 1 : 0,
                                                          err);
  PRBF_CHECK_LAUNCH();
}

}  // namespace

void gemm_bf16_tc(int M, int N, int K, const __nv_bfloat16* A, int lda, const __nv_bfloat16* B, int ldb, float* C,
                  int ldc, __nv_bfloat16* Cb, int ldcb, const float* bias, bool relu, unsigned* err, cudaStream_t s) {
  if (M <= 0 || N <= 0 || K <= 0) return;
  if (N > 256) throw Error(PRBF_ERR_ARG, "GEMM N above 256");
  if (N <= 16) {
    const CUtensorMap ta = tile_map(A, M, K, lda, GM), tb = tile_map(B, N, K, ldb, 16);
    launch_gemm<16>(ta, tb, M, N, K, C, ldc, Cb, ldcb, bias, relu, err, s);
  } else {
    const CUtensorMap ta = tile_map(A, M, K, lda, GM), tb = tile_map(B, N, K, ldb, 256);
    launch_gemm<256>(ta, tb, M, N, K, C, ldc, Cb, ldcb, bias, relu, err, s);
  }
}

}  // namespace prbf
