// cellsort.cu -- the cell-list build (get_cluster) on the GPU: bounding box, cell index
// per point, stable LSD radix sort of (cell, original index), cell start offsets, and
// the permutation gathers.
//
// Reference: 2d/get_cluster.h:176-190 (grid), :233-264 (counts and offsets),
// :279-286 (sorted-slot writes in ascending original index, i.e. a stable sort);
// 3d/get_cluster.h:96-101 (3D cell index iz*nx*ny + ix*ny + iy).
#include <cfloat>

#include "device.h"

namespace prbf {
namespace {

constexpr int kBboxThreads = 256;
constexpr int kBboxBlocks = 304;  // 2 x 152 SMs

__global__ void k_bbox_partial(int n, const double* __restrict__ x, const double* __restrict__ y,
                               const double* __restrict__ z, double* __restrict__ part) {
  double lo[3] = {DBL_MAX, DBL_MAX, DBL_MAX}, hi[3] = {-DBL_MAX, -DBL_MAX, -DBL_MAX};
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    double v[3] = {x[i], y[i], z ? z[i] : 0.0};
#pragma unroll
    for (int d = 0; d < 3; d++) {
      lo[d] = fmin(lo[d], v[d]);
      hi[d] = fmax(hi[d], v[d]);
    }
  }
  __shared__ double s[6][kBboxThreads / 32];
  int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
  for (int d = 0; d < 3; d++) {
    for (int o = 16; o > 0; o >>= 1) {
      lo[d] = fmin(lo[d], __shfl_xor_sync(0xffffffffu, lo[d], o));
      hi[d] = fmax(hi[d], __shfl_xor_sync(0xffffffffu, hi[d], o));
    }
    if (lane == 0) {
      s[2 * d][w] = lo[d];
      s[2 * d + 1][w] = hi[d];
    }
  }
  __syncthreads();
  if (threadIdx.x < 6) {
    int d = threadIdx.x;
    double r = s[d][0];
    for (int k = 1; k < kBboxThreads / 32; k++) r = (d & 1) ? fmax(r, s[d][k]) : fmin(r, s[d][k]);
    part[blockIdx.x * 6 + d] = r;
  }
}

__global__ void k_bbox_final(int nparts, const double* __restrict__ part, double* __restrict__ out) {
  int d = threadIdx.x;
  if (d >= 6) return;
  double r = part[d];
  for (int k = 1; k < nparts; k++) r = (d & 1) ? fmax(r, part[k * 6 + d]) : fmin(r, part[k * 6 + d]);
  out[d] = r;
}

// ---- exclusive scan (reduce-then-scan, recursive over block sums) -------------------
constexpr int kScanThreads = 256;
constexpr int kScanItems = 8;
constexpr int kScanTile = kScanThreads * kScanItems;

template <class T>
__device__ T block_exclusive(T v, T* s_warp, T* total) {
  int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  T inc = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    T t = __shfl_up_sync(0xffffffffu, inc, o);
    if (lane >= o) inc += t;
  }
  if (lane == 31) s_warp[w] = inc;
  __syncthreads();
  if (w == 0) {
    T sv = lane < kScanThreads / 32 ? s_warp[lane] : T(0);
    T si = sv;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      T t = __shfl_up_sync(0xffffffffu, si, o);
      if (lane >= o) si += t;
    }
    if (lane < kScanThreads / 32) s_warp[lane] = si - sv;
    if (lane == kScanThreads / 32 - 1) *total = si;
  }
  __syncthreads();
  return s_warp[w] + inc - v;
}

template <class T>
__global__ void k_scan_tiles(const T* __restrict__ in, T* __restrict__ out, T* __restrict__ sums,
                             long long n) {
  __shared__ T s_warp[kScanThreads / 32];
  __shared__ T total;
  long long base = (long long)blockIdx.x * kScanTile + (long long)threadIdx.x * kScanItems;
  T v[kScanItems];
  T acc = 0;
#pragma unroll
  for (int k = 0; k < kScanItems; k++) {
    long long i = base + k;
    v[k] = i < n ? in[i] : T(0);
    acc += v[k];
  }
  T pre = block_exclusive<T>(acc, s_warp, &total);
#pragma unroll
  for (int k = 0; k < kScanItems; k++) {
    long long i = base + k;
    if (i < n) out[i] = pre;
    pre += v[k];
  }
  if (threadIdx.x == 0 && sums) sums[blockIdx.x] = total;
}

template <class T>
__global__ void k_scan_add(T* __restrict__ out, const T* __restrict__ sums, long long n) {
  long long base = (long long)blockIdx.x * kScanTile;
  T add = sums[blockIdx.x];
  for (int k = threadIdx.x; k < kScanTile; k += kScanThreads) {
    long long i = base + k;
    if (i < n) out[i] += add;
  }
}

template <class T>
void scan_impl(const T* in, T* out, long long n, Workspace& ws, int slot, cudaStream_t s) {
  if (n <= 0) return;
  long long nb = (n + kScanTile - 1) / kScanTile;
  if (nb == 1) {
    k_scan_tiles<T><<<1, kScanThreads, 0, s>>>(in, out, nullptr, n);
    PRBF_CHECK_LAUNCH();
    return;
  }
  T* sums = (T*)ws.get(slot, (size_t)nb * sizeof(T));
  k_scan_tiles<T><<<(unsigned)nb, kScanThreads, 0, s>>>(in, out, sums, n);
  PRBF_CHECK_LAUNCH();
  scan_impl<T>(sums, sums, nb, ws, slot + 1, s);
  k_scan_add<T><<<(unsigned)nb, kScanThreads, 0, s>>>(out, sums, n);
  PRBF_CHECK_LAUNCH();
}

// ---- cell index and counts ---------------------------------------------------------
__global__ void k_cell_ids(Grid g, int n, const double* __restrict__ x, const double* __restrict__ y,
                           const double* __restrict__ z, unsigned* __restrict__ key,
                           int* __restrict__ val, int* __restrict__ count, unsigned* err) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  // (int)floor((x - xmin)/box_length), 2d/get_cluster.h:234-236
  double fx = floor((x[i] - g.xmin) / g.box);
  double fy = floor((y[i] - g.ymin) / g.box);
  double fz = g.dim == 3 ? floor((z[i] - g.zmin) / g.box) : 0.0;
  bool ok = fx >= 0.0 && fx < (double)g.nx && fy >= 0.0 && fy < (double)g.ny && fz >= 0.0 &&
            fz < (double)g.nz;
  int c = 0;
  if (ok) {
    c = cell_of(g, (int)fx, (int)fy, (int)fz);
  } else {
    atomicOr(err, DEV_ERR_RANGE);
  }
  key[i] = (unsigned)c;
  val[i] = i;
  atomicAdd(&count[c], 1);
}

// ---- stable LSD radix sort, 8-bit digits ----------------------------------------------
constexpr int kRadixThreads = 256;
constexpr int kRadixItems = 16;
constexpr int kRadixTile = kRadixThreads * kRadixItems;  // 4096 keys per tile
constexpr int kRadixWarps = kRadixThreads / 32;

// hist[digit * ntiles + tile] = number of keys of this tile with this digit.
__global__ void k_radix_hist(const unsigned* __restrict__ key, int n, int shift,
                             int* __restrict__ hist, int ntiles) {
  __shared__ int s_h[256];
  s_h[threadIdx.x] = 0;
  __syncthreads();
  int base = blockIdx.x * kRadixTile;
  for (int k = threadIdx.x; k < kRadixTile; k += kRadixThreads) {
    int i = base + k;
    if (i < n) atomicAdd(&s_h[(key[i] >> shift) & 255u], 1);
  }
  __syncthreads();
  hist[threadIdx.x * ntiles + blockIdx.x] = s_h[threadIdx.x];
}

// Stable scatter: keys of a tile are ranked in index order, 256 consecutive keys per
// round; within a warp, peers with equal digit are found with __match_any_sync.
__global__ void __launch_bounds__(kRadixThreads) k_radix_scatter(
    const unsigned* __restrict__ key_in, const int* __restrict__ val_in, unsigned* __restrict__ key_out,
    int* __restrict__ val_out, int n, int shift, const int* __restrict__ offs, int ntiles) {
  __shared__ int s_base[256];
  __shared__ int s_run[256];
  __shared__ int s_wcnt[kRadixWarps][256];
  int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
  s_base[tid] = offs[tid * ntiles + blockIdx.x];
  s_run[tid] = 0;
  const unsigned lt_mask = (1u << lane) - 1u;
  int tile0 = blockIdx.x * kRadixTile;
  for (int r = 0; r < kRadixItems; r++) {
#pragma unroll
    for (int k = 0; k < kRadixWarps; k++) s_wcnt[k][tid] = 0;
    __syncthreads();
    int i = tile0 + r * kRadixThreads + tid;
    bool valid = i < n;
    unsigned kk = valid ? key_in[i] : 0u;
    int vv = valid ? val_in[i] : 0;
    unsigned d = valid ? (kk >> shift) & 255u : 256u;  // 256 = no digit
    unsigned peers = __match_any_sync(0xffffffffu, d);
    int rank = __popc(peers & lt_mask);
    if (valid && rank == 0) s_wcnt[w][d] = __popc(peers);
    __syncthreads();
    {  // exclusive prefix over warps for digit tid, carried across rounds in s_run
      int run = s_run[tid];
#pragma unroll
      for (int k = 0; k < kRadixWarps; k++) {
        int c = s_wcnt[k][tid];
        s_wcnt[k][tid] = run;
        run += c;
      }
      s_run[tid] = run;
    }
    __syncthreads();
    if (valid) {
      int pos = s_base[d] + s_wcnt[w][d] + rank;
      key_out[pos] = kk;
      val_out[pos] = vv;
    }
    __syncthreads();
  }
}

__global__ void k_gather(int n, const int* __restrict__ perm, const double* __restrict__ in,
                         double* __restrict__ out) {
  int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k < n) out[k] = in[perm[k]];
}

__global__ void k_scatter(int n, const int* __restrict__ perm, const double* __restrict__ in,
                          double* __restrict__ out) {
  int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k < n) out[perm[k]] = in[k];
}

}  // namespace

void bbox_dev(int n, const double* x, const double* y, const double* z, double* out6, Workspace& ws,
              cudaStream_t s) {
  int blocks = std::min(kBboxBlocks, std::max(1, ceil_div(n, kBboxThreads)));
  double* part = (double*)ws.get(0, sizeof(double) * 6 * blocks);
  k_bbox_partial<<<blocks, kBboxThreads, 0, s>>>(n, x, y, z, part);
  PRBF_CHECK_LAUNCH();
  k_bbox_final<<<1, 32, 0, s>>>(blocks, part, out6);
  PRBF_CHECK_LAUNCH();
}

void scan_exclusive_dev(const int* in, int* out, long long n, Workspace& ws, int slot, cudaStream_t s) {
  scan_impl<int>(in, out, n, ws, slot, s);
}
void scan_exclusive_dev(const long long* in, long long* out, long long n, Workspace& ws, int slot,
                        cudaStream_t s) {
  scan_impl<long long>(in, out, n, ws, slot, s);
}

void cell_sort_dev(const Grid& g, int n, const double* x, const double* y, const double* z, int* perm,
                   int* cell_start, unsigned* err, Workspace& ws, cudaStream_t s) {
  // workspace slots: 1 keys A, 2 keys B, 3 vals B, 4 histograms, 5.. scans
  unsigned* keyA = (unsigned*)ws.get(1, sizeof(unsigned) * (size_t)n);
  unsigned* keyB = (unsigned*)ws.get(2, sizeof(unsigned) * (size_t)n);
  int* valB = (int*)ws.get(3, sizeof(int) * (size_t)n);
  PRBF_CUDA(cudaMemsetAsync(cell_start, 0, sizeof(int) * ((size_t)g.ncell + 1), s));
  // counts land in cell_start[0..ncell-1], then an exclusive scan over ncell+1 entries
  k_cell_ids<<<ceil_div(n, 256), 256, 0, s>>>(g, n, x, y, z, keyA, perm, cell_start, err);
  PRBF_CHECK_LAUNCH();
  scan_exclusive_dev(cell_start, cell_start, (long long)g.ncell + 1, ws, 5, s);

  int bits = 0;
  while (bits < 31 && (1u << bits) < (unsigned)g.ncell) bits++;
  int passes = (bits + 7) / 8;
  int ntiles = ceil_div(n, kRadixTile);
  int* hist = (int*)ws.get(4, sizeof(int) * 256 * (size_t)ntiles);
  unsigned* kin = keyA;
  int* vin = perm;
  unsigned* kout = keyB;
  int* vout = valB;
  for (int p = 0; p < passes; p++) {
    int shift = 8 * p;
    k_radix_hist<<<ntiles, kRadixThreads, 0, s>>>(kin, n, shift, hist, ntiles);
    PRBF_CHECK_LAUNCH();
    scan_exclusive_dev(hist, hist, 256LL * ntiles, ws, 8, s);
    k_radix_scatter<<<ntiles, kRadixThreads, 0, s>>>(kin, vin, kout, vout, n, shift, hist, ntiles);
    PRBF_CHECK_LAUNCH();
    std::swap(kin, kout);
    std::swap(vin, vout);
  }
  if (vin != perm) PRBF_CUDA(cudaMemcpyAsync(perm, vin, sizeof(int) * (size_t)n, cudaMemcpyDeviceToDevice, s));
}

void gather_dev(int n, const int* perm, const double* in, double* out, cudaStream_t s) {
  if (n <= 0) return;
  k_gather<<<ceil_div(n, 256), 256, 0, s>>>(n, perm, in, out);
  PRBF_CHECK_LAUNCH();
}

void scatter_dev(int n, const int* perm, const double* in, double* out, cudaStream_t s) {
  if (n <= 0) return;
  k_scatter<<<ceil_div(n, 256), 256, 0, s>>>(n, perm, in, out);
  PRBF_CHECK_LAUNCH();
}

}  // namespace prbf

// ---- cell sort without allocation -------------------------------------------------------
// prbf_cell_sort_static (declared in include/petrbf_gb300.h) sorts into caller-provided
// device buffers and takes every temporary from one fixed device array of this file, so
// it never calls cudaMalloc or cudaFree. The array lives on every GPU that loads the
// library until the process exits; all calls share it.
#include <mutex>
#include <new>

#include "context.h"

namespace prbf {
namespace {

constexpr int kStaticMaxPoints = PRBF_STATIC_SORT_MAX_POINTS;
constexpr long long kStaticMaxScan = 2048LL * 4096;  // entries a two-level scan can take
constexpr int kStaticTiles = (kStaticMaxPoints + kRadixTile - 1) / kRadixTile;
// byte offsets inside the scratch array (each 256-aligned)
constexpr size_t kOffKeyA = 0;
constexpr size_t kOffKeyB = kOffKeyA + sizeof(unsigned) * (size_t)kStaticMaxPoints;
constexpr size_t kOffValB = kOffKeyB + sizeof(unsigned) * (size_t)kStaticMaxPoints;
constexpr size_t kOffHist = kOffValB + sizeof(int) * (size_t)kStaticMaxPoints;
constexpr size_t kOffSums1 = kOffHist + sizeof(int) * 256 * (size_t)kStaticTiles;
constexpr size_t kOffSums2 = kOffSums1 + sizeof(int) * 4096;
constexpr size_t kOffBboxPart = kOffSums2 + 256;
constexpr size_t kOffBbox = kOffBboxPart + sizeof(double) * 6 * kBboxBlocks;
constexpr size_t kOffErr = kOffBbox + 256;
constexpr size_t kStaticScratchBytes = kOffErr + 256;

static __device__ __align__(256) unsigned char g_static_sort_scratch[kStaticScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_static_mu;
unsigned char* g_static_addr[kMaxDevices] = {nullptr};

// Device address of the scratch array for the current device, looked up once per device.
int static_scratch(unsigned char** out) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return PRBF_ERR_CUDA;
  std::lock_guard<std::mutex> lock(g_static_mu);
  if (!g_static_addr[dev]) {
    void* p = nullptr;
    if (cudaGetSymbolAddress(&p, g_static_sort_scratch) != cudaSuccess || !p) {
      cudaGetLastError();  // leave no stale error for a later launch check
      return PRBF_ERR_CUDA;
    }
    g_static_addr[dev] = (unsigned char*)p;
  }
  *out = g_static_addr[dev];
  return PRBF_OK;
}

// Exclusive scan of n <= kStaticMaxScan ints with the partial sums in the scratch array.
void static_scan(int* data, long long n, int* sums1, int* sums2, cudaStream_t s) {
  long long nb1 = (n + kScanTile - 1) / kScanTile;
  if (nb1 == 1) {
    k_scan_tiles<int><<<1, kScanThreads, 0, s>>>(data, data, nullptr, n);
    return;
  }
  k_scan_tiles<int><<<(unsigned)nb1, kScanThreads, 0, s>>>(data, data, sums1, n);
  long long nb2 = (nb1 + kScanTile - 1) / kScanTile;
  if (nb2 == 1) {
    k_scan_tiles<int><<<1, kScanThreads, 0, s>>>(sums1, sums1, nullptr, nb1);
  } else {
    k_scan_tiles<int><<<(unsigned)nb2, kScanThreads, 0, s>>>(sums1, sums1, sums2, nb1);
    k_scan_tiles<int><<<1, kScanThreads, 0, s>>>(sums2, sums2, nullptr, nb2);
    k_scan_add<int><<<(unsigned)nb2, kScanThreads, 0, s>>>(sums1, sums2, nb1);
  }
  k_scan_add<int><<<(unsigned)nb1, kScanThreads, 0, s>>>(data, sums1, n);
}

}  // namespace
}  // namespace prbf

extern "C" int prbf_cell_sort_static(int dim, int n, const double* x, const double* y, const double* z,
                                     double sigma, int nsigma_box, int sigma_buffer, int sigma_trunc,
                                     int* perm, int* cell_start, int cell_start_len, int* ncell_out,
                                     void* stream) {
  using namespace prbf;
  if ((dim != 2 && dim != 3) || n <= 0 || !x || !y || (dim == 3 && !z) || !perm || !cell_start ||
      cell_start_len <= 0)
    return PRBF_ERR_ARG;
  if (n > kStaticMaxPoints) return PRBF_ERR_CAPACITY;  // beyond the fixed scratch array
  cudaStream_t s = (cudaStream_t)stream;
  unsigned char* base = nullptr;
  int st = static_scratch(&base);
  if (st) return st;
  unsigned* keyA = (unsigned*)(base + kOffKeyA);
  unsigned* keyB = (unsigned*)(base + kOffKeyB);
  int* valB = (int*)(base + kOffValB);
  int* hist = (int*)(base + kOffHist);
  int* sums1 = (int*)(base + kOffSums1);
  int* sums2 = (int*)(base + kOffSums2);
  double* bpart = (double*)(base + kOffBboxPart);
  double* bbox = (double*)(base + kOffBbox);
  unsigned* err = (unsigned*)(base + kOffErr);
  try {
    // the error word is the only scratch that must start at zero
    PRBF_CUDA(cudaMemsetAsync(err, 0, sizeof(unsigned), s));
    int blocks = std::min(kBboxBlocks, std::max(1, ceil_div(n, kBboxThreads)));
    k_bbox_partial<<<blocks, kBboxThreads, 0, s>>>(n, x, y, dim == 3 ? z : nullptr, bpart);
    k_bbox_final<<<1, 32, 0, s>>>(blocks, bpart, bbox);
    PRBF_CHECK_LAUNCH();
    double b[6];
    PRBF_CUDA(cudaMemcpyAsync(b, bbox, sizeof(b), cudaMemcpyDeviceToHost, s));
    PRBF_CUDA(cudaStreamSynchronize(s));
    Grid g = make_grid(dim, b, sigma, nsigma_box, sigma_buffer, sigma_trunc);
    // the grid follows from the points' bounding box: report its size before any capacity
    // refusal, so that a caller whose cell_start buffer is too short learns what to allocate
    if (ncell_out) *ncell_out = g.ncell;
    if ((long long)g.ncell + 1 > cell_start_len || (long long)g.ncell + 1 > kStaticMaxScan)
      return PRBF_ERR_CAPACITY;
    PRBF_CUDA(cudaMemsetAsync(cell_start, 0, sizeof(int) * ((size_t)g.ncell + 1), s));
    k_cell_ids<<<ceil_div(n, 256), 256, 0, s>>>(g, n, x, y, dim == 3 ? z : nullptr, keyA, perm, cell_start, err);
    PRBF_CHECK_LAUNCH();
    static_scan(cell_start, (long long)g.ncell + 1, sums1, sums2, s);
    int bits = 0;
    while (bits < 31 && (1u << bits) < (unsigned)g.ncell) bits++;
    int passes = (bits + 7) / 8;
    int ntiles = ceil_div(n, kRadixTile);
    unsigned *kin = keyA, *kout = keyB;
    int *vin = perm, *vout = valB;
    for (int p = 0; p < passes; p++) {
      k_radix_hist<<<ntiles, kRadixThreads, 0, s>>>(kin, n, 8 * p, hist, ntiles);
      static_scan(hist, 256LL * ntiles, sums1, sums2, s);
      k_radix_scatter<<<ntiles, kRadixThreads, 0, s>>>(kin, vin, kout, vout, n, 8 * p, hist, ntiles);
      PRBF_CHECK_LAUNCH();
      std::swap(kin, kout);
      std::swap(vin, vout);
    }
    if (vin != perm)
      PRBF_CUDA(cudaMemcpyAsync(perm, vin, sizeof(int) * (size_t)n, cudaMemcpyDeviceToDevice, s));
    unsigned herr = 0;
    PRBF_CUDA(cudaMemcpyAsync(&herr, err, sizeof(unsigned), cudaMemcpyDeviceToHost, s));
    PRBF_CUDA(cudaStreamSynchronize(s));
    if (herr & DEV_ERR_RANGE) return PRBF_ERR_RANGE;
    if (herr & DEV_ERR_TIMEOUT) return PRBF_ERR_TIMEOUT;
    if (herr & (DEV_ERR_CAPACITY | DEV_ERR_INDEX)) return PRBF_ERR_CAPACITY;
    if (herr) return PRBF_ERR_CUDA;  // no other bit is raised by these kernels
    return PRBF_OK;
  } catch (const Error& e) {
    return e.status;
  } catch (const std::bad_alloc&) {
    return PRBF_ERR_CAPACITY;  // host memory exhausted
  } catch (const std::exception&) {
    return PRBF_ERR_ARG;
  }
}
