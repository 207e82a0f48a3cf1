// device.h -- device memory ownership and the kernel entry points shared between
// translation units.
#pragma once
#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "common.cuh"

namespace prbf {

// Owning device buffer (cudaMalloc / cudaFree), grow-only.
template <class T>
struct DevBuf {
  T* p = nullptr;
  size_t n = 0;
  DevBuf() = default;
  DevBuf(const DevBuf&) = delete;
  DevBuf& operator=(const DevBuf&) = delete;
  ~DevBuf() { release(); }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    n = 0;
  }
  // Ensures capacity for `count` elements; contents are not preserved on growth.
  T* reserve(size_t count) {
    if (count <= n && p) return p;
    release();
    size_t bytes = count * sizeof(T);
    if (bytes == 0) bytes = 16;
    const cudaError_t e = cudaMalloc((void**)&p, bytes);
    if (e != cudaSuccess) {
      p = nullptr;
      cudaGetLastError();  // an allocation failure is not sticky: later launch checks must not see it
      if (e == cudaErrorMemoryAllocation)
        throw Error(PRBF_ERR_CAPACITY, "device memory exhausted (" + std::to_string(bytes) + " bytes requested)");
      throw Error(PRBF_ERR_CUDA, std::string("cudaMalloc: ") + cudaGetErrorString(e));
    }
    n = count;
    return p;
  }
  T* get() const { return p; }
};

// Temporary device storage handed to multi-kernel operations (sort, scans, Krylov
// reductions). Slots are reused between calls and only ever grow.
struct Workspace {
  std::vector<DevBuf<unsigned char>*> slots;
  ~Workspace() {
    for (auto* s : slots) delete s;
  }
  void* get(int id, size_t bytes) {
    while ((int)slots.size() <= id) slots.push_back(new DevBuf<unsigned char>());
    return slots[id]->reserve(bytes < 256 ? 256 : bytes);
  }
};

// ---- cellsort.cu -------------------------------------------------------------------
// Min/max of each coordinate into out6 (device): xmin xmax ymin ymax zmin zmax.
void bbox_dev(int n, const double* x, const double* y, const double* z, double* out6,
              Workspace& ws, cudaStream_t s);
// Exclusive scan of n values into out (in-place allowed); returns nothing, total is
// out[n-1]+in[n-1] for callers that keep in.
void scan_exclusive_dev(const int* in, int* out, long long n, Workspace& ws, int slot,
                        cudaStream_t s);
void scan_exclusive_dev(const long long* in, long long* out, long long n, Workspace& ws,
                        int slot, cudaStream_t s);
// Stable sort of n points into cells: perm[k] = caller index of the k-th sorted point,
// cell_start[c] = first sorted position of cell c (ncell+1 entries). err receives
// DEV_ERR_RANGE if a point lies outside the grid.
void cell_sort_dev(const Grid& g, int n, const double* x, const double* y, const double* z,
                   int* perm, int* cell_start, unsigned* err, Workspace& ws, cudaStream_t s);
// out[k] = in[perm[k]] for k < n (double), and the inverse scatter out[perm[k]] = in[k].
void gather_dev(int n, const int* perm, const double* in, double* out, cudaStream_t s);
void scatter_dev(int n, const int* perm, const double* in, double* out, cudaStream_t s);

// ---- gauss.cu ----------------------------------------------------------------------
// Sorted point set on the device (SoA, padded so 16-byte bulk copies of any range stay
// inside the allocation).
struct PointsView {
  int n;
  const double* x;
  const double* y;
  const double* z;  // null in 2D
  const int* cell_start;
};

// Work list of a truncated Gaussian sum: one item per (target cell, tile of targets).
struct GaussPlan {
  Grid g;
  int nitems = 0;
  int max_tile = 0;
  long long pairs = 0;
  int max_trunc = 0;
  int grid = 0;           // CTAs of a launch (0: one per item; fewer: persistent rounds)
  bool batched = false;   // cells index a concatenation of grids (grids, cprob)
  DevBuf<int2> items;     // (cell, first target of the tile)
  DevBuf<int> trunc_cnt;  // truncation-set size per target cell
  DevBuf<Grid> grids;     // batched: one grid per problem (with its first global cell)
  DevBuf<int> cprob;      // batched: problem of each global cell
  SegSkip seg;            // batched: skip the items of stopped problems (when seg.done set)
  // FP32 form: per-source FP32 cell-relative coordinates and truncation masks (built by
  // gauss_plan_dev when nb_trunc <= 7 and ny < 65536), and a FP32 copy of <= 4 weight
  // vectors at stride g32_stride
  bool f32_ready = false;
  long long g32_stride = 0;
  DevBuf<float> su, sv, sw, g32;
  DevBuf<unsigned long long> smask;
  // FP64 matvec with each exponential used for both rows (targets == sources, every cell
  // <= 128 points): K partial slots of pstride entries per weight vector, for up to sym_nv
  // vectors per launch (set sym_nv before gauss_plan_dev; kept zero between products), and
  // each point's cell y index
  bool sym_ready = false;
  int sym_nv = 1;
  int sym_K = 0;
  long long sym_pstride = 0;
  DevBuf<double> sym_part;
  DevBuf<unsigned long long> sym_cy;
  int sym_nitems = 0;      // batches: one item per non-empty cell (else the plan's items)
  int sym_ncs = 0;         // batches: entries of the global cell starts (else g.ncell + 1)
  DevBuf<int2> sym_items;
};

// Builds the work list and the truncation-set sizes; sets plan.pairs / max_trunc. forms:
// also the FP32 form's source data and the symmetric FP64 form's buffers (a plan used only
// for its sizes passes false).
void gauss_plan_dev(GaussPlan& plan, const PointsView& tgt, const PointsView& src,
                    unsigned* err, Workspace& ws, cudaStream_t s, bool forms = true);
// FP32 form's source data of a batch (each problem with its own grid and scale, grids with
// their first global cell); sets plan.f32_ready when every grid qualifies.
void gauss_plan_f32_batch(GaussPlan& plan, const std::vector<Grid>& grids, const PointsView& src, cudaStream_t s);
// Symmetric FP64 form of a batch (every grid with the same window, every cell <= 128
// points; hcs: the global cell starts on the host); false when it does not apply.
bool gauss_plan_sym_batch(GaussPlan& plan, const std::vector<Grid>& grids, const PointsView& src,
                          const std::vector<int>& hcs, cudaStream_t s);
// w[i] = sum_{j in trunc(cell(i))} g[j] exp(-|t_i - s_j|^2 / (2 sigma^2)) / (2 pi sigma^2)
// for all sorted targets i; g must be a padded device vector of src.n (+2) entries.
// w = A g for nv weight vectors at stride vstride (even; vectors padded as the sources)
void gauss_sum_dev(const GaussPlan& plan, const PointsView& tgt, const PointsView& src,
                   const double* g, double* w, bool fp32, unsigned* err, cudaStream_t s,
                   const int* skip = nullptr, int nv = 1, long long vstride = 0);

// Device address of the FP64 exponential table of the sums (n = 1024 entries of the
// T[j]-folded cubic, 4 coefficients each), uploaded to the current device on first use.
// Kernels of other files use it through exp_neg_tab (common.cuh), so every FP64 Gaussian
// of the library evaluates exp the same way.
const double* exp_table_dev(cudaStream_t s);

}  // namespace prbf
