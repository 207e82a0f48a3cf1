// rasm.cu -- restricted additive Schwarz preconditioner on the GPU.
//
// Subdomain of cell c = its buffer set (2d/get_buffer.h:9-77: the centre points first,
// then the neighbour points inside the buffer box), block A_c = phi(|x_i - x_j|) over all
// pairs of the subdomain, untruncated (mysubmat, 2d/matmult.cxx:53-104). The restricted
// apply writes only the centre points (is_local = first n_c entries of is,
// 2d/rbf_interpolation.cxx:214-229):  (B r)[centre(c)] = (A_c^-1 r[buffer(c)])[0:n_c].
//
// Two apply forms. Plain FP64: the packed Cholesky factor of every block is kept (about
// n_b^2/2 doubles per block) and each apply runs a blocked forward substitution plus a
// back substitution on the centre block only; triangular solves are backward stable, so
// GMRES reaches the same true residual as with the reference's LU solves. An explicit
// inverse applied as a GEMV is not: its rounding (eps |A_c^-1| |r|) caps the attainable
// true residual near 1e-11 on the 2D configurations. Mixed form: S_c = the n_c centre
// rows of A_c^-1 (n_c x n_b, FP32) once, so an apply is one batched GEMV that streams
// S_c from HBM; the outer FP64 refinement removes its error. Per block (one CTA):
//   order the block neighbours first, centre last; K = 2 pi sigma^2 A_c, entries in (0, 1];
//   left-looking tiled Cholesky K = L L^T over 64-column tiles -- FP64: k_chol_fp64 on the
//   CUDA cores, in an operation order a CPU restatement reproduces bit for bit; FP32:
//   k_chol_tc, updates and panel solves on the tensor cores;
//   FP32 restricted form: S_c = 2 pi sigma^2 X^T with X = K^-1 E_centre, from Z = X^T solving
//   Z L L^T = E_centre^T by substitutions on the tensor cores in the same kernel, stored
//   row-major in the block's column order.
// Blocks whose factorisation meets a non-positive pivot are retried with a diagonal shift,
// or (FP64, on request) factored by LU with partial pivoting.
#include <algorithm>
#include <cmath>
#include <vector>

#include "rasm.h"

namespace prbf {
namespace {

constexpr int TB = 64;         // tile edge
constexpr int NTH = 256;       // threads per CTA (16 x 16, 4 x 4 outputs each)
constexpr int kAsmCtas = 16;   // CTAs per block of the assembly (a warp per row)
static_assert(NTH == 256 && TB == 64, "the tile kernels map 16 x 16 threads onto 4 x 4 outputs each");
// inner chunk of the tile GEMM: FP32 is latency-bound on its operand loads, so it takes
// wider chunks; FP64 is bound by the FP64 pipe and keeps shared memory small
template <class T>
struct KCOf {
  static constexpr int v = std::is_same<T, float>::value ? 32 : 16;
};

template <class T>
struct SP {  // padded shared row strides (16-byte aligned rows)
  static constexpr int S = std::is_same<T, float>::value ? TB + 4 : TB + 2;
};

// ---- buffer lists ------------------------------------------------------------------
// One warp per cell. mode 0: count; mode 1: fill idx[boff[c] ...] in the reference's
// order (2d/get_buffer.h:31-77, 3d twin): the centre points first, then the neighbour
// cells in jx, jy (, jz) order, each cell's points ascending. In 2D the cells jy0 .. jy1
// of a column jx are one contiguous range of the sorted points; in 3D (cell index
// iz nx ny + ix ny + iy) consecutive jz are not, so the window is walked cell by cell.
__global__ void k_buffer_lists(Grid g, const double* __restrict__ x, const double* __restrict__ y,
                               const double* __restrict__ z, const int* __restrict__ cs, int mode,
                               int* __restrict__ cnt, const long long* __restrict__ boff,
                               int* __restrict__ idx) {
  int c = blockIdx.x * (blockDim.x / 32) + (threadIdx.x >> 5);
  int lane = threadIdx.x & 31;
  if (c >= g.ncell) return;
  int c0 = cs[c], c1 = cs[c + 1];
  if (c0 == c1) {  // empty cell: npbufferi = 0 (2d/get_buffer.h:169-171)
    if (mode == 0 && lane == 0) cnt[c] = 0;
    return;
  }
  int ix, iy, iz;
  cell_xyz(g, c, ix, iy, iz);
  double xc = centre_coord(g.xmin, ix, g.box), yc = centre_coord(g.ymin, iy, g.box);
  double zc = g.dim == 3 ? centre_coord(g.zmin, iz, g.box) : 0.0;
  double L = g.buffer_len;
  int nb = g.nb_buffer;
  int jx0 = max(0, ix - nb), jx1 = min(g.nx - 1, ix + nb);
  int jy0 = max(0, iy - nb), jy1 = min(g.ny - 1, iy + nb);
  int jz0 = g.dim == 3 ? max(0, iz - nb) : 0, jz1 = g.dim == 3 ? min(g.nz - 1, iz + nb) : 0;
  long long pos = mode ? boff[c] : 0;
  int n = 0;
  // centre points first
  for (int j = c0 + lane; j < c1; j += 32)
    if (mode) idx[pos + (j - c0)] = j;
  n = c1 - c0;
  // points [a, b) of the window that pass the buffer box test, in order (the centre
  // cell's own points are skipped: they lead the list)
  auto scan = [&](int a, int b) {
    for (int j0 = a; j0 < b; j0 += 32) {
      int j = j0 + lane;
      bool in = false;
      if (j < b && !(j >= c0 && j < c1)) {
        in = fabs(x[j] - xc) < L && fabs(y[j] - yc) < L;
        if (g.dim == 3) in = in && fabs(z[j] - zc) < L;
      }
      unsigned bal = __ballot_sync(0xffffffffu, in);
      if (mode && in) idx[pos + n + __popc(bal & ((1u << lane) - 1u))] = j;
      n += __popc(bal);
    }
  };
  if (g.dim == 2) {
    for (int jx = jx0; jx <= jx1; jx++) scan(cs[cell_of(g, jx, jy0, 0)], cs[cell_of(g, jx, jy1, 0) + 1]);
  } else {
    for (int jx = jx0; jx <= jx1; jx++)
      for (int jy = jy0; jy <= jy1; jy++)
        for (int jz = jz0; jz <= jz1; jz++) {
          const int cc = cell_of(g, jx, jy, jz);
          if (cc != c) scan(cs[cc], cs[cc + 1]);
        }
  }
  if (mode == 0 && lane == 0) cnt[c] = n;
}

// ---- block assembly ----------------------------------------------------------------
// FP32 form: every coordinate as an unevaluated sum of two floats, v = h + l (h = v
// rounded, l = the rest rounded), so that a difference is (h_a - h_b) + (l_a - l_b) in FP32
// (within 1.5 ulp of the exact difference, as against 0.5 ulp for an FP64 difference
// rounded once) without the FP64 pipe.
__global__ void k_split_hl(long long n, const double* __restrict__ v, float2* __restrict__ out) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const double a = v[i];
    const float h = (float)a;
    out[i] = make_float2(h, (float)(a - (double)h));
  }
}

// K[i][j] = exp(-|x_a - x_b|^2 / (2 sigma^2)) (+ shift on the diagonal), block order
// neighbours first then centre: block row i < n1 -> buffer entry nc + i, else i - n1.
// Lower triangle only (the factorisation reads nothing else). hl (FP32 form): the n
// points' coordinates split by k_split_hl, dim arrays of n one after the other. FP64 form:
// the differences as the reference forms them (x_a - x_b), |d|^2 = fma(dy, dy, dx dx)
// (+ fma(dz, dz, .)), and the exponential of the sums' table (exp_neg_tab, kexp = 1024 /
// (2 sigma^2 ln2)), every operation rounded as written.
// FP32 rows of the block assembly: one warp, lanes along row i (columns 0..i), the split
// coordinates from shared memory, the exponential as the FP32 sums take it (ex2.approx);
// the diagonal shift is added by the lane that wrote the diagonal.
__device__ __forceinline__ float asm_ex2(float x) {
  float y;
  asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}
template <int DIM>
__device__ __forceinline__ void asm_row_f32(float* __restrict__ Arow, const float2* s_hl, int nbk, int i, float c2,
                                            float sh, int lane) {
  float2 ha[DIM];
#pragma unroll
  for (int d = 0; d < DIM; d++) ha[d] = s_hl[d * nbk + i];
  for (int j = lane; j <= i; j += 32) {
    float r2 = 0.f;
#pragma unroll
    for (int d = 0; d < DIM; d++) {
      const float2 hb = s_hl[d * nbk + j];
      const float dd = (ha[d].x - hb.x) + (ha[d].y - hb.y);
      r2 = fmaf(dd, dd, r2);
    }
    Arow[j] = asm_ex2(-r2 * c2);
  }
  if (sh != 0.f && lane == (i & 31)) Arow[i] += sh;
}

template <class T>
__global__ void k_assemble(int nblk, const int* __restrict__ blk_cell, const long long* __restrict__ boff,
                           const int* __restrict__ cs, const int* __restrict__ idx,
                           const long long* __restrict__ koff, const double* __restrict__ x,
                           const double* __restrict__ y, const double* __restrict__ z, int dim, double inv2s2_all,
                           const double* __restrict__ cell_sig, double shift, T* __restrict__ K,
                           const unsigned char* __restrict__ only, const float2* __restrict__ hl, long long n,
                           double kexp_all, const double* __restrict__ tab) {
  int b = blockIdx.y;
  if (b >= nblk || (only && !only[b])) return;
  int c = blk_cell[b];
  const double inv2s2 = cell_sig ? 1.0 / (2.0 * cell_sig[c] * cell_sig[c]) : inv2s2_all;
  const double kexp = cell_sig ? kexp_of_sigma(cell_sig[c]) : kexp_all;
  int nbk = (int)(boff[c + 1] - boff[c]);
  int nc = cs[c + 1] - cs[c], n1 = nbk - nc;
  const int* id = idx + boff[c];
  T* A = K + koff[b];
  // FP32: the block's split coordinates staged in shared memory once (block order), so an
  // entry reads its column's coordinates from there instead of gathering them per entry
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float2* s_hl = (float2*)smem_raw;  // dim x nbk (FP32 form only)
  if constexpr (std::is_same<T, float>::value) {
    for (int j = threadIdx.x; j < nbk; j += blockDim.x) {
      const int pb = id[j < n1 ? nc + j : j - n1];
      for (int d = 0; d < dim; d++) s_hl[d * nbk + j] = hl[d * n + pb];
    }
    __syncthreads();
  }
  // a warp per row (rows dealt round-robin over the block's CTAs and warps), lanes along it
  const int nw = blockDim.x >> 5, lane = threadIdx.x & 31;
  if constexpr (std::is_same<T, float>::value) {
    const float c2 = (float)(inv2s2 * 1.4426950408889634), sh = (float)shift;
    for (int i = blockIdx.x * nw + (threadIdx.x >> 5); i < nbk; i += gridDim.x * nw) {
      if (dim == 3)
        asm_row_f32<3>(A + (long long)i * nbk, s_hl, nbk, i, c2, sh, lane);
      else
        asm_row_f32<2>(A + (long long)i * nbk, s_hl, nbk, i, c2, sh, lane);
    }
  } else {
    for (int i = blockIdx.x * nw + (threadIdx.x >> 5); i < nbk; i += gridDim.x * nw) {
      const int pa = id[i < n1 ? nc + i : i - n1];
      const double xa = x[pa], ya = y[pa], za = dim == 3 ? z[pa] : 0.0;
      for (int j = lane; j <= i; j += 32) {
        const int pb = id[j < n1 ? nc + j : j - n1];
        const double dx = __dsub_rn(xa, x[pb]), dy = __dsub_rn(ya, y[pb]);
        double r2 = __fma_rn(dy, dy, __dmul_rn(dx, dx));
        if (dim == 3) {
          const double dz = __dsub_rn(za, z[pb]);
          r2 = __fma_rn(dz, dz, r2);
        }
        double v = exp_neg_tab(r2, kexp, tab);
        if (i == j) v = __dadd_rn(v, shift);
        A[(long long)i * nbk + j] = v;
      }
    }
  }
}

// ---- tile machinery (one CTA = one block) -------------------------------------------
template <class T>
struct Tiles {
  T* As;  // [2][KC][S] (double buffered)
  T* Bs;  // [2][KC][S]
  T* C;   // [TB][S] staging tile
  T* M;   // [TB][S] current diagonal inverse
};

// A KC x TB chunk of an operand, element (r, m) at src[(row0 + r) * ld + col0 + m] if
// !trans, else src[(row0 + m) * ld + col0 + r]; out-of-range entries are zero. Fetched
// into registers (issued early, so the loads overlap the previous chunk's arithmetic),
// then written to shared memory as dst[m][r].
template <class T>
struct Chunk {
  static constexpr int KC = KCOf<T>::v;
  static constexpr int PER = KC * TB / NTH;
  T v[PER];
  __device__ __forceinline__ void fetch(const T* src, long long ld, int row0, int col0, int nr, int nm, bool trans) {
#pragma unroll
    for (int q = 0; q < PER; q++) {
      int e = threadIdx.x + q * NTH, r, m;
      if (!trans) {
        m = e % KC;
        r = e / KC;
      } else {
        r = e % TB;
        m = e / TB;
      }
      v[q] = (r < nr && m < nm) ? (trans ? src[(long long)(row0 + m) * ld + col0 + r]
                                          : src[(long long)(row0 + r) * ld + col0 + m])
                                : T(0);
    }
  }
  __device__ __forceinline__ void store(T* dst, bool trans) const {
    constexpr int S = SP<T>::S;
#pragma unroll
    for (int q = 0; q < PER; q++) {
      int e = threadIdx.x + q * NTH;
      int r = trans ? e % TB : e / KC, m = trans ? e / TB : e % KC;
      dst[m * S + r] = v[q];
    }
  }
};

// acc[4][4] -= sum_m As[m][r] Bs[m][c] over the first mm entries of the staged chunk.
// Rows at or past nr (the tile's height) are zero padding that is never stored: their
// threads skip the arithmetic, whole warps where the tile ends above their 8 rows (the
// short last tile of a block), and a partial chunk stops at mm.
// Output mapping of a 64 x 64 tile over the 256 threads: 4 x 4 blocks (ty, tx) of the 16 x 16
// block grid, thread 16 ty + tx; or, for a diagonal tile of the factorisation (only its
// lower part is kept), its 136 blocks with tx <= ty on threads 0 .. 135, so that warps 5 .. 7
// issue no arithmetic there. Each entry still receives the same operations in the same order.
struct TileMap {
  int ty, tx;
  bool on;
};
__device__ __forceinline__ TileMap tile_map(bool lower_blocks) {
  const int t = threadIdx.x;
  if (!lower_blocks) return TileMap{t / 16, t % 16, true};
  if (t >= 136) return TileMap{0, 0, false};
  int by = 0;
  while ((by + 1) * (by + 2) / 2 <= t) by++;  // row of block t in the lower triangle
  return TileMap{by, t - by * (by + 1) / 2, true};
}

template <class T>
__device__ __forceinline__ void mma_chunk(const T* As, const T* Bs, T acc[4][4], int ty, int tx, int nr, int mm) {
  if (4 * ty >= nr) return;
  constexpr int S = SP<T>::S;
  auto step = [&](int m) {
    T a[4], b[4];
#pragma unroll
    for (int q = 0; q < 4; q++) {
      a[q] = As[m * S + ty * 4 + q];
      b[q] = Bs[m * S + tx * 4 + q];
    }
#pragma unroll
    for (int p = 0; p < 4; p++)
#pragma unroll
      for (int q = 0; q < 4; q++) acc[p][q] = fma(-a[p], b[q], acc[p][q]);
  };
  if (mm == KCOf<T>::v) {
#pragma unroll
    for (int m = 0; m < KCOf<T>::v; m++) step(m);
  } else {
#pragma unroll 4
    for (int m = 0; m < mm; m++) step(m);
  }
}

// acc -= opA(P) opB(Q) over an inner dimension of length nm (chunks of KC).
// opA(P)(r, m): P row-major with leading dim ldp, origin (pr, pc), transposed if ta.
// opB(Q)(c, m): likewise.
template <class T>
__device__ void tile_update(Tiles<T>& t, T acc[4][4], const T* P, long long ldp, int pr, int pc, int nr, bool ta,
                            const T* Q, long long ldq, int qr, int qc, int ncol, bool tb, int nm,
                            TileMap mp = tile_map(false)) {
  constexpr int KC = KCOf<T>::v;
  constexpr int S = SP<T>::S;
  const int ty = mp.ty, tx = mp.tx;
  const int nchunk = (nm + KC - 1) / KC;
  Chunk<T> ca, cb;
  auto fetch = [&](int m0) {
    int mm = min(KC, nm - m0);
    if (!ta)
      ca.fetch(P, ldp, pr, pc + m0, nr, mm, false);
    else
      ca.fetch(P, ldp, pr + m0, pc, nr, mm, true);
    if (!tb)
      cb.fetch(Q, ldq, qr, qc + m0, ncol, mm, false);
    else
      cb.fetch(Q, ldq, qr + m0, qc, ncol, mm, true);
  };
  __syncthreads();  // the previous user of the staging buffers is done
  if (nchunk > 0) fetch(0);
  for (int c = 0; c < nchunk; c++) {
    T* As = t.As + (c & 1) * KC * S;
    T* Bs = t.Bs + (c & 1) * KC * S;
    ca.store(As, ta);
    cb.store(Bs, tb);
    __syncthreads();
    if (c + 1 < nchunk) fetch((c + 1) * KC);  // in flight during this chunk's arithmetic
    if (mp.on) mma_chunk<T>(As, Bs, acc, ty, tx, nr, min(KC, nm - c * KC));
  }
}

template <class T>
__device__ void acc_to_smem(T* C, const T acc[4][4], TileMap mp = tile_map(false)) {
  constexpr int S = SP<T>::S;
  if (!mp.on) return;
  const int ty = mp.ty, tx = mp.tx;
#pragma unroll
  for (int p = 0; p < 4; p++)
#pragma unroll
    for (int q = 0; q < 4; q++) C[(ty * 4 + p) * S + tx * 4 + q] = acc[p][q];
}

// Ordered form of the diagonal-tile Cholesky (plain FP64 factor form): the h x h leading
// part of C (lower) becomes L_kk in place, rd[j] = 1 / L_kk[j][j]. Column j: s = sqrt(c_jj),
// r = 1/s, l_ij = c_ij * r, then c_il = fma(-l_ij, l_lj, c_il) for j < l <= i. Every entry
// thus receives its updates in ascending column order, each one rounding, exactly as the
// unblocked right-looking Cholesky with those operations computes it. Returns false if a
// pivot is not positive (it is then taken as 1 and the block retried with a shift).
// Entries outside h x h are set to the identity.
template <class T>
__device__ bool potrf_rd(T* C, T* rd, int h) {
  constexpr int S = SP<T>::S;
  __shared__ int s_bad;
  if (threadIdx.x == 0) s_bad = 0;
  __syncthreads();
  for (int e = threadIdx.x; e < TB * TB; e += NTH) {
    int r = e / TB, c = e % TB;
    if (r >= h || c >= h) C[r * S + c] = (r == c) ? T(1) : T(0);
    if (c > r) C[r * S + c] = T(0);
  }
  __syncthreads();
  const int ty = threadIdx.x / 16, tx = threadIdx.x % 16;
  for (int j = 0; j < h; j++) {
    T d = C[j * S + j];
    if (!(d > T(0))) {
      if (threadIdx.x == 0) s_bad = 1;
      d = T(1);
    }
    const T sq = sqrt(d);
    const T rc = T(1) / sq;
    __syncthreads();
    for (int i = j + 1 + threadIdx.x; i < h; i += NTH) C[i * S + j] = C[i * S + j] * rc;
    __syncthreads();
    if (threadIdx.x == 0) {
      C[j * S + j] = sq;
      rd[j] = rc;
    }
    T ci[4], cl[4];
#pragma unroll
    for (int p = 0; p < 4; p++) {
      const int i = 4 * ty + p, l = 4 * tx + p;
      ci[p] = (i > j && i < h) ? C[i * S + j] : T(0);
      cl[p] = (l > j && l < h) ? C[l * S + j] : T(0);
    }
#pragma unroll
    for (int p = 0; p < 4; p++)
#pragma unroll
      for (int q = 0; q < 4; q++) {
        const int i = 4 * ty + p, l = 4 * tx + q;
        if (l > j && l <= i && i < h) C[i * S + l] = fma(-ci[p], cl[q], C[i * S + l]);
      }
    __syncthreads();
  }
  for (int j = h + threadIdx.x; j < TB; j += NTH) rd[j] = T(1);
  __syncthreads();
  return s_bad == 0;
}

// Panel solve of the ordered factor form: rows of C (a tile below the diagonal, after its
// trailing updates) become C L_kk^-T in place: for k = 0 .. hk-1, l_rk = c_rk * rd[k], then
// c_rj = fma(-l_rk, L_kk[j][k], c_rj) for k < j < hk -- per entry the same sequence as the
// unblocked algorithm, with no explicit inverse. Four threads per row, thread sub owning
// columns sub + 4m (register-resident; k is unrolled so every index is static); the pivot
// column's owner scales and broadcasts within its quad. Rows at or past hi are zero padding
// (whole warps beyond them return). All threads of a warp reach every shuffle.
template <class T>
__device__ void trsm_rows(T* C, const T* Lk, const T* rd, int hi, int hk) {
  constexpr int S = SP<T>::S;
  static_assert(TB == 64 && NTH == 256, "64 rows x 4 threads");
  const int r = threadIdx.x >> 2, sub = threadIdx.x & 3, lane = threadIdx.x & 31;
  if ((r & ~7) >= hi) return;  // warp-uniform: every row of this warp is padding
  T c[16];
#pragma unroll
  for (int m = 0; m < 16; m++) c[m] = C[r * S + sub + 4 * m];
  const T* lrow = Lk + sub * S;  // row sub + 4m of L_kk at lrow[4 m S] (static offsets)
#pragma unroll
  for (int k = 0; k < TB; k++) {
    if (k >= hk) break;
    const int owner = k & 3, m0 = k >> 2;
    T x = c[m0] * rd[k];
    x = __shfl_sync(0xffffffffu, x, (lane & ~3) | owner);
    if (sub == owner) c[m0] = x;
    if (sub > owner) c[m0] = fma(-x, lrow[4 * m0 * S + k], c[m0]);
#pragma unroll
    for (int m = m0 + 1; m < 16; m++) c[m] = fma(-x, lrow[4 * m * S + k], c[m]);
  }
#pragma unroll
  for (int m = 0; m < 16; m++) C[r * S + sub + 4 * m] = c[m];
}

template <class T>
__device__ void load_acc(const T* src, long long ld, int r0, int c0, int nr, int nc, T acc[4][4], bool lower_only,
                         TileMap mp = tile_map(false)) {
  const int ty = mp.ty, tx = mp.tx;
#pragma unroll
  for (int p = 0; p < 4; p++)
#pragma unroll
    for (int q = 0; q < 4; q++) {
      int r = ty * 4 + p, c = tx * 4 + q;
      bool ok = mp.on && r < nr && c < nc && (!lower_only || (r0 + r) >= (c0 + c));
      acc[p][q] = ok ? src[(long long)(r0 + r) * ld + c0 + c] : T(0);
    }
}

// Tile boundaries: neighbour part [0, n1) in TB steps, centre part [n1, nb) in TB steps.
__device__ __forceinline__ void tile_range(int t, int n1, int nb, int kc1, int& r0, int& h) {
  if (t < kc1) {
    r0 = t * TB;
    h = min(TB, n1 - r0);
  } else {
    r0 = n1 + (t - kc1) * TB;
    h = min(TB, nb - r0);
  }
}

// Packed factor rows: row i holds L[i][0..i] padded to a multiple of PackA<T> elements, so
// every row starts aligned and 8-element segments at multiples of 8 load as vectors. FP32
// rows are padded to 32 bytes, the DRAM sector: the substitutions stream 128-byte row
// segments, which then cover four whole sectors instead of straddling five. FP64 rows
// are padded to 16 bytes. rowoff(i) = sum_{r<i} A ceil((r+1)/A) = A (A q(q+1)/2 + rr (q+1)),
// q = i / A, rr = i % A.
template <class T>
struct PackA {
  static constexpr int v = std::is_same<T, float>::value ? 8 : 2;
};
template <class T>
__host__ __device__ __forceinline__ long long rowoff(long long i) {
  constexpr long long A = PackA<T>::v;
  const long long q = i / A, rr = i % A;
  return A * (A * q * (q + 1) / 2 + rr * (q + 1));
}

// ---- diagonal tiles of the tensor-core Cholesky -----------------------------------------
// The h x h leading part of C (lower, stride S) becomes L_kk and M its inverse (lower),
// entries outside h x h the identity (a non-positive pivot is taken as 1 and reported).
// Warp w owns columns 8w .. 8w + 7 and lane l rows l and l + 32 of them: 16 entries per
// thread, in registers for the whole factorisation.
// Step j: every warp applies the published column j of L to its own columns; then the
// owner of column j + 1, whose entries are now final, takes the pivot, scales the column
// and publishes it into the other half of a double buffer -- one CTA barrier per column,
// no shared-memory read-modify-write. The inverse needs no CTA barrier: forward
// substitution L M = I by rows, each warp on its own columns, row k's eight entries
// broadcast from their lane by shuffles. Pivots are applied as reciprocals, one IEEE
// division per column instead of one per entry: with a division per entry the inverse
// took eight times as long (clock64 per CTA on 900-point blocks).

// The owner warp of column j (Q = j % 8) takes the pivot, scales the column and writes it to
// buf with zeros at and above the diagonal.
template <int Q>
__device__ __forceinline__ void potrf_pub(float (&a)[2][8], int j, float* buf, float* rdg, int* s_bad, int h) {
  const int lane = threadIdx.x & 31;
  float d = __shfl_sync(0xffffffffu, j < 32 ? a[0][Q] : a[1][Q], j & 31);
  if (!(d > 0.f)) {
    if (lane == 0 && j < h) *s_bad = 1;
    d = 1.f;
  }
  const float s = sqrtf(d), rs = 1.f / s;
#pragma unroll
  for (int hh = 0; hh < 2; hh++) {
    const int i = lane + 32 * hh;
    float v = a[hh][Q];
    if (i > j)
      v *= rs;
    else if (i == j)
      v = s;
    a[hh][Q] = v;
    buf[i] = i > j ? v : 0.f;
  }
  if (lane == 0) rdg[j] = rs;
}

// j % 8 as a template argument (constant once the caller's loop is unrolled)
__device__ __forceinline__ void potrf_pub_j(float (&a)[2][8], int j, float* buf, float* rdg, int* s_bad, int h) {
  switch (j & 7) {
    case 0: potrf_pub<0>(a, j, buf, rdg, s_bad, h); break;
    case 1: potrf_pub<1>(a, j, buf, rdg, s_bad, h); break;
    case 2: potrf_pub<2>(a, j, buf, rdg, s_bad, h); break;
    case 3: potrf_pub<3>(a, j, buf, rdg, s_bad, h); break;
    case 4: potrf_pub<4>(a, j, buf, rdg, s_bad, h); break;
    case 5: potrf_pub<5>(a, j, buf, rdg, s_bad, h); break;
    case 6: potrf_pub<6>(a, j, buf, rdg, s_bad, h); break;
    default: potrf_pub<7>(a, j, buf, rdg, s_bad, h); break;
  }
}

__device__ bool potrf_trtri_w(float* C, float* M, int h) {
  constexpr int S = SP<float>::S;
  static_assert(NTH == 256 && TB == 64, "eight warps of eight columns, two rows per lane");
  __shared__ __align__(16) float colb[2][TB];
  __shared__ float rdg[TB];  // 1 / l_jj
  __shared__ int s_bad;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  float a[2][8];
#pragma unroll
  for (int hh = 0; hh < 2; hh++)
#pragma unroll
    for (int q = 0; q < 8; q++) {
      const int i = lane + 32 * hh, l = 8 * w + q;
      a[hh][q] = (i < h && l < h) ? (l <= i ? C[i * S + l] : 0.f) : (i == l ? 1.f : 0.f);
    }
  if (threadIdx.x == 0) s_bad = 0;
  if (w == 0) potrf_pub<0>(a, 0, colb[0], rdg, &s_bad, h);
  __syncthreads();
  for (int jb = 0; jb < TB / 8; jb++) {
#pragma unroll
    for (int jj = 0; jj < 8; jj++) {
      const int j = 8 * jb + jj;
      const float* cb = colb[j & 1];
      const float ci[2] = {cb[lane], cb[lane + 32]};
      const float4 c0 = *(const float4*)(cb + 8 * w), c1 = *(const float4*)(cb + 8 * w + 4);
      const float cl[8] = {c0.x, c0.y, c0.z, c0.w, c1.x, c1.y, c1.z, c1.w};
      // zeros at and above the diagonal of column j leave rows <= j and column j as they are
#pragma unroll
      for (int hh = 0; hh < 2; hh++)
#pragma unroll
        for (int q = 0; q < 8; q++) a[hh][q] = fma(-ci[hh], cl[q], a[hh][q]);
      if (j + 1 < TB && w == ((j + 1) >> 3)) potrf_pub_j(a, j + 1, colb[(j + 1) & 1], rdg, &s_bad, h);
      __syncthreads();
    }
  }
#pragma unroll
  for (int hh = 0; hh < 2; hh++)
#pragma unroll
    for (int q = 0; q < 8; q++) {
      const int i = lane + 32 * hh, l = 8 * w + q;
      C[i * S + l] = l <= i ? a[hh][q] : 0.f;
    }
  __syncthreads();
  // M = L^-1: x[i][c] starts at delta_ic; row k: m_kc = x[k][c] / l_kk, then x[i][c] -= l_ik m_kc
  // for the rows below. Rows above a warp's first column give m_kc = 0 for all its columns, so
  // the warp starts at row 8w; rows 0..31 live in the lanes' first half, 32..63 in the second.
#pragma unroll
  for (int hh = 0; hh < 2; hh++)
#pragma unroll
    for (int q = 0; q < 8; q++) a[hh][q] = (lane + 32 * hh == 8 * w + q) ? 1.f : 0.f;
  for (int k = 8 * w; k < 32; k++) {  // pivot row in the first half: every second-half row updates
    const float rkk = rdg[k];
    const float lik0 = C[lane * S + k], lik1 = C[(lane + 32) * S + k];
    float mk[8];
#pragma unroll
    for (int q = 0; q < 8; q++) {
      const float v = a[0][q] * rkk;  // the owner lane's value is the one kept
      if (lane == k) a[0][q] = v;
      mk[q] = __shfl_sync(0xffffffffu, v, k);
    }
    if (lane > k) {
#pragma unroll
      for (int q = 0; q < 8; q++) a[0][q] = fma(-lik0, mk[q], a[0][q]);
    }
#pragma unroll
    for (int q = 0; q < 8; q++) a[1][q] = fma(-lik1, mk[q], a[1][q]);
  }
  for (int k = max(32, 8 * w); k < TB; k++) {  // pivot row in the second half
    const float rkk = rdg[k];
    const float lik1 = C[(lane + 32) * S + k];
    float mk[8];
#pragma unroll
    for (int q = 0; q < 8; q++) {
      const float v = a[1][q] * rkk;
      if (lane == k - 32) a[1][q] = v;
      mk[q] = __shfl_sync(0xffffffffu, v, k - 32);
    }
    if (lane + 32 > k) {
#pragma unroll
      for (int q = 0; q < 8; q++) a[1][q] = fma(-lik1, mk[q], a[1][q]);
    }
  }
#pragma unroll
  for (int hh = 0; hh < 2; hh++)
#pragma unroll
    for (int q = 0; q < 8; q++) M[(lane + 32 * hh) * S + 8 * w + q] = a[hh][q];
  __syncthreads();
  return s_bad == 0;
}

// ---- FP32 block Cholesky on the tensor cores (tcgen05, 3xTF32) ------------------------
// The trailing updates C_ik -= sum_p L_ip L_kp^T and the panel solves L_ik = C_ik L_kk^-T
// of the left-looking tile Cholesky are GEMMs: each runs as tcgen05.mma kind::tf32 with
// M = 128 rows (two 64-row tiles of the column), N = 64, accumulating in TMEM. FP32
// accuracy comes from splitting every operand x = hi + lo (hi = x rounded to TF32, lo =
// the rest, also TF32): A B ~ Ahi Bhi + Ahi Blo + Alo Bhi. Operands go through shared
// memory in 32-column chunks in the canonical K-major layout without swizzle (core
// matrices of 8 rows x 16 bytes; element (r, k) at (r/8)*SBO + (k/4)*128 + (r%8)*16 +
// (k%4)*4 bytes, SBO = 8 core matrices = 1024 bytes, LBO = 128 bytes). One elected thread
// issues the MMAs and commits them to an mbarrier; the diagonal tiles are factored and
// inverted on the CUDA cores (potrf_trtri_w). Writes L (lower part) over the dense block;
// the factor form then packs it (k_pack_factor), the restricted S_c form computes S_c in
// the same kernel from L and the diagonal inverses (below).
constexpr int TC_KCH = 32;  // K columns per operand chunk

__device__ __forceinline__ uint32_t tc_smem(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }


__device__ __forceinline__ uint64_t tc_desc(uint32_t addr) {
  constexpr uint32_t lbo = 128, sbo = (TC_KCH / 4) * 128;
  uint64_t d = (uint64_t)((addr & 0x3FFFF) >> 4);
  d |= (uint64_t)(lbo >> 4) << 16;
  d |= (uint64_t)(sbo >> 4) << 32;
  d |= (uint64_t)1 << 46;  // descriptor version for tcgen05; base offset 0, no swizzle
  return d;
}

__device__ __forceinline__ void tc_split(float x, float& hi, float& lo) {
  hi = __uint_as_float((__float_as_uint(x) + 0x1000u) & 0xFFFFE000u);  // TF32, nearest
  lo = x - hi;
}

struct TcStage {
  float* ahi;  // [128][TC_KCH] canonical
  float* alo;
  float* bhi;  // [64][TC_KCH]
  float* blo;
};

// D (TMEM, 128 x 64 FP32) += A B^T over one staged chunk (TC_KCH = 4 MMAs of K = 8, 3 terms)
__device__ __forceinline__ void tc_issue(uint32_t tmem, const TcStage& st, bool first) {
  constexpr uint32_t idesc = (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(64 >> 3) << 17) |
                             ((uint32_t)(128 >> 4) << 24);  // D F32, A/B TF32, K-major, N 64, M 128
  const float* as[3] = {st.ahi, st.ahi, st.alo};
  const float* bs[3] = {st.bhi, st.blo, st.bhi};
#pragma unroll
  for (int ks = 0; ks < TC_KCH / 8; ks++)
#pragma unroll
    for (int t = 0; t < 3; t++) {
      const uint64_t da = tc_desc(tc_smem(as[t]) + ks * 256), db = tc_desc(tc_smem(bs[t]) + ks * 256);
      const uint32_t acc = (first && ks == 0 && t == 0) ? 0u : 1u;
      asm volatile(
          "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}" ::"r"(
              tmem),
          "l"(da), "l"(db), "r"(idesc), "r"(acc));
    }
}

// Commit the issued MMAs (elected thread) and wait (all threads, bounded); false on timeout.
__device__ __forceinline__ bool tc_commit_wait(uint64_t* bar, unsigned& phase) {
  if (threadIdx.x == 0)
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(tc_smem(bar))
                 : "memory");
  const bool ok = mbar_wait(bar, phase);
  phase ^= 1u;
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  return ok;
}

__device__ __forceinline__ void tc_sync() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}

// 32 columns of the thread's TMEM row: warp w reads lanes 32 (w % 4) .., column half w / 4
__device__ __forceinline__ void tc_load32(uint32_t tmem, float v[32]) {
  const int w = threadIdx.x >> 5;
  const uint32_t addr = tmem + ((uint32_t)(32 * (w & 3)) << 16) + (uint32_t)(32 * (w >> 2));
  uint32_t r[32];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16,%17,%18,"
      "%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]),
        "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]),
        "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(addr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int j = 0; j < 32; j++) v[j] = __uint_as_float(r[j]);
}

// One operand chunk in registers: A rows [ar0, ar0 + 128) (valid below ar_end and at or
// above ar_skip), columns [c0, c0 + 32) (valid below c_end) of the dense block, and B rows
// [br0, br0 + 64) (valid below br_end) from the dense block (Msm null) or from the diagonal
// inverse M in shared memory. Each warp instruction covers one core matrix (8 rows x 4
// columns: lane l -> row l/4, column l%4), so the global loads touch 8 row segments of 16
// bytes and the shared-memory stores are 32 consecutive words; all loads are issued before
// any is used.
struct TcRegs {
  float a[16], b[8];
};

// Bsrc: the matrix the B rows come from when not from Msm (same row stride nb as A); bt:
// B is the transpose of Bsrc, element (r, k) at Bsrc[(c0 + k) nb + br0 + r] (a warp
// instruction then reads 4 rows of Bsrc, 32 contiguous bytes each).
__device__ __forceinline__ void tc_fetch(TcRegs& R, const float* A, int nb, int ar0, int ar_skip, int ar_end, int c0,
                                         int c_end, int br0, int br_end, const float* Msm, int mcol0,
                                         const float* Bsrc = nullptr, bool bt = false) {
  constexpr int S = SP<float>::S;
  if (!Bsrc) Bsrc = A;
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
#pragma unroll
  for (int i = 0; i < 16; i++) {  // A: core matrices w*16 + i (row group cm/8, column group cm%8)
    const int cm = w * 16 + i, r = (cm >> 3) * 8 + (lane >> 2), k = (cm & 7) * 4 + (lane & 3);
    const int row = ar0 + r;
    R.a[i] = (row < ar_end && row >= ar_skip && c0 + k < c_end) ? A[(long long)row * nb + c0 + k] : 0.f;
  }
#pragma unroll
  for (int i = 0; i < 8; i++) {  // B: core matrices w*8 + i
    const int cm = w * 8 + i, r = (cm >> 3) * 8 + (lane >> 2), k = (cm & 7) * 4 + (lane & 3);
    const int row = br0 + r;
    float x = 0.f;
    if (row < br_end) {
      if (Msm)
        x = Msm[r * S + mcol0 + k];
      else if (c0 + k < c_end)
        x = bt ? Bsrc[(long long)(c0 + k) * nb + row] : Bsrc[(long long)row * nb + c0 + k];
    }
    R.b[i] = x;
  }
}

// Core matrix cm of a chunk occupies words [32 cm, 32 cm + 32) in the canonical layout.
__device__ __forceinline__ void tc_store(const TcStage& st, const TcRegs& R) {
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
#pragma unroll
  for (int i = 0; i < 16; i++) {
    float h, l;
    tc_split(R.a[i], h, l);
    st.ahi[(w * 16 + i) * 32 + lane] = h;
    st.alo[(w * 16 + i) * 32 + lane] = l;
  }
#pragma unroll
  for (int i = 0; i < 8; i++) {
    float h, l;
    tc_split(R.b[i], h, l);
    st.bhi[(w * 8 + i) * 32 + lane] = h;
    st.blo[(w * 8 + i) * 32 + lane] = l;
  }
}

size_t chol_tc_smem() {
  return sizeof(float) * (2 * 128 * TC_KCH + 2 * 64 * TC_KCH + 2 * TB * SP<float>::S) + 64;
}

// The MMA pipeline of one 128 x 64 product: D (TMEM) = sum over the columns [k0, k1) of
// Asrc rows [ar0, ar0 + 128) (valid in [ar_skip, ar_end)) times B^T, B the rows [br0,
// br_end) of Bsrc (of its transpose with bt) or, with Msm, the rows of M in shared memory at
// column c - k0. Chunks of 32 columns; the next chunk's loads are in flight while the tensor
// cores work. Returns false (error flagged, s_abort set) if an MMA commit is not seen in time.
__device__ bool tc_gemm(const TcStage& st, uint32_t tmem, uint64_t* bar, unsigned& phase, int* s_abort,
                        unsigned* err, const float* Asrc, int ld, int ar0, int ar_skip, int ar_end, const float* Bsrc,
                        int br0, int br_end, const float* Msm, int k0, int k1, bool bt = false) {
  TcRegs R;
  tc_fetch(R, Asrc, ld, ar0, ar_skip, ar_end, k0, k1, br0, br_end, Msm, 0, Bsrc, bt);
  for (int c0 = k0; c0 < k1; c0 += TC_KCH) {
    tc_store(st, R);
    tc_sync();
    if (threadIdx.x == 0) tc_issue(tmem, st, c0 == k0);
    if (c0 + TC_KCH < k1)
      tc_fetch(R, Asrc, ld, ar0, ar_skip, ar_end, c0 + TC_KCH, k1, br0, br_end, Msm, c0 + TC_KCH - k0, Bsrc, bt);
    if (!tc_commit_wait(bar, phase)) {
      if (threadIdx.x == 0) {
        atomicOr(err, DEV_ERR_TIMEOUT);
        *s_abort = 1;
      }
    }
    __syncthreads();
    if (*s_abort) return false;
  }
  return true;
}

// The 128 x 64 result in TMEM through shared memory (Et, over the idle operand stage) into
// dst rows [r0, r0 + 128) below r_end, columns [c0, c0 + h): dst -= D (sub) or dst = D.
__device__ void tc_epi(uint32_t tmem, float* Et, float* dst, long long ld, int r0, int r_end, int c0, int h, bool sub) {
  constexpr int kEtS = TB + 1;
  const int tid = threadIdx.x, w = tid >> 5;
  {
    float v[32];
    tc_load32(tmem, v);
    const int r_own = 32 * (w & 3) + (tid & 31), cbase = 32 * (w >> 2);
#pragma unroll
    for (int j = 0; j < 32; j++) Et[r_own * kEtS + cbase + j] = v[j];
  }
  __syncthreads();
  constexpr int kRmw = 8;
  for (int e0 = 0; e0 < 128 * TB; e0 += kRmw * NTH) {
    float a[kRmw];
#pragma unroll
    for (int g = 0; g < kRmw; g++) {
      const int e = e0 + g * NTH + tid, rr = e / TB, col = e % TB, row = r0 + rr;
      a[g] = (sub && row < r_end && col < h) ? dst[(long long)row * ld + c0 + col] : 0.f;
    }
#pragma unroll
    for (int g = 0; g < kRmw; g++) {
      const int e = e0 + g * NTH + tid, rr = e / TB, col = e % TB, row = r0 + rr;
      if (row < r_end && col < h) dst[(long long)row * ld + c0 + col] = sub ? a[g] - Et[rr * kEtS + col] : Et[rr * kEtS + col];
    }
  }
  __syncthreads();
}

__global__ void __launch_bounds__(NTH, 2) k_chol_tc(int nblk, const int* __restrict__ blk_cell,
                                                     const long long* __restrict__ boff, const int* __restrict__ cs,
                                                     const long long* __restrict__ koff, float* __restrict__ K,
                                                     const long long* __restrict__ xoff, float* __restrict__ Xw,
                                                     unsigned char* __restrict__ bad,
                                                     const unsigned char* __restrict__ only, int mode,
                                                     const long long* __restrict__ soff, float* __restrict__ Sout,
                                                     double out_scale_all, const double* __restrict__ cell_sig,
                                                     unsigned* __restrict__ err) {
  const int b = blockIdx.x;
  if (b >= nblk || (only && !only[b])) return;
  constexpr int S = SP<float>::S;
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  float* base = (float*)smem_raw;
  TcStage st;
  st.ahi = base;
  st.alo = st.ahi + 128 * TC_KCH;
  st.bhi = st.alo + 128 * TC_KCH;
  st.blo = st.bhi + 64 * TC_KCH;
  float* Ct = st.blo + 64 * TC_KCH;  // [TB][S] diagonal tile
  float* Mt = Ct + TB * S;           // [TB][S] its inverse
  // epilogue staging of a 128 x 64 result, over the operand stage (48 KB >= 128 x 65 floats)
  constexpr int kEtS = TB + 1;
  static_assert(128 * kEtS <= 2 * 128 * TC_KCH + 2 * 64 * TC_KCH, "epilogue staging fits the operand stage");
  float* Et = base;
  __shared__ __align__(8) uint64_t bar;
  __shared__ uint32_t tmem_base;
  __shared__ int s_abort;
  const int tid = threadIdx.x, w = tid >> 5;

  const int c = blk_cell[b];
  const int nb = (int)(boff[c + 1] - boff[c]);
  const int nc = cs[c + 1] - cs[c], n1 = mode == 1 ? nb : nb - nc;
  const int kc1 = (n1 + TB - 1) / TB;
  const int ntile = kc1 + (mode == 1 ? 0 : (nc + TB - 1) / TB);
  const int nct = ntile - kc1;
  float* A = K + koff[b];
  float* Minv_all = Xw + xoff[b];  // mode 0: the diagonal tiles' inverses, TB x TB each
  (void)nct;

  if (tid == 0) {
    mbar_init(&bar, 1);
    s_abort = 0;
  }
  if (w == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(tc_smem(&tmem_base)),
                 "r"(64));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  tc_sync();
  const uint32_t tmem = tmem_base;
  unsigned phase = 0;
  bool ok = true;
  const int r_own = 32 * (w & 3) + (tid & 31), cbase = 32 * (w >> 2);  // TMEM row / column half

  for (int k = 0; k < ntile && !s_abort; k++) {
    int rk, hk;
    tile_range(k, n1, nb, kc1, rk, hk);
    for (int pr = rk; pr < nb && !s_abort; pr += 128) {
      // ---- update: C = A[pr.., rk..] - sum over columns [0, rk) (rows pr .. pr + 127)
      if (rk > 0) {
        // next chunk's loads in flight while the tensor cores work on this one
        TcRegs R;
        tc_fetch(R, A, nb, pr, pr, nb, 0, rk, rk, rk + hk, nullptr, 0);
        for (int c0 = 0; c0 < rk; c0 += TC_KCH) {
          tc_store(st, R);
          tc_sync();
          if (tid == 0) tc_issue(tmem, st, c0 == 0);
          if (c0 + TC_KCH < rk) tc_fetch(R, A, nb, pr, pr, nb, c0 + TC_KCH, rk, rk, rk + hk, nullptr, 0);
          if (!tc_commit_wait(&bar, phase)) {
            if (tid == 0) {
              atomicOr(err, DEV_ERR_TIMEOUT);
              s_abort = 1;
            }
          }
          __syncthreads();
          if (s_abort) break;
        }
        if (s_abort) break;
        // the 128 x 64 update goes through shared memory (the operand stage, idle once the
        // MMAs have committed), so the read-modify-write of the block is row-coalesced
        {
          float v[32];
          tc_load32(tmem, v);
#pragma unroll
          for (int j = 0; j < 32; j++) Et[r_own * kEtS + cbase + j] = v[j];
        }
        __syncthreads();
        // the diagonal tile keeps its lower part; rows below take the whole tile width. A
        // thread's eight loads of the block are all issued before its first store (one
        // load latency per eight entries instead of one per entry)
        constexpr int kRmw = 8;
        static_assert((128 * TB) % (kRmw * NTH) == 0, "whole groups");
        for (int e0 = 0; e0 < 128 * TB; e0 += kRmw * NTH) {
          float a[kRmw];
#pragma unroll
          for (int g = 0; g < kRmw; g++) {
            const int e = e0 + g * NTH + tid, rr = e / TB, col = e % TB, row = pr + rr;
            const bool in = row < nb && col < hk && (row >= rk + hk || col <= row - rk);
            a[g] = in ? A[(long long)row * nb + rk + col] : 0.f;
          }
#pragma unroll
          for (int g = 0; g < kRmw; g++) {
            const int e = e0 + g * NTH + tid, rr = e / TB, col = e % TB, row = pr + rr;
            if (row < nb && col < hk && (row >= rk + hk || col <= row - rk))
              A[(long long)row * nb + rk + col] = a[g] - Et[rr * kEtS + col];
          }
        }
        __syncthreads();
      }
      // ---- the diagonal tile (first panel of the column): factor and invert it
      if (pr == rk) {
        for (int e = tid; e < TB * TB; e += NTH) {
          const int r = e / TB, cc = e % TB;
          Ct[r * S + cc] = (r < hk && cc <= r) ? A[(long long)(rk + r) * nb + rk + cc] : 0.f;
        }
        __syncthreads();
        ok = potrf_trtri_w(Ct, Mt, hk) && ok;
        for (int e = tid; e < TB * TB; e += NTH) {
          const int r = e / TB, cc = e % TB;
          if (r < hk && cc <= r) A[(long long)(rk + r) * nb + rk + cc] = Ct[r * S + cc];
          if (mode == 0) Minv_all[(long long)k * TB * TB + e] = Mt[r * S + cc];
        }
        __syncthreads();
      }
      // ---- panel solve of the rows below the diagonal tile: L = C M^T (M = L_kk^-1)
      if (pr + 128 > rk + hk && rk + hk < nb) {
        TcRegs R;
        for (int c0 = 0; c0 < TB; c0 += TC_KCH) {
          tc_fetch(R, A, nb, pr, rk + hk, nb, rk + c0, rk + hk, 0, hk, Mt, c0);
          tc_store(st, R);
          tc_sync();
          if (tid == 0) tc_issue(tmem, st, c0 == 0);
          if (!tc_commit_wait(&bar, phase)) {
            if (tid == 0) {
              atomicOr(err, DEV_ERR_TIMEOUT);
              s_abort = 1;
            }
          }
          __syncthreads();
          if (s_abort) break;
        }
        if (s_abort) break;
        {
          float v[32];
          tc_load32(tmem, v);
#pragma unroll
          for (int j = 0; j < 32; j++) Et[r_own * kEtS + cbase + j] = v[j];
        }
        __syncthreads();  // every thread has read its C row and staged its result
        for (int e = tid; e < 128 * TB; e += NTH) {
          const int rr = e / TB, col = e % TB, row = pr + rr;
          if (row < nb && row >= rk + hk && col < hk) A[(long long)row * nb + rk + col] = Et[rr * kEtS + col];
        }
        __syncthreads();
      }
    }
  }

  // ---- S_c = 2 pi sigma^2 X^T, X the centre columns of K^-1 (mode 0) --------------------
  // Z = X^T (n_c x n_b, row-major, written in place at S_c) solves Z L L^T = E_c^T, E_c the
  // centre columns of the identity. Forward, over the centre tiles I only (Z is zero left
  // of them): Z_I = (E_I^T - Z[:, n1..r_I) L_I,[n1..r_I)^T) M_II^T. Back, over all tiles
  // from the last: Z_J = (Z_J - Z[:, r_J + h_J..) (L^T)_J,[r_J + h_J..)^T) M_JJ with the rows
  // of L^T read as columns of L (transposed fetch). Every product is a 128-row panel of Z (128
  // centre points per pass) times 64 rows of L, L^T or M on the tensor cores, the same MMA pipeline
  // as the factorisation. The centre columns are scaled once they are final; the neighbour
  // columns, linear in them, then come out scaled.
  if (mode == 0 && ok && !s_abort) {
    float* Z = Sout + soff[c];
    const float zscale = (float)(cell_sig ? 2.0 * M_PI * cell_sig[c] * cell_sig[c] : out_scale_all);
    for (int n = w; n < nc; n += NTH / 32) {  // a warp per row of Z
      float* zr = Z + (long long)n * nb;
      for (int j = tid & 31; j < nb; j += 32) zr[j] = j == n1 + n ? 1.f : 0.f;
    }
    __syncthreads();
    for (int pr = 0; pr < nc && !s_abort; pr += 128) {
      for (int I = kc1; I < ntile && !s_abort; I++) {  // forward
        int rI, hI;
        tile_range(I, n1, nb, kc1, rI, hI);
        if (rI > n1) {
          if (!tc_gemm(st, tmem, &bar, phase, &s_abort, err, Z, nb, pr, pr, nc, A, rI, rI + hI, nullptr, n1, rI))
            break;
          tc_epi(tmem, Et, Z, nb, pr, nc, rI, hI, true);
        }
        for (int e = tid; e < TB * TB; e += NTH) Mt[(e / TB) * S + e % TB] = Minv_all[(long long)I * TB * TB + e];
        __syncthreads();
        if (!tc_gemm(st, tmem, &bar, phase, &s_abort, err, Z, nb, pr, pr, nc, nullptr, 0, hI, Mt, rI, rI + hI)) break;
        tc_epi(tmem, Et, Z, nb, pr, nc, rI, hI, false);
      }
      for (int J = ntile - 1; J >= 0 && !s_abort; J--) {  // back
        int rJ, hJ;
        tile_range(J, n1, nb, kc1, rJ, hJ);
        if (J == kc1 - 1) {  // the centre columns are final: scale them
          for (int n = pr + w; n < min(pr + 128, nc); n += NTH / 32)
            for (int j = n1 + (tid & 31); j < nb; j += 32) Z[(long long)n * nb + j] *= zscale;
          __syncthreads();
        }
        if (rJ + hJ < nb) {
          if (!tc_gemm(st, tmem, &bar, phase, &s_abort, err, Z, nb, pr, pr, nc, A, rJ, rJ + hJ, nullptr, rJ + hJ, nb,
                       true))
            break;
          tc_epi(tmem, Et, Z, nb, pr, nc, rJ, hJ, true);
        }
        for (int e = tid; e < TB * TB; e += NTH)  // M_JJ^T
          Mt[(e % TB) * S + e / TB] = Minv_all[(long long)J * TB * TB + e];
        __syncthreads();
        if (!tc_gemm(st, tmem, &bar, phase, &s_abort, err, Z, nb, pr, pr, nc, nullptr, 0, hJ, Mt, rJ, rJ + hJ)) break;
        tc_epi(tmem, Et, Z, nb, pr, nc, rJ, hJ, false);
      }
      if (kc1 == 0 && !s_abort) {  // no neighbour tiles: the centre columns are all of Z
        for (int n = pr + w; n < min(pr + 128, nc); n += NTH / 32)
          for (int j = n1 + (tid & 31); j < nb; j += 32) Z[(long long)n * nb + j] *= zscale;
        __syncthreads();
      }
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (w == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(64));
  if (tid == 0) bad[b] = (ok && !s_abort) ? 0 : 1;
}

// After k_chol_tc (factor form): each block's L packed by rows as the substitutions read
// it -- row i holds L_A[i][0..i-1], then 1 / L_A[i][i] (the substitutions multiply), L_A =
// L_K sqrt(1 / (2 pi sigma^2)) the factor of A = K / (2 pi sigma^2). One CTA per block, a
// warp per row.
__global__ void __launch_bounds__(NTH) k_pack_factor(int nblk, const int* __restrict__ blk_cell,
                                                    const long long* __restrict__ boff,
                                                    const long long* __restrict__ koff, const float* __restrict__ K,
                                                    double scale_all, const double* __restrict__ cell_sig,
                                                    const unsigned char* __restrict__ only,
                                                    const long long* __restrict__ loff, float* __restrict__ Lpack) {
  const int b = blockIdx.x;
  if (b >= nblk || (only && !only[b])) return;
  const int c = blk_cell[b];
  const int nb = (int)(boff[c + 1] - boff[c]);
  // per-block scale (batches of problems with their own sigma)
  const float sc = (float)(cell_sig ? sqrt(1.0 / (2.0 * M_PI * cell_sig[c] * cell_sig[c])) : scale_all);
  const float* A = K + koff[b];
  float* Lp = Lpack + loff[c];
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  for (int i = w; i < nb; i += NTH / 32) {
    const long long o = rowoff<float>(i);
    for (int j = lane; j <= i; j += 32) {
      const float v = A[(long long)i * nb + j] * sc;
      Lp[o + j] = j == i ? 1.f / v : v;
    }
  }
}

// ---- plain FP64 factor form: ordered block Cholesky -----------------------------------
// One CTA per block: left-looking Cholesky of K over uniform 64 x 64 tiles. A tile starts
// from K, receives the trailing updates of the earlier tile columns in ascending column
// order (tile_update accumulates into the tile itself), and is then finished by potrf_rd
// (diagonal tile) or trsm_rows (tiles below it). Every entry of L thus sees exactly the
// operation sequence of the unblocked right-looking Cholesky written with fma, sqrt and
// reciprocal pivots -- a CPU restatement of that loop reproduces the factor bit for bit.
// The factor is then packed as the apply reads it: row i holds L_A[i][0..i-1] and
// 1 / L_A[i][i], L_A = L_K sqrt(1 / (2 pi sigma^2)) the factor of A = K / (2 pi sigma^2).
__global__ void __launch_bounds__(NTH, 2) k_chol_fp64(int nblk, const int* __restrict__ blk_cell,
                                                   const long long* __restrict__ boff,
                                                   const long long* __restrict__ koff, double* __restrict__ K,
                                                   double out_scale_all, const double* __restrict__ cell_sig,
                                                   unsigned char* __restrict__ bad,
                                                   const unsigned char* __restrict__ only,
                                                   const long long* __restrict__ loff, double* __restrict__ Lpack) {
  using T = double;
  const int b = blockIdx.x;
  if (b >= nblk || (only && !only[b])) return;
  double out_scale = out_scale_all;  // sqrt(1 / (2 pi sigma^2)), per cell for a batch
  if (cell_sig) {
    const double sg = cell_sig[blk_cell[b]];
    out_scale = sqrt(1.0 / (2.0 * M_PI * sg * sg));
  }
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ T s_rd[TB];
  constexpr int S = SP<T>::S;
  constexpr int KC = KCOf<T>::v;
  Tiles<T> t;
  t.As = (T*)smem_raw;
  t.Bs = t.As + 2 * KC * S;
  t.C = t.Bs + 2 * KC * S;
  t.M = t.C + TB * S;
  const int c = blk_cell[b];
  const int nb = (int)(boff[c + 1] - boff[c]);
  const int ntile = (nb + TB - 1) / TB;
  T* A = K + koff[b];
  bool ok = true;
  for (int k = 0; k < ntile; k++) {
    const int rk = k * TB, hk = min(TB, nb - rk);
    for (int i = k; i < ntile; i++) {
      const int ri = i * TB, hi = min(TB, nb - ri);
      const TileMap mp = tile_map(i == k);  // a diagonal tile: its lower blocks only
      T acc[4][4];
      load_acc<T>(A, nb, ri, rk, hi, hk, acc, true, mp);
      for (int p = 0; p < k; p++) {
        const int rp = p * TB, hp = min(TB, nb - rp);
        tile_update<T>(t, acc, A, nb, ri, rp, hi, false, A, nb, rk, rp, hk, false, hp, mp);
      }
      __syncthreads();
      acc_to_smem<T>(t.C, acc, mp);  // potrf_rd zeroes the upper part it does not write
      __syncthreads();
      if (i == k) {
        ok = potrf_rd<T>(t.C, s_rd, hk) && ok;
        // store L_kk and keep it in M for the panel solves of this tile column
        for (int e = threadIdx.x; e < TB * TB; e += NTH) {
          const int r = e / TB, cc = e % TB;
          const T v = t.C[r * S + cc];
          if (r < hk && cc <= r) A[(long long)(rk + r) * nb + rk + cc] = v;
          t.M[r * S + cc] = v;
        }
      } else {
        trsm_rows<T>(t.C, t.M, s_rd, hi, hk);
        __syncthreads();
        for (int e = threadIdx.x; e < TB * TB; e += NTH) {
          const int r = e / TB, cc = e % TB;
          if (r < hi && cc < hk) A[(long long)(ri + r) * nb + rk + cc] = t.C[r * S + cc];
        }
      }
      __syncthreads();
    }
  }
  T* Lp = Lpack + loff[c];
  const T sc = (T)out_scale;
  for (int i = 0; i < nb; i++) {
    const long long o = rowoff<T>(i);
    for (int j = threadIdx.x; j <= i; j += NTH) {
      const T v = A[(long long)i * nb + j] * sc;
      Lp[o + j] = j == i ? T(1) / v : v;
    }
  }
  if (threadIdx.x == 0) bad[b] = ok ? 0 : 1;
}

// ---- apply: out[centre(c)] = S_c r[buffer(c) in block order] --------------------------
template <class T>
__global__ void __launch_bounds__(128) k_apply(int ncell, const long long* __restrict__ boff,
                                               const int* __restrict__ cs, const int* __restrict__ idx,
                                               const long long* __restrict__ soff, const T* __restrict__ S,
                                               const double* __restrict__ r, double* __restrict__ out,
                                               const int* __restrict__ skip) {
  if (skip && *skip) return;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* rv = (T*)smem_raw;
  int c = blockIdx.x;
  int nb = (int)(boff[c + 1] - boff[c]);
  if (nb == 0) return;
  int nc = cs[c + 1] - cs[c], n1 = nb - nc;
  const int* id = idx + boff[c];
  for (int j = threadIdx.x; j < nb; j += blockDim.x) rv[j] = (T)r[id[j < n1 ? nc + j : j - n1]];
  __syncthreads();
  const T* Sc = S + soff[c];
  int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
  for (int row = w; row < nc; row += nw) {
    const T* sr = Sc + (long long)row * nb;
    T s = T(0);
    for (int j = lane; j < nb; j += 32) s = fma(sr[j], rv[j], s);
    s = warp_sum(s);
    if (lane == 0) out[cs[c] + row] = (double)s;
  }
}

// ---- apply with the factor: out[centre(c)] = (L^-T L^-1 r_c)[centre] ----------------
// Forward substitution over the whole block (32-row panels: warp 0 solves the diagonal
// triangle from shared memory, all warps update the rows below with coalesced row
// segments), then the back substitution with L22^T only, since the centre unknowns are
// the last n_c: x2 = L22^-T y2. With full set (basic Schwarz) the back substitution runs
// over the whole block and the whole solution goes to the block's slots of Y (slot =
// position in the buffer list); k_asm_gather then sums each point's slots in block order,
// so the result does not depend on the order the blocks ran in. NV right-hand sides
// (vectors at stride vs, slots at stride ys) share every load of the factor.
template <class T, int NV>
__global__ void __launch_bounds__(256) k_apply_tri(int ncell, const long long* __restrict__ boff,
                                                   const int* __restrict__ cs, const int* __restrict__ idx,
                                                   const long long* __restrict__ loff, const T* __restrict__ Lpack,
                                                   const double* __restrict__ r, double* __restrict__ out,
                                                   long long vs, const int* __restrict__ skip, int full,
                                                   double* __restrict__ Y, long long ys, SegSkip seg,
                                                   const int* __restrict__ lu_of_cell) {
  if (skip && *skip) return;
  if (seg.cell_done(blockIdx.x)) return;
  if (lu_of_cell && lu_of_cell[blockIdx.x] >= 0) return;  // factored by LU: k_apply_lu
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ T tri[32][33];
  const int c = blockIdx.x;
  const int nb = (int)(boff[c + 1] - boff[c]);
  if (nb == 0) return;
  T* y = (T*)smem_raw;  // NV x nb
  const int nc = cs[c + 1] - cs[c], n1 = nb - nc;
  const int* id = idx + boff[c];
  const T* L = Lpack + loff[c];
  const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5, nw = blockDim.x >> 5;
  for (int j = tid; j < nb; j += blockDim.x) {
    const int p = id[j < n1 ? nc + j : j - n1];
#pragma unroll
    for (int v = 0; v < NV; v++) y[v * nb + j] = (T)r[v * vs + p];
  }
  __syncthreads();
  // forward: L y = r
  for (int p0 = 0; p0 < nb; p0 += 32) {
    const int np = min(32, nb - p0);
    for (int e = tid; e < 32 * 32; e += blockDim.x) {
      int i = e >> 5, j = e & 31;
      tri[i][j] = (i < np && j <= i) ? L[rowoff<T>(p0 + i) + p0 + j] : T(0);
    }
    __syncthreads();
    if (w == 0) {
      T ri[NV];
#pragma unroll
      for (int v = 0; v < NV; v++) ri[v] = lane < np ? y[v * nb + p0 + lane] : T(0);
      for (int j = 0; j < np; j++) {
        const T d = tri[j][j], l = tri[lane][j];
#pragma unroll
        for (int v = 0; v < NV; v++) {
          if (lane == j) ri[v] = ri[v] * d;  // reciprocal diagonal
          T yj = __shfl_sync(0xffffffffu, ri[v], j);
          if (lane > j) ri[v] = fma(-l, yj, ri[v]);
        }
      }
      if (lane < np)
#pragma unroll
        for (int v = 0; v < NV; v++) y[v * nb + p0 + lane] = ri[v];
    }
    __syncthreads();
    // rows below the panel: y[i] -= L[i][p0 .. p0+np) . y[p0 ..]. Four lanes per row, each
    // with 8 contiguous entries, so 8 rows per warp pass and 2 shuffle levels: on GB300's
    // narrow FP64 pipe a full warp reduction per row would cost 5x the row's FMAs.
    {
      const int sub = lane & 3, rw = lane >> 2;
      T ysv[NV][8];
#pragma unroll
      for (int v = 0; v < NV; v++)
#pragma unroll
        for (int q = 0; q < 8; q++) ysv[v][q] = (sub * 8 + q < np) ? y[v * nb + p0 + sub * 8 + q] : T(0);
      for (int i0 = p0 + np + 8 * w; i0 < nb; i0 += 8 * nw) {
        const long long i = i0 + rw;
        T acc[NV];
#pragma unroll
        for (int v = 0; v < NV; v++) acc[v] = T(0);
        if (i < nb) {
          // rows below a panel only exist when the panel is full (np = 32): all 8 entries
          // of the segment lie inside row i, 16-byte aligned
          T lv[8];
          const T* Li = L + rowoff<T>(i) + p0 + sub * 8;
          if constexpr (sizeof(T) == 8) {
#pragma unroll
            for (int q = 0; q < 4; q++) {
              const double2 t2 = reinterpret_cast<const double2*>(Li)[q];
              lv[2 * q] = t2.x;
              lv[2 * q + 1] = t2.y;
            }
          } else {
#pragma unroll
            for (int q = 0; q < 2; q++) {
              const float4 t4 = reinterpret_cast<const float4*>(Li)[q];
              lv[4 * q] = t4.x;
              lv[4 * q + 1] = t4.y;
              lv[4 * q + 2] = t4.z;
              lv[4 * q + 3] = t4.w;
            }
          }
#pragma unroll
          for (int q = 0; q < 8; q++)
#pragma unroll
            for (int v = 0; v < NV; v++) acc[v] = fma(lv[q], ysv[v][q], acc[v]);
        }
#pragma unroll
        for (int v = 0; v < NV; v++) {
          acc[v] += __shfl_xor_sync(0xffffffffu, acc[v], 1);
          acc[v] += __shfl_xor_sync(0xffffffffu, acc[v], 2);
        }
        if (sub == 0 && i < nb)
#pragma unroll
          for (int v = 0; v < NV; v++) y[v * nb + i] -= acc[v];
      }
    }
    __syncthreads();
  }
  // backward on the trailing block (rows b0 ..): L22^T x2 = y2, panels from the bottom
  const int b0 = full ? 0 : n1, nback = nb - b0;
  for (int pe = nback; pe > 0; pe -= 32) {
    const int p0 = max(0, pe - 32), np = pe - p0;
    // tri[i][j] = L22[p0 + i][p0 + j], j <= i
    for (int e = tid; e < 32 * 32; e += blockDim.x) {
      int i = e >> 5, j = e & 31;
      long long row = b0 + p0 + i;
      tri[i][j] = (i < np && j <= i) ? L[rowoff<T>(row) + b0 + p0 + j] : T(0);
    }
    __syncthreads();
    if (w == 0) {  // x_i = (y_i - sum_{j > i} L22[j][i] x_j) / L22[i][i], i = np-1 .. 0
      T xi[NV];
#pragma unroll
      for (int v = 0; v < NV; v++) xi[v] = lane < np ? y[v * nb + b0 + p0 + lane] : T(0);
      for (int j = np - 1; j >= 0; j--) {
        const T d = tri[j][j], l = tri[j][lane];
#pragma unroll
        for (int v = 0; v < NV; v++) {
          if (lane == j) xi[v] = xi[v] * d;  // reciprocal diagonal
          T xj = __shfl_sync(0xffffffffu, xi[v], j);
          if (lane < j) xi[v] = fma(-l, xj, xi[v]);
        }
      }
      if (lane < np)
#pragma unroll
        for (int v = 0; v < NV; v++) y[v * nb + b0 + p0 + lane] = xi[v];
    }
    __syncthreads();
    // rows above the panel: y2[k] -= sum_{j in panel} L22[p0 + j][k] x_j, k < p0
    for (int k = tid; k < p0; k += blockDim.x) {
      T acc[NV];
#pragma unroll
      for (int v = 0; v < NV; v++) acc[v] = T(0);
      for (int j = 0; j < np; j++) {
        long long row = b0 + p0 + j;
        const T lv = L[rowoff<T>(row) + b0 + k];
#pragma unroll
        for (int v = 0; v < NV; v++) acc[v] = fma(lv, y[v * nb + b0 + p0 + j], acc[v]);
      }
#pragma unroll
      for (int v = 0; v < NV; v++) y[v * nb + b0 + k] -= acc[v];
    }
    __syncthreads();
  }
  if (full) {
    double* Yc = Y + boff[c];
    for (int j = tid; j < nb; j += blockDim.x)
#pragma unroll
      for (int v = 0; v < NV; v++) Yc[v * ys + (j < n1 ? nc + j : j - n1)] = (double)y[v * nb + j];
  } else {
    for (int i = tid; i < nc; i += blockDim.x)
#pragma unroll
      for (int v = 0; v < NV; v++) out[v * vs + cs[c] + i] = (double)y[v * nb + n1 + i];
  }
}

// ---- FP32 apply with the factor, one warp per block -----------------------------------
// The FP32 substitutions stream the packed factor twice and are bound by HBM, so no warp
// of them may wait on another: each warp solves a whole block with its own y in shared
// memory (no CTA barrier). Forward, 32-row panels from the top: lane i holds row p0+i of
// the panel triangle in registers (its own 16-byte-aligned row segment), the panel's y is
// solved by shuffles, and the rows below are updated four lanes per row, eight entries
// each, four rows per lane in flight. Backward (L^T x = y over the whole block for basic
// Schwarz, over the centre rows for the restricted form), 32-row panels aligned to
// multiples of 32 from the bottom: lane i holds column P0+i of the panel triangle, and
// the rows above are updated from the panel rows' contiguous segments L[P0+j][k], each
// lane owning four consecutive k and keeping eight 16-byte loads in flight. Every access
// stays inside the row it addresses: a segment starting at a multiple of 4 at or below
// the row index lies inside the row's padded extent.
constexpr int kTrwWarps = 4;

template <int NV>
__global__ void __launch_bounds__(kTrwWarps * 32) k_apply_trw(int ncell, const long long* __restrict__ boff,
                                                             const int* __restrict__ cs, const int* __restrict__ idx,
                                                             const long long* __restrict__ loff,
                                                             const float* __restrict__ Lpack,
                                                             const double* __restrict__ r, double* __restrict__ out,
                                                             long long vs, const int* __restrict__ skip, int full,
                                                             double* __restrict__ Y, long long ys, SegSkip seg,
                                                             int ldy) {
  if (skip && *skip) return;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int c = blockIdx.x * kTrwWarps + wid;
  if (c >= ncell || seg.cell_done(c)) return;
  const int nb = (int)(boff[c + 1] - boff[c]);
  if (nb == 0) return;
  float* y = (float*)smem_raw + (size_t)wid * NV * ldy;  // NV x ldy
  const int nc = cs[c + 1] - cs[c], n1 = nb - nc;
  const int* id = idx + boff[c];
  const float* L = Lpack + loff[c];
  constexpr unsigned FULL = 0xffffffffu;
  for (int j = lane; j < nb; j += 32) {
    const int p = id[j < n1 ? nc + j : j - n1];
#pragma unroll
    for (int v = 0; v < NV; v++) y[v * ldy + j] = (float)r[v * vs + p];
  }
  __syncwarp();
  // ---- forward: L y = r ----
  const int sub = lane & 3, rw = lane >> 2;
  for (int p0 = 0; p0 < nb; p0 += 32) {
    const int np = min(32, nb - p0);
    const bool act = lane < np;
    float lrow[32];
    {
      const float4* Li = reinterpret_cast<const float4*>(L + rowoff<float>(p0 + lane) + p0);
#pragma unroll
      for (int q = 0; q < 8; q++) {
        float4 t = make_float4(0.f, 0.f, 0.f, 0.f);
        if (act && 4 * q <= lane) t = Li[q];
        lrow[4 * q] = t.x;
        lrow[4 * q + 1] = t.y;
        lrow[4 * q + 2] = t.z;
        lrow[4 * q + 3] = t.w;
      }
    }
    float ri[NV];
#pragma unroll
    for (int v = 0; v < NV; v++) ri[v] = act ? y[v * ldy + p0 + lane] : 0.f;
#pragma unroll
    for (int j = 0; j < 32; j++) {
      if (j < np) {
#pragma unroll
        for (int v = 0; v < NV; v++) {
          if (lane == j) ri[v] *= lrow[j];  // reciprocal diagonal
          const float yj = __shfl_sync(FULL, ri[v], j);
          if (lane > j) ri[v] = fmaf(-lrow[j], yj, ri[v]);
        }
      }
    }
    if (act)
#pragma unroll
      for (int v = 0; v < NV; v++) y[v * ldy + p0 + lane] = ri[v];
    // rows below the panel (only when it is full): y[i] -= L[i][p0 .. p0+32) . y[p0 ..]
    if (p0 + 32 < nb) {
      float ysv[NV][8];
#pragma unroll
      for (int v = 0; v < NV; v++)
#pragma unroll
        for (int q = 0; q < 8; q++) ysv[v][q] = __shfl_sync(FULL, ri[v], sub * 8 + q);
      for (int i0 = p0 + 32; i0 < nb; i0 += 32) {
        float4 lv[4][2];
#pragma unroll
        for (int u = 0; u < 4; u++) {
          const int i = i0 + 8 * u + rw;
          if (i < nb) {
            const float4* Li = reinterpret_cast<const float4*>(L + rowoff<float>(i) + p0 + sub * 8);
            lv[u][0] = Li[0];
            lv[u][1] = Li[1];
          } else {
            lv[u][0] = lv[u][1] = make_float4(0.f, 0.f, 0.f, 0.f);
          }
        }
#pragma unroll
        for (int u = 0; u < 4; u++) {
          const int i = i0 + 8 * u + rw;
          float acc[NV];
#pragma unroll
          for (int v = 0; v < NV; v++) {
            float a = lv[u][0].x * ysv[v][0];
            a = fmaf(lv[u][0].y, ysv[v][1], a);
            a = fmaf(lv[u][0].z, ysv[v][2], a);
            a = fmaf(lv[u][0].w, ysv[v][3], a);
            a = fmaf(lv[u][1].x, ysv[v][4], a);
            a = fmaf(lv[u][1].y, ysv[v][5], a);
            a = fmaf(lv[u][1].z, ysv[v][6], a);
            a = fmaf(lv[u][1].w, ysv[v][7], a);
            a += __shfl_xor_sync(FULL, a, 1);
            a += __shfl_xor_sync(FULL, a, 2);
            acc[v] = a;
          }
          if (sub == 0 && i < nb)
#pragma unroll
            for (int v = 0; v < NV; v++) y[v * ldy + i] -= acc[v];
        }
      }
    }
    __syncwarp();
  }
  // ---- backward: L22^T x2 = y2 over rows [b0, nb) ----
  const int b0 = full ? 0 : n1;
  for (int pt = (nb - 1) & ~31; pt >= 0 && pt + 32 > b0; pt -= 32) {
    const int P0 = max(pt, b0), np = min(nb, pt + 32) - P0;
    float lcol[32];
#pragma unroll
    for (int j = 0; j < 32; j++) lcol[j] = (j < np && lane <= j) ? L[rowoff<float>(P0 + j) + P0 + lane] : 0.f;
    float xi[NV];
#pragma unroll
    for (int v = 0; v < NV; v++) xi[v] = lane < np ? y[v * ldy + P0 + lane] : 0.f;
#pragma unroll
    for (int j = 31; j >= 0; j--) {
      if (j < np) {
#pragma unroll
        for (int v = 0; v < NV; v++) {
          if (lane == j) xi[v] *= lcol[j];
          const float xj = __shfl_sync(FULL, xi[v], j);
          if (lane < j) xi[v] = fmaf(-lcol[j], xj, xi[v]);
        }
      }
    }
    if (lane < np)
#pragma unroll
      for (int v = 0; v < NV; v++) y[v * ldy + P0 + lane] = xi[v];
    __syncwarp();
    // rows above the panel: y2[k] -= sum_j L[P0+j][k] x_j, b0 <= k < P0 (k4 starts at b0
    // rounded down to 4; the entries outside [b0, P0) are read but not applied)
    for (int k4 = (b0 & ~3) + 4 * lane; k4 < P0; k4 += 128) {
      float acc[NV][4];
#pragma unroll
      for (int v = 0; v < NV; v++) acc[v][0] = acc[v][1] = acc[v][2] = acc[v][3] = 0.f;
      for (int j0 = 0; j0 < np; j0 += 8) {
        float4 lv[8];
#pragma unroll
        for (int u = 0; u < 8; u++)
          lv[u] = j0 + u < np ? *reinterpret_cast<const float4*>(L + rowoff<float>(P0 + j0 + u) + k4)
                              : make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
        for (int u = 0; u < 8; u++) {
          if (j0 + u < np) {
#pragma unroll
            for (int v = 0; v < NV; v++) {
              const float xj = y[v * ldy + P0 + j0 + u];
              acc[v][0] = fmaf(lv[u].x, xj, acc[v][0]);
              acc[v][1] = fmaf(lv[u].y, xj, acc[v][1]);
              acc[v][2] = fmaf(lv[u].z, xj, acc[v][2]);
              acc[v][3] = fmaf(lv[u].w, xj, acc[v][3]);
            }
          }
        }
      }
#pragma unroll
      for (int v = 0; v < NV; v++)
#pragma unroll
        for (int e = 0; e < 4; e++)
          if (k4 + e >= b0 && k4 + e < P0) y[v * ldy + k4 + e] -= acc[v][e];
    }
    __syncwarp();
  }
  if (full) {
    double* Yc = Y + boff[c];
    for (int j = lane; j < nb; j += 32)
#pragma unroll
      for (int v = 0; v < NV; v++) Yc[v * ys + (j < n1 ? nc + j : j - n1)] = (double)y[v * ldy + j];
  } else {
    for (int i = lane; i < nc; i += 32)
#pragma unroll
      for (int v = 0; v < NV; v++) out[v * vs + cs[c] + i] = (double)y[v * ldy + n1 + i];
  }
}

// ---- LU fallback of the FP64 form (one CTA per block, in global memory) -------------
// For the few blocks whose ordered Cholesky meets a non-positive pivot: K (lower triangle
// as assembled) mirrored to a full matrix, then LU with partial pivoting -- pivot the first
// row of largest |a_ik| (a tree reduction that keeps the smaller row on ties), full rows
// swapped, l_ik = a_ik / a_kk, a_ij = fma(-l_ik, a_kj, a_ij) -- the entry-wise operations of
// the unblocked loop, so a CPU restatement of that loop reproduces the factor bit for bit.
// bad[b] = 1 on an exactly zero pivot (where PETSc's LU stops).
constexpr int kLuThreads = 256;

__global__ void __launch_bounds__(kLuThreads) k_lu_fp64(int nlu, const int* __restrict__ lucell,
                                                        const long long* __restrict__ boff,
                                                        const long long* __restrict__ koff, double* __restrict__ LU,
                                                        const long long* __restrict__ poff, int* __restrict__ piv,
                                                        unsigned char* __restrict__ bad) {
  const int b = blockIdx.x;
  if (b >= nlu) return;
  const int c = lucell[b];
  const int n = (int)(boff[c + 1] - boff[c]);
  double* A = LU + koff[b];
  int* pv = piv + poff[b];
  const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
  constexpr int NW = kLuThreads / 32;
  __shared__ double s_v[kLuThreads];
  __shared__ int s_i[kLuThreads];
  __shared__ int s_bad;
  for (int i = w; i < n; i += NW)
    for (int j = i + 1 + lane; j < n; j += 32) A[(long long)i * n + j] = A[(long long)j * n + i];
  if (tid == 0) s_bad = 0;
  __syncthreads();
  for (int k = 0; k < n; k++) {
    double bv = -1.0;
    int bi = n;
    for (int i = k + tid; i < n; i += kLuThreads) {
      const double v = fabs(A[(long long)i * n + k]);
      if (v > bv) {
        bv = v;
        bi = i;
      }
    }
    s_v[tid] = bv;
    s_i[tid] = bi;
    __syncthreads();
    for (int st = kLuThreads / 2; st > 0; st >>= 1) {
      if (tid < st) {
        const double ov = s_v[tid + st];
        const int oi = s_i[tid + st];
        if (ov > s_v[tid] || (ov == s_v[tid] && oi < s_i[tid])) {
          s_v[tid] = ov;
          s_i[tid] = oi;
        }
      }
      __syncthreads();
    }
    const int p = s_i[0];
    const bool zero = p >= n || s_v[0] == 0.0;
    if (tid == 0) {
      pv[k] = zero ? k : p;
      if (zero) s_bad = 1;
    }
    if (zero) break;  // uniform over the CTA
    if (p != k)
      for (int j = tid; j < n; j += kLuThreads) {
        const double t = A[(long long)k * n + j];
        A[(long long)k * n + j] = A[(long long)p * n + j];
        A[(long long)p * n + j] = t;
      }
    __syncthreads();
    const double d = A[(long long)k * n + k];
    for (int i = k + 1 + tid; i < n; i += kLuThreads) A[(long long)i * n + k] = __ddiv_rn(A[(long long)i * n + k], d);
    __syncthreads();
    for (int i = k + 1 + w; i < n; i += NW) {
      const double l = A[(long long)i * n + k];
      for (int j = k + 1 + lane; j < n; j += 32)
        A[(long long)i * n + j] = __fma_rn(-l, A[(long long)k * n + j], A[(long long)i * n + j]);
    }
    __syncthreads();
  }
  __syncthreads();
  if (tid == 0) bad[b] = (unsigned char)s_bad;
}

// The LU blocks' share of an apply: y <- 2 pi sigma^2 K^-1 y in the entry-wise order of the
// sequential solve (interchanges in order; forward, y_i receiving fma(-l_ik, y_k, .) for
// ascending k; backward, descending k with the division by the pivot when y_k is final),
// then the restricted (centre rows) or basic (all slots) output of k_apply_tri.
__global__ void __launch_bounds__(kLuThreads) k_apply_lu(int nlu, const int* __restrict__ lucell,
                                                         const long long* __restrict__ boff,
                                                         const int* __restrict__ cs, const int* __restrict__ idx,
                                                         const long long* __restrict__ koff,
                                                         const double* __restrict__ LU,
                                                         const long long* __restrict__ poff,
                                                         const int* __restrict__ piv, const double* __restrict__ r,
                                                         double* __restrict__ out, long long vs, int nv,
                                                         const int* __restrict__ skip, int full,
                                                         double* __restrict__ Y, long long ys, SegSkip seg,
                                                         double scale_all, const double* __restrict__ cell_sig) {
  if (skip && *skip) return;
  const int b = blockIdx.x;
  if (b >= nlu) return;
  const int c = lucell[b];
  if (seg.cell_done(c)) return;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int nb = (int)(boff[c + 1] - boff[c]);
  const int nc = cs[c + 1] - cs[c], n1 = nb - nc;
  const int* id = idx + boff[c];
  const double* A = LU + koff[b];
  const int* pv = piv + poff[b];
  double* y = (double*)smem_raw;  // nv x nb
  const int tid = threadIdx.x;
  for (int j = tid; j < nb; j += kLuThreads) {
    const int p = id[j < n1 ? nc + j : j - n1];
    for (int v = 0; v < nv; v++) y[v * nb + j] = r[v * vs + p];
  }
  __syncthreads();
  if (tid < nv)
    for (int k = 0; k < nb; k++) {
      const int p = pv[k];
      if (p != k) {
        const double t = y[tid * nb + k];
        y[tid * nb + k] = y[tid * nb + p];
        y[tid * nb + p] = t;
      }
    }
  __syncthreads();
  for (int k = 0; k < nb; k++) {
    for (int i = k + 1 + tid; i < nb; i += kLuThreads) {
      const double l = A[(long long)i * nb + k];
      for (int v = 0; v < nv; v++) y[v * nb + i] = __fma_rn(-l, y[v * nb + k], y[v * nb + i]);
    }
    __syncthreads();
  }
  for (int k = nb - 1; k >= 0; k--) {
    if (tid < nv) y[tid * nb + k] = __ddiv_rn(y[tid * nb + k], A[(long long)k * nb + k]);
    __syncthreads();
    for (int i = tid; i < k; i += kLuThreads) {
      const double u = A[(long long)i * nb + k];
      for (int v = 0; v < nv; v++) y[v * nb + i] = __fma_rn(-u, y[v * nb + k], y[v * nb + i]);
    }
    __syncthreads();
  }
  const double scale = cell_sig ? 2.0 * M_PI * cell_sig[c] * cell_sig[c] : scale_all;
  if (full) {
    double* Yc = Y + boff[c];
    for (int j = tid; j < nb; j += kLuThreads)
      for (int v = 0; v < nv; v++) Yc[v * ys + (j < n1 ? nc + j : j - n1)] = __dmul_rn(y[v * nb + j], scale);
  } else {
    for (int i = tid; i < nc; i += kLuThreads)
      for (int v = 0; v < nv; v++) out[v * vs + cs[c] + i] = __dmul_rn(y[v * nb + n1 + i], scale);
  }
}

// basic Schwarz: out[i] = sum of the slots of point i (ascending slot = ascending block)
__global__ void k_asm_gather(int n, int nv, const long long* __restrict__ inv_off,
                             const long long* __restrict__ inv_slot, const double* __restrict__ Y, long long ys,
                             double* __restrict__ out, long long vs, const int* __restrict__ skip) {
  if (skip && *skip) return;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    for (int v = 0; v < nv; v++) {
      double s = 0.0;
      for (long long k = inv_off[i]; k < inv_off[i + 1]; k++) s += Y[v * ys + inv_slot[k]];
      out[v * vs + i] = s;
    }
}

// inverse of the buffer lists: per point, the slots that hold it
__global__ void k_inv_count(long long nslot, const int* __restrict__ idx, long long* __restrict__ cnt) {
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < nslot; k += (long long)gridDim.x * blockDim.x)
    atomicAdd((unsigned long long*)&cnt[idx[k]], 1ull);
}

__global__ void k_inv_fill(long long nslot, const int* __restrict__ idx, const long long* __restrict__ off,
                           long long* __restrict__ cur, long long* __restrict__ slot) {
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < nslot; k += (long long)gridDim.x * blockDim.x) {
    int i = idx[k];
    long long p = (long long)atomicAdd((unsigned long long*)&cur[i], 1ull);
    slot[off[i] + p] = k;
  }
}

// each point's few slots in ascending order (insertion sort)
__global__ void k_inv_sort(int n, const long long* __restrict__ off, long long* __restrict__ slot) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    long long a = off[i], e = off[i + 1];
    for (long long k = a + 1; k < e; k++) {
      long long v = slot[k], j = k - 1;
      while (j >= a && slot[j] > v) {
        slot[j + 1] = slot[j];
        j--;
      }
      slot[j + 1] = v;
    }
  }
}

template <class T>
size_t chol_smem() {
  return sizeof(T) * (4 * KCOf<T>::v * SP<T>::S + 2 * TB * SP<T>::S);
}

}  // namespace

void rasm_build(RasmPlan& R, const PointSet& P, bool fp32, Workspace& ws, unsigned* err, cudaStream_t s,
                double ws_budget_bytes, bool factor, bool basic) {
  const Grid& g = P.g;
  int* cnt = (int*)ws.get(40, sizeof(int) * ((size_t)g.ncell + 1));
  k_buffer_lists<<<ceil_div(g.ncell, 8), 256, 0, s>>>(g, P.x.get(), P.y.get(), P.view().z, P.cs.get(), 0, cnt,
                                                      nullptr, nullptr);
  PRBF_CHECK_LAUNCH();
  std::vector<int> hcnt(g.ncell), hcs(g.ncell + 1);
  PRBF_CUDA(cudaMemcpyAsync(hcnt.data(), cnt, sizeof(int) * g.ncell, cudaMemcpyDeviceToHost, s));
  PRBF_CUDA(cudaMemcpyAsync(hcs.data(), P.cs.get(), sizeof(int) * (g.ncell + 1), cudaMemcpyDeviceToHost, s));
  PRBF_CUDA(cudaStreamSynchronize(s));
  std::vector<long long> hb(g.ncell + 1);
  hb[0] = 0;
  for (int c = 0; c < g.ncell; c++) hb[c + 1] = hb[c] + hcnt[c];
  R.boff.reserve(g.ncell + 1);
  R.idx.reserve(std::max<long long>(hb[g.ncell], 1));
  PRBF_CUDA(cudaMemcpyAsync(R.boff.get(), hb.data(), sizeof(long long) * (g.ncell + 1), cudaMemcpyHostToDevice, s));
  k_buffer_lists<<<ceil_div(g.ncell, 8), 256, 0, s>>>(g, P.x.get(), P.y.get(), P.view().z, P.cs.get(), 1, cnt,
                                                      R.boff.get(), R.idx.get());
  PRBF_CHECK_LAUNCH();
  BlockGeom G;
  G.dim = g.dim;
  G.n = P.n;
  G.ncell = g.ncell;
  G.x = P.x.get();
  G.y = P.y.get();
  G.z = P.view().z;
  G.cs = P.cs.get();
  G.sigma = g.sigma;
  rasm_factor(R, G, hcnt, hcs, fp32, ws, err, s, ws_budget_bytes, factor, basic);
}

void rasm_block_K(const RasmPlan& R, const PointSet& P, int cell, int nb, double* K_dev, Workspace& ws,
                  cudaStream_t s) {
  int* dbc = (int*)ws.get(41, sizeof(int));
  long long* dk = (long long*)ws.get(42, sizeof(long long) * 2);
  const long long hk[2] = {0, (long long)nb * nb};
  PRBF_CUDA(cudaMemcpyAsync(dbc, &cell, sizeof(int), cudaMemcpyHostToDevice, s));
  PRBF_CUDA(cudaMemcpyAsync(dk, hk, sizeof(hk), cudaMemcpyHostToDevice, s));
  PRBF_CUDA(cudaMemsetAsync(K_dev, 0, sizeof(double) * (size_t)nb * nb, s));
  const Grid& g = P.g;
  k_assemble<double><<<dim3(64, 1), 256, 0, s>>>(1, dbc, R.boff.get(), P.cs.get(), R.idx.get(), dk, P.x.get(),
                                                  P.y.get(), P.view().z, g.dim, 1.0 / (2.0 * g.sigma * g.sigma),
                                                  nullptr, 0.0, K_dev, nullptr, nullptr, 0, kexp_of_sigma(g.sigma),
                                                  exp_table_dev(s));
  PRBF_CHECK_LAUNCH();
  PRBF_CUDA(cudaStreamSynchronize(s));  // the host copies of dbc / dk stay valid until here
}

void rasm_factor_rows(const RasmPlan& R, int cell, int nb, double* out, cudaStream_t s) {
  if (std::binary_search(R.lu_cells.begin(), R.lu_cells.end(), cell))
    throw Error(PRBF_ERR_STATE, "the block of this cell was factored by LU (no Cholesky factor)");
  if (!R.factor || R.fp32) throw Error(PRBF_ERR_STATE, "the plan keeps no FP64 factor");
  long long lo[2];
  PRBF_CUDA(cudaMemcpyAsync(lo, R.loff.get() + cell, sizeof(lo), cudaMemcpyDeviceToHost, s));
  PRBF_CUDA(cudaStreamSynchronize(s));
  if (lo[1] - lo[0] != rowoff<double>(nb)) throw Error(PRBF_ERR_STATE, "factor size does not match the block");
  std::vector<double> h((size_t)(lo[1] - lo[0]));
  PRBF_CUDA(cudaMemcpyAsync(h.data(), R.L64.get() + lo[0], sizeof(double) * h.size(), cudaMemcpyDeviceToHost, s));
  PRBF_CUDA(cudaStreamSynchronize(s));
  for (long long i = 0; i < nb; i++)
    std::copy(h.begin() + rowoff<double>(i), h.begin() + rowoff<double>(i) + i + 1, out + i * (i + 1) / 2);
}

void rasm_buffer_lists(const PointSet& P, int* counts_dev, const long long* boff_dev, int* idx_dev, cudaStream_t s) {
  const Grid& g = P.g;
  k_buffer_lists<<<ceil_div(g.ncell, 8), 256, 0, s>>>(g, P.x.get(), P.y.get(), P.view().z, P.cs.get(),
                                                      boff_dev ? 1 : 0, counts_dev, boff_dev, idx_dev);
  PRBF_CHECK_LAUNCH();
}

namespace {
// The LU fallback's blocks (cells, any order): K assembled unshifted into their own
// storage, factored by k_lu_fp64; a zero pivot is the reference's PETSc LU failure.
void lu_build(RasmPlan& R, const BlockGeom& G, const std::vector<int>& hcnt, std::vector<int> cells, Workspace& ws,
              cudaStream_t s) {
  std::sort(cells.begin(), cells.end());
  const int nlu = (int)cells.size();
  std::vector<long long> hk(nlu + 1, 0), hp(nlu + 1, 0);
  std::vector<int> hmap(G.ncell, -1);
  for (int b = 0; b < nlu; b++) {
    const long long nb = hcnt[cells[b]];
    hk[b + 1] = hk[b] + nb * nb;
    hp[b + 1] = hp[b] + nb;
    hmap[cells[b]] = b;
  }
  R.lucell.reserve(nlu);
  R.lukoff.reserve(nlu + 1);
  R.lupoff.reserve(nlu + 1);
  R.lu_of_cell.reserve(G.ncell);
  R.LU64.reserve(std::max<long long>(hk[nlu], 1));
  R.lupiv.reserve(std::max<long long>(hp[nlu], 1));
  PRBF_CUDA(cudaMemcpyAsync(R.lucell.get(), cells.data(), sizeof(int) * nlu, cudaMemcpyHostToDevice, s));
  PRBF_CUDA(cudaMemcpyAsync(R.lukoff.get(), hk.data(), sizeof(long long) * (nlu + 1), cudaMemcpyHostToDevice, s));
  PRBF_CUDA(cudaMemcpyAsync(R.lupoff.get(), hp.data(), sizeof(long long) * (nlu + 1), cudaMemcpyHostToDevice, s));
  PRBF_CUDA(cudaMemcpyAsync(R.lu_of_cell.get(), hmap.data(), sizeof(int) * G.ncell, cudaMemcpyHostToDevice, s));
  const double inv2s2 = 1.0 / (2.0 * G.sigma * G.sigma);
  for (int b0 = 0; b0 < nlu; b0 += 65535) {  // gridDim.y of the assembly
    const int m = std::min(65535, nlu - b0);
    k_assemble<double><<<dim3(64, m), 256, 0, s>>>(m, R.lucell.get() + b0, R.boff.get(), G.cs, R.idx.get(),
                                                   R.lukoff.get() + b0, G.x, G.y, G.z, G.dim, inv2s2, G.cell_sigma,
                                                   0.0, R.LU64.get(), nullptr, nullptr, 0, kexp_of_sigma(G.sigma),
                                                   exp_table_dev(s));
    PRBF_CHECK_LAUNCH();
  }
  unsigned char* dbad = (unsigned char*)ws.get(50, nlu);
  k_lu_fp64<<<nlu, kLuThreads, 0, s>>>(nlu, R.lucell.get(), R.boff.get(), R.lukoff.get(), R.LU64.get(),
                                        R.lupoff.get(), R.lupiv.get(), dbad);
  PRBF_CHECK_LAUNCH();
  std::vector<unsigned char> hbad(nlu);
  PRBF_CUDA(cudaMemcpyAsync(hbad.data(), dbad, nlu, cudaMemcpyDeviceToHost, s));
  PRBF_CUDA(cudaStreamSynchronize(s));
  for (int b = 0; b < nlu; b++)
    if (hbad[b])
      throw Error(PRBF_ERR_FACTOR, "zero pivot in the LU of a subdomain block (duplicated points): the reference's "
                                   "PETSc LU stops here as well");
  R.nlu = nlu;
  R.lu_cells = cells;
}
}  // namespace

void rasm_factor(RasmPlan& R, const BlockGeom& G, const std::vector<int>& hcnt, const std::vector<int>& hcs, bool fp32,
                 Workspace& ws, unsigned* err, cudaStream_t s, double ws_budget_bytes, bool factor, bool basic) {
  const int ncell = G.ncell;
  R.fp32 = fp32;
  R.ncell = ncell;
  // several right-hand sides per launch pay off in FP32 (the factor read is shared); the
  // FP64 solves are bound by the FP64 pipe and lose occupancy with more vectors
  if (!fp32) R.max_nv = 1;
  // host plan: offsets of S_c, the list of non-empty blocks (largest first, so the batches
  // of the factorisation keep similar sizes together and the long blocks start early)
  std::vector<long long> hso(ncell + 1);
  std::vector<int> blk;
  hso[0] = 0;
  R.max_nb = 0;
  R.max_nc = 0;
  for (int c = 0; c < ncell; c++) {
    long long nbk = hcnt[c], nc = hcs[c + 1] - hcs[c];
    hso[c + 1] = hso[c] + nbk * nc;
    if (nbk) blk.push_back(c);
    R.max_nb = std::max<int>(R.max_nb, (int)nbk);
    R.max_nc = std::max<int>(R.max_nc, (int)nc);
  }
  if (G.cell_sigma)
    std::stable_sort(blk.begin(), blk.end(), [&](int a, int b) { return hcnt[a] > hcnt[b]; });
  R.nblocks = (int)blk.size();
  R.soff.reserve(ncell + 1);
  PRBF_CUDA(cudaMemcpyAsync(R.soff.get(), hso.data(), sizeof(long long) * (ncell + 1), cudaMemcpyHostToDevice, s));
  size_t esz = fp32 ? sizeof(float) : sizeof(double);
  // FP64 form keeps the packed Cholesky factors (backward-stable triangular solves at
  // every apply); the FP32 form keeps S_c (one GEMV per apply)
  R.basic = basic;
  R.n = G.n;
  R.factor = !fp32 || factor || basic;
  if (basic) {
    // slots of each point (deterministic summation of the block solutions)
    long long nslot = 0;
    for (int c = 0; c < ncell; c++) nslot += hcnt[c];
    R.nslot = nslot;
    R.Y.reserve(std::max<long long>(nslot, 1) * std::max(1, std::min(4, R.max_nv)));
    R.inv_off.reserve((size_t)G.n + 1);
    R.inv_slot.reserve(std::max<long long>(nslot, 1));
    long long* cur = (long long*)ws.get(47, sizeof(long long) * ((size_t)G.n + 1));
    PRBF_CUDA(cudaMemsetAsync(R.inv_off.get(), 0, sizeof(long long) * ((size_t)G.n + 1), s));
    PRBF_CUDA(cudaMemsetAsync(cur, 0, sizeof(long long) * ((size_t)G.n + 1), s));
    const int gb = (int)std::max<long long>(1, std::min<long long>((nslot + 255) / 256, 8 * 152));
    if (nslot) k_inv_count<<<gb, 256, 0, s>>>(nslot, R.idx.get(), R.inv_off.get());
    PRBF_CHECK_LAUNCH();
    scan_exclusive_dev(R.inv_off.get(), R.inv_off.get(), (long long)G.n + 1, ws, 48, s);
    if (nslot) k_inv_fill<<<gb, 256, 0, s>>>(nslot, R.idx.get(), R.inv_off.get(), cur, R.inv_slot.get());
    k_inv_sort<<<ceil_div(G.n, 256), 256, 0, s>>>(G.n, R.inv_off.get(), R.inv_slot.get());
    PRBF_CHECK_LAUNCH();
  }
  if (R.factor) {
    std::vector<long long> hl(ncell + 1);
    hl[0] = 0;
    for (int c = 0; c < ncell; c++) hl[c + 1] = hl[c] + (fp32 ? rowoff<float>(hcnt[c]) : rowoff<double>(hcnt[c]));
    R.loff.reserve(ncell + 1);
    PRBF_CUDA(cudaMemcpyAsync(R.loff.get(), hl.data(), sizeof(long long) * (ncell + 1), cudaMemcpyHostToDevice, s));
    if (fp32)
      R.L32.reserve(std::max<long long>(hl[ncell], 1));
    else
      R.L64.reserve(std::max<long long>(hl[ncell], 1));
    PRBF_CUDA(cudaStreamSynchronize(s));
  } else {
    R.S32.reserve(std::max<long long>(hso[ncell], 1));
  }

  // batches of blocks within the workspace budget: K (nb^2) and, for the S_c form, the
  // diagonal tiles' inverses (ntile TB^2)
  const double inv2s2 = 1.0 / (2.0 * G.sigma * G.sigma);
  const double out_scale = 2.0 * M_PI * G.sigma * G.sigma;  // A = K/(2 pi sigma^2): A^-1 = 2 pi sigma^2 K^-1
  const size_t smem = chol_smem<double>();  // the FP64 factorisation's tiles
  // FP32 assembly: the largest block's split coordinates in shared memory
  const size_t asm_smem = fp32 ? sizeof(float2) * (size_t)G.dim * std::max(R.max_nb, 1) : 0;
  if (fp32) {
    if (asm_smem > 200 * 1024) throw Error(PRBF_ERR_CAPACITY, "subdomain larger than the assembly's shared memory");
    PRBF_CUDA(cudaFuncSetAttribute(k_assemble<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)asm_smem));
    PRBF_CUDA(cudaFuncSetAttribute(k_chol_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)chol_tc_smem()));
  } else
    PRBF_CUDA(cudaFuncSetAttribute(k_chol_fp64, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  R.nfallback = 0;
  R.retried.clear();
  R.nlu = 0;
  R.lu_cells.clear();
  R.lu_scale = 2.0 * M_PI * G.sigma * G.sigma;
  R.lu_cell_sigma = G.cell_sigma;
  std::vector<int> lu_cells;
  // FP32 form: the coordinates split into float pairs once (the assembly then stays on the
  // FP32 pipes)
  float2* hl = nullptr;
  if (fp32) {
    hl = (float2*)ws.get(55, sizeof(float2) * (size_t)G.dim * std::max(G.n, 1));
    const double* xyz[3] = {G.x, G.y, G.z};
    const int gb = (int)std::max<long long>(1, std::min<long long>(((long long)G.n + 255) / 256, 8 * 152));
    for (int d = 0; d < G.dim; d++) k_split_hl<<<gb, 256, 0, s>>>(G.n, xyz[d], hl + (size_t)d * G.n);
    PRBF_CHECK_LAUNCH();
  }
  size_t pos = 0;
  std::vector<long long> hk, hx;
  std::vector<int> bc;
  std::vector<unsigned char> hbad;
  while (pos < blk.size()) {
    hk.assign(1, 0);
    hx.assign(1, 0);
    bc.clear();
    size_t q = pos;
    while (q < blk.size()) {
      int c = blk[q];
      long long nbk = hcnt[c], nc = hcs[c + 1] - hcs[c];
      long long n1 = nbk - nc;
      long long ntile = (n1 + TB - 1) / TB + (nc + TB - 1) / TB;
      long long ke = nbk * nbk, xe = R.factor ? 1 : ntile * TB * TB;  // S_c form: FP32 only
      if (!bc.empty() && (double)(hk.back() + ke + hx.back() + xe) * esz > ws_budget_bytes) break;
      if (bc.size() >= 65535) break;  // gridDim.y of the assembly
      bc.push_back(c);
      hk.push_back(hk.back() + ke);
      hx.push_back(hx.back() + xe);
      q++;
    }
    int nb_batch = (int)bc.size();
    int* dbc = (int*)ws.get(41, sizeof(int) * nb_batch);
    long long* dk = (long long*)ws.get(42, sizeof(long long) * (nb_batch + 1));
    long long* dx = (long long*)ws.get(43, sizeof(long long) * (nb_batch + 1));
    unsigned char* dbad = (unsigned char*)ws.get(44, nb_batch);
    void* Kw = ws.get(45, (size_t)hk.back() * esz);
    void* Xw = ws.get(46, (size_t)hx.back() * esz);
    PRBF_CUDA(cudaMemcpyAsync(dbc, bc.data(), sizeof(int) * nb_batch, cudaMemcpyHostToDevice, s));
    PRBF_CUDA(cudaMemcpyAsync(dk, hk.data(), sizeof(long long) * (nb_batch + 1), cudaMemcpyHostToDevice, s));
    PRBF_CUDA(cudaMemcpyAsync(dx, hx.data(), sizeof(long long) * (nb_batch + 1), cudaMemcpyHostToDevice, s));
    for (int attempt = 0; attempt < 3; attempt++) {
      const unsigned char* only = attempt ? dbad : nullptr;
      // diagonal shift of the retries (relative to the unit diagonal of K)
      double shift = attempt == 0 ? 0.0 : (fp32 ? (attempt == 1 ? 1e-5 : 1e-3) : (attempt == 1 ? 1e-12 : 1e-9));
      dim3 ag(kAsmCtas, nb_batch);
      if (fp32) {
        k_assemble<float><<<ag, 256, asm_smem, s>>>(nb_batch, dbc, R.boff.get(), G.cs, R.idx.get(), dk, G.x, G.y, G.z, G.dim,
                                             inv2s2, G.cell_sigma, shift, (float*)Kw, only, hl, (long long)G.n,
                                             0.0, nullptr);
        PRBF_CHECK_LAUNCH();
        // the Cholesky on the tensor cores (and S_c), then the packed factor
        k_chol_tc<<<nb_batch, NTH, chol_tc_smem(), s>>>(nb_batch, dbc, R.boff.get(), G.cs, dk, (float*)Kw, dx,
                                                        (float*)Xw, dbad, only, R.factor ? 1 : 0, R.soff.get(),
                                                        R.factor ? nullptr : R.S32.get(), out_scale, G.cell_sigma,
                                                        err);
        PRBF_CHECK_LAUNCH();
        if (R.factor)
          k_pack_factor<<<nb_batch, NTH, 0, s>>>(nb_batch, dbc, R.boff.get(), dk, (const float*)Kw,
                                                  std::sqrt(1.0 / out_scale), G.cell_sigma, only, R.loff.get(),
                                                  R.L32.get());
      } else {
        k_assemble<double><<<ag, 256, 0, s>>>(nb_batch, dbc, R.boff.get(), G.cs, R.idx.get(), dk, G.x, G.y, G.z,
                                              G.dim, inv2s2, G.cell_sigma, shift, (double*)Kw, only, nullptr, 0,
                                              kexp_of_sigma(G.sigma), exp_table_dev(s));
        PRBF_CHECK_LAUNCH();
        k_chol_fp64<<<nb_batch, NTH, smem, s>>>(nb_batch, dbc, R.boff.get(), dk, (double*)Kw,
                                                std::sqrt(1.0 / out_scale), G.cell_sigma, dbad, only, R.loff.get(),
                                                R.L64.get());
      }
      PRBF_CHECK_LAUNCH();
      hbad.resize(nb_batch);
      PRBF_CUDA(cudaMemcpyAsync(hbad.data(), dbad, nb_batch, cudaMemcpyDeviceToHost, s));
      PRBF_CUDA(cudaStreamSynchronize(s));
      int nbad = 0;
      for (int k = 0; k < nb_batch; k++) {
        nbad += hbad[k] ? 1 : 0;
        if (hbad[k] && attempt == 0) R.retried.push_back(bc[k]);
      }
      if (nbad == 0) break;
      if (!fp32 && R.lu_fallback) {  // factored by LU after the batches, unshifted
        for (int k = 0; k < nb_batch; k++)
          if (hbad[k]) lu_cells.push_back(bc[k]);
        R.nfallback += nbad;
        break;
      }
      if (attempt == 2) throw Error(PRBF_ERR_FACTOR, "subdomain block not positive definite after shifted retries");
      R.nfallback += nbad;
    }
    pos = q;
  }
  if (!lu_cells.empty()) lu_build(R, G, hcnt, lu_cells, ws, s);
}

namespace {
int trw_ldy(const RasmPlan& R) { return (std::max(R.max_nb, 1) + 3) & ~3; }

template <class T>
void apply_tri_nv(const RasmPlan& R, const T* Lp, const int* cs, const double* r, double* out, long long vs, int nv,
                  cudaStream_t s, const int* skip) {
  const int full = R.basic ? 1 : 0;
  if constexpr (std::is_same<T, float>::value) {
    const int ldy = trw_ldy(R);
    const size_t sm = (size_t)kTrwWarps * nv * ldy * sizeof(float);
    const int grid = ceil_div(R.ncell, kTrwWarps);
    switch (nv) {
      case 1:
        k_apply_trw<1><<<grid, kTrwWarps * 32, sm, s>>>(R.ncell, R.boff.get(), cs, R.idx.get(), R.loff.get(), Lp, r,
                                                        out, vs, skip, full, R.Y.get(), R.nslot, R.seg, ldy);
        break;
      case 2:
        k_apply_trw<2><<<grid, kTrwWarps * 32, sm, s>>>(R.ncell, R.boff.get(), cs, R.idx.get(), R.loff.get(), Lp, r,
                                                        out, vs, skip, full, R.Y.get(), R.nslot, R.seg, ldy);
        break;
      case 3:
        k_apply_trw<3><<<grid, kTrwWarps * 32, sm, s>>>(R.ncell, R.boff.get(), cs, R.idx.get(), R.loff.get(), Lp, r,
                                                        out, vs, skip, full, R.Y.get(), R.nslot, R.seg, ldy);
        break;
      default:
        k_apply_trw<4><<<grid, kTrwWarps * 32, sm, s>>>(R.ncell, R.boff.get(), cs, R.idx.get(), R.loff.get(), Lp, r,
                                                        out, vs, skip, full, R.Y.get(), R.nslot, R.seg, ldy);
        break;
    }
  } else {
    const size_t sm = (size_t)nv * R.max_nb * sizeof(T);
    const int* luc = R.nlu ? R.lu_of_cell.get() : nullptr;
    switch (nv) {
      case 1:
        k_apply_tri<T, 1><<<R.ncell, 256, sm, s>>>(R.ncell, R.boff.get(), cs, R.idx.get(), R.loff.get(), Lp, r, out,
                                                   vs, skip, full, R.Y.get(), R.nslot, R.seg, luc);
        break;
      case 2:
        k_apply_tri<T, 2><<<R.ncell, 256, sm, s>>>(R.ncell, R.boff.get(), cs, R.idx.get(), R.loff.get(), Lp, r, out,
                                                   vs, skip, full, R.Y.get(), R.nslot, R.seg, luc);
        break;
      case 3:
        k_apply_tri<T, 3><<<R.ncell, 256, sm, s>>>(R.ncell, R.boff.get(), cs, R.idx.get(), R.loff.get(), Lp, r, out,
                                                   vs, skip, full, R.Y.get(), R.nslot, R.seg, luc);
        break;
      default:
        k_apply_tri<T, 4><<<R.ncell, 256, sm, s>>>(R.ncell, R.boff.get(), cs, R.idx.get(), R.loff.get(), Lp, r, out,
                                                   vs, skip, full, R.Y.get(), R.nslot, R.seg, luc);
        break;
    }
  }
  PRBF_CHECK_LAUNCH();
}

template <class T>
void set_tri_smem(const RasmPlan& R) {
  for (int nv = 1; nv <= std::max(1, std::min(4, R.max_nv)); nv++) {
    size_t sm;
    const void* f;
    if constexpr (std::is_same<T, float>::value) {
      sm = (size_t)kTrwWarps * nv * trw_ldy(R) * sizeof(float);
      f = nv == 1 ? (const void*)k_apply_trw<1>
                  : nv == 2 ? (const void*)k_apply_trw<2> : nv == 3 ? (const void*)k_apply_trw<3> : (const void*)k_apply_trw<4>;
    } else {
      sm = (size_t)nv * std::max(R.max_nb, 1) * sizeof(T) + sizeof(T) * 32 * 33;
      f = nv == 1 ? (const void*)k_apply_tri<T, 1>
                  : nv == 2 ? (const void*)k_apply_tri<T, 2>
                            : nv == 3 ? (const void*)k_apply_tri<T, 3> : (const void*)k_apply_tri<T, 4>;
    }
    if (sm > 220 * 1024) throw Error(PRBF_ERR_CAPACITY, "subdomain larger than the apply kernel's shared memory");
    PRBF_CUDA(cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   (int)(std::is_same<T, float>::value ? sm : sm - sizeof(T) * 32 * 33)));
  }
}
}  // namespace

void rasm_apply(const RasmPlan& R, const int* cs, const double* r, double* out, cudaStream_t s, const int* skip, int nv,
                long long vstride) {
  if (R.nblocks == 0 || nv <= 0) return;
  const int step = std::max(1, std::min(4, R.max_nv));
  for (int v0 = 0; v0 < nv; v0 += step) {
    const int k = std::min(step, nv - v0);
    const double* rv = r + v0 * vstride;
    double* ov = out + v0 * vstride;
    if (R.factor) {
      if (R.fp32) {
        apply_tri_nv<float>(R, R.L32.get(), cs, rv, ov, vstride, k, s, skip);
      } else {
        apply_tri_nv<double>(R, R.L64.get(), cs, rv, ov, vstride, k, s, skip);
        if (R.nlu) {
          k_apply_lu<<<R.nlu, kLuThreads, (size_t)k * R.max_nb * sizeof(double), s>>>(
              R.nlu, R.lucell.get(), R.boff.get(), cs, R.idx.get(), R.lukoff.get(), R.LU64.get(), R.lupoff.get(),
              R.lupiv.get(), rv, ov, vstride, k, skip, R.basic ? 1 : 0, R.Y.get(), R.nslot, R.seg, R.lu_scale,
              R.lu_cell_sigma);
          PRBF_CHECK_LAUNCH();
        }
      }
    } else {
      for (int v = 0; v < k; v++) {
        const size_t sm = (size_t)R.max_nb * sizeof(float);
        k_apply<float><<<R.ncell, 128, sm, s>>>(R.ncell, R.boff.get(), cs, R.idx.get(), R.soff.get(), R.S32.get(),
                                                rv + v * vstride, ov + v * vstride, skip);
        PRBF_CHECK_LAUNCH();
      }
    }
    if (R.basic) {
      k_asm_gather<<<ceil_div(R.n, 256), 256, 0, s>>>(R.n, k, R.inv_off.get(), R.inv_slot.get(), R.Y.get(), R.nslot,
                                                      ov, vstride, skip);
      PRBF_CHECK_LAUNCH();
    }
  }
}

void rasm_set_apply_smem(const RasmPlan& R) {
  if (R.nlu) {
    const size_t sm = (size_t)std::max(1, std::min(4, R.max_nv)) * std::max(R.max_nb, 1) * sizeof(double);
    if (sm > 220 * 1024) throw Error(PRBF_ERR_CAPACITY, "subdomain larger than the LU apply's shared memory");
    PRBF_CUDA(cudaFuncSetAttribute(k_apply_lu, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
  }
  if (R.factor) {
    if (R.fp32)
      set_tri_smem<float>(R);
    else
      set_tri_smem<double>(R);
  } else {
    size_t sm = (size_t)std::max(R.max_nb, 1) * sizeof(float);
    if (sm > 220 * 1024) throw Error(PRBF_ERR_CAPACITY, "subdomain larger than the apply kernel's shared memory");
    PRBF_CUDA(cudaFuncSetAttribute(k_apply<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
  }
}

}  // namespace prbf
