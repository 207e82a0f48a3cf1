// gauss.cu -- truncated Gaussian sums on sm_103a: the matvec of the solve (mymatmult,
// 2d/matmult.cxx:6-51; 3d/matmult.cxx:6-52) and the evaluation of the interpolant at
// other targets (get_vorticity, 2d/get_vorticity.h:9-27).
//
//   w_i = sum_{j in T(c(i))} g_j exp(-|x_i - x_j|^2 / (2 sigma^2)) / (2 pi sigma^2)
//
// T(c) is the truncation set of the target's cell c (2d/get_trunc.h:9-78): every source
// of cell c, plus the sources of the cells within +-nb_trunc whose per-axis distance to
// the centre of c is below trunc_len. The box test is evaluated in FP64 exactly as in the
// reference, so the set is identical.
//
// One CTA works on one (target cell, tile of <= kTileT targets) item:
//   1. the neighbour cells of a column (fixed jx [, jz], jy0..jy1) are one contiguous range
//      of the cell-sorted source arrays; ranges are staged into shared memory with TMA bulk
//      copies (cp.async.bulk) completing on an mbarrier (bounded wait);
//   2. the CTA filters the staged sources with the box test and compacts the passing ones,
//      in order, into a second shared buffer (as cell-relative, scaled coordinates);
//   3. each warp takes groups of kGroup targets, its lanes stride over the compacted
//      sources, and the partial sums are reduced with warp shuffles.
// FP64 form: exp on the FP64 pipe with a table-folded polynomial (12 FP64 instructions
// per pair, range reduction bits and the 2^-m scaling on the integer pipe); coordinates
// relative to the cell centre, unscaled, so x_t - x_s rounds as in the reference. FP32
// form: scaled FP32 coordinates relative to the cell centre and the SFU exp2.
//
// NV weight vectors (several right-hand sides of one point set, NV <= 4) are summed in
// one pass: each pair's exponential is computed once and multiplies NV weights.
#include <algorithm>
#include <atomic>
#include <cmath>

#include "device.h"

namespace prbf {
namespace {

constexpr int kThreads = 128;  // 4 warps
constexpr int kWarps = kThreads / 32;
constexpr int kTileT = 128;    // targets per work item
constexpr int kGroup = 4;      // targets per warp pass
constexpr int kRawCap = 1024;  // staged raw sources per fill (incl. alignment padding)
constexpr int kMaxPieces = 64; // source ranges per fill
constexpr int kMaxRanges = 256; // column ranges of an item kept in shared memory

// exp table: e^a with a = -L*d, d >= 0, L = ln2/n:  k = rint(d), r = k - d in [-1/2, 1/2],
// e^a = 2^(-k/n) e^(L r) = 2^-m T[j] p(r),  k = m*n + j; the table holds T[j] c_i
// interleaved per j. Large table: n = 1024 and the cubic interpolating e^(L r) at the 4
// Chebyshev nodes of [-1/2, 1/2] (near-minimax, |p - e^(Lr)| / e^(Lr) <= 2 (L/4)^4 / 4! ~
// 7e-17): 11 FP64 instructions per 2D pair. Small table: n = 256 and the quartic Taylor
// polynomial (remainder (L/2)^5 / 5! ~ 4e-17), for the kernels whose shared memory would
// otherwise drop to one CTA per SM (3D, and 2D with more than two weight vectors).
template <bool BIG>
struct ExpTab {
  static constexpr int bits = BIG ? 10 : 8, n = 1 << bits, poly = BIG ? 4 : 5;
};
template <int DIM, int NV>
struct UseBigTabSym {  // the symmetric sum keeps the 256-entry table in 3D (two CTAs per SM)
  static constexpr bool v = DIM == 2 && NV <= 2;
};
template <int DIM, int NV>
struct UseBigTab {
  // 2D one or two vectors; 3D every vector count of the one-sided sum (its staging buffers
  // are sized so that the large table still leaves two CTAs per SM, Cfg)
  static constexpr bool v = DIM == 2 ? NV <= 2 : true;
};
__device__ double d_tab_big[ExpTab<true>::n * ExpTab<true>::poly];  // copied into shared memory by each CTA
__device__ double d_tab_small[ExpTab<false>::n * ExpTab<false>::poly];

template <int DIM, bool F32, int NV>
struct Cfg {
  // 3D FP64: smaller fills and compaction buffers, so that the 1024-entry exp table (one
  // FP64 instruction per pair fewer than the 256-entry quartic) fits two CTAs per SM
  static constexpr bool k3d64 = DIM == 3 && !F32;
  static constexpr int kComp = k3d64 ? (NV > 1 ? 768 : 1024) : (NV > 1 ? 1024 : 2048);
  static constexpr int kRaw = k3d64 ? 512 : kRawCap;
  using T = typename std::conditional<F32, float, double>::type;
};

struct Piece {
  int raw_off;  // smem index of the first valid element
  int count;    // valid elements
  int gstart;   // global (sorted) index of the first valid element
};

constexpr size_t align16(size_t v) { return (v + 15) & ~(size_t)15; }

// Dynamic shared memory carve-up of k_gauss (byte offsets, each 16-byte aligned).
template <int DIM, bool F32, int NV>
struct Layout {
  using T = typename Cfg<DIM, F32, NV>::T;
  static constexpr int NA = DIM + NV;
  static constexpr size_t raw = 0;
  static constexpr size_t comp = align16(raw + sizeof(double) * NA * Cfg<DIM, F32, NV>::kRaw);
  static constexpr size_t tgt = align16(comp + sizeof(T) * NA * Cfg<DIM, F32, NV>::kComp);
  static constexpr size_t acc = align16(tgt + sizeof(T) * DIM * kTileT);
  static constexpr size_t tab = align16(acc + sizeof(T) * NV * kTileT);
  using ET = ExpTab<UseBigTab<DIM, NV>::v>;
  static constexpr size_t pieces = align16(tab + (F32 ? 0 : sizeof(double) * ET::poly * ET::n));
  static constexpr size_t bar = align16(pieces + sizeof(Piece) * kMaxPieces);
  static constexpr size_t total = bar + 16;
};

__device__ __forceinline__ double hi_sub(double v, int m20) {
  // v * 2^-m for a normal positive v: subtract m from the exponent field
  int hi = __double2hiint(v) - m20;
  return __hiloint2double(hi, __double2loint(v));
}

__device__ __forceinline__ float ex2_approx(float x) {
  float y;
  asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}

// Per-problem constants of the sum (from sigma): FP32 coordinate scale, FP64 exponent
// factor, normalisation. The host computes the same expressions for single problems.
struct SumConsts {
  double scale, kexp, norm;
};

__host__ __device__ inline SumConsts sum_consts(double sigma, bool f32, int ntab) {
  const double ln2 = 0.6931471805599453;  // ln 2 rounded to double
  SumConsts k;
  k.scale = f32 ? sqrt(1.0 / (2.0 * sigma * sigma * ln2)) : 1.0;
  k.kexp = (double)ntab / (2.0 * sigma * sigma * ln2);
  k.norm = 1.0 / (2 * 3.141592653589793 * sigma * sigma);
  return k;
}

// Items are processed in rounds of gridDim.x (snake order over the list, which a batched
// plan sorts by decreasing cost): with one CTA per item this is the plain launch, with
// fewer CTAs it is a persistent kernel. BATCH: the item's cell indexes a concatenation of
// grids (cell -> problem -> Grid with its first global cell and sigma).
// FP64 forms run two CTAs per SM (shared memory): registers are not the limit there
template <bool F32>
struct GaussMinBlocks {
  static constexpr int v = F32 ? 1 : 2;
};

template <int DIM, bool F32, int NV, bool BATCH>
__global__ void __launch_bounds__(kThreads, GaussMinBlocks<F32>::v) k_gauss(
    Grid g0, const Grid* __restrict__ grids, const int* __restrict__ cprob, const int2* __restrict__ items, int nitems,
    const double* __restrict__ tx, const double* __restrict__ ty, const double* __restrict__ tz,
    const int* __restrict__ cs_t, const double* __restrict__ sx, const double* __restrict__ sy,
    const double* __restrict__ sz, const double* __restrict__ sg, const int* __restrict__ cs_s, double* __restrict__ w,
    long long vstride, SumConsts k0, SegSkip seg, unsigned* err, const int* __restrict__ skip) {
  if (skip && *skip) return;
  using C = Cfg<DIM, F32, NV>;
  using T = typename C::T;
  constexpr int NA = DIM + NV;  // staged arrays: coordinates + weights
  extern __shared__ __align__(16) unsigned char smem[];
  const Layout<DIM, F32, NV> lay;
  double* raw = (double*)(smem + lay.raw);      // NA x C::kRaw (FP64, as stored in HBM)
  T* comp = (T*)(smem + lay.comp);              // NA x kComp (compacted truncation set)
  T* tgt = (T*)(smem + lay.tgt);                // DIM x kTileT
  T* acc = (T*)(smem + lay.acc);                // NV x kTileT
  double* tab = (double*)(smem + lay.tab);      // exp table (FP64 form only)
  using ET = ExpTab<UseBigTab<DIM, NV>::v>;
  Piece* pieces = (Piece*)(smem + lay.pieces);  // kMaxPieces
  uint64_t* bar = (uint64_t*)(smem + lay.bar);
  __shared__ int s_wsum[kWarps];
  __shared__ int s_fill[3];  // npieces, valid total, done flag
  __shared__ int s_cursor[2];
  __shared__ int s_abort;

  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
  if (!F32)
    for (int i = tid; i < ET::n * ET::poly; i += kThreads) tab[i] = (UseBigTab<DIM, NV>::v ? d_tab_big : d_tab_small)[i];
  if (tid == 0) mbar_init(bar, 1);
  unsigned phase = 0;
  const int G = gridDim.x;

  for (int round = 0; (long long)round * G < nitems; round++) {
    const int it = (round & 1) ? round * G + (G - 1 - (int)blockIdx.x) : round * G + (int)blockIdx.x;
    if (it >= nitems) continue;
    const int2 item = items[it];
    const int ic = item.x, t0 = item.y;
    Grid g = g0;
    SumConsts kc = k0;
    if constexpr (BATCH) {
      if (seg.cell_done(ic)) continue;  // a stopped problem (uniform over the CTA)
      g = grids[cprob[ic]];
      kc = sum_consts(g.sigma, F32, ET::n);
    }
    const double scale = kc.scale, kexp = kc.kexp;
    const int cb = g.cbase;
    const int nt = min(kTileT, cs_t[ic + 1] - t0);
    int ix, iy, iz;
    cell_xyz(g, ic - cb, ix, iy, iz);
    const double xc = centre_coord(g.xmin, ix, g.box);
    const double yc = centre_coord(g.ymin, iy, g.box);
    const double zc = DIM == 3 ? centre_coord(g.zmin, iz, g.box) : 0.0;
    const double L = g.trunc_len;
    const int c0 = cs_s[ic], c1 = cs_s[ic + 1];
    const int nb = g.nb_trunc;
    const int jx0 = max(0, ix - nb), jx1 = min(g.nx - 1, ix + nb);
    const int jy0 = max(0, iy - nb), jy1 = min(g.ny - 1, iy + nb);
    const int jz0 = DIM == 3 ? max(0, iz - nb) : 0, jz1 = DIM == 3 ? min(g.nz - 1, iz + nb) : 0;
    const int ncolx = jx1 - jx0 + 1;
    const int nranges = ncolx * (jz1 - jz0 + 1);

    __syncthreads();  // the previous item's readers of tgt/acc/comp are done
    for (int t = tid; t < nt; t += kThreads) {
      tgt[t] = (T)((tx[t0 + t] - xc) * scale);
      tgt[kTileT + t] = (T)((ty[t0 + t] - yc) * scale);
      if (DIM == 3) tgt[2 * kTileT + t] = (T)((tz[t0 + t] - zc) * scale);
#pragma unroll
      for (int v = 0; v < NV; v++) acc[v * kTileT + t] = T(0);
    }
    if (tid == 0) {
      s_cursor[0] = 0;  // range index
      s_cursor[1] = -1; // position inside the range (-1: start of range)
      s_abort = 0;
    }
    __syncthreads();

    int ncomp = 0;
    const int ngroups = (nt + kGroup - 1) / kGroup;

    // pair loop over comp[0, ncomp) for all targets of the tile
    auto flush = [&]() {
      for (int gi = wid; gi < ngroups; gi += kWarps) {
        T tu[kGroup], tv[kGroup], tw[kGroup];
        T a[kGroup][NV];
#pragma unroll
        for (int k = 0; k < kGroup; k++) {
          int t = min(gi * kGroup + k, nt - 1);
          tu[k] = tgt[t];
          tv[k] = tgt[kTileT + t];
          tw[k] = DIM == 3 ? tgt[2 * kTileT + t] : T(0);
#pragma unroll
          for (int v = 0; v < NV; v++) a[k][v] = T(0);
        }
        for (int j = lane; j < ncomp; j += 32) {
          T su = comp[j], sv = comp[C::kComp + j];
          T sw = DIM == 3 ? comp[2 * C::kComp + j] : T(0);
          T sgj[NV];
#pragma unroll
          for (int v = 0; v < NV; v++) sgj[v] = comp[(DIM + v) * C::kComp + j];
#pragma unroll
          for (int k = 0; k < kGroup; k++) {
            T du = tu[k] - su, dv = tv[k] - sv;
            T d2 = du * du;
            d2 = fma(dv, dv, d2);
            if (DIM == 3) {
              T dw = tw[k] - sw;
              d2 = fma(dw, dw, d2);
            }
            if constexpr (F32) {
              const float e = ex2_approx(-d2);
#pragma unroll
              for (int v = 0; v < NV; v++) a[k][v] = fmaf(sgj[v], e, a[k][v]);
            } else {
              // d2 = |x_t - x_s|^2 (unscaled: the differences are exact as in the reference);
              // in units of L = ln2/n the exponent is kexp*d2, kexp = n/(2 sigma^2 ln2):
              // k = rint(kexp d2) (fused), r = k - kexp d2 in [-1/2, 1/2] with a single rounding
              const double magic = 6755399441055744.0;  // 1.5 * 2^52
              double kd = fma(d2, kexp, magic);
              int kk = __double2loint(kd);
              double r = fma(-d2, kexp, kd - magic);
              int j8 = kk & (ET::n - 1);
              // m <= 900 keeps every scaled coefficient normal (2^-900 ~ 1e-271)
              int m20 = min(kk >> ET::bits, 900) << 20;
              double q;
              if constexpr (ET::poly == 4) {
                const double2 c01 = *(const double2*)(tab + 4 * j8);
                const double2 c23 = *(const double2*)(tab + 4 * j8 + 2);
                q = hi_sub(c23.y, m20);
                q = fma(r, q, hi_sub(c23.x, m20));
                q = fma(r, q, hi_sub(c01.y, m20));
                q = fma(r, q, hi_sub(c01.x, m20));
              } else {
                const double* cj = tab + ET::poly * j8;
                q = hi_sub(cj[ET::poly - 1], m20);
#pragma unroll
                for (int i = ET::poly - 2; i >= 0; i--) q = fma(r, q, hi_sub(cj[i], m20));
              }
#pragma unroll
              for (int v = 0; v < NV; v++) a[k][v] = fma(sgj[v], q, a[k][v]);
            }
          }
        }
        // the four target sums over the warp by a reduce-scatter butterfly (6 adds per
        // vector instead of 4 x 5; FP64 adds run on the narrow FP64 pipe): lane 8 k ends
        // with target k
        static_assert(kGroup == 4, "reduce-scatter of four sums");
        const bool h16 = lane & 16, h8 = lane & 8;
        const int t = gi * kGroup + (lane >> 3);
#pragma unroll
        for (int v = 0; v < NV; v++) {
          T k0 = h16 ? a[2][v] : a[0][v], k1 = h16 ? a[3][v] : a[1][v];
          k0 += __shfl_xor_sync(0xffffffffu, h16 ? a[0][v] : a[2][v], 16);
          k1 += __shfl_xor_sync(0xffffffffu, h16 ? a[1][v] : a[3][v], 16);
          T kp = h8 ? k1 : k0;
          kp += __shfl_xor_sync(0xffffffffu, h8 ? k0 : k1, 8);
          kp += __shfl_xor_sync(0xffffffffu, kp, 4);
          kp += __shfl_xor_sync(0xffffffffu, kp, 2);
          kp += __shfl_xor_sync(0xffffffffu, kp, 1);
          if ((lane & 7) == 0 && t < nt) acc[v * kTileT + t] += kp;
        }
      }
      ncomp = 0;
    };

    while (true) {
      // ---- plan and issue one fill (thread 0) -----------------------------------------
      if (tid == 0) {
        int r = s_cursor[0], p = s_cursor[1];
        int used = 0, np = 0, valid = 0;
        unsigned bytes = 0;
        while (r < nranges && np < kMaxPieces && C::kRaw - used >= 4) {
          int jx = jx0 + r % ncolx, jz = jz0 + r / ncolx;
          // (the FP64 kernel keeps no range table: with three weight vectors two CTAs per SM
          // fill the shared memory to within a few hundred bytes)
          int a = cs_s[cb + cell_of(g, jx, jy0, jz)], b = cs_s[cb + cell_of(g, jx, jy1, jz) + 1];
          int s = p < 0 ? a : p;
          if (s >= b) {
            r++;
            p = -1;
            continue;
          }
          int s_al = s & ~1;
          int room = (C::kRaw - used) & ~1;
          int e_al = min((b + 1) & ~1, s_al + room);
          int e = min(b, e_al);
          pieces[np].raw_off = used + (s - s_al);
          pieces[np].count = e - s;
          pieces[np].gstart = s;
          np++;
          valid += e - s;
          used += e_al - s_al;
          bytes += (unsigned)(e_al - s_al) * 8u * NA;
          if (e >= b) {
            r++;
            p = -1;
          } else {
            p = e;
          }
        }
        s_cursor[0] = r;
        s_cursor[1] = p;
        s_fill[0] = np;
        s_fill[1] = valid;
        s_fill[2] = (np == 0);
        if (np > 0) {
          fence_proxy_async_smem();
          mbar_expect_tx(bar, bytes);
          for (int q = 0; q < np; q++) {
            int s = pieces[q].gstart, s_al = s & ~1;
            int len = ((s + pieces[q].count + 1) & ~1) - s_al;
            int dst = pieces[q].raw_off - (s - s_al);
            bulk_g2s(raw + dst, sx + s_al, len * 8u, bar);
            bulk_g2s(raw + C::kRaw + dst, sy + s_al, len * 8u, bar);
            if (DIM == 3) bulk_g2s(raw + 2 * C::kRaw + dst, sz + s_al, len * 8u, bar);
#pragma unroll
            for (int v = 0; v < NV; v++)
              bulk_g2s(raw + (DIM + v) * C::kRaw + dst, sg + v * vstride + s_al, len * 8u, bar);
          }
        }
      }
      __syncthreads();
      if (s_fill[2]) break;
      if (!mbar_wait(bar, phase)) {
        if (tid == 0) {
          atomicOr(err, DEV_ERR_TIMEOUT);
          s_abort = 1;
        }
      }
      phase ^= 1u;
      __syncthreads();
      if (s_abort) {
        // let the copies of this fill land (bounded) before the CTA exits
        mbar_wait(bar, phase ^ 1u, 1u << 20);
        return;
      }
      // ---- make room, then filter + compact in order ----------------------------------
      if (ncomp + s_fill[1] > C::kComp) {
        flush();
        __syncthreads();
      }
      const int np = s_fill[0];
      for (int q = 0; q < np; q++) {
        const Piece pc = pieces[q];
        for (int e0 = 0; e0 < pc.count; e0 += kThreads) {
          int e = e0 + tid;
          bool in = false;
          double vx = 0, vy = 0, vz = 0;
          int ro = 0;
          if (e < pc.count) {
            int j = pc.gstart + e;
            ro = pc.raw_off + e;
            vx = raw[ro];
            vy = raw[C::kRaw + ro];
            if (DIM == 3) vz = raw[2 * C::kRaw + ro];
            // centre cell unconditionally (2d/get_trunc.h:31-39), neighbours by the box test
            // fabs(xj - xc) < trunc_length && ... (2d/get_trunc.h:63; 3d/get_trunc.h:70-72)
            bool boxin = fabs(vx - xc) < L && fabs(vy - yc) < L;
            if (DIM == 3) boxin = boxin && fabs(vz - zc) < L;
            in = (j >= c0 && j < c1) || boxin;
          }
          unsigned bal = __ballot_sync(0xffffffffu, in);
          if (lane == 0) s_wsum[wid] = __popc(bal);
          __syncthreads();
          int pre = 0, tot = 0;
#pragma unroll
          for (int k = 0; k < kWarps; k++) {
            int c = s_wsum[k];
            pre += k < wid ? c : 0;
            tot += c;
          }
          if (in) {
            int pos = ncomp + pre + __popc(bal & ((1u << lane) - 1u));
            comp[pos] = (T)((vx - xc) * scale);
            comp[C::kComp + pos] = (T)((vy - yc) * scale);
            if (DIM == 3) comp[2 * C::kComp + pos] = (T)((vz - zc) * scale);
#pragma unroll
            for (int v = 0; v < NV; v++) comp[(DIM + v) * C::kComp + pos] = (T)raw[(DIM + v) * C::kRaw + ro];
          }
          ncomp += tot;
          __syncthreads();
        }
      }
    }
    flush();
    __syncthreads();
    for (int t = tid; t < nt; t += kThreads)
#pragma unroll
      for (int v = 0; v < NV; v++) w[v * vstride + t0 + t] = (double)acc[v * kTileT + t] * kc.norm;
  }
}

// ---- FP32 form with precomputed source data ------------------------------------------
// Once per point set, for every source j of cell (jx, jy, jz): FP32 coordinates relative
// to its own cell centre, scaled (u, v, w), and a 64-bit word holding, per axis, bit k
// (k = 0 .. 2 nb) = the reference's FP64 box test |x_j - xc| < trunc_len against the
// centre of the target cell at offset k - nb from the source's cell (the same arithmetic
// as the FP64 kernel, so the truncation set is identical), and jy in the top 16 bits. The
// per-source filter is then integer work and the target-relative coordinate is
// u_j + (jx - ix) box scale, one FP32 add (the FP64 path rounds once from FP64 instead).
constexpr int kMaskBits = 15;    // 2 nb + 1 <= 15 bits per axis: nb_trunc <= 7
constexpr int kMaskY = kMaskBits, kMaskZ = 2 * kMaskBits, kMaskCellY = 48;
constexpr int kAlignF = 4;       // elements per 16 bytes (FP32 arrays; the masks use 2 x 16)

__global__ void k_src_f32(Grid g, const int* __restrict__ cs, const double* __restrict__ x,
                          const double* __restrict__ y, const double* __restrict__ z, double scale,
                          float* __restrict__ U, float* __restrict__ V, float* __restrict__ W,
                          unsigned long long* __restrict__ M) {
  const int nb = g.nb_trunc;
  const double L = g.trunc_len;
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < g.ncell; c += gridDim.x * blockDim.x) {
    int ix, iy, iz;
    cell_xyz(g, c, ix, iy, iz);
    const double xc = centre_coord(g.xmin, ix, g.box), yc = centre_coord(g.ymin, iy, g.box);
    const double zc = g.dim == 3 ? centre_coord(g.zmin, iz, g.box) : 0.0;
    for (int j = cs[c]; j < cs[c + 1]; j++) {
      unsigned long long m = (unsigned long long)iy << kMaskCellY;
      for (int k = 0; k <= 2 * nb; k++) {
        const int o = k - nb;  // source cell - target cell
        if (fabs(x[j] - centre_coord(g.xmin, ix - o, g.box)) < L) m |= 1ull << k;
        if (fabs(y[j] - centre_coord(g.ymin, iy - o, g.box)) < L) m |= 1ull << (kMaskY + k);
        if (g.dim == 3 && fabs(z[j] - centre_coord(g.zmin, iz - o, g.box)) < L) m |= 1ull << (kMaskZ + k);
      }
      U[j] = (float)((x[j] - xc) * scale);
      V[j] = (float)((y[j] - yc) * scale);
      if (g.dim == 3) W[j] = (float)((z[j] - zc) * scale);
      M[j] = m;
    }
  }
}

__global__ void k_to_f32(int n, int nv, long long vs_in, long long vs_out, const double* __restrict__ in,
                         float* __restrict__ out, const int* __restrict__ skip) {
  if (skip && *skip) return;
  for (int v = 0; v < nv; v++)
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
      out[v * vs_out + i] = (float)in[v * vs_in + i];
}

// The FP32 items are latency-bound on the fills (3D: 16 targets of a 2-sigma cell):
// smaller fills and compaction buffers let more CTAs share an SM (sizes timed on GB300:
// 3D 384/768 and 2D 512/1024 beat 1024/2048 by 9 % and 6 %).
template <int DIM, int NV>
struct LayoutF {
  static constexpr int NF = DIM + NV;  // FP32 staged arrays: coordinates + weights
  static constexpr int RC = DIM == 3 ? 384 : 512;      // staged sources per fill
  static constexpr int kComp = DIM == 3 ? 768 : 1024;  // compacted sources (>= RC)
  static_assert(kComp >= RC, "a fill must fit the compaction buffer");
  // a compacted source is one float4 (coordinates, then weights) and, when NF > 4, a
  // float2 or float4 with the remaining weights: two shared loads per source in the pair loop
  static constexpr int NX = NF <= 4 ? 0 : (NF <= 6 ? 2 : 4);
  static_assert(NF <= 8, "at most four weight vectors");
  static constexpr size_t rawf = 0;
  static constexpr size_t rawm = align16(rawf + sizeof(float) * NF * RC);
  static constexpr size_t comp = align16(rawm + sizeof(unsigned long long) * RC);  // float4 x kComp
  static constexpr size_t compx = align16(comp + sizeof(float) * 4 * kComp);        // NX floats x kComp
  static constexpr size_t tgt = align16(compx + sizeof(float) * NX * kComp);
  static constexpr size_t acc = align16(tgt + sizeof(float) * DIM * kTileT);
  static constexpr size_t pieces = align16(acc + sizeof(float) * NV * kTileT);
  static constexpr size_t bar = align16(pieces + sizeof(Piece) * kMaxPieces);
  static constexpr size_t total = bar + 16;
};

// BATCH: as k_gauss (the item's cell indexes a concatenation of grids); the source data
// of each problem were built with its own grid and scale.
template <int DIM, int NV, bool BATCH>
__global__ void __launch_bounds__(kThreads, 6) k_gauss_f32m(
    Grid g0, const Grid* __restrict__ grids, const int* __restrict__ cprob, SegSkip seg,
    const int2* __restrict__ items, int nitems, const double* __restrict__ tx, const double* __restrict__ ty,
    const double* __restrict__ tz, const int* __restrict__ cs_t, const float* __restrict__ su,
    const float* __restrict__ sv, const float* __restrict__ sw, const unsigned long long* __restrict__ smask,
    const float* __restrict__ sg, long long vs_g, const int* __restrict__ cs_s, double* __restrict__ w,
    long long vs_w, double scale0, double norm0, unsigned* err, const int* __restrict__ skip) {
  if (skip && *skip) return;
  using Lay = LayoutF<DIM, NV>;
  constexpr int NF = Lay::NF, RC = Lay::RC, NX = Lay::NX;
  extern __shared__ __align__(16) unsigned char smem[];
  float* rawf = (float*)(smem + Lay::rawf);                           // NF x RC
  unsigned long long* rawm = (unsigned long long*)(smem + Lay::rawm);  // RC
  float4* comp = (float4*)(smem + Lay::comp);                         // KC
  float* compx = (float*)(smem + Lay::compx);                         // KC x NX
  float* tgt = (float*)(smem + Lay::tgt);                             // DIM x kTileT
  float* acc = (float*)(smem + Lay::acc);                             // NV x kTileT
  constexpr int KC = Lay::kComp;
  Piece* pieces = (Piece*)(smem + Lay::pieces);
  uint64_t* bar = (uint64_t*)(smem + Lay::bar);
  __shared__ int s_wsum[kWarps];
  __shared__ int s_fill[3];
  __shared__ int s_cursor[2];
  __shared__ int s_abort;
  __shared__ int s_ra[kMaxRanges], s_rb[kMaxRanges];  // source ranges of the item's columns
  __shared__ int s_prange[kMaxPieces];  // range index of each piece

  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
  if (tid == 0) mbar_init(bar, 1);
  unsigned phase = 0;
  const int G = gridDim.x;

  for (int round = 0; (long long)round * G < nitems; round++) {
    const int it = (round & 1) ? round * G + (G - 1 - (int)blockIdx.x) : round * G + (int)blockIdx.x;
    if (it >= nitems) continue;
    const int2 item = items[it];
    const int ic = item.x, t0 = item.y;
    Grid g = g0;
    double scale = scale0, norm = norm0;
    if constexpr (BATCH) {
      if (seg.cell_done(ic)) continue;  // a stopped problem (uniform over the CTA)
      g = grids[cprob[ic]];
      const SumConsts k = sum_consts(g.sigma, true, 0);
      scale = k.scale;
      norm = k.norm;
    }
    const int cb = g.cbase;
    const float boxs = (float)(g.box * scale);
    const int nb = g.nb_trunc;
    const int nt = min(kTileT, cs_t[ic + 1] - t0);
    int ix, iy, iz;
    cell_xyz(g, ic - cb, ix, iy, iz);
    const double xc = centre_coord(g.xmin, ix, g.box);
    const double yc = centre_coord(g.ymin, iy, g.box);
    const double zc = DIM == 3 ? centre_coord(g.zmin, iz, g.box) : 0.0;
    const int c0 = cs_s[ic], c1 = cs_s[ic + 1];
    const int jx0 = max(0, ix - nb), jx1 = min(g.nx - 1, ix + nb);
    const int jy0 = max(0, iy - nb), jy1 = min(g.ny - 1, iy + nb);
    const int jz0 = DIM == 3 ? max(0, iz - nb) : 0, jz1 = DIM == 3 ? min(g.nz - 1, iz + nb) : 0;
    const int ncolx = jx1 - jx0 + 1;
    const int nranges = ncolx * (jz1 - jz0 + 1);

    __syncthreads();
    for (int r = tid; r < min(nranges, kMaxRanges); r += kThreads) {
      const int jx = jx0 + r % ncolx, jz = jz0 + r / ncolx;
      s_ra[r] = cs_s[cb + cell_of(g, jx, jy0, jz)];
      s_rb[r] = cs_s[cb + cell_of(g, jx, jy1, jz) + 1];
    }
    for (int t = tid; t < nt; t += kThreads) {
      tgt[t] = (float)((tx[t0 + t] - xc) * scale);
      tgt[kTileT + t] = (float)((ty[t0 + t] - yc) * scale);
      if (DIM == 3) tgt[2 * kTileT + t] = (float)((tz[t0 + t] - zc) * scale);
#pragma unroll
      for (int v = 0; v < NV; v++) acc[v * kTileT + t] = 0.f;
    }
    if (tid == 0) {
      s_cursor[0] = 0;
      s_cursor[1] = -1;
      s_abort = 0;
    }
    __syncthreads();

    int ncomp = 0;
    const int ngroups = (nt + kGroup - 1) / kGroup;
    auto flush = [&]() {
      for (int gi = wid; gi < ngroups; gi += kWarps) {
        float tu[kGroup], tv[kGroup], tw[kGroup], a[kGroup][NV];
#pragma unroll
        for (int k = 0; k < kGroup; k++) {
          int t = min(gi * kGroup + k, nt - 1);
          tu[k] = tgt[t];
          tv[k] = tgt[kTileT + t];
          tw[k] = DIM == 3 ? tgt[2 * kTileT + t] : 0.f;
#pragma unroll
          for (int v = 0; v < NV; v++) a[k][v] = 0.f;
        }
        for (int j = lane; j < ncomp; j += 32) {
          float rec[4 + NX];
          {
            const float4 c4 = comp[j];
            rec[0] = c4.x;
            rec[1] = c4.y;
            rec[2] = c4.z;
            rec[3] = c4.w;
            if constexpr (NX == 2) {
              const float2 c2 = reinterpret_cast<const float2*>(compx)[j];
              rec[4] = c2.x;
              rec[5] = c2.y;
            } else if constexpr (NX == 4) {
              const float4 c4b = reinterpret_cast<const float4*>(compx)[j];
              rec[4] = c4b.x;
              rec[5] = c4b.y;
              rec[6] = c4b.z;
              rec[7] = c4b.w;
            }
          }
          const float cu = rec[0], cv = rec[1], cw = DIM == 3 ? rec[2] : 0.f;
          float gj[NV];
#pragma unroll
          for (int v = 0; v < NV; v++) gj[v] = rec[DIM + v];
#pragma unroll
          for (int k = 0; k < kGroup; k++) {
            float du = tu[k] - cu, dv = tv[k] - cv;
            float d2 = fmaf(dv, dv, du * du);
            if (DIM == 3) {
              float dw = tw[k] - cw;
              d2 = fmaf(dw, dw, d2);
            }
            const float e = ex2_approx(-d2);
#pragma unroll
            for (int v = 0; v < NV; v++) a[k][v] = fmaf(gj[v], e, a[k][v]);
          }
        }
        // the four target sums over the warp by a butterfly that halves the values each lane
        // carries (6 shuffles per vector instead of 4 x 5): lane 8 k ends with target k
        static_assert(kGroup == 4, "reduce-scatter of four sums");
        const bool h16 = lane & 16, h8 = lane & 8;
        const int t = gi * kGroup + (lane >> 3);
#pragma unroll
        for (int v = 0; v < NV; v++) {
          float k0 = h16 ? a[2][v] : a[0][v], k1 = h16 ? a[3][v] : a[1][v];
          k0 += __shfl_xor_sync(0xffffffffu, h16 ? a[0][v] : a[2][v], 16);
          k1 += __shfl_xor_sync(0xffffffffu, h16 ? a[1][v] : a[3][v], 16);
          float kp = h8 ? k1 : k0;
          kp += __shfl_xor_sync(0xffffffffu, h8 ? k0 : k1, 8);
          kp += __shfl_xor_sync(0xffffffffu, kp, 4);
          kp += __shfl_xor_sync(0xffffffffu, kp, 2);
          kp += __shfl_xor_sync(0xffffffffu, kp, 1);
          if ((lane & 7) == 0 && t < nt) acc[v * kTileT + t] += kp;
        }
      }
      ncomp = 0;
    };

    while (true) {
      if (tid == 0) {
        int r = s_cursor[0], p = s_cursor[1];
        int used = 0, np = 0, valid = 0;
        unsigned bytes = 0;
        while (r < nranges && np < kMaxPieces && RC - used >= kAlignF) {
          int jx = jx0 + r % ncolx, jz = jz0 + r / ncolx;
          int a, b;
          if (r < kMaxRanges) {
            a = s_ra[r];
            b = s_rb[r];
          } else {
            a = cs_s[cb + cell_of(g, jx, jy0, jz)];
            b = cs_s[cb + cell_of(g, jx, jy1, jz) + 1];
          }
          int s = p < 0 ? a : p;
          if (s >= b) {
            r++;
            p = -1;
            continue;
          }
          int s_al = s & ~(kAlignF - 1);
          int room = (RC - used) & ~(kAlignF - 1);
          int e_al = min((b + kAlignF - 1) & ~(kAlignF - 1), s_al + room);
          int e = min(b, e_al);
          pieces[np].raw_off = used + (s - s_al);
          pieces[np].count = e - s;
          pieces[np].gstart = s;
          s_prange[np] = r;
          np++;
          valid += e - s;
          used += e_al - s_al;
          bytes += (unsigned)(e_al - s_al) * (4u * NF + 8u);
          if (e >= b) {
            r++;
            p = -1;
          } else {
            p = e;
          }
        }
        s_cursor[0] = r;
        s_cursor[1] = p;
        s_fill[0] = np;
        s_fill[1] = valid;
        s_fill[2] = (np == 0);
        if (np > 0) {
          fence_proxy_async_smem();
          mbar_expect_tx(bar, bytes);
          for (int q = 0; q < np; q++) {
            int s = pieces[q].gstart, s_al = s & ~(kAlignF - 1);
            int len = ((s + pieces[q].count + kAlignF - 1) & ~(kAlignF - 1)) - s_al;
            int dst = pieces[q].raw_off - (s - s_al);
            bulk_g2s(rawf + dst, su + s_al, len * 4u, bar);
            bulk_g2s(rawf + RC + dst, sv + s_al, len * 4u, bar);
            if (DIM == 3) bulk_g2s(rawf + 2 * RC + dst, sw + s_al, len * 4u, bar);
#pragma unroll
            for (int v = 0; v < NV; v++) bulk_g2s(rawf + (DIM + v) * RC + dst, sg + v * vs_g + s_al, len * 4u, bar);
            bulk_g2s(rawm + dst, smask + s_al, len * 8u, bar);
          }
        }
      }
      __syncthreads();
      if (s_fill[2]) break;
      if (!mbar_wait(bar, phase)) {
        if (tid == 0) {
          atomicOr(err, DEV_ERR_TIMEOUT);
          s_abort = 1;
        }
      }
      phase ^= 1u;
      __syncthreads();
      if (s_abort) {
        mbar_wait(bar, phase ^ 1u, 1u << 20);
        return;
      }
      if (ncomp + s_fill[1] > KC) {
        flush();
        __syncthreads();
      }
      const int np = s_fill[0];
      for (int q = 0; q < np; q++) {
        const Piece pc = pieces[q];
        const int r = s_prange[q];
        const int jx = jx0 + r % ncolx, jz = jz0 + r / ncolx;
        const int kx = jx - ix + nb, kz = jz - iz + nb;
        const float offx = (float)(jx - ix) * boxs, offz = (float)(jz - iz) * boxs;
        for (int e0 = 0; e0 < pc.count; e0 += kThreads) {
          int e = e0 + tid;
          bool in = false;
          int ro = 0;
          unsigned long long m = 0;
          if (e < pc.count) {
            const int j = pc.gstart + e;
            ro = pc.raw_off + e;
            m = rawm[ro];
            const int ky = (int)(m >> kMaskCellY) - iy + nb;
            bool boxin = ((m >> kx) & (m >> (kMaskY + ky)) & 1ull) != 0;
            if (DIM == 3) boxin = boxin && ((m >> (kMaskZ + kz)) & 1ull);
            // centre cell unconditionally (2d/get_trunc.h:31-39)
            in = (j >= c0 && j < c1) || boxin;
          }
          unsigned bal = __ballot_sync(0xffffffffu, in);
          if (lane == 0) s_wsum[wid] = __popc(bal);
          __syncthreads();
          int pre = 0, tot = 0;
#pragma unroll
          for (int k = 0; k < kWarps; k++) {
            int c = s_wsum[k];
            pre += k < wid ? c : 0;
            tot += c;
          }
          if (in) {
            int pos = ncomp + pre + __popc(bal & ((1u << lane) - 1u));
            const int jy = (int)(m >> kMaskCellY);
            float rec[4 + NX];
#pragma unroll
            for (int q = 0; q < 4 + NX; q++) rec[q] = 0.f;
            rec[0] = rawf[ro] + offx;
            rec[1] = rawf[RC + ro] + (float)(jy - iy) * boxs;
            if (DIM == 3) rec[2] = rawf[2 * RC + ro] + offz;
#pragma unroll
            for (int v = 0; v < NV; v++) rec[DIM + v] = rawf[(DIM + v) * RC + ro];
            comp[pos] = make_float4(rec[0], rec[1], rec[2], rec[3]);
            if constexpr (NX == 2)
              reinterpret_cast<float2*>(compx)[pos] = make_float2(rec[4], rec[5]);
            else if constexpr (NX == 4)
              reinterpret_cast<float4*>(compx)[pos] = make_float4(rec[4], rec[5], rec[6], rec[7]);
          }
          ncomp += tot;
          __syncthreads();
        }
      }
    }
    flush();
    __syncthreads();
    for (int t = tid; t < nt; t += kThreads)
#pragma unroll
      for (int v = 0; v < NV; v++)
        w[v * vs_w + t0 + t] = (double)acc[v * kTileT + t] * norm;
  }
}

// ---- FP64 matvec with each exponential used for both rows --------------------------
// When the targets are the sources (the matvec of the solve), the pair (i, j) enters row i
// when j is in T(c(i)) and row j when i is in T(c(j)), with the same exponential. One CTA
// per cell c1 (at most kTileT points): its own points against themselves (each pair once,
// both rows inside c1: the centre cell is taken unconditionally), then against the points
// of the upper half of
// its neighbour window -- the window cells with a larger cell index -- computing each
// exponential once and adding it to row i when j is in T(c1) (the FP64 box test against
// c1's centre, as the reference's) and to row j when i is in T(c(j)) (the target's box-test
// bits against the centres of the cells around its own, same arithmetic). Row j's share
// goes to the partial slot part[o][j], o the window offset of c(j) from c1 -- each slot is
// written by one CTA only -- and k_sym_gather adds the slots to the rows in a fixed order,
// zeroing them for the next product. Two ordered pairs cost 12 FP64 instructions in 2D
// (distance 4, exponential 6, two accumulations) against 2 x 11.
// Lanes own sources (SPL at a time), each warp walks all targets in groups of kGroup, and
// the per-target sums go to per-warp rows of shared memory that are added in warp order
// at the end: the result does not depend on scheduling. Every index the kernel forms for a
// global access is bounds-checked; an out-of-range one sets DEV_ERR_INDEX and is skipped.
constexpr int kSymRC = 512;   // staged sources per fill
constexpr int kSymMaxK = 32;  // partial slots per point and vector (upper window cells)

// NV weight vectors (right-hand sides) share each pair's exponential, as in k_gauss.
template <int DIM, int NV>
struct LayoutS {
  static constexpr int KC = NV == 1 ? 1024 : 768;  // compacted sources
  static constexpr int NA = DIM + NV + 1;  // staged arrays: coordinates, weights, cell-y word
  using ET = ExpTab<UseBigTabSym<DIM, NV>::v>;
  static constexpr size_t raw = 0;                                                     // NA x RC
  static constexpr size_t comp = align16(raw + sizeof(double) * NA * kSymRC);           // (DIM+NV) x KC
  static constexpr size_t code = align16(comp + sizeof(double) * (DIM + NV) * KC);      // KC
  static constexpr size_t jidx = align16(code + sizeof(int) * KC);                      // KC
  static constexpr size_t tgt = align16(jidx + sizeof(int) * KC);                       // (DIM+NV) x kTileT
  static constexpr size_t tmask = align16(tgt + sizeof(double) * (DIM + NV) * kTileT);  // kTileT
  static constexpr size_t acct = align16(tmask + sizeof(unsigned long long) * kTileT);  // kWarps x NV x kTileT
  static constexpr size_t tab = align16(acct + sizeof(double) * kWarps * NV * kTileT);
  static constexpr size_t pieces = align16(tab + sizeof(double) * ET::poly * ET::n);
  static constexpr size_t prange = align16(pieces + sizeof(Piece) * kMaxPieces);
  static constexpr size_t bar = align16(prange + sizeof(int) * kMaxPieces);
  static constexpr size_t total = bar + 16;
};

// Range r of c1's walk: 0 = c1 itself; 1 = the cells above c1 in its column; then the
// columns to its right (jy0 .. jy1) in its plane; then (3D) every column of the planes
// above. Sorted positions [a, b), cell offsets dx, dz from c1.
__device__ __forceinline__ void sym_range(const Grid& g, const int* __restrict__ cs, int ncs, int r, int c1, int ix,
                                          int iy, int iz, int jx0, int jx1, int jy0, int jy1, int& a, int& b, int& dx,
                                          int& dz) {
  const int cb = g.cbase;
  if (r == 0) {
    a = cs[c1];
    b = cs[c1 + 1];
    dx = dz = 0;
    return;
  }
  int cx, cz, y0;
  if (r == 1) {
    cx = ix;
    cz = iz;
    y0 = iy + 1;
  } else {
    const int r2 = r - 2, right = jx1 - ix;
    y0 = jy0;
    if (r2 < right) {
      cx = ix + 1 + r2;
      cz = iz;
    } else {
      const int ncolx = jx1 - jx0 + 1, r3 = r2 - right;
      cz = iz + 1 + r3 / ncolx;
      cx = jx0 + r3 % ncolx;
    }
  }
  dx = cx - ix;
  dz = cz - iz;
  const int ca = cb + cell_of(g, cx, y0, cz), ce = cb + cell_of(g, cx, jy1, cz) + 1;
  if (y0 > jy1 || ca < 0 || ce >= ncs) {  // (out-of-range cells: the caller's bounds check)
    a = b = y0 > jy1 ? 0 : -1;
    return;
  }
  a = cs[ca];
  b = cs[ce];
}

// BATCH: as k_gauss (the cell indexes a concatenation of grids, stopped problems skipped);
// every problem's window has the same K.
template <int DIM, int NV, bool BATCH>
__global__ void __launch_bounds__(kThreads) k_gauss_sym(
    Grid g0, const Grid* __restrict__ grids, const int* __restrict__ cprob, SegSkip seg,
    const int2* __restrict__ items, int nitems, const double* __restrict__ sx,
    const double* __restrict__ sy, const double* __restrict__ sz, const double* __restrict__ sg, long long vs,
    const unsigned long long* __restrict__ pcy, const int* __restrict__ cs, double* __restrict__ w,
    double* __restrict__ part, long long pstride, int K, int n, int ncs, SumConsts k0, unsigned* err,
    const int* __restrict__ skip) {
  if (skip && *skip) return;
  using Lay = LayoutS<DIM, NV>;
  using ET = typename Lay::ET;
  constexpr int NA = Lay::NA, RC = kSymRC, KC = Lay::KC;
  // sources per lane at a time: each group of kGroup targets ends in a warp reduction of
  // its kGroup x NV sums, amortised over SPL x kGroup pairs
  constexpr int SPL = NV == 1 ? 4 : 2;
  extern __shared__ __align__(16) unsigned char smem[];
  double* raw = (double*)(smem + Lay::raw);
  double* comp = (double*)(smem + Lay::comp);
  int* ccode = (int*)(smem + Lay::code);
  int* cj = (int*)(smem + Lay::jidx);
  double* tgt = (double*)(smem + Lay::tgt);
  unsigned long long* tmk = (unsigned long long*)(smem + Lay::tmask);
  double* acct = (double*)(smem + Lay::acct);
  double* tab = (double*)(smem + Lay::tab);
  Piece* pieces = (Piece*)(smem + Lay::pieces);
  int* prange = (int*)(smem + Lay::prange);
  uint64_t* bar = (uint64_t*)(smem + Lay::bar);
  __shared__ int s_wsum[kWarps];
  __shared__ int s_fill[3];
  __shared__ int s_cursor[2];
  __shared__ int s_abort;
  __shared__ unsigned long long s_tor;

  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
  for (int i = tid; i < ET::n * ET::poly; i += kThreads) tab[i] = (UseBigTabSym<DIM, NV>::v ? d_tab_big : d_tab_small)[i];
  if (tid == 0) mbar_init(bar, 1);
  unsigned phase = 0;
  const int G = gridDim.x;

  for (int round = 0; (long long)round * G < nitems; round++) {
    const int it = (round & 1) ? round * G + (G - 1 - (int)blockIdx.x) : round * G + (int)blockIdx.x;
    if (it >= nitems) continue;
    const int c1 = items[it].x, t0 = items[it].y;
    if (c1 < 0 || c1 + 1 >= ncs) {  // bounds check: record and skip the item
      if (threadIdx.x == 0) atomicOr(err, DEV_ERR_INDEX);
      continue;
    }
    Grid g = g0;
    SumConsts kc = k0;
    if constexpr (BATCH) {
      if (seg.cell_done(c1)) continue;  // a stopped problem (uniform over the CTA)
      g = grids[cprob[c1]];
      kc = sum_consts(g.sigma, false, ET::n);
    }
    const int nb = g.nb_trunc, W = 2 * nb + 1;
    const double L = g.trunc_len, kexp = kc.kexp;
    const int nt = min(kTileT, cs[c1 + 1] - t0);  // every cell has at most kTileT points here
    if (t0 < 0 || nt < 0 || t0 + nt > n) {  // bounds check: record and skip the item
      if (threadIdx.x == 0) atomicOr(err, DEV_ERR_INDEX);
      continue;
    }
    int ix, iy, iz;
    cell_xyz(g, c1 - g.cbase, ix, iy, iz);
    const double xc = centre_coord(g.xmin, ix, g.box);
    const double yc = centre_coord(g.ymin, iy, g.box);
    const double zc = DIM == 3 ? centre_coord(g.zmin, iz, g.box) : 0.0;
    const int jx0 = max(0, ix - nb), jx1 = min(g.nx - 1, ix + nb);
    const int jy0 = max(0, iy - nb), jy1 = min(g.ny - 1, iy + nb);
    const int jz1 = DIM == 3 ? min(g.nz - 1, iz + nb) : iz;
    const int nranges = 2 + (jx1 - ix) + (DIM == 3 ? (jz1 - iz) * (jx1 - jx0 + 1) : 0);

    __syncthreads();  // the previous item's readers are done
    if (tid == 0) s_tor = 0ull;
    __syncthreads();
    for (int t = tid; t < kTileT; t += kThreads) {
      double xt = 0.0, yt = 0.0, zt = 0.0, gt[NV];
#pragma unroll
      for (int v = 0; v < NV; v++) gt[v] = 0.0;
      unsigned long long m = 0ull;
      if (t < nt) {
        xt = sx[t0 + t];
        yt = sy[t0 + t];
        if (DIM == 3) zt = sz[t0 + t];
#pragma unroll
        for (int v = 0; v < NV; v++) gt[v] = sg[v * vs + t0 + t];
        // the reference's box test of this point against the centres of the cells at
        // offsets -nb .. nb of its own (2d/get_trunc.h:63): bit o + nb per axis
        for (int o = -nb; o <= nb; o++) {
          if (fabs(xt - centre_coord(g.xmin, ix + o, g.box)) < L) m |= 1ull << (o + nb);
          if (fabs(yt - centre_coord(g.ymin, iy + o, g.box)) < L) m |= 1ull << (kMaskY + o + nb);
          if (DIM == 3 && fabs(zt - centre_coord(g.zmin, iz + o, g.box)) < L) m |= 1ull << (kMaskZ + o + nb);
        }
        atomicOr(&s_tor, m);
      }
      tgt[t] = xt - xc;
      tgt[kTileT + t] = yt - yc;
      if (DIM == 3) tgt[2 * kTileT + t] = zt - zc;
#pragma unroll
      for (int v = 0; v < NV; v++) tgt[(DIM + v) * kTileT + t] = gt[v];  // zero in the padding slots
      tmk[t] = m;
#pragma unroll
      for (int q = 0; q < kWarps * NV; q++) acct[q * kTileT + t] = 0.0;
    }
    if (tid == 0) {
      s_cursor[0] = 0;
      s_cursor[1] = -1;
      s_abort = 0;
    }
    __syncthreads();
    const unsigned long long tor = s_tor;

    int ncomp = 0;
    const int ngroups = (nt + kGroup - 1) / kGroup;
    auto flush = [&]() {
      for (int s0 = wid * 32; s0 < ncomp; s0 += kWarps * 32 * SPL) {
        double px[SPL], py[SPL], pz[SPL], pg[SPL][NV], accs[SPL][NV];
        int kx[SPL], ky[SPL], kz[SPL], sidx[SPL], smax[SPL];
        bool self[SPL], valid[SPL];
#pragma unroll
        for (int m = 0; m < SPL; m++) {
          const int idx = s0 + lane + m * kWarps * 32;
          valid[m] = idx < ncomp;
          const int cd = valid[m] ? ccode[idx] : -1;
          self[m] = cd < 0;
          // c1's own points are compacted first, in order: source position idx is target
          // idx. Their pairs are taken once (idx >= t), both rows inside c1; a warp whose
          // own points all precede a group's targets skips that group.
          sidx[m] = idx;
          smax[m] = __reduce_max_sync(0xffffffffu, !valid[m] ? -1 : (self[m] ? idx : 0x7fffffff));
          kx[m] = cd & 255;
          ky[m] = kMaskY + ((cd >> 8) & 255);
          kz[m] = kMaskZ + ((cd >> 16) & 255);
          px[m] = valid[m] ? comp[idx] : 0.0;
          py[m] = valid[m] ? comp[KC + idx] : 0.0;
          pz[m] = (DIM == 3 && valid[m]) ? comp[2 * KC + idx] : 0.0;
#pragma unroll
          for (int v = 0; v < NV; v++) {
            pg[m][v] = valid[m] ? comp[(DIM + v) * KC + idx] : 0.0;
            accs[m][v] = 0.0;
          }
        }
        for (int gi = 0; gi < ngroups; gi++) {
          double tu[kGroup], tv[kGroup], tw[kGroup], tg[kGroup][NV], a[kGroup][NV];
          unsigned long long tm[kGroup];
#pragma unroll
          for (int k = 0; k < kGroup; k++) {
            const int t = gi * kGroup + k;  // < kTileT: the padding slots carry zeros
            tu[k] = tgt[t];
            tv[k] = tgt[kTileT + t];
            tw[k] = DIM == 3 ? tgt[2 * kTileT + t] : 0.0;
#pragma unroll
            for (int v = 0; v < NV; v++) {
              tg[k][v] = tgt[(DIM + v) * kTileT + t];
              a[k][v] = 0.0;
            }
            tm[k] = tmk[t];
          }
#pragma unroll
          for (int m = 0; m < SPL; m++) {
            if (smax[m] < gi * kGroup) continue;
#pragma unroll
            for (int k = 0; k < kGroup; k++) {
              const int t = gi * kGroup + k;
              const double du = tu[k] - px[m], dv = tv[k] - py[m];
              double d2 = du * du;
              d2 = fma(dv, dv, d2);
              if (DIM == 3) {
                const double dw = tw[k] - pz[m];
                d2 = fma(dw, dw, d2);
              }
              const double magic = 6755399441055744.0;  // 1.5 * 2^52 (see k_gauss)
              const double kd = fma(d2, kexp, magic);
              const int kk = __double2loint(kd);
              const double r = fma(-d2, kexp, kd - magic);
              const int j8 = kk & (ET::n - 1);
              const int m20 = min(kk >> ET::bits, 900) << 20;
              double q;
              if constexpr (ET::poly == 4) {
                const double2 c01 = *(const double2*)(tab + 4 * j8);
                const double2 c23 = *(const double2*)(tab + 4 * j8 + 2);
                q = hi_sub(c23.y, m20);
                q = fma(r, q, hi_sub(c23.x, m20));
                q = fma(r, q, hi_sub(c01.y, m20));
                q = fma(r, q, hi_sub(c01.x, m20));
              } else {
                const double* cjt = tab + ET::poly * j8;
                q = hi_sub(cjt[ET::poly - 1], m20);
#pragma unroll
                for (int i = ET::poly - 2; i >= 0; i--) q = fma(r, q, hi_sub(cjt[i], m20));
              }
              // row i (pg = 0 unless j is in T(c1)); own points: the pair once, idx >= t
              const bool use_i = !self[m] || sidx[m] >= t;
#pragma unroll
              for (int v = 0; v < NV; v++) a[k][v] = fma(use_i ? pg[m][v] : 0.0, q, a[k][v]);
              // row j: target i in T(c(j)) -- its bits at c(j)'s offset -- or, for an own
              // point, the other row of the pair (idx > t)
              unsigned long long bit = (tm[k] >> kx[m]) & (tm[k] >> ky[m]);
              if (DIM == 3) bit &= tm[k] >> kz[m];
              const bool use_j = self[m] ? sidx[m] > t : (bit & 1ull) != 0;
#pragma unroll
              for (int v = 0; v < NV; v++) accs[m][v] = fma(use_j ? tg[k][v] : 0.0, q, accs[m][v]);
            }
          }
          // the four target sums over the warp by a butterfly that halves the values each
          // lane carries (6 FP64 adds per lane instead of 4 x 5): lane 8 k ends with target k
          static_assert(kGroup == 4, "reduce-scatter of four sums");
          const bool h16 = lane & 16, h8 = lane & 8;
          const int t = gi * kGroup + (lane >> 3);
#pragma unroll
          for (int v = 0; v < NV; v++) {
            double k0 = h16 ? a[2][v] : a[0][v], k1 = h16 ? a[3][v] : a[1][v];
            k0 += __shfl_xor_sync(0xffffffffu, h16 ? a[0][v] : a[2][v], 16);
            k1 += __shfl_xor_sync(0xffffffffu, h16 ? a[1][v] : a[3][v], 16);
            double kp = h8 ? k1 : k0;
            kp += __shfl_xor_sync(0xffffffffu, h8 ? k0 : k1, 8);
            kp += __shfl_xor_sync(0xffffffffu, kp, 4);
            kp += __shfl_xor_sync(0xffffffffu, kp, 2);
            kp += __shfl_xor_sync(0xffffffffu, kp, 1);
            if ((lane & 7) == 0 && t < nt) acct[(wid * NV + v) * kTileT + t] += kp;
          }
        }
        __syncwarp();  // the group sums' writes to this warp's row come first
#pragma unroll
        for (int m = 0; m < SPL; m++) {
          const int idx = s0 + lane + m * kWarps * 32;
          if (valid[m] && self[m]) {  // row idx of c1 itself
            if (idx < nt) {
#pragma unroll
              for (int v = 0; v < NV; v++) acct[(wid * NV + v) * kTileT + idx] += accs[m][v];
            } else {
              atomicOr(err, DEV_ERR_INDEX);
            }
          }
          if (valid[m] && !self[m]) {
            const int ddx = kx[m] - nb, ddy = ky[m] - kMaskY - nb, ddz = DIM == 3 ? kz[m] - kMaskZ - nb : 0;
            const int key = (ddz * W + ddx) * W + ddy;  // > 0 for the upper half of the window
            const int jj = cj[idx];
            if (key >= 1 && key <= K && jj >= 0 && jj < n) {
#pragma unroll
              for (int v = 0; v < NV; v++)
                part[((long long)v * K + key - 1) * pstride + jj] = accs[m][v] * kc.norm;
            } else {
              atomicOr(err, DEV_ERR_INDEX);
            }
          }
        }
        __syncwarp();
      }
      ncomp = 0;
    };

    while (true) {
      // ---- plan and issue one fill (thread 0) -----------------------------------------
      if (tid == 0) {
        int r = s_cursor[0], p = s_cursor[1];
        int used = 0, np = 0, valid = 0;
        unsigned bytes = 0;
        while (r < nranges && np < kMaxPieces && RC - used >= 4) {
          int a, b, ddx, ddz;
          sym_range(g, cs, ncs, r, c1, ix, iy, iz, jx0, jx1, jy0, jy1, a, b, ddx, ddz);
          if (a < 0 || b > n || a > b) {  // bounds check: record and skip the range
            atomicOr(err, DEV_ERR_INDEX);
            a = b = 0;
          }
          int s = p < 0 ? a : p;
          if (s >= b) {
            r++;
            p = -1;
            continue;
          }
          int s_al = s & ~1;
          int room = (RC - used) & ~1;
          int e_al = min((b + 1) & ~1, s_al + room);
          int e = min(b, e_al);
          pieces[np].raw_off = used + (s - s_al);
          pieces[np].count = e - s;
          pieces[np].gstart = s;
          prange[np] = r;
          np++;
          valid += e - s;
          used += e_al - s_al;
          bytes += (unsigned)(e_al - s_al) * 8u * NA;
          if (e >= b) {
            r++;
            p = -1;
          } else {
            p = e;
          }
        }
        s_cursor[0] = r;
        s_cursor[1] = p;
        s_fill[0] = np;
        s_fill[1] = valid;
        s_fill[2] = (np == 0);
        if (np > 0) {
          fence_proxy_async_smem();
          mbar_expect_tx(bar, bytes);
          for (int q = 0; q < np; q++) {
            int s = pieces[q].gstart, s_al = s & ~1;
            int len = ((s + pieces[q].count + 1) & ~1) - s_al;
            int dst = pieces[q].raw_off - (s - s_al);
            bulk_g2s(raw + dst, sx + s_al, len * 8u, bar);
            bulk_g2s(raw + RC + dst, sy + s_al, len * 8u, bar);
            if (DIM == 3) bulk_g2s(raw + 2 * RC + dst, sz + s_al, len * 8u, bar);
#pragma unroll
            for (int v = 0; v < NV; v++) bulk_g2s(raw + (DIM + v) * RC + dst, sg + v * vs + s_al, len * 8u, bar);
            bulk_g2s(raw + (DIM + NV) * RC + dst, pcy + s_al, len * 8u, bar);
          }
        }
      }
      __syncthreads();
      if (s_fill[2]) break;
      if (!mbar_wait(bar, phase)) {
        if (tid == 0) {
          atomicOr(err, DEV_ERR_TIMEOUT);
          s_abort = 1;
        }
      }
      phase ^= 1u;
      __syncthreads();
      if (s_abort) {
        mbar_wait(bar, phase ^ 1u, 1u << 20);
        return;
      }
      if (ncomp + s_fill[1] > KC) {
        flush();
        __syncthreads();
      }
      const int np = s_fill[0];
      for (int q = 0; q < np; q++) {
        const Piece pc = pieces[q];
        const int r = prange[q];
        int a_, b_, ddx, ddz;
        sym_range(g, cs, ncs, r, c1, ix, iy, iz, jx0, jx1, jy0, jy1, a_, b_, ddx, ddz);
        for (int e0 = 0; e0 < pc.count; e0 += kThreads) {
          const int e = e0 + tid;
          bool in = false;
          double vx = 0, vy = 0, vz = 0, vg[NV];
#pragma unroll
          for (int v = 0; v < NV; v++) vg[v] = 0.0;
          int code = -1, j = 0;
          if (e < pc.count) {
            j = pc.gstart + e;
            const int ro = pc.raw_off + e;
            vx = raw[ro];
            vy = raw[RC + ro];
            if (DIM == 3) vz = raw[2 * RC + ro];
#pragma unroll
            for (int v = 0; v < NV; v++) vg[v] = raw[(DIM + v) * RC + ro];
            if (r == 0) {
              in = true;  // the centre cell, unconditionally (2d/get_trunc.h:31-39)
            } else {
              const int ddy = (int)__double_as_longlong(raw[(DIM + NV) * RC + ro]) - iy;
              // (the planes above a 3D cell take every column of the window: dx may be negative)
              if (ddy < -nb || ddy > nb || ddx < -nb || ddx > nb || ddz < 0 || ddz > nb) atomicOr(err, DEV_ERR_INDEX);
              // j in T(c1): the box test against c1's centre (2d/get_trunc.h:63)
              bool fij = fabs(vx - xc) < L && fabs(vy - yc) < L;
              if (DIM == 3) fij = fij && fabs(vz - zc) < L;
              // some target of c1 may lie in T(c(j)): keep the source for row j
              unsigned long long pb = (tor >> (ddx + nb)) & (tor >> (kMaskY + ddy + nb));
              if (DIM == 3) pb &= tor >> (kMaskZ + ddz + nb);
              in = fij || (pb & 1ull);
              if (!fij)
#pragma unroll
                for (int v = 0; v < NV; v++) vg[v] = 0.0;
              code = (ddx + nb) | ((ddy + nb) << 8) | ((ddz + nb) << 16);
            }
          }
          unsigned bal = __ballot_sync(0xffffffffu, in);
          if (lane == 0) s_wsum[wid] = __popc(bal);
          __syncthreads();
          int pre = 0, tot = 0;
#pragma unroll
          for (int k = 0; k < kWarps; k++) {
            const int c = s_wsum[k];
            pre += k < wid ? c : 0;
            tot += c;
          }
          if (in) {
            const int pos = ncomp + pre + __popc(bal & ((1u << lane) - 1u));
            comp[pos] = vx - xc;
            comp[KC + pos] = vy - yc;
            if (DIM == 3) comp[2 * KC + pos] = vz - zc;
#pragma unroll
            for (int v = 0; v < NV; v++) comp[(DIM + v) * KC + pos] = vg[v];
            ccode[pos] = code;
            cj[pos] = j;
          }
          ncomp += tot;
          __syncthreads();
        }
      }
    }
    flush();
    __syncthreads();
    for (int t = tid; t < nt; t += kThreads)
#pragma unroll
      for (int v = 0; v < NV; v++) {
        double s = 0.0;
#pragma unroll
        for (int q = 0; q < kWarps; q++) s += acct[(q * NV + v) * kTileT + t];
        w[v * vs + t0 + t] = s * kc.norm;
      }
  }
}

// Rows += their partial slots (offset order), slots back to zero for the next product.
__global__ void k_sym_gather(int n, int nv, int K, long long pstride, double* __restrict__ part,
                             double* __restrict__ w, long long vs, const int* __restrict__ skip) {
  if (skip && *skip) return;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    for (int v = 0; v < nv; v++) {
      double s = 0.0;
      for (int o = 0; o < K; o++) {
        double* slot = part + ((long long)v * K + o) * pstride + i;
        const double x = *slot;
        if (__double_as_longlong(x) != 0) {  // an integer test: the FP64 pipe is for the sums
          s += x;
          *slot = 0.0;
        }
      }
      w[v * vs + i] += s;
    }
}

// Cell y index of every sorted point (the symmetric sum's per-source cell), as 64-bit words.
__global__ void k_cell_y(Grid g, const int* __restrict__ cs, unsigned long long* __restrict__ out) {
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < g.ncell; c += gridDim.x * blockDim.x) {
    int ix, iy, iz;
    cell_xyz(g, c, ix, iy, iz);
    for (int j = cs[c]; j < cs[c + 1]; j++) out[j] = (unsigned long long)iy;
  }
}

__global__ void k_max_cell(int ncell, const int* __restrict__ cs, int* __restrict__ out) {
  int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c < ncell) atomicMax(out, cs[c + 1] - cs[c]);
}

// ---- work list and truncation-set sizes ----------------------------------------------
__global__ void k_item_counts(int ncell, const int* __restrict__ cs_t, int* __restrict__ cnt) {
  int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c < ncell) cnt[c] = (cs_t[c + 1] - cs_t[c] + kTileT - 1) / kTileT;
}

__global__ void k_item_fill(int ncell, const int* __restrict__ cs_t, const int* __restrict__ off,
                            int2* __restrict__ items) {
  int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= ncell) return;
  int a = cs_t[c], b = cs_t[c + 1], o = off[c];
  for (int t = a; t < b; t += kTileT) items[o++] = make_int2(c, t);
}

// One warp per target cell: size of its truncation set (0 for an empty target cell,
// 2d/get_trunc.h:76-78); accumulates the pair count and the maximum.
__global__ void k_trunc_count(Grid g, const int* __restrict__ cs_t, const double* __restrict__ sx,
                              const double* __restrict__ sy, const double* __restrict__ sz,
                              const int* __restrict__ cs_s, int* __restrict__ cnt,
                              unsigned long long* __restrict__ pairs, int* __restrict__ maxc) {
  int c = blockIdx.x * (blockDim.x / 32) + (threadIdx.x >> 5);
  int lane = threadIdx.x & 31;
  if (c >= g.ncell) return;
  int ntg = cs_t[c + 1] - cs_t[c];
  if (ntg == 0) {
    if (lane == 0) cnt[c] = 0;
    return;
  }
  int ix, iy, iz;
  cell_xyz(g, c, ix, iy, iz);
  double xc = centre_coord(g.xmin, ix, g.box), yc = centre_coord(g.ymin, iy, g.box);
  double zc = g.dim == 3 ? centre_coord(g.zmin, iz, g.box) : 0.0;
  double L = g.trunc_len;
  int nb = g.nb_trunc;
  int jx0 = max(0, ix - nb), jx1 = min(g.nx - 1, ix + nb);
  int jy0 = max(0, iy - nb), jy1 = min(g.ny - 1, iy + nb);
  int jz0 = g.dim == 3 ? max(0, iz - nb) : 0, jz1 = g.dim == 3 ? min(g.nz - 1, iz + nb) : 0;
  int c0 = cs_s[c], c1 = cs_s[c + 1];
  int n = 0;
  for (int jz = jz0; jz <= jz1; jz++)
    for (int jx = jx0; jx <= jx1; jx++) {
      int a = cs_s[cell_of(g, jx, jy0, jz)], b = cs_s[cell_of(g, jx, jy1, jz) + 1];
      for (int j = a + lane; j < b; j += 32) {
        bool in = fabs(sx[j] - xc) < L && fabs(sy[j] - yc) < L;
        if (g.dim == 3) in = in && fabs(sz[j] - zc) < L;
        n += ((j >= c0 && j < c1) || in) ? 1 : 0;
      }
    }
  for (int o = 16; o > 0; o >>= 1) n += __shfl_xor_sync(0xffffffffu, n, o);
  if (lane == 0) {
    cnt[c] = n;
    atomicAdd(pairs, (unsigned long long)n * (unsigned long long)ntg);
    atomicMax(maxc, n);
  }
}

bool g_tab_ready[64] = {false};

void upload_table(cudaStream_t s) {
  int dev = 0;
  PRBF_CUDA(cudaGetDevice(&dev));
  if (dev < 64 && g_tab_ready[dev]) return;
  // Large table: c_i = monomial coefficients of the cubic through (r_k, e^(L r_k)) at the
  // Chebyshev nodes r_k = cos((2k+1) pi / 8) / 2 (Newton divided differences, then
  // expanded), in long double; small table: c_i = L^i / i!. Then T[j] = 2^(-j/n) and the
  // folded coefficients T[j] c_i.
  static double h2[ExpTab<true>::n * ExpTab<true>::poly], h3[ExpTab<false>::n * ExpTab<false>::poly];
  const long double PI = 3.141592653589793238462643383279502884L;
  {
    constexpr int NP = ExpTab<true>::poly, NT = ExpTab<true>::n;
    const long double L = logl(2.0L) / NT;
    long double xr[NP], dd[NP], c[NP];
    for (int k = 0; k < NP; k++) {
      xr[k] = 0.5L * cosl((2 * k + 1) * PI / (2 * NP));
      dd[k] = expl(L * xr[k]);
      c[k] = 0.0L;
    }
    for (int lev = 1; lev < NP; lev++)
      for (int k = NP - 1; k >= lev; k--) dd[k] = (dd[k] - dd[k - 1]) / (xr[k] - xr[k - lev]);
    for (int k = NP - 1; k >= 0; k--) {  // Newton form -> monomials (Horner)
      for (int i = NP - 1; i > 0; i--) c[i] = c[i - 1] - xr[k] * c[i];
      c[0] = dd[k] - xr[k] * c[0];
    }
    for (int j = 0; j < NT; j++) {
      long double t = exp2l(-(long double)j / NT);
      for (int i = 0; i < NP; i++) h2[j * NP + i] = (double)(t * c[i]);
    }
  }
  {
    constexpr int NP = ExpTab<false>::poly, NT = ExpTab<false>::n;
    const long double L = logl(2.0L) / NT;
    for (int j = 0; j < NT; j++) {
      long double t = exp2l(-(long double)j / NT), f = 1.0L, lp = 1.0L;
      for (int i = 0; i < NP; i++) {
        h3[j * NP + i] = (double)(t * lp / f);
        lp *= L;
        f *= (long double)(i + 1);
      }
    }
  }
  PRBF_CUDA(cudaMemcpyToSymbolAsync(d_tab_big, h2, sizeof(h2), 0, cudaMemcpyHostToDevice, s));
  PRBF_CUDA(cudaMemcpyToSymbolAsync(d_tab_small, h3, sizeof(h3), 0, cudaMemcpyHostToDevice, s));
  PRBF_CUDA(cudaStreamSynchronize(s));
  if (dev < 64) g_tab_ready[dev] = true;
}

template <int DIM, bool F32, int NV>
size_t smem_bytes() {
  return Layout<DIM, F32, NV>::total;
}

template <int DIM, bool F32, int NV, bool BATCH>
void launch(const GaussPlan& P, const PointsView& t, const PointsView& s, const double* gv, double* w,
            long long vstride, unsigned* err, const int* skip, cudaStream_t st) {
  size_t sm = smem_bytes<DIM, F32, NV>();
  static_assert(Layout<DIM, F32, NV>::total <= 227 * 1024, "k_gauss shared memory");
  static std::atomic<bool> attr_set[64];  // per device: attribute set (idempotent, thread-safe)
  int dev = 0;
  PRBF_CUDA(cudaGetDevice(&dev));
  if (dev >= 64 || !attr_set[dev]) {
    PRBF_CUDA(
        cudaFuncSetAttribute(k_gauss<DIM, F32, NV, BATCH>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
    if (dev < 64) attr_set[dev] = true;
  }
  // FP32: coordinates scaled so that |dx|^2 is the exponent in units of ln2 (exp2).
  // FP64: unscaled cell-relative coordinates; kexp = n / (2 sigma^2 ln2) converts |dx|^2
  // to units of ln2/n (n the exp table size) inside the fused range reduction.
  const SumConsts k0 = sum_consts(P.g.sigma, F32, ExpTab<UseBigTab<DIM, NV>::v>::n);
  const int grid = P.grid > 0 ? std::min(P.grid, P.nitems) : P.nitems;
  k_gauss<DIM, F32, NV, BATCH><<<grid, kThreads, sm, st>>>(P.g, P.grids.get(), P.cprob.get(), P.items.get(), P.nitems,
                                                           t.x, t.y, t.z, t.cell_start, s.x, s.y, s.z, gv,
                                                           s.cell_start, w, vstride, k0, P.seg, err, skip);
  PRBF_CHECK_LAUNCH();
}

template <int DIM, int NV, bool BATCH>
void launch_sym_k(const GaussPlan& P, const PointsView& s, const double* gv, double* w, long long vs, unsigned* err,
                  const int* skip, cudaStream_t st) {
  constexpr size_t sm = LayoutS<DIM, NV>::total;
  static_assert(sm <= 227 * 1024, "k_gauss_sym shared memory");
  static std::atomic<bool> attr_set[64];  // per device: attribute set (idempotent, thread-safe)
  int dev = 0;
  PRBF_CUDA(cudaGetDevice(&dev));
  if (dev >= 64 || !attr_set[dev]) {
    PRBF_CUDA(
        cudaFuncSetAttribute(k_gauss_sym<DIM, NV, BATCH>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
    if (dev < 64) attr_set[dev] = true;
  }
  const SumConsts k0 = sum_consts(P.g.sigma, false, LayoutS<DIM, NV>::ET::n);
  // one item per cell: the plan's own items (cells within one tile) or, for a batch, its
  // per-cell list
  const int2* it = P.sym_nitems > 0 ? P.sym_items.get() : P.items.get();
  const int nit = P.sym_nitems > 0 ? P.sym_nitems : P.nitems;
  const int grid = P.sym_nitems > 0 ? nit : (P.grid > 0 ? std::min(P.grid, nit) : nit);
  k_gauss_sym<DIM, NV, BATCH><<<grid, kThreads, sm, st>>>(P.g, P.grids.get(), P.cprob.get(), P.seg, it, nit, s.x,
                                                          s.y, s.z, gv, vs, P.sym_cy.get(), s.cell_start, w,
                                                          P.sym_part.get(), P.sym_pstride, P.sym_K, s.n,
                                                          P.sym_ncs > 0 ? P.sym_ncs : P.g.ncell + 1, k0, err, skip);
  PRBF_CHECK_LAUNCH();
}

template <int DIM, int NV>
void launch_sym(const GaussPlan& P, const PointsView& s, const double* gv, double* w, long long vs, unsigned* err,
                const int* skip, cudaStream_t st) {
  if (P.batched)
    launch_sym_k<DIM, NV, true>(P, s, gv, w, vs, err, skip, st);
  else
    launch_sym_k<DIM, NV, false>(P, s, gv, w, vs, err, skip, st);
  const int gb = std::max(1, std::min(ceil_div(s.n, 256), 8 * 152));
  k_sym_gather<<<gb, 256, 0, st>>>(s.n, NV, P.sym_K, P.sym_pstride, P.sym_part.get(), w, vs, skip);
  PRBF_CHECK_LAUNCH();
}

template <int DIM>
void launch_sym_nv(const GaussPlan& P, const PointsView& s, const double* gv, double* w, int nv, long long vs,
                   unsigned* err, const int* skip, cudaStream_t st) {
  for (int v0 = 0; v0 < nv; v0 += 4) {
    const double* g0 = gv + v0 * vs;
    double* w0 = w + v0 * vs;
    switch (std::min(4, nv - v0)) {
      case 1: launch_sym<DIM, 1>(P, s, g0, w0, vs, err, skip, st); break;
      case 2: launch_sym<DIM, 2>(P, s, g0, w0, vs, err, skip, st); break;
      case 3: launch_sym<DIM, 3>(P, s, g0, w0, vs, err, skip, st); break;
      default: launch_sym<DIM, 4>(P, s, g0, w0, vs, err, skip, st); break;
    }
  }
}

template <int DIM, int NV, bool BATCH>
void launch_f32m(const GaussPlan& P, const PointsView& t, const PointsView& s, const double* gv, double* w,
                 long long vstride, unsigned* err, const int* skip, cudaStream_t st) {
  constexpr size_t sm = LayoutF<DIM, NV>::total;
  static_assert(sm <= 227 * 1024, "k_gauss_f32m shared memory");
  static std::atomic<bool> attr_set[64];  // per device: attribute set (idempotent, thread-safe)
  int dev = 0;
  PRBF_CUDA(cudaGetDevice(&dev));
  if (dev >= 64 || !attr_set[dev]) {
    PRBF_CUDA(cudaFuncSetAttribute(k_gauss_f32m<DIM, NV, BATCH>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   (int)sm));
    if (dev < 64) attr_set[dev] = true;
  }
  const SumConsts k0 = sum_consts(P.g.sigma, true, 0);
  k_to_f32<<<4 * 152, 256, 0, st>>>(s.n, NV, vstride, P.g32_stride, gv, P.g32.get(), skip);
  PRBF_CHECK_LAUNCH();
  const int grid = P.grid > 0 ? std::min(P.grid, P.nitems) : P.nitems;
  k_gauss_f32m<DIM, NV, BATCH><<<grid, kThreads, sm, st>>>(
      P.g, P.grids.get(), P.cprob.get(), P.seg, P.items.get(), P.nitems, t.x, t.y, t.z, t.cell_start, P.su.get(),
      P.sv.get(), P.sw.get(), P.smask.get(), P.g32.get(), P.g32_stride, s.cell_start, w, vstride, k0.scale, k0.norm,
      err, skip);
  PRBF_CHECK_LAUNCH();
}

template <int DIM, bool F32>
void launch_nv(const GaussPlan& P, const PointsView& t, const PointsView& s, const double* gv, double* w, int nv,
               long long vstride, unsigned* err, const int* skip, cudaStream_t st) {
  if (F32 && P.f32_ready && P.batched) {
    for (int v = 0; v < nv; v++)
      launch_f32m<DIM, 1, true>(P, t, s, gv + v * vstride, w + v * vstride, vstride, err, skip, st);
    return;
  }
  if (F32 && P.f32_ready) {
    for (int v0 = 0; v0 < nv; v0 += 4) {
      const double* g0 = gv + v0 * vstride;
      double* w0 = w + v0 * vstride;
      switch (std::min(4, nv - v0)) {
        case 1: launch_f32m<DIM, 1, false>(P, t, s, g0, w0, vstride, err, skip, st); break;
        case 2: launch_f32m<DIM, 2, false>(P, t, s, g0, w0, vstride, err, skip, st); break;
        case 3: launch_f32m<DIM, 3, false>(P, t, s, g0, w0, vstride, err, skip, st); break;
        default: launch_f32m<DIM, 4, false>(P, t, s, g0, w0, vstride, err, skip, st); break;
      }
    }
    return;
  }
  if (P.batched) {  // a batch of problems: the problems are the segments of one vector
    for (int v = 0; v < nv; v++) launch<DIM, F32, 1, true>(P, t, s, gv + v * vstride, w + v * vstride, vstride, err, skip, st);
    return;
  }
  for (int v0 = 0; v0 < nv; v0 += 4) {
    const double* g0 = gv + v0 * vstride;
    double* w0 = w + v0 * vstride;
    switch (std::min(4, nv - v0)) {
      case 1: launch<DIM, F32, 1, false>(P, t, s, g0, w0, vstride, err, skip, st); break;
      case 2: launch<DIM, F32, 2, false>(P, t, s, g0, w0, vstride, err, skip, st); break;
      case 3: launch<DIM, F32, 3, false>(P, t, s, g0, w0, vstride, err, skip, st); break;
      default: launch<DIM, F32, 4, false>(P, t, s, g0, w0, vstride, err, skip, st); break;
    }
  }
}

}  // namespace

// The FP32 form's masks hold 2 nb_trunc + 1 bits per axis and the cell y in 16 bits.
static bool f32_grid_ok(const Grid& g) { return 2 * g.nb_trunc + 1 <= kMaskBits && g.ny < 65536; }

static void alloc_f32(GaussPlan& plan, int dim, int n, cudaStream_t s) {
  const long long n8 = (long long)n + 8;
  plan.su.reserve(n8);
  plan.sv.reserve(n8);
  plan.sw.reserve(dim == 3 ? n8 : 1);
  plan.smask.reserve(n8);
  plan.g32_stride = ((long long)n + 8 + 31) / 32 * 32;
  plan.g32.reserve(4 * plan.g32_stride);
  PRBF_CUDA(cudaMemsetAsync(plan.g32.get(), 0, sizeof(float) * 4 * plan.g32_stride, s));
  for (auto* b : {&plan.su, &plan.sv}) PRBF_CUDA(cudaMemsetAsync(b->get(), 0, sizeof(float) * n8, s));
  if (dim == 3) PRBF_CUDA(cudaMemsetAsync(plan.sw.get(), 0, sizeof(float) * n8, s));
  PRBF_CUDA(cudaMemsetAsync(plan.smask.get(), 0, sizeof(unsigned long long) * n8, s));
}

void gauss_plan_dev(GaussPlan& plan, const PointsView& tgt, const PointsView& src, unsigned* err,
                    Workspace& ws, cudaStream_t s, bool forms) {
  (void)err;
  const Grid& g = plan.g;
  int* cnt = (int*)ws.get(20, sizeof(int) * ((size_t)g.ncell + 1));
  k_item_counts<<<ceil_div(g.ncell, 256), 256, 0, s>>>(g.ncell, tgt.cell_start, cnt);
  PRBF_CHECK_LAUNCH();
  PRBF_CUDA(cudaMemsetAsync(cnt + g.ncell, 0, sizeof(int), s));
  scan_exclusive_dev(cnt, cnt, (long long)g.ncell + 1, ws, 21, s);
  int nitems = 0;
  PRBF_CUDA(cudaMemcpyAsync(&nitems, cnt + g.ncell, sizeof(int), cudaMemcpyDeviceToHost, s));
  PRBF_CUDA(cudaStreamSynchronize(s));
  plan.nitems = nitems;
  plan.items.reserve(std::max(nitems, 1));
  k_item_fill<<<ceil_div(g.ncell, 256), 256, 0, s>>>(g.ncell, tgt.cell_start, cnt, plan.items.get());
  PRBF_CHECK_LAUNCH();
  plan.trunc_cnt.reserve(g.ncell);
  struct {
    unsigned long long pairs;
    int maxc;
    int pad;
  } h{0, 0, 0};
  void* d = ws.get(24, sizeof(h));
  PRBF_CUDA(cudaMemsetAsync(d, 0, sizeof(h), s));
  k_trunc_count<<<ceil_div(g.ncell, 8), 256, 0, s>>>(g, tgt.cell_start, src.x, src.y, src.z,
                                                     src.cell_start, plan.trunc_cnt.get(),
                                                     (unsigned long long*)d, (int*)((char*)d + 8));
  PRBF_CHECK_LAUNCH();
  PRBF_CUDA(cudaMemcpyAsync(&h, d, sizeof(h), cudaMemcpyDeviceToHost, s));
  PRBF_CUDA(cudaStreamSynchronize(s));
  plan.pairs = (long long)h.pairs;
  plan.max_trunc = h.maxc;
  plan.max_tile = kTileT;
  upload_table(s);
  // FP32 form's source data
  plan.f32_ready = false;
  plan.sym_ready = false;
  plan.sym_nitems = 0;
  plan.sym_ncs = 0;
  if (!forms) return;
  if (f32_grid_ok(g) && src.n > 0) {
    alloc_f32(plan, g.dim, src.n, s);
    const SumConsts k32 = sum_consts(g.sigma, true, 0);
    k_src_f32<<<ceil_div(g.ncell, 128), 128, 0, s>>>(g, src.cell_start, src.x, src.y, src.z, k32.scale,
                                                     plan.su.get(), plan.sv.get(), plan.sw.get(), plan.smask.get());
    PRBF_CHECK_LAUNCH();
    plan.f32_ready = true;
  }
  // symmetric FP64 matvec: the same point set on both sides, every cell within one item
  // (<= kTileT points), 2 nb + 1 mask bits per axis, at most kSymMaxK partial slots per
  // point and vector (each product writes and gathers them: the 7 x 7 x 7 window of a 3D
  // cutoff of 2.8 cells has 171, whose traffic costs more than the halved exponentials
  // save), and the slots within 1/8 of the free device memory
  if (tgt.x == src.x && tgt.n == src.n && src.n > 0 && 2 * g.nb_trunc + 1 <= kMaskBits && (g.dim == 2 || g.dim == 3)) {
    int* dmax = (int*)ws.get(25, sizeof(int));
    PRBF_CUDA(cudaMemsetAsync(dmax, 0, sizeof(int), s));
    k_max_cell<<<ceil_div(g.ncell, 256), 256, 0, s>>>(g.ncell, src.cell_start, dmax);
    PRBF_CHECK_LAUNCH();
    int hmax = 0;
    PRBF_CUDA(cudaMemcpyAsync(&hmax, dmax, sizeof(int), cudaMemcpyDeviceToHost, s));
    PRBF_CUDA(cudaStreamSynchronize(s));
    const int W = 2 * g.nb_trunc + 1;
    const int K = g.dim == 2 ? (W * W - 1) / 2 : (W * W * W - 1) / 2;
    const long long pstride = ((long long)src.n + 8 + 31) / 32 * 32;
    size_t free_b = 0, total_b = 0;
    PRBF_CUDA(cudaMemGetInfo(&free_b, &total_b));
    const int nvs = std::max(1, std::min(4, plan.sym_nv));
    const double bytes = (double)K * nvs * pstride * sizeof(double) + (double)(src.n + 8) * 8;
    if (hmax <= kTileT && K >= 1 && K <= kSymMaxK && bytes <= 0.125 * (double)free_b) {
      plan.sym_K = K;
      plan.sym_nv = nvs;
      plan.sym_pstride = pstride;
      plan.sym_part.reserve((size_t)K * nvs * pstride);
      PRBF_CUDA(cudaMemsetAsync(plan.sym_part.get(), 0, sizeof(double) * (size_t)K * nvs * pstride, s));
      plan.sym_cy.reserve((size_t)src.n + 8);
      PRBF_CUDA(cudaMemsetAsync(plan.sym_cy.get(), 0, sizeof(unsigned long long) * ((size_t)src.n + 8), s));
      k_cell_y<<<std::max(1, std::min(ceil_div(g.ncell, 256), 8 * 152)), 256, 0, s>>>(g, src.cell_start,
                                                                                   plan.sym_cy.get());
      PRBF_CHECK_LAUNCH();
      plan.sym_ready = true;
    }
  }
}

bool gauss_plan_sym_batch(GaussPlan& plan, const std::vector<Grid>& grids, const PointsView& src,
                          const std::vector<int>& hcs, cudaStream_t s) {
  plan.sym_ready = false;
  plan.sym_nitems = 0;
  if (grids.empty() || src.n <= 0) return false;
  const int nb = grids[0].nb_trunc, dim = grids[0].dim;
  for (const Grid& g : grids)
    if (g.nb_trunc != nb || 2 * nb + 1 > kMaskBits) return false;
  const int W = 2 * nb + 1;
  const int K = dim == 2 ? (W * W - 1) / 2 : (W * W * W - 1) / 2;
  if (K < 1 || K > kSymMaxK) return false;
  // one item per non-empty cell, each cell within one item; largest first
  std::vector<int2> its;
  const int ncell = (int)hcs.size() - 1;
  for (int c = 0; c < ncell; c++) {
    const int m = hcs[c + 1] - hcs[c];
    if (m > kTileT) return false;
    if (m > 0) its.push_back(make_int2(c, hcs[c]));
  }
  std::stable_sort(its.begin(), its.end(),
                   [&](const int2& a, const int2& b) { return hcs[a.x + 1] - hcs[a.x] > hcs[b.x + 1] - hcs[b.x]; });
  const long long pstride = ((long long)src.n + 8 + 31) / 32 * 32;
  size_t free_b = 0, total_b = 0;
  PRBF_CUDA(cudaMemGetInfo(&free_b, &total_b));
  if ((double)K * pstride * sizeof(double) + (double)(src.n + 8) * 8 > 0.125 * (double)free_b) return false;
  plan.sym_K = K;
  plan.sym_nv = 1;
  plan.sym_ncs = (int)hcs.size();
  plan.sym_pstride = pstride;
  plan.sym_part.reserve((size_t)K * pstride);
  PRBF_CUDA(cudaMemsetAsync(plan.sym_part.get(), 0, sizeof(double) * (size_t)K * pstride, s));
  plan.sym_cy.reserve((size_t)src.n + 8);
  PRBF_CUDA(cudaMemsetAsync(plan.sym_cy.get(), 0, sizeof(unsigned long long) * ((size_t)src.n + 8), s));
  for (const Grid& g : grids)
    k_cell_y<<<std::max(1, std::min(ceil_div(g.ncell, 256), 8 * 152)), 256, 0, s>>>(g, src.cell_start + g.cbase,
                                                                                  plan.sym_cy.get());
  PRBF_CHECK_LAUNCH();
  plan.sym_items.reserve(std::max<size_t>(its.size(), 1));
  PRBF_CUDA(cudaMemcpyAsync(plan.sym_items.get(), its.data(), sizeof(int2) * its.size(), cudaMemcpyHostToDevice, s));
  PRBF_CUDA(cudaStreamSynchronize(s));
  plan.sym_nitems = (int)its.size();
  plan.sym_ready = true;
  return true;
}

void gauss_plan_f32_batch(GaussPlan& plan, const std::vector<Grid>& grids, const PointsView& src, cudaStream_t s) {
  plan.f32_ready = false;
  if (src.n <= 0) return;
  for (const Grid& g : grids)
    if (!f32_grid_ok(g)) return;
  alloc_f32(plan, grids[0].dim, src.n, s);
  for (const Grid& g : grids) {
    // the problem's cells are cell_start[cbase .. cbase + ncell]; its points keep their
    // global positions
    const SumConsts k32 = sum_consts(g.sigma, true, 0);
    k_src_f32<<<ceil_div(g.ncell, 128), 128, 0, s>>>(g, src.cell_start + g.cbase, src.x, src.y, src.z, k32.scale,
                                                     plan.su.get(), plan.sv.get(), plan.sw.get(), plan.smask.get());
    PRBF_CHECK_LAUNCH();
  }
  plan.f32_ready = true;
}

void gauss_sum_dev(const GaussPlan& P, const PointsView& t, const PointsView& s, const double* gv,
                   double* w, bool fp32, unsigned* err, cudaStream_t st, const int* skip, int nv,
                   long long vstride) {
  if (P.nitems == 0 || nv <= 0) return;
  if (nv > 1 && (vstride % 2 || vstride < t.n || vstride < s.n))
    throw Error(PRBF_ERR_ARG, "vector stride must be even and cover the points");
  if (!fp32 && P.sym_ready && std::min(nv, 4) <= P.sym_nv && t.x == s.x && t.n == s.n) {
    if (P.g.dim == 2)
      launch_sym_nv<2>(P, s, gv, w, nv, vstride, err, skip, st);
    else
      launch_sym_nv<3>(P, s, gv, w, nv, vstride, err, skip, st);
    return;
  }
  if (P.g.dim == 2) {
    if (fp32)
      launch_nv<2, true>(P, t, s, gv, w, nv, vstride, err, skip, st);
    else
      launch_nv<2, false>(P, t, s, gv, w, nv, vstride, err, skip, st);
  } else {
    if (fp32)
      launch_nv<3, true>(P, t, s, gv, w, nv, vstride, err, skip, st);
    else
      launch_nv<3, false>(P, t, s, gv, w, nv, vstride, err, skip, st);
  }
}

const double* exp_table_dev(cudaStream_t s) {
  static std::atomic<const double*> addr[64];
  int dev = 0;
  PRBF_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 64) throw Error(PRBF_ERR_CUDA, "device index beyond the table cache");
  upload_table(s);
  const double* p = addr[dev].load();
  if (!p) {
    void* q = nullptr;
    PRBF_CUDA(cudaGetSymbolAddress(&q, d_tab_big));
    p = (const double*)q;
    addr[dev].store(p);
  }
  return p;
}

}  // namespace prbf
