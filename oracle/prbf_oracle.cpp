/*
 * prbf_oracle.cpp -- TEST INFRASTRUCTURE ONLY (checker and timed CPU baseline).
 *
 * Plain C++ restatement of PetRBF's solve path. Every function names the reference
 * file:line (paths inside the petrbf project) that it restates. Built with
 * -ffp-contract=off so that each floating-point expression is evaluated exactly as
 * written in the reference (no fused multiply-add), which makes cell membership and
 * the truncation/buffer box tests bit-reproducible.
 *
 * Not product code: only tests/, bench.py (cpu_baseline / --impl reference) and
 * __graft_entry__.smoke() load this library, and only as the checker.
 *
 * What pins it: the cell sort, truncation and buffer sets, dense blocks, matvec and
 * evaluation agree bit for bit with the reference's own code compiled here against a
 * sequential PETSc/MPI stand-in (tests/test_oracle.py on the fixtures of tests/golden).
 * GMRES, PCASM and the dense LU live in PETSc, a third-party "developer version" that the
 * reference does not vendor or pin: they are restated from PETSc's documented defaults,
 * and for them parity is unpinned (no golden vector of iterations or residual histories;
 * converged answers are pinned through true residuals and converged weights).
 */
#include "prbf_oracle.h"

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <mutex>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

const double kEpsf = 1e-6;  // 2d/par.h:153

enum {
  OK = 0,
  ERR_ARG = 1,
  ERR_RANGE = 2,
  ERR_SINGULAR = 3,
};

// PETSc KSPConvergedReason values used for the solve status.
enum {
  CONVERGED_RTOL = 2,
  CONVERGED_ATOL = 3,
  DIVERGED_ITS = -3,
  DIVERGED_DTOL = -4,
  DIVERGED_BREAKDOWN = -5,
  DIVERGED_NANORINF = -9,
};

inline void cell_coords(const orc_grid* g, int ic, int* ix, int* iy, int* iz) {
  if (g->dim == 2) {
    *ix = ic / g->ny;
    *iy = ic % g->ny;
    *iz = 0;
  } else {
    int nxy = g->nx * g->ny;
    *iz = ic / nxy;
    int rem = ic % nxy;
    *ix = rem / g->ny;
    *iy = rem % g->ny;
  }
}

// Cell linear index: 2d/get_cluster.h:80 (ix*ny+iy), 3d/get_cluster.h:101 (iz*nx*ny+ix*ny+iy).
inline int cell_index(const orc_grid* g, int ix, int iy, int iz) {
  if (g->dim == 2) return ix * g->ny + iy;
  return iz * g->nx * g->ny + ix * g->ny + iy;
}

// Cell centre: 2d/get_cluster.h:217-218, 3d/get_cluster.h:79-81.
inline void cell_centre(const orc_grid* g, int ix, int iy, int iz, double* xc, double* yc,
                        double* zc) {
  *xc = g->xmin + (ix + 0.5) * g->box;
  *yc = g->ymin + (iy + 0.5) * g->box;
  *zc = g->dim == 3 ? g->zmin + (iz + 0.5) * g->box : 0.0;
}

inline int point_cell(const orc_grid* g, double x, double y, double z) {
  // 2d/get_cluster.h:234-236 ; 3d/get_cluster.h:98-101
  int ix = (int)floor((x - g->xmin) / g->box);
  int iy = (int)floor((y - g->ymin) / g->box);
  int iz = 0;
  if (g->dim == 3) iz = (int)floor((z - g->zmin) / g->box);
  if (ix < 0 || ix >= g->nx || iy < 0 || iy >= g->ny || iz < 0 ||
      (g->dim == 3 && iz >= g->nz))
    return -1;
  return cell_index(g, ix, iy, iz);
}

// Neighbour-cell walk shared by get_trunc and get_buffer: centre first, then the
// neighbour cells in jx, jy (, jz) order, skipping the centre
// (2d/get_trunc.h:23-73, 2d/get_buffer.h:13-77, 3d twins).
template <class F>
void walk_neighbours(const orc_grid* g, int ic, int nb, F&& visit_cell) {
  int ix, iy, iz;
  cell_coords(g, ic, &ix, &iy, &iz);
  int jx0 = std::max(0, ix - nb), jx1 = std::min(g->nx - 1, ix + nb);
  int jy0 = std::max(0, iy - nb), jy1 = std::min(g->ny - 1, iy + nb);
  int jz0 = 0, jz1 = 0;
  if (g->dim == 3) {
    jz0 = std::max(0, iz - nb);
    jz1 = std::min(g->nz - 1, iz + nb);
  }
  for (int jx = jx0; jx <= jx1; jx++)
    for (int jy = jy0; jy <= jy1; jy++)
      for (int jz = jz0; jz <= jz1; jz++) {
        if (g->dim == 2) {
          if (ix != jx || iy != jy) visit_cell(cell_index(g, jx, jy, 0));
        } else {
          if (ix != jx || iy != jy || iz != jz) visit_cell(cell_index(g, jx, jy, jz));
        }
      }
}

// Truncation set of target cell ic as indices into the sorted source arrays
// (2d/get_trunc.h:9-78; 3d/get_trunc.h:9-90).
int trunc_set(const orc_grid* g, int ic, const double* sx, const double* sy,
              const double* sz, const int* cs_src, const int* cs_tgt, int* out) {
  if (cs_tgt[ic] >= cs_tgt[ic + 1]) return 0;  // empty target cell: nptruncj = 0
  int ix, iy, iz;
  cell_coords(g, ic, &ix, &iy, &iz);
  double xc, yc, zc;
  cell_centre(g, ix, iy, iz, &xc, &yc, &zc);
  int n = 0;
  for (int j = cs_src[ic]; j < cs_src[ic + 1]; j++) {
    if (out) out[n] = j;
    n++;
  }
  const double L = g->trunc_len;
  walk_neighbours(g, ic, g->nb_trunc, [&](int jc) {
    for (int j = cs_src[jc]; j < cs_src[jc + 1]; j++) {
      bool in = fabs(sx[j] - xc) < L && fabs(sy[j] - yc) < L;
      if (g->dim == 3) in = in && fabs(sz[j] - zc) < L;
      if (in) {
        if (out) out[n] = j;
        n++;
      }
    }
  });
  return n;
}

// Buffer (RASM subdomain) of cell ic, centre points first (2d/get_buffer.h:9-77).
int buffer_set(const orc_grid* g, int ic, const double* x, const double* y, const double* z,
               const int* cs, int* out) {
  if (cs[ic] >= cs[ic + 1]) return 0;
  int ix, iy, iz;
  cell_coords(g, ic, &ix, &iy, &iz);
  double xc, yc, zc;
  cell_centre(g, ix, iy, iz, &xc, &yc, &zc);
  int n = 0;
  for (int j = cs[ic]; j < cs[ic + 1]; j++) {
    if (out) out[n] = j;
    n++;
  }
  const double L = g->buffer_len;
  walk_neighbours(g, ic, g->nb_buffer, [&](int jc) {
    for (int j = cs[jc]; j < cs[jc + 1]; j++) {
      bool in = fabs(x[j] - xc) < L && fabs(y[j] - yc) < L;
      if (g->dim == 3) in = in && fabs(z[j] - zc) < L;
      if (in) {
        if (out) out[n] = j;
        n++;
      }
    }
  });
  return n;
}

// Kernel entry phi(|xi-xj|) exactly as written in 2d/matmult.cxx:39-40 / 83-93
// (3d/matmult.cxx:40-41): exp(-r^2/(2 sigma^2)) / (2 pi sigma^2), 2D normalisation in 3D.
inline double phi(double sigma, double dx, double dy, double dz, int dim) {
  double r2 = dim == 3 ? dx * dx + dy * dy + dz * dz : dx * dx + dy * dy;
  return exp(-(r2) / (2 * sigma * sigma)) / (2 * M_PI * sigma * sigma);
}

// ---------------------------------------------------------------------------------------
// The GPU library's FP64 arithmetic for the Schwarz blocks, restated (the "chol" form).
// The reference factors each block with PETSc's dense LU; the GPU library instead takes the
// Cholesky factor of K = 2 pi sigma^2 A_c with the block's neighbour points first and its
// centre points last, evaluates exp with its own table, and applies the factor by
// substitutions in a fixed operation order. Restating that arithmetic here lets a test
// compare the GPU's factors bit for bit and run GMRES with the same preconditioner, so the
// two Krylov histories differ only by the rounding of the Gaussian sums and the dots.
// ---------------------------------------------------------------------------------------

// exp table of n = 1024 entries: tab[4 j + i] = 2^(-j/n) c_i, c_i the monomial coefficients
// of the cubic through (r_k, e^(L r_k)) at the Chebyshev nodes r_k = cos((2k+1) pi/8) / 2
// of [-1/2, 1/2], L = ln2/n (Newton divided differences, expanded), in long double.
const double* exp_table() {
  static double tab[4096];
  static std::once_flag once;
  std::call_once(once, [] {
    const int NP = 4, NT = 1024;
    const long double PI = 3.141592653589793238462643383279502884L;
    const long double L = logl(2.0L) / NT;
    long double xr[NP], dd[NP], c[NP];
    for (int k = 0; k < NP; k++) {
      xr[k] = 0.5L * cosl((2 * k + 1) * PI / (2 * NP));
      dd[k] = expl(L * xr[k]);
      c[k] = 0.0L;
    }
    for (int lev = 1; lev < NP; lev++)
      for (int k = NP - 1; k >= lev; k--) dd[k] = (dd[k] - dd[k - 1]) / (xr[k] - xr[k - lev]);
    for (int k = NP - 1; k >= 0; k--) {
      for (int i = NP - 1; i > 0; i--) c[i] = c[i - 1] - xr[k] * c[i];
      c[0] = dd[k] - xr[k] * c[0];
    }
    for (int j = 0; j < NT; j++) {
      long double t = exp2l(-(long double)j / NT);
      for (int i = 0; i < NP; i++) tab[j * NP + i] = (double)(t * c[i]);
    }
  });
  return tab;
}

inline double kexp_of_sigma(double sigma) { return 1024.0 / (2.0 * sigma * sigma * 0.6931471805599453); }

inline double pow2_lower(double v, int m) {  // v * 2^-m by the exponent field
  uint64_t b;
  memcpy(&b, &v, 8);
  b -= (uint64_t)m << 52;
  memcpy(&v, &b, 8);
  return v;
}

// exp(-d2 / (2 sigma^2)), kexp = kexp_of_sigma(sigma): k = rint(kexp d2) by the 1.5 * 2^52
// addition, r = k - kexp d2 in one rounding, k = 1024 m + j, 2^-m T[j] p(r) by Horner
// (m capped at 900).
inline double exp_neg_tab(double d2, double kexp) {
  const double* tab = exp_table();
  const double magic = 6755399441055744.0;
  const double kd = std::fma(d2, kexp, magic);
  uint64_t b;
  memcpy(&b, &kd, 8);
  const int kk = (int)(uint32_t)(b & 0xffffffffu);
  const double r = std::fma(-d2, kexp, kd - magic);
  const int m = std::min(kk >> 10, 900);
  const double* c = tab + 4 * (kk & 1023);
  double q = pow2_lower(c[3], m);
  q = std::fma(r, q, pow2_lower(c[2], m));
  q = std::fma(r, q, pow2_lower(c[1], m));
  q = std::fma(r, q, pow2_lower(c[0], m));
  return q;
}

// Buffer-list entry of block row i: neighbours (entries nc ..) first, then the centre.
inline int gpu_row(int i, int nb, int nc) { return i < nb - nc ? nc + i : i - (nb - nc); }

// K[i][j], j <= i, of the block whose buffer list (centre first) is id: the differences
// as the reference forms them, |d|^2 = fma(dy, dy, dx dx) (+ fma(dz, dz, .)), the table
// exp, plus shift on the diagonal. Row-major nb x nb, lower triangle written.
void gpu_block_K(int dim, int nb, int nc, const int* id, const double* x, const double* y,
                 const double* z, double kexp, double shift, double* K) {
  for (int i = 0; i < nb; i++) {
    const int a = id[gpu_row(i, nb, nc)];
    for (int j = 0; j <= i; j++) {
      const int b = id[gpu_row(j, nb, nc)];
      const double dx = x[a] - x[b], dy = y[a] - y[b];
      double r2 = std::fma(dy, dy, dx * dx);
      if (dim == 3) {
        const double dz = z[a] - z[b];
        r2 = std::fma(dz, dz, r2);
      }
      double v = exp_neg_tab(r2, kexp);
      if (i == j) v = v + shift;
      K[(size_t)i * nb + j] = v;
    }
  }
}

// Unblocked right-looking Cholesky of K (lower, row-major) in the GPU's operation order:
// pivot column j: s = sqrt(a_jj) (a non-positive pivot is taken as 1 and reported),
// r = 1/s, l_ij = a_ij * r, then a_il = fma(-l_ij, l_lj, a_il) for j < l <= i. Every
// entry thus receives fma updates for the columns before its own in ascending order and
// is then scaled. This loop is the definition; chol_blocked below computes the same
// operations per entry faster. The work array U is the transpose (U[j][i] = L[i][j]).
bool chol_unblocked(int n, const double* K, double* U, double* L) {
  for (int i = 0; i < n; i++)
    for (int j = 0; j <= i; j++) U[(size_t)j * n + i] = K[(size_t)i * n + j];
  bool ok = true;
  for (int j = 0; j < n; j++) {
    double* uj = U + (size_t)j * n;
    double d = uj[j];
    if (!(d > 0.0)) {
      ok = false;
      d = 1.0;
    }
    const double sq = sqrt(d), rc = 1.0 / sq;
    uj[j] = sq;
    for (int i = j + 1; i < n; i++) uj[i] = uj[i] * rc;
    for (int l = j + 1; l < n; l++) {
      double* ul = U + (size_t)l * n;
      const double f = uj[l];
      for (int i = l; i < n; i++) ul[i] = std::fma(-f, uj[i], ul[i]);
    }
  }
  for (int i = 0; i < n; i++)
    for (int j = 0; j <= i; j++) L[(size_t)i * n + j] = U[(size_t)j * n + i];
  return ok;
}

// The same Cholesky, right-looking over panels of 16 columns, on the transposed work array
// U (U[j][i] = L[i][j], row-major): the panel's columns are factored in order, each
// updating the panel's later rows at once; then every row below the panel takes the
// panel's 16 updates in ascending order while it sits in cache (each update one
// vectorised pass over the row). Per entry this is chol_unblocked's operation sequence,
// so the factors are bit-identical; the trailing rows are read once per panel instead of
// once per column. Reads K's lower triangle; writes U.
bool chol_blocked(int n, const double* K, double* U) {
  for (int i = 0; i < n; i++)
    for (int j = 0; j <= i; j++) U[(size_t)j * n + i] = K[(size_t)i * n + j];
  bool ok = true;
  const int P = 16;
  for (int j0 = 0; j0 < n; j0 += P) {
    const int j1 = std::min(n, j0 + P);
    for (int j = j0; j < j1; j++) {
      double* uj = U + (size_t)j * n;
      double d = uj[j];
      if (!(d > 0.0)) {
        ok = false;
        d = 1.0;
      }
      const double sq = sqrt(d), rc = 1.0 / sq;
      uj[j] = sq;
      for (int i = j + 1; i < n; i++) uj[i] = uj[i] * rc;
      for (int l = j + 1; l < j1; l++) {
        double* ul = U + (size_t)l * n;
        const double f = uj[l];
        for (int i = l; i < n; i++) ul[i] = std::fma(-f, uj[i], ul[i]);
      }
    }
    for (int l = j1; l < n; l++) {
      double* ul = U + (size_t)l * n;
      for (int j = j0; j < j1; j++) {
        const double* uj = U + (size_t)j * n;
        const double f = uj[l];
        for (int i = l; i < n; i++) ul[i] = std::fma(-f, uj[i], ul[i]);
      }
    }
  }
  return ok;
}

// Factor of the block K (lower, row-major) packed as the apply reads it: row i =
// L_A[i][0..i-1] followed by 1 / L_A[i][i], L_A = L_K * sc the factor of A = K / (2 pi
// sigma^2). U: n x n scratch. Returns false on a non-positive pivot.
bool gpu_chol_pack(int n, const double* K, double sc, double* U, double* Lp) {
  const bool ok = chol_blocked(n, K, U);
  for (int i = 0; i < n; i++) {
    double* row = Lp + (size_t)i * (i + 1) / 2;
    for (int j = 0; j < i; j++) row[j] = U[(size_t)j * n + i] * sc;
    row[i] = 1.0 / (U[(size_t)i * n + i] * sc);
  }
  return ok;
}

// The GPU apply's substitutions on one block vector y (block order), packed factor Lp:
// forward over the whole block in 32-row panels (inside a panel, y_i receives
// fma(-l_ij, y_j, .) for ascending j and is then multiplied by the reciprocal pivot; a row
// below the panel subtracts ((a0 + a1) + (a2 + a3)), a_s the fma chain over 8 entries of
// the panel from zero), then the back substitution over rows b0 .. nb-1 in 32-row panels
// from the bottom (inside a panel descending; a row above a panel subtracts the fma chain
// over the panel's entries from zero).
void gpu_tri_apply(int nb, int b0, const double* Lp, double* y) {
  auto L = [&](long long i, long long j) { return Lp[i * (i + 1) / 2 + j]; };
  for (int p0 = 0; p0 < nb; p0 += 32) {
    const int np = std::min(32, nb - p0);
    for (int i = p0; i < p0 + np; i++) {
      double v = y[i];
      for (int j = p0; j < i; j++) v = std::fma(-L(i, j), y[j], v);
      y[i] = v * L(i, i);
    }
    for (int i = p0 + np; i < nb; i++) {
      double a[4];
      for (int sb = 0; sb < 4; sb++) {
        double t = 0.0;
        for (int q = 0; q < 8; q++) t = std::fma(L(i, p0 + 8 * sb + q), y[p0 + 8 * sb + q], t);
        a[sb] = t;
      }
      y[i] = y[i] - ((a[0] + a[1]) + (a[2] + a[3]));
    }
  }
  const int nback = nb - b0;
  for (int pe = nback; pe > 0; pe -= 32) {
    const int p0 = std::max(0, pe - 32), np = pe - p0;
    const int o = b0 + p0;
    for (int i = np - 1; i >= 0; i--) {
      double v = y[o + i];
      for (int j = np - 1; j > i; j--) v = std::fma(-L(o + j, o + i), y[o + j], v);
      y[o + i] = v * L(o + i, o + i);
    }
    for (int k = 0; k < p0; k++) {
      double acc = 0.0;
      for (int j = 0; j < np; j++) acc = std::fma(L(o + j, b0 + k), y[o + j], acc);
      y[b0 + k] = y[b0 + k] - acc;
    }
  }
}

// The GPU library's LU fallback for a block whose ordered Cholesky meets a non-positive
// pivot (PETSc's -sub_pc_type lu semantics on its blocks, restated in its arithmetic): K
// mirrored to a full matrix, then LU with partial pivoting -- pivot the first row of
// largest |a_ik|, full rows swapped, l_ik = a_ik / a_kk, a_ij = fma(-l_ik, a_kj, a_ij).
// Returns false on an exactly zero pivot (where PETSc's LU stops).
bool gpu_lu_factor(int n, double* A, int* piv) {
  for (int i = 0; i < n; i++)
    for (int j = i + 1; j < n; j++) A[(size_t)i * n + j] = A[(size_t)j * n + i];
  for (int k = 0; k < n; k++) {
    int p = k;
    double amax = fabs(A[(size_t)k * n + k]);
    for (int i = k + 1; i < n; i++) {
      const double v = fabs(A[(size_t)i * n + k]);
      if (v > amax) {
        amax = v;
        p = i;
      }
    }
    piv[k] = p;
    if (amax == 0.0) return false;
    if (p != k)
      for (int j = 0; j < n; j++) std::swap(A[(size_t)k * n + j], A[(size_t)p * n + j]);
    const double d = A[(size_t)k * n + k];
    for (int i = k + 1; i < n; i++) {
      double* ri = A + (size_t)i * n;
      const double l = ri[k] / d;
      ri[k] = l;
      const double* rk = A + (size_t)k * n;
      for (int j = k + 1; j < n; j++) ri[j] = std::fma(-l, rk[j], ri[j]);
    }
  }
  return true;
}

// Its solve, y <- scale * K^-1 y in the GPU's per-entry order: the row interchanges in
// order, forward (unit lower) with fma over ascending columns, backward with fma over
// descending columns and a division by the pivot, then the scale (2 pi sigma^2).
void gpu_lu_solve(int n, const double* A, const int* piv, double scale, double* y) {
  for (int k = 0; k < n; k++)
    if (piv[k] != k) std::swap(y[k], y[piv[k]]);
  for (int i = 0; i < n; i++) {
    const double* ri = A + (size_t)i * n;
    double v = y[i];
    for (int j = 0; j < i; j++) v = std::fma(-ri[j], y[j], v);
    y[i] = v;
  }
  for (int i = n - 1; i >= 0; i--) {
    const double* ri = A + (size_t)i * n;
    double v = y[i];
    for (int j = n - 1; j > i; j--) v = std::fma(-ri[j], y[j], v);
    y[i] = v / ri[i];
  }
  for (int i = 0; i < n; i++) y[i] = y[i] * scale;
}

// Deterministic sum: fixed 256 chunks summed in order, independent of thread count.
double det_dot(int n, const double* a, const double* b) {
  const int nch = 256;
  double part[nch];
#pragma omp parallel for schedule(static)
  for (int c = 0; c < nch; c++) {
    long long lo = (long long)n * c / nch, hi = (long long)n * (c + 1) / nch;
    double s = 0;
    for (long long i = lo; i < hi; i++) s += a[i] * b[i];
    part[c] = s;
  }
  double s = 0;
  for (int c = 0; c < nch; c++) s += part[c];
  return s;
}

struct Rasm {
  int n = 0;
  int ncell = 0;
  std::vector<int> cs;                // cell starts (sorted order)
  std::vector<long long> off;         // buffer list offsets
  std::vector<int> idx;               // buffer lists
  std::vector<long long> aoff;        // factor offsets (nb*nb each)
  std::vector<double> lu;             // LU factors (row-major)
  std::vector<int> piv;               // pivot rows, per block (offset = off)
  int basic = 0;                      // PETSc -pc_asm_type basic instead of restrict
  int kind = 0;                       // 0: dense LU (the reference's); 1: the GPU's Cholesky;
                                      // 2: the GPU's Cholesky with its LU fallback
  double sigma = 0.0;
  std::vector<long long> coff;        // kind 1: packed-factor offsets (nb (nb + 1) / 2 each)
  std::vector<double> chol;           // kind 1: packed factors (gpu_chol_pack)
  int nshifted = 0;                   // kind 1: blocks refactored with a diagonal shift
                                      // (kind 2: blocks refactored by LU)
  std::vector<long long> luoff;       // kind 2: per cell, offset of its LU factor or -1
  std::vector<double> lub;            // kind 2: LU factors of those blocks (nb x nb each)
  std::vector<int> lupiv;             // kind 2: their pivot rows (nb each, at luoff / nb)
  std::vector<long long> lupoff;      // kind 2: per cell, offset of its pivots
};

// Dense LU with partial pivoting (row interchanges), the algorithm PETSc's
// -sub_pc_type lu uses for -sub_mat_type dense (LAPACK getrf semantics).
int lu_factor(int n, double* A, int* piv) {
  for (int k = 0; k < n; k++) {
    int p = k;
    double amax = fabs(A[(size_t)k * n + k]);
    for (int i = k + 1; i < n; i++) {
      double v = fabs(A[(size_t)i * n + k]);
      if (v > amax) {
        amax = v;
        p = i;
      }
    }
    piv[k] = p;
    if (amax == 0.0) return ERR_SINGULAR;
    if (p != k) {
      for (int j = 0; j < n; j++) std::swap(A[(size_t)k * n + j], A[(size_t)p * n + j]);
    }
    double inv = 1.0 / A[(size_t)k * n + k];
    for (int i = k + 1; i < n; i++) {
      double* ri = A + (size_t)i * n;
      double l = ri[k] * inv;
      ri[k] = l;
      if (l != 0.0) {
        const double* rk = A + (size_t)k * n;
        for (int j = k + 1; j < n; j++) ri[j] -= l * rk[j];
      }
    }
  }
  return OK;
}

void lu_solve(int n, const double* A, const int* piv, double* b) {
  for (int k = 0; k < n; k++) {
    if (piv[k] != k) std::swap(b[k], b[piv[k]]);
  }
  for (int i = 0; i < n; i++) {
    const double* ri = A + (size_t)i * n;
    double s = b[i];
    for (int j = 0; j < i; j++) s -= ri[j] * b[j];
    b[i] = s;
  }
  for (int i = n - 1; i >= 0; i--) {
    const double* ri = A + (size_t)i * n;
    double s = b[i];
    for (int j = i + 1; j < n; j++) s -= ri[j] * b[j];
    b[i] = s / ri[i];
  }
}

void gauss_sum_impl(const orc_grid* g, const double* tx, const double* ty, const double* tz,
                    const int* cs_tgt, const double* sx, const double* sy, const double* sz,
                    const double* sg, const int* cs_src, double* w, bool texp = false,
                    bool reverse = false) {
  const double kexp = kexp_of_sigma(g->sigma);
#pragma omp parallel
  {
    std::vector<int> list;
#pragma omp for schedule(dynamic, 4)
    for (int ic = 0; ic < g->ncell; ic++) {
      if (cs_tgt[ic] >= cs_tgt[ic + 1]) continue;
      int cnt = trunc_set(g, ic, sx, sy, sz, cs_src, cs_tgt, nullptr);
      list.resize(std::max<size_t>(list.size(), (size_t)cnt));
      trunc_set(g, ic, sx, sy, sz, cs_src, cs_tgt, list.data());
      // 2d/matmult.cxx:33-43 (3d/matmult.cxx:33-44)
      for (int i = cs_tgt[ic]; i < cs_tgt[ic + 1]; i++) {
        double acc = 0;
        for (int u = 0; u < cnt; u++) {
          // reverse: the same terms summed last to first (a rounding-order probe)
          int j = list[reverse ? cnt - 1 - u : u];
          double dx = tx[i] - sx[j];
          double dy = ty[i] - sy[j];
          // same grouping as the reference: (g * exp(.)) / (2 pi sigma^2)
          double r2 = g->dim == 3 ? dx * dx + dy * dy + (tz[i] - sz[j]) * (tz[i] - sz[j])
                                  : dx * dx + dy * dy;
          const double e = texp ? exp_neg_tab(r2, kexp) : exp(-(r2) / (2 * g->sigma * g->sigma));
          acc += sg[j] * e / (2 * M_PI * g->sigma * g->sigma);
        }
        w[i] = acc;
      }
    }
  }
}

}  // namespace

extern "C" {

int orc_num_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

// 2d/get_cluster.h:176-190 ; 3d/get_cluster.h:21-44 ; widths: 2d/get_trunc.h:14, 2d/get_buffer.h:11
int orc_grid_make(int dim, double pxmin, double pxmax, double pymin, double pymax,
                  double pzmin, double pzmax, double sigma, int nsigma_box,
                  int sigma_buffer, int sigma_trunc, orc_grid* g) {
  if (!g || (dim != 2 && dim != 3) || !(sigma > 0) || nsigma_box <= 0) return ERR_ARG;
  memset(g, 0, sizeof(*g));
  g->dim = dim;
  g->sigma = sigma;
  g->nsigma_box = nsigma_box;
  g->sigma_buffer = sigma_buffer;
  g->sigma_trunc = sigma_trunc;
  g->nb_buffer = (int)ceil((sigma_buffer - nsigma_box + kEpsf) / 2 / nsigma_box);
  g->nb_trunc = (int)ceil((sigma_trunc - nsigma_box + kEpsf) / 2 / nsigma_box);
  if (g->nb_buffer < 0) g->nb_buffer = 0;
  if (g->nb_trunc < 0) g->nb_trunc = 0;
  double xmin = pxmin - kEpsf, xmax = pxmax + kEpsf;
  double ymin = pymin - kEpsf, ymax = pymax + kEpsf;
  double zmin = pzmin - kEpsf, zmax = pzmax + kEpsf;
  g->xmin = xmin;
  g->ymin = ymin;
  g->zmin = dim == 3 ? zmin : 0.0;
  g->box = nsigma_box * sigma + kEpsf;
  g->nx = (int)ceil((xmax - xmin) / g->box);
  g->ny = (int)ceil((ymax - ymin) / g->box);
  g->nz = dim == 3 ? (int)ceil((zmax - zmin) / g->box) : 1;
  long long nc = (long long)g->nx * g->ny * g->nz;
  if (g->nx <= 0 || g->ny <= 0 || g->nz <= 0 || nc > (1LL << 30)) return ERR_RANGE;
  g->ncell = (int)nc;
  g->trunc_len = sigma_trunc * sigma / 2 + kEpsf;
  g->buffer_len = sigma_buffer * sigma / 2 + kEpsf;
  return OK;
}

int orc_cell_ids(const orc_grid* g, int n, const double* x, const double* y, const double* z,
                 int* cell) {
  int bad = 0;
#pragma omp parallel for reduction(| : bad)
  for (int i = 0; i < n; i++) {
    cell[i] = point_cell(g, x[i], y[i], g->dim == 3 ? z[i] : 0.0);
    if (cell[i] < 0) bad = 1;
  }
  return bad ? ERR_RANGE : OK;
}

// Stable counting sort by cell (2d/get_cluster.h:233-264 counts and offsets,
// 2d/get_cluster.h:279-286 sorted-slot writes in ascending original index).
int orc_cell_sort(const orc_grid* g, int n, const double* x, const double* y, const double* z,
                  int* perm, int* cell_start) {
  std::vector<int> cell(n);
  int st = orc_cell_ids(g, n, x, y, z, cell.data());
  if (st) return st;
  std::vector<int> cnt(g->ncell + 1, 0);
  for (int i = 0; i < n; i++) cnt[cell[i]]++;
  cell_start[0] = 0;
  for (int c = 0; c < g->ncell; c++) cell_start[c + 1] = cell_start[c] + cnt[c];
  std::vector<int> pos(cell_start, cell_start + g->ncell);
  for (int i = 0; i < n; i++) perm[pos[cell[i]]++] = i;
  return OK;
}

int orc_trunc_counts(const orc_grid* g, const double* sx, const double* sy, const double* sz,
                     const int* cs_src, const int* cs_tgt, int* counts) {
#pragma omp parallel for schedule(dynamic, 16)
  for (int ic = 0; ic < g->ncell; ic++)
    counts[ic] = trunc_set(g, ic, sx, sy, sz, cs_src, cs_tgt, nullptr);
  return OK;
}

int orc_trunc_list(const orc_grid* g, int cell, const double* sx, const double* sy,
                   const double* sz, const int* cs_src, const int* cs_tgt, int* idx) {
  if (cell < 0 || cell >= g->ncell) return -1;
  return trunc_set(g, cell, sx, sy, sz, cs_src, cs_tgt, idx);
}

int orc_gauss_sum(const orc_grid* g, const double* tx, const double* ty, const double* tz,
                  const int* cs_tgt, const double* sx, const double* sy, const double* sz,
                  const double* sg, const int* cs_src, double* w) {
  gauss_sum_impl(g, tx, ty, tz, cs_tgt, sx, sy, sz, sg, cs_src, w);
  return OK;
}

int orc_buffer_counts(const orc_grid* g, const double* x, const double* y, const double* z,
                      const int* cs, int* counts) {
#pragma omp parallel for schedule(dynamic, 16)
  for (int ic = 0; ic < g->ncell; ic++) counts[ic] = buffer_set(g, ic, x, y, z, cs, nullptr);
  return OK;
}

int orc_buffer_fill(const orc_grid* g, const double* x, const double* y, const double* z,
                    const int* cs, const long long* offsets, int* idx) {
#pragma omp parallel for schedule(dynamic, 16)
  for (int ic = 0; ic < g->ncell; ic++) buffer_set(g, ic, x, y, z, cs, idx + offsets[ic]);
  return OK;
}

// Dense subdomain block, all pairs, no truncation (2d/matmult.cxx:83-93).
int orc_block(const orc_grid* g, int nb, const int* idx, const double* x, const double* y,
              const double* z, double* A) {
  for (int i = 0; i < nb; i++)
    for (int j = 0; j < nb; j++) {
      int a = idx[i], b = idx[j];
      double dz = g->dim == 3 ? z[a] - z[b] : 0.0;
      A[(size_t)i * nb + j] = phi(g->sigma, x[a] - x[b], y[a] - y[b], dz, g->dim);
    }
  return OK;
}

void* orc_rasm_create(const orc_grid* g, int n, const double* x, const double* y,
                      const double* z, const int* cs, int* status) {
  return orc_rasm_create_kind(g, n, x, y, z, cs, 0, status);
}

// kind 1: the GPU library's blocks (table exp, neighbours first, K = 2 pi sigma^2 A_c),
// ordered Cholesky with the GPU's shifted retries (diagonal + 1e-12, then + 1e-9, relative
// to K's unit diagonal) for blocks with a non-positive pivot, packed factors.
static int rasm_build_chol(const orc_grid* g, Rasm* R, const std::vector<int>& cnt, const double* x,
                           const double* y, const double* z, bool lu_fallback) {
  R->coff.assign(g->ncell + 1, 0);
  for (int c = 0; c < g->ncell; c++)
    R->coff[c + 1] = R->coff[c] + (long long)cnt[c] * (cnt[c] + 1) / 2;
  R->chol.resize(R->coff[g->ncell]);
  const double kexp = kexp_of_sigma(g->sigma);
  const double out_scale = 2.0 * M_PI * g->sigma * g->sigma;
  const double sc = sqrt(1.0 / out_scale);
  int bad = 0, shifted = 0;
  std::vector<unsigned char> need_lu(g->ncell, 0);
#pragma omp parallel reduction(| : bad) reduction(+ : shifted)
  {
    std::vector<double> K, U;
#pragma omp for schedule(dynamic, 1)
    for (int c = 0; c < g->ncell; c++) {
      const int nb = cnt[c];
      if (!nb) continue;
      const int nc = R->cs[c + 1] - R->cs[c];
      K.resize((size_t)nb * nb);
      U.resize((size_t)nb * nb);
      bool ok = false;
      for (int attempt = 0; attempt < 3 && !ok; attempt++) {
        const double shift = attempt == 0 ? 0.0 : (attempt == 1 ? 1e-12 : 1e-9);
        gpu_block_K(g->dim, nb, nc, R->idx.data() + R->off[c], x, y, z, kexp, shift, K.data());
        ok = gpu_chol_pack(nb, K.data(), sc, U.data(), R->chol.data() + R->coff[c]);
        if (!ok && attempt == 0) {
          shifted++;
          if (lu_fallback) {
            need_lu[c] = 1;
            ok = true;  // factored below
          }
        }
      }
      if (!ok) bad = 1;
    }
  }
  R->nshifted = shifted;
  if (lu_fallback) {
    // the LU fallback (kind 2), blocks in cell order
    R->luoff.assign(g->ncell, -1);
    R->lupoff.assign(g->ncell, -1);
    long long a = 0, p = 0;
    for (int c = 0; c < g->ncell; c++)
      if (need_lu[c]) {
        R->luoff[c] = a;
        R->lupoff[c] = p;
        a += (long long)cnt[c] * cnt[c];
        p += cnt[c];
      }
    R->lub.assign(a, 0.0);
    R->lupiv.assign(p, 0);
    for (int c = 0; c < g->ncell; c++) {
      if (!need_lu[c]) continue;
      const int nb = cnt[c], nc = R->cs[c + 1] - R->cs[c];
      double* K = R->lub.data() + R->luoff[c];
      gpu_block_K(g->dim, nb, nc, R->idx.data() + R->off[c], x, y, z, kexp, 0.0, K);
      if (!gpu_lu_factor(nb, K, R->lupiv.data() + R->lupoff[c])) bad = 1;
    }
  }
  return bad ? ERR_SINGULAR : OK;
}

static bool lu_block(const Rasm* R, int c) { return R->kind == 2 && R->luoff[c] >= 0; }

void* orc_rasm_create_kind(const orc_grid* g, int n, const double* x, const double* y,
                           const double* z, const int* cs, int kind, int* status) {
  Rasm* R = new Rasm;
  R->kind = (kind == 1 || kind == 2) ? kind : 0;
  R->sigma = g->sigma;
  R->n = n;
  R->ncell = g->ncell;
  R->cs.assign(cs, cs + g->ncell + 1);
  std::vector<int> cnt(g->ncell);
  orc_buffer_counts(g, x, y, z, cs, cnt.data());
  R->off.resize(g->ncell + 1);
  R->aoff.resize(g->ncell + 1);
  R->off[0] = 0;
  R->aoff[0] = 0;
  for (int c = 0; c < g->ncell; c++) {
    R->off[c + 1] = R->off[c] + cnt[c];
    R->aoff[c + 1] = R->aoff[c] + (long long)cnt[c] * cnt[c];
  }
  R->idx.resize(R->off[g->ncell]);
  orc_buffer_fill(g, x, y, z, cs, R->off.data(), R->idx.data());
  if (R->kind >= 1) {
    int st = rasm_build_chol(g, R, cnt, x, y, z, R->kind == 2);
    if (status) *status = st;
    return R;
  }
  R->piv.resize(R->off[g->ncell]);
  R->lu.resize(R->aoff[g->ncell]);
  int bad = 0;
  // mysubmat (2d/matmult.cxx:53-104) + the per-block dense LU of -sub_pc_type lu.
#pragma omp parallel for schedule(dynamic, 1) reduction(| : bad)
  for (int c = 0; c < g->ncell; c++) {
    int nb = cnt[c];
    if (!nb) continue;
    double* A = R->lu.data() + R->aoff[c];
    orc_block(g, nb, R->idx.data() + R->off[c], x, y, z, A);
    if (lu_factor(nb, A, R->piv.data() + R->off[c])) bad = 1;
  }
  if (status) *status = bad ? ERR_SINGULAR : OK;
  return R;
}

int orc_rasm_set_type(void* h, int basic) {
  if (!h) return ERR_ARG;
  ((Rasm*)h)->basic = basic ? 1 : 0;
  return OK;
}

// Basic additive Schwarz (PCASM type basic, selectable through the reference's
// KSPSetFromOptions, 2d/rbf_interpolation.cxx:211): out = sum_c R_c^T A_c^-1 R_c r over the
// same subdomains; the block solutions are added in cell order (deterministic).
static void asm_basic_apply(const Rasm* R, const double* r, double* out) {
  std::vector<double> sol(R->off[R->ncell]);
#pragma omp parallel for schedule(dynamic, 4)
  for (int c = 0; c < R->ncell; c++) {
    long long nb = R->off[c + 1] - R->off[c];
    if (!nb) continue;
    double* buf = sol.data() + R->off[c];
    const int* id = R->idx.data() + R->off[c];
    if (R->kind >= 1) {
      const int nc = R->cs[c + 1] - R->cs[c];
      std::vector<double> yb(nb);
      for (long long j = 0; j < nb; j++) yb[j] = r[id[gpu_row((int)j, (int)nb, nc)]];
      if (lu_block(R, c))
        gpu_lu_solve((int)nb, R->lub.data() + R->luoff[c], R->lupiv.data() + R->lupoff[c],
                     2.0 * M_PI * R->sigma * R->sigma, yb.data());
      else
        gpu_tri_apply((int)nb, 0, R->chol.data() + R->coff[c], yb.data());
      for (long long j = 0; j < nb; j++) buf[gpu_row((int)j, (int)nb, nc)] = yb[j];
      continue;
    }
    for (long long i = 0; i < nb; i++) buf[i] = r[id[i]];
    lu_solve((int)nb, R->lu.data() + R->aoff[c], R->piv.data() + R->off[c], buf);
  }
  for (int i = 0; i < R->n; i++) out[i] = 0.0;
  for (long long k = 0; k < R->off[R->ncell]; k++) out[R->idx[k]] += sol[k];
}

// Restricted additive Schwarz apply: subdomain = buffer set ("is"), prolongation only
// onto the centre points ("is_local" = first n_c entries), 2d/rbf_interpolation.cxx:213-229.
int orc_rasm_apply(void* h, const double* r, double* out) {
  Rasm* R = (Rasm*)h;
  if (R->basic) {
    asm_basic_apply(R, r, out);
    return OK;
  }
#pragma omp parallel
  {
    std::vector<double> buf;
#pragma omp for schedule(dynamic, 4)
    for (int c = 0; c < R->ncell; c++) {
      long long nb = R->off[c + 1] - R->off[c];
      if (!nb) continue;
      buf.resize(nb);
      const int* id = R->idx.data() + R->off[c];
      int nc = R->cs[c + 1] - R->cs[c];
      if (R->kind >= 1) {
        const int n1 = (int)nb - nc;
        for (long long j = 0; j < nb; j++) buf[j] = r[id[gpu_row((int)j, (int)nb, nc)]];
        if (lu_block(R, c))
          gpu_lu_solve((int)nb, R->lub.data() + R->luoff[c], R->lupiv.data() + R->lupoff[c],
                       2.0 * M_PI * R->sigma * R->sigma, buf.data());
        else
          gpu_tri_apply((int)nb, n1, R->chol.data() + R->coff[c], buf.data());
        for (int i = 0; i < nc; i++) out[R->cs[c] + i] = buf[n1 + i];
        continue;
      }
      for (long long i = 0; i < nb; i++) buf[i] = r[id[i]];
      lu_solve((int)nb, R->lu.data() + R->aoff[c], R->piv.data() + R->off[c], buf.data());
      for (int i = 0; i < nc; i++) out[R->cs[c] + i] = buf[i];
    }
  }
  return OK;
}

void orc_rasm_destroy(void* h) { delete (Rasm*)h; }

int orc_rasm_block_info(void* h, int cell, int* nb, int* nc, int* nshifted) {
  Rasm* R = (Rasm*)h;
  if (!R || cell < 0 || cell >= R->ncell) return ERR_ARG;
  if (nb) *nb = (int)(R->off[cell + 1] - R->off[cell]);
  if (nc) *nc = R->cs[cell + 1] - R->cs[cell];
  if (nshifted) *nshifted = R->nshifted;
  return OK;
}

int orc_rasm_factor_rows(void* h, int cell, double* out) {
  Rasm* R = (Rasm*)h;
  if (!R || R->kind < 1 || cell < 0 || cell >= R->ncell || lu_block(R, cell)) return ERR_ARG;
  std::copy(R->chol.begin() + R->coff[cell], R->chol.begin() + R->coff[cell + 1], out);
  return OK;
}

// The blocked Cholesky against its definition on one SPD block K (n x n, row-major lower
// read; the full matrix is not modified): 1 if every entry of the two factors is
// bit-identical (and both report the same pivot status), else 0.
int orc_chol_blocked_matches_unblocked(int n, const double* K) {
  std::vector<double> U1((size_t)n * n), L1((size_t)n * n), U2((size_t)n * n);
  const bool ok1 = chol_unblocked(n, K, U1.data(), L1.data());
  const bool ok2 = chol_blocked(n, K, U2.data());
  if (ok1 != ok2) return 0;
  for (int i = 0; i < n; i++)
    for (int j = 0; j <= i; j++)
      if (memcmp(&L1[(size_t)i * n + j], &U2[(size_t)j * n + i], sizeof(double)) != 0) return 0;
  return 1;
}

int orc_gpu_block(const orc_grid* g, int nb, int nc, const int* idx, const double* x, const double* y,
                  const double* z, double* K) {
  if (!g || nb <= 0 || nc < 0 || nc > nb) return ERR_ARG;
  gpu_block_K(g->dim, nb, nc, idx, x, y, z, kexp_of_sigma(g->sigma), 0.0, K);
  return OK;
}

// GMRES(restart), left preconditioning, classical Gram-Schmidt without refinement,
// Givens rotations, preconditioned-residual convergence test relative to the first
// preconditioned residual: PETSc KSPGMRES / KSPConvergedDefault defaults, invoked at
// 2d/rbf_interpolation.cxx:210-232 with options 2d/Makefile:7. Restated from PETSc's
// documented algorithm (PETSc is not part of the reference; parity unpinned).
int orc_gmres(const orc_grid* g, int n, const double* x, const double* y, const double* z,
              const int* cs, void* rasm, const double* b, const double* x0, double rtol,
              double abstol, double dtol, int restart, int max_it, double* xsol, int* its_out,
              int* reason_out, double* hist) {
  return orc_gmres_ex(g, n, x, y, z, cs, rasm, b, x0, rtol, abstol, dtol, restart, max_it, xsol,
                      its_out, reason_out, hist, 0);
}

// flags bit 2: the Gaussian sums take the GPU library's table exp instead of libm's exp;
// bit 3: every row of the sums adds its terms in reverse order (same terms, another
// rounding order -- shows how far the stopping point moves with rounding alone).
int orc_gmres_ex(const orc_grid* g, int n, const double* x, const double* y, const double* z,
                 const int* cs, void* rasm, const double* b, const double* x0, double rtol,
                 double abstol, double dtol, int restart, int max_it, double* xsol, int* its_out,
                 int* reason_out, double* hist, int flags) {
  const bool texp = (flags & 4) != 0, rev = (flags & 8) != 0;
  const double haptol = 1e-30;
  int m = restart;
  std::vector<double> V((size_t)(m + 1) * n), t(n), w(n);
  std::vector<double> H((size_t)(m + 1) * m, 0.0), cc(m), ss(m), grs(m + 1);
  for (int i = 0; i < n; i++) xsol[i] = x0 ? x0[i] : 0.0;
  auto apply_BA = [&](const double* v, double* out) {
    gauss_sum_impl(g, x, y, z, cs, x, y, z, v, cs, t.data(), texp, rev);
    orc_rasm_apply(rasm, t.data(), out);
  };
  int its = 0, reason = 0;
  double rnorm0 = 0, ttol = 0;
  auto converged = [&](int k, double rnorm) -> int {
    if (k == 0) {
      rnorm0 = rnorm;
      ttol = std::max(rtol * rnorm0, abstol);
    }
    if (rnorm != rnorm) return DIVERGED_NANORINF;
    if (rnorm <= ttol) return rnorm < abstol ? CONVERGED_ATOL : CONVERGED_RTOL;
    if (rnorm >= dtol * rnorm0) return DIVERGED_DTOL;
    return 0;
  };
  while (!reason) {
    // v0 = B (b - A x)
    gauss_sum_impl(g, x, y, z, cs, x, y, z, xsol, cs, t.data(), texp, rev);
    for (int i = 0; i < n; i++) w[i] = b[i] - t[i];
    double* v0 = V.data();
    orc_rasm_apply(rasm, w.data(), v0);
    double beta = sqrt(det_dot(n, v0, v0));
    if (its == 0 && hist) hist[0] = beta;
    if (beta == 0.0) {
      reason = CONVERGED_ATOL;
      break;
    }
    reason = converged(its, beta);
    if (reason) break;
    for (int i = 0; i < n; i++) v0[i] /= beta;
    grs.assign(m + 1, 0.0);
    grs[0] = beta;
    int it = 0;
    bool hapend = false;
    while (!reason && it < m && its < max_it) {
      double* vk = V.data() + (size_t)it * n;
      double* vn = V.data() + (size_t)(it + 1) * n;
      apply_BA(vk, vn);
      // classical Gram-Schmidt: all coefficients from the same vector, then one update
      std::vector<double> hcol(it + 2, 0.0);
      for (int j = 0; j <= it; j++) hcol[j] = det_dot(n, vn, V.data() + (size_t)j * n);
      for (int j = 0; j <= it; j++) {
        const double* vj = V.data() + (size_t)j * n;
        double hj = hcol[j];
        for (int i = 0; i < n; i++) vn[i] -= hj * vj[i];
      }
      double tt = sqrt(det_dot(n, vn, vn));
      double hapbnd = fabs(tt / grs[it]);
      if (hapbnd > haptol) hapbnd = haptol;
      if (tt > hapbnd) {
        for (int i = 0; i < n; i++) vn[i] /= tt;
      } else {
        hapend = true;
      }
      hcol[it + 1] = tt;
      // apply earlier rotations, build the new one, rotate the residual vector
      for (int j = 0; j < it; j++) {
        double a = hcol[j], bb = hcol[j + 1];
        hcol[j] = cc[j] * a + ss[j] * bb;
        hcol[j + 1] = -ss[j] * a + cc[j] * bb;
      }
      double rr = sqrt(hcol[it] * hcol[it] + hcol[it + 1] * hcol[it + 1]);
      if (rr == 0.0) {
        reason = DIVERGED_BREAKDOWN;
        break;
      }
      cc[it] = hcol[it] / rr;
      ss[it] = hcol[it + 1] / rr;
      grs[it + 1] = -ss[it] * grs[it];
      grs[it] = cc[it] * grs[it];
      hcol[it] = cc[it] * hcol[it] + ss[it] * hcol[it + 1];
      for (int j = 0; j <= it; j++) H[(size_t)j * m + it] = hcol[j];
      double res = fabs(grs[it + 1]);
      it++;
      its++;
      if (hist) hist[its] = res;
      reason = converged(its, res);
      if (hapend && !reason) reason = DIVERGED_BREAKDOWN;
    }
    // x += V y, H y = grs (upper triangular, size it)
    if (it > 0) {
      std::vector<double> yv(it);
      for (int k = it - 1; k >= 0; k--) {
        double s = grs[k];
        for (int j = k + 1; j < it; j++) s -= H[(size_t)k * m + j] * yv[j];
        double d = H[(size_t)k * m + k];
        yv[k] = d != 0.0 ? s / d : 0.0;
      }
      for (int j = 0; j < it; j++) {
        const double* vj = V.data() + (size_t)j * n;
        for (int i = 0; i < n; i++) xsol[i] += yv[j] * vj[i];
      }
    }
    if (!reason && its >= max_it) reason = DIVERGED_ITS;
  }
  if (its_out) *its_out = its;
  if (reason_out) *reason_out = reason;
  return OK;
}

// rbf_interpolation (2d/rbf_interpolation.cxx:25-310; 3d:26-334): bounding box, cell
// sort, solve in cell order from a zero guess, weights back in the caller's order.
int orc_rbf_interpolation(int dim, int n, const double* x, const double* y, const double* z,
                          const double* f, double sigma, int nsigma_box, int sigma_buffer,
                          int sigma_trunc, double rtol, int restart, int max_it, double* g_out,
                          int* its, int* reason, int pc_flags) {
  const int pc_basic = pc_flags & 1;
  if (n <= 0) return ERR_ARG;
  double b[6] = {x[0], x[0], y[0], y[0], dim == 3 ? z[0] : 0, dim == 3 ? z[0] : 0};
  for (int i = 0; i < n; i++) {
    b[0] = std::min(b[0], x[i]);
    b[1] = std::max(b[1], x[i]);
    b[2] = std::min(b[2], y[i]);
    b[3] = std::max(b[3], y[i]);
    if (dim == 3) {
      b[4] = std::min(b[4], z[i]);
      b[5] = std::max(b[5], z[i]);
    }
  }
  orc_grid g;
  int st = orc_grid_make(dim, b[0], b[1], b[2], b[3], b[4], b[5], sigma, nsigma_box,
                         sigma_buffer, sigma_trunc, &g);
  if (st) return st;
  std::vector<int> perm(n), cs(g.ncell + 1);
  st = orc_cell_sort(&g, n, x, y, z, perm.data(), cs.data());
  if (st) return st;
  std::vector<double> xs(n), ys(n), zs(dim == 3 ? n : 0), fs(n), gs(n);
  for (int k = 0; k < n; k++) {
    xs[k] = x[perm[k]];
    ys[k] = y[perm[k]];
    if (dim == 3) zs[k] = z[perm[k]];
    fs[k] = f[perm[k]];
  }
  const double* zp = dim == 3 ? zs.data() : nullptr;
  void* R = orc_rasm_create_kind(&g, n, xs.data(), ys.data(), zp, cs.data(),
                                 (pc_flags & 2) ? ((pc_flags & 16) ? 2 : 1) : 0, &st);
  if (st) {
    orc_rasm_destroy(R);
    return st;
  }
  orc_rasm_set_type(R, pc_basic);
  orc_gmres_ex(&g, n, xs.data(), ys.data(), zp, cs.data(), R, fs.data(), nullptr, rtol, 1e-50,
               1e5, restart, max_it, gs.data(), its, reason, nullptr, pc_flags);
  orc_rasm_destroy(R);
  for (int k = 0; k < n; k++) g_out[perm[k]] = gs[k];
  return OK;
}

// vorticity_evaluation (2d/vorticity_evaluation.cxx:26-299, 2d/get_vorticity.h:9-27):
// one grid over the union bounding box, targets and sources each cell-sorted.
int orc_vorticity_evaluation(int dim, int nt, const double* xt, const double* yt,
                             const double* zt, int ns, const double* xs, const double* ys,
                             const double* zs, const double* gs, double sigma, int nsigma_box,
                             int sigma_buffer, int sigma_trunc, double* w_out) {
  if (nt <= 0 || ns <= 0) return ERR_ARG;
  double b[6] = {xt[0], xt[0], yt[0], yt[0], dim == 3 ? zt[0] : 0, dim == 3 ? zt[0] : 0};
  auto upd = [&](int n, const double* x, const double* y, const double* z) {
    for (int i = 0; i < n; i++) {
      b[0] = std::min(b[0], x[i]);
      b[1] = std::max(b[1], x[i]);
      b[2] = std::min(b[2], y[i]);
      b[3] = std::max(b[3], y[i]);
      if (dim == 3) {
        b[4] = std::min(b[4], z[i]);
        b[5] = std::max(b[5], z[i]);
      }
    }
  };
  upd(nt, xt, yt, zt);
  upd(ns, xs, ys, zs);
  orc_grid g;
  int st = orc_grid_make(dim, b[0], b[1], b[2], b[3], b[4], b[5], sigma, nsigma_box,
                         sigma_buffer, sigma_trunc, &g);
  if (st) return st;
  std::vector<int> pt(nt), ps(ns), ct(g.ncell + 1), cs(g.ncell + 1);
  if ((st = orc_cell_sort(&g, nt, xt, yt, zt, pt.data(), ct.data()))) return st;
  if ((st = orc_cell_sort(&g, ns, xs, ys, zs, ps.data(), cs.data()))) return st;
  std::vector<double> txs(nt), tys(nt), tzs(dim == 3 ? nt : 0), sxs(ns), sys(ns),
      szs(dim == 3 ? ns : 0), sgs(ns), w(nt);
  for (int k = 0; k < nt; k++) {
    txs[k] = xt[pt[k]];
    tys[k] = yt[pt[k]];
    if (dim == 3) tzs[k] = zt[pt[k]];
  }
  for (int k = 0; k < ns; k++) {
    sxs[k] = xs[ps[k]];
    sys[k] = ys[ps[k]];
    if (dim == 3) szs[k] = zs[ps[k]];
    sgs[k] = gs[ps[k]];
  }
  gauss_sum_impl(&g, txs.data(), tys.data(), dim == 3 ? tzs.data() : nullptr, ct.data(),
                 sxs.data(), sys.data(), dim == 3 ? szs.data() : nullptr, sgs.data(),
                 cs.data(), w.data());
  for (int k = 0; k < nt; k++) w_out[pt[k]] = w[k];
  return OK;
}

}  // extern "C"
