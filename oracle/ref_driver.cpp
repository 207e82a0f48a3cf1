/*
 * ref_driver.cpp -- TEST INFRASTRUCTURE ONLY.
 *
 * Drives the reference's own code, compiled unmodified from the reference tree
 * (REF_DIM=2: 2d/, REF_DIM=3: 3d/) against the sequential PETSc/MPI stand-in in
 * oracle/ref_stub/, to produce golden vectors for the oracle:
 *   cell sort      -- Get_cluster::get_cluster (2d/get_cluster.h:15-276)
 *   truncation set -- Get_trunc::get_trunc     (2d/get_trunc.h:9-87)
 *   buffer set     -- Get_buffer::get_buffer   (2d/get_buffer.h:9-90)
 *   matvec         -- mymatmult                (2d/matmult.cxx:6-51)
 *   dense blocks   -- mysubmat                 (2d/matmult.cxx:53-104)
 *   evaluation     -- Get_vorticity            (2d/get_vorticity.h:9-27)
 * The set-up around those calls (bounding box, permutation of the inputs into cell
 * order) restates what rbf_interpolation / vorticity_evaluation do with PETSc
 * scatters (2d/rbf_interpolation.cxx:59-171, 2d/vorticity_evaluation.cxx:55-222).
 * Built only where the reference sources exist (never shipped, never in the product).
 */
#include "par.h"
#include "get_cluster.h"
#include "get_buffer.h"
#include "get_trunc.h"
#include "get_vorticity.h"

extern PetscErrorCode mymatmult(Mat, Vec, Vec);
extern PetscErrorCode mysubmat(Mat, PetscInt, const IS*, const IS*, MatReuse, Mat**);

namespace {
PARTICLE P;
CLUSTER C;
BOTH B;
int N = 0;
std::vector<int> perm;
std::vector<double> xs, ys, zs, ws;
Vec gvec = nullptr;

template <class T>
void bbox(int n, const double* v, T* lo, T* hi) {
  *lo = v[0];
  *hi = v[0];
  for (int i = 1; i < n; i++) {
    *lo = std::min<T>(*lo, v[i]);
    *hi = std::max<T>(*hi, v[i]);
  }
}
}  // namespace

extern "C" {

int ref_dim(void) { return REF_DIM; }

int ref_setup(int n, const double* x, const double* y, const double* z, double sigma,
              int nsigma_box, int sigma_buffer, int sigma_trunc) {
  P = PARTICLE();
  C = CLUSTER();
  N = n;
  P.sigma = sigma;
  bbox(n, x, &P.xmin, &P.xmax);
  bbox(n, y, &P.ymin, &P.ymax);
#if REF_DIM == 3
  bbox(n, z, &P.zmin, &P.zmax);
#endif
  C.nsigma_box = nsigma_box;
  C.sigma_buffer = sigma_buffer;
  C.sigma_trunc = sigma_trunc;
  C.file = 0;
  P.ni = P.nj = n;
  P.ista = P.jsta = 0;
  P.iend = P.jend = n;
  P.nilocal = P.njlocal = n;
  P.xil = P.xjl = const_cast<double*>(x);
  P.yil = P.yjl = const_cast<double*>(y);
#if REF_DIM == 3
  P.zil = P.zjl = const_cast<double*>(z);
#endif
  Get_cluster cl;
  cl.get_cluster(&P, &C);
  perm.resize(n);
  for (int k = 0; k < n; k++) perm[k] = (int)P.ii->a[k];
  xs.resize(n);
  ys.resize(n);
  zs.resize(n);
  ws.assign(n, 0.0);
  for (int k = 0; k < n; k++) {
    xs[k] = x[perm[k]];
    ys[k] = y[perm[k]];
    zs[k] = REF_DIM == 3 ? z[perm[k]] : 0.0;
  }
  P.xil = P.xjl = xs.data();
  P.yil = P.yjl = ys.data();
#if REF_DIM == 3
  P.zil = P.zjl = zs.data();
#endif
  VecCreate(PETSC_COMM_WORLD, &gvec);
  VecSetSizes(gvec, n, PETSC_DETERMINE);
  P.gi = gvec;
  P.gil = P.gjl = gvec->a.data();
  P.wil = ws.data();
  B.p = &P;
  B.c = &C;
  return C.n;
}

void ref_grid(int* ints, double* dbls) {
  ints[0] = C.nx;
  ints[1] = C.ny;
#if REF_DIM == 3
  ints[2] = C.nz;
#else
  ints[2] = 1;
#endif
  ints[3] = C.n;
  ints[4] = C.neighbor_trunc;
  ints[5] = C.neighbor_buffer;
  ints[6] = C.maxtrunc;   // scratch capacity of get_trunc (xjt, yjt, ...)
  ints[7] = C.maxbuffer;  // scratch capacity of get_buffer (xib, ..., idx)
  dbls[0] = C.xmin;
  dbls[1] = C.ymin;
#if REF_DIM == 3
  dbls[2] = C.zmin;
#else
  dbls[2] = 0.0;
#endif
  dbls[3] = C.box_length;
}

void ref_perm(int* out) { std::copy(perm.begin(), perm.end(), out); }

void ref_cell_start(int* cs) {
  for (int ic = 0; ic < C.n; ic++) cs[ic] = C.ista[ic];
  cs[C.n] = N;
}

void ref_trunc_counts(int* counts) {
  for (int ic = 0; ic < C.n; ic++) {
    Get_trunc t;
    t.get_trunc(&P, &C, ic);
    counts[ic] = C.nptruncj;
  }
}

int ref_trunc_set(int ic, double* xo, double* yo, double* zo) {
  Get_trunc t;
  t.get_trunc(&P, &C, ic);
  for (int i = 0; i < C.nptruncj; i++) {
    xo[i] = C.xjt[i];
    yo[i] = C.yjt[i];
#if REF_DIM == 3
    zo[i] = C.zjt[i];
#else
    zo[i] = 0.0;
#endif
  }
  return C.nptruncj;
}

int ref_buffer(int ic, int* idx) {
  Get_buffer b;
  b.get_buffer(&P, &C, ic);
  for (int i = 0; i < C.npbufferi; i++) idx[i] = C.idx[i];
  return C.npbufferi;
}

int ref_matvec(const double* g_sorted, double* y_sorted) {
  Vec X, Y;
  VecCreate(PETSC_COMM_WORLD, &X);
  VecSetSizes(X, N, PETSC_DETERMINE);
  VecCreate(PETSC_COMM_WORLD, &Y);
  VecSetSizes(Y, N, PETSC_DETERMINE);
  std::copy(g_sorted, g_sorted + N, X->a.begin());
  Mat M;
  MatCreate(PETSC_COMM_WORLD, &M);
  M->ctx = &B;
  int ierr = mymatmult(M, X, Y);
  std::copy(Y->a.begin(), Y->a.end(), y_sorted);
  VecDestroy(&X);
  VecDestroy(&Y);
  MatDestroy(&M);
  return ierr;
}

/* Dense blocks of the listed cells, concatenated row-major; returns total entries. */
long long ref_blocks(int ncells, const int* cells, double* out) {
  Mat Pm;
  MatCreate(PETSC_COMM_WORLD, &Pm);
  Pm->ctx = &B;
  Mat* sub = nullptr;
  int ierr = mysubmat(Pm, C.nclocal, nullptr, nullptr, MAT_INITIAL_MATRIX, &sub);
  if (ierr) return -1;
  long long off = 0;
  for (int k = 0; k < ncells; k++) {
    Mat m = sub[cells[k] - C.icsta];
    if (out) std::copy(m->a.begin(), m->a.end(), out + off);
    off += (long long)m->a.size();
  }
  for (int ic = 0; ic < C.nclocal; ic++) MatDestroy(&sub[ic]);
  std::free(sub);
  MatDestroy(&Pm);
  return off;
}

int ref_vorticity(int nt, const double* xt, const double* yt, const double* zt, int ns,
                  const double* xsrc, const double* ysrc, const double* zsrc, const double* gsrc,
                  double sigma, int nsigma_box, int sigma_buffer, int sigma_trunc, double* w_out) {
  PARTICLE Q = PARTICLE();
  CLUSTER D = CLUSTER();
  Q.sigma = sigma;
  double a, b, c2, d;
  bbox(nt, xt, &a, &b);
  bbox(ns, xsrc, &c2, &d);
  Q.xmin = std::min(a, c2);
  Q.xmax = std::max(b, d);
  bbox(nt, yt, &a, &b);
  bbox(ns, ysrc, &c2, &d);
  Q.ymin = std::min(a, c2);
  Q.ymax = std::max(b, d);
#if REF_DIM == 3
  bbox(nt, zt, &a, &b);
  bbox(ns, zsrc, &c2, &d);
  Q.zmin = std::min(a, c2);
  Q.zmax = std::max(b, d);
#endif
  D.nsigma_box = nsigma_box;
  D.sigma_buffer = sigma_buffer;
  D.sigma_trunc = sigma_trunc;
  D.file = 0;
  Q.ni = nt;
  Q.nj = ns;
  Q.ista = Q.jsta = 0;
  Q.iend = nt;
  Q.jend = ns;
  Q.nilocal = nt;
  Q.njlocal = ns;
  Q.xil = const_cast<double*>(xt);
  Q.yil = const_cast<double*>(yt);
  Q.xjl = const_cast<double*>(xsrc);
  Q.yjl = const_cast<double*>(ysrc);
#if REF_DIM == 3
  Q.zil = const_cast<double*>(zt);
  Q.zjl = const_cast<double*>(zsrc);
#endif
  Get_cluster cl;
  cl.get_cluster(&Q, &D);
  std::vector<int> pi(nt), pj(ns);
  for (int k = 0; k < nt; k++) pi[k] = (int)Q.ii->a[k];
  for (int k = 0; k < ns; k++) pj[k] = (int)Q.jj->a[k];
  std::vector<double> txs(nt), tys(nt), tzs(nt), sxs(ns), sys(ns), szs(ns), sgs(ns), w(nt);
  for (int k = 0; k < nt; k++) {
    txs[k] = xt[pi[k]];
    tys[k] = yt[pi[k]];
    tzs[k] = REF_DIM == 3 ? zt[pi[k]] : 0.0;
  }
  for (int k = 0; k < ns; k++) {
    sxs[k] = xsrc[pj[k]];
    sys[k] = ysrc[pj[k]];
    szs[k] = REF_DIM == 3 ? zsrc[pj[k]] : 0.0;
    sgs[k] = gsrc[pj[k]];
  }
  Q.xil = txs.data();
  Q.yil = tys.data();
  Q.xjl = sxs.data();
  Q.yjl = sys.data();
#if REF_DIM == 3
  Q.zil = tzs.data();
  Q.zjl = szs.data();
#endif
  Q.gjl = sgs.data();
  Q.wil = w.data();
  Get_vorticity v;
  v.get_vorticity(&Q, &D);
  for (int k = 0; k < nt; k++) w_out[pi[k]] = w[k];
  return 0;
}

}  // extern "C"
