// Test driver for the PETSc glue (petrbf_gb300/glue/petrbf_petsc.cxx): built against the
// sequential PETSc stand-in (oracle/ref_stub) and the CUDA library, it calls the
// reference's entry points the way the reference's callers do -- rbf_interpolation and
// vorticity_evaluation on Vecs (2d/main.cxx:124-125), the MatShell MATOP_MULT body
// mymatmult and a PCShell apply on a shell context, and RBFInterpolation with the
// reference's C++ signature (3d/wrapper.cxx:20-23) -- and writes the results for the
// Python test to compare with the C ABI's.
//
// Input (binary, native endianness): int n, nt, n3; double sigma, sigma3; int nbox,
// nbuf, ntrunc, nbox3, nbuf3, ntrunc3; double x[n], y[n], f[n], r[n], xt[nt], yt[nt];
// float xg[n3], yg[n3], zg[n3], wg[n3], xp[n3], yp[n3], zp[n3], gp[n3].
// Output: int its, status[6]; double g[n], w[nt], Ar[n], Br[n]; float wg_solve[n3],
// wg_eval[n3].
#include <petscksp.h>

#include <cstdio>
#include <vector>

#include "petrbf_petsc.h"

static Vec vec_of(const std::vector<double>& a) {
  Vec v;
  VecCreate(PETSC_COMM_WORLD, &v);
  VecSetSizes(v, (PetscInt)a.size(), PETSC_DETERMINE);
  PetscScalar* p;
  VecGetArray(v, &p);
  for (size_t i = 0; i < a.size(); i++) p[i] = a[i];
  VecRestoreArray(v, &p);
  return v;
}

static std::vector<double> vals(Vec v) {
  PetscInt n;
  VecGetLocalSize(v, &n);
  const PetscScalar* p;
  VecGetArrayRead(v, &p);
  std::vector<double> out(p, p + n);
  VecRestoreArrayRead(v, &p);
  return out;
}

template <class T>
static bool rd(FILE* f, std::vector<T>& a, size_t n) {
  a.resize(n);
  return fread(a.data(), sizeof(T), n, f) == n;
}

int main(int argc, char** argv) {
  if (argc != 3) return 2;
  FILE* in = std::fopen(argv[1], "rb");
  if (!in) return 2;
  int hdr[3];
  double sg[2];
  int prm[6];
  if (fread(hdr, sizeof(int), 3, in) != 3 || fread(sg, sizeof(double), 2, in) != 2 ||
      fread(prm, sizeof(int), 6, in) != 6)
    return 2;
  const int n = hdr[0], nt = hdr[1], n3 = hdr[2];
  std::vector<double> x, y, f, r, xt, yt;
  std::vector<float> xg, yg, zg, wg, xp, yp, zp, gp;
  if (!rd(in, x, n) || !rd(in, y, n) || !rd(in, f, n) || !rd(in, r, n) || !rd(in, xt, nt) || !rd(in, yt, nt) ||
      !rd(in, xg, n3) || !rd(in, yg, n3) || !rd(in, zg, n3) || !rd(in, wg, n3) || !rd(in, xp, n3) ||
      !rd(in, yp, n3) || !rd(in, zp, n3) || !rd(in, gp, n3))
    return 2;
  std::fclose(in);
  int status[6] = {0, 0, 0, 0, 0, 0}, its = -1;
  // rbf_interpolation, then the interpolant at the targets
  Vec xi = vec_of(x), yi = vec_of(y), wi = vec_of(f), gi = vec_of(std::vector<double>(n, 0.0));
  status[0] = rbf_interpolation(xi, yi, gi, wi, sg[0], prm[0], prm[1], prm[2], &its);
  Vec xv = vec_of(xt), yv = vec_of(yt), wv = vec_of(std::vector<double>(nt, 0.0));
  status[1] = vorticity_evaluation(xv, yv, wv, xi, yi, gi, sg[0], prm[0], prm[1], prm[2]);
  // the shell operator and preconditioner on the same points
  prbf_ctx* ctx = nullptr;
  status[2] = petrbf_shell_create(xi, yi, nullptr, sg[0], prm[0], prm[1], prm[2], PRBF_PREC_FP64, &ctx);
  Mat A;
  MatCreate(PETSC_COMM_WORLD, &A);
  MatShellSetContext(A, ctx);
  _p_PC pcs;
  PC pc = &pcs;
  PCShellSetContext(pc, ctx);
  Vec rv = vec_of(r), Ar = vec_of(std::vector<double>(n, 0.0)), Br = vec_of(std::vector<double>(n, 0.0));
  if (!status[2]) {
    status[3] = mymatmult(A, rv, Ar);
    status[4] = petrbf_pcapply(pc, rv, Br);
  }
  petrbf_shell_destroy(&ctx);
  MatDestroy(&A);
  // RBFInterpolation (3d/wrapper.cxx): solve on the particles themselves, then evaluate a
  // shifted particle field at the grid first (xg[0] != xp[0])
  std::vector<float> w_solve = wg, w_eval = wg;
  status[5] = RBFInterpolation(0, nullptr, n3, xg.data(), yg.data(), zg.data(), w_solve.data(), n3, xg.data(),
                               yg.data(), zg.data(), wg.data(), (float)sg[1], prm[3], prm[4], prm[5]);
  if (!status[5])
    status[5] = RBFInterpolation(0, nullptr, n3, xg.data(), yg.data(), zg.data(), w_eval.data(), n3, xp.data(),
                                 yp.data(), zp.data(), gp.data(), (float)sg[1], prm[3], prm[4], prm[5]);
  FILE* out = std::fopen(argv[2], "wb");
  if (!out) return 2;
  fwrite(&its, sizeof(int), 1, out);
  fwrite(status, sizeof(int), 6, out);
  for (Vec v : {gi, wv, Ar, Br}) {
    std::vector<double> a = vals(v);
    fwrite(a.data(), sizeof(double), a.size(), out);
  }
  fwrite(w_solve.data(), sizeof(float), n3, out);
  fwrite(w_eval.data(), sizeof(float), n3, out);
  std::fclose(out);
  for (Vec v : {xi, yi, wi, gi, xv, yv, wv, rv, Ar, Br}) VecDestroy(&v);
  return 0;
}
