// petrbf_petsc.cxx -- the reference's PETSc entry points on the GB300 library (declared in
// include/petrbf_petsc.h). Compiled into a PETSc application's build against its PETSc
// headers and linked with -lpetrbf_gb300 -lcudart; the tests compile it against a
// sequential stand-in. Each function borrows the Vecs' arrays (VecGetArray / Restore, as
// the reference does, 2d/rbf_interpolation.cxx:202-208), calls the C ABI, and returns
// the reference's error convention.
#include <petscksp.h>

#include <cstdio>
#include <vector>

#include "petrbf_petsc.h"

namespace {

PetscErrorCode lib_error(prbf_ctx* ctx, int st, const char* what) {
  std::fprintf(stderr, "petrbf_gb300: %s: %s (%s)\n", what, prbf_status_string(st),
               ctx ? prbf_last_error(ctx) : "");
  return PETSC_ERR_LIB;
}

// A context with the reference's solver options (GMRES(30), rtol 1e-13, zero guess,
// restricted Schwarz, FP64, LU on the blocks the Cholesky cannot factor; 2d/Makefile:7).
int make_ctx(int dim, double sigma, int nsigma_box, int sigma_buffer, int sigma_trunc, prbf_ctx** ctx) {
  prbf_params p;
  prbf_params_default(&p);
  p.block_fallback = PRBF_FALLBACK_LU;
  p.dim = dim;
  p.sigma = sigma;
  p.nsigma_box = nsigma_box;
  p.sigma_buffer = sigma_buffer;
  p.sigma_trunc = sigma_trunc;
  return prbf_ctx_create(&p, ctx);
}

// Borrowed read-only arrays of up to three coordinate Vecs plus their common length.
struct Coords {
  Vec v[3] = {nullptr, nullptr, nullptr};
  const PetscScalar* a[3] = {nullptr, nullptr, nullptr};
  PetscInt n = 0;
  PetscErrorCode get(Vec x, Vec y, Vec z) {
    v[0] = x;
    v[1] = y;
    v[2] = z;
    PetscErrorCode ierr = VecGetLocalSize(x, &n);
    CHKERRQ(ierr);
    for (int d = 0; d < 3; d++)
      if (v[d]) {
        PetscInt m = 0;
        ierr = VecGetLocalSize(v[d], &m);
        CHKERRQ(ierr);
        if (m != n) return PETSC_ERR_LIB;
        ierr = VecGetArrayRead(v[d], &a[d]);
        CHKERRQ(ierr);
      }
    return 0;
  }
  ~Coords() {
    for (int d = 0; d < 3; d++)
      if (v[d] && a[d]) VecRestoreArrayRead(v[d], &a[d]);
  }
};

PetscErrorCode interpolate(int dim, Vec xi, Vec yi, Vec zi, Vec gi, Vec wi, double sigma, int nsigma_box,
                           int sigma_buffer, int sigma_trunc, int* its) {
  Coords c;
  PetscErrorCode ierr = c.get(xi, yi, zi);
  CHKERRQ(ierr);
  PetscInt nw = 0, ng = 0;
  ierr = VecGetLocalSize(wi, &nw);
  CHKERRQ(ierr);
  ierr = VecGetLocalSize(gi, &ng);
  CHKERRQ(ierr);
  if (nw != c.n || ng != c.n) return PETSC_ERR_LIB;
  prbf_ctx* ctx = nullptr;
  int st = make_ctx(dim, sigma, nsigma_box, sigma_buffer, sigma_trunc, &ctx);
  if (st) return lib_error(nullptr, st, "context");
  const PetscScalar* w = nullptr;
  PetscScalar* g = nullptr;
  VecGetArrayRead(wi, &w);
  VecGetArray(gi, &g);
  prbf_stats s;
  st = prbf_interpolate(ctx, (int)c.n, c.a[0], c.a[1], c.a[2], w, 1, g, &s);
  VecRestoreArrayRead(wi, &w);
  VecRestoreArray(gi, &g);
  if (its) *its = s.its;  // KSPGetIterationNumber (2d/rbf_interpolation.cxx:234)
  ierr = st ? lib_error(ctx, st, "rbf_interpolation") : 0;
  prbf_ctx_destroy(ctx);
  return ierr;
}

PetscErrorCode evaluate(int dim, Vec xi, Vec yi, Vec zi, Vec wi, Vec xj, Vec yj, Vec zj, Vec gj, double sigma,
                        int nsigma_box, int sigma_buffer, int sigma_trunc) {
  Coords t, s;
  PetscErrorCode ierr = t.get(xi, yi, zi);
  CHKERRQ(ierr);
  ierr = s.get(xj, yj, zj);
  CHKERRQ(ierr);
  PetscInt nw = 0, ng = 0;
  ierr = VecGetLocalSize(wi, &nw);
  CHKERRQ(ierr);
  ierr = VecGetLocalSize(gj, &ng);
  CHKERRQ(ierr);
  if (nw != t.n || ng != s.n) return PETSC_ERR_LIB;
  prbf_ctx* ctx = nullptr;
  int st = make_ctx(dim, sigma, nsigma_box, sigma_buffer, sigma_trunc, &ctx);
  if (st) return lib_error(nullptr, st, "context");
  const PetscScalar* g = nullptr;
  PetscScalar* w = nullptr;
  VecGetArrayRead(gj, &g);
  VecGetArray(wi, &w);
  st = prbf_evaluate(ctx, (int)t.n, t.a[0], t.a[1], t.a[2], (int)s.n, s.a[0], s.a[1], s.a[2], g, w);
  VecRestoreArrayRead(gj, &g);
  VecRestoreArray(wi, &w);
  ierr = st ? lib_error(ctx, st, "vorticity_evaluation") : 0;
  prbf_ctx_destroy(ctx);
  return ierr;
}

}  // namespace

PetscErrorCode rbf_interpolation(Vec xi, Vec yi, Vec gi, Vec wi, double sigma, int nsigma_box, int sigma_buffer,
                                 int sigma_trunc, int* its) {
  return interpolate(2, xi, yi, nullptr, gi, wi, sigma, nsigma_box, sigma_buffer, sigma_trunc, its);
}

PetscErrorCode rbf_interpolation(Vec xi, Vec yi, Vec zi, Vec gi, Vec wi, double sigma, int nsigma_box,
                                 int sigma_buffer, int sigma_trunc, int* its) {
  return interpolate(3, xi, yi, zi, gi, wi, sigma, nsigma_box, sigma_buffer, sigma_trunc, its);
}

PetscErrorCode vorticity_evaluation(Vec xi, Vec yi, Vec wi, Vec xj, Vec yj, Vec gj, double sigma, int nsigma_box,
                                    int sigma_buffer, int sigma_trunc) {
  return evaluate(2, xi, yi, nullptr, wi, xj, yj, nullptr, gj, sigma, nsigma_box, sigma_buffer, sigma_trunc);
}

PetscErrorCode vorticity_evaluation(Vec xi, Vec yi, Vec zi, Vec wi, Vec xj, Vec yj, Vec zj, Vec gj, double sigma,
                                    int nsigma_box, int sigma_buffer, int sigma_trunc) {
  return evaluate(3, xi, yi, zi, wi, xj, yj, zj, gj, sigma, nsigma_box, sigma_buffer, sigma_trunc);
}

PetscErrorCode petrbf_shell_create(Vec xi, Vec yi, Vec zi, double sigma, int nsigma_box, int sigma_buffer,
                                   int sigma_trunc, int precision, prbf_ctx** ctx) {
  if (!ctx) return PETSC_ERR_LIB;
  *ctx = nullptr;
  Coords c;
  PetscErrorCode ierr = c.get(xi, yi, zi);
  CHKERRQ(ierr);
  int st = make_ctx(zi ? 3 : 2, sigma, nsigma_box, sigma_buffer, sigma_trunc, ctx);
  if (st) return lib_error(nullptr, st, "context");
  st = prbf_matvec_setup(*ctx, (int)c.n, c.a[0], c.a[1], c.a[2]);
  if (!st) st = prbf_pc_setup(*ctx, precision);
  if (st) {
    ierr = lib_error(*ctx, st, "shell set-up");
    prbf_ctx_destroy(*ctx);
    *ctx = nullptr;
    return ierr;
  }
  return 0;
}

PetscErrorCode mymatmult(Mat A, Vec x, Vec y) {
  prbf_ctx* ctx = nullptr;
  PetscErrorCode ierr = MatShellGetContext(A, (void**)&ctx);
  CHKERRQ(ierr);
  const PetscScalar* xa = nullptr;
  PetscScalar* ya = nullptr;
  VecGetArrayRead(x, &xa);
  VecGetArray(y, &ya);
  const int st = prbf_matvec(ctx, xa, ya);
  VecRestoreArrayRead(x, &xa);
  VecRestoreArray(y, &ya);
  return st ? lib_error(ctx, st, "mymatmult") : 0;
}

PetscErrorCode petrbf_pcapply(PC pc, Vec r, Vec z) {
  prbf_ctx* ctx = nullptr;
  PetscErrorCode ierr = PCShellGetContext(pc, (void**)&ctx);
  CHKERRQ(ierr);
  const PetscScalar* ra = nullptr;
  PetscScalar* za = nullptr;
  VecGetArrayRead(r, &ra);
  VecGetArray(z, &za);
  const int st = prbf_pc_apply(ctx, ra, za);
  VecRestoreArrayRead(r, &ra);
  VecRestoreArray(z, &za);
  return st ? lib_error(ctx, st, "PC apply") : 0;
}

PetscErrorCode petrbf_shell_destroy(prbf_ctx** ctx) {
  if (ctx && *ctx) {
    prbf_ctx_destroy(*ctx);
    *ctx = nullptr;
  }
  return 0;
}
