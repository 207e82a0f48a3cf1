/*
 * Sequential PETSc stand-in -- TEST INFRASTRUCTURE ONLY.
 *
 * Provides just the Vec/Mat/IS calls that the reference's cell-list, truncation,
 * buffer, matvec, block and evaluation code makes (2d|3d/get_cluster.h,
 * get_trunc.h, get_buffer.h, get_vorticity.h, matmult.cxx), on one process with
 * plain dense storage, so those files compile unmodified and produce golden vectors.
 * KSP and PCASM are deliberately absent: the Krylov solver is not exercised through this
 * stand-in. The few extra Vec/Mat/PC shell calls at the end let the package's PETSc glue
 * (petrbf_gb300/glue/petrbf_petsc.cxx) compile and run against it in the tests, with the
 * signatures PETSc declares for them.
 */
#ifndef PRBF_REF_STUB_PETSCKSP_H
#define PRBF_REF_STUB_PETSCKSP_H
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <vector>
#include "mpi.h"

typedef int PetscErrorCode;
typedef int PetscInt;
typedef double PetscScalar;
typedef double PetscReal;
typedef int PetscBool;

struct _p_Vec { std::vector<double> a; };
struct _p_Mat { int m = 0, n = 0; std::vector<double> a; void* ctx = nullptr; };
struct _p_IS { std::vector<int> i; };
typedef _p_Vec* Vec;
typedef _p_Mat* Mat;
typedef _p_IS* IS;
typedef enum { MAT_INITIAL_MATRIX, MAT_REUSE_MATRIX } MatReuse;
typedef enum { INSERT_VALUES, ADD_VALUES } InsertMode;
typedef enum { SCATTER_FORWARD, SCATTER_REVERSE } ScatterMode;
typedef enum { MAT_FLUSH_ASSEMBLY, MAT_FINAL_ASSEMBLY } MatAssemblyType;

#define PETSC_COMM_WORLD 0
#define PETSC_COMM_SELF 1
#define PETSC_DETERMINE (-1)
#define PETSC_DECIDE (-1)
#define PETSC_NULL nullptr
#define CHKERRQ(e) do { if (e) return (e); } while (0)
#define PetscFunctionBegin
#define PetscFunctionReturn(v) return (v)

static inline PetscErrorCode VecCreate(MPI_Comm, Vec* v) { *v = new _p_Vec; return 0; }
static inline PetscErrorCode VecSetSizes(Vec v, PetscInt n, PetscInt) { v->a.assign(n, 0.0); return 0; }
static inline PetscErrorCode VecSetFromOptions(Vec) { return 0; }
static inline PetscErrorCode VecSetValues(Vec v, PetscInt n, const PetscInt* ix, const PetscScalar* y, InsertMode m) {
  for (int k = 0; k < n; k++) { if (m == INSERT_VALUES) v->a[ix[k]] = y[k]; else v->a[ix[k]] += y[k]; }
  return 0;
}
static inline PetscErrorCode VecAssemblyBegin(Vec) { return 0; }
static inline PetscErrorCode VecAssemblyEnd(Vec) { return 0; }
static inline PetscErrorCode VecGhostUpdateBegin(Vec, InsertMode, ScatterMode) { return 0; }
static inline PetscErrorCode VecGhostUpdateEnd(Vec, InsertMode, ScatterMode) { return 0; }
static inline PetscErrorCode VecGetArray(Vec v, PetscScalar** p) { *p = v->a.data(); return 0; }
static inline PetscErrorCode VecRestoreArray(Vec, PetscScalar**) { return 0; }
static inline PetscErrorCode VecDestroy(Vec* v) { delete *v; *v = nullptr; return 0; }
static inline PetscErrorCode PetscLogFlops(double) { return 0; }

template <class T>
static inline PetscErrorCode PetscMalloc(size_t sz, T** p) { *p = (T*)std::calloc(1, sz); return 0; }

static inline PetscErrorCode MatCreate(MPI_Comm, Mat* m) { *m = new _p_Mat; return 0; }
static inline PetscErrorCode MatShellGetContext(Mat m, void** c) { *c = m->ctx; return 0; }
static inline PetscErrorCode MatSetOptionsPrefix(Mat, const char*) { return 0; }
static inline PetscErrorCode MatSetSizes(Mat m, PetscInt a, PetscInt b, PetscInt, PetscInt) {
  m->m = a; m->n = b; m->a.assign((size_t)a * b, 0.0); return 0;
}
static inline PetscErrorCode MatSetFromOptions(Mat) { return 0; }
static inline PetscErrorCode MatSeqAIJSetPreallocation(Mat, PetscInt, const PetscInt*) { return 0; }
static inline PetscErrorCode MatSetUp(Mat) { return 0; }
static inline PetscErrorCode MatSetValues(Mat m, PetscInt nr, const PetscInt* ir, PetscInt nc, const PetscInt* ic,
                                          const PetscScalar* v, InsertMode) {
  for (int i = 0; i < nr; i++) for (int j = 0; j < nc; j++) m->a[(size_t)ir[i] * m->n + ic[j]] = v[(size_t)i * nc + j];
  return 0;
}
static inline PetscErrorCode MatAssemblyBegin(Mat, MatAssemblyType) { return 0; }
static inline PetscErrorCode MatAssemblyEnd(Mat, MatAssemblyType) { return 0; }
static inline PetscErrorCode MatDestroy(Mat* m) { delete *m; *m = nullptr; return 0; }

// ---- for the PETSc glue of the package (one process: local = global sizes) ----------
#define PETSC_ERR_LIB 76
struct _p_PC { void* ctx = nullptr; };
typedef _p_PC* PC;
static inline PetscErrorCode VecGetLocalSize(Vec v, PetscInt* n) { *n = (PetscInt)v->a.size(); return 0; }
static inline PetscErrorCode VecGetArrayRead(Vec v, const PetscScalar** p) { *p = v->a.data(); return 0; }
static inline PetscErrorCode VecRestoreArrayRead(Vec, const PetscScalar**) { return 0; }
static inline PetscErrorCode MatShellSetContext(Mat m, void* c) { m->ctx = c; return 0; }
static inline PetscErrorCode PCShellGetContext(PC pc, void* c) { *(void**)c = pc->ctx; return 0; }
static inline PetscErrorCode PCShellSetContext(PC pc, void* c) { pc->ctx = c; return 0; }
#endif
