/*
 * petrbf_petsc.h -- the reference's PETSc-facing entry points, over the C ABI of
 * petrbf_gb300.h (C++, include after petscksp.h). Implemented by
 * petrbf_gb300/glue/petrbf_petsc.cxx, which a PETSc application compiles into its own
 * build (it needs the application's PETSc headers; the CUDA library itself does not).
 * Same names, arguments and meaning as the reference's functions, so the reference's
 * callers (main, the 3D wrapper, an external vortex code) relink without source changes.
 *
 * Errors follow the reference's convention: 0 on success, else a nonzero PetscErrorCode
 * (PETSC_ERR_LIB when the library returns a status; the status is logged on stderr with
 * its message).
 */
#ifndef PETRBF_PETSC_H
#define PETRBF_PETSC_H
#include "petrbf_gb300.h"

/* rbf_interpolation (2d/rbf_interpolation.cxx:25-26): weights gi with A gi = wi, its the
 * GMRES iterations. Vecs in the caller's order; gi is overwritten. */
PetscErrorCode rbf_interpolation(Vec xi, Vec yi, Vec gi, Vec wi, double sigma, int nsigma_box, int sigma_buffer,
                                 int sigma_trunc, int* its);
/* the 3D form (3d/rbf_interpolation.cxx:26-27) */
PetscErrorCode rbf_interpolation(Vec xi, Vec yi, Vec zi, Vec gi, Vec wi, double sigma, int nsigma_box,
                                 int sigma_buffer, int sigma_trunc, int* its);
/* vorticity_evaluation (2d/vorticity_evaluation.cxx:26-27): wi at the targets (xi, yi)
 * from the sources (xj, yj) with weights gj. */
PetscErrorCode vorticity_evaluation(Vec xi, Vec yi, Vec wi, Vec xj, Vec yj, Vec gj, double sigma, int nsigma_box,
                                    int sigma_buffer, int sigma_trunc);
/* the 3D form (3d/vorticity_evaluation.cxx:26-27) */
PetscErrorCode vorticity_evaluation(Vec xi, Vec yi, Vec zi, Vec wi, Vec xj, Vec yj, Vec zj, Vec gj, double sigma,
                                    int nsigma_box, int sigma_buffer, int sigma_trunc);

/* For a caller that keeps PETSc's own KSP and moves only the operator and the Schwarz
 * preconditioner to the GPU: petrbf_shell_create sorts the points into cells and builds
 * the Schwarz blocks once (the set-up of 2d/rbf_interpolation.cxx:110-230, in FP64 or,
 * precision PRBF_PREC_MIXED, FP32 blocks); give the context to MatShellSetContext and
 * PCShellSetContext. mymatmult is the MATOP_MULT body with the reference's signature
 * (2d/matmult.cxx:6; registered at 2d/rbf_interpolation.cxx:190-191), y = A x in the Vecs'
 * order; petrbf_pcapply is a PCShell apply, z = B r (the restricted additive Schwarz that
 * PCASM builds from mysubmat's blocks, 2d/rbf_interpolation.cxx:213-229). The context
 * must outlive the Mat and PC; petrbf_shell_destroy frees it. zi null in 2D. */
PetscErrorCode petrbf_shell_create(Vec xi, Vec yi, Vec zi, double sigma, int nsigma_box, int sigma_buffer,
                                   int sigma_trunc, int precision, prbf_ctx** ctx);
PetscErrorCode mymatmult(Mat A, Vec x, Vec y);
PetscErrorCode petrbf_pcapply(PC pc, Vec r, Vec z);
PetscErrorCode petrbf_shell_destroy(prbf_ctx** ctx);
#endif
