/*
 * prbf_oracle.h -- TEST INFRASTRUCTURE ONLY.
 *
 * CPU restatement of PetRBF's solve path (cell list, truncation and buffer sets,
 * truncated Gaussian matvec, dense subdomain blocks, dense LU with partial pivoting (and,
 * as a second form, the GPU library's own block Cholesky arithmetic restated),
 * restricted additive Schwarz, GMRES(restart) with left preconditioning, evaluation).
 * It is the checker for the CUDA path and the timed CPU baseline; the product never
 * links, loads or calls it.
 *
 * Parity status: the cell list, truncation/buffer sets, matvec, blocks and evaluation
 * are pinned against the reference's own code (get_cluster.h, get_trunc.h,
 * get_buffer.h, get_vorticity.h, matmult.cxx compiled unmodified against a sequential
 * PETSc/MPI stand-in, see oracle/ref_driver.cpp). GMRES, PCASM and the dense LU live
 * in PETSc, which is not part of the reference and not available here: those pieces
 * restate PETSc's documented defaults and are "parity unpinned" (iteration counts and
 * residual histories); their converged answers are pinned mathematically by the
 * residual they reach.
 */
#ifndef PRBF_ORACLE_H
#define PRBF_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

/* Cell grid, as computed by 2d/get_cluster.h:176-190 (3d/get_cluster.h:21-44). */
typedef struct {
  int dim;
  int nx, ny, nz, ncell;
  int nsigma_box, sigma_buffer, sigma_trunc;
  int nb_trunc, nb_buffer;  /* neighbor_trunc, neighbor_buffer */
  double sigma;
  double xmin, ymin, zmin;  /* particle minimum - epsf */
  double box;               /* nsigma_box*sigma + epsf */
  double trunc_len;         /* sigma_trunc*sigma/2 + epsf  (2d/get_trunc.h:14) */
  double buffer_len;        /* sigma_buffer*sigma/2 + epsf (2d/get_buffer.h:11) */
} orc_grid;

int orc_grid_make(int dim, double pxmin, double pxmax, double pymin, double pymax,
                  double pzmin, double pzmax, double sigma, int nsigma_box,
                  int sigma_buffer, int sigma_trunc, orc_grid* g);
int orc_cell_ids(const orc_grid* g, int n, const double* x, const double* y,
                 const double* z, int* cell);
int orc_cell_sort(const orc_grid* g, int n, const double* x, const double* y,
                  const double* z, int* perm, int* cell_start);
int orc_trunc_counts(const orc_grid* g, const double* sx, const double* sy,
                     const double* sz, const int* cs_src, const int* cs_tgt,
                     int* counts);
int orc_trunc_list(const orc_grid* g, int cell, const double* sx, const double* sy,
                   const double* sz, const int* cs_src, const int* cs_tgt, int* idx);
int orc_gauss_sum(const orc_grid* g, const double* tx, const double* ty,
                  const double* tz, const int* cs_tgt, const double* sx,
                  const double* sy, const double* sz, const double* sg,
                  const int* cs_src, double* w);
int orc_buffer_counts(const orc_grid* g, const double* x, const double* y,
                      const double* z, const int* cs, int* counts);
int orc_buffer_fill(const orc_grid* g, const double* x, const double* y,
                    const double* z, const int* cs, const long long* offsets, int* idx);
int orc_block(const orc_grid* g, int nb, const int* idx, const double* x,
              const double* y, const double* z, double* A);

void* orc_rasm_create(const orc_grid* g, int n, const double* x, const double* y,
                      const double* z, const int* cs, int* status);
/* kind 0: dense LU with partial pivoting (PETSc's -sub_pc_type lu, the reference's);
 * kind 1: the GPU library's arithmetic -- blocks K = 2 pi sigma^2 A_c with the neighbour
 * points first, its table exp, the ordered Cholesky and the apply's substitution order;
 * kind 2: kind 1 with the GPU's LU fallback (a block whose Cholesky meets a non-positive
 * pivot is factored by LU with partial pivoting instead of shifted; a zero pivot fails). */
void* orc_rasm_create_kind(const orc_grid* g, int n, const double* x, const double* y,
                           const double* z, const int* cs, int kind, int* status);
int orc_rasm_block_info(void* h, int cell, int* nb, int* nc, int* nshifted);
/* kind 1: the packed factor rows of a cell (row i: L_A[i][0..i-1], 1/L_A[i][i]) */
int orc_rasm_factor_rows(void* h, int cell, double* out);
/* 1 if kind 1's blocked Cholesky reproduces the unblocked loop it restates bit for bit on
 * the SPD matrix K (n x n row-major, lower triangle read) */
int orc_chol_blocked_matches_unblocked(int n, const double* K);
/* kind 1's block K (nb x nb row-major, lower triangle, neighbours first) of one buffer list */
int orc_gpu_block(const orc_grid* g, int nb, int nc, const int* idx, const double* x,
                  const double* y, const double* z, double* K);
int orc_rasm_apply(void* h, const double* r, double* out);
int orc_rasm_set_type(void* h, int basic);  /* 1: basic additive Schwarz (-pc_asm_type basic) */
void orc_rasm_destroy(void* h);

int orc_gmres(const orc_grid* g, int n, const double* x, const double* y,
              const double* z, const int* cs, void* rasm, const double* b,
              const double* x0, double rtol, double abstol, double dtol, int restart,
              int max_it, double* xsol, int* its, int* reason, double* hist);

int orc_gmres_ex(const orc_grid* g, int n, const double* x, const double* y,
                 const double* z, const int* cs, void* rasm, const double* b,
                 const double* x0, double rtol, double abstol, double dtol, int restart,
                 int max_it, double* xsol, int* its, int* reason, double* hist, int flags);

/* pc_flags: bit 0 basic additive Schwarz (-pc_asm_type basic); bit 1 the GPU's Cholesky
 * blocks (kind 1) instead of LU; bit 2 the GPU's table exp in the Gaussian sums; bit 3 the
 * sums' terms added in reverse order (a rounding-order probe); bit 4 with bit 1, the LU
 * fallback (kind 2). */
int orc_rbf_interpolation(int dim, int n, const double* x, const double* y,
                          const double* z, const double* f, double sigma,
                          int nsigma_box, int sigma_buffer, int sigma_trunc,
                          double rtol, int restart, int max_it, double* g_out,
                          int* its, int* reason, int pc_flags);
int orc_vorticity_evaluation(int dim, int nt, const double* xt, const double* yt,
                             const double* zt, int ns, const double* xs,
                             const double* ys, const double* zs, const double* gs,
                             double sigma, int nsigma_box, int sigma_buffer,
                             int sigma_trunc, double* w_out);
int orc_num_threads(void);

#ifdef __cplusplus
}
#endif
#endif
