/*
 * petrbf_gb300.h -- C ABI of the GB300 implementation of PetRBF's solve path.
 *
 * Plain C types only (no CUDA or torch types). Every function returns an int status
 * (PRBF_OK = 0) unless noted; no exception crosses this boundary. Host pointers unless
 * the name ends in _dev. A context owns its device memory and one CUDA stream; use one
 * context per host thread.
 *
 * Reference interfaces this ABI replaces (paths inside the petrbf project):
 *   rbf_interpolation      2d/rbf_interpolation.cxx:25-26, 3d/rbf_interpolation.cxx:26-27
 *   vorticity_evaluation   2d/vorticity_evaluation.cxx:26-27, 3d/vorticity_evaluation.cxx
 *   MatShell MATOP_MULT    mymatmult, 2d/matmult.cxx:6 (registered at 2d/rbf_interpolation.cxx:190)
 *   MATOP_GET_SUBMATRICES  mysubmat, 2d/matmult.cxx:53 (registered at 2d/rbf_interpolation.cxx:198)
 *   RBFInterpolation       3d/wrapper.cxx:20-23 (library entry of librbf.a)
 *   gpumatmult             2d/gpumatmult.cu:65-67 (the reference's C++ -> CUDA seam)
 */
#ifndef PETRBF_GB300_H
#define PETRBF_GB300_H

#ifdef __cplusplus
extern "C" {
#endif

/* Status codes. */
enum {
  PRBF_OK = 0,
  PRBF_ERR_ARG = 1,           /* bad argument (null pointer, n <= 0, dim not 2/3, ...) */
  PRBF_ERR_RANGE = 2,         /* parameters or coordinates outside the supported range */
  PRBF_ERR_CAPACITY = 3,      /* a size exceeds a kernel or scratch capacity, or device or
                               host memory is exhausted */
  PRBF_ERR_CUDA = 4,          /* CUDA runtime error (message in prbf_last_error) */
  PRBF_ERR_NOT_CONVERGED = 5, /* iteration limit reached (KSP_DIVERGED_ITS) */
  PRBF_ERR_BREAKDOWN = 6,     /* GMRES breakdown (KSP_DIVERGED_BREAKDOWN) */
  PRBF_ERR_NAN = 7,           /* NaN or Inf in the residual (KSP_DIVERGED_NANORINF) */
  PRBF_ERR_STATE = 8,         /* call out of order (e.g. matvec before matvec_setup) */
  PRBF_ERR_FACTOR = 9,        /* a subdomain block could not be factorised */
  PRBF_ERR_DIVERGED = 10,     /* residual grew past dtol (KSP_DIVERGED_DTOL) */
  PRBF_ERR_TIMEOUT = 11       /* a bounded device wait gave up (device error word set) */
};

/* Arithmetic of a solve. */
enum {
  PRBF_PREC_FP64 = 0,  /* FP64 matvec, FP64 block factors, FP64 GMRES (plain form) */
  PRBF_PREC_MIXED = 1  /* FP32 matvec + FP32 block Cholesky inside FP64 iterative refinement */
};

/* Initial guess of a solve. */
enum {
  PRBF_GUESS_ZERO = 0,    /* zero initial guess, as the reference (no KSPSetInitialGuessNonzero) */
  PRBF_GUESS_LEARNED = 1  /* per-cell MLP guess (weights from prbf_guess_set_weights) */
};

/* Schwarz preconditioner type (PETSc -pc_asm_type; the reference leaves PCASM's default,
 * restrict, in place and reads further options through KSPSetFromOptions at
 * 2d/rbf_interpolation.cxx:211, 3d/rbf_interpolation.cxx:227). */
enum {
  PRBF_PC_RASM = 0,  /* restricted: each block's solution is kept on its centre cell only */
  PRBF_PC_ASM = 1    /* basic: every block's whole solution is added back (symmetric B) */
};

/* What the FP64 set-up does with a block whose Cholesky meets a non-positive pivot (a
 * near-singular block: clustered or duplicated points). The reference factors every block
 * by PETSc's dense LU with partial pivoting (-sub_pc_type lu, 2d/Makefile:7), which solves
 * such a block unshifted and stops with an error on an exactly zero pivot.
 * PRBF_FALLBACK_LU does the same for those blocks (LU with partial pivoting of the
 * library's block; a zero pivot returns PRBF_ERR_FACTOR); PRBF_FALLBACK_SHIFT (default)
 * refactors them with a diagonal shift of 1e-12, then 1e-9, relative to the unit
 * diagonal, so that duplicated points still give a usable preconditioner. The FP32
 * set-up of the mixed form always shifts (its refinement falls back to the FP64 form). */
enum {
  PRBF_FALLBACK_SHIFT = 0,
  PRBF_FALLBACK_LU = 1
};

/* Flags of prbf_matvec_dev. */
enum {
  PRBF_ORDER_CALLER = 0, /* vectors in the order the points were given */
  PRBF_ORDER_CELL = 1,   /* vectors in cell-sorted order (the solver's internal order) */
  PRBF_MATVEC_FP32 = 2   /* FP32 pair arithmetic (the mixed-precision inner matvec) */
};

typedef struct {
  int dim;           /* 2 or 3 */
  double sigma;      /* Gaussian standard deviation */
  int nsigma_box;    /* cell edge in units of sigma */
  int sigma_buffer;  /* RASM subdomain box width in units of sigma */
  int sigma_trunc;   /* truncation box width in units of sigma */
  double rtol;       /* relative tolerance on the preconditioned residual (default 1e-13) */
  double abstol;     /* absolute tolerance (default 1e-50) */
  double dtol;       /* divergence tolerance (default 1e5) */
  int restart;       /* GMRES restart length (default 30) */
  int max_it;        /* iteration limit (default 1000) */
  int precision;     /* PRBF_PREC_* */
  int guess;         /* PRBF_GUESS_* */
  int device;        /* CUDA device ordinal (default 0) */
  int pc_type;       /* PRBF_PC_* (default PRBF_PC_RASM) */
  int block_fallback; /* PRBF_FALLBACK_* (default PRBF_FALLBACK_SHIFT) */
} prbf_params;

typedef struct {
  int its;                  /* Krylov iterations (KSPGetIterationNumber; inner total if mixed) */
  int reason;               /* KSPConvergedReason-style code: 2 rtol, 3 atol, <0 diverged */
  int outer_its;            /* iterative-refinement steps (mixed) */
  int ncell;                /* cells of the grid */
  int max_block;            /* largest RASM subdomain */
  int nblocks_fallback;     /* blocks that needed a diagonal shift, an LU or an FP64 refactor */
  double rnorm0, rnorm;     /* first and last preconditioned residual norm */
  double true_rel_resid;    /* ||f - A g||_2 / ||f||_2 in FP64 after the solve */
  double t_sort_ms;         /* cell-list build */
  double t_setup_ms;        /* RASM set-up (buffer lists, blocks, factors) */
  double t_solve_ms;        /* Krylov / refinement iterations */
  double t_total_ms;        /* whole call incl. host<->device copies */
  long long pairs_per_matvec;
  int guess_used;           /* 1 if the learned guess was kept (0: zero guess or dropped) */
  double guess_rel_resid;   /* ||f - A g0||_2 / ||f||_2 of the learned guess (mixed) or its
                               preconditioned residual relative to ||B f|| (plain); 1 = zero */
  double t_guess_ms;        /* learned-guess inference */
  int fp64_fallback;        /* mixed form: 1 if the refinement stalled (a system too
                               ill-conditioned for FP32) and the call was solved in FP64 */
} prbf_stats;

typedef struct prbf_ctx prbf_ctx;

/* Defaults: the reference's run options (2d/Makefile:7: -ksp_rtol 1e-13, -ksp_max_it 1000)
 * with PETSc's GMRES(30), dtol 1e5 and abstol 1e-50, FP64, zero guess, restricted Schwarz,
 * device 0. */
void prbf_params_default(prbf_params* p);
/* Text of a status code (no reference counterpart: the reference reports through CHKERRQ). */
const char* prbf_status_string(int status);

/* A context holds what rbf_interpolation builds and tears down on every call -- the solver
 * (KSPCreate, 2d/rbf_interpolation.cxx:210), the shell operators M and P (:190-198) and
 * their destruction (:296-307) -- kept across calls with its device memory and one stream. */
int prbf_ctx_create(const prbf_params* p, prbf_ctx** out);
int prbf_ctx_destroy(prbf_ctx* ctx);
/* Last error message of this context (valid until the next call on it; no reference
 * counterpart: CHKERRQ prints and returns). */
const char* prbf_last_error(const prbf_ctx* ctx);
/* The context's CUDA stream (a cudaStream_t), for event timing by the caller (no reference
 * counterpart). */
void* prbf_ctx_stream(prbf_ctx* ctx);
/* Waits for the context's stream (no reference counterpart: the reference's calls block). */
int prbf_ctx_synchronize(prbf_ctx* ctx);
/* Self-test of the failure path of the kernels' bounded waits (no counterpart in the
 * reference): a one-warp kernel polls, max_polls times (1 .. 2^20), an mbarrier that
 * nothing completes, raises the device error word and the call returns PRBF_ERR_TIMEOUT,
 * as any library call does when a kernel's copy or MMA wait gives up. The context stays
 * usable. */
int prbf_selftest_wait_timeout(prbf_ctx* ctx, unsigned max_polls);

/* rbf_interpolation: weights g with A g = f for n points; nrhs right-hand sides stored
 * one after the other (f[r*n + i]); weights written the same way, in the caller's order.
 * Replaces rbf_interpolation (2d/rbf_interpolation.cxx:25-26; 3d:26-27). z is ignored in
 * 2D. */
int prbf_interpolate(prbf_ctx* ctx, int n, const double* x, const double* y, const double* z,
                     const double* f, int nrhs, double* g_out, prbf_stats* stats);

/* vorticity_evaluation: w_i = sum over the truncation set of g_j phi(|x_i - x_j|) at nt
 * targets from ns sources (2d/vorticity_evaluation.cxx:26-27, 2d/get_vorticity.h:9-27). */
int prbf_evaluate(prbf_ctx* ctx, int nt, const double* xt, const double* yt, const double* zt,
                  int ns, const double* xs, const double* ys, const double* zs,
                  const double* gs, double* w_out);

/* MatShell seam: prbf_matvec_setup builds the cell list of n points on the GPU and keeps
 * it resident; prbf_matvec then applies the truncated Gaussian operator like the
 * reference's MATOP_MULT callback mymatmult (2d/matmult.cxx:6-51), host vectors in the
 * caller's order. prbf_matvec_dev takes device pointers (PRBF_ORDER_* | PRBF_MATVEC_FP32). */
int prbf_matvec_setup(prbf_ctx* ctx, int n, const double* x, const double* y, const double* z);
/* mymatmult (2d/matmult.cxx:6-51; 3d/matmult.cxx:6-52) on host vectors */
int prbf_matvec(prbf_ctx* ctx, const double* x_in, double* y_out);
/* mymatmult on device vectors: the GPU path of 2d/matmultgpu.cxx:9-97 without its per-call
 * packing and copies */
int prbf_matvec_dev(prbf_ctx* ctx, const double* x_in_dev, double* y_out_dev, int flags);
/* Cell-list queries after prbf_matvec_setup: sorted position -> caller index, per-cell
 * start offsets (ncell+1 ints), truncation-set sizes (ncell ints), and grid info
 * (ints: nx ny nz ncell nb_trunc nb_buffer max_trunc; doubles: xmin ymin zmin box). */
int prbf_matvec_info(prbf_ctx* ctx, int* ints7, double* dbls4, long long* pairs);
/* Kernels one cell-order product of the matvec seam launches (fp32 = 0: the FP64 sum, 2
 * when it takes the symmetric form -- each exponential used for both rows of a point pair,
 * the reverse contributions added by a second kernel -- else 1; fp32 = 1: the weight
 * conversion and the FP32 sum) and whether the FP64 product is symmetric. */
int prbf_matvec_kernels(prbf_ctx* ctx, int fp32, int* kernels, int* symmetric);
/* the cell sort's permutation (Get_cluster::get_cluster, 2d/get_cluster.h:123-130; the
 * isort of 2d/rbf_interpolation.cxx:124-128) */
int prbf_get_permutation(prbf_ctx* ctx, int* perm_out);
/* the per-cell point ranges (ista/iend of CLUSTER, 2d/par.h:71-124) as ncell + 1 starts */
int prbf_get_cell_start(prbf_ctx* ctx, int* cell_start_out);
/* the truncation-set size of every cell (Get_trunc::get_trunc, 2d/get_trunc.h:9-87) */
int prbf_get_trunc_counts(prbf_ctx* ctx, int* counts_out);

/* RASM preconditioner of the points given to prbf_matvec_setup: the reference's P shell
 * (MATOP_GET_SUBMATRICES = mysubmat, 2d/matmult.cxx:53-104) applied as PCASM with the
 * restricted prolongation of 2d/rbf_interpolation.cxx:213-229 (or, with the context's
 * pc_type = PRBF_PC_ASM, the basic one). precision PRBF_PREC_FP64 factorises the blocks in
 * FP64, PRBF_PREC_MIXED in FP32. prbf_pc_apply computes z = B r (host vectors, caller
 * order). */
int prbf_pc_setup(prbf_ctx* ctx, int precision);
/* PCApply of that PCASM (2d/rbf_interpolation.cxx:213-229) */
int prbf_pc_apply(prbf_ctx* ctx, const double* r, double* z);
/* Read-back of the Schwarz subdomains built by prbf_pc_setup (no counterpart in the
 * reference, whose blocks live inside PETSc): the buffer lists of Get_buffer::get_buffer
 * (2d/get_buffer.h:9-90) -- off_out[c] .. off_out[c+1]-1 (ncell + 1 entries; ncell from
 * prbf_matvec_info) index idx_out, which holds each cell's subdomain as sorted positions,
 * centre points first, in the reference's order. Either pointer may be null (call once with
 * idx_out null to learn off_out[ncell]). */
int prbf_pc_buffer_lists(prbf_ctx* ctx, long long* off_out, int* idx_out);
/* One subdomain block of cell `cell` (mysubmat, 2d/matmult.cxx:83-93): nb_out / nc_out its
 * size and centre-point count; K_out (nb x nb, nullable) the block as the FP64 factorisation
 * assembles it, K = 2 pi sigma^2 A_c, rows and columns in the factorisation's order
 * (neighbour points -- buffer entries nc .. nb-1 -- first, then the centre points), before
 * any diagonal shift; L_out (nb (nb + 1) / 2, nullable, FP64 set-up only) the packed factor
 * as the apply reads it: row i holds L[i][0..i-1] and then 1 / L[i][i], where L L^T = A_c in
 * that order. Returns PRBF_ERR_STATE for L_out after a mixed-precision set-up, or for a
 * block that PRBF_FALLBACK_LU factored by LU. */
int prbf_pc_block(prbf_ctx* ctx, int cell, int* nb_out, int* nc_out, double* K_out, double* L_out);

/* ---- batches of independent problems (no reference counterpart: the reference solves
 * one problem per call; this is the replica form for many small problems on one GPU) ---- */

/* One problem of a batch; dimension, tolerances, restart, iteration limit, precision and
 * the Schwarz type come from the context's parameters (zero guess). PRBF_PREC_FP64 solves
 * every problem with FP64 GMRES; PRBF_PREC_MIXED runs FP64 iterative refinement per
 * problem (true residual ||f - A g||_2 <= rtol ||f||_2) around GMRES with FP32 Gaussian
 * sums and FP32 block factors. */
typedef struct {
  int n;
  const double *x, *y, *z;  /* caller-order coordinates (z null in 2D) */
  const double* f;          /* right-hand side */
  double sigma;
  int nsigma_box, sigma_buffer, sigma_trunc;
  double* g_out;            /* weights, caller order (n entries) */
} prbf_problem;

typedef struct {
  int nprob;
  int nconverged;           /* problems that met the tolerance */
  int max_its, total_its;   /* GMRES iterations: slowest problem, sum over problems */
  long long points;
  long long pairs_per_matvec;
  int ncell, nblocks, min_block, max_block, nblocks_fallback;
  int tile, grid;           /* Gaussian-sum schedule chosen by the autotuner (grid 0: one
                               CTA per item) */
  double max_true_rel_resid;/* max over problems of ||f - A g||_2 / ||f||_2 */
  double t_sort_ms;         /* uploads, cell lists, truncation and buffer sizes */
  double t_setup_ms;        /* batched block factorisation */
  double t_tune_ms;         /* autotuning (0 when the schedule came from the cache) */
  double t_solve_ms;        /* lockstep GMRES */
  double t_total_ms;
  double t_matvec_ms;       /* one FP64 Gaussian sum over the whole batch (CUDA events, with
                               the chosen schedule): pairs_per_matvec / t_matvec_ms is its rate */
  double t_matvec32_ms;     /* the same for the FP32 sum (mixed form; else 0) */
  int outer_its;            /* mixed form: refinement steps of the slowest problem */
  int nprob_fp64;           /* mixed form: problems too ill-conditioned for FP32 (a block
                               whose FP32 Cholesky needed a shift, or a refinement step that
                               did not halve the FP64 residual), solved as an FP64 batch */
} prbf_batch_stats;

/* Solves every problem with GMRES + Schwarz blocks in one set of launches per iteration
 * (rbf_interpolation per problem, 2d/rbf_interpolation.cxx:25-310); its_out / reason_out
 * (nullable) receive each problem's iterations and KSPConvergedReason-style code. When a
 * problem stops short of the tolerance the call returns its status (the first failure in
 * problem order) with every problem's weights, iterations and reason written. */
int prbf_batch_interpolate(prbf_ctx* ctx, int nprob, const prbf_problem* probs, int* its_out, int* reason_out,
                           prbf_batch_stats* stats);

/* RBFInterpolation (3d/wrapper.cxx:20-105): FP32 in/out, evaluates the particles
 * (xp, yp, zp, gp) at the grid points first when xg[0] != xp[0], then solves on the
 * grid and writes the weights over wg. argc/argv are accepted and ignored. Arguments are
 * checked before any CUDA call: ng <= 0, a null grid array, or a particle array missing
 * when the particles are to be evaluated return PRBF_ERR_ARG. */
int prbf_RBFInterpolation(int argc, char** argv, int ng, float* xg, float* yg, float* zg,
                          float* wg, int np, float* xp, float* yp, float* zp, float* gp,
                          float sigma, int nsigma_box, int sigma_buffer, int sigma_trunc);

/* The reference's C++ -> CUDA seam gpumatmult (2d/gpumatmult.cu:65-67; 3d/gpumatmult.cu:73-75),
 * same argument meaning, for callers that keep the reference's host packer
 * (2d/matmultgpu.cxx:9-97): iblok blocks of 128 FP32 target slots (tX, tY[, tZ]; slots past a
 * cell's points zero-padded), the blocks' truncation sets packed one after the other
 * (sX, sY[, sZ], sG; block b's at offset[b] .. offset[b+1]-1, iblok + 1 offsets), sigma, and
 * the capacities the caller allocated (numCluster*128 target slots, numCluster*numTrunc
 * sources; iblok <= numCluster, offset[iblok] <= numCluster*numTrunc). Writes
 * tW[128 b + i] = sum_j sG_j exp(-|t - s_j|^2 / (2 sigma^2)) / (2 pi sigma^2) for the
 * 128 * iblok slots (the 3D form keeps this 2D normalisation, as the reference's does).
 * FP32 arithmetic on the caller's coordinates, the exponential on the special-function unit
 * (ex2.approx, subnormal terms flushed to zero) where the reference calls exp: each slot is
 * within 1e-5 x sum_j |sG_j phi_ij| of the exactly rounded sum of the same FP32 inputs and
 * within 2e-5 (same measure) of the reference kernel's own output, not bit-identical to it.
 * Host pointers; the call is synchronous and
 * returns a PRBF_* status (the reference's returns void and checks nothing). Device
 * buffers are grow-only and kept per device for the life of the process, as the
 * reference's statics are; concurrent calls are serialised. */
int prbf_gpumatmult_2d(const float* tX, const float* tY, float* tW, const float* sX, const float* sY,
                       const float* sG, const int* offset, int iblok, float sigma, int numCluster,
                       int numTrunc);
/* the 3D seam, 3d/gpumatmult.cu:73-75 (3d/matmultgpu.cxx:7 packs its arrays) */
int prbf_gpumatmult_3d(const float* tX, const float* tY, const float* tZ, float* tW, const float* sX,
                       const float* sY, const float* sZ, const float* sG, const int* offset, int iblok,
                       float sigma, int numCluster, int numTrunc);

/* Cell sort that allocates nothing (no counterpart in the reference). For callers that
 * must not allocate device memory themselves -- an application that reserves the whole
 * GPU for its own memory pool, or a latency-critical loop that cannot afford the device
 * synchronisation cudaMalloc/cudaFree imply -- it sorts n points into the same cells, in
 * the same order, as prbf_matvec_setup: perm_dev[k] = caller index of the k-th sorted
 * point, cell_start_dev[c] = first sorted position of cell c (ncell + 1 entries; the grid
 * is derived from the points' bounding box, so the caller passes the capacity it
 * allocated and receives ncell, also when that capacity is too small, so it learns what to
 * allocate). All pointers are device pointers; stream may be null.
 * Every temporary comes from one fixed device array inside the library
 * (PRBF_STATIC_SORT_SCRATCH_MIB MiB, held on every GPU that loads the library until the
 * process exits). Limits: n <= PRBF_STATIC_SORT_MAX_POINTS and ncell + 1 <= 8,388,608;
 * beyond them the call returns PRBF_ERR_CAPACITY without touching perm_dev or
 * cell_start_dev (ncell_out is still written when the cell count is the limit hit). The first
 * call on a device looks up the array's device address (cudaGetSymbolAddress) with that
 * device current; make that first call before any stream capture. All calls share the
 * array: calls that overlap on the GPU (other threads, other streams) race and must be
 * serialised by the caller. The call synchronises the stream twice: to read the bounding
 * box back, and to read the kernels' status word at the end. */
#define PRBF_STATIC_SORT_MAX_POINTS 1048576
#define PRBF_STATIC_SORT_SCRATCH_MIB 13
int prbf_cell_sort_static(int dim, int n, const double* x_dev, const double* y_dev, const double* z_dev,
                          double sigma, int nsigma_box, int sigma_buffer, int sigma_trunc,
                          int* perm_dev, int* cell_start_dev, int cell_start_len, int* ncell_out,
                          void* stream);

#ifdef __cplusplus
}
/* The same entry under the reference's own name and C++ linkage (3d/wrapper.cxx:20-23):
 * a caller that linked librbf.a keeps its declaration and call and links this library. */
int RBFInterpolation(int argc, char** argv, int ng, float* xg, float* yg, float* zg, float* wg, int np, float* xp,
                     float* yp, float* zp, float* gp, float sigma, int nsigma_box, int sigma_buffer, int sigma_trunc);
#endif
#endif
