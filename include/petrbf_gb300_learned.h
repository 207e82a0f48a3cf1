/*
 * petrbf_gb300_learned.h -- the learned initial guess (no counterpart in the reference).
 *
 * A per-cell MLP maps the particles of a 3 x 3 neighbourhood of fine cells (2 sigma edge,
 * up to 64 particles: offsets/sigma, right-hand-side values, presence) to starting weights
 * of the centre cell. Three hidden layers of width 256, BF16 weights, FP32 accumulation;
 * forward, backward and Adam are this library's own CUDA kernels. The solve treats the
 * guess as a hint only: GMRES (or the refinement loop) runs to the same tolerance, relative
 * to the zero-guess residual, and a guess whose residual is larger than the zero guess's is
 * dropped.
 */
#ifndef PETRBF_GB300_LEARNED_H
#define PETRBF_GB300_LEARNED_H

#include "petrbf_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

enum {
  PRBF_MLP_PTS = 64,   /* particles per patch */
  PRBF_MLP_IN = 256,   /* input features per patch (4 per particle) */
  PRBF_MLP_HID = 256,  /* hidden width */
  PRBF_MLP_OUT = 16    /* centre-cell weights per patch */
};

typedef struct prbf_mlp prbf_mlp;

/* Number of FP32 parameters (layer by layer: W[out][in] row-major, then b[out]). */
long long prbf_mlp_param_count(void);
int prbf_mlp_create(int device, unsigned long long seed, prbf_mlp** out);
int prbf_mlp_destroy(prbf_mlp* m);
int prbf_mlp_get_weights(prbf_mlp* m, float* w_out);
int prbf_mlp_set_weights(prbf_mlp* m, const float* w);
/* Y[n][16] = network(X[n][256]) (host arrays). */
int prbf_mlp_forward(prbf_mlp* m, int n, const float* X, float* Y);
/* Masked mean-squared error of the outputs against T with mask M (n x 16) and its gradient
 * with respect to all parameters (host arrays; grad_out has prbf_mlp_param_count entries). */
int prbf_mlp_loss_grad(prbf_mlp* m, int n, const float* X, const float* T, const float* M, float* loss,
                       float* grad_out);
/* Adam training over n patches (host arrays, copied to the device once): epochs passes of
 * shuffled mini-batches; loss_per_epoch (nullable) receives the mean training loss. */
int prbf_mlp_train(prbf_mlp* m, int n, const float* X, const float* T, const float* M, int epochs, int batch,
                   float lr, unsigned long long seed, float* loss_per_epoch);

/* Patches of n points (2D, caller order): features X[npatch][256] and per-patch output
 * scale; with g given, training targets T and masks M [npatch][16]. Call with X null to
 * get npatch only. */
int prbf_guess_patches(prbf_ctx* ctx, int n, const double* x, const double* y, const double* f, const double* g,
                       float* X, float* scale, float* T, float* M, int* npatch);
/* Installs trained weights in the context; solves with params.guess = PRBF_GUESS_LEARNED
 * then start from the network's guess. */
int prbf_guess_set_weights(prbf_ctx* ctx, const float* w);
/* The guess itself (caller order), for inspection. */
int prbf_guess_eval(prbf_ctx* ctx, int n, const double* x, const double* y, const double* f, double* g0);

#ifdef __cplusplus
}
#endif
#endif
