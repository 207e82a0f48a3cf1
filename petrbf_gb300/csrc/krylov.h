// krylov.h -- device GMRES (krylov.cu).
#pragma once
#include "context.h"

namespace prbf {

// Device-resident Krylov state (one per solve).
struct KState {
  int k;         // Arnoldi index inside the current cycle
  int its;       // total iterations (KSPGetIterationNumber)
  int done;      // stop flag
  int reason;    // KSPConvergedReason-style code
  int maxit;
  int hist_cap;
  double rtol, abstol, dtol;
  double rnorm0, ttol;
  double res;    // residual estimate |grs[k]|
  double scale;  // 1 / norm of the vector being normalised
  double beta0;  // first preconditioned residual norm
  int fixed_ref; // rnorm0 / ttol given by the caller (not taken from the first residual)
};

struct KResult {
  int its = 0, reason = 0;
  double rnorm0 = 0, rnorm = 0;
  bool guess_used = false;
  double guess_beta = 0;  // first preconditioned residual of the given x
};

// y = A x and z = B r on cell-sorted vectors; kernels return immediately when *skip != 0
// (skip may be null). Inputs are padded device vectors.
struct Operator {
  virtual ~Operator() = default;
  virtual void apply_A(const double* x, double* y, const int* skip, cudaStream_t s) const = 0;
  virtual void apply_B(const double* r, double* z, const int* skip, cudaStream_t s) const = 0;
};

// GMRES(m) workspace and driver. solve() runs cycles until the device state says stop;
// each cycle is a prologue (v0 = B(b - A x)), up to m Arnoldi iterations (one CUDA-graph
// conditional while node when use_graph), and the solution update x += V y.
struct Krylov {
  int n = 0, m = 0, nblk = 0, chunk = 0;
  long long ld = 0;
  DevBuf<double> V, w, t, vcur, part, part2, h, H, cc, ss, grs, yv;
  DevBuf<KState> st;
  double* hist = nullptr;  // optional device residual history (hist_cap + 1 entries)
  int hist_cap = 0;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  const Operator* graph_op = nullptr;

  ~Krylov();
  void init(int n, int m, cudaStream_t s);
  void reset_graph();
  // rnorm_ref > 0: converge relative to rnorm_ref (e.g. ||B b|| when x starts from a
  // guess) instead of the first residual; guard: if the first residual of a nonzero x is
  // above rnorm_ref, x is reset to zero (the guess is dropped). guess_used reports which.
  KResult solve(const Operator& op, const double* b, double* x, bool zero_x, double rtol, double abstol, double dtol,
                int maxit, bool use_graph, cudaStream_t s, double rnorm_ref = 0.0, bool guard = false);

 private:
  void iteration(const Operator& op, cudaStream_t s, cudaGraphConditionalHandle cond, int use_cond);
  void build_graph(const Operator& op, cudaStream_t s);
};

void axpy_dev(int n, double a, const double* x, double* y, cudaStream_t s);

}  // namespace prbf
