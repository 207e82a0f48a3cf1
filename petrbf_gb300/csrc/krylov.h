// krylov.h -- device GMRES over one or many independent systems (krylov.cu).
#pragma once
#include <vector>

#include "context.h"

namespace prbf {

// Device-resident state of one system (segment).
struct KSeg {
  int k;         // Arnoldi vectors completed in the current cycle
  int its;       // total iterations (KSPGetIterationNumber)
  int done;      // stop flag
  int reason;    // KSPConvergedReason-style code
  int maxit;
  int fixed_ref; // rnorm0 / ttol given by the caller (not taken from the first residual)
  double rtol, abstol, dtol;
  double rnorm0, ttol;
  double res;    // residual estimate |grs[k]|
  double scale;  // 1 / norm of the vector being normalised
  double beta0;  // first preconditioned residual norm
};

// Lockstep state shared by all segments.
struct KGlob {
  int k;     // Arnoldi index of the cycle (the same for every active segment)
  int done;  // every segment stopped: the skip flag of the operators
  int pad[2];
};

struct KResult {
  int its = 0, reason = 0;
  double rnorm0 = 0, rnorm = 0;
  bool guess_used = false;
  double guess_beta = 0;  // first preconditioned residual of the given x
};

// y = A x and z = B r on cell-sorted vectors (all segments at once); kernels return
// immediately when *skip != 0 (skip may be null). Inputs are padded device vectors.
// Relative tolerance of the FP32 inner GMRES of the mixed-precision refinement. The FP32
// operators agree with the FP64 ones to about 1e-4 of the residual on these systems, so
// an outer step gains about that much whatever the inner solve does past it; 1e-5 keeps
// the outer step count of a 1e-6 inner tolerance (3D vortex ring 128^3: 3 FP64 residuals
// either way) with a fifth fewer inner iterations, 1e-4 adds an outer step.
constexpr double kInnerRtol = 1e-5;

struct Operator {
  virtual ~Operator() = default;
  virtual void apply_A(const double* x, double* y, const int* skip, cudaStream_t s) const = 0;
  virtual void apply_B(const double* r, double* z, const int* skip, cudaStream_t s) const = 0;
};

// GMRES(m) for nseg independent systems whose unknowns are the segments
// [off_s, off_s + len_s) of one device vector (the operators are block diagonal over the
// segments). Each segment has its own Krylov basis (segment of the shared basis vectors),
// Hessenberg matrix, rotations and convergence test; the segments advance in lockstep and
// a segment that has stopped is skipped. solve() runs cycles until every segment has
// stopped; each cycle is a prologue (v0 = B(b - A x)), up to m Arnoldi iterations (one
// CUDA-graph conditional while node when use_graph) and the update x += V y.
struct Krylov {
  int nseg = 0, m = 0, nblk = 0, chunk = 0;
  long long total = 0, ld = 0;
  std::vector<long long> off;  // segment offsets (host)
  std::vector<int> len;        // segment lengths (host)
  DevBuf<int> bseg;            // per reduction block: segment
  DevBuf<int2> brange;         // per reduction block: [lo, hi)
  DevBuf<int> sblk;            // per segment: first block (nseg + 1)
  DevBuf<double> V, w, t, vcur, part, part2, h, H, cc, ss, grs, yv;
  DevBuf<KSeg> st;
  DevBuf<KGlob> gl;
  double* hist = nullptr;  // optional device residual history of segment 0 (hist_cap + 1)
  int hist_cap = 0;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  const Operator* graph_op = nullptr;

  ~Krylov();
  // one system of n unknowns
  void init(int n, int m, cudaStream_t s);
  // nseg systems at the given offsets (non-overlapping; total >= the end of the last)
  void init(const std::vector<long long>& off, const std::vector<int>& len, long long total, int m, cudaStream_t s);
  bool same_layout(const std::vector<long long>& o, const std::vector<int>& l, int m_) const {
    return o == off && l == len && m_ == m;
  }
  void reset_graph();
  // rnorm_ref (host, one per segment, may be null) > 0: converge relative to it (e.g.
  // ||B b|| when x starts from a guess) instead of the first residual; guard: a segment
  // whose first residual from a nonzero x is above rnorm_ref is restarted from zero (the
  // guess is dropped). guess_used reports which.
  std::vector<KResult> solve(const Operator& op, const double* b, double* x, bool zero_x, double rtol, double abstol,
                             double dtol, int maxit, bool use_graph, cudaStream_t s, const double* rnorm_ref = nullptr,
                             bool guard = false);

 private:
  void iteration(const Operator& op, cudaStream_t s, cudaGraphConditionalHandle cond, int use_cond);
  void build_graph(const Operator& op, cudaStream_t s);
};

void axpy_dev(int n, double a, const double* x, double* y, cudaStream_t s);
// Per-segment squared norms of v (host result, one per segment).
std::vector<double> seg_norm2_host(const Krylov& K, const double* v, cudaStream_t s);

}  // namespace prbf
