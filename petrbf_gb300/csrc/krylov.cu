// krylov.cu -- GMRES(m) on the device: left-preconditioned, classical Gram-Schmidt,
// Givens rotations, preconditioned-residual convergence test relative to the first
// residual. These are PETSc's KSPGMRES / KSPConvergedDefault defaults, which the
// reference selects at 2d/rbf_interpolation.cxx:210-232 with the options of
// 2d/Makefile:7 (restated from PETSc's documented algorithm; PETSc is not part of the
// reference).
//
// The Krylov state (iteration counters, Hessenberg column, rotations, residual estimate,
// stop flag) lives in device memory, so one Arnoldi iteration is a fixed sequence of
// kernels. It is captured once as the body of a CUDA-graph conditional while node whose
// condition the Givens kernel sets (continue while not stopped and k < restart).
#include <algorithm>
#include <cmath>
#include <vector>

#include "krylov.h"

namespace prbf {
namespace {

constexpr int KT = 256;

__device__ __forceinline__ double block_sum(double v, double* sh) {
  v = warp_sum(v);
  int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) sh[w] = v;
  __syncthreads();
  double s = 0;
  if (threadIdx.x == 0)
    for (int k = 0; k < (int)(blockDim.x >> 5); k++) s += sh[k];
  return s;  // valid in thread 0
}

// part[b*(m+1) + j] = sum over block b's chunk of V_j . w, j <= k
__global__ void __launch_bounds__(KT) k_multidot(const KState* __restrict__ st, const double* __restrict__ V, long long ld,
                                                 const double* __restrict__ w, int n, int chunk, double* __restrict__ part,
                                                 int mp1) {
  if (st->done) return;
  __shared__ double sh[KT / 32];
  int k = st->k;
  int lo = blockIdx.x * chunk, hi = min(n, lo + chunk);
  for (int j = 0; j <= k; j++) {
    const double* vj = V + (long long)j * ld;
    double s = 0;
    for (int i = lo + threadIdx.x; i < hi; i += KT) s = fma(vj[i], w[i], s);
    s = block_sum(s, sh);
    if (threadIdx.x == 0) part[(long long)blockIdx.x * mp1 + j] = s;
  }
}

// h[j] = sum_b part[b][j] (fixed order: deterministic)
__global__ void k_reduce_h(const KState* __restrict__ st, const double* __restrict__ part, int nb, int mp1,
                           double* __restrict__ h) {
  if (st->done) return;
  int k = st->k;
  int j = threadIdx.x;
  if (j <= k) {
    double s = 0;
    for (int b = 0; b < nb; b++) s += part[(long long)b * mp1 + j];
    h[j] = s;
  }
}

// w -= sum_{j<=k} h_j V_j ; part2[b] = sum of w^2 over the block's chunk
__global__ void __launch_bounds__(KT) k_update_norm(const KState* __restrict__ st, const double* __restrict__ V, long long ld,
                                                    const double* __restrict__ h, double* __restrict__ w, int n, int chunk,
                                                    double* __restrict__ part2) {
  if (st->done) return;
  __shared__ double sh[KT / 32];
  __shared__ double hs[64];
  int k = st->k;
  if (threadIdx.x <= k && threadIdx.x < 64) hs[threadIdx.x] = h[threadIdx.x];
  __syncthreads();
  int lo = blockIdx.x * chunk, hi = min(n, lo + chunk);
  double s2 = 0;
  for (int i = lo + threadIdx.x; i < hi; i += KT) {
    double wi = w[i];
    for (int j = 0; j <= k; j++) wi = fma(-hs[j], V[(long long)j * ld + i], wi);
    w[i] = wi;
    s2 = fma(wi, wi, s2);
  }
  s2 = block_sum(s2, sh);
  if (threadIdx.x == 0) part2[blockIdx.x] = s2;
}

__device__ int converged_default(KState* s, int n, double rnorm) {
  // KSPConvergedDefault: rnorm0 at iteration 0, ttol = max(rtol rnorm0, abstol)
  if (n == 0 && !s->fixed_ref) {
    s->rnorm0 = rnorm;
    s->ttol = fmax(s->rtol * rnorm, s->abstol);
  }
  if (!(rnorm == rnorm) || isinf(rnorm)) return -9;
  if (rnorm <= s->ttol) return rnorm < s->abstol ? 3 : 2;
  if (rnorm >= s->dtol * s->rnorm0) return -4;
  return 0;
}

// New Hessenberg column: norm, happy-breakdown test, rotations, residual estimate,
// convergence; sets the while-node condition.
__global__ void k_givens(KState* __restrict__ s, const double* __restrict__ h, const double* __restrict__ part2, int nb,
                         double* __restrict__ H, double* __restrict__ cc, double* __restrict__ ss, double* __restrict__ grs,
                         double* __restrict__ hist, int m, cudaGraphConditionalHandle cond, int use_cond) {
  if (threadIdx.x != 0) return;
  if (!s->done) {
    int k = s->k;
    double t2 = 0;
    for (int b = 0; b < nb; b++) t2 += part2[b];
    double tt = sqrt(t2);
    double col[65];
    for (int j = 0; j <= k; j++) col[j] = h[j];
    // happy breakdown bound (haptol = 1e-30)
    double hapbnd = fabs(tt / grs[k]);
    if (hapbnd > 1e-30) hapbnd = 1e-30;
    bool hapend = !(tt > hapbnd);
    s->scale = hapend ? 0.0 : 1.0 / tt;
    col[k + 1] = tt;
    for (int j = 0; j < k; j++) {
      double a = col[j], b = col[j + 1];
      col[j] = cc[j] * a + ss[j] * b;
      col[j + 1] = -ss[j] * a + cc[j] * b;
    }
    double rr = sqrt(col[k] * col[k] + col[k + 1] * col[k + 1]);
    int reason = 0;
    if (rr == 0.0) {
      reason = -5;
    } else {
      cc[k] = col[k] / rr;
      ss[k] = col[k + 1] / rr;
      grs[k + 1] = -ss[k] * grs[k];
      grs[k] = cc[k] * grs[k];
      col[k] = cc[k] * col[k] + ss[k] * col[k + 1];
      for (int j = 0; j <= k; j++) H[j * m + k] = col[j];
      double res = fabs(grs[k + 1]);
      s->res = res;
      s->k = k + 1;
      s->its += 1;
      if (hist && s->its <= s->hist_cap) hist[s->its] = res;
      reason = converged_default(s, s->its, res);
      if (hapend && !reason) reason = -5;
      if (!reason && s->its >= s->maxit) reason = -3;
    }
    if (reason) {
      s->reason = reason;
      s->done = 1;
    }
  }
  if (use_cond) cudaGraphSetConditional(cond, (!s->done && s->k < m) ? 1u : 0u);
}

// V_{k} = w * scale (k already advanced by k_givens), and the next matvec input
__global__ void k_next_vector(const KState* __restrict__ st, const double* __restrict__ w, double* __restrict__ V, long long ld,
                              double* __restrict__ vcur, int n) {
  if (st->done) return;  // the solution uses V_0 .. V_{k-1} only
  double sc = st->scale;
  int k = st->k;
  if (sc == 0.0) return;
  double* vk = V + (long long)k * ld;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    double v = w[i] * sc;
    vk[i] = v;
    vcur[i] = v;
  }
}

// ---- cycle prologue / epilogue -------------------------------------------------------
__global__ void k_residual(int n, const double* __restrict__ b, const double* __restrict__ ax, double* __restrict__ r,
                           int zero_x) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    r[i] = zero_x ? b[i] : b[i] - ax[i];
}

__global__ void __launch_bounds__(KT) k_norm2_part(const double* __restrict__ w, int n, int chunk, double* __restrict__ part) {
  __shared__ double sh[KT / 32];
  int lo = blockIdx.x * chunk, hi = min(n, lo + chunk);
  double s = 0;
  for (int i = lo + threadIdx.x; i < hi; i += KT) s = fma(w[i], w[i], s);
  s = block_sum(s, sh);
  if (threadIdx.x == 0) part[blockIdx.x] = s;
}

__global__ void k_cycle_init(KState* __restrict__ s, const double* __restrict__ part, int nb, double* __restrict__ grs,
                             int m, double* __restrict__ hist) {
  if (threadIdx.x != 0) return;
  double t2 = 0;
  for (int b = 0; b < nb; b++) t2 += part[b];
  double beta = sqrt(t2);
  for (int j = 0; j <= m; j++) grs[j] = 0.0;
  grs[0] = beta;
  s->k = 0;
  s->res = beta;
  if (s->its == 0 && hist) hist[0] = beta;
  int reason = 0;
  if (beta == 0.0)
    reason = 3;
  else
    reason = converged_default(s, s->its, beta);
  if (!reason && s->its >= s->maxit) reason = -3;
  if (reason) {
    s->reason = reason;
    s->done = 1;
  }
  s->scale = beta > 0 ? 1.0 / beta : 0.0;
  if (s->its == 0) s->beta0 = beta;
}

__global__ void k_first_vector(const KState* __restrict__ st, const double* __restrict__ w, double* __restrict__ V,
                               double* __restrict__ vcur, int n) {
  if (st->done) return;
  double sc = st->scale;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    double v = w[i] * sc;
    V[i] = v;
    vcur[i] = v;
  }
}

// y = H^-1 grs (upper triangular k x k)
__global__ void k_solve_y(const KState* __restrict__ s, const double* __restrict__ H, const double* __restrict__ grs,
                          double* __restrict__ yv, int m) {
  if (threadIdx.x != 0) return;
  int k = s->k;
  for (int r = k - 1; r >= 0; r--) {
    double t = grs[r];
    for (int j = r + 1; j < k; j++) t -= H[r * m + j] * yv[j];
    double d = H[r * m + r];
    yv[r] = d != 0.0 ? t / d : 0.0;
  }
}

__global__ void k_update_x(const KState* __restrict__ s, const double* __restrict__ V, long long ld,
                           const double* __restrict__ yv, double* __restrict__ x, int n) {
  int k = s->k;
  if (k == 0) return;
  __shared__ double ys[64];
  if (threadIdx.x < k) ys[threadIdx.x] = yv[threadIdx.x];
  __syncthreads();
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    double xi = x[i];
    for (int j = 0; j < k; j++) xi = fma(ys[j], V[(long long)j * ld + i], xi);
    x[i] = xi;
  }
}

__global__ void k_axpy(int n, double a, const double* __restrict__ xv, double* __restrict__ yv) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) yv[i] = fma(a, xv[i], yv[i]);
}

}  // namespace

void Krylov::init(int n_, int m_, cudaStream_t s) {
  if (m_ <= 0 || m_ > 60) throw Error(PRBF_ERR_ARG, "restart must be in [1, 60]");
  n = n_;
  m = m_;
  ld = ((long long)n + 4 + 31) / 32 * 32;
  V.reserve((size_t)(m + 1) * ld);
  w.reserve(ld);
  t.reserve(ld);
  vcur.reserve(ld);
  PRBF_CUDA(cudaMemsetAsync(vcur.get(), 0, sizeof(double) * ld, s));
  nblk = 2 * 152;
  chunk = (n + nblk - 1) / nblk;
  chunk = (chunk + 31) / 32 * 32;
  nblk = std::max(1, (n + chunk - 1) / chunk);
  part.reserve((size_t)nblk * (m + 1));
  part2.reserve(nblk);
  h.reserve(m + 1);
  H.reserve((size_t)(m + 1) * m);
  cc.reserve(m);
  ss.reserve(m);
  grs.reserve(m + 1);
  yv.reserve(m + 1);
  st.reserve(1);
}

Krylov::~Krylov() { reset_graph(); }

void Krylov::reset_graph() {
  if (exec) cudaGraphExecDestroy(exec);
  if (graph) cudaGraphDestroy(graph);
  exec = nullptr;
  graph = nullptr;
}

void Krylov::iteration(const Operator& op, cudaStream_t s, cudaGraphConditionalHandle cond, int use_cond) {
  KState* S = st.get();
  op.apply_A(vcur.get(), t.get(), &S->done, s);
  op.apply_B(t.get(), w.get(), &S->done, s);
  k_multidot<<<nblk, KT, 0, s>>>(S, V.get(), ld, w.get(), n, chunk, part.get(), m + 1);
  k_reduce_h<<<1, 64, 0, s>>>(S, part.get(), nblk, m + 1, h.get());
  k_update_norm<<<nblk, KT, 0, s>>>(S, V.get(), ld, h.get(), w.get(), n, chunk, part2.get());
  k_givens<<<1, 32, 0, s>>>(S, h.get(), part2.get(), nblk, H.get(), cc.get(), ss.get(), grs.get(), hist, m, cond,
                            use_cond);
  k_next_vector<<<nblk, KT, 0, s>>>(S, w.get(), V.get(), ld, vcur.get(), n);
  PRBF_CHECK_LAUNCH();
}

void Krylov::build_graph(const Operator& op, cudaStream_t s) {
  reset_graph();
  PRBF_CUDA(cudaGraphCreate(&graph, 0));
  cudaGraphConditionalHandle cond;
  PRBF_CUDA(cudaGraphConditionalHandleCreate(&cond, graph, 1, cudaGraphCondAssignDefault));
  cudaGraphNodeParams cp = {};
  cp.type = cudaGraphNodeTypeConditional;
  cp.conditional.handle = cond;
  cp.conditional.type = cudaGraphCondTypeWhile;
  cp.conditional.size = 1;
  cudaGraphNode_t node;
  PRBF_CUDA(cudaGraphAddNode(&node, graph, nullptr, nullptr, 0, &cp));
  cudaGraph_t body = cp.conditional.phGraph_out[0];
  PRBF_CUDA(cudaStreamBeginCaptureToGraph(s, body, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed));
  try {
    iteration(op, s, cond, 1);
  } catch (...) {
    cudaGraph_t dummy = nullptr;
    cudaStreamEndCapture(s, &dummy);
    cudaGetLastError();
    graph_op = nullptr;
    throw;
  }
  cudaGraph_t captured;
  PRBF_CUDA(cudaStreamEndCapture(s, &captured));
  PRBF_CUDA(cudaGraphInstantiate(&exec, graph, 0));
  graph_op = &op;
}

KResult Krylov::solve(const Operator& op, const double* b, double* x, bool zero_x, double rtol, double abstol, double dtol,
                      int maxit, bool use_graph, cudaStream_t s, double rnorm_ref, bool guard) {
  KState h0{};
  h0.rtol = rtol;
  h0.abstol = abstol;
  h0.dtol = dtol;
  h0.maxit = maxit;
  h0.hist_cap = hist_cap;
  if (rnorm_ref > 0) {
    h0.fixed_ref = 1;
    h0.rnorm0 = rnorm_ref;
    h0.ttol = std::max(rtol * rnorm_ref, abstol);
  }
  PRBF_CUDA(cudaMemcpyAsync(st.get(), &h0, sizeof(KState), cudaMemcpyHostToDevice, s));
  bool xzero = zero_x;
  KState hs{};
  KResult r;
  r.guess_used = !zero_x;
  for (int cycle = 0;; cycle++) {
    // v0 = B (b - A x); with a zero guess the product A x is skipped (as KSPInitialResidual)
    auto prologue = [&]() {
      if (!xzero) op.apply_A(x, t.get(), nullptr, s);
      k_residual<<<nblk, KT, 0, s>>>(n, b, t.get(), t.get(), xzero ? 1 : 0);
      op.apply_B(t.get(), w.get(), nullptr, s);
      k_norm2_part<<<nblk, KT, 0, s>>>(w.get(), n, chunk, part2.get());
      k_cycle_init<<<1, 32, 0, s>>>(st.get(), part2.get(), nblk, grs.get(), m, hist);
      k_first_vector<<<nblk, KT, 0, s>>>(st.get(), w.get(), V.get(), vcur.get(), n);
      PRBF_CHECK_LAUNCH();
    };
    prologue();
    if (cycle == 0 && !zero_x && (guard || rnorm_ref > 0)) {
      PRBF_CUDA(cudaMemcpyAsync(&hs, st.get(), sizeof(KState), cudaMemcpyDeviceToHost, s));
      PRBF_CUDA(cudaStreamSynchronize(s));
      r.guess_beta = hs.res;
      if (guard && rnorm_ref > 0 && !(hs.res <= rnorm_ref)) {
        // the guess is worse than starting from zero: drop it
        PRBF_CUDA(cudaMemsetAsync(x, 0, sizeof(double) * n, s));
        PRBF_CUDA(cudaMemcpyAsync(st.get(), &h0, sizeof(KState), cudaMemcpyHostToDevice, s));
        xzero = true;
        r.guess_used = false;
        prologue();
      }
    }
    // capture after the first eager prologue, so launch-configuration errors of the
    // operators surface outside the capture
    if (use_graph && graph_op != &op) build_graph(op, s);
    if (use_graph) {
      PRBF_CUDA(cudaGraphLaunch(exec, s));
    } else {
      for (int it = 0; it < m; it++) iteration(op, s, 0, 0);
    }
    k_solve_y<<<1, 32, 0, s>>>(st.get(), H.get(), grs.get(), yv.get(), m);
    k_update_x<<<nblk, KT, 0, s>>>(st.get(), V.get(), ld, yv.get(), x, n);
    PRBF_CHECK_LAUNCH();
    PRBF_CUDA(cudaMemcpyAsync(&hs, st.get(), sizeof(KState), cudaMemcpyDeviceToHost, s));
    PRBF_CUDA(cudaStreamSynchronize(s));
    xzero = false;
    if (hs.done) break;
    if (cycle > maxit + 1) break;  // cannot happen: each cycle advances its or stops
  }
  r.its = hs.its;
  r.reason = hs.reason;
  r.rnorm0 = hs.beta0;
  r.rnorm = hs.res;
  return r;
}

double norm2_host(const double* v, int n, Workspace& ws, cudaStream_t s) {
  int chunk = ((n + 303) / 304 + 31) / 32 * 32;
  int nb = std::max(1, (n + chunk - 1) / chunk);
  double* part = (double*)ws.get(50, sizeof(double) * nb);
  k_norm2_part<<<nb, KT, 0, s>>>(v, n, chunk, part);
  PRBF_CHECK_LAUNCH();
  std::vector<double> h(nb);
  PRBF_CUDA(cudaMemcpyAsync(h.data(), part, sizeof(double) * nb, cudaMemcpyDeviceToHost, s));
  PRBF_CUDA(cudaStreamSynchronize(s));
  double t = 0;
  for (double q : h) t += q;
  return std::sqrt(t);
}

void axpy_dev(int n, double a, const double* x, double* y, cudaStream_t s) {
  k_axpy<<<304, 256, 0, s>>>(n, a, x, y);
  PRBF_CHECK_LAUNCH();
}

}  // namespace prbf
