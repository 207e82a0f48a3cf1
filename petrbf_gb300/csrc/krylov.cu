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
// condition a one-block kernel sets (continue while some system is running and
// k < restart).
//
// Several independent systems (right-hand sides of one operator, or the problems of a
// batch) are solved together: each is a segment of the device vectors and has its own
// basis, Hessenberg matrix, rotations and stopping test, so every segment follows the
// same iterates as a solve of its own; reductions run over fixed per-segment blocks in a
// fixed order (deterministic, and for one segment the same blocks as a single solve).
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <vector>

#include "krylov.h"

namespace prbf {
namespace {

constexpr int KT = 256;
constexpr int KMAXM = 60;

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

// part[b*(m+1) + j] = sum over block b's range of V_j . w, j <= k. The basis vectors are
// taken JG at a time: one pass over the block's range reads w once and V_j0..V_j0+JG-1 into
// JG accumulators, and one block reduction serves all JG of them. Each accumulator sees its
// products in the same order as a loop over one j would, and each partial sum is the warp
// sum followed by the warps' sums in warp order, so the result does not depend on JG.
constexpr int JG = 16;

__global__ void __launch_bounds__(KT) k_multidot(const KGlob* __restrict__ G, const KSeg* __restrict__ S,
                                                 const int* __restrict__ bseg, const int2* __restrict__ brange,
                                                 const double* __restrict__ V, long long ld, const double* __restrict__ w,
                                                 double* __restrict__ part, int mp1) {
  if (G->done || S[bseg[blockIdx.x]].done) return;
  __shared__ double sh[JG][KT / 32];
  const int k = G->k;
  const int2 rg = brange[blockIdx.x];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  for (int j0 = 0; j0 <= k; j0 += JG) {
    const int nj = min(JG, k + 1 - j0);
    const double* v0 = V + (long long)j0 * ld;
    double acc[JG];
#pragma unroll
    for (int q = 0; q < JG; q++) acc[q] = 0.0;
    for (int i = rg.x + threadIdx.x; i < rg.y; i += KT) {
      const double wi = w[i];
#pragma unroll
      for (int q = 0; q < JG; q++)
        if (q < nj) acc[q] = fma(v0[(long long)q * ld + i], wi, acc[q]);
    }
#pragma unroll
    for (int q = 0; q < JG; q++) {
      const double t = warp_sum(acc[q]);
      if (lane == 0) sh[q][wid] = t;
    }
    __syncthreads();
    if (threadIdx.x < nj) {
      double t = 0;
      for (int u = 0; u < KT / 32; u++) t += sh[threadIdx.x][u];
      part[(long long)blockIdx.x * mp1 + j0 + threadIdx.x] = t;
    }
    __syncthreads();
  }
}

// h[s][j] = sum over segment s's blocks of part[b][j] (fixed order): one block per segment
__global__ void k_reduce_h(const KGlob* __restrict__ G, const KSeg* __restrict__ S, const int* __restrict__ sblk,
                           const double* __restrict__ part, int mp1, double* __restrict__ h) {
  const int sg = blockIdx.x;
  if (G->done || S[sg].done) return;
  int k = G->k;
  int j = threadIdx.x;
  if (j <= k) {
    double s = 0;
    for (int b = sblk[sg]; b < sblk[sg + 1]; b++) s += part[(long long)b * mp1 + j];
    h[(long long)sg * mp1 + j] = s;
  }
}

// w -= sum_{j<=k} h_j V_j ; part2[b] = sum of w^2 over the block's range
__global__ void __launch_bounds__(KT) k_update_norm(const KGlob* __restrict__ G, const KSeg* __restrict__ S,
                                                    const int* __restrict__ bseg, const int2* __restrict__ brange,
                                                    const double* __restrict__ V, long long ld,
                                                    const double* __restrict__ h, int mp1, double* __restrict__ w,
                                                    double* __restrict__ part2) {
  const int sg = bseg[blockIdx.x];
  if (G->done || S[sg].done) return;
  __shared__ double sh[KT / 32];
  __shared__ double hs[64];
  int k = G->k;
  if (threadIdx.x <= k && threadIdx.x < 64) hs[threadIdx.x] = h[(long long)sg * mp1 + threadIdx.x];
  __syncthreads();
  const int2 rg = brange[blockIdx.x];
  double s2 = 0;
  for (int i = rg.x + threadIdx.x; i < rg.y; i += KT) {
    double wi = w[i];
    // JG loads issued together, the fmas in j order
    for (int j0 = 0; j0 <= k; j0 += JG) {
      const int nj = min(JG, k + 1 - j0);
      const double* v0 = V + (long long)j0 * ld + i;
      double vq[JG];
#pragma unroll
      for (int q = 0; q < JG; q++) vq[q] = q < nj ? v0[(long long)q * ld] : 0.0;
#pragma unroll
      for (int q = 0; q < JG; q++)
        if (q < nj) wi = fma(-hs[j0 + q], vq[q], wi);
    }
    w[i] = wi;
    s2 = fma(wi, wi, s2);
  }
  s2 = block_sum(s2, sh);
  if (threadIdx.x == 0) part2[blockIdx.x] = s2;
}

__device__ int converged_default(KSeg* s, int n, double rnorm) {
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

// New Hessenberg column of each running segment (one thread each): norm, happy-breakdown
// test, rotations, residual estimate, convergence.
__global__ void k_givens(const KGlob* __restrict__ G, KSeg* __restrict__ S, int nseg, const int* __restrict__ sblk,
                         const double* __restrict__ h, const double* __restrict__ part2, double* __restrict__ H,
                         double* __restrict__ cc, double* __restrict__ ss, double* __restrict__ grs,
                         double* __restrict__ hist, int hist_cap, int m) {
  const int sg = blockIdx.x * blockDim.x + threadIdx.x;
  if (sg >= nseg || G->done) return;
  KSeg* s = S + sg;
  if (s->done) return;
  const int mp1 = m + 1;
  const double* hh = h + (long long)sg * mp1;
  double* Hs = H + (long long)sg * mp1 * m;
  double* c = cc + (long long)sg * m;
  double* sn = ss + (long long)sg * m;
  double* g = grs + (long long)sg * mp1;
  int k = s->k;
  double t2 = 0;
  for (int b = sblk[sg]; b < sblk[sg + 1]; b++) t2 += part2[b];
  double tt = sqrt(t2);
  double col[KMAXM + 1];
  for (int j = 0; j <= k; j++) col[j] = hh[j];
  // happy breakdown bound (haptol = 1e-30)
  double hapbnd = fabs(tt / g[k]);
  if (hapbnd > 1e-30) hapbnd = 1e-30;
  bool hapend = !(tt > hapbnd);
  s->scale = hapend ? 0.0 : 1.0 / tt;
  col[k + 1] = tt;
  for (int j = 0; j < k; j++) {
    double a = col[j], b = col[j + 1];
    col[j] = c[j] * a + sn[j] * b;
    col[j + 1] = -sn[j] * a + c[j] * b;
  }
  double rr = sqrt(col[k] * col[k] + col[k + 1] * col[k + 1]);
  int reason = 0;
  if (rr == 0.0) {
    reason = -5;
  } else {
    c[k] = col[k] / rr;
    sn[k] = col[k + 1] / rr;
    g[k + 1] = -sn[k] * g[k];
    g[k] = c[k] * g[k];
    col[k] = c[k] * col[k] + sn[k] * col[k + 1];
    for (int j = 0; j <= k; j++) Hs[j * m + k] = col[j];
    double res = fabs(g[k + 1]);
    s->res = res;
    s->k = k + 1;
    s->its += 1;
    if (sg == 0 && hist && s->its <= hist_cap) hist[s->its] = res;
    reason = converged_default(s, s->its, res);
    if (hapend && !reason) reason = -5;
    if (!reason && s->its >= s->maxit) reason = -3;
  }
  if (reason) {
    s->reason = reason;
    s->done = 1;
  }
}

// Lockstep bookkeeping (one block): advance k (after an iteration) or reset it (after a
// prologue), set done when every segment has stopped, and the while-node condition.
__global__ void k_sync(KGlob* __restrict__ G, const KSeg* __restrict__ S, int nseg, int reset, int m,
                       cudaGraphConditionalHandle cond, int use_cond) {
  __shared__ int running;
  if (threadIdx.x == 0) running = 0;
  __syncthreads();
  int any = 0;
  for (int i = threadIdx.x; i < nseg; i += blockDim.x) any |= S[i].done ? 0 : 1;
  if (any) atomicOr(&running, 1);
  __syncthreads();
  if (threadIdx.x != 0) return;
  if (reset)
    G->k = 0;
  else if (!G->done)
    G->k += 1;
  G->done = running ? 0 : 1;
  if (use_cond) cudaGraphSetConditional(cond, (!G->done && G->k < m) ? 1u : 0u);
}

// V_k = w * scale (k already advanced), and the next matvec input
__global__ void k_next_vector(const KGlob* __restrict__ G, const KSeg* __restrict__ S, const int* __restrict__ bseg,
                              const int2* __restrict__ brange, const double* __restrict__ w, double* __restrict__ V,
                              long long ld, double* __restrict__ vcur) {
  const KSeg& s = S[bseg[blockIdx.x]];
  if (G->done || s.done) return;  // the solution uses V_0 .. V_{k-1} only
  double sc = s.scale;
  int k = G->k;
  if (sc == 0.0) return;
  double* vk = V + (long long)k * ld;
  const int2 rg = brange[blockIdx.x];
  for (int i = rg.x + threadIdx.x; i < rg.y; i += blockDim.x) {
    double v = w[i] * sc;
    vk[i] = v;
    vcur[i] = v;
  }
}

// ---- cycle prologue / epilogue -------------------------------------------------------
__global__ void k_residual(const int2* __restrict__ brange, const double* __restrict__ b, const double* __restrict__ ax,
                           double* __restrict__ r, int zero_x) {
  const int2 rg = brange[blockIdx.x];
  for (int i = rg.x + threadIdx.x; i < rg.y; i += blockDim.x) r[i] = zero_x ? b[i] : b[i] - ax[i];
}

__global__ void __launch_bounds__(KT) k_norm2_part(const int2* __restrict__ brange, const double* __restrict__ w,
                                                   double* __restrict__ part) {
  __shared__ double sh[KT / 32];
  const int2 rg = brange[blockIdx.x];
  double s = 0;
  for (int i = rg.x + threadIdx.x; i < rg.y; i += KT) s = fma(w[i], w[i], s);
  s = block_sum(s, sh);
  if (threadIdx.x == 0) part[blockIdx.x] = s;
}

__global__ void k_cycle_init(KSeg* __restrict__ S, int nseg, const int* __restrict__ sblk,
                             const double* __restrict__ part, double* __restrict__ grs, int m,
                             double* __restrict__ hist) {
  const int sg = blockIdx.x * blockDim.x + threadIdx.x;
  if (sg >= nseg) return;
  KSeg* s = S + sg;
  s->k = 0;
  if (s->done) return;
  double t2 = 0;
  for (int b = sblk[sg]; b < sblk[sg + 1]; b++) t2 += part[b];
  double beta = sqrt(t2);
  double* g = grs + (long long)sg * (m + 1);
  for (int j = 0; j <= m; j++) g[j] = 0.0;
  g[0] = beta;
  s->res = beta;
  if (sg == 0 && s->its == 0 && hist) hist[0] = beta;
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

__global__ void k_first_vector(const KGlob* __restrict__ G, const KSeg* __restrict__ S, const int* __restrict__ bseg,
                               const int2* __restrict__ brange, const double* __restrict__ w, double* __restrict__ V,
                               double* __restrict__ vcur) {
  const KSeg& s = S[bseg[blockIdx.x]];
  if (G->done || s.done) return;
  double sc = s.scale;
  const int2 rg = brange[blockIdx.x];
  for (int i = rg.x + threadIdx.x; i < rg.y; i += blockDim.x) {
    double v = w[i] * sc;
    V[i] = v;
    vcur[i] = v;
  }
}

// y = H^-1 grs (upper triangular k x k), one thread per segment
__global__ void k_solve_y(const KSeg* __restrict__ S, int nseg, const double* __restrict__ H,
                          const double* __restrict__ grs, double* __restrict__ yv, int m) {
  const int sg = blockIdx.x * blockDim.x + threadIdx.x;
  if (sg >= nseg) return;
  const int k = S[sg].k, mp1 = m + 1;
  const double* Hs = H + (long long)sg * mp1 * m;
  const double* g = grs + (long long)sg * mp1;
  double* y = yv + (long long)sg * mp1;
  for (int r = k - 1; r >= 0; r--) {
    double t = g[r];
    for (int j = r + 1; j < k; j++) t -= Hs[r * m + j] * y[j];
    double d = Hs[r * m + r];
    y[r] = d != 0.0 ? t / d : 0.0;
  }
}

__global__ void k_update_x(const KSeg* __restrict__ S, const int* __restrict__ bseg, const int2* __restrict__ brange,
                           const double* __restrict__ V, long long ld, const double* __restrict__ yv, int mp1,
                           double* __restrict__ x) {
  const int sg = bseg[blockIdx.x];
  const int k = S[sg].k;
  if (k == 0) return;
  __shared__ double ys[64];
  if (threadIdx.x < k) ys[threadIdx.x] = yv[(long long)sg * mp1 + threadIdx.x];
  __syncthreads();
  const int2 rg = brange[blockIdx.x];
  for (int i = rg.x + threadIdx.x; i < rg.y; i += blockDim.x) {
    double xi = x[i];
    for (int j = 0; j < k; j++) xi = fma(ys[j], V[(long long)j * ld + i], xi);
    x[i] = xi;
  }
}

__global__ void k_axpy(int n, double a, const double* __restrict__ xv, double* __restrict__ yv) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) yv[i] = fma(a, xv[i], yv[i]);
}

}  // namespace

void Krylov::init(int n_, int m_, cudaStream_t s) { init({0}, {n_}, (long long)n_, m_, s); }

void Krylov::init(const std::vector<long long>& off_, const std::vector<int>& len_, long long total_, int m_,
                  cudaStream_t s) {
  if (m_ <= 0 || m_ > KMAXM) throw Error(PRBF_ERR_ARG, "restart must be in [1, 60]");
  if (off_.empty() || off_.size() != len_.size()) throw Error(PRBF_ERR_ARG, "bad segment layout");
  reset_graph();
  off = off_;
  len = len_;
  nseg = (int)off.size();
  m = m_;
  total = total_;
  long long sum = 0;
  for (int i = 0; i < nseg; i++) {
    if (off[i] < 0 || len[i] < 0 || off[i] + len[i] > total) throw Error(PRBF_ERR_ARG, "bad segment");
    sum += len[i];
  }
  ld = (total + 4 + 31) / 32 * 32;
  // reduction blocks: the same chunk for every segment (about two blocks per SM overall)
  chunk = (int)((sum + 303) / 304);
  chunk = std::max(32, (chunk + 31) / 32 * 32);
  std::vector<int> hb, hs(nseg + 1);
  std::vector<int2> hr;
  for (int i = 0; i < nseg; i++) {
    hs[i] = (int)hb.size();
    int nb = std::max(1, (len[i] + chunk - 1) / chunk);
    for (int b = 0; b < nb; b++) {
      long long lo = off[i] + (long long)b * chunk, hi = std::min(off[i] + len[i], lo + chunk);
      hb.push_back(i);
      hr.push_back(make_int2((int)lo, (int)std::max(lo, hi)));
    }
  }
  hs[nseg] = (int)hb.size();
  nblk = (int)hb.size();
  if (total > 0x7fffffffLL) throw Error(PRBF_ERR_CAPACITY, "vector longer than 2^31");
  bseg.reserve(nblk);
  brange.reserve(nblk);
  sblk.reserve(nseg + 1);
  PRBF_CUDA(cudaMemcpyAsync(bseg.get(), hb.data(), sizeof(int) * nblk, cudaMemcpyHostToDevice, s));
  PRBF_CUDA(cudaMemcpyAsync(brange.get(), hr.data(), sizeof(int2) * nblk, cudaMemcpyHostToDevice, s));
  PRBF_CUDA(cudaMemcpyAsync(sblk.get(), hs.data(), sizeof(int) * (nseg + 1), cudaMemcpyHostToDevice, s));
  V.reserve((size_t)(m + 1) * ld);
  w.reserve(ld);
  t.reserve(ld);
  vcur.reserve(ld);
  for (auto* v : {&w, &t, &vcur}) PRBF_CUDA(cudaMemsetAsync(v->get(), 0, sizeof(double) * ld, s));
  PRBF_CUDA(cudaMemsetAsync(V.get(), 0, sizeof(double) * (m + 1) * ld, s));
  part.reserve((size_t)nblk * (m + 1));
  part2.reserve(nblk);
  h.reserve((size_t)nseg * (m + 1));
  H.reserve((size_t)nseg * (m + 1) * m);
  cc.reserve((size_t)nseg * m);
  ss.reserve((size_t)nseg * m);
  grs.reserve((size_t)nseg * (m + 1));
  yv.reserve((size_t)nseg * (m + 1));
  st.reserve(nseg);
  gl.reserve(1);
  PRBF_CUDA(cudaStreamSynchronize(s));
}

Krylov::~Krylov() { reset_graph(); }

void Krylov::reset_graph() {
  if (exec) cudaGraphExecDestroy(exec);
  if (graph) cudaGraphDestroy(graph);
  exec = nullptr;
  graph = nullptr;
  graph_op = nullptr;
}

void Krylov::iteration(const Operator& op, cudaStream_t s, cudaGraphConditionalHandle cond, int use_cond) {
  KSeg* S = st.get();
  KGlob* G = gl.get();
  const int sg_blocks = (nseg + 63) / 64;
  op.apply_A(vcur.get(), t.get(), &G->done, s);
  op.apply_B(t.get(), w.get(), &G->done, s);
  k_multidot<<<nblk, KT, 0, s>>>(G, S, bseg.get(), brange.get(), V.get(), ld, w.get(), part.get(), m + 1);
  k_reduce_h<<<nseg, 64, 0, s>>>(G, S, sblk.get(), part.get(), m + 1, h.get());
  k_update_norm<<<nblk, KT, 0, s>>>(G, S, bseg.get(), brange.get(), V.get(), ld, h.get(), m + 1, w.get(), part2.get());
  k_givens<<<sg_blocks, 64, 0, s>>>(G, S, nseg, sblk.get(), h.get(), part2.get(), H.get(), cc.get(), ss.get(), grs.get(),
                                    hist, hist_cap, m);
  k_sync<<<1, 256, 0, s>>>(G, S, nseg, 0, m, cond, use_cond);
  k_next_vector<<<nblk, KT, 0, s>>>(G, S, bseg.get(), brange.get(), w.get(), V.get(), ld, vcur.get());
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

// PRBF_KRYLOV_EAGER=1 launches the iterations one kernel at a time instead of through the
// graph's while node (same kernels, same results): profilers list the kernels of a
// conditional graph body poorly, so a launch list of a solve is taken this way.
static bool krylov_eager() {
  static const bool e = [] {
    const char* v = std::getenv("PRBF_KRYLOV_EAGER");
    return v && v[0] == '1';
  }();
  return e;
}

std::vector<KResult> Krylov::solve(const Operator& op, const double* b, double* x, bool zero_x, double rtol,
                                   double abstol, double dtol, int maxit, bool use_graph, cudaStream_t s,
                                   const double* rnorm_ref, bool guard) {
  if (krylov_eager()) use_graph = false;
  std::vector<KSeg> h0(nseg);
  for (int i = 0; i < nseg; i++) {
    KSeg& q = h0[i];
    q = KSeg{};
    q.rtol = rtol;
    q.abstol = abstol;
    q.dtol = dtol;
    q.maxit = maxit;
    if (rnorm_ref && rnorm_ref[i] > 0) {
      q.fixed_ref = 1;
      q.rnorm0 = rnorm_ref[i];
      q.ttol = std::max(rtol * rnorm_ref[i], abstol);
    }
  }
  PRBF_CUDA(cudaMemcpyAsync(st.get(), h0.data(), sizeof(KSeg) * nseg, cudaMemcpyHostToDevice, s));
  PRBF_CUDA(cudaMemsetAsync(gl.get(), 0, sizeof(KGlob), s));
  bool xzero = zero_x;
  std::vector<KSeg> hs(nseg);
  KGlob hg{};
  std::vector<KResult> r(nseg);
  for (auto& q : r) q.guess_used = !zero_x;
  const int sg_blocks = (nseg + 63) / 64;
  for (int cycle = 0;; cycle++) {
    // v0 = B (b - A x); with a zero guess the product A x is skipped (as KSPInitialResidual)
    auto prologue = [&]() {
      if (!xzero) op.apply_A(x, t.get(), nullptr, s);
      k_residual<<<nblk, KT, 0, s>>>(brange.get(), b, t.get(), t.get(), xzero ? 1 : 0);
      op.apply_B(t.get(), w.get(), nullptr, s);
      k_norm2_part<<<nblk, KT, 0, s>>>(brange.get(), w.get(), part2.get());
      k_cycle_init<<<sg_blocks, 64, 0, s>>>(st.get(), nseg, sblk.get(), part2.get(), grs.get(), m, hist);
      k_sync<<<1, 256, 0, s>>>(gl.get(), st.get(), nseg, 1, m, 0, 0);
      k_first_vector<<<nblk, KT, 0, s>>>(gl.get(), st.get(), bseg.get(), brange.get(), w.get(), V.get(), vcur.get());
      PRBF_CHECK_LAUNCH();
    };
    prologue();
    if (cycle == 0 && !zero_x && (guard || rnorm_ref)) {
      PRBF_CUDA(cudaMemcpyAsync(hs.data(), st.get(), sizeof(KSeg) * nseg, cudaMemcpyDeviceToHost, s));
      PRBF_CUDA(cudaStreamSynchronize(s));
      bool redo = false;
      for (int i = 0; i < nseg; i++) {
        r[i].guess_beta = hs[i].res;
        if (guard && rnorm_ref && rnorm_ref[i] > 0 && !(hs[i].res <= rnorm_ref[i])) {
          // the guess is worse than starting from zero: drop it for this system
          PRBF_CUDA(cudaMemsetAsync(x + off[i], 0, sizeof(double) * len[i], s));
          r[i].guess_used = false;
          redo = true;
        }
      }
      if (redo) {
        PRBF_CUDA(cudaMemcpyAsync(st.get(), h0.data(), sizeof(KSeg) * nseg, cudaMemcpyHostToDevice, s));
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
    k_solve_y<<<sg_blocks, 64, 0, s>>>(st.get(), nseg, H.get(), grs.get(), yv.get(), m);
    k_update_x<<<nblk, KT, 0, s>>>(st.get(), bseg.get(), brange.get(), V.get(), ld, yv.get(), m + 1, x);
    PRBF_CHECK_LAUNCH();
    PRBF_CUDA(cudaMemcpyAsync(&hg, gl.get(), sizeof(KGlob), cudaMemcpyDeviceToHost, s));
    PRBF_CUDA(cudaStreamSynchronize(s));
    xzero = false;
    if (hg.done) break;
    if (cycle > maxit + 1) break;  // cannot happen: each cycle advances its or stops
  }
  PRBF_CUDA(cudaMemcpyAsync(hs.data(), st.get(), sizeof(KSeg) * nseg, cudaMemcpyDeviceToHost, s));
  PRBF_CUDA(cudaStreamSynchronize(s));
  for (int i = 0; i < nseg; i++) {
    r[i].its = hs[i].its;
    r[i].reason = hs[i].reason;
    r[i].rnorm0 = hs[i].beta0;
    r[i].rnorm = hs[i].res;
  }
  return r;
}

std::vector<double> seg_norm2_host(const Krylov& K, const double* v, cudaStream_t s) {
  k_norm2_part<<<K.nblk, KT, 0, s>>>(K.brange.get(), v, K.part2.get());
  PRBF_CHECK_LAUNCH();
  std::vector<double> hp(K.nblk), out(K.nseg, 0.0);
  std::vector<int> hb(K.nblk);
  PRBF_CUDA(cudaMemcpyAsync(hp.data(), K.part2.get(), sizeof(double) * K.nblk, cudaMemcpyDeviceToHost, s));
  PRBF_CUDA(cudaMemcpyAsync(hb.data(), K.bseg.get(), sizeof(int) * K.nblk, cudaMemcpyDeviceToHost, s));
  PRBF_CUDA(cudaStreamSynchronize(s));
  for (int b = 0; b < K.nblk; b++) out[hb[b]] += hp[b];
  return out;
}

void axpy_dev(int n, double a, const double* x, double* y, cudaStream_t s) {
  k_axpy<<<304, 256, 0, s>>>(n, a, x, y);
  PRBF_CHECK_LAUNCH();
}

}  // namespace prbf
