// solve.cu -- rbf_interpolation on the GPU (2d/rbf_interpolation.cxx:25-310,
// 3d/rbf_interpolation.cxx:26-334) and the RBFInterpolation library entry
// (3d/wrapper.cxx:20-105).
//
// Plain form (PRBF_PREC_FP64): cell sort, FP64 RASM set-up, GMRES(restart) from a zero
// guess with the RASM preconditioner on the left, stopping on the preconditioned residual
// relative to the first one (PETSc's defaults for the reference's options).
// Mixed form (PRBF_PREC_MIXED): FP64 iterative refinement, x += d with A d = r solved
// approximately by GMRES whose matvec and RASM blocks are FP32; FP64 is kept for the outer
// residual matvec, the Arnoldi vectors and Hessenberg least squares, and the update. It
// stops on the true residual ||f - A g||_2 <= rtol ||f||_2. Refinement contracts the
// residual by about cond(A) u_fp32 per step, so a system too ill-conditioned for FP32
// (tightly clustered points) stalls: a step that does not halve the FP64 residual, or a
// non-finite one, hands the call to the plain form (FP64 blocks, FP64 GMRES from zero).
#include <algorithm>
#include <chrono>
#include <climits>
#include <cmath>
#include <cstring>
#include <vector>

#include "krylov.h"
#include "mlp.h"
#include "rasm.h"
#include "trace.h"

namespace prbf {

namespace {

// A and B over nv right-hand sides stored at stride vstride
struct GaussRasmOp : Operator {
  const GaussPlan* plan = nullptr;
  PointsView v{};
  const RasmPlan* rasm = nullptr;
  bool fp32 = false;
  unsigned* err = nullptr;
  int nv = 1;
  long long vstride = 0;
  void apply_A(const double* x, double* y, const int* skip, cudaStream_t s) const override {
    gauss_sum_dev(*plan, v, v, x, y, fp32, err, s, skip, nv, vstride);
  }
  void apply_B(const double* r, double* z, const int* skip, cudaStream_t s) const override {
    rasm_apply(*rasm, v.cell_start, r, z, s, skip, nv, vstride);
  }
};

double now_ms() {
  using namespace std::chrono;
  return duration<double, std::milli>(steady_clock::now().time_since_epoch()).count();
}

}  // namespace


struct SolveState {
  PointSet pts;
  GaussPlan plan;
  RasmPlan rasm;
  Krylov kry;
  DevBuf<double> b, x, r, d, tmp;
  GaussRasmOp op64, op32;
  RasmPlan pc;  // preconditioner of the matvec seam (prbf_pc_setup)
  bool pc_ready = false;
};

Ctx::~Ctx() {
  delete solve;
  solve = nullptr;
  delete guess;
  guess = nullptr;
  batch_state_free(batch);
  batch = nullptr;
  ctx_stream_release(*this);
}

// Solve for every right-hand side; f and g_out are host arrays (nrhs x n, caller order).
static void interpolate(Ctx& c, int n, const double* x, const double* y, const double* z, const double* f, int nrhs,
                        double* g_out, prbf_stats* stats) {
  const double t_begin = now_ms();
  const prbf_params& p = c.p;
  const int dim = p.dim;
  if (!c.solve) c.solve = new SolveState();
  SolveState& S = *c.solve;
  // ---- cell list -----------------------------------------------------------------------
  {
    TraceRange tr("InitCluster");
    DevBuf<double> ux, uy, uz;
    c.upload(ux, x, n);
    c.upload(uy, y, n);
    if (dim == 3) c.upload(uz, z, n);
    double bb[6];
    bbox_host(c, n, ux.get(), uy.get(), dim == 3 ? uz.get() : nullptr, bb);
    Grid g = make_grid(dim, bb, p.sigma, p.nsigma_box, p.sigma_buffer, p.sigma_trunc);
    build_points(c, S.pts, g, n, ux.get(), uy.get(), dim == 3 ? uz.get() : nullptr);
    PRBF_CUDA(cudaStreamSynchronize(c.stream));
  }
  const double t_sorted = now_ms();
  // ---- operator and RASM set-up ----------------------------------------------------------
  TraceRange tr_mat("InitMat");
  S.plan.g = S.pts.g;
  S.plan.sym_nv = std::min(4, nrhs);  // right-hand sides summed together by the symmetric form
  gauss_plan_dev(S.plan, S.pts.view(), S.pts.view(), c.err.get(), c.ws, c.stream);
  const bool mixed = p.precision == PRBF_PREC_MIXED;
  size_t free_b = 0, total_b = 0;
  PRBF_CUDA(cudaMemGetInfo(&free_b, &total_b));
  double budget = std::min(16.0e9, 0.25 * (double)free_b);
  // FP32 blocks: S_c (one GEMV per apply) in 2D; in 3D the blocks are too ill-conditioned
  // for an explicit FP32 inverse, so the FP32 factor is kept and applied by substitution
  S.rasm.max_nv = std::min(4, nrhs);
  S.rasm.lu_fallback = p.block_fallback == PRBF_FALLBACK_LU;
  rasm_build(S.rasm, S.pts, mixed, c.ws, c.err.get(), c.stream, budget, mixed && dim == 3,
             p.pc_type == PRBF_PC_ASM);
  rasm_set_apply_smem(S.rasm);
  c.check_device_error("RASM set-up");
  const double t_setup = now_ms();
  tr_mat.end();

  // right-hand sides: segments of one vector at a 32-aligned stride, solved in lockstep
  // (the matvec computes each pair's exponential once for all of them)
  const int nv = nrhs;
  const long long ldn = ((long long)n + 4 + 31) / 32 * 32;
  const long long len_all = ldn * nv + 32;
  if (ldn * nv > (long long)INT_MAX)
    throw Error(PRBF_ERR_CAPACITY, "points x right-hand sides must stay below 2^31 (solve in several calls)");
  S.op64.plan = S.op32.plan = &S.plan;
  S.op64.v = S.op32.v = S.pts.view();
  S.op64.rasm = S.op32.rasm = &S.rasm;
  S.op64.err = S.op32.err = c.err.get();
  S.op64.fp32 = false;
  S.op32.fp32 = true;
  S.op64.nv = S.op32.nv = nv;
  S.op64.vstride = S.op32.vstride = ldn;
  S.b.reserve(len_all);
  S.x.reserve(len_all);
  S.r.reserve(len_all);
  S.d.reserve(len_all);
  S.tmp.reserve(len_all);
  for (auto* v : {&S.b, &S.x, &S.r, &S.d, &S.tmp})
    PRBF_CUDA(cudaMemsetAsync(v->get(), 0, sizeof(double) * len_all, c.stream));
  std::vector<long long> offs(nv);
  std::vector<int> lens(nv, n);
  for (int v = 0; v < nv; v++) offs[v] = v * ldn;
  if (!S.kry.same_layout(offs, lens, p.restart)) S.kry.init(offs, lens, len_all, p.restart, c.stream);
  S.kry.graph_op = nullptr;  // operators are rebuilt per call

  const bool use_guess = p.guess == PRBF_GUESS_LEARNED;
  if (use_guess && (dim != 2 || !c.guess || !c.guess->ready))
    throw Error(PRBF_ERR_STATE, "learned guess requested without installed weights (2D only)");
  prbf_stats st{};
  st.ncell = S.pts.g.ncell;
  st.max_block = S.rasm.max_nb;
  st.nblocks_fallback = S.rasm.nfallback;
  st.pairs_per_matvec = S.plan.pairs;
  for (int v = 0; v < nv; v++) {
    PRBF_CUDA(cudaMemcpyAsync(S.tmp.get(), f + (size_t)v * n, sizeof(double) * n, cudaMemcpyHostToDevice, c.stream));
    gather_dev(n, S.pts.perm.get(), S.tmp.get(), S.b.get() + v * ldn, c.stream);
  }
  PRBF_CUDA(cudaMemsetAsync(S.tmp.get(), 0, sizeof(double) * len_all, c.stream));
  PRBF_CUDA(cudaStreamSynchronize(c.stream));
  const double ts0 = now_ms();
  TraceRange tr_solve("KSPSolve");
  if (use_guess) {
    // x0 from the network, in the solver's cell order (its inputs are the sorted points)
    for (int v = 0; v < nv; v++)
      guess_compute(c, *c.guess, n, S.pts.x.get(), S.pts.y.get(), S.b.get() + v * ldn, S.x.get() + v * ldn);
    PRBF_CUDA(cudaStreamSynchronize(c.stream));
    st.t_guess_ms = now_ms() - ts0;
  }
  std::vector<int> reason(nv, 0), its(nv, 0), outer(nv, 0);
  std::vector<double> rnorm0(nv, 0.0), rnorm(nv, 0.0);
  // mixed form: when the refinement stops on its own FP64 residual test, rnorm holds the
  // true residual of the final weights and the reported one needs no extra matvec
  std::vector<double> true_rel(nv, 0.0);
  bool resid_current = false;
  // the plain form: GMRES on A x = b with the FP64 operators (from the guess in x, or zero)
  auto plain_solve = [&](bool from_guess) {
    std::vector<double> ref(nv, 0.0);
    if (from_guess) {
      // converge relative to the zero-guess residual ||B b||, whatever the guess
      S.op64.apply_B(S.b.get(), S.tmp.get(), nullptr, c.stream);
      std::vector<double> q = seg_norm2_host(S.kry, S.tmp.get(), c.stream);
      for (int v = 0; v < nv; v++) ref[v] = std::sqrt(q[v]);
    }
    std::vector<KResult> kr = S.kry.solve(S.op64, S.b.get(), S.x.get(), !from_guess, p.rtol, p.abstol, p.dtol,
                                          p.max_it, true, c.stream, from_guess ? ref.data() : nullptr, from_guess);
    int used = 0;
    double gres = 0;
    for (int v = 0; v < nv; v++) {
      its[v] += kr[v].its;
      reason[v] = kr[v].reason;
      rnorm0[v] = kr[v].rnorm0;
      rnorm[v] = kr[v].rnorm;
      used += kr[v].guess_used ? 1 : 0;
      gres = std::max(gres, ref[v] > 0 ? kr[v].guess_beta / ref[v] : 1.0);
    }
    if (from_guess) {
      st.guess_used = used == nv ? 1 : 0;
      st.guess_rel_resid = gres;
    }
  };
  if (!mixed) {
    plain_solve(use_guess);
  } else {
    std::vector<double> bnorm = seg_norm2_host(S.kry, S.b.get(), c.stream);
    for (auto& q : bnorm) q = std::sqrt(q);
    bool xzero = !use_guess;
    int inner_max = 0;
    const int nall = (int)(ldn * nv);
    std::vector<double> prev(nv, 0.0);
    bool stalled = false;
    for (int it = 0; it < 50 && !stalled; it++) {
      // r = b - A x in FP64 (all right-hand sides)
      if (xzero) {
        PRBF_CUDA(cudaMemcpyAsync(S.r.get(), S.b.get(), sizeof(double) * nall, cudaMemcpyDeviceToDevice, c.stream));
      } else {
        S.op64.apply_A(S.x.get(), S.tmp.get(), nullptr, c.stream);
        PRBF_CUDA(cudaMemcpyAsync(S.r.get(), S.b.get(), sizeof(double) * nall, cudaMemcpyDeviceToDevice, c.stream));
        axpy_dev(nall, -1.0, S.tmp.get(), S.r.get(), c.stream);
      }
      std::vector<double> rn = seg_norm2_host(S.kry, S.r.get(), c.stream);
      for (auto& q : rn) q = std::sqrt(q);
      if (it == 0 && use_guess) {
        int used = 0;
        double gres = 0;
        for (int v = 0; v < nv; v++) {
          gres = std::max(gres, bnorm[v] > 0 ? rn[v] / bnorm[v] : 1.0);
          if (rn[v] <= bnorm[v]) {
            used++;
            continue;
          }
          // worse than zero: drop the guess of this right-hand side
          PRBF_CUDA(cudaMemsetAsync(S.x.get() + v * ldn, 0, sizeof(double) * n, c.stream));
          PRBF_CUDA(cudaMemcpyAsync(S.r.get() + v * ldn, S.b.get() + v * ldn, sizeof(double) * n,
                                    cudaMemcpyDeviceToDevice, c.stream));
          rn[v] = bnorm[v];
        }
        st.guess_used = used == nv ? 1 : 0;
        st.guess_rel_resid = gres;
      }
      bool all = true;
      for (int v = 0; v < nv; v++) {
        if (it == 0) rnorm0[v] = rn[v];
        if (reason[v]) {
          // stopped earlier: keep it out of the inner solve (zero residual stops at once)
          PRBF_CUDA(cudaMemsetAsync(S.r.get() + v * ldn, 0, sizeof(double) * n, c.stream));
          continue;
        }
        rnorm[v] = rn[v];
        if (!(rn[v] == rn[v]) || std::isinf(rn[v])) {
          stalled = true;
        } else if (rn[v] <= p.rtol * bnorm[v] || rn[v] <= p.abstol) {
          reason[v] = rn[v] <= p.abstol ? 3 : 2;
        } else if (it > 0 && !(rn[v] <= 0.5 * prev[v])) {
          stalled = true;
        } else if (inner_max >= p.max_it) {
          reason[v] = -3;
        } else {
          outer[v]++;
          prev[v] = rn[v];
          all = false;
          continue;
        }
        if (stalled) break;
        PRBF_CUDA(cudaMemsetAsync(S.r.get() + v * ldn, 0, sizeof(double) * n, c.stream));
      }
      if (stalled) break;
      if (all) {
        resid_current = true;
        for (int v = 0; v < nv; v++) true_rel[v] = bnorm[v] > 0 ? rnorm[v] / bnorm[v] : rnorm[v];
        break;
      }
      PRBF_CUDA(cudaMemsetAsync(S.d.get(), 0, sizeof(double) * len_all, c.stream));
      int budget_its = std::min(p.max_it - inner_max, 4 * p.restart);
      std::vector<KResult> in = S.kry.solve(S.op32, S.r.get(), S.d.get(), true, kInnerRtol, 0.0, 1e10, budget_its, true,
                                            c.stream);
      int step = 0;
      bool progress = false;
      for (int v = 0; v < nv; v++) {
        if (reason[v]) continue;
        its[v] += in[v].its;
        step = std::max(step, in[v].its);
        progress = progress || in[v].its > 0;
      }
      inner_max += step;
      axpy_dev(nall, 1.0, S.d.get(), S.x.get(), c.stream);
      xzero = false;
      if (!progress) stalled = true;
    }
    if (stalled) {
      // FP64 blocks and FP64 GMRES from zero for every right-hand side (the inner
      // iterations spent so far stay counted)
      S.kry.reset_graph();
      rasm_build(S.rasm, S.pts, false, c.ws, c.err.get(), c.stream, budget, false, p.pc_type == PRBF_PC_ASM);
      rasm_set_apply_smem(S.rasm);
      c.check_device_error("RASM set-up (FP64 fallback)");
      PRBF_CUDA(cudaMemsetAsync(S.x.get(), 0, sizeof(double) * len_all, c.stream));
      std::fill(reason.begin(), reason.end(), 0);
      st.fp64_fallback = 1;
      resid_current = false;
      plain_solve(false);
    } else {
      for (int v = 0; v < nv; v++)
        if (!reason[v]) reason[v] = -3;
    }
  }
  PRBF_CUDA(cudaStreamSynchronize(c.stream));
  const double t_solve = now_ms() - ts0;
  tr_solve.end();
  TraceRange tr_post("Post Processing");
  c.check_device_error("solve");
  // weights back in the caller's order (2d/rbf_interpolation.cxx:246-265)
  for (int v = 0; v < nv; v++) {
    scatter_dev(n, S.pts.perm.get(), S.x.get() + v * ldn, S.tmp.get(), c.stream);
    PRBF_CUDA(cudaMemcpyAsync(g_out + (size_t)v * n, S.tmp.get(), sizeof(double) * n, cudaMemcpyDeviceToHost,
                              c.stream));
  }
  // true residual ||b - A x|| / ||b|| in FP64 (reported, not part of the solve)
  if (!resid_current) {
    S.op64.apply_A(S.x.get(), S.r.get(), nullptr, c.stream);
    axpy_dev((int)(ldn * nv), -1.0, S.b.get(), S.r.get(), c.stream);
    std::vector<double> rr = seg_norm2_host(S.kry, S.r.get(), c.stream),
                        bn = seg_norm2_host(S.kry, S.b.get(), c.stream);
    for (int v = 0; v < nv; v++) {
      double q = std::sqrt(rr[v]), bq = std::sqrt(bn[v]);
      true_rel[v] = bq > 0 ? q / bq : q;
    }
  }
  // reason: the first failure if any, else 2 (rtol) unless every system stopped on atol
  st.reason = 3;
  for (int v = 0; v < nv; v++) {
    st.true_rel_resid = std::max(st.true_rel_resid, true_rel[v]);
    st.its += its[v];
    st.outer_its += outer[v];
    if (st.reason < 0) continue;
    if (reason[v] < 0 || reason[v] == 2) st.reason = reason[v];
  }
  st.rnorm0 = rnorm0[nv - 1];
  st.rnorm = rnorm[nv - 1];
  st.t_sort_ms = t_sorted - t_begin;
  st.t_setup_ms = t_setup - t_sorted;
  st.t_solve_ms = t_solve;
  st.t_total_ms = now_ms() - t_begin;
  if (stats) *stats = st;
  if (st.reason == -3) throw Error(PRBF_ERR_NOT_CONVERGED, "iteration limit reached before the tolerance");
  if (st.reason == -5) throw Error(PRBF_ERR_BREAKDOWN, "GMRES breakdown");
  if (st.reason == -9) throw Error(PRBF_ERR_NAN, "NaN or Inf residual");
  if (st.reason == -4) throw Error(PRBF_ERR_DIVERGED, "residual grew past dtol");
}

}  // namespace prbf

using namespace prbf;

extern "C" {

int prbf_interpolate(prbf_ctx* ctx, int n, const double* x, const double* y, const double* z, const double* f, int nrhs,
                     double* g_out, prbf_stats* stats) {
  return ctx_call(ctx, [&](Ctx& c) {
    if (n <= 0 || n > (1 << 30)) throw Error(PRBF_ERR_ARG, "point count must be in [1, 2^30]");
    if (!x || !y || (c.p.dim == 3 && !z) || !f || !g_out || nrhs <= 0)
      throw Error(PRBF_ERR_ARG, "null array or nrhs <= 0");
    interpolate(c, n, x, y, z, f, nrhs, g_out, stats);
  });
}

int prbf_pc_setup(prbf_ctx* ctx, int precision) {
  return ctx_call(ctx, [&](Ctx& c) {
    if (!c.mv_ready) throw Error(PRBF_ERR_STATE, "prbf_matvec_setup has not been called");
    if (precision != PRBF_PREC_FP64 && precision != PRBF_PREC_MIXED) throw Error(PRBF_ERR_ARG, "bad precision");
    if (!c.solve) c.solve = new SolveState();
    c.solve->pc_ready = false;
    size_t free_b = 0, total_b = 0;
    PRBF_CUDA(cudaMemGetInfo(&free_b, &total_b));
    const bool fp32 = precision == PRBF_PREC_MIXED;
    c.solve->pc.lu_fallback = c.p.block_fallback == PRBF_FALLBACK_LU;
    rasm_build(c.solve->pc, c.mv_pts, fp32, c.ws, c.err.get(), c.stream, std::min(16.0e9, 0.25 * (double)free_b),
               fp32 && c.mv_pts.g.dim == 3, c.p.pc_type == PRBF_PC_ASM);
    rasm_set_apply_smem(c.solve->pc);
    c.check_device_error("RASM set-up");
    c.solve->pc_ready = true;
  });
}

int prbf_pc_apply(prbf_ctx* ctx, const double* r, double* z) {
  return ctx_call(ctx, [&](Ctx& c) {
    if (!c.solve || !c.solve->pc_ready) throw Error(PRBF_ERR_STATE, "prbf_pc_setup has not been called");
    if (!r || !z) throw Error(PRBF_ERR_ARG, "null vector");
    int n = c.mv_pts.n;
    PRBF_CUDA(cudaMemcpyAsync(c.vtmp.get(), r, sizeof(double) * n, cudaMemcpyHostToDevice, c.stream));
    gather_dev(n, c.mv_pts.perm.get(), c.vtmp.get(), c.vin.get(), c.stream);
    rasm_apply(c.solve->pc, c.mv_pts.cs.get(), c.vin.get(), c.vout.get(), c.stream);
    scatter_dev(n, c.mv_pts.perm.get(), c.vout.get(), c.vtmp.get(), c.stream);
    PRBF_CUDA(cudaMemcpyAsync(z, c.vtmp.get(), sizeof(double) * n, cudaMemcpyDeviceToHost, c.stream));
    c.check_device_error("pc apply");
  });
}

int prbf_pc_buffer_lists(prbf_ctx* ctx, long long* off_out, int* idx_out) {
  return ctx_call(ctx, [&](Ctx& c) {
    if (!c.solve || !c.solve->pc_ready) throw Error(PRBF_ERR_STATE, "prbf_pc_setup has not been called");
    const RasmPlan& R = c.solve->pc;
    const int ncell = c.mv_pts.g.ncell;
    std::vector<long long> off(ncell + 1);
    PRBF_CUDA(cudaMemcpyAsync(off.data(), R.boff.get(), sizeof(long long) * (ncell + 1), cudaMemcpyDeviceToHost,
                              c.stream));
    PRBF_CUDA(cudaStreamSynchronize(c.stream));
    if (off_out) std::copy(off.begin(), off.end(), off_out);
    if (idx_out && off[ncell] > 0) {
      PRBF_CUDA(cudaMemcpyAsync(idx_out, R.idx.get(), sizeof(int) * off[ncell], cudaMemcpyDeviceToHost, c.stream));
      PRBF_CUDA(cudaStreamSynchronize(c.stream));
    }
  });
}

int prbf_pc_block(prbf_ctx* ctx, int cell, int* nb_out, int* nc_out, double* K_out, double* L_out) {
  return ctx_call(ctx, [&](Ctx& c) {
    if (!c.solve || !c.solve->pc_ready) throw Error(PRBF_ERR_STATE, "prbf_pc_setup has not been called");
    const RasmPlan& R = c.solve->pc;
    if (cell < 0 || cell >= c.mv_pts.g.ncell) throw Error(PRBF_ERR_ARG, "no such cell");
    long long bo[2];
    int cs2[2];
    PRBF_CUDA(cudaMemcpyAsync(bo, R.boff.get() + cell, sizeof(bo), cudaMemcpyDeviceToHost, c.stream));
    PRBF_CUDA(cudaMemcpyAsync(cs2, c.mv_pts.cs.get() + cell, sizeof(cs2), cudaMemcpyDeviceToHost, c.stream));
    PRBF_CUDA(cudaStreamSynchronize(c.stream));
    const int nb = (int)(bo[1] - bo[0]), nc = cs2[1] - cs2[0];
    if (nb_out) *nb_out = nb;
    if (nc_out) *nc_out = nc;
    if (nb == 0) return;
    if (K_out) {
      double* Kd = (double*)c.ws.get(56, sizeof(double) * (size_t)nb * nb);
      rasm_block_K(R, c.mv_pts, cell, nb, Kd, c.ws, c.stream);
      PRBF_CUDA(cudaMemcpyAsync(K_out, Kd, sizeof(double) * (size_t)nb * nb, cudaMemcpyDeviceToHost, c.stream));
      PRBF_CUDA(cudaStreamSynchronize(c.stream));
      for (int i = 0; i < nb; i++)
        for (int j = 0; j < i; j++) K_out[(size_t)j * nb + i] = K_out[(size_t)i * nb + j];
      c.check_device_error("block read-back");
    }
    if (L_out) rasm_factor_rows(R, cell, nb, L_out, c.stream);
  });
}

// 3d/wrapper.cxx:20-105 with the same argument meaning. It creates its own context on
// device 0 (the reference calls PetscInitialize on every call) and frees it on return.
int prbf_RBFInterpolation(int argc, char** argv, int ng, float* xg, float* yg, float* zg, float* wg, int np, float* xp,
                          float* yp, float* zp, float* gp, float sigma, int nsigma_box, int sigma_buffer,
                          int sigma_trunc) {
  (void)argc;
  (void)argv;
  if (ng <= 0 || !xg || !yg || !zg || !wg) return PRBF_ERR_ARG;
  // the particle field is evaluated at the grid points first when the first grid point
  // differs from the first particle (3d/wrapper.cxx:93-95)
  const bool eval_first = np > 0 && xp && std::fabs(xg[0] - xp[0]) > kEpsf;
  if (eval_first && (!yp || !zp || !gp)) return PRBF_ERR_ARG;
  prbf_params p;
  prbf_params_default(&p);
  p.block_fallback = PRBF_FALLBACK_LU;  // the reference's -sub_pc_type lu on singular blocks
  p.dim = 3;
  p.sigma = sigma;
  p.nsigma_box = nsigma_box;
  p.sigma_buffer = sigma_buffer;
  p.sigma_trunc = sigma_trunc;
  prbf_ctx* ctx = nullptr;
  int st = prbf_ctx_create(&p, &ctx);
  if (st) return st;
  std::vector<double> xi(xg, xg + ng), yi(yg, yg + ng), zi(zg, zg + ng), wi(wg, wg + ng), gi(ng);
  if (eval_first) {
    std::vector<double> xj(xp, xp + np), yj(yp, yp + np), zj(zp, zp + np), gj(gp, gp + np);
    st = prbf_evaluate(ctx, ng, xi.data(), yi.data(), zi.data(), np, xj.data(), yj.data(), zj.data(), gj.data(),
                       wi.data());
  }
  if (!st) st = prbf_interpolate(ctx, ng, xi.data(), yi.data(), zi.data(), wi.data(), 1, gi.data(), nullptr);
  if (!st)
    for (int i = 0; i < ng; i++) wg[i] = (float)gi[i];  // weights written over wg (3d/wrapper.cxx:98-101)
  prbf_ctx_destroy(ctx);
  return st;
}

}  // extern "C"

// The reference's library entry with its own C++ signature and linkage (3d/wrapper.cxx:20-23,
// the symbol librbf.a exports), so a program built against librbf.a links against this
// library unchanged.
int RBFInterpolation(int argc, char** argv, int ng, float* xg, float* yg, float* zg, float* wg, int np, float* xp,
                     float* yp, float* zp, float* gp, float sigma, int nsigma_box, int sigma_buffer, int sigma_trunc) {
  return prbf_RBFInterpolation(argc, argv, ng, xg, yg, zg, wg, np, xp, yp, zp, gp, sigma, nsigma_box, sigma_buffer,
                               sigma_trunc);
}
