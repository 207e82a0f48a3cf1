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
// stops on the true residual ||f - A g||_2 <= rtol ||f||_2.
#include <chrono>
#include <cmath>
#include <cstring>
#include <vector>

#include "krylov.h"
#include "mlp.h"
#include "rasm.h"

namespace prbf {

namespace {

struct GaussRasmOp : Operator {
  const GaussPlan* plan = nullptr;
  PointsView v{};
  const RasmPlan* rasm = nullptr;
  bool fp32 = false;
  unsigned* err = nullptr;
  void apply_A(const double* x, double* y, const int* skip, cudaStream_t s) const override {
    gauss_sum_dev(*plan, v, v, x, y, fp32, err, s, skip);
  }
  void apply_B(const double* r, double* z, const int* skip, cudaStream_t s) const override {
    rasm_apply(*rasm, v.cell_start, r, z, s, skip);
  }
};

double now_ms() {
  using namespace std::chrono;
  return duration<double, std::milli>(steady_clock::now().time_since_epoch()).count();
}

}  // namespace

double norm2_host(const double* v, int n, Workspace& ws, cudaStream_t s);

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
  S.plan.g = S.pts.g;
  gauss_plan_dev(S.plan, S.pts.view(), S.pts.view(), c.err.get(), c.ws, c.stream);
  const bool mixed = p.precision == PRBF_PREC_MIXED;
  size_t free_b = 0, total_b = 0;
  PRBF_CUDA(cudaMemGetInfo(&free_b, &total_b));
  double budget = std::min(16.0e9, 0.25 * (double)free_b);
  // FP32 blocks: S_c (one GEMV per apply) in 2D; in 3D the blocks are too ill-conditioned
  // for an explicit FP32 inverse, so the FP32 factor is kept and applied by substitution
  rasm_build(S.rasm, S.pts, mixed, c.ws, c.err.get(), c.stream, budget, mixed && dim == 3,
             p.pc_type == PRBF_PC_ASM);
  rasm_set_apply_smem(S.rasm);
  c.check_device_error("RASM set-up");
  const double t_setup = now_ms();

  S.op64.plan = S.op32.plan = &S.plan;
  S.op64.v = S.op32.v = S.pts.view();
  S.op64.rasm = S.op32.rasm = &S.rasm;
  S.op64.err = S.op32.err = c.err.get();
  S.op64.fp32 = false;
  S.op32.fp32 = true;
  const long long ld = (long long)n + 4;
  S.b.reserve(ld);
  S.x.reserve(ld);
  S.r.reserve(ld);
  S.d.reserve(ld);
  S.tmp.reserve(ld);
  for (auto* v : {&S.b, &S.x, &S.r, &S.d, &S.tmp}) PRBF_CUDA(cudaMemsetAsync(v->get(), 0, sizeof(double) * ld, c.stream));
  if (S.kry.n != n || S.kry.m != p.restart) {
    S.kry.reset_graph();
    S.kry.init(n, p.restart, c.stream);
  }
  S.kry.graph_op = nullptr;  // operators are rebuilt per call

  const bool use_guess = p.guess == PRBF_GUESS_LEARNED;
  if (use_guess && (dim != 2 || !c.guess || !c.guess->ready))
    throw Error(PRBF_ERR_STATE, "learned guess requested without installed weights (2D only)");
  prbf_stats st{};
  st.ncell = S.pts.g.ncell;
  st.max_block = S.rasm.max_nb;
  st.nblocks_fallback = S.rasm.nfallback;
  st.pairs_per_matvec = S.plan.pairs;
  double t_solve = 0;
  for (int rhs = 0; rhs < nrhs; rhs++) {
    const double* fr = f + (size_t)rhs * n;
    PRBF_CUDA(cudaMemcpyAsync(S.tmp.get(), fr, sizeof(double) * n, cudaMemcpyHostToDevice, c.stream));
    gather_dev(n, S.pts.perm.get(), S.tmp.get(), S.b.get(), c.stream);
    PRBF_CUDA(cudaMemsetAsync(S.x.get(), 0, sizeof(double) * ld, c.stream));
    PRBF_CUDA(cudaStreamSynchronize(c.stream));
    const double ts0 = now_ms();
    if (use_guess) {
      // x0 from the network, in the solver's cell order (its inputs are the sorted points)
      guess_compute(c, *c.guess, n, S.pts.x.get(), S.pts.y.get(), S.b.get(), S.x.get());
      st.t_guess_ms += now_ms() - ts0;
    }
    KResult kr;
    int outer = 0, inner_its = 0;
    if (!mixed) {
      double ref = 0.0;
      if (use_guess) {
        // converge relative to the zero-guess residual ||B b||, whatever the guess
        S.op64.apply_B(S.b.get(), S.tmp.get(), nullptr, c.stream);
        ref = norm2_host(S.tmp.get(), n, c.ws, c.stream);
      }
      kr = S.kry.solve(S.op64, S.b.get(), S.x.get(), !use_guess, p.rtol, p.abstol, p.dtol, p.max_it, true, c.stream,
                       ref, use_guess);
      inner_its = kr.its;
      if (use_guess) {
        st.guess_used = kr.guess_used ? 1 : 0;
        st.guess_rel_resid = ref > 0 ? kr.guess_beta / ref : 1.0;
      }
    } else {
      const double bnorm = norm2_host(S.b.get(), n, c.ws, c.stream);
      bool xzero = !use_guess;
      kr.reason = 0;
      for (outer = 0; outer < 50; outer++) {
        // r = b - A x in FP64
        if (xzero) {
          PRBF_CUDA(cudaMemcpyAsync(S.r.get(), S.b.get(), sizeof(double) * n, cudaMemcpyDeviceToDevice, c.stream));
        } else {
          S.op64.apply_A(S.x.get(), S.r.get(), nullptr, c.stream);
          axpy_dev(n, -1.0, S.b.get(), S.r.get(), c.stream);  // r = Ax - b
          PRBF_CUDA(cudaMemcpyAsync(S.tmp.get(), S.r.get(), sizeof(double) * n, cudaMemcpyDeviceToDevice, c.stream));
          PRBF_CUDA(cudaMemsetAsync(S.r.get(), 0, sizeof(double) * n, c.stream));
          axpy_dev(n, -1.0, S.tmp.get(), S.r.get(), c.stream);  // r = b - Ax
        }
        double rn = norm2_host(S.r.get(), n, c.ws, c.stream);
        if (outer == 0 && use_guess) {
          st.guess_rel_resid = bnorm > 0 ? rn / bnorm : 1.0;
          st.guess_used = rn <= bnorm ? 1 : 0;
          if (!st.guess_used) {  // worse than zero: drop the guess
            PRBF_CUDA(cudaMemsetAsync(S.x.get(), 0, sizeof(double) * ld, c.stream));
            PRBF_CUDA(cudaMemcpyAsync(S.r.get(), S.b.get(), sizeof(double) * n, cudaMemcpyDeviceToDevice, c.stream));
            xzero = true;
            rn = bnorm;
          }
        }
        if (outer == 0) kr.rnorm0 = rn;
        kr.rnorm = rn;
        if (!(rn == rn)) {
          kr.reason = -9;
          break;
        }
        if (rn <= p.rtol * bnorm || rn <= p.abstol) {
          kr.reason = rn <= p.abstol ? 3 : 2;
          break;
        }
        if (inner_its >= p.max_it) {
          kr.reason = -3;
          break;
        }
        PRBF_CUDA(cudaMemsetAsync(S.d.get(), 0, sizeof(double) * ld, c.stream));
        int budget_its = std::min(p.max_it - inner_its, 4 * p.restart);
        KResult in = S.kry.solve(S.op32, S.r.get(), S.d.get(), true, 1e-6, 0.0, 1e10, budget_its, true, c.stream);
        inner_its += in.its;
        axpy_dev(n, 1.0, S.d.get(), S.x.get(), c.stream);
        xzero = false;
        if (in.its == 0) {
          kr.reason = -5;
          break;
        }
      }
      if (!kr.reason) kr.reason = -3;
    }
    PRBF_CUDA(cudaStreamSynchronize(c.stream));
    t_solve += now_ms() - ts0;
    c.check_device_error("solve");
    // weights back in the caller's order (2d/rbf_interpolation.cxx:246-265)
    scatter_dev(n, S.pts.perm.get(), S.x.get(), S.tmp.get(), c.stream);
    PRBF_CUDA(cudaMemcpyAsync(g_out + (size_t)rhs * n, S.tmp.get(), sizeof(double) * n, cudaMemcpyDeviceToHost, c.stream));
    // true residual ||b - A x|| / ||b|| in FP64 (reported, not part of the solve)
    S.op64.apply_A(S.x.get(), S.r.get(), nullptr, c.stream);
    axpy_dev(n, -1.0, S.b.get(), S.r.get(), c.stream);
    double rr = norm2_host(S.r.get(), n, c.ws, c.stream), bn = norm2_host(S.b.get(), n, c.ws, c.stream);
    st.its += inner_its;
    st.outer_its += outer;
    st.reason = kr.reason;
    st.rnorm0 = kr.rnorm0;
    st.rnorm = kr.rnorm;
    st.true_rel_resid = std::max(st.true_rel_resid, bn > 0 ? rr / bn : rr);
    if (kr.reason < 0) break;
  }
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
  if (!ctx) return PRBF_ERR_ARG;
  Ctx& c = ctx->c;
  try {
    c.last_error.clear();
    PRBF_CUDA(cudaSetDevice(c.device));
    if (n <= 0 || n > (1 << 30)) throw Error(PRBF_ERR_ARG, "point count must be in [1, 2^30]");
    if (!x || !y || (c.p.dim == 3 && !z) || !f || !g_out || nrhs <= 0)
      throw Error(PRBF_ERR_ARG, "null array or nrhs <= 0");
    interpolate(c, n, x, y, z, f, nrhs, g_out, stats);
    return PRBF_OK;
  } catch (const Error& e) {
    c.last_error = e.what();
    return e.status;
  } catch (const std::exception& e) {
    c.last_error = e.what();
    return PRBF_ERR_ARG;
  }
}

int prbf_pc_setup(prbf_ctx* ctx, int precision) {
  if (!ctx) return PRBF_ERR_ARG;
  Ctx& c = ctx->c;
  try {
    c.last_error.clear();
    PRBF_CUDA(cudaSetDevice(c.device));
    if (!c.mv_ready) throw Error(PRBF_ERR_STATE, "prbf_matvec_setup has not been called");
    if (precision != PRBF_PREC_FP64 && precision != PRBF_PREC_MIXED) throw Error(PRBF_ERR_ARG, "bad precision");
    if (!c.solve) c.solve = new SolveState();
    c.solve->pc_ready = false;
    size_t free_b = 0, total_b = 0;
    PRBF_CUDA(cudaMemGetInfo(&free_b, &total_b));
    const bool fp32 = precision == PRBF_PREC_MIXED;
    rasm_build(c.solve->pc, c.mv_pts, fp32, c.ws, c.err.get(), c.stream, std::min(16.0e9, 0.25 * (double)free_b),
               fp32 && c.mv_pts.g.dim == 3, c.p.pc_type == PRBF_PC_ASM);
    rasm_set_apply_smem(c.solve->pc);
    c.check_device_error("RASM set-up");
    c.solve->pc_ready = true;
    return PRBF_OK;
  } catch (const Error& e) {
    c.last_error = e.what();
    return e.status;
  }
}

int prbf_pc_apply(prbf_ctx* ctx, const double* r, double* z) {
  if (!ctx) return PRBF_ERR_ARG;
  Ctx& c = ctx->c;
  try {
    c.last_error.clear();
    PRBF_CUDA(cudaSetDevice(c.device));
    if (!c.solve || !c.solve->pc_ready) throw Error(PRBF_ERR_STATE, "prbf_pc_setup has not been called");
    if (!r || !z) throw Error(PRBF_ERR_ARG, "null vector");
    int n = c.mv_pts.n;
    PRBF_CUDA(cudaMemcpyAsync(c.vtmp.get(), r, sizeof(double) * n, cudaMemcpyHostToDevice, c.stream));
    gather_dev(n, c.mv_pts.perm.get(), c.vtmp.get(), c.vin.get(), c.stream);
    rasm_apply(c.solve->pc, c.mv_pts.cs.get(), c.vin.get(), c.vout.get(), c.stream);
    scatter_dev(n, c.mv_pts.perm.get(), c.vout.get(), c.vtmp.get(), c.stream);
    PRBF_CUDA(cudaMemcpyAsync(z, c.vtmp.get(), sizeof(double) * n, cudaMemcpyDeviceToHost, c.stream));
    c.check_device_error("pc apply");
    return PRBF_OK;
  } catch (const Error& e) {
    c.last_error = e.what();
    return e.status;
  }
}

// 3d/wrapper.cxx:20-105 with the same argument meaning. It creates its own context on
// device 0 (the reference calls PetscInitialize on every call) and frees it on return.
int prbf_RBFInterpolation(int argc, char** argv, int ng, float* xg, float* yg, float* zg, float* wg, int np, float* xp,
                          float* yp, float* zp, float* gp, float sigma, int nsigma_box, int sigma_buffer,
                          int sigma_trunc) {
  (void)argc;
  (void)argv;
  if (ng <= 0 || !xg || !yg || !zg || !wg) return PRBF_ERR_ARG;
  prbf_params p;
  prbf_params_default(&p);
  p.dim = 3;
  p.sigma = sigma;
  p.nsigma_box = nsigma_box;
  p.sigma_buffer = sigma_buffer;
  p.sigma_trunc = sigma_trunc;
  prbf_ctx* ctx = nullptr;
  int st = prbf_ctx_create(&p, &ctx);
  if (st) return st;
  std::vector<double> xi(xg, xg + ng), yi(yg, yg + ng), zi(zg, zg + ng), wi(wg, wg + ng), gi(ng);
  // the particle field is evaluated at the grid points first when the first grid point
  // differs from the first particle (3d/wrapper.cxx:93-95)
  if (np > 0 && xp && std::fabs(xg[0] - xp[0]) > kEpsf) {
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
