// capi.cu -- C ABI: context, the MatShell matvec seam (mymatmult) and the evaluation of
// the interpolant (vorticity_evaluation). The solve (rbf_interpolation) is in solve.cu.
#include <chrono>
#include <cmath>
#include <cstring>

#include "context.h"

namespace prbf {

Grid make_grid(int dim, const double* b, double sigma, int nsigma_box, int sigma_buffer,
               int sigma_trunc) {
  if (dim != 2 && dim != 3) throw Error(PRBF_ERR_ARG, "dim must be 2 or 3");
  if (!(sigma > 0) || !std::isfinite(sigma)) throw Error(PRBF_ERR_ARG, "sigma must be > 0");
  if (nsigma_box <= 0 || sigma_buffer < 0 || sigma_trunc < 0)
    throw Error(PRBF_ERR_ARG, "box widths must be positive");
  for (int k = 0; k < 2 * dim; k++)
    if (!std::isfinite(b[k])) throw Error(PRBF_ERR_RANGE, "non-finite coordinate");
  Grid g{};
  g.dim = dim;
  g.sigma = sigma;
  // neighbor_buffer / neighbor_trunc (2d/get_cluster.h:176-177)
  g.nb_buffer = (int)std::ceil((sigma_buffer - nsigma_box + kEpsf) / 2 / nsigma_box);
  g.nb_trunc = (int)std::ceil((sigma_trunc - nsigma_box + kEpsf) / 2 / nsigma_box);
  if (g.nb_buffer < 0) g.nb_buffer = 0;
  if (g.nb_trunc < 0) g.nb_trunc = 0;
  double xmin = b[0] - kEpsf, xmax = b[1] + kEpsf;
  double ymin = b[2] - kEpsf, ymax = b[3] + kEpsf;
  double zmin = dim == 3 ? b[4] - kEpsf : 0.0, zmax = dim == 3 ? b[5] + kEpsf : 0.0;
  g.xmin = xmin;
  g.ymin = ymin;
  g.zmin = zmin;
  g.box = nsigma_box * sigma + kEpsf;
  double fx = std::ceil((xmax - xmin) / g.box), fy = std::ceil((ymax - ymin) / g.box);
  double fz = dim == 3 ? std::ceil((zmax - zmin) / g.box) : 1.0;
  if (!(fx * fy * fz < 1073741824.0)) throw Error(PRBF_ERR_RANGE, "cell grid exceeds 2^30 cells");
  g.nx = (int)fx;
  g.ny = (int)fy;
  g.nz = (int)fz;
  g.ncell = g.nx * g.ny * g.nz;
  g.trunc_len = sigma_trunc * sigma / 2 + kEpsf;
  g.buffer_len = sigma_buffer * sigma / 2 + kEpsf;
  return g;
}

void ctx_stream_release(Ctx& c) {
  if (c.stream) cudaStreamSynchronize(c.stream);
  if (c.stream) cudaStreamDestroy(c.stream);
  c.stream = nullptr;
}

void Ctx::check_device_error(const char* what) {
  unsigned h = 0;
  PRBF_CUDA(cudaMemcpyAsync(&h, err.get(), sizeof(unsigned), cudaMemcpyDeviceToHost, stream));
  PRBF_CUDA(cudaStreamSynchronize(stream));
  if (h) {
    PRBF_CUDA(cudaMemsetAsync(err.get(), 0, sizeof(unsigned), stream));
    if (h & DEV_ERR_RANGE) throw Error(PRBF_ERR_RANGE, std::string(what) + ": point outside the cell grid or non-finite");
    if (h & DEV_ERR_TIMEOUT) throw Error(PRBF_ERR_TIMEOUT, std::string(what) + ": bounded device wait gave up");
    if (h & DEV_ERR_CAPACITY) throw Error(PRBF_ERR_CAPACITY, std::string(what) + ": device capacity exceeded");
    if (h & DEV_ERR_FACTOR) throw Error(PRBF_ERR_FACTOR, std::string(what) + ": block factorisation failed");
    if (h & DEV_ERR_INDEX)
      throw Error(PRBF_ERR_CAPACITY, std::string(what) + ": a kernel's bounds check caught an index out of range");
  }
}

void Ctx::upload(DevBuf<double>& dst, const double* src, int n, int pad) {
  dst.reserve((size_t)n + pad);
  PRBF_CUDA(cudaMemcpyAsync(dst.get(), src, sizeof(double) * n, cudaMemcpyHostToDevice, stream));
  if (pad) PRBF_CUDA(cudaMemsetAsync(dst.get() + n, 0, sizeof(double) * pad, stream));
}

void bbox_host(Ctx& c, int n, const double* dx, const double* dy, const double* dz, double* out6) {
  double* d = (double*)c.ws.get(30, sizeof(double) * 6);
  bbox_dev(n, dx, dy, dz, d, c.ws, c.stream);
  PRBF_CUDA(cudaMemcpyAsync(out6, d, sizeof(double) * 6, cudaMemcpyDeviceToHost, c.stream));
  PRBF_CUDA(cudaStreamSynchronize(c.stream));
}

void build_points(Ctx& c, PointSet& ps, const Grid& g, int n, const double* dx, const double* dy,
                  const double* dz) {
  ps.n = n;
  ps.g = g;
  ps.perm.reserve(n);
  ps.cs.reserve((size_t)g.ncell + 1);
  cell_sort_dev(g, n, dx, dy, dz, ps.perm.get(), ps.cs.get(), c.err.get(), c.ws, c.stream);
  c.check_device_error("cell sort");
  DevBuf<double>* dst[3] = {&ps.x, &ps.y, &ps.z};
  const double* src[3] = {dx, dy, dz};
  for (int d = 0; d < g.dim; d++) {
    dst[d]->reserve((size_t)n + 4);
    PRBF_CUDA(cudaMemsetAsync(dst[d]->get() + n, 0, sizeof(double) * 4, c.stream));
    gather_dev(n, ps.perm.get(), src[d], dst[d]->get(), c.stream);
  }
}

}  // namespace prbf

using namespace prbf;

namespace {

void check_n(int n) {
  if (n <= 0 || n > (1 << 30)) throw Error(PRBF_ERR_ARG, "point count must be in [1, 2^30]");
}

void upload_coords(Ctx& c, int n, const double* x, const double* y, const double* z, DevBuf<double>& bx,
                   DevBuf<double>& by, DevBuf<double>& bz) {
  if (!x || !y || (c.p.dim == 3 && !z)) throw Error(PRBF_ERR_ARG, "null coordinate array");
  c.upload(bx, x, n);
  c.upload(by, y, n);
  if (c.p.dim == 3) c.upload(bz, z, n);
}

}  // namespace

namespace prbf {
namespace {
// A wait that nothing completes: one warp initialises an mbarrier that expects one arrival
// which never comes, polls it max_polls times with the bounded wait of the kernels, and
// raises DEV_ERR_TIMEOUT -- the path a lost copy or MMA completion takes, run without
// leaving anything behind (no copy or MMA is in flight, the barrier dies with the CTA).
__global__ void k_selftest_wait(unsigned max_polls, unsigned* err) {
  __shared__ __align__(8) uint64_t bar;
  if (threadIdx.x == 0) mbar_init(&bar, 1);
  __syncthreads();
  const bool done = mbar_wait(&bar, 0, max_polls);
  if (!done && threadIdx.x == 0) atomicOr(err, DEV_ERR_TIMEOUT);
}
}  // namespace
}  // namespace prbf

extern "C" {

void prbf_params_default(prbf_params* p) {
  if (!p) return;
  std::memset(p, 0, sizeof(*p));
  p->dim = 2;
  p->sigma = 0.025;
  p->nsigma_box = 8;
  p->sigma_buffer = 24;
  p->sigma_trunc = 24;
  p->rtol = 1e-13;
  p->abstol = 1e-50;
  p->dtol = 1e5;
  p->restart = 30;
  p->max_it = 1000;
  p->precision = PRBF_PREC_FP64;
  p->guess = PRBF_GUESS_ZERO;
  p->device = 0;
  p->pc_type = PRBF_PC_RASM;
  p->block_fallback = PRBF_FALLBACK_SHIFT;
}

const char* prbf_status_string(int s) {
  switch (s) {
    case PRBF_OK: return "ok";
    case PRBF_ERR_ARG: return "bad argument";
    case PRBF_ERR_RANGE: return "out of range";
    case PRBF_ERR_CAPACITY: return "capacity exceeded";
    case PRBF_ERR_CUDA: return "CUDA error";
    case PRBF_ERR_NOT_CONVERGED: return "not converged";
    case PRBF_ERR_BREAKDOWN: return "breakdown";
    case PRBF_ERR_NAN: return "NaN or Inf residual";
    case PRBF_ERR_STATE: return "call out of order";
    case PRBF_ERR_FACTOR: return "block factorisation failed";
    case PRBF_ERR_DIVERGED: return "diverged";
    case PRBF_ERR_TIMEOUT: return "device wait timed out";
    default: return "unknown status";
  }
}

int prbf_ctx_create(const prbf_params* p, prbf_ctx** out) {
  if (!p || !out) return PRBF_ERR_ARG;
  *out = nullptr;
  if (p->dim != 2 && p->dim != 3) return PRBF_ERR_ARG;
  if (!(p->sigma > 0) || p->nsigma_box <= 0 || p->restart <= 0 || p->max_it < 0) return PRBF_ERR_ARG;
  if (p->pc_type != PRBF_PC_RASM && p->pc_type != PRBF_PC_ASM) return PRBF_ERR_ARG;
  if (p->block_fallback != PRBF_FALLBACK_SHIFT && p->block_fallback != PRBF_FALLBACK_LU) return PRBF_ERR_ARG;
  prbf_ctx* ctx = new (std::nothrow) prbf_ctx();
  if (!ctx) return PRBF_ERR_CAPACITY;
  ctx->c.p = *p;
  ctx->c.device = p->device;
  try {
    int ndev = 0;
    PRBF_CUDA(cudaGetDeviceCount(&ndev));
    if (p->device < 0 || p->device >= ndev) throw Error(PRBF_ERR_ARG, "no such CUDA device");
    PRBF_CUDA(cudaSetDevice(p->device));
    PRBF_CUDA(cudaStreamCreateWithFlags(&ctx->c.stream, cudaStreamNonBlocking));
    ctx->c.err.reserve(4);
    PRBF_CUDA(cudaMemsetAsync(ctx->c.err.get(), 0, 16, ctx->c.stream));
  } catch (const Error& e) {
    int st = e.status;
    delete ctx;
    return st;
  }
  *out = ctx;
  return PRBF_OK;
}

int prbf_ctx_destroy(prbf_ctx* ctx) {
  if (!ctx) return PRBF_ERR_ARG;
  cudaSetDevice(ctx->c.device);
  delete ctx;
  return PRBF_OK;
}

const char* prbf_last_error(const prbf_ctx* ctx) { return ctx ? ctx->c.last_error.c_str() : "null context"; }

void* prbf_ctx_stream(prbf_ctx* ctx) { return ctx ? (void*)ctx->c.stream : nullptr; }

int prbf_ctx_synchronize(prbf_ctx* ctx) {
  return ctx_call(ctx, [&](Ctx& c) { PRBF_CUDA(cudaStreamSynchronize(c.stream)); });
}

int prbf_selftest_wait_timeout(prbf_ctx* ctx, unsigned max_polls) {
  return ctx_call(ctx, [&](Ctx& c) {
    if (max_polls == 0 || max_polls > (1u << 20)) throw Error(PRBF_ERR_ARG, "max_polls must be in [1, 2^20]");
    k_selftest_wait<<<1, 32, 0, c.stream>>>(max_polls, c.err.get());
    PRBF_CHECK_LAUNCH();
    c.check_device_error("self-test wait");
  });
}

int prbf_matvec_setup(prbf_ctx* ctx, int n, const double* x, const double* y, const double* z) {
  return ctx_call(ctx, [&](Ctx& c) {
    check_n(n);
    c.mv_ready = false;
    DevBuf<double> ux, uy, uz;
    upload_coords(c, n, x, y, z, ux, uy, uz);
    double b[6];
    bbox_host(c, n, ux.get(), uy.get(), c.p.dim == 3 ? uz.get() : nullptr, b);
    Grid g = make_grid(c.p.dim, b, c.p.sigma, c.p.nsigma_box, c.p.sigma_buffer, c.p.sigma_trunc);
    build_points(c, c.mv_pts, g, n, ux.get(), uy.get(), c.p.dim == 3 ? uz.get() : nullptr);
    c.mv_plan.g = g;
    gauss_plan_dev(c.mv_plan, c.mv_pts.view(), c.mv_pts.view(), c.err.get(), c.ws, c.stream);
    c.vin.reserve((size_t)n + 4);
    c.vout.reserve((size_t)n + 4);
    c.vtmp.reserve((size_t)n + 4);
    PRBF_CUDA(cudaMemsetAsync(c.vin.get(), 0, sizeof(double) * (n + 4), c.stream));
    PRBF_CUDA(cudaStreamSynchronize(c.stream));
    c.mv_ready = true;
  });
}

int prbf_matvec_dev(prbf_ctx* ctx, const double* xin, double* yout, int flags) {
  return ctx_call(ctx, [&](Ctx& c) {
    if (!c.mv_ready) throw Error(PRBF_ERR_STATE, "prbf_matvec_setup has not been called");
    if (!xin || !yout) throw Error(PRBF_ERR_ARG, "null vector");
    int n = c.mv_pts.n;
    bool fp32 = (flags & PRBF_MATVEC_FP32) != 0;
    PointsView v = c.mv_pts.view();
    if (flags & PRBF_ORDER_CELL) {
      PRBF_CUDA(cudaMemcpyAsync(c.vin.get(), xin, sizeof(double) * n, cudaMemcpyDeviceToDevice, c.stream));
      gauss_sum_dev(c.mv_plan, v, v, c.vin.get(), yout, fp32, c.err.get(), c.stream);
    } else {
      gather_dev(n, c.mv_pts.perm.get(), xin, c.vin.get(), c.stream);
      gauss_sum_dev(c.mv_plan, v, v, c.vin.get(), c.vout.get(), fp32, c.err.get(), c.stream);
      scatter_dev(n, c.mv_pts.perm.get(), c.vout.get(), yout, c.stream);
    }
    PRBF_CHECK_LAUNCH();
  });
}

int prbf_matvec(prbf_ctx* ctx, const double* xin, double* yout) {
  return ctx_call(ctx, [&](Ctx& c) {
    if (!c.mv_ready) throw Error(PRBF_ERR_STATE, "prbf_matvec_setup has not been called");
    if (!xin || !yout) throw Error(PRBF_ERR_ARG, "null vector");
    int n = c.mv_pts.n;
    PointsView v = c.mv_pts.view();
    PRBF_CUDA(cudaMemcpyAsync(c.vtmp.get(), xin, sizeof(double) * n, cudaMemcpyHostToDevice, c.stream));
    gather_dev(n, c.mv_pts.perm.get(), c.vtmp.get(), c.vin.get(), c.stream);
    gauss_sum_dev(c.mv_plan, v, v, c.vin.get(), c.vout.get(), false, c.err.get(), c.stream);
    scatter_dev(n, c.mv_pts.perm.get(), c.vout.get(), c.vtmp.get(), c.stream);
    PRBF_CUDA(cudaMemcpyAsync(yout, c.vtmp.get(), sizeof(double) * n, cudaMemcpyDeviceToHost, c.stream));
    c.check_device_error("matvec");
  });
}

int prbf_matvec_kernels(prbf_ctx* ctx, int fp32, int* kernels, int* symmetric) {
  return ctx_call(ctx, [&](Ctx& c) {
    if (!c.mv_ready) throw Error(PRBF_ERR_STATE, "prbf_matvec_setup has not been called");
    const bool sym = !fp32 && c.mv_plan.sym_ready;
    if (kernels) *kernels = fp32 ? (c.mv_plan.f32_ready ? 2 : 1) : (sym ? 2 : 1);
    if (symmetric) *symmetric = sym ? 1 : 0;
  });
}

int prbf_matvec_info(prbf_ctx* ctx, int* ints7, double* dbls4, long long* pairs) {
  return ctx_call(ctx, [&](Ctx& c) {
    if (!c.mv_ready) throw Error(PRBF_ERR_STATE, "prbf_matvec_setup has not been called");
    const Grid& g = c.mv_pts.g;
    if (ints7) {
      int v[7] = {g.nx, g.ny, g.nz, g.ncell, g.nb_trunc, g.nb_buffer, c.mv_plan.max_trunc};
      std::memcpy(ints7, v, sizeof(v));
    }
    if (dbls4) {
      double d[4] = {g.xmin, g.ymin, g.zmin, g.box};
      std::memcpy(dbls4, d, sizeof(d));
    }
    if (pairs) *pairs = c.mv_plan.pairs;
  });
}

int prbf_get_permutation(prbf_ctx* ctx, int* perm) {
  return ctx_call(ctx, [&](Ctx& c) {
    if (!c.mv_ready) throw Error(PRBF_ERR_STATE, "prbf_matvec_setup has not been called");
    if (!perm) throw Error(PRBF_ERR_ARG, "null output");
    PRBF_CUDA(cudaMemcpyAsync(perm, c.mv_pts.perm.get(), sizeof(int) * c.mv_pts.n, cudaMemcpyDeviceToHost, c.stream));
    PRBF_CUDA(cudaStreamSynchronize(c.stream));
  });
}

int prbf_get_cell_start(prbf_ctx* ctx, int* cs) {
  return ctx_call(ctx, [&](Ctx& c) {
    if (!c.mv_ready) throw Error(PRBF_ERR_STATE, "prbf_matvec_setup has not been called");
    if (!cs) throw Error(PRBF_ERR_ARG, "null output");
    PRBF_CUDA(cudaMemcpyAsync(cs, c.mv_pts.cs.get(), sizeof(int) * ((size_t)c.mv_pts.g.ncell + 1),
                              cudaMemcpyDeviceToHost, c.stream));
    PRBF_CUDA(cudaStreamSynchronize(c.stream));
  });
}

int prbf_get_trunc_counts(prbf_ctx* ctx, int* counts) {
  return ctx_call(ctx, [&](Ctx& c) {
    if (!c.mv_ready) throw Error(PRBF_ERR_STATE, "prbf_matvec_setup has not been called");
    if (!counts) throw Error(PRBF_ERR_ARG, "null output");
    PRBF_CUDA(cudaMemcpyAsync(counts, c.mv_plan.trunc_cnt.get(), sizeof(int) * c.mv_pts.g.ncell,
                              cudaMemcpyDeviceToHost, c.stream));
    PRBF_CUDA(cudaStreamSynchronize(c.stream));
  });
}

int prbf_evaluate(prbf_ctx* ctx, int nt, const double* xt, const double* yt, const double* zt, int ns,
                  const double* xs, const double* ys, const double* zs, const double* gs, double* w_out) {
  return ctx_call(ctx, [&](Ctx& c) {
    check_n(nt);
    check_n(ns);
    if (!gs || !w_out) throw Error(PRBF_ERR_ARG, "null array");
    const int dim = c.p.dim;
    DevBuf<double> tx, ty, tz, sx, sy, sz, sg, sgs, w;
    upload_coords(c, nt, xt, yt, zt, tx, ty, tz);
    upload_coords(c, ns, xs, ys, zs, sx, sy, sz);
    c.upload(sg, gs, ns);
    // one grid over the union bounding box (2d/vorticity_evaluation.cxx:59-70)
    double bt[6], bs[6], b[6];
    bbox_host(c, nt, tx.get(), ty.get(), dim == 3 ? tz.get() : nullptr, bt);
    bbox_host(c, ns, sx.get(), sy.get(), dim == 3 ? sz.get() : nullptr, bs);
    for (int k = 0; k < 6; k++) b[k] = (k & 1) ? std::max(bt[k], bs[k]) : std::min(bt[k], bs[k]);
    Grid g = make_grid(dim, b, c.p.sigma, c.p.nsigma_box, c.p.sigma_buffer, c.p.sigma_trunc);
    PointSet T, S;
    build_points(c, T, g, nt, tx.get(), ty.get(), dim == 3 ? tz.get() : nullptr);
    build_points(c, S, g, ns, sx.get(), sy.get(), dim == 3 ? sz.get() : nullptr);
    sgs.reserve((size_t)ns + 4);
    PRBF_CUDA(cudaMemsetAsync(sgs.get() + ns, 0, sizeof(double) * 4, c.stream));
    gather_dev(ns, S.perm.get(), sg.get(), sgs.get(), c.stream);
    GaussPlan plan;
    plan.g = g;
    gauss_plan_dev(plan, T.view(), S.view(), c.err.get(), c.ws, c.stream);
    w.reserve((size_t)nt + 4);
    PRBF_CUDA(cudaMemsetAsync(w.get(), 0, sizeof(double) * nt, c.stream));
    gauss_sum_dev(plan, T.view(), S.view(), sgs.get(), w.get(), false, c.err.get(), c.stream);
    scatter_dev(nt, T.perm.get(), w.get(), tx.get(), c.stream);
    PRBF_CUDA(cudaMemcpyAsync(w_out, tx.get(), sizeof(double) * nt, cudaMemcpyDeviceToHost, c.stream));
    c.check_device_error("evaluate");
  });
}

}  // extern "C"
