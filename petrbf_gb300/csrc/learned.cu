// learned.cu -- C ABI of the learned initial guess (include/petrbf_gb300_learned.h):
// network training, patch extraction, and the guess used by the solve.
#include <chrono>
#include <cmath>
#include <cstring>
#include <vector>

#include "../../include/petrbf_gb300_learned.h"
#include "mlp.h"

namespace prbf {
namespace {

__global__ void k_gather_rows(const int* __restrict__ idx, int nb, const float* __restrict__ src, float* __restrict__ dst,
                              int ncols) {
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < (long long)nb * ncols;
       e += (long long)gridDim.x * blockDim.x) {
    int r = (int)(e / ncols), k = (int)(e % ncols);
    dst[e] = src[(long long)idx[r] * ncols + k];
  }
}

uint64_t mix64(uint64_t& s) {
  uint64_t z = (s += 0x9E3779B97F4A7C15ull);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

Grid fine_grid(const double* b6, double sigma) { return make_grid(2, b6, sigma, MLP_NBOX, 0, 0); }

}  // namespace

// Guess for n points given on the device in any order (x, y, f); g written in that order.
void guess_compute(Ctx& c, Mlp& net, int n, const double* x, const double* y, const double* f, double* g) {
  double b[6];
  bbox_host(c, n, x, y, nullptr, b);
  PointSet P;
  build_points(c, P, fine_grid(b, c.p.sigma), n, x, y, nullptr);
  DevBuf<double> ff, gf;
  ff.reserve((size_t)n + 4);
  gf.reserve((size_t)n + 4);
  gather_dev(n, P.perm.get(), f, ff.get(), c.stream);
  DevBuf<int> cells;
  int nc = fine_cells(c, P, c.ws, cells);
  DevBuf<float> X, sc;
  X.reserve((size_t)nc * MLP_IN);
  sc.reserve(nc);
  patches_dev(c, P, ff.get(), nullptr, cells.get(), nc, X.get(), sc.get(), nullptr, nullptr);
  net.forward(X.get(), nc, c.stream);
  unpatch_dev(c, P, cells.get(), nc, net.out(), sc.get(), gf.get());
  scatter_dev(n, P.perm.get(), gf.get(), g, c.stream);
  net.check(c.stream);
}

}  // namespace prbf

using namespace prbf;

struct prbf_mlp {
  int device = 0;
  cudaStream_t stream = nullptr;
  Mlp net;
  DevBuf<float> X, T, M, Xb, Tb, Mb, loss;
  DevBuf<int> idx;
  ~prbf_mlp() {
    if (stream) {
      cudaStreamSynchronize(stream);
      cudaStreamDestroy(stream);
    }
  }
};

namespace {

template <class F>
int mlp_guard(prbf_mlp* m, F&& f) {
  if (!m) return PRBF_ERR_ARG;
  try {
    PRBF_CUDA(cudaSetDevice(m->device));
    f(*m);
    return PRBF_OK;
  } catch (const Error& e) {
    return e.status;
  } catch (const std::bad_alloc&) {
    return PRBF_ERR_CAPACITY;
  } catch (const std::exception&) {
    return PRBF_ERR_ARG;
  }
}

void upload_f(DevBuf<float>& d, const float* h, size_t n, cudaStream_t s) {
  d.reserve(std::max<size_t>(n, 1));
  PRBF_CUDA(cudaMemcpyAsync(d.get(), h, sizeof(float) * n, cudaMemcpyHostToDevice, s));
}

void upload_d(DevBuf<double>& d, const double* h, int n, cudaStream_t s) {
  d.reserve((size_t)n + 4);
  PRBF_CUDA(cudaMemcpyAsync(d.get(), h, sizeof(double) * n, cudaMemcpyHostToDevice, s));
  PRBF_CUDA(cudaMemsetAsync(d.get() + n, 0, sizeof(double) * 4, s));
}

}  // namespace

extern "C" {

long long prbf_mlp_param_count(void) { return (long long)mlp_param_count(); }

int prbf_mlp_create(int device, unsigned long long seed, prbf_mlp** out) {
  if (!out) return PRBF_ERR_ARG;
  *out = nullptr;
  prbf_mlp* m = new (std::nothrow) prbf_mlp();
  if (!m) return PRBF_ERR_CAPACITY;
  m->device = device;
  int st = mlp_guard(m, [&](prbf_mlp& q) {
    PRBF_CUDA(cudaStreamCreateWithFlags(&q.stream, cudaStreamNonBlocking));
    q.net.init(seed, q.stream);
    q.loss.reserve(4);
    PRBF_CUDA(cudaStreamSynchronize(q.stream));
  });
  if (st) {
    delete m;
    return st;
  }
  *out = m;
  return PRBF_OK;
}

int prbf_mlp_destroy(prbf_mlp* m) {
  if (!m) return PRBF_ERR_ARG;
  cudaSetDevice(m->device);
  delete m;
  return PRBF_OK;
}

int prbf_mlp_get_weights(prbf_mlp* m, float* w_out) {
  return mlp_guard(m, [&](prbf_mlp& q) {
    if (!w_out) throw Error(PRBF_ERR_ARG, "null output");
    PRBF_CUDA(cudaMemcpyAsync(w_out, q.net.w.get(), sizeof(float) * mlp_param_count(), cudaMemcpyDeviceToHost, q.stream));
    PRBF_CUDA(cudaStreamSynchronize(q.stream));
  });
}

int prbf_mlp_set_weights(prbf_mlp* m, const float* w) {
  return mlp_guard(m, [&](prbf_mlp& q) {
    if (!w) throw Error(PRBF_ERR_ARG, "null weights");
    q.net.set_weights(w, q.stream);
    PRBF_CUDA(cudaStreamSynchronize(q.stream));
  });
}

int prbf_mlp_forward(prbf_mlp* m, int n, const float* X, float* Y) {
  return mlp_guard(m, [&](prbf_mlp& q) {
    if (n <= 0 || !X || !Y) throw Error(PRBF_ERR_ARG, "bad arguments");
    upload_f(q.X, X, (size_t)n * MLP_IN, q.stream);
    q.net.forward(q.X.get(), n, q.stream);
    PRBF_CUDA(cudaMemcpyAsync(Y, q.net.out(), sizeof(float) * n * MLP_OUT, cudaMemcpyDeviceToHost, q.stream));
    q.net.check(q.stream);
  });
}

int prbf_mlp_loss_grad(prbf_mlp* m, int n, const float* X, const float* T, const float* M, float* loss,
                       float* grad_out) {
  return mlp_guard(m, [&](prbf_mlp& q) {
    if (n <= 0 || !X || !T || !M) throw Error(PRBF_ERR_ARG, "bad arguments");
    double cnt = 0;
    for (long long i = 0; i < (long long)n * MLP_OUT; i++) cnt += M[i];
    if (cnt <= 0) throw Error(PRBF_ERR_ARG, "empty mask");
    upload_f(q.X, X, (size_t)n * MLP_IN, q.stream);
    upload_f(q.T, T, (size_t)n * MLP_OUT, q.stream);
    upload_f(q.M, M, (size_t)n * MLP_OUT, q.stream);
    PRBF_CUDA(cudaMemsetAsync(q.loss.get(), 0, sizeof(float), q.stream));
    q.net.forward(q.X.get(), n, q.stream);
    q.net.backward(q.X.get(), q.T.get(), q.M.get(), n, (float)(1.0 / cnt), q.loss.get(), q.stream);
    if (loss) PRBF_CUDA(cudaMemcpyAsync(loss, q.loss.get(), sizeof(float), cudaMemcpyDeviceToHost, q.stream));
    if (grad_out)
      PRBF_CUDA(cudaMemcpyAsync(grad_out, q.net.grad.get(), sizeof(float) * mlp_param_count(), cudaMemcpyDeviceToHost,
                                q.stream));
    q.net.check(q.stream);
  });
}

int prbf_mlp_train(prbf_mlp* m, int n, const float* X, const float* T, const float* M, int epochs, int batch, float lr,
                   unsigned long long seed, float* loss_per_epoch) {
  return mlp_guard(m, [&](prbf_mlp& q) {
    if (n <= 0 || !X || !T || !M || epochs < 0 || batch <= 0) throw Error(PRBF_ERR_ARG, "bad arguments");
    cudaStream_t s = q.stream;
    upload_f(q.X, X, (size_t)n * MLP_IN, s);
    upload_f(q.T, T, (size_t)n * MLP_OUT, s);
    upload_f(q.M, M, (size_t)n * MLP_OUT, s);
    std::vector<double> rowcnt(n);
    for (int r = 0; r < n; r++) {
      double c = 0;
      for (int j = 0; j < MLP_OUT; j++) c += M[(size_t)r * MLP_OUT + j];
      rowcnt[r] = c;
    }
    q.Xb.reserve((size_t)batch * MLP_IN);
    q.Tb.reserve((size_t)batch * MLP_OUT);
    q.Mb.reserve((size_t)batch * MLP_OUT);
    q.idx.reserve(n);
    std::vector<int> perm(n);
    uint64_t rs = seed;
    for (int ep = 0; ep < epochs; ep++) {
      for (int i = 0; i < n; i++) perm[i] = i;
      for (int i = n - 1; i > 0; i--) std::swap(perm[i], perm[(int)(mix64(rs) % (uint64_t)(i + 1))]);
      PRBF_CUDA(cudaMemcpyAsync(q.idx.get(), perm.data(), sizeof(int) * n, cudaMemcpyHostToDevice, s));
      PRBF_CUDA(cudaMemsetAsync(q.loss.get(), 0, sizeof(float), s));
      int nbatch = 0;
      for (int b0 = 0; b0 < n; b0 += batch) {
        int nb = std::min(batch, n - b0);
        double cnt = 0;
        for (int r = b0; r < b0 + nb; r++) cnt += rowcnt[perm[r]];
        if (cnt <= 0) continue;
        const int* id = q.idx.get() + b0;
        k_gather_rows<<<256, 256, 0, s>>>(id, nb, q.X.get(), q.Xb.get(), MLP_IN);
        k_gather_rows<<<64, 256, 0, s>>>(id, nb, q.T.get(), q.Tb.get(), MLP_OUT);
        k_gather_rows<<<64, 256, 0, s>>>(id, nb, q.M.get(), q.Mb.get(), MLP_OUT);
        PRBF_CHECK_LAUNCH();
        q.net.forward(q.Xb.get(), nb, s);
        q.net.backward(q.Xb.get(), q.Tb.get(), q.Mb.get(), nb, (float)(1.0 / cnt), q.loss.get(), s);
        q.net.adam(lr, s);
        nbatch++;
      }
      float l = 0;
      PRBF_CUDA(cudaMemcpyAsync(&l, q.loss.get(), sizeof(float), cudaMemcpyDeviceToHost, s));
      q.net.check(s);
      if (loss_per_epoch) loss_per_epoch[ep] = nbatch ? l / nbatch : 0.f;
    }
  });
}

int prbf_guess_patches(prbf_ctx* ctx, int n, const double* x, const double* y, const double* f, const double* g,
                       float* X, float* scale, float* T, float* M, int* npatch) {
  return ctx_call(ctx, [&](Ctx& c) {
    if (c.p.dim != 2) throw Error(PRBF_ERR_ARG, "the learned guess is 2D");
    if (n <= 0 || !x || !y || !f || !npatch) throw Error(PRBF_ERR_ARG, "bad arguments");
    DevBuf<double> ux, uy, uf, ug, ff, gf;
    upload_d(ux, x, n, c.stream);
    upload_d(uy, y, n, c.stream);
    upload_d(uf, f, n, c.stream);
    double b[6];
    bbox_host(c, n, ux.get(), uy.get(), nullptr, b);
    PointSet P;
    build_points(c, P, fine_grid(b, c.p.sigma), n, ux.get(), uy.get(), nullptr);
    DevBuf<int> cells;
    int nc = fine_cells(c, P, c.ws, cells);
    *npatch = nc;
    if (!X) return;
    ff.reserve((size_t)n + 4);
    gather_dev(n, P.perm.get(), uf.get(), ff.get(), c.stream);
    DevBuf<float> dX, dS, dT, dM;
    dX.reserve((size_t)nc * MLP_IN);
    dS.reserve(nc);
    const bool tgt = g && T && M;
    if (tgt) {
      upload_d(ug, g, n, c.stream);
      gf.reserve((size_t)n + 4);
      gather_dev(n, P.perm.get(), ug.get(), gf.get(), c.stream);
      dT.reserve((size_t)nc * MLP_OUT);
      dM.reserve((size_t)nc * MLP_OUT);
    }
    patches_dev(c, P, ff.get(), tgt ? gf.get() : nullptr, cells.get(), nc, dX.get(), dS.get(), tgt ? dT.get() : nullptr,
                tgt ? dM.get() : nullptr);
    PRBF_CUDA(cudaMemcpyAsync(X, dX.get(), sizeof(float) * nc * MLP_IN, cudaMemcpyDeviceToHost, c.stream));
    if (scale) PRBF_CUDA(cudaMemcpyAsync(scale, dS.get(), sizeof(float) * nc, cudaMemcpyDeviceToHost, c.stream));
    if (tgt) {
      PRBF_CUDA(cudaMemcpyAsync(T, dT.get(), sizeof(float) * nc * MLP_OUT, cudaMemcpyDeviceToHost, c.stream));
      PRBF_CUDA(cudaMemcpyAsync(M, dM.get(), sizeof(float) * nc * MLP_OUT, cudaMemcpyDeviceToHost, c.stream));
    }
    PRBF_CUDA(cudaStreamSynchronize(c.stream));
  });
}

int prbf_guess_set_weights(prbf_ctx* ctx, const float* w) {
  return ctx_call(ctx, [&](Ctx& c) {
    if (!w) throw Error(PRBF_ERR_ARG, "null weights");
    if (!c.guess) c.guess = new Mlp();
    c.guess->set_weights(w, c.stream);
    PRBF_CUDA(cudaStreamSynchronize(c.stream));
  });
}

int prbf_guess_eval(prbf_ctx* ctx, int n, const double* x, const double* y, const double* f, double* g0) {
  return ctx_call(ctx, [&](Ctx& c) {
    if (c.p.dim != 2) throw Error(PRBF_ERR_ARG, "the learned guess is 2D");
    if (!c.guess || !c.guess->ready) throw Error(PRBF_ERR_STATE, "no learned-guess weights installed");
    if (n <= 0 || !x || !y || !f || !g0) throw Error(PRBF_ERR_ARG, "bad arguments");
    DevBuf<double> ux, uy, uf, ug;
    upload_d(ux, x, n, c.stream);
    upload_d(uy, y, n, c.stream);
    upload_d(uf, f, n, c.stream);
    ug.reserve((size_t)n + 4);
    guess_compute(c, *c.guess, n, ux.get(), uy.get(), uf.get(), ug.get());
    PRBF_CUDA(cudaMemcpyAsync(g0, ug.get(), sizeof(double) * n, cudaMemcpyDeviceToHost, c.stream));
    PRBF_CUDA(cudaStreamSynchronize(c.stream));
  });
}

}  // extern "C"
