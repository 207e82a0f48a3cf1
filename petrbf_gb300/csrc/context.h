// context.h -- the prbf_ctx behind the C ABI and the host-side helpers shared by the
// C-ABI translation units.
#pragma once
#include <exception>
#include <memory>
#include <new>
#include <string>

#include "device.h"

namespace prbf {

// A cell-sorted point set resident in HBM.
struct PointSet {
  int n = 0;
  Grid g{};
  DevBuf<double> x, y, z;  // sorted coordinates, n + 4 entries (padding for bulk copies)
  DevBuf<int> perm;        // sorted position -> caller index
  DevBuf<int> cs;          // cell start offsets, ncell + 1
  PointsView view() const { return PointsView{n, x.get(), y.get(), g.dim == 3 ? z.get() : nullptr, cs.get()}; }
};

// Grid from a bounding box, with the reference's arithmetic (host FP64, unfused):
// 2d/get_cluster.h:176-190, 3d/get_cluster.h:21-44, 2d/get_trunc.h:14, 2d/get_buffer.h:11.
Grid make_grid(int dim, const double* bbox6, double sigma, int nsigma_box, int sigma_buffer,
               int sigma_trunc);

struct SolveState;  // solve.cu
struct BatchState;  // batch.cu
void batch_state_free(BatchState* b);
struct Mlp;         // mlp.h (learned initial guess)

struct Ctx {
  prbf_params p{};
  int device = 0;
  cudaStream_t stream = nullptr;
  std::string last_error;
  Workspace ws;
  DevBuf<unsigned> err;  // device error word (DEV_ERR_* bits)
  // matvec seam (prbf_matvec_setup / prbf_matvec)
  PointSet mv_pts;
  GaussPlan mv_plan;
  bool mv_ready = false;
  DevBuf<double> vin, vout, vtmp;  // padded vectors of the matvec seam
  SolveState* solve = nullptr;  // owned; released by ~Ctx (solve.cu)
  Mlp* guess = nullptr;         // owned; learned-guess network (prbf_guess_set_weights)
  BatchState* batch = nullptr;  // owned; state of prbf_batch_interpolate
  ~Ctx();

  void check_device_error(const char* what);
  void upload(DevBuf<double>& dst, const double* src, int n, int pad = 4);
};

// Synchronises and destroys the context's stream (used by ~Ctx, defined in solve.cu).
void ctx_stream_release(Ctx& c);

// Builds a cell-sorted point set from device-resident caller-order coordinates.
void build_points(Ctx& c, PointSet& ps, const Grid& g, int n, const double* dx, const double* dy,
                  const double* dz);
// Device bounding box of one or two point sets, returned on the host (6 doubles).
void bbox_host(Ctx& c, int n, const double* dx, const double* dy, const double* dz, double* out6);

}  // namespace prbf

struct prbf_ctx {
  prbf::Ctx c;
};

namespace prbf {

// Body of a C-ABI entry point on a context: selects the context's device, runs f(ctx->c)
// and turns every exception into a status, with its message in last_error (no exception
// crosses the C ABI).
template <class F>
int ctx_call(prbf_ctx* ctx, F&& f) {
  if (!ctx) return PRBF_ERR_ARG;
  Ctx& c = ctx->c;
  try {
    c.last_error.clear();
    PRBF_CUDA(cudaSetDevice(c.device));
    f(c);
    return PRBF_OK;
  } catch (const Error& e) {
    c.last_error = e.what();
    return e.status;
  } catch (const std::bad_alloc&) {
    c.last_error = "host allocation failed";
    return PRBF_ERR_CAPACITY;
  } catch (const std::exception& e) {
    c.last_error = e.what();
    return PRBF_ERR_ARG;
  }
}

}  // namespace prbf
