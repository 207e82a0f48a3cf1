// batch.cu -- many independent interpolation problems solved together on one GPU: the
// replica form of rbf_interpolation (2d/rbf_interpolation.cxx:25-310) for a batch of
// point sets of uneven size, each with its own sigma and box widths.
//
// Layout: the problems' cell-sorted points are concatenated into one set of SoA arrays,
// their grids into one cell index space (Grid::cbase = the problem's first global cell),
// so that one operator covers the whole batch and is block diagonal over the problems:
//   * the Gaussian sum is one launch over the items (cell, tile of targets) of every
//     problem, ordered by decreasing cost and run by a persistent grid whose tile size and
//     CTA count an autotuner picks by timing candidates on a sample of the items;
//   * the Schwarz blocks of all problems are factorised in the same batches (largest
//     first, each block with its problem's sigma) and applied in one launch;
//   * GMRES runs one Krylov segment per problem, in lockstep, each with its own basis,
//     Hessenberg matrix and stopping test (the same iterates as a solve of its own).
// Mixed form: the sums and block factors are FP32 and GMRES solves the correction
// equation of an FP64 iterative refinement run per problem (the single-problem mixed
// form of solve.cu over all problems at once); a problem whose FP64 residual has met the
// tolerance drops out of the FP64 residual sums as well. Refinement contracts by about
// cond(A) u_fp32 per step, so a problem too ill-conditioned for FP32 -- one with a block
// whose FP32 Cholesky met a non-positive pivot (cond(A) >= cond(block) ~ 1/u_fp32), or
// whose refinement step did not halve its FP64 residual -- is solved again, with the
// others of its kind, as an FP64 batch.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <vector>

#include "krylov.h"
#include "rasm.h"
#include "trace.h"

namespace prbf {

namespace {

double now_ms() {
  using namespace std::chrono;
  return duration<double, std::milli>(steady_clock::now().time_since_epoch()).count();
}

__global__ void k_add_copy_int(long long n, const int* __restrict__ in, int add, int* __restrict__ out) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    out[i] = in[i] + add;
}

__global__ void k_add_inplace_int(long long n, int add, int* __restrict__ v) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    v[i] += add;
}

__global__ void k_fill_cells(int n, int prob, double sigma, int* __restrict__ cprob, double* __restrict__ csig) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) {
    cprob[i] = prob;
    csig[i] = sigma;
  }
}

int blocks_for(long long n) { return (int)std::max<long long>(1, std::min<long long>((n + 255) / 256, 4 * 152)); }

// A and B of the whole batch (one vector; the problems are its segments)
struct BatchOp : Operator {
  const GaussPlan* plan = nullptr;
  PointsView v{};
  const RasmPlan* rasm = nullptr;
  unsigned* err = nullptr;
  bool fp32 = false;
  void apply_A(const double* x, double* y, const int* skip, cudaStream_t s) const override {
    gauss_sum_dev(*plan, v, v, x, y, fp32, err, s, skip);
  }
  void apply_B(const double* r, double* z, const int* skip, cudaStream_t s) const override {
    rasm_apply(*rasm, v.cell_start, r, z, s, skip);
  }
};

// A pair of timing events, destroyed on every path out (errors throw).
struct EventPair {
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  EventPair() {
    PRBF_CUDA(cudaEventCreate(&e0));
    PRBF_CUDA(cudaEventCreate(&e1));
  }
  ~EventPair() {
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
  }
  EventPair(const EventPair&) = delete;
  EventPair& operator=(const EventPair&) = delete;
  float ms() const {
    PRBF_CUDA(cudaEventSynchronize(e1));
    float t = 0;
    PRBF_CUDA(cudaEventElapsedTime(&t, e0, e1));
    return t;
  }
};

struct Schedule {
  int tile = 128;
  int grid = 0;  // CTAs (0: one per item)
  double ms = 0;
};

}  // namespace

struct BatchState {
  int nprob = 0, dim = 2;
  std::vector<int> n, ncell;
  std::vector<long long> poff;
  std::vector<int> coff;
  long long npts = 0;
  int ncell_tot = 0;
  DevBuf<double> x, y, z, csig;
  DevBuf<int> cs, perm, cprob, trunc;
  std::vector<int> hcs, htrunc;
  GaussPlan plan;
  RasmPlan rasm;
  Krylov kry;
  BatchOp op, op32;
  DevBuf<double> b, sol, r, tmp, d;
  DevBuf<int> odone;  // mixed form: per problem, its FP64 residual met the tolerance
};

namespace {
// Schedules picked by the autotuner, per device and batch shape (precision, dimension,
// problems, points), kept for the life of the process.
std::map<std::pair<int, long long>, Schedule>& schedule_cache() {
  static std::map<std::pair<int, long long>, Schedule> m;
  return m;
}
std::mutex& schedule_mutex() {  // contexts on several host threads share the cache
  static std::mutex m;
  return m;
}
}  // namespace

void batch_state_free(BatchState* b) { delete b; }

namespace {

// Items (global cell, first target) for a tile size, by decreasing cost (targets x
// truncation-set size); stable, so equal costs keep the cell order.
std::vector<int2> make_items(const BatchState& B, int tile, long long* pairs) {
  struct It {
    long long cost;
    int2 v;
  };
  std::vector<It> v;
  long long p = 0;
  for (int c = 0; c < B.ncell_tot; c++) {
    int a = B.hcs[c], e = B.hcs[c + 1];
    for (int t = a; t < e; t += tile) {
      long long nt = std::min(tile, e - t);
      v.push_back({nt * (long long)B.htrunc[c], make_int2(c, t)});
      p += nt * (long long)B.htrunc[c];
    }
  }
  std::stable_sort(v.begin(), v.end(), [](const It& a, const It& b) { return a.cost > b.cost; });
  std::vector<int2> out(v.size());
  for (size_t i = 0; i < v.size(); i++) out[i] = v[i].v;
  if (pairs) *pairs = p;
  return out;
}

void upload_items(GaussPlan& P, const std::vector<int2>& items, cudaStream_t s) {
  P.nitems = (int)items.size();
  P.items.reserve(std::max<size_t>(items.size(), 1));
  PRBF_CUDA(cudaMemcpyAsync(P.items.get(), items.data(), sizeof(int2) * items.size(), cudaMemcpyHostToDevice, s));
  PRBF_CUDA(cudaStreamSynchronize(s));
}

// Times the batched sum (FP64, or FP32 for the mixed form, whose iterations are FP32) for
// (tile, grid) candidates on a strided sample of the items (an eighth, keeping the cost
// distribution) and keeps the fastest.
Schedule autotune(Ctx& c, BatchState& B, const double* vin, double* vout, bool fp32) {
  const int tiles[3] = {32, 64, 128};
  const int grids[3] = {0, 152 * 3, 152 * 6};
  Schedule best;
  best.ms = 1e300;
  EventPair ev;
  for (int tile : tiles) {
    std::vector<int2> all = make_items(B, tile, nullptr), sample;
    for (size_t i = 0; i < all.size(); i += 8) sample.push_back(all[i]);
    upload_items(B.plan, sample, c.stream);
    for (int grid : grids) {
      B.plan.grid = grid;
      gauss_sum_dev(B.plan, B.op.v, B.op.v, vin, vout, fp32, c.err.get(), c.stream);  // warm-up
      PRBF_CUDA(cudaEventRecord(ev.e0, c.stream));
      for (int k = 0; k < 2; k++) gauss_sum_dev(B.plan, B.op.v, B.op.v, vin, vout, fp32, c.err.get(), c.stream);
      PRBF_CUDA(cudaEventRecord(ev.e1, c.stream));
      const float ms = ev.ms();
      if (ms < best.ms) {
        best.ms = ms;
        best.tile = tile;
        best.grid = grid;
      }
    }
  }
  c.check_device_error("autotune");
  return best;
}

void batch_interpolate(Ctx& c, int nprob, const prbf_problem* probs, int* its_out, int* reason_out,
                       prbf_batch_stats* bs) {
  const double t_begin = now_ms();
  TraceRange tr_cluster("batch InitCluster");
  const prbf_params& p = c.p;
  const int dim = p.dim;
  if (nprob <= 0 || !probs) throw Error(PRBF_ERR_ARG, "empty batch");
  if (p.precision != PRBF_PREC_FP64 && p.precision != PRBF_PREC_MIXED) throw Error(PRBF_ERR_ARG, "bad precision");
  const bool mixed = p.precision == PRBF_PREC_MIXED;
  if (p.guess != PRBF_GUESS_ZERO) throw Error(PRBF_ERR_ARG, "batches start from a zero guess");
  for (int i = 0; i < nprob; i++) {
    const prbf_problem& q = probs[i];
    if (q.n <= 0 || !q.x || !q.y || (dim == 3 && !q.z) || !q.f || !q.g_out) throw Error(PRBF_ERR_ARG, "bad problem");
    if (!(q.sigma > 0)) throw Error(PRBF_ERR_ARG, "sigma must be > 0");
  }
  if (!c.batch) c.batch = new BatchState();
  BatchState& B = *c.batch;
  // the symmetric form's buffers describe the previous call's points (an outer batch whose
  // ill-conditioned problems are solved by this call reuses the state): off until rebuilt
  // for these points, after the autotuner
  B.plan.sym_ready = false;
  B.plan.sym_nitems = 0;
  B.nprob = nprob;
  B.dim = dim;
  B.n.assign(nprob, 0);
  B.ncell.assign(nprob, 0);
  B.poff.assign(nprob + 1, 0);
  B.coff.assign(nprob + 1, 0);

  // ---- pass 1: per problem cell sort, truncation sizes, buffer counts ------------------
  std::vector<std::unique_ptr<PointSet>> loc(nprob);
  std::vector<int> hcnt_all;
  DevBuf<double> ux, uy, uz;
  long long pairs = 0;
  for (int i = 0; i < nprob; i++) {
    const prbf_problem& q = probs[i];
    c.upload(ux, q.x, q.n);
    c.upload(uy, q.y, q.n);
    if (dim == 3) c.upload(uz, q.z, q.n);
    double bb[6];
    bbox_host(c, q.n, ux.get(), uy.get(), dim == 3 ? uz.get() : nullptr, bb);
    Grid g = make_grid(dim, bb, q.sigma, q.nsigma_box, q.sigma_buffer, q.sigma_trunc);
    loc[i].reset(new PointSet());
    build_points(c, *loc[i], g, q.n, ux.get(), uy.get(), dim == 3 ? uz.get() : nullptr);
    B.n[i] = q.n;
    B.ncell[i] = g.ncell;
    B.poff[i + 1] = B.poff[i] + q.n;
    B.coff[i + 1] = B.coff[i] + g.ncell;
    if (B.coff[i + 1] > 0x3fffffff || B.poff[i + 1] > 0x3fffffff) throw Error(PRBF_ERR_CAPACITY, "batch too large");
  }
  B.npts = B.poff[nprob];
  B.ncell_tot = B.coff[nprob];
  const int N = (int)B.npts, NC = B.ncell_tot;
  for (auto* v : {&B.x, &B.y, &B.z}) v->reserve((size_t)N + 4);
  B.csig.reserve(NC);
  B.cs.reserve((size_t)NC + 1);
  B.perm.reserve(N);
  B.cprob.reserve(NC);
  B.trunc.reserve(NC);
  for (auto* v : {&B.x, &B.y, &B.z}) PRBF_CUDA(cudaMemsetAsync(v->get() + N, 0, sizeof(double) * 4, c.stream));
  std::vector<Grid> hgrids(nprob);
  hcnt_all.assign(NC, 0);
  for (int i = 0; i < nprob; i++) {
    PointSet& P = *loc[i];
    const long long po = B.poff[i];
    const int co = B.coff[i], nc = B.ncell[i], ni = B.n[i];
    PRBF_CUDA(cudaMemcpyAsync(B.x.get() + po, P.x.get(), sizeof(double) * ni, cudaMemcpyDeviceToDevice, c.stream));
    PRBF_CUDA(cudaMemcpyAsync(B.y.get() + po, P.y.get(), sizeof(double) * ni, cudaMemcpyDeviceToDevice, c.stream));
    if (dim == 3)
      PRBF_CUDA(cudaMemcpyAsync(B.z.get() + po, P.z.get(), sizeof(double) * ni, cudaMemcpyDeviceToDevice, c.stream));
    PRBF_CUDA(cudaMemcpyAsync(B.perm.get() + po, P.perm.get(), sizeof(int) * ni, cudaMemcpyDeviceToDevice, c.stream));
    k_add_copy_int<<<blocks_for(nc + 1), 256, 0, c.stream>>>(nc + 1, P.cs.get(), (int)po, B.cs.get() + co);
    k_fill_cells<<<(nc + 255) / 256, 256, 0, c.stream>>>(nc, i, probs[i].sigma, B.cprob.get() + co, B.csig.get() + co);
    PRBF_CHECK_LAUNCH();
    // truncation-set sizes (the per-problem plan) and buffer-list sizes
    GaussPlan lp;
    lp.g = P.g;
    gauss_plan_dev(lp, P.view(), P.view(), c.err.get(), c.ws, c.stream, false);
    PRBF_CUDA(cudaMemcpyAsync(B.trunc.get() + co, lp.trunc_cnt.get(), sizeof(int) * nc, cudaMemcpyDeviceToDevice,
                              c.stream));
    pairs += lp.pairs;
    int* cnt = (int*)c.ws.get(61, sizeof(int) * ((size_t)nc + 1));
    rasm_buffer_lists(P, cnt, nullptr, nullptr, c.stream);
    PRBF_CUDA(cudaMemcpyAsync(hcnt_all.data() + co, cnt, sizeof(int) * nc, cudaMemcpyDeviceToHost, c.stream));
    Grid g = P.g;
    g.cbase = co;
    hgrids[i] = g;
  }
  PRBF_CUDA(cudaStreamSynchronize(c.stream));
  c.check_device_error("batch set-up");
  B.hcs.resize((size_t)NC + 1);
  B.htrunc.resize(NC);
  PRBF_CUDA(cudaMemcpyAsync(B.hcs.data(), B.cs.get(), sizeof(int) * (NC + 1), cudaMemcpyDeviceToHost, c.stream));
  PRBF_CUDA(cudaMemcpyAsync(B.htrunc.data(), B.trunc.get(), sizeof(int) * NC, cudaMemcpyDeviceToHost, c.stream));
  PRBF_CUDA(cudaStreamSynchronize(c.stream));
  // the global cell starts close every problem at the next one's first point
  B.plan.g = hgrids[0];
  B.plan.g.cbase = 0;
  B.plan.batched = true;
  B.plan.pairs = pairs;
  B.plan.max_tile = 128;
  B.plan.grids.reserve(nprob);
  B.plan.cprob.reserve(NC);
  PRBF_CUDA(cudaMemcpyAsync(B.plan.grids.get(), hgrids.data(), sizeof(Grid) * nprob, cudaMemcpyHostToDevice, c.stream));
  PRBF_CUDA(cudaMemcpyAsync(B.plan.cprob.get(), B.cprob.get(), sizeof(int) * NC, cudaMemcpyDeviceToDevice, c.stream));
  B.plan.f32_ready = false;
  if (mixed)
    gauss_plan_f32_batch(B.plan, hgrids,
                         PointsView{N, B.x.get(), B.y.get(), dim == 3 ? B.z.get() : nullptr, B.cs.get()}, c.stream);

  // ---- pass 2: buffer lists into the global block arrays, then one batched factorisation
  std::vector<long long> hb((size_t)NC + 1);
  hb[0] = 0;
  for (int k = 0; k < NC; k++) hb[k + 1] = hb[k] + hcnt_all[k];
  B.rasm.boff.reserve((size_t)NC + 1);
  B.rasm.idx.reserve(std::max<long long>(hb[NC], 1));
  PRBF_CUDA(cudaMemcpyAsync(B.rasm.boff.get(), hb.data(), sizeof(long long) * (NC + 1), cudaMemcpyHostToDevice,
                            c.stream));
  for (int i = 0; i < nprob; i++) {
    const int co = B.coff[i];
    int* cnt = (int*)c.ws.get(61, sizeof(int) * ((size_t)B.ncell[i] + 1));
    rasm_buffer_lists(*loc[i], cnt, B.rasm.boff.get() + co, B.rasm.idx.get(), c.stream);
    long long a = hb[co], e = hb[co + B.ncell[i]];
    if (e > a) k_add_inplace_int<<<blocks_for(e - a), 256, 0, c.stream>>>(e - a, (int)B.poff[i], B.rasm.idx.get() + a);
    PRBF_CHECK_LAUNCH();
  }
  PRBF_CUDA(cudaStreamSynchronize(c.stream));
  loc.clear();
  const double t_sorted = now_ms();
  tr_cluster.end();
  TraceRange tr_mat("batch InitMat");
  BlockGeom G;
  G.dim = dim;
  G.n = N;
  G.ncell = NC;
  G.x = B.x.get();
  G.y = B.y.get();
  G.z = dim == 3 ? B.z.get() : nullptr;
  G.cs = B.cs.get();
  G.sigma = probs[0].sigma;
  G.cell_sigma = B.csig.get();
  size_t free_b = 0, total_b = 0;
  PRBF_CUDA(cudaMemGetInfo(&free_b, &total_b));
  B.rasm.lu_fallback = p.block_fallback == PRBF_FALLBACK_LU;
  rasm_factor(B.rasm, G, hcnt_all, B.hcs, mixed, c.ws, c.err.get(), c.stream, std::min(16.0e9, 0.25 * (double)free_b),
              true, p.pc_type == PRBF_PC_ASM);
  rasm_set_apply_smem(B.rasm);
  c.check_device_error("batch RASM set-up");
  const double t_setup = now_ms();
  tr_mat.end();

  // ---- operator, schedule, Krylov segments ---------------------------------------------
  B.op.plan = &B.plan;
  B.op.v = PointsView{N, B.x.get(), B.y.get(), dim == 3 ? B.z.get() : nullptr, B.cs.get()};
  B.op.rasm = &B.rasm;
  B.op.err = c.err.get();
  B.op.fp32 = false;
  B.op32 = B.op;
  B.op32.fp32 = true;
  const long long ldv = (long long)N + 64;
  for (auto* v : {&B.b, &B.sol, &B.r, &B.tmp, &B.d}) {
    v->reserve(ldv);
    PRBF_CUDA(cudaMemsetAsync(v->get(), 0, sizeof(double) * ldv, c.stream));
  }
  for (int i = 0; i < nprob; i++) {
    PRBF_CUDA(cudaMemcpyAsync(B.tmp.get(), probs[i].f, sizeof(double) * B.n[i], cudaMemcpyHostToDevice, c.stream));
    gather_dev(B.n[i], B.perm.get() + B.poff[i], B.tmp.get(), B.b.get() + B.poff[i], c.stream);
  }
  PRBF_CUDA(cudaMemsetAsync(B.tmp.get(), 0, sizeof(double) * ldv, c.stream));
  const std::pair<int, long long> key(c.device, ((long long)(mixed ? 1 : 0) << 62) ^ ((long long)dim << 60) ^
                                                    ((long long)nprob << 40) ^ (long long)N);
  Schedule sch;
  double t_tune = 0;
  bool cached = false;
  {
    std::lock_guard<std::mutex> lk(schedule_mutex());
    auto hit = schedule_cache().find(key);
    if (hit != schedule_cache().end()) {
      sch = hit->second;
      cached = true;
    }
  }
  if (!cached) {
    const double tt0 = now_ms();
    TraceRange tr_tune("batch autotune");
    sch = autotune(c, B, B.b.get(), B.tmp.get(), mixed);
    t_tune = now_ms() - tt0;
    std::lock_guard<std::mutex> lk(schedule_mutex());
    schedule_cache()[key] = sch;
  }
  long long pairs_check = 0;
  upload_items(B.plan, make_items(B, sch.tile, &pairs_check), c.stream);
  B.plan.grid = sch.grid;
  // FP64 sums in the symmetric form where it applies (each exponential for both rows of a
  // point pair; the autotuned schedule then serves the FP32 sums of the mixed form)
  gauss_plan_sym_batch(B.plan, hgrids, PointsView{N, B.x.get(), B.y.get(), dim == 3 ? B.z.get() : nullptr, B.cs.get()},
                       B.hcs, c.stream);
  // one timed Gaussian sum with the chosen schedule, per precision in use (rates reported)
  auto time_sum = [&](bool fp32) {
    EventPair ev;
    gauss_sum_dev(B.plan, B.op.v, B.op.v, B.b.get(), B.tmp.get(), fp32, c.err.get(), c.stream);
    PRBF_CUDA(cudaEventRecord(ev.e0, c.stream));
    gauss_sum_dev(B.plan, B.op.v, B.op.v, B.b.get(), B.tmp.get(), fp32, c.err.get(), c.stream);
    PRBF_CUDA(cudaEventRecord(ev.e1, c.stream));
    const float ms = ev.ms();
    PRBF_CUDA(cudaMemsetAsync(B.tmp.get(), 0, sizeof(double) * ldv, c.stream));
    return (double)ms;
  };
  const double t_mv = time_sum(false), t_mv32 = mixed ? time_sum(true) : 0.0;
  std::vector<long long> offs(B.poff.begin(), B.poff.end() - 1);
  if (!B.kry.same_layout(offs, B.n, p.restart)) B.kry.init(offs, B.n, ldv, p.restart, c.stream);
  B.kry.graph_op = nullptr;

  // ---- solve ----------------------------------------------------------------------------
  // stopped problems drop out of the Gaussian sum and the block solves (their stop flags
  // are the Krylov per-system states)
  static_assert(sizeof(KSeg) % sizeof(int) == 0, "KSeg stride");
  SegSkip seg;
  seg.cprob = B.cprob.get();
  seg.done = &B.kry.st.get()->done;
  seg.stride = (int)(sizeof(KSeg) / sizeof(int));
  B.plan.seg = seg;
  B.rasm.seg = seg;
  PRBF_CUDA(cudaStreamSynchronize(c.stream));
  const double ts0 = now_ms();
  TraceRange tr_solve("batch KSPSolve");
  std::vector<int> its(nprob, 0), reason(nprob, 0), outer(nprob, 0);
  std::vector<char> to64(nprob, 0);  // mixed form: problems handed to the FP64 batch
  std::vector<double> true_rel(nprob, 0.0);
  bool resid_current = false;
  if (!mixed) {
    std::vector<KResult> kr =
        B.kry.solve(B.op, B.b.get(), B.sol.get(), true, p.rtol, p.abstol, p.dtol, p.max_it, true, c.stream);
    for (int i = 0; i < nprob; i++) {
      its[i] = kr[i].its;
      reason[i] = kr[i].reason;
    }
  } else {
    // FP64 iterative refinement of every problem: r = f - A g (FP64 sums, skipping the
    // problems that have stopped), stop test on ||r|| <= rtol ||f||, then A d = r by GMRES
    // with FP32 operators to kInnerRtol and g += d in FP64.
    B.odone.reserve(nprob);
    PRBF_CUDA(cudaMemsetAsync(B.odone.get(), 0, sizeof(int) * nprob, c.stream));
    SegSkip oseg;
    oseg.cprob = B.cprob.get();
    oseg.done = B.odone.get();
    oseg.stride = 1;
    std::vector<double> bnorm = seg_norm2_host(B.kry, B.b.get(), c.stream);
    for (auto& q : bnorm) q = std::sqrt(q);
    std::vector<double> rnorm(nprob, 0.0), prev(nprob, 0.0);
    std::vector<int> hdone(nprob, 0);
    // problems with a block that needed a shifted FP32 factorisation go to FP64 at once
    for (int cell : B.rasm.retried) {
      int i = (int)(std::upper_bound(B.coff.begin(), B.coff.end(), cell) - B.coff.begin()) - 1;
      if (i >= 0 && i < nprob) to64[i] = 1;
    }
    bool xzero = true;
    int inner_max = 0;
    for (int it = 0; it < 50; it++) {
      if (xzero) {
        PRBF_CUDA(cudaMemcpyAsync(B.r.get(), B.b.get(), sizeof(double) * N, cudaMemcpyDeviceToDevice, c.stream));
      } else {
        B.plan.seg = oseg;
        B.op.apply_A(B.sol.get(), B.tmp.get(), nullptr, c.stream);
        B.plan.seg = seg;  // the correction solve skips on the Krylov stop flags
        PRBF_CUDA(cudaMemcpyAsync(B.r.get(), B.b.get(), sizeof(double) * N, cudaMemcpyDeviceToDevice, c.stream));
        axpy_dev(N, -1.0, B.tmp.get(), B.r.get(), c.stream);
      }
      std::vector<double> rn = seg_norm2_host(B.kry, B.r.get(), c.stream);
      bool all = true, newly = false;
      for (int i = 0; i < nprob; i++) {
        if (!reason[i] && !to64[i]) {
          const double q = std::sqrt(rn[i]);
          rnorm[i] = q;
          if (!(q == q) || std::isinf(q)) {
            to64[i] = 1;
          } else if (q <= p.rtol * bnorm[i] || q <= p.abstol) {
            reason[i] = q <= p.abstol ? 3 : 2;
          } else if (it > 0 && !(q <= 0.5 * prev[i])) {
            to64[i] = 1;
          } else if (inner_max >= p.max_it) {
            reason[i] = -3;
          } else {
            outer[i]++;
            prev[i] = q;
            all = false;
            continue;
          }
        }
        // stopped: out of the correction solve (a zero residual stops at once) and out of
        // the next FP64 residual sums
        PRBF_CUDA(cudaMemsetAsync(B.r.get() + B.poff[i], 0, sizeof(double) * B.n[i], c.stream));
        if (!hdone[i]) {
          hdone[i] = 1;
          newly = true;
        }
      }
      if (newly)
        PRBF_CUDA(cudaMemcpyAsync(B.odone.get(), hdone.data(), sizeof(int) * nprob, cudaMemcpyHostToDevice, c.stream));
      if (all) {
        resid_current = true;
        for (int i = 0; i < nprob; i++) true_rel[i] = bnorm[i] > 0 ? rnorm[i] / bnorm[i] : rnorm[i];
        break;
      }
      PRBF_CUDA(cudaMemsetAsync(B.d.get(), 0, sizeof(double) * ldv, c.stream));
      const int budget_its = std::min(p.max_it - inner_max, 4 * p.restart);
      std::vector<KResult> in =
          B.kry.solve(B.op32, B.r.get(), B.d.get(), true, kInnerRtol, 0.0, 1e10, budget_its, true, c.stream);
      int step = 0;
      bool progress = false;
      for (int i = 0; i < nprob; i++) {
        if (reason[i] || to64[i]) continue;
        its[i] += in[i].its;
        step = std::max(step, in[i].its);
        progress = progress || in[i].its > 0;
      }
      inner_max += step;
      axpy_dev(N, 1.0, B.d.get(), B.sol.get(), c.stream);
      xzero = false;
      if (!progress) {
        for (int i = 0; i < nprob; i++)
          if (!reason[i]) to64[i] = 1;
        break;
      }
    }
    for (int i = 0; i < nprob; i++)
      if (!reason[i] && !to64[i]) reason[i] = -3;
  }
  PRBF_CUDA(cudaStreamSynchronize(c.stream));
  const double t_solve = now_ms() - ts0;
  tr_solve.end();
  B.plan.seg = SegSkip{};
  B.rasm.seg = SegSkip{};
  B.kry.reset_graph();  // the captured launches carry the stop flags
  c.check_device_error("batch solve");

  // ---- weights back in each caller's order; true residuals --------------------------------
  for (int i = 0; i < nprob; i++) {
    scatter_dev(B.n[i], B.perm.get() + B.poff[i], B.sol.get() + B.poff[i], B.tmp.get(), c.stream);
    PRBF_CUDA(cudaMemcpyAsync(probs[i].g_out, B.tmp.get(), sizeof(double) * B.n[i], cudaMemcpyDeviceToHost, c.stream));
    PRBF_CUDA(cudaStreamSynchronize(c.stream));
  }
  if (!resid_current) {
    B.op.apply_A(B.sol.get(), B.r.get(), nullptr, c.stream);
    PRBF_CUDA(cudaMemcpyAsync(B.tmp.get(), B.b.get(), sizeof(double) * N, cudaMemcpyDeviceToDevice, c.stream));
    axpy_dev(N, -1.0, B.r.get(), B.tmp.get(), c.stream);
    std::vector<double> rr = seg_norm2_host(B.kry, B.tmp.get(), c.stream),
                        bn = seg_norm2_host(B.kry, B.b.get(), c.stream);
    for (int i = 0; i < nprob; i++) {
      double q = std::sqrt(rr[i]), bq = std::sqrt(bn[i]);
      true_rel[i] = bq > 0 ? q / bq : q;
    }
  }
  prbf_batch_stats st{};
  st.nprob = nprob;
  st.points = N;
  st.pairs_per_matvec = pairs;
  st.ncell = NC;
  st.nblocks = B.rasm.nblocks;
  st.max_block = B.rasm.max_nb;
  st.min_block = 0;
  {
    int mn = 1 << 30;
    for (int v : hcnt_all)
      if (v > 0) mn = std::min(mn, v);
    st.min_block = mn == (1 << 30) ? 0 : mn;
  }
  st.nblocks_fallback = B.rasm.nfallback;
  st.tile = sch.tile;
  st.grid = sch.grid;
  // problems too ill-conditioned for FP32: one FP64 batch of their own (it reuses this
  // context's batch state, whose results have all been read back above)
  std::vector<int> sub_idx;
  for (int i = 0; i < nprob; i++)
    if (to64[i]) sub_idx.push_back(i);
  prbf_batch_stats sst{};
  if (!sub_idx.empty()) {
    std::vector<prbf_problem> sub;
    for (int i : sub_idx) sub.push_back(probs[i]);
    std::vector<int> sits(sub.size()), sreason(sub.size());
    struct Restore {
      prbf_params& p;
      int prec;
      ~Restore() { p.precision = prec; }
    } restore{c.p, c.p.precision};
    c.p.precision = PRBF_PREC_FP64;
    try {
      batch_interpolate(c, (int)sub.size(), sub.data(), sits.data(), sreason.data(), &sst);
    } catch (const Error& e) {
      // a problem of the FP64 batch stopped short of the tolerance: its iterations, reason
      // and the batch statistics are already written, and the status is raised below
      if (e.status != PRBF_ERR_NOT_CONVERGED && e.status != PRBF_ERR_BREAKDOWN && e.status != PRBF_ERR_NAN &&
          e.status != PRBF_ERR_DIVERGED)
        throw;
    }
    for (size_t k = 0; k < sub_idx.size(); k++) {
      its[sub_idx[k]] += sits[k];
      reason[sub_idx[k]] = sreason[k];
      true_rel[sub_idx[k]] = 0.0;
    }
    st.max_true_rel_resid = std::max(st.max_true_rel_resid, sst.max_true_rel_resid);
    st.nprob_fp64 = (int)sub_idx.size();
    st.nblocks_fallback += sst.nblocks_fallback;
  }
  int worst = 0;
  for (int i = 0; i < nprob; i++) {
    st.max_true_rel_resid = std::max(st.max_true_rel_resid, true_rel[i]);
    st.max_its = std::max(st.max_its, its[i]);
    st.outer_its = std::max(st.outer_its, outer[i]);
    st.total_its += its[i];
    st.nconverged += reason[i] > 0 ? 1 : 0;
    if (reason[i] < 0 && worst == 0) worst = reason[i];
    if (its_out) its_out[i] = its[i];
    if (reason_out) reason_out[i] = reason[i];
  }
  // (the FP64 batch of the mixed form's ill-conditioned problems counts in each phase)
  st.t_sort_ms = t_sorted - t_begin + sst.t_sort_ms;
  st.t_setup_ms = t_setup - t_sorted + sst.t_setup_ms;
  st.t_tune_ms = t_tune + sst.t_tune_ms;
  st.t_solve_ms = t_solve + sst.t_solve_ms;
  st.t_total_ms = now_ms() - t_begin;
  st.t_matvec_ms = t_mv;
  st.t_matvec32_ms = t_mv32;
  if (bs) *bs = st;
  if (worst == -3) throw Error(PRBF_ERR_NOT_CONVERGED, "a problem of the batch reached the iteration limit");
  if (worst == -5) throw Error(PRBF_ERR_BREAKDOWN, "GMRES breakdown in a problem of the batch");
  if (worst == -9) throw Error(PRBF_ERR_NAN, "NaN or Inf residual in a problem of the batch");
  if (worst == -4) throw Error(PRBF_ERR_DIVERGED, "a problem of the batch diverged");
}

}  // namespace
}  // namespace prbf

using namespace prbf;

extern "C" {

int prbf_batch_interpolate(prbf_ctx* ctx, int nprob, const prbf_problem* probs, int* its_out, int* reason_out,
                           prbf_batch_stats* stats) {
  return ctx_call(ctx, [&](Ctx& c) { batch_interpolate(c, nprob, probs, its_out, reason_out, stats); });
}

}  // extern "C"
