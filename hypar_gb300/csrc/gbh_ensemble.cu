// gbh_ensemble.cu -- HyPar's ensemble mode (EnsembleSimulation, several
// independent simulations of possibly different grid sizes advanced together
// by one TimeRK, src/TimeIntegration/TimeInitialize.c:58-85 and TimeRK.c:126-195)
// as a batched solver.
//
// All members share the model, schemes, time step and Butcher table (as in the
// reference, where they share solver.inp); sizes, boundaries and initial data
// are per member.  Their arrays are concatenated; every Runge-Kutta stage is
// one launch per direction over all members (each thread finds its member in a
// table of thread offsets), and a whole step is captured once in a CUDA graph
// and replayed.  The launch form per direction -- segment walker (one thread per
// segment of a grid line) or tiles of 32/64/128 interfaces (one block per tile,
// set as a negative segment length) -- is chosen by timing.
#include <algorithm>
#include <cstring>
#include <vector>

#include "gbh_internal.h"

namespace gbh {
cudaError_t launch_batched_euler1d(int, int, int, const MemberDev*, int, long long, const double*, double*,
                                   const double*, const PhysParams&, const StageEpi&, int, int, unsigned long long*,
                                   cudaStream_t);
cudaError_t launch_batched_euler2d(int, int, int, const MemberDev*, int, long long, const double*, double*,
                                   const double*, const PhysParams&, const StageEpi&, int, int, unsigned long long*,
                                   cudaStream_t);
cudaError_t launch_batched_ns3d(int, int, int, const MemberDev*, int, long long, const double*, double*,
                                const double*, const PhysParams&, const StageEpi&, int, int, unsigned long long*,
                                cudaStream_t);
cudaError_t launch_pack(double*, const double*, const DevGeom&, int, int, cudaStream_t);
}  // namespace gbh

using namespace gbh;

#define CK(call)                                                                                      \
  do {                                                                                                \
    cudaError_t e_ = (call);                                                                          \
    if (e_ != cudaSuccess) {                                                                          \
      gbh_set_error("%s:%d: %s: %s", __FILE__, __LINE__, #call, cudaGetErrorString(e_));              \
      return GB_ERR_CUDA;                                                                             \
    }                                                                                                 \
  } while (0)

struct gb_ensemble {
  int nm = 0;
  std::vector<gb_config> cfg;
  gb_config base;
  PhysParams pp;
  int device = 0;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  std::vector<MemberDev> mem;
  std::vector<long long> nvals;  // values per member (with ghosts)
  // staging array for interior-layout host copies of one member (the largest
  // member's size; allocated on first use, kept)
  double* d_stage = nullptr;
  size_t stage_vals = 0;
  long long total_vals = 0, total_dx = 0;
  long long total_thr[3] = {0, 0, 0};
  int seg[3] = {32, 32, 32}, block[3] = {128, 128, 128};
  // tile forms only: the persistent work-list kernel (one counter per stage and
  // direction, cleared at the start of every step) instead of one block per tile
  bool persist[3] = {false, false, false};
  unsigned long long* d_ctr = nullptr;
  double* d_u = nullptr;
  double* d_acc = nullptr;
  double* d_P[4] = {nullptr, nullptr, nullptr, nullptr};
  double* d_H = nullptr;
  double* d_dx = nullptr;
  MemberDev* d_mem = nullptr;
  cudaGraphExec_t gexec = nullptr;
  // conservation check: boundary-flux accumulators of every member (MemberDev
  // bnd_off), the members' initial volume integrals, a reduction buffer
  double* d_bnd = nullptr;
  long long bnd_n = 0;
  bool cons_on = false;
  std::vector<double> V0;
  double* d_red = nullptr;
  bool graph_dirty = true;
  bool use_graph = true;
  double t = 0.0;
};

static void rebuild_table(gb_ensemble* e) {
  for (int d = 0; d < 3; d++) e->total_thr[d] = 0;
  for (int m = 0; m < e->nm; m++) {
    MemberDev& md = e->mem[m];
    for (int d = 0; d < 3; d++) {
      md.seg[d] = e->seg[d];
      if (d >= e->base.ndims) {
        md.ntrans[d] = 0;
        md.nseg[d] = 0;
        md.start[d] = e->total_thr[d];
        continue;
      }
      long long ntr = 1;
      for (int k = 0; k < e->base.ndims; k++)
        if (k != d) ntr *= md.G.dim[k];
      md.ntrans[d] = ntr;
      // walker: threads (segments x lines); tiles: blocks (tiles x lines)
      const int ti = -e->seg[d];
      md.nseg[d] = e->seg[d] > 0 ? (md.G.dim[d] + e->seg[d] - 1) / e->seg[d] : (md.G.dim[d] + ti - 2) / (ti - 1);
      md.start[d] = e->total_thr[d];
      e->total_thr[d] += ntr * md.nseg[d];
    }
  }
}

static int upload_table(gb_ensemble* e) {
  rebuild_table(e);
  CK(cudaMemcpyAsync(e->d_mem, e->mem.data(), sizeof(MemberDev) * e->nm, cudaMemcpyHostToDevice, e->stream));
  CK(cudaStreamSynchronize(e->stream));
  e->graph_dirty = true;
  return GB_OK;
}

static cudaError_t launch_dir(gb_ensemble* e, int st, int d, const double* U, const StageEpi& ep) {
  const gb_config& c = e->base;
  const int tile = e->seg[d] < 0 ? -e->seg[d] : 0;
  unsigned long long* ctr = (tile && e->persist[d]) ? e->d_ctr + 3 * st + d : nullptr;
  if (tile && !ctr && e->total_thr[d] > 0x7fffffffLL) return cudaErrorInvalidConfiguration;  // one block per tile
  if (c.model == GB_MODEL_EULER1D)
    return launch_batched_euler1d(d, c.interp, c.upwind, e->d_mem, e->nm, e->total_thr[d], U, e->d_H, e->d_dx,
                                  e->pp, ep, e->block[d], tile, ctr, e->stream);
  if (c.model == GB_MODEL_EULER2D)
    return launch_batched_euler2d(d, c.interp, c.upwind, e->d_mem, e->nm, e->total_thr[d], U, e->d_H, e->d_dx,
                                  e->pp, ep, e->block[d], tile, ctr, e->stream);
  return launch_batched_ns3d(d, c.interp, c.upwind, e->d_mem, e->nm, e->total_thr[d], U, e->d_H, e->d_dx, e->pp,
                             ep, e->block[d], tile, ctr, e->stream);
}

// The launches of one Runge-Kutta step (ns stages x ndims directions).
static int step_launches(gb_ensemble* e) {
  const gb_config& c = e->base;
  const int ns = c.rk_nstages;
  int touched[4] = {0, 0, 0, 0};
  if (e->persist[0] || e->persist[1] || e->persist[2])
    CK(cudaMemsetAsync(e->d_ctr, 0, sizeof(unsigned long long) * 12, e->stream));
  for (int st = 0; st < ns; st++) {
    double* U = (st == 0 || !touched[st]) ? e->d_u : e->d_P[st];
    StageEpi ep;
    memset(&ep, 0, sizeof(ep));
    ep.mode = EPI_RK;
    ep.stage = st;
    ep.nstages = ns;
    ep.cb = c.dt * c.rk_b[st];
    ep.need_u = (st == 0);
    for (int t = 0; t < 4; t++) {
      ep.touched[t] = touched[t];
      ep.P[t] = e->d_P[t];
      if (t > st && t < ns) {
        ep.ca[t] = c.dt * c.rk_A[4 * t + st];
        if (ep.ca[t] != 0.0 && !touched[t]) ep.need_u = 1;
      }
    }
    ep.u = e->d_u;
    ep.acc = e->d_acc;
    ep.uout = (ns == 1) ? e->d_acc : e->d_u;
    for (int d = 0; d < c.ndims; d++) {
      StageEpi x = ep;
      x.first = (d == 0);
      x.last = (d == c.ndims - 1);
      if (e->cons_on) {
        x.bnd = e->d_bnd;  // each member's block at its bnd_off
        x.bw = ep.cb;
      }
      CK(launch_dir(e, st, d, U, x));
    }
    for (int t = st + 1; t < ns; t++)
      if (ep.ca[t] != 0.0) touched[t] = 1;
  }
  return GB_OK;
}

extern "C" int gb_ensemble_create(const gb_config* cfgs, const double* const* dxinvs, int nsims, int device,
                                  gb_ensemble** out) {
  if (!cfgs || !dxinvs || !out || nsims < 1) {
    gbh_set_error("gb_ensemble_create: bad argument");
    return GB_ERR_ARG;
  }
  *out = nullptr;
  for (int m = 0; m < nsims; m++) {
    int rc = gbh_validate(&cfgs[m]);
    if (rc) return rc;
    if (cfgs[m].upwind == GB_UPWIND_SWFS) {
      gbh_set_error("ensemble member %d: Steger-Warming upwinding is not available in the ensemble; use a gb_solver", m);
      return GB_ERR_UNSUPPORTED;
    }
    for (int z = 0; z < cfgs[m].nzones; z++)
      if (cfgs[m].zones[z][0] == GB_BC_SPONGE) {
        gbh_set_error("ensemble member %d: sponge zones are not available in the ensemble; use a gb_solver", m);
        return GB_ERR_UNSUPPORTED;
      }
    const gb_config &a = cfgs[0], &b = cfgs[m];
    if (a.model != b.model || a.interp != b.interp || a.upwind != b.upwind || a.gamma != b.gamma ||
        a.weno_eps != b.weno_eps || a.rk_nstages != b.rk_nstages || a.dt != b.dt ||
        memcmp(a.rk_A, b.rk_A, sizeof(a.rk_A)) || memcmp(a.rk_b, b.rk_b, sizeof(a.rk_b))) {
      gbh_set_error("ensemble member %d differs from member 0 in model, schemes or time step", m);
      return GB_ERR_ARG;
    }
    if (b.model == GB_MODEL_NS3D && b.Re > 0) {
      gbh_set_error("viscous NavierStokes3D ensembles are not supported");
      return GB_ERR_UNSUPPORTED;
    }
    if (b.gravity[0] != 0.0 || b.gravity[1] != 0.0 || b.gravity[2] != 0.0) {
      gbh_set_error("ensembles with gravity are not supported");
      return GB_ERR_UNSUPPORTED;
    }
    if (b.hyp_scheme != GB_SCHEME_WENO5) {
      gbh_set_error("ensembles take WENO5 only (member %d asks for CRWENO5)", m);
      return GB_ERR_UNSUPPORTED;
    }
    if (b.weno_weights != GB_WENO_JS) {
      gbh_set_error("ensembles take Jiang-Shu WENO5 weights only (member %d asks for type %d)", m, b.weno_weights);
      return GB_ERR_UNSUPPORTED;
    }
  }
  gb_ensemble* e = new gb_ensemble();
  e->nm = nsims;
  e->cfg.assign(cfgs, cfgs + nsims);
  e->base = cfgs[0];
  if (device >= 0 && cudaSetDevice(device) != cudaSuccess) {
    gbh_set_error("cudaSetDevice(%d) failed", device);
    delete e;
    return GB_ERR_CUDA;
  }
  cudaGetDevice(&e->device);
  e->pp.gamma = e->base.gamma;
  e->pp.gm1 = e->base.gamma - 1.0;
  e->pp.inv_gm1 = 1.0 / (e->base.gamma - 1.0);
  e->pp.eps = e->base.weno_eps;
  e->pp.wtype = WENO_W_JS;
  e->pp.gf = e->pp.gg = nullptr;
  e->mem.resize(nsims);
  e->nvals.resize(nsims);
  long long off = 0, dxo = 0;
  for (int m = 0; m < nsims; m++) {
    MemberDev& md = e->mem[m];
    memset(&md, 0, sizeof(md));
    std::vector<int> memz;
    long long np = gbh_geometry(cfgs[m], md.G, &memz);
    if (!memz.empty()) {
      gbh_set_error("ensemble member %d: boundary zones must cover whole faces", m);
      delete e;
      return GB_ERR_UNSUPPORTED;
    }
    md.off = off;
    e->nvals[m] = np * cfgs[m].nvars;
    off += e->nvals[m];
    for (int d = 0; d < cfgs[m].ndims; d++) {
      md.dx_off[d] = dxo;
      dxo += cfgs[m].dim[d] + 2 * cfgs[m].ghosts;
    }
  }
  e->total_vals = off;
  e->total_dx = dxo;
  size_t bytes = (size_t)off * sizeof(double);
  cudaError_t ce = cudaSuccess;
  auto A = [&](double** p, size_t n) {
    if (ce == cudaSuccess) ce = cudaMalloc((void**)p, n);
    if (ce == cudaSuccess) ce = cudaMemset(*p, 0, n);
  };
  A(&e->d_u, bytes);
  A(&e->d_acc, bytes);
  for (int k = 1; k < e->base.rk_nstages; k++) A(&e->d_P[k], bytes);
  if (e->base.ndims > 1) A(&e->d_H, bytes);
  A(&e->d_dx, dxo * sizeof(double));
  if (ce == cudaSuccess) ce = cudaMalloc((void**)&e->d_mem, sizeof(MemberDev) * nsims);
  if (ce == cudaSuccess) ce = cudaMalloc((void**)&e->d_ctr, sizeof(unsigned long long) * 12);
  if (ce == cudaSuccess) ce = cudaStreamCreateWithFlags(&e->stream, cudaStreamNonBlocking);
  if (ce == cudaSuccess) e->own_stream = true;
  for (int m = 0; m < nsims && ce == cudaSuccess; m++) {
    long long n = 0;
    for (int d = 0; d < cfgs[m].ndims; d++) n += cfgs[m].dim[d] + 2 * cfgs[m].ghosts;
    ce = cudaMemcpy(e->d_dx + e->mem[m].dx_off[0], dxinvs[m], n * sizeof(double), cudaMemcpyHostToDevice);
  }
  if (ce != cudaSuccess) {
    gbh_set_error("gb_ensemble_create: %s", cudaGetErrorString(ce));
    gb_ensemble_destroy(e);
    return ce == cudaErrorMemoryAllocation ? GB_ERR_NOMEM : GB_ERR_CUDA;
  }
  e->use_graph = e->base.rk_nstages > 1;
  int rc = upload_table(e);
  if (rc) {
    gb_ensemble_destroy(e);
    return rc;
  }
  *out = e;
  return GB_OK;
}

extern "C" void gb_ensemble_destroy(gb_ensemble* e) {
  if (!e) return;
  if (e->gexec) cudaGraphExecDestroy(e->gexec);
  cudaFree(e->d_u);
  cudaFree(e->d_stage);
  cudaFree(e->d_acc);
  for (int k = 0; k < 4; k++) cudaFree(e->d_P[k]);
  cudaFree(e->d_H);
  cudaFree(e->d_dx);
  cudaFree(e->d_mem);
  cudaFree(e->d_ctr);
  cudaFree(e->d_bnd);
  cudaFree(e->d_red);
  if (e->own_stream && e->stream) cudaStreamDestroy(e->stream);
  delete e;
}

extern "C" int gb_ensemble_size(const gb_ensemble* e) { return e ? e->nm : 0; }

extern "C" int gb_ensemble_set_stream(gb_ensemble* e, void* stream) {
  if (!e) { gbh_set_error("null ensemble"); return GB_ERR_ARG; }
  if (e->own_stream && e->stream) {
    cudaStreamSynchronize(e->stream);
    cudaStreamDestroy(e->stream);
  }
  e->own_stream = false;
  if (stream) {
    e->stream = (cudaStream_t)stream;
  } else {
    CK(cudaStreamCreateWithFlags(&e->stream, cudaStreamNonBlocking));
    e->own_stream = true;
  }
  e->graph_dirty = true;
  return GB_OK;
}

extern "C" int gb_ensemble_sync(gb_ensemble* e) {
  if (!e) { gbh_set_error("null ensemble"); return GB_ERR_ARG; }
  CK(cudaStreamSynchronize(e->stream));
  return GB_OK;
}

// The kept staging array, grown to n values if needed.
static cudaError_t stage_array(gb_ensemble* e, size_t n) {
  if (e->d_stage && e->stage_vals >= n) return cudaSuccess;
  cudaError_t ce = cudaStreamSynchronize(e->stream);
  if (ce != cudaSuccess) return ce;
  cudaFree(e->d_stage);
  e->d_stage = nullptr;
  e->stage_vals = 0;
  ce = cudaMalloc((void**)&e->d_stage, n * sizeof(double));
  if (ce == cudaSuccess) e->stage_vals = n;
  return ce;
}

extern "C" int gb_ensemble_set_state(gb_ensemble* e, int m, const double* u, int layout, int mem) {
  if (!e || !u || m < 0 || m >= e->nm) { gbh_set_error("gb_ensemble_set_state: bad argument"); return GB_ERR_ARG; }
  const gb_config& c = e->cfg[m];
  double* dst = e->d_u + e->mem[m].off;
  size_t bytes = (size_t)e->nvals[m] * sizeof(double);
  if (layout == GB_LAYOUT_GHOSTED) {
    CK(cudaMemcpyAsync(dst, u, bytes, mem == GB_MEM_HOST ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToDevice,
                       e->stream));
  } else {
    size_t nint = c.nvars;
    for (int d = 0; d < c.ndims; d++) nint *= c.dim[d];
    const double* src = u;
    if (mem == GB_MEM_HOST) {
      CK(stage_array(e, nint));
      CK(cudaMemcpyAsync(e->d_stage, u, nint * sizeof(double), cudaMemcpyHostToDevice, e->stream));
      src = e->d_stage;
    }
    CK(launch_pack(dst, src, e->mem[m].G, c.nvars, 0, e->stream));
  }
  CK(cudaMemcpyAsync(e->d_acc + e->mem[m].off, dst, bytes, cudaMemcpyDeviceToDevice, e->stream));
  for (int k = 1; k < e->base.rk_nstages; k++)
    CK(cudaMemcpyAsync(e->d_P[k] + e->mem[m].off, dst, bytes, cudaMemcpyDeviceToDevice, e->stream));
  CK(cudaStreamSynchronize(e->stream));
  e->t = 0.0;
  return GB_OK;
}

extern "C" int gb_ensemble_get_state(gb_ensemble* e, int m, double* u, int layout, int mem) {
  if (!e || !u || m < 0 || m >= e->nm) { gbh_set_error("gb_ensemble_get_state: bad argument"); return GB_ERR_ARG; }
  const gb_config& c = e->cfg[m];
  const double* src = e->d_u + e->mem[m].off;
  if (layout == GB_LAYOUT_GHOSTED) {
    CK(cudaMemcpyAsync(u, src, (size_t)e->nvals[m] * sizeof(double),
                       mem == GB_MEM_HOST ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice, e->stream));
  } else {
    size_t nint = c.nvars;
    for (int d = 0; d < c.ndims; d++) nint *= c.dim[d];
    double* dst = u;
    if (mem == GB_MEM_HOST) {
      CK(stage_array(e, nint));
      dst = e->d_stage;
    }
    CK(launch_pack(dst, src, e->mem[m].G, c.nvars, 1, e->stream));
    if (mem == GB_MEM_HOST) CK(cudaMemcpyAsync(u, e->d_stage, nint * sizeof(double), cudaMemcpyDeviceToHost, e->stream));
  }
  CK(cudaStreamSynchronize(e->stream));
  return GB_OK;
}

extern "C" int gb_ensemble_step(gb_ensemble* e, int nsteps) {
  if (!e || nsteps < 0) { gbh_set_error("gb_ensemble_step: bad argument"); return GB_ERR_ARG; }
  if (!e->use_graph) {
    for (int n = 0; n < nsteps; n++) {
      int rc = step_launches(e);
      if (rc) return rc;
      double* tmp = e->d_u;  // one-stage scheme: the new solution was written to acc
      e->d_u = e->d_acc;
      e->d_acc = tmp;
      e->t += e->base.dt;
    }
    return GB_OK;
  }
  if (e->graph_dirty || !e->gexec) {
    if (e->gexec) {
      cudaGraphExecDestroy(e->gexec);
      e->gexec = nullptr;
    }
    cudaGraph_t g;
    CK(cudaStreamBeginCapture(e->stream, cudaStreamCaptureModeThreadLocal));
    int rc = step_launches(e);
    cudaError_t ce = cudaStreamEndCapture(e->stream, &g);
    if (rc) return rc;
    if (ce != cudaSuccess) { gbh_set_error("graph capture: %s", cudaGetErrorString(ce)); return GB_ERR_CUDA; }
    ce = cudaGraphInstantiate(&e->gexec, g, 0);
    cudaGraphDestroy(g);
    if (ce != cudaSuccess) { gbh_set_error("graph instantiate: %s", cudaGetErrorString(ce)); return GB_ERR_CUDA; }
    e->graph_dirty = false;
  }
  for (int n = 0; n < nsteps; n++) {
    CK(cudaGraphLaunch(e->gexec, e->stream));
    e->t += e->base.dt;
  }
  return GB_OK;
}

extern "C" int gb_ensemble_set_launch(gb_ensemble* e, int dir, int seg, int block) {
  if (!e || dir < 0 || dir >= e->base.ndims) { gbh_set_error("gb_ensemble_set_launch: bad argument"); return GB_ERR_ARG; }
  if (seg < 0 && seg != -32 && seg != -64 && seg != -128) {
    gbh_set_error("gb_ensemble_set_launch: a tile form is -32, -64 or -128 (got %d)", seg);
    return GB_ERR_ARG;
  }
  const int nseg = seg != 0 ? seg : e->seg[dir];
  if (block == -1 && nseg >= 0) {
    gbh_set_error("gb_ensemble_set_launch: the persistent work-list form (block -1) takes a tile form");
    return GB_ERR_ARG;
  }
  if (block < -1 || (block > 0 && (block % 32 || block > 128))) {
    gbh_set_error("gb_ensemble_set_launch: block %d (a multiple of 32 up to 128, or -1)", block);
    return GB_ERR_ARG;
  }
  e->seg[dir] = nseg;
  if (block == -1) e->persist[dir] = true;
  if (block > 0) {
    e->block[dir] = block;
    e->persist[dir] = false;
  }
  if (nseg >= 0) e->persist[dir] = false;
  return upload_table(e);
}

extern "C" int gb_ensemble_get_launch(gb_ensemble* e, int dir, int* seg, int* block) {
  if (!e || dir < 0 || dir >= e->base.ndims || !seg || !block) { gbh_set_error("bad argument"); return GB_ERR_ARG; }
  *seg = e->seg[dir];
  *block = e->persist[dir] ? -1 : e->block[dir];
  return GB_OK;
}

extern "C" double gb_ensemble_time(const gb_ensemble* e) { return e ? e->t : 0.0; }

// Segment length / block per direction by timing whole graph-replayed steps
// (directions tuned one after the other); the state is restored afterwards.
extern "C" int gb_ensemble_autotune(gb_ensemble* e, int reps) {
  if (!e) { gbh_set_error("null ensemble"); return GB_ERR_ARG; }
  if (reps < 1) reps = 1;
  size_t bytes = (size_t)e->total_vals * sizeof(double);
  double* save = nullptr;
  CK(cudaMallocAsync((void**)&save, bytes, e->stream));
  CK(cudaMemcpyAsync(save, e->d_u, bytes, cudaMemcpyDeviceToDevice, e->stream));
  double t0 = e->t;
  const bool cons_was = e->cons_on;  // the trial steps add no boundary fluxes
  e->cons_on = false;
  e->graph_dirty = true;
  cudaEvent_t a, b;
  CK(cudaEventCreate(&a));
  CK(cudaEventCreate(&b));
  int rc = GB_OK;
  const int cand[] = {8, 12, 16, 20, 24, 27, 32, 40, 48, 54, 64, -32, -64, -128};
  for (int d = 0; d < e->base.ndims && !rc; d++) {
    float best = 1e30f;
    int bs = e->seg[d], bb = e->block[d];
    bool bp = e->persist[d];
    for (int sg : cand) {
      for (int blk : {128, 64, -1}) {
        // a tile's block is its interfaces; -1: the tile's persistent work-list form
        if (sg < 0 && blk == 64) continue;
        if (sg > 0 && blk < 0) continue;
        e->seg[d] = sg;
        e->block[d] = blk > 0 ? blk : 128;
        e->persist[d] = blk < 0;
        rc = upload_table(e);
        if (!rc) rc = gb_ensemble_step(e, 1);
        if (rc) break;
        CK(cudaEventRecord(a, e->stream));
        rc = gb_ensemble_step(e, reps);
        CK(cudaEventRecord(b, e->stream));
        CK(cudaEventSynchronize(b));
        float ms = 0.f;
        cudaEventElapsedTime(&ms, a, b);
        if (!rc && ms < best) {
          best = ms;
          bs = sg;
          bb = e->block[d];
          bp = e->persist[d];
        }
      }
      if (rc) break;
    }
    e->seg[d] = bs;
    e->block[d] = bb;
    e->persist[d] = bp;
    if (!rc) rc = upload_table(e);
  }
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  CK(cudaMemcpyAsync(e->d_u, save, bytes, cudaMemcpyDeviceToDevice, e->stream));
  CK(cudaMemcpyAsync(e->d_acc, save, bytes, cudaMemcpyDeviceToDevice, e->stream));
  for (int k = 1; k < e->base.rk_nstages; k++)
    CK(cudaMemcpyAsync(e->d_P[k], save, bytes, cudaMemcpyDeviceToDevice, e->stream));
  CK(cudaFreeAsync(save, e->stream));
  CK(cudaStreamSynchronize(e->stream));
  e->t = t0;
  e->cons_on = cons_was;
  e->graph_dirty = true;
  return rc;
}

// CalculateError for one member against its exact solution (exact_<k>.inp).
extern "C" int gb_ensemble_error(gb_ensemble* e, int member, const double* uex, int layout, int mem, double* err) {
  if (!e || !uex || !err || member < 0 || member >= e->nm) {
    gbh_set_error("gb_ensemble_error: bad argument");
    return GB_ERR_ARG;
  }
  const MemberDev& md = e->mem[member];
  const gb_config& c = e->cfg[member];
  if (!e->d_red) CK(cudaMalloc((void**)&e->d_red, CONS_RED_DOUBLES * sizeof(double)));
  const size_t nval = (size_t)e->nvals[member];
  double* ex = nullptr;
  CK(cudaMallocAsync((void**)&ex, nval * sizeof(double), e->stream));
  double* tmp = nullptr;
  cudaError_t ce = cudaSuccess;
  if (layout == GB_LAYOUT_GHOSTED) {
    ce = cudaMemcpyAsync(ex, uex, nval * sizeof(double), mem == GB_MEM_HOST ? cudaMemcpyHostToDevice
                                                                             : cudaMemcpyDeviceToDevice, e->stream);
  } else {
    size_t nint = (size_t)c.nvars;
    for (int d = 0; d < c.ndims; d++) nint *= c.dim[d];
    const double* src = uex;
    if (mem == GB_MEM_HOST) {
      ce = cudaMallocAsync((void**)&tmp, nint * sizeof(double), e->stream);
      if (ce == cudaSuccess) ce = cudaMemcpyAsync(tmp, uex, nint * sizeof(double), cudaMemcpyHostToDevice, e->stream);
      src = tmp;
    }
    if (ce == cudaSuccess) ce = launch_pack(ex, src, md.G, c.nvars, 0, e->stream);
  }
  int rc = GB_OK;
  if (ce != cudaSuccess) {
    gbh_set_error("gb_ensemble_error: %s", cudaGetErrorString(ce));
    rc = GB_ERR_CUDA;
  } else {
    rc = grid_error(e->d_u + md.off, ex, md.G, c.nvars, e->d_red, e->stream, err);
  }
  if (tmp) cudaFreeAsync(tmp, e->stream);
  cudaFreeAsync(ex, e->stream);
  return rc;
}

extern "C" int gb_ensemble_conservation_begin(gb_ensemble* e) {
  if (!e) { gbh_set_error("gb_ensemble_conservation_begin: null ensemble"); return GB_ERR_ARG; }
  if (!e->d_bnd) {
    long long n = 0;
    for (int m = 0; m < e->nm; m++)
      for (int d = 0; d < e->cfg[m].ndims; d++) {
        e->mem[m].bnd_off[d] = n;
        n += 2 * cons_lines(e->cfg[m], d) * e->cfg[m].nvars;
      }
    e->bnd_n = n;
    CK(cudaMalloc((void**)&e->d_bnd, n * sizeof(double)));
    CK(cudaMalloc((void**)&e->d_red, CONS_RED_DOUBLES * sizeof(double)));
    int rc = upload_table(e);
    if (rc) return rc;
  }
  CK(cudaMemsetAsync(e->d_bnd, 0, e->bnd_n * sizeof(double), e->stream));
  e->V0.assign((size_t)e->nm * 5, 0.0);
  for (int m = 0; m < e->nm; m++) {
    const MemberDev& md = e->mem[m];
    const int nd = e->cfg[m].ndims;
    int rc = cons_volume(e->d_u + md.off, e->d_dx + md.dx_off[0], md.G, nd > 1 ? md.dx_off[1] - md.dx_off[0] : 0,
                         nd > 2 ? md.dx_off[2] - md.dx_off[0] : 0, e->cfg[m].nvars, e->d_red, e->stream,
                         &e->V0[(size_t)m * 5]);
    if (rc) return rc;
  }
  e->cons_on = true;
  e->graph_dirty = true;
  return GB_OK;
}

extern "C" int gb_ensemble_conservation_error(gb_ensemble* e, int member, double* err) {
  if (!e || !err || member < 0 || member >= e->nm) {
    gbh_set_error("gb_ensemble_conservation_error: bad argument");
    return GB_ERR_ARG;
  }
  if (!e->cons_on) { gbh_set_error("gb_ensemble_conservation_error: no gb_ensemble_conservation_begin"); return GB_ERR_ARG; }
  const MemberDev& md = e->mem[member];
  const gb_config& c = e->cfg[member];
  double V[5];
  int rc = cons_volume(e->d_u + md.off, e->d_dx + md.dx_off[0], md.G, c.ndims > 1 ? md.dx_off[1] - md.dx_off[0] : 0,
                       c.ndims > 2 ? md.dx_off[2] - md.dx_off[0] : 0, c.nvars, e->d_red, e->stream, V);
  if (rc) return rc;
  double mid[3] = {1.0, 1.0, 1.0};
  for (int k = 0; k < c.ndims; k++)
    CK(cudaMemcpyAsync(&mid[k], e->d_dx + md.dx_off[k] + c.ghosts + c.dim[k] / 2, sizeof(double),
                       cudaMemcpyDeviceToHost, e->stream));
  return cons_error(c, e->d_bnd, md.bnd_off, V, &e->V0[(size_t)member * 5], mid, e->d_red, e->stream, err);
}
