// gbh_api.cu -- the solver object, the Runge-Kutta driver and the C ABI of
// libgbhypar (declared in include/gbhypar.h).
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "gbh_internal.h"
#include "gbh_solver.h"
#include "gbhypar.h"

namespace gbh {
cudaError_t launch_hyp_euler1d(int, int, int, const double*, double*, const double*, const DevGeom&,
                               const PhysParams&, const StageEpi&, const HypLaunch&, cudaStream_t);
cudaError_t launch_hyp_euler2d(int, int, int, const double*, double*, const double*, const DevGeom&,
                               const PhysParams&, const StageEpi&, const HypLaunch&, cudaStream_t);
cudaError_t launch_hyp_ns3d(int, int, int, const double*, double*, const double*, const DevGeom&,
                            const PhysParams&, const StageEpi&, const HypLaunch&, cudaStream_t);
cudaError_t launch_hyp_euler1d_w(int, int, int, const double*, double*, const double*, const DevGeom&,
                                 const PhysParams&, const StageEpi&, const HypLaunch&, cudaStream_t);
cudaError_t launch_hyp_euler2d_w(int, int, int, const double*, double*, const double*, const DevGeom&,
                                 const PhysParams&, const StageEpi&, const HypLaunch&, cudaStream_t);
cudaError_t launch_hyp_ns3d_w(int, int, int, const double*, double*, const double*, const DevGeom&,
                              const PhysParams&, const StageEpi&, const HypLaunch&, cudaStream_t);
cudaError_t launch_hyp_crweno(int, int, int, bool, bool, const double*, double*, const double*, const DevGeom&,
                              const PhysParams&, const StageEpi&, const HypLaunch&, double*, double*, double*,
                              cudaStream_t);
size_t crweno_scratch_doubles(int, int, long long, bool, bool, bool);
cudaError_t launch_hyp_euler1d_grav(int, int, int, const double*, double*, const double*, const DevGeom&,
                                   const PhysParams&, const StageEpi&, const HypLaunch&, cudaStream_t);
cudaError_t launch_hyp_ns3d_grav(int, int, const double*, double*, const double*, const DevGeom&,
                                 const PhysParams&, const StageEpi&, const HypLaunch&, cudaStream_t);
cudaError_t launch_unfused_euler1d(int, int, int, double*, const double*, const double*, const double*,
                                   const double*, const double*, const DevGeom&, const PhysParams&, cudaStream_t);
cudaError_t launch_unfused_euler2d(int, int, int, double*, const double*, const double*, const double*,
                                   const double*, const double*, const DevGeom&, const PhysParams&, cudaStream_t);
cudaError_t launch_unfused_ns3d(int, int, int, double*, const double*, const double*, const double*,
                                const double*, const double*, const DevGeom&, const PhysParams&, cudaStream_t);
cudaError_t launch_interp_euler1d(int, int, int, int, double*, const double*, const double*, const DevGeom&,
                                  const PhysParams&, cudaStream_t);
cudaError_t launch_interp_euler2d(int, int, int, int, double*, const double*, const double*, const DevGeom&,
                                  const PhysParams&, cudaStream_t);
cudaError_t launch_interp_ns3d(int, int, int, int, double*, const double*, const double*, const DevGeom&,
                               const PhysParams&, cudaStream_t);
cudaError_t launch_visc(const double*, double*, double*, double*, const double*, const DevGeom&,
                        const ViscParams&, int, cudaStream_t);
cudaError_t launch_bc_zone(double*, const DevGeom&, int, const int*, const double*, double, cudaStream_t);
cudaError_t launch_bc_zone_t(double*, const DevGeom&, int, const int*, const double*, double, const double*, int, int,
                             cudaStream_t);
cudaError_t launch_sponge(double*, const double*, const DevGeom&, int, const int*, const double*, const double*,
                          cudaStream_t);
cudaError_t launch_finite_check(const double*, const DevGeom&, int, int*, cudaStream_t);
cudaError_t launch_pack(double*, const double*, const DevGeom&, int, int, cudaStream_t);
}  // namespace gbh

using namespace gbh;

static thread_local char g_err[1024] = "";

extern "C" void gbh_set_error(const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof(g_err), fmt, ap);
  va_end(ap);
}

extern "C" const char* gb_last_error(void) { return g_err; }

#define CK(call)                                                                  \
  do {                                                                            \
    cudaError_t e_ = (call);                                                      \
    if (e_ != cudaSuccess) {                                                      \
      gbh_set_error("%s:%d: %s: %s", __FILE__, __LINE__, #call, cudaGetErrorString(e_)); \
      return GB_ERR_CUDA;                                                         \
    }                                                                             \
  } while (0)


static cudaEvent_t ev_get(gb_solver* s) {
  if (!s->pool.empty()) {
    cudaEvent_t e = s->pool.back();
    s->pool.pop_back();
    return e;
  }
  cudaEvent_t e;
  cudaEventCreate(&e);
  return e;
}

// Record the start of a launch group of class `cls` (returns the record index).
static int prof_begin(gb_solver* s, int cls) {
  if (!s->prof) return -1;
  gb_solver::Rec r;
  r.cls = cls;
  r.a = ev_get(s);
  r.b = ev_get(s);
  cudaEventRecord(r.a, s->stream);
  s->recs.push_back(r);
  return (int)s->recs.size() - 1;
}
static void prof_end(gb_solver* s, int idx) {
  if (idx < 0) return;
  cudaEventRecord(s->recs[idx].b, s->stream);
}
static int prof_drain(gb_solver* s) {
  for (auto& r : s->recs) {
    cudaError_t e = cudaEventSynchronize(r.b);
    if (e != cudaSuccess) { gbh_set_error("profiler: %s", cudaGetErrorString(e)); return GB_ERR_CUDA; }
    float ms = 0.f;
    cudaEventElapsedTime(&ms, r.a, r.b);
    s->prof_ms[r.cls] += ms;
    s->prof_n[r.cls] += 1;
    s->pool.push_back(r.a);
    s->pool.push_back(r.b);
  }
  s->recs.clear();
  return GB_OK;
}

static cudaError_t launch_hyp(gb_solver* s, int dir, const double* U, const StageEpi& ep) {
  const gb_config& c = s->cfg;
  const double* dx = s->d_dxinv + s->dx_off[dir];
  if (s->gravity && !s->d_grav) return cudaErrorInvalidValue;  // gb_solver_set_gravity_field not called (checked by callers)
  if (c.hyp_scheme == GB_SCHEME_CRWENO5)
    return launch_hyp_crweno(c.model, dir, c.upwind, c.interp == GB_INTERP_CHARACTERISTIC, s->gravity, U, s->d_H,
                             dx, s->G, s->pp, ep, s->hl[dir], s->d_crX, s->d_crC, s->d_crF, s->stream);
  if (s->gravity) {
    if (c.model == GB_MODEL_EULER1D)
      return launch_hyp_euler1d_grav(dir, c.interp, c.upwind, U, s->d_H, dx, s->G, s->pp, ep, s->hl[dir],
                                     s->stream);
    return launch_hyp_ns3d_grav(dir, c.interp, U, s->d_H, dx, s->G, s->pp, ep, s->hl[dir], s->stream);
  }
  if (s->pp.wtype != WENO_W_JS) {
    if (c.model == GB_MODEL_EULER1D)
      return launch_hyp_euler1d_w(dir, c.interp, c.upwind, U, s->d_H, dx, s->G, s->pp, ep, s->hl[dir], s->stream);
    if (c.model == GB_MODEL_EULER2D)
      return launch_hyp_euler2d_w(dir, c.interp, c.upwind, U, s->d_H, dx, s->G, s->pp, ep, s->hl[dir], s->stream);
    return launch_hyp_ns3d_w(dir, c.interp, c.upwind, U, s->d_H, dx, s->G, s->pp, ep, s->hl[dir], s->stream);
  }
  if (c.model == GB_MODEL_EULER1D)
    return launch_hyp_euler1d(dir, c.interp, c.upwind, U, s->d_H, dx, s->G, s->pp, ep, s->hl[dir], s->stream);
  if (c.model == GB_MODEL_EULER2D)
    return launch_hyp_euler2d(dir, c.interp, c.upwind, U, s->d_H, dx, s->G, s->pp, ep, s->hl[dir], s->stream);
  return launch_hyp_ns3d(dir, c.interp, c.upwind, U, s->d_H, dx, s->G, s->pp, ep, s->hl[dir], s->stream);
}

static cudaError_t launch_unfused(gb_solver* s, int kind, int dir, double* out, const double* a, const double* b,
                                  const double* c2, const double* d, const double* u) {
  const gb_config& c = s->cfg;
  if (c.model == GB_MODEL_EULER1D)
    return launch_unfused_euler1d(kind, dir, c.upwind, out, a, b, c2, d, u, s->G, s->pp, s->stream);
  if (c.model == GB_MODEL_EULER2D)
    return launch_unfused_euler2d(kind, dir, c.upwind, out, a, b, c2, d, u, s->G, s->pp, s->stream);
  return launch_unfused_ns3d(kind, dir, c.upwind, out, a, b, c2, d, u, s->G, s->pp, s->stream);
}

// The boundary zones kept in memory (all zones: `all`) applied to u at time t.
static int apply_mem_bcs(gb_solver* s, double* u, bool all, double t) {
  int pr = -1;
  for (int z = 0; z < s->cfg.nzones; z++) {
    bool use = all;
    if (!use)
      for (int k : s->mem_zones)
        if (k == z) use = true;
    if (use) {
      const int type = s->cfg.zones[z][0];
      const double* tf = nullptr;
      int tn = 0, it = 0;
      if (type == GB_BC_THERMAL_SLIP_WALL || type == GB_BC_THERMAL_NOSLIP_WALL) {
        if (!s->d_tfield[z]) {
          gbh_set_error("boundary zone %d is a thermal wall: call gb_solver_set_zone_temperature first", z);
          return GB_ERR_ARG;
        }
        // the last time level at or before t (BCThermalNoslipWall.c:55-57)
        tn = (int)s->ttimes[z].size();
        it = tn - 1;
        while (it > 0 && s->ttimes[z][it] > t) it--;
        tf = s->d_tfield[z];
      } else if (type == GB_BC_TURBULENT_INFLOW) {
        if (!s->d_tfield[z]) {
          gbh_set_error("boundary zone %d is a turbulent inflow: call gb_solver_set_zone_inflow first", z);
          return GB_ERR_ARG;
        }
        // the slice the mean flow has carried in by time t, over a period of 2 pi
        // (BCTurbulentSupersonicInflow.c:44-48)
        tn = s->fn[z];
        const double xt = s->cfg.zone_data[z][1 + s->cfg.zones[z][1]] * t;
        const double L = 2.0 * (4.0 * atan(1.0));
        const double pos = (xt / L) * ((double)tn);
        if (!(pos > -1.0 && pos < 2147483648.0)) {  // int(pos) >= 0 and representable
          gbh_set_error("turbulent inflow zone %d: slice position %g at t = %g is outside the data", z, pos, t);
          return GB_ERR_ARG;
        }
        it = ((int)pos) % tn;
        tf = s->d_tfield[z];
      }
      if (pr < 0) pr = prof_begin(s, GB_PROF_BC);
      CK(launch_bc_zone_t(u, s->G, s->cfg.nvars, s->cfg.zones[z], s->cfg.zone_data[z], s->cfg.gamma, tf, tn, it,
                          s->stream));
    }
  }
  prof_end(s, pr);
  return GB_OK;
}

extern "C" int gb_solver_set_zone_temperature(gb_solver* s, int zone, int ntimes, const double* times,
                                              const double* field) {
  if (!s || zone < 0 || zone >= s->cfg.nzones || ntimes < 1 || !times || !field) {
    gbh_set_error("gb_solver_set_zone_temperature: bad argument");
    return GB_ERR_ARG;
  }
  const int* q = s->cfg.zones[zone];
  if (q[0] != GB_BC_THERMAL_SLIP_WALL && q[0] != GB_BC_THERMAL_NOSLIP_WALL) {
    gbh_set_error("gb_solver_set_zone_temperature: zone %d is not a thermal wall", zone);
    return GB_ERR_ARG;
  }
  size_t n = (size_t)ntimes;
  for (int d = 0; d < s->cfg.ndims; d++)
    if (d != q[1]) n *= (size_t)(q[6 + d] - q[3 + d] > 0 ? q[6 + d] - q[3 + d] : 0);
  if (n == 0) return GB_OK;  // an empty zone
  cudaFree(s->d_tfield[zone]);
  s->d_tfield[zone] = nullptr;
  CK(cudaMalloc((void**)&s->d_tfield[zone], n * sizeof(double)));
  CK(cudaMemcpy(s->d_tfield[zone], field, n * sizeof(double), cudaMemcpyHostToDevice));
  s->ttimes[zone].assign(times, times + ntimes);
  return GB_OK;
}

extern "C" int gb_solver_set_zone_inflow(gb_solver* s, int zone, int n, const double* data) {
  if (!s || zone < 0 || zone >= s->cfg.nzones || n < 1 || !data) {
    gbh_set_error("gb_solver_set_zone_inflow: bad argument");
    return GB_ERR_ARG;
  }
  const int* q = s->cfg.zones[zone];
  if (q[0] != GB_BC_TURBULENT_INFLOW) {
    gbh_set_error("gb_solver_set_zone_inflow: zone %d is not a turbulent inflow", zone);
    return GB_ERR_ARG;
  }
  size_t cnt = (size_t)n * s->cfg.nvars;
  for (int d = 0; d < s->cfg.ndims; d++)
    if (d != q[1]) cnt *= (size_t)s->cfg.dim[d];
  cudaFree(s->d_tfield[zone]);
  s->d_tfield[zone] = nullptr;
  s->fn[zone] = 0;
  CK(cudaMalloc((void**)&s->d_tfield[zone], cnt * sizeof(double)));
  CK(cudaMemcpy(s->d_tfield[zone], data, cnt * sizeof(double), cudaMemcpyHostToDevice));
  s->fn[zone] = n;
  return GB_OK;
}

extern "C" int gb_solver_set_zone_sponge(gb_solver* s, int zone, const double* sigma) {
  if (!s || zone < 0 || zone >= s->cfg.nzones) {
    gbh_set_error("gb_solver_set_zone_sponge: bad argument");
    return GB_ERR_ARG;
  }
  const int* q = s->cfg.zones[zone];
  if (q[0] != GB_BC_SPONGE) {
    gbh_set_error("gb_solver_set_zone_sponge: zone %d is not a sponge", zone);
    return GB_ERR_ARG;
  }
  const int n = q[6 + q[1]] - q[3 + q[1]];
  if (n <= 0) return GB_OK;  // an empty zone
  if (!sigma) {
    gbh_set_error("gb_solver_set_zone_sponge: null sigma");
    return GB_ERR_ARG;
  }
  cudaFree(s->d_sigma[zone]);
  s->d_sigma[zone] = nullptr;
  CK(cudaMalloc((void**)&s->d_sigma[zone], n * sizeof(double)));
  CK(cudaMemcpy(s->d_sigma[zone], sigma, n * sizeof(double), cudaMemcpyHostToDevice));
  return GB_OK;
}

static bool zone_empty(const gb_config& c, int z) {
  for (int d = 0; d < c.ndims; d++)
    if (c.zones[z][6 + d] <= c.zones[z][3 + d]) return true;
  return false;
}

// Every sponge zone's source term added into src (SourceFunction.c:50-76, zone order).
static int add_sponges(gb_solver* s, double* src, const double* U) {
  for (int z = 0; z < s->cfg.nzones; z++) {
    if (s->cfg.zones[z][0] != GB_BC_SPONGE || zone_empty(s->cfg, z)) continue;
    if (!s->d_sigma[z]) {
      gbh_set_error("boundary zone %d is a sponge: call gb_solver_set_zone_sponge first", z);
      return GB_ERR_ARG;
    }
    CK(launch_sponge(src, U, s->G, s->cfg.nvars, s->cfg.zones[z], s->cfg.zone_data[z], s->d_sigma[z], s->stream));
  }
  return GB_OK;
}

// Right-hand side of U into `epi` (EPI_RHS or EPI_RK): boundary zones kept in
// memory, the viscous term, then one fused hyperbolic launch per direction.
static int gravity_ready(gb_solver* s) {
  if (s->gravity && !s->d_grav) {
    gbh_set_error("gravity: call gb_solver_set_gravity_field before evaluating the right-hand side");
    return GB_ERR_ARG;
  }
  return GB_OK;
}

static int rhs_launches(gb_solver* s, double* U, StageEpi ep, double t) {
  if (int rc = gravity_ready(s)) return rc;
  int rc = apply_mem_bcs(s, U, false, t);
  if (rc) return rc;
  ep.par = nullptr;
  if (s->viscous) {
    int pr = prof_begin(s, GB_PROF_VISC);
    CK(launch_visc(U, s->d_Q, s->d_Gr, s->d_par, s->d_dxinv, s->G, s->vp, s->visc_seg, s->stream));
    prof_end(s, pr);
    ep.par = s->d_par;
  }
  if (s->sponge) {
    // the sponge joins the parabolic term the stage epilogue adds (rhs = par - hyp)
    int pr = prof_begin(s, GB_PROF_BC);
    if (!s->viscous) CK(cudaMemsetAsync(s->d_par, 0, s->nvals * sizeof(double), s->stream));
    rc = add_sponges(s, s->d_par, U);
    prof_end(s, pr);
    if (rc) return rc;
    ep.par = s->d_par;
  }
  int nd = s->cfg.ndims;
  for (int d = 0; d < nd; d++) {
    StageEpi e = ep;
    e.first = (d == 0);
    e.last = (d == nd - 1);
    if (ep.mode == EPI_RK && s->cons_on) {
      e.bnd = s->d_bnd + s->bnd_off[d];
      e.bw = ep.cb;
    }
    int pr = prof_begin(s, GB_PROF_HYP_X + d);
    CK(launch_hyp(s, d, U, e));
    prof_end(s, pr);
  }
  return GB_OK;
}

int gbh_validate(const gb_config* c) {
  if (!c) { gbh_set_error("null config"); return GB_ERR_ARG; }
  int nd = c->model == GB_MODEL_EULER1D ? 1 : c->model == GB_MODEL_EULER2D ? 2 : c->model == GB_MODEL_NS3D ? 3 : 0;
  if (!nd) { gbh_set_error("unknown model %d", c->model); return GB_ERR_ARG; }
  if (c->ndims != nd || c->nvars != nd + 2) { gbh_set_error("ndims/nvars do not match the model"); return GB_ERR_ARG; }
  if (c->ghosts != 3) { gbh_set_error("ghosts must be 3"); return GB_ERR_ARG; }
  for (int d = 0; d < nd; d++)
    if (c->dim[d] < 3) { gbh_set_error("dim[%d] = %d < 3", d, c->dim[d]); return GB_ERR_ARG; }
  if (c->interp != GB_INTERP_COMPONENTS && c->interp != GB_INTERP_CHARACTERISTIC) { gbh_set_error("bad interp"); return GB_ERR_ARG; }
  if (c->upwind < 0 || c->upwind > 4) { gbh_set_error("bad upwind"); return GB_ERR_ARG; }
  if (c->upwind == GB_UPWIND_RUSANOV && c->model == GB_MODEL_EULER2D) {
    gbh_set_error("Euler2D offers no Rusanov upwinding");
    return GB_ERR_UNSUPPORTED;
  }
  if (c->upwind == GB_UPWIND_SWFS && c->model == GB_MODEL_NS3D) {
    gbh_set_error("NavierStokes3D offers no Steger-Warming upwinding");
    return GB_ERR_UNSUPPORTED;
  }
  if (c->rk_nstages < 1 || c->rk_nstages > 4) { gbh_set_error("rk_nstages must be 1..4"); return GB_ERR_ARG; }
  if (!(c->gamma > 1.0)) { gbh_set_error("gamma must exceed 1"); return GB_ERR_ARG; }
  if (!(c->weno_eps > 0.0)) { gbh_set_error("weno_eps must be positive"); return GB_ERR_ARG; }
  if (c->weno_weights < GB_WENO_JS || c->weno_weights > GB_WENO_NONE) { gbh_set_error("bad weno_weights"); return GB_ERR_ARG; }
  if (c->hyp_scheme != GB_SCHEME_WENO5 && c->hyp_scheme != GB_SCHEME_CRWENO5) { gbh_set_error("bad hyp_scheme"); return GB_ERR_ARG; }
  if (c->gravity[0] != 0.0 || c->gravity[1] != 0.0 || c->gravity[2] != 0.0) {
    if (c->model == GB_MODEL_EULER2D) { gbh_set_error("gravity: Euler2D has none"); return GB_ERR_UNSUPPORTED; }
    if (c->model == GB_MODEL_EULER1D) {
      if (c->upwind != GB_UPWIND_ROE && c->upwind != GB_UPWIND_LLF) {
        gbh_set_error("flows with gravity need roe or llf-char upwinding (Euler1DInitialize.c:144)");
        return GB_ERR_ARG;
      }
      if (c->grav_type != 0 && c->grav_type != 1) { gbh_set_error("gravity_type must be 0 or 1"); return GB_ERR_ARG; }
    } else {
      if (c->upwind != GB_UPWIND_RUSANOV) {
        gbh_set_error("flows with gravity need rusanov upwinding (NavierStokes3DInitialize.c:371)");
        return GB_ERR_ARG;
      }
      if (!(c->rho_ref > 0.0) || !(c->p_ref > 0.0)) { gbh_set_error("gravity needs positive rho_ref and p_ref"); return GB_ERR_ARG; }
    }
  }
  if (c->nzones < 0 || c->nzones > GB_MAX_ZONES) { gbh_set_error("bad nzones"); return GB_ERR_ARG; }
  for (int z = 0; z < c->nzones; z++) {
    const int* q = c->zones[z];
    if (q[0] < GB_BC_PERIODIC || q[0] > GB_BC_REFLECT || q[1] < 0 || q[1] >= nd ||
        (q[2] != 1 && q[2] != -1)) {
      gbh_set_error("bad zone %d", z);
      return GB_ERR_ARG;
    }
    if (q[0] == GB_BC_SPONGE) {
      // interior points only (CalculateLocalExtent, InitializeBoundaries.c:382-393)
      bool empty = false, inside = true;
      for (int d = 0; d < nd; d++) {
        if (q[6 + d] <= q[3 + d]) empty = true;
        if (q[3 + d] < 0 || q[6 + d] > c->dim[d]) inside = false;
      }
      if (!empty && !inside) { gbh_set_error("sponge zone %d must cover interior points only", z); return GB_ERR_ARG; }
      continue;
    }
    if (q[0] > GB_BC_DIRICHLET && q[0] != GB_BC_REFLECT && q[0] != GB_BC_SLIP_WALL && nd < 2) {
      gbh_set_error("zone %d: inflow / outflow / no-slip boundaries need Euler2D or NavierStokes3D", z);
      return GB_ERR_UNSUPPORTED;
    }
    if ((q[0] == GB_BC_THERMAL_SLIP_WALL || q[0] == GB_BC_THERMAL_NOSLIP_WALL) && c->model != GB_MODEL_NS3D) {
      gbh_set_error("zone %d: thermal walls need NavierStokes3D", z);
      return GB_ERR_UNSUPPORTED;
    }
    if (q[0] == GB_BC_TURBULENT_INFLOW) {
      if (c->model != GB_MODEL_NS3D) {
        gbh_set_error("zone %d: turbulent inflow needs NavierStokes3D", z);
        return GB_ERR_UNSUPPORTED;
      }
      // the inflow data spans the grid across the zone's dimension
      for (int d = 0; d < nd; d++)
        if (d != q[1] && q[6 + d] > q[3 + d] && (q[3 + d] < 0 || q[6 + d] > c->dim[d])) {
          gbh_set_error("zone %d: a turbulent inflow's transverse extent must lie within the grid", z);
          return GB_ERR_ARG;
        }
    }
    for (int d = 0; d < nd; d++) {
      int lo = -c->ghosts, hi = c->dim[d] + c->ghosts;
      if (q[3 + d] < lo || q[6 + d] > hi) { gbh_set_error("zone %d extent out of range", z); return GB_ERR_ARG; }
    }
    int d = q[1];
    bool ok = (q[2] == 1) ? (q[3 + d] == -c->ghosts && q[6 + d] == 0) : (q[3 + d] == c->dim[d] && q[6 + d] == c->dim[d] + c->ghosts);
    if (!ok) { gbh_set_error("zone %d: extent along its own dimension must be the ghost layer", z); return GB_ERR_ARG; }
  }
  return GB_OK;
}

// Geometry of a configuration: strides with ghosts, and per face whether the
// boundary is folded into the halo loads (exactly one zone covering the whole
// face) or applied in memory by bc_zone_kernel (zone indices into mem_zones).
long long gbh_geometry(const gb_config& c, DevGeom& G, std::vector<int>* mem_zones) {
  G.nd = c.ndims;
  G.g = c.ghosts;
  long long st = 1;
  for (int d = 0; d < 3; d++) {
    G.dim[d] = d < c.ndims ? c.dim[d] : 1;
    G.stride[d] = d < c.ndims ? st : 0;
    if (d < c.ndims) st *= (c.dim[d] + 2 * c.ghosts);
    G.bclo[d] = G.bchi[d] = FOLD_MEMORY;
  }
  for (int d = 0; d < c.ndims; d++)
    for (int side = 0; side < 2; side++) {
      int face = side == 0 ? 1 : -1, cnt = 0, which = -1;
      for (int z = 0; z < c.nzones; z++)
        if (c.zones[z][0] != GB_BC_SPONGE && c.zones[z][1] == d && c.zones[z][2] == face) { cnt++; which = z; }
      bool full = false;
      // only periodic and extrapolate (a copy of one interior cell) fold into the loads
      if (cnt == 1 && c.zones[which][0] != GB_BC_PERIODIC && c.zones[which][0] != GB_BC_EXTRAPOLATE) cnt = 0;
      if (cnt == 1) {
        full = true;
        for (int e = 0; e < c.ndims; e++)
          if (e != d && (c.zones[which][3 + e] > 0 || c.zones[which][6 + e] < c.dim[e])) full = false;
      }
      int mode = FOLD_MEMORY;
      if (full) mode = c.zones[which][0] == GB_BC_PERIODIC ? FOLD_PERIODIC : FOLD_MIRROR;
      if (side == 0) G.bclo[d] = mode; else G.bchi[d] = mode;
      if (mem_zones)
        for (int z = 0; z < c.nzones; z++)
          if (c.zones[z][0] != GB_BC_SPONGE && c.zones[z][1] == d && c.zones[z][2] == face && !full)
            mem_zones->push_back(z);
    }
  return st;
}

extern "C" int gb_solver_create(const gb_config* cfg, const double* dxinv, int device, gb_solver** out) {
  if (!out || !dxinv) { gbh_set_error("gb_solver_create: null argument"); return GB_ERR_ARG; }
  *out = nullptr;
  int rc = gbh_validate(cfg);
  if (rc) return rc;
  gb_solver* s = new gb_solver();
  s->cfg = *cfg;
  const gb_config& c = s->cfg;
  if (device >= 0) {
    cudaError_t e = cudaSetDevice(device);
    if (e != cudaSuccess) { gbh_set_error("cudaSetDevice(%d): %s", device, cudaGetErrorString(e)); delete s; return GB_ERR_CUDA; }
  }
  cudaGetDevice(&s->device);
  s->npts_wg = gbh_geometry(c, s->G, &s->mem_zones);
  long long st = s->npts_wg;
  s->nvals = (size_t)st * c.nvars;
  s->pp.gamma = c.gamma;
  s->pp.gm1 = c.gamma - 1.0;
  s->pp.inv_gm1 = 1.0 / (c.gamma - 1.0);
  s->pp.eps = c.weno_eps;
  s->pp.wtype = c.weno_weights;
  s->pp.gf = s->pp.gg = nullptr;
  for (int d = 0; d < 3; d++) s->pp.grav[d] = c.gravity[d];
  // NavierStokes3D: RT = p0 / rho0; Euler1D's source has no such factor (RT = 1)
  s->pp.RT = (c.model == GB_MODEL_NS3D && c.rho_ref > 0) ? c.p_ref / c.rho_ref : 1.0;
  s->gravity = c.model != GB_MODEL_EULER2D && (c.gravity[0] != 0.0 || c.gravity[1] != 0.0 || c.gravity[2] != 0.0);
  s->viscous = (c.model == GB_MODEL_NS3D) && (c.Re > 0);
  double Re_eff = c.Re / c.Minf;  // NavierStokes3DInitialize.c:368
  s->vp.gamma = c.gamma;
  s->vp.gm1 = c.gamma - 1.0;
  s->vp.inv_gm1 = 1.0 / (c.gamma - 1.0);
  s->vp.inv_Re = 1.0 / Re_eff;
  s->vp.inv_Pr = 1.0 / c.Pr;
  s->vp.order = c.par_scheme == 2 ? 2 : 4;
  for (int d = 0; d < 3; d++) {
    s->hl[d].seg = 32;
    s->hl[d].block = 128;
  }
  long long off = 0;
  for (int d = 0; d < c.ndims; d++) {
    s->dx_off[d] = off;
    off += c.dim[d] + 2 * c.ghosts;
  }
  size_t bytes = s->nvals * sizeof(double);
  cudaError_t e = cudaSuccess;
  auto A = [&](double** p, size_t n) {
    if (e == cudaSuccess) e = cudaMalloc((void**)p, n);
    if (e == cudaSuccess) e = cudaMemset(*p, 0, n);
  };
  A(&s->d_u, bytes);
  A(&s->d_acc, bytes);
  for (int k = 1; k < c.rk_nstages; k++) A(&s->d_P[k], bytes);
  if (c.ndims > 1 || s->gravity) A(&s->d_H, bytes);  // gravity: gb_SourceFunction's second pass
  if (c.hyp_scheme == GB_SCHEME_CRWENO5) {
    // the largest direction's interface values and elimination scratch
    const bool chr = c.interp == GB_INTERP_CHARACTERISTIC;
    size_t nx = 0, nc = 0;
    for (int d = 0; d < c.ndims; d++) {
      long long lines = 1;
      for (int e = 0; e < c.ndims; e++)
        if (e != d) lines *= c.dim[e];
      size_t a = crweno_scratch_doubles(c.nvars, c.dim[d] + 1, lines, chr, false, s->gravity);
      size_t b = crweno_scratch_doubles(c.nvars, c.dim[d] + 1, lines, chr, true, s->gravity);
      nx = a > nx ? a : nx;
      nc = b > nc ? b : nc;
    }
    A(&s->d_crX, nx * sizeof(double));
    A(&s->d_crC, nc * sizeof(double));
    if (!chr) A(&s->d_crF, bytes);
  }
  for (int z = 0; z < c.nzones; z++)
    if (c.zones[z][0] == GB_BC_SPONGE && !zone_empty(c, z)) s->sponge = true;
  if (s->viscous || s->sponge) A(&s->d_par, bytes);
  if (s->viscous) {
    A(&s->d_Q, (size_t)st * 6 * sizeof(double));
    A(&s->d_Gr, (size_t)st * 12 * sizeof(double));
  }
  A(&s->d_dxinv, off * sizeof(double));
  if (e == cudaSuccess) e = cudaMalloc((void**)&s->d_flag, sizeof(int));
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking);
  if (e == cudaSuccess) s->own_stream = true;
  if (e == cudaSuccess) e = cudaMemcpy(s->d_dxinv, dxinv, off * sizeof(double), cudaMemcpyHostToDevice);
  if (e != cudaSuccess) {
    gbh_set_error("gb_solver_create: %s", cudaGetErrorString(e));
    gb_solver_destroy(s);
    return e == cudaErrorMemoryAllocation ? GB_ERR_NOMEM : GB_ERR_CUDA;
  }
  *out = s;
  return GB_OK;
}

extern "C" void gb_solver_destroy(gb_solver* s) {
  if (!s) return;
  cudaFree(s->d_u);
  cudaFree(s->d_acc);
  for (int k = 0; k < 4; k++) cudaFree(s->d_P[k]);
  cudaFree(s->d_U0);
  for (int z = 0; z < GB_MAX_ZONES; z++) {
    cudaFree(s->d_tfield[z]);
    cudaFree(s->d_sigma[z]);
  }
  cudaFree(s->d_stage);
  cudaFree(s->d_H);
  cudaFree(s->d_crX);
  cudaFree(s->d_crC);
  cudaFree(s->d_crF);
  cudaFree(s->d_par);
  cudaFree(s->d_Q);
  cudaFree(s->d_Gr);
  cudaFree(s->d_dxinv);
  cudaFree(s->d_flag);
  cudaFree(s->d_snap);
  cudaFree(s->d_red);
  cudaFree(s->d_grav);
  cudaFree(s->d_bnd);
  prof_drain(s);
  for (cudaEvent_t e : s->pool) cudaEventDestroy(e);
  if (s->own_stream && s->stream) cudaStreamDestroy(s->stream);
  delete s;
}

extern "C" int gb_solver_profile(gb_solver* s, int enable) {
  if (!s) { gbh_set_error("null solver"); return GB_ERR_ARG; }
  int rc = prof_drain(s);
  for (int k = 0; k < GB_PROF_CLASSES; k++) {
    s->prof_ms[k] = 0.0;
    s->prof_n[k] = 0;
  }
  s->prof = enable != 0;
  return rc;
}

extern "C" int gb_solver_profile_read(gb_solver* s, double* ms, long long* launches) {
  if (!s || !ms || !launches) { gbh_set_error("null argument"); return GB_ERR_ARG; }
  int rc = prof_drain(s);
  for (int k = 0; k < GB_PROF_CLASSES; k++) {
    ms[k] = s->prof_ms[k];
    launches[k] = s->prof_n[k];
  }
  return rc;
}

extern "C" const gb_config* gb_solver_config(const gb_solver* s) { return s ? &s->cfg : nullptr; }

extern "C" int gb_solver_set_stream(gb_solver* s, void* stream) {
  if (!s) { gbh_set_error("null solver"); return GB_ERR_ARG; }
  if (s->own_stream && s->stream) {
    cudaStreamSynchronize(s->stream);
    cudaStreamDestroy(s->stream);
    s->own_stream = false;
    s->stream = nullptr;
  }
  if (stream) {
    s->stream = (cudaStream_t)stream;
  } else {
    CK(cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking));
    s->own_stream = true;
  }
  return GB_OK;
}

extern "C" int gb_solver_sync(gb_solver* s) {
  if (!s) { gbh_set_error("null solver"); return GB_ERR_ARG; }
  CK(cudaStreamSynchronize(s->stream));
  return GB_OK;
}

extern "C" int gb_solver_set_gravity_field(gb_solver* s, const double* fg) {
  if (!s || !fg) { gbh_set_error("gb_solver_set_gravity_field: null argument"); return GB_ERR_ARG; }
  if (!s->gravity) { gbh_set_error("gb_solver_set_gravity_field: the configuration has no gravity"); return GB_ERR_ARG; }
  if (!s->d_grav) CK(cudaMalloc((void**)&s->d_grav, 2 * s->npts_wg * sizeof(double)));
  CK(cudaMemcpy(s->d_grav, fg, 2 * s->npts_wg * sizeof(double), cudaMemcpyHostToDevice));
  s->pp.gf = s->d_grav;
  s->pp.gg = s->d_grav + s->npts_wg;
  return GB_OK;
}

extern "C" int gb_solver_set_launch(gb_solver* s, int dir, int seg, int block) {
  if (!s || dir < 0 || dir >= s->cfg.ndims) { gbh_set_error("gb_solver_set_launch: bad argument"); return GB_ERR_ARG; }
  // -t: tiles of t interfaces; -8 / -16: lane groups (Euler1D component-wise WENO5, no gravity)
  const bool lanes_ok = s->cfg.model == GB_MODEL_EULER1D && s->cfg.interp == GB_INTERP_COMPONENTS && !s->gravity &&
                        s->cfg.hyp_scheme == GB_SCHEME_WENO5;
  if ((seg == -8 || seg == -16) && !lanes_ok) {
    gbh_set_error("gb_solver_set_launch: lane groups (-8, -16) need Euler1D, component-wise WENO5, no gravity");
    return GB_ERR_ARG;
  }
  if (seg > 0 || seg == -32 || seg == -64 || seg == -128 || seg == -8 || seg == -16) s->hl[dir].seg = seg;
  if (block > 0) {
    if (block % 32 || block > 128) { gbh_set_error("block must be a multiple of 32, at most 128"); return GB_ERR_ARG; }
    s->hl[dir].block = block;
  }
  return GB_OK;
}

// Copy between the interior (no ghosts) and ghosted layouts on the device.
extern "C" int gb_solver_set_state(gb_solver* s, const double* u, int layout, int mem) {
  if (!s || !u) { gbh_set_error("gb_solver_set_state: null argument"); return GB_ERR_ARG; }
  size_t bytes = s->nvals * sizeof(double);
  if (layout == GB_LAYOUT_GHOSTED) {
    CK(cudaMemcpyAsync(s->d_u, u, bytes, mem == GB_MEM_HOST ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToDevice,
                       s->stream));
  } else {
    size_t nint = 1;
    for (int d = 0; d < s->cfg.ndims; d++) nint *= s->cfg.dim[d];
    const double* src = u;
    if (mem == GB_MEM_HOST) {
      // a kept staging array: allocating and freeing one per call made every call
      // pay for the memory pool's trimming at the next synchronisation
      if (!s->d_stage) CK(cudaMalloc((void**)&s->d_stage, nint * s->cfg.nvars * sizeof(double)));
      CK(cudaMemcpyAsync(s->d_stage, u, nint * s->cfg.nvars * sizeof(double), cudaMemcpyHostToDevice, s->stream));
      src = s->d_stage;
    }
    CK(launch_pack(s->d_u, src, s->G, s->cfg.nvars, 0, s->stream));
  }
  // every work array starts with the same ghost values as u
  CK(cudaMemcpyAsync(s->d_acc, s->d_u, bytes, cudaMemcpyDeviceToDevice, s->stream));
  for (int k = 1; k < s->cfg.rk_nstages; k++)
    CK(cudaMemcpyAsync(s->d_P[k], s->d_u, bytes, cudaMemcpyDeviceToDevice, s->stream));
  s->t = 0.0;
  s->iter = 0;
  return GB_OK;
}

extern "C" int gb_solver_get_state(gb_solver* s, double* u, int layout, int mem) {
  if (!s || !u) { gbh_set_error("gb_solver_get_state: null argument"); return GB_ERR_ARG; }
  size_t bytes = s->nvals * sizeof(double);
  if (layout == GB_LAYOUT_GHOSTED) {
    CK(cudaMemcpyAsync(u, s->d_u, bytes, mem == GB_MEM_HOST ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice,
                       s->stream));
  } else {
    size_t nint = 1;
    for (int d = 0; d < s->cfg.ndims; d++) nint *= s->cfg.dim[d];
    size_t ib = nint * s->cfg.nvars * sizeof(double);
    double* dst = u;
    if (mem == GB_MEM_HOST) {
      if (!s->d_stage) CK(cudaMalloc((void**)&s->d_stage, ib));
      dst = s->d_stage;
    }
    CK(launch_pack(dst, s->d_u, s->G, s->cfg.nvars, 1, s->stream));
    if (mem == GB_MEM_HOST) CK(cudaMemcpyAsync(u, s->d_stage, ib, cudaMemcpyDeviceToHost, s->stream));
  }
  CK(cudaStreamSynchronize(s->stream));
  return GB_OK;
}

extern "C" double* gb_solver_state(gb_solver* s) { return s ? s->d_u : nullptr; }
extern "C" double gb_solver_time(const gb_solver* s) { return s ? s->t : 0.0; }
extern "C" int gb_solver_set_time(gb_solver* s, double t) {
  if (!s) { gbh_set_error("gb_solver_set_time: null solver"); return GB_ERR_ARG; }
  s->t = t;
  return GB_OK;
}

// A hook installed with gb_solver_set_hooks, called with the solver's queued work
// finished; the device is synchronised again after it returns, so the hook may
// use any stream.
template <typename F>
static int call_hook(gb_solver* s, const char* name, F&& f) {
  CK(cudaStreamSynchronize(s->stream));
  int r = f();
  if (r) {
    gbh_set_error("%s hook returned %d", name, r);
    return GB_ERR_HOOK;
  }
  CK(cudaDeviceSynchronize());
  return GB_OK;
}

// One Runge-Kutta step (TimeRK, src/TimeIntegration/TimeRK.c:126-195) as
// nstages x ndims fused launches.  With hooks installed: PreStep before the
// step (TimePreStep.c:122-124), PostStage on every stage state before its
// right-hand side (TimeRK.c:155-162), PostStep after it (TimePostStep.c:95-97).
int gbh_rk_step(gb_solver* s) {
  const gb_config& c = s->cfg;
  const int ns = c.rk_nstages;
  const double dt = c.dt;
  int touched[4] = {0, 0, 0, 0};
  if (s->pre_step) {
    int rc = call_hook(s, "PreStep", [&] { return s->pre_step(s->d_u, s->hook_solver, s->hook_mpi, s->t); });
    if (rc) return rc;
  }
  for (int st = 0; st < ns; st++) {
    double* U = (st == 0 || !touched[st]) ? s->d_u : s->d_P[st];
    if (s->post_stage) {
      // the reference hands PostStage a copy of the stage state (U[stage] = u + ...),
      // never u itself: a stage that reads u gets it copied first
      if (U == s->d_u) {
        if (!s->d_U0) CK(cudaMalloc((void**)&s->d_U0, s->nvals * sizeof(double)));
        CK(cudaMemcpyAsync(s->d_U0, s->d_u, s->nvals * sizeof(double), cudaMemcpyDeviceToDevice, s->stream));
        U = s->d_U0;
      }
      const double ts = s->t + c.rk_c[st] * dt;
      int rc = call_hook(s, "PostStage", [&] { return s->post_stage(U, s->hook_solver, s->hook_mpi, ts); });
      if (rc) return rc;
    }
    StageEpi ep;
    memset(&ep, 0, sizeof(ep));
    ep.mode = EPI_RK;
    ep.stage = st;
    ep.nstages = ns;
    ep.cb = dt * c.rk_b[st];
    ep.need_u = (st == 0);
    for (int t = 0; t < 4; t++) {
      ep.ca[t] = 0.0;
      ep.touched[t] = touched[t];
      ep.P[t] = s->d_P[t];
      if (t > st && t < ns) {
        ep.ca[t] = dt * c.rk_A[4 * t + st];
        if (ep.ca[t] != 0.0 && !touched[t]) ep.need_u = 1;
      }
    }
    ep.u = s->d_u;
    ep.acc = s->d_acc;
    ep.uout = (ns == 1) ? s->d_acc : s->d_u;
    int rc = rhs_launches(s, U, ep, s->t + c.rk_c[st] * dt);
    if (rc) return rc;
    for (int t = st + 1; t < ns; t++)
      if (ep.ca[t] != 0.0) touched[t] = 1;
  }
  if (ns == 1) {
    double* tmp = s->d_u;
    s->d_u = s->d_acc;
    s->d_acc = tmp;
  }
  s->t += dt;
  const int done = s->iter++;
  if (s->post_step) {
    int rc = call_hook(s, "PostStep",
                       [&] { return s->post_step(s->d_u, s->hook_solver, s->hook_mpi, s->t, done); });
    if (rc) return rc;
  }
  return GB_OK;
}

extern "C" int gb_solver_set_hooks(gb_solver* s, int (*PreStage)(int, double**, void*, void*, double),
                                   int (*PostStage)(double*, void*, void*, double),
                                   int (*PreStep)(double*, void*, void*, double),
                                   int (*PostStep)(double*, void*, void*, double, int), void* solver,
                                   void* mpi) {
  if (!s) { gbh_set_error("gb_solver_set_hooks: null solver"); return GB_ERR_ARG; }
  if (PreStage) {
    // TimeRK.c:144-152: the reference refuses a PreStage hook ("Call to
    // solver->PreStage() commented out!")
    gbh_set_error("gb_solver_set_hooks: PreStage is not called by the reference's TimeRK either");
    return GB_ERR_UNSUPPORTED;
  }
  s->post_stage = PostStage;
  s->pre_step = PreStep;
  s->post_step = PostStep;
  s->hook_solver = solver;
  s->hook_mpi = mpi;
  return GB_OK;
}

extern "C" int gb_solver_step(gb_solver* s, int nsteps) {
  if (!s || nsteps < 0) { gbh_set_error("gb_solver_step: bad argument"); return GB_ERR_ARG; }
  for (int n = 0; n < nsteps; n++) {
    int rc = gbh_rk_step(s);
    if (rc) return rc;
  }
  CK(cudaGetLastError());
  return GB_OK;
}

extern "C" int gb_solver_get_launch(gb_solver* s, int dir, int* seg, int* block) {
  if (!s || dir < 0 || dir >= s->cfg.ndims || !seg || !block) { gbh_set_error("gb_solver_get_launch: bad argument"); return GB_ERR_ARG; }
  *seg = s->hl[dir].seg;
  *block = s->hl[dir].block;
  return GB_OK;
}

// Launch-shape autotuner.  The fused kernels are bound by the FP64 pipe, which
// a few warps per SM saturate, so the shape mostly decides how evenly the
// walk segments spread over the SMs (a partial last wave idles SMs) against the
// per-segment overhead (a six-cell window warm-up and one extra interface).
// Candidates: segment lengths that give 1..4 full waves of 4 warps per SM, plus
// fixed lengths; each is timed on `reps` steps of the resident solution, which
// is restored afterwards.
extern "C" int gb_solver_autotune(gb_solver* s, int reps) {
  if (!s) { gbh_set_error("null solver"); return GB_ERR_ARG; }
  if (reps < 1) reps = 1;
  int sms = 0;
  CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, s->device));
  size_t bytes = s->nvals * sizeof(double);
  double* save = nullptr;
  CK(cudaMallocAsync((void**)&save, bytes, s->stream));
  CK(cudaMemcpyAsync(save, s->d_u, bytes, cudaMemcpyDeviceToDevice, s->stream));
  double t0 = s->t;
  bool prof_was = s->prof;
  const bool cons_was = s->cons_on;  // the trial steps add no boundary fluxes
  s->cons_on = false;
  // nor do they call the HyPar hooks: they are not steps of the run
  auto post_stage = s->post_stage;
  auto pre_step = s->pre_step;
  auto post_step = s->post_step;
  const int iter0 = s->iter;
  s->post_stage = nullptr;
  s->pre_step = nullptr;
  s->post_step = nullptr;
  const gb_config& c = s->cfg;
  int rc = GB_OK;
  for (int d = 0; d < c.ndims && !rc; d++) {
    int N = c.dim[d];
    long long ntrans = 1;
    for (int e = 0; e < c.ndims; e++)
      if (e != d) ntrans *= c.dim[e];
    std::vector<int> segs;
    for (int w = 1; w <= 4; w++) {
      double lanes = (double)w * sms * 4 * 32;
      long long nseg = (long long)(lanes / (double)ntrans + 0.5);
      if (nseg < 1) nseg = 1;
      int sg = (int)((N + nseg - 1) / nseg);
      segs.push_back(sg);
    }
    for (int sg : {8, 16, 24, 32, 48, 64}) segs.push_back(sg);
    // Small grids (at most four waves of 4 warps per SM at one interface per
    // thread) cannot fill the SMs with long segments: there, also 1-3
    // interfaces per thread and 32-thread blocks, spreading the few threads
    // over more SMs at the price of recomputing the segments' first interfaces.
    const bool small = (double)ntrans * N <= 4.0 * sms * 4 * 32;
    if (small)
      for (int sg : {1, 2, 3}) segs.push_back(sg);
    std::vector<int> blocks = {128, 64};
    if (small) blocks.push_back(32);
    // shared-memory tiles of 32 / 64 / 128 interfaces (seg = -tile; not with gravity
    // or CRWENO5, whose kernels have no tile form)
    if (!s->gravity && c.hyp_scheme == GB_SCHEME_WENO5)
      for (int ti : {32, 64, 128}) segs.push_back(-ti);
    // lane groups of 8 / 16 interfaces (Euler1D component-wise: short lines)
    if (!s->gravity && c.hyp_scheme == GB_SCHEME_WENO5 && c.model == GB_MODEL_EULER1D &&
        c.interp == GB_INTERP_COMPONENTS)
      for (int ti : {8, 16}) segs.push_back(-ti);
    double best = 1e30;
    HypLaunch bestL = s->hl[d];
    for (int sg : segs) {
      if (sg > 0 && (sg < (small ? 1 : 4) || sg > N)) continue;
      if (sg < 0 && -sg > 2 * (N + 1)) continue;
      for (int blk : blocks) {
        if (sg < 0 && blk != blocks[0]) continue;  // a tile's block is the tile
        s->hl[d].seg = sg;
        s->hl[d].block = blk;
        rc = gbh_rk_step(s);  // warm
        if (!rc) rc = gb_solver_profile(s, 1);
        for (int r = 0; r < reps && !rc; r++) rc = gbh_rk_step(s);
        double ms[GB_PROF_CLASSES];
        long long nl[GB_PROF_CLASSES];
        if (!rc) rc = gb_solver_profile_read(s, ms, nl);
        if (rc) break;
        if (ms[GB_PROF_HYP_X + d] < best) {
          best = ms[GB_PROF_HYP_X + d];
          bestL = s->hl[d];
        }
      }
      if (rc) break;
    }
    s->hl[d] = bestL;
  }
  gb_solver_profile(s, prof_was ? 1 : 0);
  CK(cudaMemcpyAsync(s->d_u, save, bytes, cudaMemcpyDeviceToDevice, s->stream));
  CK(cudaMemcpyAsync(s->d_acc, save, bytes, cudaMemcpyDeviceToDevice, s->stream));
  for (int k = 1; k < c.rk_nstages; k++)
    CK(cudaMemcpyAsync(s->d_P[k], save, bytes, cudaMemcpyDeviceToDevice, s->stream));
  CK(cudaFreeAsync(save, s->stream));
  CK(cudaStreamSynchronize(s->stream));
  s->t = t0;
  s->cons_on = cons_was;
  s->post_stage = post_stage;
  s->pre_step = pre_step;
  s->post_step = post_step;
  s->iter = iter0;
  return rc;
}

extern "C" int gb_solver_check_finite(gb_solver* s, int* finite) {
  if (!s || !finite) { gbh_set_error("null argument"); return GB_ERR_ARG; }
  int h = 0;
  CK(cudaMemsetAsync(s->d_flag, 0, sizeof(int), s->stream));
  CK(launch_finite_check(s->d_u, s->G, s->cfg.nvars, s->d_flag, s->stream));
  CK(cudaMemcpyAsync(&h, s->d_flag, sizeof(int), cudaMemcpyDeviceToHost, s->stream));
  CK(cudaStreamSynchronize(s->stream));
  *finite = h ? 0 : 1;
  return GB_OK;
}

// ---------------------------------------------------------------------------
// HyPar function-pointer surface.
// ---------------------------------------------------------------------------
extern "C" int gb_FFunction(double* f, double* u, int dir, void* sv, double t);
extern "C" int gb_Upwind(double* fI, double* fL, double* fR, double* uL, double* uR, double* u, int dir, void* sv,
                         double t);

static gb_solver* S(void* sv) { return (gb_solver*)sv; }

extern "C" int gb_HyperbolicFunction(double* hyp, double* u, void* sv, void* m, double t, int LimFlag,
                                     int (*F)(double*, double*, int, void*, double),
                                     int (*Upw)(double*, double*, double*, double*, double*, double*, int, void*,
                                                double)) {
  (void)m;
  (void)t;
  (void)LimFlag;
  gb_solver* s = S(sv);
  if (!s || !hyp || !u) { gbh_set_error("gb_HyperbolicFunction: null argument"); return GB_ERR_ARG; }
  if (F == nullptr && Upw == nullptr) {
    // HyperbolicFunction.c:66: no flux function means a zero hyperbolic term
    CK(cudaMemsetAsync(hyp, 0, s->nvals * sizeof(double), s->stream));
    return GB_OK;
  }
  if (F != gb_FFunction || (Upw != nullptr && Upw != gb_Upwind)) {
    gbh_set_error("gb_HyperbolicFunction: flux/upwind must be gb_FFunction/gb_Upwind");
    return GB_ERR_UNSUPPORTED;
  }
  if (int rc = gravity_ready(s)) return rc;
  CK(cudaMemsetAsync(hyp, 0, s->nvals * sizeof(double), s->stream));
  StageEpi ep;
  memset(&ep, 0, sizeof(ep));
  ep.mode = EPI_HYP;
  double* H = s->d_H;
  s->d_H = hyp;  // accumulate straight into the caller's array
  int rc = GB_OK;
  for (int d = 0; d < s->cfg.ndims && !rc; d++) {
    StageEpi e = ep;
    e.first = (d == 0);
    e.last = (d == s->cfg.ndims - 1);
    cudaError_t ce = launch_hyp(s, d, u, e);
    if (ce != cudaSuccess) { gbh_set_error("gb_HyperbolicFunction: %s", cudaGetErrorString(ce)); rc = GB_ERR_CUDA; }
  }
  s->d_H = H;
  return rc;
}

extern "C" int gb_ParabolicFunction(double* par, double* u, void* sv, void* m, double t) {
  (void)m;
  (void)t;
  gb_solver* s = S(sv);
  if (!s || !par || !u) { gbh_set_error("gb_ParabolicFunction: null argument"); return GB_ERR_ARG; }
  CK(cudaMemsetAsync(par, 0, s->nvals * sizeof(double), s->stream));
  if (!s->viscous) return GB_OK;
  CK(launch_visc(u, s->d_Q, s->d_Gr, par, s->d_dxinv, s->G, s->vp, s->visc_seg, s->stream));
  return GB_OK;
}

// out = a - out, elementwise
static __global__ void sub_kernel(double* __restrict__ out, const double* __restrict__ a, long long n) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = a[i] - out[i];
}

extern "C" int gb_SourceFunction(double* source, double* u, void* sv, void* m, double t) {
  (void)u;
  (void)m;
  (void)t;
  gb_solver* s = S(sv);
  if (!s || !source) { gbh_set_error("gb_SourceFunction: null argument"); return GB_ERR_ARG; }
  if (s->gravity) {
    // The well-balanced source (NavierStokes3DSource.c) interpolates the gravity
    // field with the flux's own WENO weights, so the direction kernels evaluate it
    // in their epilogue.  Here: source = hyp - (hyp - source), the hyperbolic term
    // without and with the source subtracted.
    if (!u) { gbh_set_error("gb_SourceFunction: null argument"); return GB_ERR_ARG; }
    if (int rc = gravity_ready(s)) return rc;
    double* H = s->d_H;
    CK(cudaMemsetAsync(source, 0, s->nvals * sizeof(double), s->stream));
    CK(cudaMemsetAsync(H, 0, s->nvals * sizeof(double), s->stream));
    int rc = GB_OK;
    for (int pass = 0; pass < 2 && !rc; pass++) {
      s->d_H = pass == 0 ? source : H;
      StageEpi ep;
      memset(&ep, 0, sizeof(ep));
      ep.mode = EPI_HYP;
      ep.with_source = pass == 0;
      for (int d = 0; d < s->cfg.ndims && !rc; d++) {
        StageEpi e = ep;
        e.first = (d == 0);
        e.last = (d == s->cfg.ndims - 1);
        cudaError_t ce = launch_hyp(s, d, u, e);
        if (ce != cudaSuccess) { gbh_set_error("gb_SourceFunction: %s", cudaGetErrorString(ce)); rc = GB_ERR_CUDA; }
      }
    }
    s->d_H = H;
    if (rc) return rc;
    const long long n = (long long)s->nvals;
    sub_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s->stream>>>(source, H, n);
    CK(cudaGetLastError());
    return u ? add_sponges(s, source, u) : GB_OK;
  }
  CK(cudaMemsetAsync(source, 0, s->nvals * sizeof(double), s->stream));
  if (s->sponge) {
    if (!u) { gbh_set_error("gb_SourceFunction: null argument"); return GB_ERR_ARG; }
    return add_sponges(s, source, u);
  }
  return GB_OK;
}

extern "C" int gb_FFunction(double* f, double* u, int dir, void* sv, double t) {
  (void)t;
  gb_solver* s = S(sv);
  if (!s || !f || !u || dir < 0 || dir >= s->cfg.ndims) { gbh_set_error("gb_FFunction: bad argument"); return GB_ERR_ARG; }
  CK(launch_unfused(s, 0, dir, f, nullptr, nullptr, nullptr, nullptr, u));
  return GB_OK;
}

extern "C" int gb_GFunction(double* f, double* u, int dir, void* sv, double t) {
  (void)u;
  (void)t;
  gb_solver* s = S(sv);
  if (!s || !f || dir < 0 || dir >= s->cfg.ndims) { gbh_set_error("gb_GFunction: bad argument"); return GB_ERR_ARG; }
  CK(cudaMemsetAsync(f, 0, s->nvals * sizeof(double), s->stream));
  return GB_OK;
}

extern "C" int gb_UFunction(double* uC, double* u, int dir, void* sv, void* m, double t) {
  (void)m;
  (void)t;
  gb_solver* s = S(sv);
  if (!s || !uC || !u) { gbh_set_error("gb_UFunction: bad argument"); return GB_ERR_ARG; }
  if (s->gravity && !s->d_grav) return gravity_ready(s);
  CK(launch_unfused(s, 1, dir < 0 ? 0 : dir, uC, nullptr, nullptr, nullptr, nullptr, u));
  return GB_OK;
}

extern "C" int gb_Upwind(double* fI, double* fL, double* fR, double* uL, double* uR, double* u, int dir, void* sv,
                         double t) {
  (void)t;
  gb_solver* s = S(sv);
  if (!s || !fI || !fL || !fR || !uL || !uR || !u || dir < 0 || dir >= s->cfg.ndims) {
    gbh_set_error("gb_Upwind: bad argument");
    return GB_ERR_ARG;
  }
  if (s->gravity && !s->d_grav) return gravity_ready(s);
  CK(launch_unfused(s, 2, dir, fI, fL, fR, uL, uR, u));
  return GB_OK;
}

// SetInterpLimiterVar (include/hypar.h:234): the reference computes the WENO5
// weights of fC and u here and stores them for the next four
// InterpolateInterfacesHyp calls (HyperbolicFunction.c:201-215, which pass the
// same fC and u); gb_InterpolateInterfacesHyp evaluates them from those arrays
// itself, so this only checks its arguments.
extern "C" int gb_SetInterpLimiterVar(double* fC, double* u, double* x, int dir, void* sv, void* m) {
  (void)x;
  (void)m;
  gb_solver* s = S(sv);
  if (!s || !fC || !u || dir < 0 || dir >= s->cfg.ndims) {
    gbh_set_error("gb_SetInterpLimiterVar: bad argument");
    return GB_ERR_ARG;
  }
  return GB_OK;
}

// InterpolateInterfacesHyp (include/hypar.h:224): WENO5 interface values of fC along
// dir, left-biased for upw > 0, right-biased for upw < 0, with the weights of fC
// (uflag 0) or of u (uflag 1), component-wise or characteristic as configured.
extern "C" int gb_InterpolateInterfacesHyp(double* fI, double* fC, double* u, double* x, int upw, int dir, void* sv,
                                           void* m, int uflag) {
  (void)x;
  (void)m;
  gb_solver* s = S(sv);
  if (!s || !fI || !fC || !u || dir < 0 || dir >= s->cfg.ndims || upw == 0) {
    gbh_set_error("gb_InterpolateInterfacesHyp: bad argument");
    return GB_ERR_ARG;
  }
  if (s->cfg.hyp_scheme != GB_SCHEME_WENO5) {
    gbh_set_error("gb_InterpolateInterfacesHyp: WENO5 only (CRWENO5 runs through the fused kernels)");
    return GB_ERR_UNSUPPORTED;
  }
  const gb_config& c = s->cfg;
  const int chr = c.interp == GB_INTERP_CHARACTERISTIC, left = upw > 0, uf = uflag != 0;
  if (c.model == GB_MODEL_EULER1D) CK(launch_interp_euler1d(dir, chr, left, uf, fI, fC, u, s->G, s->pp, s->stream));
  else if (c.model == GB_MODEL_EULER2D)
    CK(launch_interp_euler2d(dir, chr, left, uf, fI, fC, u, s->G, s->pp, s->stream));
  else CK(launch_interp_ns3d(dir, chr, left, uf, fI, fC, u, s->G, s->pp, s->stream));
  return GB_OK;
}

extern "C" int gb_ApplyBoundaryConditions(void* sv, void* m, double* u, double* uref, double t) {
  (void)m;
  (void)uref;
  gb_solver* s = S(sv);
  if (!s || !u) { gbh_set_error("gb_ApplyBoundaryConditions: null argument"); return GB_ERR_ARG; }
  return apply_mem_bcs(s, u, true, t);
}

extern "C" int gb_RHSFunctionExplicit(double* rhs, double* u, void* sv, void* m, double t) {
  (void)m;
  gb_solver* s = S(sv);
  if (!s || !rhs || !u) { gbh_set_error("gb_RHSFunctionExplicit: null argument"); return GB_ERR_ARG; }
  int rc = apply_mem_bcs(s, u, true, t);  // TimeRHSFunctionExplicit.c:46 fills u's ghosts in place
  if (rc) return rc;
  CK(cudaMemsetAsync(rhs, 0, s->nvals * sizeof(double), s->stream));
  StageEpi ep;
  memset(&ep, 0, sizeof(ep));
  ep.mode = EPI_RHS;
  ep.rhs = rhs;
  std::vector<int> keep;
  keep.swap(s->mem_zones);  // already applied above
  rc = rhs_launches(s, u, ep, t);
  keep.swap(s->mem_zones);
  return rc;
}

extern "C" int gb_TimeRK(void* ts) {
  gb_solver* s = S(ts);
  if (!s) { gbh_set_error("gb_TimeRK: null argument"); return GB_ERR_ARG; }
  int rc = gbh_rk_step(s);
  if (rc) return rc;
  CK(cudaGetLastError());
  return GB_OK;
}
