/*
 * gbhypar_attach.c -- the HyPar-side binding of libgbhypar (see gbhypar_attach.h).
 *
 * Compiled against HyPar's include/ directory (include/hypar.h, boundaryconditions.h,
 * interpolation.h, timeintegration_struct.h, simulation_object.h and the physics-model
 * headers) and linked with libgbhypar.so.  A maintainer calls gbshim_attach() after
 * InitializePhysics (src/Simulation/InitializePhysics.c:84-160) for every simulation,
 * and sets TS->RHSFunction = gbshim_RHSFunction (src/TimeIntegration/TimeInitialize.c:175)
 * or solver->TimeIntegrate = gbshim_TimeRK.
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <basic.h>
#include <boundaryconditions.h>
#include <hypar.h>
#include <interpolation.h>
#include <mpivars_struct.h>
#include <simulation_object.h>
#include <timeintegration_struct.h>

#include "gbhypar_attach.h"

/* The physics models' parameter structs.  Their headers define some of the same
 * macro names with different values (_MODEL_NDIMS_, _MODEL_NVARS_, ...), so each is
 * read by a function of its own with the previous header's names undefined. */
#include <physicalmodels/euler1d.h>
static void read_euler1d(const void *phys, gb_config *c, double *g, int *gtype) {
  const Euler1D *p = (const Euler1D *)phys;
  c->gamma = p->gamma;
  *g = p->grav;
  *gtype = p->grav_type;
}
static const double *euler1d_field(const void *phys) { return ((const Euler1D *)phys)->grav_field; }
static const char *euler1d_upwind(const void *phys) { return ((const Euler1D *)phys)->upw_choice; }
#undef _MODEL_NDIMS_
#undef _MODEL_NVARS_
#undef _XDIR_
#undef _YDIR_
#undef _ROE_
#undef _RF_
#undef _LLF_
#undef _SWFS_
#undef _RUSANOV_
#include <physicalmodels/euler2d.h>
static void read_euler2d(const void *phys, gb_config *c) { c->gamma = ((const Euler2D *)phys)->gamma; }
static const char *euler2d_upwind(const void *phys) { return ((const Euler2D *)phys)->upw_choice; }
#undef _MODEL_NDIMS_
#undef _MODEL_NVARS_
#undef _XDIR_
#undef _YDIR_
#undef _ROE_
#undef _RF_
#undef _LLF_
#undef _SWFS_
#undef _RUSANOV_
#include <physicalmodels/navierstokes3d.h>
static void read_ns3d(const void *phys, gb_config *c) {
  const NavierStokes3D *p = (const NavierStokes3D *)phys;
  c->gamma = p->gamma;
  /* NavierStokes3DInitialize.c:368 stores Re / Minf; gb_config takes physics.inp's Re */
  c->Re = p->Re * p->Minf;
  c->Pr = p->Pr;
  c->Minf = p->Minf;
  c->gravity[0] = p->grav_x;
  c->gravity[1] = p->grav_y;
  c->gravity[2] = p->grav_z;
  c->rho_ref = p->rho0;
  c->p_ref = p->p0;
  c->R_gas = p->R;
  c->HB = p->HB;
  c->N_bv = p->N_bv;
}
static const char *ns3d_upwind(const void *phys) { return ((const NavierStokes3D *)phys)->upw_choice; }
static void ns3d_fields(const void *phys, const double **f, const double **g) {
  *f = ((const NavierStokes3D *)phys)->grav_field_f;
  *g = ((const NavierStokes3D *)phys)->grav_field_g;
}

static int unsupported(const char *what, const char *value) {
  fprintf(stderr, "gbhypar: %s \"%s\" is outside libgbhypar's path\n", what, value);
  return GB_ERR_UNSUPPORTED;
}

int gbshim_config(void *s, gb_config *c) {
  const HyPar *solver = (const HyPar *)s;
  memset(c, 0, sizeof(*c));
  /* the NavierStokes3D parameters' defaults (NavierStokes3DInitialize.c), as the
   * library's reader leaves them for every model */
  c->Re = -1.0;
  c->Pr = 0.72;
  c->Minf = 1.0;
  c->rho_ref = 1.0;
  c->p_ref = 1.0;
  c->R_gas = 1.0;
  const char *upw;
  double g1 = 0.0;
  int gtype = 0;
  if (!strcmp(solver->model, "euler1d")) {
    c->model = GB_MODEL_EULER1D;
    read_euler1d(solver->physics, c, &g1, &gtype);
    c->gravity[0] = g1;
    c->grav_type = gtype;
    upw = euler1d_upwind(solver->physics);
  } else if (!strcmp(solver->model, "euler2d")) {
    c->model = GB_MODEL_EULER2D;
    read_euler2d(solver->physics, c);
    upw = euler2d_upwind(solver->physics);
  } else if (!strcmp(solver->model, "navierstokes3d")) {
    c->model = GB_MODEL_NS3D;
    read_ns3d(solver->physics, c);
    upw = ns3d_upwind(solver->physics);
  } else {
    return unsupported("model", solver->model);
  }
  c->ndims = solver->ndims;
  c->nvars = solver->nvars;
  c->ghosts = solver->ghosts;
  for (int d = 0; d < 3; d++) c->dim[d] = d < solver->ndims ? solver->dim_local[d] : 1;
  if (!strcmp(solver->interp_type, "characteristic")) c->interp = GB_INTERP_CHARACTERISTIC;
  else if (!strcmp(solver->interp_type, "components")) c->interp = GB_INTERP_COMPONENTS;
  else return unsupported("hyp_interp_type", solver->interp_type);
  if (!strcmp(upw, "roe")) c->upwind = GB_UPWIND_ROE;
  else if (!strcmp(upw, "llf-char")) c->upwind = GB_UPWIND_LLF;
  else if (!strcmp(upw, "rf-char")) c->upwind = GB_UPWIND_RF;
  else if (!strcmp(upw, "rusanov")) c->upwind = GB_UPWIND_RUSANOV;
  else if (!strcmp(upw, "steger-warming")) c->upwind = GB_UPWIND_SWFS;
  else return unsupported("upwinding", upw);
  if (!strcmp(solver->spatial_scheme_hyp, "weno5")) c->hyp_scheme = GB_SCHEME_WENO5;
  else if (!strcmp(solver->spatial_scheme_hyp, "crweno5")) c->hyp_scheme = GB_SCHEME_CRWENO5;
  else return unsupported("hyp_space_scheme", solver->spatial_scheme_hyp);
  if (solver->flag_ib) return unsupported("immersed_body", solver->ib_filename);
  /* the viscous term's first derivatives (nonconservative-2stage, InitializeSolvers.c:129-141) */
  if (c->model == GB_MODEL_NS3D && c->Re > 0) {
    if (strcmp(solver->spatial_type_par, "nonconservative-2stage"))
      return unsupported("par_space_type", solver->spatial_type_par);
    if (!strcmp(solver->spatial_scheme_par, "2")) c->par_scheme = 2;
    else if (!strcmp(solver->spatial_scheme_par, "4")) c->par_scheme = 4;
    else return unsupported("par_space_scheme", solver->spatial_scheme_par);
  }

  /* weno.inp, with the reader's precedence: no_limiting > yc > borges > mapped > JS */
  const WENOParameters *w = (const WENOParameters *)solver->interp;
  if (!w) return unsupported("interpolation parameters", "none");
  c->weno_eps = w->eps;
  c->weno_weights = w->no_limiting ? GB_WENO_NONE
                  : w->yc          ? GB_WENO_YC
                  : w->borges      ? GB_WENO_BORGES
                  : w->mapped      ? GB_WENO_MAPPED
                                   : GB_WENO_JS;

  /* boundary zones with their index extents (InitializeBoundaries.c) and values */
  const DomainBoundary *b = (const DomainBoundary *)solver->boundary;
  if (solver->nBoundaryZones > GB_MAX_ZONES) return unsupported("boundary zone count", "> 12");
  c->nzones = solver->nBoundaryZones;
  for (int z = 0; z < c->nzones; z++) {
    const DomainBoundary *B = &b[z];
    static const struct { const char *name; int code; } types[] = {
        {"periodic", GB_BC_PERIODIC},          {"extrapolate", GB_BC_EXTRAPOLATE},
        {"dirichlet", GB_BC_DIRICHLET},        {"slip-wall", GB_BC_SLIP_WALL},
        {"noslip-wall", GB_BC_NOSLIP_WALL},    {"subsonic-inflow", GB_BC_SUBSONIC_INFLOW},
        {"subsonic-outflow", GB_BC_SUBSONIC_OUTFLOW}, {"supersonic-inflow", GB_BC_SUPERSONIC_INFLOW},
        {"supersonic-outflow", GB_BC_SUPERSONIC_OUTFLOW}, {"subsonic-ambivalent", GB_BC_SUBSONIC_AMBIVALENT},
        {"thermal-slip-wall", GB_BC_THERMAL_SLIP_WALL}, {"thermal-noslip-wall", GB_BC_THERMAL_NOSLIP_WALL},
        {"sponge", GB_BC_SPONGE}, {"turbulent-supersonic-inflow", GB_BC_TURBULENT_INFLOW},
        {"reflect", GB_BC_REFLECT}};
    int code = 0;
    for (size_t t = 0; t < sizeof(types) / sizeof(types[0]); t++)
      if (!strcmp(B->bctype, types[t].name)) code = types[t].code;
    if (!code) return unsupported("boundary type", B->bctype);
    int *q = c->zones[z];
    q[0] = code;
    q[1] = B->dim;
    q[2] = B->face;
    for (int d = 0; d < 3; d++) {
      q[3 + d] = d < c->ndims ? B->is[d] : 0;
      q[6 + d] = d < c->ndims ? B->ie[d] : 1;
    }
    double *v = c->zone_data[z];
    int nd = c->ndims;
    switch (code) {
      case GB_BC_DIRICHLET:
        for (int k = 0; k < c->nvars; k++) v[k] = B->DirichletValue[k];
        break;
      case GB_BC_SPONGE:
        for (int k = 0; k < c->nvars; k++) v[k] = B->SpongeValue[k];
        break;
      case GB_BC_SLIP_WALL:
      case GB_BC_NOSLIP_WALL:
      case GB_BC_THERMAL_SLIP_WALL:
      case GB_BC_THERMAL_NOSLIP_WALL:
        for (int k = 0; k < nd; k++) v[k] = B->FlowVelocity[k];
        break;
      case GB_BC_SUBSONIC_INFLOW:
        v[0] = B->FlowDensity;
        for (int k = 0; k < nd; k++) v[1 + k] = B->FlowVelocity[k];
        break;
      case GB_BC_SUBSONIC_OUTFLOW:
        v[0] = B->FlowPressure;
        break;
      case GB_BC_SUPERSONIC_INFLOW:
      case GB_BC_SUBSONIC_AMBIVALENT:
      case GB_BC_TURBULENT_INFLOW:
        v[0] = B->FlowDensity;
        for (int k = 0; k < nd; k++) v[1 + k] = B->FlowVelocity[k];
        v[1 + nd] = B->FlowPressure;
        break;
      default:
        break;
    }
  }

  /* time integration: explicit Runge-Kutta (solver->msti, TimeExplicitRKInitialize), or
   * forward Euler (TimeForwardEuler.c), which is the one-stage table */
  if (!strcmp(solver->time_scheme, "euler")) {
    c->rk_nstages = 1;
    c->rk_A[0] = 0.0;
    c->rk_b[0] = 1.0;
    c->rk_c[0] = 0.0;
  } else {
    if (strcmp(solver->time_scheme, "rk")) return unsupported("time_scheme", solver->time_scheme);
    const ExplicitRKParameters *rk = (const ExplicitRKParameters *)solver->msti;
    if (!rk || rk->nstages < 1 || rk->nstages > 4) return unsupported("time_scheme_type", solver->time_scheme_type);
    c->rk_nstages = rk->nstages;
    for (int i = 0; i < rk->nstages; i++) {
      for (int j = 0; j < rk->nstages; j++) c->rk_A[4 * i + j] = rk->A[i * rk->nstages + j];
      c->rk_b[i] = rk->b[i];
      c->rk_c[i] = rk->c[i];
    }
  }
  c->dt = solver->dt;
  c->n_iter = solver->n_iter;
  c->file_op_iter = solver->file_op_iter;
  c->restart_iter = solver->restart_iter;
  c->screen_op_iter = solver->screen_op_iter > 0 ? solver->screen_op_iter : 1;
  c->write_residual = solver->write_residual;
  c->cons_check = !strcmp(solver->ConservationCheck, "yes");
  return GB_OK;
}

/* HyPar solver -> gb_solver, without a field added to HyPar's struct. */
enum { MAX_ATTACHED = 256 };
static struct { const void *hypar; gb_solver *gb; } attached[MAX_ATTACHED];

gb_solver *gbshim_solver(void *solver) {
  for (int i = 0; i < MAX_ATTACHED; i++)
    if (attached[i].hypar == solver) return attached[i].gb;
  return NULL;
}

static int shim_Hyp(double *h, double *u, void *s, void *m, double t, int lim,
                    int (*F)(double *, double *, int, void *, double),
                    int (*U)(double *, double *, double *, double *, double *, double *, int, void *, double)) {
  (void)F;
  (void)U;
  return gb_HyperbolicFunction(h, u, gbshim_solver(s), m, t, lim, gb_FFunction, gb_Upwind);
}
static int shim_Par(double *p, double *u, void *s, void *m, double t) {
  return gb_ParabolicFunction(p, u, gbshim_solver(s), m, t);
}
static int shim_Src(double *q, double *u, void *s, void *m, double t) {
  return gb_SourceFunction(q, u, gbshim_solver(s), m, t);
}
static int shim_BC(void *s, void *m, double *u, double *ur, double t) {
  return gb_ApplyBoundaryConditions(gbshim_solver(s), m, u, ur, t);
}

int gbshim_RHSFunction(double *rhs, double *u, void *s, void *m, double t) {
  return gb_RHSFunctionExplicit(rhs, u, gbshim_solver(s), m, t);
}

int gbshim_attach(void *s, void *mpi) {
  HyPar *solver = (HyPar *)s;
  gb_config c;
  int rc = gbshim_config(solver, &c);
  if (rc) return rc;
  int slot = -1;
  for (int i = 0; i < MAX_ATTACHED && slot < 0; i++)
    if (!attached[i].hypar || attached[i].hypar == solver) slot = i;
  if (slot < 0) {
    fprintf(stderr, "gbhypar: more than %d solvers attached\n", MAX_ATTACHED);
    return GB_ERR_ARG;
  }
  if (attached[slot].gb) gbshim_detach(solver);
  int device = 0;
#if defined(HAVE_CUDA)
  device = solver->gpu_device_no;
#endif
  gb_solver *gb = NULL;
  rc = gb_solver_create(&c, solver->dxinv, device, &gb);
  if (rc) {
    fprintf(stderr, "gbhypar: %s\n", gb_last_error());
    return rc;
  }
  /* gravity fields, host arrays with ghosts: f then g (NavierStokes3D), 1/S then S (Euler1D) */
  const long n = solver->npoints_local_wghosts;
  double *fg = NULL;
  if (c.model == GB_MODEL_NS3D && (c.gravity[0] != 0.0 || c.gravity[1] != 0.0 || c.gravity[2] != 0.0)) {
    const double *f, *g;
    ns3d_fields(solver->physics, &f, &g);
    fg = (double *)malloc(sizeof(double) * 2 * n);
    if (fg) {
      memcpy(fg, f, sizeof(double) * n);
      memcpy(fg + n, g, sizeof(double) * n);
    }
  } else if (c.model == GB_MODEL_EULER1D && c.gravity[0] != 0.0) {
    const double *S = euler1d_field(solver->physics);
    fg = (double *)malloc(sizeof(double) * 2 * n);
    if (fg)
      for (long i = 0; i < n; i++) {
        fg[i] = 1.0 / S[i];
        fg[n + i] = S[i];
      }
  }
  if (fg) {
    rc = gb_solver_set_gravity_field(gb, fg);
    free(fg);
    if (rc) {
      fprintf(stderr, "gbhypar: %s\n", gb_last_error());
      gb_solver_destroy(gb);
      return rc;
    }
  }
  /* thermal walls: the wall temperature HyPar read (BCReadTemperatureData), time levels
   * and field over the zone's extent */
  for (int z = 0; z < c.nzones; z++) {
    const DomainBoundary *B = &((const DomainBoundary *)solver->boundary)[z];
    if (c.zones[z][0] != GB_BC_THERMAL_SLIP_WALL && c.zones[z][0] != GB_BC_THERMAL_NOSLIP_WALL) continue;
    rc = gb_solver_set_zone_temperature(gb, z, B->UnsteadyTemperatureSize[B->dim], B->UnsteadyTimeLevels,
                                        B->UnsteadyTemperatureData);
    if (rc) {
      fprintf(stderr, "gbhypar: %s\n", gb_last_error());
      gb_solver_destroy(gb);
      return rc;
    }
  }
  /* turbulent inflow zones: the inflow data HyPar read (BCReadTurbulentInflowData) */
  for (int z = 0; z < c.nzones; z++) {
    const DomainBoundary *B = &((const DomainBoundary *)solver->boundary)[z];
    if (c.zones[z][0] != GB_BC_TURBULENT_INFLOW || !B->UnsteadyDirichletData) continue;
    rc = gb_solver_set_zone_inflow(gb, z, B->UnsteadyDirichletSize[B->dim], B->UnsteadyDirichletData);
    if (rc) {
      fprintf(stderr, "gbhypar: %s\n", gb_last_error());
      gb_solver_destroy(gb);
      return rc;
    }
  }
  /* sponge zones: sigma over the zone's indices along its dimension, from HyPar's grid
   * (solver->x, ghost points included) and the zone's bounds (BCSponge.c:49-54) */
  for (int z = 0; z < c.nzones; z++) {
    const DomainBoundary *B = &((const DomainBoundary *)solver->boundary)[z];
    if (c.zones[z][0] != GB_BC_SPONGE || !B->on_this_proc) continue;
    const int dim = B->dim, n = B->ie[dim] - B->is[dim];
    if (n <= 0) continue;
    int off = 0;
    for (int d = 0; d < dim; d++) off += solver->dim_local[d] + 2 * solver->ghosts;
    double *sigma = (double *)malloc(sizeof(double) * n);
    if (!sigma) {
      gb_solver_destroy(gb);
      return GB_ERR_NOMEM;
    }
    const double xs = B->xmin[dim], xe = B->xmax[dim];
    for (int k = 0; k < n; k++) {
      const double x = solver->x[off + solver->ghosts + B->is[dim] + k];
      sigma[k] = B->face > 0 ? (x - xs) / (xe - xs) : (x - xe) / (xs - xe);
    }
    rc = gb_solver_set_zone_sponge(gb, z, sigma);
    free(sigma);
    if (rc) {
      fprintf(stderr, "gbhypar: %s\n", gb_last_error());
      gb_solver_destroy(gb);
      return rc;
    }
  }
  /* the fused step calls the physics model's PostStage on every stage state; HyPar's
   * own TimePreStep / TimePostStep keep calling PreStep / PostStep */
  rc = gb_solver_set_hooks(gb, NULL, solver->PostStage, NULL, NULL, solver, mpi);
  if (rc) {
    fprintf(stderr, "gbhypar: %s\n", gb_last_error());
    gb_solver_destroy(gb);
    return rc;
  }
  attached[slot].hypar = solver;
  attached[slot].gb = gb;
  solver->HyperbolicFunction = shim_Hyp;
  solver->ParabolicFunction = shim_Par;
  solver->SourceFunction = shim_Src;
  solver->ApplyBoundaryConditions = shim_BC;
  return GB_OK;
}

void gbshim_detach(void *solver) {
  for (int i = 0; i < MAX_ATTACHED; i++)
    if (attached[i].hypar == solver) {
      gb_solver_destroy(attached[i].gb);
      attached[i].hypar = NULL;
      attached[i].gb = NULL;
    }
}

int gbshim_TimeRK(void *ts) {
  TimeIntegration *TS = (TimeIntegration *)ts;
  SimulationObject *sim = (SimulationObject *)TS->simulation;
  for (int ns = 0; ns < TS->nsims; ns++) {
    HyPar *solver = &sim[ns].solver;
    gb_solver *gb = gbshim_solver(solver);
    if (!gb) {
      fprintf(stderr, "gbhypar: simulation %d has no attached solver (gbshim_attach)\n", ns);
      return GB_ERR_ARG;
    }
    /* the solution: HyPar's device copy in a CUDA build, its host array otherwise */
    double *u = solver->u;
    int mem = GB_MEM_HOST;
#if defined(HAVE_CUDA)
    if (solver->use_gpu) {
      u = solver->gpu_u;
      mem = GB_MEM_DEVICE;
    }
#endif
    int rc = gb_solver_set_state(gb, u, GB_LAYOUT_GHOSTED, mem);
    if (!rc) rc = gb_solver_set_time(gb, TS->waqt);
    if (!rc) rc = gb_TimeRK(gb);
    if (!rc) rc = gb_solver_get_state(gb, u, GB_LAYOUT_GHOSTED, mem);
    if (rc) {
      fprintf(stderr, "gbhypar: %s\n", gb_last_error());
      return rc;
    }
  }
  return GB_OK;
}
