/*
 * gbh_oracle.c -- CPU restatement of HyPar's explicit WENO5 RHS and RK step.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the parity checker for the CUDA
 * product and the timed CPU baseline; it is never linked into libgbhypar.
 *
 * It restates the reference's formulas in the reference's operation order and
 * must be compiled with -ffp-contract=off (no fused multiply-add), like the
 * reference's own -std=c99 build, so that it reproduces the reference CPU
 * results bit for bit.  Each routine cites the reference file:line it follows
 * (paths relative to the HyPar source tree).
 *
 * Organisation differs from the reference where that changes no value: the
 * reference stores WENO weights for the whole grid (WENOInitialize.c:135-205)
 * and interface arrays per dimension; here each grid line is processed on its
 * own (OpenMP over lines), computing every weight exactly where it is used.
 */
#include "gbh_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define MAXV 5

static int g_threads = 0;
void orc_set_threads(int n) { g_threads = n; }
int orc_get_threads(void) {
#ifdef _OPENMP
  return g_threads > 0 ? g_threads : omp_get_max_threads();
#else
  return 1;
#endif
}
#ifdef _OPENMP
#define NTHR (g_threads > 0 ? g_threads : omp_get_max_threads())
#endif

/* ------------------------------------------------------------------------ */
/* problem set-up                                                            */
/* ------------------------------------------------------------------------ */

orc_problem *orc_problem_create(int model, int ndims, const int *dim, int ghosts,
                                int upwind, int interp, double gamma, double eps,
                                double Re_over_Minf, double Pr, int nzones,
                                const int *zones, const double *dxinv) {
  if (ndims < 1 || ndims > 3 || nzones < 0 || nzones > 12) return NULL;
  orc_problem *p = (orc_problem *)calloc(1, sizeof(orc_problem));
  p->model = model;
  p->ndims = ndims;
  p->nvars = (model == ORC_EULER1D) ? 3 : (model == ORC_EULER2D ? 4 : 5);
  p->ghosts = ghosts;
  for (int d = 0; d < 3; d++) p->dim[d] = (d < ndims) ? dim[d] : 1;
  p->upwind = upwind;
  p->interp = interp;
  p->gamma = gamma;
  p->eps = eps;
  p->Re = Re_over_Minf;
  p->Pr = Pr;
  p->nzones = nzones;
  for (int z = 0; z < nzones; z++) {
    const int *q = zones + 9 * z;
    p->zones[z].type = q[0];
    p->zones[z].dim = q[1];
    p->zones[z].face = q[2];
    for (int d = 0; d < 3; d++) {
      p->zones[z].is[d] = q[3 + d];
      p->zones[z].ie[d] = q[6 + d];
    }
  }
  int nx = 0;
  for (int d = 0; d < ndims; d++) nx += dim[d] + 2 * ghosts;
  p->dxinv = (double *)malloc(sizeof(double) * nx);
  memcpy(p->dxinv, dxinv, sizeof(double) * nx);
  return p;
}

void orc_set_weights(orc_problem *p, int weights) { p->weights = weights; }
void orc_set_scheme(orc_problem *p, int scheme) { p->scheme = scheme; }

static void strides_wg(const orc_problem *p, long *s);
static long pidx(const orc_problem *p, const long *s, const int *i);

/* NavierStokes3DGravityField (NavierStokes3DGravityField.c:36-153): the
 * hydrostatic density / pressure variations f, g from the coordinates (ghost
 * coordinates included), then every face's ghost layer copied from its mirror
 * interior points.  raiseto(x, a) = exp(a log x) (include/math_ops.h:37). */
int orc_set_gravity(orc_problem *p, const double *xg, double gx, double gy, double gz, double rho0, double p0,
                    double R, int HB, double Nbv) {
  if (p->model != ORC_NS3D) return 1;
  long np = orc_npoints_wghosts(p);
  long s[3];
  strides_wg(p, s);
  int g = p->ghosts, *dim = p->dim;
  free(p->gf);
  free(p->gg);
  p->gf = (double *)malloc(sizeof(double) * np);
  p->gg = (double *)malloc(sizeof(double) * np);
  p->grav[0] = gx;
  p->grav[1] = gy;
  p->grav[2] = gz;
  p->RT = p0 / rho0;
  p->has_grav = (gx != 0.0) || (gy != 0.0) || (gz != 0.0);
  double RT = p0 / rho0, gamma = p->gamma;
  double Cp = gamma * R / (gamma - 1.0);
  double T0 = p0 / (rho0 * R);
  long off[3] = {0, dim[0] + 2 * g, dim[0] + 2 * g + dim[1] + 2 * g};
  for (int k = 0; k < dim[2] + 2 * g; k++)
    for (int j = 0; j < dim[1] + 2 * g; j++)
      for (int i = 0; i < dim[0] + 2 * g; i++) {
        long q = i * s[0] + j * s[1] + k * s[2];
        double x = xg[off[0] + i], y = xg[off[1] + j], z = xg[off[2] + k];
        double f, gv;
        if (HB == 1) {
          f = exp((gx * x + gy * y + gz * z) / RT);
          gv = exp(-(gx * x + gy * y + gz * z) / RT);
        } else if (HB == 2) {
          f = exp((-1.0 / (gamma - 1.0)) * log((1.0 - (gx * x + gy * y + gz * z) / (Cp * T0))));
          gv = exp((gamma / (gamma - 1.0)) * log((1.0 - (gx * x + gy * y + gz * z) / (Cp * T0))));
        } else if (HB == 3) {
          if (gx != 0 || gy != 0) return 1;
          double Pexner = 1 + ((gz * gz) / (Cp * T0 * Nbv * Nbv)) * (exp(-(Nbv * Nbv / gz) * z) - 1.0);
          f = exp((-1.0 / (gamma - 1.0)) * log(Pexner)) * exp(Nbv * Nbv * z / gz);
          gv = exp((gamma / (gamma - 1.0)) * log(Pexner));
        } else {
          f = gv = 1.0;
        }
        p->gf[q] = f;
        p->gg[q] = gv;
      }
  /* ghost layers of each face from the mirror interior points, over the
     interior transverse range (the reference's loops) */
  for (int d = 0; d < 3; d++) {
    for (int side = 0; side < 2; side++) {
      int b[3] = {dim[0], dim[1], dim[2]};
      b[d] = g;
      for (int c2 = 0; c2 < b[2]; c2++)
        for (int c1 = 0; c1 < b[1]; c1++)
          for (int c0 = 0; c0 < b[0]; c0++) {
            int ib[3] = {c0, c1, c2}, gi[3], ii[3];
            for (int e = 0; e < 3; e++) gi[e] = ii[e] = ib[e];
            if (side == 0) {
              gi[d] = ib[d] - g;
              ii[d] = g - 1 - ib[d];
            } else {
              gi[d] = dim[d] + ib[d];
              ii[d] = dim[d] - 1 - ib[d];
            }
            long q1 = pidx(p, s, gi), q2 = pidx(p, s, ii);
            p->gf[q1] = p->gf[q2];
            p->gg[q1] = p->gg[q2];
          }
    }
  }
  return 0;
}

/* Euler1DGravityField (Euler1DGravityField.c:23-95): S = exp(-g x) (type 0) or
 * exp(-phi), phi = -sin(2 pi x)/(2 pi) (type 1), at every point with ghosts from the
 * ghost-extrapolated grid; for type 0 the ghost layers copied from their mirror
 * interior points.  Stored as gg = S and gf = 1.0 / S (the modified solution and the
 * source scale by the latter, Euler1DModifiedSolution.c:48, Euler1DSource.c:71). */
int orc_set_gravity_1d(orc_problem *p, const double *xg, double g, int type) {
  if (p->model != ORC_EULER1D) return 1;
  long np = orc_npoints_wghosts(p);
  int gh = p->ghosts, N = p->dim[0];
  free(p->gf);
  free(p->gg);
  p->gf = (double *)malloc(sizeof(double) * np);
  p->gg = (double *)malloc(sizeof(double) * np);
  for (long i = 0; i < np; i++) {
    double x = xg[i];
    if (type == 0) {
      p->gg[i] = exp(-g * x);
    } else if (type == 1) {
      double pi = 4.0 * atan(1.0);
      double phi = -sin(2 * pi * x) / (2 * pi);
      p->gg[i] = exp(-phi);
    } else {
      return 1;
    }
  }
  if (type != 1)
    for (int b = 0; b < gh; b++) {
      p->gg[b] = p->gg[gh + (gh - 1 - b)];
      p->gg[N + gh + b] = p->gg[gh + (N - 1 - b)];
    }
  for (long i = 0; i < np; i++) p->gf[i] = 1.0 / p->gg[i];
  p->grav[0] = g;
  p->grav[1] = p->grav[2] = 0.0;
  p->RT = 1.0;
  p->has_grav = g != 0.0;
  return 0;
}

/* f then g (each with ghost points); zeros when no field is set */
void orc_get_gravity(const orc_problem *p, double *out) {
  long np = orc_npoints_wghosts(p);
  for (long q = 0; q < np; q++) {
    out[q] = p->gf ? p->gf[q] : 0.0;
    out[np + q] = p->gg ? p->gg[q] : 0.0;
  }
}

void orc_set_zone_data(orc_problem *p, int z, const double *data) {
  if (z < 0 || z >= p->nzones) return;
  for (int k = 0; k < 8; k++) p->zones[z].data[k] = data[k];
}

int orc_set_zone_temperature(orc_problem *p, int z, int n, const double *times, const double *field) {
  if (z < 0 || z >= p->nzones || n < 1) return 1;
  const orc_zone *b = &p->zones[z];
  long size = n;
  for (int d = 0; d < p->ndims; d++)
    if (d != b->dim) size *= (b->ie[d] - b->is[d]);
  free(p->ttimes[z]);
  free(p->tfield[z]);
  p->tn[z] = n;
  p->ttimes[z] = (double *)malloc(sizeof(double) * n);
  p->tfield[z] = (double *)malloc(sizeof(double) * size);
  memcpy(p->ttimes[z], times, sizeof(double) * n);
  memcpy(p->tfield[z], field, sizeof(double) * size);
  return 0;
}

void orc_set_time(orc_problem *p, double t) { p->t = t; }

int orc_set_zone_inflow(orc_problem *p, int z, int n, const double *data) {
  if (z < 0 || z >= p->nzones || p->zones[z].type != ORC_BC_TURBULENT_INFLOW || n < 1) return 1;
  long cnt = (long)n * p->nvars;
  for (int d = 0; d < p->ndims; d++)
    if (d != p->zones[z].dim) cnt *= p->dim[d];
  free(p->fdata[z]);
  p->fdata[z] = (double *)malloc(sizeof(double) * cnt);
  memcpy(p->fdata[z], data, sizeof(double) * cnt);
  p->fn[z] = n;
  return 0;
}

int orc_set_zone_sponge(orc_problem *p, int z, const double *x, double xmin, double xmax) {
  if (z < 0 || z >= p->nzones || p->zones[z].type != ORC_BC_SPONGE) return 1;
  const int n = p->dim[p->zones[z].dim];
  free(p->sx[z]);
  p->sx[z] = (double *)malloc(sizeof(double) * n);
  memcpy(p->sx[z], x, sizeof(double) * n);
  p->sxmin[z] = xmin;
  p->sxmax[z] = xmax;
  return 0;
}

/* BCSpongeSource (src/BoundaryConditions/BCSponge.c:34-61) for every sponge zone, in
 * zone order (SourceFunction.c:63-76): over the zone's interior points,
 * src -= sigma (u - u_ref), sigma = (x - x_start) / (x_end - x_start) on face +1 and
 * (x - x_end) / (x_start - x_end) on face -1. */
static int sponge_source(const orc_problem *p, const double *u, double *src) {
  long s[3];
  strides_wg(p, s);
  const int nd = p->ndims, nv = p->nvars;
  for (int z = 0; z < p->nzones; z++) {
    const orc_zone *b = &p->zones[z];
    if (b->type != ORC_BC_SPONGE) continue;
    int bounds[3] = {1, 1, 1}, ib[3] = {0, 0, 0};
    long count = 1;
    for (int d = 0; d < nd; d++) {
      bounds[d] = b->ie[d] - b->is[d];
      count *= (bounds[d] > 0 ? bounds[d] : 0);
    }
    if (!count) continue;
    if (!p->sx[z]) return 1;
    for (long c = 0; c < count; c++) {
      long r = c;
      int ig[3] = {0, 0, 0};
      for (int d = 0; d < nd; d++) {
        ib[d] = (int)(r % bounds[d]);
        r /= bounds[d];
        ig[d] = ib[d] + b->is[d];
      }
      const double x = p->sx[z][ig[b->dim]], xs = p->sxmin[z], xe = p->sxmax[z];
      double sigma;
      if (b->face > 0) sigma = (x - xs) / (xe - xs);
      else sigma = (x - xe) / (xs - xe);
      const long q = pidx(p, s, ig);
      for (int v = 0; v < nv; v++) src[nv * q + v] -= (sigma * (u[nv * q + v] - b->data[v]));
    }
  }
  return 0;
}

void orc_problem_destroy(orc_problem *p) {
  if (!p) return;
  for (int z = 0; z < 12; z++) {
    free(p->ttimes[z]);
    free(p->tfield[z]);
    free(p->sx[z]);
    free(p->fdata[z]);
  }
  free(p->gf);
  free(p->gg);
  free(p->dxinv);
  free(p);
}

long orc_npoints_wghosts(const orc_problem *p) {
  long n = 1;
  for (int d = 0; d < p->ndims; d++) n *= (p->dim[d] + 2 * p->ghosts);
  return n;
}

static void strides_wg(const orc_problem *p, long *s) {
  s[0] = 1;
  for (int d = 1; d < 3; d++)
    s[d] = (d < p->ndims) ? s[d - 1] * (p->dim[d - 1] + 2 * p->ghosts) : 0;
}

/* 1-D point index of an interior-relative multi-index (include/arrayfunctions.h:40-47). */
static long pidx(const orc_problem *p, const long *s, const int *i) {
  long q = 0;
  for (int d = 0; d < p->ndims; d++) q += (long)(i[d] + p->ghosts) * s[d];
  return q;
}

/* ------------------------------------------------------------------------ */
/* boundary conditions                                                       */
/* ------------------------------------------------------------------------ */

/* BCPeriodicU (src/BoundaryConditions/BCPeriodic.c:36-56, single rank along dim)
 * and BCExtrapolateU (src/BoundaryConditions/BCExtrapolate.c:29-46, a mirror copy). */
/* Ghost state of the wall and inflow / outflow types from the mirror interior
 * state w, 2-D (Euler2D/NavierStokes2D flow variables) and 3-D branches of
 * BCSlipWall.c, BCNoslipWall.c, BCSubsonicInflow.c, BCSubsonicOutflow.c,
 * BCSupersonicInflow.c, BCSupersonicOutflow.c and BCSubsonicAmbivalent.c (which
 * takes inflow's or outflow's rule by `inflow`, the sign of the extrapolated face
 * velocity along the inward normal). */
static int bc_ghost(const orc_zone *b, int nd, double gamma, const double *w, double *out, int inflow,
                    double Tb) {
  double inv_gamma_m1 = 1.0 / (gamma - 1.0);
  double rho = 0, vel[3] = {0, 0, 0}, energy, pressure = 0, vsq;
  if (nd == 1) {
    /* BCSlipWall.c:38-76, the 1-D branch (Euler1D flow variables, euler1d.h:81-88) */
    if (b->type != ORC_BC_SLIP_WALL) return 1;
    rho = w[0];
    vel[0] = w[1] / rho;
    pressure = (w[2] - 0.5 * rho * vel[0] * vel[0]) * (gamma - 1.0);
    const double ug = 2.0 * b->data[0] - vel[0];
    out[0] = rho;
    out[1] = rho * ug;
    out[2] = inv_gamma_m1 * pressure + 0.5 * rho * ug * ug;
    return 0;
  }
  if (b->type != ORC_BC_SUPERSONIC_INFLOW) {
    rho = w[0];
    if (nd == 2) {
      vel[0] = w[1] / rho;
      vel[1] = w[2] / rho;
      energy = w[3];
      vsq = (vel[0] * vel[0]) + (vel[1] * vel[1]);
    } else {
      vel[0] = (rho == 0) ? 0 : w[1] / rho;
      vel[1] = (rho == 0) ? 0 : w[2] / rho;
      vel[2] = (rho == 0) ? 0 : w[3] / rho;
      energy = w[4];
      vsq = vel[0] * vel[0] + vel[1] * vel[1] + vel[2] * vel[2];
    }
    pressure = (energy - 0.5 * rho * vsq) * (gamma - 1.0);
  }
  double rho_g = rho, v_g[3] = {vel[0], vel[1], vel[2]}, p_g = pressure;
  switch (b->type) {
    case ORC_BC_SLIP_WALL: v_g[b->dim] = 2.0 * b->data[b->dim] - vel[b->dim]; break;
    case ORC_BC_NOSLIP_WALL:
      for (int d = 0; d < nd; d++) v_g[d] = 2.0 * b->data[d] - vel[d];
      break;
    case ORC_BC_SUBSONIC_INFLOW:
      rho_g = b->data[0];
      for (int d = 0; d < nd; d++) v_g[d] = b->data[1 + d];
      break;
    case ORC_BC_SUBSONIC_OUTFLOW: p_g = b->data[0]; break;
    case ORC_BC_SUPERSONIC_INFLOW:
      rho_g = b->data[0];
      for (int d = 0; d < nd; d++) v_g[d] = b->data[1 + d];
      p_g = b->data[1 + nd];
      break;
    case ORC_BC_SUPERSONIC_OUTFLOW: break;
    case ORC_BC_THERMAL_SLIP_WALL:
      /* BCThermalSlipWall.c:86-105 (3-D): the normal velocity mirrored about the wall's,
       * the pressure from the extrapolated density and the wall temperature */
      v_g[b->dim] = 2.0 * b->data[b->dim] - vel[b->dim];
      p_g = rho_g * Tb;
      break;
    case ORC_BC_THERMAL_NOSLIP_WALL:
      /* BCThermalNoslipWall.c:86-105 (3-D): every velocity component mirrored */
      for (int d = 0; d < nd; d++) v_g[d] = 2.0 * b->data[d] - vel[d];
      p_g = rho_g * Tb;
      break;
    case ORC_BC_SUBSONIC_AMBIVALENT:
      /* BCSubsonicAmbivalent.c:105-117: inflow takes density and velocity, outflow the
       * pressure (data: rho, velocity, pressure) */
      if (inflow) {
        rho_g = b->data[0];
        for (int d = 0; d < nd; d++) v_g[d] = b->data[1 + d];
      } else {
        p_g = b->data[1 + nd];
      }
      break;
    default: return 1;
  }
  double e_g;
  if (nd == 2) e_g = inv_gamma_m1 * p_g + 0.5 * rho_g * (v_g[0] * v_g[0] + v_g[1] * v_g[1]);
  else e_g = inv_gamma_m1 * p_g + 0.5 * rho_g * (v_g[0] * v_g[0] + v_g[1] * v_g[1] + v_g[2] * v_g[2]);
  out[0] = rho_g;
  for (int d = 0; d < nd; d++) out[1 + d] = rho_g * v_g[d];
  out[nd + 1] = e_g;
  return 0;
}

static int apply_bc_at(const orc_problem *p, double *u, double t) {
  long s[3];
  strides_wg(p, s);
  int nd = p->ndims, nv = p->nvars, g = p->ghosts;
  for (int z = 0; z < p->nzones; z++) {
    const orc_zone *b = &p->zones[z];
    if (b->type == ORC_BC_SPONGE) continue; /* a source term (BCSpongeUDummy) */
    int bounds[3] = {1, 1, 1}, ib[3] = {0, 0, 0};
    long count = 1;
    for (int d = 0; d < nd; d++) {
      bounds[d] = b->ie[d] - b->is[d];
      if (bounds[d] <= 0) count = 0;
      count *= (bounds[d] > 0 ? bounds[d] : 0);
    }
    if (!count) continue;
    /* thermal walls: the time level in use, the last one at or before t
     * (BCThermalNoslipWall.c:55-57) */
    int it = 0;
    if (b->type == ORC_BC_THERMAL_SLIP_WALL || b->type == ORC_BC_THERMAL_NOSLIP_WALL) {
      if (!p->tn[z]) return 1;
      it = p->tn[z] - 1;
      while (p->ttimes[z][it] > t && it > 0) it--;
    }
    if (b->type == ORC_BC_TURBULENT_INFLOW) {
      /* BCTurbulentSupersonicInflow.c:44-48: the slice the mean flow carried in by t,
       * the data spanning a length of 2 pi */
      if (!p->fn[z] || nd != 3) return 1;
      double xt = b->data[1 + b->dim] * t;
      int N = p->fn[z];
      double L = 2.0 * (4.0 * atan(1.0));
      it = ((int)((xt / L) * ((double)N))) % N;
      if (it < 0) return 1; /* the reference would read outside its data */
    }
    for (long c = 0; c < count; c++) {
      long r = c;
      for (int d = 0; d < nd; d++) { ib[d] = (int)(r % bounds[d]); r /= bounds[d]; }
      int ig[3], isrc[3];
      for (int d = 0; d < nd; d++) { ig[d] = ib[d] + b->is[d]; isrc[d] = ig[d]; }
      int dd = b->dim, N = p->dim[dd];
      if (b->type == ORC_BC_PERIODIC) {
        if (b->face == 1) isrc[dd] = ib[dd] + N - g;
        else isrc[dd] = ib[dd];
      } else {
        /* extrapolate and the wall / inflow / outflow types read the mirror point */
        if (b->face == 1) isrc[dd] = g - 1 - ib[dd];
        else isrc[dd] = N - ib[dd] - 1;
      }
      long p1 = pidx(p, s, ig), p2 = pidx(p, s, isrc);
      if (b->type == ORC_BC_PERIODIC || b->type == ORC_BC_EXTRAPOLATE) {
        for (int v = 0; v < nv; v++) u[nv * p1 + v] = u[nv * p2 + v];
      } else if (b->type == ORC_BC_REFLECT) {
        /* BCReflectU (BCReflect.c:22-44): the mirror point scaled by -1 */
        for (int v = 0; v < nv; v++) u[nv * p1 + v] = -1.0 * u[nv * p2 + v];
      } else if (b->type == ORC_BC_DIRICHLET) {
        /* BCDirichletU (BCDirichlet.c:27-41) */
        for (int v = 0; v < nv; v++) u[nv * p1 + v] = b->data[v];
      } else if (b->type == ORC_BC_TURBULENT_INFLOW) {
        /* BCTurbulentSupersonicInflowU (BCTurbulentSupersonicInflow.c:54-85): the mean
         * supersonic inflow plus the velocity fluctuations of slice `it` at the zone-
         * relative transverse indices */
        int index1[3] = {ib[0], ib[1], ib[2]};
        index1[dd] = it;
        long q = 0, stride = 1;
        for (int d = 0; d < nd; d++) {
          q += stride * index1[d];
          stride *= (d == dd ? p->fn[z] : p->dim[d]);
        }
        const double *fl = p->fdata[z] + q * nv;
        double inv_gamma_m1 = 1.0 / (p->gamma - 1.0);
        double rho_gpt = b->data[0], pressure_gpt = b->data[4];
        double uvel_gpt = b->data[1], vvel_gpt = b->data[2], wvel_gpt = b->data[3];
        uvel_gpt += fl[1];
        vvel_gpt += fl[2];
        wvel_gpt += fl[3];
        double energy_gpt = inv_gamma_m1 * pressure_gpt +
                            0.5 * rho_gpt * (uvel_gpt * uvel_gpt + vvel_gpt * vvel_gpt + wvel_gpt * wvel_gpt);
        u[nv * p1 + 0] = rho_gpt;
        u[nv * p1 + 1] = rho_gpt * uvel_gpt;
        u[nv * p1 + 2] = rho_gpt * vvel_gpt;
        u[nv * p1 + 3] = rho_gpt * wvel_gpt;
        u[nv * p1 + 4] = energy_gpt;
      } else if (nd == 2 || nd == 3) {
        int inflow = 0;
        if (b->type == ORC_BC_SUBSONIC_AMBIVALENT) {
          /* BCSubsonicAmbivalent.c:70-92: the face velocity extrapolated (second order)
           * from the boundary cell and its neighbour at this transverse position,
           * 1.5 v_1 - 0.5 v_2, projected on the inward normal face * e_dim */
          int i1[3], i2[3];
          for (int d = 0; d < nd; d++) i1[d] = i2[d] = ig[d];
          i1[dd] = b->face == 1 ? 0 : N - 1;
          i2[dd] = b->face == 1 ? 1 : N - 2;
          const double *w1 = u + nv * pidx(p, s, i1), *w2 = u + nv * pidx(p, s, i2);
          double vb[3] = {0, 0, 0}, vn = 0.0;
          for (int d = 0; d < nd; d++) {
            double v1 = (nd == 3 && w1[0] == 0) ? 0 : w1[1 + d] / w1[0];
            double v2 = (nd == 3 && w2[0] == 0) ? 0 : w2[1 + d] / w2[0];
            vb[d] = 1.5 * v1 - 0.5 * v2;
          }
          for (int d = 0; d < nd; d++) vn = vn + vb[d] * (d == dd ? (double)b->face : 0.0);
          inflow = vn > 0;
        }
        double Tb = 0.0;
        if (b->type == ORC_BC_THERMAL_SLIP_WALL || b->type == ORC_BC_THERMAL_NOSLIP_WALL) {
          /* the field index of this point: zone-relative indices, the time level along dim */
          long q = 0, stride = 1;
          for (int d = 0; d < nd; d++) {
            q += stride * (d == dd ? it : ib[d]);
            stride *= (d == dd ? p->tn[z] : bounds[d]);
          }
          Tb = p->tfield[z][q];
        }
        if (bc_ghost(b, nd, p->gamma, u + nv * p2, u + nv * p1, inflow, Tb)) return 1;
      } else if (b->type == ORC_BC_SLIP_WALL) {
        /* the 1-D slip wall */
        if (bc_ghost(b, nd, p->gamma, u + nv * p2, u + nv * p1, 0, 0.0)) return 1;
      } else {
        return 1;
      }
    }
  }
  return 0;
}


int orc_apply_bc(const orc_problem *p, double *u) { return apply_bc_at(p, u, p->t); }

/* ------------------------------------------------------------------------ */
/* physical models: flux, Roe average, eigen-structure                        */
/* ------------------------------------------------------------------------ */

/* Euler1D -- include/physicalmodels/euler1d.h:81-270 */
static void e1_flux(double *f, const double *u, double gamma) {
  double rho = u[0], v = u[1] / rho, e = u[2];
  double P = (e - 0.5 * rho * v * v) * (gamma - 1.0);
  f[0] = rho * v;
  f[1] = rho * v * v + P;
  f[2] = (e + P) * v;
}
static void e1_roeavg(double *ua, const double *uL, const double *uR, double gamma) {
  double rhoL = uL[0], vL = uL[1] / rhoL, eL = uL[2];
  double PL = (eL - 0.5 * rhoL * vL * vL) * (gamma - 1.0);
  double cLsq = gamma * PL / rhoL;
  double HL = 0.5 * vL * vL + cLsq / (gamma - 1.0);
  double rhoR = uR[0], vR = uR[1] / rhoR, eR = uR[2];
  double PR = (eR - 0.5 * rhoR * vR * vR) * (gamma - 1.0);
  double cRsq = gamma * PR / rhoR;
  double HR = 0.5 * vR * vR + cRsq / (gamma - 1.0);
  double tL = sqrt(rhoL), tR = sqrt(rhoR);
  double rho = tL * tR;
  double v = (tL * vL + tR * vR) / (tL + tR);
  double H = (tL * HL + tR * HR) / (tL + tR);
  double csq = (gamma - 1.0) * (H - 0.5 * v * v);
  double P = csq * rho / gamma;
  double e = P / (gamma - 1.0) + 0.5 * rho * v * v;
  ua[0] = rho;
  ua[1] = rho * v;
  ua[2] = e;
}
static void e1_eig(double *D, const double *u, double gamma) {
  double rho = u[0], v = u[1] / rho, e = u[2];
  double P = (e - 0.5 * rho * v * v) * (gamma - 1.0);
  double c = sqrt(gamma * P / rho);
  D[0] = v;
  D[1] = (v - c);
  D[2] = (v + c);
}
static void e1_left(double *L, const double *u, double gamma) {
  double rho = u[0], v = u[1] / rho, e = u[2];
  double P = (e - 0.5 * rho * v * v) * (gamma - 1.0);
  double c = sqrt(gamma * P / rho);
  L[1 * 3 + 0] = ((gamma - 1) / (rho * c)) * (-(v * v) / 2 - c * v / (gamma - 1));
  L[1 * 3 + 1] = ((gamma - 1) / (rho * c)) * (v + c / (gamma - 1));
  L[1 * 3 + 2] = ((gamma - 1) / (rho * c)) * (-1);
  L[0 * 3 + 0] = ((gamma - 1) / (rho * c)) * (rho * (-(v * v) / 2 + c * c / (gamma - 1)) / c);
  L[0 * 3 + 1] = ((gamma - 1) / (rho * c)) * (rho * v / c);
  L[0 * 3 + 2] = ((gamma - 1) / (rho * c)) * (-rho / c);
  L[2 * 3 + 0] = ((gamma - 1) / (rho * c)) * ((v * v) / 2 - c * v / (gamma - 1));
  L[2 * 3 + 1] = ((gamma - 1) / (rho * c)) * (-v + c / (gamma - 1));
  L[2 * 3 + 2] = ((gamma - 1) / (rho * c)) * (1);
}
static void e1_right(double *R, const double *u, double gamma) {
  double rho = u[0], v = u[1] / rho, e = u[2];
  double P = (e - 0.5 * rho * v * v) * (gamma - 1.0);
  double c = sqrt(gamma * P / rho);
  R[0 * 3 + 1] = -rho / (2 * c);
  R[1 * 3 + 1] = -rho * (v - c) / (2 * c);
  R[2 * 3 + 1] = -rho * ((v * v) / 2 + (c * c) / (gamma - 1) - c * v) / (2 * c);
  R[0 * 3 + 0] = 1;
  R[1 * 3 + 0] = v;
  R[2 * 3 + 0] = v * v / 2;
  R[0 * 3 + 2] = rho / (2 * c);
  R[1 * 3 + 2] = rho * (v + c) / (2 * c);
  R[2 * 3 + 2] = rho * ((v * v) / 2 + (c * c) / (gamma - 1) + c * v) / (2 * c);
}

/* Euler2D -- include/physicalmodels/euler2d.h:44-230 */
static void e2_flux(double *f, const double *u, int dir, double gamma) {
  double rho = u[0], vx = u[1] / rho, vy = u[2] / rho, e = u[3];
  double vsq = (vx * vx) + (vy * vy);
  double P = (e - 0.5 * rho * vsq) * (gamma - 1.0);
  if (dir == 0) {
    f[0] = rho * vx;
    f[1] = rho * vx * vx + P;
    f[2] = rho * vx * vy;
    f[3] = (e + P) * vx;
  } else {
    f[0] = rho * vy;
    f[1] = rho * vy * vx;
    f[2] = rho * vy * vy + P;
    f[3] = (e + P) * vy;
  }
}
static void e2_roeavg(double *ua, const double *uL, const double *uR, double gamma) {
  double rhoL = uL[0], vxL = uL[1] / rhoL, vyL = uL[2] / rhoL, eL = uL[3];
  double vsqL = (vxL * vxL) + (vyL * vyL);
  double PL = (eL - 0.5 * rhoL * vsqL) * (gamma - 1.0);
  double cLsq = gamma * PL / rhoL;
  double HL = 0.5 * (vxL * vxL + vyL * vyL) + cLsq / (gamma - 1.0);
  double rhoR = uR[0], vxR = uR[1] / rhoR, vyR = uR[2] / rhoR, eR = uR[3];
  double vsqR = (vxR * vxR) + (vyR * vyR);
  double PR = (eR - 0.5 * rhoR * vsqR) * (gamma - 1.0);
  double cRsq = gamma * PR / rhoR;
  double HR = 0.5 * (vxR * vxR + vyR * vyR) + cRsq / (gamma - 1.0);
  double tL = sqrt(rhoL), tR = sqrt(rhoR);
  double rho = tL * tR;
  double vx = (tL * vxL + tR * vxR) / (tL + tR);
  double vy = (tL * vyL + tR * vyR) / (tL + tR);
  double H = (tL * HL + tR * HR) / (tL + tR);
  double vsq = vx * vx + vy * vy;
  double csq = (gamma - 1.0) * (H - 0.5 * vsq);
  double P = csq * rho / gamma;
  double e = P / (gamma - 1.0) + 0.5 * rho * vsq;
  ua[0] = rho;
  ua[1] = rho * vx;
  ua[2] = rho * vy;
  ua[3] = e;
}
static void e2_eig(double *D, const double *u, int dir, double gamma) {
  double rho = u[0], vx = u[1] / rho, vy = u[2] / rho, e = u[3];
  double vsq = (vx * vx) + (vy * vy);
  double P = (e - 0.5 * rho * vsq) * (gamma - 1.0);
  double c = sqrt(gamma * P / rho);
  double vn = (dir == 0) ? vx : vy;
  if (dir == 0) { D[0] = vn - c; D[1] = vn + c; D[2] = vn; D[3] = vn; }
  else { D[0] = vn - c; D[1] = vn; D[2] = vn + c; D[3] = vn; }
}
static void e2_left(double *L, const double *u, int dir, double ga) {
  double gm1 = ga - 1.0;
  double rho = u[0], vx = u[1] / rho, vy = u[2] / rho, e = u[3];
  double vsq = (vx * vx) + (vy * vy);
  double P = (e - 0.5 * rho * vsq) * (ga - 1.0);
  double ek = 0.5 * (vx * vx + vy * vy);
  double a = sqrt(ga * P / rho);
  double nx = 0, ny = 0, un;
  if (dir == 0) {
    un = vx; nx = 1.0;
    L[0 * 4 + 0] = (gm1 * ek + a * un) / (2 * a * a);
    L[0 * 4 + 1] = ((-gm1) * vx - a * nx) / (2 * a * a);
    L[0 * 4 + 2] = ((-gm1) * vy - a * ny) / (2 * a * a);
    L[0 * 4 + 3] = gm1 / (2 * a * a);
    L[3 * 4 + 0] = (a * a - gm1 * ek) / (a * a);
    L[3 * 4 + 1] = (gm1 * vx) / (a * a);
    L[3 * 4 + 2] = (gm1 * vy) / (a * a);
    L[3 * 4 + 3] = (-gm1) / (a * a);
    L[1 * 4 + 0] = (gm1 * ek - a * un) / (2 * a * a);
    L[1 * 4 + 1] = ((-gm1) * vx + a * nx) / (2 * a * a);
    L[1 * 4 + 2] = ((-gm1) * vy + a * ny) / (2 * a * a);
    L[1 * 4 + 3] = gm1 / (2 * a * a);
    L[2 * 4 + 0] = (vy - un * ny) / nx;
    L[2 * 4 + 1] = ny;
    L[2 * 4 + 2] = (ny * ny - 1.0) / nx;
    L[2 * 4 + 3] = 0.0;
  } else {
    un = vy; ny = 1.0;
    L[0 * 4 + 0] = (gm1 * ek + a * un) / (2 * a * a);
    L[0 * 4 + 1] = ((1.0 - ga) * vx - a * nx) / (2 * a * a);
    L[0 * 4 + 2] = ((1.0 - ga) * vy - a * ny) / (2 * a * a);
    L[0 * 4 + 3] = gm1 / (2 * a * a);
    L[3 * 4 + 0] = (a * a - gm1 * ek) / (a * a);
    L[3 * 4 + 1] = gm1 * vx / (a * a);
    L[3 * 4 + 2] = gm1 * vy / (a * a);
    L[3 * 4 + 3] = (1.0 - ga) / (a * a);
    L[2 * 4 + 0] = (gm1 * ek - a * un) / (2 * a * a);
    L[2 * 4 + 1] = ((1.0 - ga) * vx + a * nx) / (2 * a * a);
    L[2 * 4 + 2] = ((1.0 - ga) * vy + a * ny) / (2 * a * a);
    L[2 * 4 + 3] = gm1 / (2 * a * a);
    L[1 * 4 + 0] = (un * nx - vx) / ny;
    L[1 * 4 + 1] = (1.0 - nx * nx) / ny;
    L[1 * 4 + 2] = -nx;
    L[1 * 4 + 3] = 0;
  }
}
static void e2_right(double *R, const double *u, int dir, double ga) {
  double gm1 = ga - 1.0;
  double rho = u[0], vx = u[1] / rho, vy = u[2] / rho, e = u[3];
  double vsq = (vx * vx) + (vy * vy);
  double P = (e - 0.5 * rho * vsq) * (ga - 1.0);
  double ek = 0.5 * (vx * vx + vy * vy);
  double a = sqrt(ga * P / rho);
  double h0 = a * a / gm1 + ek;
  double nx = 0, ny = 0, un;
  if (dir == 0) {
    un = vx; nx = 1.0;
    R[0 * 4 + 0] = 1.0; R[1 * 4 + 0] = vx - a * nx; R[2 * 4 + 0] = vy - a * ny; R[3 * 4 + 0] = h0 - a * un;
    R[0 * 4 + 3] = 1.0; R[1 * 4 + 3] = vx; R[2 * 4 + 3] = vy; R[3 * 4 + 3] = ek;
    R[0 * 4 + 1] = 1.0; R[1 * 4 + 1] = vx + a * nx; R[2 * 4 + 1] = vy + a * ny; R[3 * 4 + 1] = h0 + a * un;
    R[0 * 4 + 2] = 0.0; R[1 * 4 + 2] = ny; R[2 * 4 + 2] = -nx; R[3 * 4 + 2] = vx * ny - vy * nx;
  } else {
    un = vy; ny = 1.0;
    R[0 * 4 + 0] = 1.0; R[1 * 4 + 0] = vx - a * nx; R[2 * 4 + 0] = vy - a * ny; R[3 * 4 + 0] = h0 - a * un;
    R[0 * 4 + 3] = 1.0; R[1 * 4 + 3] = vx; R[2 * 4 + 3] = vy; R[3 * 4 + 3] = ek;
    R[0 * 4 + 2] = 1.0; R[1 * 4 + 2] = vx + a * nx; R[2 * 4 + 2] = vy + a * ny; R[3 * 4 + 2] = h0 + a * un;
    R[0 * 4 + 1] = 0; R[1 * 4 + 1] = ny; R[2 * 4 + 1] = -nx; R[3 * 4 + 1] = vx * ny - vy * nx;
  }
}

/* NavierStokes3D -- include/physicalmodels/navierstokes3d.h:98-480 */
#define NS_FLOWVAR(u, rho, vx, vy, vz, e, P, gamma)       \
  do {                                                    \
    double vsq_;                                          \
    rho = (u)[0];                                         \
    vx = (rho == 0) ? 0 : (u)[1] / rho;                   \
    vy = (rho == 0) ? 0 : (u)[2] / rho;                   \
    vz = (rho == 0) ? 0 : (u)[3] / rho;                   \
    e = (u)[4];                                           \
    vsq_ = vx * vx + vy * vy + vz * vz;                   \
    P = (e - 0.5 * rho * vsq_) * (gamma - 1.0);           \
  } while (0)

static void ns_flux(double *f, const double *u, int dir, double gamma) {
  double rho, vx, vy, vz, e, P;
  NS_FLOWVAR(u, rho, vx, vy, vz, e, P, gamma);
  if (dir == 0) {
    f[0] = rho * vx; f[1] = rho * vx * vx + P; f[2] = rho * vx * vy; f[3] = rho * vx * vz; f[4] = (e + P) * vx;
  } else if (dir == 1) {
    f[0] = rho * vy; f[1] = rho * vy * vx; f[2] = rho * vy * vy + P; f[3] = rho * vy * vz; f[4] = (e + P) * vy;
  } else {
    f[0] = rho * vz; f[1] = rho * vz * vx; f[2] = rho * vz * vy; f[3] = rho * vz * vz + P; f[4] = (e + P) * vz;
  }
}
static void ns_roeavg(double *ua, const double *uL, const double *uR, double gamma) {
  double rho, vx, vy, vz, e, P, H;
  double rhoL, vxL, vyL, vzL, eL, PL, HL, cLsq;
  double rhoR, vxR, vyR, vzR, eR, PR, HR, cRsq;
  NS_FLOWVAR(uL, rhoL, vxL, vyL, vzL, eL, PL, gamma);
  cLsq = gamma * PL / rhoL;
  HL = 0.5 * (vxL * vxL + vyL * vyL + vzL * vzL) + cLsq / (gamma - 1.0);
  NS_FLOWVAR(uR, rhoR, vxR, vyR, vzR, eR, PR, gamma);
  cRsq = gamma * PR / rhoR;
  HR = 0.5 * (vxR * vxR + vyR * vyR + vzR * vzR) + cRsq / (gamma - 1.0);
  double tL = sqrt(rhoL), tR = sqrt(rhoR);
  rho = tL * tR;
  vx = (tL * vxL + tR * vxR) / (tL + tR);
  vy = (tL * vyL + tR * vyR) / (tL + tR);
  vz = (tL * vzL + tR * vzR) / (tL + tR);
  H = (tL * HL + tR * HR) / (tL + tR);
  P = (H - 0.5 * (vx * vx + vy * vy + vz * vz)) * (rho * (gamma - 1.0)) / gamma;
  e = P / (gamma - 1.0) + 0.5 * rho * (vx * vx + vy * vy + vz * vz);
  ua[0] = rho; ua[1] = rho * vx; ua[2] = rho * vy; ua[3] = rho * vz; ua[4] = e;
}
static void ns_eig(double *D, const double *u, int dir, double gamma) {
  double rho, vx, vy, vz, e, P;
  NS_FLOWVAR(u, rho, vx, vy, vz, e, P, gamma);
  double c = sqrt(gamma * P / rho);
  if (dir == 0) { D[0] = vx; D[1] = vx - c; D[2] = vx; D[3] = vx; D[4] = vx + c; }
  else if (dir == 1) { D[0] = vy; D[1] = vy; D[2] = vy - c; D[3] = vy; D[4] = vy + c; }
  else { D[0] = vz; D[1] = vz; D[2] = vz; D[3] = vz - c; D[4] = vz + c; }
}
static void ns_left(double *L, const double *u, int dir, double ga) {
  double gm1 = ga - 1.0;
  double rho, vx, vy, vz, e, P, a, ek;
  NS_FLOWVAR(u, rho, vx, vy, vz, e, P, ga);
  ek = 0.5 * (vx * vx + vy * vy + vz * vz);
  a = sqrt(ga * P / rho);
  if (dir == 0) {
    L[1 * 5 + 0] = (gm1 * ek + a * vx) / (2 * a * a);
    L[1 * 5 + 1] = ((-gm1) * vx - a) / (2 * a * a);
    L[1 * 5 + 2] = ((-gm1) * vy) / (2 * a * a);
    L[1 * 5 + 3] = ((-gm1) * vz) / (2 * a * a);
    L[1 * 5 + 4] = gm1 / (2 * a * a);
    L[0 * 5 + 0] = (a * a - gm1 * ek) / (a * a);
    L[0 * 5 + 1] = (gm1 * vx) / (a * a);
    L[0 * 5 + 2] = (gm1 * vy) / (a * a);
    L[0 * 5 + 3] = (gm1 * vz) / (a * a);
    L[0 * 5 + 4] = (-gm1) / (a * a);
    L[4 * 5 + 0] = (gm1 * ek - a * vx) / (2 * a * a);
    L[4 * 5 + 1] = ((-gm1) * vx + a) / (2 * a * a);
    L[4 * 5 + 2] = ((-gm1) * vy) / (2 * a * a);
    L[4 * 5 + 3] = ((-gm1) * vz) / (2 * a * a);
    L[4 * 5 + 4] = gm1 / (2 * a * a);
    L[2 * 5 + 0] = vy; L[2 * 5 + 1] = 0.0; L[2 * 5 + 2] = -1.0; L[2 * 5 + 3] = 0.0; L[2 * 5 + 4] = 0.0;
    L[3 * 5 + 0] = -vz; L[3 * 5 + 1] = 0.0; L[3 * 5 + 2] = 0.0; L[3 * 5 + 3] = 1.0; L[3 * 5 + 4] = 0.0;
  } else if (dir == 1) {
    L[2 * 5 + 0] = (gm1 * ek + a * vy) / (2 * a * a);
    L[2 * 5 + 1] = ((1.0 - ga) * vx) / (2 * a * a);
    L[2 * 5 + 2] = ((1.0 - ga) * vy - a) / (2 * a * a);
    L[2 * 5 + 3] = ((1.0 - ga) * vz) / (2 * a * a);
    L[2 * 5 + 4] = gm1 / (2 * a * a);
    L[0 * 5 + 0] = (a * a - gm1 * ek) / (a * a);
    L[0 * 5 + 1] = gm1 * vx / (a * a);
    L[0 * 5 + 2] = gm1 * vy / (a * a);
    L[0 * 5 + 3] = gm1 * vz / (a * a);
    L[0 * 5 + 4] = (1.0 - ga) / (a * a);
    L[4 * 5 + 0] = (gm1 * ek - a * vy) / (2 * a * a);
    L[4 * 5 + 1] = ((1.0 - ga) * vx) / (2 * a * a);
    L[4 * 5 + 2] = ((1.0 - ga) * vy + a) / (2 * a * a);
    L[4 * 5 + 3] = ((1.0 - ga) * vz) / (2 * a * a);
    L[4 * 5 + 4] = gm1 / (2 * a * a);
    L[1 * 5 + 0] = -vx; L[1 * 5 + 1] = 1.0; L[1 * 5 + 2] = 0.0; L[1 * 5 + 3] = 0.0; L[1 * 5 + 4] = 0;
    L[3 * 5 + 0] = vz; L[3 * 5 + 1] = 0.0; L[3 * 5 + 2] = 0.0; L[3 * 5 + 3] = -1.0; L[3 * 5 + 4] = 0;
  } else {
    L[3 * 5 + 0] = (gm1 * ek + a * vz) / (2 * a * a);
    L[3 * 5 + 1] = ((1.0 - ga) * vx) / (2 * a * a);
    L[3 * 5 + 2] = ((1.0 - ga) * vy) / (2 * a * a);
    L[3 * 5 + 3] = ((1.0 - ga) * vz - a) / (2 * a * a);
    L[3 * 5 + 4] = gm1 / (2 * a * a);
    L[0 * 5 + 0] = (a * a - gm1 * ek) / (a * a);
    L[0 * 5 + 1] = gm1 * vx / (a * a);
    L[0 * 5 + 2] = gm1 * vy / (a * a);
    L[0 * 5 + 3] = gm1 * vz / (a * a);
    L[0 * 5 + 4] = (1.0 - ga) / (a * a);
    L[4 * 5 + 0] = (gm1 * ek - a * vz) / (2 * a * a);
    L[4 * 5 + 1] = ((1.0 - ga) * vx) / (2 * a * a);
    L[4 * 5 + 2] = ((1.0 - ga) * vy) / (2 * a * a);
    L[4 * 5 + 3] = ((1.0 - ga) * vz + a) / (2 * a * a);
    L[4 * 5 + 4] = gm1 / (2 * a * a);
    L[1 * 5 + 0] = vx; L[1 * 5 + 1] = -1.0; L[1 * 5 + 2] = 0.0; L[1 * 5 + 3] = 0.0; L[1 * 5 + 4] = 0;
    L[2 * 5 + 0] = -vy; L[2 * 5 + 1] = 0.0; L[2 * 5 + 2] = 1.0; L[2 * 5 + 3] = 0.0; L[2 * 5 + 4] = 0;
  }
}
static void ns_right(double *R, const double *u, int dir, double ga) {
  double gm1 = ga - 1.0;
  double rho, vx, vy, vz, e, P, ek, a, h0;
  NS_FLOWVAR(u, rho, vx, vy, vz, e, P, ga);
  ek = 0.5 * (vx * vx + vy * vy + vz * vz);
  a = sqrt(ga * P / rho);
  h0 = a * a / gm1 + ek;
#define RR(r, c) R[(r) * 5 + (c)]
  if (dir == 0) {
    RR(0, 1) = 1.0; RR(1, 1) = vx - a; RR(2, 1) = vy; RR(3, 1) = vz; RR(4, 1) = h0 - a * vx;
    RR(0, 0) = 1.0; RR(1, 0) = vx; RR(2, 0) = vy; RR(3, 0) = vz; RR(4, 0) = ek;
    RR(0, 4) = 1.0; RR(1, 4) = vx + a; RR(2, 4) = vy; RR(3, 4) = vz; RR(4, 4) = h0 + a * vx;
    RR(0, 2) = 0.0; RR(1, 2) = 0.0; RR(2, 2) = -1.0; RR(3, 2) = 0.0; RR(4, 2) = -vy;
    RR(0, 3) = 0.0; RR(1, 3) = 0.0; RR(2, 3) = 0.0; RR(3, 3) = 1.0; RR(4, 3) = vz;
  } else if (dir == 1) {
    RR(0, 2) = 1.0; RR(1, 2) = vx; RR(2, 2) = vy - a; RR(3, 2) = vz; RR(4, 2) = h0 - a * vy;
    RR(0, 0) = 1.0; RR(1, 0) = vx; RR(2, 0) = vy; RR(3, 0) = vz; RR(4, 0) = ek;
    RR(0, 4) = 1.0; RR(1, 4) = vx; RR(2, 4) = vy + a; RR(3, 4) = vz; RR(4, 4) = h0 + a * vy;
    RR(0, 1) = 0.0; RR(1, 1) = 1.0; RR(2, 1) = 0.0; RR(3, 1) = 0.0; RR(4, 1) = vx;
    RR(0, 3) = 0.0; RR(1, 3) = 0.0; RR(2, 3) = 0.0; RR(3, 3) = -1.0; RR(4, 3) = -vz;
  } else {
    RR(0, 3) = 1.0; RR(1, 3) = vx; RR(2, 3) = vy; RR(3, 3) = vz - a; RR(4, 3) = h0 - a * vz;
    RR(0, 0) = 1.0; RR(1, 0) = vx; RR(2, 0) = vy; RR(3, 0) = vz; RR(4, 0) = ek;
    RR(0, 4) = 1.0; RR(1, 4) = vx; RR(2, 4) = vy; RR(3, 4) = vz + a; RR(4, 4) = h0 + a * vz;
    RR(0, 1) = 0.0; RR(1, 1) = -1.0; RR(2, 1) = 0.0; RR(3, 1) = 0.0; RR(4, 1) = -vx;
    RR(0, 2) = 0.0; RR(1, 2) = 0.0; RR(2, 2) = 1.0; RR(3, 2) = 0.0; RR(4, 2) = vy;
  }
#undef RR
}

/* Model dispatch. */
static void m_flux(const orc_problem *p, double *f, const double *u, int dir) {
  if (p->model == ORC_EULER1D) e1_flux(f, u, p->gamma);
  else if (p->model == ORC_EULER2D) e2_flux(f, u, dir, p->gamma);
  else ns_flux(f, u, dir, p->gamma);
}
static void m_roeavg(const orc_problem *p, double *ua, const double *uL, const double *uR) {
  if (p->model == ORC_EULER1D) e1_roeavg(ua, uL, uR, p->gamma);
  else if (p->model == ORC_EULER2D) e2_roeavg(ua, uL, uR, p->gamma);
  else ns_roeavg(ua, uL, uR, p->gamma);
}
static void m_eig(const orc_problem *p, double *D, const double *u, int dir) {
  if (p->model == ORC_EULER1D) e1_eig(D, u, p->gamma);
  else if (p->model == ORC_EULER2D) e2_eig(D, u, dir, p->gamma);
  else ns_eig(D, u, dir, p->gamma);
}
static void m_left(const orc_problem *p, double *L, const double *u, int dir) {
  if (p->model == ORC_EULER1D) e1_left(L, u, p->gamma);
  else if (p->model == ORC_EULER2D) e2_left(L, u, dir, p->gamma);
  else ns_left(L, u, dir, p->gamma);
}
static void m_right(const orc_problem *p, double *R, const double *u, int dir) {
  if (p->model == ORC_EULER1D) e1_right(R, u, p->gamma);
  else if (p->model == ORC_EULER2D) e2_right(R, u, dir, p->gamma);
  else ns_right(R, u, dir, p->gamma);
}

/* UFunction: Euler1D u*(1/grav_field) with grav_field = exp(0) = 1
 * (Euler1DModifiedSolution.c:23-50); NavierStokes3D recomputes the energy
 * (NavierStokes3DModifiedSolution.c:31-70) with f = g = 1 at zero gravity;
 * Euler2D has none (uC = u). */
static void m_ufunc(const orc_problem *p, double *uC, const double *u, long q) {
  int nv = p->nvars;
  if (p->model == ORC_NS3D) {
    /* NavierStokes3DModifiedSolution.c:52-66 */
    double inv_gamma_m1 = 1.0 / (p->gamma - 1.0);
    double rho, uvel, vvel, wvel, E, P;
    double f = p->gf ? p->gf[q] : 1.0, g = p->gg ? p->gg[q] : 1.0;
    NS_FLOWVAR(u, rho, uvel, vvel, wvel, E, P, p->gamma);
    (void)E;
    uC[0] = u[0] * f;
    uC[1] = u[1] * f;
    uC[2] = u[2] * f;
    uC[3] = u[3] * f;
    uC[4] = (P * inv_gamma_m1) * (1.0 / g) + (0.5 * rho * (uvel * uvel + vvel * vvel + wvel * wvel)) * f;
  } else if (p->model == ORC_EULER1D) {
    /* Euler1DModifiedSolution.c:48: uC = u / S (gf holds 1.0 / S) */
    const double a = p->gf ? p->gf[q] : (1.0 / 1.0);
    for (int v = 0; v < nv; v++) uC[v] = a * u[v];
  } else {
    for (int v = 0; v < nv; v++) uC[v] = u[v];
  }
}

/* ------------------------------------------------------------------------ */
/* WENO5 (Jiang-Shu weights)                                                  */
/* ------------------------------------------------------------------------ */

/* _WENOWeights_v_JS_ (include/interpolation.h:265-285), one component. */
static inline void weno_js(const double *c, double m3, double m2, double m1, double p1, double p2, double eps,
                           double *w1, double *w2, double *w3) {
  static const double thirteen_by_twelve = 13.0 / 12.0;
  static const double one_fourth = 1.0 / 4.0;
  const double c1 = c[0], c2 = c[1], c3 = c[2];
  double b1, b2, b3, a1, a2, a3, a_sum_inv;
  b1 = thirteen_by_twelve * (m3 - 2 * m2 + m1) * (m3 - 2 * m2 + m1)
       + one_fourth * (m3 - 4 * m2 + 3 * m1) * (m3 - 4 * m2 + 3 * m1);
  a1 = c1 / ((b1 + eps) * (b1 + eps));
  b2 = thirteen_by_twelve * (m2 - 2 * m1 + p1) * (m2 - 2 * m1 + p1)
       + one_fourth * (m2 - p1) * (m2 - p1);
  a2 = c2 / ((b2 + eps) * (b2 + eps));
  b3 = thirteen_by_twelve * (m1 - 2 * p1 + p2) * (m1 - 2 * p1 + p2)
       + one_fourth * (3 * m1 - 4 * p1 + p2) * (3 * m1 - 4 * p1 + p2);
  a3 = c3 / ((b3 + eps) * (b3 + eps));
  a_sum_inv = 1.0 / (a1 + a2 + a3);
  *w1 = a1 * a_sum_inv;
  *w2 = a2 * a_sum_inv;
  *w3 = a3 * a_sum_inv;
}

/* _WENOWeights_v_M_ (include/interpolation.h:319-345): JS weights, then the
 * mapping of Henrick, Aslam & Powers and a second normalisation. */
static inline void weno_m(const double *c, double m3, double m2, double m1, double p1, double p2, double eps,
                          double *w1, double *w2, double *w3) {
  const double c1 = c[0], c2 = c[1], c3 = c[2];
  double a1, a2, a3, a_sum_inv;
  weno_js(c, m3, m2, m1, p1, p2, eps, w1, w2, w3);
  a1 = *w1 * (c1 + c1 * c1 - 3 * c1 * *w1 + *w1 * *w1) / (c1 * c1 + *w1 * (1.0 - 2.0 * c1));
  a2 = *w2 * (c2 + c2 * c2 - 3 * c2 * *w2 + *w2 * *w2) / (c2 * c2 + *w2 * (1.0 - 2.0 * c2));
  a3 = *w3 * (c3 + c3 * c3 - 3 * c3 * *w3 + *w3 * *w3) / (c3 * c3 + *w3 * (1.0 - 2.0 * c3));
  a_sum_inv = 1.0 / (a1 + a2 + a3);
  *w1 = a1 * a_sum_inv;
  *w2 = a2 * a_sum_inv;
  *w3 = a3 * a_sum_inv;
}

/* Smoothness indicators of _WENOWeights_v_* (include/interpolation.h). */
static inline void weno_betas(double m3, double m2, double m1, double p1, double p2, double *b1,
                              double *b2, double *b3) {
  static const double thirteen_by_twelve = 13.0 / 12.0;
  static const double one_fourth = 1.0 / 4.0;
  *b1 = thirteen_by_twelve * (m3 - 2 * m2 + m1) * (m3 - 2 * m2 + m1)
        + one_fourth * (m3 - 4 * m2 + 3 * m1) * (m3 - 4 * m2 + 3 * m1);
  *b2 = thirteen_by_twelve * (m2 - 2 * m1 + p1) * (m2 - 2 * m1 + p1)
        + one_fourth * (m2 - p1) * (m2 - p1);
  *b3 = thirteen_by_twelve * (m1 - 2 * p1 + p2) * (m1 - 2 * p1 + p2)
        + one_fourth * (3 * m1 - 4 * p1 + p2) * (3 * m1 - 4 * p1 + p2);
}

/* _WENOWeights_v_Z_ (tau = |b3-b1|, include/interpolation.h:417-437) and
 * _WENOWeights_v_YC_ (tau = (m3-4m2+6m1-4p1+p2)^2, :474-494). */
static inline void weno_tau(const double *c, double tau, double b1, double b2, double b3, double eps, double *w1,
                            double *w2, double *w3) {
  const double c1 = c[0], c2 = c[1], c3 = c[2];
  double a1, a2, a3, a_sum_inv;
  a1 = c1 * (1.0 + (tau / (b1 + eps)) * (tau / (b1 + eps)));
  a2 = c2 * (1.0 + (tau / (b2 + eps)) * (tau / (b2 + eps)));
  a3 = c3 * (1.0 + (tau / (b3 + eps)) * (tau / (b3 + eps)));
  a_sum_inv = 1.0 / (a1 + a2 + a3);
  *w1 = a1 * a_sum_inv;
  *w2 = a2 * a_sum_inv;
  *w3 = a3 * a_sum_inv;
}

/* The weights of one biased stencil for the problem's formulation
 * (WENOFifthOrderCalculateWeights.c:57-60; no_limiting keeps the optimal
 * weights of WENOFifthOrderInitializeWeights). */
/* Optimal weights: WENO5 (include/interpolation.h:228-232) and CRWENO5 at interior
 * interfaces (:234-238). */
static const double WENO_C[3] = {0.1, 0.6, 0.3};
static const double CRWENO_C[3] = {0.2, 0.5, 0.3};

/* The weights of one biased stencil for the problem's formulation and the optimal
 * weights c (WENOFifthOrderCalculateWeights.c:57-60 and :205-225; no_limiting keeps
 * the optimal weights of WENOFifthOrderInitializeWeights). */
static inline void weno_w_c(int type, const double *c, double m3, double m2, double m1, double p1, double p2,
                            double eps, double *w1, double *w2, double *w3) {
  double b1, b2, b3, tau;
  switch (type) {
    case ORC_WENO_MAPPED: weno_m(c, m3, m2, m1, p1, p2, eps, w1, w2, w3); return;
    case ORC_WENO_BORGES:
      weno_betas(m3, m2, m1, p1, p2, &b1, &b2, &b3);
      tau = fabs(b3 - b1);
      weno_tau(c, tau, b1, b2, b3, eps, w1, w2, w3);
      return;
    case ORC_WENO_YC:
      weno_betas(m3, m2, m1, p1, p2, &b1, &b2, &b3);
      tau = (m3 - 4 * m2 + 6 * m1 - 4 * p1 + p2) * (m3 - 4 * m2 + 6 * m1 - 4 * p1 + p2);
      weno_tau(c, tau, b1, b2, b3, eps, w1, w2, w3);
      return;
    case ORC_WENO_NONE: *w1 = c[0]; *w2 = c[1]; *w3 = c[2]; return;
    default: weno_js(c, m3, m2, m1, p1, p2, eps, w1, w2, w3); return;
  }
}

static inline void weno_w(int type, double m3, double m2, double m1, double p1, double p2, double eps,
                          double *w1, double *w2, double *w3) {
  weno_w_c(type, WENO_C, m3, m2, m1, p1, p2, eps, w1, w2, w3);
}

/* Interp1PrimFifthOrderWENO (Interp1PrimFifthOrderWENO.c:143-158), one component. */
static inline double weno_interp(double w1, double w2, double w3, double fm3, double fm2,
                                 double fm1, double fp1, double fp2) {
  static const double one_sixth = 1.0 / 6.0;
  double f1 = (2 * one_sixth) * fm3 + (-7 * one_sixth) * fm2 + (11 * one_sixth) * fm1;
  double f2 = (-one_sixth) * fm2 + (5 * one_sixth) * fm1 + (2 * one_sixth) * fp1;
  double f3 = (2 * one_sixth) * fm1 + (5 * one_sixth) * fp1 + (-one_sixth) * fp2;
  return w1 * f1 + w2 * f2 + w3 * f3;
}

/* Interp1PrimFifthOrderWENOChar (Interp1PrimFifthOrderWENOChar.c:170-188): the
 * characteristic candidate stencils and their weighted sum. */
static inline double weno_interp_char(double w1, double w2, double w3, double fm3, double fm2,
                                      double fm1, double fp1, double fp2) {
  static const double one_sixth = 1.0 / 6.0;
  double f1 = (2 * one_sixth) * fm3 - (7.0 * one_sixth) * fm2 + (11.0 * one_sixth) * fm1;
  double f2 = (-one_sixth) * fm2 + (5.0 * one_sixth) * fm1 + (2 * one_sixth) * fp1;
  double f3 = (2 * one_sixth) * fm1 + (5 * one_sixth) * fp1 - (one_sixth) * fp2;
  return w1 * f1 + w2 * f2 + w3 * f3;
}

/* MatVecMult (include/matmult_native.h:116-123): y = A x, sums from zero. */
static inline void matvec(int n, double *y, const double *A, const double *x) {
  for (int i = 0; i < n; i++) {
    y[i] = 0;
    for (int j = 0; j < n; j++) y[i] += A[i * n + j] * x[j];
  }
}
/* MatMult (include/matmult_native.h:18-27). */
static inline void matmul(int n, double *C, const double *X, const double *Y) {
  for (int i = 0; i < n; i++)
    for (int j = 0; j < n; j++) {
      C[i * n + j] = 0.0;
      for (int k = 0; k < n; k++) C[i * n + j] += X[i * n + k] * Y[k * n + j];
    }
}

#define absolute(a) ((a) < 0 ? -(a) : (a))
#define max2(a, b) ((a) > (b) ? (a) : (b))
#define max3(a, b, c) max2(max2((a), (b)), max2((b), (c)))

/* ------------------------------------------------------------------------ */
/* Upwinding (one interface)                                                  */
/* ------------------------------------------------------------------------ */

/* fI from fL,fR,uL,uR and the cell-centre states uCL (cell left of the
 * interface) and uCR (right).  Roe: Euler1DUpwindRoe (Euler1DUpwind.c:30-113),
 * Euler2DUpwindRoe (Euler2DUpwind.c:10-66), NavierStokes3DUpwindRoe
 * (NavierStokes3DUpwind.c:40-139).  LLF: Euler1DUpwindLLF (Euler1DUpwind.c:212-290),
 * Euler2DUpwindLLF (Euler2DUpwind.c:139-210), NavierStokes3DUpwindLLF
 * (NavierStokes3DUpwind.c:244-318).  RF: Euler2DUpwindRF (Euler2DUpwind.c:68-137),
 * and the same form for Euler1D/NavierStokes3D. */
/* Rusanov's wave speed |v_dir| + c of a state (Euler1DUpwindRusanov takes
 * c = gamma P / rho there, without the square root, Euler1DUpwind.c:394-404;
 * NavierStokes3DUpwindRusanov, NavierStokes3DUpwind.c:392-403). */
static double rusanov_speed(const orc_problem *p, const double *u, int dir) {
  double g = p->gamma;
  if (p->model == ORC_EULER1D) {
    double rho = u[0], v = u[1] / rho, e = u[2];
    double P = (e - 0.5 * rho * v * v) * (g - 1.0);
    double c = g * P / rho;
    return c + absolute(v);
  }
  double rho = u[0];
  double vx = (rho == 0) ? 0 : u[1] / rho, vy = (rho == 0) ? 0 : u[2] / rho, vz = (rho == 0) ? 0 : u[3] / rho;
  double e = u[4], vsq = vx * vx + vy * vy + vz * vz;
  double P = (e - 0.5 * rho * vsq) * (g - 1.0);
  double c = sqrt(g * P / rho);
  double vel[3] = {vx, vy, vz};
  return c + absolute(vel[dir]);
}

/* Steger-Warming flux vector splitting of one state: Euler1DUpwindSWFS
 * (src/PhysicalModels/Euler1D/Euler1DUpwind.c:336-350) and Euler2DUpwindSWFS
 * (src/PhysicalModels/Euler2D/Euler2DUpwind.c:244-276), plus (plus = 1) or minus part. */
static void swfs_split(const orc_problem *p, int dir, const double *u, int plus, double *f) {
  double gamma = p->gamma;
  if (p->model == ORC_EULER1D) {
    double rho = u[0], v = u[1] / rho, e = u[2];
    double P = (e - 0.5 * rho * v * v) * (gamma - 1.0);
    double c = sqrt(gamma * P / rho);
    double term = rho / (2.0 * gamma);
    if (plus) {
      f[0] = term * (2 * gamma * v + c - v);
      f[1] = term * (2 * (gamma - 1.0) * v * v + (v + c) * (v + c));
      f[2] = term * ((gamma - 1.0) * v * v * v + 0.5 * (v + c) * (v + c) * (v + c) +
                     ((3.0 - gamma) * (v + c) * c * c) / (2.0 * (gamma - 1.0)));
    } else {
      f[0] = term * (v - c);
      f[1] = term * (v - c) * (v - c);
      f[2] = term * (0.5 * (v - c) * (v - c) * (v - c) + ((3.0 - gamma) * (v - c) * c * c) / (2.0 * (gamma - 1.0)));
    }
    return;
  }
  double rho = u[0], vx = u[1] / rho, vy = u[2] / rho, e = u[3];
  double vsq = (vx * vx) + (vy * vy);
  double P = (e - 0.5 * rho * vsq) * (gamma - 1.0);
  double c = sqrt(gamma * P / rho);
  double term = rho / (2.0 * gamma);
  double kx = (dir == 0 ? 1.0 : 0.0), ky = (dir == 1 ? 1.0 : 0.0), l[4];
  l[0] = l[1] = kx * vx + ky * vy;
  l[2] = l[0] + c;
  l[3] = l[0] - c;
  for (int k = 0; k < 4; k++) {
    if (plus && l[k] < 0.0) l[k] = 0.0;
    if (!plus && l[k] > 0.0) l[k] = 0.0;
  }
  f[0] = term * (2.0 * (gamma - 1.0) * l[0] + l[2] + l[3]);
  f[1] = term * (2.0 * (gamma - 1.0) * l[0] * vx + l[2] * (vx + c * kx) + l[3] * (vx - c * kx));
  f[2] = term * (2.0 * (gamma - 1.0) * l[0] * vy + l[2] * (vy + c * ky) + l[3] * (vy - c * ky));
  f[3] = term * ((gamma - 1.0) * l[0] * (vx * vx + vy * vy) +
                 0.5 * l[2] * ((vx + c * kx) * (vx + c * kx) + (vy + c * ky) * (vy + c * ky)) +
                 0.5 * l[3] * ((vx - c * kx) * (vx - c * kx) + (vy - c * ky) * (vy - c * ky)) +
                 ((3.0 - gamma) * (l[2] + l[3]) * c * c) / (2.0 * (gamma - 1.0)));
}

static void upwind(const orc_problem *p, int dir, double *fI, const double *fL, const double *fR,
                   const double *uL, const double *uR, const double *uCL, const double *uCR, long qL, long qR) {
  int nv = p->nvars;
  double uavg[MAXV], D[MAXV], L[MAXV * MAXV], R[MAXV * MAXV];
  if (p->upwind == ORC_UPW_SWFS) {
    /* by the Mach number of the Roe average of the reconstructed states: fR, fL or
     * F+(uL) + F-(uR) */
    m_roeavg(p, uavg, uL, uR);
    double rho = uavg[0], vn = uavg[1 + dir] / rho, P;
    if (p->model == ORC_EULER1D) {
      P = (uavg[2] - 0.5 * rho * vn * vn) * (p->gamma - 1.0); /* _Euler1DGetFlowVar_ */
    } else {
      double vx = uavg[1] / rho, vy = uavg[2] / rho;
      double vsq = (vx * vx) + (vy * vy);
      P = (uavg[3] - 0.5 * rho * vsq) * (p->gamma - 1.0); /* _Euler2DGetFlowVar_ */
    }
    double mach = vn / sqrt(p->gamma * P / rho);
    if (mach < -1.0) {
      for (int v = 0; v < nv; v++) fI[v] = fR[v];
    } else if (mach < 1.0) {
      double fp[MAXV], fm[MAXV];
      swfs_split(p, dir, uL, 1, fp);
      swfs_split(p, dir, uR, 0, fm);
      for (int v = 0; v < nv; v++) fI[v] = fp[v] + fm[v];
    } else {
      for (int v = 0; v < nv; v++) fI[v] = fL[v];
    }
    return;
  }
  if (p->upwind == ORC_UPW_RUSANOV) {
    /* fI = (fL+fR)/2 - kappa max3(speeds of the cell-centre states and their
     * Roe average) (uR-uL)/2, kappa = 1 without gravity */
    double udiff[MAXV];
    m_roeavg(p, uavg, uCL, uCR);
    for (int v = 0; v < nv; v++) udiff[v] = 0.5 * (uR[v] - uL[v]);
    double alphaL = rusanov_speed(p, uCL, dir);
    double alphaR = rusanov_speed(p, uCR, dir);
    double alphaavg = rusanov_speed(p, uavg, dir);
    double kappa = p->gg ? max2(p->gg[qL], p->gg[qR]) : max2(1.0, 1.0);
    double alpha = kappa * max3(alphaL, alphaR, alphaavg);
    for (int v = 0; v < nv; v++) fI[v] = 0.5 * (fL[v] + fR[v]) - alpha * udiff[v];
    return;
  }
  if (p->upwind == ORC_UPW_ROE) {
    double udiff[MAXV], DL[MAXV * MAXV], modA[MAXV * MAXV], udiss[MAXV];
    for (int v = 0; v < nv; v++) udiff[v] = 0.5 * (uR[v] - uL[v]);
    if (p->model == ORC_EULER2D) m_roeavg(p, uavg, uL, uR);
    else m_roeavg(p, uavg, uCL, uCR);
    m_eig(p, D, uavg, dir);
    m_left(p, L, uavg, dir);
    m_right(p, R, uavg, dir);
    if (p->model == ORC_EULER1D) {
      /* Euler1DUpwind.c:79-82: the dissipation scaled by max(S_L, S_R) of the gravity field */
      double kappa = p->gg ? max2(p->gg[qL], p->gg[qR]) : max2(1.0, 1.0);
      for (int k = 0; k < nv; k++) D[k] = kappa * absolute(D[k]);
    } else {
      double delta = 0.000001, delta2 = delta * delta;
      for (int k = 0; k < nv; k++)
        D[k] = (absolute(D[k]) < delta ? (D[k] * D[k] + delta2) / (2 * delta) : absolute(D[k]));
    }
    double Dm[MAXV * MAXV];
    for (int i = 0; i < nv * nv; i++) Dm[i] = 0;
    for (int k = 0; k < nv; k++) Dm[k * nv + k] = D[k];
    matmul(nv, DL, Dm, L);
    matmul(nv, modA, R, DL);
    matvec(nv, udiss, modA, udiff);
    for (int v = 0; v < nv; v++) fI[v] = 0.5 * (fL[v] + fR[v]) - udiss[v];
  } else {
    double fcL[MAXV], fcR[MAXV], ucL[MAXV], ucR[MAXV], fc[MAXV];
    double eigL[MAXV], eigC[MAXV], eigR[MAXV];
    int cellcentre = (p->model == ORC_EULER1D);
    if (cellcentre) m_roeavg(p, uavg, uCL, uCR);
    else m_roeavg(p, uavg, uL, uR);
    m_left(p, L, uavg, dir);
    m_right(p, R, uavg, dir);
    matvec(nv, ucL, L, uL);
    matvec(nv, ucR, L, uR);
    matvec(nv, fcL, L, fL);
    matvec(nv, fcR, L, fR);
    m_eig(p, eigL, cellcentre ? uCL : uL, dir);
    m_eig(p, eigR, cellcentre ? uCR : uR, dir);
    m_eig(p, eigC, uavg, dir);
    for (int k = 0; k < nv; k++) {
      if (p->upwind == ORC_UPW_RF) {
        if ((eigL[k] > 0) && (eigC[k] > 0) && (eigR[k] > 0)) { fc[k] = fcL[k]; continue; }
        if ((eigL[k] < 0) && (eigC[k] < 0) && (eigR[k] < 0)) { fc[k] = fcR[k]; continue; }
      }
      double alpha = max3(absolute(eigL[k]), absolute(eigC[k]), absolute(eigR[k]));
      if (p->model == ORC_EULER1D && p->upwind == ORC_UPW_LLF) /* Euler1DUpwind.c:249, :268 */
        alpha = (p->gg ? max2(p->gg[qL], p->gg[qR]) : 1.0) * alpha;
      fc[k] = 0.5 * (fcL[k] + fcR[k] + alpha * (ucL[k] - ucR[k]));
    }
    matvec(nv, fI, R, fc);
  }
}

/* ------------------------------------------------------------------------ */
/* Hyperbolic term                                                           */
/* ------------------------------------------------------------------------ */

/* HyperbolicFunction (src/HyParFunctions/HyperbolicFunction.c:31-126) with
 * ReconstructHyperbolic (:167-222): per dimension, the cell flux, the WENO
 * weights from (fC, u) (WENOFifthOrderCalculateWeights.c:111-236 / :760-896),
 * uC = UFunction(u), the four interpolations, upwinding, and
 * hyp += dxinv*(F[j+1/2]-F[j-1/2]) accumulated dimension by dimension. */
/* tridiagLU (src/TridiagLU/tridiagLU.c:90-274) on one rank, one system of n rows
 * (a: sub-, b: main, c: super-diagonal, x: right-hand side, overwritten with the
 * solution): elimination of the sub-diagonal, then back-substitution, with the
 * reference's operations (the fill-in a[i] = -factor a[i-1] stays zero since
 * a[0] = 0, and the missing next-rank value xp1 is zero). */
static int tridiag_solve(int n, double *a, double *b, double *c, double *x) {
  for (int i = 1; i < n; i++) {
    if (b[i - 1] == 0) return -1;
    double factor = a[i] / b[i - 1];
    b[i] -= factor * c[i - 1];
    a[i] = -factor * a[i - 1];
    x[i] -= factor * x[i - 1];
  }
  const double xp1 = 0.0;
  if (b[n - 1] == 0) return -1;
  x[n - 1] = (x[n - 1] - a[n - 1] * x[0] - c[n - 1] * xp1) / b[n - 1];
  for (int i = n - 2; i > -1; i--) {
    if (b[i] == 0) return -1;
    x[i] = (x[i] - c[i] * x[i + 1] - a[i] * x[0]) / b[i];
  }
  return 0;
}

/* Interp1PrimFifthOrderCRWENO (Interp1PrimFifthOrderCRWENO.c:124-199) on one grid
 * line of N cells, for the four interface reconstructions k = 0 fL, 1 fR (values fC,
 * weights from fC), 2 uL, 3 uR (values uC, weights from u) and, with a source function
 * sC (gravity), k = 4 sL, 5 sR (values sC, the weights of fL and fR: the source's
 * InterpolateInterfacesHyp calls pass uflag 0, Euler1DSource.c:55-56,
 * NavierStokes3DSource.c:70-71), every component: at the
 * N+1 interfaces the rows
 *   left-biased:  (2/3 w1 + 1/3 w2) F_{j-1/2} + (1/3 w1 + 2/3 w2 + 2/3 w3) F_{j+1/2}
 *                 + 1/3 w3 F_{j+3/2} = w1 (f_{j-1} + 5 f_j)/6 + w2 (5 f_j + f_{j+1})/6
 *                 + w3 (f_j + 5 f_{j+1})/6
 * (right-biased: mirrored), the weights with the CRWENO5 optimal weights
 * (WENOFifthOrderCalculateWeights.c:205-225); the first and last interfaces take the
 * explicit WENO5 value (identity rows, WENO5 optimal weights) on a single rank.
 * out[(I*nk + k)*nv + v], nk = 4 (6 with sC); work: 4 (N+1) doubles. */
static int crweno_line(const orc_problem *p, const double *fC, const double *u, const double *uC,
                       const double *sC, long base, long sd, int N, double *out, double *work) {
  static const double one_third = 1.0 / 3.0;
  static const double one_sixth = 1.0 / 6.0;
  const int nv = p->nvars, n = N + 1, nk = sC ? 6 : 4;
  double *a = work, *b = work + n, *c = work + 2 * n, *x = work + 3 * n;
  for (int k = 0; k < nk; k++) {
    const double *val = k < 2 ? fC : (k < 4 ? uC : sC), *wv = (k < 2 || k >= 4) ? fC : u;
    const int upw = (k % 2 == 0) ? 1 : -1;
    for (int v = 0; v < nv; v++) {
      for (int I = 0; I <= N; I++) {
        long qm1, qm2, qm3, qp1, qp2;
        if (upw > 0) {
          qm1 = base + (long)(I - 1) * sd;
          qm3 = qm1 - 2 * sd;
          qm2 = qm1 - sd;
          qp1 = qm1 + sd;
          qp2 = qm1 + 2 * sd;
        } else {
          qm1 = base + (long)I * sd;
          qm3 = qm1 + 2 * sd;
          qm2 = qm1 + sd;
          qp1 = qm1 - sd;
          qp2 = qm1 - 2 * sd;
        }
        const int bnd = (I == 0) || (I == N);
        double w1, w2, w3;
        weno_w_c(p->weights, bnd ? WENO_C : CRWENO_C, wv[nv * qm3 + v], wv[nv * qm2 + v], wv[nv * qm1 + v],
                 wv[nv * qp1 + v], wv[nv * qp2 + v], p->eps, &w1, &w2, &w3);
        const double fm3 = val[nv * qm3 + v], fm2 = val[nv * qm2 + v], fm1 = val[nv * qm1 + v];
        const double fp1 = val[nv * qp1 + v], fp2 = val[nv * qp2 + v];
        double f1, f2, f3;
        if (bnd) {
          f1 = (2 * one_sixth) * fm3 + (-7 * one_sixth) * fm2 + (11 * one_sixth) * fm1;
          f2 = (-one_sixth) * fm2 + (5 * one_sixth) * fm1 + (2 * one_sixth) * fp1;
          f3 = (2 * one_sixth) * fm1 + (5 * one_sixth) * fp1 + (-one_sixth) * fp2;
          a[I] = 0.0;
          b[I] = 1.0;
          c[I] = 0.0;
        } else {
          f1 = (one_sixth) * fm2 + (5 * one_sixth) * fm1;
          f2 = (5 * one_sixth) * fm1 + (one_sixth) * fp1;
          f3 = (one_sixth) * fm1 + (5 * one_sixth) * fp1;
          if (upw > 0) {
            a[I] = (2 * one_third) * w1 + (one_third) * w2;
            b[I] = (one_third) * w1 + (2 * one_third) * w2 + (2 * one_third) * w3;
            c[I] = (one_third) * w3;
          } else {
            c[I] = (2 * one_third) * w1 + (one_third) * w2;
            b[I] = (one_third) * w1 + (2 * one_third) * w2 + (2 * one_third) * w3;
            a[I] = (one_third) * w3;
          }
        }
        x[I] = w1 * f1 + w2 * f2 + w3 * f3;
      }
      if (tridiag_solve(n, a, b, c, x)) return -1;
      for (int I = 0; I <= N; I++) out[((long)I * nk + k) * nv + v] = x[I];
    }
  }
  return 0;
}

/* _MatrixInvert_ (include/matops.h:93-125): B = A^{-1} for an n x n row-major
 * matrix by elimination without pivoting on a copy of A applied to the identity,
 * then the backward sweep, in the reference's operation order. */
static void mat_invert(int n, const double *A, double *B) {
  double Ac[MAXV * MAXV];
  for (int i = 0; i < n * n; i++) Ac[i] = A[i];
  for (int i = 0; i < n * n; i++) B[i] = 0.0;
  for (int i = 0; i < n; i++) B[i * n + i] = 1.0;
  for (int i = 0; i < n - 1; i++)
    for (int j = i + 1; j < n; j++) {
      double factor = Ac[j * n + i] / Ac[i * n + i];
      for (int k = i + 1; k < n; k++) Ac[j * n + k] -= (factor * Ac[i * n + k]);
      for (int k = 0; k < j; k++) B[j * n + k] -= (factor * B[i * n + k]);
    }
  for (int i = n - 1; i >= 0; i--)
    for (int k = 0; k < n; k++) {
      double sum = 0.0;
      for (int j = i + 1; j < n; j++) sum += (Ac[i * n + j] * B[j * n + k]);
      B[i * n + k] = (B[i * n + k] - sum) / Ac[i * n + i];
    }
}
/* _MatrixMultiplySubtract_: C -= A B, one product at a time. */
static void mat_mul_sub(int n, double *C, const double *A, const double *B) {
  for (int i = 0; i < n; i++)
    for (int j = 0; j < n; j++)
      for (int k = 0; k < n; k++) C[i * n + j] -= (A[i * n + k] * B[k * n + j]);
}
/* _MatVecMultiplySubtract_: y -= A x. */
static void matvec_sub(int n, double *y, const double *A, const double *x) {
  for (int i = 0; i < n; i++)
    for (int j = 0; j < n; j++) y[i] -= (A[i * n + j] * x[j]);
}

/* blocktridiagLU (src/TridiagLU/blocktridiagLU.c) on one rank, one system of n block
 * rows of size bs (a, b, c: n bs*bs row-major blocks; x: n bs values, the solution on
 * return): elimination of the sub-diagonal blocks with the inverse of the previous
 * diagonal block, then block back-substitution (the missing next-rank values are zero). */
static void block_tridiag_solve(int n, int bs, double *a, double *b, double *c, double *x) {
  const int bs2 = bs * bs;
  double binv[MAXV * MAXV], factor[MAXV * MAXV], xt[MAXV];
  for (int i = 1; i < n; i++) {
    mat_invert(bs, b + (i - 1) * bs2, binv);
    matmul(bs, factor, a + i * bs2, binv);
    mat_mul_sub(bs, b + i * bs2, factor, c + (i - 1) * bs2);
    for (int q = 0; q < bs2; q++) a[i * bs2 + q] = 0.0;
    mat_mul_sub(bs, a + i * bs2, factor, a + (i - 1) * bs2);
    matvec_sub(bs, x + i * bs, factor, x + (i - 1) * bs);
  }
  const double xp1[MAXV] = {0.0};
  mat_invert(bs, b + (n - 1) * bs2, binv);
  matvec_sub(bs, x + (n - 1) * bs, a + (n - 1) * bs2, x);
  matvec_sub(bs, x + (n - 1) * bs, c + (n - 1) * bs2, xp1);
  matvec(bs, xt, binv, x + (n - 1) * bs);
  for (int j = 0; j < bs; j++) x[(n - 1) * bs + j] = xt[j];
  for (int i = n - 2; i > -1; i--) {
    mat_invert(bs, b + i * bs2, binv);
    matvec_sub(bs, x + i * bs, c + i * bs2, x + (i + 1) * bs);
    matvec_sub(bs, x + i * bs, a + i * bs2, x);
    matvec(bs, xt, binv, x + i * bs);
    for (int j = 0; j < bs; j++) x[i * bs + j] = xt[j];
  }
}

/* Interp1PrimFifthOrderCRWENOChar (Interp1PrimFifthOrderCRWENOChar.c:139-230) on one
 * grid line: per interface the left eigenvectors L of the Roe average of the two
 * cell-centre states, the characteristic stencils L f, and block rows
 * A = a L, B = b L, C = c L (a, b, c per characteristic field, as the component-wise
 * rows with b = w1/3 + 2 (w2 + w3)/3), right-hand side sum_k w_k f_k; the first and last
 * interfaces: B = L and the explicit WENO5 value.  Weights: the characteristic weights
 * (WENOFifthOrderCalculateWeightsChar*, projections of f and u) with the CRWENO5 /
 * WENO5 optimal weights.  With a source function sC (gravity): k = 4, 5 its left and
 * right values with the flux's weights, as crweno_line.
 * out[(I*nk + k)*nv + v], nk = 4 (6 with sC); work: (N+1) (3 nv^2 + nv) doubles. */
static int crweno_char_line(const orc_problem *p, const double *fC, const double *u, const double *uC,
                            const double *sC, long base, long sd, int N, int dir, double *out, double *work) {
  static const double one_third = 1.0 / 3.0;
  static const double one_sixth = 1.0 / 6.0;
  const int nv = p->nvars, n = N + 1, nv2 = nv * nv, nk = sC ? 6 : 4;
  double *A = work, *B = work + (long)n * nv2, *Cm = work + 2L * n * nv2, *F = work + 3L * n * nv2;
  for (int k = 0; k < nk; k++) {
    const double *val = k < 2 ? fC : (k < 4 ? uC : sC), *wv = (k < 2 || k >= 4) ? fC : u;
    const int upw = (k % 2 == 0) ? 1 : -1;
    for (int I = 0; I <= N; I++) {
      const long qm1 = upw > 0 ? base + (long)(I - 1) * sd : base + (long)I * sd;
      const long st = upw > 0 ? sd : -sd;
      const long q[5] = {qm1 - 2 * st, qm1 - st, qm1, qm1 + st, qm1 + 2 * st}; /* qm3 qm2 qm1 qp1 qp2 */
      double uavg[MAXV], L[MAXV * MAXV];
      /* the Roe average of the cells either side (symmetric in its arguments) */
      m_roeavg(p, uavg, u + nv * (base + (long)(I - 1) * sd), u + nv * (base + (long)I * sd));
      m_left(p, L, uavg, dir);
      double pw[5][MAXV], pv[5][MAXV];
      for (int m = 0; m < 5; m++) {
        matvec(nv, pw[m], L, wv + nv * q[m]);
        matvec(nv, pv[m], L, val + nv * q[m]);
      }
      const int bnd = (I == 0) || (I == N);
      double *Ai = A + (long)I * nv2, *Bi = B + (long)I * nv2, *Ci = Cm + (long)I * nv2;
      for (int v = 0; v < nv; v++) {
        double w1, w2, w3;
        weno_w_c(p->weights, bnd ? WENO_C : CRWENO_C, pw[0][v], pw[1][v], pw[2][v], pw[3][v], pw[4][v], p->eps,
                 &w1, &w2, &w3);
        const double fm3 = pv[0][v], fm2 = pv[1][v], fm1 = pv[2][v], fp1 = pv[3][v], fp2 = pv[4][v];
        double f1, f2, f3;
        if (bnd) {
          f1 = (2 * one_sixth) * fm3 - (7.0 * one_sixth) * fm2 + (11.0 * one_sixth) * fm1;
          f2 = (-one_sixth) * fm2 + (5.0 * one_sixth) * fm1 + (2 * one_sixth) * fp1;
          f3 = (2 * one_sixth) * fm1 + (5 * one_sixth) * fp1 - (one_sixth) * fp2;
          for (int e = 0; e < nv; e++) {
            Ai[v * nv + e] = 0.0;
            Ci[v * nv + e] = 0.0;
            Bi[v * nv + e] = L[v * nv + e];
          }
        } else {
          f1 = (one_sixth) * (fm2 + 5 * fm1);
          f2 = (one_sixth) * (5 * fm1 + fp1);
          f3 = (one_sixth) * (fm1 + 5 * fp1);
          const double lo = (2 * one_third) * w1 + (one_third) * w2;
          const double di = (one_third) * w1 + (2 * one_third) * (w2 + w3);
          const double up = (one_third) * w3;
          for (int e = 0; e < nv; e++) {
            Ai[v * nv + e] = (upw > 0 ? lo : up) * L[v * nv + e];
            Bi[v * nv + e] = di * L[v * nv + e];
            Ci[v * nv + e] = (upw > 0 ? up : lo) * L[v * nv + e];
          }
        }
        F[(long)I * nv + v] = w1 * f1 + w2 * f2 + w3 * f3;
      }
    }
    block_tridiag_solve(n, nv, A, B, Cm, F);
    for (int I = 0; I <= N; I++)
      for (int v = 0; v < nv; v++) out[((long)I * nk + k) * nv + v] = F[(long)I * nv + v];
  }
  return 0;
}

/* The hyperbolic term and, with gravity, NavierStokes3DSource
 * (NavierStokes3DSource.c:38-112): per direction with gravity, the source
 * function [0, phi e_d, phi] (phi = g field) interpolated with the weights of the
 * flux (InterpolateInterfacesHyp with uflag = 0 reuses them), averaged
 * (NavierStokes3DSourceUpwind), differenced and scaled by
 * [0, rho RT e_d, rho RT v_d] f. */
static int hyperbolic_source(const orc_problem *p, const double *u, double *hyp, double *src) {
  int nd = p->ndims, nv = p->nvars, g = p->ghosts;
  long s[3];
  strides_wg(p, s);
  long np = orc_npoints_wghosts(p);
  for (long i = 0; i < np * nv; i++) hyp[i] = 0.0;
  double *fC = (double *)malloc(sizeof(double) * np * nv);
  double *uC = (double *)malloc(sizeof(double) * np * nv);
  long offset = 0;
  int crweno_failed = 0;
  const int crweno = p->scheme == ORC_SCHEME_CRWENO5;
  /* CRWENO5 with gravity: the source function [0, phi e_d, phi] as a point array,
   * solved for beside the flux (Euler1DSourceFunction, NavierStokes3DSourceFunction) */
  double *sC = (crweno && src && p->has_grav) ? (double *)malloc(sizeof(double) * np * nv) : NULL;
  for (int d = 0; d < nd; d++) {
    const int dosrc = src && p->has_grav && p->grav[d] != 0.0;
#pragma omp parallel for schedule(static) num_threads(NTHR)
    for (long q = 0; q < np; q++) {
      m_flux(p, fC + nv * q, u + nv * q, d);
      m_ufunc(p, uC + nv * q, u + nv * q, q);
      if (sC && dosrc)
        for (int v = 0; v < nv; v++) sC[nv * q + v] = (v == 1 + d || v == nv - 1) ? p->gg[q] : 0.0;
    }
    int N = p->dim[d];
    long sd = s[d];
    long nouter = 1;
    int ob[3] = {1, 1, 1};
    for (int e = 0; e < nd; e++) if (e != d) { ob[e] = p->dim[e]; nouter *= p->dim[e]; }
    const double *dxinv = p->dxinv + offset;
    const double *sCd = dosrc ? sC : NULL;
    const int nk = sCd ? 6 : 4;
#pragma omp parallel num_threads(NTHR)
    {
      double *FI = (double *)malloc(sizeof(double) * (N + 1) * nv);
      double *SI = (double *)malloc(sizeof(double) * (N + 1) * nv);
      const int crchar = crweno && p->interp == ORC_INTERP_CHAR && nv > 1;
      double *CR = crweno ? (double *)malloc(sizeof(double) * (N + 1) * nv * 6) : NULL;
      double *CW = crweno ? (double *)malloc(sizeof(double) * (N + 1) * (crchar ? 3 * nv * nv + nv : 4)) : NULL;
#pragma omp for schedule(static)
      for (long lo = 0; lo < nouter; lo++) {
        int idx[3] = {0, 0, 0};
        long r = lo;
        for (int e = 0; e < nd; e++) if (e != d) { idx[e] = (int)(r % ob[e]); r /= ob[e]; }
        idx[d] = 0;
        long base = pidx(p, s, idx); /* cell 0 of this line */
        if (crchar ? crweno_char_line(p, fC, u, uC, sCd, base, sd, N, d, CR, CW)
                   : (crweno && crweno_line(p, fC, u, uC, sCd, base, sd, N, CR, CW))) {
          crweno_failed = 1;
          continue;
        }
        for (int I = 0; I <= N; I++) {
          long qm1L = base + (long)(I - 1) * sd, qm1R = base + (long)I * sd;
          long L3 = qm1L - 2 * sd, L2 = qm1L - sd, L1 = qm1L, L4 = qm1L + sd, L5 = qm1L + 2 * sd;
          long R3 = qm1R + 2 * sd, R2 = qm1R + sd, R1 = qm1R, R4 = qm1R - sd, R5 = qm1R - 2 * sd;
          double fL[MAXV], fR[MAXV], uL[MAXV], uR[MAXV];
          if (crweno) {
            for (int v = 0; v < nv; v++) {
              fL[v] = CR[((long)I * nk + 0) * nv + v];
              fR[v] = CR[((long)I * nk + 1) * nv + v];
              uL[v] = CR[((long)I * nk + 2) * nv + v];
              uR[v] = CR[((long)I * nk + 3) * nv + v];
              /* SourceUpwind (Euler1DSourceUpwind.c, NavierStokes3DSourceUpwind.c): the average */
              if (dosrc) SI[(long)I * nv + v] = 0.5 * (CR[((long)I * nk + 4) * nv + v] + CR[((long)I * nk + 5) * nv + v]);
            }
          } else if (p->interp == ORC_INTERP_COMP) {
            for (int v = 0; v < nv; v++) {
              double w1, w2, w3;
              weno_w(p->weights, fC[nv * L3 + v], fC[nv * L2 + v], fC[nv * L1 + v], fC[nv * L4 + v], fC[nv * L5 + v], p->eps, &w1, &w2, &w3);
              fL[v] = weno_interp(w1, w2, w3, fC[nv * L3 + v], fC[nv * L2 + v], fC[nv * L1 + v], fC[nv * L4 + v], fC[nv * L5 + v]);
              double sL = 0.0, sR = 0.0;
              int sv = dosrc && (v == 1 + d || v == nv - 1);
              if (dosrc)
                sL = sv ? weno_interp(w1, w2, w3, p->gg[L3], p->gg[L2], p->gg[L1], p->gg[L4], p->gg[L5])
                        : weno_interp(w1, w2, w3, 0.0, 0.0, 0.0, 0.0, 0.0);
              weno_w(p->weights, fC[nv * R3 + v], fC[nv * R2 + v], fC[nv * R1 + v], fC[nv * R4 + v], fC[nv * R5 + v], p->eps, &w1, &w2, &w3);
              fR[v] = weno_interp(w1, w2, w3, fC[nv * R3 + v], fC[nv * R2 + v], fC[nv * R1 + v], fC[nv * R4 + v], fC[nv * R5 + v]);
              if (dosrc) {
                sR = sv ? weno_interp(w1, w2, w3, p->gg[R3], p->gg[R2], p->gg[R1], p->gg[R4], p->gg[R5])
                        : weno_interp(w1, w2, w3, 0.0, 0.0, 0.0, 0.0, 0.0);
                SI[(long)I * nv + v] = 0.5 * (sL + sR);
              }
              weno_w(p->weights, u[nv * L3 + v], u[nv * L2 + v], u[nv * L1 + v], u[nv * L4 + v], u[nv * L5 + v], p->eps, &w1, &w2, &w3);
              uL[v] = weno_interp(w1, w2, w3, uC[nv * L3 + v], uC[nv * L2 + v], uC[nv * L1 + v], uC[nv * L4 + v], uC[nv * L5 + v]);
              weno_w(p->weights, u[nv * R3 + v], u[nv * R2 + v], u[nv * R1 + v], u[nv * R4 + v], u[nv * R5 + v], p->eps, &w1, &w2, &w3);
              uR[v] = weno_interp(w1, w2, w3, uC[nv * R3 + v], uC[nv * R2 + v], uC[nv * R1 + v], uC[nv * R4 + v], uC[nv * R5 + v]);
            }
          } else {
            double uavg[MAXV], L[MAXV * MAXV], R[MAXV * MAXV];
            m_roeavg(p, uavg, u + nv * qm1L, u + nv * qm1R);
            m_left(p, L, uavg, d);
            m_right(p, R, uavg, d);
            long sl[5] = {L3, L2, L1, L4, L5}, sr[5] = {R3, R2, R1, R4, R5};
            double cfl[5][MAXV], cfr[5][MAXV], cul[5][MAXV], cur[5][MAXV];  /* weights' stencils */
            double ifl[5][MAXV], ifr[5][MAXV], iul[5][MAXV], iur[5][MAXV];  /* interpolants' stencils */
            for (int k = 0; k < 5; k++) {
              matvec(nv, cfl[k], L, fC + nv * sl[k]);
              matvec(nv, cfr[k], L, fC + nv * sr[k]);
              matvec(nv, cul[k], L, u + nv * sl[k]);
              matvec(nv, cur[k], L, u + nv * sr[k]);
              matvec(nv, ifl[k], L, fC + nv * sl[k]);
              matvec(nv, ifr[k], L, fC + nv * sr[k]);
              matvec(nv, iul[k], L, uC + nv * sl[k]);
              matvec(nv, iur[k], L, uC + nv * sr[k]);
            }
            double isl[5][MAXV], isr[5][MAXV];  /* projected source-function stencils */
            if (dosrc) {
              for (int k = 0; k < 5; k++) {
                double phl[MAXV] = {0.0}, phr[MAXV] = {0.0};
                phl[1 + d] = phl[nv - 1] = p->gg[sl[k]];
                phr[1 + d] = phr[nv - 1] = p->gg[sr[k]];
                matvec(nv, isl[k], L, phl);
                matvec(nv, isr[k], L, phr);
              }
            }
            double xfl[MAXV], xfr[MAXV], xul[MAXV], xur[MAXV], xsl[MAXV], xsr[MAXV];
            for (int v = 0; v < nv; v++) {
              double w1, w2, w3;
              weno_w(p->weights, cfl[0][v], cfl[1][v], cfl[2][v], cfl[3][v], cfl[4][v], p->eps, &w1, &w2, &w3);
              xfl[v] = weno_interp_char(w1, w2, w3, ifl[0][v], ifl[1][v], ifl[2][v], ifl[3][v], ifl[4][v]);
              if (dosrc) xsl[v] = weno_interp_char(w1, w2, w3, isl[0][v], isl[1][v], isl[2][v], isl[3][v], isl[4][v]);
              weno_w(p->weights, cfr[0][v], cfr[1][v], cfr[2][v], cfr[3][v], cfr[4][v], p->eps, &w1, &w2, &w3);
              xfr[v] = weno_interp_char(w1, w2, w3, ifr[0][v], ifr[1][v], ifr[2][v], ifr[3][v], ifr[4][v]);
              if (dosrc) xsr[v] = weno_interp_char(w1, w2, w3, isr[0][v], isr[1][v], isr[2][v], isr[3][v], isr[4][v]);
              weno_w(p->weights, cul[0][v], cul[1][v], cul[2][v], cul[3][v], cul[4][v], p->eps, &w1, &w2, &w3);
              xul[v] = weno_interp_char(w1, w2, w3, iul[0][v], iul[1][v], iul[2][v], iul[3][v], iul[4][v]);
              weno_w(p->weights, cur[0][v], cur[1][v], cur[2][v], cur[3][v], cur[4][v], p->eps, &w1, &w2, &w3);
              xur[v] = weno_interp_char(w1, w2, w3, iur[0][v], iur[1][v], iur[2][v], iur[3][v], iur[4][v]);
            }
            matvec(nv, fL, R, xfl);
            matvec(nv, fR, R, xfr);
            matvec(nv, uL, R, xul);
            matvec(nv, uR, R, xur);
            if (dosrc) {
              double sLv[MAXV], sRv[MAXV];
              matvec(nv, sLv, R, xsl);
              matvec(nv, sRv, R, xsr);
              for (int v = 0; v < nv; v++) SI[(long)I * nv + v] = 0.5 * (sLv[v] + sRv[v]);
            }
          }
          upwind(p, d, FI + (long)I * nv, fL, fR, uL, uR, u + nv * qm1L, u + nv * qm1R, qm1L, qm1R);
        }
        for (int i = 0; i < N; i++) {
          long q = base + (long)i * sd;
          for (int v = 0; v < nv; v++)
            hyp[nv * q + v] += dxinv[g + i] * (FI[(long)(i + 1) * nv + v] - FI[(long)i * nv + v]);
        }
        if (dosrc) {
          for (int i = 0; i < N; i++) {
            long q = base + (long)i * sd;
            double term[5];
            if (p->model == ORC_EULER1D) {
              /* Euler1DSource.c:67-72: [0, rho, rho v] (the field's 1/S applied below) */
              double rho = u[nv * q], vel = u[nv * q + 1] / rho;
              term[0] = 0.0;
              term[1] = rho;
              term[2] = rho * vel;
            } else {
              double rho, vel[3], E, P;
              NS_FLOWVAR((u + nv * q), rho, vel[0], vel[1], vel[2], E, P, p->gamma);
              (void)E;
              (void)P;
              term[0] = 0.0;
              term[1] = rho * p->RT * (d == 0);
              term[2] = rho * p->RT * (d == 1);
              term[3] = rho * p->RT * (d == 2);
              term[4] = rho * p->RT * vel[d];
            }
            for (int v = 0; v < nv; v++)
              src[nv * q + v] += ((term[v] * p->gf[q]) * (SI[(long)(i + 1) * nv + v] - SI[(long)i * nv + v]) *
                                  dxinv[g + i]);
          }
        }
      }
      free(FI);
      free(SI);
      free(CR);
      free(CW);
    }
    offset += p->dim[d] + 2 * g;
  }
  free(fC);
  free(uC);
  free(sC);
  return crweno_failed ? -1 : 0;
}

/* ------------------------------------------------------------------------ */
/* NavierStokes3D viscous term                                               */
/* ------------------------------------------------------------------------ */

/* FirstDerivativeFourthOrderCentral (src/FirstDerivative/FirstDerivativeFourthOrder.c:36-129):
 * lines along dir over the full ghost extent, for interior transverse indices only. */
static void deriv4(const orc_problem *p, double *Df, const double *f, int dir) {
  int nd = p->ndims, nv = p->nvars, g = p->ghosts;
  long s[3];
  strides_wg(p, s);
  static const double one_twelve = 1.0 / 12.0;
  int N = p->dim[dir];
  long sd = s[dir];
  long nouter = 1;
  int ob[3] = {1, 1, 1};
  for (int e = 0; e < nd; e++) if (e != dir) { ob[e] = p->dim[e]; nouter *= p->dim[e]; }
#pragma omp parallel for schedule(static) num_threads(NTHR)
  for (long lo = 0; lo < nouter; lo++) {
    int idx[3] = {0, 0, 0};
    long r = lo;
    for (int e = 0; e < nd; e++) if (e != dir) { idx[e] = (int)(r % ob[e]); r /= ob[e]; }
    idx[dir] = -g;
    long b = pidx(p, s, idx); /* first ghost point of the line */
    for (int i = -g; i < N + g; i++) {
      long qC = b + (long)(i + g) * sd;
      for (int v = 0; v < nv; v++) {
        double val;
#define F(k) f[(qC + (long)(k) * sd) * nv + v]
        if (i == -g)
          val = (-25 * F(0) + 48 * F(1) - 36 * F(2) + 16 * F(3) - 3 * F(4)) * one_twelve;
        else if (i == -g + 1)
          val = (-3 * F(-1) - 10 * F(0) + 18 * F(1) - 6 * F(2) + F(3)) * one_twelve;
        else if (i < N + g - 2)
          val = (F(-2) - 8 * F(-1) + 8 * F(1) - F(2)) * one_twelve;
        else if (i == N + g - 2)
          val = (-F(-3) + 6 * F(-2) - 18 * F(-1) + 10 * F(0) + 3 * F(1)) * one_twelve;
        else
          val = (3 * F(-4) - 16 * F(-3) + 36 * F(-2) - 48 * F(-1) + 25 * F(0)) * one_twelve;
#undef F
        Df[qC * nv + v] = val;
      }
    }
  }
}

/* FirstDerivativeFirstOrder (src/FirstDerivative/FirstDerivativeFirstOrder.c:36-86):
 * forward at the first point of the ghost-extended line, backward at its last, and in
 * between bias 1 (forward) or -1 (backward), as the reference writes it; lines with
 * interior transverse indices only. */
static void deriv1(const orc_problem *p, double *Df, const double *f, int dir, int bias) {
  int nd = p->ndims, nv = p->nvars, g = p->ghosts;
  long s[3];
  strides_wg(p, s);
  int N = p->dim[dir];
  long sd = s[dir];
  long nouter = 1;
  int ob[3] = {1, 1, 1};
  for (int e = 0; e < nd; e++) if (e != dir) { ob[e] = p->dim[e]; nouter *= p->dim[e]; }
#pragma omp parallel for schedule(static) num_threads(NTHR)
  for (long lo = 0; lo < nouter; lo++) {
    int idx[3] = {0, 0, 0};
    long r = lo;
    for (int e = 0; e < nd; e++) if (e != dir) { idx[e] = (int)(r % ob[e]); r /= ob[e]; }
    idx[dir] = -g;
    long b = pidx(p, s, idx);
    for (int i = -g; i < N + g; i++) {
      long qC = b + (long)(i + g) * sd;
      for (int v = 0; v < nv; v++) {
        double val;
#define F(k) f[(qC + (long)(k) * sd) * nv + v]
        if (i == -g) val = F(1) - F(0);
        else if (i == N + g - 1) val = F(0) - F(-1);
        else val = (bias > 0 ? bias : 0) * F(1) - bias * F(0) + (bias < 0 ? bias : 0) * F(-1);
#undef F
        Df[qC * nv + v] = val;
      }
    }
  }
}

void orc_set_par_scheme(orc_problem *p, int scheme) { p->par_scheme = scheme; }

/* the first derivative of par_space_scheme (InitializeSolvers.c:129-141) */
static void deriv_par(const orc_problem *p, double *Df, const double *f, int dir, int bias) {
  if (p->par_scheme == 2) deriv1(p, Df, f, dir, bias);
  else deriv4(p, Df, f, dir);
}

/* NavierStokes3DParabolicFunction (NavierStokes3DParabolicFunction.c:50-325),
 * including its single-rank behaviour: derivative arrays start at zero and are
 * filled only on lines with interior transverse indices, so cross derivatives
 * at ghost points stay zero. */
int orc_parabolic(const orc_problem *p, const double *u, double *par) {
  long np = orc_npoints_wghosts(p);
  int nv = p->nvars, g = p->ghosts;
  for (long i = 0; i < np * nv; i++) par[i] = 0.0;
  if (p->model != ORC_NS3D || p->Re <= 0) return 0;
  static const double two_third = 2.0 / 3.0;
  double inv_gamma_m1 = 1.0 / (p->gamma - 1.0);
  double inv_Re = 1.0 / p->Re;
  double inv_Pr = 1.0 / p->Pr;
  double *Q = (double *)calloc(np * nv, sizeof(double));
  double *QX = (double *)calloc(np * nv, sizeof(double));
  double *QY = (double *)calloc(np * nv, sizeof(double));
  double *QZ = (double *)calloc(np * nv, sizeof(double));
  double *FV = (double *)calloc(np * nv, sizeof(double));
  double *FD = (double *)calloc(np * nv, sizeof(double));
  int imax = p->dim[0], jmax = p->dim[1], kmax = p->dim[2];
  long s[3];
  strides_wg(p, s);
#pragma omp parallel for schedule(static) num_threads(NTHR)
  for (long q = 0; q < np; q++) {
    double energy, pressure;
    double *Qp = Q + q * nv;
    NS_FLOWVAR(u + q * nv, Qp[0], Qp[1], Qp[2], Qp[3], energy, pressure, p->gamma);
    (void)energy;
    Qp[4] = p->gamma * pressure / Qp[0];
  }
  deriv_par(p, QX, Q, 0, 1);
  deriv_par(p, QY, Q, 1, 1);
  deriv_par(p, QZ, Q, 2, 1);
  const double *dxi = p->dxinv, *dyi = p->dxinv + imax + 2 * g, *dzi = dyi + jmax + 2 * g;
#pragma omp parallel for schedule(static) num_threads(NTHR)
  for (int k = -g; k < kmax + g; k++)
    for (int j = -g; j < jmax + g; j++)
      for (int i = -g; i < imax + g; i++) {
        long q = ((long)(i + g) * s[0] + (long)(j + g) * s[1] + (long)(k + g) * s[2]) * nv;
        for (int v = 0; v < nv; v++) {
          QX[q + v] *= dxi[i + g];
          QY[q + v] *= dyi[j + g];
          QZ[q + v] *= dzi[k + g];
        }
      }
  for (int dir = 0; dir < 3; dir++) {
#pragma omp parallel for schedule(static) num_threads(NTHR)
    for (long q = 0; q < np; q++) {
      const double *Qp = Q + q * nv, *X = QX + q * nv, *Y = QY + q * nv, *Z = QZ + q * nv;
      double *Fv = FV + q * nv;
      double uvel = Qp[1], vvel = Qp[2], wvel = Qp[3], T = Qp[4];
      double mu = exp(0.76 * log(T));
      if (dir == 0) {
        double Tx = X[4], ux = X[1], vx = X[2], wx = X[3], uy = Y[1], vy = Y[2], uz = Z[1], wz = Z[3];
        double tau_xx = two_third * (mu * inv_Re) * (2 * ux - vy - wz);
        double tau_xy = (mu * inv_Re) * (uy + vx);
        double tau_xz = (mu * inv_Re) * (uz + wx);
        double qx = (mu * inv_Re * inv_gamma_m1 * inv_Pr) * Tx;
        Fv[0] = 0.0; Fv[1] = tau_xx; Fv[2] = tau_xy; Fv[3] = tau_xz;
        Fv[4] = uvel * tau_xx + vvel * tau_xy + wvel * tau_xz + qx;
      } else if (dir == 1) {
        double Ty = Y[4], ux = X[1], vx = X[2], uy = Y[1], vy = Y[2], wy = Y[3], vz = Z[2], wz = Z[3];
        double tau_yx = (mu * inv_Re) * (uy + vx);
        double tau_yy = two_third * (mu * inv_Re) * (-ux + 2 * vy - wz);
        double tau_yz = (mu * inv_Re) * (vz + wy);
        double qy = (mu * inv_Re * inv_gamma_m1 * inv_Pr) * Ty;
        Fv[0] = 0.0; Fv[1] = tau_yx; Fv[2] = tau_yy; Fv[3] = tau_yz;
        Fv[4] = uvel * tau_yx + vvel * tau_yy + wvel * tau_yz + qy;
      } else {
        double Tz = Z[4], ux = X[1], wx = X[3], vy = Y[2], wy = Y[3], uz = Z[1], vz = Z[2], wz = Z[3];
        double tau_zx = (mu * inv_Re) * (uz + wx);
        double tau_zy = (mu * inv_Re) * (vz + wy);
        double tau_zz = two_third * (mu * inv_Re) * (-ux - vy + 2 * wz);
        double qz = (mu * inv_Re * inv_gamma_m1 * inv_Pr) * Tz;
        Fv[0] = 0.0; Fv[1] = tau_zx; Fv[2] = tau_zy; Fv[3] = tau_zz;
        Fv[4] = uvel * tau_zx + vvel * tau_zy + wvel * tau_zz + qz;
      }
    }
    deriv_par(p, FD, FV, dir, -1);
    const double *di = (dir == 0) ? dxi : (dir == 1 ? dyi : dzi);
#pragma omp parallel for schedule(static) num_threads(NTHR)
    for (int k = 0; k < kmax; k++)
      for (int j = 0; j < jmax; j++)
        for (int i = 0; i < imax; i++) {
          long q = ((long)(i + g) * s[0] + (long)(j + g) * s[1] + (long)(k + g) * s[2]) * nv;
          int id = (dir == 0) ? i : (dir == 1 ? j : k);
          double dinv = di[id + g];
          for (int v = 0; v < nv; v++) par[q + v] += (dinv * FD[q + v]);
        }
  }
  free(Q); free(QX); free(QY); free(QZ); free(FV); free(FD);
  return 0;
}

/* ------------------------------------------------------------------------ */
/* RHS and RK                                                                */
/* ------------------------------------------------------------------------ */

/* TimeRHSFunctionExplicit (src/TimeIntegration/TimeRHSFunctionExplicit.c:30-98):
 * rhs = 0; rhs += -1*hyp; rhs += par; rhs += source (zero here). */
/* <Model>ComputeCFL (Euler1DComputeCFL.c:16-44, Euler2DComputeCFL.c:14-39,
 * NavierStokes3DComputeCFL.c:18-49): max over interior points and dimensions of
 * (|v_d| + c) dt dxinv_d, with the flow variables of _<Model>GetFlowVar_. */
double orc_cfl(const orc_problem *p, const double *u, double dt) {
  const int nd = p->ndims, nv = p->nvars, g = p->ghosts;
  long stride[3] = {1, 1, 1}, doff[3] = {0, 0, 0};
  for (int d = 1; d < nd; d++) stride[d] = stride[d - 1] * (p->dim[d - 1] + 2 * g);
  for (int d = 1; d < nd; d++) doff[d] = doff[d - 1] + p->dim[d - 1] + 2 * g;
  double max_cfl = 0;
  int n2 = nd > 1 ? p->dim[1] : 1, n3 = nd > 2 ? p->dim[2] : 1;
  for (int k = 0; k < n3; k++)
    for (int j = 0; j < n2; j++)
      for (int i = 0; i < p->dim[0]; i++) {
        int idx[3] = {i, j, k};
        long q = 0;
        for (int d = 0; d < nd; d++) q += (idx[d] + g) * stride[d];
        const double *w = u + nv * q;
        double rho = w[0], vel[3] = {0, 0, 0}, vsq, P, c;
        for (int d = 0; d < nd; d++) vel[d] = w[1 + d] / rho;
        vsq = vel[0] * vel[0];
        if (nd > 1) vsq = vsq + vel[1] * vel[1];
        if (nd > 2) vsq = vsq + vel[2] * vel[2];
        P = (w[nv - 1] - 0.5 * rho * vsq) * (p->gamma - 1.0);
        c = sqrt(p->gamma * P / rho);
        for (int d = 0; d < nd; d++) {
          double dxinv = p->dxinv[doff[d] + idx[d] + g];
          double local = ((vel[d] < 0 ? -vel[d] : vel[d]) + c) * dt * dxinv;
          if (local > max_cfl) max_cfl = local;
        }
      }
  return max_cfl;
}

int orc_hyperbolic(const orc_problem *p, const double *u, double *hyp) {
  return hyperbolic_source(p, u, hyp, NULL);
}

/* SourceFunction (NavierStokes3DSource.c): the gravity source at every point
 * (zero at ghost points and without gravity) */
int orc_source(const orc_problem *p, const double *u, double *src) {
  long n = orc_npoints_wghosts(p) * p->nvars;
  double *hyp = (double *)malloc(sizeof(double) * n);
  for (long i = 0; i < n; i++) src[i] = 0.0;
  int rc = hyperbolic_source(p, u, hyp, src);
  if (!rc) rc = sponge_source(p, u, src);
  free(hyp);
  return rc;
}

static int rhs_at(const orc_problem *p, double *u, double *rhs, double t) {
  long n = orc_npoints_wghosts(p) * p->nvars;
  double *hyp = (double *)malloc(sizeof(double) * n);
  double *par = (double *)malloc(sizeof(double) * n);
  double *src = (double *)calloc(n, sizeof(double));
  if (apply_bc_at(p, u, t)) {
    free(hyp);
    free(par);
    free(src);
    return -1;
  }
  int rc = hyperbolic_source(p, u, hyp, src);
  if (!rc) rc = sponge_source(p, u, src);
  orc_parabolic(p, u, par);
#pragma omp parallel for schedule(static) num_threads(NTHR)
  for (long i = 0; i < n; i++) {
    double r = 0.0;
    r += -1.0 * hyp[i];
    r += 1.0 * par[i];
    r += 1.0 * src[i];
    rhs[i] = r;
  }
  free(hyp);
  free(par);
  free(src);
  return rc;
}

int orc_rhs(const orc_problem *p, double *u, double *rhs) { return rhs_at(p, u, rhs, p->t); }

/* TimeRK (src/TimeIntegration/TimeRK.c:126-195) for one simulation:
 * U[s] = u + sum_{i<s} (dt*A[s][i]) Udot[i];  Udot[s] = RHS(U[s]);
 * u += (dt*b[s]) Udot[s], all over the full array including ghost points. */
int orc_rk(const orc_problem *p, int nstages, const double *A, const double *b,
           double *u, double dt, int nsteps) {
  long n = orc_npoints_wghosts(p) * p->nvars;
  double *U = (double *)malloc(sizeof(double) * n);
  double *Udot = (double *)malloc(sizeof(double) * n * nstages);
  double t = p->t;
  for (int step = 0; step < nsteps; step++) {
    apply_bc_at(p, u, t); /* TimePreStep */
    for (int st = 0; st < nstages; st++) {
      memcpy(U, u, sizeof(double) * n);
      double c = 0.0; /* the stage's time fraction: the row sum of A (c of the tableau) */
      for (int i = 0; i < st; i++) {
        double a = dt * A[st * nstages + i];
        c += A[st * nstages + i];
        const double *k = Udot + (long)i * n;
#pragma omp parallel for schedule(static) num_threads(NTHR)
        for (long q = 0; q < n; q++) U[q] += a * k[q];
      }
      if (rhs_at(p, U, Udot + (long)st * n, t + c * dt)) {
        free(U);
        free(Udot);
        return -1;
      }
    }
    for (int st = 0; st < nstages; st++) {
      double a = dt * b[st];
      const double *k = Udot + (long)st * n;
#pragma omp parallel for schedule(static) num_threads(NTHR)
      for (long q = 0; q < n; q++) u[q] += a * k[q];
    }
    t += dt;
  }
  free(U);
  free(Udot);
  return 0;
}
