/*
 * gbh_inputs.c -- HyPar input decks on the host (C).
 *
 * Reads the files HyPar reads for this path, with the reference's formats and
 * defaults:
 *   solver.inp   ReadInputs           (src/Simulation/ReadInputs.c:94-440)
 *   physics.inp  Euler1DInitialize / Euler2DInitialize / NavierStokes3DInitialize
 *                (src/PhysicalModels/Euler1D/Euler1DInitialize.c:71-140,
 *                 Euler2D/Euler2DInitialize.c:21-70, NavierStokes3D/NavierStokes3DInitialize.c:116-370)
 *   weno.inp     WENOInitialize       (src/InterpolationFunctions/WENOInitialize.c:34-112)
 *   boundary.inp InitializeBoundaries (src/Simulation/InitializeBoundaries.c:75-180)
 *                with the index extents of CalculateLocalExtent (:365-420) and
 *                FindInterval (src/MathFunctions/FindInterval.c:19-45)
 *   initial.inp  ReadArraySerial      (src/IOFunctions/ReadArray.c:150-300), ghost grid
 *                extrapolation (:68-88) and dxinv (src/Simulation/InitialSolution.c:69-99)
 * Options outside this library's path (other models, schemes, boundary types,
 * gravity, MPI decompositions) are rejected with GB_ERR_UNSUPPORTED.
 */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "gbhypar.h"

void gbh_set_error(const char *fmt, ...);

struct gb_inputs {
  gb_config cfg;
  double *x;      /* interior grid, sum dim */
  double *dxinv;  /* with ghosts */
  double *u0;     /* interior solution */
  double *uex;    /* exact solution (exact.inp), or NULL */
  double *grav;   /* gravity fields f then g at every point with ghosts, or NULL */
  /* thermal walls: per zone the wall temperature's time levels and field, or NULL */
  int tn[GB_MAX_ZONES];
  double *ttimes[GB_MAX_ZONES], *tfield[GB_MAX_ZONES];
  /* sponge zones: per zone sigma along the zone's dimension, or NULL */
  int sn[GB_MAX_ZONES];
  double *sigma[GB_MAX_ZONES];
  /* turbulent inflow zones: per zone the number of slices and the inflow data, or NULL */
  int fn[GB_MAX_ZONES];
  double *fdata[GB_MAX_ZONES];
  char op_overwrite[64];
  char op_format[64];
};

#define MAXS 512

static FILE *open_in(const char *dir, const char *name, const char *mode) {
  char path[4096];
  if (dir && dir[0]) snprintf(path, sizeof(path), "%s/%s", dir, name);
  else snprintf(path, sizeof(path), "%s", name);
  return fopen(path, mode);
}

int gb_rk_table(const char *type, int *ns, double *A, double *b, double *c) {
  /* TimeExplicitRKInitialize (src/TimeIntegration/TimeExplicitRKInitialize.c:28-80) */
  for (int i = 0; i < 16; i++) A[i] = 0.0;
  for (int i = 0; i < 4; i++) b[i] = c[i] = 0.0;
  if (!strcmp(type, "1fe")) {
    *ns = 1;
    b[0] = 1.0;
  } else if (!strcmp(type, "22")) {
    *ns = 2;
    A[2] = 1.0;
    c[1] = 1.0;
    b[0] = b[1] = 0.5;
  } else if (!strcmp(type, "33")) {
    *ns = 3;
    A[3] = 2.0 / 3.0;
    A[6] = 2.0 / 3.0 - 1.0 / 4.0;
    A[7] = 1.0 / 4.0;
    c[1] = 2.0 / 3.0;
    c[2] = 2.0 / 3.0;
    b[0] = 1.0 / 4.0;
    b[1] = -1.0 / 4.0;
    b[2] = 1.0;
  } else if (!strcmp(type, "44")) {
    *ns = 4;
    A[4] = 0.5;
    A[9] = 0.5;
    A[14] = 1.0;
    c[1] = c[2] = 0.5;
    c[3] = 1.0;
    b[0] = 1.0 / 6.0;
    b[1] = 1.0 / 3.0;
    b[2] = 1.0 / 3.0;
    b[3] = 1.0 / 6.0;
  } else if (!strcmp(type, "ssprk3") || !strcmp(type, "tvdrk3")) {
    *ns = 3;
    A[3] = 1.0;
    A[6] = 0.25;
    A[7] = 0.25;
    c[1] = 1.0;
    c[2] = 0.5;
    b[0] = b[1] = 1.0 / 6.0;
    b[2] = 2.0 / 3.0;
  } else {
    gbh_set_error("time_scheme_type %s is not an explicit RK scheme of this library", type);
    return GB_ERR_UNSUPPORTED;
  }
  /* store A with row stride 4 */
  double T[16];
  for (int i = 0; i < 16; i++) T[i] = 0.0;
  for (int i = 0; i < *ns; i++)
    for (int j = 0; j < *ns; j++) T[4 * i + j] = A[(*ns) * i + j];
  for (int i = 0; i < 16; i++) A[i] = T[i];
  return GB_OK;
}

/* FindInterval (src/MathFunctions/FindInterval.c:19-45). */
static void find_interval(double a, double b, const double *x, int N, int *imin, int *imax) {
  *imax = -1;
  *imin = N;
  double min_dx = x[1] - x[0];
  for (int i = 2; i < N; i++) {
    double dx = x[i] - x[i - 1];
    if (dx < min_dx) min_dx = dx;
  }
  double tol = 1e-10 * min_dx;
  for (int i = 0; i < N; i++)
    if (x[i] <= (b + tol)) *imax = i + 1;
  for (int i = N - 1; i > -1; i--)
    if (x[i] >= (a - tol)) *imin = i;
}

typedef struct {
  int ndims, nvars, ghosts, n_iter, file_op_iter, restart_iter, screen_op_iter;
  int size[3], iproc[3];
  int member, nsims;   /* which simulation of an ensemble (simulation.inp) */
  double dt;
  char time_scheme[MAXS], time_scheme_type[MAXS], hyp_space_scheme[MAXS], interp_type[MAXS];
  char par_space_type[MAXS], par_space_scheme[MAXS], model[MAXS], ip_file_type[MAXS];
  char op_overwrite[MAXS], hyp_flux_split[MAXS], cons_check[MAXS], op_format[MAXS], input_mode[MAXS];
  char ib_file[MAXS];      /* immersed_body ("none": no immersed body) */
  int size_ex[3], have_size_ex;
} solver_inp;

static int read_solver_inp(const char *dir, solver_inp *si, int member, int nsims) {
  memset(si, 0, sizeof(*si));
  si->member = member;
  si->nsims = nsims;
  si->ndims = 1;
  si->nvars = 1;
  si->ghosts = 1;
  si->file_op_iter = 1000;
  si->screen_op_iter = 1;
  strcpy(si->time_scheme, "euler");
  strcpy(si->time_scheme_type, " ");
  strcpy(si->hyp_space_scheme, "1");
  strcpy(si->interp_type, "characteristic");
  strcpy(si->par_space_type, "nonconservative-1stage");
  strcpy(si->par_space_scheme, "2");
  strcpy(si->ip_file_type, "ascii");
  strcpy(si->op_overwrite, "no");
  strcpy(si->model, "none");
  strcpy(si->hyp_flux_split, "no");
  strcpy(si->ib_file, "none");
  strcpy(si->cons_check, "no");
  strcpy(si->op_format, "text");  /* ReadInputs.c:140 */
  strcpy(si->input_mode, "serial");
  FILE *in = open_in(dir, "solver.inp", "r");
  if (!in) {
    gbh_set_error("file solver.inp not found");
    return GB_ERR_INPUT;
  }
  char w[MAXS];
  int ok = 1;
  if (fscanf(in, "%511s", w) != 1 || strcmp(w, "begin")) {
    fclose(in);
    gbh_set_error("illegal format in solver.inp");
    return GB_ERR_INPUT;
  }
  int have_ndims = 0;
  while (ok) {
    if (fscanf(in, "%511s", w) != 1) { ok = 0; break; }
    if (!strcmp(w, "end")) break;
    int r = 1;
    if (!strcmp(w, "ndims")) { r = fscanf(in, "%d", &si->ndims); have_ndims = 1; }
    else if (!strcmp(w, "nvars")) r = fscanf(in, "%d", &si->nvars);
    else if (!strcmp(w, "size") || !strcmp(w, "iproc") || !strcmp(w, "size_exact")) {
      if (!have_ndims || si->ndims < 1 || si->ndims > 3) { ok = 0; break; }
      /* "size" lists ndims values for every simulation of an ensemble
         (ReadInputs.c:189-206); "iproc" and "size_exact" likewise per simulation */
      int *dst = !strcmp(w, "size") ? si->size : (!strcmp(w, "iproc") ? si->iproc : si->size_ex);
      if (!strcmp(w, "size_exact")) si->have_size_ex = 1;
      for (int n = 0; n < si->nsims && r == 1; n++)
        for (int d = 0; d < si->ndims; d++) {
          int val;
          r = fscanf(in, "%d", &val);
          if (r != 1) break;
          if (dst && n == si->member) dst[d] = val;
        }
    }
    else if (!strcmp(w, "ghost")) r = fscanf(in, "%d", &si->ghosts);
    else if (!strcmp(w, "n_iter")) r = fscanf(in, "%d", &si->n_iter);
    else if (!strcmp(w, "time_scheme")) r = fscanf(in, "%511s", si->time_scheme);
    else if (!strcmp(w, "time_scheme_type")) r = fscanf(in, "%511s", si->time_scheme_type);
    else if (!strcmp(w, "hyp_space_scheme")) r = fscanf(in, "%511s", si->hyp_space_scheme);
    else if (!strcmp(w, "hyp_flux_split")) r = fscanf(in, "%511s", si->hyp_flux_split);
    else if (!strcmp(w, "hyp_interp_type")) r = fscanf(in, "%511s", si->interp_type);
    else if (!strcmp(w, "par_space_type")) r = fscanf(in, "%511s", si->par_space_type);
    else if (!strcmp(w, "par_space_scheme")) r = fscanf(in, "%511s", si->par_space_scheme);
    else if (!strcmp(w, "dt")) r = fscanf(in, "%lf", &si->dt);
    else if (!strcmp(w, "file_op_iter")) r = fscanf(in, "%d", &si->file_op_iter);
    else if (!strcmp(w, "restart_iter")) r = fscanf(in, "%d", &si->restart_iter);
    else if (!strcmp(w, "screen_op_iter")) r = fscanf(in, "%d", &si->screen_op_iter);
    else if (!strcmp(w, "ip_file_type")) r = fscanf(in, "%511s", si->ip_file_type);
    else if (!strcmp(w, "op_overwrite")) r = fscanf(in, "%511s", si->op_overwrite);
    else if (!strcmp(w, "model")) r = fscanf(in, "%511s", si->model);
    else if (!strcmp(w, "conservation_check")) r = fscanf(in, "%511s", si->cons_check);
    else if (!strcmp(w, "op_file_format")) r = fscanf(in, "%511s", si->op_format);
    else if (!strcmp(w, "immersed_body")) r = fscanf(in, "%511s", si->ib_file);
    else if (!strcmp(w, "input_mode") || !strcmp(w, "output_mode")) {
      char mode[MAXS];
      r = fscanf(in, "%511s", mode);
      if (r == 1 && strcmp(mode, "serial")) { int nio; r = fscanf(in, "%d", &nio); }
      if (r == 1 && !strcmp(w, "input_mode")) snprintf(si->input_mode, MAXS, "%s", mode);
    } else {
      char useless[MAXS];  /* every other keyword takes one value */
      r = fscanf(in, "%511s", useless);
    }
    if (r != 1) ok = 0;
  }
  fclose(in);
  if (!ok) {
    gbh_set_error("could not parse solver.inp");
    return GB_ERR_INPUT;
  }
  return GB_OK;
}

static void grid_ghosts(const double *x, int n, int g, double *X);

/* The hydrostatic fields of NavierStokes3DGravityField.c:36-153: f (density) and g
 * (pressure) from the grid with ghost coordinates for the balance type HB, then
 * every face's ghost layer copied from its mirror interior points.
 * raiseto(x, a) = exp(a log x) (include/math_ops.h:37). */
static int gravity_fields(const gb_config *c, gb_inputs *res) {
  const int g = c->ghosts;
  long n[3] = {c->dim[0] + 2 * g, c->dim[1] + 2 * g, c->dim[2] + 2 * g}, np = n[0] * n[1] * n[2];
  double *X[3];
  long off = 0;
  for (int d = 0; d < 3; d++) {
    X[d] = (double *)malloc(sizeof(double) * n[d]);
    grid_ghosts(res->x + off, c->dim[d], g, X[d]);
    off += c->dim[d];
  }
  res->grav = (double *)malloc(sizeof(double) * 2 * np);
  double *f = res->grav, *gg = res->grav + np;
  const double gx = c->gravity[0], gy = c->gravity[1], gz = c->gravity[2];
  const double p0 = c->p_ref, rho0 = c->rho_ref, RT = p0 / rho0, gamma = c->gamma, R = c->R_gas;
  const double Cp = gamma * R / (gamma - 1.0), T0 = p0 / (rho0 * R), Nbv = c->N_bv;
  if (c->HB == 3 && (gx != 0 || gy != 0)) {
    for (int d = 0; d < 3; d++) free(X[d]);
    gbh_set_error("HB = 3 is implemented only for gravity along z");
    return GB_ERR_INPUT;
  }
  for (long k = 0; k < n[2]; k++)
    for (long j = 0; j < n[1]; j++)
      for (long i = 0; i < n[0]; i++) {
        const long p = i + n[0] * (j + n[1] * k);
        const double x = X[0][i], y = X[1][j], z = X[2][k];
        if (c->HB == 1) {
          f[p] = exp((gx * x + gy * y + gz * z) / RT);
          gg[p] = exp(-(gx * x + gy * y + gz * z) / RT);
        } else if (c->HB == 2) {
          f[p] = exp((-1.0 / (gamma - 1.0)) * log((1.0 - (gx * x + gy * y + gz * z) / (Cp * T0))));
          gg[p] = exp((gamma / (gamma - 1.0)) * log((1.0 - (gx * x + gy * y + gz * z) / (Cp * T0))));
        } else if (c->HB == 3) {
          double Pexner = 1 + ((gz * gz) / (Cp * T0 * Nbv * Nbv)) * (exp(-(Nbv * Nbv / gz) * z) - 1.0);
          f[p] = exp((-1.0 / (gamma - 1.0)) * log(Pexner)) * exp(Nbv * Nbv * z / gz);
          gg[p] = exp((gamma / (gamma - 1.0)) * log(Pexner));
        } else {
          f[p] = gg[p] = 1.0;
        }
      }
  for (int d = 0; d < 3; d++) {
    long b[3] = {c->dim[0], c->dim[1], c->dim[2]};
    b[d] = g;
    for (int side = 0; side < 2; side++)
      for (long c2 = 0; c2 < b[2]; c2++)
        for (long c1 = 0; c1 < b[1]; c1++)
          for (long c0 = 0; c0 < b[0]; c0++) {
            long ib[3] = {c0, c1, c2}, gi[3], ii[3];
            for (int e = 0; e < 3; e++) gi[e] = ii[e] = ib[e] + g;
            if (side == 0) {
              gi[d] = ib[d];
              ii[d] = g + (g - 1 - ib[d]);
            } else {
              gi[d] = c->dim[d] + g + ib[d];
              ii[d] = g + (c->dim[d] - 1 - ib[d]);
            }
            long q1 = gi[0] + n[0] * (gi[1] + n[1] * gi[2]), q2 = ii[0] + n[0] * (ii[1] + n[1] * ii[2]);
            f[q1] = f[q2];
            gg[q1] = gg[q2];
          }
  }
  for (int d = 0; d < 3; d++) free(X[d]);
  return GB_OK;
}

/* Euler1DGravityField (Euler1DGravityField.c:23-95): S = exp(-g x) (gravity_type 0) or
 * exp(-phi), phi = -sin(2 pi x)/(2 pi) (type 1), from the grid with ghost coordinates;
 * for type 0 the ghost layers copied from their mirror interior points.  Stored as
 * 1.0/S then S (the modified solution and the source scale by the first, the
 * dissipation by the second). */
static int gravity_field_1d(const gb_config *c, gb_inputs *res) {
  const int g = c->ghosts, N = c->dim[0];
  const long n = N + 2 * g;
  double *X = (double *)malloc(sizeof(double) * n);
  grid_ghosts(res->x, N, g, X);
  res->grav = (double *)malloc(sizeof(double) * 2 * n);
  double *f = res->grav, *S = res->grav + n;
  for (long i = 0; i < n; i++) {
    if (c->grav_type == 0) {
      S[i] = exp(-c->gravity[0] * X[i]);
    } else {
      double pi = 4.0 * atan(1.0);
      double phi = -sin(2 * pi * X[i]) / (2 * pi);
      S[i] = exp(-phi);
    }
  }
  if (c->grav_type != 1)
    for (int b = 0; b < g; b++) {
      S[b] = S[g + (g - 1 - b)];
      S[N + g + b] = S[g + (N - 1 - b)];
    }
  for (long i = 0; i < n; i++) f[i] = 1.0 / S[i];
  free(X);
  return GB_OK;
}

/* A solution file in HyPar's input format (ReadArray.c): binary = x then u
 * (point-major); ascii = x then u variable by variable.  Returns -1 (no error
 * message) when the file is absent and `required` is 0. */
static int read_solution(const char *dir, const char *name, const char *type, long nx, long npts, int nvars,
                         double *x, double *u, int required) {
  int bin = !strcmp(type, "bin") || !strcmp(type, "binary");
  if (!bin && strcmp(type, "ascii")) {
    gbh_set_error("ip_file_type %s invalid", type);
    return GB_ERR_INPUT;
  }
  FILE *in = open_in(dir, name, bin ? "rb" : "r");
  if (!in) {
    if (!required) return -1;
    gbh_set_error("solution file %s not found", name);
    return GB_ERR_INPUT;
  }
  int bad = 0;
  if (bin) {
    size_t a = fread(x, sizeof(double), nx, in);
    size_t b = fread(u, sizeof(double), npts * nvars, in);
    bad = (long)a != nx || (long)b != npts * nvars;
  } else {
    for (long i = 0; i < nx && !bad; i++) bad = fscanf(in, "%lf", &x[i]) != 1;
    for (int v = 0; v < nvars && !bad; v++)
      for (long p = 0; p < npts && !bad; p++) bad = fscanf(in, "%lf", &u[p * nvars + v]) != 1;
  }
  fclose(in);
  if (bad) {
    gbh_set_error("%s is too short or malformed", name);
    return GB_ERR_INPUT;
  }
  return GB_OK;
}

/* Generic "begin key value ... end" reader for physics.inp / weno.inp. */
typedef struct { const char *key; char type; void *dst; } kv_t;
typedef struct { int hb; double nbv; } hb_t;

static int read_kv_file(const char *dir, const char *name, kv_t *kv, int nkv, int required) {
  FILE *in = open_in(dir, name, "r");
  if (!in) {
    if (required) {
      gbh_set_error("file %s not found", name);
      return GB_ERR_INPUT;
    }
    return GB_OK; /* reference: optional, defaults apply */
  }
  char w[MAXS];
  if (fscanf(in, "%511s", w) != 1 || strcmp(w, "begin")) {
    fclose(in);
    gbh_set_error("illegal format in %s", name);
    return GB_ERR_INPUT;
  }
  for (;;) {
    if (fscanf(in, "%511s", w) != 1) {
      fclose(in);
      gbh_set_error("could not parse %s", name);
      return GB_ERR_INPUT;
    }
    if (!strcmp(w, "end")) break;
    int found = 0, r = 1;
    for (int i = 0; i < nkv; i++) {
      if (strcmp(w, kv[i].key)) continue;
      found = 1;
      if (kv[i].type == 'd') r = fscanf(in, "%lf", (double *)kv[i].dst);
      else if (kv[i].type == 'i') r = fscanf(in, "%d", (int *)kv[i].dst);
      else if (kv[i].type == 'v') {  /* three doubles (physics.inp gravity) */
        double *v3 = (double *)kv[i].dst;
        r = fscanf(in, "%lf %lf %lf", &v3[0], &v3[1], &v3[2]) == 3;
      } else if (kv[i].type == 'h') {  /* HB, and N_bv after HB = 3 (NavierStokes3DInitialize.c:238-250) */
        hb_t *hb = (hb_t *)kv[i].dst;
        r = fscanf(in, "%d", &hb->hb);
        if (r == 1 && hb->hb == 3) r = fscanf(in, "%lf", &hb->nbv);
      } else r = fscanf(in, "%511s", (char *)kv[i].dst);
      break;
    }
    if (!found) {
      char useless[MAXS];
      r = fscanf(in, "%511s", useless);
    }
    if (r != 1) {
      fclose(in);
      gbh_set_error("could not parse %s", name);
      return GB_ERR_INPUT;
    }
  }
  fclose(in);
  return GB_OK;
}

static void grid_ghosts(const double *x, int n, int g, double *X) {
  for (int i = 0; i < n; i++) X[g + i] = x[i];
  for (int i = 0; i < g; i++) {
    int delta = g - i;
    X[i] = X[g] + ((double)delta) * (X[g] - X[g + 1]);
  }
  for (int i = n + g; i < n + 2 * g; i++) {
    int delta = i - (n + g - 1);
    X[i] = X[n + g - 1] + ((double)delta) * (X[n + g - 1] - X[n + g - 2]);
  }
}

void gb_inputs_free(gb_inputs *in) {
  if (!in) return;
  free(in->x);
  free(in->dxinv);
  free(in->u0);
  free(in->uex);
  free(in->grav);
  for (int z = 0; z < GB_MAX_ZONES; z++) {
    free(in->ttimes[z]);
    free(in->tfield[z]);
    free(in->sigma[z]);
    free(in->fdata[z]);
  }
  free(in);
}

int gb_inputs_zone_inflow(const gb_inputs *in, int zone, int *n, const double **data) {
  if (!in || !n || !data || zone < 0 || zone >= GB_MAX_ZONES) {
    gbh_set_error("gb_inputs_zone_inflow: bad argument");
    return GB_ERR_ARG;
  }
  *n = in->fn[zone];
  *data = in->fdata[zone];
  return GB_OK;
}

int gb_inputs_zone_sponge(const gb_inputs *in, int zone, int *n, const double **sigma) {
  if (!in || !n || !sigma || zone < 0 || zone >= GB_MAX_ZONES) {
    gbh_set_error("gb_inputs_zone_sponge: bad argument");
    return GB_ERR_ARG;
  }
  *n = in->sn[zone];
  *sigma = in->sigma[zone];
  return GB_OK;
}

int gb_inputs_zone_temperature(const gb_inputs *in, int zone, int *ntimes, const double **times,
                               const double **field) {
  if (!in || !ntimes || !times || !field || zone < 0 || zone >= GB_MAX_ZONES) {
    gbh_set_error("gb_inputs_zone_temperature: bad argument");
    return GB_ERR_ARG;
  }
  *ntimes = in->tn[zone];
  *times = in->ttimes[zone];
  *field = in->tfield[zone];
  return GB_OK;
}

/* The wall temperature file of a thermal-wall zone (BCReadTemperatureData,
 * src/BoundaryConditions/BCIO.c:147-260, one rank): int rank[ndims], int size[ndims]
 * (size[dim]: the number of time levels; the other sizes: the zone's extent), double
 * times[size[dim]], double field[prod size], dimension 0 fastest. */
static int read_temperature(const char *dir, const char *name, const gb_config *c, const int *zone,
                            gb_inputs *res, int z) {
  FILE *f = open_in(dir, name, "rb");
  if (!f) {
    gbh_set_error("boundary.inp zone %d: cannot open the temperature file %s", z, name);
    return GB_ERR_INPUT;
  }
  const int nd = c->ndims, dim = zone[1];
  int rank[3] = {0, 0, 0}, size[3] = {1, 1, 1};
  int bad = fread(rank, sizeof(int), nd, f) != (size_t)nd || fread(size, sizeof(int), nd, f) != (size_t)nd;
  long total = 1;
  for (int d = 0; d < nd && !bad; d++) {
    if (size[d] < 1) bad = 1;
    else if (d != dim && size[d] != zone[6 + d] - zone[3 + d]) bad = 2;
    total *= size[d];
  }
  if (bad) {
    fclose(f);
    gbh_set_error("temperature file %s: %s", name,
                  bad == 2 ? "its size does not match the zone's extent" : "malformed header");
    return GB_ERR_INPUT;
  }
  res->tn[z] = size[dim];
  res->ttimes[z] = (double *)malloc(sizeof(double) * size[dim]);
  res->tfield[z] = (double *)malloc(sizeof(double) * total);
  if (fread(res->ttimes[z], sizeof(double), size[dim], f) != (size_t)size[dim] ||
      fread(res->tfield[z], sizeof(double), total, f) != (size_t)total) {
    fclose(f);
    gbh_set_error("temperature file %s: truncated", name);
    return GB_ERR_INPUT;
  }
  fclose(f);
  return GB_OK;
}

/* The inflow data file of a turbulent supersonic inflow zone (BCReadTurbulentInflowData,
 * src/BoundaryConditions/BCIO.c:19-139, one rank): int rank[ndims] (all 0), int
 * size[ndims] (size[dim]: the number of slices; the other sizes: the grid's), then
 * nvars doubles per point, dimension 0 fastest. */
static int read_inflow(const char *dir, const char *name, const gb_config *c, const int *zone, gb_inputs *res,
                       int z) {
  FILE *f = open_in(dir, name, "rb");
  if (!f) {
    gbh_set_error("boundary.inp zone %d: cannot open the inflow data file %s", z, name);
    return GB_ERR_INPUT;
  }
  const int nd = c->ndims, dim = zone[1];
  int rank[3] = {0, 0, 0}, size[3] = {1, 1, 1};
  int bad = fread(rank, sizeof(int), nd, f) != (size_t)nd || fread(size, sizeof(int), nd, f) != (size_t)nd;
  long total = c->nvars;
  for (int d = 0; d < nd && !bad; d++) {
    if (size[d] < 1) bad = 1;
    else if (rank[d] != 0) bad = 3;
    else if (d != dim && size[d] != c->dim[d]) bad = 2;
    total *= size[d];
  }
  if (bad) {
    fclose(f);
    gbh_set_error("inflow data file %s: %s", name,
                  bad == 2 ? "its size does not match the grid" : bad == 3 ? "data of a rank other than 0"
                                                                        : "malformed header");
    return GB_ERR_INPUT;
  }
  res->fn[z] = size[dim];
  res->fdata[z] = (double *)malloc(sizeof(double) * total);
  if (!res->fdata[z] || fread(res->fdata[z], sizeof(double), total, f) != (size_t)total) {
    fclose(f);
    gbh_set_error("inflow data file %s: truncated", name);
    return GB_ERR_INPUT;
  }
  fclose(f);
  return GB_OK;
}

const gb_config *gb_inputs_config(const gb_inputs *in) { return in ? &in->cfg : NULL; }
const double *gb_inputs_x(const gb_inputs *in) { return in ? in->x : NULL; }
const double *gb_inputs_dxinv(const gb_inputs *in) { return in ? in->dxinv : NULL; }
const double *gb_inputs_u0(const gb_inputs *in) { return in ? in->u0 : NULL; }
const double *gb_inputs_exact(const gb_inputs *in) { return in ? in->uex : NULL; }
const double *gb_inputs_gravity_field(const gb_inputs *in) { return in ? in->grav : NULL; }
const char *gbh_inputs_op_overwrite(const gb_inputs *in) { return in ? in->op_overwrite : "yes"; }
const char *gbh_inputs_op_format(const gb_inputs *in) { return in ? in->op_format : "binary"; }

int gb_inputs_nsims(const char *dir) {
  /* simulation.inp (src/Simulation/EnsembleSimulationsDefine.cpp:41-70): "begin nsims N end" */
  FILE *in = open_in(dir, "simulation.inp", "r");
  if (!in) return 1;
  char w[MAXS];
  int n = 1;
  if (fscanf(in, "%511s", w) == 1 && !strcmp(w, "begin")) {
    while (fscanf(in, "%511s", w) == 1 && strcmp(w, "end")) {
      if (!strcmp(w, "nsims")) {
        if (fscanf(in, "%d", &n) != 1) n = -1;
      } else {
        char useless[MAXS];
        if (fscanf(in, "%511s", useless) != 1) break;
      }
    }
  } else {
    n = -1;
  }
  fclose(in);
  return n;
}

static void member_name(char *out, size_t sz, const char *root, int member, int nsims) {
  /* <root>_<index>.inp with the index zero-padded to (int)log10(nsims)+1 digits
     (InitialSolution.c:36-41, GetStringFromInteger) */
  if (nsims <= 1) {
    snprintf(out, sz, "%s.inp", root);
    return;
  }
  int width = (int)log10((double)nsims) + 1;
  snprintf(out, sz, "%s_%0*d.inp", root, width, member);
}

/* The solution file of solver.inp's input_mode (ReadArray.c:41-56): serial reads
 * <root>.inp in ip_file_type; "parallel" the one I/O rank's binary file
 * <root>_par.inp.0000 (ReadArrayParallel, :355-380: its grid then its solution,
 * which on one rank is the whole of each); "mpi-io" the binary <root>_mpi.inp
 * (ReadArrayMPI_IO, :532-540). */
static const char *input_file(char *out, size_t sz, const char *root, int member, int nsims, const char *mode,
                              const char *ip_type) {
  char base[240];
  member_name(base, sizeof(base), root, member, nsims);
  if (!strcmp(mode, "serial")) {
    snprintf(out, sz, "%s", base);
    return ip_type;
  }
  base[strlen(base) - 4] = 0;  /* drop ".inp" */
  if (!strcmp(mode, "parallel")) snprintf(out, sz, "%s_par.inp.0000", base);
  else snprintf(out, sz, "%s_mpi.inp", base);
  return "binary";
}

int gb_inputs_read(const char *dir, gb_inputs **out) { return gb_inputs_read_member(dir, 0, 1, out); }

int gb_inputs_read_member(const char *dir, int member, int nsims, gb_inputs **out) {
  if (!out || nsims < 1 || member < 0 || member >= nsims) {
    gbh_set_error("gb_inputs_read_member: bad argument");
    return GB_ERR_ARG;
  }
  *out = NULL;
  solver_inp si;
  int rc = read_solver_inp(dir, &si, member, nsims);
  if (rc) return rc;
  gb_config c;
  memset(&c, 0, sizeof(c));
  if (!strcmp(si.model, "euler1d")) c.model = GB_MODEL_EULER1D;
  else if (!strcmp(si.model, "euler2d")) c.model = GB_MODEL_EULER2D;
  else if (!strcmp(si.model, "navierstokes3d")) c.model = GB_MODEL_NS3D;
  else {
    gbh_set_error("model %s is not one of euler1d, euler2d, navierstokes3d", si.model);
    return GB_ERR_UNSUPPORTED;
  }
  int want_nd = c.model == GB_MODEL_EULER1D ? 1 : (c.model == GB_MODEL_EULER2D ? 2 : 3);
  int want_nv = want_nd + 2;
  if (si.ndims != want_nd || si.nvars != want_nv) {
    gbh_set_error("%s needs ndims %d and nvars %d", si.model, want_nd, want_nv);
    return GB_ERR_INPUT;
  }
  c.ndims = si.ndims;
  c.nvars = si.nvars;
  c.ghosts = si.ghosts;
  for (int d = 0; d < 3; d++) c.dim[d] = d < c.ndims ? si.size[d] : 1;
  for (int d = 0; d < c.ndims; d++) {
    /* three points are the fewest whose ghost layers (3 deep) the boundaries fill from
     * interior points: the quasi-2-D NavierStokes3D decks run with 3 along z */
    if (c.dim[d] < 3) {
      gbh_set_error("size along dimension %d is %d (at least 3 needed)", d, c.dim[d]);
      return GB_ERR_INPUT;
    }
    if (si.iproc[d] > 1) fprintf(stderr, "gbhypar: iproc %d along dimension %d ignored (one GPU holds the whole domain)\n", si.iproc[d], d);
  }
  if (c.ghosts != 3) {
    gbh_set_error("ghost must be 3 for weno5 (got %d)", c.ghosts);
    return GB_ERR_UNSUPPORTED;
  }
  if (!strcmp(si.hyp_space_scheme, "weno5")) {
    c.hyp_scheme = GB_SCHEME_WENO5;
  } else if (!strcmp(si.hyp_space_scheme, "crweno5")) {
    c.hyp_scheme = GB_SCHEME_CRWENO5;
  } else {
    gbh_set_error("hyp_space_scheme %s not supported (weno5, crweno5)", si.hyp_space_scheme);
    return GB_ERR_UNSUPPORTED;
  }
  /* hyp_flux_split yes: only the implicit-explicit integrators split the flux
   * (ComputeRHSOperators.c); explicit Runge-Kutta evaluates the whole flux, so for
   * Euler1D and NavierStokes3D it changes nothing, and Euler2D refuses it
   * (Euler2DInitialize.c:79-85) */
  if (strcmp(si.hyp_flux_split, "no") && c.model == GB_MODEL_EULER2D) {
    gbh_set_error("hyp_flux_split %s: Euler2D has no splitting of the hyperbolic term", si.hyp_flux_split);
    return GB_ERR_INPUT;
  }
  if (strcmp(si.ib_file, "none")) {
    gbh_set_error("immersed_body %s: immersed boundaries are not available in this library", si.ib_file);
    return GB_ERR_UNSUPPORTED;
  }
  if (si.have_size_ex)
    for (int d = 0; d < si.ndims; d++)
      if (si.size_ex[d] != si.size[d]) {
        gbh_set_error("size_exact differs from size: an exact solution on another grid is not available");
        return GB_ERR_UNSUPPORTED;
      }
  if (!strcmp(si.interp_type, "components")) c.interp = GB_INTERP_COMPONENTS;
  else if (!strcmp(si.interp_type, "characteristic")) c.interp = GB_INTERP_CHARACTERISTIC;
  else {
    gbh_set_error("hyp_interp_type %s invalid", si.interp_type);
    return GB_ERR_INPUT;
  }
  /* forward Euler (solver.inp's default, TimeForwardEuler.c: u += dt RHS(u)) is the
   * one-stage table: the same update, bit for bit (dt b_0 = dt) */
  const int euler = !strcmp(si.time_scheme, "euler");
  if (strcmp(si.time_scheme, "rk") && !euler) {
    gbh_set_error("time_scheme %s not supported (rk and euler only)", si.time_scheme);
    return GB_ERR_UNSUPPORTED;
  }
  rc = gb_rk_table(euler ? "1fe" : si.time_scheme_type, &c.rk_nstages, c.rk_A, c.rk_b, c.rk_c);
  if (rc) return rc;
  c.dt = si.dt;
  c.n_iter = si.n_iter;
  c.file_op_iter = si.file_op_iter;
  c.restart_iter = si.restart_iter;
  c.screen_op_iter = si.screen_op_iter > 0 ? si.screen_op_iter : 1;
  c.cons_check = !strcmp(si.cons_check, "yes");  /* ReadInputs.c:323: "yes" turns it on */
  c.write_residual = 0;  /* the reference reads no keyword for it either (ReadInputs.c:125) */

  /* physics.inp */
  char upw[MAXS] = "roe";
  c.gamma = 1.4;
  c.Re = -1.0;
  c.Pr = 0.72;
  c.Minf = 1.0;
  double grav[3] = {0.0, 0.0, 0.0};
  hb_t hb = {0, 0.0};
  c.rho_ref = 1.0;
  c.p_ref = 1.0;
  c.R_gas = 1.0;
  /* NavierStokes3DInitialize.c:141-260 (gravity gx gy gz, ...); Euler1DInitialize.c:98-130
     (gravity g, gravity_type) */
  kv_t pk[] = {{"gamma", 'd', &c.gamma}, {"upwinding", 's', upw}, {"gravity", c.model == GB_MODEL_NS3D ? 'v' : 'd', grav},
               {"Pr", 'd', &c.Pr}, {"Re", 'd', &c.Re}, {"Minf", 'd', &c.Minf},
               {"rho_ref", 'd', &c.rho_ref}, {"p_ref", 'd', &c.p_ref}, {"R", 'd', &c.R_gas}, {"HB", 'h', &hb},
               {"gravity_type", 'i', &c.grav_type}};
  rc = read_kv_file(dir, "physics.inp", pk, 11, 0);
  if (rc) return rc;
  if (c.model == GB_MODEL_EULER2D && grav[0] != 0.0) {
    gbh_set_error("gravity: Euler2D has none");
    return GB_ERR_UNSUPPORTED;
  }
  for (int d = 0; d < 3; d++) c.gravity[d] = (c.model == GB_MODEL_NS3D || d == 0) ? grav[d] : 0.0;
  if (c.model == GB_MODEL_EULER2D) c.gravity[0] = 0.0;
  c.HB = hb.hb;
  c.N_bv = hb.nbv;
  if (!strcmp(upw, "roe")) c.upwind = GB_UPWIND_ROE;
  else if (!strcmp(upw, "llf-char")) c.upwind = GB_UPWIND_LLF;
  else if (!strcmp(upw, "rf-char")) c.upwind = GB_UPWIND_RF;
  else if (!strcmp(upw, "rusanov") && c.model != GB_MODEL_EULER2D) c.upwind = GB_UPWIND_RUSANOV;
  else if (!strcmp(upw, "steger-warming") && c.model != GB_MODEL_NS3D) c.upwind = GB_UPWIND_SWFS;
  else {
    gbh_set_error("upwinding %s not supported (roe, llf-char, rf-char; rusanov for Euler1D / NavierStokes3D; "
                  "steger-warming for Euler1D / Euler2D)", upw);
    return GB_ERR_UNSUPPORTED;
  }
  if (c.model == GB_MODEL_NS3D && (c.gravity[0] != 0.0 || c.gravity[1] != 0.0 || c.gravity[2] != 0.0) &&
      c.upwind != GB_UPWIND_RUSANOV) {
    /* NavierStokes3DInitialize.c:370-378 */
    gbh_set_error("rusanov upwinding is needed for flows with gravitational forces");
    return GB_ERR_INPUT;
  }
  if (c.model == GB_MODEL_EULER1D && c.gravity[0] != 0.0 && c.upwind != GB_UPWIND_ROE && c.upwind != GB_UPWIND_LLF) {
    /* Euler1DInitialize.c:144-150 */
    gbh_set_error("llf-char or roe upwinding is needed for flows with gravitational forces");
    return GB_ERR_INPUT;
  }
  if (c.model == GB_MODEL_EULER1D && c.gravity[0] != 0.0 && c.grav_type != 0 && c.grav_type != 1) {
    gbh_set_error("gravity_type %d not supported (0, 1)", c.grav_type);
    return GB_ERR_INPUT;
  }
  if (c.model == GB_MODEL_NS3D && c.Re > 0) {
    if (strcmp(si.par_space_type, "nonconservative-2stage")) {
      gbh_set_error("NavierStokes3D needs par_space_type nonconservative-2stage");
      return GB_ERR_INPUT;
    }
    if (strcmp(si.par_space_scheme, "4") && strcmp(si.par_space_scheme, "2")) {
      gbh_set_error("par_space_scheme %s not supported (2 or 4)", si.par_space_scheme);
      return GB_ERR_UNSUPPORTED;
    }
    c.par_scheme = !strcmp(si.par_space_scheme, "2") ? 2 : 4;
  }

  /* weno.inp */
  int mapped = 0, borges = 0, yc = 0, no_limiting = 0;
  c.weno_eps = 1e-6;
  kv_t wk[] = {{"mapped", 'i', &mapped}, {"borges", 'i', &borges}, {"yc", 'i', &yc},
               {"no_limiting", 'i', &no_limiting}, {"epsilon", 'd', &c.weno_eps}};
  rc = read_kv_file(dir, "weno.inp", wk, 5, 0);
  if (rc) return rc;
  /* WENOFifthOrderCalculateWeights.c:57-60 (yc, then borges, then mapped);
   * no_limiting skips the weights altogether (InitializeSolvers.c:219) */
  c.weno_weights = no_limiting ? GB_WENO_NONE
                 : yc          ? GB_WENO_YC
                 : borges      ? GB_WENO_BORGES
                 : mapped      ? GB_WENO_MAPPED
                               : GB_WENO_JS;

  gb_inputs *res = (gb_inputs *)calloc(1, sizeof(gb_inputs));
  snprintf(res->op_overwrite, sizeof(res->op_overwrite), "%s", si.op_overwrite);
  snprintf(res->op_format, sizeof(res->op_format), "%s", si.op_format);
  /* InitializeSolvers.c:419-436: text, tecplot2d, tecplot3d, binary / bin, none */
  if (strcmp(si.op_format, "text") && strcmp(si.op_format, "tecplot2d") && strcmp(si.op_format, "tecplot3d") &&
      strcmp(si.op_format, "binary") && strcmp(si.op_format, "bin") && strcmp(si.op_format, "none")) {
    gbh_set_error("%s is not a supported file format", si.op_format);
    gb_inputs_free(res);
    return GB_ERR_INPUT;
  }
  long nx = 0, nxg = 0, npts = 1;
  for (int d = 0; d < c.ndims; d++) {
    nx += c.dim[d];
    nxg += c.dim[d] + 2 * c.ghosts;
    npts *= c.dim[d];
  }
  res->x = (double *)calloc(nx, sizeof(double));
  res->dxinv = (double *)calloc(nxg, sizeof(double));
  res->u0 = (double *)calloc(npts * c.nvars, sizeof(double));

  /* initial.inp, and exact.inp when present (ExactSolution.c, same format) */
  char iname[256], bname[256], ename[256];
  if (strcmp(si.input_mode, "serial") && strcmp(si.input_mode, "parallel") && strcmp(si.input_mode, "mpi-io")) {
    gbh_set_error("input_mode %s invalid (serial, parallel, mpi-io)", si.input_mode);
    gb_inputs_free(res);
    return GB_ERR_INPUT;
  }
  const char *itype = input_file(iname, sizeof(iname), "initial", member, nsims, si.input_mode, si.ip_file_type);
  member_name(bname, sizeof(bname), "boundary", member, nsims);
  const char *etype = input_file(ename, sizeof(ename), "exact", member, nsims, si.input_mode, si.ip_file_type);
  rc = read_solution(dir, iname, itype, nx, npts, c.nvars, res->x, res->u0, 1);
  if (rc) {
    gb_inputs_free(res);
    return rc;
  }
  {
    double *xd = (double *)calloc(nx, sizeof(double));
    double *ue = (double *)calloc(npts * c.nvars, sizeof(double));
    rc = read_solution(dir, ename, etype, nx, npts, c.nvars, xd, ue, 0);
    free(xd);
    if (rc == GB_OK) {
      res->uex = ue;
    } else {
      free(ue);
      if (rc != -1) {
        gb_inputs_free(res);
        return rc;
      }
      rc = GB_OK;
    }
  }

  /* dxinv with ghosts */
  {
    long off = 0, offg = 0;
    for (int d = 0; d < c.ndims; d++) {
      int n = c.dim[d], g = c.ghosts;
      double *X = (double *)malloc(sizeof(double) * (n + 2 * g));
      grid_ghosts(res->x + off, n, g, X);
      double *D = res->dxinv + offg;
      for (int i = 0; i < n; i++) D[i + g] = 2.0 / (X[i + 1 + g] - X[i - 1 + g]);
      for (int i = 0; i < g; i++) D[i] = D[g];
      for (int i = n + g; i < n + 2 * g; i++) D[i] = D[n + g - 1];
      free(X);
      off += n;
      offg += n + 2 * g;
    }
  }

  /* gravity fields (NavierStokes3DGravityField.c:36-153, Euler1DGravityField.c:23-95) */
  if (c.gravity[0] != 0.0 || c.gravity[1] != 0.0 || c.gravity[2] != 0.0) {
    rc = c.model == GB_MODEL_EULER1D ? gravity_field_1d(&c, res) : gravity_fields(&c, res);
    if (rc) {
      gb_inputs_free(res);
      return rc;
    }
  }

  /* boundary_<index>.inp, else boundary.inp (InitializeBoundaries.c:55-75) */
  {
    FILE *in = open_in(dir, bname, "r");
    if (!in) in = open_in(dir, "boundary.inp", "r");
    if (!in) {
      gb_inputs_free(res);
      gbh_set_error("boundary condition file boundary.inp not found");
      return GB_ERR_INPUT;
    }
    int nb = 0;
    if (fscanf(in, "%d", &nb) != 1 || nb < 0 || nb > GB_MAX_ZONES) {
      fclose(in);
      gb_inputs_free(res);
      gbh_set_error("boundary.inp: bad zone count");
      return GB_ERR_INPUT;
    }
    c.nzones = nb;
    for (int z = 0; z < nb; z++) {
      char type[MAXS];
      int dim, face;
      double xmin[3], xmax[3];
      int bad = fscanf(in, "%511s %d %d", type, &dim, &face) != 3;
      for (int d = 0; d < c.ndims && !bad; d++) bad = fscanf(in, "%lf %lf", &xmin[d], &xmax[d]) != 2;
      if (bad || dim < 0 || dim >= c.ndims || (face != 1 && face != -1)) {
        fclose(in);
        gb_inputs_free(res);
        gbh_set_error("boundary.inp: bad zone %d", z);
        return GB_ERR_INPUT;
      }
      /* type-specific values after the extents (InitializeBoundaries.c:109-188) */
      static const struct { const char *name; int code; int nvals; } bct[] = {
          {"periodic", GB_BC_PERIODIC, 0},           {"extrapolate", GB_BC_EXTRAPOLATE, 0},
          {"dirichlet", GB_BC_DIRICHLET, -1},        {"slip-wall", GB_BC_SLIP_WALL, -2},
          {"noslip-wall", GB_BC_NOSLIP_WALL, -2},    {"subsonic-inflow", GB_BC_SUBSONIC_INFLOW, -3},
          {"subsonic-outflow", GB_BC_SUBSONIC_OUTFLOW, 1},
          {"supersonic-inflow", GB_BC_SUPERSONIC_INFLOW, -4},
          {"supersonic-outflow", GB_BC_SUPERSONIC_OUTFLOW, 0},
          {"subsonic-ambivalent", GB_BC_SUBSONIC_AMBIVALENT, -4},
          {"thermal-slip-wall", GB_BC_THERMAL_SLIP_WALL, -2},
          {"thermal-noslip-wall", GB_BC_THERMAL_NOSLIP_WALL, -2},
          {"sponge", GB_BC_SPONGE, -1},
          {"turbulent-supersonic-inflow", GB_BC_TURBULENT_INFLOW, -4},
          {"reflect", GB_BC_REFLECT, 0}};
      int tcode = 0, nvals = 0;
      for (size_t t = 0; t < sizeof(bct) / sizeof(bct[0]); t++)
        if (!strcmp(type, bct[t].name)) {
          tcode = bct[t].code;
          /* -1: nvars values; -2: ndims; -3: 1 + ndims; -4: 2 + ndims */
          nvals = bct[t].nvals == -1 ? c.nvars : bct[t].nvals == -2 ? c.ndims
                : bct[t].nvals == -3 ? 1 + c.ndims : bct[t].nvals == -4 ? 2 + c.ndims : bct[t].nvals;
        }
      if (!tcode) {
        fclose(in);
        gb_inputs_free(res);
        gbh_set_error("boundary type %s not supported", type);
        return GB_ERR_UNSUPPORTED;
      }
      for (int k = 0; k < 8; k++) c.zone_data[z][k] = 0.0;
      for (int k = 0; k < nvals && !bad; k++) bad = fscanf(in, "%lf", &c.zone_data[z][k]) != 1;
      /* thermal walls: then the name of the wall temperature file (InitializeBoundaries.c:180-187) */
      const int thermal = tcode == GB_BC_THERMAL_SLIP_WALL || tcode == GB_BC_THERMAL_NOSLIP_WALL;
      const int turbulent = tcode == GB_BC_TURBULENT_INFLOW;
      char tname[MAXS] = "";
      if (!bad && (thermal || turbulent)) bad = fscanf(in, "%511s", tname) != 1;
      if (bad) {
        fclose(in);
        gb_inputs_free(res);
        gbh_set_error("boundary.inp: zone %d (%s) lacks its values", z, type);
        return GB_ERR_INPUT;
      }
      /* BCSlipWall.c has a 1-D branch (Euler1D); the other wall and inflow / outflow
       * types have 2-D and 3-D ones only */
      if (tcode > GB_BC_DIRICHLET && tcode != GB_BC_SPONGE && tcode != GB_BC_REFLECT && tcode != GB_BC_SLIP_WALL &&
          c.ndims < 2) {
        fclose(in);
        gb_inputs_free(res);
        gbh_set_error("boundary type %s needs Euler2D or NavierStokes3D", type);
        return GB_ERR_UNSUPPORTED;
      }
      if ((thermal || turbulent) && c.model != GB_MODEL_NS3D) {
        fclose(in);
        gb_inputs_free(res);
        gbh_set_error("boundary type %s needs NavierStokes3D (the reference's branch is 3-D only)", type);
        return GB_ERR_UNSUPPORTED;
      }
      int *zz = c.zones[z];
      zz[0] = tcode;
      zz[1] = dim;
      zz[2] = face;
      long off = 0;
      for (int d = 0; d < 3; d++) {
        int is = 0, ie = 1;
        if (d < c.ndims) {
          if (d == dim && tcode != GB_BC_SPONGE) {
            if (face == 1) { is = -c.ghosts; ie = 0; }
            else { is = c.dim[d]; ie = c.dim[d] + c.ghosts; }
          } else {
            find_interval(xmin[d], xmax[d], res->x + off, c.dim[d], &is, &ie);
          }
          off += c.dim[d];
        }
        zz[3 + d] = is;
        zz[6 + d] = ie;
      }
      if (tcode == GB_BC_SPONGE) {
        /* sigma over the zone's indices along its dimension (BCSponge.c:49-54) */
        long xo = 0;
        for (int d = 0; d < dim; d++) xo += c.dim[d];
        const int n = zz[6 + dim] > zz[3 + dim] ? zz[6 + dim] - zz[3 + dim] : 0;
        res->sn[z] = n;
        if (n) {
          res->sigma[z] = (double *)malloc(sizeof(double) * n);
          if (!res->sigma[z]) {
            fclose(in);
            gb_inputs_free(res);
            gbh_set_error("out of host memory");
            return GB_ERR_NOMEM;
          }
          const double xs = xmin[dim], xe = xmax[dim];
          for (int k = 0; k < n; k++) {
            const double xk = res->x[xo + zz[3 + dim] + k];
            res->sigma[z][k] = face > 0 ? (xk - xs) / (xe - xs) : (xk - xe) / (xs - xe);
          }
        }
      }
      if (turbulent) {
        int rc = read_inflow(dir, tname, &c, zz, res, z);
        if (rc) {
          fclose(in);
          gb_inputs_free(res);
          return rc;
        }
      }
      if (thermal) {
        int rc = read_temperature(dir, tname, &c, zz, res, z);
        if (rc) {
          fclose(in);
          gb_inputs_free(res);
          return rc;
        }
      }
    }
    fclose(in);
  }
  res->cfg = c;
  *out = res;
  return GB_OK;
}

int gb_write_binary(const char *path, int ndims, int nvars, const int *dim, const double *x, const double *u) {
  /* WriteBinary (src/IOFunctions/WriteBinary.c) */
  FILE *out = fopen(path, "wb");
  if (!out) {
    gbh_set_error("could not open %s for writing", path);
    return GB_ERR_INPUT;
  }
  long nx = 0, n = 1;
  for (int d = 0; d < ndims; d++) {
    nx += dim[d];
    n *= dim[d];
  }
  fwrite(&ndims, sizeof(int), 1, out);
  fwrite(&nvars, sizeof(int), 1, out);
  fwrite(dim, sizeof(int), ndims, out);
  fwrite(x, sizeof(double), nx, out);
  fwrite(u, sizeof(double), n * nvars, out);
  fclose(out);
  return GB_OK;
}

/* WriteText (src/IOFunctions/WriteText.c) and WriteTecplot2D / WriteTecplot3D
 * (WriteTecplot2D.c, WriteTecplot3D.c): per point, dimension 0 fastest, the grid
 * indices, the coordinates and the variables; the Tecplot forms first write a
 * VARIABLES / ZONE header. */
static int write_points(FILE *out, int ndims, int nvars, const int *dim, const double *x, const double *u) {
  long n = 1;
  for (int d = 0; d < ndims; d++) n *= dim[d];
  int idx[3] = {0, 0, 0};
  for (long p = 0; p < n; p++) {
    long r = p;
    for (int d = 0; d < ndims; d++) {
      idx[d] = (int)(r % dim[d]);
      r /= dim[d];
    }
    for (int d = 0; d < ndims; d++) fprintf(out, "%4d ", idx[d]);
    int off = 0;
    for (int d = 0; d < ndims; d++) {
      fprintf(out, "%+1.16E ", x[off + idx[d]]);
      off += dim[d];
    }
    for (int v = 0; v < nvars; v++) fprintf(out, "%+1.16E ", u[(long)nvars * p + v]);
    fprintf(out, "\n");
  }
  return GB_OK;
}

int gb_write_text(const char *path, int ndims, int nvars, const int *dim, const double *x, const double *u) {
  FILE *out = fopen(path, "w");
  if (!out) {
    gbh_set_error("could not open %s for writing", path);
    return GB_ERR_INPUT;
  }
  write_points(out, ndims, nvars, dim, x, u);
  fclose(out);
  return GB_OK;
}

int gb_write_tecplot(const char *path, int ndims, int nvars, const int *dim, const double *x, const double *u) {
  if (ndims != 2 && ndims != 3) {
    gbh_set_error("gb_write_tecplot: 2-D or 3-D grids only (ndims = %d)", ndims);
    return GB_ERR_ARG;
  }
  FILE *out = fopen(path, "w");
  if (!out) {
    gbh_set_error("could not open %s for writing", path);
    return GB_ERR_INPUT;
  }
  fprintf(out, ndims == 2 ? "VARIABLES=\"I\",\"J\",\"X\",\"Y\"," : "VARIABLES=\"I\",\"J\",\"K\",\"X\",\"Y\",\"Z\",");
  for (int v = 0; v < nvars; v++) fprintf(out, "\"%d%d\",", (v / 10) % 10, v % 10);  /* "00", "01", ... */
  fprintf(out, "\n");
  if (ndims == 2) fprintf(out, "ZONE I=%d,J=%d,F=POINT\n", dim[0], dim[1]);
  else fprintf(out, "ZONE I=%d,J=%d,K=%d,F=POINT\n", dim[0], dim[1], dim[2]);
  write_points(out, ndims, nvars, dim, x, u);
  fclose(out);
  return GB_OK;
}

/* A binary solution file (WriteBinary.c layout): ndims, nvars, dims, x, u. */
static int read_binary_solution(const char *path, int *ndims, int *nvars, int *dim, double **u, long *n) {
  FILE *in = fopen(path, "rb");
  if (!in) {
    gbh_set_error("could not open %s", path);
    return GB_ERR_INPUT;
  }
  int ok = fread(ndims, sizeof(int), 1, in) == 1 && fread(nvars, sizeof(int), 1, in) == 1 && *ndims >= 1 &&
           *ndims <= 3 && *nvars >= 1 && fread(dim, sizeof(int), *ndims, in) == (size_t)*ndims;
  long nx = 0, np = 1;
  for (int d = 0; ok && d < *ndims; d++) {
    if (dim[d] < 1) ok = 0;
    nx += dim[d];
    np *= dim[d];
  }
  double *buf = ok ? (double *)malloc(sizeof(double) * (nx + np * (*nvars))) : NULL;
  ok = ok && buf && fread(buf, sizeof(double), nx + np * (*nvars), in) == (size_t)(nx + np * (*nvars));
  fclose(in);
  if (!ok) {
    free(buf);
    gbh_set_error("%s is not a HyPar binary solution file", path);
    return GB_ERR_INPUT;
  }
  memmove(buf, buf + nx, sizeof(double) * np * (*nvars));
  *u = buf;
  *n = np;
  return GB_OK;
}

int gb_diff_binary(const char *sol_path, const char *ref_path, double *abs_norms, double *rel_norms) {
  /* Extras/hyparDiff.c:272-371: d = ref - sol; L1 = sum|d| / npoints, L2 = sqrt(sum d^2 /
   * npoints), Linf = max|d| over every variable; relative to the reference's own norms
   * when all three exceed 1e-14, else the absolute ones. */
  if (!sol_path || !ref_path || !abs_norms || !rel_norms) {
    gbh_set_error("gb_diff_binary: null argument");
    return GB_ERR_ARG;
  }
  int nd1, nv1, nd2, nv2, d1[3], d2[3];
  double *a = NULL, *b = NULL;
  long n1, n2;
  int rc = read_binary_solution(sol_path, &nd1, &nv1, d1, &a, &n1);
  if (!rc) rc = read_binary_solution(ref_path, &nd2, &nv2, d2, &b, &n2);
  if (!rc && (nd1 != nd2 || nv1 != nv2)) {
    gbh_set_error("%s and %s differ in ndims or nvars", sol_path, ref_path);
    rc = GB_ERR_INPUT;
  }
  for (int d = 0; !rc && d < nd1; d++)
    if (d1[d] != d2[d]) {
      gbh_set_error("%s and %s differ in size", sol_path, ref_path);
      rc = GB_ERR_INPUT;
    }
  if (!rc) {
    const long size = n2 * nv2;
    double s1 = 0.0, s2 = 0.0, mx = 0.0, e1 = 0.0, e2 = 0.0, emx = 0.0;
    for (long i = 0; i < size; i++) {
      const double r = b[i], dd = r - a[i];
      s1 += fabs(r);
      s2 += r * r;
      if (fabs(r) > mx) mx = fabs(r);
      e1 += fabs(dd);
      e2 += dd * dd;
      if (fabs(dd) > emx) emx = fabs(dd);
    }
    const double np = (double)n2, tol = 1e-14;
    const double nrm[3] = {s1 / np, sqrt(s2 / np), mx};
    abs_norms[0] = e1 / np;
    abs_norms[1] = sqrt(e2 / np);
    abs_norms[2] = emx;
    for (int k = 0; k < 3; k++)
      rel_norms[k] = (nrm[0] > tol && nrm[1] > tol && nrm[2] > tol) ? abs_norms[k] / nrm[k] : abs_norms[k];
  }
  free(a);
  free(b);
  return rc;
}

int gb_op_to_initial(const char *op_path, const char *initial_path) {
  /* Extras/BinaryOPToInitialSolution.c: the header (ndims, nvars, dims) is
   * dropped, x and u are written as a binary initial.inp. */
  if (!op_path || !initial_path) {
    gbh_set_error("gb_op_to_initial: null path");
    return GB_ERR_ARG;
  }
  FILE *in = fopen(op_path, "rb");
  if (!in) {
    gbh_set_error("could not open %s", op_path);
    return GB_ERR_INPUT;
  }
  int ndims = 0, nvars = 0, dims[3] = {0, 0, 0};
  int bad = fread(&ndims, sizeof(int), 1, in) != 1 || fread(&nvars, sizeof(int), 1, in) != 1 || ndims < 1 ||
            ndims > 3 || nvars < 1 || fread(dims, sizeof(int), ndims, in) != (size_t)ndims;
  long nx = 0, nu = nvars;
  for (int d = 0; d < ndims && !bad; d++) {
    if (dims[d] < 1) bad = 1;
    nx += dims[d];
    nu *= dims[d];
  }
  double *buf = bad ? NULL : (double *)malloc(sizeof(double) * (nx + nu));
  if (!bad) bad = !buf || fread(buf, sizeof(double), nx + nu, in) != (size_t)(nx + nu);
  fclose(in);
  if (bad) {
    free(buf);
    gbh_set_error("%s is not a HyPar binary solution file", op_path);
    return GB_ERR_INPUT;
  }
  FILE *out = fopen(initial_path, "wb");
  if (!out) {
    free(buf);
    gbh_set_error("could not open %s for writing", initial_path);
    return GB_ERR_INPUT;
  }
  size_t w = fwrite(buf, sizeof(double), nx + nu, out);
  fclose(out);
  free(buf);
  if (w != (size_t)(nx + nu)) {
    gbh_set_error("short write to %s", initial_path);
    return GB_ERR_INPUT;
  }
  return GB_OK;
}
