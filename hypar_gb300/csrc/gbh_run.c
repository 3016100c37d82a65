/*
 * gbh_run.c -- gb_run_case(): HyPar's main() for this path, on one GPU.
 *
 * Follows the reference driver's order (src/main.cpp:334-473): read the
 * inputs, set up the solver, run n_iter Runge-Kutta steps, and write the
 * solution in solver.inp's op_file_format (binary .bin, text / Tecplot .dat):
 * op.<ext> when op_overwrite is "yes", else op_00000.<ext>, op_00001.<ext>, ...
 * every file_op_iter steps (src/Simulation/OutputSolution.cpp:25-140).
 */
#define _POSIX_C_SOURCE 200809L /* clock_gettime */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#include "gbhypar.h"

void gbh_set_error(const char *fmt, ...);
const char *gbh_inputs_op_overwrite(const gb_inputs *in);
const char *gbh_inputs_op_format(const gb_inputs *in);

/* The solution file of op_file_format (InitializeSolvers.c:419-436, WriteArray.c:
   root, "_" and the five-digit index unless op_overwrite is "yes", then ".bin" for
   binary, ".dat" for text and Tecplot; nothing for "none").  A Tecplot form that
   does not fit the grid's dimension writes nothing and says so, as the reference's
   writers do. */
static int write_file(const char *dir, const char *root, int index, const char *fmt, const gb_config *c,
                      const double *x, const double *u) {
  if (!strcmp(fmt, "none")) return GB_OK;
  const int bin = !strcmp(fmt, "binary") || !strcmp(fmt, "bin");
  char name[256], path[4400];
  if (index >= 0) snprintf(name, sizeof(name), "%s_%05d%s", root, index, bin ? ".bin" : ".dat");
  else snprintf(name, sizeof(name), "%s%s", root, bin ? ".bin" : ".dat");
  if (dir && dir[0]) snprintf(path, sizeof(path), "%s/%s", dir, name);
  else snprintf(path, sizeof(path), "%s", name);
  if (bin) return gb_write_binary(path, c->ndims, c->nvars, c->dim, x, u);
  if (!strcmp(fmt, "text")) return gb_write_text(path, c->ndims, c->nvars, c->dim, x, u);
  if ((!strcmp(fmt, "tecplot2d") && c->ndims != 2) || (!strcmp(fmt, "tecplot3d") && c->ndims != 3)) {
    fprintf(stderr, "Error: %s is for %s problems only (ndims = %d); %s not written.\n", fmt,
            fmt[7] == '2' ? "2-dimensional" : "3-dimensional", c->ndims, name);
    return GB_OK;
  }
  return gb_write_tecplot(path, c->ndims, c->nvars, c->dim, x, u);
}

static int write_op(const char *dir, int index, const char *fmt, const gb_config *c, const double *x,
                    gb_solver *s, double *buf) {
  if (!strcmp(fmt, "none")) return GB_OK;
  int rc = gb_solver_get_state(s, buf, GB_LAYOUT_INTERIOR, GB_MEM_HOST);
  if (rc) return rc;
  return write_file(dir, "op", index, fmt, c, x, buf);
}

static int write_errors(const char *dir, const gb_config *c, const double *err, double runtime) {
  /* SimulationWriteErrors.c:74-81: sizes, iproc, dt, L1 L2 Linf, solver and total runtimes */
  char path[4200];
  if (dir && dir[0]) snprintf(path, sizeof(path), "%s/errors.dat", dir);
  else snprintf(path, sizeof(path), "errors.dat");
  FILE *out = fopen(path, "w");
  if (!out) {
    gbh_set_error("could not open %s for writing", path);
    return GB_ERR_INPUT;
  }
  for (int d = 0; d < c->ndims; d++) fprintf(out, "%4d ", c->dim[d]);
  for (int d = 0; d < c->ndims; d++) fprintf(out, "%4d ", 1);
  fprintf(out, "%1.16E  ", c->dt);
  fprintf(out, "%1.16E %1.16E %1.16E   ", err[0], err[1], err[2]);
  fprintf(out, "%1.16E %1.16E\n", runtime, runtime);
  fclose(out);
  return GB_OK;
}

/* SimulationWriteErrors.c:82-99: conservation<_k>.dat (sizes, iproc, dt, the
   conservation error per variable, -1 without conservation_check) and
   function_counts<_k>.dat (n_iter and the calls of the hyperbolic, parabolic and
   source functions). */
static int write_counts(const char *dir, const char *suffix, const gb_config *c, const double *cons, int nsteps) {
  char path[4400];
  const char *names[2] = {"conservation", "function_counts"};
  for (int f = 0; f < 2; f++) {
    if (dir && dir[0]) snprintf(path, sizeof(path), "%s/%s%s.dat", dir, names[f], suffix);
    else snprintf(path, sizeof(path), "%s%s.dat", names[f], suffix);
    FILE *out = fopen(path, "w");
    if (!out) {
      gbh_set_error("could not open %s for writing", path);
      return GB_ERR_INPUT;
    }
    if (f == 0) {
      for (int d = 0; d < c->ndims; d++) fprintf(out, "%4d ", c->dim[d]);
      for (int d = 0; d < c->ndims; d++) fprintf(out, "%4d ", 1);
      fprintf(out, "%1.16E  ", c->dt);
      for (int v = 0; v < c->nvars; v++) fprintf(out, "%1.16E ", cons ? cons[v] : -1.0);
      fprintf(out, "\n");
    } else {
      /* one hyperbolic term per stage; the parabolic one counts when it is not zero
         (NavierStokes3DParabolicFunction.c:72, Re > 0), the source one when the model
         has a source function (Euler1D, NavierStokes3D: SourceFunction.c:47) */
      const int calls = nsteps * c->rk_nstages;
      const int par = (c->model == GB_MODEL_NS3D && c->Re > 0.0) ? calls : 0;
      const int sou = (c->model == GB_MODEL_EULER1D || c->model == GB_MODEL_NS3D) ? calls : 0;
      fprintf(out, "%d\n%d\n%d\n%d\n", c->n_iter, calls, par, sou);
    }
    fclose(out);
  }
  return GB_OK;
}

static int run_ensemble(const char *dir, int device, int verbose, int nsims) {
  gb_inputs **in = (gb_inputs **)calloc(nsims, sizeof(gb_inputs *));
  gb_config *cf = (gb_config *)calloc(nsims, sizeof(gb_config));
  const double **dx = (const double **)calloc(nsims, sizeof(double *));
  int rc = GB_OK;
  for (int m = 0; m < nsims && !rc; m++) {
    rc = gb_inputs_read_member(dir, m, nsims, &in[m]);
    if (!rc) {
      cf[m] = *gb_inputs_config(in[m]);
      dx[m] = gb_inputs_dxinv(in[m]);
    }
  }
  gb_ensemble *e = NULL;
  if (!rc) rc = gb_ensemble_create(cf, dx, nsims, device, &e);
  long nmax = 0;
  for (int m = 0; m < nsims && !rc; m++) {
    long n = cf[m].nvars;
    for (int d = 0; d < cf[m].ndims; d++) n *= cf[m].dim[d];
    if (n > nmax) nmax = n;
    rc = gb_ensemble_set_state(e, m, gb_inputs_u0(in[m]), GB_LAYOUT_INTERIOR, GB_MEM_HOST);
  }
  if (!rc && cf[0].cons_check) rc = gb_ensemble_conservation_begin(e);
  double *buf = (double *)malloc(sizeof(double) * (nmax > 0 ? nmax : 1));
  int overwrite = !rc && !strcmp(gbh_inputs_op_overwrite(in[0]), "yes");
  int every = cf[0].file_op_iter > 0 ? cf[0].file_op_iter : cf[0].n_iter;
  int width = 1;
  for (int n = nsims; n >= 10; n /= 10) width++;
  int k = 0;
  const char *fmt = rc ? "none" : gbh_inputs_op_format(in[0]);
  if (width > 9) width = 9;
  struct timespec t0, t1;
  clock_gettime(CLOCK_MONOTONIC, &t0);
  for (int it = 0; !rc && it <= cf[0].n_iter;) {
    int write = (!overwrite && (it % every == 0 || it == cf[0].n_iter)) || (overwrite && it == cf[0].n_iter);
    for (int m = 0; write && strcmp(fmt, "none") && m < nsims && !rc; m++) {
      char root[64];
      snprintf(root, sizeof(root), "op_%0*d", width, m);  /* OutputSolution.cpp:53-58 */
      rc = gb_ensemble_get_state(e, m, buf, GB_LAYOUT_INTERIOR, GB_MEM_HOST);
      if (!rc) rc = write_file(dir, root, overwrite ? -1 : k, fmt, &cf[m], gb_inputs_x(in[m]), buf);
    }
    if (write && !overwrite) k++;
    if (it == cf[0].n_iter) break;
    int chunk = every;
    if (it + chunk > cf[0].n_iter) chunk = cf[0].n_iter - it;
    if (!rc) rc = gb_ensemble_step(e, chunk);
    it += chunk;
    if (!rc && verbose) printf("gbhypar: ensemble of %d, iteration %d / %d\n", nsims, it, cf[0].n_iter);
  }
  if (!rc) rc = gb_ensemble_sync(e);
  clock_gettime(CLOCK_MONOTONIC, &t1);
  const double runtime = (t1.tv_sec - t0.tv_sec) + 1e-9 * (t1.tv_nsec - t0.tv_nsec);
  /* per member: errors_<k>.dat (-1 without exact_<k>.inp), conservation_<k>.dat,
     function_counts_<k>.dat */
  for (int m = 0; m < nsims && !rc; m++) {
    char suffix[32];
    snprintf(suffix, sizeof(suffix), "_%0*d", width, m);
    double cons[5], err[3] = {-1.0, -1.0, -1.0};
    if (cf[m].cons_check) rc = gb_ensemble_conservation_error(e, m, cons);
    if (!rc) rc = write_counts(dir, suffix, &cf[m], cf[m].cons_check ? cons : NULL, cf[m].n_iter);
    /* CalculateError.c:42-47: exact_<k>.inp of each member */
    if (!rc && gb_inputs_exact(in[m]))
      rc = gb_ensemble_error(e, m, gb_inputs_exact(in[m]), GB_LAYOUT_INTERIOR, GB_MEM_HOST, err);
    if (!rc && verbose && err[0] >= 0) {
      printf("Computed errors for domain %d:\n", m);
      printf("  L1         Error           : %1.16E\n", err[0]);
      printf("  L2         Error           : %1.16E\n", err[1]);
      printf("  Linfinity  Error           : %1.16E\n", err[2]);
    }
    if (!rc) {
      char path[4400];  /* errors_<k>.dat */
      if (dir && dir[0]) snprintf(path, sizeof(path), "%s/errors%s.dat", dir, suffix);
      else snprintf(path, sizeof(path), "errors%s.dat", suffix);
      FILE *out = fopen(path, "w");
      if (!out) {
        gbh_set_error("could not open %s for writing", path);
        rc = GB_ERR_INPUT;
        break;
      }
      for (int d = 0; d < cf[m].ndims; d++) fprintf(out, "%4d ", cf[m].dim[d]);
      for (int d = 0; d < cf[m].ndims; d++) fprintf(out, "%4d ", 1);
      fprintf(out, "%1.16E  ", cf[m].dt);
      fprintf(out, "%1.16E %1.16E %1.16E   ", err[0], err[1], err[2]);
      fprintf(out, "%1.16E %1.16E\n", runtime, runtime);
      fclose(out);
    }
  }
  free(buf);
  gb_ensemble_destroy(e);
  for (int m = 0; m < nsims; m++) gb_inputs_free(in[m]);
  free(in);
  free(cf);
  free(dx);
  return rc;
}

int gb_run_case(const char *dir, int device, int verbose) {
  int nsims = gb_inputs_nsims(dir);
  if (nsims < 1) {
    gbh_set_error("simulation.inp is malformed");
    return GB_ERR_INPUT;
  }
  if (nsims > 1) return run_ensemble(dir, device, verbose, nsims);
  gb_inputs *in = NULL;
  int rc = gb_inputs_read(dir, &in);
  if (rc) return rc;
  const gb_config *c = gb_inputs_config(in);
  gb_solver *s = NULL;
  rc = gb_solver_create(c, gb_inputs_dxinv(in), device, &s);
  if (rc) {
    gb_inputs_free(in);
    return rc;
  }
  long n = c->nvars;
  for (int d = 0; d < c->ndims; d++) n *= c->dim[d];
  double *buf = (double *)malloc(sizeof(double) * n);
  rc = gb_solver_set_state(s, gb_inputs_u0(in), GB_LAYOUT_INTERIOR, GB_MEM_HOST);
  if (!rc && gb_inputs_gravity_field(in)) rc = gb_solver_set_gravity_field(s, gb_inputs_gravity_field(in));
  /* thermal walls: the wall temperature read with the deck */
  for (int z = 0; !rc && z < gb_inputs_config(in)->nzones; z++) {
    int nt = 0;
    const double *tt = NULL, *tf = NULL;
    rc = gb_inputs_zone_temperature(in, z, &nt, &tt, &tf);
    if (!rc && nt) rc = gb_solver_set_zone_temperature(s, z, nt, tt, tf);
    /* sponge zones: sigma computed with the deck */
    int ns = 0;
    const double *sg = NULL;
    if (!rc) rc = gb_inputs_zone_sponge(in, z, &ns, &sg);
    if (!rc && ns) rc = gb_solver_set_zone_sponge(s, z, sg);
    /* turbulent inflow zones: the inflow data read with the deck */
    int nf = 0;
    const double *fd = NULL;
    if (!rc) rc = gb_inputs_zone_inflow(in, z, &nf, &fd);
    if (!rc && nf) rc = gb_solver_set_zone_inflow(s, z, nf, fd);
  }
  /* InitialSolution.c:118: the volume integral of the initial solution */
  if (!rc && c->cons_check) rc = gb_solver_conservation_begin(s);
  const int overwrite = !strcmp(gbh_inputs_op_overwrite(in), "yes");
  const char *fmt = gbh_inputs_op_format(in);
  const int every = c->file_op_iter > 0 ? c->file_op_iter : c->n_iter;
  const int screen = c->screen_op_iter > 0 ? c->screen_op_iter : 1;
  const int R = c->restart_iter > 0 ? c->restart_iter : 0;
  /* a restart run starts at t = restart_iter * dt (TimeInitialize.c:49-52) and
     fast-forwards the file index over the outputs before it (InitializeSolvers.c:438-442) */
  int k = 0;
  for (int t = 0; t < R; t++)
    if ((t + 1) % every == 0) k++;
  if (!rc) rc = gb_solver_set_time(s, R * c->dt);
  if (!rc && !overwrite && R == 0) rc = write_op(dir, k++, fmt, c, gb_inputs_x(in), s, buf);
  FILE *resid = NULL;
  if (!rc && c->write_residual) {
    char path[4200];
    if (dir && dir[0]) snprintf(path, sizeof(path), "%s/residual.out", dir);
    else snprintf(path, sizeof(path), "residual.out");
    resid = fopen(path, "w");
  }
  struct timespec t0, t1;
  clock_gettime(CLOCK_MONOTONIC, &t0);
  /* Solve.cpp:97-152: a report every screen_op_iter iterations (TimePreStep CFL,
     TimePostStep norm, TimePrintStep line), an output every file_op_iter */
  for (int it = R; it < c->n_iter && !rc;) {
    int next_screen = (it / screen + 1) * screen;
    int next_out = (it / every + 1) * every;
    int target = c->n_iter;
    if (next_screen < target) target = next_screen;
    if (next_out < target) target = next_out;
    const int report = (target % screen == 0);
    struct timespec a, b;
    clock_gettime(CLOCK_MONOTONIC, &a);
    double cfl = -1.0, norm = -1.0;
    if (report) rc = gb_solver_step_report(s, target - it, &cfl, &norm);
    else rc = gb_solver_step(s, target - it);
    clock_gettime(CLOCK_MONOTONIC, &b);
    double wc = (b.tv_sec - a.tv_sec) + 1e-9 * (b.tv_nsec - a.tv_nsec);
    it = target;
    if (rc) break;
    if (report) {
      /* TimePrintStep.c:30-56, with the conservation error when it is checked */
      double cons[5], ce = 0.0;
      if (c->cons_check) {
        rc = gb_solver_conservation_error(s, cons);
        if (rc) break;
        for (int v = 0; v < c->nvars; v++) ce += cons[v] * cons[v];
        ce = sqrt(ce);
      }
      if (verbose) {
        printf("iter=%7d  t=%1.3E  CFL=%1.3E  norm=%1.4E  wctime: %1.1E (s)  ", it, gb_solver_time(s), cfl, norm, wc);
        if (c->cons_check) printf("  cons_err=%1.4E\n", ce);
        else printf("\n");
      }
      if (resid) fprintf(resid, "%10d\t%E\t%E\n", it, gb_solver_time(s), norm);
    }
    if (!overwrite && it % every == 0 && it < c->n_iter) rc = write_op(dir, k++, fmt, c, gb_inputs_x(in), s, buf);
  }
  clock_gettime(CLOCK_MONOTONIC, &t1);
  const double solver_runtime = (t1.tv_sec - t0.tv_sec) + 1e-9 * (t1.tv_nsec - t0.tv_nsec);
  if (resid) fclose(resid);
  if (!rc) rc = write_op(dir, overwrite ? -1 : k++, fmt, c, gb_inputs_x(in), s, buf);
  if (!rc) {
    int fin = 1;
    rc = gb_solver_check_finite(s, &fin);
    if (!rc && !fin) {
      gbh_set_error("the solution contains NaN or Inf");
      rc = GB_ERR_NONFINITE;
    }
  }
  /* CalculateError + SimulationWriteErrors: errors.dat (-1 without exact.inp) */
  if (!rc) {
    double err[3] = {-1.0, -1.0, -1.0};
    if (gb_inputs_exact(in)) rc = gb_solver_error(s, gb_inputs_exact(in), GB_LAYOUT_INTERIOR, GB_MEM_HOST, err);
    if (!rc) rc = write_errors(dir, c, err, solver_runtime);
    if (!rc && verbose && err[0] >= 0) {
      printf("Computed errors for domain 0:\n");
      printf("  L1         Error           : %1.16E\n", err[0]);
      printf("  L2         Error           : %1.16E\n", err[1]);
      printf("  Linfinity  Error           : %1.16E\n", err[2]);
    }
    double cons[5];
    if (!rc && c->cons_check) rc = gb_solver_conservation_error(s, cons);
    if (!rc) rc = write_counts(dir, "", c, c->cons_check ? cons : NULL, c->n_iter - R);
    if (!rc && verbose && c->cons_check) {
      printf("Conservation Errors:\n");
      for (int v = 0; v < c->nvars; v++) printf("\t%1.16E\n", cons[v]);
    }
  }
  free(buf);
  gb_solver_destroy(s);
  gb_inputs_free(in);
  return rc;
}
