/*
 * gbh_run.c -- gb_run_case(): HyPar's main() for this path, on one GPU.
 *
 * Follows the reference driver's order (src/main.cpp:334-473): read the
 * inputs, set up the solver, run n_iter Runge-Kutta steps, and write the
 * solution in HyPar's binary format: op.bin when op_overwrite is "yes", else
 * op_00000.bin, op_00001.bin, ... every file_op_iter steps
 * (src/Simulation/OutputSolution.cpp:50-140).
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "gbhypar.h"

void gbh_set_error(const char *fmt, ...);
const char *gbh_inputs_op_overwrite(const gb_inputs *in);

static int write_op(const char *dir, const char *name, const gb_config *c, const double *x, gb_solver *s,
                    double *buf) {
  int rc = gb_solver_get_state(s, buf, GB_LAYOUT_INTERIOR, GB_MEM_HOST);
  if (rc) return rc;
  char path[4096];
  if (dir && dir[0]) snprintf(path, sizeof(path), "%s/%s", dir, name);
  else snprintf(path, sizeof(path), "%s", name);
  return gb_write_binary(path, c->ndims, c->nvars, c->dim, x, buf);
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
  double *buf = (double *)malloc(sizeof(double) * (nmax > 0 ? nmax : 1));
  int overwrite = !rc && !strcmp(gbh_inputs_op_overwrite(in[0]), "yes");
  int every = cf[0].file_op_iter > 0 ? cf[0].file_op_iter : cf[0].n_iter;
  int width = 1;
  for (int n = nsims; n >= 10; n /= 10) width++;
  int k = 0;
  char name[160], path[4400];
  if (width > 9) width = 9;
  for (int it = 0; !rc && it <= cf[0].n_iter;) {
    int write = (!overwrite && (it % every == 0 || it == cf[0].n_iter)) || (overwrite && it == cf[0].n_iter);
    for (int m = 0; write && m < nsims && !rc; m++) {
      rc = gb_ensemble_get_state(e, m, buf, GB_LAYOUT_INTERIOR, GB_MEM_HOST);
      if (overwrite) snprintf(name, sizeof(name), "op_%0*d.bin", width, m);
      else snprintf(name, sizeof(name), "op_%0*d_%05d.bin", width, m, k);
      if (dir && dir[0]) snprintf(path, sizeof(path), "%s/%s", dir, name);
      else snprintf(path, sizeof(path), "%s", name);
      if (!rc) rc = gb_write_binary(path, cf[m].ndims, cf[m].nvars, cf[m].dim, gb_inputs_x(in[m]), buf);
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
  int overwrite = !strcmp(gbh_inputs_op_overwrite(in), "yes");
  int every = c->file_op_iter > 0 ? c->file_op_iter : c->n_iter;
  int k = 0;
  char name[64];
  if (!rc && !overwrite) {
    snprintf(name, sizeof(name), "op_%05d.bin", k++);
    rc = write_op(dir, name, c, gb_inputs_x(in), s, buf);
  }
  for (int it = 0; it < c->n_iter && !rc;) {
    int chunk = every;
    if (it + chunk > c->n_iter) chunk = c->n_iter - it;
    rc = gb_solver_step(s, chunk);
    it += chunk;
    if (!rc && verbose) printf("gbhypar: iteration %d / %d, t = %.6e\n", it, c->n_iter, gb_solver_time(s));
    if (!rc && !overwrite && (it % every == 0 || it == c->n_iter)) {
      snprintf(name, sizeof(name), "op_%05d.bin", k++);
      rc = write_op(dir, name, c, gb_inputs_x(in), s, buf);
    }
  }
  if (!rc && overwrite) rc = write_op(dir, "op.bin", c, gb_inputs_x(in), s, buf);
  if (!rc) {
    int fin = 1;
    rc = gb_solver_check_finite(s, &fin);
    if (!rc && !fin) {
      gbh_set_error("the solution contains NaN or Inf");
      rc = GB_ERR_NONFINITE;
    }
  }
  free(buf);
  gb_solver_destroy(s);
  gb_inputs_free(in);
  return rc;
}
