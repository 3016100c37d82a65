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

int gb_run_case(const char *dir, int device, int verbose) {
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
