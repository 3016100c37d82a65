/*
 * gbhypar_main.c -- command-line driver: `gbhypar [case_dir] [device]` runs a HyPar
 * input deck (solver.inp, physics.inp, boundary.inp, weno.inp, initial.inp) on the
 * GPU, like the reference's HyPar executable does on the CPU;
 * `gbhypar diff [-a abs_tol] [-r rel_tol] sol.bin ref.bin` compares two binary
 * solution files like the reference's Extras/hyparDiff (default tolerances 1e-14;
 * prints the norms of the difference when a tolerance is exceeded).
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "gbhypar.h"

static int diff_main(int argc, char **argv) {
  double abs_tol = 1e-14, rel_tol = 1e-14;
  const char *files[2] = {NULL, NULL};
  int nf = 0;
  for (int i = 2; i < argc; i++) {
    if ((!strcmp(argv[i], "-a") || !strcmp(argv[i], "-r")) && i + 1 < argc) {
      double v = strtod(argv[i + 1], NULL);
      if (argv[i][1] == 'a') abs_tol = v;
      else rel_tol = v;
      i++;
    } else if (nf < 2) {
      files[nf++] = argv[i];
    }
  }
  if (nf != 2) {
    fprintf(stderr, "usage: gbhypar diff [-a abs_tol] [-r rel_tol] sol.bin ref.bin\n");
    return 2;
  }
  double a[3], r[3];
  int rc = gb_diff_binary(files[0], files[1], a, r);
  if (rc) {
    printf("%s\n", gb_last_error());
    return 0;  /* the reference's tool reports a size mismatch and exits 0 */
  }
  int ok = 1;
  for (int k = 0; k < 3; k++)
    if (a[k] > abs_tol || r[k] > rel_tol) ok = 0;
  if (!ok) {
    printf("%s and %s differ.\n", files[0], files[1]);
    printf("Norms of the difference between the two solutions:\n");
    printf("  L1  : %1.6e (abs), %1.6e (rel)\n", a[0], r[0]);
    printf("  L2  : %1.6e (abs), %1.6e (rel)\n", a[1], r[1]);
    printf("  Linf: %1.6e (abs), %1.6e (rel)\n", a[2], r[2]);
  }
  return 0;
}

int main(int argc, char **argv) {
  if (argc > 1 && !strcmp(argv[1], "diff")) return diff_main(argc, argv);
  const char *dir = argc > 1 ? argv[1] : ".";
  int dev = argc > 2 ? atoi(argv[2]) : 0;
  int rc = gb_run_case(dir, dev, 1);
  if (rc) {
    fprintf(stderr, "gbhypar: error %d: %s\n", rc, gb_last_error());
    return 1;
  }
  printf("gbhypar: done\n");
  return 0;
}
