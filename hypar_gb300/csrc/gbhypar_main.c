/*
 * gbhypar_main.c -- command-line driver: `gbhypar [case_dir]` runs a HyPar
 * input deck (solver.inp, physics.inp, boundary.inp, weno.inp, initial.inp)
 * on the GPU, like the reference's HyPar executable does on the CPU.
 */
#include <stdio.h>
#include <stdlib.h>

#include "gbhypar.h"

int main(int argc, char **argv) {
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
