// shim_config_main.cpp -- test driver of the HyPar-side binding
// (hypar_gb300/shim/gbhypar_attach.c), linked against the reference's own objects
// (oracle/_ref/libhypar_ref.a) and libgbhypar.so by tests/test_shim.py.
//
// In the current directory (an input deck) it runs the reference's start-up
// sequence (src/main.cpp:334-420) up to InitializePhysicsData, then prints the
// gb_config that gbshim_config() reads from the reference's initialised structs,
// one "name value..." line per field, and the status gbshim_attach() returns
// (GB_ERR_CUDA where no GPU is present).
#include <cstdio>

#include <single_simulation.h>

#include "gbhypar_attach.h"

class Harness : public SingleSimulation {
 public:
  SimulationObject* obj() { return m_sim; }
};

int main() {
  Harness h;
  if (h.define(0, 1) || h.ReadInputs() || h.Initialize() || h.InitialSolution() || h.InitializeBoundaries() ||
      h.InitializeImmersedBoundaries() || h.InitializeSolvers() || h.InitializePhysics() ||
      h.InitializePhysicsData())
    return 1;
  HyPar* solver = &h.obj()->solver;
  gb_config c;
  int rc = gbshim_config(solver, &c);
  printf("config_rc %d\n", rc);
  if (rc) return 0;
  printf("model %d\nndims %d\nnvars %d\nghosts %d\n", c.model, c.ndims, c.nvars, c.ghosts);
  printf("dim %d %d %d\n", c.dim[0], c.dim[1], c.dim[2]);
  printf("interp %d\nupwind %d\nhyp_scheme %d\nweno_weights %d\n", c.interp, c.upwind, c.hyp_scheme,
         c.weno_weights);
  printf("gamma %.17g\nweno_eps %.17g\nRe %.17g\nPr %.17g\nMinf %.17g\n", c.gamma, c.weno_eps, c.Re, c.Pr, c.Minf);
  printf("gravity %.17g %.17g %.17g\n", c.gravity[0], c.gravity[1], c.gravity[2]);
  printf("rho_ref %.17g\np_ref %.17g\nR_gas %.17g\nN_bv %.17g\nHB %d\ngrav_type %d\n", c.rho_ref, c.p_ref,
         c.R_gas, c.N_bv, c.HB, c.grav_type);
  printf("nzones %d\n", c.nzones);
  for (int z = 0; z < c.nzones; z++) {
    printf("zone%d", z);
    for (int k = 0; k < 9; k++) printf(" %d", c.zones[z][k]);
    printf("\nzone_data%d", z);
    for (int k = 0; k < 8; k++) printf(" %.17g", c.zone_data[z][k]);
    printf("\n");
  }
  printf("rk_nstages %d\nrk_A", c.rk_nstages);
  for (int k = 0; k < 16; k++) printf(" %.17g", c.rk_A[k]);
  printf("\nrk_b");
  for (int k = 0; k < 4; k++) printf(" %.17g", c.rk_b[k]);
  printf("\nrk_c");
  for (int k = 0; k < 4; k++) printf(" %.17g", c.rk_c[k]);
  printf("\ndt %.17g\nn_iter %d\nfile_op_iter %d\nrestart_iter %d\nscreen_op_iter %d\ncons_check %d\npar_scheme %d\n",
         c.dt, c.n_iter, c.file_op_iter, c.restart_iter, c.screen_op_iter, c.cons_check, c.par_scheme);
  printf("attach_rc %d\n", gbshim_attach(solver, &h.obj()->mpi));
  return 0;
}
