// ref_rhs_harness.cpp -- drives the REFERENCE HyPar build (oracle/_ref/libhypar_ref.a,
// compiled from the reference sources by oracle/Makefile.ref) through its own
// start-up sequence (src/main.cpp:334-420) in the current directory, then
// calls its TimeRHSFunctionExplicit (src/TimeIntegration/TimeRHSFunctionExplicit.c:30)
// once on the initial solution and dumps the result.  The reference keeps no
// per-RHS output of its own, so this is how the oracle restatement is pinned
// against the reference per right-hand-side evaluation.
//
// Test infrastructure only; built only where the reference sources exist.
//
// Output file (argv[1]): int32 ndims, nvars, ghosts, dim[ndims]; then float64
// dxinv[sum(dim+2g)], u_in[npts_wg*nvars], u_bc[npts_wg*nvars] (ghosts filled
// by the RHS call), rhs[npts_wg*nvars].
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include <single_simulation.h>

extern "C" int TimeRHSFunctionExplicit(double*, double*, void*, void*, double);

class RefHarness : public SingleSimulation {
 public:
  SimulationObject* obj() { return m_sim; }
};

int main(int argc, char** argv) {
  if (argc < 2) {
    fprintf(stderr, "usage: %s <out.bin>\n", argv[0]);
    return 2;
  }
  RefHarness h;
  if (h.define(0, 1)) return 1;
  if (h.ReadInputs()) return 1;
  if (h.Initialize()) return 1;
  if (h.InitialSolution()) return 1;
  if (h.InitializeBoundaries()) return 1;
  if (h.InitializeImmersedBoundaries()) return 1;
  if (h.InitializeSolvers()) return 1;
  if (h.InitializePhysics()) return 1;
  if (h.InitializePhysicsData()) return 1;

  HyPar* solver = &h.obj()->solver;
  MPIVariables* mpi = &h.obj()->mpi;
  int ndims = solver->ndims, nvars = solver->nvars, g = solver->ghosts;
  long n = (long)solver->npoints_local_wghosts * nvars;
  long nx = 0;
  for (int d = 0; d < ndims; d++) nx += solver->dim_local[d] + 2 * g;

  std::vector<double> u_in(solver->u, solver->u + n);
  std::vector<double> u(u_in);
  std::vector<double> rhs(n, 0.0);
  TimeRHSFunctionExplicit(rhs.data(), u.data(), solver, mpi, 0.0);
  // the model's CFL of the initial solution (solver->u) for the deck's dt
  double cfl = solver->ComputeCFL ? solver->ComputeCFL(solver, mpi, solver->dt, 0.0) : -1.0;

  FILE* f = fopen(argv[1], "wb");
  if (!f) return 1;
  fwrite(&ndims, sizeof(int), 1, f);
  fwrite(&nvars, sizeof(int), 1, f);
  fwrite(&g, sizeof(int), 1, f);
  fwrite(solver->dim_local, sizeof(int), ndims, f);
  fwrite(solver->dxinv, sizeof(double), nx, f);
  fwrite(u_in.data(), sizeof(double), n, f);
  fwrite(u.data(), sizeof(double), n, f);
  fwrite(rhs.data(), sizeof(double), n, f);
  fwrite(&cfl, sizeof(double), 1, f);
  fclose(f);
  printf("ref_rhs_harness: wrote %s (%ld values)\n", argv[1], n);
  return 0;
}
