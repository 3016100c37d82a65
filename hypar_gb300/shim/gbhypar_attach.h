/*
 * gbhypar_attach.h -- the HyPar-side binding of libgbhypar.
 *
 * gbhypar_attach.c is compiled inside (or against) HyPar's source tree: it reads
 * HyPar's own solver, physics-model, WENO, boundary and Runge-Kutta structs and
 * installs libgbhypar's entry points in HyPar's function pointers.  Nothing in
 * HyPar's structs changes: each HyPar solver is mapped to its gb_solver through a
 * table kept here.
 *
 * Arrays: HyPar hands these functions its gpu_* arrays when it runs with use_gpu
 * (TimeRK's GPU branch, src/TimeIntegration/TimeRK.c:39-120), which is the mode
 * this binding is for: libgbhypar's entry points take device arrays.
 */
#ifndef GBHYPAR_ATTACH_H
#define GBHYPAR_ATTACH_H

#include <gbhypar.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Fill a gb_config from an initialised HyPar solver (after InitializeSolvers and
 * InitializePhysics; `solver` is a HyPar*).  Returns GB_OK, or GB_ERR_UNSUPPORTED
 * (with a message on stderr) for a model, scheme or boundary outside libgbhypar's
 * path. */
int gbshim_config(void *solver, gb_config *c);

/* Create the gb_solver of `solver` (a HyPar*, with its MPIVariables* `mpi`) on
 * HyPar's gpu_device_no, hand it the gravity fields of the physics model, install
 * HyperbolicFunction, ParabolicFunction, SourceFunction and
 * ApplyBoundaryConditions, and pass the physics model's PostStage hook to the
 * fused step.  Returns GB_OK or a GB_ERR_* code (message on stderr). */
int gbshim_attach(void *solver, void *mpi);

/* The gb_solver attached to `solver`, or NULL. */
gb_solver *gbshim_solver(void *solver);

/* Destroy the gb_solver attached to `solver` (a no-op if none). */
void gbshim_detach(void *solver);

/* TimeIntegration.RHSFunction (include/timeintegration_struct.h:98) through
 * gb_RHSFunctionExplicit of the attached solver. */
int gbshim_RHSFunction(double *rhs, double *u, void *solver, void *mpi, double t);

/* HyPar's TimeIntegrate for the "rk" scheme (TimeRK, src/TimeIntegration/TimeRK.c:35),
 * `ts` a TimeIntegration*: every simulation's solution (gpu_u) is advanced one fused
 * step by its gb_solver at the integrator's time.  HyPar's TimePreStep / TimePostStep
 * stay around it and call PreStep / PostStep themselves. */
int gbshim_TimeRK(void *ts);

#ifdef __cplusplus
}
#endif

#endif
