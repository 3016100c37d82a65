/*
 * gbhypar.h -- C ABI of libgbhypar, a GB300 (sm_103a) implementation of
 * HyPar's explicit finite-difference right-hand side (WENO5 + Roe/LLF/RF
 * upwinding + flux difference, NavierStokes3D viscous term) and explicit
 * Runge-Kutta step, for the Euler1D, Euler2D and NavierStokes3D models.
 *
 * Two layers:
 *
 *  1. HyPar's solver / physics-model function-pointer surface, with the
 *     reference's exact signatures (include/hypar.h:211-359 of HyPar).  Each
 *     gb_* function can be assigned to the matching HyPar pointer; `void *s`
 *     is a gb_solver handle instead of HyPar's solver struct and `void *m`
 *     (the MPI object) is ignored.  Array arguments are DEVICE pointers in
 *     HyPar's layout: ghost points on every side, dimension 0 fastest, the
 *     nvars components of a point contiguous (include/arrayfunctions.h:40-47).
 *
 *  2. A fused fast path: the solver keeps the solution resident on the GPU
 *     and gb_solver_step() advances whole Runge-Kutta steps, one fused kernel
 *     per direction per stage (the stage update folded into the last one).
 *
 * Every function returns GB_OK (0) or a GB_ERR_* code; gb_last_error() gives
 * the message.  Nothing aborts the process.
 */
#ifndef GBHYPAR_H
#define GBHYPAR_H

#ifdef __cplusplus
extern "C" {
#endif

#define GB_OK 0
#define GB_ERR_ARG 1          /* invalid argument or configuration */
#define GB_ERR_CUDA 2         /* a CUDA call failed */
#define GB_ERR_INPUT 3        /* an input file is missing or malformed */
#define GB_ERR_UNSUPPORTED 4  /* valid HyPar option outside this library's path */
#define GB_ERR_NOMEM 5        /* device or host allocation failed */
#define GB_ERR_NONFINITE 6    /* the solution contains NaN or Inf */
#define GB_ERR_HOOK 7         /* a hook installed with gb_solver_set_hooks returned nonzero */

enum { GB_MODEL_EULER1D = 1, GB_MODEL_EULER2D = 2, GB_MODEL_NS3D = 3 };
enum { GB_UPWIND_ROE = 0, GB_UPWIND_LLF = 1, GB_UPWIND_RF = 2, GB_UPWIND_RUSANOV = 3 /* Euler1D, NS3D */,
       GB_UPWIND_SWFS = 4 /* physics.inp "steger-warming": Euler1D, Euler2D */ };
enum { GB_INTERP_COMPONENTS = 0, GB_INTERP_CHARACTERISTIC = 1 };
/* boundary.inp types (include/boundaryconditions.h): periodic and extrapolate for every
 * model; dirichlet for every model; slip-wall for every model (BCSlipWall.c has a
 * 1-D branch); the other wall and inflow/outflow types, and the subsonic "ambivalent"
 * one (inflow or outflow point by point, by the sign of the extrapolated face
 * velocity), for Euler2D and NavierStokes3D (the reference has no 1-D branch for
 * them); the thermal walls (slip / no-slip, the ghost
 * pressure from the extrapolated density and a wall temperature given per time
 * level in a file) for NavierStokes3D (BCThermalSlipWall.c, BCThermalNoslipWall.c).
 * sponge (every model) fills no ghost point: over its extent of interior points it adds
 * -sigma (u - u_ref) to the source term, sigma rising linearly from 0 at the zone's inner
 * edge to 1 at its outer one along the zone's dimension (BCSponge.c:34-61); its extent is
 * an interior index range in every dimension (CalculateLocalExtent,
 * InitializeBoundaries.c:382-393) and sigma comes through gb_inputs_zone_sponge /
 * gb_solver_set_zone_sponge.  turbulent-supersonic-inflow (NavierStokes3D): the supersonic
 * inflow state with velocity fluctuations added, taken from a slice of inflow data that
 * advances with the mean flow (BCTurbulentSupersonicInflow.c); the data comes through
 * gb_inputs_zone_inflow / gb_solver_set_zone_inflow.  reflect (every model): the ghost
 * points take the negated mirror interior values, every component (BCReflect.c:22-44). */
enum { GB_BC_PERIODIC = 1, GB_BC_EXTRAPOLATE = 2, GB_BC_DIRICHLET = 3, GB_BC_SLIP_WALL = 4,
       GB_BC_NOSLIP_WALL = 5, GB_BC_SUBSONIC_INFLOW = 6, GB_BC_SUBSONIC_OUTFLOW = 7,
       GB_BC_SUPERSONIC_INFLOW = 8, GB_BC_SUPERSONIC_OUTFLOW = 9, GB_BC_SUBSONIC_AMBIVALENT = 10,
       GB_BC_THERMAL_SLIP_WALL = 11, GB_BC_THERMAL_NOSLIP_WALL = 12, GB_BC_SPONGE = 13,
       GB_BC_TURBULENT_INFLOW = 14, GB_BC_REFLECT = 15 };
enum { GB_LAYOUT_INTERIOR = 0, GB_LAYOUT_GHOSTED = 1 };
/* WENO5 nonlinear weights (weno.inp: yc > borges > mapped > Jiang-Shu, and
 * no_limiting = 1 keeps the optimal weights; WENOFifthOrderCalculateWeights.c:40-64). */
enum { GB_WENO_JS = 0, GB_WENO_MAPPED = 1, GB_WENO_BORGES = 2, GB_WENO_YC = 3, GB_WENO_NONE = 4 };
enum { GB_MEM_HOST = 0, GB_MEM_DEVICE = 1 };
/* hyp_space_scheme: weno5, or crweno5 (compact WENO5, a tridiagonal solve per grid
 * line, block tridiagonal for the characteristic form; with gravity the source
 * function is solved for with the flux's rows; Interp1PrimFifthOrderCRWENO.c,
 * Interp1PrimFifthOrderCRWENOChar.c) */
enum { GB_SCHEME_WENO5 = 0, GB_SCHEME_CRWENO5 = 1 };

#define GB_MAX_ZONES 12

/* Solver configuration: what HyPar reads from solver.inp, physics.inp,
 * weno.inp and boundary.inp (after CalculateLocalExtent). */
typedef struct gb_config {
  int model;                /* GB_MODEL_* */
  int ndims, nvars, ghosts; /* ghosts must be 3 (WENO5) */
  int dim[3];               /* interior points per dimension */
  int interp;               /* GB_INTERP_* (hyp_interp_type) */
  int upwind;               /* GB_UPWIND_* (physics.inp "upwinding") */
  double gamma;             /* physics.inp gamma */
  double weno_eps;          /* weno.inp epsilon (Jiang-Shu weights) */
  double Re, Pr, Minf;      /* NavierStokes3D physics.inp; Re <= 0: inviscid */
  int nzones;               /* boundary zones */
  int zones[GB_MAX_ZONES][9];  /* type, dim, face, is[3], ie[3] (index extents) */
  int rk_nstages;           /* explicit Runge-Kutta Butcher table */
  double rk_A[16], rk_b[4], rk_c[4];
  double dt;                /* time step */
  int n_iter;               /* number of steps (solver.inp n_iter) */
  int file_op_iter;         /* output interval (solver.inp file_op_iter) */
  int weno_weights;         /* GB_WENO_*; the batched ensemble and the adjoint take Jiang-Shu only */
  int restart_iter;         /* solver.inp restart_iter: first iteration, t0 = restart_iter * dt */
  int screen_op_iter;       /* solver.inp screen_op_iter: CFL / norm report interval */
  int write_residual;       /* solver.inp write_residual: residual.out with the norms */
  /* per zone, the values boundary.inp gives after the extents: dirichlet: nvars values;
   * slip-wall / noslip-wall: wall velocity (ndims); subsonic-inflow: rho, velocity;
   * subsonic-outflow: pressure; supersonic-inflow, subsonic-ambivalent and
   * turbulent-supersonic-inflow: rho, velocity, pressure; thermal-slip-wall / thermal-noslip-wall: wall velocity (the temperature
   * comes through gb_inputs_zone_temperature / gb_solver_set_zone_temperature); sponge:
   * the nvars values of the state it relaxes to */
  double zone_data[GB_MAX_ZONES][8];
  /* NavierStokes3D gravity (physics.inp gravity, rho_ref, p_ref, R, HB, N_bv); a nonzero
   * acceleration needs upwinding rusanov (NavierStokes3DInitialize.c:371) and the
   * hydrostatic fields of gb_solver_set_gravity_field */
  double gravity[3], rho_ref, p_ref, R_gas, N_bv;
  int HB;
  int hyp_scheme;           /* GB_SCHEME_* (solver.inp hyp_space_scheme) */
  /* Euler1D gravity: gravity[0] is physics.inp "gravity", grav_type its gravity_type (0:
   * field exp(-g x), 1: exp(sin(2 pi x)/(2 pi))); needs roe or llf-char upwinding
   * (Euler1DInitialize.c:144); the field comes through gb_solver_set_gravity_field as
   * 1/S then S */
  int grav_type;
  /* solver.inp conservation_check yes: the driver reports the conservation error
   * (gb_solver_conservation_*) */
  int cons_check;
  /* NavierStokes3D viscous term, solver.inp par_space_scheme of the
   * nonconservative-2stage form (InitializeSolvers.c:129-141): 4 (or 0): fourth-order
   * central first derivatives; 2: first-order one-sided ones, forward for the
   * gradients and backward for the flux divergence (FirstDerivativeFirstOrder.c) */
  int par_scheme;
} gb_config;

typedef struct gb_solver gb_solver;
typedef struct gb_inputs gb_inputs;

/* Message of the last failed call on this thread. */
const char *gb_last_error(void);

/* ---- input decks (the reference's readers: src/Simulation/ReadInputs.c,
 *      InitializeBoundaries.c, WENOInitialize.c, <Model>Initialize.c,
 *      src/IOFunctions/ReadArray.c, src/Simulation/InitialSolution.c) ---- */

/* Read solver.inp, physics.inp, boundary.inp, weno.inp and initial.inp from
 * `dir` (NULL: current directory). */
int gb_inputs_read(const char *dir, gb_inputs **out);
void gb_inputs_free(gb_inputs *in);
const gb_config *gb_inputs_config(const gb_inputs *in);
/* Interior grid coordinates, sum_d dim[d] values. */
const double *gb_inputs_x(const gb_inputs *in);
/* 2/(x[i+1]-x[i-1]) per point with ghosts, sum_d (dim[d]+2*ghosts) values. */
const double *gb_inputs_dxinv(const gb_inputs *in);
/* Initial solution, interior points, nvars per point, dimension 0 fastest. */
const double *gb_inputs_u0(const gb_inputs *in);
/* Exact solution from exact.inp (same format as initial.inp,
 * src/HyParFunctions/ExactSolution.c), or NULL when the deck has none. */
const double *gb_inputs_exact(const gb_inputs *in);
/* NavierStokes3D gravity: the hydrostatic density / pressure variations f and g
 * (NavierStokes3DGravityField.c) at every point with ghosts, f then g (2 x the
 * points with ghosts), or NULL without gravity. */
const double *gb_inputs_gravity_field(const gb_inputs *in);
/* Thermal walls: the wall temperature the deck's file gives for boundary zone `zone`
 * (BCReadTemperatureData, src/BoundaryConditions/BCIO.c:147): ntimes time levels
 * (times), and the field over the zone's extent with the time level along the zone's
 * own dimension, dimension 0 fastest; ntimes = 0 and NULL arrays for other zones.
 * The arrays belong to `in`. */
int gb_inputs_zone_temperature(const gb_inputs *in, int zone, int *ntimes, const double **times,
                               const double **field);
/* Sponge zones: sigma at each index of the zone's extent along its own dimension,
 * n = ie - is values, (x - x_start) / (x_end - x_start) from the grid coordinates and
 * the zone's bounds as boundary.inp gives them (BCSponge.c:49-54); n = 0 and NULL for
 * other zones.  The array belongs to `in`. */
int gb_inputs_zone_sponge(const gb_inputs *in, int zone, int *n, const double **sigma);
/* Turbulent supersonic inflow zones: the inflow data file of boundary zone `zone`
 * (BCReadTurbulentInflowData, src/BoundaryConditions/BCIO.c:19-139, one rank): n slices
 * along the zone's dimension, the grid's size along the others, nvars values per point
 * (components 1..3 are the velocity fluctuations), dimension 0 fastest; n = 0 and NULL
 * for other zones.  The array belongs to `in`. */
int gb_inputs_zone_inflow(const gb_inputs *in, int zone, int *n, const double **data);
/* Ensemble decks (simulation.inp "nsims", one "size" per simulation in
 * solver.inp, initial_<k>.inp and boundary_<k>.inp or boundary.inp; index k
 * zero-padded to (int)log10(nsims)+1 digits, src/Simulation/InitialSolution.c:36-41):
 * number of simulations in `dir` (1 without simulation.inp, -1 if malformed),
 * and the deck of simulation `member`. */
int gb_inputs_nsims(const char *dir);
int gb_inputs_read_member(const char *dir, int member, int nsims, gb_inputs **out);
/* Runge-Kutta Butcher table of TimeExplicitRKInitialize for a solver.inp
 * time_scheme_type ("1fe", "22", "33", "44", "ssprk3"). */
int gb_rk_table(const char *type, int *nstages, double *A, double *b, double *c);

/* ---- solver lifetime and the fused fast path ---- */

/* Create a solver on CUDA device `device` (-1: current).  dxinv: host array
 * of sum_d (dim[d]+2*ghosts) values. */
int gb_solver_create(const gb_config *cfg, const double *dxinv, int device, gb_solver **out);
void gb_solver_destroy(gb_solver *s);
const gb_config *gb_solver_config(const gb_solver *s);
/* Use a caller-owned cudaStream_t (NULL: the solver's own stream). */
int gb_solver_set_stream(gb_solver *s, void *stream);
/* NavierStokes3D gravity: upload the fields f, g (host, 2 x the points with
 * ghosts, as gb_inputs_gravity_field); required before stepping a configuration
 * with gravity. */
int gb_solver_set_gravity_field(gb_solver *s, const double *fg);
/* Thermal walls: upload the wall temperature of boundary zone `zone` (host arrays, as
 * gb_inputs_zone_temperature gives them: ntimes time levels, the field over the zone's
 * extent with the time level along the zone's own dimension, dimension 0 fastest).
 * Each right-hand side at time t uses the last level at or before t
 * (BCThermalNoslipWall.c:55-57); required before stepping such a configuration. */
int gb_solver_set_zone_temperature(gb_solver *s, int zone, int ntimes, const double *times, const double *field);
/* Sponge zones: upload sigma of boundary zone `zone` (host array of ie - is values along
 * the zone's own dimension, as gb_inputs_zone_sponge gives it); required before
 * evaluating a right-hand side of such a configuration.  The sponge term joins the
 * source term of every right-hand side (SourceFunction.c:50-76). */
int gb_solver_set_zone_sponge(gb_solver *s, int zone, const double *sigma);
/* Turbulent supersonic inflow zones: upload the inflow data of boundary zone `zone` (host
 * array laid out as gb_inputs_zone_inflow gives it, n slices).  At time t the ghost
 * points take slice int(u_dim t / (2 pi) * n) mod n (BCTurbulentSupersonicInflow.c:44-48);
 * a time at which that index is negative (inflow velocity against the zone's dimension)
 * is refused with GB_ERR_ARG, where the reference would read outside its data.  The
 * zone's transverse extent must lie within the grid.  Required before stepping such a
 * configuration. */
int gb_solver_set_zone_inflow(gb_solver *s, int zone, int n, const double *data);
/* Wait for all work queued by the solver. */
int gb_solver_sync(gb_solver *s);
/* Copy a solution in or out (layout GB_LAYOUT_*, memory GB_MEM_*). */
int gb_solver_set_state(gb_solver *s, const double *u, int layout, int mem);
int gb_solver_get_state(gb_solver *s, double *u, int layout, int mem);
/* Device pointer of the resident ghosted solution (valid until the next step). */
double *gb_solver_state(gb_solver *s);
/* Advance nsteps Runge-Kutta steps of size cfg->dt on the resident solution. */
int gb_solver_step(gb_solver *s, int nsteps);
/* Simulation time of the resident solution (set_state resets it to 0). */
double gb_solver_time(const gb_solver *s);
int gb_solver_set_time(gb_solver *s, double t);
/* Around-the-step quantities of the reference, reduced on the device:
 * gb_solver_cfl: maximum CFL of the resident solution with cfg->dt
 * (<Model>ComputeCFL, the reference's operation order: bit-identical);
 * gb_solver_step_report: advance nsteps steps and return the CFL of the state
 * the last step starts from (TimePreStep.c:93-100) and the norm of that step's
 * change, sqrt(sum (u_new-u_old)^2 / npoints) (TimePostStep.c:38-60) (either
 * pointer may be NULL);
 * gb_solver_error: L1, L2, Linf errors of the resident solution against an
 * exact one (layout GB_LAYOUT_*, memory GB_MEM_*), relative to the exact
 * solution's norms when those exceed 1e-15 (CalculateError.c:27-110). */
int gb_solver_cfl(gb_solver *s, double *cfl);
int gb_solver_step_report(gb_solver *s, int nsteps, double *cfl, double *norm);
int gb_solver_error(gb_solver *s, const double *uex, int layout, int mem, double *err);
/* The conservation check (solver.inp conservation_check; TimePostStep.c:78-92).
 * _begin records the volume integral sum u dV of the current state
 * (VolumeIntegral.c; InitialSolution.c:118) and from then on every step adds, per
 * grid line and boundary face, dt b_s times the interface flux of the hyperbolic
 * term leaving the domain (HyperbolicFunction.c:101-106, TimeRK.c:174-192).
 * _error writes, per variable, |V + B - V0| / max(|V0|, 1) with V the volume
 * integral now and B the time integral of the boundary fluxes times the faces'
 * areas (BoundaryIntegral.c, CalculateConservationError.c). */
int gb_solver_conservation_begin(gb_solver *s);
int gb_solver_conservation_error(gb_solver *s, double *err);
/* Launch shape of the fused kernels: interfaces walked per thread (seg) and
 * threads per block, per direction (values <= 0 keep the current ones); seg = -32,
 * -64 or -128 selects shared-memory tiles of that many interfaces per block (one
 * interface per thread, for small grids; block is then the tile); seg = -8 or -16
 * (Euler1D, component-wise WENO5, no gravity) tiles of that many interfaces with 8
 * lanes per interface, one per reconstruction (for short 1-D lines). */
int gb_solver_set_launch(gb_solver *s, int dir, int seg, int block);
int gb_solver_get_launch(gb_solver *s, int dir, int *seg, int *block);
/* Choose seg/block per direction by timing candidates on `reps` steps of the
 * resident solution (restored afterwards): segment lengths that spread the
 * walk evenly over the SMs in 1..4 waves, and fixed lengths 8..64. */
int gb_solver_autotune(gb_solver *s, int reps);
/* 1 if every value of the resident interior solution is finite, else 0. */
int gb_solver_check_finite(gb_solver *s, int *finite);

/* Launch-group profiler (the counterpart of the reference's GPU_STAT timers):
 * when enabled, a CUDA event pair on the solver's stream brackets every launch
 * group; gb_solver_profile_read() waits for them and returns, per class, the
 * accumulated milliseconds and the number of kernel launches.  Enabling or
 * disabling resets the counters. */
enum { GB_PROF_HYP_X = 0, GB_PROF_HYP_Y = 1, GB_PROF_HYP_Z = 2, GB_PROF_VISC = 3, GB_PROF_BC = 4,
       GB_PROF_CLASSES = 5 };
int gb_solver_profile(gb_solver *s, int enable);
int gb_solver_profile_read(gb_solver *s, double *ms, long long *launches);

/* ---- batched ensemble: HyPar's ensemble mode (several independent
 *      simulations, possibly of different sizes, one TimeRK) ----
 * Members share model, schemes, time step and Butcher table and differ in size,
 * boundaries and initial data.  Every Runge-Kutta stage is one launch per
 * direction over all members; gb_ensemble_step replays one captured CUDA graph
 * per step.  Inviscid models only; boundary zones must cover whole faces. */
typedef struct gb_ensemble gb_ensemble;
int gb_ensemble_create(const gb_config *cfgs, const double *const *dxinvs, int nsims, int device, gb_ensemble **out);
void gb_ensemble_destroy(gb_ensemble *e);
int gb_ensemble_size(const gb_ensemble *e);
int gb_ensemble_set_stream(gb_ensemble *e, void *stream);
int gb_ensemble_sync(gb_ensemble *e);
int gb_ensemble_set_state(gb_ensemble *e, int member, const double *u, int layout, int mem);
int gb_ensemble_get_state(gb_ensemble *e, int member, double *u, int layout, int mem);
int gb_ensemble_step(gb_ensemble *e, int nsteps);
double gb_ensemble_time(const gb_ensemble *e);
/* Launch shape per direction, as gb_solver_set_launch: seg > 0 interfaces walked per
 * thread, seg = -32, -64 or -128 one block per tile of that many interfaces of a
 * member's grid line; 0 keeps the current value.  With a tile form, block = -1
 * selects the persistent work-list kernel (HyPar's ensemble mode,
 * src/TimeIntegration/TimeRK.c:164-170, as one launch per stage and direction of as
 * many blocks as the SMs hold, taking the members' tiles from an atomic counter),
 * block > 0 the grid launch of one block per tile; get_launch reports -1 for the
 * persistent form. */
int gb_ensemble_set_launch(gb_ensemble *e, int dir, int seg, int block);
int gb_ensemble_get_launch(gb_ensemble *e, int dir, int *seg, int *block);
/* Choose seg/block (walker or tiles) per direction by timing graph-replayed steps
 * (state restored). */
int gb_ensemble_autotune(gb_ensemble *e, int reps);
/* CalculateError of one member against its exact solution (as gb_solver_error). */
int gb_ensemble_error(gb_ensemble *e, int member, const double *uex, int layout, int mem, double *err);
/* The conservation check of every member (as gb_solver_conservation_*). */
int gb_ensemble_conservation_begin(gb_ensemble *e);
int gb_ensemble_conservation_error(gb_ensemble *e, int member, double *err);

/* Read the deck in `dir`, run n_iter steps on the GPU and write op.bin (and
 * op_NNNNN.bin every file_op_iter steps when op_overwrite is "no") in HyPar's
 * binary format (src/IOFunctions/WriteBinary.c); an ensemble deck
 * (simulation.inp) runs as one batched ensemble and writes op_<k>.bin /
 * op_<k>_NNNNN.bin per simulation.  The drop-in for HyPar's main() on this path. */
int gb_run_case(const char *dir, int device, int verbose);
/* Write a HyPar binary solution file from an interior solution. */
int gb_write_binary(const char *path, int ndims, int nvars, const int *dim, const double *x, const double *u);
/* The same as HyPar's text file (WriteText.c: per point the grid indices, the
 * coordinates and the variables, dimension 0 fastest) and Tecplot point file
 * (WriteTecplot2D.c / WriteTecplot3D.c: that with a VARIABLES / ZONE header; 2-D
 * and 3-D grids). */
int gb_write_text(const char *path, int ndims, int nvars, const int *dim, const double *x, const double *u);
int gb_write_tecplot(const char *path, int ndims, int nvars, const int *dim, const double *x, const double *u);
/* Compare two binary solution files as the reference's Extras/hyparDiff.c does: the
 * L1 / L2 / Linf norms of (ref - sol) over every variable, absolute and relative to the
 * reference's norms (absolute when any of those is below 1e-14).  GB_ERR_INPUT when the
 * files differ in ndims, nvars or size. */
int gb_diff_binary(const char *sol_path, const char *ref_path, double *abs_norms, double *rel_norms);
/* Convert a binary solution file (op*.bin) into a binary initial.inp, for a
 * restart (the reference's Extras/BinaryOPToInitialSolution.c). */
int gb_op_to_initial(const char *op_path, const char *initial_path);

/* Measure the device's FP64 fused-multiply-add throughput (TFLOP/s, an FMA
 * counted as two operations) with a register-resident DFMA loop: the
 * denominator of the FP64-pipe roofline of the fused kernels. */
int gb_probe_fp64_peak(double *tflops);
/* No counterpart in the reference: evaluates, for n device doubles x, the fused
 * kernels' refined reciprocal, square root and reciprocal square root (rcp_nr,
 * sqrt_nr, rsqrt_nr; rsqrt_nr may be NULL) beside the correctly rounded 1/x and
 * sqrt(x) (rcp_ieee, sqrt_ieee), all device arrays, so the refinements' error
 * bound can be checked directly.  Synchronises the device. */
int gb_probe_rcp_sqrt(const double *x, double *rcp_nr, double *rcp_ieee, double *sqrt_nr, double *sqrt_ieee,
                      double *rsqrt_nr, long long n);

/* ---- HyPar's function-pointer surface (device arrays, HyPar layout) ---- */

/* HyperbolicFunction (include/hypar.h:250-253, src/HyParFunctions/HyperbolicFunction.c:31).
 * FluxFunction / UpwindFunction must be gb_FFunction / gb_Upwind (or NULL for
 * the solver's configured ones): the pair selects the fused kernels. */
int gb_HyperbolicFunction(double *hyp, double *u, void *s, void *m, double t, int LimFlag,
                          int (*FluxFunction)(double *, double *, int, void *, double),
                          int (*UpwindFunction)(double *, double *, double *, double *, double *, double *,
                                                int, void *, double));
/* ParabolicFunction (include/hypar.h:256; NavierStokes3DParabolicFunction.c:50).
 * Zero for the Euler models. */
int gb_ParabolicFunction(double *par, double *u, void *s, void *m, double t);
/* SourceFunction (include/hypar.h:259): the gravity source term (Euler1D,
 * NavierStokes3D with gravity: Euler1DSource.c, NavierStokes3DSource.c), else zero. */
int gb_SourceFunction(double *source, double *u, void *s, void *m, double t);
/* FFunction (include/hypar.h:276): cell flux along dir at every point. */
int gb_FFunction(double *f, double *u, int dir, void *s, double t);
/* GFunction (include/hypar.h:310): these models define none; writes zeros. */
int gb_GFunction(double *f, double *u, int dir, void *s, double t);
/* UFunction (include/hypar.h:321): modified solution uC at every point. */
int gb_UFunction(double *uC, double *u, int dir, void *s, void *m, double t);
/* Upwind (include/hypar.h:295): interface flux from reconstructed values;
 * fI, fL, fR, uL, uR are interface arrays (no ghosts, dim[dir]+1 along dir). */
int gb_Upwind(double *fI, double *fL, double *fR, double *uL, double *uR, double *u, int dir, void *s,
              double t);
/* SetInterpLimiterVar (include/hypar.h:234): checks its arguments; the WENO5 weights
 * the reference stores here are evaluated by gb_InterpolateInterfacesHyp from the same
 * fC and u (HyperbolicFunction.c:201-215 passes the same arrays to both on the explicit
 * path, LimFlag = 1).  Weights frozen across calls (LimFlag = 0, which only HyPar's
 * implicit time integrators use) are not kept. */
int gb_SetInterpLimiterVar(double *fC, double *u, double *x, int dir, void *s, void *m);
/* InterpolateInterfacesHyp (include/hypar.h:224; Interp1PrimFifthOrderWENO.c,
 * Interp1PrimFifthOrderWENOChar.c): WENO5 values fI at the interfaces along dir
 * (interface array, dim[dir]+1 along dir, no ghosts) of the ghosted cell array fC,
 * left-biased for upw > 0, right-biased for upw < 0, with the nonlinear weights of
 * fC (uflag 0) or of u (uflag 1); characteristic in the Roe eigenvectors of u when
 * configured.  Ghost points are read as they are (apply the boundaries first).
 * WENO5 only. */
int gb_InterpolateInterfacesHyp(double *fI, double *fC, double *u, double *x, int upw, int dir, void *s, void *m,
                                int uflag);
/* ApplyBoundaryConditions (include/hypar.h:214): fills ghost points of u in place. */
int gb_ApplyBoundaryConditions(void *s, void *m, double *u, double *uref, double t);
/* TimeIntegration.RHSFunction = TimeRHSFunctionExplicit
 * (include/timeintegration_struct.h:98, src/TimeIntegration/TimeRHSFunctionExplicit.c:30):
 * applies the boundary conditions to u in place, rhs = -hyp + par + source. */
int gb_RHSFunctionExplicit(double *rhs, double *u, void *s, void *m, double t);
/* TimeRK (src/TimeIntegration/TimeRK.c:35) for `ts` = a gb_solver: one
 * Runge-Kutta step of the resident solution.  HyPar passes its TimeIntegration*
 * here; a binding maps it to the gb_solver of each simulation (INTEGRATION.md's
 * gbshim_TimeRK does, for the solution in HyPar's gpu_u array) and installs
 * the physics model's stage / step hooks with gb_solver_set_hooks. */
int gb_TimeRK(void *ts);
/* HyPar's stage and step hooks (include/hypar.h:334-341) for the fused step
 * (gb_TimeRK, gb_solver_step and the monitored step): PreStep(u, solver, mpi, t)
 * before each step (TimePreStep.c:122-124); PostStage(U_s, solver, mpi, t_s) on
 * every stage state before its right-hand side, t_s = t + c_s dt (TimeRK.c:155-162),
 * with U_s a copy where the stage's state is the solution itself, as the
 * reference's U[stage] is; PostStep(u, solver, mpi, t + dt, iter) after each step
 * (TimePostStep.c:95-97), iter = the 0-based index of the step just taken since
 * the last gb_solver_set_state.  `solver` and `mpi` are passed through (HyPar's
 * HyPar* and MPIVariables*); arrays are the solver's DEVICE arrays.  Each hook is
 * called on the host with the solver's stream synchronised, and the device is
 * synchronised again after it returns.  NULL removes a hook.  A non-NULL
 * PreStage returns GB_ERR_UNSUPPORTED, as the reference's TimeRK refuses it
 * (TimeRK.c:144-152).  A hook returning nonzero stops the step with GB_ERR_HOOK.
 * The autotuner's trial steps call no hook. */
int gb_solver_set_hooks(gb_solver *s, int (*PreStage)(int, double **, void *, void *, double),
                        int (*PostStage)(double *, void *, void *, double),
                        int (*PreStep)(double *, void *, void *, double),
                        int (*PostStep)(double *, void *, void *, double, int), void *solver, void *mpi);

/* ---- discrete adjoint and tangent-linear model ----
 * No counterpart in the reference (which has no derivative code): derivatives
 * of this library's own discrete operator -- the right-hand side of Euler2D
 * with component-wise WENO5 (Jiang-Shu weights, the derivative of the
 * nonlinear weights included) and Roe upwinding (through the Roe average, the
 * eigen-structure and Harten's entropy fix), and of n explicit Runge-Kutta
 * steps.  Every boundary face must be one whole-face periodic or extrapolate
 * zone.  Arrays are DEVICE arrays in HyPar's ghosted layout; only interior
 * entries are read or written (ghost entries of outputs are left as they are,
 * except where a call says it clears them).
 *
 * gb_adjoint_create: nsteps steps of cfg->dt; ncheck checkpoints (<= 0:
 * ceil(sqrt(nsteps)); 1 keeps every state of the whole run).  The run is cut
 * into ncheck segments: the forward sweep stores u at the start of each and
 * every stage state of the last; the backward sweep recomputes each earlier
 * segment once from its checkpoint with the fused forward kernels, keeping its
 * stage states, then reverses it step by step.  Per kept stage the forward
 * kernels also record an interface tape for the reversal: 72 doubles per
 * interface when those tapes fit in 60 % of the device memory left free by the
 * states, else 8 (gb_adjoint_info reports the bytes held). */
typedef struct gb_adjoint gb_adjoint;
int gb_adjoint_create(const gb_config *cfg, const double *dxinv, int nsteps, int ncheck, int device,
                      gb_adjoint **out);
/* As gb_adjoint_create with a cap on the wide tapes' bytes: < 0 the automatic
 * choice above, 0 always the 8-double tape, > 0 wide tapes up to that many bytes. */
int gb_adjoint_create_ex(const gb_config *cfg, const double *dxinv, int nsteps, int ncheck, int device,
                         long long wide_tape_max, gb_adjoint **out);
void gb_adjoint_destroy(gb_adjoint *a);
int gb_adjoint_set_stream(gb_adjoint *a, void *stream);
int gb_adjoint_sync(gb_adjoint *a);
/* Launch shape: which = 0, 1 the fused forward kernels along x, y (seg,
 * block); 2, 3 the adjoint kernel's segment length along x, y (block: the
 * threads per block of its single launch, shared by 2 and 3). */
int gb_adjoint_set_launch(gb_adjoint *a, int which, int seg, int block);
int gb_adjoint_get_launch(const gb_adjoint *a, int which, int *seg, int *block);
/* Segment length, number of segments, steps recomputed by the last backward
 * sweep, device bytes held. */
int gb_adjoint_info(const gb_adjoint *a, int *seglen, int *nseg, long long *recomputed, long long *bytes);
/* ubar = (dR/du)^T kbar for the right-hand side R (ubar cleared first). */
int gb_adjoint_rhs_vjp(gb_adjoint *a, const double *u, const double *kbar, double *ubar);
/* k = R(u), dk = (dR/du) du, by an independent dual-number kernel written in
 * the reference's dense-matrix form of the Roe flux. */
int gb_adjoint_rhs_jvp(gb_adjoint *a, const double *u, const double *du, double *k, double *dk);
/* Forward sweep: uT = nsteps steps from u0, storing the checkpoints. */
int gb_adjoint_forward(gb_adjoint *a, const double *u0, double *uT);
/* Backward sweep of the last forward sweep: ubar0 = (duT/du0)^T ubarT. */
int gb_adjoint_backward(gb_adjoint *a, const double *ubarT, double *ubar0);
/* Tangent-linear model: uT and duT = (duT/du0) du0 through nsteps steps of
 * the dual-number right-hand side. */
int gb_adjoint_tlm(gb_adjoint *a, const double *u0, const double *du0, double *uT, double *duT);

/* ---- right-hand side without device allocation ----
 * No counterpart in the reference.  For callers that must not allocate device
 * memory (code running inside a memory pool or arena it does not own, hosts
 * with a locked-down allocator, allocation-free sections of a time loop): the
 * rhs of gb_RHSFunctionExplicit for an INVISCID configuration, with no
 * gb_solver and no device allocation.  cfg: the configuration (the
 * Runge-Kutta fields are ignored, rk_nstages included); dxinv: DEVICE array of sum_d
 * (dim[d]+2*ghosts) values; u, rhs: DEVICE arrays in HyPar's ghosted layout
 * (u's ghost points are filled in place, as gb_RHSFunctionExplicit does);
 * stream: a cudaStream_t (NULL: the legacy default stream).  Work is queued on
 * `stream`; the call does not wait for it.
 * The directions before the last accumulate into a library-wide device array
 * of GB_NOALLOC_SCRATCH_BYTES (64 MiB) that every GPU loading the library
 * holds until exit; a 2-D or 3-D grid whose ghosted solution is larger is
 * rejected with GB_ERR_ARG (1-D grids need no scratch).  With 3 ghost points
 * the largest grids that fit are 1442 x 1442 for Euler2D and 112^3 for
 * NavierStokes3D (non-square grids: prod_d (dim[d]+6) * nvars * 8 bytes
 * <= 64 MiB).  Viscous NS3D (Re > 0)
 * returns GB_ERR_UNSUPPORTED.  All calls on a device share that array: calls
 * whose work overlaps on the GPU (different streams, no ordering between
 * them) race and give wrong results; keep them on one stream or order them.
 * The first call on each device looks the array's address up
 * (cudaGetSymbolAddress) with that device current: make it before any stream
 * capture begins.  The address is cached for the life of the process; after a
 * cudaDeviceReset of that device the cache is stale, so do not call this entry
 * point on a device that has been reset. */
#define GB_NOALLOC_SCRATCH_BYTES (64ull << 20)
int gb_rhs_explicit_noalloc(const gb_config *cfg, const double *dxinv, double *rhs, double *u, void *stream);

#ifdef __cplusplus
}
#endif
#endif
