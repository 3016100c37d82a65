/*
 * gbh_oracle.h -- CPU restatement of HyPar's explicit WENO5 right-hand side
 * and Runge-Kutta step, used ONLY as the parity checker and as the timed CPU
 * baseline.  It is test infrastructure: the GPU product never links it.
 *
 * Every routine restates the reference's arithmetic in the same operation
 * order (compiled with -ffp-contract=off), so that on the same inputs it
 * reproduces the reference CPU build bit for bit; the pinning test compares it
 * against the reference itself, built from source into oracle/_ref/.
 *
 * Layout (as the reference, include/arrayfunctions.h:40-47): arrays carry
 * `ghosts` ghost points on every side, dimension 0 is the fastest index and
 * the `nvars` components of a point are contiguous (u[nvars*p + v]).
 */
#ifndef GBH_ORACLE_H
#define GBH_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

enum { ORC_EULER1D = 1, ORC_EULER2D = 2, ORC_NS3D = 3 };
enum { ORC_UPW_ROE = 0, ORC_UPW_LLF = 1, ORC_UPW_RF = 2, ORC_UPW_RUSANOV = 3, ORC_UPW_SWFS = 4 };
enum { ORC_INTERP_COMP = 0, ORC_INTERP_CHAR = 1 };
enum { ORC_BC_PERIODIC = 1, ORC_BC_EXTRAPOLATE = 2, ORC_BC_DIRICHLET = 3, ORC_BC_SLIP_WALL = 4,
       ORC_BC_NOSLIP_WALL = 5, ORC_BC_SUBSONIC_INFLOW = 6, ORC_BC_SUBSONIC_OUTFLOW = 7,
       ORC_BC_SUPERSONIC_INFLOW = 8, ORC_BC_SUPERSONIC_OUTFLOW = 9, ORC_BC_SUBSONIC_AMBIVALENT = 10,
       ORC_BC_THERMAL_SLIP_WALL = 11, ORC_BC_THERMAL_NOSLIP_WALL = 12, ORC_BC_SPONGE = 13,
       ORC_BC_TURBULENT_INFLOW = 14, ORC_BC_REFLECT = 15 };

/* One boundary zone, as DomainBoundary after CalculateLocalExtent
 * (src/Simulation/InitializeBoundaries.c:365-420): the slab covers index
 * range [is[d], ie[d]) in every dimension d, with is[dim] = -ghosts,
 * ie[dim] = 0 on face +1 and is[dim] = N, ie[dim] = N+ghosts on face -1. */
typedef struct {
  int type, dim, face;
  int is[3], ie[3];
  double data[8];   /* boundary.inp values after the extents (Dirichlet values, wall velocity, ...) */
} orc_zone;

typedef struct {
  int model, ndims, nvars, ghosts, dim[3];
  int upwind, interp;
  double gamma, eps;
  double Re, Pr;        /* Re already divided by Minf (NavierStokes3DInitialize.c:368); Re<=0: inviscid */
  int nzones;
  orc_zone zones[12];
  double *dxinv;        /* sum_d (dim[d]+2*ghosts), per point 2/(x[i+1]-x[i-1]) */
  int weights;          /* ORC_WENO_*: nonlinear weight formulation */
  int scheme;           /* ORC_SCHEME_*: hyp_space_scheme */
  /* NavierStokes3D gravity (well-balanced form): acceleration, RT = p0/rho0 and the
   * hydrostatic fields f (density) and g (pressure) at every point with ghosts */
  int has_grav;
  double grav[3], RT;
  double *gf, *gg;
  /* the time the boundaries of orc_apply_bc / orc_rhs are evaluated at (orc_rk
   * starts its steps there), and per thermal-wall zone the wall temperature's time
   * levels and field (BCReadTemperatureData layout: the zone's extent with the time
   * level along its own dimension) */
  double t;
  int tn[12];
  double *ttimes[12], *tfield[12];
  /* per sponge zone the interior grid coordinates along its dimension and its bounds
   * there (boundary.inp xmin, xmax) */
  double *sx[12], sxmin[12], sxmax[12];
  /* per turbulent inflow zone the number of slices and the inflow data */
  int fn[12];
  double *fdata[12];
  /* NavierStokes3D par_space_scheme: 4 (0: 4) or 2 */
  int par_scheme;
} orc_problem;

/* WENO5 weights: Jiang-Shu, mapped (Henrick-Aslam-Powers), Borges (WENO-Z),
 * Yamaleev-Carpenter, or the optimal weights (no_limiting). */
enum { ORC_WENO_JS = 0, ORC_WENO_MAPPED = 1, ORC_WENO_BORGES = 2, ORC_WENO_YC = 3, ORC_WENO_NONE = 4 };
void orc_set_weights(orc_problem *p, int weights);
/* hyp_space_scheme: WENO5, or CRWENO5 (compact, a tridiagonal solve per grid line;
 * component-wise, without gravity) */
enum { ORC_SCHEME_WENO5 = 0, ORC_SCHEME_CRWENO5 = 1 };
void orc_set_scheme(orc_problem *p, int scheme);
/* NavierStokes3D gravity: acceleration (gx, gy, gz), reference density and
 * pressure, gas constant R, hydrostatic balance type HB (1, 2, 3; N_bv for 3)
 * and the grid with ghost coordinates, sum_d (dim[d]+2g) values
 * (NavierStokes3DGravityField.c). */
int orc_set_gravity(orc_problem *p, const double *xg, double gx, double gy, double gz, double rho0, double p0,
                    double R, int HB, double Nbv);
void orc_get_gravity(const orc_problem *p, double *out);
/* Euler1D gravity (physics.inp gravity, gravity_type 0 or 1) from the grid with ghost
 * coordinates (Euler1DGravityField.c): gg = S, gf = 1/S. */
int orc_set_gravity_1d(orc_problem *p, const double *xg, double g, int type);
/* The values boundary.inp gives for zone z after its extents (8 doubles). */
void orc_set_zone_data(orc_problem *p, int z, const double *data);
/* Thermal walls: the wall temperature of zone z at n time levels (times[n]) over the
 * zone's extent (field: the zone's extent per dimension, n along the zone's own
 * dimension, dimension 0 fastest); copied. */
int orc_set_zone_temperature(orc_problem *p, int z, int n, const double *times, const double *field);
/* The time of orc_apply_bc and orc_rhs and the start time of orc_rk. */
void orc_set_time(orc_problem *p, double t);
/* Sponge zones: the interior grid coordinates along zone z's dimension (dim[dim] values)
 * and the zone's bounds there, boundary.inp's xmin and xmax of that dimension. */
int orc_set_zone_sponge(orc_problem *p, int z, const double *x, double xmin, double xmax);
/* Turbulent inflow zones: n slices of inflow data (the grid's size across the zone's
 * dimension, n along it, nvars values per point, dimension 0 fastest). */
int orc_set_zone_inflow(orc_problem *p, int z, int n, const double *data);
/* NavierStokes3D viscous term: par_space_scheme 2 or 4. */
void orc_set_par_scheme(orc_problem *p, int scheme);

/* Create/destroy a problem.  zones: nzones x 9 ints (type,dim,face,is[3],ie[3]);
 * dxinv: sum_d (dim[d]+2g) doubles (copied). */
orc_problem *orc_problem_create(int model, int ndims, const int *dim, int ghosts,
                                int upwind, int interp, double gamma, double eps,
                                double Re_over_Minf, double Pr, int nzones,
                                const int *zones, const double *dxinv);
void orc_problem_destroy(orc_problem *p);

/* Number of points with ghosts. */
long orc_npoints_wghosts(const orc_problem *p);

/* Boundary ghost fill on u in place (ApplyBoundaryConditions). */
int orc_apply_bc(const orc_problem *p, double *u);
/* Hyperbolic term hyp (with ghosts, ghosts zero) from a BC-filled u. */
int orc_hyperbolic(const orc_problem *p, const double *u, double *hyp);
/* NavierStokes3D viscous term par (with ghosts) from a BC-filled u. */
int orc_parabolic(const orc_problem *p, const double *u, double *par);
/* TimeRHSFunctionExplicit: fills u's ghosts in place, rhs = -hyp + par. */
/* gravity source term, zero elsewhere (SourceFunction) */
int orc_source(const orc_problem *p, const double *u, double *src);
int orc_rhs(const orc_problem *p, double *u, double *rhs);
/* TimeRK over nsteps steps of the Butcher tableau (A: ns x ns row major, b). */
int orc_rk(const orc_problem *p, int nstages, const double *A, const double *b,
           double *u, double dt, int nsteps);
/* Maximum CFL of a ghosted solution for time step dt (<Model>ComputeCFL). */
double orc_cfl(const orc_problem *p, const double *u, double dt);
/* Set the OpenMP thread count used by the oracle (<=0: library default). */
void orc_set_threads(int n);
int orc_get_threads(void);

#ifdef __cplusplus
}
#endif
#endif
