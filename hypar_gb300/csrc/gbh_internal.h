// gbh_internal.h -- structures shared by the CUDA translation units of
// libgbhypar (not part of the public C ABI, which is include/gbhypar.h).
#pragma once

#include <cuda_runtime.h>

#include <vector>

#include "gbhypar.h"

#include "gbh_device.cuh"

namespace gbh {

// Ghost-cell source along one face, folded into every halo load:
// memory = read the ghost point stored in the array (filled by the boundary
// kernel), periodic = wrap to the opposite interior cell, mirror = HyPar's
// "extrapolate" boundary (a mirror copy, BCExtrapolate.c:37-38).
enum { FOLD_MEMORY = 0, FOLD_PERIODIC = 1, FOLD_MIRROR = 2 };

struct DevGeom {
  int nd, g;
  int dim[3];
  long long stride[3];   // point strides including ghosts
  int bclo[3], bchi[3];  // FOLD_* per face
};

// What the last direction of a stage does with the accumulated hyperbolic
// term (hyp = sum over directions of dxinv (F[j+1/2]-F[j-1/2])):
//   EPI_HYP  : store hyp into H (first direction) or add it to H
//   EPI_RHS  : rhs = -hyp + par  into `rhs`
//   EPI_RK   : k = -hyp + par, then the Runge-Kutta stage update
enum { EPI_HYP = 0, EPI_RHS = 1, EPI_RK = 2 };

// The adjoint's wide interface tape (Euler2D): uL, uR (8 values), then per component
// the smoothness terms B (6) and normalisation reciprocals (2) of the f pair and of
// the u pair.
constexpr int TAPE_WIDE = 8 + 4 * 16;

struct StageEpi {
  int mode;        // EPI_*
  int first;       // this direction is the first one (H is not read)
  int last;        // this direction is the last one
  const double* par;  // viscous term or nullptr
  double* rhs;        // EPI_RHS output
  // Runge-Kutta stage update (EPI_RK): with k this stage's right-hand side,
  //   acc   = (stage == 0 ? u : acc) + cb k        (u = acc on the last stage)
  //   P[t]  = (touched[t] ? P[t] : u) + ca[t] k    for later stages t with ca[t] != 0
  int stage, nstages;
  double cb;
  double ca[4];
  int touched[4];
  int need_u;      // u is read this stage (first stage, or a P[t] is first touched)
  double* u;       // current solution (read)
  double* uout;    // where the last stage writes the new solution
  double* acc;
  double* P[4];
  // Euler2D component-wise only: when set, the reconstructed interface states
  // uL, uR of this direction are written here, 8 values per interface at
  // ((line * (N + 1)) + interface) * 8 (the adjoint reads them back).
  double* tape;
  // EPI_HYP only: also subtract the gravity source (NavierStokes3D with gravity),
  // so that the hyperbolic term with and without it give the source by difference.
  int with_source;
  // Conservation check (EPI_RK): when set, the interface flux at I = 0 and I = N of
  // every line is accumulated here, times -bw and +bw: ntrans x nvars values for
  // face 0, then as many for face N (HyperbolicFunction.c:101-106, TimeRK.c:188-192).
  double* bnd;
  double bw;
};

// NavierStokes3D viscous-term constants (NavierStokes3DParabolicFunction.c:76-79).
struct ViscParams {
  double gamma, gm1, inv_Re, inv_Pr, inv_gm1;
  int order;  // first derivatives: 4 (fourth-order central) or 2 (first-order one-sided)
};

// Per-launch configuration of the hyperbolic kernels.
struct HypLaunch {
  int seg;         // interfaces walked by one thread
  int block;       // threads per block
};

// Ensemble member as seen by the batched kernel: its geometry, where its
// arrays start inside the batched arrays, and which threads of a launch along
// each direction are its (start[d] .. start[d] + ntrans[d]*nseg[d]).
struct MemberDev {
  DevGeom G;
  long long off;         // first value of the member in every state array
  long long dx_off[3];   // first dxinv value of each direction
  long long start[3];    // first thread of the member per direction
  long long ntrans[3];
  int nseg[3], seg[3];
  long long bnd_off[3];  // the member's conservation-check accumulators per direction
};

// Conservation check reductions (gbh_monitor.cu).
long long cons_lines(const gb_config& c, int d);
int cons_volume(const double* u, const double* dxinv, const DevGeom& G, long long dxo1, long long dxo2, int nv,
                double* red, cudaStream_t st, double* V);
int cons_error(const gb_config& c, const double* bnd, const long long* off, const double* V, const double* V0,
               const double* dxmid, double* red, cudaStream_t st, double* err);
constexpr int CONS_RED_DOUBLES = 3 * 1024;  // the reduction buffer cons_volume / cons_error need
int grid_error(const double* u, const double* uex, const DevGeom& G, int nv, double* red, cudaStream_t st,
               double* err);

}  // namespace gbh

int gbh_validate(const gb_config* c);
long long gbh_geometry(const gb_config& c, gbh::DevGeom& G, std::vector<int>* mem_zones);
extern "C" void gbh_set_error(const char* fmt, ...);
