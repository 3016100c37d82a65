// gbh_solver.h -- the gb_solver object, shared by the translation units that
// operate on a solver (not part of the public C ABI).
#pragma once

#include <vector>

#include "gbh_internal.h"

struct gb_solver {
  gb_config cfg;
  gbh::DevGeom G;
  gbh::PhysParams pp;
  gbh::ViscParams vp;
  int device = 0;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  long long npts_wg = 0;
  size_t nvals = 0;
  double* d_u = nullptr;
  double* d_acc = nullptr;
  double* d_P[4] = {nullptr, nullptr, nullptr, nullptr};
  double* d_H = nullptr;
  double* d_par = nullptr;
  double* d_Q = nullptr;
  double* d_Gr = nullptr;
  double* d_dxinv = nullptr;
  double* d_snap = nullptr;  // copy of u before a monitored step (allocated on first use)
  double* d_red = nullptr;   // reduction partials (allocated on first use)
  double* d_grav = nullptr;  // gravity fields f, g (NavierStokes3D with gravity)
  double* d_crX = nullptr;   // CRWENO5: interface values / elimination right-hand sides
  double* d_crC = nullptr;   // CRWENO5: normalised super-diagonal of the elimination
  double* d_crF = nullptr;   // CRWENO5 (component-wise): cell fluxes of the current direction
  bool gravity = false;
  // conservation check: per direction and face, the lines' boundary-flux time
  // integrals (allocated by gb_solver_conservation_begin)
  double* d_bnd = nullptr;
  long long bnd_off[3] = {0, 0, 0};
  long long bnd_n = 0;
  bool cons_on = false;
  double V0[5] = {0, 0, 0, 0, 0};
  int* d_flag = nullptr;
  std::vector<int> mem_zones;  // zone indices applied in memory before each RHS
  gbh::HypLaunch hl[3];
  int visc_seg = 16;
  double t = 0.0;
  // HyPar's stage / step hooks (include/hypar.h:334-341), installed with
  // gb_solver_set_hooks and called on the host by every fused step
  int (*post_stage)(double*, void*, void*, double) = nullptr;
  int (*pre_step)(double*, void*, void*, double) = nullptr;
  int (*post_step)(double*, void*, void*, double, int) = nullptr;
  void* hook_solver = nullptr;
  void* hook_mpi = nullptr;
  double* d_U0 = nullptr;  // stage state handed to PostStage where the stage reads u itself
  // thermal walls: per zone the wall temperature's time levels (host) and field (device)
  std::vector<double> ttimes[GB_MAX_ZONES];
  double* d_tfield[GB_MAX_ZONES] = {};
  // sponge zones: sigma along the zone's dimension (device), and whether any zone is one
  double* d_sigma[GB_MAX_ZONES] = {};
  // staging array for interior-layout host copies (allocated on first use, kept)
  double* d_stage = nullptr;
  // turbulent inflow zones: the number of slices of the inflow data (held in d_tfield)
  int fn[GB_MAX_ZONES] = {};
  bool sponge = false;
  int iter = 0;            // steps taken since the state was set (PostStep's iteration index)
  long long dx_off[3] = {0, 0, 0};
  bool viscous = false;
  // launch profiler: an event pair around every launch group, read on demand
  bool prof = false;
  struct Rec { int cls; cudaEvent_t a, b; };
  std::vector<Rec> recs;
  std::vector<cudaEvent_t> pool;
  double prof_ms[GB_PROF_CLASSES] = {0};
  long long prof_n[GB_PROF_CLASSES] = {0};
};

// One Runge-Kutta step of the resident solution (the fused launches).
int gbh_rk_step(gb_solver* s);
