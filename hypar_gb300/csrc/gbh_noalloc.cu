// gbh_noalloc.cu -- gb_rhs_explicit_noalloc: the explicit right-hand side of
// an inviscid configuration computed without allocating any device memory.
//
// Who needs it: callers that may not allocate device memory themselves or
// through this library -- code running inside a memory pool or arena they
// do not own, hosts whose allocator is locked down, or allocation-free
// sections of a time-stepping loop.  gb_RHSFunctionExplicit needs a gb_solver,
// and gb_solver_create allocates the solution, stage and accumulator arrays.
//
// This entry point computes the same rhs as gb_RHSFunctionExplicit, with the
// same fused direction kernels, but takes every array from the caller and
// keeps the one intermediate those kernels need -- the hyperbolic term
// accumulated over the directions before the last -- in a file-scope device
// array of GB_NOALLOC_SCRATCH_BYTES.  That array is part of the library's
// device image: every GPU that loads the library holds it until the process
// exits.
#include <cstring>
#include <mutex>

#include "gbh_internal.h"

namespace gbh {
cudaError_t launch_hyp_euler1d(int, int, int, const double*, double*, const double*, const DevGeom&,
                               const PhysParams&, const StageEpi&, const HypLaunch&, cudaStream_t);
cudaError_t launch_hyp_euler2d(int, int, int, const double*, double*, const double*, const DevGeom&,
                               const PhysParams&, const StageEpi&, const HypLaunch&, cudaStream_t);
cudaError_t launch_hyp_ns3d(int, int, int, const double*, double*, const double*, const DevGeom&,
                            const PhysParams&, const StageEpi&, const HypLaunch&, cudaStream_t);
cudaError_t launch_hyp_euler1d_w(int, int, int, const double*, double*, const double*, const DevGeom&,
                                 const PhysParams&, const StageEpi&, const HypLaunch&, cudaStream_t);
cudaError_t launch_hyp_euler2d_w(int, int, int, const double*, double*, const double*, const DevGeom&,
                                 const PhysParams&, const StageEpi&, const HypLaunch&, cudaStream_t);
cudaError_t launch_hyp_ns3d_w(int, int, int, const double*, double*, const double*, const DevGeom&,
                              const PhysParams&, const StageEpi&, const HypLaunch&, cudaStream_t);
cudaError_t launch_bc_zone(double*, const DevGeom&, int, const int*, const double*, double, cudaStream_t);
}  // namespace gbh

using namespace gbh;

// The shared scratch: the hyperbolic term of the directions before the last,
// in the ghosted layout of the solution.
static __device__ __align__(256) double g_noalloc_scratch[GB_NOALLOC_SCRATCH_BYTES / sizeof(double)];

// Address of g_noalloc_scratch per device, looked up on the first call made
// with that device current.  The cache lives as long as the process: after
// cudaDeviceReset (or anything else that destroys and re-creates the device's
// primary context, which may load the module at a new address) it is stale, so
// a process that resets a device must not call this entry point afterwards.
static constexpr int kMaxDevices = 64;
static std::mutex g_noalloc_mu;
static double* g_noalloc_ptr[kMaxDevices];

static int noalloc_scratch(double** out) {
  int dev = -1;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) {
    gbh_set_error("gb_rhs_explicit_noalloc: cudaGetDevice: %s", cudaGetErrorString(e));
    return GB_ERR_CUDA;
  }
  if (dev < 0 || dev >= kMaxDevices) {
    gbh_set_error("gb_rhs_explicit_noalloc: device %d beyond the %d supported", dev, kMaxDevices);
    return GB_ERR_ARG;
  }
  std::lock_guard<std::mutex> lock(g_noalloc_mu);
  if (!g_noalloc_ptr[dev]) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p) {
      gbh_set_error("gb_rhs_explicit_noalloc: cudaGetSymbolAddress on device %d: %s", dev,
                    e != cudaSuccess ? cudaGetErrorString(e) : "null address");
      return GB_ERR_CUDA;
    }
    g_noalloc_ptr[dev] = (double*)p;
  }
  *out = g_noalloc_ptr[dev];
  return GB_OK;
}

#define NA_CK(x)                                                                        \
  do {                                                                                  \
    cudaError_t e_ = (x);                                                               \
    if (e_ != cudaSuccess) {                                                            \
      gbh_set_error("gb_rhs_explicit_noalloc: %s", cudaGetErrorString(e_));             \
      return GB_ERR_CUDA;                                                               \
    }                                                                                   \
  } while (0)

extern "C" int gb_rhs_explicit_noalloc(const gb_config* cfg, const double* dxinv, double* rhs, double* u,
                                       void* stream) {
  if (!cfg || !dxinv || !rhs || !u) {
    gbh_set_error("gb_rhs_explicit_noalloc: null argument");
    return GB_ERR_ARG;
  }
  // The Runge-Kutta fields play no part in a right-hand side: validate the rest
  // of the configuration with a one-stage table in their place.
  gb_config checked = *cfg;
  checked.rk_nstages = 1;
  int rc = gbh_validate(&checked);
  if (rc) return rc;
  const gb_config& c = *cfg;
  if (c.gravity[0] != 0.0 || c.gravity[1] != 0.0 || c.gravity[2] != 0.0) {
    gbh_set_error("gb_rhs_explicit_noalloc: gravity is not available here; use gb_RHSFunctionExplicit");
    return GB_ERR_UNSUPPORTED;
  }
  for (int z = 0; z < c.nzones; z++)
    if (c.zones[z][0] == GB_BC_THERMAL_SLIP_WALL || c.zones[z][0] == GB_BC_THERMAL_NOSLIP_WALL) {
      gbh_set_error("gb_rhs_explicit_noalloc: thermal walls need the temperature field of a gb_solver; "
                    "use gb_RHSFunctionExplicit");
      return GB_ERR_UNSUPPORTED;
    } else if (c.zones[z][0] == GB_BC_TURBULENT_INFLOW) {
      gbh_set_error("gb_rhs_explicit_noalloc: turbulent inflow needs the inflow data of a gb_solver; "
                    "use gb_RHSFunctionExplicit");
      return GB_ERR_UNSUPPORTED;
    } else if (c.zones[z][0] == GB_BC_SPONGE) {
      gbh_set_error("gb_rhs_explicit_noalloc: sponge zones need the sigma of a gb_solver; use gb_RHSFunctionExplicit");
      return GB_ERR_UNSUPPORTED;
    }
  if (c.hyp_scheme != GB_SCHEME_WENO5) {
    gbh_set_error("gb_rhs_explicit_noalloc: CRWENO5 needs scratch for its line solves; use gb_RHSFunctionExplicit");
    return GB_ERR_UNSUPPORTED;
  }
  if (c.model == GB_MODEL_NS3D && c.Re > 0) {
    gbh_set_error("gb_rhs_explicit_noalloc: the viscous term is not available here (Re > 0); "
                  "use gb_RHSFunctionExplicit");
    return GB_ERR_UNSUPPORTED;
  }
  DevGeom G;
  const long long npts = gbh_geometry(c, G, nullptr);
  const size_t nvals = (size_t)npts * c.nvars;
  const size_t need = c.ndims > 1 ? nvals * sizeof(double) : 0;
  if (need > (size_t)GB_NOALLOC_SCRATCH_BYTES) {
    gbh_set_error("gb_rhs_explicit_noalloc: the grid needs %zu bytes of scratch, the limit is %llu bytes; "
                  "use gb_RHSFunctionExplicit",
                  need, (unsigned long long)GB_NOALLOC_SCRATCH_BYTES);
    return GB_ERR_ARG;
  }
  double* H = nullptr;
  rc = noalloc_scratch(&H);
  if (rc) return rc;
  cudaStream_t st = (cudaStream_t)stream;

  // As gb_RHSFunctionExplicit: every boundary zone fills u's ghost points in
  // place, then rhs (ghosts included) is cleared and its interior written.
  for (int z = 0; z < c.nzones; z++) NA_CK(launch_bc_zone(u, G, c.nvars, c.zones[z], c.zone_data[z], c.gamma, st));
  NA_CK(cudaMemsetAsync(rhs, 0, nvals * sizeof(double), st));

  PhysParams pp{};
  pp.gamma = c.gamma;
  pp.gm1 = c.gamma - 1.0;
  pp.inv_gm1 = 1.0 / (c.gamma - 1.0);
  pp.eps = c.weno_eps;
  pp.wtype = c.weno_weights;
  pp.gf = pp.gg = nullptr;
  pp.RT = 1.0;  // no gravity here: grav[] stays zero, as in a solver without gravity
  HypLaunch hl;
  hl.seg = 32;
  hl.block = 128;
  StageEpi ep;
  memset(&ep, 0, sizeof(ep));
  ep.mode = EPI_RHS;
  ep.rhs = rhs;
  ep.par = nullptr;
  // Nothing in the scratch has to start at zero: the first direction stores
  // its term at every interior point and the later ones read only those.
  const double* dx = dxinv;
  for (int d = 0; d < c.ndims; d++) {
    StageEpi e = ep;
    e.first = (d == 0);
    e.last = (d == c.ndims - 1);
    if (pp.wtype != WENO_W_JS) {
      if (c.model == GB_MODEL_EULER1D) NA_CK(launch_hyp_euler1d_w(d, c.interp, c.upwind, u, H, dx, G, pp, e, hl, st));
      else if (c.model == GB_MODEL_EULER2D) NA_CK(launch_hyp_euler2d_w(d, c.interp, c.upwind, u, H, dx, G, pp, e, hl, st));
      else NA_CK(launch_hyp_ns3d_w(d, c.interp, c.upwind, u, H, dx, G, pp, e, hl, st));
    } else if (c.model == GB_MODEL_EULER1D) {
      NA_CK(launch_hyp_euler1d(d, c.interp, c.upwind, u, H, dx, G, pp, e, hl, st));
    } else if (c.model == GB_MODEL_EULER2D) {
      NA_CK(launch_hyp_euler2d(d, c.interp, c.upwind, u, H, dx, G, pp, e, hl, st));
    } else {
      NA_CK(launch_hyp_ns3d(d, c.interp, c.upwind, u, H, dx, G, pp, e, hl, st));
    }
    dx += c.dim[d] + 2 * c.ghosts;
  }
  return GB_OK;
}
