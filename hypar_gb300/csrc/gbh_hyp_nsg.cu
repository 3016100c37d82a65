// The fused hyperbolic kernels with gravity (well-balanced source, gravity-modified
// solution, scaled dissipation), every weight formulation: NavierStokes3D (Rusanov)
// and Euler1D (Roe, LLF).
#include "gbh_hyp_impl.cuh"
namespace gbh {
cudaError_t launch_hyp_ns3d_grav(int dir, int chr, const double* U, double* H, const double* dxinv_dir,
                                 const DevGeom& G, const PhysParams& pp, const StageEpi& ep, const HypLaunch& L,
                                 cudaStream_t s) {
  if (pp.wtype != WENO_W_JS) return launch_hyp_ns3d_gravity<true>(dir, chr, U, H, dxinv_dir, G, pp, ep, L, s);
  return launch_hyp_ns3d_gravity<false>(dir, chr, U, H, dxinv_dir, G, pp, ep, L, s);
}
cudaError_t launch_hyp_euler1d_grav(int dir, int chr, int upw, const double* U, double* H, const double* dxinv_dir,
                                   const DevGeom& G, const PhysParams& pp, const StageEpi& ep, const HypLaunch& L,
                                   cudaStream_t s) {
  if (pp.wtype != WENO_W_JS) return launch_hyp_euler1d_gravity<true>(dir, chr, upw, U, H, dxinv_dir, G, pp, ep, L, s);
  return launch_hyp_euler1d_gravity<false>(dir, chr, upw, U, H, dxinv_dir, G, pp, ep, L, s);
}
}  // namespace gbh
