// EULER1D fused hyperbolic kernels with the mapped / Borges / Yamaleev-Carpenter /
// optimal (no_limiting) WENO5 weights, selected at run time by PhysParams::wtype.
#include "gbh_hyp_impl.cuh"
namespace gbh {
cudaError_t launch_hyp_euler1d_w(int dir, int chr, int upw, const double* U, double* H, const double* dxinv_dir,
                                 const DevGeom& G, const PhysParams& pp, const StageEpi& ep, const HypLaunch& L,
                                 cudaStream_t s) {
  return launch_hyp_model<MODEL_EULER1D, true>(dir, chr, upw, U, H, dxinv_dir, G, pp, ep, L, s);
}
}  // namespace gbh
