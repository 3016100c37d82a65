// NS3D instantiation of the fused hyperbolic kernel and the unfused pieces.
#include "gbh_hyp_impl.cuh"
namespace gbh {
cudaError_t launch_hyp_ns3d(int dir, int chr, int upw, const double* U, double* H, const double* dxinv_dir,
                               const DevGeom& G, const PhysParams& pp, const StageEpi& ep, const HypLaunch& L,
                               cudaStream_t s) {
  return launch_hyp_model<MODEL_NS3D>(dir, chr, upw, U, H, dxinv_dir, G, pp, ep, L, s);
}
cudaError_t launch_unfused_ns3d(int kind, int dir, int upw, double* out, const double* a, const double* b,
                                   const double* c, const double* d, const double* u, const DevGeom& G,
                                   const PhysParams& pp, cudaStream_t s) {
  return launch_unfused_model<MODEL_NS3D>(kind, dir, upw, out, a, b, c, d, u, G, pp, s);
}
cudaError_t launch_interp_ns3d(int dir, int chr, int left, int uf, double* fI, const double* fC, const double* u,
                                const DevGeom& G, const PhysParams& pp, cudaStream_t s) {
  return launch_interp_model<MODEL_NS3D>(dir, chr, left, uf, fI, fC, u, G, pp, s);
}
}  // namespace gbh
