// EULER2D instantiation of the fused hyperbolic kernel and the unfused pieces.
#include "gbh_hyp_impl.cuh"
namespace gbh {
cudaError_t launch_hyp_euler2d(int dir, int chr, int upw, const double* U, double* H, const double* dxinv_dir,
                               const DevGeom& G, const PhysParams& pp, const StageEpi& ep, const HypLaunch& L,
                               cudaStream_t s) {
  return launch_hyp_model<MODEL_EULER2D>(dir, chr, upw, U, H, dxinv_dir, G, pp, ep, L, s);
}
// Component-wise Jiang-Shu WENO5 + Roe (the adjoint's configuration) writing the
// wide tape (TAPE_WIDE doubles per interface) into ep.tape.
cudaError_t launch_hyp_euler2d_wide_tape(int dir, const double* U, double* H, const double* dxinv_dir,
                                         const DevGeom& G, const PhysParams& pp, const StageEpi& ep,
                                         const HypLaunch& L, cudaStream_t s) {
  if (!ep.tape) return cudaErrorInvalidValue;
  if (dir == 0) return launch_dir<MODEL_EULER2D, false, UPW_ROE, 0, false, false, true>(U, H, dxinv_dir, G, pp, ep, L, s);
  if (dir == 1) return launch_dir<MODEL_EULER2D, false, UPW_ROE, 1, false, false, true>(U, H, dxinv_dir, G, pp, ep, L, s);
  return cudaErrorInvalidValue;
}
cudaError_t launch_unfused_euler2d(int kind, int dir, int upw, double* out, const double* a, const double* b,
                                   const double* c, const double* d, const double* u, const DevGeom& G,
                                   const PhysParams& pp, cudaStream_t s) {
  return launch_unfused_model<MODEL_EULER2D>(kind, dir, upw, out, a, b, c, d, u, G, pp, s);
}
cudaError_t launch_interp_euler2d(int dir, int chr, int left, int uf, double* fI, const double* fC, const double* u,
                                const DevGeom& G, const PhysParams& pp, cudaStream_t s) {
  return launch_interp_model<MODEL_EULER2D>(dir, chr, left, uf, fI, fC, u, G, pp, s);
}
}  // namespace gbh
