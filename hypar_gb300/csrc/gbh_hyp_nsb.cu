// NS3D instantiation of the batched (ensemble) kernels: the segment
// walker and the tile form over all members of an ensemble.
#include "gbh_hyp_impl.cuh"
namespace gbh {
cudaError_t launch_batched_ns3d(int dir, int chr, int upw, const MemberDev* mem, int nmem, long long total,
                                const double* U, double* H, const double* dxinv, const PhysParams& pp,
                                const StageEpi& ep, int block, int tile, unsigned long long* counter,
                                cudaStream_t s) {
  return launch_batched_model<MODEL_NS3D>(dir, chr, upw, mem, nmem, total, U, H, dxinv, pp, ep, block, tile, counter, s);
}
}  // namespace gbh
