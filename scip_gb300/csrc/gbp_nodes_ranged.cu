// The node kernel with ranged-row propagation (GBP_FLAG_RANGEDROW) compiled in, in a translation unit of its own so
// that it builds in parallel with gbp_kernels.cu.
#include "gbp_nodes.cuh"

namespace gbp {
cudaError_t launchNodesRanged(cudaStream_t st, int grid, int nt, const NodesArgs& A) {
  return launchNodesT<true>(st, grid, nt, A);
}
cudaError_t nodesOccupancyRanged(int nt, int minb, int* blocksPerSm) { return nodesOccupancyT<true>(nt, minb, blocksPerSm); }
}  // namespace gbp
