// Fast-numerics candidate kernel: hardware reciprocal square root,
// approximate division and contraction of multiply-add (--fmad=true) in the
// RIS candidate loop, whose results only weight the reservoir.
#include "ris_binned.cuh"

namespace risltc {
cudaError_t launch_candidates_fast(const RisParams& p, cudaStream_t stream, int grid) {
	return launch_candidates_binned<FastNumerics>(p, stream, grid);
}
}  // namespace risltc
