// Fast numerics instantiation: hardware reciprocal square root, approximate
// division and contraction of multiply-add (compiled with --fmad=true).
#include "shade_kernel.cuh"

namespace risltc {
cudaError_t launch_shade_fast(const ShadeParams& p, cudaStream_t stream, int grid) {
	shade_kernel<FastNumerics><<<grid, 128, 0, stream>>>(p);
	return cudaGetLastError();
}
}  // namespace risltc
