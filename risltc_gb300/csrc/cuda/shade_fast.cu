// Fast numerics instantiation: hardware reciprocal square root, approximate
// division and contraction of multiply-add (compiled with --fmad=true).
#include "ris_kernels.cuh"

namespace risltc {
cudaError_t launch_shade_fast(const ShadeParams& p, cudaStream_t stream, int grid) {
	shade_kernel<FastNumerics><<<grid, 128, 0, stream>>>(p);
	return cudaGetLastError();
}
cudaError_t launch_ris_fast(const RisParams& p, cudaStream_t stream, int grid) {
	ris_candidates_kernel<FastNumerics><<<grid, 128, 0, stream>>>(p);
	cudaError_t e = cudaGetLastError();
	if (e != cudaSuccess) return e;
	ris_shade_kernel<FastNumerics><<<grid, 128, 0, stream>>>(p);
	return cudaGetLastError();
}
}  // namespace risltc
