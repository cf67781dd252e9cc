// Exact numerics instantiation: compiled with --fmad=false and IEEE division
// and square root, so every operation matches the CPU restatement bit for bit.
#include "ris_kernels.cuh"

namespace risltc {
cudaError_t launch_shade_exact(const ShadeParams& p, cudaStream_t stream, int grid) {
	shade_kernel<ExactNumerics><<<grid, 128, 0, stream>>>(p);
	return cudaGetLastError();
}
cudaError_t launch_trace_exact(const SceneView& s, const float4* rays, uint32_t count, uint32_t* hits, uint32_t* error,
                               cudaStream_t stream, int grid) {
	trace_shadow_kernel<ExactNumerics><<<grid, 128, 0, stream>>>(s, rays, count, hits, error);
	return cudaGetLastError();
}
cudaError_t launch_ris_exact(const RisParams& p, cudaStream_t stream, int grid) {
	ris_candidates_kernel<ExactNumerics><<<grid, 128, 0, stream>>>(p);
	cudaError_t e = cudaGetLastError();
	if (e != cudaSuccess) return e;
	ris_shade_kernel<ExactNumerics><<<grid, 128, 0, stream>>>(p);
	return cudaGetLastError();
}
}  // namespace risltc
