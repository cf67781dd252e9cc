// Exact numerics instantiation: compiled with --fmad=false and IEEE division
// and square root, so every operation matches the CPU restatement bit for bit.
#include "ris_kernels.cuh"

namespace risltc {
cudaError_t launch_shade_exact(const ShadeParams& p, cudaStream_t stream, int grid, cudaEvent_t* events) {
	if (events) cudaEventRecord(events[0], stream);
	shade_kernel<ExactNumerics><<<grid, 128, 0, stream>>>(p);
	cudaError_t e = cudaGetLastError();
	if (events) {
		cudaEventRecord(events[1], stream);
		cudaEventRecord(events[2], stream);
	}
	return e;
}
cudaError_t launch_trace_exact(const SceneView& s, const float4* rays, uint32_t count, uint32_t* hits, uint32_t* error,
                               cudaStream_t stream, int grid) {
	trace_shadow_kernel<ExactNumerics><<<grid, 128, 0, stream>>>(s, rays, count, hits, error);
	return cudaGetLastError();
}
// events (may be null): recorded before, between and after the two kernels.
cudaError_t launch_ris_exact(const RisParams& p, cudaStream_t stream, int grid, cudaEvent_t* events) {
	if (events) cudaEventRecord(events[0], stream);
	ris_candidates_kernel<ExactNumerics><<<grid, 128, 0, stream>>>(p);
	cudaError_t e = cudaGetLastError();
	if (e != cudaSuccess) return e;
	if (events) cudaEventRecord(events[1], stream);
	ris_shade_kernel<ExactNumerics><<<grid, 128, 0, stream>>>(p);
	e = cudaGetLastError();
	if (events) cudaEventRecord(events[2], stream);
	return e;
}
}  // namespace risltc
