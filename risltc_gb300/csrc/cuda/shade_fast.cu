// Fast numerics instantiation: hardware reciprocal square root, approximate
// division and contraction of multiply-add (compiled with --fmad=true).
#include "ris_kernels.cuh"

namespace risltc {
cudaError_t launch_shade_fast(const ShadeParams& p, cudaStream_t stream, int grid, cudaEvent_t* events) {
	if (events) cudaEventRecord(events[0], stream);
	shade_kernel<FastNumerics><<<grid, 128, 0, stream>>>(p);
	cudaError_t e = cudaGetLastError();
	if (events) {
		cudaEventRecord(events[1], stream);
		cudaEventRecord(events[2], stream);
	}
	return e;
}
// events (may be null): recorded before, between and after the two kernels.
cudaError_t launch_ris_fast(const RisParams& p, cudaStream_t stream, int grid, cudaEvent_t* events) {
	if (events) cudaEventRecord(events[0], stream);
	ris_candidates_kernel<FastNumerics><<<grid, 128, 0, stream>>>(p);
	cudaError_t e = cudaGetLastError();
	if (e != cudaSuccess) return e;
	if (events) cudaEventRecord(events[1], stream);
	ris_shade_kernel<FastNumerics><<<grid, 128, 0, stream>>>(p);
	e = cudaGetLastError();
	if (events) cudaEventRecord(events[2], stream);
	return e;
}
}  // namespace risltc
