// Instantiations compiled with --fmad=false and IEEE division and square
// root: everything that must match the CPU restatement bit for bit, plus the
// fused kernel's fast-candidate variant (its candidate loop uses hardware
// reciprocal square root; its final shading stays exact).
#include "ris_batch.cuh"

namespace risltc {
cudaError_t launch_shade(const ShadeParams& p, cudaStream_t stream, int grid, cudaEvent_t* events, bool fast) {
	if (events) cudaEventRecord(events[0], stream);
	if (fast)
		shade_kernel<FastNumerics, ExactNumerics><<<grid, kShadeThreads, 0, stream>>>(p);
	else
		shade_kernel<ExactNumerics, ExactNumerics><<<grid, kShadeThreads, 0, stream>>>(p);
	cudaError_t e = cudaGetLastError();
	if (events)
		for (int k = 1; k != RISLTC_PROFILE_PHASES + 1; ++k) cudaEventRecord(events[k], stream);
	return e;
}
cudaError_t launch_candidates_exact(const RisParams& p, cudaStream_t stream, int grid_cap, int tile) {
	if (tile == risltc_tile_32x8) return launch_candidates_binned<ExactNumerics, 32, 8>(p, stream, grid_cap);
	if (tile == risltc_tile_per_pixel) {
		ris_candidates_kernel<ExactNumerics>
		    <<<grid_for_pixels((size_t) p.width * p.height, grid_cap), 128, 0, stream>>>(p);
		return cudaGetLastError();
	}
	return launch_candidates_tile_exact(p, stream, grid_cap, tile);
}
cudaError_t launch_ris_shade(const RisParams& p, cudaStream_t stream, int grid) {
	ris_shade_kernel<ExactNumerics><<<grid, kShadeThreads, 0, stream>>>(p);
	return cudaGetLastError();
}
cudaError_t launch_proposal(const ProposalParams& p, cudaStream_t stream, int grid) {
	proposal_kernel<<<grid, 32 * kProposalWarps, proposal_smem_bytes(p.clusters.count), stream>>>(p);
	return cudaGetLastError();
}
cudaError_t launch_ris_sample(const RisParams& p, cudaStream_t stream, int grid) {
	ris_sample_kernel<ExactNumerics><<<grid, kSampleThreads, 0, stream>>>(p);
	return cudaGetLastError();
}
cudaError_t launch_shadow_sort(const RisParams& p, cudaStream_t stream, int grid) {
	light_bucket_scan_kernel<<<1, 1024, 0, stream>>>(p.light_rays, (uint32_t) p.scene.light_count, p.ray_count);
	cudaError_t e = cudaGetLastError();
	if (e != cudaSuccess) return e;
	shadow_scatter_kernel<<<grid, 128, 0, stream>>>(p);
	return cudaGetLastError();
}
cudaError_t launch_shadow_trace(const RisParams& p, cudaStream_t stream, int grid) {
	shadow_trace_kernel<ExactNumerics><<<grid, 128, 0, stream>>>(p.scene, p.rays, p.ray_count, p.hits, p.error);
	return cudaGetLastError();
}
cudaError_t launch_ris_resolve(const RisParams& p, cudaStream_t stream, int grid) {
	ris_resolve_kernel<ExactNumerics><<<grid, 128, 0, stream>>>(p);
	return cudaGetLastError();
}
cudaError_t launch_candidates_batch_exact(const RisBatch& b, cudaStream_t stream, int grid_cap, int tile) {
	if (tile == risltc_tile_32x8) return launch_candidates_batch<ExactNumerics, 32, 8>(b, stream, grid_cap);
	return launch_candidates_batch_tile_exact(b, stream, grid_cap, tile);
}
cudaError_t launch_batch_estimator(const RisBatch& b, cudaStream_t stream, int pixel_grid, int pf_grid, int ray_grid) {
	ris_sample_batch_kernel<ExactNumerics><<<pixel_grid, kSampleThreads, 0, stream>>>(b);
	cudaError_t e = cudaGetLastError();
	if (e != cudaSuccess) return e;
	light_bucket_scan_batch_kernel<<<b.count, 1024, 0, stream>>>(b);
	if ((e = cudaGetLastError()) != cudaSuccess) return e;
	shadow_scatter_batch_kernel<<<pf_grid, 128, 0, stream>>>(b);
	if ((e = cudaGetLastError()) != cudaSuccess) return e;
	shadow_trace_batch_kernel<ExactNumerics><<<ray_grid, 128, 0, stream>>>(b);
	if ((e = cudaGetLastError()) != cudaSuccess) return e;
	ris_resolve_batch_kernel<ExactNumerics><<<pixel_grid, 128, 0, stream>>>(b);
	return cudaGetLastError();
}
cudaError_t launch_trace_exact(const SceneView& s, const float4* rays, uint32_t count, uint32_t* hits, uint32_t* error,
                               cudaStream_t stream, int grid) {
	trace_shadow_kernel<ExactNumerics><<<grid, 128, 0, stream>>>(s, rays, count, hits, error);
	return cudaGetLastError();
}
}  // namespace risltc
