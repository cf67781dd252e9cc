// Fast-numerics candidate kernel: hardware reciprocal square root,
// approximate division and contraction of multiply-add (--fmad=true) in the
// RIS candidate loop, whose results only weight the reservoir.
#include "ris_batch.cuh"

namespace risltc {
cudaError_t launch_candidates_fast(const RisParams& p, cudaStream_t stream, int grid_cap, int tile) {
	if (tile == risltc_tile_32x8) return launch_candidates_binned<FastNumerics, 32, 8>(p, stream, grid_cap);
	if (tile == risltc_tile_per_pixel) {
		ris_candidates_kernel<FastNumerics>
		    <<<grid_for_pixels((size_t) p.width * p.height, grid_cap), 128, 0, stream>>>(p);
		return cudaGetLastError();
	}
	return launch_candidates_tile_fast(p, stream, grid_cap, tile);
}
cudaError_t launch_candidates_batch_fast(const RisBatch& b, cudaStream_t stream, int grid_cap, int tile) {
	if (tile == risltc_tile_32x8) return launch_candidates_batch<FastNumerics, 32, 8>(b, stream, grid_cap);
	return launch_candidates_batch_tile_fast(b, stream, grid_cap, tile);
}
}  // namespace risltc
