// The RIS candidate kernel's tile shapes other than the default 32 x 8 and
// one thread per pixel, for one numerics mode per compilation: built twice,
// with RISLTC_TILE_FAST 0 (exact numerics: --fmad=false, IEEE division and
// square root) and 1 (fast numerics: contraction allowed).
#include "ris_batch.cuh"

namespace risltc {

#if RISLTC_TILE_FAST
using TileNumerics = FastNumerics;
cudaError_t launch_candidates_tile_fast(const RisParams& p, cudaStream_t stream, int grid_cap, int tile) {
#else
using TileNumerics = ExactNumerics;
cudaError_t launch_candidates_tile_exact(const RisParams& p, cudaStream_t stream, int grid_cap, int tile) {
#endif
	switch (tile) {
	case risltc_tile_16x8:
		return launch_candidates_binned<TileNumerics, 16, 8>(p, stream, grid_cap);
	case risltc_tile_8x8:
		return launch_candidates_binned<TileNumerics, 8, 8>(p, stream, grid_cap);
	case risltc_tile_32x4:
		return launch_candidates_binned<TileNumerics, 32, 4>(p, stream, grid_cap);
	case risltc_tile_16x4:
		return launch_candidates_binned<TileNumerics, 16, 4>(p, stream, grid_cap);
	default:
		return cudaErrorInvalidValue;
	}
}

#if RISLTC_TILE_FAST
cudaError_t launch_candidates_batch_tile_fast(const RisBatch& b, cudaStream_t stream, int grid_cap, int tile) {
#else
cudaError_t launch_candidates_batch_tile_exact(const RisBatch& b, cudaStream_t stream, int grid_cap, int tile) {
#endif
	switch (tile) {
	case risltc_tile_16x8:
		return launch_candidates_batch<TileNumerics, 16, 8>(b, stream, grid_cap);
	case risltc_tile_8x8:
		return launch_candidates_batch<TileNumerics, 8, 8>(b, stream, grid_cap);
	case risltc_tile_32x4:
		return launch_candidates_batch<TileNumerics, 32, 4>(b, stream, grid_cap);
	case risltc_tile_16x4:
		return launch_candidates_batch<TileNumerics, 16, 4>(b, stream, grid_cap);
	default:
		return cudaErrorInvalidValue;
	}
}

}  // namespace risltc
