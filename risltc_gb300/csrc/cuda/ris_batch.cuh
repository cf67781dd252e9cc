// ris_batch.cuh - the wavefront pipeline of the default configuration run
// over a batch of frames (risltc_shade_batch) with one launch per phase: the
// candidate, sample, bucket-scan, scatter, trace and resolve kernels each
// take their work units (warp tiles, pixels, lights, pixel-frames, rays)
// from the concatenation of all items' units, so a batch of small and large
// frames fills the GPU in six launches instead of six per item.
//
// Every unit runs the single-frame kernels' body (binned_tile, sample_pixel,
// light_bucket_scan, scatter_pixel_frame, the trace loop, resolve_pixel) with
// its item's parameters, so each item's results are bit-identical to its own
// risltc_shade call.  The items' parameters travel in kernel parameter space
// (RisBatch, about 4.6 KB for 16 items) and are captured by value into a
// CUDA graph.
#pragma once
#include "ris_binned.cuh"
#include "ris_wavefront.cuh"

namespace risltc {

// Items per whole-batch launch; risltc_shade_batch runs larger batches in
// groups of this many.
constexpr int kBatchItems = 16;

struct RisBatch {
	uint32_t count;
	// Prefix sums over the items of their candidate tiles (kPixels pixels
	// each, for the tile shape of the launch), pixels and pixel-frames.
	uint32_t tile_begin[kBatchItems + 1];
	uint32_t pixel_begin[kBatchItems + 1];
	uint32_t pf_begin[kBatchItems + 1];
	// The candidate kernel's per-warp p_hat slots (for the launch's grid).
	float* p_hat_scratch;
	uint32_t* tile_cursor;  // the next warp tile over all items (zeroed before each launch)
	// Fetch cursor of the batch's concatenated ray queue (zeroed by the scan
	// kernel); the items' queue lengths are in their ray_count[0].
	uint32_t* ray_cursor;
	RisParams item[kBatchItems];
};

// The item whose units begin[k] .. begin[k + 1] - 1 hold unit u (begin has
// count + 1 entries, u < begin[count]).
RL_DEV uint32_t batch_item(const uint32_t* begin, uint32_t count, uint32_t u) {
	uint32_t lo = 0, hi = count - 1;
	while (lo < hi) {
		const uint32_t mid = (lo + hi + 1) >> 1;
		if (begin[mid] <= u)
			lo = mid;
		else
			hi = mid - 1;
	}
	return lo;
}

template <class P, int kPixels, int kChunk>
__global__ void __launch_bounds__(32 * kBinnedWarps, BinnedMinBlocks<P>::value)
ris_candidates_batch_kernel(const __grid_constant__ RisBatch b) {
	extern __shared__ __align__(16) unsigned char smem_raw[];
	using Tile = WarpTile<BinnedSuper<P>::value, kPixels, kChunk>;
	Tile& tile = reinterpret_cast<Tile*>(smem_raw)[threadIdx.x / 32];
	float* const phat = b.p_hat_scratch + (size_t) (blockIdx.x * kBinnedWarps + threadIdx.x / 32) * kPHatSlot;
	const uint32_t tiles = b.tile_begin[b.count];
	for (uint32_t u = next_warp_tile(b.tile_cursor); u < tiles; u = next_warp_tile(b.tile_cursor)) {
		const uint32_t k = batch_item(b.tile_begin, b.count, u);
		binned_tile<P, kPixels, kChunk>(b.item[k], tile, phat, u - b.tile_begin[k]);
	}
}

template <class P, int kPixels, int kChunk>
cudaError_t launch_candidates_batch(const RisBatch& b, cudaStream_t stream, int grid_cap) {
	static std::atomic<uint64_t> configured{0};
	static std::atomic<int> resident[64];
	int device = 0;
	const cudaError_t e = configure_candidate_kernel(ris_candidates_batch_kernel<P, kPixels, kChunk>,
	                                                 binned_smem_bytes<P, kPixels, kChunk>(), configured, resident, device);
	if (e != cudaSuccess) return e;
	const cudaError_t z = cudaMemsetAsync(b.tile_cursor, 0, sizeof(uint32_t), stream);
	if (z != cudaSuccess) return z;
	const size_t blocks = ((size_t) b.tile_begin[b.count] + kBinnedWarps - 1) / kBinnedWarps;
	const int grid = (int) std::max<size_t>(
	    1, std::min<size_t>(blocks, (size_t) std::min(grid_cap, resident[device & 63].load())));
	ris_candidates_batch_kernel<P, kPixels, kChunk>
	    <<<grid, 32 * kBinnedWarps, binned_smem_bytes<P, kPixels, kChunk>(), stream>>>(b);
	return cudaGetLastError();
}

template <class P>
__global__ void __launch_bounds__(kSampleThreads, RISLTC_SAMPLE_MIN_BLOCKS) ris_sample_batch_kernel(const __grid_constant__ RisBatch b) {
	__shared__ PsaPolygon poly[kSampleThreads];
	const uint32_t total = b.pixel_begin[b.count];
	for (uint32_t u = blockIdx.x * blockDim.x + threadIdx.x; u < total; u += gridDim.x * blockDim.x) {
		const uint32_t k = batch_item(b.pixel_begin, b.count, u);
		sample_pixel<P>(b.item[k], u - b.pixel_begin[k], poly[threadIdx.x]);
	}
}

// One block of 1024 threads per item.
static __global__ void __launch_bounds__(1024) light_bucket_scan_batch_kernel(const __grid_constant__ RisBatch b) {
	const RisParams& pr = b.item[blockIdx.x];
	light_bucket_scan(pr.light_rays, (uint32_t) pr.scene.light_count, pr.ray_count);
	if (blockIdx.x == 0 && threadIdx.x == 0) *b.ray_cursor = 0;
}

static __global__ void __launch_bounds__(128) shadow_scatter_batch_kernel(const __grid_constant__ RisBatch b) {
	const uint32_t total = b.pf_begin[b.count];
	for (uint32_t u = blockIdx.x * blockDim.x + threadIdx.x; u < total; u += gridDim.x * blockDim.x) {
		const uint32_t k = batch_item(b.pf_begin, b.count, u);
		scatter_pixel_frame(b.item[k], u - b.pf_begin[k]);
	}
}

// Persistent any-hit tracing of all items' queues as one queue (the items'
// queues one after another), with the lane refill of shadow_trace_kernel;
// each lane traverses its ray's item's BVH and writes its item's outcome.
template <class P>
__global__ void __launch_bounds__(128, RISLTC_TRACE_MIN_BLOCKS) shadow_trace_batch_kernel(const __grid_constant__ RisBatch b) {
	__shared__ uint32_t ray_begin[kBatchItems + 1];
	if (threadIdx.x == 0) {
		uint32_t total = 0;
		for (uint32_t k = 0; k != b.count; ++k) {
			ray_begin[k] = total;
			total += b.item[k].ray_count[0];
		}
		ray_begin[b.count] = total;
	}
	__syncthreads();
	const uint32_t n = ray_begin[b.count];
	const uint32_t lane = threadIdx.x % 32;
	uint32_t* const error = b.item[0].error;
	int32_t stack[kBvhStack];
	TraceRay r;
	SceneView s = {};
	uint8_t* hits = nullptr;
	uint32_t slot = 0;
	bool busy = false, drained = false;
	for (;;) {
		const uint32_t idle = __ballot_sync(0xffffffffu, !busy);
		if (drained && idle == 0xffffffffu) break;
		if (!drained && __popc(idle) >= RISLTC_TRACE_REFILL) {
			const int leader = __ffs(idle) - 1;
			uint32_t base = 0;
			if ((int) lane == leader) base = atomicAdd(b.ray_cursor, (uint32_t) __popc(idle));
			base = __shfl_sync(0xffffffffu, base, leader);
			drained = base + (uint32_t) __popc(idle) >= n;
			if (!busy) {
				const uint32_t g = base + (uint32_t) __popc(idle & ((1u << lane) - 1u));
				if (g < n) {
					const uint32_t k = batch_item(ray_begin, b.count, g);
					const RisParams& pr = b.item[k];
					s.pairs = pr.scene.pairs;
					s.triangles = pr.scene.triangles;
					s.triangle_count = pr.scene.triangle_count;
					hits = pr.hits;
					const ShadowRay* ray = pr.rays + (g - ray_begin[k]);
					const float4 a = __ldg(&ray->origin_slot), d = __ldg(&ray->dir_tmax);
					slot = __float_as_uint(a.w);
					const int st = trace_begin<P>(s, r, mk3(a.x, a.y, a.z), mk3(d.x, d.y, d.z), 1.0e-3f, d.w);
					if (st == kTraceContinue)
						busy = true;
					else
						hits[slot] = st == kTraceHit ? 1 : 0;
				}
			}
			continue;
		}
		if (busy) {
			const int st = trace_step<P>(s, r, stack, error);
			if (st != kTraceContinue) {
				hits[slot] = st == kTraceHit ? 1 : 0;
				busy = false;
			}
		}
	}
}

template <class P> __global__ void __launch_bounds__(128) ris_resolve_batch_kernel(const __grid_constant__ RisBatch b) {
	const uint32_t total = b.pixel_begin[b.count];
	for (uint32_t u = blockIdx.x * blockDim.x + threadIdx.x; u < total; u += gridDim.x * blockDim.x) {
		const uint32_t k = batch_item(b.pixel_begin, b.count, u);
		resolve_pixel<P>(b.item[k], u - b.pixel_begin[k]);
	}
}

// Launchers (shade_exact.cu; the candidate kernel's tile shapes as in the
// single-frame path: 32 x 8 there, the others in candidate_tiles.cu).
cudaError_t launch_candidates_batch_exact(const RisBatch& b, cudaStream_t stream, int grid_cap, int tile);
cudaError_t launch_candidates_batch_fast(const RisBatch& b, cudaStream_t stream, int grid_cap, int tile);
cudaError_t launch_candidates_batch_tile_exact(const RisBatch& b, cudaStream_t stream, int grid_cap, int tile);
cudaError_t launch_candidates_batch_tile_fast(const RisBatch& b, cudaStream_t stream, int grid_cap, int tile);
// Sample, scan, scatter, trace and resolve kernels of the batch, with the
// given grids (the scan runs one block per item).
cudaError_t launch_batch_estimator(const RisBatch& b, cudaStream_t stream, int pixel_grid, int pf_grid, int ray_grid);

}  // namespace risltc
