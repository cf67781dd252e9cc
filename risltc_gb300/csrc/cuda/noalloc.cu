// noalloc.cu - risltc_shade_noalloc: the candidate/shading kernel pair of
// risltc_shade with its scratch (the reservoir records between the two
// kernels and the error word) in a fixed, statically allocated device array
// instead of context-owned memory.
//
// Who needs it: code that may not allocate device memory while it renders -
// a plugin inside a host application that owns the device memory budget (a
// game engine or content-creation tool with its own allocator), or a frame
// loop that must not stall other streams (cudaMalloc and cudaFree
// synchronise the device).  Such a caller creates the scene once, where
// allocation is allowed, and then shades every frame through this entry
// point, which allocates nothing.
#include <atomic>
#include <cstring>
#include <cuda_runtime.h>
#include "ris_kernels.cuh"

risltc::SceneView risltc_scene_view(const risltc_scene_t* scene);
int risltc_scene_device_ordinal(const risltc_scene_t* scene);


// The scratch: reservoir records for up to RISLTC_NOALLOC_MAX_PIXEL_FRAMES
// pixel-frames, then one error word.  Every GPU that loads the library holds
// it (4 MiB + 256 bytes) until the process exits.
struct NoallocScratch {
	risltc::ReservoirRecord records[RISLTC_NOALLOC_MAX_PIXEL_FRAMES];
	uint32_t error;
};
static __device__ __align__(256) NoallocScratch g_noalloc_scratch;

namespace {

constexpr int kMaxDevices = 64;
// Device address of g_noalloc_scratch per device ordinal, resolved on the
// first call made with that device current.  Host threads that make their
// first calls at the same time each resolve the same address and store it;
// the slots are atomic so that those stores do not race.
std::atomic<NoallocScratch*> g_scratch_address[kMaxDevices];

int to_status(cudaError_t e) {
	if (e == cudaSuccess) return RISLTC_OK;
	if (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver) return RISLTC_ERROR_NO_DEVICE;
	return RISLTC_ERROR_CUDA;
}

}  // namespace

EXTERN_C int risltc_shade_noalloc(const risltc_scene_t* scene, const risltc_gbuffer_t* gbuffer,
                                  const risltc_settings_t* settings, noise_table_t* noise, uint32_t animate,
                                  uint32_t frame_count, float* out_rgb, double* accum,
                                  risltc_reservoir_t* reservoirs, void* stream) {
	if (!scene || !gbuffer || !gbuffer->planes || !settings || !noise || frame_count == 0 || gbuffer->width == 0 ||
	    gbuffer->height == 0)
		return RISLTC_ERROR_INVALID_ARGUMENT;
	if (settings->polygon_sampling_technique != sample_polygon_ltc_cp || settings->light_sampling != light_reservoir ||
	    settings->sample_count_light != 1 || settings->proposal != risltc_proposal_uniform)
		return RISLTC_ERROR_UNSUPPORTED;
	if (settings->candidate_count < 1 || settings->candidate_count > 4096 || settings->sample_count < 1 ||
	    settings->sample_count > 64 || (int) settings->mis_heuristic < 0 ||
	    settings->mis_heuristic >= mis_heuristic_count ||
	    (settings->numerics != risltc_numerics_exact && settings->numerics != risltc_numerics_fast))
		return RISLTC_ERROR_INVALID_ARGUMENT;
	const uint64_t pixel_frames = (uint64_t) gbuffer->width * gbuffer->height * frame_count;
	if (pixel_frames > RISLTC_NOALLOC_MAX_PIXEL_FRAMES) return RISLTC_ERROR_TOO_LARGE;
	int device = 0;
	cudaError_t e = cudaGetDevice(&device);
	if (e != cudaSuccess) return to_status(e);
	if (device < 0 || device >= kMaxDevices) return RISLTC_ERROR_UNSUPPORTED;
	// The scene's buffers must be in the current device's memory: the
	// kernels run there and read them.
	if (risltc_scene_device_ordinal(scene) != device) return RISLTC_ERROR_INVALID_ARGUMENT;
	NoallocScratch* scratch = g_scratch_address[device].load(std::memory_order_relaxed);
	if (!scratch) {
		void* address = nullptr;
		e = cudaGetSymbolAddress(&address, g_noalloc_scratch);
		if (e != cudaSuccess) return to_status(e);
		scratch = (NoallocScratch*) address;
		g_scratch_address[device].store(scratch, std::memory_order_relaxed);
	}
	cudaStream_t s = (cudaStream_t) stream;
	// The records are written in full before they are read; only the error
	// word has to start at zero.
	e = cudaMemsetAsync(&scratch->error, 0, sizeof(uint32_t), s);
	if (e != cudaSuccess) return to_status(e);
	risltc::RisParams r;
	memset(&r, 0, sizeof(r));
	r.scene = risltc_scene_view(scene);
	r.gbuffer = gbuffer->planes;
	r.primitive = gbuffer->primitive;
	r.width = gbuffer->width;
	r.height = gbuffer->height;
	r.candidate_count = (int) settings->candidate_count;
	r.mis_heuristic = (int) settings->mis_heuristic;
	r.sample_count = (int) settings->sample_count;
	r.mis_visibility_estimate = settings->mis_visibility_estimate;
	r.fast_atan = (int) settings->fast_atan;
	r.shadows = (int) settings->shadows;
	r.noise_seed = noise->random_seed;
	r.animate = animate;
	r.frame_count = frame_count;
	r.records = scratch->records;
	r.out_rgb = out_rgb;
	r.accum = accum;
	r.reservoirs = reservoirs;
	r.error = &scratch->error;
	int sms = 0;
	e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
	if (e != cudaSuccess) return to_status(e);
	if (sms < 1) return RISLTC_ERROR_CUDA;
	size_t blocks = ((size_t) gbuffer->width * gbuffer->height + 127) / 128;
	if (blocks > (size_t) sms * 16) blocks = (size_t) sms * 16;
	// No p_hat scratch: the candidate kernel with one thread per pixel.
	e = risltc::launch_ris(r, s, (int) blocks, (int) blocks, nullptr, settings->numerics == risltc_numerics_fast,
	                       risltc_tile_per_pixel, sms * 16);
	if (e != cudaSuccess) return to_status(e);
	uint32_t bits = 0;
	e = cudaMemcpyAsync(&bits, &scratch->error, sizeof(bits), cudaMemcpyDeviceToHost, s);
	if (e == cudaSuccess) e = cudaStreamSynchronize(s);
	if (e != cudaSuccess) return to_status(e);
	noise->random_seed += frame_count;
	if (bits & risltc::kErrorTraversalLimit) return RISLTC_ERROR_TRAVERSAL_LIMIT;
	return bits ? RISLTC_ERROR_VERTEX_COUNT : RISLTC_OK;
}
