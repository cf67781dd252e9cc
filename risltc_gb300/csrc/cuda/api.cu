// api.cu - the device half of the C ABI in include/risltc.h: contexts,
// scene upload, frame shading and shadow queries.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <vector>
#include <cuda_runtime.h>
#include "gbuffer.cuh"
#include "mlp.cuh"
#include "mlp_tc.cuh"
#include "mlp_train_tc.cuh"
#include "mlp_train_tc_wide.cuh"
#include "ris_batch.cuh"

// Triangles per BVH leaf before the SAH is consulted.
#ifndef RISLTC_BVH_LEAF
#define RISLTC_BVH_LEAF 4
#endif

namespace risltc {
cudaError_t launch_proposal(const ProposalParams& p, cudaStream_t stream, int grid);
cudaError_t launch_shade(const ShadeParams& p, cudaStream_t stream, int grid, cudaEvent_t* events, bool fast);
cudaError_t launch_trace_exact(const SceneView& s, const float4* rays, uint32_t count, uint32_t* hits, uint32_t* error,
                               cudaStream_t stream, int grid);
}  // namespace risltc

struct risltc_ctx_s {
	int device;
	cudaStream_t stream;
	int sm_count;
	uint32_t* d_error;
	// Staging for risltc_shade_host, grown on demand.
	float* d_gbuffer;
	uint32_t* d_primitive;
	float* d_rgb;
	size_t pixel_capacity;
	float* h_pinned_rgb;
	// Reservoir records between the candidate and shading kernels.
	risltc::ReservoirRecord* d_records;
	size_t record_capacity;
	// The binned candidate kernel's per-warp p_hat slots: one region per
	// stream that may run it at the same time (the context's stream and the
	// batch streams share regions 0..RISLTC_BATCH_STREAMS-1), each with a slot
	// per warp of the largest grid (sm_count * kCandidateBlocksPerSm blocks of
	// 4 warps).
	float* d_phat;
	int phat_regions;
	// Proposal candidates (light, pdf) per pixel-frame and candidate.
	risltc::ProposalCandidate* d_candidates;
	size_t candidate_capacity;
	// The learned proposal's logits (BF16) per pixel and cluster.
	__nv_bfloat16* d_logits;
	size_t logit_capacity;
	// The shading phase's state between its sample, shadow-ray and resolve
	// kernels: a 64-byte sample record per pixel-frame, up to two 32-byte
	// shadow rays per pixel-frame (as staged, then grouped by light), their
	// outcomes, the queue length and fetch cursor, and the per-light bucket
	// counters.
	risltc::SampleRecord* d_samples;
	risltc::ShadowRay* d_staged;
	risltc::ShadowRay* d_rays;
	uint8_t* d_hits;
	uint32_t* d_ray_count;
	uint32_t* d_light_rays;
	size_t wavefront_capacity;
	size_t light_capacity;
	size_t queue_capacity;  // ray queues (2 words each) in d_ray_count
	// risltc_shade_batch: items run on these streams, forked from and joined
	// back to the context's stream.
	cudaStream_t batch_streams[RISLTC_BATCH_STREAMS];
	cudaEvent_t batch_fork, batch_join[RISLTC_BATCH_STREAMS];
	int batch_streams_created;
	// Kernel timing: five events per shading call (before, between and after
	// the phases), up to 64 calls between queries.
	// Fault injection (risltc_ctx_inject_fault): RISLTC_FAULT_* bits, each
	// consumed by the next launch it applies to.
	uint32_t inject;
	int profiling;
	int timed_calls;
	cudaEvent_t events[64][RISLTC_PROFILE_PHASES + 1];
	// Kernels of this library launched through the context (risltc_ctx_launch_count).
	uint64_t kernel_launches;
	// Whether the last risltc_shade call queued its shadow rays (queue 0 of
	// d_ray_count then holds their number: risltc_ctx_ray_count).
	int rays_queued;
	int events_created;
};

struct risltc_scene_s {
	risltc_ctx_t* ctx;
	risltc::SceneView view;
	void* d_lights;
	void* d_ltc;
	void* d_pairs;
	void* d_triangles;
	uint32_t max_vertex_count;
	uint32_t bvh_depth;
	// Cluster structure of the lights (risltc_scene_set_clusters).
	risltc::ClusterView clusters;
	void* d_cluster_offsets;
	void* d_cluster_spans;
	void* d_cluster_lane;  // lane-major bounds, power and sizes (ClusterView::*_lane)
	void* d_light_cluster;
	void* d_cluster_bounds;
	void* d_cluster_power;
	// The learned proposal's model (risltc_scene_set_model), not owned.
	risltc_model_t* model;
};

struct risltc_model_s {
	risltc_ctx_t* ctx;
	int cluster_count;
	int parameter_count;
	float* d_params;             // FP32 parameters (risltc_model_parameter_count)
	__nv_bfloat16* d_weights;    // their BF16 copy used by the kernels
	float center[3], inv_half_extent;
	// Online training (risltc_model_set_training): gradient, Adam moments.
	float* d_grad;
	float* d_adam_m;
	float* d_adam_v;
	int training;
	float learning_rate;
	uint32_t pixel_stride;
	uint32_t steps;
	float shadowed_weight;
	uint32_t training_flags;     // RISLTC_TRAIN_*
	float* d_shaded;             // frame 0's shaded luminance of the training pixels
	size_t shaded_capacity;
};

namespace {

int cuda_status(cudaError_t e) {
	if (e == cudaSuccess) return RISLTC_OK;
	if (e == cudaErrorMemoryAllocation) return RISLTC_ERROR_OUT_OF_MEMORY;
	if (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver) return RISLTC_ERROR_NO_DEVICE;
	return RISLTC_ERROR_CUDA;
}

int grid_for(const risltc_ctx_t* ctx, size_t items) {
	// Resident CTAs per SM times SMs; the kernels are grid-stride loops.
	size_t blocks = (items + 127) / 128;
	size_t cap = (size_t) ctx->sm_count * 16;
	if (blocks > cap) blocks = cap;
	return (int) (blocks ? blocks : 1);
}

// The BVH's device layout for traversal: the root's record {bmin, reference,
// bmax, 0} (8 floats), then one 16-float record per inner node holding both
// children's records.  A reference is an inner node's record index (>= 0) or
// a leaf, -(1 + (first triangle << 3 | triangle count)) with 1..7 triangles;
// a larger leaf becomes a small subtree of leaves of at most 7 triangles, all
// with the leaf's box, so the triangles tested for a ray do not change.  Inner
// nodes are numbered depth first.  nodes: risltc_bvh_t's 8-float nodes
// {bmin, left child or first triangle, bmax, count}, children adjacent.
std::vector<float> child_pair_nodes(const float* nodes, uint32_t node_count) {
	(void) node_count;
	auto word = [&](uint32_t n, int k) {
		int32_t w;
		memcpy(&w, nodes + 8 * (size_t) n + k, sizeof(w));
		return w;
	};
	struct Pending {
		int32_t record;
		bool split;          // a range of a large leaf, else an inner node
		uint32_t node;       // the inner node, or the leaf whose box the range keeps
		uint32_t first, count;
	};
	std::vector<float> out(8);
	std::vector<Pending> stack;
	auto new_record = [&]() {
		out.resize(out.size() + 16);
		return (int32_t) ((out.size() - 8) / 16 - 1);
	};
	// The reference of a child: node's box and either node itself or the
	// triangle range [first, first + count) of the leaf node.
	auto reference = [&](uint32_t node, bool range, uint32_t first, uint32_t count) -> int32_t {
		if (!range && word(node, 7) == 0) {
			const int32_t r = new_record();
			stack.push_back({r, false, node, 0, 0});
			return r;
		}
		if (!range) {
			first = (uint32_t) word(node, 3);
			count = (uint32_t) word(node, 7);
		}
		if (count <= 7) return -(1 + (int32_t) ((first << 3) | count));
		const int32_t r = new_record();
		stack.push_back({r, true, node, first, count});
		return r;
	};
	auto put = [&](size_t at, uint32_t box_node, int32_t ref) {
		memcpy(out.data() + at, nodes + 8 * (size_t) box_node, 8 * sizeof(float));
		memcpy(out.data() + at + 3, &ref, sizeof(ref));
		out[at + 7] = 0.0f;
	};
	put(0, 0, reference(0, false, 0, 0));
	while (!stack.empty()) {
		const Pending p = stack.back();
		stack.pop_back();
		const size_t at = 8 + 16 * (size_t) p.record;
		if (p.split) {
			const uint32_t half = p.count / 2;
			const int32_t r0 = reference(p.node, true, p.first, half);
			const int32_t r1 = reference(p.node, true, p.first + half, p.count - half);
			put(at, p.node, r0);
			put(at + 8, p.node, r1);
		} else {
			const uint32_t left = (uint32_t) word(p.node, 3);
			const int32_t r0 = reference(left, false, 0, 0);
			const int32_t r1 = reference(left + 1, false, 0, 0);
			put(at, left, r0);
			put(at + 8, left + 1, r1);
		}
	}
	return out;
}

int reserve_wavefront(risltc_ctx_t* ctx, size_t pixel_frames, size_t light_count, size_t queues = 1) {
	cudaError_t e = cudaSuccess;
	if (queues > ctx->queue_capacity) {
		cudaStreamSynchronize(ctx->stream);
		cudaFree(ctx->d_ray_count);
		ctx->d_ray_count = nullptr;
		ctx->queue_capacity = 0;
		if ((e = cudaMalloc(&ctx->d_ray_count, 2 * queues * sizeof(uint32_t))) != cudaSuccess) return cuda_status(e);
		ctx->queue_capacity = queues;
	}
	if (light_count > ctx->light_capacity) {
		cudaStreamSynchronize(ctx->stream);
		cudaFree(ctx->d_light_rays);
		ctx->d_light_rays = nullptr;
		ctx->light_capacity = 0;
		if ((e = cudaMalloc(&ctx->d_light_rays, light_count * risltc::kLightCounterStride * sizeof(uint32_t))) !=
		    cudaSuccess)
			return cuda_status(e);
		ctx->light_capacity = light_count;
	}
	if (pixel_frames <= ctx->wavefront_capacity) return RISLTC_OK;
	cudaStreamSynchronize(ctx->stream);
	cudaFree(ctx->d_samples);
	cudaFree(ctx->d_staged);
	cudaFree(ctx->d_rays);
	cudaFree(ctx->d_hits);
	ctx->d_samples = nullptr;
	ctx->d_staged = nullptr;
	ctx->d_rays = nullptr;
	ctx->d_hits = nullptr;
	ctx->wavefront_capacity = 0;
	e = cudaMalloc(&ctx->d_samples, pixel_frames * sizeof(risltc::SampleRecord));
	if (e == cudaSuccess) e = cudaMalloc(&ctx->d_staged, 2 * pixel_frames * sizeof(risltc::ShadowRay));
	if (e == cudaSuccess) e = cudaMalloc(&ctx->d_rays, 2 * pixel_frames * sizeof(risltc::ShadowRay));
	if (e == cudaSuccess) e = cudaMalloc(&ctx->d_hits, 2 * pixel_frames);
	if (e != cudaSuccess) return cuda_status(e);
	ctx->wavefront_capacity = pixel_frames;
	return RISLTC_OK;
}

}  // namespace

EXTERN_C int risltc_ctx_create(risltc_ctx_t** out, int device, void* stream) {
	if (!out) return RISLTC_ERROR_INVALID_ARGUMENT;
	*out = nullptr;
	int count = 0;
	cudaError_t e = cudaGetDeviceCount(&count);
	if (e != cudaSuccess || count == 0) return RISLTC_ERROR_NO_DEVICE;
	if (device < 0 || device >= count) return RISLTC_ERROR_INVALID_ARGUMENT;
	if ((e = cudaSetDevice(device)) != cudaSuccess) return cuda_status(e);
	risltc_ctx_t* ctx = (risltc_ctx_t*) calloc(1, sizeof(risltc_ctx_t));
	if (!ctx) return RISLTC_ERROR_OUT_OF_MEMORY;
	ctx->device = device;
	ctx->stream = (cudaStream_t) stream;
	cudaDeviceGetAttribute(&ctx->sm_count, cudaDevAttrMultiProcessorCount, device);
	if ((e = cudaMalloc(&ctx->d_error, sizeof(uint32_t))) != cudaSuccess ||
	    (e = cudaMemsetAsync(ctx->d_error, 0, sizeof(uint32_t), ctx->stream)) != cudaSuccess) {
		cudaFree(ctx->d_error);
		free(ctx);
		return cuda_status(e);
	}
	*out = ctx;
	return RISLTC_OK;
}

EXTERN_C void risltc_ctx_destroy(risltc_ctx_t* ctx) {
	if (!ctx) return;
	cudaSetDevice(ctx->device);
	cudaStreamSynchronize(ctx->stream);
	cudaFree(ctx->d_error);
	cudaFree(ctx->d_gbuffer);
	cudaFree(ctx->d_primitive);
	cudaFree(ctx->d_rgb);
	cudaFreeHost(ctx->h_pinned_rgb);
	cudaFree(ctx->d_records);
	cudaFree(ctx->d_phat);
	cudaFree(ctx->d_candidates);
	cudaFree(ctx->d_logits);
	cudaFree(ctx->d_samples);
	cudaFree(ctx->d_staged);
	cudaFree(ctx->d_rays);
	cudaFree(ctx->d_hits);
	cudaFree(ctx->d_ray_count);
	cudaFree(ctx->d_light_rays);
	for (int i = 0; i < ctx->batch_streams_created; ++i) {
		cudaStreamDestroy(ctx->batch_streams[i]);
		cudaEventDestroy(ctx->batch_join[i]);
	}
	if (ctx->batch_streams_created) cudaEventDestroy(ctx->batch_fork);
	for (int i = 0; i < ctx->events_created; ++i)
		for (int k = 0; k != RISLTC_PROFILE_PHASES + 1; ++k) cudaEventDestroy(ctx->events[i][k]);
	free(ctx);
}

EXTERN_C int risltc_scene_create(risltc_ctx_t* ctx, const float* lights_std140, uint32_t light_count,
                                 uint32_t max_vertex_count, const risltc_ltc_table_t* ltc, const float* triangles,
                                 uint32_t triangle_count, risltc_scene_t** out) {
	if (!ctx || !out || !lights_std140 || light_count == 0 || !ltc || !ltc->texels0 || !ltc->texels1 ||
	    max_vertex_count < 3 || max_vertex_count > RISLTC_MAX_LIGHT_VERTEX_COUNT || (triangle_count && !triangles))
		return RISLTC_ERROR_INVALID_ARGUMENT;
	*out = nullptr;
	// Leaf references hold the first triangle in 28 bits; the candidate
	// kernel's items hold a light in 22 bits.
	if (triangle_count >= (1u << 28) || light_count >= (1u << 22)) return RISLTC_ERROR_TOO_LARGE;
	// Finite occluders keep the traversal's box tests free of NaN.
	for (size_t i = 0; i != 9 * (size_t) triangle_count; ++i)
		if (!std::isfinite(triangles[i])) return RISLTC_ERROR_NON_FINITE;
	cudaSetDevice(ctx->device);
	// Lights: 160-byte records {radiance, vertex_count | plane | 8 x {xyz, 0}},
	// then the vertex counts as bytes.
	const size_t stride = 12 + 4 * (size_t) max_vertex_count;
	std::vector<float> lights((size_t) light_count * risltc::kLightWords, 0.0f);
	for (uint32_t i = 0; i != light_count; ++i) {
		const float* s = lights_std140 + i * stride;
		float* d = lights.data() + (size_t) i * risltc::kLightWords;
		uint32_t vc;
		memcpy(&vc, s + 8, 4);
		if (vc < 3 || vc > max_vertex_count) return RISLTC_ERROR_VERTEX_COUNT;
		d[0] = s[0];
		d[1] = s[1];
		d[2] = s[2];
		memcpy(d + 3, &vc, 4);
		for (int c = 0; c != 4; ++c) d[4 + c] = s[4 + c];
		for (uint32_t v = 0; v != RISLTC_MAX_LIGHT_VERTEX_COUNT; ++v) {
			const float* src = s + 12 + 4 * (v < vc ? v : 0);
			d[8 + 4 * v + 0] = src[0];
			d[8 + 4 * v + 1] = src[1];
			d[8 + 4 * v + 2] = src[2];
			d[8 + 4 * v + 3] = 0.0f;
		}
	}
	// LTC: 8 floats per texel {m00, -m02, m11, m20, m22, albedo, 0, 0}.
	size_t texels = (size_t) ltc->roughness_count * ltc->inclination_count * ltc->fresnel_count;
	std::vector<float> ltc_dev(texels * risltc::kLtcTexelWords, 0.0f);
	for (size_t t = 0; t != texels; ++t) {
		for (int c = 0; c != 4; ++c) ltc_dev[8 * t + c] = ltc->texels0[4 * t + c];
		ltc_dev[8 * t + 4] = ltc->texels1[2 * t + 0];
		ltc_dev[8 * t + 5] = ltc->texels1[2 * t + 1];
	}
	risltc_bvh_t bvh;
	memset(&bvh, 0, sizeof(bvh));
	if (triangle_count) {
		int st = risltc_bvh_build(&bvh, triangles, triangle_count, RISLTC_BVH_LEAF);
		if (st) return st;
	}
	risltc_scene_t* scene = (risltc_scene_t*) calloc(1, sizeof(risltc_scene_t));
	if (!scene) {
		risltc_bvh_destroy(&bvh);
		return RISLTC_ERROR_OUT_OF_MEMORY;
	}
	scene->ctx = ctx;
	scene->max_vertex_count = max_vertex_count;
	scene->bvh_depth = bvh.depth;
	cudaError_t e = cudaSuccess;
	auto upload = [&](void** dst, const void* src, size_t bytes) {
		if (e != cudaSuccess || bytes == 0) return;
		e = cudaMalloc(dst, bytes);
		if (e == cudaSuccess) e = cudaMemcpy(*dst, src, bytes, cudaMemcpyHostToDevice);
	};
	{
		// After the records, one byte per light with its vertex count: the
		// candidate kernel bins its draws by vertex count from this 16 KB
		// table (16,384 lights) instead of each record's first sector.
		const size_t records = lights.size();
		lights.resize(records + (light_count + 3) / 4, 0.0f);
		uint8_t* counts = reinterpret_cast<uint8_t*>(lights.data() + records);
		for (uint32_t i = 0; i != light_count; ++i) {
			uint32_t vc;
			memcpy(&vc, lights.data() + (size_t) i * risltc::kLightWords + 3, 4);
			counts[i] = (uint8_t) vc;
		}
	}
	upload(&scene->d_lights, lights.data(), lights.size() * sizeof(float));
	upload(&scene->d_ltc, ltc_dev.data(), ltc_dev.size() * sizeof(float));
	if (triangle_count) {
		const std::vector<float> pairs = child_pair_nodes(bvh.nodes, bvh.node_count);
		upload(&scene->d_pairs, pairs.data(), pairs.size() * sizeof(float));
		upload(&scene->d_triangles, bvh.triangles, (size_t) bvh.triangle_count * 12 * sizeof(float));
	}
	risltc_bvh_destroy(&bvh);
	if (e != cudaSuccess) {
		risltc_scene_destroy(scene);
		return cuda_status(e);
	}
	risltc::SceneView& v = scene->view;
	v.lights = (const float4*) scene->d_lights;
	v.light_count = (int) light_count;
	v.ltc = (const float4*) scene->d_ltc;
	v.ltc_width = (int) ltc->roughness_count;
	v.ltc_height = (int) ltc->inclination_count;
	v.ltc_layers = (int) ltc->fresnel_count;
	v.ltc_constants[0] = ltc->constants.fresnel_index_factor;
	v.ltc_constants[1] = ltc->constants.fresnel_index_summand;
	v.ltc_constants[2] = ltc->constants.roughness_factor;
	v.ltc_constants[3] = ltc->constants.roughness_summand;
	v.ltc_constants[4] = ltc->constants.inclination_factor;
	v.ltc_constants[5] = ltc->constants.inclination_summand;
	v.pairs = (const float4*) scene->d_pairs;
	v.triangles = (const float4*) scene->d_triangles;
	v.triangle_count = (int) triangle_count;
	*out = scene;
	return RISLTC_OK;
}

// The device view of a scene, for the allocation-free entry point (noalloc.cu).
risltc::SceneView risltc_scene_view(const risltc_scene_t* scene) { return scene->view; }

// The device ordinal whose memory holds the scene's buffers (the ordinal its
// context was created with).
int risltc_scene_device_ordinal(const risltc_scene_t* scene) { return scene->ctx->device; }
// A test fakes a scene's device ordinal through these two offsets (the
// context pointer first in the scene, the ordinal first in the context).
static_assert(offsetof(risltc_scene_s, ctx) == 0, "scene layout");
static_assert(offsetof(risltc_ctx_s, device) == 0, "context layout");

EXTERN_C void risltc_scene_destroy(risltc_scene_t* scene) {
	if (!scene) return;
	cudaSetDevice(scene->ctx->device);
	cudaStreamSynchronize(scene->ctx->stream);
	cudaFree(scene->d_lights);
	cudaFree(scene->d_ltc);
	cudaFree(scene->d_pairs);
	cudaFree(scene->d_triangles);
	cudaFree(scene->d_cluster_offsets);
	cudaFree(scene->d_cluster_spans);
	cudaFree(scene->d_cluster_lane);
	cudaFree(scene->d_light_cluster);
	cudaFree(scene->d_cluster_bounds);
	cudaFree(scene->d_cluster_power);
	free(scene);
}

EXTERN_C int risltc_scene_set_clusters(risltc_scene_t* scene, const uint32_t* offsets, uint32_t cluster_count) {
	if (!scene || !offsets || cluster_count == 0 || cluster_count > (uint32_t) risltc::kMaxClusters)
		return RISLTC_ERROR_INVALID_ARGUMENT;
	const uint32_t n = (uint32_t) scene->view.light_count;
	if (offsets[0] != 0 || offsets[cluster_count] != n) return RISLTC_ERROR_INVALID_ARGUMENT;
	for (uint32_t c = 0; c != cluster_count; ++c)
		if (offsets[c + 1] < offsets[c]) return RISLTC_ERROR_INVALID_ARGUMENT;
	cudaSetDevice(scene->ctx->device);
	cudaStreamSynchronize(scene->ctx->stream);
	// The device light records {radiance, count}, plane, 8 vertex slots, as
	// std140 rows for risltc_cluster_summaries.
	std::vector<float> rec((size_t) n * risltc::kLightWords);
	cudaError_t e = cudaMemcpy(rec.data(), scene->d_lights, rec.size() * sizeof(float), cudaMemcpyDeviceToHost);
	if (e != cudaSuccess) return cuda_status(e);
	const uint32_t maxv = risltc::kMaxLightVertices;
	const size_t stride = 12 + 4 * (size_t) maxv;
	std::vector<float> std140(stride * n, 0.0f);
	for (uint32_t l = 0; l != n; ++l) {
		const float* r = &rec[(size_t) l * risltc::kLightWords];
		float* row = &std140[stride * l];
		for (int a = 0; a != 3; ++a) row[a] = r[a];
		for (int a = 0; a != 4; ++a) row[4 + a] = r[4 + a];
		memcpy(row + 8, r + 3, sizeof(float));
		for (uint32_t v = 0; v != maxv; ++v)
			for (int a = 0; a != 3; ++a) row[12 + 4 * v + a] = r[8 + 4 * v + a];
	}
	std::vector<float> bounds(4 * (size_t) cluster_count), power(cluster_count);
	int st = risltc_cluster_summaries(std140.data(), n, maxv, offsets, cluster_count, bounds.data(), power.data());
	if (st) return st;
	std::vector<uint32_t> light_cluster(n);
	std::vector<uint32_t> spans(2 * (size_t) cluster_count);
	for (uint32_t c = 0; c != cluster_count; ++c) {
		spans[2 * c] = offsets[c];
		spans[2 * c + 1] = offsets[c + 1] - offsets[c];
		for (uint32_t l = offsets[c]; l != offsets[c + 1]; ++l) light_cluster[l] = c;
	}
	// Lane-major copies: slot j * 32 + l holds cluster l * per_lane + j.
	const uint32_t per_lane = (cluster_count + 31) / 32, slots = 32 * per_lane;
	std::vector<float> lane_data(4 * (size_t) slots + 2 * (size_t) slots, 0.0f);
	float* bounds_lane = lane_data.data();
	float* power_lane = bounds_lane + 4 * (size_t) slots;
	uint32_t* size_lane = reinterpret_cast<uint32_t*>(power_lane + slots);
	for (uint32_t l = 0; l != 32; ++l) {
		for (uint32_t j = 0; j != per_lane; ++j) {
			const uint32_t c = l * per_lane + j, t = j * 32 + l;
			if (c >= cluster_count) continue;
			for (int a = 0; a != 4; ++a) bounds_lane[4 * (size_t) t + a] = bounds[4 * (size_t) c + a];
			power_lane[t] = power[c];
			size_lane[t] = offsets[c + 1] - offsets[c];
		}
	}
	cudaFree(scene->d_cluster_offsets);
	cudaFree(scene->d_cluster_spans);
	cudaFree(scene->d_cluster_lane);
	cudaFree(scene->d_light_cluster);
	cudaFree(scene->d_cluster_bounds);
	cudaFree(scene->d_cluster_power);
	scene->d_cluster_offsets = scene->d_cluster_spans = scene->d_cluster_lane = scene->d_light_cluster =
	    scene->d_cluster_bounds = scene->d_cluster_power = nullptr;
	scene->clusters = risltc::ClusterView{};
	auto upload = [&](void** dst, const void* src, size_t bytes) {
		if (e != cudaSuccess) return;
		e = cudaMalloc(dst, bytes);
		if (e == cudaSuccess) e = cudaMemcpy(*dst, src, bytes, cudaMemcpyHostToDevice);
	};
	upload(&scene->d_cluster_offsets, offsets, sizeof(uint32_t) * (cluster_count + 1));
	upload(&scene->d_cluster_spans, spans.data(), sizeof(uint32_t) * spans.size());
	upload(&scene->d_cluster_lane, lane_data.data(), sizeof(float) * lane_data.size());
	upload(&scene->d_light_cluster, light_cluster.data(), sizeof(uint32_t) * n);
	upload(&scene->d_cluster_bounds, bounds.data(), sizeof(float) * bounds.size());
	upload(&scene->d_cluster_power, power.data(), sizeof(float) * power.size());
	if (e != cudaSuccess) return cuda_status(e);
	scene->clusters.offsets = (const uint32_t*) scene->d_cluster_offsets;
	scene->clusters.spans = (const uint2*) scene->d_cluster_spans;
	scene->clusters.bounds_lane = (const float4*) scene->d_cluster_lane;
	scene->clusters.power_lane = (const float*) scene->d_cluster_lane + 4 * (size_t) slots;
	scene->clusters.size_lane = (const uint32_t*) scene->d_cluster_lane + 5 * (size_t) slots;
	scene->clusters.light_cluster = (const uint32_t*) scene->d_light_cluster;
	scene->clusters.bounds = (const float4*) scene->d_cluster_bounds;
	scene->clusters.power = (const float*) scene->d_cluster_power;
	scene->clusters.count = (int) cluster_count;
	return RISLTC_OK;
}

static int validate_settings(const risltc_settings_t* s) {
	if (!s) return RISLTC_ERROR_INVALID_ARGUMENT;
	if (s->polygon_sampling_technique != sample_polygon_ltc_cp &&
	    s->polygon_sampling_technique != sample_polygon_projected_solid_angle &&
	    s->polygon_sampling_technique != sample_polygon_projected_solid_angle_biased &&
	    s->polygon_sampling_technique != sample_polygon_area_turk)
		return RISLTC_ERROR_UNSUPPORTED;
	if ((int) s->mis_heuristic < 0 || s->mis_heuristic >= mis_heuristic_count) return RISLTC_ERROR_INVALID_ARGUMENT;
	if (s->light_sampling != light_uniform && s->light_sampling != light_reservoir) return RISLTC_ERROR_INVALID_ARGUMENT;
	if (s->candidate_count < 1 || s->candidate_count > 4096 || s->sample_count < 1 || s->sample_count > 64 ||
	    s->sample_count_light < 1 || s->sample_count_light > 64)
		return RISLTC_ERROR_INVALID_ARGUMENT;
	if (s->numerics != risltc_numerics_exact && s->numerics != risltc_numerics_fast) return RISLTC_ERROR_INVALID_ARGUMENT;
	if ((int) s->tile < 0 || s->tile >= risltc_tile_count) return RISLTC_ERROR_INVALID_ARGUMENT;
	if (s->proposal != risltc_proposal_uniform && s->proposal != risltc_proposal_clusters &&
	    s->proposal != risltc_proposal_learned)
		return RISLTC_ERROR_INVALID_ARGUMENT;
	if (s->proposal != risltc_proposal_uniform) {
		if (!(s->proposal_uniform_fraction > 0.0f && s->proposal_uniform_fraction <= 1.0f))
			return RISLTC_ERROR_INVALID_ARGUMENT;
		// Proposals feed the RIS candidates of the default configuration.
		if (s->polygon_sampling_technique != sample_polygon_ltc_cp || s->light_sampling != light_reservoir ||
		    s->sample_count_light != 1)
			return RISLTC_ERROR_UNSUPPORTED;
	}
	return RISLTC_OK;
}

namespace {

bool valid_call(const risltc_scene_t* scene, const risltc_gbuffer_t* gbuffer, const noise_table_t* noise,
                uint32_t frame_count) {
	return scene && gbuffer && gbuffer->planes && noise && frame_count != 0 && gbuffer->width != 0 &&
	       gbuffer->height != 0 && (uint64_t) gbuffer->width * gbuffer->height <= 0xffffffffull / 32;
}

bool uses_ris_pipeline(const risltc_settings_t* s) {
	return s->polygon_sampling_technique == sample_polygon_ltc_cp && s->light_sampling == light_reservoir &&
	       s->sample_count_light == 1;
}

// Shadow rays in their own pass for one sample per technique; the queue's
// hit slots (2 per pixel-frame) are 32-bit.
bool uses_ray_queue(const risltc_scene_t* scene, const risltc_settings_t* s, size_t pixel_frames) {
	return uses_ris_pipeline(s) && s->shadows && scene->view.triangle_count && s->sample_count == 1 &&
	       pixel_frames < (1ull << 31);
}

// One call's share of the context's scratch.
struct Scratch {
	risltc::ReservoirRecord* records;
	float* p_hat;
	risltc::ProposalCandidate* candidates;
	__nv_bfloat16* logits;
	risltc::SampleRecord* samples;
	risltc::ShadowRay* staged;
	risltc::ShadowRay* rays;
	uint8_t* hits;
	uint32_t* ray_count;
	uint32_t* light_rays;
};

bool uses_proposal(const risltc_settings_t* s) { return s->proposal != risltc_proposal_uniform; }

int reserve_logits(risltc_ctx_t* ctx, size_t need) {
	if (need <= ctx->logit_capacity) return RISLTC_OK;
	cudaSetDevice(ctx->device);
	cudaStreamSynchronize(ctx->stream);
	cudaFree(ctx->d_logits);
	ctx->d_logits = nullptr;
	ctx->logit_capacity = 0;
	cudaError_t e = cudaMalloc(&ctx->d_logits, need * sizeof(__nv_bfloat16));
	if (e != cudaSuccess) return cuda_status(e);
	ctx->logit_capacity = need;
	return RISLTC_OK;
}

// One Adam step (Kingma & Ba 2015, beta 0.9 / 0.999) on the model's
// accumulated gradient, which it clears (stream-ordered).
cudaError_t launch_adam(risltc_model_t* m, cudaStream_t stream) {
	m->steps += 1;
	const double b1 = 0.9, b2 = 0.999;
	risltc::mlp_adam_kernel<<<64, 256, 0, stream>>>(m->d_params, m->d_grad, m->d_adam_m, m->d_adam_v, m->d_weights,
	                                               m->parameter_count, m->cluster_count, m->learning_rate, (float) b1,
	                                               (float) b2, 1e-8f,
	                                               (float) (1.0 - std::pow(b1, (double) m->steps)),
	                                               (float) (1.0 - std::pow(b2, (double) m->steps)));
	return cudaGetLastError();
}

// One training step of the scene's model on frame 0's candidates of the
// training pixels, then an Adam update (stream-ordered).
cudaError_t launch_training(risltc_ctx_t* ctx, cudaStream_t stream, const risltc_scene_t* scene,
                            const risltc_gbuffer_t* gbuffer, const risltc::ProposalCandidate* candidates,
                            int candidate_count, uint32_t stride, uint32_t phase, const float* shaded,
                            const risltc::ReservoirRecord* records) {
	risltc_model_t* m = scene->model;
	const uint32_t np = gbuffer->width * gbuffer->height;
	const uint32_t n_train = np > phase ? (np - phase + stride - 1) / stride : 0;
	if (n_train == 0) return cudaSuccess;
	risltc::MlpTrainParams t;
	memset(&t, 0, sizeof(t));
	t.gbuffer = gbuffer->planes;
	t.width = gbuffer->width;
	t.height = gbuffer->height;
	t.params = m->d_params;
	t.grad = m->d_grad;
	t.k_count = m->cluster_count;
	for (int a = 0; a != 3; ++a) t.center[a] = m->center[a];
	t.inv_half_extent = m->inv_half_extent;
	t.offsets = scene->clusters.offsets;
	t.light_cluster = scene->clusters.light_cluster;
	t.light_count = (uint32_t) scene->view.light_count;
	t.primitive = gbuffer->primitive;
	t.candidates = candidates;
	t.candidate_count = candidate_count;
	t.stride = stride;
	t.phase = phase;
	t.inv_batch = 1.0f / (float) n_train;
	t.shaded = shaded;
	t.records = reinterpret_cast<const int4*>(records);
	t.shadowed_weight = m->shadowed_weight;
	t.weights = m->d_weights;
	t.error = ctx->d_error;
	static std::atomic<uint64_t> configured{0};
	const uint64_t bit = 1ull << (ctx->device & 63);
	if (!(configured.load() & bit)) {
		cudaError_t e = cudaFuncSetAttribute(risltc::mlp_train_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
		                                     (int) risltc::mlp_train_smem_bytes(risltc::kMaxClusters));
		if (e == cudaSuccess)
			e = cudaFuncSetAttribute(risltc::mlp_train_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
			                         (int) risltc::kTtSmemBytes);
		if (e == cudaSuccess)
			e = cudaFuncSetAttribute(risltc::mlp_train_tc_wide_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
			                         (int) risltc::kTwSmemBytes);
		if (e != cudaSuccess) return e;
		configured.fetch_or(bit);
	}
	if (m->cluster_count <= risltc::kTtMaxClusters && !(m->training_flags & RISLTC_TRAIN_CUDA_CORES)) {
		// One CTA per SM (its shared memory and all 512 tensor-memory columns).
		t.skip_issue = (ctx->inject & RISLTC_FAULT_TRAIN_TENSOR_WAIT) ? 1u : 0u;
		ctx->inject &= ~(uint32_t) RISLTC_FAULT_TRAIN_TENSOR_WAIT;
		const int blocks = (int) std::min<uint32_t>((n_train + risltc::kTcRows - 1) / risltc::kTcRows,
		                                            (uint32_t) ctx->sm_count);
		risltc::mlp_train_tc_kernel<<<blocks, risltc::kTcThreads, risltc::kTtSmemBytes, stream>>>(t);
	} else if (m->cluster_count <= risltc::kTwMaxClusters && !(m->training_flags & RISLTC_TRAIN_CUDA_CORES)) {
		// More than 256 clusters: the output layer in chunks of 128.
		t.skip_issue = (ctx->inject & RISLTC_FAULT_TRAIN_TENSOR_WAIT) ? 1u : 0u;
		ctx->inject &= ~(uint32_t) RISLTC_FAULT_TRAIN_TENSOR_WAIT;
		const int blocks = (int) std::min<uint32_t>((n_train + risltc::kTcRows - 1) / risltc::kTcRows,
		                                            (uint32_t) ctx->sm_count);
		risltc::mlp_train_tc_wide_kernel<<<blocks, risltc::kTcThreads, risltc::kTwSmemBytes, stream>>>(t);
	} else {
		// Two blocks per SM where their shared memory fits (up to about 500
		// clusters), one otherwise.
		const int blocks = (int) std::min<uint32_t>((n_train + risltc::kTrainPixels - 1) / risltc::kTrainPixels,
		                                            (uint32_t) ctx->sm_count * 2);
		risltc::mlp_train_kernel<<<blocks, risltc::kTrainThreads, risltc::mlp_train_smem_bytes(m->cluster_count),
		                           stream>>>(t);
	}
	cudaError_t e = cudaGetLastError();
	if (e == cudaSuccess) ctx->kernel_launches += 1;
	if (e != cudaSuccess || (m->training_flags & RISLTC_TRAIN_ACCUMULATE_ONLY)) return e;
	e = launch_adam(m, stream);
	if (e == cudaSuccess) ctx->kernel_launches += 1;
	return e;
}

// The model's logits for every pixel of the G-buffer into logits.
cudaError_t launch_logits(risltc_ctx_t* ctx, cudaStream_t stream, const risltc_model_t* m,
                          const risltc_gbuffer_t* gbuffer, __nv_bfloat16* logits) {
	risltc::MlpParams q;
	memset(&q, 0, sizeof(q));
	q.gbuffer = gbuffer->planes;
	q.primitive = gbuffer->primitive;
	q.width = gbuffer->width;
	q.height = gbuffer->height;
	q.weights = m->d_weights;
	q.params = m->d_params;
	q.k_count = m->cluster_count;
	for (int a = 0; a != 3; ++a) q.center[a] = m->center[a];
	q.inv_half_extent = m->inv_half_extent;
	q.logits = logits;
	q.error = ctx->d_error;
	q.skip_issue = (ctx->inject & RISLTC_FAULT_TENSOR_WAIT) ? 1u : 0u;
	ctx->inject &= ~(uint32_t) RISLTC_FAULT_TENSOR_WAIT;
	static std::atomic<uint64_t> configured{0};
	const uint64_t bit = 1ull << (ctx->device & 63);
	if (!(configured.load() & bit)) {
		cudaError_t e = cudaFuncSetAttribute(risltc::mlp_logits_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
		                                     (int) risltc::mlp_tc_smem_bytes(risltc::kMaxClusters));
		if (e != cudaSuccess) return e;
		configured.fetch_or(bit);
	}
	// At most two CTAs per SM fit in shared memory, so the two 256-column
	// tensor-memory allocations of an SM never wait for each other.
	const size_t tiles = ((size_t) gbuffer->width * gbuffer->height + risltc::kTcRows - 1) / risltc::kTcRows;
	const int grid = (int) std::min<size_t>(tiles, (size_t) ctx->sm_count * 2);
	risltc::mlp_logits_tc_kernel<<<grid, risltc::kTcThreads, risltc::mlp_tc_smem_bytes(m->cluster_count), stream>>>(q);
	const cudaError_t e = cudaGetLastError();
	if (e == cudaSuccess) ctx->kernel_launches += 1;
	return e;
}

int reserve_candidates(risltc_ctx_t* ctx, size_t need) {
	if (need <= ctx->candidate_capacity) return RISLTC_OK;
	cudaSetDevice(ctx->device);
	cudaStreamSynchronize(ctx->stream);
	cudaFree(ctx->d_candidates);
	ctx->d_candidates = nullptr;
	ctx->candidate_capacity = 0;
	cudaError_t e = cudaMalloc(&ctx->d_candidates, need * sizeof(risltc::ProposalCandidate));
	if (e != cudaSuccess) return cuda_status(e);
	ctx->candidate_capacity = need;
	return RISLTC_OK;
}

// One region: a p_hat slot per warp of the largest candidate grid, then 64
// words whose first two are the region's candidate-tile and sample cursors.
size_t phat_slot_floats(const risltc_ctx_t* ctx) {
	return (size_t) ctx->sm_count * risltc::kCandidateBlocksPerSm * risltc::kBinnedWarps * risltc::kPHatSlot;
}
size_t phat_region_floats(const risltc_ctx_t* ctx) { return phat_slot_floats(ctx) + 64; }

int reserve_phat(risltc_ctx_t* ctx, int regions) {
	if (regions <= ctx->phat_regions) return RISLTC_OK;
	cudaSetDevice(ctx->device);
	cudaStreamSynchronize(ctx->stream);
	cudaFree(ctx->d_phat);
	ctx->d_phat = nullptr;
	ctx->phat_regions = 0;
	cudaError_t e = cudaMalloc(&ctx->d_phat, sizeof(float) * phat_region_floats(ctx) * regions);
	if (e != cudaSuccess) return cuda_status(e);
	ctx->phat_regions = regions;
	return RISLTC_OK;
}

int reserve_records(risltc_ctx_t* ctx, size_t need) {
	if (need <= ctx->record_capacity) return RISLTC_OK;
	cudaSetDevice(ctx->device);
	cudaStreamSynchronize(ctx->stream);
	cudaFree(ctx->d_records);
	ctx->d_records = nullptr;
	ctx->record_capacity = 0;
	cudaError_t e = cudaMalloc(&ctx->d_records, need * sizeof(risltc::ReservoirRecord));
	if (e != cudaSuccess) return cuda_status(e);
	ctx->record_capacity = need;
	return RISLTC_OK;
}

// The parameters of the candidate/estimator kernels of one frame set of the
// default configuration (LTC-CP, reservoir, one light sample) with its
// share of the scratch: the reservoir records, p_hat slots and, with the ray
// queue, the wavefront buffers.
risltc::RisParams ris_params(const risltc_ctx_t* ctx, const Scratch& sc, const risltc_scene_t* scene,
                             const risltc_gbuffer_t* gbuffer, const risltc_settings_t* settings, uint32_t noise_seed,
                             uint32_t animate, uint32_t frame_count, float* out_rgb, double* accum,
                             risltc_reservoir_t* reservoirs, bool ray_queue) {
	risltc::RisParams r;
	memset(&r, 0, sizeof(r));
	r.scene = scene->view;
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
	r.noise_seed = noise_seed;
	r.animate = animate;
	r.frame_count = frame_count;
	r.records = sc.records;
	r.p_hat_scratch = sc.p_hat;
	r.tile_cursor = sc.p_hat ? reinterpret_cast<uint32_t*>(sc.p_hat + phat_slot_floats(ctx)) : nullptr;
	r.sample_cursor = r.tile_cursor ? r.tile_cursor + 1 : nullptr;
	if (ray_queue) {
		r.samples = sc.samples;
		r.staged = sc.staged;
		r.rays = sc.rays;
		r.light_rays = sc.light_rays;
		r.ray_count = sc.ray_count;
		r.hits = sc.hits;
	}
	r.out_rgb = out_rgb;
	r.accum = accum;
	r.reservoirs = reservoirs;
	r.error = ctx->d_error;
	return r;
}

// Enqueues one frame set on `stream` with its scratch already reserved.
int shade_one(risltc_ctx_t* ctx, cudaStream_t stream, const Scratch& sc, const risltc_scene_t* scene,
              const risltc_gbuffer_t* gbuffer, const risltc_settings_t* settings, uint32_t noise_seed,
              uint32_t animate, uint32_t frame_count, float* out_rgb, double* accum, risltc_reservoir_t* reservoirs,
              cudaEvent_t* events) {
	risltc::ShadeParams p;
	memset(&p, 0, sizeof(p));
	p.scene = scene->view;
	p.gbuffer = gbuffer->planes;
	p.primitive = gbuffer->primitive;
	p.width = gbuffer->width;
	p.height = gbuffer->height;
	p.technique = (int) settings->polygon_sampling_technique;
	p.light_sampling = (int) settings->light_sampling;
	p.mis_heuristic = (int) settings->mis_heuristic;
	p.candidate_count = (int) settings->candidate_count;
	p.sample_count = (int) settings->sample_count;
	p.light_samples = (int) settings->sample_count_light;
	p.mis_visibility_estimate = settings->mis_visibility_estimate;
	p.fast_atan = (int) settings->fast_atan;
	p.shadows = (int) settings->shadows;
	p.noise_seed = noise_seed;
	p.animate = animate;
	p.frame_count = frame_count;
	p.out_rgb = out_rgb;
	p.accum = accum;
	p.reservoirs = reservoirs;
	p.error = ctx->d_error;
	const size_t pixels = (size_t) gbuffer->width * gbuffer->height;
	const bool fast = settings->numerics == risltc_numerics_fast;
	cudaError_t e;
	if (uses_proposal(settings)) {
		risltc::ProposalParams q;
		memset(&q, 0, sizeof(q));
		q.scene = scene->view;
		q.clusters = scene->clusters;
		q.gbuffer = gbuffer->planes;
		q.primitive = gbuffer->primitive;
		q.width = gbuffer->width;
		q.height = gbuffer->height;
		q.candidate_count = (int) settings->candidate_count;
		q.noise_seed = noise_seed;
		q.animate = animate;
		q.frame_count = frame_count;
		q.uniform_fraction = settings->proposal_uniform_fraction;
		q.logits = nullptr;
		if (settings->proposal == risltc_proposal_learned) {
			e = launch_logits(ctx, stream, scene->model, gbuffer, sc.logits);
			if (e != cudaSuccess) return cuda_status(e);
			q.logits = sc.logits;
		}
		q.out = sc.candidates;
		const int warps = (int) ((pixels + risltc::kProposalWarps - 1) / risltc::kProposalWarps);
		e = risltc::launch_proposal(q, stream, std::min(warps, ctx->sm_count * 16));
		if (e != cudaSuccess) return cuda_status(e);
		ctx->kernel_launches += 1;
	}
	if (uses_ris_pipeline(settings)) {
		// The reference's default configuration: candidate and shading
		// kernels with reservoir records in between.
		risltc::RisParams r = ris_params(ctx, sc, scene, gbuffer, settings, noise_seed, animate, frame_count, out_rgb,
		                                 accum, reservoirs, uses_ray_queue(scene, settings, pixels * frame_count));
		r.candidates = uses_proposal(settings) ? sc.candidates : nullptr;
		const risltc_model_t* model = scene->model;
		const bool train = settings->proposal == risltc_proposal_learned && model && model->training;
		if (train) {
			r.train_candidates = sc.candidates;
			r.train_stride = model->pixel_stride;
			r.train_phase = noise_seed % model->pixel_stride;
			if (model->shadowed_weight > 0.0f && uses_ray_queue(scene, settings, pixels * frame_count)) {
				risltc_model_t* mm = scene->model;
				if (mm->shaded_capacity < pixels) {
					cudaFree(mm->d_shaded);
					mm->d_shaded = nullptr;
					mm->shaded_capacity = 0;
					if ((e = cudaMalloc(&mm->d_shaded, pixels * sizeof(float))) != cudaSuccess) return cuda_status(e);
					mm->shaded_capacity = pixels;
				}
				r.train_shaded = mm->d_shaded;
			}
		}
		e = risltc::launch_ris(r, stream, grid_for(ctx, pixels), grid_for(ctx, 2 * pixels * frame_count), events,
		                       fast, (int) settings->tile, ctx->sm_count * 16);
		// Candidates, then the estimator: sample, bucket scan, scatter, trace
		// and resolve kernels, or one shading kernel with inline rays.
		if (e == cudaSuccess) ctx->kernel_launches += r.samples ? 6 : 2;
		if (e == cudaSuccess && train)
			e = launch_training(ctx, stream, scene, gbuffer, sc.candidates, r.candidate_count, r.train_stride,
			                    r.train_phase, r.train_shaded, r.records);
	} else {
		e = risltc::launch_shade(p, stream, grid_for(ctx, pixels), events, fast);
		if (e == cudaSuccess) ctx->kernel_launches += 1;
	}
	return e == cudaSuccess ? RISLTC_OK : cuda_status(e);
}

}  // namespace

namespace {

int check_shade_call(const risltc_ctx_t* ctx, const risltc_scene_t* scene, const risltc_gbuffer_t* gbuffer,
                     const risltc_settings_t* settings, const noise_table_t* noise, uint32_t frame_count) {
	if (!ctx || !valid_call(scene, gbuffer, noise, frame_count)) return RISLTC_ERROR_INVALID_ARGUMENT;
	int st = validate_settings(settings);
	if (st) return st;
	if (uses_proposal(settings) && scene->clusters.count == 0) return RISLTC_ERROR_INVALID_ARGUMENT;
	if (settings->proposal == risltc_proposal_learned && !scene->model) return RISLTC_ERROR_INVALID_ARGUMENT;
	return RISLTC_OK;
}

// risltc_shade after its checks: grows the scratch and launches on the
// context's stream with the given events (may be null).
int shade_on_context(risltc_ctx_t* ctx, const risltc_scene_t* scene, const risltc_gbuffer_t* gbuffer,
                     const risltc_settings_t* settings, uint32_t noise_seed, uint32_t animate, uint32_t frame_count,
                     float* out_rgb, double* accum, risltc_reservoir_t* reservoirs, cudaEvent_t* events) {
	int st;
	const size_t pixel_frames = (size_t) gbuffer->width * gbuffer->height * frame_count;
	if (uses_proposal(settings) && (st = reserve_candidates(ctx, pixel_frames * settings->candidate_count)))
		return st;
	if (settings->proposal == risltc_proposal_learned &&
	    (st = reserve_logits(ctx, (size_t) gbuffer->width * gbuffer->height * scene->clusters.count)))
		return st;
	if (uses_ris_pipeline(settings)) {
		if ((st = reserve_records(ctx, pixel_frames))) return st;
		if ((st = reserve_phat(ctx, 1))) return st;
		if (uses_ray_queue(scene, settings, pixel_frames) &&
		    (st = reserve_wavefront(ctx, pixel_frames, scene->view.light_count)))
			return st;
	}
	const Scratch sc{ctx->d_records, ctx->d_phat, ctx->d_candidates, ctx->d_logits, ctx->d_samples, ctx->d_staged,
	                 ctx->d_rays, ctx->d_hits, ctx->d_ray_count, ctx->d_light_rays};
	st = shade_one(ctx, ctx->stream, sc, scene, gbuffer, settings, noise_seed, animate, frame_count, out_rgb, accum,
	               reservoirs, events);
	ctx->rays_queued = st == RISLTC_OK && uses_ris_pipeline(settings) && uses_ray_queue(scene, settings, pixel_frames);
	return st;
}

}  // namespace

EXTERN_C int risltc_shade(risltc_ctx_t* ctx, const risltc_scene_t* scene, const risltc_gbuffer_t* gbuffer,
                          const risltc_settings_t* settings, noise_table_t* noise, uint32_t animate,
                          uint32_t frame_count, float* out_rgb, double* accum, risltc_reservoir_t* reservoirs) {
	int st = check_shade_call(ctx, scene, gbuffer, settings, noise, frame_count);
	if (st) return st;
	cudaSetDevice(ctx->device);
	cudaEvent_t* events = nullptr;
	if (ctx->profiling && ctx->timed_calls < 64) {
		int i = ctx->timed_calls++;
		if (i >= ctx->events_created) {
			for (int k = 0; k != RISLTC_PROFILE_PHASES + 1; ++k) cudaEventCreate(&ctx->events[i][k]);
			ctx->events_created = i + 1;
		}
		events = ctx->events[i];
	}
	st = shade_on_context(ctx, scene, gbuffer, settings, noise->random_seed, animate, frame_count, out_rgb, accum,
	                      reservoirs, events);
	if (st) return st;
	noise->random_seed += frame_count;
	return RISLTC_OK;
}

namespace {

// Timing events of one shading call for the autotuner, destroyed with the
// object.
struct TuneEvents {
	cudaEvent_t e[RISLTC_PROFILE_PHASES + 1] = {};
	int created = 0;
	cudaError_t create() {
		for (; created != RISLTC_PROFILE_PHASES + 1; ++created) {
			cudaError_t r = cudaEventCreate(&e[created]);
			if (r != cudaSuccess) return r;
		}
		return cudaSuccess;
	}
	~TuneEvents() {
		for (int k = 0; k != created; ++k) cudaEventDestroy(e[k]);
	}
};

int fastest_tile(const float* ms) {
	int best = 0;
	for (int t = 1; t != risltc_tile_count; ++t)
		if (ms[t] < ms[best]) best = t;
	return best;
}

}  // namespace

EXTERN_C int risltc_autotune(risltc_ctx_t* ctx, const risltc_scene_t* scene, const risltc_gbuffer_t* gbuffer,
                             risltc_settings_t* settings, const noise_table_t* noise, uint32_t frame_count,
                             uint32_t repeats, float* ms_per_tile) {
	int st = check_shade_call(ctx, scene, gbuffer, settings, noise, frame_count);
	if (st) return st;
	if (repeats == 0 || repeats > 1000) return RISLTC_ERROR_INVALID_ARGUMENT;
	float ms[risltc_tile_count] = {};
	if (uses_ris_pipeline(settings)) {
		cudaSetDevice(ctx->device);
		TuneEvents ev;
		cudaError_t e = ev.create();
		if (e != cudaSuccess) return cuda_status(e);
		risltc_settings_t s = *settings;
		for (int t = 0; t != risltc_tile_count; ++t) {
			s.tile = (risltc_tile_t) t;
			for (uint32_t r = 0; r <= repeats; ++r) {
				st = shade_on_context(ctx, scene, gbuffer, &s, noise->random_seed, 1, frame_count, nullptr, nullptr,
				                      nullptr, ev.e);
				if (st) return st;
				if ((e = cudaEventSynchronize(ev.e[4])) != cudaSuccess) return cuda_status(e);
				float candidates = 0.0f;
				if ((e = cudaEventElapsedTime(&candidates, ev.e[0], ev.e[1])) != cudaSuccess) return cuda_status(e);
				if (r > 0) ms[t] += candidates / (float) repeats;
			}
		}
		settings->tile = (risltc_tile_t) fastest_tile(ms);
	}
	if (ms_per_tile)
		for (int t = 0; t != risltc_tile_count; ++t) ms_per_tile[t] = ms[t];
	return RISLTC_OK;
}

EXTERN_C int risltc_autotune_batch(risltc_ctx_t* ctx, risltc_batch_item_t* items, uint32_t item_count,
                                   uint32_t repeats, float* ms_per_tile) {
	if (!ctx || (!items && item_count) || repeats == 0 || repeats > 1000) return RISLTC_ERROR_INVALID_ARGUMENT;
	float ms[risltc_tile_count] = {};
	bool tiled = false;
	for (uint32_t i = 0; i != item_count; ++i) {
		if (!items[i].noise) return RISLTC_ERROR_INVALID_ARGUMENT;
		int st = validate_settings(&items[i].settings);
		if (st) return st;
		tiled = tiled || uses_ris_pipeline(&items[i].settings);
	}
	if (tiled) {
		cudaSetDevice(ctx->device);
		TuneEvents ev;
		cudaError_t e = ev.create();
		if (e != cudaSuccess) return cuda_status(e);
		std::vector<uint32_t> seeds(item_count);
		std::vector<risltc_tile_t> tiles(item_count);
		for (uint32_t i = 0; i != item_count; ++i) {
			seeds[i] = items[i].noise->random_seed;
			tiles[i] = items[i].settings.tile;
		}
		// Puts back the seeds the batch calls advanced (items may share a
		// noise table) and, on failure, the tiles.
		auto restore = [&](bool tiles_too) {
			for (uint32_t i = 0; i != item_count; ++i) {
				items[i].noise->random_seed = seeds[i];
				if (tiles_too) items[i].settings.tile = tiles[i];
			}
		};
		for (int t = 0; t != risltc_tile_count; ++t) {
			for (uint32_t i = 0; i != item_count; ++i) items[i].settings.tile = (risltc_tile_t) t;
			for (uint32_t r = 0; r <= repeats; ++r) {
				e = cudaEventRecord(ev.e[0], ctx->stream);
				int st = e == cudaSuccess ? risltc_shade_batch(ctx, items, item_count) : cuda_status(e);
				restore(false);
				if (st == RISLTC_OK && (e = cudaEventRecord(ev.e[1], ctx->stream)) != cudaSuccess) st = cuda_status(e);
				if (st == RISLTC_OK && (e = cudaEventSynchronize(ev.e[1])) != cudaSuccess) st = cuda_status(e);
				float call = 0.0f;
				if (st == RISLTC_OK && (e = cudaEventElapsedTime(&call, ev.e[0], ev.e[1])) != cudaSuccess)
					st = cuda_status(e);
				if (st) {
					restore(true);
					return st;
				}
				if (r > 0) ms[t] += call / (float) repeats;
			}
		}
		const int best = fastest_tile(ms);
		for (uint32_t i = 0; i != item_count; ++i) items[i].settings.tile = (risltc_tile_t) best;
	}
	if (ms_per_tile)
		for (int t = 0; t != risltc_tile_count; ++t) ms_per_tile[t] = ms[t];
	return RISLTC_OK;
}

namespace {

uint32_t tile_pixels(risltc_tile_t tile) {
	switch (tile) {
	case risltc_tile_16x8:
	case risltc_tile_16x4:
		return 16;
	case risltc_tile_8x8:
		return 8;
	default:
		return 32;
	}
}

// Whether every item runs the default configuration with plain RIS
// candidates and its shadow rays through the ray queue, all with the same
// numerics and binned tile shape, and each group of kBatchItems items holds
// fewer than 2^31 pixel-frames: then risltc_shade_batch runs one launch per
// phase for the whole batch.
bool batch_is_fused(const risltc_batch_item_t* items, uint32_t item_count) {
	size_t group = 0;
	for (uint32_t i = 0; i != item_count; ++i) {
		const risltc_batch_item_t& it = items[i];
		const size_t pf = (size_t) it.gbuffer.width * it.gbuffer.height * it.frame_count;
		if (!uses_ray_queue(it.scene, &it.settings, pf) || uses_proposal(&it.settings) ||
		    it.settings.numerics != items[0].settings.numerics || it.settings.tile != items[0].settings.tile ||
		    it.settings.tile == risltc_tile_per_pixel)
			return false;
		group = (i % risltc::kBatchItems == 0) ? pf : group + pf;
		if (group >= (1ull << 31)) return false;
	}
	return item_count > 0;
}

// The whole batch with one launch per phase (groups of kBatchItems items),
// on the context's stream; the scratch is reserved.  queues: the items' ray
// queues, followed by the trace's fetch cursor.
int shade_batch_fused(risltc_ctx_t* ctx, const risltc_batch_item_t* items, uint32_t item_count, size_t queues) {
	const risltc_tile_t tile = items[0].settings.tile;
	const bool fast = items[0].settings.numerics == risltc_numerics_fast;
	const uint32_t px_per_tile = tile_pixels(tile);
	size_t r_off = 0, w_off = 0, l_off = 0;
	for (uint32_t g0 = 0; g0 < item_count; g0 += risltc::kBatchItems) {
		const uint32_t gn = std::min<uint32_t>(item_count - g0, (uint32_t) risltc::kBatchItems);
		risltc::RisBatch b;
		memset(&b, 0, sizeof(b));
		b.count = gn;
		b.p_hat_scratch = ctx->d_phat;
		b.tile_cursor = reinterpret_cast<uint32_t*>(ctx->d_phat + phat_slot_floats(ctx));
		b.ray_cursor = ctx->d_ray_count + 2 * queues;
		uint32_t tiles = 0, pixels = 0, pfs = 0;
		const size_t l_begin = l_off;
		for (uint32_t k = 0; k != gn; ++k) {
			const risltc_batch_item_t& it = items[g0 + k];
			const uint32_t np = it.gbuffer.width * it.gbuffer.height;
			const uint32_t pf = np * it.frame_count;
			Scratch sc{};
			sc.records = ctx->d_records + r_off;
			sc.p_hat = ctx->d_phat;
			sc.samples = ctx->d_samples + w_off;
			sc.staged = ctx->d_staged + 2 * w_off;
			sc.rays = ctx->d_rays + 2 * w_off;
			sc.hits = ctx->d_hits + 2 * w_off;
			sc.ray_count = ctx->d_ray_count + 2 * (size_t) (g0 + k);
			sc.light_rays = ctx->d_light_rays + l_off * risltc::kLightCounterStride;
			b.item[k] = ris_params(ctx, sc, it.scene, &it.gbuffer, &it.settings, it.noise->random_seed, it.animate,
			                       it.frame_count, it.out_rgb, it.accum, it.reservoirs, true);
			b.tile_begin[k] = tiles;
			b.pixel_begin[k] = pixels;
			b.pf_begin[k] = pfs;
			tiles += (np + px_per_tile - 1) / px_per_tile;
			pixels += np;
			pfs += pf;
			r_off += pf;
			w_off += pf;
			l_off += (size_t) it.scene->view.light_count;
		}
		b.tile_begin[gn] = tiles;
		b.pixel_begin[gn] = pixels;
		b.pf_begin[gn] = pfs;
		cudaError_t e = cudaMemsetAsync(ctx->d_light_rays + l_begin * risltc::kLightCounterStride, 0,
		                                sizeof(uint32_t) * (l_off - l_begin) * risltc::kLightCounterStride, ctx->stream);
		if (e == cudaSuccess)
			e = fast ? risltc::launch_candidates_batch_fast(b, ctx->stream, ctx->sm_count * 16, (int) tile)
			         : risltc::launch_candidates_batch_exact(b, ctx->stream, ctx->sm_count * 16, (int) tile);
		if (e == cudaSuccess)
			e = risltc::launch_batch_estimator(b, ctx->stream, grid_for(ctx, pixels), grid_for(ctx, pfs),
			                                   grid_for(ctx, 2 * (size_t) pfs));
		if (e != cudaSuccess) return cuda_status(e);
		ctx->kernel_launches += 6;
	}
	for (uint32_t i = 0; i != item_count; ++i) items[i].noise->random_seed += items[i].frame_count;
	return RISLTC_OK;
}

}  // namespace

EXTERN_C int risltc_shade_batch(risltc_ctx_t* ctx, const risltc_batch_item_t* items, uint32_t item_count) {
	if (!ctx || (!items && item_count)) return RISLTC_ERROR_INVALID_ARGUMENT;
	if (item_count == 0) return RISLTC_OK;
	// Validate everything before any work; size the scratch for all items.
	size_t records = 0, wavefront = 0, lights = 0, queues = 0, candidates = 0, logits = 0;
	for (uint32_t i = 0; i != item_count; ++i) {
		const risltc_batch_item_t& it = items[i];
		if (!valid_call(it.scene, &it.gbuffer, it.noise, it.frame_count) || it.scene->ctx != ctx)
			return RISLTC_ERROR_INVALID_ARGUMENT;
		int st = validate_settings(&it.settings);
		if (st) return st;
		if (uses_proposal(&it.settings) && it.scene->clusters.count == 0) return RISLTC_ERROR_INVALID_ARGUMENT;
		if (it.settings.proposal == risltc_proposal_learned && !it.scene->model) return RISLTC_ERROR_INVALID_ARGUMENT;
		const size_t pf = (size_t) it.gbuffer.width * it.gbuffer.height * it.frame_count;
		if (uses_proposal(&it.settings)) candidates += pf * it.settings.candidate_count;
		if (it.settings.proposal == risltc_proposal_learned)
			logits += (size_t) it.gbuffer.width * it.gbuffer.height * it.scene->clusters.count;
		if (uses_ris_pipeline(&it.settings)) records += pf;
		if (uses_ray_queue(it.scene, &it.settings, pf)) {
			wavefront += pf;
			lights += (size_t) it.scene->view.light_count;
			++queues;
		}
	}
	cudaSetDevice(ctx->device);
	int st;
	if (records && (st = reserve_records(ctx, records))) return st;
	if (records && (st = reserve_phat(ctx, RISLTC_BATCH_STREAMS))) return st;
	if (candidates && (st = reserve_candidates(ctx, candidates))) return st;
	if (logits && (st = reserve_logits(ctx, logits))) return st;
	// One more queue slot than items: the whole-batch trace's fetch cursor.
	if (queues && (st = reserve_wavefront(ctx, wavefront, lights, queues + 1))) return st;
	if (batch_is_fused(items, item_count)) return shade_batch_fused(ctx, items, item_count, queues);
	cudaError_t e = cudaSuccess;
	if (!ctx->batch_streams_created) {
		e = cudaEventCreateWithFlags(&ctx->batch_fork, cudaEventDisableTiming);
		for (int k = 0; k != RISLTC_BATCH_STREAMS && e == cudaSuccess; ++k) {
			e = cudaStreamCreateWithFlags(&ctx->batch_streams[k], cudaStreamNonBlocking);
			if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ctx->batch_join[k], cudaEventDisableTiming);
			if (e == cudaSuccess) ctx->batch_streams_created = k + 1;
		}
		if (e != cudaSuccess) return cuda_status(e);
	}
	// Fork: every stream waits for the work already on the context's stream.
	const int streams = item_count < (uint32_t) RISLTC_BATCH_STREAMS ? (int) item_count : RISLTC_BATCH_STREAMS;
	if ((e = cudaEventRecord(ctx->batch_fork, ctx->stream)) != cudaSuccess) return cuda_status(e);
	for (int k = 0; k != streams; ++k)
		if ((e = cudaStreamWaitEvent(ctx->batch_streams[k], ctx->batch_fork, 0)) != cudaSuccess) return cuda_status(e);
	size_t r_off = 0, w_off = 0, l_off = 0, q_off = 0, c_off = 0, g_off = 0;
	for (uint32_t i = 0; i != item_count; ++i) {
		const risltc_batch_item_t& it = items[i];
		const size_t pf = (size_t) it.gbuffer.width * it.gbuffer.height * it.frame_count;
		Scratch sc{};
		if (uses_ris_pipeline(&it.settings)) {
			sc.records = ctx->d_records + r_off;
			sc.p_hat = ctx->d_phat + phat_region_floats(ctx) * (i % RISLTC_BATCH_STREAMS);
			r_off += pf;
		}
		if (uses_proposal(&it.settings)) {
			sc.candidates = ctx->d_candidates + c_off;
			c_off += pf * it.settings.candidate_count;
		}
		if (it.settings.proposal == risltc_proposal_learned) {
			sc.logits = ctx->d_logits + g_off;
			g_off += (size_t) it.gbuffer.width * it.gbuffer.height * it.scene->clusters.count;
		}
		if (uses_ray_queue(it.scene, &it.settings, pf)) {
			sc.samples = ctx->d_samples + w_off;
			sc.staged = ctx->d_staged + 2 * w_off;
			sc.rays = ctx->d_rays + 2 * w_off;
			sc.hits = ctx->d_hits + 2 * w_off;
			sc.ray_count = ctx->d_ray_count + 2 * q_off;
			sc.light_rays = ctx->d_light_rays + l_off * risltc::kLightCounterStride;
			w_off += pf;
			l_off += (size_t) it.scene->view.light_count;
			++q_off;
		}
		st = shade_one(ctx, ctx->batch_streams[i % RISLTC_BATCH_STREAMS], sc, it.scene, &it.gbuffer, &it.settings,
		               it.noise->random_seed, it.animate, it.frame_count, it.out_rgb, it.accum, it.reservoirs,
		               nullptr);
		if (st) return st;
	}
	// Join: the context's stream waits for every item.
	for (int k = 0; k != streams; ++k) {
		if ((e = cudaEventRecord(ctx->batch_join[k], ctx->batch_streams[k])) != cudaSuccess) return cuda_status(e);
		if ((e = cudaStreamWaitEvent(ctx->stream, ctx->batch_join[k], 0)) != cudaSuccess) return cuda_status(e);
	}
	for (uint32_t i = 0; i != item_count; ++i) items[i].noise->random_seed += items[i].frame_count;
	return RISLTC_OK;
}

EXTERN_C int risltc_ctx_reserve(risltc_ctx_t* ctx, uint32_t width, uint32_t height, uint32_t frame_count) {
	if (!ctx || width == 0 || height == 0 || frame_count == 0) return RISLTC_ERROR_INVALID_ARGUMENT;
	return reserve_records(ctx, (size_t) width * height * frame_count);
}

static int ensure_staging(risltc_ctx_t* ctx, size_t pixels) {
	if (pixels <= ctx->pixel_capacity) return RISLTC_OK;
	cudaStreamSynchronize(ctx->stream);
	cudaFree(ctx->d_gbuffer);
	cudaFree(ctx->d_primitive);
	cudaFree(ctx->d_rgb);
	ctx->d_gbuffer = nullptr;
	ctx->d_primitive = nullptr;
	ctx->d_rgb = nullptr;
	ctx->pixel_capacity = 0;
	cudaError_t e = cudaMalloc(&ctx->d_gbuffer, pixels * RISLTC_GBUFFER_PLANES * sizeof(float));
	if (e == cudaSuccess) e = cudaMalloc(&ctx->d_primitive, pixels * sizeof(uint32_t));
	if (e == cudaSuccess) e = cudaMalloc(&ctx->d_rgb, pixels * 3 * sizeof(float));
	if (e != cudaSuccess) return cuda_status(e);
	ctx->pixel_capacity = pixels;
	return RISLTC_OK;
}

EXTERN_C int risltc_shade_host(risltc_ctx_t* ctx, const risltc_scene_t* scene, uint32_t width, uint32_t height,
                               const float* gbuffer_planes, const uint32_t* primitive,
                               const risltc_settings_t* settings, noise_table_t* noise, uint32_t animate,
                               uint32_t frame_count, float* out_rgb) {
	if (!ctx || !scene || !gbuffer_planes || !out_rgb || width == 0 || height == 0) return RISLTC_ERROR_INVALID_ARGUMENT;
	cudaSetDevice(ctx->device);
	size_t pixels = (size_t) width * height;
	int st = ensure_staging(ctx, pixels);
	if (st) return st;
	cudaError_t e = cudaMemcpyAsync(ctx->d_gbuffer, gbuffer_planes, pixels * RISLTC_GBUFFER_PLANES * sizeof(float),
	                                cudaMemcpyHostToDevice, ctx->stream);
	if (e == cudaSuccess && primitive)
		e = cudaMemcpyAsync(ctx->d_primitive, primitive, pixels * sizeof(uint32_t), cudaMemcpyHostToDevice, ctx->stream);
	if (e != cudaSuccess) return cuda_status(e);
	risltc_gbuffer_t g = {width, height, ctx->d_gbuffer, primitive ? ctx->d_primitive : nullptr};
	st = risltc_shade(ctx, scene, &g, settings, noise, animate, frame_count, ctx->d_rgb, nullptr, nullptr);
	if (st) return st;
	e = cudaMemcpyAsync(out_rgb, ctx->d_rgb, pixels * 3 * sizeof(float), cudaMemcpyDeviceToHost, ctx->stream);
	if (e != cudaSuccess) return cuda_status(e);
	return risltc_ctx_check(ctx);
}

EXTERN_C int risltc_trace_shadow(risltc_ctx_t* ctx, const risltc_scene_t* scene, const float* rays, uint32_t ray_count,
                                 uint32_t* hits) {
	if (!ctx || !scene || (ray_count && (!rays || !hits))) return RISLTC_ERROR_INVALID_ARGUMENT;
	if (ray_count == 0) return RISLTC_OK;
	cudaSetDevice(ctx->device);
	cudaError_t e = risltc::launch_trace_exact(scene->view, (const float4*) rays, ray_count, hits, ctx->d_error,
	                                           ctx->stream, grid_for(ctx, ray_count));
	if (e == cudaSuccess) ctx->kernel_launches += 1;
	return cuda_status(e);
}

EXTERN_C int risltc_ctx_ray_count(risltc_ctx_t* ctx, uint32_t* rays) {
	if (!ctx || !rays) return RISLTC_ERROR_INVALID_ARGUMENT;
	*rays = 0;
	if (!ctx->rays_queued || !ctx->d_ray_count) return RISLTC_OK;
	cudaSetDevice(ctx->device);
	cudaError_t e = cudaMemcpyAsync(rays, ctx->d_ray_count, sizeof(uint32_t), cudaMemcpyDeviceToHost, ctx->stream);
	if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
	return cuda_status(e);
}

EXTERN_C int risltc_ctx_launch_count(const risltc_ctx_t* ctx, uint64_t* launches) {
	if (!ctx || !launches) return RISLTC_ERROR_INVALID_ARGUMENT;
	*launches = ctx->kernel_launches;
	return RISLTC_OK;
}

EXTERN_C int risltc_ctx_profile(risltc_ctx_t* ctx, int enable, float* phase_ms, uint32_t* calls) {
	if (!ctx) return RISLTC_ERROR_INVALID_ARGUMENT;
	cudaSetDevice(ctx->device);
	int status = RISLTC_OK;
	if (phase_ms) {
		for (int k = 0; k != RISLTC_PROFILE_PHASES; ++k) phase_ms[k] = 0.0f;
		cudaError_t e = cudaStreamSynchronize(ctx->stream);
		if (e != cudaSuccess) return cuda_status(e);
		for (int i = 0; i != ctx->timed_calls; ++i) {
			for (int k = 0; k != RISLTC_PROFILE_PHASES; ++k) {
				float ms = 0.0f;
				if (cudaEventElapsedTime(&ms, ctx->events[i][k], ctx->events[i][k + 1]) != cudaSuccess)
					status = RISLTC_ERROR_CUDA;
				phase_ms[k] += ms;
			}
		}
	}
	if (calls) *calls = (uint32_t) ctx->timed_calls;
	ctx->timed_calls = 0;
	ctx->profiling = enable;
	return status;
}

EXTERN_C int risltc_ctx_inject_fault(risltc_ctx_t* ctx, uint32_t faults) {
	if (!ctx || (faults & ~(uint32_t) (RISLTC_FAULT_TENSOR_WAIT | RISLTC_FAULT_TRAIN_TENSOR_WAIT)))
		return RISLTC_ERROR_INVALID_ARGUMENT;
	ctx->inject |= faults;
	return RISLTC_OK;
}

EXTERN_C int risltc_ctx_check(risltc_ctx_t* ctx) {
	if (!ctx) return RISLTC_ERROR_INVALID_ARGUMENT;
	cudaSetDevice(ctx->device);
	uint32_t bits = 0;
	cudaError_t e = cudaMemcpyAsync(&bits, ctx->d_error, sizeof(bits), cudaMemcpyDeviceToHost, ctx->stream);
	if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
	if (e != cudaSuccess) return cuda_status(e);
	if (bits) {
		cudaMemsetAsync(ctx->d_error, 0, sizeof(uint32_t), ctx->stream);
		cudaStreamSynchronize(ctx->stream);
		if (bits & risltc::kErrorTraversalLimit) return RISLTC_ERROR_TRAVERSAL_LIMIT;
		if (bits & risltc::kErrorTensorWait) return RISLTC_ERROR_DEVICE_TIMEOUT;
		return RISLTC_ERROR_VERTEX_COUNT;
	}
	return RISLTC_OK;
}

EXTERN_C const char* risltc_status_string(int status) {
	switch (status) {
	case RISLTC_OK: return "ok";
	case RISLTC_ERROR_INVALID_ARGUMENT: return "invalid argument";
	case RISLTC_ERROR_VERTEX_COUNT: return "light vertex count outside 3..8 (or above the scene maximum)";
	case RISLTC_ERROR_CUDA: return "CUDA error";
	case RISLTC_ERROR_TRAVERSAL_LIMIT: return "BVH traversal exceeded its iteration or stack limit";
	case RISLTC_ERROR_NON_FINITE: return "non-finite input";
	case RISLTC_ERROR_NO_DEVICE: return "no CUDA device";
	case RISLTC_ERROR_OUT_OF_MEMORY: return "out of memory";
	case RISLTC_ERROR_IO: return "file could not be read";
	case RISLTC_ERROR_UNSUPPORTED: return "unsupported setting";
	case RISLTC_ERROR_DEVICE_TIMEOUT: return "a device-side wait exceeded its limit";
	case RISLTC_ERROR_TOO_LARGE: return "frame larger than the static scratch of risltc_shade_noalloc";
	default: return "unknown status";
	}
}

// ------------------------------------------------------------ learned model --

EXTERN_C uint32_t risltc_model_parameter_count(uint32_t cluster_count) {
	return (uint32_t) risltc::mlp_layout((int) cluster_count).total;
}

static int model_upload(risltc_model_t* m, const float* host) {
	cudaSetDevice(m->ctx->device);
	cudaError_t e = cudaMemcpy(m->d_params, host, sizeof(float) * m->parameter_count, cudaMemcpyHostToDevice);
	if (e != cudaSuccess) return cuda_status(e);
	risltc::mlp_convert_kernel<<<64, 256, 0, m->ctx->stream>>>(m->d_params, m->d_weights, m->parameter_count,
	                                                           m->cluster_count);
	e = cudaGetLastError();
	if (e == cudaSuccess) e = cudaStreamSynchronize(m->ctx->stream);
	return cuda_status(e);
}

EXTERN_C int risltc_model_create(risltc_ctx_t* ctx, uint32_t cluster_count, uint64_t seed, risltc_model_t** out) {
	if (!ctx || !out || cluster_count == 0 || cluster_count > (uint32_t) risltc::kMaxClusters || cluster_count % 8)
		return RISLTC_ERROR_INVALID_ARGUMENT;
	*out = nullptr;
	risltc_model_t* m = (risltc_model_t*) calloc(1, sizeof(risltc_model_t));
	if (!m) return RISLTC_ERROR_OUT_OF_MEMORY;
	m->ctx = ctx;
	m->cluster_count = (int) cluster_count;
	m->parameter_count = (int) risltc_model_parameter_count(cluster_count);
	m->inv_half_extent = 1.0f;
	cudaSetDevice(ctx->device);
	cudaError_t e = cudaMalloc(&m->d_params, sizeof(float) * m->parameter_count);
	// The operand-layout weights; W3's padding rows stay zero.
	const size_t weight_bytes = sizeof(__nv_bfloat16) * (size_t) risltc::mlp_weight_elements((int) cluster_count);
	if (e == cudaSuccess) e = cudaMalloc(&m->d_weights, weight_bytes);
	if (e == cudaSuccess) e = cudaMemset(m->d_weights, 0, weight_bytes);
	for (float** buf : {&m->d_grad, &m->d_adam_m, &m->d_adam_v}) {
		if (e == cudaSuccess) e = cudaMalloc(buf, sizeof(float) * m->parameter_count);
		if (e == cudaSuccess) e = cudaMemset(*buf, 0, sizeof(float) * m->parameter_count);
	}
	m->learning_rate = 1e-3f;
	m->pixel_stride = 64;
	m->shadowed_weight = 0.5f;
	if (e != cudaSuccess) {
		risltc_model_destroy(m);
		return cuda_status(e);
	}
	// He-uniform weights (the output layer scaled by 0.1 so that the first
	// proposal is close to uniform), zero biases; splitmix64 for the seed.
	std::vector<float> host(m->parameter_count, 0.0f);
	const risltc::MlpLayout lay = risltc::mlp_layout(m->cluster_count);
	uint64_t state = seed;
	auto next = [&]() {
		uint64_t z = (state += 0x9E3779B97F4A7C15ull);
		z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
		z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
		z ^= z >> 31;
		return (double) (z >> 11) * (1.0 / 9007199254740992.0);
	};
	auto fill = [&](int offset, int count, int fan_in, double scale) {
		const double bound = scale * std::sqrt(6.0 / fan_in);
		for (int j = 0; j != count; ++j) host[offset + j] = (float) ((2.0 * next() - 1.0) * bound);
	};
	fill(lay.w1, risltc::kMlpHidden * risltc::kMlpFeatures, 130, 1.0);
	fill(lay.w2, risltc::kMlpHidden * risltc::kMlpHidden, risltc::kMlpHidden, 1.0);
	fill(lay.w3, m->cluster_count * risltc::kMlpHidden, risltc::kMlpHidden, 0.1);
	// The padding features (130..143) carry no weight.
	for (int o = 0; o != risltc::kMlpHidden; ++o)
		for (int f = 130; f != risltc::kMlpFeatures; ++f) host[lay.w1 + o * risltc::kMlpFeatures + f] = 0.0f;
	const int st = model_upload(m, host.data());
	if (st) {
		risltc_model_destroy(m);
		return st;
	}
	*out = m;
	return RISLTC_OK;
}

EXTERN_C void risltc_model_destroy(risltc_model_t* model) {
	if (!model) return;
	cudaSetDevice(model->ctx->device);
	cudaStreamSynchronize(model->ctx->stream);
	cudaFree(model->d_params);
	cudaFree(model->d_weights);
	cudaFree(model->d_grad);
	cudaFree(model->d_adam_m);
	cudaFree(model->d_adam_v);
	cudaFree(model->d_shaded);
	free(model);
}

EXTERN_C int risltc_model_set_params(risltc_model_t* model, const float* params) {
	if (!model || !params) return RISLTC_ERROR_INVALID_ARGUMENT;
	return model_upload(model, params);
}

EXTERN_C int risltc_model_get_params(const risltc_model_t* model, float* params) {
	if (!model || !params) return RISLTC_ERROR_INVALID_ARGUMENT;
	cudaSetDevice(model->ctx->device);
	cudaError_t e = cudaStreamSynchronize(model->ctx->stream);
	if (e == cudaSuccess)
		e = cudaMemcpy(params, model->d_params, sizeof(float) * model->parameter_count, cudaMemcpyDeviceToHost);
	return cuda_status(e);
}

EXTERN_C int risltc_model_set_input_transform(risltc_model_t* model, const float center[3], float half_extent) {
	if (!model || !center || !(half_extent > 0.0f)) return RISLTC_ERROR_INVALID_ARGUMENT;
	for (int a = 0; a != 3; ++a) model->center[a] = center[a];
	model->inv_half_extent = 1.0f / half_extent;
	return RISLTC_OK;
}

EXTERN_C int risltc_scene_set_model(risltc_scene_t* scene, risltc_model_t* model) {
	if (!scene) return RISLTC_ERROR_INVALID_ARGUMENT;
	if (model && (model->ctx != scene->ctx || model->cluster_count != scene->clusters.count))
		return RISLTC_ERROR_INVALID_ARGUMENT;
	scene->model = model;
	return RISLTC_OK;
}

EXTERN_C int risltc_model_logits(risltc_ctx_t* ctx, const risltc_model_t* model, const risltc_gbuffer_t* gbuffer,
                                 float* logits) {
	if (!ctx || !model || !gbuffer || !gbuffer->planes || !logits || model->ctx != ctx || gbuffer->width == 0 ||
	    gbuffer->height == 0)
		return RISLTC_ERROR_INVALID_ARGUMENT;
	const size_t count = (size_t) gbuffer->width * gbuffer->height * model->cluster_count;
	int st = reserve_logits(ctx, count);
	if (st) return st;
	cudaError_t e = launch_logits(ctx, ctx->stream, model, gbuffer, ctx->d_logits);
	if (e == cudaSuccess) {
		risltc::bf16_to_f32_kernel<<<256, 256, 0, ctx->stream>>>(ctx->d_logits, logits, count);
		e = cudaGetLastError();
	}
	return cuda_status(e);
}

EXTERN_C int risltc_model_set_training(risltc_model_t* model, int enable, float learning_rate, uint32_t pixel_stride) {
	if (!model || !(learning_rate > 0.0f) || pixel_stride == 0) return RISLTC_ERROR_INVALID_ARGUMENT;
	model->training = enable != 0;
	model->learning_rate = learning_rate;
	model->pixel_stride = pixel_stride;
	return RISLTC_OK;
}

EXTERN_C int risltc_model_set_target_mix(risltc_model_t* model, float shadowed_weight) {
	if (!model || !(shadowed_weight >= 0.0f && shadowed_weight <= 1.0f)) return RISLTC_ERROR_INVALID_ARGUMENT;
	model->shadowed_weight = shadowed_weight;
	return RISLTC_OK;
}

EXTERN_C int risltc_model_set_training_flags(risltc_model_t* model, uint32_t flags) {
	if (!model || (flags & ~(uint32_t) (RISLTC_TRAIN_CUDA_CORES | RISLTC_TRAIN_ACCUMULATE_ONLY)))
		return RISLTC_ERROR_INVALID_ARGUMENT;
	model->training_flags = flags;
	return RISLTC_OK;
}

EXTERN_C int risltc_model_get_gradient(risltc_model_t* model, float* gradient, int clear) {
	if (!model || !gradient) return RISLTC_ERROR_INVALID_ARGUMENT;
	cudaSetDevice(model->ctx->device);
	cudaError_t e = cudaStreamSynchronize(model->ctx->stream);
	if (e == cudaSuccess)
		e = cudaMemcpy(gradient, model->d_grad, sizeof(float) * model->parameter_count, cudaMemcpyDeviceToHost);
	if (e == cudaSuccess && clear) e = cudaMemset(model->d_grad, 0, sizeof(float) * model->parameter_count);
	return cuda_status(e);
}

EXTERN_C int risltc_model_apply_update(risltc_model_t* model) {
	if (!model) return RISLTC_ERROR_INVALID_ARGUMENT;
	cudaSetDevice(model->ctx->device);
	const cudaError_t e = launch_adam(model, model->ctx->stream);
	if (e == cudaSuccess) model->ctx->kernel_launches += 1;
	return cuda_status(e);
}

static_assert(sizeof(risltc_candidate_t) == sizeof(risltc::ProposalCandidate) &&
                  offsetof(risltc_candidate_t, weight) == offsetof(risltc::ProposalCandidate, pdf),
              "candidate layout");
static_assert(sizeof(risltc_reservoir_t) == sizeof(risltc::ReservoirRecord), "reservoir layout");

EXTERN_C int risltc_model_train(risltc_ctx_t* ctx, const risltc_scene_t* scene, const risltc_gbuffer_t* gbuffer,
                                const risltc_candidate_t* candidates, uint32_t candidate_count, uint32_t stride,
                                uint32_t phase, const float* shaded, const risltc_reservoir_t* reservoirs) {
	if (!ctx || !scene || scene->ctx != ctx || !scene->model || !gbuffer || !gbuffer->planes || !candidates ||
	    gbuffer->width == 0 || gbuffer->height == 0 || candidate_count == 0 || candidate_count > 4096 ||
	    stride == 0 || phase >= stride || (shaded && !reservoirs))
		return RISLTC_ERROR_INVALID_ARGUMENT;
	if (scene->clusters.count != scene->model->cluster_count) return RISLTC_ERROR_INVALID_ARGUMENT;
	if ((uint64_t) gbuffer->width * gbuffer->height >= (1ull << 31)) return RISLTC_ERROR_TOO_LARGE;
	cudaSetDevice(ctx->device);
	return cuda_status(launch_training(ctx, ctx->stream, scene, gbuffer,
	                                   reinterpret_cast<const risltc::ProposalCandidate*>(candidates),
	                                   (int) candidate_count, stride, phase, shaded,
	                                   reinterpret_cast<const risltc::ReservoirRecord*>(reservoirs)));
}

// ------------------------------------------------------------- G-buffers --

EXTERN_C int risltc_gbuffer_heightfield(risltc_ctx_t* ctx, const risltc_heightfield_t* hf, uint32_t width,
                                        uint32_t height, float* planes, uint32_t* primitive) {
	if (!ctx || !hf || !planes || width == 0 || height == 0 || hf->wave_count > RISLTC_MAX_WAVES ||
	    !(hf->fov_y > 0.0f && hf->fov_y < 3.1f) || (uint64_t) width * height > 0xffffffffull / 32)
		return RISLTC_ERROR_INVALID_ARGUMENT;
	risltc::HeightfieldParams p;
	memset(&p, 0, sizeof(p));
	// Camera basis in double: forward towards the origin, right, up.
	const double c[3] = {hf->camera[0], hf->camera[1], hf->camera[2]};
	const double len = std::sqrt(c[0] * c[0] + c[1] * c[1] + c[2] * c[2]);
	if (!(len > 0.0)) return RISLTC_ERROR_INVALID_ARGUMENT;
	const double f[3] = {-c[0] / len, -c[1] / len, -c[2] / len};
	double r[3] = {f[1], -f[0], 0.0};  // cross(f, z)
	const double rl = std::sqrt(r[0] * r[0] + r[1] * r[1]);
	if (!(rl > 0.0)) return RISLTC_ERROR_INVALID_ARGUMENT;
	for (double& x : r) x /= rl;
	const double u[3] = {r[1] * f[2] - r[2] * f[1], r[2] * f[0] - r[0] * f[2], r[0] * f[1] - r[1] * f[0]};
	for (int a = 0; a != 3; ++a) {
		p.camera[a] = hf->camera[a];
		p.forward[a] = (float) f[a];
		p.right[a] = (float) r[a];
		p.up[a] = (float) u[a];
	}
	const double th = std::tan(0.5 * hf->fov_y);
	p.tan_half_y = (float) th;
	p.tan_half_x = (float) (th * width / height);
	p.wave_count = (int) hf->wave_count;
	double hmax = 0.0;
	for (uint32_t w = 0; w != hf->wave_count; ++w) {
		for (int k = 0; k != 4; ++k) p.waves[w][k] = hf->waves[w][k];
		hmax += std::fabs(hf->waves[w][0]);
	}
	p.max_height = (float) hmax;
	p.material_seed = hf->material_seed;
	p.roughness_min = hf->roughness_min;
	p.roughness_max = hf->roughness_max;
	p.albedo_min = hf->albedo_min;
	p.albedo_max = hf->albedo_max;
	p.fresnel_0 = hf->fresnel_0;
	p.width = width;
	p.height = height;
	p.planes = planes;
	p.primitive = primitive;
	cudaSetDevice(ctx->device);
	risltc::heightfield_gbuffer_kernel<<<grid_for(ctx, (size_t) width * height), 128, 0, ctx->stream>>>(p);
	const cudaError_t e = cudaGetLastError();
	if (e == cudaSuccess) ctx->kernel_launches += 1;
	return cuda_status(e);
}
