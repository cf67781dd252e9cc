// ris_kernels.cuh - the two-kernel pipeline for the reference's default
// configuration (LTC-CP target, light_reservoir, LIGHT_SAMPLES == 1):
//
//   ris_candidates_kernel: per pixel and frame, the M-candidate RIS loop of
//     shading_pass.frag.glsl:723-736 with the LTC target of :421-456; writes
//     one 16-byte reservoir record (light, w_sum, p_hat, noise state).
//   ris_shade_kernel: per pixel and frame, the final estimator of :738-759
//     (evaluate_polygonal_light_shading_peters, :292-397) for the chosen
//     light, continuing the same noise stream, with its shadow rays.
//
// Splitting the two phases keeps each kernel's register footprint and code
// small.  Results are bit-identical to the fused kernel (same operations in
// the same order).
#pragma once
#include "proposal.cuh"
#include "shade_kernel.cuh"

namespace risltc {

struct ReservoirRecord {
	int32_t light_index;
	float w_sum;
	float p_hat;
	uint32_t seed;  // noise state after the candidate loop
};

// The warp's next tile from the launch's cursor (lane 0 takes it, the warp
// shares it): warps take tiles as they finish the previous one, so no warp
// is left with a tail of tiles while the others idle.
RL_DEV uint32_t next_warp_tile(uint32_t* cursor) {
	uint32_t t = 0;
	if (threadIdx.x % 32 == 0) t = atomicAdd(cursor, 1u);
	return __shfl_sync(0xffffffffu, t, 0);
}

struct RisParams {
	SceneView scene;
	const float* gbuffer;
	const uint32_t* primitive;
	uint32_t width, height;
	int candidate_count;
	int mis_heuristic;
	int sample_count;
	float mis_visibility_estimate;
	int fast_atan;
	int shadows;
	uint32_t noise_seed;
	uint32_t animate;
	uint32_t frame_count;
	ReservoirRecord* records;  // [frame][pixel] scratch
	// Per-warp scratch of the binned candidate kernel (one slot of 32 x 32
	// floats per warp of the grid); null selects the one-thread-per-pixel
	// candidate kernel.
	float* p_hat_scratch;
	uint32_t* tile_cursor;         // the binned candidate kernel's next warp tile (zeroed before each launch)
	uint32_t* sample_cursor;       // the sample kernel's next 32 pixels (zeroed before each launch)
	// Candidates drawn by a proposal ([frame][pixel][candidate]); null: each
	// candidate is drawn uniformly from the pixel's noise as in the reference.
	const ProposalCandidate* candidates;
	// With train_stride != 0, frame 0's candidates of the pixels with
	// i % train_stride == train_phase get their RIS weight p_hat / pdf written
	// over the pdf (the training data of the learned proposal).
	ProposalCandidate* train_candidates;
	uint32_t train_stride, train_phase;
	// Frame 0's shaded luminance (with visibility) of those pixels, from the
	// resolve kernel (may be null).
	float* train_shaded;
	// Shadow rays traced in their own pass (null: traced in ris_shade_kernel).
	struct SampleRecord* samples;  // [frame][pixel]
	struct ShadowRay* staged;      // [frame][pixel][technique], as generated
	struct ShadowRay* rays;        // the traced ones grouped by light
	uint32_t* light_rays;          // per light: ray count, then bucket cursor
	uint32_t* ray_count;           // [queue length, trace fetch cursor]
	uint8_t* hits;                 // [frame][pixel][technique] occlusion
	float* out_rgb;
	double* accum;
	risltc_reservoir_t* reservoirs;
	uint32_t* error;
};

// Sum of integrate_edge over the n edges of an unclipped polygon in slot
// order (calculate_ltc with vc == n): edges 0..n-2, then the closing edge
// n-1 -> 0.  All array indices are static.
template <class P> RL_DEV float ltc_integral_unclipped(const f3 (&v)[kMaxLightVertices], uint32_t n) {
	f3 nv[kMaxLightVertices];
#pragma unroll
	for (int i = 0; i != kMaxLightVertices; ++i) nv[i] = (i < (int) n) ? normalize<P>(v[i]) : v[i];
	f3 last = nv[2];
#pragma unroll
	for (int j = 3; j != kMaxLightVertices; ++j)
		if (j + 1 == (int) n) last = nv[j];
	float result = 0.0f;
#pragma unroll
	for (int i = 0; i + 1 != kMaxLightVertices; ++i)
		if (i + 1 < (int) n) result += integrate_edge<P>(nv[i], nv[i + 1]);
	result += integrate_edge<P>(last, nv[0]);
	return fabsf(result);
}

struct PolygonVerts {
	f3 v[kMaxLightVertices];
};

// Partially clipped polygon: the general clipper and integral (about 1% of
// candidates).  Takes the vertices by value so the caller's copy can stay in
// registers.  Returns -1 when the polygon clips to nothing.
template <class P> __device__ __noinline__ float ltc_integral_clipped(PolygonVerts in, uint32_t n) {
	f3 v[kMaxPolygonVertices];
	for (int i = 0; i != kMaxLightVertices; ++i) v[i] = in.v[i];
	uint32_t vc = clip_polygon<P>(n, v);
	return vc > 0 ? calculate_ltc<P>(vc, v) : -1.0f;
}

// The LTC integral of one light record's polygon transformed by m
// (mat4x3 * vec4(v, 1)), with the y coordinate negated when flip_y is set;
// clipped_away reports a polygon entirely below the horizon.  Negating the
// transformed y equals transforming with the y row of m negated, bit for bit
// (negation is exact and rounding symmetric): the side flip of
// shading_pass.frag.glsl:424-428.  Vertices stream from the record.
template <class P>
RL_DEV float ltc_integral(const mat43& m, bool flip_y, const float4* record, uint32_t n, bool& clipped_away) {
	PolygonVerts t;
	uint32_t above = 0;
#pragma unroll
	for (int j = 0; j != kMaxLightVertices; ++j) {
		// Slots past the count hold vertex 0, so they are always valid.
		float4 q = __ldg(record + 2 + j);
		t.v[j] = mul_point(m, mk3(q.x, q.y, q.z));
		t.v[j].y = flip_y ? -t.v[j].y : t.v[j].y;
		if (j < (int) n && t.v[j].z > 0.0f) ++above;
	}
	clipped_away = above == 0;
	if (above == n) return ltc_integral_unclipped<P>(t.v, n);
	if (above == 0) return 0.0f;
	float r = ltc_integral_clipped<P>(t, n);
	clipped_away = r < 0.0f;
	return clipped_away ? 0.0f : r;
}

// Per-pixel state of the candidate loop.
struct CandidateFrame {
	f3 position;
	f3 diffuse_albedo;
	float ltc_albedo;
	mat43 w2s;     // world to shading space
	mat43 w2c[2];  // shading_to_cosine * w2s, [1] with the y row of w2s negated
};

// evaluate_polygonal_light_shading with SAMPLE_POLYGON_LTC_CP,
// shading_pass.frag.glsl:421-456, for one candidate light record.
template <class P> RL_DEV f3 ltc_cp_candidate(const CandidateFrame& cf, const float4* record) {
	float4 head = __ldg(record), pl = __ldg(record + 1);
	const f3 radiance = mk3(head.x, head.y, head.z);
	const uint32_t n = __float_as_uint(head.w);
	const float plane[4] = {pl.x, pl.y, pl.z, pl.w};
	const int flip = plane_dot(cf.position, plane) < 0.0f ? 1 : 0;
	f3 result = splat(0.0f);
	bool clipped_away;
	float cd = ltc_integral<P>(cf.w2s, flip != 0, record, n, clipped_away);
	f3 diffuse = clipped_away ? splat(0.0f) : mul(scale(cf.diffuse_albedo, cd), radiance);
	result = add(result, diffuse);
	mat43 w2c;
#pragma unroll
	for (int c = 0; c != 4; ++c) {
		w2c.c[c].x = flip ? cf.w2c[1].c[c].x : cf.w2c[0].c[c].x;
		w2c.c[c].y = flip ? cf.w2c[1].c[c].y : cf.w2c[0].c[c].y;
		w2c.c[c].z = flip ? cf.w2c[1].c[c].z : cf.w2c[0].c[c].z;
	}
	float cs = ltc_integral<P>(w2c, false, record, n, clipped_away);
	f3 ggx = clipped_away ? splat(0.0f) : mul(splat(cs * cf.ltc_albedo), radiance);
	return add(result, ggx);
}

#ifndef RISLTC_CANDIDATE_MIN_BLOCKS
#define RISLTC_CANDIDATE_MIN_BLOCKS 5
#endif
template <class P>
__global__ void __launch_bounds__(128, RISLTC_CANDIDATE_MIN_BLOCKS) ris_candidates_kernel(RisParams pr) {
	const uint32_t np = pr.width * pr.height;
	const int n = pr.scene.light_count;
	const float p = P::rcp((float) n);
	for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < np; i += gridDim.x * blockDim.x) {
		if (pr.primitive && pr.primitive[i] == 0xffffffffu) {
			for (uint32_t f = 0; f != pr.frame_count; ++f)
				pr.records[(size_t) f * np + i] = ReservoirRecord{-1, 0.0f, 0.0f, 0u};
			continue;
		}
		const float* g = pr.gbuffer;
		const size_t snp = np;
		f3 position = mk3(g[0 * snp + i], g[1 * snp + i], g[2 * snp + i]);
		f3 normal = mk3(g[3 * snp + i], g[4 * snp + i], g[5 * snp + i]);
		f3 outgoing = mk3(g[6 * snp + i], g[7 * snp + i], g[8 * snp + i]);
		f3 fresnel_0 = mk3(g[13 * snp + i], g[14 * snp + i], g[15 * snp + i]);
		float roughness = g[16 * snp + i];
		CandidateFrame cf;
		cf.position = position;
		cf.diffuse_albedo = mk3(g[10 * snp + i], g[11 * snp + i], g[12 * snp + i]);
		{
			float fl = dot(fresnel_0, mk3(0.2126f, 0.7152f, 0.0722f));
			Ltc ltc = get_ltc_coefficients<P>(pr.scene, fl, roughness, position, normal, outgoing);
			cf.ltc_albedo = ltc.albedo;
			cf.w2s = ltc.world_to_shading;
			mat43 flipped = ltc.world_to_shading;
#pragma unroll
			for (int c = 0; c != 4; ++c) flipped.c[c].y = -flipped.c[c].y;
			cf.w2c[0] = mul(ltc.shading_to_cosine, cf.w2s);
			cf.w2c[1] = mul(ltc.shading_to_cosine, flipped);
		}
		const uint32_t x = i % pr.width, y = i / pr.width;
		for (uint32_t f = 0; f != pr.frame_count; ++f) {
			uint32_t rn_x = pr.animate ? wang_random_number((pr.noise_seed + f) * 4u) : 0u;
			uint32_t seed = get_noise_accessor(x, y, pr.width, rn_x);
			float w_sum = 0.0f, sample_value = 0.0f;
			int res_index = -1;
			for (int c = 0; c != pr.candidate_count; ++c) {
				int idx = (int) (get_noise_1(seed) * (float) n);
				idx = idx > n - 1 ? n - 1 : idx;
				float pc = p;
				if (pr.candidates) {
					const ProposalCandidate q = pr.candidates[((size_t) f * np + i) * pr.candidate_count + c];
					idx = q.light;
					pc = q.pdf;
				}
				{
					// The next candidate's index is two LCG steps ahead: start
					// pulling its record (two cache lines) into L1 now.
					uint32_t ahead = 1664525u * (1664525u * seed + 1013904223u) + 1013904223u;
					int next = (int) (__uint2float_rn(ahead) * 2.3283064365386962890625e-10f * (float) n);
					next = next > n - 1 ? n - 1 : next;
					const char* rec = (const char*) light_record(pr.scene, next);
					asm volatile("prefetch.global.L1 [%0];" ::"l"(rec));
					asm volatile("prefetch.global.L1 [%0];" ::"l"(rec + 128));
				}
				f3 color = ltc_cp_candidate<P>(cf, light_record(pr.scene, idx));
				float p_hat = P::sqrt(dot(color, color));
				float w = P::div(p_hat, pc);
				float rnd = get_noise_1(seed);
				w_sum += w;
				if (w > 0.0f && rnd < P::div(w, w_sum)) {
					res_index = idx;
					sample_value = p_hat;
				}
			}
			pr.records[(size_t) f * np + i] = ReservoirRecord{res_index, w_sum, sample_value, seed};
		}
	}
}

template <class P> __global__ void __launch_bounds__(kShadeThreads) ris_shade_kernel(RisParams pr) {
	__shared__ PsaPolygon polys[2][kShadeThreads];
	const uint32_t np = pr.width * pr.height;
	ShadeParams sp;  // the fields psa_mis_shade and polygon_visibility read
	sp.scene = pr.scene;
	sp.technique = sample_polygon_ltc_cp;
	sp.mis_heuristic = pr.mis_heuristic;
	sp.sample_count = pr.sample_count;
	sp.mis_visibility_estimate = pr.mis_visibility_estimate;
	sp.fast_atan = pr.fast_atan;
	sp.shadows = pr.shadows;
	sp.error = pr.error;
	for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < np; i += gridDim.x * blockDim.x) {
		risltc_reservoir_t* res = pr.reservoirs ? pr.reservoirs + i : nullptr;
		if (pr.primitive && pr.primitive[i] == 0xffffffffu) {
			if (res) *res = risltc_reservoir_t{-1, 0.0f, 0.0f, 0u};
			if (pr.out_rgb) {
				pr.out_rgb[3 * (size_t) i + 0] = 0.0f;
				pr.out_rgb[3 * (size_t) i + 1] = 0.0f;
				pr.out_rgb[3 * (size_t) i + 2] = 0.0f;
			}
			continue;
		}
		const float* g = pr.gbuffer;
		const size_t snp = np;
		ShadingData sd;
		sd.position = mk3(g[0 * snp + i], g[1 * snp + i], g[2 * snp + i]);
		sd.normal = mk3(g[3 * snp + i], g[4 * snp + i], g[5 * snp + i]);
		sd.outgoing = mk3(g[6 * snp + i], g[7 * snp + i], g[8 * snp + i]);
		sd.lambert_outgoing = g[9 * snp + i];
		sd.diffuse_albedo = mk3(g[10 * snp + i], g[11 * snp + i], g[12 * snp + i]);
		sd.fresnel_0 = mk3(g[13 * snp + i], g[14 * snp + i], g[15 * snp + i]);
		sd.roughness = g[16 * snp + i];
		float fl = dot(sd.fresnel_0, mk3(0.2126f, 0.7152f, 0.0722f));
		const Ltc ltc = get_ltc_coefficients<P>(pr.scene, fl, sd.roughness, sd.position, sd.normal, sd.outgoing);
		f3 sum = splat(0.0f);
		double acc[3] = {0.0, 0.0, 0.0};
		for (uint32_t f = 0; f != pr.frame_count; ++f) {
			ReservoirRecord r = pr.records[(size_t) f * np + i];
			f3 final_color = splat(0.0f);
			if (r.light_index >= 0) {
				Light l;
				load_light(pr.scene, r.light_index, l);
				uint32_t seed = r.seed;
				f3 color = psa_mis_shade<P>(sp, sd, ltc, l, seed, true, true, polys[0][threadIdx.x], polys[1][threadIdx.x]);
				float W = P::div(r.w_sum, (float) pr.candidate_count * r.p_hat);
				if (r.p_hat == 0.0f) W = 0.0f;
				f3 cw = scale(color, W);
				final_color = add(final_color, mk3(P::div(cw.x, 1.0f), P::div(cw.y, 1.0f), P::div(cw.z, 1.0f)));
			}
			if (isnan(final_color.x) || isnan(final_color.y) || isnan(final_color.z) || isinf(final_color.x) ||
			    isinf(final_color.y) || isinf(final_color.z))
				final_color = mk3(1.0f, 0.0f, 0.8f);
			if (f == 0 && res) *res = risltc_reservoir_t{r.light_index, r.w_sum, r.p_hat, 0u};
			sum = add(sum, final_color);
			acc[0] += (double) final_color.x;
			acc[1] += (double) final_color.y;
			acc[2] += (double) final_color.z;
		}
		if (pr.out_rgb) {
			f3 mean = pr.frame_count == 1 ? sum : scale(sum, 1.0f / (float) pr.frame_count);
			pr.out_rgb[3 * (size_t) i + 0] = mean.x;
			pr.out_rgb[3 * (size_t) i + 1] = mean.y;
			pr.out_rgb[3 * (size_t) i + 2] = mean.z;
		}
		if (pr.accum) {
			pr.accum[3 * (size_t) i + 0] += acc[0];
			pr.accum[3 * (size_t) i + 1] += acc[1];
			pr.accum[3 * (size_t) i + 2] += acc[2];
		}
	}
}

// Words between consecutive lights' ray counters (the sample and scatter
// kernels' atomics and the bucket scan): one 32-byte sector per counter
// spreads the millions of atomics per launch over many L2 slices (packed
// counters: ray sort + trace 1.64 ms per 1080p frame; one per sector: 1.53).
constexpr uint32_t kLightCounterStride = 8;

// Blocks of 128 threads for one thread per pixel, at most grid_cap.
inline int grid_for_pixels(size_t pixels, int grid_cap) {
	const size_t blocks = (pixels + 127) / 128;
	return (int) (blocks == 0 ? 1 : (blocks < (size_t) grid_cap ? blocks : (size_t) grid_cap));
}

// The candidate kernel with the tile shape `tile` (a risltc_tile_t); grid_cap
// is the largest grid the p_hat scratch has warp slots for.  The default and
// per-pixel shapes live with the other kernels of each numerics mode, the
// rest in their own translation units (launch_candidates_tile_*).
cudaError_t launch_candidates_exact(const RisParams& p, cudaStream_t stream, int grid_cap, int tile);
cudaError_t launch_candidates_fast(const RisParams& p, cudaStream_t stream, int grid_cap, int tile);
cudaError_t launch_candidates_tile_exact(const RisParams& p, cudaStream_t stream, int grid_cap, int tile);
cudaError_t launch_candidates_tile_fast(const RisParams& p, cudaStream_t stream, int grid_cap, int tile);
cudaError_t launch_ris_shade(const RisParams& p, cudaStream_t stream, int grid);
cudaError_t launch_ris_sample(const RisParams& p, cudaStream_t stream, int grid);
cudaError_t launch_shadow_sort(const RisParams& p, cudaStream_t stream, int grid);
cudaError_t launch_shadow_trace(const RisParams& p, cudaStream_t stream, int grid);
cudaError_t launch_ris_resolve(const RisParams& p, cudaStream_t stream, int grid);

// The candidate kernel (fast or exact numerics, tile shape `tile`, at most
// grid_cap blocks), then the shading phase (always exact): ris_shade_kernel,
// or with p.samples set the sample kernel, the shadow rays' grouping by light
// and trace, and the resolve kernel.  events (may be null) holds five events,
// recorded before, between and after the phases (the last three together for
// ris_shade_kernel).
inline cudaError_t launch_ris(const RisParams& p, cudaStream_t stream, int grid, int trace_grid, cudaEvent_t* events,
                              bool fast, int tile, int grid_cap) {
	if (events) cudaEventRecord(events[0], stream);
	cudaError_t e = fast ? launch_candidates_fast(p, stream, grid_cap, tile)
	                     : launch_candidates_exact(p, stream, grid_cap, tile);
	if (e != cudaSuccess) return e;
	if (events) cudaEventRecord(events[1], stream);
	if (p.samples) {
		e = cudaMemsetAsync(p.light_rays, 0, sizeof(uint32_t) * p.scene.light_count * kLightCounterStride, stream);
		if (e == cudaSuccess) e = cudaMemsetAsync(p.sample_cursor, 0, sizeof(uint32_t), stream);
		if (e == cudaSuccess) e = launch_ris_sample(p, stream, grid);
		if (e != cudaSuccess) return e;
		if (events) cudaEventRecord(events[2], stream);
		e = launch_shadow_sort(p, stream, grid);
		if (e != cudaSuccess) return e;
		if (events) cudaEventRecord(events[3], stream);
		e = launch_shadow_trace(p, stream, trace_grid);
		if (e != cudaSuccess) return e;
		if (events) cudaEventRecord(events[4], stream);
		e = launch_ris_resolve(p, stream, grid);
		if (events) cudaEventRecord(events[5], stream);
	} else {
		e = launch_ris_shade(p, stream, grid);
		if (events)
			for (int k = 2; k != RISLTC_PROFILE_PHASES + 1; ++k) cudaEventRecord(events[k], stream);
	}
	return e;
}

}  // namespace risltc
