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
#include "shade_kernel.cuh"

namespace risltc {

struct ReservoirRecord {
	int32_t light_index;
	float w_sum;
	float p_hat;
	uint32_t seed;  // noise state after the candidate loop
};

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
	float* out_rgb;
	double* accum;
	risltc_reservoir_t* reservoirs;
	uint32_t* error;
};

// Sum of integrate_edge over the n edges of an unclipped polygon, in slot
// order (calculate_ltc with vc == n), all indices static.
template <class P> RL_DEV float ltc_integral_unclipped(const f3 (&v)[kMaxLightVertices], uint32_t n) {
	f3 nv[kMaxLightVertices];
#pragma unroll
	for (int i = 0; i != kMaxLightVertices; ++i) nv[i] = normalize<P>(v[i]);
	float result = 0.0f;
#pragma unroll
	for (int i = 0; i != kMaxLightVertices; ++i) {
		if (i < (int) n) {
			f3 next = nv[0];
#pragma unroll
			for (int j = 1; j != kMaxLightVertices; ++j)
				if (j == i + 1 && j < (int) n) next = nv[j];
			result += integrate_edge<P>(nv[i], next);
		}
	}
	return fabsf(result);
}

// Partially clipped polygon: the general clipper and integral (about 1% of
// candidates).  Returns -1 when the polygon clips to nothing.
template <class P> __device__ __noinline__ float ltc_integral_clipped(const f3* v_in, uint32_t n) {
	f3 v[kMaxPolygonVertices];
	for (int i = 0; i != kMaxLightVertices; ++i) v[i] = v_in[i];
	uint32_t vc = clip_polygon<P>(n, v);
	return vc > 0 ? calculate_ltc<P>(vc, v) : -1.0f;
}

// The LTC integral of one light transformed by m (mat4x3 * vec4(v, 1));
// clipped_away reports a polygon entirely below the horizon.
template <class P> RL_DEV float ltc_integral(const mat43& m, const Light& l, bool& clipped_away) {
	f3 t[kMaxLightVertices];
	uint32_t above = 0;
#pragma unroll
	for (int j = 0; j != kMaxLightVertices; ++j) {
		t[j] = mul_point(m, l.v[j]);
		if (j < (int) l.vertex_count && t[j].z > 0.0f) ++above;
	}
	clipped_away = above == 0;
	if (above == l.vertex_count) return ltc_integral_unclipped<P>(t, l.vertex_count);
	if (above == 0) return 0.0f;
	float r = ltc_integral_clipped<P>(t, l.vertex_count);
	clipped_away = r < 0.0f;
	return clipped_away ? 0.0f : r;
}

// Per-pixel state of the candidate loop.
struct CandidateFrame {
	f3 position;
	f3 diffuse_albedo;
	float ltc_albedo;
	mat43 w2s[2];  // world to shading space, [1]: y row negated (the side flip)
	mat43 w2c[2];  // shading_to_cosine * w2s[side]
};

// evaluate_polygonal_light_shading with SAMPLE_POLYGON_LTC_CP,
// shading_pass.frag.glsl:421-456, for one candidate light.
template <class P> RL_DEV f3 ltc_cp_candidate(const CandidateFrame& cf, const Light& l) {
	const int flip = plane_dot(cf.position, l.plane) < 0.0f ? 1 : 0;
	f3 result = splat(0.0f);
	bool clipped_away;
	float cd = ltc_integral<P>(cf.w2s[flip], l, clipped_away);
	f3 diffuse = clipped_away ? splat(0.0f) : mul(scale(cf.diffuse_albedo, cd), l.radiance);
	result = add(result, diffuse);
	float cs = ltc_integral<P>(cf.w2c[flip], l, clipped_away);
	f3 ggx = clipped_away ? splat(0.0f) : mul(splat(cs * cf.ltc_albedo), l.radiance);
	return add(result, ggx);
}

template <class P> __global__ void __launch_bounds__(128) ris_candidates_kernel(RisParams pr) {
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
			cf.w2s[0] = ltc.world_to_shading;
			cf.w2s[1] = ltc.world_to_shading;
#pragma unroll
			for (int c = 0; c != 4; ++c) cf.w2s[1].c[c].y = -cf.w2s[1].c[c].y;
			cf.w2c[0] = mul(ltc.shading_to_cosine, cf.w2s[0]);
			cf.w2c[1] = mul(ltc.shading_to_cosine, cf.w2s[1]);
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
				Light l;
				load_light(pr.scene, idx, l);
				f3 color = ltc_cp_candidate<P>(cf, l);
				float p_hat = P::sqrt(dot(color, color));
				float w = P::div(p_hat, p);
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

template <class P> __global__ void __launch_bounds__(128) ris_shade_kernel(RisParams pr) {
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
				f3 color = psa_mis_shade<P>(sp, sd, ltc, l, seed, true, true);
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

}  // namespace risltc
