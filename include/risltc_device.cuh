// risltc_device.cuh - the shading path's device routines under the names and
// argument meanings of the reference's GLSL, for CUDA code that composes its
// own kernels (header only; sm_103a).
//
//   GLSL routine (reference file:line)                          CUDA here
//   get_noise_accessor      noise_utility.glsl:77-84            get_noise_accessor
//   get_noise_1 / _2        noise_utility.glsl:87-95            get_noise_1 / get_noise_2
//   insert_in_reservoir     reservoir.glsl:34-41                insert_in_reservoir
//   get_ltc_coefficients    ltc_utility.glsl:56-88              get_ltc_coefficients
//   evaluate_ltc_density    ltc_utility.glsl:100-105            evaluate_ltc_density
//   clip_polygon            polygon_clipping.glsl:35-225        clip_polygon
//   calculate_ltc           polygon_sampling.glsl:523-530       calculate_ltc
//   prepare_projected_solid_angle_polygon_sampling  :545-613    same name
//   sample_projected_solid_angle_polygon            :772-828    same name
//   evaluate_brdf           brdfs.glsl:58-93                    evaluate_brdf
//
// Differences from GLSL: arrays are passed by pointer with the clipped vertex
// count, calculate_ltc sums the clipped polygon's own edges, and every
// routine takes a numerics policy (risltc::ExactNumerics or
// risltc::FastNumerics) as its template argument.
#pragma once
#include "../risltc_gb300/csrc/cuda/shade_psa.cuh"

namespace risltc {
namespace glsl {

using noise_accessor_t = uint32_t;
using projected_solid_angle_polygon_t = PsaPolygon;
using ltc_coefficients_t = Ltc;
using shading_data_t = ShadingData;

struct reservoir_t {
	float w_sum;
	int light_index;
	float sample_value;
};

RL_DEV noise_accessor_t get_noise_accessor(uint32_t px, uint32_t py, uint32_t width, uint32_t random_number_x) {
	return risltc::get_noise_accessor(px, py, width, random_number_x);
}
RL_DEV float get_noise_1(noise_accessor_t& a) { return risltc::get_noise_1(a); }
RL_DEV f2 get_noise_2(noise_accessor_t& a) { return risltc::get_noise_2(a); }

RL_DEV void initialize_reservoir(reservoir_t& r) {
	r.w_sum = 0.0f;
	r.light_index = -1;
	r.sample_value = 0.0f;
}
template <class P> RL_DEV void insert_in_reservoir(reservoir_t& r, float w, int light_index, float sample_value, float rnd) {
	r.w_sum += w;
	if (w > 0.0f && rnd < P::div(w, r.w_sum)) {
		r.light_index = light_index;
		r.sample_value = sample_value;
	}
}

template <class P>
RL_DEV ltc_coefficients_t get_ltc_coefficients(const SceneView& s, float fresnel_0, float roughness, f3 position,
                                               f3 normal, f3 outgoing) {
	return risltc::get_ltc_coefficients<P>(s, fresnel_0, roughness, position, normal, outgoing);
}
template <class P> RL_DEV float evaluate_ltc_density(const ltc_coefficients_t& ltc, f3 dir, float rcp_psa) {
	return risltc::evaluate_ltc_density<P>(ltc, dir, rcp_psa);
}
template <class P> RL_DEV uint32_t clip_polygon(uint32_t vertex_count, f3 v[kMaxPolygonVertices]) {
	return risltc::clip_polygon<P>(vertex_count, v);
}
template <class P> RL_DEV float calculate_ltc(uint32_t vertex_count, f3 v[kMaxPolygonVertices]) {
	return risltc::calculate_ltc<P>(vertex_count, v);
}
template <class P>
RL_DEV projected_solid_angle_polygon_t prepare_projected_solid_angle_polygon_sampling(uint32_t vertex_count,
                                                                                      const f3 v[kMaxPolygonVertices],
                                                                                      bool fast_atan = false) {
	projected_solid_angle_polygon_t p;
	prepare_psa<P>(p, vertex_count, v, fast_atan);
	return p;
}
template <class P>
RL_DEV f3 sample_projected_solid_angle_polygon(const projected_solid_angle_polygon_t& p, f2 random_numbers,
                                               bool fast_atan = false, bool biased = false) {
	return sample_psa<P>(p, random_numbers, fast_atan, biased);
}
template <class P> RL_DEV f3 evaluate_brdf(const shading_data_t& d, f3 incoming) {
	return risltc::evaluate_brdf<P>(d, incoming);
}

}  // namespace glsl
}  // namespace risltc
