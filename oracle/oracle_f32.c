/* FP32 instantiation of the oracle: the reference's own precision.
   TEST INFRASTRUCTURE (see oracle.h). */
#include <math.h>
#include "../include/risltc_math.h"

#define R float
#define RC(x) x##f
#define R_FMA(a, b, c) fmaf((a), (b), (c))
#define R_SQRT(x) sqrtf(x)
#define R_ATAN(x) rl_atanf(x)
#define R_ACOS(x) rl_acosf(x)
#define R_SINCOS(x, s, c) rl_sincosf((x), (s), (c))
#define R_FLOOR(x) floorf(x)
#define R_SIGNBIT(x) (signbit(x) != 0)
#define R_ISINF(x) (isinf(x) != 0)
#define R_INF INFINITY
/* Flip every exponent bit (polygon_sampling.glsl:626). */
#define R_EXPONENT_FLIP(x) rl_u2f(rl_f2u(x) ^ 0x7F800000u)
#define ORACLE_SUFFIX _f32
#define ORACLE_OUT_T float
#include "oracle_core.h"

/* Internal routines exported for known-answer tests. */
uint32_t oracle_f32_clip_polygon(uint32_t n, float* xyz, uint32_t max_polygon_vertex_count, int reference_limits) {
	vec3_t v[OR_MAXP];
	for (uint32_t i = 0; i != max_polygon_vertex_count; ++i) v[i] = V3(xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2]);
	uint32_t vc = clip_polygon(n, v, max_polygon_vertex_count, reference_limits);
	for (uint32_t i = 0; i != max_polygon_vertex_count; ++i) {
		xyz[3 * i] = v[i].x;
		xyz[3 * i + 1] = v[i].y;
		xyz[3 * i + 2] = v[i].z;
	}
	return vc;
}
float oracle_f32_calculate_ltc(uint32_t vc, const float* xyz) {
	vec3_t v[OR_MAXP];
	for (uint32_t i = 0; i != vc; ++i) v[i] = V3(xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2]);
	return calculate_ltc(vc, v, vc, 0);
}
/* Prepares PSA sampling of a clipped polygon (first vertex not repeated) and
   draws count samples from the given random pairs; returns the polygon's
   projected solid angle. */
float oracle_f32_psa_sample(uint32_t vc, const float* xyz, uint32_t count, const float* rnd, float* out_dirs,
                            float* out_errors) {
	vec3_t v[OR_MAXP + 1];
	for (uint32_t i = 0; i != vc; ++i) v[i] = V3(xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2]);
	v[vc] = v[0];
	projected_solid_angle_polygon_t p;
	g_oracle_fast_atan = 0;
	g_oracle_biased_psa = 0;
	/* The slot count the routines wrap at: vc + 1 (the first vertex
	   repeated), at most the struct's OR_MAXP slots; a polygon that fills
	   them all (an 8-gon clipped to 9 vertices) wraps to slot 0 itself, as
	   in the shading path. */
	const uint32_t maxp = vc + 1 < OR_MAXP ? vc + 1 : OR_MAXP;
	prepare_projected_solid_angle_polygon_sampling(&p, vc, v, maxp);
	for (uint32_t k = 0; k != count; ++k) {
		vec3_t d = sample_projected_solid_angle_polygon(&p, V2(rnd[2 * k], rnd[2 * k + 1]), maxp);
		out_dirs[3 * k] = d.x;
		out_dirs[3 * k + 1] = d.y;
		out_dirs[3 * k + 2] = d.z;
		if (out_errors) {
			/* Backward error: area from the sector start to the sample versus
			   the target (compute_projected_solid_angle_polygon_sampling_error,
			   polygon_sampling.glsl:846-906, first component). */
			out_errors[k] = 0.0f;
			if (!is_central_case(&p)) {
				float target = rnd[2 * k] * p.projected_solid_angle;
				float sector = 0.0f;
				vec2_t outer = V2(0.0f, 0.0f), inner = p.inner_ellipse_0, dir_0 = V2(0.0f, 0.0f);
				for (uint32_t i = 0; i != vc; ++i) {
					if ((i > 1 && i + 1 == vc) || (i > 0 && target < 0.0f)) break;
					sector = p.sector_projected_solid_angles[i];
					target -= sector;
					vec2_t ve = p.ellipses[i];
					int vi = is_inner_ellipse(ve);
					if (i == 0) outer = ve;
					else {
						inner = vi ? ve : inner;
						outer = vi ? outer : ve;
					}
					dir_0 = p.vertices[i];
				}
				target += sector;
				float sampled = get_area_between_ellipses_in_sector(inner, get_ellipse_rsqrt_det(inner), outer,
				                                                    get_ellipse_rsqrt_det(outer), dir_0, V2(d.x, d.y));
				out_errors[k] = (target - sampled) / p.projected_solid_angle;
			}
		}
	}
	return p.projected_solid_angle;
}

/* Any-hit query of the scene (brute force or through its BVH); rays are
   {origin xyz, t_min, direction xyz, t_max}. */
void oracle_f32_any_hit(const oracle_scene_t* s, const float* rays, uint32_t count, uint32_t* hits) {
	for (uint32_t i = 0; i != count; ++i) {
		const float* r = rays + 8 * (size_t) i;
		hits[i] = (uint32_t) any_hit(s, V3(r[0], r[1], r[2]), V3(r[4], r[5], r[6]), r[3], r[7]);
	}
}

/* The cluster proposal's candidates of one shading point (position x,
   normal n, pixel px, py of a width-wide frame): settings->candidate_count
   lights with their probabilities. */
void oracle_f32_proposal(const oracle_scene_t* s, const oracle_settings_t* st, const float* x, const float* n,
                         uint32_t px, uint32_t py, uint32_t width, int32_t* lights, float* pdfs) {
	static proposal_candidate_t out[OR_MAX_CANDIDATES];
	if (st->candidate_count > OR_MAX_CANDIDATES || s->cluster_count <= 0 || s->cluster_count > OR_MAX_CLUSTERS) return;
	proposal_draw(s, st, x, n, px, py, width, out);
	for (int c = 0; c != st->candidate_count; ++c) {
		lights[c] = out[c].light;
		pdfs[c] = out[c].pdf;
	}
}

/* The LTC-CP target p_hat = length(evaluate_polygonal_light_shading) of every
   light at pixel i of the G-buffer (shading_pass.frag.glsl:421-456, 732). */
void oracle_f32_ltc_cp_targets(const oracle_scene_t* s, const oracle_settings_t* st, const oracle_gbuffer_t* gbuffer,
                               uint32_t i, float* p_hat) {
	ctx_t c;
	c.scene = s;
	c.settings = st;
	c.maxv = (uint32_t) s->max_light_vertex_count;
	c.maxp = c.maxv + 1;
	const size_t np = (size_t) gbuffer->width * gbuffer->height;
	const float* g = gbuffer->planes;
	shading_data_t sd;
	sd.position = V3(g[0 * np + i], g[1 * np + i], g[2 * np + i]);
	sd.normal = V3(g[3 * np + i], g[4 * np + i], g[5 * np + i]);
	sd.outgoing = V3(g[6 * np + i], g[7 * np + i], g[8 * np + i]);
	sd.lambert_outgoing = g[9 * np + i];
	sd.diffuse_albedo = V3(g[10 * np + i], g[11 * np + i], g[12 * np + i]);
	sd.fresnel_0 = V3(g[13 * np + i], g[14 * np + i], g[15 * np + i]);
	sd.roughness = g[16 * np + i];
	float fl = v3_dot(sd.fresnel_0, V3(0.2126f, 0.7152f, 0.0722f));
	ltc_coefficients_t ltc = get_ltc_coefficients(s, fl, sd.roughness, sd.position, sd.normal, sd.outgoing);
	for (int l = 0; l != s->light_count; ++l) {
		light_t light;
		load_light(s, l, &light);
		p_hat[l] = v3_length(ltc_cp_target(&c, &sd, ltc, &light));
	}
}
