/* oracle_core.h - CPU restatement of risltc's per-pixel shading path.
 * Restates upstream risltc routines (GPLv3; the polygon_sampling.glsl parts
 * also BSD-3, whose notice is retained in NOTICE).
 *
 * TEST INFRASTRUCTURE.  This is the oracle: the checker the CUDA kernels are
 * compared against, and the CPU baseline that bench.py times.  The product
 * (risltc_gb300/, include/) never includes, links or runs anything under
 * oracle/.
 *
 * The code is included by oracle_f32.c (R = float, the reference's precision)
 * and oracle_f64.c (R = double, the ground-truth twin).  Every function
 * follows one reference routine; the citation is given above each.  All paths
 * are relative to the reference repository (ishaanshah/risltc).
 *
 * Evaluation conventions (shared with oracle/ref/glsl_shim.hpp and the CUDA
 * kernels' exact mode, which is what makes them agree bit for bit):
 * dot products and matrix-vector products add left to right, no a*b+c is
 * contracted, normalize(v) = v * (1/sqrt(dot(v,v))), max(x,y) = x<y ? y : x,
 * and the FP32 transcendentals come from include/risltc_math.h.
 *
 * Requires before inclusion: R, RC(literal), R_FMA, R_SQRT, R_ATAN, R_ACOS,
 * R_SINCOS, R_FLOOR, R_SIGNBIT, R_ISINF, R_EXPONENT_FLIP, R_INF, ORACLE_SUFFIX.
 */
#include <stdint.h>
#include <stddef.h>
#include <string.h>
#include "oracle.h"

#define OR_CAT2(a, b) a##b
#define OR_CAT(a, b) OR_CAT2(a, b)
#define OR_EXPORT(name) OR_CAT(name, ORACLE_SUFFIX)

#define OR_MAXV 8
#define OR_MAXP 9

#define OR_PI RC(3.1415926535897932384626433832795)
#define OR_INV_PI RC(0.31830988618379067153776752674503)
#define OR_HALF_PI RC(1.5707963267948966192313216916398)

typedef struct { R x, y; } vec2_t;
typedef struct { R x, y, z; } vec3_t;
typedef struct { R x, y, z, w; } vec4_t;
typedef struct { vec2_t c[2]; } mat2_t;
typedef struct { vec3_t c[3]; } mat3_t;
typedef struct { vec3_t c[4]; } mat4x3_t;

static inline R rmax(R x, R y) { return (x < y) ? y : x; }
static inline R rmin(R x, R y) { return (y < x) ? y : x; }
static inline R rclamp(R x, R lo, R hi) { return rmin(rmax(x, lo), hi); }
static inline R rabs(R x) { return R_SIGNBIT(x) ? -x : x; }

static inline vec2_t V2(R x, R y) { vec2_t r; r.x = x; r.y = y; return r; }
static inline vec3_t V3(R x, R y, R z) { vec3_t r; r.x = x; r.y = y; r.z = z; return r; }
static inline vec2_t v2_add(vec2_t a, vec2_t b) { return V2(a.x + b.x, a.y + b.y); }
static inline vec2_t v2_sub(vec2_t a, vec2_t b) { return V2(a.x - b.x, a.y - b.y); }
static inline vec2_t v2_scale(vec2_t a, R s) { return V2(a.x * s, a.y * s); }
static inline vec2_t v2_neg(vec2_t a) { return V2(-a.x, -a.y); }
static inline R v2_dot(vec2_t a, vec2_t b) { return a.x * b.x + a.y * b.y; }
static inline vec2_t v2_fma(vec2_t a, vec2_t b, vec2_t c) { return V2(R_FMA(a.x, b.x, c.x), R_FMA(a.y, b.y, c.y)); }
static inline vec2_t v2_normalize(vec2_t a) { return v2_scale(a, RC(1.0) / R_SQRT(v2_dot(a, a))); }
/* rotate_90, polygon_sampling.glsl:285-287 */
static inline vec2_t rotate_90(vec2_t v) { return V2(-v.y, v.x); }
static inline vec3_t v3_add(vec3_t a, vec3_t b) { return V3(a.x + b.x, a.y + b.y, a.z + b.z); }
static inline vec3_t v3_sub(vec3_t a, vec3_t b) { return V3(a.x - b.x, a.y - b.y, a.z - b.z); }
static inline vec3_t v3_mul(vec3_t a, vec3_t b) { return V3(a.x * b.x, a.y * b.y, a.z * b.z); }
static inline vec3_t v3_div(vec3_t a, vec3_t b) { return V3(a.x / b.x, a.y / b.y, a.z / b.z); }
static inline vec3_t v3_scale(vec3_t a, R s) { return V3(a.x * s, a.y * s, a.z * s); }
static inline vec3_t v3_adds(vec3_t a, R s) { return V3(a.x + s, a.y + s, a.z + s); }
static inline vec3_t v3_neg(vec3_t a) { return V3(-a.x, -a.y, -a.z); }
static inline vec3_t v3_splat(R s) { return V3(s, s, s); }
static inline R v3_dot(vec3_t a, vec3_t b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static inline R v3_length(vec3_t a) { return R_SQRT(v3_dot(a, a)); }
static inline vec3_t v3_normalize(vec3_t a) { return v3_scale(a, RC(1.0) / R_SQRT(v3_dot(a, a))); }
static inline vec3_t v3_cross(vec3_t a, vec3_t b) {
	return V3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
static inline vec3_t v3_fma(vec3_t a, vec3_t b, vec3_t c) {
	return V3(R_FMA(a.x, b.x, c.x), R_FMA(a.y, b.y, c.y), R_FMA(a.z, b.z, c.z));
}
static inline vec3_t v3_max(vec3_t a, vec3_t b) { return V3(rmax(a.x, b.x), rmax(a.y, b.y), rmax(a.z, b.z)); }
/* dot(vec4(p, 1.0), plane): the last term is plane.w * 1. */
static inline R plane_dot(vec3_t p, const R plane[4]) {
	return p.x * plane[0] + p.y * plane[1] + p.z * plane[2] + RC(1.0) * plane[3];
}
static inline vec3_t m3_mul(const mat3_t* m, vec3_t v) {
	return v3_add(v3_add(v3_scale(m->c[0], v.x), v3_scale(m->c[1], v.y)), v3_scale(m->c[2], v.z));
}
/* mat4x3 * vec4(p, 1.0) */
static inline vec3_t m43_mul_point(const mat4x3_t* m, vec3_t p) {
	vec3_t r = v3_add(v3_add(v3_scale(m->c[0], p.x), v3_scale(m->c[1], p.y)), v3_scale(m->c[2], p.z));
	return v3_add(r, v3_scale(m->c[3], RC(1.0)));
}
/* mat3 * mat4x3, column by column */
static inline mat4x3_t m3_mul_m43(const mat3_t* a, const mat4x3_t* b) {
	mat4x3_t r;
	for (int i = 0; i != 4; ++i) r.c[i] = m3_mul(a, b->c[i]);
	return r;
}
/* (transpose(mat4x3) * dir).xyz = (dot(c0, d), dot(c1, d), dot(c2, d)) */
static inline vec3_t m43_transpose_mul(const mat4x3_t* m, vec3_t d) {
	return V3(v3_dot(m->c[0], d), v3_dot(m->c[1], d), v3_dot(m->c[2], d));
}
static inline R m2_det(const mat2_t* m) { return m->c[0].x * m->c[1].y - m->c[1].x * m->c[0].y; }
static inline mat2_t outer2(vec2_t col, vec2_t row) {
	mat2_t r;
	r.c[0] = v2_scale(col, row.x);
	r.c[1] = v2_scale(col, row.y);
	return r;
}

/* ------------------------------------------------------------------------ */
/* Noise: noise_utility.glsl:26-95 (integer arithmetic, identical in both
   precisions; draws are FP32 values as in the reference). */
static uint32_t murmur_hash3_mix(uint32_t hash, uint32_t k) {
	k *= 0xcc9e2d51u;
	k = (k << 15) | (k >> 17);
	k *= 0x1b873593u;
	hash ^= k;
	hash = ((hash << 13) | (hash >> 19)) * 5u + 0xe6546b64u;
	return hash;
}
static uint32_t murmur_hash3_finalize(uint32_t hash) {
	hash ^= hash >> 16;
	hash *= 0x85ebca6bu;
	hash ^= hash >> 13;
	hash *= 0xc2b2ae35u;
	hash ^= hash >> 16;
	return hash;
}
/* get_noise_gen: one LCG step, float(seed) * 2^-32 */
static R get_noise_1(uint32_t* seed) {
	*seed = 1664525u * *seed + 1013904223u;
	float u = (float) *seed * 2.3283064365386962890625e-10f;
	return (R) u;
}
static vec2_t get_noise_2(uint32_t* seed) {
	R a = get_noise_1(seed);
	R b = get_noise_1(seed);
	return V2(a, b);
}
/* get_noise_accessor, noise_utility.glsl:77-84 */
static uint32_t get_noise_accessor(uint32_t px, uint32_t py, uint32_t width, uint32_t random_number_x) {
	uint32_t index = murmur_hash3_mix(0u, px + py * width);
	return murmur_hash3_finalize(murmur_hash3_mix(index, random_number_x));
}

/* ------------------------------------------------------------------------ */
/* Shading data (brdfs.glsl:22-39) and LTC coefficients (ltc_utility.glsl:30-49) */
typedef struct {
	vec3_t position, normal, outgoing;
	R lambert_outgoing;
	vec3_t diffuse_albedo, fresnel_0;
	R roughness;
} shading_data_t;

typedef struct {
	mat4x3_t world_to_shading_space;
	mat3_t shading_to_cosine_space;
	mat3_t cosine_to_shading_space;
	R albedo;
	R shading_to_cosine_space_determinant;
} ltc_coefficients_t;

/* Texel fetch with clamp to edge; texels are [layer][height][width][channels]. */
static R ltc_texel(const float* t, int w, int h, int channels, int layer, int y, int x, int c) {
	x = x < 0 ? 0 : (x >= w ? w - 1 : x);
	y = y < 0 ? 0 : (y >= h ? h - 1 : y);
	return (R) t[(((size_t) layer * h + y) * w + x) * channels + c];
}

/* textureLod on the LTC arrays: bilinear in FP32 arithmetic with clamp to
   edge and nearest layer (the reference samples UNORM16 textures with the
   hardware filter, ltc_table.c:170-182). */
static void ltc_fetch(const oracle_scene_t* s, vec3_t coord, R out0[4], R out1[2]) {
	R layer_f = coord.z + RC(0.5);
	int layer = (int) layer_f;
	layer = layer < 0 ? 0 : (layer >= s->ltc_layers ? s->ltc_layers - 1 : layer);
	R fu = coord.x * (R) s->ltc_width - RC(0.5);
	R fv = coord.y * (R) s->ltc_height - RC(0.5);
	R iu = R_FLOOR(fu), iv = R_FLOOR(fv);
	R ax = fu - iu, ay = fv - iv;
	int x0 = (int) iu, y0 = (int) iv;
	for (int t = 0; t != 2; ++t) {
		const float* tex = t ? s->ltc1 : s->ltc0;
		int ch = t ? 2 : 4;
		for (int c = 0; c != ch; ++c) {
			R t00 = ltc_texel(tex, s->ltc_width, s->ltc_height, ch, layer, y0, x0, c);
			R t10 = ltc_texel(tex, s->ltc_width, s->ltc_height, ch, layer, y0, x0 + 1, c);
			R t01 = ltc_texel(tex, s->ltc_width, s->ltc_height, ch, layer, y0 + 1, x0, c);
			R t11 = ltc_texel(tex, s->ltc_width, s->ltc_height, ch, layer, y0 + 1, x0 + 1, c);
			R top = t00 * (RC(1.0) - ax) + t10 * ax;
			R bottom = t01 * (RC(1.0) - ax) + t11 * ax;
			R v = top * (RC(1.0) - ay) + bottom * ay;
			if (t) out1[c] = v; else out0[c] = v;
		}
	}
}

/* get_ltc_coefficients, ltc_utility.glsl:56-88 */
static ltc_coefficients_t get_ltc_coefficients(const oracle_scene_t* s, R fresnel_0, R roughness, vec3_t p, vec3_t n,
                                               vec3_t wo) {
	ltc_coefficients_t ltc;
	const float* k = s->ltc_constants;
	R normal_dot_outgoing = v3_dot(n, wo);
	R inclination = R_ACOS(rclamp(normal_dot_outgoing, RC(0.0), RC(1.0)));
	vec3_t tc = V3(R_FMA(R_SQRT(rclamp(roughness, RC(0.0), RC(1.0))), (R) k[2], (R) k[3]),
	               R_FMA(inclination, (R) k[4], (R) k[5]),
	               R_FMA(rclamp(fresnel_0, RC(0.0), RC(1.0)), (R) k[0], (R) k[1]));
	R d0[4], d1[2];
	ltc_fetch(s, tc, d0, d1);
	ltc.shading_to_cosine_space.c[0] = V3(d0[0], RC(0.0), -d0[1]);
	ltc.shading_to_cosine_space.c[1] = V3(RC(0.0), d0[2], RC(0.0));
	ltc.shading_to_cosine_space.c[2] = V3(d0[3], RC(0.0), d1[0]);
	ltc.albedo = d1[1];
	R determinant_2x2 = d0[0] * d1[0] + d0[1] * d0[3];
	ltc.shading_to_cosine_space_determinant = d0[2] * determinant_2x2;
	R inv_determinant_2x2 = RC(1.0) / determinant_2x2;
	ltc.cosine_to_shading_space.c[0] = V3(d1[0] * inv_determinant_2x2, RC(0.0), d0[1] * inv_determinant_2x2);
	ltc.cosine_to_shading_space.c[1] = V3(RC(0.0), RC(1.0) / d0[2], RC(0.0));
	ltc.cosine_to_shading_space.c[2] = V3(-d0[3] * inv_determinant_2x2, RC(0.0), d0[0] * inv_determinant_2x2);
	vec3_t x_axis = v3_normalize(v3_fma(v3_splat(-normal_dot_outgoing), n, wo));
	vec3_t y_axis = v3_cross(n, x_axis);
	/* rotation = transpose(mat3(x, y, n)); its columns are (x[j], y[j], n[j]) */
	mat3_t rot;
	rot.c[0] = V3(x_axis.x, y_axis.x, n.x);
	rot.c[1] = V3(x_axis.y, y_axis.y, n.y);
	rot.c[2] = V3(x_axis.z, y_axis.z, n.z);
	mat3_t neg_rot;
	for (int i = 0; i != 3; ++i) neg_rot.c[i] = v3_neg(rot.c[i]);
	ltc.world_to_shading_space.c[0] = rot.c[0];
	ltc.world_to_shading_space.c[1] = rot.c[1];
	ltc.world_to_shading_space.c[2] = rot.c[2];
	ltc.world_to_shading_space.c[3] = m3_mul(&neg_rot, p);
	return ltc;
}

/* evaluate_ltc_density, ltc_utility.glsl:100-105 */
static R evaluate_ltc_density(const ltc_coefficients_t* ltc, vec3_t dir, R rcp_projected_solid_angle) {
	vec3_t dc = m3_mul(&ltc->shading_to_cosine_space, dir);
	R l2 = v3_dot(dc, dc);
	R density = rmax(RC(0.0), dc.z) * ltc->shading_to_cosine_space_determinant / (l2 * l2);
	return density * rcp_projected_solid_angle;
}

/* ------------------------------------------------------------------------ */
/* iz0, polygon_clipping.glsl:19-25 */
static vec3_t iz0(vec3_t lhs, vec3_t rhs) {
	R l = lhs.z / (lhs.z - rhs.z);
	return V3(R_FMA(l, rhs.x, R_FMA(-l, lhs.x, lhs.x)), R_FMA(l, rhs.y, R_FMA(-l, lhs.y, lhs.y)), RC(0.0));
}

/* clip_polygon, polygon_clipping.glsl:35-225.
 *
 * The reference is an auto-generated switch over (vertex count, sign
 * pattern).  Restated as the rule that reproduces its table: the vertices
 * with z > 0 form one cyclic run v_s..v_e (any other pattern clips to
 * nothing); the output cycle is [iz0(v_{s-1}, v_s), v_s, ..., v_e,
 * iz0(v_e, v_{e+1})], written in place at the rotation that needs the fewest
 * generated assignments (vertices that leave their slot, plus the trailing
 * copy of v[0] to slot vc unless it already holds that value), ties going to
 * the fewest moved vertices and then to the first rotation in enumeration
 * order.  v[vc] = v[0] when vc < max_polygon_vertex_count; slots above vc are
 * left untouched.  With reference_limits, 8-gons clip to nothing because the
 * reference packs the vertex count into the low three bits of its case label.
 */
static uint32_t clip_polygon(uint32_t n, vec3_t v[], uint32_t max_polygon_vertex_count, int reference_limits) {
	int above[OR_MAXP];
	uint32_t k = 0;
	if (n < 3 || n > OR_MAXV || (reference_limits && n > 7)) return 0;
	for (uint32_t i = 0; i != n; ++i) {
		above[i] = v[i].z > RC(0.0);
		k += (uint32_t) above[i];
	}
	if (k == 0) return 0;
	if (k == n) {
		if (n < max_polygon_vertex_count) v[n] = v[0];
		return n;
	}
	uint32_t starts = 0, s = 0;
	for (uint32_t i = 0; i != n; ++i)
		if (above[i] && !above[(i + n - 1) % n]) {
			++starts;
			s = i;
		}
	if (starts != 1) return 0;
	uint32_t e = (s + k - 1) % n, vc = k + 2;
	vec3_t cyc[OR_MAXP + 1];
	cyc[0] = iz0(v[(s + n - 1) % n], v[s]);
	for (uint32_t j = 0; j != k; ++j) cyc[1 + j] = v[(s + j) % n];
	cyc[k + 1] = iz0(v[e], v[(e + 1) % n]);
	uint32_t best_cost = 0xffffffffu, best_r = 0;
	for (uint32_t shift = 0; shift != vc; ++shift) {
		uint32_t r = (vc - shift) % vc, moved = 0;
		for (uint32_t j = 1; j <= k; ++j) moved += ((r + j) % vc) != ((s + j - 1) % n);
		uint32_t j0 = (vc - r) % vc;
		uint32_t trailing = !(vc < n && j0 >= 1 && j0 <= k && ((s + j0 - 1) % n) == vc);
		uint32_t cost = (moved + trailing) * 64u + moved;
		if (cost < best_cost) {
			best_cost = cost;
			best_r = r;
		}
	}
	vec3_t out[OR_MAXP + 1];
	for (uint32_t j = 0; j != vc; ++j) out[(best_r + j) % vc] = cyc[j];
	for (uint32_t j = 0; j != vc; ++j) v[j] = out[j];
	if (vc < max_polygon_vertex_count) v[vc] = v[0];
	return vc;
}

/* ------------------------------------------------------------------------ */
/* integrateEdgeVec, polygon_sampling.glsl:508-521, on pre-normalised
   vertices (normalize() is deterministic, so normalising each vertex once
   gives the same bits as normalising it once per adjacent edge). */
static R integrate_edge_normalized(vec3_t v1, vec3_t v2) {
	R x = v3_dot(v1, v2);
	R y = rabs(x);
	R a = RC(0.8543985) + (RC(0.4965155) + RC(0.0145206) * y) * y;
	R b = RC(3.4175940) + (RC(4.1616724) + y) * y;
	R v = a / b;
	R theta_sintheta = (x > RC(0.0)) ? v : RC(0.5) * (RC(1.0) / R_SQRT(rmax(RC(1.0) - x * x, RC(1e-7)))) - v;
	return (v1.x * v2.y - v1.y * v2.x) * theta_sintheta;
}

/* calculate_ltc, polygon_sampling.glsl:523-530.  The reference integrates
   over all MAX_POLYGON_VERTEX_COUNT slots with wrap-around, including slots
   the clipper did not write.  The product integrates the clipped polygon's
   own vc edges; reference_slots = 1 reproduces the reference's sum over all
   slots (stale slots and all) for the pinning tests. */
static R calculate_ltc(uint32_t vc, const vec3_t v[], uint32_t max_polygon_vertex_count, int reference_slots) {
	vec3_t nv[OR_MAXP];
	uint32_t count = reference_slots ? max_polygon_vertex_count : vc;
	for (uint32_t i = 0; i != count; ++i) nv[i] = v3_normalize(v[i]);
	R result = RC(0.0);
	for (uint32_t i = 0; i != count; ++i) result += integrate_edge_normalized(nv[i], nv[(i + 1) % count]);
	return rabs(result);
}

/* ------------------------------------------------------------------------ */
/* Projected solid angle sampling, polygon_sampling.glsl:231-828 */
typedef struct {
	uint32_t vertex_count;
	vec2_t vertices[OR_MAXP];
	vec2_t ellipses[OR_MAXP];
	vec2_t inner_ellipse_0;
	R sector_projected_solid_angles[OR_MAXP];
	R projected_solid_angle;
} projected_solid_angle_polygon_t;

/* fast_positive_atan, polygon_sampling.glsl:84-98 */
static R fast_positive_atan(R y) {
	R rx, ry, rz;
	rx = (rabs(y) > RC(1.0)) ? (RC(1.0) / rabs(y)) : rabs(y);
	ry = rx * rx;
	rz = R_FMA(ry, RC(0.02083509974181652), RC(-0.08513300120830536));
	rz = R_FMA(ry, rz, RC(0.18014100193977356));
	rz = R_FMA(ry, rz, RC(-0.3302994966506958));
	ry = R_FMA(ry, rz, RC(0.9998660087585449));
	rz = R_FMA(RC(-2.0) * ry, rx, OR_HALF_PI);
	rz = (rabs(y) > RC(1.0)) ? rz : RC(0.0);
	rx = R_FMA(rx, ry, rz);
	return (y < RC(0.0)) ? (OR_PI - rx) : rx;
}

/* positive_atan, polygon_sampling.glsl:105-112 */
static int g_oracle_fast_atan;
static R positive_atan(R tangent) {
	if (g_oracle_fast_atan) return fast_positive_atan(tangent);
	R offset = (tangent < RC(0.0)) ? OR_PI : RC(0.0);
	return R_ATAN(tangent) + offset;
}

/* mix_fma, polygon_sampling.glsl:184-186 */
static inline R mix_fma(R x, R y, R a) { return R_FMA(a, y, R_FMA(-a, x, x)); }

/* kahan, polygon_sampling.glsl:262-269 */
static inline R kahan(R a, R b, R c, R d) {
	R cd = c * d;
	R error = R_FMA(c, d, -cd);
	R result = R_FMA(a, b, -cd);
	return result - error;
}

/* cross_stable, polygon_sampling.glsl:274-280 */
static inline vec3_t cross_stable(vec3_t l, vec3_t r) {
	return V3(kahan(l.y, r.z, l.z, r.y), kahan(l.z, r.x, l.x, r.z), kahan(l.x, r.y, l.y, r.x));
}

/* is_inner_ellipse (sign bit of x), polygon_sampling.glsl:293-300 */
static inline int is_inner_ellipse(vec2_t e) { return R_SIGNBIT(e.x) ? 1 : 0; }
/* is_central_case, polygon_sampling.glsl:305-307 */
static inline int is_central_case(const projected_solid_angle_polygon_t* p) { return p->inner_ellipse_0.x > RC(0.0); }

/* ellipse_from_edge, polygon_sampling.glsl:318-327 */
static vec2_t ellipse_from_edge(vec3_t v0, vec3_t v1) {
	vec3_t normal = cross_stable(v0, v1);
	R scaling = RC(1.0) / normal.z;
	scaling = is_inner_ellipse(V2(normal.x, normal.y)) ? -scaling : scaling;
	vec2_t ellipse = V2(normal.x * scaling, normal.y * scaling);
	ellipse.x = (normal.z != RC(0.0)) ? ellipse.x : R_INF;
	return ellipse;
}

/* ellipse_transform, polygon_sampling.glsl:333-335 */
static inline vec2_t ellipse_transform(vec2_t e, vec2_t p) { return v2_fma(V2(v2_dot(e, p), v2_dot(e, p)), e, p); }
/* get_ellipse_det / rsqrt_det, polygon_sampling.glsl:341-349 */
static inline R get_ellipse_det(vec2_t e) { return R_FMA(e.x, e.x, R_FMA(e.y, e.y, RC(1.0))); }
static inline R get_ellipse_rsqrt_det(vec2_t e) { return RC(1.0) / R_SQRT(get_ellipse_det(e)); }
/* polygon_sampling.glsl:352-373 */
static inline R get_ellipse_direction_factor_rsq(vec2_t e, vec2_t d) {
	R ed = v2_dot(e, d);
	R dd = v2_dot(d, d);
	return R_FMA(ed, ed, dd);
}
static inline R get_ellipse_direction_factor(vec2_t e, vec2_t d) {
	return RC(1.0) / R_SQRT(get_ellipse_direction_factor_rsq(e, d));
}
static inline R get_ellipse_normalized_direction_factor(vec2_t e, vec2_t d) {
	R ed = v2_dot(e, d);
	return RC(1.0) / R_SQRT(R_FMA(ed, ed, RC(1.0)));
}

/* polygon_sampling.glsl:378-383 */
static R get_area_between_ellipses_in_sector_from_tangents(R inner_rsqrt_det, R inner_tangent, R outer_rsqrt_det,
                                                           R outer_tangent) {
	R inner_area = inner_rsqrt_det * positive_atan(inner_tangent);
	R result = R_FMA(outer_rsqrt_det, positive_atan(outer_tangent), -inner_area);
	return (result > RC(0.0)) ? (RC(0.5) * result) : RC(0.0);
}

/* polygon_sampling.glsl:391-398 */
static R get_area_between_ellipses_in_sector(vec2_t inner, R inner_rsqrt_det, vec2_t outer, R outer_rsqrt_det,
                                             vec2_t dir_0, vec2_t dir_1) {
	R det_dirs = rmax(RC(0.0), v2_dot(dir_1, rotate_90(dir_0)));
	R inner_dot = inner_rsqrt_det * v2_dot(dir_0, ellipse_transform(inner, dir_1));
	R outer_dot = outer_rsqrt_det * v2_dot(dir_0, ellipse_transform(outer, dir_1));
	return get_area_between_ellipses_in_sector_from_tangents(inner_rsqrt_det, det_dirs / inner_dot, outer_rsqrt_det,
	                                                         det_dirs / outer_dot);
}

/* polygon_sampling.glsl:406-413 */
static R get_ellipse_area_in_sector(vec2_t e, vec2_t dir_0, vec2_t dir_1) {
	R rsqrt_det = get_ellipse_rsqrt_det(e);
	R det_dirs = rmax(RC(0.0), v2_dot(dir_1, rotate_90(dir_0)));
	R ellipse_dot = rsqrt_det * v2_dot(dir_0, ellipse_transform(e, dir_1));
	R area = RC(0.5) * rsqrt_det * positive_atan(det_dirs / ellipse_dot);
	return (rsqrt_det > RC(0.0)) ? area : RC(0.0);
}

/* compare_and_swap, polygon_sampling.glsl:422-436 */
static void compare_and_swap(projected_solid_angle_polygon_t* p, uint32_t lhs, uint32_t rhs) {
	vec2_t lhs_copy = p->vertices[lhs];
	R normal_z = kahan(lhs_copy.x, -p->vertices[rhs].y, lhs_copy.y, -p->vertices[rhs].x);
	int swap = (normal_z == RC(0.0)) ? (R_ISINF(p->ellipses[rhs].x) ? 1 : 0) : (normal_z > RC(0.0));
	p->vertices[lhs] = swap ? p->vertices[rhs] : lhs_copy;
	p->vertices[rhs] = swap ? lhs_copy : p->vertices[rhs];
	lhs_copy = p->ellipses[lhs];
	p->ellipses[lhs] = swap ? p->ellipses[rhs] : lhs_copy;
	p->ellipses[rhs] = swap ? lhs_copy : p->ellipses[rhs];
}

/* sort_convex_polygon_vertices, polygon_sampling.glsl:441-506 */
static void sort_convex_polygon_vertices(projected_solid_angle_polygon_t* p) {
	switch (p->vertex_count) {
	case 3:
		compare_and_swap(p, 1, 2);
		break;
	case 4:
		compare_and_swap(p, 1, 3);
		break;
	case 5:
		compare_and_swap(p, 2, 4);
		compare_and_swap(p, 1, 3);
		compare_and_swap(p, 1, 2);
		compare_and_swap(p, 0, 3);
		compare_and_swap(p, 3, 4);
		break;
	case 6:
		compare_and_swap(p, 3, 5);
		compare_and_swap(p, 2, 4);
		compare_and_swap(p, 1, 5);
		compare_and_swap(p, 0, 4);
		compare_and_swap(p, 4, 5);
		compare_and_swap(p, 1, 3);
		break;
	case 7:
		compare_and_swap(p, 2, 5);
		compare_and_swap(p, 1, 6);
		compare_and_swap(p, 5, 6);
		compare_and_swap(p, 3, 4);
		compare_and_swap(p, 0, 4);
		compare_and_swap(p, 4, 6);
		compare_and_swap(p, 1, 3);
		compare_and_swap(p, 3, 5);
		compare_and_swap(p, 4, 5);
		break;
	case 8:
		compare_and_swap(p, 2, 6);
		compare_and_swap(p, 3, 7);
		compare_and_swap(p, 1, 5);
		compare_and_swap(p, 0, 4);
		compare_and_swap(p, 4, 6);
		compare_and_swap(p, 5, 7);
		compare_and_swap(p, 6, 7);
		compare_and_swap(p, 4, 5);
		compare_and_swap(p, 1, 3);
		break;
	case 9:
		/* Only 8-gons clipped to 9 vertices get here (the reference stops at
		   8-vertex networks): adjacent compare-and-swap passes. */
		for (uint32_t i = 1; i != 9; ++i)
			for (uint32_t j = i; j != 0; --j) compare_and_swap(p, j - 1, j);
		break;
	default:
		break;
	}
	compare_and_swap(p, 0, 2);
	if (p->vertex_count >= 4) compare_and_swap(p, 2, 3);
	compare_and_swap(p, 0, 1);
}

/* prepare_projected_solid_angle_polygon_sampling, polygon_sampling.glsl:545-613 */
static void prepare_projected_solid_angle_polygon_sampling(projected_solid_angle_polygon_t* p, uint32_t vertex_count,
                                                           const vec3_t v[], uint32_t max_polygon_vertex_count) {
	uint32_t maxp = max_polygon_vertex_count;
	p->vertex_count = vertex_count;
	p->inner_ellipse_0 = V2(RC(1.0), RC(0.0));
	p->vertices[0] = V2(v[0].x, v[0].y);
	p->ellipses[0] = ellipse_from_edge(v[0], v[1]);
	vec2_t previous_ellipse = p->ellipses[0];
	for (uint32_t i = 1; i != maxp; ++i) {
		p->vertices[i] = V2(v[i].x, v[i].y);
		if (i > 2 && i == vertex_count) break;
		vec2_t ellipse = ellipse_from_edge(v[i], v[(i + 1) % maxp]);
		int ellipse_inner = is_inner_ellipse(ellipse);
		p->ellipses[i] = ellipse_inner ? previous_ellipse : ellipse;
		p->inner_ellipse_0 =
		    (is_inner_ellipse(previous_ellipse) && !ellipse_inner) ? previous_ellipse : p->inner_ellipse_0;
		previous_ellipse = ellipse;
	}
	{
		vec2_t ellipse = p->ellipses[0];
		int ellipse_inner = is_inner_ellipse(ellipse);
		p->ellipses[0] = ellipse_inner ? previous_ellipse : ellipse;
		p->inner_ellipse_0 =
		    (is_inner_ellipse(previous_ellipse) && !ellipse_inner) ? previous_ellipse : p->inner_ellipse_0;
	}
	p->projected_solid_angle = RC(0.0);
	if (is_central_case(p)) {
		for (uint32_t i = 0; i != maxp; ++i) {
			if (i > 2 && i == vertex_count) break;
			p->sector_projected_solid_angles[i] =
			    get_ellipse_area_in_sector(p->ellipses[i], p->vertices[i], p->vertices[(i + 1) % maxp]);
			p->projected_solid_angle += p->sector_projected_solid_angles[i];
		}
	} else {
		sort_convex_polygon_vertices(p);
		vec2_t inner_ellipse = p->inner_ellipse_0;
		R inner_rsqrt_det = get_ellipse_rsqrt_det(inner_ellipse);
		vec2_t outer_ellipse = V2(RC(0.0), RC(0.0));
		R outer_rsqrt_det = RC(0.0);
		for (uint32_t i = 0; i != maxp - 1; ++i) {
			if (i > 1 && i + 1 == vertex_count) break;
			vec2_t vertex_ellipse = p->ellipses[i];
			int vertex_inner = is_inner_ellipse(vertex_ellipse);
			R vertex_rsqrt_det = get_ellipse_rsqrt_det(vertex_ellipse);
			if (i == 0) {
				outer_ellipse = vertex_ellipse;
				outer_rsqrt_det = vertex_rsqrt_det;
			} else {
				inner_ellipse = vertex_inner ? vertex_ellipse : inner_ellipse;
				inner_rsqrt_det = vertex_inner ? vertex_rsqrt_det : inner_rsqrt_det;
				outer_ellipse = vertex_inner ? outer_ellipse : vertex_ellipse;
				outer_rsqrt_det = vertex_inner ? outer_rsqrt_det : vertex_rsqrt_det;
			}
			p->sector_projected_solid_angles[i] = get_area_between_ellipses_in_sector(
			    inner_ellipse, inner_rsqrt_det, outer_ellipse, outer_rsqrt_det, p->vertices[i], p->vertices[i + 1]);
			p->projected_solid_angle += p->sector_projected_solid_angles[i];
		}
	}
}

/* normalize_approx_and_flip, polygon_sampling.glsl:622-634 */
static vec2_t normalize_approx_and_flip(vec2_t rhs, vec2_t semi_circle) {
	R scaling = rabs(rhs.x) + rabs(rhs.y);
	scaling = R_EXPONENT_FLIP(scaling);
	scaling = (v2_dot(rhs, semi_circle) >= RC(0.0)) ? scaling : -scaling;
	return v2_scale(rhs, scaling);
}

/* solve_homogeneous_quadratic, polygon_sampling.glsl:648-653 */
static vec2_t solve_homogeneous_quadratic(const mat2_t* q) {
	R coeff_xy = RC(0.5) * (q->c[0].y + q->c[1].x);
	R sqrt_discriminant = R_SQRT(rmax(RC(0.0), coeff_xy * coeff_xy - q->c[0].x * q->c[1].y));
	R scaled_root = rabs(coeff_xy) + sqrt_discriminant;
	return (coeff_xy >= RC(0.0)) ? V2(scaled_root, -q->c[0].x) : V2(q->c[1].y, scaled_root);
}

/* sample_sector_between_ellipses, polygon_sampling.glsl:668-762 */
static int g_oracle_biased_psa;
static vec2_t sample_sector_between_ellipses(vec2_t random_numbers, R target_area, vec2_t inner_ellipse,
                                             vec2_t outer_ellipse, vec2_t dir_0, vec2_t dir_1,
                                             uint32_t iteration_count) {
	vec2_t quad_dirs[3];
	quad_dirs[0] = v2_normalize(dir_0);
	quad_dirs[2] = v2_normalize(dir_1);
	quad_dirs[1] = v2_add(quad_dirs[0], quad_dirs[2]);
	R nf[2][3];
	nf[0][0] = get_ellipse_normalized_direction_factor(inner_ellipse, quad_dirs[0]);
	nf[0][1] = get_ellipse_direction_factor(inner_ellipse, quad_dirs[1]);
	nf[0][2] = get_ellipse_normalized_direction_factor(inner_ellipse, quad_dirs[2]);
	nf[1][0] = get_ellipse_normalized_direction_factor(outer_ellipse, quad_dirs[0]);
	nf[1][1] = get_ellipse_direction_factor(outer_ellipse, quad_dirs[1]);
	nf[1][2] = get_ellipse_normalized_direction_factor(outer_ellipse, quad_dirs[2]);
	R sector_areas[2];
	sector_areas[0] = nf[1][0] * nf[1][1] - nf[0][0] * nf[0][1];
	sector_areas[1] = nf[1][1] * nf[1][2] - nf[0][1] * nf[0][2];
	R target_quad_area = mix_fma(-sector_areas[0], sector_areas[1], random_numbers.x);
	int first = target_quad_area <= RC(0.0);
	quad_dirs[2] = first ? quad_dirs[0] : quad_dirs[2];
	nf[0][2] = first ? nf[0][0] : nf[0][2];
	nf[1][2] = first ? nf[1][0] : nf[1][2];
	target_quad_area += first ? sector_areas[0] : -sector_areas[1];
	{
		mat2_t m;
		m.c[0] = quad_dirs[1];
		m.c[1] = quad_dirs[2];
		target_quad_area *= rabs(m2_det(&m));
	}
	vec2_t quad_normals[2];
	quad_normals[0] = v2_add(v2_scale(quad_dirs[1], nf[0][1]), v2_scale(quad_dirs[2], nf[0][2]));
	quad_normals[1] = v2_add(v2_scale(quad_dirs[1], nf[1][1]), v2_scale(quad_dirs[2], nf[1][2]));
	quad_normals[0] = ellipse_transform(inner_ellipse, quad_normals[0]);
	quad_normals[1] = ellipse_transform(outer_ellipse, quad_normals[1]);
	R quad_offsets[2];
	quad_offsets[0] = v2_dot(quad_normals[0], quad_dirs[1]) * nf[0][1];
	quad_offsets[1] = v2_dot(quad_normals[1], quad_dirs[1]) * nf[1][1];
	mat2_t quadratic = outer2(v2_scale(rotate_90(quad_dirs[2]), quad_offsets[1] * nf[1][2]), quad_normals[0]);
	{
		vec2_t col = v2_add(v2_scale(rotate_90(quad_dirs[2]), quad_offsets[0] * nf[0][2]),
		                    v2_scale(quad_normals[0], target_quad_area));
		mat2_t sub = outer2(col, quad_normals[1]);
		quadratic.c[0] = v2_sub(quadratic.c[0], sub.c[0]);
		quadratic.c[1] = v2_sub(quadratic.c[1], sub.c[1]);
	}
	vec2_t current_dir = solve_homogeneous_quadratic(&quadratic);
	if (!g_oracle_biased_psa) {
		R acceptable_error = RC(1.0e-5);
		iteration_count =
		    (rabs(random_numbers.x - RC(0.5)) <= RC(0.5) - acceptable_error) ? iteration_count : 0u;
		R inner_rsqrt_det = get_ellipse_rsqrt_det(inner_ellipse);
		R outer_rsqrt_det = get_ellipse_rsqrt_det(outer_ellipse);
		for (uint32_t i = 0; i != iteration_count; ++i) {
			current_dir = normalize_approx_and_flip(current_dir, quad_dirs[1]);
			vec2_t inner_dir = ellipse_transform(inner_ellipse, current_dir);
			vec2_t outer_dir = ellipse_transform(outer_ellipse, current_dir);
			R det_dirs = rmax(RC(0.0), v2_dot(current_dir, rotate_90(quad_dirs[0])));
			R error = target_area - get_area_between_ellipses_in_sector_from_tangents(
			                            inner_rsqrt_det, det_dirs / (inner_rsqrt_det * v2_dot(quad_dirs[0], inner_dir)),
			                            outer_rsqrt_det, det_dirs / (outer_rsqrt_det * v2_dot(quad_dirs[0], outer_dir)));
			mat2_t a = outer2(v2_sub(inner_dir, outer_dir), rotate_90(current_dir));
			mat2_t b = outer2(v2_scale(inner_dir, RC(2.0) * error), outer_dir);
			quadratic.c[0] = v2_sub(a.c[0], b.c[0]);
			quadratic.c[1] = v2_sub(a.c[1], b.c[1]);
			current_dir = solve_homogeneous_quadratic(&quadratic);
		}
	}
	current_dir = (v2_dot(current_dir, quad_dirs[1]) >= RC(0.0)) ? current_dir : v2_neg(current_dir);
	R inner_factor = RC(1.0) / get_ellipse_direction_factor_rsq(inner_ellipse, current_dir);
	R outer_factor = RC(1.0) / get_ellipse_direction_factor_rsq(outer_ellipse, current_dir);
	return v2_scale(current_dir, R_SQRT(mix_fma(inner_factor, outer_factor, random_numbers.y)));
}

/* sample_projected_solid_angle_polygon, polygon_sampling.glsl:772-828 */
static vec3_t sample_projected_solid_angle_polygon(const projected_solid_angle_polygon_t* p, vec2_t random_numbers,
                                                   uint32_t max_polygon_vertex_count) {
	uint32_t maxp = max_polygon_vertex_count;
	R target = random_numbers.x * p->projected_solid_angle;
	vec3_t sampled_dir;
	vec2_t outer_ellipse = V2(RC(0.0), RC(0.0));
	vec2_t dir_0 = V2(RC(0.0), RC(0.0));
	if (is_central_case(p)) {
		for (uint32_t i = 0; i != maxp; ++i) {
			if (i > 0) target -= p->sector_projected_solid_angles[i - 1];
			outer_ellipse = p->ellipses[i];
			dir_0 = p->vertices[i];
			if ((i >= 2 && i + 1 == p->vertex_count) || target < p->sector_projected_solid_angles[i]) break;
		}
		R sqrt_det = R_SQRT(get_ellipse_det(outer_ellipse));
		R angle = RC(2.0) * target * sqrt_det;
		R sa, ca;
		R_SINCOS(angle, &sa, &ca);
		vec2_t xy = v2_add(v2_scale(dir_0, ca * sqrt_det), v2_scale(rotate_90(ellipse_transform(outer_ellipse, dir_0)), sa));
		xy = v2_scale(xy, R_SQRT(random_numbers.y / get_ellipse_direction_factor_rsq(outer_ellipse, xy)));
		sampled_dir.x = xy.x;
		sampled_dir.y = xy.y;
	} else {
		R sector_psa = RC(0.0);
		vec2_t inner_ellipse = p->inner_ellipse_0;
		vec2_t dir_1 = V2(RC(0.0), RC(0.0));
		for (uint32_t i = 0; i != maxp - 1; ++i) {
			vec2_t vertex_ellipse = p->ellipses[i];
			if (i == 0) {
				outer_ellipse = vertex_ellipse;
			} else {
				target -= p->sector_projected_solid_angles[i - 1];
				int vertex_inner = is_inner_ellipse(vertex_ellipse);
				inner_ellipse = vertex_inner ? vertex_ellipse : inner_ellipse;
				outer_ellipse = vertex_inner ? outer_ellipse : vertex_ellipse;
			}
			dir_0 = p->vertices[i];
			dir_1 = p->vertices[i + 1];
			sector_psa = p->sector_projected_solid_angles[i];
			if ((i >= 1 && i + 2 == p->vertex_count) || target < sector_psa) break;
		}
		random_numbers.x = target / sector_psa;
		vec2_t xy = sample_sector_between_ellipses(random_numbers, target, inner_ellipse, outer_ellipse, dir_0, dir_1, 2u);
		sampled_dir.x = xy.x;
		sampled_dir.y = xy.y;
	}
	sampled_dir.z = R_SQRT(rmax(RC(0.0), R_FMA(-sampled_dir.x, sampled_dir.x, R_FMA(-sampled_dir.y, sampled_dir.y, RC(1.0)))));
	return sampled_dir;
}

/* ------------------------------------------------------------------------ */
/* evaluate_brdf (diffuse and specular), brdfs.glsl:58-93 with
   fresnel_schlick :43-47 */
static vec3_t evaluate_brdf(const shading_data_t* d, vec3_t wi) {
	vec3_t half_vector = v3_normalize(v3_add(wi, d->outgoing));
	R lambert_incoming = v3_dot(d->normal, wi);
	R outgoing_dot_half = v3_dot(d->outgoing, half_vector);
	vec3_t brdf = v3_add(v3_splat(RC(0.0)), d->diffuse_albedo);
	R normal_dot_half = v3_dot(d->normal, half_vector);
	R r2 = d->roughness * d->roughness;
	R ggx = R_FMA(R_FMA(normal_dot_half, r2, -normal_dot_half), normal_dot_half, RC(1.0));
	ggx = r2 / (ggx * ggx);
	R masking = lambert_incoming *
	            R_SQRT(R_FMA(R_FMA(-d->lambert_outgoing, r2, d->lambert_outgoing), d->lambert_outgoing, r2));
	R shadowing = d->lambert_outgoing * R_SQRT(R_FMA(R_FMA(-lambert_incoming, r2, lambert_incoming), lambert_incoming, r2));
	R smith = RC(0.5) / (masking + shadowing);
	R flipped = RC(1.0) - rclamp(outgoing_dot_half, RC(0.0), RC(1.0));
	R flipped_squared = flipped * flipped;
	R t = flipped_squared * flipped * flipped_squared;
	vec3_t f0 = d->fresnel_0;
	vec3_t fresnel = v3_add(f0, v3_scale(v3_sub(v3_splat(RC(1.0)), f0), t));
	R lum = v3_dot(fresnel, V3(RC(0.21263901), RC(0.71516868), RC(0.07219232)));
	brdf = v3_adds(brdf, ggx * smith * lum);
	return v3_scale(brdf, OR_INV_PI);
}

/* get_mis_estimate, shading_pass.frag.glsl:219-269 */
static vec3_t get_mis_estimate(int heuristic, vec3_t integrand, vec3_t sampled_weight, R sampled_density,
                               vec3_t other_weight, R other_density, R visibility_estimate) {
	switch (heuristic) {
	case ORACLE_MIS_BALANCE:
		return v3_scale(integrand, RC(1.0) / (sampled_density + other_density));
	case ORACLE_MIS_POWER:
		return v3_scale(integrand, sampled_density /
		                               (sampled_density * sampled_density + other_density * other_density));
	case ORACLE_MIS_WEIGHTED: {
		vec3_t ws = v3_add(v3_scale(sampled_weight, sampled_density), v3_scale(other_weight, other_density));
		return v3_div(v3_mul(sampled_weight, integrand), ws);
	}
	case ORACLE_MIS_OPTIMAL: {
		R balance = RC(1.0) / (sampled_density + other_density);
		vec3_t ws = v3_add(v3_scale(sampled_weight, sampled_density), v3_scale(other_weight, other_density));
		return v3_add(v3_scale(sampled_weight, visibility_estimate),
		              v3_scale(v3_sub(integrand, v3_scale(ws, visibility_estimate)), balance));
	}
	default: {
		R balance = RC(1.0) / (sampled_density + other_density);
		vec3_t ws = v3_add(v3_scale(sampled_weight, sampled_density), v3_scale(other_weight, other_density));
		vec3_t weighted = v3_div(sampled_weight, ws);
		vec3_t mixed = v3_splat(R_FMA(-visibility_estimate, balance, balance));
		mixed = v3_fma(v3_splat(visibility_estimate), weighted, mixed);
		return v3_mul(mixed, integrand);
	}
	}
}

/* ------------------------------------------------------------------------ */
/* Scene access */
typedef struct {
	R radiance[3];
	R plane[4];
	uint32_t vertex_count;
	vec3_t v[OR_MAXV];
} light_t;

static void load_light(const oracle_scene_t* s, int index, light_t* l) {
	const float* f = s->lights + (size_t) index * (size_t) (12 + 4 * s->max_light_vertex_count);
	for (int i = 0; i != 3; ++i) l->radiance[i] = (R) f[i];
	for (int i = 0; i != 4; ++i) l->plane[i] = (R) f[4 + i];
	memcpy(&l->vertex_count, f + 8, 4);
	for (int j = 0; j != s->max_light_vertex_count; ++j) l->v[j] = V3((R) f[12 + 4 * j], (R) f[13 + 4 * j], (R) f[14 + 4 * j]);
}

/* Any-hit shadow query: the project's ray/triangle test, brute force or
   through the scene's BVH (same answer: the boxes are conservative). */
static int ray_triangle(vec3_t o, vec3_t d, const float* t, R t_min, R t_max) {
	vec3_t v0 = V3((R) t[0], (R) t[1], (R) t[2]), e1 = V3((R) t[4], (R) t[5], (R) t[6]);
	vec3_t e2 = V3((R) t[8], (R) t[9], (R) t[10]);
	vec3_t p = v3_cross(d, e2);
	R det = v3_dot(e1, p);
	if (!(det != RC(0.0))) return 0;
	R inv = RC(1.0) / det;
	vec3_t sv = v3_sub(o, v0);
	R u = v3_dot(sv, p) * inv;
	if (!(u >= RC(0.0) && u <= RC(1.0))) return 0;
	vec3_t q = v3_cross(sv, e1);
	R v = v3_dot(d, q) * inv;
	if (!(v >= RC(0.0) && u + v <= RC(1.0))) return 0;
	R tt = v3_dot(e2, q) * inv;
	return tt >= t_min && tt <= t_max;
}

/* Traversal tallies of the op-counting build (no-ops elsewhere). */
#ifndef ORACLE_COUNT_BOX
#define ORACLE_COUNT_BOX() ((void) 0)
#define ORACLE_COUNT_TRIANGLE() ((void) 0)
#endif

static int any_hit(const oracle_scene_t* s, vec3_t o, vec3_t d, R t_min, R t_max) {
	if (s->triangle_count == 0) return 0;
	if (!s->bvh_nodes) {
		for (int k = 0; k != s->triangle_count; ++k)
			if (ray_triangle(o, d, s->triangles + 12 * (size_t) k, t_min, t_max)) return 1;
		return 0;
	}
	/* Stack traversal of the binary BVH: node = {bmin xyz, left_or_first,
	   bmax xyz, count}; count == 0 marks an interior node whose children are
	   left and left + 1. */
	R inv_d[3] = {RC(1.0) / d.x, RC(1.0) / d.y, RC(1.0) / d.z};
	R org[3] = {o.x, o.y, o.z};
	int32_t stack[64];
	int sp = 0;
	stack[sp++] = 0;
	while (sp) {
		const float* n = s->bvh_nodes + 8 * (size_t) stack[--sp];
		ORACLE_COUNT_BOX();
		R lo = t_min, hi = t_max;
		for (int a = 0; a != 3; ++a) {
			R t0 = ((R) n[a] - org[a]) * inv_d[a];
			R t1 = ((R) n[4 + a] - org[a]) * inv_d[a];
			R tn = t0 < t1 ? t0 : t1, tf = t0 < t1 ? t1 : t0;
			if (tn == tn && tn > lo) lo = tn;
			if (tf == tf && tf < hi) hi = tf;
		}
		if (!(lo <= hi)) continue;
		int32_t first, count;
		memcpy(&first, n + 3, 4);
		memcpy(&count, n + 7, 4);
		if (count == 0) {
			if (sp + 2 > 64) return 1; /* cannot happen for the builder's depth bound */
			stack[sp++] = first + 1;
			stack[sp++] = first;
		} else {
			for (int k = 0; k != count; ++k) {
				ORACLE_COUNT_TRIANGLE();
				if (ray_triangle(o, d, s->triangles + 12 * (size_t) (first + k), t_min, t_max)) return 1;
			}
		}
	}
	return 0;
}

/* get_polygon_visibility, shading_pass.frag.glsl:112-129 */
static int get_polygon_visibility(const oracle_scene_t* s, int visibility, vec3_t dir, vec3_t p, const light_t* l) {
	if (!visibility) return 0;
	if (s->triangle_count == 0) return 1;
	R max_t = -plane_dot(p, l->plane) / (dir.x * l->plane[0] + dir.y * l->plane[1] + dir.z * l->plane[2]);
	max_t -= RC(1e-3);
	R min_t = RC(1.0e-3);
	return !any_hit(s, p, dir, min_t, max_t);
}

/* Flip the y row of world_to_shading_space when the shading point is behind
   the light's plane, shading_pass.frag.glsl:300-304 and :424-428. */
static void side_flip(ltc_coefficients_t* ltc, const shading_data_t* sd, const light_t* l) {
	R side = plane_dot(sd->position, l->plane);
	for (int i = 0; i != 4; ++i)
		ltc->world_to_shading_space.c[i].y = (side < RC(0.0)) ? -ltc->world_to_shading_space.c[i].y
		                                                      : ltc->world_to_shading_space.c[i].y;
}

typedef struct {
	const oracle_scene_t* scene;
	const oracle_settings_t* settings;
	uint32_t maxv, maxp;
} ctx_t;

/* LTC_CP branch of evaluate_polygonal_light_shading (the RIS target),
   shading_pass.frag.glsl:421-456 */
static vec3_t ltc_cp_target(const ctx_t* c, const shading_data_t* sd, ltc_coefficients_t ltc, const light_t* l) {
	side_flip(&ltc, sd, l);
	vec3_t result = v3_splat(RC(0.0));
	vec3_t verts[OR_MAXP];
	for (uint32_t i = 0; i != c->maxp; ++i) verts[i] = V3(RC(0.0), RC(0.0), RC(1.0));
	for (uint32_t i = 0; i != c->maxv; ++i) verts[i] = m43_mul_point(&ltc.world_to_shading_space, l->v[i]);
	uint32_t vc = clip_polygon(l->vertex_count, verts, c->maxp, c->settings->reference_slots);
	vec3_t radiance = V3(l->radiance[0], l->radiance[1], l->radiance[2]);
	vec3_t diffuse = v3_splat(RC(0.0));
	if (vc > 0)
		diffuse = v3_mul(v3_scale(sd->diffuse_albedo, calculate_ltc(vc, verts, c->maxp, c->settings->reference_slots)),
		                 radiance);
	result = v3_add(result, diffuse);
	mat4x3_t w2c = m3_mul_m43(&ltc.shading_to_cosine_space, &ltc.world_to_shading_space);
	for (uint32_t i = 0; i != c->maxp; ++i) verts[i] = V3(RC(0.0), RC(0.0), RC(1.0));
	for (uint32_t i = 0; i != c->maxv; ++i) verts[i] = m43_mul_point(&w2c, l->v[i]);
	vc = clip_polygon(l->vertex_count, verts, c->maxp, c->settings->reference_slots);
	vec3_t ggx = v3_splat(RC(0.0));
	if (vc > 0)
		ggx = v3_mul(v3_splat(calculate_ltc(vc, verts, c->maxp, c->settings->reference_slots) * ltc.albedo), radiance);
	return v3_add(result, ggx);
}

/* Prepares the diffuse (shading space) and specular (cosine space) PSA
   polygons; shared by evaluate_polygonal_light_shading_peters
   (shading_pass.frag.glsl:309-337) and the PSA branch (:462-490).
   Returns 0 if the polygon is below the horizon. */
static int prepare_both(const ctx_t* c, const ltc_coefficients_t* ltc, const light_t* l,
                        projected_solid_angle_polygon_t* polygon_diffuse,
                        projected_solid_angle_polygon_t* polygon_specular) {
	for (uint32_t i = 0; i != 2; ++i) {
		mat4x3_t w2l = (i == 0) ? ltc->world_to_shading_space
		                        : m3_mul_m43(&ltc->shading_to_cosine_space, &ltc->world_to_shading_space);
		if (i > 0) *polygon_diffuse = *polygon_specular;
		vec3_t verts[OR_MAXP];
		for (uint32_t j = 0; j != c->maxp; ++j) verts[j] = V3(RC(0.0), RC(0.0), RC(1.0));
		for (uint32_t j = 0; j != c->maxv; ++j) verts[j] = m43_mul_point(&w2l, l->v[j]);
		uint32_t vc = clip_polygon(l->vertex_count, verts, c->maxp, c->settings->reference_slots);
		if (vc == 0 && i == 0) return 0;
		if (vc == 0) {
			polygon_specular->projected_solid_angle = RC(0.0);
			break;
		}
		prepare_projected_solid_angle_polygon_sampling(polygon_specular, vc, verts, c->maxp);
	}
	return 1;
}

/* evaluate_polygonal_light_shading_peters (final_shadowed = 1, the LTC_CP
   final estimator, shading_pass.frag.glsl:292-397) and the PSA branch of
   evaluate_polygonal_light_shading (final_shadowed = 0, :458-550). */
static vec3_t psa_mis_shade(const ctx_t* c, const shading_data_t* sd, ltc_coefficients_t ltc, const light_t* l,
                            uint32_t* seed, int peters, int visibility_in) {
	const oracle_settings_t* st = c->settings;
	vec3_t result = v3_splat(RC(0.0));
	side_flip(&ltc, sd, l);
	projected_solid_angle_polygon_t polygon_diffuse, polygon_specular;
	if (!prepare_both(c, &ltc, l, &polygon_diffuse, &polygon_specular)) return result;
	if (polygon_diffuse.projected_solid_angle == RC(0.0)) return result;
	R specular_weight = ltc.albedo * polygon_specular.projected_solid_angle;
	vec3_t diffuse_albedo = v3_max(sd->diffuse_albedo, v3_splat(RC(0.01)));
	vec3_t diffuse_weight = v3_scale(diffuse_albedo, polygon_diffuse.projected_solid_angle);
	uint32_t technique_count = (polygon_specular.projected_solid_angle > RC(0.0)) ? 2u : 1u;
	R rcp_d = RC(1.0) / polygon_diffuse.projected_solid_angle;
	R rcp_s = RC(1.0) / polygon_specular.projected_solid_angle;
	vec3_t specular_weight_rgb = v3_splat(specular_weight);
	vec3_t radiance = V3(l->radiance[0], l->radiance[1], l->radiance[2]);
	if (st->mis_heuristic == ORACLE_MIS_OPTIMAL) {
		vec3_t radiance_over_pi = v3_scale(radiance, OR_INV_PI);
		diffuse_weight = v3_mul(diffuse_weight, radiance_over_pi);
		specular_weight_rgb = v3_mul(specular_weight_rgb, radiance_over_pi);
	}
	for (int i = 0; i != st->sample_count; ++i) {
		vec3_t dir_d = sample_projected_solid_angle_polygon(&polygon_diffuse, get_noise_2(seed), c->maxp);
		vec3_t dir_s = V3(RC(0.0), RC(0.0), RC(1.0));
		if (polygon_specular.projected_solid_angle > RC(0.0)) {
			dir_s = sample_projected_solid_angle_polygon(&polygon_specular, get_noise_2(seed), c->maxp);
			dir_s = v3_normalize(m3_mul(&ltc.cosine_to_shading_space, dir_s));
		}
		for (uint32_t j = 0; j != technique_count; ++j) {
			vec3_t dir = (j == 0) ? dir_d : dir_s;
			if (dir.z <= RC(0.0)) continue;
			R diffuse_density = dir.z * rcp_d;
			R specular_density = evaluate_ltc_density(&ltc, dir, rcp_s);
			vec3_t world_dir = m43_transpose_mul(&ltc.world_to_shading_space, dir);
			vec3_t integrand;
			int visibility;
			if (peters) {
				/* get_polygon_radiance_visibility_brdf_product, :188-197 */
				visibility = v3_dot(sd->normal, world_dir) > RC(0.0);
				visibility = get_polygon_visibility(c->scene, visibility, world_dir, sd->position, l);
				vec3_t rb = visibility ? v3_mul(radiance, evaluate_brdf(sd, world_dir)) : v3_splat(RC(0.0));
				integrand = v3_scale(rb, dir.z);
			} else {
				/* get_polygon_radiance_brdf_product, :200-207 */
				int curr_visibility = visibility_in;
				int side_visibility = v3_dot(sd->normal, world_dir) > RC(0.0);
				vec3_t rb;
				if (!side_visibility) {
					rb = v3_splat(RC(0.0));
				} else {
					curr_visibility = get_polygon_visibility(c->scene, curr_visibility, world_dir, sd->position, l);
					curr_visibility = side_visibility && curr_visibility;
					rb = v3_mul(radiance, evaluate_brdf(sd, world_dir));
				}
				integrand = v3_scale(rb, dir.z);
				integrand = (curr_visibility || !visibility_in) ? integrand : v3_splat(RC(0.0));
				visibility = 1;
			}
			if (j == 0 && polygon_specular.projected_solid_angle <= RC(0.0))
				result = v3_add(result, visibility ? v3_scale(integrand, RC(1.0) / diffuse_density) : v3_splat(RC(0.0)));
			else if (j == 0)
				result = v3_add(result, get_mis_estimate(st->mis_heuristic, integrand, diffuse_weight, diffuse_density,
				                                         specular_weight_rgb, specular_density,
				                                         (R) st->mis_visibility_estimate));
			else
				result = v3_add(result, get_mis_estimate(st->mis_heuristic, integrand, specular_weight_rgb,
				                                         specular_density, diffuse_weight, diffuse_density,
				                                         (R) st->mis_visibility_estimate));
		}
	}
	return v3_scale(result, RC(1.0) / (R) st->sample_count);
}

/* sample_area_polygon_turk, polygon_sampling_related_work.glsl:35-43.  Like
   the reference, it samples the triangle of vertices 0, 1 and 2 (Turk's
   square-root parametrisation), not a fan over the whole polygon. */
static vec3_t sample_area_polygon_turk(const light_t* l, vec2_t random_numbers) {
	R sqrt_random_0 = R_SQRT(random_numbers.x);
	R b0 = RC(1.0) - sqrt_random_0, b1 = sqrt_random_0 * random_numbers.y;
	R b2 = R_FMA(-sqrt_random_0, random_numbers.y, sqrt_random_0);
	return v3_add(v3_add(v3_scale(l->v[0], b0), v3_scale(l->v[1], b1)), v3_scale(l->v[2], b2));
}

/* get_polygon_area, shading_pass.frag.glsl:146-150: the area of the triangle
   of vertices 0, 1 and 2 */
static R get_polygon_area(const light_t* l) {
	vec3_t v1 = v3_sub(l->v[1], l->v[0]);
	vec3_t v2 = v3_sub(l->v[2], l->v[0]);
	return v3_length(cross_stable(v1, v2)) / RC(2.0);
}

/* get_area_sample_density, polygon_sampling_related_work.glsl:57-64 */
static R get_area_sample_density(vec3_t* out_dir, vec3_t light_sample, vec3_t shading_position,
                                  vec3_t light_normal, R light_area) {
	vec3_t dir = v3_sub(light_sample, shading_position);
	R distance_squared = v3_dot(dir, dir);
	R normalization = RC(1.0) / R_SQRT(distance_squared);
	dir = v3_scale(dir, normalization);
	*out_dir = dir;
	R projected_area = rabs(v3_dot(light_normal, dir)) * light_area;
	return distance_squared / projected_area;
}

/* The SAMPLE_POLYGON_AREA_TURK branch of evaluate_polygonal_light_shading
   (shading_pass.frag.glsl:411-418) with get_polygonal_light_mis_estimate
   (:281-287) and get_polygon_radiance_brdf_product (:200-207).  With
   eval_only the stored light_sample is evaluated and no noise is drawn;
   *visibility is traced only when it comes in true. */
static vec3_t area_turk_shade(const ctx_t* c, const shading_data_t* sd, const light_t* l, vec3_t* light_sample,
                              int eval_only, int* visibility, uint32_t* seed) {
	const oracle_settings_t* st = c->settings;
	vec3_t result = v3_splat(RC(0.0));
	vec3_t radiance = V3(l->radiance[0], l->radiance[1], l->radiance[2]);
	vec3_t light_normal = V3(l->plane[0], l->plane[1], l->plane[2]);
	for (int i = 0; i != st->sample_count; ++i) {
		if (!eval_only) *light_sample = sample_area_polygon_turk(l, get_noise_2(seed));
		vec3_t dir;
		R density = get_area_sample_density(&dir, *light_sample, sd->position, light_normal, get_polygon_area(l));
		R lambert = v3_dot(sd->normal, dir);
		vec3_t rb = v3_splat(RC(0.0));
		if (v3_dot(sd->normal, dir) > RC(0.0)) {
			*visibility = get_polygon_visibility(c->scene, *visibility, dir, sd->position, l);
			rb = v3_mul(radiance, evaluate_brdf(sd, dir));
		}
		result = v3_add(result, (density > RC(0.0)) ? v3_scale(rb, lambert / density) : v3_splat(RC(0.0)));
	}
	return v3_scale(result, RC(1.0) / (R) st->sample_count);
}

/* ------------------------------------------------------------------------ */
/* Cluster proposal of the RIS candidates.  Not in the reference (which draws
   candidates uniformly, shading_pass.frag.glsl:728-733): restates the CUDA
   path's proposal_kernel in FP32 whatever R is, including the order of its
   warp-wide sums (32 lanes, each summing a block of clusters, then an
   inclusive Hillis-Steele scan over the lanes). */
#define OR_MAX_CLUSTERS 1024
#define OR_MAX_CANDIDATES 4096
typedef struct {
	int32_t light;
	float pdf;
} proposal_candidate_t;

static float noise_f32(uint32_t* seed) {
	*seed = 1664525u * *seed + 1013904223u;
	return (float) *seed * 2.3283064365386962890625e-10f;
}

/* cluster_weight: power times a cosine bound over the clamped distance cubed */
static float cluster_weight_f32(const float* bound, float power, const float* x, const float* n) {
	const float v0 = bound[0] - x[0], v1 = bound[1] - x[1], v2 = bound[2] - x[2];
	const float d2 = v0 * v0 + v1 * v1 + v2 * v2;
	const float h = n[0] * v0 + n[1] * v1 + n[2] * v2;
	const float rr = bound[3] * bound[3];
	const float dd = d2 > rr ? d2 : rr;
	float up = h + bound[3];
	up = up > 0.0f ? up : 0.0f;
	return (power * up) / (dd * sqrtf(dd));
}

static void proposal_draw(const oracle_scene_t* s, const oracle_settings_t* st, const float* x, const float* n,
                          uint32_t px, uint32_t py, uint32_t width, proposal_candidate_t* out) {
	const int k_count = s->cluster_count, n_lights = s->light_count;
	const int per_lane = (k_count + 31) / 32;
	const float a = st->proposal_uniform_fraction;
	float cdf[OR_MAX_CLUSTERS], incl[32], next[32];
	for (int lane = 0; lane != 32; ++lane) {
		float local = 0.0f;
		for (int j = 0; j != per_lane; ++j) {
			const int k = lane * per_lane + j;
			if (k >= k_count) break;
			const int empty = s->cluster_offsets[k + 1] == s->cluster_offsets[k];
			const float w = empty ? 0.0f : cluster_weight_f32(s->cluster_bounds + 4 * k, s->cluster_power[k], x, n);
			local += w;
			cdf[k] = local;
		}
		incl[lane] = local;
	}
	for (int d = 1; d < 32; d <<= 1) {
		for (int l = 0; l != 32; ++l) next[l] = (l >= d) ? incl[l] + incl[l - d] : incl[l];
		for (int l = 0; l != 32; ++l) incl[l] = next[l];
	}
	const float total = incl[31];
	for (int lane = 0; lane != 32; ++lane) {
		const float excl = lane == 0 ? 0.0f : incl[lane - 1];
		for (int j = 0; j != per_lane; ++j) {
			const int k = lane * per_lane + j;
			if (k >= k_count) break;
			cdf[k] = excl + cdf[k];
		}
	}
	const int proposal = total > 0.0f && total <= 3.0e38f;
	const uint32_t base = get_noise_accessor(px, py, width, st->random_number_proposal);
	for (int c = 0; c != st->candidate_count; ++c) {
		uint32_t sd = base ^ ((uint32_t) c * 0x9E3779B9u);
		const float u0 = noise_f32(&sd), u1 = noise_f32(&sd), u2 = noise_f32(&sd);
		int light;
		if (!proposal || u0 < a) {
			light = (int) (u1 * (float) n_lights);
			if (light > n_lights - 1) light = n_lights - 1;
		} else {
			const float t = u1 * total;
			int lo = 0, hi = k_count - 1;
			while (lo < hi) {
				const int mid = (lo + hi) >> 1;
				if (cdf[mid] > t)
					hi = mid;
				else
					lo = mid + 1;
			}
			while (lo > 0 && s->cluster_offsets[lo + 1] == s->cluster_offsets[lo]) --lo;
			const uint32_t first = s->cluster_offsets[lo], size = s->cluster_offsets[lo + 1] - first;
			uint32_t j = (uint32_t) (u2 * (float) size);
			if (j > size - 1) j = size - 1;
			light = (int) (first + j);
		}
		float pdf = 1.0f / (float) n_lights;
		if (proposal) {
			const uint32_t k = s->light_cluster[light];
			const float mass = cdf[k] - (k > 0 ? cdf[k - 1] : 0.0f);
			const uint32_t size = s->cluster_offsets[k + 1] - s->cluster_offsets[k];
			pdf = a / (float) n_lights + ((1.0f - a) * (mass / total)) / (float) size;
		}
		out[c].light = light;
		out[c].pdf = pdf;
	}
}

/* Per-pixel body of the shading pass, shading_pass.frag.glsl:674-770 */
static void shade_pixel(const ctx_t* c, const shading_data_t* sd, uint32_t seed, R out_rgb[3],
                        oracle_reservoir_t* out_res, const proposal_candidate_t* candidates) {
	const oracle_settings_t* st = c->settings;
	const oracle_scene_t* s = c->scene;
	int n = s->light_count;
	vec3_t final_color = v3_splat(RC(0.0));
	R fresnel_luminance = v3_dot(sd->fresnel_0, V3(RC(0.2126), RC(0.7152), RC(0.0722)));
	ltc_coefficients_t ltc =
	    get_ltc_coefficients(s, fresnel_luminance, sd->roughness, sd->position, sd->normal, sd->outgoing);
	int peters = st->polygon_sampling_technique == ORACLE_TECHNIQUE_LTC_CP;
	int area_turk = st->polygon_sampling_technique == ORACLE_TECHNIQUE_AREA_TURK;
	/* The sampled light position of the area technique, carried from
	   candidate to candidate and stored in the reservoir (:704, 735). */
	vec3_t light_sample = v3_splat(RC(0.0));
	if (out_res) {
		out_res->light_index = -1;
		out_res->w_sum = 0.0;
		out_res->sample_value = 0.0;
	}
	if (st->light_sampling == ORACLE_LIGHT_UNIFORM) {
		for (int i = 0; i != st->light_samples; ++i) {
			int light_idx = (int) (get_noise_1(&seed) * (R) n);
			if (light_idx > n - 1) light_idx = n - 1;
			light_t l;
			load_light(s, light_idx, &l);
			int visibility = 1;
			vec3_t shade = area_turk ? area_turk_shade(c, sd, &l, &light_sample, 0, &visibility, &seed)
			                         : psa_mis_shade(c, sd, ltc, &l, &seed, peters, 1);
			vec3_t result = v3_scale(shade, (R) n);
			R ls = (R) st->light_samples;
			result = V3(result.x / ls, result.y / ls, result.z / ls);
			final_color = v3_add(final_color, v3_scale(result, visibility ? RC(1.0) : RC(0.0)));
			if (out_res && i == 0) out_res->light_index = light_idx;
		}
	} else {
		for (int j = 0; j != st->light_samples; ++j) {
			R w_sum = RC(0.0), sample_value = RC(0.0);
			int res_index = -1;
			vec3_t res_light_sample = v3_splat(RC(0.0));
			int m = st->candidate_count;
			for (int i = 0; i != m; ++i) {
				int light_idx = (int) (get_noise_1(&seed) * (R) n);
				if (light_idx > n - 1) light_idx = n - 1;
				R p = RC(1.0) / (R) n;
				if (candidates) {
					light_idx = candidates[i].light;
					p = (R) candidates[i].pdf;
				}
				light_t l;
				load_light(s, light_idx, &l);
				vec3_t color;
				if (peters) {
					color = ltc_cp_target(c, sd, ltc, &l);
				} else if (area_turk) {
					int dummy_visibility = 0;
					color = area_turk_shade(c, sd, &l, &light_sample, 0, &dummy_visibility, &seed);
				} else {
					color = psa_mis_shade(c, sd, ltc, &l, &seed, 0, 0);
				}
				R p_hat = v3_length(color);
				R w = p_hat / p;
				/* insert_in_reservoir, reservoir.glsl:34-41 */
				R rnd = get_noise_1(&seed);
				w_sum += w;
				if (w > RC(0.0) && rnd < (w / w_sum)) {
					res_index = light_idx;
					res_light_sample = light_sample;
					sample_value = p_hat;
				}
			}
			if (out_res && j == 0) {
				out_res->light_index = res_index;
				out_res->w_sum = (double) w_sum;
				out_res->sample_value = (double) sample_value;
			}
			if (res_index >= 0) {
				light_t l;
				load_light(s, res_index, &l);
				int visibility = 1;
				vec3_t color = area_turk ? area_turk_shade(c, sd, &l, &res_light_sample, 1, &visibility, &seed)
				                         : psa_mis_shade(c, sd, ltc, &l, &seed, peters, 1);
				R p_hat = sample_value;
				R W = w_sum / ((R) m * p_hat);
				/* The area technique has no p_hat == 0 guard but multiplies
				   by the traced visibility (:749-756). */
				if (!area_turk && p_hat == RC(0.0)) W = RC(0.0);
				if (area_turk) W = W * (visibility ? RC(1.0) : RC(0.0));
				vec3_t cw = v3_scale(color, W);
				R ls = (R) st->light_samples;
				final_color = v3_add(final_color, V3(cw.x / ls, cw.y / ls, cw.z / ls));
			}
		}
	}
	/* NaN or infinity becomes pink, shading_pass.frag.glsl:764-767 */
	if (final_color.x != final_color.x || final_color.y != final_color.y || final_color.z != final_color.z ||
	    R_ISINF(final_color.x) || R_ISINF(final_color.y) || R_ISINF(final_color.z))
		final_color = V3(RC(1.0), RC(0.0), RC(0.8));
	out_rgb[0] = final_color.x;
	out_rgb[1] = final_color.y;
	out_rgb[2] = final_color.z;
}

/* Shades pixel i = y * width + x of the G-buffer (its own noise seed from
   x, y and the frame's random number, noise_utility.glsl:77-84), writing its
   colour to out_rgb[0..2] and, if res is not NULL, its reservoir. */
static void render_pixel(const ctx_t* c, const oracle_gbuffer_t* gbuffer, uint32_t random_number_x, size_t i,
                         ORACLE_OUT_T* out_rgb, oracle_reservoir_t* res) {
	const oracle_scene_t* scene = c->scene;
	const oracle_settings_t* settings = c->settings;
	const size_t np = (size_t) gbuffer->width * gbuffer->height;
	const float* g = gbuffer->planes;
	const uint32_t x = (uint32_t) (i % (size_t) gbuffer->width), y = (uint32_t) (i / (size_t) gbuffer->width);
	R rgb[3] = {RC(0.0), RC(0.0), RC(0.0)};
	if (gbuffer->primitive && gbuffer->primitive[i] == 0xffffffffu) {
		if (res) {
			res->light_index = -1;
			res->w_sum = 0.0;
			res->sample_value = 0.0;
		}
	} else {
		shading_data_t sd;
		sd.position = V3((R) g[0 * np + i], (R) g[1 * np + i], (R) g[2 * np + i]);
		sd.normal = V3((R) g[3 * np + i], (R) g[4 * np + i], (R) g[5 * np + i]);
		sd.outgoing = V3((R) g[6 * np + i], (R) g[7 * np + i], (R) g[8 * np + i]);
		sd.lambert_outgoing = (R) g[9 * np + i];
		sd.diffuse_albedo = V3((R) g[10 * np + i], (R) g[11 * np + i], (R) g[12 * np + i]);
		sd.fresnel_0 = V3((R) g[13 * np + i], (R) g[14 * np + i], (R) g[15 * np + i]);
		sd.roughness = (R) g[16 * np + i];
		uint32_t seed = get_noise_accessor(x, y, (uint32_t) gbuffer->width, random_number_x);
		proposal_candidate_t candidates[OR_MAX_CANDIDATES];
		const int proposal = settings->proposal && settings->light_sampling == ORACLE_LIGHT_RESERVOIR &&
		                     scene->cluster_count > 0 && settings->candidate_count <= OR_MAX_CANDIDATES;
		if (proposal) {
			const float xp[3] = {g[0 * np + i], g[1 * np + i], g[2 * np + i]};
			const float nn[3] = {g[3 * np + i], g[4 * np + i], g[5 * np + i]};
			proposal_draw(scene, settings, xp, nn, x, y, (uint32_t) gbuffer->width, candidates);
		}
		shade_pixel(c, &sd, seed, rgb, res, proposal ? candidates : NULL);
	}
	out_rgb[0] = (ORACLE_OUT_T) rgb[0];
	out_rgb[1] = (ORACLE_OUT_T) rgb[1];
	out_rgb[2] = (ORACLE_OUT_T) rgb[2];
}

static int make_ctx(ctx_t* c, const oracle_scene_t* scene, const oracle_settings_t* settings) {
	c->scene = scene;
	c->settings = settings;
	c->maxv = (uint32_t) scene->max_light_vertex_count;
	c->maxp = c->maxv + 1;
	if (c->maxv < 3 || c->maxv > OR_MAXV || scene->light_count <= 0) return 1;
	g_oracle_fast_atan = settings->fast_atan;
	g_oracle_biased_psa = settings->polygon_sampling_technique == ORACLE_TECHNIQUE_PSA_BIASED;
	return 0;
}

/* Renders rows [row_begin, row_end) of one frame. */
int OR_EXPORT(oracle_render)(const oracle_scene_t* scene, const oracle_settings_t* settings,
                             const oracle_gbuffer_t* gbuffer, uint32_t random_number_x, int row_begin, int row_end,
                             ORACLE_OUT_T* out_rgb, oracle_reservoir_t* out_reservoirs) {
	ctx_t c;
	if (make_ctx(&c, scene, settings)) return 1;
	for (int y = row_begin; y < row_end; ++y) {
		for (int x = 0; x != gbuffer->width; ++x) {
			const size_t i = (size_t) y * gbuffer->width + x;
			render_pixel(&c, gbuffer, random_number_x, i, out_rgb + 3 * i, out_reservoirs ? out_reservoirs + i : NULL);
		}
	}
	return 0;
}

/* Renders the listed pixels of one frame (indices y * width + x into the
   full G-buffer), each with the noise seed of its own position, so that a
   sample of a large frame reproduces that frame's pixels exactly.  Output k
   (out_rgb[3k..3k+2], out_reservoirs[k]) belongs to pixels[k]. */
int OR_EXPORT(oracle_render_pixels)(const oracle_scene_t* scene, const oracle_settings_t* settings,
                                    const oracle_gbuffer_t* gbuffer, uint32_t random_number_x,
                                    const uint32_t* pixels, size_t begin, size_t end, ORACLE_OUT_T* out_rgb,
                                    oracle_reservoir_t* out_reservoirs) {
	ctx_t c;
	if (make_ctx(&c, scene, settings)) return 1;
	const size_t np = (size_t) gbuffer->width * gbuffer->height;
	for (size_t k = begin; k < end; ++k) {
		if (pixels[k] >= np) return 1;
		render_pixel(&c, gbuffer, random_number_x, pixels[k], out_rgb + 3 * k, out_reservoirs ? out_reservoirs + k : NULL);
	}
	return 0;
}
