// shade_kernel.cuh - the per-pixel shading kernel and the shadow-ray kernel.
// Instantiated by shade_exact.cu and shade_fast.cu with one numerics policy.
// Restates upstream risltc routines (GPLv3): see NOTICE.
#pragma once
#include "shade_psa.cuh"

namespace risltc {

enum : uint32_t {
	kErrorTraversalLimit = 1u << 0,
	kErrorVertexCount = 1u << 1,
};

struct ShadeParams {
	SceneView scene;
	const float* gbuffer;        // 17 planes
	const uint32_t* primitive;   // may be null
	uint32_t width, height;
	int technique;               // sample_polygon_technique_t
	int light_sampling;          // light_sampling_strategies_t
	int mis_heuristic;
	int candidate_count;
	int sample_count;
	int light_samples;
	float mis_visibility_estimate;
	int fast_atan;
	int shadows;
	uint32_t noise_seed;         // noise_table_t::random_seed of the first frame
	uint32_t animate;
	uint32_t frame_count;
	float* out_rgb;              // may be null
	double* accum;               // may be null
	risltc_reservoir_t* reservoirs;  // may be null
	uint32_t* error;             // error bits (atomicOr)
};

// Any-hit traversal of the BVH in its child-pair layout (SceneView::pairs).
// Each step does one unit of work: test one triangle of the current leaf, or
// visit one inner node (load both children's boxes, continue with a hit
// child, keep the other on the stack).  Lanes of a warp thus run the same
// short step whatever part of the tree they are in.  A triangle is tested
// exactly when every box on its path is hit, so the answer equals a
// brute-force test of all triangles given conservative boxes; only the order
// of the tests differs, which an any-hit query does not see.
struct TraceRay {
	f3 o, d;
	float inv[3];
	float t_min, t_max;
	int32_t node;     // next reference to visit (kNoNode: pop the stack)
	uint32_t leaf_first, leaf_left;  // triangles of the current leaf still to test
	int sp;
	uint32_t visits;
	bool minmax;      // no slab product can be NaN: the min/max form applies
};

enum : int { kTraceContinue = 0, kTraceMiss = 1, kTraceHit = 2 };
constexpr int32_t kNoNode = INT32_MIN;

// Slab test of one box against the ray's [t_min, t_max]; *entry gets the
// entry distance.  Per axis t0 = (bmin - o) * inv, t1 = (bmax - o) * inv;
// the interval is narrowed by min(t0, t1) and max(t0, t1), an endpoint that
// is NaN leaving its side unchanged.  When no product can be NaN (finite box
// and origin, finite non-zero inv) the same result comes from IEEE min/max
// instructions, used then.
RL_DEV bool ray_box(const TraceRay& r, float4 lo, float4 hi, float* entry) {
	const float bmin[3] = {lo.x, lo.y, lo.z}, bmax[3] = {hi.x, hi.y, hi.z};
	const float org[3] = {r.o.x, r.o.y, r.o.z};
	float t0s = r.t_min, t1s = r.t_max;
	if (r.minmax) {
#pragma unroll
		for (int ax = 0; ax != 3; ++ax) {
			const float t0 = (bmin[ax] - org[ax]) * r.inv[ax];
			const float t1 = (bmax[ax] - org[ax]) * r.inv[ax];
			t0s = fmaxf(t0s, fminf(t0, t1));
			t1s = fminf(t1s, fmaxf(t0, t1));
		}
	} else {
#pragma unroll
		for (int ax = 0; ax != 3; ++ax) {
			const float t0 = (bmin[ax] - org[ax]) * r.inv[ax];
			const float t1 = (bmax[ax] - org[ax]) * r.inv[ax];
			const float tn = t0 < t1 ? t0 : t1, tf = t0 < t1 ? t1 : t0;
			if (tn == tn && tn > t0s) t0s = tn;
			if (tf == tf && tf < t1s) t1s = tf;
		}
	}
	*entry = t0s;
	return t0s <= t1s;
}

// Moller-Trumbore with the triangle stored as {v0, e1, e2}; a hit with t in
// [t_min, t_max] counts.
template <class P> RL_DEV bool ray_triangle(const TraceRay& r, const float4* t) {
	const float4 q0 = __ldg(t), q1 = __ldg(t + 1), q2 = __ldg(t + 2);
	const f3 v0 = mk3(q0.x, q0.y, q0.z), e1 = mk3(q1.x, q1.y, q1.z), e2 = mk3(q2.x, q2.y, q2.z);
	const f3 p = cross(r.d, e2);
	const float det = dot(e1, p);
	if (!(det != 0.0f)) return false;
	const float id = P::rcp(det);
	const f3 sv = sub(r.o, v0);
	const float u = dot(sv, p) * id;
	if (!(u >= 0.0f && u <= 1.0f)) return false;
	const f3 q = cross(sv, e1);
	const float v = dot(r.d, q) * id;
	if (!(v >= 0.0f && u + v <= 1.0f)) return false;
	const float tt = dot(e2, q) * id;
	return tt >= r.t_min && tt <= r.t_max;
}

// Sets up the ray and tests the root box: kTraceMiss, or kTraceContinue.
template <class P> RL_DEV int trace_begin(const SceneView& s, TraceRay& r, f3 o, f3 d, float t_min, float t_max) {
	r.o = o;
	r.d = d;
	r.inv[0] = P::rcp(d.x);
	r.inv[1] = P::rcp(d.y);
	r.inv[2] = P::rcp(d.z);
	r.t_min = t_min;
	r.t_max = t_max;
	r.sp = 0;
	r.visits = 0;
	r.leaf_left = 0;
	r.leaf_first = 0;
	// Boxes are finite (the scene rejects non-finite triangles); with a
	// finite origin and finite non-zero inv no slab product is NaN, and with
	// t_min and t_max not NaN neither is an interval end.
	r.minmax = !isnan(t_min) && !isnan(t_max);
	const float oc[3] = {o.x, o.y, o.z};
#pragma unroll
	for (int ax = 0; ax != 3; ++ax)
		r.minmax = r.minmax && isfinite(oc[ax]) && isfinite(r.inv[ax]) && r.inv[ax] != 0.0f;
	if (s.triangle_count == 0) return kTraceMiss;
	const float4 lo = __ldg(s.pairs), hi = __ldg(s.pairs + 1);
	float entry;
	if (!ray_box(r, lo, hi, &entry)) return kTraceMiss;
	r.node = __float_as_int(lo.w);
	return kTraceContinue;
}

// The ray's next unit of work: kWorkTriangle (the current leaf's next
// triangle) or kWorkNode (an inner node), resolving the current reference or
// the top of the stack and opening leaves on the way; kWorkDone when nothing
// is left.  Calling it again before the work is done returns the same unit.
enum : int { kWorkTriangle = 0, kWorkNode = 1, kWorkDone = 2 };
RL_DEV int trace_next(TraceRay& r, const int32_t* stack) {
	if (r.leaf_left != 0) return kWorkTriangle;
	for (;;) {
		if (r.node == kNoNode) {
			if (r.sp == 0) return kWorkDone;
			r.node = stack[--r.sp];
		}
		if (r.node >= 0) return kWorkNode;
		const uint32_t code = (uint32_t) (-(r.node + 1));
		r.leaf_first = code >> 3;
		r.leaf_left = code & 7u;
		r.node = kNoNode;
		if (r.leaf_left != 0) return kWorkTriangle;
	}
}

// One triangle test of the current leaf: kTraceHit or kTraceContinue.
template <class P> RL_DEV int trace_triangle(const SceneView& s, TraceRay& r) {
	const bool hit = ray_triangle<P>(r, s.triangles + 3 * (size_t) r.leaf_first);
	++r.leaf_first;
	--r.leaf_left;
	return hit ? kTraceHit : kTraceContinue;
}

// One inner node: both child boxes, the nearer hit child next and the other
// pushed.  kTraceContinue, or kTraceMiss with the error recorded when the
// stack is full.
RL_DEV int trace_node(const SceneView& s, TraceRay& r, int32_t* stack, uint32_t* error) {
	const float4* n = s.pairs + 2 + 4 * (size_t) r.node;
	const float4 lo0 = __ldg(n), hi0 = __ldg(n + 1), lo1 = __ldg(n + 2), hi1 = __ldg(n + 3);
	float e0, e1;
	const bool h0 = ray_box(r, lo0, hi0, &e0), h1 = ray_box(r, lo1, hi1, &e1);
	const int32_t ref0 = __float_as_int(lo0.w), ref1 = __float_as_int(lo1.w);
	if (h0 && h1) {
		if (r.sp >= kBvhStack) {
			atomicOr(error, kErrorTraversalLimit);
			return kTraceMiss;
		}
		// The nearer child first: an occluder near the origin ends the
		// query early.
		const bool second_first = e1 < e0;
		stack[r.sp++] = second_first ? ref0 : ref1;
		r.node = second_first ? ref1 : ref0;
	} else {
		r.node = h0 ? ref0 : (h1 ? ref1 : kNoNode);
	}
	return kTraceContinue;
}

// One step: one triangle test or one inner node.  Gives up after
// kTraversalLimit steps or on a stack overflow, records the error and
// reports "not occluded".
template <class P> RL_DEV int trace_step(const SceneView& s, TraceRay& r, int32_t* stack, uint32_t* error) {
	if (++r.visits > kTraversalLimit) {
		atomicOr(error, kErrorTraversalLimit);
		return kTraceMiss;
	}
	const int work = trace_next(r, stack);
	if (work == kWorkDone) return kTraceMiss;
	return work == kWorkTriangle ? trace_triangle<P>(s, r) : trace_node(s, r, stack, error);
}

// Any-hit query; true if occluded.
template <class P> RL_DEV bool any_hit(const SceneView& s, f3 o, f3 d, float t_min, float t_max, uint32_t* error) {
	TraceRay r;
	int32_t stack[kBvhStack];
	int st = trace_begin<P>(s, r, o, d, t_min, t_max);
	while (st == kTraceContinue) st = trace_step<P>(s, r, stack, error);
	return st == kTraceHit;
}

// get_polygon_visibility, shading_pass.frag.glsl:112-129
template <class P>
RL_DEV bool polygon_visibility(const ShadeParams& pr, bool visibility, f3 dir, f3 p, const Light& l) {
	if (!visibility) return false;
	if (!pr.shadows || pr.scene.triangle_count == 0) return true;
	float max_t = P::div(-plane_dot(p, l.plane), dir.x * l.plane[0] + dir.y * l.plane[1] + dir.z * l.plane[2]);
	max_t -= 1e-3f;
	return !any_hit<P>(pr.scene, p, dir, 1.0e-3f, max_t, pr.error);
}

RL_DEV void side_flip(Ltc& ltc, const ShadingData& sd, const Light& l) {
	float side = plane_dot(sd.position, l.plane);
#pragma unroll
	for (int i = 0; i != 4; ++i) ltc.world_to_shading.c[i].y = (side < 0.0f) ? -ltc.world_to_shading.c[i].y : ltc.world_to_shading.c[i].y;
}

// RIS target of the LTC_CP technique, shading_pass.frag.glsl:421-456
template <class P> RL_DEV f3 ltc_cp_target(const ShadingData& sd, Ltc ltc, const Light& l) {
	side_flip(ltc, sd, l);
	uint32_t n = l.vertex_count;
	f3 verts[kMaxPolygonVertices];
#pragma unroll
	for (int i = 0; i != kMaxLightVertices; ++i)
		if (i < (int) n) verts[i] = mul_point(ltc.world_to_shading, l.v[i]);
	uint32_t vc = clip_polygon<P>(n, verts);
	f3 result = splat(0.0f);
	f3 diffuse = splat(0.0f);
	if (vc > 0) diffuse = mul(scale(sd.diffuse_albedo, calculate_ltc<P>(vc, verts)), l.radiance);
	result = add(result, diffuse);
	mat43 w2c = mul(ltc.shading_to_cosine, ltc.world_to_shading);
#pragma unroll
	for (int i = 0; i != kMaxLightVertices; ++i)
		if (i < (int) n) verts[i] = mul_point(w2c, l.v[i]);
	vc = clip_polygon<P>(n, verts);
	f3 ggx = splat(0.0f);
	if (vc > 0) ggx = mul(splat(calculate_ltc<P>(vc, verts) * ltc.albedo), l.radiance);
	return add(result, ggx);
}

// evaluate_polygonal_light_shading_peters (peters = true,
// shading_pass.frag.glsl:292-397) and the PSA branch of
// evaluate_polygonal_light_shading (peters = false, :458-550)
// One polygon's transform to local space, clip_polygon and
// prepare_projected_solid_angle_polygon_sampling (shading_pass.frag.glsl:
// 315-336).  Out of line so that the kernels hold one copy of this long
// code, shared by the diffuse and specular passes.  Returns the clipped
// vertex count (0: nothing left, p untouched).
template <class P>
__device__ __noinline__ uint32_t prepare_space(mat43 w2l, const Light& l, PsaPolygon& p, bool fa) {
	const uint32_t n = l.vertex_count;
	f3 verts[kMaxPolygonVertices];
#pragma unroll
	for (int j = 0; j != kMaxLightVertices; ++j)
		if (j < (int) n) verts[j] = mul_point(w2l, l.v[j]);
	const uint32_t vc = clip_polygon<P>(n, verts);
	if (vc != 0) prepare_psa<P>(p, vc, verts, fa);
	return vc;
}

// prepare_space with the vertices read from the light's device record
// (the same values as load_light gives), so that callers need not keep a
// Light in memory for the call.  Inlined: its one caller runs it in a loop
// over the two spaces, so the code is not duplicated, and an out-of-line call
// saved the caller's live registers to local memory (sample kernel 3.98 ->
// 3.79 ms per 4-frame 1080p launch inlined).
template <class P>
RL_DEV uint32_t prepare_space_record(const mat43& w2l, const float4* record, PsaPolygon& p, bool fa) {
	const uint32_t n = __float_as_uint(__ldg(record).w);
	f3 verts[kMaxPolygonVertices];
#pragma unroll
	for (int j = 0; j != kMaxLightVertices; ++j) {
		if (j < (int) n) {
			const float4 q = __ldg(record + 2 + j);
			verts[j] = mul_point(w2l, mk3(q.x, q.y, q.z));
		}
	}
	const uint32_t vc = clip_polygon<P>(n, verts);
	if (vc != 0) prepare_psa<P>(p, vc, verts, fa);
	return vc;
}

// The side flip and both polygons' PSA sampling preparations of
// evaluate_polygonal_light_shading_peters (shading_pass.frag.glsl:298-341):
// pd in shading space, ps in cosine space.  Returns false when the estimate
// is zero (the polygon clips to nothing or has no projected solid angle in
// shading space).
template <class P>
RL_DEV bool psa_prepare_both(const ShadeParams& pr, const ShadingData& sd, Ltc& ltc, const Light& l, PsaPolygon& pd,
                             PsaPolygon& ps) {
	const bool fa = pr.fast_atan != 0;
	side_flip(ltc, sd, l);
	if (prepare_space<P>(ltc.world_to_shading, l, pd, fa) == 0) return false;
	if (prepare_space<P>(mul(ltc.shading_to_cosine, ltc.world_to_shading), l, ps, fa) == 0) ps.psa = 0.0f;
	return pd.psa != 0.0f;
}

// Threads per block of the kernels that shade with psa_mis_shade.  Each
// thread's two PSA polygon buffers (196 bytes each, dynamically indexed)
// are slots of shared-memory arrays, 49 words apart, so the lanes' words of
// one index fall in distinct banks; in local memory the resident warps'
// buffers did not stay in L1.
constexpr int kShadeThreads = 128;
// pd and ps are the thread's two polygon buffers.
template <class P>
RL_DEV f3 psa_mis_shade(const ShadeParams& pr, const ShadingData& sd, Ltc ltc, const Light& l, uint32_t& seed,
                        bool peters, bool visibility_in, PsaPolygon& pd, PsaPolygon& ps) {
	const bool fa = pr.fast_atan != 0;
	const bool biased = pr.technique == sample_polygon_projected_solid_angle_biased;
	f3 result = splat(0.0f);
	if (!psa_prepare_both<P>(pr, sd, ltc, l, pd, ps)) return result;
	float specular_weight = ltc.albedo * ps.psa;
	f3 diffuse_weight = scale(max3(sd.diffuse_albedo, splat(0.01f)), pd.psa);
	int technique_count = (ps.psa > 0.0f) ? 2 : 1;
	float rcp_d = P::rcp(pd.psa);
	float rcp_s = P::rcp(ps.psa);
	f3 specular_weight_rgb = splat(specular_weight);
	if (pr.mis_heuristic == mis_heuristic_optimal) {
		f3 rop = scale(l.radiance, kInvPi);
		diffuse_weight = mul(diffuse_weight, rop);
		specular_weight_rgb = mul(specular_weight_rgb, rop);
	}
	for (int i = 0; i != pr.sample_count; ++i) {
		f3 dir_d = sample_psa<P>(pd, get_noise_2(seed), fa, biased);
		f3 dir_s = mk3(0.0f, 0.0f, 1.0f);
		if (ps.psa > 0.0f) {
			dir_s = sample_psa<P>(ps, get_noise_2(seed), fa, biased);
			dir_s = normalize<P>(mul(ltc.cosine_to_shading, dir_s));
		}
		for (int j = 0; j != technique_count; ++j) {
			f3 dir = (j == 0) ? dir_d : dir_s;
			if (dir.z <= 0.0f) continue;
			float diffuse_density = dir.z * rcp_d;
			float specular_density = evaluate_ltc_density<P>(ltc, dir, rcp_s);
			f3 world_dir = transpose_mul(ltc.world_to_shading, dir);
			f3 integrand;
			bool visibility;
			if (peters) {
				visibility = dot(sd.normal, world_dir) > 0.0f;
				visibility = polygon_visibility<P>(pr, visibility, world_dir, sd.position, l);
				f3 rb = visibility ? mul(l.radiance, evaluate_brdf<P>(sd, world_dir)) : splat(0.0f);
				integrand = scale(rb, dir.z);
			} else {
				bool cur = visibility_in;
				bool side_vis = dot(sd.normal, world_dir) > 0.0f;
				f3 rb;
				if (!side_vis) {
					rb = splat(0.0f);
				} else {
					cur = polygon_visibility<P>(pr, cur, world_dir, sd.position, l);
					cur = side_vis && cur;
					rb = mul(l.radiance, evaluate_brdf<P>(sd, world_dir));
				}
				integrand = scale(rb, dir.z);
				integrand = (cur || !visibility_in) ? integrand : splat(0.0f);
				visibility = true;
			}
			if (j == 0 && ps.psa <= 0.0f)
				result = add(result, visibility ? scale(integrand, P::rcp(diffuse_density)) : splat(0.0f));
			else if (j == 0)
				result = add(result, mis_estimate<P>(pr.mis_heuristic, integrand, diffuse_weight, diffuse_density,
				                                     specular_weight_rgb, specular_density, pr.mis_visibility_estimate));
			else
				result = add(result, mis_estimate<P>(pr.mis_heuristic, integrand, specular_weight_rgb, specular_density,
				                                     diffuse_weight, diffuse_density, pr.mis_visibility_estimate));
		}
	}
	return scale(result, P::rcp((float) pr.sample_count));
}

// Body of shading_pass.frag.glsl:main (:674-770) for one pixel and frame.
// C is the numerics of the RIS candidate evaluation, P of everything else.
// sample_area_polygon_turk, polygon_sampling_related_work.glsl:35-43.  Like
// the reference, it samples the triangle of vertices 0, 1 and 2.
RL_DEV f3 sample_area_polygon_turk(const Light& l, f2 rnd) {
	const float s = __fsqrt_rn(rnd.x);
	const float b0 = 1.0f - s, b1 = s * rnd.y, b2 = __fmaf_rn(-s, rnd.y, s);
	return add(add(scale(l.v[0], b0), scale(l.v[1], b1)), scale(l.v[2], b2));
}

// get_polygon_area, shading_pass.frag.glsl:146-150 (vertices 0, 1, 2)
template <class P> RL_DEV float polygon_area(const Light& l) {
	const f3 c = cross_stable(sub(l.v[1], l.v[0]), sub(l.v[2], l.v[0]));
	return P::div(P::sqrt(dot(c, c)), 2.0f);
}

// The SAMPLE_POLYGON_AREA_TURK branch of evaluate_polygonal_light_shading
// (shading_pass.frag.glsl:411-418) with get_area_sample_density
// (polygon_sampling_related_work.glsl:57-64), get_polygonal_light_mis_estimate
// (:281-287) and get_polygon_radiance_brdf_product (:200-207).  With
// eval_only the stored light_sample is evaluated and no noise is drawn;
// visibility is traced only when it comes in true.
template <class P>
RL_DEV f3 area_turk_shade(const ShadeParams& pr, const ShadingData& sd, const Light& l, f3& light_sample,
                          bool eval_only, bool& visibility, uint32_t& seed) {
	f3 result = splat(0.0f);
	const f3 normal = mk3(l.plane[0], l.plane[1], l.plane[2]);
	for (int i = 0; i != pr.sample_count; ++i) {
		if (!eval_only) light_sample = sample_area_polygon_turk(l, get_noise_2(seed));
		f3 dir = sub(light_sample, sd.position);
		const float d2 = dot(dir, dir);
		dir = scale(dir, P::rsqrt(d2));
		const float projected_area = fabsf(dot(normal, dir)) * polygon_area<P>(l);
		const float density = P::div(d2, projected_area);
		const float lambert = dot(sd.normal, dir);
		f3 rb = splat(0.0f);
		if (dot(sd.normal, dir) > 0.0f) {
			visibility = polygon_visibility<P>(pr, visibility, dir, sd.position, l);
			rb = mul(l.radiance, evaluate_brdf<P>(sd, dir));
		}
		result = add(result, density > 0.0f ? scale(rb, P::div(lambert, density)) : splat(0.0f));
	}
	return scale(result, P::rcp((float) pr.sample_count));
}

template <class C, class P>
RL_DEV f3 shade_pixel(const ShadeParams& pr, const ShadingData& sd, const Ltc& ltc, uint32_t seed, bool first_frame,
                      risltc_reservoir_t* res_out, PsaPolygon& pd, PsaPolygon& ps) {
	const int n = pr.scene.light_count;
	const bool peters = pr.technique == sample_polygon_ltc_cp;
	const bool area_turk = pr.technique == sample_polygon_area_turk;
	// The area technique's sampled light position, carried from candidate to
	// candidate and kept by the reservoir (shading_pass.frag.glsl:704, 735).
	f3 light_sample = splat(0.0f);
	f3 final_color = splat(0.0f);
	risltc_reservoir_t rec;
	rec.light_index = -1;
	rec.w_sum = 0.0f;
	rec.sample_value = 0.0f;
	rec.padding = 0;
	if (pr.light_sampling == light_uniform) {
		for (int i = 0; i != pr.light_samples; ++i) {
			int idx = (int) (get_noise_1(seed) * (float) n);
			idx = idx > n - 1 ? n - 1 : idx;
			Light l;
			load_light(pr.scene, idx, l);
			bool visibility = true;
			const f3 shade = area_turk ? area_turk_shade<P>(pr, sd, l, light_sample, false, visibility, seed)
			                           : psa_mis_shade<P>(pr, sd, ltc, l, seed, peters, true, pd, ps);
			f3 r = scale(shade, (float) n);
			float ls = (float) pr.light_samples;
			r = mk3(P::div(r.x, ls), P::div(r.y, ls), P::div(r.z, ls));
			final_color = add(final_color, scale(r, visibility ? 1.0f : 0.0f));
			if (i == 0) rec.light_index = idx;
		}
	} else {
		for (int j = 0; j != pr.light_samples; ++j) {
			float w_sum = 0.0f, sample_value = 0.0f;
			int res_index = -1;
			f3 res_light_sample = splat(0.0f);
			const int m = pr.candidate_count;
			const float p = P::rcp((float) n);
			for (int i = 0; i != m; ++i) {
				int idx = (int) (get_noise_1(seed) * (float) n);
				idx = idx > n - 1 ? n - 1 : idx;
				Light l;
				load_light(pr.scene, idx, l);
				f3 color;
				if (peters) {
					color = ltc_cp_target<C>(sd, ltc, l);
				} else if (area_turk) {
					bool dummy_visibility = false;
					color = area_turk_shade<C>(pr, sd, l, light_sample, false, dummy_visibility, seed);
				} else {
					color = psa_mis_shade<C>(pr, sd, ltc, l, seed, false, false, pd, ps);
				}
				float p_hat = C::sqrt(dot(color, color));
				float w = C::div(p_hat, p);
				// insert_in_reservoir, reservoir.glsl:34-41
				float rnd = get_noise_1(seed);
				w_sum += w;
				if (w > 0.0f && rnd < C::div(w, w_sum)) {
					res_index = idx;
					res_light_sample = light_sample;
					sample_value = p_hat;
				}
			}
			if (j == 0) {
				rec.light_index = res_index;
				rec.w_sum = w_sum;
				rec.sample_value = sample_value;
			}
			if (res_index >= 0) {
				Light l;
				load_light(pr.scene, res_index, l);
				bool visibility = true;
				const f3 color = area_turk ? area_turk_shade<P>(pr, sd, l, res_light_sample, true, visibility, seed)
				                           : psa_mis_shade<P>(pr, sd, ltc, l, seed, peters, true, pd, ps);
				float W = P::div(w_sum, (float) m * sample_value);
				// The area technique has no p_hat == 0 guard but multiplies by
				// the traced visibility (shading_pass.frag.glsl:749-756).
				if (!area_turk && sample_value == 0.0f) W = 0.0f;
				if (area_turk) W = W * (visibility ? 1.0f : 0.0f);
				f3 cw = scale(color, W);
				float ls = (float) pr.light_samples;
				final_color = add(final_color, mk3(P::div(cw.x, ls), P::div(cw.y, ls), P::div(cw.z, ls)));
			}
		}
	}
	if (isnan(final_color.x) || isnan(final_color.y) || isnan(final_color.z) || isinf(final_color.x) ||
	    isinf(final_color.y) || isinf(final_color.z))
		final_color = mk3(1.0f, 0.0f, 0.8f);
	if (first_frame && res_out) *res_out = rec;
	return final_color;
}

template <class C, class P> __global__ void __launch_bounds__(kShadeThreads) shade_kernel(ShadeParams pr) {
	__shared__ PsaPolygon polys[2][kShadeThreads];
	const uint32_t np = pr.width * pr.height;
	for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < np; i += gridDim.x * blockDim.x) {
		const uint32_t x = i % pr.width, y = i / pr.width;
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
		ShadingData sd;
		sd.position = mk3(g[0 * (size_t) np + i], g[1 * (size_t) np + i], g[2 * (size_t) np + i]);
		sd.normal = mk3(g[3 * (size_t) np + i], g[4 * (size_t) np + i], g[5 * (size_t) np + i]);
		sd.outgoing = mk3(g[6 * (size_t) np + i], g[7 * (size_t) np + i], g[8 * (size_t) np + i]);
		sd.lambert_outgoing = g[9 * (size_t) np + i];
		sd.diffuse_albedo = mk3(g[10 * (size_t) np + i], g[11 * (size_t) np + i], g[12 * (size_t) np + i]);
		sd.fresnel_0 = mk3(g[13 * (size_t) np + i], g[14 * (size_t) np + i], g[15 * (size_t) np + i]);
		sd.roughness = g[16 * (size_t) np + i];
		float fl = dot(sd.fresnel_0, mk3(0.2126f, 0.7152f, 0.0722f));
		const Ltc ltc = get_ltc_coefficients<P>(pr.scene, fl, sd.roughness, sd.position, sd.normal, sd.outgoing);
		f3 sum = splat(0.0f);
		double acc[3] = {0.0, 0.0, 0.0};
		for (uint32_t f = 0; f != pr.frame_count; ++f) {
			uint32_t rn_x = pr.animate ? wang_random_number((pr.noise_seed + f) * 4u) : 0u;
			uint32_t seed = get_noise_accessor(x, y, pr.width, rn_x);
			f3 c = shade_pixel<C, P>(pr, sd, ltc, seed, f == 0, res, polys[0][threadIdx.x], polys[1][threadIdx.x]);
			sum = add(sum, c);
			acc[0] += (double) c.x;
			acc[1] += (double) c.y;
			acc[2] += (double) c.z;
		}
		if (pr.out_rgb) {
			float inv = 1.0f / (float) pr.frame_count;
			f3 mean = pr.frame_count == 1 ? sum : scale(sum, inv);
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

// Batch of independent any-hit queries (risltc_trace_shadow).
template <class P>
__global__ void __launch_bounds__(128) trace_shadow_kernel(SceneView s, const float4* rays, uint32_t count,
                                                          uint32_t* hits, uint32_t* error) {
	for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < count; i += gridDim.x * blockDim.x) {
		float4 a = rays[2 * (size_t) i], b = rays[2 * (size_t) i + 1];
		hits[i] = any_hit<P>(s, mk3(a.x, a.y, a.z), mk3(b.x, b.y, b.z), a.w, b.w, error) ? 1u : 0u;
	}
}

}  // namespace risltc
