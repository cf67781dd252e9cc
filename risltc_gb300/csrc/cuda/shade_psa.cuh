// shade_psa.cuh - projected solid angle sampling of convex polygons on the
// device (polygon_sampling.glsl:231-828), plus the BRDF and MIS weights
// (brdfs.glsl:43-93, shading_pass.frag.glsl:219-269).
// Restates upstream risltc routines (GPLv3; the polygon_sampling.glsl parts
// also BSD-3, whose notice is retained in NOTICE).
#pragma once
#include "shade_device.cuh"

namespace risltc {

struct PsaPolygon {
	uint32_t vertex_count;
	f2 vertices[kMaxPolygonVertices];
	f2 ellipses[kMaxPolygonVertices];
	f2 inner_ellipse_0;
	float sector_psa[kMaxPolygonVertices];
	float psa;
};

// fast_positive_atan, polygon_sampling.glsl:84-98
template <class P> RL_DEV float fast_positive_atan(float y) {
	float ay = fabsf(y);
	float rx = (ay > 1.0f) ? P::rcp(ay) : ay;
	float ry = rx * rx;
	float rz = __fmaf_rn(ry, 0.02083509974181652f, -0.08513300120830536f);
	rz = __fmaf_rn(ry, rz, 0.18014100193977356f);
	rz = __fmaf_rn(ry, rz, -0.3302994966506958f);
	ry = __fmaf_rn(ry, rz, 0.9998660087585449f);
	rz = __fmaf_rn(-2.0f * ry, rx, kHalfPi);
	rz = (ay > 1.0f) ? rz : 0.0f;
	rx = __fmaf_rn(rx, ry, rz);
	return (y < 0.0f) ? (kPi - rx) : rx;
}

// positive_atan, polygon_sampling.glsl:105-112
template <class P> RL_DEV float positive_atan(float t, bool fast_atan) {
	if (fast_atan) return fast_positive_atan<P>(t);
	float offset = (t < 0.0f) ? kPi : 0.0f;
	return rl_atanf(t) + offset;
}

RL_DEV float mix_fma(float x, float y, float a) { return __fmaf_rn(a, y, __fmaf_rn(-a, x, x)); }
RL_DEV float kahan(float a, float b, float c, float d) {
	float cd = c * d;
	float err = __fmaf_rn(c, d, -cd);
	return __fmaf_rn(a, b, -cd) - err;
}
RL_DEV f3 cross_stable(f3 l, f3 r) {
	return {kahan(l.y, r.z, l.z, r.y), kahan(l.z, r.x, l.x, r.z), kahan(l.x, r.y, l.y, r.x)};
}
RL_DEV bool is_inner_ellipse(f2 e) { return (__float_as_uint(e.x) & 0x80000000u) != 0; }
RL_DEV bool is_central_case(const PsaPolygon& p) { return p.inner_ellipse_0.x > 0.0f; }

template <class P> RL_DEV f2 ellipse_from_edge(f3 v0, f3 v1) {
	f3 n = cross_stable(v0, v1);
	float s = P::rcp(n.z);
	s = is_inner_ellipse(mk2(n.x, n.y)) ? -s : s;
	f2 e = mk2(n.x * s, n.y * s);
	e.x = (n.z != 0.0f) ? e.x : __int_as_float(0x7f800000);
	return e;
}
RL_DEV f2 ellipse_transform(f2 e, f2 p) {
	float d = dot(e, p);
	return fma2(mk2(d, d), e, p);
}
RL_DEV float ellipse_det(f2 e) { return __fmaf_rn(e.x, e.x, __fmaf_rn(e.y, e.y, 1.0f)); }
template <class P> RL_DEV float ellipse_rsqrt_det(f2 e) { return P::rsqrt(ellipse_det(e)); }
RL_DEV float direction_factor_rsq(f2 e, f2 d) {
	float ed = dot(e, d);
	float dd = dot(d, d);
	return __fmaf_rn(ed, ed, dd);
}
template <class P> RL_DEV float direction_factor(f2 e, f2 d) { return P::rsqrt(direction_factor_rsq(e, d)); }
template <class P> RL_DEV float normalized_direction_factor(f2 e, f2 d) {
	float ed = dot(e, d);
	return P::rsqrt(__fmaf_rn(ed, ed, 1.0f));
}

template <class P>
RL_DEV float area_between_from_tangents(float inner_rsd, float inner_t, float outer_rsd, float outer_t, bool fa) {
	float inner_area = inner_rsd * positive_atan<P>(inner_t, fa);
	float result = __fmaf_rn(outer_rsd, positive_atan<P>(outer_t, fa), -inner_area);
	return (result > 0.0f) ? (0.5f * result) : 0.0f;
}

template <class P>
RL_DEV float area_between_in_sector(f2 inner, float inner_rsd, f2 outer, float outer_rsd, f2 d0, f2 d1, bool fa) {
	float det_dirs = fmax_glsl(0.0f, dot(d1, rotate_90(d0)));
	float inner_dot = inner_rsd * dot(d0, ellipse_transform(inner, d1));
	float outer_dot = outer_rsd * dot(d0, ellipse_transform(outer, d1));
	return area_between_from_tangents<P>(inner_rsd, P::div(det_dirs, inner_dot), outer_rsd, P::div(det_dirs, outer_dot),
	                                     fa);
}

template <class P> RL_DEV float ellipse_area_in_sector(f2 e, f2 d0, f2 d1, bool fa) {
	float rsd = ellipse_rsqrt_det<P>(e);
	float det_dirs = fmax_glsl(0.0f, dot(d1, rotate_90(d0)));
	float ed = rsd * dot(d0, ellipse_transform(e, d1));
	float area = 0.5f * rsd * positive_atan<P>(P::div(det_dirs, ed), fa);
	return (rsd > 0.0f) ? area : 0.0f;
}

RL_DEV void compare_and_swap(PsaPolygon& p, int lhs, int rhs) {
	f2 lc = p.vertices[lhs];
	float nz = kahan(lc.x, -p.vertices[rhs].y, lc.y, -p.vertices[rhs].x);
	bool swap = (nz == 0.0f) ? isinf(p.ellipses[rhs].x) : (nz > 0.0f);
	p.vertices[lhs] = swap ? p.vertices[rhs] : lc;
	p.vertices[rhs] = swap ? lc : p.vertices[rhs];
	lc = p.ellipses[lhs];
	p.ellipses[lhs] = swap ? p.ellipses[rhs] : lc;
	p.ellipses[rhs] = swap ? lc : p.ellipses[rhs];
}

// sort_convex_polygon_vertices, polygon_sampling.glsl:441-506: the
// reference's sorting network for each vertex count (3..8), as a table of
// compare-and-swap pairs (lhs << 4 | rhs) run in the reference's order, then
// the three common steps.  One loop instead of a switch keeps the code small.
// 8-gons clipped to 9 vertices (beyond the reference's networks) use adjacent
// compare-and-swap passes.
__device__ __constant__ uint8_t kSortPairs[67] = {
    0x12,                                                        // 3
    0x13,                                                        // 4
    0x24, 0x13, 0x12, 0x03, 0x34,                                // 5
    0x35, 0x24, 0x15, 0x04, 0x45, 0x13,                          // 6
    0x25, 0x16, 0x56, 0x34, 0x04, 0x46, 0x13, 0x35, 0x45,        // 7
    0x26, 0x37, 0x15, 0x04, 0x46, 0x57, 0x67, 0x45, 0x13,        // 8
    0x01,                                                        // 9: i = 1
    0x12, 0x01,                                                  //    i = 2
    0x23, 0x12, 0x01,                                            //    i = 3
    0x34, 0x23, 0x12, 0x01,                                      //    i = 4
    0x45, 0x34, 0x23, 0x12, 0x01,                                //    i = 5
    0x56, 0x45, 0x34, 0x23, 0x12, 0x01,                          //    i = 6
    0x67, 0x56, 0x45, 0x34, 0x23, 0x12, 0x01,                    //    i = 7
    0x78, 0x67, 0x56, 0x45, 0x34, 0x23, 0x12, 0x01,              //    i = 8
};
// The pairs of vertex count c are kSortPairs[kSortStart[c], kSortStart[c + 1]).
__device__ __constant__ uint8_t kSortStart[11] = {0, 0, 0, 0, 1, 2, 7, 13, 22, 31, 67};

RL_DEV void sort_convex_polygon_vertices(PsaPolygon& p) {
	const uint32_t c = p.vertex_count < 10u ? p.vertex_count : 0u;
	const uint32_t end = kSortStart[c + 1];
	for (uint32_t k = kSortStart[c]; k < end; ++k) {
		const uint32_t pair = kSortPairs[k];
		compare_and_swap(p, (int) (pair >> 4), (int) (pair & 15u));
	}
	compare_and_swap(p, 0, 2);
	if (p.vertex_count >= 4) compare_and_swap(p, 2, 3);
	compare_and_swap(p, 0, 1);
}

// prepare_projected_solid_angle_polygon_sampling, polygon_sampling.glsl:545-613
template <class P> RL_DEV void prepare_psa(PsaPolygon& p, uint32_t vc, const f3 v[kMaxPolygonVertices], bool fa) {
	p.vertex_count = vc;
	p.inner_ellipse_0 = mk2(1.0f, 0.0f);
	p.vertices[0] = mk2(v[0].x, v[0].y);
	p.ellipses[0] = ellipse_from_edge<P>(v[0], v[1]);
	f2 previous = p.ellipses[0];
#pragma unroll 1
	for (uint32_t i = 1; i != vc; ++i) {
		p.vertices[i] = mk2(v[i].x, v[i].y);
		f2 e = ellipse_from_edge<P>(v[i], v[(i + 1 == vc) ? 0 : i + 1]);
		bool inner = is_inner_ellipse(e);
		p.ellipses[i] = inner ? previous : e;
		p.inner_ellipse_0 = (is_inner_ellipse(previous) && !inner) ? previous : p.inner_ellipse_0;
		previous = e;
	}
	{
		f2 e = p.ellipses[0];
		bool inner = is_inner_ellipse(e);
		p.ellipses[0] = inner ? previous : e;
		p.inner_ellipse_0 = (is_inner_ellipse(previous) && !inner) ? previous : p.inner_ellipse_0;
	}
	p.psa = 0.0f;
	if (is_central_case(p)) {
#pragma unroll 1
		for (uint32_t i = 0; i != vc; ++i) {
			p.sector_psa[i] = ellipse_area_in_sector<P>(p.ellipses[i], p.vertices[i], p.vertices[(i + 1 == vc) ? 0 : i + 1], fa);
			p.psa += p.sector_psa[i];
		}
	} else {
		sort_convex_polygon_vertices(p);
		f2 inner = p.inner_ellipse_0;
		float inner_rsd = ellipse_rsqrt_det<P>(inner);
		f2 outer = mk2(0.0f, 0.0f);
		float outer_rsd = 0.0f;
#pragma unroll 1
		for (uint32_t i = 0; i + 1 != vc; ++i) {
			f2 ve = p.ellipses[i];
			bool vi = is_inner_ellipse(ve);
			float vr = ellipse_rsqrt_det<P>(ve);
			if (i == 0) {
				outer = ve;
				outer_rsd = vr;
			} else {
				inner = vi ? ve : inner;
				inner_rsd = vi ? vr : inner_rsd;
				outer = vi ? outer : ve;
				outer_rsd = vi ? outer_rsd : vr;
			}
			p.sector_psa[i] = area_between_in_sector<P>(inner, inner_rsd, outer, outer_rsd, p.vertices[i], p.vertices[i + 1], fa);
			p.psa += p.sector_psa[i];
		}
	}
}

// normalize_approx_and_flip, polygon_sampling.glsl:622-634
RL_DEV f2 normalize_approx_and_flip(f2 rhs, f2 semi_circle) {
	float s = fabsf(rhs.x) + fabsf(rhs.y);
	s = __uint_as_float(__float_as_uint(s) ^ 0x7F800000u);
	s = (dot(rhs, semi_circle) >= 0.0f) ? s : -s;
	return scale(rhs, s);
}

struct Mat2 {
	f2 c0, c1;
};
RL_DEV Mat2 outer2(f2 col, f2 row) { return {scale(col, row.x), scale(col, row.y)}; }

// solve_homogeneous_quadratic, polygon_sampling.glsl:648-653
template <class P> RL_DEV f2 solve_homogeneous_quadratic(const Mat2& q) {
	float cxy = 0.5f * (q.c0.y + q.c1.x);
	float sd = P::sqrt(fmax_glsl(0.0f, cxy * cxy - q.c0.x * q.c1.y));
	float sr = fabsf(cxy) + sd;
	return (cxy >= 0.0f) ? mk2(sr, -q.c0.x) : mk2(q.c1.y, sr);
}

// sample_sector_between_ellipses, polygon_sampling.glsl:668-762
template <class P>
RL_DEV f2 sample_sector_between_ellipses(f2 rnd, float target_area, f2 inner, f2 outer, f2 dir_0, f2 dir_1,
                                         uint32_t iterations, bool fa, bool biased) {
	f2 qd0 = normalize<P>(dir_0);
	f2 qd2 = normalize<P>(dir_1);
	f2 qd1 = add(qd0, qd2);
	float n00 = normalized_direction_factor<P>(inner, qd0);
	float n01 = direction_factor<P>(inner, qd1);
	float n02 = normalized_direction_factor<P>(inner, qd2);
	float n10 = normalized_direction_factor<P>(outer, qd0);
	float n11 = direction_factor<P>(outer, qd1);
	float n12 = normalized_direction_factor<P>(outer, qd2);
	float sa0 = n10 * n11 - n00 * n01;
	float sa1 = n11 * n12 - n01 * n02;
	float tqa = mix_fma(-sa0, sa1, rnd.x);
	bool first = tqa <= 0.0f;
	qd2 = first ? qd0 : qd2;
	n02 = first ? n00 : n02;
	n12 = first ? n10 : n12;
	tqa += first ? sa0 : -sa1;
	tqa *= fabsf(qd1.x * qd2.y - qd2.x * qd1.y);
	f2 qn0 = add(scale(qd1, n01), scale(qd2, n02));
	f2 qn1 = add(scale(qd1, n11), scale(qd2, n12));
	qn0 = ellipse_transform(inner, qn0);
	qn1 = ellipse_transform(outer, qn1);
	float qo0 = dot(qn0, qd1) * n01;
	float qo1 = dot(qn1, qd1) * n11;
	Mat2 quadratic = outer2(scale(rotate_90(qd2), qo1 * n12), qn0);
	{
		f2 col = add(scale(rotate_90(qd2), qo0 * n02), scale(qn0, tqa));
		Mat2 sb = outer2(col, qn1);
		quadratic.c0 = sub(quadratic.c0, sb.c0);
		quadratic.c1 = sub(quadratic.c1, sb.c1);
	}
	f2 cur = solve_homogeneous_quadratic<P>(quadratic);
	if (!biased) {
		iterations = (fabsf(rnd.x - 0.5f) <= 0.5f - 1.0e-5f) ? iterations : 0u;
		float irsd = ellipse_rsqrt_det<P>(inner);
		float orsd = ellipse_rsqrt_det<P>(outer);
#pragma unroll 1
		for (uint32_t i = 0; i != iterations; ++i) {
			cur = normalize_approx_and_flip(cur, qd1);
			f2 idir = ellipse_transform(inner, cur);
			f2 odir = ellipse_transform(outer, cur);
			float det_dirs = fmax_glsl(0.0f, dot(cur, rotate_90(qd0)));
			float err = target_area - area_between_from_tangents<P>(irsd, P::div(det_dirs, irsd * dot(qd0, idir)), orsd,
			                                                      P::div(det_dirs, orsd * dot(qd0, odir)), fa);
			Mat2 a = outer2(sub(idir, odir), rotate_90(cur));
			Mat2 b = outer2(scale(idir, 2.0f * err), odir);
			quadratic.c0 = sub(a.c0, b.c0);
			quadratic.c1 = sub(a.c1, b.c1);
			cur = solve_homogeneous_quadratic<P>(quadratic);
		}
	}
	cur = (dot(cur, qd1) >= 0.0f) ? cur : neg(cur);
	float inner_factor = P::rcp(direction_factor_rsq(inner, cur));
	float outer_factor = P::rcp(direction_factor_rsq(outer, cur));
	return scale(cur, P::sqrt(mix_fma(inner_factor, outer_factor, rnd.y)));
}

// sample_projected_solid_angle_polygon, polygon_sampling.glsl:772-828
template <class P> RL_DEV f3 sample_psa(const PsaPolygon& p, f2 rnd, bool fa, bool biased) {
	float target = rnd.x * p.psa;
	f2 xy;
	if (is_central_case(p)) {
		f2 outer = mk2(0.0f, 0.0f), d0 = mk2(0.0f, 0.0f);
#pragma unroll 1
		for (uint32_t i = 0; i != p.vertex_count; ++i) {
			if (i > 0) target -= p.sector_psa[i - 1];
			outer = p.ellipses[i];
			d0 = p.vertices[i];
			if ((i >= 2 && i + 1 == p.vertex_count) || target < p.sector_psa[i]) break;
		}
		float sqrt_det = P::sqrt(ellipse_det(outer));
		float angle = 2.0f * target * sqrt_det;
		float sa, ca;
		rl_sincosf(angle, &sa, &ca);
		xy = add(scale(d0, ca * sqrt_det), scale(rotate_90(ellipse_transform(outer, d0)), sa));
		xy = scale(xy, P::sqrt(P::div(rnd.y, direction_factor_rsq(outer, xy))));
	} else {
		float sector = 0.0f;
		f2 inner = p.inner_ellipse_0, outer = mk2(0.0f, 0.0f), d0 = mk2(0.0f, 0.0f), d1 = mk2(0.0f, 0.0f);
#pragma unroll 1
		for (uint32_t i = 0; i + 1 != p.vertex_count; ++i) {
			f2 ve = p.ellipses[i];
			if (i == 0) {
				outer = ve;
			} else {
				target -= p.sector_psa[i - 1];
				bool vi = is_inner_ellipse(ve);
				inner = vi ? ve : inner;
				outer = vi ? outer : ve;
			}
			d0 = p.vertices[i];
			d1 = p.vertices[i + 1];
			sector = p.sector_psa[i];
			if ((i >= 1 && i + 2 == p.vertex_count) || target < sector) break;
		}
		rnd.x = P::div(target, sector);
		xy = sample_sector_between_ellipses<P>(rnd, target, inner, outer, d0, d1, 2u, fa, biased);
	}
	float z = P::sqrt(fmax_glsl(0.0f, __fmaf_rn(-xy.x, xy.x, __fmaf_rn(-xy.y, xy.y, 1.0f))));
	return mk3(xy.x, xy.y, z);
}

// evaluate_brdf (diffuse + specular), brdfs.glsl:58-93
template <class P> RL_DEV f3 evaluate_brdf(const ShadingData& d, f3 wi) {
	f3 h = normalize<P>(add(wi, d.outgoing));
	float li = dot(d.normal, wi);
	float oh = dot(d.outgoing, h);
	f3 brdf = add(splat(0.0f), d.diffuse_albedo);
	float nh = dot(d.normal, h);
	float r2 = d.roughness * d.roughness;
	float ggx = __fmaf_rn(__fmaf_rn(nh, r2, -nh), nh, 1.0f);
	ggx = P::div(r2, ggx * ggx);
	float lo = d.lambert_outgoing;
	float masking = li * P::sqrt(__fmaf_rn(__fmaf_rn(-lo, r2, lo), lo, r2));
	float shadowing = lo * P::sqrt(__fmaf_rn(__fmaf_rn(-li, r2, li), li, r2));
	float smith = P::div(0.5f, masking + shadowing);
	float flipped = 1.0f - clamp_glsl(oh, 0.0f, 1.0f);
	float fs = flipped * flipped;
	float t = fs * flipped * fs;
	f3 f0 = d.fresnel_0;
	f3 fresnel = add(f0, scale(sub(splat(1.0f), f0), t));
	float lum = dot(fresnel, mk3(0.21263901f, 0.71516868f, 0.07219232f));
	brdf = adds(brdf, ggx * smith * lum);
	return scale(brdf, kInvPi);
}

// get_mis_estimate, shading_pass.frag.glsl:219-269
template <class P>
RL_DEV f3 mis_estimate(int heuristic, f3 integrand, f3 sw, float sd, f3 ow, float od, float v) {
	switch (heuristic) {
	case mis_heuristic_balance:
		return scale(integrand, P::rcp(sd + od));
	case mis_heuristic_power:
		return scale(integrand, P::div(sd, sd * sd + od * od));
	case mis_heuristic_weighted: {
		f3 ws = add(scale(sw, sd), scale(ow, od));
		return div3<P>(mul(sw, integrand), ws);
	}
	case mis_heuristic_optimal: {
		float balance = P::rcp(sd + od);
		f3 ws = add(scale(sw, sd), scale(ow, od));
		return add(scale(sw, v), scale(sub(integrand, scale(ws, v)), balance));
	}
	default: {
		float balance = P::rcp(sd + od);
		f3 ws = add(scale(sw, sd), scale(ow, od));
		f3 weighted = div3<P>(sw, ws);
		f3 mixed = splat(__fmaf_rn(-v, balance, balance));
		mixed = fma3(splat(v), weighted, mixed);
		return mul(mixed, integrand);
	}
	}
}

}  // namespace risltc
