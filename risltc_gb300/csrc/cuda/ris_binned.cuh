// ris_binned.cuh - the RIS candidate phase as a warp-per-tile kernel with
// work binning.
//
// Each warp owns kPixels consecutive pixels (32, 16 or 8: the tile's pixels
// per warp) and takes their candidates in super-chunks of kSuper, each made
// of chunks of kChunk (the tile's candidates per pixel per chunk; 8 or 4).
// Per chunk the warp
//   1. draws every pixel's candidate lights from that pixel's noise stream
//      (the LCG sequence of shading_pass.frag.glsl:728-736: a light draw, then
//      the reservoir draw, per candidate);
//   2. sorts the chunk's (pixel, candidate) items by the light's vertex count
//      with a counting sort over the warp, so that the lanes of one step
//      mostly evaluate polygons with the same number of vertices;
//   3. evaluates the items with each pixel's LTC frame read from shared
//      memory, in a form without branches (correctly rounded square roots
//      from sqrt_tuckerman); an item whose polygon is partially clipped in
//      either space, or outside that form's range, is deferred to a list
//      that the warp evaluates 32 at a time, so the clipping path runs with
//      full warps.
// A frame's super-chunk is a unit; after up to four units (a window) the
// last deferred items of the window are evaluated and
//   4. each lane replays its pixel's reservoir updates in candidate order
//      (insert_in_reservoir, reservoir.glsl:34-41), unit by unit, drawing the
//      same noise again.
// Every p_hat is computed by the same operations on the same values as in
// ris_candidates_kernel and the reservoir sees them in the same order, so the
// reservoir records are bit-identical.
// Restates upstream risltc routines (GPLv3): see NOTICE.
#pragma once
#include <algorithm>
#include <atomic>
#include "ris_kernels.cuh"

namespace risltc {

// Blocks per SM the candidate kernel is compiled for (register budget):
// measured best 5 in exact numerics (96 registers; 19.2 against 19.9 ms per
// 4-frame 1080p launch with 4) and 4 in fast numerics, whose paired form
// spills at 96 registers.
#ifndef RISLTC_BINNED_MIN_BLOCKS_EXACT
#define RISLTC_BINNED_MIN_BLOCKS_EXACT 5
#endif
#ifndef RISLTC_BINNED_MIN_BLOCKS_FAST
#define RISLTC_BINNED_MIN_BLOCKS_FAST 4
#endif

// A warp's p_hat values, [window unit][pixel lane][candidate], live in its
// slot of RisParams::p_hat_scratch (global memory, L2/L1): keeping them out
// of shared memory leaves room in the SM's combined L1/shared storage for
// the light records the candidates read.  A slot holds 4096 values: four
// 32-pixel super-chunks of 32 candidates in the default tile.
constexpr int kPHatSlot = 4096;
// The candidate kernels run at most this many blocks per SM (their grid is
// one resident wave); the p_hat scratch has a slot per warp of such a grid.
constexpr int kCandidateBlocksPerSm = 8;

// Candidates per pixel per super-chunk (measured best: 32 in exact numerics,
// 16 in fast numerics, where the smaller tile leaves more L1 for the lights).
#ifndef RISLTC_BINNED_SUPER_EXACT
#define RISLTC_BINNED_SUPER_EXACT 32
#endif
template <class P> struct BinnedSuper {
	static constexpr int value = RISLTC_BINNED_SUPER_EXACT;
};
template <> struct BinnedSuper<FastNumerics> {
	static constexpr int value = 16;
};
template <class P> struct BinnedMinBlocks {
	static constexpr int value = RISLTC_BINNED_MIN_BLOCKS_EXACT;
};
template <> struct BinnedMinBlocks<FastNumerics> {
	static constexpr int value = RISLTC_BINNED_MIN_BLOCKS_FAST;
};
// A pixel's LTC frame in 11 16-byte words (an odd number of them, so that
// the 16-byte reads of 8 lanes from different pixels spread over the banks).
constexpr int kFrameQuads = 11;
constexpr int kBinnedWarps = 4;              // warps per block
constexpr int kBins = kMaxLightVertices - 2; // vertex counts 3..8

template <int kSuper, int kPixels, int kChunk> struct WarpTile {
	static constexpr int kItems = kPixels * kChunk;  // items per warp per chunk
	static constexpr int kDeferred = kItems + 32;     // deferred items pending at most
	static_assert(kItems < 1024, "10-bit bin counters");
	static_assert(kSuper % kChunk == 0 && kPixels * kSuper <= 1024, "super-chunk layout (10-bit slots)");
	float4 frame[kPixels][kFrameQuads];
	// Items as light << 10 | slot, slot = pixel lane * kSuper + candidate of
	// the super-chunk (below 1024; lights below 2^22).
	uint32_t item[kItems];
	uint32_t deferred[kDeferred];
	uint8_t deferred_unit[kDeferred];  // the window unit of each deferred item
	uint32_t deferred_count;
};

// Frame layout (16-byte words): 0 {position, LTC albedo}, 1 {diffuse
// albedo, 0}, 2-4 world to shading, 5-7 world to cosine, 8-10 its y-flipped
// counterpart; each mat4x3's 12 floats column-major across three words.
RL_DEV void store_matrix(float4* q, const mat43& m) {
	q[0] = make_float4(m.c[0].x, m.c[0].y, m.c[0].z, m.c[1].x);
	q[1] = make_float4(m.c[1].y, m.c[1].z, m.c[2].x, m.c[2].y);
	q[2] = make_float4(m.c[2].z, m.c[3].x, m.c[3].y, m.c[3].z);
}
RL_DEV mat43 load_matrix(const float4* q) {
	const float4 a = q[0], b = q[1], c = q[2];
	mat43 m;
	m.c[0] = mk3(a.x, a.y, a.z);
	m.c[1] = mk3(a.w, b.x, b.y);
	m.c[2] = mk3(b.z, b.w, c.x);
	m.c[3] = mk3(c.y, c.z, c.w);
	return m;
}
RL_DEV void store_frame(float4* f, const CandidateFrame& cf) {
	f[0] = make_float4(cf.position.x, cf.position.y, cf.position.z, cf.ltc_albedo);
	f[1] = make_float4(cf.diffuse_albedo.x, cf.diffuse_albedo.y, cf.diffuse_albedo.z, 0.0f);
	store_matrix(f + 2, cf.w2s);
	store_matrix(f + 5, cf.w2c[0]);
	store_matrix(f + 8, cf.w2c[1]);
}

// A light vertex (slot j of the record) in local space: mat4x3 * vec4(v, 1)
// with y negated when negate_y is set (the side flip).
RL_DEV f3 local_vertex(const mat43& t, const float4* record, uint32_t j, bool negate_y) {
	const float4 q = __ldg(record + 2 + j);
	f3 v = mul_point(t, mk3(q.x, q.y, q.z));
	v.y = negate_y ? -v.y : v.y;
	return v;
}

// The partially clipped case, streamed: the integral calculate_ltc gives
// over the polygon clip_polygon makes (mask: the vertices above z = 0, one
// bit each), with the clipped vertices produced one at a time in the order of
// clip_polygon's output slots: the cycle [entry, the run above the horizon,
// exit] starting at its rotation, the run's vertices transformed again from
// the light record.  The same values in the same order as clip_polygon
// followed by calculate_ltc, without a vertex array.  -1 when the polygon
// clips to nothing.  With kChecked, uses the branch-free normalisation and
// edge integral and clears ok where they do not apply.
template <class P, bool kChecked>
RL_DEV float clipped_integral(const mat43& t, const float4* record, uint32_t n, bool negate_y, uint32_t mask, bool& ok) {
	const uint32_t k = __popc(mask);
	const uint32_t s = clip_run_start(n, mask);
	if (s == n) return -1.0f;
	const uint32_t e = clip_wrap(s + k - 1, n), vc = k + 2;
	const f3 entry = iz0<P>(local_vertex(t, record, clip_wrap(s + n - 1, n), negate_y), local_vertex(t, record, s, negate_y));
	const f3 exit = iz0<P>(local_vertex(t, record, e, negate_y), local_vertex(t, record, clip_wrap(e + 1, n), negate_y));
	const uint32_t j0 = clip_wrap(vc - clip_rotation(n, k, s), vc);  // cycle element of slot 0
	f3 first = splat(0.0f), prev = splat(0.0f);
	float r = 0.0f;
#pragma unroll 1
	for (uint32_t slot = 0; slot != vc; ++slot) {
		const uint32_t j = clip_wrap(j0 + slot, vc);
		const f3 v = j == 0 ? entry : (j == k + 1 ? exit : local_vertex(t, record, clip_wrap(s + j - 1, n), negate_y));
		const f3 cur = kChecked ? normalize_checked<P>(v, ok) : normalize<P>(v);
		if (slot == 0)
			first = cur;
		else
			r += kChecked ? integrate_edge_checked<P>(prev, cur, ok) : integrate_edge<P>(prev, cur);
		prev = cur;
	}
	r += kChecked ? integrate_edge_checked<P>(prev, first, ok) : integrate_edge<P>(prev, first);
	return fabsf(r);
}

// One candidate (ltc_cp_candidate, then p_hat = length(color)) with the
// frame in shared memory.  The two LTC integrals run in one loop over the
// spaces.  Each polygon streams vertex by vertex from the light record (the
// next vertex's load issued before the current one is used): every vertex is
// transformed, counted if above the horizon, normalised and joined to the
// previous one in the edge order of calculate_ltc (edges 0-1, ...,
// (n-2)-(n-1), then (n-1)-0).  The sum is kept when the whole polygon is
// above the horizon (the common case); a polygon entirely below contributes
// nothing, and a partially clipped one goes through clip_polygon instead.
// The code stays small and the vertex count of a sorted group is uniform
// across the warp.  With allow_clip false, returns false as soon as a space
// clips the polygon partially; the caller defers the item.
template <class P, bool kChecked>
RL_DEV bool binned_candidate(const float4* f, const float4* record, bool allow_clip, float& p_hat) {
	// kChecked: the branch-free forms (normalize_checked,
	// integrate_edge_checked, sqrt_checked); false when any of them does not
	// apply (a squared length outside the square root's range, an edge of 90
	// degrees or more), and the caller takes the general forms.
	bool ok = true;
	const float4 head = __ldg(record), pl = __ldg(record + 1);
	const uint32_t n = __float_as_uint(head.w);
	const float plane[4] = {pl.x, pl.y, pl.z, pl.w};
	const float4 f0 = f[0];
	const bool flip = plane_dot(mk3(f0.x, f0.y, f0.z), plane) < 0.0f;
	float integral[2];
	bool away[2];
#pragma unroll 1
	for (int s = 0; s != 2; ++s) {
		const mat43 t = load_matrix(f + (s == 0 ? 2 : (flip ? 8 : 5)));
		const bool negate_y = s == 0 && flip;
		float4 q = __ldg(record + 2);
		f3 v = mul_point(t, mk3(q.x, q.y, q.z));
		v.y = negate_y ? -v.y : v.y;
		q = __ldg(record + 3);
		uint32_t mask = v.z > 0.0f ? 1u : 0u;  // bit j: vertex j above the horizon
		const f3 first = kChecked ? normalize_checked<P>(v, ok) : normalize<P>(v);
		f3 prev = first;
		float r = 0.0f;
#pragma unroll 1
		for (uint32_t j = 1; j != n; ++j) {
			v = mul_point(t, mk3(q.x, q.y, q.z));
			v.y = negate_y ? -v.y : v.y;
			q = __ldg(record + 2 + min(j + 1, (uint32_t) kMaxLightVertices - 1));
			mask |= (v.z > 0.0f ? 1u : 0u) << j;
			const f3 cur = kChecked ? normalize_checked<P>(v, ok) : normalize<P>(v);
			r += kChecked ? integrate_edge_checked<P>(prev, cur, ok) : integrate_edge<P>(prev, cur);
			prev = cur;
		}
		r += kChecked ? integrate_edge_checked<P>(prev, first, ok) : integrate_edge<P>(prev, first);
		if (kChecked && !ok) return false;
		bool a = false;
		if (mask == (1u << n) - 1u) {
			r = fabsf(r);
		} else if (mask == 0) {
			r = 0.0f;
			a = true;
		} else {
			if (!allow_clip) return false;
			r = clipped_integral<P, kChecked>(t, record, n, negate_y, mask, ok);
			if (kChecked && !ok) return false;
			a = r < 0.0f;
			r = a ? 0.0f : r;
		}
		if (s == 0) {
			integral[0] = r;
			away[0] = a;
		} else {
			integral[1] = r;
			away[1] = a;
		}
	}
	const f3 radiance = mk3(head.x, head.y, head.z);
	f3 result = splat(0.0f);
	const float4 f1 = f[1];
	const f3 diffuse = away[0] ? splat(0.0f) : mul(scale(mk3(f1.x, f1.y, f1.z), integral[0]), radiance);
	result = add(result, diffuse);
	const f3 ggx = away[1] ? splat(0.0f) : mul(splat(integral[1] * f[0].w), radiance);
	const f3 color = add(result, ggx);
	if (kChecked) {
		p_hat = sqrt_checked<P>(dot(color, color), ok);
		return ok;
	}
	p_hat = P::sqrt(dot(color, color));
	return true;
}

// ---------------------------------------------------------------------------
// The same candidate with both spaces in the two lanes of Blackwell's paired
// FP32 instructions (FADD2 / FMUL2 / FFMA2 on float2; lane .x the shading
// space, lane .y the cosine space).  Both spaces walk the same vertices, so
// every transform, dot product, scale and edge-integral step of the two
// spaces is one paired instruction.  Each lane performs the scalar version's
// operations on the same operands in the same order, and a paired IEEE add
// or multiply rounds each lane exactly as the scalar one does: the values are
// bit-identical.  Exact numerics keeps every multiply and add separate; fast
// numerics contracts them into paired fused multiply-adds.
#ifndef RISLTC_CANDIDATE_PAIRS
#define RISLTC_CANDIDATE_PAIRS 0
#endif
// Unroll factor of the paired vertex loop.
#ifndef RISLTC_PAIR_UNROLL
#define RISLTC_PAIR_UNROLL 1
#endif
constexpr int kPairUnroll = RISLTC_PAIR_UNROLL;

// The paired operations.  Fast numerics uses the paired instructions
// (FADD2 / FMUL2 / FFMA2), which the code generator may contract into fused
// multiply-adds.  Exact numerics must not be contracted, and the code
// generator contracts a paired multiply followed by a paired add into FFMA2
// even with --fmad=false and explicit rounding modifiers (measured: every
// exact-numerics frame then differed from the oracle).  So by default exact
// numerics computes each lane with its own correctly rounded scalar
// operation (__fadd_rn / __fmul_rn, never contracted); the loop still
// carries both spaces' independent dependency chains side by side.
// RISLTC_PAIR_OPS selects the form for exact numerics: 0 scalar per lane,
// 1 paired PTX add/mul, 2 paired fused multiply-adds with exact one and
// zero operands (RN(a * b + -0) = RN(a * b), RN(a * 1 + b) = RN(a + b)).
#ifndef RISLTC_PAIR_OPS
#define RISLTC_PAIR_OPS 0
#endif
#if RISLTC_PAIR_OPS == 1
RL_DEV float2 add2(float2 a, float2 b) {
	float2 d;
	asm("{\n\t.reg .b64 a, b, d;\n\tmov.b64 a, {%2, %3};\n\tmov.b64 b, {%4, %5};\n\t"
	    "add.rn.f32x2 d, a, b;\n\tmov.b64 {%0, %1}, d;\n\t}"
	    : "=f"(d.x), "=f"(d.y)
	    : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y));
	return d;
}
RL_DEV float2 mul2(float2 a, float2 b) {
	float2 d;
	asm("{\n\t.reg .b64 a, b, d;\n\tmov.b64 a, {%2, %3};\n\tmov.b64 b, {%4, %5};\n\t"
	    "mul.rn.f32x2 d, a, b;\n\tmov.b64 {%0, %1}, d;\n\t}"
	    : "=f"(d.x), "=f"(d.y)
	    : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y));
	return d;
}
#elif RISLTC_PAIR_OPS == 2
RL_DEV float2 add2(float2 a, float2 b) { return __ffma2_rn(a, make_float2(1.0f, 1.0f), b); }
RL_DEV float2 mul2(float2 a, float2 b) { return __ffma2_rn(a, b, make_float2(-0.0f, -0.0f)); }
#else
RL_DEV float2 add2(float2 a, float2 b) { return make_float2(__fadd_rn(a.x, b.x), __fadd_rn(a.y, b.y)); }
RL_DEV float2 mul2(float2 a, float2 b) { return make_float2(__fmul_rn(a.x, b.x), __fmul_rn(a.y, b.y)); }
#endif
// Fast numerics: the paired instructions, contraction allowed.
struct PairFast {
	static RL_DEV float2 add(float2 a, float2 b) { return __fadd2_rn(a, b); }
	static RL_DEV float2 mul(float2 a, float2 b) { return __fmul2_rn(a, b); }
	static RL_DEV float2 mad(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
};
struct PairExact {
	static RL_DEV float2 add(float2 a, float2 b) { return add2(a, b); }
	static RL_DEV float2 mul(float2 a, float2 b) { return mul2(a, b); }
	static RL_DEV float2 mad(float2 a, float2 b, float2 c) { return add2(mul2(a, b), c); }
};
template <class P> struct PairOps {
	using type = PairExact;
};
template <> struct PairOps<FastNumerics> {
	using type = PairFast;
};
RL_DEV float2 pair(float a) { return make_float2(a, a); }
// a * b + c (contracted in fast numerics), a + b and a * b in both lanes.
template <class P> RL_DEV float2 mad2(float2 a, float2 b, float2 c) { return PairOps<P>::type::mad(a, b, c); }
template <class P> RL_DEV float2 padd(float2 a, float2 b) { return PairOps<P>::type::add(a, b); }
template <class P> RL_DEV float2 pmul(float2 a, float2 b) { return PairOps<P>::type::mul(a, b); }

struct f3x2 {
	float2 x, y, z;
};
// mat4x3 * vec4(p, 1) in both lanes: ((c0 p.x + c1 p.y) + c2 p.z) + c3.
struct mat43x2 {
	f3x2 c[4];
};
template <class P> RL_DEV f3x2 mul_point2(const mat43x2& m, float4 q) {
	const float2 px = pair(q.x), py = pair(q.y), pz = pair(q.z);
	f3x2 r;
	r.x = padd<P>(mad2<P>(m.c[2].x, pz, mad2<P>(m.c[1].x, py, pmul<P>(m.c[0].x, px))), m.c[3].x);
	r.y = padd<P>(mad2<P>(m.c[2].y, pz, mad2<P>(m.c[1].y, py, pmul<P>(m.c[0].y, px))), m.c[3].y);
	r.z = padd<P>(mad2<P>(m.c[2].z, pz, mad2<P>(m.c[1].z, py, pmul<P>(m.c[0].z, px))), m.c[3].z);
	return r;
}
template <class P> RL_DEV float2 dot2(const f3x2& a, const f3x2& b) {
	return mad2<P>(a.z, b.z, mad2<P>(a.y, b.y, pmul<P>(a.x, b.x)));
}
template <class P> RL_DEV f3x2 normalize2(const f3x2& a) {
	const float2 d = dot2<P>(a, a);
	const float2 s = make_float2(P::rsqrt(d.x), P::rsqrt(d.y));
	return {pmul<P>(a.x, s), pmul<P>(a.y, s), pmul<P>(a.z, s)};
}
// normalize2 with the branch-free square root of normalize_checked (exact
// numerics; ok cleared outside its range).
template <class P> RL_DEV f3x2 normalize2_checked(const f3x2& a, bool& ok) { return normalize2<P>(a); }
template <> RL_DEV f3x2 normalize2_checked<ExactNumerics>(const f3x2& a, bool& ok) {
	const float2 d = dot2<ExactNumerics>(a, a);
	ok = ok && tuckerman_range(d.x) && tuckerman_range(d.y);
	const float2 s = make_float2(rcp_markstein(sqrt_tuckerman(d.x)), rcp_markstein(sqrt_tuckerman(d.y)));
	return {pmul<ExactNumerics>(a.x, s), pmul<ExactNumerics>(a.y, s), pmul<ExactNumerics>(a.z, s)};
}
// integrate_edge on both lanes.
template <class P> RL_DEV float2 integrate_edge2(const f3x2& v1, const f3x2& v2) {
	const float2 x = dot2<P>(v1, v2);
	const float2 y = make_float2(fabsf(x.x), fabsf(x.y));
	const float2 a = padd<P>(pair(0.8543985f), pmul<P>(mad2<P>(pair(0.0145206f), y, pair(0.4965155f)), y));
	const float2 b = padd<P>(pair(3.4175940f), pmul<P>(padd<P>(pair(4.1616724f), y), y));
	float2 ts = make_float2(P::div_edge(a.x, b.x), P::div_edge(a.y, b.y));
	if (!(x.x > 0.0f)) ts.x = 0.5f * P::rsqrt(fmax_glsl(1.0f - x.x * x.x, 1e-7f)) - ts.x;
	if (!(x.y > 0.0f)) ts.y = 0.5f * P::rsqrt(fmax_glsl(1.0f - x.y * x.y, 1e-7f)) - ts.y;
	const float2 cz = padd<P>(pmul<P>(v1.x, v2.y), pmul<P>(make_float2(-v1.y.x, -v1.y.y), v2.x));
	return pmul<P>(cz, ts);
}

template <class P, bool kChecked = false>
RL_DEV bool binned_candidate_pair(const float4* f, const float4* record, bool allow_clip, float& p_hat) {
	bool ok = true;
	const float4 head = __ldg(record), pl = __ldg(record + 1);
	const uint32_t n = __float_as_uint(head.w);
	const float plane[4] = {pl.x, pl.y, pl.z, pl.w};
	const float4 f0 = f[0];
	const bool flip = plane_dot(mk3(f0.x, f0.y, f0.z), plane) < 0.0f;
	// Lane .x: world to shading space (y negated on a flip); lane .y: world
	// to cosine space (the y-flipped matrix on a flip).
	const mat43 ms = load_matrix(f + 2), mc = load_matrix(f + (flip ? 8 : 5));
	mat43x2 t;
#pragma unroll
	for (int c = 0; c != 4; ++c) {
		t.c[c].x = make_float2(ms.c[c].x, mc.c[c].x);
		t.c[c].y = make_float2(ms.c[c].y, mc.c[c].y);
		t.c[c].z = make_float2(ms.c[c].z, mc.c[c].z);
	}
	// Vertices 0 and 1 first; then iteration j normalises vertex j + 1 while
	// it integrates edge (j - 1, j), so the two dependency chains overlap.
	// The edges are added in calculate_ltc's order: (0, 1), ..., (n - 2,
	// n - 1), then (n - 1, 0).
	const float4 q0 = __ldg(record + 2), q1 = __ldg(record + 3);
	float4 q = __ldg(record + 4);
	f3x2 v = mul_point2<P>(t, q0);
	if (flip) v.y.x = -v.y.x;
	uint32_t above_s = v.z.x > 0.0f ? 1u : 0u, above_c = v.z.y > 0.0f ? 1u : 0u;  // bit j: vertex j above
	const f3x2 first = kChecked ? normalize2_checked<P>(v, ok) : normalize2<P>(v);
	v = mul_point2<P>(t, q1);
	if (flip) v.y.x = -v.y.x;
	above_s |= (v.z.x > 0.0f ? 1u : 0u) << 1;
	above_c |= (v.z.y > 0.0f ? 1u : 0u) << 1;
	f3x2 prev = first, cur = kChecked ? normalize2_checked<P>(v, ok) : normalize2<P>(v);
	float2 r = pair(0.0f);
#pragma unroll kPairUnroll
	for (uint32_t j = 1; j != n; ++j) {
		f3x2 next = first;
		if (j + 1 != n) {
			v = mul_point2<P>(t, q);
			if (flip) v.y.x = -v.y.x;
			q = __ldg(record + 2 + min(j + 2, (uint32_t) kMaxLightVertices - 1));
			above_s |= (v.z.x > 0.0f ? 1u : 0u) << (j + 1);
			above_c |= (v.z.y > 0.0f ? 1u : 0u) << (j + 1);
			next = kChecked ? normalize2_checked<P>(v, ok) : normalize2<P>(v);
		}
		r = padd<P>(r, integrate_edge2<P>(prev, cur));
		prev = cur;
		cur = next;
	}
	r = padd<P>(r, integrate_edge2<P>(prev, first));
	if (kChecked && !ok) return false;
	const uint32_t all = (1u << n) - 1u;
	const bool partial_s = above_s != all && above_s != 0, partial_c = above_c != all && above_c != 0;
	if ((partial_s || partial_c) && !allow_clip) return false;
	float integral[2];
	bool away[2];
	const uint32_t above[2] = {above_s, above_c};
	const float sum[2] = {r.x, r.y};
#pragma unroll
	for (int s = 0; s != 2; ++s) {
		float rs = sum[s];
		bool a = false;
		if (above[s] == all) {
			rs = fabsf(rs);
		} else if (above[s] == 0) {
			rs = 0.0f;
			a = true;
		} else {
			const mat43 ts = s == 0 ? ms : mc;
			bool unused = true;
			rs = clipped_integral<P, false>(ts, record, n, s == 0 && flip, above[s], unused);
			a = rs < 0.0f;
			rs = a ? 0.0f : rs;
		}
		integral[s] = rs;
		away[s] = a;
	}
	const f3 radiance = mk3(head.x, head.y, head.z);
	f3 result = splat(0.0f);
	const float4 f1 = f[1];
	const f3 diffuse = away[0] ? splat(0.0f) : mul(scale(mk3(f1.x, f1.y, f1.z), integral[0]), radiance);
	result = add(result, diffuse);
	const f3 ggx = away[1] ? splat(0.0f) : mul(splat(integral[1] * f[0].w), radiance);
	const f3 color = add(result, ggx);
	p_hat = P::sqrt(dot(color, color));
	return true;
}

// The candidate evaluation the binned kernel uses: the paired form in fast
// numerics (measured 12% faster there: 0.325 against 0.290 Gsamples/s on
// the 1080p 16K-light frame), the sequential scalar form in exact numerics,
// where the paired structure with one scalar operation per lane measured
// slower (29.4 against 24.7 ms per 4-frame launch of the candidate kernel).
// RISLTC_CANDIDATE_PAIRS=1 selects the paired form for exact numerics too.
template <class P>
RL_DEV bool evaluate_candidate(const float4* f, const float4* record, bool allow_clip, float& p_hat) {
#if RISLTC_CANDIDATE_PAIRS
	return allow_clip ? binned_candidate_pair<P, false>(f, record, true, p_hat)
	                  : binned_candidate_pair<P, true>(f, record, false, p_hat);
#else
	// The first pass (allow_clip false) takes the branch-free square root;
	// deferred items are evaluated with the general one.
	if (!allow_clip) return binned_candidate<P, true>(f, record, false, p_hat);
	// Deferred items: the branch-free forms where they apply (every item
	// seen so far), the general ones otherwise.
	return binned_candidate<P, true>(f, record, true, p_hat) || binned_candidate<P, false>(f, record, true, p_hat);
#endif
}
template <>
RL_DEV bool evaluate_candidate<FastNumerics>(const float4* f, const float4* record, bool allow_clip, float& p_hat) {
	return binned_candidate_pair<FastNumerics>(f, record, allow_clip, p_hat);
}

// One warp tile t (pixels t * kPixels .. + kPixels - 1) of one frame set:
// candidates, evaluation, replay and reservoir records for all frames.
// tile is the warp's shared-memory tile, phat its p_hat slot.
template <class P, int kPixels, int kChunk>
RL_DEV void binned_tile(const RisParams& pr, WarpTile<BinnedSuper<P>::value, kPixels, kChunk>& tile, float* phat,
                        uint32_t t) {
	constexpr int kSuper = BinnedSuper<P>::value;
	const uint32_t lane = threadIdx.x % 32;
	const uint32_t np = pr.width * pr.height;
	const int n_lights = pr.scene.light_count;
	const float p = P::rcp((float) n_lights);
	// With uniform candidates and a power-of-two light count, p is a power of
	// two and p_hat / p equals p_hat * (1 / p) bit for bit (scaling by a
	// power of two is exact): the replay multiplies instead of dividing.
	const bool scale_weight = !pr.candidates && (n_lights & (n_lights - 1)) == 0;
	const float inv_p = (float) n_lights;
	// Lanes kPixels..31 own no pixel: they draw nothing and only evaluate
	// items of the sorted lists.
	const bool own = lane < (uint32_t) kPixels;
	{
		const uint32_t i = t * kPixels + lane;
		const bool valid = own && i < np && !(pr.primitive && pr.primitive[i] == 0xffffffffu);
		if (valid) {
			const float* g = pr.gbuffer;
			const size_t snp = np;
			const f3 position = mk3(g[0 * snp + i], g[1 * snp + i], g[2 * snp + i]);
			const f3 normal = mk3(g[3 * snp + i], g[4 * snp + i], g[5 * snp + i]);
			const f3 outgoing = mk3(g[6 * snp + i], g[7 * snp + i], g[8 * snp + i]);
			const f3 fresnel_0 = mk3(g[13 * snp + i], g[14 * snp + i], g[15 * snp + i]);
			const float roughness = g[16 * snp + i];
			CandidateFrame cf;
			cf.position = position;
			cf.diffuse_albedo = mk3(g[10 * snp + i], g[11 * snp + i], g[12 * snp + i]);
			const float fl = dot(fresnel_0, mk3(0.2126f, 0.7152f, 0.0722f));
			const Ltc ltc = get_ltc_coefficients<P>(pr.scene, fl, roughness, position, normal, outgoing);
			cf.ltc_albedo = ltc.albedo;
			cf.w2s = ltc.world_to_shading;
			mat43 flipped = ltc.world_to_shading;
#pragma unroll
			for (int c = 0; c != 4; ++c) flipped.c[c].y = -flipped.c[c].y;
			cf.w2c[0] = mul(ltc.shading_to_cosine, cf.w2s);
			cf.w2c[1] = mul(ltc.shading_to_cosine, flipped);
			store_frame(tile.frame[lane], cf);
		}
		__syncwarp();
		const uint32_t x = i % pr.width, y = i / pr.width;
		// The noise state at the start of frame f (get_noise_accessor with
		// the frame's random offset).
		auto frame_seed = [&](uint32_t f) -> uint32_t {
			if (!valid) return 0u;
			const uint32_t rn_x = pr.animate ? wang_random_number((pr.noise_seed + f) * 4u) : 0u;
			return get_noise_accessor(x, y, pr.width, rn_x);
		};
		// The tile's work comes in units of one frame's super-chunk.  Up to
		// kWindow units are evaluated before their reservoirs are replayed, so
		// that deferred items of several units share the general path's
		// rounds: unit u of the window keeps its p_hat values at
		// phat[u * kUnitSlots + slot].
		constexpr uint32_t kUnitSlots = (uint32_t) (kPixels * kSuper);
		constexpr uint32_t kWindow = (uint32_t) kPHatSlot / kUnitSlots;
		const uint32_t units_per_frame = ((uint32_t) pr.candidate_count + kSuper - 1) / kSuper;
		const uint32_t units = pr.frame_count * units_per_frame;
		// The replay's cursor: frame rf, its next super-chunk rcs, and the
		// frame's reservoir so far.
		uint32_t rf = 0, rcs = 0, seed = 0;
		float w_sum = 0.0f, sample_value = 0.0f;
		int res_index = -1;
		uint32_t window = 0;  // units evaluated since the last replay
		uint32_t draw = 0;    // the draw phase's noise state
		if (lane == 0) tile.deferred_count = 0;
		__syncwarp();
		for (uint32_t unit = 0; unit != units; ++unit) {
			const uint32_t f = unit / units_per_frame, cs = (unit % units_per_frame) * kSuper;
			if (cs == 0) draw = frame_seed(f);
			const int super_count = min(kSuper, pr.candidate_count - (int) cs);
			float* const uphat = phat + window * kUnitSlots;
			{
				for (int c0 = 0; c0 < super_count; c0 += kChunk) {
					const int chunk = min(kChunk, super_count - c0);
					// 1. This lane's candidate lights; bin them by vertex count
					//    (six 10-bit counters).
					int light[kChunk];
					uint32_t bin[kChunk];
					unsigned long long counts = 0;
#pragma unroll
					for (int k = 0; k != kChunk; ++k) {
						light[k] = -1;
						bin[k] = kBins;
						if (valid && k < chunk) {
							int idx = (int) (get_noise_1(draw) * (float) n_lights);
							idx = idx > n_lights - 1 ? n_lights - 1 : idx;
							if (pr.candidates)
								idx = pr.candidates[((size_t) f * np + i) * pr.candidate_count + cs + c0 + k].light;
							get_noise_1(draw);
							light[k] = idx;
							bin[k] = light_vertex_count(pr.scene, idx) - 3u;
							counts += 1ull << (10 * bin[k]);
						}
					}
					// 2. Counting sort: exclusive scan of the counters across
					//    the warp, then each bin's start.
					unsigned long long prefix = counts;
#pragma unroll
					for (int d = 1; d < 32; d <<= 1) {
						const unsigned long long o = __shfl_up_sync(0xffffffffu, prefix, d);
						if ((int) lane >= d) prefix += o;
					}
					const unsigned long long totals = __shfl_sync(0xffffffffu, prefix, 31);
					prefix -= counts;
					uint32_t start[kBins + 1];
					start[0] = 0;
#pragma unroll
					for (int b = 0; b != kBins; ++b)
						start[b + 1] = start[b] + (uint32_t) ((totals >> (10 * b)) & 1023u);
					const uint32_t item_count = start[kBins];
#pragma unroll
					for (int k = 0; k != kChunk; ++k) {
						if (bin[k] < kBins) {
							const uint32_t b = bin[k];
							uint32_t s = 0;
#pragma unroll
							for (int q = 0; q != kBins; ++q)
								if (q == (int) b) s = start[q];
							const uint32_t pos = s + (uint32_t) ((prefix >> (10 * b)) & 1023u);
							prefix += 1ull << (10 * b);
							tile.item[pos] = ((uint32_t) light[k] << 10) | (lane * kSuper + c0 + k);
						}
					}
					__syncwarp();
					// 3. Evaluate the sorted items, 32 at a time; defer partial
					//    clips (with their unit), and evaluate deferred items
					//    whenever 32 are pending.
					for (uint32_t base = 0; base < item_count; base += 32) {
						const uint32_t it = base + lane;
						if (it < item_count) {
							const uint32_t item = tile.item[it];
							const uint32_t slot = item & 1023u;
							const int32_t l = (int32_t) (item >> 10);
							float ph;
							if (evaluate_candidate<P>(tile.frame[slot / kSuper], light_record(pr.scene, l), false, ph)) {
								uphat[slot] = ph;
							} else {
								const uint32_t d = atomicAdd(&tile.deferred_count, 1u);
								tile.deferred[d] = item;
								tile.deferred_unit[d] = (uint8_t) window;
							}
						}
					}
					__syncwarp();
					for (uint32_t pending = tile.deferred_count; pending >= 32; pending -= 32) {
						const uint32_t d = pending - 32 + lane;
						const uint32_t slot = tile.deferred[d] & 1023u;
						float ph = 0.0f;
						evaluate_candidate<P>(tile.frame[slot / kSuper], light_record(pr.scene, (int) (tile.deferred[d] >> 10)),
						                      true, ph);
						phat[tile.deferred_unit[d] * kUnitSlots + slot] = ph;
						__syncwarp();
						if (lane == 0) tile.deferred_count = pending - 32;
						__syncwarp();
					}
				}
			}
			++window;
			if (window != kWindow && unit + 1 != units) continue;
			// The window's remaining deferred items.
			const uint32_t rest = tile.deferred_count;
			if (lane < rest) {
				const uint32_t slot = tile.deferred[lane] & 1023u;
				float ph = 0.0f;
				evaluate_candidate<P>(tile.frame[slot / kSuper], light_record(pr.scene, (int) (tile.deferred[lane] >> 10)),
				                      true, ph);
				phat[tile.deferred_unit[lane] * kUnitSlots + slot] = ph;
			}
			__syncwarp();
			if (lane == 0) tile.deferred_count = 0;
			__syncwarp();
			// 4. Reservoir updates of the window's units in candidate order,
			//    drawing the same noise again; a frame's record is written
			//    after its last super-chunk.
			for (uint32_t u = 0; u != window; ++u) {
				if (rcs == 0) {
					seed = frame_seed(rf);
					w_sum = 0.0f;
					sample_value = 0.0f;
					res_index = -1;
				}
				const int rcount = min(kSuper, pr.candidate_count - (int) rcs);
				const float* const rphat = phat + u * kUnitSlots + lane * kSuper;
				if (valid) {
#pragma unroll 4
					for (int k = 0; k < rcount; ++k) {
						int idx = (int) (get_noise_1(seed) * (float) n_lights);
						idx = idx > n_lights - 1 ? n_lights - 1 : idx;
						float pk = p;
						if (pr.candidates) {
							const ProposalCandidate q =
							    pr.candidates[((size_t) rf * np + i) * pr.candidate_count + rcs + k];
							idx = q.light;
							pk = q.pdf;
						}
						const float rnd = get_noise_1(seed);
						const float p_hat = rphat[k];
						const float w = scale_weight ? p_hat * inv_p : P::div(p_hat, pk);
						if (pr.train_stride && rf == 0 && i % pr.train_stride == pr.train_phase)
							pr.train_candidates[(size_t) i * pr.candidate_count + rcs + k].pdf = w;
						w_sum += w;
						if (w > 0.0f && rnd < P::div(w, w_sum)) {
							res_index = idx;
							sample_value = p_hat;
						}
					}
				}
				rcs += kSuper;
				if (rcs >= (uint32_t) pr.candidate_count) {
					if (valid)
						pr.records[(size_t) rf * np + i] = ReservoirRecord{res_index, w_sum, sample_value, seed};
					else if (own && i < np)
						pr.records[(size_t) rf * np + i] = ReservoirRecord{-1, 0.0f, 0.0f, 0u};
					++rf;
					rcs = 0;
				}
			}
			window = 0;
			__syncwarp();
		}
		__syncwarp();
	}
}

template <class P, int kPixels, int kChunk>
__global__ void __launch_bounds__(32 * kBinnedWarps, BinnedMinBlocks<P>::value)
ris_candidates_binned_kernel(const __grid_constant__ RisParams pr) {
	extern __shared__ __align__(16) unsigned char smem_raw[];
	using Tile = WarpTile<BinnedSuper<P>::value, kPixels, kChunk>;
	Tile& tile = reinterpret_cast<Tile*>(smem_raw)[threadIdx.x / 32];
	float* const phat = pr.p_hat_scratch + (size_t) (blockIdx.x * kBinnedWarps + threadIdx.x / 32) * kPHatSlot;
	const uint32_t tiles = (pr.width * pr.height + kPixels - 1) / kPixels;
	for (uint32_t t = next_warp_tile(pr.tile_cursor); t < tiles; t = next_warp_tile(pr.tile_cursor))
		binned_tile<P, kPixels, kChunk>(pr, tile, phat, t);
}

template <class P, int kPixels, int kChunk> constexpr size_t binned_smem_bytes() {
	return sizeof(WarpTile<BinnedSuper<P>::value, kPixels, kChunk>) * kBinnedWarps;
}

// First launch of a candidate kernel on a device: raises its shared-memory
// limit (above the 48 KB available without opting in) and stores in
// resident[device] the blocks that fit on the device at once (resident
// blocks per SM times the SM count), the kernel's persistent grid: one wave
// whose warps take tiles from the launch's cursor until none is left.  Done once
// per device, so that later launches, including those captured into a CUDA
// graph, make no other runtime call.
template <class Kernel>
cudaError_t configure_candidate_kernel(Kernel kernel, size_t smem, std::atomic<uint64_t>& configured,
                                       std::atomic<int>* resident, int& device) {
	cudaError_t e = cudaGetDevice(&device);
	if (e != cudaSuccess) return e;
	const uint64_t bit = 1ull << (device & 63);
	if (configured.load() & bit) return cudaSuccess;
	e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int) smem);
	int sms = 0, per_sm = 0;
	if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
	if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, 32 * kBinnedWarps, smem);
	if (e != cudaSuccess) return e;
	resident[device & 63].store(std::max(1, sms * std::min(per_sm, kCandidateBlocksPerSm)));
	configured.fetch_or(bit);
	return cudaSuccess;
}

// Launches the binned candidate kernel.  Its shared memory exceeds the 48 KB
// available without opting in, so the limit is raised the first time the
// kernel runs on a device (once, so that later launches, including those
// captured into a CUDA graph, make no other runtime call).
// grid_cap is the largest grid the p_hat scratch has warp slots for.
template <class P, int kPixels, int kChunk>
cudaError_t launch_candidates_binned(const RisParams& p, cudaStream_t stream, int grid_cap) {
	const size_t pixels = (size_t) p.width * p.height;
	const size_t blocks = (pixels + kPixels * kBinnedWarps - 1) / (kPixels * kBinnedWarps);
	const int grid = (int) std::max<size_t>(1, std::min<size_t>(blocks, (size_t) grid_cap));
	// Without p_hat scratch (the allocation-free entry point), the kernel with
	// one thread per pixel computes the same records.
	if (!p.p_hat_scratch) {
		ris_candidates_kernel<P><<<grid_for_pixels(pixels, grid_cap), 128, 0, stream>>>(p);
		return cudaGetLastError();
	}
	static std::atomic<uint64_t> configured{0};
	static std::atomic<int> resident[64];
	int device = 0;
	const cudaError_t e = configure_candidate_kernel(ris_candidates_binned_kernel<P, kPixels, kChunk>,
	                                                 binned_smem_bytes<P, kPixels, kChunk>(), configured, resident, device);
	if (e != cudaSuccess) return e;
	const cudaError_t z = cudaMemsetAsync(p.tile_cursor, 0, sizeof(uint32_t), stream);
	if (z != cudaSuccess) return z;
	ris_candidates_binned_kernel<P, kPixels, kChunk>
	    <<<std::min(grid, resident[device & 63].load()), 32 * kBinnedWarps, binned_smem_bytes<P, kPixels, kChunk>(),
	       stream>>>(p);
	return cudaGetLastError();
}

}  // namespace risltc
