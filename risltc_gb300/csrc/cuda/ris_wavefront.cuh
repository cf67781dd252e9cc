// ris_wavefront.cuh - the shading phase of the two-kernel pipeline with its
// shadow rays traced in a separate pass:
//
//   ris_sample_kernel: per pixel and frame, the estimator of
//     evaluate_polygonal_light_shading_peters (shading_pass.frag.glsl:292-397)
//     for the chosen light up to the visibility test.  For each of its (at
//     most two) samples it stores the MIS-weighted contribution for both
//     outcomes of the shadow ray and stages the ray.
//   light_bucket_scan_kernel, shadow_scatter_kernel: group the rays by light
//     (a counting sort), so that the rays of one warp start near each other
//     and aim at the same polygon.
//   shadow_trace_kernel: one any-hit query per queued ray, with a small
//     register footprint and no divergence from the shading code around it.
//   ris_resolve_kernel: per pixel, picks each sample's contribution by its
//     ray's outcome and finishes the frame and the accumulation exactly as
//     ris_shade_kernel does.
// The contributions are the same operations on the same values, added in
// the same order, so the pixels are bit-identical to ris_shade_kernel's.
// Used for one sample per technique (SAMPLE_COUNT == 1, the reference's
// default) with shadows on.
// Restates upstream risltc routines (GPLv3): see NOTICE.
#pragma once
#include "ris_kernels.cuh"

namespace risltc {

// Per-sample mode, two bits per technique j in SampleRecord::flags.
enum : uint32_t {
	kSampleSkip = 0,    // no contribution (dir.z <= 0 or no such sample)
	kSampleFixed = 1,   // contribution c[j][0], no ray needed
	kSampleTraced = 2,  // c[j][0] if the ray is unoccluded, else c[j][1]
	kSampleNoLight = 1u << 8,  // empty reservoir: the frame's colour is zero
};

// The estimator's state between the sample and resolve kernels (64 bytes).
struct SampleRecord {
	float c[2][2][3];  // [technique][unoccluded, occluded][rgb]
	float W;           // the reservoir's unbiased contribution weight
	uint32_t flags;
	uint32_t pad[2];
};
static_assert(sizeof(SampleRecord) == 64, "SampleRecord layout");

// A queued shadow ray: origin and the hit slot (2 * pixel-frame + technique),
// direction and t_max (t_min is get_polygon_visibility's 1e-3).
struct ShadowRay {
	float4 origin_slot;
	float4 dir_tmax;
};

// Technique j's two contributions (unoccluded, occluded) into floats
// 6j .. 6j + 5 of a sample record.
RL_DEV void store_contributions(SampleRecord* dst, int j, f3 c0, f3 c1) {
	float* f = reinterpret_cast<float*>(dst);
	if (j == 0) {
		*reinterpret_cast<float4*>(f) = make_float4(c0.x, c0.y, c0.z, c1.x);
		*reinterpret_cast<float2*>(f + 4) = make_float2(c1.y, c1.z);
	} else {
		*reinterpret_cast<float2*>(f + 6) = make_float2(c0.x, c0.y);
		*reinterpret_cast<float4*>(f + 8) = make_float4(c0.z, c1.x, c1.y, c1.z);
	}
}

// evaluate_polygonal_light_shading_peters for SAMPLE_COUNT == 1 up to the
// visibility test.  Writes both techniques' contributions into *dst (zero
// where a technique has none) and each traced technique's shadow ray into
// staged[j] as soon as they are known, and returns the techniques' modes.
// l is the light whose device record is `record`; poly is the thread's
// polygon buffer.
template <class P>
RL_DEV uint32_t psa_mis_emit(const ShadeParams& pr, const ShadingData& sd, Ltc ltc, const Light& l,
                             const float4* record, uint32_t& seed, SampleRecord* dst, ShadowRay* staged,
                             PsaPolygon& poly) {
	const bool fa = pr.fast_atan != 0;
	const bool biased = pr.technique == sample_polygon_projected_solid_angle_biased;
	side_flip(ltc, sd, l);
	// One polygon buffer serves both spaces: the shading-space polygon is
	// prepared and sampled, then the cosine-space one is prepared into the
	// same storage and sampled (if it has a projected solid angle).  The
	// samples draw the noise in the reference's order (diffuse, then
	// specular), and after sampling only the projected solid angles are
	// needed, so the values equal those of psa_prepare_both followed by both
	// samples.
	float psa[2] = {0.0f, 0.0f};
	int technique_count = 1;
	f3 dir_d = mk3(0.0f, 0.0f, 1.0f), dir_s = mk3(0.0f, 0.0f, 1.0f);
#pragma unroll 1
	for (int j = 0; j != 2; ++j) {
		const uint32_t vc = prepare_space_record<P>(j == 0 ? ltc.world_to_shading
		                                                  : mul(ltc.shading_to_cosine, ltc.world_to_shading),
		                                           record, poly, fa);
		psa[j] = vc == 0 ? 0.0f : poly.psa;
		if (j == 0 && (vc == 0 || psa[0] == 0.0f)) {
			store_contributions(dst, 0, splat(0.0f), splat(0.0f));
			store_contributions(dst, 1, splat(0.0f), splat(0.0f));
			return 0;
		}
		if (j == 1 && !(psa[1] > 0.0f)) break;
		const f3 dir = sample_psa<P>(poly, get_noise_2(seed), fa, biased);
		if (j == 0) {
			dir_d = dir;
		} else {
			dir_s = normalize<P>(mul(ltc.cosine_to_shading, dir));
			technique_count = 2;
		}
	}
	float specular_weight = ltc.albedo * psa[1];
	f3 diffuse_weight = scale(max3(sd.diffuse_albedo, splat(0.01f)), psa[0]);
	float rcp_d = P::rcp(psa[0]);
	float rcp_s = P::rcp(psa[1]);
	f3 specular_weight_rgb = splat(specular_weight);
	if (pr.mis_heuristic == mis_heuristic_optimal) {
		f3 rop = scale(l.radiance, kInvPi);
		diffuse_weight = mul(diffuse_weight, rop);
		specular_weight_rgb = mul(specular_weight_rgb, rop);
	}
	const bool shadows = pr.shadows && pr.scene.triangle_count != 0;
	uint32_t modes = 0;
#pragma unroll 1
	for (int j = 0; j != 2; ++j) {
		f3 dir = (j == 0) ? dir_d : dir_s;
		if (j >= technique_count || dir.z <= 0.0f) {
			store_contributions(dst, j, splat(0.0f), splat(0.0f));
			continue;
		}
		float diffuse_density = dir.z * rcp_d;
		float specular_density = evaluate_ltc_density<P>(ltc, dir, rcp_s);
		f3 world_dir = transpose_mul(ltc.world_to_shading, dir);
		const bool side = dot(sd.normal, world_dir) > 0.0f;
		const bool traced = side && shadows;
		const f3 rb_lit = side ? mul(l.radiance, evaluate_brdf<P>(sd, world_dir)) : splat(0.0f);
		// This technique's weight and density first, the other's second.
		const f3 own_weight = j == 0 ? diffuse_weight : specular_weight_rgb;
		const f3 other_weight = j == 0 ? specular_weight_rgb : diffuse_weight;
		const float own_density = j == 0 ? diffuse_density : specular_density;
		const float other_density = j == 0 ? specular_density : diffuse_density;
		// Outcome 0: visible iff side (unoccluded or untraced); outcome 1:
		// occluded.
		f3 c[2] = {splat(0.0f), splat(0.0f)};
#pragma unroll 1
		for (int o = 0; o != (traced ? 2 : 1); ++o) {
			const bool visibility = (o == 0) ? side : false;
			f3 integrand = scale(visibility ? rb_lit : splat(0.0f), dir.z);
			f3 r;
			if (j == 0 && psa[1] <= 0.0f)
				r = visibility ? scale(integrand, P::rcp(diffuse_density)) : splat(0.0f);
			else
				r = mis_estimate<P>(pr.mis_heuristic, integrand, own_weight, own_density, other_weight, other_density,
				                    pr.mis_visibility_estimate);
			if (o == 0) c[0] = r; else c[1] = r;
		}
		store_contributions(dst, j, c[0], c[1]);
		if (traced) {
			// get_polygon_visibility, shading_pass.frag.glsl:112-129
			float max_t = P::div(-plane_dot(sd.position, l.plane),
			                     world_dir.x * l.plane[0] + world_dir.y * l.plane[1] + world_dir.z * l.plane[2]);
			max_t -= 1e-3f;
			staged[j] = ShadowRay{make_float4(sd.position.x, sd.position.y, sd.position.z, 0.0f),
			                      make_float4(world_dir.x, world_dir.y, world_dir.z, max_t)};
		}
		modes |= (traced ? kSampleTraced : kSampleFixed) << (2 * j);
	}
	return modes;
}

RL_DEV void store_sample(SampleRecord* dst, const f3 (&c)[2][2], float W, uint32_t flags) {
	float4* q = reinterpret_cast<float4*>(dst);
	q[0] = make_float4(c[0][0].x, c[0][0].y, c[0][0].z, c[0][1].x);
	q[1] = make_float4(c[0][1].y, c[0][1].z, c[1][0].x, c[1][0].y);
	q[2] = make_float4(c[1][0].z, c[1][1].x, c[1][1].y, c[1][1].z);
	q[3] = make_float4(W, __uint_as_float(flags), 0.0f, 0.0f);
}

#ifndef RISLTC_SAMPLE_MIN_BLOCKS
#define RISLTC_SAMPLE_MIN_BLOCKS 4
#endif
// Threads per block of the sample kernels.  Each thread's PSA polygon buffer
// (196 bytes, indexed by the sorting network and the sector search) is a
// slot of a shared-memory array: slots are 49 words apart, so the lanes'
// words of one index fall in 32 distinct banks.  In local memory the 16
// resident warps' buffers (about 240 KB per SM) did not stay in L1 (sample
// kernel 5.71 ms per 4-frame 1080p launch, 4.14 ms with the shared slots).
constexpr int kSampleThreads = 128;
// The sample phase of pixel i (all frames of the call); i may be past the
// frame (the thread then does nothing).
template <class P> RL_DEV void sample_pixel(const RisParams& pr, uint32_t i, PsaPolygon& poly) {
	const uint32_t np = pr.width * pr.height;
	ShadeParams sp;  // the fields psa_prepare_both and psa_mis_emit read
	sp.scene = pr.scene;
	sp.technique = sample_polygon_ltc_cp;
	sp.mis_heuristic = pr.mis_heuristic;
	sp.sample_count = 1;
	sp.mis_visibility_estimate = pr.mis_visibility_estimate;
	sp.fast_atan = pr.fast_atan;
	sp.shadows = pr.shadows;
	sp.error = pr.error;
	{
		const bool active = i < np && !(pr.primitive && pr.primitive[i] == 0xffffffffu);
		ShadingData sd;
		Ltc ltc;
		if (active) {
			const float* g = pr.gbuffer;
			const size_t snp = np;
			sd.position = mk3(g[0 * snp + i], g[1 * snp + i], g[2 * snp + i]);
			sd.normal = mk3(g[3 * snp + i], g[4 * snp + i], g[5 * snp + i]);
			sd.outgoing = mk3(g[6 * snp + i], g[7 * snp + i], g[8 * snp + i]);
			sd.lambert_outgoing = g[9 * snp + i];
			sd.diffuse_albedo = mk3(g[10 * snp + i], g[11 * snp + i], g[12 * snp + i]);
			sd.fresnel_0 = mk3(g[13 * snp + i], g[14 * snp + i], g[15 * snp + i]);
			sd.roughness = g[16 * snp + i];
			float fl = dot(sd.fresnel_0, mk3(0.2126f, 0.7152f, 0.0722f));
			ltc = get_ltc_coefficients<P>(pr.scene, fl, sd.roughness, sd.position, sd.normal, sd.outgoing);
		}
		for (uint32_t f = 0; f != pr.frame_count; ++f) {
			const size_t pf = (size_t) f * np + i;
			uint32_t modes = 0;
			int light = -1;
			if (active) {
				const ReservoirRecord r = pr.records[pf];
				light = r.light_index;
				if (r.light_index >= 0) {
					Light l;
					load_light(pr.scene, r.light_index, l);
					uint32_t seed = r.seed;
					// Contributions and staged rays go to memory inside.
					modes = psa_mis_emit<P>(sp, sd, ltc, l, light_record(pr.scene, r.light_index), seed,
					                        pr.samples + pf, pr.staged + 2 * pf, poly);
					float W = P::div(r.w_sum, (float) pr.candidate_count * r.p_hat);
					if (r.p_hat == 0.0f) W = 0.0f;
					*reinterpret_cast<float2*>(reinterpret_cast<float*>(pr.samples + pf) + 12) =
					    make_float2(W, __uint_as_float(modes));
				} else {
					const f3 zero[2][2] = {{splat(0.0f), splat(0.0f)}, {splat(0.0f), splat(0.0f)}};
					store_sample(pr.samples + pf, zero, 0.0f, kSampleNoLight);
				}
			}
			// Count the staged rays for their light's bucket.
			const bool t0 = (modes & 3u) == kSampleTraced, t1 = ((modes >> 2) & 3u) == kSampleTraced;
			if (t0 || t1) atomicAdd(pr.light_rays + (size_t) light * kLightCounterStride, (t0 ? 1u : 0u) + (t1 ? 1u : 0u));
		}
	}
}

// Each warp takes 32 consecutive pixels at a time from the launch's cursor.
template <class P>
__global__ void __launch_bounds__(kSampleThreads, RISLTC_SAMPLE_MIN_BLOCKS) ris_sample_kernel(const __grid_constant__ RisParams pr) {
	__shared__ PsaPolygon poly[kSampleThreads];
	const uint32_t np = pr.width * pr.height;
	const uint32_t chunks = (np + 31) / 32;
	for (uint32_t c = next_warp_tile(pr.sample_cursor); c < chunks; c = next_warp_tile(pr.sample_cursor))
		sample_pixel<P>(pr, c * 32 + threadIdx.x % 32, poly[threadIdx.x]);
}

// Exclusive prefix sum of the per-light ray counts, in place (each becomes
// its bucket's first queue position); the total goes to ray_count[0] and the
// trace kernel's fetch cursor ray_count[1] is reset.  One block of 1024
// threads.
RL_DEV void light_bucket_scan(uint32_t* light_rays, uint32_t light_count, uint32_t* ray_count) {
	__shared__ uint32_t warp_offset[32];
	__shared__ uint32_t chunk_total;
	const uint32_t lane = threadIdx.x % 32, warp = threadIdx.x / 32;
	uint32_t carry = 0;
	for (uint32_t base = 0; base < light_count; base += 1024) {
		const uint32_t i = base + threadIdx.x;
		const uint32_t v = i < light_count ? light_rays[(size_t) i * kLightCounterStride] : 0u;
		uint32_t incl = v;
#pragma unroll
		for (int d = 1; d < 32; d <<= 1) {
			const uint32_t o = __shfl_up_sync(0xffffffffu, incl, d);
			if ((int) lane >= d) incl += o;
		}
		if (lane == 31) warp_offset[warp] = incl;
		__syncthreads();
		if (warp == 0) {
			const uint32_t w = warp_offset[lane];
			uint32_t wi = w;
#pragma unroll
			for (int d = 1; d < 32; d <<= 1) {
				const uint32_t o = __shfl_up_sync(0xffffffffu, wi, d);
				if ((int) lane >= d) wi += o;
			}
			warp_offset[lane] = wi - w;
			if (lane == 31) chunk_total = wi;
		}
		__syncthreads();
		if (i < light_count) light_rays[(size_t) i * kLightCounterStride] = carry + warp_offset[warp] + incl - v;
		carry += chunk_total;
		__syncthreads();
	}
	if (threadIdx.x == 0) {
		ray_count[0] = carry;
		ray_count[1] = 0;  // the trace kernel's fetch cursor
	}
}
static __global__ void __launch_bounds__(1024) light_bucket_scan_kernel(uint32_t* light_rays, uint32_t light_count,
                                                                 uint32_t* ray_count) {
	light_bucket_scan(light_rays, light_count, ray_count);
}

// Moves the staged rays into their light's bucket, tagging each with its hit
// slot.
// The staged rays of pixel-frame pf into their light's bucket.
RL_DEV void scatter_pixel_frame(const RisParams& pr, size_t pf) {
	const uint32_t np = pr.width * pr.height;
	{
		const uint32_t i = (uint32_t) (pf % np);
		if (pr.primitive && pr.primitive[i] == 0xffffffffu) return;
		const uint32_t flags = __float_as_uint(reinterpret_cast<const float4*>(pr.samples + pf)[3].y);
		if (flags & kSampleNoLight) return;
		const bool t0 = (flags & 3u) == kSampleTraced, t1 = ((flags >> 2) & 3u) == kSampleTraced;
		if (!t0 && !t1) return;
		uint32_t at = atomicAdd(pr.light_rays + (size_t) pr.records[pf].light_index * kLightCounterStride,
		                        (t0 ? 1u : 0u) + (t1 ? 1u : 0u));
		const uint32_t slot = 2u * (uint32_t) pf;
		if (t0) {
			ShadowRay q = pr.staged[2 * pf];
			q.origin_slot.w = __uint_as_float(slot);
			pr.rays[at++] = q;
		}
		if (t1) {
			ShadowRay q = pr.staged[2 * pf + 1];
			q.origin_slot.w = __uint_as_float(slot + 1);
			pr.rays[at] = q;
		}
	}
}
static __global__ void __launch_bounds__(128) shadow_scatter_kernel(const __grid_constant__ RisParams pr) {
	const size_t total = (size_t) pr.width * pr.height * pr.frame_count;
	for (size_t pf = blockIdx.x * (size_t) blockDim.x + threadIdx.x; pf < total; pf += (size_t) gridDim.x * blockDim.x)
		scatter_pixel_frame(pr, pf);
}

#ifndef RISLTC_TRACE_MIN_BLOCKS
#define RISLTC_TRACE_MIN_BLOCKS 1
#endif
#ifndef RISLTC_TRACE_REFILL
#define RISLTC_TRACE_REFILL 8
#endif
// Persistent any-hit tracing of the queue (queue[0] rays; queue[1] is the
// fetch cursor, zero at launch).  Each lane holds one ray and advances it by
// one unit of work (a triangle test or an inner node) per iteration;
// whenever RISLTC_TRACE_REFILL or more lanes of a warp are idle they fetch
// the next rays together, so lanes do not wait for the warp's longest ray.
template <class P>
__global__ void __launch_bounds__(128, RISLTC_TRACE_MIN_BLOCKS) shadow_trace_kernel(SceneView s, const ShadowRay* rays, uint32_t* queue,
                                                           uint8_t* hits, uint32_t* error) {
	const uint32_t n = queue[0];
	const uint32_t lane = threadIdx.x % 32;
	int32_t stack[kBvhStack];
	TraceRay r;
	uint32_t slot = 0;
	bool busy = false, drained = false;
	for (;;) {
		const uint32_t idle = __ballot_sync(0xffffffffu, !busy);
		if (drained && idle == 0xffffffffu) break;
		if (!drained && __popc(idle) >= RISLTC_TRACE_REFILL) {
			const int leader = __ffs(idle) - 1;
			uint32_t base = 0;
			if ((int) lane == leader) base = atomicAdd(queue + 1, (uint32_t) __popc(idle));
			base = __shfl_sync(0xffffffffu, base, leader);
			drained = base + (uint32_t) __popc(idle) >= n;
			if (!busy) {
				const uint32_t k = base + (uint32_t) __popc(idle & ((1u << lane) - 1u));
				if (k < n) {
					const float4 a = __ldg(&rays[k].origin_slot), b = __ldg(&rays[k].dir_tmax);
					slot = __float_as_uint(a.w);
					const int st = trace_begin<P>(s, r, mk3(a.x, a.y, a.z), mk3(b.x, b.y, b.z), 1.0e-3f, b.w);
					if (st == kTraceContinue)
						busy = true;
					else
						hits[slot] = st == kTraceHit ? 1 : 0;
				}
			}
			continue;
		}
		if (busy) {
			const int st = trace_step<P>(s, r, stack, error);
			if (st != kTraceContinue) {
				hits[slot] = st == kTraceHit ? 1 : 0;
				busy = false;
			}
		}
	}
}

// The resolve phase of pixel i (all frames of the call).
template <class P> RL_DEV void resolve_pixel(const RisParams& pr, uint32_t i) {
	const uint32_t np = pr.width * pr.height;
	{
		risltc_reservoir_t* res = pr.reservoirs ? pr.reservoirs + i : nullptr;
		if (pr.primitive && pr.primitive[i] == 0xffffffffu) {
			if (res) *res = risltc_reservoir_t{-1, 0.0f, 0.0f, 0u};
			if (pr.out_rgb) {
				pr.out_rgb[3 * (size_t) i + 0] = 0.0f;
				pr.out_rgb[3 * (size_t) i + 1] = 0.0f;
				pr.out_rgb[3 * (size_t) i + 2] = 0.0f;
			}
			return;
		}
		f3 sum = splat(0.0f);
		double acc[3] = {0.0, 0.0, 0.0};
		for (uint32_t f = 0; f != pr.frame_count; ++f) {
			const size_t pf = (size_t) f * np + i;
			const float4* q = reinterpret_cast<const float4*>(pr.samples + pf);
			const float4 q0 = q[0], q1 = q[1], q2 = q[2], q3 = q[3];
			const uint32_t flags = __float_as_uint(q3.y);
			f3 final_color = splat(0.0f);
			if (!(flags & kSampleNoLight)) {
				const f3 c[2][2] = {{mk3(q0.x, q0.y, q0.z), mk3(q0.w, q1.x, q1.y)},
				                    {mk3(q1.z, q1.w, q2.x), mk3(q2.y, q2.z, q2.w)}};
				f3 result = splat(0.0f);
#pragma unroll
				for (int j = 0; j != 2; ++j) {
					const uint32_t mode = (flags >> (2 * j)) & 3u;
					if (mode == kSampleSkip) continue;
					const bool occluded = mode == kSampleTraced && pr.hits[2 * pf + j] != 0;
					result = add(result, occluded ? c[j][1] : c[j][0]);
				}
				const f3 color = scale(result, P::rcp(1.0f));
				const f3 cw = scale(color, q3.x);
				final_color = add(final_color, mk3(P::div(cw.x, 1.0f), P::div(cw.y, 1.0f), P::div(cw.z, 1.0f)));
			}
			const bool finite = !(isnan(final_color.x) || isnan(final_color.y) || isnan(final_color.z) ||
			                      isinf(final_color.x) || isinf(final_color.y) || isinf(final_color.z));
			if (f == 0 && pr.train_shaded && pr.train_stride && i % pr.train_stride == pr.train_phase)
				pr.train_shaded[i] =
				    finite ? 0.2126f * final_color.x + 0.7152f * final_color.y + 0.0722f * final_color.z : 0.0f;
			if (!finite) final_color = mk3(1.0f, 0.0f, 0.8f);
			if (f == 0 && res) {
				const ReservoirRecord r = pr.records[pf];
				*res = risltc_reservoir_t{r.light_index, r.w_sum, r.p_hat, 0u};
			}
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

template <class P> __global__ void __launch_bounds__(128) ris_resolve_kernel(const __grid_constant__ RisParams pr) {
	const uint32_t np = pr.width * pr.height;
	for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < np; i += gridDim.x * blockDim.x)
		resolve_pixel<P>(pr, i);
}

}  // namespace risltc
