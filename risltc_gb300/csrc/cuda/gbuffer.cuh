// gbuffer.cuh - a G-buffer producer: primary rays against a sum-of-sines
// heightfield, then the shading data of the hit (the role of the reference's
// visibility pass and get_shading_data, shading_pass.frag.glsl:571-672, for
// the synthetic heightfield scenes; the reference rasterises meshes).
//
// Per pixel: a pinhole camera ray (looking at the origin, z up); the first
// sign change of z - h(x, y) along the ray within the heightfield's height
// band by 10 uniform steps, refined by 12 bisections; the geometric normal
// from the heightfield's gradient, adapted into the outgoing direction's
// hemisphere as get_shading_data does (:666-670); material from a per-pixel
// hash.  Pixels whose ray misses get primitive 0xFFFFFFFF.
#pragma once
#include "shade_device.cuh"

namespace risltc {

constexpr int kMaxWaves = 16;

struct HeightfieldParams {
	float camera[3];
	float forward[3], right[3], up[3];
	float tan_half_x, tan_half_y;
	int wave_count;
	float waves[kMaxWaves][4];  // amplitude, frequency x, frequency y, phase
	float max_height;           // sum of the amplitudes
	uint32_t material_seed;
	float roughness_min, roughness_max, albedo_min, albedo_max, fresnel_0;
	uint32_t width, height;
	float* planes;              // 17 planes of width * height floats
	uint32_t* primitive;
};

RL_DEV float hf_height(const HeightfieldParams& p, float x, float y) {
	float h = 0.0f;
	for (int w = 0; w != p.wave_count; ++w) h += p.waves[w][0] * sinf(p.waves[w][1] * x + p.waves[w][2] * y + p.waves[w][3]);
	return h;
}

// A uniform number in [0, 1) from a pixel, a seed and a stream index
// (murmur3 finaliser of a mixed key).
RL_DEV float hf_uniform(uint32_t pixel, uint32_t seed, uint32_t stream) {
	uint32_t h = pixel * 0x9E3779B1u ^ (seed + stream * 0x85EBCA77u);
	h ^= h >> 16;
	h *= 0x85ebca6bu;
	h ^= h >> 13;
	h *= 0xc2b2ae35u;
	h ^= h >> 16;
	return (float) (h >> 8) * (1.0f / 16777216.0f);
}

static __global__ void __launch_bounds__(128) heightfield_gbuffer_kernel(HeightfieldParams p) {
	const uint32_t np = p.width * p.height;
	for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < np; i += gridDim.x * blockDim.x) {
		const uint32_t x = i % p.width, y = i / p.width;
		const float u = (((float) x + 0.5f) / (float) p.width * 2.0f - 1.0f) * p.tan_half_x;
		const float v = (1.0f - ((float) y + 0.5f) / (float) p.height * 2.0f) * p.tan_half_y;
		f3 d = mk3(p.forward[0] + u * p.right[0] + v * p.up[0], p.forward[1] + u * p.right[1] + v * p.up[1],
		           p.forward[2] + u * p.right[2] + v * p.up[2]);
		d = scale(d, rsqrtf(dot(d, d)));
		const f3 cam = mk3(p.camera[0], p.camera[1], p.camera[2]);
		const bool valid = d.z < -1e-3f;
		const float dz = valid ? d.z : -1.0f;
		const float t_lo = (cam.z - p.max_height) / -dz, t_hi = (cam.z + p.max_height) / -dz;
		auto g = [&](float t) { return (cam.z + t * d.z) - hf_height(p, cam.x + t * d.x, cam.y + t * d.y); };
		float a = t_lo, b = t_hi, prev = t_lo;
		bool found = false;
		for (int k = 1; k <= 10 && !found; ++k) {
			const float t = t_lo + (t_hi - t_lo) * (float) k / 10.0f;
			if (g(t) <= 0.0f) {
				a = prev;
				b = t;
				found = true;
			}
			prev = t;
		}
		for (int k = 0; k != 12; ++k) {
			const float m = 0.5f * (a + b);
			if (g(m) <= 0.0f)
				b = m;
			else
				a = m;
		}
		const float t = 0.5f * (a + b);
		const f3 pos = add(cam, scale(d, t));
		float gx = 0.0f, gy = 0.0f;
		for (int w = 0; w != p.wave_count; ++w) {
			const float c = p.waves[w][0] * cosf(p.waves[w][1] * pos.x + p.waves[w][2] * pos.y + p.waves[w][3]);
			gx += c * p.waves[w][1];
			gy += c * p.waves[w][2];
		}
		f3 n = mk3(-gx, -gy, 1.0f);
		n = scale(n, rsqrtf(dot(n, n)));
		f3 wo = sub(cam, pos);
		wo = scale(wo, rsqrtf(dot(wo, wo)));
		const float off = fmaxf(0.0f, 1.0e-3f - dot(n, wo));
		n = add(n, scale(wo, off));
		n = scale(n, rsqrtf(dot(n, n)));
		const float rough = p.roughness_min + (p.roughness_max - p.roughness_min) * hf_uniform(i, p.material_seed, 0);
		float alb[3];
		for (int c = 0; c != 3; ++c)
			alb[c] = p.albedo_min + (p.albedo_max - p.albedo_min) * hf_uniform(i, p.material_seed, 1 + c);
		const size_t s = np;
		float* q = p.planes;
		q[0 * s + i] = pos.x;
		q[1 * s + i] = pos.y;
		q[2 * s + i] = pos.z;
		q[3 * s + i] = n.x;
		q[4 * s + i] = n.y;
		q[5 * s + i] = n.z;
		q[6 * s + i] = wo.x;
		q[7 * s + i] = wo.y;
		q[8 * s + i] = wo.z;
		q[9 * s + i] = dot(n, wo);
		for (int c = 0; c != 3; ++c) q[(10 + c) * s + i] = alb[c];
		for (int c = 0; c != 3; ++c) q[(13 + c) * s + i] = p.fresnel_0;
		q[16 * s + i] = rough;
		if (p.primitive) p.primitive[i] = (valid && found) ? 0u : 0xFFFFFFFFu;
	}
}

}  // namespace risltc
