// ref_harness.hpp - drives the reference's lowered shading pass per pixel.
//
// Test infrastructure: appended to the lowered GLSL by oracle/ref/build_ref.py
// and compiled into oracle/_ref/*.so; only tests/golden/make_golden.py loads it.
//
// It plays the role of the reference's Vulkan frame: it fills the uniforms of
// shared_constants.glsl, the light buffer (the std140 layout written by
// write_lights, main.c:456-490), the LTC texture arrays and the noise
// constants, then runs shading_pass_main() once per pixel with gl_FragCoord at
// the pixel centre and reads back g_out_color.  Shadow ray queries
// (get_polygon_visibility, shading_pass.frag.glsl:112-129) become a
// brute-force any-hit loop over the occluder triangles with the project's
// ray/triangle test (Moller-Trumbore on precomputed v0, e1 = v1 - v0,
// e2 = v2 - v0).

struct RefInputs {
	int width, height;
	// G-buffer, 17 planes of width*height floats: position xyz, normal xyz,
	// outgoing xyz, lambert_outgoing, diffuse_albedo rgb, fresnel_0 rgb,
	// roughness.
	const float* gbuffer;
	// Optional per-pixel primitive id; 0xFFFFFFFF marks background.
	const uint32_t* primitive;
	// Light buffer, std140: 12 + 4*MAX_POLYGONAL_LIGHT_VERTEX_COUNT floats per
	// light (radiance, pad, plane, vertex_count, pad x3, vertices with w pad).
	const float* lights;
	int light_count;
	// LTC texture arrays: tex0 has 4 channels, tex1 has 2 channels.
	const float* ltc0;
	const float* ltc1;
	int ltc_width, ltc_height, ltc_layers;
	float ltc_constants[6];
	uint32_t noise_random_numbers[4];
	float mis_visibility_estimate;
	// Occluders: 9 floats per triangle (v0, e1, e2).
	const float* triangles;
	int triangle_count;
};

static const RefInputs* g_ref_in = nullptr;
static int g_ref_pixel_index = 0;
int g_ref_light_count = 0;

shading_data_t get_shading_data(ivec2 pixel, int, vec3) {
	const float* g = g_ref_in->gbuffer;
	size_t n = (size_t) g_ref_in->width * g_ref_in->height;
	size_t i = (size_t) pixel.y * g_ref_in->width + pixel.x;
	shading_data_t s;
	s.position = vec3(g[0 * n + i], g[1 * n + i], g[2 * n + i]);
	s.normal = vec3(g[3 * n + i], g[4 * n + i], g[5 * n + i]);
	s.outgoing = vec3(g[6 * n + i], g[7 * n + i], g[8 * n + i]);
	s.lambert_outgoing = g[9 * n + i];
	s.diffuse_albedo = vec3(g[10 * n + i], g[11 * n + i], g[12 * n + i]);
	s.fresnel_0 = vec3(g[13 * n + i], g[14 * n + i], g[15 * n + i]);
	s.roughness = g[16 * n + i];
	return s;
}

uvec4 subpassLoad(const usubpassInput&) {
	uint prim = g_ref_in->primitive ? g_ref_in->primitive[g_ref_pixel_index] : 0u;
	return uvec4(prim);
}

bool glsl_shim_any_hit(const vec3& o, const vec3& d, float t_min, float t_max) {
	for (int k = 0; k != g_ref_in->triangle_count; ++k) {
		const float* t = g_ref_in->triangles + 9 * (size_t) k;
		vec3 v0(t[0], t[1], t[2]), e1(t[3], t[4], t[5]), e2(t[6], t[7], t[8]);
		vec3 p = cross(d, e2);
		float det = dot(e1, p);
		if (!(det != 0.0f)) continue;
		float inv = 1.0f / det;
		vec3 s = o - v0;
		float u = dot(s, p) * inv;
		if (!(u >= 0.0f && u <= 1.0f)) continue;
		vec3 q = cross(s, e1);
		float v = dot(d, q) * inv;
		if (!(v >= 0.0f && u + v <= 1.0f)) continue;
		float tt = dot(e2, q) * inv;
		if (tt >= t_min && tt <= t_max) return true;
	}
	return false;
}

extern "C" int ref_max_light_vertex_count() { return MAX_POLYGONAL_LIGHT_VERTEX_COUNT; }
extern "C" int ref_candidate_count() { return RISLTC_REF_M; }

// Renders one frame.  out_rgb: 3*width*height floats (pixel-major rgb).
// out_reads: per pixel, the number of light-buffer reads and the last index
// read (2 ints per pixel); with LIGHT_SAMPLES == 1 and RIS, the reservoir's
// light is the last read iff the count is RISLTC_REF_M + 1.
extern "C" int ref_render(const RefInputs* in, float* out_rgb, int32_t* out_reads) {
	static thread_local polygonal_light_t* lights = nullptr;
	g_ref_in = in;
	std::vector<polygonal_light_t> storage((size_t) (in->light_count > 0 ? in->light_count : 1));
	const int stride = 12 + 4 * MAX_POLYGONAL_LIGHT_VERTEX_COUNT;
	for (int l = 0; l != in->light_count; ++l) {
		const float* f = in->lights + (size_t) l * stride;
		polygonal_light_t& pl = storage[l];
		pl.surface_radiance = vec3(f[0], f[1], f[2]);
		pl.plane = vec4(f[4], f[5], f[6], f[7]);
		uint32_t vc;
		std::memcpy(&vc, f + 8, 4);
		pl.vertex_count = vc;
		for (int j = 0; j != MAX_POLYGONAL_LIGHT_VERTEX_COUNT; ++j)
			pl.vertices_world_space[j] = vec3(f[12 + 4 * j], f[13 + 4 * j], f[14 + 4 * j]);
	}
	lights = storage.data();
	g_polygonal_lights.lights = lights;
	g_polygonal_lights.count = in->light_count;
	g_ref_light_count = in->light_count;
	g_ltc_tables[0] = sampler2DArray{in->ltc0, in->ltc_width, in->ltc_height, in->ltc_layers, 4};
	g_ltc_tables[1] = sampler2DArray{in->ltc1, in->ltc_width, in->ltc_height, in->ltc_layers, 2};
	g_ltc_constants.fresnel_index_factor = in->ltc_constants[0];
	g_ltc_constants.fresnel_index_summand = in->ltc_constants[1];
	g_ltc_constants.roughness_factor = in->ltc_constants[2];
	g_ltc_constants.roughness_summand = in->ltc_constants[3];
	g_ltc_constants.inclination_factor = in->ltc_constants[4];
	g_ltc_constants.inclination_summand = in->ltc_constants[5];
	g_noise_random_numbers = uvec4(in->noise_random_numbers[0], in->noise_random_numbers[1],
	                               in->noise_random_numbers[2], in->noise_random_numbers[3]);
	g_viewport_size = uvec2((uint) in->width, (uint) in->height);
	g_mis_visibility_estimate = in->mis_visibility_estimate;
	g_exposure_factor = 1.0f;
	g_roughness_factor = 1.0f;
	g_error_factor = 1.0f;
	g_pixel_to_ray_direction_world_space = mat3(vec3(0.0f), vec3(0.0f), vec3(0.0f, 0.0f, 1.0f));
	for (int y = 0; y != in->height; ++y) {
		for (int x = 0; x != in->width; ++x) {
			int i = y * in->width + x;
			g_ref_pixel_index = i;
			g_polygonal_lights.log_size = 0;
			gl_FragCoord = vec4((float) x + 0.5f, (float) y + 0.5f, 0.0f, 1.0f);
			g_out_color = vec4(0.0f);
			shading_pass_main();
			out_rgb[3 * (size_t) i + 0] = g_out_color.x;
			out_rgb[3 * (size_t) i + 1] = g_out_color.y;
			out_rgb[3 * (size_t) i + 2] = g_out_color.z;
			if (out_reads) {
				int ls = g_polygonal_lights.log_size;
				out_reads[2 * (size_t) i + 0] = ls;
				out_reads[2 * (size_t) i + 1] = ls > 0 ? g_polygonal_lights.log[ls - 1] : -1;
			}
		}
	}
	g_ref_in = nullptr;
	return 0;
}
