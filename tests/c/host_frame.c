/* host_frame.c - a C99 host program that shades one frame through the C ABI,
 * written against include/risltc.h alone, the way the reference's host code
 * drives its shading pass (src/main.c:456-490 packs the lights, 2955-3041
 * renders a frame): polygonal_light_t records filled through
 * set_polygonal_light_vertex_count / update_polygonal_light, the std140 light
 * buffer from risltc_write_lights, an LTC table, the frame's noise constants
 * from set_noise_constants, then a context, a scene with occluders and
 * risltc_shade_host.
 *
 *   host_frame <output directory> <width> <height> <lights> <occluders>
 *
 * The scene is a plane of polygonal lights (3 to 8 vertices, facing down)
 * over a G-buffer on z = 0 seen from (0, -6, 4), with random occluder
 * triangles between them.  Writes the inputs it built (lights.f32 in the
 * std140 layout, gbuffer.f32 as 17 planes, triangles.f32, ltc0.f32,
 * ltc1.f32, ltc_constants.f32), the shaded image (image.f32, RGB per pixel)
 * and meta.txt ("max_vertex_count light_count triangle_count
 * random_number_x"), so that a test can shade the same frame with the
 * oracle.  Exits with the first failing call's risltc status (0 when the
 * frame was shaded). */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "risltc.h"

/* splitmix64 for the scene's random numbers. */
static uint64_t g_state = 0x243F6A8885A308D3ull;
static double uniform(double lo, double hi) {
	uint64_t z = (g_state += 0x9E3779B97F4A7C15ull);
	z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
	z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
	z ^= z >> 31;
	return lo + (hi - lo) * (double) (z >> 11) * (1.0 / 9007199254740992.0);
}

static int write_file(const char* dir, const char* name, const void* data, size_t bytes) {
	char path[4096];
	FILE* f;
	size_t written;
	snprintf(path, sizeof(path), "%s/%s", dir, name);
	f = fopen(path, "wb");
	if (!f) return RISLTC_ERROR_IO;
	written = fwrite(data, 1, bytes, f);
	return (fclose(f) == 0 && written == bytes) ? RISLTC_OK : RISLTC_ERROR_IO;
}

int main(int argc, char** argv) {
	const char* dir;
	uint32_t width, height, light_count, triangle_count, max_vertex_count, i, k;
	size_t pixels, stride;
	polygonal_light_t* lights;
	float *light_buffer, *planes, *triangles, *image, constants[6];
	risltc_ltc_table_t table;
	noise_table_t noise;
	uint32_t random_numbers[4];
	risltc_settings_t settings;
	risltc_ctx_t* ctx = NULL;
	risltc_scene_t* scene = NULL;
	int status;
	FILE* meta;
	char path[4096];

	if (argc != 6) {
		fprintf(stderr, "usage: %s <output directory> <width> <height> <lights> <occluders>\n", argv[0]);
		return RISLTC_ERROR_INVALID_ARGUMENT;
	}
	dir = argv[1];
	width = (uint32_t) strtoul(argv[2], NULL, 10);
	height = (uint32_t) strtoul(argv[3], NULL, 10);
	light_count = (uint32_t) strtoul(argv[4], NULL, 10);
	triangle_count = (uint32_t) strtoul(argv[5], NULL, 10);
	if (width == 0 || height == 0 || light_count == 0) return RISLTC_ERROR_INVALID_ARGUMENT;
	pixels = (size_t) width * height;

	/* Lights: regular polygons in their plane, rotated to face down (z
	   rotation first, then x by pi, as the Euler angles of
	   update_polygonal_light, polygonal_light.c:49-62). */
	lights = (polygonal_light_t*) calloc(light_count, sizeof(polygonal_light_t));
	if (!lights) return RISLTC_ERROR_OUT_OF_MEMORY;
	for (i = 0; i != light_count; ++i) {
		polygonal_light_t* l = &lights[i];
		const uint32_t n = 3 + (uint32_t) uniform(0.0, 6.0);
		const double radius = uniform(0.15, 0.6);
		set_polygonal_light_vertex_count(l, n);
		l->rotation_angles[0] = (float) (3.14159265358979 + uniform(-0.5, 0.5));
		l->rotation_angles[1] = (float) uniform(-0.5, 0.5);
		l->rotation_angles[2] = (float) uniform(0.0, 6.28318530717959);
		l->scaling_x = 1.0f;
		l->scaling_y = 1.0f;
		l->translation[0] = (float) uniform(-5.0, 5.0);
		l->translation[1] = (float) uniform(-5.0, 5.0);
		l->translation[2] = (float) uniform(1.0, 3.0);
		for (k = 0; k != 3; ++k) l->radiant_flux[k] = (float) exp(uniform(log(0.1), log(10.0)));
		for (k = 0; k != n; ++k) {
			const double a = 6.28318530717959 * (double) k / (double) n;
			l->vertices_plane_space[4 * k + 0] = (float) (radius * cos(a));
			l->vertices_plane_space[4 * k + 1] = (float) (radius * sin(a));
		}
		update_polygonal_light(l);
	}
	max_vertex_count = risltc_max_light_vertex_count(lights, light_count);
	stride = 12 + 4 * (size_t) max_vertex_count;
	light_buffer = (float*) calloc(stride * light_count, sizeof(float));
	planes = (float*) calloc(RISLTC_GBUFFER_PLANES * pixels, sizeof(float));
	triangles = (float*) calloc(9 * (size_t) (triangle_count ? triangle_count : 1), sizeof(float));
	image = (float*) calloc(3 * pixels, sizeof(float));
	if (!light_buffer || !planes || !triangles || !image) return RISLTC_ERROR_OUT_OF_MEMORY;
	status = risltc_write_lights(light_buffer, lights, light_count, max_vertex_count);
	if (status) return status;

	/* G-buffer: the plane z = 0 over [-5, 5]^2, normal +z, seen from
	   (0, -6, 4); GGX roughness U[0.1, 0.9], albedo U[0.2, 0.8], F0 = 0.02. */
	for (i = 0; i != height; ++i) {
		for (k = 0; k != width; ++k) {
			const size_t p = (size_t) i * width + k;
			const float x = -5.0f + 10.0f * ((float) k + 0.5f) / (float) width;
			const float y = 5.0f - 10.0f * ((float) i + 0.5f) / (float) height;
			float wo[3];
			float len;
			int c;
			wo[0] = 0.0f - x;
			wo[1] = -6.0f - y;
			wo[2] = 4.0f;
			len = sqrtf(wo[0] * wo[0] + wo[1] * wo[1] + wo[2] * wo[2]);
			planes[0 * pixels + p] = x;
			planes[1 * pixels + p] = y;
			planes[2 * pixels + p] = 0.0f;
			planes[3 * pixels + p] = 0.0f;
			planes[4 * pixels + p] = 0.0f;
			planes[5 * pixels + p] = 1.0f;
			for (c = 0; c != 3; ++c) planes[(6 + c) * pixels + p] = wo[c] / len;
			planes[9 * pixels + p] = wo[2] / len;
			for (c = 0; c != 3; ++c) planes[(10 + c) * pixels + p] = (float) uniform(0.2, 0.8);
			for (c = 0; c != 3; ++c) planes[(13 + c) * pixels + p] = 0.02f;
			planes[16 * pixels + p] = (float) uniform(0.1, 0.9);
		}
	}
	/* Occluders: triangles with edges of 0.05..0.5 in [-5, 5]^2 x [0.2, 0.9]. */
	for (i = 0; i != triangle_count; ++i) {
		float* t = triangles + 9 * (size_t) i;
		for (k = 0; k != 3; ++k) t[k] = (float) (k == 2 ? uniform(0.2, 0.9) : uniform(-5.0, 5.0));
		for (k = 3; k != 9; ++k) t[k] = t[k % 3] + (float) uniform(-0.3, 0.3);
	}

	status = risltc_ltc_table_synthetic(&table, 0, 64, 64);
	if (status) return status;
	/* The noise constants of the frame this program shades (frame 0). */
	noise.random_seed = 0;
	set_noise_constants(NULL, NULL, random_numbers, &noise, 1);
	noise.random_seed = 0;

	constants[0] = table.constants.fresnel_index_factor;
	constants[1] = table.constants.fresnel_index_summand;
	constants[2] = table.constants.roughness_factor;
	constants[3] = table.constants.roughness_summand;
	constants[4] = table.constants.inclination_factor;
	constants[5] = table.constants.inclination_summand;
	status = write_file(dir, "lights.f32", light_buffer, stride * light_count * sizeof(float));
	if (!status) status = write_file(dir, "gbuffer.f32", planes, RISLTC_GBUFFER_PLANES * pixels * sizeof(float));
	if (!status) status = write_file(dir, "triangles.f32", triangles, 9 * (size_t) triangle_count * sizeof(float));
	if (!status) {
		const size_t texels = (size_t) table.roughness_count * table.inclination_count * table.fresnel_count;
		status = write_file(dir, "ltc0.f32", table.texels0, 4 * texels * sizeof(float));
		if (!status) status = write_file(dir, "ltc1.f32", table.texels1, 2 * texels * sizeof(float));
		if (!status) status = write_file(dir, "ltc_constants.f32", constants, sizeof(constants));
	}
	snprintf(path, sizeof(path), "%s/meta.txt", dir);
	meta = fopen(path, "w");
	if (!meta) return RISLTC_ERROR_IO;
	fprintf(meta, "%u %u %u %u %u %u\n", max_vertex_count, light_count, triangle_count, random_numbers[0], width,
	        height);
	fclose(meta);
	if (status) return status;

	/* The device part: context, scene, one frame of the default settings. */
	status = risltc_ctx_create(&ctx, 0, NULL);
	if (!status)
		status = risltc_scene_create(ctx, light_buffer, light_count, max_vertex_count, &table,
		                             triangle_count ? triangles : NULL, triangle_count, &scene);
	if (!status) {
		risltc_default_settings(&settings);
		status = risltc_shade_host(ctx, scene, width, height, planes, NULL, &settings, &noise, 1, 1, image);
	}
	if (!status) status = write_file(dir, "image.f32", image, 3 * pixels * sizeof(float));
	if (status) fprintf(stderr, "host_frame: %s\n", risltc_status_string(status));

	risltc_scene_destroy(scene);
	risltc_ctx_destroy(ctx);
	risltc_ltc_table_destroy(&table);
	risltc_destroy_lights(lights, light_count);
	free(light_buffer);
	free(planes);
	free(triangles);
	free(image);
	return status;
}
