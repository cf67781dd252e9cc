/* Host model of polygonal lights and of the per-frame noise constants.
 * Restates upstream risltc code (GPLv3): see NOTICE.
 *
 * Restates src/polygonal_light.c, write_lights (src/main.c:456-490),
 * set_noise_constants (src/noise_table.c:24-28) and wang_random_number
 * (src/math_utilities.h:50-57).  The arithmetic is written in the same order
 * as the reference (and compiled without contraction), so the world-space
 * vertices, planes and areas are bit-identical to the reference's.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include "../../../include/risltc.h"

int set_polygonal_light_vertex_count(polygonal_light_t* light, uint32_t vertex_count) {
	if (light->vertex_count == vertex_count && light->vertices_plane_space && light->vertices_world_space) return 0;
	size_t bytes = sizeof(float) * 4 * vertex_count;
	float* plane_space = (float*) calloc(1, bytes ? bytes : 1);
	float* world_space = (float*) calloc(1, bytes ? bytes : 1);
	if (light->vertices_plane_space) {
		uint32_t keep = vertex_count < light->vertex_count ? vertex_count : light->vertex_count;
		memcpy(plane_space, light->vertices_plane_space, sizeof(float) * 4 * keep);
	}
	free(light->vertices_plane_space);
	free(light->vertices_world_space);
	light->vertices_plane_space = plane_space;
	light->vertices_world_space = world_space;
	light->vertex_count = vertex_count;
	/* The reference compares after assigning, so it always reports 0. */
	return 0;
}

void update_polygonal_light(polygonal_light_t* light) {
	light->inv_scaling_x = 1.0f / light->scaling_x;
	light->inv_scaling_y = 1.0f / light->scaling_y;
	/* Rotation about z, then y, then x. */
	const float cos_x = cosf(light->rotation_angles[0]), sin_x = sinf(light->rotation_angles[0]);
	const float cos_y = cosf(light->rotation_angles[1]), sin_y = sinf(light->rotation_angles[1]);
	const float cos_z = cosf(light->rotation_angles[2]), sin_z = sinf(light->rotation_angles[2]);
	const float cos_x_sin_y = cos_x * sin_y;
	const float sin_x_sin_y = sin_x * sin_y;
	float r[3][4];
	r[0][0] = cos_y * cos_z;
	r[0][1] = -cos_y * sin_z;
	r[0][2] = -sin_y;
	r[1][0] = -sin_x_sin_y * cos_z + cos_x * sin_z;
	r[1][1] = sin_x_sin_y * sin_z + cos_x * cos_z;
	r[1][2] = -sin_x * cos_y;
	r[2][0] = cos_x_sin_y * cos_z + sin_x * sin_z;
	r[2][1] = -cos_x_sin_y * sin_z + sin_x * cos_z;
	r[2][2] = cos_x * cos_y;
	r[0][3] = r[1][3] = r[2][3] = 0.0f;
	memcpy(light->rotation, r, sizeof(r));
	const float scale[2] = {light->scaling_x, light->scaling_y};
	for (uint32_t v = 0; v != light->vertex_count; ++v) {
		for (uint32_t row = 0; row != 3; ++row) {
			float acc = light->translation[row];
			for (uint32_t col = 0; col != 2; ++col)
				acc += scale[col] * r[row][col] * light->vertices_plane_space[v * 4 + col];
			light->vertices_world_space[v * 4 + row] = acc;
		}
	}
	/* The plane normal is the rotated z axis. */
	for (uint32_t row = 0; row != 3; ++row) light->plane[row] = r[row][2];
	light->plane[3] = -(r[0][2] * light->translation[0] + r[1][2] * light->translation[1] + r[2][2] * light->translation[2]);
	/* Signed area of the triangle fan around vertex 0, in plane space. */
	float signed_area = 0.0f;
	const float* p = light->vertices_plane_space;
	for (uint32_t i = 0; i + 2 < light->vertex_count; ++i) {
		float a00 = p[(i + 2) * 4 + 0] - p[0], a01 = p[(i + 1) * 4 + 0] - p[0];
		float a10 = p[(i + 2) * 4 + 1] - p[1], a11 = p[(i + 1) * 4 + 1] - p[1];
		signed_area += 0.5f * (a00 * a11 - a01 * a10);
	}
	signed_area *= scale[0] * scale[1];
	float abs_area = (signed_area < 0.0f) ? -signed_area : signed_area;
	light->area = abs_area;
	light->rcp_area = 1.0f / abs_area;
	for (uint32_t c = 0; c != 3; ++c) light->surface_radiance[c] = light->radiant_flux[c];
	/* Wrong winding: flip the plane. */
	for (uint32_t c = 0; c != 4; ++c) light->plane[c] = (signed_area > 0.0f) ? light->plane[c] : -light->plane[c];
}

polygonal_light_t duplicate_polygonal_light(const polygonal_light_t* light) {
	polygonal_light_t copy = *light;
	copy.texture_file_path = NULL;
	if (light->texture_file_path) {
		size_t len = strlen(light->texture_file_path) + 1;
		copy.texture_file_path = (char*) malloc(len);
		memcpy(copy.texture_file_path, light->texture_file_path, len);
	}
	copy.vertex_count = 0;
	copy.vertices_plane_space = NULL;
	copy.vertices_world_space = NULL;
	set_polygonal_light_vertex_count(&copy, light->vertex_count);
	memcpy(copy.vertices_plane_space, light->vertices_plane_space, sizeof(float) * 4 * light->vertex_count);
	return copy;
}

void destroy_polygonal_light(polygonal_light_t* light) {
	free(light->vertices_plane_space);
	free(light->vertices_world_space);
	free(light->texture_file_path);
	memset(light, 0, sizeof(*light));
}

uint32_t risltc_wang_random_number(uint32_t seed) {
	seed = (seed ^ 61u) ^ (seed >> 16);
	seed *= 9u;
	seed = seed ^ (seed >> 4);
	seed *= 0x27d4eb2du;
	seed = seed ^ (seed >> 15);
	return seed;
}

void set_noise_constants(uint32_t resolution_mask[2], uint32_t* texture_index_mask, uint32_t random_numbers[4],
                         noise_table_t* noise, uint32_t animate_noise) {
	(void) resolution_mask;
	(void) texture_index_mask;
	for (uint32_t i = 0; i != 4; ++i)
		random_numbers[i] = animate_noise ? risltc_wang_random_number(noise->random_seed * 4u + i) : i * 0x123456u;
	++noise->random_seed;
}

uint32_t risltc_max_light_vertex_count(const polygonal_light_t* lights, uint32_t count) {
	uint32_t m = 3;
	for (uint32_t i = 0; lights && i != count; ++i)
		if (lights[i].vertex_count > m) m = lights[i].vertex_count;
	return m;
}

int risltc_write_lights(float* data, polygonal_light_t* lights, uint32_t count, uint32_t max_vertex_count) {
	if (!data || (!lights && count) || max_vertex_count < 3 || max_vertex_count > RISLTC_MAX_LIGHT_VERTEX_COUNT)
		return RISLTC_ERROR_INVALID_ARGUMENT;
	const size_t stride = 12 + 4 * (size_t) max_vertex_count;
	for (uint32_t i = 0; i != count; ++i) {
		polygonal_light_t* l = &lights[i];
		if (l->vertex_count < 3 || l->vertex_count > max_vertex_count || !l->vertices_world_space)
			return RISLTC_ERROR_VERTEX_COUNT;
		update_polygonal_light(l);
		float* d = data + i * stride;
		polygonal_light_upload_t up;
		memset(&up, 0, sizeof(up));
		for (int c = 0; c != 3; ++c) up.surface_radiance[c] = l->surface_radiance[c];
		for (int c = 0; c != 4; ++c) up.plane[c] = l->plane[c];
		up.vertex_count = l->vertex_count;
		memcpy(d, &up, POLYGONAL_LIGHT_FIXED_CONSTANT_BUFFER_SIZE);
		for (uint32_t v = 0; v != max_vertex_count; ++v) {
			const float* src = l->vertices_world_space + 4 * (v < l->vertex_count ? v : 0);
			d[12 + 4 * v + 0] = src[0];
			d[12 + 4 * v + 1] = src[1];
			d[12 + 4 * v + 2] = src[2];
			d[12 + 4 * v + 3] = 0.0f;
		}
	}
	return RISLTC_OK;
}

void risltc_default_settings(risltc_settings_t* s) {
	if (!s) return;
	memset(s, 0, sizeof(*s));
	s->polygon_sampling_technique = sample_polygon_ltc_cp;
	s->light_sampling = light_reservoir;
	s->mis_heuristic = mis_heuristic_optimal_clamped;
	s->candidate_count = 32;
	s->sample_count = 1;
	s->sample_count_light = 1;
	s->mis_visibility_estimate = 0.5f;
	s->fast_atan = 0;
	s->shadows = 1;
	s->numerics = risltc_numerics_exact;
	s->proposal = risltc_proposal_uniform;
	s->proposal_uniform_fraction = 0.1f;
	s->tile = risltc_tile_32x8;
}
