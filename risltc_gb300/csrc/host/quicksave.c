/* Quicksave files of the reference renderer: the camera and the polygonal
 * lights of a scene, as written by quick_save and read by quick_load
 * (src/main.c:45-125) and by the Blender exporter
 * (tools/io_export_lights_blender.py:11-112).
 *
 * Layout (little-endian, 64-bit host):
 *   first_person_camera_t (48 bytes, src/camera.h:29-49)
 *   uint32 legacy_count (0), uint32 light_count
 *   per light:
 *     the first POLYGONAL_LIGHT_QUICKSAVE_SIZE = 88 bytes of
 *       polygonal_light_t (rotation_angles .. texturing_technique),
 *     uint64 path_size, then path_size bytes of texture path (with its NUL),
 *     two 8-byte pointers written as zero,
 *     4 * vertex_count floats of vertices_plane_space.
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include "../../../include/risltc.h"

#define QUICKSAVE_LIGHT_BYTES (sizeof(float) * 20 + sizeof(uint32_t) * 2)
/* Sanity limits on sizes read from a file. */
#define QUICKSAVE_MAX_VERTICES 65536u
#define QUICKSAVE_MAX_PATH (1u << 20)

void risltc_destroy_lights(polygonal_light_t* lights, uint32_t light_count) {
	if (!lights) return;
	for (uint32_t i = 0; i != light_count; ++i) destroy_polygonal_light(&lights[i]);
	free(lights);
}

int risltc_quick_load(const char* path, risltc_camera_t* camera, polygonal_light_t** lights_out,
                      uint32_t* light_count_out) {
	if (!path || !lights_out || !light_count_out) return RISLTC_ERROR_INVALID_ARGUMENT;
	*lights_out = NULL;
	*light_count_out = 0;
	FILE* f = fopen(path, "rb");
	if (!f) return RISLTC_ERROR_IO;
	risltc_camera_t cam;
	uint32_t legacy_count = 0, count = 0;
	int status = RISLTC_OK;
	if (fread(&cam, sizeof(cam), 1, f) != 1 || fread(&legacy_count, sizeof(uint32_t), 1, f) != 1 ||
	    fread(&count, sizeof(uint32_t), 1, f) != 1) {
		fclose(f);
		return RISLTC_ERROR_IO;
	}
	polygonal_light_t* lights = (polygonal_light_t*) calloc(count ? count : 1, sizeof(polygonal_light_t));
	if (!lights) {
		fclose(f);
		return RISLTC_ERROR_OUT_OF_MEMORY;
	}
	uint32_t loaded = 0;
	for (; loaded != count; ++loaded) {
		polygonal_light_t* light = &lights[loaded];
		uint64_t path_size = 0, pointers[2];
		if (fread(light, QUICKSAVE_LIGHT_BYTES, 1, f) != 1 || fread(&path_size, sizeof(path_size), 1, f) != 1) {
			status = RISLTC_ERROR_IO;
			break;
		}
		/* The fixed part carries vertex_count; the pointers are re-created. */
		const uint32_t vertex_count = light->vertex_count;
		light->texture_file_path = NULL;
		light->vertices_plane_space = NULL;
		light->vertices_world_space = NULL;
		light->vertex_count = 0;
		/* Quick fix for legacy files, as in quick_load. */
		if (light->scaling_y <= 0.0f) light->scaling_y = light->scaling_x;
		if (vertex_count > QUICKSAVE_MAX_VERTICES || path_size > QUICKSAVE_MAX_PATH) {
			status = RISLTC_ERROR_IO;
			break;
		}
		if (path_size) {
			light->texture_file_path = (char*) malloc(path_size);
			if (!light->texture_file_path || fread(light->texture_file_path, 1, path_size, f) != path_size) {
				status = RISLTC_ERROR_IO;
				++loaded;
				break;
			}
			light->texture_file_path[path_size - 1] = '\0';
		}
		if (fread(pointers, sizeof(pointers), 1, f) != 1) {
			status = RISLTC_ERROR_IO;
			++loaded;
			break;
		}
		set_polygonal_light_vertex_count(light, vertex_count);
		if (vertex_count &&
		    fread(light->vertices_plane_space, sizeof(float), 4 * (size_t) vertex_count, f) != 4 * (size_t) vertex_count) {
			status = RISLTC_ERROR_IO;
			++loaded;
			break;
		}
		/* Derived members (rotation, world-space vertices, plane, area), as
		   the renderer computes them before use. */
		update_polygonal_light(light);
	}
	fclose(f);
	if (status != RISLTC_OK) {
		risltc_destroy_lights(lights, loaded);
		return status;
	}
	if (camera) *camera = cam;
	*lights_out = lights;
	*light_count_out = count;
	return RISLTC_OK;
}

int risltc_quick_save(const char* path, const risltc_camera_t* camera, const polygonal_light_t* lights,
                      uint32_t light_count) {
	if (!path || !camera || (!lights && light_count)) return RISLTC_ERROR_INVALID_ARGUMENT;
	FILE* f = fopen(path, "wb");
	if (!f) return RISLTC_ERROR_IO;
	int ok = fwrite(camera, sizeof(*camera), 1, f) == 1;
	const uint32_t legacy_count = 0;
	ok = ok && fwrite(&legacy_count, sizeof(uint32_t), 1, f) == 1;
	ok = ok && fwrite(&light_count, sizeof(uint32_t), 1, f) == 1;
	for (uint32_t i = 0; ok && i != light_count; ++i) {
		const polygonal_light_t* light = &lights[i];
		ok = fwrite(light, QUICKSAVE_LIGHT_BYTES, 1, f) == 1;
		const uint64_t path_size = light->texture_file_path ? (uint64_t) strlen(light->texture_file_path) + 1 : 0;
		ok = ok && fwrite(&path_size, sizeof(path_size), 1, f) == 1;
		if (ok && path_size) ok = fwrite(light->texture_file_path, 1, path_size, f) == path_size;
		const uint64_t null_pointers[2] = {0, 0};
		ok = ok && fwrite(null_pointers, sizeof(null_pointers), 1, f) == 1;
		if (ok && light->vertex_count)
			ok = fwrite(light->vertices_plane_space, sizeof(float), 4 * (size_t) light->vertex_count, f) ==
			     4 * (size_t) light->vertex_count;
	}
	if (fclose(f) != 0) ok = 0;
	return ok ? RISLTC_OK : RISLTC_ERROR_IO;
}
