/* OpenMP frame driver over the FP32 oracle: the CPU baseline that bench.py
   times ("the reference GLSL routines compiled as C99 with OpenMP on the
   host cores").  Rows are scheduled dynamically.  TEST INFRASTRUCTURE. */
#include <omp.h>
#include "oracle.h"

int oracle_max_threads(void) { return omp_get_max_threads(); }

int oracle_render_frame_f32(const oracle_scene_t* scene, const oracle_settings_t* settings,
                            const oracle_gbuffer_t* gbuffer, uint32_t random_number_x, int threads, int row_begin,
                            int row_end, float* out_rgb, oracle_reservoir_t* out_reservoirs, double* out_seconds) {
	int status = 0;
	if (threads <= 0) threads = omp_get_max_threads();
	double t0 = omp_get_wtime();
#pragma omp parallel for schedule(dynamic, 1) num_threads(threads) reduction(| : status)
	for (int y = row_begin; y < row_end; ++y)
		status |= oracle_render_f32(scene, settings, gbuffer, random_number_x, y, y + 1, out_rgb, out_reservoirs);
	if (out_seconds) *out_seconds = omp_get_wtime() - t0;
	return status;
}

/* The listed pixels of one frame (see oracle_render_pixels_f32), in chunks
   of 64 scheduled dynamically over the threads. */
int oracle_render_pixels_omp_f32(const oracle_scene_t* scene, const oracle_settings_t* settings,
                                 const oracle_gbuffer_t* gbuffer, uint32_t random_number_x, const uint32_t* pixels,
                                 int count, int threads, float* out_rgb, oracle_reservoir_t* out_reservoirs,
                                 double* out_seconds) {
	int status = 0;
	if (threads <= 0) threads = omp_get_max_threads();
	double t0 = omp_get_wtime();
#pragma omp parallel for schedule(dynamic, 1) num_threads(threads) reduction(| : status)
	for (int b = 0; b < count; b += 64) {
		const int e = b + 64 < count ? b + 64 : count;
		status |= oracle_render_pixels_f32(scene, settings, gbuffer, random_number_x, pixels, (size_t) b, (size_t) e,
		                                   out_rgb, out_reservoirs);
	}
	if (out_seconds) *out_seconds = omp_get_wtime() - t0;
	return status;
}

/* Any-hit queries of oracle_f32_any_hit over the threads (rays are
   independent). */
void oracle_f32_any_hit(const oracle_scene_t* s, const float* rays, uint32_t count, uint32_t* hits);
void oracle_f32_any_hit_omp(const oracle_scene_t* s, const float* rays, uint32_t count, uint32_t* hits) {
#pragma omp parallel for schedule(dynamic, 64)
	for (int64_t i = 0; i < (int64_t) count; ++i) oracle_f32_any_hit(s, rays + 8 * i, 1, hits + i);
}
