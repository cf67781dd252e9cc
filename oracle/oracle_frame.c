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
