/* LTC tables without Vulkan: the quantisation of load_ltc_table
 * Restates upstream risltc code (GPLv3): see NOTICE.
 * (src/ltc_table.c:82-116) and its sampling constants (:184-192), the fit
 * file reader (:31-50), and a seeded synthetic fit that stands in for the
 * reference's fit files (not distributed with the reference).
 */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include "../../../include/risltc.h"

#define LTC_PI_F 3.1415926535897932384626433832795f

/* One fit record {m00, m02, m11, m20, albedo} of the LTC matrix
   M = [[d0, 0, d1], [0, d2, 0], [d3, 0, 1]]: store its adjugate (the inverse
   up to a factor) normalised so the largest magnitude is 1, as
   (m00, -m02, m11, m20 | m22, albedo), each clamped to [0, 1]. */
static void quantize_record(const float d[5], float out0[4], float out1[2], int unorm16) {
	float inv[3][3] = {{d[2], 0.0f, -d[1] * d[2]}, {0.0f, d[0] - d[1] * d[3], 0.0f}, {-d[2] * d[3], 0.0f, d[0] * d[2]}};
	float max_magnitude = fabsf(inv[0][0]);
	for (int k = 0; k != 3; ++k)
		for (int l = 0; l != 3; ++l)
			if (max_magnitude < fabsf(inv[k][l])) max_magnitude = fabsf(inv[k][l]);
	for (int k = 0; k != 3; ++k)
		for (int l = 0; l != 3; ++l) inv[k][l] /= max_magnitude;
	const float values[6] = {inv[0][0], inv[0][2], inv[1][1], inv[2][0], inv[2][2], d[4]};
	for (int i = 0; i != 6; ++i) {
		float v = values[i] * ((i == 1) ? -1.0f : 1.0f);
		if (v < 0.0f) v = 0.0f;
		if (v > 1.0f) v = 1.0f;
		if (unorm16) v = (float) (uint16_t) (v * 65535.0f + 0.5f) / 65535.0f;
		if (i < 4) out0[i] = v; else out1[i - 4] = v;
	}
}

static void set_constants(risltc_ltc_table_t* t) {
	memset(&t->constants, 0, sizeof(t->constants));
	t->constants.fresnel_index_factor = (float) (t->fresnel_count - 1);
	t->constants.fresnel_index_summand = 0.0f;
	t->constants.roughness_factor = (float) (t->roughness_count - 1) / (float) t->roughness_count;
	t->constants.roughness_summand = 0.5f / (float) t->roughness_count;
	t->constants.inclination_factor = (float) (t->inclination_count - 1) / (0.5f * LTC_PI_F * t->inclination_count);
	t->constants.inclination_summand = 0.5f / (float) t->inclination_count;
}

static int allocate(risltc_ltc_table_t* t, uint32_t rough, uint32_t incl, uint32_t layers) {
	memset(t, 0, sizeof(*t));
	size_t n = (size_t) rough * incl * layers;
	t->texels0 = (float*) malloc(n * 4 * sizeof(float));
	t->texels1 = (float*) malloc(n * 2 * sizeof(float));
	if (!t->texels0 || !t->texels1) {
		free(t->texels0);
		free(t->texels1);
		memset(t, 0, sizeof(*t));
		return RISLTC_ERROR_OUT_OF_MEMORY;
	}
	t->roughness_count = rough;
	t->inclination_count = incl;
	t->fresnel_count = layers;
	return RISLTC_OK;
}

int risltc_ltc_table_from_fit(risltc_ltc_table_t* table, const float* fit, uint32_t resolution, uint32_t fresnel_count,
                              int quantize_unorm16) {
	if (!table || !fit || resolution < 2 || fresnel_count < 1) return RISLTC_ERROR_INVALID_ARGUMENT;
	int status = allocate(table, resolution, resolution, fresnel_count);
	if (status) return status;
	size_t per_layer = (size_t) resolution * resolution;
	for (size_t i = 0; i != per_layer * fresnel_count; ++i)
		quantize_record(fit + 5 * i, table->texels0 + 4 * i, table->texels1 + 2 * i, quantize_unorm16);
	set_constants(table);
	return RISLTC_OK;
}

int risltc_load_ltc_table(risltc_ltc_table_t* table, const char* directory, uint32_t fresnel_count,
                          int quantize_unorm16) {
	if (!table || !directory || fresnel_count < 1) return RISLTC_ERROR_INVALID_ARGUMENT;
	float* fit = NULL;
	uint64_t resolution = 0;
	for (uint32_t i = 0; i != fresnel_count; ++i) {
		char path[4096];
		snprintf(path, sizeof(path), "%s/fit%u.dat", directory, i);
		FILE* f = fopen(path, "rb");
		if (!f) {
			free(fit);
			return RISLTC_ERROR_IO;
		}
		uint64_t res = 0;
		if (fread(&res, sizeof(res), 1, f) != 1 || res < 2 || res > 4096 || (resolution && res != resolution)) {
			fclose(f);
			free(fit);
			return RISLTC_ERROR_IO;
		}
		if (!fit) {
			resolution = res;
			fit = (float*) malloc(sizeof(float) * 5 * res * res * fresnel_count);
			if (!fit) {
				fclose(f);
				return RISLTC_ERROR_OUT_OF_MEMORY;
			}
		}
		size_t count = 5 * (size_t) res * res;
		size_t got = fread(fit + count * i, sizeof(float), count, f);
		fclose(f);
		if (got != count) {
			free(fit);
			return RISLTC_ERROR_IO;
		}
	}
	int status = risltc_ltc_table_from_fit(table, fit, (uint32_t) resolution, fresnel_count, quantize_unorm16);
	free(fit);
	return status;
}

static uint64_t splitmix64(uint64_t* state) {
	uint64_t z = (*state += 0x9E3779B97F4A7C15ull);
	z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
	z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
	return z ^ (z >> 31);
}

static double uniform01(uint64_t* state) { return (double) (splitmix64(state) >> 11) * (1.0 / 9007199254740992.0); }

/* Smooth synthetic fit over (linear roughness r in [0,1], inclination t in
   [0, pi/2]): M = [[a, 0, b], [0, a, 0], [d, 0, 1]] with a = 1 + 6 (1 - r)^2,
   b = 0.3 sin(t) (1 - r) >= 0 and d = -0.4 sin(t) (1 - r) <= 0 (so every stored
   entry is non-negative), each modulated by a seeded low-frequency wave of
   amplitude 5%; albedo = 0.1 + 0.8 (1 - r) cos(t)^0.3. */
int risltc_ltc_table_synthetic(risltc_ltc_table_t* table, uint64_t seed, uint32_t roughness_count,
                               uint32_t inclination_count) {
	if (!table || roughness_count < 2 || inclination_count < 2) return RISLTC_ERROR_INVALID_ARGUMENT;
	uint64_t state = seed;
	double phase[4], freq[4];
	for (int i = 0; i != 4; ++i) {
		phase[i] = 6.283185307179586 * uniform01(&state);
		freq[i] = 1.0 + 2.0 * uniform01(&state);
	}
	size_t n = (size_t) roughness_count * inclination_count;
	float* fit = (float*) malloc(sizeof(float) * 5 * n);
	if (!fit) return RISLTC_ERROR_OUT_OF_MEMORY;
	for (uint32_t y = 0; y != inclination_count; ++y) {
		double t = 0.5 * 3.141592653589793 * y / (inclination_count - 1);
		for (uint32_t x = 0; x != roughness_count; ++x) {
			double r = (double) x / (roughness_count - 1);
			double w[4];
			for (int i = 0; i != 4; ++i) w[i] = 1.0 + 0.05 * sin(freq[i] * (2.0 * r + t) + phase[i]);
			double a = (1.0 + 6.0 * (1.0 - r) * (1.0 - r)) * w[0];
			double b = 0.3 * sin(t) * (1.0 - r) * w[1];
			double d = -0.4 * sin(t) * (1.0 - r) * w[2];
			double albedo = (0.1 + 0.8 * (1.0 - r) * pow(cos(t) > 0.0 ? cos(t) : 0.0, 0.3)) * w[3];
			float* rec = fit + 5 * ((size_t) y * roughness_count + x);
			rec[0] = (float) a;
			rec[1] = (float) b;
			rec[2] = (float) a;
			rec[3] = (float) d;
			rec[4] = (float) (albedo < 0.0 ? 0.0 : (albedo > 1.0 ? 1.0 : albedo));
		}
	}
	int status = allocate(table, roughness_count, inclination_count, 1);
	if (status == RISLTC_OK) {
		for (size_t i = 0; i != n; ++i) quantize_record(fit + 5 * i, table->texels0 + 4 * i, table->texels1 + 2 * i, 0);
		set_constants(table);
	}
	free(fit);
	return status;
}

void risltc_ltc_table_destroy(risltc_ltc_table_t* table) {
	if (!table) return;
	free(table->texels0);
	free(table->texels1);
	memset(table, 0, sizeof(*table));
}
