/* Light clusters for the cluster proposal of the RIS candidates (a row the
 * reference does not have: its candidates are drawn uniformly over all lights,
 * shading_pass.frag.glsl:728-733).
 *
 * k-means (Lloyd's algorithm with k-means++ seeding, Arthur & Vassilvitskii
 * 2007) of the lights' centres.  All arithmetic is in double with a splitmix64
 * stream, compiled without contraction, so the result is the same on every
 * host.  The output lists the lights cluster by cluster (ascending light index
 * inside a cluster) and the clusters' summaries used by the proposal kernels.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include "../../../include/risltc.h"

static uint64_t splitmix64(uint64_t* state) {
	uint64_t z = (*state += 0x9E3779B97F4A7C15ull);
	z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
	z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
	return z ^ (z >> 31);
}

static double uniform01(uint64_t* state) { return (double) (splitmix64(state) >> 11) * (1.0 / 9007199254740992.0); }

static double dist2(const double* a, const float* b) {
	const double dx = a[0] - b[0], dy = a[1] - b[1], dz = a[2] - b[2];
	return dx * dx + dy * dy + dz * dz;
}

int risltc_cluster_lights(const float* centers, uint32_t light_count, uint32_t cluster_count, uint64_t seed,
                          uint32_t iterations, uint32_t* order, uint32_t* offsets) {
	if (!centers || !order || !offsets || light_count == 0 || cluster_count == 0 || cluster_count > light_count)
		return RISLTC_ERROR_INVALID_ARGUMENT;
	const uint32_t n = light_count, k = cluster_count;
	double* means = (double*) malloc(sizeof(double) * 3 * k);
	double* d2 = (double*) malloc(sizeof(double) * n);
	double* sums = (double*) malloc(sizeof(double) * 4 * k);
	uint32_t* label = (uint32_t*) malloc(sizeof(uint32_t) * n);
	if (!means || !d2 || !sums || !label) {
		free(means);
		free(d2);
		free(sums);
		free(label);
		return RISLTC_ERROR_OUT_OF_MEMORY;
	}
	uint64_t rng = seed;
	/* k-means++ seeding: the first centre uniformly, then each next one with
	   probability proportional to the squared distance to the nearest. */
	uint32_t first = (uint32_t) (uniform01(&rng) * n);
	if (first >= n) first = n - 1;
	for (int a = 0; a != 3; ++a) means[a] = centers[3 * first + a];
	for (uint32_t i = 0; i != n; ++i) d2[i] = dist2(means, centers + 3 * i);
	for (uint32_t c = 1; c != k; ++c) {
		double total = 0.0;
		for (uint32_t i = 0; i != n; ++i) total += d2[i];
		uint32_t pick = n - 1;
		if (total > 0.0) {
			double target = uniform01(&rng) * total, acc = 0.0;
			for (uint32_t i = 0; i != n; ++i) {
				acc += d2[i];
				if (acc > target) {
					pick = i;
					break;
				}
			}
		} else {
			pick = (uint32_t) (uniform01(&rng) * n);
			if (pick >= n) pick = n - 1;
		}
		for (int a = 0; a != 3; ++a) means[3 * c + a] = centers[3 * pick + a];
		for (uint32_t i = 0; i != n; ++i) {
			const double d = dist2(means + 3 * c, centers + 3 * i);
			if (d < d2[i]) d2[i] = d;
		}
	}
	/* Lloyd iterations; ties go to the lower cluster index. */
	for (uint32_t it = 0; it <= iterations; ++it) {
		int changed = 0;
		for (uint32_t i = 0; i != n; ++i) {
			uint32_t best = 0;
			double best_d = dist2(means, centers + 3 * i);
			for (uint32_t c = 1; c != k; ++c) {
				const double d = dist2(means + 3 * c, centers + 3 * i);
				if (d < best_d) {
					best_d = d;
					best = c;
				}
			}
			if (it == 0 || label[i] != best) changed = 1;
			label[i] = best;
		}
		if (!changed || it == iterations) break;
		memset(sums, 0, sizeof(double) * 4 * k);
		for (uint32_t i = 0; i != n; ++i) {
			double* s = sums + 4 * label[i];
			for (int a = 0; a != 3; ++a) s[a] += centers[3 * i + a];
			s[3] += 1.0;
		}
		for (uint32_t c = 0; c != k; ++c)
			if (sums[4 * c + 3] > 0.0)
				for (int a = 0; a != 3; ++a) means[3 * c + a] = sums[4 * c + a] / sums[4 * c + 3];
	}
	/* Counting sort of the lights by cluster (stable). */
	memset(offsets, 0, sizeof(uint32_t) * (k + 1));
	for (uint32_t i = 0; i != n; ++i) ++offsets[label[i] + 1];
	for (uint32_t c = 0; c != k; ++c) offsets[c + 1] += offsets[c];
	for (uint32_t c = 0; c != k; ++c) sums[c] = (double) offsets[c];  /* cursors */
	for (uint32_t i = 0; i != n; ++i) order[(uint32_t) sums[label[i]]++] = i;
	free(means);
	free(d2);
	free(sums);
	free(label);
	return RISLTC_OK;
}

int risltc_cluster_summaries(const float* lights_std140, uint32_t light_count, uint32_t max_vertex_count,
                             const uint32_t* offsets, uint32_t cluster_count, float* bounds, float* power) {
	if (!lights_std140 || !offsets || !bounds || !power || cluster_count == 0 || max_vertex_count < 3 ||
	    offsets[0] != 0 || offsets[cluster_count] != light_count)
		return RISLTC_ERROR_INVALID_ARGUMENT;
	const size_t stride = 12 + 4 * (size_t) max_vertex_count;
	for (uint32_t c = 0; c != cluster_count; ++c)
		if (offsets[c + 1] < offsets[c]) return RISLTC_ERROR_INVALID_ARGUMENT;
	for (uint32_t c = 0; c != cluster_count; ++c) {
		double centre[3] = {0.0, 0.0, 0.0}, radius = 0.0, watts = 0.0;
		uint32_t count = 0;
		for (uint32_t l = offsets[c]; l != offsets[c + 1]; ++l) {
			const float* row = lights_std140 + stride * l;
			uint32_t nv;
			memcpy(&nv, row + 8, sizeof(nv));
			if (nv > max_vertex_count) return RISLTC_ERROR_VERTEX_COUNT;
			const float* v = row + 12;
			for (uint32_t i = 0; i != nv; ++i)
				for (int a = 0; a != 3; ++a) centre[a] += v[4 * i + a];
			count += nv;
			/* Area by a fan from vertex 0; luminance of the radiance. */
			double area = 0.0;
			for (uint32_t i = 1; i + 1 < nv; ++i) {
				double e1[3], e2[3];
				for (int a = 0; a != 3; ++a) {
					e1[a] = (double) v[4 * i + a] - v[a];
					e2[a] = (double) v[4 * (i + 1) + a] - v[a];
				}
				const double cx = e1[1] * e2[2] - e1[2] * e2[1], cy = e1[2] * e2[0] - e1[0] * e2[2],
				             cz = e1[0] * e2[1] - e1[1] * e2[0];
				area += 0.5 * sqrt(cx * cx + cy * cy + cz * cz);
			}
			watts += (0.2126 * row[0] + 0.7152 * row[1] + 0.0722 * row[2]) * area;
		}
		if (count)
			for (int a = 0; a != 3; ++a) centre[a] /= count;
		for (int a = 0; a != 3; ++a) bounds[4 * c + a] = (float) centre[a];
		for (uint32_t l = offsets[c]; l != offsets[c + 1]; ++l) {
			const float* row = lights_std140 + stride * l;
			uint32_t nv;
			memcpy(&nv, row + 8, sizeof(nv));
			for (uint32_t i = 0; i != nv; ++i) {
				/* Distance to the stored (float) centre, so the sphere holds
				   the vertices around the centre the kernels use. */
				double d2 = 0.0;
				for (int a = 0; a != 3; ++a) {
					const double d = (double) row[12 + 4 * i + a] - (double) bounds[4 * c + a];
					d2 += d * d;
				}
				if (sqrt(d2) > radius) radius = sqrt(d2);
			}
		}
		/* Rounded up so that the sphere still holds every vertex. */
		bounds[4 * c + 3] = nextafterf((float) radius, INFINITY);
		power[c] = (float) watts;
	}
	return RISLTC_OK;
}
