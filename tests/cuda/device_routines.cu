// device_routines.cu - a caller's own kernel composed from the GLSL-named
// device routines of include/risltc_device.cuh (clip_polygon,
// calculate_ltc, prepare_projected_solid_angle_polygon_sampling,
// sample_projected_solid_angle_polygon), the way a plugin would reuse them.
// Built by the tests into a shared library with the exact-numerics flags
// (--fmad=false, IEEE division and square root) and compared with the oracle.
//
// risltc_test_polygon_routines: for each of `count` polygons of n[c] (3..8)
// local-space vertices (xyz[c][8][3]), clips it to z >= 0, stores the clipped
// count and vertices (clipped[c][9][3]), calculate_ltc of the clipped polygon
// (ltc[c]), its projected solid angle (psa[c]) and `samples` sampled
// directions for the random pairs rnd[c][s][2] (dirs[c][s][3]); polygons that
// clip to nothing store count 0.  Host pointers; returns a cudaError_t.
#include <cuda_runtime.h>

#include "risltc_device.cuh"

namespace {

using risltc::ExactNumerics;
using risltc::f3;
namespace glsl = risltc::glsl;

constexpr int kMaxSamples = 8;

__global__ void polygon_routines_kernel(int count, const uint32_t* n, const float* xyz, int samples, const float* rnd,
                                        uint32_t* clipped_count, float* clipped, float* ltc, float* psa, float* dirs) {
	const int c = blockIdx.x * blockDim.x + threadIdx.x;
	if (c >= count) return;
	f3 v[risltc::kMaxPolygonVertices];
	for (int j = 0; j != risltc::kMaxPolygonVertices; ++j)
		v[j] = j < risltc::kMaxLightVertices
		           ? risltc::mk3(xyz[(c * 8 + j) * 3 + 0], xyz[(c * 8 + j) * 3 + 1], xyz[(c * 8 + j) * 3 + 2])
		           : risltc::mk3(0.0f, 0.0f, 0.0f);
	const uint32_t vc = glsl::clip_polygon<ExactNumerics>(n[c], v);
	clipped_count[c] = vc;
	for (uint32_t j = 0; j != vc; ++j) {
		clipped[(c * 9 + j) * 3 + 0] = v[j].x;
		clipped[(c * 9 + j) * 3 + 1] = v[j].y;
		clipped[(c * 9 + j) * 3 + 2] = v[j].z;
	}
	if (vc == 0) return;
	ltc[c] = glsl::calculate_ltc<ExactNumerics>(vc, v);
	const glsl::projected_solid_angle_polygon_t p =
	    glsl::prepare_projected_solid_angle_polygon_sampling<ExactNumerics>(vc, v);
	psa[c] = p.psa;
	for (int s = 0; s < samples && s < kMaxSamples; ++s) {
		const f3 d = glsl::sample_projected_solid_angle_polygon<ExactNumerics>(
		    p, risltc::mk2(rnd[(c * samples + s) * 2], rnd[(c * samples + s) * 2 + 1]));
		dirs[(c * samples + s) * 3 + 0] = d.x;
		dirs[(c * samples + s) * 3 + 1] = d.y;
		dirs[(c * samples + s) * 3 + 2] = d.z;
	}
}

}  // namespace

extern "C" int risltc_test_polygon_routines(int count, const uint32_t* n, const float* xyz, int samples,
                                            const float* rnd, uint32_t* clipped_count, float* clipped, float* ltc,
                                            float* psa, float* dirs) {
	if (count <= 0 || samples < 0 || samples > kMaxSamples) return (int) cudaErrorInvalidValue;
	const size_t sizes[9] = {count * sizeof(uint32_t), count * 24 * sizeof(float), count * samples * 2 * sizeof(float),
	                         count * sizeof(uint32_t), count * 27 * sizeof(float), count * sizeof(float),
	                         count * sizeof(float), count * samples * 3 * sizeof(float) + 4, 0};
	void* d[8] = {};
	cudaError_t e = cudaSuccess;
	for (int i = 0; i != 8 && e == cudaSuccess; ++i) e = cudaMalloc(&d[i], sizes[i] + 4);
	if (e == cudaSuccess) e = cudaMemcpy(d[0], n, sizes[0], cudaMemcpyHostToDevice);
	if (e == cudaSuccess) e = cudaMemcpy(d[1], xyz, sizes[1], cudaMemcpyHostToDevice);
	if (e == cudaSuccess) e = cudaMemcpy(d[2], rnd, sizes[2], cudaMemcpyHostToDevice);
	for (int i = 3; i != 8 && e == cudaSuccess; ++i) e = cudaMemset(d[i], 0, sizes[i]);
	if (e == cudaSuccess) {
		polygon_routines_kernel<<<(count + 127) / 128, 128>>>(
		    count, (const uint32_t*) d[0], (const float*) d[1], samples, (const float*) d[2], (uint32_t*) d[3],
		    (float*) d[4], (float*) d[5], (float*) d[6], (float*) d[7]);
		e = cudaGetLastError();
	}
	if (e == cudaSuccess) e = cudaDeviceSynchronize();
	if (e == cudaSuccess) e = cudaMemcpy(clipped_count, d[3], sizes[3], cudaMemcpyDeviceToHost);
	if (e == cudaSuccess) e = cudaMemcpy(clipped, d[4], sizes[4], cudaMemcpyDeviceToHost);
	if (e == cudaSuccess) e = cudaMemcpy(ltc, d[5], sizes[5], cudaMemcpyDeviceToHost);
	if (e == cudaSuccess) e = cudaMemcpy(psa, d[6], sizes[6], cudaMemcpyDeviceToHost);
	if (e == cudaSuccess && samples) e = cudaMemcpy(dirs, d[7], count * samples * 3 * sizeof(float), cudaMemcpyDeviceToHost);
	for (int i = 0; i != 8; ++i) cudaFree(d[i]);
	return (int) e;
}
