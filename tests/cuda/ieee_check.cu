// ieee_check.cu - exhaustive check of the Markstein sequences of
// shade_device.cuh (sqrt_markstein, rcp_markstein, div_markstein) against
// CUDA's correctly rounded intrinsics, on this GPU's approximation units.
//
// risltc_test_markstein(counts) fills counts[7]:
//   0 square roots differing from __fsqrt_rn over every positive normal float;
//   1 reciprocals differing from __frcp_rn over every float in [2^-126, 2^126);
//   2 reciprocal square roots rcp(sqrt(x)) differing from
//     __frcp_rn(__fsqrt_rn(x)) over every positive normal float;
//   3 reciprocals differing over every divisor in [2, 16);
//   4 quotients differing from __fdiv_rn for every divisor in [2, 16) with
//     eight numerators each, spread over [0.5, 2);
//   5 the number of quotients checked;
//   6 quotients differing from __fdiv_rn over 2^28 pseudo-random pairs whose
//     magnitudes span [2^-60, 2^60] (either sign), the operand range of
//     ExactNumerics::div_moderate.
// Returns a cudaError_t.
#include <cuda_runtime.h>

#include "../../risltc_gb300/csrc/cuda/shade_device.cuh"

namespace {

__global__ void markstein_unary_kernel(unsigned long long* counts) {
	const uint64_t lo = 0x00800000u, hi = 0x7F800000u;  // positive normal floats
	unsigned long long bad[3] = {0, 0, 0};
	for (uint64_t u = lo + blockIdx.x * (uint64_t) blockDim.x + threadIdx.x; u < hi;
	     u += (uint64_t) gridDim.x * blockDim.x) {
		const float x = __uint_as_float((uint32_t) u);
		bad[0] += risltc::sqrt_markstein(x) != __fsqrt_rn(x);
		if (u < 0x7E800000u) bad[1] += risltc::rcp_markstein(x) != __frcp_rn(x);
		bad[2] += risltc::rcp_markstein(risltc::sqrt_markstein(x)) != __frcp_rn(__fsqrt_rn(x));
	}
	for (int k = 0; k != 3; ++k)
		if (bad[k]) atomicAdd(counts + k, bad[k]);
}

__global__ void markstein_div_kernel(unsigned long long* counts) {
	const uint32_t lo = 0x40000000u, hi = 0x41800000u;  // [2, 16)
	unsigned long long bad_rcp = 0, bad_div = 0, checked = 0;
	for (uint32_t u = lo + blockIdx.x * blockDim.x + threadIdx.x; u < hi; u += gridDim.x * blockDim.x) {
		const float b = __uint_as_float(u);
		const float y = risltc::rcp_markstein(b);
		bad_rcp += y != __frcp_rn(b);
		uint32_t h = u * 2654435761u;
		for (int k = 0; k != 8; ++k) {
			h = h * 1664525u + 1013904223u;
			// A numerator in [0.5, 2): exponent -1 or 0, random significand.
			const float a = __uint_as_float(((k & 1) ? 0x3F000000u : 0x3F800000u) | (h >> 9));
			bad_div += risltc::div_markstein(a, b, y) != __fdiv_rn(a, b);
			++checked;
		}
	}
	atomicAdd(counts + 3, bad_rcp);
	atomicAdd(counts + 4, bad_div);
	atomicAdd(counts + 5, checked);
}

__global__ void markstein_wide_div_kernel(unsigned long long* counts) {
	unsigned long long bad = 0;
	for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < (1u << 28); i += gridDim.x * blockDim.x) {
		uint32_t h = i * 2654435761u + 12345u;
		h ^= h >> 15;
		h *= 2246822519u;
		h ^= h >> 13;
		uint32_t g = h * 3266489917u + i;
		g ^= g >> 16;
		// Exponents 67..187 (2^-60 .. 2^60), random significands and signs.
		const float a = __uint_as_float(((h >> 31) << 31) | ((67u + (h >> 8) % 121u) << 23) | (g >> 9));
		const float b = __uint_as_float((((g >> 30) & 1u) << 31) | ((67u + (g >> 1) % 121u) << 23) | (h & 0x7FFFFFu));
		bad += risltc::div_markstein(a, b, risltc::rcp_markstein(b)) != __fdiv_rn(a, b);
	}
	if (bad) atomicAdd(counts + 6, bad);
}

}  // namespace

extern "C" int risltc_test_markstein(unsigned long long* counts) {
	unsigned long long* d = nullptr;
	cudaError_t e = cudaMalloc(&d, 7 * sizeof(unsigned long long));
	if (e == cudaSuccess) e = cudaMemset(d, 0, 7 * sizeof(unsigned long long));
	if (e == cudaSuccess) {
		markstein_unary_kernel<<<152 * 16, 256>>>(d);
		markstein_div_kernel<<<152 * 16, 256>>>(d);
		markstein_wide_div_kernel<<<152 * 16, 256>>>(d);
		e = cudaGetLastError();
	}
	if (e == cudaSuccess) e = cudaDeviceSynchronize();
	if (e == cudaSuccess) e = cudaMemcpy(counts, d, 7 * sizeof(unsigned long long), cudaMemcpyDeviceToHost);
	cudaFree(d);
	return (int) e;
}
