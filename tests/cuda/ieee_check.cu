// ieee_check.cu - exhaustive check of the Markstein sequences of
// shade_device.cuh (rcp_markstein, rsqrt_markstein, div_markstein) and of its
// branch-free square root (sqrt_tuckerman) against CUDA's correctly rounded
// intrinsics, on this GPU's approximation unit.
//
// risltc_test_markstein(counts) fills counts[7]:
//   0 reciprocals differing from __frcp_rn over every float in [2^-126, 2^126);
//   1 reciprocal square roots differing from __frcp_rn(__fsqrt_rn(x)) over
//     every 32-bit pattern x (bitwise; results that are both NaN agree);
//   2 quotients differing from __fdiv_rn for every divisor in [2, 16) with
//     eight numerators each, spread over [0.5, 2) (the edge integral's
//     operands lie in [0.85, 1.37] / [3.41, 8.58]);
//   3 the number of quotients checked;
//   4 quotients differing over 2^28 pseudo-random pairs with numerators in
//     [0.85, 1.37] and divisors in [3.41, 8.58];
//   5 square roots differing from __fsqrt_rn over every float in
//     [2^-76, 2^126];
//   6 the number of 32-bit patterns tuckerman_range admits.
// Returns a cudaError_t.
#include <cuda_runtime.h>

#include "../../risltc_gb300/csrc/cuda/shade_device.cuh"

namespace {

__device__ bool same(float a, float b) {
	return __float_as_uint(a) == __float_as_uint(b) || (isnan(a) && isnan(b));
}

__global__ void markstein_unary_kernel(unsigned long long* counts) {
	unsigned long long bad[2] = {0, 0};
	for (uint64_t u = blockIdx.x * (uint64_t) blockDim.x + threadIdx.x; u < (1ull << 32);
	     u += (uint64_t) gridDim.x * blockDim.x) {
		const float x = __uint_as_float((uint32_t) u);
		const uint32_t mag = (uint32_t) u & 0x7fffffffu;
		if (mag >= 0x00800000u && mag < 0x7e800000u) bad[0] += !same(risltc::rcp_markstein(x), __frcp_rn(x));
		bad[1] += !same(risltc::rsqrt_markstein(x), __frcp_rn(__fsqrt_rn(x)));
	}
	for (int k = 0; k != 2; ++k)
		if (bad[k]) atomicAdd(counts + k, bad[k]);
}

__global__ void markstein_div_kernel(unsigned long long* counts) {
	const uint32_t lo = 0x40000000u, hi = 0x41800000u;  // [2, 16)
	unsigned long long bad = 0, checked = 0;
	for (uint32_t u = lo + blockIdx.x * blockDim.x + threadIdx.x; u < hi; u += gridDim.x * blockDim.x) {
		const float b = __uint_as_float(u);
		uint32_t h = u * 2654435761u;
		for (int k = 0; k != 8; ++k) {
			h = h * 1664525u + 1013904223u;
			// A numerator in [0.5, 2): exponent -1 or 0, random significand.
			const float a = __uint_as_float(((k & 1) ? 0x3F000000u : 0x3F800000u) | (h >> 9));
			bad += !same(risltc::div_markstein(a, b), __fdiv_rn(a, b));
			++checked;
		}
	}
	atomicAdd(counts + 2, bad);
	atomicAdd(counts + 3, checked);
}

__global__ void markstein_edge_div_kernel(unsigned long long* counts) {
	unsigned long long bad = 0;
	for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < (1u << 28); i += gridDim.x * blockDim.x) {
		uint32_t h = i * 2654435761u + 12345u;
		h ^= h >> 15;
		h *= 2246822519u;
		h ^= h >> 13;
		uint32_t g = h * 3266489917u + i;
		g ^= g >> 16;
		const float a = 0.85f + 0.52f * ((float) (h >> 8) * (1.0f / 16777216.0f));
		const float b = 3.41f + 5.17f * ((float) (g >> 8) * (1.0f / 16777216.0f));
		bad += !same(risltc::div_markstein(a, b), __fdiv_rn(a, b));
	}
	if (bad) atomicAdd(counts + 4, bad);
}

// Every float d in [2^-76, 2^126]: the branch-free square root against
// __fsqrt_rn (counter 5), and the range test (counter 6 counts the floats it
// admits; the range holds 0x7e800000 - 0x19800000 + 1 of them).
__global__ void tuckerman_sqrt_kernel(unsigned long long* counts) {
	const uint32_t lo = 0x19800000u, hi = 0x7e800000u;
	unsigned long long bad = 0;
	for (uint32_t u = lo + blockIdx.x * blockDim.x + threadIdx.x; u <= hi; u += gridDim.x * blockDim.x)
		bad += !same(risltc::sqrt_tuckerman(__uint_as_float(u)), __fsqrt_rn(__uint_as_float(u)));
	if (bad) atomicAdd(counts + 5, bad);
	unsigned long long admitted = 0;
	for (uint64_t u = blockIdx.x * (uint64_t) blockDim.x + threadIdx.x; u < (1ull << 32);
	     u += (uint64_t) gridDim.x * blockDim.x)
		admitted += risltc::tuckerman_range(__uint_as_float((uint32_t) u)) ? 1 : 0;
	atomicAdd(counts + 6, admitted);
}

}  // namespace

extern "C" int risltc_test_markstein(unsigned long long* counts) {
	unsigned long long* d = nullptr;
	cudaError_t e = cudaMalloc(&d, 7 * sizeof(unsigned long long));
	if (e == cudaSuccess) e = cudaMemset(d, 0, 7 * sizeof(unsigned long long));
	if (e == cudaSuccess) {
		markstein_unary_kernel<<<152 * 16, 256>>>(d);
		markstein_div_kernel<<<152 * 16, 256>>>(d);
		markstein_edge_div_kernel<<<152 * 16, 256>>>(d);
		tuckerman_sqrt_kernel<<<152 * 16, 256>>>(d);
		e = cudaGetLastError();
	}
	if (e == cudaSuccess) e = cudaDeviceSynchronize();
	if (e == cudaSuccess) e = cudaMemcpy(counts, d, 7 * sizeof(unsigned long long), cudaMemcpyDeviceToHost);
	cudaFree(d);
	return (int) e;
}
