// mlp.cuh - the learned cluster proposal's model: a small MLP from a shading
// point to logits over the light clusters (not in the reference).
//
//   inputs (10): position (centred and scaled by the model's input
//     transform), normal, outgoing direction, roughness;
//   encoding (144): per input u: u, sin(2^k pi u), cos(2^k pi u), k = 0..5
//     (130 features, zero-padded to 144), the higher frequencies from
//     sincospi(u) by the double-angle formulas;
//   layer 1: 144 -> 64, ReLU; layer 2: 64 -> 64, ReLU; layer 3: 64 -> K.
//
// Weights are BF16 for inference (each layer stored [out][in]), biases FP32.
// The forward pass runs on the tcgen05 tensor cores (mlp_tc.cuh); online
// training runs there too for up to 256 clusters (mlp_train_tc.cuh), and in
// FP32 on the CUDA cores (below) for larger models or on request.
#pragma once
#include <cuda_bf16.h>
#include "proposal.cuh"
#include "shade_device.cuh"

namespace risltc {

constexpr int kMlpInputs = 10;
constexpr int kMlpFrequencies = 6;
constexpr int kMlpFeatures = 144;  // 10 * 13 = 130, padded to a multiple of 16
constexpr int kMlpHidden = 64;

// Offsets (in floats) of the parameters in the model's FP32 parameter vector.
struct MlpLayout {
	int w1, b1, w2, b2, w3, b3, total;
};
inline __host__ __device__ MlpLayout mlp_layout(int k_count) {
	MlpLayout l;
	l.w1 = 0;
	l.b1 = l.w1 + kMlpHidden * kMlpFeatures;
	l.w2 = l.b1 + kMlpHidden;
	l.b2 = l.w2 + kMlpHidden * kMlpHidden;
	l.w3 = l.b2 + kMlpHidden;
	l.b3 = l.w3 + k_count * kMlpHidden;
	l.total = l.b3 + k_count;
	return l;
}

// The BF16 weights in the tensor cores' operand layout: W1 (64 x 144), W2
// (64 x 64) and W3 (k_count rows, zero rows up to a multiple of 16, x 64),
// each K-major in 8x8 core matrices (element (row, col) of a matrix with k
// columns at byte ((row / 8) * (k / 8) + col / 8) * 128 + (row % 8) * 16 +
// (col % 8) * 2), one after another, so that a kernel stages all three with
// one bulk copy.
__host__ __device__ constexpr uint32_t tc_offset(int row, int col, int k) {
	return (uint32_t) (((row >> 3) * (k >> 3) + (col >> 3)) * 128 + (row & 7) * 16 + (col & 7) * 2);
}
__host__ __device__ inline int mlp_padded_clusters(int k_count) { return (k_count + 15) / 16 * 16; }
__host__ __device__ inline int mlp_weight_elements(int k_count) {
	return kMlpHidden * kMlpFeatures + kMlpHidden * kMlpHidden + mlp_padded_clusters(k_count) * kMlpHidden;
}
// Element of the operand-layout weights holding parameter j, or -1 for a bias.
__host__ __device__ inline int mlp_weight_slot(int j, int k_count) {
	const MlpLayout l = mlp_layout(k_count);
	if (j >= l.w1 && j < l.b1) return (int) tc_offset((j - l.w1) / kMlpFeatures, (j - l.w1) % kMlpFeatures, kMlpFeatures) / 2;
	const int w2_base = kMlpHidden * kMlpFeatures, w3_base = w2_base + kMlpHidden * kMlpHidden;
	if (j >= l.w2 && j < l.b2) return w2_base + (int) tc_offset((j - l.w2) / kMlpHidden, (j - l.w2) % kMlpHidden, kMlpHidden) / 2;
	if (j >= l.w3 && j < l.b3) return w3_base + (int) tc_offset((j - l.w3) / kMlpHidden, (j - l.w3) % kMlpHidden, kMlpHidden) / 2;
	return -1;
}

struct MlpParams {
	const float* gbuffer;
	const uint32_t* primitive;
	uint32_t width, height;
	const __nv_bfloat16* weights;  // BF16 weights in the operand layout (mlp_weight_slot)
	const float* params;           // FP32 parameter vector (biases read from here)
	int k_count;                   // clusters, a multiple of 8
	float center[3], inv_half_extent;
	__nv_bfloat16* logits;         // [pixel][k_count]
	uint32_t* error;               // the context's error word
	uint32_t skip_issue;           // fault injection: issue no tensor-core products
};

// Input `input` (0..9) of pixel i: position (centred and scaled), normal,
// outgoing direction, roughness.
RL_DEV float mlp_input(const float* g, uint32_t np, uint32_t i, const float center[3], float inv_half_extent,
                       int input) {
	const size_t snp = np;
	if (input < 3) return (g[input * snp + i] - center[input]) * inv_half_extent;
	return g[(input < 9 ? input : 16) * snp + i];
}

// The 13 features of one input x: x, sin(2^k pi x) for k = 0..5, then
// cos(2^k pi x) for k = 0..5.  sincospi once, then the double-angle
// formulas (sin 2a = 2 sin a cos a, cos 2a = (cos a - sin a)(cos a + sin a));
// their FP32 error stays far below the BF16 rounding of the features.
RL_DEV void mlp_encode(float x, float out[13]) {
	out[0] = x;
	float s, c;
	sincospif(x, &s, &c);
#pragma unroll
	for (int k = 0; k != kMlpFrequencies; ++k) {
		out[1 + k] = s;
		out[1 + kMlpFrequencies + k] = c;
		const float s2 = 2.0f * s * c, c2 = (c - s) * (c + s);
		s = s2;
		c = c2;
	}
}

RL_DEV uint32_t pack_bf16x2(float lo, float hi) {
	const __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
	return *reinterpret_cast<const uint32_t*>(&v);
}

// Whether parameter j is a weight of one of layer 1's padding features
// (130..143), whose BF16 copy is always zero.
__host__ __device__ inline bool mlp_padding_weight(int j) {
	return j < kMlpHidden * kMlpFeatures && j % kMlpFeatures >= kMlpInputs * 13;
}

// FP32 parameters to the BF16 operand-layout weights (zero padding rows are
// left as the allocation's zeros).
static __global__ void mlp_convert_kernel(const float* params, __nv_bfloat16* weights, int count, int k_count) {
	for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < count; j += gridDim.x * blockDim.x) {
		const int slot = mlp_weight_slot(j, k_count);
		if (slot >= 0) weights[slot] = __float2bfloat16_rn(mlp_padding_weight(j) ? 0.0f : params[j]);
	}
}

// BF16 logits to FP32 (for inspection).
static __global__ void bf16_to_f32_kernel(const __nv_bfloat16* in, float* out, size_t count) {
	for (size_t j = blockIdx.x * (size_t) blockDim.x + threadIdx.x; j < count; j += (size_t) gridDim.x * blockDim.x)
		out[j] = __bfloat162float(in[j]);
}

}  // namespace risltc

namespace risltc {

// ----------------------------------------------------------------- training --
// Online training of the proposal on the RIS candidates of a frame: for each
// training pixel the candidates' weights w = p_hat / p (the LTC-CP target
// over the proposal probability, written back by the candidate kernel) give
// an estimate of each cluster's share of the pixel's unshadowed shading,
// F_c; the loss is the cross entropy between the normalised estimate
// T_c = F_c / sum F and q = softmax(logits), whose gradient in the logits is
// (q - T) / B over the B training pixels.  The shadowed part: the frame's
// final estimate f(y) W for the chosen light y is an unbiased estimate of the
// shadowed shading of y's cluster alone (RIS integrates f times the cluster's
// indicator), so with s = lum(f W) over the unshadowed estimate sum w / M
// (clamped to 4) it adds s (q - onehot(cluster(y))) / B; the two parts are
// mixed by shadowed_weight.  Forward and backward run in FP32 from the FP32 master
// parameters, one block per 32 training pixels, partial weight gradients
// summed in shared memory and added to the gradient vector once per block.
// In the products lane l takes training pixel l and each warp a share of the
// outputs, so every weight load is the same address across the warp (one
// broadcast) and the activations are read from shared-memory rows whose odd
// strides put the 32 pixels in 32 banks.
constexpr int kTrainPixels = 32;   // training pixels per block step (one per lane)
constexpr int kTrainThreads = 256;
constexpr int kTrainWarps = kTrainThreads / 32;
constexpr int kFeatStride = kMlpFeatures + 1;   // odd row strides in shared memory
constexpr int kHiddenStride = kMlpHidden + 1;
__host__ __device__ inline int train_logit_stride(int k_count) { return k_count | 1; }

struct MlpTrainParams {
	const float* gbuffer;
	uint32_t width, height;
	const float* params;          // FP32 parameter vector
	float* grad;                  // FP32 gradient vector (accumulated)
	int k_count;
	float center[3], inv_half_extent;
	const uint32_t* offsets;      // cluster offsets (light -> cluster via light_cluster)
	const uint32_t* light_cluster;
	uint32_t light_count;         // candidates naming another light are skipped
	const uint32_t* primitive;
	// Frame 0's candidates [pixel][candidate] after the candidate kernel wrote
	// each training pixel's RIS weights w = p_hat / p into their pdf field.
	const ProposalCandidate* candidates;
	int candidate_count;
	uint32_t stride, phase;       // training pixels: i % stride == phase
	float inv_batch;              // 1 / number of training pixels
	// The shadowed part of the target (may be null): the frame's shaded
	// luminance per training pixel and its reservoir records (the chosen
	// light in .x), weighted by shadowed_weight against the unshadowed
	// candidate target.
	const float* shaded;
	const int4* records;
	float shadowed_weight;
	// Read by the tensor-core kernel only.
	const __nv_bfloat16* weights;  // BF16 weights in the operand layout
	uint32_t* error;               // the context's error word
	uint32_t skip_issue;           // fault injection: issue no tensor-core products
};

inline size_t mlp_train_smem_bytes(int k_count) {
	return sizeof(float) * kTrainPixels * (kFeatStride + 4 * kHiddenStride + train_logit_stride(k_count));
}

static __global__ void __launch_bounds__(kTrainThreads) mlp_train_kernel(MlpTrainParams pr) {
	extern __shared__ __align__(16) float train_smem[];
	const int k_count = pr.k_count;
	const MlpLayout lay = mlp_layout(k_count);
	const int ks = train_logit_stride(k_count);
	float* feat = train_smem;                          // [32][145]
	float* h1 = feat + kTrainPixels * kFeatStride;     // [32][65]
	float* h2 = h1 + kTrainPixels * kHiddenStride;     // [32][65]
	float* dz = h2 + kTrainPixels * kHiddenStride;     // [32][ks] logits, then their gradient
	float* d2 = dz + kTrainPixels * ks;                // [32][65]
	float* d1 = d2 + kTrainPixels * kHiddenStride;     // [32][65]
	const uint32_t np = pr.width * pr.height;
	const uint32_t n_train = np > pr.phase ? (np - pr.phase + pr.stride - 1) / pr.stride : 0;
	const int tid = threadIdx.x, px = tid % 32, warp = tid / 32;
	for (uint32_t base = blockIdx.x * kTrainPixels; base < n_train; base += gridDim.x * kTrainPixels) {
		// Encode the block's training pixels (invalid ones get zero weight).
		for (int idx = tid; idx < kTrainPixels * kMlpInputs; idx += kTrainThreads) {
			const int r = idx / kMlpInputs, input = idx % kMlpInputs;
			const uint32_t j = base + r, i = pr.phase + j * pr.stride;
			float e[13];
			mlp_encode(j < n_train ? mlp_input(pr.gbuffer, np, i, pr.center, pr.inv_half_extent, input) : 0.0f, e);
#pragma unroll
			for (int kind = 0; kind != 13; ++kind) feat[r * kFeatStride + input * 13 + kind] = j < n_train ? e[kind] : 0.0f;
		}
		for (int idx = tid; idx < kTrainPixels * (kMlpFeatures - kMlpInputs * 13); idx += kTrainThreads) {
			const int r = idx / (kMlpFeatures - kMlpInputs * 13), f = kMlpInputs * 13 + idx % (kMlpFeatures - kMlpInputs * 13);
			feat[r * kFeatStride + f] = 0.0f;
		}
		__syncthreads();
		// Forward: h1, h2 (ReLU), logits; lane = pixel, warps share the outputs.
		for (int o = warp; o < kMlpHidden; o += kTrainWarps) {
			float acc = pr.params[lay.b1 + o];
			const float* w = pr.params + lay.w1 + o * kMlpFeatures;
			for (int f = 0; f != kMlpFeatures; ++f) acc += w[f] * feat[px * kFeatStride + f];
			h1[px * kHiddenStride + o] = fmaxf(acc, 0.0f);
		}
		__syncthreads();
		for (int o = warp; o < kMlpHidden; o += kTrainWarps) {
			float acc = pr.params[lay.b2 + o];
			const float* w = pr.params + lay.w2 + o * kMlpHidden;
			for (int f = 0; f != kMlpHidden; ++f) acc += w[f] * h1[px * kHiddenStride + f];
			h2[px * kHiddenStride + o] = fmaxf(acc, 0.0f);
		}
		__syncthreads();
		for (int o = warp; o < k_count; o += kTrainWarps) {
			float acc = pr.params[lay.b3 + o];
			const float* w = pr.params + lay.w3 + o * kMlpHidden;
			for (int f = 0; f != kMlpHidden; ++f) acc += w[f] * h2[px * kHiddenStride + f];
			dz[px * ks + o] = acc;
		}
		__syncthreads();
		// Softmax and target per pixel: one warp per pixel.
		for (int r = tid / 32; r < kTrainPixels; r += kTrainThreads / 32) {
			const int lane = tid % 32;
			const uint32_t j = base + r, i = pr.phase + j * pr.stride;
			const bool valid = j < n_train && !(pr.primitive && pr.primitive[i] == 0xffffffffu);
			float* z = dz + r * ks;
			float m = -INFINITY;
			for (int c = lane; c < k_count; c += 32) m = fmaxf(m, z[c]);
			for (int d = 16; d != 0; d >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, d));
			float sum = 0.0f;
			for (int c = lane; c < k_count; c += 32) {
				const float e = __expf(z[c] - m);
				z[c] = e;
				sum += e;
			}
			for (int d = 16; d != 0; d >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, d);
			// Target: the candidates' weights summed per cluster.
			float total = 0.0f;
			if (valid)
				for (int c = lane; c < pr.candidate_count; c += 32) total += pr.candidates[(size_t) i * pr.candidate_count + c].pdf;
			for (int d = 16; d != 0; d >>= 1) total += __shfl_xor_sync(0xffffffffu, total, d);
			__syncwarp();
			const bool learn = valid && total > 0.0f && total <= 3.0e38f;
			const float inv_sum = 1.0f / sum;
			const float wu = pr.shaded ? 1.0f - pr.shadowed_weight : 1.0f;
			float ss = 0.0f;
			int chosen = -1;
			if (learn && pr.shaded) {
				chosen = pr.records[i].x;
				ss = chosen >= 0 ? pr.shaded[i] / (total / (float) pr.candidate_count) : 0.0f;
				ss = pr.shadowed_weight * fminf(fmaxf(ss, 0.0f), 4.0f);
			}
			for (int c = lane; c < k_count; c += 32) z[c] = learn ? (wu + ss) * z[c] * inv_sum * pr.inv_batch : 0.0f;
			__syncwarp();
			if (learn) {
				for (int c = lane; c < pr.candidate_count; c += 32) {
					const ProposalCandidate q = pr.candidates[(size_t) i * pr.candidate_count + c];
					if (q.pdf > 0.0f && (uint32_t) q.light < pr.light_count)
						atomicAdd(&z[pr.light_cluster[q.light]], -wu * q.pdf / total * pr.inv_batch);
				}
				if (lane == 0 && chosen >= 0 && (uint32_t) chosen < pr.light_count && ss > 0.0f)
					atomicAdd(&z[pr.light_cluster[chosen]], -ss * pr.inv_batch);
			}
			__syncwarp();
		}
		__syncthreads();
		// Backward: d2 = (W3^T dz) * [h2 > 0], d1 = (W2^T d2) * [h1 > 0];
		// lane = pixel, warps share the outputs.
		for (int f = warp; f < kMlpHidden; f += kTrainWarps) {
			float acc = 0.0f;
			for (int o = 0; o != k_count; ++o) acc += pr.params[lay.w3 + o * kMlpHidden + f] * dz[px * ks + o];
			d2[px * kHiddenStride + f] = h2[px * kHiddenStride + f] > 0.0f ? acc : 0.0f;
		}
		__syncthreads();
		for (int f = warp; f < kMlpHidden; f += kTrainWarps) {
			float acc = 0.0f;
			for (int o = 0; o != kMlpHidden; ++o) acc += pr.params[lay.w2 + o * kMlpHidden + f] * d2[px * kHiddenStride + o];
			d1[px * kHiddenStride + f] = h1[px * kHiddenStride + f] > 0.0f ? acc : 0.0f;
		}
		__syncthreads();
		// Weight gradients summed over the block's pixels, added once.
		for (int idx = tid; idx < k_count * (kMlpHidden + 1); idx += kTrainThreads) {
			const int o = idx / (kMlpHidden + 1), f = idx % (kMlpHidden + 1);
			float acc = 0.0f;
			for (int r = 0; r != kTrainPixels; ++r)
				acc += dz[r * ks + o] * (f < kMlpHidden ? h2[r * kHiddenStride + f] : 1.0f);
			if (acc != 0.0f) atomicAdd(pr.grad + (f < kMlpHidden ? lay.w3 + o * kMlpHidden + f : lay.b3 + o), acc);
		}
		for (int idx = tid; idx < kMlpHidden * (kMlpHidden + 1); idx += kTrainThreads) {
			const int o = idx / (kMlpHidden + 1), f = idx % (kMlpHidden + 1);
			float acc = 0.0f;
			for (int r = 0; r != kTrainPixels; ++r)
				acc += d2[r * kHiddenStride + o] * (f < kMlpHidden ? h1[r * kHiddenStride + f] : 1.0f);
			if (acc != 0.0f) atomicAdd(pr.grad + (f < kMlpHidden ? lay.w2 + o * kMlpHidden + f : lay.b2 + o), acc);
		}
		for (int idx = tid; idx < kMlpHidden * (kMlpFeatures + 1); idx += kTrainThreads) {
			const int o = idx / (kMlpFeatures + 1), f = idx % (kMlpFeatures + 1);
			float acc = 0.0f;
			for (int r = 0; r != kTrainPixels; ++r)
				acc += d1[r * kHiddenStride + o] * (f < kMlpFeatures ? feat[r * kFeatStride + f] : 1.0f);
			if (acc != 0.0f) atomicAdd(pr.grad + (f < kMlpFeatures ? lay.w1 + o * kMlpFeatures + f : lay.b1 + o), acc);
		}
		__syncthreads();
	}
}

// Adam (Kingma & Ba 2015) on the FP32 parameters; clears the gradient and
// refreshes the BF16 copy.  The padding features' weights stay zero.
static __global__ void mlp_adam_kernel(float* params, float* grad, float* m, float* v, __nv_bfloat16* weights, int count,
                                       int k_count, float learning_rate, float beta1, float beta2, float epsilon,
                                       float correction1, float correction2) {
	for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < count; j += gridDim.x * blockDim.x) {
		const float g = grad[j];
		const float mj = beta1 * m[j] + (1.0f - beta1) * g;
		const float vj = beta2 * v[j] + (1.0f - beta2) * g * g;
		m[j] = mj;
		v[j] = vj;
		const bool padding = mlp_padding_weight(j);
		float p = params[j];
		if (!padding) p -= learning_rate * (mj / correction1) / (sqrtf(vj / correction2) + epsilon);
		params[j] = p;
		const int slot = mlp_weight_slot(j, k_count);
		if (slot >= 0) weights[slot] = __float2bfloat16_rn(padding ? 0.0f : p);
		grad[j] = 0.0f;
	}
}

}  // namespace risltc
