// mlp_train_tc.cuh - online training of the proposal MLP on the tcgen05
// tensor cores (up to 256 clusters): forward pass, softmax cross-entropy
// gradient, the backward products and the weight gradients of a training
// step, with BF16 operands and FP32 accumulators.
//
// One CTA of four warps per SM takes tiles of 128 training pixels.  All
// operands live in shared memory in the K-major 8x8 core-matrix layout of
// the forward pass ([pixel][feature] for activations and gradients,
// [out][in] for weights).  The products that contract over the pixels (the
// weight gradients) and over a weight matrix's rows (the input gradients)
// read the same bytes through MN-major descriptors, so nothing is stored
// twice.  Per tile:
//   D1 = E W1^T, H1 = ReLU(D1 + b1); D2 = H1 W2^T, H2 = ReLU(D2 + b2);
//   logits in chunks of 128 clusters, BF16 into DZ, softmax per pixel;
//   DZ = (q - T) / B as in the CUDA-core kernel (each thread subtracts its
//   own pixel's target T from its row);
//   dh2 = DZ W3 and dW3 += DZ^T [H2 | 1]; DZ2 = dh2 * [H2 > 0];
//   dh1 = DZ2 W2 and dW2 += DZ2^T [H1 | 1]; DZ1 = dh1 * [H1 > 0];
//   dW1 += DZ1^T E (feature 130 of E is 1, so its column is db1).
// The weight gradients accumulate in tensor memory over all tiles of the
// CTA and are added to the FP32 gradient vector once at the end.  Tensor
// memory (512 columns): 0..127 the per-tile products, 128..287 dW3 (80
// columns per 128-cluster chunk: 64 weights, the bias, 15 zeros), 288..367
// dW2, 368..511 dW1.  The hidden layers' M = 64 weight-gradient products run
// at M = 128; their upper 64 rows read the following bytes of shared memory
// and are discarded.
#pragma once
#include "mlp_tc.cuh"

namespace risltc {

constexpr int kTtMaxClusters = 256;
constexpr int kTtHiddenCols = 80;                    // stored hidden columns: 64 values, 1.0, 15 zeros
constexpr int kTtOnesFeature = kMlpInputs * 13;     // feature 130 (a padding feature, zero weight)
constexpr uint32_t kTtColumns = 512;
constexpr uint32_t kTtGrad3 = 128, kTtGrad2 = 288, kTtGrad1 = 368;
// Shared memory (bytes).
constexpr uint32_t kTtW1 = 0;
constexpr uint32_t kTtW2 = kTtW1 + kMlpHidden * kMlpFeatures * 2;
constexpr uint32_t kTtW3 = kTtW2 + kMlpHidden * kMlpHidden * 2;
constexpr uint32_t kTtE = kTtW3 + kTtMaxClusters * kMlpHidden * 2;
constexpr uint32_t kTtH1 = kTtE + kTcRows * kMlpFeatures * 2;
constexpr uint32_t kTtH2 = kTtH1 + kTcRows * kTtHiddenCols * 2;
constexpr uint32_t kTtDz = kTtH2 + kTcRows * kTtHiddenCols * 2;
constexpr uint32_t kTtD = kTtDz + kTcRows * kTtMaxClusters * 2;  // DZ2, then DZ1
constexpr uint32_t kTtBias = kTtD + kTcRows * kMlpHidden * 2;    // b1, b2, b3 (FP32)
constexpr uint32_t kTtBar = kTtBias + (2 * kMlpHidden + kTtMaxClusters) * 4;
constexpr uint32_t kTtSlot = kTtBar + 16;
constexpr uint32_t kTtSmemBytes = kTtSlot + 8;
// The M = 128 reads of DZ2/DZ1 reach 1 KB past their buffer (into the biases).
static_assert(kTtBias - kTtD + (2 * kMlpHidden + kTtMaxClusters) * 4 >= 14 * 1024 + 16 * 128 + 1024 + 128,
              "the discarded rows of the hidden weight-gradient products stay in shared memory");
static_assert(kTtSmemBytes <= 232448, "fits one CTA per SM");

// Shared-memory descriptor (no swizzle, version 1): `leading` is the byte
// distance between core matrices along K, `stride` along M or N, for both
// K-major and MN-major operands.
RL_DEV uint64_t tc_descriptor_mn(uint32_t addr, uint32_t leading, uint32_t stride) {
	return (uint64_t) ((addr & 0x3FFFFu) >> 4) | ((uint64_t) (leading >> 4) << 16) | ((uint64_t) (stride >> 4) << 32) |
	       (1ull << 46);
}
constexpr uint32_t kTcAMajorMN = 1u << 15, kTcBMajorMN = 1u << 16;

// 16 consecutive FP32 columns of this thread's tensor-memory lane.
RL_DEV void tc_load16(uint32_t taddr, uint32_t (&v)[16]) {
	asm volatile(
	    "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15}, [%16];\n"
	    : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]), "=r"(v[8]),
	      "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15])
	    : "r"(taddr));
}

RL_DEV float bf16_lo(uint32_t w) { return __uint_as_float(w << 16); }
RL_DEV float bf16_hi(uint32_t w) { return __uint_as_float(w & 0xFFFF0000u); }

static __global__ void __launch_bounds__(kTcThreads, 1) mlp_train_tc_kernel(MlpTrainParams pr) {
	extern __shared__ __align__(1024) unsigned char tt_smem[];
	const int k_count = pr.k_count;
	const int k_pad = mlp_padded_clusters(k_count);
	const int chunks = (k_pad + kTcChunk - 1) / kTcChunk;
	const uint32_t dz_rows = (uint32_t) (k_pad / 8) * 128;  // DZ: bytes between 8-pixel groups
	const MlpLayout lay = mlp_layout(k_count);
	const uint32_t tid = threadIdx.x, warp = tid / 32;
	const uint32_t base = smem_address(tt_smem);
	float* b1 = reinterpret_cast<float*>(tt_smem + kTtBias);
	float* b2 = b1 + kMlpHidden;
	float* b3 = b2 + kMlpHidden;
	for (int j = tid; j < kMlpHidden; j += kTcThreads) {
		b1[j] = pr.params[lay.b1 + j];
		b2[j] = pr.params[lay.b2 + j];
	}
	for (int j = tid; j < kTtMaxClusters; j += kTcThreads) b3[j] = j < k_count ? pr.params[lay.b3 + j] : 0.0f;
	// Columns 64..79 of H1 and H2: 1.0 then zeros (never overwritten).
	for (int idx = tid; idx < kTcRows * 16; idx += kTcThreads) {
		const int r = idx / 16, c = kMlpHidden + idx % 16;
		const __nv_bfloat16 v = __float2bfloat16_rn(c == kMlpHidden ? 1.0f : 0.0f);
		*reinterpret_cast<__nv_bfloat16*>(tt_smem + kTtH1 + tc_offset(r, c, kTtHiddenCols)) = v;
		*reinterpret_cast<__nv_bfloat16*>(tt_smem + kTtH2 + tc_offset(r, c, kTtHiddenCols)) = v;
	}
	const uint32_t bar = base + kTtBar, bar_weights = bar + 8;
	if (tid == 0) {
		for (int k = 0; k != 2; ++k) asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(bar + 8 * k) : "memory");
		asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
		const uint32_t bytes = (uint32_t) mlp_weight_elements(k_count) * 2;
		mbarrier_expect_bytes(bar_weights, bytes);
		bulk_copy_to_shared(base + kTtW1, pr.weights, bytes, bar_weights);
	}
	if (warp == 0) {
		asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(base + kTtSlot),
		             "r"(kTtColumns)
		             : "memory");
		asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
	}
	fence_async_shared();
	tc_fence_before();
	__syncthreads();
	tc_fence_after();
	const uint32_t tmem = *reinterpret_cast<volatile uint32_t*>(tt_smem + kTtSlot);
	const uint32_t lane_base = (warp * 32) << 16;
	const uint32_t np = pr.width * pr.height;
	const uint32_t n_train = np > pr.phase ? (np - pr.phase + pr.stride - 1) / pr.stride : 0;
	const uint32_t tiles = (n_train + kTcRows - 1) / kTcRows;
	const int mc = pr.candidate_count;
	uint32_t parity = 0;
	bool product_pending = false;
	const bool weights_ok = __syncthreads_or(!tc_wait(bar_weights, 0)) == 0;
	bool failed = !weights_ok;
	auto issue = [&](auto products) {
		if (tid == 0 && !pr.skip_issue) {
			products();
			tc_commit(bar);
		}
	};
	auto await_products = [&] {
		const bool ok = tc_wait(bar, parity);
		parity ^= 1u;
		failed = __syncthreads_or(!ok) != 0;
		product_pending = failed && !pr.skip_issue;
		tc_fence_after();
	};
	auto sync_for_products = [&] {
		fence_async_shared();
		tc_fence_before();
		__syncthreads();
		tc_fence_after();
	};
	// Row tid of the 64 transient columns + bias, ReLU, BF16 into H.
	auto hidden_epilogue = [&](uint32_t h, const float* bias) {
		for (int c = 0; c != kMlpHidden; c += 32) {
			uint32_t v[32];
			tc_load32(tmem + lane_base + (uint32_t) c, v);
			tc_wait_load();
#pragma unroll
			for (int q = 0; q != 4; ++q) {
				uint4 out;
				uint32_t* o = &out.x;
#pragma unroll
				for (int k = 0; k != 4; ++k) {
					const int j = 8 * q + 2 * k;
					o[k] = pack_bf16x2(fmaxf(__uint_as_float(v[j]) + bias[c + j], 0.0f),
					                   fmaxf(__uint_as_float(v[j + 1]) + bias[c + j + 1], 0.0f));
				}
				*reinterpret_cast<uint4*>(tt_smem + h + tc_offset((int) tid, c + 8 * q, kTtHiddenCols)) = out;
			}
		}
		sync_for_products();
	};
	// Row tid of the 64 transient columns where H > 0, else 0, BF16 into the
	// DZ2/DZ1 buffer.
	auto gradient_epilogue = [&](uint32_t h) {
		for (int c = 0; c != kMlpHidden; c += 32) {
			uint32_t v[32];
			tc_load32(tmem + lane_base + (uint32_t) c, v);
			tc_wait_load();
#pragma unroll
			for (int q = 0; q != 4; ++q) {
				const uint4 act = *reinterpret_cast<const uint4*>(tt_smem + h + tc_offset((int) tid, c + 8 * q, kTtHiddenCols));
				const uint32_t* a = &act.x;
				uint4 out;
				uint32_t* o = &out.x;
#pragma unroll
				for (int k = 0; k != 4; ++k) {
					const int j = 8 * q + 2 * k;
					o[k] = pack_bf16x2(bf16_lo(a[k]) > 0.0f ? __uint_as_float(v[j]) : 0.0f,
					                   bf16_hi(a[k]) > 0.0f ? __uint_as_float(v[j + 1]) : 0.0f);
				}
				*reinterpret_cast<uint4*>(tt_smem + kTtD + tc_offset((int) tid, c + 8 * q, kMlpHidden)) = out;
			}
		}
		sync_for_products();
	};
	bool accumulated = false;  // the weight gradients in tensor memory hold at least one tile
	for (uint32_t tile = blockIdx.x; tile < tiles && !failed; tile += gridDim.x) {
		const uint32_t j0 = tile * kTcRows;
		// Thread tid takes the tile's row tid: training pixel j0 + tid.  Its
		// inputs are loaded together, then encoded into E (feature 130 is 1.0).
		const uint32_t my_j = j0 + tid, my_i = pr.phase + my_j * pr.stride;
		const bool in = my_j < n_train;
		{
			float x[kMlpInputs];
#pragma unroll
			for (int input = 0; input != kMlpInputs; ++input)
				x[input] = in ? mlp_input(pr.gbuffer, np, my_i, pr.center, pr.inv_half_extent, input) : 0.0f;
#pragma unroll
			for (int input = 0; input != kMlpInputs; ++input) {
				float e[13];
				mlp_encode(x[input], e);
#pragma unroll
				for (int kind = 0; kind != 13; ++kind)
					*reinterpret_cast<__nv_bfloat16*>(tt_smem + kTtE + tc_offset((int) tid, input * 13 + kind, kMlpFeatures)) =
					    __float2bfloat16_rn(in ? e[kind] : 0.0f);
			}
#pragma unroll
			for (int f = kTtOnesFeature; f != kMlpFeatures; ++f)
				*reinterpret_cast<__nv_bfloat16*>(tt_smem + kTtE + tc_offset((int) tid, f, kMlpFeatures)) =
				    __float2bfloat16_rn(f == kTtOnesFeature ? 1.0f : 0.0f);
		}
		sync_for_products();
		issue([&] {
			for (int k = 0; k != kMlpFeatures / 16; ++k)
				tc_mma(tmem, tc_descriptor(base + kTtE + 256 * k, kMlpFeatures),
				       tc_descriptor(base + kTtW1 + 256 * k, kMlpFeatures), tc_instruction(kTcRows, kMlpHidden), k > 0);
		});
		// While layer 1 runs: the total candidate weight of this thread's pixel.
		const ProposalCandidate* cand = pr.candidates + (size_t) my_i * mc;
		const bool valid = in && !(pr.primitive && pr.primitive[my_i] == 0xffffffffu);
		float total = 0.0f;
		if (valid) {
#pragma unroll 8
			for (int c = 0; c < mc; ++c) total += cand[c].pdf;
		}
		const bool learn = valid && total > 0.0f && total <= 3.0e38f;
		const float wu = pr.shaded ? 1.0f - pr.shadowed_weight : 1.0f;
		float ss = 0.0f;
		int chosen = -1;
		if (learn && pr.shaded) {
			chosen = pr.records[my_i].x;
			ss = chosen >= 0 ? pr.shaded[my_i] / (total / (float) mc) : 0.0f;
			ss = pr.shadowed_weight * fminf(fmaxf(ss, 0.0f), 4.0f);
		}
		const float coef = learn ? (wu + ss) * pr.inv_batch : 0.0f;
		await_products();
		if (failed) break;
		hidden_epilogue(kTtH1, b1);
		issue([&] {
			for (int k = 0; k != kMlpHidden / 16; ++k)
				tc_mma(tmem, tc_descriptor(base + kTtH1 + 256 * k, kTtHiddenCols),
				       tc_descriptor(base + kTtW2 + 256 * k, kMlpHidden), tc_instruction(kTcRows, kMlpHidden), k > 0);
		});
		await_products();
		if (failed) break;
		hidden_epilogue(kTtH2, b2);
		// Logits, 128 clusters per product, BF16 into DZ; the row maximum.
		float zmax = -INFINITY;
		for (int ch = 0; ch != chunks && !failed; ++ch) {
			const int c0 = ch * kTcChunk, n = min(kTcChunk, k_pad - c0);
			issue([&] {
				for (int k = 0; k != kMlpHidden / 16; ++k)
					tc_mma(tmem, tc_descriptor(base + kTtH2 + 256 * k, kTtHiddenCols),
					       tc_descriptor(base + kTtW3 + (uint32_t) c0 * 128 + 256 * k, kMlpHidden),
					       tc_instruction(kTcRows, n), k > 0);
			});
			await_products();
			if (failed) break;
			for (int c = 0; c < n; c += 32) {
				uint32_t v[32];
				tc_load32(tmem + lane_base + (uint32_t) c, v);
				tc_wait_load();
#pragma unroll
				for (int q = 0; q != 4; ++q) {
					if (c + 8 * q >= n) continue;
					uint4 out;
					uint32_t* o = &out.x;
#pragma unroll
					for (int k = 0; k != 4; ++k) {
						const int j = 8 * q + 2 * k, col = c0 + c + j;
						const float lo = col < k_count ? __uint_as_float(v[j]) + b3[col] : 0.0f;
						const float hi = col + 1 < k_count ? __uint_as_float(v[j + 1]) + b3[col + 1] : 0.0f;
						o[k] = pack_bf16x2(lo, hi);
						if (col < k_count) zmax = fmaxf(zmax, bf16_lo(o[k]));
						if (col + 1 < k_count) zmax = fmaxf(zmax, bf16_hi(o[k]));
					}
					*reinterpret_cast<uint4*>(tt_smem + kTtDz + tc_offset((int) tid, c0 + c + 8 * q, k_pad)) = out;
				}
			}
			tc_fence_before();
			__syncthreads();
			tc_fence_after();
		}
		if (failed) break;
		// DZ = coef softmax(z) on this thread's row (zero for padding clusters).
		float sum = 0.0f;
		for (int c = 0; c < k_count; c += 8) {
			const uint4 u = *reinterpret_cast<const uint4*>(tt_smem + kTtDz + tc_offset((int) tid, c, k_pad));
			const uint32_t* w = &u.x;
#pragma unroll
			for (int k = 0; k != 4; ++k) sum += __expf(bf16_lo(w[k]) - zmax) + __expf(bf16_hi(w[k]) - zmax);
		}
		const float scale = coef / sum;
		for (int c = 0; c < k_count; c += 8) {
			uint4* p = reinterpret_cast<uint4*>(tt_smem + kTtDz + tc_offset((int) tid, c, k_pad));
			const uint4 u = *p;
			const uint32_t* w = &u.x;
			uint4 out;
			uint32_t* o = &out.x;
#pragma unroll
			for (int k = 0; k != 4; ++k)
				o[k] = pack_bf16x2(scale * __expf(bf16_lo(w[k]) - zmax), scale * __expf(bf16_hi(w[k]) - zmax));
			*p = out;
		}
		// Minus the target, on this thread's own row: the candidates' weights
		// into their clusters, the shadowed part into the chosen light's.
		if (learn) {
			const float unshadowed = wu / total * pr.inv_batch;
#pragma unroll 8
			for (int c = 0; c < mc; ++c) {
				const ProposalCandidate q = cand[c];
				if (q.pdf > 0.0f && (uint32_t) q.light < pr.light_count) {
					__nv_bfloat16* z = reinterpret_cast<__nv_bfloat16*>(
					    tt_smem + kTtDz + tc_offset((int) tid, (int) pr.light_cluster[q.light], k_pad));
					*z = __float2bfloat16_rn(__bfloat162float(*z) - unshadowed * q.pdf);
				}
			}
			if (chosen >= 0 && (uint32_t) chosen < pr.light_count && ss > 0.0f) {
				__nv_bfloat16* z = reinterpret_cast<__nv_bfloat16*>(
				    tt_smem + kTtDz + tc_offset((int) tid, (int) pr.light_cluster[chosen], k_pad));
				*z = __float2bfloat16_rn(__bfloat162float(*z) - ss * pr.inv_batch);
			}
		}
		sync_for_products();
		// dh2 = DZ W3 (W3 read MN-major: N = hidden, K = clusters) and
		// dW3 += DZ^T [H2 | 1] (both MN-major, K = pixels).
		issue([&] {
			for (int k = 0; k != k_pad / 16; ++k)
				tc_mma(tmem, tc_descriptor(base + kTtDz + 256 * k, k_pad),
				       tc_descriptor_mn(base + kTtW3 + 2048 * k, 1024, 128), tc_instruction(kTcRows, kMlpHidden) | kTcBMajorMN,
				       k > 0);
			for (int ch = 0; ch != chunks; ++ch)
				for (int k = 0; k != kTcRows / 16; ++k)
					tc_mma(tmem + kTtGrad3 + 80 * ch,
					       tc_descriptor_mn(base + kTtDz + 2048 * ch + 2 * dz_rows * k, dz_rows, 128),
					       tc_descriptor_mn(base + kTtH2 + 2 * 1280 * k, 1280, 128),
					       tc_instruction(kTcRows, kTtHiddenCols) | kTcAMajorMN | kTcBMajorMN, accumulated || k > 0);
		});
		await_products();
		if (failed) break;
		gradient_epilogue(kTtH2);
		// dh1 = DZ2 W2 (W2 MN-major) and dW2 += DZ2^T [H1 | 1].
		issue([&] {
			for (int k = 0; k != kMlpHidden / 16; ++k)
				tc_mma(tmem, tc_descriptor(base + kTtD + 256 * k, kMlpHidden),
				       tc_descriptor_mn(base + kTtW2 + 2048 * k, 1024, 128), tc_instruction(kTcRows, kMlpHidden) | kTcBMajorMN,
				       k > 0);
			for (int k = 0; k != kTcRows / 16; ++k)
				tc_mma(tmem + kTtGrad2, tc_descriptor_mn(base + kTtD + 2048 * k, 1024, 128),
				       tc_descriptor_mn(base + kTtH1 + 2 * 1280 * k, 1280, 128),
				       tc_instruction(kTcRows, kTtHiddenCols) | kTcAMajorMN | kTcBMajorMN, accumulated || k > 0);
		});
		await_products();
		if (failed) break;
		gradient_epilogue(kTtH1);  // DZ1 replaces DZ2 (its products are done)
		// dW1 += DZ1^T E.
		issue([&] {
			for (int k = 0; k != kTcRows / 16; ++k)
				tc_mma(tmem + kTtGrad1, tc_descriptor_mn(base + kTtD + 2048 * k, 1024, 128),
				       tc_descriptor_mn(base + kTtE + 2 * 2304 * k, 2304, 128),
				       tc_instruction(kTcRows, kMlpFeatures) | kTcAMajorMN | kTcBMajorMN, accumulated || k > 0);
		});
		await_products();
		accumulated = true;
	}
	if (!failed && accumulated) {
		// Lane tid of each accumulator: cluster (dW3) or hidden unit (dW2, dW1).
		for (int ch = 0; ch != chunks; ++ch) {
			const int c = ch * kTcChunk + (int) tid;
			for (int col = 0; col != kTtHiddenCols; col += 16) {
				uint32_t v[16];
				tc_load16(tmem + lane_base + kTtGrad3 + 80 * ch + (uint32_t) col, v);
				tc_wait_load();
				if (c >= k_count) continue;
#pragma unroll
				for (int q = 0; q != 16; ++q) {
					const float g = __uint_as_float(v[q]);
					const int f = col + q;
					if (g == 0.0f || f > kMlpHidden) continue;
					atomicAdd(pr.grad + (f < kMlpHidden ? lay.w3 + c * kMlpHidden + f : lay.b3 + c), g);
				}
			}
		}
		for (int col = 0; col != kTtHiddenCols; col += 16) {
			uint32_t v[16];
			tc_load16(tmem + lane_base + kTtGrad2 + (uint32_t) col, v);
			tc_wait_load();
			if (tid >= (uint32_t) kMlpHidden) continue;
#pragma unroll
			for (int q = 0; q != 16; ++q) {
				const float g = __uint_as_float(v[q]);
				const int f = col + q;
				if (g == 0.0f || f > kMlpHidden) continue;
				atomicAdd(pr.grad + (f < kMlpHidden ? lay.w2 + (int) tid * kMlpHidden + f : lay.b2 + (int) tid), g);
			}
		}
		for (int col = 0; col != kMlpFeatures; col += 16) {
			uint32_t v[16];
			tc_load16(tmem + lane_base + kTtGrad1 + (uint32_t) col, v);
			tc_wait_load();
			if (tid >= (uint32_t) kMlpHidden) continue;
#pragma unroll
			for (int q = 0; q != 16; ++q) {
				const float g = __uint_as_float(v[q]);
				const int f = col + q;
				if (g == 0.0f || f > kTtOnesFeature) continue;
				atomicAdd(pr.grad + (f < kTtOnesFeature ? lay.w1 + (int) tid * kMlpFeatures + f : lay.b1 + (int) tid), g);
			}
		}
	}
	if (failed) {
		if (tid == 0) atomicOr(pr.error, kErrorTensorWait);
		if (product_pending) tc_wait(bar, parity ^ 1u);
		if (!weights_ok) tc_wait(bar_weights, 0);
	}
	tc_fence_before();
	__syncthreads();
	if (warp == 0) {
		tc_fence_after();
		asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(kTtColumns) : "memory");
	}
}

}  // namespace risltc
