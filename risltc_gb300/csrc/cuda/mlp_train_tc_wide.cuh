// mlp_train_tc_wide.cuh - online training of the proposal MLP on the tcgen05
// tensor cores for models of more than 256 clusters (up to 1024): the same
// training step as mlp_train_tc_kernel (forward pass, softmax cross-entropy
// gradient, backward products, weight gradients; BF16 operands, FP32
// accumulators), with the output layer taken in chunks of 128 clusters so
// that neither its weights nor its logits have to fit on chip at once.
//
// One CTA of four warps per SM takes tiles of 128 training pixels.  W1 and W2
// arrive in one bulk copy; W3 streams by chunk (16 KB each) into two shared
// buffers by bulk copies issued one chunk ahead.  Per tile:
//   D1 = E W1^T, H1 = ReLU(D1 + b1); D2 = H1 W2^T, H2 = ReLU(D2 + b2);
//   pass A, per chunk: its logits (BF16, as in inference) and the running
//     maximum and sum of exp(z - max) of each pixel's row (online softmax);
//   pass B, per chunk: its logits again, DZ_c = coef exp(z - max) / sum in
//     BF16 minus the pixel's targets in this chunk (each subtraction rounded
//     to BF16, in candidate order, as in mlp_train_tc_kernel), then
//     dh2 += DZ_c W3_c (accumulated over the chunks in tensor memory) and
//     dW3_c = DZ_c^T [H2 | 1], added to the FP32 gradient with vector
//     atomics (the chunks' weight gradients do not fit in tensor memory);
//   DZ2 = dh2 * [H2 > 0]; dh1 = DZ2 W2 and dW2 += DZ2^T [H1 | 1];
//   DZ1 = dh1 * [H1 > 0]; dW1 += DZ1^T E (feature 130 of E is 1: db1).
// dW2 and dW1 accumulate in tensor memory over the CTA's tiles and are added
// once at the end.  Tensor memory (512 columns): 0..127 the per-tile
// products, 128..191 dh2, 192..271 dW3 of the current chunk, 272..351 dW2,
// 352..495 dW1.  Every wait is bounded (kTcWaitNs); on a timeout the kernel
// records kErrorTensorWait, waits (bounded) for its products and copies in
// flight, frees its tensor memory and returns.
#pragma once
#include "mlp_train_tc.cuh"

namespace risltc {

constexpr int kTwMaxClusters = 1024;
constexpr uint32_t kTwChunkBytes = kTcChunk * kMlpHidden * 2;  // one W3 chunk: 16 KB
constexpr uint32_t kTwDh2 = 128, kTwGrad3 = 192, kTwGrad2 = 272, kTwGrad1 = 352;
// Shared memory (bytes).
constexpr uint32_t kTwW1 = 0;
constexpr uint32_t kTwW2 = kTwW1 + kMlpHidden * kMlpFeatures * 2;
constexpr uint32_t kTwW3 = kTwW2 + kMlpHidden * kMlpHidden * 2;  // two chunk buffers
constexpr uint32_t kTwE = kTwW3 + 2 * kTwChunkBytes;
constexpr uint32_t kTwH1 = kTwE + kTcRows * kMlpFeatures * 2;
constexpr uint32_t kTwH2 = kTwH1 + kTcRows * kTtHiddenCols * 2;
constexpr uint32_t kTwDz = kTwH2 + kTcRows * kTtHiddenCols * 2;   // one chunk: 128 pixels x 128 clusters
constexpr uint32_t kTwD = kTwDz + kTcRows * kTcChunk * 2;         // DZ2, then DZ1
constexpr uint32_t kTwBias = kTwD + kTcRows * kMlpHidden * 2;     // b1, b2, b3 (FP32)
constexpr uint32_t kTwBar = kTwBias + (2 * kMlpHidden + kTwMaxClusters) * 4;  // products, W1W2, W3 buffers 0 and 1
constexpr uint32_t kTwSlot = kTwBar + 32;
constexpr uint32_t kTwSmemBytes = kTwSlot + 8;
// The M = 128 reads of DZ2 / DZ1 (MN-major, 64 real rows) reach past their
// buffer into the biases, as in mlp_train_tc_kernel.
static_assert(kTwBar - kTwD >= 14 * 1024 + 16 * 128 + 1024 + 128, "discarded rows stay in shared memory");
static_assert(kTwW3 % 1024 == 0 && kTwE % 1024 == 0 && kTwH1 % 1024 == 0 && kTwH2 % 1024 == 0 &&
                  kTwDz % 1024 == 0 && kTwD % 1024 == 0,
              "operand buffers 1 KB aligned");
static_assert(kTwSmemBytes <= 232448, "fits one CTA per SM");

static __global__ void __launch_bounds__(kTcThreads, 1) mlp_train_tc_wide_kernel(MlpTrainParams pr) {
	extern __shared__ __align__(1024) unsigned char tw_smem[];
	const int k_count = pr.k_count;
	const int k_pad = mlp_padded_clusters(k_count);
	const int chunks = (k_pad + kTcChunk - 1) / kTcChunk;
	const MlpLayout lay = mlp_layout(k_count);
	const uint32_t tid = threadIdx.x, warp = tid / 32;
	const uint32_t base = smem_address(tw_smem);
	float* b1 = reinterpret_cast<float*>(tw_smem + kTwBias);
	float* b2 = b1 + kMlpHidden;
	float* b3 = b2 + kMlpHidden;
	for (int j = tid; j < kMlpHidden; j += kTcThreads) {
		b1[j] = pr.params[lay.b1 + j];
		b2[j] = pr.params[lay.b2 + j];
	}
	for (int j = tid; j < kTwMaxClusters; j += kTcThreads) b3[j] = j < k_count ? pr.params[lay.b3 + j] : 0.0f;
	// Columns 64..79 of H1 and H2: 1.0 then zeros (never overwritten).
	for (int idx = tid; idx < kTcRows * 16; idx += kTcThreads) {
		const int r = idx / 16, c = kMlpHidden + idx % 16;
		const __nv_bfloat16 v = __float2bfloat16_rn(c == kMlpHidden ? 1.0f : 0.0f);
		*reinterpret_cast<__nv_bfloat16*>(tw_smem + kTwH1 + tc_offset(r, c, kTtHiddenCols)) = v;
		*reinterpret_cast<__nv_bfloat16*>(tw_smem + kTwH2 + tc_offset(r, c, kTtHiddenCols)) = v;
	}
	const uint32_t bar = base + kTwBar, bar_weights = bar + 8, bar_w3 = bar + 16;  // bar_w3 + 8 b: buffer b
	const char* w3_global = reinterpret_cast<const char*>(pr.weights) + kTwW3;  // W3 follows W1 and W2
	if (tid == 0) {
		for (int k = 0; k != 4; ++k) asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(bar + 8 * k) : "memory");
		asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
		mbarrier_expect_bytes(bar_weights, kTwW3);
		bulk_copy_to_shared(base + kTwW1, pr.weights, kTwW3, bar_weights);
	}
	if (warp == 0) {
		asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(base + kTwSlot),
		             "r"(kTtColumns)
		             : "memory");
		asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
	}
	fence_async_shared();
	tc_fence_before();
	__syncthreads();
	tc_fence_after();
	const uint32_t tmem = *reinterpret_cast<volatile uint32_t*>(tw_smem + kTwSlot);
	const uint32_t lane_base = (warp * 32) << 16;
	const uint32_t np = pr.width * pr.height;
	const uint32_t n_train = np > pr.phase ? (np - pr.phase + pr.stride - 1) / pr.stride : 0;
	const uint32_t tiles = (n_train + kTcRows - 1) / kTcRows;
	const int mc = pr.candidate_count;
	uint32_t parity = 0;
	bool product_pending = false;
	bool failed = __syncthreads_or(!tc_wait(bar_weights, 0)) != 0;
	const bool weights_ok = !failed;
	// W3 chunk copies: the seq-th copy of the CTA goes to buffer seq & 1 and
	// completes phase (seq >> 1) & 1 of that buffer's mbarrier.
	uint32_t copies_issued = 0, copies_waited = 0;
	auto copy_chunk = [&](int c) {
		if (tid == 0) {
			const uint32_t b = copies_issued & 1u;
			const uint32_t bytes = (uint32_t) min(kTcChunk, k_pad - c * kTcChunk) * kMlpHidden * 2;
			mbarrier_expect_bytes(bar_w3 + 8 * b, bytes);
			bulk_copy_to_shared(base + kTwW3 + b * kTwChunkBytes, w3_global + (size_t) c * kTwChunkBytes, bytes,
			                    bar_w3 + 8 * b);
		}
		++copies_issued;
	};
	// Waits for the oldest copy not yet waited for; returns its buffer's
	// shared address.
	auto await_chunk = [&]() -> uint32_t {
		const uint32_t b = copies_waited & 1u, ph = (copies_waited >> 1) & 1u;
		const bool ok = tc_wait(bar_w3 + 8 * b, ph);
		++copies_waited;
		failed = __syncthreads_or(!ok) != 0;
		return base + kTwW3 + b * kTwChunkBytes;
	};
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
				*reinterpret_cast<uint4*>(tw_smem + h + tc_offset((int) tid, c + 8 * q, kTtHiddenCols)) = out;
			}
		}
		sync_for_products();
	};
	// Row tid of the 64 columns at `col` where H > 0, else 0, BF16 into D.
	auto gradient_epilogue = [&](uint32_t col, uint32_t h) {
		for (int c = 0; c != kMlpHidden; c += 32) {
			uint32_t v[32];
			tc_load32(tmem + lane_base + col + (uint32_t) c, v);
			tc_wait_load();
#pragma unroll
			for (int q = 0; q != 4; ++q) {
				const uint4 act = *reinterpret_cast<const uint4*>(tw_smem + h + tc_offset((int) tid, c + 8 * q, kTtHiddenCols));
				const uint32_t* a = &act.x;
				uint4 out;
				uint32_t* o = &out.x;
#pragma unroll
				for (int k = 0; k != 4; ++k) {
					const int j = 8 * q + 2 * k;
					o[k] = pack_bf16x2(bf16_lo(a[k]) > 0.0f ? __uint_as_float(v[j]) : 0.0f,
					                   bf16_hi(a[k]) > 0.0f ? __uint_as_float(v[j + 1]) : 0.0f);
				}
				*reinterpret_cast<uint4*>(tw_smem + kTwD + tc_offset((int) tid, c + 8 * q, kMlpHidden)) = out;
			}
		}
		sync_for_products();
	};
	// Logits of chunk c (n clusters) into tensor-memory columns 0..n-1.
	auto logits_product = [&](uint32_t w3, int n) {
		issue([&] {
			for (int k = 0; k != kMlpHidden / 16; ++k)
				tc_mma(tmem, tc_descriptor(base + kTwH2 + 256 * k, kTtHiddenCols), tc_descriptor(w3 + 256 * k, kMlpHidden),
				       tc_instruction(kTcRows, n), k > 0);
		});
	};
	bool accumulated = false;  // dW2 and dW1 in tensor memory hold at least one tile
	for (uint32_t tile = blockIdx.x; tile < tiles && !failed; tile += gridDim.x) {
		const uint32_t j0 = tile * kTcRows;
		const uint32_t my_j = j0 + tid, my_i = pr.phase + my_j * pr.stride;
		const bool in = my_j < n_train;
		copy_chunk(0);  // the tile's first W3 chunk, during layers 1 and 2
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
					*reinterpret_cast<__nv_bfloat16*>(tw_smem + kTwE + tc_offset((int) tid, input * 13 + kind, kMlpFeatures)) =
					    __float2bfloat16_rn(in ? e[kind] : 0.0f);
			}
#pragma unroll
			for (int f = kTtOnesFeature; f != kMlpFeatures; ++f)
				*reinterpret_cast<__nv_bfloat16*>(tw_smem + kTwE + tc_offset((int) tid, f, kMlpFeatures)) =
				    __float2bfloat16_rn(f == kTtOnesFeature ? 1.0f : 0.0f);
		}
		sync_for_products();
		issue([&] {
			for (int k = 0; k != kMlpFeatures / 16; ++k)
				tc_mma(tmem, tc_descriptor(base + kTwE + 256 * k, kMlpFeatures),
				       tc_descriptor(base + kTwW1 + 256 * k, kMlpFeatures), tc_instruction(kTcRows, kMlpHidden), k > 0);
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
		hidden_epilogue(kTwH1, b1);
		issue([&] {
			for (int k = 0; k != kMlpHidden / 16; ++k)
				tc_mma(tmem, tc_descriptor(base + kTwH1 + 256 * k, kTtHiddenCols),
				       tc_descriptor(base + kTwW2 + 256 * k, kMlpHidden), tc_instruction(kTcRows, kMlpHidden), k > 0);
		});
		await_products();
		if (failed) break;
		hidden_epilogue(kTwH2, b2);
		// Pass A: each row's maximum logit m and sum of exp(z - m).
		float zmax = -INFINITY, zsum = 0.0f;
		for (int u = 0; u != 2 * chunks && !failed; ++u) {
			const int ch = u % chunks, c0 = ch * kTcChunk, n = min(kTcChunk, k_pad - c0);
			const bool pass_b = u >= chunks;
			const uint32_t w3 = await_chunk();
			if (failed) break;
			if (u + 1 < 2 * chunks) copy_chunk((u + 1) % chunks);
			logits_product(w3, n);
			await_products();
			if (failed) break;
			if (!pass_b) {
				float cmax = -INFINITY;
				for (int c = 0; c < n; c += 32) {
					uint32_t v[32];
					tc_load32(tmem + lane_base + (uint32_t) c, v);
					tc_wait_load();
#pragma unroll
					for (int j = 0; j != 32; ++j) {
						const int col = c0 + c + j;
						if (c + j < n && col < k_count) {
							const float zj = __bfloat162float(__float2bfloat16_rn(__uint_as_float(v[j]) + b3[col]));
							cmax = fmaxf(cmax, zj);
						}
					}
				}
				const float m = fmaxf(zmax, cmax);
				float s = zsum * __expf(zmax - m);
				if (zmax == -INFINITY) s = 0.0f;
				for (int c = 0; c < n; c += 32) {
					uint32_t v[32];
					tc_load32(tmem + lane_base + (uint32_t) c, v);
					tc_wait_load();
#pragma unroll
					for (int j = 0; j != 32; ++j) {
						const int col = c0 + c + j;
						if (c + j < n && col < k_count)
							s += __expf(__bfloat162float(__float2bfloat16_rn(__uint_as_float(v[j]) + b3[col])) - m);
					}
				}
				zmax = m;
				zsum = s;
				tc_fence_before();
				__syncthreads();
				tc_fence_after();
				continue;
			}
			// Pass B: DZ of this chunk, BF16, minus this chunk's targets.
			const float scale = coef / zsum;
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
						const float lo = col < k_count
						                     ? scale * __expf(__bfloat162float(__float2bfloat16_rn(__uint_as_float(v[j]) + b3[col])) - zmax)
						                     : 0.0f;
						const float hi =
						    col + 1 < k_count
						        ? scale * __expf(__bfloat162float(__float2bfloat16_rn(__uint_as_float(v[j + 1]) + b3[col + 1])) - zmax)
						        : 0.0f;
						o[k] = pack_bf16x2(lo, hi);
					}
					*reinterpret_cast<uint4*>(tw_smem + kTwDz + tc_offset((int) tid, c + 8 * q, kTcChunk)) = out;
				}
			}
			if (learn) {
				const float unshadowed = wu / total * pr.inv_batch;
				for (int c = 0; c < mc; ++c) {
					const ProposalCandidate q = cand[c];
					if (q.pdf > 0.0f && (uint32_t) q.light < pr.light_count) {
						const int cl = (int) pr.light_cluster[q.light] - c0;
						if (cl >= 0 && cl < n) {
							__nv_bfloat16* zp = reinterpret_cast<__nv_bfloat16*>(tw_smem + kTwDz + tc_offset((int) tid, cl, kTcChunk));
							*zp = __float2bfloat16_rn(__bfloat162float(*zp) - unshadowed * q.pdf);
						}
					}
				}
				if (chosen >= 0 && (uint32_t) chosen < pr.light_count && ss > 0.0f) {
					const int cl = (int) pr.light_cluster[chosen] - c0;
					if (cl >= 0 && cl < n) {
						__nv_bfloat16* zp = reinterpret_cast<__nv_bfloat16*>(tw_smem + kTwDz + tc_offset((int) tid, cl, kTcChunk));
						*zp = __float2bfloat16_rn(__bfloat162float(*zp) - ss * pr.inv_batch);
					}
				}
			}
			sync_for_products();
			// dh2 += DZ_c W3_c (W3 read MN-major: N = hidden, K = clusters)
			// and dW3_c = DZ_c^T [H2 | 1] (both MN-major, K = pixels).
			issue([&] {
				for (int k = 0; k != n / 16; ++k)
					tc_mma(tmem + kTwDh2, tc_descriptor(base + kTwDz + 256 * k, kTcChunk), tc_descriptor_mn(w3 + 2048 * k, 1024, 128),
					       tc_instruction(kTcRows, kMlpHidden) | kTcBMajorMN, ch > 0 || k > 0);
				for (int k = 0; k != kTcRows / 16; ++k)
					tc_mma(tmem + kTwGrad3, tc_descriptor_mn(base + kTwDz + 2 * 2048 * k, 2048, 128),
					       tc_descriptor_mn(base + kTwH2 + 2 * 1280 * k, 1280, 128),
					       tc_instruction(kTcRows, kTtHiddenCols) | kTcAMajorMN | kTcBMajorMN, k > 0);
			});
			await_products();
			if (failed) break;
			// Lane tid of dW3_c: cluster c0 + tid; weights and bias added to
			// the gradient (16-byte aligned rows of 64 floats).
			const int cl = c0 + (int) tid;
			for (int col = 0; col != kTtHiddenCols; col += 16) {
				uint32_t v[16];
				tc_load16(tmem + lane_base + kTwGrad3 + (uint32_t) col, v);
				tc_wait_load();
				if (cl >= k_count) continue;
				if (col < kMlpHidden) {
					float4* g = reinterpret_cast<float4*>(pr.grad + lay.w3 + (size_t) cl * kMlpHidden + col);
#pragma unroll
					for (int q = 0; q != 4; ++q) {
						const float4 a = make_float4(__uint_as_float(v[4 * q]), __uint_as_float(v[4 * q + 1]),
						                             __uint_as_float(v[4 * q + 2]), __uint_as_float(v[4 * q + 3]));
						if (a.x != 0.0f || a.y != 0.0f || a.z != 0.0f || a.w != 0.0f) atomicAdd(g + q, a);
					}
				} else if (__uint_as_float(v[0]) != 0.0f) {
					atomicAdd(pr.grad + lay.b3 + cl, __uint_as_float(v[0]));
				}
			}
			tc_fence_before();
			__syncthreads();
			tc_fence_after();
		}
		if (failed) break;
		gradient_epilogue(kTwDh2, kTwH2);
		// dh1 = DZ2 W2 (W2 MN-major) and dW2 += DZ2^T [H1 | 1].
		issue([&] {
			for (int k = 0; k != kMlpHidden / 16; ++k)
				tc_mma(tmem, tc_descriptor(base + kTwD + 256 * k, kMlpHidden), tc_descriptor_mn(base + kTwW2 + 2048 * k, 1024, 128),
				       tc_instruction(kTcRows, kMlpHidden) | kTcBMajorMN, k > 0);
			for (int k = 0; k != kTcRows / 16; ++k)
				tc_mma(tmem + kTwGrad2, tc_descriptor_mn(base + kTwD + 2048 * k, 1024, 128),
				       tc_descriptor_mn(base + kTwH1 + 2 * 1280 * k, 1280, 128),
				       tc_instruction(kTcRows, kTtHiddenCols) | kTcAMajorMN | kTcBMajorMN, accumulated || k > 0);
		});
		await_products();
		if (failed) break;
		gradient_epilogue(0, kTwH1);  // DZ1 replaces DZ2 (its products are done)
		// dW1 += DZ1^T E.
		issue([&] {
			for (int k = 0; k != kTcRows / 16; ++k)
				tc_mma(tmem + kTwGrad1, tc_descriptor_mn(base + kTwD + 2048 * k, 1024, 128),
				       tc_descriptor_mn(base + kTwE + 2 * 2304 * k, 2304, 128),
				       tc_instruction(kTcRows, kMlpFeatures) | kTcAMajorMN | kTcBMajorMN, accumulated || k > 0);
		});
		await_products();
		accumulated = true;
	}
	if (!failed && accumulated) {
		for (int col = 0; col != kTtHiddenCols; col += 16) {
			uint32_t v[16];
			tc_load16(tmem + lane_base + kTwGrad2 + (uint32_t) col, v);
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
			tc_load16(tmem + lane_base + kTwGrad1 + (uint32_t) col, v);
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
	// Every W3 copy issued completes before the CTA leaves (bounded waits).
	while (copies_waited != copies_issued) {
		const uint32_t b = copies_waited & 1u, ph = (copies_waited >> 1) & 1u;
		tc_wait(bar_w3 + 8 * b, ph);
		++copies_waited;
	}
	tc_fence_before();
	__syncthreads();
	if (warp == 0) {
		tc_fence_after();
		asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(kTtColumns) : "memory");
	}
}

}  // namespace risltc
