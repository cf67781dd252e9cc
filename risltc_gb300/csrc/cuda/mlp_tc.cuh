// mlp_tc.cuh - the proposal MLP's forward pass on the 5th-generation tensor
// cores (tcgen05, sm_100 family).
//
// One CTA of four warps per tile of 128 pixels.  The encoded features
// (128 x 144), the hidden activations (128 x 64) and the three weight
// matrices live in shared memory as K-major BF16 operands in 8x8 core
// matrices (no swizzle); one thread issues the products
//   D1 = A1 W1^T (K = 144), D2 = A2 W2^T (K = 64), D3 = A3 W3^T (K = 64,
//   up to 128 clusters per product)
// with FP32 accumulators in tensor memory (256 columns per CTA: D1 and D2 in
// columns 0..63, D3 in 64..191), and each warp moves its 32 rows (pixels)
// from tensor memory to registers for the epilogues: bias, ReLU and BF16
// rounding back into shared memory for the next product, or bias and BF16
// rounding of the logits to global memory.  Every wait on the tensor cores
// is bounded; on a timeout the kernel records kErrorTensorWait, waits once
// more (bounded) for its products in flight, frees its tensor memory and
// returns.
#pragma once
#include "mlp.cuh"

namespace risltc {

constexpr int kTcRows = 128;      // pixels per tile: M of every product
constexpr int kTcThreads = 128;   // warp w reads tensor-memory lanes 32w .. 32w + 31
constexpr uint32_t kTcColumns = 256;
constexpr int kTcChunk = 128;     // clusters per layer-3 product (N)
constexpr uint64_t kTcWaitNs = 1000000000ull;  // a tensor-core wait gives up after one second
constexpr uint32_t kErrorTensorWait = 1u << 2;  // error-word bit: a tensor-core wait ran out

RL_DEV uint32_t smem_address(const void* p) { return (uint32_t) __cvta_generic_to_shared(p); }

// Shared-memory matrix descriptor of a K-major operand with k columns whose
// first core matrix is at shared address addr (no swizzle): core matrices
// 128 bytes apart along K (leading byte offset), 8-row groups (k / 8) * 128
// bytes apart (stride byte offset); bits 46-48 hold the descriptor version 1.
RL_DEV uint64_t tc_descriptor(uint32_t addr, int k) {
	const uint64_t leading = 128, stride = (uint64_t) (k >> 3) * 128;
	return (uint64_t) ((addr & 0x3FFFFu) >> 4) | ((leading >> 4) << 16) | ((stride >> 4) << 32) | (1ull << 46);
}

// Instruction descriptor of kind::f16: FP32 accumulator, BF16 A and B, both
// K-major, M x N.
__host__ __device__ constexpr uint32_t tc_instruction(int m, int n) {
	return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t) (n >> 3) << 17) | ((uint32_t) (m >> 4) << 24);
}

// D (tensor memory) = A B^T (+ D if accumulate).
RL_DEV void tc_mma(uint32_t d, uint64_t a, uint64_t b, uint32_t instruction, uint32_t accumulate) {
	asm volatile(
	    "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
	    "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n"
	    :
	    : "r"(d), "l"(a), "l"(b), "r"(instruction), "r"(accumulate)
	    : "memory");
}

// The mbarrier at shared address bar completes its phase when the products
// issued so far by this thread are done.
RL_DEV void tc_commit(uint32_t bar) {
	asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(bar)
	             : "memory");
}

RL_DEV bool mbarrier_try_wait(uint32_t bar, uint32_t parity) {
	uint32_t done;
	asm volatile(
	    "{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\nselp.u32 %0, 1, 0, p;\n}\n"
	    : "=r"(done)
	    : "r"(bar), "r"(parity)
	    : "memory");
	return done != 0;
}

RL_DEV uint64_t global_ns() {
	uint64_t t;
	asm volatile("mov.u64 %0, %%globaltimer;\n" : "=l"(t));
	return t;
}

// Waits for phase `parity` of the mbarrier for at most kTcWaitNs (and at
// most 2^28 polls).
RL_DEV bool tc_wait(uint32_t bar, uint32_t parity) {
	const uint64_t t0 = global_ns();
	for (uint32_t i = 0; i != (1u << 28); ++i) {
		if (mbarrier_try_wait(bar, parity)) return true;
		if ((i & 255u) == 255u && global_ns() - t0 > kTcWaitNs) return false;
	}
	return false;
}

// The mbarrier's phase also waits for `bytes` of asynchronous copies (one
// arrival by this thread).
RL_DEV void mbarrier_expect_bytes(uint32_t bar, uint32_t bytes) {
	asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(bar), "r"(bytes) : "memory");
}

// Bulk copy (TMA, no tensor map) of `bytes` (a multiple of 16; both
// addresses 16-byte aligned) from global memory into this CTA's shared
// memory, counted on the mbarrier.
RL_DEV void bulk_copy_to_shared(uint32_t dst, const void* src, uint32_t bytes, uint32_t bar) {
	asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];\n" ::"r"(dst),
	             "l"(src), "r"(bytes), "r"(bar)
	             : "memory");
}

RL_DEV void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory"); }
RL_DEV void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory"); }
RL_DEV void tc_wait_load() { asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory"); }
// Makes this thread's shared-memory writes visible to the tensor cores.
RL_DEV void fence_async_shared() { asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory"); }

// 32 consecutive FP32 columns of this thread's tensor-memory lane.
RL_DEV void tc_load32(uint32_t taddr, uint32_t (&v)[32]) {
	asm volatile(
	    "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];\n"
	    : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]), "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15]), "=r"(v[16]), "=r"(v[17]), "=r"(v[18]), "=r"(v[19]), "=r"(v[20]), "=r"(v[21]), "=r"(v[22]), "=r"(v[23]), "=r"(v[24]), "=r"(v[25]), "=r"(v[26]), "=r"(v[27]), "=r"(v[28]), "=r"(v[29]), "=r"(v[30]), "=r"(v[31])
	    : "r"(taddr));
}

// Shared memory of the kernel for k_count clusters: W1, W2, W3 (rows padded
// to a multiple of 16; together the operand-layout weights of one bulk copy),
// A1, A2, the biases, three mbarriers (products, weights, inputs) and the
// tensor memory address.  A tile's 10 input rows (128 floats each) are
// staged in the first 5 KB of A2, which is free from a tile's last layer-3
// product until the next tile's first epilogue.
struct TcLayout {
	uint32_t w1, w2, w3, a1, a2, b1, b2, b3, bar, slot, total, weight_bytes;
	int k_pad;
};
__host__ __device__ inline TcLayout tc_layout(int k_count) {
	TcLayout l;
	l.k_pad = mlp_padded_clusters(k_count);
	l.weight_bytes = (uint32_t) mlp_weight_elements(k_count) * 2;
	l.w1 = 0;
	l.w2 = l.w1 + kMlpHidden * kMlpFeatures * 2;
	l.w3 = l.w2 + kMlpHidden * kMlpHidden * 2;
	l.a1 = l.w3 + (uint32_t) l.k_pad * kMlpHidden * 2;
	l.a2 = l.a1 + kTcRows * kMlpFeatures * 2;
	l.b1 = l.a2 + kTcRows * kMlpHidden * 2;
	l.b2 = l.b1 + kMlpHidden * 4;
	l.b3 = l.b2 + kMlpHidden * 4;
	l.bar = (l.b3 + (uint32_t) l.k_pad * 4 + 7) / 8 * 8;
	l.slot = l.bar + 3 * 8;
	l.total = l.slot + 8;
	return l;
}
static_assert(kMlpInputs * kTcRows * 4 <= kTcRows * kMlpHidden * 2, "inputs fit in A2");

// G-buffer plane of MLP input k (position, normal, outgoing, roughness).
RL_DEV int mlp_input_plane(int k) { return k < 9 ? k : 16; }

static __global__ void __launch_bounds__(kTcThreads, 1) mlp_logits_tc_kernel(MlpParams pr) {
	extern __shared__ __align__(1024) unsigned char tc_smem[];
	const int k_count = pr.k_count;
	const MlpLayout lay = mlp_layout(k_count);
	const TcLayout tl = tc_layout(k_count);
	const uint32_t tid = threadIdx.x, warp = tid / 32;
	const uint32_t base = smem_address(tc_smem);
	float* b1 = reinterpret_cast<float*>(tc_smem + tl.b1);
	float* b2 = reinterpret_cast<float*>(tc_smem + tl.b2);
	float* b3 = reinterpret_cast<float*>(tc_smem + tl.b3);
	const float* inputs = reinterpret_cast<const float*>(tc_smem + tl.a2);  // [10][128] while staged
	for (int j = tid; j < kMlpHidden; j += kTcThreads) {
		b1[j] = pr.params[lay.b1 + j];
		b2[j] = pr.params[lay.b2 + j];
	}
	for (int j = tid; j < tl.k_pad; j += kTcThreads) b3[j] = j < k_count ? pr.params[lay.b3 + j] : 0.0f;
	const uint32_t bar = base + tl.bar, bar_weights = bar + 8, bar_inputs = bar + 16;
	const uint32_t np = pr.width * pr.height;
	const uint32_t tiles = (np + kTcRows - 1) / kTcRows;
	// A tile's input rows come by bulk copy when every row is 16-byte aligned
	// and a multiple of 16 bytes long, else by plain loads.
	const bool bulk_inputs = np % 4 == 0 && (reinterpret_cast<uintptr_t>(pr.gbuffer) & 15) == 0;
	// Bulk copies issued and waited for on the inputs' mbarrier (the same on
	// every thread: the issue decisions are uniform).
	uint32_t inputs_issued = 0, inputs_waited = 0;
	auto fetch_inputs = [&](uint32_t tile) {
		if (tid == 0) {
			const uint32_t p0 = tile * kTcRows, rows = min((uint32_t) kTcRows, np - p0);
			mbarrier_expect_bytes(bar_inputs, kMlpInputs * rows * 4);
			for (int k = 0; k != kMlpInputs; ++k)
				bulk_copy_to_shared(base + tl.a2 + k * kTcRows * 4, pr.gbuffer + (size_t) mlp_input_plane(k) * np + p0,
				                    rows * 4, bar_inputs);
		}
		++inputs_issued;
	};
	if (tid == 0) {
		for (int k = 0; k != 3; ++k) asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(bar + 8 * k) : "memory");
		asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
		// The weights in one bulk copy.
		mbarrier_expect_bytes(bar_weights, tl.weight_bytes);
		bulk_copy_to_shared(base + tl.w1, pr.weights, tl.weight_bytes, bar_weights);
	}
	if (bulk_inputs && blockIdx.x < tiles) fetch_inputs(blockIdx.x);  // the first tile's inputs
	if (warp == 0) {
		asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(base + tl.slot),
		             "r"(kTcColumns)
		             : "memory");
		asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
	}
	fence_async_shared();
	tc_fence_before();
	__syncthreads();
	tc_fence_after();
	const uint32_t tmem = *reinterpret_cast<volatile uint32_t*>(tc_smem + tl.slot);
	const uint32_t d12 = tmem, d3 = tmem + 64;
	const uint32_t lane_base = (warp * 32) << 16;  // this warp's tensor-memory lanes
	uint32_t parity = 0;
	bool product_pending = false;
	const bool weights_ok = __syncthreads_or(!tc_wait(bar_weights, 0)) == 0;
	bool failed = !weights_ok;
	// One product group: issued by thread 0, then every thread waits for it.
	// With pr.skip_issue (fault injection) nothing is issued or committed, so
	// the wait runs out.
	auto run = [&](auto issue) {
		if (tid == 0 && !pr.skip_issue) {
			issue();
			tc_commit(bar);
		}
		const bool ok = tc_wait(bar, parity);
		parity ^= 1u;
		failed = __syncthreads_or(!ok) != 0;
		product_pending = failed && !pr.skip_issue;
		tc_fence_after();
	};
	// Epilogue of a hidden layer: row tid of D (64 columns) + bias, ReLU,
	// BF16 into A2.
	auto hidden_epilogue = [&](const float* bias) {
		for (int c = 0; c != kMlpHidden; c += 32) {
			uint32_t v[32];
			tc_load32(d12 + lane_base + (uint32_t) c, v);
			tc_wait_load();
#pragma unroll
			for (int q = 0; q != 4; ++q) {
				uint4 out;
				uint32_t* o = &out.x;
#pragma unroll
				for (int h = 0; h != 4; ++h) {
					const int j = 8 * q + 2 * h;
					o[h] = pack_bf16x2(fmaxf(__uint_as_float(v[j]) + bias[c + j], 0.0f),
					                   fmaxf(__uint_as_float(v[j + 1]) + bias[c + j + 1], 0.0f));
				}
				*reinterpret_cast<uint4*>(tc_smem + tl.a2 + tc_offset((int) tid, c + 8 * q, kMlpHidden)) = out;
			}
		}
		fence_async_shared();
		tc_fence_before();
		__syncthreads();
		tc_fence_after();
	};
	for (uint32_t tile = blockIdx.x; tile < tiles && !failed; tile += gridDim.x) {
		const uint32_t p0 = tile * kTcRows;
		if (bulk_inputs) {
			// This tile's input rows (issued during the previous tile).
			failed = __syncthreads_or(!tc_wait(bar_inputs, inputs_waited & 1u)) != 0;
			if (failed) break;
			++inputs_waited;
		}
		// Encode the tile's pixels into A1.
		for (int idx = tid; idx < kTcRows * kMlpInputs; idx += kTcThreads) {
			const int r = idx / kMlpInputs, input = idx % kMlpInputs;
			const uint32_t i = p0 + (uint32_t) r;
			float x = 0.0f;
			if (i < np) {
				if (bulk_inputs) {
					x = inputs[input * kTcRows + r];
					if (input < 3) x = (x - pr.center[input]) * pr.inv_half_extent;
				} else {
					x = mlp_input(pr.gbuffer, np, i, pr.center, pr.inv_half_extent, input);
				}
			}
			float e[13];
			mlp_encode(x, e);
#pragma unroll
			for (int kind = 0; kind != 13; ++kind)
				*reinterpret_cast<__nv_bfloat16*>(tc_smem + tl.a1 + tc_offset(r, input * 13 + kind, kMlpFeatures)) =
				    __float2bfloat16_rn(i < np ? e[kind] : 0.0f);
		}
		for (int idx = tid; idx < kTcRows * (kMlpFeatures - 130); idx += kTcThreads)
			*reinterpret_cast<__nv_bfloat16*>(
			    tc_smem + tl.a1 + tc_offset(idx / (kMlpFeatures - 130), 130 + idx % (kMlpFeatures - 130), kMlpFeatures)) =
			    __float2bfloat16_rn(0.0f);
		fence_async_shared();
		tc_fence_before();
		__syncthreads();
		tc_fence_after();
		run([&] {
			for (int k = 0; k != kMlpFeatures / 16; ++k)
				tc_mma(d12, tc_descriptor(base + tl.a1 + 256 * k, kMlpFeatures),
				       tc_descriptor(base + tl.w1 + 256 * k, kMlpFeatures), tc_instruction(kTcRows, kMlpHidden), k > 0);
		});
		if (failed) break;
		hidden_epilogue(b1);
		run([&] {
			for (int k = 0; k != kMlpHidden / 16; ++k)
				tc_mma(d12, tc_descriptor(base + tl.a2 + 256 * k, kMlpHidden),
				       tc_descriptor(base + tl.w2 + 256 * k, kMlpHidden), tc_instruction(kTcRows, kMlpHidden), k > 0);
		});
		if (failed) break;
		hidden_epilogue(b2);
		const uint32_t row = p0 + tid;
		for (int c0 = 0; c0 < tl.k_pad && !failed; c0 += kTcChunk) {
			const int n = min(kTcChunk, tl.k_pad - c0);
			run([&] {
				for (int k = 0; k != kMlpHidden / 16; ++k)
					tc_mma(d3, tc_descriptor(base + tl.a2 + 256 * k, kMlpHidden),
					       tc_descriptor(base + tl.w3 + (uint32_t) c0 * 128 + 256 * k, kMlpHidden),
					       tc_instruction(kTcRows, n), k > 0);
			});
			if (failed) break;
			// After the tile's last product A2 is free: the next tile's inputs
			// arrive there while this tile's logits are written.
			if (c0 + kTcChunk >= tl.k_pad && bulk_inputs && tile + gridDim.x < tiles) fetch_inputs(tile + gridDim.x);
			for (int c = 0; c < n; c += 32) {
				uint32_t v[32];
				tc_load32(d3 + lane_base + (uint32_t) c, v);
				tc_wait_load();
				if (row < np) {
					__nv_bfloat16* dst = pr.logits + (size_t) row * k_count + c0 + c;
#pragma unroll
					for (int q = 0; q != 4; ++q) {
						const int j0 = c0 + c + 8 * q;
						if (j0 + 8 > k_count) continue;  // k_count is a multiple of 8
						uint4 out;
						uint32_t* o = &out.x;
#pragma unroll
						for (int h = 0; h != 4; ++h) {
							const int j = 8 * q + 2 * h;
							o[h] = pack_bf16x2(__uint_as_float(v[j]) + b3[c0 + c + j],
							                   __uint_as_float(v[j + 1]) + b3[c0 + c + j + 1]);
						}
						*reinterpret_cast<uint4*>(dst + 8 * q) = out;
					}
				}
			}
			tc_fence_before();
			__syncthreads();
			tc_fence_after();
		}
	}
	if (failed) {
		// Record the timeout, then wait (bounded) for whatever is still in
		// flight: a product, the weights' copy, input copies.
		if (tid == 0) atomicOr(pr.error, kErrorTensorWait);
		if (product_pending) tc_wait(bar, parity ^ 1u);
		if (!weights_ok) tc_wait(bar_weights, 0);
		while (inputs_waited < inputs_issued) tc_wait(bar_inputs, inputs_waited++ & 1u);
	}
	tc_fence_before();
	__syncthreads();
	if (warp == 0) {
		tc_fence_after();
		asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(kTcColumns) : "memory");
	}
}

inline size_t mlp_tc_smem_bytes(int k_count) { return tc_layout(k_count).total; }

}  // namespace risltc
