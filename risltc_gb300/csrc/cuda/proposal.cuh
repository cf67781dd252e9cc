// proposal.cuh - a cluster proposal for the RIS candidates.
//
// The reference draws every RIS candidate uniformly over all lights
// (shading_pass.frag.glsl:728-733, p = 1/N).  Here, with lights listed
// cluster by cluster, each pixel gets a distribution q over the clusters and
// draws each candidate from the defensive mixture
//     p(light) = a / N + (1 - a) * q(cluster of light) / |cluster|,
// a = the uniform fraction; the candidate kernel then weighs it with
// w = p_hat / p(light), which keeps RIS unbiased for any q (Talbot et al.
// 2005; the reservoir's W = w_sum / (M p_hat) is unchanged).
//
// q is proportional to per-cluster weights: either a power / distance bound
// (cluster_weight below) or exp of the logits of a learned model.  The
// proposal kernel runs one warp per pixel: lane l sums the weights of a
// block of clusters, a warp scan turns the sums into the cumulative
// distribution (in shared memory), and the warp draws the pixel's candidates
// for all frames of the call by inverse transform sampling.  Every
// probability written out is computed from the same cumulative values that
// the draw compares against.
#pragma once
#include <cuda_bf16.h>
#include "shade_device.cuh"

namespace risltc {

struct ClusterView {
	const uint32_t* offsets;        // cluster_count + 1: cluster c holds lights offsets[c] .. offsets[c + 1]
	const uint2* spans;             // cluster_count: {offsets[c], light count of c}
	// The same per-cluster data lane-major for the proposal kernel's weight
	// pass, where lane l takes clusters l * per_lane .. + per_lane - 1
	// (per_lane = ceil(count / 32)): entry j * 32 + l holds cluster
	// l * per_lane + j (zeros past the last cluster), so a warp's loads of its
	// j-th clusters are contiguous.
	const float4* bounds_lane;
	const float* power_lane;
	const uint32_t* size_lane;
	const uint32_t* light_cluster;  // light_count: the cluster of each light
	const float4* bounds;           // cluster_count: centre xyz, radius of a sphere around its lights
	const float* power;             // cluster_count: sum of luminance x area of its lights
	int count;
};

struct ProposalCandidate {
	int32_t light;
	float pdf;
};

constexpr int kMaxClusters = 1024;
constexpr int kProposalWarps = 4;
constexpr int kLogitCache = 8;  // logits per lane kept in registers (256 clusters: all of them)

struct ProposalParams {
	SceneView scene;
	ClusterView clusters;
	const float* gbuffer;
	const uint32_t* primitive;
	uint32_t width, height;
	int candidate_count;
	uint32_t noise_seed, animate, frame_count;
	float uniform_fraction;
	const __nv_bfloat16* logits;  // [pixel][cluster], or null for cluster_weight
	ProposalCandidate* out;       // [frame][pixel][candidate]
};

// The unnormalised heuristic weight of a cluster for a shading point x with
// normal n: the cluster's power times an upper bound of the cosine towards its
// bounding sphere over the squared distance (both clamped by the radius).
RL_DEV float cluster_weight(float4 bound, float power, f3 x, f3 n) {
	const f3 v = sub(mk3(bound.x, bound.y, bound.z), x);
	const float d2 = dot(v, v);
	const float h = dot(n, v);
	const float rr = bound.w * bound.w;
	const float dd = d2 > rr ? d2 : rr;
	float up = h + bound.w;
	up = up > 0.0f ? up : 0.0f;
	return __fdiv_rn(power * up, dd * __fsqrt_rn(dd));
}

// Shared-memory slot of cumulative weight k: one pad word per 8 clusters, so
// that the lanes' blocks of 8 start in different banks.
RL_DEV int cdf_slot(int k) { return k + (k >> 3); }

// The noise stream of candidate c of a pixel-frame: the pixel's accessor for
// the frame's second noise number, decorrelated per candidate.
RL_DEV uint32_t proposal_stream(uint32_t x, uint32_t y, uint32_t width, uint32_t noise_seed, uint32_t f,
                                uint32_t animate, uint32_t c) {
	const uint32_t rn = animate ? wang_random_number((noise_seed + f) * 4u + 1u) : 0x123456u;
	return get_noise_accessor(x, y, width, rn) ^ (c * 0x9E3779B9u);
}

// Words of one warp's cumulative weights in shared memory (with the pads).
__host__ __device__ inline int proposal_cdf_words(int cluster_count) { return cluster_count + (cluster_count >> 3) + 1; }

static __global__ void __launch_bounds__(32 * kProposalWarps) proposal_kernel(ProposalParams pr) {
	extern __shared__ float proposal_smem[];
	const uint32_t lane = threadIdx.x % 32;
	const int k_count = pr.clusters.count;
	float* cdf = proposal_smem + (threadIdx.x / 32) * proposal_cdf_words(k_count);
	const uint32_t np = pr.width * pr.height;
	const int n_lights = pr.scene.light_count;
	const int per_lane = (k_count + 31) / 32;
	const float a = pr.uniform_fraction;
	const int k0 = (int) lane * per_lane;  // this lane's block of clusters
	const uint32_t stride = gridDim.x * kProposalWarps;
	// The next pixel's inputs are loaded while the current one is processed
	// (software pipelining over the warp's pixels): its background flag, its
	// position and normal (heuristic weights) or the first kLogitCache logits
	// of this lane's block (learned weights).
	struct Inputs {
		bool skip;
		f3 x, n;
		float logit[kLogitCache];
	};
	auto fetch = [&](uint32_t p, Inputs& in) {
		in.skip = pr.primitive && pr.primitive[p] == 0xffffffffu;
		if (pr.logits) {
			const __nv_bfloat16* row = pr.logits + (size_t) p * k_count + k0;
			if (per_lane == kLogitCache && k_count % kLogitCache == 0) {
				// The lane's 8 logits in one 16-byte load.
				const uint4 q = __ldg(reinterpret_cast<const uint4*>(row));
				const uint32_t w[4] = {q.x, q.y, q.z, q.w};
#pragma unroll
				for (int j = 0; j != kLogitCache; ++j)
					in.logit[j] = __uint_as_float((j & 1) ? (w[j / 2] & 0xffff0000u) : (w[j / 2] << 16));
			} else {
#pragma unroll
				for (int j = 0; j != kLogitCache; ++j)
					in.logit[j] = (j < per_lane && k0 + j < k_count) ? __bfloat162float(row[j]) : -INFINITY;
			}
			in.x = in.n = splat(0.0f);  // unused by learned weights
		} else {
			const float* g = pr.gbuffer;
			const size_t snp = np;
			in.x = mk3(g[0 * snp + p], g[1 * snp + p], g[2 * snp + p]);
			in.n = mk3(g[3 * snp + p], g[4 * snp + p], g[5 * snp + p]);
		}
	};
	Inputs next;
	uint32_t i = blockIdx.x * kProposalWarps + threadIdx.x / 32;
	if (i < np) fetch(i, next);
	for (; i < np; i += stride) {
		const Inputs cur = next;
		if (i + stride < np) fetch(i + stride, next);
		if (cur.skip) continue;
		const f3 x = cur.x, n = cur.n;
		// This lane's block of clusters: inclusive prefix sums.
		float local = 0.0f;
		float logit_max = -INFINITY;
		float cached[kLogitCache];
		if (pr.logits) {
			const __nv_bfloat16* row = pr.logits + (size_t) i * k_count + k0;
#pragma unroll
			for (int j = 0; j != kLogitCache; ++j) {
				cached[j] = cur.logit[j];
				logit_max = fmaxf(logit_max, cached[j]);
			}
			for (int j = kLogitCache; j < per_lane; ++j)
				if (k0 + j < k_count) logit_max = fmaxf(logit_max, __bfloat162float(row[j]));
			for (int d = 16; d != 0; d >>= 1) logit_max = fmaxf(logit_max, __shfl_xor_sync(0xffffffffu, logit_max, d));
		}
#pragma unroll
		for (int j = 0; j != kLogitCache; ++j) {
			const int k = k0 + j;
			if (j < per_lane && k < k_count) {
				const uint32_t t = (uint32_t) j * 32 + lane;
				const bool empty = pr.clusters.size_lane[t] == 0;
				float w;
				if (pr.logits)
					w = empty ? 0.0f : __expf(cached[j] - logit_max);
				else
					w = empty ? 0.0f : cluster_weight(pr.clusters.bounds_lane[t], pr.clusters.power_lane[t], x, n);
				local += w;
				cdf[cdf_slot(k)] = local;
			}
		}
		for (int j = kLogitCache; j < per_lane; ++j) {
			const int k = k0 + j;
			if (k >= k_count) break;
			const uint32_t t = (uint32_t) j * 32 + lane;
			const bool empty = pr.clusters.size_lane[t] == 0;
			float w;
			if (pr.logits)
				w = empty ? 0.0f : __expf(__bfloat162float(pr.logits[(size_t) i * k_count + k]) - logit_max);
			else
				w = empty ? 0.0f : cluster_weight(pr.clusters.bounds_lane[t], pr.clusters.power_lane[t], x, n);
			local += w;
			cdf[cdf_slot(k)] = local;
		}
		// Inclusive scan of the lanes' sums, then offset each block.
		float incl = local;
		for (int d = 1; d < 32; d <<= 1) {
			const float o = __shfl_up_sync(0xffffffffu, incl, d);
			if ((int) lane >= d) incl += o;
		}
		float excl = __shfl_up_sync(0xffffffffu, incl, 1);
		excl = lane == 0 ? 0.0f : excl;
		const float total = __shfl_sync(0xffffffffu, incl, 31);
		for (int j = 0; j != per_lane; ++j) {
			const int k = k0 + j;
			if (k >= k_count) break;
			cdf[cdf_slot(k)] = excl + cdf[cdf_slot(k)];
		}
		__syncwarp();
		const bool proposal = total > 0.0f && total <= 3.0e38f;
		const uint32_t x_pix = i % pr.width, y_pix = i / pr.width;
		const int per_frame = pr.candidate_count;
		// The pixel's draws of all frames, spread over the lanes (each draw
		// has its own noise stream, so any lane may take any draw).
		const uint32_t draws = pr.frame_count * (uint32_t) per_frame;
		for (uint32_t d = lane; d < draws; d += 32) {
			const uint32_t f = d / (uint32_t) per_frame;
			const int c = (int) (d % (uint32_t) per_frame);
			{
				uint32_t s = proposal_stream(x_pix, y_pix, pr.width, pr.noise_seed, f, pr.animate, (uint32_t) c);
				const float u0 = get_noise_1(s), u1 = get_noise_1(s), u2 = get_noise_1(s);
				int light;
				if (!proposal || u0 < a) {
					light = (int) (u1 * (float) n_lights);
					light = light > n_lights - 1 ? n_lights - 1 : light;
				} else {
					// First cluster whose cumulative weight exceeds u1 * total.
					const float t = u1 * total;
					int lo = 0, hi = k_count - 1;
					while (lo < hi) {
						const int mid = (lo + hi) >> 1;
						if (cdf[cdf_slot(mid)] > t)
							hi = mid;
						else
							lo = mid + 1;
					}
					// Rounding can leave t at the top: take the last non-empty cluster.
					uint2 span = pr.clusters.spans[lo];
					while (lo > 0 && span.y == 0) span = pr.clusters.spans[--lo];
					const uint32_t first = span.x, size = span.y;
					uint32_t j = (uint32_t) (u2 * (float) size);
					j = j > size - 1 ? size - 1 : j;
					light = (int) (first + j);
				}
				float pdf = __frcp_rn((float) n_lights);
				if (proposal) {
					const uint32_t k = pr.clusters.light_cluster[light];
					const float mass = cdf[cdf_slot((int) k)] - (k > 0 ? cdf[cdf_slot((int) k - 1)] : 0.0f);
					const uint32_t size = pr.clusters.spans[k].y;
					pdf = __fadd_rn(__fdiv_rn(a, (float) n_lights),
					                __fdiv_rn(__fmul_rn(1.0f - a, __fdiv_rn(mass, total)), (float) size));
				}
				pr.out[((size_t) f * np + i) * per_frame + c] = ProposalCandidate{light, pdf};
			}
		}
		__syncwarp();
	}
}

inline size_t proposal_smem_bytes(int cluster_count) {
	return sizeof(float) * kProposalWarps * proposal_cdf_words(cluster_count);
}

}  // namespace risltc
