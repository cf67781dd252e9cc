/* risltc_math.h - single-precision transcendental kernels shared by the host
 * library, the CUDA kernels and the CPU restatement of the shading path.
 *
 * Why these exist: the shading path calls atan (positive_atan in
 * polygon_sampling.glsl:105-112), acos (get_ltc_coefficients,
 * ltc_utility.glsl:59) and cos/sin (sample_projected_solid_angle_polygon,
 * polygon_sampling.glsl:793).  GLSL leaves their precision to the driver, and
 * glibc and the CUDA math library differ from each other by an ulp here and
 * there.  Routing every caller through the functions below, which are built
 * only from IEEE-754 add, multiply, fused multiply-add, divide and square root
 * (all correctly rounded on both the CPU and the GPU), makes the CPU and the
 * GPU produce identical bits.
 *
 * Methods (coefficients fitted for this project by least squares on
 * Chebyshev nodes, weighted to relative error; the script
 * risltc_gb300/csrc/fit_math_coeffs.py refits them by that method and
 * measures the FP32 error of the committed values):
 *  - atan: reduction to [0,1] by atan(x) = pi/2 - atan(1/x), then an odd
 *    polynomial r*P(r^2) of degree 21.  Max error 1.5 ulp on [0,1].
 *  - sin/cos: Cody-Waite reduction by pi/2 (three-part constant, valid for
 *    |x| < 2^14), then minimax-style polynomials on [-pi/4, pi/4].
 *  - acos: acos(x) = 2*atan(sqrt((1-x)/(1+x))).
 *
 * All functions are C99 and compile unchanged as CUDA __host__ __device__.
 */
#ifndef RISLTC_MATH_H
#define RISLTC_MATH_H

#include <stdint.h>
#include <string.h>

#ifdef __CUDACC__
#define RL_HD __host__ __device__ __forceinline__
#else
#define RL_HD static inline
#endif

/* Correctly rounded fused multiply-add and square root.  No <math.h> is
   included so that C++ users can define GLSL-style overloads freely. */
#ifdef __CUDA_ARCH__
#define RL_FMAF(a, b, c) __fmaf_rn((a), (b), (c))
#define RL_SQRTF(x) __fsqrt_rn(x)
#else
#define RL_FMAF(a, b, c) __builtin_fmaf((a), (b), (c))
#define RL_SQRTF(x) __builtin_sqrtf(x)
#endif

#define RL_PI_F 3.14159265358979323846f
#define RL_HALF_PI_F 1.57079632679489661923f

RL_HD uint32_t rl_f2u(float x) {
#ifdef __CUDA_ARCH__
	return __float_as_uint(x);
#else
	uint32_t u;
	memcpy(&u, &x, sizeof(u));
	return u;
#endif
}

RL_HD float rl_u2f(uint32_t u) {
#ifdef __CUDA_ARCH__
	return __uint_as_float(u);
#else
	float x;
	memcpy(&x, &u, sizeof(x));
	return x;
#endif
}

RL_HD float rl_fabsf(float x) { return rl_u2f(rl_f2u(x) & 0x7fffffffu); }

RL_HD float rl_copysignf(float magnitude, float sign) {
	return rl_u2f((rl_f2u(magnitude) & 0x7fffffffu) | (rl_f2u(sign) & 0x80000000u));
}

/* atan on [0, 1]: r * P(r^2). */
RL_HD float rl_atan_unit(float r) {
	float s = r * r;
	float p = 0.0009419943671673536f;
	p = RL_FMAF(p, s, -0.006421414203941822f);
	p = RL_FMAF(p, s, 0.02053668536245823f);
	p = RL_FMAF(p, s, -0.042188216000795364f);
	p = RL_FMAF(p, s, 0.06550370901823044f);
	p = RL_FMAF(p, s, -0.08719014376401901f);
	p = RL_FMAF(p, s, 0.1103052943944931f);
	p = RL_FMAF(p, s, -0.14274851977825165f);
	p = RL_FMAF(p, s, 0.199991837143898f);
	p = RL_FMAF(p, s, -0.3333330452442169f);
	p = p * s;
	return RL_FMAF(r, p, r);
}

/* Arc tangent, odd, result in [-pi/2, pi/2]; NaN propagates. */
RL_HD float rl_atanf(float x) {
	float a = rl_fabsf(x);
	int big = a > 1.0f;
	float r = big ? (1.0f / a) : a;
	float t = rl_atan_unit(r);
	t = big ? (RL_HALF_PI_F - t) : t;
	return rl_copysignf(t, x);
}

/* Arc cosine on [-1, 1] via the half-angle tangent. */
RL_HD float rl_acosf(float x) {
	float q = (1.0f - x) / (1.0f + x);
	return 2.0f * rl_atanf(RL_SQRTF(q));
}

/* Sine and cosine of x, |x| < 2^14, through a quadrant reduction by pi/2. */
RL_HD void rl_sincosf(float x, float* out_sin, float* out_cos) {
	/* k = nearest integer to x * 2/pi; the float cast truncates, so bias
	   by +-0.5 first. */
	float kf = x * 0.6366197466850281f;
	kf = (kf >= 0.0f) ? (float) (int32_t) (kf + 0.5f) : (float) (int32_t) (kf - 0.5f);
	int32_t k = (int32_t) kf;
	/* pi/2 = P1 + P2 + P3 where P1 and P2 carry 12 significant bits, so
	   kf*P1 and kf*P2 are exact. */
	float r = RL_FMAF(-kf, 1.5703125f, x);
	r = RL_FMAF(-kf, 0.0004837512969970703f, r);
	r = RL_FMAF(-kf, 7.549790126404332e-08f, r);
	float s = r * r;
	float ps = 2.718006953728036e-06f;
	ps = RL_FMAF(ps, s, -0.0001983929832931608f);
	ps = RL_FMAF(ps, s, 0.008333329111337662f);
	ps = RL_FMAF(ps, s, -0.1666666716337204f);
	float sin_r = RL_FMAF(r * s, ps, r);
	float pc = -2.7208196229366877e-07f;
	pc = RL_FMAF(pc, s, 2.479949216649402e-05f);
	pc = RL_FMAF(pc, s, -0.0013888883404433727f);
	pc = RL_FMAF(pc, s, 0.0416666679084301f);
	float cos_r = RL_FMAF(s * s, pc, RL_FMAF(-0.5f, s, 1.0f));
	uint32_t q = ((uint32_t) k) & 3u;
	float sv = (q & 1u) ? cos_r : sin_r;
	float cv = (q & 1u) ? sin_r : cos_r;
	sv = (q & 2u) ? -sv : sv;
	cv = ((q + 1u) & 2u) ? -cv : cv;
	*out_sin = sv;
	*out_cos = cv;
}

RL_HD float rl_sinf(float x) {
	float s, c;
	rl_sincosf(x, &s, &c);
	return s;
}

RL_HD float rl_cosf(float x) {
	float s, c;
	rl_sincosf(x, &s, &c);
	return c;
}

#endif /* RISLTC_MATH_H */
