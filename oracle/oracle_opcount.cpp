// Op-counting instantiation of the oracle: the same restatement
// (oracle_core.h) with R = a float that tallies every arithmetic operation.
// bench.py's CPU-baseline leg uses it to fix the algorithmic FP32 work per
// pixel-sample of the benchmark workload (the numerator of the roofline).
// TEST INFRASTRUCTURE (see oracle.h).
#include <cmath>
#include <cstdint>
#include <cstring>
#include "../include/risltc_math.h"

struct OracleOpCounts {
	uint64_t add, mul, fma, div, sqrt, atan, sincos, acos, cmp;
	uint64_t boxes, triangles;  // BVH box tests and ray-triangle tests of the shadow queries
};
static OracleOpCounts g_ops;

struct CF {
	float v;
	CF() : v(0.0f) {}
	CF(float x) : v(x) {}
	CF(double x) : v((float) x) {}
	CF(int x) : v((float) x) {}
	CF(unsigned x) : v((float) x) {}
	explicit operator float() const { return v; }
	explicit operator double() const { return v; }
	explicit operator int() const { return (int) v; }
};
static inline CF operator+(CF a, CF b) { ++g_ops.add; return CF(a.v + b.v); }
static inline CF operator-(CF a, CF b) { ++g_ops.add; return CF(a.v - b.v); }
static inline CF operator*(CF a, CF b) { ++g_ops.mul; return CF(a.v * b.v); }
static inline CF operator/(CF a, CF b) { ++g_ops.div; return CF(a.v / b.v); }
static inline CF operator-(CF a) { return CF(-a.v); }
static inline CF& operator+=(CF& a, CF b) { a = a + b; return a; }
static inline CF& operator-=(CF& a, CF b) { a = a - b; return a; }
static inline CF& operator*=(CF& a, CF b) { a = a * b; return a; }
static inline bool operator<(CF a, CF b) { ++g_ops.cmp; return a.v < b.v; }
static inline bool operator>(CF a, CF b) { ++g_ops.cmp; return a.v > b.v; }
static inline bool operator<=(CF a, CF b) { ++g_ops.cmp; return a.v <= b.v; }
static inline bool operator>=(CF a, CF b) { ++g_ops.cmp; return a.v >= b.v; }
static inline bool operator==(CF a, CF b) { ++g_ops.cmp; return a.v == b.v; }
static inline bool operator!=(CF a, CF b) { ++g_ops.cmp; return a.v != b.v; }
static inline CF cf_fma(CF a, CF b, CF c) { ++g_ops.fma; return CF(__builtin_fmaf(a.v, b.v, c.v)); }
static inline CF cf_sqrt(CF a) { ++g_ops.sqrt; return CF(__builtin_sqrtf(a.v)); }
static inline CF cf_atan(CF a) { ++g_ops.atan; return CF(rl_atanf(a.v)); }
static inline CF cf_acos(CF a) { ++g_ops.acos; return CF(rl_acosf(a.v)); }
static inline void cf_sincos(CF a, CF* s, CF* c) {
	++g_ops.sincos;
	float fs, fc;
	rl_sincosf(a.v, &fs, &fc);
	*s = CF(fs);
	*c = CF(fc);
}

#define R CF
#define RC(x) CF(x##f)
#define R_FMA(a, b, c) cf_fma((a), (b), (c))
#define R_SQRT(x) cf_sqrt(x)
#define R_ATAN(x) cf_atan(x)
#define R_ACOS(x) cf_acos(x)
#define R_SINCOS(x, s, c) cf_sincos((x), (s), (c))
#define R_FLOOR(x) CF(std::floor((x).v))
#define R_SIGNBIT(x) (std::signbit((x).v))
#define R_ISINF(x) (std::isinf((x).v))
#define R_INF CF(INFINITY)
#define R_EXPONENT_FLIP(x) CF(rl_u2f(rl_f2u((x).v) ^ 0x7F800000u))
#define ORACLE_COUNT_BOX() (++g_ops.boxes)
#define ORACLE_COUNT_TRIANGLE() (++g_ops.triangles)
#define ORACLE_SUFFIX _opcount_impl
#define ORACLE_OUT_T float
#include "oracle_core.h"

// Renders rows [row_begin, row_end) with the counting arithmetic and returns
// the tallies.
extern "C" int oracle_opcount_render(const oracle_scene_t* scene, const oracle_settings_t* settings,
                                     const oracle_gbuffer_t* gbuffer, uint32_t random_number_x, int row_begin,
                                     int row_end, float* out_rgb, OracleOpCounts* counts) {
	memset(&g_ops, 0, sizeof(g_ops));
	int status = oracle_render_opcount_impl(scene, settings, gbuffer, random_number_x, row_begin, row_end, out_rgb,
	                                        nullptr);
	if (counts) *counts = g_ops;
	return status;
}
