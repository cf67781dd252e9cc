/* FP64 instantiation of the oracle: the ground-truth twin.  Same algorithm,
   double arithmetic, libm transcendentals; random numbers stay the FP32
   values of the reference's noise stream.  TEST INFRASTRUCTURE (see oracle.h). */
#include <math.h>
#include <string.h>
#include <stdint.h>

static inline double or_exponent_flip(double x) {
	uint64_t u;
	memcpy(&u, &x, 8);
	u ^= 0x7FF0000000000000ull;
	memcpy(&x, &u, 8);
	return x;
}
static inline void or_sincos(double x, double* s, double* c) {
	*s = sin(x);
	*c = cos(x);
}
#define R double
#define RC(x) x
#define R_FMA(a, b, c) fma((a), (b), (c))
#define R_SQRT(x) sqrt(x)
#define R_ATAN(x) atan(x)
#define R_ACOS(x) acos(x)
#define R_SINCOS(x, s, c) or_sincos((x), (s), (c))
#define R_FLOOR(x) floor(x)
#define R_SIGNBIT(x) (signbit(x) != 0)
#define R_ISINF(x) (isinf(x) != 0)
#define R_INF INFINITY
#define R_EXPONENT_FLIP(x) or_exponent_flip(x)
#define ORACLE_SUFFIX _f64
#define ORACLE_OUT_T double
#include "oracle_core.h"
