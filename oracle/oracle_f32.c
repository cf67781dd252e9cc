/* FP32 instantiation of the oracle: the reference's own precision.
   TEST INFRASTRUCTURE (see oracle.h). */
#include <math.h>
#include "../include/risltc_math.h"

#define R float
#define RC(x) x##f
#define R_FMA(a, b, c) fmaf((a), (b), (c))
#define R_SQRT(x) sqrtf(x)
#define R_ATAN(x) rl_atanf(x)
#define R_ACOS(x) rl_acosf(x)
#define R_SINCOS(x, s, c) rl_sincosf((x), (s), (c))
#define R_FLOOR(x) floorf(x)
#define R_SIGNBIT(x) (signbit(x) != 0)
#define R_ISINF(x) (isinf(x) != 0)
#define R_INF INFINITY
/* Flip every exponent bit (polygon_sampling.glsl:626). */
#define R_EXPONENT_FLIP(x) rl_u2f(rl_f2u(x) ^ 0x7F800000u)
#define ORACLE_SUFFIX _f32
#define ORACLE_OUT_T float
#include "oracle_core.h"
