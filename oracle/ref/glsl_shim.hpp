// glsl_shim.hpp - a minimal GLSL 4.6 environment in C++17, used only to
// compile the reference renderer's own shading-pass GLSL on the CPU (the
// pinning reference for the oracle; see oracle/ref/build_ref.py).
//
// Test infrastructure: nothing in the product includes this file.
//
// Conventions, identical in the C99 oracle and in the CUDA kernels' "exact"
// numerics mode (so all three agree bit for bit):
//  - no contraction of a*b+c (the file is compiled with -ffp-contract=off);
//    fma() is the correctly rounded fused multiply-add;
//  - dot(a, b) = ((a.x*b.x + a.y*b.y) + a.z*b.z) [+ a.w*b.w], left to right;
//  - M * v = ((col0*v[0] + col1*v[1]) + col2*v[2]) [+ col3*v[3]], per row;
//  - normalize(v) = v * inversesqrt(dot(v, v)), inversesqrt(x) = 1/sqrt(x);
//  - max(x, y) = (x < y) ? y : x, min(x, y) = (y < x) ? y : x;
//  - atan/acos/sin/cos are the project's own kernels from risltc_math.h;
//  - default-constructed (uninitialised) vectors read as (0, 0, 1).  GLSL
//    leaves them undefined; (0,0,1) is the value for which the reference's
//    calculate_ltc() (polygon_sampling.glsl:523-530), which also integrates
//    over unwritten array slots, adds exactly zero for them.
#pragma once
#include <cstdint>
#include <cstring>
#include "../../include/risltc_math.h"

typedef unsigned int uint;

struct vec2;
struct vec3;
struct vec4;
struct ivec2;
struct uvec2;

// ---- swizzle proxies (storage-compatible views inside the vector unions) --
template <int N, int A, int B> struct Sw2 {
	float e[N];
	inline operator vec2() const;
	inline Sw2& operator=(const vec2& rhs);
	inline Sw2& operator=(const Sw2& rhs) { return *this = (vec2) rhs; }
	inline Sw2& operator*=(float rhs);
	inline Sw2& operator+=(const vec2& rhs);
};
template <int N, int A, int B, int C> struct Sw3 {
	float e[N];
	inline operator vec3() const;
	inline Sw3& operator=(const vec3& rhs);
	inline Sw3& operator=(const Sw3& rhs) { return *this = (vec3) rhs; }
};

struct vec2 {
	union {
		struct { float x, y; };
		struct { float r, g; };
		float e[2];
		Sw2<2, 0, 1> xy;
		Sw2<2, 1, 0> yx;
		Sw2<2, 0, 1> rg;
	};
	vec2() : x(0.0f), y(0.0f) {}
	explicit vec2(float s) : x(s), y(s) {}
	vec2(float a, float b) : x(a), y(b) {}
	vec2(const vec2& o) : x(o.x), y(o.y) {}
	vec2& operator=(const vec2& o) { x = o.x; y = o.y; return *this; }
	inline explicit vec2(const ivec2& o);
	float& operator[](int i) { return e[i]; }
	float operator[](int i) const { return e[i]; }
};

struct vec3 {
	union {
		struct { float x, y, z; };
		struct { float r, g, b; };
		float e[3];
		Sw2<3, 0, 1> xy;
		Sw2<3, 1, 2> yz;
		Sw2<3, 1, 0> yx;
		Sw2<3, 0, 1> rg;
		Sw3<3, 0, 1, 2> xyz;
		Sw3<3, 0, 1, 2> rgb;
	};
	vec3() : x(0.0f), y(0.0f), z(1.0f) {}
	explicit vec3(float s) : x(s), y(s), z(s) {}
	vec3(float a, float b, float c) : x(a), y(b), z(c) {}
	vec3(const vec2& v, float c) : x(v.x), y(v.y), z(c) {}
	vec3(float a, const vec2& v) : x(a), y(v.x), z(v.y) {}
	inline vec3(const ivec2& v, float c);
	vec3(const vec3& o) : x(o.x), y(o.y), z(o.z) {}
	vec3& operator=(const vec3& o) { x = o.x; y = o.y; z = o.z; return *this; }
	float& operator[](int i) { return e[i]; }
	float operator[](int i) const { return e[i]; }
};

struct vec4 {
	union {
		struct { float x, y, z, w; };
		struct { float r, g, b, a; };
		float e[4];
		Sw2<4, 0, 1> xy;
		Sw2<4, 2, 3> zw;
		Sw2<4, 0, 1> rg;
		Sw3<4, 0, 1, 2> xyz;
		Sw3<4, 0, 1, 2> rgb;
	};
	vec4() : x(0.0f), y(0.0f), z(0.0f), w(0.0f) {}
	explicit vec4(float s) : x(s), y(s), z(s), w(s) {}
	vec4(float a, float b, float c, float d) : x(a), y(b), z(c), w(d) {}
	vec4(const vec3& v, float d) : x(v.x), y(v.y), z(v.z), w(d) {}
	vec4(const vec4& o) : x(o.x), y(o.y), z(o.z), w(o.w) {}
	vec4& operator=(const vec4& o) { x = o.x; y = o.y; z = o.z; w = o.w; return *this; }
	float& operator[](int i) { return e[i]; }
	float operator[](int i) const { return e[i]; }
};

template <int N, int A, int B> inline Sw2<N, A, B>::operator vec2() const { return vec2(e[A], e[B]); }
template <int N, int A, int B> inline Sw2<N, A, B>& Sw2<N, A, B>::operator=(const vec2& rhs) {
	float a = rhs.x, b = rhs.y;
	e[A] = a;
	e[B] = b;
	return *this;
}
template <int N, int A, int B> inline Sw2<N, A, B>& Sw2<N, A, B>::operator*=(float rhs) {
	e[A] = e[A] * rhs;
	e[B] = e[B] * rhs;
	return *this;
}
template <int N, int A, int B> inline Sw2<N, A, B>& Sw2<N, A, B>::operator+=(const vec2& rhs) {
	e[A] = e[A] + rhs.x;
	e[B] = e[B] + rhs.y;
	return *this;
}
template <int N, int A, int B, int C> inline Sw3<N, A, B, C>::operator vec3() const { return vec3(e[A], e[B], e[C]); }
template <int N, int A, int B, int C> inline Sw3<N, A, B, C>& Sw3<N, A, B, C>::operator=(const vec3& rhs) {
	float a = rhs.x, b = rhs.y, c = rhs.z;
	e[A] = a;
	e[B] = b;
	e[C] = c;
	return *this;
}

struct ivec2 {
	int x, y;
	ivec2() : x(0), y(0) {}
	ivec2(int a, int b) : x(a), y(b) {}
	explicit ivec2(const vec2& v) : x((int) v.x), y((int) v.y) {}
};
inline vec2::vec2(const ivec2& o) : x((float) o.x), y((float) o.y) {}
inline vec3::vec3(const ivec2& v, float c) : x((float) v.x), y((float) v.y), z(c) {}

struct uvec2 {
	uint x, y;
	uvec2() : x(0), y(0) {}
	uvec2(uint a, uint b) : x(a), y(b) {}
	uvec2(const ivec2& v) : x((uint) v.x), y((uint) v.y) {}
	uint& operator[](int i) { return i ? y : x; }
	uint operator[](int i) const { return i ? y : x; }
};
struct USw2 {
	uint e[4];
	operator uvec2() const { return uvec2(e[0], e[1]); }
};
struct uvec4 {
	union {
		struct { uint x, y, z, w; };
		struct { uint r, g, b, a; };
		USw2 rg;
	};
	uvec4() : x(0), y(0), z(0), w(0) {}
	explicit uvec4(uint s) : x(s), y(s), z(s), w(s) {}
	uvec4(uint a, uint b, uint c, uint d) : x(a), y(b), z(c), w(d) {}
};

// ---- scalar built-ins ----------------------------------------------------
inline float fma(float a, float b, float c) { return __builtin_fmaf(a, b, c); }
inline float abs(float x) { return rl_fabsf(x); }
inline int abs(int x) { return x < 0 ? -x : x; }
inline float max(float x, float y) { return (x < y) ? y : x; }
inline float min(float x, float y) { return (y < x) ? y : x; }
inline int max(int x, int y) { return (x < y) ? y : x; }
inline uint max(uint x, uint y) { return (x < y) ? y : x; }
inline float clamp(float x, float lo, float hi) { return min(max(x, lo), hi); }
inline float sqrt(float x) { return __builtin_sqrtf(x); }
inline float inversesqrt(float x) { return 1.0f / __builtin_sqrtf(x); }
inline float atan(float x) { return rl_atanf(x); }
inline float acos(float x) { return rl_acosf(x); }
inline float sin(float x) { return rl_sinf(x); }
inline float cos(float x) { return rl_cosf(x); }
inline float tan(float x) { return rl_sinf(x) / rl_cosf(x); }
inline float pow(float x, float y) { return __builtin_powf(x, y); }
inline float log2(float x) { return __builtin_log2f(x); }
inline float log10(float x) { return __builtin_log10f(x); }
inline float mix(float x, float y, float a) { return x * (1.0f - a) + y * a; }
inline bool isinf(float x) { return __builtin_isinf(x); }
inline bool isnan(float x) { return __builtin_isnan(x); }
inline uint floatBitsToUint(float x) { return rl_f2u(x); }
inline float uintBitsToFloat(uint u) { return rl_u2f(u); }
template <class T> inline T nonuniformEXT(T x) { return x; }

// ---- vector arithmetic ---------------------------------------------------
#define GLSL_VEC_BINOP(OP)                                                              \
	inline vec2 operator OP(const vec2& a, const vec2& b) { return vec2(a.x OP b.x, a.y OP b.y); } \
	inline vec3 operator OP(const vec3& a, const vec3& b) { return vec3(a.x OP b.x, a.y OP b.y, a.z OP b.z); } \
	inline vec4 operator OP(const vec4& a, const vec4& b) { return vec4(a.x OP b.x, a.y OP b.y, a.z OP b.z, a.w OP b.w); } \
	inline vec2 operator OP(const vec2& a, float s) { return vec2(a.x OP s, a.y OP s); }         \
	inline vec3 operator OP(const vec3& a, float s) { return vec3(a.x OP s, a.y OP s, a.z OP s); } \
	inline vec2 operator OP(float s, const vec2& a) { return vec2(s OP a.x, s OP a.y); }         \
	inline vec3 operator OP(float s, const vec3& a) { return vec3(s OP a.x, s OP a.y, s OP a.z); } \
	inline vec4 operator OP(const vec4& a, float s) { return vec4(a.x OP s, a.y OP s, a.z OP s, a.w OP s); }
GLSL_VEC_BINOP(+)
GLSL_VEC_BINOP(-)
GLSL_VEC_BINOP(*)
GLSL_VEC_BINOP(/)
#undef GLSL_VEC_BINOP
inline vec2 operator-(const vec2& a) { return vec2(-a.x, -a.y); }
inline vec3 operator-(const vec3& a) { return vec3(-a.x, -a.y, -a.z); }
inline vec2& operator+=(vec2& a, const vec2& b) { a = a + b; return a; }
inline vec3& operator+=(vec3& a, const vec3& b) { a = a + b; return a; }
inline vec2& operator-=(vec2& a, const vec2& b) { a = a - b; return a; }
inline vec3& operator-=(vec3& a, const vec3& b) { a = a - b; return a; }
inline vec2& operator*=(vec2& a, float s) { a = a * s; return a; }
inline vec3& operator*=(vec3& a, float s) { a = a * s; return a; }
inline vec3& operator*=(vec3& a, const vec3& b) { a = a * b; return a; }
inline vec3& operator/=(vec3& a, float s) { a = a / s; return a; }
inline vec3& operator+=(vec3& a, float s) { a = a + s; return a; }
inline vec3 operator*(const vec3& a, int s) { return a * (float) s; }

inline float dot(const vec2& a, const vec2& b) { return a.x * b.x + a.y * b.y; }
inline float dot(const vec3& a, const vec3& b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline float dot(const vec4& a, const vec4& b) { return a.x * b.x + a.y * b.y + a.z * b.z + a.w * b.w; }
inline float length(const vec2& a) { return sqrt(dot(a, a)); }
inline float length(const vec3& a) { return sqrt(dot(a, a)); }
inline vec2 normalize(const vec2& a) { return a * inversesqrt(dot(a, a)); }
inline vec3 normalize(const vec3& a) { return a * inversesqrt(dot(a, a)); }
inline vec3 cross(const vec3& a, const vec3& b) {
	return vec3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
inline vec2 fma(const vec2& a, const vec2& b, const vec2& c) { return vec2(fma(a.x, b.x, c.x), fma(a.y, b.y, c.y)); }
inline vec3 fma(const vec3& a, const vec3& b, const vec3& c) {
	return vec3(fma(a.x, b.x, c.x), fma(a.y, b.y, c.y), fma(a.z, b.z, c.z));
}
inline vec2 abs(const vec2& a) { return vec2(abs(a.x), abs(a.y)); }
inline vec3 abs(const vec3& a) { return vec3(abs(a.x), abs(a.y), abs(a.z)); }
inline vec3 max(const vec3& a, const vec3& b) { return vec3(max(a.x, b.x), max(a.y, b.y), max(a.z, b.z)); }
inline vec3 mix(const vec3& x, const vec3& y, float a) { return x * (1.0f - a) + y * a; }

// ---- matrices (column major, columns are vectors) -------------------------
struct mat2 {
	vec2 c[2];
	mat2() {}
	mat2(const vec2& a, const vec2& b) { c[0] = a; c[1] = b; }
	vec2& operator[](int i) { return c[i]; }
	const vec2& operator[](int i) const { return c[i]; }
};
inline float determinant(const mat2& m) { return m[0][0] * m[1][1] - m[1][0] * m[0][1]; }
inline mat2 outerProduct(const vec2& col, const vec2& row) { return mat2(col * row.x, col * row.y); }
inline mat2 operator-(const mat2& a, const mat2& b) { return mat2(a[0] - b[0], a[1] - b[1]); }
inline mat2& operator-=(mat2& a, const mat2& b) { a = a - b; return a; }
inline mat2 transpose(const mat2& m) { return mat2(vec2(m[0][0], m[1][0]), vec2(m[0][1], m[1][1])); }

struct mat3 {
	vec3 c[3];
	mat3() {}
	mat3(const vec3& a, const vec3& b, const vec3& d) { c[0] = a; c[1] = b; c[2] = d; }
	mat3(float a0, float a1, float a2, float b0, float b1, float b2, float d0, float d1, float d2) {
		c[0] = vec3(a0, a1, a2); c[1] = vec3(b0, b1, b2); c[2] = vec3(d0, d1, d2);
	}
	vec3& operator[](int i) { return c[i]; }
	const vec3& operator[](int i) const { return c[i]; }
};
inline vec3 operator*(const mat3& m, const vec3& v) { return m[0] * v.x + m[1] * v.y + m[2] * v.z; }
inline mat3 transpose(const mat3& m) {
	return mat3(vec3(m[0].x, m[1].x, m[2].x), vec3(m[0].y, m[1].y, m[2].y), vec3(m[0].z, m[1].z, m[2].z));
}
inline mat3 operator-(const mat3& m) { return mat3(-m[0], -m[1], -m[2]); }
inline float determinant(const mat3& m) { return dot(m[0], cross(m[1], m[2])); }

struct mat4x3 {
	vec3 c[4];
	mat4x3() {}
	mat4x3(const vec3& a, const vec3& b, const vec3& d, const vec3& e) { c[0] = a; c[1] = b; c[2] = d; c[3] = e; }
	vec3& operator[](int i) { return c[i]; }
	const vec3& operator[](int i) const { return c[i]; }
};
inline vec3 operator*(const mat4x3& m, const vec4& v) { return m[0] * v.x + m[1] * v.y + m[2] * v.z + m[3] * v.w; }
inline mat4x3 operator*(const mat3& a, const mat4x3& b) { return mat4x3(a * b[0], a * b[1], a * b[2], a * b[3]); }

struct mat3x4 {
	vec4 c[3];
};
inline mat3x4 transpose(const mat4x3& m) {
	mat3x4 t;
	for (int i = 0; i != 3; ++i) t.c[i] = vec4(m[0][i], m[1][i], m[2][i], m[3][i]);
	return t;
}
inline vec4 operator*(const mat3x4& m, const vec3& v) { return m.c[0] * v.x + m.c[1] * v.y + m.c[2] * v.z; }

struct mat4 {
	vec4 c[4];
};

// ---- resources the shading pass declares ----------------------------------
// LTC tables: two texture arrays sampled bilinearly with clamp-to-edge and
// nearest array layer.  Texels are FP32 (the reference stores UNORM16).
struct sampler2DArray {
	const float* texels;  // [layer][height][width][channels]
	int width, height, layers, channels;
};
inline vec4 glsl_texel(const sampler2DArray& s, int layer, int y, int x) {
	x = x < 0 ? 0 : (x >= s.width ? s.width - 1 : x);
	y = y < 0 ? 0 : (y >= s.height ? s.height - 1 : y);
	const float* t = s.texels + (((size_t) layer * s.height + y) * s.width + x) * s.channels;
	vec4 r(0.0f);
	for (int i = 0; i != s.channels; ++i) r[i] = t[i];
	return r;
}
// Bilinear filter in FP32: coordinate u*W - 0.5 split into integer and
// fraction; result = (t00*(1-fx) + t10*fx)*(1-fy) + (t01*(1-fx) + t11*fx)*fy.
inline vec4 textureLod(const sampler2DArray& s, const vec3& coord, float) {
	float layer_f = coord.z + 0.5f;
	int layer = (int) layer_f;
	layer = layer < 0 ? 0 : (layer >= s.layers ? s.layers - 1 : layer);
	float fu = coord.x * (float) s.width - 0.5f;
	float fv = coord.y * (float) s.height - 0.5f;
	float iu = __builtin_floorf(fu), iv = __builtin_floorf(fv);
	float ax = fu - iu, ay = fv - iv;
	int x0 = (int) iu, y0 = (int) iv;
	vec4 t00 = glsl_texel(s, layer, y0, x0), t10 = glsl_texel(s, layer, y0, x0 + 1);
	vec4 t01 = glsl_texel(s, layer, y0 + 1, x0), t11 = glsl_texel(s, layer, y0 + 1, x0 + 1);
	vec4 r;
	for (int i = 0; i != 4; ++i) {
		float top = t00[i] * (1.0f - ax) + t10[i] * ax;
		float bottom = t01[i] * (1.0f - ax) + t11[i] * ax;
		r[i] = top * (1.0f - ay) + bottom * ay;
	}
	return r;
}

// Resources of the visibility buffer / mesh path.  They only need to compile:
// the harness replaces get_shading_data() with a G-buffer read.
struct utextureBuffer {};
struct textureBuffer {};
struct usubpassInput {};
struct sampler2D {};
uvec4 subpassLoad(const usubpassInput&);
inline uvec4 texelFetch(const utextureBuffer&, int) { return uvec4(0u); }
inline vec4 texelFetch(const textureBuffer&, int) { return vec4(0.0f); }
inline vec4 textureGrad(const sampler2D&, const vec2&, const vec2&, const vec2&) { return vec4(0.0f); }

// Ray queries: any-hit against the harness's triangle list.
struct accelerationStructureEXT {};
struct rayQueryEXT {
	vec3 origin, direction;
	float t_min, t_max;
	bool hit;
};
enum {
	gl_RayFlagsTerminateOnFirstHitEXT = 4,
	gl_RayFlagsOpaqueEXT = 1,
	gl_RayFlagsSkipClosestHitShaderEXT = 8,
	gl_RayQueryCommittedIntersectionNoneEXT = 0,
	gl_RayQueryCommittedIntersectionTriangleEXT = 1,
};
bool glsl_shim_any_hit(const vec3& origin, const vec3& direction, float t_min, float t_max);
inline void rayQueryInitializeEXT(rayQueryEXT& q, const accelerationStructureEXT&, uint, uint, const vec3& o, float t_min,
                                  const vec3& d, float t_max) {
	q.origin = o;
	q.direction = d;
	q.t_min = t_min;
	q.t_max = t_max;
	q.hit = false;
}
inline bool rayQueryProceedEXT(rayQueryEXT& q) {
	q.hit = glsl_shim_any_hit(q.origin, q.direction, q.t_min, q.t_max);
	return false;
}
inline int rayQueryGetIntersectionTypeEXT(const rayQueryEXT& q, bool) {
	return q.hit ? gl_RayQueryCommittedIntersectionTriangleEXT : gl_RayQueryCommittedIntersectionNoneEXT;
}

// The light buffer: records every index the shader reads, so the harness can
// recover the light chosen by the reservoir (the last read after the
// candidate loop).  Out-of-range reads are clamped to the last light.
template <class T> struct GlslLightArray {
	T* lights = nullptr;
	int count = 0;
	int log[4096];
	int log_size = 0;
	T& operator[](int i) {
		if (log_size < 4096) log[log_size++] = i;
		if (i < 0) i = 0;
		if (i >= count) i = count - 1;
		return lights[i];
	}
};

// Runtime light count (the reference bakes POLYGONAL_LIGHT_COUNT into the
// shader as a define; here the define expands to this variable).
extern int g_ref_light_count;
