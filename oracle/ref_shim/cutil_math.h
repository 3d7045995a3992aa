/* Self-written float2/3/4 operator set with the semantics the reference's
 * helper files rely on (component-wise IEEE single-precision operations,
 * dot = x*x' + y*y' + z*z' evaluated left to right, length = sqrtf(dot),
 * make_float3(float4) drops w, make_float4(float3) sets w = 0).
 * Oracle build only; compiled with -ffp-contract=off so every operation
 * rounds separately. */
#ifndef FG_SHIM_CUTIL_MATH_H
#define FG_SHIM_CUTIL_MATH_H
#include <cmath>
#include "vector_types.h"
#include "vector_functions.h"
using std::sqrt;

static inline float3 make_float3(float s) { return make_float3(s, s, s); }
static inline float3 make_float3(float4 a) { return make_float3(a.x, a.y, a.z); }
static inline float4 make_float4(float3 a) { return make_float4(a.x, a.y, a.z, 0.0f); }
static inline float4 make_float4(float s) { return make_float4(s, s, s, s); }

/* float3 */
static inline float3 operator+(float3 a, float3 b) { return make_float3(a.x + b.x, a.y + b.y, a.z + b.z); }
static inline float3 operator-(float3 a, float3 b) { return make_float3(a.x - b.x, a.y - b.y, a.z - b.z); }
static inline float3 operator-(float3 a) { return make_float3(-a.x, -a.y, -a.z); }
static inline float3 operator*(float3 a, float3 b) { return make_float3(a.x * b.x, a.y * b.y, a.z * b.z); }
static inline float3 operator*(float3 a, float s) { return make_float3(a.x * s, a.y * s, a.z * s); }
static inline float3 operator*(float s, float3 a) { return make_float3(s * a.x, s * a.y, s * a.z); }
static inline float3 operator/(float3 a, float s) { return make_float3(a.x / s, a.y / s, a.z / s); }
static inline void operator+=(float3 &a, float3 b) { a.x += b.x; a.y += b.y; a.z += b.z; }
static inline void operator-=(float3 &a, float3 b) { a.x -= b.x; a.y -= b.y; a.z -= b.z; }
static inline void operator*=(float3 &a, float s) { a.x *= s; a.y *= s; a.z *= s; }
static inline float dot(float3 a, float3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static inline float length(float3 v) { return sqrtf(dot(v, v)); }

/* float4 */
static inline float4 operator+(float4 a, float4 b) { return make_float4(a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w); }
static inline float4 operator-(float4 a, float4 b) { return make_float4(a.x - b.x, a.y - b.y, a.z - b.z, a.w - b.w); }
static inline float4 operator*(float4 a, float s) { return make_float4(a.x * s, a.y * s, a.z * s, a.w * s); }
static inline float4 operator*(float s, float4 a) { return make_float4(s * a.x, s * a.y, s * a.z, s * a.w); }
static inline float4 operator/(float4 a, float s) { return make_float4(a.x / s, a.y / s, a.z / s, a.w / s); }
static inline void operator+=(float4 &a, float4 b) { a.x += b.x; a.y += b.y; a.z += b.z; a.w += b.w; }
static inline void operator*=(float4 &a, float s) { a.x *= s; a.y *= s; a.z *= s; a.w *= s; }
static inline float dot(float4 a, float4 b) { return a.x * b.x + a.y * b.y + a.z * b.z + a.w * b.w; }
static inline float length(float4 v) { return sqrtf(dot(v, v)); }

#endif
