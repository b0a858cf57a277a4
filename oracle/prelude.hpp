// prelude.hpp — what the oracle includes first (test infrastructure).
//
// System headers, the C ABI's structs, and the scalar math glsl.hpp builds on,
// as overloads for float and double. The oracle's FP64 instance (VVO_FP64,
// built by oracle_api64.cpp) then defines `float` as `double`, so that the
// same restatement of the shaders computes in double precision: literals
// keep their single-precision values (the shaders' constants), texel decode
// and encode of 32-bit formats name f32 (a real 4-byte float the macro leaves
// alone), and the uniform block is converted from its std140 bytes.
#pragma once
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <thread>
#include <vector>

#include "../include/volpt.h"

typedef float f32;

#define VVO_MATH1(name, f, d) \
    inline float name(float x) { return f(x); } \
    inline double name(double x) { return d(x); }
VVO_MATH1(gl_fabs, __builtin_fabsf, __builtin_fabs)
VVO_MATH1(gl_floor, __builtin_floorf, __builtin_floor)
VVO_MATH1(gl_ceil, __builtin_ceilf, __builtin_ceil)
VVO_MATH1(gl_trunc, __builtin_truncf, __builtin_trunc)
VVO_MATH1(gl_round, __builtin_roundf, __builtin_round)
VVO_MATH1(gl_rint, __builtin_rintf, __builtin_rint)
VVO_MATH1(gl_sqrt, __builtin_sqrtf, __builtin_sqrt)
VVO_MATH1(gl_exp, __builtin_expf, __builtin_exp)
VVO_MATH1(gl_exp2, __builtin_exp2f, __builtin_exp2)
VVO_MATH1(gl_log, __builtin_logf, __builtin_log)
VVO_MATH1(gl_log2, __builtin_log2f, __builtin_log2)
VVO_MATH1(gl_sin, __builtin_sinf, __builtin_sin)
VVO_MATH1(gl_cos, __builtin_cosf, __builtin_cos)
VVO_MATH1(gl_tan, __builtin_tanf, __builtin_tan)
VVO_MATH1(gl_asin, __builtin_asinf, __builtin_asin)
VVO_MATH1(gl_acos, __builtin_acosf, __builtin_acos)
VVO_MATH1(gl_atan, __builtin_atanf, __builtin_atan)
#undef VVO_MATH1
inline float gl_pow(float x, float y) { return __builtin_powf(x, y); }
inline double gl_pow(double x, double y) { return __builtin_pow(x, y); }
inline float gl_atan2(float y, float x) { return __builtin_atan2f(y, x); }
inline double gl_atan2(double y, double x) { return __builtin_atan2(y, x); }

#ifdef VVO_FP64
#define float double
#endif
