// Host stand-ins for the CUDA intrinsics that ggdmc_gb300/csrc/device_common.cuh
// uses, so that tests/test_density32_host.py can compile its FP32 trial
// density for the CPU.  Each is the operation the intrinsic names, in host
// arithmetic (the device's approximate reciprocal, divide and exponentials
// become the correctly rounded or libm forms).
#pragma once
#include <cmath>
#include <cstdint>
#include <cstring>
#include <math.h>
#include <vector_functions.h>
#include <vector_types.h>

static inline double sinpi(double x) { return sin(M_PI * x); }
static inline float sinpif(float x) { return (float)sin(M_PI * (double)x); }
static inline float rsqrtf(float x) { return 1.0f / sqrtf(x); }
static inline float __frcp_rn(float x) { return 1.0f / x; }
static inline float __fdividef(float a, float b) { return a / b; }
// __logf: glibc declares a symbol of that name that it does not export
static inline float ggdmc_host_logf(float x) { return logf(x); }
#define __logf ggdmc_host_logf
static inline unsigned __float_as_uint(float f) { unsigned u; std::memcpy(&u, &f, 4); return u; }
static inline float __uint_as_float(unsigned u) { float f; std::memcpy(&f, &u, 4); return f; }
static inline float __int_as_float(int u) { float f; std::memcpy(&f, &u, 4); return f; }
static inline unsigned __umulhi(unsigned a, unsigned b) { return (unsigned)(((uint64_t)a * b) >> 32); }
static inline double __dmul_rn(double a, double b) { return a * b; }
static inline double __dadd_rn(double a, double b) { return a + b; }
static inline double __dsub_rn(double a, double b) { return a - b; }
static inline double __ddiv_rn(double a, double b) { return a / b; }
