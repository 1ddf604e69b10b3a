// Device prelude for the JIT-compiled sandengine kernels (NVRTC, sm_103a).
// Included before the generated rule code (namespace se_gen), which calls these helpers.
#pragma once

#ifndef SE_HAVE_STDINT
typedef unsigned int uint32_t;
typedef int int32_t;
typedef unsigned long long uint64_t;
typedef long long int64_t;
typedef unsigned char uint8_t;
typedef unsigned short uint16_t;
#endif

// Material ids fixed by the rule language (materials.rs:52-78): EMPTY, NULL, WALL.
#define SE_EMPTY 0u
#define SE_NULL 1u
#define SE_WALL 2u

// hash43's lanes are RN(float(u)) / float(0xffffffff) = RN(float(u)) * 2^-32 exactly
// (math.glsl:74-79; the divisor rounds to 2^32).
__device__ __forceinline__ float se_randf(uint32_t h) { return __fmul_rn(__uint2float_rn(h), 0x1p-32f); }

// Cells of type WALL or NULL never move (operations.glsl:16-23).  Only the materials
// WALL (id 2) and NULL (id 1) carry those types: user materials must name a declared
// type, and the language does not let a user type be called NULL or WALL.
__device__ __forceinline__ bool se_pinned(uint32_t m) { return (m - 1u) < 2u; }
__device__ __forceinline__ void se_swap(uint32_t& a, uint32_t& b) {
  if (!(se_pinned(a) | se_pinned(b))) {
    const uint32_t t = a;
    a = b;
    b = t;
  }
}

// GLSL integer/float helpers used by generated conditions.
__device__ __forceinline__ int se_iabs(int x) { return x < 0 ? (int)(0u - (unsigned)x) : x; }
__device__ __forceinline__ int se_min(int a, int b) { return b < a ? b : a; }
__device__ __forceinline__ int se_max(int a, int b) { return a < b ? b : a; }
__device__ __forceinline__ unsigned se_min(unsigned a, unsigned b) { return b < a ? b : a; }
__device__ __forceinline__ unsigned se_max(unsigned a, unsigned b) { return a < b ? b : a; }
__device__ __forceinline__ float se_fmin(float a, float b) { return b < a ? b : a; }
__device__ __forceinline__ float se_fmax(float a, float b) { return a < b ? b : a; }
__device__ __forceinline__ int se_idiv(int a, int b) { return b == 0 ? 0 : (b == -1 ? (int)(0u - (unsigned)a) : a / b); }
__device__ __forceinline__ unsigned se_udiv(unsigned a, unsigned b) { return b == 0u ? 0u : a / b; }
__device__ __forceinline__ int se_imod(int a, int b) { return (b == 0 || b == -1) ? 0 : a % b; }
__device__ __forceinline__ unsigned se_umod(unsigned a, unsigned b) { return b == 0u ? 0u : a % b; }
