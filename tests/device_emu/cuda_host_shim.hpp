// Host shim for compiling the JIT kernel source with g++.  TEST INFRASTRUCTURE ONLY.
//
// The kernels are instantiated with one thread per CTA: every phase of the tile kernel
// is a loop over independent work items ("for i = threadIdx.x; i < N; i += NT"), so one
// thread doing all items in order, with barriers as no-ops, computes what the CTA does.
// This checks the kernel template's index logic and the generated rule code on the CPU;
// CUDA compilation and hardware behaviour are covered by the GPU tests.
#pragma once
#include <cmath>
#include <cstdint>
#define SE_HAVE_STDINT
#define __device__
#define __host__
#define __global__
#define __grid_constant__
#define __forceinline__ inline
#define __launch_bounds__(...)
#define __shared__
#define __align__(n)
struct se_emu_dim3 {
  unsigned x = 0, y = 0, z = 0;
};
inline se_emu_dim3 threadIdx, blockIdx, blockDim, gridDim;
inline void __syncthreads() {}
struct uint4 {
  unsigned x, y, z, w;
};
struct uint2 {
  unsigned x, y;
};
inline uint2 make_uint2(unsigned a, unsigned b) { return uint2{a, b}; }
struct int4 {
  int x, y, z, w;
};
inline uint4 make_uint4(unsigned a, unsigned b, unsigned c, unsigned d) { return uint4{a, b, c, d}; }
template <class T>
inline T __ldg(const T* p) { return *p; }
inline float __fmul_rn(float a, float b) { return a * b; }
inline float __fadd_rn(float a, float b) { return a + b; }
inline float __fsub_rn(float a, float b) { return a - b; }
inline float __fdiv_rn(float a, float b) { return a / b; }
inline float __fsqrt_rn(float x) { return std::sqrt(x); }
inline float __uint2float_rn(unsigned u) { return (float)u; }
inline float __int2float_rn(int i) { return (float)i; }
inline int __float2int_rz(float f) { return (int)f; }
inline float __uint_as_float(unsigned u) {
  float f;
  __builtin_memcpy(&f, &u, 4);
  return f;
}
inline unsigned __funnelshift_rc(unsigned lo, unsigned hi, unsigned s) {  // shift clamped to 32
  const unsigned long long v = ((unsigned long long)hi << 32) | lo;
  return (unsigned)(v >> (s > 32u ? 32u : s));
}
inline unsigned __funnelshift_r(unsigned lo, unsigned hi, unsigned s) {
  const unsigned long long v = ((unsigned long long)hi << 32) | lo;
  return (unsigned)(v >> (s & 31));
}
inline unsigned __byte_perm(unsigned x, unsigned y, unsigned s) {
  const unsigned long long v = ((unsigned long long)y << 32) | x;
  unsigned r = 0;
  for (int i = 0; i < 4; ++i) {
    const unsigned sel = (s >> (4 * i)) & 7u;
    r |= (unsigned)((v >> (8 * sel)) & 0xffu) << (8 * i);
  }
  return r;
}
// Warp operations for a warp of one thread (lane 0).
inline unsigned __ballot_sync(unsigned, bool p) { return p ? 1u : 0u; }
template <class T>
inline T __shfl_sync(unsigned, T v, int) { return v; }
template <class T>
inline T __shfl_up_sync(unsigned, T v, unsigned) { return v; }  // lane 0: its own value
inline int __popc(unsigned v) { return __builtin_popcount(v); }
inline unsigned max(unsigned a, unsigned b) { return a > b ? a : b; }
inline int __ffs(unsigned v) { return __builtin_ffs((int)v); }
inline unsigned atomicOr(unsigned* p, unsigned v) {
  const unsigned old = *p;
  *p = old | v;
  return old;
}
inline int atomicAdd(int* p, int v) {
  const int old = *p;
  *p = old + v;
  return old;
}
