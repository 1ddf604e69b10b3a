// GLSL 4.30 -> C++20 shim.  TEST INFRASTRUCTURE ONLY (oracle).
//
// Lets shader text compile as C++ after the mechanical rewrites in oracle/glsl2cpp.py:
// vector types with component-wise operators, the builtins the sandengine compute shader
// calls, fixed-size arrays with .length(), and CPU-side textures/images.
//
// Arithmetic is strict IEEE-754 binary32 (the translation unit is built with
// -ffp-contract=off and without -ffast-math): uint->float conversion rounds to nearest
// even, sqrt is correctly rounded, and pow(x, 2.0) is x*x (what shader compilers emit for
// that form).  These are the fixed semantics the GPU kernels must reproduce bit-exactly
// on the grid state.  No math-library header is included, so builtin overloads are the
// only candidates for GLSL's int->float argument conversions.
#pragma once

#include <type_traits>

typedef unsigned int uint;

static inline float se_sqrtf(float x) { return __builtin_sqrtf(x); }

struct uvec2;
struct uvec3;
struct uvec4;
struct ivec2;
struct ivec4;

struct vec2 {
  float x = 0, y = 0;
  vec2() = default;
  vec2(float a, float b) : x(a), y(b) {}
  explicit vec2(float a) : x(a), y(a) {}
  vec2(const uvec2& u);
  vec2(const ivec2& u);
};
struct vec3 {
  float x = 0, y = 0, z = 0;
  vec3() = default;
  vec3(float a, float b, float c) : x(a), y(b), z(c) {}
  explicit vec3(float a) : x(a), y(a), z(a) {}
};
struct vec4 {
  union { float x; float r; };
  union { float y; float g; };
  union { float z; float b; };
  union { float w; float a; };
  vec4() : x(0), y(0), z(0), w(0) {}
  vec4(float a_, float b_, float c_, float d_) : x(a_), y(b_), z(c_), w(d_) {}
  explicit vec4(float v) : x(v), y(v), z(v), w(v) {}
  vec4(const vec3& v, float d_) : x(v.x), y(v.y), z(v.z), w(d_) {}
  vec4(const uvec4& u);
  vec4(const ivec4& u);
  vec3 rgb() const { return vec3(x, y, z); }
  vec2 xy() const { return vec2(x, y); }
  void set_rgb(const vec3& v) { x = v.x; y = v.y; z = v.z; }  // `v.rgb = e` (glsl2cpp)
};

struct ivec2 {
  int x = 0, y = 0;
  ivec2() = default;
  ivec2(int a, int b) : x(a), y(b) {}
  explicit ivec2(const vec2& v) : x((int)v.x), y((int)v.y) {}
  explicit ivec2(const uvec2& v);
};
struct ivec4 {
  union { int x; int r; };
  union { int y; int g; };
  union { int z; int b; };
  union { int w; int a; };
  ivec4() : x(0), y(0), z(0), w(0) {}
  ivec4(int a_, int b_, int c_, int d_) : x(a_), y(b_), z(c_), w(d_) {}
  explicit ivec4(const vec4& v) : x((int)v.x), y((int)v.y), z((int)v.z), w((int)v.w) {}
};
struct uvec2 {
  uint x = 0, y = 0;
  uvec2() = default;
  uvec2(uint a, uint b) : x(a), y(b) {}
};
struct uvec3 {
  uint x = 0, y = 0, z = 0;
  uvec3() = default;
  uvec3(uint a, uint b, uint c) : x(a), y(b), z(c) {}
  uvec3(const ivec2& v, int c) : x((uint)v.x), y((uint)v.y), z((uint)c) {}
  uvec2 xy() const { return uvec2(x, y); }
};
struct uvec4 {
  uint x = 0, y = 0, z = 0, w = 0;
  uvec4() = default;
  uvec4(uint a, uint b, uint c, uint d) : x(a), y(b), z(c), w(d) {}
};

inline vec2::vec2(const uvec2& u) : x((float)u.x), y((float)u.y) {}
inline vec2::vec2(const ivec2& u) : x((float)u.x), y((float)u.y) {}
inline vec4::vec4(const uvec4& u) : x((float)u.x), y((float)u.y), z((float)u.z), w((float)u.w) {}
inline vec4::vec4(const ivec4& u) : x((float)u.x), y((float)u.y), z((float)u.z), w((float)u.w) {}
inline ivec2::ivec2(const uvec2& v) : x((int)v.x), y((int)v.y) {}

// ---- float vector arithmetic ------------------------------------------------------------
#define SE_V2(op)                                                                          \
  inline vec2 operator op(vec2 a, vec2 b) { return vec2(a.x op b.x, a.y op b.y); }       \
  inline vec2 operator op(vec2 a, float b) { return vec2(a.x op b, a.y op b); }          \
  inline vec2 operator op(float a, vec2 b) { return vec2(a op b.x, a op b.y); }
#define SE_V3(op)                                                                          \
  inline vec3 operator op(vec3 a, vec3 b) { return vec3(a.x op b.x, a.y op b.y, a.z op b.z); } \
  inline vec3 operator op(vec3 a, float b) { return vec3(a.x op b, a.y op b, a.z op b); }  \
  inline vec3 operator op(float a, vec3 b) { return vec3(a op b.x, a op b.y, a op b.z); }
#define SE_V4(op)                                                                          \
  inline vec4 operator op(vec4 a, vec4 b) {                                                \
    return vec4(a.x op b.x, a.y op b.y, a.z op b.z, a.w op b.w);                           \
  }                                                                                        \
  inline vec4 operator op(vec4 a, float b) { return vec4(a.x op b, a.y op b, a.z op b, a.w op b); } \
  inline vec4 operator op(float a, vec4 b) { return vec4(a op b.x, a op b.y, a op b.z, a op b.w); }
SE_V2(+) SE_V2(-) SE_V2(*) SE_V2(/)
SE_V3(+) SE_V3(-) SE_V3(*) SE_V3(/)
SE_V4(+) SE_V4(-) SE_V4(*) SE_V4(/)
inline vec2 operator-(vec2 a) { return vec2(-a.x, -a.y); }
inline vec2& operator+=(vec2& a, vec2 b) { a = a + b; return a; }
inline vec2& operator*=(vec2& a, float b) { a = a * b; return a; }
inline vec4& operator+=(vec4& a, vec4 b) { a = a + b; return a; }
inline vec4& operator*=(vec4& a, vec4 b) { a = a * b; return a; }
inline vec3& operator+=(vec3& a, vec3 b) { a = a + b; return a; }
inline vec4& operator/=(vec4& a, float b) { a = a / b; return a; }
inline bool operator==(vec3 a, vec3 b) { return a.x == b.x && a.y == b.y && a.z == b.z; }
inline bool operator!=(vec3 a, vec3 b) { return !(a == b); }
inline bool operator==(const vec4& a, const vec4& b) {
  return a.x == b.x && a.y == b.y && a.z == b.z && a.w == b.w;
}

// ---- int vector arithmetic (two's-complement wrap, as GLSL defines it) -------------------
inline int se_wadd(int a, int b) { return (int)((uint)a + (uint)b); }
inline int se_wsub(int a, int b) { return (int)((uint)a - (uint)b); }
inline int se_wmul(int a, int b) { return (int)((uint)a * (uint)b); }
inline ivec2 operator+(ivec2 a, ivec2 b) { return ivec2(se_wadd(a.x, b.x), se_wadd(a.y, b.y)); }
inline ivec2 operator-(ivec2 a, ivec2 b) { return ivec2(se_wsub(a.x, b.x), se_wsub(a.y, b.y)); }
inline ivec2 operator*(ivec2 a, int b) { return ivec2(se_wmul(a.x, b), se_wmul(a.y, b)); }
inline ivec2 operator/(ivec2 a, int b) { return ivec2(a.x / b, a.y / b); }
inline ivec2 operator&(ivec2 a, int b) { return ivec2(a.x & b, a.y & b); }
inline ivec2& operator+=(ivec2& a, ivec2 b) { a = a + b; return a; }
inline ivec2& operator-=(ivec2& a, ivec2 b) { a = a - b; return a; }
inline bool operator==(ivec2 a, ivec2 b) { return a.x == b.x && a.y == b.y; }

inline uvec4 operator*(uint a, uvec4 b) { return uvec4(a * b.x, a * b.y, a * b.z, a * b.w); }
inline uvec4 operator>>(uvec4 a, int s) { return uvec4(a.x >> s, a.y >> s, a.z >> s, a.w >> s); }
inline uvec4& operator^=(uvec4& a, uvec4 b) {
  a.x ^= b.x; a.y ^= b.y; a.z ^= b.z; a.w ^= b.w; return a;
}
inline uvec4& operator*=(uvec4& a, uint b) { a.x *= b; a.y *= b; a.z *= b; a.w *= b; return a; }

struct mat2 {  // column-major, as GLSL
  float c0x, c0y, c1x, c1y;
  mat2(float a, float b, float c, float d) : c0x(a), c0y(b), c1x(c), c1y(d) {}
};
inline vec2 operator*(const mat2& m, vec2 v) {
  return vec2(m.c0x * v.x + m.c1x * v.y, m.c0y * v.x + m.c1y * v.y);
}

// ---- builtins -----------------------------------------------------------------------------
inline float sqrt(float x) { return se_sqrtf(x); }
inline float pow(float x, float y) { return y == 2.0f ? x * x : __builtin_powf(x, y); }
inline float floor(float x) { return __builtin_floorf(x); }
inline vec2 floor(vec2 v) { return vec2(floor(v.x), floor(v.y)); }
inline float fract(float x) { return x - floor(x); }
inline vec2 fract(vec2 v) { return vec2(fract(v.x), fract(v.y)); }
// GLSL leaves sin's precision to the driver.  The oracle fixes it to this evaluation (the
// one the GPU colour pass makes): binary64 with Cody and Waite's argument reduction (W. J.
// Cody, W. Waite, Software Manual for the Elementary Functions, 1980; pi/2 as three 21-bit
// parts and a binary64 tail) and the Taylor series of sin (to r^17) or cos (to r^18) on
// |r| <= pi/4, rounded once to binary32: within 1 ulp of sin(x).  Compiled without
// contraction, so every operation rounds as the GPU's explicit intrinsics do.
inline float se_sin(float xf) {
  const double x = (double)xf;
  if (!(__builtin_fabs(x) < 0x1p52)) return (float)(x - x);
  if (__builtin_fabs(x) < 0x1p-12) return xf;  // sin(x) rounds to x (keeps the sign of zero)
  const double k = __builtin_floor(x * 0x1.45f306dc9c883p-1 + 0.5);
  double r = x - k * 0x1.921fb0p+0;
  r = r - k * 0x1.5110bp-22;
  r = r - k * 0x1.18469p-44;
  r = r - k * 0x1.13198a2e03707p-65;
  const double r2 = r * r;
  const double ps_c[8] = {0x1.952c77030ad4ap-49, -0x1.ae7f3e733b81fp-41, 0x1.6124613a86d09p-33,
                          -0x1.ae64567f544e4p-26, 0x1.71de3a556c734p-19, -0x1.a01a01a01a01ap-13,
                          0x1.1111111111111p-7, -0x1.5555555555555p-3};  // (-1)^n / (2n+1)!, n = 8..1
  const double pc_c[9] = {-0x1.6827863b97d97p-53, 0x1.ae7f3e733b81fp-45, -0x1.93974a8c07c9dp-37,
                          0x1.1eed8eff8d898p-29, -0x1.27e4fb7789f5cp-22, 0x1.a01a01a01a01ap-16,
                          -0x1.6c16c16c16c17p-10, 0x1.5555555555555p-5, -0.5};  // (-1)^n / (2n)!, n = 9..1
  double ps = ps_c[0];
  for (int i = 1; i < 8; ++i) ps = ps * r2 + ps_c[i];
  const double sn = r + (r * r2) * ps;
  double pc = pc_c[0];
  for (int i = 1; i < 9; ++i) pc = pc * r2 + pc_c[i];
  const double cs = 1.0 + r2 * pc;
  const double q = k - 4.0 * __builtin_floor(k * 0.25);  // k mod 4, exact
  const double v = q == 0.0 ? sn : q == 1.0 ? cs : q == 2.0 ? -sn : -cs;
  return (float)v;
}
inline float sin(float x) { return se_sin(x); }
inline vec2 sin(vec2 v) { return vec2(sin(v.x), sin(v.y)); }
inline float cos(float x) { return __builtin_cosf(x); }
inline float tan(float x) { return __builtin_tanf(x); }
inline float abs(float x) { return x < 0 ? -x : x; }
inline int abs(int x) { return x < 0 ? (int)(0u - (uint)x) : x; }
inline ivec2 abs(ivec2 v) { return ivec2(abs(v.x), abs(v.y)); }
inline float max(float a, float b) { return a < b ? b : a; }
inline vec3 max(vec3 a, float b) { return vec3(max(a.x, b), max(a.y, b), max(a.z, b)); }
inline vec4 max(vec4 a, vec4 b) { return vec4(max(a.x, b.x), max(a.y, b.y), max(a.z, b.z), max(a.w, b.w)); }
inline float min(float a, float b) { return b < a ? b : a; }
inline float clamp(float x, float lo, float hi) { return min(max(x, lo), hi); }
inline float step(float edge, float x) { return x < edge ? 0.0f : 1.0f; }
inline float dot(vec2 a, vec2 b) { return a.x * b.x + a.y * b.y; }
inline float dot(vec3 a, vec3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline float dot(vec4 a, vec4 b) { return a.x * b.x + a.y * b.y + a.z * b.z + a.w * b.w; }
inline float length(vec2 v) { return sqrt(dot(v, v)); }
inline float distance(vec2 a, vec2 b) { return length(a - b); }
inline vec3 mix(vec3 x, vec3 y, float a) { return x * (1.0f - a) + y * a; }
inline vec4 mix(vec4 x, vec4 y, float a) { return x * (1.0f - a) + y * a; }
inline float exp(float x) { return __builtin_expf(x); }
inline float log2(float x) { return __builtin_log2f(x); }
inline vec2 clamp(vec2 x, vec2 lo, vec2 hi) { return vec2(clamp(x.x, lo.x, hi.x), clamp(x.y, lo.y, hi.y)); }
inline vec3 clamp(vec3 x, vec3 lo, vec3 hi) {
  return vec3(clamp(x.x, lo.x, hi.x), clamp(x.y, lo.y, hi.y), clamp(x.z, lo.z, hi.z));
}
inline float smoothstep(float e0, float e1, float x) {  // the GLSL specification's definition
  const float t = clamp((x - e0) / (e1 - e0), 0.0f, 1.0f);
  return t * t * (3.0f - 2.0f * t);
}
inline vec2 smoothstep(vec2 e0, vec2 e1, vec2 x) {
  return vec2(smoothstep(e0.x, e1.x, x.x), smoothstep(e0.y, e1.y, x.y));
}

// ---- fixed-size arrays with GLSL's .length() ---------------------------------------------
template <class T, int N>
struct garr {
  T v[N];
  garr() = default;
  template <class... A>
    requires(!(sizeof...(A) == 1 && (std::is_same_v<std::decay_t<A>, garr> && ...)))
  garr(A... a) : v{a...} {}
  T& operator[](int i) { return v[i]; }
  const T& operator[](int i) const { return v[i]; }
  int length() const { return N; }
};

// ---- CPU textures (RGBA32F) -----------------------------------------------------------------
// The fragment stage's filtered, mipmapped samplers are oracle/frag_driver.cpp's.
#ifndef SE_GLSL_FRAGMENT
struct sampler2D {
  const float* data = nullptr;  // W*H*4 floats, row-major
  int w = 0, h = 0;
};
#endif
struct image2D {
  float* data = nullptr;
  int w = 0, h = 0;
};
struct uimage2D {
  uint* data = nullptr;
  int w = 0, h = 0;
};
#ifndef SE_GLSL_FRAGMENT
inline vec4 texelFetch(const sampler2D& s, ivec2 p, int) {
  // Out-of-range fetches return 0 (robust buffer access); the shader guards its fetches.
  if (p.x < 0 || p.y < 0 || p.x >= s.w || p.y >= s.h || !s.data) return vec4(0.0f);
  const float* t = s.data + 4 * ((long)p.y * s.w + p.x);
  return vec4(t[0], t[1], t[2], t[3]);
}
#endif
inline void imageStore(image2D& im, ivec2 p, vec4 v) {
  if (p.x < 0 || p.y < 0 || p.x >= im.w || p.y >= im.h || !im.data) return;
  float* t = im.data + 4 * ((long)p.y * im.w + p.x);
  t[0] = v.x; t[1] = v.y; t[2] = v.z; t[3] = v.w;
}
inline void imageStore(image2D& im, ivec2 p, ivec4 v) { imageStore(im, p, vec4(v)); }
inline vec4 imageLoad(image2D& im, ivec2 p) {
  if (p.x < 0 || p.y < 0 || p.x >= im.w || p.y >= im.h || !im.data) return vec4(0.0f);
  const float* t = im.data + 4 * ((long)p.y * im.w + p.x);
  return vec4(t[0], t[1], t[2], t[3]);
}
