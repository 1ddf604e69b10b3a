// Colour and light passes (the reference's setCell outputs other than the cell id),
// shaders/compute/operations.glsl:99-169 with math.glsl:40-44,82-106.
//
// Every float operation is an explicit round-to-nearest intrinsic in the shader's order, so
// nothing is contracted into FMAs: the light pass and the colour equal a strict-IEEE CPU
// evaluation bit for bit.  GLSL leaves the precision of sin to the driver; the colour's
// noise fixes it to se_sin (below), which the CPU oracle evaluates with the same binary64
// operations.
#include "render.hpp"

#include <algorithm>

namespace se::rt {
namespace {

__device__ __forceinline__ float fadd(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float fsub(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float fmul(float a, float b) { return __fmul_rn(a, b); }
// GLSL max / min / clamp as the spec defines them (max(a, b) = a < b ? b : a)
__device__ __forceinline__ float gmax(float a, float b) { return a < b ? b : a; }
__device__ __forceinline__ float gmin(float a, float b) { return b < a ? b : a; }
__device__ __forceinline__ float gclamp(float x, float lo, float hi) { return gmin(gmax(x, lo), hi); }

// sin of a binary32 argument: evaluated in binary64 and rounded once to binary32.
// Argument reduction by Cody and Waite's method (W. J. Cody, W. Waite, Software Manual for
// the Elementary Functions, 1980): k = the nearest integer to x * 2/pi, r = x - k * pi/2
// with pi/2 split into three 21-bit parts (k * part is exact for |k| < 2^32) and a
// binary64 tail, so r carries about 2^-100 absolute error for |x| < 2^30.  Then the Taylor
// series of sin (to r^17) or cos (to r^18) on |r| <= pi/4 (truncation below 1e-19),
// chosen and signed by k mod 4.  The result is the correctly rounded sinf(x) except when
// the binary64 value lies within about 1e-16 (relative) of a rounding boundary; it is
// within 1 ulp of sin(x), inside CUDA's documented 2-ulp bound for sinf.  Every operation
// is an explicit round-to-nearest binary64 intrinsic (no contraction), so the CPU oracle's
// restatement gives the same bits.  |x| < 2^-12 gives x (the correctly rounded value);
// |x| >= 2^52 (never met: the noise's arguments stay below 2^30) gives x - x (NaN for
// infinities and NaN, else 0).
__device__ __forceinline__ float se_sin(float xf) {
  const double x = (double)xf;
  if (!(fabs(x) < 0x1p52)) return (float)__dsub_rn(x, x);
  if (fabs(x) < 0x1p-12) return xf;  // sin(x) rounds to x (keeps the sign of zero)
  const double k = floor(__dadd_rn(__dmul_rn(x, 0x1.45f306dc9c883p-1), 0.5));
  double r = __dsub_rn(x, __dmul_rn(k, 0x1.921fb0p+0));
  r = __dsub_rn(r, __dmul_rn(k, 0x1.5110bp-22));
  r = __dsub_rn(r, __dmul_rn(k, 0x1.18469p-44));
  r = __dsub_rn(r, __dmul_rn(k, 0x1.13198a2e03707p-65));
  const double r2 = __dmul_rn(r, r);
  // Taylor coefficients (-1)^n / (2n+1)! and (-1)^n / (2n)!, rounded to binary64
  double ps = 0x1.952c77030ad4ap-49;                       // 1/17!
  ps = __dadd_rn(__dmul_rn(ps, r2), -0x1.ae7f3e733b81fp-41);  // -1/15!
  ps = __dadd_rn(__dmul_rn(ps, r2), 0x1.6124613a86d09p-33);   // 1/13!
  ps = __dadd_rn(__dmul_rn(ps, r2), -0x1.ae64567f544e4p-26);  // -1/11!
  ps = __dadd_rn(__dmul_rn(ps, r2), 0x1.71de3a556c734p-19);   // 1/9!
  ps = __dadd_rn(__dmul_rn(ps, r2), -0x1.a01a01a01a01ap-13);  // -1/7!
  ps = __dadd_rn(__dmul_rn(ps, r2), 0x1.1111111111111p-7);    // 1/5!
  ps = __dadd_rn(__dmul_rn(ps, r2), -0x1.5555555555555p-3);   // -1/3!
  const double sn = __dadd_rn(r, __dmul_rn(__dmul_rn(r, r2), ps));
  double pc = -0x1.6827863b97d97p-53;                      // -1/18!
  pc = __dadd_rn(__dmul_rn(pc, r2), 0x1.ae7f3e733b81fp-45);   // 1/16!
  pc = __dadd_rn(__dmul_rn(pc, r2), -0x1.93974a8c07c9dp-37);  // -1/14!
  pc = __dadd_rn(__dmul_rn(pc, r2), 0x1.1eed8eff8d898p-29);   // 1/12!
  pc = __dadd_rn(__dmul_rn(pc, r2), -0x1.27e4fb7789f5cp-22);  // -1/10!
  pc = __dadd_rn(__dmul_rn(pc, r2), 0x1.a01a01a01a01ap-16);   // 1/8!
  pc = __dadd_rn(__dmul_rn(pc, r2), -0x1.6c16c16c16c17p-10);  // -1/6!
  pc = __dadd_rn(__dmul_rn(pc, r2), 0x1.5555555555555p-5);    // 1/4!
  pc = __dadd_rn(__dmul_rn(pc, r2), -0.5);                    // -1/2!
  const double cs = __dadd_rn(1.0, __dmul_rn(r2, pc));
  const double q = __dsub_rn(k, __dmul_rn(4.0, floor(__dmul_rn(k, 0.25))));  // k mod 4, exact
  const double v = q == 0.0 ? sn : q == 1.0 ? cs : q == 2.0 ? -sn : -cs;
  return __double2float_rn(v);
}

// old_hash2 component: -1 + 2 * fract(sin(q) * 43758.5453123)
__device__ __forceinline__ float grad_component(float q) {
  const float v = fmul(se_sin(q), 43758.5453123f);
  return fadd(-1.0f, fmul(2.0f, fsub(v, floorf(v))));
}
__device__ __forceinline__ void grad(float qx, float qy, float& gx, float& gy) {
  gx = grad_component(fadd(fmul(qx, 127.1f), fmul(qy, 311.7f)));
  gy = grad_component(fadd(fmul(qx, 269.5f), fmul(qy, 183.3f)));
}

// _noise: 2D simplex noise
__device__ float simplex(float px, float py) {
  const float K1 = 0.366025404f, K2 = 0.211324865f;
  const float s = fmul(fadd(px, py), K1);
  const float ix = floorf(fadd(px, s)), iy = floorf(fadd(py, s));
  const float t = fmul(fadd(ix, iy), K2);
  const float ax = fadd(fsub(px, ix), t), ay = fadd(fsub(py, iy), t);
  const float m = ax < ay ? 0.0f : 1.0f;  // step(a.y, a.x)
  const float ox = m, oy = fsub(1.0f, m);
  const float bx = fadd(fsub(ax, ox), K2), by = fadd(fsub(ay, oy), K2);
  const float c2 = fmul(2.0f, K2);
  const float cx = fadd(fsub(ax, 1.0f), c2), cy = fadd(fsub(ay, 1.0f), c2);
  const float h0 = gmax(fsub(0.5f, fadd(fmul(ax, ax), fmul(ay, ay))), 0.0f);
  const float h1 = gmax(fsub(0.5f, fadd(fmul(bx, bx), fmul(by, by))), 0.0f);
  const float h2 = gmax(fsub(0.5f, fadd(fmul(cx, cx), fmul(cy, cy))), 0.0f);
  float g0x, g0y, g1x, g1y, g2x, g2y;
  grad(ix, iy, g0x, g0y);
  grad(fadd(ix, ox), fadd(iy, oy), g1x, g1y);
  grad(fadd(ix, 1.0f), fadd(iy, 1.0f), g2x, g2y);
  const float n0 = fmul(fmul(fmul(fmul(h0, h0), h0), h0), fadd(fmul(ax, g0x), fmul(ay, g0y)));
  const float n1 = fmul(fmul(fmul(fmul(h1, h1), h1), h1), fadd(fmul(bx, g1x), fmul(by, g1y)));
  const float n2 = fmul(fmul(fmul(fmul(h2, h2), h2), h2), fadd(fmul(cx, g2x), fmul(cy, g2y)));
  return fadd(0.25f, fmul(0.5f, fadd(fadd(fmul(n0, 70.0f), fmul(n1, 70.0f)), fmul(n2, 70.0f))));
}

// The 2D kernels take their row blocks from by0 + blockIdx.y: a tall world is covered by
// several launches, as a grid's y extent stops at 65535.
__global__ void __launch_bounds__(256) se_noise_kernel(float* __restrict__ out, int W, int H, int by0) {
  const int x = blockIdx.x * 32 + (threadIdx.x & 31), y = (by0 + blockIdx.y) * 8 + (threadIdx.x >> 5);
  if (x >= W || y >= H) return;
  float px = (float)x, py = (float)y, f = 0.0f;
  for (int o = 1; o < 4; ++o) {  // noise(p, 3 octaves, lacunarity 2, frequency 0.25)
    f = fadd(f, fmul(__fdiv_rn(1.0f, (float)o), simplex(fmul(px, 0.25f), fmul(py, 0.25f))));
    px = fmul(px, 2.0f);
    py = fmul(py, 2.0f);
  }
  out[(size_t)y * W + x] = f;
}

__device__ __forceinline__ uint32_t mat_index(uint32_t id, int nmat) { return id < (uint32_t)nmat ? id : 1u; }

// One cell per thread, grid-stride: id, cached noise -> RGBA32F.
__global__ void __launch_bounds__(256) se_color_kernel(const uint32_t* __restrict__ grid,
                                                       const float* __restrict__ noise, float4* __restrict__ out,
                                                       long long n, const RenderMat* __restrict__ mats, int nmat) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    const uint32_t m = mat_index(__ldg(grid + i), nmat);
    const RenderMat* r = mats + m;
    float4 c = make_float4(__ldg(r->color + 0), __ldg(r->color + 1), __ldg(r->color + 2), __ldg(r->color + 3));
    if (__ldg(&r->flags) & kRenderNoise) {
      const float d = fmul(__ldg(noise + i), 0.25f);
      c.x = gclamp(fsub(c.x, d), 0.0f, 1.0f);
      c.y = gclamp(fsub(c.y, d), 0.0f, 1.0f);
      c.z = gclamp(fsub(c.z, d), 0.0f, 1.0f);
    }
    out[i] = c;
  }
}

// The colour of one cell and its alpha.
__device__ __forceinline__ float4 cell_color(uint32_t id, float nz, const RenderMat* __restrict__ mats, int nmat) {
  const RenderMat* r = mats + mat_index(id, nmat);
  float4 c = make_float4(__ldg(r->color + 0), __ldg(r->color + 1), __ldg(r->color + 2), __ldg(r->color + 3));
  if (__ldg(&r->flags) & kRenderNoise) {
    const float d = fmul(nz, 0.25f);
    c.x = gclamp(fsub(c.x, d), 0.0f, 1.0f);
    c.y = gclamp(fsub(c.y, d), 0.0f, 1.0f);
    c.z = gclamp(fsub(c.z, d), 0.0f, 1.0f);
  }
  return c;
}

// Thread = cells (2x, 2y) .. (2x + 1, 2y + 1): their colours, and (alpha1 != null, x < dw,
// y < dh) the level-1 alpha ((a00 + a10) + a01 + a11) * 0.25 in the mip kernel's order.
// At an odd last row or column the pair's second index is clamped, as the mip's is.
__global__ void __launch_bounds__(256) se_color_mip_kernel(const uint32_t* __restrict__ grid,
                                                           const float* __restrict__ noise, float4* __restrict__ out,
                                                           float* __restrict__ alpha1, int W, int H, int dw, int dh,
                                                           const RenderMat* __restrict__ mats, int nmat, int by0) {
  const int x = blockIdx.x * 32 + (threadIdx.x & 31), y = (by0 + blockIdx.y) * 8 + (threadIdx.x >> 5);
  const int c0 = 2 * x, r0 = 2 * y;
  if (c0 >= W || r0 >= H) return;
  const bool pair = c0 + 1 < W;
  float a[2][2];
#pragma unroll
  for (int dr = 0; dr < 2; ++dr) {
    const int r = min(r0 + dr, H - 1);
    const size_t i = (size_t)r * W + c0;
    uint32_t id0, id1;
    float n0, n1;
    if (pair && (W & 1) == 0) {  // 8-byte aligned pairs
      const uint2 g = __ldg(reinterpret_cast<const uint2*>(grid + i));
      const float2 z = __ldg(reinterpret_cast<const float2*>(noise + i));
      id0 = g.x, id1 = g.y, n0 = z.x, n1 = z.y;
    } else {
      id0 = __ldg(grid + i), n0 = __ldg(noise + i);
      id1 = pair ? __ldg(grid + i + 1) : id0;
      n1 = pair ? __ldg(noise + i + 1) : n0;
    }
    const float4 k0 = cell_color(id0, n0, mats, nmat), k1 = cell_color(id1, n1, mats, nmat);
    if (r == r0 + dr) {
      out[i] = k0;
      if (pair) out[i + 1] = k1;
    }
    a[dr][0] = k0.w;
    a[dr][1] = k1.w;
  }
  if (alpha1 && x < dw && y < dh)
    alpha1[(size_t)y * dw + x] = fmul(fadd(fadd(fadd(a[0][0], a[0][1]), a[1][0]), a[1][1]), 0.25f);
}

// Light pass over a 64 x 16 tile per CTA.  The tile plus a one-cell ring is staged in
// shared memory as each cell's contribution to its neighbours' blend,
// (rgb * keep * a, a) for its previous light (rgb, a), where keep is 0 when its old cell is a
// light obstacle, else 1; plus a byte that marks cells outside the world.
// Thread t computes the cells (t % 64, t / 64 + 4 j), j < 4: a warp touches 32 consecutive
// cells of a row, so shared-memory reads and global loads / stores are contiguous.
constexpr int LTW = 64, LTH = 16, LSW = LTW + 2, LSH = LTH + 2;

// GLSL max (a < b ? b : a).  CLEAN: neither argument is NaN or -0, where the hardware
// maximum returns the same value in one instruction instead of a compare and a select.
template <bool CLEAN>
__device__ __forceinline__ float lmax(float a, float b) {
  return CLEAN ? fmaxf(a, b) : gmax(a, b);
}

// The 8-neighbour blend for the staged cell s0.  INTERIOR: all 8 neighbours lie in the
// world (no checks; the mean's division by 8 is the product by 0.125, the same correctly
// rounded quotient).  CLEAN: every staged value is a non-negative number or +inf (so are
// the running maxima, which start at +0).
template <bool INTERIOR, bool CLEAN>
__device__ __forceinline__ float4 light_blend(const float4* sl, const uint8_t* sk, int s0) {
  // neighbours in getDiagonalNeighbours order: DOWN, UP, DOWNLEFT, UPLEFT, DOWNRIGHT,
  // UPRIGHT, RIGHT, LEFT (offsets in the staged array)
  constexpr int NOFF[8] = {LSW, -LSW, LSW - 1, -LSW - 1, LSW + 1, -LSW + 1, 1, -1};
  float a0 = 0.0f, a1 = 0.0f, a2 = 0.0f, a3 = 0.0f, m0 = 0.0f, m1 = 0.0f, m2 = 0.0f, maxf = 0.0f;
  int num = 0;
#pragma unroll
  for (int n = 0; n < 8; ++n) {
    const int s = s0 + NOFF[n];
    if (!INTERIOR && sk[s]) continue;  // outside the world
    const float4 c = sl[s];
    const float t0 = c.x, t1 = c.y, t2 = c.z, a = c.w;
    const float falloff = a == 0.0f ? maxf : a;
    a0 = fadd(a0, t0);
    a1 = fadd(a1, t1);
    a2 = fadd(a2, t2);
    a3 = fadd(a3, falloff);
    // clean: a == 0 leaves maxf (>= +0) as it is either way, so the running maximum need
    // not wait for the falloff select
    maxf = CLEAN ? fmaxf(a, maxf) : gmax(falloff, maxf);
    ++num;
    m0 = lmax<CLEAN>(m0, t0);  // the alpha of the maximum is not used (mix takes .rgb)
    m1 = lmax<CLEAN>(m1, t1);
    m2 = lmax<CLEAN>(m2, t2);
  }
  if (INTERIOR) {
    a0 = fmul(a0, 0.125f);
    a1 = fmul(a1, 0.125f);
    a2 = fmul(a2, 0.125f);
    a3 = fmul(a3, 0.125f);
  } else if (num > 0) {
    const float fn = (float)num;
    a0 = __fdiv_rn(a0, fn);
    a1 = __fdiv_rn(a1, fn);
    a2 = __fdiv_rn(a2, fn);
    a3 = __fdiv_rn(a3, fn);
  }
  // mix(avg.rgb, max.rgb, 0.5) = avg * (1 - 0.5) + max * 0.5
  return make_float4(fadd(fmul(a0, 0.5f), fmul(m0, 0.5f)), fadd(fmul(a1, 0.5f), fmul(m1, 0.5f)),
                     fadd(fmul(a2, 0.5f), fmul(m2, 0.5f)), a3);
}

// TALL: the row blocks start at by0 (a world with more than 65535 of them takes several
// launches); otherwise by0 is 0 and unused, which keeps the common kernel's code as tight
// as it measured best.
template <bool TALL>
__global__ void __launch_bounds__(256, 5) se_light_kernel(const uint32_t* __restrict__ old_grid,
                                                       const uint32_t* __restrict__ new_grid,
                                                       const float4* __restrict__ lin, float4* __restrict__ lout,
                                                       int W, int H, const RenderMat* __restrict__ mats, int nmat,
                                                       int by0) {
  constexpr int NT = 256, NS = LSW * LSH, NU = (NS + NT - 1) / NT;
  __shared__ float4 sl[NS];  // contribution (rgb * keep * a, a) per staged cell
  __shared__ uint8_t sk[NS];  // 1: outside the world
  const int X0 = blockIdx.x * LTW, Y0 = (TALL ? by0 + (int)blockIdx.y : (int)blockIdx.y) * LTH;
  // Issue every global load of this thread first (staged ids and light, then the new ids
  // of its four cells), so that they are in flight together.
  uint32_t ids[NU];
  float4 ls[NU];
  bool in[NU];
#pragma unroll
  for (int u = 0; u < NU; ++u) {
    const int i = threadIdx.x + u * NT;
    const int r = i / LSW, c = i - r * LSW;
    const int gx = X0 - 1 + c, gy = Y0 - 1 + r;
    in[u] = i < NS && gx >= 0 && gy >= 0 && gx < W && gy < H;
    if (in[u]) {
      const size_t q = (size_t)gy * W + gx;
      ids[u] = __ldg(old_grid + q);
      ls[u] = __ldg(lin + q);
    }
  }
  const int cx = threadIdx.x & 63;
  uint32_t nid[4];
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    const int x = X0 + cx, y = Y0 + (threadIdx.x >> 6) + 4 * j;
    nid[j] = (x < W && y < H) ? __ldg(new_grid + (size_t)y * W + x) : 0u;
  }
  uint32_t top = 0;  // the largest bit pattern staged by this thread
#pragma unroll
  for (int u = 0; u < NU; ++u) {
    const int i = threadIdx.x + u * NT;
    if (i >= NS) break;
    if (in[u]) {
      const float keep = (__ldg(&mats[mat_index(ids[u], nmat)].flags) & kRenderObstacle) ? 0.0f : 1.0f;
      const float4 l = ls[u];
      // light_data = light * vec4(vec3(keep), 1.0); contribution = (light_data.rgb * a, a)
      const float4 c =
          make_float4(fmul(fmul(l.x, keep), l.w), fmul(fmul(l.y, keep), l.w), fmul(fmul(l.z, keep), l.w), l.w);
      sl[i] = c;
      sk[i] = 0;
      top = max(top, max(max(__float_as_uint(c.x), __float_as_uint(c.y)),
                         max(__float_as_uint(c.z), __float_as_uint(c.w))));
    } else {
      sl[i] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
      sk[i] = 1;
    }
  }
  // Patterns up to 0x7f800000 are +0 .. +inf: no NaN, no -0 (nor any negative value).
  const bool clean = !__syncthreads_or(top > 0x7f800000u);
  const bool interior = X0 >= 1 && Y0 >= 1 && X0 + LTW + 1 <= W && Y0 + LTH + 1 <= H;
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    const int cy = (threadIdx.x >> 6) + 4 * j;
    const int x = X0 + cx, y = Y0 + cy;
    if (x >= W || y >= H) continue;
    const RenderMat* nm = mats + mat_index(nid[j], nmat);
    float4 L;
    if (__ldg(&nm->flags) & kRenderEmits) {
      L = make_float4(__ldg(nm->emission + 0), __ldg(nm->emission + 1), __ldg(nm->emission + 2),
                      __ldg(nm->emission + 3));
    } else if (y == 0) {
      L = make_float4(1.0f, 1.0f, 1.0f, 0.999999f);
    } else {
      const int s0 = (cy + 1) * LSW + cx + 1;
      if (clean)
        L = interior ? light_blend<true, true>(sl, sk, s0) : light_blend<false, true>(sl, sk, s0);
      else
        L = interior ? light_blend<true, false>(sl, sk, s0) : light_blend<false, false>(sl, sk, s0);
    }
    lout[(size_t)y * W + x] = L;
  }
}

// ---- headless composite ---------------------------------------------------------------
__device__ __forceinline__ int mirror_index(int i, int n) {  // GL_MIRRORED_REPEAT on texel indices
  if ((unsigned)i < (unsigned)n) return i;  // almost every tap
  if (i == -1) return 0;
  if (i == n) return n - 1;
  const int p = 2 * n;
  int m = i % p;
  if (m < 0) m += p;
  return m >= n ? p - 1 - m : m;
}
__device__ __forceinline__ float4 tap(const float4* t, int w, int h, int i, int j) {
  return __ldg(t + (size_t)mirror_index(j, h) * w + mirror_index(i, w));
}
__device__ __forceinline__ float lerp4(float t00, float t10, float t01, float t11, float w00, float w10, float w01,
                                       float w11) {
  return fadd(fadd(fadd(fmul(t00, w00), fmul(t10, w10)), fmul(t01, w01)), fmul(t11, w11));
}
__device__ float4 sample_linear(const float4* t, int w, int h, float u, float v) {
  const float x = fsub(fmul(u, (float)w), 0.5f), y = fsub(fmul(v, (float)h), 0.5f);
  const float fx = floorf(x), fy = floorf(y);
  const float a = fsub(x, fx), b = fsub(y, fy);
  const int i = (int)fx, j = (int)fy;
  float4 t00, t10, t01, t11;
  if ((unsigned)i < (unsigned)(w - 1) && (unsigned)j < (unsigned)(h - 1)) {  // all four taps inside: no wrap
    const float4* p = t + (size_t)j * w + i;
    t00 = __ldg(p), t10 = __ldg(p + 1), t01 = __ldg(p + w), t11 = __ldg(p + w + 1);
  } else {
    t00 = tap(t, w, h, i, j), t10 = tap(t, w, h, i + 1, j), t01 = tap(t, w, h, i, j + 1),
    t11 = tap(t, w, h, i + 1, j + 1);
  }
  const float w00 = fmul(fsub(1.0f, a), fsub(1.0f, b)), w10 = fmul(a, fsub(1.0f, b)), w01 = fmul(fsub(1.0f, a), b),
              w11 = fmul(a, b);
  return make_float4(lerp4(t00.x, t10.x, t01.x, t11.x, w00, w10, w01, w11),
                     lerp4(t00.y, t10.y, t01.y, t11.y, w00, w10, w01, w11),
                     lerp4(t00.z, t10.z, t01.z, t11.z, w00, w10, w01, w11),
                     lerp4(t00.w, t10.w, t01.w, t11.w, w00, w10, w01, w11));
}
// One channel of a texture whose texel (i, j) is t[S * (j * w + i)]: S = 4 reads the
// alpha of an RGBA level, S = 1 an alpha level.  4-byte taps.
template <int S>
__device__ __forceinline__ float tap_a(const float* t, int w, int h, int i, int j) {
  return __ldg(t + (size_t)S * ((size_t)mirror_index(j, h) * w + mirror_index(i, w)));
}
template <int S>
__device__ float sample_linear_a(const float* t, int w, int h, float u, float v) {
  const float x = fsub(fmul(u, (float)w), 0.5f), y = fsub(fmul(v, (float)h), 0.5f);
  const float fx = floorf(x), fy = floorf(y);
  const float a = fsub(x, fx), b = fsub(y, fy);
  const int i = (int)fx, j = (int)fy;
  float t00, t10, t01, t11;
  if ((unsigned)i < (unsigned)(w - 1) && (unsigned)j < (unsigned)(h - 1)) {  // all four taps inside: no wrap
    const float* p = t + (size_t)S * ((size_t)j * w + i);
    t00 = __ldg(p), t10 = __ldg(p + S), t01 = __ldg(p + (size_t)S * w), t11 = __ldg(p + (size_t)S * w + S);
  } else {
    t00 = tap_a<S>(t, w, h, i, j), t10 = tap_a<S>(t, w, h, i + 1, j), t01 = tap_a<S>(t, w, h, i, j + 1),
    t11 = tap_a<S>(t, w, h, i + 1, j + 1);
  }
  const float w00 = fmul(fsub(1.0f, a), fsub(1.0f, b)), w10 = fmul(a, fsub(1.0f, b)), w01 = fmul(fsub(1.0f, a), b),
              w11 = fmul(a, b);
  return lerp4(t00, t10, t01, t11, w00, w10, w01, w11);
}
// sampleBlurred(tex, uv, radius, gamma).a with lod = log2(radius), from its three textureLod
// samples at lod - 1, lod, lod + 1: weights exp(-gamma * (lod - i)^2) = w_side, 1, w_side.
__device__ __forceinline__ float blurred_alpha(float lo, float mid, float hi, float w_side) {
  float acc = fadd(0.0f, fmul(lo, w_side));
  acc = fadd(acc, fmul(mid, 1.0f));
  acc = fadd(acc, fmul(hi, w_side));
  return __fdiv_rn(acc, fadd(fadd(fadd(0.0f, w_side), 1.0f), w_side));
}

__global__ void __launch_bounds__(256) se_mip_alpha_kernel(const float* __restrict__ src, int sw, int sh,
                                                           float* __restrict__ dst, int dw, int dh, int by0) {
  const int x = blockIdx.x * 32 + (threadIdx.x & 31), y = (by0 + blockIdx.y) * 8 + (threadIdx.x >> 5);
  if (x >= dw || y >= dh) return;
  const int x0 = min(2 * x, sw - 1), x1 = min(2 * x + 1, sw - 1), y0 = min(2 * y, sh - 1), y1 = min(2 * y + 1, sh - 1);
  const float a = __ldg(src + (size_t)y0 * sw + x0), b = __ldg(src + (size_t)y0 * sw + x1),
              c = __ldg(src + (size_t)y1 * sw + x0), d = __ldg(src + (size_t)y1 * sw + x1);
  dst[(size_t)y * dw + x] = fmul(fadd(fadd(fadd(a, b), c), d), 0.25f);
}

// The part of a fragment that depends only on the pixelated coordinate (pu, pv): the
// clamped light and the occlusion.
struct Shared {
  float lr, lg, lb, occ;
};
__device__ Shared shared_terms(const CompositeSrc& m, const float4* __restrict__ light, float pu, float pv, float ws0,
                               float ws1, float ws2) {
  float4 li = light ? sample_linear(light, m.w, m.h, pu, pv) : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
  // The three sampleBlurred calls (lod 1, 4, 5) take textureLod at lods 0..2, 3..5 and 4..6:
  // seven distinct samples.  lod 0 is a magnification (level 0, nearest); lod l >= 1 reads
  // the alpha level in slot l, bilinearly.
  const float s0 = tap_a<4>(&m.color->w, m.w, m.h, (int)floorf(fmul(pu, (float)m.w)), (int)floorf(fmul(pv, (float)m.h)));
  float s[kOccLods];
#pragma unroll
  for (int l = 1; l < kOccLods; ++l) s[l] = sample_linear_a<1>(m.alpha[l], m.aw[l], m.ah[l], pu, pv);
  float occ = fsub(1.0f, blurred_alpha(s0, s[1], s[2], ws0));
  const float occ2 = fsub(1.0f, blurred_alpha(s[3], s[4], s[5], ws1));
  const float occ3 = fsub(1.0f, blurred_alpha(s[4], s[5], s[6], ws2));
  occ = gclamp(fadd(occ, fadd(fmul(occ2, 0.4f), fmul(occ3, 0.25f))), 0.0f, 1.0f);
  return Shared{gclamp(li.x, 0.0f, 1.0f), gclamp(li.y, 0.0f, 1.0f), gclamp(li.z, 0.0f, 1.0f), occ};
}

// Thread = 2 x 2 pixels (columns 2k, 2k + 1 share pu; rows share pv when W <= H, else
// the shared terms are computed per row).
__device__ __forceinline__ int coords_len(int n) { return (n + 4) & ~3; }  // round_up(n + 1, 4)

// The column and row tables (uv, pixelated uv, nearest texel): one thread per column / row.
// d = 1 / pixelate with pixelate = W / 2, as the fragment computes them.
__global__ void __launch_bounds__(256) se_composite_coords_kernel(float* __restrict__ u, int* __restrict__ ix,
                                                                  float* __restrict__ pu, float* __restrict__ v,
                                                                  int* __restrict__ iy, float* __restrict__ pv,
                                                                  int W, int H, float d) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t < coords_len(W)) {
    const float ut = __fdiv_rn(fadd((float)t, 0.5f), (float)W);
    u[t] = t < W ? ut : 0.0f;
    ix[t] = t < W ? mirror_index((int)floorf(fmul(ut, (float)W)), W) : 0;
    // column pair t: its even column 2t (column 2t + 1 pixelates to the same u)
    const float ue = __fdiv_rn(fadd((float)(2 * t), 0.5f), (float)W);
    pu[t] = 2 * t < W ? fmul(floorf(__fdiv_rn(ue, d)), d) : 0.0f;
  }
  if (t < coords_len(H)) {
    const float vt = __fdiv_rn(fadd((float)t, 0.5f), (float)H);
    v[t] = t < H ? vt : 0.0f;
    iy[t] = t < H ? mirror_index((int)floorf(fmul(vt, (float)H)), H) : 0;
    pv[t] = t < H ? fmul(floorf(__fdiv_rn(vt, d)), d) : 0.0f;
  }
}

__global__ void __launch_bounds__(256, 4) se_composite_kernel(const CompositeSrc m, const CompositeCoords cc,
                                                           const float4* __restrict__ light,
                                                           const float4* __restrict__ bg, int bw, int bh, float ws0,
                                                           float ws1, float ws2, float4* __restrict__ out, int by0) {
  const int W = m.w, H = m.h;
  const int c0 = 2 * (blockIdx.x * 32 + (threadIdx.x & 31)), r0 = 2 * ((by0 + blockIdx.y) * 8 + (threadIdx.x >> 5));
  if (c0 >= W || r0 >= H) return;
  // c0 and r0 are even: 8-byte aligned pair loads, in bounds up to index W / H
  const float2 us = __ldg(reinterpret_cast<const float2*>(cc.u + c0));
  const int2 ixs = __ldg(reinterpret_cast<const int2*>(cc.ix + c0));
  const float pu = __ldg(cc.pu + (c0 >> 1));
  const float2 vs = __ldg(reinterpret_cast<const float2*>(cc.v + r0));
  const int2 iys = __ldg(reinterpret_cast<const int2*>(cc.iy + r0));
  const float2 pv2 = __ldg(reinterpret_cast<const float2*>(cc.pv + r0));
  const float pvs[2] = {pv2.x, pv2.y};
  Shared sh[2];
#pragma unroll
  for (int dr = 0; dr < 2; ++dr) {
    if (r0 + dr >= H) break;
    sh[dr] = (dr == 1 && pvs[1] == pvs[0]) ? sh[0] : shared_terms(m, light, pu, pvs[dr], ws0, ws1, ws2);
  }
  const float ambient = 0.1f;
#pragma unroll
  for (int dr = 0; dr < 2; ++dr) {
    const int r = r0 + dr;
    if (r >= H) break;
    const float v = dr ? vs.y : vs.x;
    const int ty = dr ? iys.y : iys.x;
    const Shared& S = sh[dr];
    const float sky = fmul(0.5f, fsub(1.0f, pvs[dr]));
    const float shade = fadd(ambient, fmul(S.occ, fsub(1.0f, ambient)));
    const float base = fadd(ambient, sky);
#pragma unroll
    for (int dc = 0; dc < 2; ++dc) {
      const int cx = c0 + dc;
      if (cx >= W) break;
      const float u = dc ? us.y : us.x;
      // texture(color_tex, uv, 0.0): a magnification, the nearest texel
      float4 col = __ldg(m.color + (size_t)ty * W + (dc ? ixs.y : ixs.x));
      col.x = gclamp(fmul(col.x, shade), 0.0f, 1.0f);
      col.y = gclamp(fmul(col.y, shade), 0.0f, 1.0f);
      col.z = gclamp(fmul(col.z, shade), 0.0f, 1.0f);
      const float4 b = bg ? sample_linear(bg, bw, bh, u, fsub(1.0f, v)) : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
      const float ia = fsub(1.0f, col.w);
      float4 o;  // mix(bg, col, col.a) * vec4(ambient + sky + light, 1.0)
      o.x = fmul(fadd(fmul(b.x, ia), fmul(col.x, col.w)), fadd(base, S.lr));
      o.y = fmul(fadd(fmul(b.y, ia), fmul(col.y, col.w)), fadd(base, S.lg));
      o.z = fmul(fadd(fmul(b.z, ia), fmul(col.z, col.w)), fadd(base, S.lb));
      o.w = fmul(fadd(fmul(b.w, ia), fmul(col.w, col.w)), 1.0f);
      out[(size_t)r * W + cx] = o;
    }
  }
}

// Launches fn(by0, n) for the row blocks [by0, by0 + n) of a 2D grid, n <= 65535.
template <class F>
void for_row_blocks(int blocks, F&& fn) {
  for (int by0 = 0; by0 < blocks; by0 += 65535) fn(by0, (unsigned)std::min(65535, blocks - by0));
}

}  // namespace

cudaError_t render_mip_alpha(const float* src, int sw, int sh, float* dst, cudaStream_t s) {
  const int dw = mip_next(sw), dh = mip_next(sh);
  for_row_blocks((dh + 7) / 8, [&](int by0, unsigned n) {
    se_mip_alpha_kernel<<<dim3((unsigned)((dw + 31) / 32), n), 256, 0, s>>>(src, sw, sh, dst, dw, dh, by0);
  });
  return cudaGetLastError();
}

cudaError_t render_color_mip(const uint32_t* grid, const float* noise, float4* out, float* alpha1, int W, int H,
                             const RenderMat* mats, int nmat, cudaStream_t s) {
  const int tx = (W + 1) / 2, ty = (H + 1) / 2;
  for_row_blocks((ty + 7) / 8, [&](int by0, unsigned n) {
    se_color_mip_kernel<<<dim3((unsigned)((tx + 31) / 32), n), 256, 0, s>>>(grid, noise, out, alpha1, W, H,
                                                                            mip_next(W), mip_next(H), mats, nmat, by0);
  });
  return cudaGetLastError();
}

size_t composite_coords_bytes(int W, int H) {
  return sizeof(float) * 3 * ((size_t)((W + 4) & ~3) + (size_t)((H + 4) & ~3));
}

cudaError_t render_composite_coords(void* buf, int W, int H, CompositeCoords* out, cudaStream_t s) {
  const int LW = (W + 4) & ~3, LH = (H + 4) & ~3;
  float* f = static_cast<float*>(buf);
  float* u = f;
  int* ix = reinterpret_cast<int*>(f + LW);
  float* pu = f + 2 * (size_t)LW;
  float* v = f + 3 * (size_t)LW;
  int* iy = reinterpret_cast<int*>(v + LH);
  float* pv = v + 2 * (size_t)LH;
  const float pixelate = (float)W / 2.0f;  // fragment140.glsl: pixelate = resolution.x / 2
  const float d = 1.0f / pixelate;
  const int n = std::max(LW, LH);
  se_composite_coords_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(u, ix, pu, v, iy, pv, W, H, d);
  *out = CompositeCoords{u, ix, pu, v, iy, pv};
  return cudaGetLastError();
}

cudaError_t render_composite(const CompositeSrc& src, const CompositeCoords& coords, const float4* light,
                             const float4* bg, int bw, int bh, const float w_side[3], float4* out, cudaStream_t s) {
  for_row_blocks((src.h + 15) / 16, [&](int by0, unsigned n) {
    se_composite_kernel<<<dim3((unsigned)((src.w + 63) / 64), n), 256, 0, s>>>(src, coords, light, bg, bw, bh, w_side[0],
                                                                              w_side[1], w_side[2], out, by0);
  });
  return cudaGetLastError();
}

cudaError_t render_noise(float* noise, int W, int H, cudaStream_t s) {
  for_row_blocks((H + 7) / 8, [&](int by0, unsigned n) {
    se_noise_kernel<<<dim3((unsigned)((W + 31) / 32), n), 256, 0, s>>>(noise, W, H, by0);
  });
  return cudaGetLastError();
}

cudaError_t render_color(const uint32_t* grid, const float* noise, float4* out, int W, int H, const RenderMat* mats,
                         int nmat, cudaStream_t s) {
  const long long n = (long long)W * H;
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const long long blocks = std::min<long long>((n + 255) / 256, (long long)sms * 8);
  se_color_kernel<<<(unsigned)(blocks > 0 ? blocks : 1), 256, 0, s>>>(grid, noise, out, n, mats, nmat);
  return cudaGetLastError();
}

cudaError_t light_pass(const uint32_t* old_grid, const uint32_t* new_grid, const float4* light_in, float4* light_out,
                       int W, int H, const RenderMat* mats, int nmat, cudaStream_t s) {
  const int rows = (H + LTH - 1) / LTH;
  const dim3 g((unsigned)((W + LTW - 1) / LTW), (unsigned)std::min(rows, 65535));
  if (rows <= 65535)
    se_light_kernel<false><<<g, 256, 0, s>>>(old_grid, new_grid, light_in, light_out, W, H, mats, nmat, 0);
  else
    for_row_blocks(rows, [&](int by0, unsigned n) {
      se_light_kernel<true><<<dim3(g.x, n), 256, 0, s>>>(old_grid, new_grid, light_in, light_out, W, H, mats, nmat,
                                                         by0);
    });
  return cudaGetLastError();
}

}  // namespace se::rt
