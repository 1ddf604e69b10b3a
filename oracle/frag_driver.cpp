// Driver that runs the reference's own fragment shader (shaders/fragment140.glsl) on the
// CPU, one invocation per output pixel.  TEST INFRASTRUCTURE ONLY.  `ref_frag.inc` is that
// file's text passed through oracle/glsl2cpp.py's fragment_to_cpp; it is generated into
// oracle/_ref/ by oracle/build.py from the reference tree and never committed.
//
// The shader's samplers follow OpenGL's texture filtering formulas in binary32 with the
// choices the headless composite fixes (the GL driver leaves them open):
//   * one fragment per texel: the fragment at column c, row r (rows top to bottom) reads
//     v_tex_coords = ((c + 0.5) / W, (r + 0.5) / H), so texture() samples at lambda = 0 (+
//     its bias), a magnification;
//   * color_tex: magnification NEAREST, minification LINEAR_MIPMAP_NEAREST over a
//     pyramid of 2x2 box-filtered levels (given by the caller); textureLod picks level
//     ceil(lod + 0.5) - 1 (lod <= 0.5: level 0), clamped to the last level, and filters it
//     bilinearly; lod <= 0 is a magnification;
//   * light_tex and background_tex: LINEAR, one level; an unbound sampler reads 0;
//   * wrap MIRRORED_REPEAT on texel indices;
//   * bilinear = ((t00 w00 + t10 w10) + t01 w01) + t11 w11 with w00 = (1 - a)(1 - b),
//     w10 = a(1 - b), w01 = (1 - a) b, w11 = a b, at x = u W - 0.5, y = v H - 0.5.
// fwidth (used only by helpers main() does not call) returns 0.
#include <cstdint>
#include <vector>

#define SE_GLSL_FRAGMENT 1
#include "glsl_shim.hpp"

struct SeLevel {
  const float* t;  // w * h RGBA32F texels, row-major
  int w, h;
};
struct sampler2D {
  std::vector<SeLevel> levels;  // level 0 first; empty: no texture bound
  bool mag_linear = false;
};

namespace {

int mirrored(int i, int n) {  // GL_MIRRORED_REPEAT on a texel index
  const int p = 2 * n;
  int m = i % p;
  if (m < 0) m += p;
  return m >= n ? p - 1 - m : m;
}

vec4 fetch(const SeLevel& L, int i, int j) {
  const float* t = L.t + 4 * ((int64_t)mirrored(j, L.h) * L.w + mirrored(i, L.w));
  return vec4(t[0], t[1], t[2], t[3]);
}

vec4 nearest(const SeLevel& L, vec2 uv) {
  return fetch(L, (int)floor(uv.x * (float)L.w), (int)floor(uv.y * (float)L.h));
}

vec4 bilinear(const SeLevel& L, vec2 uv) {
  const float x = uv.x * (float)L.w - 0.5f, y = uv.y * (float)L.h - 0.5f;
  const float fx = floor(x), fy = floor(y);
  const float a = x - fx, b = y - fy;
  const int i = (int)fx, j = (int)fy;
  const vec4 t00 = fetch(L, i, j), t10 = fetch(L, i + 1, j), t01 = fetch(L, i, j + 1), t11 = fetch(L, i + 1, j + 1);
  const float w00 = (1.0f - a) * (1.0f - b), w10 = a * (1.0f - b), w01 = (1.0f - a) * b, w11 = a * b;
  return ((t00 * w00 + t10 * w10) + t01 * w01) + t11 * w11;
}

vec4 sample_at(const sampler2D& s, vec2 uv, float lambda) {
  if (s.levels.empty()) return vec4(0.0f);
  if (lambda <= 0.0f) return s.mag_linear ? bilinear(s.levels[0], uv) : nearest(s.levels[0], uv);
  int d = lambda <= 0.5f ? 0 : (int)__builtin_ceilf(lambda + 0.5f) - 1;
  if (d > (int)s.levels.size() - 1) d = (int)s.levels.size() - 1;
  return bilinear(s.levels[(size_t)d], uv);
}

}  // namespace

vec4 texture(const sampler2D& s, vec2 uv, float bias = 0.0f) { return sample_at(s, uv, bias); }
vec4 textureLod(const sampler2D& s, vec2 uv, float lod) { return sample_at(s, uv, lod); }
ivec2 textureSize(const sampler2D& s, int) {
  return s.levels.empty() ? ivec2(0, 0) : ivec2(s.levels[0].w, s.levels[0].h);
}
vec2 fwidth(vec2) { return vec2(0.0f, 0.0f); }

#include "ref_frag.inc"

extern "C" {

#define SE_EXPORT __attribute__((visibility("default")))

// levels: the colour field's pyramid (level 0 = the field, W x H); light: W x H or null;
// bg: bw x bh or null.  out: W x H RGBA32F, the shader's f_color per pixel.
SE_EXPORT void ref_frag_composite(const float* const* levels, const int* lw, const int* lh, int nlevels,
                                  const float* light, const float* bg, int bw, int bh, float* out) {
  const int W = lw[0], H = lh[0];
  color_tex = sampler2D{};
  for (int l = 0; l < nlevels; ++l) color_tex.levels.push_back(SeLevel{levels[l], lw[l], lh[l]});
  color_tex.mag_linear = false;
  light_tex = sampler2D{};
  if (light) light_tex.levels.push_back(SeLevel{light, W, H});
  light_tex.mag_linear = true;
  background_tex = sampler2D{};
  if (bg) background_tex.levels.push_back(SeLevel{bg, bw, bh});
  background_tex.mag_linear = true;
  tex_size = vec2((float)W, (float)H);
  frame = 0;
  for (int r = 0; r < H; ++r)
    for (int c = 0; c < W; ++c) {
      v_tex_coords = vec2(((float)c + 0.5f) / (float)W, ((float)r + 0.5f) / (float)H);
      glsl_main();
      float* o = out + 4 * ((int64_t)r * W + c);
      o[0] = f_color.x;
      o[1] = f_color.y;
      o[2] = f_color.z;
      o[3] = f_color.w;
    }
}

}  // extern "C"
