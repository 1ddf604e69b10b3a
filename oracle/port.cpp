// Oracle port: a hand-written CPU restatement of one sandengine frame.
// TEST INFRASTRUCTURE ONLY.  The product never links or calls this file; tests, smoke()
// and bench.py's CPU-baseline leg use it as the checker and as the timed CPU baseline.
//
// Restates, for the grid state (the cell ids):
//   shaders/compute/falling_sand.glsl:122-184  main(): frame==1 clear, modification pass
//   shaders/compute/falling_sand.glsl:61-118   simulate(): Margolus block update
//   shaders/compute/operations.glsl:16-23      guarded swap(Cell, Cell)
//   shaders/compute/operations.glsl:25-34      getMargolusOffset
//   shaders/compute/operations.glsl:45-57      getCell with SCREEN_IS_BORDER (WALL outside)
//   shaders/compute/math.glsl:28-38,74-79      hash4i / hash43
// and the two other outputs of setCell (port_color, port_light):
//   shaders/compute/operations.glsl:99-169     colour with noise, light propagation
//   shaders/compute/math.glsl:40-44,82-106     old_hash2, _noise, noise
// The per-ruleset part (TYPE_/MAT_ defines, isType_ checkers, rule_* functions and the
// apply*Rules callers) is the GLSL text the oracle front end emits for the rule set,
// rewritten by oracle/glsl2cpp.py and compiled through oracle/glsl_shim.hpp.
//
// Unlike the shader (one invocation per cell, each recomputing its whole 2x2 block),
// the port visits each block once, computes the block's four results from the pre-edit
// grid in place (blocks are disjoint and read only their own cells), and then applies
// the modification pass to the cells it hits.  That ordering gives every cell exactly
// the value main() stores for it.
#include <cstdint>
#include <cstring>
#include <vector>

#include "glsl_shim.hpp"

// falling_sand.glsl:12-19 and cell.glsl:4-11 (same members, same order).
struct Material {
  bool operator==(const Material&) const = default;
  int id;
  vec4 color;
  float density;
  vec4 emission;
  int type;
};
struct Cell {
  bool operator==(const Cell&) const = default;
  Material mat;
  ivec2 pos;
};
static inline Cell newCell(Material mat, ivec2 pos) { return Cell(mat, pos); }

#include "gen_materials.inc"

// operations.glsl:16-23: WALL and NULL cells never move.
static inline void swap(Cell& a, Cell& b) {
  if (a.mat.type == TYPE_WALL || b.mat.type == TYPE_WALL || a.mat.type == TYPE_NULL ||
      b.mat.type == TYPE_NULL)
    return;
  Cell t = a;
  a = b;
  b = t;
}

// The shader's uniforms that rule conditions may read (falling_sand.glsl:31-34); set by
// port_step before any block is visited.
static int frame = 0;
static ivec2 simSize;

#include "gen_rules.inc"

namespace {

Material g_by_id[256];
int g_nmat = 0;

void init_table() {
  if (g_nmat) return;
  auto all = materials();
  g_nmat = all.length();
  for (int i = 0; i < 256; ++i) g_by_id[i] = MAT_NULL;  // materials.glsl getMaterialFromID
  for (int i = 0; i < g_nmat; ++i)
    if (all[i].id >= 0 && all[i].id < 256) g_by_id[all[i].id] = all[i];
}

inline Material material_from_id(int64_t id) {
  return (id >= 0 && id < 256) ? g_by_id[id] : MAT_NULL;
}

// math.glsl:28-38 (hash4i) and :74-79 (hash43): lowbias32-style mix on four lanes;
// lane/0xffffffff rounds the divisor to 2^32, so each lane is RN(float(u)) * 2^-32.
inline vec4 hash43(uint32_t px, uint32_t py, uint32_t pz) {
  uint32_t x = px * 461u + py * 2131u + pz * 2131u * 2131u;
  uint32_t l[4] = {x * 213u, x * 2131u, x * 21313u, x * 213132u};
  for (auto& v : l) {
    v ^= v >> 16;
    v *= 0x7feb352du;
    v ^= v >> 15;
    v *= 0x846ca68bu;
    v ^= v >> 16;
  }
  const float d = (float)0xffffffffu;
  return vec4((float)l[0] / d, (float)l[1] / d, (float)l[2] / d, (float)l[3] / d);
}

// operations.glsl:25-34
inline ivec2 margolus_offset(int frame) {
  int f = frame % 4;
  if (f == 1) return ivec2(1, 1);
  if (f == 2) return ivec2(0, 1);
  if (f == 3) return ivec2(1, 0);
  return ivec2(0, 0);
}

struct Grid {
  uint32_t* g;
  int W, H;
  bool in(int x, int y) const { return x >= 0 && y >= 0 && x < W && y < H; }
  // operations.glsl:45-57 with SCREEN_IS_BORDER
  Cell get(ivec2 p) const {
    if (!in(p.x, p.y)) return newCell(MAT_WALL, p);
    return Cell(material_from_id(g[(int64_t)p.y * W + p.x]), p);
  }
  void put(ivec2 p, const Cell& c) {
    if (in(p.x, p.y)) g[(int64_t)p.y * W + p.x] = (uint32_t)c.mat.id;
  }
};

// falling_sand.glsl:61-118 for the block whose top-left cell is o.
inline void simulate_block(Grid& G, ivec2 o, int frame) {
  Cell self = G.get(o);
  Cell right = G.get(o + ivec2(1, 0));
  Cell down = G.get(o + ivec2(0, 1));
  Cell downright = G.get(o + ivec2(1, 1));
  if (self.mat == MAT_EMPTY && right.mat == MAT_EMPTY && down.mat == MAT_EMPTY &&
      downright.mat == MAT_EMPTY)
    return;  // all four stay EMPTY
  vec4 rand = hash43((uint32_t)o.x, (uint32_t)o.y, (uint32_t)frame);
  bool mirror = rand.x < 0.5f;
  if (mirror) {
    swap(self, right);
    swap(down, downright);
  }
  applyMirroredRules(self, right, down, downright, rand, o);
  if (mirror) {
    swap(self, right);
    swap(down, downright);
  }
  if (!mirror)
    applyRightRules(self, right, down, downright, rand, o);
  else
    applyLeftRules(self, right, down, downright, rand, o);
  G.put(o, self);
  G.put(o + ivec2(1, 0), right);
  G.put(o + ivec2(0, 1), down);
  G.put(o + ivec2(1, 1), downright);
}

// One SimModification as the 32-byte std140 record (simulation.rs:45-56).
struct Mod {
  int32_t px, py, shape, size, mat, pad[3];
};

// falling_sand.glsl:134-179: the last mod (in order) that hits a cell decides its
// material; a NULL result (unknown id) means "not modified".
inline bool modified_material(const Mod* mods, int n, ivec2 pos, int* out_id) {
  bool got = false;
  Material fin = MAT_NULL;
  for (int i = 0; i < n; ++i) {
    const Mod& m = mods[i];
    if (m.size == 0) break;
    ivec2 d = abs(ivec2(m.px, m.py) - pos);
    Material mat = material_from_id(m.mat);
    switch (m.shape) {
      case 0: {
        float dist = sqrt(pow((float)d.x, 2.0f) + pow((float)d.y, 2.0f));
        if (dist <= (float)m.size) {
          got = true;
          fin = mat;
        }
        break;
      }
      case 1:
        if (d.x <= m.size && d.y <= m.size) {
          got = true;
          fin = mat;
        }
        break;
    }
  }
  if (got && fin != MAT_NULL) {
    *out_id = fin.id;
    return true;
  }
  return false;
}

}  // namespace

extern "C" {

#define SE_EXPORT __attribute__((visibility("default")))

SE_EXPORT int port_num_materials() {
  init_table();
  return g_nmat;
}

// Advances the grid by one frame with frame counter `frame` (the value after the
// host's `frame += 1`, simulation.rs:201).  `mods` holds `nmods` 32-byte records; at most
// 256 are seen (simulation.rs:205) and the scan stops at the first with size 0.
SE_EXPORT void port_step(uint32_t* grid, int W, int H, int frame, const void* mods_raw, int nmods,
               int nthreads) {
  init_table();
  if (nthreads <= 0) nthreads = 1;
  if (frame == 1) {  // falling_sand.glsl:128-131
    memset(grid, 0, sizeof(uint32_t) * (size_t)W * H);
    return;
  }
  Grid G{grid, W, H};
  ::frame = frame;
  ::simSize = ivec2(W, H);
  const ivec2 off = margolus_offset(frame);
  const int nbx = (W - 1 + off.x) / 2 + 1;
  const int nby = (H - 1 + off.y) / 2 + 1;
#pragma omp parallel for schedule(static) num_threads(nthreads)
  for (int j = 0; j < nby; ++j)
    for (int i = 0; i < nbx; ++i) simulate_block(G, ivec2(2 * i - off.x, 2 * j - off.y), frame);

  const Mod* mods = (const Mod*)mods_raw;
  int n = nmods < 256 ? nmods : 256;
  if (n <= 0 || mods[0].size == 0) return;
  int live = 0;
  while (live < n && mods[live].size != 0) ++live;
  // Cells a mod can hit lie in [p - r, p + r] when |r| < 2^22 and |p| < 2^30 (the float
  // circle test cannot round a farther cell inside); other mods scan the whole grid.
  int64_t x0 = INT64_MAX, x1 = INT64_MIN, y0 = INT64_MAX, y1 = INT64_MIN;
  for (int i = 0; i < live; ++i) {
    const Mod& m = mods[i];
    int64_t r = m.size < 0 ? -(int64_t)m.size : m.size;
    bool normal = r < (1 << 22) && m.px > -(1 << 30) && m.px < (1 << 30) && m.py > -(1 << 30) &&
                  m.py < (1 << 30);
    if (!normal) {
      x0 = y0 = INT64_MIN / 4;
      x1 = y1 = INT64_MAX / 4;
      break;
    }
    if (m.px - r < x0) x0 = m.px - r;
    if (m.px + r > x1) x1 = m.px + r;
    if (m.py - r < y0) y0 = m.py - r;
    if (m.py + r > y1) y1 = m.py + r;
  }
  int ylo = (int)(y0 < 0 ? 0 : y0), yhi = (int)(y1 >= H ? H - 1 : y1);
  int xlo = (int)(x0 < 0 ? 0 : x0), xhi = (int)(x1 >= W ? W - 1 : x1);
#pragma omp parallel for schedule(static) num_threads(nthreads)
  for (int y = ylo; y <= yhi; ++y)
    for (int x = xlo; x <= xhi; ++x) {
      int id;
      if (modified_material(mods, live, ivec2(x, y), &id)) grid[(int64_t)y * W + x] = (uint32_t)id;
    }
}

// Runs `nframes` frames; the world's counter is `frame0` before the first one and the
// mods apply to the first frame only (the reference clears its mod list after each run).
SE_EXPORT void port_run(uint32_t* grid, int W, int H, int frame0, int nframes, const void* mods,
              int nmods, int nthreads) {
  for (int k = 0; k < nframes; ++k)
    port_step(grid, W, H, frame0 + k + 1, k == 0 ? mods : nullptr, k == 0 ? nmods : 0, nthreads);
}

// ---- colour and light (the rest of setCell, operations.glsl:99-169) ---------------------
// Scalar restatement in the shader's evaluation order (dot products left to right,
// max(a, b) = a < b ? b : a, mix(x, y, a) = x * (1 - a) + y * a), compiled without
// contraction, so the compiled reference shader gives the same bits on the same libm.

}  // extern "C"
namespace {

extern "C" {
// sin as the oracle evaluates it (glsl_shim.hpp se_sin), for n arguments.
SE_EXPORT void port_sin(const float* in, float* out, int n) {
  for (int i = 0; i < n; ++i) out[i] = se_sin(in[i]);
}
}  // extern "C"

// math.glsl:40-44 old_hash2, one component: -1 + 2 * fract(sin(q) * 43758.5453123).
inline float grad_component(float q) {
  const float v = sin(q) * 43758.5453123f;
  return -1.0f + 2.0f * fract(v);
}

// math.glsl:82-96 _noise (2D simplex noise with the sin-based gradient hash).
inline float simplex(float px, float py) {
  const float K1 = 0.366025404f, K2 = 0.211324865f;
  const float s = (px + py) * K1;
  const float ix = floor(px + s), iy = floor(py + s);
  const float t = (ix + iy) * K2;
  const float ax = (px - ix) + t, ay = (py - iy) + t;
  const float m = step(ay, ax);
  const float ox = m, oy = 1.0f - m;
  const float bx = (ax - ox) + K2, by = (ay - oy) + K2;
  const float c2 = 2.0f * K2;
  const float cx = (ax - 1.0f) + c2, cy = (ay - 1.0f) + c2;
  const float h0 = max(0.5f - (ax * ax + ay * ay), 0.0f);
  const float h1 = max(0.5f - (bx * bx + by * by), 0.0f);
  const float h2 = max(0.5f - (cx * cx + cy * cy), 0.0f);
  // gradients at the three corners i, i + o, i + 1 (old_hash2: dot with (127.1, 311.7) and
  // (269.5, 183.3))
  auto grad = [](float qx, float qy, float& gx, float& gy) {
    gx = grad_component(qx * 127.1f + qy * 311.7f);
    gy = grad_component(qx * 269.5f + qy * 183.3f);
  };
  float g0x, g0y, g1x, g1y, g2x, g2y;
  grad(ix, iy, g0x, g0y);
  grad(ix + ox, iy + oy, g1x, g1y);
  grad(ix + 1.0f, iy + 1.0f, g2x, g2y);
  const float n0 = h0 * h0 * h0 * h0 * (ax * g0x + ay * g0y);
  const float n1 = h1 * h1 * h1 * h1 * (bx * g1x + by * g1y);
  const float n2 = h2 * h2 * h2 * h2 * (cx * g2x + cy * g2y);
  return 0.25f + 0.5f * (n0 * 70.0f + n1 * 70.0f + n2 * 70.0f);
}

// math.glsl:98-106 noise(p, octaves = 3, lacunarity = 2, frequency = 0.25), as setCell calls it.
inline float cell_noise(float px, float py) {
  float f = 0.0f;
  for (int o = 1; o < 4; ++o) {
    f = f + (1.0f / (float)o) * simplex(px * 0.25f, py * 0.25f);
    px = px * 2.0f;
    py = py * 2.0f;
  }
  return f;
}

// operations.glsl:68-70
inline bool light_obstacle(const Material& m, ivec2 p) {
  return m.emission.x == 0.0f && m.emission.y == 0.0f && m.emission.z == 0.0f && !isType_EMPTY(Cell(m, p));
}

}  // namespace
extern "C" {

// output_color for a grid (operations.glsl:100-108): the material colour, darkened by
// noise(pos) / 4 and clamped to [0, 1] for every material but EMPTY.  RGBA per cell.
SE_EXPORT void port_color(const uint32_t* grid, int W, int H, float* out) {
  init_table();
  for (int y = 0; y < H; ++y)
    for (int x = 0; x < W; ++x) {
      const Material mt = material_from_id(grid[(int64_t)y * W + x]);
      vec4 c = mt.color;
      if (!(mt == MAT_EMPTY)) {
        const float r = cell_noise((float)x, (float)y) * 0.25f;
        c.x = clamp(c.x - r, 0.0f, 1.0f);
        c.y = clamp(c.y - r, 0.0f, 1.0f);
        c.z = clamp(c.z - r, 0.0f, 1.0f);
      }
      float* o = out + 4 * ((int64_t)y * W + x);
      o[0] = c.x;
      o[1] = c.y;
      o[2] = c.z;
      o[3] = c.w;
    }
}

// output_light of one frame (operations.glsl:114-166): the new cell's emission if it
// emits; the sky value on row 0; else the mean of the 8 neighbours' light (the previous
// frame's, with its colour masked where the neighbour's old cell is a light obstacle),
// blended half-way towards their per-channel maximum.  old/new: the grids before and
// after the frame; RGBA per cell.
SE_EXPORT void port_light(const uint32_t* old_grid, const uint32_t* new_grid, const float* lin, float* lout, int W,
                          int H) {
  init_table();
  static const int dx[8] = {0, 0, -1, -1, 1, 1, 1, -1};  // math.glsl:154-166 order
  static const int dy[8] = {1, -1, 1, -1, 1, -1, 0, 0};
  for (int y = 0; y < H; ++y)
    for (int x = 0; x < W; ++x) {
      const Material nm = material_from_id(new_grid[(int64_t)y * W + x]);
      float L[4];
      if (nm.emission.x != 0.0f || nm.emission.y != 0.0f || nm.emission.z != 0.0f) {
        L[0] = nm.emission.x, L[1] = nm.emission.y, L[2] = nm.emission.z, L[3] = nm.emission.w;
      } else if (y == 0) {
        L[0] = L[1] = L[2] = 1.0f;
        L[3] = 0.999999f;
      } else {
        float avg[4] = {0, 0, 0, 0}, mx[4] = {0, 0, 0, 0}, maxf = 0.0f;
        int num = 0;
        for (int n = 0; n < 8; ++n) {
          const int qx = x + dx[n], qy = y + dy[n];
          if (qx < 0 || qy < 0 || qx >= W || qy >= H) continue;
          const int64_t q = (int64_t)qy * W + qx;
          const float keep = light_obstacle(material_from_id(old_grid[q]), ivec2(qx, qy)) ? 0.0f : 1.0f;
          const float* l = lin + 4 * q;
          const float r = l[0] * keep, g = l[1] * keep, b = l[2] * keep, a = l[3] * 1.0f;
          const float falloff = a == 0.0f ? maxf : a;
          const float t[4] = {r * a, g * a, b * a, falloff};
          for (int c = 0; c < 4; ++c) avg[c] = avg[c] + t[c];
          maxf = max(falloff, maxf);
          ++num;
          for (int c = 0; c < 4; ++c) mx[c] = max(mx[c], t[c]);
        }
        if (num > 0)
          for (int c = 0; c < 4; ++c) avg[c] = avg[c] / (float)num;
        for (int c = 0; c < 3; ++c) L[c] = avg[c] * (1.0f - 0.5f) + mx[c] * 0.5f;
        L[3] = avg[3];
      }
      float* o = lout + 4 * ((int64_t)y * W + x);
      for (int c = 0; c < 4; ++c) o[c] = L[c];
    }
}

// ---- headless composite (shaders/fragment140.glsl:70-100) ----------------------------------
// One output pixel per texel (the full-screen quad of renderer.rs:212-246 at the grid's
// size), texel rows top to bottom, so the fragment at column c, row r samples
// uv = ((c + 0.5) / W, (r + 0.5) / H) (vertex140.glsl flips v, the window origin is at the
// bottom).  GL's texture filtering and mipmap generation are left to the driver; this
// restatement fixes them to the spec's formulas in binary32: mirrored-repeat wrap,
// nearest and bilinear taps, LINEAR_MIPMAP_NEAREST level choice (level ceil(lod + 0.5) - 1
// for lod > 0.5, the magnification filter for lod <= 0), a 2x2 box-filter pyramid with the
// last row / column repeated for odd sizes, pow(x, 2.0) = x * x.  The blur weights
// exp(-gamma) arrive precomputed (w[0..2] for gamma 0.5, 0.35, 0.2).

}  // extern "C"
namespace {

struct Level {
  const float* t;  // RGBA
  int w, h;
};

inline int mirror(int i, int n) {  // GL_MIRRORED_REPEAT on texel indices
  const int p = 2 * n;
  int m = i % p;
  if (m < 0) m += p;
  return m >= n ? p - 1 - m : m;
}

inline void texel(const Level& L, int i, int j, float o[4]) {
  const float* p = L.t + 4 * ((int64_t)mirror(j, L.h) * L.w + mirror(i, L.w));
  for (int c = 0; c < 4; ++c) o[c] = p[c];
}

inline void sample_nearest(const Level& L, float u, float v, float o[4]) {
  texel(L, (int)floor(u * (float)L.w), (int)floor(v * (float)L.h), o);
}

inline void sample_linear(const Level& L, float u, float v, float o[4]) {
  const float x = u * (float)L.w - 0.5f, y = v * (float)L.h - 0.5f;
  const float fx = floor(x), fy = floor(y);
  const float a = x - fx, b = y - fy;
  const int i = (int)fx, j = (int)fy;
  float t00[4], t10[4], t01[4], t11[4];
  texel(L, i, j, t00);
  texel(L, i + 1, j, t10);
  texel(L, i, j + 1, t01);
  texel(L, i + 1, j + 1, t11);
  const float w00 = (1.0f - a) * (1.0f - b), w10 = a * (1.0f - b), w01 = (1.0f - a) * b, w11 = a * b;
  for (int c = 0; c < 4; ++c) o[c] = ((t00[c] * w00 + t10[c] * w10) + t01[c] * w01) + t11[c] * w11;
}

// textureLod with MAG NEAREST / MIN LINEAR_MIPMAP_NEAREST
inline void sample_lod(const std::vector<Level>& mips, float u, float v, float lod, float o[4]) {
  if (lod <= 0.0f) return sample_nearest(mips[0], u, v, o);
  int d = lod <= 0.5f ? 0 : (int)__builtin_ceilf(lod + 0.5f) - 1;
  if (d > (int)mips.size() - 1) d = (int)mips.size() - 1;
  sample_linear(mips[(size_t)d], u, v, o);
}

// fragment140.glsl:37-50 sampleBlurred(tex, uv, radius, gamma), alpha only (the only
// channel main() reads); lod = log2(radius) is exact for 2, 16, 32.
inline float blurred_alpha(const std::vector<Level>& mips, float u, float v, float lod, float w_side) {
  float acc = 0.0f, wsum = 0.0f;
  for (int k = -1; k <= 1; ++k) {
    const float i = lod + (float)k;
    const float w = k == 0 ? 1.0f : w_side;  // exp(-gamma * pow(lod - i, 2))
    float t[4];
    sample_lod(mips, u, v, i, t);
    acc = acc + t[3] * w;
    wsum = wsum + w;
  }
  return acc / wsum;
}

}  // namespace
extern "C" {

// The box-filter pyramid of an RGBA level: out (w/2 or 1) x (h/2 or 1), each texel the
// mean of a 2x2 block (indices clamped to the source).
SE_EXPORT void port_mip_level(const float* src, int sw, int sh, float* dst) {
  const int dw = sw > 1 ? sw / 2 : 1, dh = sh > 1 ? sh / 2 : 1;
  for (int y = 0; y < dh; ++y)
    for (int x = 0; x < dw; ++x) {
      const int x0 = 2 * x < sw ? 2 * x : sw - 1, x1 = 2 * x + 1 < sw ? 2 * x + 1 : sw - 1;
      const int y0 = 2 * y < sh ? 2 * y : sh - 1, y1 = 2 * y + 1 < sh ? 2 * y + 1 : sh - 1;
      for (int c = 0; c < 4; ++c) {
        float s = src[4 * ((int64_t)y0 * sw + x0) + c] + src[4 * ((int64_t)y0 * sw + x1) + c];
        s = s + src[4 * ((int64_t)y1 * sw + x0) + c];
        s = s + src[4 * ((int64_t)y1 * sw + x1) + c];
        dst[4 * ((int64_t)y * dw + x) + c] = s * 0.25f;
      }
    }
}

// fragment140.glsl:70-100 for every pixel.  color: the colour field with its pyramid
// (levels[0] = color, as port_mip_level makes them, nlevels of them); light: the light
// field (or null: zero light); bg: background RGBA of bw x bh (or null: transparent).
SE_EXPORT void port_composite(const float* const* levels, const int* lw, const int* lh, int nlevels,
                              const float* light, const float* bg, int bw, int bh, const float* w_side, float* out) {
  std::vector<Level> mips;
  for (int l = 0; l < nlevels; ++l) mips.push_back(Level{levels[l], lw[l], lh[l]});
  const int W = lw[0], H = lh[0];
  const Level lightL{light, W, H}, bgL{bg, bw, bh};
  const float pixelate = (float)W / 2.0f;
  const float d = 1.0f / pixelate;
  for (int r = 0; r < H; ++r)
    for (int cix = 0; cix < W; ++cix) {
      const float u = ((float)cix + 0.5f) / (float)W, v = ((float)r + 0.5f) / (float)H;
      const float pu = floor(u / d) * d, pv = floor(v / d) * d;
      float col[4];
      sample_nearest(mips[0], u, v, col);  // texture(color_tex, uv, 0.0): 1:1, magnification
      float li[4] = {0, 0, 0, 0};
      if (light) sample_linear(lightL, pu, pv, li);
      for (int c = 0; c < 3; ++c) li[c] = clamp(li[c], 0.0f, 1.0f);
      float occ = 1.0f - blurred_alpha(mips, pu, pv, 1.0f, w_side[0]);
      const float occ2 = 1.0f - blurred_alpha(mips, pu, pv, 4.0f, w_side[1]);
      const float occ3 = 1.0f - blurred_alpha(mips, pu, pv, 5.0f, w_side[2]);
      occ = occ + (occ2 * 0.4f + occ3 * 0.25f);
      occ = clamp(occ, 0.0f, 1.0f);
      const float ambient = 0.1f;
      const float sky = 0.5f * (1.0f - pv);
      const float shade = ambient + occ * (1.0f - ambient);
      for (int c = 0; c < 3; ++c) col[c] = clamp(col[c] * shade, 0.0f, 1.0f);
      float b[4] = {0, 0, 0, 0};
      if (bg) sample_linear(bgL, u, 1.0f - v, b);
      float* o = out + 4 * ((int64_t)r * W + cix);
      for (int c = 0; c < 4; ++c) o[c] = b[c] * (1.0f - col[3]) + col[c] * col[3];  // mix(bg, col, col.a)
      for (int c = 0; c < 3; ++c) o[c] = o[c] * ((ambient + sky) + li[c]);
      o[3] = o[3] * 1.0f;
    }
}

// hash43 lanes, exposed for known-answer tests of the RNG.
SE_EXPORT void port_hash43(int x, int y, int frame, float* out4) {
  vec4 r = hash43((uint32_t)x, (uint32_t)y, (uint32_t)frame);
  out4[0] = r.x;
  out4[1] = r.y;
  out4[2] = r.z;
  out4[3] = r.w;
}

}  // extern "C"
