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

// hash43 lanes, exposed for known-answer tests of the RNG.
SE_EXPORT void port_hash43(int x, int y, int frame, float* out4) {
  vec4 r = hash43((uint32_t)x, (uint32_t)y, (uint32_t)frame);
  out4[0] = r.x;
  out4[1] = r.y;
  out4[2] = r.z;
  out4[3] = r.w;
}

}  // extern "C"
