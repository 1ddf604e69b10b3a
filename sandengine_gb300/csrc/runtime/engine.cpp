#include "engine.hpp"
#include "trace.hpp"

#include <algorithm>
#include <cstring>
#include <set>

#include "../../../include/sandengine.h"

namespace se::rt {

namespace {
Status cuda_fail(const char* what, cudaError_t e) {
  return {SE_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e)};
}
#define SE_CUDA(call)                               \
  do {                                              \
    cudaError_t _e = (call);                        \
    if (_e != cudaSuccess) return cuda_fail(#call, _e); \
  } while (0)
}  // namespace

std::string Ruleset::device_source() const {
  return (checked ? std::string("#define SE_CHECKED 1\n") : std::string()) + kernel_source(cuda.source);
}

Status Ruleset::check_word(unsigned int* word, bool reset) {
  if (!checked) return {SE_ERR_INVALID_ARGUMENT, "the rule set was not compiled as a CHECKED build"};
  Status s = ensure_loaded();
  if (!s.ok()) return s;
  void* p = nullptr;
  size_t bytes = 0;
  SE_CUDA(cudaLibraryGetGlobal(&p, &bytes, module->lib, "se_check_word"));
  SE_CUDA(cudaDeviceSynchronize());
  SE_CUDA(cudaMemcpy(word, p, sizeof(unsigned int), cudaMemcpyDeviceToHost));
  if (reset) SE_CUDA(cudaMemset(p, 0, sizeof(unsigned int)));
  return Status::Ok();
}

Status Ruleset::compile() {
  std::lock_guard<std::mutex> g(mu);
  if (compiled) return Status::Ok();
  if (codegen_code) return {codegen_code, codegen_message};
  std::string log;
  if (!compile_cubin(device_source(), &cubin, &log)) return {SE_ERR_COMPILE, "NVRTC: " + log};
  compiled = true;
  return Status::Ok();
}

Status Ruleset::ensure_loaded() {
  Status s = compile();
  if (!s.ok()) return s;
  std::lock_guard<std::mutex> g(mu);
  if (module) return Status::Ok();
  auto m = std::make_unique<Module>();
  std::string err;
  if (!m->load(cubin, lut_shape(), &err)) return {SE_ERR_CUDA, err};
  if (cuda.lut_entries) {  // build the block transition table with the rules themselves
    const size_t table = ((size_t)cuda.lut_entries * sizeof(uint16_t) + 15) & ~(size_t)15;
    cudaError_t e = cudaMalloc(&d_lut, table + (size_t)cuda.lut_static_words * 4);
    if (e != cudaSuccess) return {SE_ERR_OUT_OF_MEMORY, std::string("cudaMalloc: ") + cudaGetErrorString(e)};
    void* args[] = {(void*)&d_lut};
    const unsigned blocks = (unsigned)std::min<unsigned long long>((cuda.lut_entries + 255) / 256, 4096);
    SE_CUDA(cudaLaunchKernel((const void*)m->get("se_build_lut"), dim3(blocks), dim3(256), args, 0, nullptr));
    const unsigned sblocks = (unsigned)((cuda.lut_static_words + 255) / 256);
    SE_CUDA(cudaLaunchKernel((const void*)m->get("se_build_static"), dim3(sblocks), dim3(256), args, 0, nullptr));
    SE_CUDA(cudaDeviceSynchronize());
  }
  {  // render table (operations.glsl:68-70, 100-108, 126): colour, emission and flags
    std::set<std::string> empty_types = {"EMPTY"};  // isType_EMPTY: EMPTY and its child types
    for (const auto& t : parsed.types)
      if (t.name == "EMPTY") empty_types.insert(t.children.begin(), t.children.end());
    std::vector<RenderMat> table(parsed.materials.size());
    for (size_t i = 0; i < table.size(); ++i) {
      const auto& mt = parsed.materials[i];
      RenderMat& r = table[i];
      memset(&r, 0, sizeof r);
      for (int c = 0; c < 4; ++c) r.color[c] = mt.color[c], r.emission[c] = mt.emission[c];
      const bool dark = mt.emission[0] == 0.0f && mt.emission[1] == 0.0f && mt.emission[2] == 0.0f;
      if (!dark) r.flags |= kRenderEmits;  // vec3 != vec3(0.0): some component differs
      if (dark && !empty_types.count(mt.mattype)) r.flags |= kRenderObstacle;
      if (i != 0) r.flags |= kRenderNoise;  // mat != MAT_EMPTY
    }
    cudaError_t e = cudaMalloc(&d_render, table.size() * sizeof(RenderMat));
    if (e != cudaSuccess) return {SE_ERR_OUT_OF_MEMORY, std::string("cudaMalloc: ") + cudaGetErrorString(e)};
    SE_CUDA(cudaMemcpy(d_render, table.data(), table.size() * sizeof(RenderMat), cudaMemcpyHostToDevice));
  }
  module = std::move(m);
  return Status::Ok();
}

Ruleset::~Ruleset() {
  if (d_lut) cudaFree(d_lut);
  if (d_render) cudaFree(d_render);
}

World::~World() {
  for (auto& set : timed)
    for (auto& t : set) {
      cudaEventDestroy(t.a);
      cudaEventDestroy(t.b);
    }
  if (buf[0]) cudaFree(buf[0]);
  if (buf[1]) cudaFree(buf[1]);
  for (auto* l : light)
    if (l) cudaFree(l);
  if (d_noise) cudaFree(d_noise);
  if (d_color) cudaFree(d_color);
  for (auto* m : mips) cudaFree(m);
  if (d_coords) cudaFree(d_coords);
  for (auto& cs : copy_streams)
    if (cs) cudaStreamSynchronize(cs);
  for (int i = 0; i < 2; ++i) {
    if (stage[i]) cudaFree(stage[i]);
    if (stage_ready[i]) cudaEventDestroy(stage_ready[i]);
    for (auto& e : stage_done[i])
      if (e) cudaEventDestroy(e);
    if (stage8[i]) cudaFree(stage8[i]);
    if (stage8_ready[i]) cudaEventDestroy(stage8_ready[i]);
    for (auto& e : stage8_done[i])
      if (e) cudaEventDestroy(e);
  }
  for (auto& cs : copy_streams)
    if (cs) cudaStreamDestroy(cs);
  if (d_composite) cudaFree(d_composite);
  if (d_bg) cudaFree(d_bg);
  if (d_scratch) cudaFree(d_scratch);
  if (own_stream) cudaStreamDestroy(own_stream);
}

Status World::create(std::shared_ptr<Ruleset> r, int w, int h) {
  if (w <= 0 || h <= 0) return {SE_ERR_INVALID_ARGUMENT, "world size must be positive"};
  if (w > kMaxSide || h > kMaxSide) return {SE_ERR_INVALID_ARGUMENT, "world sides are limited to 1048576 cells"};
  if ((int64_t)w * h > (int64_t)1 << 36) return {SE_ERR_INVALID_ARGUMENT, "world too large"};
  rs = std::move(r);
  W = w;
  H = h;
  if (wh == 0) wh = h;
  Status s = rs->ensure_loaded();
  if (!s.ok()) return s;
  SE_CUDA(cudaStreamCreateWithFlags(&own_stream, cudaStreamNonBlocking));
  stream = own_stream;
  const size_t bytes = (size_t)W * H * sizeof(uint32_t);
  for (int i = 0; i < 2; ++i) {
    cudaError_t e = cudaMalloc(&buf[i], bytes);
    if (e != cudaSuccess) return {SE_ERR_OUT_OF_MEMORY, std::string("cudaMalloc: ") + cudaGetErrorString(e)};
  }
  {
    cudaError_t e = cudaMalloc(&d_scratch, 258 * sizeof(unsigned long long));
    if (e != cudaSuccess) return {SE_ERR_OUT_OF_MEMORY, std::string("cudaMalloc: ") + cudaGetErrorString(e)};
  }
  SE_CUDA(cudaMemsetAsync(buf[0], 0, bytes, stream));  // Simulation::new: all-zero textures
  SE_CUDA(cudaStreamSynchronize(stream));
  return Status::Ok();
}

Status World::create_band(std::shared_ptr<Ruleset> r, int w, int world_h, int row0, int rows, int hal) {
  if (w <= 0 || world_h <= 0 || rows <= 0 || row0 < 0 || (int64_t)row0 + rows > world_h || hal < 0)
    return {SE_ERR_INVALID_ARGUMENT, "band rows must lie within the world and the halo be >= 0"};
  if (w > kMaxSide || world_h > kMaxSide) return {SE_ERR_INVALID_ARGUMENT, "world sides are limited to 1048576 cells"};
  const int a = std::max(0, row0 - hal), b = (int)std::min<int64_t>(world_h, (int64_t)row0 + rows + hal);
  wh = world_h;
  ya = a;
  halo = hal;
  return create(std::move(r), w, b - a);
}

int World::default_k() const {
  if (steps_per_launch > 0) return steps_per_launch;
  return fused ? fused->kmax : 1;
}

static const TileVariant* pick_variant(int k) {
  const TileVariant* best = nullptr;
  for (const TileVariant& t : tile_variants())
    if (t.kmax >= k && (!best || t.kmax < best->kmax)) best = &t;
  return best;
}

Status World::autotune(int reps, int* best_k) {
  TraceRange trace("se_world_autotune");
  if (reps < 1) reps = 1;
  const int f0 = frame + 1 >= 2 ? frame + 1 : 2;  // trial frames never hit the frame-1 clear
  struct Restore {
    bool& flag;
    bool saved;
    ~Restore() { flag = saved; }
  } restore{timing, timing};
  timing = false;  // trials are not part of any measured region
  cudaEvent_t a, b;
  SE_CUDA(cudaEventCreate(&a));
  SE_CUDA(cudaEventCreate(&b));
  double best_multi = 0, best_one = 0;
  const TileVariant *vm = nullptr, *v1 = nullptr;
  for (const TileVariant& v : tile_variants()) {
    Status s = launch_tiles(f0, v.kmax, &v, false);  // warm-up
    if (!s.ok()) return s;
    SE_CUDA(cudaEventRecord(a, stream));
    for (int r = 0; r < reps; ++r) {
      s = launch_tiles(f0, v.kmax, &v, false);
      if (!s.ok()) return s;
    }
    SE_CUDA(cudaEventRecord(b, stream));
    SE_CUDA(cudaEventSynchronize(b));
    float ms = 0;
    SE_CUDA(cudaEventElapsedTime(&ms, a, b));
    const double rate = (double)W * H * v.kmax * reps / (ms > 0 ? ms : 1e-6);  // cell updates per ms
    if (v.kmax == 1 && rate > best_one) best_one = rate, v1 = &v;
    if (rate > best_multi) best_multi = rate, vm = &v;
  }
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  fused = vm;
  single = v1;
  if (best_k) *best_k = vm ? vm->kmax : 1;
  return Status::Ok();
}

Status launch_tile_kernel(const Ruleset& rs, const TileVariant& v, const uint32_t* src, uint32_t* dst, int W, int H,
                          int f0, int k, int ya, int yb, cudaStream_t stream, const EditParams* edits, int nedits) {
  if (v.kmax < k || k < 1) return {SE_ERR_INVALID_ARGUMENT, "no kernel variant for this many frames per launch"};
  if (ya < 0 || yb > H || ya >= yb) return {SE_ERR_INVALID_ARGUMENT, "tile rows outside the world"};
  if (edits && (nedits < 1 || nedits > SE_MAX_MODIFICATIONS))
    return {SE_ERR_INVALID_ARGUMENT, "an edit launch takes 1..256 modifications"};
  cudaKernel_t kern = rs.module->get(edits ? v.edit_name() : v.name());
  const uint16_t* lut = rs.d_lut;
  // se_tile_impl's order; the edit variant adds the edit list (by value) and its length
  void* args[] = {(void*)&src, (void*)&dst, &W, &H, &f0, &k, (void*)&lut, &ya, &yb, (void*)edits, &nedits};
  dim3 grid((unsigned)((W + v.tw - 1) / v.tw), (unsigned)((yb - ya + v.th - 1) / v.th));
  SE_CUDA(cudaLaunchKernel((const void*)kern, grid, dim3((unsigned)v.nt), args, tile_smem_bytes(v, rs.lut_shape()),
                           stream));
  return Status::Ok();
}

Status World::launch_tiles(int f0, int k, const TileVariant* v, bool commit, const EditParams* edits, int nedits) {
  if (!v || v->kmax < k) return {SE_ERR_INVALID_ARGUMENT, "no kernel variant for this many frames per launch"};
  Timed* t = nullptr;
  if (timing) {
    Status s = timing_begin(0, (long long)W * H, k, &t);
    if (!s.ok()) return s;
  }
  Status s = launch_tile_kernel(*rs, *v, buf[cur], buf[cur ^ 1], W, wh, f0, k, ya, ya + H, stream, edits, nedits);
  if (!s.ok()) return s;
  if (t) SE_CUDA(cudaEventRecord(t->b, stream));
  if (commit) cur ^= 1;
  return Status::Ok();
}

Status World::timing_begin(int pass, long long cells, int frames, Timed** out) {
  auto& set = timed[pass];
  if (timed_used[pass] == set.size()) {
    Timed n{};
    SE_CUDA(cudaEventCreate(&n.a));
    SE_CUDA(cudaEventCreate(&n.b));
    set.push_back(n);
  }
  Timed* t = &set[timed_used[pass]++];
  t->cells = cells;
  t->frames = frames;
  SE_CUDA(cudaEventRecord(t->a, stream));
  *out = t;
  return Status::Ok();
}

Status World::timing_peek_frames(int frames, double* ms, long long* launches) {
  SE_CUDA(cudaStreamSynchronize(stream));
  double tot = 0;
  long long n = 0;
  const auto& set = timed[0];
  for (size_t i = 0; i < timed_used[0]; ++i) {
    if (set[i].frames != frames) continue;
    float m = 0;
    SE_CUDA(cudaEventElapsedTime(&m, set[i].a, set[i].b));
    tot += m;
    ++n;
  }
  *ms = tot;
  *launches = n;
  return Status::Ok();
}

Status World::timing_read(int pass, double* ms, long long* launches, long long* cell_frames, long long* cells) {
  if (pass < 0 || pass > 3)
    return {SE_ERR_INVALID_ARGUMENT, "pass must be 0 (tiles), 1 (light), 2 (colour) or 3 (composite)"};
  SE_CUDA(cudaStreamSynchronize(stream));
  double tot = 0;
  long long cf = 0, c = 0;
  const auto& set = timed[pass];
  for (size_t i = 0; i < timed_used[pass]; ++i) {
    float m = 0;
    SE_CUDA(cudaEventElapsedTime(&m, set[i].a, set[i].b));
    tot += m;
    cf += set[i].cells * set[i].frames;
    c += set[i].cells;
  }
  *ms = tot;
  *launches = (long long)timed_used[pass];
  *cell_frames = cf;
  *cells = c;
  timed_used[pass] = 0;
  return Status::Ok();
}

long long fill_edit_params(const Ruleset& rs, int W, int row0, int rows, const se_modification* mods, int nlive,
                           EditParams* out) {
  EditParams& p = *out;
  memset(&p, 0, sizeof p);
  long long total = 0;
  const int nmat = rs.num_materials();
  for (int i = 0; i < nlive; ++i) {
    const se_modification& m = mods[i];
    int* r = &p.mods[8 * i];
    r[0] = m.position[0];
    r[1] = m.position[1];
    r[2] = m.mod_shape;
    r[3] = m.mod_size;
    r[4] = (m.mod_matID >= 0 && m.mod_matID < nmat) ? m.mod_matID : 1;  // getMaterialFromID
    // Cells the mod can hit: [p - r, p + r] when |r| < 2^22 and |p| < 2^30 (no cell
    // farther away passes the binary32 circle test); otherwise the whole grid.
    int64_t rad = m.mod_size < 0 ? -(int64_t)m.mod_size : m.mod_size;
    bool normal = rad < (1 << 22) && m.position[0] > -(1 << 30) && m.position[0] < (1 << 30) &&
                  m.position[1] > -(1 << 30) && m.position[1] < (1 << 30);
    int64_t x0 = 0, y0 = row0, x1 = W - 1, y1 = (int64_t)row0 + rows - 1;
    if (normal) {
      x0 = std::max<int64_t>(0, m.position[0] - rad);
      x1 = std::min<int64_t>(W - 1, m.position[0] + rad);
      y0 = std::max<int64_t>(row0, m.position[1] - rad);
      y1 = std::min<int64_t>((int64_t)row0 + rows - 1, m.position[1] + rad);
    }
    p.start[i] = total;
    if (x1 >= x0 && y1 >= y0) {
      p.box[4 * i + 0] = (int)x0;
      p.box[4 * i + 1] = (int)y0;
      p.box[4 * i + 2] = (int)x1;
      p.box[4 * i + 3] = (int)y1;
      total += (x1 - x0 + 1) * (y1 - y0 + 1);
    } else {  // empty: x1 < x0
      p.box[4 * i + 0] = 0;
      p.box[4 * i + 1] = 0;
      p.box[4 * i + 2] = -1;
      p.box[4 * i + 3] = -1;
    }
  }
  p.start[nlive] = total;
  return total;
}

Status launch_edit_on(const Ruleset& rs, uint32_t* grid, int W, int row0, int rows, const se_modification* mods,
                      int nlive, cudaStream_t stream) {
  EditParams p;
  long long total = fill_edit_params(rs, W, row0, rows, mods, nlive, &p);
  if (total == 0) return Status::Ok();
  cudaKernel_t kern = rs.module->get("se_edit");
  uint32_t* g = grid;
  int Wv = W, Hv = row0 + rows, n = nlive, r0 = row0;
  void* args[] = {(void*)&g, &Wv, &Hv, &n, &total, &p, &r0};
  dim3 blocks((unsigned)((total + 255) / 256));
  SE_CUDA(cudaLaunchKernel((const void*)kern, blocks, dim3(256), args, 0, stream));
  return Status::Ok();
}

Status World::step(int nframes, const se_modification* mods, int nmods) {
  TraceRange trace("se_world_step");
  if (nframes < 0) return {SE_ERR_INVALID_ARGUMENT, "nframes must be >= 0"};
  if (nmods < 0 || (nmods > 0 && !mods)) return {SE_ERR_INVALID_ARGUMENT, "bad modification list"};
  if ((int64_t)frame + nframes > INT32_MAX) return {SE_ERR_INVALID_ARGUMENT, "frame counter would overflow i32"};
  if (halo >= 0 && nframes > halo)
    return {SE_ERR_INVALID_ARGUMENT, "a band advances at most `halo` frames between halo exchanges"};
  int nlive = 0;
  const int nseen = std::min(nmods, SE_MAX_MODIFICATIONS);  // simulation.rs:205
  while (nlive < nseen && mods[nlive].mod_size != 0) ++nlive;  // falling_sand.glsl:139-141
  const TileVariant* vmulti = nullptr;
  if (steps_per_launch > 0) {
    vmulti = pick_variant(steps_per_launch);
  } else {
    if (!fused && nframes >= 2) {
      Status s = autotune(2, nullptr);
      if (!s.ok()) return s;
    }
    vmulti = fused ? fused : pick_variant(1);
  }
  const TileVariant* vone = single ? single : pick_variant(1);
  const int kdef = steps_per_launch > 0 ? steps_per_launch : vmulti->kmax;
  if (light[0]) {  // one frame at a time, each followed by the light pass
    for (int i = 0; i < nframes; ++i) {
      const int f = frame + 1 + i;
      if (f == 1) {  // the clear goes to the spare buffer: the light pass reads the old grid
        SE_CUDA(cudaMemsetAsync(buf[cur ^ 1], 0, (size_t)W * H * sizeof(uint32_t), stream));
        cur ^= 1;
      } else if (i == 0 && nlive > 0) {  // the frame and its edit pass in one launch
        fill_edit_params(*rs, W, ya, H, mods, nlive, &edit_params);
        Status s = launch_tiles(f, 1, vone, true, &edit_params, nlive);
        if (!s.ok()) return s;
      } else {
        Status s = launch_tiles(f, 1, vone);
        if (!s.ok()) return s;
      }
      Status s = light_frame();
      if (!s.ok()) return s;
    }
    frame += nframes;
    return Status::Ok();
  }
  int i = 0;
  while (i < nframes) {
    const int f = frame + 1 + i;
    if (f == 1) {  // falling_sand.glsl:128-131: clear, mods ignored
      SE_CUDA(cudaMemsetAsync(buf[cur], 0, (size_t)W * H * sizeof(uint32_t), stream));
      ++i;
      continue;
    }
    const int k = std::min(kdef, nframes - i);
    const TileVariant* v = k == 1 ? vone : vmulti;
    if (i == 0 && nlive > 0) {  // the edit pass runs inside the launch, after its first frame
      fill_edit_params(*rs, W, ya, H, mods, nlive, &edit_params);
      Status s = launch_tiles(f, k, v, true, &edit_params, nlive);
      if (!s.ok()) return s;
      i += k;
      continue;
    }
    Status s = launch_tiles(f, k, v);
    if (!s.ok()) return s;
    i += k;
  }
  frame += nframes;
  return Status::Ok();
}

Status World::set_light(bool on) {
  if (on && halo >= 0) return {SE_ERR_INVALID_ARGUMENT, "the light field is not kept for bands"};
  if (!on) {
    for (auto*& l : light)
      if (l) cudaFree(l), l = nullptr;
    return Status::Ok();
  }
  if (light[0]) return Status::Ok();
  const size_t bytes = (size_t)W * H * sizeof(float4);
  for (auto*& l : light) {
    cudaError_t e = cudaMalloc(&l, bytes);
    if (e != cudaSuccess) {
      set_light(false);
      return {SE_ERR_OUT_OF_MEMORY, std::string("cudaMalloc: ") + cudaGetErrorString(e)};
    }
  }
  SE_CUDA(cudaMemsetAsync(light[0], 0, bytes, stream));
  lcur = 0;
  return Status::Ok();
}

Status World::light_frame() {
  Timed* t = nullptr;
  if (timing) {
    Status s = timing_begin(1, (long long)W * H, 1, &t);
    if (!s.ok()) return s;
  }
  SE_CUDA(light_pass(buf[cur ^ 1], buf[cur], light[lcur], light[lcur ^ 1], W, H, rs->d_render,
                     rs->num_materials(), stream));
  if (t) SE_CUDA(cudaEventRecord(t->b, stream));
  lcur ^= 1;
  return Status::Ok();
}

Status World::render_color(float* alpha1) {
  TraceRange trace("se_world_render_color");
  if (halo >= 0) return {SE_ERR_INVALID_ARGUMENT, "colours are rendered for whole worlds"};
  if (!d_noise) {
    cudaError_t e = cudaMalloc(&d_noise, (size_t)W * H * sizeof(float));
    if (e != cudaSuccess) return {SE_ERR_OUT_OF_MEMORY, std::string("cudaMalloc: ") + cudaGetErrorString(e)};
    SE_CUDA(render_noise(d_noise, W, H, stream));
  }
  if (!d_color) {
    cudaError_t e = cudaMalloc(&d_color, (size_t)W * H * sizeof(float4));
    if (e != cudaSuccess) return {SE_ERR_OUT_OF_MEMORY, std::string("cudaMalloc: ") + cudaGetErrorString(e)};
  }
  Timed* t = nullptr;
  if (timing) {
    Status s = timing_begin(2, (long long)W * H, 1, &t);
    if (!s.ok()) return s;
  }
  if (alpha1)
    SE_CUDA(render_color_mip(buf[cur], d_noise, d_color, alpha1, W, H, rs->d_render, rs->num_materials(), stream));
  else
    SE_CUDA(se::rt::render_color(buf[cur], d_noise, d_color, W, H, rs->d_render, rs->num_materials(), stream));
  if (t) SE_CUDA(cudaEventRecord(t->b, stream));
  return Status::Ok();
}

Status World::composite(const float* bg, int bw, int bh) {
  TraceRange trace("se_world_composite");
  if (bg && (bw <= 0 || bh <= 0)) return {SE_ERR_INVALID_ARGUMENT, "background size must be positive"};
  // pyramid sizes (level 0 is the colour field); the alpha levels are allocated once, and a
  // 1 x 1 field keeps a copy of its alpha in place of level 1
  int lw[kMaxMipLevels], lh[kMaxMipLevels], n = 1;
  lw[0] = W;
  lh[0] = H;
  for (; (lw[n - 1] > 1 || lh[n - 1] > 1) && n < kMaxMipLevels; ++n) {
    lw[n] = mip_next(lw[n - 1]);
    lh[n] = mip_next(lh[n - 1]);
  }
  for (int l = (int)mips.size() + 1; l < std::max(n, 2); ++l) {
    float* m = nullptr;
    cudaError_t e = cudaMalloc(&m, (l < n ? (size_t)lw[l] * (size_t)lh[l] : 1) * sizeof(float));
    if (e != cudaSuccess) return {SE_ERR_OUT_OF_MEMORY, std::string("cudaMalloc: ") + cudaGetErrorString(e)};
    mips.push_back(m);
  }
  // colours and level 1 in one pass, then the smaller levels
  Status s = render_color(n > 1 ? mips[0] : nullptr);
  if (!s.ok()) return s;
  for (int l = 2; l < n; ++l) SE_CUDA(render_mip_alpha(mips[(size_t)l - 2], lw[l - 1], lh[l - 1], mips[(size_t)l - 1], stream));
  if (n == 1)
    SE_CUDA(cudaMemcpyAsync(mips[0], &d_color->w, sizeof(float), cudaMemcpyDeviceToDevice, stream));
  CompositeSrc src{};
  src.color = d_color;
  src.w = W;
  src.h = H;
  for (int l = 1; l < kOccLods; ++l) {
    const int lv = std::max(1, std::min(l, n - 1));  // the level textureLod reads at lod l
    src.alpha[l] = mips[(size_t)lv - 1];
    src.aw[l] = lv < n ? lw[lv] : 1;
    src.ah[l] = lv < n ? lh[lv] : 1;
  }
  const float4* bgd = nullptr;
  if (bg) {
    const size_t bytes = (size_t)bw * bh * sizeof(float4);
    if (bytes > bg_cap) {
      if (d_bg) cudaFree(d_bg);
      d_bg = nullptr;
      bg_cap = 0;
      cudaError_t e = cudaMalloc(&d_bg, bytes);
      if (e != cudaSuccess) return {SE_ERR_OUT_OF_MEMORY, std::string("cudaMalloc: ") + cudaGetErrorString(e)};
      bg_cap = bytes;
    }
    SE_CUDA(cudaMemcpyAsync(d_bg, bg, bytes, cudaMemcpyDefault, stream));
    bgd = d_bg;
  }
  if (!d_composite) {
    cudaError_t e = cudaMalloc(&d_composite, (size_t)W * H * sizeof(float4));
    if (e != cudaSuccess) return {SE_ERR_OUT_OF_MEMORY, std::string("cudaMalloc: ") + cudaGetErrorString(e)};
  }
  if (!d_coords) {
    cudaError_t e = cudaMalloc(&d_coords, composite_coords_bytes(W, H));
    if (e != cudaSuccess) return {SE_ERR_OUT_OF_MEMORY, std::string("cudaMalloc: ") + cudaGetErrorString(e)};
    SE_CUDA(render_composite_coords(d_coords, W, H, &coords, stream));
  }
  Timed* t = nullptr;
  if (timing) {
    s = timing_begin(3, (long long)W * H, 1, &t);
    if (!s.ok()) return s;
  }
  SE_CUDA(render_composite(src, coords, light[0] ? light[lcur] : nullptr, bgd, bw, bh, kBlurSideWeight, d_composite,
                           stream));
  if (t) SE_CUDA(cudaEventRecord(t->b, stream));
  return Status::Ok();
}

Status World::ensure_copy_streams() {
  if (!copy_streams[0])
    for (auto& cs : copy_streams) SE_CUDA(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
  return Status::Ok();
}

Status World::read_grid_u8_overlapped(uint8_t* host) {
  const size_t cells = (size_t)W * H;
  const int nmat = rs->num_materials();
  if (nmat > 256) return {SE_ERR_INVALID_ARGUMENT, "ids fit a byte only for rule sets of at most 256 materials"};
  Status st = ensure_copy_streams();
  if (!st.ok()) return st;
  if (!stage8[0]) {
    for (int i = 0; i < 2; ++i) {
      cudaError_t e = cudaMalloc(&stage8[i], cells);
      if (e != cudaSuccess) return {SE_ERR_OUT_OF_MEMORY, std::string("cudaMalloc: ") + cudaGetErrorString(e)};
      SE_CUDA(cudaEventCreateWithFlags(&stage8_ready[i], cudaEventDisableTiming));
      for (int c = 0; c < kCopyStreams; ++c) {
        SE_CUDA(cudaEventCreateWithFlags(&stage8_done[i][c], cudaEventDisableTiming));
        SE_CUDA(cudaEventRecord(stage8_done[i][c], copy_streams[c]));
      }
    }
  }
  const int i = stage8_i;
  stage8_i ^= 1;
  for (int c = 0; c < kCopyStreams; ++c)  // the previous host copy out of this stage has finished
    SE_CUDA(cudaStreamWaitEvent(stream, stage8_done[i][c], 0));
  SE_CUDA(pack_ids_u8(buf[cur], stage8[i], cells, (uint32_t)nmat, stream));
  SE_CUDA(cudaEventRecord(stage8_ready[i], stream));
  const size_t part = (cells + kCopyStreams - 1) / kCopyStreams;
  for (int c = 0; c < kCopyStreams; ++c) {
    const size_t a = std::min(cells, (size_t)c * part), b = std::min(cells, a + part);
    SE_CUDA(cudaStreamWaitEvent(copy_streams[c], stage8_ready[i], 0));
    if (b > a) SE_CUDA(cudaMemcpyAsync(host + a, stage8[i] + a, b - a, cudaMemcpyDeviceToHost, copy_streams[c]));
    SE_CUDA(cudaEventRecord(stage8_done[i][c], copy_streams[c]));
  }
  return Status::Ok();
}

Status World::read_grid_overlapped(uint32_t* host) {
  const size_t cells = (size_t)W * H, bytes = cells * sizeof(uint32_t);
  Status cs_st = ensure_copy_streams();
  if (!cs_st.ok()) return cs_st;
  if (!stage[0]) {
    for (int i = 0; i < 2; ++i) {
      cudaError_t e = cudaMalloc(&stage[i], bytes);
      if (e != cudaSuccess) return {SE_ERR_OUT_OF_MEMORY, std::string("cudaMalloc: ") + cudaGetErrorString(e)};
      SE_CUDA(cudaEventCreateWithFlags(&stage_ready[i], cudaEventDisableTiming));
      for (int c = 0; c < kCopyStreams; ++c) {
        SE_CUDA(cudaEventCreateWithFlags(&stage_done[i][c], cudaEventDisableTiming));
        SE_CUDA(cudaEventRecord(stage_done[i][c], copy_streams[c]));
      }
    }
  }
  const int i = stage_i;
  stage_i ^= 1;
  for (int c = 0; c < kCopyStreams; ++c)  // the previous host copy out of this stage has finished
    SE_CUDA(cudaStreamWaitEvent(stream, stage_done[i][c], 0));
  SE_CUDA(cudaMemcpyAsync(stage[i], buf[cur], bytes, cudaMemcpyDeviceToDevice, stream));
  SE_CUDA(cudaEventRecord(stage_ready[i], stream));
  const size_t part = (cells + kCopyStreams - 1) / kCopyStreams;
  for (int c = 0; c < kCopyStreams; ++c) {
    const size_t a = std::min(cells, (size_t)c * part), b = std::min(cells, a + part);
    SE_CUDA(cudaStreamWaitEvent(copy_streams[c], stage_ready[i], 0));
    if (b > a)
      SE_CUDA(cudaMemcpyAsync(host + a, stage[i] + a, (b - a) * sizeof(uint32_t), cudaMemcpyDeviceToHost,
                              copy_streams[c]));
    SE_CUDA(cudaEventRecord(stage_done[i][c], copy_streams[c]));
  }
  return Status::Ok();
}

Status World::synchronize_all() {
  SE_CUDA(cudaStreamSynchronize(stream));
  for (auto& cs : copy_streams)
    if (cs) SE_CUDA(cudaStreamSynchronize(cs));
  return Status::Ok();
}

Status World::digest(unsigned long long* out) {
  SE_CUDA(grid_digest(buf[cur], (unsigned long long)W * H, d_scratch, stream));
  SE_CUDA(cudaMemcpyAsync(out, d_scratch, sizeof(unsigned long long), cudaMemcpyDeviceToHost, stream));
  SE_CUDA(cudaStreamSynchronize(stream));
  return Status::Ok();
}

Status World::histogram(unsigned long long* counts, int nbins) {
  if (nbins < 1 || nbins > 257) return {SE_ERR_INVALID_ARGUMENT, "nbins must be in [1, 257]"};
  SE_CUDA(grid_histogram(buf[cur], (unsigned long long)W * H, nbins, d_scratch, stream));
  SE_CUDA(cudaMemcpyAsync(counts, d_scratch, sizeof(unsigned long long) * (size_t)nbins, cudaMemcpyDeviceToHost,
                          stream));
  SE_CUDA(cudaStreamSynchronize(stream));
  return Status::Ok();
}

}  // namespace se::rt
