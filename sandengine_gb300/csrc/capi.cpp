// The C ABI (include/sandengine.h).  Every entry point catches everything: no exception
// or abort crosses the boundary.
#include <cstdio>
#include <cstring>
#include <fstream>
#include <memory>
#include <sstream>
#include <string>

#include "../../include/sandengine.h"
#include "lang/codegen.hpp"
#include "lang/lang.hpp"
#include "runtime/batch.hpp"
#include "runtime/engine.hpp"
#include "runtime/server.hpp"
#include "runtime/snapshot.hpp"

#define SE_API extern "C" __attribute__((visibility("default")))

struct se_ruleset {
  std::shared_ptr<se::rt::Ruleset> rs;
};
struct se_world {
  std::unique_ptr<se::rt::World> w;
};

namespace {

thread_local std::string g_last_error;

int fail(int code, const std::string& msg) {
  g_last_error = msg;
  return code;
}
int ret(const se::rt::Status& s) {
  if (!s.ok()) return fail(s.code, s.msg);
  return SE_OK;
}

int parse_kind_code(const std::string& kind) {
  if (kind == "MissingField") return SE_ERR_MISSING_FIELD;
  if (kind == "InvalidType") return SE_ERR_INVALID_TYPE;
  if (kind == "NotFound") return SE_ERR_NOT_FOUND;
  if (kind == "NotRecognized") return SE_ERR_NOT_RECOGNIZED;
  if (kind == "Yaml") return SE_ERR_YAML;
  if (kind == "Panic") return SE_ERR_PANIC;
  if (kind == "Glsl") return SE_ERR_GLSL;
  if (kind == "Unsupported") return SE_ERR_UNSUPPORTED;
  return SE_ERR_INVALID_ARGUMENT;
}

template <class F>
int guard(F&& f) {
  try {
    return f();
  } catch (const std::bad_alloc&) {
    return fail(SE_ERR_OUT_OF_MEMORY, "host allocation failed");
  } catch (const std::exception& e) {
    return fail(SE_ERR_INVALID_ARGUMENT, e.what());
  } catch (...) {
    return fail(SE_ERR_INVALID_ARGUMENT, "unknown error");
  }
}

}  // namespace

SE_API const char* se_last_error(void) { return g_last_error.c_str(); }
SE_API int se_version(void) { return 100; }

SE_API int se_ruleset_parse(const char* yaml_text, se_ruleset** out) {
  return guard([&] {
    if (!yaml_text || !out) return fail(SE_ERR_INVALID_ARGUMENT, "null argument");
    *out = nullptr;
    auto rs = std::make_shared<se::rt::Ruleset>();
    se::lang::ParseError err;
    if (!se::lang::parse_string(yaml_text, &rs->parsed, &err)) return fail(parse_kind_code(err.kind), err.message);
    rs->materials_glsl = se::lang::materials_glsl(rs->parsed);
    rs->rules_glsl = se::lang::rules_glsl(rs->parsed);
    // Like the reference, parsing succeeds even when the generated rule code cannot be
    // built; that failure is reported when the kernels are built (se_ruleset_compile,
    // se_world_create), where the reference panics building its shader.
    if (!se::lang::generate_cuda(rs->parsed, &rs->cuda, &err)) {
      rs->codegen_code = parse_kind_code(err.kind);
      rs->codegen_message = err.message;
    }
    *out = new se_ruleset{rs};
    return (int)SE_OK;
  });
}

SE_API int se_ruleset_parse_path(const char* path, se_ruleset** out) {
  return guard([&] {
    if (!path || !out) return fail(SE_ERR_INVALID_ARGUMENT, "null argument");
    std::ifstream f(path, std::ios::binary);
    if (!f) return fail(SE_ERR_INVALID_ARGUMENT, std::string("cannot read ") + path);
    std::stringstream ss;
    ss << f.rdbuf();
    std::string text = ss.str();
    return se_ruleset_parse(text.c_str(), out);
  });
}

SE_API int se_ruleset_text(const se_ruleset* rs, int which, char* buf, size_t cap, size_t* len) {
  return guard([&] {
    if (!rs) return fail(SE_ERR_INVALID_ARGUMENT, "null ruleset");
    const std::string* s;
    std::string full;
    if (which == 0) s = &rs->rs->materials_glsl;
    else if (which == 1) s = &rs->rs->rules_glsl;
    else if (which == 2) s = &rs->rs->cuda.source;
    else if (which == 3) s = &(full = rs->rs->device_source());
    else return fail(SE_ERR_INVALID_ARGUMENT, "which must be 0, 1, 2 or 3");
    if (len) *len = s->size();
    if (buf && cap) {
      size_t n = std::min(cap - 1, s->size());
      memcpy(buf, s->data(), n);
      buf[n] = '\0';
      if (n < s->size()) return fail(SE_ERR_BUFFER_TOO_SMALL, "buffer too small");
    }
    return (int)SE_OK;
  });
}

SE_API int se_ruleset_set_checked(se_ruleset* rs, int enable) {
  return guard([&] {
    if (!rs) return fail(SE_ERR_INVALID_ARGUMENT, "null ruleset");
    std::lock_guard<std::mutex> g(rs->rs->mu);
    if (rs->rs->compiled) return fail(SE_ERR_INVALID_ARGUMENT, "the rule set is already compiled");
    rs->rs->checked = enable != 0;
    return (int)SE_OK;
  });
}

SE_API int se_ruleset_check_word(se_ruleset* rs, unsigned int* word, int reset) {
  return guard([&] {
    if (!rs || !word) return fail(SE_ERR_INVALID_ARGUMENT, "null argument");
    return ret(rs->rs->check_word(word, reset != 0));
  });
}

SE_API int se_ruleset_compile(se_ruleset* rs) {
  return guard([&] {
    if (!rs) return fail(SE_ERR_INVALID_ARGUMENT, "null ruleset");
    return ret(rs->rs->compile());
  });
}

SE_API int se_ruleset_table(se_ruleset* rs, uint16_t* table, size_t cap_entries, uint32_t* bits, size_t cap_words,
                            unsigned long long* entries, unsigned long long* static_words) {
  return guard([&] {
    if (!rs || !entries || !static_words) return fail(SE_ERR_INVALID_ARGUMENT, "null argument");
    se::rt::Ruleset& r = *rs->rs;
    se::rt::Status s = r.ensure_loaded();
    if (!s.ok()) return ret(s);
    *entries = r.cuda.lut_entries;
    *static_words = r.cuda.lut_static_words;
    if (!r.d_lut) return (int)SE_OK;
    if (table) {
      const size_t n = (size_t)std::min<unsigned long long>(cap_entries, r.cuda.lut_entries);
      cudaError_t e = cudaMemcpy(table, r.d_lut, n * sizeof(uint16_t), cudaMemcpyDeviceToHost);
      if (e != cudaSuccess) return fail(SE_ERR_CUDA, std::string("cudaMemcpy: ") + cudaGetErrorString(e));
    }
    if (bits) {
      const size_t off = ((size_t)r.cuda.lut_entries * sizeof(uint16_t) + 15) & ~(size_t)15;
      const size_t n = (size_t)std::min<unsigned long long>(cap_words, r.cuda.lut_static_words);
      cudaError_t e = cudaMemcpy(bits, reinterpret_cast<const char*>(r.d_lut) + off, n * 4, cudaMemcpyDeviceToHost);
      if (e != cudaSuccess) return fail(SE_ERR_CUDA, std::string("cudaMemcpy: ") + cudaGetErrorString(e));
    }
    return (int)SE_OK;
  });
}

SE_API int se_ruleset_num_materials(const se_ruleset* rs, int* n) {
  return guard([&] {
    if (!rs || !n) return fail(SE_ERR_INVALID_ARGUMENT, "null argument");
    *n = rs->rs->num_materials();
    return (int)SE_OK;
  });
}

SE_API int se_ruleset_material_id(const se_ruleset* rs, const char* name, int* id) {
  return guard([&] {
    if (!rs || !name || !id) return fail(SE_ERR_INVALID_ARGUMENT, "null argument");
    for (auto& m : rs->rs->parsed.materials)
      if (m.name == name) {
        *id = (int)m.id;
        return (int)SE_OK;
      }
    return fail(SE_ERR_NOT_FOUND, std::string("no material named ") + name);
  });
}

SE_API void se_ruleset_free(se_ruleset* rs) { delete rs; }

SE_API int se_world_create_band(se_ruleset* rs, int width, int world_height, int row0, int rows, int halo,
                                se_world** out) {
  return guard([&] {
    if (!rs || !out) return fail(SE_ERR_INVALID_ARGUMENT, "null argument");
    *out = nullptr;
    auto w = std::make_unique<se::rt::World>();
    se::rt::Status s = w->create_band(rs->rs, width, world_height, row0, rows, halo);
    if (!s.ok()) return ret(s);
    *out = new se_world{std::move(w)};
    return (int)SE_OK;
  });
}

SE_API int se_world_band_info(const se_world* w, int* buffer_row0, int* buffer_rows, int* world_height,
                              int* halo) {
  return guard([&] {
    if (!w || !buffer_row0 || !buffer_rows || !world_height || !halo)
      return fail(SE_ERR_INVALID_ARGUMENT, "null argument");
    *buffer_row0 = w->w->ya;
    *buffer_rows = w->w->H;
    *world_height = w->w->wh;
    *halo = w->w->halo;
    return (int)SE_OK;
  });
}

SE_API int se_world_copy_rows(se_world* w, int row, int nrows, void* ptr, int to_world) {
  return guard([&] {
    if (!w || !ptr || nrows < 0) return fail(SE_ERR_INVALID_ARGUMENT, "bad argument");
    auto& W = *w->w;
    if (row < W.ya || (int64_t)row + nrows > (int64_t)W.ya + W.H)
      return fail(SE_ERR_INVALID_ARGUMENT, "rows outside the world's buffer");
    if (nrows == 0) return (int)SE_OK;
    uint32_t* g = W.buf[W.cur] + (size_t)(row - W.ya) * W.W;
    const size_t bytes = (size_t)nrows * W.W * sizeof(uint32_t);
    cudaError_t e = to_world ? cudaMemcpyAsync(g, ptr, bytes, cudaMemcpyDefault, W.stream)
                             : cudaMemcpyAsync(ptr, g, bytes, cudaMemcpyDefault, W.stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(W.stream);
    if (e != cudaSuccess) return fail(SE_ERR_CUDA, std::string("cudaMemcpyAsync: ") + cudaGetErrorString(e));
    return (int)SE_OK;
  });
}

SE_API int se_world_set_light(se_world* w, int enable) {
  return guard([&] {
    if (!w) return fail(SE_ERR_INVALID_ARGUMENT, "null world");
    return ret(w->w->set_light(enable != 0));
  });
}

// Copies between the current light field (device) and a host or device RGBA32F buffer.
static int light_copy(se_world* w, void* p, size_t n_floats, bool to_world) {
  if (!w || !p) return fail(SE_ERR_INVALID_ARGUMENT, "null argument");
  auto& W = *w->w;
  if (!W.light[0]) return fail(SE_ERR_INVALID_ARGUMENT, "the light field is off (se_world_set_light)");
  const size_t need = (size_t)W.W * W.H * 4;
  if (n_floats < need) return fail(SE_ERR_INVALID_ARGUMENT, "buffer smaller than width * height * 4 floats");
  float4* l = W.light[W.lcur];
  cudaError_t e = to_world ? cudaMemcpyAsync(l, p, need * 4, cudaMemcpyDefault, W.stream)
                           : cudaMemcpyAsync(p, l, need * 4, cudaMemcpyDefault, W.stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(W.stream);
  if (e != cudaSuccess) return fail(SE_ERR_CUDA, std::string("cudaMemcpyAsync: ") + cudaGetErrorString(e));
  return (int)SE_OK;
}

SE_API int se_world_get_light(se_world* w, float* rgba, size_t n_floats) {
  return guard([&] { return light_copy(w, rgba, n_floats, false); });
}

SE_API int se_world_set_light_field(se_world* w, const float* rgba, size_t n_floats) {
  return guard([&] { return light_copy(w, const_cast<float*>(rgba), n_floats, true); });
}

SE_API int se_world_render_color(se_world* w, float* rgba, size_t n_floats) {
  return guard([&] {
    if (!w || !rgba) return fail(SE_ERR_INVALID_ARGUMENT, "null argument");
    auto& W = *w->w;
    const size_t need = (size_t)W.W * W.H * 4;
    if (n_floats < need) return fail(SE_ERR_INVALID_ARGUMENT, "buffer smaller than width * height * 4 floats");
    se::rt::Status s = W.render_color();
    if (!s.ok()) return ret(s);
    cudaError_t e = cudaMemcpyAsync(rgba, W.d_color, need * 4, cudaMemcpyDefault, W.stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(W.stream);
    if (e != cudaSuccess) return fail(SE_ERR_CUDA, std::string("cudaMemcpyAsync: ") + cudaGetErrorString(e));
    return (int)SE_OK;
  });
}

SE_API int se_world_render_color_device(se_world* w, float** rgba) {
  return guard([&] {
    if (!w || !rgba) return fail(SE_ERR_INVALID_ARGUMENT, "null argument");
    se::rt::Status s = w->w->render_color();
    if (!s.ok()) return ret(s);
    *rgba = reinterpret_cast<float*>(w->w->d_color);
    return (int)SE_OK;
  });
}

SE_API int se_world_composite(se_world* w, const float* bg_rgba, int bg_w, int bg_h, float* out_rgba,
                              size_t n_floats) {
  return guard([&] {
    if (!w || !out_rgba) return fail(SE_ERR_INVALID_ARGUMENT, "null argument");
    auto& W = *w->w;
    const size_t need = (size_t)W.W * W.H * 4;
    if (n_floats < need) return fail(SE_ERR_INVALID_ARGUMENT, "buffer smaller than width * height * 4 floats");
    se::rt::Status s = W.composite(bg_rgba, bg_w, bg_h);
    if (!s.ok()) return ret(s);
    cudaError_t e = cudaMemcpyAsync(out_rgba, W.d_composite, need * 4, cudaMemcpyDefault, W.stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(W.stream);
    if (e != cudaSuccess) return fail(SE_ERR_CUDA, std::string("cudaMemcpyAsync: ") + cudaGetErrorString(e));
    return (int)SE_OK;
  });
}

SE_API int se_world_composite_device(se_world* w, const float* bg_rgba, int bg_w, int bg_h, float** out_rgba) {
  return guard([&] {
    if (!w || !out_rgba) return fail(SE_ERR_INVALID_ARGUMENT, "null argument");
    se::rt::Status s = w->w->composite(bg_rgba, bg_w, bg_h);
    if (!s.ok()) return ret(s);
    *out_rgba = reinterpret_cast<float*>(w->w->d_composite);
    return (int)SE_OK;
  });
}

SE_API int se_world_create(se_ruleset* rs, int width, int height, se_world** out) {
  return guard([&] {
    if (!rs || !out) return fail(SE_ERR_INVALID_ARGUMENT, "null argument");
    *out = nullptr;
    auto w = std::make_unique<se::rt::World>();
    se::rt::Status s = w->create(rs->rs, width, height);
    if (!s.ok()) return ret(s);
    *out = new se_world{std::move(w)};
    return (int)SE_OK;
  });
}

SE_API void se_world_destroy(se_world* w) {
  if (w && w->w && w->w->stream) cudaStreamSynchronize(w->w->stream);
  delete w;
}

SE_API int se_world_set_stream(se_world* w, void* s) {
  return guard([&] {
    if (!w) return fail(SE_ERR_INVALID_ARGUMENT, "null world");
    w->w->stream = s ? (cudaStream_t)s : w->w->own_stream;
    return (int)SE_OK;
  });
}

SE_API int se_world_get_stream(se_world* w, void** s) {
  return guard([&] {
    if (!w || !s) return fail(SE_ERR_INVALID_ARGUMENT, "null argument");
    *s = (void*)w->w->stream;
    return (int)SE_OK;
  });
}

SE_API int se_world_set_steps_per_launch(se_world* w, int k) {
  return guard([&] {
    if (!w || k < 0) return fail(SE_ERR_INVALID_ARGUMENT, "bad argument");
    int kmax = 0;
    for (auto& t : se::rt::tile_variants()) kmax = std::max(kmax, t.kmax);
    if (k > kmax) return fail(SE_ERR_INVALID_ARGUMENT, "at most " + std::to_string(kmax) + " frames per launch");
    w->w->steps_per_launch = k;
    return (int)SE_OK;
  });
}

SE_API int se_world_set_tile(se_world* w, int tile_w, int tile_h, int k) {
  return guard([&] {
    if (!w) return fail(SE_ERR_INVALID_ARGUMENT, "null world");
    for (auto& t : se::rt::tile_variants())
      if (t.tw == tile_w && t.th == tile_h && t.kmax == k) {
        auto& W = *w->w;
        if (k == 1) {
          W.single = &t;
        } else {
          W.fused = &t;
          W.steps_per_launch = 0;
        }
        return (int)SE_OK;
      }
    return fail(SE_ERR_INVALID_ARGUMENT, "no compiled tile variant " + std::to_string(tile_w) + "x" +
                                             std::to_string(tile_h) + " with " + std::to_string(k) +
                                             " frames per launch");
  });
}

SE_API int se_world_get_tile(const se_world* w, int* tile_w, int* tile_h, int* k) {
  return guard([&] {
    if (!w || !tile_w || !tile_h || !k) return fail(SE_ERR_INVALID_ARGUMENT, "null argument");
    const auto& W = *w->w;
    const se::rt::TileVariant* v = W.steps_per_launch > 0 ? nullptr : W.fused;
    if (!v)
      for (auto& t : se::rt::tile_variants())
        if (t.kmax >= std::max(1, W.steps_per_launch) && (!v || t.kmax < v->kmax)) v = &t;
    *tile_w = v ? v->tw : 0;
    *tile_h = v ? v->th : 0;
    *k = v ? v->kmax : 0;
    return (int)SE_OK;
  });
}

namespace {
int grid_copy(se_world* w, void* host, size_t count, bool to_device, bool sync) {
  if (!w || !host) return fail(SE_ERR_INVALID_ARGUMENT, "null argument");
  auto& W = *w->w;
  if (count != (size_t)W.W * W.H) return fail(SE_ERR_INVALID_ARGUMENT, "count must be width*height");
  const size_t bytes = count * sizeof(uint32_t);
  cudaError_t e = to_device ? cudaMemcpyAsync(W.buf[W.cur], host, bytes, cudaMemcpyHostToDevice, W.stream)
                            : cudaMemcpyAsync(host, W.buf[W.cur], bytes, cudaMemcpyDeviceToHost, W.stream);
  if (e == cudaSuccess && sync) e = cudaStreamSynchronize(W.stream);
  if (e != cudaSuccess) return fail(SE_ERR_CUDA, std::string("grid copy: ") + cudaGetErrorString(e));
  return (int)SE_OK;
}
}  // namespace

SE_API int se_world_set_grid(se_world* w, const uint32_t* cells, size_t count) {
  return guard([&] { return grid_copy(w, (void*)cells, count, true, true); });
}
SE_API int se_world_get_grid(se_world* w, uint32_t* cells, size_t count) {
  return guard([&] { return grid_copy(w, cells, count, false, true); });
}
SE_API int se_world_set_grid_async(se_world* w, const uint32_t* cells, size_t count) {
  return guard([&] { return grid_copy(w, (void*)cells, count, true, false); });
}
SE_API int se_world_get_grid_async(se_world* w, uint32_t* cells, size_t count) {
  return guard([&] { return grid_copy(w, cells, count, false, false); });
}

SE_API int se_world_read_grid_u8_overlapped(se_world* w, uint8_t* cells, size_t count) {
  return guard([&] {
    if (!w || !cells) return fail(SE_ERR_INVALID_ARGUMENT, "null argument");
    if (count != (size_t)w->w->W * w->w->H) return fail(SE_ERR_INVALID_ARGUMENT, "count must be width * height");
    return ret(w->w->read_grid_u8_overlapped(cells));
  });
}

SE_API int se_world_read_grid_overlapped(se_world* w, uint32_t* cells, size_t count) {
  return guard([&] {
    if (!w || !cells) return fail(SE_ERR_INVALID_ARGUMENT, "null argument");
    if (count != (size_t)w->w->W * w->w->H) return fail(SE_ERR_INVALID_ARGUMENT, "count must be width * height");
    return ret(w->w->read_grid_overlapped(cells));
  });
}

SE_API int se_world_device_grid(se_world* w, uint32_t** p) {
  return guard([&] {
    if (!w || !p) return fail(SE_ERR_INVALID_ARGUMENT, "null argument");
    *p = w->w->buf[w->w->cur];
    return (int)SE_OK;
  });
}

SE_API int se_world_set_frame(se_world* w, int32_t frame) {
  return guard([&] {
    if (!w) return fail(SE_ERR_INVALID_ARGUMENT, "null world");
    if (frame < 0) return fail(SE_ERR_INVALID_ARGUMENT, "frame must be >= 0 (frame % 4 of a negative is undefined in GLSL)");
    w->w->frame = frame;
    return (int)SE_OK;
  });
}

SE_API int se_world_get_frame(const se_world* w, int32_t* frame) {
  return guard([&] {
    if (!w || !frame) return fail(SE_ERR_INVALID_ARGUMENT, "null argument");
    *frame = w->w->frame;
    return (int)SE_OK;
  });
}

SE_API int se_world_step(se_world* w, int nframes, const se_modification* mods, int nmods) {
  return guard([&] {
    if (!w) return fail(SE_ERR_INVALID_ARGUMENT, "null world");
    return ret(w->w->step(nframes, mods, nmods));
  });
}

SE_API int se_world_synchronize(se_world* w) {
  return guard([&] {
    if (!w) return fail(SE_ERR_INVALID_ARGUMENT, "null world");
    return ret(w->w->synchronize_all());
  });
}

SE_API int se_world_digest(se_world* w, uint64_t* digest) {
  return guard([&] {
    if (!w || !digest) return fail(SE_ERR_INVALID_ARGUMENT, "null argument");
    unsigned long long d = 0;
    se::rt::Status s = w->w->digest(&d);
    if (!s.ok()) return ret(s);
    *digest = d;
    return (int)SE_OK;
  });
}

SE_API int se_world_histogram(se_world* w, uint64_t* counts, int nbins) {
  return guard([&] {
    if (!w || !counts) return fail(SE_ERR_INVALID_ARGUMENT, "null argument");
    return ret(w->w->histogram(reinterpret_cast<unsigned long long*>(counts), nbins));
  });
}

// Material counts of any device grid without allocating device memory: the counters live
// in a fixed static device array (see se_grid_histogram_noalloc in include/sandengine.h).
SE_API int se_grid_histogram_noalloc(const uint32_t* device_cells, uint64_t count, int nbins,
                                     uint64_t* host_counts, void* cuda_stream) {
  return guard([&] {
    if (!device_cells || !host_counts) return fail(SE_ERR_INVALID_ARGUMENT, "null argument");
    const int maxb = se::rt::noalloc_max_bins();
    if (nbins < 1 || nbins > maxb)
      return fail(SE_ERR_INVALID_ARGUMENT, "nbins must be in [1, " + std::to_string(maxb) +
                                               "]: the allocation-free histogram has a fixed scratch of " +
                                               std::to_string(maxb) + " counters");
    cudaError_t e = se::rt::histogram_noalloc(device_cells, (unsigned long long)count, nbins,
                                              reinterpret_cast<unsigned long long*>(host_counts),
                                              (cudaStream_t)cuda_stream);
    if (e != cudaSuccess) return fail(SE_ERR_CUDA, std::string("histogram (no-alloc): ") + cudaGetErrorString(e));
    return (int)SE_OK;
  });
}

SE_API int se_world_autotune(se_world* w, int reps, int* best_k) {
  return guard([&] {
    if (!w) return fail(SE_ERR_INVALID_ARGUMENT, "null world");
    int k = 0;
    se::rt::Status s = w->w->autotune(reps, &k);
    if (!s.ok()) return ret(s);
    w->w->steps_per_launch = 0;
    if (best_k) *best_k = k;
    return (int)SE_OK;
  });
}

SE_API int se_world_set_timing(se_world* w, int enable) {
  return guard([&] {
    if (!w) return fail(SE_ERR_INVALID_ARGUMENT, "null world");
    w->w->timing = enable != 0;
    for (auto& u : w->w->timed_used) u = 0;
    return (int)SE_OK;
  });
}

SE_API int se_world_read_timing(se_world* w, double* kernel_ms, long long* launches, long long* cell_frames,
                                long long* cells) {
  return guard([&] {
    if (!w || !kernel_ms || !launches || !cell_frames || !cells) return fail(SE_ERR_INVALID_ARGUMENT, "null argument");
    return ret(w->w->timing_read(0, kernel_ms, launches, cell_frames, cells));
  });
}

SE_API int se_world_peek_timing_frames(se_world* w, int frames, double* kernel_ms, long long* launches) {
  return guard([&] {
    if (!w || !kernel_ms || !launches) return fail(SE_ERR_INVALID_ARGUMENT, "null argument");
    return ret(w->w->timing_peek_frames(frames, kernel_ms, launches));
  });
}

SE_API int se_world_read_pass_timing(se_world* w, int pass, double* kernel_ms, long long* launches,
                                     long long* cells) {
  return guard([&] {
    if (!w || !kernel_ms || !launches || !cells) return fail(SE_ERR_INVALID_ARGUMENT, "null argument");
    long long cf = 0;
    return ret(w->w->timing_read(pass, kernel_ms, launches, &cf, cells));
  });
}

// ---- batches ---------------------------------------------------------------------------
struct se_batch {
  std::unique_ptr<se::rt::Batch> b;
};

SE_API int se_batch_create(se_ruleset* rs, int n, const int* widths, const int* heights, se_batch** out) {
  return guard([&] {
    if (!rs || !out) return fail(SE_ERR_INVALID_ARGUMENT, "null argument");
    *out = nullptr;
    auto b = std::make_unique<se::rt::Batch>();
    se::rt::Status s = b->create(rs->rs, n, widths, heights);
    if (!s.ok()) return ret(s);
    *out = new se_batch{std::move(b)};
    return (int)SE_OK;
  });
}

SE_API void se_batch_destroy(se_batch* b) {
  if (b && b->b && b->b->stream) cudaStreamSynchronize(b->b->stream);
  delete b;
}

SE_API int se_batch_set_grid(se_batch* b, int world, const uint32_t* cells, size_t count) {
  return guard([&] {
    if (!b) return fail(SE_ERR_INVALID_ARGUMENT, "null batch");
    return ret(b->b->set_grid(world, cells, count));
  });
}

SE_API int se_batch_get_grid(se_batch* b, int world, uint32_t* cells, size_t count) {
  return guard([&] {
    if (!b) return fail(SE_ERR_INVALID_ARGUMENT, "null batch");
    return ret(b->b->get_grid(world, cells, count));
  });
}

SE_API int se_batch_set_frame(se_batch* b, int world, int32_t frame) {
  return guard([&] {
    if (!b) return fail(SE_ERR_INVALID_ARGUMENT, "null batch");
    return ret(b->b->set_frame(world, frame));
  });
}

SE_API int se_batch_get_frame(const se_batch* b, int world, int32_t* frame) {
  return guard([&] {
    if (!b || !frame || world < 0 || world >= b->b->n) return fail(SE_ERR_INVALID_ARGUMENT, "bad argument");
    *frame = b->b->desc[(size_t)world].frame;
    return (int)SE_OK;
  });
}

SE_API int se_batch_step(se_batch* b, int nframes) {
  return guard([&] {
    if (!b) return fail(SE_ERR_INVALID_ARGUMENT, "null batch");
    return ret(b->b->step(nframes));
  });
}

SE_API int se_batch_step_plain(se_batch* b, int nframes) {
  return guard([&] {
    if (!b) return fail(SE_ERR_INVALID_ARGUMENT, "null batch");
    return ret(b->b->step_plain(nframes));
  });
}

SE_API int se_batch_autotune(se_batch* b, int reps, int* best_k) {
  return guard([&] {
    if (!b) return fail(SE_ERR_INVALID_ARGUMENT, "null batch");
    return ret(b->b->autotune(reps, best_k));
  });
}

SE_API int se_batch_set_steps_per_launch(se_batch* b, int k) {
  return guard([&] {
    if (!b || k < 1) return fail(SE_ERR_INVALID_ARGUMENT, "k must be >= 1");
    const se::rt::TileVariant* v = nullptr;
    for (auto& t : se::rt::tile_variants())
      if (t.kmax >= k && (!v || t.kmax < v->kmax)) v = &t;
    if (!v) return fail(SE_ERR_INVALID_ARGUMENT, "no kernel variant for this many frames per launch");
    b->b->steps_per_launch = k;
    return ret(b->b->set_variant(v));
  });
}

SE_API int se_batch_set_resident_limit(se_batch* b, size_t bytes) {
  return guard([&] {
    if (!b) return fail(SE_ERR_INVALID_ARGUMENT, "null batch");
    return ret(b->b->set_resident_limit(bytes));
  });
}

SE_API int se_batch_synchronize(se_batch* b) {
  return guard([&] {
    if (!b) return fail(SE_ERR_INVALID_ARGUMENT, "null batch");
    cudaError_t e = cudaStreamSynchronize(b->b->stream);
    if (e != cudaSuccess) return fail(SE_ERR_CUDA, std::string("synchronize: ") + cudaGetErrorString(e));
    return (int)SE_OK;
  });
}

SE_API int se_batch_get_stream(se_batch* b, void** s) {
  return guard([&] {
    if (!b || !s) return fail(SE_ERR_INVALID_ARGUMENT, "null argument");
    *s = (void*)b->b->stream;
    return (int)SE_OK;
  });
}

SE_API int se_batch_info(const se_batch* b, int* resident_worlds, int* tiled_worlds, long long* cells,
                         int* steps_per_launch) {
  return guard([&] {
    if (!b) return fail(SE_ERR_INVALID_ARGUMENT, "null batch");
    int r = 0;
    for (auto& c : b->b->resident) r += (int)c.ids.size();
    if (resident_worlds) *resident_worlds = r;
    if (tiled_worlds) *tiled_worlds = (int)b->b->tiled.size();
    if (cells) *cells = b->b->cells;
    if (steps_per_launch) *steps_per_launch = b->b->variant ? b->b->variant->kmax : 0;
    return (int)SE_OK;
  });
}

// ---- serving -----------------------------------------------------------------------------
struct se_server {
  std::unique_ptr<se::rt::Server> s;
};

SE_API int se_server_create(se_ruleset* rs, long long budget_bytes, se_server** out) {
  return guard([&] {
    if (!rs || !out) return fail(SE_ERR_INVALID_ARGUMENT, "null argument");
    *out = nullptr;
    auto s = std::make_unique<se::rt::Server>();
    se::rt::Status st = s->create(rs->rs, budget_bytes);
    if (!st.ok()) return ret(st);
    *out = new se_server{std::move(s)};
    return (int)SE_OK;
  });
}

SE_API void se_server_destroy(se_server* s) { delete s; }

SE_API int se_server_set_frames_per_iteration(se_server* s, int k) {
  return guard([&] {
    if (!s) return fail(SE_ERR_INVALID_ARGUMENT, "null server");
    return ret(s->s->set_frames_per_iteration(k));
  });
}

SE_API int se_server_open_session(se_server* s, int width, int height, const uint32_t* cells, int32_t frame,
                                  int* session) {
  return guard([&] {
    if (!s || !session) return fail(SE_ERR_INVALID_ARGUMENT, "null argument");
    return ret(s->s->open_session(width, height, cells, frame, session));
  });
}

SE_API int se_server_close_session(se_server* s, int session) {
  return guard([&] {
    if (!s) return fail(SE_ERR_INVALID_ARGUMENT, "null server");
    return ret(s->s->close_session(session));
  });
}

SE_API int se_server_submit(se_server* s, int session, int nframes, const se_modification* mods, int nmods,
                            double arrival_ms, int* request) {
  return guard([&] {
    if (!s || !request) return fail(SE_ERR_INVALID_ARGUMENT, "null argument");
    return ret(s->s->submit(session, nframes, mods, nmods, arrival_ms, request));
  });
}

SE_API int se_server_run(se_server* s, int plain) {
  return guard([&] {
    if (!s) return fail(SE_ERR_INVALID_ARGUMENT, "null server");
    return ret(s->s->run(plain != 0));
  });
}

SE_API int se_server_stats_get(se_server* s, se_server_stats* out) {
  return guard([&] {
    if (!s || !out) return fail(SE_ERR_INVALID_ARGUMENT, "null argument");
    return ret(s->s->stats(out));
  });
}

SE_API int se_server_cancel(se_server* s, int request) {
  return guard([&] {
    if (!s) return fail(SE_ERR_INVALID_ARGUMENT, "null server");
    return ret(s->s->cancel(request));
  });
}

SE_API int se_server_request_latency(se_server* s, int request, double* latency_ms) {
  return guard([&] {
    if (!s || !latency_ms) return fail(SE_ERR_INVALID_ARGUMENT, "null argument");
    return ret(s->s->request_latency(request, latency_ms));
  });
}

SE_API int se_server_start(se_server* s, int plain) {
  return guard([&] {
    if (!s) return fail(SE_ERR_INVALID_ARGUMENT, "null server");
    return ret(s->s->start(plain != 0));
  });
}

SE_API int se_server_stop(se_server* s) {
  return guard([&] {
    if (!s) return fail(SE_ERR_INVALID_ARGUMENT, "null server");
    return ret(s->s->stop());
  });
}

SE_API int se_server_wait(se_server* s, int request, double timeout_ms, double* latency_ms) {
  return guard([&] {
    if (!s) return fail(SE_ERR_INVALID_ARGUMENT, "null server");
    bool done = false;
    return ret(s->s->wait(request, timeout_ms, &done, latency_ms));
  });
}

SE_API int se_server_poll(se_server* s, int request, int* done, double* latency_ms) {
  return guard([&] {
    if (!s || !done) return fail(SE_ERR_INVALID_ARGUMENT, "null argument");
    bool d = false;
    se::rt::Status st = s->s->wait(request, 0.0, &d, latency_ms);
    *done = d ? 1 : 0;
    if (st.code == SE_ERR_TIMEOUT) return (int)SE_OK;  // not done yet: *done = 0
    return ret(st);
  });
}

SE_API int se_server_get_grid(se_server* s, int session, uint32_t* cells, size_t count) {
  return guard([&] {
    if (!s || !cells) return fail(SE_ERR_INVALID_ARGUMENT, "null argument");
    return ret(s->s->get_grid(session, cells, count));
  });
}

// ---- snapshots ---------------------------------------------------------------------------
namespace {
se::rt::SnapshotHeader snapshot_header_for(const se::rt::Ruleset& rs, int W, int H, int32_t frame) {
  se::rt::SnapshotHeader h;
  h.width = (uint32_t)W;
  h.height = (uint32_t)H;
  h.frame = frame;
  h.num_materials = (uint32_t)rs.num_materials();
  h.ruleset_hash = se::rt::ruleset_fingerprint(rs.materials_glsl, rs.rules_glsl);
  return h;
}
int check_snapshot_matches(const se::rt::Ruleset& rs, const se::rt::SnapshotHeader& h) {
  if (h.num_materials != (uint32_t)rs.num_materials() ||
      h.ruleset_hash != se::rt::ruleset_fingerprint(rs.materials_glsl, rs.rules_glsl))
    return fail(SE_ERR_INVALID_ARGUMENT, "the snapshot was saved with a different rule set");
  return (int)SE_OK;
}
}  // namespace

SE_API int se_snapshot_info(const char* path, int* width, int* height, int32_t* frame) {
  return guard([&] {
    if (!path) return fail(SE_ERR_INVALID_ARGUMENT, "null path");
    se::rt::SnapshotHeader h;
    std::string err;
    if (!se::rt::snapshot_read_header(path, &h, &err)) return fail(SE_ERR_INVALID_ARGUMENT, err);
    if (width) *width = (int)h.width;
    if (height) *height = (int)h.height;
    if (frame) *frame = h.frame;
    return (int)SE_OK;
  });
}

SE_API int se_world_save(se_world* w, const char* path) {
  return guard([&] {
    if (!w || !path) return fail(SE_ERR_INVALID_ARGUMENT, "null argument");
    auto& W = *w->w;
    if (W.halo >= 0) return fail(SE_ERR_INVALID_ARGUMENT, "snapshots hold whole worlds, not bands");
    std::vector<uint32_t> cells((size_t)W.W * W.H);
    int rc = grid_copy(w, cells.data(), cells.size(), false, true);
    if (rc) return rc;
    std::string err;
    if (!se::rt::snapshot_write(path, snapshot_header_for(*W.rs, W.W, W.H, W.frame), cells.data(), &err))
      return fail(SE_ERR_INVALID_ARGUMENT, err);
    return (int)SE_OK;
  });
}

SE_API int se_world_load(se_world* w, const char* path) {
  return guard([&] {
    if (!w || !path) return fail(SE_ERR_INVALID_ARGUMENT, "null argument");
    auto& W = *w->w;
    if (W.halo >= 0) return fail(SE_ERR_INVALID_ARGUMENT, "snapshots hold whole worlds, not bands");
    se::rt::SnapshotHeader h;
    std::vector<uint32_t> cells;
    std::string err;
    if (!se::rt::snapshot_read(path, &h, &cells, &err)) return fail(SE_ERR_INVALID_ARGUMENT, err);
    if ((int)h.width != W.W || (int)h.height != W.H)
      return fail(SE_ERR_INVALID_ARGUMENT, "the snapshot's size differs from the world's");
    int rc = check_snapshot_matches(*W.rs, h);
    if (rc) return rc;
    rc = grid_copy(w, cells.data(), cells.size(), true, true);
    if (rc) return rc;
    W.frame = h.frame;
    return (int)SE_OK;
  });
}

SE_API int se_server_save_session(se_server* s, int session, const char* path) {
  return guard([&] {
    if (!s || !path) return fail(SE_ERR_INVALID_ARGUMENT, "null argument");
    int w = 0, h = 0;
    int32_t frame = 0;
    std::vector<uint32_t> cells;
    se::rt::Status st = s->s->session_state(session, &w, &h, &frame, &cells);
    if (!st.ok()) return ret(st);
    std::string err;
    if (!se::rt::snapshot_write(path, snapshot_header_for(*s->s->rs, w, h, frame), cells.data(), &err))
      return fail(SE_ERR_INVALID_ARGUMENT, err);
    return (int)SE_OK;
  });
}

SE_API int se_server_open_session_from(se_server* s, const char* path, int* session) {
  return guard([&] {
    if (!s || !path || !session) return fail(SE_ERR_INVALID_ARGUMENT, "null argument");
    se::rt::SnapshotHeader h;
    std::vector<uint32_t> cells;
    std::string err;
    if (!se::rt::snapshot_read(path, &h, &cells, &err)) return fail(SE_ERR_INVALID_ARGUMENT, err);
    int rc = check_snapshot_matches(*s->s->rs, h);
    if (rc) return rc;
    return ret(s->s->open_session((int)h.width, (int)h.height, cells.data(), h.frame, session));
  });
}

SE_API int se_server_get_frame(se_server* s, int session, int32_t* frame) {
  return guard([&] {
    if (!s || !frame) return fail(SE_ERR_INVALID_ARGUMENT, "null argument");
    return ret(s->s->session_state(session, nullptr, nullptr, frame, nullptr));
  });
}
