// Rule sets and worlds behind the C ABI.
#pragma once

#include <cuda_runtime.h>

#include <memory>
#include <mutex>
#include <string>
#include <vector>

#include "../lang/codegen.hpp"
#include "../lang/lang.hpp"
#include "../kernels/render.hpp"
#include "jit.hpp"

struct se_modification;

namespace se::rt {

// Longest world side (cells): tile grids stay within a launch's 65535 rows of CTAs.  A world
// also holds at most 2^36 cells.
constexpr int kMaxSide = 1 << 20;

struct Status {
  int code = 0;
  std::string msg;
  bool ok() const { return code == 0; }
  static Status Ok() { return {}; }
};

struct Ruleset {
  lang::ParsingResult parsed;
  std::string materials_glsl, rules_glsl;
  lang::CudaRules cuda;
  int codegen_code = 0;  // non-zero: the CUDA back end rejected the rule GLSL
  std::string codegen_message;
  std::string cubin;
  bool compiled = false;
  std::mutex mu;
  std::unique_ptr<Module> module;  // loaded on first use on a device
  // Block transition table (when cuda.lut_entries > 0), followed 16-byte aligned by the
  // bitset of static keys.
  uint16_t* d_lut = nullptr;
  // Per-material colour / emission / flags for the colour and light passes.
  RenderMat* d_render = nullptr;
  ~Ruleset();
  LutShape lut_shape() const { return {cuda.lut_entries, cuda.lut_static_words}; }
  // CHECKED build: the module is compiled with SE_CHECKED (index checks recorded in the
  // device word se_check_word); set before the first compile.
  bool checked = false;
  std::string device_source() const;
  Status check_word(unsigned int* word, bool reset);
  int num_materials() const { return (int)parsed.materials.size(); }
  Status compile();
  Status ensure_loaded();
};

// Host-side copy of the edit pass inputs, passed to se_edit by value (kernel parameter
// space holds up to 32 KB, so no device buffer or staging copy is needed).
struct alignas(16) EditParams {  // layout of SeEditParams in kernels/margolus.cuh
  int mods[256 * 8];  // 256 SeMod records of 8 ints
  int box[256 * 4];   // int4 x0, y0, x1, y1
  long long start[257];
};
static_assert(sizeof(EditParams) == 14352, "must match the device struct");

struct World {
  std::shared_ptr<Ruleset> rs;
  int W = 0, H = 0;  // buffer size: the whole world, or a band with its halo rows
  // A band of a taller world (halo >= 0): the buffers hold world rows [ya, ya + H) of a
  // W x wh world, the band's own rows plus up to `halo` rows either side.  Whole world:
  // wh = H, ya = 0, halo = -1.
  int wh = 0, ya = 0, halo = -1;
  int32_t frame = 0;
  uint32_t* buf[2] = {nullptr, nullptr};
  int cur = 0;
  unsigned long long* d_scratch = nullptr;  // 258 words for digests and histograms
  cudaStream_t own_stream = nullptr, stream = nullptr;
  int steps_per_launch = 0;  // 0: chosen by the autotuner on the first multi-frame step
  const TileVariant* fused = nullptr;   // variant for multi-frame launches
  const TileVariant* single = nullptr;  // variant for one-frame launches (edit frames)
  ~World();
  Status create(std::shared_ptr<Ruleset> r, int w, int h);
  // The band [row0, row0 + rows) of a w x world_h world with `halo` rows either side.
  Status create_band(std::shared_ptr<Ruleset> r, int w, int world_h, int row0, int rows, int halo);
  Status step(int nframes, const se_modification* mods, int nmods);
  // k frames with counters f0.. from buf[cur] into buf[cur^1]; commit=false leaves cur
  // (the world's state) unchanged, for tuning trials.
  Status launch_tiles(int f0, int k, const TileVariant* v, bool commit = true, const EditParams* edits = nullptr,
                      int nedits = 0);
  // Times every tile variant on this world (without changing it) and keeps the fastest
  // multi-frame and one-frame variants.  *best_k gets the chosen frames per launch.
  Status autotune(int reps, int* best_k);
  EditParams edit_params;  // the edit list of the current step's first launch (copied at launch)
  int default_k() const;
  // Opt-in per-launch CUDA-event timing (for roofline measurements) of the tile kernel
  // (pass 0), the light pass (1), the colour pass (2) and the composite (3, its pyramid
  // excluded).
  bool timing = false;
  struct Timed {
    cudaEvent_t a, b;
    long long cells;  // cells the launch covered
    int frames;       // frames the launch advanced
  };
  std::vector<Timed> timed[4];
  size_t timed_used[4] = {0, 0, 0, 0};
  Status timing_begin(int pass, long long cells, int frames, Timed** out);
  Status timing_read(int pass, double* ms, long long* launches, long long* cell_frames, long long* cells);
  Status timing_peek_frames(int frames, double* ms, long long* launches);  // tile launches of `frames` frames
  Status digest(unsigned long long* out);
  Status histogram(unsigned long long* counts, int nbins);

  // Colour and light outputs of the reference's setCell (opt-in).  With light on, every
  // frame runs as a one-frame launch followed by the light pass over the frame's old and
  // new grids; light[lcur] is the current field (RGBA32F per cell, zero at creation as the
  // reference's textures are).  The noise term of the colour depends only on the position
  // and is computed once per world.
  float4* light[2] = {nullptr, nullptr};
  int lcur = 0;
  float* d_noise = nullptr;
  float4* d_color = nullptr;
  Status set_light(bool on);
  Status light_frame();  // light pass for the frame just taken (old grid buf[cur ^ 1])
  // The current grid's colours into d_color; with alpha1, also the pyramid's level-1 alpha.
  Status render_color(float* alpha1 = nullptr);
  // Headless composite of the current grid (colour, its pyramid, the light field when
  // kept, an optional background image) into d_composite (RGBA32F per cell).
  std::vector<float*> mips;  // the colour pyramid's levels 1.. (alpha only)
  void* d_coords = nullptr;  // the composite's column and row tables (built once)
  CompositeCoords coords{};
  float4* d_composite = nullptr;
  float4* d_bg = nullptr;
  size_t bg_cap = 0;
  Status composite(const float* bg, int bw, int bh);

  // Grid read-back overlapped with the next frames: the grid is snapshotted on the world's
  // stream (device copy into one of two staging buffers) and copied to the host on a copy
  // stream, so the world's next launches do not wait for the host copy.
  // The host copy is split over kCopyStreams streams (and so over the device's copy
  // engines), each carrying one contiguous part of the grid.
  static constexpr int kCopyStreams = 4;
  uint32_t* stage[2] = {nullptr, nullptr};
  cudaStream_t copy_streams[kCopyStreams] = {};
  cudaEvent_t stage_ready[2] = {nullptr, nullptr};
  cudaEvent_t stage_done[2][kCopyStreams] = {};
  int stage_i = 0;
  Status read_grid_overlapped(uint32_t* host);
  // The same with the ids packed into bytes on the device first (a quarter of the bytes
  // over the host link); their own staging buffers and events.
  uint8_t* stage8[2] = {nullptr, nullptr};
  cudaEvent_t stage8_ready[2] = {nullptr, nullptr};
  cudaEvent_t stage8_done[2][kCopyStreams] = {};
  int stage8_i = 0;
  Status read_grid_u8_overlapped(uint8_t* host);
  Status ensure_copy_streams();
  Status synchronize_all();  // the world's stream and the copy stream
};

// One launch of a single-world tile kernel (se_tile_*): k frames with counters f0.. over
// the world rows [ya, yb) of a W x H world held by src / dst (the whole world: 0, H).  The
// one place that builds this kernel's argument list.
// With `edits` (nedits live mods), the edit pass of the first frame runs inside the launch
// (se_tile_edit_*).
Status launch_tile_kernel(const Ruleset& rs, const TileVariant& v, const uint32_t* src, uint32_t* dst, int W, int H,
                          int f0, int k, int ya, int yb, cudaStream_t stream, const EditParams* edits = nullptr,
                          int nedits = 0);

// The edit pass inputs for `nlive` mods over world rows [row0, row0 + rows) of a W-wide
// world: records with their materials mapped through getMaterialFromID and the bounding
// boxes of the cells each can hit (empty boxes have x1 < x0).  Returns the box cells.
long long fill_edit_params(const Ruleset& rs, int W, int row0, int rows, const se_modification* mods, int nlive,
                           EditParams* p);

// The edit pass (se_edit) for `nlive` mods over world rows [row0, row0 + rows) of a W-wide
// world, held by `grid`.
Status launch_edit_on(const Ruleset& rs, uint32_t* grid, int W, int row0, int rows, const se_modification* mods,
                      int nlive, cudaStream_t stream);

cudaError_t grid_digest(const uint32_t* g, unsigned long long n, unsigned long long* d_out, cudaStream_t s);
cudaError_t grid_histogram(const uint32_t* g, unsigned long long n, int nbins, unsigned long long* d_counts,
                           cudaStream_t s);
// Each cell's material id as one byte (unknown ids NULL), nmat <= 256, on stream s.
cudaError_t pack_ids_u8(const uint32_t* g, uint8_t* out, unsigned long long n, uint32_t nmat, cudaStream_t s);
int noalloc_max_bins();
cudaError_t histogram_noalloc(const uint32_t* g, unsigned long long n, int nbins, unsigned long long* host_counts,
                              cudaStream_t s);

}  // namespace se::rt
