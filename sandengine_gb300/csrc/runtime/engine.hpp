// Rule sets and worlds behind the C ABI.
#pragma once

#include <cuda_runtime.h>

#include <memory>
#include <mutex>
#include <string>
#include <vector>

#include "../lang/codegen.hpp"
#include "../lang/lang.hpp"
#include "jit.hpp"

struct se_modification;

namespace se::rt {

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
  int W = 0, H = 0;
  int32_t frame = 0;
  uint32_t* buf[2] = {nullptr, nullptr};
  int cur = 0;
  unsigned long long* d_scratch = nullptr;  // 258 words for digests and histograms
  cudaStream_t own_stream = nullptr, stream = nullptr;
  int steps_per_launch = 0;  // 0: default
  ~World();
  Status create(std::shared_ptr<Ruleset> r, int w, int h);
  Status step(int nframes, const se_modification* mods, int nmods);
  // k frames with counters f0.. from buf[cur] into buf[cur^1]
  Status launch_tiles(int f0, int k);
  Status launch_edit(const se_modification* mods, int nlive);
  int default_k() const;
  Status digest(unsigned long long* out);
  Status histogram(unsigned long long* counts, int nbins);
};

cudaError_t grid_digest(const uint32_t* g, unsigned long long n, unsigned long long* d_out, cudaStream_t s);
cudaError_t grid_histogram(const uint32_t* g, unsigned long long n, int nbins, unsigned long long* d_counts,
                           cudaStream_t s);

}  // namespace se::rt
