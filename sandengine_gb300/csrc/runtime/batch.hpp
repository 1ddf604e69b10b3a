// Many independent worlds advanced together.
#pragma once

#include <cuda_runtime.h>

#include <map>
#include <memory>
#include <vector>

#include "engine.hpp"

namespace se::rt {

// Device layout of one world (SeWorldDesc in kernels/margolus.cuh).
struct WorldDesc {
  uint32_t* buf0;
  uint32_t* buf1;
  int W, H;
  int frame;
  int cur;
  int pad0, pad1;
};
static_assert(sizeof(WorldDesc) == 40, "must match SeWorldDesc");
struct TileJob {  // SeTileJob
  int world, x0, y0, pad;
};

struct Batch {
  std::shared_ptr<Ruleset> rs;
  int n = 0;
  std::vector<WorldDesc> desc;  // host mirror (kept equal to the device copy)
  WorldDesc* d_desc = nullptr;
  uint32_t* arena = nullptr;
  long long cells = 0;
  // worlds held wholly in shared memory, in size classes launched side by side
  struct Resident {
    std::vector<int> ids;
    int* d_ids = nullptr;
    size_t smem = 0;
    int threads = 256;
  };
  std::vector<Resident> resident;
  std::vector<int> tiled;  // worlds advanced by tile passes
  const TileVariant* variant = nullptr;
  int steps_per_launch = 0;  // 0: autotune on first use
  std::vector<TileJob> jobs;
  TileJob* d_jobs = nullptr;
  size_t d_jobs_cap = 0;
  cudaStream_t stream = nullptr, side[4] = {nullptr, nullptr, nullptr, nullptr};
  cudaEvent_t fork = nullptr, join[4] = {nullptr, nullptr, nullptr, nullptr};
  std::map<int, cudaGraphExec_t> graphs;  // by frames per launch

  ~Batch();
  Status create(std::shared_ptr<Ruleset> r, int count, const int* widths, const int* heights);
  Status set_grid(int i, const uint32_t* host, size_t count);
  Status get_grid(int i, uint32_t* host, size_t count);
  Status set_frame(int i, int32_t f);
  Status step(int nframes);
  Status step_plain(int nframes);
  Status autotune(int reps, int* best_k);
  Status set_variant(const TileVariant* v);
  Status invalidate_graphs();
  // Worlds whose whole-world CTA needs at most `bytes` of shared memory stay resident; the
  // others take tile passes (0: none resident).  Rebuilds the classes and the job list.
  Status set_resident_limit(size_t bytes);
  size_t resident_limit = 0;

 private:
  Status classify();
  Status launch_body(int nframes, cudaStream_t s);
  Status upload_desc();
};

}  // namespace se::rt
