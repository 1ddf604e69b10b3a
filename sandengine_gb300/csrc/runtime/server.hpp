// Serving: simulation sessions resident in HBM, "advance N frames + apply edits" requests
// batched continuously.
#pragma once

#include <cuda_runtime.h>

#include <deque>
#include <map>
#include <memory>
#include <vector>

#include "../../../include/sandengine.h"
#include "batch.hpp"
#include "engine.hpp"

namespace se::rt {

struct Server {
  struct Session {
    int W = 0, H = 0;
    int32_t frame = 0;
    int cur = 0;
    bool open = true;
    bool resident = false;
    bool was_evicted = false;
    size_t off = 0, bytes = 0;           // arena block (2 buffers) while resident
    std::vector<uint32_t> host;          // current grid while evicted
    long long last_use = 0;              // iteration that last touched it (LRU)
    int active = -1;                     // request being served
    std::deque<int> queue;               // admitted requests waiting for this session
    uint32_t* buf(int i) const;
    Server* srv = nullptr;
  };
  struct Request {
    int session = 0;
    int nframes = 0, remaining = 0;
    std::vector<se_modification> mods;
    double arrival_ms = 0;
    bool started = false;
    bool cancelled = false;  // withdrawn before it started (se_server_cancel)
    long long iter = -1;  // iteration that completed it
    double done_ms = -1;
  };

  std::shared_ptr<Ruleset> rs;
  size_t budget = 0;
  char* arena = nullptr;
  std::map<size_t, size_t> free_blocks;  // offset -> size
  size_t used = 0, peak_used = 0;
  std::vector<Session> sessions;
  std::vector<Request> requests;
  size_t first_pending = 0;   // requests before this index have been served
  size_t last_run_begin = 0;  // first request of the last run
  const TileVariant* variant = nullptr;
  cudaStream_t stream = nullptr;
  // pinned staging for per-iteration descriptors, in a ring guarded by events
  static constexpr int kRing = 4;
  struct Stage {
    WorldDesc* desc = nullptr;
    int* prefix = nullptr;
    size_t cap = 0;
    cudaEvent_t ev = nullptr;
    WorldDesc* d_desc = nullptr;
    int* d_prefix = nullptr;
  } ring[kRing];
  std::vector<cudaEvent_t> iter_events;
  long long iterations = 0, evictions = 0, restores = 0;
  double cell_updates = 0;
  double wall_ms = 0;

  ~Server();
  Status create(std::shared_ptr<Ruleset> r, long long budget_bytes);
  Status set_frames_per_iteration(int k);
  Status open_session(int w, int h, const uint32_t* cells, int32_t frame, int* id);
  Status close_session(int id);
  Status submit(int session, int nframes, const se_modification* mods, int nmods, double arrival_ms, int* id);
  // Withdraws a request that has not been run yet: the next run skips it and its session's
  // frame counter does not move for it.
  Status cancel(int request);
  Status run(bool plain);
  Status get_grid(int session, uint32_t* host, size_t count);
  Status stats(se_server_stats* out);

 private:
  bool alloc(size_t bytes, size_t* off);
  void release(size_t off, size_t bytes);
  Status make_resident(int s, bool* ok);
  Status evict(int s);
  Status run_batched();
  Status run_plain();
  Status stage_reserve(Stage& st, size_t n);
};

}  // namespace se::rt
