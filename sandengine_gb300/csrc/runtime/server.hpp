// Serving: simulation sessions resident in HBM, "advance N frames + apply edits" requests
// batched continuously.
#pragma once

#include <cuda_runtime.h>

#include <chrono>
#include <condition_variable>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <thread>
#include <vector>

#include "../../../include/sandengine.h"
#include "batch.hpp"
#include "engine.hpp"

namespace se::rt {

// Two ways to serve:
//  * replay (run): every request queued before the call, each with an arrival time; the call
//    serves them in real time and returns when all are done;
//  * live (start ... stop): a loop on its own host thread serves requests as they are
//    submitted, from any thread, until stop.  A request's arrival is the moment it is
//    submitted; wait / poll report its completion.
// Both run the same scheduler (serve_batched / serve_plain).  Every member the loop and the
// API calls share is guarded by `mu`; the loop never holds a reference into `sessions` or
// `requests` across a point where it releases the lock (other threads may append to them).
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
    bool done = false;       // its last frame has completed on the GPU
    double done_ms = -1;     // completion time on the GPU, from the run's time origin
  };
  using Clock = std::chrono::steady_clock;

  std::shared_ptr<Ruleset> rs;
  size_t budget = 0;
  char* arena = nullptr;
  std::map<size_t, size_t> free_blocks;  // offset -> size
  size_t used = 0, peak_used = 0;
  std::vector<Session> sessions;
  std::vector<Request> requests;
  size_t first_pending = 0;   // replay: requests before this index have been served
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
  // The run's time origin (an event and the host clock read when it completed), and the
  // iterations in flight: each records an event, with the requests it completes.
  cudaEvent_t t0 = nullptr;
  Clock::time_point host_t0;
  struct Inflight {
    cudaEvent_t ev;
    std::vector<int> completes;
    cudaEvent_t start = nullptr;  // recorded before the iteration's first launch, if any
  };
  std::deque<Inflight> inflight;
  std::vector<cudaEvent_t> event_pool;
  long long iterations = 0, evictions = 0, restores = 0;
  double cell_updates = 0;
  double wall_ms = 0;
  double restore_ms_total = 0;  // host time spent restoring evicted sessions
  double kernel_ms = 0;         // GPU time of the last run's iterations (first launch to end)

  // live loop
  std::mutex mu;
  std::condition_variable cv_work;  // the loop waits here for submissions
  std::condition_variable cv_done;  // wait() waits here for completions
  std::thread loop;
  bool live = false, stopping = false;
  bool loop_running = false;
  int device = 0;  // the device the server was created on (its loop thread selects it)
  Status loop_status;    // the loop's first failure (then it stops serving)
  std::deque<int> inbox;  // live: submitted requests not yet admitted, in arrival order

  ~Server();
  Status create(std::shared_ptr<Ruleset> r, long long budget_bytes);
  Status set_frames_per_iteration(int k);
  Status open_session(int w, int h, const uint32_t* cells, int32_t frame, int* id);
  Status close_session(int id);
  Status submit(int session, int nframes, const se_modification* mods, int nmods, double arrival_ms, int* id);
  // Withdraws a request that has not started: it is skipped and its session's frame counter
  // does not move for it.
  Status cancel(int request);
  Status run(bool plain);  // replay
  Status start(bool plain);  // live
  Status stop();            // live: serves what was submitted, then ends the loop
  // Waits up to timeout_ms (< 0: no limit) for a request; *done tells whether it completed.
  Status wait(int request, double timeout_ms, bool* done, double* latency_ms);
  Status request_latency(int request, double* latency_ms);
  Status get_grid(int session, uint32_t* host, size_t count);
  Status session_state(int session, int* w, int* h, int32_t* frame, std::vector<uint32_t>* cells);
  Status stats(se_server_stats* out);

 private:
  bool alloc(size_t bytes, size_t* off);
  void release(size_t off, size_t bytes);
  Status make_resident(int s, bool* ok);
  Status evict(int s);
  Status begin_run();
  Status serve_batched(std::unique_lock<std::mutex>& lk);
  Status serve_plain(std::unique_lock<std::mutex>& lk);
  Status stage_reserve(Stage& st, size_t n);
  cudaEvent_t take_event();
  // Records the end of an iteration (whose first launch followed `start`, when not null).
  Status record_iteration(std::vector<int> completes, cudaEvent_t start = nullptr);
  // Retires finished iterations (all of them when `all`, waiting for the GPU with the lock
  // released), stamping their requests' completion times.
  Status retire(std::unique_lock<std::mutex>& lk, bool all);
  Status throttle(std::unique_lock<std::mutex>& lk, size_t max_inflight);
  Status get_grid_locked(int session, uint32_t* host, size_t count);
};

}  // namespace se::rt
