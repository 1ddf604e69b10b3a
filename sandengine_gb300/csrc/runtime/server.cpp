#include "server.hpp"
#include "trace.hpp"

#include <algorithm>
#include <chrono>
#include <climits>
#include <cstring>
#include <mutex>
#include <thread>

namespace se::rt {

namespace {
Status cuda_fail(const char* what, cudaError_t e) {
  return {SE_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e)};
}
#define SE_CUDA(call)                                   \
  do {                                                  \
    cudaError_t _e = (call);                            \
    if (_e != cudaSuccess) return cuda_fail(#call, _e); \
  } while (0)

using Clock = std::chrono::steady_clock;
double ms_since(Clock::time_point t0) {
  return std::chrono::duration<double, std::milli>(Clock::now() - t0).count();
}
size_t session_bytes(int W, int H) { return 2 * (((size_t)W * H * 4 + 255) & ~(size_t)255); }
}  // namespace

uint32_t* Server::Session::buf(int i) const {
  return reinterpret_cast<uint32_t*>(srv->arena + off + (i ? bytes / 2 : 0));
}

Server::~Server() {
  if (loop.joinable()) stop();
  if (stream) cudaStreamSynchronize(stream);
  for (auto& f : inflight) cudaEventDestroy(f.ev);
  for (auto& e : event_pool) cudaEventDestroy(e);
  if (t0) cudaEventDestroy(t0);
  for (auto& st : ring) {
    if (st.desc) cudaFreeHost(st.desc);
    if (st.prefix) cudaFreeHost(st.prefix);
    if (st.d_desc) cudaFree(st.d_desc);
    if (st.d_prefix) cudaFree(st.d_prefix);
    if (st.ev) cudaEventDestroy(st.ev);
  }
  if (arena) cudaFree(arena);
  if (stream) cudaStreamDestroy(stream);
}

Status Server::create(std::shared_ptr<Ruleset> r, long long budget_bytes) {
  if (budget_bytes < 4096) return {SE_ERR_INVALID_ARGUMENT, "budget must be at least 4 KiB"};
  rs = std::move(r);
  Status s = rs->ensure_loaded();
  if (!s.ok()) return s;
  budget = ((size_t)budget_bytes) & ~(size_t)255;
  {
    cudaError_t e = cudaMalloc(&arena, budget);
    if (e != cudaSuccess) return {SE_ERR_OUT_OF_MEMORY, std::string("cudaMalloc(budget): ") + cudaGetErrorString(e)};
  }
  free_blocks[0] = budget;
  SE_CUDA(cudaGetDevice(&device));
  SE_CUDA(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
  SE_CUDA(cudaEventCreate(&t0));
  for (auto& st : ring) SE_CUDA(cudaEventCreateWithFlags(&st.ev, cudaEventDisableTiming));
  return set_frames_per_iteration(8);
}

Status Server::set_frames_per_iteration(int k) {
  std::lock_guard<std::mutex> g(mu);
  if (live) return {SE_ERR_INVALID_ARGUMENT, "the frames per iteration cannot change while the server runs"};
  // The first compiled variant with the fewest frames >= k: for k = 8 the 128x64 tiles,
  // which serve sessions of 128-2048 cells a side best (the serving benchmark's highest
  // throughput, 770 G cell-updates/s, against 690-734 G with 256x128, 128x128 or 256x64
  // tiles): their smaller halo loss on the large tiles does not make up for the waste on
  // the small sessions and the coarser work units of an iteration.
  const TileVariant* v = nullptr;
  for (const TileVariant& t : tile_variants())
    if (t.kmax >= k && (!v || t.kmax < v->kmax)) v = &t;
  if (!v || k < 1) return {SE_ERR_INVALID_ARGUMENT, "no kernel variant for this many frames per iteration"};
  variant = v;
  return Status::Ok();
}

bool Server::alloc(size_t bytes, size_t* off) {
  for (auto it = free_blocks.begin(); it != free_blocks.end(); ++it) {
    if (it->second < bytes) continue;
    *off = it->first;
    const size_t rest = it->second - bytes;
    const size_t roff = it->first + bytes;
    free_blocks.erase(it);
    if (rest) free_blocks[roff] = rest;
    used += bytes;
    peak_used = std::max(peak_used, used);
    return true;
  }
  return false;
}

void Server::release(size_t off, size_t bytes) {
  used -= bytes;
  auto it = free_blocks.emplace(off, bytes).first;
  auto nx = std::next(it);
  if (nx != free_blocks.end() && it->first + it->second == nx->first) {
    it->second += nx->second;
    free_blocks.erase(nx);
  }
  if (it != free_blocks.begin()) {
    auto pv = std::prev(it);
    if (pv->first + pv->second == it->first) {
      pv->second += it->second;
      free_blocks.erase(it);
    }
  }
}

Status Server::open_session(int w, int h, const uint32_t* cells, int32_t frame, int* id) {
  std::lock_guard<std::mutex> g(mu);
  if (w <= 0 || h <= 0) return {SE_ERR_INVALID_ARGUMENT, "session size must be positive"};
  if (w > kMaxSide || h > kMaxSide) return {SE_ERR_INVALID_ARGUMENT, "world sides are limited to 1048576 cells"};
  if (frame < 0) return {SE_ERR_INVALID_ARGUMENT, "frame must be >= 0"};
  if (session_bytes(w, h) > budget) return {SE_ERR_BUDGET, "the session alone exceeds the HBM budget"};
  Session s;
  s.srv = this;
  s.W = w;
  s.H = h;
  s.frame = frame;
  if (cells) s.host.assign(cells, cells + (size_t)w * h);
  sessions.push_back(std::move(s));
  *id = (int)sessions.size() - 1;
  return Status::Ok();
}

Status Server::cancel(int request) {
  std::lock_guard<std::mutex> g(mu);
  if (request < 0 || request >= (int)requests.size()) return {SE_ERR_INVALID_ARGUMENT, "bad request"};
  Request& r = requests[(size_t)request];
  if (r.started || r.done) return {SE_ERR_INVALID_ARGUMENT, "only a request that has not started can be cancelled"};
  r.cancelled = true;
  cv_done.notify_all();
  return Status::Ok();
}

Status Server::close_session(int id) {
  std::lock_guard<std::mutex> g(mu);
  if (id < 0 || id >= (int)sessions.size() || !sessions[(size_t)id].open)
    return {SE_ERR_INVALID_ARGUMENT, "bad session"};
  Session& s = sessions[(size_t)id];
  if (s.active >= 0 || !s.queue.empty()) return {SE_ERR_INVALID_ARGUMENT, "session has requests in flight"};
  for (size_t r = 0; r < requests.size(); ++r)
    if (requests[r].session == id && !requests[r].cancelled && !requests[r].done)
      return {SE_ERR_INVALID_ARGUMENT, "session has queued requests"};
  if (s.resident) {
    SE_CUDA(cudaStreamSynchronize(stream));
    release(s.off, s.bytes);
  }
  s.resident = false;
  s.open = false;
  s.host.clear();
  s.host.shrink_to_fit();
  return Status::Ok();
}

Status Server::submit(int session, int nframes, const se_modification* mods, int nmods, double arrival_ms, int* id) {
  std::lock_guard<std::mutex> g(mu);
  if (live && stopping) return {SE_ERR_INVALID_ARGUMENT, "the server is stopping"};
  if (session < 0 || session >= (int)sessions.size() || !sessions[(size_t)session].open)
    return {SE_ERR_INVALID_ARGUMENT, "bad session"};
  if (nframes < 1) return {SE_ERR_INVALID_ARGUMENT, "nframes must be >= 1"};
  if (nmods < 0 || (nmods > 0 && !mods)) return {SE_ERR_INVALID_ARGUMENT, "bad modification list"};
  Request r;
  r.session = session;
  r.nframes = r.remaining = nframes;
  r.arrival_ms = arrival_ms;
  const int nseen = std::min(nmods, SE_MAX_MODIFICATIONS);  // simulation.rs:205
  for (int i = 0; i < nseen && mods[i].mod_size != 0; ++i) r.mods.push_back(mods[i]);
  if (live) r.arrival_ms = ms_since(host_t0);  // a live request arrives when it is submitted
  requests.push_back(std::move(r));
  *id = (int)requests.size() - 1;
  if (live) {
    inbox.push_back(*id);
    cv_work.notify_one();
  }
  return Status::Ok();
}

Status Server::evict(int id) {
  Session& s = sessions[(size_t)id];
  s.host.resize((size_t)s.W * s.H);
  SE_CUDA(cudaMemcpyAsync(s.host.data(), s.buf(s.cur), s.host.size() * 4, cudaMemcpyDeviceToHost, stream));
  SE_CUDA(cudaStreamSynchronize(stream));
  release(s.off, s.bytes);
  s.resident = false;
  s.was_evicted = true;
  ++evictions;
  return Status::Ok();
}

Status Server::make_resident(int id, bool* ok) {
  Session& s = sessions[(size_t)id];
  *ok = true;
  if (s.resident) return Status::Ok();
  const size_t bytes = session_bytes(s.W, s.H);
  size_t off = 0;
  while (!alloc(bytes, &off)) {
    int victim = -1;  // least recently used idle session
    for (size_t i = 0; i < sessions.size(); ++i) {
      const Session& c = sessions[i];
      if ((int)i == id || !c.resident || c.active >= 0) continue;
      if (victim < 0 || c.last_use < sessions[(size_t)victim].last_use) victim = (int)i;
    }
    if (victim < 0) {
      *ok = false;
      return Status::Ok();
    }
    Status st = evict(victim);
    if (!st.ok()) return st;
  }
  s.off = off;
  s.bytes = bytes;
  s.resident = true;
  if (s.host.empty()) {
    SE_CUDA(cudaMemsetAsync(s.buf(s.cur), 0, (size_t)s.W * s.H * 4, stream));
  } else {
    const Clock::time_point tr = Clock::now();
    SE_CUDA(cudaMemcpyAsync(s.buf(s.cur), s.host.data(), s.host.size() * 4, cudaMemcpyHostToDevice, stream));
    SE_CUDA(cudaStreamSynchronize(stream));  // the host copy may be released now
    if (s.was_evicted) {
      ++restores;
      restore_ms_total += ms_since(tr);
    }
    s.host.clear();
    s.host.shrink_to_fit();
  }
  return Status::Ok();
}

Status Server::stage_reserve(Stage& st, size_t n) {
  if (st.cap >= n + 1) return Status::Ok();
  size_t cap = std::max<size_t>(64, 2 * (n + 1));
  if (st.desc) cudaFreeHost(st.desc);
  if (st.prefix) cudaFreeHost(st.prefix);
  if (st.d_desc) cudaFree(st.d_desc);
  if (st.d_prefix) cudaFree(st.d_prefix);
  SE_CUDA(cudaMallocHost(&st.desc, cap * sizeof(WorldDesc)));
  SE_CUDA(cudaMallocHost(&st.prefix, cap * sizeof(int)));
  SE_CUDA(cudaMalloc(&st.d_desc, cap * sizeof(WorldDesc)));
  SE_CUDA(cudaMalloc(&st.d_prefix, cap * sizeof(int)));
  st.cap = cap;
  return Status::Ok();
}

// The time origin of a run: an event on the stream, and the host clock once it completed.
Status Server::begin_run() {
  iterations = 0;
  cell_updates = 0;
  wall_ms = 0;
  kernel_ms = 0;
  SE_CUDA(cudaEventRecord(t0, stream));
  SE_CUDA(cudaEventSynchronize(t0));
  host_t0 = Clock::now();
  return Status::Ok();
}

cudaEvent_t Server::take_event() {
  cudaEvent_t ev = nullptr;
  if (!event_pool.empty()) {
    ev = event_pool.back();
    event_pool.pop_back();
  } else if (cudaEventCreate(&ev) != cudaSuccess) {
    ev = nullptr;
  }
  return ev;
}

Status Server::record_iteration(std::vector<int> completes, cudaEvent_t start) {
  cudaEvent_t ev = take_event();
  if (!ev) return cuda_fail("cudaEventCreate", cudaGetLastError());
  SE_CUDA(cudaEventRecord(ev, stream));
  inflight.push_back({ev, std::move(completes), start});
  return Status::Ok();
}

Status Server::retire(std::unique_lock<std::mutex>& lk, bool all) {
  bool any = false;
  while (!inflight.empty()) {  // only the serving thread changes `inflight`
    cudaEvent_t ev = inflight.front().ev;
    cudaError_t q = cudaEventQuery(ev);
    if (q == cudaErrorNotReady) {
      if (!all) break;
      lk.unlock();
      q = cudaEventSynchronize(ev);
      lk.lock();
    }
    if (q != cudaSuccess) return cuda_fail("cudaEventSynchronize", q);
    float ms = 0;
    SE_CUDA(cudaEventElapsedTime(&ms, t0, ev));
    for (int r : inflight.front().completes) {
      requests[(size_t)r].done = true;
      requests[(size_t)r].done_ms = ms;
    }
    wall_ms = std::max(wall_ms, (double)ms);
    if (cudaEvent_t st = inflight.front().start) {
      float k = 0;
      SE_CUDA(cudaEventElapsedTime(&k, st, ev));
      kernel_ms += k;
      event_pool.push_back(st);
    }
    event_pool.push_back(ev);
    inflight.pop_front();
    any = true;
  }
  if (any) cv_done.notify_all();
  return Status::Ok();
}

// At most `max_inflight` iterations queued on the GPU: the host plans ahead, but not far.
Status Server::throttle(std::unique_lock<std::mutex>& lk, size_t max_inflight) {
  while (inflight.size() > max_inflight) {
    cudaEvent_t ev = inflight.front().ev;
    lk.unlock();
    cudaError_t e = cudaEventSynchronize(ev);
    lk.lock();
    if (e != cudaSuccess) return cuda_fail("cudaEventSynchronize", e);
    Status s = retire(lk, false);
    if (!s.ok()) return s;
  }
  return Status::Ok();
}

Status Server::run(bool plain) {
  std::unique_lock<std::mutex> lk(mu);
  if (live) return {SE_ERR_INVALID_ARGUMENT, "the server's live loop is running (se_server_stop first)"};
  last_run_begin = first_pending;
  Status s = begin_run();
  if (!s.ok()) return s;
  s = plain ? serve_plain(lk) : serve_batched(lk);
  if (!s.ok()) return s;
  s = retire(lk, true);
  if (!s.ok()) return s;
  first_pending = requests.size();
  return Status::Ok();
}

Status Server::start(bool plain) {
  std::unique_lock<std::mutex> lk(mu);
  if (live || loop.joinable()) return {SE_ERR_INVALID_ARGUMENT, "the server is already running"};
  for (size_t i = first_pending; i < requests.size(); ++i)
    if (!requests[i].cancelled && !requests[i].done)
      return {SE_ERR_INVALID_ARGUMENT, "requests queued for se_server_run are still pending"};
  first_pending = requests.size();
  last_run_begin = requests.size();
  Status s = begin_run();
  if (!s.ok()) return s;
  live = true;
  stopping = false;
  loop_running = true;
  loop_status = Status::Ok();
  loop = std::thread([this, plain] {
    cudaSetDevice(device);  // the runtime's current device is per host thread
    std::unique_lock<std::mutex> l(mu);
    Status st = plain ? serve_plain(l) : serve_batched(l);
    if (st.ok()) st = retire(l, true);
    loop_status = st;
    loop_running = false;
    cv_done.notify_all();
  });
  return Status::Ok();
}

Status Server::stop() {
  {
    std::lock_guard<std::mutex> g(mu);
    if (!live) return {SE_ERR_INVALID_ARGUMENT, "the server is not running"};
    stopping = true;
  }
  cv_work.notify_all();
  loop.join();
  std::lock_guard<std::mutex> g(mu);
  live = false;
  stopping = false;
  first_pending = requests.size();
  return loop_status;
}

Status Server::wait(int request, double timeout_ms, bool* done, double* latency_ms) {
  std::unique_lock<std::mutex> lk(mu);
  if (request < 0 || request >= (int)requests.size()) return {SE_ERR_INVALID_ARGUMENT, "bad request"};
  auto settled = [&] {
    const Request& r = requests[(size_t)request];
    return r.done || r.cancelled || !loop_running;
  };
  if (timeout_ms < 0)
    cv_done.wait(lk, settled);
  else
    cv_done.wait_for(lk, std::chrono::duration<double, std::milli>(timeout_ms), settled);
  const Request& r = requests[(size_t)request];
  *done = r.done;
  if (r.cancelled) return {SE_ERR_CANCELLED, "the request was cancelled"};
  if (r.done) {
    if (latency_ms) *latency_ms = r.done_ms - r.arrival_ms;
    return Status::Ok();
  }
  if (!loop_running && live) {
    if (!loop_status.ok()) return loop_status;
    return {SE_ERR_INVALID_ARGUMENT, "the serving loop ended before the request completed"};
  }
  if (!live) return {SE_ERR_INVALID_ARGUMENT, "the request has not been served (se_server_run or se_server_start)"};
  return {SE_ERR_TIMEOUT, "the request has not completed yet"};
}

Status Server::request_latency(int request, double* latency_ms) {
  std::lock_guard<std::mutex> g(mu);
  if (request < 0 || request >= (int)requests.size()) return {SE_ERR_INVALID_ARGUMENT, "bad request"};
  const Request& r = requests[(size_t)request];
  if (r.cancelled) return {SE_ERR_INVALID_ARGUMENT, "request was cancelled"};
  if (!r.done) return {SE_ERR_INVALID_ARGUMENT, "request has not been served"};
  *latency_ms = r.done_ms - r.arrival_ms;
  return Status::Ok();
}

// Continuous batching.  Each iteration advances every active session by up to K frames in
// one launch (1 frame when its request starts with edits, followed by the edit pass), so
// sessions join and leave between iterations.  Progress is known on the host, so the host
// plans iterations ahead of the GPU (at most two in flight) and timestamps completions with
// events.  Replay: the queued requests are admitted as their arrival times pass.  Live:
// submitted requests are admitted at the next iteration; with nothing to do the loop
// retires what is in flight and sleeps until a submission or stop.
Status Server::serve_batched(std::unique_lock<std::mutex>& lk) {
  TraceRange trace("se_server_serve_batched");
  std::vector<int> pend;  // replay only
  if (!live) {
    for (size_t i = first_pending; i < requests.size(); ++i)
      if (!requests[i].cancelled) pend.push_back((int)i);
    std::stable_sort(pend.begin(), pend.end(),
                     [&](int a, int b) { return requests[(size_t)a].arrival_ms < requests[(size_t)b].arrival_ms; });
  }
  const int K = variant->kmax;
  const size_t smem = tile_smem_bytes(*variant, rs->lut_shape());
  cudaKernel_t kern = rs->module->get(variant->serve_name());
  const uint16_t* lut = rs->d_lut;
  size_t next = 0;
  std::deque<int> waiting;  // sessions with queued requests, in order of their turn
  std::vector<int> active;
  long long it = 0;
  auto admit = [&](int rid) {
    if (requests[(size_t)rid].cancelled) return;
    const int sid = requests[(size_t)rid].session;
    Session& ss = sessions[(size_t)sid];
    const bool idle = ss.active < 0 && ss.queue.empty();
    ss.queue.push_back(rid);
    if (idle) waiting.push_back(sid);
  };
  auto finish = [&](int sid, std::vector<int>& completes) {  // sid's request completes in this iteration
    Session& ss = sessions[(size_t)sid];
    completes.push_back(ss.active);
    ss.active = -1;
    if (!ss.queue.empty()) waiting.push_back(sid);
  };
  for (;;) {
    if (live) {
      while (!inbox.empty()) {
        admit(inbox.front());
        inbox.pop_front();
      }
    } else {
      const double now = ms_since(host_t0);
      while (next < pend.size() && requests[(size_t)pend[next]].arrival_ms <= now) admit(pend[next++]);
    }
    std::vector<int> instant;  // requests that finished before any frame of work (frame-1 clear only)
    while (!waiting.empty()) {
      const int sid = waiting.front();
      {
        Session& ss = sessions[(size_t)sid];
        while (!ss.queue.empty() && requests[(size_t)ss.queue.front()].cancelled) ss.queue.pop_front();
        if (ss.queue.empty()) {
          waiting.pop_front();
          continue;
        }
      }
      bool ok = true;
      Status st = make_resident(sid, &ok);
      if (!st.ok()) return st;
      if (!ok) break;  // no memory until running sessions finish
      waiting.pop_front();
      Session& ss = sessions[(size_t)sid];
      ss.active = ss.queue.front();
      ss.queue.pop_front();
      Request& r = requests[(size_t)ss.active];
      if (ss.frame == 0) {  // frame 1 clears the grid and ignores the mods (falling_sand.glsl:128-131)
        SE_CUDA(cudaMemsetAsync(ss.buf(ss.cur), 0, (size_t)ss.W * ss.H * 4, stream));
        ss.frame = 1;
        r.remaining -= 1;
        r.mods.clear();
        r.started = true;
        cell_updates += (double)ss.W * ss.H;
        if (r.remaining == 0) {
          instant.push_back(sid);
          continue;
        }
      }
      active.push_back(sid);
    }
    if (!instant.empty()) {
      std::vector<int> completes;
      for (int sid : instant) finish(sid, completes);
      Status st = record_iteration(std::move(completes));
      if (!st.ok()) return st;
    }
    if (active.empty()) {
      if (!waiting.empty()) {  // nothing runs, yet a waiting session does not fit
        bool any_active = false;
        for (auto& ss : sessions) any_active = any_active || ss.active >= 0;
        if (!any_active && (live || next >= pend.size()))
          return {SE_ERR_BUDGET, "a session does not fit the HBM budget"};
      }
      if (live) {
        if (stopping && inbox.empty() && waiting.empty()) break;
        Status st = retire(lk, true);  // everything admitted so far has completed
        if (!st.ok()) return st;
        cv_work.wait(lk, [&] { return stopping || !inbox.empty(); });
        continue;
      }
      if (next >= pend.size() && waiting.empty()) break;
      if (next < pend.size()) {
        const double wait = requests[(size_t)pend[next]].arrival_ms - ms_since(host_t0);
        if (wait > 0.05) {
          lk.unlock();
          std::this_thread::sleep_for(std::chrono::microseconds((long long)(wait * 1000 * 0.9)));
          lk.lock();
        }
      }
      continue;
    }
    // ---- one iteration over every active session
    Stage& stg = ring[it % kRing];
    if (it >= kRing) SE_CUDA(cudaEventSynchronize(stg.ev));  // at most two iterations are in flight
    Status st = stage_reserve(stg, active.size());
    if (!st.ok()) return st;
    int total = 0;
    std::vector<int> ks(active.size());
    for (size_t a = 0; a < active.size(); ++a) {
      Session& ss = sessions[(size_t)active[a]];
      const Request& r = requests[(size_t)ss.active];
      const int k = (!r.started && !r.mods.empty()) ? 1 : std::min(K, r.remaining);
      ks[a] = k;
      stg.desc[a] = WorldDesc{ss.buf(0), ss.buf(1), ss.W, ss.H, ss.frame, ss.cur, k, 0};
      stg.prefix[a] = total;
      total += ((ss.W + variant->tw - 1) / variant->tw) * ((ss.H + variant->th - 1) / variant->th);
    }
    stg.prefix[active.size()] = total;
    SE_CUDA(cudaMemcpyAsync(stg.d_desc, stg.desc, active.size() * sizeof(WorldDesc), cudaMemcpyHostToDevice, stream));
    SE_CUDA(cudaMemcpyAsync(stg.d_prefix, stg.prefix, (active.size() + 1) * sizeof(int), cudaMemcpyHostToDevice,
                            stream));
    cudaEvent_t started = take_event();
    if (!started) return cuda_fail("cudaEventCreate", cudaGetLastError());
    SE_CUDA(cudaEventRecord(started, stream));
    {
      const WorldDesc* dd = stg.d_desc;
      const int* pp = stg.d_prefix;
      int na = (int)active.size();
      void* args[] = {(void*)&dd, (void*)&pp, &na, (void*)&lut};
      SE_CUDA(cudaLaunchKernel((const void*)kern, dim3((unsigned)total), dim3((unsigned)variant->nt), args, smem,
                               stream));
    }
    SE_CUDA(cudaEventRecord(stg.ev, stream));
    ++it;
    ++iterations;
    std::vector<int> still;
    std::vector<int> done;
    for (size_t a = 0; a < active.size(); ++a) {
      const int sid = active[a];
      Session& ss = sessions[(size_t)sid];
      Request& r = requests[(size_t)ss.active];
      const int k = ks[a];
      ss.frame += k;
      ss.cur ^= 1;
      ss.last_use = it;
      r.remaining -= k;
      cell_updates += (double)ss.W * ss.H * k;
      if (!r.started && !r.mods.empty()) {
        st = launch_edit_on(*rs, ss.buf(ss.cur), ss.W, 0, ss.H, r.mods.data(), (int)r.mods.size(), stream);
        if (!st.ok()) return st;
      }
      r.started = true;
      if (r.remaining == 0) done.push_back(sid);
      else still.push_back(sid);
    }
    std::vector<int> completes;
    for (int sid : done) finish(sid, completes);
    st = record_iteration(std::move(completes), started);
    if (!st.ok()) return st;
    active.swap(still);
    st = throttle(lk, 2);
    if (!st.ok()) return st;
    st = retire(lk, false);
    if (!st.ok()) return st;
  }
  return Status::Ok();
}

// One request at a time in arrival order, one launch per frame (plus the edit pass after
// its first frame): the way the reference advances a world.
Status Server::serve_plain(std::unique_lock<std::mutex>& lk) {
  TraceRange trace("se_server_serve_plain");
  std::vector<int> pend;  // replay only
  if (!live) {
    for (size_t i = first_pending; i < requests.size(); ++i)
      if (!requests[i].cancelled) pend.push_back((int)i);
    std::stable_sort(pend.begin(), pend.end(),
                     [&](int a, int b) { return requests[(size_t)a].arrival_ms < requests[(size_t)b].arrival_ms; });
  }
  const TileVariant* v1 = nullptr;
  for (const TileVariant& t : tile_variants())
    if (t.kmax == 1) {
      v1 = &t;
      break;
    }
  size_t next = 0;
  for (;;) {
    int ri = -1;
    if (live) {
      if (inbox.empty()) {
        if (stopping) break;
        Status st = retire(lk, true);
        if (!st.ok()) return st;
        cv_work.wait(lk, [&] { return stopping || !inbox.empty(); });
        continue;
      }
      ri = inbox.front();
      inbox.pop_front();
    } else {
      if (next >= pend.size()) break;
      ri = pend[next++];
      const double wait = requests[(size_t)ri].arrival_ms - ms_since(host_t0);
      if (wait > 0.05) {
        lk.unlock();
        std::this_thread::sleep_for(std::chrono::microseconds((long long)(wait * 1000)));
        lk.lock();
      }
    }
    if (requests[(size_t)ri].cancelled) continue;
    const int sid = requests[(size_t)ri].session;
    bool ok = true;
    Status st = make_resident(sid, &ok);
    if (!st.ok()) return st;
    if (!ok) return {SE_ERR_BUDGET, "a session does not fit the HBM budget"};
    Session& ss = sessions[(size_t)sid];
    Request& r = requests[(size_t)ri];
    r.started = true;
    cudaEvent_t started = take_event();
    if (!started) return cuda_fail("cudaEventCreate", cudaGetLastError());
    SE_CUDA(cudaEventRecord(started, stream));
    for (int i = 0; i < r.remaining; ++i) {
      const int f = ss.frame + 1;
      if (f == 1) {
        SE_CUDA(cudaMemsetAsync(ss.buf(ss.cur), 0, (size_t)ss.W * ss.H * 4, stream));
      } else {
        st = launch_tile_kernel(*rs, *v1, ss.buf(ss.cur), ss.buf(ss.cur ^ 1), ss.W, ss.H, f, 1, 0, ss.H, stream);
        if (!st.ok()) return st;
        ss.cur ^= 1;
        if (i == 0 && !r.mods.empty()) {
          st = launch_edit_on(*rs, ss.buf(ss.cur), ss.W, 0, ss.H, r.mods.data(), (int)r.mods.size(), stream);
          if (!st.ok()) return st;
        }
      }
      ss.frame = f;
    }
    cell_updates += (double)ss.W * ss.H * r.remaining;
    r.remaining = 0;
    ++iterations;
    ss.last_use = iterations;
    st = record_iteration({ri}, started);
    if (!st.ok()) return st;
    st = throttle(lk, 2);
    if (!st.ok()) return st;
    st = retire(lk, false);
    if (!st.ok()) return st;
  }
  return Status::Ok();
}

Status Server::get_grid(int id, uint32_t* host, size_t count) {
  std::lock_guard<std::mutex> g(mu);
  return get_grid_locked(id, host, count);
}

Status Server::session_state(int id, int* w, int* h, int32_t* frame, std::vector<uint32_t>* cells) {
  std::lock_guard<std::mutex> g(mu);
  if (id < 0 || id >= (int)sessions.size()) return {SE_ERR_INVALID_ARGUMENT, "bad session"};
  const Session& s = sessions[(size_t)id];
  if (w) *w = s.W;
  if (h) *h = s.H;
  if (frame) *frame = s.frame;
  if (!cells) return Status::Ok();
  cells->resize((size_t)s.W * s.H);
  return get_grid_locked(id, cells->data(), cells->size());
}

Status Server::get_grid_locked(int id, uint32_t* host, size_t count) {
  if (id < 0 || id >= (int)sessions.size()) return {SE_ERR_INVALID_ARGUMENT, "bad session"};
  const Session& s = sessions[(size_t)id];
  if (count != (size_t)s.W * s.H) return {SE_ERR_INVALID_ARGUMENT, "count must be width*height"};
  if (s.resident) {
    SE_CUDA(cudaMemcpyAsync(host, s.buf(s.cur), count * 4, cudaMemcpyDeviceToHost, stream));
    SE_CUDA(cudaStreamSynchronize(stream));
  } else if (s.host.empty()) {
    memset(host, 0, count * 4);
  } else {
    memcpy(host, s.host.data(), count * 4);
  }
  return Status::Ok();
}

Status Server::stats(se_server_stats* out) {
  std::lock_guard<std::mutex> g(mu);
  std::vector<double> lat;
  const size_t end = live ? requests.size() : std::min(first_pending, requests.size());
  for (size_t i = last_run_begin; i < end; ++i)
    if (requests[i].done) lat.push_back(requests[i].done_ms - requests[i].arrival_ms);
  memset(out, 0, sizeof *out);
  out->requests = (long long)lat.size();
  if (!lat.empty()) {
    std::sort(lat.begin(), lat.end());
    auto pct = [&](double q) { return lat[std::min(lat.size() - 1, (size_t)(q / 100.0 * (lat.size() - 1) + 0.5))]; };
    out->p50_ms = pct(50);
    out->p99_ms = pct(99);
    double sum = 0;
    for (double x : lat) sum += x;
    out->mean_ms = sum / lat.size();
    out->max_ms = lat.back();
  }
  out->wall_ms = wall_ms;
  out->cell_updates = cell_updates;
  out->iterations = iterations;
  out->evictions = evictions;
  out->restores = restores;
  out->restore_ms = restores ? restore_ms_total / (double)restores : 0.0;
  out->peak_resident_bytes = (long long)peak_used;
  out->kernel_ms = kernel_ms;
  return Status::Ok();
}

}  // namespace se::rt
