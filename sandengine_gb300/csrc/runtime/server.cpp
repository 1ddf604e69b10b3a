#include "server.hpp"
#include "trace.hpp"

#include <algorithm>
#include <chrono>
#include <climits>
#include <cstring>
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
  if (stream) cudaStreamSynchronize(stream);
  for (auto& e : iter_events) cudaEventDestroy(e);
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
  SE_CUDA(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
  for (auto& st : ring) SE_CUDA(cudaEventCreateWithFlags(&st.ev, cudaEventDisableTiming));
  return set_frames_per_iteration(8);
}

Status Server::set_frames_per_iteration(int k) {
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
  if (request < (int)first_pending || request >= (int)requests.size())
    return {SE_ERR_INVALID_ARGUMENT, "only a request that has not been run can be cancelled"};
  requests[(size_t)request].cancelled = true;
  return Status::Ok();
}

Status Server::close_session(int id) {
  if (id < 0 || id >= (int)sessions.size() || !sessions[(size_t)id].open)
    return {SE_ERR_INVALID_ARGUMENT, "bad session"};
  Session& s = sessions[(size_t)id];
  if (s.active >= 0 || !s.queue.empty()) return {SE_ERR_INVALID_ARGUMENT, "session has requests in flight"};
  for (size_t r = first_pending; r < requests.size(); ++r)
    if (requests[r].session == id && !requests[r].cancelled)
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
  requests.push_back(std::move(r));
  *id = (int)requests.size() - 1;
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
    SE_CUDA(cudaMemcpyAsync(s.buf(s.cur), s.host.data(), s.host.size() * 4, cudaMemcpyHostToDevice, stream));
    SE_CUDA(cudaStreamSynchronize(stream));  // the host copy may be released now
    if (s.was_evicted) ++restores;
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

Status Server::run(bool plain) {
  for (auto& e : iter_events) cudaEventDestroy(e);
  iter_events.clear();
  iterations = 0;
  cell_updates = 0;
  wall_ms = 0;
  last_run_begin = first_pending;
  Status s = plain ? run_plain() : run_batched();
  if (!s.ok()) return s;
  SE_CUDA(cudaStreamSynchronize(stream));
  for (size_t i = last_run_begin; i < requests.size(); ++i) {
    Request& r = requests[i];
    float ms = 0;
    if (r.iter >= 0) SE_CUDA(cudaEventElapsedTime(&ms, iter_events[0], iter_events[(size_t)r.iter]));
    r.done_ms = ms;
    wall_ms = std::max(wall_ms, (double)ms);
  }
  return Status::Ok();
}

// Continuous batching.  Each iteration advances every active session by up to K frames in
// one launch (1 frame when its request starts with edits, followed by the edit pass), so
// sessions join and leave between iterations.  Progress is known on the host, so the host
// plans iterations ahead of the GPU (at most two in flight) and timestamps completions with
// events.
Status Server::run_batched() {
  TraceRange trace("se_server_run_batched");
  std::vector<int> pend;
  for (size_t i = first_pending; i < requests.size(); ++i)
    if (!requests[i].cancelled) pend.push_back((int)i);
  std::stable_sort(pend.begin(), pend.end(),
                   [&](int a, int b) { return requests[(size_t)a].arrival_ms < requests[(size_t)b].arrival_ms; });
  cudaEvent_t t0;
  SE_CUDA(cudaEventCreate(&t0));
  SE_CUDA(cudaEventRecord(t0, stream));
  SE_CUDA(cudaEventSynchronize(t0));
  iter_events.push_back(t0);  // index 0: the time origin
  const Clock::time_point host_t0 = Clock::now();
  const int K = variant->kmax;
  const size_t smem = tile_smem_bytes(*variant, rs->lut_shape());
  cudaKernel_t kern = rs->module->get(variant->serve_name());
  const uint16_t* lut = rs->d_lut;
  size_t next = 0;
  std::deque<int> waiting;  // sessions with queued requests, in order of their turn
  std::vector<int> active;
  long long it = 0;
  auto finish = [&](int sid) {  // request of session sid completes at the iteration being recorded
    Session& ss = sessions[(size_t)sid];
    requests[(size_t)ss.active].iter = (long long)iter_events.size();
    ss.active = -1;
    if (!ss.queue.empty()) waiting.push_back(sid);
  };
  for (;;) {
    const double now = ms_since(host_t0);
    while (next < pend.size() && requests[(size_t)pend[next]].arrival_ms <= now) {
      Session& ss = sessions[(size_t)requests[(size_t)pend[next]].session];
      const bool idle = ss.active < 0 && ss.queue.empty();
      ss.queue.push_back(pend[next]);
      if (idle) waiting.push_back(requests[(size_t)pend[next]].session);
      ++next;
    }
    std::vector<int> instant;  // requests that finished before any frame of work (frame-1 clear only)
    while (!waiting.empty()) {
      const int sid = waiting.front();
      Session& ss = sessions[(size_t)sid];
      bool ok = true;
      Status st = make_resident(sid, &ok);
      if (!st.ok()) return st;
      if (!ok) break;  // no memory until running sessions finish
      waiting.pop_front();
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
      for (int sid : instant) finish(sid);
      cudaEvent_t ev;
      SE_CUDA(cudaEventCreate(&ev));
      SE_CUDA(cudaEventRecord(ev, stream));
      iter_events.push_back(ev);
    }
    if (active.empty()) {
      if (next >= pend.size() && waiting.empty()) break;
      if (!waiting.empty() && next >= pend.size()) {
        bool any_active = false;
        for (auto& ss : sessions) any_active = any_active || ss.active >= 0;
        if (!any_active) return {SE_ERR_BUDGET, "a session does not fit the HBM budget"};
      }
      if (next < pend.size()) {
        const double wait = requests[(size_t)pend[next]].arrival_ms - ms_since(host_t0);
        if (wait > 0.05) std::this_thread::sleep_for(std::chrono::microseconds((long long)(wait * 1000 * 0.9)));
      }
      continue;
    }
    // ---- one iteration over every active session
    Stage& stg = ring[it % kRing];
    if (it >= kRing) SE_CUDA(cudaEventSynchronize(stg.ev));
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
    for (int sid : done) finish(sid);
    cudaEvent_t ev;
    SE_CUDA(cudaEventCreate(&ev));
    SE_CUDA(cudaEventRecord(ev, stream));
    iter_events.push_back(ev);
    active.swap(still);
    if (iter_events.size() > 3) SE_CUDA(cudaEventSynchronize(iter_events[iter_events.size() - 3]));
  }
  first_pending = requests.size();
  return Status::Ok();
}

// One request at a time in arrival order, one launch per frame (plus the edit pass after
// its first frame): the way the reference advances a world.
Status Server::run_plain() {
  TraceRange trace("se_server_run_plain");
  std::vector<int> pend;
  for (size_t i = first_pending; i < requests.size(); ++i)
    if (!requests[i].cancelled) pend.push_back((int)i);
  std::stable_sort(pend.begin(), pend.end(),
                   [&](int a, int b) { return requests[(size_t)a].arrival_ms < requests[(size_t)b].arrival_ms; });
  const TileVariant* v1 = nullptr;
  for (const TileVariant& t : tile_variants())
    if (t.kmax == 1) {
      v1 = &t;
      break;
    }
  cudaEvent_t t0;
  SE_CUDA(cudaEventCreate(&t0));
  SE_CUDA(cudaEventRecord(t0, stream));
  SE_CUDA(cudaEventSynchronize(t0));
  iter_events.push_back(t0);
  const Clock::time_point host_t0 = Clock::now();
  for (int ri : pend) {
    Request& r = requests[(size_t)ri];
    const double wait = r.arrival_ms - ms_since(host_t0);
    if (wait > 0.05) std::this_thread::sleep_for(std::chrono::microseconds((long long)(wait * 1000)));
    Session& ss = sessions[(size_t)r.session];
    bool ok = true;
    Status st = make_resident(r.session, &ok);
    if (!st.ok()) return st;
    if (!ok) return {SE_ERR_BUDGET, "a session does not fit the HBM budget"};
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
    cudaEvent_t ev;
    SE_CUDA(cudaEventCreate(&ev));
    SE_CUDA(cudaEventRecord(ev, stream));
    iter_events.push_back(ev);
    r.iter = (long long)iter_events.size() - 1;
  }
  first_pending = requests.size();
  return Status::Ok();
}

Status Server::get_grid(int id, uint32_t* host, size_t count) {
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
  std::vector<double> lat;
  for (size_t i = last_run_begin; i < first_pending && i < requests.size(); ++i)
    if (requests[i].done_ms >= 0) lat.push_back(requests[i].done_ms - requests[i].arrival_ms);
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
  out->peak_resident_bytes = (long long)peak_used;
  return Status::Ok();
}

}  // namespace se::rt
