#include "batch.hpp"
#include "trace.hpp"

#include <algorithm>
#include <climits>
#include <cstring>

#include "../../../include/sandengine.h"

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

// Shared memory of a whole world in se_resident: the array (row stride a multiple of 8, a
// WALL border), a 48-byte header and a chunk list of one u16 entry per chunk.
size_t resident_bytes(int W, int H, const LutShape& lut) {
  (void)lut;
  const size_t SW = (size_t)(((W + 7) & ~7) + 8), SH = (size_t)H + 2;
  const size_t cap = (SW / 8) * (SH / 2);
  return ((SW * SH + 15) & ~(size_t)15) + 48 + ((2 * cap + 15) & ~(size_t)15);
}
}  // namespace

Batch::~Batch() {
  for (auto& kv : graphs) cudaGraphExecDestroy(kv.second);
  for (auto& r : resident)
    if (r.d_ids) cudaFree(r.d_ids);
  if (d_jobs) cudaFree(d_jobs);
  if (d_desc) cudaFree(d_desc);
  if (arena) cudaFree(arena);
  for (int i = 0; i < 4; ++i) {
    if (side[i]) cudaStreamDestroy(side[i]);
    if (join[i]) cudaEventDestroy(join[i]);
  }
  if (fork) cudaEventDestroy(fork);
  if (stream) cudaStreamDestroy(stream);
}

Status Batch::create(std::shared_ptr<Ruleset> r, int count, const int* widths, const int* heights) {
  if (count <= 0 || !widths || !heights) return {SE_ERR_INVALID_ARGUMENT, "need at least one world"};
  rs = std::move(r);
  Status s = rs->ensure_loaded();
  if (!s.ok()) return s;
  n = count;
  size_t bytes = 0;
  std::vector<size_t> off(2 * (size_t)n);
  for (int i = 0; i < n; ++i) {
    if (widths[i] <= 0 || heights[i] <= 0) return {SE_ERR_INVALID_ARGUMENT, "world sizes must be positive"};
    if (widths[i] > kMaxSide || heights[i] > kMaxSide)
      return {SE_ERR_INVALID_ARGUMENT, "world sides are limited to 1048576 cells"};
    const size_t b = ((size_t)widths[i] * heights[i] * 4 + 255) & ~(size_t)255;
    off[2 * i] = bytes;
    bytes += b;
    off[2 * i + 1] = bytes;
    bytes += b;
    cells += (long long)widths[i] * heights[i];
  }
  {
    cudaError_t e = cudaMalloc(&arena, bytes);
    if (e != cudaSuccess) return {SE_ERR_OUT_OF_MEMORY, std::string("cudaMalloc(batch): ") + cudaGetErrorString(e)};
  }
  SE_CUDA(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
  for (int i = 0; i < 4; ++i) {
    SE_CUDA(cudaStreamCreateWithFlags(&side[i], cudaStreamNonBlocking));
    SE_CUDA(cudaEventCreateWithFlags(&join[i], cudaEventDisableTiming));
  }
  SE_CUDA(cudaEventCreateWithFlags(&fork, cudaEventDisableTiming));
  SE_CUDA(cudaMemsetAsync(arena, 0, bytes, stream));
  desc.resize((size_t)n);
  for (int i = 0; i < n; ++i)
    desc[(size_t)i] = WorldDesc{reinterpret_cast<uint32_t*>(reinterpret_cast<char*>(arena) + off[2 * (size_t)i]),
                                reinterpret_cast<uint32_t*>(reinterpret_cast<char*>(arena) + off[2 * (size_t)i + 1]),
                                widths[i], heights[i], 0, 0, 0, 0};
  resident_limit = rs->module->max_dyn_smem;
  s = classify();
  if (!s.ok()) return s;
  SE_CUDA(cudaMalloc(&d_desc, sizeof(WorldDesc) * (size_t)n));
  s = upload_desc();
  if (!s.ok()) return s;
  SE_CUDA(cudaStreamSynchronize(stream));
  return Status::Ok();
}

Status Batch::classify() {
  const size_t maxsm = rs->module->max_dyn_smem;
  const LutShape lut = rs->lut_shape();
  // size classes for whole-world CTAs: occupancy is set by the largest world of a class
  const size_t class_max[3] = {40 * 1024, 100 * 1024, maxsm};
  const int class_threads[3] = {256, 512, 1024};
  for (auto& R : resident)
    if (R.d_ids) cudaFree(R.d_ids);
  resident.assign(3, Resident{});
  tiled.clear();
  for (int i = 0; i < n; ++i) {
    const size_t rb = resident_bytes(desc[(size_t)i].W, desc[(size_t)i].H, lut);
    int cls = -1;
    if (rb <= resident_limit)
      for (int c = 0; c < 3; ++c)
        if (rb <= class_max[c]) {
          cls = c;
          break;
        }
    if (cls < 0) tiled.push_back(i);
    else resident[(size_t)cls].ids.push_back(i);
  }
  for (int c = 0; c < 3; ++c) {
    Resident& R = resident[(size_t)c];
    R.threads = class_threads[c];
    std::sort(R.ids.begin(), R.ids.end(), [&](int a, int b) {
      return (long long)desc[(size_t)a].W * desc[(size_t)a].H > (long long)desc[(size_t)b].W * desc[(size_t)b].H;
    });
    for (int id : R.ids) R.smem = std::max(R.smem, resident_bytes(desc[(size_t)id].W, desc[(size_t)id].H, lut));
    if (!R.ids.empty()) {
      SE_CUDA(cudaMalloc(&R.d_ids, R.ids.size() * sizeof(int)));
      SE_CUDA(cudaMemcpyAsync(R.d_ids, R.ids.data(), R.ids.size() * sizeof(int), cudaMemcpyHostToDevice, stream));
    }
  }
  SE_CUDA(cudaStreamSynchronize(stream));
  return Status::Ok();
}

Status Batch::set_resident_limit(size_t bytes) {
  resident_limit = bytes;
  Status s = classify();
  if (!s.ok()) return s;
  if (variant) return set_variant(variant);  // the tile job list
  return invalidate_graphs();
}

Status Batch::upload_desc() {
  SE_CUDA(cudaMemcpyAsync(d_desc, desc.data(), sizeof(WorldDesc) * (size_t)n, cudaMemcpyHostToDevice, stream));
  return Status::Ok();
}

Status Batch::invalidate_graphs() {
  for (auto& kv : graphs) cudaGraphExecDestroy(kv.second);
  graphs.clear();
  return Status::Ok();
}

Status Batch::set_variant(const TileVariant* v) {
  variant = v;
  jobs.clear();
  for (int w : tiled) {
    const WorldDesc& d = desc[(size_t)w];
    for (int y = 0; y < d.H; y += v->th)
      for (int x = 0; x < d.W; x += v->tw) jobs.push_back(TileJob{w, x, y, 0});
  }
  if (jobs.size() > d_jobs_cap) {
    if (d_jobs) cudaFree(d_jobs);
    d_jobs = nullptr;
    SE_CUDA(cudaMalloc(&d_jobs, jobs.size() * sizeof(TileJob)));
    d_jobs_cap = jobs.size();
  }
  if (!jobs.empty())
    SE_CUDA(cudaMemcpyAsync(d_jobs, jobs.data(), jobs.size() * sizeof(TileJob), cudaMemcpyHostToDevice, stream));
  SE_CUDA(cudaStreamSynchronize(stream));
  return invalidate_graphs();
}

Status Batch::set_grid(int i, const uint32_t* host, size_t count) {
  if (i < 0 || i >= n || !host) return {SE_ERR_INVALID_ARGUMENT, "bad world index"};
  const WorldDesc& d = desc[(size_t)i];
  if (count != (size_t)d.W * d.H) return {SE_ERR_INVALID_ARGUMENT, "count must be width*height"};
  SE_CUDA(cudaMemcpyAsync(d.cur ? d.buf1 : d.buf0, host, count * 4, cudaMemcpyHostToDevice, stream));
  SE_CUDA(cudaStreamSynchronize(stream));
  return Status::Ok();
}

Status Batch::get_grid(int i, uint32_t* host, size_t count) {
  if (i < 0 || i >= n || !host) return {SE_ERR_INVALID_ARGUMENT, "bad world index"};
  const WorldDesc& d = desc[(size_t)i];
  if (count != (size_t)d.W * d.H) return {SE_ERR_INVALID_ARGUMENT, "count must be width*height"};
  SE_CUDA(cudaMemcpyAsync(host, d.cur ? d.buf1 : d.buf0, count * 4, cudaMemcpyDeviceToHost, stream));
  SE_CUDA(cudaStreamSynchronize(stream));
  return Status::Ok();
}

Status Batch::set_frame(int i, int32_t f) {
  if (i < 0 || i >= n) return {SE_ERR_INVALID_ARGUMENT, "bad world index"};
  if (f < 0) return {SE_ERR_INVALID_ARGUMENT, "frame must be >= 0"};
  desc[(size_t)i].frame = f;
  SE_CUDA(cudaMemcpyAsync(d_desc + i, &desc[(size_t)i], sizeof(WorldDesc), cudaMemcpyHostToDevice, stream));
  SE_CUDA(cudaStreamSynchronize(stream));
  return Status::Ok();
}

Status Batch::launch_body(int F, cudaStream_t s) {
  const int k = variant->kmax;
  const int P = tiled.empty() ? 0 : (F + k - 1) / k;
  const uint16_t* lut = rs->d_lut;
  SE_CUDA(cudaEventRecord(fork, s));
  for (size_t c = 0; c < resident.size(); ++c) {
    const Resident& R = resident[c];
    if (R.ids.empty()) continue;
    SE_CUDA(cudaStreamWaitEvent(side[c], fork, 0));
    int frames = F, flip = P & 1;
    const WorldDesc* dd = d_desc;
    const int* ids = R.d_ids;
    void* args[] = {(void*)&dd, (void*)&ids, &frames, &flip, (void*)&lut};
    SE_CUDA(cudaLaunchKernel((const void*)rs->module->get("se_resident"), dim3((unsigned)R.ids.size()),
                             dim3((unsigned)R.threads), args, R.smem, side[c]));
    SE_CUDA(cudaEventRecord(join[c], side[c]));
  }
  const size_t smem = tile_smem_bytes(*variant, rs->lut_shape());
  for (int p = 0; p < P; ++p) {
    int pass = p, done = p * k, kp = std::min(k, F - p * k);
    const WorldDesc* dd = d_desc;
    const TileJob* jb = d_jobs;
    void* args[] = {(void*)&dd, (void*)&jb, &pass, &done, &kp, (void*)&lut};
    SE_CUDA(cudaLaunchKernel((const void*)rs->module->get(variant->multi_name()), dim3((unsigned)jobs.size()),
                             dim3((unsigned)variant->nt), args, smem, s));
  }
  for (size_t c = 0; c < resident.size(); ++c)
    if (!resident[c].ids.empty()) SE_CUDA(cudaStreamWaitEvent(s, join[c], 0));
  {
    WorldDesc* dd = d_desc;
    int nn = n, frames = F, passes = P;
    void* args[] = {(void*)&dd, &nn, &frames, &passes};
    SE_CUDA(cudaLaunchKernel((const void*)rs->module->get("se_batch_finalize"), dim3((unsigned)((n + 255) / 256)),
                             dim3(256), args, 0, s));
  }
  return Status::Ok();
}

Status Batch::autotune(int reps, int* best_k) {
  if (reps < 1) reps = 1;
  const TileVariant* best = nullptr;
  if (tiled.empty()) {
    for (const TileVariant& v : tile_variants())
      if (!best || v.kmax > best->kmax) best = &v;  // only the pass count matters
  } else {
    cudaEvent_t a, b;
    SE_CUDA(cudaEventCreate(&a));
    SE_CUDA(cudaEventCreate(&b));
    long long tiled_cells = 0;
    for (int w : tiled) tiled_cells += (long long)desc[(size_t)w].W * desc[(size_t)w].H;
    double best_rate = 0;
    for (const TileVariant& v : tile_variants()) {
      Status s = set_variant(&v);
      if (!s.ok()) return s;
      const size_t smem = tile_smem_bytes(v, rs->lut_shape());
      const uint16_t* lut = rs->d_lut;
      const WorldDesc* dd = d_desc;
      const TileJob* jb = d_jobs;
      int pass = 0, done = 0, kp = v.kmax;
      void* args[] = {(void*)&dd, (void*)&jb, &pass, &done, &kp, (void*)&lut};
      // pass 0 reads the current buffers and writes the spare ones: the worlds are unchanged
      for (int r = 0; r <= reps; ++r) {
        if (r == 1) SE_CUDA(cudaEventRecord(a, stream));
        SE_CUDA(cudaLaunchKernel((const void*)rs->module->get(v.multi_name()), dim3((unsigned)jobs.size()),
                                 dim3((unsigned)v.nt), args, smem, stream));
      }
      SE_CUDA(cudaEventRecord(b, stream));
      SE_CUDA(cudaEventSynchronize(b));
      float ms = 0;
      SE_CUDA(cudaEventElapsedTime(&ms, a, b));
      const double rate = (double)tiled_cells * v.kmax * reps / (ms > 0 ? ms : 1e-6);
      if (rate > best_rate) best_rate = rate, best = &v;
    }
    cudaEventDestroy(a);
    cudaEventDestroy(b);
  }
  Status s = set_variant(best);
  if (!s.ok()) return s;
  if (best_k) *best_k = best->kmax;
  return Status::Ok();
}

Status Batch::step(int F) {
  TraceRange trace("se_batch_step");
  if (F < 0) return {SE_ERR_INVALID_ARGUMENT, "nframes must be >= 0"};
  if (F == 0) return Status::Ok();
  int zero = 0;
  int32_t maxf = 0;
  for (auto& d : desc) {
    zero += d.frame == 0;
    maxf = std::max(maxf, d.frame);
  }
  if ((int64_t)maxf + F > INT32_MAX) return {SE_ERR_INVALID_ARGUMENT, "frame counter would overflow i32"};
  if (zero && zero != n)
    return {SE_ERR_INVALID_ARGUMENT, "worlds at frame 0 clear on their next frame; give all worlds of a batch "
                                     "frame 0 or none"};
  if (zero == n) {  // frame 1 clears every world (falling_sand.glsl:128-131)
    for (auto& d : desc) {
      SE_CUDA(cudaMemsetAsync(d.cur ? d.buf1 : d.buf0, 0, (size_t)d.W * d.H * 4, stream));
      d.frame = 1;
    }
    Status s = upload_desc();
    if (!s.ok()) return s;
    if (--F == 0) return Status::Ok();
  }
  if (!variant) {
    Status s = steps_per_launch > 0 ? Status::Ok() : autotune(2, nullptr);
    if (!s.ok()) return s;
    if (!variant) {
      const TileVariant* v = nullptr;
      for (const TileVariant& t : tile_variants())
        if (t.kmax >= steps_per_launch && (!v || t.kmax < v->kmax)) v = &t;
      s = set_variant(v);
      if (!s.ok()) return s;
    }
  }
  auto it = graphs.find(F);
  if (it == graphs.end()) {
    cudaGraph_t g;
    SE_CUDA(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal));
    Status s = launch_body(F, stream);
    cudaError_t e = cudaStreamEndCapture(stream, &g);
    if (!s.ok()) return s;
    if (e != cudaSuccess) return cuda_fail("cudaStreamEndCapture", e);
    cudaGraphExec_t ex;
    e = cudaGraphInstantiate(&ex, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return cuda_fail("cudaGraphInstantiate", e);
    it = graphs.emplace(F, ex).first;
  }
  SE_CUDA(cudaGraphLaunch(it->second, stream));
  const int k = variant->kmax;
  const int P = tiled.empty() ? 0 : (F + k - 1) / k;
  for (auto& d : desc) {
    d.frame += F;
    d.cur ^= P & 1;
  }
  return Status::Ok();
}

Status Batch::step_plain(int F) {
  if (F < 0) return {SE_ERR_INVALID_ARGUMENT, "nframes must be >= 0"};
  const TileVariant* v1 = nullptr;
  for (const TileVariant& t : tile_variants())
    if (t.kmax == 1) {
      v1 = &t;
      break;
    }
  for (int f = 0; f < F; ++f) {
    for (auto& d : desc) {
      const int fr = d.frame + 1;
      if (fr == 1) {
        SE_CUDA(cudaMemsetAsync(d.cur ? d.buf1 : d.buf0, 0, (size_t)d.W * d.H * 4, stream));
      } else {
        const uint32_t* src = d.cur ? d.buf1 : d.buf0;
        uint32_t* dst = d.cur ? d.buf0 : d.buf1;
        Status s = launch_tile_kernel(*rs, *v1, src, dst, d.W, d.H, fr, 1, 0, d.H, stream);
        if (!s.ok()) return s;
        d.cur ^= 1;
      }
      d.frame = fr;
    }
  }
  return upload_desc();
}

}  // namespace se::rt
