#include "engine.hpp"

#include <algorithm>
#include <cstring>

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

Status Ruleset::compile() {
  std::lock_guard<std::mutex> g(mu);
  if (compiled) return Status::Ok();
  if (codegen_code) return {codegen_code, codegen_message};
  std::string log;
  if (!compile_cubin(kernel_source(cuda.source), &cubin, &log)) return {SE_ERR_COMPILE, "NVRTC: " + log};
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
  if (!m->load(cubin, &err)) return {SE_ERR_CUDA, err};
  module = std::move(m);
  return Status::Ok();
}

World::~World() {
  if (buf[0]) cudaFree(buf[0]);
  if (buf[1]) cudaFree(buf[1]);
  if (d_scratch) cudaFree(d_scratch);
  if (own_stream) cudaStreamDestroy(own_stream);
}

Status World::create(std::shared_ptr<Ruleset> r, int w, int h) {
  if (w <= 0 || h <= 0) return {SE_ERR_INVALID_ARGUMENT, "world size must be positive"};
  if ((int64_t)w * h > (int64_t)1 << 36) return {SE_ERR_INVALID_ARGUMENT, "world too large"};
  rs = std::move(r);
  W = w;
  H = h;
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

int World::default_k() const {
  if (steps_per_launch > 0) return steps_per_launch;
  return 1;
}

static const TileVariant* pick_variant(int k) {
  const TileVariant* best = nullptr;
  for (const TileVariant& t : tile_variants())
    if (t.kmax >= k && (!best || t.kmax < best->kmax)) best = &t;
  return best;
}

Status World::launch_tiles(int f0, int k) {
  const TileVariant* v = pick_variant(k);
  if (!v) return {SE_ERR_INVALID_ARGUMENT, "no kernel variant for this many frames per launch"};
  cudaKernel_t kern = rs->module->get(v->name());
  const uint32_t* src = buf[cur];
  uint32_t* dst = buf[cur ^ 1];
  int Wv = W, Hv = H;
  void* args[] = {(void*)&src, (void*)&dst, &Wv, &Hv, &f0, &k};
  dim3 grid((unsigned)((W + v->tw - 1) / v->tw), (unsigned)((H + v->th - 1) / v->th));
  SE_CUDA(cudaLaunchKernel((const void*)kern, grid, dim3((unsigned)v->nt), args, v->smem_bytes(), stream));
  cur ^= 1;
  return Status::Ok();
}

Status World::launch_edit(const se_modification* mods, int nlive) {
  EditParams p;
  memset(&p, 0, sizeof p);
  long long total = 0;
  const int nmat = rs->num_materials();
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
    int64_t x0 = 0, y0 = 0, x1 = W - 1, y1 = H - 1;
    if (normal) {
      x0 = std::max<int64_t>(0, m.position[0] - rad);
      x1 = std::min<int64_t>(W - 1, m.position[0] + rad);
      y0 = std::max<int64_t>(0, m.position[1] - rad);
      y1 = std::min<int64_t>(H - 1, m.position[1] + rad);
    }
    p.start[i] = total;
    if (x1 >= x0 && y1 >= y0) {
      p.box[4 * i + 0] = (int)x0;
      p.box[4 * i + 1] = (int)y0;
      p.box[4 * i + 2] = (int)x1;
      p.box[4 * i + 3] = (int)y1;
      total += (x1 - x0 + 1) * (y1 - y0 + 1);
    } else {
      p.box[4 * i + 0] = 0;
      p.box[4 * i + 1] = 0;
      p.box[4 * i + 2] = 0;
      p.box[4 * i + 3] = 0;
    }
  }
  p.start[nlive] = total;
  if (total == 0) return Status::Ok();
  cudaKernel_t kern = rs->module->get("se_edit");
  uint32_t* g = buf[cur];
  int Wv = W, Hv = H, n = nlive;
  void* args[] = {(void*)&g, &Wv, &Hv, &n, &total, &p};
  dim3 grid((unsigned)((total + 255) / 256));
  SE_CUDA(cudaLaunchKernel((const void*)kern, grid, dim3(256), args, 0, stream));
  return Status::Ok();
}

Status World::step(int nframes, const se_modification* mods, int nmods) {
  if (nframes < 0) return {SE_ERR_INVALID_ARGUMENT, "nframes must be >= 0"};
  if (nmods < 0 || (nmods > 0 && !mods)) return {SE_ERR_INVALID_ARGUMENT, "bad modification list"};
  if ((int64_t)frame + nframes > INT32_MAX) return {SE_ERR_INVALID_ARGUMENT, "frame counter would overflow i32"};
  int nlive = 0;
  const int nseen = std::min(nmods, SE_MAX_MODIFICATIONS);  // simulation.rs:205
  while (nlive < nseen && mods[nlive].mod_size != 0) ++nlive;  // falling_sand.glsl:139-141
  const int kdef = std::max(1, default_k());
  int i = 0;
  while (i < nframes) {
    const int f = frame + 1 + i;
    if (f == 1) {  // falling_sand.glsl:128-131: clear, mods ignored
      SE_CUDA(cudaMemsetAsync(buf[cur], 0, (size_t)W * H * sizeof(uint32_t), stream));
      ++i;
      continue;
    }
    if (i == 0 && nlive > 0) {
      Status s = launch_tiles(f, 1);
      if (!s.ok()) return s;
      s = launch_edit(mods, nlive);
      if (!s.ok()) return s;
      ++i;
      continue;
    }
    const int k = std::min(kdef, nframes - i);
    Status s = launch_tiles(f, k);
    if (!s.ok()) return s;
    i += k;
  }
  frame += nframes;
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
