#include "jit.hpp"

#include <nvrtc.h>
#include <sys/stat.h>
#include <unistd.h>

#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <functional>
#include <mutex>
#include <sstream>

#include "kernel_src.inc"  // SE_PRELUDE_SRC, SE_MARGOLUS_SRC (generated from csrc/kernels)

namespace se::rt {

std::string TileVariant::name() const {
  return "se_tile_" + std::to_string(tw) + "x" + std::to_string(th) + "_k" + std::to_string(kmax);
}

std::string TileVariant::edit_name() const {
  return "se_tile_edit_" + std::to_string(tw) + "x" + std::to_string(th) + "_k" + std::to_string(kmax);
}

// Tile shapes and fusion depths compiled into every rule-set module; the launcher and the
// autotuner choose among them.  Larger tiles recompute a smaller share of halo cells per
// fused step (128x64 at k=8: 1.41x the tile's cells; 256x128 at k=8: 1.20x).  The shared
// array must stay under 65,536 cells (16-bit offsets in the chunk list).
const std::vector<TileVariant>& tile_variants() {
  static const std::vector<TileVariant> v = {
      {128, 64, 1, 256},  {256, 32, 1, 256},  {128, 32, 1, 256},  {128, 64, 2, 256},
      {128, 64, 4, 256},  {128, 64, 8, 256},  {128, 128, 8, 256}, {128, 128, 16, 256},
      {256, 64, 4, 256},  {64, 64, 4, 256},   {256, 128, 8, 512}, {192, 128, 8, 256},
      {256, 128, 4, 512}, {256, 64, 8, 256},
  };
  return v;
}

std::string kernel_source(const std::string& generated_rules) {
  std::ostringstream o;
  o << SE_PRELUDE_SRC << "\n" << generated_rules << "\n" << SE_MARGOLUS_SRC << "\n";
  for (const TileVariant& t : tile_variants()) {
    o << "extern \"C\" __global__ void __launch_bounds__(" << t.nt << ") " << t.name()
      << "(const uint32_t* __restrict__ src, uint32_t* __restrict__ dst, int W, int H, int f0, int k,"
         " const uint16_t* __restrict__ lut, int ya, int yb) {\n"
      << "  se_tile_impl<" << t.tw << ", " << t.th << ", " << t.kmax << ", " << t.nt
      << ">(src, dst, W, H, f0, k, lut, ya, yb);\n}\n";
    // the edit list travels in the parameter space, read in place (__grid_constant__)
    o << "extern \"C\" __global__ void __launch_bounds__(" << t.nt << ") " << t.edit_name()
      << "(const uint32_t* __restrict__ src, uint32_t* __restrict__ dst, int W, int H, int f0, int k,"
         " const uint16_t* __restrict__ lut, int ya, int yb, const __grid_constant__ SeEditParams edits,"
         " int nedits) {\n"
      << "  se_tile_impl<" << t.tw << ", " << t.th << ", " << t.kmax << ", " << t.nt
      << ">(src, dst, W, H, f0, k, lut, ya, yb, &edits, nedits);\n}\n";
    o << "extern \"C\" __global__ void __launch_bounds__(" << t.nt << ") " << t.multi_name()
      << "(const SeWorldDesc* __restrict__ worlds, const SeTileJob* __restrict__ jobs, int pass,"
         " int frames_done, int k, const uint16_t* __restrict__ lut) {\n"
      << "  se_mtile_impl<" << t.tw << ", " << t.th << ", " << t.kmax << ", " << t.nt
      << ">(worlds, jobs, pass, frames_done, k, lut);\n}\n";
    o << "extern \"C\" __global__ void __launch_bounds__(" << t.nt << ") " << t.serve_name()
      << "(const SeWorldDesc* __restrict__ descs, const int* __restrict__ prefix, int nactive,"
         " const uint16_t* __restrict__ lut) {\n"
      << "  se_stile_impl<" << t.tw << ", " << t.th << ", " << t.kmax << ", " << t.nt
      << ">(descs, prefix, nactive, lut);\n}\n";
  }
  return o.str();
}

std::string TileVariant::serve_name() const {
  return "se_stile_" + std::to_string(tw) + "x" + std::to_string(th) + "_k" + std::to_string(kmax);
}

std::string TileVariant::multi_name() const {
  return "se_mtile_" + std::to_string(tw) + "x" + std::to_string(th) + "_k" + std::to_string(kmax);
}

namespace {

std::string cache_dir() {
  if (const char* d = getenv("SE_CACHE_DIR")) return d;
  if (const char* x = getenv("XDG_CACHE_HOME")) return std::string(x) + "/sandengine_gb300";
  if (const char* h = getenv("HOME")) return std::string(h) + "/.cache/sandengine_gb300";
  return "";
}

std::string hex_digest(const std::string& s) {
  // FNV-1a 64 twice with different offsets: a cache key, not a security boundary.
  uint64_t a = 1469598103934665603ull, b = 1099511628211ull * 7ull + 13ull;
  for (unsigned char c : s) {
    a = (a ^ c) * 1099511628211ull;
    b = (b ^ c) * 0x100000001b3ull + 0x9e3779b97f4a7c15ull;
  }
  char buf[40];
  snprintf(buf, sizeof buf, "%016llx%016llx", (unsigned long long)a, (unsigned long long)b);
  return buf;
}

const std::vector<std::string>& nvrtc_options() {
  static const std::vector<std::string> o = {"-arch=sm_103a", "--std=c++17", "--fmad=false", "-lineinfo",
                                             "--extra-device-vectorization"};
  return o;
}

std::mutex g_cache_mu;

}  // namespace

bool compile_cubin(const std::string& src, std::string* cubin, std::string* log) {
  int maj = 0, min = 0;
  nvrtcVersion(&maj, &min);
  std::string key_src = src + "\n//nvrtc " + std::to_string(maj) + "." + std::to_string(min);
  for (auto& o : nvrtc_options()) key_src += "\n//" + o;
  const std::string key = hex_digest(key_src);
  const std::string dir = cache_dir();
  const std::string path = dir.empty() ? "" : dir + "/" + key + ".cubin";
  {
    std::lock_guard<std::mutex> g(g_cache_mu);
    if (!path.empty()) {
      std::ifstream f(path, std::ios::binary);
      if (f) {
        std::stringstream ss;
        ss << f.rdbuf();
        *cubin = ss.str();
        if (!cubin->empty()) return true;
      }
    }
  }
  nvrtcProgram prog;
  if (nvrtcCreateProgram(&prog, src.c_str(), "sandengine_rules.cu", 0, nullptr, nullptr) != NVRTC_SUCCESS) {
    *log = "nvrtcCreateProgram failed";
    return false;
  }
  std::vector<const char*> opts;
  for (auto& o : nvrtc_options()) opts.push_back(o.c_str());
  nvrtcResult rc = nvrtcCompileProgram(prog, (int)opts.size(), opts.data());
  size_t lsz = 0;
  nvrtcGetProgramLogSize(prog, &lsz);
  std::string lg(lsz, '\0');
  if (lsz) nvrtcGetProgramLog(prog, lg.data());
  if (rc != NVRTC_SUCCESS) {
    *log = std::string(nvrtcGetErrorString(rc)) + "\n" + lg;
    nvrtcDestroyProgram(&prog);
    return false;
  }
  size_t csz = 0;
  nvrtcGetCUBINSize(prog, &csz);
  cubin->assign(csz, '\0');
  nvrtcGetCUBIN(prog, cubin->data());
  nvrtcDestroyProgram(&prog);
  if (!path.empty()) {
    std::lock_guard<std::mutex> g(g_cache_mu);
    std::string cmd_dir = dir;
    // mkdir -p
    for (size_t i = 1; i <= cmd_dir.size(); ++i)
      if (i == cmd_dir.size() || cmd_dir[i] == '/') mkdir(cmd_dir.substr(0, i).c_str(), 0755);
    std::string tmp = path + ".tmp" + std::to_string(getpid());
    std::ofstream f(tmp, std::ios::binary);
    if (f) {
      f.write(cubin->data(), (std::streamsize)cubin->size());
      f.close();
      rename(tmp.c_str(), path.c_str());
    }
  }
  return true;
}

Module::~Module() {
  if (lib) cudaLibraryUnload(lib);
}

size_t tile_smem_bytes(const TileVariant& t, const LutShape& lut) {
  (void)lut;
  size_t b = (t.smem_bytes() + 15) & ~(size_t)15;
  // 48-byte header (slack, list counters, uniform-material flags), then the per-step list
  // of chunks (4 blocks) to evaluate, one u16 offset each
  b += 48 + ((2 * (size_t)(t.sw() / 8) * (size_t)(t.sh() / 2) + 15) & ~(size_t)15);
  return b;
}

bool Module::load(const std::string& cubin, const LutShape& lut, std::string* err) {
  cudaError_t e = cudaLibraryLoadData(&lib, cubin.data(), nullptr, nullptr, 0, nullptr, nullptr, 0);
  if (e != cudaSuccess) {
    *err = std::string("cudaLibraryLoadData: ") + cudaGetErrorString(e);
    lib = nullptr;
    return false;
  }
  std::vector<std::string> names = {"se_edit", "se_resident", "se_batch_finalize"};
  if (lut.entries) {
    names.push_back("se_build_lut");
    names.push_back("se_build_static");
  }
  for (auto& t : tile_variants()) {
    names.push_back(t.name());
    names.push_back(t.edit_name());
    names.push_back(t.multi_name());
    names.push_back(t.serve_name());
  }
  for (auto& n : names) {
    cudaKernel_t k;
    e = cudaLibraryGetKernel(&k, lib, n.c_str());
    if (e != cudaSuccess) {
      *err = "cudaLibraryGetKernel(" + n + "): " + cudaGetErrorString(e);
      return false;
    }
    kernels[n] = k;
  }
  for (auto& t : tile_variants()) {
    for (const std::string& n : {t.name(), t.edit_name(), t.multi_name(), t.serve_name()}) {
      e = cudaFuncSetAttribute((const void*)kernels[n], cudaFuncAttributeMaxDynamicSharedMemorySize,
                               (int)tile_smem_bytes(t, lut));
      if (e != cudaSuccess) {
        *err = std::string("cudaFuncSetAttribute: ") + cudaGetErrorString(e);
        return false;
      }
    }
  }
  int dev = 0, optin = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  cudaFuncAttributes fa{};
  e = cudaFuncGetAttributes(&fa, (const void*)kernels["se_resident"]);
  if (e != cudaSuccess) {
    *err = std::string("cudaFuncGetAttributes(se_resident): ") + cudaGetErrorString(e);
    return false;
  }
  // static shared memory (the rule set's property tables) counts against the same limit
  max_dyn_smem = (size_t)optin - fa.sharedSizeBytes;
  e = cudaFuncSetAttribute((const void*)kernels["se_resident"], cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)max_dyn_smem);
  if (e != cudaSuccess) {
    *err = std::string("cudaFuncSetAttribute(se_resident): ") + cudaGetErrorString(e);
    return false;
  }
  return true;
}

cudaKernel_t Module::get(const std::string& name) const {
  auto it = kernels.find(name);
  return it == kernels.end() ? nullptr : it->second;
}

}  // namespace se::rt
