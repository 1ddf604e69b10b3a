// NVRTC compilation of a rule set's kernels for sm_103a, with an on-disk cubin cache, and
// loading through the CUDA runtime's library API (no link-time dependency on libcuda).
#pragma once

#include <cuda_runtime.h>

#include <map>
#include <string>
#include <vector>

namespace se::rt {

// A tile-kernel instantiation: TW x TH output cells, up to KMAX frames per launch.
struct TileVariant {
  int tw, th, kmax, nt;
  std::string name() const;        // single-world kernel
  std::string edit_name() const;   // single-world kernel with the first frame's edit pass
  std::string multi_name() const;  // many-world (tile job list) kernel
  std::string serve_name() const;  // serving iteration kernel (per-world frame counts)
  int halo_x() const { return ((kmax + 3) / 4) * 4; }
  int halo_y() const { return kmax; }
  int sw() const { return tw + 2 * halo_x(); }  // shared array: tile plus halo
  int sh() const { return th + 2 * halo_y(); }
  size_t smem_bytes() const { return (size_t)sw() * (size_t)sh(); }
};
const std::vector<TileVariant>& tile_variants();

// Size of a rule set's block transition table: its u16 entries and the 32-bit words of the
// bitset of static keys that follows it (both 0 without a table).
struct LutShape {
  unsigned long long entries = 0, static_words = 0;
};
// Dynamic shared memory of a tile launch: the u8 tile, then the per-step list of chunks to
// evaluate.  The block transition table and its static-key bitset stay in global memory
// (read through the read-only cache).
size_t tile_smem_bytes(const TileVariant& t, const LutShape& lut);

// Full device source: prelude + generated rules + kernel template + instantiations.
std::string kernel_source(const std::string& generated_rules);

// Compiles `src` to an sm_103a cubin (cached by content hash).  No GPU needed.
bool compile_cubin(const std::string& src, std::string* cubin, std::string* log);

struct Module {
  cudaLibrary_t lib = nullptr;
  std::map<std::string, cudaKernel_t> kernels;
  size_t max_dyn_smem = 0;  // opt-in dynamic shared memory per CTA on this device
  ~Module();
  bool load(const std::string& cubin, const LutShape& lut, std::string* err);
  cudaKernel_t get(const std::string& name) const;
};

}  // namespace se::rt
