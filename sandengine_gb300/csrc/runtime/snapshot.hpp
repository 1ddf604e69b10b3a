// World snapshots: the grid and the frame counter, which together are the whole state of a
// world (RAND depends on the frame, falling_sand.glsl:83; the block offset on frame % 4,
// operations.glsl:25-34).
//
// File layout (little-endian):
//   0  char[4]  "SEW1"
//   4  u32      header bytes (32)
//   8  u32      width
//  12  u32      height
//  16  i32      frame counter (before the next frame)
//  20  u32      number of materials of the rule set
//  24  u64      FNV-1a 64 of the rule set's generated GLSL (gen/materials.glsl + gen/rules.glsl)
//  32  u32[width*height]  cells, row-major
#pragma once

#include <cstdint>
#include <string>
#include <vector>

namespace se::rt {

struct SnapshotHeader {
  uint32_t width = 0, height = 0;
  int32_t frame = 0;
  uint32_t num_materials = 0;
  uint64_t ruleset_hash = 0;
};

uint64_t ruleset_fingerprint(const std::string& materials_glsl, const std::string& rules_glsl);
bool snapshot_write(const std::string& path, const SnapshotHeader& h, const uint32_t* cells, std::string* err);
bool snapshot_read_header(const std::string& path, SnapshotHeader* h, std::string* err);
bool snapshot_read(const std::string& path, SnapshotHeader* h, std::vector<uint32_t>* cells, std::string* err);

}  // namespace se::rt
