#include "snapshot.hpp"

#include <cstdio>
#include <cstring>

namespace se::rt {

namespace {
void put32(unsigned char* p, uint32_t v) {
  for (int i = 0; i < 4; ++i) p[i] = (unsigned char)(v >> (8 * i));
}
void put64(unsigned char* p, uint64_t v) {
  for (int i = 0; i < 8; ++i) p[i] = (unsigned char)(v >> (8 * i));
}
uint32_t get32(const unsigned char* p) {
  uint32_t v = 0;
  for (int i = 0; i < 4; ++i) v |= (uint32_t)p[i] << (8 * i);
  return v;
}
uint64_t get64(const unsigned char* p) {
  uint64_t v = 0;
  for (int i = 0; i < 8; ++i) v |= (uint64_t)p[i] << (8 * i);
  return v;
}
constexpr uint32_t kHeader = 32;
}  // namespace

uint64_t ruleset_fingerprint(const std::string& a, const std::string& b) {
  uint64_t h = 1469598103934665603ull;
  for (const std::string* s : {&a, &b})
    for (unsigned char c : *s) h = (h ^ c) * 1099511628211ull;
  return h;
}

bool snapshot_write(const std::string& path, const SnapshotHeader& h, const uint32_t* cells, std::string* err) {
  FILE* f = fopen(path.c_str(), "wb");
  if (!f) {
    *err = "cannot open " + path + " for writing";
    return false;
  }
  unsigned char hdr[kHeader] = {'S', 'E', 'W', '1'};
  put32(hdr + 4, kHeader);
  put32(hdr + 8, h.width);
  put32(hdr + 12, h.height);
  put32(hdr + 16, (uint32_t)h.frame);
  put32(hdr + 20, h.num_materials);
  put64(hdr + 24, h.ruleset_hash);
  bool ok = fwrite(hdr, 1, kHeader, f) == kHeader;
  const size_t n = (size_t)h.width * h.height;
  std::vector<unsigned char> row(4 * (size_t)h.width);
  for (size_t y = 0; ok && y < h.height; ++y) {  // explicit little-endian cells
    for (size_t x = 0; x < h.width; ++x) put32(row.data() + 4 * x, cells[y * h.width + x]);
    ok = fwrite(row.data(), 1, row.size(), f) == row.size();
  }
  (void)n;
  if (fclose(f) != 0) ok = false;
  if (!ok) *err = "write to " + path + " failed";
  return ok;
}

bool snapshot_read_header(const std::string& path, SnapshotHeader* h, std::string* err) {
  FILE* f = fopen(path.c_str(), "rb");
  if (!f) {
    *err = "cannot open " + path;
    return false;
  }
  unsigned char hdr[kHeader];
  const bool ok = fread(hdr, 1, kHeader, f) == kHeader;
  fclose(f);
  if (!ok || memcmp(hdr, "SEW1", 4) != 0 || get32(hdr + 4) != kHeader) {
    *err = path + " is not a sandengine world snapshot";
    return false;
  }
  h->width = get32(hdr + 8);
  h->height = get32(hdr + 12);
  h->frame = (int32_t)get32(hdr + 16);
  h->num_materials = get32(hdr + 20);
  h->ruleset_hash = get64(hdr + 24);
  if (h->width == 0 || h->height == 0 || (uint64_t)h->width * h->height > (1ull << 36) || h->frame < 0) {
    *err = path + ": invalid snapshot header";
    return false;
  }
  return true;
}

bool snapshot_read(const std::string& path, SnapshotHeader* h, std::vector<uint32_t>* cells, std::string* err) {
  if (!snapshot_read_header(path, h, err)) return false;
  FILE* f = fopen(path.c_str(), "rb");
  if (!f) {
    *err = "cannot open " + path;
    return false;
  }
  fseek(f, (long)kHeader, SEEK_SET);
  cells->resize((size_t)h->width * h->height);
  std::vector<unsigned char> row(4 * (size_t)h->width);
  bool ok = true;
  for (size_t y = 0; ok && y < h->height; ++y) {
    ok = fread(row.data(), 1, row.size(), f) == row.size();
    for (size_t x = 0; ok && x < h->width; ++x) (*cells)[y * h->width + x] = get32(row.data() + 4 * x);
  }
  fclose(f);
  if (!ok) *err = path + ": truncated snapshot";
  return ok;
}

}  // namespace se::rt
