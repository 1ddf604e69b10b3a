// Margolus 2x2 block update kernels (JIT-compiled with the generated rule code).
//
// One frame of the reference (shaders/compute/falling_sand.glsl:61-184) launches one
// invocation per cell, and each invocation recomputes its whole 2x2 block.  Here one
// thread computes one block once and writes all four cells, and a CTA advances a tile of
// the grid by up to KMAX frames in shared memory (temporal blocking):
//
//   load   the tile plus a halo of HX columns / HY rows from the source grid (u32 ids ->
//          u8 in shared memory; unknown ids become NULL, cells outside the world WALL);
//   step   k times: every block lying wholly inside the shared array is updated in place
//          (blocks are disjoint, so a step is race-free), then a CTA barrier;
//   store  the interior TW x TH cells (u8 -> u32) to the destination grid.
//
// A block's update reads only its own four cells, so an error at the edge of the shared
// array can spread at most one cell per step: after k <= KMAX steps every cell at least
// KMAX cells from the array edge is exact, and HX, HY >= KMAX.  Cells outside the world
// stay WALL because blocks never write them back (getCell returns WALL there on every
// frame, operations.glsl:45-57).
#pragma once

// Margolus offset of a frame (operations.glsl:25-34): frame%4 = 0,1,2,3 ->
// (0,0), (1,1), (0,1), (1,0).
__device__ __forceinline__ int se_off_x(int f) { return f & 1; }
__device__ __forceinline__ int se_off_y(int f) { return ((f + 1) >> 1) & 1; }

// hash4i's mixing of one lane (math.glsl:28-38).
__device__ __forceinline__ uint32_t se_mix(uint32_t v) {
  v ^= v >> 16;
  v *= 0x7feb352du;
  v ^= v >> 15;
  v *= 0x846ca68bu;
  v ^= v >> 16;
  return v;
}

// Cell value -> material id as getMaterialFromID sees it (unknown ids are NULL).
__device__ __forceinline__ uint32_t se_norm(uint32_t v) { return v < (uint32_t)SE_NMAT ? v : SE_NULL; }

// simulate() for the block with top-left cell (gx, gy) (falling_sand.glsl:72-114).
// The caller has already skipped all-EMPTY blocks (:77-79).
// rand.x < 0.5 <=> RN(float(h0)) < 2^31 <=> h0 < 2^31 - 64 (2^31 - 64 rounds to 2^31).
__device__ __forceinline__ void se_rules_hashed(uint32_t& a, uint32_t& b, uint32_t& c, uint32_t& d, uint32_t h0,
                                                uint32_t h1, uint32_t h2, uint32_t h3, int gx, int gy, int f,
                                                int W, int H) {
  const bool mirror = h0 < 0x7fffffc0u;
  if (mirror) {
    se_swap(a, b);
    se_swap(c, d);
  }
  se_gen::apply_mirrored(a, b, c, d, h0, h1, h2, h3, gx, gy, f, W, H);
  if (mirror) {
    se_swap(a, b);
    se_swap(c, d);
  }
  if (!mirror)
    se_gen::apply_right(a, b, c, d, h0, h1, h2, h3, gx, gy, f, W, H);
  else
    se_gen::apply_left(a, b, c, d, h0, h1, h2, h3, gx, gy, f, W, H);
}

// hash43(uvec3(origin, frame)) lanes (math.glsl:74-79), then the rules.
__device__ __forceinline__ void se_block(uint32_t& a, uint32_t& b, uint32_t& c, uint32_t& d, int gx, int gy,
                                         int f, int W, int H) {
  const uint32_t x = (uint32_t)gx * 461u + (uint32_t)gy * 2131u + (uint32_t)f * 4541161u;
  const uint32_t h0 = se_mix(x * 213u), h1 = se_mix(x * 2131u), h2 = se_mix(x * 21313u),
                 h3 = se_mix(x * 213132u);
  se_rules_hashed(a, b, c, d, h0, h1, h2, h3, gx, gy, f, W, H);
}

#ifdef SE_LUT
// Fills the block transition table: entry i holds the four output ids (4 bits each) of
// the block and hash intervals that se_gen::lut_index maps to i.  Keys naming an id >=
// SE_NMAT never occur (cells are normalised on load) and keep their input.
extern "C" __global__ void __launch_bounds__(256) se_build_lut(uint16_t* __restrict__ lut) {
  se_gen::init_tables(threadIdx.x, blockDim.x);
  __syncthreads();
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < SE_LUT_ENTRIES; i += gridDim.x * blockDim.x) {
    uint32_t a, b, c, d, h0, h1, h2, h3;
    se_gen::lut_decode(i, a, b, c, d, h0, h1, h2, h3);
    if (a < SE_NMAT && b < SE_NMAT && c < SE_NMAT && d < SE_NMAT && (a | b | c | d) != 0u)
      se_rules_hashed(a, b, c, d, h0, h1, h2, h3, 0, 0, 0, 0, 0);  // the rules read no position
    lut[i] = (uint16_t)(a | (b << 4) | (c << 8) | (d << 12));
  }
}
// Tables up to this size are copied into shared memory by each CTA.
#define SE_LUT_SMEM_MAX_ENTRIES 16384u
#endif

// One block's update: the block transition table when the rule set has one, else the
// generated rules.
__device__ __forceinline__ void se_block_update(uint32_t& a, uint32_t& b, uint32_t& c, uint32_t& d, int gx, int gy,
                                                int f, int W, int H, const uint16_t* __restrict__ lut) {
#ifdef SE_LUT
  const uint32_t x = (uint32_t)gx * 461u + (uint32_t)gy * 2131u + (uint32_t)f * 4541161u;
  const uint32_t h0 = se_mix(x * 213u), h1 = se_mix(x * 2131u), h2 = se_mix(x * 21313u), h3 = se_mix(x * 213132u);
  const uint32_t idx = se_gen::lut_index(a, b, c, d, h0, h1, h2, h3);
#if SE_LUT_ENTRIES <= SE_LUT_SMEM_MAX_ENTRIES
  const uint32_t o = lut[idx];  // shared-memory copy
#else
  const uint32_t o = __ldg(lut + idx);
#endif
  a = o & 15u;
  b = (o >> 4) & 15u;
  c = (o >> 8) & 15u;
  d = o >> 12;
#else
  se_block(a, b, c, d, gx, gy, f, W, H);
#endif
}

// Writes a block back into the shared array; slots outside the world stay WALL.
__device__ __forceinline__ void se_block_store(uint8_t* p, int SW, uint32_t a, uint32_t b, uint32_t c, uint32_t d,
                                               int gx, int gy, int W, int H, bool edge) {
  if (!edge) {
    p[0] = (uint8_t)a;
    p[1] = (uint8_t)b;
    p[SW] = (uint8_t)c;
    p[SW + 1] = (uint8_t)d;
  } else {
    const bool x0 = gx >= 0 && gx < W, x1 = gx + 1 >= 0 && gx + 1 < W;
    const bool y0 = gy >= 0 && gy < H, y1 = gy + 1 >= 0 && gy + 1 < H;
    if (x0 && y0) p[0] = (uint8_t)a;
    if (x1 && y0) p[1] = (uint8_t)b;
    if (x0 && y1) p[SW] = (uint8_t)c;
    if (x1 && y1) p[SW + 1] = (uint8_t)d;
  }
}

// One step over the shared array: every block wholly inside it.  OX and ly0 are the
// parities of the first block column / row in shared-array coordinates: a block's global
// top-left cell is congruent to the frame's offset modulo 2, and the array starts at global
// (gx0, gy0).  OX is compile-time so the block index split is a constant division.
template <int SW, int SH, int OX, int NT>
__device__ __forceinline__ void se_tile_step(uint8_t* sm, int ly0, int gx0, int gy0, int f, int W, int H,
                                             bool edge, const uint16_t* __restrict__ lut) {
  constexpr int NBX = (SW - OX) / 2;
  const int nb = NBX * ((SH - ly0) / 2);
  for (int bi = threadIdx.x; bi < nb; bi += NT) {
    const int j = bi / NBX, i = bi - j * NBX;
    const int lx = OX + 2 * i, ly = ly0 + 2 * j;
    uint8_t* p = sm + ly * SW + lx;
    uint32_t a = p[0], b = p[1], c = p[SW], d = p[SW + 1];
    if ((a | b | c | d) == 0u) continue;  // all EMPTY stays EMPTY
    const int gx = gx0 + lx, gy = gy0 + ly;
    se_block_update(a, b, c, d, gx, gy, f, W, H, lut);
    se_block_store(p, SW, a, b, c, d, gx, gy, W, H, edge);
  }
}

// The same over a shared array whose size is only known at run time (whole worlds); the
// block index is split with a float reciprocal and a +-1 correction.
__device__ __forceinline__ void se_step_rt(uint8_t* sm, int SW, int SH, int ox, int ly0, int gx0, int gy0, int f,
                                           int W, int H, const uint16_t* __restrict__ lut) {
  const int nbx = (SW - ox) / 2;
  const int nb = nbx * ((SH - ly0) / 2);
  const float inv = 1.0f / (float)nbx;
  for (int bi = threadIdx.x; bi < nb; bi += blockDim.x) {
    int j = __float2int_rz((float)bi * inv);
    int i = bi - j * nbx;
    if (i >= nbx) {
      ++j;
      i -= nbx;
    } else if (i < 0) {
      --j;
      i += nbx;
    }
    const int lx = ox + 2 * i, ly = ly0 + 2 * j;
    uint8_t* p = sm + ly * SW + lx;
    uint32_t a = p[0], b = p[1], c = p[SW], d = p[SW + 1];
    if ((a | b | c | d) == 0u) continue;
    const int gx = gx0 + lx, gy = gy0 + ly;
    se_block_update(a, b, c, d, gx, gy, f, W, H, lut);
    se_block_store(p, SW, a, b, c, d, gx, gy, W, H, true);
  }
}

// Copies a small block transition table into shared memory at byte offset `off`;
// returns the table to use.
__device__ __forceinline__ const uint16_t* se_lut_to_smem(const uint16_t* __restrict__ lut, uint8_t* smem, int off,
                                                         int nt) {
#if defined(SE_LUT) && SE_LUT_ENTRIES <= SE_LUT_SMEM_MAX_ENTRIES
  uint16_t* slut = reinterpret_cast<uint16_t*>(smem + off);
  for (uint32_t i = threadIdx.x; i < SE_LUT_ENTRIES / 2u; i += nt)
    reinterpret_cast<uint32_t*>(slut)[i] = __ldg(reinterpret_cast<const uint32_t*>(lut) + i);
  return slut;
#else
  return lut;
#endif
}

// Loads rows [gy0, gy0 + SH) x columns [gx0, gx0 + SW) of a W x H grid into the u8 array
// (row stride SW, a multiple of 4; gx0 a multiple of 4): ids normalised, outside = WALL.
__device__ __forceinline__ void se_load_region(uint8_t* sm, int SW, int SH, const uint32_t* __restrict__ src, int W,
                                               int H, int gx0, int gy0, int nt) {
  const int wpr = SW / 4;
  const bool vec = (W & 3) == 0;
  const float inv = 1.0f / (float)wpr;
  for (int i = threadIdx.x; i < wpr * SH; i += nt) {
    int r = __float2int_rz((float)i * inv);
    int c = i - r * wpr;
    if (c >= wpr) {
      ++r;
      c -= wpr;
    } else if (c < 0) {
      --r;
      c += wpr;
    }
    const int gy = gy0 + r, gx = gx0 + 4 * c;
    uint32_t packed;
    if (gy < 0 || gy >= H) {
      packed = 0x02020202u;
    } else if (vec && gx >= 0 && gx + 3 < W) {
      const uint4 v = __ldg(reinterpret_cast<const uint4*>(src + (size_t)gy * W + gx));
      packed = se_norm(v.x) | (se_norm(v.y) << 8) | (se_norm(v.z) << 16) | (se_norm(v.w) << 24);
    } else {
      packed = 0;
      for (int e = 0; e < 4; ++e) {
        const int x = gx + e;
        const uint32_t id = (x >= 0 && x < W) ? se_norm(__ldg(src + (size_t)gy * W + x)) : SE_WALL;
        packed |= id << (8 * e);
      }
    }
    *reinterpret_cast<uint32_t*>(sm + r * SW + 4 * c) = packed;
  }
}

// Stores the rows [0, TH) x columns [0, TW) of the array region that starts at (hx, hy)
// to the grid at (X0, Y0), clipped to the world.
__device__ __forceinline__ void se_store_region(const uint8_t* sm, int SW, int hx, int hy, int TW, int TH,
                                                uint32_t* __restrict__ dst, int W, int H, int X0, int Y0, int nt) {
  const int owpr = (TW + 3) / 4;
  const bool vec = (W & 3) == 0;
  const float inv = 1.0f / (float)owpr;
  for (int i = threadIdx.x; i < owpr * TH; i += nt) {
    int r = __float2int_rz((float)i * inv);
    int c = i - r * owpr;
    if (c >= owpr) {
      ++r;
      c -= owpr;
    } else if (c < 0) {
      --r;
      c += owpr;
    }
    const int gy = Y0 + r, gx = X0 + 4 * c;
    if (gy >= H || gx >= W) continue;
    const uint32_t packed = *reinterpret_cast<const uint32_t*>(sm + (r + hy) * SW + hx + 4 * c);
    if (vec && gx + 3 < W) {
      const uint4 v = make_uint4(packed & 0xffu, (packed >> 8) & 0xffu, (packed >> 16) & 0xffu, packed >> 24);
      *reinterpret_cast<uint4*>(dst + (size_t)gy * W + gx) = v;
    } else {
      for (int e = 0; e < 4; ++e)
        if (gx + e < W) dst[(size_t)gy * W + gx + e] = (packed >> (8 * e)) & 0xffu;
    }
  }
}

// Advances the tile with top-left cell (X0, Y0) of a W x H world by k <= KMAX frames whose
// counters are f0, f0+1, ... (all >= 2; the host handles the frame-1 clear).
template <int TW, int TH, int KMAX, int NT>
__device__ __forceinline__ void se_tile_run(const uint32_t* __restrict__ src, uint32_t* __restrict__ dst, int W,
                                            int H, int f0, int k, const uint16_t* __restrict__ lut, int X0, int Y0) {
  constexpr int HX = ((KMAX + 3) / 4) * 4, HY = KMAX;
  constexpr int SW = TW + 2 * HX, SH = TH + 2 * HY, WPR = SW / 4;
  static_assert(TW % 4 == 0, "tile width must be a multiple of 4");
  static_assert(HX % 2 == 0 && TW % 2 == 0, "gx0 must be even");
  extern __shared__ __align__(16) uint8_t se_smem[];
  uint8_t* sm = se_smem;
  se_gen::init_tables(threadIdx.x, NT);
  lut = se_lut_to_smem(lut, se_smem, (SW * SH + 15) & ~15, NT);
  const int gx0 = X0 - HX, gy0 = Y0 - HY;
  const bool vec = (W & 3) == 0;

  for (int i = threadIdx.x; i < WPR * SH; i += NT) {
    const int r = i / WPR, c = i - r * WPR;
    const int gy = gy0 + r, gx = gx0 + 4 * c;
    uint32_t packed;
    if (gy < 0 || gy >= H) {
      packed = 0x02020202u;
    } else if (vec && gx >= 0 && gx + 3 < W) {
      const uint4 v = __ldg(reinterpret_cast<const uint4*>(src + (size_t)gy * W + gx));
      packed = se_norm(v.x) | (se_norm(v.y) << 8) | (se_norm(v.z) << 16) | (se_norm(v.w) << 24);
    } else {
      packed = 0;
      for (int e = 0; e < 4; ++e) {
        const int x = gx + e;
        const uint32_t id = (x >= 0 && x < W) ? se_norm(__ldg(src + (size_t)gy * W + x)) : SE_WALL;
        packed |= id << (8 * e);
      }
    }
    *reinterpret_cast<uint32_t*>(sm + r * SW + 4 * c) = packed;
  }
  __syncthreads();

  const bool edge = gx0 < 0 || gy0 < 0 || gx0 + SW > W || gy0 + SH > H;
  for (int s = 0; s < k; ++s) {
    const int f = f0 + s;
    const int ly0 = (se_off_y(f) + gy0) & 1;  // gy0 = Y0 - HY is odd when HY is
    if (se_off_x(f) == 0)
      se_tile_step<SW, SH, 0, NT>(sm, ly0, gx0, gy0, f, W, H, edge, lut);
    else
      se_tile_step<SW, SH, 1, NT>(sm, ly0, gx0, gy0, f, W, H, edge, lut);
    __syncthreads();
  }

  constexpr int OWPR = TW / 4;
  for (int i = threadIdx.x; i < OWPR * TH; i += NT) {
    const int r = i / OWPR, c = i - r * OWPR;
    const int gy = Y0 + r, gx = X0 + 4 * c;
    if (gy >= H || gx >= W) continue;
    const uint32_t packed = *reinterpret_cast<const uint32_t*>(sm + (r + HY) * SW + HX + 4 * c);
    if (vec && gx + 3 < W) {
      const uint4 v = make_uint4(packed & 0xffu, (packed >> 8) & 0xffu, (packed >> 16) & 0xffu, packed >> 24);
      *reinterpret_cast<uint4*>(dst + (size_t)gy * W + gx) = v;
    } else {
      for (int e = 0; e < 4; ++e)
        if (gx + e < W) dst[(size_t)gy * W + gx + e] = (packed >> (8 * e)) & 0xffu;
    }
  }
}

// Single world: the tile is (blockIdx.x, blockIdx.y).
template <int TW, int TH, int KMAX, int NT>
__device__ __forceinline__ void se_tile_impl(const uint32_t* __restrict__ src, uint32_t* __restrict__ dst, int W,
                                             int H, int f0, int k, const uint16_t* __restrict__ lut) {
  se_tile_run<TW, TH, KMAX, NT>(src, dst, W, H, f0, k, lut, blockIdx.x * TW, blockIdx.y * TH);
}

// ---- many worlds -------------------------------------------------------------------------
// A world of a batch.  `frame` is the counter before its next frame and `cur` the buffer
// holding its grid; both live on the device and advance in se_batch_finalize, so repeated
// launches of a captured graph need no host updates.
struct SeWorldDesc {
  uint32_t* buf0;
  uint32_t* buf1;
  int W, H;
  int frame;
  int cur;
  int pad0, pad1;
};
// One tile job: a tile of a world too large to stay in shared memory.
struct SeTileJob {
  int world, x0, y0, pad;
};

// Pass `pass` of a multi-pass launch: k frames for every tile job, after `frames_done`
// frames of earlier passes.  The grid to read is the world's buffer cur ^ (pass & 1).
template <int TW, int TH, int KMAX, int NT>
__device__ __forceinline__ void se_mtile_impl(const SeWorldDesc* __restrict__ worlds,
                                              const SeTileJob* __restrict__ jobs, int pass, int frames_done, int k,
                                              const uint16_t* __restrict__ lut) {
  const SeTileJob job = jobs[blockIdx.x];
  const SeWorldDesc w = worlds[job.world];
  const int in = w.cur ^ (pass & 1);
  const uint32_t* src = in ? w.buf1 : w.buf0;
  uint32_t* dst = in ? w.buf0 : w.buf1;
  se_tile_run<TW, TH, KMAX, NT>(src, dst, w.W, w.H, w.frame + 1 + frames_done, k, lut, job.x0, job.y0);
}

// One serving iteration: descs[a] is the a-th active world, with its frames for this
// iteration in pad0 (1..KMAX); prefix[a] is the first CTA of world a (prefix[n] = grid).
// Each world reads its current buffer and writes the other one.
template <int TW, int TH, int KMAX, int NT>
__device__ __forceinline__ void se_stile_impl(const SeWorldDesc* __restrict__ descs, const int* __restrict__ prefix,
                                              int nactive, const uint16_t* __restrict__ lut) {
  const int t = blockIdx.x;
  int lo = 0, hi = nactive - 1;  // last a with prefix[a] <= t
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (prefix[mid] <= t) lo = mid;
    else hi = mid - 1;
  }
  const SeWorldDesc w = descs[lo];
  const int local = t - prefix[lo];
  const int tiles_x = (w.W + TW - 1) / TW;
  const int ty = local / tiles_x, tx = local - ty * tiles_x;
  const uint32_t* src = w.cur ? w.buf1 : w.buf0;
  uint32_t* dst = w.cur ? w.buf0 : w.buf1;
  se_tile_run<TW, TH, KMAX, NT>(src, dst, w.W, w.H, w.frame + 1, w.pad0, lut, tx * TW, ty * TH);
}

// Whole-world launch: CTA b holds world ids[b] entirely in shared memory (plus a WALL
// border: 4 columns each side for aligned loads, 1 row above and below), advances it by
// `frames` frames and stores it to the buffer cur ^ out_flip.  Nothing outside the world is
// ever written back, so the border stays WALL for every frame, as getCell returns there.
extern "C" __global__ void __launch_bounds__(1024) se_resident(const SeWorldDesc* __restrict__ worlds,
                                                               const int* __restrict__ ids, int frames, int out_flip,
                                                               const uint16_t* __restrict__ lut) {
  extern __shared__ __align__(16) uint8_t se_smem[];
  const SeWorldDesc w = worlds[ids[blockIdx.x]];
  const int SW = ((w.W + 3) & ~3) + 8, SH = w.H + 2;
  const int gx0 = -4, gy0 = -1;
  se_gen::init_tables(threadIdx.x, blockDim.x);
  lut = se_lut_to_smem(lut, se_smem, (SW * SH + 15) & ~15, blockDim.x);
  const uint32_t* src = w.cur ? w.buf1 : w.buf0;
  uint32_t* dst = (w.cur ^ out_flip) ? w.buf1 : w.buf0;
  se_load_region(se_smem, SW, SH, src, w.W, w.H, gx0, gy0, blockDim.x);
  __syncthreads();
  for (int s = 0; s < frames; ++s) {
    const int f = w.frame + 1 + s;
    se_step_rt(se_smem, SW, SH, se_off_x(f), (se_off_y(f) + gy0) & 1, gx0, gy0, f, w.W, w.H, lut);
    __syncthreads();
  }
  se_store_region(se_smem, SW, 4, 1, w.W, w.H, dst, w.W, w.H, 0, 0, blockDim.x);
}

// After a launch of `frames` frames in `passes` passes: advance every world's counter and
// current buffer.
extern "C" __global__ void __launch_bounds__(256) se_batch_finalize(SeWorldDesc* __restrict__ worlds, int n,
                                                                    int frames, int passes) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) {
    worlds[i].frame += frames;
    worlds[i].cur ^= passes & 1;
  }
}

// ---- modification (edit) pass ------------------------------------------------------------
// One 32-byte SimModification record (sandengine-core/src/simulation.rs:45-56), with
// mod_matID already mapped through getMaterialFromID (unknown ids -> NULL) by the host.
struct SeMod {
  int px, py, shape, size, mat, pad0, pad1, pad2;
};

// falling_sand.glsl:143-160 for one mod and one cell.
__device__ __forceinline__ bool se_mod_hits(const SeMod& m, int x, int y) {
  const int dx = se_iabs((int)((unsigned)m.px - (unsigned)x));
  const int dy = se_iabs((int)((unsigned)m.py - (unsigned)y));
  if (m.shape == 0) {  // MODSHAPE_CIRCLE: sqrt(pow(dx,2) + pow(dy,2)) <= size in binary32
    const float fx = __int2float_rn(dx), fy = __int2float_rn(dy);
    const float dist = __fsqrt_rn(__fadd_rn(__fmul_rn(fx, fx), __fmul_rn(fy, fy)));
    return dist <= __int2float_rn(m.size);
  }
  if (m.shape == 1) return dx <= m.size && dy <= m.size;  // MODSHAPE_SQUARE
  return false;
}

// The edit pass runs after the frame's block update, on the updated grid: a cell hit by
// any mod ends with the material of the LAST mod that hits it, unless that material is
// NULL (falling_sand.glsl:134-179); other cells keep their simulated value.  Thread t
// handles one cell of mod q's bounding box (boxes[q] = x0, y0, x1, y1 inclusive, clipped
// to the world; starts[q] = first thread of mod q) and writes only if q is the last mod
// hitting it.  The mod list travels in the kernel's parameter space (14 KB).
struct SeEditParams {
  SeMod mods[256];
  int4 boxes[256];
  long long starts[257];
};

extern "C" __global__ void __launch_bounds__(256) se_edit(uint32_t* __restrict__ grid, int W, int H, int nmods,
                                                          long long total, const SeEditParams p) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= total) return;
  int lo = 0, hi = nmods - 1;  // last q with starts[q] <= t
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (p.starts[mid] <= t) lo = mid;
    else hi = mid - 1;
  }
  const int q = lo;
  const int4 bx = p.boxes[q];
  const long long w = (long long)bx.z - bx.x + 1;
  const long long off = t - p.starts[q];
  const int x = bx.x + (int)(off % w), y = bx.y + (int)(off / w);
  if (!se_mod_hits(p.mods[q], x, y)) return;
  for (int r = q + 1; r < nmods; ++r)
    if (se_mod_hits(p.mods[r], x, y)) return;
  if (p.mods[q].mat == (int)SE_NULL) return;
  grid[(size_t)y * W + x] = (uint32_t)p.mods[q].mat;
}
