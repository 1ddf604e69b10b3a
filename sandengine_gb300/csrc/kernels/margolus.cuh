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
// the block and hash intervals that se_gen::lut_index maps to i, as a | c << 4 | b << 8 |
// d << 12 (top-left, bottom-left, top-right, bottom-right: the bytes of two entries side
// by side are then the block's columns, see se_chunk_eval).  Keys naming an id >= SE_NMAT
// never occur (cells are normalised on load) and keep their input.
extern "C" __global__ void __launch_bounds__(256) se_build_lut(uint16_t* __restrict__ lut) {
  se_gen::init_tables(threadIdx.x, blockDim.x);
  __syncthreads();
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < SE_LUT_ENTRIES; i += gridDim.x * blockDim.x) {
    uint32_t a, b, c, d, h0, h1, h2, h3;
    se_gen::lut_decode(i, a, b, c, d, h0, h1, h2, h3);
    if (a < SE_NMAT && b < SE_NMAT && c < SE_NMAT && d < SE_NMAT && (a | b | c | d) != 0u)
      se_rules_hashed(a, b, c, d, h0, h1, h2, h3, 0, 0, 0, 0, 0);  // the rules read no position
    lut[i] = (uint16_t)(a | (c << 4) | (b << 8) | (d << 12));
  }
}
// The bitset of static keys follows the table at this byte offset.  Bit `key` is set when
// the table maps the block with that key to itself for every hash value.
#define SE_LUT_STATIC_OFF ((SE_LUT_ENTRIES * 2u + 15u) & ~15u)

// Fills the static-key bitset after se_build_lut, one thread per 32-bit word.  Table
// indices are key * C + hash class (se_gen::lut_index), so a key's entries are contiguous.
extern "C" __global__ void __launch_bounds__(256) se_build_static(uint16_t* __restrict__ lut) {
  constexpr uint32_t C = SE_LUT_ENTRIES / SE_LUT_KEYS, M = (1u << SE_LUT_BITS) - 1u;
  uint32_t* st = reinterpret_cast<uint32_t*>(reinterpret_cast<uint8_t*>(lut) + SE_LUT_STATIC_OFF);
  const uint32_t w = blockIdx.x * blockDim.x + threadIdx.x;
  if (w >= SE_LUT_STATIC_WORDS) return;
  uint32_t word = 0;
  for (uint32_t j = 0; j < 32u && w * 32u + j < SE_LUT_KEYS; ++j) {
    const uint32_t key = w * 32u + j;
    // se_gen::lut_key's column order, and se_build_lut's entry layout (the same order)
    const uint32_t a = key & M, c = (key >> SE_LUT_BITS) & M, b = (key >> (2 * SE_LUT_BITS)) & M,
                   d = (key >> (3 * SE_LUT_BITS)) & M;
    const uint32_t self = a | (c << 4) | (b << 8) | (d << 12);
    bool same = true;
    for (uint32_t q = 0; q < C; ++q) same = same && lut[key * C + q] == self;
    if (same) word |= 1u << j;
  }
  st[w] = word;
}

#endif

// Index checks of the CHECKED build (module compiled with SE_CHECKED): a failed check sets
// its bit in se_check_word and the access is skipped (or the index clamped) instead of
// trapping, so the host can read what went wrong and the context stays usable.  Bits: 1
// table index, 2 shared-array index, 4 chunk-list capacity, 8 chunk window, 16 global
// index, 32 edit index.  Without SE_CHECKED every check is the constant true.
#ifdef SE_CHECKED
__device__ unsigned int se_check_word;
__device__ __forceinline__ bool se_check(bool ok, unsigned int bit) {
  if (!ok) atomicOr(&se_check_word, bit);
  return ok;
}
#else
__device__ __forceinline__ constexpr bool se_check(bool, unsigned int) { return true; }
#endif

// One block's update: the block transition table when the rule set has one, else the
// generated rules.
__device__ __forceinline__ void se_block_update(uint32_t& a, uint32_t& b, uint32_t& c, uint32_t& d, int gx, int gy,
                                                int f, int W, int H, const uint16_t* __restrict__ lut) {
#ifdef SE_LUT
  const uint32_t x = (uint32_t)gx * 461u + (uint32_t)gy * 2131u + (uint32_t)f * 4541161u;
  const uint32_t h0 = se_mix(x * 213u), h1 = se_mix(x * 2131u), h2 = se_mix(x * 21313u), h3 = se_mix(x * 213132u);
  uint32_t idx = se_gen::lut_index(a, b, c, d, h0, h1, h2, h3);
  if (!se_check(idx < SE_LUT_ENTRIES, 1u)) idx = 0;
  const uint32_t o = __ldg(lut + idx);
  a = o & 15u;
  c = (o >> 4) & 15u;  // entry layout a | c << 4 | b << 8 | d << 12 (se_build_lut)
  b = (o >> 8) & 15u;
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

// Every tile runs each step in two phases over chunks of four horizontally adjacent
// blocks (8 cells x 2 rows):
//  1. The collect phase reads every chunk: in a tile inside the world two adjacent chunks
//     per lane with one 16-byte load per row (se_chunk_collect_pairs), else one chunk per
//     lane with two 8-byte loads (se_chunk_collect).  A chunk whose 16 cells are one
//     material m whose block of four m cells never changes is left as it is (with a
//     transition table: EMPTY, and in a typical rule set the solids and liquids at rest;
//     without one: EMPTY, which the shader itself leaves alone); the others are appended
//     to a list of array offsets (a warp reserves its slots with one atomicAdd).  The
//     blocks of a row past its last whole chunk are updated right there.  In a tile
//     reaching past the world, chunks wholly outside it are left alone and chunks with
//     cells outside it fill the list from its far end.
//  2. se_chunk_process updates the listed chunks, one chunk per thread: with a table
//     word-wide and with four independent lookups, else block by block with the rules;
//     then the chunks with cells outside the world, block by block, those cells kept WALL.
// Chunks are skipped whole, so the lanes that evaluate blocks do so together rather than
// waiting on one another; blocks of one step are disjoint, so the list order is free.

// Shared-memory layout after the cell array: 16 bytes of slack (chunk
// loads at odd offsets read up to 3 bytes past a row), the list counters of alternate steps
// (chunks to evaluate, then chunks with cells outside the world, which fill the list from
// its far end), one flag byte per material id < 16, then the list.
#define SE_HDR_CNT 16
#define SE_HDR_FLAGS 32
#define SE_HDR_LIST 48

// flags[m] = 1 when the block of four m cells is static: from se_build_static's bitset
// with a transition table, else EMPTY only.
__device__ __forceinline__ void se_uniform_flags(const uint16_t* __restrict__ lut, uint8_t* flags, int nt) {
#ifdef SE_LUT
  const uint32_t* st = reinterpret_cast<const uint32_t*>(reinterpret_cast<const uint8_t*>(lut) + SE_LUT_STATIC_OFF);
#endif
  for (uint32_t m = threadIdx.x; m < 16u; m += nt) {
    uint32_t bit = m == 0u;
#ifdef SE_LUT
    bit = 0;
    if (m < SE_NMAT && m < (1u << SE_LUT_BITS)) {
      const uint32_t key = se_gen::lut_key(m, m, m, m);
      bit = (__ldg(st + (key >> 5)) >> (key & 31u)) & 1u;
    }
#endif
    flags[m] = (uint8_t)bit;
  }
}
// The 16 flag bytes as a bit mask (bit m = flags[m]).
__device__ __forceinline__ uint32_t se_flags_mask(const uint8_t* flags) {
  const uint4 v = *reinterpret_cast<const uint4*>(flags);
  // (w & 0x01010101) * 0x01020408 gathers the low bit of each byte into bits 24..27
  const uint32_t m0 = ((v.x & 0x01010101u) * 0x01020408u) >> 24, m1 = ((v.y & 0x01010101u) * 0x01020408u) >> 24,
                 m2 = ((v.z & 0x01010101u) * 0x01020408u) >> 24, m3 = ((v.w & 0x01010101u) * 0x01020408u) >> 24;
  return (m0 & 15u) | ((m1 & 15u) << 4) | ((m2 & 15u) << 8) | ((m3 & 15u) << 12);
}

// True when p is a multiple of `align` bytes (a CHECKED-build check of vector accesses).
__device__ __forceinline__ bool se_aligned(const void* p, unsigned align) {
  return (reinterpret_cast<unsigned long long>(p) & (align - 1u)) == 0u;
}

// 8 consecutive cells at p.  OX = 0: p is 8-byte aligned; OX = 1: one byte past that (an
// 8-byte load from p - 1 and a 4-byte load after it).
template <int OX>
__device__ __forceinline__ void se_ld8(const uint8_t* p, uint32_t& lo, uint32_t& hi) {
  if (OX == 0) {
    if (!se_check(se_aligned(p, 8), 2u)) {
      lo = hi = 0x02020202u;
      return;
    }
    const uint2 v = *reinterpret_cast<const uint2*>(p);
    lo = v.x;
    hi = v.y;
  } else {
    if (!se_check(se_aligned(p - 1, 8), 2u)) {
      lo = hi = 0x02020202u;
      return;
    }
    const uint2 v = *reinterpret_cast<const uint2*>(p - 1);
    const uint32_t w2 = *reinterpret_cast<const uint32_t*>(p + 7);
    lo = __funnelshift_r(v.x, v.y, 8);
    hi = __funnelshift_r(v.y, w2, 8);
  }
}
template <int OX>
__device__ __forceinline__ void se_st8(uint8_t* p, uint32_t lo, uint32_t hi) {
  if (OX == 0) {
    *reinterpret_cast<uint2*>(p) = make_uint2(lo, hi);
  } else {  // byte, half-word, word, byte
    p[0] = (uint8_t)lo;
    *reinterpret_cast<uint16_t*>(p + 1) = (uint16_t)(lo >> 8);
    *reinterpret_cast<uint32_t*>(p + 3) = (lo >> 24) | (hi << 8);
    p[7] = (uint8_t)(hi >> 24);
  }
}

#ifdef SE_LUT
// Table index of a block's key with hash base x.
__device__ __forceinline__ uint32_t se_lut_key_index(uint32_t key, uint32_t x) {
  const uint32_t h0 = se_mix(x * 213u), h1 = se_mix(x * 2131u), h2 = se_mix(x * 21313u), h3 = se_mix(x * 213132u);
  return se_gen::lut_index_key(key, h0, h1, h2, h3);
}
// Table index of a block given as the 4 bytes [a, b, c, d] (ids < 16) with hash base x.
__device__ __forceinline__ uint32_t se_lut_word_index(uint32_t abcd, uint32_t x) {
  return se_lut_key_index(se_gen::lut_key(abcd & 0xffu, (abcd >> 8) & 0xffu, (abcd >> 16) & 0xffu, abcd >> 24), x);
}
__device__ __forceinline__ uint32_t se_lut_fetch(const uint16_t* __restrict__ lut, uint32_t idx) {
  if (!se_check(idx < SE_LUT_ENTRIES, 1u)) idx = 0;
  return __ldg(lut + idx);
}
#endif

// Appends `entry` for the lanes with `dyn` set; every lane of the warp calls it.  The list
// holds `cap` entries; DOWN fills it from the far end (entry i at cap - 1 - i).
template <bool DOWN = false>
__device__ __forceinline__ void se_list_push(bool dyn, uint32_t entry, uint16_t* __restrict__ list,
                                             int* __restrict__ cnt, int cap) {
  const uint32_t m = __ballot_sync(0xffffffffu, dyn);
  if (m == 0u) return;
  const int lane = threadIdx.x & 31;
  int base = 0;
  if (lane == 0) base = atomicAdd(cnt, __popc(m));
  base = __shfl_sync(0xffffffffu, base, 0);
  const int at = base + __popc(m & ((1u << lane) - 1u));
  if (dyn && se_check(at < cap, 4u)) list[DOWN ? cap - 1 - at : at] = (uint16_t)entry;
}

// The blocks of rows ly0 + 2 j, j in [0, nby), past the last whole chunk of each row,
// updated right away.
template <int SW, int SH, int OX, int NT, bool EDGE>
__device__ __forceinline__ void se_rem_blocks(uint8_t* sm, int ly0, int nby, int gx0, int gy0, int f, int W, int H,
                                              const uint16_t* __restrict__ lut) {
  constexpr int NBX = (SW - OX) / 2, NCX = NBX / 4, REM = NBX - 4 * NCX;
  if (REM) {
    for (int t = threadIdx.x; t < nby * REM; t += NT) {
      const int j = t / REM, r = t - j * REM;
      const int lx = OX + 2 * (4 * NCX + r), ly = ly0 + 2 * j;
      if (!se_check((ly + 1) * SW + lx + 1 < SW * SH, 2u)) continue;
      uint8_t* p = sm + ly * SW + lx;
      uint32_t a = p[0], b = p[1], c = p[SW], d = p[SW + 1];
      if ((a | b | c | d) == 0u) continue;
      const int gx = gx0 + lx, gy = gy0 + ly;
      se_block_update(a, b, c, d, gx, gy, f, W, H, lut);
      se_block_store(p, SW, a, b, c, d, gx, gy, W, H, EDGE);
    }
  }
}

// A chunk (rows a0 a1 / b0 b1) that is 16 cells of one material whose block is static.
__device__ __forceinline__ bool se_uniform_static(uint32_t a0, uint32_t a1, uint32_t b0, uint32_t b1,
                                                  uint32_t umask) {
  // all 16 bytes equal: the four words equal, and a0 equal to its byte 0 broadcast
  const uint32_t diff = (a0 ^ a1) | (a0 ^ b0) | (a0 ^ b1) | (a0 ^ __byte_perm(a0, 0u, 0x0000));
  // for a uniform chunk a0 & 31 is its material (< 16; the wrapping funnel shift reads
  // only those bits), and bit m of umask (< 2^16) its static flag
  return diff == 0u && (__funnelshift_r(umask, 0u, a0) & 1u) != 0u;
}

// 16 consecutive cells at p (two chunks' rows).  OX = 0: p is 8-byte aligned (16-byte when
// SW is a multiple of 16); OX = 1: one byte past that.
template <int SW, int OX>
__device__ __forceinline__ void se_ld16(const uint8_t* p, uint32_t& w0, uint32_t& w1, uint32_t& w2, uint32_t& w3) {
  if (SW % 16 == 0 && !se_check(se_aligned(p - OX, 16), 2u)) {
    w0 = w1 = w2 = w3 = 0x02020202u;
    return;
  }
  if (OX == 0 && SW % 16 == 0) {
    const uint4 v = *reinterpret_cast<const uint4*>(p);
    w0 = v.x;
    w1 = v.y;
    w2 = v.z;
    w3 = v.w;
  } else if (OX == 0) {
    se_ld8<0>(p, w0, w1);
    se_ld8<0>(p + 8, w2, w3);
  } else if (SW % 16 == 0) {  // p - 1 is 16-byte aligned: one 16-byte load and the word after it
    const uint4 v = *reinterpret_cast<const uint4*>(p - 1);
    const uint32_t u4 = *reinterpret_cast<const uint32_t*>(p + 15);
    w0 = __funnelshift_r(v.x, v.y, 8);
    w1 = __funnelshift_r(v.y, v.z, 8);
    w2 = __funnelshift_r(v.z, v.w, 8);
    w3 = __funnelshift_r(v.w, u4, 8);
  } else {
    const uint32_t* q = reinterpret_cast<const uint32_t*>(p - 1);
    const uint32_t u0 = q[0], u1 = q[1], u2 = q[2], u3 = q[3], u4 = q[4];
    w0 = __funnelshift_r(u0, u1, 8);
    w1 = __funnelshift_r(u1, u2, 8);
    w2 = __funnelshift_r(u2, u3, 8);
    w3 = __funnelshift_r(u3, u4, 8);
  }
}

// Appends `off` for lanes with d0 and `off + 8` for lanes with d1; one atomicAdd per warp.
__device__ __forceinline__ void se_list_push2(bool d0, bool d1, uint32_t off, uint16_t* __restrict__ list,
                                              int* __restrict__ cnt, int cap) {
  const uint32_t m0 = __ballot_sync(0xffffffffu, d0), m1 = __ballot_sync(0xffffffffu, d1);
  if ((m0 | m1) == 0u) return;
  const int lane = threadIdx.x & 31;
  const uint32_t lt = (1u << lane) - 1u;
  int base = 0;
  if (lane == 0) base = atomicAdd(cnt, __popc(m0) + __popc(m1));
  base = __shfl_sync(0xffffffffu, base, 0);
  int at = base + __popc(m0 & lt) + __popc(m1 & lt);
  if (d0) {
    if (se_check(at < cap, 4u)) list[at] = (uint16_t)off;
    ++at;
  }
  if (d1 && se_check(at < cap, 4u)) list[at] = (uint16_t)(off + 8u);
}

// The collect phase of a tile wholly inside the world, two horizontally adjacent chunks per
// lane (one pair of loads per row, one list reservation per warp for both): block rows
// ly0 + 2 j, j in [jlo, jlo + nby).
template <int SW, int SH, int OX, int NT>
__device__ __forceinline__ void se_chunk_collect_pairs(uint8_t* sm, int ly0, int jlo, int nby, int gx0, int gy0,
                                                       int f, int W, int H, const uint16_t* __restrict__ lut,
                                                       uint32_t umask, uint16_t* __restrict__ list,
                                                       int* __restrict__ cnt) {
  static_assert(NT % 32 == 0 || NT == 1, "whole warps");
  static_assert(SW % 8 == 0 && SW * SH <= 65536, "8-byte rows, 16-bit offsets");
  constexpr int NBX = (SW - OX) / 2, NCX = NBX / 4, NPX = (NCX + 1) / 2;
  constexpr int CAP = (SW / 8) * (SH / 2);
  ly0 += 2 * jlo;
  const int np = NPX * nby;
  for (int base = threadIdx.x & ~31; base < np; base += NT) {  // warp-uniform trip count
    const int pi = base + (threadIdx.x & 31);
    bool d0 = false, d1 = false;
    int off = 0;
    if (pi < np) {
      const int j = pi / NPX, qp = pi - j * NPX;
      off = (ly0 + 2 * j) * SW + OX + 16 * qp;
      // a pair at an odd offset reads up to 19 bytes from off: at most 3 past the row (the
      // next row, or the 16-byte slack after the array)
      if (!se_check(off >= 0 && off + SW + 19 <= ((SW * SH + 15) & ~15) + 16, 8u)) off = 0;
      uint32_t a0, a1, a2, a3, b0, b1, b2, b3;
      se_ld16<SW, OX>(sm + off, a0, a1, a2, a3);
      se_ld16<SW, OX>(sm + off + SW, b0, b1, b2, b3);
      d0 = !se_uniform_static(a0, a1, b0, b1, umask);
      // an odd chunk count leaves the last pair with one chunk
      d1 = (NCX % 2 == 0 || 2 * qp + 1 < NCX) && !se_uniform_static(a2, a3, b2, b3, umask);
    }
    se_list_push2(d0, d1, (uint32_t)off, list, cnt, CAP);
  }
  se_rem_blocks<SW, SH, OX, NT, false>(sm, ly0, nby, gx0, gy0, f, W, H, lut);
}

// Block rows ly0 + 2 j, j in [jlo, jlo + nby), are collected (the rows a step still needs).
// In an edge tile (part of the array outside the world) chunks wholly outside the world are
// left alone, and chunks partly outside go to the far end of the list (counted in bcnt),
// to be updated block by block with the slots outside the world kept WALL.
template <int SW, int SH, int OX, int NT, bool EDGE>
__device__ __forceinline__ void se_chunk_collect(uint8_t* sm, int ly0, int jlo, int nby, int gx0, int gy0, int f,
                                                 int W, int H, const uint16_t* __restrict__ lut, uint32_t umask,
                                                 uint16_t* __restrict__ list, int* __restrict__ cnt,
                                                 int* __restrict__ bcnt) {
  static_assert(NT % 32 == 0 || NT == 1, "whole warps");
  static_assert(SW % 8 == 0 && SW * SH <= 65536, "8-byte rows, 16-bit offsets");
  constexpr int NBX = (SW - OX) / 2, NCX = NBX / 4, REM = NBX - 4 * NCX;
  constexpr int CAP = (SW / 8) * (SH / 2);  // list capacity (tile_smem_bytes sizes it)
  ly0 += 2 * jlo;
  const int nc = NCX * nby;
  for (int base = threadIdx.x & ~31; base < nc; base += NT) {  // warp-uniform trip count
    const int ci = base + (threadIdx.x & 31);
    bool dyn = false, border = false;
    int off = 0;
    if (ci < nc) {
      const int j = ci / NCX, q = ci - j * NCX;
      off = (ly0 + 2 * j) * SW + OX + 8 * q;
      // chunk loads at odd offsets read up to 3 bytes past the chunk: the 16-byte slack
      if (!se_check(off >= 0 && off + SW + 11 <= ((SW * SH + 15) & ~15) + 16, 8u)) off = 0;
      bool inside = true;
      if (EDGE) {
        const int gx = gx0 + OX + 8 * q, gy = gy0 + ly0 + 2 * j;
        inside = gx >= 0 && gx + 7 < W && gy >= 0 && gy + 1 < H;
        border = !inside && gx + 7 >= 0 && gx < W && gy + 1 >= 0 && gy < H;
      }
      if (inside) {
        uint32_t a0, a1, b0, b1;
        se_ld8<OX>(sm + off, a0, a1);
        se_ld8<OX>(sm + off + SW, b0, b1);
        const uint32_t m = a0 & 0xffu;
        const bool uniform = ((a0 ^ a1) | (a0 ^ b0) | (a0 ^ b1)) == 0u && a0 == m * 0x01010101u;
        dyn = !(uniform && m < 16u && ((umask >> m) & 1u));
      }
    }
    se_list_push(dyn, (uint32_t)off, list, cnt, CAP);
    if (EDGE) se_list_push<true>(border, (uint32_t)off, list, bcnt, CAP);
  }
  se_rem_blocks<SW, SH, OX, NT, EDGE>(sm, ly0, nby, gx0, gy0, f, W, H, lut);
}

#ifdef SE_LUT
// Updates the chunk (4 blocks, 8 x 2 cells) at p, row stride SW, whose first block's hash
// base is x, with word-wide shared-memory access.
template <int OX>
__device__ __forceinline__ void se_chunk_eval(uint8_t* p, int SW, uint32_t x, const uint16_t* __restrict__ lut) {
  uint32_t a0, a1, b0, b1;
  se_ld8<OX>(p, a0, a1);
  se_ld8<OX>(p + SW, b0, b1);
  // The four blocks' keys; block origins are 2 cells apart (x + 922 each).  No branch on
  // all-EMPTY blocks (the table maps them to themselves), so the four lookups are in flight
  // together.
#if SE_LUT_BITS == 4
  // A row word holds 4 cells (< 16 each), so top + (bottom << 4) holds in byte j the column
  // top_j | bottom_j << 4, and its two halves are the two blocks' keys in se_gen::lut_key's
  // column order (key0 | key1 << 16); the nibbles do not overlap, so the sum is an OR.
  const uint32_t k01 = b0 * 16u + a0;
  const uint32_t k23 = b1 * 16u + a1;
  const uint32_t i0 = se_lut_key_index(k01 & 0xffffu, x), i1 = se_lut_key_index(k01 >> 16, x + 922u);
  const uint32_t i2 = se_lut_key_index(k23 & 0xffffu, x + 1844u), i3 = se_lut_key_index(k23 >> 16, x + 2766u);
#else
  const uint32_t i0 = se_lut_word_index(__byte_perm(a0, b0, 0x5410), x);
  const uint32_t i1 = se_lut_word_index(__byte_perm(a0, b0, 0x7632), x + 922u);
  const uint32_t i2 = se_lut_word_index(__byte_perm(a1, b1, 0x5410), x + 1844u);
  const uint32_t i3 = se_lut_word_index(__byte_perm(a1, b1, 0x7632), x + 2766u);
#endif
  const uint32_t o0 = se_lut_fetch(lut, i0), o1 = se_lut_fetch(lut, i1), o2 = se_lut_fetch(lut, i2),
                 o3 = se_lut_fetch(lut, i3);
  // Entries are a | c << 4 | b << 8 | d << 12: a block's bytes are its columns [a|c, b|d].
  // Two blocks' entries side by side are [a|c, b|d, a'|c', b'|d']; their low nibbles are
  // the top row [a, b, a', b'] and their high nibbles the bottom row [c, d, c', d'].
  const uint32_t P01 = __byte_perm(o0, o1, 0x5410), P23 = __byte_perm(o2, o3, 0x5410);
  se_st8<OX>(p, P01 & 0x0f0f0f0fu, P23 & 0x0f0f0f0fu);
  se_st8<OX>(p + SW, (P01 >> 4) & 0x0f0f0f0fu, (P23 >> 4) & 0x0f0f0f0fu);
}
#endif

// The chunks with cells outside the world (edge tiles), from the far end of the chunk list,
// block by block with those cells kept WALL.
template <int SW, int SH, int NT>
__device__ __forceinline__ void se_border_process(uint8_t* sm, const uint16_t* __restrict__ list, int nb, int gx0,
                                                  int gy0, int f, int W, int H, const uint16_t* __restrict__ lut) {
  constexpr int CAP = (SW / 8) * (SH / 2);
  for (int i = threadIdx.x; i < nb; i += NT) {
    if (!se_check(i < CAP, 4u)) break;
    const int off = list[CAP - 1 - i];
    if (!se_check(off + SW + 7 < SW * SH, 8u)) continue;
    const int ly = off / SW, lx = off - ly * SW;
    for (int kb = 0; kb < 4; ++kb) {
      uint8_t* p = sm + off + 2 * kb;
      uint32_t a = p[0], b = p[1], c = p[SW], d = p[SW + 1];
      if ((a | b | c | d) == 0u) continue;  // all EMPTY stays EMPTY
      const int gx = gx0 + lx + 2 * kb, gy = gy0 + ly;
      se_block_update(a, b, c, d, gx, gy, f, W, H, lut);
      se_block_store(p, SW, a, b, c, d, gx, gy, W, H, true);
    }
  }
}

template <int SW, int SH, int OX, int NT>
__device__ __forceinline__ void se_chunk_process(uint8_t* sm, const uint16_t* __restrict__ list, int n, int gx0,
                                                 int gy0, int f, int W, int H, const uint16_t* __restrict__ lut) {
  const uint32_t xf = (uint32_t)f * 4541161u;
  // the hash base (gx0 + lx) 461 + (gy0 + ly) 2131 + f 4541161 of the chunk at offset
  // off = ly SW + lx is xb + 461 off + (2131 - 461 SW) ly (mod 2^32)
  const uint32_t xb = (uint32_t)gx0 * 461u + (uint32_t)gy0 * 2131u + xf;
  constexpr uint32_t XROW = 2131u - 461u * (uint32_t)SW;
  for (int i = threadIdx.x; i < n; i += NT) {
    if (!se_check(i < (SW / 8) * (SH / 2), 4u)) break;
    const int off = list[i];
    if (!se_check(off + SW + 11 <= ((SW * SH + 15) & ~15) + 16, 8u)) continue;
    const int ly = off / SW, lx = off - ly * SW;
#ifdef SE_LUT
    (void)lx, (void)W, (void)H;
    const uint32_t x = xb + (uint32_t)off * 461u + (uint32_t)ly * XROW;
    se_chunk_eval<OX>(sm + off, SW, x, lut);
#else
    (void)xb;
    (void)xf;
    for (int kb = 0; kb < 4; ++kb) {  // the generated rules, block by block
      uint8_t* p = sm + off + 2 * kb;
      uint32_t a = p[0], b = p[1], c = p[SW], d = p[SW + 1];
      if ((a | b | c | d) == 0u) continue;
      se_block(a, b, c, d, gx0 + lx + 2 * kb, gy0 + ly, f, W, H);
      p[0] = (uint8_t)a;
      p[1] = (uint8_t)b;
      p[SW] = (uint8_t)c;
      p[SW + 1] = (uint8_t)d;
    }
#endif
  }
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
    if (se_check(r >= 0 && r < SH && c >= 0 && c < wpr, 2u))
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
    if (!se_check(gy >= 0 && gx >= 0 && r >= 0 && c >= 0, 16u)) continue;
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

// ---- modification (edit) records ------------------------------------------------------
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

// The edit pass inside a tile launch, after the block update of its first frame: every
// array cell of the world (and of the buffer rows [ya, yb)) hit by a mod of `p` takes the
// material of the last mod hitting it unless that material is NULL (the rule of se_edit
// below, falling_sand.glsl:134-179).  Block partners were updated from the pre-edit values,
// as every invocation of the reference's frame reads the input texture.  Mods are visited
// in order; a cell is written only by the last mod that hits it, so no two threads write
// one cell and the mods need no barrier between them.
__device__ __forceinline__ void se_tile_edits(uint8_t* sm, int SW, int SH, int gx0, int gy0, int W, int H, int ya,
                                              int yb, const SeEditParams* __restrict__ p, int n, int nt) {
  const int rx0 = gx0 > 0 ? gx0 : 0, rx1 = (gx0 + SW < W ? gx0 + SW : W) - 1;
  const int ylo = ya > 0 ? ya : 0, yhi = yb < H ? yb : H;
  const int ry0 = gy0 > ylo ? gy0 : ylo, ry1 = (gy0 + SH < yhi ? gy0 + SH : yhi) - 1;
  for (int q = 0; q < n; ++q) {
    const int4 b = p->boxes[q];
    if (p->mods[q].mat == (int)SE_NULL) continue;  // its cells keep the simulated value
    const int x0 = b.x > rx0 ? b.x : rx0, x1 = b.z < rx1 ? b.z : rx1;
    const int y0 = b.y > ry0 ? b.y : ry0, y1 = b.w < ry1 ? b.w : ry1;
    if (x0 > x1 || y0 > y1) continue;
    const SeMod m = p->mods[q];
    const int w = x1 - x0 + 1, cnt = w * (y1 - y0 + 1);
    for (int t = threadIdx.x; t < cnt; t += nt) {
      const int y = y0 + t / w, x = x0 + t % w;
      if (!se_mod_hits(m, x, y)) continue;
      bool later = false;
      for (int r = q + 1; r < n && !later; ++r) {
        const int4 rb = p->boxes[r];
        later = x >= rb.x && x <= rb.z && y >= rb.y && y <= rb.w && se_mod_hits(p->mods[r], x, y);
      }
      const int i = (y - gy0) * SW + (x - gx0);
      if (!later && se_check(i >= 0 && i < SW * SH, 32u)) sm[i] = (uint8_t)m.mat;
    }
  }
}

// Advances the tile with top-left cell (X0, Y0) of a W x H world by k <= KMAX frames whose
// counters are f0, f0+1, ... (all >= 2; the host handles the frame-1 clear).
// src and dst hold the world rows [ya, yb) (row gy at (gy - ya) * W): the whole world, or a
// band of it with its halo.  Rows outside the buffer read as WALL, like those outside the
// world; inside the world that is wrong, but a wrong cell can only spread one row per
// frame, so after n frames every row at least n rows inside the buffer is exact.  Hashes,
// block parities and the world border use world coordinates.
template <int TW, int TH, int KMAX, int NT>
__device__ __forceinline__ void se_tile_run(const uint32_t* __restrict__ src, uint32_t* __restrict__ dst, int W,
                                            int H, int f0, int k, const uint16_t* __restrict__ lut, int X0, int Y0,
                                            int ya, int yb, const SeEditParams* __restrict__ edits = nullptr,
                                            int nedits = 0) {
  constexpr int HX = ((KMAX + 3) / 4) * 4, HY = KMAX;
  constexpr int SW = TW + 2 * HX, SH = TH + 2 * HY, WPR = SW / 4;
  static_assert(TW % 4 == 0, "tile width must be a multiple of 4");
  static_assert(HX % 2 == 0 && TW % 2 == 0, "gx0 must be even");
  extern __shared__ __align__(16) uint8_t se_smem[];
  uint8_t* sm = se_smem;
  se_gen::init_tables(threadIdx.x, NT);
  constexpr int HDR = (SW * SH + 15) & ~15;
  int* cnt = reinterpret_cast<int*>(se_smem + HDR + SE_HDR_CNT);
  uint8_t* flags = se_smem + HDR + SE_HDR_FLAGS;
  uint16_t* list = reinterpret_cast<uint16_t*>(se_smem + HDR + SE_HDR_LIST);
  for (int i = threadIdx.x; i < 4; i += NT) cnt[i] = 0;  // [s & 1]: to evaluate, [2 + (s & 1)]: border
  se_uniform_flags(lut, flags, NT);
  const int gx0 = X0 - HX, gy0 = Y0 - HY;
  const bool vec = (W & 3) == 0;

  if (vec && gx0 >= 0 && gy0 >= ya && gx0 + SW <= W && gy0 + SH <= yb) {
    // The region lies inside the world (and the buffer): four 16-byte loads per thread are
    // issued before any is converted, so they are in flight together.
    constexpr int NL = WPR * SH;
    const uint32_t* base = src + (size_t)(gy0 - ya) * W + gx0;
    for (int i0 = threadIdx.x; i0 < NL; i0 += 4 * NT) {
      uint4 v[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const int i = i0 + u * NT;
        if (i < NL) {
          const int r = i / WPR, c = i - r * WPR;
          if (!se_check(gy0 - ya + r < yb - ya && gx0 + 4 * c + 3 < W, 16u)) {
            v[u] = make_uint4(SE_WALL, SE_WALL, SE_WALL, SE_WALL);
            continue;
          }
          v[u] = __ldg(reinterpret_cast<const uint4*>(base + (size_t)r * W + 4 * c));
        }
      }
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const int i = i0 + u * NT;
        if (i < NL) {  // word r * WPR + c of the array is word i (rows are WPR = SW / 4 words)
          // one unsigned maximum tells whether all four ids name materials (after the first
          // launch they always do); only otherwise is each id mapped (unknown -> NULL)
          const uint32_t mx = max(max(v[u].x, v[u].y), max(v[u].z, v[u].w));
          uint32_t packed = __byte_perm(__byte_perm(v[u].x, v[u].y, 0x0040), __byte_perm(v[u].z, v[u].w, 0x0040),
                                        0x5410);
          if (mx >= (uint32_t)SE_NMAT)
            packed = __byte_perm(__byte_perm(se_norm(v[u].x), se_norm(v[u].y), 0x0040),
                                 __byte_perm(se_norm(v[u].z), se_norm(v[u].w), 0x0040), 0x5410);
          reinterpret_cast<uint32_t*>(sm)[i] = packed;
        }
      }
    }
  } else {
    for (int i = threadIdx.x; i < WPR * SH; i += NT) {
      const int r = i / WPR, c = i - r * WPR;
      const int gy = gy0 + r, gx = gx0 + 4 * c;
      uint32_t packed;
      if (gy < ya || gy >= yb) {
        packed = 0x02020202u;
      } else if (vec && gx >= 0 && gx + 3 < W) {
        const uint4 v = __ldg(reinterpret_cast<const uint4*>(src + (size_t)(gy - ya) * W + gx));
        packed = se_norm(v.x) | (se_norm(v.y) << 8) | (se_norm(v.z) << 16) | (se_norm(v.w) << 24);
      } else {
        packed = 0;
        for (int e = 0; e < 4; ++e) {
          const int x = gx + e;
          const uint32_t id = (x >= 0 && x < W) ? se_norm(__ldg(src + (size_t)(gy - ya) * W + x)) : SE_WALL;
          packed |= id << (8 * e);
        }
      }
      *reinterpret_cast<uint32_t*>(sm + r * SW + 4 * c) = packed;
    }
  }
  __syncthreads();

  const bool edge = gx0 < 0 || gy0 < 0 || gx0 + SW > W || gy0 + SH > H;
  const uint32_t umask = se_flags_mask(flags);
  for (int s = 0; s < k; ++s) {
    const int f = f0 + s;
    const int ly0 = (se_off_y(f) + gy0) & 1;  // gy0 = Y0 - HY is odd when HY is
    // Rows the stored interior [HY, HY + TH) still depends on after this step: within
    // k - 1 - s of it.  A block reads only its own cells, so the blocks meeting those
    // rows (origin rows HY - k + s .. HY + TH + k - 2 - s) are all that step s must
    // update; the others hold values that no stored cell reads.
    const int lymin = HY - k + s, lymax = HY + TH + k - 2 - s;
    const int jlo = lymin > ly0 ? (lymin - ly0 + 1) >> 1 : 0;
    const int jend = (SH - ly0) / 2 - 1, jneed = (lymax - ly0) >> 1;
    const int jhi = jneed < jend ? jneed : jend;
    int* c = cnt + (s & 1);
    int* bc = cnt + 2 + (s & 1);
    const int nby = jhi - jlo + 1;
    if (edge) {
      if (se_off_x(f) == 0)
        se_chunk_collect<SW, SH, 0, NT, true>(sm, ly0, jlo, nby, gx0, gy0, f, W, H, lut, umask, list, c, bc);
      else
        se_chunk_collect<SW, SH, 1, NT, true>(sm, ly0, jlo, nby, gx0, gy0, f, W, H, lut, umask, list, c, bc);
    } else {
      if (se_off_x(f) == 0)
        se_chunk_collect_pairs<SW, SH, 0, NT>(sm, ly0, jlo, nby, gx0, gy0, f, W, H, lut, umask, list, c);
      else
        se_chunk_collect_pairs<SW, SH, 1, NT>(sm, ly0, jlo, nby, gx0, gy0, f, W, H, lut, umask, list, c);
    }
    __syncthreads();
    const int n = *c, nb = *bc;
    if (threadIdx.x == 0) cnt[(s + 1) & 1] = cnt[2 + ((s + 1) & 1)] = 0;  // last read in step s - 1
    if (se_off_x(f) == 0)
      se_chunk_process<SW, SH, 0, NT>(sm, list, n, gx0, gy0, f, W, H, lut);
    else
      se_chunk_process<SW, SH, 1, NT>(sm, list, n, gx0, gy0, f, W, H, lut);
    se_border_process<SW, SH, NT>(sm, list, nb, gx0, gy0, f, W, H, lut);
    __syncthreads();
    if (s == 0 && nedits > 0) {  // the first frame's edits (the host passes them only then)
      se_tile_edits(sm, SW, SH, gx0, gy0, W, H, ya, yb, edits, nedits, NT);
      __syncthreads();
    }
  }

  constexpr int OWPR = TW / 4;
  if (vec && X0 + TW <= W && Y0 + TH <= yb && Y0 >= ya) {
    // the interior lies inside the world and the buffer: no bounds to check
    uint32_t* out0 = dst + (size_t)(Y0 - ya) * W + X0;
    for (int i = threadIdx.x; i < OWPR * TH; i += NT) {
      const int r = i / OWPR, c = i - r * OWPR;
      const uint32_t packed = *reinterpret_cast<const uint32_t*>(sm + (r + HY) * SW + HX + 4 * c);
      *reinterpret_cast<uint4*>(out0 + (size_t)r * W + 4 * c) =
          make_uint4(__byte_perm(packed, 0u, 0x4440), __byte_perm(packed, 0u, 0x4441),
                     __byte_perm(packed, 0u, 0x4442), __byte_perm(packed, 0u, 0x4443));
    }
    return;
  }
  for (int i = threadIdx.x; i < OWPR * TH; i += NT) {
    const int r = i / OWPR, c = i - r * OWPR;
    const int gy = Y0 + r, gx = X0 + 4 * c;
    if (gy >= yb || gx >= W) continue;
    if (!se_check(gy >= ya, 16u)) continue;
    const uint32_t packed = *reinterpret_cast<const uint32_t*>(sm + (r + HY) * SW + HX + 4 * c);
    uint32_t* out = dst + (size_t)(gy - ya) * W;
    if (vec && gx + 3 < W) {
      const uint4 v = make_uint4(packed & 0xffu, (packed >> 8) & 0xffu, (packed >> 16) & 0xffu, packed >> 24);
      *reinterpret_cast<uint4*>(out + gx) = v;
    } else {
      for (int e = 0; e < 4; ++e)
        if (gx + e < W) out[gx + e] = (packed >> (8 * e)) & 0xffu;
    }
  }
}

// One world, or the band of world rows [ya, yb) held by src and dst: the tile is
// (blockIdx.x, blockIdx.y) counted from row ya.
// With `edits`, the first frame's edit pass runs inside the launch (se_tile_edits).
template <int TW, int TH, int KMAX, int NT>
__device__ __forceinline__ void se_tile_impl(const uint32_t* __restrict__ src, uint32_t* __restrict__ dst, int W,
                                             int H, int f0, int k, const uint16_t* __restrict__ lut, int ya, int yb,
                                             const SeEditParams* __restrict__ edits = nullptr, int nedits = 0) {
  if (ya < 0 || yb > H || ya >= yb || k < 1 || k > KMAX) return;  // the host validates these too
  if (nedits < 0 || nedits > 256) return;
  se_tile_run<TW, TH, KMAX, NT>(src, dst, W, H, f0, k, lut, blockIdx.x * TW, ya + blockIdx.y * TH, ya, yb, edits,
                                nedits);
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
  se_tile_run<TW, TH, KMAX, NT>(src, dst, w.W, w.H, w.frame + 1 + frames_done, k, lut, job.x0, job.y0, 0, w.H);
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
  se_tile_run<TW, TH, KMAX, NT>(src, dst, w.W, w.H, w.frame + 1, w.pad0, lut, tx * TW, ty * TH, 0, w.H);
}

// A chunk of a whole world in shared memory at array offset `off` (row ly, column lx; the
// array's cell (0, 0) is world cell (gx0, gy0)), all of its cells inside the world.
template <int OX>
__device__ __forceinline__ void se_rt_chunk(uint8_t* sm, int SW, int off, int ly, int lx, int gx0, int gy0, int f,
                                            int W, int H, const uint16_t* __restrict__ lut) {
#ifdef SE_LUT
  (void)W, (void)H;
  const uint32_t x = (uint32_t)(gx0 + lx) * 461u + (uint32_t)(gy0 + ly) * 2131u + (uint32_t)f * 4541161u;
  se_chunk_eval<OX>(sm + off, SW, x, lut);
#else
  (void)lut;
  for (int kb = 0; kb < 4; ++kb) {  // the generated rules, block by block
    uint8_t* p = sm + off + 2 * kb;
    uint32_t a = p[0], b = p[1], c = p[SW], d = p[SW + 1];
    if ((a | b | c | d) == 0u) continue;
    se_block(a, b, c, d, gx0 + lx + 2 * kb, gy0 + ly, f, W, H);
    p[0] = (uint8_t)a;
    p[1] = (uint8_t)b;
    p[SW] = (uint8_t)c;
    p[SW + 1] = (uint8_t)d;
  }
#endif
}

// j = i / n and i - j n for 0 <= i < 2^22 (a float reciprocal and a +-1 correction).
__device__ __forceinline__ void se_divmod_rt(int i, int n, float inv, int& j, int& r) {
  j = __float2int_rz((float)i * inv);
  r = i - j * n;
  if (r >= n) {
    ++j;
    r -= n;
  } else if (r < 0) {
    --j;
    r += n;
  }
}

// One frame of a whole world held in shared memory (se_resident's array: row stride SW, a
// multiple of 8; rows ly0 + 2 j are the block rows), as the tile kernel's edge tiles run
// a step: the collect phase lists the chunks of world cells that are not uniform static
// (entries are array offset / 8, which fits 16 bits for any array that fits in shared
// memory) and puts the chunks with cells outside the world at the far end of the list;
// after a barrier the listed chunks are evaluated word-wide and the border chunks block by
// block, their cells outside the world kept WALL; the blocks of a row past its last whole
// chunk are updated in the collect phase.  cnt[0] / cnt[1] count the two ends of the list;
// the caller zeroes them before the step, and `next` (the other step's pair) is zeroed here
// once the counts are read.
template <int OX>
__device__ __forceinline__ void se_rt_step(uint8_t* sm, int SW, int SH, int ly0, int gx0, int gy0, int f, int W,
                                           int H, const uint16_t* __restrict__ lut, uint32_t umask,
                                           uint16_t* __restrict__ list, int cap, int* cnt, int* next) {
  const int nt = blockDim.x;
  const int nbx = (SW - OX) / 2, ncx = nbx / 4, rem = nbx - 4 * ncx, nby = (SH - ly0) / 2;
  const int nc = ncx * nby, sw8 = SW >> 3;
  const float inv_ncx = 1.0f / (float)ncx, inv_sw8 = 1.0f / (float)sw8;
  for (int base = threadIdx.x & ~31; base < nc; base += nt) {  // warp-uniform trip count
    const int ci = base + (threadIdx.x & 31);
    bool dyn = false, border = false;
    uint32_t e = 0;
    if (ci < nc) {
      int j, q;
      se_divmod_rt(ci, ncx, inv_ncx, j, q);
      const int ly = ly0 + 2 * j, lx = OX + 8 * q;
      const int off = ly * SW + lx;
      e = (uint32_t)(off >> 3);
      const int gx = gx0 + lx, gy = gy0 + ly;
      const bool inside = gx >= 0 && gx + 7 < W && gy >= 0 && gy + 1 < H;
      border = !inside && gx + 7 >= 0 && gx < W && gy + 1 >= 0 && gy < H;
      if (inside && se_check(off + SW + 11 <= ((SW * SH + 15) & ~15) + 16, 8u)) {
        uint32_t a0, a1, b0, b1;
        se_ld8<OX>(sm + off, a0, a1);
        se_ld8<OX>(sm + off + SW, b0, b1);
        dyn = !se_uniform_static(a0, a1, b0, b1, umask);
      }
    }
    se_list_push(dyn, e, list, cnt, cap);
    se_list_push<true>(border, e, list, cnt + 1, cap);
  }
  for (int t = threadIdx.x; t < nby * rem; t += nt) {  // blocks past the last whole chunk of a row
    const int j = t / rem, r = t - j * rem;
    const int lx = OX + 2 * (4 * ncx + r), ly = ly0 + 2 * j;
    if (!se_check((ly + 1) * SW + lx + 1 < SW * SH, 2u)) continue;
    uint8_t* p = sm + ly * SW + lx;
    uint32_t a = p[0], b = p[1], c = p[SW], d = p[SW + 1];
    if ((a | b | c | d) == 0u) continue;
    const int gx = gx0 + lx, gy = gy0 + ly;
    se_block_update(a, b, c, d, gx, gy, f, W, H, lut);
    se_block_store(p, SW, a, b, c, d, gx, gy, W, H, true);
  }
  __syncthreads();
  const int n = cnt[0], nb = cnt[1];
  if (threadIdx.x == 0) next[0] = next[1] = 0;  // last read in the previous step
  for (int i = threadIdx.x; i < n; i += nt) {
    if (!se_check(i < cap, 4u)) break;
    int ly, q;
    se_divmod_rt(list[i], sw8, inv_sw8, ly, q);
    const int lx = OX + 8 * q, off = ly * SW + lx;
    if (!se_check(off >= 0 && off + SW + 11 <= ((SW * SH + 15) & ~15) + 16, 8u)) continue;
    se_rt_chunk<OX>(sm, SW, off, ly, lx, gx0, gy0, f, W, H, lut);
  }
  for (int i = threadIdx.x; i < nb; i += nt) {  // chunks with cells outside the world
    if (!se_check(i < cap, 4u)) break;
    int ly, q;
    se_divmod_rt(list[cap - 1 - i], sw8, inv_sw8, ly, q);
    const int lx = OX + 8 * q;
    if (!se_check(ly >= 0 && (ly + 1) * SW + lx + 7 < SW * SH, 8u)) continue;
    for (int kb = 0; kb < 4; ++kb) {
      uint8_t* p = sm + ly * SW + lx + 2 * kb;
      uint32_t a = p[0], b = p[1], c = p[SW], d = p[SW + 1];
      if ((a | b | c | d) == 0u) continue;  // all EMPTY stays EMPTY
      const int gx = gx0 + lx + 2 * kb, gy = gy0 + ly;
      se_block_update(a, b, c, d, gx, gy, f, W, H, lut);
      se_block_store(p, SW, a, b, c, d, gx, gy, W, H, true);
    }
  }
}

// Whole-world launch: CTA b holds world ids[b] entirely in shared memory (plus a WALL
// border: 4 columns on the left and at least 4 on the right, the row stride a multiple of
// 8; 1 row above and below), advances it by `frames` frames and stores it to the buffer
// cur ^ out_flip.  Nothing outside the world is ever written back, so the border stays
// WALL for every frame, as getCell returns there.  After the array (rounded up to 16
// bytes): 16 bytes of slack, the list counters of alternate frames, the uniform-material
// flags, then the chunk list (SE_HDR_* offsets, as in the tile kernel), one entry per chunk.
extern "C" __global__ void __launch_bounds__(1024) se_resident(const SeWorldDesc* __restrict__ worlds,
                                                               const int* __restrict__ ids, int frames, int out_flip,
                                                               const uint16_t* __restrict__ lut) {
  extern __shared__ __align__(16) uint8_t se_smem[];
  const SeWorldDesc w = worlds[ids[blockIdx.x]];
  const int SW = ((w.W + 7) & ~7) + 8, SH = w.H + 2;
  const int gx0 = -4, gy0 = -1;
  const int HDR = (SW * SH + 15) & ~15, cap = (SW / 8) * (SH / 2);
  int* cnt = reinterpret_cast<int*>(se_smem + HDR + SE_HDR_CNT);
  uint8_t* flags = se_smem + HDR + SE_HDR_FLAGS;
  uint16_t* list = reinterpret_cast<uint16_t*>(se_smem + HDR + SE_HDR_LIST);
  se_gen::init_tables(threadIdx.x, blockDim.x);
  for (int i = threadIdx.x; i < 4; i += blockDim.x) cnt[i] = 0;
  se_uniform_flags(lut, flags, blockDim.x);
  const uint32_t* src = w.cur ? w.buf1 : w.buf0;
  uint32_t* dst = (w.cur ^ out_flip) ? w.buf1 : w.buf0;
  se_load_region(se_smem, SW, SH, src, w.W, w.H, gx0, gy0, blockDim.x);
  __syncthreads();
  const uint32_t umask = se_flags_mask(flags);
  for (int s = 0; s < frames; ++s) {
    const int f = w.frame + 1 + s;
    const int ly0 = (se_off_y(f) + gy0) & 1;
    int* c = cnt + 2 * (s & 1);
    int* nx = cnt + 2 * ((s + 1) & 1);
    if (se_off_x(f) == 0)
      se_rt_step<0>(se_smem, SW, SH, ly0, gx0, gy0, f, w.W, w.H, lut, umask, list, cap, c, nx);
    else
      se_rt_step<1>(se_smem, SW, SH, ly0, gx0, gy0, f, w.W, w.H, lut, umask, list, cap, c, nx);
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
// grid holds world rows from row0 on (the boxes lie within them).
extern "C" __global__ void __launch_bounds__(256) se_edit(uint32_t* __restrict__ grid, int W, int H, int nmods,
                                                          long long total, const SeEditParams p, int row0) {
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
  if (se_check(y >= row0 && y < H && x >= 0 && x < W, 32u))  // H: the grid's last row + 1
    grid[(size_t)(y - row0) * W + x] = (uint32_t)p.mods[q].mat;
}
