"""CPU emulation of the JIT device code.  TEST INFRASTRUCTURE ONLY.

Compiles the exact source handed to NVRTC (Ruleset.kernel_source) with g++ against
cuda_host_shim.hpp and runs the tile kernels with one thread per CTA (see the shim's
header) and the edit kernel thread by thread.  With ``lut=False`` the block transition
table is compiled out, so the direct rule-evaluation path runs instead.  The source is
compiled as the CHECKED build (SE_CHECKED): an emulated launch whose index checks fail
raises.
"""
import ctypes
import hashlib
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(os.path.dirname(os.path.dirname(HERE)), "oracle", "_build")

VARIANTS = [(128, 64, 1), (256, 32, 1), (128, 32, 1), (128, 64, 2), (128, 64, 4), (128, 64, 8),
            (128, 128, 8), (128, 128, 16), (256, 64, 4), (64, 64, 4), (256, 128, 8), (192, 128, 8),
            (256, 128, 4), (256, 64, 8)]

DRIVER = r'''
alignas(16) uint8_t se_smem[1 << 21];
static uint16_t* g_lut = nullptr;
extern "C" const uint16_t* emu_lut() { return g_lut; }
// the checker itself: one failed check of each kind (CPU self-test of the CHECKED build)
extern "C" void emu_check_selftest() {
  for (unsigned bit = 1; bit <= 32; bit <<= 1) (void)se_check(false, bit);
}
// index checks of the CHECKED build: failed-check bits since the last call, then cleared
extern "C" unsigned emu_check_word() {
  const unsigned w = se_check_word;
  se_check_word = 0;
  return w;
}
extern "C" uint32_t emu_lut_index_key(uint32_t i, uint32_t h0, uint32_t h1, uint32_t h2, uint32_t h3) {
#ifdef SE_LUT
  return se_gen::lut_index_key(i, h0, h1, h2, h3);
#else
  return 0;
#endif
}
// entries whose decoded cells and representative hashes do not index back to themselves
extern "C" unsigned long long emu_lut_roundtrip_failures() {
#ifdef SE_LUT
  unsigned long long bad = 0;
  for (uint32_t i = 0; i < SE_LUT_ENTRIES; ++i) {
    uint32_t a, b, c, d, h0, h1, h2, h3;
    se_gen::lut_decode(i, a, b, c, d, h0, h1, h2, h3);
    if (se_gen::lut_index(a, b, c, d, h0, h1, h2, h3) != i) ++bad;
  }
  return bad;
#else
  return 0;
#endif
}
extern "C" const uint32_t* emu_static() {
#ifdef SE_LUT
  return reinterpret_cast<const uint32_t*>(reinterpret_cast<const uint8_t*>(g_lut) + SE_LUT_STATIC_OFF);
#else
  return nullptr;
#endif
}
extern "C" unsigned emu_static_words() {
#ifdef SE_LUT
  return SE_LUT_STATIC_WORDS;
#else
  return 0;
#endif
}
extern "C" int emu_build_lut() {
#ifdef SE_LUT
  g_lut = reinterpret_cast<uint16_t*>(new uint32_t[(SE_LUT_STATIC_OFF + 4u * SE_LUT_STATIC_WORDS) / 4u]);
  blockDim.x = 1; gridDim.x = 1; threadIdx.x = 0; blockIdx.x = 0;
  se_build_lut(g_lut);
  for (unsigned w = 0; w < SE_LUT_STATIC_WORDS; ++w) { blockIdx.x = w; se_build_static(g_lut); }
  blockIdx.x = 0;
  return 1;
#else
  return 0;
#endif
}
#define EMU_TILE(TW, TH, K) \
extern "C" void emu_tile_##TW##x##TH##_k##K(const uint32_t* src, uint32_t* dst, int W, int H, int f0, int k, \
                                           int ya, int yb) { \
  blockDim.x = 1; threadIdx.x = 0; \
  for (unsigned by = 0; by < (unsigned)((yb - ya + TH - 1) / TH); ++by) \
    for (unsigned bx = 0; bx < (unsigned)((W + TW - 1) / TW); ++bx) { \
      blockIdx.x = bx; blockIdx.y = by; \
      se_tile_impl<TW, TH, K, 1>(src, dst, W, H, f0, k, g_lut, ya, yb); \
    } \
}
@TILES@
#define EMU_TILE_EDIT(TW, TH, K) \
extern "C" void emu_tile_edit_##TW##x##TH##_k##K(const uint32_t* src, uint32_t* dst, int W, int H, int f0, int k, \
                                                int ya, int yb, const void* edits, int nedits) { \
  blockDim.x = 1; threadIdx.x = 0; \
  for (unsigned by = 0; by < (unsigned)((yb - ya + TH - 1) / TH); ++by) \
    for (unsigned bx = 0; bx < (unsigned)((W + TW - 1) / TW); ++bx) { \
      blockIdx.x = bx; blockIdx.y = by; \
      se_tile_impl<TW, TH, K, 1>(src, dst, W, H, f0, k, g_lut, ya, yb, \
                                 reinterpret_cast<const SeEditParams*>(edits), nedits); \
    } \
}
@TILE_EDITS@
#define EMU_MTILE(TW, TH, K) \
extern "C" void emu_mtile_##TW##x##TH##_k##K(const SeWorldDesc* worlds, const SeTileJob* jobs, int njobs, \
                                             int pass, int done, int k) { \
  blockDim.x = 1; threadIdx.x = 0; \
  for (int j = 0; j < njobs; ++j) { \
    blockIdx.x = j; \
    se_mtile_impl<TW, TH, K, 1>(worlds, jobs, pass, done, k, g_lut); \
  } \
}
@MTILES@
extern "C" void emu_stile_128x64_k8(const SeWorldDesc* descs, const int* prefix, int n) {
  blockDim.x = 1; threadIdx.x = 0;
  for (int t = 0; t < prefix[n]; ++t) {
    blockIdx.x = t;
    se_stile_impl<128, 64, 8, 1>(descs, prefix, n, g_lut);
  }
}
extern "C" void emu_resident(const SeWorldDesc* worlds, const int* ids, int nids, int frames, int flip) {
  blockDim.x = 1; threadIdx.x = 0;
  for (int j = 0; j < nids; ++j) {
    blockIdx.x = j;
    se_resident(worlds, ids, frames, flip, g_lut);
  }
}
extern "C" void emu_finalize(SeWorldDesc* worlds, int n, int frames, int passes) {
  blockDim.x = 1; threadIdx.x = 0;
  for (int i = 0; i < n; ++i) {
    blockIdx.x = i;
    se_batch_finalize(worlds, n, frames, passes);
  }
}
extern "C" void emu_edit(uint32_t* grid, int W, int H, int nmods, long long total, const void* params) {
  const SeEditParams& p = *reinterpret_cast<const SeEditParams*>(params);
  blockDim.x = 256;
  for (long long t = 0; t < total; ++t) {
    blockIdx.x = (unsigned)(t / 256);
    threadIdx.x = (unsigned)(t % 256);
    se_edit(grid, W, H, nmods, total, p, 0);
  }
}
'''


class Emu:
    def __init__(self, ruleset, lut: bool = True):
        src = ruleset.kernel_source
        if not lut:
            src = src.replace("#define SE_LUT 1\n", "")
        if "#define SE_CHECKED" not in src:  # every emulated launch runs the index checks
            src = "#define SE_CHECKED 1\n" + src
        tiles = "\n".join(f"EMU_TILE({a}, {b}, {c})" for a, b, c in VARIANTS)
        tile_edits = "\n".join(f"EMU_TILE_EDIT({a}, {b}, {c})" for a, b, c in VARIANTS)
        mtiles = "\n".join(f"EMU_MTILE({a}, {b}, {c})" for a, b, c in VARIANTS)
        code = ('#include "cuda_host_shim.hpp"\n' + src +
                DRIVER.replace("@TILES@", tiles).replace("@TILE_EDITS@", tile_edits)
                .replace("@MTILES@", mtiles))
        with open(os.path.join(HERE, "cuda_host_shim.hpp")) as f:
            shim = f.read()
        key = hashlib.sha256((code + shim).encode()).hexdigest()[:16]
        d = os.path.join(OUT, "emu_" + key)
        so = os.path.join(d, "emu.so")
        if not os.path.exists(so):
            os.makedirs(d, exist_ok=True)
            cpp = os.path.join(d, "emu.cpp")
            with open(cpp, "w") as f:
                f.write(code)
            tmp = so + f".tmp{os.getpid()}"
            r = subprocess.run(["g++", "-std=c++17", "-O1", "-fPIC", "-shared", "-ffp-contract=off",
                                "-fno-strict-aliasing", "-w", f"-I{HERE}", cpp, "-o", tmp],
                               capture_output=True, text=True)
            if r.returncode:
                raise RuntimeError(r.stderr[-4000:])
            os.replace(tmp, so)
        self.lib = ctypes.CDLL(so)
        self.lib.emu_check_word.restype = ctypes.c_uint
        self.nmat = ruleset.num_materials
        self.has_lut = bool(self.lib.emu_build_lut())
        self._checked()

    def _checked(self):
        w = self.lib.emu_check_word()
        if w:
            raise AssertionError(f"index check failed in the emulated kernel (check word {w:#x})")

    def tiles(self, src: np.ndarray, f0: int, k: int, variant=None, band=None) -> np.ndarray:
        """k frames (counters f0..f0+k-1) with one launch of the tile kernel.  With
        ``band = (world_height, ya)``, ``src`` holds world rows [ya, ya + src rows)."""
        if variant is None:
            variant = min((v for v in VARIANTS if v[2] >= k), key=lambda v: v[2])
        fn = getattr(self.lib, "emu_tile_%dx%d_k%d" % variant)
        fn.argtypes = [ctypes.c_void_p, ctypes.c_void_p] + [ctypes.c_int] * 6
        rows, W = src.shape
        H, ya = band if band else (rows, 0)
        dst = np.zeros_like(src)
        fn(src.ctypes.data, dst.ctypes.data, W, H, f0, k, ya, ya + rows)
        self._checked()
        return dst

    def batch(self, grids, frames0, F, k, resident, variant=(128, 64, 8)):
        """Advances worlds by F frames the way a batch launch does: worlds in ``resident``
        by the whole-world kernel, the others by ceil(F/k) tile passes, then finalize.
        Returns the new grids and frame counters."""
        n = len(grids)
        desc = np.zeros(n, dtype=[("b0", "<u8"), ("b1", "<u8"), ("W", "<i4"), ("H", "<i4"), ("frame", "<i4"),
                                  ("cur", "<i4"), ("p0", "<i4"), ("p1", "<i4")])
        bufs = []
        for i, g in enumerate(grids):
            a, b = np.ascontiguousarray(g, dtype=np.uint32).copy(), np.zeros_like(g, dtype=np.uint32)
            bufs.append((a, b))
            desc[i] = (a.ctypes.data, b.ctypes.data, g.shape[1], g.shape[0], frames0[i], 0, 0, 0)
        tiled = [i for i in range(n) if i not in resident]
        P = (F + k - 1) // k if tiled else 0
        vp = ctypes.c_void_p
        if resident:
            ids = np.array(resident, dtype=np.int32)
            self.lib.emu_resident.argtypes = [vp, vp, ctypes.c_int, ctypes.c_int, ctypes.c_int]
            self.lib.emu_resident(desc.ctypes.data, ids.ctypes.data, len(ids), F, P & 1)
        if tiled:
            tw, th, _ = variant
            jobs = np.array([(w, x, y, 0) for w in tiled for y in range(0, grids[w].shape[0], th)
                             for x in range(0, grids[w].shape[1], tw)], dtype=np.int32)
            fn = getattr(self.lib, "emu_mtile_%dx%d_k%d" % variant)
            fn.argtypes = [vp, vp, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int]
            for p in range(P):
                fn(desc.ctypes.data, jobs.ctypes.data, len(jobs), p, p * k, min(k, F - p * k))
        self.lib.emu_finalize.argtypes = [vp, ctypes.c_int, ctypes.c_int, ctypes.c_int]
        self.lib.emu_finalize(desc.ctypes.data, n, F, P)
        self._checked()
        out = [bufs[i][int(desc[i]["cur"])] for i in range(n)]
        return out, [int(f) for f in desc["frame"]]

    def serve_iteration(self, grids, frames, ks):
        """One serving iteration (128x64 tiles, up to 8 frames): world a advances ks[a]
        frames from counter frames[a].  Returns the new grids."""
        n = len(grids)
        desc = np.zeros(n, dtype=[("b0", "<u8"), ("b1", "<u8"), ("W", "<i4"), ("H", "<i4"), ("frame", "<i4"),
                                  ("cur", "<i4"), ("k", "<i4"), ("p1", "<i4")])
        outs, prefix, total = [], [], 0
        for a, g in enumerate(grids):
            src = np.ascontiguousarray(g, dtype=np.uint32)
            dst = np.zeros_like(src)
            outs.append((src, dst))
            desc[a] = (src.ctypes.data, dst.ctypes.data, g.shape[1], g.shape[0], frames[a], 0, ks[a], 0)
            prefix.append(total)
            total += ((g.shape[1] + 127) // 128) * ((g.shape[0] + 63) // 64)
        prefix.append(total)
        pre = np.array(prefix, dtype=np.int32)
        self.lib.emu_stile_128x64_k8.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int]
        self.lib.emu_stile_128x64_k8(desc.ctypes.data, pre.ctypes.data, n)
        self._checked()
        return [o[1] for o in outs]

    def tiles_edit(self, src: np.ndarray, f0: int, k: int, mods, variant=None) -> np.ndarray:
        """k frames with one launch of the tile kernel's edit variant: the first frame's edit
        pass (``mods``) inside the launch."""
        if variant is None:
            variant = min((v for v in VARIANTS if v[2] >= k), key=lambda v: v[2])
        fn = getattr(self.lib, "emu_tile_edit_%dx%d_k%d" % variant)
        fn.argtypes = [ctypes.c_void_p, ctypes.c_void_p] + [ctypes.c_int] * 6 + [ctypes.c_void_p, ctypes.c_int]
        H, W = src.shape
        buf, nlive, _ = self.edit_params(W, H, mods)
        dst = np.zeros_like(src)
        fn(src.ctypes.data, dst.ctypes.data, W, H, f0, k, 0, H, buf.ctypes.data, nlive)
        self._checked()
        return dst

    def edit_params(self, W: int, H: int, mods):
        """The SeEditParams block (as int32 words), the live mod count and the box cells,
        prepared as runtime/engine.cpp's fill_edit_params does."""
        buf = np.zeros(14352 // 4, dtype=np.int32)
        m = buf[:2048].reshape(256, 8)
        box = buf[2048:3072].reshape(256, 4)
        start = buf[3072:3072 + 514].view(np.int64)
        live = []
        for mod in mods[:256]:
            if mod[3] == 0:
                break
            live.append(mod)
        total = 0
        for i, (px, py, shape, size, mat) in enumerate(live):
            m[i, :5] = (px, py, shape, size, mat if 0 <= mat < self.nmat else 1)
            r = abs(size)
            normal = r < (1 << 22) and abs(px) < (1 << 30) and abs(py) < (1 << 30)
            x0, y0, x1, y1 = 0, 0, W - 1, H - 1
            if normal:
                x0, x1, y0, y1 = max(0, px - r), min(W - 1, px + r), max(0, py - r), min(H - 1, py + r)
            start[i] = total
            if x1 >= x0 and y1 >= y0:
                box[i] = (x0, y0, x1, y1)
                total += (x1 - x0 + 1) * (y1 - y0 + 1)
            else:
                box[i] = (0, 0, -1, -1)
        start[len(live)] = total
        return buf, len(live), total

    def edit(self, grid: np.ndarray, mods) -> None:
        """The edit pass in place; host-side preparation as in runtime/engine.cpp."""
        H, W = grid.shape
        buf, nlive, total = self.edit_params(W, H, mods)
        if total:
            self.lib.emu_edit.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                          ctypes.c_longlong, ctypes.c_void_p]
            self.lib.emu_edit(grid.ctypes.data, W, H, nlive, total, buf.ctypes.data)
            self._checked()
