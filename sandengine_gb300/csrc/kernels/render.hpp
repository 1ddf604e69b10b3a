// The colour and light outputs of the reference's setCell (shaders/compute/operations.glsl
// :99-169), as ahead-of-time sm_103a kernels that read a per-material table.  Plain C++
// declarations, shared by the kernels (render.cu) and the runtime.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace se::rt {

// One material's render data.  Ids >= the table size read entry 1 (NULL), as
// getMaterialFromID returns MAT_NULL for unknown ids.
struct RenderMat {
  float color[4];
  float emission[4];
  uint32_t flags;  // kRender* bits
  uint32_t pad[3];
};
enum : uint32_t {
  kRenderEmits = 1,     // emission.rgb != vec3(0): the cell's light is its emission
  kRenderObstacle = 2,  // isLightObstacle: emission.rgb == vec3(0) and not of type EMPTY
  kRenderNoise = 4,     // mat != MAT_EMPTY: the colour is darkened by the noise
};

// noise(vec2(x, y), 3, 2.0, 0.25) (math.glsl:98-106) for every cell of a W x H world.
cudaError_t render_noise(float* noise, int W, int H, cudaStream_t s);
// output_color (RGBA32F) of a grid, from the cached noise field.
cudaError_t render_color(const uint32_t* grid, const float* noise, float4* out, int W, int H, const RenderMat* mats,
                         int nmat, cudaStream_t s);
// output_light of the frame that took old_grid to new_grid, from the previous light field.
cudaError_t light_pass(const uint32_t* old_grid, const uint32_t* new_grid, const float4* light_in, float4* light_out,
                       int W, int H, const RenderMat* mats, int nmat, cudaStream_t s);

// Headless composite (shaders/fragment140.glsl:70-100): the colour field's box-filter
// pyramid, then one RGBA32F pixel per texel.  GL filtering is fixed to the spec's formulas
// in binary32 (mirrored-repeat wrap, nearest / bilinear taps, LINEAR_MIPMAP_NEAREST level
// choice); the three blur weights exp(-gamma) for gamma 0.5, 0.35, 0.2 are passed in.
// The fragment reads levels above 0 only through their alpha (the occlusion's
// textureLod(...).a), so those levels are kept as alpha alone: the same box-filter sums of
// the alpha channel, a quarter of the bytes.
constexpr int kMaxMipLevels = 24;
// The occlusion's textureLod calls use the integer lods 0 .. 6.
constexpr int kOccLods = 7;
// What the composite samples: the colour field (level 0) and, for lod l = 1 .. 6, the alpha
// level textureLod reads at lod l.  With LINEAR_MIPMAP_NEAREST that is level
// ceil(l + 0.5) - 1 = l, or the last level of a shorter pyramid; a 1 x 1 field has no level
// 1, and its slots hold a copy of its own alpha.
struct CompositeSrc {
  const float4* color;
  int w, h;
  const float* alpha[kOccLods];  // [0] is unused
  int aw[kOccLods], ah[kOccLods];
};
// exp(-gamma) for the three sampleBlurred calls (gamma 0.5, 0.35, 0.2), rounded to binary32.
constexpr float kBlurSideWeight[3] = {0.606530666f, 0.704688072f, 0.818730772f};
// Size of the next level: halved, at least 1.
inline int mip_next(int n) { return n > 1 ? n / 2 : 1; }
// output_color as render_color, plus (alpha1 != null) the pyramid's level-1 alpha,
// mip_next(W) x mip_next(H): a cell's alpha is its material's colour alpha, so the level
// comes from the same pass instead of a second read of the RGBA field.
cudaError_t render_color_mip(const uint32_t* grid, const float* noise, float4* out, float* alpha1, int W, int H,
                             const RenderMat* mats, int nmat, cudaStream_t s);
// The next alpha level (mip_next(sw) x mip_next(sh)) from an alpha level.
cudaError_t render_mip_alpha(const float* src, int sw, int sh, float* dst, cudaStream_t s);
// Column and row tables of the composite, functions of the field's size only (built once):
// u = (c + 0.5) / W and the column of its nearest texel, the pixelated u of each column
// pair (floor(u / d) * d at its even column, d = 1 / (W / 2)), and per row v, its nearest
// row and the pixelated v.  Arrays hold round_up(W + 1, 4) / round_up(H + 1, 4) entries, so
// that the pair loads of an odd last column or row stay in bounds.
struct CompositeCoords {
  const float* u;
  const int* ix;
  const float* pu;
  const float* v;
  const int* iy;
  const float* pv;
};
size_t composite_coords_bytes(int W, int H);
// Fills `buf` (composite_coords_bytes(W, H), 16-byte aligned) and points `out` into it.
cudaError_t render_composite_coords(void* buf, int W, int H, CompositeCoords* out, cudaStream_t s);
cudaError_t render_composite(const CompositeSrc& src, const CompositeCoords& coords, const float4* light,
                             const float4* bg, int bw, int bh, const float w_side[3], float4* out, cudaStream_t s);

}  // namespace se::rt
