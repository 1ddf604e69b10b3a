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

}  // namespace se::rt
