// Driver that runs the reference's own compute shader on the CPU.
// TEST INFRASTRUCTURE ONLY.  `ref_shader.inc` is the reference's flattened
// shaders/compute/falling_sand.glsl (its includes inlined by the reference's flattening
// rule, with gen/materials.glsl and gen/rules.glsl for the rule set under test), passed
// through oracle/glsl2cpp.py.  It is generated into oracle/_ref/ by oracle/build.py
// from the reference tree and never committed.
//
// One call = one glium dispatch (sandengine-core/src/simulation.rs:220-234): every
// invocation inside simSize runs main(); invocations outside it return at once
// (falling_sand.glsl:124-126), so they are not visited.  Invocations are independent:
// each reads the input textures and writes only its own texel.
#include <cstdint>
#include <cstring>

#include "glsl_shim.hpp"

static thread_local uvec3 gl_GlobalInvocationID;

#include "ref_shader.inc"

extern "C" {

#define SE_EXPORT __attribute__((visibility("default")))

// in_data/out_data: RGBA32F W*H*4 (cell id in .r); in_light/out_light and out_color:
// RGBA32F W*H*4.  mods: `nmods` 32-byte SimModification records (simulation.rs:45-56).
SE_EXPORT void ref_dispatch_rows(const float* in_data, float* out_data, float* out_color,
                                 const float* in_light, float* out_light, int W, int H, int frame_value,
                                 const void* mods_raw, int nmods, int nthreads, int y0, int y1);

SE_EXPORT void ref_dispatch(const float* in_data, float* out_data, float* out_color, const float* in_light,
                  float* out_light, int W, int H, int frame_value, const void* mods_raw,
                  int nmods, int nthreads) {
  ref_dispatch_rows(in_data, out_data, out_color, in_light, out_light, W, H, frame_value, mods_raw, nmods,
                    nthreads, 0, H);
}

// The invocations of rows [y0, y1) only (a bounded sample of a dispatch, for timing).
SE_EXPORT void ref_dispatch_rows(const float* in_data, float* out_data, float* out_color,
                                 const float* in_light, float* out_light, int W, int H, int frame_value,
                                 const void* mods_raw, int nmods, int nthreads, int y0, int y1) {
  input_data = sampler2D{in_data, W, H};
  output_data = image2D{out_data, W, H};
  output_color = image2D{out_color, W, H};
  input_light = sampler2D{in_light, W, H};
  output_light = image2D{out_light, W, H};
  output_effects = image2D{nullptr, 0, 0};
  collision_data = image2D{nullptr, 0, 0};
  simSize = ivec2(W, H);
  frame = frame_value;
  moveRight = false;
  time = 0.0f;
  const int32_t* m = (const int32_t*)mods_raw;
  for (int i = 0; i < 256; ++i) {
    SimModification s{};
    if (i < nmods) {
      s.position = ivec2(m[8 * i + 0], m[8 * i + 1]);
      s.mod_shape = m[8 * i + 2];
      s.mod_size = m[8 * i + 3];
      s.mod_matID = m[8 * i + 4];
    } else {
      s.position = ivec2(0, 0);
      s.mod_shape = 0;
      s.mod_size = 0;
      s.mod_matID = 0;
    }
    sim_modifications[i] = s;
  }
  if (nthreads <= 0) nthreads = 1;
  // work items of 256 invocations along a row, so that bands of a few rows still keep every
  // thread busy
  constexpr int kSpan = 256;
  const long long spans = (W + kSpan - 1) / kSpan, items = (long long)(y1 - y0) * spans;
#pragma omp parallel for schedule(dynamic, 4) num_threads(nthreads)
  for (long long t = 0; t < items; ++t) {
    const int y = y0 + (int)(t / spans), x0 = (int)(t % spans) * kSpan;
    const int x1 = x0 + kSpan < W ? x0 + kSpan : W;
    for (int x = x0; x < x1; ++x) {
      gl_GlobalInvocationID = uvec3((uint)x, (uint)y, 0u);
      glsl_main();
    }
  }
}

}  // extern "C"
