// CUDA back end of the rule language.
//
// Input: the parsed rule set and, for every used rule, the GLSL function text that
// sandengine-lang would emit (lang::rule_glsl).  The GLSL rule bodies are parsed as GLSL
// (statements: blocks, if/else, return, swap(a, b), x = newCell(MAT_m, pos); expressions
// over the four block cells, rand, pos, frame and simSize) and re-emitted as device
// functions over material ids.  A cell is its material id in a 32-bit register: member
// access goes through per-material tables (density, type, id, colour, emission), type
// checks become material bit sets, and comparisons of rand.x/y/z/w against constants
// become exact integer comparisons on the hash lanes (RN(float(u)) * 2^-32 is monotone in
// u, so `rand.y <= p` is `lane <= T` for one threshold T computed on the host).
//
// GLSL that would not compile in the reference shader is reported as kind "Glsl";
// valid GLSL outside the translated subset (cell positions, calls into other shader
// functions, nondeterministic uniforms) as "Unsupported".
#pragma once

#include <string>

#include "lang.hpp"

namespace se::lang {

struct CudaRules {
  std::string source;  // device code, namespace se_gen (see kernels/margolus.cuh)
  int num_materials = 0;
  bool uses_rand_lane[4] = {false, false, false, false};
  // Entries of the block transition table (u16 each), 0 when the rules need the direct
  // evaluation path (they read positions / the frame, use rand as a number, or there are
  // more than 16 materials).
  unsigned long long lut_entries = 0;
  // 32-bit words of the table's "static block" bitset (one bit per four-cell key: the block
  // never changes, whatever the hash), stored after the table.
  unsigned long long lut_static_words = 0;
};

bool generate_cuda(const ParsingResult& r, CudaRules* out, ParseError* err);

}  // namespace se::lang
