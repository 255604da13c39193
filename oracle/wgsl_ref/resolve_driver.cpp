// resolve_driver.cpp — evaluates the reference's display fragment shader
// (shaders/resolve.wgsl: fs :76-121 with aces :23-26, agx :28-51,
// to_srgb :53-57, hash12 :59-63, lum :65-67, load :69-74), mechanically
// translated by translate.py (translate_subset) into resolve_ref.inc.
//
// TEST INFRASTRUCTURE.  Built by build_ref.py into oracle/_ref/ only where the
// reference checkout exists; tests/golden/make_resolve.py stores its outputs
// as the resolve fixture.  The fragment runs at every pixel centre
// (@builtin(position) = (x + 0.5, y + 0.5)) of a w x h image held in the
// `acc` texture; R is the Res uniform (a, b, c: 12 floats).
#include <array>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <type_traits>
#include <vector>

#include "../film_oracle.hpp"
#include "resolve_ref.inc"

extern "C" {

// rgba: w*h*4 floats (the HDR image, row-major); res: R.a, R.b, R.c;
// out: w*h*4 doubles, the fragment's output colour (sRGB in [0, 1], alpha 1)
void wgres_run(uint32_t w, uint32_t h, const float* rgba, const float* res, double* out) {
  using namespace wgres;
  const size_t n = (size_t)w * h;
  acc.w = w;
  acc.v.resize(n);
  for (size_t c = 0; c < n; ++c) acc.v[c] = vec4<f32>(rgba[4 * c], rgba[4 * c + 1], rgba[4 * c + 2], rgba[4 * c + 3]);
  R.a = vec4<f32>(res[0], res[1], res[2], res[3]);
  R.b = vec4<f32>(res[4], res[5], res[6], res[7]);
  R.c = vec4<f32>(res[8], res[9], res[10], res[11]);
  for (uint32_t y = 0; y < h; ++y)
    for (uint32_t x = 0; x < w; ++x) {
      VOut in;
      in.pos = vec4<f32>(f32(x) + f32(0.5), f32(y) + f32(0.5), f32(0), f32(1));
      const vec4<f32> o = fs(in);
      double* d = out + 4 * ((size_t)y * w + x);
      d[0] = o.x; d[1] = o.y; d[2] = o.z; d[3] = o.w;
    }
}

}  // extern "C"
