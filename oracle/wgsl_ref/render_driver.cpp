// render_driver.cpp — evaluates the reference's relief and colour sampling
// (shaders/render.wgsl: surf_cubic :335-353, base_slope :628-638,
// color_sharp :706-750, wet_bilinear :394-406) and its key-light shadow march
// (surf_bilinear :314-326, shadow_at :846-866), mechanically translated by
// translate.py (translate_subset) into render_ref.inc.
//
// TEST INFRASTRUCTURE.  Built by build_ref.py into oracle/_ref/ only where the
// reference checkout exists; tests/golden/make_relief.py stores its outputs
// as the relief fixture.  The camera is the non-beauty one (cam.jitter.z = 0,
// cam.ortho.z = 0: the colour plane has the film's resolution), so the
// translated functions never reach the stubbed beauty-mode helpers.
#include <array>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <type_traits>
#include <vector>

#include "../film_oracle.hpp"
#include "render_ref.inc"

extern "C" {

void wgrr_set(uint32_t w, uint32_t h, float width_m, float height_m, float dx, const float* hp, const float* mp,
              const float* rgba) {
  using namespace wgrr;
  cam = Cam{};
  cam.canvas = vec4<f32>(width_m, height_m, dx, f32(0));
  cam.size = vec4<u32>(w, h, 0u, 0u);
  const size_t n = (size_t)w * h;
  hbuf.v.assign(hp, hp + n);
  mbuf.v.assign(mp, mp + n);
  color_tex.w = w;
  color_tex.v.resize(n);
  for (size_t c = 0; c < n; ++c)
    color_tex.v[c] = vec4<f32>(rgba[4 * c], rgba[4 * c + 1], rgba[4 * c + 2], rgba[4 * c + 3]);
}

// out per point: surf_cubic, base_slope.x, base_slope.y, color_sharp rgba, wet_bilinear
void wgrr_sample(const double* pts, uint32_t n, double* out) {
  using namespace wgrr;
  for (uint32_t k = 0; k < n; ++k) {
    const vec2<f32> p((f32)pts[2 * k], (f32)pts[2 * k + 1]);
    const vec2<f32> sl = base_slope(p);
    const vec4<f32> col = color_sharp(p);
    double* o = out + 8 * (size_t)k;
    o[0] = surf_cubic(p);
    o[1] = sl.x;
    o[2] = sl.y;
    o[3] = col.x; o[4] = col.y; o[5] = col.z; o[6] = col.w;
    o[7] = wet_bilinear(p);
  }
}

// cam.canvas.w: the top of the relief volume the shadow march stops at
void wgrr_set_top(float top) { wgrr::cam.canvas.w = top; }

// out per point (x, y, z0): surf_bilinear(x, y), shadow_at((x, y), z0, light)
void wgrr_shadow(const double* pts, uint32_t n, const double* light, double* out) {
  using namespace wgrr;
  const vec3<f32> l((f32)light[0], (f32)light[1], (f32)light[2]);
  for (uint32_t k = 0; k < n; ++k) {
    const vec2<f32> p((f32)pts[3 * k], (f32)pts[3 * k + 1]);
    out[2 * k] = surf_bilinear(p);
    out[2 * k + 1] = shadow_at(p, (f32)pts[3 * k + 2], l);
  }
}

}  // extern "C"
