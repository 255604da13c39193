// render_fs_driver.cpp — evaluates the reference renderer's fragment shader
// (shaders/render.wgsl: fs :985-1116 with lit :1118-1143 and every function
// they reach: the ray march over the relief, the tool micro-relief of the
// detail texture, the canvas weave, the beauty-mode colour, the key-light
// shadow, ambient occlusion, the environment, softbox and GGX lobes, tonemap
// and sRGB), mechanically translated by translate.py (translate_subset) into
// render_fs_ref.inc, in f32 with one rounding per operation.
//
// TEST INFRASTRUCTURE.  Built by build_ref.py into oracle/_ref/ only where the
// reference checkout exists; tests/golden/make_render_lit.py stores its
// outputs as the lit-render fixture.
#include <array>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <type_traits>
#include <vector>

#include "../film_oracle.hpp"
#include "render_fs_ref.inc"

extern "C" {

// cam: the Cam uniform as the renderer writes it, 76 words in field order
// (inv_vp 16, eye 4, canvas 4, light 4, size 4 (u32), sky 4, ground 4, vp 16,
// jitter 4, ortho 4, basis_r 4, basis_u 4, lens 4), matrices column-major.
void wgrf_set(const float* cam_words, uint32_t w, uint32_t h, const float* hp, const float* mp, const float* rgba,
              const float* detail, const uint32_t* tf) {
  using namespace wgrf;
  const float* q = cam_words;
  auto m4 = [&](mat4x4<f32>& m) { for (int k = 0; k < 16; ++k) m.m[k] = (f32)*q++; };
  auto v4 = [&](vec4<f32>& v) { v = vec4<f32>((f32)q[0], (f32)q[1], (f32)q[2], (f32)q[3]); q += 4; };
  cam = Cam{};
  m4(cam.inv_vp);
  v4(cam.eye);
  v4(cam.canvas);
  v4(cam.light);
  uint32_t sz[4];
  std::memcpy(sz, q, 16);
  q += 4;
  cam.size = vec4<u32>(sz[0], sz[1], sz[2], sz[3]);
  v4(cam.sky);
  v4(cam.ground);
  m4(cam.vp);
  v4(cam.jitter);
  v4(cam.ortho);
  v4(cam.basis_r);
  v4(cam.basis_u);
  v4(cam.lens);
  const size_t n = (size_t)w * h;
  hbuf.v.assign(hp, hp + n);
  mbuf.v.assign(mp, mp + n);
  color_tex.w = w;
  color_tex.v.resize(n);
  detail_tex.w = w;
  detail_tex.v.resize(n);
  for (size_t c = 0; c < n; ++c) {
    color_tex.v[c] = vec4<f32>(rgba[4 * c], rgba[4 * c + 1], rgba[4 * c + 2], rgba[4 * c + 3]);
    detail_tex.v[c] = vec4<f32>(detail[4 * c], detail[4 * c + 1], detail[4 * c + 2], detail[4 * c + 3]);
  }
  const size_t nt = (size_t)((w + 15) / 16) * ((h + 15) / 16);
  tile_flags.v.assign(tf, tf + nt);
}

// out per point: the fragment's rgba for a pixel whose interpolated ndc is (x, y)
void wgrf_fs(const double* ndc, uint32_t n, double* out) {
  using namespace wgrf;
  for (uint32_t k = 0; k < n; ++k) {
    VOut in{};
    in.ndc = vec2<f32>((f32)ndc[2 * k], (f32)ndc[2 * k + 1]);
    const vec4<f32> c = fs(in);
    for (int e = 0; e < 4; ++e) out[4 * k + e] = c[e];
  }
}

}  // extern "C"
