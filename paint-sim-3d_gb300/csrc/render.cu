// render.cu — the renderer's fragment shader over the film (shaders/render.wgsl
// fs :985-1116 and lit :1118-1143, with every function they reach): per
// output pixel, the camera ray (orthographic, perspective or thin-lens) is
// marched over the relief h + m and refined by bisection, the hit point takes
// the tool micro-relief of the detail texel (brush and knife grooves, roller
// stipple, the skin's wrinkles), the sharpened or beauty-mode colour, the
// canvas weave where the paint is thin, and is lit by the key light (shadow
// march), ambient occlusion, the environment with its softboxes and the
// GGX lobes (anisotropic along the stroke), then tonemapped to sRGB.
//
// The film supplies the renderer's bindings: h and m (hbuf, mbuf), the
// colour plane (color_tex, rgba16f at the film's resolution), the detail
// texel the strata pass writes with the colour (detail_tex, shade.wgsl:61-64)
// and the tile activity flags.  The camera is the renderer's uniform as the
// caller fills it (cf_render_cam, the layout of render.wgsl:1-15).
//
// Every function follows the shader's f32 arithmetic in its order of
// operations; this file is compiled without multiply-add contraction, so the
// image equals the shader's one-rounding-per-operation evaluation up to the
// last bits of the transcendental functions.
//
// The helpers that the march and the lighting reach from several call sites
// are __noinline__, and the longer loops are not unrolled: inlined whole, the
// kernel's code outgrew the instruction cache and most warps stalled on
// instruction fetch (5.4 ms per 1920x1080 frame against 2.7 ms now).
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <cstdint>

#include "film_handle.h"

namespace {

// One out-of-line copy of each CUDA math function the shader calls from
// many sites (the same functions, so the same results): the kernel's code
// shrinks by a seventh and the frame takes 2.67 instead of 2.96 ms.
__device__ __noinline__ float o_sinf(float x) { return sinf(x); }
__device__ __noinline__ float o_cosf(float x) { return cosf(x); }
__device__ __noinline__ float o_powf(float x, float y) { return powf(x, y); }
__device__ __noinline__ float o_expf(float x) { return expf(x); }

using cfk::Film;

// ---- small vector algebra (componentwise, in the shader's operand order)
__device__ __forceinline__ float2 v2(float a, float b) { return make_float2(a, b); }
__device__ __forceinline__ float3 v3(float a, float b, float c) { return make_float3(a, b, c); }
__device__ __forceinline__ float2 operator+(float2 a, float2 b) { return v2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ float2 operator-(float2 a, float2 b) { return v2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ float2 operator*(float2 a, float2 b) { return v2(a.x * b.x, a.y * b.y); }
__device__ __forceinline__ float2 operator*(float2 a, float s) { return v2(a.x * s, a.y * s); }
__device__ __forceinline__ float2 operator*(float s, float2 a) { return v2(s * a.x, s * a.y); }
__device__ __forceinline__ float2 operator/(float2 a, float s) { return v2(a.x / s, a.y / s); }
__device__ __forceinline__ float3 operator+(float3 a, float3 b) { return v3(a.x + b.x, a.y + b.y, a.z + b.z); }
__device__ __forceinline__ float3 operator-(float3 a, float3 b) { return v3(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ float3 operator*(float3 a, float3 b) { return v3(a.x * b.x, a.y * b.y, a.z * b.z); }
__device__ __forceinline__ float3 operator*(float3 a, float s) { return v3(a.x * s, a.y * s, a.z * s); }
__device__ __forceinline__ float3 operator*(float s, float3 a) { return v3(s * a.x, s * a.y, s * a.z); }
__device__ __forceinline__ float3 operator/(float3 a, float s) { return v3(a.x / s, a.y / s, a.z / s); }
__device__ __forceinline__ float3 operator-(float3 a) { return v3(-a.x, -a.y, -a.z); }
__device__ __forceinline__ float4 operator+(float4 a, float4 b) { return make_float4(a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w); }
__device__ __forceinline__ float4 operator*(float4 a, float s) { return make_float4(a.x * s, a.y * s, a.z * s, a.w * s); }
__device__ __forceinline__ float4 operator*(float s, float4 a) { return make_float4(s * a.x, s * a.y, s * a.z, s * a.w); }
__device__ __forceinline__ float4 operator/(float4 a, float s) { return make_float4(a.x / s, a.y / s, a.z / s, a.w / s); }
__device__ __forceinline__ float dot2(float2 a, float2 b) { return 0.f + a.x * b.x + a.y * b.y; }
__device__ __forceinline__ float dot3(float3 a, float3 b) { return 0.f + a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ float len2(float2 a) { return sqrtf(dot2(a, a)); }
__device__ __forceinline__ float len3(float3 a) { return sqrtf(dot3(a, a)); }
__device__ __forceinline__ float2 nrm2(float2 a) { return a / len2(a); }
__device__ __forceinline__ float3 nrm3(float3 a) { return a / len3(a); }
__device__ __forceinline__ float3 cross3(float3 a, float3 b) {
  return v3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
__device__ __forceinline__ float mixf(float a, float b, float t) { return a * (1.0f - t) + b * t; }
__device__ __forceinline__ float3 mix3(float3 a, float3 b, float t) { return a * (1.0f - t) + b * t; }
__device__ __forceinline__ float4 mix4(float4 a, float4 b, float t) { return a * (1.0f - t) + b * t; }
__device__ __forceinline__ float clampf(float x, float lo, float hi) { return fminf(fmaxf(x, lo), hi); }
__device__ __forceinline__ float sstep(float e0, float e1, float x) {
  const float t = clampf((x - e0) / (e1 - e0), 0.f, 1.f);
  return t * t * (3.0f - 2.0f * t);
}
__device__ __forceinline__ float fractf(float x) { return x - floorf(x); }
__device__ __forceinline__ float2 floor2(float2 a) { return v2(floorf(a.x), floorf(a.y)); }
__device__ __forceinline__ float2 fract2(float2 a) { return v2(fractf(a.x), fractf(a.y)); }
__device__ __forceinline__ float sel4(float4 v, int k) { return k == 0 ? v.x : (k == 1 ? v.y : (k == 2 ? v.z : v.w)); }
__device__ __forceinline__ float3 rgb(float4 c) { return v3(c.x, c.y, c.z); }

// render.wgsl:25-93
constexpr float TAU = 6.2831853f, PI = 3.14159265f;
constexpr float METHOD_BRUSH = 4.0f, METHOD_KNIFE = 5.0f, METHOD_ROLLER = 6.0f;
constexpr float ROLLER_STIPPLE_DEPTH = 14e-6f, ROLLER_STIPPLE_SCALE = 0.7e-3f, ROLLER_STIPPLE_STRETCH = 1.6f;
constexpr float F0_PAINT = 0.04f, BRISTLE_SPACING = 0.35e-3f, BRISTLE_DEPTH = 25e-6f, KNIFE_SPACING = 0.09e-3f;
constexpr float KNIFE_DEPTH = 6e-6f, GROOVE_FULL_DEPTH_AT = 0.3e-3f, WRINKLE_WAVELENGTH = 0.8e-3f;
constexpr float WRINKLE_HEIGHT = 8e-6f, THIN_FILM_MATTE = 0.12e-3f, SIGMA_PAINT = 0.035f, KEY_HALF_ANGLE = 0.12f;
constexpr float SOFTBOX_HALF_W = 0.45f, SOFTBOX_HALF_H = 0.3f, SOFTBOX_RADIANCE = 5.0f;
constexpr int AO_DIRS = 6, AO_STEPS = 4;
constexpr float FILL_RADIANCE = 0.35f, COAT_ROUGH = 0.07f, GRAIN_SCALE = 0.6e-3f, WEAVE_PERIOD = 1.4e-3f;
constexpr float LAMP_DIST = 1.3f, HWARP_FINE = 0.06e-3f, HWARP_COARSE = 0.12e-3f, CWARP_ISO = 0.22e-3f;
constexpr float CWARP_STREAK = 0.45e-3f, STREAK_WIDTH = 0.11e-3f, STREAK_LENGTH = 2.8e-3f;
constexpr float TELEGRAPH_DEPTH = 0.09e-3f, IMPASTO_FRACTION = 0.05f, IMPASTO_MAX = 25e-6f, ZENITH_DIM = 0.2f;
constexpr float PINHOLE_CELL = 0.7e-3f, PINHOLE_RATE = 0.05f, BEAUTY_SOFTBOX_SCALE = 1.5f;
constexpr float BEAUTY_SOFTBOX_RADIANCE = 1.6f, PAINT_HUE_DRIFT = 0.035f, PAINT_TONE_DRIFT = 0.06f;
constexpr float BEAUTY_MIN_ALPHA = 0.035f, FIREFLY_CLAMP = 40.0f, BEAUTY_PENUMBRA = 0.03f, SHADOW_BIAS = 2e-6f;
constexpr float CLUMP_WIDTH = 1.1e-3f, CLUMP_ELONGATION = 14.0f, CLUMP_DEPTH = 14e-6f, DRY_GLOSS_FLOOR = 0.06f;
constexpr float DRY_GLOSS_SCALE = 0.5f, COLOR_CRISP = 2.2f, MARBLE_R1 = 1.2e-3f, MARBLE_R2 = 2.6e-3f;
constexpr float MARBLE_MIN_CONTRAST = 0.03f, MARBLE_SCALE = 1.6e-3f, MARBLE_SOFT = 0.06f, MARBLE_STRENGTH = 0.85f;
constexpr float MARBLE_SELECT = 6.0f, EDGE_MIN_STEP = 15e-6f, EDGE_ISO = 0.3f, EDGE_ISO_SOFT = 0.08f;
__device__ __forceinline__ float3 floor_color() { return v3(0.052f, 0.055f, 0.061f); }
__device__ __forceinline__ float3 horizon_glow() { return v3(0.62f, 0.6f, 0.56f); }
__device__ __forceinline__ float3 fill_tint() { return v3(0.86f, 0.92f, 1.0f); }

// The renderer's bindings (render.wgsl:17-23).
struct R {
  cf_render_cam cam;
  const float* h;
  const float* m;
  const ushort4* color;
  const ushort4* detail;
  const uint32_t* tile_flags;
  __device__ bool beauty() const { return cam.jitter[2] > 0.5f; }  // render.wgsl:249-251
};
__device__ __forceinline__ float4 f16x4(ushort4 u) {
  return make_float4(__half2float(__ushort_as_half(u.x)), __half2float(__ushort_as_half(u.y)),
                     __half2float(__ushort_as_half(u.z)), __half2float(__ushort_as_half(u.w)));
}

// ---- noise (render.wgsl:180-247)
__device__ float hash21(float2 p) {
  float2 q = fract2(p * v2(0.1031f, 0.1030f));
  const float d = dot2(q, v2(q.y, q.x) + v2(33.33f, 33.33f));
  q = v2(q.x + d, q.y + d);
  return fractf((q.x + q.y) * q.x);
}
__device__ float vnoise(float2 p) {
  const float2 i = floor2(p), f = fract2(p);
  const float2 u = f * f * v2(3.0f - 2.0f * f.x, 3.0f - 2.0f * f.y);
  const float a = hash21(i), b = hash21(i + v2(1.0f, 0.0f)), c = hash21(i + v2(0.0f, 1.0f)),
              d = hash21(i + v2(1.0f, 1.0f));
  return mixf(mixf(a, b, u.x), mixf(c, d, u.x), u.y) * 2.0f - 1.0f;
}
__device__ float2 hash22(float2 p) {
  float3 q = v3(fractf(p.x * 0.1031f), fractf(p.y * 0.1030f), fractf(p.x * 0.0973f));
  const float d = dot3(q, v3(q.y, q.z, q.x) + v3(33.33f, 33.33f, 33.33f));
  q = v3(q.x + d, q.y + d, q.z + d);
  return fract2((v2(q.x, q.x) + v2(q.y, q.z)) * v2(q.z, q.y));
}
__device__ float gnoise(float2 p) {
  const float2 i = floor2(p), f = fract2(p);
  const float2 u = f * f * f * v2(f.x * (f.x * 6.0f - 15.0f) + 10.0f, f.y * (f.y * 6.0f - 15.0f) + 10.0f);
  const float2 one = v2(1.0f, 1.0f);
  const float2 ga = hash22(i) * 2.0f - one, gb = hash22(i + v2(1.0f, 0.0f)) * 2.0f - one,
               gc = hash22(i + v2(0.0f, 1.0f)) * 2.0f - one, gd = hash22(i + v2(1.0f, 1.0f)) * 2.0f - one;
  const float a = dot2(ga, f), b = dot2(gb, f - v2(1.0f, 0.0f)), c = dot2(gc, f - v2(0.0f, 1.0f)),
              d = dot2(gd, f - v2(1.0f, 1.0f));
  return 1.4f * mixf(mixf(a, b, u.x), mixf(c, d, u.x), u.y);
}
__device__ __noinline__ float fbm(float2 p, int octaves) {
  float2 q = p;
  float amp = 0.5f, sum = 0.0f, norm = 0.0f;
  for (int k = 0; k < octaves; ++k) {
    sum += amp * gnoise(q);
    norm += amp;
    q = v2(1.6f * q.x - 1.2f * q.y, 1.2f * q.x + 1.6f * q.y) + v2(3.1f, 1.7f);
    amp *= 0.5f;
  }
  return sum / norm;
}
__device__ __noinline__ float fbm_filtered(const R& X, float2 p, float scale, int octaves) {
  float2 q = p / scale;
  float amp = 0.5f, sum = 0.0f, norm = 0.0f, size = scale;
  for (int k = 0; k < octaves; ++k) {
    const float keep = 1.0f - sstep(0.5f, 1.5f, X.cam.jitter[3] / size);
    sum += amp * gnoise(q) * keep;
    norm += amp;
    q = v2(1.6f * q.x - 1.2f * q.y, 1.2f * q.x + 1.6f * q.y) + v2(3.1f, 1.7f);
    amp *= 0.5f;
    size *= 0.5f;
  }
  return sum / norm;
}

// ---- canvas (render.wgsl:94-178)
__device__ __noinline__ float3 weave(float2 p) {
  const float2 q = p / WEAVE_PERIOD;
  const float wx = 1.0f + 0.35f * vnoise(v2(floorf(q.x) * 0.37f, q.y * 0.11f));
  const float wy = 1.0f + 0.35f * vnoise(v2(q.x * 0.11f, floorf(q.y) * 0.37f) + v2(5.0f, 3.0f));
  const float ox = 0.25f * vnoise(v2(floorf(q.y) * 0.5f, 1.0f));
  const float oy = 0.25f * vnoise(v2(floorf(q.x) * 0.5f, 7.0f));
  const float fx = fractf(q.x + ox + 0.08f * vnoise(p / 6.0e-3f));
  const float fy = fractf(q.y + oy + 0.08f * vnoise(p / 6.0e-3f + v2(2.0f, 4.0f)));
  const float warp = wx * (1.0f - o_powf(fabsf(fx - 0.5f) * 2.0f, 1.6f));
  const float weft = wy * (1.0f - o_powf(fabsf(fy - 0.5f) * 2.0f, 1.6f));
  const float over = fractf(0.5f * floorf(q.x) + 0.5f * floorf(q.y)) < 0.5f ? 0.0f : 1.0f;
  const float top = mixf(warp, weft, over);
  const float fibres = vnoise(p / 0.22e-3f + v2(fx, fy)) * vnoise(p / 0.7e-3f + v2(4.0f, 2.0f));
  return v3(top, fmaxf(warp, weft), fibres);
}
__device__ __noinline__ float3 canvas_albedo(float2 p, float3 base) {
  const float3 w = weave(p);
  const float thread = 0.16f * (w.y - 0.6f) + 0.05f * w.z;
  const float slub = 0.08f * fmaxf(vnoise(p / 2.3e-3f + v2(5.0f, 1.0f)) - 0.5f, 0.0f) / 0.5f;
  const float drift = 0.05f * vnoise(p / 0.08f) + 0.03f * vnoise(p / 0.025f + v2(11.0f, 4.0f));
  const float3 tint = v3(1.0f + 0.02f * vnoise(p / 0.05f + v2(2.0f, 9.0f)), 1.0f,
                         1.0f - 0.025f * vnoise(p / 0.06f + v2(8.0f, 3.0f)));
  return base * (1.0f + thread + slub + drift) * tint;
}
__device__ float canvas_bump(float2 p) {
  const float3 w = weave(p);
  return 14e-6f * (w.x - 0.5f) + 4e-6f * w.z;
}
__device__ __noinline__ float canvas_bump_levelled(float2 p, float hp) {
  const float2 q = p / WEAVE_PERIOD;
  const float ox = 0.25f * vnoise(v2(floorf(q.y) * 0.5f, 1.0f));
  const float oy = 0.25f * vnoise(v2(floorf(q.x) * 0.5f, 7.0f));
  const float fx = q.x + ox + 0.08f * vnoise(p / 6.0e-3f);
  const float fy = q.y + oy + 0.08f * vnoise(p / 6.0e-3f + v2(2.0f, 4.0f));
  const float warp = 0.5f - 0.5f * o_cosf(TAU * fx);
  const float weft = 0.5f - 0.5f * o_cosf(TAU * fy);
  const float over = fractf(0.5f * floorf(q.x) + 0.5f * floorf(q.y)) < 0.5f ? 0.0f : 1.0f;
  const float sharp = o_expf(-hp / (0.4f * TELEGRAPH_DEPTH));
  const float top = mixf(warp, weft, over);
  return mixf(14e-6f * (warp * weft - 0.25f), canvas_bump(p), sharp) * o_expf(-hp / TELEGRAPH_DEPTH) +
         3e-6f * (top - 0.5f) * (1.0f - sharp) * o_expf(-hp / TELEGRAPH_DEPTH);
}
__device__ __noinline__ float pinholes(float2 p, float hp) {
  const float2 g = floor2(p / PINHOLE_CELL);
  float z = 0.0f;
#pragma unroll 1
  for (int b = -1; b <= 1; ++b)
#pragma unroll 1
    for (int a = -1; a <= 1; ++a) {
      const float2 c = g + v2((float)a, (float)b);
      const float2 r = hash22(c * 0.731f + v2(0.17f, 0.61f));
      const float r2 = hash21(c * 0.413f + v2(0.93f, 0.29f));
      if (r2 > PINHOLE_RATE) continue;
      const float2 centre = (c + v2(0.15f, 0.15f) + 0.7f * r) * PINHOLE_CELL;
      const float radius = mixf(0.025e-3f, 0.09e-3f, r.x * r.y) * fminf(hp / 0.4e-3f, 1.0f);
      const float d = len2(p - centre) / fmaxf(radius, 1e-6f);
      const float crater = -(1.0f - sstep(0.0f, 1.0f, d)) + 0.35f * o_expf(-(d - 1.15f) * (d - 1.15f) * 8.0f);
      z += crater * radius * 0.45f;
    }
  return z;
}
__device__ __noinline__ float2 specks(float2 p) {
  const float cell = 0.35e-3f;
  const float2 g = floor2(p / cell);
  const float r = hash21(g * 0.173f + v2(0.31f, 0.77f));
  const float r2 = hash21(g * 0.291f + v2(0.59f, 0.13f));
  const float2 centre = (g + v2(0.2f + 0.6f * r, 0.2f + 0.6f * r2)) * cell;
  const float d = len2(p - centre) / (cell * (0.08f + 0.12f * r2));
  const float hit = 1.0f - sstep(0.6f, 1.0f, d);
  return v2(r > 0.985f ? hit : 0.0f, r < 0.012f ? hit : 0.0f);
}
__device__ __noinline__ float lamp_falloff(const R& X, float2 p) {
  const float3 l = nrm3(v3(X.cam.light[0], X.cam.light[1], X.cam.light[2]));
  const float3 centre = v3(0.5f * X.cam.canvas[0], 0.5f * X.cam.canvas[1], 0.0f);
  const float3 lamp = centre + l * LAMP_DIST;
  const float3 d = lamp - v3(p.x, p.y, 0.0f);
  const float dl = len3(d);
  const float cosine = fmaxf(dot3(d / dl, l), 0.0f);
  return (LAMP_DIST * LAMP_DIST) / (dl * dl) * o_powf(cosine, 1.5f);
}

// ---- beauty-mode warps (render.wgsl:253-267)
__device__ __noinline__ float2 hwarp(const R& X, float2 p) {
  if (!X.beauty()) return p;
  const float2 a = v2(fbm(p / 0.7e-3f, 3), fbm(p / 0.7e-3f + v2(17.1f, 3.7f), 3));
  const float2 b = v2(gnoise(p / 3.5e-3f + v2(5.2f, 1.3f)), gnoise(p / 3.5e-3f + v2(9.4f, 2.8f)));
  return p + HWARP_FINE * a + HWARP_COARSE * b;
}
__device__ float2 streak_coords(float2 p, float2 dir) {
  const float2 n = v2(-dir.y, dir.x);
  return v2(dot2(p, n), dot2(p, dir));
}
__device__ __noinline__ float granulation(float2 p) {
  return 0.6f * vnoise(p / GRAIN_SCALE) + 0.3f * vnoise(p / (GRAIN_SCALE * 0.41f) + v2(7.3f, 2.1f)) +
         0.1f * vnoise(p / (GRAIN_SCALE * 3.7f) + v2(1.7f, 9.2f));
}
// render.wgsl:269-281
__device__ __noinline__ bool near_paint(const R& X, float2 p) {
  const int tw = (int)((X.cam.size[0] + 15u) / 16u), th = (int)((X.cam.size[1] + 15u) / 16u);
  const float s = X.cam.canvas[2] * 16.0f;
  const int gx = (int)floorf(p.x / s), gy = (int)floorf(p.y / s);
#pragma unroll 1
  for (int dj = -2; dj <= 2; ++dj)
#pragma unroll 1
    for (int di = -2; di <= 2; ++di) {
      const int x = gx + di, y = gy + dj;
      if (x >= 0 && y >= 0 && x < tw && y < th && (X.tile_flags[x + y * tw] & 1u) != 0u) return true;
    }
  return false;
}

// ---- the relief (render.wgsl:305-406)
__device__ __forceinline__ bool off_canvas(const R& X, float2 p) {
  return p.x < 0.0f || p.y < 0.0f || p.x > X.cam.canvas[0] || p.y > X.cam.canvas[1];
}
__device__ float surf_at(const R& X, int i, int j) {
  const int w = (int)X.cam.size[0], hh = (int)X.cam.size[1];
  const uint32_t ii = (uint32_t)min(max(i, 0), w - 1), jj = (uint32_t)min(max(j, 0), hh - 1);
  const uint32_t c = jj * X.cam.size[0] + ii;
  return X.h[c] + X.m[c];
}
__device__ float wet_at(const R& X, int i, int j) {
  const int w = (int)X.cam.size[0], hh = (int)X.cam.size[1];
  const uint32_t ii = (uint32_t)min(max(i, 0), w - 1), jj = (uint32_t)min(max(j, 0), hh - 1);
  return X.h[jj * X.cam.size[0] + ii];
}
__device__ __noinline__ float surf_bilinear(const R& X, float2 p) {
  if (off_canvas(X, p)) return 0.0f;
  const float2 g = p / X.cam.canvas[2] - v2(0.5f, 0.5f);
  const float2 f = floor2(g), t = g - f;
  const int i = (int)f.x, j = (int)f.y;
  const float a = surf_at(X, i, j), b = surf_at(X, i + 1, j), c = surf_at(X, i, j + 1), d = surf_at(X, i + 1, j + 1);
  return mixf(mixf(a, b, t.x), mixf(c, d, t.x), t.y);
}
__device__ float4 cr_w(float t) {
  const float t2 = t * t, t3 = t2 * t, u = 1.0f - t;
  return make_float4(u * u * u, 3.0f * t3 - 6.0f * t2 + 4.0f, -3.0f * t3 + 3.0f * t2 + 3.0f * t + 1.0f, t3) / 6.0f;
}
__device__ __noinline__ float surf_cubic(const R& X, float2 p) {
  if (off_canvas(X, p)) return 0.0f;
  const float2 g = p / X.cam.canvas[2] - v2(0.5f, 0.5f);
  const float2 f = floor2(g), t = g - f;
  const int i = (int)f.x, j = (int)f.y;
  const float4 wx = cr_w(t.x), wy = cr_w(t.y);
  float s = 0.0f;
  for (int b = -1; b <= 2; ++b) {
    float row = 0.0f;
    for (int a = -1; a <= 2; ++a) row += sel4(wx, a + 1) * surf_at(X, i + a, j + b);
    s += sel4(wy, b + 1) * row;
  }
  return fmaxf(s, 0.0f);
}
__device__ __noinline__ float wet_bilinear(const R& X, float2 p) {
  if (off_canvas(X, p)) return 0.0f;
  const float2 g = p / X.cam.canvas[2] - v2(0.5f, 0.5f);
  const float2 f = floor2(g), t = g - f;
  const int i = (int)f.x, j = (int)f.y;
  const float a = wet_at(X, i, j), b = wet_at(X, i + 1, j), c = wet_at(X, i, j + 1), d = wet_at(X, i + 1, j + 1);
  return mixf(mixf(a, b, t.x), mixf(c, d, t.x), t.y);
}

// ---- the detail texel and the tool micro-relief (render.wgsl:408-535)
struct Detail {
  float2 dir;
  float brush, knife, roller, cure, yield_pa, thickness;
};
__device__ float4 detail_texel(const R& X, int i, int j) {
  const int w = (int)X.cam.size[0], hh = (int)X.cam.size[1];
  float sc = X.cam.ortho[2];
  if (sc <= 0.0f) sc = 1.0f;
  const int ci = (int)floorf(((float)min(max(i, 0), w - 1) + 0.5f) * sc);
  const int cj = (int)floorf(((float)min(max(j, 0), hh - 1) + 0.5f) * sc);
  return f16x4(X.detail[(uint32_t)cj * X.cam.size[0] + (uint32_t)ci]);
}
__device__ __noinline__ Detail detail_params(const R& X, float2 p) {
  const float2 g = p / X.cam.canvas[2] - v2(0.5f, 0.5f);
  const float2 f = floor2(g), t = g - f;
  const int i = (int)f.x, j = (int)f.y;
  const float wts[4] = {(1.0f - t.x) * (1.0f - t.y), t.x * (1.0f - t.y), (1.0f - t.x) * t.y, t.x * t.y};
  Detail d;
  float2 dir = v2(0.0f, 0.0f);
  d.brush = d.knife = d.roller = d.cure = d.yield_pa = d.thickness = 0.0f;
  for (int k = 0; k < 4; ++k) {
    const float4 a = detail_texel(X, i + (k & 1), j + (k >> 1));
    const float wk = wts[k];
    const float method = floorf(a.x);
    const float ang = (fractf(a.x) - 0.5f) * TAU;
    dir = dir + wk * v2(o_cosf(ang), o_sinf(ang));
    d.brush += wk * (fabsf(method - METHOD_BRUSH) < 0.5f ? 1.0f : 0.0f);
    d.knife += wk * (fabsf(method - METHOD_KNIFE) < 0.5f ? 1.0f : 0.0f);
    d.roller += wk * (fabsf(method - METHOD_ROLLER) < 0.5f ? 1.0f : 0.0f);
    d.cure += wk * a.y;
    d.yield_pa += wk * a.z;
    d.thickness += wk * a.w;
  }
  d.dir = len2(dir) < 1e-4f ? v2(1.0f, 0.0f) : nrm2(dir);
  return d;
}
__device__ __noinline__ float groove_profile(float across, float along, float spacing) {
  const float k = TAU / spacing;
  const float drift = 0.6f * o_sinf(along * TAU / 0.021f);
  const float drift2 = 0.4f * o_sinf(along * TAU / 0.013f + 1.7f);
  return 0.5f * o_cosf(across * k + drift) + 0.3f * o_cosf(across * k * 1.62f + drift2 + 2.1f) +
         0.2f * o_cosf(across * k * 0.57f + 0.5f * drift);
}
__device__ __noinline__ float wrinkle_profile(float2 p, float wavelength) {
  const float k = TAU / wavelength;
  const float q1 = dot2(p, v2(0.93f, 0.37f)) * k * 0.13f;
  const float q2 = dot2(p, v2(-0.21f, 0.98f)) * k * 0.11f;
  const float q3 = dot2(p, v2(0.6f, -0.8f)) * k * 0.17f;
  const float ph1 = 2.4f * o_sinf(q2) + 1.1f * o_sinf(q3 + 1.0f);
  const float ph2 = 2.4f * o_sinf(q3) + 1.1f * o_sinf(q1 + 2.0f);
  const float ph3 = 2.4f * o_sinf(q1) + 1.1f * o_sinf(q2 + 3.0f);
  const float2 d0 = v2(1.0f, 0.0f), d1 = v2(0.5f, 0.8660254f), d2 = v2(-0.5f, 0.8660254f);
  const float s = o_cosf(dot2(p, d0) * k + ph1) + o_cosf(dot2(p, d1) * k + ph2) + o_cosf(dot2(p, d2) * k + ph3);
  const float patches = 0.6f + 0.4f * o_sinf(q1 * 0.7f + 1.0f) * o_sinf(q2 * 0.8f);
  return s / 3.0f * patches;
}
__device__ float groove_depth(float nominal, float spacing, float yield_pa, float footprint) {
  const float k = TAU / spacing;
  const float held = yield_pa / (SIGMA_PAINT * k * k);
  const float resolved = 1.0f - sstep(0.2f, 0.5f, footprint / spacing);
  return fminf(nominal, held) * resolved;
}
__device__ __noinline__ float micro(const R& X, float2 p, const Detail& d) {
  const float footprint = X.cam.jitter[3];
  if (footprint >= 0.5f * WRINKLE_WAVELENGTH) return 0.0f;
  const float hp = d.thickness;
  if (hp <= 2e-5f) return canvas_bump(p) * (1.0f - sstep(0.0f, 0.5f * WRINKLE_WAVELENGTH, footprint));
  const float across = dot2(p, v2(-d.dir.y, d.dir.x));
  const float along = dot2(p, d.dir);
  const float carry = fminf(hp / GROOVE_FULL_DEPTH_AT, 1.0f);
  float z = 0.0f;
  if (d.brush > 0.0f)
    z += d.brush * groove_depth(BRISTLE_DEPTH, BRISTLE_SPACING, d.yield_pa, footprint) * carry *
         groove_profile(across, along, BRISTLE_SPACING);
  if (d.knife > 0.0f)
    z += d.knife * groove_depth(KNIFE_DEPTH, KNIFE_SPACING, d.yield_pa, footprint) * carry *
         groove_profile(across, along, KNIFE_SPACING);
  if (d.roller > 0.0f) {
    const float resolved = 1.0f - sstep(0.2f, 0.6f, footprint / ROLLER_STIPPLE_SCALE);
    const float peel = fbm_filtered(X, v2(across, along / ROLLER_STIPPLE_STRETCH), ROLLER_STIPPLE_SCALE, 3);
    z += d.roller * ROLLER_STIPPLE_DEPTH * fminf(hp / 4e-5f, 1.0f) * resolved * peel;
  }
  const float skin = d.cure * sstep(0.5e-3f, 1.5e-3f, hp) * (1.0f - sstep(0.2f, 0.5f, footprint / WRINKLE_WAVELENGTH));
  if (skin > 0.0f) z += WRINKLE_HEIGHT * skin * wrinkle_profile(p, WRINKLE_WAVELENGTH);
  if (X.beauty()) {
    z += canvas_bump_levelled(p, hp) * (1.0f - sstep(0.0f, 0.5f * WRINKLE_WAVELENGTH, footprint));
    const float amp = clampf(IMPASTO_FRACTION * hp, 1.0e-6f, IMPASTO_MAX) * mixf(0.45f, 1.0f, d.cure);
    const float tool = clampf(d.brush + d.knife, 0.0f, 1.0f);
    const float2 sc = streak_coords(p, d.dir);
    const float aniso = fbm_filtered(X, v2(sc.x / 0.6f, sc.y / 3.0f), 0.25e-3f, 4);
    const float iso = fbm_filtered(X, p, 0.35e-3f, 4);
    z += amp * mixf(iso, aniso, 0.35f + 0.65f * tool);
    const float clump = fbm_filtered(X, v2(sc.x, sc.y / CLUMP_ELONGATION), CLUMP_WIDTH, 4);
    z += tool * carry * CLUMP_DEPTH * clump;
    const float pin_fade = sstep(0.08e-3f, 0.3e-3f, hp) * (1.0f - sstep(0.02e-3f, 0.06e-3f, footprint));
    if (pin_fade > 0.0f) z += pin_fade * pinholes(p, hp);
  }
  return z;
}
__device__ __noinline__ float2 micro_slope(const R& X, float2 p, const Detail& d) {
  const float e = 0.06f * X.cam.canvas[2];
  const float mx = micro(X, p + v2(e, 0.0f), d) - micro(X, p - v2(e, 0.0f), d);
  const float my = micro(X, p + v2(0.0f, e), d) - micro(X, p - v2(0.0f, e), d);
  return v2(mx, my) / (2.0f * e);
}
// render.wgsl:537-553
__device__ __noinline__ float edge_factor(const R& X, float2 p) {
  const float2 g = p / X.cam.canvas[2] - v2(0.5f, 0.5f);
  const float2 f = floor2(g);
  const int i = (int)f.x, j = (int)f.y;
  float hmax = 0.0f, hmin = 1e9f;
#pragma unroll 1
  for (int b = -1; b <= 2; ++b)
    for (int a = -1; a <= 2; ++a) {
      const float v = wet_at(X, i + a, j + b);
      hmax = fmaxf(hmax, v);
      hmin = fminf(hmin, v);
    }
  if (hmax <= 1e-6f) return 0.0f;
  return sstep(0.3f, 0.8f, 1.0f - hmin / hmax);
}
// render.wgsl:555-616: the relief smoothed by a Gaussian with the meniscus
// capped at the contact angle (beauty mode)
__device__ __noinline__ float surf_smooth(const R& X, float2 p) {
  if (off_canvas(X, p)) return 0.0f;
  const float dx = X.cam.canvas[2];
  const float2 g = p / dx - v2(0.5f, 0.5f);
  const float2 f = floor2(g), t = g - f;
  const int i = (int)f.x, j = (int)f.y;
  const float sig2 = 0.45f;
  float wx[6], wy[6], dwx[6], dwy[6];
  float nx = 0.0f, ny = 0.0f, dnx = 0.0f, dny = 0.0f;
  for (int a = 0; a < 6; ++a) {
    const float da = (float)(a - 2) - t.x, db = (float)(a - 2) - t.y;
    wx[a] = o_expf(-da * da / (2.0f * sig2));
    wy[a] = o_expf(-db * db / (2.0f * sig2));
    dwx[a] = wx[a] * da / sig2;
    dwy[a] = wy[a] * db / sig2;
    nx += wx[a];
    ny += wy[a];
    dnx += dwx[a];
    dny += dwy[a];
  }
  float num = 0.0f, num2 = 0.0f, dnumx = 0.0f, dnumy = 0.0f;
  for (int b = 0; b < 6; ++b) {
    float row = 0.0f, row2 = 0.0f, drow = 0.0f;
    for (int a = 0; a < 6; ++a) {
      const float sv = surf_at(X, i + a - 2, j + b - 2);
      row += wx[a] * sv;
      row2 += wx[a] * sv * sv;
      drow += dwx[a] * sv;
    }
    num += wy[b] * row;
    num2 += wy[b] * row2;
    dnumx += wy[b] * drow;
    dnumy += dwy[b] * row;
  }
  const float nn = nx * ny;
  const float hb = num / nn;
  if (hb <= 1e-7f) return fmaxf(hb, 0.0f);
  const float hin = fmaxf(num2 / fmaxf(num, 1e-12f), hb);
  const float gx = (dnumx * nx - num * dnx) / (nx * nn);
  const float gy = (dnumy * ny - num * dny) / (ny * nn);
  const float gm = fmaxf(len2(v2(gx, gy)) / dx, 1e-3f);
  const float d = (hb - 0.35f * hin) / gm;
  if (d <= 0.0f) return 0.0f;
  const float lc = 2.0e-3f;
  const float scale = fminf(hin, 2.0f * lc);
  const float cap = hin * tanhf(d * X.cam.ortho[1] / scale);
  return fminf(hb, cap);
}
// render.wgsl:618-642
__device__ __noinline__ float surf_march(const R& X, float2 p) {
  if (X.beauty()) return surf_cubic(X, hwarp(X, p));
  return surf_bilinear(X, p);
}
__device__ __noinline__ float surf_hit(const R& X, float2 p, const Detail& d) {
  if (X.beauty()) return surf_smooth(X, hwarp(X, p)) + micro(X, p, d);
  return surf_bilinear(X, p) + micro(X, p, d);
}
__device__ __noinline__ float2 base_slope(const R& X, float2 p) {
  const float e = 0.7f * X.cam.canvas[2];
  if (X.beauty()) {
    const float sx = surf_smooth(X, hwarp(X, p + v2(e, 0.0f))) - surf_smooth(X, hwarp(X, p - v2(e, 0.0f)));
    const float sy = surf_smooth(X, hwarp(X, p + v2(0.0f, e))) - surf_smooth(X, hwarp(X, p - v2(0.0f, e)));
    return v2(sx, sy) / (2.0f * e);
  }
  const float sx = surf_cubic(X, p + v2(e, 0.0f)) - surf_cubic(X, p - v2(e, 0.0f));
  const float sy = surf_cubic(X, p + v2(0.0f, e)) - surf_cubic(X, p - v2(0.0f, e));
  return v2(sx, sy) / (2.0f * e);
}
__device__ float3 normal_from_slope(float2 s) { return nrm3(v3(-s.x, -s.y, 1.0f)); }
__device__ __noinline__ float3 normal_bilinear(const R& X, float2 p) {
  const float e = 0.7f * X.cam.canvas[2];
  const float sx = surf_bilinear(X, p + v2(e, 0.0f)) - surf_bilinear(X, p - v2(e, 0.0f));
  const float sy = surf_bilinear(X, p + v2(0.0f, e)) - surf_bilinear(X, p - v2(0.0f, e));
  return nrm3(v3(-sx / (2.0f * e), -sy / (2.0f * e), 1.0f));
}

// ---- colour (render.wgsl:644-844)
__device__ float4 col_at(const R& X, int i, int j) {
  const int w = (int)X.cam.size[0], hh = (int)X.cam.size[1];
  float sc = X.cam.ortho[2];
  if (sc <= 0.0f) sc = 1.0f;
  const int ci = (int)floorf(((float)min(max(i, 0), w - 1) + 0.5f) * sc);
  const int cj = (int)floorf(((float)min(max(j, 0), hh - 1) + 0.5f) * sc);
  return f16x4(X.color[(uint32_t)cj * X.cam.size[0] + (uint32_t)ci]);
}
__device__ float4 coarse_col(const R& X, int i, int j) {
  const int w = (int)X.cam.size[0], hh = (int)X.cam.size[1];  // the colour plane has the film's size
  return f16x4(X.color[(uint32_t)min(max(j, 0), hh - 1) * X.cam.size[0] + (uint32_t)min(max(i, 0), w - 1)]);
}
__device__ float crisp_t(float t) {
  const float a = o_powf(t, COLOR_CRISP);
  return a / (a + o_powf(1.0f - t, COLOR_CRISP));
}
__device__ __noinline__ float4 color_crisp(const R& X, float2 p) {
  float sc = X.cam.ortho[2];
  if (sc <= 0.0f) sc = 1.0f;
  const float cdx = X.cam.canvas[2] / sc;
  const float2 g = p / cdx - v2(0.5f, 0.5f);
  const float2 f = floor2(g), t = g - f;
  const int i = (int)f.x, j = (int)f.y;
  const float tx = crisp_t(t.x), ty = crisp_t(t.y);
  const float4 a = coarse_col(X, i, j), b = coarse_col(X, i + 1, j), c = coarse_col(X, i, j + 1),
               d = coarse_col(X, i + 1, j + 1);
  return mix4(mix4(a, b, tx), mix4(c, d, tx), ty);
}
__device__ __noinline__ float4 color_beauty(const R& X, float2 p) {
  float sc = X.cam.ortho[2];
  if (sc <= 0.0f) sc = 1.0f;
  const float cdx = X.cam.canvas[2] / sc;
  const float2 g = p / cdx - v2(0.5f, 0.5f);
  const float2 f = floor2(g), t = g - f;
  const int i = (int)f.x, j = (int)f.y;
  float hs[16];
  float hmin = 1e9f, hmax = 0.0f;
  for (int k = 0; k < 16; ++k) {
    const int a = k % 4 - 1, b = k / 4 - 1;
    const float2 centre = (v2((float)(i + a), (float)(j + b)) + v2(0.5f, 0.5f)) * cdx;
    const float hv = surf_bilinear(X, centre);
    hs[k] = hv;
    hmin = fminf(hmin, hv);
    hmax = fmaxf(hmax, hv);
  }
  const float4 crisp = color_crisp(X, p);
  if (hmax <= 1e-7f) return crisp;
  const float range = hmax - hmin;
  const float edge = sstep(0.3f, 0.6f, range / hmax) * sstep(EDGE_MIN_STEP, 2.0f * EDGE_MIN_STEP, range);
  if (edge <= 0.0f) return crisp;
  const float4 wx = cr_w(t.x), wy = cr_w(t.y);
  float4 cin = make_float4(0.f, 0.f, 0.f, 0.f), cout = cin;
  float win = 1e-12f, wout = 1e-12f;
  for (int k = 0; k < 16; ++k) {
    const int a = k % 4, b = k / 4;
    const float w = sel4(wx, a) * sel4(wy, b) + 0.02f;
    const float rel = (hs[k] - hmin) / range;
    const float4 c = coarse_col(X, i + a - 1, j + b - 1);
    const float w_in = w * rel * rel * rel;
    const float w_out = w * (1.0f - rel) * (1.0f - rel) * (1.0f - rel);
    cin = cin + w_in * c;
    cout = cout + w_out * c;
    win += w_in;
    wout += w_out;
  }
  cin = cin / win;
  cout = cout / wout;
  const float hb = (surf_cubic(X, p) - hmin) / range;
  const float s = sstep(EDGE_ISO - EDGE_ISO_SOFT, EDGE_ISO + EDGE_ISO_SOFT, hb);
  return mix4(crisp, mix4(cout, cin, s), edge);
}
__device__ __noinline__ float4 color_sharp(const R& X, float2 p) {
  if (X.beauty()) return color_beauty(X, p);
  const float2 g = p / X.cam.canvas[2] - v2(0.5f, 0.5f);
  const float2 f = floor2(g), t = g - f;
  const int i = (int)f.x, j = (int)f.y;
  const float4 wb = make_float4((1.0f - t.x) * (1.0f - t.y), t.x * (1.0f - t.y), (1.0f - t.x) * t.y, t.x * t.y);
  const float4 hw = make_float4(wet_at(X, i, j), wet_at(X, i + 1, j), wet_at(X, i, j + 1), wet_at(X, i + 1, j + 1));
  const float4 c0 = col_at(X, i, j), c1 = col_at(X, i + 1, j), c2 = col_at(X, i, j + 1), c3 = col_at(X, i + 1, j + 1);
  const float4 cbil = wb.x * c0 + wb.y * c1 + wb.z * c2 + wb.w * c3;
  const float hmax = fmaxf(fmaxf(hw.x, hw.y), fmaxf(hw.z, hw.w));
  const float hmin = fminf(fminf(hw.x, hw.y), fminf(hw.z, hw.w));
  if (hmax <= 1e-6f) return cbil;
  const float e = 1.0f - hmin / hmax;
  const float edge = sstep(0.3f, 0.6f, e);
  if (edge <= 0.0f) return cbil;
  const float4 wx = cr_w(t.x), wy = cr_w(t.y);
  float hb = 0.0f, hb2 = 0.0f;
#pragma unroll 1
  for (int b = -1; b <= 2; ++b)
    for (int a = -1; a <= 2; ++a) {
      const float wv = sel4(wx, a + 1) * sel4(wy, b + 1);
      const float hv = wet_at(X, i + a, j + b);
      hb += wv * hv;
      hb2 += wv * hv * hv;
    }
  hb = fmaxf(hb, 0.0f);
  const float hin = hb2 / fmaxf(hb, 1e-9f);
  const float4 win = make_float4(wb.x * hw.x, wb.y * hw.y, wb.z * hw.z, wb.w * hw.w);
  const float4 wout = make_float4(wb.x * (hmax - hw.x), wb.y * (hmax - hw.y), wb.z * (hmax - hw.z), wb.w * (hmax - hw.w));
  const float sin_ = fmaxf(win.x + win.y + win.z + win.w, 1e-12f);
  const float sout = fmaxf(wout.x + wout.y + wout.z + wout.w, 1e-12f);
  const float4 cin = (win.x * c0 + win.y * c1 + win.z * c2 + win.w * c3) / sin_;
  const float4 cout = (wout.x * c0 + wout.y * c1 + wout.z * c2 + wout.w * c3) / sout;
  const float s = sstep(0.25f, 0.45f, hb / fmaxf(hin, 1e-9f));
  const float4 cedge = mix4(cout, cin, s);
  const float4 r = mix4(cbil, cedge, edge);
  return make_float4(r.x, r.y, r.z, cbil.w);
}
__device__ __noinline__ float2 cwarp(const R& X, float2 p, const Detail& d) {
  const float2 q = hwarp(X, p);
  if (!X.beauty()) return q;
  const float free_ = 1.0f - edge_factor(X, q);
  const float2 sc = streak_coords(p, d.dir);
  const float streak = fbm(v2(sc.x / STREAK_WIDTH, sc.y / STREAK_LENGTH), 4);
  const float2 n = v2(-d.dir.y, d.dir.x);
  const float tool = clampf(d.brush + d.knife, 0.0f, 1.0f);
  const float2 iso = v2(fbm(p / 1.3e-3f + v2(4.1f, 8.3f), 4), fbm(p / 1.3e-3f + v2(1.9f, 6.6f), 4));
  return q + free_ * (n * streak * CWARP_STREAK * (0.35f + 0.65f * tool) + iso * CWARP_ISO);
}
// the colour plane through the renderer's sampler (linear filtering,
// clamp-to-edge, one level): the blend of the 4 texels around uv * size - 0.5
__device__ __noinline__ float4 sample_color(const R& X, float2 uv) {
  const int w = (int)X.cam.size[0], h = (int)X.cam.size[1];
  const float gx = uv.x * (float)w - 0.5f, gy = uv.y * (float)h - 0.5f;
  const float fx = floorf(gx), fy = floorf(gy);
  const float ax = gx - fx, ay = gy - fy;
  const int i0 = (int)fx, j0 = (int)fy;
  auto at = [&](int i, int j) {
    i = min(max(i, 0), w - 1);
    j = min(max(j, 0), h - 1);
    return f16x4(X.color[(uint32_t)j * X.cam.size[0] + (uint32_t)i]);
  };
  return (at(i0, j0) * (1.0f - ax) + at(i0 + 1, j0) * ax) * (1.0f - ay) +
         (at(i0, j0 + 1) * (1.0f - ax) + at(i0 + 1, j0 + 1) * ax) * ay;
}
__device__ __noinline__ float3 marble(const R& X, float2 p, float3 c, const Detail& d) {
  const float2 inv = v2(1.0f / X.cam.canvas[0], 1.0f / X.cam.canvas[1]);
  float3 mean = c;
  float3 cols[16];
  for (int k = 0; k < 16; ++k) {
    const float ring = k >= 8 ? MARBLE_R2 : MARBLE_R1;
    const float ang = ((float)k + (k >= 8 ? 0.5f : 0.0f)) * TAU / 8.0f;
    const float2 q = p + v2(o_cosf(ang), o_sinf(ang)) * ring;
    cols[k] = rgb(sample_color(X, q * inv));
    mean = mean + cols[k];
  }
  mean = mean / 17.0f;
  float spread = 1e-6f;
  for (int k = 0; k < 16; ++k) spread = fmaxf(spread, dot3(cols[k] - mean, cols[k] - mean));
  float3 a = v3(0.0f, 0.0f, 0.0f);
  float wa = 0.0f;
  for (int k = 0; k < 16; ++k) {
    const float w = o_expf(MARBLE_SELECT * (dot3(cols[k] - mean, cols[k] - mean) / spread - 1.0f));
    a = a + w * cols[k];
    wa += w;
  }
  a = a / wa;
  float spread_a = 1e-6f;
  for (int k = 0; k < 16; ++k) spread_a = fmaxf(spread_a, dot3(cols[k] - a, cols[k] - a));
  float3 b = v3(0.0f, 0.0f, 0.0f);
  float wb = 0.0f;
  for (int k = 0; k < 16; ++k) {
    const float w = o_expf(MARBLE_SELECT * (dot3(cols[k] - a, cols[k] - a) / spread_a - 1.0f));
    b = b + w * cols[k];
    wb += w;
  }
  b = b / wb;
  const float3 ab = b - a;
  const float l2 = dot3(ab, ab);
  if (l2 < MARBLE_MIN_CONTRAST * MARBLE_MIN_CONTRAST) return c;
  const float f = clampf(dot3(c - a, ab) / l2, 0.0f, 1.0f);
  const float3 resid = c - (a + ab * f);
  const float on_line = 1.0f - sstep(0.08f, 0.25f, len3(resid) / sqrtf(l2));
  const float2 scp = streak_coords(p, d.dir);
  const float tool = clampf(d.brush + d.knife, 0.0f, 1.0f);
  const float n_iso = fbm(p / MARBLE_SCALE + v2(2.3f, 7.7f), 5);
  const float n_str = fbm(v2(scp.x / (0.35f * MARBLE_SCALE), scp.y / (4.0f * MARBLE_SCALE)), 5);
  const float n = mixf(n_iso, n_str, 0.4f + 0.6f * tool);
  const float thr = 0.5f + 0.55f * n;
  const float soft = MARBLE_SOFT + 0.6f * X.cam.jitter[3] / MARBLE_SCALE;
  const float fs = sstep(thr - soft, thr + soft, f);
  const float fm = mixf(f, fs, MARBLE_STRENGTH * on_line);
  const float3 r = a + ab * fm + resid;
  return v3(fmaxf(r.x, 0.0f), fmaxf(r.y, 0.0f), fmaxf(r.z, 0.0f));
}

// ---- light (render.wgsl:846-983)
__device__ __noinline__ float shadow_at(const R& X, float2 p, float z0, float3 l) {
  if (l.z <= 0.05f) return 1.0f;
  const float step = X.cam.canvas[2] * 1.5f;
  float spread = tanf(KEY_HALF_ANGLE), zstart = z0;
  if (X.beauty()) {
    spread = BEAUTY_PENUMBRA;
    zstart = fmaxf(z0, surf_march(X, p)) + SHADOW_BIAS;
  }
  float sh = 1.0f;
#pragma unroll 1
  for (int k = 1; k <= 20; ++k) {
    const float d = (float)k * step;
    const float2 q = p + v2(l.x, l.y) / l.z * d;
    const float zs = surf_march(X, q);
    const float zr = zstart + d;
    if (zr > X.cam.canvas[3]) break;
    const float penumbra = d * spread / l.z + 0.5f * step;
    sh = fminf(sh, 1.0f - clampf((zs - zr) / penumbra, 0.0f, 1.0f));
  }
  return sh;
}
__device__ __noinline__ float ambient_occlusion(const R& X, float2 p, float z0, const Detail& d) {
  const float step = X.cam.canvas[2] * 2.0f;
  float open = 0.0f;
#pragma unroll 1
  for (int k = 0; k < AO_DIRS; ++k) {
    const float ang = ((float)k + 0.5f) * TAU / (float)AO_DIRS;
    const float2 dir = v2(o_cosf(ang), o_sinf(ang));
    float horizon = 0.0f;
#pragma unroll 1
    for (int i = 1; i <= AO_STEPS; ++i) {
      const float dist = (float)i * step;
      const float rise = surf_hit(X, p + dir * dist, d) - z0;
      horizon = fmaxf(horizon, rise / dist);
    }
    open += 1.0f - horizon / sqrtf(1.0f + horizon * horizon);
  }
  return open / (float)AO_DIRS;
}
__device__ __noinline__ float softbox(float3 dir, float3 l, float rough, float hw, float hh) {
  const float3 side = nrm3(cross3(v3(0.0f, 0.0f, 1.0f), l));
  const float3 upv = cross3(l, side);
  const float cos_l = dot3(dir, l);
  if (cos_l <= 0.0f) return 0.0f;
  const float u = atan2f(dot3(dir, side), cos_l);
  const float v = atan2f(dot3(dir, upv), cos_l);
  const float edge = 0.03f + 0.7f * rough;
  const float inside = (1.0f - sstep(hw - edge, hw + edge, fabsf(u))) * (1.0f - sstep(hh - edge, hh + edge, fabsf(v)));
  const float fill = (hw * hh) / ((hw + edge) * (hh + edge));
  return inside * fill;
}
__device__ __noinline__ float3 env_radiance(const R& X, float3 dir, float rough) {
  const float3 sky = v3(X.cam.sky[0], X.cam.sky[1], X.cam.sky[2]);
  const float3 ground = v3(X.cam.ground[0], X.cam.ground[1], X.cam.ground[2]);
  const float soft = 0.08f + 0.9f * rough;
  const float up = sstep(-soft, soft, dir.z);
  const float band = o_expf(-fabsf(dir.z) / (0.12f + 0.6f * rough));
  float zenith = 1.0f;
  if (X.beauty()) zenith = mixf(1.0f, ZENITH_DIM, sstep(0.2f, 0.9f, dir.z) * (1.0f - rough));
  float3 e = mix3(ground, sky * zenith, up) + horizon_glow() * 0.5f * band;
  const float3 l = nrm3(v3(X.cam.light[0], X.cam.light[1], X.cam.light[2]));
  const float box_scale = X.beauty() ? BEAUTY_SOFTBOX_SCALE : 1.0f;
  const float box_radiance = X.beauty() ? BEAUTY_SOFTBOX_RADIANCE * X.cam.light[3] / PI
                                        : SOFTBOX_RADIANCE * X.cam.light[3] / 2.6f;
  e = e + softbox(dir, l, rough, SOFTBOX_HALF_W * box_scale, SOFTBOX_HALF_H * box_scale) *
              v3(box_radiance, box_radiance, box_radiance);
  const float3 lf = nrm3(v3(-l.x * 0.9f, -l.y * 0.9f, fmaxf(l.z * 0.7f, 0.25f)));
  e = e + softbox(dir, lf, rough, SOFTBOX_HALF_W * 1.4f, SOFTBOX_HALF_H * 1.6f) * fill_tint() *
              (FILL_RADIANCE * SOFTBOX_RADIANCE * X.cam.light[3] / 2.6f);
  return e;
}
__device__ float d_ggx_aniso(float3 n, float3 t, float3 b, float3 hvec, float at, float ab) {
  const float th = dot3(t, hvec) / at, bh = dot3(b, hvec) / ab, nh = dot3(n, hvec);
  const float d = th * th + bh * bh + nh * nh;
  return 1.0f / (PI * at * ab * d * d);
}
__device__ float d_ggx(float ndh, float a2) {
  const float d = ndh * ndh * (a2 - 1.0f) + 1.0f;
  return a2 / (PI * d * d);
}
__device__ float v_smith(float ndv, float ndl, float a2) {
  const float gv = ndl * sqrtf(ndv * ndv * (1.0f - a2) + a2);
  const float gl = ndv * sqrtf(ndl * ndl * (1.0f - a2) + a2);
  return 0.5f / fmaxf(gv + gl, 1e-5f);
}
__device__ __noinline__ float spec_lobe(const R& X, float3 n, float3 v, float3 l, float rough, float f0) {
  const float3 hvec = nrm3(v + l);
  const float a = fmaxf(rough * rough, 0.002f);
  const float a_wide = X.beauty() ? fmaxf(a, BEAUTY_MIN_ALPHA) : fminf(a + o_sinf(KEY_HALF_ANGLE), 1.0f);
  const float a2 = a_wide * a_wide;
  const float ndh = fmaxf(dot3(n, hvec), 0.0f), ndv = fmaxf(dot3(n, v), 1e-3f), ndl = fmaxf(dot3(n, l), 0.0f);
  const float f = f0 + (1.0f - f0) * o_powf(1.0f - fmaxf(dot3(v, hvec), 0.0f), 5.0f);
  return d_ggx(ndh, a2) * v_smith(ndv, ndl, a_wide * a_wide) * f;
}
__device__ __noinline__ float spec_lobe_aniso(const R& X, float3 n, float3 v, float3 l, float rough, float f0, float aniso,
                                 float2 tdir) {
  if (aniso <= 0.01f) return spec_lobe(X, n, v, l, rough, f0);
  const float3 hvec = nrm3(v + l);
  const float a = fmaxf(rough * rough, 0.002f);
  const float a_wide = X.beauty() ? fmaxf(a, BEAUTY_MIN_ALPHA) : fminf(a + o_sinf(KEY_HALF_ANGLE), 1.0f);
  float3 t = v3(tdir.x, tdir.y, 0.0f);
  t = nrm3(t - n * dot3(t, n));
  const float3 b = cross3(n, t);
  const float at = fmaxf(a_wide * (1.0f - 0.6f * aniso), 0.002f);
  const float ab = fminf(a_wide * (1.0f + 1.2f * aniso), 1.0f);
  const float ndv = fmaxf(dot3(n, v), 1e-3f), ndl = fmaxf(dot3(n, l), 0.0f);
  const float f = f0 + (1.0f - f0) * o_powf(1.0f - fmaxf(dot3(v, hvec), 0.0f), 5.0f);
  const float a2 = at * ab;
  return d_ggx_aniso(n, t, b, hvec, at, ab) * v_smith(ndv, ndl, a2) * f;
}
__device__ float env_dfg(float f0, float rough, float ndv) {
  const float4 c0 = make_float4(-1.0f, -0.0275f, -0.572f, 0.022f), c1 = make_float4(1.0f, 0.0425f, 1.04f, -0.04f);
  const float4 r = rough * c0 + c1;
  const float a004 = fminf(r.x * r.x, exp2f(-9.28f * ndv)) * r.x + r.y;
  const float scale = a004 * -1.04f + r.z;
  const float bias = a004 * 1.04f + r.w;
  return f0 * scale + bias;
}
__device__ float3 tonemap(float3 c) {
  const float a = 2.51f, b = 0.03f, cc = 2.43f, d = 0.59f, e = 0.14f;
  auto one = [&](float x) { return clampf((x * (a * x + b)) / (x * (cc * x + d) + e), 0.0f, 1.0f); };
  return v3(one(c.x), one(c.y), one(c.z));
}
__device__ float3 to_srgb(float3 c) {
  auto one = [](float x) { return x <= 0.0031308f ? x * 12.92f : 1.055f * o_powf(x, 1.0f / 2.4f) - 0.055f; };
  return v3(one(c.x), one(c.y), one(c.z));
}
__device__ float3 reflect3(float3 i, float3 n) { return i - 2.0f * dot3(n, i) * n; }
__device__ __noinline__ float3 lit(const R& X, float3 n, float3 v, float3 l, float sh, float ao, float3 albedo, float rough,
                      float cure, float coat, float aniso, float2 tdir, float falloff) {
  const float ndl = fmaxf(dot3(n, l), 0.0f);
  const float ndv = fmaxf(dot3(n, v), 1e-3f);
  const float sun = X.cam.light[3] * falloff;
  const float f_env = env_dfg(F0_PAINT, rough, ndv);
  const float kd = 1.0f - f_env;
  const float3 ambient = env_radiance(X, n, 1.0f) * ao;
  const float lambert = X.beauty() ? 1.0f / PI : 1.0f;
  const float3 diffuse = albedo * kd * (v3(sun * ndl * sh * lambert, sun * ndl * sh * lambert, sun * ndl * sh * lambert) + ambient);
  float spec = spec_lobe_aniso(X, n, v, l, rough, F0_PAINT, aniso, tdir);
  spec += 0.35f * cure * spec_lobe(X, n, v, l, fmaxf(rough, 0.55f), F0_PAINT);
  const float direct = spec * sun * ndl * sh;
  const float3 rv = reflect3(-v, n);
  const float occlusion = clampf(o_powf(ndv + ao, exp2f(-16.0f * rough - 1.0f)) - 1.0f + ao, 0.0f, 1.0f);
  const float3 env = env_radiance(X, rv, rough) * f_env * occlusion;
  const float base_spec = X.beauty() ? 1.0f - coat : 1.0f;
  float3 c = diffuse + (v3(direct, direct, direct) + env) * base_spec;
  if (coat > 0.0f) {
    const float fc = env_dfg(F0_PAINT, COAT_ROUGH, ndv);
    const float coat_direct = spec_lobe(X, n, v, l, COAT_ROUGH, F0_PAINT) * sun * ndl * sh;
    const float occ_c = clampf(o_powf(ndv + ao, exp2f(-16.0f * COAT_ROUGH - 1.0f)) - 1.0f + ao, 0.0f, 1.0f);
    const float3 coat_env = env_radiance(X, rv, COAT_ROUGH) * fc * occ_c;
    c = c * (1.0f - coat * fc) + coat * (v3(coat_direct, coat_direct, coat_direct) + coat_env);
  }
  return c;
}
__device__ float3 mat_ray(const cf_render_cam& cam, float x, float y, float z) {  // (inv_vp * (x, y, z, 1)).xyz / w
  float r[4];
  for (int k = 0; k < 4; ++k) r[k] = cam.inv_vp[k] * x + cam.inv_vp[4 + k] * y + cam.inv_vp[8 + k] * z + cam.inv_vp[12 + k] * 1.0f;
  return v3(r[0], r[1], r[2]) / r[3];
}

// ---- the fragment (render.wgsl:985-1116)
__device__ float4 fs(const R& X, float2 ndc_in) {
  const float2 ndc = ndc_in + v2(X.cam.jitter[0], X.cam.jitter[1]);
  float3 a = mat_ray(X.cam, ndc.x, ndc.y, 0.0f);
  float3 dir = nrm3(mat_ray(X.cam, ndc.x, ndc.y, 1.0f) - a);
  if (X.cam.ortho[0] > 0.5f) {
    const float2 pxy = (ndc * 0.5f + v2(0.5f, 0.5f)) * v2(X.cam.canvas[0], X.cam.canvas[1]);
    a = v3(pxy.x, pxy.y, 1.0f);
    dir = v3(0.0f, 0.0f, -1.0f);
  } else if (X.cam.lens[3] > 0.5f) {
    const float3 br = v3(X.cam.basis_r[0], X.cam.basis_r[1], X.cam.basis_r[2]);
    const float3 bu = v3(X.cam.basis_u[0], X.cam.basis_u[1], X.cam.basis_u[2]);
    const float3 fwd = cross3(bu, br);
    const float fd = X.cam.lens[2] / fmaxf(dot3(dir, fwd), 1e-3f);
    const float3 fp = a + dir * fd;
    a = a + br * X.cam.lens[0] + bu * X.cam.lens[1];
    dir = nrm3(fp - a);
  }
  const float3 bg = mix3(v3(X.cam.ground[0], X.cam.ground[1], X.cam.ground[2]), v3(X.cam.sky[0], X.cam.sky[1], X.cam.sky[2]),
                         clampf(dir.z * 0.5f + 0.5f, 0.0f, 1.0f));
  if (fabsf(dir.z) < 1e-5f) { const float3 c = to_srgb(tonemap(bg)); return make_float4(c.x, c.y, c.z, 1.0f); }
  const float t1 = -a.z / dir.z;
  if (t1 < 0.0f) { const float3 c = to_srgb(tonemap(bg)); return make_float4(c.x, c.y, c.z, 1.0f); }
  const float top = X.cam.canvas[3];
  float t0 = 0.0f;
  if (a.z > top) t0 = (top - a.z) / dir.z;
  const float span = fmaxf(t1 - t0, 0.0f);
  const float horiz = span * len2(v2(dir.x, dir.y));
  const int nsteps = min(max((int)ceilf(horiz / X.cam.canvas[2]), 1), 96);
  const float step = span / (float)nsteps;
  float ta = t0, tb = t1;
  bool found = false;
#pragma unroll 1
  for (int k = 1; k <= nsteps; ++k) {
    const float tk = t0 + (float)k * step;
    const float3 q = a + dir * tk;
    if (q.z <= surf_march(X, v2(q.x, q.y))) {
      tb = tk;
      found = true;
      break;
    }
    ta = tk;
  }
  float t = t1;
  const float3 qb = a + dir * tb;
  const Detail detail = detail_params(X, v2(qb.x, qb.y));
  if (found) {
#pragma unroll 1
    for (int r = 0; r < 8; ++r) {
      const float tm = 0.5f * (ta + tb);
      const float3 q = a + dir * tm;
      if (q.z <= surf_hit(X, v2(q.x, q.y), detail)) tb = tm;
      else ta = tm;
    }
    t = tb;
  }
  const float3 hit = a + dir * t;
  const float2 p = v2(hit.x, hit.y);
  const float W = X.cam.canvas[0], H = X.cam.canvas[1];
  if (p.x < 0.0f || p.y < 0.0f || p.x > W || p.y > H) {
    const float3 c = to_srgb(tonemap(floor_color()));
    return make_float4(c.x, c.y, c.z, 1.0f);
  }
  const float3 v = -dir;
  const float3 l = nrm3(v3(X.cam.light[0], X.cam.light[1], X.cam.light[2]));
  if (!near_paint(X, p) && X.cam.jitter[2] <= 0.5f) {
    const float4 cs = color_sharp(X, p);
    const float3 c = to_srgb(tonemap(lit(X, normal_bilinear(X, p), v, l, 1.0f, 1.0f, rgb(cs), cs.w, 0.0f, 0.0f, 0.0f,
                                         v2(1.0f, 0.0f), 1.0f)));
    return make_float4(c.x, c.y, c.z, 1.0f);
  }
  const float2 ms = micro_slope(X, p, detail);
  const float3 n = normal_from_slope(base_slope(X, p) + ms);
  const float slope = len2(v2(n.x, n.y)) / fmaxf(n.z, 1e-3f);
  float2 pc = p;
  if (slope > 0.4f) {
    const float2 up = nrm2(v2(-n.x, -n.y));
    pc = p + up * X.cam.canvas[2] * (0.5f + clampf(slope, 0.0f, 3.0f) * 0.5f);
    pc = v2(clampf(pc.x, 0.0f, W), clampf(pc.y, 0.0f, H));
  }
  const float2 pcw = cwarp(X, pc, detail);
  float4 col = color_sharp(X, pcw);
  if (X.beauty() && detail.thickness > 0.02e-3f) {
    const float3 m = marble(X, pcw, rgb(col), detail);
    col = make_float4(m.x, m.y, m.z, col.w);
  }
  const float thin = 0.3f * (1.0f - sstep(0.0f, THIN_FILM_MATTE, detail.thickness)) * sstep(0.0f, 1e-5f, detail.thickness);
  float rough = clampf(col.w + 0.3f * len2(ms) + thin, 0.03f, 0.95f);
  if (X.beauty()) {
    const float paint_cover = sstep(0.0f, 0.08e-3f, detail.thickness);
    const float gloss = DRY_GLOSS_FLOOR + (col.w - DRY_GLOSS_FLOOR) * DRY_GLOSS_SCALE;
    const float patchy = 0.75f + 0.5f * (0.5f + 0.5f * fbm(p / 2.5e-3f + v2(6.1f, 2.4f), 3));
    rough = clampf(mixf(col.w, gloss * patchy, paint_cover) + thin, 0.03f, 0.95f);
  }
  const float z0 = surf_hit(X, p, detail);
  const float sh = shadow_at(X, p, z0, l);
  const float ao = ambient_occlusion(X, p, z0, detail);
  float3 albedo = rgb(col);
  const float painted = sstep(0.0f, 0.08e-3f, detail.thickness);
  if (painted > 0.0f) {
    const float g = granulation(p);
    albedo = albedo * (1.0f + 0.045f * g * painted);
    const float rim = edge_factor(X, p);
    albedo = albedo * (1.0f - 0.10f * rim * painted);
  }
  if (X.beauty() && painted > 0.0f) {
    const float2 sc = streak_coords(p, detail.dir);
    const float tool = clampf(detail.brush + detail.knife, 0.0f, 1.0f);
    const float st = fbm_filtered(X, v2(sc.x, sc.y / 25.0f), 0.09e-3f, 4);
    albedo = albedo * (1.0f + 0.16f * st * (0.3f + 0.7f * tool) * painted);
    const float cl = fbm_filtered(X, v2(sc.x, sc.y / CLUMP_ELONGATION), CLUMP_WIDTH, 3);
    albedo = albedo * (1.0f + 0.10f * cl * tool * painted);
    const float thin_paint = 1.0f - sstep(0.03e-3f, 0.25e-3f, detail.thickness);
    const float3 wv = weave(p);
    albedo = albedo * (1.0f + 0.22f * thin_paint * (wv.x - 0.55f) * painted);
  }
  const float bare = 1.0f - sstep(0.0f, 0.15e-3f, detail.thickness);
  if (bare > 0.0f) albedo = mix3(albedo, canvas_albedo(p, albedo), bare);
  if (X.beauty() && painted > 0.0f) {
    const float3 hue = v3(fbm(p / 6e-3f + v2(1.3f, 5.1f), 3), fbm(p / 6e-3f + v2(7.7f, 2.2f), 3),
                          fbm(p / 6e-3f + v2(4.4f, 9.9f), 3));
    const float tone = fbm(p / 2.2e-3f + v2(3.3f, 0.7f), 4);
    albedo = albedo * ((v3(1.0f, 1.0f, 1.0f) + PAINT_HUE_DRIFT * hue) * (1.0f + PAINT_TONE_DRIFT * tone * painted));
  }
  const float2 sp = specks(p);
  albedo = mix3(albedo, v3(0.85f, 0.83f, 0.8f), 0.7f * sp.x * (0.4f + 0.6f * bare));
  albedo = albedo * (1.0f - 0.6f * sp.y);
  const float rough_var = 1.0f + 0.18f * vnoise(p / 0.45e-3f + v2(3.0f, 8.0f)) * painted;
  const float rough_s = clampf(rough * rough_var, 0.03f, 0.95f);
  const float wetness = wet_bilinear(X, p);
  const float coat = sstep(0.02e-3f, 0.25e-3f, wetness) * (1.0f - 0.7f * detail.cure) * (1.0f - thin / 0.3f);
  const float aniso = clampf(0.7f * detail.brush + 0.5f * detail.knife, 0.0f, 0.8f) * sstep(0.0f, 0.15e-3f, detail.thickness);
  const float falloff = X.cam.jitter[2] > 0.5f ? lamp_falloff(X, p) : 1.0f;
  const float3 c = lit(X, n, v, l, sh, ao, albedo, rough_s, detail.cure, coat, aniso, detail.dir, falloff);
  if (X.cam.jitter[2] > 0.5f) {
    auto fc = [](float x) { return x != x ? 0.0f : fminf(x, FIREFLY_CLAMP); };
    return make_float4(fc(c.x), fc(c.y), fc(c.z), 1.0f);
  }
  const float3 o = to_srgb(tonemap(c));
  return make_float4(o.x, o.y, o.z, 1.0f);
}

// One thread per pixel of a width x height target; the pixel centre's ndc as
// the full-screen triangle interpolates it (y up).
__global__ void __launch_bounds__(128, 8) k_render_lit(R X, uint32_t width, uint32_t height, float4* out_f32,
                                                    uint32_t* out_rgba8) {
  const uint32_t px = blockIdx.x * 16u + threadIdx.x, py = blockIdx.y * 8u + threadIdx.y;
  if (px >= width || py >= height) return;
  const float2 ndc = v2(2.0f * ((float)px + 0.5f) / (float)width - 1.0f, 1.0f - 2.0f * ((float)py + 0.5f) / (float)height);
  const float4 c = fs(X, ndc);
  const size_t o = (size_t)py * width + px;
  if (out_f32) out_f32[o] = c;
  if (out_rgba8) {
    auto q = [](float x) { return (uint32_t)fminf(fmaxf(x * 255.0f + 0.5f, 0.0f), 255.0f); };
    out_rgba8[o] = q(c.x) | (q(c.y) << 8) | (q(c.z) << 16) | (q(c.w) << 24);
  }
}

}  // namespace

extern "C" {

cf_status cf_render_lit(cf_film* f, const cf_render_cam* cam, uint32_t width, uint32_t height, float* rgba_f32,
                        uint8_t* rgba8, void* stream) {
  if (!f || !cam || width == 0 || height == 0 || (!rgba_f32 && !rgba8)) return CF_ERR_INVALID_ARG;
  if ((reinterpret_cast<uintptr_t>(rgba_f32) & 15u) != 0u || (reinterpret_cast<uintptr_t>(rgba8) & 3u) != 0u)
    return CF_ERR_INVALID_ARG;
  if (cam->size[0] != f->w || cam->size[1] != f->h) return CF_ERR_INVALID_ARG;
  R X;
  X.cam = *cam;
  X.h = f->F.hh;
  X.m = f->F.m;
  X.color = f->F.color;
  X.detail = f->F.detail;
  X.tile_flags = f->F.tile_flags;
  const dim3 b(16, 8), g((width + 15u) / 16u, (height + 7u) / 8u);
  k_render_lit<<<g, b, 0, static_cast<cudaStream_t>(stream)>>>(X, width, height, reinterpret_cast<float4*>(rgba_f32),
                                                                 reinterpret_cast<uint32_t*>(rgba8));
  return cudaGetLastError() == cudaSuccess ? CF_OK : CF_ERR_CUDA;
}

}  // extern "C"
