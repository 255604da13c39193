// relief.cu — the render pass's reading of the film (shaders/render.wgsl):
// the relief height and slope and the colour at any canvas point, as the
// renderer samples them with its plain camera (no beauty mode: cam.jitter.z
// = 0; the colour plane at the film's resolution: cam.ortho.z = 0), and a
// headless top-down view of the film built on them.
//
//   surf_at, surf_cubic        render.wgsl:305-312, 328-353 (cubic B-spline)
//   wet_at, wet_bilinear       render.wgsl:355-361, 394-406
//   col_at, color_sharp        render.wgsl:644-652, 706-750
//   base_slope, normal_from_slope  render.wgsl:628-642
//   surf_bilinear, shadow_at   render.wgsl:314-326, 846-866 (the key light's
//                              shadow march over the relief; surf_march is
//                              surf_bilinear with the plain camera)
//
// The sampling follows the shader's f32 arithmetic; the view's shading (a
// key light and an ambient term over the sampled colour and normal) is this
// library's, not the renderer's look-development lighting.
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <cstdint>

#include "film_handle.h"

namespace {

using cfk::Film;

__device__ __forceinline__ float surf_at(const Film& F, int i, int j) {
  const int ii = min(max(i, 0), (int)F.w - 1), jj = min(max(j, 0), (int)F.h - 1);
  const uint32_t c = (uint32_t)jj * F.w + (uint32_t)ii;
  return F.hh[c] + F.m[c];
}
__device__ __forceinline__ float wet_at(const Film& F, int i, int j) {
  const int ii = min(max(i, 0), (int)F.w - 1), jj = min(max(j, 0), (int)F.h - 1);
  return F.hh[(uint32_t)jj * F.w + (uint32_t)ii];
}
__device__ __forceinline__ float4 col_at(const Film& F, int i, int j) {
  const int ii = min(max(i, 0), (int)F.w - 1), jj = min(max(j, 0), (int)F.h - 1);
  const ushort4 u = F.color[(uint32_t)jj * F.w + (uint32_t)ii];
  return make_float4(__half2float(__ushort_as_half(u.x)), __half2float(__ushort_as_half(u.y)),
                     __half2float(__ushort_as_half(u.z)), __half2float(__ushort_as_half(u.w)));
}
// render.wgsl:328-333
__device__ __forceinline__ float4 cr_w(float t) {
  const float t2 = t * t, t3 = t2 * t, u = 1.0f - t;
  return make_float4(u * u * u / 6.0f, (3.0f * t3 - 6.0f * t2 + 4.0f) / 6.0f,
                     (-3.0f * t3 + 3.0f * t2 + 3.0f * t + 1.0f) / 6.0f, t3 / 6.0f);
}
__device__ __forceinline__ float sel(float4 v, int k) { return k == 0 ? v.x : (k == 1 ? v.y : (k == 2 ? v.z : v.w)); }

struct Canvas {
  float wm, hm, dx;
};
__device__ __forceinline__ bool outside(const Canvas& cv, float px, float py) {
  return px < 0.f || py < 0.f || px > cv.wm || py > cv.hm;
}
// render.wgsl:335-353
__device__ float surf_cubic(const Film& F, const Canvas& cv, float px, float py) {
  if (outside(cv, px, py)) return 0.f;
  const float gx = px / cv.dx - 0.5f, gy = py / cv.dx - 0.5f;
  const float fx = floorf(gx), fy = floorf(gy);
  const int i = (int)fx, j = (int)fy;
  const float4 wx = cr_w(gx - fx), wy = cr_w(gy - fy);
  float s = 0.f;
  for (int b = -1; b <= 2; ++b) {
    float row = 0.f;
    for (int a = -1; a <= 2; ++a) row += sel(wx, a + 1) * surf_at(F, i + a, j + b);
    s += sel(wy, b + 1) * row;
  }
  return fmaxf(s, 0.f);
}
// render.wgsl:394-406, mix(a, b, t) = a (1 - t) + b t
__device__ float wet_bilinear(const Film& F, const Canvas& cv, float px, float py) {
  if (outside(cv, px, py)) return 0.f;
  const float gx = px / cv.dx - 0.5f, gy = py / cv.dx - 0.5f;
  const float fx = floorf(gx), fy = floorf(gy), tx = gx - fx, ty = gy - fy;
  const int i = (int)fx, j = (int)fy;
  const float a = wet_at(F, i, j), b = wet_at(F, i + 1, j), c = wet_at(F, i, j + 1), d = wet_at(F, i + 1, j + 1);
  const float r0 = a * (1.0f - tx) + b * tx, r1 = c * (1.0f - tx) + d * tx;
  return r0 * (1.0f - ty) + r1 * ty;
}
// render.wgsl:314-326, mix(a, b, t) = a (1 - t) + b t
__device__ float surf_bilinear(const Film& F, const Canvas& cv, float px, float py) {
  if (outside(cv, px, py)) return 0.f;
  const float gx = px / cv.dx - 0.5f, gy = py / cv.dx - 0.5f;
  const float fx = floorf(gx), fy = floorf(gy), tx = gx - fx, ty = gy - fy;
  const int i = (int)fx, j = (int)fy;
  const float a = surf_at(F, i, j), b = surf_at(F, i + 1, j), c = surf_at(F, i, j + 1), d = surf_at(F, i + 1, j + 1);
  const float r0 = a * (1.0f - tx) + b * tx, r1 = c * (1.0f - tx) + d * tx;
  return r0 * (1.0f - ty) + r1 * ty;
}
// render.wgsl:846-866 with the plain camera: 20 steps of 1.5 cells along the
// light over the bilinear relief from height z0, stopping once the ray is
// above `top` (cam.canvas.w); each step darkens by how far the relief rises
// above the ray, over a penumbra that widens with the distance.
__device__ float shadow_at(const Film& F, const Canvas& cv, float px, float py, float z0, float3 l, float top) {
  if (l.z <= 0.05f) return 1.0f;
  const float step = cv.dx * 1.5f;
  const float spread = tanf(0.12f);  // KEY_HALF_ANGLE
  const float sx = l.x / l.z, sy = l.y / l.z;
  float sh = 1.0f;
  for (int k = 1; k <= 20; ++k) {
    const float d = (float)k * step;
    const float zs = surf_bilinear(F, cv, px + sx * d, py + sy * d);
    const float zr = z0 + d;
    if (zr > top) break;
    const float pen = d * spread / l.z + 0.5f * step;
    sh = fminf(sh, 1.0f - fminf(fmaxf((zs - zr) / pen, 0.f), 1.f));
  }
  return sh;
}
// render.wgsl:628-638 (plain camera)
__device__ float2 base_slope(const Film& F, const Canvas& cv, float px, float py) {
  const float e = 0.7f * cv.dx;
  const float sx = surf_cubic(F, cv, px + e, py) - surf_cubic(F, cv, px - e, py);
  const float sy = surf_cubic(F, cv, px, py + e) - surf_cubic(F, cv, px, py - e);
  return make_float2(sx / (2.0f * e), sy / (2.0f * e));
}
__device__ __forceinline__ float smoothstep(float e0, float e1, float x) {
  const float t = fminf(fmaxf((x - e0) / (e1 - e0), 0.f), 1.f);
  return t * t * (3.0f - 2.0f * t);
}
__device__ __forceinline__ float4 f4_axpy(float4 acc, float w, float4 c) {
  return make_float4(acc.x + w * c.x, acc.y + w * c.y, acc.z + w * c.z, acc.w + w * c.w);
}
// render.wgsl:706-750 (plain camera: bilinear colour, sharpened where the
// wet height has an edge inside the 2x2 footprint)
__device__ float4 color_sharp(const Film& F, const Canvas& cv, float px, float py) {
  const float gx = px / cv.dx - 0.5f, gy = py / cv.dx - 0.5f;
  const float fx = floorf(gx), fy = floorf(gy), tx = gx - fx, ty = gy - fy;
  const int i = (int)fx, j = (int)fy;
  const float4 wb = make_float4((1.0f - tx) * (1.0f - ty), tx * (1.0f - ty), (1.0f - tx) * ty, tx * ty);
  const float4 hw = make_float4(wet_at(F, i, j), wet_at(F, i + 1, j), wet_at(F, i, j + 1), wet_at(F, i + 1, j + 1));
  const float4 c0 = col_at(F, i, j), c1 = col_at(F, i + 1, j), c2 = col_at(F, i, j + 1), c3 = col_at(F, i + 1, j + 1);
  float4 cbil = make_float4(0.f, 0.f, 0.f, 0.f);
  cbil = f4_axpy(cbil, wb.x, c0);
  cbil = f4_axpy(cbil, wb.y, c1);
  cbil = f4_axpy(cbil, wb.z, c2);
  cbil = f4_axpy(cbil, wb.w, c3);
  const float hmax = fmaxf(fmaxf(hw.x, hw.y), fmaxf(hw.z, hw.w));
  const float hmin = fminf(fminf(hw.x, hw.y), fminf(hw.z, hw.w));
  if (hmax <= 1e-6f) return cbil;
  const float edge = smoothstep(0.3f, 0.6f, 1.0f - hmin / hmax);
  if (edge <= 0.f) return cbil;
  const float4 wx = cr_w(tx), wy = cr_w(ty);
  float hb = 0.f, hb2 = 0.f;
  for (int b = -1; b <= 2; ++b)
    for (int a = -1; a <= 2; ++a) {
      const float wv = sel(wx, a + 1) * sel(wy, b + 1);
      const float hv = wet_at(F, i + a, j + b);
      hb += wv * hv;
      hb2 += wv * hv * hv;
    }
  hb = fmaxf(hb, 0.f);
  const float hin = hb2 / fmaxf(hb, 1e-9f);
  const float4 win = make_float4(wb.x * hw.x, wb.y * hw.y, wb.z * hw.z, wb.w * hw.w);
  const float4 wout = make_float4(wb.x * (hmax - hw.x), wb.y * (hmax - hw.y), wb.z * (hmax - hw.z), wb.w * (hmax - hw.w));
  const float sin_ = fmaxf(win.x + win.y + win.z + win.w, 1e-12f);
  const float sout = fmaxf(wout.x + wout.y + wout.z + wout.w, 1e-12f);
  float4 cin = make_float4(0.f, 0.f, 0.f, 0.f), cout = make_float4(0.f, 0.f, 0.f, 0.f);
  cin = f4_axpy(f4_axpy(f4_axpy(f4_axpy(cin, win.x, c0), win.y, c1), win.z, c2), win.w, c3);
  cout = f4_axpy(f4_axpy(f4_axpy(f4_axpy(cout, wout.x, c0), wout.y, c1), wout.z, c2), wout.w, c3);
  cin = make_float4(cin.x / sin_, cin.y / sin_, cin.z / sin_, cin.w / sin_);
  cout = make_float4(cout.x / sout, cout.y / sout, cout.z / sout, cout.w / sout);
  const float s = smoothstep(0.25f, 0.45f, hb / fmaxf(hin, 1e-9f));
  const float4 ce = make_float4(cout.x * (1.0f - s) + cin.x * s, cout.y * (1.0f - s) + cin.y * s,
                                cout.z * (1.0f - s) + cin.z * s, cout.w * (1.0f - s) + cin.w * s);
  return make_float4(cbil.x * (1.0f - edge) + ce.x * edge, cbil.y * (1.0f - edge) + ce.y * edge,
                     cbil.z * (1.0f - edge) + ce.z * edge, cbil.w);
}

// out per point: surf_cubic, base_slope (x, y), color_sharp (r, g, b, a), wet_bilinear
__global__ void __launch_bounds__(256) k_sample_relief(Film F, Canvas cv, const float2* __restrict__ pts, uint32_t n,
                                                       float* __restrict__ out) {
  const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  const float2 p = pts[k];
  const float2 sl = base_slope(F, cv, p.x, p.y);
  const float4 col = color_sharp(F, cv, p.x, p.y);
  float* o = out + 8 * (size_t)k;
  o[0] = surf_cubic(F, cv, p.x, p.y);
  o[1] = sl.x;
  o[2] = sl.y;
  o[3] = col.x;
  o[4] = col.y;
  o[5] = col.z;
  o[6] = col.w;
  o[7] = wet_bilinear(F, cv, p.x, p.y);
}

// out per point (x, y, z0): surf_bilinear, shadow_at
__global__ void __launch_bounds__(256) k_relief_shadow(Film F, Canvas cv, const float3* __restrict__ pts, uint32_t n,
                                                       float3 l, float top, float2* __restrict__ out) {
  const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  const float3 p = pts[k];
  out[k] = make_float2(surf_bilinear(F, cv, p.x, p.y), shadow_at(F, cv, p.x, p.y, p.z, l, top));
}

// linear -> sRGB (resolve.wgsl:52-56), then 8 bits
__device__ __forceinline__ uint32_t srgb8(float c) {
  c = fminf(fmaxf(c, 0.f), 1.f);
  const float v = c <= 0.0031308f ? 12.92f * c : 1.055f * powf(c, 1.0f / 2.4f) - 0.055f;
  return (uint32_t)__float2int_rn(fminf(fmaxf(v, 0.f), 1.f) * 255.0f);
}

__global__ void __launch_bounds__(256) k_render_relief(Film F, Canvas cv, cf_relief_view v, float3 l,
                                                       uint32_t* __restrict__ out) {
  const uint32_t x = blockIdx.x * 16 + threadIdx.x, y = blockIdx.y * 16 + threadIdx.y;
  if (x >= v.width || y >= v.height) return;
  const float px = v.x0 + ((float)x + 0.5f) * v.pixel_m, py = v.y0 + ((float)y + 0.5f) * v.pixel_m;
  const float2 sl = base_slope(F, cv, px, py);
  const float nl = rsqrtf(sl.x * sl.x + sl.y * sl.y + 1.0f);  // normal_from_slope (render.wgsl:640-642)
  const float diff = fmaxf((-sl.x * l.x - sl.y * l.y + l.z) * nl, 0.f);
  const float4 col = color_sharp(F, cv, px, py);
  const float k = v.ambient + (1.0f - v.ambient) * diff;
  out[(size_t)y * v.width + x] =
      srgb8(col.x * k) | (srgb8(col.y * k) << 8) | (srgb8(col.z * k) << 16) | (255u << 24);
}

Canvas canvas_of(const cf_film* f) { return Canvas{f->S.width_m, f->S.height_m, f->S.width_m / (float)f->w}; }

// The kernels read points and write results as float2 / float3 / uint32
// vectors: a buffer that is valid byte by byte but not aligned to them is
// refused here rather than faulting on the device.
bool aligned(const void* p, uintptr_t a) { return (reinterpret_cast<uintptr_t>(p) & (a - 1)) == 0; }

}  // namespace

extern "C" {

cf_status cf_sample_relief(cf_film* f, const float* points, uint32_t n, float* out, void* stream) {
  if (!f || (n && (!points || !out))) return fail(f, CF_ERR_INVALID_ARG, "cf_sample_relief");
  if (n && (!aligned(points, 8) || !aligned(out, 4)))
    return fail(f, CF_ERR_INVALID_ARG, "cf_sample_relief: points must be 8-byte and out 4-byte aligned");
  if (n == 0) return CF_OK;
  k_sample_relief<<<(n + 255) / 256, 256, 0, (cudaStream_t)stream>>>(f->F, canvas_of(f), (const float2*)points, n,
                                                                      out);
  CUDA_TRY(f, cudaGetLastError());
  return CF_OK;
}

cf_status cf_relief_shadow(cf_film* f, const float* points, uint32_t n, const float* light, float top, float* out,
                           void* stream) {
  if (!f || !light || (n && (!points || !out))) return fail(f, CF_ERR_INVALID_ARG, "cf_relief_shadow");
  if (n && (!aligned(points, 4) || !aligned(out, 8)))
    return fail(f, CF_ERR_INVALID_ARG, "cf_relief_shadow: points must be 4-byte and out 8-byte aligned");
  if (n == 0) return CF_OK;
  const float3 l = make_float3(light[0], light[1], light[2]);
  k_relief_shadow<<<(n + 255) / 256, 256, 0, (cudaStream_t)stream>>>(f->F, canvas_of(f), (const float3*)points, n, l,
                                                                      top, (float2*)out);
  CUDA_TRY(f, cudaGetLastError());
  return CF_OK;
}

cf_status cf_render_relief(cf_film* f, const cf_relief_view* v, uint8_t* rgba8, void* stream) {
  if (!f || !v || !rgba8 || v->width == 0 || v->height == 0 || !(v->pixel_m > 0.f))
    return fail(f, CF_ERR_INVALID_ARG, "cf_render_relief");
  if (!aligned(rgba8, 4)) return fail(f, CF_ERR_INVALID_ARG, "cf_render_relief: rgba8 must be 4-byte aligned");
  float lx = v->light[0], ly = v->light[1], lz = v->light[2];
  const float ll = std::sqrt(lx * lx + ly * ly + lz * lz);
  if (!(ll > 0.f)) return fail(f, CF_ERR_INVALID_ARG, "cf_render_relief: light");
  const float3 l = make_float3(lx / ll, ly / ll, lz / ll);
  const dim3 g((v->width + 15) / 16, (v->height + 15) / 16), b(16, 16);
  k_render_relief<<<g, b, 0, (cudaStream_t)stream>>>(f->F, canvas_of(f), *v, l, (uint32_t*)rgba8);
  CUDA_TRY(f, cudaGetLastError());
  return CF_OK;
}

}  // extern "C"
