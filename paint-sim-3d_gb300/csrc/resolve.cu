// resolve.cu — the display epilogue of resolve.wgsl:23-121 on the film's
// colour plane: exposure, bloom, sharpen, vignette, AgX or ACES tone map,
// grain and the sRGB transfer, written as RGBA8.
//
// The reference applies it to the renderer's HDR accumulation texture; with
// no graphics pipeline here the input is the film's linear-RGB colour plane
// (the headless stand-in for color_tex), one pixel per cell, pixel (x, y) =
// cell (x, y).
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include "film_handle.h"

namespace {

struct V3 {
  float x, y, z;
};
__device__ __forceinline__ V3 v3(float a) { return {a, a, a}; }
__device__ __forceinline__ V3 operator+(V3 a, V3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
__device__ __forceinline__ V3 operator-(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
__device__ __forceinline__ V3 operator*(V3 a, V3 b) { return {a.x * b.x, a.y * b.y, a.z * b.z}; }
__device__ __forceinline__ V3 operator*(V3 a, float s) { return {a.x * s, a.y * s, a.z * s}; }
__device__ __forceinline__ V3 operator/(V3 a, V3 b) { return {a.x / b.x, a.y / b.y, a.z / b.z}; }
__device__ __forceinline__ V3 vclamp(V3 a, float lo, float hi) {
  return {fminf(fmaxf(a.x, lo), hi), fminf(fmaxf(a.y, lo), hi), fminf(fmaxf(a.z, lo), hi)};
}
__device__ __forceinline__ V3 vmax(V3 a, float lo) { return {fmaxf(a.x, lo), fmaxf(a.y, lo), fmaxf(a.z, lo)}; }
__device__ __forceinline__ V3 vpow(V3 a, float e) { return {powf(a.x, e), powf(a.y, e), powf(a.z, e)}; }
__device__ __forceinline__ float lum(V3 c) { return c.x * 0.2126f + c.y * 0.7152f + c.z * 0.0722f; }
__device__ __forceinline__ float smooth(float e0, float e1, float x) {
  float t = fminf(fmaxf((x - e0) / (e1 - e0), 0.f), 1.f);
  return t * t * (3.0f - 2.0f * t);
}
// WGSL mat3x3 * vec3 with column vectors c0, c1, c2
__device__ __forceinline__ V3 mul(const float m[9], V3 v) {
  return {m[0] * v.x + m[3] * v.y + m[6] * v.z, m[1] * v.x + m[4] * v.y + m[7] * v.z,
          m[2] * v.x + m[5] * v.y + m[8] * v.z};
}

__device__ V3 aces(V3 c) {  // resolve.wgsl:23-26
  const float a = 2.51f, b = 0.03f, cc = 2.43f, d = 0.59f, e = 0.14f;
  return vclamp((c * (c * a + v3(b))) / (c * (c * cc + v3(d)) + v3(e)), 0.f, 1.f);
}

__device__ V3 agx(V3 c) {  // resolve.wgsl:28-50
  const float inset[9] = {0.842479062253094f, 0.0423282422610123f, 0.0423756549057051f,
                          0.0784335999999992f, 0.878468636469772f, 0.0784336f,
                          0.0792237451477643f, 0.0791661274605434f, 0.879142973793104f};
  const float outset[9] = {1.1968790051f, -0.0528968518f, -0.0529716355f, -0.0980208811f, 1.1519031299f,
                           -0.0980434501f, -0.0990297441f, -0.0989611768f, 1.1510736726f};
  const float min_ev = -12.47393f, max_ev = 4.026069f;
  V3 v = mul(inset, vmax(c, 1e-10f));
  v = {log2f(v.x), log2f(v.y), log2f(v.z)};
  v = vclamp(v, min_ev, max_ev);
  v = (v - v3(min_ev)) / v3(max_ev - min_ev);
  const V3 x2 = v * v, x4 = x2 * x2;
  v = x4 * x2 * 15.5f - x4 * v * 40.14f + x4 * 31.96f - x2 * v * 6.868f + x2 * 0.4298f + v * 0.1191f - v3(0.00232f);
  v = vclamp(v, 0.f, 1.f);
  const float l = lum(v);
  v = vpow(v, 1.35f);
  v = v3(l) + (v - v3(l)) * 1.4f;
  v = mul(outset, vclamp(v, 0.f, 1.f));
  return vpow(vclamp(v, 0.f, 1.f), 2.2f);
}

__device__ float to_srgb1(float c) {  // resolve.wgsl:52-56
  return c <= 0.0031308f ? c * 12.92f : 1.055f * powf(c, 1.0f / 2.4f) - 0.055f;
}

// f32 with one rounding per operation (no contraction): the hash takes fract
// of products near 1e4, where a fused multiply-add would change its value.
__device__ float fract(float x) { return __fsub_rn(x, floorf(x)); }
__device__ float hash12(float px, float py) {  // resolve.wgsl:58-62
  float qx = fract(__fmul_rn(px, 0.1031f)), qy = fract(__fmul_rn(py, 0.1030f));
  const float d = __fadd_rn(__fmul_rn(qx, __fadd_rn(qy, 33.33f)), __fmul_rn(qy, __fadd_rn(qx, 33.33f)));
  qx = __fadd_rn(qx, d);
  qy = __fadd_rn(qy, d);
  return fract(__fmul_rn(__fadd_rn(qx, qy), qx));
}

__device__ __forceinline__ V3 load(const ushort4* col, int w, int h, int x, int y, float scale) {
  x = min(max(x, 0), w - 1);
  y = min(max(y, 0), h - 1);
  const ushort4 p = col[(size_t)y * w + x];
  return V3{__half2float(__ushort_as_half(p.x)), __half2float(__ushort_as_half(p.y)),
            __half2float(__ushort_as_half(p.z))} * scale;
}

// resolve.wgsl:76-121 for one pixel
__global__ void __launch_bounds__(256) k_resolve(const ushort4* __restrict__ col, int w, int h, cf_resolve_params R,
                                                 uchar4* __restrict__ out) {
  const int x = blockIdx.x * 16 + threadIdx.x, y = blockIdx.y * 16 + threadIdx.y;
  if (x >= w || y >= h) return;
  const float exposure = exp2f(R.exposure_ev);
  V3 c = load(col, w, h, x, y, R.scale) * exposure;
  if (R.bloom > 0.f) {
    const float radius = fmaxf((float)h * 0.02f, 4.0f);
    V3 glow = v3(0.f);
    float wsum = 0.f;
    for (int k = 0; k < 32; ++k) {
      const float fk = (float)k + 0.5f;
      const float r = radius * sqrtf(fk / 32.0f);
      const float ang = fk * 2.399963f;
      const int ox = (int)(cosf(ang) * r), oy = (int)(sinf(ang) * r);
      const V3 s = load(col, w, h, x + ox, y + oy, R.scale) * exposure;
      const float l = lum(s);
      const float wk = 1.0f - fk / 33.0f;
      glow = glow + s * (fmaxf(l - 1.6f, 0.f) / fmaxf(l, 1e-4f) * wk);
      wsum += wk;
    }
    c = c + glow * (R.bloom * 0.35f / wsum);
  }
  if (R.sharpen > 0.f) {
    const V3 blur = (load(col, w, h, x + 1, y, R.scale) + load(col, w, h, x - 1, y, R.scale) +
                     load(col, w, h, x, y + 1, R.scale) + load(col, w, h, x, y - 1, R.scale)) * exposure * 0.25f;
    const V3 base = load(col, w, h, x, y, R.scale) * exposure;
    c = vmax(c + (base - blur) * R.sharpen, 0.f);
  }
  // the fragment position is the pixel centre
  const float px = (float)x + 0.5f, py = (float)y + 0.5f;
  const float ux = px / (float)w - 0.5f, uy = py / (float)h - 0.5f;
  const float vig = 1.0f - R.vignette * smooth(0.15f, 0.75f, (ux * ux + uy * uy) * 2.0f);
  c = c * vig;
  V3 m = R.agx ? agx(c) : aces(c);
  if (R.grain > 0.f) {
    const float g = (hash12(__fadd_rn(px, 0.37f), __fadd_rn(py, 0.11f)) - 0.5f) * 2.0f;
    const float shade = 1.0f - smooth(0.f, 1.f, lum(m));
    m = vclamp(m + v3(g * R.grain * (0.35f + 0.65f * shade)), 0.f, 1.f);
  }
  auto q8 = [](float v) { return (unsigned char)__float2int_rn(fminf(fmaxf(v, 0.f), 1.f) * 255.0f); };
  out[(size_t)y * w + x] = make_uchar4(q8(to_srgb1(m.x)), q8(to_srgb1(m.y)), q8(to_srgb1(m.z)), 255);
}

}  // namespace

extern "C" cf_status cf_resolve(cf_film* f, const cf_resolve_params* params, void* rgba8_device, void* stream) {
  if (!f || !params || !rgba8_device) return fail(f, CF_ERR_INVALID_ARG, "cf_resolve: null");
  const dim3 g((f->w + 15) / 16, (f->h + 15) / 16), b(16, 16);
  k_resolve<<<g, b, 0, (cudaStream_t)stream>>>(f->F.color, (int)f->w, (int)f->h, *params, (uchar4*)rgba8_device);
  CUDA_TRY(f, cudaGetLastError());
  return CF_OK;
}
