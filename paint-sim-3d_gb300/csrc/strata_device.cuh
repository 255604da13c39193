// strata_device.cuh — the 4-layer material stack of strata.wgsl:1-155, the
// rheology composition of cure.wgsl:3-117 and the KM shade of
// shade.wgsl:28-84, as device functions over an in-register stack.
//
// A Stack is the WGSL `Stack`: 4 thicknesses, 4 cure fractions and 4 x 16
// pigment slots.  Slot 15 (the per-cell power-law index, 0 = global) is mixed
// like slot 14.
#pragma once

#include "film_device.cuh"

namespace cfk {

struct Stack {
  float th[4];
  float cu[4];
  float pg[4][16];
};

template <int MODE>
__device__ __forceinline__ void stack_load(const Film& F, const float4* sh, const float4* scu, const uint4* pig,
                                           uint32_t c, Stack& s) {
  float4 t = sh[c], u = scu[c];
  s.th[0] = t.x; s.th[1] = t.y; s.th[2] = t.z; s.th[3] = t.w;
  s.cu[0] = u.x; s.cu[1] = u.y; s.cu[2] = u.z; s.cu[3] = u.w;
#pragma unroll
  for (int k = 0; k < 4; ++k) PigIO<MODE>::load(F, pig, c, k, s.pg[k]);
}
template <int MODE>
__device__ __forceinline__ void stack_store(const Film& F, float4* sh, float4* scu, uint4* pig, uint32_t c,
                                            const Stack& s) {
  sh[c] = make_float4(s.th[0], s.th[1], s.th[2], s.th[3]);
  scu[c] = make_float4(s.cu[0], s.cu[1], s.cu[2], s.cu[3]);
#pragma unroll
  for (int k = 0; k < 4; ++k) PigIO<MODE>::store(F, pig, c, k, s.pg[k]);
}

__device__ __forceinline__ float pig_dist(const float* a, const float* b) {  // strata.wgsl:37-43
  float d = 0.f;
#pragma unroll
  for (int q = 0; q < 13; ++q) d += fabsf(a[q] - b[q]);
  return d;
}
// strata.wgsl:45-60 into `o` (may alias a)
__device__ __forceinline__ void pig_mix(const float* a, float wa, const float* b, float wb, float* o) {
  float w = fmaxf(wa + wb, 1e-20f);
  float t[16];
#pragma unroll
  for (int q = 0; q < 16; ++q) t[q] = (a[q] * wa + b[q] * wb) / w;
#pragma unroll
  for (int slot = 14; slot <= 15; ++slot) {
    float va = a[slot] > 0.f ? wa : 0.f;
    float vb = b[slot] > 0.f ? wb : 0.f;
    t[slot] = (va + vb > 0.f) ? (a[slot] * va + b[slot] * vb) / (va + vb) : 0.f;
  }
#pragma unroll
  for (int q = 0; q < 16; ++q) o[q] = t[q];
}
__device__ __forceinline__ uint32_t stack_count(const Stack& s) {  // strata.wgsl:62-68
  uint32_t n = 0;
#pragma unroll
  for (int k = 0; k < 4; ++k)
    if (s.th[k] > 0.f) n = k + 1;
  return n;
}
__device__ inline void stack_merge(Stack& s, int a) {  // strata.wgsl:70-85
  int b = a + 1;
  float ta = s.th[a], tb = s.th[b];
  pig_mix(s.pg[a], ta, s.pg[b], tb, s.pg[a]);
  s.cu[a] = (s.cu[a] * ta + s.cu[b] * tb) / fmaxf(ta + tb, 1e-20f);
  s.th[a] = ta + tb;
  for (int k = b; k < 3; ++k) {
    s.th[k] = s.th[k + 1];
    s.cu[k] = s.cu[k + 1];
#pragma unroll
    for (int q = 0; q < 16; ++q) s.pg[k][q] = s.pg[k + 1][q];
  }
  s.th[3] = 0.f;
  s.cu[3] = 0.f;
}
__device__ inline void stack_compact(Stack& s, float tiny) {  // strata.wgsl:87-103
  for (int sweep = 0; sweep < 4; ++sweep)
#pragma unroll
    for (int k = 0; k < 3; ++k)
      if (s.th[k] <= 0.f && s.th[k + 1] > 0.f) {
        s.th[k] = s.th[k + 1];
        s.cu[k] = s.cu[k + 1];
#pragma unroll
        for (int q = 0; q < 16; ++q) s.pg[k][q] = s.pg[k + 1][q];
        s.th[k + 1] = 0.f;
        s.cu[k + 1] = 0.f;
      }
  for (int k = 0; k < 3; ++k)
    if (s.th[k] > 0.f && s.th[k] < tiny && s.th[k + 1] > 0.f) stack_merge(s, k);
}
// strata.wgsl:105-131
__device__ inline void stack_push_top(Stack& s, float vol, const float* pg, float cv, float tiny, float close_d) {
  if (vol <= 0.f) return;
  uint32_t n = stack_count(s);
  if (n > 0) {
    int t = (int)n - 1;
    bool close = pig_dist(s.pg[t], pg) < close_d || s.th[t] < tiny;
    if (close) {
      pig_mix(s.pg[t], s.th[t], pg, vol, s.pg[t]);
      s.cu[t] = (s.cu[t] * s.th[t] + cv * vol) / (s.th[t] + vol);
      s.th[t] += vol;
      return;
    }
  }
  if (n == 4) {
    int best = 0;
    float bd = 1e30f;
    for (int k = 0; k < 3; ++k) {
      float d = pig_dist(s.pg[k], s.pg[k + 1]);
      if (d < bd) { bd = d; best = k; }
    }
    stack_merge(s, best);
  }
  uint32_t t = stack_count(s);
  s.th[t] = vol;
#pragma unroll
  for (int q = 0; q < 16; ++q) s.pg[t][q] = pg[q];
  s.cu[t] = cv;
}
// km.wgsl:17-33 for all bands at once: K,S of one stratum's pigment mix.
__device__ __forceinline__ void layer_weights(const float* pg, const float* tab, float w[12], float& scale) {
  float amount = 0.f, weight = 0.f;
#pragma unroll
  for (int q = 0; q < 12; ++q) {
    float c = pg[q];
    float ww = c > 0.f ? c * tab[q * 40 + 34] : 0.f;
    w[q] = ww;
    if (c > 0.f) { amount += c; weight += ww; }
  }
  scale = amount / fmaxf(weight, 1e-9f);
}
__device__ __forceinline__ void layer_ks_band(const float* pg, const float w[12], float scale, const float* tab, int b,
                                              float& k, float& s) {
  k = 0.f;
  s = 0.f;
#pragma unroll
  for (int q = 0; q < 12; ++q) {
    if (pg[q] > 0.f) {
      k += w[q] * tab[q * 40 + b];
      s += w[q] * tab[q * 40 + 16 + b];
    }
  }
  k = k * scale;
  s = s * scale;
}
// layer_ks_band from a band-major copy of the table: kst[24 b + p] = K of
// pigment p in band b, kst[24 b + 12 + p] = its S (16-byte aligned), read as
// six 16-byte loads instead of 24 scalar ones.  Every pigment is added: a
// pigment with no amount has w = 0 (layer_weights), and adding w * K = +0 to
// these non-negative sums leaves them bit for bit as layer_ks_band's.
__device__ __forceinline__ void layer_ks_band_t(const float w[12], float scale, const float* kst, int b, float& k,
                                                float& s) {
  const float4* t = reinterpret_cast<const float4*>(kst + b * 24);
  k = 0.f;
  s = 0.f;
#pragma unroll
  for (int g = 0; g < 3; ++g) {  // pigments 4g .. 4g + 3
    const float4 kq = t[g], sq = t[3 + g];
    k += w[4 * g] * kq.x;
    s += w[4 * g] * sq.x;
    k += w[4 * g + 1] * kq.y;
    s += w[4 * g + 1] * sq.y;
    k += w[4 * g + 2] * kq.z;
    s += w[4 * g + 2] * sq.z;
    k += w[4 * g + 3] * kq.w;
    s += w[4 * g + 3] * sq.w;
  }
  k = k * scale;
  s = s * scale;
}

// shade.wgsl:51-56 for a composite spectrum r: the surface correction
// (Saunderson, k1 = 0.04, k2 from 0.4 dry to 0.6 wet), the CMF x D65 sums to
// XYZ and XYZ -> linear sRGB (km.wgsl:51-62), clamped at 0.
__device__ __forceinline__ void surface_rgb(const float* cm, const float r[16], float wt, float rgb[3]) {
  const float k1 = 0.04f;
  const float k2 = 0.4f * (1.0f - wt) + 0.6f * wt;
  float X = 0.f, Y = 0.f, Z = 0.f;
#pragma unroll
  for (int b = 0; b < 16; ++b) {
    const float rb = __fdividef((1.0f - k1) * (1.0f - k2) * r[b], fmaxf(1.0f - k2 * r[b], 1e-3f));  // colour is stored as f16
    X += rb * cm[3 * b];
    Y += rb * cm[3 * b + 1];
    Z += rb * cm[3 * b + 2];
  }
  rgb[0] = fmaxf(3.2406f * X - 1.5372f * Y - 0.4986f * Z, 0.f);
  rgb[1] = fmaxf(-0.9689f * X + 1.8758f * Y + 0.0415f * Z, 0.f);
  rgb[2] = fmaxf(0.0557f * X - 0.2040f * Y + 1.0570f * Z, 0.f);
}
// shade.wgsl:57-62: the roughness from the top stratum's cure, the relief m
// and the film height h.
__device__ __forceinline__ float surface_rough(float cure_top, float hv, float mv) {
  auto smooth = [](float e0, float e1, float x) {
    float t = fminf(fmaxf((x - e0) / (e1 - e0), 0.f), 1.f);
    return t * t * (3.0f - 2.0f * t);
  };
  const float painted = smooth(60e-6f, 150e-6f, mv);
  const float ct = fmaxf(hv > 0.f ? cure_top : 0.f, painted * (1.0f - smooth(0.f, 50e-6f, hv)));
  const float sq = sqrtf(ct);
  float rough = 0.06f * (1.0f - sq) + 0.35f * sq;
  if (hv <= 0.f) rough = 0.85f * (1.0f - painted) + 0.35f * painted;
  return rough;
}
// shade.wgsl:61-64: the detail texel the renderer reads for a cell whose top
// wet stratum has cure fraction cure_top (0 for a dry cell): the lay method
// plus the stroke's turn, cure_top as the surface roughness sees it, the
// yield stress and the paint's thickness above the weave
template <int MODE>
__device__ __forceinline__ ushort4 detail_texel(const Film& F, uint32_t c, float cure_top, float hv, float mv) {
  auto smooth = [](float e0, float e1, float x) {
    float t = fminf(fmaxf((x - e0) / (e1 - e0), 0.f), 1.f);
    return t * t * (3.0f - 2.0f * t);
  };
  const float painted = smooth(60e-6f, 150e-6f, mv);
  const float ct = fmaxf(hv > 0.f ? cure_top : 0.f, painted * (1.0f - smooth(0.f, 50e-6f, hv)));
  const uint32_t lv = F.lay[c];
  const float turn = (float)((lv >> 8u) & 0xffffu) / 65536.0f;
  return make_ushort4((unsigned short)f_to_h16((float)(lv & 0xffu) + turn), (unsigned short)f_to_h16(ct),
                      (unsigned short)f_to_h16(rtau<MODE>(F, c)), (unsigned short)f_to_h16(hv + fmaxf(mv - 60e-6f, 0.f)));
}
// the cure fraction of the top stratum with paint (0 when none)
__device__ __forceinline__ float top_cure(const float th[4], const float cu[4]) {
  float ct = 0.f;
#pragma unroll
  for (int k = 0; k < 4; ++k)
    if (th[k] > 0.f) ct = cu[k];
  return ct;
}
__device__ __forceinline__ ushort4 pack_color(const float rgb[3], float rough) {
  return make_ushort4((unsigned short)f_to_h16(rgb[0]), (unsigned short)f_to_h16(rgb[1]),
                      (unsigned short)f_to_h16(rgb[2]), (unsigned short)f_to_h16(rough));
}

// Per-cell accumulation over the final strata, bottom to top, of
//  - the pigment part of the rheology composition (cure.wgsl:3-48), kept as
//    agg = (mu_base, 3 ln(1 - tf), tau_base (1 - tf)^4, n) for the next cure
//    (rheo_from_parts adds the cure-dependent part), and
//  - the KM shade (shade.wgsl:28-84): each stratum composited over the
//    substrate, then the surface correction and XYZ -> linear sRGB.
// The per-cell paths (fill, cure commit, state upload, deposits) go through
// this one accumulator, so their colour and aggregates are bitwise alike; the
// strata pass shades with the half-warp form of the same sums (LaneAcc in
// strata_lane.cuh), whose tree-ordered sums may differ from it in the last
// bits.
struct CellAcc {
  // composition
  float total, lnmu, tau, thin, wsum, nsum, nw;
  // shade
  float r[16];
  float wet, cure_top, ssum;
  uint32_t cnt;
  bool bad;

  __device__ __forceinline__ void begin(const uint16_t* rf) {
    total = lnmu = tau = thin = wsum = nsum = nw = 0.f;
    wet = cure_top = ssum = 0.f;
    cnt = 0;
    bad = false;
    const uint4* p = reinterpret_cast<const uint4*>(rf);
    uint4 a = p[0], b = p[1];
    uint32_t wv[8] = {a.x, a.y, a.z, a.w, b.x, b.y, b.z, b.w};
#pragma unroll
    for (int k = 0; k < 8; ++k) {
      r[2 * k] = h16_to_f(wv[k] & 0xffffu);
      r[2 * k + 1] = h16_to_f(wv[k] >> 16);
    }
  }
  // the composition part of a stratum of thickness t > 0 (cure.wgsl:3-48)
  __device__ __forceinline__ void add_comp(float t, const float* pg, const float* lnmu_tab) {
    total += t;
    float csum = 0.f, lm = 0.f, ty = 0.f;
#pragma unroll
    for (int q = 0; q < 12; ++q) {
      float cc = pg[q];
      if (cc > 0.f) {
        csum += cc;
        lm += cc * lnmu_tab[q];
        ty += cc * pg[13];
      }
    }
    if (pg[14] > 0.f) lm = csum * (pg[14] - 10.0f);
    if (csum > 0.f) {
      lnmu += t * lm / csum;
      tau += t * ty / csum;
      wsum += t;
      if (pg[15] > 0.f) { nsum += t * pg[15]; nw += t; }
    }
    thin += t * pg[12];
  }
  // stratum k (in order 0..3) of thickness t, cure u and slots pg
  __device__ __forceinline__ void add(int k, float t, float u, const float* pg, float hv, const float* lnmu_tab,
                                      const float* tab, bool debug) {
    add_with(k, t, u, pg, hv, lnmu_tab, tab, debug, [&](const float* w, float sc, int b, float& kk, float& ss) {
      layer_ks_band(pg, w, sc, tab, b, kk, ss);
    });
  }
  // the same with the K, S table band-major in shared memory (layer_ks_band_t)
  __device__ __forceinline__ void add_t(int k, float t, float u, const float* pg, float hv, const float* lnmu_tab,
                                        const float* tab, const float* kst, bool debug) {
    add_with(k, t, u, pg, hv, lnmu_tab, tab, debug, [&](const float* w, float sc, int b, float& kk, float& ss) {
      layer_ks_band_t(w, sc, kst, b, kk, ss);
    });
  }
  template <class KsBand>
  __device__ __forceinline__ void add_with(int k, float t, float u, const float* pg, float hv, const float* lnmu_tab,
                                           const float* tab, bool debug, KsBand ks_band) {
    ssum += t;
    if (t > 0.f) {
      add_comp(t, pg, lnmu_tab);
      if (hv > 0.f) {
        float w[12], sc;
        layer_weights(pg, tab, w, sc);
#pragma unroll 4
        for (int b = 0; b < 16; ++b) {
          float kk, ss, rr, tt;
          ks_band(w, sc, b, kk, ss);
          km_layer(kk, ss, t, rr, tt);
          r[b] = composite(rr, tt, r[b]);
        }
        wet = 1.0f - u;
        cure_top = u;
      }
      cnt = k + 1;
      if (debug) {
        float cs = 0.f;
#pragma unroll
        for (int q = 0; q < 13; ++q) cs += pg[q];
        if (!(cs > 0.f)) bad = true;
      }
    }
  }
  __device__ __forceinline__ float4 agg(const cf_params& P) const {
    if (total <= 0.f) return make_float4(0.f, 0.f, 0.f, P.phys[2]);
    float mu = logf(P.misc[2]);
    float ty = 0.f;
    if (wsum > 0.f) { mu = lnmu / wsum; ty = tau / wsum; }
    float tf = fminf(fmaxf(thin / total, 0.f), 0.95f);
    return make_float4(mu, 3.0f * logf(1.0f - tf), ty * powf(1.0f - tf, 4.0f), nw > 0.f ? nsum / nw : P.phys[2]);
  }
  __device__ __forceinline__ ushort4 color(const cf_params& P, const float* cm, float hv, float mv) const {
    float rgb[3];
    surface_rgb(cm, r, hv > 0.f ? wet : 0.f, rgb);
    const float rough = surface_rough(cure_top, hv, mv);
    if (P.flags[0] == 1u && hv > 0.f) {  // shade.wgsl:65-82 invariant view
      if (ssum <= 0.f) { rgb[0] = 0.f; rgb[1] = 0.f; rgb[2] = 1.f; }
      else if (bad) { rgb[0] = 1.f; rgb[1] = 0.f; rgb[2] = 0.f; }
      else if (fabsf(ssum - hv) > 0.01f * hv) { rgb[0] = 0.f; rgb[1] = 1.f; rgb[2] = 0.f; }
      else { float v = 0.3f + 0.15f * (float)cnt; rgb[0] = v; rgb[1] = v; rgb[2] = v; }
    }
    return make_ushort4((unsigned short)f_to_h16(rgb[0]), (unsigned short)f_to_h16(rgb[1]),
                        (unsigned short)f_to_h16(rgb[2]), (unsigned short)f_to_h16(rough));
  }
};

// Completes cure.wgsl:40-47 with the cure fractions u of strata of thickness t.
__device__ __forceinline__ void rheo_from_parts(const cf_params& P, float4 agg, const float t[4], const float u[4],
                                                float& mu_o, float& ty_o, float& n_o) {
  float total = 0.f, cur = 0.f;
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    if (t[k] <= 0.f) continue;
    total += t[k];
    cur += t[k] * u[k];
  }
  if (total <= 0.f) { mu_o = 1.f; ty_o = 0.f; n_o = P.phys[2]; return; }
  float cb = cur / total;
  float mu = agg.x + (agg.y + P.cure[2] * cb * cb);
  ty_o = agg.z + P.cure[1] * cb * cb;
  mu_o = expf(mu);
  n_o = agg.w;
}

// ln of each pigment's table viscosity (cure.wgsl:3-48 reads it per stratum).
__device__ __forceinline__ void lnmu_table(const float* pigtab, float out[12]) {
#pragma unroll
  for (int q = 0; q < 12; ++q) out[q] = logf(fmaxf(pigtab[q * 40 + 32], 1e-3f));
}

// The composition aggregates alone of a whole in-register stack (bitwise the
// ones finish_stack gives), for passes that change a stack but not its colour.
__device__ inline float4 stack_agg(const cf_params& P, const float* lnmu_tab, const Stack& s) {
  CellAcc a;
  a.total = a.lnmu = a.tau = a.thin = a.wsum = a.nsum = a.nw = 0.f;
#pragma unroll
  for (int k = 0; k < 4; ++k)
    if (s.th[k] > 0.f) a.add_comp(s.th[k], s.pg[k], lnmu_tab);
  return a.agg(P);
}

// Aggregates and colour of a whole in-register stack.
__device__ inline void finish_stack(const cf_params& P, const float* lnmu_tab, const float* tab, const float* cm,
                                    const uint16_t* rf, float hv, float mv, const Stack& s, float4& agg,
                                    ushort4& col) {
  CellAcc a;
  a.begin(rf);
  const bool dbg = P.flags[0] == 1u;
#pragma unroll
  for (int k = 0; k < 4; ++k) a.add(k, s.th[k], s.cu[k], s.pg[k], hv, lnmu_tab, tab, dbg);
  agg = a.agg(P);
  col = a.color(P, cm, hv, mv);
}

}  // namespace cfk
