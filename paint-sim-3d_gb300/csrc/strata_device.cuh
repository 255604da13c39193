// strata_device.cuh — the 4-layer material stack of strata.wgsl:1-155 and the
// rheology/cure composition of cure.wgsl:3-117, as device functions.
//
// A Stack lives in the thread's registers/local memory: 4 thicknesses, 4 cure
// fractions and 4 x 16 pigment slots, exactly the WGSL `Stack`.  Slot 15 (the
// per-cell power-law index, 0 = global) is mixed like slot 14.
#pragma once

#include "film_device.cuh"

namespace cfk {

struct Stack {
  float th[4];
  float cu[4];
  float pg[4][16];
};

template <int MODE>
__device__ __forceinline__ void stack_load(const Film& F, const void* pig, uint32_t c, Stack& s) {
  float4 t = F.sh[c], u = F.scu[c];
  s.th[0] = t.x; s.th[1] = t.y; s.th[2] = t.z; s.th[3] = t.w;
  s.cu[0] = u.x; s.cu[1] = u.y; s.cu[2] = u.z; s.cu[3] = u.w;
  using Pig = typename Prec<MODE>::Pig;
#pragma unroll
  for (int k = 0; k < 4; ++k) load_pig16<Pig>((const Pig*)pig + (size_t)c * 64 + 16 * k, s.pg[k]);
}
template <int MODE>
__device__ __forceinline__ void stack_store(float4* th, float4* cu, void* pig, uint32_t c, const Stack& s) {
  th[c] = make_float4(s.th[0], s.th[1], s.th[2], s.th[3]);
  cu[c] = make_float4(s.cu[0], s.cu[1], s.cu[2], s.cu[3]);
  using Pig = typename Prec<MODE>::Pig;
#pragma unroll
  for (int k = 0; k < 4; ++k) store_pig16<Pig>((Pig*)pig + (size_t)c * 64 + 16 * k, s.pg[k]);
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
// strata.wgsl:133-155
__device__ inline void stack_add_band(Stack& s, float zlo, float zhi, float vol, const float* pg, float cv, float tiny,
                               float close_d) {
  if (vol <= 0.f) return;
  float span = fmaxf(zhi - zlo, 1e-12f);
  float z0 = 0.f, above = vol;
  for (int k = 0; k < 4; ++k) {
    float tk = s.th[k];
    if (tk <= 0.f) break;
    float z1 = z0 + tk;
    float ov = fmaxf(fminf(zhi, z1) - fmaxf(zlo, z0), 0.f);
    float part = vol * ov / span;
    if (part > 0.f) {
      pig_mix(s.pg[k], tk, pg, part, s.pg[k]);
      s.cu[k] = (s.cu[k] * tk + cv * part) / (tk + part);
      s.th[k] = tk + part;
      above -= part;
    }
    z0 = z1;
  }
  if (above > 1e-14f) stack_push_top(s, above, pg, cv, tiny, close_d);
}

// cure.wgsl:3-48 (equivalently packed_rheo :62-117): (mu, tau_y, n)
__device__ inline void composition_rheo(const cf_params& P, const float* pigtab, const Stack& s, float& mu_o, float& ty_o,
                                 float& n_o) {
  float total = 0.f, lnmu = 0.f, tau = 0.f, thin = 0.f, wsum = 0.f, cur = 0.f, nsum = 0.f, nw = 0.f;
  for (int k = 0; k < 4; ++k) {
    float t = s.th[k];
    if (t <= 0.f) continue;
    total += t;
    cur += t * s.cu[k];
    float csum = 0.f, lm = 0.f, ty = 0.f;
    for (int q = 0; q < 12; ++q) {
      float cc = s.pg[k][q];
      if (cc > 0.f) {
        csum += cc;
        lm += cc * logf(fmaxf(__ldg(pigtab + q * 40 + 32), 1e-3f));
        ty += cc * s.pg[k][13];
      }
    }
    if (s.pg[k][14] > 0.f) lm = csum * (s.pg[k][14] - 10.0f);
    if (csum > 0.f) {
      lnmu += t * lm / csum;
      tau += t * ty / csum;
      wsum += t;
      if (s.pg[k][15] > 0.f) { nsum += t * s.pg[k][15]; nw += t; }
    }
    thin += t * s.pg[k][12];
  }
  if (total <= 0.f) { mu_o = 1.f; ty_o = 0.f; n_o = P.phys[2]; return; }
  float mu = logf(P.misc[2]);
  float ty = 0.f;
  if (wsum > 0.f) { mu = lnmu / wsum; ty = tau / wsum; }
  float tf = fminf(fmaxf(thin / total, 0.f), 0.95f);
  float cb = cur / total;
  mu += 3.0f * logf(1.0f - tf) + P.cure[2] * cb * cb;
  ty = ty * powf(1.0f - tf, 4.0f) + P.cure[1] * cb * cb;
  mu_o = expf(mu);
  ty_o = ty;
  n_o = nw > 0.f ? nsum / nw : P.phys[2];
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

}  // namespace cfk
