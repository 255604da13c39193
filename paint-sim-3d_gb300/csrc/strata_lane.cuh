// strata_lane.cuh — the strata stack (strata.wgsl:37-155) and the KM shade
// with composition (shade.wgsl:28-84, cure.wgsl:3-48) for one cell per
// half-warp.
//
// Lane q (0..15) of the half-warp holds pigment slot q of each of the four
// strata; in the shade it also owns band q.  Thicknesses and cure fractions
// are kept by every lane and stay equal on all 16 lanes, because every lane
// computes them from the same values in the same order, and the half-warp
// sums are xor butterflies, which give every lane the same bits.  So each
// branch on them is taken by the whole half-warp, and the shuffles inside
// such a branch see all 16 lanes.
//
// Pigment mixes take one division per lane instead of sixteen per thread, the
// per-band KM work of a stratum is one band per lane, and no stack slot is
// indexed at run time from local memory.
#pragma once

#include "strata_device.cuh"

namespace cfk {

struct HalfWarp {
  unsigned mask;  // the half-warp's 16 lanes
  int q;          // slot / band of this lane
  __device__ __forceinline__ explicit HalfWarp(int lane) : mask(0xffffu << (lane & 16)), q(lane & 15) {}
  __device__ __forceinline__ float sum(float v) const {
    v += __shfl_xor_sync(mask, v, 8, 16);
    v += __shfl_xor_sync(mask, v, 4, 16);
    v += __shfl_xor_sync(mask, v, 2, 16);
    v += __shfl_xor_sync(mask, v, 1, 16);
    return v;
  }
  __device__ __forceinline__ float get(float v, int slot) const { return __shfl_sync(mask, v, slot, 16); }
};

template <class T>
__device__ __forceinline__ T get4(const T (&v)[4], int k) {
  return k == 0 ? v[0] : k == 1 ? v[1] : k == 2 ? v[2] : v[3];
}
template <class T>
__device__ __forceinline__ void set4(T (&v)[4], int k, T x) {
#pragma unroll
  for (int i = 0; i < 4; ++i)
    if (i == k) v[i] = x;
}

// Slot q of stratum k of cell c in a chunk-major pigment plane.
template <int MODE>
struct PigLane {
  static constexpr bool F32 = MODE == CF_PREC_FP32;
  __device__ static __forceinline__ size_t at(const Film& F, uint32_t c, int k, int q) {
    if constexpr (F32) return ((size_t)(k * 4 + (q >> 2)) * F.n + c) * 4 + (q & 3);
    else return ((size_t)(k * 2 + (q >> 3)) * F.n + c) * 8 + (q & 7);
  }
  __device__ static __forceinline__ float load(const Film& F, const uint4* base, uint32_t c, int k, int q) {
    if constexpr (F32) return reinterpret_cast<const float*>(base)[at(F, c, k, q)];
    else {
      uint32_t b = reinterpret_cast<const uint16_t*>(base)[at(F, c, k, q)];
      return MODE == CF_PREC_REFERENCE ? h16_to_f(b) : slot_from_b16(b, q);
    }
  }
  __device__ static __forceinline__ void store(const Film& F, uint4* base, uint32_t c, int k, int q, float v) {
    if constexpr (F32) reinterpret_cast<float*>(base)[at(F, c, k, q)] = v;
    else reinterpret_cast<uint16_t*>(base)[at(F, c, k, q)] =
        (uint16_t)(MODE == CF_PREC_REFERENCE ? f_to_h16(v) : b16_from_slot(v, q));
  }
  // the value a store of slot q followed by a load gives
  __device__ static __forceinline__ float round(float v, int q) {
    if constexpr (F32) return v;
    else if constexpr (MODE == CF_PREC_REFERENCE) return h16_to_f(f_to_h16(v));
    else return slot_from_b16(b16_from_slot(v, q), q);
  }
};

struct LaneStack {
  float th[4];  // equal on all lanes
  float cu[4];  // equal on all lanes
  float pg[4];  // this lane's slot of each stratum
};

// pig_mix (strata.wgsl:45-60) for this lane's slot: slots 14 and 15
// (ln mu + 10, flow index) mix over the carriers that have a value.  Every
// lane runs the same instructions (selects, one fast division of at most 2
// ulp): the half-warp does not split on the slot.
__device__ __forceinline__ float lane_mix(int q, float a, float wa, float b, float wb) {
  const bool carried = q >= 14;
  const float va = (carried && !(a > 0.f)) ? 0.f : wa;
  const float vb = (carried && !(b > 0.f)) ? 0.f : wb;
  const float den = carried ? va + vb : fmaxf(wa + wb, 1e-20f);
  const float r = __fdividef(a * va + b * vb, den);
  return (carried && !(den > 0.f)) ? 0.f : r;
}
// pig_dist (strata.wgsl:37-43) over slots 0..12
__device__ __forceinline__ float lane_dist(const HalfWarp& H, float a, float b) {
  return H.sum(H.q < 13 ? fabsf(a - b) : 0.f);
}
__device__ __forceinline__ uint32_t lane_count(const LaneStack& s) {  // strata.wgsl:62-68
  uint32_t n = 0;
#pragma unroll
  for (int k = 0; k < 4; ++k)
    if (s.th[k] > 0.f) n = k + 1;
  return n;
}
// strata.wgsl:70-85: stratum a+1 merged into a, the ones above move down
__device__ __forceinline__ void lane_merge(const HalfWarp& H, LaneStack& s, int a) {
  const float ta = get4(s.th, a), tb = get4(s.th, a + 1);
  const float pm = lane_mix(H.q, get4(s.pg, a), ta, get4(s.pg, a + 1), tb);
  const float cm = __fdividef(get4(s.cu, a) * ta + get4(s.cu, a + 1) * tb, fmaxf(ta + tb, 1e-20f));
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    if (k == a) {
      s.pg[k] = pm;
      s.cu[k] = cm;
      s.th[k] = ta + tb;
    } else if (k > a) {
      if (k < 3) {
        s.th[k] = s.th[k + 1];
        s.cu[k] = s.cu[k + 1];
        s.pg[k] = s.pg[k + 1];
      } else {
        s.th[3] = 0.f;
        s.cu[3] = 0.f;
      }
    }
  }
}
__device__ __forceinline__ void lane_compact(const HalfWarp& H, LaneStack& s, float tiny) {  // strata.wgsl:87-103
  // Each pass changes nothing unless one of its conditions holds for the stack
  // as it enters the pass, so a stack without a gap (or without a thin
  // stratum under another) skips that pass's unrolled, predicated moves.
  auto gap = [&](int k) { return s.th[k] <= 0.f && s.th[k + 1] > 0.f; };
  if (gap(0) || gap(1) || gap(2)) {
#pragma unroll
    for (int sweep = 0; sweep < 4; ++sweep)
#pragma unroll
      for (int k = 0; k < 3; ++k)
        if (gap(k)) {
          s.th[k] = s.th[k + 1];
          s.cu[k] = s.cu[k + 1];
          s.pg[k] = s.pg[k + 1];
          s.th[k + 1] = 0.f;
          s.cu[k + 1] = 0.f;
        }
  }
  auto thin = [&](int k) { return s.th[k] > 0.f && s.th[k] < tiny && s.th[k + 1] > 0.f; };
  if (thin(0) || thin(1) || thin(2)) {
#pragma unroll
    for (int k = 0; k < 3; ++k)
      if (thin(k)) lane_merge(H, s, k);
  }
}
// strata.wgsl:105-131
__device__ __forceinline__ void lane_push_top(const HalfWarp& H, LaneStack& s, float vol, float pin, float cv,
                                              float tiny, float close_d) {
  if (vol <= 0.f) return;
  const uint32_t n = lane_count(s);
  if (n > 0) {
    const int t = (int)n - 1;
    const float tt = get4(s.th, t), pt = get4(s.pg, t);
    const bool close = lane_dist(H, pt, pin) < close_d || tt < tiny;
    if (close) {
      set4(s.pg, t, lane_mix(H.q, pt, tt, pin, vol));
      set4(s.cu, t, __fdividef(get4(s.cu, t) * tt + cv * vol, tt + vol));
      set4(s.th, t, tt + vol);
      return;
    }
  }
  if (n == 4) {
    const float d0 = lane_dist(H, s.pg[0], s.pg[1]);
    const float d1 = lane_dist(H, s.pg[1], s.pg[2]);
    const float d2 = lane_dist(H, s.pg[2], s.pg[3]);
    int best = 0;
    float bd = 1e30f;
    if (d0 < bd) { bd = d0; best = 0; }
    if (d1 < bd) { bd = d1; best = 1; }
    if (d2 < bd) { bd = d2; best = 2; }
    lane_merge(H, s, best);
  }
  const int t = (int)lane_count(s);
  set4(s.th, t, vol);
  set4(s.pg, t, pin);
  set4(s.cu, t, cv);
}
// strata.wgsl:133-155
__device__ __forceinline__ void lane_add_band(const HalfWarp& H, LaneStack& s, float zlo, float zhi, float vol,
                                              float pin, float cv, float tiny, float close_d) {
  if (vol <= 0.f) return;
  const float span = fmaxf(zhi - zlo, 1e-12f);
  float z0 = 0.f, above = vol;
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    const float tk = s.th[k];
    if (tk <= 0.f) break;
    // from here up the strata lie above the band: their overlaps are 0, so
    // their parts are +0 and change nothing
    if (z0 >= zhi) break;
    const float z1 = z0 + tk;
    const float ov = fmaxf(fminf(zhi, z1) - fmaxf(zlo, z0), 0.f);
    // exact division (`above` below is compared with 1e-14), skipped where
    // the overlap is 0 and the part therefore +0
    const float part = ov > 0.f ? vol * ov / span : 0.f;
    if (part > 0.f) {
      s.pg[k] = lane_mix(H.q, s.pg[k], tk, pin, part);
      s.cu[k] = __fdividef(s.cu[k] * tk + cv * part, tk + part);
      s.th[k] = tk + part;
      above -= part;
    }
    z0 = z1;
  }
  if (above > 1e-14f) lane_push_top(H, s, above, pin, cv, tiny, close_d);
}

// CellAcc with one band per lane: the composition sums are half-warp sums
// over the 12 pigment lanes, the reflectance of band q stays in lane q.
struct LaneAcc {
  float total, lnmu, tau, thin, wsum, nsum, nw;  // equal on all lanes
  float r;                                       // band q
  float wet, cure_top, ssum;
  uint32_t cnt;
  bool bad;

  __device__ __forceinline__ void begin(const HalfWarp& H, const uint16_t* rf) {
    total = lnmu = tau = thin = wsum = nsum = nw = 0.f;
    wet = cure_top = ssum = 0.f;
    cnt = 0;
    bad = false;
    r = h16_to_f(rf[H.q]);
  }
  // xs: 32 floats of the half-warp's shared memory, 16-byte aligned, where
  // the lanes leave their slot and pigment weight for the others to read
  // (four vector loads instead of sixteen shuffles)
  __device__ __forceinline__ void add(const HalfWarp& H, int k, float t, float u, float pg, float hv,
                                      const float* lnmu_tab, const float* tab, float* xs, bool debug) {
    ssum += t;
    if (!(t > 0.f)) return;
    total += t;
    const int q = H.q;
    const float cc = (q < 12 && pg > 0.f) ? pg : 0.f;
    const float wq = cc * tab[(q < 12 ? q : 0) * 40 + 34];
    __syncwarp(H.mask);  // the previous stratum's (or caller's) values have been read
    xs[q] = pg;
    xs[16 + q] = wq;
    __syncwarp(H.mask);
    const float4 ps = reinterpret_cast<const float4*>(xs)[3];
    const float p12 = ps.x, p13 = ps.y, p14 = ps.z, p15 = ps.w;
    const float csum = H.sum(cc);
    float lm = H.sum(cc * lnmu_tab[q < 12 ? q : 0]);
    const float ty = H.sum(cc * p13);
    if (p14 > 0.f) lm = csum * (p14 - 10.0f);
    if (csum > 0.f) {
      lnmu += t * lm / csum;
      tau += t * ty / csum;
      wsum += t;
      if (p15 > 0.f) { nsum += t * p15; nw += t; }
    }
    thin += t * p12;
    if (hv > 0.f) {
      // km.wgsl:17-33: weights w_p = c_p g_p of the pigment lanes, then band q
      const float scale = csum / fmaxf(H.sum(wq), 1e-9f);
      const float4 w0 = reinterpret_cast<const float4*>(xs)[4], w1 = reinterpret_cast<const float4*>(xs)[5],
                   w2 = reinterpret_cast<const float4*>(xs)[6];
      const float w[12] = {w0.x, w0.y, w0.z, w0.w, w1.x, w1.y, w1.z, w1.w, w2.x, w2.y, w2.z, w2.w};
      float kk = 0.f, ss = 0.f;
#pragma unroll
      for (int p = 0; p < 12; ++p) {
        kk += w[p] * tab[p * 40 + q];
        ss += w[p] * tab[p * 40 + 16 + q];
      }
      float rr, tt;
      km_layer(kk * scale, ss * scale, t, rr, tt);
      r = composite(rr, tt, r);
      wet = 1.0f - u;
      cure_top = u;
    }
    cnt = k + 1;
    if (debug) {
      const float cs = H.sum(q < 13 ? pg : 0.f);
      if (!(cs > 0.f)) bad = true;
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
  __device__ __forceinline__ ushort4 color(const HalfWarp& H, const cf_params& P, const float* cm, float hv,
                                           float mv) const {
    const float k1 = 0.04f;
    const float wt = hv > 0.f ? wet : 0.f;
    const float k2 = 0.4f * (1.0f - wt) + 0.6f * wt;
    const float rb = __fdividef((1.0f - k1) * (1.0f - k2) * r, fmaxf(1.0f - k2 * r, 1e-3f));  // colour is stored as f16
    const float X = H.sum(rb * cm[3 * H.q]), Y = H.sum(rb * cm[3 * H.q + 1]), Z = H.sum(rb * cm[3 * H.q + 2]);
    float rgb[3] = {3.2406f * X - 1.5372f * Y - 0.4986f * Z, -0.9689f * X + 1.8758f * Y + 0.0415f * Z,
                    0.0557f * X - 0.2040f * Y + 1.0570f * Z};
#pragma unroll
    for (int c = 0; c < 3; ++c) rgb[c] = fmaxf(rgb[c], 0.f);
    auto smooth = [](float e0, float e1, float x) {
      float t = fminf(fmaxf((x - e0) / (e1 - e0), 0.f), 1.f);
      return t * t * (3.0f - 2.0f * t);
    };
    const float painted = smooth(60e-6f, 150e-6f, mv);
    const float ct = fmaxf(hv > 0.f ? cure_top : 0.f, painted * (1.0f - smooth(0.f, 50e-6f, hv)));
    const float sq = sqrtf(ct);
    float rough = 0.06f * (1.0f - sq) + 0.35f * sq;
    if (hv <= 0.f) rough = 0.85f * (1.0f - painted) + 0.35f * painted;
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

}  // namespace cfk
