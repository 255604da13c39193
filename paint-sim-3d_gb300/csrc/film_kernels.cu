// film_kernels.cu — sm_103a kernels of the thin-film step, one per dispatch of
// Film::encode_frame (src/film/mod.rs:1322-1462), plus stats and state I/O.
//
// Launch geometry: one 16x16 block per 16x16 activity tile.  A tile-list
// dispatch of the reference (dispatch_workgroups_indirect over the active
// tiles) becomes a full-grid launch whose blocks on inactive tiles return at
// once, so the active set stays on the device and the frame has no host
// round trip.  Dispatches whose invocations read what the same dispatch
// writes in the reference (nose, strata_fill) read a snapshot here.
#include <cuda_runtime.h>

#include <string_view>

#include "film_device.cuh"
#include "film_kernels.h"
#include "strata_device.cuh"

namespace cfk {

#define TILE_PROLOGUE                                              \
  const int i = (int)(blockIdx.x * 16 + threadIdx.x);              \
  const int j = (int)(blockIdx.y * 16 + threadIdx.y);              \
  if ((F.tile_flags[blockIdx.x + blockIdx.y * F.tw] & ACTIVE) == 0u) return; \
  if (i >= (int)F.w || j >= (int)F.h) return;                      \
  const uint32_t c = idx(F, i, j);                                 \
  const DevParams& D = *F.P;                                       \
  const cf_params& P = D.p;                                        \
  (void)P;

// film.wgsl:1365-1391
__global__ void __launch_bounds__(256) k_mark_tiles(Film F) {
  __shared__ uint32_t any;
  if (threadIdx.x == 0 && threadIdx.y == 0) any = 0u;
  __syncthreads();
  const int i = (int)(blockIdx.x * 16 + threadIdx.x), j = (int)(blockIdx.y * 16 + threadIdx.y);
  if (i < (int)F.w && j < (int)F.h) {
    uint32_t c = idx(F, i, j);
    float hv = F.hh[c];
    if (hv > 0.f) {
      uint32_t bits = 1u;
      if (threadIdx.x < 8) bits |= 2u;
      if (threadIdx.x >= 8) bits |= 4u;
      if (threadIdx.y < 8) bits |= 8u;
      if (threadIdx.y >= 8) bits |= 16u;
      if (fabsf(hv - F.h_frame[c]) > FRAME_EPS) bits |= MOVED;
      atomicOr(&any, bits);
    }
  }
  __syncthreads();
  if (threadIdx.x == 0 && threadIdx.y == 0) {
    uint32_t t = blockIdx.x + blockIdx.y * F.tw;
    uint32_t flags = any;
    if (F.tile_moved[t] != 0u) flags |= MOVED;
    F.tile_moved[t] = 0u;
    F.tile_flags[t] = flags;
  }
}

// film.wgsl:1393-1425 (bit 32 is written in place; the bits read are not it)
__global__ void __launch_bounds__(256) k_compact_tiles(Film F, int all_active) {
  uint32_t nt = F.tw * F.th;
  uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nt) return;
  int tx = (int)(t % F.tw), ty = (int)(t / F.tw);
  uint32_t own = F.tile_flags[t];
  uint32_t any = own & MOVED;
  for (int dy = -1; dy <= 1; ++dy)
    for (int dx = -1; dx <= 1; ++dx) {
      if (dx == 0 && dy == 0) continue;
      int x = tx + dx, y = ty + dy;
      if (x >= 0 && y >= 0 && x < (int)F.tw && y < (int)F.th) {
        uint32_t fl = F.tile_flags[(uint32_t)x + (uint32_t)y * F.tw];
        bool need = true;
        if (dx == 1 && (fl & 2u) == 0u) need = false;
        if (dx == -1 && (fl & 4u) == 0u) need = false;
        if (dy == 1 && (fl & 8u) == 0u) need = false;
        if (dy == -1 && (fl & 16u) == 0u) need = false;
        if (need) any |= fl & MOVED;
      }
    }
  if (all_active) any = 1u;
  if (any != 0u) {
    F.tile_flags[t] = (own & ~ACTIVE) | ACTIVE;
    atomicAdd(&F.stats->active_tiles, 1u);
  } else {
    F.tile_flags[t] = own & 31u;
  }
}

// cure.wgsl:119-159 (full grid)
template <int MODE>
__global__ void __launch_bounds__(256) k_cure(Film F) {
  const int i = (int)(blockIdx.x * 16 + threadIdx.x), j = (int)(blockIdx.y * 16 + threadIdx.y);
  if (i >= (int)F.w || j >= (int)F.h) return;
  const uint32_t c = idx(F, i, j);
  const cf_params& P = F.P->p;
  float hv = F.hh[c];
  if (hv <= 0.f) { set_rheo<MODE>(F, c, 1.f, 0.f, P.phys[2]); return; }
  float rate = P.cure[0] * P.frame_dt;
  float4 t4 = F.sh[c], c4 = F.scu[c];
  float t[4] = {t4.x, t4.y, t4.z, t4.w}, u[4] = {c4.x, c4.y, c4.z, c4.w};
#pragma unroll
  for (int k = 0; k < 4; ++k) u[k] = t[k] > 0.f ? fminf(u[k] + rate, 1.f) : u[k];
  Stack s;
  stack_load<MODE>(F, F.pig, c, s);
#pragma unroll
  for (int k = 0; k < 4; ++k) s.cu[k] = u[k];
  if (!(t[0] > 0.f && u[0] >= 1.f)) {
    F.scu[c] = make_float4(u[0], u[1], u[2], u[3]);
    float mu, ty, n;
    composition_rheo(P, F.pigtab, s, mu, ty, n);
    set_rheo<MODE>(F, c, mu, ty, n);
    return;
  }
  float committed = 0.f;
  uint32_t guard = 0;
  uint16_t* rf = F.refl + (size_t)c * 16;
  while (s.th[0] > 0.f && s.cu[0] >= 1.f && guard < 4u) {
    guard++;
    float w[12], sc;
    layer_weights(s.pg[0], F.pigtab, w, sc);
    for (int b = 0; b < 16; ++b) {
      float kk, ss, rr, tt;
      layer_ks_band(s.pg[0], w, sc, F.pigtab, b, kk, ss);
      km_layer(kk, ss, s.th[0], rr, tt);
      float v = composite(rr, tt, half_at(rf, b));
      rf[b] = __half_as_ushort(__float2half_rn(v));
    }
    committed += s.th[0];
    F.m[c] = F.m[c] + s.th[0] * (1.0f - 0.04f) * (1.0f - fminf(fmaxf(s.pg[0][12], 0.f), 0.95f));
    s.th[0] = 0.f;
    s.cu[0] = 0.f;
    stack_compact(s, P.misc[0]);
  }
  if (committed > 0.f) F.hh[c] = fmaxf(F.hh[c] - committed, 0.f);
  float mu, ty, n;
  composition_rheo(P, F.pigtab, s, mu, ty, n);
  set_rheo<MODE>(F, c, mu, ty, n);
  stack_store<MODE>(F.sh, F.scu, F.pig, c, s);
}

// film.wgsl:1427-1434
__global__ void __launch_bounds__(256) k_clear_acc(Film F) {
  TILE_PROLOGUE
  F.acc[c] = make_float4(0.f, 0.f, 0.f, 0.f);
  F.h_frame[c] = F.hh[c];
}

// film.wgsl:16-42
__global__ void __launch_bounds__(256) k_laplacian(Film F) {
  TILE_PROLOGUE
  float hv = F.hh[c];
  float s0 = hv + F.m[c];
  float hold = 0.f, pl = 0.f;
  if (hv > 0.f) hold = hold_level(P, nose_dist(F, c));
  float u0 = s0 - hold;
  float ax = usurf(F, P, i - 1, j) + usurf(F, P, i + 1, j) + usurf(F, P, i, j - 1) + usurf(F, P, i, j + 1);
  float dg = usurf(F, P, i - 1, j - 1) + usurf(F, P, i + 1, j - 1) + usurf(F, P, i - 1, j + 1) +
             usurf(F, P, i + 1, j + 1);
  float l = (W_AXIS * ax + W_DIAG_LAP * dg - (4.0f * W_AXIS + 4.0f * W_DIAG_LAP) * u0) * P.inv_dx * P.inv_dx;
  if (hv > 0.f) {
    float d = nose_dist(F, c);
    if (d <= 3.0f) {
      float2 n = F.fnorm[c];
      if (n.x * n.x + n.y * n.y > 0.5f) pl = line_pressure(F, P, i, j) * expf(-(d - 1.0f) * 0.7f);
    }
  }
  F.pres[c] = make_float2(-P.phys[1] * l + disjoining(P, hv), P.phys[0] * P.g[2] * (s0 - hold) + pl);
}

// film.wgsl:58-87
template <int MODE>
__global__ void __launch_bounds__(256) k_plug(Film F) {
  TILE_PROLOGUE
  F.tmp[c] = 0.f;
  if (F.hh[c] <= 0.f) return;
  float gb = P.phys[0] * D.gxy;
  if (gb < 1e-6f) return;
  float sum = 0.f, mass = 0.f;
  bool yielding = false;
  for (int dy = -3; dy <= 3; ++dy)
    for (int dx = -3; dx <= 3; ++dx) {
      int x = i + dx, y = j + dy;
      if (!in_grid(F, x, y)) continue;
      uint32_t n = idx(F, x, y);
      float hn = F.hh[n];
      if (hn <= 0.f) continue;
      float rx = rmu<MODE>(F, n), ry = rtau<MODE>(F, n);
      if (ry > 0.f) yielding = true;
      float q, yy, up;
      hb_flux(gb, hn, fmaxf(rx, 1e-4f), ry, rn<MODE>(F, n), q, yy, up);
      sum += q;
      mass += hn;
    }
  if (!yielding || mass <= 0.f) return;
  F.tmp[c] = sum / mass;
}

// film.wgsl:448-455
template <int MODE>
__global__ void __launch_bounds__(256) k_fluxes(Film F) {
  TILE_PROLOGUE
  float q[4];
#pragma unroll 1
  for (int k = 0; k < 4; ++k) q[k] = face_k<MODE>(F, D, i, j, k).q;
  F.flux[c] = make_float4(q[0], q[1], q[2], q[3]);
}

// film.wgsl:516-537
__device__ __forceinline__ bool nb_ok(const Film& F, int i, int j) { return in_grid(F, i, j) && cell_active(F, i, j); }
__global__ void __launch_bounds__(256) k_limiter(Film F) {
  TILE_PROLOGUE
  float4 f = F.flux[c];
  float out = fmaxf(f.x, 0.f) + fmaxf(f.y, 0.f) + fmaxf(f.z, 0.f) + fmaxf(f.w, 0.f);
  if (nb_ok(F, i - 1, j)) out += fmaxf(-F.flux[idx(F, i - 1, j)].x, 0.f);
  if (nb_ok(F, i, j - 1)) out += fmaxf(-F.flux[idx(F, i, j - 1)].y, 0.f);
  if (nb_ok(F, i - 1, j - 1)) out += fmaxf(-F.flux[idx(F, i - 1, j - 1)].z, 0.f);
  if (nb_ok(F, i - 1, j + 1)) out += fmaxf(-F.flux[idx(F, i - 1, j + 1)].w, 0.f);
  float a = 1.f;
  if (out > 0.f) a = fminf(1.f, 0.5f * F.hh[c] * P.dx / (P.dt * out));
  F.alpha[c] = a;
}

// wetting back-fill: film.wgsl:847-860 / strata.wgsl:314-322
template <int MODE>
__device__ __forceinline__ void backfill(const Film& F, uint32_t c, uint32_t src, float hn) {
  float4 ts = F.sh[src];
  int ks = 0;
  if (ts.x > 0.f) ks = 0;
  if (ts.y > 0.f) ks = 1;
  if (ts.z > 0.f) ks = 2;
  if (ts.w > 0.f) ks = 3;
  F.sh[c] = make_float4(hn, 0.f, 0.f, 0.f);
  using Pig = typename Prec<MODE>::Pig;
  copy_pig16<Pig>(pig_at<MODE>(F.pig, c, 0), pig_at<MODE>(F.pig, src, ks));
#pragma unroll
  for (int k = 1; k < 4; ++k) zero_pig16<Pig>(pig_at<MODE>(F.pig, c, k));
  float4 cs = F.scu[src];
  float cv = ks == 0 ? cs.x : (ks == 1 ? cs.y : (ks == 2 ? cs.z : cs.w));
  F.scu[c] = make_float4(cv, 0.f, 0.f, 0.f);
}

// film.wgsl:539-561, 803-863
template <int MODE>
__global__ void __launch_bounds__(256) k_apply(Film F) {
  const int i = (int)(blockIdx.x * 16 + threadIdx.x), j = (int)(blockIdx.y * 16 + threadIdx.y);
  if ((F.tile_flags[blockIdx.x + blockIdx.y * F.tw] & ACTIVE) == 0u) return;
  bool moved = false;
  if (i < (int)F.w && j < (int)F.h) {
    const cf_params& P = F.P->p;
    uint32_t c = idx(F, i, j);
    float ac = F.alpha[c];
    float best = 0.f, div = 0.f;
    uint32_t src = c;
    float4 f4 = F.flux[c];
    float f[4] = {f4.x, f4.y, f4.z, f4.w};
    bool hx = i + 1 < (int)F.w, hy = j + 1 < (int)F.h, hm = j > 0;
    uint32_t cbs[4] = {hx ? c + 1 : c, hy ? c + F.w : c, (hx && hy) ? c + F.w + 1 : c, (hx && hm) ? c - F.w + 1 : c};
    bool has[4] = {hx, hy, hx && hy, hx && hm};
    float accv[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      float q = f[k], ab = ac;
      if (q < 0.f && has[k]) {
        ab = F.alpha[cbs[k]];
        if (-q * ab > best) { best = -q * ab; src = cbs[k]; }
      }
      div += q * ab;
      accv[k] = q * ab;
    }
    auto nb_face = [&](float q, uint32_t cn) {
      float an = F.alpha[cn];
      if (q < 0.f) an = ac;
      if (q * an > best) { best = q * an; src = cn; }
      div -= q * an;
    };
    if (nb_ok(F, i - 1, j)) nb_face(F.flux[c - 1].x, c - 1);
    if (nb_ok(F, i, j - 1)) nb_face(F.flux[c - F.w].y, c - F.w);
    if (nb_ok(F, i - 1, j - 1)) nb_face(F.flux[c - F.w - 1].z, c - F.w - 1);
    if (nb_ok(F, i - 1, j + 1)) nb_face(F.flux[c + F.w - 1].w, c + F.w - 1);
    float h0 = F.hh[c];
    float hn = fmaxf(h0 - P.dt * div * P.inv_dx, 0.f);
    if (hn < h0 && hn < DRAINED_FILM) hn = 0.f;
    F.hh[c] = hn;
    moved = fabsf(hn - h0) > MOVE_EPS;
    if (h0 <= 0.f && src != c) {
      set_rheo<MODE>(F, c, rmu<MODE>(F, src), rtau<MODE>(F, src), rn<MODE>(F, src));
      backfill<MODE>(F, c, src, hn);
    }
    float4 a = F.acc[c];
    F.acc[c] = make_float4(a.x + accv[0] * P.dt, a.y + accv[1] * P.dt, a.z + accv[2] * P.dt, a.w + accv[3] * P.dt);
  }
  if (__syncthreads_or(moved) && threadIdx.x == 0 && threadIdx.y == 0)
    F.tile_moved[blockIdx.x + blockIdx.y * F.tw] = 1u;
}

// film.wgsl:680-723, reading delta_old (Jacobi)
__global__ void __launch_bounds__(256) k_nose(Film F) {
  TILE_PROLOGUE
  if (F.hh[c] <= 0.f) {
    F.delta[c] = 0u;
    F.fnorm[c] = make_float2(0.f, 0.f);
    return;
  }
  int bx = 64, by = 64;
  float bd = 1e9f;
  for (int dj = -1; dj <= 1; ++dj)
    for (int di = -1; di <= 1; ++di) {
      int x = i + di, y = j + dj;
      if (!in_grid(F, x, y)) continue;
      uint32_t n = idx(F, x, y);
      int cx = di, cy = dj;
      if (F.hh[n] > 0.f) {
        uint32_t dn = F.delta_old[n];
        if ((dn & 0x10000u) == 0u) continue;
        int ox, oy;
        unpack_off(dn, ox, oy);
        cx = ox + di;
        cy = oy + dj;
        int tx = i + cx, ty = j + cy;
        if (!in_grid(F, tx, ty)) continue;
        if (F.hh[idx(F, tx, ty)] > 0.f) continue;
      } else if (di == 0 && dj == 0) {
        continue;
      }
      float d = off_len(cx, cy);
      if (d < bd) { bd = d; bx = cx; by = cy; }
    }
  if (bd > 1e8f) {
    F.delta[c] = 0u;
    F.fnorm[c] = make_float2(0.f, 0.f);
    return;
  }
  F.delta[c] = pack_off(bx, by);
  F.fnorm[c] = bd <= 3.0f ? front_normal(F, P, c) : make_float2(0.f, 0.f);
}

// film.wgsl:457-473
__device__ __forceinline__ float4 band_split(const Film& F, uint32_t cu, float hf, float y, float up, float total,
                                             float n) {
  float4 s = F.sh[cu];
  float hu = s.x + s.y + s.z + s.w;
  if (hu <= 0.f) return make_float4(total, 0.f, 0.f, 0.f);
  float fr[4] = {s.x / hu, s.y / hu, s.z / hu, s.w / hu};
  if (y > 0.f && up > 0.f) {
    float k = hf / hu;
    float z1 = s.x * k;
    float z2 = z1 + s.y * k;
    float z3 = z2 + s.z * k;
    float z4 = z3 + s.w * k;
    float b[4] = {band_flux(up, y, 0.f, z1, n), band_flux(up, y, z1, z2, n), band_flux(up, y, z2, z3, n),
                  band_flux(up, y, z3, z4, n)};
    float bs = b[0] + b[1] + b[2] + b[3];
    if (bs > 0.f) {
#pragma unroll
      for (int q = 0; q < 4; ++q) fr[q] = b[q] / bs;
    }
  }
  return make_float4(fr[0] * total, fr[1] * total, fr[2] * total, fr[3] * total);
}

// film.wgsl:475-514
template <int MODE>
__global__ void __launch_bounds__(256) k_strata_split(Film F) {
  TILE_PROLOGUE
  float4 a4 = F.acc[c];
  float a[4] = {a4.x, a4.y, a4.z, a4.w};
  const int ni[4] = {1, 0, 1, 1}, nj[4] = {0, 1, 1, -1};
  bool ok[4] = {i + 1 < (int)F.w, j + 1 < (int)F.h, i + 1 < (int)F.w && j + 1 < (int)F.h, i + 1 < (int)F.w && j > 0};
#pragma unroll 1
  for (int k = 0; k < 4; ++k) {
    FaceOut ff = face_k<MODE>(F, D, i, j, k);
    float4 o = make_float4(0.f, 0.f, 0.f, 0.f);
    if (a[k] != 0.f && ok[k]) {
      uint32_t cb = idx(F, i + ni[k], j + nj[k]);
      uint32_t cu = a[k] < 0.f ? cb : c;
      o = band_split(F, cu, 0.5f * (F.hh[c] + F.hh[cb]), ff.y, ff.up, a[k], ff.n);
    }
    F.acc_s[4 * (size_t)c + k] = o;
  }
}

// film.wgsl:1330-1361, plus the device-wide max/min the adaptive step reads
template <int MODE>
__global__ void __launch_bounds__(256) k_reduce_tiles(Film F) {
  const cf_params& P = F.P->p;
  float hm = 0.f, mm = 1e9f;
  for (int dy = 0; dy < 4; ++dy)
    for (int dx = 0; dx < 4; ++dx) {
      int i = blockIdx.x * 64 + threadIdx.x * 4 + dx, j = blockIdx.y * 64 + threadIdx.y * 4 + dy;
      if (i < (int)F.w && j < (int)F.h) {
        uint32_t c = idx(F, i, j);
        float v = F.hh[c];
        if (v > 4.0f * P.ein[3]) { hm = fmaxf(hm, v); mm = fminf(mm, rmu<MODE>(F, c)); }
      }
    }
  for (int o = 16; o > 0; o >>= 1) {
    hm = fmaxf(hm, __shfl_xor_sync(0xffffffffu, hm, o));
    mm = fminf(mm, __shfl_xor_sync(0xffffffffu, mm, o));
  }
  __shared__ float sh[8], sm[8];
  int lane = (threadIdx.y * 16 + threadIdx.x) & 31, wid = (threadIdx.y * 16 + threadIdx.x) >> 5;
  if (lane == 0) { sh[wid] = hm; sm[wid] = mm; }
  __syncthreads();
  if (wid == 0) {
    hm = lane < 8 ? sh[lane] : 0.f;
    mm = lane < 8 ? sm[lane] : 1e9f;
    for (int o = 4; o > 0; o >>= 1) {
      hm = fmaxf(hm, __shfl_xor_sync(0xffffffffu, hm, o));
      mm = fminf(mm, __shfl_xor_sync(0xffffffffu, mm, o));
    }
    if (lane == 0) {
      F.stats64[blockIdx.x + blockIdx.y * gridDim.x] = make_float2(hm, mm);
      atomicMax(&F.stats->h_max_bits, __float_as_uint(hm));
      atomicMin(&F.stats->mu_min_bits, __float_as_uint(mm));
    }
  }
}

// strata.wgsl:157-173
__global__ void __launch_bounds__(256) k_strata_limit(Film F) {
  TILE_PROLOGUE
  float out[4];
  const float4* as = F.acc_s + 4 * (size_t)c;
  float4 a0 = as[0], a1 = as[1], a2 = as[2], a3 = as[3];
  out[0] = fmaxf(a0.x, 0.f) + fmaxf(a1.x, 0.f) + fmaxf(a2.x, 0.f) + fmaxf(a3.x, 0.f);
  out[1] = fmaxf(a0.y, 0.f) + fmaxf(a1.y, 0.f) + fmaxf(a2.y, 0.f) + fmaxf(a3.y, 0.f);
  out[2] = fmaxf(a0.z, 0.f) + fmaxf(a1.z, 0.f) + fmaxf(a2.z, 0.f) + fmaxf(a3.z, 0.f);
  out[3] = fmaxf(a0.w, 0.f) + fmaxf(a1.w, 0.f) + fmaxf(a2.w, 0.f) + fmaxf(a3.w, 0.f);
  auto addn = [&](uint32_t n, int f) {
    float4 v = F.acc_s[4 * (size_t)n + f];
    out[0] += fmaxf(-v.x, 0.f);
    out[1] += fmaxf(-v.y, 0.f);
    out[2] += fmaxf(-v.z, 0.f);
    out[3] += fmaxf(-v.w, 0.f);
  };
  if (i > 0 && cell_active(F, i - 1, j)) addn(c - 1, 0);
  if (j > 0 && cell_active(F, i, j - 1)) addn(c - F.w, 1);
  if (i > 0 && j > 0 && cell_active(F, i - 1, j - 1)) addn(c - F.w - 1, 2);
  if (i > 0 && j + 1 < (int)F.h && cell_active(F, i - 1, j + 1)) addn(c + F.w - 1, 3);
  float4 th = F.sh[c];
  float t[4] = {th.x, th.y, th.z, th.w}, a[4];
#pragma unroll
  for (int k = 0; k < 4; ++k) a[k] = out[k] > 0.f ? fminf(1.f, t[k] * P.dx / out[k]) : 1.f;
  F.alpha_s[c] = make_float4(a[0], a[1], a[2], a[3]);
}

__device__ __forceinline__ float sel4(float4 v, int k) {
  return k == 0 ? v.x : (k == 1 ? v.y : (k == 2 ? v.z : v.w));
}
__device__ __forceinline__ float4 neg4(float4 v) { return make_float4(-v.x, -v.y, -v.z, -v.w); }

// strata.wgsl:175-188; the face volumes arrive by value (one per stratum).
template <int MODE>
__device__ __forceinline__ void inflow_from(const Film& F, const cf_params& P, Stack& s, uint32_t cn, float4 f) {
  const float4 an4 = F.alpha_s[cn], th4 = F.sh[cn], cu4 = F.scu[cn];
  float z0 = 0.f;
  using Pig = typename Prec<MODE>::Pig;
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    const float thn = sel4(th4, k);
    const float z1 = z0 + thn;
    const float v = sel4(f, k) * sel4(an4, k) * P.inv_dx;
    if (v > 0.f && thn > 0.f) {
      float pg[16];
      load_pig16<Pig>(pig_at<MODE>(F.pig, cn, k), pg);
      stack_add_band(s, z0, z1, v, pg, sel4(cu4, k), P.misc[0], P.misc[1]);
    }
    z0 = z1;
  }
}

// strata.wgsl:190-274
template <int MODE>
__global__ void __launch_bounds__(256) k_strata_update(Film F) {
  TILE_PROLOGUE
  using Pig = typename Prec<MODE>::Pig;
  const float4* as = F.acc_s + 4 * (size_t)c;
  float4 fr4 = as[0], fu4 = as[1], fd4 = as[2], fe4 = as[3];
  float4 z4 = make_float4(0.f, 0.f, 0.f, 0.f);
  float4 fl4 = z4, fdn4 = z4, fll4 = z4, flu4 = z4;
  uint32_t cl = c, cd = c, cll = c, clu = c;
  if (i > 0 && cell_active(F, i - 1, j)) { cl = c - 1; fl4 = F.acc_s[4 * (size_t)cl]; }
  if (j > 0 && cell_active(F, i, j - 1)) { cd = c - F.w; fdn4 = F.acc_s[4 * (size_t)cd + 1]; }
  if (i > 0 && j > 0 && cell_active(F, i - 1, j - 1)) { cll = c - F.w - 1; fll4 = F.acc_s[4 * (size_t)cll + 2]; }
  if (i > 0 && j + 1 < (int)F.h && cell_active(F, i - 1, j + 1)) { clu = c + F.w - 1; flu4 = F.acc_s[4 * (size_t)clu + 3]; }
  auto nz = [](float4 v) { return v.x != 0.f || v.y != 0.f || v.z != 0.f || v.w != 0.f; };
  if (!(nz(fr4) || nz(fu4) || nz(fd4) || nz(fe4) || nz(fl4) || nz(fdn4) || nz(fll4) || nz(flu4))) {
    float hc = F.hh[c];
    float4 t4 = F.sh[c];
    float th[4] = {fmaxf(t4.x, 0.f), fmaxf(t4.y, 0.f), fmaxf(t4.z, 0.f), fmaxf(t4.w, 0.f)};
    float nt[4] = {0.f, 0.f, 0.f, 0.f};
    float4 cu = F.scu[c];
    if (hc <= 0.f) {
      cu = z4;
    } else {
      float sum = th[0] + th[1] + th[2] + th[3];
#pragma unroll
      for (int k = 0; k < 4; ++k) nt[k] = th[k];
      if (sum > 0.f) {
        float sc = hc / sum;
#pragma unroll
        for (int k = 0; k < 4; ++k) nt[k] = th[k] * sc;
      }
    }
    bool plain = true;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      if (nt[k] <= 0.f && nt[k + 1] > 0.f) plain = false;
      if (nt[k] > 0.f && nt[k] < P.misc[0] && nt[k + 1] > 0.f) plain = false;
    }
    if (plain) {
      F.sh2[c] = make_float4(nt[0], nt[1], nt[2], nt[3]);
      F.scu2[c] = cu;
#pragma unroll
      for (int k = 0; k < 4; ++k) copy_pig16<Pig>(pig_at<MODE>(F.pig2, c, k), pig_at<MODE>(F.pig, c, k));
      return;
    }
  }
  Stack s;
  stack_load<MODE>(F, F.pig, c, s);
  const float4 a4 = F.alpha_s[c];
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    float out = fmaxf(sel4(fr4, k), 0.f) + fmaxf(sel4(fu4, k), 0.f) + fmaxf(sel4(fd4, k), 0.f) +
                fmaxf(sel4(fe4, k), 0.f) + fmaxf(-sel4(fl4, k), 0.f) + fmaxf(-sel4(fdn4, k), 0.f) +
                fmaxf(-sel4(fll4, k), 0.f) + fmaxf(-sel4(flu4, k), 0.f);
    s.th[k] = fmaxf(s.th[k] - out * sel4(a4, k) * P.inv_dx, 0.f);
  }
  if (i + 1 < (int)F.w) inflow_from<MODE>(F, P, s, c + 1, neg4(fr4));
  if (j + 1 < (int)F.h) inflow_from<MODE>(F, P, s, c + F.w, neg4(fu4));
  if (i + 1 < (int)F.w && j + 1 < (int)F.h) inflow_from<MODE>(F, P, s, c + F.w + 1, neg4(fd4));
  if (i + 1 < (int)F.w && j > 0) inflow_from<MODE>(F, P, s, c - F.w + 1, neg4(fe4));
  if (cl != c) inflow_from<MODE>(F, P, s, cl, fl4);
  if (cd != c) inflow_from<MODE>(F, P, s, cd, fdn4);
  if (cll != c) inflow_from<MODE>(F, P, s, cll, fll4);
  if (clu != c) inflow_from<MODE>(F, P, s, clu, flu4);
  float hc = F.hh[c];
  float sum = s.th[0] + s.th[1] + s.th[2] + s.th[3];
  if (hc <= 0.f) {
#pragma unroll
    for (int k = 0; k < 4; ++k) { s.th[k] = 0.f; s.cu[k] = 0.f; }
  } else if (sum > 0.f) {
    float kk = hc / sum;
#pragma unroll
    for (int q = 0; q < 4; ++q) s.th[q] *= kk;
  }
  stack_compact(s, P.misc[0]);
  stack_store<MODE>(F.sh2, F.scu2, F.pig2, c, s);
}

// strata.wgsl:276-286
template <int MODE>
__global__ void __launch_bounds__(256) k_copy_back(Film F) {
  TILE_PROLOGUE
  using Pig = typename Prec<MODE>::Pig;
  F.sh[c] = F.sh2[c];
  F.scu[c] = F.scu2[c];
#pragma unroll
  for (int k = 0; k < 4; ++k) copy_pig16<Pig>(pig_at<MODE>(F.pig, c, k), pig_at<MODE>(F.pig2, c, k));
}

// strata.wgsl:288-323, Jacobi in two passes: select reads only the sums of
// the current strata; apply writes only cells that had no strata, and its
// sources always have strata, so no pass reads what it writes.
__global__ void __launch_bounds__(256) k_fill_select(Film F) {
  TILE_PROLOGUE
  int32_t src = -1;
  float hc = F.hh[c];
  if (hc > 0.f) {
    float4 th = F.sh[c];
    if (!(th.x + th.y + th.z + th.w > 0.f)) {
      uint32_t cand[4];
      int nc = 0;
      if (i > 0) cand[nc++] = c - 1;
      if (j > 0) cand[nc++] = c - F.w;
      if (i + 1 < (int)F.w) cand[nc++] = c + 1;
      if (j + 1 < (int)F.h) cand[nc++] = c + F.w;
      float best = 0.f;
      for (int q = 0; q < nc; ++q) {
        float4 tn = F.sh[cand[q]];
        float ts = tn.x + tn.y + tn.z + tn.w;
        if (ts > best) { best = ts; src = (int32_t)cand[q]; }
      }
    }
  }
  F.fill_src[c] = src;
}
template <int MODE>
__global__ void __launch_bounds__(256) k_fill_apply(Film F) {
  TILE_PROLOGUE
  int32_t src = F.fill_src[c];
  if (src < 0) return;
  backfill<MODE>(F, c, (uint32_t)src, F.hh[c]);
}

// shade.wgsl:28-84 (colour and roughness; full grid)
template <int MODE>
__global__ void __launch_bounds__(256) k_shade(Film F) {
  __shared__ float tab[12 * 40];
  __shared__ float cm[48];
  int tid = threadIdx.y * 16 + threadIdx.x;
  for (int q = tid; q < 480; q += 256) tab[q] = F.pigtab[q];
  if (tid < 48) cm[tid] = F.cmf[tid];
  __syncthreads();
  const int i = (int)(blockIdx.x * 16 + threadIdx.x), j = (int)(blockIdx.y * 16 + threadIdx.y);
  if (i >= (int)F.w || j >= (int)F.h) return;
  const uint32_t c = idx(F, i, j);
  const cf_params& P = F.P->p;
  using Pig = typename Prec<MODE>::Pig;
  float r[16];
  const uint16_t* rf = F.refl + (size_t)c * 16;
  {
    const uint4* p = reinterpret_cast<const uint4*>(rf);
    uint4 a = p[0], b = p[1];
    uint32_t wv[8] = {a.x, a.y, a.z, a.w, b.x, b.y, b.z, b.w};
#pragma unroll
    for (int k = 0; k < 8; ++k) {
      r[2 * k] = h16_to_f(wv[k] & 0xffffu);
      r[2 * k + 1] = h16_to_f(wv[k] >> 16);
    }
  }
  float hv = F.hh[c];
  float wet = 0.f, cure_top = 0.f;
  float4 th4 = F.sh[c], cu4 = F.scu[c];
  float th[4] = {th4.x, th4.y, th4.z, th4.w}, cu[4] = {cu4.x, cu4.y, cu4.z, cu4.w};
  if (hv > 0.f) {
    for (int k = 0; k < 4; ++k) {
      float t = th[k];
      if (t <= 0.f) continue;
      float pg[16];
      load_pig16<Pig>(pig_at<MODE>(F.pig, c, k), pg);
      float w[12], sc;
      layer_weights(pg, tab, w, sc);
#pragma unroll 4
      for (int b = 0; b < 16; ++b) {
        float kk, ss, rr, tt;
        layer_ks_band(pg, w, sc, tab, b, kk, ss);
        km_layer(kk, ss, t, rr, tt);
        r[b] = composite(rr, tt, r[b]);
      }
      wet = 1.0f - cu[k];
      cure_top = cu[k];
    }
  }
  const float k1 = 0.04f;
  float k2 = 0.4f * (1.0f - wet) + 0.6f * wet;
  float X = 0.f, Y = 0.f, Z = 0.f;
#pragma unroll
  for (int b = 0; b < 16; ++b) {
    float rb = (1.0f - k1) * (1.0f - k2) * r[b] / fmaxf(1.0f - k2 * r[b], 1e-3f);
    X += rb * cm[3 * b];
    Y += rb * cm[3 * b + 1];
    Z += rb * cm[3 * b + 2];
  }
  float rgb[3] = {3.2406f * X - 1.5372f * Y - 0.4986f * Z, -0.9689f * X + 1.8758f * Y + 0.0415f * Z,
                  0.0557f * X - 0.2040f * Y + 1.0570f * Z};
#pragma unroll
  for (int q = 0; q < 3; ++q) rgb[q] = fmaxf(rgb[q], 0.f);
  auto smooth = [](float e0, float e1, float x) {
    float t = fminf(fmaxf((x - e0) / (e1 - e0), 0.f), 1.f);
    return t * t * (3.0f - 2.0f * t);
  };
  float mv = F.m[c];
  float painted = smooth(60e-6f, 150e-6f, mv);
  cure_top = fmaxf(cure_top, painted * (1.0f - smooth(0.f, 50e-6f, hv)));
  float sq = sqrtf(cure_top);
  float rough = 0.06f * (1.0f - sq) + 0.35f * sq;
  if (hv <= 0.f) rough = 0.85f * (1.0f - painted) + 0.35f * painted;
  if (P.flags[0] == 1u && hv > 0.f) {  // shade.wgsl:65-82 invariant view
    float ssum = th[0] + th[1] + th[2] + th[3];
    bool bad = false;
    uint32_t cnt = 0;
    for (int k = 0; k < 4; ++k) {
      if (th[k] > 0.f) cnt = k + 1;
      if (th[k] <= 0.f) continue;
      float pg[16];
      load_pig16<Pig>(pig_at<MODE>(F.pig, c, k), pg);
      float cs = 0.f;
      for (int q = 0; q < 13; ++q) cs += pg[q];
      if (!(cs > 0.f)) bad = true;
    }
    if (ssum <= 0.f) { rgb[0] = 0.f; rgb[1] = 0.f; rgb[2] = 1.f; }
    else if (bad) { rgb[0] = 1.f; rgb[1] = 0.f; rgb[2] = 0.f; }
    else if (fabsf(ssum - hv) > 0.01f * hv) { rgb[0] = 0.f; rgb[1] = 1.f; rgb[2] = 0.f; }
    else { float v = 0.3f + 0.15f * (float)cnt; rgb[0] = v; rgb[1] = v; rgb[2] = v; }
  }
  F.color[c] = make_ushort4(__half_as_ushort(__float2half_rn(rgb[0])), __half_as_ushort(__float2half_rn(rgb[1])),
                            __half_as_ushort(__float2half_rn(rgb[2])), __half_as_ushort(__float2half_rn(rough)));
}

// FP64 mass / NaN census (compute_stats, src/main.rs:1679-1773)
__global__ void __launch_bounds__(256) k_mass(Film F) {
  size_t n = (size_t)F.w * F.h;
  double sh = 0.0, sm = 0.0;
  unsigned long long wet = 0, nan = 0;
  for (size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x; c < n; c += (size_t)gridDim.x * blockDim.x) {
    float hv = F.hh[c];
    if (!isfinite(hv)) { nan++; continue; }
    sh += (double)hv;
    sm += (double)F.m[c];
    if (hv > 0.f) wet++;
  }
  for (int o = 16; o > 0; o >>= 1) {
    sh += __shfl_xor_sync(0xffffffffu, sh, o);
    sm += __shfl_xor_sync(0xffffffffu, sm, o);
    wet += __shfl_xor_sync(0xffffffffu, wet, o);
    nan += __shfl_xor_sync(0xffffffffu, nan, o);
  }
  if ((threadIdx.x & 31) == 0) {
    atomicAdd(&F.stats->wet_sum, sh);
    atomicAdd(&F.stats->relief_sum, sm);
    atomicAdd(&F.stats->wet_cells, wet);
    atomicAdd(&F.stats->nan_cells, nan);
  }
}

__global__ void k_stats_reset(Film F) {
  F.stats->h_max_bits = 0u;
  F.stats->mu_min_bits = __float_as_uint(1e9f);
  F.stats->active_tiles = 0u;
}
__global__ void k_mass_reset(Film F) {
  F.stats->wet_sum = 0.0;
  F.stats->relief_sum = 0.0;
  F.stats->wet_cells = 0ull;
  F.stats->nan_cells = 0ull;
}

// Device-side adaptive dt (choose_substeps formulas, src/film/mod.rs:919-933,
// one substep per frame) and the dt-dependent fields of update_params
// (src/film/mod.rs:869-917).  Round-to-nearest intrinsics keep the f32
// arithmetic identical to the host's (no contraction).
__global__ void k_adaptive_params(DevParams* Dp, DevStats* S) {
  DevParams D = *Dp;
  cf_params& P = D.p;
  float h_stat = __uint_as_float(S->h_max_bits);
  float mu_raw = __uint_as_float(S->mu_min_bits);
  float mu_stat = mu_raw > 1e8f ? 1.0f : mu_raw;
  float dx = P.dx;
  // adaptive dt
  float h_max = fmaxf(h_stat, 1e-5f);
  float mu = fmaxf(mu_stat, 1e-3f);
  float speed = fminf(__fdiv_rn(__fmul_rn(__fmul_rn(__fmul_rn(D.s_rho, D.gxy), h_max), h_max), mu), D.s_vcap);
  float dt = D.dt_max;
  if (speed > 1e-6f) dt = fminf(dt, __fdiv_rn(__fmul_rn(0.5f, dx), speed));
  float mob = __fdiv_rn(__fmul_rn(__fmul_rn(h_max, h_max), h_max), __fmul_rn(3.0f, mu));
  float hyd = __fmul_rn(__fmul_rn(D.s_rho, D.s_gz), fminf(mob, D.s_mcap_hydro));
  if (hyd > 0.f) dt = fminf(dt, __fdiv_rn(__fmul_rn(__fmul_rn(0.2f, dx), dx), hyd));
  float dx2 = __fmul_rn(dx, dx), dx4 = __fmul_rn(dx2, dx2);
  float cap = __fmul_rn(__fmul_rn(32.0f, D.s_sigma), fminf(mob, D.s_mcap));
  if (cap > 0.f) dt = fminf(dt, __fdiv_rn(dx4, cap));
  // update_params(frame_dt = dt, substeps = 1)
  float frame_dt = dt;
  float m_cap_exp = __fdiv_rn(__fmul_rn(__fmul_rn(__fmul_rn(__fmul_rn(0.5f, dx), dx), dx), dx),
                              __fmul_rn(__fmul_rn(32.0f, D.s_sigma), dt));
  float m_cap = fmaxf(fminf(D.s_mcap, m_cap_exp), 1e-14f);
  float gz01 = fmaxf(D.s_gz, 0.1f);
  float m_exp = __fdiv_rn(__fmul_rn(__fmul_rn(0.1f, dx), dx), __fmul_rn(__fmul_rn(dt, D.s_rho), gz01));
  P.dt = dt;
  P.frame_dt = frame_dt;
  P.phys[3] = D.s_capillary ? m_cap : 0.0f;
  P.misc[3] = fminf(m_exp, D.s_mcap_hydro);
  float cap_explicit = fminf(m_exp, D.s_mcap_hydro);
  float h_big = fmaxf(h_stat, 1e-4f);
  float mu3 = __fmul_rn(3.0f, fmaxf(mu_stat, 1e-3f));
  float m_phys_cap = __fdiv_rn(__fmul_rn(__fmul_rn(h_big, h_big), h_big), mu3);
  float m_phys = __fsub_rn(m_phys_cap, cap_explicit);
  float kappa = __fdiv_rn(__fmul_rn(__fmul_rn(frame_dt, D.s_rho), gz01), dx2);
  uint32_t n_i = 0;
  if (m_phys > 0.f) {
    float v = fmaxf(ceilf(__fdiv_rn(__fmul_rn(kappa, m_phys), 40.0f)), 1.0f);
    n_i = min((uint32_t)v, 4u);
  }
  float dt_i = __fdiv_rn(frame_dt, (float)max(n_i, 1u));
  P.front[2] = __fdiv_rn(__fmul_rn(__fmul_rn(40.0f, dx), dx), __fmul_rn(__fmul_rn(dt_i, D.s_rho), gz01));
  P.front[3] = dt_i;
  float m_cap_impl = __fdiv_rn(__fmul_rn(__fdiv_rn(D.s_cap_cond, 28.0f), dx4), __fmul_rn(dt_i, D.s_sigma));
  float m_c = D.s_cap_implicit ? fminf(m_phys_cap, m_cap_impl) : 0.0f;
  P.front3[0] = __fdiv_rn(__fmul_rn(__fmul_rn(dt_i, D.s_sigma), m_c), dx4);
  P.front3[1] = __fdiv_rn(__fmul_rn(m_c, D.s_sigma), __fmul_rn(dx2, dx));
  P.front3[2] = m_c;
  D.implicit_steps = D.s_implicit ? n_i : 0u;
  D.frames += 1;
  *Dp = D;
  S->last_dt = dt;
}

// ---- state I/O conversions ----
template <class T>
__global__ void k_pig_import(Film F, const void* src, int fmt, size_t nslots) {
  size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (q >= nslots) return;
  float v;
  if (fmt == CF_PIG_F32) v = ((const float*)src)[q];
  else if (fmt == CF_PIG_F16) v = __half2float(((const __half*)src)[q]);
  else v = __bfloat162float(((const __nv_bfloat16*)src)[q]);
  ((T*)F.pig)[q] = from_f<T>(v);
}
template <class T>
__global__ void k_pig_export(Film F, void* dst, int fmt, size_t nslots) {
  size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (q >= nslots) return;
  float v = to_f(((const T*)F.pig)[q]);
  if (fmt == CF_PIG_F32) ((float*)dst)[q] = v;
  else if (fmt == CF_PIG_F16) ((__half*)dst)[q] = __float2half_rn(v);
  else ((__nv_bfloat16*)dst)[q] = __float2bfloat16_rn(v);
}
template <class Rh>
__global__ void k_rheo_import(Film F, const float2* src, float n_global, size_t n) {
  size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (c >= n) return;
  float2 v = src[c];
  ((Rh*)F.mu)[c] = from_f<Rh>(v.x);
  ((Rh*)F.tau)[c] = from_f<Rh>(v.y);
  ((Rh*)F.nn)[c] = from_f<Rh>(n_global);
}
template <class Rh>
__global__ void k_rheo_export(Film F, float2* dst, size_t n) {
  size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (c >= n) return;
  dst[c] = make_float2(to_f(((const Rh*)F.mu)[c]), to_f(((const Rh*)F.tau)[c]));
}
__global__ void k_fill_u32(uint32_t* p, uint32_t v, size_t n) {
  size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (q < n) p[q] = v;
}

// ---------------------------------------------------------------- host --

static inline dim3 tiles_grid(const Film& F) { return dim3(F.tw, F.th); }

template <int MODE>
static void frame_t(const Film& F, uint32_t substeps, int all_active, cudaStream_t st) {
  dim3 g = tiles_grid(F), b(16, 16);
  uint32_t nt = F.tw * F.th;
  k_stats_reset<<<1, 1, 0, st>>>(F);
  k_mark_tiles<<<g, b, 0, st>>>(F);
  k_compact_tiles<<<(nt + 255) / 256, 256, 0, st>>>(F, all_active);
  k_cure<MODE><<<g, b, 0, st>>>(F);
  k_clear_acc<<<g, b, 0, st>>>(F);
  for (uint32_t s = 0; s < substeps; ++s) {
    k_laplacian<<<g, b, 0, st>>>(F);
    k_plug<MODE><<<g, b, 0, st>>>(F);
    k_fluxes<MODE><<<g, b, 0, st>>>(F);
    k_limiter<<<g, b, 0, st>>>(F);
    k_apply<MODE><<<g, b, 0, st>>>(F);
    cudaMemcpyAsync(F.delta_old, F.delta, sizeof(uint32_t) * (size_t)F.w * F.h, cudaMemcpyDeviceToDevice, st);
    k_nose<<<g, b, 0, st>>>(F);
  }
  k_laplacian<<<g, b, 0, st>>>(F);
  k_strata_split<MODE><<<g, b, 0, st>>>(F);
  k_reduce_tiles<MODE><<<dim3((F.w + 63) / 64, (F.h + 63) / 64), b, 0, st>>>(F);
  k_strata_limit<<<g, b, 0, st>>>(F);
  k_strata_update<MODE><<<g, b, 0, st>>>(F);
  k_copy_back<MODE><<<g, b, 0, st>>>(F);
  for (int r = 0; r < 6; ++r) {
    k_fill_select<<<g, b, 0, st>>>(F);
    k_fill_apply<MODE><<<g, b, 0, st>>>(F);
  }
  k_shade<MODE><<<g, b, 0, st>>>(F);
}

void launch_frame(const Film& F, int mode, uint32_t substeps, int all_active, cudaStream_t st) {
  if (mode == CF_PREC_REFERENCE) frame_t<CF_PREC_REFERENCE>(F, substeps, all_active, st);
  else if (mode == CF_PREC_FP32) frame_t<CF_PREC_FP32>(F, substeps, all_active, st);
  else frame_t<CF_PREC_BF16>(F, substeps, all_active, st);
}

void launch_adaptive_params(DevParams* Dp, DevStats* S, cudaStream_t st) { k_adaptive_params<<<1, 1, 0, st>>>(Dp, S); }

template <int MODE>
static void cure_only_t(const Film& F, cudaStream_t st) {
  k_cure<MODE><<<tiles_grid(F), dim3(16, 16), 0, st>>>(F);
}
void launch_cure(const Film& F, int mode, cudaStream_t st) {
  if (mode == CF_PREC_REFERENCE) cure_only_t<CF_PREC_REFERENCE>(F, st);
  else if (mode == CF_PREC_FP32) cure_only_t<CF_PREC_FP32>(F, st);
  else cure_only_t<CF_PREC_BF16>(F, st);
}

template <int MODE>
static void reduce_only_t(const Film& F, cudaStream_t st) {
  k_stats_reset<<<1, 1, 0, st>>>(F);
  k_reduce_tiles<MODE><<<dim3((F.w + 63) / 64, (F.h + 63) / 64), dim3(16, 16), 0, st>>>(F);
}
void launch_reduce(const Film& F, int mode, cudaStream_t st) {
  if (mode == CF_PREC_REFERENCE) reduce_only_t<CF_PREC_REFERENCE>(F, st);
  else if (mode == CF_PREC_FP32) reduce_only_t<CF_PREC_FP32>(F, st);
  else reduce_only_t<CF_PREC_BF16>(F, st);
}

void launch_mass(const Film& F, int sms, cudaStream_t st) {
  k_mass_reset<<<1, 1, 0, st>>>(F);
  k_mass<<<sms * 4, 256, 0, st>>>(F);
}

void launch_fill_u32(uint32_t* p, uint32_t v, size_t n, cudaStream_t st) {
  if (n) k_fill_u32<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(p, v, n);
}

void launch_pig_import(const Film& F, int mode, const void* src, int fmt, size_t nslots, cudaStream_t st) {
  unsigned g = (unsigned)((nslots + 255) / 256);
  if (mode == CF_PREC_REFERENCE) k_pig_import<__half><<<g, 256, 0, st>>>(F, src, fmt, nslots);
  else if (mode == CF_PREC_FP32) k_pig_import<float><<<g, 256, 0, st>>>(F, src, fmt, nslots);
  else k_pig_import<__nv_bfloat16><<<g, 256, 0, st>>>(F, src, fmt, nslots);
}
void launch_pig_export(const Film& F, int mode, void* dst, int fmt, size_t nslots, cudaStream_t st) {
  unsigned g = (unsigned)((nslots + 255) / 256);
  if (mode == CF_PREC_REFERENCE) k_pig_export<__half><<<g, 256, 0, st>>>(F, dst, fmt, nslots);
  else if (mode == CF_PREC_FP32) k_pig_export<float><<<g, 256, 0, st>>>(F, dst, fmt, nslots);
  else k_pig_export<__nv_bfloat16><<<g, 256, 0, st>>>(F, dst, fmt, nslots);
}
void launch_rheo_import(const Film& F, int mode, const float2* src, float n_global, size_t n, cudaStream_t st) {
  unsigned g = (unsigned)((n + 255) / 256);
  if (mode == CF_PREC_BF16) k_rheo_import<__nv_bfloat16><<<g, 256, 0, st>>>(F, src, n_global, n);
  else k_rheo_import<float><<<g, 256, 0, st>>>(F, src, n_global, n);
}
void launch_rheo_export(const Film& F, int mode, float2* dst, size_t n, cudaStream_t st) {
  unsigned g = (unsigned)((n + 255) / 256);
  if (mode == CF_PREC_BF16) k_rheo_export<__nv_bfloat16><<<g, 256, 0, st>>>(F, dst, n);
  else k_rheo_export<float><<<g, 256, 0, st>>>(F, dst, n);
}

// Single dispatches for parity tests (kernel ids follow the WGSL names).
int launch_one(const Film& F, int mode, const char* name, int all_active, cudaStream_t st) {
  dim3 g = tiles_grid(F), b(16, 16);
  uint32_t nt = F.tw * F.th;
  std::string_view n(name);
#define CFK_T(K) \
  (mode == CF_PREC_REFERENCE ? (void)K<CF_PREC_REFERENCE><<<g, b, 0, st>>>(F) : mode == CF_PREC_FP32 ? (void)K<CF_PREC_FP32><<<g, b, 0, st>>>(F) : (void)K<CF_PREC_BF16><<<g, b, 0, st>>>(F))
  if (n == "mark_tiles") k_mark_tiles<<<g, b, 0, st>>>(F);
  else if (n == "compact_tiles") { k_stats_reset<<<1, 1, 0, st>>>(F); k_compact_tiles<<<(nt + 255) / 256, 256, 0, st>>>(F, all_active); }
  else if (n == "cure_step") CFK_T(k_cure);
  else if (n == "clear_acc") k_clear_acc<<<g, b, 0, st>>>(F);
  else if (n == "laplacian") k_laplacian<<<g, b, 0, st>>>(F);
  else if (n == "plug") CFK_T(k_plug);
  else if (n == "fluxes") CFK_T(k_fluxes);
  else if (n == "limiter") k_limiter<<<g, b, 0, st>>>(F);
  else if (n == "apply") CFK_T(k_apply);
  else if (n == "nose") {
    cudaMemcpyAsync(F.delta_old, F.delta, sizeof(uint32_t) * (size_t)F.w * F.h, cudaMemcpyDeviceToDevice, st);
    k_nose<<<g, b, 0, st>>>(F);
  }
  else if (n == "strata_split") CFK_T(k_strata_split);
  else if (n == "reduce_tiles") launch_reduce(F, mode, st);
  else if (n == "strata_limit") k_strata_limit<<<g, b, 0, st>>>(F);
  else if (n == "strata_update") CFK_T(k_strata_update);
  else if (n == "strata_copy_back") CFK_T(k_copy_back);
  else if (n == "strata_fill") { k_fill_select<<<g, b, 0, st>>>(F); CFK_T(k_fill_apply); }
  else if (n == "shade_full") CFK_T(k_shade);
  else return 0;
#undef CFK_T
  return 1;
}

}  // namespace cfk
