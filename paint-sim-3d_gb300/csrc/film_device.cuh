// film_device.cuh — per-cell device functions of the thin-film step (sm_103a).
//
// Each function restates one WGSL helper of the reference; the comment names
// the shader file and line range it follows.  Arithmetic is FP32 as in the
// reference; CUDA's own expf/logf/powf/sqrtf/atanf are used throughout.
//
// Planes are addressed through `Film`, a POD of device pointers (one per
// plane, reference layout) that every kernel receives by value.
#pragma once

#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <stdint.h>

#include "../../include/canvaz_film.h"

namespace cfk {

constexpr float W_AXIS = 0.6666667f;      // film.wgsl:105
constexpr float W_DIAG_FLUX = 0.23570226f;  // film.wgsl:106
constexpr float W_DIAG_LAP = 0.16666667f;   // film.wgsl:107
constexpr float MOVE_EPS = 1e-6f;           // film.wgsl:108
constexpr float FRAME_EPS = 2e-6f;          // film.wgsl:109
constexpr float DRAINED_FILM = 1e-9f;       // film.wgsl:1
constexpr uint32_t MOVED = 64u;
constexpr uint32_t ACTIVE = 32u;

// Device-resident parameters: the packed Params uniform plus the settings the
// adaptive step re-derives dt-dependent fields from.
struct DevParams {
  cf_params p;
  float gxy;            // |g.xy| (m/s^2)
  float s_rho, s_sigma, s_vcap, s_mcap, s_mcap_hydro, s_cap_cond, s_gz;
  int32_t s_capillary;  // capillary && !no_cap
  int32_t s_cap_implicit;
  int32_t s_implicit;
  float dt_max;         // adaptive step upper bound
  uint32_t implicit_steps;
  uint32_t implicit_iters;  // FilmSettings::implicit_iters
  uint32_t frames;
  // per-film constants of the front terms (settings only, never dt):
  float hold1;          // hold_level(1) (film.wgsl:153-156)
  float cox_theta;      // atan(tan theta) (film.wgsl:236-244)
  float cox_span;       // max(front.x - hold_level(1), 1e-6)
  float cox_adv;        // min(theta + front2.x, 3.1)
  float gc_max;         // sigma / (1 mm)^2, the capillary gradient cap of yield_cap (film.wgsl:44-49)
};

// Scalars of a film's implicit CG solve (film.wgsl cg_s[0], cg_s[1]) and the
// count of blocks that have written their tile partial in the current launch.
struct CgState {
  float rz, pq, alpha, beta;  // cg_s[0]
  float s1x, dv, tv, s0x;     // cg_s[1]: rz of the init, sum of h changes, sum of h, last rz
  uint32_t blocks_done;
  uint32_t pad[7];
};

// Global reductions written by the stats kernels.
struct DevStats {
  uint32_t h_max_bits;   // max h over cells with h > 4 h_min (float bits, h >= 0)
  uint32_t mu_min_bits;  // min mu over the same cells (float bits, mu > 0)
  uint32_t active_tiles;
  uint32_t fill_count;   // entries of Film::fill_list (wet active cells the strata pass left without strata)
  double wet_sum;        // sum(h)
  double relief_sum;     // sum(m)
  unsigned long long wet_cells;
  unsigned long long nan_cells;
  float last_dt;
  uint32_t full_count;   // entries of Film::full_list (cells of the strata full path)
  uint32_t tma_timeouts; // tiles whose staged loads did not arrive within the wait limit (0 unless faulty)
};

template <int MODE> struct Prec;
template <> struct Prec<CF_PREC_REFERENCE> { using Pig = __half; using Rh = float; };
template <> struct Prec<CF_PREC_FP32> { using Pig = float; using Rh = float; };
template <> struct Prec<CF_PREC_BF16> { using Pig = __nv_bfloat16; using Rh = __nv_bfloat16; };

__device__ __forceinline__ float to_f(float v) { return v; }
__device__ __forceinline__ float to_f(__half v) { return __half2float(v); }
__device__ __forceinline__ float to_f(__nv_bfloat16 v) { return __bfloat162float(v); }
template <class T> __device__ __forceinline__ T from_f(float v);
template <> __device__ __forceinline__ float from_f<float>(float v) { return v; }
template <> __device__ __forceinline__ __half from_f<__half>(float v) { return __float2half_rn(v); }
template <> __device__ __forceinline__ __nv_bfloat16 from_f<__nv_bfloat16>(float v) { return __float2bfloat16_rn(v); }

// All device planes of one film.  Strata thicknesses and cure fractions come
// in two generations (cur / nxt) that swap every frame, so the strata pass
// never copies them back.  The pigments have one plane: only the cells of the
// strata full path change them, and those write their new slots to the side
// plane pig2 first, copied back after the pass (other cells read their
// neighbours' pigments during it).  Pigment slots are stored chunk-major:
// 16-byte chunk q of stratum k of cell c lives at chunk index (k * QN + q) * n
// + c (QN = chunks per stratum), so a warp reads 512 contiguous bytes per
// load.  acc_s is face-major: face f of cell c at f * n + c.
struct Film {
  uint32_t w, h, tw, th;  // grid and 16x16 tile counts
  uint32_t n;             // cells
  const DevParams* P;
  DevStats* stats;
  float* hh;       // h
  float* m;
  void* mu;        // rheo.x  (Rh)
  void* tau;       // rheo.y  (Rh)
  void* nn;        // power-law index (Rh)
  uint32_t* delta;
  uint32_t* delta_old;
  uint32_t* lay;
  float2* pres;
  float2* fnorm;
  float4* flux;
  float4* acc;
  float4* acc_s;   // 4 faces x n, face-major
  float4* alpha_s;
  float* alpha;
  float* tmp;
  float* h_frame;
  float* h_next;   // heights after apply, until the nose commits them to h
  float4* sh;      // strata_h, current generation
  float4* scu;     // strata_cure
  uint4* pig;      // pigment chunks
  float4* sh2;     // next generation
  float4* scu2;
  uint4* pig2;     // new pigments of the strata full path's cells (side plane)
  float4* agg;     // composition aggregates for the next cure (see composition_parts)
  uint16_t* refl;  // 16 half per cell
  ushort4* color;  // rgba16f
  ushort4* detail; // rgba16f: the renderer's detail texel (shade.wgsl:61-64)
  uint32_t* tile_flags;
  uint32_t* tile_moved;
  int32_t* fill_src;
  uint32_t* fflags;  // bit f: strata_split wrote a nonzero acc_s face f this frame
  uint8_t* shade_state;  // SHADE_*: what of a cell's colour is still current (below)
  float4* spec;          // composite spectrum of a wet cell (SHADE_WET): band 4q+e at chunk q*n + c, component e
  uint32_t* full_list;  // cells of the strata full path (DevStats::full_count)
  uint32_t* fill_list;  // strata fill candidates (DevStats::fill_count)
  // implicit CG planes (null when the film's settings turn the implicit
  // hydrostatic step off): face mobilities, diagonal, solution, residual,
  // direction (cg_p as the last step left it; cg_pa / cg_pb alternate during
  // a solve), A p (then the new h), weighted Laplacians, tile partials
  float4* cg_m;
  float *cg_d, *cg_x, *cg_r, *cg_p, *cg_pa, *cg_pb, *cg_q, *cg_t, *cg_t2, *cg_part, *cg_part2;
  CgState* cg;
  uint32_t* cg_cnt;  // per group of 32 tiles: blocks that have written their partial
  uint32_t persist_blocks;  // grid of the list kernels: a few blocks per SM
  uint32_t all_active;      // keep every tile active (settings.all_active)
  const float* pigtab;  // 12 x 40
  const float* cmf;     // 16 x 3
  // TMA descriptors of the planes the tile kernels stage (FLOW_MAPS of them,
  // in that order), 64-byte aligned in device memory; null where the grid's
  // row pitch is not a multiple of 16 bytes (the tiles then load them
  // themselves)
  const CUtensorMap* tmap;
};
// Film::shade_state of a cell.  The KM shade of a wet cell composites each
// stratum over the substrate (the composite spectrum depends on the strata's
// thicknesses and pigments, the substrate reflectance and the pigment
// table), then applies the surface correction, whose wetness follows the top
// stratum's cure (which ages every frame).  SHADE_WET keeps the composite
// spectrum in Film::spec, valid for the cell's current thicknesses and
// pigments: the strata pass reuses it while the thicknesses it computes are
// bit for bit the current ones, and redoes only the surface correction.
// The strata pass's shades (fast path and full path) set it with the spectrum
// they computed; every other writer of a cell's strata, pigments or substrate
// resets the state to SHADE_NONE.  SHADE_DRY: the colour holds the dry cell's colour,
// which depends only on the substrate, the relief and the CMF table.
// SHADE_DRY2: the same, and the strata pass has written zero thicknesses and
// cure fractions for the cell into both strata generations (it was dry in an
// active tile two passes running), so a pass that finds it dry again has
// nothing to read or write for it.
constexpr uint8_t SHADE_NONE = 0, SHADE_DRY = 1, SHADE_WET = 2, SHADE_DRY2 = 3;
// Planes staged by tensor loads (the flow, laplacian, limiter + apply and
// nose tiles), in Film::tmap order.
enum FlowMap { MAP_H = 0, MAP_M, MAP_DELTA, MAP_MU, MAP_TAU, MAP_N, MAP_DELTA_OLD, MAP_FLUX, MAP_H_NEXT, FLOW_MAPS };

__device__ __forceinline__ uint32_t idx(const Film& F, int i, int j) { return (uint32_t)j * F.w + (uint32_t)i; }
// Entry e of a packed tile table (film index, tile index).  A null table is
// the identity over film 0, the view of a film stepped alone: its blocks
// take their tile from the block index and skip the table's load.
__device__ __forceinline__ uint2 tile_entry(const uint2* tiles, uint32_t e) {
  return tiles != nullptr ? tiles[e] : make_uint2(0u, e);
}
__device__ __forceinline__ bool in_grid(const Film& F, int i, int j) {
  return i >= 0 && j >= 0 && i < (int)F.w && j < (int)F.h;
}
// Appends v to a device list; one atomic per warp (the threads of the warp
// that append at this point).
// Folds a tile's h max and mu min (float bits of positive values) into the
// film's: the film's value is read first and the atomic issued only where the
// tile's would change it.  Within a pass the max only grows and the min only
// shrinks, so a stale read costs at most an atomic that changes nothing.
__device__ __forceinline__ void fold_cfl(DevStats* st, float hm, float mm) {
  const uint32_t hb = __float_as_uint(hm), mb = __float_as_uint(mm);
  if (hb > *reinterpret_cast<volatile uint32_t*>(&st->h_max_bits)) atomicMax(&st->h_max_bits, hb);
  if (mb < *reinterpret_cast<volatile uint32_t*>(&st->mu_min_bits)) atomicMin(&st->mu_min_bits, mb);
}
__device__ __forceinline__ void list_append(uint32_t* list, uint32_t* count, uint32_t v) {
  const unsigned m = __activemask();
  const int lane = (int)((threadIdx.y * blockDim.x + threadIdx.x) & 31u);
  const int leader = __ffs(m) - 1;
  uint32_t base = 0;
  if (lane == leader) base = atomicAdd(count, (uint32_t)__popc(m));
  base = __shfl_sync(m, base, leader);
  list[base + __popc(m & ((1u << lane) - 1u))] = v;
}

__device__ __forceinline__ bool cell_active(const Film& F, int i, int j) {  // film.wgsl:128-131
  return (F.tile_flags[(uint32_t)(i >> 4) + (uint32_t)(j >> 4) * F.tw] & ACTIVE) != 0u;
}
__device__ __forceinline__ int refl_i(const Film& F, int i) {  // common.wgsl:152-158
  int w = (int)F.w, r = i;
  if (r < 0) r = -r - 1;
  if (r >= w) r = 2 * w - r - 1;
  return min(max(r, 0), w - 1);
}
__device__ __forceinline__ int refl_j(const Film& F, int j) {
  int hh = (int)F.h, r = j;
  if (r < 0) r = -r - 1;
  if (r >= hh) r = 2 * hh - r - 1;
  return min(max(r, 0), hh - 1);
}
__device__ __forceinline__ float4 acc_face(const Film& F, uint32_t c, int f) { return F.acc_s[(size_t)f * F.n + c]; }
// Face f of cell c as this frame's strata_split left it.  strata_split writes
// only the faces it evaluates and sets bit f of the cell's face flags where
// the split is nonzero, so a face whose bit is clear carries no strata flux
// (its acc_s entry may be stale and is not read).
__device__ __forceinline__ float4 acc_face_live(const Film& F, uint32_t c, int f, uint32_t flags) {
  return ((flags >> f) & 1u) ? acc_face(F, c, f) : make_float4(0.f, 0.f, 0.f, 0.f);
}

template <int MODE>
__device__ __forceinline__ float rmu(const Film& F, uint32_t c) {
  return to_f(((const typename Prec<MODE>::Rh*)F.mu)[c]);
}
template <int MODE>
__device__ __forceinline__ float rtau(const Film& F, uint32_t c) {
  return to_f(((const typename Prec<MODE>::Rh*)F.tau)[c]);
}
template <int MODE>
__device__ __forceinline__ float rn(const Film& F, uint32_t c) {
  return to_f(((const typename Prec<MODE>::Rh*)F.nn)[c]);
}
template <int MODE>
__device__ __forceinline__ void set_rheo(const Film& F, uint32_t c, float mu, float tau, float n) {
  using Rh = typename Prec<MODE>::Rh;
  ((Rh*)F.mu)[c] = from_f<Rh>(mu);
  ((Rh*)F.tau)[c] = from_f<Rh>(tau);
  ((Rh*)F.nn)[c] = from_f<Rh>(n);
}

// IEEE half / bfloat16 bits <-> float without type punning.
__device__ __forceinline__ float h16_to_f(uint32_t bits) { return __half2float(__ushort_as_half((unsigned short)bits)); }
__device__ __forceinline__ uint32_t f_to_h16(float v) { return (uint32_t)__half_as_ushort(__float2half_rn(v)); }
__device__ __forceinline__ float b16_to_f(uint32_t bits) { return __uint_as_float(bits << 16); }
__device__ __forceinline__ uint32_t f_to_b16(float v) { return (uint32_t)__bfloat16_as_ushort(__float2bfloat16_rn(v)); }

// Pigment slot 14 carries a stratum's viscosity override as ln mu + 10 (0 =
// none: the pigments' own viscosities apply; cure.wgsl:3-48).  Its values lie
// in about 9.3..13.9, where bfloat16's 8 significant bits step by 0.0625 and
// would put mu off by up to 6 %.  BF16 storage therefore keeps mu itself in
// that slot (Pa s, 0 = none): 8 bits on mu hold it to 0.2 %.  Every other
// slot, and the value the kernels compute with, stay as the reference has
// them.
constexpr int SLOT_LNMU = 14;
__device__ __forceinline__ uint32_t b16_from_slot(float v, int slot) {
  if (slot == SLOT_LNMU) return v > 0.f ? f_to_b16(expf(v - 10.0f)) : 0u;
  return f_to_b16(v);
}
__device__ __forceinline__ float slot_from_b16(uint32_t bits, int slot) {
  if (slot == SLOT_LNMU) return bits != 0u ? logf(b16_to_f(bits)) + 10.0f : 0.f;
  return b16_to_f(bits);
}

// ---- pigment slots: 16 per stratum, 4 strata per cell, chunk-major ----
template <int MODE>
struct PigIO {
  using Pig = typename Prec<MODE>::Pig;
  static constexpr int QN = 16 * (int)sizeof(Pig) / 16;  // 16-byte chunks per stratum
  __device__ static __forceinline__ size_t at(const Film& F, uint32_t c, int k, int q) {
    return (size_t)(k * QN + q) * F.n + c;
  }
  // 16 slot values of stratum k of cell c from `base` (cur or nxt generation)
  __device__ static __forceinline__ void load(const Film& F, const uint4* base, uint32_t c, int k, float o[16]) {
#pragma unroll
    for (int q = 0; q < QN; ++q) {
      uint4 v = base[at(F, c, k, q)];
      uint32_t wv[4] = {v.x, v.y, v.z, v.w};
      if constexpr (MODE == CF_PREC_FP32) {
#pragma unroll
        for (int e = 0; e < 4; ++e) o[4 * q + e] = __uint_as_float(wv[e]);
      } else {
#pragma unroll
        for (int e = 0; e < 4; ++e) {
          if constexpr (MODE == CF_PREC_REFERENCE) {
            o[8 * q + 2 * e] = h16_to_f(wv[e] & 0xffffu);
            o[8 * q + 2 * e + 1] = h16_to_f(wv[e] >> 16);
          } else {
            o[8 * q + 2 * e] = slot_from_b16(wv[e] & 0xffffu, 8 * q + 2 * e);
            o[8 * q + 2 * e + 1] = slot_from_b16(wv[e] >> 16, 8 * q + 2 * e + 1);
          }
        }
      }
    }
  }
  __device__ static __forceinline__ void store(const Film& F, uint4* base, uint32_t c, int k, const float v[16]) {
#pragma unroll
    for (int q = 0; q < QN; ++q) {
      uint32_t wv[4];
      if constexpr (MODE == CF_PREC_FP32) {
#pragma unroll
        for (int e = 0; e < 4; ++e) wv[e] = __float_as_uint(v[4 * q + e]);
      } else {
#pragma unroll
        for (int e = 0; e < 4; ++e) {
          if constexpr (MODE == CF_PREC_REFERENCE) wv[e] = f_to_h16(v[8 * q + 2 * e]) | (f_to_h16(v[8 * q + 2 * e + 1]) << 16);
          else wv[e] = b16_from_slot(v[8 * q + 2 * e], 8 * q + 2 * e) |
                       (b16_from_slot(v[8 * q + 2 * e + 1], 8 * q + 2 * e + 1) << 16);
        }
      }
      base[at(F, c, k, q)] = make_uint4(wv[0], wv[1], wv[2], wv[3]);
    }
  }
  // the value of slot `slot` as the store above keeps it
  __device__ static __forceinline__ float round(float v, int slot) {
    if constexpr (MODE == CF_PREC_FP32) return v;
    else if constexpr (MODE == CF_PREC_REFERENCE) return h16_to_f(f_to_h16(v));
    else return slot_from_b16(b16_from_slot(v, slot), slot);
  }
  // bit-exact copy of stratum ks of cell cs (in src) to stratum kd of cell cd (in dst)
  __device__ static __forceinline__ void copy(const Film& F, uint4* dst, uint32_t cd, int kd, const uint4* src,
                                              uint32_t cs, int ks) {
#pragma unroll
    for (int q = 0; q < QN; ++q) dst[at(F, cd, kd, q)] = src[at(F, cs, ks, q)];
  }
  __device__ static __forceinline__ void zero(const Film& F, uint4* dst, uint32_t c, int k) {
#pragma unroll
    for (int q = 0; q < QN; ++q) dst[at(F, c, k, q)] = make_uint4(0u, 0u, 0u, 0u);
  }
};

__device__ __forceinline__ float half_at(const uint16_t* p, int k) {
  return __half2float(__ushort_as_half(p[k]));
}

// ---- film.wgsl helpers ----

// film.wgsl:570-585
__device__ __forceinline__ uint32_t pack_off(int dx, int dy) {
  uint32_t ux = (uint32_t)min(max(dx + 128, 0), 255);
  uint32_t uy = (uint32_t)min(max(dy + 128, 0), 255);
  return (ux << 8) | uy | 0x10000u;
}
__device__ __forceinline__ void unpack_off(uint32_t bits, int& ox, int& oy) {
  if ((bits & 0x10000u) == 0u) { ox = 64; oy = 64; return; }
  ox = (int)((bits >> 8) & 0xffu) - 128;
  oy = (int)(bits & 0xffu) - 128;
}
__device__ __forceinline__ float off_len(int ox, int oy) { return sqrtf((float)(ox * ox + oy * oy)); }
__device__ __forceinline__ float nose_dist(const Film& F, uint32_t c) {
  int ox, oy;
  unpack_off(F.delta[c], ox, oy);
  return off_len(ox, oy);
}
// film.wgsl:153-156
__device__ __forceinline__ float hold_level(const cf_params& P, float d) {
  return P.front[0] * (1.0f - expf(-(fmaxf(d, 1.0f) - 0.5f) * P.front[1]));
}
// common.wgsl:190-195
__device__ __forceinline__ float disjoining(const cf_params& P, float hv) {
  float x = fmaxf(1.0f - hv / P.cure[3], 0.0f);
  return P.ein[2] * x * x;
}
__device__ __forceinline__ float sgnf(float x) { return x > 0.f ? 1.f : (x < 0.f ? -1.f : 0.f); }

// film.wgsl:94-107 with the evaluation's power-law index n
__device__ __forceinline__ void hb_flux(float gmag, float hf, float mu, float ty, float n, float& q, float& y,
                                        float& up) {
  q = 0.f; y = 0.f; up = 0.f;
  if (gmag < 1e-9f || hf <= 0.f) return;
  float yy = fmaxf(hf - ty / gmag, 0.f);
  if (yy <= 0.f) return;
  float u;
  if (fabsf(n - 1.0f) < 1e-4f) u = 0.5f * gmag / mu * yy * yy;
  else u = n / (n + 1.0f) * powf(gmag / mu, 1.0f / n) * powf(yy, (n + 1.0f) / n);
  q = u * (hf - n * yy / (2.0f * n + 1.0f));
  y = yy;
  up = u;
}
// film.wgsl:109-126
__device__ __forceinline__ float band_flux(float up, float y, float za, float zb, float n) {
  float ta = 0.f, tb = 0.f;
  if (y > 0.f) {
    float ra = fmaxf(y - za, 0.f) / y;
    float rb = fmaxf(y - zb, 0.f) / y;
    if (fabsf(n - 1.0f) < 1e-4f) {
      ta = ra * ra * ra;
      tb = rb * rb * rb;
    } else {
      float e = (2.0f * n + 1.0f) / n;
      ta = powf(ra, e);
      tb = powf(rb, e);
    }
  }
  return up * ((zb - za) - n / (2.0f * n + 1.0f) * y * (ta - tb));
}

// film.wgsl:190-201
__device__ __forceinline__ float line_pressure(const Film& F, const cf_params& P, int i, int j) {
  if (i < 1 || j < 1 || i + 1 >= (int)F.w || j + 1 >= (int)F.h) return 0.f;
  float2 nl = F.fnorm[idx(F, i - 1, j)], nr = F.fnorm[idx(F, i + 1, j)];
  float2 nd = F.fnorm[idx(F, i, j - 1)], nu = F.fnorm[idx(F, i, j + 1)];
  if (nl.x * nl.x + nl.y * nl.y < 0.5f || nr.x * nr.x + nr.y * nr.y < 0.5f || nd.x * nd.x + nd.y * nd.y < 0.5f ||
      nu.x * nu.x + nu.y * nu.y < 0.5f)
    return 0.f;
  float curv = (nr.x - nl.x + nu.y - nd.y) * 0.5f * P.inv_dx;
  return P.phys[1] * curv * P.front2[2];
}

// film.wgsl:134-145
__device__ __forceinline__ uint32_t feeders(const Film& F, const cf_params& P, uint32_t c) {
  int i = (int)(c % F.w), j = (int)(c / F.w);
  float thr = 2.0f * F.hh[c] + P.ein[3];
  uint32_t n = 0;
  if (i > 0 && F.hh[idx(F, i - 1, j)] > thr) n++;
  if (i + 1 < (int)F.w && F.hh[idx(F, i + 1, j)] > thr) n++;
  if (j > 0 && F.hh[idx(F, i, j - 1)] > thr) n++;
  if (j + 1 < (int)F.h && F.hh[idx(F, i, j + 1)] > thr) n++;
  return n;
}
// film.wgsl:160-180, with the heights of the 5 x 5 neighbourhood read through
// hgt(x, y) (the plane, or a tile's box staged in shared memory)
template <class HF>
__device__ __forceinline__ float2 front_normal_at(const Film& F, const cf_params& P, int i, int j, HF hgt) {
  float dx = 0.f, dy = 0.f;
#pragma unroll
  for (int dj = -2; dj <= 2; ++dj)
#pragma unroll
    for (int di = -2; di <= 2; ++di) {
      if (di == 0 && dj == 0) continue;
      if (di * di + dj * dj > 5) continue;
      int x = i + di, y = j + dj;
      if (!in_grid(F, x, y)) continue;
      if (hgt(x, y) <= P.ein[3]) {
        float dd = (float)(di * di + dj * dj);
        dx += (float)di / dd;
        dy += (float)dj / dd;
      }
    }
  float l = sqrtf(dx * dx + dy * dy);
  if (l < 1e-6f) return make_float2(0.f, 0.f);
  return make_float2(dx / l, dy / l);
}
static __device__ __noinline__ float2 front_normal(const Film& F, const cf_params& P, uint32_t c) {
  return front_normal_at(F, P, (int)(c % F.w), (int)(c / F.w), [&](int x, int y) { return F.hh[idx(F, x, y)]; });
}
// film.wgsl:182-188
__device__ __forceinline__ float wet_gain(float2 n) {
  const float s2 = 0.70710678f;
  float w = W_AXIS * (fmaxf(n.x, 0.f) + fmaxf(-n.x, 0.f) + fmaxf(n.y, 0.f) + fmaxf(-n.y, 0.f));
  w += W_DIAG_FLUX * (fmaxf(s2 * (n.x + n.y), 0.f) + fmaxf(-s2 * (n.x + n.y), 0.f) + fmaxf(s2 * (n.x - n.y), 0.f) +
                      fmaxf(-s2 * (n.x - n.y), 0.f));
  float mm = fmaxf(fmaxf(fabsf(n.x), fabsf(n.y)), 1e-3f);
  return 1.0f / (mm * fmaxf(w, 1e-3f));
}
// film.wgsl:203-222
static __device__ __noinline__ float front_shape(const Film& F, const cf_params& P, uint32_t c, float2 n) {
  int i = (int)(c % F.w), j = (int)(c / F.w);
  float w = 0.f, w0 = 0.f;
  for (int dj = -3; dj <= 3; ++dj)
    for (int di = -3; di <= 3; ++di) {
      if (di == 0 && dj == 0) continue;
      if (di * di + dj * dj > 9) continue;
      if ((float)di * n.x + (float)dj * n.y < -0.5f) w0 += 1.f;
      int x = i + di, y = j + dj;
      if (!in_grid(F, x, y)) continue;
      if (F.hh[idx(F, x, y)] > P.ein[3]) w += 1.f;
    }
  if (w0 < 1.f || ((uint32_t)P.front2[3] & 2u) != 0u) return 1.f;
  return powf(fminf(fmaxf(w / w0, 0.f), 2.5f), P.front2[1]);
}
// film.wgsl:224-229
template <int MODE>
__device__ __forceinline__ float wet_threshold(const Film& F, const DevParams& D, uint32_t c) {
  const cf_params& P = D.p;
  float ty = rtau<MODE>(F, c);
  float need = fmaxf(ty / (P.phys[0] * fmaxf(F.hh[c], 1e-4f)) - D.gxy, 0.f);
  float ycap = need / fmaxf(P.g[2], 1e-3f) * P.dx;
  return fmaxf(D.hold1, ycap);
}
__device__ __forceinline__ float front_dist(const Film& F, uint32_t c) {  // film.wgsl:231-234
  if (F.hh[c] <= 0.f) return 0.f;
  return nose_dist(F, c);
}
// film.wgsl:236-244
__device__ __forceinline__ float cox_speed(const DevParams& D, float excess, float mu) {
  if (excess <= 0.f) return 0.f;
  const float theta = D.cox_theta, adv = D.cox_adv;
  float th = theta + (3.14159265f - theta) * fminf(fmaxf(excess / D.cox_span, 0.f), 1.f);
  if (th <= adv) return 0.f;
  return D.p.phys[1] * (th * th * th - adv * adv * adv) / (132.0f * fmaxf(mu, 1e-4f));
}
// film.wgsl:246-265
static __device__ __noinline__ float cell_excess(const Film& F, const cf_params& P, uint32_t c) {
  float e = F.hh[c] - hold_level(P, front_dist(F, c));
  int ox, oy;
  unpack_off(F.delta[c], ox, oy);
  float ol = off_len(ox, oy);
  if (ol > 0.5f && ol < 60.0f) {
    float dirx = (float)ox * (-1.0f / ol), diry = (float)oy * (-1.0f / ol);
    float bx = 0.5f * sgnf((float)(-ox)), by = 0.5f * sgnf((float)(-oy));
    int ci = (int)(c % F.w), cj = (int)(c / F.w);
    for (uint32_t k = 0; k < 3; ++k) {
      float reach = (float)(4u << k);
      int sx = (int)(dirx * reach + bx), sy = (int)(diry * reach + by);  // toward zero
      int ri = ci + sx, rj = cj + sy;
      if (!in_grid(F, ri, rj)) break;
      uint32_t cr = idx(F, ri, rj);
      if (F.hh[cr] <= 0.f) break;
      e = fmaxf(e, F.hh[cr] - hold_level(P, front_dist(F, cr)));
    }
  }
  return e;
}
// film.wgsl:267-295: (speed term, direction sign)
template <int MODE>
__device__ float2 rim_translation(const Film& F, const DevParams& D, uint32_t ca, uint32_t cb, float hf, float2 fd) {
  const cf_params& P = D.p;
  if (((uint32_t)P.front2[3] & 1u) != 0u) return make_float2(0.f, 0.f);
  float da = front_dist(F, ca), db = front_dist(F, cb);
  if (fmaxf(da, db) > 3.0f / P.front[1]) return make_float2(0.f, 0.f);
  float ha = F.hh[ca], hb = F.hh[cb];
  float2 n = make_float2(0.f, 0.f);
  if (da > db && ha > 0.f) n = F.fnorm[ca];
  else if (db > da && hb > 0.f) n = F.fnorm[cb];
  else {
    if (ha > 0.f) { float2 a = F.fnorm[ca]; n.x += a.x; n.y += a.y; }
    if (hb > 0.f) { float2 b = F.fnorm[cb]; n.x += b.x; n.y += b.y; }
  }
  float nl = sqrtf(n.x * n.x + n.y * n.y);
  if (nl < 1e-6f) return make_float2(0.f, 0.f);
  n.x = n.x / nl;
  n.y = n.y / nl;
  float s = n.x * fd.x + n.y * fd.y;
  if (fabsf(s) < 1e-4f) return make_float2(0.f, 0.f);
  uint32_t src = ca, dst = cb;
  if (s < 0.f) { src = cb; dst = ca; }
  if (F.hh[src] <= 0.f) return make_float2(0.f, 0.f);
  float e = cell_excess(F, P, src);
  if (e <= 0.f) return make_float2(0.f, 0.f);
  float e_out = -D.hold1;
  if (F.hh[dst] > 0.f) e_out = cell_excess(F, P, dst);
  float room = fminf(fmaxf(1.0f - fmaxf(e_out, 0.f) / e, 0.f), 1.f);
  float u = cox_speed(D, e, rmu<MODE>(F, src));
  float t = P.front2[0];
  float mixv = 1.0f * (1.0f - t) + fabsf(s) * t;
  return make_float2(u * hf * room * mixv, sgnf(s));
}

struct FaceOut {
  float q, y, up, n;
};

// Where face() reads the heights and plug mobilities of its two cells: a
// pair source from PtGlobal / PtTile below (h(false), tmp(false): cell a;
// h(true), tmp(true): cell b).
// film.wgsl:297-372 (face between cell a and neighbour b)
template <int MODE, class Pair>
__device__ FaceOut face(const Film& F, const DevParams& D, const Pair& pt, uint32_t ca, uint32_t cb, float2 gcap,
                        float2 ghyd, float2 gtilt, bool diag, float2 fd) {
  const cf_params& P = D.p;
  FaceOut out = {0.f, 0.f, 0.f, 0.f};
  float ha = pt.h(false), hb = pt.h(true);
  float hf = 0.5f * (ha + hb);
  if (hf <= 0.f) return out;
  float shape = 1.f, proj = 1.f;
  bool wetting = false;
  if (fminf(ha, hb) <= 0.f) {
    uint32_t wet = ha > 0.f ? ca : cb;
    uint32_t dry = ha > 0.f ? cb : ca;
    if ((ha > 0.f ? ha : hb) <= wet_threshold<MODE>(F, D, wet)) return out;
    wetting = true;
    float2 n = F.fnorm[wet];
    if (n.x * n.x + n.y * n.y < 0.5f) n = front_normal(F, P, wet);
    float toward = ha > 0.f ? 1.f : -1.f;
    proj = fmaxf(n.x * (fd.x * toward) + n.y * (fd.y * toward), 0.f);
    if (proj <= 0.f) return out;
    shape = front_shape(F, P, dry, n) * wet_gain(n);
    if (shape <= 0.f) return out;
  }
  float ray = rtau<MODE>(F, ca), rby = rtau<MODE>(F, cb);
  float wa = ha / (ha + hb);
  float wb = 1.0f - wa;
  float ty = wa * ray + wb * rby;
  float na = rn<MODE>(F, ca), nb = rn<MODE>(F, cb);
  float nf = na == nb ? na : wa * na + wb * nb;
  float thin = fminf(ha, hb) / hf;
  float fcap = thin * thin * thin;
  // yield_cap (film.wgsl:44-49)
  float2 yc = make_float2(gcap.x * fcap, gcap.y * fcap);
  {
    float gcl = sqrtf(yc.x * yc.x + yc.y * yc.y);
    const float gc_max = D.gc_max;
    if (!(ty <= 0.f || gcl <= gc_max)) {
      float sc = gc_max / gcl;
      yc.x = yc.x * sc;
      yc.y = yc.y * sc;
    }
  }
  float2 gg = make_float2(yc.x + ghyd.x + gtilt.x, yc.y + ghyd.y + gtilt.y);
  float gmag = sqrtf(gg.x * gg.x + gg.y * gg.y);
  float ydep = hf;  // yield_depth (film.wgsl:89-92)
  if (ty > 0.f) ydep = gg.x >= 0.f ? ha : hb;
  float qq = 0.f, qy = 0.f, qup = 0.f;
  // hb_flux gives zero, without reading mu, for a face with no gradient or
  // below its yield stress (y = ydep - ty / |g| <= 0): the log-mean viscosity
  // (film.wgsl:326, an exp and two logs) is evaluated only where it is used
  if (!(gmag < 1e-9f || ydep <= 0.f) && fmaxf(ydep - ty / gmag, 0.f) > 0.f) {
    const float rax = rmu<MODE>(F, ca), rbx = rmu<MODE>(F, cb);
    const float mu = expf(wa * logf(fmaxf(rax, 1e-4f)) + wb * logf(fmaxf(rbx, 1e-4f)));
    hb_flux(gmag, ydep, mu, ty, nf, qq, qy, qup);
  }
  float meff = qq > 0.f ? qq / fmaxf(gmag, 1e-9f) : 0.f;
  float mtilt = meff;
  if (ty > 0.f) {  // plug_mobility (film.wgsl:51-56)
    float gb = sqrtf(gtilt.x * gtilt.x + gtilt.y * gtilt.y);
    if (gb < 1e-6f) mtilt = 0.f;
    else {
      const bool ub = !(gtilt.x >= 0.f);
      mtilt = pt.tmp(ub) * pt.h(ub) / gb;
    }
  }
  if (meff <= 0.f && mtilt <= 0.f) return out;
  float fcap2 = powf(thin, P.front3[3]);
  float qn = mtilt * gtilt.x + fminf(meff, P.misc[3]) * ghyd.x + fminf(meff, P.phys[3]) * (gcap.x * fcap2);
  float2 tr = rim_translation<MODE>(F, D, ca, cb, hf, fd);
  const float vcap = 2.f;
  if (wetting) {
    float want = tr.x * 2.0f * (ha > 0.f ? ha : hb) / fmaxf(hf, 1e-9f);
    qn = tr.y * fmaxf(qn * tr.y * proj, want) * shape;
    if (fabsf(qn) > vcap * hf) qn = sgnf(qn) * vcap * hf;
  } else {
    if (tr.x > 0.f) qn = tr.y * fmaxf(qn * tr.y, tr.x);
    if (fabsf(qn) > vcap * hf) qn = sgnf(qn) * vcap * hf;
    float lo = fminf(ha, hb), hi = fmaxf(ha, hb);
    if (lo < 0.5f * hi) {
      if (diag) qn = 0.f;
      else {
        uint32_t tgt = cb;
        if (hb > ha) tgt = ca;
        uint32_t nfd = feeders(F, P, tgt);
        qn = qn / powf((float)max(nfd, 1u), 0.7f);
      }
    }
  }
  out.q = qn;
  out.y = qy;
  out.up = qup;
  out.n = nf;
  return out;
}

__device__ __forceinline__ float2 pres_at(const Film& F, int i, int j) {
  return F.pres[idx(F, refl_i(F, i), refl_j(F, j))];
}
__device__ __forceinline__ float2 pres_wet(const Film& F, int i, int j, float2 fb) {
  uint32_t c = idx(F, refl_i(F, i), refl_j(F, j));
  float2 p = F.pres[c];
  if (F.hh[c] > 0.f) return p;
  return make_float2(fb.x, p.y);
}

// Sources of the pressures (laplacian) and plug mobilities (plug) the face
// fluxes read.  PtGlobal reads the film's planes, as the dispatches of the
// reference leave them; PtTile reads the flow kernel's shared memory, where
// the tile and its 1-cell ring were evaluated just before (cells of the ring
// in inactive tiles hold the planes' values, as the reference leaves them).
struct PtGlobal {
  const Film& F;
  // the faces it is given may be of dry pairs or inactive neighbours
  static constexpr bool kListed = false;
  struct Pair {
    const float* t;
    const float* hp;
    uint32_t a, b;
    __device__ __forceinline__ float tmp(bool bsel) const { return t[bsel ? b : a]; }
    __device__ __forceinline__ float h(bool bsel) const { return hp[bsel ? b : a]; }
  };
  __device__ __forceinline__ float2 pres(int i, int j) const { return pres_at(F, i, j); }
  __device__ __forceinline__ float2 pwet(int i, int j, float2 fb) const { return pres_wet(F, i, j, fb); }
  __device__ __forceinline__ float hat(int i, int j) const { return F.hh[idx(F, i, j)]; }
  __device__ __forceinline__ Pair pair(int, int, uint32_t ca, int, int, uint32_t cb) const {
    return {F.tmp, F.hh, ca, cb};
  }
};
// Shared-memory boxes of a flow tile on 18 x 18 cells from (i0 - 1, j0 - 1):
// the pressures, plug mobilities and heights, where the positions outside
// the grid hold the values of the cells they reflect to (common.wgsl:152-158),
// so a lookup needs no reflection.  The tile lists only the faces whose
// neighbour is in the grid and active and whose pair is not dry (kListed).
struct PtTile {
  static constexpr bool kListed = true;
  const float2* sp;
  const float* st;
  const float* sh;
  int i0, j0;
  struct Pair {
    const float* t;
    const float* hp;
    int a, b;
    __device__ __forceinline__ float tmp(bool bsel) const { return t[bsel ? b : a]; }
    __device__ __forceinline__ float h(bool bsel) const { return hp[bsel ? b : a]; }
  };
  __device__ __forceinline__ int at18(int i, int j) const { return (j - j0 + 1) * 18 + (i - i0 + 1); }
  __device__ __forceinline__ float2 pres(int i, int j) const { return sp[at18(i, j)]; }
  __device__ __forceinline__ float2 pwet(int i, int j, float2 fb) const {
    const int q = at18(i, j);
    const float2 p = sp[q];
    if (sh[q] > 0.f) return p;
    return make_float2(fb.x, p.y);
  }
  __device__ __forceinline__ float hat(int i, int j) const { return sh[at18(i, j)]; }
  __device__ __forceinline__ Pair pair(int i, int j, uint32_t, int x, int y, uint32_t) const {
    return {st, sh, at18(i, j), at18(x, y)};
  }
};

// film.wgsl:375-446, face k in {0: +x, 1: +y, 2: +x+y, 3: +x-y}.  The
// direction only selects the neighbour, the pressure-gradient stencil, the
// tilt components and the weight; face() then runs once, so a kernel holds a
// single copy of it.
template <int MODE, class PT>
__device__ FaceOut face_k(const Film& F, const DevParams& D, const PT& pt, int i, int j, int k) {
  const cf_params& P = D.p;
  FaceOut z = {0.f, 0.f, 0.f, 0.f};
  const float s2 = 0.70710678f;
  const bool diag = k >= 2;
  const int di = k == 1 ? 0 : 1, dj = k == 0 ? 0 : (k == 3 ? -1 : 1);
  const int x = i + di, y = j + dj;
  if constexpr (!PT::kListed) {
    if (!(in_grid(F, x, y) && cell_active(F, x, y))) return z;
    if (!(0.5f * (F.hh[idx(F, i, j)] + F.hh[idx(F, x, y)]) > 0.f)) return z;  // face() is zero on a dry pair
  }
  const uint32_t c = idx(F, i, j), cb = idx(F, x, y);
  const float2 p00 = pt.pres(i, j), pb = pt.pres(x, y);
  const float2 gxy = make_float2(P.phys[0] * P.g[0], P.phys[0] * P.g[1]);
  float2 gcap, ghyd, gt, fd;
  float wgt;
  if (!diag) {
    // normal gradient across the face, tangential one from the 4 cells beside it
    const int ti = k == 0 ? 0 : 1, tj = k == 0 ? 1 : 0;
    const float2 gm = make_float2(-(pb.x - p00.x) * P.inv_dx, -(pb.y - p00.y) * P.inv_dx);
    const float2 a = pt.pwet(i + ti, j + tj, p00), b = pt.pwet(x + ti, y + tj, pb);
    const float2 cc = pt.pwet(i - ti, j - tj, p00), d = pt.pwet(x - ti, y - tj, pb);
    const float2 pt = make_float2(a.x + b.x - cc.x - d.x, a.y + b.y - cc.y - d.y);
    const float2 gtt = make_float2(-pt.x * 0.25f * P.inv_dx, -pt.y * 0.25f * P.inv_dx);
    gcap = make_float2(gm.x, gtt.x);
    ghyd = make_float2(gm.y, gtt.y);
    gt = k == 0 ? gxy : make_float2(gxy.y, gxy.x);
    fd = k == 0 ? make_float2(1.f, 0.f) : make_float2(0.f, 1.f);
    wgt = W_AXIS;
  } else {
    const float2 ga = make_float2(-(pb.x - p00.x) * P.inv_dx * s2, -(pb.y - p00.y) * P.inv_dx * s2);
    const float2 pa = pt.pwet(i + 1, j, p00), pc = pt.pwet(i, j + dj, pb);
    const float2 gp = make_float2(-(pa.x - pc.x) * P.inv_dx * s2, -(pa.y - pc.y) * P.inv_dx * s2);
    const float hs = P.ein[3];
    const bool open = fminf(pt.hat(i, j), pt.hat(x, y)) > 0.f || pt.hat(i + 1, j) > hs || pt.hat(i, j + dj) > hs;
    if (!open) return z;
    gcap = make_float2(ga.x, gp.x);
    ghyd = make_float2(ga.y, gp.y);
    gt = k == 2 ? make_float2((gxy.x + gxy.y) * s2, (gxy.x - gxy.y) * s2)
                : make_float2((gxy.x - gxy.y) * s2, (gxy.x + gxy.y) * s2);
    fd = make_float2(s2, k == 2 ? s2 : -s2);
    wgt = W_DIAG_FLUX;
  }
  FaceOut f = face<MODE>(F, D, pt.pair(i, j, c, x, y, cb), c, cb, gcap, ghyd, gt, diag, fd);
  f.q *= wgt;
  return f;
}

// ---- Kubelka-Munk (km.wgsl) ----
__device__ __forceinline__ void km_layer(float k, float s, float t, float& r, float& tr) {  // km.wgsl:1-11
  if (k + s < 1e-6f || t <= 0.f) { r = 0.f; tr = 1.f; return; }
  float bs = sqrtf(fmaxf(k * (k + 2.0f * s), 0.f));
  float arg = fminf(bs * t, 20.0f);
  float e = expf(arg);
  const float ie = __frcp_rn(e);  // e >= 1: a correctly rounded reciprocal
  float sh = 0.5f * (e - ie);
  float ch = 0.5f * (e + ie);
  float den = (k + s) * sh + bs * ch;
  if (den < 1e-12f) { r = 0.f; tr = 1.f; return; }
  const float iden = __frcp_rn(den);
  r = s * sh * iden;
  tr = bs * iden;
}
__device__ __forceinline__ float composite(float r, float t, float rb) {  // km.wgsl:13-15
  return r + __fdividef(t * t * rb, fmaxf(1.0f - r * rb, 1e-4f));
}

}  // namespace cfk
