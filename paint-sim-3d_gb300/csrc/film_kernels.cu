// film_kernels.cu — sm_103a kernels of the thin-film step and their host
// launchers.  The frame follows Film::encode_frame (src/film/mod.rs:1322-1462):
//
//   mark_tiles, compact_tiles          16x16 tile activity (film.wgsl:1365-1425)
//   cure                               cure.wgsl:119-159, from per-frame aggregates
//   [clear_acc + laplacian], plug, fluxes, limiter, apply, nose   per substep
//   laplacian, strata_split, reduce_tiles
//   strata pass: strata_limit + strata_update + shade_full + the next frame's
//                rheology aggregates: a grid kernel takes the fast path and
//                lists the other cells, a list kernel (one cell per
//                half-warp) takes the full path, then the listed cells'
//                pigments are copied back
//   strata_fill x 6                    one block over the fill candidates
//
// Launch geometry: one 16x16 block per 16x16 activity tile.  A tile-list
// dispatch of the reference becomes a full-grid launch whose blocks on
// inactive tiles return at once (or, for the strata pass, carry their strata
// over), so the active set stays on the device and the frame needs no host
// round trip.  Dispatches whose invocations read what the same dispatch
// writes in the reference (nose, strata_fill) read a snapshot or run in two
// passes (Jacobi semantics).
#include <cuda_runtime.h>

#include <string_view>

#include "film_device.cuh"
#include "film_kernels.h"
#include "strata_device.cuh"
#include "strata_lane.cuh"
#include "tma.cuh"

namespace cfk {

// A kernel body works on one 16x16 tile T of film F.  The single-film
// kernels bind T to blockIdx; the packed kernels (k*_packed) take film and
// tile from an entry of a tile table that spans many films.
struct TileId {
  uint32_t x, y;
};

#define TILE_PROLOGUE                                              \
  const int i = (int)(T.x * 16 + threadIdx.x);                     \
  const int j = (int)(T.y * 16 + threadIdx.y);                     \
  if ((F.tile_flags[T.x + T.y * F.tw] & ACTIVE) == 0u) return;     \
  if (i >= (int)F.w || j >= (int)F.h) return;                      \
  const uint32_t c = idx(F, i, j);                                 \
  const DevParams& D = *F.P;                                       \
  const cf_params& P = D.p;                                        \
  (void)P;

__device__ __forceinline__ float sel4(float4 v, int k) {
  return k == 0 ? v.x : (k == 1 ? v.y : (k == 2 ? v.z : v.w));
}
__device__ __forceinline__ float4 neg4(float4 v) { return make_float4(-v.x, -v.y, -v.z, -v.w); }
__device__ __forceinline__ bool nb_ok(const Film& F, int i, int j) { return in_grid(F, i, j) && cell_active(F, i, j); }

// film.wgsl:1365-1391, one warp per 16x16 tile: lane l takes half a row
// (row l/2, columns 8(l%2)..+7), every load of the tile is issued before any
// is used, and a warp OR replaces the workgroup atomics.
__device__ __forceinline__ void mark_tile(const Film& F, uint32_t t) {
  const uint32_t lane = threadIdx.x & 31u;
  const uint32_t moved_before = lane == 0u ? F.tile_moved[t] : 0u;
  const int i0 = (int)((t % F.tw) * 16u + (lane & 1u) * 8u), j = (int)((t / F.tw) * 16u + (lane >> 1));
  float hv[8], hf[8];
  if ((F.w & 3u) == 0u && i0 + 8 <= (int)F.w && j < (int)F.h) {
    // the half row as two 16-byte loads per plane (planes are 256-byte
    // aligned, rows start on a multiple of 4 cells, i0 on a multiple of 8)
    const uint32_t c = idx(F, i0, j);
    const float4* ph = reinterpret_cast<const float4*>(F.hh + c);
    const float4* pf = reinterpret_cast<const float4*>(F.h_frame + c);
    const float4 a0 = ph[0], a1 = ph[1], b0 = pf[0], b1 = pf[1];
    hv[0] = a0.x; hv[1] = a0.y; hv[2] = a0.z; hv[3] = a0.w; hv[4] = a1.x; hv[5] = a1.y; hv[6] = a1.z; hv[7] = a1.w;
    hf[0] = b0.x; hf[1] = b0.y; hf[2] = b0.z; hf[3] = b0.w; hf[4] = b1.x; hf[5] = b1.y; hf[6] = b1.z; hf[7] = b1.w;
  } else {
#pragma unroll
    for (int k = 0; k < 8; ++k) {
      const bool in = i0 + k < (int)F.w && j < (int)F.h;
      const uint32_t c = in ? idx(F, i0 + k, j) : 0u;
      hv[k] = in ? F.hh[c] : 0.f;
      hf[k] = in ? F.h_frame[c] : 0.f;
    }
  }
  uint32_t bits = 0u;
#pragma unroll
  for (int k = 0; k < 8; ++k)
    if (hv[k] > 0.f) {
      bits |= 1u | ((lane & 1u) ? 4u : 2u) | ((lane >> 1) < 8u ? 8u : 16u);
      if (fabsf(hv[k] - hf[k]) > FRAME_EPS) bits |= MOVED;
    }
  bits = __reduce_or_sync(0xffffffffu, bits);
  if (lane == 0u) {
    if (moved_before != 0u) bits |= MOVED;
    F.tile_moved[t] = 0u;
    F.tile_flags[t] = bits;
  }
}

// film.wgsl:1393-1425 (bit 32 is written in place; the bits read are not it).
// Returns whether the tile is active; the caller counts the active tiles.
__device__ __forceinline__ bool compact_tile(const Film& F, uint32_t t, int all_active) {
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
    return true;
  }
  F.tile_flags[t] = own & 31u;
  return false;
}

// The commit of the bottom stratum into the relief (cure.wgsl:119-159), the
// rare branch of cure_tile: out of line so that the common path keeps few
// registers.
template <int MODE>
static __device__ __noinline__ void cure_commit(const Film& F, const cf_params& P, uint32_t c, float4 u4) {
  const float u[4] = {u4.x, u4.y, u4.z, u4.w};
  Stack s;
  stack_load<MODE>(F, F.sh, F.scu, F.pig, c, s);
#pragma unroll
  for (int k = 0; k < 4; ++k) s.cu[k] = u[k];
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
  float lt[12];
  lnmu_table(F.pigtab, lt);
  float4 agg;
  ushort4 col_unused;
  finish_stack(P, lt, F.pigtab, F.cmf, F.refl + (size_t)c * 16, F.hh[c], F.m[c], s, agg, col_unused);
  float mu, ty, n;
  rheo_from_parts(P, agg, s.th, s.cu, mu, ty, n);
  set_rheo<MODE>(F, c, mu, ty, n);
  stack_store<MODE>(F, F.sh, F.scu, F.pig, c, s);
  F.agg[c] = agg;
  F.shade_state[c] = SHADE_NONE;  // strata and substrate changed
}
// cure.wgsl:119-159 (full grid).  The pigment part of the composition comes
// from agg (written by the last strata pass); the stack is only read when
// the bottom stratum commits.
template <int MODE>
__device__ __forceinline__ void cure_tile(const Film& F, TileId T) {
  const int i = (int)(T.x * 16 + threadIdx.x), j = (int)(T.y * 16 + threadIdx.y);
  if (i >= (int)F.w || j >= (int)F.h) return;
  const uint32_t c = idx(F, i, j);
  const cf_params& P = F.P->p;
  float hv = F.hh[c];
  if (hv <= 0.f) { set_rheo<MODE>(F, c, 1.f, 0.f, P.phys[2]); return; }
  float rate = P.cure[0] * P.frame_dt;
  // the aggregates load with the strata, ahead of the cure store (which
  // the compiler could not move them past)
  const float4 t4 = F.sh[c], c4 = F.scu[c], ag = F.agg[c];
  float t[4] = {t4.x, t4.y, t4.z, t4.w}, u[4] = {c4.x, c4.y, c4.z, c4.w};
#pragma unroll
  for (int k = 0; k < 4; ++k) u[k] = t[k] > 0.f ? fminf(u[k] + rate, 1.f) : u[k];
  if (!(t[0] > 0.f && u[0] >= 1.f)) {
    F.scu[c] = make_float4(u[0], u[1], u[2], u[3]);
    float mu, ty, n;
    rheo_from_parts(P, ag, t, u, mu, ty, n);
    set_rheo<MODE>(F, c, mu, ty, n);
    return;
  }
  cure_commit<MODE>(F, P, c, make_float4(u[0], u[1], u[2], u[3]));
}

// film.wgsl:1427-1434
__device__ __forceinline__ void clear_acc_tile(const Film& F, TileId T) {
  TILE_PROLOGUE
  F.acc[c] = make_float4(0.f, 0.f, 0.f, 0.f);
  F.h_frame[c] = F.hh[c];
}

// film.wgsl:58-87.  The HB flux of every cell of the tile and its 3-cell
// halo is evaluated once into shared memory; each cell then sums its 7x7
// window in the reference's row-major order, so the result is identical to
// evaluating the flux 49 times per cell.
template <int MODE>
__device__ __forceinline__ void plug_tile(const Film& F, TileId T) {
  constexpr int R = 3, S = 16 + 2 * R;
  __shared__ float2 sqm[S * S];  // flux q and mass h of each window cell (0, 0 where dry or outside)
  __shared__ uint8_t sy[S * S];  // bit 0: wet cell in the grid, bit 1: tau_y > 0
  if ((F.tile_flags[T.x + T.y * F.tw] & ACTIVE) == 0u) return;
  const DevParams& D = *F.P;
  const cf_params& P = D.p;
  const float gb = P.phys[0] * D.gxy;
  const int x0 = (int)T.x * 16 - R, y0 = (int)T.y * 16 - R;
  const int tid = threadIdx.y * 16 + threadIdx.x;
  for (int q = tid; q < S * S; q += 256) {
    int x = x0 + q % S, y = y0 + q / S;
    float qq = 0.f, mass = 0.f;
    uint8_t yl = 0;
    if (in_grid(F, x, y)) {
      uint32_t n = idx(F, x, y);
      float hn = F.hh[n];
      if (hn > 0.f) {
        float rx = rmu<MODE>(F, n), ry = rtau<MODE>(F, n);
        yl = (uint8_t)(1u | (ry > 0.f ? 2u : 0u));
        float yy, up;
        hb_flux(gb, hn, fmaxf(rx, 1e-4f), ry, rn<MODE>(F, n), qq, yy, up);
        mass = hn;
      }
    }
    sqm[q] = make_float2(qq, mass);
    sy[q] = yl;
  }
  __syncthreads();
  const int i = (int)(T.x * 16 + threadIdx.x), j = (int)(T.y * 16 + threadIdx.y);
  if (i >= (int)F.w || j >= (int)F.h) return;
  const uint32_t c = idx(F, i, j);
  F.tmp[c] = 0.f;
  if (F.hh[c] <= 0.f) return;
  if (gb < 1e-6f) return;
  // The reference adds the wet cells of the window in row-major order; the
  // dry and outside ones hold q = mass = +0 here, and adding +0 to these
  // non-negative sums leaves them bit for bit as they are, so every window
  // cell is added without a branch.
  float sum = 0.f, mass = 0.f;
  uint32_t fl = 0u;
  for (int dy = 0; dy < 7; ++dy)
#pragma unroll
    for (int dx = 0; dx < 7; ++dx) {
      const int q = (threadIdx.y + dy) * S + threadIdx.x + dx;
      const float2 v = sqm[q];
      fl |= sy[q];
      sum += v.x;
      mass += v.y;
    }
  if (!(fl & 2u) || mass <= 0.f) return;
  F.tmp[c] = sum / mass;
}

// film.wgsl:516-537
// 64 threads per tile, 4 cells each (rows y, y + 4, y + 8, y + 12): every
// load of the 4 cells is issued before any of them is used, so a warp keeps
// 4x the bytes in flight behind the tile's dependent prologue.
__device__ __forceinline__ void limiter_tile(const Film& F, TileId T) {
  if ((F.tile_flags[T.x + T.y * F.tw] & ACTIVE) == 0u) return;
  const cf_params& P = F.P->p;
  const int i = (int)(T.x * 16 + threadIdx.x), W = (int)F.w, H = (int)F.h;
  const bool al = i > 0 && cell_active(F, i - 1, (int)T.y * 16);  // the left tile (all 4 rows share it)
  float4 f[4];
  float nl[4], nd[4], ndl[4], ndu[4], hv[4];
#pragma unroll
  for (int r = 0; r < 4; ++r) {
    const int j = (int)(T.y * 16 + threadIdx.y + 4 * r);
    f[r] = make_float4(0.f, 0.f, 0.f, 0.f);
    nl[r] = nd[r] = ndl[r] = ndu[r] = hv[r] = 0.f;
    if (i >= W || j >= H) continue;
    const uint32_t c = idx(F, i, j);
    f[r] = F.flux[c];
    hv[r] = F.hh[c];
    if (i > 0) nl[r] = F.flux[c - 1].x;
    if (j > 0) nd[r] = F.flux[c - F.w].y;
    if (i > 0 && j > 0) ndl[r] = F.flux[c - F.w - 1].z;
    if (i > 0 && j + 1 < H) ndu[r] = F.flux[c + F.w - 1].w;
  }
#pragma unroll
  for (int r = 0; r < 4; ++r) {
    const int j = (int)(T.y * 16 + threadIdx.y + 4 * r);
    if (i >= W || j >= H) continue;
    float out = fmaxf(f[r].x, 0.f) + fmaxf(f[r].y, 0.f) + fmaxf(f[r].z, 0.f) + fmaxf(f[r].w, 0.f);
    // neighbours of the left tile column, the tile row below and above (film.wgsl nb_ok)
    const bool l_ok = i > 0 && ((i & 15) ? true : al);
    if (l_ok) out += fmaxf(-nl[r], 0.f);
    if (j > 0 && cell_active(F, i, j - 1)) out += fmaxf(-nd[r], 0.f);
    if (i > 0 && j > 0 && cell_active(F, i - 1, j - 1)) out += fmaxf(-ndl[r], 0.f);
    if (i > 0 && j + 1 < H && cell_active(F, i - 1, j + 1)) out += fmaxf(-ndu[r], 0.f);
    float a = 1.f;
    if (out > 0.f) a = fminf(1.f, 0.5f * hv[r] * P.dx / (P.dt * out));
    F.alpha[idx(F, i, j)] = a;
  }
}

// wetting back-fill (film.wgsl:847-860 / strata.wgsl:314-322) on the current
// strata generation: cell c takes the top stratum of src
template <int MODE>
__device__ __forceinline__ void backfill(const Film& F, uint32_t c, uint32_t src, float hn) {
  float4 ts = F.sh[src];
  int ks = 0;
  if (ts.x > 0.f) ks = 0;
  if (ts.y > 0.f) ks = 1;
  if (ts.z > 0.f) ks = 2;
  if (ts.w > 0.f) ks = 3;
  F.sh[c] = make_float4(hn, 0.f, 0.f, 0.f);
  PigIO<MODE>::copy(F, F.pig, c, 0, F.pig, src, ks);
#pragma unroll
  for (int k = 1; k < 4; ++k) PigIO<MODE>::zero(F, F.pig, c, k);
  float4 cs = F.scu[src];
  float cv = ks == 0 ? cs.x : (ks == 1 ? cs.y : (ks == 2 ? cs.z : cs.w));
  F.scu[c] = make_float4(cv, 0.f, 0.f, 0.f);
  F.shade_state[c] = SHADE_NONE;  // new strata and pigments
}

// film.wgsl:539-561, 803-863
template <int MODE>
// Every tile (active or not) also snapshots delta into delta_old for the
// nose that follows (apply does not write delta).
__device__ __forceinline__ void apply_tile(const Film& F, TileId T) {
  // 128 threads per tile, 2 cells each (rows y and y + 8): every load of
  // both cells (the neighbours in the grid unconditionally, their activity
  // applied after) is issued before the first use.
  constexpr int R = 2;
  const int i = (int)(T.x * 16 + threadIdx.x);
  const bool ci = i < (int)F.w;
#pragma unroll
  for (int r = 0; r < R; ++r) {
    const int j = (int)(T.y * 16 + threadIdx.y + 8 * r);
    if (ci && j < (int)F.h) F.delta_old[idx(F, i, j)] = F.delta[idx(F, i, j)];
  }
  if ((F.tile_flags[T.x + T.y * F.tw] & ACTIVE) == 0u) return;
  const cf_params& P = F.P->p;
  bool moved = false;
  uint32_t cc[R], cbs[R][4], cl[R], cd[R], cdl[R], cul[R];
  float ac[R], abn[R][4], ql[R], qd[R], qdl[R], qul[R], al[R], ad[R], adl[R], aul[R], h0[R];
  float4 f4[R], a4[R];
#pragma unroll
  for (int r = 0; r < R; ++r) {
    const int j = (int)(T.y * 16 + threadIdx.y + 8 * r);
    const bool in = ci && j < (int)F.h;
    const uint32_t c = in ? idx(F, i, j) : 0u;
    cc[r] = c;
    const bool hx = i + 1 < (int)F.w, hy = j + 1 < (int)F.h, hm = j > 0, hl = i > 0;
    cbs[r][0] = hx ? c + 1 : c;
    cbs[r][1] = hy ? c + F.w : c;
    cbs[r][2] = (hx && hy) ? c + F.w + 1 : c;
    cbs[r][3] = (hx && hm) ? c - F.w + 1 : c;
    cl[r] = hl ? c - 1 : c;
    cd[r] = hm ? c - F.w : c;
    cdl[r] = (hl && hm) ? c - F.w - 1 : c;
    cul[r] = (hl && hy) ? c + F.w - 1 : c;
    if (!in) continue;
    ac[r] = F.alpha[c];
    f4[r] = F.flux[c];
#pragma unroll
    for (int k = 0; k < 4; ++k) abn[r][k] = F.alpha[cbs[r][k]];
    ql[r] = F.flux[cl[r]].x;
    qd[r] = F.flux[cd[r]].y;
    qdl[r] = F.flux[cdl[r]].z;
    qul[r] = F.flux[cul[r]].w;
    al[r] = F.alpha[cl[r]];
    ad[r] = F.alpha[cd[r]];
    adl[r] = F.alpha[cdl[r]];
    aul[r] = F.alpha[cul[r]];
    h0[r] = F.hh[c];
    a4[r] = F.acc[c];
  }
#pragma unroll
  for (int r = 0; r < R; ++r) {
    const int j = (int)(T.y * 16 + threadIdx.y + 8 * r);
    if (!(ci && j < (int)F.h)) continue;
    const uint32_t c = cc[r];
    const bool hx = i + 1 < (int)F.w, hy = j + 1 < (int)F.h, hm = j > 0, hl = i > 0;
    const bool has[4] = {hx, hy, hx && hy, hx && hm};
    float best = 0.f, div = 0.f;
    uint32_t src = c;
    const float f[4] = {f4[r].x, f4[r].y, f4[r].z, f4[r].w};
    float accv[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      float q = f[k], ab = ac[r];
      if (q < 0.f && has[k]) {
        ab = abn[r][k];
        if (-q * ab > best) { best = -q * ab; src = cbs[r][k]; }
      }
      div += q * ab;
      accv[k] = q * ab;
    }
    auto nb_face = [&](float q, float an, uint32_t cn) {
      if (q < 0.f) an = ac[r];
      if (q * an > best) { best = q * an; src = cn; }
      div -= q * an;
    };
    if (hl && cell_active(F, i - 1, j)) nb_face(ql[r], al[r], cl[r]);
    if (hm && cell_active(F, i, j - 1)) nb_face(qd[r], ad[r], cd[r]);
    if (hl && hm && cell_active(F, i - 1, j - 1)) nb_face(qdl[r], adl[r], cdl[r]);
    if (hl && hy && cell_active(F, i - 1, j + 1)) nb_face(qul[r], aul[r], cul[r]);
    float hn = fmaxf(h0[r] - P.dt * div * P.inv_dx, 0.f);
    if (hn < h0[r] && hn < DRAINED_FILM) hn = 0.f;
    F.hh[c] = hn;
    moved = moved || fabsf(hn - h0[r]) > MOVE_EPS;
    if (h0[r] <= 0.f && src != c) {
      set_rheo<MODE>(F, c, rmu<MODE>(F, src), rtau<MODE>(F, src), rn<MODE>(F, src));
      backfill<MODE>(F, c, src, hn);
    }
    const float4 a = a4[r];
    F.acc[c] = make_float4(a.x + accv[0] * P.dt, a.y + accv[1] * P.dt, a.z + accv[2] * P.dt, a.w + accv[3] * P.dt);
  }
  if (__syncthreads_or(moved) && threadIdx.x == 0 && threadIdx.y == 0)
    F.tile_moved[T.x + T.y * F.tw] = 1u;
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

// film.wgsl:1330-1361 over one 16x16 tile: the device-wide max / min the
// adaptive step reads (order-independent, so the tile shape does not matter).
template <int MODE>
__device__ __forceinline__ void reduce16_tile(const Film& F, TileId T) {
  const cf_params& P = F.P->p;
  float hm = 0.f, mm = 1e9f;
  const int i = (int)(T.x * 16 + threadIdx.x), j = (int)(T.y * 16 + threadIdx.y);
  if (i < (int)F.w && j < (int)F.h) {
    uint32_t c = idx(F, i, j);
    float v = F.hh[c];
    if (v > 4.0f * P.ein[3]) { hm = v; mm = rmu<MODE>(F, c); }
  }
  for (int o = 16; o > 0; o >>= 1) {
    hm = fmaxf(hm, __shfl_xor_sync(0xffffffffu, hm, o));
    mm = fminf(mm, __shfl_xor_sync(0xffffffffu, mm, o));
  }
  // one pair of atomics per tile, and none for a tile without such a cell
  // (its partials are the identities 0 and 1e9)
  __shared__ float sh[8], sm[8];
  const int tid = threadIdx.y * 16 + threadIdx.x;
  if ((tid & 31) == 0) { sh[tid >> 5] = hm; sm[tid >> 5] = mm; }
  __syncthreads();
  if (tid == 0) {
#pragma unroll
    for (int w = 1; w < 8; ++w) { hm = fmaxf(hm, sh[w]); mm = fminf(mm, sm[w]); }
    if (hm > 0.f) fold_cfl(F.stats, hm, mm);
  }
}

// strata.wgsl:157-173 for one active cell
__device__ __forceinline__ float4 strata_limit_at(const Film& F, const cf_params& P, int i, int j) {
  uint32_t c = idx(F, i, j);
  const uint32_t f0 = F.fflags[c];
  float4 a0 = acc_face_live(F, c, 0, f0), a1 = acc_face_live(F, c, 1, f0), a2 = acc_face_live(F, c, 2, f0),
         a3 = acc_face_live(F, c, 3, f0);
  float out[4];
  out[0] = fmaxf(a0.x, 0.f) + fmaxf(a1.x, 0.f) + fmaxf(a2.x, 0.f) + fmaxf(a3.x, 0.f);
  out[1] = fmaxf(a0.y, 0.f) + fmaxf(a1.y, 0.f) + fmaxf(a2.y, 0.f) + fmaxf(a3.y, 0.f);
  out[2] = fmaxf(a0.z, 0.f) + fmaxf(a1.z, 0.f) + fmaxf(a2.z, 0.f) + fmaxf(a3.z, 0.f);
  out[3] = fmaxf(a0.w, 0.f) + fmaxf(a1.w, 0.f) + fmaxf(a2.w, 0.f) + fmaxf(a3.w, 0.f);
  auto addn = [&](uint32_t n, int f) {
    float4 v = acc_face_live(F, n, f, F.fflags[n]);
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
  return make_float4(a[0], a[1], a[2], a[3]);
}

// strata_limit as a dispatch of its own (inspection only; the strata pass
// computes the same values in shared memory)
__device__ __forceinline__ void strata_limit_tile(const Film& F, TileId T) {
  TILE_PROLOGUE
  F.alpha_s[c] = strata_limit_at(F, P, i, j);
}

// Face flags from a whole acc_s plane (for an inspection dispatch of
// strata_limit or of the strata pass that does not follow a strata_split, on
// an uploaded acc_s).
__device__ __forceinline__ void face_flags_tile(const Film& F, TileId T) {
  TILE_PROLOGUE
  uint32_t flags = 0u;
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    float4 o = acc_face(F, c, k);
    if (o.x != 0.f || o.y != 0.f || o.z != 0.f || o.w != 0.f) flags |= 1u << k;
  }
  F.fflags[c] = flags;
}

// Whether the stack renormalised to h is not compact (strata.wgsl:222-228),
// which sends a cell without strata fluxes down the full path as well.
__device__ __forceinline__ bool not_compact(const cf_params& P, float hc, float4 t4) {
  if (hc <= 0.f) return false;
  float th[4] = {fmaxf(t4.x, 0.f), fmaxf(t4.y, 0.f), fmaxf(t4.z, 0.f), fmaxf(t4.w, 0.f)};
  float nt[4] = {th[0], th[1], th[2], th[3]};
  float sum = th[0] + th[1] + th[2] + th[3];
  if (sum > 0.f) {
    float sc = hc / sum;
#pragma unroll
    for (int k = 0; k < 4; ++k) nt[k] = th[k] * sc;
  }
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    if (nt[k] <= 0.f && nt[k + 1] > 0.f) return true;
    if (nt[k] > 0.f && nt[k] < P.misc[0] && nt[k + 1] > 0.f) return true;
  }
  return false;
}

// ---- face passes: fluxes and strata_split over the live faces of a tile ----
// Face k of cell (i, j) joins cell (i + FACE_DI[k], j + FACE_DJ[k]).
__device__ __constant__ int FACE_DI[4] = {1, 0, 1, 1};
__device__ __constant__ int FACE_DJ[4] = {0, 1, 1, -1};

// The block's faces that need evaluation, compacted in shared memory and
// grouped by direction: a warp then evaluates 32 faces of (mostly) one
// direction instead of 32 cells of which few have a live face, and no lane
// waits on a dry neighbour.  Entries are cell positions within the tile.
struct TileFaces {
  uint8_t cell[4][256];
  uint32_t count[4];
};
// Lists face k of the cell in slot `slot` of the tile (y * 16 + x) when
// `live` (every thread of the block calls this, with the same k).
__device__ __forceinline__ void tile_faces_add(TileFaces& S, int k, bool live, int slot) {
  const int lane = (int)(threadIdx.y * 16 + threadIdx.x) & 31;
  const unsigned m = __ballot_sync(0xffffffffu, live);
  uint32_t base = 0;
  if (lane == 0 && m) base = atomicAdd(&S.count[k], (uint32_t)__popc(m));
  base = __shfl_sync(0xffffffffu, base, 0);
  if (live) S.cell[k][base + __popc(m & ((1u << lane) - 1u))] = (uint8_t)slot;
}
__device__ __forceinline__ void tile_faces_add(TileFaces& S, int k, bool live) {
  tile_faces_add(S, k, live, (int)(threadIdx.y * 16 + threadIdx.x));
}
// Runs fn(k, i, j, c) for every listed face, the block's NT threads in turn.
template <int NT = 256, class Fn>
__device__ __forceinline__ void tile_faces_each(const Film& F, TileId T, const TileFaces& S, Fn fn) {
  const uint32_t n0 = S.count[0], n1 = n0 + S.count[1], n2 = n1 + S.count[2], n3 = n2 + S.count[3];
  for (uint32_t e = threadIdx.y * 16 + threadIdx.x; e < n3; e += NT) {
    const int k = e < n0 ? 0 : e < n1 ? 1 : e < n2 ? 2 : 3;
    const uint32_t base = k == 0 ? 0u : k == 1 ? n0 : k == 2 ? n1 : n2;
    const uint32_t t = S.cell[k][e - base];
    const int i = (int)(T.x * 16 + (t & 15u)), j = (int)(T.y * 16 + (t >> 4));
    fn(k, i, j, idx(F, i, j));
  }
}

// fluxes (film.wgsl:448-455) for one tile: the active cells' flux is zeroed,
// then the faces that face_k does not return zero for at once (the neighbour
// in the grid and active, 0.5 (h_a + h_b) > 0) are evaluated.
template <int MODE>
__device__ __forceinline__ void fluxes_tile(const Film& F, TileId T) {
  __shared__ TileFaces S;
  if ((F.tile_flags[T.x + T.y * F.tw] & ACTIVE) == 0u) return;
  const int i = (int)(T.x * 16 + threadIdx.x), j = (int)(T.y * 16 + threadIdx.y);
  const bool in = i < (int)F.w && j < (int)F.h;
  if (threadIdx.y == 0 && threadIdx.x < 4) S.count[threadIdx.x] = 0u;
  __syncthreads();
  const uint32_t c = in ? idx(F, i, j) : 0u;
  const float hc = in ? F.hh[c] : 0.f;
  if (in) F.flux[c] = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    const int x = i + FACE_DI[k], y = j + FACE_DJ[k];
    tile_faces_add(S, k, in && in_grid(F, x, y) && cell_active(F, x, y) && 0.5f * (hc + F.hh[idx(F, x, y)]) > 0.f);
  }
  __syncthreads();
  const DevParams& D = *F.P;
  float* fl = reinterpret_cast<float*>(F.flux);
  tile_faces_each(F, T, S, [&](int k, int fi, int fj, uint32_t fc) {
    fl[4 * (size_t)fc + k] = face_k<MODE>(F, D, PtGlobal{F}, fi, fj, k).q;
  });
}

// ---- the flow tile: laplacian + plug + fluxes of one substep, fused ----
// The reference's dispatches laplacian -> plug -> fluxes (film.wgsl:16-87,
// 448-455) pass the pressures and plug mobilities of every cell through
// device memory.  A flow block does the three for one 16x16 tile: it stages
// h, m, the front offsets and the rheology of the tile and a 4-cell halo in
// shared memory (tensor loads where the film has descriptors), evaluates the
// surface levels on the tile + 2 rings, the pressures and plug mobilities of
// the tile + 1 ring (what the faces read), then the faces.  Each value is the
// expression the separate kernels evaluate, so the fluxes are the separate
// dispatches' to rounding.  The plug mobilities of the tile go to the tmp
// plane (strata_split reads the last substep's); the pressures stay on chip:
// laplacian is dispatched again before strata_split, and no other kernel
// reads them in between.
constexpr int FB = 24;                 // staged box: tile + 4 cells each side
constexpr uint32_t FLOW_WAIT_POLLS = 1u << 22;
struct FlowSmem {
  float h[FB * FB];                    // box origin (i0 - 4, j0 - 4)
  float m[FB * FB];
  uint32_t dl[FB * FB];
  uint32_t rh[3][FB * FB];             // mu, tau, n: f32 24 x 24, or bf16 32 x 24 from (i0 - 8, j0 - 4)
  float su[20 * 20];                   // surface levels, origin (i0 - 2, j0 - 2)
  float2 pres[18 * 18];                // origin (i0 - 1, j0 - 1)
  float tmp[18 * 18];
  float hr[18 * 18];                   // h, positions outside the grid reflected
  float2 qm[FB * FB];                  // plug flux q and mass h of the window cells
  uint8_t yl[FB * FB];
  TileFaces faces;
  uint64_t bar;
};
template <int MODE>
__device__ __forceinline__ float staged_rh(const FlowSmem& S, int plane, int b) {
  if constexpr (MODE == CF_PREC_BF16) {
    const int bx = b % FB, by = b / FB;
    return b16_to_f(reinterpret_cast<const uint16_t*>(S.rh[plane])[by * 32 + bx + 4]);
  } else {
    return __uint_as_float(S.rh[plane][b]);
  }
}
// The tile's box of h, m and the front offsets (and with RHEO, where `rheo`
// is set, the three rheology planes) into shared memory: tensor loads when
// the film has descriptors, else loads by the block's threads (zero outside
// the grid, as the tensor loads fill).  Returns false (counted in the film's
// stats) when the tensor loads did not arrive within the wait limit.
// The block's tensor loads into shared memory: tma_block_arm initialises the
// barrier (every thread calls it; thread 0 then arms it with the expected
// bytes and issues the loads), tma_block_wait waits for them, bounded.  A
// block whose loads did not arrive within the limit counts a timeout in the
// film's stats, lets the loads still in flight land (bounded again) and
// returns false: the caller leaves the tile.
__device__ __forceinline__ void tma_block_arm(uint64_t* bar, int tid) {
  if (tid == 0) {
    mbar_init(bar, 1);
    mbar_fence_init();
  }
  __syncthreads();
}
__device__ __forceinline__ bool tma_block_wait(const Film& F, uint64_t* bar, int tid) {
  const bool arrived = __syncthreads_and(mbar_wait_bounded(bar, 0, FLOW_WAIT_POLLS));
  if (!arrived) {
    if (tid == 0) {
      atomicAdd(&F.stats->tma_timeouts, 1u);
      mbar_wait_bounded(bar, 0, FLOW_WAIT_POLLS);
    }
    __syncthreads();
    return false;
  }
  __syncthreads();
  if (tid == 0) mbar_inval(bar);
  return true;
}
template <int MODE, bool RHEO, class Smem, int NT = 256>
__device__ __forceinline__ bool stage_box(const Film& F, Smem& S, int i0, int j0, int tid, bool rheo = RHEO) {
  constexpr bool B16 = MODE == CF_PREC_BF16;
  if (F.tmap != nullptr) {
    tma_block_arm(&S.bar, tid);
    if (tid == 0) {
      const uint32_t rb = B16 ? 32 * FB * 2 : FB * FB * 4;
      mbar_arrive_expect_tx(&S.bar, 3u * FB * FB * 4u + (RHEO && rheo ? 3u * rb : 0u));
      tma_load_2d(S.h, F.tmap + MAP_H, i0 - 4, j0 - 4, &S.bar);
      tma_load_2d(S.m, F.tmap + MAP_M, i0 - 4, j0 - 4, &S.bar);
      tma_load_2d(S.dl, F.tmap + MAP_DELTA, i0 - 4, j0 - 4, &S.bar);
      if constexpr (RHEO) {
        if (rheo) {
          const int rx = B16 ? i0 - 8 : i0 - 4;
          tma_load_2d(S.rh[0], F.tmap + MAP_MU, rx, j0 - 4, &S.bar);
          tma_load_2d(S.rh[1], F.tmap + MAP_TAU, rx, j0 - 4, &S.bar);
          tma_load_2d(S.rh[2], F.tmap + MAP_N, rx, j0 - 4, &S.bar);
        }
      }
    }
    return tma_block_wait(F, &S.bar, tid);
  }
  for (int q = tid; q < FB * FB; q += NT) {
    const int x = i0 - 4 + q % FB, y = j0 - 4 + q / FB;
    const bool in = in_grid(F, x, y);
    const uint32_t c = in ? idx(F, x, y) : 0u;
    S.h[q] = in ? F.hh[c] : 0.f;
    S.m[q] = in ? F.m[c] : 0.f;
    S.dl[q] = in ? F.delta[c] : 0u;
  }
  if constexpr (RHEO) {
    if (rheo) {
      if constexpr (B16) {
        for (int q = tid; q < 32 * FB; q += NT) {
          const int x = i0 - 8 + q % 32, y = j0 - 4 + q / 32;
          const bool in = in_grid(F, x, y);
          const uint32_t c = in ? idx(F, x, y) : 0u;
          const uint16_t* pl[3] = {(const uint16_t*)F.mu, (const uint16_t*)F.tau, (const uint16_t*)F.nn};
#pragma unroll
          for (int r = 0; r < 3; ++r) reinterpret_cast<uint16_t*>(S.rh[r])[q] = in ? pl[r][c] : (uint16_t)0;
        }
      } else {
        for (int q = tid; q < FB * FB; q += NT) {
          const int x = i0 - 4 + q % FB, y = j0 - 4 + q / FB;
          const bool in = in_grid(F, x, y);
          const uint32_t c = in ? idx(F, x, y) : 0u;
          const float* pl[3] = {(const float*)F.mu, (const float*)F.tau, (const float*)F.nn};
#pragma unroll
          for (int r = 0; r < 3; ++r) S.rh[r][q] = in ? __float_as_uint(pl[r][c]) : 0u;
        }
      }
    }
  }
  __syncthreads();
  return true;
}
// Surface levels (film.wgsl:147-151) of the tile + 2 rings, reflected at the
// grid's edges as the laplacian reads them.
template <class Smem, int NT = 256>
__device__ __forceinline__ void tile_surface(const Film& F, const cf_params& P, Smem& S, int i0, int j0, int tid) {
  for (int q = tid; q < 20 * 20; q += NT) {
    const int b = (refl_j(F, j0 - 2 + q / 20) - j0 + 4) * FB + (refl_i(F, i0 - 2 + q % 20) - i0 + 4);
    const float hv = S.h[b];
    int ox, oy;
    unpack_off(S.dl[b], ox, oy);
    S.su[q] = S.h[b] + S.m[b] - (hv > 0.f ? hold_level(P, off_len(ox, oy)) : 0.f);
  }
}
// The laplacian's pressure (film.wgsl:16-42) of cell (x, y) at (px, py) of the
// tile's 18 x 18 box, from the surface levels in shared memory.
template <class Smem>
__device__ __forceinline__ float2 tile_pres(const Film& F, const cf_params& P, const Smem& S, int i0, int j0, int px,
                                            int py, int x, int y, uint32_t c) {
  const int b = (y - j0 + 4) * FB + (x - i0 + 4);
  const float hv = S.h[b];
  const float* u = &S.su[(py + 1) * 20 + px + 1];
  const float u0 = u[0];
  float pl = 0.f;
  const float ax = u[-1] + u[1] + u[-20] + u[20];
  const float dg = u[-21] + u[-19] + u[19] + u[21];
  const float l = (W_AXIS * ax + W_DIAG_LAP * dg - (4.0f * W_AXIS + 4.0f * W_DIAG_LAP) * u0) * P.inv_dx * P.inv_dx;
  if (hv > 0.f) {
    int ox, oy;
    unpack_off(S.dl[b], ox, oy);
    const float d = off_len(ox, oy);
    if (d <= 3.0f) {
      const float2 n = F.fnorm[c];
      if (n.x * n.x + n.y * n.y > 0.5f) pl = line_pressure(F, P, x, y) * expf(-(d - 1.0f) * 0.7f);
    }
  }
  return make_float2(-P.phys[1] * l + disjoining(P, hv), P.phys[0] * P.g[2] * u0 + pl);
}
// film.wgsl:16-42; with CLEAR the kernel also does clear_acc (film.wgsl:1427-1434)
// for its cell, which the reference dispatches just before the first laplacian.
// The tile's box of h, m and the front offsets is staged as the flow tile
// stages it (tensor loads, a 4-cell halo), the surface levels of the tile + 2
// rings are evaluated once into shared memory (one exp each instead of 9 per
// cell), and each cell's pressure is the flow tile's expression over them,
// the 9-point sum in the reference's order.
struct LapSmem {
  float h[FB * FB];                    // box origin (i0 - 4, j0 - 4)
  float m[FB * FB];
  uint32_t dl[FB * FB];
  float su[20 * 20];                   // surface levels, origin (i0 - 2, j0 - 2)
  uint64_t bar;
};
template <bool CLEAR>
__device__ __forceinline__ void laplacian_tile(const Film& F, TileId T) {
  // 128 threads per tile, 2 cells each (rows y and y + 8): twice the tiles
  // of 256-thread blocks in flight on an SM, to hide the staging's latency
  __shared__ __align__(128) LapSmem S;
  if ((F.tile_flags[T.x + T.y * F.tw] & ACTIVE) == 0u) return;
  const cf_params& P = F.P->p;
  const int tid = threadIdx.y * 16 + threadIdx.x;
  const int i0 = (int)T.x * 16, j0 = (int)T.y * 16;
  if (!stage_box<CF_PREC_FP32, false, LapSmem, 128>(F, S, i0, j0, tid)) return;
  tile_surface<LapSmem, 128>(F, P, S, i0, j0, tid);
  __syncthreads();
#pragma unroll
  for (int r = 0; r < 2; ++r) {
    const int ty = (int)threadIdx.y + 8 * r;
    const int i = i0 + (int)threadIdx.x, j = j0 + ty;
    if (i >= (int)F.w || j >= (int)F.h) continue;
    const uint32_t c = idx(F, i, j);
    if (CLEAR) {
      F.acc[c] = make_float4(0.f, 0.f, 0.f, 0.f);
      F.h_frame[c] = S.h[(ty + 4) * FB + threadIdx.x + 4];
    }
    F.pres[c] = tile_pres(F, P, S, i0, j0, (int)threadIdx.x + 1, ty + 1, i, j, c);
  }
}

// Boxes of two 4-byte planes (24 x 24 cells from (i0 - 4, j0 - 4), zero
// outside the grid) into shared memory, as stage_box does: tensor loads
// where the film has descriptors, else loads by the block's threads.
// Returns false (counted in the film's stats) when the tensor loads did not
// arrive within the wait limit.
template <int NT = 256>
__device__ __forceinline__ bool stage_pair(const Film& F, uint64_t* bar, int i0, int j0, int tid, uint32_t* da,
                                           int ma, const uint32_t* sa, uint32_t* db, int mb, const uint32_t* sb) {
  if (F.tmap != nullptr) {
    tma_block_arm(bar, tid);
    if (tid == 0) {
      mbar_arrive_expect_tx(bar, 2u * FB * FB * 4u);
      tma_load_2d(da, F.tmap + ma, i0 - 4, j0 - 4, bar);
      tma_load_2d(db, F.tmap + mb, i0 - 4, j0 - 4, bar);
    }
    return tma_block_wait(F, bar, tid);
  }
  for (int q = tid; q < FB * FB; q += NT) {
    const int x = i0 - 4 + q % FB, y = j0 - 4 + q / FB;
    const bool in = in_grid(F, x, y);
    const uint32_t c = in ? idx(F, x, y) : 0u;
    da[q] = in ? sa[c] : 0u;
    db[q] = in ? sb[c] : 0u;
  }
  __syncthreads();
  return true;
}

// film.wgsl:680-723, reading delta_old (Jacobi).  The tile's box of h and
// delta_old (4-cell halo) is staged in shared memory; the 3 x 3 scan and the
// front normal's 5 x 5 neighbourhood read it there, and a candidate's target
// cell outside the box reads the plane.  With NEXT (the frame) the heights
// are the ones the fused limiter + apply left in h_next, and each cell's is
// committed to h here; without it (the single dispatch) they are h.
struct NoseSmem {
  float h[FB * FB];                    // box origin (i0 - 4, j0 - 4)
  uint32_t dl[FB * FB];                // delta_old
  uint64_t bar;
};
template <bool NEXT>
__device__ __forceinline__ void nose_cell(const Film& F, const cf_params& P, const NoseSmem& S, const float* hs, int i0,
                                          int j0, int i, int j) {
  const uint32_t c = idx(F, i, j);
  auto at = [&](int x, int y) { return (y - j0 + 4) * FB + (x - i0 + 4); };
  if (NEXT) F.hh[c] = S.h[at(i, j)];
  if (S.h[at(i, j)] <= 0.f) {
    F.delta[c] = 0u;
    F.fnorm[c] = make_float2(0.f, 0.f);
    return;
  }
  int bx = 64, by = 64;
  float bd = 1e9f;
#pragma unroll
  for (int dj = -1; dj <= 1; ++dj)
#pragma unroll
    for (int di = -1; di <= 1; ++di) {
      int x = i + di, y = j + dj;
      if (!in_grid(F, x, y)) continue;
      int cx = di, cy = dj;
      if (S.h[at(x, y)] > 0.f) {
        uint32_t dn = S.dl[at(x, y)];
        if ((dn & 0x10000u) == 0u) continue;
        int ox, oy;
        unpack_off(dn, ox, oy);
        cx = ox + di;
        cy = oy + dj;
        int tx = i + cx, ty = j + cy;
        if (!in_grid(F, tx, ty)) continue;
        const bool boxed = tx >= i0 - 4 && tx < i0 + 20 && ty >= j0 - 4 && ty < j0 + 20;
        if ((boxed ? S.h[at(tx, ty)] : hs[idx(F, tx, ty)]) > 0.f) continue;
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
  F.fnorm[c] = bd <= 3.0f ? front_normal_at(F, P, i, j, [&](int x, int y) { return S.h[at(x, y)]; })
                          : make_float2(0.f, 0.f);
}
template <bool NEXT>
__device__ __forceinline__ void nose_tile(const Film& F, TileId T) {
  // 128 threads per tile, 2 cells each (rows y and y + 8), as the laplacian
  __shared__ __align__(128) NoseSmem S;
  if ((F.tile_flags[T.x + T.y * F.tw] & ACTIVE) == 0u) return;
  const cf_params& P = F.P->p;
  const int tid = threadIdx.y * 16 + threadIdx.x;
  const int i0 = (int)T.x * 16, j0 = (int)T.y * 16;
  const float* hs = NEXT ? F.h_next : F.hh;
  if (!stage_pair<128>(F, &S.bar, i0, j0, tid, reinterpret_cast<uint32_t*>(S.h), NEXT ? MAP_H_NEXT : MAP_H,
                       reinterpret_cast<const uint32_t*>(hs), S.dl, MAP_DELTA_OLD, F.delta_old))
    return;
#pragma unroll
  for (int r = 0; r < 2; ++r) {
    const int i = i0 + (int)threadIdx.x, j = j0 + (int)threadIdx.y + 8 * r;
    if (i < (int)F.w && j < (int)F.h) nose_cell<NEXT>(F, P, S, hs, i0, j0, i, j);
  }
}

// ---- limiter + apply, fused ----
// film.wgsl:516-537 (limiter) and 539-561, 803-863 (apply) for one tile.
// Only apply reads the limiter's alpha, so it stays in shared memory: the
// block stages the flux of the tile + 2 rings and h with a 4-cell halo
// (tensor loads), evaluates alpha on the tile + 1 ring (the expression of
// limiter_tile), then applies the tile's own cells (apply_tile's, from
// shared memory).  A ring cell's alpha needs its height before apply, which
// the neighbouring tile's block may already have replaced; so the new heights
// go to h_next, and the nose (NEXT), which runs next and reads them there,
// commits them to h.  Every tile, active or not, snapshots delta into
// delta_old for the nose, and an inactive tile copies h to h_next, so that
// the nose finds every cell's height there.
struct LaSmem {
  float4 fx[20 * 20];                  // flux, origin (i0 - 2, j0 - 2)
  float h[FB * FB];                    // h, origin (i0 - 4, j0 - 4)
  float al[18 * 18];                   // alpha, origin (i0 - 1, j0 - 1)
  uint32_t act[9];                     // ACTIVE of the 3 x 3 tiles around this one
  uint64_t bar;
};
// apply (film.wgsl:539-561, 803-863) of cell (i, j) = (i0 + tx, j0 + ty)
// from the block's shared memory; returns whether its height moved
template <int MODE>
__device__ __forceinline__ bool apply_cell(const Film& F, const cf_params& P, const LaSmem& S, TileId T, int tx, int ty,
                                           float4 a4) {
  const int i = (int)T.x * 16 + tx, j = (int)T.y * 16 + ty;
  const uint32_t c = idx(F, i, j);
  auto live = [&](int x, int y) {
    return in_grid(F, x, y) && S.act[((y >> 4) - (int)T.y + 1) * 3 + ((x >> 4) - (int)T.x + 1)] != 0u;
  };
  const int a0 = (ty + 1) * 18 + tx + 1;  // the cell in al
  const int f0 = (ty + 2) * 20 + tx + 2;  // and in fx
  const bool hx = i + 1 < (int)F.w, hy = j + 1 < (int)F.h, hm = j > 0, hl = i > 0;
  const bool has[4] = {hx, hy, hx && hy, hx && hm};
  const uint32_t cbs[4] = {c + 1, c + F.w, c + F.w + 1, c - F.w + 1};
  const int abx[4] = {a0 + 1, a0 + 18, a0 + 19, a0 - 17};
  const float ac = S.al[a0];
  const float4 f4 = S.fx[f0];
  const float f[4] = {f4.x, f4.y, f4.z, f4.w};
  float best = 0.f, div = 0.f;
  uint32_t src = c;
  float accv[4];
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    float q = f[k], ab = ac;
    if (q < 0.f && has[k]) {
      ab = S.al[abx[k]];
      if (-q * ab > best) { best = -q * ab; src = cbs[k]; }
    }
    div += q * ab;
    accv[k] = q * ab;
  }
  auto nb_face = [&](float q, float an, uint32_t cn) {
    if (q < 0.f) an = ac;
    if (q * an > best) { best = q * an; src = cn; }
    div -= q * an;
  };
  if (hl && live(i - 1, j)) nb_face(S.fx[f0 - 1].x, S.al[a0 - 1], c - 1);
  if (hm && live(i, j - 1)) nb_face(S.fx[f0 - 20].y, S.al[a0 - 18], c - F.w);
  if (hl && hm && live(i - 1, j - 1)) nb_face(S.fx[f0 - 21].z, S.al[a0 - 19], c - F.w - 1);
  if (hl && hy && live(i - 1, j + 1)) nb_face(S.fx[f0 + 19].w, S.al[a0 + 17], c + F.w - 1);
  const float h0 = S.h[(ty + 4) * FB + tx + 4];
  float hn = fmaxf(h0 - P.dt * div * P.inv_dx, 0.f);
  if (hn < h0 && hn < DRAINED_FILM) hn = 0.f;
  F.h_next[c] = hn;
  if (h0 <= 0.f && src != c) {
    set_rheo<MODE>(F, c, rmu<MODE>(F, src), rtau<MODE>(F, src), rn<MODE>(F, src));
    backfill<MODE>(F, c, src, hn);
  }
  F.acc[c] = make_float4(a4.x + accv[0] * P.dt, a4.y + accv[1] * P.dt, a4.z + accv[2] * P.dt, a4.w + accv[3] * P.dt);
  return fabsf(hn - h0) > MOVE_EPS;
}
template <int MODE>
__device__ __forceinline__ void limit_apply_tile(const Film& F, TileId T) {
  // 128 threads per tile, 2 cells each (rows y and y + 8)
  __shared__ __align__(128) LaSmem S;
  const int tid = threadIdx.y * 16 + threadIdx.x;
  const int i0 = (int)T.x * 16, j0 = (int)T.y * 16;
  const int i = i0 + (int)threadIdx.x;
  bool in[2];
  uint32_t c[2];
#pragma unroll
  for (int r = 0; r < 2; ++r) {
    const int j = j0 + (int)threadIdx.y + 8 * r;
    in[r] = i < (int)F.w && j < (int)F.h;
    c[r] = in[r] ? idx(F, i, j) : 0u;
  }
  if ((F.tile_flags[T.x + T.y * F.tw] & ACTIVE) == 0u) {
#pragma unroll
    for (int r = 0; r < 2; ++r)
      if (in[r]) {
        F.delta_old[c[r]] = F.delta[c[r]];
        F.h_next[c[r]] = F.hh[c[r]];
      }
    return;
  }
  const cf_params& P = F.P->p;
  // the tensor loads first (the flux as floats, 4 a cell), then the block's
  // own loads while they are in flight
  const bool tma = F.tmap != nullptr;
  if (tma) {
    tma_block_arm(&S.bar, tid);
    if (tid == 0) {
      mbar_arrive_expect_tx(&S.bar, 20u * 20u * 16u + FB * FB * 4u);
      tma_load_2d(S.fx, F.tmap + MAP_FLUX, 4 * (i0 - 2), j0 - 2, &S.bar);
      tma_load_2d(S.h, F.tmap + MAP_H, i0 - 4, j0 - 4, &S.bar);
    }
  }
  // both cells' loads before either store
  float4 a4[2];
  float dl[2];
#pragma unroll
  for (int r = 0; r < 2; ++r) {
    a4[r] = in[r] ? F.acc[c[r]] : make_float4(0.f, 0.f, 0.f, 0.f);
    dl[r] = in[r] ? F.delta[c[r]] : 0.f;
  }
#pragma unroll
  for (int r = 0; r < 2; ++r)
    if (in[r]) F.delta_old[c[r]] = dl[r];
  if (tid < 9) {
    const int tx = (int)T.x + tid % 3 - 1, ty = (int)T.y + tid / 3 - 1;
    S.act[tid] = tx >= 0 && ty >= 0 && tx < (int)F.tw && ty < (int)F.th ? F.tile_flags[tx + ty * F.tw] & ACTIVE : 0u;
  }
  if (tma) {
    if (!tma_block_wait(F, &S.bar, tid)) return;
  } else {
    for (int q = tid; q < 20 * 20; q += 128) {
      const int x = i0 - 2 + q % 20, y = j0 - 2 + q / 20;
      S.fx[q] = in_grid(F, x, y) ? F.flux[idx(F, x, y)] : make_float4(0.f, 0.f, 0.f, 0.f);
    }
    for (int q = tid; q < FB * FB; q += 128) {
      const int x = i0 - 4 + q % FB, y = j0 - 4 + q / FB;
      S.h[q] = in_grid(F, x, y) ? F.hh[idx(F, x, y)] : 0.f;
    }
    __syncthreads();
  }
  // cell_active for cells within 2 of the tile: in the grid and in an active tile
  auto live = [&](int x, int y) {
    return in_grid(F, x, y) && S.act[((y >> 4) - (int)T.y + 1) * 3 + ((x >> 4) - (int)T.x + 1)] != 0u;
  };
  // limiter (film.wgsl:516-537) on the tile + 1 ring
  for (int q = tid; q < 18 * 18; q += 128) {
    const int px = q % 18, py = q / 18, x = i0 - 1 + px, y = j0 - 1 + py;
    float a = 1.f;  // cells outside the grid or in inactive tiles: apply reads no alpha of them
    if (live(x, y)) {
      const float4* f = &S.fx[(py + 1) * 20 + px + 1];
      float out = fmaxf(f[0].x, 0.f) + fmaxf(f[0].y, 0.f) + fmaxf(f[0].z, 0.f) + fmaxf(f[0].w, 0.f);
      if (x > 0 && live(x - 1, y)) out += fmaxf(-f[-1].x, 0.f);
      if (y > 0 && live(x, y - 1)) out += fmaxf(-f[-20].y, 0.f);
      if (x > 0 && y > 0 && live(x - 1, y - 1)) out += fmaxf(-f[-21].z, 0.f);
      if (x > 0 && y + 1 < (int)F.h && live(x - 1, y + 1)) out += fmaxf(-f[19].w, 0.f);
      if (out > 0.f) a = fminf(1.f, 0.5f * S.h[(py + 3) * FB + px + 3] * P.dx / (P.dt * out));
    }
    S.al[q] = a;
  }
  __syncthreads();
  bool moved = false;
#pragma unroll
  for (int r = 0; r < 2; ++r)
    if (in[r]) moved = apply_cell<MODE>(F, P, S, T, (int)threadIdx.x, (int)threadIdx.y + 8 * r, a4[r]) || moved;
  if (__syncthreads_or(moved) && tid == 0) F.tile_moved[T.x + T.y * F.tw] = 1u;
}

template <int MODE, bool CLEAR>
__device__ __forceinline__ void flow_tile(const Film& F, TileId T) {
  __shared__ __align__(128) FlowSmem S;
  if ((F.tile_flags[T.x + T.y * F.tw] & ACTIVE) == 0u) return;
  const DevParams& D = *F.P;
  const cf_params& P = D.p;
  const int tid = threadIdx.y * 16 + threadIdx.x;
  const int i0 = (int)T.x * 16, j0 = (int)T.y * 16;
  // the rheology is read from shared memory only by the plug window, which a
  // flat canvas (gb < 1e-6) skips
  const float gb = P.phys[0] * D.gxy;
  if (!stage_box<MODE, true>(F, S, i0, j0, tid, gb >= 1e-6f)) return;
  auto box = [&](int x, int y) { return (y - j0 + 4) * FB + (x - i0 + 4); };
  {
    // a tile whose cells and 1-cell ring are all dry has no face with flux
    // (every face needs a wet cell) and no plug mobility (only wet cells have
    // one): its cells take zero flux and mobility, and clear_acc
    bool wet = false;
    for (int q = tid; q < 18 * 18; q += 256) wet = wet || S.h[(q / 18 + 3) * FB + q % 18 + 3] > 0.f;
    if (!__syncthreads_or(wet)) {
      const int i = i0 + (int)threadIdx.x, j = j0 + (int)threadIdx.y;
      if (i < (int)F.w && j < (int)F.h) {
        const uint32_t c = idx(F, i, j);
        if (CLEAR) {
          F.acc[c] = make_float4(0.f, 0.f, 0.f, 0.f);
          F.h_frame[c] = S.h[box(i, j)];
        }
        F.tmp[c] = 0.f;
        F.flux[c] = make_float4(0.f, 0.f, 0.f, 0.f);
      }
      return;
    }
  }
  tile_surface(F, P, S, i0, j0, tid);
  // plug: the HB flux and mass of every window cell (film.wgsl:58-87); on a
  // flat canvas (gb < 1e-6) every plug mobility is 0 and none is needed
  if (gb >= 1e-6f) {
    for (int q = tid; q < FB * FB; q += 256) {
      const int x = i0 - 4 + q % FB, y = j0 - 4 + q / FB;
      float qq = 0.f, mass = 0.f;
      uint8_t yl = 0;
      const float hn = S.h[q];
      if (in_grid(F, x, y) && hn > 0.f) {
        const float rx = staged_rh<MODE>(S, 0, q), ry = staged_rh<MODE>(S, 1, q);
        yl = (uint8_t)(1u | (ry > 0.f ? 2u : 0u));
        float yy, up;
        hb_flux(gb, hn, fmaxf(rx, 1e-4f), ry, staged_rh<MODE>(S, 2, q), qq, yy, up);
        mass = hn;
      }
      S.qm[q] = make_float2(qq, mass);
      S.yl[q] = yl;
    }
  }
  if (tid < 4) S.faces.count[tid] = 0u;
  __syncthreads();
  // pressures (film.wgsl:16-42) and plug mobilities of the tile + 1 ring;
  // ring cells in inactive tiles keep the planes' values
  for (int q = tid; q < 18 * 18; q += 256) {
    const int px = q % 18, py = q / 18, x = i0 - 1 + px, y = j0 - 1 + py;
    if (!in_grid(F, x, y)) {
      // the height of the cell it reflects to (every such cell the faces
      // read lies in the staged box)
      const int rx = refl_i(F, x) - i0 + 4, ry = refl_j(F, y) - j0 + 4;
      S.hr[q] = rx >= 0 && rx < FB && ry >= 0 && ry < FB ? S.h[ry * FB + rx] : 0.f;
      continue;
    }
    S.hr[q] = S.h[box(x, y)];
    const uint32_t c = idx(F, x, y);
    if (!cell_active(F, x, y)) {
      S.pres[q] = F.pres[c];
      S.tmp[q] = F.tmp[c];
      continue;
    }
    S.pres[q] = tile_pres(F, P, S, i0, j0, px, py, x, y, c);
    const float hv = S.h[box(x, y)];
    float t = 0.f;
    if (hv > 0.f && gb >= 1e-6f) {
      float sum = 0.f, mass = 0.f;
      uint32_t fl = 0u;
      for (int dy = 0; dy < 7; ++dy)
#pragma unroll
        for (int dx = 0; dx < 7; ++dx) {
          const int w = (py + dy) * FB + px + dx;
          const float2 v = S.qm[w];
          fl |= S.yl[w];
          sum += v.x;
          mass += v.y;
        }
      if ((fl & 2u) && mass > 0.f) t = sum / mass;
    }
    S.tmp[q] = t;
  }
  __syncthreads();
  // the tile's own cells: clear_acc (film.wgsl:1427-1434) with the first
  // substep, the plug mobility to the plane, the flux zeroed, the live faces
  // listed by direction
  const int i = i0 + (int)threadIdx.x, j = j0 + (int)threadIdx.y;
  const bool in = i < (int)F.w && j < (int)F.h;
  const uint32_t c = in ? idx(F, i, j) : 0u;
  const float hc = in ? S.h[box(i, j)] : 0.f;
  if (in) {
    if (CLEAR) {
      F.acc[c] = make_float4(0.f, 0.f, 0.f, 0.f);
      F.h_frame[c] = hc;
    }
    F.tmp[c] = S.tmp[(threadIdx.y + 1) * 18 + threadIdx.x + 1];
    F.flux[c] = make_float4(0.f, 0.f, 0.f, 0.f);
  }
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    const int x = i + FACE_DI[k], y = j + FACE_DJ[k];
    tile_faces_add(S.faces, k, in && in_grid(F, x, y) && cell_active(F, x, y) && 0.5f * (hc + S.h[box(x, y)]) > 0.f);
  }
  // on the grid's edges: the ring positions outside the grid take the
  // pressure of the cell they reflect to
  if (i0 == 0 || j0 == 0 || i0 + 17 > (int)F.w || j0 + 17 > (int)F.h) {
    for (int q = tid; q < 18 * 18; q += 256) {
      const int x = i0 - 1 + q % 18, y = j0 - 1 + q / 18;
      if (in_grid(F, x, y)) continue;
      const int rx = refl_i(F, x) - i0 + 1, ry = refl_j(F, y) - j0 + 1;
      if (rx >= 0 && rx < 18 && ry >= 0 && ry < 18) S.pres[q] = S.pres[ry * 18 + rx];
    }
  }
  __syncthreads();
  const PtTile pt{S.pres, S.tmp, S.hr, i0, j0};
  float* fl = reinterpret_cast<float*>(F.flux);
  tile_faces_each(F, T, S.faces, [&](int k, int fi, int fj, uint32_t fc) {
    fl[4 * (size_t)fc + k] = face_k<MODE>(F, D, pt, fi, fj, k).q;
  });
}

// strata_split (film.wgsl:475-514) for one tile: every face with a frame
// flux is recomputed and its flux split over the upstream cell's strata; the
// face flags (bit f: face f's split is nonzero) are gathered in shared memory.
// The reference zeroes acc_s first; here the faces not written keep stale
// values, and every reader takes a face only where its flag is set
// (acc_face_live), which reads the same values without the 64 B per cell of
// zeroing.
template <int MODE>
__device__ __forceinline__ void strata_split_tile(const Film& F, TileId T) {
  // 128 threads per tile, 2 cells each (slots t and t + 128: rows y and y + 8)
  __shared__ TileFaces S;
  __shared__ uint32_t flags[256];
  if ((F.tile_flags[T.x + T.y * F.tw] & ACTIVE) == 0u) return;
  const int tid = threadIdx.y * 16 + threadIdx.x;
  const int i = (int)(T.x * 16 + threadIdx.x);
  if (tid < 4) S.count[tid] = 0u;
  flags[tid] = 0u;
  flags[tid + 128] = 0u;
  __syncthreads();
  bool in[2];
  uint32_t c[2];
  float4 a4[2];
#pragma unroll
  for (int r = 0; r < 2; ++r) {
    const int j = (int)(T.y * 16 + threadIdx.y + 8 * r);
    in[r] = i < (int)F.w && j < (int)F.h;
    c[r] = in[r] ? idx(F, i, j) : 0u;
    a4[r] = in[r] ? F.acc[c[r]] : make_float4(0.f, 0.f, 0.f, 0.f);
  }
#pragma unroll
  for (int r = 0; r < 2; ++r) {
    const int j = (int)(T.y * 16 + threadIdx.y + 8 * r);
#pragma unroll
    for (int k = 0; k < 4; ++k)
      tile_faces_add(S, k, in[r] && sel4(a4[r], k) != 0.f && in_grid(F, i + FACE_DI[k], j + FACE_DJ[k]), tid + 128 * r);
  }
  __syncthreads();
  const DevParams& D = *F.P;
  tile_faces_each<128>(F, T, S, [&](int k, int fi, int fj, uint32_t fc) {
    const float a = sel4(F.acc[fc], k);
    const FaceOut ff = face_k<MODE>(F, D, PtGlobal{F}, fi, fj, k);
    const uint32_t cb = idx(F, fi + FACE_DI[k], fj + FACE_DJ[k]);
    const uint32_t cu = a < 0.f ? cb : fc;
    const float4 o = band_split(F, cu, 0.5f * (F.hh[fc] + F.hh[cb]), ff.y, ff.up, a, ff.n);
    F.acc_s[(size_t)k * F.n + fc] = o;
    if (o.x != 0.f || o.y != 0.f || o.z != 0.f || o.w != 0.f)
      atomicOr(&flags[(fj - (int)T.y * 16) * 16 + (fi - (int)T.x * 16)], 1u << k);
  });
  __syncthreads();
#pragma unroll
  for (int r = 0; r < 2; ++r)
    if (in[r]) F.fflags[c[r]] = flags[tid + 128 * r];
}

__device__ __forceinline__ void load_tables(const Film& F, float* tab, float* cm, float* ltab, int tid, int nthreads) {
  for (int q = tid; q < 480; q += nthreads) tab[q] = F.pigtab[q];
  if (tid < 48) cm[tid] = F.cmf[tid];
  if (tid < 12) ltab[tid] = logf(fmaxf(F.pigtab[tid * 40 + 32], 1e-3f));
}

// A warp of the strata fast path shades its cells lane by lane when at least
// this many of its lanes have one (see strata_fast_cell).
constexpr int FAST_SHADE_LANES = 20;
// Shared memory of a strata fast-path block: the tables, and the tile's cells
// to shade with the thicknesses, cure fractions and h the fast path gave them.
struct FastShade {
  alignas(16) float kst[16 * 24];  // band-major K, S (layer_ks_band_t)
  float tab[480];
  float cm[48];
  float ltab[12];
  float4 nt[256], cu[256];
  float h[256];
  uint32_t list[256];
  uint32_t count;
  alignas(16) float xs[8][32];  // per half-warp scratch of the lane shade
};

// Strata pass, part 1, over every cell.  Active cells with a strata flux on a
// face or a stack that is not compact are listed for part 2, with their
// strata_limit alpha (strata.wgsl:157-173; 1 without fluxes).  Every other
// cell takes the fast path of strata_update (strata.wgsl:212-237): the stack
// renormalised to h into the next generation of thicknesses, its pigments left
// in place (this path never changes them).  Inactive tiles carry their strata
// over and are shaded, as the reference's full-grid shade does.  Active wet
// cells left without strata become strata_fill candidates.  Returns what the
// cell's shade (shade.wgsl:28-84) needs, with its inputs left in the block's
// FastShade slot: FAST_NOTHING (a dry cell whose colour is current, or a cell
// of the full path), FAST_SHADE (the composite spectrum, the composition
// aggregates and the colour: the tile function shades it by lane or by
// half-warp) or FAST_COLOR (a wet cell whose thicknesses came out bit for bit
// the ones its cached spectrum was composited for: only the surface
// correction, which follows the cure).
constexpr int FAST_NOTHING = 0, FAST_SHADE = 1, FAST_COLOR = 2;
template <int MODE>
__device__ __forceinline__ int strata_fast_cell(const Film& F, const cf_params& P, TileId T, int i, int j,
                                                uint32_t c, float hc, FastShade& sh, int tid) {
  const bool act = (F.tile_flags[T.x + T.y * F.tw] & ACTIVE) != 0u;
  // The cell's loads are issued together: strata, dry flag and, in an active
  // tile, the face flags of the cell and of the 4 neighbours whose faces
  // touch it (their activity tested after).  ft: whether any of the 8 faces
  // carries a strata flux (the face flags of strata_split); only then is the
  // strata_limit alpha below 1 and does strata_update move material into or
  // out of the cell.
  const uint8_t state = F.shade_state[c];
  // a cell whose cached spectrum may be reused: its 64 bytes are fetched
  // towards L2 while the strata and face flags load
  if (state == SHADE_WET) {
#pragma unroll
    for (int q = 0; q < 4; ++q) asm volatile("prefetch.L2 [%0];" ::"l"(F.spec + (size_t)q * F.n + c));
  }
  // a cell dry two passes running in an active tile holds zeros in both
  // generations: unless a strata flux reaches it below, nothing to do
  const bool dry2 = act && hc <= 0.f && state == SHADE_DRY2;
  const float4 z4 = make_float4(0.f, 0.f, 0.f, 0.f);
  float4 t4 = dry2 ? z4 : F.sh[c], cu = dry2 ? z4 : F.scu[c];
  if (act) {
    const bool hl = i > 0, hd = j > 0, hu = j + 1 < (int)F.h;
    const uint32_t f0 = F.fflags[c], fl = hl ? F.fflags[c - 1] : 0u, fd = hd ? F.fflags[c - F.w] : 0u,
                   fdl = (hl && hd) ? F.fflags[c - F.w - 1] : 0u, ful = (hl && hu) ? F.fflags[c + F.w - 1] : 0u;
    const bool ft = f0 != 0u || ((fl & 1u) && cell_active(F, i - 1, j)) || ((fd & 2u) && cell_active(F, i, j - 1)) ||
                    ((fdl & 4u) && cell_active(F, i - 1, j - 1)) || ((ful & 8u) && cell_active(F, i - 1, j + 1));
    if (ft || not_compact(P, hc, t4)) {
      F.alpha_s[c] = ft ? strata_limit_at(F, P, i, j) : make_float4(1.f, 1.f, 1.f, 1.f);
      // The full path reads the cell's 4 faces and the 4 its active left,
      // lower, lower-left and upper-left neighbours own, unmasked: those
      // strata_split did not write this frame are zeroed here (a face is
      // zeroed by at most its two cells, both writing zero, and read under
      // its flag only until the full path).
#pragma unroll
      for (int k = 0; k < 4; ++k)
        if (!((f0 >> k) & 1u)) F.acc_s[(size_t)k * F.n + c] = z4;
      if (hl && !(fl & 1u) && cell_active(F, i - 1, j)) F.acc_s[c - 1] = z4;
      if (hd && !(fd & 2u) && cell_active(F, i, j - 1)) F.acc_s[F.n + c - F.w] = z4;
      if (hl && hd && !(fdl & 4u) && cell_active(F, i - 1, j - 1)) F.acc_s[2 * (size_t)F.n + c - F.w - 1] = z4;
      if (hl && hu && !(ful & 8u) && cell_active(F, i - 1, j + 1)) F.acc_s[3 * (size_t)F.n + c + F.w - 1] = z4;
      list_append(F.full_list, &F.stats->full_count, c);
      return FAST_NOTHING;
    }
    if (dry2) return FAST_NOTHING;
  }
  float nt[4] = {t4.x, t4.y, t4.z, t4.w};
  if (act) {
    float th[4] = {fmaxf(t4.x, 0.f), fmaxf(t4.y, 0.f), fmaxf(t4.z, 0.f), fmaxf(t4.w, 0.f)};
    if (hc <= 0.f) {
      cu = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
      for (int k = 0; k < 4; ++k) nt[k] = 0.f;
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
    if (hc > 0.f && !(nt[0] + nt[1] + nt[2] + nt[3] > 0.f)) list_append(F.fill_list, &F.stats->fill_count, c);
  }
  F.sh2[c] = make_float4(nt[0], nt[1], nt[2], nt[3]);
  F.scu2[c] = cu;
  // A dry cell's colour depends on its substrate reflectance, its relief and
  // the CMF table only (the stack and the params enter wet cells' colour),
  // and those do not change while it stays dry: when the last shade already
  // saw it dry, its colour is current.  A wet cell's composite spectrum
  // depends on its thicknesses, pigments and substrate: while the state says
  // the cached one is current for the thicknesses it entered with, and it
  // leaves with the same ones, the spectrum is reused (not in the invariant
  // debug view, which reads the pigments).
  sh.nt[tid] = make_float4(nt[0], nt[1], nt[2], nt[3]);
  sh.cu[tid] = cu;
  sh.h[tid] = hc;
  if (hc <= 0.f) {
    // zeros now in both generations when this pass wrote zeros and the
    // current one held zeros
    const bool zeros = act && t4.x == 0.f && t4.y == 0.f && t4.z == 0.f && t4.w == 0.f && cu.x == 0.f &&
                       cu.y == 0.f && cu.z == 0.f && cu.w == 0.f;
    const bool shaded = state == SHADE_DRY || state == SHADE_DRY2;
    const uint8_t next = shaded && zeros ? SHADE_DRY2 : SHADE_DRY;
    if (next != state) F.shade_state[c] = next;
    return shaded ? FAST_NOTHING : FAST_SHADE;
  }
  if (state == SHADE_WET && P.flags[0] != 1u && nt[0] == t4.x && nt[1] == t4.y && nt[2] == t4.z && nt[3] == t4.w)
    return FAST_COLOR;
  if (state != SHADE_WET) F.shade_state[c] = SHADE_WET;  // the shade below caches the spectrum
  return FAST_SHADE;
}
// The colour of a FAST_COLOR cell: its cached composite spectrum through the
// surface correction with this frame's cure (bit for bit what CellAcc gives
// for the same strata; the aggregates do not depend on the cure and stay).
template <int MODE>
__device__ __forceinline__ void fast_color_cached(const Film& F, uint32_t c, const FastShade& sh, int tid) {
  const float4 nt = sh.nt[tid], cu = sh.cu[tid];
  float wet = 0.f, cure_top = 0.f;
#pragma unroll
  for (int k = 0; k < 4; ++k)
    if (sel4(nt, k) > 0.f) {
      wet = 1.0f - sel4(cu, k);
      cure_top = sel4(cu, k);
    }
  // every load (m, the detail texel's lay and yield stress, the spectrum)
  // goes out before the first store
  const float mv = F.m[c];
  const ushort4 dt = detail_texel<MODE>(F, c, cure_top, sh.h[tid], mv);
  float r[16];
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    const float4 v = F.spec[(size_t)q * F.n + c];
    r[4 * q] = v.x; r[4 * q + 1] = v.y; r[4 * q + 2] = v.z; r[4 * q + 3] = v.w;
  }
  float rgb[3];
  surface_rgb(sh.cm, r, wet, rgb);
  F.color[c] = pack_color(rgb, surface_rough(cure_top, sh.h[tid], mv));
  F.detail[c] = dt;
}
// The shade and aggregates of one cell the fast path left to shade, by its
// own lane (CellAcc).
template <int MODE>
__device__ __forceinline__ void fast_shade_lane(const Film& F, const cf_params& P, uint32_t c, const FastShade& sh,
                                                int tid) {
  const float4 nt = sh.nt[tid], cu = sh.cu[tid];
  const float hc = sh.h[tid];
  CellAcc acc;
  acc.begin(F.refl + (size_t)c * 16);
  const bool dbg = P.flags[0] == 1u;
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    const float tk = sel4(nt, k);
    if (tk > 0.f) {
      float pg[16];
      PigIO<MODE>::load(F, F.pig, c, k, pg);
      acc.add_t(k, tk, sel4(cu, k), pg, hc, sh.ltab, sh.tab, sh.kst, dbg);
    } else {
      acc.ssum += tk;
    }
  }
  // the next cure reads the aggregates of wet cells only; a wet cell's
  // composite spectrum is cached for the frames its strata stay as they are
  const float mv = F.m[c];
  const ushort4 dt = detail_texel<MODE>(F, c, acc.cure_top, hc, mv);  // its loads before the stores
  if (hc > 0.f) {
    F.agg[c] = acc.agg(P);
#pragma unroll
    for (int q = 0; q < 4; ++q)
      F.spec[(size_t)q * F.n + c] = make_float4(acc.r[4 * q], acc.r[4 * q + 1], acc.r[4 * q + 2], acc.r[4 * q + 3]);
  }
  F.color[c] = acc.color(P, sh.cm, hc, mv);
  F.detail[c] = dt;
}
// The shade (shade.wgsl:28-84) and composition aggregates (cure.wgsl:3-48)
// of the tile's cells that the fast path listed: one cell per half-warp, the
// lanes over pigment slots and bands (strata_lane.cuh, as the full path),
// so a warp shades two cells with all of its lanes instead of one lane per
// wet cell of the tile.
template <int MODE>
__device__ __forceinline__ void fast_shade_cells(const Film& F, const cf_params& P, TileId T, FastShade& sh, int tid) {
  const HalfWarp H(tid & 31);
  const bool dbg = P.flags[0] == 1u;
  const uint32_t n = sh.count;
  for (uint32_t e = (uint32_t)(tid >> 4); e < n; e += 8u) {  // the block's 8 half-warps
    const uint32_t t = sh.list[e];
    const uint32_t c = idx(F, (int)(T.x * 16 + (t & 15u)), (int)(T.y * 16 + (t >> 4)));
    const float hc = sh.h[t];
    const float4 nt = sh.nt[t], cu = sh.cu[t];
    LaneAcc acc;
    acc.begin(H, F.refl + (size_t)c * 16);
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const float tk = sel4(nt, k);
      const float pg = tk > 0.f ? PigLane<MODE>::load(F, F.pig, c, k, H.q) : 0.f;
      acc.add(H, k, tk, sel4(cu, k), pg, hc, sh.ltab, sh.tab, sh.xs[tid >> 4], dbg);
    }
    const float4 agg = acc.agg(P);
    const float mv = F.m[c];
    const ushort4 dt = detail_texel<MODE>(F, c, acc.cure_top, hc, mv);  // its loads before the stores
    const ushort4 col = acc.color(H, P, sh.cm, hc, mv);
    if (hc > 0.f) reinterpret_cast<float*>(F.spec)[((size_t)(H.q >> 2) * F.n + c) * 4 + (H.q & 3)] = acc.r;
    if (H.q == 0) {
      if (hc > 0.f) F.agg[c] = agg;  // the next cure reads the aggregates of wet cells only
      F.color[c] = col;
      F.detail[c] = dt;
    }
  }
}
// ... for one tile, together with the CFL reduction of reduce_tiles
// (film.wgsl:1330-1361; the strata pass changes neither h nor mu, so the
// order-independent max / min equal the reference's).
template <int MODE>
__device__ __forceinline__ void strata_fast_tile(const Film& F, TileId T) {
  // 128 threads per tile, 2 cells each (slots t and t + 128: rows y and y + 8)
  __shared__ FastShade sh;
  __shared__ float red_h[4], red_m[4];
  const int tid = threadIdx.y * 16 + threadIdx.x;
  // the CMF table (all a cached colour needs) is loaded with the cells' own
  // loads; the pigment tables only in blocks that shade a cell
  const float cmv = tid < 48 ? F.cmf[tid] : 0.f;
  if (tid == 0) sh.count = 0u;
  const cf_params& P = F.P->p;
  float hm = 0.f, mm = 1e9f;
  int need[2];
  uint32_t c[2];
#pragma unroll 1
  for (int r = 0; r < 2; ++r) {
    const int t = tid + 128 * r;
    const int i = (int)(T.x * 16 + (t & 15)), j = (int)(T.y * 16 + (t >> 4));
    need[r] = FAST_NOTHING;
    c[r] = 0u;
    if (i < (int)F.w && j < (int)F.h) {
      c[r] = idx(F, i, j);
      const float hc = F.hh[c[r]];
      if (hc > 4.0f * P.ein[3]) { hm = fmaxf(hm, hc); mm = fminf(mm, rmu<MODE>(F, c[r])); }
      need[r] = strata_fast_cell<MODE>(F, P, T, i, j, c[r], hc, sh, t);
    }
  }
  if (tid < 48) sh.cm[tid] = cmv;
  if (__syncthreads_or(need[0] == FAST_SHADE || need[1] == FAST_SHADE)) {
    for (int q = tid; q < 480; q += 128) sh.tab[q] = F.pigtab[q];
    if (tid < 12) sh.ltab[tid] = logf(fmaxf(F.pigtab[tid * 40 + 32], 1e-3f));
    for (int e = tid; e < 16 * 24; e += 128) {
      const int b = e / 24, r = e % 24;
      sh.kst[e] = F.pigtab[(r < 12 ? r : r - 12) * 40 + (r < 12 ? 0 : 16) + b];
    }
    __syncthreads();
  }
#pragma unroll 1
  for (int r = 0; r < 2; ++r) {
    const int t = tid + 128 * r;
    if (need[r] == FAST_COLOR) fast_color_cached<MODE>(F, c[r], sh, t);
    const bool shade = need[r] == FAST_SHADE;
    // Where at least FAST_SHADE_LANES lanes of the warp have a cell to
    // shade, each shades its own; where fewer do, the cells are shaded after
    // the tile's pass by half-warps (fast_shade_cells), which costs about
    // 1/20 of a warp-wide shade per cell.
    const unsigned want = __ballot_sync(0xffffffffu, shade);
    if (shade) {
      if (__popc(want) >= FAST_SHADE_LANES) fast_shade_lane<MODE>(F, P, c[r], sh, t);
      else list_append(sh.list, &sh.count, (uint32_t)t);
    }
  }
  for (int o = 16; o > 0; o >>= 1) {
    hm = fmaxf(hm, __shfl_xor_sync(0xffffffffu, hm, o));
    mm = fminf(mm, __shfl_xor_sync(0xffffffffu, mm, o));
  }
  if ((tid & 31) == 0) { red_h[tid >> 5] = hm; red_m[tid >> 5] = mm; }
  __syncthreads();
  if (tid == 0) {
#pragma unroll
    for (int w = 1; w < 4; ++w) { hm = fmaxf(hm, red_h[w]); mm = fminf(mm, red_m[w]); }
    if (hm > 0.f) fold_cfl(F.stats, hm, mm);
  }
  fast_shade_cells<MODE>(F, P, T, sh, tid);
}

// strata.wgsl:175-188 with one cell per half-warp: the material that
// neighbour cn sends over a face (volumes f, one per stratum; positive =
// towards this cell) scaled by the neighbour's alpha.  The neighbour is read
// only when some stratum flows in, and then it is active with its alpha
// written by part 1 (a nonzero face flags both of its cells), or inactive,
// where strata_limit leaves alpha at 1.
// The gathered neighbourhood of a cell of the full path, one per half-warp:
// the cell's 8 faces (towards the cell positive; zero where absent), the 8
// neighbours' strata thicknesses, cure fractions and strata_limit alphas (1
// for a neighbour in an inactive tile, whose alpha is not applied), and the
// pigment slots of the neighbour strata that flow into the cell, in the
// order strata_update takes them.  Lanes 0-7 load face and thicknesses of
// neighbour q, lanes 8-15 the same and its cure fractions and alpha, and
// decide which of its strata flow; then the half-warp loads the flowing
// strata's slots four at a time.  So a cell's loads are a few instructions
// of the half-warp whose latencies overlap, instead of a chain of broadcast
// loads in the inflow loop.
struct FullStage {
  float4 f[8], th[8], cu[8], an[8];
  uint32_t cn[8];
  float pin[32][16];
};

// Strata pass, part 2: the listed cells, one per half-warp, over a grid of a
// few blocks per SM.  The full strata_update (strata.wgsl:238-273) builds the
// new stack: own outflow, inflow from the 8 neighbours, renormalisation to h
// and compaction.  Thicknesses go to the next generation, pigment slots to
// the side plane (copied back by k_strata_commit), then the cell is shaded
// and composed from the stored (rounded) slots.
// List entries first, first + stride, ... of film F; the tables are in
// shared memory.
template <int MODE>
__device__ __forceinline__ void strata_full_film(const Film& F, const float* tab, const float* cm, const float* ltab,
                                                 FullStage& S, uint32_t count, uint32_t first, uint32_t stride) {
  const HalfWarp H((int)(threadIdx.x & 31u));
  const cf_params& P = F.P->p;
  const bool dbg = P.flags[0] == 1u;
  const float4 z4 = make_float4(0.f, 0.f, 0.f, 0.f);
  for (uint32_t e = first; e < count; e += stride) {
    const uint32_t c = F.full_list[e];
    const int i = (int)(c % F.w), j = (int)(c / F.w);
    const float hc = F.hh[c];
    // neighbour nb of lane q & 7, in the reference's order: right, up,
    // up-right, down-right, left, down, down-left, up-left.  Faces 0-3 are
    // the cell's own (right, up, up-right, down-right) negated, faces 4-7 the
    // ones the active left, lower, lower-left and upper-left neighbours own;
    // the strata fast path has zeroed those strata_split did not write.
    const int nb = H.q & 7;
    // (di + 1, dj + 1) of neighbour nb in bits 2 nb, 2 nb + 1
    const int di = (int)((0x04a6u >> (2 * nb)) & 3u) - 1;
    const int dj = (int)((0x8129u >> (2 * nb)) & 3u) - 1;
    const int ni = i + di, nj = j + dj;
    const bool inb = ni >= 0 && nj >= 0 && ni < (int)F.w && nj < (int)F.h;
    const bool nact = inb && cell_active(F, ni, nj);
    const bool ok = nb < 4 ? inb : nact;  // the reference's inflow guards
    const uint32_t cn = inb ? idx(F, ni, nj) : c;
    __syncwarp(H.mask);  // the previous cell's stage has been read
    const float4 f = nb < 4 ? neg4(acc_face(F, c, nb)) : nact ? acc_face(F, cn, nb - 4) : z4;
    const float4 tn = ok ? F.sh[cn] : z4;
    uint32_t nib = 0u;
    if (H.q < 8) {
      S.f[nb] = f;
      S.th[nb] = tn;
      S.cn[nb] = cn;
    } else {
      const float4 an = nact ? F.alpha_s[cn] : make_float4(1.f, 1.f, 1.f, 1.f);
      S.cu[nb] = ok ? F.scu[cn] : z4;
      S.an[nb] = an;
      // the strata of neighbour nb that flow into the cell: a positive
      // limited flux and a positive thickness (strata.wgsl:248-262)
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        const float v = sel4(f, k) * sel4(an, k) * P.inv_dx;
        if (ok && v > 0.f && sel4(tn, k) > 0.f) nib |= 1u << k;
      }
    }
    // bit 4 nb + k: stratum k of neighbour nb flows in (the inflow order)
    const uint32_t fm = __reduce_or_sync(H.mask, nib << (4 * nb));
    LaneStack s;
    {
      const float4 t = F.sh[c], u = F.scu[c];
      s.th[0] = t.x; s.th[1] = t.y; s.th[2] = t.z; s.th[3] = t.w;
      s.cu[0] = u.x; s.cu[1] = u.y; s.cu[2] = u.z; s.cu[3] = u.w;
#pragma unroll
      for (int k = 0; k < 4; ++k) s.pg[k] = PigLane<MODE>::load(F, F.pig, c, k, H.q);
    }
    const float4 a4 = F.alpha_s[c];
    // the flowing strata's pigment slots, four loads in flight at a time
    {
      uint32_t m = fm;
      int slot = 0;
#pragma unroll 1
      while (m) {
        float v[4];
        int got = 0;
#pragma unroll
        for (int u = 0; u < 4; ++u)
          if (m) {
            const int b = __ffs(m) - 1;
            m &= m - 1u;
            v[u] = PigLane<MODE>::load(F, F.pig, S.cn[b >> 2], b & 3, H.q);
            got = u + 1;
          }
#pragma unroll
        for (int u = 0; u < 4; ++u)
          if (u < got) S.pin[slot + u][H.q] = v[u];
        slot += got;
      }
    }
    __syncwarp(H.mask);
    {
      float4 out = z4;
#pragma unroll
      for (int n = 0; n < 8; ++n) {
        const float4 g = S.f[n];
        out.x += fmaxf(-g.x, 0.f);
        out.y += fmaxf(-g.y, 0.f);
        out.z += fmaxf(-g.z, 0.f);
        out.w += fmaxf(-g.w, 0.f);
      }
      s.th[0] = fmaxf(s.th[0] - out.x * a4.x * P.inv_dx, 0.f);
      s.th[1] = fmaxf(s.th[1] - out.y * a4.y * P.inv_dx, 0.f);
      s.th[2] = fmaxf(s.th[2] - out.z * a4.z * P.inv_dx, 0.f);
      s.th[3] = fmaxf(s.th[3] - out.w * a4.w * P.inv_dx, 0.f);
    }
    // the inflows in the reference's order (neighbours 0-7, each from its
    // bottom stratum up): stratum k of neighbour nb lays the band [z0, z1)
    // of the neighbour's stack over this cell's; one copy of the stack code
    // serves all of them
    {
      int slot = 0;
#pragma unroll 1
      for (uint32_t m = fm; m; m &= m - 1u, ++slot) {
        const int b = __ffs(m) - 1, nb = b >> 2, k = b & 3;
        const float* th = reinterpret_cast<const float*>(&S.th[nb]);
        float z0 = 0.f;
#pragma unroll
        for (int kk = 0; kk < 3; ++kk)
          if (kk < k) z0 = z0 + th[kk];
        const float z1 = z0 + th[k];
        const float v = reinterpret_cast<const float*>(&S.f[nb])[k] * reinterpret_cast<const float*>(&S.an[nb])[k] *
                        P.inv_dx;
        lane_add_band(H, s, z0, z1, v, S.pin[slot][H.q], reinterpret_cast<const float*>(&S.cu[nb])[k], P.misc[0],
                      P.misc[1]);
      }
    }
    const float sum = s.th[0] + s.th[1] + s.th[2] + s.th[3];
    if (hc <= 0.f) {
#pragma unroll
      for (int k = 0; k < 4; ++k) { s.th[k] = 0.f; s.cu[k] = 0.f; }
    } else if (sum > 0.f) {
      const float kk = hc / sum;
#pragma unroll
      for (int k = 0; k < 4; ++k) s.th[k] *= kk;
    }
    lane_compact(H, s, P.misc[0]);
    if (H.q == 0) {
      F.sh2[c] = make_float4(s.th[0], s.th[1], s.th[2], s.th[3]);
      F.scu2[c] = make_float4(s.cu[0], s.cu[1], s.cu[2], s.cu[3]);
      if (hc > 0.f && !(s.th[0] + s.th[1] + s.th[2] + s.th[3] > 0.f)) {
        const uint32_t at = atomicAdd(&F.stats->fill_count, 1u);
        F.fill_list[at] = c;
      }
    }
    LaneAcc acc;
    acc.begin(H, F.refl + (size_t)c * 16);
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const float pk = get4(s.pg, k);
      PigLane<MODE>::store(F, F.pig2, c, k, H.q, pk);
      acc.add(H, k, get4(s.th, k), get4(s.cu, k), PigLane<MODE>::round(pk, H.q), hc, ltab, tab,
              reinterpret_cast<float*>(S.f), dbg);
    }
    const float4 agg = acc.agg(P);
    const float mv = F.m[c];
    const ushort4 dt = detail_texel<MODE>(F, c, acc.cure_top, hc, mv);  // its loads before the stores
    const ushort4 col = acc.color(H, P, cm, hc, mv);
    // the composite spectrum of the new stack (its thicknesses and stored
    // slots) is cached for the next frames' fast path, as its own shades are
    if (hc > 0.f) reinterpret_cast<float*>(F.spec)[((size_t)(H.q >> 2) * F.n + c) * 4 + (H.q & 3)] = acc.r;
    if (H.q == 0) {
      F.agg[c] = agg;
      F.color[c] = col;
      F.detail[c] = dt;
      F.shade_state[c] = hc <= 0.f ? SHADE_DRY : SHADE_WET;
    }
  }
}
// Copies the listed cells' new pigment slots from the side plane back into
// the pigment plane (consecutive threads take consecutive list entries).
template <int MODE>
__device__ __forceinline__ void strata_commit_film(const Film& F, size_t first, size_t stride) {
  constexpr uint32_t CH = 4u * PigIO<MODE>::QN;  // 16-byte chunks per cell
  const uint32_t count = F.stats->full_count;
  const size_t units = (size_t)count * CH;
  for (size_t u = first; u < units; u += stride) {
    const uint32_t ch = (uint32_t)(u / count), e = (uint32_t)(u % count);
    const size_t at = (size_t)ch * F.n + F.full_list[e];
    F.pig[at] = F.pig2[at];
  }
}
// strata_fill (strata.wgsl:288-323) x 6 over the candidates of the strata
// pass, in one block: select reads only strata sums, apply writes only cells
// that had none, and a block barrier separates the two (Jacobi semantics, as
// the reference's two dispatches per iteration).  A cell that is not a
// candidate has h <= 0, lies in an inactive tile or has strata, and so
// selects no source in any of the six iterations.
template <int MODE>
__device__ __forceinline__ void fill_list_film(const Film& F, float* lt) {
  const uint32_t count = F.stats->fill_count;
  if (count == 0u) return;
  const cf_params& P = F.P->p;
  if (threadIdx.x < 12) lt[threadIdx.x] = logf(fmaxf(F.pigtab[threadIdx.x * 40 + 32], 1e-3f));
  __syncthreads();
  for (int r = 0; r < 6; ++r) {
    for (uint32_t e = threadIdx.x; e < count; e += blockDim.x) {
      const uint32_t c = F.fill_list[e];
      const int i = (int)(c % F.w), j = (int)(c / F.w);
      int32_t src = -1;
      const float4 th = F.sh[c];
      if (!(th.x + th.y + th.z + th.w > 0.f)) {
        uint32_t cand[4];
        int nc = 0;
        if (i > 0) cand[nc++] = c - 1;
        if (j > 0) cand[nc++] = c - F.w;
        if (i + 1 < (int)F.w) cand[nc++] = c + 1;
        if (j + 1 < (int)F.h) cand[nc++] = c + F.w;
        float best = 0.f;
        for (int q = 0; q < nc; ++q) {
          const float4 tn = F.sh[cand[q]];
          const float ts = tn.x + tn.y + tn.z + tn.w;
          if (ts > best) { best = ts; src = (int32_t)cand[q]; }
        }
      }
      F.fill_src[e] = src;
    }
    __syncthreads();
    for (uint32_t e = threadIdx.x; e < count; e += blockDim.x) {
      const int32_t src = F.fill_src[e];
      if (src < 0) continue;
      const uint32_t c = F.fill_list[e];
      const float hc = F.hh[c];
      backfill<MODE>(F, c, (uint32_t)src, hc);
      Stack s;
      stack_load<MODE>(F, F.sh, F.scu, F.pig, c, s);
      float4 agg;
      ushort4 col;
      finish_stack(P, lt, F.pigtab, F.cmf, F.refl + (size_t)c * 16, hc, F.m[c], s, agg, col);
      F.agg[c] = agg;
      F.color[c] = col;
      F.detail[c] = detail_texel<MODE>(F, c, top_cure(s.th, s.cu), hc, F.m[c]);
      F.shade_state[c] = hc <= 0.f ? SHADE_DRY : SHADE_NONE;
    }
    __syncthreads();
  }
}
// strata_fill as one select + apply pair over the whole grid (inspection
// dispatch; the frame runs k_fill_list).
__device__ __forceinline__ void fill_select_tile(const Film& F, TileId T) {
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
// ...and re-shades the filled cell and refreshes its aggregates.
template <int MODE>
__device__ __forceinline__ void fill_apply_tile(const Film& F, TileId T) {
  TILE_PROLOGUE
  int32_t src = F.fill_src[c];
  if (src < 0) return;
  float hc = F.hh[c];
  backfill<MODE>(F, c, (uint32_t)src, hc);
  Stack s;
  stack_load<MODE>(F, F.sh, F.scu, F.pig, c, s);
  float lt[12];
  lnmu_table(F.pigtab, lt);
  float4 agg;
  ushort4 col;
  finish_stack(P, lt, F.pigtab, F.cmf, F.refl + (size_t)c * 16, hc, F.m[c], s, agg, col);
  F.agg[c] = agg;
  F.color[c] = col;
  F.detail[c] = detail_texel<MODE>(F, c, top_cure(s.th, s.cu), hc, F.m[c]);
  F.shade_state[c] = hc <= 0.f ? SHADE_DRY : SHADE_NONE;
}

// Aggregates and colour of the current state (after a state upload, or for
// an inspection dispatch of cure or shade).
template <int MODE>
__device__ __forceinline__ void compose_tile(const Film& F, TileId T, int shade) {
  const int i = (int)(T.x * 16 + threadIdx.x), j = (int)(T.y * 16 + threadIdx.y);
  if (i >= (int)F.w || j >= (int)F.h) return;
  const uint32_t c = idx(F, i, j);
  const cf_params& P = F.P->p;
  Stack s;
  stack_load<MODE>(F, F.sh, F.scu, F.pig, c, s);
  float lt[12];
  lnmu_table(F.pigtab, lt);
  float4 agg;
  ushort4 col;
  finish_stack(P, lt, F.pigtab, F.cmf, F.refl + (size_t)c * 16, F.hh[c], F.m[c], s, agg, col);
  F.agg[c] = agg;
  if (shade) {
    F.color[c] = col;
    F.detail[c] = detail_texel<MODE>(F, c, top_cure(s.th, s.cu), F.hh[c], F.m[c]);
    F.shade_state[c] = F.hh[c] <= 0.f ? SHADE_DRY : SHADE_NONE;
  }
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

__device__ __forceinline__ void stats_reset_film(const Film& F) {
  F.stats->h_max_bits = 0u;
  F.stats->mu_min_bits = __float_as_uint(1e9f);
  F.stats->active_tiles = 0u;
  F.stats->fill_count = 0u;
  F.stats->full_count = 0u;
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
__device__ __forceinline__ void adaptive_params_film(DevParams* Dp, DevStats* S) {
  DevParams D = *Dp;
  cf_params& P = D.p;
  float h_stat = __uint_as_float(S->h_max_bits);
  float mu_raw = __uint_as_float(S->mu_min_bits);
  float mu_stat = mu_raw > 1e8f ? 1.0f : mu_raw;
  float dx = P.dx;
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

// ---- state I/O: reference pigment layout [cell][stratum][slot] <-> chunks ----
// A block transposes 32 cells through shared memory: it reads their 64 slots
// as one contiguous run (the source may be pinned host memory read over the
// link), then writes each chunk plane's 32 cells as one contiguous run.
template <int MODE>
__global__ void __launch_bounds__(256) k_pig_import_t(Film F, uint4* dst, const void* src, int fmt) {
  constexpr int QN = PigIO<MODE>::QN, PER = 16 / QN, CB = 32;
  __shared__ float sv[CB][65];
  const size_t c0 = (size_t)blockIdx.x * CB;
  const int ncell = (int)min((size_t)CB, (size_t)F.n - c0);
  for (int e = threadIdx.x; e < ncell * 64; e += blockDim.x) {
    const size_t s = c0 * 64 + (size_t)e;
    float x;
    if (fmt == CF_PIG_F32) x = ((const float*)src)[s];
    else if (fmt == CF_PIG_F16) x = h16_to_f(((const uint16_t*)src)[s]);
    else x = slot_from_b16(((const uint16_t*)src)[s], e % 16);
    sv[e / 64][e % 64] = x;
  }
  __syncthreads();
  for (int e = threadIdx.x; e < 4 * QN * CB; e += blockDim.x) {
    const int cl = e % CB, plane = e / CB;
    if (cl >= ncell) continue;
    const int k = plane / QN, q = plane % QN;
    const float* v = &sv[cl][16 * k + q * PER];
    uint32_t wv[4];
    for (int w = 0; w < 4; ++w) {
      if (MODE == CF_PREC_FP32) wv[w] = __float_as_uint(v[w]);
      else if (MODE == CF_PREC_REFERENCE) wv[w] = f_to_h16(v[2 * w]) | (f_to_h16(v[2 * w + 1]) << 16);
      else wv[w] = b16_from_slot(v[2 * w], q * PER + 2 * w) | (b16_from_slot(v[2 * w + 1], q * PER + 2 * w + 1) << 16);
    }
    dst[PigIO<MODE>::at(F, (uint32_t)(c0 + cl), k, q)] = make_uint4(wv[0], wv[1], wv[2], wv[3]);
  }
}
// The inverse transpose: a block reads each chunk plane's run of 32 cells,
// then writes the 32 cells' 64 slots as one contiguous run (the destination
// may be page-locked host memory written over the link).
template <int MODE>
__global__ void __launch_bounds__(256) k_pig_export_t(Film F, const uint4* srcp, void* dst, int fmt) {
  constexpr int QN = PigIO<MODE>::QN, PER = 16 / QN, CB = 32;
  __shared__ float sv[CB][65];
  const size_t c0 = (size_t)blockIdx.x * CB;
  const int ncell = (int)min((size_t)CB, (size_t)F.n - c0);
  for (int e = threadIdx.x; e < 4 * QN * CB; e += blockDim.x) {
    const int cl = e % CB, plane = e / CB;
    if (cl >= ncell) continue;
    const int k = plane / QN, q = plane % QN;
    const uint4 u = srcp[PigIO<MODE>::at(F, (uint32_t)(c0 + cl), k, q)];
    const uint32_t wv[4] = {u.x, u.y, u.z, u.w};
    float* v = &sv[cl][16 * k + q * PER];
    for (int x = 0; x < PER; ++x) {
      if (MODE == CF_PREC_FP32) v[x] = __uint_as_float(wv[x]);
      else {
        const uint32_t bits = (x & 1) ? (wv[x / 2] >> 16) : (wv[x / 2] & 0xffffu);
        v[x] = MODE == CF_PREC_REFERENCE ? h16_to_f(bits) : slot_from_b16(bits, q * PER + x);
      }
    }
  }
  __syncthreads();
  for (int e = threadIdx.x; e < ncell * 64; e += blockDim.x) {
    const size_t s = c0 * 64 + (size_t)e;
    const float x = sv[e / 64][e % 64];
    if (fmt == CF_PIG_F32) ((float*)dst)[s] = x;
    else if (fmt == CF_PIG_F16) ((uint16_t*)dst)[s] = (uint16_t)f_to_h16(x);
    else ((uint16_t*)dst)[s] = (uint16_t)b16_from_slot(x, e % 16);
  }
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

// delta -> delta_old for one tile (the inspection dispatch of nose; in the
// frame, apply takes this snapshot)
__device__ __forceinline__ void copy_delta_tile(const Film& F, TileId T) {
  const int i = (int)(T.x * 16 + threadIdx.x), j = (int)(T.y * 16 + threadIdx.y);
  if (i < (int)F.w && j < (int)F.h) {
    const uint32_t c = idx(F, i, j);
    F.delta_old[c] = F.delta[c];
  }
}

// ------------------------------------------------------ packed kernels --
// One launch per dispatch for many films: block b takes entry b of a tile
// table (film index, tile index), so canvases of any size share the grid.
// The film records are read-only for the launch.

#define PACKED_ARGS const Film* __restrict__ films, const uint2* __restrict__ tiles, uint32_t ntiles
// Without WALK, block b is table entry b (one 16x16 tile).  With WALK (the
// instances a batch launches when its tuning groups tiles), block b takes
// the run of consecutive entries [b * per, (b + 1) * per) with per =
// ceil(ntiles / gridDim.x): a strip of tiles along a row (a 32 x 16 or
// 64 x 16 launch tile), or, with a grid of a few blocks per SM, the table in
// long runs (persistent).  The loop is a separate instance because the
// registers it keeps live slowed the one-tile kernels by 12-25 %; each tile's
// body is the same code in both.
#define PACKED_TILES(WALK, ...)                                                 \
  {                                                                             \
    if constexpr (!(WALK)) {                                                    \
      if (blockIdx.x >= ntiles) return;                                         \
      const uint2 pe_ = tile_entry(tiles, blockIdx.x);                          \
      const Film& F = films[pe_.x];                                             \
      const TileId T{pe_.y % F.tw, pe_.y / F.tw};                               \
      __VA_ARGS__;                                                              \
    } else {                                                                    \
      const uint32_t per_ = (ntiles + gridDim.x - 1u) / gridDim.x;              \
      const uint32_t e0_ = blockIdx.x * per_, e1_ = min(ntiles, e0_ + per_);    \
      for (uint32_t e_ = e0_; e_ < e1_; ++e_) {                                 \
        if (e_ != e0_) __syncthreads(); /* shared memory of the last tile */    \
        const uint2 pe_ = tile_entry(tiles, e_);                                \
        const Film& F = films[pe_.x];                                           \
        const TileId T{pe_.y % F.tw, pe_.y / F.tw};                             \
        __VA_ARGS__;                                                            \
      }                                                                         \
    }                                                                           \
  }
// eight blocks per SM (32 registers): the common path is a handful of loads
// and an exp; the rare commit branch is out of line and may spill
template <int MODE, bool WALK = false>
__global__ void __launch_bounds__(256, 8) kp_cure(PACKED_ARGS) { PACKED_TILES(WALK, cure_tile<MODE>(F, T)) }
template <bool WALK = false>
__global__ void __launch_bounds__(256) kp_clear_acc(PACKED_ARGS) { PACKED_TILES(WALK, clear_acc_tile(F, T)) }
template <bool CLEAR, bool WALK = false>
__global__ void __launch_bounds__(128, 16) kp_laplacian(PACKED_ARGS) { PACKED_TILES(WALK, laplacian_tile<CLEAR>(F, T)) }
template <int MODE, bool WALK = false>
__global__ void __launch_bounds__(256) kp_plug(PACKED_ARGS) { PACKED_TILES(WALK, plug_tile<MODE>(F, T)) }
// three blocks per SM: the face code needs no more than 64 registers, and
// the occupancy hides its dependent loads
template <int MODE, bool WALK = false>
__global__ void __launch_bounds__(256, 6) kp_fluxes(PACKED_ARGS) { PACKED_TILES(WALK, fluxes_tile<MODE>(F, T)) }
template <int MODE, bool CLEAR, bool WALK = false>
__global__ void __launch_bounds__(256, 6) kp_flow(PACKED_ARGS) { PACKED_TILES(WALK, flow_tile<MODE, CLEAR>(F, T)) }
template <int MODE, bool WALK = false>
__global__ void __launch_bounds__(128, 16) kp_strata_split(PACKED_ARGS) { PACKED_TILES(WALK, strata_split_tile<MODE>(F, T)) }
template <bool WALK = false>
__global__ void __launch_bounds__(64) kp_limiter(PACKED_ARGS) { PACKED_TILES(WALK, limiter_tile(F, T)) }
// eight blocks of 128 per SM (64 registers for the two cells' loads in flight)
template <int MODE, bool WALK = false>
__global__ void __launch_bounds__(128, 8) kp_apply(PACKED_ARGS) { PACKED_TILES(WALK, apply_tile<MODE>(F, T)) }
template <bool WALK = false>
__global__ void __launch_bounds__(256) kp_copy_delta(PACKED_ARGS) { PACKED_TILES(WALK, copy_delta_tile(F, T)) }
template <bool NEXT, bool WALK = false>
__global__ void __launch_bounds__(128, 16) kp_nose(PACKED_ARGS) { PACKED_TILES(WALK, nose_tile<NEXT>(F, T)) }
template <int MODE, bool WALK = false>
__global__ void __launch_bounds__(128, 16) kp_limit_apply(PACKED_ARGS) { PACKED_TILES(WALK, limit_apply_tile<MODE>(F, T)) }

template <int MODE, bool WALK = false>
__global__ void __launch_bounds__(256) kp_reduce(PACKED_ARGS) { PACKED_TILES(WALK, reduce16_tile<MODE>(F, T)) }
template <int MODE, bool WALK = false>
__global__ void __launch_bounds__(128, 12) kp_strata_fast(PACKED_ARGS) { PACKED_TILES(WALK, strata_fast_tile<MODE>(F, T)) }
template <bool WALK = false>
__global__ void __launch_bounds__(256) kp_strata_limit(PACKED_ARGS) { PACKED_TILES(WALK, strata_limit_tile(F, T)) }
template <bool WALK = false>
__global__ void __launch_bounds__(256) kp_face_flags(PACKED_ARGS) { PACKED_TILES(WALK, face_flags_tile(F, T)) }
template <bool WALK = false>
__global__ void __launch_bounds__(256) kp_fill_select(PACKED_ARGS) { PACKED_TILES(WALK, fill_select_tile(F, T)) }
template <int MODE, bool WALK = false>
__global__ void __launch_bounds__(256) kp_fill_apply(PACKED_ARGS) { PACKED_TILES(WALK, fill_apply_tile<MODE>(F, T)) }
template <int MODE, bool WALK = false>
__global__ void __launch_bounds__(256) kp_compose(PACKED_ARGS, int shade) { PACKED_TILES(WALK, compose_tile<MODE>(F, T, shade)) }
__global__ void __launch_bounds__(256) kp_mark_tiles(PACKED_ARGS) {
  const uint32_t e = blockIdx.x * 8u + (threadIdx.x >> 5);
  if (e >= ntiles) return;
  const uint2 pe = tile_entry(tiles, e);
  mark_tile(films[pe.x], pe.y);
}
// One thread per tile; the active tiles of a warp are counted with one atomic
// per film instead of one per tile (all the tiles of a film otherwise add to
// the same counter).
__global__ void __launch_bounds__(256) kp_compact_tiles(PACKED_ARGS) {
  const uint32_t e = blockIdx.x * blockDim.x + threadIdx.x;
  const bool in = e < ntiles;
  const uint2 pe = in ? tile_entry(tiles, e) : make_uint2(0u, 0u);
  const bool act = in && compact_tile(films[pe.x], pe.y, (int)films[pe.x].all_active);
  const unsigned m = __ballot_sync(0xffffffffu, act);
  if (act) {
    const unsigned same = __match_any_sync(m, pe.x);
    if ((threadIdx.x & 31u) == (unsigned)(__ffs(same) - 1))
      atomicAdd(&films[pe.x].stats->active_tiles, (uint32_t)__popc(same));
  }
}
#undef PACKED_TILES
#undef PACKED_ARGS
// per film: one thread each
__global__ void kp_stats_reset(const Film* __restrict__ films, uint32_t nfilms) {
  const uint32_t f = blockIdx.x * blockDim.x + threadIdx.x;
  if (f < nfilms) stats_reset_film(films[f]);
}
__global__ void kp_adaptive_params(const Film* __restrict__ films, uint32_t nfilms) {
  const uint32_t f = blockIdx.x * blockDim.x + threadIdx.x;
  if (f < nfilms) adaptive_params_film(const_cast<DevParams*>(films[f].P), films[f].stats);
}
// the strata full path over every film's list, with the film's tables
template <int MODE>
__global__ void __launch_bounds__(256, 4) kp_strata_full(const Film* __restrict__ films, uint32_t nfilms) {
  __shared__ float tab[480];
  __shared__ float cm[48];
  __shared__ float ltab[12];
  __shared__ FullStage stage[16];  // one per half-warp
  for (uint32_t f = 0; f < nfilms; ++f) {
    const Film& F = films[f];
    const uint32_t count = F.stats->full_count;
    const uint32_t first = blockIdx.x * (blockDim.x >> 4);
    if (first >= count) continue;  // the same for the whole block
    __syncthreads();
    load_tables(F, tab, cm, ltab, threadIdx.x, 256);
    __syncthreads();
    strata_full_film<MODE>(F, tab, cm, ltab, stage[threadIdx.x >> 4], count, first + (threadIdx.x >> 4),
                           gridDim.x * (blockDim.x >> 4));
  }
}
template <int MODE>
__global__ void __launch_bounds__(256) kp_strata_commit(const Film* __restrict__ films, uint32_t nfilms) {
  for (uint32_t f = 0; f < nfilms; ++f)
    strata_commit_film<MODE>(films[f], blockIdx.x * (size_t)blockDim.x + threadIdx.x, (size_t)gridDim.x * blockDim.x);
}
// one block per film
template <int MODE>
__global__ void __launch_bounds__(1024) kp_fill_list(const Film* __restrict__ films, uint32_t nfilms) {
  __shared__ float lt[12];
  if (blockIdx.x < nfilms) fill_list_film<MODE>(films[blockIdx.x], lt);
}

// ---------------------------------------------------------------- host --

// Launches K<MODE> for the run-time precision `mode`.
#define CFK_LAUNCH(K, G, B, ST, ...)                                    \
  do {                                                                  \
    if (mode == CF_PREC_REFERENCE) K<CF_PREC_REFERENCE><<<G, B, 0, ST>>>(__VA_ARGS__); \
    else if (mode == CF_PREC_FP32) K<CF_PREC_FP32><<<G, B, 0, ST>>>(__VA_ARGS__);     \
    else K<CF_PREC_BF16><<<G, B, 0, ST>>>(__VA_ARGS__);                 \
  } while (0)

template <int MODE>
static uint32_t frame_packed_t(const PackedFrame& V, uint32_t substeps, int adaptive, cudaStream_t st) {
  const Film* A = V.films;
  const uint2* T = V.tiles;
  const uint32_t nt = V.ntiles, nf = V.nfilms;
  if (nf == 0u || nt == 0u) return 0u;
  const uint32_t fb = (nf + 127u) / 128u;
  // blocks of the per-tile kernels (see PACKED_TILES); the implicit steps'
  // kernels keep one block per tile
  const uint32_t tg = V.tile_grid != 0u && V.tile_grid < nt ? V.tile_grid : nt;
  uint32_t n = 0;
  dim3 b(16, 16);
  using TileKernel = void (*)(const Film*, const uint2*, uint32_t);
  // the one-tile instance, or the walking one over a grid of tg blocks
  auto tl = [&](TileKernel one, TileKernel walk, dim3 B) {
    if (tg < nt) walk<<<tg, B, 0, st>>>(A, T, nt);
    else one<<<nt, B, 0, st>>>(A, T, nt);
  };
  if (adaptive) { kp_adaptive_params<<<fb, 128, 0, st>>>(A, nf); ++n; }
  kp_stats_reset<<<fb, 128, 0, st>>>(A, nf);
  kp_mark_tiles<<<(nt + 7u) / 8u, 256, 0, st>>>(A, T, nt);
  kp_compact_tiles<<<(nt + 255u) / 256u, 256, 0, st>>>(A, T, nt);
  tl(kp_cure<MODE, false>, kp_cure<MODE, true>, b);
  n += 4;
  // clear_acc runs with the first laplacian of the frame: the first implicit
  // step's (src/film/mod.rs:1371-1376) or the first substep's
  const uint32_t isteps = V.implicit_steps;
  if (substeps == 0 && isteps == 0) { tl(kp_clear_acc<false>, kp_clear_acc<true>, b); ++n; }
  for (uint32_t s = 0; s < isteps; ++s) {
    if (s == 0) kp_laplacian<true><<<nt, dim3(16, 8), 0, st>>>(A, T, nt);
    else kp_laplacian<false><<<nt, dim3(16, 8), 0, st>>>(A, T, nt);
    n += 1 + launch_cg_step(V, MODE, s, V.implicit_iters, V.cap_implicit, st);
  }
  for (uint32_t s = 0; s < substeps; ++s) {
    // laplacian + plug + fluxes as one flow launch (with clear_acc on the
    // frame's first)
    if (s == 0 && isteps == 0) tl(kp_flow<MODE, true, false>, kp_flow<MODE, true, true>, b);
    else tl(kp_flow<MODE, false, false>, kp_flow<MODE, false, true>, b);
    // limiter + apply (alpha on chip, new heights to h_next), then the nose,
    // which commits them
    tl(kp_limit_apply<MODE, false>, kp_limit_apply<MODE, true>, dim3(16, 8));
    tl(kp_nose<true, false>, kp_nose<true, true>, dim3(16, 8));
    n += 3;
  }
  tl(kp_laplacian<false, false>, kp_laplacian<false, true>, dim3(16, 8));
  tl(kp_strata_split<MODE, false>, kp_strata_split<MODE, true>, dim3(16, 8));
  tl(kp_strata_fast<MODE, false>, kp_strata_fast<MODE, true>, dim3(16, 8));  // with the CFL reduction
  kp_strata_full<MODE><<<V.persist_blocks, 256, 0, st>>>(A, nf);
  kp_strata_commit<MODE><<<V.persist_blocks, 256, 0, st>>>(A, nf);
  kp_fill_list<MODE><<<nf, 1024, 0, st>>>(V.films_next, nf);
  return n + 6;
}

uint32_t launch_frame_packed(const PackedFrame& V, int mode, uint32_t substeps, int adaptive, cudaStream_t st) {
  if (mode == CF_PREC_REFERENCE) return frame_packed_t<CF_PREC_REFERENCE>(V, substeps, adaptive, st);
  if (mode == CF_PREC_FP32) return frame_packed_t<CF_PREC_FP32>(V, substeps, adaptive, st);
  return frame_packed_t<CF_PREC_BF16>(V, substeps, adaptive, st);
}

void launch_cure(const PackedFrame& V, int mode, cudaStream_t st) {
  CFK_LAUNCH(kp_cure, V.ntiles, dim3(16, 16), st, V.films, V.tiles, V.ntiles);
}

void launch_compose(const PackedFrame& V, int mode, int shade, cudaStream_t st) {
  CFK_LAUNCH(kp_compose, V.ntiles, dim3(16, 16), st, V.films, V.tiles, V.ntiles, shade);
}

void launch_reduce(const PackedFrame& V, int mode, cudaStream_t st) {
  kp_stats_reset<<<(V.nfilms + 127u) / 128u, 128, 0, st>>>(V.films, V.nfilms);
  CFK_LAUNCH(kp_reduce, V.ntiles, dim3(16, 16), st, V.films, V.tiles, V.ntiles);
}

void launch_mass(const Film& F, int sms, cudaStream_t st) {
  k_mass_reset<<<1, 1, 0, st>>>(F);
  k_mass<<<sms * 4, 256, 0, st>>>(F);
}

void launch_fill_u32(uint32_t* p, uint32_t v, size_t n, cudaStream_t st) {
  if (n) k_fill_u32<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(p, v, n);
}

void launch_pig_import(const Film& F, int mode, uint4* dst, const void* src, int fmt, cudaStream_t st) {
  const unsigned g = (unsigned)(((size_t)F.n + 31) / 32);
  if (mode == CF_PREC_REFERENCE) k_pig_import_t<CF_PREC_REFERENCE><<<g, 256, 0, st>>>(F, dst, src, fmt);
  else if (mode == CF_PREC_FP32) k_pig_import_t<CF_PREC_FP32><<<g, 256, 0, st>>>(F, dst, src, fmt);
  else k_pig_import_t<CF_PREC_BF16><<<g, 256, 0, st>>>(F, dst, src, fmt);
}
void launch_pig_export(const Film& F, int mode, const uint4* srcp, void* dst, int fmt, cudaStream_t st) {
  const unsigned g = (unsigned)(((size_t)F.n + 31) / 32);
  if (mode == CF_PREC_REFERENCE) k_pig_export_t<CF_PREC_REFERENCE><<<g, 256, 0, st>>>(F, srcp, dst, fmt);
  else if (mode == CF_PREC_FP32) k_pig_export_t<CF_PREC_FP32><<<g, 256, 0, st>>>(F, srcp, dst, fmt);
  else k_pig_export_t<CF_PREC_BF16><<<g, 256, 0, st>>>(F, srcp, dst, fmt);
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

// Single dispatches for parity checks, named after the WGSL entry points,
// on the same kernels as the frame.  "strata_pass" runs strata_limit +
// strata_update + shade into the other thickness generation (returns 2: the
// caller swaps the film's generations) and "strata_fill" one select/apply pair
// over the whole grid.  Returns 0 for an unknown name.
int launch_one(const PackedFrame& V, int mode, const char* name, cudaStream_t st) {
  const Film* A = V.films;
  const uint2* T = V.tiles;
  const uint32_t nt = V.ntiles, nf = V.nfilms, fb = (nf + 127u) / 128u;
  const dim3 b(16, 16);
  std::string_view n(name);
  if (n == "mark_tiles") kp_mark_tiles<<<(nt + 7u) / 8u, 256, 0, st>>>(A, T, nt);
  else if (n == "compact_tiles") {
    kp_stats_reset<<<fb, 128, 0, st>>>(A, nf);
    kp_compact_tiles<<<(nt + 255u) / 256u, 256, 0, st>>>(A, T, nt);
  }
  else if (n == "cure_step") { launch_compose(V, mode, 0, st); launch_cure(V, mode, st); }
  else if (n == "clear_acc") kp_clear_acc<<<nt, b, 0, st>>>(A, T, nt);
  else if (n == "laplacian") kp_laplacian<false><<<nt, dim3(16, 8), 0, st>>>(A, T, nt);
  else if (n == "plug") CFK_LAUNCH(kp_plug, nt, b, st, A, T, nt);
  else if (n == "fluxes") CFK_LAUNCH(kp_fluxes, nt, b, st, A, T, nt);
  else if (n == "flow") {  // laplacian + plug + fluxes fused, as the frame runs them
    if (mode == CF_PREC_REFERENCE) kp_flow<CF_PREC_REFERENCE, false><<<nt, b, 0, st>>>(A, T, nt);
    else if (mode == CF_PREC_FP32) kp_flow<CF_PREC_FP32, false><<<nt, b, 0, st>>>(A, T, nt);
    else kp_flow<CF_PREC_BF16, false><<<nt, b, 0, st>>>(A, T, nt);
  }
  else if (n == "limiter") kp_limiter<<<nt, dim3(16, 4), 0, st>>>(A, T, nt);
  else if (n == "apply") CFK_LAUNCH(kp_apply, nt, dim3(16, 8), st, A, T, nt);
  else if (n == "nose") {
    kp_copy_delta<<<nt, b, 0, st>>>(A, T, nt);  // the snapshot the frame's apply takes
    kp_nose<false><<<nt, dim3(16, 8), 0, st>>>(A, T, nt);
  }
  // limiter + apply fused, as the frame runs them: the new heights in h_next
  else if (n == "limit_apply") CFK_LAUNCH(kp_limit_apply, nt, dim3(16, 8), st, A, T, nt);
  else if (n == "strata_split") CFK_LAUNCH(kp_strata_split, nt, dim3(16, 8), st, A, T, nt);
  else if (n == "reduce_tiles") launch_reduce(V, mode, st);
  else if (n == "strata_limit") {  // the face flags of the acc_s plane it is given
    kp_face_flags<<<nt, b, 0, st>>>(A, T, nt);
    kp_strata_limit<<<nt, b, 0, st>>>(A, T, nt);
  }
  else if (n == "strata_pass") {
    kp_stats_reset<<<fb, 128, 0, st>>>(A, nf);
    kp_face_flags<<<nt, b, 0, st>>>(A, T, nt);
    CFK_LAUNCH(kp_strata_fast, nt, dim3(16, 8), st, A, T, nt);
    CFK_LAUNCH(kp_strata_full, V.persist_blocks, 256, st, A, nf);
    CFK_LAUNCH(kp_strata_commit, V.persist_blocks, 256, st, A, nf);
    return 2;
  }
  else if (n == "strata_fill") {
    kp_fill_select<<<nt, b, 0, st>>>(A, T, nt);
    CFK_LAUNCH(kp_fill_apply, nt, b, st, A, T, nt);
  }
  else if (n == "shade_full") launch_compose(V, mode, 1, st);
  else return 0;
  return 1;
}

}  // namespace cfk
