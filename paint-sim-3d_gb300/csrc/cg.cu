// cg.cu — the implicit hydrostatic steps of a frame (film.wgsl:895-1302,
// dispatched by Film::encode_frame, src/film/mod.rs:1373-1408): per step a
// Jacobi-preconditioned conjugate-gradient solve of the hydrostatic flow of
// the frame over the active tiles, then the flux it implies and a mass
// rescale.
//
// Layout of the work (one film alone or many in a packed launch):
//  - kp_cg_setup: the face mobilities cg_m (and, with the implicit capillary
//    term, cg_t / cg_t2, the weighted Laplacians of h and of the hold level);
//  - kp_cg_init: diagonal, right-hand side, residual, first direction;
//  - per iteration, two launches over the tiles and two small ones for the
//    film scalars: kp_cg_iter_a forms the new search direction
//    p_k = r / d + beta p_{k-1} of its own cell and of its active neighbours
//    on the fly (so the reference's cg_iter_c needs no launch of its own),
//    writes it to one of two ping-pong planes and computes q = A p_k;
//    kp_cg_iter_b updates x and r;
//  - kp_cg_finish: the flux of the step into acc, the new h into a side plane
//    (neighbours read h as of before the dispatch), the final direction into
//    cg_p; kp_cg_rescale: the mass correction and the h commit.
// Each sum over a film (p.q, r.z, the mass change) is a per-tile tree sum
// written by every block of the film; the film's total, in tile order, comes
// from kp_cg_scalars (one block per film) in the iterations, and from the
// last block to finish (an atomic count, no waiting) in the once-per-step
// kernels.  A neighbour in an inactive tile
// is read as the reference reads it: its cg_m and cg_p as the last step that
// covered it left them.
#include "film_kernels.h"

namespace cfk {

namespace {

__device__ __forceinline__ float kappa(const cf_params& P) {  // film.wgsl:925-927
  return P.front[3] * P.phys[0] * P.g[2] * P.inv_dx * P.inv_dx;
}
__device__ __forceinline__ float hold_u(const Film& F, const cf_params& P, uint32_t c) {  // film.wgsl:929-933
  float hold = 0.f;
  if (F.hh[c] > 0.f) hold = hold_level(P, nose_dist(F, c));
  return F.m[c] - hold;
}

// film.wgsl:895-923: the mobility of a face (the face's flow index as in face())
template <int MODE>
__device__ float face_mob(const Film& F, const cf_params& P, uint32_t ca, uint32_t cb, float2 gcap, float2 ghyd,
                          float2 gtilt, bool diag) {
  const float ha = F.hh[ca], hb = F.hh[cb];
  if (fminf(ha, hb) <= 0.f) return 0.f;
  const float hf = 0.5f * (ha + hb);
  const float rax = rmu<MODE>(F, ca), ray = rtau<MODE>(F, ca);
  const float rbx = rmu<MODE>(F, cb), rby = rtau<MODE>(F, cb);
  const float wa = ha / (ha + hb);
  const float wb = 1.0f - wa;
  const float mu = expf(wa * logf(fmaxf(rax, 1e-4f)) + wb * logf(fmaxf(rbx, 1e-4f)));
  const float ty = wa * ray + wb * rby;
  const float na = rn<MODE>(F, ca), nb = rn<MODE>(F, cb);
  const float nf = na == nb ? na : wa * na + wb * nb;
  const float thin = fminf(ha, hb) / hf;
  const float fcap = thin * thin * thin;
  float2 yc = make_float2(gcap.x * fcap, gcap.y * fcap);  // yield_cap (film.wgsl:44-49)
  {
    const float gcl = sqrtf(yc.x * yc.x + yc.y * yc.y);
    const float gc_max = P.phys[1] / (1e-3f * 1e-3f);
    if (!(ty <= 0.f || gcl <= gc_max)) {
      const float sc = gc_max / gcl;
      yc.x = yc.x * sc;
      yc.y = yc.y * sc;
    }
  }
  const float2 gg = make_float2(yc.x + ghyd.x + gtilt.x, yc.y + ghyd.y + gtilt.y);
  const float gmag = sqrtf(gg.x * gg.x + gg.y * gg.y);
  float ydep = hf;  // yield_depth (film.wgsl:89-92)
  if (ty > 0.f) ydep = gg.x >= 0.f ? ha : hb;
  float qq, qy, qup;
  hb_flux(gmag, ydep, mu, ty, nf, qq, qy, qup);
  if (qq <= 0.f) return 0.f;
  float mob = fminf(fmaxf(qq / gmag - P.misc[3], 0.f), P.front[2]);
  if (fminf(ha, hb) < 0.5f * fmaxf(ha, hb)) {
    if (diag) return 0.f;
    const uint32_t tgt = hb > ha ? ca : cb;
    mob = mob / powf((float)max(feeders(F, P, tgt), 1u), 0.7f);
  }
  return mob;
}

// film.wgsl:994-1010: neighbour k of (i, j) and the weighted mobility of the
// face to it; faces 4..7 belong to the lower-left neighbours
__device__ __forceinline__ bool cg_nb(const Film& F, int k, int i, int j, uint32_t& nc, float& mw) {
  const uint32_t c = idx(F, i, j);
  nc = 0u;
  mw = 0.f;
  const int W = (int)F.w, H = (int)F.h;
  switch (k) {
    case 0: if (i + 1 < W) { nc = idx(F, i + 1, j); mw = W_AXIS * F.cg_m[c].x; } break;
    case 1: if (j + 1 < H) { nc = idx(F, i, j + 1); mw = W_AXIS * F.cg_m[c].y; } break;
    case 2: if (i + 1 < W && j + 1 < H) { nc = idx(F, i + 1, j + 1); mw = W_DIAG_LAP * F.cg_m[c].z; } break;
    case 3: if (i + 1 < W && j > 0) { nc = idx(F, i + 1, j - 1); mw = W_DIAG_LAP * F.cg_m[c].w; } break;
    case 4: if (i > 0) { nc = idx(F, i - 1, j); mw = W_AXIS * F.cg_m[nc].x; } break;
    case 5: if (j > 0) { nc = idx(F, i, j - 1); mw = W_AXIS * F.cg_m[nc].y; } break;
    case 6: if (i > 0 && j > 0) { nc = idx(F, i - 1, j - 1); mw = W_DIAG_LAP * F.cg_m[nc].z; } break;
    default: if (i > 0 && j + 1 < H) { nc = idx(F, i - 1, j + 1); mw = W_DIAG_LAP * F.cg_m[nc].w; } break;
  }
  return mw > 0.f;
}

// film.wgsl:1023-1043: sum over wet active neighbours of w (v(n) - v(c))
template <class Src>
__device__ __forceinline__ float lap_w(const Film& F, int i, int j, uint32_t c, Src v) {
  const float vc = v(c);
  float acc_v = 0.f;
  for (int dj = -1; dj <= 1; ++dj)
    for (int di = -1; di <= 1; ++di) {
      if (di == 0 && dj == 0) continue;
      const int x = i + di, y = j + dj;
      if (x < 0 || y < 0 || x >= (int)F.w || y >= (int)F.h) continue;
      if (!cell_active(F, x, y)) continue;
      const uint32_t n = idx(F, x, y);
      if (F.hh[n] <= 0.f) continue;
      const float w = (di != 0 && dj != 0) ? W_DIAG_LAP : W_AXIS;
      acc_v += w * (v(n) - vc);
    }
  return acc_v;
}
// film.wgsl:1045-1064
__device__ __forceinline__ float lap_diag(const Film& F, int i, int j) {
  float s1 = 0.f, s2 = 0.f;
  for (int dj = -1; dj <= 1; ++dj)
    for (int di = -1; di <= 1; ++di) {
      if (di == 0 && dj == 0) continue;
      const int x = i + di, y = j + dj;
      if (x < 0 || y < 0 || x >= (int)F.w || y >= (int)F.h) continue;
      if (!cell_active(F, x, y)) continue;
      if (F.hh[idx(F, x, y)] <= 0.f) continue;
      const float w = (di != 0 && dj != 0) ? W_DIAG_LAP : W_AXIS;
      s1 += w;
      s2 += w * w;
    }
  return s1 * s1 + s2;
}

// The sum of a 256-thread block's values (the shader sums its workgroup
// with a tree, film.wgsl:1099-1107; this is a tree too, by warp shuffles, then
// over the 8 warps): every thread gets the total.
__device__ __forceinline__ float block_tree(float* sv, float v) {
  const uint32_t li = threadIdx.y * 16u + threadIdx.x;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  __syncthreads();  // sv may still be read by a previous call
  if ((li & 31u) == 0u) sv[li >> 5] = v;
  __syncthreads();
  float t = sv[0];
#pragma unroll
  for (int w = 1; w < 8; ++w) t += sv[w];
  return t;
}

// Writes this block's tile partial(s), then reports whether it is the last
// block of the film to do so (the caller then sums the film's partials).  The
// count is two-level: a counter per group of 32 tiles, and the film's counter
// taken only by each group's last block, so no address takes more than a few
// hundred atomics per launch (one counter per film serialised 16 k atomics at
// 2048^2, tens of microseconds per launch).
__device__ __forceinline__ bool last_block(const Film& F, uint32_t t, float part, float part2, bool two) {
  __shared__ uint32_t s_last;
  if (threadIdx.x == 0 && threadIdx.y == 0) {
    F.cg_part[t] = part;
    if (two) F.cg_part2[t] = part2;
    __threadfence();
    const uint32_t nt = F.tw * F.th, g = t >> 5, ng = (nt + 31u) >> 5;
    const uint32_t in_group = min(32u, nt - (g << 5));
    s_last = 0u;
    if (atomicAdd(&F.cg_cnt[g], 1u) == in_group - 1u) {
      F.cg_cnt[g] = 0u;  // every block of the group has counted
      __threadfence();
      s_last = atomicAdd(&F.cg->blocks_done, 1u) == ng - 1u ? 1u : 0u;
    }
  }
  __syncthreads();
  if (s_last) __threadfence();
  return s_last != 0u;
}

// The film's total of the tile partials, by the last block: each thread's
// strided sum over the tiles in order, then the tree (as total_parts,
// film.wgsl:1157-1168, over every tile; inactive tiles add 0).
__device__ __forceinline__ float film_total(const Film& F, const float* part, float* sv) {
  const uint32_t li = threadIdx.y * 16u + threadIdx.x, nt = F.tw * F.th;
  float v = 0.f;
  for (uint32_t t = li; t < nt; t += 256u) v += __ldcg(part + t);
  return block_tree(sv, v);
}

#define CG_ARGS const Film* __restrict__ films, const uint2* __restrict__ tiles, uint32_t ntiles
#define CG_TILE                                                          \
  if (blockIdx.x >= ntiles) return;                                      \
  const uint2 pe_ = tile_entry(tiles, blockIdx.x);                       \
  const Film& F = films[pe_.x];                                          \
  const DevParams& D = *F.P;                                             \
  const cf_params& P = D.p;                                              \
  const uint32_t t = pe_.y;                                              \
  const int i = (int)((t % F.tw) * 16u + threadIdx.x);                   \
  const int j = (int)((t / F.tw) * 16u + threadIdx.y);                   \
  const bool tile_on = (F.tile_flags[t] & ACTIVE) != 0u;                 \
  const bool cell_on = tile_on && i < (int)F.w && j < (int)F.h;          \
  const uint32_t c = cell_on ? idx(F, i, j) : 0u;                        \
  (void)c;

// film.wgsl:935-987 (+ cg_lap_h, film.wgsl:1073-1078, when the implicit
// capillary term is on)
template <int MODE>
__global__ void __launch_bounds__(256) kp_cg_setup(CG_ARGS, uint32_t step) {
  CG_TILE
  if (step >= D.implicit_steps || !cell_on) return;
  float4 mob = make_float4(0.f, 0.f, 0.f, 0.f);
  const float2 p00 = pres_at(F, i, j);
  const float2 gxy = make_float2(P.phys[0] * P.g[0], P.phys[0] * P.g[1]);
  const float s2 = 0.70710678f;
  if (i + 1 < (int)F.w && cell_active(F, i + 1, j)) {
    const float2 p10 = pres_at(F, i + 1, j);
    const float2 gm = make_float2(-(p10.x - p00.x) * P.inv_dx, -(p10.y - p00.y) * P.inv_dx);
    const float2 a = pres_wet(F, i, j + 1, p00), b = pres_wet(F, i + 1, j + 1, p10);
    const float2 cc = pres_wet(F, i, j - 1, p00), d = pres_wet(F, i + 1, j - 1, p10);
    const float2 pt = make_float2(a.x + b.x - cc.x - d.x, a.y + b.y - cc.y - d.y);
    const float2 gt = make_float2(-pt.x * 0.25f * P.inv_dx, -pt.y * 0.25f * P.inv_dx);
    mob.x = face_mob<MODE>(F, P, c, idx(F, i + 1, j), make_float2(gm.x, gt.x), make_float2(gm.y, gt.y), gxy, false);
  }
  if (j + 1 < (int)F.h && cell_active(F, i, j + 1)) {
    const float2 p01 = pres_at(F, i, j + 1);
    const float2 gm = make_float2(-(p01.x - p00.x) * P.inv_dx, -(p01.y - p00.y) * P.inv_dx);
    const float2 a = pres_wet(F, i + 1, j, p00), b = pres_wet(F, i + 1, j + 1, p01);
    const float2 cc = pres_wet(F, i - 1, j, p00), d = pres_wet(F, i - 1, j + 1, p01);
    const float2 pt = make_float2(a.x + b.x - cc.x - d.x, a.y + b.y - cc.y - d.y);
    const float2 gt = make_float2(-pt.x * 0.25f * P.inv_dx, -pt.y * 0.25f * P.inv_dx);
    mob.y = face_mob<MODE>(F, P, c, idx(F, i, j + 1), make_float2(gm.x, gt.x), make_float2(gm.y, gt.y),
                           make_float2(gxy.y, gxy.x), false);
  }
  if (i + 1 < (int)F.w && j + 1 < (int)F.h && cell_active(F, i + 1, j + 1)) {
    const float2 p11 = pres_at(F, i + 1, j + 1);
    const float2 ga = make_float2(-(p11.x - p00.x) * P.inv_dx * s2, -(p11.y - p00.y) * P.inv_dx * s2);
    const float2 pa = pres_wet(F, i + 1, j, p00), pb = pres_wet(F, i, j + 1, p11);
    const float2 gp = make_float2(-(pa.x - pb.x) * P.inv_dx * s2, -(pa.y - pb.y) * P.inv_dx * s2);
    const float2 gt = make_float2((gxy.x + gxy.y) * s2, (gxy.x - gxy.y) * s2);
    mob.z = face_mob<MODE>(F, P, c, idx(F, i + 1, j + 1), make_float2(ga.x, gp.x), make_float2(ga.y, gp.y), gt,
                           true);
  }
  if (i + 1 < (int)F.w && j > 0 && cell_active(F, i + 1, j - 1)) {
    const float2 p1m = pres_at(F, i + 1, j - 1);
    const float2 ga = make_float2(-(p1m.x - p00.x) * P.inv_dx * s2, -(p1m.y - p00.y) * P.inv_dx * s2);
    const float2 pa = pres_wet(F, i + 1, j, p00), pb = pres_wet(F, i, j - 1, p1m);
    const float2 gp = make_float2(-(pa.x - pb.x) * P.inv_dx * s2, -(pa.y - pb.y) * P.inv_dx * s2);
    const float2 gt = make_float2((gxy.x - gxy.y) * s2, (gxy.x + gxy.y) * s2);
    mob.w = face_mob<MODE>(F, P, c, idx(F, i + 1, j - 1), make_float2(ga.x, gp.x), make_float2(ga.y, gp.y), gt,
                           true);
  }
  F.cg_m[c] = mob;
  if (P.front3[0] != 0.f) {  // cg_lap_h
    F.cg_t[c] = lap_w(F, i, j, c, [&](uint32_t n) { return F.hh[n]; });
    F.cg_t2[c] = lap_w(F, i, j, c, [&](uint32_t n) { return hold_u(F, P, n); });
  }
}

// film.wgsl:1110-1141 and cg_reduce_init (film.wgsl:1170-1176)
__global__ void __launch_bounds__(256) kp_cg_init(CG_ARGS, uint32_t step) {
  CG_TILE
  if (step >= D.implicit_steps) return;
  __shared__ float sv[256];
  float v = 0.f;
  if (cell_on) {
    const float k = kappa(P), hc = F.hh[c], uc = hold_u(F, P, c);
    float diag = 1.0f, b = hc, ax = hc;
    for (int f = 0; f < 8; ++f) {
      uint32_t nc;
      float mw;
      if (cg_nb(F, f, i, j, nc, mw)) {
        diag += k * mw;
        b += k * mw * (hold_u(F, P, nc) - uc);
        ax += k * mw * (hc - F.hh[nc]);
      }
    }
    if (hc > 0.f) {
      const float cc = P.front3[0];
      diag += cc * lap_diag(F, i, j);
      b -= cc * lap_w(F, i, j, c, [&](uint32_t n) { return F.cg_t2[n]; });
      ax += cc * lap_w(F, i, j, c, [&](uint32_t n) { return F.cg_t[n]; });
    }
    const float r = b - ax;
    F.cg_d[c] = diag;
    F.cg_x[c] = hc;
    F.cg_r[c] = r;
    F.cg_pa[c] = r / diag;
    v = r * r / diag;
  }
  const float part = block_tree(sv, v);
  if (last_block(F, t, part, 0.f, false)) {
    const float rz = film_total(F, F.cg_part, sv);
    if (threadIdx.x == 0 && threadIdx.y == 0) {
      CgState& S = *F.cg;
      S.rz = rz; S.pq = 0.f; S.alpha = 0.f; S.beta = 0.f;
      S.s1x = rz; S.dv = 0.f; S.tv = 0.f; S.s0x = 0.f;
      S.blocks_done = 0u;
    }
  }
}

// The search direction of iteration `it` at cell n: the init's one for it = 0,
// else r / d + beta p_{it-1} (film.wgsl:1150-1155); an inactive cell keeps the
// last one the reference left in cg_p.
__device__ __forceinline__ float dir_at(const Film& F, uint32_t n, bool active, uint32_t it, float beta,
                                        const float* prev) {
  if (!active) return F.cg_p[n];
  if (it == 0u) return prev[n];
  return F.cg_r[n] / F.cg_d[n] + beta * prev[n];
}

// cg_lap_p (film.wgsl:1066-1071), only with the implicit capillary term: it
// also forms the direction of the iteration (kp_cg_iter_a then reads it).
__global__ void __launch_bounds__(256) kp_cg_lap_p(CG_ARGS, uint32_t step, uint32_t it) {
  CG_TILE
  if (step >= D.implicit_steps || it >= D.implicit_iters || !cell_on) return;
  const float* prev = (it & 1u) || it == 0u ? F.cg_pa : F.cg_pb;  // p_{it-1}; the init's p for it = 0
  const float beta = F.cg->beta;
  auto p_of = [&](uint32_t n) {
    const int x = (int)(n % F.w), y = (int)(n / F.w);
    return dir_at(F, n, cell_active(F, x, y), it, beta, prev);
  };
  F.cg_t[c] = lap_w(F, i, j, c, p_of);
  F.cg_q[c] = p_of(c);  // the new direction, stored by kp_cg_iter_a
}

// cg_iter_a (film.wgsl:1109-1120, apply_a :1083-1094) and cg_reduce_a
// (film.wgsl:1214-1222); with the fused cg_iter_c of the previous iteration.
// Without the implicit capillary term, the block first stages the directions
// of its tile and a one-cell halo, and the mobilities of the tile and of its
// lower-left halo, in shared memory (coalesced loads; each cell then reads
// its 8 neighbours there).
__global__ void __launch_bounds__(256) kp_cg_iter_a(CG_ARGS, uint32_t step, uint32_t it, int from_lap) {
  CG_TILE
  if (step >= D.implicit_steps || it >= D.implicit_iters) return;
  __shared__ float sv[256];
  __shared__ float sp[18][18];
  __shared__ float4 sm[18][17];
  // p_it goes to cg_pa for even it, cg_pb for odd; p_{it-1} is in the other
  // (for it = 0 the init's direction, in cg_pa)
  const float* prev = (it & 1u) || it == 0u ? F.cg_pa : F.cg_pb;
  float* cur = (it & 1u) ? F.cg_pb : F.cg_pa;
  const float beta = F.cg->beta;
  float v = 0.f;
  if (!from_lap) {
    const int x0 = (int)(t % F.tw) * 16 - 1, y0 = (int)(t / F.tw) * 16 - 1;
    const int li = (int)(threadIdx.y * 16u + threadIdx.x);
    if (tile_on) {
      for (int e = li; e < 18 * 18; e += 256) {
        const int x = x0 + e % 18, y = y0 + e / 18;
        float pv = 0.f;
        float4 mv = make_float4(0.f, 0.f, 0.f, 0.f);
        if (x >= 0 && y >= 0 && x < (int)F.w && y < (int)F.h) {
          const uint32_t n = idx(F, x, y);
          // the loads of both cases are issued together (dir_at's choice after them)
          const bool act = cell_active(F, x, y);
          const float pp = prev[n], pk = F.cg_p[n];
          if (it == 0u) pv = act ? pp : pk;
          else {
            const float r = F.cg_r[n], d = F.cg_d[n];
            pv = act ? r / d + beta * pp : pk;
          }
          if (e % 18 < 17) mv = F.cg_m[n];
        }
        sp[e / 18][e % 18] = pv;
        if (e % 18 < 17) sm[e / 18][e % 18] = mv;
      }
    }
    __syncthreads();
    if (cell_on) {
      const int lx = (int)threadIdx.x + 1, ly = (int)threadIdx.y + 1;
      const float pc = sp[ly][lx];
      const float k = kappa(P);
      const int W = (int)F.w, H = (int)F.h;
      const float4 m0 = sm[ly][lx];
      float acc_v = pc;
      // the order of cg_nb (film.wgsl:994-1010)
      if (i + 1 < W && W_AXIS * m0.x > 0.f) acc_v += k * (W_AXIS * m0.x) * (pc - sp[ly][lx + 1]);
      if (j + 1 < H && W_AXIS * m0.y > 0.f) acc_v += k * (W_AXIS * m0.y) * (pc - sp[ly + 1][lx]);
      if (i + 1 < W && j + 1 < H && W_DIAG_LAP * m0.z > 0.f)
        acc_v += k * (W_DIAG_LAP * m0.z) * (pc - sp[ly + 1][lx + 1]);
      if (i + 1 < W && j > 0 && W_DIAG_LAP * m0.w > 0.f) acc_v += k * (W_DIAG_LAP * m0.w) * (pc - sp[ly - 1][lx + 1]);
      if (i > 0 && W_AXIS * sm[ly][lx - 1].x > 0.f) acc_v += k * (W_AXIS * sm[ly][lx - 1].x) * (pc - sp[ly][lx - 1]);
      if (j > 0 && W_AXIS * sm[ly - 1][lx].y > 0.f) acc_v += k * (W_AXIS * sm[ly - 1][lx].y) * (pc - sp[ly - 1][lx]);
      if (i > 0 && j > 0 && W_DIAG_LAP * sm[ly - 1][lx - 1].z > 0.f)
        acc_v += k * (W_DIAG_LAP * sm[ly - 1][lx - 1].z) * (pc - sp[ly - 1][lx - 1]);
      if (i > 0 && j + 1 < H && W_DIAG_LAP * sm[ly + 1][lx - 1].w > 0.f)
        acc_v += k * (W_DIAG_LAP * sm[ly + 1][lx - 1].w) * (pc - sp[ly + 1][lx - 1]);
      v = pc * acc_v;
      cur[c] = pc;  // other blocks read p_{it-1} from the other plane
      F.cg_q[c] = acc_v;
    }
  } else if (cell_on) {
    const float pc = F.cg_q[c];
    const float k = kappa(P);
    float acc_v = pc;
    for (int f = 0; f < 8; ++f) {
      uint32_t nc;
      float mw;
      if (cg_nb(F, f, i, j, nc, mw)) {
        const int x = (int)(nc % F.w), y = (int)(nc / F.w);
        const float pn = dir_at(F, nc, cell_active(F, x, y), it, beta, prev);
        acc_v += k * mw * (pc - pn);
      }
    }
    if (F.hh[c] > 0.f && P.front3[0] != 0.f)
      acc_v += P.front3[0] * lap_w(F, i, j, c, [&](uint32_t n) { return F.cg_t[n]; });
    v = pc * acc_v;
    cur[c] = pc;  // other blocks read p_{it-1} from the other plane
    F.cg_q[c] = acc_v;
  }
  const float part = block_tree(sv, v);
  if (threadIdx.x == 0 && threadIdx.y == 0) F.cg_part[t] = part;  // summed by kp_cg_scalars
}

// cg_iter_b (film.wgsl:1122-1135) and cg_reduce_b (film.wgsl:1224-1232)
__global__ void __launch_bounds__(256) kp_cg_iter_b(CG_ARGS, uint32_t step, uint32_t it) {
  CG_TILE
  if (step >= D.implicit_steps || it >= D.implicit_iters) return;
  __shared__ float sv[256];
  const float* cur = (it & 1u) ? F.cg_pb : F.cg_pa;
  const float alpha = F.cg->alpha;
  float v = 0.f;
  if (cell_on) {
    const float r = F.cg_r[c] - alpha * F.cg_q[c];
    F.cg_x[c] = F.cg_x[c] + alpha * cur[c];
    F.cg_r[c] = r;
    v = r * r / F.cg_d[c];
  }
  const float part = block_tree(sv, v);
  if (threadIdx.x == 0 && threadIdx.y == 0) F.cg_part[t] = part;  // summed by kp_cg_scalars
}

// cg_reduce_a (film.wgsl:1214-1222) after kp_cg_iter_a, cg_reduce_b
// (:1224-1232) after kp_cg_iter_b: one block per film sums its tile partials
// (each thread's strided sum in tile order, then the tree) and updates the
// film's scalars.  A separate launch instead of a last-block count: at 2048^2
// the fence and atomics of 16 k blocks made the iteration kernels several
// times slower than their loads.
__global__ void __launch_bounds__(256) kp_cg_scalars(const Film* __restrict__ films, uint32_t nfilms, uint32_t step,
                                                     uint32_t it, int after_b) {
  if (blockIdx.x >= nfilms) return;
  const Film& F = films[blockIdx.x];
  const DevParams& D = *F.P;
  if (step >= D.implicit_steps || it >= D.implicit_iters) return;
  __shared__ float sv[256];
  const float total = film_total(F, F.cg_part, sv);
  if (threadIdx.x == 0 && threadIdx.y == 0) {
    CgState& S = *F.cg;
    if (!after_b) {
      S.pq = total;
      S.alpha = total > 0.f ? S.rz / total : 0.f;
      S.beta = 0.f;
    } else {
      S.beta = S.rz > 0.f ? total / S.rz : 0.f;
      S.rz = total;
    }
  }
}

// cg_lap_u (film.wgsl:1080-1085), only with the implicit capillary term
__global__ void __launch_bounds__(256) kp_cg_lap_u(CG_ARGS, uint32_t step) {
  CG_TILE
  if (step >= D.implicit_steps || !cell_on) return;
  F.cg_t[c] = lap_w(F, i, j, c, [&](uint32_t n) { return F.cg_x[n] + hold_u(F, P, n); });
}

// film.wgsl:1227-1274 and cg_reduce_mass (film.wgsl:1190-1207).  The new h
// goes to cg_q (kp_cg_rescale commits it), so every read of a neighbour's h
// sees the h of before the dispatch.  The final direction of the solve (the
// reference's last cg_iter_c) is kept in cg_p for later steps' reads.
__global__ void __launch_bounds__(256) kp_cg_finish(CG_ARGS, uint32_t step) {
  CG_TILE
  if (step >= D.implicit_steps) return;
  __shared__ float sv[256], stv[256];
  __shared__ uint32_t s_moved;
  const uint32_t li = threadIdx.y * 16u + threadIdx.x;
  if (li == 0u) s_moved = 0u;
  __syncthreads();
  float dv = 0.f, tv = 0.f;
  if (cell_on) {
    const uint32_t last = D.implicit_iters - 1u;
    const float* plast = (last & 1u) ? F.cg_pb : F.cg_pa;
    F.cg_p[c] = F.cg_r[c] / F.cg_d[c] + F.cg->beta * plast[c];
    const float h0 = F.hh[c], hn = fmaxf(F.cg_x[c], 0.f);
    const float rg = P.phys[0] * P.g[2] * P.inv_dx;
    auto pot = [&](uint32_t n) { return F.cg_x[n] + hold_u(F, P, n); };  // film.wgsl:1227-1229
    const float pc = pot(c);
    float4 f = make_float4(0.f, 0.f, 0.f, 0.f);
    const float4 mob = F.cg_m[c];
    if (mob.x > 0.f) f.x = W_AXIS * mob.x * rg * (pc - pot(idx(F, i + 1, j)));
    if (mob.y > 0.f) f.y = W_AXIS * mob.y * rg * (pc - pot(idx(F, i, j + 1)));
    if (mob.z > 0.f) f.z = W_DIAG_FLUX * mob.z * rg * (pc - pot(idx(F, i + 1, j + 1))) * 0.70710678f;
    if (mob.w > 0.f) f.w = W_DIAG_FLUX * mob.w * rg * (pc - pot(idx(F, i + 1, j - 1))) * 0.70710678f;
    if (h0 > 0.f && P.front3[1] != 0.f) {
      const float kc = P.front3[1], tc = F.cg_t[c];
      auto wet_on = [&](int x, int y) { return F.hh[idx(F, x, y)] > 0.f && cell_active(F, x, y); };
      if (i + 1 < (int)F.w && wet_on(i + 1, j)) f.x += W_AXIS * kc * (F.cg_t[idx(F, i + 1, j)] - tc);
      if (j + 1 < (int)F.h && wet_on(i, j + 1)) f.y += W_AXIS * kc * (F.cg_t[idx(F, i, j + 1)] - tc);
      if (i + 1 < (int)F.w && j + 1 < (int)F.h && wet_on(i + 1, j + 1))
        f.z += W_DIAG_FLUX * kc * (F.cg_t[idx(F, i + 1, j + 1)] - tc) * 0.70710678f;
      if (i + 1 < (int)F.w && j > 0 && wet_on(i + 1, j - 1))
        f.w += W_DIAG_FLUX * kc * (F.cg_t[idx(F, i + 1, j - 1)] - tc) * 0.70710678f;
    }
    const float4 a = F.acc[c];
    const float fw = P.front[3];
    F.acc[c] = make_float4(a.x + f.x * fw, a.y + f.y * fw, a.z + f.z * fw, a.w + f.w * fw);
    F.cg_q[c] = hn;
    if (fabsf(hn - h0) > MOVE_EPS) s_moved = 1u;
    dv = hn - h0;
    tv = hn;
  }
  stv[li] = tv;
  const float part = block_tree(sv, dv);  // its barriers also publish stv and s_moved
  float part2 = 0.f;
  if (li == 0u) {
    for (int k = 0; k < 256; ++k) part2 += stv[k];  // thread 0's sequential sum (film.wgsl:1268-1272)
    if (s_moved) F.tile_moved[t] = 1u;
  }
  if (last_block(F, t, part, part2, true)) {
    const float sdv = film_total(F, F.cg_part, sv);
    const float stot = film_total(F, F.cg_part2, stv);
    if (li == 0u) {
      CgState& S = *F.cg;
      S.dv = sdv;
      S.tv = stot;
      S.s0x = S.rz;
      S.blocks_done = 0u;
    }
  }
}

// cg_rescale (film.wgsl:1179-1188) with the commit of cg_finish's h
__global__ void __launch_bounds__(256) kp_cg_rescale(CG_ARGS, uint32_t step) {
  CG_TILE
  if (step >= D.implicit_steps || !cell_on) return;
  const float hn = F.cg_q[c];
  const CgState& S = *F.cg;
  if (S.tv <= 0.f) {
    F.hh[c] = hn;
    return;
  }
  const float fr = 1.0f - S.dv / S.tv;
  F.hh[c] = fmaxf(hn * fr, 0.f);
}

}  // namespace

uint32_t launch_cg_step(const PackedFrame& V, int mode, uint32_t step, uint32_t iters, bool cap_implicit,
                        cudaStream_t st) {
  const Film* A = V.films;
  const uint2* T = V.tiles;
  const uint32_t nt = V.ntiles;
  const dim3 b(16, 16);
  uint32_t n = 0;
  if (mode == CF_PREC_REFERENCE) kp_cg_setup<CF_PREC_REFERENCE><<<nt, b, 0, st>>>(A, T, nt, step);
  else if (mode == CF_PREC_FP32) kp_cg_setup<CF_PREC_FP32><<<nt, b, 0, st>>>(A, T, nt, step);
  else kp_cg_setup<CF_PREC_BF16><<<nt, b, 0, st>>>(A, T, nt, step);
  kp_cg_init<<<nt, b, 0, st>>>(A, T, nt, step);
  n += 2;
  for (uint32_t it = 0; it < iters; ++it) {
    if (cap_implicit) { kp_cg_lap_p<<<nt, b, 0, st>>>(A, T, nt, step, it); ++n; }
    kp_cg_iter_a<<<nt, b, 0, st>>>(A, T, nt, step, it, cap_implicit ? 1 : 0);
    kp_cg_scalars<<<V.nfilms, b, 0, st>>>(A, V.nfilms, step, it, 0);
    kp_cg_iter_b<<<nt, b, 0, st>>>(A, T, nt, step, it);
    kp_cg_scalars<<<V.nfilms, b, 0, st>>>(A, V.nfilms, step, it, 1);
    n += 4;
  }
  if (cap_implicit) { kp_cg_lap_u<<<nt, b, 0, st>>>(A, T, nt, step); ++n; }
  kp_cg_finish<<<nt, b, 0, st>>>(A, T, nt, step);
  kp_cg_rescale<<<nt, b, 0, st>>>(A, T, nt, step);
  return n + 2;
}

}  // namespace cfk
