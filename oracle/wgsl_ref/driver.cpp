// driver.cpp — runs the mechanically translated reference shaders.
//
// TEST INFRASTRUCTURE.  Compiled (by build_ref.py, only where the reference
// checkout exists) together with the translation generated by translate.py
// into oracle/_ref/libwgslref.so.  It dispatches the translated WGSL entry
// points in the order of Film::encode_frame (src/film/mod.rs:1322-1462):
//  - tile-list dispatches iterate the active tiles that the translated
//    compact_tiles appended, 16x16 invocations each;
//  - full-grid dispatches (cure_step, shade_full) iterate every invocation;
//  - mark_tiles runs barrier phase by barrier phase;
//  - apply's begin/end_motion workgroup flag and reduce_tiles' shared-memory
//    tree (a max/min) are emulated here around the translated per-cell code;
//  - nose and strata_fill read `__old` snapshots (Jacobi semantics).
//  - deposits uploaded by wgr_set_deposits are laid by the translated
//    deposit entry point at the start of the next frame;
//  - the implicit hydrostatic CG steps (wgr_set_implicit) run after
//    clear_acc; their workgroup and single-workgroup sums are completed in the
//    shader's tree order, and cg_finish reads h as of before the dispatch.
// One film per process (the translated buffers are module globals).
#include <algorithm>
#include <array>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <string>
#include <type_traits>
#include <vector>

#include "../film_oracle.hpp"
#include "ref_shaders.inc"

// Workgroup-at-a-time definitions of the helpers whose barriers sit inside
// them (common.wgsl:112-120, film.wgsl:1099-1107 and 1157-1168): the driver
// runs a workgroup's 256 invocations one after the other, then finishes the
// barrier's work in the shader's order.
namespace wg {
u32 wg_flag = 0u, wg_slot = 0u;
bool wg_reduced = false;
void begin_motion(u32) {}
void end_motion(bool moved, vec3<u32>, u32) {
  if (moved) wg_flag = 1u;
}
void wg_reduce(u32 li, f32 v, u32 slot) {
  wg_sum[li] = v;
  wg_slot = slot;
  wg_reduced = true;
}
// the shader's tree: for s = 128, 64, .., 1: a[li] += a[li + s] for li < s
f32 tree_sum(array<f32, 256>& a) {
  for (u32 st = 128u; st > 0u; st >>= 1u)
    for (u32 li = 0; li < st; ++li) a[li] += a[li + st];
  return a[0];
}
// each invocation's strided sum of the tile partials, then the tree
f32 total_parts(u32) {
  const u32 n = active_count[0];
  for (u32 l = 0; l < 256u; ++l) {
    f32 v = f32(0);
    for (u32 t = l; t < n; t += 256u) v += cg_part[t];
    wg_sum[l] = v;
  }
  return tree_sum(wg_sum);
}
}  // namespace wg

using namespace wg;

namespace {
u32 W = 0, H = 0, TW = 0, TH = 0;
size_t N = 0;

template <class T>
void sz(RtBuf<T>& b, size_t n) { b.v.assign(n, T{}); }

void dispatch_tiles(void (*fn)(vec3<u32>, vec3<u32>)) {
  u32 n = active_count[0];
  for (u32 w = 0; w < n; ++w)
    for (u32 ly = 0; ly < 16; ++ly)
      for (u32 lx = 0; lx < 16; ++lx) fn(vec3<u32>(w, 0, 0), vec3<u32>(lx, ly, 0));
}

void dispatch_full(void (*fn)(vec3<u32>)) {
  for (u32 y = 0; y < TH * 16; ++y)
    for (u32 x = 0; x < TW * 16; ++x) fn(vec3<u32>(x, y, 0));
}

void run_mark_tiles() {
  for (u32 ty = 0; ty < TH; ++ty)
    for (u32 tx = 0; tx < TW; ++tx) {
      vec3<u32> wid(tx, ty, 0);
      for (int ph = 0; ph < 3; ++ph)
        for (u32 ly = 0; ly < 16; ++ly)
          for (u32 lx = 0; lx < 16; ++lx) {
            vec3<u32> lid(lx, ly, 0);
            u32 li = ly * 16 + lx;
            if (ph == 0) mark_tiles__p0(wid, lid, li);
            else if (ph == 1) mark_tiles__p1(wid, lid, li);
            else mark_tiles__p2(wid, lid, li);
          }
    }
}

void run_compact_tiles() {
  u32 nt = TW * TH;
  for (u32 x = 0; x < ((nt + 255) / 256) * 256; ++x) compact_tiles(vec3<u32>(x, 0, 0));
}

void run_apply() {
  u32 n = active_count[0];
  for (u32 w = 0; w < n; ++w) {
    bool any = false;
    for (u32 ly = 0; ly < 16; ++ly)
      for (u32 lx = 0; lx < 16; ++lx) {
        vec3<u32> id = tile_cell(vec3<u32>(w, 0, 0), vec3<u32>(lx, ly, 0));
        if (in_grid(id)) any = apply_cell(id) || any;
      }
    if (any) tile_moved[tile_list[w]] = 1u;
  }
}

void run_reduce_tiles() {
  u32 tw = P.tiles.x, th = P.tiles.y;
  for (u32 ty = 0; ty < th; ++ty)
    for (u32 tx = 0; tx < tw; ++tx) {
      f32 hm = 0, mm = f32(1e9f);
      for (u32 j = ty * 64; j < std::min(H, ty * 64 + 64); ++j)
        for (u32 i = tx * 64; i < std::min(W, tx * 64 + 64); ++i) {
          u32 c = idx(i, j);
          f32 v = h[c];
          if (v > f32(4.0f) * P.ein.w) { hm = std::max(hm, v); mm = std::min(mm, rheo[c].x); }
        }
      stats_out[tx + ty * tw] = vec2<f32>(hm, mm);
    }
}

void run_nose() {
  delta__old.v = delta.v;
  dispatch_tiles(nose);
}

void run_strata_fill() {
  strata_h__old.v = strata_h.v;
  strata_pig__old.v = strata_pig.v;
  strata_cure__old.v = strata_cure.v;
  dispatch_tiles(strata_fill);
}

bool dep_pending = false;  // deposits uploaded since the last frame
u32 impl_steps = 0u, impl_iters = 40u;  // Film::implicit_steps, FilmSettings::implicit_iters

// A tile-list dispatch of an entry with workgroup sums: invocations run in
// descending local index, so the li == 0 code after a barrier sees every
// invocation's workgroup writes; the partial of wg_reduce and the moved flag
// of end_motion are completed after each workgroup.
void dispatch_tiles_wg(void (*fn)(vec3<u32>, vec3<u32>, u32)) {
  u32 n = active_count[0];
  for (u32 w = 0; w < n; ++w) {
    wg_flag = 0u;
    wg_reduced = false;
    for (int li = 255; li >= 0; --li) fn(vec3<u32>(w, 0, 0), vec3<u32>((u32)li % 16u, (u32)li / 16u, 0), (u32)li);
    if (wg_reduced) cg_part[wg_slot] = tree_sum(wg_sum);
    if (wg_flag) tile_moved[tile_list[w]] = 1u;
  }
}

// single-workgroup reductions: invocation 0 writes
void dispatch_one(void (*fn)(u32)) {
  for (int li = 255; li >= 0; --li) fn((u32)li);
}

// cg_reduce_mass (film.wgsl:1190-1207): two strided sums and trees
void run_cg_reduce_mass() {
  const u32 n = active_count[0];
  array<f32, 256> a{}, b{};
  for (u32 l = 0; l < 256u; ++l) {
    f32 d = f32(0), tot = f32(0);
    for (u32 t = l; t < n; t += 256u) { d += cg_part[t]; tot += cg_part2[t]; }
    a[l] = d;
    b[l] = tot;
  }
  for (u32 st = 128u; st > 0u; st >>= 1u)
    for (u32 li = 0; li < st; ++li) { a[li] += a[li + st]; b[li] += b[li + st]; }
  const vec4<f32> s1 = cg_s[1];
  cg_s[1] = vec4<f32>(s1.x, a[0], b[0], cg_s[0].x);
}

// cg_finish writes h[c] while its neighbours' pot() reads h: the reads see
// the h of before the dispatch (Jacobi, as in the oracle).
void run_cg_finish() {
  std::vector<f32> h_old = h.v, h_new = h.v;
  u32 n = active_count[0];
  for (u32 w = 0; w < n; ++w) {
    wg_flag = 0u;
    wg_reduced = false;
    for (int li = 255; li >= 0; --li) {
      vec3<u32> wid(w, 0, 0), lid((u32)li % 16u, (u32)li / 16u, 0);
      cg_finish(wid, lid, (u32)li);
      vec3<u32> id = tile_cell(wid, lid);
      if (in_grid(id)) {
        u32 c = idx(id.x, id.y);
        h_new[c] = h[c];
        h[c] = h_old[c];
      }
    }
    if (wg_reduced) cg_part[wg_slot] = tree_sum(wg_sum);
    if (wg_flag) tile_moved[tile_list[w]] = 1u;
  }
  h.v = h_new;
}

// Film::encode_frame's implicit hydrostatic steps (src/film/mod.rs:1373-1408)
void run_implicit() {
  for (u32 s = 0; s < impl_steps; ++s) {
    dispatch_tiles(laplacian);
    dispatch_tiles(cg_setup);
    dispatch_tiles(cg_lap_h);
    dispatch_tiles_wg(cg_init);
    dispatch_one(cg_reduce_init);
    for (u32 it = 0; it < impl_iters; ++it) {
      dispatch_tiles(cg_lap_p);
      dispatch_tiles_wg(cg_iter_a);
      dispatch_one(cg_reduce_a);
      dispatch_tiles_wg(cg_iter_b);
      dispatch_one(cg_reduce_b);
      dispatch_tiles(cg_iter_c);
    }
    dispatch_tiles(cg_lap_u);
    run_cg_finish();
    run_cg_reduce_mass();
    dispatch_tiles(cg_rescale);
  }
}

void encode_frame(u32 substeps) {
  if (dep_pending) dispatch_full(deposit);  // the "pre" pass of Film::encode_frame
  dep_pending = false;
  active_count[0] = 0;
  run_mark_tiles();
  run_compact_tiles();
  dispatch_full(cure_step);
  dispatch_tiles(clear_acc);
  run_implicit();
  for (u32 s = 0; s < substeps; ++s) {
    dispatch_tiles(laplacian);
    dispatch_tiles(plug);
    dispatch_tiles(fluxes);
    dispatch_tiles(limiter);
    run_apply();
    run_nose();
  }
  dispatch_tiles(laplacian);
  dispatch_tiles(strata_split);
  run_reduce_tiles();
  dispatch_tiles(strata_limit);
  dispatch_tiles(strata_update);
  dispatch_tiles(strata_copy_back);
  for (int r = 0; r < 6; ++r) run_strata_fill();
  dispatch_full(shade_full);
}

f32 hv(uint16_t b) { return (f32)cfo::f16_value(b); }
uint16_t hb(double x) { return cfo::f16_bits(cfo::round_f16(x)); }

}  // namespace

extern "C" {

void wgr_create(uint32_t w, uint32_t h_) {
  W = w; H = h_; TW = (w + 15) / 16; TH = (h_ + 15) / 16; N = (size_t)w * h_;
  sz(h, N); sz(m, N); sz(rheo, N); sz(pres, N); sz(flux, N); sz(acc, N); sz(alpha, N); sz(delta, N);
  sz(tmp, N); sz(acc_s, 4 * N); sz(strata_h, N); sz(strata_pig, 8 * N); sz(strata_cure, N);
  sz(sub_refl, 8 * N); sz(pigtab, 12 * 40); sz(cmf, 48); sz(strata_h2, N); sz(strata_pig2, 8 * N);
  sz(alpha_s, N); sz(strata_cure2, N); sz(tile_flags, TW * TH); sz(tile_list, TW * TH);
  sz(active_count, 4); sz(tile_moved, TW * TH); sz(lay, N);
  sz(stats_out, ((w + 63) / 64) * ((h_ + 63) / 64)); sz(h_frame, N); sz(fnorm, N);
  sz(cg_m, N); sz(cg_d, N); sz(cg_x, N); sz(cg_r, N); sz(cg_p, N); sz(cg_q, N); sz(cg_t, N); sz(cg_t2, N);
  sz(cg_part, TW * TH); sz(cg_part2, TW * TH); sz(cg_s, 2);
  color_out.w = w; color_out.v.assign(N, vec4<f32>(f32(0)));
  detail_out.w = w; detail_out.v.assign(N, vec4<f32>(f32(0)));
}

void wgr_set_params(const cf_params* p) {
  P.size = vec2<u32>(p->size[0], p->size[1]);
  P.tiles = vec2<u32>(p->tiles[0], p->tiles[1]);
  P.dx = p->dx; P.dt = p->dt; P.inv_dx = p->inv_dx; P.frame_dt = p->frame_dt;
  auto v4 = [](const float* a) { return vec4<f32>(a[0], a[1], a[2], a[3]); };
  P.g = v4(p->g); P.phys = v4(p->phys); P.ein = v4(p->ein); P.cure = v4(p->cure); P.misc = v4(p->misc);
  P.flags = vec4<u32>(p->flags[0], p->flags[1], p->flags[2], p->flags[3]);
  P.front = v4(p->front); P.front2 = v4(p->front2); P.front3 = v4(p->front3);
}

void wgr_set_tables(const float* pt, const float* cm) {
  for (int i = 0; i < 480; ++i) pigtab[i] = pt[i];
  for (int i = 0; i < 48; ++i) cmf[i] = cm[i];
}

void wgr_encode_frame(uint32_t substeps) { encode_frame(substeps); }

// Film::implicit_steps (update_params) and FilmSettings::implicit_iters
void wgr_set_implicit(uint32_t steps, uint32_t iters) {
  impl_steps = steps;
  impl_iters = iters;
}

// write_state scratch clearing (src/film/mod.rs:1307-1317)
void wgr_after_write_state() {
  for (auto& v : pres.v) v = vec2<f32>(f32(0));
  for (auto& v : flux.v) v = vec4<f32>(f32(0));
  for (auto& v : acc.v) v = vec4<f32>(f32(0));
  for (auto& v : alpha.v) v = 0;
  for (auto& v : delta.v) v = 0;
  for (auto& v : tmp.v) v = 0;
  for (auto& v : acc_s.v) v = vec4<f32>(f32(0));
  for (auto& v : strata_h2.v) v = vec4<f32>(f32(0));
  for (auto& v : strata_pig2.v) v = vec4<u32>(0u);
  for (auto& v : alpha_s.v) v = vec4<f32>(f32(0));
  for (auto& v : tile_moved.v) v = 1u;
}

// Deposits for the next frame with their 64x64-cell tile tables, as the
// host's upload_deposits (src/film/mod.rs:1175-1224) writes them.
void wgr_set_deposits(const cf_deposit* d, uint32_t n, const uint32_t* start, const uint32_t* count, uint32_t nt,
                      const uint32_t* items, uint32_t ni) {
  deposits.v.assign(std::max(n, 1u), Deposit{});
  for (uint32_t k = 0; k < n; ++k) {
    Deposit& o = deposits.v[k];
    o.p0 = vec2<f32>(d[k].p0[0], d[k].p0[1]);
    o.p1 = vec2<f32>(d[k].p1[0], d[k].p1[1]);
    o.n0 = vec2<f32>(d[k].n0[0], d[k].n0[1]);
    o.n1 = vec2<f32>(d[k].n1[0], d[k].n1[1]);
    o.r0 = d[k].r0; o.r1 = d[k].r1; o.h0 = d[k].h0; o.vol = d[k].vol;
    o.kind = d[k].kind;
    o.pig0 = vec4<u32>(d[k].pig[0], d[k].pig[1], d[k].pig[2], d[k].pig[3]);
    o.pig1 = vec4<u32>(d[k].pig[4], d[k].pig[5], d[k].pig[6], d[k].pig[7]);
  }
  tile_start.v.assign(start, start + nt);
  tile_count.v.assign(count, count + nt);
  tile_items.v.assign(items, items + ni);
  if (ni == 0) tile_items.v.assign(1, 0u);
  dep_pending = ni > 0;
}

int wgr_run(const char* k) {
  std::string s(k);
  if (s == "mark_tiles") { active_count[0] = 0; run_mark_tiles(); }
  else if (s == "compact_tiles") run_compact_tiles();
  else if (s == "cure_step") dispatch_full(cure_step);
  else if (s == "clear_acc") dispatch_tiles(clear_acc);
  else if (s == "laplacian") dispatch_tiles(laplacian);
  else if (s == "plug") dispatch_tiles(plug);
  else if (s == "fluxes") dispatch_tiles(fluxes);
  else if (s == "limiter") dispatch_tiles(limiter);
  else if (s == "apply") run_apply();
  else if (s == "nose") run_nose();
  else if (s == "strata_split") dispatch_tiles(strata_split);
  else if (s == "reduce_tiles") run_reduce_tiles();
  else if (s == "strata_limit") dispatch_tiles(strata_limit);
  else if (s == "strata_update") dispatch_tiles(strata_update);
  else if (s == "strata_copy_back") dispatch_tiles(strata_copy_back);
  else if (s == "strata_fill") run_strata_fill();
  else if (s == "shade_full") dispatch_full(shade_full);
  else if (s == "deposit") dispatch_full(deposit);
  else return 0;
  return 1;
}

uint32_t wgr_active_count() { return active_count[0]; }

// Exchange a plane in the oracle's layout (float64 values):
//  rheo 3/cell (mu, tau, n: n is not stored by the reference), strata_* 4/cell,
//  strata_pig 64 slots/cell, sub_refl 16 bands/cell, pres 2, flux/acc 4,
//  acc_s 16, fnorm 2, delta/tile words as integers, color 4/cell.
int wgr_buffer(const char* name, double* io, int write) {
  std::string n(name);
  auto scal = [&](RtBuf<f32>& b) {
    for (size_t i = 0; i < b.v.size(); ++i) { if (write) b.v[i] = (f32)io[i]; else io[i] = (double)b.v[i]; }
  };
  auto uns = [&](RtBuf<u32>& b) {
    for (size_t i = 0; i < b.v.size(); ++i) { if (write) b.v[i] = (u32)io[i]; else io[i] = (double)b.v[i]; }
  };
  auto v2 = [&](RtBuf<vec2<f32>>& b) {
    for (size_t i = 0; i < b.v.size(); ++i)
      for (int k = 0; k < 2; ++k) { if (write) b.v[i][k] = (f32)io[2 * i + k]; else io[2 * i + k] = (double)b.v[i][k]; }
  };
  auto v4 = [&](RtBuf<vec4<f32>>& b) {
    for (size_t i = 0; i < b.v.size(); ++i)
      for (int k = 0; k < 4; ++k) { if (write) b.v[i][k] = (f32)io[4 * i + k]; else io[4 * i + k] = (double)b.v[i][k]; }
  };
  auto halves = [&](auto& words, size_t per) {  // per = u32 words per cell
    for (size_t i = 0; i < words.size(); ++i)
      for (int k = 0; k < 2; ++k) {
        size_t slot = 2 * i + k;
        if (write) {
          uint16_t b = hb(io[slot]);
          words[i] = k == 0 ? ((words[i] & 0xffff0000u) | b) : ((words[i] & 0xffffu) | ((u32)b << 16));
        } else {
          io[slot] = (double)hv((uint16_t)(k == 0 ? (words[i] & 0xffffu) : (words[i] >> 16)));
        }
      }
    (void)per;
  };
  if (n == "h") scal(h);
  else if (n == "m") scal(m);
  else if (n == "alpha") scal(alpha);
  else if (n == "tmp") scal(tmp);
  else if (n == "h_frame") scal(h_frame);
  else if (n == "rheo") {
    for (size_t i = 0; i < N; ++i) {
      if (write) rheo.v[i] = vec2<f32>((f32)io[3 * i], (f32)io[3 * i + 1]);
      else { io[3 * i] = rheo.v[i].x; io[3 * i + 1] = rheo.v[i].y; io[3 * i + 2] = P.phys.z; }
    }
  }
  else if (n == "pres") v2(pres);
  else if (n == "fnorm") v2(fnorm);
  else if (n == "flux") v4(flux);
  else if (n == "acc") v4(acc);
  else if (n == "acc_s") v4(acc_s);
  else if (n == "alpha_s") v4(alpha_s);
  else if (n == "strata_h") v4(strata_h);
  else if (n == "strata_cure") v4(strata_cure);
  else if (n == "strata_h2") v4(strata_h2);
  else if (n == "strata_cure2") v4(strata_cure2);
  else if (n == "strata_pig" || n == "strata_pig2") {
    auto& b = n == "strata_pig" ? strata_pig : strata_pig2;
    std::vector<u32> words(b.v.size() * 4);
    for (size_t i = 0; i < b.v.size(); ++i) for (int k = 0; k < 4; ++k) words[4 * i + k] = b.v[i][k];
    halves(words, 32);
    if (write) for (size_t i = 0; i < b.v.size(); ++i) for (int k = 0; k < 4; ++k) b.v[i][k] = words[4 * i + k];
  }
  else if (n == "sub_refl") halves(sub_refl.v, 8);
  else if (n == "delta") {
    for (size_t i = 0; i < N; ++i) {
      if (write) delta.v[i] = bitcast<f32>((u32)io[i]);
      else io[i] = (double)bitcast<u32>(delta.v[i]);
    }
  }
  else if (n == "lay") uns(lay);
  else if (n == "tile_flags") uns(tile_flags);
  else if (n == "tile_moved") uns(tile_moved);
  else if (n == "stats") {
    for (size_t i = 0; i < stats_out.v.size(); ++i)
      for (int k = 0; k < 2; ++k) { if (write) stats_out.v[i][k] = (f32)io[2 * i + k]; else io[2 * i + k] = stats_out.v[i][k]; }
  }
  else if (n == "color") {
    for (size_t i = 0; i < N; ++i)
      for (int k = 0; k < 4; ++k) { if (write) color_out.v[i][k] = (f32)io[4 * i + k]; else io[4 * i + k] = color_out.v[i][k]; }
  }
  else return 0;
  return 1;
}

}  // extern "C"
