// film_oracle.hpp — CPU restatement of the Canvaz thin-film step.
//
// TEST INFRASTRUCTURE.  This is the oracle that the CUDA product is checked
// against; it is never linked into the product library and never runs on the
// product path.  Only tests/, __graft_entry__.smoke() and bench.py's CPU
// baseline may load it.
//
// It restates, function by function and in the dispatch order of
// Film::encode_frame (src/film/mod.rs:1322-1462), the WGSL entry points of
//   shaders/common.wgsl, shaders/film.wgsl (explicit path), shaders/strata.wgsl,
//   shaders/cure.wgsl, shaders/km.wgsl, shaders/shade.wgsl
// and the host parameter packing of src/film/mod.rs:861-933.
// `R` is the arithmetic type: double gives the FP64 oracle, float the FP32
// mirror of the reference (the CPU baseline).  Parameters are packed in f32
// exactly as the reference does, then widened to R.
//
// Pinning: the reference has no golden vectors for this path.  The oracle is
// pinned against a mechanical WGSL->C++ translation of the reference shaders
// (oracle/wgsl_ref/, run where the reference sources are present) through the
// fixtures in tests/golden/.
//
// Two reference dispatches read neighbour values that the same dispatch writes
// (nose: delta, film.wgsl:702-721; strata_fill: strata_*, strata.wgsl:307-315).
// On a GPU their result depends on scheduling; here both use Jacobi semantics
// (every invocation reads the values from before the dispatch).
//
// Extensions beyond the reference (both reduce to the reference exactly when
// unused):
//  - per-cell power-law index n: pigment slot 15 (> 0 overrides the global
//    P.phys.z), mixed like slot 14; a face uses the h-weighted mean of its two
//    cells' n (or the common value when they agree);
//  - storage precision of the pigment slots (f16 = reference, f32, bf16).
#pragma once

#include <algorithm>
#include <array>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#include "../include/canvaz_film.h"

namespace cfo {

// ---------------------------------------------------------------- rounding --

// Round to a binary format with `mant` fraction bits and minimum normal
// exponent `emin` (round to nearest even), saturating to +-inf above `maxv`.
inline double round_format(double x, int mant, int emin, double maxv) {
  if (x == 0.0 || !std::isfinite(x)) return x;
  int e;
  std::frexp(std::fabs(x), &e);  // |x| = f * 2^e, f in [0.5, 1)
  int lead = std::max(e - 1, emin);
  double q = std::ldexp(1.0, lead - mant);
  double r = std::nearbyint(x / q) * q;
  if (std::fabs(r) > maxv) return x > 0 ? INFINITY : -INFINITY;
  return r;
}
inline double round_f16(double x) { return round_format(x, 10, -14, 65504.0); }
inline double round_bf16(double x) { return round_format(x, 7, -126, 3.3895313892515355e38); }

inline uint16_t f16_bits(double x) {
  // x must already be representable in f16
  if (x == 0.0) return std::signbit(x) ? 0x8000 : 0;
  uint16_t s = std::signbit(x) ? 0x8000 : 0;
  double a = std::fabs(x);
  if (std::isinf(a)) return s | 0x7c00;
  if (std::isnan(a)) return 0x7e00;
  int e;
  double f = std::frexp(a, &e);  // a = f 2^e
  int E = e - 1;                  // a = 1.xxx 2^E
  if (E < -14) {                  // subnormal
    return s | (uint16_t)std::lround(a * std::ldexp(1.0, 24));
  }
  uint16_t mant = (uint16_t)std::lround((f * 2.0 - 1.0) * 1024.0);
  return s | (uint16_t)((E + 15) << 10) | mant;
}
inline double f16_value(uint16_t b) {
  int s = b >> 15, E = (b >> 10) & 31, M = b & 1023;
  double v;
  if (E == 0) v = std::ldexp((double)M, -24);
  else if (E == 31) v = M ? NAN : INFINITY;
  else v = std::ldexp(1.0 + M / 1024.0, E - 15);
  return s ? -v : v;
}

// Storage rounding of the value of pigment slot `slot`.  BF16 storage keeps
// slot 14 (the viscosity override ln mu + 10, 0 = none) as mu itself, so that
// slot rounds on mu (bfloat16 on ln mu + 10 would step by 0.0625 there).
inline double round_pig(double x, int mode, int slot) {
  if (mode == CF_PIG_F16) return round_f16(x);
  if (mode == CF_PIG_BF16) {
    if (slot == 14) return x > 0.0 ? std::log(round_bf16(std::exp(x - 10.0))) + 10.0 : 0.0;
    return round_bf16(x);
  }
  return (double)(float)x;
}

// ------------------------------------------------------------- constants --

constexpr int STRATA = 4, NPIG = 12, NB = 16, PIG_STRIDE = 40, SLOTS = 16;
constexpr uint32_t MOVED = 64u;      // film.wgsl:104
constexpr int WAKE_BAND = 8;         // film.wgsl:2
constexpr int PLUG_RADIUS = 3;       // film.wgsl:3

template <class R>
struct V2 {
  R x, y;
};

// ---------------------------------------------------------------- params --

// Params (src/film/mod.rs:5-23) packed in f32 exactly as update_params does.
struct ParamsF {
  cf_params p;
  uint32_t implicit_steps;
};

inline void settings_default(cf_settings* s) {
  // FilmSettings::default, src/film/mod.rs:315-350
  std::memset(s, 0, sizeof(*s));
  s->width_m = 1.2f; s->height_m = 0.8f; s->rho = 1000.0f; s->sigma = 0.035f;
  s->n_index = 1.0f; s->m_cap = 1.0e-8f; s->contact_angle_deg = 45.0f;
  s->hysteresis_deg = 15.0f; s->h_star = 2.0e-5f; s->raw_canvas = 1;
  s->weave_um = 25.0f; s->cure_rate = 1.0f / 600.0f; s->tau_cure = 300.0f;
  s->lnmu_cure = 5.0f; s->v_cap = 1.0f; s->tilt_deg = 0.0f; s->tilt_dir_deg = -90.0f;
  s->gravity = 9.81f; s->medium_mu = 0.08f; s->debug_view = 0; s->h_min = 1.5e-5f;
  s->m_cap_hydro = 1.0e-7f; s->max_substeps = 64; s->min_substeps = 4;
  s->implicit_iters = 40; s->implicit_hydro = 1; s->slump = 0; s->capillary = 1;
  s->capillary_implicit = 0; s->no_hold = 0; s->no_transl = 0; s->no_shape = 0;
  s->no_cap = 0; s->kshape = 1.0f; s->kline = 0.0f; s->hyst_deg = -1.0f;
  s->fcap_exp = 2.5f; s->cap_cond = 80.0f; s->all_active = 0;
}

inline float to_rad(float d) { return d * (3.14159265358979323846f / 180.0f); }

// Film::gravity_vec, src/film/mod.rs:861-867
inline void gravity_vec(const cf_settings& s, float g[3]) {
  float tilt = to_rad(s.tilt_deg), dir = to_rad(s.tilt_dir_deg);
  float gxy = s.gravity * std::sin(tilt);
  g[0] = gxy * std::cos(dir);
  g[1] = gxy * std::sin(dir);
  g[2] = std::max(s.gravity * std::cos(tilt), 0.0f);
}

// Film::update_params, src/film/mod.rs:869-917 (f32 arithmetic as in Rust).
// h_max / h_max_pending / mu_min are the host-side stats the reference keeps.
inline ParamsF update_params(const cf_settings& s, uint32_t W, uint32_t H, float frame_dt,
                             uint32_t substeps, float h_max, float h_max_pending, float mu_min) {
  ParamsF out;
  cf_params& P = out.p;
  std::memset(&P, 0, sizeof(P));
  float dx = s.width_m / (float)W;
  P.size[0] = W; P.size[1] = H;
  P.tiles[0] = (W + 63) / 64; P.tiles[1] = (H + 63) / 64;
  P.dx = dx; P.inv_dx = 1.0f / dx;
  float g[3];
  gravity_vec(s, g);
  float theta = to_rad(s.contact_angle_deg);
  float pi_a = 3.0f * s.sigma * (1.0f - std::cos(theta)) / s.h_star;
  float dt = frame_dt / (float)substeps;
  float m_cap_exp = 0.5f * dx * dx * dx * dx / (32.0f * s.sigma * dt);
  float m_cap = std::max(std::min(s.m_cap, m_cap_exp), 1e-14f);
  float m_exp = 0.1f * dx * dx / (dt * s.rho * std::max(g[2], 0.1f));
  P.dt = dt;
  P.frame_dt = frame_dt;
  P.g[0] = g[0]; P.g[1] = g[1]; P.g[2] = g[2]; P.g[3] = s.gravity;
  P.phys[0] = s.rho; P.phys[1] = s.sigma; P.phys[2] = s.n_index;
  P.phys[3] = (s.capillary && !s.no_cap) ? m_cap : 0.0f;
  float lc = std::sqrt(s.sigma / (s.rho * 9.81f));
  P.ein[0] = std::max(std::tan(theta), 0.05f);
  P.ein[1] = lc * std::sin(0.5f * theta);
  P.ein[2] = pi_a;
  P.ein[3] = s.h_min;
  P.cure[0] = s.cure_rate; P.cure[1] = s.tau_cure; P.cure[2] = s.lnmu_cure; P.cure[3] = s.h_star;
  P.misc[0] = 2.0e-6f; P.misc[1] = 0.12f; P.misc[2] = s.medium_mu;
  P.misc[3] = std::min(m_exp, s.m_cap_hydro);
  P.flags[0] = s.debug_view; P.flags[1] = (uint32_t)(s.slump != 0); P.flags[2] = 0; P.flags[3] = 0;
  float lc_z = std::sqrt(s.sigma / (s.rho * std::max(g[2], 0.1f)));
  float cap_explicit = std::min(m_exp, s.m_cap_hydro);
  float h_big = std::max(std::max(h_max, h_max_pending), 1e-4f);
  float m_phys = h_big * h_big * h_big / (3.0f * std::max(mu_min, 1e-3f)) - cap_explicit;
  float k_max = 40.0f;
  float kappa_frame = frame_dt * s.rho * std::max(g[2], 0.1f) / (dx * dx);
  uint32_t n_i = 0;
  if (m_phys > 0.0f) {
    float v = std::max(std::ceil(kappa_frame * m_phys / k_max), 1.0f);
    n_i = std::min((uint32_t)v, 4u);
  }
  float dt_i = frame_dt / (float)std::max(n_i, 1u);
  float m_imp_max = k_max * dx * dx / (dt_i * s.rho * std::max(g[2], 0.1f));
  out.implicit_steps = s.implicit_hydro ? n_i : 0;
  float m_phys_cap = h_big * h_big * h_big / (3.0f * std::max(mu_min, 1e-3f));
  float dx2 = dx * dx, dx4 = dx2 * dx2;  // powi(4)
  float m_cap_impl = (s.cap_cond / 28.0f) * dx4 / (dt_i * s.sigma);
  float m_c = s.capillary_implicit ? std::min(m_phys_cap, m_cap_impl) : 0.0f;
  float cc = dt_i * s.sigma * m_c / dx4;
  float kc = m_c * s.sigma / (dx * dx * dx);
  P.front3[0] = cc; P.front3[1] = kc; P.front3[2] = m_c; P.front3[3] = s.fcap_exp;
  P.front[0] = s.no_hold ? 0.0f : 2.0f * lc_z * std::sin(0.5f * theta);
  P.front[1] = dx / lc_z;
  P.front[2] = m_imp_max;
  P.front[3] = dt_i;
  float hyst = s.hyst_deg >= 0.0f ? s.hyst_deg : s.hysteresis_deg;
  uint32_t fl = (uint32_t)(s.no_transl != 0) | ((uint32_t)(s.no_shape != 0) << 1);
  P.front2[0] = to_rad(hyst); P.front2[1] = s.kshape; P.front2[2] = s.kline; P.front2[3] = (float)fl;
  return out;
}

// Film::choose_substeps, src/film/mod.rs:919-933
inline uint32_t choose_substeps(const cf_settings& s, uint32_t W, float frame_dt, float h_max_stat,
                                float h_max_pending, float mu_min_stat) {
  float g[3];
  gravity_vec(s, g);
  float dx = s.width_m / (float)W;
  float gxy = std::sqrt(g[0] * g[0] + g[1] * g[1]);
  float h_max = std::max(std::max(h_max_stat, h_max_pending), 1e-5f);
  float mu = std::max(mu_min_stat, 1e-3f);
  float speed = std::min(s.rho * gxy * h_max * h_max / mu, s.v_cap);
  float dt_cfl = speed > 1e-6f ? 0.5f * dx / speed : frame_dt;
  float mob = h_max * h_max * h_max / (3.0f * mu);
  uint32_t n_hyd = (uint32_t)std::max(std::ceil(frame_dt * s.rho * g[2] * std::min(mob, s.m_cap_hydro) / (0.2f * dx * dx)), 1.0f);
  float dx2 = dx * dx, dx4 = dx2 * dx2;
  uint32_t n_cap = (uint32_t)std::max(std::ceil(frame_dt * 32.0f * s.sigma * std::min(mob, s.m_cap) / dx4), 1.0f);
  uint32_t n_cfl = (uint32_t)std::max(std::ceil(frame_dt / dt_cfl), 1.0f);
  uint32_t n = std::max(std::max(n_cfl, n_hyd), n_cap);
  return std::min(std::max(n, s.min_substeps), s.max_substeps);
}

// Adaptive substep (extension, same formulas as choose_substeps, one substep
// per frame): dt = min(dt_max, dt_cfl, dt_hyd, dt_cap), f32 arithmetic.
inline float adaptive_dt(const cf_settings& s, uint32_t W, float dt_max, float h_max_stat, float mu_min_stat) {
  float g[3];
  gravity_vec(s, g);
  float dx = s.width_m / (float)W;
  float gxy = std::sqrt(g[0] * g[0] + g[1] * g[1]);
  float h_max = std::max(h_max_stat, 1e-5f);
  float mu = std::max(mu_min_stat, 1e-3f);
  float speed = std::min(s.rho * gxy * h_max * h_max / mu, s.v_cap);
  float dt = dt_max;
  if (speed > 1e-6f) dt = std::min(dt, 0.5f * dx / speed);
  float mob = h_max * h_max * h_max / (3.0f * mu);
  float hyd = s.rho * g[2] * std::min(mob, s.m_cap_hydro);
  if (hyd > 0.0f) dt = std::min(dt, 0.2f * dx * dx / hyd);
  float dx2 = dx * dx, dx4 = dx2 * dx2;
  float cap = 32.0f * s.sigma * std::min(mob, s.m_cap);
  if (cap > 0.0f) dt = std::min(dt, dx4 / cap);
  return dt;
}

// substrate_refl, src/film/mod.rs:188-210 (raw canvas or primed white)
inline void substrate_bands(int raw, float out[16]) {
  for (int b = 0; b < 16; ++b) {
    float t = (float)b / 15.0f;
    out[b] = raw ? 0.50f + 0.16f * t : 0.84f + 0.04f * t;
  }
}

// weave, src/film/mod.rs:212-233
inline void weave(uint32_t w, uint32_t h, float dx, float amp, float* out) {
  for (size_t i = 0; i < (size_t)w * h; ++i) out[i] = 0.0f;
  if (amp <= 0.0f) return;
  float period = 1.4e-3f;
  float k = 6.28318530717958647692f / period;
  for (uint32_t j = 0; j < h; ++j) {
    float y = ((float)j + 0.5f) * dx;
    for (uint32_t i = 0; i < w; ++i) {
      float x = ((float)i + 0.5f) * dx;
      uint32_t hsh = (i * 73856093u) ^ (j * 19349663u);
      hsh ^= hsh >> 13;
      hsh *= 0x5bd1e995u;
      hsh ^= hsh >> 15;
      float r = (float)(hsh & 0xffff) / 65535.0f * 2.0f - 1.0f;
      float sv = std::sin(k * x) * std::sin(k * y);
      out[(size_t)j * w + i] = amp * (1.0f + 0.6f * sv + 0.4f * r);
    }
  }
}

// ------------------------------------------------------------------ film --

template <class R>
struct Film {
  using V = V2<R>;
  struct Face { R q, y, up, n; };
  struct Stack { R th[4]; R cu[4]; R pg[4][16]; };

  uint32_t W, H, TW, TH;  // TW/TH: 16x16 activity tiles
  size_t N;
  int pig_mode;
  cf_settings S;
  ParamsF PF;
  float h_max_stat = 0.0f, mu_min_stat = 1.0f, h_max_pending = 0.0f;
  uint32_t active_tiles = 0;

  // Params widened to R
  R dx, dt, inv_dx, frame_dt, g[4], phys[4], ein[4], cure[4], misc[4], front[4], front2[4], front3[4];
  uint32_t flags[4];

  // tables
  std::vector<R> pigtab;  // 12 x 40
  std::vector<R> cmf;     // 16 x 3

  // persistent state (src/film/mod.rs:1277-1279)
  std::vector<R> h, m, rheo /*3N*/, sh /*4N*/, scu /*4N*/, pig /*64N*/, refl /*16N*/;
  std::vector<uint32_t> lay;
  // scratch that persists between dispatches (stale values are observable)
  std::vector<R> pres /*2N*/, flux /*4N*/, acc /*4N*/, alpha, tmp, acc_s /*16N*/, alpha_s /*4N*/;
  std::vector<R> sh2, scu2, pig2, h_frame, fnorm /*2N*/;
  std::vector<uint32_t> delta, tile_flags, tile_moved;
  std::vector<R> stats;  // 2 x tiles64
  std::vector<R> color;  // 4N
  std::vector<R> detail;  // 4N: the renderer's detail texel (shade.wgsl:61-64)

  Film(uint32_t w, uint32_t hh, const cf_settings& s, int pig_storage)
      : W(w), H(hh), TW((w + 15) / 16), TH((hh + 15) / 16), N((size_t)w * hh), pig_mode(pig_storage), S(s) {
    h.assign(N, 0); m.assign(N, 0); rheo.assign(3 * N, 0); sh.assign(4 * N, 0); scu.assign(4 * N, 0);
    pig.assign(64 * N, 0); refl.assign(16 * N, 0); lay.assign(N, 0);
    pres.assign(2 * N, 0); flux.assign(4 * N, 0); acc.assign(4 * N, 0); alpha.assign(N, 0); tmp.assign(N, 0);
    acc_s.assign(16 * N, 0); alpha_s.assign(4 * N, 0); sh2.assign(4 * N, 0); scu2.assign(4 * N, 0);
    pig2.assign(64 * N, 0); h_frame.assign(N, 0); fnorm.assign(2 * N, 0);
    delta.assign(N, 0); tile_flags.assign((size_t)TW * TH, 0); tile_moved.assign((size_t)TW * TH, 0);
    stats.assign(2 * (size_t)((w + 63) / 64) * ((hh + 63) / 64), 0);
    color.assign(4 * N, 0);
    detail.assign(4 * N, 0);
    pigtab.assign(NPIG * PIG_STRIDE, 0);
    cmf.assign(NB * 3, 0);
    // Film::new :686-693: substrate refl, weave relief, rheo = (1, 0)
    float bands[16];
    substrate_bands(s.raw_canvas, bands);
    for (size_t c = 0; c < N; ++c)
      for (int b = 0; b < 16; ++b) refl[16 * c + b] = (R)round_f16(bands[b]);
    std::vector<float> wv(N);
    weave(W, H, s.width_m / (float)W, s.weave_um * 1e-6f, wv.data());
    for (size_t c = 0; c < N; ++c) {
      m[c] = wv[c];
      rheo[3 * c] = 1; rheo[3 * c + 1] = 0; rheo[3 * c + 2] = s.n_index;
    }
    set_params(update_params(S, W, H, 1.0f / 60.0f, 1, 0.0f, 0.0f, 1.0f));
  }

  void set_params(const ParamsF& pf) {
    PF = pf;
    const cf_params& P = pf.p;
    dx = P.dx; dt = P.dt; inv_dx = P.inv_dx; frame_dt = P.frame_dt;
    for (int k = 0; k < 4; ++k) {
      g[k] = P.g[k]; phys[k] = P.phys[k]; ein[k] = P.ein[k]; cure[k] = P.cure[k]; misc[k] = P.misc[k];
      front[k] = P.front[k]; front2[k] = P.front2[k]; front3[k] = P.front3[k]; flags[k] = P.flags[k];
    }
  }

  void do_update_params(float fdt, uint32_t substeps) {
    set_params(update_params(S, W, H, fdt, substeps, h_max_stat, h_max_pending, mu_min_stat));
  }

  void set_tables(const float* pt, const float* cm) {
    for (int i = 0; i < NPIG * PIG_STRIDE; ++i) pigtab[i] = pt[i];
    for (int i = 0; i < NB * 3; ++i) cmf[i] = cm[i];
  }

  // Film::write_state :1303-1320 scratch clearing and tile marking
  void after_write_state() {
    std::fill(pres.begin(), pres.end(), R(0)); std::fill(flux.begin(), flux.end(), R(0));
    std::fill(acc.begin(), acc.end(), R(0)); std::fill(alpha.begin(), alpha.end(), R(0));
    std::fill(delta.begin(), delta.end(), 0u); std::fill(tmp.begin(), tmp.end(), R(0));
    std::fill(acc_s.begin(), acc_s.end(), R(0)); std::fill(sh2.begin(), sh2.end(), R(0));
    std::fill(pig2.begin(), pig2.end(), R(0)); std::fill(alpha_s.begin(), alpha_s.end(), R(0));
    std::fill(tile_moved.begin(), tile_moved.end(), 1u);
  }

  // ---------------------------------------------------------- helpers --
  static R F(float v) { return (R)v; }
  size_t idx(int i, int j) const { return (size_t)j * W + (size_t)i; }
  bool in_grid(int i, int j) const { return i >= 0 && j >= 0 && i < (int)W && j < (int)H; }
  static R len(R x, R y) { return std::sqrt(x * x + y * y); }
  static R sgn(R x) { return x > 0 ? R(1) : (x < 0 ? R(-1) : R(0)); }
  static R clampR(R x, R lo, R hi) { return std::min(std::max(x, lo), hi); }
  static R mixR(R a, R b, R t) { return a * (R(1) - t) + b * t; }
  static R smooth(R e0, R e1, R x) {
    R t = clampR((x - e0) / (e1 - e0), R(0), R(1));
    return t * t * (R(3) - R(2) * t);
  }
  R pig_store(R v, int slot) const { return (R)round_pig((double)v, pig_mode, slot); }

  // common.wgsl:140-171
  bool cell_active(int i, int j) const {
    return (tile_flags[(size_t)(i / 16) + (size_t)(j / 16) * TW] & 32u) != 0u;
  }
  int refl_i(int i) const {
    int w = (int)W, r = i;
    if (r < 0) r = -r - 1;
    if (r >= w) r = 2 * w - r - 1;
    return std::min(std::max(r, 0), w - 1);
  }
  int refl_j(int j) const {
    int hh = (int)H, r = j;
    if (r < 0) r = -r - 1;
    if (r >= hh) r = 2 * hh - r - 1;
    return std::min(std::max(r, 0), hh - 1);
  }
  // common.wgsl:190-195
  R disjoining(R hv) const {
    R hs = cure[3], a = ein[2];
    R x = std::max(R(1) - hv / hs, R(0));
    return a * x * x;
  }

  // film.wgsl:570-585 packed offset to the nearest dry cell
  static uint32_t pack_off(int ddx, int ddy) {
    uint32_t ux = (uint32_t)std::min(std::max(ddx + 128, 0), 255);
    uint32_t uy = (uint32_t)std::min(std::max(ddy + 128, 0), 255);
    return (ux << 8) | uy | 0x10000u;
  }
  static void unpack_off(uint32_t bits, int& ox, int& oy) {
    if ((bits & 0x10000u) == 0u) { ox = 64; oy = 64; return; }
    ox = (int)((bits >> 8) & 0xffu) - 128;
    oy = (int)(bits & 0xffu) - 128;
  }
  R nose_dist(size_t c) const {
    int ox, oy;
    unpack_off(delta[c], ox, oy);
    return len((R)ox, (R)oy);
  }
  // film.wgsl:153-156
  R hold_level(R d) const { return front[0] * (R(1) - std::exp(-(std::max(d, R(1)) - F(0.5f)) * front[1])); }
  // film.wgsl:147-151
  R usurf(int i, int j) const {
    size_t c = idx(refl_i(i), refl_j(j));
    R hold = 0;
    if (h[c] > 0) hold = hold_level(nose_dist(c));
    return h[c] + m[c] - hold;
  }
  V fn(size_t c) const { return V{fnorm[2 * c], fnorm[2 * c + 1]}; }
  V pr(size_t c) const { return V{pres[2 * c], pres[2 * c + 1]}; }

  // film.wgsl:190-201
  R line_pressure(size_t c) const {
    int i = (int)(c % W), j = (int)(c / W);
    if (i < 1 || j < 1 || i + 1 >= (int)W || j + 1 >= (int)H) return 0;
    V nl = fn(idx(i - 1, j)), nr = fn(idx(i + 1, j)), nd = fn(idx(i, j - 1)), nu = fn(idx(i, j + 1));
    if (nl.x * nl.x + nl.y * nl.y < F(0.5f) || nr.x * nr.x + nr.y * nr.y < F(0.5f) ||
        nd.x * nd.x + nd.y * nd.y < F(0.5f) || nu.x * nu.x + nu.y * nu.y < F(0.5f))
      return 0;
    R curv = (nr.x - nl.x + nu.y - nd.y) * F(0.5f) * inv_dx;
    return phys[1] * curv * front2[2];
  }

  // film.wgsl:16-42 laplacian
  void k_laplacian_cell(int i, int j) {
    size_t c = idx(i, j);
    R hv = h[c];
    R s0 = hv + m[c];
    R hold = 0, pl = 0;
    if (hv > 0) hold = hold_level(nose_dist(c));
    R u0 = s0 - hold;
    R ax = usurf(i - 1, j) + usurf(i + 1, j) + usurf(i, j - 1) + usurf(i, j + 1);
    R dg = usurf(i - 1, j - 1) + usurf(i + 1, j - 1) + usurf(i - 1, j + 1) + usurf(i + 1, j + 1);
    const R WA = F(0.6666667f), WL = F(0.16666667f);
    R l = (WA * ax + WL * dg - (F(4.0f) * WA + F(4.0f) * WL) * u0) * inv_dx * inv_dx;
    if (hv > 0) {
      R d = nose_dist(c);
      if (d <= R(3)) {
        V n = fn(c);
        if (n.x * n.x + n.y * n.y > F(0.5f)) pl = line_pressure(c) * std::exp(-(d - R(1)) * F(0.7f));
      }
    }
    pres[2 * c] = -phys[1] * l + disjoining(hv);
    pres[2 * c + 1] = phys[0] * g[2] * (s0 - hold) + pl;
  }

  // film.wgsl:94-107 (n is the power-law index of the evaluation)
  void hb_flux(R gmag, R hf, R mu, R ty, R n, R out[3]) const {
    out[0] = out[1] = out[2] = 0;
    if (gmag < F(1e-9f) || hf <= 0) return;
    R y = std::max(hf - ty / gmag, R(0));
    if (y <= 0) return;
    R up;
    if (std::fabs(n - R(1)) < F(1e-4f)) up = F(0.5f) * gmag / mu * y * y;
    else up = n / (n + R(1)) * std::pow(gmag / mu, R(1) / n) * std::pow(y, (n + R(1)) / n);
    R q = up * (hf - n * y / (R(2) * n + R(1)));
    out[0] = q; out[1] = y; out[2] = up;
  }
  // film.wgsl:109-126
  R band_flux(R up, R y, R za, R zb, R n) const {
    R ta = 0, tb = 0;
    if (y > 0) {
      R ra = std::max(y - za, R(0)) / y;
      R rb = std::max(y - zb, R(0)) / y;
      if (std::fabs(n - R(1)) < F(1e-4f)) { ta = ra * ra * ra; tb = rb * rb * rb; }
      else {
        R e = (R(2) * n + R(1)) / n;
        ta = std::pow(ra, e);
        tb = std::pow(rb, e);
      }
    }
    return up * ((zb - za) - n / (R(2) * n + R(1)) * y * (ta - tb));
  }

  // Per-cell flow index (extension): rheo plane component 2.
  R cell_n(size_t c) const { return rheo[3 * c + 2]; }

  // film.wgsl:58-87 plug
  void k_plug_cell(int i, int j) {
    size_t c = idx(i, j);
    tmp[c] = 0;
    if (h[c] <= 0) return;
    R gb = phys[0] * len(g[0], g[1]);
    if (gb < F(1e-6f)) return;
    R sum = 0, mass = 0;
    bool yielding = false;
    for (int dy = -PLUG_RADIUS; dy <= PLUG_RADIUS; ++dy)
      for (int dxi = -PLUG_RADIUS; dxi <= PLUG_RADIUS; ++dxi) {
        int x = i + dxi, y = j + dy;
        if (!in_grid(x, y)) continue;
        size_t n = idx(x, y);
        R hn = h[n];
        if (hn <= 0) continue;
        R rx = rheo[3 * n], ry = rheo[3 * n + 1];
        if (ry > 0) yielding = true;
        R q[3];
        hb_flux(gb, hn, std::max(rx, F(1e-4f)), ry, cell_n(n), q);
        sum += q[0];
        mass += hn;
      }
    if (!yielding || mass <= 0) return;
    tmp[c] = sum / mass;
  }

  // film.wgsl:44-49
  V yield_cap(V gc, R ty) const {
    R gcl = len(gc.x, gc.y);
    R gc_max = phys[1] / (F(1e-3f) * F(1e-3f));
    if (ty <= 0 || gcl <= gc_max) return gc;
    return V{gc.x * (gc_max / gcl), gc.y * (gc_max / gcl)};
  }
  // film.wgsl:51-56
  R plug_mobility(size_t ca, size_t cb, V gt) const {
    R gb = len(gt.x, gt.y);
    if (gb < F(1e-6f)) return 0;
    size_t up = gt.x >= 0 ? ca : cb;
    return tmp[up] * h[up] / gb;
  }
  // film.wgsl:89-92
  R yield_depth(size_t ca, size_t cb, R hf, R ty, V gg) const {
    if (ty <= 0) return hf;
    return gg.x >= 0 ? h[ca] : h[cb];
  }
  // film.wgsl:134-145
  uint32_t feeders(size_t c) const {
    int i = (int)(c % W), j = (int)(c / W);
    R thr = R(2) * h[c] + ein[3];
    uint32_t n = 0;
    if (i > 0 && h[idx(i - 1, j)] > thr) n++;
    if (i + 1 < (int)W && h[idx(i + 1, j)] > thr) n++;
    if (j > 0 && h[idx(i, j - 1)] > thr) n++;
    if (j + 1 < (int)H && h[idx(i, j + 1)] > thr) n++;
    return n;
  }
  // film.wgsl:160-180
  V front_normal(size_t c) const {
    int i = (int)(c % W), j = (int)(c / W);
    R dxs = 0, dys = 0;
    for (int dj = -2; dj <= 2; ++dj)
      for (int di = -2; di <= 2; ++di) {
        if (di == 0 && dj == 0) continue;
        int x = i + di, y = j + dj;
        if (!in_grid(x, y)) continue;
        if (di * di + dj * dj > 5) continue;
        if (h[idx(x, y)] <= ein[3]) {
          R dd = (R)(di * di + dj * dj);
          dxs += (R)di / dd;
          dys += (R)dj / dd;
        }
      }
    R l = len(dxs, dys);
    if (l < F(1e-6f)) return V{0, 0};
    return V{dxs / l, dys / l};
  }
  // film.wgsl:182-188
  R wet_gain(V n) const {
    const R s2 = F(0.70710678f), WA = F(0.6666667f), WD = F(0.23570226f);
    R w = WA * (std::max(n.x, R(0)) + std::max(-n.x, R(0)) + std::max(n.y, R(0)) + std::max(-n.y, R(0)));
    w += WD * (std::max(s2 * (n.x + n.y), R(0)) + std::max(-s2 * (n.x + n.y), R(0)) +
               std::max(s2 * (n.x - n.y), R(0)) + std::max(-s2 * (n.x - n.y), R(0)));
    R mm = std::max(std::max(std::fabs(n.x), std::fabs(n.y)), F(1e-3f));
    return R(1) / (mm * std::max(w, F(1e-3f)));
  }
  // film.wgsl:203-222
  R front_shape(size_t c, V n) const {
    int i = (int)(c % W), j = (int)(c / W);
    R w = 0, w0 = 0;
    for (int dj = -3; dj <= 3; ++dj)
      for (int di = -3; di <= 3; ++di) {
        if (di == 0 && dj == 0) continue;
        if (di * di + dj * dj > 9) continue;
        if ((R)di * n.x + (R)dj * n.y < F(-0.5f)) w0 += R(1);
        int x = i + di, y = j + dj;
        if (!in_grid(x, y)) continue;
        if (h[idx(x, y)] > ein[3]) w += R(1);
      }
    if (w0 < R(1) || ((uint32_t)front2[3] & 2u) != 0u) return 1;
    return std::pow(clampR(w / w0, R(0), F(2.5f)), front2[1]);
  }
  // film.wgsl:224-229
  R wet_threshold(size_t c) const {
    R ty = rheo[3 * c + 1];
    R need = std::max(ty / (phys[0] * std::max(h[c], F(1e-4f))) - len(g[0], g[1]), R(0));
    R ycap = need / std::max(g[2], F(1e-3f)) * dx;
    return std::max(hold_level(R(1)), ycap);
  }
  R front_dist(size_t c) const {  // film.wgsl:231-234
    if (h[c] <= 0) return 0;
    return nose_dist(c);
  }
  // film.wgsl:236-244
  R cox_speed(R excess, R mu) const {
    if (excess <= 0) return 0;
    R theta = std::atan(ein[0]);
    R span = std::max(front[0] - hold_level(R(1)), F(1e-6f));
    R th = theta + (F(3.14159265f) - theta) * clampR(excess / span, R(0), R(1));
    R adv = std::min(theta + front2[0], F(3.1f));
    if (th <= adv) return 0;
    return phys[1] * (th * th * th - adv * adv * adv) / (F(132.0f) * std::max(mu, F(1e-4f)));
  }
  // film.wgsl:246-265
  R cell_excess(size_t c) const {
    R e = h[c] - hold_level(front_dist(c));
    int ox, oy;
    unpack_off(delta[c], ox, oy);
    R ol = len((R)ox, (R)oy);
    if (ol > F(0.5f) && ol < F(60.0f)) {
      R dirx = (R)ox * (R(-1) / ol), diry = (R)oy * (R(-1) / ol);
      R bx = F(0.5f) * sgn((R)(-ox)), by = F(0.5f) * sgn((R)(-oy));
      int ci = (int)(c % W), cj = (int)(c / W);
      for (uint32_t k = 0; k < 3; ++k) {
        R reach = (R)(4u << k);
        int sx = (int)(dirx * reach + bx), sy = (int)(diry * reach + by);  // truncation toward zero
        int ri = ci + sx, rj = cj + sy;
        if (!in_grid(ri, rj)) break;
        size_t cr = idx(ri, rj);
        if (h[cr] <= 0) break;
        e = std::max(e, h[cr] - hold_level(front_dist(cr)));
      }
    }
    return e;
  }
  // film.wgsl:267-295 → (speed term, direction sign)
  V rim_translation(size_t ca, size_t cb, R hf, V fd) const {
    if (((uint32_t)front2[3] & 1u) != 0u) return V{0, 0};
    R da = front_dist(ca), db = front_dist(cb);
    if (std::max(da, db) > R(3) / front[1]) return V{0, 0};
    V n{0, 0};
    if (da > db && h[ca] > 0) n = fn(ca);
    else if (db > da && h[cb] > 0) n = fn(cb);
    else {
      if (h[ca] > 0) { V a = fn(ca); n.x += a.x; n.y += a.y; }
      if (h[cb] > 0) { V b = fn(cb); n.x += b.x; n.y += b.y; }
    }
    R nl = len(n.x, n.y);
    if (nl < F(1e-6f)) return V{0, 0};
    n.x = n.x / nl; n.y = n.y / nl;
    R s = n.x * fd.x + n.y * fd.y;
    if (std::fabs(s) < F(1e-4f)) return V{0, 0};
    size_t src = ca, dst = cb;
    if (s < 0) { src = cb; dst = ca; }
    if (h[src] <= 0) return V{0, 0};
    R e = cell_excess(src);
    if (e <= 0) return V{0, 0};
    R e_out = -hold_level(R(1));
    if (h[dst] > 0) e_out = cell_excess(dst);
    R room = clampR(R(1) - std::max(e_out, R(0)) / e, R(0), R(1));
    R u = cox_speed(e, rheo[3 * src]);
    return V{u * hf * room * mixR(R(1), std::fabs(s), front2[0]), sgn(s)};
  }

  // film.wgsl:297-372
  Face face(size_t ca, size_t cb, V gcap, V ghyd, V gtilt, bool diag, V fd) const {
    Face out{0, 0, 0, 0};
    R ha = h[ca], hb = h[cb];
    R hf = F(0.5f) * (ha + hb);
    if (hf <= 0) return out;
    R shape = 1, proj = 1;
    bool wetting = false;
    if (std::min(ha, hb) <= 0) {
      size_t wet = ha > 0 ? ca : cb;
      size_t dry = ha > 0 ? cb : ca;
      if (h[wet] <= wet_threshold(wet)) return out;
      wetting = true;
      V n = fn(wet);
      if (n.x * n.x + n.y * n.y < F(0.5f)) n = front_normal(wet);
      R toward = ha > 0 ? R(1) : R(-1);
      proj = std::max(n.x * (fd.x * toward) + n.y * (fd.y * toward), R(0));
      if (proj <= 0) return out;
      shape = front_shape(dry, n) * wet_gain(n);
      if (shape <= 0) return out;
    }
    R rax = rheo[3 * ca], ray = rheo[3 * ca + 1], rbx = rheo[3 * cb], rby = rheo[3 * cb + 1];
    R wa = ha / (ha + hb);
    R wb = R(1) - wa;
    R mu = std::exp(wa * std::log(std::max(rax, F(1e-4f))) + wb * std::log(std::max(rbx, F(1e-4f))));
    R ty = wa * ray + wb * rby;
    R na = cell_n(ca), nb = cell_n(cb);
    R nf = na == nb ? na : wa * na + wb * nb;
    R thin = std::min(ha, hb) / hf;
    R fcap = thin * thin * thin;
    V yc = yield_cap(V{gcap.x * fcap, gcap.y * fcap}, ty);
    V gg{yc.x + ghyd.x + gtilt.x, yc.y + ghyd.y + gtilt.y};
    R gmag = len(gg.x, gg.y);
    R qy[3];
    hb_flux(gmag, yield_depth(ca, cb, hf, ty, gg), mu, ty, nf, qy);
    R meff = qy[0] > 0 ? qy[0] / std::max(gmag, F(1e-9f)) : R(0);
    R mtilt = meff;
    if (ty > 0) mtilt = plug_mobility(ca, cb, gtilt);
    if (meff <= 0 && mtilt <= 0) return out;
    R fcap2 = std::pow(thin, front3[3]);
    R qn = mtilt * gtilt.x + std::min(meff, misc[3]) * ghyd.x + std::min(meff, phys[3]) * (gcap.x * fcap2);
    V tr = rim_translation(ca, cb, hf, fd);
    const R vcap = 2;
    if (wetting) {
      size_t wet = ha > 0 ? ca : cb;
      R want = tr.x * R(2) * h[wet] / std::max(hf, F(1e-9f));
      qn = tr.y * std::max(qn * tr.y * proj, want) * shape;
      if (std::fabs(qn) > vcap * hf) qn = sgn(qn) * vcap * hf;
    } else {
      if (tr.x > 0) qn = tr.y * std::max(qn * tr.y, tr.x);
      if (std::fabs(qn) > vcap * hf) qn = sgn(qn) * vcap * hf;
      R lo = std::min(ha, hb), hi = std::max(ha, hb);
      if (lo < F(0.5f) * hi) {
        if (diag) qn = 0;
        else {
          size_t tgt = cb;
          if (hb > ha) tgt = ca;
          uint32_t nf2 = feeders(tgt);
          qn = qn / std::pow((R)std::max(nf2, 1u), F(0.7f));
        }
      }
    }
    out.q = qn; out.y = qy[1]; out.up = qy[2]; out.n = nf;
    return out;
  }

  V pressure_at(int i, int j) const { return pr(idx(refl_i(i), refl_j(j))); }
  V pressure_wet(int i, int j, V fb) const {
    size_t c = idx(refl_i(i), refl_j(j));
    V p = pr(c);
    if (h[c] > 0) return p;
    return V{fb.x, p.y};
  }

  // film.wgsl:375-446
  void face_pair(int i, int j, Face ff[4]) const {
    size_t c = idx(i, j);
    for (int k = 0; k < 4; ++k) ff[k] = Face{0, 0, 0, 0};
    V p00 = pressure_at(i, j);
    V gxy{phys[0] * g[0], phys[0] * g[1]};
    const R s2 = F(0.70710678f), wa = F(0.6666667f), wd = F(0.23570226f);
    if (i + 1 < (int)W && cell_active(i + 1, j)) {
      size_t cb = idx(i + 1, j);
      V p10 = pressure_at(i + 1, j);
      V gm{-(p10.x - p00.x) * inv_dx, -(p10.y - p00.y) * inv_dx};
      V a = pressure_wet(i, j + 1, p00), b = pressure_wet(i + 1, j + 1, p10);
      V cc = pressure_wet(i, j - 1, p00), d = pressure_wet(i + 1, j - 1, p10);
      V pt{a.x + b.x - cc.x - d.x, a.y + b.y - cc.y - d.y};
      V gt{-pt.x * F(0.25f) * inv_dx, -pt.y * F(0.25f) * inv_dx};
      ff[0] = face(c, cb, V{gm.x, gt.x}, V{gm.y, gt.y}, gxy, false, V{1, 0});
      ff[0].q *= wa;
    }
    if (j + 1 < (int)H && cell_active(i, j + 1)) {
      size_t cb = idx(i, j + 1);
      V p01 = pressure_at(i, j + 1);
      V gm{-(p01.x - p00.x) * inv_dx, -(p01.y - p00.y) * inv_dx};
      V a = pressure_wet(i + 1, j, p00), b = pressure_wet(i + 1, j + 1, p01);
      V cc = pressure_wet(i - 1, j, p00), d = pressure_wet(i - 1, j + 1, p01);
      V pt{a.x + b.x - cc.x - d.x, a.y + b.y - cc.y - d.y};
      V gt{-pt.x * F(0.25f) * inv_dx, -pt.y * F(0.25f) * inv_dx};
      ff[1] = face(c, cb, V{gm.x, gt.x}, V{gm.y, gt.y}, V{gxy.y, gxy.x}, false, V{0, 1});
      ff[1].q *= wa;
    }
    R hs = ein[3];
    if (i + 1 < (int)W && j + 1 < (int)H && cell_active(i + 1, j + 1)) {
      size_t cb = idx(i + 1, j + 1);
      V p11 = pressure_at(i + 1, j + 1);
      V ga{-(p11.x - p00.x) * inv_dx * s2, -(p11.y - p00.y) * inv_dx * s2};
      V pa = pressure_wet(i + 1, j, p00), pb = pressure_wet(i, j + 1, p11);
      V gp{-(pa.x - pb.x) * inv_dx * s2, -(pa.y - pb.y) * inv_dx * s2};
      V gt{(gxy.x + gxy.y) * s2, (gxy.x - gxy.y) * s2};
      bool open = std::min(h[c], h[cb]) > 0 || h[idx(i + 1, j)] > hs || h[idx(i, j + 1)] > hs;
      if (open) {
        ff[2] = face(c, cb, V{ga.x, gp.x}, V{ga.y, gp.y}, gt, true, V{s2, s2});
        ff[2].q *= wd;
      }
    }
    if (i + 1 < (int)W && j > 0 && cell_active(i + 1, j - 1)) {
      size_t cb = idx(i + 1, j - 1);
      V p1m = pressure_at(i + 1, j - 1);
      V ga{-(p1m.x - p00.x) * inv_dx * s2, -(p1m.y - p00.y) * inv_dx * s2};
      V pa = pressure_wet(i + 1, j, p00), pb = pressure_wet(i, j - 1, p1m);
      V gp{-(pa.x - pb.x) * inv_dx * s2, -(pa.y - pb.y) * inv_dx * s2};
      V gt{(gxy.x - gxy.y) * s2, (gxy.x + gxy.y) * s2};
      bool open = std::min(h[c], h[cb]) > 0 || h[idx(i + 1, j)] > hs || h[idx(i, j - 1)] > hs;
      if (open) {
        ff[3] = face(c, cb, V{ga.x, gp.x}, V{ga.y, gp.y}, gt, true, V{s2, -s2});
        ff[3].q *= wd;
      }
    }
  }

  // film.wgsl:448-455
  void k_fluxes_cell(int i, int j) {
    Face ff[4];
    face_pair(i, j, ff);
    size_t c = idx(i, j);
    for (int k = 0; k < 4; ++k) flux[4 * c + k] = ff[k].q;
  }

  bool nb_ok(int i, int j) const { return in_grid(i, j) && cell_active(i, j); }

  // film.wgsl:521-537
  void k_limiter_cell(int i, int j) {
    size_t c = idx(i, j);
    const R* f = &flux[4 * c];
    R out = std::max(f[0], R(0)) + std::max(f[1], R(0)) + std::max(f[2], R(0)) + std::max(f[3], R(0));
    if (nb_ok(i - 1, j)) out += std::max(-flux[4 * idx(i - 1, j) + 0], R(0));
    if (nb_ok(i, j - 1)) out += std::max(-flux[4 * idx(i, j - 1) + 1], R(0));
    if (nb_ok(i - 1, j - 1)) out += std::max(-flux[4 * idx(i - 1, j - 1) + 2], R(0));
    if (nb_ok(i - 1, j + 1)) out += std::max(-flux[4 * idx(i - 1, j + 1) + 3], R(0));
    R a = 1;
    if (out > 0) a = std::min(R(1), F(0.5f) * h[c] * dx / (dt * out));
    alpha[c] = a;
  }

  // apply back-fill (film.wgsl:847-860, also strata.wgsl:314-322)
  void backfill_from(size_t c, size_t src, R hn, const std::vector<R>& shs, const std::vector<R>& pgs,
                     const std::vector<R>& cus) {
    int ks = 0;
    for (int k = 0; k < 4; ++k) if (shs[4 * src + k] > 0) ks = k;
    sh[4 * c] = hn; sh[4 * c + 1] = 0; sh[4 * c + 2] = 0; sh[4 * c + 3] = 0;
    for (int s = 0; s < 16; ++s) pig[64 * c + s] = pgs[64 * src + 16 * ks + s];
    for (int s = 16; s < 64; ++s) pig[64 * c + s] = 0;
    R cv = cus[4 * src + ks];
    scu[4 * c] = cv; scu[4 * c + 1] = 0; scu[4 * c + 2] = 0; scu[4 * c + 3] = 0;
  }

  // film.wgsl:539-561, 803-863; returns "moved"
  bool k_apply_cell(int i, int j) {
    size_t c = idx(i, j);
    R ac = alpha[c];
    R best = 0, div = 0;
    size_t src = c;
    R accv[4];
    const R* f = &flux[4 * c];
    bool hx = i + 1 < (int)W, hy = j + 1 < (int)H, hm = j > 0;
    size_t cbs[4] = {hx ? idx(i + 1, j) : c, hy ? idx(i, j + 1) : c, (hx && hy) ? idx(i + 1, j + 1) : c,
                     (hx && hm) ? idx(i + 1, j - 1) : c};
    bool has[4] = {hx, hy, hx && hy, hx && hm};
    for (int k = 0; k < 4; ++k) {  // own_face
      R q = f[k];
      R ab = ac;
      if (q < 0 && has[k]) {
        ab = alpha[cbs[k]];
        if (-q * ab > best) { best = -q * ab; src = cbs[k]; }
      }
      div += q * ab;
      accv[k] = q * ab;
    }
    auto nb_face = [&](R q, size_t cn) {
      R an = alpha[cn];
      if (q < 0) an = ac;
      if (q * an > best) { best = q * an; src = cn; }
      div -= q * an;
    };
    if (nb_ok(i - 1, j)) { size_t cn = idx(i - 1, j); nb_face(flux[4 * cn + 0], cn); }
    if (nb_ok(i, j - 1)) { size_t cn = idx(i, j - 1); nb_face(flux[4 * cn + 1], cn); }
    if (nb_ok(i - 1, j - 1)) { size_t cn = idx(i - 1, j - 1); nb_face(flux[4 * cn + 2], cn); }
    if (nb_ok(i - 1, j + 1)) { size_t cn = idx(i - 1, j + 1); nb_face(flux[4 * cn + 3], cn); }
    R h0 = h[c];
    R hn = std::max(h0 - dt * div * inv_dx, R(0));
    if (hn < h0 && hn < F(1e-9f)) hn = 0;
    h[c] = hn;
    bool moved = std::fabs(hn - h0) > F(1e-6f);
    if (h0 <= 0 && src != c) {
      rheo[3 * c] = rheo[3 * src]; rheo[3 * c + 1] = rheo[3 * src + 1]; rheo[3 * c + 2] = rheo[3 * src + 2];
      backfill_from(c, src, hn, sh, pig, scu);
    }
    for (int k = 0; k < 4; ++k) acc[4 * c + k] += accv[k] * dt;
    return moved;
  }

  // film.wgsl:680-723 (Jacobi: `dold` is delta before the dispatch)
  void k_nose_cell(int i, int j, const std::vector<uint32_t>& dold) {
    size_t c = idx(i, j);
    if (h[c] <= 0) { delta[c] = 0; fnorm[2 * c] = 0; fnorm[2 * c + 1] = 0; return; }
    int bx = 64, by = 64;
    R bd = F(1e9f);
    for (int dj = -1; dj <= 1; ++dj)
      for (int di = -1; di <= 1; ++di) {
        int x = i + di, y = j + dj;
        if (!in_grid(x, y)) continue;
        size_t n = idx(x, y);
        int cx = di, cy = dj;
        if (h[n] > 0) {
          if ((dold[n] & 0x10000u) == 0u) continue;
          int ox, oy;
          unpack_off(dold[n], ox, oy);
          cx = ox + di; cy = oy + dj;
          int tx = i + cx, ty = j + cy;
          if (!in_grid(tx, ty)) continue;
          if (h[idx(tx, ty)] > 0) continue;
        } else if (di == 0 && dj == 0) {
          continue;
        }
        R d = len((R)cx, (R)cy);
        if (d < bd) { bd = d; bx = cx; by = cy; }
      }
    if (bd > F(1e8f)) { delta[c] = 0; fnorm[2 * c] = 0; fnorm[2 * c + 1] = 0; return; }
    delta[c] = pack_off(bx, by);
    if (bd <= R(3)) { V n = front_normal(c); fnorm[2 * c] = n.x; fnorm[2 * c + 1] = n.y; }
    else { fnorm[2 * c] = 0; fnorm[2 * c + 1] = 0; }
  }

  // film.wgsl:457-473
  void band_split(size_t cu, R hf, R y, R up, R total, R n, R out[4]) const {
    const R* s = &sh[4 * cu];
    R hu = s[0] + s[1] + s[2] + s[3];
    if (hu <= 0) { out[0] = total; out[1] = out[2] = out[3] = 0; return; }
    R frac[4] = {s[0] / hu, s[1] / hu, s[2] / hu, s[3] / hu};
    if (y > 0 && up > 0) {
      R k = hf / hu;
      R z1 = s[0] * k;
      R z2 = z1 + s[1] * k;
      R z3 = z2 + s[2] * k;
      R z4 = z3 + s[3] * k;
      R b[4] = {band_flux(up, y, 0, z1, n), band_flux(up, y, z1, z2, n), band_flux(up, y, z2, z3, n),
                band_flux(up, y, z3, z4, n)};
      R bs = b[0] + b[1] + b[2] + b[3];
      if (bs > 0) for (int q = 0; q < 4; ++q) frac[q] = b[q] / bs;
    }
    for (int q = 0; q < 4; ++q) out[q] = frac[q] * total;
  }

  // film.wgsl:475-514
  void k_strata_split_cell(int i, int j) {
    size_t c = idx(i, j);
    Face ff[4];
    face_pair(i, j, ff);
    const R* a = &acc[4 * c];
    R o[4][4] = {};
    int ni[4] = {i + 1, i, i + 1, i + 1}, nj[4] = {j, j + 1, j + 1, j - 1};
    bool ok[4] = {i + 1 < (int)W, j + 1 < (int)H, i + 1 < (int)W && j + 1 < (int)H, i + 1 < (int)W && j > 0};
    for (int f = 0; f < 4; ++f) {
      if (a[f] != 0 && ok[f]) {
        size_t cb = idx(ni[f], nj[f]);
        size_t cu = a[f] < 0 ? cb : c;
        band_split(cu, F(0.5f) * (h[c] + h[cb]), ff[f].y, ff[f].up, a[f], ff[f].n, o[f]);
      }
    }
    for (int f = 0; f < 4; ++f)
      for (int k = 0; k < 4; ++k) acc_s[16 * c + 4 * f + k] = o[f][k];
  }

  // strata.wgsl:157-173
  void k_strata_limit_cell(int i, int j) {
    size_t c = idx(i, j);
    R out[4];
    for (int k = 0; k < 4; ++k)
      out[k] = std::max(acc_s[16 * c + k], R(0)) + std::max(acc_s[16 * c + 4 + k], R(0)) +
               std::max(acc_s[16 * c + 8 + k], R(0)) + std::max(acc_s[16 * c + 12 + k], R(0));
    auto addn = [&](int x, int y, int f) {
      size_t n = idx(x, y);
      for (int k = 0; k < 4; ++k) out[k] += std::max(-acc_s[16 * n + 4 * f + k], R(0));
    };
    if (i > 0 && cell_active(i - 1, j)) addn(i - 1, j, 0);
    if (j > 0 && cell_active(i, j - 1)) addn(i, j - 1, 1);
    if (i > 0 && j > 0 && cell_active(i - 1, j - 1)) addn(i - 1, j - 1, 2);
    if (i > 0 && j + 1 < (int)H && cell_active(i - 1, j + 1)) addn(i - 1, j + 1, 3);
    for (int k = 0; k < 4; ++k) {
      R a = 1;
      if (out[k] > 0) a = std::min(R(1), sh[4 * c + k] * dx / out[k]);
      alpha_s[4 * c + k] = a;
    }
  }

  // ---- stack (strata.wgsl:1-155) ----
  void stack_load(size_t c, Stack& s) const {
    for (int k = 0; k < 4; ++k) {
      s.th[k] = sh[4 * c + k];
      s.cu[k] = scu[4 * c + k];
      for (int q = 0; q < 16; ++q) s.pg[k][q] = pig[64 * c + 16 * k + q];
    }
  }
  void stack_store_to(size_t c, const Stack& s, std::vector<R>& th, std::vector<R>& cu, std::vector<R>& pg) const {
    for (int k = 0; k < 4; ++k) {
      th[4 * c + k] = s.th[k];
      cu[4 * c + k] = s.cu[k];
      for (int q = 0; q < 16; ++q) pg[64 * c + 16 * k + q] = pig_store(s.pg[k][q], q);
    }
  }
  static R pig_dist(const R* a, const R* b) {
    R d = 0;
    for (int q = 0; q < 13; ++q) d += std::fabs(a[q] - b[q]);
    return d;
  }
  // strata.wgsl:45-60 (slot 15 mixed like slot 14: extension)
  static void pig_mix(const R* a, R wa, const R* b, R wb, R* o) {
    R w = std::max(wa + wb, (R)1e-20f);
    R t[16];
    for (int q = 0; q < 16; ++q) t[q] = (a[q] * wa + b[q] * wb) / w;
    for (int slot = 14; slot <= 15; ++slot) {
      R va = a[slot] > 0 ? wa : R(0);
      R vb = b[slot] > 0 ? wb : R(0);
      if (va + vb > 0) t[slot] = (a[slot] * va + b[slot] * vb) / (va + vb);
      else t[slot] = 0;
    }
    for (int q = 0; q < 16; ++q) o[q] = t[q];
  }
  static uint32_t stack_count(const Stack& s) {
    uint32_t n = 0;
    for (int k = 0; k < 4; ++k) if (s.th[k] > 0) n = k + 1;
    return n;
  }
  void stack_merge(Stack& s, int a) const {
    int b = a + 1;
    R ta = s.th[a], tb = s.th[b];
    pig_mix(s.pg[a], ta, s.pg[b], tb, s.pg[a]);
    s.cu[a] = (s.cu[a] * ta + s.cu[b] * tb) / std::max(ta + tb, (R)1e-20f);
    s.th[a] = ta + tb;
    for (int k = b; k < 3; ++k) {
      s.th[k] = s.th[k + 1];
      s.cu[k] = s.cu[k + 1];
      for (int q = 0; q < 16; ++q) s.pg[k][q] = s.pg[k + 1][q];
    }
    s.th[3] = 0;
    s.cu[3] = 0;
  }
  void stack_compact(Stack& s) const {
    for (int sweep = 0; sweep < 4; ++sweep)
      for (int k = 0; k < 3; ++k)
        if (s.th[k] <= 0 && s.th[k + 1] > 0) {
          s.th[k] = s.th[k + 1];
          s.cu[k] = s.cu[k + 1];
          for (int q = 0; q < 16; ++q) s.pg[k][q] = s.pg[k + 1][q];
          s.th[k + 1] = 0;
          s.cu[k + 1] = 0;
        }
    R tiny = misc[0];
    for (int k = 0; k < 3; ++k)
      if (s.th[k] > 0 && s.th[k] < tiny && s.th[k + 1] > 0) stack_merge(s, k);
  }
  void stack_push_top(Stack& s, R vol, const R* pg, R cv) const {
    if (vol <= 0) return;
    uint32_t n = stack_count(s);
    if (n > 0) {
      int t = (int)n - 1;
      bool close = pig_dist(s.pg[t], pg) < misc[1] || s.th[t] < misc[0];
      if (close) {
        pig_mix(s.pg[t], s.th[t], pg, vol, s.pg[t]);
        s.cu[t] = (s.cu[t] * s.th[t] + cv * vol) / (s.th[t] + vol);
        s.th[t] += vol;
        return;
      }
    }
    if (n == 4) {
      int best = 0;
      R bd = (R)1e30f;
      for (int k = 0; k < 3; ++k) {
        R d = pig_dist(s.pg[k], s.pg[k + 1]);
        if (d < bd) { bd = d; best = k; }
      }
      stack_merge(s, best);
    }
    uint32_t t = stack_count(s);
    s.th[t] = vol;
    for (int q = 0; q < 16; ++q) s.pg[t][q] = pg[q];
    s.cu[t] = cv;
  }
  void stack_add_band(Stack& s, R zlo, R zhi, R vol, const R* pg, R cv) const {
    if (vol <= 0) return;
    R span = std::max(zhi - zlo, (R)1e-12f);
    R z0 = 0, above = vol;
    for (int k = 0; k < 4; ++k) {
      R tk = s.th[k];
      if (tk <= 0) break;
      R z1 = z0 + tk;
      R ov = std::max(std::min(zhi, z1) - std::max(zlo, z0), R(0));
      R part = vol * ov / span;
      if (part > 0) {
        pig_mix(s.pg[k], tk, pg, part, s.pg[k]);
        s.cu[k] = (s.cu[k] * tk + cv * part) / (tk + part);
        s.th[k] = tk + part;
        above -= part;
      }
      z0 = z1;
    }
    if (above > (R)1e-14f) stack_push_top(s, above, pg, cv);
  }
  // strata.wgsl:175-188
  void inflow_from(Stack& s, size_t cn, const R f[4]) const {
    R z0 = 0;
    for (int k = 0; k < 4; ++k) {
      R thn = sh[4 * cn + k];
      R z1 = z0 + thn;
      R v = f[k] * alpha_s[4 * cn + k] * inv_dx;
      if (v > 0 && thn > 0) stack_add_band(s, z0, z1, v, &pig[64 * cn + 16 * k], scu[4 * cn + k]);
      z0 = z1;
    }
  }

  // strata.wgsl:190-274
  void k_strata_update_cell(int i, int j) {
    size_t c = idx(i, j);
    R fr[4], fu[4], fdg[4], feg[4], fl[4] = {0, 0, 0, 0}, fd[4] = {0, 0, 0, 0}, fll[4] = {0, 0, 0, 0},
                                    flu[4] = {0, 0, 0, 0};
    for (int k = 0; k < 4; ++k) {
      fr[k] = acc_s[16 * c + k]; fu[k] = acc_s[16 * c + 4 + k];
      fdg[k] = acc_s[16 * c + 8 + k]; feg[k] = acc_s[16 * c + 12 + k];
    }
    size_t cl = c, cd = c, cll = c, clu = c;
    if (i > 0 && cell_active(i - 1, j)) { cl = idx(i - 1, j); for (int k = 0; k < 4; ++k) fl[k] = acc_s[16 * cl + k]; }
    if (j > 0 && cell_active(i, j - 1)) { cd = idx(i, j - 1); for (int k = 0; k < 4; ++k) fd[k] = acc_s[16 * cd + 4 + k]; }
    if (i > 0 && j > 0 && cell_active(i - 1, j - 1)) { cll = idx(i - 1, j - 1); for (int k = 0; k < 4; ++k) fll[k] = acc_s[16 * cll + 8 + k]; }
    if (i > 0 && j + 1 < (int)H && cell_active(i - 1, j + 1)) { clu = idx(i - 1, j + 1); for (int k = 0; k < 4; ++k) flu[k] = acc_s[16 * clu + 12 + k]; }
    bool allzero = true;
    for (int k = 0; k < 4; ++k)
      if (fr[k] != 0 || fu[k] != 0 || fdg[k] != 0 || feg[k] != 0 || fl[k] != 0 || fd[k] != 0 || fll[k] != 0 || flu[k] != 0)
        allzero = false;
    if (allzero) {
      R hc = h[c];
      R th[4], nt[4] = {0, 0, 0, 0}, cu[4];
      for (int k = 0; k < 4; ++k) { th[k] = std::max(sh[4 * c + k], R(0)); cu[k] = scu[4 * c + k]; }
      if (hc <= 0) {
        for (int k = 0; k < 4; ++k) cu[k] = 0;
      } else {
        R sum = th[0] + th[1] + th[2] + th[3];
        for (int k = 0; k < 4; ++k) nt[k] = th[k];
        if (sum > 0) { R sc = hc / sum; for (int k = 0; k < 4; ++k) nt[k] = th[k] * sc; }
      }
      bool plain = true;
      for (int k = 0; k < 3; ++k) {
        if (nt[k] <= 0 && nt[k + 1] > 0) plain = false;
        if (nt[k] > 0 && nt[k] < misc[0] && nt[k + 1] > 0) plain = false;
      }
      if (plain) {
        for (int k = 0; k < 4; ++k) { sh2[4 * c + k] = nt[k]; scu2[4 * c + k] = cu[k]; }
        for (int q = 0; q < 64; ++q) pig2[64 * c + q] = pig[64 * c + q];
        return;
      }
    }
    Stack s;
    stack_load(c, s);
    R out[4];
    for (int k = 0; k < 4; ++k)
      out[k] = std::max(fr[k], R(0)) + std::max(fu[k], R(0)) + std::max(fdg[k], R(0)) + std::max(feg[k], R(0)) +
               std::max(-fl[k], R(0)) + std::max(-fd[k], R(0)) + std::max(-fll[k], R(0)) + std::max(-flu[k], R(0));
    for (int k = 0; k < 4; ++k) s.th[k] = std::max(s.th[k] - out[k] * alpha_s[4 * c + k] * inv_dx, R(0));
    R neg[4];
    if (i + 1 < (int)W) { for (int k = 0; k < 4; ++k) neg[k] = -fr[k]; inflow_from(s, idx(i + 1, j), neg); }
    if (j + 1 < (int)H) { for (int k = 0; k < 4; ++k) neg[k] = -fu[k]; inflow_from(s, idx(i, j + 1), neg); }
    if (i + 1 < (int)W && j + 1 < (int)H) { for (int k = 0; k < 4; ++k) neg[k] = -fdg[k]; inflow_from(s, idx(i + 1, j + 1), neg); }
    if (i + 1 < (int)W && j > 0) { for (int k = 0; k < 4; ++k) neg[k] = -feg[k]; inflow_from(s, idx(i + 1, j - 1), neg); }
    if (cl != c) inflow_from(s, cl, fl);
    if (cd != c) inflow_from(s, cd, fd);
    if (cll != c) inflow_from(s, cll, fll);
    if (clu != c) inflow_from(s, clu, flu);
    R hc = h[c];
    R sum = s.th[0] + s.th[1] + s.th[2] + s.th[3];
    if (hc <= 0) {
      for (int k = 0; k < 4; ++k) { s.th[k] = 0; s.cu[k] = 0; }
    } else if (sum > 0) {
      R kk = hc / sum;
      for (int q = 0; q < 4; ++q) s.th[q] *= kk;
    }
    stack_compact(s);
    stack_store_to(c, s, sh2, scu2, pig2);
  }

  // strata.wgsl:276-286
  void k_copy_back_cell(int i, int j) {
    size_t c = idx(i, j);
    for (int k = 0; k < 4; ++k) { sh[4 * c + k] = sh2[4 * c + k]; scu[4 * c + k] = scu2[4 * c + k]; }
    for (int q = 0; q < 64; ++q) pig[64 * c + q] = pig2[64 * c + q];
  }

  // strata.wgsl:288-323 (Jacobi: *_old are the planes before the dispatch)
  void k_strata_fill_cell(int i, int j, const std::vector<R>& sho, const std::vector<R>& pgo,
                          const std::vector<R>& cuo) {
    size_t c = idx(i, j);
    R hc = h[c];
    if (hc <= 0) return;
    const R* th = &sho[4 * c];
    if (th[0] + th[1] + th[2] + th[3] > 0) return;
    size_t src = c;
    R best = 0;
    size_t cands[4];
    int nc = 0;
    if (i > 0) cands[nc++] = idx(i - 1, j);
    if (j > 0) cands[nc++] = idx(i, j - 1);
    if (i + 1 < (int)W) cands[nc++] = idx(i + 1, j);
    if (j + 1 < (int)H) cands[nc++] = idx(i, j + 1);
    for (int q = 0; q < nc; ++q) {
      const R* tn = &sho[4 * cands[q]];
      R tsum = tn[0] + tn[1] + tn[2] + tn[3];
      if (tsum > best) { best = tsum; src = cands[q]; }
    }
    if (src == c) return;
    backfill_from(c, src, hc, sho, pgo, cuo);
  }

  // ---- cure (cure.wgsl) ----
  // cure.wgsl:3-48 / 62-117 over an unpacked stack; returns (mu, tau, n)
  void composition_rheo(const Stack& s, R out[3]) const {
    R total = 0, lnmu = 0, tau = 0, thin = 0, wsum = 0, cur = 0, nsum = 0, nw = 0;
    for (int k = 0; k < 4; ++k) {
      R t = s.th[k];
      if (t <= 0) continue;
      total += t;
      cur += t * s.cu[k];
      R csum = 0, lm = 0, ty = 0;
      for (int q = 0; q < NPIG; ++q) {
        R cc = s.pg[k][q];
        if (cc > 0) {
          csum += cc;
          lm += cc * std::log(std::max(pigtab[q * PIG_STRIDE + 32], F(1e-3f)));
          ty += cc * s.pg[k][13];
        }
      }
      if (s.pg[k][14] > 0) lm = csum * (s.pg[k][14] - R(10));
      if (csum > 0) {
        lnmu += t * lm / csum;
        tau += t * ty / csum;
        wsum += t;
        if (s.pg[k][15] > 0) { nsum += t * s.pg[k][15]; nw += t; }
      }
      thin += t * s.pg[k][12];
    }
    if (total <= 0) { out[0] = 1; out[1] = 0; out[2] = phys[2]; return; }
    R mu = std::log(misc[2]);
    R ty = 0;
    if (wsum > 0) { mu = lnmu / wsum; ty = tau / wsum; }
    R tf = clampR(thin / total, R(0), F(0.95f));
    R cb = cur / total;
    mu += R(3) * std::log(R(1) - tf) + cure[2] * cb * cb;
    ty = ty * std::pow(R(1) - tf, R(4)) + cure[1] * cb * cb;
    out[0] = std::exp(mu);
    out[1] = ty;
    out[2] = nw > 0 ? nsum / nw : phys[2];
  }

  // km.wgsl:1-33
  void km_layer(R k, R s, R t, R& rr, R& tt) const {
    if (k + s < F(1e-6f) || t <= 0) { rr = 0; tt = 1; return; }
    R bs = std::sqrt(std::max(k * (k + R(2) * s), R(0)));
    R arg = std::min(bs * t, R(20));
    R e = std::exp(arg);
    R shh = F(0.5f) * (e - R(1) / e);
    R ch = F(0.5f) * (e + R(1) / e);
    R den = (k + s) * shh + bs * ch;
    if (den < F(1e-12f)) { rr = 0; tt = 1; return; }
    rr = s * shh / den;
    tt = bs / den;
  }
  static R composite(R rr, R tt, R rb) { return rr + tt * tt * rb / std::max(R(1) - rr * rb, F(1e-4f)); }
  void layer_ks(const R* pg, int band, R& k, R& s) const {
    k = 0; s = 0;
    R amount = 0, weight = 0;
    for (int q = 0; q < NPIG; ++q) {
      R c = pg[q];
      if (c > 0) {
        R w = c * pigtab[q * PIG_STRIDE + 34];
        k += w * pigtab[q * PIG_STRIDE + band];
        s += w * pigtab[q * PIG_STRIDE + NB + band];
        amount += c;
        weight += w;
      }
    }
    R sc = amount / std::max(weight, F(1e-9f));
    k = k * sc;
    s = s * sc;
  }

  // cure.wgsl:119-159 (full grid)
  void k_cure_cell(size_t c) {
    if (h[c] <= 0) { rheo[3 * c] = 1; rheo[3 * c + 1] = 0; rheo[3 * c + 2] = phys[2]; return; }
    R rate = cure[0] * frame_dt;
    R t[4], u[4];
    for (int k = 0; k < 4; ++k) {
      t[k] = sh[4 * c + k];
      u[k] = t[k] > 0 ? std::min(scu[4 * c + k] + rate, R(1)) : scu[4 * c + k];
    }
    if (!(t[0] > 0 && u[0] >= R(1))) {
      for (int k = 0; k < 4; ++k) scu[4 * c + k] = u[k];
      Stack s;
      stack_load(c, s);  // packed_rheo reads the stored slots
      for (int k = 0; k < 4; ++k) s.cu[k] = u[k];
      R r[3];
      composition_rheo(s, r);
      rheo[3 * c] = r[0]; rheo[3 * c + 1] = r[1]; rheo[3 * c + 2] = r[2];
      return;
    }
    Stack s;
    stack_load(c, s);
    for (int k = 0; k < 4; ++k) s.cu[k] = u[k];
    R committed = 0;
    uint32_t guard = 0;
    while (s.th[0] > 0 && s.cu[0] >= R(1) && guard < 4u) {
      guard++;
      for (int b = 0; b < NB; ++b) {
        R kk, ss, rr, tt;
        layer_ks(s.pg[0], b, kk, ss);
        km_layer(kk, ss, s.th[0], rr, tt);
        refl[16 * c + b] = (R)round_f16((double)composite(rr, tt, refl[16 * c + b]));
      }
      committed += s.th[0];
      m[c] = m[c] + s.th[0] * (R(1) - F(0.04f)) * (R(1) - clampR(s.pg[0][12], R(0), F(0.95f)));
      s.th[0] = 0;
      s.cu[0] = 0;
      stack_compact(s);
    }
    if (committed > 0) h[c] = std::max(h[c] - committed, R(0));
    R r[3];
    composition_rheo(s, r);
    rheo[3 * c] = r[0]; rheo[3 * c + 1] = r[1]; rheo[3 * c + 2] = r[2];
    stack_store_to(c, s, sh, scu, pig);
  }

  // shade.wgsl:28-84: the colour and the renderer's detail texel
  void k_shade_cell(size_t c) {
    R r[NB];
    for (int b = 0; b < NB; ++b) r[b] = refl[16 * c + b];
    R hv = h[c], wet = 0, cure_top = 0;
    if (hv > 0) {
      for (int k = 0; k < 4; ++k) {
        R t = sh[4 * c + k];
        if (t <= 0) continue;
        const R* pg = &pig[64 * c + 16 * k];
        for (int b = 0; b < NB; ++b) {
          R kk, ss, rr, tt;
          layer_ks(pg, b, kk, ss);
          km_layer(kk, ss, t, rr, tt);
          r[b] = composite(rr, tt, r[b]);
        }
        wet = R(1) - scu[4 * c + k];
        cure_top = scu[4 * c + k];
      }
    }
    R k1 = F(0.04f);
    R k2 = mixR(F(0.4f), F(0.6f), wet);
    for (int b = 0; b < NB; ++b) r[b] = (R(1) - k1) * (R(1) - k2) * r[b] / std::max(R(1) - k2 * r[b], F(1e-3f));
    R X = 0, Y = 0, Z = 0;
    for (int b = 0; b < NB; ++b) { X += r[b] * cmf[3 * b]; Y += r[b] * cmf[3 * b + 1]; Z += r[b] * cmf[3 * b + 2]; }
    R rgb[3] = {F(3.2406f) * X - F(1.5372f) * Y - F(0.4986f) * Z, F(-0.9689f) * X + F(1.8758f) * Y + F(0.0415f) * Z,
                F(0.0557f) * X - F(0.2040f) * Y + F(1.0570f) * Z};
    for (int q = 0; q < 3; ++q) rgb[q] = std::max(rgb[q], R(0));
    R painted = smooth(F(60e-6f), F(150e-6f), m[c]);
    cure_top = std::max(cure_top, painted * (R(1) - smooth(R(0), F(50e-6f), hv)));
    R rough = mixR(F(0.06f), F(0.35f), std::sqrt(cure_top));
    if (hv <= 0) rough = mixR(F(0.85f), F(0.35f), painted);
    if (flags[0] == 1u && hv > 0) {
      const R* th = &sh[4 * c];
      R ssum = th[0] + th[1] + th[2] + th[3];
      bool bad = false;
      uint32_t cnt = 0;
      for (int k = 0; k < 4; ++k) {
        if (th[k] > 0) cnt = k + 1;
        if (th[k] <= 0) continue;
        R cs = 0;
        for (int q = 0; q < 13; ++q) cs += pig[64 * c + 16 * k + q];
        if (!(cs > 0)) bad = true;
      }
      if (ssum <= 0) { rgb[0] = 0; rgb[1] = 0; rgb[2] = 1; }
      else if (bad) { rgb[0] = 1; rgb[1] = 0; rgb[2] = 0; }
      else if (std::fabs(ssum - hv) > F(0.01f) * hv) { rgb[0] = 0; rgb[1] = 1; rgb[2] = 0; }
      else { R v = F(0.3f) + F(0.15f) * (R)cnt; rgb[0] = v; rgb[1] = v; rgb[2] = v; }
    }
    color[4 * c] = rgb[0]; color[4 * c + 1] = rgb[1]; color[4 * c + 2] = rgb[2]; color[4 * c + 3] = rough;
    // shade.wgsl:61-64: lay method + stroke turn, cure_top, yield stress, thickness above the weave
    const uint32_t lv = lay[c];
    const R turn = (R)(lv >> 8u & 0xffffu) / F(65536.0f);
    detail[4 * c] = (R)(lv & 0xffu) + turn;
    detail[4 * c + 1] = cure_top;
    detail[4 * c + 2] = rheo[3 * c + 1];
    detail[4 * c + 3] = hv + std::max(m[c] - F(60e-6f), R(0));
  }

  // ---- tile activity (film.wgsl:1365-1425) ----
  void k_mark_tiles() {
    for (uint32_t ty = 0; ty < TH; ++ty)
      for (uint32_t tx = 0; tx < TW; ++tx) {
        uint32_t any = 0;
        for (int ly = 0; ly < 16; ++ly)
          for (int lx = 0; lx < 16; ++lx) {
            int i = tx * 16 + lx, j = ty * 16 + ly;
            if (i >= (int)W || j >= (int)H) continue;
            size_t c = idx(i, j);
            if (h[c] > 0) {
              uint32_t bits = 1u;
              if (lx < WAKE_BAND) bits |= 2u;
              if (lx >= 16 - WAKE_BAND) bits |= 4u;
              if (ly < WAKE_BAND) bits |= 8u;
              if (ly >= 16 - WAKE_BAND) bits |= 16u;
              if (std::fabs(h[c] - h_frame[c]) > F(2e-6f)) bits |= MOVED;
              any |= bits;
            }
          }
        size_t t = tx + (size_t)ty * TW;
        if (tile_moved[t] != 0u) any |= MOVED;
        tile_moved[t] = 0u;
        tile_flags[t] = any;
      }
  }
  void k_compact_tiles() {
    std::vector<uint32_t> fl = tile_flags;  // bit 32 updates do not affect the bits read
    active_tiles = 0;
    for (uint32_t t = 0; t < TW * TH; ++t) {
      int tx = (int)(t % TW), ty = (int)(t / TW);
      uint32_t any = fl[t] & MOVED;
      for (int dy = -1; dy <= 1; ++dy)
        for (int dxi = -1; dxi <= 1; ++dxi) {
          if (dxi == 0 && dy == 0) continue;
          int x = tx + dxi, y = ty + dy;
          if (x >= 0 && y >= 0 && x < (int)TW && y < (int)TH) {
            uint32_t f = fl[x + (size_t)y * TW];
            bool need = true;
            if (dxi == 1 && (f & 2u) == 0u) need = false;
            if (dxi == -1 && (f & 4u) == 0u) need = false;
            if (dy == 1 && (f & 8u) == 0u) need = false;
            if (dy == -1 && (f & 16u) == 0u) need = false;
            if (need) any |= f & MOVED;
          }
        }
      if (S.all_active) any = 1u;  // extension: every tile active
      if (any != 0u) { tile_flags[t] = fl[t] | 32u; active_tiles++; }
      else tile_flags[t] = fl[t] & 31u;
    }
  }

  // film.wgsl:1330-1361
  void k_reduce_tiles() {
    uint32_t tw = (W + 63) / 64, th = (H + 63) / 64;
    R hmx = 0, mmn = F(1e9f);
    for (uint32_t ty = 0; ty < th; ++ty)
      for (uint32_t tx = 0; tx < tw; ++tx) {
        R hm = 0, mm = F(1e9f);
        for (uint32_t j = ty * 64; j < std::min(H, ty * 64 + 64); ++j)
          for (uint32_t i = tx * 64; i < std::min(W, tx * 64 + 64); ++i) {
            size_t c = idx(i, j);
            R v = h[c];
            if (v > R(4) * ein[3]) { hm = std::max(hm, v); mm = std::min(mm, rheo[3 * c]); }
          }
        stats[2 * (tx + ty * tw)] = hm;
        stats[2 * (tx + ty * tw) + 1] = mm;
        hmx = std::max(hmx, hm);
        mmn = std::min(mmn, mm);
      }
    // poll_stats (src/film/mod.rs:944-968): the pending deposit height is
    // forgotten once stats that include the deposits arrive
    h_max_stat = (float)hmx;
    mu_min_stat = mmn > F(1e8f) ? 1.0f : (float)mmn;
    if (dep_items.empty()) h_max_pending = 0.0f;
  }

  // ---- dispatch helpers ----
  // Every dispatch below writes only its own cell (nose and strata_fill read
  // a snapshot), so rows run in parallel without changing any result.
  template <class Fn>
  void for_active(Fn fn) {
#pragma omp parallel for schedule(dynamic, 4)
    for (int j = 0; j < (int)H; ++j)
      for (int i = 0; i < (int)W; ++i)
        if (cell_active(i, j)) fn(i, j);
  }

  void run_laplacian() { for_active([&](int i, int j) { k_laplacian_cell(i, j); }); }
  void run_plug() { for_active([&](int i, int j) { k_plug_cell(i, j); }); }
  void run_fluxes() { for_active([&](int i, int j) { k_fluxes_cell(i, j); }); }
  void run_limiter() { for_active([&](int i, int j) { k_limiter_cell(i, j); }); }
  void run_apply() {
    std::vector<uint8_t> mvc(N, 0);
    for_active([&](int i, int j) { mvc[idx(i, j)] = k_apply_cell(i, j) ? 1 : 0; });
    for (size_t c = 0; c < N; ++c)
      if (mvc[c]) tile_moved[(c % W) / 16 + ((c / W) / 16) * TW] = 1u;
  }
  void run_nose() {
    std::vector<uint32_t> dold = delta;
    for_active([&](int i, int j) { k_nose_cell(i, j, dold); });
  }
  void run_clear_acc() {
    for_active([&](int i, int j) {
      size_t c = idx(i, j);
      for (int k = 0; k < 4; ++k) acc[4 * c + k] = 0;
      h_frame[c] = h[c];
    });
  }
  void run_strata_split() { for_active([&](int i, int j) { k_strata_split_cell(i, j); }); }
  void run_strata_limit() { for_active([&](int i, int j) { k_strata_limit_cell(i, j); }); }
  void run_strata_update() { for_active([&](int i, int j) { k_strata_update_cell(i, j); }); }
  void run_copy_back() { for_active([&](int i, int j) { k_copy_back_cell(i, j); }); }
  void run_strata_fill() {
    std::vector<R> sho = sh, pgo = pig, cuo = scu;
    for_active([&](int i, int j) { k_strata_fill_cell(i, j, sho, pgo, cuo); });
  }
  void run_cure() {
#pragma omp parallel for schedule(static)
    for (long c = 0; c < (long)N; ++c) k_cure_cell((size_t)c);
  }
  void run_shade() {
#pragma omp parallel for schedule(static)
    for (long c = 0; c < (long)N; ++c) k_shade_cell((size_t)c);
  }

  // ---- implicit hydrostatic CG steps (film.wgsl:895-1207; dispatched by
  // Film::encode_frame, src/film/mod.rs:1373-1408) ----
  // The system and the flux of each step live on the active tiles; planes
  // of inactive tiles keep the values of the last step that covered them,
  // and the reference reads those (cg_m, cg_p of a neighbour) as they are.
  std::vector<R> cg_m /*4N*/, cg_d, cg_x, cg_r, cg_p, cg_q, cg_t, cg_t2;
  std::vector<R> cg_part, cg_part2;  // per active tile (list position)
  R cg_s[2][4] = {};
  std::vector<uint32_t> cg_tiles;  // active tiles in compact_tiles' order

  void cg_alloc() {
    if (cg_d.size() == N) return;
    cg_m.assign(4 * N, 0);
    for (auto* v : {&cg_d, &cg_x, &cg_r, &cg_p, &cg_q, &cg_t, &cg_t2}) v->assign(N, 0);
    cg_part.assign((size_t)TW * TH, 0);
    cg_part2.assign((size_t)TW * TH, 0);
  }
  // film.wgsl:895-923 (the mobility of a face; the flow index of the face as
  // in face(): the per-cell extension reduces to phys.z)
  R face_mob(size_t ca, size_t cb, V gcap, V ghyd, V gtilt, bool diag) const {
    R ha = h[ca], hb = h[cb];
    if (std::min(ha, hb) <= 0) return 0;
    R hf = F(0.5f) * (ha + hb);
    R rax = rheo[3 * ca], ray = rheo[3 * ca + 1], rbx = rheo[3 * cb], rby = rheo[3 * cb + 1];
    R wa = ha / (ha + hb);
    R wb = R(1) - wa;
    R mu = std::exp(wa * std::log(std::max(rax, F(1e-4f))) + wb * std::log(std::max(rbx, F(1e-4f))));
    R ty = wa * ray + wb * rby;
    R na = cell_n(ca), nb = cell_n(cb);
    R nf = na == nb ? na : wa * na + wb * nb;
    R thin = std::min(ha, hb) / hf;
    R fcap = thin * thin * thin;
    V yc = yield_cap(V{gcap.x * fcap, gcap.y * fcap}, ty);
    V gg{yc.x + ghyd.x + gtilt.x, yc.y + ghyd.y + gtilt.y};
    R gmag = len(gg.x, gg.y);
    R qy[3];
    hb_flux(gmag, yield_depth(ca, cb, hf, ty, gg), mu, ty, nf, qy);
    if (qy[0] <= 0) return 0;
    R mob = std::min(std::max(qy[0] / gmag - misc[3], R(0)), front[2]);
    if (std::min(ha, hb) < F(0.5f) * std::max(ha, hb)) {
      if (diag) return 0;
      size_t tgt = hb > ha ? ca : cb;
      mob = mob / std::pow((R)std::max(feeders(tgt), 1u), F(0.7f));
    }
    return mob;
  }
  R kappa() const { return front[3] * phys[0] * g[2] * inv_dx * inv_dx; }  // film.wgsl:925-927
  R hold_u(size_t c) const {  // film.wgsl:929-933
    R hold = 0;
    if (h[c] > 0) hold = hold_level(nose_dist(c));
    return m[c] - hold;
  }
  // film.wgsl:935-987
  void k_cg_setup_cell(int i, int j) {
    size_t c = idx(i, j);
    R mob[4] = {0, 0, 0, 0};
    V p00 = pressure_at(i, j);
    V gxy{phys[0] * g[0], phys[0] * g[1]};
    const R s2 = F(0.70710678f);
    if (i + 1 < (int)W && cell_active(i + 1, j)) {
      size_t cb = idx(i + 1, j);
      V p10 = pressure_at(i + 1, j);
      V gm{-(p10.x - p00.x) * inv_dx, -(p10.y - p00.y) * inv_dx};
      V a = pressure_wet(i, j + 1, p00), b = pressure_wet(i + 1, j + 1, p10);
      V cc = pressure_wet(i, j - 1, p00), d = pressure_wet(i + 1, j - 1, p10);
      V pt{a.x + b.x - cc.x - d.x, a.y + b.y - cc.y - d.y};
      V gt{-pt.x * F(0.25f) * inv_dx, -pt.y * F(0.25f) * inv_dx};
      mob[0] = face_mob(c, cb, V{gm.x, gt.x}, V{gm.y, gt.y}, gxy, false);
    }
    if (j + 1 < (int)H && cell_active(i, j + 1)) {
      size_t cb = idx(i, j + 1);
      V p01 = pressure_at(i, j + 1);
      V gm{-(p01.x - p00.x) * inv_dx, -(p01.y - p00.y) * inv_dx};
      V a = pressure_wet(i + 1, j, p00), b = pressure_wet(i + 1, j + 1, p01);
      V cc = pressure_wet(i - 1, j, p00), d = pressure_wet(i - 1, j + 1, p01);
      V pt{a.x + b.x - cc.x - d.x, a.y + b.y - cc.y - d.y};
      V gt{-pt.x * F(0.25f) * inv_dx, -pt.y * F(0.25f) * inv_dx};
      mob[1] = face_mob(c, cb, V{gm.x, gt.x}, V{gm.y, gt.y}, V{gxy.y, gxy.x}, false);
    }
    if (i + 1 < (int)W && j + 1 < (int)H && cell_active(i + 1, j + 1)) {
      size_t cb = idx(i + 1, j + 1);
      V p11 = pressure_at(i + 1, j + 1);
      V ga{-(p11.x - p00.x) * inv_dx * s2, -(p11.y - p00.y) * inv_dx * s2};
      V pa = pressure_wet(i + 1, j, p00), pb = pressure_wet(i, j + 1, p11);
      V gp{-(pa.x - pb.x) * inv_dx * s2, -(pa.y - pb.y) * inv_dx * s2};
      V gt{(gxy.x + gxy.y) * s2, (gxy.x - gxy.y) * s2};
      mob[2] = face_mob(c, cb, V{ga.x, gp.x}, V{ga.y, gp.y}, gt, true);
    }
    if (i + 1 < (int)W && j > 0 && cell_active(i + 1, j - 1)) {
      size_t cb = idx(i + 1, j - 1);
      V p1m = pressure_at(i + 1, j - 1);
      V ga{-(p1m.x - p00.x) * inv_dx * s2, -(p1m.y - p00.y) * inv_dx * s2};
      V pa = pressure_wet(i + 1, j, p00), pb = pressure_wet(i, j - 1, p1m);
      V gp{-(pa.x - pb.x) * inv_dx * s2, -(pa.y - pb.y) * inv_dx * s2};
      V gt{(gxy.x - gxy.y) * s2, (gxy.x + gxy.y) * s2};
      mob[3] = face_mob(c, cb, V{ga.x, gp.x}, V{ga.y, gp.y}, gt, true);
    }
    for (int k = 0; k < 4; ++k) cg_m[4 * c + k] = mob[k];
  }
  // film.wgsl:994-1010: neighbour k of (i, j) and the weighted mobility of
  // the face to it (the faces of the lower-left neighbours are theirs)
  bool cg_nb(int k, int i, int j, size_t& nc, R& mw) const {
    size_t c = idx(i, j);
    nc = 0;
    mw = 0;
    const R wa = F(0.6666667f), wd = F(0.16666667f);
    switch (k) {
      case 0: if (i + 1 < (int)W) { nc = idx(i + 1, j); mw = wa * cg_m[4 * c]; } break;
      case 1: if (j + 1 < (int)H) { nc = idx(i, j + 1); mw = wa * cg_m[4 * c + 1]; } break;
      case 2: if (i + 1 < (int)W && j + 1 < (int)H) { nc = idx(i + 1, j + 1); mw = wd * cg_m[4 * c + 2]; } break;
      case 3: if (i + 1 < (int)W && j > 0) { nc = idx(i + 1, j - 1); mw = wd * cg_m[4 * c + 3]; } break;
      case 4: if (i > 0) { nc = idx(i - 1, j); mw = wa * cg_m[4 * nc]; } break;
      case 5: if (j > 0) { nc = idx(i, j - 1); mw = wa * cg_m[4 * nc + 1]; } break;
      case 6: if (i > 0 && j > 0) { nc = idx(i - 1, j - 1); mw = wd * cg_m[4 * nc + 2]; } break;
      default: if (i > 0 && j + 1 < (int)H) { nc = idx(i - 1, j + 1); mw = wd * cg_m[4 * nc + 3]; } break;
    }
    return mw > 0;
  }
  // film.wgsl:1012-1021
  R lap_src(size_t c, int which) const {
    switch (which) {
      case 0: return cg_p[c];
      case 1: return h[c];
      case 2: return cg_t2[c];
      case 3: return cg_t[c];
      case 4: return cg_x[c] + hold_u(c);
      default: return hold_u(c);
    }
  }
  // film.wgsl:1023-1043
  R lap_w(int i, int j, size_t c, int which) const {
    R vc = lap_src(c, which), acc_v = 0;
    for (int dj = -1; dj <= 1; ++dj)
      for (int di = -1; di <= 1; ++di) {
        if (di == 0 && dj == 0) continue;
        int x = i + di, y = j + dj;
        if (x < 0 || y < 0 || x >= (int)W || y >= (int)H) continue;
        if (!cell_active(x, y)) continue;
        size_t n = idx(x, y);
        if (h[n] <= 0) continue;
        R w = (di != 0 && dj != 0) ? F(0.16666667f) : F(0.6666667f);
        acc_v += w * (lap_src(n, which) - vc);
      }
    return acc_v;
  }
  // film.wgsl:1045-1064
  R lap_diag(int i, int j) const {
    R s1 = 0, s2 = 0;
    for (int dj = -1; dj <= 1; ++dj)
      for (int di = -1; di <= 1; ++di) {
        if (di == 0 && dj == 0) continue;
        int x = i + di, y = j + dj;
        if (x < 0 || y < 0 || x >= (int)W || y >= (int)H) continue;
        if (!cell_active(x, y)) continue;
        if (h[idx(x, y)] <= 0) continue;
        R w = (di != 0 && dj != 0) ? F(0.16666667f) : F(0.6666667f);
        s1 += w;
        s2 += w * w;
      }
    return s1 * s1 + s2;
  }
  // film.wgsl:1085-1095
  R apply_a(int i, int j, size_t c) const {
    R k = kappa(), pc = cg_p[c], acc_v = pc;
    for (int f = 0; f < 8; ++f) {
      size_t nc;
      R mw;
      if (cg_nb(f, i, j, nc, mw)) acc_v += k * mw * (pc - cg_p[nc]);
    }
    if (h[c] > 0) acc_v += front3[0] * lap_w(i, j, c, 3);
    return acc_v;
  }
  // film.wgsl:1110-1141
  R k_cg_init_cell(int i, int j) {
    size_t c = idx(i, j);
    R k = kappa(), hc = h[c], uc = hold_u(c);
    R diag = 1, b = hc, ax = hc;
    for (int f = 0; f < 8; ++f) {
      size_t nc;
      R mw;
      if (cg_nb(f, i, j, nc, mw)) {
        diag += k * mw;
        b += k * mw * (hold_u(nc) - uc);
        ax += k * mw * (hc - h[nc]);
      }
    }
    if (hc > 0) {
      R cc = front3[0];
      diag += cc * lap_diag(i, j);
      b -= cc * lap_w(i, j, c, 2);
      ax += cc * lap_w(i, j, c, 3);
    }
    R r = b - ax;
    cg_d[c] = diag;
    cg_x[c] = hc;
    cg_r[c] = r;
    cg_p[c] = r / diag;
    return r * r / diag;
  }
  R pot(size_t c, const std::vector<R>& hh) const {  // film.wgsl:1227-1229, h as of before cg_finish
    R hold = 0;
    if (hh[c] > 0) hold = hold_level(nose_dist(c));
    return cg_x[c] + (m[c] - hold);
  }
  // film.wgsl:1232-1274 (reads h as of before the dispatch: Jacobi)
  void k_cg_finish_cell(int i, int j, const std::vector<R>& h_old, R& dv, R& tv, bool& moved) {
    size_t c = idx(i, j);
    R h0 = h_old[c], hn = std::max(cg_x[c], R(0));
    R rg = phys[0] * g[2] * inv_dx, pc = pot(c, h_old);
    const R wa = F(0.6666667f), wdf = F(0.23570226f), s2 = F(0.70710678f);
    R f[4] = {0, 0, 0, 0};
    const R* mob = &cg_m[4 * c];
    if (mob[0] > 0) f[0] = wa * mob[0] * rg * (pc - pot(idx(i + 1, j), h_old));
    if (mob[1] > 0) f[1] = wa * mob[1] * rg * (pc - pot(idx(i, j + 1), h_old));
    if (mob[2] > 0) f[2] = wdf * mob[2] * rg * (pc - pot(idx(i + 1, j + 1), h_old)) * s2;
    if (mob[3] > 0) f[3] = wdf * mob[3] * rg * (pc - pot(idx(i + 1, j - 1), h_old)) * s2;
    if (h0 > 0) {
      R kc = front3[1], tc = cg_t[c];
      if (i + 1 < (int)W) { size_t n = idx(i + 1, j); if (h_old[n] > 0 && cell_active(i + 1, j)) f[0] += wa * kc * (cg_t[n] - tc); }
      if (j + 1 < (int)H) { size_t n = idx(i, j + 1); if (h_old[n] > 0 && cell_active(i, j + 1)) f[1] += wa * kc * (cg_t[n] - tc); }
      if (i + 1 < (int)W && j + 1 < (int)H) { size_t n = idx(i + 1, j + 1); if (h_old[n] > 0 && cell_active(i + 1, j + 1)) f[2] += wdf * kc * (cg_t[n] - tc) * s2; }
      if (i + 1 < (int)W && j > 0) { size_t n = idx(i + 1, j - 1); if (h_old[n] > 0 && cell_active(i + 1, j - 1)) f[3] += wdf * kc * (cg_t[n] - tc) * s2; }
    }
    for (int k = 0; k < 4; ++k) acc[4 * c + k] += f[k] * front[3];
    h[c] = hn;
    moved = std::fabs(hn - h0) > F(1e-6f);
    dv = hn - h0;
    tv = hn;
  }
  // the shader's workgroup tree: for s = 128 .. 1, a[li] += a[li + s]
  static R tree256(R* a) {
    for (int st = 128; st > 0; st >>= 1)
      for (int li = 0; li < st; ++li) a[li] += a[li + st];
    return a[0];
  }
  // total_parts (film.wgsl:1157-1168): strided sums of the tile partials, then the tree
  R total_parts(const std::vector<R>& part) const {
    R a[256];
    for (size_t l = 0; l < 256; ++l) {
      R v = 0;
      for (size_t t = l; t < cg_tiles.size(); t += 256) v += part[t];
      a[l] = v;
    }
    return tree256(a);
  }
  // a tile-list dispatch whose invocations each give one value v (0 outside
  // the grid) summed per tile by the workgroup tree into part[w]
  template <class Fn>
  void cg_tiles_sum(std::vector<R>& part, Fn fn) {
#pragma omp parallel for schedule(dynamic, 1)
    for (long w = 0; w < (long)cg_tiles.size(); ++w) {
      uint32_t t = cg_tiles[w];
      R a[256];
      for (int li = 0; li < 256; ++li) {
        int i = (int)(t % TW) * 16 + li % 16, j = (int)(t / TW) * 16 + li / 16;
        a[li] = in_grid(i, j) ? fn(i, j) : R(0);
      }
      part[w] = tree256(a);
    }
  }
  template <class Fn>
  void cg_tiles_each(Fn fn) {
#pragma omp parallel for schedule(dynamic, 1)
    for (long w = 0; w < (long)cg_tiles.size(); ++w) {
      uint32_t t = cg_tiles[w];
      for (int li = 0; li < 256; ++li) {
        int i = (int)(t % TW) * 16 + li % 16, j = (int)(t / TW) * 16 + li / 16;
        if (in_grid(i, j)) fn(i, j);
      }
    }
  }
  // one implicit step (src/film/mod.rs:1374-1407)
  void run_implicit_step(uint32_t iters) {
    cg_alloc();
    cg_tiles.clear();
    for (uint32_t t = 0; t < TW * TH; ++t)
      if (tile_flags[t] & 32u) cg_tiles.push_back(t);
    run_laplacian();
    cg_tiles_each([&](int i, int j) { k_cg_setup_cell(i, j); });
    cg_tiles_each([&](int i, int j) {  // cg_lap_h
      size_t c = idx(i, j);
      cg_t[c] = lap_w(i, j, c, 1);
      cg_t2[c] = lap_w(i, j, c, 5);
    });
    cg_tiles_sum(cg_part, [&](int i, int j) { return k_cg_init_cell(i, j); });
    R rz = total_parts(cg_part);  // cg_reduce_init
    for (int k = 0; k < 4; ++k) cg_s[0][k] = cg_s[1][k] = 0;
    cg_s[0][0] = cg_s[1][0] = rz;
    for (uint32_t it = 0; it < iters; ++it) {
      cg_tiles_each([&](int i, int j) { size_t c = idx(i, j); cg_t[c] = lap_w(i, j, c, 0); });  // cg_lap_p
      cg_tiles_sum(cg_part, [&](int i, int j) {  // cg_iter_a
        size_t c = idx(i, j);
        R q = apply_a(i, j, c);
        cg_q[c] = q;
        return cg_p[c] * q;
      });
      {  // cg_reduce_a
        R pq = total_parts(cg_part), alpha = 0;
        if (pq > 0) alpha = cg_s[0][0] / pq;
        cg_s[0][1] = pq;
        cg_s[0][2] = alpha;
        cg_s[0][3] = 0;
      }
      R alpha = cg_s[0][2];
      cg_tiles_sum(cg_part, [&](int i, int j) {  // cg_iter_b
        size_t c = idx(i, j);
        R r = cg_r[c] - alpha * cg_q[c];
        cg_x[c] = cg_x[c] + alpha * cg_p[c];
        cg_r[c] = r;
        return r * r / cg_d[c];
      });
      {  // cg_reduce_b
        R rz2 = total_parts(cg_part), beta = 0;
        if (cg_s[0][0] > 0) beta = rz2 / cg_s[0][0];
        cg_s[0][0] = rz2;
        cg_s[0][3] = beta;
      }
      R beta = cg_s[0][3];
      cg_tiles_each([&](int i, int j) { size_t c = idx(i, j); cg_p[c] = cg_r[c] / cg_d[c] + beta * cg_p[c]; });
    }
    cg_tiles_each([&](int i, int j) { size_t c = idx(i, j); cg_t[c] = lap_w(i, j, c, 4); });  // cg_lap_u
    {  // cg_finish
      std::vector<R> h_old = h;
#pragma omp parallel for schedule(dynamic, 1)
      for (long w = 0; w < (long)cg_tiles.size(); ++w) {
        uint32_t t = cg_tiles[w];
        R a[256], tv_sum = 0;
        bool any = false;
        R tvs[256];
        for (int li = 0; li < 256; ++li) {
          int i = (int)(t % TW) * 16 + li % 16, j = (int)(t / TW) * 16 + li / 16;
          R dv = 0, tv = 0;
          bool mv = false;
          if (in_grid(i, j)) k_cg_finish_cell(i, j, h_old, dv, tv, mv);
          a[li] = dv;
          tvs[li] = tv;
          any = any || mv;
        }
        cg_part[w] = tree256(a);
        for (int li = 0; li < 256; ++li) tv_sum += tvs[li];
        cg_part2[w] = tv_sum;
        if (any) tile_moved[t] = 1u;
      }
    }
    {  // cg_reduce_mass
      R a[256], b[256];
      for (size_t l = 0; l < 256; ++l) {
        R d = 0, tot = 0;
        for (size_t t = l; t < cg_tiles.size(); t += 256) { d += cg_part[t]; tot += cg_part2[t]; }
        a[l] = d;
        b[l] = tot;
      }
      for (int st = 128; st > 0; st >>= 1)
        for (int li = 0; li < st; ++li) { a[li] += a[li + st]; b[li] += b[li + st]; }
      R x1 = cg_s[1][0], s0x = cg_s[0][0];
      cg_s[1][0] = x1; cg_s[1][1] = a[0]; cg_s[1][2] = b[0]; cg_s[1][3] = s0x;
    }
    if (cg_s[1][2] > 0) {  // cg_rescale
      R fr = R(1) - cg_s[1][1] / cg_s[1][2];
      cg_tiles_each([&](int i, int j) { size_t c = idx(i, j); h[c] = std::max(h[c] * fr, R(0)); });
    }
  }

  // ---- deposits (shaders/deposit.wgsl; tables binned by upload_deposits,
  // src/film/mod.rs:1175-1224, on the host) ----
  std::vector<cf_deposit> deps;
  std::vector<uint32_t> dep_start, dep_count, dep_items;  // per 64x64-cell tile

  // deposit.wgsl:6-29; mix(a, b, t) = a (1 - t) + b t as WGSL defines it
  static R ribbon_height(R px, R py, const cf_deposit& d) {
    R abx = (R)d.p1[0] - (R)d.p0[0], aby = (R)d.p1[1] - (R)d.p0[1];
    R l2 = abx * abx + aby * aby;
    R r0 = d.r0, r1 = d.r1, h0 = d.h0;
    if (l2 <= 0) {
      R qx = px - (R)d.p0[0], qy = py - (R)d.p0[1];
      R x = std::sqrt(qx * qx + qy * qy) / r0;
      return x < 1 ? h0 * (1 - x * x) : R(0);
    }
    R l = std::sqrt(l2);
    R ux = abx / l, uy = aby / l;
    R q0x = px - (R)d.p0[0], q0y = py - (R)d.p0[1], q1x = px - (R)d.p1[0], q1y = py - (R)d.p1[1];
    bool cs = (d.kind & 2u) != 0u, ce = (d.kind & 4u) != 0u;
    if (!cs && q0x * (R)d.n0[0] + q0y * (R)d.n0[1] < 0) return 0;
    if (!ce && q1x * (R)d.n1[0] + q1y * (R)d.n1[1] >= 0) return 0;
    R u = q0x * ux + q0y * uy;
    if (u < -r0 || u > l + r1) return 0;
    R dist = std::fabs(q0x * uy - q0y * ux);
    if (cs && u < 0) dist = std::sqrt(q0x * q0x + q0y * q0y);
    if (ce && u > l) dist = std::sqrt(q1x * q1x + q1y * q1y);
    R t = std::min(std::max(u / l, R(0)), R(1));
    R rt = r0 * (1 - t) + r1 * t;
    R x = dist / rt;
    return x < 1 ? h0 * (rt / r0) * (1 - x * x) : R(0);
  }
  // common.wgsl:81-84
  static uint32_t lay_pack(uint32_t method, R ux, R uy) {
    R turn = std::atan2(uy, ux) / R(6.2831853f) + R(0.5f);
    return (method & 0xffu) | ((uint32_t)(std::min(std::max(turn, R(0)), R(1)) * R(65535)) << 8);
  }
  // deposit.wgsl:31-75 over every cell of the grid
  void run_deposit() {
    if (dep_items.empty() || dep_count.empty()) return;
    uint32_t t64 = (W + 63) / 64;
#pragma omp parallel for schedule(static)
    for (long jj = 0; jj < (long)H; ++jj) {
      uint32_t j = (uint32_t)jj;
      for (uint32_t i = 0; i < W; ++i) {
        uint32_t tile = i / 64 + (j / 64) * t64;
        uint32_t n = dep_count[tile];
        if (n == 0) continue;
        uint32_t start = dep_start[tile];
        size_t c = idx(i, j);
        R px = ((R)i + R(0.5)) * dx, py = ((R)j + R(0.5)) * dx;
        Stack s;
        stack_load(c, s);
        R added = 0, top_add = 0;
        uint32_t top_lay = 0;
        for (uint32_t q = 0; q < n; ++q) {
          const cf_deposit& d = deps[dep_items[start + q]];
          R abx = (R)d.p1[0] - (R)d.p0[0], aby = (R)d.p1[1] - (R)d.p0[1];
          R along = std::min(std::max(((px - (R)d.p0[0]) * abx + (py - (R)d.p0[1]) * aby) /
                                          std::max(abx * abx + aby * aby, (R)1e-30f),
                                      R(0)),
                             R(1));
          R reach = R(1.415f) * (R)std::max(d.r0, d.r1) + R(0.6f) * dx;
          R ox = px - (R)d.p0[0] - along * abx, oy = py - (R)d.p0[1] - along * aby;
          if (ox * ox + oy * oy > reach * reach) continue;
          R add = 0;
          for (int sy = 0; sy < 4; ++sy)
            for (int sx = 0; sx < 4; ++sx)
              add += R(0.0625f) * ribbon_height(px + ((R)sx - R(1.5)) * (R(0.25f) * dx),
                                                py + ((R)sy - R(1.5)) * (R(0.25f) * dx), d);
          if (add > 0) {
            R pg[16];
            for (int k = 0; k < 8; ++k) {  // unpack2x16float pairs (common.wgsl:173-180)
              pg[2 * k] = (R)f16_value((uint16_t)(d.pig[k] & 0xffffu));
              pg[2 * k + 1] = (R)f16_value((uint16_t)(d.pig[k] >> 16));
            }
            stack_push_top(s, add, pg, R(0));
            added += add;
            if (add > top_add) {
              top_add = add;
              R ex = abx + (R)1e-9f, ey = aby;
              R el = std::sqrt(ex * ex + ey * ey);
              top_lay = lay_pack(d.kind >> 8, ex / el, ey / el);
            }
          }
        }
        if (added > 0) {
          h[c] = h[c] + added;
          lay[c] = top_lay;
          tile_moved[i / 16 + (j / 16) * TW] = 1u;  // mark_moved
          stack_compact(s);
          stack_store_to(c, s, sh, scu, pig);
        }
      }
    }
  }

  // Film::encode_frame, src/film/mod.rs:1322-1462 (simulation portion;
  // journal / brush / knife / slump / pool8 are not on the path).  The
  // deposits uploaded since the last frame are laid first, then dropped; the
  // implicit hydrostatic steps run after clear_acc.
  void encode_frame(uint32_t substeps) {
    if (!dep_items.empty()) run_deposit();
    dep_items.clear();
    k_mark_tiles();
    k_compact_tiles();
    run_cure();
    run_clear_acc();
    for (uint32_t s = 0; s < PF.implicit_steps; ++s) run_implicit_step(S.implicit_iters);
    for (uint32_t s = 0; s < substeps; ++s) {
      run_laplacian();
      run_plug();
      run_fluxes();
      run_limiter();
      run_apply();
      run_nose();
    }
    run_laplacian();
    run_strata_split();
    k_reduce_tiles();
    run_strata_limit();
    run_strata_update();
    run_copy_back();
    for (int r = 0; r < 6; ++r) run_strata_fill();
    run_shade();
  }

  // One adaptive step (see adaptive_dt): dt from the stats of the last frame.
  float step_adaptive(float dt_max) {
    float d = adaptive_dt(S, W, dt_max, h_max_stat, mu_min_stat);
    do_update_params(d, 1);
    encode_frame(1);
    return d;
  }

  // Film::dry_now, src/film/mod.rs:1230-1244
  void dry_now() {
    float saved = (float)cure[0];
    cure[0] = (R)(4.0f / std::max(PF.p.frame_dt, 1e-4f));
    run_cure();
    cure[0] = (R)saved;
  }

  double mass() const {
    double s = 0;
    for (size_t c = 0; c < N; ++c) s += (double)h[c] + (double)m[c];
    return s * (double)PF.p.dx * (double)PF.p.dx;
  }
};

}  // namespace cfo
