// capi.cu — the C ABI of include/canvaz_film.h over the sm_103a kernels.
//
// A cf_film owns one device arena holding every per-cell plane (the
// reference's buffers of Film::new, src/film/mod.rs:586-628, in the same
// layout) plus the device-resident params and stats.  All entry points return
// cf_status; CUDA errors are caught and reported through cf_last_error.
#include <cuda.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <new>
#include <string>
#include <vector>

#include "../../include/canvaz_film.h"
#include "film_handle.h"
#include "film_kernels.h"

static std::string g_create_err;

static float to_rad(float d) { return d * (3.14159265358979323846f / 180.0f); }

static void gravity_vec(const cf_settings& s, float g[3]) {  // src/film/mod.rs:861-867
  float tilt = to_rad(s.tilt_deg), dir = to_rad(s.tilt_dir_deg);
  float gxy = s.gravity * std::sin(tilt);
  g[0] = gxy * std::cos(dir);
  g[1] = gxy * std::sin(dir);
  g[2] = std::fmax(s.gravity * std::cos(tilt), 0.0f);
}

// Film::update_params, src/film/mod.rs:869-917 (f32 arithmetic as in Rust).
static void pack_params_impl(const cf_settings& s, uint32_t w, uint32_t h, float frame_dt, uint32_t substeps,
                             float h_max_stat, float h_max_pending, float mu_min_stat, cf_params& P,
                             uint32_t& implicit_steps) {
  std::memset(&P, 0, sizeof(P));
  float dx = s.width_m / (float)w;
  P.size[0] = w; P.size[1] = h;
  P.tiles[0] = (w + 63) / 64; P.tiles[1] = (h + 63) / 64;
  P.dx = dx; P.inv_dx = 1.0f / dx;
  float g[3];
  gravity_vec(s, g);
  float theta = to_rad(s.contact_angle_deg);
  float pi_a = 3.0f * s.sigma * (1.0f - std::cos(theta)) / s.h_star;
  float dt = frame_dt / (float)substeps;
  float m_cap_exp = 0.5f * dx * dx * dx * dx / (32.0f * s.sigma * dt);
  float m_cap = std::fmax(std::fmin(s.m_cap, m_cap_exp), 1e-14f);
  float m_exp = 0.1f * dx * dx / (dt * s.rho * std::fmax(g[2], 0.1f));
  P.dt = dt; P.frame_dt = frame_dt;
  P.g[0] = g[0]; P.g[1] = g[1]; P.g[2] = g[2]; P.g[3] = s.gravity;
  P.phys[0] = s.rho; P.phys[1] = s.sigma; P.phys[2] = s.n_index;
  P.phys[3] = (s.capillary && !s.no_cap) ? m_cap : 0.0f;
  float lc = std::sqrt(s.sigma / (s.rho * 9.81f));
  P.ein[0] = std::fmax(std::tan(theta), 0.05f);
  P.ein[1] = lc * std::sin(0.5f * theta);
  P.ein[2] = pi_a;
  P.ein[3] = s.h_min;
  P.cure[0] = s.cure_rate; P.cure[1] = s.tau_cure; P.cure[2] = s.lnmu_cure; P.cure[3] = s.h_star;
  P.misc[0] = 2.0e-6f; P.misc[1] = 0.12f; P.misc[2] = s.medium_mu; P.misc[3] = std::fmin(m_exp, s.m_cap_hydro);
  P.flags[0] = s.debug_view; P.flags[1] = (uint32_t)(s.slump != 0);
  float lc_z = std::sqrt(s.sigma / (s.rho * std::fmax(g[2], 0.1f)));
  float cap_explicit = std::fmin(m_exp, s.m_cap_hydro);
  float h_big = std::fmax(std::fmax(h_max_stat, h_max_pending), 1e-4f);
  float m_phys = h_big * h_big * h_big / (3.0f * std::fmax(mu_min_stat, 1e-3f)) - cap_explicit;
  float kappa_frame = frame_dt * s.rho * std::fmax(g[2], 0.1f) / (dx * dx);
  uint32_t n_i = 0;
  if (m_phys > 0.0f) {
    float v = std::fmax(std::ceil(kappa_frame * m_phys / 40.0f), 1.0f);
    n_i = std::min((uint32_t)v, 4u);
  }
  float dt_i = frame_dt / (float)std::max(n_i, 1u);
  P.front[2] = 40.0f * dx * dx / (dt_i * s.rho * std::fmax(g[2], 0.1f));
  P.front[3] = dt_i;
  implicit_steps = s.implicit_hydro ? n_i : 0;
  float m_phys_cap = h_big * h_big * h_big / (3.0f * std::fmax(mu_min_stat, 1e-3f));
  float dx2 = dx * dx, dx4 = dx2 * dx2;
  float m_cap_impl = (s.cap_cond / 28.0f) * dx4 / (dt_i * s.sigma);
  float m_c = s.capillary_implicit ? std::fmin(m_phys_cap, m_cap_impl) : 0.0f;
  P.front3[0] = dt_i * s.sigma * m_c / dx4;
  P.front3[1] = m_c * s.sigma / (dx * dx * dx);
  P.front3[2] = m_c;
  P.front3[3] = s.fcap_exp;
  P.front[0] = s.no_hold ? 0.0f : 2.0f * lc_z * std::sin(0.5f * theta);
  P.front[1] = dx / lc_z;
  float hyst = s.hyst_deg >= 0.0f ? s.hyst_deg : s.hysteresis_deg;
  uint32_t fl = (uint32_t)(s.no_transl != 0) | ((uint32_t)(s.no_shape != 0) << 1);
  P.front2[0] = to_rad(hyst); P.front2[1] = s.kshape; P.front2[2] = s.kline; P.front2[3] = (float)fl;
}

static void pack_params(cf_film* f, float frame_dt, uint32_t substeps) {
  pack_params_impl(f->S, f->w, f->h, frame_dt, substeps, f->h_max_stat, f->h_max_pending, f->mu_min_stat, f->P,
                   f->implicit_steps);
  f->params_dirty = true;
}

static void fill_devparams(cf_film* f, DevParams& D, float dt_max) {
  std::memset(&D, 0, sizeof(D));
  D.p = f->P;
  float g[3];
  gravity_vec(f->S, g);
  D.gxy = std::sqrt(g[0] * g[0] + g[1] * g[1]);
  D.s_rho = f->S.rho; D.s_sigma = f->S.sigma; D.s_vcap = f->S.v_cap; D.s_mcap = f->S.m_cap;
  D.s_mcap_hydro = f->S.m_cap_hydro; D.s_cap_cond = f->S.cap_cond; D.s_gz = g[2];
  D.s_capillary = f->S.capillary && !f->S.no_cap;
  D.s_cap_implicit = f->S.capillary_implicit;
  D.s_implicit = f->S.implicit_hydro;
  D.dt_max = dt_max;
  D.implicit_steps = f->implicit_steps;
  D.implicit_iters = f->S.implicit_iters;
  D.frames = f->frames;
  const cf_params& P = f->P;
  D.hold1 = P.front[0] * (1.0f - std::exp(-0.5f * P.front[1]));
  D.cox_theta = std::atan(P.ein[0]);
  D.cox_span = std::fmax(P.front[0] - D.hold1, 1e-6f);
  D.cox_adv = std::fmin(D.cox_theta + P.front2[0], 3.1f);
  D.gc_max = P.phys[1] / (1e-3f * 1e-3f);  // one f32 division, as each face did it
}

// Copies the host-packed params to the device on `st`.  The pinned staging
// buffer is rewritten only after the previous copy out of it has executed.
cf_status upload_params(cf_film* f, cudaStream_t st, float dt_max) {
  if (!f->params_dirty) return CF_OK;
  CUDA_TRY(f, cudaEventSynchronize(f->params_ev));
  fill_devparams(f, *f->h_params, dt_max);
  CUDA_TRY(f, cudaMemcpyAsync(f->d_params, f->h_params, sizeof(DevParams), cudaMemcpyHostToDevice, st));
  CUDA_TRY(f, cudaEventRecord(f->params_ev, st));
  f->params_dirty = false;
  return CF_OK;
}

static cf_status check_launch(cf_film* f) {
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    f->err = std::string("kernel launch: ") + cudaGetErrorString(e);
    return CF_ERR_CUDA;
  }
  return CF_OK;
}

extern "C" {

cf_status cf_settings_default(cf_settings* s) {  // FilmSettings::default, src/film/mod.rs:315-350
  if (!s) return CF_ERR_INVALID_ARG;
  std::memset(s, 0, sizeof(*s));
  s->width_m = 1.2f; s->height_m = 0.8f; s->rho = 1000.0f; s->sigma = 0.035f; s->n_index = 1.0f;
  s->m_cap = 1.0e-8f; s->contact_angle_deg = 45.0f; s->hysteresis_deg = 15.0f; s->h_star = 2.0e-5f;
  s->raw_canvas = 1; s->weave_um = 25.0f; s->cure_rate = 1.0f / 600.0f; s->tau_cure = 300.0f;
  s->lnmu_cure = 5.0f; s->v_cap = 1.0f; s->tilt_deg = 0.0f; s->tilt_dir_deg = -90.0f; s->gravity = 9.81f;
  s->medium_mu = 0.08f; s->debug_view = 0; s->h_min = 1.5e-5f; s->m_cap_hydro = 1.0e-7f;
  s->max_substeps = 64; s->min_substeps = 4; s->implicit_iters = 40; s->implicit_hydro = 1; s->slump = 0;
  s->capillary = 1; s->capillary_implicit = 0; s->kshape = 1.0f; s->kline = 0.0f; s->hyst_deg = -1.0f;
  s->fcap_exp = 2.5f; s->cap_cond = 80.0f; s->all_active = 0;
  return CF_OK;
}

const char* cf_last_error(const cf_film* f) { return f ? f->err.c_str() : g_create_err.c_str(); }

cf_status cf_pack_params(const cf_settings* s, uint32_t w, uint32_t h, float frame_dt, uint32_t substeps,
                         float h_max, float mu_min, cf_params* out, uint32_t* implicit_steps) {
  if (!s || !out || w == 0 || h == 0 || !(frame_dt > 0.f) || substeps == 0) return CF_ERR_INVALID_ARG;
  uint32_t ni = 0;
  pack_params_impl(*s, w, h, frame_dt, substeps, h_max, 0.0f, mu_min, *out, ni);
  if (implicit_steps) *implicit_steps = ni;
  return CF_OK;
}

}  // extern "C"

// cuTensorMapEncodeTiled, found through the runtime (the library does not
// link the driver library itself); null where the driver does not offer it.
using EncodeTiledFn = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                   const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                   CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
static EncodeTiledFn encode_tiled() {
  static EncodeTiledFn fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q{};
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<EncodeTiledFn>(p);
    cudaGetLastError();
  });
  return fn;
}

// The tile kernels' descriptors (cfk::FlowMap order): h, m, the front
// offsets, their snapshot and the heights after apply as 24 x 24 boxes of
// 4-byte cells, the rheology planes as 24 x 24 boxes of f32 or 32 x 24 boxes
// of bf16, the flux as 20 x 20 boxes of 16-byte cells; zero fill outside the
// grid.  Each
// row pitch must be a multiple of 16 bytes, and the grid at least one box:
// returns false otherwise (the tile then stages with plain loads).
static bool encode_flow_maps(const cfk::Film& F, int precision, CUtensorMap maps[cfk::FLOW_MAPS]) {
  EncodeTiledFn enc = encode_tiled();
  const bool b16 = precision == CF_PREC_BF16;
  const size_t rb = b16 ? 2 : 4;
  if (!enc || F.w < 32 || F.h < 24 || (F.w * 4u) % 16u != 0u || (F.w * rb) % 16u != 0u) return false;
  auto one = [&](CUtensorMap* m, void* base, CUtensorMapDataType t, size_t esz, cuuint32_t box_w) {
    const cuuint64_t dims[2] = {F.w, F.h};
    const cuuint64_t strides[1] = {(cuuint64_t)F.w * esz};
    const cuuint32_t box[2] = {box_w, 24};
    const cuuint32_t es[2] = {1, 1};
    return enc(m, t, 2, base, dims, strides, box, es, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
               CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
  };
  // the flux plane (4 floats a cell) as a 4w x h grid of floats, in 80 x 20
  // boxes: 20 x 20 cells
  auto flux_map = [&](CUtensorMap* m) {
    const cuuint64_t dims[2] = {4ull * F.w, F.h};
    const cuuint64_t strides[1] = {(cuuint64_t)F.w * 16};
    const cuuint32_t box[2] = {80, 20};
    const cuuint32_t es[2] = {1, 1};
    return enc(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, F.flux, dims, strides, box, es, CU_TENSOR_MAP_INTERLEAVE_NONE,
               CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
               CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
  };
  const CUtensorMapDataType rt = b16 ? CU_TENSOR_MAP_DATA_TYPE_BFLOAT16 : CU_TENSOR_MAP_DATA_TYPE_FLOAT32;
  const cuuint32_t rw = b16 ? 32 : 24;
  return one(&maps[cfk::MAP_H], F.hh, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, 24) &&
         one(&maps[cfk::MAP_M], F.m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, 24) &&
         one(&maps[cfk::MAP_DELTA], F.delta, CU_TENSOR_MAP_DATA_TYPE_UINT32, 4, 24) &&
         one(&maps[cfk::MAP_MU], F.mu, rt, rb, rw) && one(&maps[cfk::MAP_TAU], F.tau, rt, rb, rw) &&
         one(&maps[cfk::MAP_N], F.nn, rt, rb, rw) &&
         one(&maps[cfk::MAP_DELTA_OLD], F.delta_old, CU_TENSOR_MAP_DATA_TYPE_UINT32, 4, 24) &&
         one(&maps[cfk::MAP_H_NEXT], F.h_next, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, 24) &&
         flux_map(&maps[cfk::MAP_FLUX]);
}

// The device planes of a film (n cells, nt tiles) in arena order; add(p, bytes)
// receives each plane's pointer slot and size.
template <class Add>
static void carve_planes(cfk::Film& F, size_t n, size_t nt, int precision, bool cg, Add add) {
  const size_t pig_b = precision == CF_PREC_FP32 ? 4 : 2, rh_b = precision == CF_PREC_BF16 ? 2 : 4;
  add((void**)&F.hh, 4 * n); add((void**)&F.m, 4 * n); add(&F.mu, rh_b * n); add(&F.tau, rh_b * n);
  add(&F.nn, rh_b * n); add((void**)&F.delta, 4 * n); add((void**)&F.delta_old, 4 * n);
  add((void**)&F.lay, 4 * n); add((void**)&F.pres, 8 * n); add((void**)&F.fnorm, 8 * n);
  add((void**)&F.flux, 16 * n); add((void**)&F.acc, 16 * n); add((void**)&F.acc_s, 64 * n);
  add((void**)&F.alpha_s, 16 * n); add((void**)&F.alpha, 4 * n); add((void**)&F.tmp, 4 * n);
  add((void**)&F.h_frame, 4 * n); add((void**)&F.h_next, 4 * n); add((void**)&F.sh, 16 * n); add((void**)&F.scu, 16 * n);
  add((void**)&F.sh2, 16 * n); add((void**)&F.scu2, 16 * n); add((void**)&F.pig, 64 * pig_b * n);
  add((void**)&F.pig2, 64 * pig_b * n); add((void**)&F.agg, 16 * n); add((void**)&F.refl, 32 * n);
  add((void**)&F.color, 8 * n); add((void**)&F.detail, 8 * n); add((void**)&F.tile_flags, 4 * nt); add((void**)&F.tile_moved, 4 * nt);
  add((void**)&F.fill_src, 4 * n); add((void**)&F.fflags, 4 * n); add((void**)&F.shade_state, n);
  add((void**)&F.spec, 64 * n);
  add((void**)&F.full_list, 4 * n); add((void**)&F.fill_list, 4 * n);
  if (cg) {  // implicit hydrostatic step (settings.implicit_hydro)
    add((void**)&F.cg_m, 16 * n);
    for (float** p : {&F.cg_d, &F.cg_x, &F.cg_r, &F.cg_p, &F.cg_pa, &F.cg_pb, &F.cg_q, &F.cg_t, &F.cg_t2})
      add((void**)p, 4 * n);
    add((void**)&F.cg_part, 4 * nt); add((void**)&F.cg_part2, 4 * nt); add((void**)&F.cg, sizeof(cfk::CgState));
    add((void**)&F.cg_cnt, 4 * ((nt + 31) / 32));
  }
}

extern "C" {

cf_status cf_film_bytes(uint32_t w, uint32_t h, int32_t precision, uint64_t* bytes) {
  if (!bytes || w == 0 || h == 0 || w > 65536 || h > 65536 || precision < 0 || precision > 2)
    return CF_ERR_INVALID_ARG;
  const size_t n = (size_t)w * h, nt = (size_t)((w + 15) / 16) * ((h + 15) / 16);
  cfk::Film F{};
  size_t total = 0;
  carve_planes(F, n, nt, precision, false, [&](void**, size_t b) { total += (b + 255) & ~(size_t)255; });
  total += sizeof(DevParams) + sizeof(DevStats) + sizeof(float) * 528 + 2 * sizeof(cfk::Film) + sizeof(uint2) * nt +
           sizeof(CUtensorMap) * cfk::FLOW_MAPS;
  *bytes = total;
  return CF_OK;
}

cf_status cf_create(const cf_settings* s, uint32_t w, uint32_t h, int32_t precision, cf_film** out) {
  if (!s || !out || w == 0 || h == 0 || w > 65536 || h > 65536 || (uint64_t)w * h > (1ull << 30) || precision < 0 ||
      precision > 2) {
    g_create_err = "cf_create: invalid argument";
    return CF_ERR_INVALID_ARG;
  }
  if (s->width_m <= 0.f || s->rho <= 0.f || s->sigma <= 0.f || s->h_star <= 0.f) {
    g_create_err = "cf_create: non-positive physical setting";
    return CF_ERR_INVALID_ARG;
  }
  *out = nullptr;
  cf_film* f = new (std::nothrow) cf_film;
  if (!f) return CF_ERR_OUT_OF_MEMORY;
  f->S = *s;
  f->w = w; f->h = h; f->tw = (w + 15) / 16; f->th = (h + 15) / 16; f->prec = precision;
  f->n = (size_t)w * h;
  auto bail = [&](cf_status st) {
    g_create_err = f->err;
    cf_destroy(f);
    return st;
  };
  if (cudaGetDevice(&f->device) != cudaSuccess) { f->err = "no CUDA device"; return bail(CF_ERR_CUDA); }
  cudaDeviceGetAttribute(&f->sms, cudaDevAttrMultiProcessorCount, f->device);
  size_t n = f->n, nt = (size_t)f->tw * f->th;
  // carve the arena (256-byte aligned planes)
  struct Slot { void** p; size_t bytes; };
  std::vector<Slot> slots;
  cfk::Film& F = f->F;
  carve_planes(F, n, nt, precision, s->implicit_hydro != 0, [&](void** p, size_t b) { slots.push_back({p, b}); });
  size_t total = 0;
  for (auto& sl : slots) total += (sl.bytes + 255) & ~(size_t)255;
  cudaError_t e = cudaMalloc(&f->arena, total);
  if (e != cudaSuccess) {
    f->err = std::string("cudaMalloc arena: ") + cudaGetErrorString(e);
    cudaGetLastError();
    return bail(CF_ERR_OUT_OF_MEMORY);
  }
  f->arena_bytes = total;
  size_t off = 0;
  for (auto& sl : slots) {
    *sl.p = (char*)f->arena + off;
    off += (sl.bytes + 255) & ~(size_t)255;
  }
  if (cudaMalloc(&f->d_params, sizeof(DevParams)) != cudaSuccess ||
      cudaMalloc(&f->d_stats, sizeof(DevStats)) != cudaSuccess ||
      cudaMalloc(&f->d_tables, sizeof(float) * (480 + 48)) != cudaSuccess ||
      cudaMallocHost(&f->h_params, sizeof(DevParams)) != cudaSuccess ||
      cudaEventCreateWithFlags(&f->params_ev, cudaEventDisableTiming) != cudaSuccess) {
    f->err = "cudaMalloc params/stats/tables";
    cudaGetLastError();
    return bail(CF_ERR_OUT_OF_MEMORY);
  }
  F.w = w; F.h = h; F.tw = f->tw; F.th = f->th; F.n = (uint32_t)n;
  F.persist_blocks = (uint32_t)std::max(f->sms, 1) * 8u;
  F.all_active = s->all_active ? 1u : 0u;
  F.P = f->d_params; F.stats = f->d_stats;
  F.pigtab = f->d_tables; F.cmf = f->d_tables + 480;
  {  // tensor-load descriptors of the flow tile's planes, where the pitch allows
    alignas(64) CUtensorMap maps[cfk::FLOW_MAPS];
    F.tmap = nullptr;
    if (encode_flow_maps(F, precision, maps)) {
      if (cudaMalloc(&f->d_tmaps, sizeof(maps)) != cudaSuccess ||
          cudaMemcpy(f->d_tmaps, maps, sizeof(maps), cudaMemcpyHostToDevice) != cudaSuccess) {
        f->err = "cudaMalloc tensor maps";
        cudaGetLastError();
        return bail(CF_ERR_OUT_OF_MEMORY);
      }
      F.tmap = f->d_tmaps;
    }
  }
  {  // the film's own packed view (see solo_view; its tile table is implicit)
    cfk::Film rec[2] = {F, F};
    std::swap(rec[1].sh, rec[1].sh2);
    std::swap(rec[1].scu, rec[1].scu2);
    if (cudaMalloc(&f->d_recs, sizeof(rec)) != cudaSuccess ||
        cudaMemcpy(f->d_recs, rec, sizeof(rec), cudaMemcpyHostToDevice) != cudaSuccess) {
      f->err = "cudaMalloc film records";
      cudaGetLastError();
      return bail(CF_ERR_OUT_OF_MEMORY);
    }
    f->sh_created = F.sh;
  }
  // Film::new: zeroed buffers, substrate refl, weave relief, rheo = (1, 0)
  if (cudaMemset(f->arena, 0, total) != cudaSuccess || cudaMemset(f->d_tables, 0, sizeof(float) * 528) != cudaSuccess ||
      cudaMemset(f->d_stats, 0, sizeof(DevStats)) != cudaSuccess) {
    f->err = "cudaMemset";
    return bail(CF_ERR_CUDA);
  }
  {
    std::vector<uint16_t> refl(16 * n);
    float bands[16];
    for (int b = 0; b < 16; ++b) {
      float t = (float)b / 15.0f;
      bands[b] = s->raw_canvas ? 0.50f + 0.16f * t : 0.84f + 0.04f * t;
    }
    uint16_t hb[16];
    for (int b = 0; b < 16; ++b) {  // f32 -> f16 round to nearest even (normal range)
      uint32_t u;
      std::memcpy(&u, &bands[b], 4);
      uint32_t sign = (u >> 16) & 0x8000u;
      int e8 = (int)((u >> 23) & 0xff) - 127 + 15;
      uint32_t mant = u & 0x7fffffu;
      uint32_t r = ((uint32_t)e8 << 10) | (mant >> 13);
      uint32_t rem = mant & 0x1fffu;
      if (rem > 0x1000u || (rem == 0x1000u && (r & 1u))) r += 1;
      hb[b] = (uint16_t)(sign | r);
    }
    for (size_t c = 0; c < n; ++c) std::memcpy(&refl[16 * c], hb, 32);
    std::vector<float> wv(n, 0.0f);
    float dx = s->width_m / (float)w, amp = s->weave_um * 1e-6f;
    if (amp > 0.0f) {  // weave, src/film/mod.rs:212-233
      float k = 6.28318530717958647692f / 1.4e-3f;
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
          wv[(size_t)j * w + i] = amp * (1.0f + 0.6f * sv + 0.4f * r);
        }
      }
    }
    std::vector<float2> rh(n, make_float2(1.0f, 0.0f));
    float2* d_rh = nullptr;
    if (cudaMemcpy(F.refl, refl.data(), 32 * n, cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemcpy(F.m, wv.data(), 4 * n, cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMalloc(&d_rh, 8 * n) != cudaSuccess ||
        cudaMemcpy(d_rh, rh.data(), 8 * n, cudaMemcpyHostToDevice) != cudaSuccess) {
      f->err = "initial upload";
      if (d_rh) cudaFree(d_rh);
      return bail(CF_ERR_CUDA);
    }
    cfk::launch_rheo_import(F, precision, d_rh, s->n_index, n, 0);
    cudaError_t e2 = cudaDeviceSynchronize();
    cudaFree(d_rh);
    if (e2 != cudaSuccess) { f->err = cudaGetErrorString(e2); return bail(CF_ERR_CUDA); }
  }
  pack_params(f, 1.0f / 60.0f, 1);
  cf_status st = upload_params(f, 0);
  if (st != CF_OK) return bail(st);
  if (cudaDeviceSynchronize() != cudaSuccess) { f->err = "sync"; return bail(CF_ERR_CUDA); }
  *out = f;
  return CF_OK;
}

cf_status cf_destroy(cf_film* f) {
  if (!f) return CF_ERR_INVALID_ARG;
  cudaDeviceSynchronize();
  if (f->batch) batch_forget(f);
  if (f->arena) cudaFree(f->arena);
  if (f->d_params) cudaFree(f->d_params);
  if (f->d_stats) cudaFree(f->d_stats);
  if (f->d_tables) cudaFree(f->d_tables);
  if (f->h_params) cudaFreeHost(f->h_params);
  if (f->params_ev) cudaEventDestroy(f->params_ev);
  if (f->d_recs) cudaFree(f->d_recs);
  if (f->d_tmaps) cudaFree(f->d_tmaps);
  if (f->d_deps) cudaFree(f->d_deps);
  if (f->d_dep_tiles) cudaFree(f->d_dep_tiles);
  if (f->d_dep_items) cudaFree(f->d_dep_items);
  delete f;
  return CF_OK;
}

cf_status cf_set_tables(cf_film* f, const float* pigtab, const float* cmf) {
  if (!f || !pigtab || !cmf) return fail(f, CF_ERR_INVALID_ARG, "cf_set_tables: null");
  CUDA_TRY(f, cudaMemcpy(f->d_tables, pigtab, sizeof(float) * 480, cudaMemcpyHostToDevice));
  CUDA_TRY(f, cudaMemcpy(f->d_tables + 480, cmf, sizeof(float) * 48, cudaMemcpyHostToDevice));
  CUDA_TRY(f, cudaMemset(f->F.shade_state, 0, f->n));  // dry colours depend on the CMF table
  return CF_OK;
}

static cf_status copy_plane(cf_film* f, void* dst, const void* src, size_t bytes, int device, bool to_dev) {
  cudaMemcpyKind k = device ? cudaMemcpyDeviceToDevice : (to_dev ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToHost);
  CUDA_TRY(f, cudaMemcpy(dst, src, bytes, k));
  return CF_OK;
}

// The address a kernel reads a host buffer at, when the buffer is page-locked
// CUDA host memory (else null: the buffer is staged through a copy).
static const void* kernel_readable_host(const void* p) {
  cudaPointerAttributes a{};
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  return a.type == cudaMemoryTypeHost ? a.devicePointer : nullptr;
}

// Where a kernel or an asynchronous copy can take a state plane from: device
// memory as it is, page-locked host memory at its device-side address; null
// for pageable host memory.
static const void* async_src(const cf_state_view* v, const void* p) {
  if (!p) return nullptr;
  return v->device ? p : kernel_readable_host(p);
}

// Everything of write_state after the planes are in place (src/film/mod.rs:
// 1307-1317): scratch cleared, every tile marked moved, the aggregates and
// colour of the uploaded strata, the tile stats.  Enqueued on `st`.
static cf_status write_state_tail(cf_film* f, cudaStream_t st) {
  cfk::Film& F = f->F;
  const size_t n = f->n, pig_b = f->prec == CF_PREC_FP32 ? 4 : 2;
  CUDA_TRY(f, cudaMemsetAsync(F.pres, 0, 8 * n, st));
  CUDA_TRY(f, cudaMemsetAsync(F.flux, 0, 16 * n, st));
  CUDA_TRY(f, cudaMemsetAsync(F.acc, 0, 16 * n, st));
  CUDA_TRY(f, cudaMemsetAsync(F.alpha, 0, 4 * n, st));
  CUDA_TRY(f, cudaMemsetAsync(F.delta, 0, 4 * n, st));
  CUDA_TRY(f, cudaMemsetAsync(F.tmp, 0, 4 * n, st));
  CUDA_TRY(f, cudaMemsetAsync(F.acc_s, 0, 64 * n, st));
  CUDA_TRY(f, cudaMemsetAsync(F.sh2, 0, 16 * n, st));
  CUDA_TRY(f, cudaMemsetAsync(F.pig2, 0, 64 * pig_b * n, st));
  CUDA_TRY(f, cudaMemsetAsync(F.alpha_s, 0, 16 * n, st));
  cfk::launch_fill_u32(F.tile_moved, 1u, (size_t)f->tw * f->th, st);
  cfk::launch_compose(solo_view(f), f->prec, 1, st);
  cfk::launch_reduce(solo_view(f), f->prec, st);
  CUDA_TRY(f, cudaGetLastError());
  return CF_OK;
}

// The planes of a view whose sources are device or page-locked host memory,
// enqueued on `st`.  Host planes move by the copy engines, so the SMs stay
// free for work on other streams: plain planes straight into place, the
// pigment and rheology planes (which change layout) into scratch planes that
// write_state clears anyway (pig2, acc_s), from which kernels convert them.
// A pigment source wider than the film's storage is converted by a kernel
// reading it in place.
// Uploads from host memory queue on the host link in call order, whatever
// stream they are on: each waits for the previous one's copies (not for its
// conversion kernels), so with several films in flight the link stays busy
// while the others compute, instead of the uploads sharing it and finishing
// together.
static std::mutex g_link_mu;
static cudaEvent_t g_link_ev[64] = {};  // per device: the last upload's copies

static cf_status write_planes_async(cf_film* f, const cf_state_view* v, cudaStream_t st) {
  cfk::Film& F = f->F;
  const size_t n = f->n;
  const cudaMemcpyKind k = v->device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
  std::unique_lock<std::mutex> link(g_link_mu, std::defer_lock);
  cudaEvent_t* link_ev = nullptr;
  if (!v->device && f->device >= 0 && f->device < 64) {
    link.lock();
    link_ev = &g_link_ev[f->device];
    if (*link_ev) CUDA_TRY(f, cudaStreamWaitEvent(st, *link_ev, 0));
    else CUDA_TRY(f, cudaEventCreateWithFlags(link_ev, cudaEventDisableTiming));
  }
  const struct { void* dst; const void* src; size_t bytes; } plain[] = {
      {F.hh, v->h, 4 * n}, {F.m, v->m, 4 * n}, {F.sh, v->strata_h, 16 * n}, {F.scu, v->strata_cure, 16 * n},
      {F.refl, v->sub_refl, 32 * n}, {F.lay, v->lay, 4 * n}};
  for (const auto& p : plain)
    if (p.src) CUDA_TRY(f, cudaMemcpyAsync(p.dst, p.src, p.bytes, k, st));
  const size_t esz = v->pig_format == CF_PIG_F32 ? 4 : 2, pig_b = f->prec == CF_PREC_FP32 ? 4 : 2;
  const bool pig_staged = v->strata_pig && !v->device && esz <= pig_b;
  if (pig_staged) CUDA_TRY(f, cudaMemcpyAsync(F.pig2, v->strata_pig, 64 * esz * n, cudaMemcpyHostToDevice, st));
  if (v->rheo && !v->device) CUDA_TRY(f, cudaMemcpyAsync(F.acc_s, v->rheo, 8 * n, cudaMemcpyHostToDevice, st));
  if (link_ev) {
    CUDA_TRY(f, cudaEventRecord(*link_ev, st));
    link.unlock();
  }
  if (v->strata_pig)
    cfk::launch_pig_import(F, f->prec, F.pig, pig_staged ? (const void*)F.pig2 : async_src(v, v->strata_pig),
                           v->pig_format, st);
  if (v->rheo)
    cfk::launch_rheo_import(F, f->prec, (const float2*)(v->device ? v->rheo : (const void*)F.acc_s), f->S.n_index,
                            n, st);
  return CF_OK;
}

static bool all_async(const cf_state_view* v) {
  for (const void* p : {v->h, v->m, v->rheo, v->strata_h, v->strata_pig, v->strata_cure, v->sub_refl, v->lay})
    if (p && !async_src(v, p)) return false;
  return true;
}

// Host-side copy of the tile stats after a write (the first adaptive step and
// update_params read them).
static cf_status refresh_host_stats(cf_film* f) {
  DevStats ds;
  CUDA_TRY(f, cudaMemcpy(&ds, f->d_stats, sizeof(ds), cudaMemcpyDeviceToHost));
  float hm, mm;
  std::memcpy(&hm, &ds.h_max_bits, 4);
  std::memcpy(&mm, &ds.mu_min_bits, 4);
  f->h_max_stat = hm;
  f->mu_min_stat = mm > 1e8f ? 1.0f : mm;
  if (f->dep_pending == 0u) f->h_max_pending = 0.f;  // stats now include the deposits (poll_stats)
  return CF_OK;
}

cf_status cf_write_state(cf_film* f, const cf_state_view* v) {
  if (!f || !v) return fail(f, CF_ERR_INVALID_ARG, "cf_write_state: null");
  if (v->pig_format < 0 || v->pig_format > 2) return fail(f, CF_ERR_INVALID_ARG, "cf_write_state: pig_format");
  cfk::Film& F = f->F;
  size_t n = f->n;
  CUDA_TRY(f, cudaDeviceSynchronize());
  cf_status st;
  if (all_async(v)) {  // everything enqueued, one wait
    if ((st = write_planes_async(f, v, 0)) != CF_OK) return st;
  } else {  // pageable host memory: plain copies, pigments and rheology staged
    if (v->h && (st = copy_plane(f, F.hh, v->h, 4 * n, v->device, true)) != CF_OK) return st;
    if (v->m && (st = copy_plane(f, F.m, v->m, 4 * n, v->device, true)) != CF_OK) return st;
    if (v->strata_h && (st = copy_plane(f, F.sh, v->strata_h, 16 * n, v->device, true)) != CF_OK) return st;
    if (v->strata_cure && (st = copy_plane(f, F.scu, v->strata_cure, 16 * n, v->device, true)) != CF_OK) return st;
    if (v->sub_refl && (st = copy_plane(f, F.refl, v->sub_refl, 32 * n, v->device, true)) != CF_OK) return st;
    if (v->lay && (st = copy_plane(f, F.lay, v->lay, 4 * n, v->device, true)) != CF_OK) return st;
    const size_t esz = v->pig_format == CF_PIG_F32 ? 4 : 2;
    if (v->rheo || v->strata_pig) {
      void* tmp = nullptr;
      size_t need = std::max(v->strata_pig ? 64 * esz * n : 0, v->rheo ? 8 * n : 0);
      CUDA_TRY(f, cudaMalloc(&tmp, need));
      cudaError_t e = cudaSuccess;
      if (v->strata_pig) {
        e = cudaMemcpy(tmp, v->strata_pig, 64 * esz * n, v->device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice);
        if (e == cudaSuccess) cfk::launch_pig_import(F, f->prec, F.pig, tmp, v->pig_format, 0);
        if (e == cudaSuccess) e = cudaDeviceSynchronize();
      }
      if (e == cudaSuccess && v->rheo) {
        e = cudaMemcpy(tmp, v->rheo, 8 * n, v->device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice);
        if (e == cudaSuccess) cfk::launch_rheo_import(F, f->prec, (const float2*)tmp, f->S.n_index, n, 0);
        if (e == cudaSuccess) e = cudaDeviceSynchronize();
      }
      cudaFree(tmp);
      if (e != cudaSuccess) { f->err = cudaGetErrorString(e); return CF_ERR_CUDA; }
    }
  }
  if ((st = write_state_tail(f, 0)) != CF_OK) return st;
  if ((st = refresh_host_stats(f)) != CF_OK) return st;
  CUDA_TRY(f, cudaDeviceSynchronize());
  return CF_OK;
}

cf_status cf_write_state_async(cf_film* f, const cf_state_view* v, void* stream) {
  if (!f || !v) return fail(f, CF_ERR_INVALID_ARG, "cf_write_state_async: null");
  if (v->pig_format < 0 || v->pig_format > 2) return fail(f, CF_ERR_INVALID_ARG, "cf_write_state_async: pig_format");
  if (!all_async(v)) return fail(f, CF_ERR_INVALID_ARG, "cf_write_state_async: a plane is in pageable host memory");
  cudaStream_t st = (cudaStream_t)stream;
  cf_status s;
  if ((s = write_planes_async(f, v, st)) != CF_OK) return s;
  if ((s = write_state_tail(f, st)) != CF_OK) return s;
  f->stats_stale = true;  // the host copy of the tile stats refreshes at the next stats read
  return CF_OK;
}

cf_status cf_clone_state(cf_film* dst, const cf_film* src, void* stream) {
  if (!dst || !src || dst == src) return fail(dst, CF_ERR_INVALID_ARG, "cf_clone_state: null or same film");
  if (dst->w != src->w || dst->h != src->h || dst->prec != src->prec || dst->device != src->device)
    return fail(dst, CF_ERR_INVALID_ARG, "cf_clone_state: size, precision or device differ");
  if (dst->arena_bytes != src->arena_bytes)  // one has the implicit CG planes, the other not
    return fail(dst, CF_ERR_INVALID_ARG, "cf_clone_state: implicit_hydro differs");
  cudaStream_t st = (cudaStream_t)stream;
  // identical (w, h, precision) give identical arena layouts: one copy moves
  // every plane, both strata generations included
  CUDA_TRY(dst, cudaMemcpyAsync(dst->arena, src->arena, src->arena_bytes, cudaMemcpyDeviceToDevice, st));
  CUDA_TRY(dst, cudaMemcpyAsync(dst->d_tables, src->d_tables, sizeof(float) * 528, cudaMemcpyDeviceToDevice, st));
  CUDA_TRY(dst, cudaMemcpyAsync(dst->d_stats, src->d_stats, sizeof(DevStats), cudaMemcpyDeviceToDevice, st));
  CUDA_TRY(dst, cudaMemcpyAsync(dst->d_params, src->d_params, sizeof(DevParams), cudaMemcpyDeviceToDevice, st));
  dst->S = src->S;
  dst->P = src->P;
  dst->implicit_steps = src->implicit_steps;
  dst->params_dirty = false;
  dst->h_max_stat = src->h_max_stat;
  dst->mu_min_stat = src->mu_min_stat;
  dst->h_max_pending = src->h_max_pending;
  dst->frames = src->frames;
  dst->total_deposited = src->total_deposited;
  dst->dep_pending = 0u;  // deposits uploaded to dst before the clone are dropped
  const bool src_swapped = src->F.sh != src->sh_created, dst_swapped = dst->F.sh != dst->sh_created;
  if (src_swapped != dst_swapped) swap_generations(dst);
  return CF_OK;
}

// The planes of a view into device or page-locked host memory, enqueued on `st`.
static cf_status read_planes_async(cf_film* f, const cf_state_view* v, cudaStream_t st) {
  cfk::Film& F = f->F;
  const size_t n = f->n;
  const cudaMemcpyKind k = v->device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
  const struct { void* dst; const void* src; size_t bytes; } plain[] = {
      {v->h, F.hh, 4 * n}, {v->m, F.m, 4 * n}, {v->strata_h, F.sh, 16 * n}, {v->strata_cure, F.scu, 16 * n},
      {v->sub_refl, F.refl, 32 * n}, {v->lay, F.lay, 4 * n}};
  for (const auto& p : plain)
    if (p.dst) CUDA_TRY(f, cudaMemcpyAsync(p.dst, p.src, p.bytes, k, st));
  if (const void* d = async_src(v, v->strata_pig)) cfk::launch_pig_export(F, f->prec, F.pig, (void*)d, v->pig_format, st);
  if (const void* d = async_src(v, v->rheo)) cfk::launch_rheo_export(F, f->prec, (float2*)d, n, st);
  CUDA_TRY(f, cudaGetLastError());
  return CF_OK;
}

cf_status cf_read_state(cf_film* f, const cf_state_view* v) {
  if (!f || !v) return fail(f, CF_ERR_INVALID_ARG, "cf_read_state: null");
  if (v->pig_format < 0 || v->pig_format > 2) return fail(f, CF_ERR_INVALID_ARG, "cf_read_state: pig_format");
  cfk::Film& F = f->F;
  size_t n = f->n;
  CUDA_TRY(f, cudaDeviceSynchronize());
  cf_status st;
  if (all_async(v)) {
    if ((st = read_planes_async(f, v, 0)) != CF_OK) return st;
    CUDA_TRY(f, cudaDeviceSynchronize());
    return CF_OK;
  }
  if (v->h && (st = copy_plane(f, v->h, F.hh, 4 * n, v->device, false)) != CF_OK) return st;
  if (v->m && (st = copy_plane(f, v->m, F.m, 4 * n, v->device, false)) != CF_OK) return st;
  if (v->strata_h && (st = copy_plane(f, v->strata_h, F.sh, 16 * n, v->device, false)) != CF_OK) return st;
  if (v->strata_cure && (st = copy_plane(f, v->strata_cure, F.scu, 16 * n, v->device, false)) != CF_OK) return st;
  if (v->sub_refl && (st = copy_plane(f, v->sub_refl, F.refl, 32 * n, v->device, false)) != CF_OK) return st;
  if (v->lay && (st = copy_plane(f, v->lay, F.lay, 4 * n, v->device, false)) != CF_OK) return st;
  size_t esz = v->pig_format == CF_PIG_F32 ? 4 : 2;
  if (v->rheo || v->strata_pig) {
    void* tmp = nullptr;
    size_t need = std::max(v->strata_pig ? 64 * esz * n : 0, v->rheo ? 8 * n : 0);
    CUDA_TRY(f, cudaMalloc(&tmp, need));
    cudaError_t e = cudaSuccess;
    if (v->strata_pig) {
      cfk::launch_pig_export(F, f->prec, F.pig, tmp, v->pig_format, 0);
      e = cudaDeviceSynchronize();
      if (e == cudaSuccess) e = cudaMemcpy(v->strata_pig, tmp, 64 * esz * n, v->device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost);
    }
    if (e == cudaSuccess && v->rheo) {
      cfk::launch_rheo_export(F, f->prec, (float2*)tmp, n, 0);
      e = cudaDeviceSynchronize();
      if (e == cudaSuccess) e = cudaMemcpy(v->rheo, tmp, 8 * n, v->device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost);
    }
    cudaFree(tmp);
    if (e != cudaSuccess) { f->err = cudaGetErrorString(e); return CF_ERR_CUDA; }
  }
  return CF_OK;
}

cf_status cf_read_state_async(cf_film* f, const cf_state_view* v, void* stream) {
  if (!f || !v) return fail(f, CF_ERR_INVALID_ARG, "cf_read_state_async: null");
  if (v->pig_format < 0 || v->pig_format > 2) return fail(f, CF_ERR_INVALID_ARG, "cf_read_state_async: pig_format");
  if (!all_async(v)) return fail(f, CF_ERR_INVALID_ARG, "cf_read_state_async: a plane is in pageable host memory");
  return read_planes_async(f, v, (cudaStream_t)stream);
}

static cf_status post_frame_stats(cf_film* f, cudaStream_t st, bool sync_host) {
  if (!sync_host) return CF_OK;
  f->stats_stale = false;
  DevStats ds;
  CUDA_TRY(f, cudaMemcpyAsync(&ds, f->d_stats, sizeof(ds), cudaMemcpyDeviceToHost, st));
  CUDA_TRY(f, cudaStreamSynchronize(st));
  float hm, mm;
  std::memcpy(&hm, &ds.h_max_bits, 4);
  std::memcpy(&mm, &ds.mu_min_bits, 4);
  f->h_max_stat = hm;
  f->mu_min_stat = mm > 1e8f ? 1.0f : mm;
  if (f->dep_pending == 0u) f->h_max_pending = 0.f;  // stats now include the deposits (poll_stats)
  return CF_OK;
}

cf_status cf_update_params(cf_film* f, float frame_dt, uint32_t substeps) {
  if (!f || !(frame_dt > 0.f) || substeps == 0) return fail(f, CF_ERR_INVALID_ARG, "cf_update_params");
  if (f->stats_stale) {  // the stats of an asynchronously written state
    CUDA_TRY(f, cudaDeviceSynchronize());
    cf_status s = refresh_host_stats(f);
    if (s != CF_OK) return s;
    f->stats_stale = false;
  }
  pack_params(f, frame_dt, substeps);
  return CF_OK;
}

cf_status cf_choose_substeps(cf_film* f, float frame_dt, uint32_t* out) {  // src/film/mod.rs:919-933
  if (!f || !out || !(frame_dt > 0.f)) return fail(f, CF_ERR_INVALID_ARG, "cf_choose_substeps");
  cf_status rs = post_frame_stats(f, 0, true);
  if (rs != CF_OK) return rs;
  const cf_settings& s = f->S;
  float g[3];
  gravity_vec(s, g);
  float dx = s.width_m / (float)f->w;
  float gxy = std::sqrt(g[0] * g[0] + g[1] * g[1]);
  float h_max = std::fmax(std::fmax(f->h_max_stat, f->h_max_pending), 1e-5f);
  float mu = std::fmax(f->mu_min_stat, 1e-3f);
  float speed = std::fmin(s.rho * gxy * h_max * h_max / mu, s.v_cap);
  float dt_cfl = speed > 1e-6f ? 0.5f * dx / speed : frame_dt;
  float mob = h_max * h_max * h_max / (3.0f * mu);
  uint32_t n_hyd = (uint32_t)std::fmax(std::ceil(frame_dt * s.rho * g[2] * std::fmin(mob, s.m_cap_hydro) / (0.2f * dx * dx)), 1.0f);
  float dx2 = dx * dx, dx4 = dx2 * dx2;
  uint32_t n_cap = (uint32_t)std::fmax(std::ceil(frame_dt * 32.0f * s.sigma * std::fmin(mob, s.m_cap) / dx4), 1.0f);
  uint32_t n_cfl = (uint32_t)std::fmax(std::ceil(frame_dt / dt_cfl), 1.0f);
  uint32_t n = std::max(std::max(n_cfl, n_hyd), n_cap);
  *out = std::min(std::max(n, s.min_substeps), s.max_substeps);
  return CF_OK;
}

cf_status cf_encode_frame(cf_film* f, uint32_t substeps, void* stream) {
  if (!f || substeps == 0 || substeps > 4096) return fail(f, CF_ERR_INVALID_ARG, "cf_encode_frame");
  if (f->S.slump) return fail(f, CF_ERR_UNSUPPORTED, "slump pass is not implemented (reference default is off)");
  cudaStream_t st = (cudaStream_t)stream;
  cf_status s = upload_params(f, st);
  if (s != CF_OK) return s;
  f->launches += launch_pending_deposits(f, st);
  cfk::PackedFrame V = solo_view(f);
  V.implicit_steps = f->S.implicit_hydro ? f->implicit_steps : 0u;
  f->launches += cfk::launch_frame_packed(V, f->prec, substeps, 0, st);
  swap_generations(f);
  if ((s = check_launch(f)) != CF_OK) return s;
  f->frames++;
  return CF_OK;
}

cf_status cf_step_adaptive(cf_film* f, float dt_max, void* stream) {
  if (!f || !(dt_max > 0.f)) return fail(f, CF_ERR_INVALID_ARG, "cf_step_adaptive");
  if (f->S.slump) return fail(f, CF_ERR_UNSUPPORTED, "slump pass is not implemented");
  cudaStream_t st = (cudaStream_t)stream;
  if (f->h_params->dt_max != dt_max) f->params_dirty = true;
  cf_status s = upload_params(f, st, dt_max);
  if (s != CF_OK) return s;
  f->launches += launch_pending_deposits(f, st);
  cfk::PackedFrame V = solo_view(f);
  // the device picks dt and with it the implicit step count (0..4): the
  // launches cover 4 steps and the film's kernels skip the ones it does not take
  V.implicit_steps = f->S.implicit_hydro ? 4u : 0u;
  f->launches += cfk::launch_frame_packed(V, f->prec, 1, 1, st);
  swap_generations(f);
  if ((s = check_launch(f)) != CF_OK) return s;
  f->frames++;
  return CF_OK;
}

cf_status cf_dry_now(cf_film* f, void* stream) {  // src/film/mod.rs:1230-1244
  if (!f) return CF_ERR_INVALID_ARG;
  cudaStream_t st = (cudaStream_t)stream;
  cf_params saved = f->P;
  f->P.cure[0] = 4.0f / std::fmax(f->P.frame_dt, 1e-4f);
  f->params_dirty = true;
  cf_status s = upload_params(f, st);
  if (s != CF_OK) return s;
  cfk::launch_cure(solo_view(f), f->prec, st);
  if ((s = check_launch(f)) != CF_OK) return s;
  CUDA_TRY(f, cudaStreamSynchronize(st));  // the pinned staging is reused below
  f->P = saved;
  f->params_dirty = true;
  return upload_params(f, st);
}

cf_status cf_color_device_ptr(cf_film* f, void** ptr) {
  if (!f || !ptr) return fail(f, CF_ERR_INVALID_ARG, "cf_color_device_ptr");
  *ptr = f->F.color;
  return CF_OK;
}

cf_status cf_read_color(cf_film* f, uint16_t* out) {
  if (!f || !out) return fail(f, CF_ERR_INVALID_ARG, "cf_read_color");
  CUDA_TRY(f, cudaDeviceSynchronize());
  CUDA_TRY(f, cudaMemcpy(out, f->F.color, 8 * f->n, cudaMemcpyDeviceToHost));
  return CF_OK;
}

cf_status cf_read_color_async(cf_film* f, uint16_t* out, void* stream) {
  if (!f || !out) return fail(f, CF_ERR_INVALID_ARG, "cf_read_color_async");
  if (!kernel_readable_host(out)) {
    cudaPointerAttributes a{};
    if (cudaPointerGetAttributes(&a, out) != cudaSuccess || a.type != cudaMemoryTypeDevice) {
      cudaGetLastError();
      return fail(f, CF_ERR_INVALID_ARG, "cf_read_color_async: destination is pageable host memory");
    }
  }
  CUDA_TRY(f, cudaMemcpyAsync(out, f->F.color, 8 * f->n, cudaMemcpyDefault, (cudaStream_t)stream));
  return CF_OK;
}

cf_status cf_get_stats(cf_film* f, cf_stats* out) {
  if (!f || !out) return fail(f, CF_ERR_INVALID_ARG, "cf_get_stats");
  CUDA_TRY(f, cudaDeviceSynchronize());
  cfk::launch_mass(f->F, f->sms, 0);
  cf_status s = check_launch(f);
  if (s != CF_OK) return s;
  DevStats ds;
  CUDA_TRY(f, cudaMemcpy(&ds, f->d_stats, sizeof(ds), cudaMemcpyDeviceToHost));
  float hm, mm;
  std::memcpy(&hm, &ds.h_max_bits, 4);
  std::memcpy(&mm, &ds.mu_min_bits, 4);
  f->h_max_stat = hm;
  f->mu_min_stat = mm > 1e8f ? 1.0f : mm;
  if (f->dep_pending == 0u) f->h_max_pending = 0.f;  // stats now include the deposits (poll_stats)
  double dx = (double)f->S.width_m / (double)f->w;
  out->h_max = hm;
  out->mu_min = f->mu_min_stat;
  out->active_tiles = ds.active_tiles;
  out->frames = f->frames;
  out->wet_volume = ds.wet_sum * dx * dx;
  out->relief_volume = ds.relief_sum * dx * dx;
  out->last_dt = ds.last_dt > 0.f ? (double)ds.last_dt : (double)f->P.dt;
  out->nan_cells = ds.nan_cells;
  out->wet_cells = ds.wet_cells;
  out->launches = f->launches;
  if (ds.tma_timeouts != 0u) {  // a flow tile's staged loads never arrived: its fluxes were not computed
    f->err = "cf_get_stats: " + std::to_string(ds.tma_timeouts) + " flow tile(s) timed out waiting for their loads";
    return CF_ERR_TIMEOUT;
  }
  return CF_OK;
}

cf_status cf_get_params(cf_film* f, cf_params* out) {
  if (!f || !out) return fail(f, CF_ERR_INVALID_ARG, "cf_get_params");
  *out = f->P;
  return CF_OK;
}

cf_status cf_sync(cf_film* f) {
  if (!f) return CF_ERR_INVALID_ARG;
  CUDA_TRY(f, cudaDeviceSynchronize());
  return post_frame_stats(f, 0, true);
}

}  // extern "C"

// ---- inspection entry points (include/canvaz_film_debug.h) ----
#include "../../include/canvaz_film_debug.h"

namespace {
int internal_pig_format(const cf_film* f) {
  return f->prec == CF_PREC_FP32 ? CF_PIG_F32 : (f->prec == CF_PREC_BF16 ? CF_PIG_BF16 : CF_PIG_F16);
}
struct PlaneRef {
  void* ptr;
  size_t bytes;
  int32_t elem;
};
bool find_plane(cf_film* f, const std::string& n, PlaneRef& r) {
  cfk::Film& F = f->F;
  size_t N = f->n, nt = (size_t)f->tw * f->th;
  int pe = f->prec == CF_PREC_FP32 ? CF_ELEM_F32 : (f->prec == CF_PREC_BF16 ? CF_ELEM_BF16 : CF_ELEM_F16);
  size_t pb = f->prec == CF_PREC_FP32 ? 4 : 2;
  int re = f->prec == CF_PREC_BF16 ? CF_ELEM_BF16 : CF_ELEM_F32;
  size_t rb = f->prec == CF_PREC_BF16 ? 2 : 4;
  struct E { const char* name; void* p; size_t b; int32_t e; } tab[] = {
      {"h", F.hh, 4 * N, CF_ELEM_F32}, {"m", F.m, 4 * N, CF_ELEM_F32}, {"mu", F.mu, rb * N, re},
      {"tau", F.tau, rb * N, re}, {"nn", F.nn, rb * N, re}, {"delta", F.delta, 4 * N, CF_ELEM_U32},
      {"lay", F.lay, 4 * N, CF_ELEM_U32}, {"pres", F.pres, 8 * N, CF_ELEM_F32}, {"fnorm", F.fnorm, 8 * N, CF_ELEM_F32},
      {"flux", F.flux, 16 * N, CF_ELEM_F32}, {"acc", F.acc, 16 * N, CF_ELEM_F32},
      {"acc_s", F.acc_s, 64 * N, CF_ELEM_F32}, {"alpha_s", F.alpha_s, 16 * N, CF_ELEM_F32},
      {"alpha", F.alpha, 4 * N, CF_ELEM_F32}, {"tmp", F.tmp, 4 * N, CF_ELEM_F32},
      {"h_next", F.h_next, 4 * N, CF_ELEM_F32}, {"delta_old", F.delta_old, 4 * N, CF_ELEM_U32},
      {"h_frame", F.h_frame, 4 * N, CF_ELEM_F32}, {"strata_h", F.sh, 16 * N, CF_ELEM_F32},
      {"strata_cure", F.scu, 16 * N, CF_ELEM_F32}, {"strata_h2", F.sh2, 16 * N, CF_ELEM_F32},
      {"strata_cure2", F.scu2, 16 * N, CF_ELEM_F32}, {"strata_pig", F.pig, 64 * pb * N, pe},
      {"strata_pig2", F.pig2, 64 * pb * N, pe}, {"sub_refl", F.refl, 32 * N, CF_ELEM_F16},
      {"color", F.color, 8 * N, CF_ELEM_F16}, {"detail", F.detail, 8 * N, CF_ELEM_F16}, {"tile_flags", F.tile_flags, 4 * nt, CF_ELEM_U32},
      {"tile_moved", F.tile_moved, 4 * nt, CF_ELEM_U32}, {"fill_src", F.fill_src, 4 * N, CF_ELEM_I32},
      {"fflags", F.fflags, 4 * N, CF_ELEM_U32},
      {"agg", F.agg, 16 * N, CF_ELEM_F32},
  };
  for (auto& e : tab)
    if (n == e.name) { r = {e.p, e.b, e.e}; return true; }
  return false;
}
}  // namespace

extern "C" {

cf_status cf_debug_plane_info(cf_film* f, const char* name, size_t* bytes, int32_t* elem) {
  if (!f || !name || !bytes || !elem) return fail(f, CF_ERR_INVALID_ARG, "cf_debug_plane_info");
  PlaneRef r;
  if (!find_plane(f, name, r)) return fail(f, CF_ERR_INVALID_ARG, "unknown plane");
  *bytes = r.bytes;
  *elem = r.elem;
  return CF_OK;
}

cf_status cf_debug_read(cf_film* f, const char* name, void* host, size_t bytes) {
  if (!f || !name || !host) return fail(f, CF_ERR_INVALID_ARG, "cf_debug_read");
  PlaneRef r;
  if (!find_plane(f, name, r) || r.bytes != bytes) return fail(f, CF_ERR_INVALID_ARG, "plane name or size");
  CUDA_TRY(f, cudaDeviceSynchronize());
  std::string n(name);
  if (n == "strata_pig" || n == "strata_pig2") {  // chunk planes -> [cell][stratum][slot]
    void* tmp = nullptr;
    CUDA_TRY(f, cudaMalloc(&tmp, bytes));
    cfk::launch_pig_export(f->F, f->prec, (const uint4*)r.ptr, tmp, internal_pig_format(f), 0);
    cudaError_t e = cudaDeviceSynchronize();
    if (e == cudaSuccess) e = cudaMemcpy(host, tmp, bytes, cudaMemcpyDeviceToHost);
    cudaFree(tmp);
    if (e != cudaSuccess) { f->err = cudaGetErrorString(e); return CF_ERR_CUDA; }
    return CF_OK;
  }
  if (n == "acc_s") {  // face-major -> [cell][face]
    // In active tiles a face counts only where strata_split set its face flag
    // (it does not clear the faces it does not write): the plane reads as the
    // reference's zeroed-then-written acc_s.
    std::vector<float4> v(4 * (size_t)f->n);
    std::vector<uint32_t> ff(f->n), tf((size_t)f->tw * f->th);
    CUDA_TRY(f, cudaMemcpy(v.data(), r.ptr, bytes, cudaMemcpyDeviceToHost));
    CUDA_TRY(f, cudaMemcpy(ff.data(), f->F.fflags, 4 * f->n, cudaMemcpyDeviceToHost));
    CUDA_TRY(f, cudaMemcpy(tf.data(), f->F.tile_flags, 4 * tf.size(), cudaMemcpyDeviceToHost));
    float4* o = (float4*)host;
    for (size_t c = 0; c < f->n; ++c) {
      const size_t i = c % f->w, j = c / f->w;
      const bool act = (tf[(i >> 4) + (j >> 4) * f->tw] & cfk::ACTIVE) != 0u;
      for (int k = 0; k < 4; ++k)
        o[4 * c + k] = (!act || ((ff[c] >> k) & 1u)) ? v[(size_t)k * f->n + c] : make_float4(0.f, 0.f, 0.f, 0.f);
    }
    return CF_OK;
  }
  CUDA_TRY(f, cudaMemcpy(host, r.ptr, bytes, cudaMemcpyDeviceToHost));
  return CF_OK;
}

cf_status cf_debug_write(cf_film* f, const char* name, const void* host, size_t bytes) {
  if (!f || !name || !host) return fail(f, CF_ERR_INVALID_ARG, "cf_debug_write");
  PlaneRef r;
  if (!find_plane(f, name, r) || r.bytes != bytes) return fail(f, CF_ERR_INVALID_ARG, "plane name or size");
  CUDA_TRY(f, cudaDeviceSynchronize());
  CUDA_TRY(f, cudaMemset(f->F.shade_state, 0, f->n));  // any plane may feed a colour
  std::string n(name);
  if (n == "strata_pig" || n == "strata_pig2") {
    void* tmp = nullptr;
    CUDA_TRY(f, cudaMalloc(&tmp, bytes));
    cudaError_t e = cudaMemcpy(tmp, host, bytes, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) {
      cfk::launch_pig_import(f->F, f->prec, (uint4*)r.ptr, tmp, internal_pig_format(f), 0);
      e = cudaDeviceSynchronize();
    }
    cudaFree(tmp);
    if (e != cudaSuccess) { f->err = cudaGetErrorString(e); return CF_ERR_CUDA; }
    return CF_OK;
  }
  if (n == "acc_s") {
    std::vector<float4> v(4 * (size_t)f->n);
    const float4* in = (const float4*)host;
    for (size_t c = 0; c < f->n; ++c)
      for (int k = 0; k < 4; ++k) v[(size_t)k * f->n + c] = in[4 * c + k];
    CUDA_TRY(f, cudaMemcpy(r.ptr, v.data(), bytes, cudaMemcpyHostToDevice));
    return CF_OK;
  }
  CUDA_TRY(f, cudaMemcpy(r.ptr, host, bytes, cudaMemcpyHostToDevice));
  return CF_OK;
}

cf_status cf_debug_run(cf_film* f, const char* kernel, void* stream) {
  if (!f || !kernel) return fail(f, CF_ERR_INVALID_ARG, "cf_debug_run");
  cudaStream_t st = (cudaStream_t)stream;
  cf_status s = upload_params(f, st);
  if (s != CF_OK) return s;
  const int r = std::strcmp(kernel, "deposit") == 0 ? (launch_pending_deposits(f, st), 1)
                                                    : cfk::launch_one(solo_view(f), f->prec, kernel, st);
  if (!r) return fail(f, CF_ERR_INVALID_ARG, "unknown kernel");
  if (r == 2) swap_generations(f);
  if ((s = check_launch(f)) != CF_OK) return s;
  CUDA_TRY(f, cudaStreamSynchronize(st));
  return CF_OK;
}

cf_status cf_debug_set_params(cf_film* f, const cf_params* p) {
  if (!f || !p) return fail(f, CF_ERR_INVALID_ARG, "cf_debug_set_params");
  f->P = *p;
  f->params_dirty = true;
  return CF_OK;
}

}  // extern "C"
