// oracle_capi.cpp — C entry points of the oracle for ctypes.
//
// TEST INFRASTRUCTURE (see film_oracle.hpp).  Built into oracle/_build/
// liboracle.so; loaded only by tests/, __graft_entry__.smoke() and the CPU
// baseline of bench.py.
#include <cstring>
#include <string>

#include "film_oracle.hpp"

namespace {

struct Handle {
  int bits;
  cfo::Film<double>* d = nullptr;
  cfo::Film<float>* f = nullptr;
};

template <class R>
struct Buf {
  std::vector<R>* r = nullptr;
  std::vector<uint32_t>* u = nullptr;
};

template <class R>
Buf<R> find(cfo::Film<R>& F, const char* name) {
  Buf<R> b;
  std::string n(name);
  if (n == "h") b.r = &F.h;
  else if (n == "m") b.r = &F.m;
  else if (n == "rheo") b.r = &F.rheo;
  else if (n == "strata_h") b.r = &F.sh;
  else if (n == "strata_cure") b.r = &F.scu;
  else if (n == "strata_pig") b.r = &F.pig;
  else if (n == "sub_refl") b.r = &F.refl;
  else if (n == "lay") b.u = &F.lay;
  else if (n == "pres") b.r = &F.pres;
  else if (n == "flux") b.r = &F.flux;
  else if (n == "acc") b.r = &F.acc;
  else if (n == "alpha") b.r = &F.alpha;
  else if (n == "tmp") b.r = &F.tmp;
  else if (n == "acc_s") b.r = &F.acc_s;
  else if (n == "alpha_s") b.r = &F.alpha_s;
  else if (n == "strata_h2") b.r = &F.sh2;
  else if (n == "strata_cure2") b.r = &F.scu2;
  else if (n == "strata_pig2") b.r = &F.pig2;
  else if (n == "h_frame") b.r = &F.h_frame;
  else if (n == "fnorm") b.r = &F.fnorm;
  else if (n == "delta") b.u = &F.delta;
  else if (n == "tile_flags") b.u = &F.tile_flags;
  else if (n == "tile_moved") b.u = &F.tile_moved;
  else if (n == "stats") b.r = &F.stats;
  else if (n == "color") b.r = &F.color;
  else if (n == "detail") b.r = &F.detail;
  return b;
}

}  // namespace

extern "C" {

void cfo_settings_default(cf_settings* s) { cfo::settings_default(s); }

// update_params packing without a film (host stats given explicitly).
void cfo_pack_params(const cf_settings* s, uint32_t w, uint32_t h, float frame_dt, uint32_t substeps, float h_max,
                     float mu_min, cf_params* out, uint32_t* implicit_steps) {
  cfo::ParamsF pf = cfo::update_params(*s, w, h, frame_dt, substeps, h_max, 0.0f, mu_min);
  *out = pf.p;
  if (implicit_steps) *implicit_steps = pf.implicit_steps;
}

void* cfo_create(uint32_t w, uint32_t h, const cf_settings* s, int pig_mode, int bits) {
  Handle* hd = new Handle;
  hd->bits = bits;
  if (bits == 32) hd->f = new cfo::Film<float>(w, h, *s, pig_mode);
  else hd->d = new cfo::Film<double>(w, h, *s, pig_mode);
  return hd;
}

void cfo_destroy(void* p) {
  Handle* hd = (Handle*)p;
  delete hd->d;
  delete hd->f;
  delete hd;
}

#define DISPATCH(hd, expr)                      \
  do {                                          \
    if ((hd)->bits == 32) { auto& F = *(hd)->f; expr; } \
    else { auto& F = *(hd)->d; expr; }          \
  } while (0)

void cfo_set_tables(void* p, const float* pigtab, const float* cmf) {
  DISPATCH((Handle*)p, F.set_tables(pigtab, cmf));
}

void cfo_update_params(void* p, float frame_dt, uint32_t substeps) {
  DISPATCH((Handle*)p, F.do_update_params(frame_dt, substeps));
}

void cfo_get_params(void* p, cf_params* out, uint32_t* implicit_steps) {
  DISPATCH((Handle*)p, { *out = F.PF.p; if (implicit_steps) *implicit_steps = F.PF.implicit_steps; });
}

void cfo_set_params(void* p, const cf_params* in) {
  DISPATCH((Handle*)p, { cfo::ParamsF pf; pf.p = *in; pf.implicit_steps = 0; F.set_params(pf); });
}

uint32_t cfo_choose_substeps(void* p, float frame_dt) {
  uint32_t n = 0;
  DISPATCH((Handle*)p, n = cfo::choose_substeps(F.S, F.W, frame_dt, F.h_max_stat, F.h_max_pending, F.mu_min_stat));
  return n;
}

void cfo_after_write_state(void* p) { DISPATCH((Handle*)p, { F.after_write_state(); F.k_reduce_tiles(); }); }

void cfo_encode_frame(void* p, uint32_t substeps) { DISPATCH((Handle*)p, F.encode_frame(substeps)); }

float cfo_step_adaptive(void* p, float dt_max) {
  float d = 0;
  DISPATCH((Handle*)p, d = F.step_adaptive(dt_max));
  return d;
}

void cfo_dry_now(void* p) { DISPATCH((Handle*)p, F.dry_now()); }

// Deposits for the next frame, already binned into 64x64-cell tiles
// (start[nt], count[nt], items[ni]) by the upload_deposits restatement, with
// the host's h_max_pending after the upload.
void cfo_set_deposits(void* p, const cf_deposit* deps, uint32_t n, const uint32_t* start, const uint32_t* count,
                      uint32_t nt, const uint32_t* items, uint32_t ni, float h_max_pending) {
  DISPATCH((Handle*)p, {
    F.deps.assign(deps, deps + n);
    F.dep_start.assign(start, start + nt);
    F.dep_count.assign(count, count + nt);
    F.dep_items.assign(items, items + ni);
    F.h_max_pending = h_max_pending;
  });
}

void cfo_host_stats(void* p, float* h_max_stat, float* h_max_pending) {
  DISPATCH((Handle*)p, { *h_max_stat = F.h_max_stat; *h_max_pending = F.h_max_pending; });
}

// stats: h_max, mu_min, active tiles, mass
void cfo_stats(void* p, float* h_max, float* mu_min, uint32_t* active, double* mass) {
  DISPATCH((Handle*)p, {
    *h_max = F.h_max_stat; *mu_min = F.mu_min_stat; *active = F.active_tiles; *mass = F.mass();
  });
}

// Runs one dispatch by its WGSL entry-point name.
int cfo_run(void* p, const char* kernel) {
  std::string k(kernel);
  int ok = 1;
  DISPATCH((Handle*)p, {
    if (k == "mark_tiles") F.k_mark_tiles();
    else if (k == "compact_tiles") F.k_compact_tiles();
    else if (k == "cure_step") F.run_cure();
    else if (k == "clear_acc") F.run_clear_acc();
    else if (k == "laplacian") F.run_laplacian();
    else if (k == "plug") F.run_plug();
    else if (k == "fluxes") F.run_fluxes();
    else if (k == "limiter") F.run_limiter();
    else if (k == "apply") F.run_apply();
    else if (k == "nose") F.run_nose();
    else if (k == "strata_split") F.run_strata_split();
    else if (k == "reduce_tiles") F.k_reduce_tiles();
    else if (k == "strata_limit") F.run_strata_limit();
    else if (k == "strata_update") F.run_strata_update();
    else if (k == "strata_copy_back") F.run_copy_back();
    else if (k == "strata_fill") F.run_strata_fill();
    else if (k == "shade_full") F.run_shade();
    else if (k == "deposit") F.run_deposit();
    else ok = 0;
  });
  return ok;
}

// Number of elements of a named plane (0 if unknown).
size_t cfo_buffer_len(void* p, const char* name) {
  size_t n = 0;
  DISPATCH((Handle*)p, {
    auto b = find(F, name);
    n = b.r ? b.r->size() : (b.u ? b.u->size() : 0);
  });
  return n;
}

// Reads (write == 0) or writes a named plane as float64 values.  Pigment and
// substrate slots are rounded to their storage format on write.
int cfo_buffer(void* p, const char* name, double* io, int write) {
  int ok = 0;
  DISPATCH((Handle*)p, {
    auto b = find(F, name);
    std::string n(name);
    if (b.r) {
      ok = 1;
      auto& v = *b.r;
      if (write) {
        bool pigp = n == "strata_pig" || n == "strata_pig2";
        bool refp = n == "sub_refl";
        for (size_t i = 0; i < v.size(); ++i) {
          double x = io[i];
          if (pigp) x = cfo::round_pig(x, F.pig_mode, (int)(i % 16));
          else if (refp) x = cfo::round_f16(x);
          v[i] = (decltype(v[0] + 0))x;
        }
      } else {
        for (size_t i = 0; i < v.size(); ++i) io[i] = (double)v[i];
      }
    } else if (b.u) {
      ok = 1;
      auto& v = *b.u;
      if (write) for (size_t i = 0; i < v.size(); ++i) v[i] = (uint32_t)io[i];
      else for (size_t i = 0; i < v.size(); ++i) io[i] = (double)v[i];
    }
  });
  return ok;
}

}  // extern "C"
