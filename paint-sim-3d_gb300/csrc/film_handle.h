// film_handle.h — the cf_film handle behind the C ABI (internal to the
// library: capi.cu and capi_batch.cu).
#pragma once

#include <cuda_runtime.h>

#include <string>
#include <utility>

#include "../../include/canvaz_film.h"
#include "film_kernels.h"

using cfk::DevParams;
using cfk::DevStats;

struct cf_film {
  cf_settings S;
  uint32_t w = 0, h = 0, tw = 0, th = 0;
  int prec = 0;
  size_t n = 0;
  cfk::Film F{};
  void* arena = nullptr;
  size_t arena_bytes = 0;
  DevParams* d_params = nullptr;
  DevStats* d_stats = nullptr;
  DevParams* h_params = nullptr;  // pinned staging of the host-packed params
  cudaEvent_t params_ev = nullptr;  // recorded after the last staging copy
  float* d_tables = nullptr;
  cf_params P{};
  uint32_t implicit_steps = 0;
  bool params_dirty = true;
  float h_max_stat = 0.f, mu_min_stat = 1.f, h_max_pending = 0.f;
  uint32_t frames = 0;
  uint64_t launches = 0;  // kernels enqueued by this film
  int device = 0, sms = 0;
  std::string err;
  cf_batch* batch = nullptr;  // the batch this film steps in, if any
  // the film's own packed view: its record as created and with the strata
  // generations swapped, and a table of its tiles
  cfk::Film* d_recs = nullptr;
  CUtensorMap* d_tmaps = nullptr;  // the flow tile's tensor-load descriptors (cfk::FLOW_MAPS), or none
  float4* sh_created = nullptr;  // F.sh at create: tells which record is current
  // deposits for the next frame (cf_upload_deposits)
  cf_deposit* d_deps = nullptr;
  uint32_t* d_dep_tiles = nullptr;  // start[nt64], count[nt64]
  uint32_t* d_dep_items = nullptr;
  size_t dep_cap = 0, dep_items_cap = 0;
  uint32_t dep_nt = 0, dep_pending = 0, dep_tiles_listed = 0;
  double total_deposited = 0.0;  // volume laid inside the canvas (upload_deposits)
  bool stats_stale = false;      // an asynchronous write changed the state since the host read the stats
};

// The view that steps this film alone (same kernels as a batch).
inline cfk::PackedFrame solo_view(const cf_film* f) {
  const int p = f->F.sh == f->sh_created ? 0 : 1;
  cfk::PackedFrame V;
  V.films = f->d_recs + p;
  V.films_next = f->d_recs + (1 - p);
  V.tiles = nullptr;  // the identity table over this film
  V.ntiles = f->tw * f->th;
  V.nfilms = 1;
  V.persist_blocks = f->F.persist_blocks;
  V.implicit_iters = f->S.implicit_iters;
  V.cap_implicit = f->S.implicit_hydro && f->S.capillary_implicit;
  return V;
}
inline void swap_generations(cf_film* f) {
  std::swap(f->F.sh, f->F.sh2);
  std::swap(f->F.scu, f->F.scu2);
}

#define CUDA_TRY(film, expr)                                                           \
  do {                                                                                 \
    cudaError_t e_ = (expr);                                                           \
    if (e_ != cudaSuccess) {                                                           \
      (film)->err = std::string(#expr) + ": " + cudaGetErrorString(e_);                \
      return e_ == cudaErrorMemoryAllocation ? CF_ERR_OUT_OF_MEMORY : CF_ERR_CUDA;     \
    }                                                                                  \
  } while (0)

inline cf_status fail(cf_film* f, cf_status s, const char* msg) {
  if (f) f->err = msg;
  return s;
}

// Copies the host-packed params to the device on `st` when they changed.
cf_status upload_params(cf_film* f, cudaStream_t st, float dt_max = 0.f);
// Removes a film from its batch (when the film is destroyed).
void batch_forget(cf_film* f);
// Enqueues the film's pending deposits (deposit.wgsl, before the frame's
// mark_tiles) and clears them; returns the number of launches.
uint32_t launch_pending_deposits(cf_film* f, cudaStream_t st);
