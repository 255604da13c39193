// capi_batch.cu — batches of films behind the C ABI (cf_batch_*).
//
// A batch keeps, per precision mode, a device table of its films' records
// and a tile table over all of their 16x16 tiles, so each dispatch of a frame
// is one launch for every film (cfk::launch_frame_packed).  The strata
// generations of each film swap every frame; the batch holds both versions of
// every record (as built, and swapped) and alternates between them, so the
// tables never change while the films step, and a captured frame replays.
#include <cuda_runtime.h>

#include <algorithm>
#include <string>
#include <utility>
#include <vector>

#include "film_handle.h"

struct cf_batch {
  struct Group {
    int mode = 0;
    std::vector<cf_film*> films;
    cfk::Film* d_films = nullptr;  // [2][nfilms]: records as built, then swapped
    uint2* d_tiles = nullptr;      // (film index, tile index); null for a group of one film (identity)
    uint32_t ntiles = 0;
    std::vector<float4*> sh_built;  // each film's current thickness plane at build
  };
  std::vector<cf_film*> films;
  std::vector<Group> groups;
  cf_batch_tuning tune{8u, 1u, 1u, 1u};
  bool built = false;
  int parity = 0;  // which half of every d_films the films are in now
  int device = -1, sms = 1;
  cudaStream_t cap = nullptr;                     // capture stream
  cudaGraphExec_t exec[2] = {nullptr, nullptr};   // frames_per_graph frames from parity 0 / 1
  uint32_t g_frames = 0, g_substeps = 0, g_blocks = 0;
  int g_adaptive = -1;
  uint64_t g_launches = 0;                        // kernel launches in one graph
  uint64_t launches = 0;
  std::string err;
};

#define BATCH_TRY(b, expr)                                                             \
  do {                                                                                 \
    cudaError_t e_ = (expr);                                                           \
    if (e_ != cudaSuccess) {                                                           \
      (b)->err = std::string(#expr) + ": " + cudaGetErrorString(e_);                   \
      return e_ == cudaErrorMemoryAllocation ? CF_ERR_OUT_OF_MEMORY : CF_ERR_CUDA;     \
    }                                                                                  \
  } while (0)

namespace {

cf_status bfail(cf_batch* b, cf_status s, const std::string& msg) {
  if (b) b->err = msg;
  return s;
}

void drop_graphs(cf_batch* b) {
  for (auto& e : b->exec)
    if (e) { cudaGraphExecDestroy(e); e = nullptr; }
  b->g_adaptive = -1;
}

// Frees the tables; the next step rebuilds them.  Waits for the device, so
// that no launch still reads them.
void release(cf_batch* b) {
  if (b->built || !b->groups.empty()) cudaDeviceSynchronize();
  drop_graphs(b);
  for (auto& g : b->groups) {
    if (g.d_films) cudaFree(g.d_films);
    if (g.d_tiles) cudaFree(g.d_tiles);
  }
  b->groups.clear();
  b->built = false;
}

cfk::Film swapped(const cfk::Film& F) {
  cfk::Film G = F;
  std::swap(G.sh, G.sh2);
  std::swap(G.scu, G.scu2);
  return G;
}

cf_status build(cf_batch* b) {
  release(b);
  for (int mode = 0; mode <= 2; ++mode) {
    cf_batch::Group g;
    g.mode = mode;
    for (cf_film* f : b->films)
      if (f->prec == mode) g.films.push_back(f);
    if (g.films.empty()) continue;
    const size_t nf = g.films.size();
    std::vector<cfk::Film> rec(2 * nf);
    std::vector<uint2> tiles;
    for (size_t k = 0; k < nf; ++k) {
      g.sh_built.push_back(g.films[k]->F.sh);
      rec[k] = g.films[k]->F;
      rec[nf + k] = swapped(g.films[k]->F);
      const uint32_t nt = g.films[k]->tw * g.films[k]->th;
      for (uint32_t t = 0; t < nt; ++t) tiles.push_back(make_uint2((uint32_t)k, t));
    }
    g.ntiles = (uint32_t)tiles.size();
    b->groups.push_back(g);
    cf_batch::Group& G = b->groups.back();
    BATCH_TRY(b, cudaMalloc(&G.d_films, sizeof(cfk::Film) * 2 * nf));
    BATCH_TRY(b, cudaMemcpy(G.d_films, rec.data(), sizeof(cfk::Film) * 2 * nf, cudaMemcpyHostToDevice));
    if (nf > 1) {  // a group of one film uses the implicit identity table, as the film alone does
      BATCH_TRY(b, cudaMalloc(&G.d_tiles, sizeof(uint2) * tiles.size()));
      BATCH_TRY(b, cudaMemcpy(G.d_tiles, tiles.data(), sizeof(uint2) * tiles.size(), cudaMemcpyHostToDevice));
    }
  }
  b->parity = 0;
  b->built = true;
  return CF_OK;
}

// Implicit hydrostatic steps to launch for a group: each film's own count
// when the host knows it, else (dt chosen on the device, or a graph replayed
// over frames whose counts differ) the most a frame takes, 4; the films'
// kernels skip the steps beyond their own count.
void implicit_view(const cf_batch::Group& g, bool fixed_count, cfk::PackedFrame& V) {
  uint32_t steps = 0, iters = 0;
  bool on = false, cap = false;
  for (const cf_film* f : g.films) {
    if (!f->S.implicit_hydro) continue;
    on = true;
    steps = std::max(steps, f->implicit_steps);
    iters = std::max(iters, f->S.implicit_iters);
    cap = cap || f->S.capillary_implicit;
  }
  V.implicit_steps = on ? (fixed_count ? steps : 4u) : 0u;
  V.implicit_iters = iters;
  V.cap_implicit = cap;
}

// Enqueues `frames` frames starting at parity p; no host bookkeeping.
uint64_t enqueue(cf_batch* b, int p, uint32_t frames, uint32_t substeps, int adaptive, bool graph, cudaStream_t st) {
  uint64_t n = 0;
  const uint32_t blocks = (uint32_t)b->sms * std::max(b->tune.list_blocks_per_sm, 1u);
  for (uint32_t r = 0; r < frames; ++r) {
    for (auto& g : b->groups) {
      const uint32_t nf = (uint32_t)g.films.size();
      cfk::PackedFrame V;
      implicit_view(g, !adaptive && !graph, V);
      V.films = g.d_films + (size_t)p * nf;
      V.films_next = g.d_films + (size_t)(1 - p) * nf;
      V.tiles = g.d_tiles;
      V.ntiles = g.ntiles;
      V.nfilms = nf;
      V.persist_blocks = blocks;
      const uint32_t tpb = std::max(b->tune.tiles_per_block, 1u);
      V.tile_grid = tpb > 1u ? (g.ntiles + tpb - 1u) / tpb : 0u;
      n += cfk::launch_frame_packed(V, g.mode, substeps, adaptive, st);
    }
    p ^= 1;
  }
  return n;
}

// Host records after `frames` frames: generations swapped, counters advanced.
void advance(cf_batch* b, uint32_t frames, uint64_t launches) {
  if (frames & 1u) {
    b->parity ^= 1;
    for (cf_film* f : b->films) swap_generations(f);
  }
  for (cf_film* f : b->films) f->frames += frames;
  b->launches += launches;
}

cf_status capture(cf_batch* b, int p, uint32_t frames, uint32_t substeps, int adaptive) {
  if (!b->cap) BATCH_TRY(b, cudaStreamCreateWithFlags(&b->cap, cudaStreamNonBlocking));
  cudaGraph_t graph = nullptr;
  BATCH_TRY(b, cudaStreamBeginCapture(b->cap, cudaStreamCaptureModeThreadLocal));
  b->g_launches = enqueue(b, p, frames, substeps, adaptive, true, b->cap);
  cudaError_t e = cudaStreamEndCapture(b->cap, &graph);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return bfail(b, CF_ERR_CUDA, std::string("graph capture: ") + cudaGetErrorString(e));
  }
  e = cudaGraphInstantiate(&b->exec[p], graph, 0);
  cudaGraphDestroy(graph);
  if (e != cudaSuccess) {
    b->exec[p] = nullptr;
    return bfail(b, CF_ERR_CUDA, std::string("graph instantiate: ") + cudaGetErrorString(e));
  }
  return CF_OK;
}

cf_status step(cf_batch* b, uint32_t frames, uint32_t substeps, float dt_max, cudaStream_t st) {
  const int adaptive = dt_max > 0.f ? 1 : 0;
  if (!adaptive && (substeps == 0 || substeps > 4096)) return bfail(b, CF_ERR_INVALID_ARG, "cf_batch_step: substeps");
  if (adaptive) substeps = 1;
  if (b->films.empty() || frames == 0) return CF_OK;
  for (cf_film* f : b->films) {
    if (f->S.slump) return bfail(b, CF_ERR_UNSUPPORTED, "slump pass is not implemented");
  }
  // a film stepped on its own since the build is in the other generation
  // than the batch's records say: rebuild them
  bool in_step = b->built;
  for (const auto& g : b->groups)
    for (size_t k = 0; k < g.films.size() && in_step; ++k)
      in_step = (g.films[k]->F.sh == g.sh_built[k]) == (b->parity == 0);
  if (!in_step) {
    cf_status s = build(b);
    if (s != CF_OK) return s;
  }
  for (cf_film* f : b->films) {
    if (adaptive && f->h_params->dt_max != dt_max) f->params_dirty = true;
    cf_status s = upload_params(f, st, adaptive ? dt_max : 0.f);
    if (s != CF_OK) return bfail(b, s, f->err);
    b->launches += launch_pending_deposits(f, st);  // before the first frame, as alone
  }
  uint32_t done = 0;
  if (b->tune.use_graph) {
    const uint32_t k = std::max(b->tune.frames_per_graph, 1u);
    const uint32_t blocks = (uint32_t)b->sms * std::max(b->tune.list_blocks_per_sm, 1u);
    if (b->g_frames != k || b->g_substeps != substeps || b->g_adaptive != adaptive || b->g_blocks != blocks) {
      drop_graphs(b);
      b->g_frames = k;
      b->g_substeps = substeps;
      b->g_adaptive = adaptive;
      b->g_blocks = blocks;
    }
    while (frames - done >= k) {
      const int p = b->parity;
      if (!b->exec[p]) {
        cf_status s = capture(b, p, k, substeps, adaptive);
        if (s != CF_OK) return s;
      }
      BATCH_TRY(b, cudaGraphLaunch(b->exec[p], st));
      advance(b, k, b->g_launches);
      done += k;
    }
  }
  if (done < frames) {
    const uint32_t rest = frames - done;
    const uint64_t n = enqueue(b, b->parity, rest, substeps, adaptive, false, st);
    BATCH_TRY(b, cudaGetLastError());
    advance(b, rest, n);
  }
  BATCH_TRY(b, cudaGetLastError());
  return CF_OK;
}

}  // namespace

void batch_forget(cf_film* f) {
  cf_batch* b = f->batch;
  if (!b) return;
  release(b);
  b->films.erase(std::remove(b->films.begin(), b->films.end(), f), b->films.end());
  f->batch = nullptr;
}

extern "C" {

cf_status cf_batch_create(cf_batch** out) {
  if (!out) return CF_ERR_INVALID_ARG;
  *out = new (std::nothrow) cf_batch;
  return *out ? CF_OK : CF_ERR_OUT_OF_MEMORY;
}

cf_status cf_batch_destroy(cf_batch* b) {
  if (!b) return CF_ERR_INVALID_ARG;
  release(b);
  for (cf_film* f : b->films) f->batch = nullptr;
  if (b->cap) cudaStreamDestroy(b->cap);
  delete b;
  return CF_OK;
}

cf_status cf_batch_add(cf_batch* b, cf_film* f) {
  if (!b || !f) return CF_ERR_INVALID_ARG;
  if (f->batch) return bfail(b, CF_ERR_INVALID_ARG, "cf_batch_add: film already in a batch");
  if (b->device >= 0 && f->device != b->device) return bfail(b, CF_ERR_INVALID_ARG, "cf_batch_add: other device");
  release(b);
  b->device = f->device;
  b->sms = std::max(f->sms, 1);
  b->films.push_back(f);
  f->batch = b;
  return CF_OK;
}

cf_status cf_batch_remove(cf_batch* b, cf_film* f) {
  if (!b || !f || f->batch != b) return bfail(b, CF_ERR_INVALID_ARG, "cf_batch_remove: film not in this batch");
  batch_forget(f);
  return CF_OK;
}

cf_status cf_batch_info(cf_batch* b, uint32_t* films, uint64_t* cells, uint64_t* launches) {
  if (!b) return CF_ERR_INVALID_ARG;
  uint64_t n = 0;
  for (cf_film* f : b->films) n += f->n;
  if (films) *films = (uint32_t)b->films.size();
  if (cells) *cells = n;
  if (launches) *launches = b->launches;
  return CF_OK;
}

cf_status cf_batch_set_tuning(cf_batch* b, const cf_batch_tuning* t) {
  if (!b || !t || t->list_blocks_per_sm == 0 || t->list_blocks_per_sm > 64 || t->frames_per_graph == 0 ||
      t->frames_per_graph > 64 || t->tiles_per_block > 4096)
    return bfail(b, CF_ERR_INVALID_ARG, "cf_batch_set_tuning");
  b->tune = *t;
  drop_graphs(b);
  return CF_OK;
}

cf_status cf_batch_get_tuning(cf_batch* b, cf_batch_tuning* t) {
  if (!b || !t) return CF_ERR_INVALID_ARG;
  *t = b->tune;
  return CF_OK;
}

cf_status cf_batch_step(cf_batch* b, uint32_t frames, uint32_t substeps, float dt_max, void* stream) {
  if (!b || !(dt_max >= 0.f)) return bfail(b, CF_ERR_INVALID_ARG, "cf_batch_step");
  return step(b, frames, substeps, dt_max, (cudaStream_t)stream);
}

cf_status cf_batch_autotune(cf_batch* b, uint32_t frames_per_trial, uint32_t substeps, float dt_max, void* stream,
                            cf_batch_tuning* best, float* best_ms) {
  if (!b || frames_per_trial == 0) return bfail(b, CF_ERR_INVALID_ARG, "cf_batch_autotune");
  if (b->films.empty()) return bfail(b, CF_ERR_INVALID_ARG, "cf_batch_autotune: empty batch");
  cudaStream_t st = (cudaStream_t)stream;
  cudaEvent_t e0, e1;
  BATCH_TRY(b, cudaEventCreate(&e0));
  BATCH_TRY(b, cudaEventCreate(&e1));
  auto trial = [&](const cf_batch_tuning& t, float& ms) -> cf_status {
    cf_status s = cf_batch_set_tuning(b, &t);
    if (s != CF_OK) return s;
    const uint32_t warm = 2 * std::max(t.use_graph ? t.frames_per_graph : 1u, 1u);
    if ((s = step(b, warm, substeps, dt_max, st)) != CF_OK) return s;
    BATCH_TRY(b, cudaEventRecord(e0, st));
    if ((s = step(b, frames_per_trial, substeps, dt_max, st)) != CF_OK) return s;
    BATCH_TRY(b, cudaEventRecord(e1, st));
    BATCH_TRY(b, cudaEventSynchronize(e1));
    BATCH_TRY(b, cudaEventElapsedTime(&ms, e0, e1));
    ms /= (float)frames_per_trial;
    return CF_OK;
  };
  cf_batch_tuning top = b->tune;
  float top_ms = 3.4e38f;
  cf_status s = CF_OK;
  // stage 1: the list-kernel grid; stage 2: how the frames are launched
  // (direct, or graphs of 1, 2 or 4 frames); stage 3: the launch tile of the
  // per-tile kernels (16x16, 32x16, 64x16, or a persistent walk with about
  // 8 blocks per SM)
  for (uint32_t bps : {4u, 8u, 16u}) {
    cf_batch_tuning t{bps, 1u, 1u, 1u};
    float ms = 0.f;
    if ((s = trial(t, ms)) != CF_OK) break;
    if (ms < top_ms) { top_ms = ms; top = t; }
  }
  if (s == CF_OK) {
    const cf_batch_tuning stage2[] = {{top.list_blocks_per_sm, 0u, 1u, 1u},
                                      {top.list_blocks_per_sm, 1u, 2u, 1u},
                                      {top.list_blocks_per_sm, 1u, 4u, 1u}};
    for (const auto& t : stage2) {
      float ms = 0.f;
      if ((s = trial(t, ms)) != CF_OK) break;
      if (ms < top_ms) { top_ms = ms; top = t; }
    }
  }
  if (s == CF_OK) {
    uint32_t tiles = 0;
    for (const auto& g : b->groups) tiles = std::max(tiles, g.ntiles);
    const uint32_t persistent = std::min(4096u, std::max(1u, tiles / (8u * (uint32_t)std::max(b->sms, 1))));
    for (uint32_t tpb : {2u, 4u, persistent}) {
      if (tpb <= 1u) continue;
      cf_batch_tuning t = top;
      t.tiles_per_block = tpb;
      float ms = 0.f;
      if ((s = trial(t, ms)) != CF_OK) break;
      if (ms < top_ms) { top_ms = ms; top = t; }
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (s != CF_OK) return s;
  cf_batch_set_tuning(b, &top);
  if (best) *best = top;
  if (best_ms) *best_ms = top_ms;
  return CF_OK;
}

const char* cf_batch_last_error(const cf_batch* b) { return b ? b->err.c_str() : "null batch"; }

}  // extern "C"
