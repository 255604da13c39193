// deposit.cu — the deposit rasteriser: paint laid on the film as ribbons,
// capsules and strokes (shaders/deposit.wgsl:1-75), its host-side records
// (Deposit, src/film/mod.rs:25-186) and their binning into 64x64-cell tiles
// (upload_deposits, src/film/mod.rs:1175-1224).
//
// Host constructors follow the Rust code operation by operation in f32 (the
// build compiles host code without contraction), so their values are the
// reference's bit for bit; the kernel follows the shader.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "film_handle.h"
#include "strata_device.cuh"

namespace {

constexpr uint32_t CAP_START = 2u, CAP_END = 4u, RECYCLED = 1u, METHOD_SHIFT = 8u;

struct Dir {
  float d[2];
  float l;
};
Dir segment_dir(const float p0[2], const float p1[2]) {  // src/film/mod.rs:56-60
  const float d0 = p1[0] - p0[0], d1 = p1[1] - p0[1];
  const float l = std::sqrt(d0 * d0 + d1 * d1);
  if (l > 0.0f) return {{d0 / l, d1 / l}, l};
  return {{1.0f, 0.0f}, 0.0f};
}

float max_radius(const cf_deposit& d) { return std::max(d.r0, d.r1); }

// Deposit::profile (src/film/mod.rs:150-185)
float profile(const cf_deposit& d, const float p[2]) {
  const Dir sd = segment_dir(d.p0, d.p1);
  const bool cap_start = (d.kind & CAP_START) != 0u, cap_end = (d.kind & CAP_END) != 0u;
  const float q0[2] = {p[0] - d.p0[0], p[1] - d.p0[1]}, q1[2] = {p[0] - d.p1[0], p[1] - d.p1[1]};
  auto len = [](const float q[2]) { return std::sqrt(q[0] * q[0] + q[1] * q[1]); };
  if (sd.l <= 0.0f) {
    const float x = len(q0) / d.r0;
    return x < 1.0f ? d.h0 * (1.0f - x * x) : 0.0f;
  }
  if (!cap_start && q0[0] * d.n0[0] + q0[1] * d.n0[1] < 0.0f) return 0.0f;
  if (!cap_end && q1[0] * d.n1[0] + q1[1] * d.n1[1] >= 0.0f) return 0.0f;
  const float u = q0[0] * sd.d[0] + q0[1] * sd.d[1];
  if (u < -d.r0 || u > sd.l + d.r1) return 0.0f;
  float dist = std::fabs(q0[0] * sd.d[1] - q0[1] * sd.d[0]);
  if (cap_start && u < 0.0f) dist = len(q0);
  if (cap_end && u > sd.l) dist = len(q1);
  const float rt = d.r0 + (d.r1 - d.r0) * std::min(std::max(u / sd.l, 0.0f), 1.0f);
  const float x = dist / rt;
  return x < 1.0f ? d.h0 * (rt / d.r0) * (1.0f - x * x) : 0.0f;
}

// Deposit::sampled_volume_in (src/film/mod.rs:115-131)
float sampled_volume_in(const cf_deposit& d, float lattice, const float lo[2], const float hi[2]) {
  const float rm = max_radius(d) + lattice;
  const int x0 = (int)std::floor(std::max(std::min(d.p0[0], d.p1[0]) - rm, lo[0]) / lattice);
  const int x1 = (int)std::ceil(std::min(std::max(d.p0[0], d.p1[0]) + rm, hi[0]) / lattice);
  const int y0 = (int)std::floor(std::max(std::min(d.p0[1], d.p1[1]) - rm, lo[1]) / lattice);
  const int y1 = (int)std::ceil(std::min(std::max(d.p0[1], d.p1[1]) + rm, hi[1]) / lattice);
  float sum = 0.0f;
  for (int i = x0; i < x1; ++i)
    for (int j = y0; j < y1; ++j) {
      const float p[2] = {((float)i + 0.5f) * lattice, ((float)j + 0.5f) * lattice};
      sum += profile(d, p);
    }
  return sum * lattice * lattice;
}
float sampled_volume(const cf_deposit& d, float lattice) {
  const float lo[2] = {-INFINITY, -INFINITY}, hi[2] = {INFINITY, INFINITY};
  return sampled_volume_in(d, lattice, lo, hi);
}

// Deposit::inside_fraction (src/film/mod.rs:133-146)
float inside_fraction(const cf_deposit& d, float w, float h) {
  const float rb = max_radius(d);
  const bool full = std::min(d.p0[0], d.p1[0]) - rb >= 0.0f && std::min(d.p0[1], d.p1[1]) - rb >= 0.0f &&
                    std::max(d.p0[0], d.p1[0]) + rb <= w && std::max(d.p0[1], d.p1[1]) + rb <= h;
  if (full) return 1.0f;
  const float lattice = 0.25f * std::max(std::min(d.r0, d.r1), 1e-4f);
  const float all = sampled_volume(d, lattice);
  if (all <= 0.0f) return 0.0f;
  const float lo[2] = {0.0f, 0.0f}, hi[2] = {w, h};
  return std::min(std::max(sampled_volume_in(d, lattice, lo, hi) / all, 0.0f), 1.0f);
}

// ---- kernel (shaders/deposit.wgsl) ----

// deposit.wgsl:6-29; mix(a, b, t) = a (1 - t) + b t as WGSL defines it
__device__ float ribbon_height(float px, float py, const cf_deposit& d) {
  const float abx = d.p1[0] - d.p0[0], aby = d.p1[1] - d.p0[1];
  const float l2 = abx * abx + aby * aby;
  if (l2 <= 0.0f) {
    const float qx = px - d.p0[0], qy = py - d.p0[1];
    const float x = sqrtf(qx * qx + qy * qy) / d.r0;
    return x < 1.0f ? d.h0 * (1.0f - x * x) : 0.0f;
  }
  const float l = sqrtf(l2);
  const float dx = abx / l, dy = aby / l;
  const float q0x = px - d.p0[0], q0y = py - d.p0[1], q1x = px - d.p1[0], q1y = py - d.p1[1];
  const bool cap_start = (d.kind & CAP_START) != 0u, cap_end = (d.kind & CAP_END) != 0u;
  if (!cap_start && q0x * d.n0[0] + q0y * d.n0[1] < 0.0f) return 0.0f;
  if (!cap_end && q1x * d.n1[0] + q1y * d.n1[1] >= 0.0f) return 0.0f;
  const float u = q0x * dx + q0y * dy;
  if (u < -d.r0 || u > l + d.r1) return 0.0f;
  float dist = fabsf(q0x * dy - q0y * dx);
  if (cap_start && u < 0.0f) dist = sqrtf(q0x * q0x + q0y * q0y);
  if (cap_end && u > l) dist = sqrtf(q1x * q1x + q1y * q1y);
  const float t = fminf(fmaxf(u / l, 0.0f), 1.0f);
  const float rt = d.r0 * (1.0f - t) + d.r1 * t;
  const float x = dist / rt;
  return x < 1.0f ? d.h0 * (rt / d.r0) * (1.0f - x * x) : 0.0f;
}

// common.wgsl:81-84
__device__ uint32_t lay_pack(uint32_t method, float dx, float dy) {
  const float turn = atan2f(dy, dx) / 6.2831853f + 0.5f;
  return (method & 0xffu) | ((uint32_t)(fminf(fmaxf(turn, 0.f), 1.f) * 65535.0f) << 8);
}

// The deposits of the cell (i, j)'s 64x64-cell tile that pass the reach test
// of deposit.wgsl:44-47 (centre within 1.415 r + 0.6 dx of the segment), in
// list order; with SAMPLE, only those whose 4x4-supersampled height add
// (deposit.wgsl:48-54) is > 0, with the add.
struct DepTables {
  const cf_deposit* deps;
  const uint32_t* tile_start;
  const uint32_t* tile_count;
  const uint32_t* tile_items;
};
template <bool SAMPLE, class Fn>
__device__ __forceinline__ void for_each_add(const cfk::Film& F, const cf_params& P, const DepTables& D, int i,
                                             int j, Fn fn) {
  const uint32_t tile = (uint32_t)(i / 64) + (uint32_t)(j / 64) * P.tiles[0];
  const uint32_t n = D.tile_count[tile];
  if (n == 0u) return;
  const uint32_t start = D.tile_start[tile];
  const float px = ((float)i + 0.5f) * P.dx, py = ((float)j + 0.5f) * P.dx;
  for (uint32_t q = 0; q < n; ++q) {
    const cf_deposit& d = D.deps[D.tile_items[start + q]];
    const float abx = d.p1[0] - d.p0[0], aby = d.p1[1] - d.p0[1];
    const float along = fminf(fmaxf(((px - d.p0[0]) * abx + (py - d.p0[1]) * aby) / fmaxf(abx * abx + aby * aby, 1e-30f),
                                    0.f), 1.f);
    const float reach = 1.415f * fmaxf(d.r0, d.r1) + 0.6f * P.dx;
    const float ox = px - d.p0[0] - along * abx, oy = py - d.p0[1] - along * aby;
    if (ox * ox + oy * oy > reach * reach) continue;
    if (!SAMPLE) {
      fn(d, 0.f, abx, aby);
      continue;
    }
    float add = 0.f;
    for (int sy = 0; sy < 4; ++sy)
      for (int sx = 0; sx < 4; ++sx) {
        const float sxf = ((float)sx - 1.5f) * (0.25f * P.dx), syf = ((float)sy - 1.5f) * (0.25f * P.dx);
        add += 0.0625f * ribbon_height(px + sxf, py + syf, d);
      }
    if (add > 0.f) fn(d, add, abx, aby);
  }
}

// Pass 1 of deposit.wgsl:31-75, over the 64x64 tiles that list deposits (the
// reference dispatches the whole grid; cells of other tiles return at once):
// lists the cells that some deposit reaches, a superset of the cells that
// receive paint.  No sampling and no stack, so the pass is light.
__global__ void __launch_bounds__(256) k_deposit_mark(cfk::Film F, DepTables D, const uint32_t* __restrict__ tiles64,
                                                      uint32_t* __restrict__ painted,
                                                      uint32_t* __restrict__ painted_count) {
  using namespace cfk;
  // block b: 16x16 sub-tile (b % 16) of the b / 16-th 64x64 tile that lists deposits
  const uint32_t t = tiles64[blockIdx.x >> 4], sub = blockIdx.x & 15u;
  const uint32_t t64w = (F.w + 63u) / 64u;
  const int i = (int)((t % t64w) * 64u + (sub & 3u) * 16u + threadIdx.x);
  const int j = (int)((t / t64w) * 64u + (sub >> 2) * 16u + threadIdx.y);
  if (i >= (int)F.w || j >= (int)F.h) return;
  const cf_params& P = F.P->p;
  bool any = false;
  for_each_add<false>(F, P, D, i, j, [&](const cf_deposit&, float, float, float) { any = true; });
  if (any) list_append(painted, painted_count, idx(F, i, j));
}

// Pass 2, one thread per listed cell: the cell's stack gets each deposit's
// add > 0 as a new top stratum (stack_push_top, strata.wgsl:105-130), then h,
// lay (the largest add's method and direction) and the tile's moved flag, as
// deposit.wgsl:59-74 writes them; a listed cell that gets no paint is left
// untouched.
template <int MODE>
__global__ void __launch_bounds__(256) k_deposit_lay(cfk::Film F, DepTables D, const uint32_t* __restrict__ painted,
                                                     const uint32_t* __restrict__ painted_count) {
  using namespace cfk;
  const cf_params& P = F.P->p;
  __shared__ float lt[12];  // ln of the pigments' table viscosities, for the aggregates
  if (threadIdx.x < 12) lt[threadIdx.x] = logf(fmaxf(F.pigtab[threadIdx.x * 40 + 32], 1e-3f));
  __syncthreads();
  const uint32_t count = *painted_count;
  for (uint32_t e = blockIdx.x * blockDim.x + threadIdx.x; e < count; e += gridDim.x * blockDim.x) {
    const uint32_t c = painted[e];
    const int i = (int)(c % F.w), j = (int)(c / F.w);
    Stack s;  // loaded when the first add arrives
    float added = 0.f, top_add = 0.f;
    uint32_t top_lay = 0u;
    for_each_add<true>(F, P, D, i, j, [&](const cf_deposit& d, float add, float abx, float aby) {
      if (added == 0.f) stack_load<MODE>(F, F.sh, F.scu, F.pig, c, s);
      float pig[16];
#pragma unroll
      for (int k = 0; k < 8; ++k) {  // unpack2x16float pairs (common.wgsl:173-180)
        pig[2 * k] = h16_to_f(d.pig[k] & 0xffffu);
        pig[2 * k + 1] = h16_to_f(d.pig[k] >> 16);
      }
      stack_push_top(s, add, pig, 0.0f, P.misc[0], P.misc[1]);
      added += add;
      if (add > top_add) {
        top_add = add;
        const float ex = abx + 1e-9f, ey = aby;
        const float el = sqrtf(ex * ex + ey * ey);
        top_lay = lay_pack(d.kind >> METHOD_SHIFT, ex / el, ey / el);
      }
    });
    if (!(added > 0.f)) continue;
    F.hh[c] = F.hh[c] + added;
    F.lay[c] = top_lay;
    F.tile_moved[(uint32_t)(i >> 4) + (uint32_t)(j >> 4) * F.tw] = 1u;  // mark_moved
    stack_compact(s, P.misc[0]);
    stack_store<MODE>(F, F.sh, F.scu, F.pig, c, s);
    F.shade_state[c] = SHADE_NONE;
    // The next cure reads the composition aggregates of the stack instead of
    // the stack itself: refresh them from the strata as stored (rounded), as
    // the strata pass does for the cells it writes.
#pragma unroll
    for (int k = 0; k < 4; ++k)
#pragma unroll
      for (int q = 0; q < 16; ++q) s.pg[k][q] = PigIO<MODE>::round(s.pg[k][q], q);
    F.agg[c] = stack_agg(P, lt, s);
  }
}

}  // namespace

// Enqueues the film's pending deposits (before the frame's mark_tiles) and
// clears them; returns the number of launches.
uint32_t launch_pending_deposits(cf_film* f, cudaStream_t st) {
  if (f->dep_pending == 0u) return 0u;
  const DepTables D{f->d_deps, f->d_dep_tiles, f->d_dep_tiles + f->dep_nt, f->d_dep_items};
  uint32_t* count = f->d_dep_tiles + 2 * f->dep_nt;
  const uint32_t* tiles64 = f->d_dep_tiles + 2 * f->dep_nt + 1;  // the 64x64 tiles that list deposits
  uint32_t* painted = f->F.fill_list;  // frame scratch: the frame's strata pass rebuilds it
  if (cudaMemsetAsync(count, 0, sizeof(uint32_t), st) != cudaSuccess) return 0u;  // deposits stay pending
  k_deposit_mark<<<f->dep_tiles_listed * 16u, dim3(16, 16), 0, st>>>(f->F, D, tiles64, painted, count);
  int sms = 0, dev = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const dim3 g((unsigned)std::max(sms, 1) * 4u), b(256);
  if (f->prec == CF_PREC_REFERENCE)
    k_deposit_lay<CF_PREC_REFERENCE><<<g, b, 0, st>>>(f->F, D, painted, count);
  else if (f->prec == CF_PREC_FP32)
    k_deposit_lay<CF_PREC_FP32><<<g, b, 0, st>>>(f->F, D, painted, count);
  else
    k_deposit_lay<CF_PREC_BF16><<<g, b, 0, st>>>(f->F, D, painted, count);
  f->dep_pending = 0u;
  return 2u;
}

extern "C" {

cf_status cf_deposit_ribbon(const float p0[2], const float p1[2], const float n0[2], const float n1[2], float r0,
                            float r1, uint32_t caps, float volume, const uint32_t pig[8], float dx,
                            cf_deposit* out) {  // src/film/mod.rs:63-80
  if (!p0 || !p1 || !n0 || !n1 || !pig || !out || !(dx > 0.f)) return CF_ERR_INVALID_ARG;
  const float min_r = 0.8f * dx;
  const float a = std::max(r0, min_r), b = std::max(r1, min_r);
  cf_deposit d{};
  std::memcpy(d.p0, p0, 8);
  std::memcpy(d.p1, p1, 8);
  std::memcpy(d.n0, n0, 8);
  std::memcpy(d.n1, n1, 8);
  d.r0 = a;
  d.r1 = b;
  d.h0 = a;
  d.vol = volume;
  d.kind = caps;
  std::memcpy(d.pig, pig, 32);
  const float lattice = 0.25f * dx;
  const float sampled = sampled_volume(d, lattice);
  const float rm = std::max(a, b);
  const float disc = 3.14159265358979323846f * rm * rm * rm / 2.0f;
  if (sampled < 0.25f * disc) {
    const float mid[2] = {0.5f * (p0[0] + p1[0]), 0.5f * (p0[1] + p1[1])};
    std::memcpy(d.p0, mid, 8);
    std::memcpy(d.p1, mid, 8);
    d.r0 = rm;
    d.r1 = rm;
    d.h0 = rm;
    d.h0 = volume / sampled_volume(d, lattice) * rm;
    *out = d;
    return CF_OK;
  }
  d.h0 = volume / sampled * a;
  *out = d;
  return CF_OK;
}

cf_status cf_deposit_capsule(const float p0[2], const float p1[2], float r, float volume, const uint32_t pig[8],
                             float dx, cf_deposit* out) {  // src/film/mod.rs:82-85
  if (!p0 || !p1) return CF_ERR_INVALID_ARG;
  const Dir sd = segment_dir(p0, p1);
  return cf_deposit_ribbon(p0, p1, sd.d, sd.d, r, r, CAP_START | CAP_END, volume, pig, dx, out);
}

cf_status cf_deposit_stroke(const float p0[2], const float p1[2], float r, float volume, const uint32_t pig[8],
                            float dx, cf_deposit* out) {  // src/film/mod.rs:87-93
  if (!p0 || !p1) return CF_ERR_INVALID_ARG;
  const Dir sd = segment_dir(p0, p1);
  if (sd.l < std::max(r, 0.8f * dx)) return cf_deposit_capsule(p0, p1, r, volume, pig, dx, out);
  return cf_deposit_ribbon(p0, p1, sd.d, sd.d, r, r, 0u, volume, pig, dx, out);
}

cf_status cf_lay_deposits(cf_film* f, void* stream) {
  if (!f) return CF_ERR_INVALID_ARG;
  if (f->S.slump) return fail(f, CF_ERR_UNSUPPORTED, "slump pass is not implemented (reference default is off)");
  cudaStream_t st = (cudaStream_t)stream;
  cf_status s = upload_params(f, st);
  if (s != CF_OK) return s;
  f->launches += launch_pending_deposits(f, st);
  CUDA_TRY(f, cudaGetLastError());
  return CF_OK;
}

cf_status cf_deposit_sampled_volume(const cf_deposit* d, float lattice, float* out) {
  if (!d || !out || !(lattice > 0.f)) return CF_ERR_INVALID_ARG;
  *out = sampled_volume(*d, lattice);
  return CF_OK;
}

cf_status cf_deposit_height_at(const cf_deposit* d, const float p[2], float* out) {
  if (!d || !p || !out) return CF_ERR_INVALID_ARG;
  *out = profile(*d, p);
  return CF_OK;
}

cf_status cf_upload_deposits(cf_film* f, const cf_deposit* deps, uint32_t count, uint32_t* sent,
                             double* total_deposited) {
  if (!f || (count && !deps)) return fail(f, CF_ERR_INVALID_ARG, "cf_upload_deposits");
  count = std::min(count, CF_MAX_DEPOSITS);  // the rest waits for the next frame
  const float dx = f->S.width_m / (float)f->w, tile_m = 64.0f * dx;
  const uint32_t tx_n = (f->w + 63) / 64, ty_n = (f->h + 63) / 64, nt = tx_n * ty_n;
  std::vector<std::vector<uint32_t>> lists(nt);
  const float wm = f->S.width_m, hm = f->S.height_m;
  for (uint32_t di = 0; di < count; ++di) {  // upload_deposits, src/film/mod.rs:1180-1205
    const cf_deposit& d = deps[di];
    const float rb = max_radius(d);
    f->h_max_pending = std::max(f->h_max_pending, d.h0 * rb / d.r0 + f->h_max_stat);
    const float minx = std::min(d.p0[0], d.p1[0]) - rb, maxx = std::max(d.p0[0], d.p1[0]) + rb;
    const float miny = std::min(d.p0[1], d.p1[1]) - rb, maxy = std::max(d.p0[1], d.p1[1]) + rb;
    const bool inside = maxx > 0.0f && maxy > 0.0f && minx < wm && miny < hm;
    if (!inside) continue;
    if ((d.kind & RECYCLED) == 0u) f->total_deposited += (double)d.vol * (double)inside_fraction(d, wm, hm);
    if (maxx < 0.0f || maxy < 0.0f) continue;
    auto clampt = [](float v, uint32_t n) {
      return (int64_t)std::min<int64_t>((int64_t)std::max(std::floor(v), 0.0f), (int64_t)n - 1);
    };
    const int64_t tx0 = clampt(minx / tile_m, tx_n), tx1 = clampt(maxx / tile_m, tx_n);
    const int64_t ty0 = clampt(miny / tile_m, ty_n), ty1 = clampt(maxy / tile_m, ty_n);
    for (int64_t ty = ty0; ty <= ty1; ++ty)
      for (int64_t tx = tx0; tx <= tx1; ++tx) lists[(size_t)(ty * tx_n + tx)].push_back(di);
  }
  std::vector<uint32_t> start(nt), cnt(nt), items, listed;
  const size_t cap = (size_t)CF_MAX_DEPOSITS * 16;  // tile_items holds 16 entries per deposit
  for (uint32_t t = 0; t < nt; ++t) {
    const size_t take = std::min(lists[t].size(), cap - items.size());
    start[t] = (uint32_t)items.size();
    cnt[t] = (uint32_t)take;
    items.insert(items.end(), lists[t].begin(), lists[t].begin() + (ptrdiff_t)take);
    if (take) listed.push_back(t);
  }
  // device copies (grown as needed; the previous frame's are no longer read
  // once the stream has passed them)
  CUDA_TRY(f, cudaDeviceSynchronize());
  if (count > f->dep_cap) {
    if (f->d_deps) cudaFree(f->d_deps);
    f->d_deps = nullptr;
    CUDA_TRY(f, cudaMalloc(&f->d_deps, sizeof(cf_deposit) * count));
    f->dep_cap = count;
  }
  if (items.size() > f->dep_items_cap) {
    if (f->d_dep_items) cudaFree(f->d_dep_items);
    f->d_dep_items = nullptr;
    CUDA_TRY(f, cudaMalloc(&f->d_dep_items, sizeof(uint32_t) * std::max<size_t>(items.size(), 1)));
    f->dep_items_cap = items.size();
  }
  if (!f->d_dep_tiles) {  // start[nt], count[nt], the painted-cell counter, the listed tiles[<= nt]
    CUDA_TRY(f, cudaMalloc(&f->d_dep_tiles, sizeof(uint32_t) * (3 * nt + 1)));
    f->dep_nt = nt;
  }
  if (count) CUDA_TRY(f, cudaMemcpy(f->d_deps, deps, sizeof(cf_deposit) * count, cudaMemcpyHostToDevice));
  CUDA_TRY(f, cudaMemcpy(f->d_dep_tiles, start.data(), sizeof(uint32_t) * nt, cudaMemcpyHostToDevice));
  CUDA_TRY(f, cudaMemcpy(f->d_dep_tiles + nt, cnt.data(), sizeof(uint32_t) * nt, cudaMemcpyHostToDevice));
  if (!items.empty()) {
    CUDA_TRY(f, cudaMemcpy(f->d_dep_items, items.data(), sizeof(uint32_t) * items.size(), cudaMemcpyHostToDevice));
    CUDA_TRY(f, cudaMemcpy(f->d_dep_tiles + 2 * nt + 1, listed.data(), sizeof(uint32_t) * listed.size(),
                           cudaMemcpyHostToDevice));
  }
  f->dep_tiles_listed = (uint32_t)listed.size();
  f->dep_pending = items.empty() ? 0u : count;
  if (sent) *sent = count;
  if (total_deposited) *total_deposited = f->total_deposited;
  return CF_OK;
}

}  // extern "C"
