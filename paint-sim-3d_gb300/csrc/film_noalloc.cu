// film_noalloc.cu — CFL statistics of a height field without any allocation.
//
// Some callers cannot allocate device memory at the moment they need these
// numbers: a render or paint loop that has done all of its cudaMalloc at
// start-up (an allocation can synchronise the device and stall a frame), a
// host that hands the library a fixed memory budget and accounts for every
// byte itself, or a plugin host that forbids allocation outside its own
// allocator.  cf_cfl_stats_noalloc serves them: it computes the same h_max /
// mu_min as the film's tile reduction (reduce_tiles) from caller-owned device
// planes, and its only scratch is the file-scope array below.
#include <cuda.h>
#include <cuda_runtime.h>

#include <mutex>

#include "../../include/canvaz_film.h"

namespace {

// One (h_max, mu_min) partial per 64 x 64 tile.  Every launch writes the
// partials of all tiles it covers before the final pass reads them, so nothing
// has to be cleared between calls.  Every call on a device shares this array.
static __device__ __align__(256) float2 g_cfl_partials[CF_NOALLOC_MAX_TILES];

constexpr int kMaxDevices = 64;

// The array's device address for the context that was current when it was
// looked up.  A context that is destroyed and created again (cudaDeviceReset
// in the caller, or a different driver context made current on the same
// device) loads the module anew, possibly at another address, so the entry is
// keyed on the context's unique id and looked up again when that id changes.
struct ScratchEntry {
  unsigned long long ctx_id;
  float2* addr;
};
ScratchEntry g_scratch[kMaxDevices] = {};
std::mutex g_setup_mu;

using CtxGetCurrentFn = CUresult (*)(CUcontext*);
using CtxGetIdFn = CUresult (*)(CUcontext, unsigned long long*);

// Driver entry points for the current context's id, found through the
// runtime (the library does not link the driver library itself).
bool driver_fns(CtxGetCurrentFn* cur, CtxGetIdFn* id) {
  static CtxGetCurrentFn s_cur = nullptr;
  static CtxGetIdFn s_id = nullptr;
  static bool s_done = false;
  if (!s_done) {
    void* a = nullptr;
    void* b = nullptr;
    cudaDriverEntryPointQueryResult qa{}, qb{};
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &a, 12000, cudaEnableDefault, &qa) == cudaSuccess &&
        cudaGetDriverEntryPointByVersion("cuCtxGetId", &b, 12000, cudaEnableDefault, &qb) == cudaSuccess &&
        qa == cudaDriverEntryPointSuccess && qb == cudaDriverEntryPointSuccess) {
      s_cur = reinterpret_cast<CtxGetCurrentFn>(a);
      s_id = reinterpret_cast<CtxGetIdFn>(b);
    }
    cudaGetLastError();
    s_done = true;
  }
  *cur = s_cur;
  *id = s_id;
  return s_cur != nullptr && s_id != nullptr;
}

// Id of the current context, 0 when none is current yet.
unsigned long long current_ctx_id(CtxGetCurrentFn cur, CtxGetIdFn id) {
  CUcontext ctx = nullptr;
  unsigned long long v = 0;
  if (cur(&ctx) != CUDA_SUCCESS || ctx == nullptr) return 0;
  if (id(ctx, &v) != CUDA_SUCCESS) return 0;
  return v;
}

// Device address of the scratch array on `dev` (current device): looked up
// once per device and context (set-up), then taken from the table.
cf_status scratch_address(int dev, float2** out) {
  if (dev < 0 || dev >= kMaxDevices) return CF_ERR_UNSUPPORTED;
  std::lock_guard<std::mutex> lock(g_setup_mu);
  CtxGetCurrentFn cur = nullptr;
  CtxGetIdFn id = nullptr;
  const bool have_ids = driver_fns(&cur, &id);
  ScratchEntry& e = g_scratch[dev];
  if (have_ids && e.addr != nullptr) {
    const unsigned long long now = current_ctx_id(cur, id);
    if (now != 0 && now == e.ctx_id) {
      *out = e.addr;
      return CF_OK;
    }
  }
  // set-up: the lookup makes the device's primary context current if no
  // context is, then the context it answered for is recorded
  void* p = nullptr;
  const cudaError_t err = cudaGetSymbolAddress(&p, g_cfl_partials);
  if (err != cudaSuccess || p == nullptr) {
    cudaGetLastError();
    return CF_ERR_CUDA;
  }
  e.addr = static_cast<float2*>(p);
  e.ctx_id = have_ids ? current_ctx_id(cur, id) : 0;
  *out = e.addr;
  return CF_OK;
}

// Pass 1: the partial of each 64 x 64 tile over the cells with h > 4 h_min
// (the reduction of film.wgsl:1330-1361).  The grid is one-dimensional, one
// block per tile in row-major tile order (tw tiles a row), so any tile count
// up to CF_NOALLOC_MAX_TILES launches, whatever the canvas's aspect.
__global__ void __launch_bounds__(256) k_cfl_tiles(const float* __restrict__ h, const float* __restrict__ mu,
                                                   uint32_t w, uint32_t hgt, uint32_t tw, float thr,
                                                   float2* partials) {
  const uint32_t bx = blockIdx.x % tw, by = blockIdx.x / tw;
  float hm = 0.f, mm = 1e9f;
  for (int dy = 0; dy < 4; ++dy)
    for (int dx = 0; dx < 4; ++dx) {
      uint32_t i = bx * 64 + threadIdx.x * 4 + dx, j = by * 64 + threadIdx.y * 4 + dy;
      if (i < w && j < hgt) {
        size_t c = (size_t)j * w + i;
        float v = h[c];
        if (v > thr) { hm = fmaxf(hm, v); mm = fminf(mm, mu[c]); }
      }
    }
  for (int o = 16; o > 0; o >>= 1) {
    hm = fmaxf(hm, __shfl_xor_sync(0xffffffffu, hm, o));
    mm = fminf(mm, __shfl_xor_sync(0xffffffffu, mm, o));
  }
  __shared__ float sh[8], sm[8];
  int t = threadIdx.y * 16 + threadIdx.x, lane = t & 31, wid = t >> 5;
  if (lane == 0) { sh[wid] = hm; sm[wid] = mm; }
  __syncthreads();
  if (wid == 0) {
    hm = lane < 8 ? sh[lane] : 0.f;
    mm = lane < 8 ? sm[lane] : 1e9f;
    for (int o = 4; o > 0; o >>= 1) {
      hm = fmaxf(hm, __shfl_xor_sync(0xffffffffu, hm, o));
      mm = fminf(mm, __shfl_xor_sync(0xffffffffu, mm, o));
    }
    if (lane == 0) partials[blockIdx.x] = make_float2(hm, mm);
  }
}

// Pass 2: one block folds the partials into (h_max, mu_min), mapping an empty
// minimum to 1 as poll_stats does (src/film/mod.rs:944-953).
__global__ void __launch_bounds__(1024) k_cfl_final(const float2* partials, uint32_t ntiles, float* out) {
  float hm = 0.f, mm = 1e9f;
  for (uint32_t t = threadIdx.x; t < ntiles; t += blockDim.x) {
    float2 p = partials[t];
    hm = fmaxf(hm, p.x);
    mm = fminf(mm, p.y);
  }
  for (int o = 16; o > 0; o >>= 1) {
    hm = fmaxf(hm, __shfl_xor_sync(0xffffffffu, hm, o));
    mm = fminf(mm, __shfl_xor_sync(0xffffffffu, mm, o));
  }
  __shared__ float sh[32], sm[32];
  int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0) { sh[wid] = hm; sm[wid] = mm; }
  __syncthreads();
  if (wid == 0) {
    hm = lane < (int)(blockDim.x >> 5) ? sh[lane] : 0.f;
    mm = lane < (int)(blockDim.x >> 5) ? sm[lane] : 1e9f;
    for (int o = 16; o > 0; o >>= 1) {
      hm = fmaxf(hm, __shfl_xor_sync(0xffffffffu, hm, o));
      mm = fminf(mm, __shfl_xor_sync(0xffffffffu, mm, o));
    }
    if (lane == 0) {
      out[0] = hm;
      out[1] = mm > 1e8f ? 1.0f : mm;
    }
  }
}

}  // namespace

extern "C" cf_status cf_cfl_stats_noalloc(const float* d_h, const float* d_mu, uint32_t w, uint32_t h, float h_min,
                                          float* d_out, void* stream) {
  if (!d_h || !d_mu || !d_out || w == 0 || h == 0) return CF_ERR_INVALID_ARG;
  const uint64_t tw64 = ((uint64_t)w + 63) / 64, th64 = ((uint64_t)h + 63) / 64;
  if (tw64 * th64 > CF_NOALLOC_MAX_TILES) return CF_ERR_INVALID_ARG;  // grid larger than the scratch
  const uint32_t tw = (uint32_t)tw64, th = (uint32_t)th64;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) {
    cudaGetLastError();
    return CF_ERR_CUDA;
  }
  float2* partials = nullptr;
  cf_status s = scratch_address(dev, &partials);
  if (s != CF_OK) return s;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  k_cfl_tiles<<<tw * th, dim3(16, 16), 0, st>>>(d_h, d_mu, w, h, tw, 4.0f * h_min, partials);
  k_cfl_final<<<1, 1024, 0, st>>>(partials, tw * th, d_out);
  if (cudaGetLastError() != cudaSuccess) return CF_ERR_CUDA;
  return CF_OK;
}
