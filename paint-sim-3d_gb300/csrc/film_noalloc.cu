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
#include <cuda_runtime.h>

#include <mutex>

#include "../../include/canvaz_film.h"

namespace {

// One (h_max, mu_min) partial per 64 x 64 tile.  Every launch writes the
// partials of all tiles it covers before the final pass reads them, so nothing
// has to be cleared between calls.  Every call on a device shares this array.
static __device__ __align__(256) float2 g_cfl_partials[CF_NOALLOC_MAX_TILES];

constexpr int kMaxDevices = 64;
float2* g_partials_addr[kMaxDevices] = {};
std::mutex g_setup_mu;

// Device address of the scratch array on `dev` (current device), looked up
// once per device.
cf_status scratch_address(int dev, float2** out) {
  if (dev < 0 || dev >= kMaxDevices) return CF_ERR_UNSUPPORTED;
  std::lock_guard<std::mutex> lock(g_setup_mu);
  if (!g_partials_addr[dev]) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_cfl_partials);
    if (e != cudaSuccess || p == nullptr) {
      cudaGetLastError();
      return CF_ERR_CUDA;
    }
    g_partials_addr[dev] = static_cast<float2*>(p);
  }
  *out = g_partials_addr[dev];
  return CF_OK;
}

// Pass 1: the partial of each 64 x 64 tile over the cells with h > 4 h_min
// (the reduction of film.wgsl:1330-1361).
__global__ void __launch_bounds__(256) k_cfl_tiles(const float* __restrict__ h, const float* __restrict__ mu,
                                                   uint32_t w, uint32_t hgt, float thr, float2* partials) {
  float hm = 0.f, mm = 1e9f;
  for (int dy = 0; dy < 4; ++dy)
    for (int dx = 0; dx < 4; ++dx) {
      uint32_t i = blockIdx.x * 64 + threadIdx.x * 4 + dx, j = blockIdx.y * 64 + threadIdx.y * 4 + dy;
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
    if (lane == 0) partials[blockIdx.x + blockIdx.y * gridDim.x] = make_float2(hm, mm);
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
  const uint32_t tw = (w + 63) / 64, th = (h + 63) / 64;
  if ((uint64_t)tw * th > CF_NOALLOC_MAX_TILES) return CF_ERR_INVALID_ARG;  // grid larger than the scratch
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) {
    cudaGetLastError();
    return CF_ERR_CUDA;
  }
  float2* partials = nullptr;
  cf_status s = scratch_address(dev, &partials);
  if (s != CF_OK) return s;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  k_cfl_tiles<<<dim3(tw, th), dim3(16, 16), 0, st>>>(d_h, d_mu, w, h, 4.0f * h_min, partials);
  k_cfl_final<<<1, 1024, 0, st>>>(partials, tw * th, d_out);
  if (cudaGetLastError() != cudaSuccess) return CF_ERR_CUDA;
  return CF_OK;
}
