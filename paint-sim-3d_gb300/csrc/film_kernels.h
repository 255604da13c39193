// film_kernels.h — host launchers of the thin-film kernels (film_kernels.cu).
#pragma once

#include <cuda_runtime.h>

#include "film_device.cuh"

namespace cfk {

// One frame of Film::encode_frame with `substeps` film substeps; swaps F's
// strata generations; returns the number of kernel launches.
uint32_t launch_frame(Film& F, int mode, uint32_t substeps, int all_active, cudaStream_t st);
// Device-side adaptive dt and dt-dependent params from the last frame's stats.
void launch_adaptive_params(DevParams* Dp, DevStats* S, cudaStream_t st);
void launch_cure(const Film& F, int mode, cudaStream_t st);
// Composition aggregates (and, with shade, the colour) of the current state.
void launch_compose(const Film& F, int mode, int shade, cudaStream_t st);
void launch_reduce(const Film& F, int mode, cudaStream_t st);
void launch_mass(const Film& F, int sms, cudaStream_t st);
void launch_fill_u32(uint32_t* p, uint32_t v, size_t n, cudaStream_t st);
// Pigments between the reference layout [cell][stratum][slot] (element
// format fmt) and the chunk-major planes `chunks`.
void launch_pig_import(const Film& F, int mode, uint4* chunks, const void* src, int fmt, cudaStream_t st);
void launch_pig_export(const Film& F, int mode, const uint4* chunks, void* dst, int fmt, cudaStream_t st);
void launch_rheo_import(const Film& F, int mode, const float2* src, float n_global, size_t n, cudaStream_t st);
void launch_rheo_export(const Film& F, int mode, float2* dst, size_t n, cudaStream_t st);
int launch_one(Film& F, int mode, const char* name, int all_active, cudaStream_t st);

}  // namespace cfk
