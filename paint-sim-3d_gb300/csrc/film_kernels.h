// film_kernels.h — host launchers of the thin-film kernels (film_kernels.cu).
#pragma once

#include <cuda_runtime.h>

#include "film_device.cuh"

namespace cfk {

// What one launch of the frame kernels covers: the records of one or more
// films of one precision mode and a table of all their 16x16 tiles.  A film
// stepped alone is a view of its own two records and tiles; a batch is a view
// of many films; both run the same compiled kernels, so a film's result does
// not depend on what else shares the launch.
struct PackedFrame {
  const Film* films;       // device array: the films as the frame starts
  const Film* films_next;  // the same films with the strata generations swapped
  const uint2* tiles;      // entries (film index, 16x16 tile index)
  uint32_t ntiles;
  uint32_t nfilms;
  uint32_t persist_blocks; // grid of the strata list kernels
  // blocks of the per-tile kernels: 0 = one per tile entry; fewer make each
  // block walk a run of consecutive entries (a strip of tiles along a row)
  uint32_t tile_grid = 0;
  // implicit hydrostatic steps launched (each film's kernels skip the steps
  // beyond its own count), CG iterations per step (each film stops at its
  // own), and whether any film has the implicit capillary term
  uint32_t implicit_steps = 0;
  uint32_t implicit_iters = 40;
  bool cap_implicit = false;
};

// The kernels of implicit step `step` (cg.cu); returns the launch count.
uint32_t launch_cg_step(const PackedFrame& V, int mode, uint32_t step, uint32_t iters, bool cap_implicit,
                        cudaStream_t st);

// One frame of Film::encode_frame for every film of V with `substeps`
// substeps (adaptive: each film's dt chosen on the device first, one
// substep); returns the number of kernel launches.  The caller swaps each
// film's generations afterwards (films_next is the next frame's films).
uint32_t launch_frame_packed(const PackedFrame& V, int mode, uint32_t substeps, int adaptive, cudaStream_t st);
// cure_step on its own (dry_now).
void launch_cure(const PackedFrame& V, int mode, cudaStream_t st);
// Composition aggregates (and, with shade, the colour) of the current state.
void launch_compose(const PackedFrame& V, int mode, int shade, cudaStream_t st);
// Stats reset + the CFL reduction (h_max, mu_min) of the current state.
void launch_reduce(const PackedFrame& V, int mode, cudaStream_t st);
// A single named dispatch (inspection); 0: unknown name, 2: the caller swaps
// the strata generations.
int launch_one(const PackedFrame& V, int mode, const char* name, cudaStream_t st);

void launch_mass(const Film& F, int sms, cudaStream_t st);
void launch_fill_u32(uint32_t* p, uint32_t v, size_t n, cudaStream_t st);
// Pigments between the reference layout [cell][stratum][slot] (element
// format fmt) and the chunk-major planes `chunks`.
void launch_pig_import(const Film& F, int mode, uint4* chunks, const void* src, int fmt, cudaStream_t st);
void launch_pig_export(const Film& F, int mode, const uint4* chunks, void* dst, int fmt, cudaStream_t st);
void launch_rheo_import(const Film& F, int mode, const float2* src, float n_global, size_t n, cudaStream_t st);
void launch_rheo_export(const Film& F, int mode, float2* dst, size_t n, cudaStream_t st);

}  // namespace cfk
