/*
 * canvaz_film_debug.h — inspection entry points of the thin-film library.
 *
 * These have no counterpart in the reference's Film API; they expose the
 * scratch planes the reference keeps in wgpu buffers (pres, flux, acc, alpha,
 * delta, tmp, acc_s, alpha_s, strata_*2, h_frame, fnorm, tile flags;
 * src/film/mod.rs:586-628), and this library's own per-cell face flags
 * ("fflags": bit f set where strata_split wrote a nonzero face f), so that a
 * single dispatch can be checked against a CPU oracle, and "h_next" and
 * "delta_old", where the frame's fused limiter + apply leaves the new heights
 * and the front-offset snapshot for the nose.  All calls are synchronous.
 */
#ifndef CANVAZ_FILM_DEBUG_H
#define CANVAZ_FILM_DEBUG_H

#include "canvaz_film.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Element kinds of a plane. */
#define CF_ELEM_F32 0
#define CF_ELEM_U32 1
#define CF_ELEM_F16 2
#define CF_ELEM_BF16 3
#define CF_ELEM_I32 4

/* Size in bytes and element kind of a named plane ("h", "pres", "strata_pig", ...). */
cf_status cf_debug_plane_info(cf_film* film, const char* name, size_t* bytes, int32_t* elem);

/* Copies a whole named plane to / from host memory (`bytes` must match). */
cf_status cf_debug_read(cf_film* film, const char* name, void* host, size_t bytes);
cf_status cf_debug_write(cf_film* film, const char* name, const void* host, size_t bytes);

/* Runs one dispatch of Film::encode_frame by its WGSL entry-point name
 * ("laplacian", "fluxes", "strata_update", "shade_full", ...; "deposit" lays
 * the deposits uploaded since the last frame and drops them), or the fused
 * kernels the frame runs in each substep: "flow" (laplacian + plug +
 * fluxes) and "limit_apply" (limiter + apply, the new heights in "h_next"). */
cf_status cf_debug_run(cf_film* film, const char* kernel, void* stream);

/* Overwrites the device params with `params` (no re-packing). */
cf_status cf_debug_set_params(cf_film* film, const cf_params* params);

#ifdef __cplusplus
}
#endif

#endif /* CANVAZ_FILM_DEBUG_H */
