/*
 * canvaz_film.h — C ABI of the GB300 (sm_103a) thin-film step.
 *
 * This library replaces the wgpu film pass of Canvaz (lukaszkujawa/paint-sim-3d):
 * the Herschel–Bulkley lubrication height update (shaders/film.wgsl), the upwind
 * strata/pigment transport (shaders/film.wgsl strata_split + shaders/strata.wgsl),
 * cure/rheology (shaders/cure.wgsl) and the Kubelka–Munk shade
 * (shaders/km.wgsl + shaders/shade.wgsl).  Every entry point below names the
 * Rust method of `impl Film` (src/film/mod.rs) it stands in for.
 *
 * Conventions
 *  - Every function returns cf_status; no exception or abort crosses the ABI.
 *  - A cf_film handle is used by one host thread at a time (the reference's
 *    Film lives on the winit thread and is not shared either).
 *  - `stream` is a cudaStream_t passed as void*; NULL means the legacy default
 *    stream.  Work is enqueued; call cf_sync (or synchronise the stream) before
 *    reading results on the host, exactly like wgpu's queue.submit + map_async.
 *  - All per-cell planes are row-major, cell (i, j) at index j * w + i.
 */
#ifndef CANVAZ_FILM_H
#define CANVAZ_FILM_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define CF_ABI_VERSION 1
#define CF_STRATA 4        /* shaders/common.wgsl:43 STRATA   */
#define CF_NPIG 12         /* shaders/common.wgsl:44 NPIG     */
#define CF_PIG_SLOTS 16    /* 12 pigments, 12 thinner, 13 yield, 14 ln(mu)+10, 15 flow index n */
#define CF_NBAND 16        /* shaders/common.wgsl:45 NBAND    */
#define CF_PIG_STRIDE 40   /* shaders/common.wgsl:46 PIG_STRIDE */
#define CF_TILE 16         /* 16x16 activity tiles, shaders/film.wgsl:1365-1425 */
#define CF_STATS_TILE 64   /* reduce_tiles tile, shaders/common.wgsl:47 TILE */

typedef enum cf_status {
    CF_OK = 0,
    CF_ERR_INVALID_ARG = 1,
    CF_ERR_OUT_OF_MEMORY = 2,
    CF_ERR_CUDA = 3,
    CF_ERR_TIMEOUT = 4,
    CF_ERR_NAN = 5,
    CF_ERR_UNSUPPORTED = 6,
    CF_ERR_NOT_READY = 7
} cf_status;

/* Storage precision of the pigment strata and of the rheology plane.
 * Height, flux, K/S and all arithmetic stay FP32 in every mode. */
typedef enum cf_precision {
    CF_PREC_REFERENCE = 0, /* f16 pigment slots, f32 rheology: the reference layout */
    CF_PREC_FP32 = 1,      /* f32 pigment slots, f32 rheology                       */
    CF_PREC_BF16 = 2       /* bf16 pigment slots, bf16 rheology (slot 14 kept as mu) */
} cf_precision;

/* Element format of the strata_pig plane handed to cf_write_state / cf_read_state. */
typedef enum cf_pig_format {
    CF_PIG_F16 = 0,  /* 4 strata x 16 slots x IEEE half: 128 B per cell (reference layout) */
    CF_PIG_F32 = 1,  /* 4 strata x 16 slots x float:     256 B per cell                    */
    CF_PIG_BF16 = 2  /* 4 strata x 16 slots x bfloat16:  128 B per cell                    */
} cf_pig_format;
/* In the bfloat16 format (and in CF_PREC_BF16 films' storage) slot 14 of each
 * stratum, whose value is the viscosity override ln mu + 10 (0 = none), is
 * stored as mu itself in Pa s (0 = none): bfloat16's 8 significant bits step
 * by 0.0625 on ln mu + 10 (about 6 % on mu) but by 0.4 % on mu.  Every other
 * slot, and every other format, stores the slot's value. */

/* FilmSettings (src/film/mod.rs:281-350).  The reference reads its ablation
 * switches from environment variables inside update_params
 * (src/film/mod.rs:870-915); here they are plain fields. */
typedef struct cf_settings {
    float width_m;            /* canvas width; dx = width_m / w          */
    float height_m;
    float rho;                /* density kg/m^3                          */
    float sigma;              /* surface tension N/m                     */
    float n_index;            /* global power-law index (slot 15 = 0)    */
    float m_cap;              /* capillary mobility cap                  */
    float contact_angle_deg;
    float hysteresis_deg;
    float h_star;             /* precursor / disjoining thickness        */
    int32_t raw_canvas;       /* substrate reflectance at cf_create      */
    float weave_um;           /* canvas weave amplitude at cf_create     */
    float cure_rate;
    float tau_cure;
    float lnmu_cure;
    float v_cap;
    float tilt_deg;
    float tilt_dir_deg;
    float gravity;
    float medium_mu;
    uint32_t debug_view;      /* 1 = invariant view in the shade        */
    float h_min;
    float m_cap_hydro;
    uint32_t max_substeps;
    uint32_t min_substeps;
    uint32_t implicit_iters;
    int32_t implicit_hydro;   /* implicit hydrostatic CG steps (film.wgsl:895-1302); fixed at cf_create */
    int32_t slump;            /* slump pass: only 0 is supported (reference default) */
    int32_t capillary;
    int32_t capillary_implicit;
    /* environment toggles of update_params */
    int32_t no_hold;          /* PAINT_NO_HOLD     */
    int32_t no_transl;        /* PAINT_NO_TRANSL   */
    int32_t no_shape;         /* PAINT_NO_SHAPE    */
    int32_t no_cap;           /* PAINT_NO_CAP      */
    float kshape;             /* PAINT_KSHAPE (1)  */
    float kline;              /* PAINT_KLINE (0)   */
    float hyst_deg;           /* PAINT_HYST; < 0 means use hysteresis_deg */
    float fcap_exp;           /* PAINT_FCAP (2.5)  */
    float cap_cond;           /* PAINT_CAPCOND (80) */
    /* extension: 1 = every 16x16 tile is active every frame (compact_tiles
     * marks all tiles); 0 = the reference's moved-tile activity. */
    int32_t all_active;
} cf_settings;

/* Params uniform (src/film/mod.rs:5-23, shaders/common.wgsl:1-17), 176 bytes. */
typedef struct cf_params {
    uint32_t size[2];
    uint32_t tiles[2];
    float dx, dt, inv_dx, frame_dt;
    float g[4];      /* (gx, gy, gz, |g|)                               */
    float phys[4];   /* (rho, sigma, n, m_cap)                          */
    float ein[4];    /* (tan theta, l_c sin(theta/2), Pi_A, h_min)      */
    float cure[4];   /* (rate, tau_cure, lnmu_cure, h_star)             */
    float misc[4];   /* (tiny stratum, merge distance, medium mu, m_hyd)*/
    uint32_t flags[4];
    float front[4];  /* (H_c, dx / l_c,z, m_imp_max, dt_i)              */
    float front2[4]; /* (hysteresis rad, kshape, kline, toggles)        */
    float front3[4]; /* (cc, kc, m_c, fcap exponent)                    */
} cf_params;

/* The eight persistent planes of Film::state_buffers (src/film/mod.rs:1277-1279),
 * plus an optional per-cell rheology flow index. Host or device pointers. */
typedef struct cf_state_view {
    void* h;            /* float[N]                  */
    void* m;            /* float[N]                  */
    void* rheo;         /* float2[N] (mu Pa s, tau_y Pa) */
    void* strata_h;     /* float4[N]                 */
    void* strata_pig;   /* 64 slots per cell, element type = pig_format */
    void* strata_cure;  /* float4[N]                 */
    void* sub_refl;     /* 16 x IEEE half per cell   */
    void* lay;          /* uint32[N]                 */
    int32_t pig_format; /* cf_pig_format             */
    int32_t device;     /* 0: host pointers, 1: device pointers */
} cf_state_view;

/* Host-side statistics (poll_stats src/film/mod.rs:935-973, compute_stats
 * src/main.rs:1679-1819).  Mass sums are FP64 on the device. */
typedef struct cf_stats {
    float h_max;           /* reduce_tiles: max h over cells with h > 4 h_min */
    float mu_min;          /* reduce_tiles: min mu over the same cells        */
    uint32_t active_tiles; /* compact_tiles count of the last frame           */
    uint32_t frames;       /* frames stepped since create                     */
    double wet_volume;     /* sum(h) dx^2                                     */
    double relief_volume;  /* sum(m) dx^2                                     */
    double last_dt;        /* substep dt of the last frame                    */
    uint64_t nan_cells;    /* non-finite h                                    */
    uint64_t wet_cells;
    uint64_t launches;     /* kernels this film has enqueued since create     */
} cf_stats;

typedef struct cf_film cf_film;

/* --- lifecycle ---------------------------------------------------------- */

/* FilmSettings::default (src/film/mod.rs:315-350). */
cf_status cf_settings_default(cf_settings* out);

/* Film::new (src/film/mod.rs:578-859): allocates the per-cell planes,
 * writes the substrate reflectance (substrate_refl :188-210), the weave relief
 * (weave :212-233) and rheo = (1, 0), then packs the params (update_params). */
cf_status cf_create(const cf_settings* settings, uint32_t w, uint32_t h,
                    int32_t precision, cf_film** out);
cf_status cf_destroy(cf_film* film);

/* Film::new :604-610 uploads pigment_table (src/color/mod.rs:243-258,
 * 12 x 40 floats) and cmf_table (src/color/mod.rs:150-171, 16 x 3 floats). */
cf_status cf_set_tables(cf_film* film, const float* pigtab, const float* cmf);

/* --- state I/O ------------------------------------------------------------ */

/* Film::write_state (src/film/mod.rs:1303-1320): uploads the planes, clears the
 * scratch planes (pres, flux, acc, alpha, delta, tmp, acc_s, strata_h2,
 * strata_pig2, alpha_s) and marks every activity tile moved.  A NULL plane
 * pointer leaves that plane unchanged.  Synchronous. */
cf_status cf_write_state(cf_film* film, const cf_state_view* state);

/* Film::read_state (src/film/mod.rs:1281-1301).  A NULL plane is skipped.
 * Synchronous. */
cf_status cf_read_state(cf_film* film, const cf_state_view* state);

/* --- per frame ------------------------------------------------------------ */

/* Film::update_params (src/film/mod.rs:869-917). */
cf_status cf_update_params(cf_film* film, float frame_dt, uint32_t substeps);

/* The packing of Film::update_params (src/film/mod.rs:869-917) without a film:
 * pure host arithmetic (f32, as the reference), usable without a GPU.
 * h_max / mu_min are the stats the reference polls (poll_stats :935-973). */
cf_status cf_pack_params(const cf_settings* settings, uint32_t w, uint32_t h, float frame_dt, uint32_t substeps,
                         float h_max, float mu_min, cf_params* out, uint32_t* implicit_steps);

/* Film::choose_substeps (src/film/mod.rs:919-933) from the stats of the last
 * frame (read back synchronously, the reference reads them 1-2 frames late). */
cf_status cf_choose_substeps(cf_film* film, float frame_dt, uint32_t* substeps);

/* Film::encode_frame (src/film/mod.rs:1322-1462), simulation portion: tile
 * activity, cure, the implicit hydrostatic steps that update_params chose
 * (each a CG solve of implicit_iters iterations), `substeps` x {laplacian,
 * plug, fluxes, limiter, apply, nose}, strata split/limit/update/copy/fill x 6,
 * tile stats and the full KM shade.  Uses the params of the last
 * cf_update_params. */
cf_status cf_encode_frame(cf_film* film, uint32_t substeps, void* stream);

/* One adaptive step: the substep dt is derived on the device from the
 * h_max / mu_min of the previous frame with the formulas of choose_substeps
 * (dt = min(dt_max, dt_cfl, dt_hyd, dt_cap)), the dt-dependent params (and
 * the implicit step count) are re-derived on the device, and one frame with
 * one substep is run.  No host round trip; graph-capturable.  With
 * implicit_hydro on, the launches cover 4 implicit steps and the film skips
 * the ones it does not take. */
cf_status cf_step_adaptive(cf_film* film, float dt_max, void* stream);

/* Film::dry_now (src/film/mod.rs:1230-1244): one cure pass with rate
 * 4 / frame_dt so every stratum commits. */
cf_status cf_dry_now(cf_film* film, void* stream);

/* --- outputs ------------------------------------------------------------- */

/* color_tex (rgba16float: linear sRGB + roughness) written by shade_full.
 * Device pointer, valid for the life of the film. */
cf_status cf_color_device_ptr(cf_film* film, void** ptr);

/* Copies the colour plane (4 x IEEE half per cell) to host memory. Synchronous. */
cf_status cf_read_color(cf_film* film, uint16_t* rgba16f_host);

/* Asynchronous forms for pipelines that keep the host link busy while
 * another film computes.  Every plane of the view must be device memory or
 * page-locked host memory (CF_ERR_INVALID_ARG otherwise); the work is
 * enqueued on `stream` and the caller waits on it.  After
 * cf_write_state_async the host's copy of the tile stats is refreshed by the
 * next cf_update_params, cf_choose_substeps, cf_get_stats or cf_sync.
 * cf_read_color_async takes a device or page-locked destination. */
cf_status cf_write_state_async(cf_film* film, const cf_state_view* view, void* stream);
cf_status cf_read_state_async(cf_film* film, const cf_state_view* view, void* stream);
cf_status cf_read_color_async(cf_film* film, uint16_t* rgba16f, void* stream);

/* Statistics of the last frame; synchronous. */
cf_status cf_get_stats(cf_film* film, cf_stats* out);

/* write_state(read_state(src)) into dst without a host round trip
 * (Film::read_state / write_state, src/film/mod.rs:1281-1320): copies src's
 * whole device state (every plane with both strata generations, tables,
 * params, stats) into dst on `stream`, so dst steps exactly as src would.
 * dst and src have the same size, precision, device and implicit_hydro.  A
 * serving loop admits a job by cloning a resident template canvas. */
cf_status cf_clone_state(cf_film* dst, const cf_film* src, void* stream);

/* Params of the last update (for parity checks of update_params). */
cf_status cf_get_params(cf_film* film, cf_params* out);

/* Waits for all work of this film. */
cf_status cf_sync(cf_film* film);

/* Human-readable text of the last error on this film (or of the last failed
 * cf_create when film is NULL). */
const char* cf_last_error(const cf_film* film);

/* Device bytes a film of w x h cells in `precision` holds (its arena, params,
 * stats, tables and tile table): what an admission policy budgets.  Pure host
 * function.  A film created with implicit_hydro holds 52 B per cell and 8 B
 * per 16x16 tile more (the CG planes). */
cf_status cf_film_bytes(uint32_t w, uint32_t h, int32_t precision, uint64_t* bytes);

/* --- deposits: paint laid on the film ------------------------------------------ */

/* Deposit (src/film/mod.rs:25-39): a ribbon segment p0 -> p1 with end
 * normals n0, n1 and radii r0, r1 (metres), peak height h0, volume vol, kind
 * (bit 0 recycled, bit 1 cap start, bit 2 cap end, bits 8+ laying method) and
 * 16 pigment slots packed as f16 pairs.  96 bytes, the reference's layout. */
typedef struct cf_deposit {
    float p0[2], p1[2], n0[2], n1[2];
    float r0, r1, h0, vol;
    uint32_t kind;
    uint32_t pad[3];
    uint32_t pig[8];
} cf_deposit;

/* Deposit::ribbon / capsule / stroke (src/film/mod.rs:63-93): h0 is set so
 * that the profile sampled on a 0.25 dx lattice holds `volume`.  Host
 * functions; f32 arithmetic in the reference's order. */
cf_status cf_deposit_ribbon(const float p0[2], const float p1[2], const float n0[2], const float n1[2], float r0,
                            float r1, uint32_t caps, float volume, const uint32_t pig[8], float dx, cf_deposit* out);
cf_status cf_deposit_capsule(const float p0[2], const float p1[2], float r, float volume, const uint32_t pig[8],
                             float dx, cf_deposit* out);
cf_status cf_deposit_stroke(const float p0[2], const float p1[2], float r, float volume, const uint32_t pig[8],
                            float dx, cf_deposit* out);
/* Deposit::sampled_volume and the profile height (src/film/mod.rs:115-185). */
cf_status cf_deposit_sampled_volume(const cf_deposit* d, float lattice, float* out);
cf_status cf_deposit_height_at(const cf_deposit* d, const float p[2], float* out);
/* upload_deposits (src/film/mod.rs:1175-1224): bins the first
 * min(count, CF_MAX_DEPOSITS) deposits into the film's 64x64-cell tiles
 * (at most 16 tile entries per deposit in all); the next frame
 * (cf_encode_frame, cf_step_adaptive or a batch step) lays them
 * (shaders/deposit.wgsl) before its mark_tiles.  *sent (may be NULL) gets the
 * number taken; the caller holds the rest for the next frame, as
 * src/main.rs:1882-1890 does.  *total_deposited (may be NULL) gets the running
 * volume laid inside the canvas.  Synchronous with the device. */
#define CF_MAX_DEPOSITS 65536u
cf_status cf_upload_deposits(cf_film* film, const cf_deposit* deps, uint32_t count, uint32_t* sent,
                             double* total_deposited);
/* Lays the uploaded deposits now, enqueued on `stream`, instead of at the
 * start of the next frame (no counterpart in the reference, which lays them
 * only inside Film::encode_frame; used where paint is laid while the film is
 * not stepped).  No-op when none are pending.  Asynchronous. */
cf_status cf_lay_deposits(cf_film* film, void* stream);

/* --- the render pass's reading of the film (shaders/render.wgsl) --------------- */

/* Relief and colour at canvas points (metres), as the renderer samples them
 * with its plain camera: per point 8 floats: surf_cubic (height of h + m,
 * :335-353), base_slope x and y (:628-638), color_sharp r, g, b, a
 * (:706-750), wet_bilinear (h, :394-406).  `points` (2 floats each) and
 * `out` are device memory; enqueued on `stream`. */
cf_status cf_sample_relief(cf_film* film, const float* points, uint32_t n, float* out, void* stream);

/* The renderer's key-light shadow (render.wgsl shadow_at :846-866, plain
 * camera): per point (x, y, z0) in metres, 2 floats: surf_bilinear(x, y)
 * (:314-326) and the shadow factor in [0, 1] of a ray from height z0 toward
 * `light` (unit vector, z up; 1 for light[2] <= 0.05), marched 20 steps of
 * 1.5 cells over the bilinear relief until it rises above `top`
 * (cam.canvas.w: the renderer passes max(h_max, s_max) + 0.5 mm).
 * `points` (3 floats each) and `out` are device memory; enqueued on
 * `stream`. */
cf_status cf_relief_shadow(cf_film* film, const float* points, uint32_t n, const float* light, float top, float* out,
                           void* stream);

/* A top-down view: pixel (x, y) samples the canvas point
 * (x0 + (x + 0.5) pixel_m, y0 + (y + 0.5) pixel_m), row 0 at the lowest y;
 * colour = color_sharp x (ambient + (1 - ambient) max(n . light, 0)) with
 * the normal of base_slope (normal_from_slope, :640-642), written as sRGB
 * RGBA8 to `rgba8` (device memory, width x height x 4 bytes).  The shading
 * is this library's, not the renderer's. */
typedef struct cf_relief_view {
    float x0, y0, pixel_m;
    uint32_t width, height;
    float light[3];
    float ambient;
    uint32_t reserved;
} cf_relief_view;
cf_status cf_render_relief(cf_film* film, const cf_relief_view* view, uint8_t* rgba8, void* stream);

/* The renderer's camera uniform (shaders/render.wgsl:1-15, CamUniform of
 * src/render/mod.rs:10-24), filled as Renderer::uniform (:162-180) fills
 * it: inv_vp and vp column-major; canvas = (width_m, height_m, dx,
 * max(h_max, s_max) + 0.5 mm); light = (direction, intensity); size =
 * (film w, h, 0, 0); jitter = (ndc offset x, y, beauty mode > 0.5, pixel
 * footprint in metres); ortho = (orthographic top-down > 0.5, tan of the
 * contact angle, colour-plane scale (0: the film's resolution), 0); basis_r,
 * basis_u: the camera's right and up; lens = (aperture offsets x, y, focus
 * distance, thin lens > 0.5). */
typedef struct cf_render_cam {
    float inv_vp[16];
    float eye[4];
    float canvas[4];
    float light[4];
    uint32_t size[4];
    float sky[4];
    float ground[4];
    float vp[16];
    float jitter[4];
    float ortho[4];
    float basis_r[4];
    float basis_u[4];
    float lens[4];
} cf_render_cam;

/* The renderer's fragment shader over the film (render.wgsl fs :985-1116, lit
 * :1118-1143): for each pixel of a width x height target (row 0 at the top,
 * the pixel centre's ndc as the full-screen triangle interpolates it), the
 * camera ray marched over the relief h + m, the tool micro-relief of the
 * film's detail texels, the sharpened (or beauty-mode) colour, the canvas
 * weave, key-light shadow, ambient occlusion, environment, softboxes and GGX
 * lobes, tonemapped to sRGB (beauty mode: linear, firefly-clamped).  Writes
 * RGBA as 4 floats a pixel to `rgba_f32` (16-byte aligned) and/or as RGBA8
 * to `rgba8` (4-byte aligned), device memory, either may be NULL but not
 * both.  cam->size must be the film's size.  Enqueued on `stream`. */
cf_status cf_render_lit(cf_film* film, const cf_render_cam* cam, uint32_t width, uint32_t height, float* rgba_f32,
                        uint8_t* rgba8, void* stream);

/* --- painting files (src/session.rs) ----------------------------------------- */

/* The header fields of a Canvaz painting file (src/session.rs:248-310). */
typedef struct cf_snapshot_info {
    uint32_t w, h;
    float tilt_deg, tilt_dir_deg, cure_rate, h_max, s_max;
    double total_deposited;
} cf_snapshot_info;

/* App::save_painting's bytes (src/session.rs:248-266: "PSIM", version 1,
 * w, h, the five header floats, total_deposited, then pack() of the eight
 * read_state planes in 32 MiB LZ4 chunks, src/session.rs:58-74).  The film's
 * w and h are written; info supplies the other header fields.  *out is
 * allocated by the library: release it with cf_snapshot_free. */
cf_status cf_snapshot_save(cf_film* film, const cf_snapshot_info* info, uint8_t** out, uint64_t* len);
cf_status cf_snapshot_free(uint8_t* buf);
/* App::open_painting (src/session.rs:277-310): checks magic, version and
 * canvas size, unpacks (src/session.rs:76-99) and writes the state
 * (write_state); fills info (may be NULL) from the header. */
cf_status cf_snapshot_load(cf_film* film, const uint8_t* data, uint64_t len, cf_snapshot_info* info);
/* The chunk coder of the painting file (lz4_flex 0.11 compress_prepend_size /
 * decompress_size_prepended): a u32 uncompressed size, then an LZ4 block.
 * Host functions.  cf_lz4_decompress with dst NULL only reports the size. */
cf_status cf_lz4_compress(const uint8_t* src, uint64_t n, uint8_t* dst, uint64_t cap, uint64_t* out_len);
cf_status cf_lz4_decompress(const uint8_t* src, uint64_t n, uint8_t* dst, uint64_t cap, uint64_t* out_len);

/* --- display epilogue ------------------------------------------------------ */

/* The Res uniform of the resolve pass (shaders/resolve.wgsl:4-8). */
typedef struct cf_resolve_params {
    float scale;        /* R.a.x: input scale                          */
    float exposure_ev;  /* R.a.y: exposure in stops                    */
    float bloom;        /* R.a.z: bloom strength (0 = off)             */
    float grain;        /* R.a.w: film grain (0 = off)                 */
    float vignette;     /* R.b.x                                       */
    float sharpen;      /* R.c.x: (0 = off)                            */
    int32_t agx;        /* R.b.w >= 0.5: AgX tone map, else ACES       */
    int32_t reserved;
} cf_resolve_params;

/* The resolve fragment (shaders/resolve.wgsl:76-121: exposure, bloom,
 * sharpen, vignette, AgX / ACES, grain, sRGB) over the film's colour plane,
 * one pixel per cell, into rgba8_device (w x h x 4 bytes, device memory), on
 * `stream`.  The reference runs it on the renderer's HDR image; here the
 * film's linear RGB is the image (no graphics pipeline). */
cf_status cf_resolve(cf_film* film, const cf_resolve_params* params, void* rgba8_device, void* stream);

/* --- batches: many films stepped together -------------------------------- */

/* A batch steps many films (canvases of any size) with one kernel launch per
 * dispatch of encode_frame: each launch covers a table of every film's 16x16
 * tiles (films of different precision modes form separate launches).  It is
 * the reference's per-frame loop over films (App::encode_sim,
 * src/main.rs:1875-1909) for many canvases at once; each film's result is the
 * same as stepping it alone.  Films join and leave between steps; a film
 * belongs to at most one batch, and cf_destroy takes it out of its batch. */
typedef struct cf_batch cf_batch;

typedef struct cf_batch_tuning {
    uint32_t list_blocks_per_sm;  /* grid of the strata list kernels, blocks per SM (default 8) */
    uint32_t use_graph;           /* 1: frames replay a captured CUDA graph (default 1)       */
    uint32_t frames_per_graph;    /* frames captured in one graph launch (default 1)          */
    uint32_t tiles_per_block;     /* consecutive 16x16 tiles a block of the per-tile kernels
                                   * walks: 1 (default; 0 reads as 1), 2 or 4 (launch tiles of
                                   * 32x16 or 64x16 cells), up to 4096 (a grid of a few blocks
                                   * per SM walking the table: persistent)                    */
} cf_batch_tuning;

cf_status cf_batch_create(cf_batch** out);
cf_status cf_batch_destroy(cf_batch* batch);
cf_status cf_batch_add(cf_batch* batch, cf_film* film);
cf_status cf_batch_remove(cf_batch* batch, cf_film* film);
cf_status cf_batch_info(cf_batch* batch, uint32_t* films, uint64_t* cells, uint64_t* launches);
cf_status cf_batch_set_tuning(cf_batch* batch, const cf_batch_tuning* tuning);
cf_status cf_batch_get_tuning(cf_batch* batch, cf_batch_tuning* tuning);

/* `frames` frames of every film, on `stream`.  dt_max > 0: adaptive frames
 * (each film's dt chosen on the device, one substep, as cf_step_adaptive);
 * dt_max == 0: each film's params of its last cf_update_params, with
 * `substeps` substeps (as cf_encode_frame). */
cf_status cf_batch_step(cf_batch* batch, uint32_t frames, uint32_t substeps, float dt_max, void* stream);

/* Project autotuner: times candidate tunings (list-kernel grid, graph or
 * direct launches, frames per graph) on this batch, `frames_per_trial` frames
 * each after a warm-up, keeps the fastest and reports it with its time per
 * frame.  It steps the films (about 8 x (frames_per_trial + 2) frames):
 * callers that need the earlier state write it back afterwards. */
cf_status cf_batch_autotune(cf_batch* batch, uint32_t frames_per_trial, uint32_t substeps, float dt_max,
                            void* stream, cf_batch_tuning* best, float* best_ms_per_frame);

/* Human-readable text of the batch's last error. */
const char* cf_batch_last_error(const cf_batch* batch);

/* --- allocation-free CFL statistics -------------------------------------- */

/* Largest grid cf_cfl_stats_noalloc accepts, in 64 x 64 tiles (65,536 tiles:
 * 268M cells, e.g. 16384 x 16384).  Its scratch is one (h_max, mu_min) pair
 * per tile, 512 KB, held by every GPU that loads the library until exit. */
#define CF_NOALLOC_MAX_TILES 65536

/* No counterpart in the reference: it is an addition for callers that must
 * not allocate device memory when they ask for these numbers (a frame loop
 * that did all its allocation at start-up, where a cudaMalloc could stall
 * the device, or a host that owns a fixed memory budget).
 *
 * Computes, from caller-owned device planes h and mu (w x h FP32, row-major),
 * the same h_max and mu_min as the film's tile reduction (over cells with
 * h > 4 h_min; mu_min = 1 when no cell qualifies) and writes them to
 * d_out[0], d_out[1] (device memory) on `stream` (NULL = legacy default).
 * It allocates nothing: its scratch is a fixed array in the library's device
 * image.  The first call on each device (and again the first call after the
 * device's context was destroyed and created anew, e.g. by cudaDeviceReset)
 * looks up that array's address with the device current; make that first
 * call before any stream capture.  Every call on a device shares the one
 * array, and every call writes all the partials it reads, so nothing is
 * cleared between calls; calls that overlap on the GPU (different streams or
 * host threads, without ordering) race.  Grids of more than
 * CF_NOALLOC_MAX_TILES tiles, of any shape (one tile wide and 65,536 tall is
 * accepted), return CF_ERR_INVALID_ARG before anything is launched. */
cf_status cf_cfl_stats_noalloc(const float* d_h, const float* d_mu, uint32_t w, uint32_t h,
                               float h_min, float* d_out, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* CANVAZ_FILM_H */
