/*
 * vt_oracle.h -- CPU oracle for the voxel ray-traversal path.
 *
 * TEST INFRASTRUCTURE ONLY.  Nothing in the shipped library links or calls
 * this code; only tests/, __graft_entry__.smoke() and the cpu_baseline /
 * reference arm of bench.py load it, as the checker and as the timed CPU
 * baseline.  It restates the reference's traversal and shading on the CPU with
 * plain scalar C (no skipping, no SIMD), compiled with -ffp-contract=off so
 * that every float operation rounds exactly as written.
 *
 * Two traversals:
 *   mode P  plane-indexed Amanatides-Woo unit-step DDA over a dense uint8 grid,
 *           with the reference's tie-break chain (map.glsl:158), zero-direction
 *           fix (map.glsl:85-90), face numbering (map.glsl:119-127) and
 *           max-step loop (map.glsl:106).
 *   mode R  traceMap itself (map.glsl:83-168) over the reference's world format
 *           (64^3 chunk table, 8^3 u32 bricks, 256^3 RGBA8 model atlas).
 *
 * Pinning.  The reference ships no golden vectors for this path.  Mode R is
 * checked bit-for-bit against the reference's own map.glsl compiled as C++
 * (oracle/build_ref.py -> oracle/_ref), and mode P against that same compiled
 * traceMap on worlds of full 8^3 models, where both describe the same voxel
 * DDA (tests/test_oracle_ref.py).
 */
#ifndef VT_ORACLE_H
#define VT_ORACLE_H

#include <stdint.h>
#include <stddef.h>
#include "../include/vt.h"

#ifdef __cplusplus
extern "C" {
#endif

/* ------------------------------------------------------------ mode P world */
typedef struct {
    int32_t dims[3];
    const uint8_t* mats;  /* dense, x fastest */
    /* derived, owned by the oracle (vto_world_init / vto_world_free) */
    uint8_t* chunk_occ;   /* per 32^3 chunk */
    int32_t chunks[3];
    /* entity occluders of the shadow pass (vt_world_set_entities): n boxes
     * {lo x, y, z, hi x, y, z}; set by the caller after vto_world_init */
    const float* entities;
    int32_t n_entities;
} vto_world;

int32_t vto_world_init(vto_world* w, const int32_t dims[3], const uint8_t* mats);
void    vto_world_free(vto_world* w);

typedef struct {
    int32_t  hit;
    uint32_t voxel;      /* linear index or 0xFFFFFFFF */
    int32_t  cell[3];
    float    t;
    int32_t  face;       /* 0..5 or -1 */
    int32_t  axis;       /* axis of the entry crossing */
    uint8_t  material;
    int32_t  steps;      /* unit crossings made */
    uint64_t mask_words; /* brick words consulted */
    uint64_t coarse_words;
} vto_trace;

/* One mode-P ray, unit stepping. */
void vto_trace_p(const vto_world* w, const float o[3], const float d[3], int32_t max_steps, vto_trace* out);

/* The pick ray (terrain_edit.comp.glsl:11-17) on the mode-P world and the
 * voxel {x, y, z, valid} an edit with edit_mode writes. */
void vto_pick_p(const vto_world* w, const vt_camera* cam, int32_t max_steps, int32_t edit_mode, vto_trace* out,
                int32_t target[4]);

/* Shading + ray generation for pixel rows [y0, y1) of a frame. */
void vto_render_rows(const vto_world* w, const uint32_t* palette, const vt_camera* cam,
                     const vt_params* p, vt_hit* out, int32_t y0, int32_t y1, vt_stats* st);
/* Whole frame on `threads` POSIX threads (rows interleaved); st may be NULL. */
int32_t vto_render(const vto_world* w, const uint32_t* palette, const vt_camera* cam,
                   const vt_params* p, vt_hit* out, int32_t threads, vt_stats* st);
/* A bounded sample: every `row_step`-th row only (for the timed CPU baseline). */
int32_t vto_render_sampled(const vto_world* w, const uint32_t* palette, const vt_camera* cam,
                           const vt_params* p, vt_hit* out, int32_t threads, int32_t row_step,
                           vt_stats* st);

/* Explicit ray list (same semantics as vt_trace_rays). */
void vto_trace_rays(const vto_world* w, const float* origins, const float* dirs, int32_t n,
                    int32_t max_steps, vt_hit* out);

/* Lambert + shadowed-sun shading of one view and its exact gradient, in FP64,
 * over the primary hit records `hits` (from vto_render with primary rays):
 *     c = pal[m] * alb[v] * (ka + kd * max(0, n . s/|s|) * V),  L = sum (c - target)^2
 * V is read from vis_in (1 = lit) when not NULL, else traced from the hit with
 * the mode-P traversal (shadow origin as in the render path); vis_out, rgb,
 * g_pal (768), g_alb (X*Y*Z) may be NULL.  Gradients are added to the outputs.
 * a_pal, a_alb, a_sun (each NULL or shaped like its gradient) receive the sum
 * of the absolute values of the per-pixel contributions to each gradient
 * element: the scale of a float32 accumulation's rounding error in that
 * element, which a parity check uses as its absolute floor. */
int32_t vto_shade_grad_f64(const vto_world* w, const vt_camera* cam, const vt_hit* hits, const double* pal,
                           const double* alb, const double sun[3], double ka, double kd, int32_t shadow_max_steps,
                           const float* target, const uint8_t* vis_in, uint8_t* vis_out, double* rgb, double* loss,
                           double* g_pal, double* g_alb, double g_sun[3], double* a_pal, double* a_alb,
                           double a_sun[3]);

/* The deterministic sine/cosine used for bounce directions. */
float vto_sinf(float x);
float vto_cosf(float x);

/* ------------------------------------------------------------ mode R world */
typedef struct {
    const uint32_t* chunks; /* 64^3 entries, 0 = empty, else brick index + 1 */
    const uint32_t* data;   /* bricks, 512 u32 each (Voxel bits) */
    uint64_t        ndata;  /* number of u32 in data */
    const uint32_t* atlas;  /* 256^3 RGBA8 texels, x + 256*(y + 256*z) */
} vto_refworld;

typedef struct {
    uint32_t data;
    float    hit_pos[3];
    float    normal[3];
    int32_t  iterations;
} vto_refhit;

void vto_tracemap(const vto_refworld* w, const float o[3], const float d[3], int32_t max_steps, vto_refhit* out);

/* The reference's primary ray for pixel (px, py) of a W x H image
 * (primary.comp.glsl:31-43): camera = C_position, C_view (16 floats as the
 * host stores them, read column-major), fov; the ray is clipped to the 512^3
 * map box and traced with traceMap(..., max_steps). */
void vto_primary_r(const vto_refworld* w, const float cam_pos[4], const float view[16], float fov, int32_t px,
                   int32_t py, int32_t width, int32_t height, int32_t max_steps, float dir_out[3], vto_refhit* out);

/* The editing pass (terrain_edit.comp.glsl:11-24): pick (UV 0, 64 steps) and
 * map_setVoxel into `data` (the pool w->data points to, writable). */
void vto_edit_r(const vto_refworld* w, uint32_t* data, const float cam_pos[4], const float view[16],
                int32_t edit_mode, vto_refhit* out);

/* traceEntities (map.glsl:172-201, the part that runs: five unit boxes, the
 * sentinel 0xFFFFFFFF on a hit). */
void vto_trace_entities(const float o[3], const float d[3], float max_distance, vto_refhit* out);
/* SkyDome2 (camera.glsl:11-19) with pow as powf. */
void vto_sky_ref(const float rd[3], float out[4]);
/* One reference frame: primary.comp + secondary.comp + blit.fragment for
 * every pixel of a W x H image (records as vt_ref_pixel). */
void vto_render_reference(const vto_refworld* w, const float cam_pos[4], const float view[16], float fov,
                          int32_t width, int32_t height, vt_ref_pixel* out);

/* The primary rays of every row_step-th row of a frame (row-major), as the
 * render path makes them: origins and dirs get 3 floats per ray. */
void vto_primary_rays(const vt_camera* cam, int32_t row_step, float* origins, float* dirs);

/* ------------------------------------------------------ seeded scenes
 * vt_oracle_gen.c: the benchmark's synthetic scenes, the same bytes as the
 * library's host generator (vt_gen_*), for runs that must not load it. */
void    vto_gen_desc_init(vt_gen_desc* d, int32_t x, int32_t y, int32_t z, float scale, uint64_t seed);
int32_t vto_gen_world(const vt_gen_desc* d, uint8_t* out, size_t nbytes, int32_t threads);
int32_t vto_gen_height(const vt_gen_desc* d, int32_t x, int32_t z);
int32_t vto_camera_look(const float pos[3], float yaw, float pitch, float fov, int32_t width, int32_t height,
                        vt_camera* out);
int32_t vto_gen_camera(const vt_gen_desc* d, uint64_t seed, int32_t width, int32_t height, vt_camera* out);
void    vto_default_palette(uint32_t pal[256]);
void    vto_gen_sun(uint64_t seed, float out[3]);

#ifdef __cplusplus
}
#endif
#endif
