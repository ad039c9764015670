/*
 * vt.h -- C ABI of the GB300 voxel ray-traversal library (libvt.so).
 *
 * Plain C99: no CUDA, no C++ and no torch types appear in any signature, so the
 * header can be consumed unchanged by a C/C++ host, by Python ctypes, or by a
 * Zig host through @cImport("vt.h").
 *
 * The entry points replace the reference engine's render path, which in the
 * reference is a set of OpenGL objects driven from Zig:
 *
 *   world / chunk upload   src/engine/voxel.zig:25-82  (VoxelBrickmap init/set/get/clear/bind)
 *   model atlas            src/engine/voxel.zig:84-132 (VoxelModelAtlas)
 *   camera                 src/engine/graphics/camera.zig:5-44 (Camera, UniformData)
 *   render-frame           src/game.zig:232-256 (primary + secondary dispatch + blit)
 *   traversal              assets/shaders/map.glsl:83-168 (traceMap)
 *
 * Conventions
 *   - Every call returns vt_status (VT_OK == 0).  On failure a message is kept
 *     in the context and returned by vt_last_error_string().
 *   - Handles are opaque, owned by the library and released with *_destroy.
 *   - Calls that take a vt_stream are asynchronous on that stream (a
 *     cudaStream_t passed as void*, NULL = the legacy default stream).  Device
 *     pointers named d_* must be device memory of the context's device.
 *   - vt_sync() waits for a stream and surfaces the device status word that the
 *     checked kernels write (VT_ERR_DEVICE_OOB); vt_wait() is the same with a
 *     deadline (VT_ERR_TIMEOUT when the stream is still busy at the deadline).
 *   - One vt_ctx per host thread; the library holds no global mutable state
 *     besides CUDA's own and the fixed device array behind
 *     vt_render_host_static.
 */
#ifndef VT_H
#define VT_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define VT_ABI_VERSION 1

/* ------------------------------------------------------------------ status */
typedef int32_t vt_status;
#define VT_OK              0
#define VT_ERR_ARG         1  /* bad argument: null pointer, size out of range, bad handle */
#define VT_ERR_OOM         2  /* device or host allocation failed */
#define VT_ERR_CUDA        3  /* a CUDA runtime call failed (message has the CUDA error) */
#define VT_ERR_DEVICE_OOB  4  /* a checked kernel saw an out-of-range index */
#define VT_ERR_TIMEOUT     5  /* a bounded wait (vt_wait) ran out before the stream was done */
#define VT_ERR_NO_DEVICE   6  /* no CUDA device / driver */
#define VT_ERR_FORMAT      7  /* malformed input file (.vox) */
#define VT_ERR_STATE       8  /* call not valid in the object's current state */

typedef struct vt_ctx vt_ctx;
typedef struct vt_world vt_world;
typedef struct vt_brickmap vt_brickmap;
typedef struct vt_batch vt_batch;
typedef void* vt_stream; /* cudaStream_t */

/* ----------------------------------------------------------------- context */
int32_t     vt_abi_version(void);
const char* vt_status_string(vt_status s);
vt_status   vt_ctx_create(int32_t device, vt_ctx** out);
vt_status   vt_ctx_destroy(vt_ctx* ctx);
const char* vt_last_error_string(const vt_ctx* ctx);
/* Waits for `stream`, then reads and clears the context's device status word
 * (skipped while no checked or instrumented launch can have set it). */
vt_status   vt_sync(vt_ctx* ctx, vt_stream stream);
/* vt_sync with a deadline, for frame loops with a time budget (the reference
 * blocks in its GL fence without one, game.zig:249-256): polls `stream` for at
 * most timeout_us microseconds and returns VT_ERR_TIMEOUT if it is still busy
 * then.  The queued work is untouched and keeps running; the caller may wait
 * again.  Once the stream is done it behaves as vt_sync. */
vt_status   vt_wait(vt_ctx* ctx, vt_stream stream, int64_t timeout_us);
/* Device name and SM count of the context's device. */
vt_status   vt_device_info(vt_ctx* ctx, char* name, int32_t name_len, int32_t* sm_count);

/* Device memory helpers, so that hosts without another CUDA binding (C, Zig,
 * ctypes) can own frame buffers.  Thin wrappers over the CUDA runtime. */
vt_status vt_device_alloc(vt_ctx* ctx, size_t nbytes, void** d_ptr);
vt_status vt_device_free(vt_ctx* ctx, void* d_ptr);
vt_status vt_host_alloc_pinned(vt_ctx* ctx, size_t nbytes, void** h_ptr);
vt_status vt_host_free_pinned(vt_ctx* ctx, void* h_ptr);
vt_status vt_memcpy_h2d(vt_ctx* ctx, void* d_dst, const void* h_src, size_t nbytes, vt_stream stream);
vt_status vt_memcpy_d2h(vt_ctx* ctx, void* h_dst, const void* d_src, size_t nbytes, vt_stream stream);
vt_status vt_memset_d(vt_ctx* ctx, void* d_dst, int32_t value, size_t nbytes, vt_stream stream);
vt_status vt_stream_create(vt_ctx* ctx, vt_stream* out);
vt_status vt_stream_destroy(vt_ctx* ctx, vt_stream stream);

/* Testing hooks for the allocation-failure paths (no counterpart in the
 * reference, whose block allocator panics when it cannot grow,
 * src/engine/graphics/gpu_block_allocator.zig:22).  Every device and pinned
 * host allocation the library makes goes through one wrapper:
 *   vt_debug_fail_alloc(n)   the n-th next allocation (n >= 1) fails as if the
 *                            device were out of memory, then the hook disarms;
 *                            n = 0 disarms it.  Process-wide.
 *   vt_debug_alloc_counts    allocations made so far, and those still live
 *                            (made minus freed), process-wide. */
void vt_debug_fail_alloc(int64_t n);
void vt_debug_alloc_counts(uint64_t* made, int64_t* live);

/* ------------------------------------------------------------------- world
 * Mode-P world: a dense grid of uint8 materials (0 = air), stored on the device
 * as 32^3 chunks.  Each chunk holds 8^3 bricks of 4^3 voxels; a brick has one
 * 64-bit occupancy word (bit = x + 4y + 16z within the brick) and 64 material
 * bytes; a chunk has one coarse occupancy bit.  Host-side layout of every
 * dense buffer handed to the library: x fastest, then y, then z
 * (index = x + X*(y + Y*z)), i.e. the reference's posToIndex order
 * (src/engine/voxel.zig:21-23).
 */
typedef struct {
    int32_t dims[3]; /* X, Y, Z in voxels, each in [1, 8192], X*Y*Z < 2^32 */
} vt_world_desc;

typedef struct {
    int32_t  dims[3];
    int32_t  chunks[3];        /* chunk counts per axis (dims rounded up to 32) */
    uint64_t mask_bytes;       /* brick occupancy words */
    uint64_t material_bytes;   /* chunk-ordered material bytes */
    uint64_t coarse_bytes;     /* per-chunk occupancy bits */
    const void* d_mask;        /* device pointers, for inspection */
    const void* d_materials;
    const void* d_coarse;
} vt_world_info;

/* VoxelBrickmap.init (voxel.zig:32-39): an empty world.  Device memory per
 * 4^3 brick of the chunk-padded grid: 64 B materials, 8 B occupancy word,
 * 8 B brick distances (one per direction octant) and 72 B kept for their
 * incremental update, about 2.4 B per voxel in all (the 512x256x512 world
 * takes 152 MiB, a 2048x256x2048 one 2.4 GiB). */
vt_status vt_world_create(vt_ctx* ctx, const vt_world_desc* desc, vt_world** out);
vt_status vt_world_destroy(vt_world* world);
/* VoxelBrickmap.clear (voxel.zig:41-44). */
vt_status vt_world_clear(vt_world* world, vt_stream stream);
/* Bulk upload of the whole grid (X*Y*Z bytes, host memory); rebuilds every
 * brick word and chunk bit on the device.  Replaces the procgen -> set loop
 * writing into the persistently mapped SSBOs (voxel.zig:58-61). */
vt_status vt_world_upload_dense(vt_world* world, const uint8_t* h_materials, size_t nbytes, vt_stream stream);
/* Upload one 32^3 chunk (32768 bytes, x fastest, cells outside dims ignored). */
vt_status vt_world_upload_chunk(vt_world* world, int32_t cx, int32_t cy, int32_t cz,
                                const uint8_t* h_chunk, vt_stream stream);
/* VoxelBrickmap.set / get (voxel.zig:58-70): single voxel write/read. */
vt_status vt_world_set_voxel(vt_world* world, int32_t x, int32_t y, int32_t z, uint8_t material, vt_stream stream);
vt_status vt_world_get_voxel(vt_world* world, int32_t x, int32_t y, int32_t z, uint8_t* material);
/* VoxelBrickmap.get (voxel.zig:63-70) over the whole grid: X*Y*Z bytes, x
 * fastest, into host memory; returns after the copy has landed. */
vt_status vt_world_download_dense(vt_world* world, uint8_t* h_materials, size_t nbytes, vt_stream stream);
/* 256-entry RGBA8 palette (R in the low byte): albedo of each material in the
 * REFERENCE shading mode (the role of the model atlas texel, map.glsl:57-60). */
vt_status vt_world_set_palette(vt_world* world, const uint32_t* h_rgba256);
vt_status vt_world_get_info(const vt_world* world, vt_world_info* info);
/* Entity occluders of the shadow pass (traceEntities, map.glsl:172-201, as
 * used by secondary.comp.glsl:42-46, which tests five hard-coded unit boxes):
 * n <= 1024 axis-aligned boxes {lo x, y, z, hi x, y, z} in voxel units.  A
 * shadow ray clear of voxels that meets a box (t >= 0) shades its pixel as
 * shadowed and sets VT_HIT_ENTITY.  Synchronous; takes effect for work queued
 * afterwards (do not call while a render of this world is in flight).  n = 0
 * removes them. */
vt_status vt_world_set_entities(vt_world* world, const float* h_boxes, int32_t n);

/* ------------------------------------------------------------------ camera
 * Mirrors Camera.UniformData (camera.zig:12-16, camera.glsl:2-6) plus the
 * target size.  view is row-major as the host math library stores it; with the
 * shader reading it column-major, a ray's direction is the row vector
 * (u, v, 1, 1) * view (primary.comp.glsl:39). */
typedef struct {
    float   pos[4];       /* ray origin in voxel units (w ignored) */
    float   view[16];     /* row-major 4x4 */
    float   fov;          /* field of view across the image width, radians */
    float   tan_half_fov; /* tan(fov/2), computed by the host (primary.comp.glsl:36) */
    int32_t width;
    int32_t height;
} vt_camera;

/* Camera.set_pos + Camera.rotate + as_uniform_data (camera.zig:18-43) with an
 * explicit convention: forward = (cos p sin y, sin p, cos p cos y), so a
 * negative pitch looks down; rows of view are right, up, forward, (0,0,0,1). */
vt_status vt_camera_look(const float pos[3], float yaw, float pitch, float fov,
                         int32_t width, int32_t height, vt_camera* out);

/* ---------------------------------------------------------------- render */
#define VT_RAYS_PRIMARY 1u
#define VT_RAYS_SHADOW  2u
#define VT_RAYS_BOUNCE  4u

#define VT_SHADE_NONE      0u /* rgba = palette albedo on hit, 0 on miss */
#define VT_SHADE_REFERENCE 1u /* primary + secondary + blit arithmetic of the reference */
#define VT_SHADE_LAMBERT   2u /* palette * albedo * (ambient + diffuse * max(0, n.s) * V) */

#define VT_FLAG_CROSSHAIR 1u  /* blit.fragment.glsl:33 */
#define VT_FLAG_VIGNETTE  2u  /* blit.fragment.glsl:15-21,34-35 */
#define VT_FLAG_CHECKED   4u  /* run the bounds-checked kernel variant */

typedef struct {
    int32_t  max_steps;         /* unit-voxel crossings a primary ray may make, +1 (map.glsl:106) */
    int32_t  shadow_max_steps;
    int32_t  bounce_max_steps;
    uint32_t rays;              /* VT_RAYS_* */
    uint32_t shade;             /* VT_SHADE_* */
    uint32_t flags;             /* VT_FLAG_* */
    uint32_t seed;              /* xor-ed into the per-pixel bounce seed */
    float    sun_dir[3];        /* shadow ray direction, used as given (camera.glsl:8) */
    float    ambient;           /* LAMBERT k_a */
    float    diffuse;           /* LAMBERT k_d */
    float    bounce_weight;     /* weight of the bounce sky term */
} vt_params;

/* One record per pixel, 16 bytes. */
typedef struct {
    uint32_t voxel;    /* x + X*(y + Y*z) of the hit voxel, 0xFFFFFFFF on miss */
    float    t;        /* entry distance of the hit voxel along the ray, -1 on miss */
    uint32_t rgba;     /* shaded colour, RGBA8, R in the low byte */
    uint8_t  face;     /* 2*axis + (dir[axis] > 0 ? 0 : 1); 0xFF on miss */
    uint8_t  material; /* material of the hit voxel, 0 on miss */
    uint8_t  flags;    /* VT_HIT_* */
    uint8_t  pad;
} vt_hit;

#define VT_HIT_PRIMARY   1u /* primary ray hit a voxel */
#define VT_HIT_SHADOWED  2u /* shadow ray hit a voxel */
#define VT_HIT_BOUNCE    4u /* bounce ray hit a voxel */
#define VT_HIT_ENTITY    8u /* shadow ray clear of voxels but met an entity box: shaded as shadowed */

void vt_params_default(vt_params* p);

/* Game.render (game.zig:232-256): primary rays, optional shadow and bounce
 * rays and the shading of primary.comp + secondary.comp + blit.fragment, fused
 * into one launch.  d_out holds width*height records, row-major, row 0 at
 * v = -1 (bottom of the image, as the GL image is addressed).
 * The first frame of a new image size and field of view in a context makes
 * that frame's table of per-column and per-row screen coordinates (one small
 * device allocation and one synchronisation of `stream`; up to 8 tables per
 * context, none inside a graph capture). */
vt_status vt_render(vt_ctx* ctx, const vt_world* world, const vt_camera* cam,
                    const vt_params* params, vt_hit* d_out, vt_stream stream);
/* Same, with host output, synchronous.  Into pinned memory (vt_host_alloc_
 * pinned) the kernel writes the records directly over the host link; into
 * pageable memory frames of >= 2^18 pixels render as 16 row bands on four
 * streams, each band copied back as soon as it is done. */
vt_status vt_render_host(vt_ctx* ctx, const vt_world* world, const vt_camera* cam,
                         const vt_params* params, vt_hit* h_out);

/* No counterpart in the reference.  vt_render_host for callers that cannot
 * allocate device memory: hosts that hand out all device memory through
 * their own allocator and forbid other allocations, and real-time frame loops
 * that must not call cudaMalloc once running (it can synchronize the device).
 * vt_render_host stages the records in a buffer the context allocates on
 * first use; this call stages them in a fixed device array compiled into the
 * library (VT_STATIC_MAX_PIXELS records, 4 MiB per device) and allocates
 * nothing.  It traces bounce rays inline (no deferred queue) and makes no
 * screen table (it uses one made earlier for the same image size, else the
 * kernel's per-block coordinates).
 *   - Frames larger than VT_STATIC_MAX_PIXELS pixels are rejected (VT_ERR_ARG).
 *   - The array is placed on a device when the first context for that device
 *     is created: vt_ctx_create looks its device address up
 *     (cudaGetSymbolAddress, with that device current), which is when CUDA's
 *     lazy module loading loads it.  It stays until the process exits.  This
 *     call therefore neither loads a module nor allocates.
 *   - All calls share the one array: calls whose work overlaps on the GPU
 *     (several host threads, several contexts) race on it. */
#define VT_STATIC_MAX_PIXELS 262144
vt_status vt_render_host_static(vt_ctx* ctx, const vt_world* world, const vt_camera* cam,
                                const vt_params* params, vt_hit* h_out);

/* Counters of one render, from an instrumented kernel variant.  The byte
 * counts are algorithmic: 8 per brick word and per coarse word consulted,
 * 1 per material byte read on a hit, 16 per record stored. */
typedef struct {
    uint64_t primary_rays;
    uint64_t primary_hits;
    uint64_t shadow_rays;
    uint64_t shadow_hits;
    uint64_t bounce_rays;
    uint64_t bounce_hits;
    uint64_t mask_words;
    uint64_t coarse_words;
    uint64_t material_bytes;
    uint64_t record_bytes;
    uint64_t steps;          /* unit-voxel crossings, all rays */
    uint64_t iterations;     /* traversal loop iterations, all rays */
} vt_stats;
vt_status vt_render_stats(vt_ctx* ctx, const vt_world* world, const vt_camera* cam,
                          const vt_params* params, vt_stats* out, vt_stream stream);

/* -------------------------------------------------------------- mode R
 * The reference's own world format and frame, on the GPU, bit for bit:
 *   map     64^3 table of brick indices (0 = empty, else brick + 1), index
 *           x + 64*(y + 64*z) (voxel.zig:21-23); bricks of 8^3 u32 voxels
 *           {ty:28, is_solid:1} indexed x + 8*y + 64*z (voxel.zig:58-61);
 *           a 512^3 voxel map (MAP_DIMENSION, map.glsl:2)
 *   atlas   8^3 RGBA8 models; model ty sits at ((ty&31)*8, (ty>>5&31)*8,
 *           (ty>>10&31)*8) of a 256^3 image (voxel.zig:94-112, map.glsl:57-60)
 *   frame   primary.comp.glsl (traceMap, 192 steps) -> G-buffer;
 *           secondary.comp.glsl (traceMap toward SUN_DIR, 48 steps, plus
 *           traceEntities) -> illumination; blit.fragment.glsl -> colour. */
typedef struct {
    uint32_t albedo;       /* frameColor, RGBA8 */
    uint32_t normal;       /* frameNormal, RGBA8 (negative components store as 0) */
    uint32_t illumination; /* frameIllumination, RGBA8 */
    uint32_t color;        /* blit output, RGBA8 */
    float    position[4];  /* framePosition, RGBA32F */
} vt_ref_pixel;            /* 32 bytes */

typedef struct {
    uint32_t data;         /* HitInfo.data: RGBA8 of the hit sub-voxel, 0 on a miss */
    float    hit_pos[3];   /* sub-voxel position, -1 on a miss */
    float    normal[3];
    int32_t  pad;
} vt_ref_hit;              /* 32 bytes */

/* VoxelBrickmap(512, 8).init + VoxelModelAtlas.init: an empty map and atlas. */
vt_status vt_brickmap_create(vt_ctx* ctx, vt_brickmap** out);
vt_status vt_brickmap_destroy(vt_brickmap* bm);
/* The whole map: h_chunks (64^3 u32) and h_bricks (nbricks * 512 u32). */
vt_status vt_brickmap_upload(vt_brickmap* bm, const uint32_t* h_chunks, const uint32_t* h_bricks, size_t nbricks);
/* One 8^3 model (512 RGBA8 texels, x + 8*(y + 8*z)) into atlas slot `slot`. */
vt_status vt_brickmap_set_model(vt_brickmap* bm, int32_t slot, const uint32_t* h_texels);
/* VoxelModelAtlas.load_block_model (voxel.zig:94-127): parses a MagicaVoxel
 * file from memory and appends its models at the next free slots (the file's
 * y and z axes swapped, colours from its RGBA chunk).  *models_loaded gets
 * the count. */
vt_status vt_brickmap_load_vox(vt_brickmap* bm, const uint8_t* h_bytes, size_t nbytes, int32_t* models_loaded);
/* The same parse into host memory (no device needed): up to max_models
 * models of 512 texels each into h_texels; *models gets the file's count. */
vt_status vt_vox_decode(const uint8_t* h_bytes, size_t nbytes, uint32_t* h_texels, int32_t max_models,
                        int32_t* models);
/* traceMap (map.glsl:83-168) over an explicit ray list (origins in world
 * units, n*3 floats each). */
vt_status vt_trace_map(vt_ctx* ctx, const vt_brickmap* bm, const float* d_origins, const float* d_dirs, int32_t n,
                       int32_t max_steps, vt_ref_hit* d_out, vt_stream stream);
/* One reference frame (game.zig:232-256) for a camera: cam.pos, cam.view (the
 * uniform's matrix) and cam.fov as the reference's UniformData; width*height
 * vt_ref_pixel records on the device.  Rows are the GL image's rows. */
vt_status vt_render_reference(vt_ctx* ctx, const vt_brickmap* bm, const vt_camera* cam, vt_ref_pixel* d_out,
                              vt_stream stream);
/* procgen (src/procgen.zig:6-70) into the reference's world format: the
 * stone floor, the heightfield columns, grass, flowers and trees, every
 * choice drawn from util.LCG (seed 0x46AE4F, util.zig:33-45) in the
 * reference's order, bricks allocated in order of first touch as
 * VoxelBrickmap(dim, 8).set does (voxel.zig:47-61).  h_chunks receives the
 * (dim/8)^3 table, h_bricks up to brick_capacity bricks of 512 u32, *nbricks
 * the count used (VT_ERR_OOM when it exceeds the capacity: call again with
 * more).  The heightfield noise (FastNoiseLite fbm in the reference, not part
 * of its sources) comes from h_noise[x*dim + z] when given, else from the
 * library's seeded value-noise fbm at ((offset + x)/10, (offset + z)/10). */
vt_status vt_procgen_reference(int32_t dim, float offset_x, float offset_z, const float* h_noise, uint64_t noise_seed,
                               uint32_t* h_chunks, uint32_t* h_bricks, size_t brick_capacity, size_t* nbricks);
/* VoxelBrickmap.get over the whole map (voxel.zig:63-70): the chunk table
 * (64^3 u32) and the first nbricks bricks (512 u32 each) back to the host,
 * after all work queued on the device. */
vt_status vt_brickmap_download(vt_brickmap* bm, uint32_t* h_chunks, uint32_t* h_bricks, size_t nbricks);
/* The editing pass (terrain_edit.comp.glsl:11-24): the pick ray through the
 * view centre traced with 64 steps, then, on a hit, edit_mode > 0 writes
 * Voxel{ty = edit_mode - 1, is_solid = 1} into the voxel in front of the hit
 * face and edit_mode == 0 clears the hit voxel, through map_setVoxel
 * (map.glsl:49-55: dropped where the chunk has no brick).  edit_mode == -1
 * only picks.  d_out (NULL allowed): one vt_ref_hit.  Asynchronous. */
vt_status vt_brickmap_edit(vt_ctx* ctx, vt_brickmap* bm, const vt_camera* cam, int32_t edit_mode, vt_ref_hit* d_out,
                           vt_stream stream);

/* ----------------------------------------------------------------- batch
 * Many scenes x cameras in one graph launch (no counterpart in the reference,
 * which renders one camera per frame, game.zig:232-256).  Under the default
 * tuning (VT_KERNEL_TILE) the graph holds one render launch per world (its
 * consecutive jobs, up to 256), whose grid covers the 16x16-pixel tiles of
 * all those jobs (the job table travels as the launch's parameters); under
 * VT_KERNEL_PER_JOB it holds one render launch per job on eight concurrent
 * chains; under VT_KERNEL_QUEUE one persistent kernel that pulls 16x16-pixel
 * units of all jobs from a device work queue.  Every job's records are
 * identical to what vt_render writes for it alone. */
typedef struct {
    const vt_world* world;
    vt_camera camera;
    vt_hit* d_out;     /* camera.width * camera.height records */
} vt_job;

/* Uploads the job table and sizes the launch.  The batch is replayed with
 * vt_batch_launch, which captures a CUDA graph on its first call (with the
 * context's tuning at that moment) and launches that graph on the given
 * stream every time. */
vt_status vt_batch_create(vt_ctx* ctx, const vt_job* jobs, int32_t n, const vt_params* params, vt_batch** out);
vt_status vt_batch_launch(vt_batch* batch, vt_stream stream);
vt_status vt_batch_destroy(vt_batch* batch);
/* Pixels (= primary rays), jobs and 16x16 work units of one launch. */
vt_status vt_batch_info(const vt_batch* batch, uint64_t* pixels, int32_t* jobs, uint32_t* units);
/* Times the batch in each launch shape (VT_KERNEL_TILE: one launch per world;
 * VT_KERNEL_PER_JOB: one launch per job; VT_KERNEL_QUEUE: one persistent
 * kernel), reps graph launches each on the context's stream (synchronous),
 * and keeps the fastest for this batch's later launches.  Every shape gives
 * identical records.  No counterpart in the reference. */
vt_status vt_batch_autotune(vt_batch* batch, int32_t reps, int32_t* best_shape, float* best_ms);

/* ------------------------------------------------------- shading adjoint
 * No counterpart in the reference (its shading is fixed-function,
 * blit.fragment.glsl:31).  Lambert + shadowed sun over the primary hits of a
 * frame, with the hit set held fixed (the discrete traversal is never
 * relaxed):
 *     c = palette[m] * albedo[v] * (ambient + diffuse * max(0, n . s/|s|) * V)
 * m, v, n from the primary hit record, V = 1 unless the shadow ray from the
 * hit toward s (traced exactly as vt_render traces it) hits a voxel; c = 0 on
 * a miss.  Loss L = sum over pixels and channels of (c - target)^2. */
typedef struct {
    const float* d_palette;  /* 256 x 3 FP32 RGB */
    const float* d_albedo;   /* X*Y*Z FP32 per-voxel scale (index x + X*(y + Y*z)), or NULL for 1 */
    float sun[3];            /* sun direction (any length) */
    float ambient;
    float diffuse;
    int32_t shadow_max_steps;
} vt_shade_inputs;

/* Forward shading: d_rgb gets width*height*3 floats.  d_hits are the records
 * of vt_render for the same camera.  With d_vis_in != NULL the shadow term is
 * read from it (one byte per pixel, 1 = lit) instead of traced; d_vis_out,
 * if not NULL, receives the traced one. */
vt_status vt_shade_forward(vt_ctx* ctx, const vt_world* world, const vt_camera* cam, const vt_hit* d_hits,
                           const vt_shade_inputs* in, const uint8_t* d_vis_in, uint8_t* d_vis_out, float* d_rgb,
                           vt_stream stream);
/* Fused forward + backward of the loss: recomputes the shading (shadow rays
 * traced again, not stored), adds the loss to *d_loss and the gradients to
 * d_grad_palette (256 x 3), d_grad_albedo (X*Y*Z, may be NULL) and
 * d_grad_sun (3).  The caller owns and zeroes these accumulators.  Gradients
 * are accumulated with float atomics, so their last bits depend on the order
 * in which blocks finish. */
vt_status vt_shade_backward(vt_ctx* ctx, const vt_world* world, const vt_camera* cam, const vt_hit* d_hits,
                            const vt_shade_inputs* in, const float* d_target, float* d_loss, float* d_grad_palette,
                            float* d_grad_albedo, float* d_grad_sun, vt_stream stream);
/* vt_shade_forward over n views (cameras, hit records, output images; the
 * shadow term traced), as one call: up to 16 views share one launch on
 * `stream`; views may differ in size. */
vt_status vt_shade_forward_views(vt_ctx* ctx, const vt_world* world, int32_t n, const vt_camera* cams,
                                 const vt_hit* const* d_hits, const vt_shade_inputs* in, float* const* d_rgb,
                                 vt_stream stream);
/* vt_shade_backward over n views (cameras, hit records, targets) into the
 * same accumulators, as one call: up to 16 views share one launch on
 * `stream`; views may differ in size. */
vt_status vt_shade_backward_views(vt_ctx* ctx, const vt_world* world, int32_t n, const vt_camera* cams,
                                  const vt_hit* const* d_hits, const vt_shade_inputs* in, const float* const* d_targets,
                                  float* d_loss, float* d_grad_palette, float* d_grad_albedo, float* d_grad_sun,
                                  vt_stream stream);

/* ------------------------------------------------------------------ tuning
 * Launch configuration of the render kernels (no counterpart in the
 * reference, whose dispatch shape is fixed at 32x32 groups, game.zig:241-248).
 * Every configuration produces identical records; only speed differs. */
#define VT_KERNEL_TILE    0 /* one thread per pixel, warp = pixel tile; a batch: one launch per chunk of jobs */
#define VT_KERNEL_QUEUE   1 /* persistent warps refilling lanes from a pixel queue */
#define VT_KERNEL_PER_JOB 2 /* as VT_KERNEL_TILE for single frames; a batch: one launch per job */
typedef struct {
    int32_t kernel;        /* VT_KERNEL_* */
    int32_t warp_tile_w;   /* VT_KERNEL_TILE: a warp's tile is w x (32/w) pixels, w in {4, 8, 16, 32} */
    int32_t occupancy;     /* VT_KERNEL_TILE: 1 = register budget capped for 4 blocks (32 warps) per SM */
    int32_t batch;         /* VT_KERNEL_QUEUE: parked lanes (1..32) that trigger a refill pass */
    int32_t share_bricks;  /* VT_KERNEL_TILE with w = 8 and the cap: 1 = lanes of a warp that look up the
                              same brick word share one load (__match_any_sync + __shfl_sync) */
    int32_t l2_persist;    /* 1 = render launches carry an L2 access-policy window over the world's brick
                              words (persisting, as much as the device's persisting L2 holds) */
    int32_t bounce_refill; /* deferred bounce rays: idle lanes (1..32) that make a warp refill; 0 = 8 */
    int32_t bounce_walk;   /* deferred bounce rays: 0 = brick-run walk (unit steps of an occupied brick
                              in an inner loop), 1 = one advance per turn for jumps and unit steps alike */
    int32_t bounce_sort;   /* deferred bounce rays: 1 = each 16x16-pixel block of the frame kernel appends
                              its rays sorted by direction (8x4 capped tiles without share_bricks; other
                              shapes append in order) */
} vt_tuning;
vt_status vt_set_tuning(vt_ctx* ctx, const vt_tuning* tuning);
vt_status vt_get_tuning(vt_ctx* ctx, vt_tuning* tuning);
/* Times every candidate configuration on this frame (reps launches each,
 * CUDA events on the context's stream), keeps the fastest in the context and
 * returns it with its mean time in ms.  With a non-NULL cache_path the choice
 * is looked up first and recorded afterwards in that text file, keyed by GPU
 * name, world size, image size and ray kinds. */
vt_status vt_autotune(vt_ctx* ctx, const vt_world* world, const vt_camera* cam, const vt_params* params,
                      int32_t reps, const char* cache_path, vt_tuning* best, float* best_ms);

/* No counterpart in the reference: a measurement aid for roofline
 * denominators.  Streams a device buffer of `bytes` (allocated and freed by
 * this call) `passes` times in one launch of a read kernel with 16-byte
 * L2-only loads; *gbs = bytes * passes / that launch's time (CUDA events on
 * the context's stream, after one warm-up launch).  A buffer that fits in L2
 * (a few tens of MiB on GB300) gives the L2 read bandwidth; one far larger
 * than L2 the HBM read bandwidth.  Synchronous. */
vt_status vt_probe_read_bandwidth(vt_ctx* ctx, uint64_t bytes, int32_t passes, float* gbs);

/* traceMap over an explicit ray list (map.glsl:83-168 semantics on the mode-P
 * world, no clipping beyond the grid box): d_origins/d_dirs are n*3 floats. */
vt_status vt_trace_rays(vt_ctx* ctx, const vt_world* world, const float* d_origins,
                        const float* d_dirs, int32_t n, int32_t max_steps,
                        vt_hit* d_out, vt_stream stream);

/* ------------------------------------------------------------ pick / edit
 * The pick ray of terrain_edit.comp.glsl:11-17 on the mode-P world: the
 * camera's ray of UV (0, 0), i.e. the primary ray of pixel (W/2, H/2) for
 * even W and H, traced with max_steps.  vt_pick returns its hit record to the
 * host (synchronous, on the context's stream). */
vt_status vt_pick(vt_ctx* ctx, vt_world* world, const vt_camera* cam, int32_t max_steps, vt_hit* h_out);
/* Pick and edit in one launch, nothing read back (terrain_edit.comp.glsl:
 * 19-24 on the mode-P world): on a hit, edit_mode 0 clears the hit voxel and
 * edit_mode 1..255 writes that material into the voxel in front of the hit
 * face (skipped outside the world); -1 only picks.  The brick word, chunk bit
 * and the empty-space distances around the voxel are updated on `stream`.
 * d_out (NULL allowed) receives the pick's vt_hit.  Edits on one world are
 * serialised by the caller (one stream per world). */
vt_status vt_edit(vt_ctx* ctx, vt_world* world, const vt_camera* cam, int32_t max_steps, int32_t edit_mode,
                  vt_hit* d_out, vt_stream stream);
/* The empty-space distances the traversal skips by (brought up to date
 * first), one field per direction octant o (bit i of o set: towards +i):
 * h_brick gets 8 fields of nchunks*512 bytes (chunk-major, brick bx + 8*(by
 * + 8*bz)), h_chunk 8 fields of nchunks bytes.  Entry of octant o: 0 if
 * occupied; for a chunk, min over occupied chunks ahead in that octant of
 * max(|dx|, |dy|, |dz|), capped at 16; for a brick, s | shape << 6 where s is
 * the min over occupied voxels ahead of max(dx, w*dy, dz), d_i counting the
 * voxel layers between the brick's far face and the voxel (0 within the
 * brick's extent), w = 2^shape, capped at 63: shape 0 for the octants moving
 * +y, and for those moving -y the shape 0..3 whose box (4 + s - 1 voxels
 * across, 4 + ((s - 1) >> shape) vertically) has the largest volume, the
 * smallest shape on a tie.  For tests and tools. */
vt_status vt_world_download_distances(vt_world* world, uint8_t* h_brick, size_t brick_bytes, uint8_t* h_chunk,
                                      size_t chunk_bytes);

/* ------------------------------------------------------------- generators
 * Seeded synthetic scenes (host code, deterministic across machines). */
typedef struct {
    int32_t  dims[3];
    float    base_height;    /* terrain height = base + amplitude * fbm, fbm in [-1, 1] */
    float    amplitude;
    float    period;         /* wavelength of the first octave (base frequency 1/period) */
    float    water_level;    /* air cells with y < water_level above the terrain become water */
    float    camera_height;  /* cameras sit this far above the terrain or water */
    int32_t  octaves;        /* lacunarity 2, gain 0.5 */
    int32_t  trees;          /* trees to plant: trunk 1x6x1 (material 5), 5^3 leaves (6) kept w.p. 0.7 */
    int32_t  caves;          /* 1 = remove solid cells where 3D value-noise fbm > cave_threshold */
    float    cave_threshold;
    float    cave_period;
    uint64_t seed;
} vt_gen_desc;
/* Defaults of the plain terrain generator scaled by `scale` (1.0: base 64,
 * amplitude 24, period 64, water 56, camera 10 voxels up, 4 octaves). */
void      vt_gen_desc_init(vt_gen_desc* desc, int32_t x, int32_t y, int32_t z, float scale, uint64_t seed);
/* Fills h_out (X*Y*Z bytes, x fastest) on `threads` host threads. */
vt_status vt_gen_world(const vt_gen_desc* desc, uint8_t* h_out, size_t nbytes, int32_t threads);
/* Terrain height at column (x, z): cells y < height are solid before caves. */
int32_t   vt_gen_height(const vt_gen_desc* desc, int32_t x, int32_t z);
/* The same scene generated on the device straight into `world` (whose dims
 * must equal desc->dims): the bytes equal vt_gen_world's.  Replaces the
 * host procgen loop (procgen.zig:6-53) and the upload; asynchronous on
 * `stream`. */
vt_status vt_world_generate(vt_world* world, const vt_gen_desc* desc, vt_stream stream);
/* A seeded pinhole camera camera_height above the terrain at a seeded column,
 * seeded yaw in [0, 360) degrees and pitch in [-30, 0] degrees, FOV 70 deg. */
vt_status vt_gen_camera(const vt_gen_desc* desc, uint64_t seed, int32_t width, int32_t height, vt_camera* out);
/* The default palette (material 0 transparent). */
vt_status vt_default_palette(uint32_t* h_rgba256);
/* A seeded sun direction (upper hemisphere). */
vt_status vt_gen_sun(uint64_t seed, float out[3]);

#ifdef __cplusplus
}
#endif
#endif /* VT_H */
