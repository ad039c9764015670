// render.cu -- the fused render-frame kernel (primary + shadow + bounce rays
// and shading in one launch) and its C-ABI entry points.
//
// Replaces the reference's per-frame work: the primary dispatch
// (primary.comp.glsl:23-69), the secondary dispatch (secondary.comp.glsl:18-51)
// and the composite (blit.fragment.glsl:23-36), which the reference runs as two
// compute passes with a G-buffer round trip and a raster pass
// (game.zig:232-256).  Here one thread follows its pixel's primary ray, then
// the shadow ray (and bounce ray) from the hit, shades, and stores one 16-byte
// record; nothing goes through memory between the passes.
#include <cstring>

#include "launch.cuh"
#include "render_pixel.cuh"

namespace vt {

// 256-thread blocks; each warp traces a compact pixel tile so that its rays
// start close together and share brick words in L1.
constexpr int kBlock = 256;  // 128 measured the same with the register cap
constexpr size_t kMaxSharedCoarse = 48 * 1024;

template <bool STATS>
__device__ __forceinline__ void flush_counters(PixelCounters& pc, unsigned long long* counters) {
    if (!STATS) return;
#pragma unroll
    for (int k = 0; k < kNumCounters; ++k) {
        const unsigned s = __reduce_add_sync(0xFFFFFFFFu, pc.v[k]);
        if ((threadIdx.x & 31) == 0 && s) atomicAdd(counters + k, (unsigned long long)s);
    }
}

// One thread per pixel.  A warp covers a TW x (32 / TW) pixel tile; the
// 256-thread block covers max(16, TW) pixels across.  OCC caps the register
// budget so that kOccBlocks blocks fit on an SM: 4 blocks (64 registers, 32
// warps, no spills) measured 4% faster on a 1080p frame than 5 (48 registers
// with spills) and 3 (uncapped, 67 registers).
constexpr int kOccBlocks = 4 * 256 / kBlock;
template <int TW>
struct BlockTile {
    static constexpr int kW = TW < 16 ? 16 : TW;     // block tile width
    static constexpr int kWarpsX = kW / TW;
    static constexpr int kH = (kBlock / 32 / kWarpsX) * (32 / TW);
    static_assert(kW <= 64 && kH <= kBlock - 64, "the column and row tables are filled by distinct threads");
};

// SHARE: the lanes of a warp that look up the same brick word share one load
// (Walker::brick_word).  BIN: deferred bounce rays are appended per block,
// sorted by direction (stage_flush).
template <bool STATS, bool CHECKED, bool SMEM, int TW, bool OCC, bool SHARE = false, bool BIN = false>
__global__ void __launch_bounds__(kBlock, OCC ? kOccBlocks : 1) k_render(WorldView w, FrameParams f, uint4* __restrict__ out,
                                                               unsigned* status, unsigned long long* counters) {
    // shared copy of the coarse bits for the model traversal (STATS or
    // CHECKED); the production walk reads the chunk distances through L1,
    // which measured faster than staging all 8 octant fields per block
    extern __shared__ uint4 s_dyn[];
    unsigned long long* s_coarse = reinterpret_cast<unsigned long long*>(s_dyn);
    using BT = BlockTile<TW>;
    // screen coordinates of the block's columns and rows, once per block
    // instead of four divisions per pixel
    __shared__ float s_col[3][BT::kW], s_row[3][BT::kH];
    const int x0 = blockIdx.x * BT::kW, y0 = f.row0 + blockIdx.y * BT::kH;
    const bool table = f.screen != nullptr;  // uniform: the frame's screen table replaces the block's
    if (!table && threadIdx.x < BT::kW) {
        s_col[0][threadIdx.x] = ray_u(f, x0 + (int)threadIdx.x);
        s_col[1][threadIdx.x] = centre_u(f, x0 + (int)threadIdx.x);
        s_col[2][threadIdx.x] = vignette_u(s_col[1][threadIdx.x]);
    } else if (!table && threadIdx.x >= 64 && threadIdx.x < 64 + BT::kH) {
        s_row[0][threadIdx.x - 64] = ray_v(f, y0 + (int)threadIdx.x - 64);
        s_row[1][threadIdx.x - 64] = centre_v(f, y0 + (int)threadIdx.x - 64);
        s_row[2][threadIdx.x - 64] = vignette_v(s_row[1][threadIdx.x - 64]);
    }
    if (SMEM)
        for (unsigned i = threadIdx.x; i < w.ncoarse; i += blockDim.x) s_coarse[i] = __ldg(w.coarse + i);
    if (SMEM || !table) __syncthreads();
    if (BIN) stage_begin();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int lx = (warp % BT::kWarpsX) * TW + (lane % TW), ly = (warp / BT::kWarpsX) * (32 / TW) + (lane / TW);
    const int px = x0 + lx, py = y0 + ly;
    PixelCounters pc;
#pragma unroll
    for (int k = 0; k < kNumCounters; ++k) pc.v[k] = 0;
    if (px < f.width && py < f.row_end) {
        PixelUV uv;
        if (table) {
            uv = table_uv(f, px, py);
        } else {
            uv.ru = s_col[0][lx];
            uv.cu = s_col[1][lx];
            uv.rv = s_row[0][ly];
            uv.cv = s_row[1][ly];
            uv.gu = s_col[2][lx];
            uv.gv = s_row[2][ly];
        }
        uint4 rec;
        if (SMEM) rec = render_pixel<STATS, CHECKED>(w, CoarseShared{s_coarse}, w.cdist, f, px, py, uv, status, pc);
        else rec = render_pixel<STATS, CHECKED, CoarseGlobal, SHARE, BIN>(w, CoarseGlobal{w.coarse}, w.cdist, f, px,
                                                                          py, uv, status, pc);
        out[(size_t)py * f.width + px] = rec;
    }
    if (BIN) stage_flush(f);
    flush_counters<STATS>(pc, counters);
}

// Explicit ray list (production traversal); record.rgba is 0.
template <bool CHECKED>
__global__ void __launch_bounds__(kBlock) k_trace_rays(WorldView w, const float* __restrict__ origins,
                                                       const float* __restrict__ dirs, int n, int max_steps,
                                                       uint4* __restrict__ out, unsigned* status) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float o[3], d[3];
#pragma unroll
    for (int j = 0; j < 3; ++j) {
        o[j] = origins[3 * i + j];
        d[j] = dirs[3 * i + j];
    }
    PRay r;
    pray_init(r, o, d);
    TraceHit h;
    TraceCounters cnt;
    const bool hit = near_origin(r.o) ? trace_fast<true, true, true>(w, w.cdist, r, max_steps, h)
                                      : trace_fast<true, true, false>(w, w.cdist, r, max_steps, h);
    if (hit) {
        const int e = h.axis;
        const bool pe = e == 0 ? r.pos[0] : (e == 1 ? r.pos[1] : r.pos[2]);
        const unsigned voxel = (unsigned)h.c[0] + (unsigned)w.dims[0] * ((unsigned)h.c[1] + (unsigned)w.dims[1] * (unsigned)h.c[2]);
        const unsigned face = 2u * (unsigned)e + (pe ? 0u : 1u);
        out[i] = make_uint4(voxel, __float_as_uint(h.t), 0u, face | (h.mat << 8) | (VT_HIT_PRIMARY << 16));
    } else {
        out[i] = make_uint4(0xFFFFFFFFu, __float_as_uint(-1.0f), 0u, 0xFFu);
    }
}

// ---------------------------------------------------------------------------
// Persistent render kernel (a tuning option: VT_KERNEL_QUEUE).
//
// A one-ray-per-thread launch leaves lanes idle: a warp runs until its longest
// primary ray ends, then again until its longest shadow ray ends, while lanes
// whose ray ended (or whose primary missed) wait.  Here every lane owns one
// pixel at a time and walks its primary, shadow and bounce rays in one loop;
// a lane whose pixel is finished takes the next pixel from the warp's batch of
// 32 queue entries, and the warp grabs a new batch from a global counter when
// the batch is used up.  Queue entries walk the image in 8 x 4 pixel tiles, so
// the lanes of a warp still trace neighbouring pixels.
constexpr int kPersistBlock = 128;
// vt_render_host splits frames of at least kPipelinePixels into
// kPipelineBands row bands (at most kMaxBands).
constexpr size_t kPipelinePixels = 1u << 18;
constexpr int kPipelineBands = 16;
static_assert(kPipelineBands <= kMaxBands, "band events");
constexpr unsigned kGrab = 32;

__device__ __forceinline__ void pixel_of(unsigned idx, unsigned tiles_x, int& px, int& py) {
    const unsigned tile = idx >> 5, l = idx & 31u;
    px = (int)((tile % tiles_x) * 8u + (l & 7u));
    py = (int)((tile / tiles_x) * 4u + (l >> 3));
}

// NEAR: the camera passes near_origin, so every ray of the frame does
// (secondary rays start inside the grid) and the walk takes the
// one-correction plane search.
template <bool NEAR>
__global__ void __launch_bounds__(kPersistBlock) k_render_persist(WorldView w, FrameParams f, uint4* __restrict__ out,
                                                                  unsigned* __restrict__ work, unsigned total,
                                                                  unsigned tiles_x, int batch) {
    const unsigned char* cd = w.cdist;
    const unsigned lane = threadIdx.x & 31u;
    const unsigned below = (1u << lane) - 1u;
    unsigned bnext = 0, bend = 0;  // the warp's batch of queue entries (warp-uniform)
    // per lane: the ray being walked (kind 1 primary, 2 shadow, 3 bounce), or
    // parked with the result of the ray that ended (res), or without a pixel
    int kind = 0, res = 0;
    bool active = false, retired = false;
    int px = 0, py = 0;
    Walker wk;
    unsigned voxel = 0, face = 0, mat = 0, flags = 0;
    float thit = 0.0f, so[3] = {0.0f, 0.0f, 0.0f}, nrm[3] = {0.0f, 0.0f, 0.0f}, bdir[3] = {0.0f, 0.0f, 0.0f};
    int e_hit = 0;
    bool pe_hit = false;

    for (;;) {
        if (active) {
            TraceHit h;
            const int s = wk.step<true, true, NEAR>(w, cd, h);
            if (s != Walker::kMore) {
                active = false;
                res = s;
                if (kind == 1 && s == Walker::kHit) {
                    voxel = (unsigned)h.c[0] + (unsigned)w.dims[0] * ((unsigned)h.c[1] + (unsigned)w.dims[1] * (unsigned)h.c[2]);
                    thit = h.t;
                    e_hit = h.axis;
                    mat = h.mat;
                }
            }
        }
        const unsigned parked = __ballot_sync(0xFFFFFFFFu, !active);
        if (__popc(parked) < batch) continue;
        if (parked == 0xFFFFFFFFu && __all_sync(0xFFFFFFFFu, retired)) break;

        // ---- one transition pass for every parked lane ----
        bool need_pixel = false;
        if (!active && !retired) {
            bool finish = false;
            if (kind == 0) {
                need_pixel = true;
            } else if (kind == 1) {
                if (res == Walker::kMiss) {
                    float o[3], d[3], col[4];
                    primary_ray(f, px, py, o, d);
                    shade_miss(f, d, col);
                    const unsigned rgba = f.shade == VT_SHADE_NONE ? 0u : composite(f, px, py, col);
                    out[(size_t)py * f.width + px] = make_uint4(0xFFFFFFFFu, __float_as_uint(-1.0f), rgba, 0xFFu);
                    need_pixel = true;
                } else {
                    flags = VT_HIT_PRIMARY;
                    pe_hit = e_hit == 0 ? wk.r.pos[0] : (e_hit == 1 ? wk.r.pos[1] : wk.r.pos[2]);
                    face = 2u * (unsigned)e_hit + (pe_hit ? 0u : 1u);
#pragma unroll
                    for (int j = 0; j < 3; ++j) {
                        nrm[j] = (j == e_hit) ? (pe_hit ? -1.0f : 1.0f) : 0.0f;
                        so[j] = __fmaf_rn(wk.r.d[j], thit, wk.r.o[j]);
                        if (j == e_hit) so[j] = so[j] + nrm[j] * 0.001f;
                    }
                    kind = 2;
                    if (f.rays & VT_RAYS_SHADOW) active = wk.start(w, so, f.sun, f.shadow_max_steps);
                    res = Walker::kMiss;  // a shadow ray that cannot start is unblocked
                }
            }
            if (!active && kind == 2) {
                if (res == Walker::kHit) flags |= VT_HIT_SHADOWED;
                kind = 3;
                if (f.rays & VT_RAYS_BOUNCE) {
                    unsigned seed = ((unsigned)px * 1973u + (unsigned)py * 9277u) ^ f.seed;
                    cosine_hemisphere(nrm, seed, bdir);
                    active = wk.start(w, so, bdir, f.bounce_max_steps);
                    res = Walker::kMiss;
                } else {
                    finish = true;
                }
            } else if (!active && kind == 3) {
                if (res == Walker::kHit) flags |= VT_HIT_BOUNCE;
                finish = true;
            }
            if (finish) {
                const unsigned alb = __ldg(w.palette + mat);
                float col[4];
                shade_hit(f, alb, e_hit, pe_hit, (flags & VT_HIT_SHADOWED) != 0,
                          (f.rays & VT_RAYS_BOUNCE) && !(flags & VT_HIT_BOUNCE), bdir, col);
                const unsigned rgba = f.shade == VT_SHADE_NONE ? alb : composite(f, px, py, col);
                out[(size_t)py * f.width + px] =
                    make_uint4(voxel, __float_as_uint(thit), rgba, face | (mat << 8) | (flags << 16));
                need_pixel = true;
            }
        }
        // ---- refill lanes without a pixel from the queue ----
        unsigned need = __ballot_sync(0xFFFFFFFFu, need_pixel);
        while (need) {
            if (bnext == bend) {
                unsigned b = 0;
                if (lane == 0) b = atomicAdd(work, kGrab);
                b = __shfl_sync(0xFFFFFFFFu, b, 0);
                bnext = b;
                bend = b + kGrab;
            }
            const unsigned avail = bend - bnext;
            const unsigned rank = __popc(need & below);
            if (need_pixel && rank < avail) {
                const unsigned idx = bnext + rank;
                need_pixel = false;
                kind = 0;
                if (idx >= total) {
                    retired = true;
                } else {
                    pixel_of(idx, tiles_x, px, py);
                    if (px < f.width && py < f.height) {
                        float o[3], d[3];
                        primary_ray(f, px, py, o, d);
                        kind = 1;
                        active = wk.start(w, o, d, f.max_steps);
                        res = Walker::kMiss;  // a primary that cannot start misses
                    }
                }
            }
            bnext += min(avail, (unsigned)__popc(need));
            // lanes whose entry was outside the image or whose primary missed
            // the grid at once take another entry in the next transition
            need = __ballot_sync(0xFFFFFFFFu, need_pixel);
        }
    }
}

FrameParams make_frame(const vt_camera* cam, const vt_params* p) {
    FrameParams f;
    for (int j = 0; j < 3; ++j) {
        f.pos[j] = cam->pos[j];
        f.sun[j] = p->sun_dir[j];
    }
    std::memcpy(f.view, cam->view, sizeof(f.view));
    f.tan_half_fov = cam->tan_half_fov;
    f.width = cam->width;
    f.height = cam->height;
    f.row0 = 0;
    f.row_end = cam->height;
    f.bounce_jobs = nullptr;
    f.bounce_count = nullptr;
    f.screen = nullptr;
    f.max_steps = p->max_steps;
    f.shadow_max_steps = p->shadow_max_steps;
    f.bounce_max_steps = p->bounce_max_steps;
    f.rays = p->rays | VT_RAYS_PRIMARY;
    f.shade = p->shade;
    f.flags = p->flags;
    f.seed = p->seed;
    f.ambient = p->ambient;
    f.diffuse = p->diffuse;
    f.bounce_weight = p->bounce_weight;
    frame_constants(f);
    return f;
}

vt_status check_frame_args(vt_ctx* ctx, const vt_world* world, const vt_camera* cam, const vt_params* p) {
    if (!ctx) return VT_ERR_ARG;
    if (!world || !cam || !p) return fail(ctx, VT_ERR_ARG, "null world, camera or params");
    if (world->ctx != ctx) return fail(ctx, VT_ERR_ARG, "world belongs to another context");
    if (cam->width <= 0 || cam->height <= 0 || cam->width > kMaxImageSide || cam->height > kMaxImageSide)
        return fail(ctx, VT_ERR_ARG, "camera size out of range (1..32768)");
    if (p->shade > VT_SHADE_LAMBERT) return fail(ctx, VT_ERR_ARG, "unknown shade mode");
    return VT_OK;
}

// Height in rows of the block tile of the production kernel for a tuning
// (bands of vt_render_host are multiples of it); 0 for the queue kernel.
int band_rows_unit(const vt_tuning& tu) {
    if (tu.kernel == VT_KERNEL_QUEUE) return 0;
    if (tu.warp_tile_w == 4) return BlockTile<4>::kH;
    if (tu.warp_tile_w == 16) return BlockTile<16>::kH;
    if (tu.warp_tile_w == 32) return BlockTile<32>::kH;
    return BlockTile<8>::kH;
}

vt_status band_streams(vt_ctx* ctx) {
    if (ctx->copy_stream) return VT_OK;
    for (int i = 0; i < kBandStreams; ++i)
        VT_CUDA(ctx, cudaStreamCreateWithFlags(&ctx->band_stream[i], cudaStreamNonBlocking));
    VT_CUDA(ctx, cudaEventCreateWithFlags(&ctx->ev_start, cudaEventDisableTiming));
    for (int i = 0; i < kMaxBands; ++i) VT_CUDA(ctx, cudaEventCreateWithFlags(&ctx->ev_band[i], cudaEventDisableTiming));
    VT_CUDA(ctx, cudaStreamCreateWithFlags(&ctx->copy_stream, cudaStreamNonBlocking));
    return VT_OK;
}

__global__ void __launch_bounds__(kBlock) k_screen_table(FrameParams f, float4* __restrict__ tab) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < f.width) {
        const float cu = centre_u(f, i);
        tab[i] = make_float4(ray_u(f, i), cu, vignette_u(cu), 0.0f);
    } else if (i < f.width + f.height) {
        const int y = i - f.width;
        const float cv = centre_v(f, y);
        tab[i] = make_float4(ray_v(f, y), cv, vignette_v(cv), 0.0f);
    }
}

// The context's screen table for the frame's size and field of view, made on
// first use (then synchronised once, so that frames on any stream may read
// it).  Null, and the kernel computes the coordinates per block, when the
// context already holds kScreenTables of them, when `create` is false (the
// allocation-free entry point) or when `st` is being captured into a graph
// (no allocation or synchronisation there).
vt_status screen_table(vt_ctx* ctx, const FrameParams& f, cudaStream_t st, bool create, const float4** out) {
    *out = nullptr;
    for (int i = 0; i < ctx->n_screen; ++i) {
        const ScreenTable& t = ctx->screen[i];
        if (t.width == f.width && t.height == f.height &&
            std::memcmp(&t.tan_half_fov, &f.tan_half_fov, sizeof(float)) == 0) {
            *out = t.d;
            return VT_OK;
        }
    }
    if (!create || ctx->n_screen >= kScreenTables) return VT_OK;
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(st, &cs) != cudaSuccess) {
        cudaGetLastError();
        return VT_OK;
    }
    if (cs != cudaStreamCaptureStatusNone) return VT_OK;
    ScreenTable t;
    t.width = f.width;
    t.height = f.height;
    t.tan_half_fov = f.tan_half_fov;
    const size_t n = (size_t)f.width + (size_t)f.height;
    VT_CUDA(ctx, vt::dev_alloc(&t.d, n * sizeof(float4)));
    k_screen_table<<<(unsigned)((n + kBlock - 1) / kBlock), kBlock, 0, st>>>(f, t.d);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) {
        vt::dev_free(t.d);
        return check_cuda(ctx, e, "screen table");
    }
    ctx->screen[ctx->n_screen++] = t;
    *out = t.d;
    return VT_OK;
}

vt_status launch_render(vt_ctx* ctx, const vt_world* world, const vt_camera* cam, const vt_params* p,
                               uint4* d_out, cudaStream_t stream, bool stats, int row0, int row1, bool allow_defer,
                               bool new_table) {
    FrameParams f = make_frame(cam, p);
    if (row1 < 0) row1 = cam->height;
    f.row0 = row0;
    f.row_end = row1;
    const int rows = row1 - row0;
    const WorldView w = world->view();
    const bool checked = (p->flags & VT_FLAG_CHECKED) != 0;
    const size_t smem = (size_t)w.ncoarse * sizeof(unsigned long long);
    const bool use_smem = (stats || checked) && smem <= kMaxSharedCoarse;
    {
        vt_status s = update_distances(const_cast<vt_world*>(world), stream);
        if (s) return s;
    }
    const size_t sm = use_smem ? smem : 0;
    const vt_tuning& tu = ctx->tuning;
    cudaAccessPolicyWindow win_storage;
    const cudaAccessPolicyWindow* win = nullptr;  // L2 window over the brick words (tuning l2_persist)
    {
        vt_status s = l2_policy(ctx, world, &win_storage, &win);
        if (s) return s;
    }
    if (!stats && !checked && tu.kernel == VT_KERNEL_QUEUE) {
        // persistent kernel over a pixel queue; the queue counter is one slot
        // of the context's ring, zeroed on this stream before the launch
        if (ctx->persist_blocks == 0) {
            int nb = 0;
            VT_CUDA(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_render_persist<true>, kPersistBlock, 0));
            ctx->persist_blocks = nb > 0 ? nb : 1;
        }
        unsigned* counter = ctx->d_work + (ctx->work_slot++ % kWorkSlots);
        VT_CUDA(ctx, cudaMemsetAsync(counter, 0, sizeof(unsigned), stream));
        const unsigned tiles_x = (unsigned)(cam->width + 7) / 8u, tiles_y = (unsigned)(cam->height + 3) / 4u;
        const unsigned total = tiles_x * tiles_y * 32u;
        const unsigned blocks = (unsigned)(ctx->sm_count * ctx->persist_blocks);
        const int batch = tu.batch;
        if (near_origin(f.pos))
            VT_CUDA(ctx, launch_kernel(k_render_persist<true>, dim3(blocks), dim3(kPersistBlock), 0, stream, win, w, f,
                                       d_out, counter, total, tiles_x, batch));
        else
            VT_CUDA(ctx, launch_kernel(k_render_persist<false>, dim3(blocks), dim3(kPersistBlock), 0, stream, win, w,
                                       f, d_out, counter, total, tiles_x, batch));
        return VT_OK;
    }
    {
        vt_status s = screen_table(ctx, f, stream, new_table, &f.screen);
        if (s) return s;
    }
    const bool defer = allow_defer && (p->rays & VT_RAYS_BOUNCE) && !stats && !checked;
    // the direction-sorted append exists for the default 8 x 4 capped tile kernel
    const bool binned = defer && tu.bounce_sort && tu.warp_tile_w == 8 && tu.occupancy && !tu.share_bricks;
    if (defer) {
        vt_status s = bounce_buffers(ctx, (size_t)cam->width * (size_t)cam->height);
        if (s) return s;
        VT_CUDA(ctx, cudaStreamWaitEvent(stream, ctx->ev_bounce, 0));
        VT_CUDA(ctx, cudaMemsetAsync(ctx->d_bounce_ctr, 0, 2 * sizeof(unsigned), stream));
        f.bounce_jobs = ctx->d_bounce_jobs;
        f.bounce_count = ctx->d_bounce_ctr;
    }
    cudaError_t le = cudaSuccess;
#define VT_LAUNCH_X(S, C, M, TW, O, SH)                                                                         \
    le = launch_kernel(k_render<S, C, M, TW, O, SH>,                                                            \
                       dim3((cam->width + BlockTile<TW>::kW - 1) / BlockTile<TW>::kW,                           \
                            (rows + BlockTile<TW>::kH - 1) / BlockTile<TW>::kH),                                \
                       dim3(kBlock), sm, stream, win, w, f, d_out, ctx->d_status, ctx->d_counters)
#define VT_LAUNCH(S, C, M, TW, O) VT_LAUNCH_X(S, C, M, TW, O, false)
#define VT_LAUNCH_M(S, C, TW, O)      \
    if (use_smem) VT_LAUNCH(S, C, true, TW, O); \
    else VT_LAUNCH(S, C, false, TW, O)
    if (stats) {
        VT_LAUNCH_M(true, true, 8, false);
    } else if (checked) {
        VT_LAUNCH_M(false, true, 8, false);
    } else if (tu.warp_tile_w == 4) {
        if (tu.occupancy) { VT_LAUNCH(false, false, false, 4, true); }
        else { VT_LAUNCH(false, false, false, 4, false); }
    } else if (tu.warp_tile_w == 16) {
        if (tu.occupancy) { VT_LAUNCH(false, false, false, 16, true); }
        else { VT_LAUNCH(false, false, false, 16, false); }
    } else if (tu.warp_tile_w == 32) {
        if (tu.occupancy) { VT_LAUNCH(false, false, false, 32, true); }
        else { VT_LAUNCH(false, false, false, 32, false); }
    } else {
        if (binned) { le = launch_kernel(k_render<false, false, false, 8, true, false, true>,
                                         dim3((cam->width + BlockTile<8>::kW - 1) / BlockTile<8>::kW,
                                              (rows + BlockTile<8>::kH - 1) / BlockTile<8>::kH),
                                         dim3(kBlock), sm, stream, win, w, f, d_out, ctx->d_status, ctx->d_counters); }
        else if (tu.occupancy && tu.share_bricks) { VT_LAUNCH_X(false, false, false, 8, true, true); }
        else if (tu.occupancy) { VT_LAUNCH(false, false, false, 8, true); }
        else { VT_LAUNCH(false, false, false, 8, false); }
    }
#undef VT_LAUNCH_M
#undef VT_LAUNCH
#undef VT_LAUNCH_X
    VT_CUDA(ctx, le);
    if (stats || checked) return note_status_writer(ctx, stream);  // the model walk checks its indexes
    if (defer) return launch_bounce(ctx, world, f, d_out, stream);
    return VT_OK;
}

}  // namespace vt

using namespace vt;

extern "C" {

void vt_params_default(vt_params* p) {
    if (!p) return;
    std::memset(p, 0, sizeof(*p));
    p->max_steps = 512;
    p->shadow_max_steps = 512;
    p->bounce_max_steps = 256;
    p->rays = VT_RAYS_PRIMARY | VT_RAYS_SHADOW;
    p->shade = VT_SHADE_REFERENCE;
    p->flags = VT_FLAG_CROSSHAIR | VT_FLAG_VIGNETTE;
    p->seed = 0;
    // SUN_DIR of the reference (camera.glsl:8)
    p->sun_dir[0] = 7.52185881e-01f;
    p->sun_dir[1] = 6.58950984e-01f;
    p->sun_dir[2] = 7.52185881e-01f;
    p->ambient = 0.2f;
    p->diffuse = 0.8f;
    p->bounce_weight = 0.3f;
}

vt_status vt_render(vt_ctx* ctx, const vt_world* world, const vt_camera* cam, const vt_params* params, vt_hit* d_out,
                    vt_stream stream) {
    vt_status s = check_frame_args(ctx, world, cam, params);
    if (s) return s;
    if (!d_out) return fail(ctx, VT_ERR_ARG, "null output buffer");
    return launch_render(ctx, world, cam, params, reinterpret_cast<uint4*>(d_out), (cudaStream_t)stream, false, 0, -1,
                         true);
}

vt_status vt_render_host(vt_ctx* ctx, const vt_world* world, const vt_camera* cam, const vt_params* params,
                         vt_hit* h_out) {
    vt_status s = check_frame_args(ctx, world, cam, params);
    if (s) return s;
    if (!h_out) return fail(ctx, VT_ERR_ARG, "null output buffer");
    const size_t W = (size_t)cam->width, H = (size_t)cam->height;
    const size_t bytes = W * H * sizeof(vt_hit);
    // Pinned host memory is mapped into the device's address space: the
    // kernel stores the records straight into it over the host link, with no
    // staging copy (1080p: 244 us per frame end to end against 288 us for the
    // band pipeline below, kernel alone 210 us).
    {
        cudaPointerAttributes pa;
        if (cudaPointerGetAttributes(&pa, h_out) == cudaSuccess && pa.type == cudaMemoryTypeHost && pa.devicePointer) {
            s = launch_render(ctx, world, cam, params, reinterpret_cast<uint4*>(pa.devicePointer), ctx->stream, false,
                              0, -1, true);
            if (s) return s;
            return vt_sync(ctx, ctx->stream);
        }
        cudaGetLastError();  // a pageable pointer is not an error
    }
    void* d_scratch = nullptr;
    s = ctx_scratch(ctx, bytes, &d_scratch);
    if (s) return s;
    uint4* d_out = reinterpret_cast<uint4*>(d_scratch);
    const int rows_tile = band_rows_unit(ctx->tuning);
    // (bounce rays go through the deferred pass, one launch for the frame)
    const bool pipelined = ctx->tuning.kernel != VT_KERNEL_QUEUE && W * H >= kPipelinePixels &&
                           (params->flags & VT_FLAG_CHECKED) == 0 && (params->rays & VT_RAYS_BOUNCE) == 0 &&
                           rows_tile > 0;
    if (!pipelined) {
        s = launch_render(ctx, world, cam, params, d_out, ctx->stream, false, 0, -1, true);
        if (s) return s;
        VT_CUDA(ctx, cudaMemcpyAsync(h_out, d_out, bytes, cudaMemcpyDeviceToHost, ctx->stream));
        return vt_sync(ctx, ctx->stream);
    }
    // Pageable memory: row bands, rendered on kBandStreams streams (so that one
    // band's tail overlaps the next band) and copied to the host each as soon
    // as it is done: the copy of the frame overlaps its rendering, except the
    // last band.
    s = band_streams(ctx);
    if (s) return s;
    s = update_distances(const_cast<vt_world*>(world), ctx->stream);
    if (s) return s;
    VT_CUDA(ctx, cudaEventRecord(ctx->ev_start, ctx->stream));
    for (int i = 0; i < kBandStreams; ++i) VT_CUDA(ctx, cudaStreamWaitEvent(ctx->band_stream[i], ctx->ev_start, 0));
    const int bands = (int)std::min<size_t>(kPipelineBands, (H + rows_tile - 1) / rows_tile);
    const int per = (int)(((H + bands - 1) / bands + rows_tile - 1) / rows_tile) * rows_tile;
    int nb = 0;
    for (int r0 = 0; r0 < (int)H; r0 += per, ++nb) {
        const int r1 = std::min((int)H, r0 + per);
        cudaStream_t bs = ctx->band_stream[nb % kBandStreams];
        s = launch_render(ctx, world, cam, params, d_out, bs, false, r0, r1);
        if (s) return s;
        VT_CUDA(ctx, cudaEventRecord(ctx->ev_band[nb], bs));
    }
    // copies queued after every launch: with pageable host memory a copy
    // returns only when done, and must not hold back the launches
    // (one copy stream: copies spread over the band streams measured slower)
    nb = 0;
    for (int r0 = 0; r0 < (int)H; r0 += per, ++nb) {
        const int r1 = std::min((int)H, r0 + per);
        VT_CUDA(ctx, cudaStreamWaitEvent(ctx->copy_stream, ctx->ev_band[nb], 0));
        VT_CUDA(ctx, cudaMemcpyAsync(h_out + (size_t)r0 * W, d_out + (size_t)r0 * W, (size_t)(r1 - r0) * W * sizeof(vt_hit),
                                     cudaMemcpyDeviceToHost, ctx->copy_stream));
    }
    // the status word rides on the copy stream: one synchronisation in all
    VT_CUDA(ctx, cudaMemcpyAsync(ctx->h_status, ctx->d_status, sizeof(unsigned), cudaMemcpyDeviceToHost,
                                 ctx->copy_stream));
    VT_CUDA(ctx, cudaStreamSynchronize(ctx->copy_stream));
    return take_status(ctx, *ctx->h_status);
}

vt_status vt_render_stats(vt_ctx* ctx, const vt_world* world, const vt_camera* cam, const vt_params* params,
                          vt_stats* out, vt_stream stream) {
    vt_status s = check_frame_args(ctx, world, cam, params);
    if (s) return s;
    if (!out) return fail(ctx, VT_ERR_ARG, "null stats");
    const size_t bytes = (size_t)cam->width * cam->height * sizeof(vt_hit);
    void* d_out = nullptr;
    s = ctx_scratch(ctx, bytes, &d_out);
    if (s) return s;
    cudaStream_t st = (cudaStream_t)stream;
    VT_CUDA(ctx, cudaMemsetAsync(ctx->d_counters, 0, kNumCounters * sizeof(unsigned long long), st));
    s = launch_render(ctx, world, cam, params, reinterpret_cast<uint4*>(d_out), st, true);
    if (s) return s;
    unsigned long long h[kNumCounters];
    VT_CUDA(ctx, cudaMemcpyAsync(h, ctx->d_counters, sizeof(h), cudaMemcpyDeviceToHost, st));
    s = vt_sync(ctx, stream);
    if (s) return s;
    static_assert(sizeof(vt_stats) == sizeof(h), "vt_stats layout");
    std::memcpy(out, h, sizeof(h));
    return VT_OK;
}

vt_status vt_trace_rays(vt_ctx* ctx, const vt_world* world, const float* d_origins, const float* d_dirs, int32_t n,
                        int32_t max_steps, vt_hit* d_out, vt_stream stream) {
    if (!ctx) return VT_ERR_ARG;
    if (!world || !d_origins || !d_dirs || !d_out || n < 0) return fail(ctx, VT_ERR_ARG, "bad trace_rays arguments");
    if (n == 0) return VT_OK;
    {
        vt_status s = update_distances(const_cast<vt_world*>(world), (cudaStream_t)stream);
        if (s) return s;
    }
    const WorldView w = world->view();
    k_trace_rays<true><<<(n + kBlock - 1) / kBlock, kBlock, 0, (cudaStream_t)stream>>>(
        w, d_origins, d_dirs, n, max_steps, reinterpret_cast<uint4*>(d_out), ctx->d_status);
    VT_CUDA(ctx, cudaGetLastError());
    return note_status_writer(ctx, (cudaStream_t)stream);
}

}  // extern "C"
