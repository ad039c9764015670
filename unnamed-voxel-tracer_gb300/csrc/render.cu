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

#include "shade.cuh"
#include "trace_p.cuh"

namespace vt {

// Pixel tile of a 256-thread block: 16 x 16 pixels, each warp an 8 x 4 tile
// so that a warp's rays start close together and share brick words in L1.
constexpr int kTileW = 16;
constexpr int kTileH = 16;
constexpr int kBlock = 256;
constexpr size_t kMaxSharedCoarse = 48 * 1024;

struct PixelCounters {
    unsigned v[kNumCounters];
};

// The instrumented and bounds-checked variants run the three-level model
// traversal (it defines the algorithmic byte counts); the production variant
// runs trace_fast.  Both give identical results.
template <bool STATS, bool CHECKED, bool MAT, class Coarse>
__device__ __forceinline__ bool trace_any(const WorldView& w, const Coarse& coarse, const unsigned char* cd,
                                          const PRay& r, int max_steps, TraceHit& h, TraceCounters& cnt,
                                          unsigned* status) {
    if (STATS || CHECKED) return trace_p<STATS, CHECKED, MAT>(w, coarse, r, max_steps, h, cnt, status);
    return trace_fast<MAT>(w, cd, r, max_steps, h);
}

template <bool STATS, bool CHECKED, class Coarse>
__device__ __forceinline__ uint4 render_pixel(const WorldView& w, const Coarse& coarse, const unsigned char* cd,
                                              const FrameParams& f, int px, int py, unsigned* status,
                                              PixelCounters& pc) {
    float o[3], d[3];
    primary_ray(f, px, py, o, d);
    PRay r;
    pray_init(r, o, d);
    TraceHit h;
    TraceCounters cnt;
    const bool hit = trace_any<STATS, CHECKED, true>(w, coarse, cd, r, f.max_steps, h, cnt, status);
    if (STATS) {
        pc.v[0] += 1;
        pc.v[9] += 16;
    }
    unsigned flags = 0, rgba, voxel = 0xFFFFFFFFu, face = 0xFFu, mat = 0;
    float t = -1.0f;
    float col[4];
    if (hit) {
        flags = VT_HIT_PRIMARY;
        voxel = (unsigned)h.c[0] + (unsigned)w.dims[0] * ((unsigned)h.c[1] + (unsigned)w.dims[1] * (unsigned)h.c[2]);
        t = h.t;
        const int e = h.axis;
        const bool pe = e == 0 ? r.pos[0] : (e == 1 ? r.pos[1] : r.pos[2]);
        face = 2u * (unsigned)e + (pe ? 0u : 1u);
        mat = h.mat;
        const unsigned alb = __ldg(w.palette + mat);
        if (STATS) {
            pc.v[1] += 1;
            pc.v[8] += 1;
        }
        float nrm[3], so[3];
#pragma unroll
        for (int j = 0; j < 3; ++j) {
            nrm[j] = (j == e) ? (pe ? -1.0f : 1.0f) : 0.0f;
            so[j] = __fmaf_rn(r.d[j], t, o[j]);
            if (j == e) so[j] = so[j] + nrm[j] * 0.001f;
        }
        bool shadowed = false;
        if (f.rays & VT_RAYS_SHADOW) {
            PRay rs;
            pray_init(rs, so, f.sun);
            TraceHit hs;
            shadowed = trace_any<STATS, CHECKED, false>(w, coarse, cd, rs, f.shadow_max_steps, hs, cnt, status);
            if (shadowed) flags |= VT_HIT_SHADOWED;
            if (STATS) {
                pc.v[2] += 1;
                pc.v[3] += shadowed ? 1u : 0u;
            }
        }
        bool bounce_open = false;
        float bdir[3] = {0.0f, 0.0f, 0.0f};
        if (f.rays & VT_RAYS_BOUNCE) {
            unsigned seed = ((unsigned)px * 1973u + (unsigned)py * 9277u) ^ f.seed;
            cosine_hemisphere(nrm, seed, bdir);
            PRay rb;
            pray_init(rb, so, bdir);
            TraceHit hb;
            const bool bh = trace_any<STATS, CHECKED, false>(w, coarse, cd, rb, f.bounce_max_steps, hb, cnt, status);
            if (bh) flags |= VT_HIT_BOUNCE;
            bounce_open = !bh;
            if (STATS) {
                pc.v[4] += 1;
                pc.v[5] += bh ? 1u : 0u;
            }
        }
        shade_hit(f, alb, e, pe, shadowed, bounce_open, bdir, col);
        rgba = f.shade == VT_SHADE_NONE ? alb : composite(f, px, py, col);
    } else {
        shade_miss(f, d, col);
        rgba = f.shade == VT_SHADE_NONE ? 0u : composite(f, px, py, col);
    }
    if (STATS) {
        pc.v[6] += cnt.mask;
        pc.v[7] += cnt.coarse;
        pc.v[10] += cnt.steps;
        pc.v[11] += cnt.iters;
    }
    return make_uint4(voxel, __float_as_uint(t), rgba, face | (mat << 8) | (flags << 16));
}

template <bool STATS>
__device__ __forceinline__ void flush_counters(PixelCounters& pc, unsigned long long* counters) {
    if (!STATS) return;
#pragma unroll
    for (int k = 0; k < kNumCounters; ++k) {
        const unsigned s = __reduce_add_sync(0xFFFFFFFFu, pc.v[k]);
        if ((threadIdx.x & 31) == 0 && s) atomicAdd(counters + k, (unsigned long long)s);
    }
}

template <bool STATS, bool CHECKED, bool SMEM>
__global__ void __launch_bounds__(kBlock) k_render(WorldView w, FrameParams f, uint4* __restrict__ out,
                                                   unsigned* status, unsigned long long* counters) {
    // shared copy of the coarse level: per-chunk distances (production) or
    // coarse bits (model traversal)
    extern __shared__ uint4 s_dyn[];
    unsigned long long* s_coarse = reinterpret_cast<unsigned long long*>(s_dyn);
    unsigned char* s_cdist = reinterpret_cast<unsigned char*>(s_dyn);
    if (SMEM) {
        if (STATS || CHECKED) {
            for (unsigned i = threadIdx.x; i < w.ncoarse; i += blockDim.x) s_coarse[i] = __ldg(w.coarse + i);
        } else {
            const uint4* src = reinterpret_cast<const uint4*>(w.cdist);
            for (unsigned i = threadIdx.x; i < (w.nchunks + 15u) / 16u; i += blockDim.x) s_dyn[i] = __ldg(src + i);
        }
        __syncthreads();
    }
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int px = blockIdx.x * kTileW + (warp & 1) * 8 + (lane & 7);
    const int py = blockIdx.y * kTileH + (warp >> 1) * 4 + (lane >> 3);
    PixelCounters pc;
#pragma unroll
    for (int k = 0; k < kNumCounters; ++k) pc.v[k] = 0;
    if (px < f.width && py < f.height) {
        uint4 rec;
        if (SMEM) rec = render_pixel<STATS, CHECKED>(w, CoarseShared{s_coarse}, s_cdist, f, px, py, status, pc);
        else rec = render_pixel<STATS, CHECKED>(w, CoarseGlobal{w.coarse}, w.cdist, f, px, py, status, pc);
        out[(size_t)py * f.width + px] = rec;
    }
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
    const bool hit = trace_fast<true>(w, w.cdist, r, max_steps, h);
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
    if (cam->width <= 0 || cam->height <= 0 || cam->width > 32768 || cam->height > 32768)
        return fail(ctx, VT_ERR_ARG, "camera size out of range (1..32768)");
    if (p->shade > VT_SHADE_LAMBERT) return fail(ctx, VT_ERR_ARG, "unknown shade mode");
    return VT_OK;
}

static vt_status launch_render(vt_ctx* ctx, const vt_world* world, const vt_camera* cam, const vt_params* p,
                               uint4* d_out, cudaStream_t stream, bool stats) {
    const FrameParams f = make_frame(cam, p);
    const WorldView w = world->view();
    const dim3 grid((cam->width + kTileW - 1) / kTileW, (cam->height + kTileH - 1) / kTileH);
    const bool checked = (p->flags & VT_FLAG_CHECKED) != 0;
    const size_t smem = (stats || checked) ? (size_t)w.ncoarse * sizeof(unsigned long long)
                                           : (size_t)((w.nchunks + 15u) / 16u) * 16u;
    const bool use_smem = smem <= kMaxSharedCoarse;
    if (world->dist_dirty) {
        vt_status s = rebuild_distances(const_cast<vt_world*>(world), stream);
        if (s) return s;
    }
    const size_t sm = use_smem ? smem : 0;
#define VT_LAUNCH(S, C, M) k_render<S, C, M><<<grid, kBlock, sm, stream>>>(w, f, d_out, ctx->d_status, ctx->d_counters)
    if (stats) {
        if (use_smem) VT_LAUNCH(true, true, true);
        else VT_LAUNCH(true, true, false);
    } else if (checked) {
        if (use_smem) VT_LAUNCH(false, true, true);
        else VT_LAUNCH(false, true, false);
    } else {
        if (use_smem) VT_LAUNCH(false, false, true);
        else VT_LAUNCH(false, false, false);
    }
#undef VT_LAUNCH
    VT_CUDA(ctx, cudaGetLastError());
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
    return launch_render(ctx, world, cam, params, reinterpret_cast<uint4*>(d_out), (cudaStream_t)stream, false);
}

vt_status vt_render_host(vt_ctx* ctx, const vt_world* world, const vt_camera* cam, const vt_params* params,
                         vt_hit* h_out) {
    vt_status s = check_frame_args(ctx, world, cam, params);
    if (s) return s;
    if (!h_out) return fail(ctx, VT_ERR_ARG, "null output buffer");
    const size_t bytes = (size_t)cam->width * cam->height * sizeof(vt_hit);
    void* d_out = nullptr;
    s = ctx_scratch(ctx, bytes, &d_out);
    if (s) return s;
    s = launch_render(ctx, world, cam, params, reinterpret_cast<uint4*>(d_out), ctx->stream, false);
    if (s) return s;
    VT_CUDA(ctx, cudaMemcpyAsync(h_out, d_out, bytes, cudaMemcpyDeviceToHost, ctx->stream));
    return vt_sync(ctx, ctx->stream);
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
    if (world->dist_dirty) {
        vt_status s = rebuild_distances(const_cast<vt_world*>(world), (cudaStream_t)stream);
        if (s) return s;
    }
    const WorldView w = world->view();
    k_trace_rays<true><<<(n + kBlock - 1) / kBlock, kBlock, 0, (cudaStream_t)stream>>>(
        w, d_origins, d_dirs, n, max_steps, reinterpret_cast<uint4*>(d_out), ctx->d_status);
    VT_CUDA(ctx, cudaGetLastError());
    return VT_OK;
}

}  // extern "C"
