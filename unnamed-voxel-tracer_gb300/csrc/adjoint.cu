// adjoint.cu -- differentiable Lambert shading over a fixed hit set.
//
//     c = palette[m] * albedo[v] * (ka + kd * max(0, n . s^) * V),  s^ = s / |s|
//     L = sum (c - target)^2
//     dL/dpalette[m]  = 2 (c - t) * albedo[v] * shade
//     dL/dalbedo[v]   = sum_k 2 (c_k - t_k) * palette[m][k] * shade
//     dL/ds           = (sum_k 2 (c_k - t_k) palette[m][k] albedo[v]) * kd * V * [n . s^ > 0]
//                       * (n - (n . s^) s^) / |s|
//
// The primary hits (voxel, face, material, t) come from vt_render and are held
// fixed; the shadow term V is recomputed here by tracing the shadow ray from
// the hit exactly as the render kernel does (same origin arithmetic, same
// traversal), instead of being stored between passes.  The backward kernel is
// the forward kernel plus the loss and gradient epilogue, one thread per
// pixel.  Palette gradients are summed per warp over the lanes that share a
// material (the warp walks its distinct materials), per block in shared
// memory, then once per block with global atomics; albedo gradients go to
// global memory with one atomic per pixel.
#include <cstring>

#include "shade.cuh"
#include "trace_p.cuh"

namespace vt {

namespace {

constexpr int kAdjBlock = 256;

struct AdjArgs {
    WorldView w;
    FrameParams f;
    const uint4* hits;
    const float* pal;
    const float* alb;
    float sun[3], sun_n[3], inv_len;
    float ka, kd;
    int shadow_steps;
    const unsigned char* vis_in;
    unsigned char* vis_out;
    float* rgb;
    const float* target;
    float* loss;
    float* gpal;
    float* galb;
    float* gsun;
};


__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xFFFFFFFFu, v, o);
    return v;
}

// One block of 16x16 pixels of the view (f, hits, target, rgb); the rest of
// the arguments are shared by all views.
template <bool BWD>
__device__ __forceinline__ void shade_block(const AdjArgs& a, const FrameParams& f, const uint4* __restrict__ hits,
                                            const float* __restrict__ target, float* __restrict__ rgb) {
    extern __shared__ float s_mem[];
    float* s_gpal = s_mem;            // 768
    float* s_acc = s_mem + 768;       // loss, sun x3
    const unsigned char* cd = a.w.cdist;
    if (BWD) {
        for (int i = threadIdx.x; i < 772; i += blockDim.x) s_mem[i] = 0.0f;
    }
    __syncthreads();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int px = blockIdx.x * 16 + (warp & 1) * 8 + (lane & 7);
    const int py = blockIdx.y * 16 + (warp >> 1) * 4 + (lane >> 3);
    const bool inside = px < f.width && py < f.height;
    const size_t p = inside ? (size_t)py * f.width + px : 0;

    bool hit = false;
    int m = 0;
    unsigned v = 0;
    float c[3] = {0.0f, 0.0f, 0.0f}, shade = 0.0f, albv = 1.0f, ndl_raw = 0.0f, nrm[3] = {0.0f, 0.0f, 0.0f};
    bool lit = false;
    if (inside) {
        const uint4 rec = hits[p];
        hit = ((rec.w >> 16) & VT_HIT_PRIMARY) != 0;
        if (hit) {
            v = rec.x;
            const float t = __uint_as_float(rec.y);
            const unsigned face = rec.w & 0xFFu;
            m = (int)((rec.w >> 8) & 0xFFu);
            const int axis = (int)(face >> 1);
            const bool pos = (face & 1u) == 0u;
            float o[3], d[3];
            primary_ray(f, px, py, o, d);
            PRay r;
            pray_init(r, o, d);
            float so[3];
#pragma unroll
            for (int j = 0; j < 3; ++j) {
                nrm[j] = (j == axis) ? (pos ? -1.0f : 1.0f) : 0.0f;
                so[j] = __fmaf_rn(r.d[j], t, o[j]);
                if (j == axis) so[j] = so[j] + nrm[j] * 0.001f;
            }
            if (a.vis_in) {
                lit = a.vis_in[p] != 0;
            } else {
                PRay rs;
                pray_init(rs, so, a.sun);
                TraceHit hs;
                lit = !trace_fast<false, true, true>(a.w, cd, rs, a.shadow_steps, hs) &&
                      !(a.w.n_entities > 0 && entity_occluded(a.w, so, a.sun));
            }
            ndl_raw = dot3(nrm, a.sun_n);
            const float ndl = ndl_raw > 0.0f ? ndl_raw : 0.0f;
            shade = a.ka + a.kd * ndl * (lit ? 1.0f : 0.0f);
            albv = a.alb ? __ldg(a.alb + v) : 1.0f;
#pragma unroll
            for (int k = 0; k < 3; ++k) c[k] = (__ldg(a.pal + 3 * m + k) * albv) * shade;
        }
    }
    if (!BWD) {
        if (inside) {
#pragma unroll
            for (int k = 0; k < 3; ++k) rgb[3 * p + k] = c[k];
            if (a.vis_out) a.vis_out[p] = (unsigned char)(hit && lit ? 1 : 0);
        }
        return;
    }

    // ---- loss and gradients
    float g[3] = {0.0f, 0.0f, 0.0f}, lossv = 0.0f;
    if (inside) {
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            const float diff = c[k] - __ldg(target + 3 * p + k);
            g[k] = 2.0f * diff;
            lossv += diff * diff;
        }
    }
    float gp[3] = {0.0f, 0.0f, 0.0f}, ga = 0.0f, gs[3] = {0.0f, 0.0f, 0.0f};
    if (hit) {
        float gb = 0.0f;
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            const float pk = __ldg(a.pal + 3 * m + k);
            gp[k] = g[k] * albv * shade;
            ga += g[k] * pk * shade;
            gb += g[k] * pk * albv;
        }
        if (lit && ndl_raw > 0.0f) {
            const float coef = gb * a.kd * a.inv_len;
#pragma unroll
            for (int k = 0; k < 3; ++k) gs[k] = coef * (nrm[k] - ndl_raw * a.sun_n[k]);
        }
    }
    // palette: one shared-memory atomic per (warp, material).  The warp walks
    // its distinct materials (few per warp) with butterfly sums, no
    // divergence.
    {
        unsigned todo = __ballot_sync(0xFFFFFFFFu, hit);
        while (todo) {
            const int leader = __ffs(todo) - 1;
            const int key = __shfl_sync(0xFFFFFFFFu, m, leader);
            const bool mine = hit && m == key;
            todo &= ~__ballot_sync(0xFFFFFFFFu, mine);
            const float s0 = warp_sum(mine ? gp[0] : 0.0f), s1 = warp_sum(mine ? gp[1] : 0.0f),
                        s2 = warp_sum(mine ? gp[2] : 0.0f);
            if (lane == leader) {
                atomicAdd(s_gpal + 3 * key + 0, s0);
                atomicAdd(s_gpal + 3 * key + 1, s1);
                atomicAdd(s_gpal + 3 * key + 2, s2);
            }
        }
    }
    // albedo: one global atomic per hit pixel (voxels differ across most of
    // a warp; the L2 absorbs the few repeats)
    if (a.galb && hit) atomicAdd(a.galb + v, ga);
    // loss and sun: warp sums, then shared memory
    {
        const float l = warp_sum(lossv), x = warp_sum(gs[0]), y = warp_sum(gs[1]), z = warp_sum(gs[2]);
        if (lane == 0) {
            atomicAdd(s_acc + 0, l);
            atomicAdd(s_acc + 1, x);
            atomicAdd(s_acc + 2, y);
            atomicAdd(s_acc + 3, z);
        }
    }
    __syncthreads();
    for (int i = threadIdx.x; i < 768; i += blockDim.x)
        if (s_gpal[i] != 0.0f) atomicAdd(a.gpal + i, s_gpal[i]);
    if (threadIdx.x == 0) {
        atomicAdd(a.loss, s_acc[0]);
        atomicAdd(a.gsun + 0, s_acc[1]);
        atomicAdd(a.gsun + 1, s_acc[2]);
        atomicAdd(a.gsun + 2, s_acc[3]);
    }
}

template <bool BWD>
__global__ void __launch_bounds__(kAdjBlock) k_shade(AdjArgs a) {
    shade_block<BWD>(a, a.f, a.hits, a.target, a.rgb);
}

// Several views of one world in one launch (blockIdx.z = view): one launch
// instead of one per view, whose tails would leave the GPU partly idle.
constexpr int kMaxViews = 16;
struct ViewP {
    float pos[3];
    float view[16];
    float tan_half_fov;
    int width, height;
    const uint4* hits;
    const float* target;
    float* rgb;
};
struct ViewsArgs {
    AdjArgs a;
    ViewP v[kMaxViews];
};
static_assert(sizeof(ViewsArgs) <= 4096, "the views travel in the kernel parameters");

// Register caps: 40 for the backward kernel (6 blocks per SM; a 12-byte
// spill) and 48 for the forward one (5 blocks), the fastest of 40/48/59
// measured on 16 views of 512x512.
template <bool BWD>
__global__ void __launch_bounds__(kAdjBlock, BWD ? 6 : 5) k_shade_views(ViewsArgs va) {
    const ViewP& V = va.v[blockIdx.z];
    if ((int)blockIdx.x * 16 >= V.width || (int)blockIdx.y * 16 >= V.height) return;  // the view is smaller
    FrameParams f = va.a.f;
#pragma unroll
    for (int j = 0; j < 3; ++j) f.pos[j] = V.pos[j];
#pragma unroll
    for (int j = 0; j < 16; ++j) f.view[j] = V.view[j];
    f.tan_half_fov = V.tan_half_fov;
    f.width = V.width;
    f.height = V.height;
    shade_block<BWD>(va.a, f, V.hits, V.target, V.rgb);
}

// Checks the arguments shared by all views, brings the distances up to date on
// st and fills the shared part of `a` (its frame from `cam`).
vt_status prepare_shade(vt_ctx* ctx, const vt_world* world, const vt_camera* cam, const vt_shade_inputs* in, AdjArgs& a,
                        cudaStream_t st) {
    if (!ctx) return VT_ERR_ARG;
    if (!world || !cam || !in || !in->d_palette) return fail(ctx, VT_ERR_ARG, "null shading argument");
    if (world->ctx != ctx) return fail(ctx, VT_ERR_ARG, "world belongs to another context");
    const float len2 = (in->sun[0] * in->sun[0] + in->sun[1] * in->sun[1]) + in->sun[2] * in->sun[2];
    if (!(len2 > 0.0f)) return fail(ctx, VT_ERR_ARG, "sun direction must be nonzero");
    {
        vt_status s = update_distances(const_cast<vt_world*>(world), st);
        if (s) return s;
    }
    vt_params p;
    vt_params_default(&p);
    for (int j = 0; j < 3; ++j) p.sun_dir[j] = in->sun[j];
    a.w = world->view();
    a.f = make_frame(cam, &p);
    a.pal = in->d_palette;
    a.alb = in->d_albedo;
    for (int j = 0; j < 3; ++j) {
        a.sun[j] = in->sun[j];
        a.sun_n[j] = a.f.sun_n[j];
    }
    a.inv_len = 1.0f / sqrtf(len2);
    a.ka = in->ambient;
    a.kd = in->diffuse;
    a.shadow_steps = in->shadow_max_steps;
    return VT_OK;
}

bool camera_size_ok(const vt_camera* cam) {
    return cam->width > 0 && cam->height > 0 && cam->width <= kMaxImageSide && cam->height <= kMaxImageSide;
}

constexpr size_t kShadeSmem = 776 * sizeof(float);

vt_status launch_shade(vt_ctx* ctx, const vt_world* world, const vt_camera* cam, const vt_hit* d_hits,
                       const vt_shade_inputs* in, AdjArgs a, bool bwd, cudaStream_t st) {
    if (!ctx) return VT_ERR_ARG;
    if (!cam || !d_hits) return fail(ctx, VT_ERR_ARG, "null shading argument");
    if (!camera_size_ok(cam)) return fail(ctx, VT_ERR_ARG, "camera size out of range (1..32768)");
    vt_status s = prepare_shade(ctx, world, cam, in, a, st);
    if (s) return s;
    a.hits = reinterpret_cast<const uint4*>(d_hits);
    const dim3 grid((cam->width + 15) / 16, (cam->height + 15) / 16);
    if (bwd) k_shade<true><<<grid, kAdjBlock, kShadeSmem, st>>>(a);
    else k_shade<false><<<grid, kAdjBlock, kShadeSmem, st>>>(a);
    VT_CUDA(ctx, cudaGetLastError());
    return VT_OK;
}

// n views in launches of up to kMaxViews (the loss and gradients of
// `a` are shared; each view has its hits and its target or output image).
vt_status launch_shade_views(vt_ctx* ctx, const vt_world* world, int32_t n, const vt_camera* cams,
                             const vt_hit* const* d_hits, const vt_shade_inputs* in, const float* const* d_targets,
                             float* const* d_rgb, AdjArgs a, bool bwd, cudaStream_t st) {
    for (int v = 0; v < n; ++v) {
        if (!d_hits[v] || (bwd ? !d_targets[v] : !d_rgb[v])) return fail(ctx, VT_ERR_ARG, "null view buffer");
        if (!camera_size_ok(&cams[v])) return fail(ctx, VT_ERR_ARG, "camera size out of range (1..32768)");
    }
    vt_status s = prepare_shade(ctx, world, &cams[0], in, a, st);
    if (s) return s;
    ViewsArgs va;
    std::memset(&va, 0, sizeof(va));
    va.a = a;
    for (int v0 = 0; v0 < n; v0 += kMaxViews) {
        const int nv = n - v0 < kMaxViews ? n - v0 : kMaxViews;
        int gw = 0, gh = 0;
        for (int i = 0; i < nv; ++i) {
            const vt_camera& c = cams[v0 + i];
            ViewP& V = va.v[i];
            for (int j = 0; j < 3; ++j) V.pos[j] = c.pos[j];
            std::memcpy(V.view, c.view, sizeof(V.view));
            V.tan_half_fov = c.tan_half_fov;
            V.width = c.width;
            V.height = c.height;
            V.hits = reinterpret_cast<const uint4*>(d_hits[v0 + i]);
            V.target = bwd ? d_targets[v0 + i] : nullptr;
            V.rgb = bwd ? nullptr : d_rgb[v0 + i];
            gw = c.width > gw ? c.width : gw;
            gh = c.height > gh ? c.height : gh;
        }
        const dim3 grid((gw + 15) / 16, (gh + 15) / 16, nv);
        if (bwd) k_shade_views<true><<<grid, kAdjBlock, kShadeSmem, st>>>(va);
        else k_shade_views<false><<<grid, kAdjBlock, kShadeSmem, st>>>(va);
        VT_CUDA(ctx, cudaGetLastError());
    }
    return VT_OK;
}

}  // namespace

}  // namespace vt

using namespace vt;

extern "C" {

vt_status vt_shade_forward(vt_ctx* ctx, const vt_world* world, const vt_camera* cam, const vt_hit* d_hits,
                           const vt_shade_inputs* in, const uint8_t* d_vis_in, uint8_t* d_vis_out, float* d_rgb,
                           vt_stream stream) {
    if (!ctx) return VT_ERR_ARG;
    if (!d_rgb) return fail(ctx, VT_ERR_ARG, "null output image");
    AdjArgs a;
    std::memset(&a, 0, sizeof(a));
    a.vis_in = d_vis_in;
    a.vis_out = d_vis_out;
    a.rgb = d_rgb;
    return launch_shade(ctx, world, cam, d_hits, in, a, false, (cudaStream_t)stream);
}

vt_status vt_shade_backward(vt_ctx* ctx, const vt_world* world, const vt_camera* cam, const vt_hit* d_hits,
                            const vt_shade_inputs* in, const float* d_target, float* d_loss, float* d_grad_palette,
                            float* d_grad_albedo, float* d_grad_sun, vt_stream stream) {
    if (!ctx) return VT_ERR_ARG;
    if (!d_target || !d_loss || !d_grad_palette || !d_grad_sun)
        return fail(ctx, VT_ERR_ARG, "null target, loss or gradient buffer");
    AdjArgs a;
    std::memset(&a, 0, sizeof(a));
    a.target = d_target;
    a.loss = d_loss;
    a.gpal = d_grad_palette;
    a.galb = d_grad_albedo;
    a.gsun = d_grad_sun;
    return launch_shade(ctx, world, cam, d_hits, in, a, true, (cudaStream_t)stream);
}

vt_status vt_shade_forward_views(vt_ctx* ctx, const vt_world* world, int32_t n, const vt_camera* cams,
                                 const vt_hit* const* d_hits, const vt_shade_inputs* in, float* const* d_rgb,
                                 vt_stream stream) {
    if (!ctx) return VT_ERR_ARG;
    if (n < 0 || (n > 0 && (!cams || !d_hits || !d_rgb))) return fail(ctx, VT_ERR_ARG, "bad view lists");
    if (n == 0) return VT_OK;
    AdjArgs a;
    std::memset(&a, 0, sizeof(a));
    return launch_shade_views(ctx, world, n, cams, d_hits, in, nullptr, d_rgb, a, false, (cudaStream_t)stream);
}

vt_status vt_shade_backward_views(vt_ctx* ctx, const vt_world* world, int32_t n, const vt_camera* cams,
                                  const vt_hit* const* d_hits, const vt_shade_inputs* in, const float* const* d_targets,
                                  float* d_loss, float* d_grad_palette, float* d_grad_albedo, float* d_grad_sun,
                                  vt_stream stream) {
    if (!ctx) return VT_ERR_ARG;
    if (n < 0 || (n > 0 && (!cams || !d_hits || !d_targets))) return fail(ctx, VT_ERR_ARG, "bad view lists");
    if (!d_loss || !d_grad_palette || !d_grad_sun) return fail(ctx, VT_ERR_ARG, "null loss or gradient buffer");
    if (n == 0) return VT_OK;
    // One launch for up to 16 views (blockIdx.z = view) instead of one per
    // view on concurrent streams.
    AdjArgs a;
    std::memset(&a, 0, sizeof(a));
    a.loss = d_loss;
    a.gpal = d_grad_palette;
    a.galb = d_grad_albedo;
    a.gsun = d_grad_sun;
    return launch_shade_views(ctx, world, n, cams, d_hits, in, d_targets, nullptr, a, true, (cudaStream_t)stream);
}
}  // extern "C"
