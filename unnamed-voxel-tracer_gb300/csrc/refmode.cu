// refmode.cu -- the reference's world format and frame on the GPU ("mode R").
//
// Restates, operation for operation, traceMap (map.glsl:83-168) with its
// fractional in-cell position, empty-voxel skipping (stepSize 3), the 0.999
// snap and the 192/48 step caps, together with the rest of the reference's
// frame: the primary pass (primary.comp.glsl:23-69), the shadow pass with
// traceEntities (secondary.comp.glsl:18-51, map.glsl:172-201) and the blit
// (blit.fragment.glsl:15-35), fused into one thread per pixel.  Compiled with
// --fmad=false, so every float operation rounds as written, and the records
// match the CPU restatement (oracle) bit for bit; only the two powf calls of
// SkyDome2 and the vignette may round differently.
//
// Device layout: the 64^3 brick-index table and the brick pool as uploaded;
// the 256^3 atlas stored model-major (slot s = (ty&31) + 32*(ty>>5&31) +
// 1024*(ty>>10&31), texel x + 8*(y + 8*z)), the same texels in the order a
// ray reads them.
#include <cmath>
#include <cstring>
#include <vector>

#include "shade.cuh"
#include "vt_internal.h"

struct vt_brickmap {
    vt_ctx* ctx = nullptr;
    unsigned* d_chunks = nullptr;  // 64^3
    unsigned* d_data = nullptr;    // nbricks * 512
    size_t nbricks = 0;
    unsigned* d_atlas = nullptr;   // 32768 * 512
    int next_model = 0;
};

namespace vt {

vt_status parse_vox(const uint8_t* bytes, size_t n, std::vector<std::vector<uint32_t>>& models);

namespace {

constexpr int kModels = 32768;
constexpr int kRefBlock = 256;

struct RefView {
    const unsigned* chunks;
    const unsigned* data;
    unsigned long long ndata;
    const unsigned* atlas;
};

struct RefHit {
    unsigned data;
    float hit_pos[3];
    float normal[3];
};

__device__ __forceinline__ unsigned ref_chunk_flags(const RefView& w, int x, int y, int z) {  // map.glsl:31-36
    if (x < 0 || y < 0 || z < 0 || x >= 64 || y >= 64 || z >= 64) return 0u;
    return __ldg(w.chunks + x + 64 * (y + z * 64));
}

__device__ __forceinline__ unsigned ref_get_voxel(const RefView& w, int x, int y, int z) {  // map.glsl:38-47
    const unsigned blk = ref_chunk_flags(w, x >> 3, y >> 3, z >> 3);
    if (blk > 0u) {
        const unsigned long long idx =
            (unsigned long long)(blk - 1u) * 512ull + (unsigned long long)((x % 8) + ((z % 8) * 8 + (y % 8)) * 8);
        if (idx >= w.ndata) return 0u;  // outside the uploaded pool reads as empty
        return __ldg(w.data + idx);
    }
    return 0u;
}

__device__ __forceinline__ unsigned ref_get_subvoxel(const RefView& w, unsigned mdl, int x, int y, int z) {  // map.glsl:57-60
    const unsigned slot = (mdl & 31u) + 32u * ((mdl / 32u) & 31u) + 1024u * ((mdl / 1024u) & 31u);
    return __ldg(w.atlas + (size_t)slot * 512u + (unsigned)(x + 8 * (y + 8 * z)));
}

__device__ __forceinline__ unsigned f2u(float x) { return x <= 0.0f ? 0u : (unsigned)x; }

// traceMap (map.glsl:83-168).
__device__ void trace_map(const RefView& w, const float o[3], const float din[3], int max_steps, RefHit& out) {
    float d[3] = {din[0], din[1], din[2]};
#pragma unroll
    for (int i = 0; i < 3; ++i)
        if (d[i] == 0.0f) d[i] = 0.001f;
    const int bounds = 8 * 512;
    int sgn[3], pos[3];
    float inv[3];
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        sgn[i] = d[i] > 0.0f ? 1 : (d[i] < 0.0f ? -1 : 0);
        pos[i] = (1 + sgn[i]) >> 1;
        inv[i] = 1.0f / d[i];
    }
    int minIdx = 0;
    float t[3] = {1.0f, 1.0f, 1.0f};
    int g[3];
    float wc[3];
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        g[i] = (int)(o[i] * 8.0f);
        wc[i] = o[i] * 8.0f - (float)g[i];
    }
    int stepSize = 0;
    for (int step = 0; step < max_steps; ++step) {
        if (g[0] >= bounds || g[1] >= bounds || g[2] >= bounds || g[0] < 0 || g[1] < 0 || g[2] < 0) break;
        int pi[3];
#pragma unroll
        for (int i = 0; i < 3; ++i) pi[i] = (int)((unsigned)g[i] + f2u(wc[i]));
        const unsigned block = ref_get_voxel(w, pi[0] >> 3, pi[1] >> 3, pi[2] >> 3);
        if (block != 0u) {
            const unsigned sub = ref_get_subvoxel(w, block & 0xFFFFFFFu, pi[0] % 8, pi[1] % 8, pi[2] % 8);
            if (sub != 0u) {
                const int faceId = minIdx == 0 ? (-pos[0] + 2) : (minIdx == 1 ? (-pos[1] + 4) : (-pos[2] + 6));
                out.data = sub;
#pragma unroll
                for (int i = 0; i < 3; ++i) {
                    out.hit_pos[i] = (float)g[i] + wc[i];
                    out.normal[i] = 0.0f;
                }
                // normals[] (map.glsl:72-79): faceId 1..6 -> -x, +x, -y, +y, -z, +z
                const int ax = (faceId - 1) >> 1;
                const float nv = ((faceId - 1) & 1) ? 1.0f : -1.0f;
                out.normal[0] = ax == 0 ? nv : 0.0f;
                out.normal[1] = ax == 1 ? nv : 0.0f;
                out.normal[2] = ax == 2 ? nv : 0.0f;
                return;
            } else if (stepSize != 0) {
#pragma unroll
                for (int i = 0; i < 3; ++i) {
                    g[i] += (int)wc[i];
                    wc[i] = wc[i] - floorf(wc[i]);
                }
                stepSize = 0;
            }
        } else if (stepSize != 3) {
#pragma unroll
            for (int i = 0; i < 3; ++i) {
                wc[i] += (float)(g[i] & 7);
                g[i] -= g[i] & 7;
            }
            stepSize = 3;
        }
#pragma unroll
        for (int i = 0; i < 3; ++i) t[i] = ((float)(pos[i] << stepSize) - wc[i]) * inv[i];
        minIdx = t[0] < t[1] ? (t[0] < t[2] ? 0 : 2) : (t[1] < t[2] ? 1 : 2);
        const float tm = minIdx == 0 ? t[0] : (minIdx == 1 ? t[1] : t[2]);
#pragma unroll
        for (int i = 0; i < 3; ++i) {
            if (i == minIdx) g[i] += (int)((unsigned)sgn[i] << stepSize);
            wc[i] += d[i] * tm;
        }
#pragma unroll
        for (int i = 0; i < 3; ++i)
            if (i == minIdx) wc[i] = (float)((1 - pos[i]) << stepSize) * 0.999f;
    }
    out.data = 0u;
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        out.hit_pos[i] = -1.0f;
        out.normal[i] = 0.0f;
    }
}

__device__ __forceinline__ float fmin_g(float a, float b) { return b < a ? b : a; }
__device__ __forceinline__ float fmax_g(float a, float b) { return a < b ? b : a; }

__device__ __forceinline__ void aabb(const float o[3], const float d[3], const float lo[3], const float hi[3],
                                     float& tn, float& tf) {  // map.glsl:21-29
    float t1[3], t2[3];
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        const float a = (lo[i] - o[i]) / d[i];
        const float b = (hi[i] - o[i]) / d[i];
        t1[i] = fmin_g(a, b);
        t2[i] = fmax_g(a, b);
    }
    tn = fmax_g(fmax_g(t1[0], t1[1]), t1[2]);
    tf = fmin_g(fmin_g(t2[0], t2[1]), t2[2]);
}

__device__ __forceinline__ float dist3(const float a[3], const float b[3]) {
    const float x = a[0] - b[0], y = a[1] - b[1], z = a[2] - b[2];
    return sqrtf((x * x + y * y) + z * z);
}

// traceEntities (map.glsl:172-201): true when one of the five boxes is hit.
__device__ bool trace_entities(const float o[3], const float d[3], float max_distance) {
    const float P[5][3] = {{256.f, 21.f, 256.f}, {251.f, 21.f, 259.f}, {253.f, 21.f, 256.f},
                           {251.f, 21.f, 256.f}, {257.f, 21.f, 261.f}};
    float prev = __int_as_float(0x7f800000);  // 1.0 / 0.0
    int id = -1;
    for (int i = 0; i < 5; ++i) {
        if (dist3(o, P[i]) >= max_distance) continue;
        const float hi[3] = {P[i][0] + 1.0f, P[i][1] + 1.0f, P[i][2] + 1.0f};
        float tn, tf;
        aabb(o, d, P[i], hi, tn, tf);
        if (tf >= tn && prev >= tf) {
            id = i;
            prev = tf;
        }
    }
    if (id < 0) return false;
    const float hi[3] = {P[id][0] + 1.0f, P[id][1] + 1.0f, P[id][2] + 1.0f};
    float tn, tf;
    aabb(o, d, P[id], hi, tn, tf);
    return tf >= tn;
}

__constant__ float kSun[3] = {7.52185881e-01f, 6.58950984e-01f, 7.52185881e-01f};  // camera.glsl:8

// SkyDome2 (camera.glsl:11-19) as written, with powf.
__device__ void sky_ref(const float rd[3], float out[4]) {
    float sn[3], rn[3];
    normalize3(kSun, sn);
    normalize3(rd, rn);
    const float s = clampf(dot3(sn, rn), 0.0f, 1.2f);
    const float dy = rd[1] * 0.2f;
    const float p8 = powf(s, 8.0f), p3 = powf(s, 3.0f);
    out[0] = ((0.6f - dy * 1.0f) + (0.15f * 0.5f)) + (0.4f * 1.0f) * p8 + 0.2f * p3;
    out[1] = ((0.71f - dy * 0.5f) + (0.15f * 0.5f)) + (0.4f * 0.6f) * p8 + 0.08f * p3;
    out[2] = ((0.75f - dy * 1.0f) + (0.15f * 0.5f)) + (0.4f * 0.1f) * p8 + 0.04f * p3;
    out[3] = 1.0f;
}

__device__ __forceinline__ unsigned pack8(const float c[4]) {
    return unorm8(c[0]) | (unorm8(c[1]) << 8) | (unorm8(c[2]) << 16) | (unorm8(c[3]) << 24);
}

__device__ __forceinline__ void unpack8(unsigned p, float c[4]) {
#pragma unroll
    for (int j = 0; j < 4; ++j) c[j] = (float)((p >> (8 * j)) & 255u) / 255.0f;
}

struct RefFrame {
    float pos[4];
    float view[16];
    float tan_half;  // tanf(fov / 2), computed on the host
    int width, height;
};

// primary.comp.glsl:35-43 from the scaled ray UV (before the fov factor):
// the view ray, clipped to the map box and traced with `steps`.
__device__ void ray_ref(const RefView& w, const RefFrame& f, float ux, float uy, int steps, float dir[3], RefHit& h) {
    ux *= f.tan_half;
    uy *= f.tan_half;
    const float v[4] = {ux, uy, 1.0f, 1.0f};
    float q[4];
#pragma unroll
    for (int i = 0; i < 4; ++i)
        q[i] = ((f.view[0 * 4 + i] * v[0] + f.view[1 * 4 + i] * v[1]) + f.view[2 * 4 + i] * v[2]) + f.view[3 * 4 + i] * v[3];
    const float len = sqrtf(((q[0] * q[0] + q[1] * q[1]) + q[2] * q[2]) + q[3] * q[3]);
    float o[3], t1[3];
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        dir[i] = q[i] / len;
        o[i] = f.pos[i];
    }
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        const float a = (0.0f - o[i]) / dir[i];
        const float b = (512.0f - o[i]) / dir[i];
        t1[i] = fmin_g(a, b);
    }
    const float tnear = fmax_g(fmax_g(t1[0], t1[1]), t1[2]);
    const float s = fmax_g(tnear, 0.0f);
    float start[3];
#pragma unroll
    for (int i = 0; i < 3; ++i) start[i] = (o[i] + dir[i] * s) - 0.001f;
    trace_map(w, start, dir, steps, h);
}

// primary.comp.glsl:31-43.
__device__ void primary_ref(const RefView& w, const RefFrame& f, int px, int py, float dir[3], RefHit& h) {
    const float ux = (float)px / (float)f.width * 2.0f - 1.0f;
    float uy = (float)py / (float)f.height * 2.0f - 1.0f;
    uy *= (float)f.height / (float)f.width;
    ray_ref(w, f, ux, uy, 192, dir, h);
}

// terrain_edit.comp.glsl:11-17: the pick ray through the view centre (UV 0),
// traced with 64 steps; then the edit its commented-out tail describes
// (:19-24): edit_mode > 0 writes Voxel{ty = edit_mode - 1, is_solid} in
// front of the hit face, edit_mode == 0 clears the hit voxel, both through
// map_setVoxel (map.glsl:49-55), which drops writes into chunks without a
// brick.  edit_mode < 0 only picks.  One thread.
__global__ void k_brickmap_edit(RefView w, unsigned* data, RefFrame f, int edit_mode, uint4* __restrict__ out) {
    float dir[3];
    RefHit h;
    ray_ref(w, f, 0.0f, 0.0f, 64, dir, h);
    if (out) {
        out[0] = make_uint4(h.data, __float_as_uint(h.hit_pos[0]), __float_as_uint(h.hit_pos[1]), __float_as_uint(h.hit_pos[2]));
        out[1] = make_uint4(__float_as_uint(h.normal[0]), __float_as_uint(h.normal[1]), __float_as_uint(h.normal[2]), 0u);
    }
    if (edit_mode < 0 || h.data == 0u) return;
    int p[3];
    unsigned voxel;
    if (edit_mode > 0) {
#pragma unroll
        for (int i = 0; i < 3; ++i) p[i] = (int)(h.hit_pos[i] + h.normal[i]) >> 3;
        voxel = (1u << 28) + (unsigned)edit_mode - 1u;
    } else {
#pragma unroll
        for (int i = 0; i < 3; ++i) p[i] = (int)h.hit_pos[i] >> 3;
        voxel = 0u;
    }
    const unsigned blk = ref_chunk_flags(w, p[0] >> 3, p[1] >> 3, p[2] >> 3);
    if (blk == 0u) return;
    const unsigned long long idx =
        (unsigned long long)(blk - 1u) * 512ull + (unsigned long long)((p[0] % 8) + ((p[2] % 8) * 8 + (p[1] % 8)) * 8);
    if (idx < w.ndata) data[idx] = voxel;
}

__global__ void __launch_bounds__(kRefBlock) k_render_reference(RefView w, RefFrame f, uint4* __restrict__ out) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int px = blockIdx.x * 16 + (warp & 1) * 8 + (lane & 7);
    const int py = blockIdx.y * 16 + (warp >> 1) * 4 + (lane >> 3);
    if (px >= f.width || py >= f.height) return;
    float dir[3];
    RefHit h;
    primary_ref(w, f, px, py, dir, h);
    unsigned albedo, normal, illum;
    float position[4];
    if (h.data != 0u) {
        albedo = h.data;
        const float n4[4] = {h.normal[0], h.normal[1], h.normal[2], 1.0f};
        normal = pack8(n4);
#pragma unroll
        for (int k = 0; k < 3; ++k) position[k] = ceilf(h.hit_pos[k]) / 8.0f;
        position[3] = 1.0f;
    } else {
        float s4[4];
        sky_ref(dir, s4);
        albedo = pack8(s4);
        normal = 0xFFFFFFFFu;
#pragma unroll
        for (int k = 0; k < 4; ++k) position[k] = -1.0f;
    }
    // secondary.comp.glsl
    if (position[0] < 0.0f || position[1] < 0.0f || position[2] < 0.0f) {
        illum = 0u;
    } else {
        float nq[4];
        unpack8(normal, nq);
        float ro[3];
#pragma unroll
        for (int k = 0; k < 3; ++k) ro[k] = position[k] + nq[k] * 0.001f;
        const float sun[3] = {kSun[0], kSun[1], kSun[2]};
        RefHit sh;
        trace_map(w, ro, sun, 48, sh);
        const float hp8[3] = {sh.hit_pos[0] / 8.0f, sh.hit_pos[1] / 8.0f, sh.hit_pos[2] / 8.0f};
        const bool ent = trace_entities(ro, sun, dist3(ro, hp8));
        const float il[4] = {sun[0], sun[1], sun[2], (ent || sh.data != 0u) ? -0.3f : 0.3f};
        illum = pack8(il);
    }
    // blit.fragment.glsl
    const float u = ((float)px + 0.5f) / (float)f.width, v = ((float)py + 0.5f) / (float)f.height;
    float col[4], il[4], s4[4];
    unpack8(albedo, col);
    unpack8(illum, il);
    sky_ref(il, s4);
#pragma unroll
    for (int k = 0; k < 4; ++k) col[k] = col[k] + il[3] * s4[k];
    const float cu = u - 0.5f, cv = v - 0.5f;
    if (sqrtf(cu * cu + cv * cv) <= 0.002f) {
        const float mixc[4] = {1.0f, 1.0f, 1.0f, 0.4f};
#pragma unroll
        for (int k = 0; k < 4; ++k) col[k] = col[k] * (1.0f - 0.5f) + mixc[k] * 0.5f;
    }
    const float g = powf((u * (1.0f - u)) * (v * (1.0f - v)) * 15.0f, 0.6f * 0.3f);
#pragma unroll
    for (int k = 0; k < 4; ++k) col[k] = g * col[k];
    const size_t p = (size_t)py * f.width + px;
    out[2 * p] = make_uint4(albedo, normal, illum, pack8(col));
    out[2 * p + 1] = make_uint4(__float_as_uint(position[0]), __float_as_uint(position[1]),
                                __float_as_uint(position[2]), __float_as_uint(position[3]));
}

__global__ void __launch_bounds__(kRefBlock) k_trace_map(RefView w, const float* __restrict__ origins,
                                                        const float* __restrict__ dirs, int n, int max_steps,
                                                        uint4* __restrict__ out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float o[3], d[3];
#pragma unroll
    for (int j = 0; j < 3; ++j) {
        o[j] = origins[3 * i + j];
        d[j] = dirs[3 * i + j];
    }
    RefHit h;
    trace_map(w, o, d, max_steps, h);
    out[2 * i] = make_uint4(h.data, __float_as_uint(h.hit_pos[0]), __float_as_uint(h.hit_pos[1]),
                            __float_as_uint(h.hit_pos[2]));
    out[2 * i + 1] = make_uint4(__float_as_uint(h.normal[0]), __float_as_uint(h.normal[1]),
                                __float_as_uint(h.normal[2]), 0u);
}

RefView view_of(const vt_brickmap* bm) {
    RefView v;
    v.chunks = bm->d_chunks;
    v.data = bm->d_data;
    v.ndata = (unsigned long long)bm->nbricks * 512ull;
    v.atlas = bm->d_atlas;
    return v;
}

void free_brickmap(vt_brickmap* bm) {
    if (bm->d_chunks) vt::dev_free(bm->d_chunks);
    if (bm->d_data) vt::dev_free(bm->d_data);
    if (bm->d_atlas) vt::dev_free(bm->d_atlas);
    delete bm;
}

}  // namespace

}  // namespace vt

using namespace vt;

extern "C" {

vt_status vt_brickmap_create(vt_ctx* ctx, vt_brickmap** out) {
    if (!ctx) return VT_ERR_ARG;
    if (!out) return fail(ctx, VT_ERR_ARG, "null output");
    *out = nullptr;
    vt_brickmap* bm = new (std::nothrow) vt_brickmap();
    if (!bm) return fail(ctx, VT_ERR_OOM, "host allocation failed");
    bm->ctx = ctx;
    cudaError_t e;
    if ((e = vt::dev_alloc(&bm->d_chunks, 64 * 64 * 64 * sizeof(unsigned))) != cudaSuccess ||
        (e = vt::dev_alloc(&bm->d_atlas, (size_t)kModels * 512 * sizeof(unsigned))) != cudaSuccess ||
        (e = cudaMemset(bm->d_chunks, 0, 64 * 64 * 64 * sizeof(unsigned))) != cudaSuccess ||
        (e = cudaMemset(bm->d_atlas, 0, (size_t)kModels * 512 * sizeof(unsigned))) != cudaSuccess) {
        free_brickmap(bm);
        return check_cuda(ctx, e, "brickmap allocation");
    }
    *out = bm;
    return VT_OK;
}

vt_status vt_brickmap_destroy(vt_brickmap* bm) {
    if (!bm) return VT_ERR_ARG;
    cudaDeviceSynchronize();
    free_brickmap(bm);
    return VT_OK;
}

vt_status vt_brickmap_upload(vt_brickmap* bm, const uint32_t* h_chunks, const uint32_t* h_bricks, size_t nbricks) {
    if (!bm) return VT_ERR_ARG;
    if (!h_chunks || (nbricks && !h_bricks)) return fail(bm->ctx, VT_ERR_ARG, "null map arrays");
    if (nbricks > (1u << 24)) return fail(bm->ctx, VT_ERR_ARG, "brick pool larger than 2^24 bricks");
    VT_CUDA(bm->ctx, cudaMemcpy(bm->d_chunks, h_chunks, 64 * 64 * 64 * sizeof(unsigned), cudaMemcpyHostToDevice));
    if (bm->d_data) {
        vt::dev_free(bm->d_data);
        bm->d_data = nullptr;
        bm->nbricks = 0;
    }
    if (nbricks) {
        VT_CUDA(bm->ctx, vt::dev_alloc(&bm->d_data, nbricks * 512 * sizeof(unsigned)));
        VT_CUDA(bm->ctx, cudaMemcpy(bm->d_data, h_bricks, nbricks * 512 * sizeof(unsigned), cudaMemcpyHostToDevice));
    }
    bm->nbricks = nbricks;
    return VT_OK;
}

vt_status vt_brickmap_set_model(vt_brickmap* bm, int32_t slot, const uint32_t* h_texels) {
    if (!bm) return VT_ERR_ARG;
    if (!h_texels || slot < 0 || slot >= kModels) return fail(bm->ctx, VT_ERR_ARG, "model slot out of range");
    VT_CUDA(bm->ctx, cudaMemcpy(bm->d_atlas + (size_t)slot * 512, h_texels, 512 * sizeof(unsigned),
                                cudaMemcpyHostToDevice));
    return VT_OK;
}

vt_status vt_brickmap_load_vox(vt_brickmap* bm, const uint8_t* h_bytes, size_t nbytes, int32_t* models_loaded) {
    if (!bm) return VT_ERR_ARG;
    if (!h_bytes) return fail(bm->ctx, VT_ERR_ARG, "null file bytes");
    std::vector<std::vector<uint32_t>> models;
    if (parse_vox(h_bytes, nbytes, models) != VT_OK) return fail(bm->ctx, VT_ERR_FORMAT, "not a MagicaVoxel file with an RGBA palette");
    if (bm->next_model + (int)models.size() > kModels) return fail(bm->ctx, VT_ERR_ARG, "model atlas full");
    for (const auto& m : models) {
        vt_status s = vt_brickmap_set_model(bm, bm->next_model, m.data());
        if (s) return s;
        ++bm->next_model;
    }
    if (models_loaded) *models_loaded = (int32_t)models.size();
    return VT_OK;
}

vt_status vt_trace_map(vt_ctx* ctx, const vt_brickmap* bm, const float* d_origins, const float* d_dirs, int32_t n,
                       int32_t max_steps, vt_ref_hit* d_out, vt_stream stream) {
    if (!ctx) return VT_ERR_ARG;
    if (!bm || !d_origins || !d_dirs || !d_out || n < 0) return fail(ctx, VT_ERR_ARG, "bad trace_map arguments");
    if (n == 0) return VT_OK;
    k_trace_map<<<(n + kRefBlock - 1) / kRefBlock, kRefBlock, 0, (cudaStream_t)stream>>>(
        view_of(bm), d_origins, d_dirs, n, max_steps, reinterpret_cast<uint4*>(d_out));
    VT_CUDA(ctx, cudaGetLastError());
    return VT_OK;
}

vt_status vt_brickmap_download(vt_brickmap* bm, uint32_t* h_chunks, uint32_t* h_bricks, size_t nbricks) {
    if (!bm) return VT_ERR_ARG;
    if (!h_chunks || (nbricks && !h_bricks) || nbricks > bm->nbricks)
        return fail(bm->ctx, VT_ERR_ARG, "null output or more bricks than uploaded");
    VT_CUDA(bm->ctx, cudaDeviceSynchronize());
    VT_CUDA(bm->ctx, cudaMemcpy(h_chunks, bm->d_chunks, 64u * 64u * 64u * 4u, cudaMemcpyDeviceToHost));
    if (nbricks) VT_CUDA(bm->ctx, cudaMemcpy(h_bricks, bm->d_data, nbricks * 512u * 4u, cudaMemcpyDeviceToHost));
    return VT_OK;
}

vt_status vt_brickmap_edit(vt_ctx* ctx, vt_brickmap* bm, const vt_camera* cam, int32_t edit_mode, vt_ref_hit* d_out,
                           vt_stream stream) {
    if (!ctx) return VT_ERR_ARG;
    if (!bm || !cam) return fail(ctx, VT_ERR_ARG, "null brickmap or camera");
    if (edit_mode < -1 || edit_mode > (1 << 28)) return fail(ctx, VT_ERR_ARG, "edit_mode must be in [-1, 2^28]");
    RefFrame f;
    for (int i = 0; i < 4; ++i) f.pos[i] = cam->pos[i];
    std::memcpy(f.view, cam->view, sizeof(f.view));
    f.tan_half = 1.0f;  // the pick ray has UV 0 and no fov factor (terrain_edit.comp.glsl:12-14)
    f.width = 1;
    f.height = 1;
    k_brickmap_edit<<<1, 1, 0, (cudaStream_t)stream>>>(view_of(bm), bm->d_data, f, edit_mode, reinterpret_cast<uint4*>(d_out));
    VT_CUDA(ctx, cudaGetLastError());
    return VT_OK;
}

vt_status vt_render_reference(vt_ctx* ctx, const vt_brickmap* bm, const vt_camera* cam, vt_ref_pixel* d_out,
                              vt_stream stream) {
    if (!ctx) return VT_ERR_ARG;
    if (!bm || !cam || !d_out) return fail(ctx, VT_ERR_ARG, "null brickmap, camera or output");
    if (cam->width <= 0 || cam->height <= 0 || cam->width > kMaxImageSide || cam->height > kMaxImageSide)
        return fail(ctx, VT_ERR_ARG, "camera size out of range (1..32768)");
    RefFrame f;
    for (int i = 0; i < 4; ++i) f.pos[i] = cam->pos[i];
    std::memcpy(f.view, cam->view, sizeof(f.view));
    f.tan_half = tanf(cam->fov / 2.0f);  // primary.comp.glsl:36, on the host's libm
    f.width = cam->width;
    f.height = cam->height;
    const dim3 grid((cam->width + 15) / 16, (cam->height + 15) / 16);
    k_render_reference<<<grid, kRefBlock, 0, (cudaStream_t)stream>>>(view_of(bm), f, reinterpret_cast<uint4*>(d_out));
    VT_CUDA(ctx, cudaGetLastError());
    return VT_OK;
}

}  // extern "C"
