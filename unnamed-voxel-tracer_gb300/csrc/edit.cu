// edit.cu -- the pick ray and voxel edits of a mode-P world, on the device.
//
// The reference's editing shader (terrain_edit.comp.glsl:11-24) traces one
// ray through the centre of the view and then sets the voxel in front of the
// hit face (place) or the hit voxel itself (remove) with map_setVoxel
// (map.glsl:49-55).  Here one block of 512 threads does the same on the
// mode-P world: thread 0 traces, the block then writes the material, the
// brick word and the chunk's coarse bit (as k_set_voxel does), and records
// the edited voxel in device memory, from where the distance passes that
// follow on the stream update the empty-space distances around it.  Nothing
// goes back to the host between the pick and the edit.
#include "render_pixel.cuh"
#include "vt_internal.h"

namespace vt {

namespace {

struct PickRay {
    float pos[3];
    float view[16];
};

// The primary ray of ray UV (0, 0) (primary.comp.glsl:31-39 with
// pixelCoords / size = 1/2): the same arithmetic as primary_ray with u = v = 0.
__device__ __forceinline__ void center_ray(const PickRay& f, float o[3], float d[3]) {
    const float u = 0.0f, v = 0.0f;
    float q[3];
#pragma unroll
    for (int j = 0; j < 3; ++j) q[j] = ((u * f.view[0 * 4 + j] + v * f.view[1 * 4 + j]) + f.view[2 * 4 + j]) + f.view[3 * 4 + j];
    const float len = __fsqrt_rn((q[0] * q[0] + q[1] * q[1]) + q[2] * q[2]);
#pragma unroll
    for (int j = 0; j < 3; ++j) {
        d[j] = __fdiv_rn(q[j], len);
        o[j] = f.pos[j];
    }
}

// edit_mode < 0: pick only; 0: clear the hit voxel; 1..255: write material
// edit_mode into the cell in front of the hit face (skipped outside the
// world).  `out` (may be null) receives the pick as a vt_hit record; d_edit
// receives {x, y, z, valid} of the voxel written.
__global__ void __launch_bounds__(512) k_pick_edit(WorldView w, unsigned long long* mask, unsigned char* mats,
                                                   unsigned long long* coarse, PickRay f, int max_steps, int edit_mode,
                                                   uint4* __restrict__ out, int* __restrict__ d_edit) {
    __shared__ int target[4];
    if (threadIdx.x == 0) {
        float o[3], d[3];
        center_ray(f, o, d);
        PRay r;
        pray_init(r, o, d);
        TraceHit h;
        const bool hit = trace_fast<true>(w, w.cdist, r, max_steps, h);
        target[3] = 0;
        if (hit) {
            const int e = h.axis;
            const bool pe = e == 0 ? r.pos[0] : (e == 1 ? r.pos[1] : r.pos[2]);
            const unsigned voxel = (unsigned)h.c[0] + (unsigned)w.dims[0] * ((unsigned)h.c[1] + (unsigned)w.dims[1] * (unsigned)h.c[2]);
            if (out) out[0] = make_uint4(voxel, __float_as_uint(h.t), 0u, (2u * (unsigned)e + (pe ? 0u : 1u)) | (h.mat << 8) | (VT_HIT_PRIMARY << 16));
            if (edit_mode >= 0) {
                int c[3] = {h.c[0], h.c[1], h.c[2]};
                if (edit_mode > 0) c[e] += pe ? -1 : 1;  // the cell the ray left through the hit face
                if (c[0] >= 0 && c[1] >= 0 && c[2] >= 0 && c[0] < w.dims[0] && c[1] < w.dims[1] && c[2] < w.dims[2]) {
                    target[0] = c[0];
                    target[1] = c[1];
                    target[2] = c[2];
                    target[3] = 1;
                }
            }
        } else if (out) {
            out[0] = make_uint4(0xFFFFFFFFu, __float_as_uint(-1.0f), 0u, 0xFFu);
        }
        if (d_edit) {
            d_edit[0] = target[0];
            d_edit[1] = target[1];
            d_edit[2] = target[2];
            d_edit[3] = target[3];
        }
    }
    __syncthreads();
    if (!target[3]) return;
    const int x = target[0], y = target[1], z = target[2];
    const unsigned ci = (unsigned)(x >> 5) + (unsigned)w.cdim[0] * ((unsigned)(y >> 5) + (unsigned)w.cdim[1] * (unsigned)(z >> 5));
    if (threadIdx.x == 0) {
        const unsigned bi = (unsigned)((x >> 2) & 7) | ((unsigned)((y >> 2) & 7) << 3) | ((unsigned)((z >> 2) & 7) << 6);
        const unsigned vb = (unsigned)(x & 3) | ((unsigned)(y & 3) << 2) | ((unsigned)(z & 3) << 4);
        const unsigned wi = ci * 512u + bi;
        mats[(size_t)wi * 64u + vb] = (unsigned char)edit_mode;
        if (edit_mode) mask[wi] |= 1ull << vb;
        else mask[wi] &= ~(1ull << vb);
    }
    __syncthreads();
    const int any = __syncthreads_or(mask[ci * 512u + threadIdx.x] != 0ull);
    if (threadIdx.x == 0) {
        const unsigned long long bit = 1ull << (ci & 63u);
        if (any) atomicOr(coarse + (ci >> 6), bit);
        else atomicAnd(coarse + (ci >> 6), ~bit);
    }
}

PickRay pick_ray(const vt_camera* cam) {
    PickRay f;
    for (int j = 0; j < 3; ++j) f.pos[j] = cam->pos[j];
    for (int j = 0; j < 16; ++j) f.view[j] = cam->view[j];
    return f;
}

vt_status launch_pick(vt_ctx* ctx, vt_world* world, const vt_camera* cam, int32_t max_steps, int32_t edit_mode,
                      vt_hit* d_out, cudaStream_t st) {
    if (!ctx) return VT_ERR_ARG;
    if (!world || !cam) return fail(ctx, VT_ERR_ARG, "null world or camera");
    if (world->ctx != ctx) return fail(ctx, VT_ERR_ARG, "world belongs to another context");
    if (max_steps < 0) return fail(ctx, VT_ERR_ARG, "max_steps must be >= 0");
    if (edit_mode < -1 || edit_mode > 255) return fail(ctx, VT_ERR_ARG, "edit_mode must be in [-1, 255]");
    vt_status s = update_distances(world, st);  // the pick walks the current distances
    if (s) return s;
    k_pick_edit<<<1, 512, 0, st>>>(world->view(), world->d_mask, world->d_mats, world->d_coarse, pick_ray(cam), max_steps,
                                   edit_mode, reinterpret_cast<uint4*>(d_out), edit_mode >= 0 ? world->d_edit : nullptr);
    VT_CUDA(ctx, cudaGetLastError());
    if (edit_mode >= 0) return update_distances_at(world, world->d_edit, st);
    return VT_OK;
}

}  // namespace

}  // namespace vt

using namespace vt;

extern "C" {

vt_status vt_pick(vt_ctx* ctx, vt_world* world, const vt_camera* cam, int32_t max_steps, vt_hit* h_out) {
    if (!ctx) return VT_ERR_ARG;
    if (!h_out) return fail(ctx, VT_ERR_ARG, "null output");
    void* scratch = nullptr;
    vt_status s = ctx_scratch(ctx, sizeof(vt_hit), &scratch);
    if (s) return s;
    cudaStream_t st = ctx->stream;
    s = launch_pick(ctx, world, cam, max_steps, -1, reinterpret_cast<vt_hit*>(scratch), st);
    if (s) return s;
    VT_CUDA(ctx, cudaMemcpyAsync(h_out, scratch, sizeof(vt_hit), cudaMemcpyDeviceToHost, st));
    VT_CUDA(ctx, cudaStreamSynchronize(st));
    return VT_OK;
}

vt_status vt_edit(vt_ctx* ctx, vt_world* world, const vt_camera* cam, int32_t max_steps, int32_t edit_mode,
                  vt_hit* d_out, vt_stream stream) {
    return launch_pick(ctx, world, cam, max_steps, edit_mode, d_out, (cudaStream_t)stream);
}

vt_status vt_world_download_distances(vt_world* w, uint8_t* h_brick, size_t brick_bytes, uint8_t* h_chunk,
                                      size_t chunk_bytes) {
    if (!w) return VT_ERR_ARG;
    const size_t nb = w->nchunks * kBricksPerChunk;
    if (!h_brick || !h_chunk || brick_bytes != kOctants * nb || chunk_bytes != kOctants * w->nchunks)
        return fail(w->ctx, VT_ERR_ARG, "distance download needs 8*nchunks*512 and 8*nchunks bytes");
    cudaStream_t st = w->ctx->stream;
    vt_status s = update_distances(w, st);
    if (s) return s;
    VT_CUDA(w->ctx, cudaMemcpyAsync(h_brick, w->d_bdist, kOctants * nb, cudaMemcpyDeviceToHost, st));
    const size_t cs = cdist_stride((unsigned)w->nchunks);
    for (int o = 0; o < kOctants; ++o)
        VT_CUDA(w->ctx, cudaMemcpyAsync(h_chunk + (size_t)o * w->nchunks, w->d_cdist + (size_t)o * cs, w->nchunks,
                                        cudaMemcpyDeviceToHost, st));
    VT_CUDA(w->ctx, cudaStreamSynchronize(st));
    return VT_OK;
}

}  // extern "C"
