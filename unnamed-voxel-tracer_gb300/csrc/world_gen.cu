// world_gen.cu -- scene generation straight into the device world, and the
// dense download of a world.
//
// The reference generates its terrain on the host and writes it voxel by
// voxel into mapped buffers (src/procgen.zig:6-53 through VoxelBrickmap.set,
// src/engine/voxel.zig:58-61).  Here the same seeded generator as the host's
// vt_gen_world (gen_noise.cuh, shared code) runs on the device and writes the
// chunk layout directly: no dense staging grid, no host traffic.  The bytes
// equal vt_gen_world's for every descriptor.
//
//   k_gen_chunks   one block per chunk, one thread per brick: the chunk's
//                  32x32 column heights in shared memory, then 64 cells per
//                  thread (terrain, water, caves), brick word and coarse bit
//   k_gen_leaves   one block per tree, one thread per leaf cell
//   k_gen_trunks   one thread per tree, after all leaves (see plant_trees on
//                  why the parallel order gives the sequential bytes)
#include "gen_noise.cuh"
#include "vt_internal.h"

namespace vt {

namespace {

__device__ __forceinline__ void cell_addr(const WorldView& w, int x, int y, int z, unsigned* wi, unsigned* vb) {
    const unsigned ci = (unsigned)(x >> 5) + (unsigned)w.cdim[0] * ((unsigned)(y >> 5) + (unsigned)w.cdim[1] * (unsigned)(z >> 5));
    const unsigned bi = (unsigned)((x >> 2) & 7) | ((unsigned)((y >> 2) & 7) << 3) | ((unsigned)((z >> 2) & 7) << 6);
    *wi = ci * 512u + bi;
    *vb = (unsigned)(x & 3) | ((unsigned)(y & 3) << 2) | ((unsigned)(z & 3) << 4);
}

// Marks cell (wi, vb) solid in the brick word and its chunk solid in the
// coarse grid.
__device__ __forceinline__ void mark_solid(unsigned long long* mask, unsigned long long* coarse, unsigned wi, unsigned vb) {
    atomicOr(mask + wi, 1ull << vb);
    const unsigned ci = wi >> 9;
    atomicOr(coarse + (ci >> 6), 1ull << (ci & 63u));
}

__global__ void __launch_bounds__(512) k_gen_chunks(WorldView w, unsigned long long* mask, unsigned char* mats,
                                                    unsigned long long* coarse, vt_gen_desc d) {
    __shared__ int heights[32 * 32];
    const unsigned ci = blockIdx.x;
    const int cx = (int)(ci % (unsigned)w.cdim[0]);
    const int cy = (int)((ci / (unsigned)w.cdim[0]) % (unsigned)w.cdim[1]);
    const int cz = (int)(ci / ((unsigned)w.cdim[0] * (unsigned)w.cdim[1]));
    for (int c = threadIdx.x; c < 32 * 32; c += blockDim.x) {
        const int gx = cx * 32 + (c & 31), gz = cz * 32 + (c >> 5);
        heights[c] = (gx < w.dims[0] && gz < w.dims[2]) ? gen::height_at(&d, gx, gz) : 0;
    }
    __syncthreads();
    const int water = (int)ceil((double)d.water_level);
    const uint64_t cave_seed = gen::stream_seed(d.seed, gen::kCaves);
    const double cave_freq = 1.0 / (double)d.cave_period;
    const int b = threadIdx.x;
    const int bx = b & 7, by = (b >> 3) & 7, bz = b >> 6;
    unsigned long long m = 0ull;
    unsigned packed[16];
    for (int z = 0; z < 4; ++z) {
        for (int y = 0; y < 4; ++y) {
            unsigned word = 0;
            for (int x = 0; x < 4; ++x) {
                const int lx = bx * 4 + x, lz = bz * 4 + z;
                const int gx = cx * 32 + lx, gy = cy * 32 + by * 4 + y, gz = cz * 32 + lz;
                unsigned v = 0;
                if (gx < w.dims[0] && gy < w.dims[1] && gz < w.dims[2])
                    v = gen::cell_material(&d, gx, gy, gz, heights[lx + 32 * lz], water, cave_seed, cave_freq);
                word |= v << (8 * x);
                if (v) m |= 1ull << (x + 4 * (y + 4 * z));
            }
            packed[y + 4 * z] = word;
        }
    }
    const unsigned wi = ci * 512u + (unsigned)b;
    uint4* dst = reinterpret_cast<uint4*>(mats + (size_t)wi * 64u);
#pragma unroll
    for (int q = 0; q < 4; ++q) dst[q] = make_uint4(packed[4 * q], packed[4 * q + 1], packed[4 * q + 2], packed[4 * q + 3]);
    mask[wi] = m;
    const int any = __syncthreads_or(m != 0ull);
    if (threadIdx.x == 0) {
        const unsigned long long bit = 1ull << (ci & 63u);
        if (any) atomicOr(coarse + (ci >> 6), bit);
        else atomicAnd(coarse + (ci >> 6), ~bit);
    }
}

// Leaf cells of tree blockIdx.x: each kept cell that holds air or water
// becomes 6.  Concurrent trees only ever write 6 over 0 or 4, so a cell
// covered by several trees ends the same whichever comes first.
__global__ void __launch_bounds__(128) k_gen_leaves(WorldView w, unsigned long long* mask, unsigned char* mats,
                                                    unsigned long long* coarse, vt_gen_desc d) {
    __shared__ int site[4];
    const int t = blockIdx.x;
    if (threadIdx.x == 0) site[3] = gen::tree_site(&d, t, &site[0], &site[1], &site[2]) ? 1 : 0;
    __syncthreads();
    const int c = threadIdx.x;
    if (!site[3] || c >= 125) return;
    const int dx = c % 5 - 2, dy = (c / 5) % 5 - 2, dz = c / 25 - 2;
    const int lx = site[0] + dx, ly = site[2] + 5 + dy, lz = site[1] + dz;
    if (lx < 0 || lz < 0 || lx >= w.dims[0] || lz >= w.dims[2] || ly >= w.dims[1]) return;
    if (!gen::leaf_kept(gen::stream_seed(d.seed, gen::kLeaves), t, dx, dy, dz)) return;
    unsigned wi, vb;
    cell_addr(w, lx, ly, lz, &wi, &vb);
    volatile unsigned char* cell = mats + (size_t)wi * 64u + vb;
    const unsigned char cur = *cell;
    if (cur != 0 && cur != 4) return;
    *cell = 6;
    mark_solid(mask, coarse, wi, vb);
}

// Trunks (material 5 over anything), after every leaf has landed.
__global__ void __launch_bounds__(256) k_gen_trunks(WorldView w, unsigned long long* mask, unsigned char* mats,
                                                    unsigned long long* coarse, vt_gen_desc d) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= d.trees) return;
    int x, z, h;
    if (!gen::tree_site(&d, t, &x, &z, &h)) return;
    for (int y = h; y < h + 6; ++y) {
        unsigned wi, vb;
        cell_addr(w, x, y, z, &wi, &vb);
        mats[(size_t)wi * 64u + vb] = 5;
        mark_solid(mask, coarse, wi, vb);
    }
}

// One block per chunk, one thread per brick: the brick's 64 bytes back to the
// x-fastest dense grid (cells outside the world are skipped).
__global__ void __launch_bounds__(512) k_gather_dense(WorldView w, const unsigned char* __restrict__ mats,
                                                      unsigned char* __restrict__ dst) {
    const unsigned ci = blockIdx.x;
    const int cx = (int)(ci % (unsigned)w.cdim[0]);
    const int cy = (int)((ci / (unsigned)w.cdim[0]) % (unsigned)w.cdim[1]);
    const int cz = (int)(ci / ((unsigned)w.cdim[0] * (unsigned)w.cdim[1]));
    const int b = threadIdx.x;
    const int bx = b & 7, by = (b >> 3) & 7, bz = b >> 6;
    const uint4* src = reinterpret_cast<const uint4*>(mats + ((size_t)ci * 512u + (unsigned)b) * 64u);
    unsigned packed[16];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        const uint4 v = src[q];
        packed[4 * q] = v.x;
        packed[4 * q + 1] = v.y;
        packed[4 * q + 2] = v.z;
        packed[4 * q + 3] = v.w;
    }
    for (int z = 0; z < 4; ++z)
        for (int y = 0; y < 4; ++y)
            for (int x = 0; x < 4; ++x) {
                const int gx = cx * 32 + bx * 4 + x, gy = cy * 32 + by * 4 + y, gz = cz * 32 + bz * 4 + z;
                if (gx < w.dims[0] && gy < w.dims[1] && gz < w.dims[2])
                    dst[(size_t)gx + (size_t)w.dims[0] * ((size_t)gy + (size_t)w.dims[1] * (size_t)gz)] =
                        (unsigned char)(packed[y + 4 * z] >> (8 * x));
            }
}

}  // namespace

}  // namespace vt

using namespace vt;

extern "C" {

vt_status vt_world_generate(vt_world* w, const vt_gen_desc* desc, vt_stream stream) {
    if (!w) return VT_ERR_ARG;
    if (!desc) return fail(w->ctx, VT_ERR_ARG, "null generator descriptor");
    for (int i = 0; i < 3; ++i)
        if (desc->dims[i] != w->dims[i]) return fail(w->ctx, VT_ERR_ARG, "generator dims must equal the world's dims");
    if (!(desc->period > 0.0f) || !(desc->cave_period > 0.0f) || desc->octaves < 1 || desc->octaves > 16 ||
        desc->trees < 0)
        return fail(w->ctx, VT_ERR_ARG, "generator descriptor out of range");
    cudaStream_t st = (cudaStream_t)stream;
    const WorldView v = w->view();
    k_gen_chunks<<<(unsigned)w->nchunks, 512, 0, st>>>(v, w->d_mask, w->d_mats, w->d_coarse, *desc);
    VT_CUDA(w->ctx, cudaGetLastError());
    if (desc->trees > 0 && w->dims[0] >= 6 && w->dims[2] >= 6) {
        k_gen_leaves<<<(unsigned)desc->trees, 128, 0, st>>>(v, w->d_mask, w->d_mats, w->d_coarse, *desc);
        VT_CUDA(w->ctx, cudaGetLastError());
        k_gen_trunks<<<(unsigned)((desc->trees + 255) / 256), 256, 0, st>>>(v, w->d_mask, w->d_mats, w->d_coarse, *desc);
        VT_CUDA(w->ctx, cudaGetLastError());
    }
    w->dist_dirty = true;
    return VT_OK;
}

vt_status vt_world_download_dense(vt_world* w, uint8_t* h_materials, size_t nbytes, vt_stream stream) {
    if (!w) return VT_ERR_ARG;
    const size_t need = (size_t)w->dims[0] * w->dims[1] * w->dims[2];
    if (!h_materials || nbytes != need) return fail(w->ctx, VT_ERR_ARG, "dense download needs exactly X*Y*Z bytes");
    unsigned char* stage = nullptr;
    vt_status s = world_stage(w, need, &stage);
    if (s) return s;
    cudaStream_t st = (cudaStream_t)stream;
    k_gather_dense<<<(unsigned)w->nchunks, 512, 0, st>>>(w->view(), w->d_mats, stage);
    VT_CUDA(w->ctx, cudaGetLastError());
    VT_CUDA(w->ctx, cudaMemcpyAsync(h_materials, stage, need, cudaMemcpyDeviceToHost, st));
    VT_CUDA(w->ctx, cudaStreamSynchronize(st));
    return VT_OK;
}

}  // extern "C"
