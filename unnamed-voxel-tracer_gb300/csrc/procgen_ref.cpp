// procgen_ref.cpp -- the reference's own world generator, in its own world
// format (host code).
//
// src/procgen.zig:6-70 fills a VoxelBrickmap(dim, 8) voxel by voxel: a stone
// floor of 16 layers, then per column (x outer, z inner) a heightfield column
// of dirt-like model ids, grass tufts, flowers and trees, every choice drawn
// from one util.LCG (src/engine/util.zig:33-45) in a fixed order.  The
// brickmap allocates a brick the first time a chunk is written
// (voxel.zig:47-61, gpu_block_allocator.zig:20-30), so the brick order is the
// order of first touch.  This file replays that sequence exactly, writing the
// chunk table and brick pool the reference's buffers would hold, ready for
// vt_brickmap_upload.
//
// The heightfield noise is FastNoiseLite's fbm (znoise), which is not part of
// the reference sources; the caller passes its values per column (or NULL
// for the library's own seeded value-noise fbm with the same range and
// scale, noise2((offset + x) / 10, (offset + z) / 10)).
#include <math.h>
#include <stdint.h>
#include <string.h>

#include <vector>

#include "../../include/vt.h"
#include "gen_noise.cuh"

namespace {

// util.LCG: seed = seed * 1103515245 + 12345 (mod 2^32), returned.
struct Lcg {
    uint32_t seed;
    uint32_t rand() {
        seed = seed * 1103515245u + 12345u;
        return seed;
    }
};

// Voxel (voxel.zig:7-19): ty in bits 0..27, is_solid in bit 28.
inline uint32_t voxel(uint32_t ty, bool solid) { return (ty & 0x0FFFFFFFu) | (solid ? (1u << 28) : 0u); }

struct Brickmap {
    int dim, cdim;
    uint32_t* chunks;
    uint32_t* bricks;
    size_t capacity, used = 0;
    bool overflow = false;

    // get_block_for_chunk (voxel.zig:47-56)
    size_t block(int cx, int cy, int cz) {
        uint32_t& idx = chunks[(size_t)cx + (size_t)cdim * ((size_t)cy + (size_t)cz * cdim)];
        if (idx > 0) return idx - 1;
        const size_t b = used++;
        idx = (uint32_t)b + 1u;
        if (b < capacity) memset(bricks + b * 512u, 0, 512u * sizeof(uint32_t));
        else overflow = true;
        return b;
    }
    // set (voxel.zig:58-61); writes beyond dim are the caller's bug in the
    // reference (unchecked); here they are dropped
    void set(int x, int y, int z, uint32_t v) {
        if (x < 0 || y < 0 || z < 0 || x >= dim || y >= dim || z >= dim) return;
        const size_t b = block(x / 8, y / 8, z / 8);
        if (b < capacity) bricks[b * 512u + (size_t)(x % 8) + (size_t)((y % 8) + (z % 8) * 8) * 8] = v;
    }
    // get (voxel.zig:63-70)
    uint32_t get(int x, int y, int z) const {
        if (x < 0 || y < 0 || z < 0 || x >= dim || y >= dim || z >= dim) return 0;
        const uint32_t idx = chunks[(size_t)(x / 8) + (size_t)cdim * ((size_t)(y / 8) + (size_t)(z / 8) * cdim)];
        if (idx == 0 || idx - 1 >= capacity) return 0;
        return bricks[(size_t)(idx - 1) * 512u + (size_t)(x % 8) + (size_t)((y % 8) + (z % 8) * 8) * 8];
    }
};

// place_tree (procgen.zig:55-70)
void place_tree(Lcg& lcg, Brickmap& w, int x, int y, int z) {
    const int trunk = (int)(lcg.rand() % 4u) + 4;
    w.set(x + 1, y, z + 1, voxel(15, true));
    for (int o = 0; o < trunk; ++o) w.set(x + 1, y + o, z + 1, voxel(14 + lcg.rand() % 3u, true));
    for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 3; ++b)
            for (int c = 0; c < 3; ++c) w.set(x + a, y + trunk + b, z + c, voxel(18 + lcg.rand() % 2u, true));
}

}  // namespace

extern "C" {

vt_status vt_procgen_reference(int32_t dim, float offset_x, float offset_z, const float* h_noise, uint64_t noise_seed,
                               uint32_t* h_chunks, uint32_t* h_bricks, size_t brick_capacity, size_t* nbricks) {
    if (dim < 8 || dim > 4096 || dim % 8 != 0 || !h_chunks || !nbricks || (brick_capacity && !h_bricks))
        return VT_ERR_ARG;
    Brickmap w;
    w.dim = dim;
    w.cdim = dim / 8;
    w.chunks = h_chunks;
    w.bricks = h_bricks;
    w.capacity = brick_capacity;
    memset(h_chunks, 0, (size_t)w.cdim * w.cdim * w.cdim * sizeof(uint32_t));
    Lcg lcg{0x46AE4Fu};
    // the stone floor: 16 layers of model 13 (procgen.zig:10-19)
    for (int x = 0; x < dim; ++x)
        for (int z = 0; z < dim; ++z)
            for (int y = 0; y < 16; ++y) w.set(x, y, z, voxel(13, true));
    const uint64_t ns = vt::gen::stream_seed(noise_seed, 7);
    for (int x = 0; x < dim; ++x) {
        for (int z = 0; z < dim; ++z) {
            float val;
            if (h_noise) {
                val = h_noise[(size_t)x * dim + z];
            } else {
                // fbm of value noise in [-1, 1), 3 octaves, at ((offset + x) / 10, (offset + z) / 10)
                const float fx = (offset_x + (float)x) / 10.0f, fz = (offset_z + (float)z) / 10.0f;
                val = (float)vt::gen::fbm2(ns, (double)fx, (double)fz, 1.0, 3);
            }
            // vh = intFromFloat(max(val * dim * 0.1, 0)) (procgen.zig:24)
            const float hf = fmaxf(val * (float)dim * 0.1f, 0.0f);
            const int vh = (int)hf;
            for (int h = 0; h < vh; ++h) {
                w.set(x, h, z, voxel(21 + lcg.rand() % 3u, true));
                if (h <= 15) w.set(x, h, z, voxel(25 + lcg.rand() % 3u, true));
                else if (h == vh - 1) w.set(x, h, z, voxel(lcg.rand() % 6u, true));
            }
            if (vh > 16) {
                if (w.get(x, vh, z) != 0) continue;  // skips the column's final draw too
                if (lcg.rand() % 5u == 0) w.set(x, vh, z, voxel(7 + lcg.rand() % 5u, false));
                if (lcg.rand() % 71u == 0) w.set(x, vh, z, voxel(7 + 5, true));
                if (lcg.rand() % 420u == 0 && x < 500 && z < 500 && x > 5 && z > 5) place_tree(lcg, w, x, vh, z);
            }
            (void)lcg.rand();
        }
    }
    *nbricks = w.used;
    return w.overflow ? VT_ERR_OOM : VT_OK;
}

}  // extern "C"
