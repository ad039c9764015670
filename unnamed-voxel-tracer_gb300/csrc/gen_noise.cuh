// gen_noise.cuh -- the seeded value-noise generator, shared by the host
// generator (gen.cpp) and the device one (world_gen.cu) so that both produce
// the same bytes: SplitMix64 hashing and IEEE double +, -, *, / and floor
// only (no contraction: host -ffp-contract=off, device --fmad=false).
#pragma once

#include <math.h>
#include <stdint.h>

#include "../../include/vt.h"

#if defined(__CUDACC__)
#define VT_HD __host__ __device__
#else
#define VT_HD
#endif

namespace vt {
namespace gen {

VT_HD inline uint64_t mix64(uint64_t z) {
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

struct SplitMix {
    uint64_t s;
    VT_HD uint64_t next() {
        s += 0x9E3779B97F4A7C15ull;
        return mix64(s);
    }
    VT_HD double uniform() { return (double)(next() >> 11) * 0x1p-53; }
};

// Lattice value in [-1, 1).
VT_HD inline double lattice(uint64_t seed, int64_t x, int64_t y, int64_t z) {
    uint64_t h = seed;
    h = mix64(h ^ ((uint64_t)x * 0x9E3779B97F4A7C15ull));
    h = mix64(h ^ ((uint64_t)y * 0xC2B2AE3D27D4EB4Full));
    h = mix64(h ^ ((uint64_t)z * 0x165667B19E3779F9ull));
    return (double)(h >> 11) * 0x1p-52 - 1.0;
}

VT_HD inline double smooth(double t) { return t * t * (3.0 - 2.0 * t); }
VT_HD inline double lerp(double a, double b, double t) { return a + (b - a) * t; }

VT_HD inline double noise2(uint64_t seed, double x, double z) {
    const double fx = floor(x), fz = floor(z);
    const int64_t ix = (int64_t)fx, iz = (int64_t)fz;
    const double sx = smooth(x - fx), sz = smooth(z - fz);
    const double a = lerp(lattice(seed, ix, 0, iz), lattice(seed, ix + 1, 0, iz), sx);
    const double b = lerp(lattice(seed, ix, 0, iz + 1), lattice(seed, ix + 1, 0, iz + 1), sx);
    return lerp(a, b, sz);
}

VT_HD inline double noise3(uint64_t seed, double x, double y, double z) {
    const double fx = floor(x), fy = floor(y), fz = floor(z);
    const int64_t ix = (int64_t)fx, iy = (int64_t)fy, iz = (int64_t)fz;
    const double sx = smooth(x - fx), sy = smooth(y - fy), sz = smooth(z - fz);
    double c[2][2];
    for (int dz = 0; dz < 2; ++dz)
        for (int dy = 0; dy < 2; ++dy)
            c[dz][dy] = lerp(lattice(seed, ix, iy + dy, iz + dz), lattice(seed, ix + 1, iy + dy, iz + dz), sx);
    return lerp(lerp(c[0][0], c[0][1], sy), lerp(c[1][0], c[1][1], sy), sz);
}

constexpr uint64_t kOctaveSalt = 0x632BE59BD9B4E019ull;

VT_HD inline double fbm2(uint64_t seed, double x, double z, double freq, int octaves) {
    double sum = 0.0, amp = 1.0, norm = 0.0;
    for (int o = 0; o < octaves; ++o) {
        sum += amp * noise2(seed + (uint64_t)o * kOctaveSalt, x * freq, z * freq);
        norm += amp;
        amp *= 0.5;
        freq *= 2.0;
    }
    return sum / norm;
}

VT_HD inline double fbm3(uint64_t seed, double x, double y, double z, double freq) {
    const double a = noise3(seed, x * freq, y * freq, z * freq);
    const double b = noise3(seed + kOctaveSalt, x * freq * 2.0, y * freq * 2.0, z * freq * 2.0);
    return (a + 0.5 * b) / 1.5;
}

VT_HD inline uint64_t stream_seed(uint64_t seed, uint64_t purpose) { return mix64(seed ^ mix64(purpose)); }

constexpr uint64_t kTerrain = 1, kCaves = 2, kTrees = 3, kLeaves = 4, kCamera = 5, kSun = 6;

VT_HD inline int height_at(const vt_gen_desc* d, int x, int z) {
    const double f = fbm2(stream_seed(d->seed, kTerrain), (double)x, (double)z, 1.0 / (double)d->period, d->octaves);
    int h = (int)floor((double)d->base_height + (double)d->amplitude * f);
    h = h < d->dims[1] - 1 ? h : d->dims[1] - 1;
    return h > 1 ? h : 1;
}


// Material of cell (x, y, z) of column height h before trees: grass on top,
// three layers of dirt, stone below, water in air below the water level,
// caves carved out of solid cells (not the bottom layer) where the 3-D fbm
// exceeds the threshold.
VT_HD inline uint8_t cell_material(const vt_gen_desc* d, int x, int y, int z, int h, int water, uint64_t cave_seed,
                                   double cave_freq) {
    uint8_t m = 0;
    if (y < h) {
        m = (y == h - 1) ? 1 : (y >= h - 4 ? 2 : 3);
        if (d->caves && y > 0 && fbm3(cave_seed, (double)x, (double)y, (double)z, cave_freq) > (double)d->cave_threshold)
            m = 0;
    } else if (y < water) {
        m = 4;
    }
    return m;
}

// Tree t of a scene: its column (x, z) from draws 2t and 2t+1 of the tree
// stream (SplitMix64 is counter based: draw k is mix64(s0 + (k+1) * gamma)),
// and its surface height h; false when the tree does not fit under the top.
VT_HD inline bool tree_site(const vt_gen_desc* d, int t, int* x, int* z, int* h) {
    const int X = d->dims[0], Y = d->dims[1], Z = d->dims[2];
    const uint64_t s0 = stream_seed(d->seed, kTrees);
    const uint64_t g = 0x9E3779B97F4A7C15ull;
    const double ux = (double)(mix64(s0 + (uint64_t)(2 * t + 1) * g) >> 11) * 0x1p-53;
    const double uz = (double)(mix64(s0 + (uint64_t)(2 * t + 2) * g) >> 11) * 0x1p-53;
    *x = 2 + (int)(ux * (double)(X - 4));
    *z = 2 + (int)(uz * (double)(Z - 4));
    *h = height_at(d, *x, *z);
    return *h + 8 < Y;
}

// Whether leaf cell (dx, dy, dz) in [-2, 2]^3 of tree t is kept (p = 0.7).
VT_HD inline bool leaf_kept(uint64_t leaf_seed, int t, int dx, int dy, int dz) {
    const uint64_t hh =
        mix64(leaf_seed ^ mix64(((uint64_t)t << 20) ^ (uint64_t)((dx + 2) + 5 * ((dy + 2) + 5 * (dz + 2)))));
    return (double)(hh >> 11) * 0x1p-53 < 0.7;
}

// Trees in seed order: a 1x6x1 trunk of material 5 standing on the column's
// surface (written over anything), then a 5^3 blob of material 6 centred on
// the trunk's top that fills only air or water.  The final bytes do not
// depend on the order: a cell any trunk covers ends as 5; otherwise a cell of
// air or water some kept leaf covers ends as 6; every other cell keeps its
// terrain material.  The device generator relies on that to plant all leaves,
// then all trunks, in parallel.
VT_HD inline void plant_trees(const vt_gen_desc* d, uint8_t* out) {
    const int X = d->dims[0], Y = d->dims[1], Z = d->dims[2];
    if (X < 6 || Z < 6) return;
    const uint64_t ls = stream_seed(d->seed, kLeaves);
    for (int t = 0; t < d->trees; ++t) {
        int x, z, h;
        if (!tree_site(d, t, &x, &z, &h)) continue;
        for (int y = h; y < h + 6; ++y) out[(size_t)x + (size_t)X * ((size_t)y + (size_t)Y * (size_t)z)] = 5;
        for (int dz = -2; dz <= 2; ++dz)
            for (int dy = -2; dy <= 2; ++dy)
                for (int dx = -2; dx <= 2; ++dx) {
                    const int lx = x + dx, ly = h + 5 + dy, lz = z + dz;
                    if (lx < 0 || lz < 0 || lx >= X || lz >= Z || ly >= Y) continue;
                    uint8_t& c = out[(size_t)lx + (size_t)X * ((size_t)ly + (size_t)Y * (size_t)lz)];
                    if (c != 0 && c != 4) continue;
                    if (leaf_kept(ls, t, dx, dy, dz)) c = 6;
                }
    }
}

}  // namespace gen
}  // namespace vt
