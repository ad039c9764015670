// gen_host.cpp -- the device generator's tree order on the host: every leaf
// of every tree (trees in reverse order), then every trunk (reverse order),
// the way k_gen_leaves / k_gen_trunks apply them, against the sequential
// plant_trees.  Both start from the same terrain (cell_material).
#include <stdint.h>
#include <string.h>

#include <vector>

#include "../../unnamed-voxel-tracer_gb300/csrc/gen_noise.cuh"

using namespace vt::gen;

static void terrain(const vt_gen_desc* d, uint8_t* out) {
    const int X = d->dims[0], Y = d->dims[1], Z = d->dims[2];
    const int water = (int)ceil((double)d->water_level);
    const uint64_t cs = stream_seed(d->seed, kCaves);
    const double cf = 1.0 / (double)d->cave_period;
    for (int z = 0; z < Z; ++z)
        for (int x = 0; x < X; ++x) {
            const int h = height_at(d, x, z);
            for (int y = 0; y < Y; ++y)
                out[(size_t)x + (size_t)X * ((size_t)y + (size_t)Y * (size_t)z)] = cell_material(d, x, y, z, h, water, cs, cf);
        }
}

extern "C" int gh_compare(const vt_gen_desc* d, uint8_t* seq, uint8_t* par) {
    const int X = d->dims[0], Y = d->dims[1], Z = d->dims[2];
    const size_t n = (size_t)X * Y * Z;
    terrain(d, seq);
    memcpy(par, seq, n);
    plant_trees(d, seq);
    if (X >= 6 && Z >= 6) {
        const uint64_t ls = stream_seed(d->seed, kLeaves);
        for (int t = d->trees - 1; t >= 0; --t) {
            int x, z, h;
            if (!tree_site(d, t, &x, &z, &h)) continue;
            for (int c = 124; c >= 0; --c) {
                const int dx = c % 5 - 2, dy = (c / 5) % 5 - 2, dz = c / 25 - 2;
                const int lx = x + dx, ly = h + 5 + dy, lz = z + dz;
                if (lx < 0 || lz < 0 || lx >= X || lz >= Z || ly >= Y) continue;
                if (!leaf_kept(ls, t, dx, dy, dz)) continue;
                uint8_t& cell = par[(size_t)lx + (size_t)X * ((size_t)ly + (size_t)Y * (size_t)lz)];
                if (cell == 0 || cell == 4) cell = 6;
            }
        }
        for (int t = d->trees - 1; t >= 0; --t) {
            int x, z, h;
            if (!tree_site(d, t, &x, &z, &h)) continue;
            for (int y = h; y < h + 6; ++y) par[(size_t)x + (size_t)X * ((size_t)y + (size_t)Y * (size_t)z)] = 5;
        }
    }
    return memcmp(seq, par, n) == 0 ? 0 : 1;
}
