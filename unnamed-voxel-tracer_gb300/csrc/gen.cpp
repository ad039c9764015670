// gen.cpp -- seeded synthetic scenes (host code).
//
// The reference fills its world with FastNoiseLite fbm terrain
// (src/procgen.zig:6-53); the scenes here use a seeded value-noise fbm
// heightmap with the same role.  Everything is built from SplitMix64 hashing
// and IEEE double +, -, *, / and floor (compiled with -ffp-contract=off), so a
// seed gives the same bytes on every machine; the camera trigonometry uses
// series written here for the same reason.
#include <math.h>
#include <stdint.h>
#include <string.h>

#include <algorithm>
#include <thread>
#include <vector>

#include "../../include/vt.h"
#include "gen_noise.cuh"

namespace {

using namespace vt::gen;

// Deterministic double sine/cosine: reduction by pi/2 split into
// 0x1.921fb5p+0 + 0x1.110b46p-26 + 0x1.1a62633145c07p-54 (each the leading
// bits of the previous remainder) and Taylor series to degree 21 / 20.
void det_sincos(double x, double* s, double* c) {
    const double k = floor(x * 0x1.45f306dc9c883p-1 + 0.5);
    double r = x - k * 0x1.921fb5p+0;
    r = r - k * 0x1.110b46p-26;
    r = r - k * 0x1.1a62633145c07p-54;
    const double r2 = r * r;
    double ps = 0.0, pc = 0.0, term = r;
    for (int n = 1; n <= 21; n += 2) {  // sin: r - r^3/3! + ...
        ps += term;
        term = -term * r2 / (double)((n + 1) * (n + 2));
    }
    term = 1.0;
    for (int n = 0; n <= 20; n += 2) {  // cos: 1 - r^2/2! + ...
        pc += term;
        term = -term * r2 / (double)((n + 1) * (n + 2));
    }
    const int q = ((int)(int64_t)k) & 3;
    switch (q) {
        case 0: *s = ps; *c = pc; break;
        case 1: *s = pc; *c = -ps; break;
        case 2: *s = -ps; *c = -pc; break;
        default: *s = -pc; *c = ps; break;
    }
}

constexpr double kPi = 3.14159265358979323846;

void fill_slab(const vt_gen_desc* d, uint8_t* out, int z0, int z1) {
    const int X = d->dims[0], Y = d->dims[1];
    const int water = (int)ceil((double)d->water_level);
    const uint64_t cs = stream_seed(d->seed, kCaves);
    const double cf = 1.0 / (double)d->cave_period;
    for (int z = z0; z < z1; ++z)
        for (int x = 0; x < X; ++x) {
            const int h = height_at(d, x, z);
            for (int y = 0; y < Y; ++y)
                out[(size_t)x + (size_t)X * ((size_t)y + (size_t)Y * (size_t)z)] = cell_material(d, x, y, z, h, water, cs, cf);
        }
}

}  // namespace

extern "C" {

void vt_gen_desc_init(vt_gen_desc* d, int32_t x, int32_t y, int32_t z, float scale, uint64_t seed) {
    if (!d) return;
    memset(d, 0, sizeof(*d));
    d->dims[0] = x;
    d->dims[1] = y;
    d->dims[2] = z;
    d->base_height = 64.0f * scale;
    d->amplitude = 24.0f * scale;
    d->period = 64.0f * scale;
    d->water_level = 56.0f * scale;
    d->camera_height = std::max(2.0f, 10.0f * scale);
    d->octaves = 4;
    d->trees = 0;
    d->caves = 0;
    d->cave_threshold = 0.6f;
    d->cave_period = 24.0f * scale;
    d->seed = seed;
}

vt_status vt_gen_world(const vt_gen_desc* d, uint8_t* out, size_t nbytes, int32_t threads) {
    if (!d || !out) return VT_ERR_ARG;
    for (int i = 0; i < 3; ++i)
        if (d->dims[i] < 1) return VT_ERR_ARG;
    if (!(d->period > 0.0f) || !(d->cave_period > 0.0f) || d->octaves < 1 || d->octaves > 16) return VT_ERR_ARG;
    const size_t need = (size_t)d->dims[0] * d->dims[1] * d->dims[2];
    if (nbytes != need) return VT_ERR_ARG;
    int nt = threads > 0 ? threads : (int)std::max(1u, std::thread::hardware_concurrency());
    nt = std::min(nt, d->dims[2]);
    std::vector<std::thread> pool;
    for (int i = 0; i < nt; ++i) {
        const int z0 = (int)((int64_t)d->dims[2] * i / nt), z1 = (int)((int64_t)d->dims[2] * (i + 1) / nt);
        pool.emplace_back(fill_slab, d, out, z0, z1);
    }
    for (auto& t : pool) t.join();
    plant_trees(d, out);
    return VT_OK;
}

int32_t vt_gen_height(const vt_gen_desc* d, int32_t x, int32_t z) { return d ? height_at(d, x, z) : 0; }

vt_status vt_camera_look(const float pos[3], float yaw, float pitch, float fov, int32_t width, int32_t height,
                         vt_camera* out) {
    if (!pos || !out || width <= 0 || height <= 0 || !(fov > 0.0f) || !(fov < 3.1f)) return VT_ERR_ARG;
    memset(out, 0, sizeof(*out));
    double sy, cy, sp, cp, sh, ch;
    det_sincos((double)yaw, &sy, &cy);
    det_sincos((double)pitch, &sp, &cp);
    det_sincos(0.5 * (double)fov, &sh, &ch);
    const double right[3] = {cy, 0.0, -sy};
    const double up[3] = {-sp * sy, cp, -sp * cy};
    const double fwd[3] = {cp * sy, sp, cp * cy};
    for (int j = 0; j < 3; ++j) {
        out->pos[j] = pos[j];
        out->view[0 * 4 + j] = (float)right[j];
        out->view[1 * 4 + j] = (float)up[j];
        out->view[2 * 4 + j] = (float)fwd[j];
        out->view[3 * 4 + j] = 0.0f;
    }
    out->pos[3] = 1.0f;
    out->view[3] = out->view[7] = out->view[11] = 0.0f;
    out->view[15] = 1.0f;
    out->fov = fov;
    out->tan_half_fov = (float)(sh / ch);
    out->width = width;
    out->height = height;
    return VT_OK;
}

vt_status vt_gen_camera(const vt_gen_desc* d, uint64_t seed, int32_t width, int32_t height, vt_camera* out) {
    if (!d || !out) return VT_ERR_ARG;
    SplitMix rng{stream_seed(d->seed ^ mix64(seed), kCamera)};
    const double fx = (0.1 + 0.8 * rng.uniform()) * (double)d->dims[0];
    const double fz = (0.1 + 0.8 * rng.uniform()) * (double)d->dims[2];
    const double yaw = 2.0 * kPi * rng.uniform();
    const double pitch = -(kPi / 6.0) * rng.uniform();
    const int h = height_at(d, (int)fx, (int)fz);
    const double top = std::max((double)h, (double)d->water_level);
    double y = top + (double)d->camera_height + 0.5;
    y = std::min(y, (double)d->dims[1] - 0.5);
    const float pos[3] = {(float)fx, (float)y, (float)fz};
    return vt_camera_look(pos, (float)yaw, (float)pitch, (float)(70.0 * kPi / 180.0), width, height, out);
}

vt_status vt_default_palette(uint32_t* pal) {
    if (!pal) return VT_ERR_ARG;
    auto rgba = [](unsigned r, unsigned g, unsigned b) { return r | (g << 8) | (b << 16) | (255u << 24); };
    pal[0] = 0;
    pal[1] = rgba(86, 160, 60);    // grass
    pal[2] = rgba(134, 96, 67);    // dirt
    pal[3] = rgba(125, 125, 125);  // stone
    pal[4] = rgba(50, 90, 200);    // water
    pal[5] = rgba(110, 80, 50);    // trunk
    pal[6] = rgba(60, 130, 50);    // leaves
    for (unsigned i = 7; i < 256; ++i) {
        const uint64_t h = mix64(0xC0104ull + i);
        pal[i] = rgba((unsigned)(h & 255), (unsigned)((h >> 8) & 255), (unsigned)((h >> 16) & 255));
    }
    return VT_OK;
}

vt_status vt_gen_sun(uint64_t seed, float out[3]) {
    if (!out) return VT_ERR_ARG;
    SplitMix rng{stream_seed(seed, kSun)};
    const double elev = (20.0 + 40.0 * rng.uniform()) * kPi / 180.0;
    const double azim = 2.0 * kPi * rng.uniform();
    double se, ce, sa, ca;
    det_sincos(elev, &se, &ce);
    det_sincos(azim, &sa, &ca);
    out[0] = (float)(ce * sa);
    out[1] = (float)se;
    out[2] = (float)(ce * ca);
    return VT_OK;
}

}  // extern "C"
