/*
 * vt_oracle_gen.c -- the seeded benchmark scenes restated in plain C, so that
 * the CPU baseline and the reference arm of the benchmark build their inputs
 * without loading the GPU library.
 *
 * TEST INFRASTRUCTURE ONLY (see vt_oracle.h).  The scenes are this project's
 * own synthetic workloads (value-noise fBm terrain in place of the
 * reference's FastNoiseLite terrain, src/procgen.zig:6-53, plus trees and
 * caves); tests/test_oracle_gen.py checks every function here against the
 * library's host generator byte for byte.
 *
 * Determinism: SplitMix64 integer hashing and IEEE double +, -, *, / and
 * floor only (compiled with -ffp-contract=off); camera and sun angles use a
 * sine/cosine written here (Cody-Waite reduction by pi/2 in three parts and
 * Taylor series), never libm's.
 */
#include <math.h>
#include <pthread.h>
#include <stdint.h>
#include <string.h>

#include "vt_oracle.h"

#define GAMMA 0x9E3779B97F4A7C15ull
#define OCTAVE_SALT 0x632BE59BD9B4E019ull
enum { P_TERRAIN = 1, P_CAVES = 2, P_TREES = 3, P_LEAVES = 4, P_CAMERA = 5, P_SUN = 6 };

static uint64_t mix(uint64_t z) {
    z ^= z >> 30;
    z *= 0xBF58476D1CE4E5B9ull;
    z ^= z >> 27;
    z *= 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

static uint64_t purpose_seed(uint64_t seed, uint64_t purpose) { return mix(seed ^ mix(purpose)); }

/* the k-th draw (k >= 1) of a SplitMix64 stream started at s0, in [0, 1) */
static double draw(uint64_t s0, uint64_t k) { return (double)(mix(s0 + k * GAMMA) >> 11) * 0x1p-53; }

/* value at an integer lattice point, in [-1, 1) */
static double lattice_value(uint64_t seed, int64_t x, int64_t y, int64_t z) {
    uint64_t h = mix(seed ^ ((uint64_t)x * GAMMA));
    h = mix(h ^ ((uint64_t)y * 0xC2B2AE3D27D4EB4Full));
    h = mix(h ^ ((uint64_t)z * 0x165667B19E3779F9ull));
    return (double)(h >> 11) * 0x1p-52 - 1.0;
}

static double fade(double t) { return t * t * (3.0 - 2.0 * t); }
static double mixd(double a, double b, double t) { return a + (b - a) * t; }

static double value2(uint64_t seed, double x, double z) {
    const double x0 = floor(x), z0 = floor(z);
    const int64_t i = (int64_t)x0, k = (int64_t)z0;
    const double u = fade(x - x0), w = fade(z - z0);
    const double near = mixd(lattice_value(seed, i, 0, k), lattice_value(seed, i + 1, 0, k), u);
    const double far = mixd(lattice_value(seed, i, 0, k + 1), lattice_value(seed, i + 1, 0, k + 1), u);
    return mixd(near, far, w);
}

static double value3(uint64_t seed, double x, double y, double z) {
    const double x0 = floor(x), y0 = floor(y), z0 = floor(z);
    const int64_t i = (int64_t)x0, j = (int64_t)y0, k = (int64_t)z0;
    const double u = fade(x - x0), v = fade(y - y0), w = fade(z - z0);
    double row[2][2];
    for (int dz = 0; dz < 2; ++dz)
        for (int dy = 0; dy < 2; ++dy)
            row[dz][dy] = mixd(lattice_value(seed, i, j + dy, k + dz), lattice_value(seed, i + 1, j + dy, k + dz), u);
    return mixd(mixd(row[0][0], row[0][1], v), mixd(row[1][0], row[1][1], v), w);
}

/* 2-D fBm: octaves of value noise, lacunarity 2, gain 0.5, normalised */
static double fbm_2d(uint64_t seed, double x, double z, double freq, int octaves) {
    double total = 0.0, amp = 1.0, weight = 0.0;
    for (int o = 0; o < octaves; ++o) {
        total += amp * value2(seed + (uint64_t)o * OCTAVE_SALT, x * freq, z * freq);
        weight += amp;
        amp *= 0.5;
        freq *= 2.0;
    }
    return total / weight;
}

/* 3-D fBm of two octaves (caves) */
static double fbm_3d(uint64_t seed, double x, double y, double z, double f) {
    const double a = value3(seed, x * f, y * f, z * f);
    const double b = value3(seed + OCTAVE_SALT, x * f * 2.0, y * f * 2.0, z * f * 2.0);
    return (a + 0.5 * b) / 1.5;
}

static int column_height(const vt_gen_desc* d, int x, int z) {
    const double f = fbm_2d(purpose_seed(d->seed, P_TERRAIN), (double)x, (double)z, 1.0 / (double)d->period,
                            d->octaves);
    int h = (int)floor((double)d->base_height + (double)d->amplitude * f);
    if (h > d->dims[1] - 1) h = d->dims[1] - 1;
    return h < 1 ? 1 : h;
}

int32_t vto_gen_height(const vt_gen_desc* d, int32_t x, int32_t z) { return column_height(d, x, z); }

void vto_gen_desc_init(vt_gen_desc* d, int32_t x, int32_t y, int32_t z, float scale, uint64_t seed) {
    memset(d, 0, sizeof(*d));
    d->dims[0] = x;
    d->dims[1] = y;
    d->dims[2] = z;
    d->base_height = 64.0f * scale;
    d->amplitude = 24.0f * scale;
    d->period = 64.0f * scale;
    d->water_level = 56.0f * scale;
    d->camera_height = 10.0f * scale < 2.0f ? 2.0f : 10.0f * scale;
    d->octaves = 4;
    d->cave_threshold = 0.6f;
    d->cave_period = 24.0f * scale;
    d->seed = seed;
}

typedef struct {
    const vt_gen_desc* d;
    uint8_t* out;
    int z0, z1;
} slab_job;

/* terrain of columns z in [z0, z1): grass on top, 3 layers of dirt, stone
 * below, water in air under the water level, caves cut out of solid cells
 * above the bottom layer */
static void* fill_terrain(void* arg) {
    const slab_job* j = (const slab_job*)arg;
    const vt_gen_desc* d = j->d;
    const int X = d->dims[0], Y = d->dims[1];
    const int water = (int)ceil((double)d->water_level);
    const uint64_t cave_seed = purpose_seed(d->seed, P_CAVES);
    const double cave_f = 1.0 / (double)d->cave_period;
    for (int z = j->z0; z < j->z1; ++z)
        for (int x = 0; x < X; ++x) {
            const int h = column_height(d, x, z);
            uint8_t* col = j->out + (size_t)x + (size_t)X * (size_t)Y * (size_t)z;
            for (int y = 0; y < Y; ++y) {
                uint8_t m = 0;
                if (y < h) {
                    m = y == h - 1 ? 1 : (y >= h - 4 ? 2 : 3);
                    if (d->caves && y > 0 &&
                        fbm_3d(cave_seed, (double)x, (double)y, (double)z, cave_f) > (double)d->cave_threshold)
                        m = 0;
                } else if (y < water) {
                    m = 4;
                }
                col[(size_t)X * (size_t)y] = m;
            }
        }
    return NULL;
}

/* tree t: column from draws 2t+1 and 2t+2 of the tree stream; 0 when it does
 * not fit under the top of the world */
static int tree_at(const vt_gen_desc* d, int t, int* x, int* z, int* h) {
    const uint64_t s0 = purpose_seed(d->seed, P_TREES);
    *x = 2 + (int)(draw(s0, (uint64_t)(2 * t + 1)) * (double)(d->dims[0] - 4));
    *z = 2 + (int)(draw(s0, (uint64_t)(2 * t + 2)) * (double)(d->dims[2] - 4));
    *h = column_height(d, *x, *z);
    return *h + 8 < d->dims[1];
}

static int leaf_kept(uint64_t leaf_seed, int t, int dx, int dy, int dz) {
    const uint64_t cell = (uint64_t)((dx + 2) + 5 * ((dy + 2) + 5 * (dz + 2)));
    return (double)(mix(leaf_seed ^ mix(((uint64_t)t << 20) ^ cell)) >> 11) * 0x1p-53 < 0.7;
}

int32_t vto_gen_world(const vt_gen_desc* d, uint8_t* out, size_t nbytes, int32_t threads) {
    const int X = d->dims[0], Y = d->dims[1], Z = d->dims[2];
    if (X < 1 || Y < 1 || Z < 1 || nbytes != (size_t)X * Y * Z) return 1;
    int nt = threads > 0 ? threads : 1;
    if (nt > Z) nt = Z;
    if (nt > 256) nt = 256;
    pthread_t tid[256];
    slab_job jobs[256];
    for (int i = 0; i < nt; ++i) {
        jobs[i].d = d;
        jobs[i].out = out;
        jobs[i].z0 = (int)((int64_t)Z * i / nt);
        jobs[i].z1 = (int)((int64_t)Z * (i + 1) / nt);
        pthread_create(&tid[i], NULL, fill_terrain, &jobs[i]);
    }
    for (int i = 0; i < nt; ++i) pthread_join(tid[i], NULL);
    if (X < 6 || Z < 6) return 0;
    /* trees in order: trunk over anything, then leaves into air or water */
    const uint64_t leaf_seed = purpose_seed(d->seed, P_LEAVES);
    for (int t = 0; t < d->trees; ++t) {
        int x, z, h;
        if (!tree_at(d, t, &x, &z, &h)) continue;
        for (int y = h; y < h + 6; ++y) out[(size_t)x + (size_t)X * ((size_t)y + (size_t)Y * z)] = 5;
        for (int dz = -2; dz <= 2; ++dz)
            for (int dy = -2; dy <= 2; ++dy)
                for (int dx = -2; dx <= 2; ++dx) {
                    const int lx = x + dx, ly = h + 5 + dy, lz = z + dz;
                    if (lx < 0 || lz < 0 || lx >= X || lz >= Z || ly >= Y) continue;
                    uint8_t* c = out + (size_t)lx + (size_t)X * ((size_t)ly + (size_t)Y * lz);
                    if ((*c == 0 || *c == 4) && leaf_kept(leaf_seed, t, dx, dy, dz)) *c = 6;
                }
    }
    return 0;
}

/* sine and cosine of x: x = k pi/2 + r with pi/2 split in three parts, then
 * Taylor series of r to degree 21 (sine) and 20 (cosine) */
static void sin_cos(double x, double* s, double* c) {
    const double k = floor(x * 0x1.45f306dc9c883p-1 + 0.5);
    double r = x - k * 0x1.921fb5p+0;
    r = r - k * 0x1.110b46p-26;
    r = r - k * 0x1.1a62633145c07p-54;
    const double r2 = r * r;
    double sn = 0.0, cs = 0.0, term = r;
    for (int n = 1; n <= 21; n += 2) {
        sn += term;
        term = -term * r2 / (double)((n + 1) * (n + 2));
    }
    term = 1.0;
    for (int n = 0; n <= 20; n += 2) {
        cs += term;
        term = -term * r2 / (double)((n + 1) * (n + 2));
    }
    switch (((int)(int64_t)k) & 3) {
        case 0: *s = sn; *c = cs; break;
        case 1: *s = cs; *c = -sn; break;
        case 2: *s = -sn; *c = -cs; break;
        default: *s = -cs; *c = sn; break;
    }
}

static const double PI = 3.14159265358979323846;

int32_t vto_camera_look(const float pos[3], float yaw, float pitch, float fov, int32_t width, int32_t height,
                        vt_camera* out) {
    if (width <= 0 || height <= 0 || !(fov > 0.0f) || !(fov < 3.1f)) return 1;
    memset(out, 0, sizeof(*out));
    double sy, cy, sp, cp, sh, ch;
    sin_cos((double)yaw, &sy, &cy);
    sin_cos((double)pitch, &sp, &cp);
    sin_cos(0.5 * (double)fov, &sh, &ch);
    /* rows of the view matrix: right, up, forward (row-vector convention) */
    const double rows[3][3] = {{cy, 0.0, -sy}, {-sp * sy, cp, -sp * cy}, {cp * sy, sp, cp * cy}};
    for (int r = 0; r < 3; ++r)
        for (int j = 0; j < 3; ++j) out->view[4 * r + j] = (float)rows[r][j];
    for (int j = 0; j < 3; ++j) out->pos[j] = pos[j];
    out->pos[3] = 1.0f;
    out->view[15] = 1.0f;
    out->fov = fov;
    out->tan_half_fov = (float)(sh / ch);
    out->width = width;
    out->height = height;
    return 0;
}

int32_t vto_gen_camera(const vt_gen_desc* d, uint64_t seed, int32_t width, int32_t height, vt_camera* out) {
    const uint64_t s0 = purpose_seed(d->seed ^ mix(seed), P_CAMERA);
    const double fx = (0.1 + 0.8 * draw(s0, 1)) * (double)d->dims[0];
    const double fz = (0.1 + 0.8 * draw(s0, 2)) * (double)d->dims[2];
    const double yaw = 2.0 * PI * draw(s0, 3);
    const double pitch = -(PI / 6.0) * draw(s0, 4);
    const int h = column_height(d, (int)fx, (int)fz);
    const double top = (double)h > (double)d->water_level ? (double)h : (double)d->water_level;
    double y = top + (double)d->camera_height + 0.5;
    if (y > (double)d->dims[1] - 0.5) y = (double)d->dims[1] - 0.5;
    const float pos[3] = {(float)fx, (float)y, (float)fz};
    return vto_camera_look(pos, (float)yaw, (float)pitch, (float)(70.0 * PI / 180.0), width, height, out);
}

static uint32_t rgba(unsigned r, unsigned g, unsigned b) { return r | (g << 8) | (b << 16) | (255u << 24); }

void vto_default_palette(uint32_t pal[256]) {
    static const unsigned named[7][3] = {{0, 0, 0},      {86, 160, 60}, {134, 96, 67}, {125, 125, 125},
                                         {50, 90, 200}, {110, 80, 50},  {60, 130, 50}};
    pal[0] = 0;
    for (int i = 1; i < 7; ++i) pal[i] = rgba(named[i][0], named[i][1], named[i][2]);
    for (unsigned i = 7; i < 256; ++i) {
        const uint64_t h = mix(0xC0104ull + i);
        pal[i] = rgba((unsigned)(h & 255u), (unsigned)((h >> 8) & 255u), (unsigned)((h >> 16) & 255u));
    }
}

void vto_gen_sun(uint64_t seed, float out[3]) {
    const uint64_t s0 = purpose_seed(seed, P_SUN);
    const double elevation = (20.0 + 40.0 * draw(s0, 1)) * PI / 180.0;
    const double azimuth = 2.0 * PI * draw(s0, 2);
    double se, ce, sa, ca;
    sin_cos(elevation, &se, &ce);
    sin_cos(azimuth, &sa, &ca);
    out[0] = (float)(ce * sa);
    out[1] = (float)se;
    out[2] = (float)(ce * ca);
}
