/*
 * vt_oracle.c -- CPU oracle (TEST INFRASTRUCTURE ONLY, see vt_oracle.h).
 *
 * Build: gcc -std=c11 -O2 -ffp-contract=off -fno-fast-math -fPIC -shared -pthread
 * (oracle/build.py).  Every float expression below is evaluated exactly as
 * written: no contraction into FMA unless fmaf() is spelled out.
 */
#include "vt_oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

#define CHUNK 32

/* ======================================================================
 * Mode P: plane-indexed Amanatides-Woo traversal (unit steps).
 *
 * For axis i the ray crosses the integer plane k at
 *     ptime_i(k) = fmaf((float)k, inv_i, -(o_i * inv_i)),   inv_i = 1/d_i,
 * a pure function of k, so every consumer computes identical crossing times.
 * Crossing events are ordered by (t ascending, axis descending): the
 * reference's selection chain
 *     t.x < t.y ? (t.x < t.z ? 0 : 2) : (t.y < t.z ? 1 : 2)   (map.glsl:158)
 * picks the smallest t and, on ties, the higher axis.
 * ====================================================================== */

typedef struct {
    float o[3], d[3], inv[3], oinv[3];
    int   pos[3];
} pray;

static float ptime(const pray* r, int i, int k) {
    return fmaf((float)k, r->inv[i], r->oinv[i]);
}

/* key(ta, a) < key(tb, b) */
static int key_lt(float ta, int a, float tb, int b) {
    return ta < tb || (ta == tb && a > b);
}

static void pray_init(pray* r, const float o[3], const float d[3]) {
    for (int i = 0; i < 3; ++i) {
        float di = d[i];
        if (di == 0.0f) di = 0.001f; /* map.glsl:85-90 */
        r->o[i] = o[i];
        r->d[i] = di;
        r->inv[i] = 1.0f / di;
        r->oinv[i] = -(o[i] * r->inv[i]);
        r->pos[i] = di > 0.0f;
    }
}

/* Is plane k of axis i crossed strictly before the event (T, e)? */
static int crossed(const pray* r, int i, int k, float T, int e) {
    return key_lt(ptime(r, i, k), i, T, e);
}

/* Cell of axis i (i != e) at the event (T, e), by bisection over [0, D-1].
 * Positive direction: the largest c whose lower plane c is crossed.
 * Negative direction: the smallest c whose upper plane c+1 is crossed. */
static int cell_at(const pray* r, int i, int D, float T, int e) {
    int lo = 0, hi = D - 1;
    if (r->pos[i]) {
        /* predicate crossed(c) is true for small c, false for large c */
        while (lo < hi) {
            int mid = lo + (hi - lo + 1) / 2;
            if (crossed(r, i, mid, T, e)) lo = mid; else hi = mid - 1;
        }
    } else {
        /* predicate crossed(c+1) is false for small c, true for large c */
        while (lo < hi) {
            int mid = lo + (hi - lo) / 2;
            if (crossed(r, i, mid + 1, T, e)) hi = mid; else lo = mid + 1;
        }
    }
    return lo;
}

/* Start state of a ray against the grid box [0, D).  Returns 0 on a miss. */
static int pray_start(const pray* r, const int32_t D[3], int c[3], float* t0, int* axis0) {
    float tin[3], tout[3];
    for (int i = 0; i < 3; ++i) {
        int a = r->pos[i] ? 0 : D[i];
        int b = r->pos[i] ? D[i] : 0;
        tin[i] = ptime(r, i, a);
        tout[i] = ptime(r, i, b);
    }
    /* entry = latest entry event (max key), exit = earliest exit event */
    int e = 0, x = 0;
    for (int i = 1; i < 3; ++i) {
        if (key_lt(tin[e], e, tin[i], i)) e = i;
        if (key_lt(tout[i], i, tout[x], x)) x = i;
    }
    float T0 = tin[e], T1 = tout[x];
    if (!key_lt(T0, e, T1, x)) return 0; /* box missed */
    if (!(T1 > 0.0f)) return 0;          /* box behind the origin */
    if (T0 >= 0.0f) {
        for (int i = 0; i < 3; ++i) {
            if (i == e) c[i] = r->pos[i] ? 0 : D[i] - 1;
            else c[i] = cell_at(r, i, D[i], T0, e);
        }
        *t0 = T0;
        *axis0 = e;
    } else {
        for (int i = 0; i < 3; ++i) {
            int ci = (int)floorf(r->o[i]);
            if (ci < 0) ci = 0;
            if (ci > D[i] - 1) ci = D[i] - 1;
            c[i] = ci;
        }
        *t0 = 0.0f;
        *axis0 = 0; /* the reference starts with minIdx = 0 (map.glsl:98) */
    }
    return 1;
}

int32_t vto_world_init(vto_world* w, const int32_t dims[3], const uint8_t* mats) {
    memset(w, 0, sizeof(*w));
    for (int i = 0; i < 3; ++i) {
        w->dims[i] = dims[i];
        w->chunks[i] = (dims[i] + CHUNK - 1) / CHUNK;
    }
    w->mats = mats;
    size_t nch = (size_t)w->chunks[0] * w->chunks[1] * w->chunks[2];
    w->chunk_occ = (uint8_t*)calloc(nch, 1);
    if (!w->chunk_occ) return 1;
    for (int z = 0; z < dims[2]; ++z)
        for (int y = 0; y < dims[1]; ++y) {
            const uint8_t* row = mats + (size_t)dims[0] * (y + (size_t)dims[1] * z);
            for (int x = 0; x < dims[0]; ++x)
                if (row[x]) {
                    size_t ci = (size_t)(x / CHUNK) + w->chunks[0] * ((size_t)(y / CHUNK) + (size_t)w->chunks[1] * (z / CHUNK));
                    w->chunk_occ[ci] = 1;
                }
        }
    return 0;
}

void vto_world_free(vto_world* w) {
    free(w->chunk_occ);
    w->chunk_occ = NULL;
}

static uint8_t voxel_at(const vto_world* w, const int c[3]) {
    return w->mats[(size_t)c[0] + (size_t)w->dims[0] * ((size_t)c[1] + (size_t)w->dims[1] * (size_t)c[2])];
}

/* Index of the 64-bit brick word a kernel consults for cell c (chunk-major,
 * 512 bricks per chunk); only compared for equality by the counters. */
static uint64_t brick_word(const vto_world* w, const int c[3], uint64_t* chunk_index) {
    uint64_t ci = (uint64_t)(c[0] >> 5) + (uint64_t)w->chunks[0] * ((uint64_t)(c[1] >> 5) + (uint64_t)w->chunks[1] * (uint64_t)(c[2] >> 5));
    uint64_t bi = (uint64_t)((c[0] >> 2) & 7) + 8u * ((uint64_t)((c[1] >> 2) & 7) + 8u * (uint64_t)((c[2] >> 2) & 7));
    *chunk_index = ci;
    return ci * 512u + bi;
}

static void trace_ray(const vto_world* w, const pray* r, int32_t max_steps, vto_trace* out) {
    int c[3];
    float t;
    int axis;
    memset(out, 0, sizeof(*out));
    out->voxel = 0xFFFFFFFFu;
    out->face = -1;
    out->t = -1.0f;
    if (!pray_start(r, w->dims, c, &t, &axis)) return;

    uint64_t last_word = ~(uint64_t)0, last_coarse = ~(uint64_t)0;
    for (int32_t n = 0; n < max_steps; ++n) {
        if ((unsigned)c[0] >= (unsigned)w->dims[0] || (unsigned)c[1] >= (unsigned)w->dims[1] ||
            (unsigned)c[2] >= (unsigned)w->dims[2])
            break;
        uint64_t ci;
        uint64_t wi = brick_word(w, c, &ci);
        if ((ci >> 6) != last_coarse) {
            last_coarse = ci >> 6;
            out->coarse_words++;
        }
        if (w->chunk_occ[ci]) {
            if (wi != last_word) {
                last_word = wi;
                out->mask_words++;
            }
            uint8_t m = voxel_at(w, c);
            if (m) {
                out->hit = 1;
                out->material = m;
                out->voxel = (uint32_t)((uint64_t)c[0] + (uint64_t)w->dims[0] * ((uint64_t)c[1] + (uint64_t)w->dims[1] * (uint64_t)c[2]));
                out->cell[0] = c[0]; out->cell[1] = c[1]; out->cell[2] = c[2];
                out->t = t;
                out->axis = axis;
                out->face = 2 * axis + (r->pos[axis] ? 0 : 1);
                out->steps = n;
                return;
            }
        }
        /* one unit crossing */
        float tn[3];
        for (int i = 0; i < 3; ++i) tn[i] = ptime(r, i, r->pos[i] ? c[i] + 1 : c[i]);
        int e = tn[0] < tn[1] ? (tn[0] < tn[2] ? 0 : 2) : (tn[1] < tn[2] ? 1 : 2);
        t = tn[e];
        axis = e;
        c[e] += r->pos[e] ? 1 : -1;
        out->steps = n + 1;
    }
}

void vto_trace_p(const vto_world* w, const float o[3], const float d[3], int32_t max_steps, vto_trace* out) {
    pray r;
    pray_init(&r, o, d);
    trace_ray(w, &r, max_steps, out);
}

/* ======================================================================
 * Deterministic sine / cosine (bounce directions).  Cody-Waite reduction by
 * pi/2 split into three floats (1.5703125 + 0x1.fb4p-12 + 0x1.4442d2p-24,
 * each the leading bits of the remainder of the previous split) and Taylor
 * polynomials of degree 9 (sin) and 10 (cos) on |r| <= pi/4, all in fmaf.
 * ====================================================================== */
static void sincos_core(float x, float* s, float* c) {
    float k = rintf(x * 0x1.45f306p-1f); /* 2/pi */
    float r = fmaf(-k, 0x1.92p+0f, x);
    r = fmaf(-k, 0x1.fb4p-12f, r);
    r = fmaf(-k, 0x1.4442d2p-24f, r);
    float r2 = r * r;
    float ps = fmaf(r2, 1.0f / 362880.0f, -1.0f / 5040.0f);
    ps = fmaf(r2, ps, 1.0f / 120.0f);
    ps = fmaf(r2, ps, -1.0f / 6.0f);
    ps = fmaf(r2 * r, ps, r);
    float pc = fmaf(r2, -1.0f / 3628800.0f, 1.0f / 40320.0f);
    pc = fmaf(r2, pc, -1.0f / 720.0f);
    pc = fmaf(r2, pc, 1.0f / 24.0f);
    pc = fmaf(r2, pc, -0.5f);
    pc = fmaf(r2, pc, 1.0f);
    int q = ((int)k) & 3;
    switch (q) {
        case 0: *s = ps; *c = pc; break;
        case 1: *s = pc; *c = -ps; break;
        case 2: *s = -ps; *c = -pc; break;
        default: *s = -pc; *c = ps; break;
    }
}
float vto_sinf(float x) { float s, c; sincos_core(x, &s, &c); return s; }
float vto_cosf(float x) { float s, c; sincos_core(x, &s, &c); return c; }

/* ======================================================================
 * Ray generation and shading.
 * ====================================================================== */

/* primary.comp.glsl:31-39, with a 3-D normalisation of the direction. */
static void primary_ray(const vt_camera* cam, int px, int py, float o[3], float d[3]) {
    float W = (float)cam->width, H = (float)cam->height;
    float u = ((float)px / W) * 2.0f - 1.0f;
    float v = ((float)py / H) * 2.0f - 1.0f;
    v = v * (H / W);
    u = u * cam->tan_half_fov;
    v = v * cam->tan_half_fov;
    const float* M = cam->view;
    float q[3];
    for (int j = 0; j < 3; ++j) q[j] = ((u * M[0 * 4 + j] + v * M[1 * 4 + j]) + M[2 * 4 + j]) + M[3 * 4 + j];
    float n2 = (q[0] * q[0] + q[1] * q[1]) + q[2] * q[2];
    float len = sqrtf(n2);
    for (int j = 0; j < 3; ++j) {
        d[j] = q[j] / len;
        o[j] = cam->pos[j];
    }
}

/* Entity occluders (traceEntities' role in secondary.comp.glsl:42-46, as a
 * list of boxes): the ray o + t d, t >= 0, against the closed box {lo, hi};
 * slab test with IEEE division, an axis without motion must lie in its slab. */
static int ray_box(const float o[3], const float d[3], const float* box) {
    float tmin = 0.0f, tmax = INFINITY;
    for (int j = 0; j < 3; ++j) {
        if (d[j] == 0.0f) {
            if (o[j] < box[j] || o[j] > box[3 + j]) return 0;
            continue;
        }
        const float a = (box[j] - o[j]) / d[j], b = (box[3 + j] - o[j]) / d[j];
        const float lo = a < b ? a : b, hi = a < b ? b : a;
        if (lo > tmin) tmin = lo;
        if (hi < tmax) tmax = hi;
    }
    return tmin <= tmax;
}

static int entity_occluded(const vto_world* w, const float o[3], const float d[3]) {
    for (int i = 0; i < w->n_entities; ++i)
        if (ray_box(o, d, w->entities + 6 * i)) return 1;
    return 0;
}

static float clampf(float x, float a, float b) { return x < a ? a : (x > b ? b : x); }

static uint32_t unorm8(float x) { return (uint32_t)(int)rintf(clampf(x, 0.0f, 1.0f) * 255.0f); }

static float dot3(const float a[3], const float b[3]) { return (a[0] * b[0] + a[1] * b[1]) + a[2] * b[2]; }

static void normalize3(const float a[3], float out[3]) {
    float len = sqrtf(dot3(a, a));
    out[0] = a[0] / len; out[1] = a[1] / len; out[2] = a[2] / len;
}

/* SkyDome2 (camera.glsl:11-19) with the sun direction as a parameter and the
 * integer powers written as products. */
static void sky(const float sun[3], const float rd[3], float col[3]) {
    float sn[3], rn[3];
    normalize3(sun, sn);
    normalize3(rd, rn);
    float s = clampf(dot3(sn, rn), 0.0f, 1.2f);
    float s2 = s * s, s3 = s2 * s, s4 = s2 * s2, s8 = s4 * s4;
    float dy = rd[1] * 0.2f;
    col[0] = ((0.6f - dy * 1.0f) + (0.15f * 0.5f)) + (0.4f * 1.0f) * s8 + 0.2f * s3;
    col[1] = ((0.71f - dy * 0.5f) + (0.15f * 0.5f)) + (0.4f * 0.6f) * s8 + 0.08f * s3;
    col[2] = ((0.75f - dy * 1.0f) + (0.15f * 0.5f)) + (0.4f * 0.1f) * s8 + 0.04f * s3;
}

static float vignette(int px, int py, int W, int H) {
    float u = ((float)px + 0.5f) / (float)W;
    float v = ((float)py + 0.5f) / (float)H;
    float a = u * (1.0f - u), b = v * (1.0f - v);
    return powf(a * b * 15.0f, 0.18f);
}

static int crosshair(int px, int py, int W, int H) {
    float u = ((float)px + 0.5f) / (float)W - 0.5f;
    float v = ((float)py + 0.5f) / (float)H - 0.5f;
    return sqrtf(u * u + v * v) <= 0.002f;
}

static uint32_t wang_hash(uint32_t* seed) { /* rng.glsl:16-24 */
    uint32_t s = (*seed ^ 61u) ^ (*seed >> 16);
    s *= 9u;
    s = s ^ (s >> 4);
    s *= 0x27d4eb2du;
    s = s ^ (s >> 15);
    *seed = s;
    return s;
}

static float rand01(uint32_t* seed) { return (float)wang_hash(seed) * 0x1p-32f; }

static void cross3(const float a[3], const float b[3], float o[3]) {
    o[0] = a[1] * b[2] - a[2] * b[1];
    o[1] = a[2] * b[0] - a[0] * b[2];
    o[2] = a[0] * b[1] - a[1] * b[0];
}

/* CosineSampleHemisphere (rng.glsl:41-55). */
static void cosine_hemisphere(const float n[3], uint32_t* seed, float out[3]) {
    float u1 = rand01(seed), u2 = rand01(seed);
    float r = sqrtf(u1);
    float theta = 6.28f * u2;
    const float up[3] = {0.0f, 1.0f, 1.0f};
    float b0[3], B[3], T[3];
    cross3(n, up, b0);
    normalize3(b0, B);
    cross3(B, n, T);
    float st = vto_sinf(theta), ct = vto_cosf(theta);
    float rs = r * st, rc = r * ct, h = sqrtf(1.0f - u1);
    float v[3];
    for (int j = 0; j < 3; ++j) v[j] = (rs * B[j] + h * n[j]) + rc * T[j];
    normalize3(v, out);
}

static void add_counts(vt_stats* st, const vto_trace* tr) {
    if (!st) return;
    st->mask_words += tr->mask_words;
    st->coarse_words += tr->coarse_words;
    st->steps += (uint64_t)tr->steps;
}

static void shade_pixel(const vto_world* w, const uint32_t* palette, const vt_camera* cam,
                        const vt_params* p, int px, int py, vt_hit* out, vt_stats* st) {
    float o[3], d[3];
    primary_ray(cam, px, py, o, d);
    vto_trace tr;
    pray r;
    pray_init(&r, o, d);
    trace_ray(w, &r, p->max_steps, &tr);
    if (st) {
        st->primary_rays++;
        st->record_bytes += 16;
        add_counts(st, &tr);
    }
    vt_hit h;
    memset(&h, 0, sizeof(h));
    float col[4] = {0, 0, 0, 0};
    int W = cam->width, H = cam->height;
    if (tr.hit) {
        if (st) { st->primary_hits++; st->material_bytes++; }
        h.voxel = tr.voxel;
        h.t = tr.t;
        h.face = (uint8_t)tr.face;
        h.material = tr.material;
        h.flags = VT_HIT_PRIMARY;
        uint32_t alb = palette[tr.material];
        float albf[4];
        for (int j = 0; j < 4; ++j) albf[j] = (float)((alb >> (8 * j)) & 255u) / 255.0f;
        /* entry point on the hit face, pushed 0.001 back along the normal
         * (secondary.comp.glsl:37) */
        int e = tr.axis;
        float nrm[3] = {0.0f, 0.0f, 0.0f};
        nrm[e] = r.pos[e] ? -1.0f : 1.0f;
        float so[3];
        for (int j = 0; j < 3; ++j) so[j] = fmaf(r.d[j], tr.t, o[j]);
        so[e] = so[e] + nrm[e] * 0.001f;
        int shadowed = 0;
        if (p->rays & VT_RAYS_SHADOW) {
            vto_trace ts;
            vto_trace_p(w, so, p->sun_dir, p->shadow_max_steps, &ts);
            if (st) { st->shadow_rays++; add_counts(st, &ts); }
            if (ts.hit) {
                shadowed = 1;
                h.flags |= VT_HIT_SHADOWED;
                if (st) st->shadow_hits++;
            } else if (entity_occluded(w, so, p->sun_dir)) {
                shadowed = 1;
                h.flags |= VT_HIT_ENTITY;
            }
        }
        int bounce_open = 0;
        float bdir[3] = {0, 0, 0};
        if (p->rays & VT_RAYS_BOUNCE) {
            uint32_t seed = ((uint32_t)px * 1973u + (uint32_t)py * 9277u) ^ p->seed;
            cosine_hemisphere(nrm, &seed, bdir);
            vto_trace tb;
            vto_trace_p(w, so, bdir, p->bounce_max_steps, &tb);
            if (st) { st->bounce_rays++; add_counts(st, &tb); }
            if (tb.hit) {
                h.flags |= VT_HIT_BOUNCE;
                if (st) st->bounce_hits++;
            } else {
                bounce_open = 1;
            }
        }
        if (p->shade == VT_SHADE_REFERENCE) {
            /* illumination.a stored in RGBA8: +0.3 -> 76/255 (0.3f * 255
             * rounds to 76.5, ties to even), -0.3 -> 0
             * (secondary.comp.glsl:45-48, gbuffer.zig:13) */
            float a = shadowed ? 0.0f : (float)unorm8(0.3f) / 255.0f;
            float sq[3];
            for (int j = 0; j < 3; ++j) sq[j] = (float)unorm8(p->sun_dir[j]) / 255.0f;
            float sc[3];
            sky(p->sun_dir, sq, sc);
            for (int j = 0; j < 3; ++j) col[j] = albf[j] + a * sc[j];
            col[3] = albf[3] + a * 1.0f;
            if (bounce_open) {
                float bc[3];
                sky(p->sun_dir, bdir, bc);
                for (int j = 0; j < 3; ++j) col[j] = col[j] + p->bounce_weight * (albf[j] * bc[j]);
            }
        } else if (p->shade == VT_SHADE_LAMBERT) {
            float sn[3];
            normalize3(p->sun_dir, sn);
            float ndl = dot3(nrm, sn);
            if (ndl < 0.0f) ndl = 0.0f;
            float vis = shadowed ? 0.0f : 1.0f;
            float k = p->ambient + p->diffuse * ndl * vis;
            for (int j = 0; j < 3; ++j) col[j] = albf[j] * k;
            col[3] = 1.0f;
        } else {
            for (int j = 0; j < 4; ++j) col[j] = albf[j];
        }
    } else {
        h.voxel = 0xFFFFFFFFu;
        h.t = -1.0f;
        h.face = 0xFF;
        h.material = 0;
        if (p->shade == VT_SHADE_REFERENCE) {
            /* sky stored into the RGBA8 albedo image (primary.comp.glsl:65) */
            float sc[3];
            sky(p->sun_dir, d, sc);
            for (int j = 0; j < 3; ++j) col[j] = (float)unorm8(sc[j]) / 255.0f;
            col[3] = 1.0f;
        }
    }
    if (p->shade == VT_SHADE_REFERENCE) {
        if ((p->flags & VT_FLAG_CROSSHAIR) && crosshair(px, py, W, H)) {
            col[0] = col[0] * 0.5f + 0.5f;
            col[1] = col[1] * 0.5f + 0.5f;
            col[2] = col[2] * 0.5f + 0.5f;
            col[3] = col[3] * 0.5f + 0.2f;
        }
        if (p->flags & VT_FLAG_VIGNETTE) {
            float g = vignette(px, py, W, H);
            for (int j = 0; j < 4; ++j) col[j] = g * col[j];
        }
    }
    if (p->shade == VT_SHADE_NONE) {
        h.rgba = tr.hit ? palette[tr.material] : 0u;
    } else {
        h.rgba = unorm8(col[0]) | (unorm8(col[1]) << 8) | (unorm8(col[2]) << 16) | (unorm8(col[3]) << 24);
    }
    *out = h;
}

void vto_primary_rays(const vt_camera* cam, int32_t row_step, float* origins, float* dirs) {
    if (row_step < 1) row_step = 1;
    size_t k = 0;
    for (int py = 0; py < cam->height; py += row_step)
        for (int px = 0; px < cam->width; ++px, ++k) primary_ray(cam, px, py, origins + 3 * k, dirs + 3 * k);
}

void vto_render_rows(const vto_world* w, const uint32_t* palette, const vt_camera* cam,
                     const vt_params* p, vt_hit* out, int32_t y0, int32_t y1, vt_stats* st) {
    for (int32_t y = y0; y < y1; ++y)
        for (int32_t x = 0; x < cam->width; ++x)
            shade_pixel(w, palette, cam, p, x, y, out + (size_t)y * cam->width + x, st);
}

typedef struct {
    const vto_world* w;
    const uint32_t* palette;
    const vt_camera* cam;
    const vt_params* p;
    vt_hit* out;
    int32_t first, stride;
    vt_stats st;
    int want_stats;
} job_t;

static void* worker(void* arg) {
    job_t* j = (job_t*)arg;
    for (int32_t y = j->first; y < j->cam->height; y += j->stride)
        vto_render_rows(j->w, j->palette, j->cam, j->p, j->out, y, y + 1, j->want_stats ? &j->st : NULL);
    return NULL;
}

static void stats_add(vt_stats* a, const vt_stats* b) {
    const uint64_t* s = (const uint64_t*)b;
    uint64_t* d = (uint64_t*)a;
    for (size_t i = 0; i < sizeof(vt_stats) / sizeof(uint64_t); ++i) d[i] += s[i];
}

int32_t vto_render_sampled(const vto_world* w, const uint32_t* palette, const vt_camera* cam,
                           const vt_params* p, vt_hit* out, int32_t threads, int32_t row_step,
                           vt_stats* st) {
    if (threads < 1) threads = 1;
    if (row_step < 1) row_step = 1;
    job_t* jobs = (job_t*)calloc((size_t)threads, sizeof(job_t));
    pthread_t* tids = (pthread_t*)calloc((size_t)threads, sizeof(pthread_t));
    if (!jobs || !tids) { free(jobs); free(tids); return 1; }
    for (int32_t i = 0; i < threads; ++i) {
        jobs[i].w = w; jobs[i].palette = palette; jobs[i].cam = cam; jobs[i].p = p; jobs[i].out = out;
        jobs[i].first = i * row_step;
        jobs[i].stride = threads * row_step;
        jobs[i].want_stats = st != NULL;
    }
    for (int32_t i = 0; i < threads; ++i) pthread_create(&tids[i], NULL, worker, &jobs[i]);
    for (int32_t i = 0; i < threads; ++i) pthread_join(tids[i], NULL);
    if (st) {
        memset(st, 0, sizeof(*st));
        for (int32_t i = 0; i < threads; ++i) stats_add(st, &jobs[i].st);
    }
    free(jobs);
    free(tids);
    return 0;
}

int32_t vto_render(const vto_world* w, const uint32_t* palette, const vt_camera* cam,
                   const vt_params* p, vt_hit* out, int32_t threads, vt_stats* st) {
    return vto_render_sampled(w, palette, cam, p, out, threads, 1, st);
}

void vto_trace_rays(const vto_world* w, const float* origins, const float* dirs, int32_t n,
                    int32_t max_steps, vt_hit* out) {
    for (int32_t i = 0; i < n; ++i) {
        vto_trace tr;
        vto_trace_p(w, origins + 3 * i, dirs + 3 * i, max_steps, &tr);
        vt_hit h;
        memset(&h, 0, sizeof(h));
        h.voxel = tr.voxel;
        h.t = tr.t;
        h.face = tr.hit ? (uint8_t)tr.face : 0xFF;
        h.material = tr.material;
        h.flags = tr.hit ? VT_HIT_PRIMARY : 0;
        h.rgba = 0u;
        out[i] = h;
    }
}

/* ======================================================================
 * Shading adjoint reference (FP64 arithmetic over the float traversal's
 * discrete hit and shadow sets).
 * ====================================================================== */
int32_t vto_shade_grad_f64(const vto_world* w, const vt_camera* cam, const vt_hit* hits, const double* pal,
                           const double* alb, const double sun[3], double ka, double kd, int32_t shadow_max_steps,
                           const float* target, const uint8_t* vis_in, uint8_t* vis_out, double* rgb, double* loss,
                           double* g_pal, double* g_alb, double g_sun[3], double* a_pal, double* a_alb,
                           double a_sun[3]) {
    const double len = sqrt(sun[0] * sun[0] + sun[1] * sun[1] + sun[2] * sun[2]);
    if (!(len > 0.0)) return 1;
    const double sn[3] = {sun[0] / len, sun[1] / len, sun[2] / len};
    const float sunf[3] = {(float)sun[0], (float)sun[1], (float)sun[2]};
    const int W = cam->width, H = cam->height;
    for (int py = 0; py < H; ++py)
        for (int px = 0; px < W; ++px) {
            const size_t p = (size_t)py * W + px;
            const vt_hit* h = hits + p;
            double c[3] = {0.0, 0.0, 0.0};
            int lit = 0;
            const int hit = (h->flags & VT_HIT_PRIMARY) != 0;
            double shade = 0.0, albv = 1.0, ndl = 0.0;
            double nrm[3] = {0.0, 0.0, 0.0};
            const int m = h->material;
            if (hit) {
                const int axis = h->face >> 1;
                const int pos = (h->face & 1) == 0;
                float o[3], d[3];
                primary_ray(cam, px, py, o, d);
                pray r;
                pray_init(&r, o, d);
                float so[3], nf[3] = {0.0f, 0.0f, 0.0f};
                nf[axis] = pos ? -1.0f : 1.0f;
                nrm[axis] = nf[axis];
                for (int j = 0; j < 3; ++j) so[j] = fmaf(r.d[j], h->t, o[j]);
                so[axis] = so[axis] + nf[axis] * 0.001f;
                if (vis_in) {
                    lit = vis_in[p] != 0;
                } else {
                    vto_trace ts;
                    vto_trace_p(w, so, sunf, shadow_max_steps, &ts);
                    lit = !ts.hit && !entity_occluded(w, so, sunf);
                }
                ndl = nrm[0] * sn[0] + nrm[1] * sn[1] + nrm[2] * sn[2];
                shade = ka + kd * (ndl > 0.0 ? ndl : 0.0) * (lit ? 1.0 : 0.0);
                albv = alb ? alb[h->voxel] : 1.0;
                for (int k = 0; k < 3; ++k) c[k] = pal[3 * m + k] * albv * shade;
            }
            if (vis_out) vis_out[p] = (uint8_t)(hit && lit);
            if (rgb)
                for (int k = 0; k < 3; ++k) rgb[3 * p + k] = c[k];
            if (!target) continue;
            double g[3], gb = 0.0, ga = 0.0;
            for (int k = 0; k < 3; ++k) {
                const double diff = c[k] - (double)target[3 * p + k];
                g[k] = 2.0 * diff;
                if (loss) *loss += diff * diff;
            }
            if (!hit) continue;
            double aa = 0.0;
            for (int k = 0; k < 3; ++k) {
                if (g_pal) g_pal[3 * m + k] += g[k] * albv * shade;
                if (a_pal) a_pal[3 * m + k] += fabs(g[k] * albv * shade);
                ga += g[k] * pal[3 * m + k] * shade;
                aa += fabs(g[k] * pal[3 * m + k] * shade);
                gb += g[k] * pal[3 * m + k] * albv;
            }
            if (g_alb) g_alb[h->voxel] += ga;
            if (a_alb) a_alb[h->voxel] += aa;
            if (lit && ndl > 0.0)
                for (int k = 0; k < 3; ++k) {
                    const double term = gb * kd * (nrm[k] - ndl * sn[k]) / len;
                    if (g_sun) g_sun[k] += term;
                    if (a_sun) a_sun[k] += fabs(term);
                }
        }
    return 0;
}

/* ======================================================================
 * Mode R: traceMap (map.glsl:83-168) restated operation by operation.
 * GLSL float->int conversions truncate toward zero; float->uint saturates
 * negative values to 0 (as the GPU's conversion does).
 * ====================================================================== */
static uint32_t f2u(float x) { return x <= 0.0f ? 0u : (uint32_t)x; }

static uint32_t ref_chunk_flags(const vto_refworld* w, int x, int y, int z) { /* map.glsl:31-36 */
    if (x < 0 || y < 0 || z < 0 || x >= 64 || y >= 64 || z >= 64) return 0;
    return w->chunks[x + 64 * (y + z * 64)];
}

static uint32_t ref_get_voxel(const vto_refworld* w, int x, int y, int z) { /* map.glsl:38-47 */
    uint32_t blk = ref_chunk_flags(w, x >> 3, y >> 3, z >> 3);
    if (blk > 0) {
        uint64_t idx = (uint64_t)(blk - 1) * 512u + (uint64_t)((x % 8) + ((z % 8) * 8 + (y % 8)) * 8);
        if (idx >= w->ndata) return 0; /* outside the uploaded pool reads as empty */
        return w->data[idx];
    }
    return 0;
}

static uint32_t ref_get_subvoxel(const vto_refworld* w, uint32_t mdl, int x, int y, int z) { /* map.glsl:57-60 */
    int ox = (int)((mdl & 31u) * 8u), oy = (int)(((mdl / 32u) & 31u) * 8u), oz = (int)(((mdl / 1024u) & 31u) * 8u);
    int ax = x + ox, ay = y + oy, az = z + oz;
    return w->atlas[(size_t)ax + 256u * ((size_t)ay + 256u * (size_t)az)];
}

void vto_tracemap(const vto_refworld* w, const float o[3], const float din[3], int32_t max_steps, vto_refhit* out) {
    static const float normals[6][3] = {{-1, 0, 0}, {1, 0, 0}, {0, -1, 0}, {0, 1, 0}, {0, 0, -1}, {0, 0, 1}};
    float d[3] = {din[0], din[1], din[2]};
    for (int i = 0; i < 3; ++i)
        if (d[i] == 0.0f) d[i] = 0.001f;
    const int bounds = 8 * 512;
    int sgn[3], pos[3];
    float inv[3];
    for (int i = 0; i < 3; ++i) {
        sgn[i] = d[i] > 0.0f ? 1 : (d[i] < 0.0f ? -1 : 0);
        pos[i] = (1 + sgn[i]) >> 1;
        inv[i] = 1.0f / d[i];
    }
    int minIdx = 0;
    float t[3] = {1.0f, 1.0f, 1.0f};
    int g[3];
    float wc[3];
    for (int i = 0; i < 3; ++i) {
        g[i] = (int)(o[i] * 8.0f);
        wc[i] = o[i] * 8.0f - (float)g[i];
    }
    int stepSize = 0;
    out->data = 0;
    out->hit_pos[0] = out->hit_pos[1] = out->hit_pos[2] = -1.0f;
    out->normal[0] = out->normal[1] = out->normal[2] = 0.0f;
    out->iterations = 0;
    for (int step = 0; step < max_steps; ++step) {
        out->iterations = step + 1;
        if (g[0] >= bounds || g[1] >= bounds || g[2] >= bounds || g[0] < 0 || g[1] < 0 || g[2] < 0) break;
        uint32_t p[3];
        for (int i = 0; i < 3; ++i) p[i] = (uint32_t)g[i] + f2u(wc[i]);
        int pi[3] = {(int)p[0], (int)p[1], (int)p[2]};
        uint32_t block = ref_get_voxel(w, pi[0] >> 3, pi[1] >> 3, pi[2] >> 3);
        if (block != 0) {
            uint32_t sub = ref_get_subvoxel(w, block & 0xFFFFFFFu, pi[0] % 8, pi[1] % 8, pi[2] % 8);
            if (sub != 0) {
                uint32_t faceId = 0;
                if (minIdx == 0) faceId = (uint32_t)(-pos[0] + 2);
                if (minIdx == 1) faceId = (uint32_t)(-pos[1] + 4);
                if (minIdx == 2) faceId = (uint32_t)(-pos[2] + 6);
                out->data = sub;
                for (int i = 0; i < 3; ++i) {
                    out->hit_pos[i] = (float)g[i] + wc[i];
                    out->normal[i] = normals[faceId - 1][i];
                }
                return;
            } else if (stepSize != 0) {
                for (int i = 0; i < 3; ++i) {
                    g[i] += (int)wc[i];
                    wc[i] = wc[i] - floorf(wc[i]);
                }
                stepSize = 0;
            }
        } else if (stepSize != 3) {
            for (int i = 0; i < 3; ++i) {
                wc[i] += (float)(g[i] & 7);
                g[i] -= g[i] & 7;
            }
            stepSize = 3;
        }
        for (int i = 0; i < 3; ++i) t[i] = ((float)(pos[i] << stepSize) - wc[i]) * inv[i];
        minIdx = t[0] < t[1] ? (t[0] < t[2] ? 0 : 2) : (t[1] < t[2] ? 1 : 2);
        g[minIdx] += (int)((unsigned)sgn[minIdx] << stepSize);
        float tm = t[minIdx];
        for (int i = 0; i < 3; ++i) wc[i] += d[i] * tm;
        wc[minIdx] = (float)((1 - pos[minIdx]) << stepSize) * 0.999f;
    }
    out->data = 0;
    out->hit_pos[0] = out->hit_pos[1] = out->hit_pos[2] = -1.0f;
    out->normal[0] = out->normal[1] = out->normal[2] = 0.0f;
}

/* primary.comp.glsl:31-43 restated: uv, fov scale, C_view * vec4(uv, 1, 1)
 * with the matrix read column-major, 4-D normalisation, intersectAABB
 * (map.glsl:21-29) against [0, 512]^3, start at o + d * max(tNear, 0) - 0.001. */
static float fmin_g(float a, float b) { return b < a ? b : a; }
static float fmax_g(float a, float b) { return a < b ? b : a; }

/* primary.comp.glsl:38-43 from the final ray UV (fov factor applied). */
static void ray_r(const vto_refworld* w, const float cam_pos[4], const float view[16], float ux, float uy,
                  int32_t max_steps, float dir_out[3], vto_refhit* out) {
    const float v[4] = {ux, uy, 1.0f, 1.0f};
    float q[4];
    for (int i = 0; i < 4; ++i)
        q[i] = ((view[0 * 4 + i] * v[0] + view[1 * 4 + i] * v[1]) + view[2 * 4 + i] * v[2]) + view[3 * 4 + i] * v[3];
    const float len = sqrtf(((q[0] * q[0] + q[1] * q[1]) + q[2] * q[2]) + q[3] * q[3]);
    float d[3], o[3], t1[3];
    for (int i = 0; i < 3; ++i) {
        d[i] = q[i] / len;
        o[i] = cam_pos[i];
    }
    for (int i = 0; i < 3; ++i) {
        const float tmin = (0.0f - o[i]) / d[i];
        const float tmax = (512.0f - o[i]) / d[i];
        t1[i] = fmin_g(tmin, tmax);
    }
    const float tnear = fmax_g(fmax_g(t1[0], t1[1]), t1[2]);
    const float s = fmax_g(tnear, 0.0f);
    float start[3];
    for (int i = 0; i < 3; ++i) start[i] = (o[i] + d[i] * s) - 0.001f;
    for (int i = 0; i < 3; ++i) dir_out[i] = d[i];
    vto_tracemap(w, start, d, max_steps, out);
}

void vto_primary_r(const vto_refworld* w, const float cam_pos[4], const float view[16], float fov, int32_t px,
                   int32_t py, int32_t width, int32_t height, int32_t max_steps, float dir_out[3], vto_refhit* out) {
    float ux = (float)px / (float)width * 2.0f - 1.0f;
    float uy = (float)py / (float)height * 2.0f - 1.0f;
    uy *= (float)height / (float)width;
    const float th = tanf(fov / 2.0f);
    ux *= th;
    uy *= th;
    ray_r(w, cam_pos, view, ux, uy, max_steps, dir_out, out);
}

/* terrain_edit.comp.glsl:11-17 (the pick: UV 0, no fov factor, 64 steps) and
 * the edit of its commented-out tail (:19-24) through map_setVoxel
 * (map.glsl:49-55): place Voxel{ty = edit_mode - 1, is_solid} at
 * ivec3(hit_pos + normal) >> 3, or clear ivec3(hit_pos) >> 3; the write is
 * dropped where the chunk has no brick (and beyond the pool). */
void vto_edit_r(const vto_refworld* w, uint32_t* data, const float cam_pos[4], const float view[16],
                int32_t edit_mode, vto_refhit* out) {
    float dir[3];
    ray_r(w, cam_pos, view, 0.0f, 0.0f, 64, dir, out);
    if (edit_mode < 0 || out->data == 0) return;
    int p[3];
    uint32_t voxel;
    for (int i = 0; i < 3; ++i)
        p[i] = edit_mode > 0 ? ((int)(out->hit_pos[i] + out->normal[i])) >> 3 : ((int)out->hit_pos[i]) >> 3;
    voxel = edit_mode > 0 ? (1u << 28) + (uint32_t)edit_mode - 1u : 0u;
    const int cx = p[0] >> 3, cy = p[1] >> 3, cz = p[2] >> 3;
    if (cx < 0 || cy < 0 || cz < 0 || cx >= 64 || cy >= 64 || cz >= 64) return;
    const uint32_t blk = w->chunks[cx + 64 * (cy + 64 * cz)];
    if (blk == 0) return;
    const uint64_t idx = (uint64_t)(blk - 1) * 512u + (uint64_t)((p[0] % 8) + ((p[2] % 8) * 8 + (p[1] % 8)) * 8);
    if (idx < w->ndata) data[idx] = voxel;
}

/* The pick ray of terrain_edit.comp.glsl:11-17 on the mode-P world: the
 * primary ray of UV (0, 0) traced with max_steps; target = {x, y, z, valid}
 * of the voxel an edit with edit_mode would write (0: the hit voxel; > 0: the
 * voxel in front of the hit face, invalid outside the world; < 0: none). */
void vto_pick_p(const vto_world* w, const vt_camera* cam, int32_t max_steps, int32_t edit_mode, vto_trace* out,
                int32_t target[4]) {
    const float u = 0.0f, v = 0.0f;
    const float* M = cam->view;
    float q[3], o[3], d[3];
    for (int j = 0; j < 3; ++j) q[j] = ((u * M[0 * 4 + j] + v * M[1 * 4 + j]) + M[2 * 4 + j]) + M[3 * 4 + j];
    const float len = sqrtf((q[0] * q[0] + q[1] * q[1]) + q[2] * q[2]);
    for (int j = 0; j < 3; ++j) {
        d[j] = q[j] / len;
        o[j] = cam->pos[j];
    }
    vto_trace_p(w, o, d, max_steps, out);
    target[0] = target[1] = target[2] = target[3] = 0;
    if (!out->hit || edit_mode < 0) return;
    int c[3] = {out->cell[0], out->cell[1], out->cell[2]};
    if (edit_mode > 0) c[out->axis] += (out->face & 1) ? 1 : -1; /* face 2a: +dir (step back -1); 2a+1: -dir */
    for (int i = 0; i < 3; ++i)
        if (c[i] < 0 || c[i] >= w->dims[i]) return;
    target[0] = c[0];
    target[1] = c[1];
    target[2] = c[2];
    target[3] = 1;
}

/* ---------------------------------------------------------------------
 * The reference frame restated: secondary.comp.glsl, traceEntities,
 * SkyDome2 with powf, blit.fragment.glsl.  Images are RGBA8 except the
 * position (RGBA32F); stores round to nearest (rintf) after clamping.
 * --------------------------------------------------------------------- */
static const float kSunDir[3] = {7.52185881e-01f, 6.58950984e-01f, 7.52185881e-01f}; /* camera.glsl:8 */

static void aabb(const float o[3], const float d[3], const float lo[3], const float hi[3], float* tnear, float* tfar) {
    float t1[3], t2[3];
    for (int i = 0; i < 3; ++i) {
        const float a = (lo[i] - o[i]) / d[i];
        const float b = (hi[i] - o[i]) / d[i];
        t1[i] = fmin_g(a, b);
        t2[i] = fmax_g(a, b);
    }
    *tnear = fmax_g(fmax_g(t1[0], t1[1]), t1[2]);
    *tfar = fmin_g(fmin_g(t2[0], t2[1]), t2[2]);
}

static float dist3(const float a[3], const float b[3]) {
    const float x = a[0] - b[0], y = a[1] - b[1], z = a[2] - b[2];
    return sqrtf((x * x + y * y) + z * z);
}

void vto_trace_entities(const float o[3], const float d[3], float max_distance, vto_refhit* out) {
    static const float pos[5][3] = {{256.f, 21.f, 256.f}, {251.f, 21.f, 259.f}, {253.f, 21.f, 256.f},
                                    {251.f, 21.f, 256.f}, {257.f, 21.f, 261.f}};
    float prev = 1.0f / 0.0f;
    uint32_t id = 0xFFFFFFFFu;
    for (int i = 0; i < 5; ++i) {
        if (dist3(o, pos[i]) >= max_distance) continue;
        const float hi[3] = {pos[i][0] + 1.0f, pos[i][1] + 1.0f, pos[i][2] + 1.0f};
        float tn, tf;
        aabb(o, d, pos[i], hi, &tn, &tf);
        if (tf >= tn && prev >= tf) {
            id = (uint32_t)i;
            prev = tf;
        }
    }
    memset(out, 0, sizeof(*out));
    if (id != 0xFFFFFFFFu) {
        const float hi[3] = {pos[id][0] + 1.0f, pos[id][1] + 1.0f, pos[id][2] + 1.0f};
        float tn, tf;
        aabb(o, d, pos[id], hi, &tn, &tf);
        if (tf >= tn) {
            out->data = 0xFFFFFFFFu;
            for (int k = 0; k < 3; ++k) out->hit_pos[k] = pos[id][k];
        }
    }
}

void vto_sky_ref(const float rd[3], float out[4]) {
    float sn[3], rn[3];
    normalize3(kSunDir, sn);
    normalize3(rd, rn);
    const float s = clampf(dot3(sn, rn), 0.0f, 1.2f);
    const float dy = rd[1] * 0.2f;
    const float p8 = powf(s, 8.0f), p3 = powf(s, 3.0f);
    out[0] = ((0.6f - dy * 1.0f) + (0.15f * 0.5f)) + (0.4f * 1.0f) * p8 + 0.2f * p3;
    out[1] = ((0.71f - dy * 0.5f) + (0.15f * 0.5f)) + (0.4f * 0.6f) * p8 + 0.08f * p3;
    out[2] = ((0.75f - dy * 1.0f) + (0.15f * 0.5f)) + (0.4f * 0.1f) * p8 + 0.04f * p3;
    out[3] = 1.0f;
}

static uint32_t pack8(const float c[4]) {
    return unorm8(c[0]) | (unorm8(c[1]) << 8) | (unorm8(c[2]) << 16) | (unorm8(c[3]) << 24);
}

static void unpack8(uint32_t p, float c[4]) {
    for (int j = 0; j < 4; ++j) c[j] = (float)((p >> (8 * j)) & 255u) / 255.0f;
}

void vto_render_reference(const vto_refworld* w, const float cam_pos[4], const float view[16], float fov,
                          int32_t width, int32_t height, vt_ref_pixel* out) {
    for (int py = 0; py < height; ++py)
        for (int px = 0; px < width; ++px) {
            vt_ref_pixel* o = out + (size_t)py * width + px;
            memset(o, 0, sizeof(*o));
            /* primary.comp.glsl */
            float dir[3];
            vto_refhit h;
            vto_primary_r(w, cam_pos, view, fov, px, py, width, height, 192, dir, &h);
            if (h.data != 0) {
                o->albedo = h.data; /* unpackUnorm4x8 stored back into RGBA8 */
                const float n4[4] = {h.normal[0], h.normal[1], h.normal[2], 1.0f};
                o->normal = pack8(n4);
                for (int k = 0; k < 3; ++k) o->position[k] = ceilf(h.hit_pos[k]) / 8.0f;
                o->position[3] = 1.0f;
            } else {
                float sky4[4];
                vto_sky_ref(dir, sky4);
                o->albedo = pack8(sky4);
                o->normal = 0xFFFFFFFFu;
                for (int k = 0; k < 4; ++k) o->position[k] = -1.0f;
            }
            /* secondary.comp.glsl */
            if (o->position[0] < 0.0f || o->position[1] < 0.0f || o->position[2] < 0.0f) {
                o->illumination = 0;
            } else {
                float nq[4];
                unpack8(o->normal, nq);
                float ro[3];
                for (int k = 0; k < 3; ++k) ro[k] = o->position[k] + nq[k] * 0.001f;
                vto_refhit sh, en;
                vto_tracemap(w, ro, kSunDir, 48, &sh);
                const float hp8[3] = {sh.hit_pos[0] / 8.0f, sh.hit_pos[1] / 8.0f, sh.hit_pos[2] / 8.0f};
                vto_trace_entities(ro, kSunDir, dist3(ro, hp8), &en);
                const float a = (en.data != 0 || sh.data != 0) ? -0.3f : 0.3f;
                const float il[4] = {kSunDir[0], kSunDir[1], kSunDir[2], a};
                o->illumination = pack8(il);
            }
            /* blit.fragment.glsl */
            const float u = ((float)px + 0.5f) / (float)width, v = ((float)py + 0.5f) / (float)height;
            float col[4], nq[4], il[4];
            unpack8(o->albedo, col);
            unpack8(o->normal, nq);
            unpack8(o->illumination, il);
            float sky4[4];
            vto_sky_ref(il, sky4); /* SkyDome2(rayPos + normal * 0.001, illumination.xyz): ro is unused */
            for (int k = 0; k < 4; ++k) col[k] = col[k] + il[3] * sky4[k];
            const float cu = u - 0.5f, cv = v - 0.5f;
            if (sqrtf(cu * cu + cv * cv) <= 0.002f) {
                const float mixc[4] = {1.0f, 1.0f, 1.0f, 0.4f};
                for (int k = 0; k < 4; ++k) col[k] = col[k] * (1.0f - 0.5f) + mixc[k] * 0.5f;
            }
            const float g = powf((u * (1.0f - u)) * (v * (1.0f - v)) * 15.0f, 0.6f * 0.3f);
            for (int k = 0; k < 4; ++k) col[k] = g * col[k];
            o->color = pack8(col);
        }
}
