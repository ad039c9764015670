// shade.cuh -- ray generation and shading on the device (mode P).
//
//   primary ray     primary.comp.glsl:31-39 (direction normalised in 3-D)
//   sky             camera.glsl:11-19 (SkyDome2, sun as a parameter, integer
//                   powers as products)
//   shadow origin   secondary.comp.glsl:37 (hit point + normal * 0.001)
//   illumination    secondary.comp.glsl:45-48 stored in RGBA8 (gbuffer.zig:13)
//   composite       blit.fragment.glsl:15-35 (illum.a * sky, crosshair, vignette)
//   bounce          rng.glsl:16-29,41-55 (wang_hash, CosineSampleHemisphere),
//                   per-pixel seed x*1973 + y*9277 (primary.comp.glsl:25)
//
// Compiled with --fmad=false: every expression rounds as written.
#pragma once

#include "unorm8.cuh"
#include "vt_internal.h"

namespace vt {

// Camera and parameters of one frame, by value in kernel parameter space.
struct FrameParams {
    float pos[3];
    float view[16];
    float tan_half_fov;
    int width, height;
    int max_steps, shadow_max_steps, bounce_max_steps;
    unsigned rays, shade, flags, seed;
    float sun[3];
    float ambient, diffuse, bounce_weight;
    // per-frame constants, computed on the host by the same code as the device
    float sun_n[3];     // normalised sun direction
    float lit_sky[3];   // SkyDome2 of the RGBA8-stored sun direction (blit.fragment.glsl:31)
    float lit_a;        // illumination alpha 0.3 stored in RGBA8
    float sun_d[3];     // the shadow rays' direction as traced (a zero component made 0.001, map.glsl:85-90)
    float sun_inv[3];   // its correctly rounded reciprocal
    float cross_r2;     // the largest x with sqrt(x) <= 0.002 (crosshair radius test without a square root)
    int row0, row_end;  // rows [row0, row_end) of the image this launch renders
    void* bounce_jobs;       // non-null: bounce rays are queued here (BounceJob), not traced inline
    unsigned* bounce_count;  // the queue's length
    const float4* screen;    // the frame's screen table (ScreenTable), or null: computed per block
};

// The per-pixel screen coordinates, each a function of the column or of the
// row alone (so a block can compute them once per column and row).
struct PixelUV {
    float ru, rv;  // the primary ray's UV (primary.comp.glsl:31-36)
    float cu, cv;  // the pixel centre in [0, 1] (vignette, crosshair)
    float gu, gv;  // the vignette's column and row factors
};

__device__ __forceinline__ float ray_u(const FrameParams& f, int px) {
    const float u = (((float)px / (float)f.width) * 2.0f) - 1.0f;
    return u * f.tan_half_fov;
}

__device__ __forceinline__ float ray_v(const FrameParams& f, int py) {
    const float W = (float)f.width, H = (float)f.height;
    float v = (((float)py / H) * 2.0f) - 1.0f;
    v = v * (H / W);
    return v * f.tan_half_fov;
}

__device__ __forceinline__ float centre_u(const FrameParams& f, int px) { return ((float)px + 0.5f) / (float)f.width; }
__device__ __forceinline__ float centre_v(const FrameParams& f, int py) { return ((float)py + 0.5f) / (float)f.height; }

// The vignette pow(15 u (1 - u) v (1 - v), 0.18) (blit.fragment.glsl:15-21,34)
// as the product of a column factor pow(15 u (1 - u), 0.18) and a row factor
// pow(v (1 - v), 0.18), so that a block computes the powers once per column
// and row.  The product is within a few ulp of the joint power.
__device__ __forceinline__ float vignette_u(float u) { return powf(15.0f * (u * (1.0f - u)), 0.18f); }
__device__ __forceinline__ float vignette_v(float v) { return powf(v * (1.0f - v), 0.18f); }

__device__ __forceinline__ PixelUV pixel_uv(const FrameParams& f, int px, int py) {
    PixelUV uv;
    uv.ru = ray_u(f, px);
    uv.rv = ray_v(f, py);
    uv.cu = centre_u(f, px);
    uv.cv = centre_v(f, py);
    uv.gu = vignette_u(uv.cu);
    uv.gv = vignette_v(uv.cv);
    return uv;
}

// PixelUV of pixel (px, py) from the frame's screen table.
__device__ __forceinline__ PixelUV table_uv(const FrameParams& f, int px, int py) {
    const float4 c = __ldg(f.screen + px), r = __ldg(f.screen + f.width + py);
    PixelUV uv;
    uv.ru = c.x;
    uv.cu = c.y;
    uv.gu = c.z;
    uv.rv = r.x;
    uv.cv = r.y;
    uv.gv = r.z;
    return uv;
}

__device__ __forceinline__ void primary_ray_uv(const FrameParams& f, const PixelUV& uv, float o[3], float d[3]) {
    const float u = uv.ru, v = uv.rv;
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

__device__ __forceinline__ void primary_ray(const FrameParams& f, int px, int py, float o[3], float d[3]) {
    primary_ray_uv(f, pixel_uv(f, px, py), o, d);
}

// Entity occluders (the role of traceEntities, map.glsl:172-201, in the
// shadow pass, secondary.comp.glsl:42-46): true when the ray o + t d, t >= 0,
// meets the closed box {lo[3], hi[3]}.  Slab test with IEEE division; an axis
// the ray does not move along is inside its slab or misses.
__host__ __device__ __forceinline__ bool ray_box(const float o[3], const float d[3], const float* box) {
    float tmin = 0.0f, tmax = INFINITY;
#pragma unroll
    for (int j = 0; j < 3; ++j) {
        if (d[j] == 0.0f) {
            if (o[j] < box[j] || o[j] > box[3 + j]) return false;
            continue;
        }
        const float a = (box[j] - o[j]) / d[j], b = (box[3 + j] - o[j]) / d[j];
        const float lo = a < b ? a : b, hi = a < b ? b : a;
        tmin = lo > tmin ? lo : tmin;
        tmax = hi < tmax ? hi : tmax;
    }
    return tmin <= tmax;
}

__device__ __forceinline__ bool entity_occluded(const WorldView& w, const float o[3], const float d[3]) {
    for (int i = 0; i < w.n_entities; ++i)
        if (ray_box(o, d, w.entities + 6 * i)) return true;
    return false;
}

// Shared by host and device: plain IEEE operators (correctly rounded division
// and square root on both sides, no contraction).
__host__ __device__ __forceinline__ float clampf(float x, float a, float b) { return x < a ? a : (x > b ? b : x); }

__host__ __device__ __forceinline__ unsigned unorm8(float x) { return (unsigned)(int)rintf(clampf(x, 0.0f, 1.0f) * 255.0f); }

__host__ __device__ __forceinline__ float dot3(const float a[3], const float b[3]) { return (a[0] * b[0] + a[1] * b[1]) + a[2] * b[2]; }

__host__ __device__ __forceinline__ void normalize3(const float a[3], float o[3]) {
    const float len = sqrtf(dot3(a, a));
    o[0] = a[0] / len;
    o[1] = a[1] / len;
    o[2] = a[2] / len;
}

__host__ __device__ __forceinline__ void sky(const float sun[3], const float rd[3], float col[3]) {
    float sn[3], rn[3];
    normalize3(sun, sn);
    normalize3(rd, rn);
    const float s = clampf(dot3(sn, rn), 0.0f, 1.2f);
    const float s2 = s * s, s3 = s2 * s, s4 = s2 * s2, s8 = s4 * s4;
    const float dy = rd[1] * 0.2f;
    col[0] = ((0.6f - dy * 1.0f) + (0.15f * 0.5f)) + (0.4f * 1.0f) * s8 + 0.2f * s3;
    col[1] = ((0.71f - dy * 0.5f) + (0.15f * 0.5f)) + (0.4f * 0.6f) * s8 + 0.08f * s3;
    col[2] = ((0.75f - dy * 1.0f) + (0.15f * 0.5f)) + (0.4f * 0.1f) * s8 + 0.04f * s3;
}

// sky() with the sun direction already normalised (FrameParams::sun_n, made
// on the host by the same normalize3): the same value without the per-call
// normalisation of the sun.
__device__ __forceinline__ void sky_n(const float sn[3], const float rd[3], float col[3]) {
    float rn[3];
    normalize3(rd, rn);
    const float s = clampf(dot3(sn, rn), 0.0f, 1.2f);
    const float s2 = s * s, s3 = s2 * s, s4 = s2 * s2, s8 = s4 * s4;
    const float dy = rd[1] * 0.2f;
    col[0] = ((0.6f - dy * 1.0f) + (0.15f * 0.5f)) + (0.4f * 1.0f) * s8 + 0.2f * s3;
    col[1] = ((0.71f - dy * 0.5f) + (0.15f * 0.5f)) + (0.4f * 0.6f) * s8 + 0.08f * s3;
    col[2] = ((0.75f - dy * 1.0f) + (0.15f * 0.5f)) + (0.4f * 0.1f) * s8 + 0.04f * s3;
}

__device__ __forceinline__ bool crosshair(const FrameParams& f, float cu, float cv) {
    const float u = cu - 0.5f, v = cv - 0.5f;
    return u * u + v * v <= f.cross_r2;
}

__device__ __forceinline__ unsigned wang_hash(unsigned& seed) {
    unsigned s = (seed ^ 61u) ^ (seed >> 16);
    s *= 9u;
    s = s ^ (s >> 4);
    s *= 0x27d4eb2du;
    s = s ^ (s >> 15);
    seed = s;
    return s;
}

__device__ __forceinline__ float rand01(unsigned& seed) { return __uint2float_rn(wang_hash(seed)) * 0x1p-32f; }

// Deterministic sine/cosine: Cody-Waite reduction by pi/2 split into three
// floats (1.5703125 + 0x1.fb4p-12 + 0x1.4442d2p-24, each the leading bits of
// the remainder of the previous split) and Taylor polynomials of degree 9 (sin)
// and 10 (cos) on |r| <= pi/4, evaluated with correctly rounded fma.
__device__ __forceinline__ void det_sincos(float x, float& s, float& c) {
    const float k = rintf(x * 0x1.45f306p-1f);
    float r = __fmaf_rn(-k, 0x1.92p+0f, x);
    r = __fmaf_rn(-k, 0x1.fb4p-12f, r);
    r = __fmaf_rn(-k, 0x1.4442d2p-24f, r);
    const float r2 = r * r;
    float ps = __fmaf_rn(r2, 1.0f / 362880.0f, -1.0f / 5040.0f);
    ps = __fmaf_rn(r2, ps, 1.0f / 120.0f);
    ps = __fmaf_rn(r2, ps, -1.0f / 6.0f);
    ps = __fmaf_rn(r2 * r, ps, r);
    float pc = __fmaf_rn(r2, -1.0f / 3628800.0f, 1.0f / 40320.0f);
    pc = __fmaf_rn(r2, pc, -1.0f / 720.0f);
    pc = __fmaf_rn(r2, pc, 1.0f / 24.0f);
    pc = __fmaf_rn(r2, pc, -0.5f);
    pc = __fmaf_rn(r2, pc, 1.0f);
    const int q = ((int)k) & 3;
    if (q == 0) { s = ps; c = pc; }
    else if (q == 1) { s = pc; c = -ps; }
    else if (q == 2) { s = -ps; c = -pc; }
    else { s = -pc; c = ps; }
}

__device__ __forceinline__ void cross3(const float a[3], const float b[3], float o[3]) {
    o[0] = a[1] * b[2] - a[2] * b[1];
    o[1] = a[2] * b[0] - a[0] * b[2];
    o[2] = a[0] * b[1] - a[1] * b[0];
}

__device__ __forceinline__ void cosine_hemisphere(const float n[3], unsigned& seed, float out[3]) {
    const float u1 = rand01(seed), u2 = rand01(seed);
    const float r = __fsqrt_rn(u1);
    const float theta = 6.28f * u2;
    const float up[3] = {0.0f, 1.0f, 1.0f};
    float b0[3], B[3], T[3];
    cross3(n, up, b0);
    normalize3(b0, B);
    cross3(B, n, T);
    float st, ct;
    det_sincos(theta, st, ct);
    const float rs = r * st, rc = r * ct, h = __fsqrt_rn(1.0f - u1);
    float v[3];
#pragma unroll
    for (int j = 0; j < 3; ++j) v[j] = (rs * B[j] + h * n[j]) + rc * T[j];
    normalize3(v, out);
}

// Colour of a primary hit in REFERENCE / LAMBERT / NONE shading.
__device__ __forceinline__ void shade_hit(const FrameParams& f, unsigned alb, int axis, bool pos_axis, bool shadowed,
                                          bool bounce_open, const float bdir[3], float col[4]) {
    float albf[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) albf[j] = unorm8_to_float((alb >> (8 * j)) & 255u);
    if (f.shade == VT_SHADE_REFERENCE) {
        const float a = shadowed ? 0.0f : f.lit_a;
#pragma unroll
        for (int j = 0; j < 3; ++j) col[j] = albf[j] + a * f.lit_sky[j];
        col[3] = albf[3] + a * 1.0f;
        if (bounce_open) {
            float bc[3];
            sky_n(f.sun_n, bdir, bc);
#pragma unroll
            for (int j = 0; j < 3; ++j) col[j] = col[j] + f.bounce_weight * (albf[j] * bc[j]);
        }
    } else if (f.shade == VT_SHADE_LAMBERT) {
        float nrm[3] = {0.0f, 0.0f, 0.0f};
        nrm[0] = axis == 0 ? (pos_axis ? -1.0f : 1.0f) : 0.0f;
        nrm[1] = axis == 1 ? (pos_axis ? -1.0f : 1.0f) : 0.0f;
        nrm[2] = axis == 2 ? (pos_axis ? -1.0f : 1.0f) : 0.0f;
        float ndl = dot3(nrm, f.sun_n);
        if (ndl < 0.0f) ndl = 0.0f;
        const float vis = shadowed ? 0.0f : 1.0f;
        const float k = f.ambient + f.diffuse * ndl * vis;
#pragma unroll
        for (int j = 0; j < 3; ++j) col[j] = albf[j] * k;
        col[3] = 1.0f;
    } else {
#pragma unroll
        for (int j = 0; j < 4; ++j) col[j] = albf[j];
    }
}

__device__ __forceinline__ void shade_miss(const FrameParams& f, const float d[3], float col[4]) {
    col[0] = col[1] = col[2] = col[3] = 0.0f;
    if (f.shade == VT_SHADE_REFERENCE) {
        float sc[3];
        sky_n(f.sun_n, d, sc);
#pragma unroll
        for (int j = 0; j < 3; ++j) col[j] = unorm8_to_float(unorm8(sc[j]));
        col[3] = 1.0f;
    }
}

__device__ __forceinline__ unsigned composite_uv(const FrameParams& f, const PixelUV& uv, float col[4]) {
    if (f.shade == VT_SHADE_REFERENCE) {
        if ((f.flags & VT_FLAG_CROSSHAIR) && crosshair(f, uv.cu, uv.cv)) {
            col[0] = col[0] * 0.5f + 0.5f;
            col[1] = col[1] * 0.5f + 0.5f;
            col[2] = col[2] * 0.5f + 0.5f;
            col[3] = col[3] * 0.5f + 0.2f;
        }
        if (f.flags & VT_FLAG_VIGNETTE) {
            const float g = uv.gu * uv.gv;
#pragma unroll
            for (int j = 0; j < 4; ++j) col[j] = g * col[j];
        }
    }
    return unorm8(col[0]) | (unorm8(col[1]) << 8) | (unorm8(col[2]) << 16) | (unorm8(col[3]) << 24);
}

__device__ __forceinline__ unsigned composite(const FrameParams& f, int px, int py, float col[4]) {
    return composite_uv(f, pixel_uv(f, px, py), col);
}

// FrameParams of a camera and parameter set (render.cu).
FrameParams make_frame(const vt_camera* cam, const vt_params* p);

// The per-frame constants of FrameParams (host side).
inline void frame_constants(FrameParams& f) {
    normalize3(f.sun, f.sun_n);
    float sq[3];
    for (int j = 0; j < 3; ++j) sq[j] = (float)unorm8(f.sun[j]) / 255.0f;
    sky(f.sun, sq, f.lit_sky);
    f.lit_a = (float)unorm8(0.3f) / 255.0f;
    for (int j = 0; j < 3; ++j) {
        f.sun_d[j] = f.sun[j] == 0.0f ? 0.001f : f.sun[j];
        f.sun_inv[j] = 1.0f / f.sun_d[j];
    }
    // square roots round monotonically: sqrt(x) <= r iff x <= the largest such x
    const float r = 0.002f;
    float x = r * r;
    while (sqrtf(x) > r) x = nextafterf(x, 0.0f);
    while (sqrtf(nextafterf(x, INFINITY)) <= r) x = nextafterf(x, INFINITY);
    f.cross_r2 = x;
}

}  // namespace vt
