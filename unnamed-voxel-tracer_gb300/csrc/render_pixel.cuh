// render_pixel.cuh -- one pixel of the render-frame path (primary, shadow and
// bounce rays, shading, the 16-byte record), shared by the single-frame and
// the batched kernels.
#pragma once

#include "bounce.cuh"
#include "shade.cuh"
#include "trace_p.cuh"

namespace vt {

struct PixelCounters {
    unsigned v[kNumCounters];
};

// The instrumented and bounds-checked variants run the three-level model
// traversal (it defines the algorithmic byte counts); the production variant
// runs trace_fast.  Both give identical results.
// NEAR: the caller knows the origin passes near_origin (secondary rays start
// on a hit inside the grid); otherwise the primary ray checks it once.
// SHARE: brick words shared between the lanes of a warp (Walker::brick_word).
template <bool STATS, bool CHECKED, bool MAT, bool NEAR, bool SHARE, class Coarse>
__device__ __forceinline__ bool trace_any(const WorldView& w, const Coarse& coarse, const unsigned char* cd,
                                          const PRay& r, int max_steps, TraceHit& h, TraceCounters& cnt,
                                          unsigned* status) {
    if (STATS || CHECKED) return trace_p<STATS, CHECKED, MAT>(w, coarse, r, max_steps, h, cnt, status);
    if (NEAR || near_origin(r.o)) return trace_fast<MAT, true, true, SHARE>(w, cd, r, max_steps, h);
    return trace_fast<MAT, true, false, SHARE>(w, cd, r, max_steps, h);
}

// uv: the pixel's screen coordinates (pixel_uv(f, px, py); the frame kernel
// reads them from the frame's screen table or its per-block tables).
// BIN: a deferred bounce ray is staged in the block's shared memory for the
// block's direction-sorted append (stage_flush) instead of appended at once.
template <bool STATS, bool CHECKED, class Coarse, bool SHARE = false, bool BIN = false>
__device__ __forceinline__ uint4 render_pixel(const WorldView& w, const Coarse& coarse, const unsigned char* cd,
                                              const FrameParams& f, int px, int py, const PixelUV& uv,
                                              unsigned* status, PixelCounters& pc) {
    float o[3], d[3];
    primary_ray_uv(f, uv, o, d);
    PRay r;
    pray_init(r, o, d);
    TraceHit h;
    TraceCounters cnt;
    const bool hit = trace_any<STATS, CHECKED, true, false, SHARE>(w, coarse, cd, r, f.max_steps, h, cnt, status);
    if (STATS) {
        pc.v[0] += 1;
        pc.v[9] += 16;
    }
    unsigned flags = 0, rgba, voxel = 0xFFFFFFFFu, face = 0xFFu, mat = 0;
    float t = -1.0f;
    float col[4];
    if (hit) {
        flags = VT_HIT_PRIMARY;
        voxel = (unsigned)h.c[0] + (unsigned)w.dims[0] * ((unsigned)h.c[1] + (unsigned)w.dims[1] * (unsigned)h.c[2]);
        t = h.t;
        const int e = h.axis;
        const bool pe = e == 0 ? r.pos[0] : (e == 1 ? r.pos[1] : r.pos[2]);
        face = 2u * (unsigned)e + (pe ? 0u : 1u);
        mat = h.mat;
        const unsigned alb = __ldg(w.palette + mat);
        if (STATS) {
            pc.v[1] += 1;
            pc.v[8] += 1;
        }
        float nrm[3], so[3];
#pragma unroll
        for (int j = 0; j < 3; ++j) {
            nrm[j] = (j == e) ? (pe ? -1.0f : 1.0f) : 0.0f;
            so[j] = __fmaf_rn(r.d[j], t, o[j]);
            if (j == e) so[j] = so[j] + nrm[j] * 0.001f;
        }
        bool shadowed = false;
        if (f.rays & VT_RAYS_SHADOW) {
            PRay rs;
            pray_init_dir(rs, so, f.sun_d, f.sun_inv);
            TraceHit hs;
            shadowed = trace_any<STATS, CHECKED, false, true, SHARE>(w, coarse, cd, rs, f.shadow_max_steps, hs, cnt, status);
            if (shadowed) flags |= VT_HIT_SHADOWED;
            if (STATS) {
                pc.v[2] += 1;
                pc.v[3] += shadowed ? 1u : 0u;
            }
            if (!shadowed && w.n_entities > 0 && entity_occluded(w, so, f.sun)) {
                shadowed = true;
                flags |= VT_HIT_ENTITY;
            }
        }
        bool bounce_open = false;
        bool deferred = false;
        float bdir[3] = {0.0f, 0.0f, 0.0f};
        if (f.rays & VT_RAYS_BOUNCE) {
            unsigned seed = ((unsigned)px * 1973u + (unsigned)py * 9277u) ^ f.seed;
            cosine_hemisphere(nrm, seed, bdir);
            deferred = !STATS && !CHECKED && f.bounce_jobs != nullptr;
        }
        if (deferred) {
            // traced and shaded by the bounce kernels (bounce.cu)
            if (BIN) stage_bounce(so, bdir, (unsigned)py * (unsigned)f.width + (unsigned)px);
            else append_bounce(f, so, bdir, (unsigned)py * (unsigned)f.width + (unsigned)px);
        } else if (f.rays & VT_RAYS_BOUNCE) {
            PRay rb;
            pray_init(rb, so, bdir);
            TraceHit hb;
            const bool bh = trace_any<STATS, CHECKED, false, true, SHARE>(w, coarse, cd, rb, f.bounce_max_steps, hb, cnt, status);
            if (bh) flags |= VT_HIT_BOUNCE;
            bounce_open = !bh;
            if (STATS) {
                pc.v[4] += 1;
                pc.v[5] += bh ? 1u : 0u;
            }
        }
        if (deferred) {
            rgba = 0u;
        } else {
            shade_hit(f, alb, e, pe, shadowed, bounce_open, bdir, col);
            rgba = f.shade == VT_SHADE_NONE ? alb : composite_uv(f, uv, col);
        }
    } else {
        shade_miss(f, d, col);
        rgba = f.shade == VT_SHADE_NONE ? 0u : composite_uv(f, uv, col);
    }
    if (STATS) {
        pc.v[6] += cnt.mask;
        pc.v[7] += cnt.coarse;
        pc.v[10] += cnt.steps;
        pc.v[11] += cnt.iters;
    }
    return make_uint4(voxel, __float_as_uint(t), rgba, face | (mat << 8) | (flags << 16));
}

}  // namespace vt
