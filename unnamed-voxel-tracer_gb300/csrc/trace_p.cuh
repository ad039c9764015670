// trace_p.cuh -- mode-P traversal on the device.
//
// A ray crosses the integer plane k of axis i at
//     ptime_i(k) = fma(k, inv_i, -(o_i * inv_i)),     inv_i = 1 / d_i,
// a pure function of k.  Crossing events are ordered by (t ascending, axis
// descending), which is the order the reference's selection chain
//     t.x < t.y ? (t.x < t.z ? 0 : 2) : (t.y < t.z ? 1 : 2)      (map.glsl:158)
// produces one unit step at a time.  Because every crossing time is a pure
// function of its plane, the traversal can leave an empty 32^3 chunk or an
// empty 4^3 brick in one jump: the exit event is the smallest of the region's
// three boundary crossings, and on each other axis the ray has crossed exactly
// the planes whose event precedes the exit.  The jump therefore lands on the
// same cell, with the same entry time, entry axis and crossing count, as unit
// stepping through the region would (the reference skips whole empty voxels
// with stepSize 3 in the same spirit, map.glsl:138-145).
//
// The max-step cutoff counts unit crossings (map.glsl:106): the cell reached
// after n crossings is tested iff n < max_steps.
//
// All arithmetic is IEEE single precision with explicit rounding: this file is
// compiled with --fmad=false and every fused multiply-add is written out.
#pragma once

#include "vt_internal.h"

namespace vt {

struct PRay {
    float o[3], d[3], inv[3], oinv[3];
    bool pos[3];
};

struct TraceCounters {
    unsigned mask = 0, coarse = 0, steps = 0, iters = 0;
};

__device__ __forceinline__ void pray_init(PRay& r, const float o[3], const float d[3]) {
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        float di = d[i] == 0.0f ? 0.001f : d[i];  // map.glsl:85-90
        r.o[i] = o[i];
        r.d[i] = di;
        r.inv[i] = __frcp_rn(di);
        r.oinv[i] = -__fmul_rn(o[i], r.inv[i]);
        r.pos[i] = di > 0.0f;
    }
}

// pray_init with a direction whose zero components are already replaced and
// whose reciprocal is given (the shadow rays of a frame share both).
__device__ __forceinline__ void pray_init_dir(PRay& r, const float o[3], const float d[3], const float inv[3]) {
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        r.o[i] = o[i];
        r.d[i] = d[i];
        r.inv[i] = inv[i];
        r.oinv[i] = -__fmul_rn(o[i], inv[i]);
        r.pos[i] = d[i] > 0.0f;
    }
}

// Whether a ray origin is near enough for the one-correction plane search
// (advance_axis<true>).
__host__ __device__ __forceinline__ bool near_origin(const float o[3]) {
    return fabsf(o[0]) < 0x1p20f && fabsf(o[1]) < 0x1p20f && fabsf(o[2]) < 0x1p20f;
}

__device__ __forceinline__ float ptime(const PRay& r, int i, int k) {
    return __fmaf_rn(__int2float_rn(k), r.inv[i], r.oinv[i]);
}

// key(ta, a) < key(tb, b)
__device__ __forceinline__ bool key_lt(float ta, int a, float tb, int b) {
    return ta < tb || (ta == tb && a > b);
}

__device__ __forceinline__ bool crossed(const PRay& r, int i, int k, float T, int e) {
    return key_lt(ptime(r, i, k), i, T, e);
}

// Cell of axis i at the event (T, e), i != e.  Positive direction: the largest
// k in [lo, K-1] whose plane k is crossed (lo if none); negative direction: the
// smallest k in [K, lo] whose plane k+1 is crossed (lo if none).  A rounded
// position p = o + d T gives the first guess g = floor(p); the exact plane
// times decide.
//
// When |o_i| < 2^20 and the cells lie in the grid (< 2^13), the guess is off
// by at most one plane: the rounding of p and of the plane times ptime(k) =
// fma(k, 1/d, -o/d) stays below 2^-24 * 2^21 = 1/8 of a cell in position, so
// plane g - 1 is crossed strictly before T and plane g + 2 strictly after, and
// one exact test up or down settles it (NEAR).  Otherwise (far origins) the
// walk corrects the guess plane by plane.
template <bool NEAR>
__device__ __forceinline__ int advance_axis(const PRay& r, int i, int lo, int K, float T, int e) {
    float p = __fmaf_rn(r.d[i], T, r.o[i]);
    int k = __float2int_rd(p);
    if (NEAR) {
        if (r.pos[i]) {
            const int hi = K - 1;
            k = min(max(k, lo), hi);
            if (k < hi && crossed(r, i, k + 1, T, e)) ++k;
            else if (k > lo && !crossed(r, i, k, T, e)) --k;
        } else {
            k = min(max(k, K), lo);
            if (k > K && crossed(r, i, k, T, e)) --k;
            else if (k < lo && !crossed(r, i, k + 1, T, e)) ++k;
        }
        return k;
    }
    if (r.pos[i]) {
        int hi = K - 1;
        k = min(max(k, lo), hi);
        while (k < hi && crossed(r, i, k + 1, T, e)) ++k;
        while (k > lo && !crossed(r, i, k, T, e)) --k;
    } else {
        k = min(max(k, K), lo);
        while (k > K && crossed(r, i, k, T, e)) --k;
        while (k < lo && !crossed(r, i, k + 1, T, e)) ++k;
    }
    return k;
}

// Start cell of a ray against the grid box [0, D).  Returns false on a miss.
__device__ __forceinline__ bool pray_start(const PRay& r, const int D[3], int c[3], float& t0, int& axis0) {
    // An origin at least one cell inside the grid on every axis (secondary
    // rays, cameras inside the world) starts in its own cell at t = 0 when
    // every reciprocal lies in [2^-100, 2^100] in magnitude: then o * inv
    // neither overflows nor underflows, its rounding error (below 2^-11 |inv|
    // for o < 2^13) is smaller than the one-cell margin times |inv|, so the
    // entry planes are crossed at negative times and the exit planes at
    // positive ones, and the box test below would take its else branch with
    // the same result.  Anything else (NaN or infinite reciprocals included)
    // takes the box test.
    if (r.o[0] >= 1.0f && r.o[1] >= 1.0f && r.o[2] >= 1.0f && r.o[0] <= (float)(D[0] - 1) &&
        r.o[1] <= (float)(D[1] - 1) && r.o[2] <= (float)(D[2] - 1) && fabsf(r.inv[0]) <= 0x1p100f &&
        fabsf(r.inv[1]) <= 0x1p100f && fabsf(r.inv[2]) <= 0x1p100f && fabsf(r.inv[0]) >= 0x1p-100f &&
        fabsf(r.inv[1]) >= 0x1p-100f && fabsf(r.inv[2]) >= 0x1p-100f) {
#pragma unroll
        for (int i = 0; i < 3; ++i) c[i] = __float2int_rd(r.o[i]);
        t0 = 0.0f;
        axis0 = 0;
        return true;
    }
    float tin[3], tout[3];
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        tin[i] = ptime(r, i, r.pos[i] ? 0 : D[i]);
        tout[i] = ptime(r, i, r.pos[i] ? D[i] : 0);
    }
    float T0 = tin[0];
    int e = 0;
    if (key_lt(T0, e, tin[1], 1)) { T0 = tin[1]; e = 1; }
    if (key_lt(T0, e, tin[2], 2)) { T0 = tin[2]; e = 2; }
    float T1 = tout[0];
    int x = 0;
    if (key_lt(tout[1], 1, T1, x)) { T1 = tout[1]; x = 1; }
    if (key_lt(tout[2], 2, T1, x)) { T1 = tout[2]; x = 2; }
    if (!key_lt(T0, e, T1, x)) return false;  // box missed
    if (!(T1 > 0.0f)) return false;           // box behind the origin
    if (T0 >= 0.0f) {
#pragma unroll
        for (int i = 0; i < 3; ++i) {
            if (i == e) c[i] = r.pos[i] ? 0 : D[i] - 1;
            else c[i] = r.pos[i] ? advance_axis<false>(r, i, 0, D[i], T0, e) : advance_axis<false>(r, i, D[i] - 1, 0, T0, e);
        }
        t0 = T0;
        axis0 = e;
    } else {
#pragma unroll
        for (int i = 0; i < 3; ++i) c[i] = min(max(__float2int_rd(r.o[i]), 0), D[i] - 1);
        t0 = 0.0f;
        axis0 = 0;  // the reference starts with minIdx = 0 (map.glsl:98)
    }
    return true;
}

// Where the coarse (per-chunk) bits are read from.
struct CoarseShared {
    const unsigned long long* s;
    __device__ __forceinline__ unsigned long long operator()(unsigned i) const { return s[i]; }
};
struct CoarseGlobal {
    const unsigned long long* g;
    __device__ __forceinline__ unsigned long long operator()(unsigned i) const { return __ldg(g + i); }
};

struct TraceHit {
    float t;
    int axis;
    int c[3];
    unsigned mat;
};

// Traverses one ray.  Returns true on a hit (filled into h; the material byte
// is read only when MAT).
//
// Loop state: the cell c, the time tm[i] of the next plane on each axis (the
// classic Amanatides-Woo tMax, always ptime of that plane), and which level of
// the hierarchy is valid for the current cell: the chunk's coarse bit and the
// brick's occupancy word are looked up again only after a crossing leaves the
// chunk or the brick.  Inside an occupied brick a unit step is one argmin and
// one axis update; an empty brick or chunk is left in one jump.
template <bool STATS, bool CHECKED, bool MAT, class Coarse>
__device__ __forceinline__ bool trace_p(const WorldView& w, const Coarse& coarse, const PRay& r, int max_steps,
                                        TraceHit& h, TraceCounters& cnt, unsigned* status) {
    int c[3];
    float t;
    int axis;
    if (!pray_start(r, w.dims, c, t, axis)) return false;
    if (max_steps <= 0) return false;
    float tm[3];
#pragma unroll
    for (int i = 0; i < 3; ++i) tm[i] = ptime(r, i, r.pos[i] ? c[i] + 1 : c[i]);
    int n = 0;
    unsigned long long word = 0ull;
    unsigned ci = 0, wi = 0;
    unsigned last_cw = 0xFFFFFFFFu;
    // 0: chunk of c not looked up; 1: chunk occupied, brick word not loaded;
    // 2: brick word of c in `word`; 3: chunk of c is empty
    int state = 0;
    for (;;) {
        if (STATS) cnt.iters++;
        if (state == 0) {
            ci = (unsigned)(c[0] >> 5) + (unsigned)w.cdim[0] * ((unsigned)(c[1] >> 5) + (unsigned)w.cdim[1] * (unsigned)(c[2] >> 5));
            const unsigned cw = ci >> 6;
            if (CHECKED && cw >= w.ncoarse) {
                atomicOr(status, kStatusOob);
                return false;
            }
            if (STATS && cw != last_cw) {
                last_cw = cw;
                cnt.coarse++;
            }
            state = ((coarse(cw) >> (ci & 63u)) & 1ull) ? 1 : 3;
        }
        if (state == 1) {
            wi = ci * 512u + ((unsigned)((c[0] >> 2) & 7) | ((unsigned)((c[1] >> 2) & 7) << 3) |
                              ((unsigned)((c[2] >> 2) & 7) << 6));
            if (CHECKED && wi >= w.nwords) {
                atomicOr(status, kStatusOob);
                return false;
            }
            word = __ldg(w.mask + wi);
            if (STATS) cnt.mask++;
            state = 2;
        }
        int sh = 5;
        if (state == 2) {
            sh = 2;
            if (word != 0ull) {
                const unsigned vb = (unsigned)(c[0] & 3) | ((unsigned)(c[1] & 3) << 2) | ((unsigned)(c[2] & 3) << 4);
                const unsigned half = (vb & 32u) ? (unsigned)(word >> 32) : (unsigned)word;
                if ((half >> (vb & 31u)) & 1u) {
                    h.mat = MAT ? (unsigned)__ldg(w.mats + (size_t)wi * 64u + vb) : 0u;
                    h.t = t;
                    h.axis = axis;
                    h.c[0] = c[0];
                    h.c[1] = c[1];
                    h.c[2] = c[2];
                    if (STATS) cnt.steps += (unsigned)n;
                    return true;
                }
                sh = 0;
            }
        }
        if (sh == 0) {
            // one unit crossing inside an occupied brick
            const int e = tm[0] < tm[1] ? (tm[0] < tm[2] ? 0 : 2) : (tm[1] < tm[2] ? 1 : 2);
            bool out = false, brick = false, chunk = false;
#pragma unroll
            for (int i = 0; i < 3; ++i) {
                if (i == e) {
                    t = tm[i];
                    c[i] += r.pos[i] ? 1 : -1;
                    tm[i] = ptime(r, i, r.pos[i] ? c[i] + 1 : c[i]);
                    const int lo = c[i] & 31;
                    brick = (lo & 3) == (r.pos[i] ? 0 : 3);
                    chunk = lo == (r.pos[i] ? 0 : 31);
                    out = (unsigned)c[i] >= (unsigned)w.dims[i];
                }
            }
            axis = e;
            ++n;
            if (n >= max_steps || out) break;
            state = chunk ? 0 : (brick ? 1 : 2);
        } else {
            // leave the empty aligned 2^sh region that contains c in one jump
            int K[3];
            float tK[3];
#pragma unroll
            for (int i = 0; i < 3; ++i) {
                const int base = c[i] & ~((1 << sh) - 1);
                K[i] = r.pos[i] ? base + (1 << sh) : base;
                tK[i] = ptime(r, i, K[i]);
            }
            const int e = tK[0] < tK[1] ? (tK[0] < tK[2] ? 0 : 2) : (tK[1] < tK[2] ? 1 : 2);
            const float T = e == 0 ? tK[0] : (e == 1 ? tK[1] : tK[2]);
            int crossings = 0;
            bool chunk = sh == 5;
#pragma unroll
            for (int i = 0; i < 3; ++i) {
                if (i == e) {
                    const int cn = r.pos[i] ? K[i] : K[i] - 1;
                    crossings += abs(cn - c[i]);
                    chunk = chunk || ((cn >> 5) != (c[i] >> 5));
                    c[i] = cn;
                    tm[i] = ptime(r, i, r.pos[i] ? cn + 1 : cn);
                } else if (key_lt(tm[i], i, T, e)) {
                    const int cn = advance_axis<false>(r, i, c[i], K[i], T, e);
                    crossings += abs(cn - c[i]);
                    c[i] = cn;
                    tm[i] = ptime(r, i, r.pos[i] ? cn + 1 : cn);
                }
            }
            n += crossings;
            t = T;
            axis = e;
            if (n >= max_steps) break;
            if ((unsigned)c[0] >= (unsigned)w.dims[0] || (unsigned)c[1] >= (unsigned)w.dims[1] ||
                (unsigned)c[2] >= (unsigned)w.dims[2])
                break;
            state = chunk ? 0 : 1;
        }
    }
    if (STATS) cnt.steps += (unsigned)min(n, max_steps);
    return false;
}

// The production traversal.  Same crossings, results and entry times as
// trace_p (the jump argument holds for any empty axis-aligned box that contains
// the current cell), with larger jumps and a cheaper unit step:
//   - an empty chunk is left through the box of chunks ahead within Chebyshev
//     radius cdist - 1 (all empty), an empty brick through the box made of
//     the brick and bdist - 1 voxel layers beyond its far faces (fewer
//     vertically for rays moving down), both from the ray's octant field (the
//     ray only moves forwards on every axis, so the exit of a box that extends
//     forwards from the current unit is the exit of the symmetric box);
//   - inside an occupied brick only the next-plane index nk and time tm of the
//     crossing axis change; the crossed plane's index tells whether the step
//     left the brick (k % 4 == 0), the chunk (k % 32 == 0) or the grid, and the
//     voxel's bit index moves by +-1, 4 or 16.
// The walk is resumable one iteration at a time (step), so that a persistent
// kernel can interleave rays of different pixels and kinds in one warp.
// cdist is the per-chunk distance array (8 octant fields, read through L1).
// Host builds of this header (the traversal tests) may count the kinds of
// steps (0 chunk jump, 1 brick jump, 2 voxel test + unit step).
#ifndef VT_STEP_HOOK
#define VT_STEP_HOOK(kind)
#endif

struct Walker {
    PRay r;
    int max_steps;
    int c[3];       // current cell (valid in states 0 and 1)
    int nk[3];      // next plane index per axis
    float tm[3];    // its crossing time
    int n;          // unit crossings made
    float t;        // entry time of the current cell
    int axis;       // axis of the crossing that entered it
    unsigned long long word;
    unsigned wi, vb;
    unsigned oct;   // direction octant: bit i set iff the ray moves towards +i
    int state;      // 0: chunk of c unknown; 1: brick of c unknown; 2: in the occupied brick `word`

    enum { kMore = 0, kHit = 1, kMiss = 2 };

    // Sets up the walk; false if the ray misses the grid or may take no step.
    __device__ __forceinline__ bool start(const WorldView& w, const float o[3], const float d[3], int steps) {
        pray_init(r, o, d);
        return start_ray(w, steps);
    }

    // The same for a ray already set up in r (its reciprocals computed once,
    // by the caller: pray_init, or pray_init_dir with a frame's shared ones).
    __device__ __forceinline__ bool start_ray(const WorldView& w, const PRay& ray, int steps) {
        r = ray;
        return start_ray(w, steps);
    }

    __device__ __forceinline__ bool start_ray(const WorldView& w, int steps) {
        max_steps = steps;
        if (!pray_start(r, w.dims, c, t, axis)) return false;
        if (steps <= 0) return false;
#pragma unroll
        for (int i = 0; i < 3; ++i) {
            nk[i] = r.pos[i] ? c[i] + 1 : c[i];
            tm[i] = ptime(r, i, nk[i]);
        }
        n = 0;
        word = 0ull;
        wi = vb = 0;
        oct = (r.pos[0] ? 1u : 0u) | (r.pos[1] ? 2u : 0u) | (r.pos[2] ? 4u : 0u);
        state = 0;
        return true;
    }

    // The plane through which the ray leaves, on axis i, the empty box around
    // cell ci: sh 5, the chunk of ci and the chunks within rad - 1 ahead; sh
    // 2, the brick of ci and s - 1 voxel layers beyond its far face, rad =
    // s | shape << 6 ((s - 1) >> shape vertically; s >= 1 in an empty brick);
    // sh 0, the cell itself (rad 1).
    __device__ __forceinline__ int exit_plane(int i, int ci, int sh, int rad) const {
        const int u = ci >> sh;
        int beyond = (rad - 1) << sh;   // cells beyond the unit's far face
        if (sh == 2) {
            const int layers = (rad & 63) - 1;
            beyond = i == 1 ? layers >> (rad >> 6) : layers;
        }
        return r.pos[i] ? ((u + 1) << sh) + beyond : (u << sh) - beyond;
    }

    // The brick word wi.  SHARE: the lanes of the warp that look up a word
    // at this point group by its index (__match_any_sync); one lane of each
    // group loads it and passes it on (__shfl_sync).
    template <bool SHARE>
    __device__ __forceinline__ unsigned long long brick_word(const WorldView& w, unsigned i) const {
#ifdef __CUDA_ARCH__
        if (SHARE) {
            const unsigned act = __activemask();
            const unsigned peers = __match_any_sync(act, i);
            const int leader = __ffs(peers) - 1;
            unsigned long long v = 0ull;
            if ((int)(threadIdx.x & 31u) == leader) v = __ldg(w.mask + i);
            return __shfl_sync(peers, v, leader);
        }
#endif
        return __ldg(w.mask + i);
    }

    // One iteration: a lookup plus a jump, or a voxel test plus a unit step
    // (RUN: unit steps until the walk leaves the occupied brick).  In a warp
    // whose lanes are in different phases every iteration pays for both the
    // jump and the unit-step code; running a lane's unit steps in one inner
    // loop pays the jump code once per brick visit instead (-4.5% on a 1080p
    // terrain frame of primary and shadow rays).
    // NEAR: the ray's origin passes near_origin (one-correction plane search).
    // SHARE: brick words shared between the lanes of a warp (brick_word).
    template <bool MAT, bool RUN = true, bool NEAR = false, bool SHARE = false>
    __device__ __forceinline__ int step(const WorldView& w, const unsigned char* cdist, TraceHit& h) {
        bool jump = false;
        int sh = 0, rad = 0;
        if (state != 2) {
            // the current cell and its chunk (nk is exact in states 0 and 1)
#pragma unroll
            for (int i = 0; i < 3; ++i) c[i] = r.pos[i] ? nk[i] - 1 : nk[i];
            const unsigned ci = (unsigned)(c[0] >> 5) + (unsigned)w.cdim[0] * ((unsigned)(c[1] >> 5) + (unsigned)w.cdim[1] * (unsigned)(c[2] >> 5));
            if (state == 0) {
                const int dc = cdist[oct * w.cstride + ci];
                if (dc) {
                    jump = true;
                    sh = 5;
                    rad = dc;
                } else {
                    state = 1;
                }
            }
            if (state == 1) {
                wi = ci * 512u + ((unsigned)((c[0] >> 2) & 7) | ((unsigned)((c[1] >> 2) & 7) << 3) | ((unsigned)((c[2] >> 2) & 7) << 6));
                word = brick_word<SHARE>(w, wi);
                if (word == 0ull) {
                    jump = true;
                    sh = 2;
                    rad = __ldg(w.bdist + (size_t)oct * w.nwords + wi);
                } else {
                    vb = (unsigned)(c[0] & 3) | ((unsigned)(c[1] & 3) << 2) | ((unsigned)(c[2] & 3) << 4);
                    state = 2;
                }
            }
        }
        if (!jump) {
          for (;;) {
            // inside an occupied brick: test the voxel, else one unit crossing
            VT_STEP_HOOK(2);
            const unsigned half = (vb & 32u) ? (unsigned)(word >> 32) : (unsigned)word;
            if ((half >> (vb & 31u)) & 1u) {
#pragma unroll
                for (int i = 0; i < 3; ++i) h.c[i] = r.pos[i] ? nk[i] - 1 : nk[i];
                h.mat = MAT ? (unsigned)__ldg(w.mats + (size_t)wi * 64u + vb) : 0u;
                h.t = t;
                h.axis = axis;
                return kHit;
            }
            const int e = tm[0] < tm[1] ? (tm[0] < tm[2] ? 0 : 2) : (tm[1] < tm[2] ? 1 : 2);
            float T = tm[0];
            int k = nk[0], xp = r.pos[0] ? w.dims[0] : 0;
            unsigned dv = r.pos[0] ? 1u : 0xFFFFFFFFu;
#pragma unroll
            for (int i = 1; i < 3; ++i) {
                if (i == e) {
                    T = tm[i];
                    k = nk[i];
                    xp = r.pos[i] ? w.dims[i] : 0;
                    dv = r.pos[i] ? (1u << (2 * i)) : (0u - (1u << (2 * i)));
                }
            }
#pragma unroll
            for (int i = 0; i < 3; ++i) {
                if (i == e) {
                    nk[i] += r.pos[i] ? 1 : -1;
                    tm[i] = ptime(r, i, nk[i]);
                }
            }
            t = T;
            axis = e;
            ++n;
            if (n >= max_steps || k == xp) return kMiss;
            if ((k & 3) == 0) {
                state = (k & 31) == 0 ? 0 : 1;
                return kMore;
            }
            vb += dv;
            if (!RUN) return kMore;
          }
        }
        // leave the empty box: the chunk and the chunks within rad - 1 ahead,
        // or the brick and rad - 1 voxel layers beyond it
        VT_STEP_HOOK(sh == 5 ? 0 : 1);
        int K[3];
        float tK[3];
#pragma unroll
        for (int i = 0; i < 3; ++i) {
            K[i] = exit_plane(i, c[i], sh, rad);
            tK[i] = ptime(r, i, K[i]);
        }
        const int e = tK[0] < tK[1] ? (tK[0] < tK[2] ? 0 : 2) : (tK[1] < tK[2] ? 1 : 2);
        const float T = e == 0 ? tK[0] : (e == 1 ? tK[1] : tK[2]);
        int crossings = 0;
#pragma unroll
        for (int i = 0; i < 3; ++i) {
            int cn = c[i];
            if (i == e) cn = r.pos[i] ? K[i] : K[i] - 1;
            else if (key_lt(tm[i], i, T, e)) cn = advance_axis<NEAR>(r, i, c[i], K[i], T, e);
            crossings += abs(cn - c[i]);
            c[i] = cn;
            nk[i] = r.pos[i] ? cn + 1 : cn;
            tm[i] = ptime(r, i, nk[i]);
        }
        n += crossings;
        t = T;
        axis = e;
        if (n >= max_steps) return kMiss;
        if ((unsigned)c[0] >= (unsigned)w.dims[0] || (unsigned)c[1] >= (unsigned)w.dims[1] ||
            (unsigned)c[2] >= (unsigned)w.dims[2])
            return kMiss;
        state = 0;
        return kMore;
    }

    // The same walk with one code path for jumps and unit steps: every turn
    // looks the cell up (unless it is in the occupied brick of the last turn),
    // then leaves a box -- an empty chunk box, an empty brick box, or the one
    // voxel that was tested -- by the same exit computation.  A warp whose
    // lanes walk unrelated rays (the bounce pass) then runs one instruction
    // stream for all of them instead of a jump path and a unit-run path; a
    // unit step costs more than in step().  The lookup reads the chunk
    // distance, the brick word and the brick distance without waiting on one
    // another (the brick index is in range for any cell of the grid).
    // Results are those of step() (every box exit is exact, see above); no
    // material is read (the bounce pass needs none).
    template <bool NEAR = false>
    __device__ __forceinline__ int step_flat(const WorldView& w, const unsigned char* cdist, TraceHit& h) {
        int sh = 0, rad = 1;
        if (state != 2) {
#pragma unroll
            for (int i = 0; i < 3; ++i) c[i] = r.pos[i] ? nk[i] - 1 : nk[i];
            const unsigned ci = (unsigned)(c[0] >> 5) + (unsigned)w.cdim[0] * ((unsigned)(c[1] >> 5) + (unsigned)w.cdim[1] * (unsigned)(c[2] >> 5));
            wi = ci * 512u + ((unsigned)((c[0] >> 2) & 7) | ((unsigned)((c[1] >> 2) & 7) << 3) | ((unsigned)((c[2] >> 2) & 7) << 6));
            const int dc = cdist[oct * w.cstride + ci];
            word = __ldg(w.mask + wi);
            const int bd = __ldg(w.bdist + (size_t)oct * w.nwords + wi);
            if (dc) {
                VT_STEP_HOOK(0);
                sh = 5;
                rad = dc;
            } else if (word == 0ull) {
                VT_STEP_HOOK(1);
                sh = 2;
                rad = bd;
            } else {
                vb = (unsigned)(c[0] & 3) | ((unsigned)(c[1] & 3) << 2) | ((unsigned)(c[2] & 3) << 4);
                state = 2;
            }
        }
        if (state == 2) {
            VT_STEP_HOOK(2);
            const unsigned half = (vb & 32u) ? (unsigned)(word >> 32) : (unsigned)word;
            if ((half >> (vb & 31u)) & 1u) {
#pragma unroll
                for (int i = 0; i < 3; ++i) h.c[i] = r.pos[i] ? nk[i] - 1 : nk[i];
                h.mat = 0u;
                h.t = t;
                h.axis = axis;
                return kHit;
            }
#pragma unroll
            for (int i = 0; i < 3; ++i) c[i] = r.pos[i] ? nk[i] - 1 : nk[i];
        }
        // leave the box: the voxel (sh 0, rad 1), or the empty chunk or
        // brick box as in step()
        int K[3];
        float tK[3];
#pragma unroll
        for (int i = 0; i < 3; ++i) {
            K[i] = exit_plane(i, c[i], sh, rad);
            tK[i] = sh == 0 ? tm[i] : ptime(r, i, K[i]);
        }
        const int e = tK[0] < tK[1] ? (tK[0] < tK[2] ? 0 : 2) : (tK[1] < tK[2] ? 1 : 2);
        const float T = e == 0 ? tK[0] : (e == 1 ? tK[1] : tK[2]);
        int crossings = 0, kx = 0;
        unsigned dv = 0;
#pragma unroll
        for (int i = 0; i < 3; ++i) {
            int cn = c[i];
            if (i == e) {
                cn = r.pos[i] ? K[i] : K[i] - 1;
                kx = K[i];                                            // the plane crossed
                dv = r.pos[i] ? (1u << (2 * i)) : 0u - (1u << (2 * i));  // the voxel's bit index moves by this
            } else if (key_lt(tm[i], i, T, e)) {
                cn = advance_axis<NEAR>(r, i, c[i], K[i], T, e);
            }
            crossings += abs(cn - c[i]);
            if (cn != c[i]) {
                nk[i] = r.pos[i] ? cn + 1 : cn;
                tm[i] = ptime(r, i, nk[i]);
            }
            c[i] = cn;
        }
        n += crossings;
        t = T;
        axis = e;
        if (n >= max_steps) return kMiss;
        if ((unsigned)c[0] >= (unsigned)w.dims[0] || (unsigned)c[1] >= (unsigned)w.dims[1] ||
            (unsigned)c[2] >= (unsigned)w.dims[2])
            return kMiss;
        // a unit step stays in the brick unless the crossed plane bounds it
        if (sh == 0 && (kx & 3) != 0) vb += dv;
        else state = 0;
        return kMore;
    }
};

template <bool MAT, bool RUN = true, bool NEAR = false, bool SHARE = false>
__device__ __forceinline__ bool trace_fast(const WorldView& w, const unsigned char* cdist, const PRay& r,
                                           int max_steps, TraceHit& h) {
    Walker wk;
    if (!wk.start_ray(w, r, max_steps)) return false;
    int s;
    while ((s = wk.step<MAT, RUN, NEAR, SHARE>(w, cdist, h)) == Walker::kMore) {
    }
    return s == Walker::kHit;
}

}  // namespace vt
