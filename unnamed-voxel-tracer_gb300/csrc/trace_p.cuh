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
// position gives the first guess; the exact plane times decide.
__device__ __forceinline__ int advance_axis(const PRay& r, int i, int lo, int K, float T, int e) {
    float p = __fmaf_rn(r.d[i], T, r.o[i]);
    int k = __float2int_rd(p);
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
            else c[i] = r.pos[i] ? advance_axis(r, i, 0, D[i], T0, e) : advance_axis(r, i, D[i] - 1, 0, T0, e);
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
template <bool STATS, bool CHECKED, bool MAT, class Coarse>
__device__ __forceinline__ bool trace_p(const WorldView& w, const Coarse& coarse, const PRay& r, int max_steps,
                                        TraceHit& h, TraceCounters& cnt, unsigned* status) {
    int c[3];
    float t;
    int axis;
    if (!pray_start(r, w.dims, c, t, axis)) return false;
    if (max_steps <= 0) return false;
    int n = 0;
    unsigned cached_wi = 0xFFFFFFFFu;
    unsigned long long word = 0ull;
    unsigned last_cw = 0xFFFFFFFFu;
    for (;;) {
        if (STATS) cnt.iters++;
        const unsigned ci = (unsigned)(c[0] >> 5) + (unsigned)w.cdim[0] * ((unsigned)(c[1] >> 5) + (unsigned)w.cdim[1] * (unsigned)(c[2] >> 5));
        const unsigned cw = ci >> 6;
        if (CHECKED && cw >= w.ncoarse) {
            atomicOr(status, kStatusOob);
            return false;
        }
        if (STATS && cw != last_cw) {
            last_cw = cw;
            cnt.coarse++;
        }
        int sh;
        if (!((coarse(cw) >> (ci & 63u)) & 1ull)) {
            sh = 5;
        } else {
            const unsigned bi = (unsigned)((c[0] >> 2) & 7) | ((unsigned)((c[1] >> 2) & 7) << 3) | ((unsigned)((c[2] >> 2) & 7) << 6);
            const unsigned wi = ci * 512u + bi;
            if (wi != cached_wi) {
                if (CHECKED && wi >= w.nwords) {
                    atomicOr(status, kStatusOob);
                    return false;
                }
                word = __ldg(w.mask + wi);
                cached_wi = wi;
                if (STATS) cnt.mask++;
            }
            if (word == 0ull) {
                sh = 2;
            } else {
                const unsigned vb = (unsigned)(c[0] & 3) | ((unsigned)(c[1] & 3) << 2) | ((unsigned)(c[2] & 3) << 4);
                if ((word >> vb) & 1ull) {
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
        // Exit of the aligned 2^sh region that contains c.
        int K[3];
        float tK[3];
#pragma unroll
        for (int i = 0; i < 3; ++i) {
            const int base = (c[i] >> sh) << sh;
            K[i] = r.pos[i] ? base + (1 << sh) : base;
            tK[i] = ptime(r, i, K[i]);
        }
        const int e = tK[0] < tK[1] ? (tK[0] < tK[2] ? 0 : 2) : (tK[1] < tK[2] ? 1 : 2);
        const float T = e == 0 ? tK[0] : (e == 1 ? tK[1] : tK[2]);
        int crossings = 0;
        if (sh) {
#pragma unroll
            for (int i = 0; i < 3; ++i) {
                if (i != e) {
                    const int nk = r.pos[i] ? c[i] + 1 : c[i];
                    if (crossed(r, i, nk, T, e)) {
                        const int cn = advance_axis(r, i, c[i], K[i], T, e);
                        crossings += abs(cn - c[i]);
                        c[i] = cn;
                    }
                }
            }
        }
#pragma unroll
        for (int i = 0; i < 3; ++i) {
            if (i == e) {
                const int cn = r.pos[i] ? K[i] : K[i] - 1;
                crossings += abs(cn - c[i]);
                c[i] = cn;
            }
        }
        n += crossings;
        t = T;
        axis = e;
        if (n >= max_steps) break;
        if ((unsigned)c[0] >= (unsigned)w.dims[0] || (unsigned)c[1] >= (unsigned)w.dims[1] ||
            (unsigned)c[2] >= (unsigned)w.dims[2])
            break;
    }
    if (STATS) cnt.steps += (unsigned)min(n, max_steps);
    return false;
}

}  // namespace vt
