// Test-only: compiles the device traversal (trace_p.cuh) as host C++ so that
// its jump logic can be compared with the unit-step oracle without a GPU, and
// so that the benchmark can time the skipping walk on the host cores beside
// the unit-step oracle (ht_world_new / ht_trace_mt).  The CUDA intrinsics it
// uses are given their IEEE host equivalents.
#include <math.h>
#include <stdint.h>
#include <string.h>
#include <limits.h>
#include <algorithm>
#include <thread>
#include <vector>

#include <cuda_runtime.h>

using std::max;
using std::min;
static inline float __fmaf_rn(float a, float b, float c) { return fmaf(a, b, c); }
static inline float __frcp_rn(float x) { return 1.0f / x; }
static inline float __fmul_rn(float a, float b) { return a * b; }
static inline float __int2float_rn(int k) { return (float)k; }
static inline int __float2int_rd(float x) {
    if (x != x) return 0;
    if (x >= 2147483647.0f) return INT_MAX;
    if (x <= -2147483648.0f) return INT_MIN;
    return (int)floorf(x);
}
template <class T> static inline T __ldg(const T* p) { return *p; }
static inline unsigned atomicOr(unsigned* p, unsigned v) { unsigned o = *p; *p |= v; return o; }

#include "../../unnamed-voxel-tracer_gb300/csrc/trace_p.cuh"

// Summed-area table of an occupancy grid: count(box) in O(1).
struct Sat {
    int gx, gy, gz;
    std::vector<int> s;
    template <class Occ>
    Sat(int x_, int y_, int z_, Occ occ) : gx(x_), gy(y_), gz(z_), s((size_t)(x_ + 1) * (y_ + 1) * (z_ + 1), 0) {
        for (int z = 0; z < gz; ++z)
            for (int y = 0; y < gy; ++y)
                for (int x = 0; x < gx; ++x)
                    at(x + 1, y + 1, z + 1) = (occ(x, y, z) ? 1 : 0) + at(x, y + 1, z + 1) + at(x + 1, y, z + 1) +
                                              at(x + 1, y + 1, z) - at(x, y, z + 1) - at(x, y + 1, z) -
                                              at(x + 1, y, z) + at(x, y, z);
    }
    int& at(int x, int y, int z) { return s[(size_t)x + (size_t)(gx + 1) * ((size_t)y + (size_t)(gy + 1) * z)]; }
    int count(int x0, int x1, int y0, int y1, int z0, int z1) {  // inclusive, clipped to the grid
        x0 = std::max(x0, 0); y0 = std::max(y0, 0); z0 = std::max(z0, 0);
        x1 = std::min(x1, gx - 1); y1 = std::min(y1, gy - 1); z1 = std::min(z1, gz - 1);
        if (x0 > x1 || y0 > y1 || z0 > z1) return 0;
        return at(x1 + 1, y1 + 1, z1 + 1) - at(x0, y1 + 1, z1 + 1) - at(x1 + 1, y0, z1 + 1) - at(x1 + 1, y1 + 1, z0) +
               at(x0, y0, z1 + 1) + at(x0, y1 + 1, z0) + at(x1 + 1, y0, z0) - at(x0, y0, z0);
    }
};

// Chunk distances: max(|dx|, |dy|, |dz|) (capped at kDistCap + 1) from each
// cell of a gx*gy*gz occupancy grid to the nearest occupied cell ahead in
// octant oct (bit i set: d_i >= 0, else d_i <= 0).  Computed independently of
// the library's separable passes: the smallest r whose box (r cells ahead)
// holds an occupied cell, counted with a summed-area table.
static std::vector<unsigned char> cheb(const std::vector<unsigned char>& occ, int gx, int gy, int gz, int oct) {
    Sat sat(gx, gy, gz, [&](int x, int y, int z) { return occ[(size_t)x + (size_t)gx * ((size_t)y + (size_t)gy * z)] != 0; });
    std::vector<unsigned char> d((size_t)gx * gy * gz);
    for (int z = 0; z < gz; ++z)
        for (int y = 0; y < gy; ++y)
            for (int x = 0; x < gx; ++x) {
                int best = vt::kDistCap + 1;
                for (int r = 0; r <= vt::kDistCap; ++r) {
                    const int x0 = (oct & 1) ? x : x - r, x1 = (oct & 1) ? x + r : x;
                    const int y0 = (oct & 2) ? y : y - r, y1 = (oct & 2) ? y + r : y;
                    const int z0 = (oct & 4) ? z : z - r, z1 = (oct & 4) ? z + r : z;
                    if (sat.count(x0, x1, y0, y1, z0, z1) > 0) {
                        best = r;
                        break;
                    }
                }
                d[(size_t)x + (size_t)gx * ((size_t)y + (size_t)gy * z)] = (unsigned char)best;
            }
    return d;
}

// Brick distances in voxel layers for octant oct: per brick of the gx*gy*gz
// brick grid, 0 if the brick holds an occupied voxel, else s | shape << 6
// where s is the smallest E (capped at kVoxCap + 1) for which the brick grown
// by E voxel layers beyond its far faces across and E >> shape layers
// vertically holds one: shape 0 for the octants moving +y, else the shape
// 0..3 whose empty box is largest (box_score; the first on a tie).  Found by
// bisection over E with a summed-area table of the voxels: independent of
// the library's separable passes.
static std::vector<unsigned char> voxel_cheb(Sat& sat, int gx, int gy, int gz, int oct) {
    int shape = 0;
    auto occupied = [&](int bx, int by, int bz, int E) {
        const int ex = E, ey = E >> shape, ez = E;
        const int x0 = (oct & 1) ? 4 * bx : 4 * bx - ex, x1 = (oct & 1) ? 4 * bx + 3 + ex : 4 * bx + 3;
        const int y0 = (oct & 2) ? 4 * by : 4 * by - ey, y1 = (oct & 2) ? 4 * by + 3 + ey : 4 * by + 3;
        const int z0 = (oct & 4) ? 4 * bz : 4 * bz - ez, z1 = (oct & 4) ? 4 * bz + 3 + ez : 4 * bz + 3;
        return sat.count(x0, x1, y0, y1, z0, z1) > 0;
    };
    std::vector<unsigned char> d((size_t)gx * gy * gz);
    for (int z = 0; z < gz; ++z)
        for (int y = 0; y < gy; ++y)
            for (int x = 0; x < gx; ++x) {
                int v = 0, best_score = -1;
                for (shape = 0; shape < ((oct & 2) ? 1 : vt::kBoxShapes) && !occupied(x, y, z, 0); ++shape) {
                    int lo = 0, hi = vt::kVoxCap;   // the largest E in [0, kVoxCap] whose box is empty
                    while (lo < hi) {
                        const int mid = (lo + hi + 1) / 2;
                        if (occupied(x, y, z, mid)) hi = mid - 1;
                        else lo = mid;
                    }
                    if (vt::box_score(lo + 1, shape) > best_score) {
                        best_score = vt::box_score(lo + 1, shape);
                        v = (lo + 1) | (shape << 6);
                    }
                }
                d[(size_t)x + (size_t)gx * ((size_t)y + (size_t)gy * z)] = (unsigned char)v;
            }
    return d;
}

// The 8 octant fields of brick and chunk distances for a world's mask words,
// in the library's layout (chunk fields `cstride` bytes apart).
static void distances(const int cd[3], const std::vector<unsigned long long>& mask, std::vector<unsigned char>& bdist,
                      std::vector<unsigned char>& cdist, size_t cstride) {
    const size_t nch = (size_t)cd[0] * cd[1] * cd[2];
    const int gx = cd[0] * 8, gy = cd[1] * 8, gz = cd[2] * 8;
    std::vector<unsigned char> cocc(nch);
    for (size_t ci = 0; ci < nch; ++ci)
        for (int bi = 0; bi < 512 && !cocc[ci]; ++bi) cocc[ci] = mask[ci * 512 + bi] != 0;
    Sat vsat(gx * 4, gy * 4, gz * 4, [&](int x, int y, int z) {
        const size_t ci = (size_t)(x >> 5) + cd[0] * ((size_t)(y >> 5) + (size_t)cd[1] * (z >> 5));
        const unsigned bi = ((x >> 2) & 7) | (((y >> 2) & 7) << 3) | (((z >> 2) & 7) << 6);
        return ((mask[ci * 512 + bi] >> ((x & 3) | ((y & 3) << 2) | ((z & 3) << 4))) & 1ull) != 0;
    });
    bdist.assign(vt::kOctants * nch * 512, 0);
    cdist.assign(vt::kOctants * cstride, 0);
    for (int o = 0; o < vt::kOctants; ++o) {
        std::vector<unsigned char> bd = voxel_cheb(vsat, gx, gy, gz, o),
                                   cdd = cheb(cocc, cd[0], cd[1], cd[2], o);
        for (int z = 0; z < gz; ++z)
            for (int y = 0; y < gy; ++y)
                for (int x = 0; x < gx; ++x) {
                    size_t ci = (size_t)(x >> 3) + cd[0] * ((size_t)(y >> 3) + (size_t)cd[1] * (z >> 3));
                    unsigned bi = (x & 7) | ((y & 7) << 3) | ((z & 7) << 6);
                    bdist[o * nch * 512 + ci * 512 + bi] = bd[(size_t)x + (size_t)gx * ((size_t)y + (size_t)gy * z)];
                }
        std::copy(cdd.begin(), cdd.end(), cdist.begin() + (size_t)o * cstride);
    }
}

// The same fields for a dense world (X*Y*Z bytes), chunk fields packed
// (nchunks bytes apart), the layout vt_world_download_distances returns.
extern "C" void ht_distances(const int32_t dims[3], const uint8_t* dense, uint8_t* h_brick, uint8_t* h_chunk) {
    int cd[3];
    for (int i = 0; i < 3; ++i) cd[i] = (dims[i] + 31) / 32;
    const size_t nch = (size_t)cd[0] * cd[1] * cd[2];
    std::vector<unsigned long long> mask(nch * 512, 0ull);
    for (int z = 0; z < dims[2]; ++z)
        for (int y = 0; y < dims[1]; ++y)
            for (int x = 0; x < dims[0]; ++x)
                if (dense[(size_t)x + (size_t)dims[0] * ((size_t)y + (size_t)dims[1] * z)]) {
                    size_t ci = (size_t)(x >> 5) + cd[0] * ((size_t)(y >> 5) + (size_t)cd[1] * (z >> 5));
                    unsigned bi = ((x >> 2) & 7) | (((y >> 2) & 7) << 3) | (((z >> 2) & 7) << 6);
                    mask[ci * 512 + bi] |= 1ull << ((x & 3) | ((y & 3) << 2) | ((z & 3) << 4));
                }
    std::vector<unsigned char> b, c;
    distances(cd, mask, b, c, nch);
    std::copy(b.begin(), b.end(), h_brick);
    std::copy(c.begin(), c.end(), h_chunk);
}

// A mode-P world in the kernel's layout (brick words, materials, coarse bits,
// octant distances), built once on the host.
struct HostWorld {
    vt::WorldView w;
    std::vector<unsigned long long> mask, coarse;
    std::vector<unsigned char> mats, bdist, cdist;
};

extern "C" void* ht_world_new(const int32_t dims[3], const uint8_t* dense) {
    HostWorld* hw = new HostWorld();
    vt::WorldView& w = hw->w;
    memset(&w, 0, sizeof(w));
    int cd[3];
    for (int i = 0; i < 3; ++i) {
        w.dims[i] = dims[i];
        cd[i] = w.cdim[i] = (dims[i] + 31) / 32;
    }
    const size_t nch = (size_t)cd[0] * cd[1] * cd[2];
    hw->mask.assign(nch * 512, 0ull);
    hw->coarse.assign((nch + 63) / 64, 0ull);
    hw->mats.assign(nch * 32768, 0);
    for (int z = 0; z < dims[2]; ++z)
        for (int y = 0; y < dims[1]; ++y)
            for (int x = 0; x < dims[0]; ++x) {
                unsigned char m = dense[(size_t)x + (size_t)dims[0] * ((size_t)y + (size_t)dims[1] * z)];
                if (!m) continue;
                size_t ci = (size_t)(x >> 5) + cd[0] * ((size_t)(y >> 5) + (size_t)cd[1] * (z >> 5));
                unsigned bi = ((x >> 2) & 7) | (((y >> 2) & 7) << 3) | (((z >> 2) & 7) << 6);
                unsigned vb = (x & 3) | ((y & 3) << 2) | ((z & 3) << 4);
                hw->mask[ci * 512 + bi] |= 1ull << vb;
                hw->mats[(ci * 512 + bi) * 64 + vb] = m;
                hw->coarse[ci >> 6] |= 1ull << (ci & 63);
            }
    const unsigned cstride = vt::cdist_stride((unsigned)nch);
    distances(cd, hw->mask, hw->bdist, hw->cdist, cstride);
    w.mask = hw->mask.data();
    w.mats = hw->mats.data();
    w.coarse = hw->coarse.data();
    w.bdist = hw->bdist.data();
    w.cdist = hw->cdist.data();
    w.nwords = (unsigned)(nch * 512);
    w.ncoarse = (unsigned)hw->coarse.size();
    w.nchunks = (unsigned)nch;
    w.cstride = cstride;
    return hw;
}

extern "C" void ht_world_free(void* p) { delete static_cast<HostWorld*>(p); }

// The production walk over n rays on `threads` host threads (rays split in
// interleaved blocks of 256): out gets per ray {voxel, t bits, material,
// face | hit << 8} (voxel 0xFFFFFFFF on a miss).
extern "C" void ht_trace_mt(const void* world, const float* origins, const float* dirs, int64_t n, int32_t max_steps,
                            uint32_t* out, int32_t threads) {
    const vt::WorldView& w = static_cast<const HostWorld*>(world)->w;
    auto work = [&](int t) {
        for (int64_t b = (int64_t)t * 256; b < n; b += (int64_t)threads * 256) {
            const int64_t e = std::min<int64_t>(n, b + 256);
            for (int64_t i = b; i < e; ++i) {
                vt::PRay r;
                vt::pray_init(r, origins + 3 * i, dirs + 3 * i);
                vt::TraceHit h;
                const bool hit = vt::near_origin(r.o) ? vt::trace_fast<true, true, true>(w, w.cdist, r, max_steps, h)
                                                      : vt::trace_fast<true, true, false>(w, w.cdist, r, max_steps, h);
                uint32_t* o = out + 4 * i;
                if (hit) {
                    o[0] = (uint32_t)h.c[0] + (uint32_t)w.dims[0] * ((uint32_t)h.c[1] + (uint32_t)w.dims[1] * (uint32_t)h.c[2]);
                    memcpy(&o[1], &h.t, 4);
                    o[2] = h.mat;
                    o[3] = (2u * h.axis + (r.pos[h.axis] ? 0u : 1u)) | (1u << 8);
                } else {
                    const float mt = -1.0f;
                    o[0] = 0xFFFFFFFFu;
                    memcpy(&o[1], &mt, 4);
                    o[2] = 0;
                    o[3] = 0xFFu;
                }
            }
        }
    };
    if (threads < 1) threads = 1;
    std::vector<std::thread> pool;
    for (int t = 1; t < threads; ++t) pool.emplace_back(work, t);
    work(0);
    for (auto& th : pool) th.join();
}

// One frame's rays on `threads` host threads: the primary ray of each entry
// (origins/dirs), and for each hit the shadow ray toward sun (origin = the hit
// point moved 0.001 off the entered face, as in the render kernel).  Returns
// the rays traced; *shadowed counts the blocked shadow rays.
extern "C" int64_t ht_frame_mt(const void* world, const float* origins, const float* dirs, int64_t n,
                               int32_t max_steps, const float sun[3], int32_t shadow_max_steps, int32_t threads,
                               int64_t* shadowed) {
    const vt::WorldView& w = static_cast<const HostWorld*>(world)->w;
    float sd[3], sinv[3];
    for (int j = 0; j < 3; ++j) {
        sd[j] = sun[j] == 0.0f ? 0.001f : sun[j];
        sinv[j] = 1.0f / sd[j];
    }
    if (threads < 1) threads = 1;
    std::vector<int64_t> rays(threads, 0), dark(threads, 0);
    auto work = [&](int t) {
        for (int64_t b = (int64_t)t * 256; b < n; b += (int64_t)threads * 256) {
            const int64_t e = std::min<int64_t>(n, b + 256);
            for (int64_t i = b; i < e; ++i) {
                vt::PRay r;
                vt::pray_init(r, origins + 3 * i, dirs + 3 * i);
                vt::TraceHit h;
                rays[t]++;
                const bool hit = vt::near_origin(r.o) ? vt::trace_fast<true, true, true>(w, w.cdist, r, max_steps, h)
                                                      : vt::trace_fast<true, true, false>(w, w.cdist, r, max_steps, h);
                if (!hit || shadow_max_steps <= 0) continue;
                float so[3];
                for (int j = 0; j < 3; ++j) {
                    so[j] = fmaf(r.d[j], h.t, origins[3 * i + j]);
                    if (j == h.axis) so[j] = so[j] + (r.pos[j] ? -1.0f : 1.0f) * 0.001f;
                }
                vt::PRay rs;
                vt::pray_init_dir(rs, so, sd, sinv);
                vt::TraceHit hs;
                rays[t]++;
                dark[t] += vt::trace_fast<false, true, true>(w, w.cdist, rs, shadow_max_steps, hs) ? 1 : 0;
            }
        }
    };
    std::vector<std::thread> pool;
    for (int t = 1; t < threads; ++t) pool.emplace_back(work, t);
    work(0);
    for (auto& th : pool) th.join();
    int64_t total = 0, blocked = 0;
    for (int t = 0; t < threads; ++t) {
        total += rays[t];
        blocked += dark[t];
    }
    if (shadowed) *shadowed = blocked;
    return total;
}

extern "C" int ht_trace_rays(const int32_t dims[3], const uint8_t* dense, const float* origins, const float* dirs,
                             int32_t n, int32_t max_steps, uint32_t* out /* n * 4 u32, vt_hit layout */,
                             uint64_t* counters /* mask, coarse */, int32_t fast) {
    vt::WorldView w;
    int cd[3];
    for (int i = 0; i < 3; ++i) {
        w.dims[i] = dims[i];
        cd[i] = w.cdim[i] = (dims[i] + 31) / 32;
    }
    const size_t nch = (size_t)cd[0] * cd[1] * cd[2];
    std::vector<unsigned long long> mask(nch * 512, 0ull), coarse((nch + 63) / 64, 0ull);
    std::vector<unsigned char> mats(nch * 32768, 0);
    for (int z = 0; z < dims[2]; ++z)
        for (int y = 0; y < dims[1]; ++y)
            for (int x = 0; x < dims[0]; ++x) {
                unsigned char m = dense[(size_t)x + (size_t)dims[0] * ((size_t)y + (size_t)dims[1] * z)];
                if (!m) continue;
                size_t ci = (size_t)(x >> 5) + cd[0] * ((size_t)(y >> 5) + (size_t)cd[1] * (z >> 5));
                unsigned bi = ((x >> 2) & 7) | (((y >> 2) & 7) << 3) | (((z >> 2) & 7) << 6);
                unsigned vb = (x & 3) | ((y & 3) << 2) | ((z & 3) << 4);
                mask[ci * 512 + bi] |= 1ull << vb;
                mats[(ci * 512 + bi) * 64 + vb] = m;
                coarse[ci >> 6] |= 1ull << (ci & 63);
            }
    w.mask = mask.data();
    w.mats = mats.data();
    w.coarse = coarse.data();
    w.palette = nullptr;
    w.nwords = (unsigned)(nch * 512);
    w.ncoarse = (unsigned)coarse.size();
    // empty-space distances in the kernel's brick order and chunk order
    const unsigned cstride = vt::cdist_stride((unsigned)nch);
    std::vector<unsigned char> bdist, cdist;
    distances(cd, mask, bdist, cdist, cstride);
    w.bdist = bdist.data();
    w.cdist = cdist.data();
    w.nchunks = (unsigned)nch;
    w.cstride = cstride;
    unsigned status = 0;
    for (int i = 0; i < n; ++i) {
        vt::PRay r;
        vt::pray_init(r, origins + 3 * i, dirs + 3 * i);
        vt::TraceHit h;
        vt::TraceCounters cnt;
        bool hit;
        if (fast) {
            // the production walk (fast 1: step, fast 2: step_flat), one step
            // at a time; counters[0] = steps taken
            vt::Walker wk;
            hit = false;
            if (wk.start(w, r.o, r.d, max_steps)) {
                int s;
                const bool near = vt::near_origin(r.o);
                do {
                    if (fast == 2) s = near ? wk.step_flat<true>(w, w.cdist, h) : wk.step_flat<false>(w, w.cdist, h);
                    else s = near ? wk.step<true, true, true>(w, w.cdist, h) : wk.step<true, true, false>(w, w.cdist, h);
                    counters[0]++;
                } while (s == vt::Walker::kMore);
                hit = s == vt::Walker::kHit;
                if (hit && fast == 2) h.mat = w.mats[(size_t)wk.wi * 64u + wk.vb];   // step_flat reads no material
            }
        } else {
            hit = vt::trace_p<true, true, true>(w, vt::CoarseGlobal{w.coarse}, r, max_steps, h, cnt, &status);
        }
        uint32_t* o = out + 4 * i;
        if (hit) {
            const int e = h.axis;
            const bool pe = r.pos[e];
            o[0] = (uint32_t)h.c[0] + (uint32_t)dims[0] * ((uint32_t)h.c[1] + (uint32_t)dims[1] * (uint32_t)h.c[2]);
            memcpy(&o[1], &h.t, 4);
            o[2] = fast ? 0u : cnt.steps;
            o[3] = (2u * e + (pe ? 0u : 1u)) | (h.mat << 8) | (1u << 16);
        } else {
            float mt = -1.0f;
            o[0] = 0xFFFFFFFFu;
            memcpy(&o[1], &mt, 4);
            o[2] = 0;
            o[3] = 0xFFu;
        }
        counters[0] += cnt.mask;
        counters[1] += cnt.coarse;
    }
    return (int)status;
}
