// tune.cu -- launch-configuration autotuner of the render kernels.
//
// The search space: the warp-tile shape of the one-thread-per-pixel kernel (a
// warp's pixel packet: 4x8, 8x4, 16x2 or 32x1 pixels) and its register budget,
// lanes sharing brick-word loads, the refill batch of the persistent
// pixel-queue kernel, an L2 persistence window over the brick words, and for
// frames with bounce rays the deferred bounce walk (its refill threshold and
// whether jumps and unit steps share one code path).  All produce identical
// records; the tuner times candidates on the caller's frame in phases (launch
// shape, then the L2 window, then the bounce pass, each phase keeping the
// fastest so far) and keeps the fastest.  Brick (4^3) and chunk (32^3) sizes
// are fixed by the data layout.  Choices can be cached in a small text file,
// one line per key:
//     <gpu name>|<X>x<Y>x<Z>|<W>x<H>|<rays>|<shade> <kernel> <tile w> <occupancy> <batch> <share> <l2> <refill> <walk> <sort> <ms>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

#include "vt_internal.h"

namespace {

bool valid(const vt_tuning& t) {
    if (t.share_bricks < 0 || t.share_bricks > 1 || t.l2_persist < 0 || t.l2_persist > 1 || t.bounce_refill < 0 ||
        t.bounce_refill > 32 || t.bounce_walk < 0 || t.bounce_walk > 1 || t.bounce_sort < 0 || t.bounce_sort > 1)
        return false;
    if (t.kernel == VT_KERNEL_TILE || t.kernel == VT_KERNEL_PER_JOB)
        return (t.warp_tile_w == 4 || t.warp_tile_w == 8 || t.warp_tile_w == 16 || t.warp_tile_w == 32) &&
               (t.occupancy == 0 || t.occupancy == 1) &&
               (!t.share_bricks || (t.warp_tile_w == 8 && t.occupancy == 1));
    if (t.kernel == VT_KERNEL_QUEUE) return t.batch >= 1 && t.batch <= 32 && !t.share_bricks;
    return false;
}

std::string cache_key(const vt_ctx* ctx, const vt_world* w, const vt_camera* cam, const vt_params* p) {
    std::ostringstream k;
    std::string name = ctx->name;
    for (char& ch : name)
        if (ch == ' ' || ch == '|') ch = '_';
    k << name << '|' << w->dims[0] << 'x' << w->dims[1] << 'x' << w->dims[2] << '|' << cam->width << 'x'
      << cam->height << '|' << (p->rays | VT_RAYS_PRIMARY) << '|' << p->shade;
    return k.str();
}

bool cache_lookup(const char* path, const std::string& key, vt_tuning* t, float* ms) {
    std::ifstream in(path);
    std::string line;
    bool found = false;
    while (std::getline(in, line)) {
        std::istringstream ls(line);
        std::string k;
        vt_tuning c;
        float m;
        if (ls >> k >> c.kernel >> c.warp_tile_w >> c.occupancy >> c.batch >> c.share_bricks >> c.l2_persist >>
                c.bounce_refill >> c.bounce_walk >> c.bounce_sort >> m &&
            k == key && valid(c)) {
            *t = c;
            *ms = m;
            found = true;  // the last record of a key wins
        }
    }
    return found;
}

void cache_store(const char* path, const std::string& key, const vt_tuning& t, float ms) {
    std::ofstream out(path, std::ios::app);
    out << key << ' ' << t.kernel << ' ' << t.warp_tile_w << ' ' << t.occupancy << ' ' << t.batch << ' '
        << t.share_bricks << ' ' << t.l2_persist << ' ' << t.bounce_refill << ' ' << t.bounce_walk << ' '
        << t.bounce_sort << ' ' << ms << '\n';
}

// Read-bandwidth probe: each thread streams 16-byte words of the buffer with
// L2-only loads (ld.global.cg, so that no pass is served from L1), four
// independent loads in flight per turn, `passes` times in one launch.  The
// XOR of everything read is kept live by a store that never happens.
constexpr int kProbeBlock = 512;
__global__ void __launch_bounds__(kProbeBlock) k_read_probe(const uint4* __restrict__ buf, size_t n16, int passes,
                                                             unsigned* __restrict__ sink) {
    const size_t stride = (size_t)gridDim.x * kProbeBlock;
    const size_t first = (size_t)blockIdx.x * kProbeBlock + threadIdx.x;
    unsigned acc = 0;
    for (int p = 0; p < passes; ++p) {
        size_t i = first;
        for (; i + 3 * stride < n16; i += 4 * stride) {
            const uint4 a = __ldcg(buf + i), b = __ldcg(buf + i + stride), c = __ldcg(buf + i + 2 * stride),
                        d = __ldcg(buf + i + 3 * stride);
            acc ^= (a.x ^ a.y ^ a.z ^ a.w) ^ (b.x ^ b.y ^ b.z ^ b.w) ^ (c.x ^ c.y ^ c.z ^ c.w) ^ (d.x ^ d.y ^ d.z ^ d.w);
        }
        for (; i < n16; i += stride) {
            const uint4 a = __ldcg(buf + i);
            acc ^= a.x ^ a.y ^ a.z ^ a.w;
        }
        acc = acc * 0x9E3779B1u + (unsigned)p;   // passes stay distinct work
    }
    if (acc == 0x2545F491u) atomicAdd(sink, 1u);
}

}  // namespace

using namespace vt;

extern "C" {

vt_status vt_probe_read_bandwidth(vt_ctx* ctx, uint64_t bytes, int32_t passes, float* gbs) {
    if (!ctx) return VT_ERR_ARG;
    if (!gbs || passes < 1 || passes > 100000 || bytes < (1u << 20) || bytes > (64ull << 30) || bytes % 16)
        return fail(ctx, VT_ERR_ARG, "probe: bytes in [1 MiB, 64 GiB], a multiple of 16; passes in [1, 100000]");
    void* buf = nullptr;
    unsigned* sink = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    cudaError_t e = dev_alloc(&buf, (size_t)bytes);
    if (e == cudaSuccess) e = dev_alloc(&sink, sizeof(unsigned));
    if (e == cudaSuccess) e = cudaMemsetAsync(buf, 0x5A, (size_t)bytes, ctx->stream);
    if (e == cudaSuccess) e = cudaEventCreate(&e0);
    if (e == cudaSuccess) e = cudaEventCreate(&e1);
    float ms = 0.0f;
    if (e == cudaSuccess) {
        int per_sm = 0;
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_read_probe, kProbeBlock, 0);
        const unsigned blocks = (unsigned)(ctx->sm_count * (per_sm > 0 ? per_sm : 1));
        const size_t n16 = (size_t)bytes / 16;
        if (e == cudaSuccess) {
            k_read_probe<<<blocks, kProbeBlock, 0, ctx->stream>>>((const uint4*)buf, n16, 1, sink);  // warm-up
            cudaEventRecord(e0, ctx->stream);
            k_read_probe<<<blocks, kProbeBlock, 0, ctx->stream>>>((const uint4*)buf, n16, passes, sink);
            cudaEventRecord(e1, ctx->stream);
            e = cudaGetLastError();
        }
        if (e == cudaSuccess) e = cudaEventSynchronize(e1);
        if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
    }
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    dev_free(sink);
    dev_free(buf);
    if (e != cudaSuccess) return check_cuda(ctx, e, "read-bandwidth probe");
    *gbs = (float)((double)bytes * (double)passes / ((double)ms * 1e-3) / 1e9);
    return VT_OK;
}

vt_status vt_set_tuning(vt_ctx* ctx, const vt_tuning* t) {
    if (!ctx) return VT_ERR_ARG;
    if (!t || !valid(*t)) return fail(ctx, VT_ERR_ARG, "invalid tuning");
    ctx->tuning = *t;
    return VT_OK;
}

vt_status vt_get_tuning(vt_ctx* ctx, vt_tuning* t) {
    if (!ctx || !t) return VT_ERR_ARG;
    *t = ctx->tuning;
    return VT_OK;
}

vt_status vt_autotune(vt_ctx* ctx, const vt_world* world, const vt_camera* cam, const vt_params* params, int32_t reps,
                      const char* cache_path, vt_tuning* best, float* best_ms) {
    if (!ctx) return VT_ERR_ARG;
    if (!world || !cam || !params) return fail(ctx, VT_ERR_ARG, "null world, camera or params");
    if (reps < 1 || reps > 10000) return fail(ctx, VT_ERR_ARG, "reps must be in [1, 10000]");
    const std::string key = cache_key(ctx, world, cam, params);
    vt_tuning found;
    float found_ms = 0.0f;
    if (cache_path && cache_lookup(cache_path, key, &found, &found_ms)) {
        ctx->tuning = found;
        if (best) *best = found;
        if (best_ms) *best_ms = found_ms;
        return VT_OK;
    }
    const size_t bytes = (size_t)cam->width * cam->height * sizeof(vt_hit);
    void* d_out = nullptr;
    vt_status s = ctx_scratch(ctx, bytes, &d_out);
    if (s) return s;
    cudaEvent_t e0, e1;
    VT_CUDA(ctx, cudaEventCreate(&e0));
    VT_CUDA(ctx, cudaEventCreate(&e1));
    const vt_tuning saved = ctx->tuning;
    vt_tuning win = saved;
    float win_ms = 0.0f;
    bool have = false;
    // times one candidate; keeps it if it is the fastest so far
    auto trial = [&](const vt_tuning& c) {
        ctx->tuning = c;
        for (int i = 0; i < 2 && !s; ++i) s = vt_render(ctx, world, cam, params, (vt_hit*)d_out, ctx->stream);
        if (!s) s = check_cuda(ctx, cudaEventRecord(e0, ctx->stream), "cudaEventRecord");
        for (int i = 0; i < reps && !s; ++i) s = vt_render(ctx, world, cam, params, (vt_hit*)d_out, ctx->stream);
        if (!s) s = check_cuda(ctx, cudaEventRecord(e1, ctx->stream), "cudaEventRecord");
        if (!s) s = check_cuda(ctx, cudaEventSynchronize(e1), "cudaEventSynchronize");
        float ms = 0.0f;
        if (!s) s = check_cuda(ctx, cudaEventElapsedTime(&ms, e0, e1), "cudaEventElapsedTime");
        if (s) return;
        ms /= (float)reps;
        if (!have || ms < win_ms) {
            win = c;
            win_ms = ms;
            have = true;
        }
    };
    // phase 1: the launch shape
    std::vector<vt_tuning> cands;
    for (int tw : {4, 8, 16, 32})
        for (int occ : {0, 1}) cands.push_back(vt_tuning{VT_KERNEL_TILE, tw, occ, 16, 0, 0, 0, 0, 0});
    cands.push_back(vt_tuning{VT_KERNEL_TILE, 8, 1, 16, 1, 0, 0, 0, 0});
    for (int b : {8, 16, 24}) cands.push_back(vt_tuning{VT_KERNEL_QUEUE, 8, 0, b, 0, 0, 0, 0, 0});
    for (const vt_tuning& c : cands)
        if (!s) trial(c);
    // phase 2: the L2 persistence window over the brick words
    if (!s) {
        vt_tuning c = win;
        c.l2_persist = 1;
        trial(c);
    }
    // phase 3: the deferred bounce pass (frames with bounce rays through the tile kernel)
    if (!s && (params->rays & VT_RAYS_BOUNCE) && win.kernel != VT_KERNEL_QUEUE) {
        const vt_tuning base = win;
        for (int sort : {0, 1})
            for (int walk : {0, 1})
                for (int refill : {4, 8, 16}) {
                    if (sort == 0 && walk == 0 && refill == 8) continue;  // the base's own (default) bounce pass
                    vt_tuning c = base;
                    c.bounce_sort = sort;
                    c.bounce_walk = walk;
                    c.bounce_refill = refill;
                    if (!s) trial(c);
                }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (s) {
        ctx->tuning = saved;
        return s;
    }
    ctx->tuning = win;
    if (cache_path) cache_store(cache_path, key, win, win_ms);
    if (best) *best = win;
    if (best_ms) *best_ms = win_ms;
    return VT_OK;
}

}  // extern "C"
