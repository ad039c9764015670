// batch.cu -- many scenes x cameras in one graph launch.
//
// A batch (jobs of a world, a camera and an output buffer each) is captured
// once into a CUDA graph and replayed with one cudaGraphLaunch.  Two shapes:
//
//   tile (default)  one production k_render launch per job, spread over
//                   kBatchChains independent chains of the graph, so that the
//                   tail of one job's launch overlaps the next jobs' work and
//                   every launch keeps its world and frame in kernel
//                   parameters (constant bank) as the single-frame path does.
//   queue           (ctx tuning VT_KERNEL_QUEUE) one persistent launch: every
//                   job is cut into 16 x 16 pixel units numbered job after
//                   job; a warp takes one unit at a time from a device
//                   counter, finds its job by binary search over the jobs'
//                   first-unit numbers and traces the unit's 256 pixels as
//                   eight 8 x 4 tiles with the same per-pixel code
//                   (render_pixel.cuh).  Its per-job state comes from global
//                   memory, which measured slower than the tile shape once
//                   the traversal itself got cheaper.
#include <algorithm>
#include <cstring>
#include <vector>

#include "render_pixel.cuh"

namespace vt {

struct JobDesc {
    WorldView w;
    FrameParams f;
    uint4* out;
    unsigned first_unit;
    unsigned units_x;
};

constexpr int kBatchBlock = 256;
constexpr int kUnit = 16;  // pixels per unit side
constexpr int kBatchChains = 8;  // 4, 8, 16 and 32 chains measured within 1% on the 64-scene batch

__global__ void __launch_bounds__(kBatchBlock, 3) k_render_batch(const JobDesc* __restrict__ jobs, int njobs,
                                                                 unsigned total_units, unsigned* __restrict__ counter) {
    const unsigned lane = threadIdx.x & 31u;
    for (;;) {
        unsigned unit = 0;
        if (lane == 0) unit = atomicAdd(counter, 1u);
        unit = __shfl_sync(0xFFFFFFFFu, unit, 0);
        if (unit >= total_units) break;
        int lo = 0, hi = njobs - 1;
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (__ldg(&jobs[mid].first_unit) <= unit) lo = mid;
            else hi = mid - 1;
        }
        const JobDesc& J = jobs[lo];
        const unsigned local = unit - J.first_unit;
        const int ux = (int)(local % J.units_x) * kUnit, uy = (int)(local / J.units_x) * kUnit;
        // world and frame are read from the job table in place (L1-cached):
        // copying the two structs into registers spills
        const WorldView& w = J.w;
        const FrameParams& f = J.f;
        for (int sub = 0; sub < 8; ++sub) {
            const int px = ux + (sub & 1) * 8 + (int)(lane & 7u);
            const int py = uy + (sub >> 1) * 4 + (int)(lane >> 3);
            if (px < f.width && py < f.height) {
                PixelCounters pc;
                J.out[(size_t)py * f.width + px] =
                    render_pixel<false, false>(w, CoarseGlobal{w.coarse}, w.cdist, f, px, py, pixel_uv(f, px, py),
                                               nullptr, pc);
            }
        }
    }
}

}  // namespace vt

struct vt_batch {
    vt_ctx* ctx = nullptr;
    std::vector<const vt_world*> worlds;
    std::vector<vt_job> jobs;
    vt_params params;
    vt::JobDesc* d_jobs = nullptr;
    unsigned* d_counter = nullptr;
    int njobs = 0;
    unsigned total_units = 0;
    unsigned long long pixels = 0;
    unsigned blocks = 0;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
};

using namespace vt;

extern "C" {

vt_status vt_batch_create(vt_ctx* ctx, const vt_job* jobs, int32_t n, const vt_params* params, vt_batch** out) {
    if (!ctx) return VT_ERR_ARG;
    if (!jobs || !params || !out || n <= 0) return fail(ctx, VT_ERR_ARG, "bad batch arguments");
    *out = nullptr;
    std::vector<JobDesc> host((size_t)n);
    unsigned long long units = 0, pixels = 0;
    vt_batch* b = new (std::nothrow) vt_batch();
    if (!b) return fail(ctx, VT_ERR_OOM, "host allocation failed");
    for (int i = 0; i < n; ++i) {
        const vt_job& j = jobs[i];
        vt_status s = check_frame_args(ctx, j.world, &j.camera, params);
        if (!s && !j.d_out) s = fail(ctx, VT_ERR_ARG, "null job output");
        if (s) {
            delete b;
            return s;
        }
        JobDesc& d = host[(size_t)i];
        d.w = j.world->view();
        d.f = make_frame(&j.camera, params);
        d.out = reinterpret_cast<uint4*>(j.d_out);
        d.first_unit = (unsigned)units;
        d.units_x = (unsigned)((j.camera.width + kUnit - 1) / kUnit);
        units += (unsigned long long)d.units_x * (unsigned)((j.camera.height + kUnit - 1) / kUnit);
        pixels += (unsigned long long)j.camera.width * (unsigned long long)j.camera.height;
        b->worlds.push_back(j.world);
        b->jobs.push_back(j);
    }
    b->params = *params;
    if (units >= (1ull << 32)) {
        delete b;
        return fail(ctx, VT_ERR_ARG, "batch too large (units >= 2^32)");
    }
    cudaError_t e;
    if ((e = vt::dev_alloc(&b->d_jobs, host.size() * sizeof(JobDesc))) != cudaSuccess ||
        (e = vt::dev_alloc(&b->d_counter, sizeof(unsigned))) != cudaSuccess ||
        (e = cudaMemcpy(b->d_jobs, host.data(), host.size() * sizeof(JobDesc), cudaMemcpyHostToDevice)) != cudaSuccess) {
        vt_batch_destroy(b);
        return check_cuda(ctx, e, "batch upload");
    }
    int per_sm = 0;
    if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_render_batch, kBatchBlock, 0)) != cudaSuccess) {
        vt_batch_destroy(b);
        return check_cuda(ctx, e, "cudaOccupancyMaxActiveBlocksPerMultiprocessor");
    }
    b->ctx = ctx;
    b->njobs = n;
    b->total_units = (unsigned)units;
    b->pixels = pixels;
    b->blocks = (unsigned)(ctx->sm_count * std::max(per_sm, 1));
    *out = b;
    return VT_OK;
}

vt_status vt_batch_launch(vt_batch* b, vt_stream stream) {
    if (!b) return VT_ERR_ARG;
    vt_ctx* ctx = b->ctx;
    cudaStream_t st = (cudaStream_t)stream;
    // stale empty-space distances are rebuilt before (outside) the graph
    for (const vt_world* w : b->worlds) {
        vt_status s = update_distances(const_cast<vt_world*>(w), st);
        if (s) return s;
    }
    if (!b->exec) {
        // capture on private streams: the legacy default stream cannot be captured
        cudaStream_t cap = nullptr;
        cudaStream_t chain[kBatchChains] = {};
        cudaEvent_t fork = nullptr, join[kBatchChains] = {};
        cudaError_t e = cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking);
        const bool queue = ctx->tuning.kernel == VT_KERNEL_QUEUE;
        vt_status s = VT_OK;
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&fork, cudaEventDisableTiming);
        for (int k = 0; k < kBatchChains && e == cudaSuccess; ++k) {
            e = cudaStreamCreateWithFlags(&chain[k], cudaStreamNonBlocking);
            if (e == cudaSuccess) e = cudaEventCreateWithFlags(&join[k], cudaEventDisableTiming);
        }
        if (e == cudaSuccess) e = cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal);
        if (e == cudaSuccess) {
            if (queue) {
                cudaMemsetAsync(b->d_counter, 0, sizeof(unsigned), cap);
                k_render_batch<<<b->blocks, kBatchBlock, 0, cap>>>(b->d_jobs, b->njobs, b->total_units, b->d_counter);
            } else {
                // fork kBatchChains chains off the capture stream, jobs round robin, join
                cudaEventRecord(fork, cap);
                for (int k = 0; k < kBatchChains; ++k) cudaStreamWaitEvent(chain[k], fork, 0);
                for (size_t j = 0; j < b->jobs.size() && !s; ++j) {
                    const vt_job& jb = b->jobs[j];
                    s = launch_render(ctx, jb.world, &jb.camera, &b->params, reinterpret_cast<uint4*>(jb.d_out),
                                      chain[j % kBatchChains], false);
                }
                for (int k = 0; k < kBatchChains; ++k) {
                    cudaEventRecord(join[k], chain[k]);
                    cudaStreamWaitEvent(cap, join[k], 0);
                }
            }
            const cudaError_t e2 = cudaStreamEndCapture(cap, &b->graph);
            if (e == cudaSuccess) e = e2;
        }
        for (int k = 0; k < kBatchChains; ++k) {
            if (chain[k]) cudaStreamDestroy(chain[k]);
            if (join[k]) cudaEventDestroy(join[k]);
        }
        if (fork) cudaEventDestroy(fork);
        if (cap) cudaStreamDestroy(cap);
        if (s) return s;
        if (e != cudaSuccess) return check_cuda(ctx, e, "batch graph capture");
        VT_CUDA(ctx, cudaGraphInstantiate(&b->exec, b->graph, 0));
    }
    VT_CUDA(ctx, cudaGraphLaunch(b->exec, st));
    // checked jobs may set the status word (their capture noted nothing)
    if (b->params.flags & VT_FLAG_CHECKED) return note_status_writer(ctx, st);
    return VT_OK;
}

vt_status vt_batch_destroy(vt_batch* b) {
    if (!b) return VT_ERR_ARG;
    cudaDeviceSynchronize();
    if (b->exec) cudaGraphExecDestroy(b->exec);
    if (b->graph) cudaGraphDestroy(b->graph);
    if (b->d_jobs) vt::dev_free(b->d_jobs);
    if (b->d_counter) vt::dev_free(b->d_counter);
    delete b;
    return VT_OK;
}

vt_status vt_batch_info(const vt_batch* b, uint64_t* pixels, int32_t* jobs, uint32_t* units) {
    if (!b) return VT_ERR_ARG;
    if (pixels) *pixels = b->pixels;
    if (jobs) *jobs = b->njobs;
    if (units) *units = b->total_units;
    return VT_OK;
}

}  // extern "C"
