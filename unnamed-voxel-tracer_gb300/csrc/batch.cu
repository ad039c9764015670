// batch.cu -- many scenes x cameras in one graph launch.
//
// A batch (jobs of a world, a camera and an output buffer each) is captured
// once into a CUDA graph and replayed with one cudaGraphLaunch.  Three shapes:
//
//   tile (default)  the consecutive jobs of each world (up to kLaunchJobs
//                   jobs and about 4 Mpixels) are ONE launch of k_render_jobs
//                   whose grid covers every 16 x 16-pixel tile of all of
//                   them, on kBatchChains concurrent chains of the graph
//                   (longest launch first, on the least loaded chain).  The launch's job table
//                   (the world, the shared frame settings, each job's camera,
//                   output and first tile) is the kernel's parameter block
//                   itself (__grid_constant__, < 32 KB): a block finds its
//                   job by a binary search over blockIdx, and the world's
//                   fields are constant-bank operands as in a single-frame
//                   launch.  The hardware hands out blocks as SMs free up, so
//                   the tiles of all cameras of a world share one launch
//                   tail.
//   per job         (VT_KERNEL_PER_JOB) one production k_render launch per
//                   job, spread over kBatchChains concurrent chains of the
//                   graph the same way, so that one job's tail overlaps the
//                   next jobs.
//   queue           (VT_KERNEL_QUEUE) one persistent launch: a warp takes
//                   16 x 16 pixel units from a device counter, finds its job
//                   by binary search over the jobs' first-unit numbers and
//                   reads the job from global memory.
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

// ---------------------------------------------------------------- tile shape
constexpr int kLaunchJobs = 256;
// A launch holds at most this many 16 x 16 blocks (about 4 Mpixels) unless
// one camera alone is larger: finer launches balance the graph's chains.
constexpr unsigned kLaunchBlocks = 16384;

// Per-job camera fields of a tile-shape launch.
struct JobCam {
    float pos[3];
    float view[16];
    float tan_half_fov;
    int width, height;
    const float4* screen;
    uint4* out;
    unsigned blocks_x;
};

// The parameter block of one k_render_jobs launch: jobs of ONE world.  The
// world and the frame settings the jobs share sit at fixed offsets (read as
// constant-bank operands, as in a single-frame launch: a dynamically indexed
// world measured 12% slower per pixel); only the cameras are indexed.  Job j
// owns the blocks [first_block[j], first_block[j + 1]) of the grid.
struct JobChunk {
    WorldView w;
    FrameParams f;  // shared settings; the camera fields are the job's
    int njobs;
    unsigned first_block[kLaunchJobs + 1];
    JobCam cam[kLaunchJobs];
};
static_assert(sizeof(JobChunk) <= 32764, "a kernel's parameters are limited to 32764 bytes");

// One thread per pixel; the 256-thread block covers a 16 x 16 tile as eight
// 8 x 4 warp tiles (the single-frame kernel's default shape), with the same
// register cap (4 blocks per SM).
template <bool CHECKED>
__global__ void __launch_bounds__(kBatchBlock, 4) k_render_jobs(const __grid_constant__ JobChunk p, unsigned* status) {
    const unsigned b = blockIdx.x;
    int lo = 0, hi = p.njobs - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (p.first_block[mid] <= b) lo = mid;
        else hi = mid - 1;
    }
    const JobCam& jc = p.cam[lo];
    FrameParams f = p.f;
#pragma unroll
    for (int k = 0; k < 3; ++k) f.pos[k] = jc.pos[k];
#pragma unroll
    for (int k = 0; k < 16; ++k) f.view[k] = jc.view[k];
    f.tan_half_fov = jc.tan_half_fov;
    f.width = jc.width;
    f.height = jc.height;
    f.row_end = jc.height;
    f.screen = jc.screen;
    const unsigned local = b - p.first_block[lo];
    const int x0 = (int)(local % jc.blocks_x) * kUnit, y0 = (int)(local / jc.blocks_x) * kUnit;
    // screen coordinates: the frame's table, else once per block
    __shared__ float s_col[3][kUnit], s_row[3][kUnit];
    const bool table = f.screen != nullptr;
    if (!table) {
        if (threadIdx.x < kUnit) {
            s_col[0][threadIdx.x] = ray_u(f, x0 + (int)threadIdx.x);
            s_col[1][threadIdx.x] = centre_u(f, x0 + (int)threadIdx.x);
            s_col[2][threadIdx.x] = vignette_u(s_col[1][threadIdx.x]);
        } else if (threadIdx.x >= 64 && threadIdx.x < 64 + kUnit) {
            s_row[0][threadIdx.x - 64] = ray_v(f, y0 + (int)threadIdx.x - 64);
            s_row[1][threadIdx.x - 64] = centre_v(f, y0 + (int)threadIdx.x - 64);
            s_row[2][threadIdx.x - 64] = vignette_v(s_row[1][threadIdx.x - 64]);
        }
        __syncthreads();
    }
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int lx = (warp & 1) * 8 + (lane & 7), ly = (warp >> 1) * 4 + (lane >> 3);
    const int px = x0 + lx, py = y0 + ly;
    if (px >= f.width || py >= f.height) return;
    PixelUV uv;
    if (table) {
        uv = table_uv(f, px, py);
    } else {
        uv.ru = s_col[0][lx];
        uv.cu = s_col[1][lx];
        uv.gu = s_col[2][lx];
        uv.rv = s_row[0][ly];
        uv.cv = s_row[1][ly];
        uv.gv = s_row[2][ly];
    }
    PixelCounters pc;
    const uint4 rec = render_pixel<false, CHECKED>(p.w, CoarseGlobal{p.w.coarse}, p.w.cdist, f, px, py, uv, status, pc);
    p.cam[lo].out[(size_t)py * f.width + px] = rec;
}

// --------------------------------------------------------------- queue shape
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
    int shape = -1;  // VT_KERNEL_* of the captured graph; -1: the context's tuning at the first launch
    std::vector<const vt_world*> worlds;
    std::vector<vt_job> jobs;
    vt_params params;
    std::vector<vt::JobChunk> chunks;    // tile shape: one launch each
    vt::JobDesc* d_jobs = nullptr;       // queue shape
    unsigned* d_counter = nullptr;
    int njobs = 0;
    unsigned total_units = 0;
    unsigned long long pixels = 0;
    unsigned blocks = 0;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
};

using namespace vt;

namespace {

// Cuts the jobs into launch chunks: consecutive jobs of one world, at most
// kLaunchJobs jobs and (unless one job alone is larger) kLaunchBlocks blocks
// each.  The frames get the context's screen tables (made here if missing: an
// allocation and a synchronisation).
vt_status build_chunks(vt_batch* b) {
    vt_ctx* ctx = b->ctx;
    b->chunks.clear();
    JobChunk* c = nullptr;
    for (size_t i = 0; i < b->jobs.size(); ++i) {
        const vt_job& j = b->jobs[i];
        FrameParams f = make_frame(&j.camera, &b->params);
        vt_status s = screen_table(ctx, f, ctx->stream, true, &f.screen);
        if (s) return s;
        const unsigned long long job_blocks = (unsigned long long)((j.camera.width + kUnit - 1) / kUnit) *
                                              (unsigned long long)((j.camera.height + kUnit - 1) / kUnit);
        if (!c || c->njobs == kLaunchJobs || c->w.mask != j.world->d_mask ||
            (c->njobs > 0 && (unsigned long long)c->first_block[c->njobs] + job_blocks > kLaunchBlocks)) {
            b->chunks.emplace_back();
            c = &b->chunks.back();
            std::memset(c, 0, sizeof(*c));
            c->w = j.world->view();
            c->f = f;
        }
        const int n = c->njobs++;
        JobCam& jc = c->cam[n];
        for (int k = 0; k < 3; ++k) jc.pos[k] = f.pos[k];
        for (int k = 0; k < 16; ++k) jc.view[k] = f.view[k];
        jc.tan_half_fov = f.tan_half_fov;
        jc.width = f.width;
        jc.height = f.height;
        jc.screen = f.screen;
        jc.out = reinterpret_cast<uint4*>(j.d_out);
        jc.blocks_x = (unsigned)((j.camera.width + kUnit - 1) / kUnit);
        const unsigned long long nb =
            (unsigned long long)jc.blocks_x * (unsigned long long)((j.camera.height + kUnit - 1) / kUnit);
        const unsigned long long end = (unsigned long long)c->first_block[n] + nb;
        if (end >= (1ull << 31)) return fail(ctx, VT_ERR_ARG, "batch launch too large (blocks >= 2^31)");
        c->first_block[n + 1] = (unsigned)end;
    }
    return VT_OK;
}

// The graph's launches over kBatchChains chains, longest first, each on the
// chain with the least work so far (weights: blocks or pixels): the chains
// end close together.  Returns (launch index, chain) in issue order.
std::vector<std::pair<size_t, int>> chain_plan(const std::vector<double>& weight) {
    std::vector<size_t> order(weight.size());
    for (size_t i = 0; i < order.size(); ++i) order[i] = i;
    std::stable_sort(order.begin(), order.end(), [&](size_t a, size_t b) { return weight[a] > weight[b]; });
    double load[kBatchChains] = {};
    std::vector<std::pair<size_t, int>> plan;
    plan.reserve(order.size());
    for (size_t i : order) {
        int best = 0;
        for (int k = 1; k < kBatchChains; ++k)
            if (load[k] < load[best]) best = k;
        load[best] += weight[i];
        plan.emplace_back(i, best);
    }
    return plan;
}

}  // namespace

extern "C" {

vt_status vt_batch_create(vt_ctx* ctx, const vt_job* jobs, int32_t n, const vt_params* params, vt_batch** out) {
    if (!ctx) return VT_ERR_ARG;
    if (!jobs || !params || !out || n <= 0) return fail(ctx, VT_ERR_ARG, "bad batch arguments");
    *out = nullptr;
    std::vector<JobDesc> host((size_t)n);
    unsigned long long units = 0, pixels = 0;
    vt_batch* b = new (std::nothrow) vt_batch();
    if (!b) return fail(ctx, VT_ERR_OOM, "host allocation failed");
    b->ctx = ctx;
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
    if ((e = dev_alloc(&b->d_jobs, host.size() * sizeof(JobDesc))) != cudaSuccess ||
        (e = dev_alloc(&b->d_counter, sizeof(unsigned))) != cudaSuccess ||
        (e = cudaMemcpy(b->d_jobs, host.data(), host.size() * sizeof(JobDesc), cudaMemcpyHostToDevice)) != cudaSuccess) {
        vt_batch_destroy(b);
        return check_cuda(ctx, e, "batch upload");
    }
    int per_sm = 0;
    if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_render_batch, kBatchBlock, 0)) != cudaSuccess) {
        vt_batch_destroy(b);
        return check_cuda(ctx, e, "cudaOccupancyMaxActiveBlocksPerMultiprocessor");
    }
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
    const bool checked = (b->params.flags & VT_FLAG_CHECKED) != 0;
    if (!b->exec) {
        if (b->shape < 0) b->shape = ctx->tuning.kernel;
        const int shape = b->shape;
        if (shape == VT_KERNEL_TILE) {
            vt_status s = build_chunks(b);   // before the capture: may make screen tables
            if (s) return s;
        }
        // capture on private streams: the legacy default stream cannot be captured
        cudaStream_t cap = nullptr;
        cudaStream_t chain[kBatchChains] = {};
        cudaEvent_t fork = nullptr, join[kBatchChains] = {};
        cudaError_t e = cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking);
        vt_status s = VT_OK;
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&fork, cudaEventDisableTiming);
        for (int k = 0; k < kBatchChains && e == cudaSuccess; ++k) {
            e = cudaStreamCreateWithFlags(&chain[k], cudaStreamNonBlocking);
            if (e == cudaSuccess) e = cudaEventCreateWithFlags(&join[k], cudaEventDisableTiming);
        }
        if (e == cudaSuccess) e = cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal);
        if (e == cudaSuccess) {
            if (shape == VT_KERNEL_QUEUE) {
                cudaMemsetAsync(b->d_counter, 0, sizeof(unsigned), cap);
                k_render_batch<<<b->blocks, kBatchBlock, 0, cap>>>(b->d_jobs, b->njobs, b->total_units, b->d_counter);
            } else {
                // fork chains off the capture stream, launches longest first on
                // the least loaded chain (chain_plan), join
                cudaEventRecord(fork, cap);
                for (int k = 0; k < kBatchChains; ++k) cudaStreamWaitEvent(chain[k], fork, 0);
                if (shape == VT_KERNEL_TILE) {
                    std::vector<double> wt(b->chunks.size());
                    for (size_t c = 0; c < wt.size(); ++c) wt[c] = b->chunks[c].first_block[b->chunks[c].njobs];
                    for (const auto& pc : chain_plan(wt)) {
                        const JobChunk& ch = b->chunks[pc.first];
                        const unsigned blocks = ch.first_block[ch.njobs];
                        if (checked)
                            k_render_jobs<true><<<blocks, kBatchBlock, 0, chain[pc.second]>>>(ch, ctx->d_status);
                        else
                            k_render_jobs<false><<<blocks, kBatchBlock, 0, chain[pc.second]>>>(ch, nullptr);
                    }
                } else {
                    std::vector<double> wt(b->jobs.size());
                    for (size_t j = 0; j < wt.size(); ++j)
                        wt[j] = (double)b->jobs[j].camera.width * (double)b->jobs[j].camera.height;
                    for (const auto& pc : chain_plan(wt)) {
                        if (s) break;
                        const vt_job& jb = b->jobs[pc.first];
                        s = launch_render(ctx, jb.world, &jb.camera, &b->params, reinterpret_cast<uint4*>(jb.d_out),
                                          chain[pc.second], false);
                    }
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
    if (checked) return note_status_writer(ctx, st);
    return VT_OK;
}

vt_status vt_batch_destroy(vt_batch* b) {
    if (!b) return VT_ERR_ARG;
    cudaDeviceSynchronize();
    if (b->exec) cudaGraphExecDestroy(b->exec);
    if (b->graph) cudaGraphDestroy(b->graph);
    vt::dev_free(b->d_jobs);
    vt::dev_free(b->d_counter);
    delete b;
    return VT_OK;
}

vt_status vt_batch_autotune(vt_batch* b, int32_t reps, int32_t* best_shape, float* best_ms) {
    if (!b) return VT_ERR_ARG;
    vt_ctx* ctx = b->ctx;
    if (reps < 1 || reps > 10000) return fail(ctx, VT_ERR_ARG, "reps must be in [1, 10000]");
    cudaEvent_t e0, e1;
    VT_CUDA(ctx, cudaEventCreate(&e0));
    VT_CUDA(ctx, cudaEventCreate(&e1));
    vt_status s = VT_OK;
    int win = -1;
    float win_ms = 0.0f;
    for (int shape : {VT_KERNEL_TILE, VT_KERNEL_PER_JOB, VT_KERNEL_QUEUE}) {
        // drop the captured graph; the next launch captures this shape
        if (b->exec) cudaGraphExecDestroy(b->exec);
        if (b->graph) cudaGraphDestroy(b->graph);
        b->exec = nullptr;
        b->graph = nullptr;
        b->shape = shape;
        for (int i = 0; i < 2 && !s; ++i) s = vt_batch_launch(b, ctx->stream);
        if (!s) s = check_cuda(ctx, cudaEventRecord(e0, ctx->stream), "cudaEventRecord");
        for (int i = 0; i < reps && !s; ++i) s = vt_batch_launch(b, ctx->stream);
        if (!s) s = check_cuda(ctx, cudaEventRecord(e1, ctx->stream), "cudaEventRecord");
        if (!s) s = check_cuda(ctx, cudaEventSynchronize(e1), "cudaEventSynchronize");
        float ms = 0.0f;
        if (!s) s = check_cuda(ctx, cudaEventElapsedTime(&ms, e0, e1), "cudaEventElapsedTime");
        if (s) break;
        ms /= (float)reps;
        if (win < 0 || ms < win_ms) {
            win = shape;
            win_ms = ms;
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (b->exec) cudaGraphExecDestroy(b->exec);
    if (b->graph) cudaGraphDestroy(b->graph);
    b->exec = nullptr;
    b->graph = nullptr;
    if (s) {
        b->shape = -1;
        return s;
    }
    b->shape = win;  // captured at the next launch
    if (best_shape) *best_shape = win;
    if (best_ms) *best_ms = win_ms;
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
