// bounce.cu -- the deferred bounce pass (see bounce.cuh): a persistent
// kernel that traces the queued bounce rays with per-lane refill, and a kernel
// that shades the pixels whose bounce ray was deferred.
#include "bounce.cuh"
#include "launch.cuh"
#include "trace_p.cuh"

namespace vt {

namespace {

constexpr int kBounceBlock = 256;
// a warp takes new rays from the queue once this many of its lanes are idle
// (tuning bounce_refill; 1, 4, 8, 16, 24 measured on a 4K cave-world frame
// with the brick-run walk: 8 is fastest)
constexpr int kRefill = 8;
// walk iterations a busy lane makes between two refill checks (1, 2, 3, 4, 8
// measured on the same frame: 2 and 3 are fastest, 4% less bounce time than 1)
constexpr int kActions = 2;

// Persistent: every warp loops until the queue is drained.  A lane walks one
// ray at a time, kActions iterations of the walk per loop turn; open[j] receives 1
// when ray j leaves without a hit (the sky lights its pixel), 0 otherwise.
// FLAT: walk with Walker::step_flat (one code path for jumps and unit steps)
// instead of Walker::step.
template <bool FLAT>
__global__ void __launch_bounds__(kBounceBlock) k_bounce_trace(WorldView w, const BounceJob* __restrict__ jobs,
                                                               const unsigned* __restrict__ counters,
                                                               unsigned* __restrict__ next, unsigned char* open,
                                                               int max_steps, int refill) {
    const unsigned total = counters[0];
    const unsigned lane = threadIdx.x & 31u;
    const unsigned below = (1u << lane) - 1u;
    Walker wk;
    bool busy = false;
    unsigned job = 0;
    for (;;) {
        const unsigned idle = __ballot_sync(0xFFFFFFFFu, !busy);
        if (idle == 0xFFFFFFFFu || __popc(idle) >= refill) {
            unsigned base = 0;
            if (lane == 0) base = atomicAdd(next, (unsigned)__popc(idle));
            base = __shfl_sync(0xFFFFFFFFu, base, 0);
            if (base >= total && idle == 0xFFFFFFFFu) break;  // drained, and nothing in flight
            if (!busy) {
                job = base + (unsigned)__popc(idle & below);
                if (job < total) {
                    const BounceJob J = jobs[job];
                    busy = wk.start(w, J.o, J.d, max_steps);
                    if (!busy) open[job] = 1;  // misses the grid or may take no step
                }
            }
        }
        if (busy) {
            TraceHit h;
            int s = Walker::kMore;
            for (int a = 0; a < kActions && s == Walker::kMore; ++a)
                s = FLAT ? wk.step_flat<true>(w, w.cdist, h) : wk.step<false, true, true>(w, w.cdist, h);
            if (s != Walker::kMore) {
                open[job] = s == Walker::kHit ? 0 : 1;
                busy = false;
            }
        }
    }
}

// One thread per deferred pixel: the shading render_pixel would have done with
// this bounce result, and the record's rgba and VT_HIT_BOUNCE flag.
__global__ void __launch_bounds__(kBounceBlock) k_bounce_finish(WorldView w, FrameParams f,
                                                                const BounceJob* __restrict__ jobs,
                                                                const unsigned* __restrict__ counters,
                                                                const unsigned char* __restrict__ open,
                                                                uint4* __restrict__ out) {
    const unsigned total = counters[0];
    for (unsigned j = blockIdx.x * blockDim.x + threadIdx.x; j < total; j += gridDim.x * blockDim.x) {
        const BounceJob J = jobs[j];
        const unsigned p = J.pixel;
        const int px = (int)(p % (unsigned)f.width), py = (int)(p / (unsigned)f.width);
        const PixelUV uv = f.screen ? table_uv(f, px, py) : pixel_uv(f, px, py);
        uint4 r = out[p];
        const unsigned face = r.w & 0xFFu, mat = (r.w >> 8) & 0xFFu;
        unsigned flags = (r.w >> 16) & 0xFFu;
        const bool shadowed = (flags & (VT_HIT_SHADOWED | VT_HIT_ENTITY)) != 0u;
        const bool bounce_open = open[j] != 0;
        if (!bounce_open) flags |= VT_HIT_BOUNCE;
        const unsigned alb = __ldg(w.palette + mat);
        float col[4];
        shade_hit(f, alb, (int)(face >> 1), (face & 1u) == 0u, shadowed, bounce_open, J.d, col);
        r.z = f.shade == VT_SHADE_NONE ? alb : composite_uv(f, uv, col);
        r.w = face | (mat << 8) | (flags << 16);
        out[p] = r;
    }
}

}  // namespace

vt_status bounce_buffers(vt_ctx* ctx, size_t pixels) {
    if (pixels <= ctx->bounce_capacity) return VT_OK;
    VT_CUDA(ctx, cudaDeviceSynchronize());
    if (ctx->d_bounce_jobs) vt::dev_free(ctx->d_bounce_jobs);
    if (ctx->d_bounce_open) vt::dev_free(ctx->d_bounce_open);
    ctx->d_bounce_jobs = nullptr;
    ctx->d_bounce_open = nullptr;
    ctx->bounce_capacity = 0;
    VT_CUDA(ctx, vt::dev_alloc(&ctx->d_bounce_jobs, pixels * sizeof(BounceJob)));
    VT_CUDA(ctx, vt::dev_alloc(&ctx->d_bounce_open, pixels));
    if (!ctx->d_bounce_ctr) VT_CUDA(ctx, vt::dev_alloc(&ctx->d_bounce_ctr, 2 * sizeof(unsigned)));
    if (!ctx->ev_bounce) VT_CUDA(ctx, cudaEventCreateWithFlags(&ctx->ev_bounce, cudaEventDisableTiming));
    ctx->bounce_capacity = pixels;
    return VT_OK;
}

vt_status launch_bounce(vt_ctx* ctx, const vt_world* world, const FrameParams& f, uint4* d_out, cudaStream_t st) {
    const WorldView w = world->view();
    const int flat = ctx->tuning.bounce_walk == 1 ? 1 : 0;
    const int refill = ctx->tuning.bounce_refill > 0 ? ctx->tuning.bounce_refill : kRefill;
    if (ctx->bounce_blocks[flat] == 0) {
        int nb = 0;
        if (flat) VT_CUDA(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_bounce_trace<true>, kBounceBlock, 0));
        else VT_CUDA(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_bounce_trace<false>, kBounceBlock, 0));
        ctx->bounce_blocks[flat] = ctx->sm_count * (nb > 0 ? nb : 1);
    }
    const BounceJob* jobs = reinterpret_cast<const BounceJob*>(ctx->d_bounce_jobs);
    cudaAccessPolicyWindow win_storage;
    const cudaAccessPolicyWindow* win = nullptr;  // L2 window over the brick words (tuning l2_persist)
    vt_status s = l2_policy(ctx, world, &win_storage, &win);
    if (s) return s;
    if (flat)
        VT_CUDA(ctx, launch_kernel(k_bounce_trace<true>, dim3(ctx->bounce_blocks[1]), dim3(kBounceBlock), 0, st, win, w,
                                   jobs, (const unsigned*)ctx->d_bounce_ctr, ctx->d_bounce_ctr + 1, ctx->d_bounce_open,
                                   f.bounce_max_steps, refill));
    else
        VT_CUDA(ctx, launch_kernel(k_bounce_trace<false>, dim3(ctx->bounce_blocks[0]), dim3(kBounceBlock), 0, st, win, w,
                                   jobs, (const unsigned*)ctx->d_bounce_ctr, ctx->d_bounce_ctr + 1, ctx->d_bounce_open,
                                   f.bounce_max_steps, refill));
    k_bounce_finish<<<ctx->sm_count * 8, kBounceBlock, 0, st>>>(w, f, jobs, ctx->d_bounce_ctr, ctx->d_bounce_open,
                                                                d_out);
    VT_CUDA(ctx, cudaGetLastError());
    // the next deferred frame of this context reuses the queue after this one
    VT_CUDA(ctx, cudaEventRecord(ctx->ev_bounce, st));
    return VT_OK;
}

}  // namespace vt
