// bounce.cuh -- bounce rays traced apart from the frame kernel.
//
// Cosine-distributed bounce rays (rng.glsl:41-55) are incoherent: within a
// warp of neighbouring pixels their lengths differ by an order of magnitude,
// so a warp tracing one per lane runs for its longest ray while most lanes
// wait (a step-sequence simulation of a terrain frame puts the useful work at
// a third of the issued work).  With deferral the frame kernel only appends
// each hit's bounce ray (origin, direction, pixel) to a queue; a persistent
// kernel traces the queue with per-lane refill (a lane whose ray ended takes
// the next queued ray as soon as a quarter of the warp is idle), and a third
// kernel shades the deferred pixels.  Every ray is walked by the same code as
// before and the records are identical.  On a 4K frame of the 1 GiB cave
// world the bounce rays' share of the frame fell from 1.49 to 1.08 ms.
#pragma once

#include "shade.cuh"

namespace vt {

struct BounceJob {
    float o[3];
    float d[3];
    unsigned pixel;
    unsigned tag;  // the frame number in per-thread slots (FrameParams::bounce_tag), else unused
};
static_assert(sizeof(BounceJob) == 32, "bounce job layout");

// Appends one bounce ray; called by the lanes of a warp that have one, with
// the warp possibly diverged (one atomic per converged group).  With a frame
// tag the ray goes to the calling thread's own slot instead (its index in
// the launch grid, so that slot order is image-tile order), tagged.
__device__ __forceinline__ void append_bounce(const FrameParams& f, const float o[3], const float d[3],
                                              unsigned pixel) {
    if (f.bounce_tag) {
        const size_t slot = ((size_t)blockIdx.y * gridDim.x + blockIdx.x) * blockDim.x + threadIdx.x;
        BounceJob* j = reinterpret_cast<BounceJob*>(f.bounce_jobs) + slot;
        j->o[0] = o[0];
        j->o[1] = o[1];
        j->o[2] = o[2];
        j->d[0] = d[0];
        j->d[1] = d[1];
        j->d[2] = d[2];
        j->pixel = pixel;
        j->tag = f.bounce_tag;
        return;
    }
    const unsigned act = __activemask();
    const unsigned lane = threadIdx.x & 31u;
    const int leader = __ffs(act) - 1;
    unsigned base = 0;
    if ((int)lane == leader) base = atomicAdd(f.bounce_count, (unsigned)__popc(act));
    base = __shfl_sync(act, base, leader);
    const unsigned slot = base + (unsigned)__popc(act & ((1u << lane) - 1u));
    BounceJob* j = reinterpret_cast<BounceJob*>(f.bounce_jobs) + slot;
    j->o[0] = o[0];
    j->o[1] = o[1];
    j->o[2] = o[2];
    j->d[0] = d[0];
    j->d[1] = d[1];
    j->d[2] = d[2];
    j->pixel = pixel;
}

}  // namespace vt
