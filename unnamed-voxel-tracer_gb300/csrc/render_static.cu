// render_static.cu -- a render-to-host entry point that allocates no device
// memory.
//
// vt_render_host stages a frame's records in a device buffer that the context
// allocates with cudaMalloc on first use (and again when a larger frame comes).
// Some callers cannot allow that: hosts that hand out all device memory
// through their own allocator and forbid other allocations, and real-time
// frame loops that must not call cudaMalloc once they run, because it can
// synchronize the whole device and stall the frame.  vt_render_host_static
// runs the same render kernel but stages the records in a fixed array
// compiled into this library, so the call itself allocates nothing.
#include <mutex>
#include <string>

#include "vt_internal.h"

namespace {

// Staging for the records of one frame (16 bytes per pixel, 4 MiB).  The
// array is placed on a device when the first context for that device is
// created (vt_ctx_create looks its address up; under CUDA's lazy module
// loading that is when the driver loads it) and stays until the process
// exits.  All calls share it: a call overwrites every record it copies out,
// so nothing needs clearing, but calls whose kernels overlap on the GPU race.
static __device__ __align__(256) uint4 g_static_records[VT_STATIC_MAX_PIXELS];

constexpr int kMaxDevices = 64;
std::mutex g_mutex;
void* g_records[kMaxDevices] = {};  // device address of g_static_records, per device

// The address looked up by static_staging_init, or null.
void* static_records(int device) {
    if (device < 0 || device >= kMaxDevices) return nullptr;
    std::lock_guard<std::mutex> lock(g_mutex);
    return g_records[device];
}

}  // namespace

// In host code the array's name is a host-side stand-in, not a device
// address; the address is looked up once per device, with that device
// current (vt_ctx_create makes it current before calling this).
vt_status vt::static_staging_init(vt_ctx* ctx) {
    if (ctx->device < 0 || ctx->device >= kMaxDevices)
        return vt::fail(ctx, VT_ERR_ARG, "device ordinal beyond the static staging table");
    std::lock_guard<std::mutex> lock(g_mutex);
    if (!g_records[ctx->device]) {
        int cur = -1;
        VT_CUDA(ctx, cudaGetDevice(&cur));
        if (cur != ctx->device) return vt::fail(ctx, VT_ERR_STATE, "static staging looked up off its device");
        void* p = nullptr;
        VT_CUDA(ctx, cudaGetSymbolAddress(&p, g_static_records));
        g_records[ctx->device] = p;
    }
    return VT_OK;
}

extern "C" vt_status vt_render_host_static(vt_ctx* ctx, const vt_world* world, const vt_camera* cam,
                                           const vt_params* params, vt_hit* h_out) {
    vt_status s = vt::check_frame_args(ctx, world, cam, params);
    if (s) return s;
    if (!h_out) return vt::fail(ctx, VT_ERR_ARG, "null output buffer");
    const unsigned long long pixels = (unsigned long long)cam->width * (unsigned long long)cam->height;
    if (pixels > VT_STATIC_MAX_PIXELS)
        return vt::fail(ctx, VT_ERR_ARG,
                        "frame of " + std::to_string(pixels) + " pixels exceeds the static staging buffer of " +
                            std::to_string(VT_STATIC_MAX_PIXELS) + " pixels (VT_STATIC_MAX_PIXELS); use vt_render_host");
    void* d = static_records(ctx->device);
    if (!d) return vt::fail(ctx, VT_ERR_STATE, "static staging array not placed on this device");
    s = vt::launch_render(ctx, world, cam, params, reinterpret_cast<uint4*>(d), ctx->stream, false, 0, -1, false,
                          false);  // no allocation: an existing screen table only
    if (s) return s;
    VT_CUDA(ctx, cudaMemcpyAsync(h_out, d, (size_t)pixels * sizeof(vt_hit), cudaMemcpyDeviceToHost, ctx->stream));
    return vt_sync(ctx, ctx->stream);
}
