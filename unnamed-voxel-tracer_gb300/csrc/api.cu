// api.cu -- context, status and device-memory entry points of the C ABI.
#include <atomic>
#include <chrono>
#include <cstdio>
#include <cstring>
#include <string>
#include <thread>

#include "vt_internal.h"

namespace vt {

vt_status fail(vt_ctx* ctx, vt_status s, const std::string& msg, cudaError_t err) {
    if (ctx) {
        ctx->last_error = msg;
        if (err != cudaSuccess) {
            ctx->last_error += ": ";
            ctx->last_error += cudaGetErrorString(err);
        }
    }
    return s;
}

vt_status check_cuda(vt_ctx* ctx, cudaError_t err, const char* what) {
    if (err == cudaSuccess) return VT_OK;
    vt_status s = VT_ERR_CUDA;
    if (err == cudaErrorMemoryAllocation) s = VT_ERR_OOM;
    if (err == cudaErrorNoDevice || err == cudaErrorInsufficientDriver) s = VT_ERR_NO_DEVICE;
    return fail(ctx, s, what, err);
}

namespace {
// The allocation hook: fail_countdown > 0 makes the allocation that brings it
// to 0 fail.  made / live count the library's allocations.
std::atomic<long long> g_fail_countdown{0};
std::atomic<unsigned long long> g_made{0};
std::atomic<long long> g_live{0};

bool hook_fails() {
    long long n = g_fail_countdown.load();
    while (n > 0) {
        if (g_fail_countdown.compare_exchange_weak(n, n - 1)) return n == 1;
    }
    return false;
}
}  // namespace

cudaError_t dev_alloc_raw(void** p, size_t bytes) {
    *p = nullptr;
    if (hook_fails()) return cudaErrorMemoryAllocation;
    const cudaError_t e = cudaMalloc(p, bytes);
    if (e == cudaSuccess) {
        g_made++;
        g_live++;
    }
    return e;
}

cudaError_t host_alloc_raw(void** p, size_t bytes) {
    *p = nullptr;
    if (hook_fails()) return cudaErrorMemoryAllocation;
    const cudaError_t e = cudaHostAlloc(p, bytes, cudaHostAllocDefault);
    if (e == cudaSuccess) {
        g_made++;
        g_live++;
    }
    return e;
}

cudaError_t dev_free(void* p) {
    if (!p) return cudaSuccess;
    const cudaError_t e = cudaFree(p);
    if (e == cudaSuccess) g_live--;
    return e;
}

cudaError_t host_free(void* p) {
    if (!p) return cudaSuccess;
    const cudaError_t e = cudaFreeHost(p);
    if (e == cudaSuccess) g_live--;
    return e;
}

vt_status l2_policy(vt_ctx* ctx, const vt_world* world, cudaAccessPolicyWindow* storage,
                    const cudaAccessPolicyWindow** out) {
    *out = nullptr;
    if (!ctx->tuning.l2_persist) return VT_OK;
    if (!ctx->l2_setaside) {
        int maxp = 0, maxw = 0;
        VT_CUDA(ctx, cudaDeviceGetAttribute(&maxp, cudaDevAttrMaxPersistingL2CacheSize, ctx->device));
        VT_CUDA(ctx, cudaDeviceGetAttribute(&maxw, cudaDevAttrMaxAccessPolicyWindowSize, ctx->device));
        ctx->l2_persist_max = (size_t)(maxp > 0 ? maxp : 0);
        ctx->l2_window_max = (size_t)(maxw > 0 ? maxw : 0);
        if (ctx->l2_persist_max) VT_CUDA(ctx, cudaDeviceSetLimit(cudaLimitPersistingL2CacheSize, ctx->l2_persist_max));
        ctx->l2_setaside = true;
    }
    if (!ctx->l2_persist_max || !ctx->l2_window_max) return VT_OK;
    const size_t words = world->nchunks * (size_t)kBricksPerChunk * 8u;
    const size_t bytes = words < ctx->l2_window_max ? words : ctx->l2_window_max;
    *storage = cudaAccessPolicyWindow{};
    storage->base_ptr = world->d_mask;
    storage->num_bytes = bytes;
    storage->hitRatio = bytes <= ctx->l2_persist_max ? 1.0f : (float)ctx->l2_persist_max / (float)bytes;
    storage->hitProp = cudaAccessPropertyPersisting;
    storage->missProp = cudaAccessPropertyStreaming;
    *out = storage;
    return VT_OK;
}

vt_status take_status(vt_ctx* ctx, unsigned st) {
    if (!st) return VT_OK;
    VT_CUDA(ctx, cudaMemset(ctx->d_status, 0, sizeof(unsigned)));
    return fail(ctx, VT_ERR_DEVICE_OOB, "a checked kernel saw an out-of-range index");
}

vt_status note_status_writer(vt_ctx* ctx, cudaStream_t st) {
    // Inside a stream capture nothing runs yet; the graph's launch notes it.
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    VT_CUDA(ctx, cudaStreamIsCapturing(st, &cs));
    if (cs != cudaStreamCaptureStatusNone) return VT_OK;
    // ev_status must complete only after every launch that may have set the
    // word since it was last read: while an earlier writer may be pending (on
    // any stream), this stream first waits for the event that covers it, so
    // the new record covers both.  (Without the wait, a vt_sync on a stream
    // whose writer ended early could declare the word clean while a longer
    // writer on another stream is still to set it.)
    if (ctx->status_dirty) VT_CUDA(ctx, cudaStreamWaitEvent(st, ctx->ev_status, 0));
    ctx->status_dirty = true;
    VT_CUDA(ctx, cudaEventRecord(ctx->ev_status, st));
    return VT_OK;
}

vt_status ctx_scratch(vt_ctx* ctx, size_t bytes, void** out) {
    if (bytes > ctx->scratch_bytes) {
        if (ctx->d_scratch) {
            VT_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
            dev_free(ctx->d_scratch);
            ctx->d_scratch = nullptr;
            ctx->scratch_bytes = 0;
        }
        VT_CUDA(ctx, dev_alloc(&ctx->d_scratch, bytes));
        ctx->scratch_bytes = bytes;
    }
    *out = ctx->d_scratch;
    return VT_OK;
}

}  // namespace vt

using namespace vt;

extern "C" {

int32_t vt_abi_version(void) { return VT_ABI_VERSION; }

const char* vt_status_string(vt_status s) {
    switch (s) {
        case VT_OK: return "ok";
        case VT_ERR_ARG: return "invalid argument";
        case VT_ERR_OOM: return "out of memory";
        case VT_ERR_CUDA: return "CUDA error";
        case VT_ERR_DEVICE_OOB: return "device index out of range";
        case VT_ERR_TIMEOUT: return "wait timed out";
        case VT_ERR_NO_DEVICE: return "no CUDA device";
        case VT_ERR_FORMAT: return "malformed input";
        case VT_ERR_STATE: return "invalid state";
        default: return "unknown status";
    }
}

vt_status vt_ctx_create(int32_t device, vt_ctx** out) {
    if (!out) return VT_ERR_ARG;
    *out = nullptr;
    int count = 0;
    cudaError_t e = cudaGetDeviceCount(&count);
    if (e != cudaSuccess || count == 0) return VT_ERR_NO_DEVICE;
    if (device < 0 || device >= count) return VT_ERR_ARG;
    vt_ctx* ctx = new (std::nothrow) vt_ctx();
    if (!ctx) return VT_ERR_OOM;
    ctx->device = device;
    vt_status s = VT_OK;
    do {
        if ((e = cudaSetDevice(device)) != cudaSuccess) { s = check_cuda(ctx, e, "cudaSetDevice"); break; }
        cudaDeviceProp prop;
        if ((e = cudaGetDeviceProperties(&prop, device)) != cudaSuccess) { s = check_cuda(ctx, e, "cudaGetDeviceProperties"); break; }
        std::snprintf(ctx->name, sizeof(ctx->name), "%s", prop.name);
        ctx->sm_count = prop.multiProcessorCount;
        if ((e = dev_alloc(&ctx->d_status, sizeof(unsigned))) != cudaSuccess) { s = check_cuda(ctx, e, "cudaMalloc"); break; }
        if ((e = cudaMemset(ctx->d_status, 0, sizeof(unsigned))) != cudaSuccess) { s = check_cuda(ctx, e, "cudaMemset"); break; }
        if ((e = dev_alloc(&ctx->d_counters, kNumCounters * sizeof(unsigned long long))) != cudaSuccess) { s = check_cuda(ctx, e, "cudaMalloc"); break; }
        if ((e = dev_alloc(&ctx->d_work, kWorkSlots * sizeof(unsigned))) != cudaSuccess) { s = check_cuda(ctx, e, "cudaMalloc"); break; }
        if ((e = host_alloc(&ctx->h_status, sizeof(unsigned))) != cudaSuccess) { s = check_cuda(ctx, e, "cudaHostAlloc"); break; }
        *ctx->h_status = 0;
        if ((e = cudaEventCreateWithFlags(&ctx->ev_status, cudaEventDisableTiming)) != cudaSuccess) { s = check_cuda(ctx, e, "cudaEventCreate"); break; }
        // blocking stream: *_host calls order after work queued on the legacy default stream
        if ((e = cudaStreamCreateWithFlags(&ctx->stream, cudaStreamDefault)) != cudaSuccess) { s = check_cuda(ctx, e, "cudaStreamCreate"); break; }
        // the device address of vt_render_host_static's fixed array, looked up
        // here so that the entry point itself never loads a module
        if ((s = static_staging_init(ctx)) != VT_OK) break;
    } while (0);
    if (s != VT_OK) {
        vt_ctx_destroy(ctx);
        return s;
    }
    *out = ctx;
    return VT_OK;
}

vt_status vt_ctx_destroy(vt_ctx* ctx) {
    if (!ctx) return VT_ERR_ARG;
    cudaSetDevice(ctx->device);
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    if (ctx->copy_stream) cudaStreamSynchronize(ctx->copy_stream);
    if (ctx->l2_setaside) {
        cudaDeviceSynchronize();
        cudaCtxResetPersistingL2Cache();
        cudaDeviceSetLimit(cudaLimitPersistingL2CacheSize, 0);
    }
    for (int i = 0; i < kBandStreams; ++i)
        if (ctx->band_stream[i]) {
            cudaStreamSynchronize(ctx->band_stream[i]);
            cudaStreamDestroy(ctx->band_stream[i]);
        }
    if (ctx->copy_stream) cudaStreamDestroy(ctx->copy_stream);
    if (ctx->ev_start) cudaEventDestroy(ctx->ev_start);
    if (ctx->h_status) host_free(ctx->h_status);
    if (ctx->ev_status) cudaEventDestroy(ctx->ev_status);
    dev_free(ctx->d_bounce_jobs);
    dev_free(ctx->d_bounce_open);
    dev_free(ctx->d_bounce_ctr);
    if (ctx->ev_bounce) cudaEventDestroy(ctx->ev_bounce);
    for (int i = 0; i < ctx->n_screen; ++i) dev_free(ctx->screen[i].d);
    for (int i = 0; i < kMaxBands; ++i)
        if (ctx->ev_band[i]) cudaEventDestroy(ctx->ev_band[i]);
    dev_free(ctx->d_scratch);
    dev_free(ctx->d_status);
    dev_free(ctx->d_counters);
    dev_free(ctx->d_work);
    if (ctx->stream) cudaStreamDestroy(ctx->stream);
    delete ctx;
    return VT_OK;
}

const char* vt_last_error_string(const vt_ctx* ctx) { return ctx ? ctx->last_error.c_str() : "null context"; }

vt_status vt_sync(vt_ctx* ctx, vt_stream stream) {
    if (!ctx) return VT_ERR_ARG;
    const cudaStream_t st = (cudaStream_t)stream;
    if (!ctx->status_dirty) {
        // no launch since the last read can have set the word
        VT_CUDA(ctx, cudaStreamSynchronize(st));
        return VT_OK;
    }
    // the read sees every status-setting launch so far if they were all done
    // before it was issued; only then is the word clean afterwards
    const cudaError_t q = cudaEventQuery(ctx->ev_status);
    if (q == cudaErrorNotReady) {
        const cudaError_t le = cudaGetLastError();  // a pending query result is no error
        if (le != cudaSuccess && le != cudaErrorNotReady) return check_cuda(ctx, le, "cudaEventQuery");
    } else if (q != cudaSuccess) {
        return check_cuda(ctx, q, "cudaEventQuery");
    }
    // the status word travels on the same stream: one synchronisation
    VT_CUDA(ctx, cudaMemcpyAsync(ctx->h_status, ctx->d_status, sizeof(unsigned), cudaMemcpyDeviceToHost, st));
    VT_CUDA(ctx, cudaStreamSynchronize(st));
    if (q == cudaSuccess) ctx->status_dirty = false;
    return take_status(ctx, *ctx->h_status);
}

vt_status vt_wait(vt_ctx* ctx, vt_stream stream, int64_t timeout_us) {
    if (!ctx || timeout_us < 0) return VT_ERR_ARG;
    const cudaStream_t st = (cudaStream_t)stream;
    const auto deadline = std::chrono::steady_clock::now() + std::chrono::microseconds(timeout_us);
    for (;;) {
        const cudaError_t q = cudaStreamQuery(st);
        if (q == cudaSuccess) return vt_sync(ctx, stream);
        if (q != cudaErrorNotReady) return check_cuda(ctx, q, "cudaStreamQuery");
        cudaGetLastError();  // a pending stream is no error
        if (std::chrono::steady_clock::now() >= deadline)
            return fail(ctx, VT_ERR_TIMEOUT,
                        "stream still busy after " + std::to_string((long long)timeout_us) + " us");
        std::this_thread::sleep_for(std::chrono::microseconds(20));
    }
}

vt_status vt_device_info(vt_ctx* ctx, char* name, int32_t name_len, int32_t* sm_count) {
    if (!ctx) return VT_ERR_ARG;
    if (name && name_len > 0) std::snprintf(name, (size_t)name_len, "%s", ctx->name);
    if (sm_count) *sm_count = ctx->sm_count;
    return VT_OK;
}

vt_status vt_device_alloc(vt_ctx* ctx, size_t nbytes, void** d_ptr) {
    if (!ctx || !d_ptr) return VT_ERR_ARG;
    *d_ptr = nullptr;
    VT_CUDA(ctx, dev_alloc(d_ptr, nbytes ? nbytes : 1));
    return VT_OK;
}

vt_status vt_device_free(vt_ctx* ctx, void* d_ptr) {
    if (!ctx) return VT_ERR_ARG;
    VT_CUDA(ctx, dev_free(d_ptr));
    return VT_OK;
}

vt_status vt_host_alloc_pinned(vt_ctx* ctx, size_t nbytes, void** h_ptr) {
    if (!ctx || !h_ptr) return VT_ERR_ARG;
    *h_ptr = nullptr;
    VT_CUDA(ctx, host_alloc(h_ptr, nbytes ? nbytes : 1));
    return VT_OK;
}

vt_status vt_host_free_pinned(vt_ctx* ctx, void* h_ptr) {
    if (!ctx) return VT_ERR_ARG;
    VT_CUDA(ctx, host_free(h_ptr));
    return VT_OK;
}

vt_status vt_memcpy_h2d(vt_ctx* ctx, void* d_dst, const void* h_src, size_t nbytes, vt_stream stream) {
    if (!ctx || (nbytes && (!d_dst || !h_src))) return VT_ERR_ARG;
    VT_CUDA(ctx, cudaMemcpyAsync(d_dst, h_src, nbytes, cudaMemcpyHostToDevice, (cudaStream_t)stream));
    return VT_OK;
}

vt_status vt_memcpy_d2h(vt_ctx* ctx, void* h_dst, const void* d_src, size_t nbytes, vt_stream stream) {
    if (!ctx || (nbytes && (!d_src || !h_dst))) return VT_ERR_ARG;
    VT_CUDA(ctx, cudaMemcpyAsync(h_dst, d_src, nbytes, cudaMemcpyDeviceToHost, (cudaStream_t)stream));
    return VT_OK;
}

vt_status vt_memset_d(vt_ctx* ctx, void* d_dst, int32_t value, size_t nbytes, vt_stream stream) {
    if (!ctx || (nbytes && !d_dst)) return VT_ERR_ARG;
    VT_CUDA(ctx, cudaMemsetAsync(d_dst, value, nbytes, (cudaStream_t)stream));
    return VT_OK;
}

vt_status vt_stream_create(vt_ctx* ctx, vt_stream* out) {
    if (!ctx || !out) return VT_ERR_ARG;
    cudaStream_t s = nullptr;
    VT_CUDA(ctx, cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
    *out = (vt_stream)s;
    return VT_OK;
}

vt_status vt_stream_destroy(vt_ctx* ctx, vt_stream stream) {
    if (!ctx) return VT_ERR_ARG;
    VT_CUDA(ctx, cudaStreamDestroy((cudaStream_t)stream));
    return VT_OK;
}

void vt_debug_fail_alloc(int64_t n) { g_fail_countdown.store(n > 0 ? (long long)n : 0); }

void vt_debug_alloc_counts(uint64_t* made, int64_t* live) {
    if (made) *made = g_made.load();
    if (live) *live = g_live.load();
}

}  // extern "C"
