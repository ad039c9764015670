// vt_internal.h -- private structures of libvt (not part of the C ABI).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>

#include "../../include/vt.h"

namespace vt {

constexpr int kChunk = 32;          // chunk edge in voxels
constexpr int kBrick = 4;           // brick edge in voxels
constexpr int kBricksPerChunk = 512;
constexpr int kChunkBytes = kChunk * kChunk * kChunk;

// Error bit of the device status word (the checked kernels' index checks).
constexpr unsigned kStatusOob = 1u;

// Device counters written by the instrumented kernels (order = vt_stats).
constexpr int kNumCounters = 12;

// Everything a traversal kernel needs to read a mode-P world.
struct WorldView {
    const unsigned long long* mask;     // brick occupancy words, chunk-major
    const unsigned char* mats;          // 64 material bytes per brick, same order
    const unsigned long long* coarse;   // one bit per chunk
    const unsigned* palette;            // 256 RGBA8
    const unsigned char* bdist;         // kOctants fields of nwords bytes (octant-major), per brick:
                                        // 0 if occupied, else (E + 1) | shape << 6: the brick plus E
                                        // voxel layers ahead in that octant (E >> shape vertically)
                                        // is empty (below)
    const unsigned char* cdist;         // kOctants fields of cstride bytes, per chunk: same, in chunks
    const float* entities;              // n_entities boxes {lo x, y, z, hi x, y, z}: shadow occluders
    int n_entities;
    int dims[3];
    int cdim[3];                        // chunk counts
    unsigned nwords;                    // number of brick words
    unsigned ncoarse;                   // number of coarse words
    unsigned nchunks;
    unsigned cstride;                   // bytes per chunk-distance field (nchunks rounded up to 16)
};

// Cap of the chunk distances: a stored value d >= 1 promises that every
// chunk within radius d - 1 ahead is empty.
constexpr int kDistCap = 15;
// Cap of the brick distances, counted in voxel layers: a stored value with
// low six bits s >= 1 promises that the brick plus s - 1 voxel layers beyond
// its far faces (fewer vertically, see kBoxShapes) holds no occupied voxel.
// Counting in voxels rather than whole bricks lets a jump out of an empty
// brick end inside the next occupied brick, at the first layer that can hold
// a voxel: 32% fewer voxel tests for the primary rays of the 1080p terrain
// frames.
constexpr int kVoxCap = 62;
// Distances are kept per direction octant.  Field o (bit i set: the ray moves
// towards +i) of a chunk c holds min over occupied chunks c' with
// sign(c'_i - c_i) in {0, that direction} of max(|dx|, |dy|, |dz|); field o of
// a brick holds the same over occupied voxels, in voxel layers beyond the
// brick's far faces, with the vertical weight below: it looks only where a
// ray of that octant can go.  A ray leaving a cell moves away from it on
// every axis, so the empty box it may jump through only has to extend
// forwards; rays that leave the terrain (shadow rays toward the sun,
// primary rays above the ground) see the open space in front of them instead
// of the terrain they came from.
constexpr int kOctants = 8;
__host__ __device__ inline unsigned cdist_stride(unsigned nchunks) { return (nchunks + 15u) / 16u * 16u; }
// The brick field of an octant whose rays move down (-y) picks, per brick, the
// shape of its empty box: vertical weight w = 2^shape, shape 0..3, s = min
// over occupied voxels of max(dx, w*dy, dz), a box of s-1 layers across and
// (s-1)/w up and down.  Flat boxes suit rays that descend towards terrain and
// skim it, tall ones rays that fall steeply past an overhang; each brick keeps
// the shape whose box is largest (box_score), the smallest weight wins a tie.  Per
// brick rather than one weight for all: 7% fewer brick jumps and 5% fewer
// walk calls for the primary rays of the 1080p terrain frames than the best
// single weight (4).  The octants of rays that move up (away from the ground:
// shadow rays towards a sun above the horizon) use plain Chebyshev (shape 0;
// other shapes gain them nothing), as does the chunk distance.
constexpr int kBoxShapes = 4;
// Volume of the box a distance s gives with vertical weight 2^shape, in
// voxels, the brick included.
__host__ __device__ constexpr int box_score(int s, int shape) {
    return (s + 3) * (s + 3) * (((s - 1) >> shape) + 4);
}
// Capacity of a world's entity box list.
constexpr int kMaxEntities = 1024;
// Largest image width and height a frame may have.
constexpr int kMaxImageSide = 32768;

}  // namespace vt

namespace vt {
// The screen coordinates of one image size and field of view: a float4 per
// column {ray u, centre u, vignette column factor, 0} followed by one per row
// {ray v, centre v, vignette row factor, 0}.  Written once, then only read
// (frames on other streams may be reading it), freed with the context.
struct ScreenTable {
    int width = 0, height = 0;
    float tan_half_fov = 0.0f;
    float4* d = nullptr;
};
constexpr int kScreenTables = 8;
}  // namespace vt

struct vt_ctx {
    int device = 0;
    int sm_count = 0;
    char name[256] = {0};
    std::string last_error;
    unsigned* d_status = nullptr;                // device status word
    unsigned long long* d_counters = nullptr;    // vt::kNumCounters
    cudaStream_t stream = nullptr;               // stream of the *_host entry points
    void* d_scratch = nullptr;                   // output staging of the *_host entry points
    size_t scratch_bytes = 0;
    unsigned* d_work = nullptr;                  // ring of pixel-queue counters of the persistent kernels
    unsigned work_slot = 0;
    int persist_blocks = 0;                      // resident blocks per SM of the persistent render kernel
    vt_tuning tuning = {VT_KERNEL_TILE, 8, 1, 16, 0, 0, 0, 0, 0};
    // the persisting-L2 set-aside has been requested (VT tuning l2_persist)
    bool l2_setaside = false;
    size_t l2_persist_max = 0;     // cudaDevAttrMaxPersistingL2CacheSize
    size_t l2_window_max = 0;      // cudaDevAttrMaxAccessPolicyWindowSize
    // vt_render_host's pipeline: row bands rendered on band streams, each
    // copied to the host on the copy stream as soon as it is done (created on
    // first use)
    cudaStream_t band_stream[4] = {nullptr, nullptr, nullptr, nullptr};
    cudaStream_t copy_stream = nullptr;
    cudaEvent_t ev_start = nullptr;
    cudaEvent_t ev_band[16] = {};
    unsigned* h_status = nullptr;  // pinned copy of d_status
    // launches that may set d_status (checked and instrumented kernels) mark
    // it dirty and record ev_status; while it is clean vt_sync need not read it
    bool status_dirty = false;
    cudaEvent_t ev_status = nullptr;
    // the deferred bounce pass (bounce.cu): ray queue, results, counters
    void* d_bounce_jobs = nullptr;
    unsigned char* d_bounce_open = nullptr;
    unsigned* d_bounce_ctr = nullptr;  // {queued, taken}
    size_t bounce_capacity = 0;
    cudaEvent_t ev_bounce = nullptr;   // the last deferred frame is done with the queue
    // screen tables of the frame sizes rendered so far (see screen_table)
    vt::ScreenTable screen[vt::kScreenTables];
    int n_screen = 0;
    int bounce_blocks[2] = {0, 0};     // resident blocks of the bounce walk kernels (brick-run, one-path)
};

namespace vt {
constexpr int kWorkSlots = 256;
constexpr int kBandStreams = 4;
constexpr int kMaxBands = 16;
}

struct vt_world {
    vt_ctx* ctx = nullptr;
    int dims[3] = {0, 0, 0};
    int cdim[3] = {0, 0, 0};
    size_t nchunks = 0;
    unsigned long long* d_mask = nullptr;
    unsigned char* d_mats = nullptr;
    unsigned long long* d_coarse = nullptr;
    size_t ncoarse = 0;
    unsigned* d_palette = nullptr;
    unsigned char* d_bdist = nullptr;
    unsigned char* d_cdist = nullptr;
    unsigned char* d_dtmp = nullptr;   // x (2 fields, 16 B/brick) and y (10 fields, 4 B/brick) pass results of the brick distances (kept)
    unsigned char* d_ctmp = nullptr;   // the same 6 fields for the chunk distances
    int* d_edit = nullptr;             // {x, y, z, valid} of the last device-side edit
    float* d_entities = nullptr;       // kMaxEntities boxes of 6 floats
    int n_entities = 0;
    bool dist_dirty = true;            // distances rebuilt before the next render
    bool dist_box = false;             // bricks in [box_lo, box_hi] edited since the last update
    int box_lo[3] = {0, 0, 0};
    int box_hi[3] = {0, 0, 0};
    unsigned char* d_stage = nullptr;  // upload staging (grown on demand)
    size_t stage_bytes = 0;

    vt::WorldView view() const {
        vt::WorldView v;
        v.mask = d_mask;
        v.mats = d_mats;
        v.coarse = d_coarse;
        v.palette = d_palette;
        v.bdist = d_bdist;
        v.cdist = d_cdist;
        v.entities = d_entities;
        v.n_entities = n_entities;
        v.nchunks = (unsigned)nchunks;
        for (int i = 0; i < 3; ++i) {
            v.dims[i] = dims[i];
            v.cdim[i] = cdim[i];
        }
        v.nwords = (unsigned)(nchunks * vt::kBricksPerChunk);
        v.ncoarse = (unsigned)ncoarse;
        v.cstride = vt::cdist_stride((unsigned)nchunks);
        return v;
    }
};

namespace vt {
// Every device and pinned-host allocation of the library goes through these
// (the testing hooks vt_debug_fail_alloc / vt_debug_alloc_counts see them):
// a failure injected by the hook reads as cudaErrorMemoryAllocation.
cudaError_t dev_alloc_raw(void** p, size_t bytes);
cudaError_t host_alloc_raw(void** p, size_t bytes);
cudaError_t dev_free(void* p);
cudaError_t host_free(void* p);
template <class T>
inline cudaError_t dev_alloc(T** p, size_t bytes) { return dev_alloc_raw(reinterpret_cast<void**>(p), bytes); }
template <class T>
inline cudaError_t host_alloc(T** p, size_t bytes) { return host_alloc_raw(reinterpret_cast<void**>(p), bytes); }
// Looks up, once per device, the device address of vt_render_host_static's
// fixed staging array (render_static.cu); called by vt_ctx_create.
vt_status static_staging_init(vt_ctx* ctx);
// Records `msg` (plus the CUDA error text when err != cudaSuccess) in the
// context and returns the matching status.
vt_status fail(vt_ctx* ctx, vt_status s, const std::string& msg, cudaError_t err = cudaSuccess);
vt_status check_cuda(vt_ctx* ctx, cudaError_t err, const char* what);
// Turns a device status word read back by the caller into the call's status
// (clearing the device word when it was set).
vt_status take_status(vt_ctx* ctx, unsigned st);
// Marks the status word as possibly set by a launch just queued on st.
vt_status note_status_writer(vt_ctx* ctx, cudaStream_t st);
// Context-owned device buffer of at least `bytes` (grown on demand).
vt_status ctx_scratch(vt_ctx* ctx, size_t bytes, void** out);
// Rebuilds the empty-space distances of a world on `st`.
vt_status rebuild_distances(vt_world* w, cudaStream_t st);
// Brings the distances up to date: a full rebuild when stale, else the
// neighbourhood of the bricks edited since the last update.
vt_status update_distances(vt_world* w, cudaStream_t st);
// update_distances, then the neighbourhood of the voxel {x, y, z, valid}
// that a kernel earlier on `st` wrote to d_cell (nothing when !valid).
vt_status update_distances_at(vt_world* w, const int* d_cell, cudaStream_t st);
// The world's staging buffer, grown to at least `bytes` (synchronises the
// device when it has to grow).
vt_status world_stage(vt_world* w, size_t bytes, unsigned char** out);
// Argument checks shared by the render entry points.
vt_status check_frame_args(vt_ctx* ctx, const vt_world* world, const vt_camera* cam, const vt_params* p);
// Queues one frame (render kernel, distances rebuilt first if stale) writing
// width*height records to d_out on `stream`.
// allow_defer: bounce rays may go through the context's deferred bounce pass
// (single-frame entry points; not inside graph capture or allocation-free
// calls).
// new_table: the frame's screen table may be made here (an allocation and one
// synchronisation, once per image size and field of view).
vt_status launch_render(vt_ctx* ctx, const vt_world* world, const vt_camera* cam, const vt_params* p, uint4* d_out,
                        cudaStream_t stream, bool stats, int row0 = 0, int row1 = -1, bool allow_defer = false,
                        bool new_table = true);
struct FrameParams;
// The context's screen table for a frame's image size and field of view
// (made on first use when `create` and the stream is not being captured;
// *out stays null when none can be had).
vt_status screen_table(vt_ctx* ctx, const FrameParams& f, cudaStream_t st, bool create, const float4** out);
// The L2 access-policy window over a world's brick words that render
// launches carry as a launch attribute (tuning l2_persist).  *out is null when
// the tuning is off or the device has no persisting L2; the first use
// reserves the device's persisting L2 for this process's context (undone
// when the context is destroyed).
vt_status l2_policy(vt_ctx* ctx, const vt_world* world, cudaAccessPolicyWindow* storage,
                    const cudaAccessPolicyWindow** out);
// The deferred bounce pass: queue buffers for `pixels` rays, and the trace +
// shade kernels for a frame whose render kernel queued them.
vt_status bounce_buffers(vt_ctx* ctx, size_t pixels);
// The context's band streams and events (created on first use).
vt_status band_streams(vt_ctx* ctx);
vt_status launch_bounce(vt_ctx* ctx, const vt_world* world, const FrameParams& f, uint4* d_out, cudaStream_t st);
}  // namespace vt

#define VT_CUDA(ctx, call)                                                      \
    do {                                                                        \
        cudaError_t _e = (call);                                                \
        if (_e != cudaSuccess) return vt::check_cuda((ctx), _e, #call);         \
    } while (0)
