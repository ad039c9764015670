// world.cu -- mode-P world storage on the device and its upload entry points.
//
// The reference keeps its world in two persistently mapped SSBOs that the host
// writes voxel by voxel (VoxelBrickmap, src/engine/voxel.zig:25-82): a 64^3
// chunk table of brick indices and a pool of 8^3 u32 bricks.  Here the host
// hands over uint8 materials (dense, or one 32^3 chunk at a time) and a kernel
// builds the traversal structures on the device:
//
//   materials  chunk-major; inside a chunk 512 bricks of 64 bytes, brick
//              b = bx + 8*(by + 8*bz), voxel v = x + 4*(y + 4*z) in the brick
//   mask       one u64 per brick, bit v set iff material != 0
//   coarse     one bit per chunk, set iff any brick word of the chunk is != 0
#include <algorithm>
#include <cstring>

#include "vt_internal.h"

namespace vt {

// One block per chunk, one thread per brick.  src is a dense x-fastest box of
// sdims voxels whose voxel (0,0,0) sits at world voxel `sorg`; world cells
// outside the source box or outside the world read as air.
__global__ void __launch_bounds__(512) k_build_chunks(WorldView w, unsigned long long* mask, unsigned char* mats,
                                                      unsigned long long* coarse, const unsigned char* __restrict__ src,
                                                      int3 sdims, int3 sorg, int3 cfirst, int3 ccount) {
    const int lin = blockIdx.x;
    const int cx = cfirst.x + lin % ccount.x;
    const int cy = cfirst.y + (lin / ccount.x) % ccount.y;
    const int cz = cfirst.z + lin / (ccount.x * ccount.y);
    const unsigned ci = (unsigned)cx + (unsigned)w.cdim[0] * ((unsigned)cy + (unsigned)w.cdim[1] * (unsigned)cz);
    const int b = threadIdx.x;
    const int bx = b & 7, by = (b >> 3) & 7, bz = b >> 6;
    const unsigned wi = ci * 512u + (unsigned)b;
    unsigned long long m = 0ull;
    unsigned packed[16];
#pragma unroll
    for (int z = 0; z < 4; ++z) {
#pragma unroll
        for (int y = 0; y < 4; ++y) {
            unsigned word = 0;
#pragma unroll
            for (int x = 0; x < 4; ++x) {
                const int gx = cx * 32 + bx * 4 + x, gy = cy * 32 + by * 4 + y, gz = cz * 32 + bz * 4 + z;
                const int sx = gx - sorg.x, sy = gy - sorg.y, sz = gz - sorg.z;
                unsigned v = 0;
                if (gx < w.dims[0] && gy < w.dims[1] && gz < w.dims[2] && sx >= 0 && sy >= 0 && sz >= 0 &&
                    sx < sdims.x && sy < sdims.y && sz < sdims.z)
                    v = src[(size_t)sx + (size_t)sdims.x * ((size_t)sy + (size_t)sdims.y * (size_t)sz)];
                word |= v << (8 * x);
                if (v) m |= 1ull << (x + 4 * (y + 4 * z));
            }
            packed[y + 4 * z] = word;
        }
    }
    uint4* dst = reinterpret_cast<uint4*>(mats + (size_t)wi * 64u);
#pragma unroll
    for (int q = 0; q < 4; ++q) dst[q] = make_uint4(packed[4 * q], packed[4 * q + 1], packed[4 * q + 2], packed[4 * q + 3]);
    mask[wi] = m;
    const int any = __syncthreads_or(m != 0ull);
    if (threadIdx.x == 0) {
        const unsigned long long bit = 1ull << (ci & 63u);
        if (any) atomicOr(coarse + (ci >> 6), bit);
        else atomicAnd(coarse + (ci >> 6), ~bit);
    }
}

// VoxelBrickmap.set (voxel.zig:58-61): one voxel, then the chunk's coarse bit.
__global__ void __launch_bounds__(512) k_set_voxel(WorldView w, unsigned long long* mask, unsigned char* mats,
                                                   unsigned long long* coarse, int x, int y, int z, unsigned mat) {
    const unsigned ci = (unsigned)(x >> 5) + (unsigned)w.cdim[0] * ((unsigned)(y >> 5) + (unsigned)w.cdim[1] * (unsigned)(z >> 5));
    const unsigned bi = (unsigned)((x >> 2) & 7) | ((unsigned)((y >> 2) & 7) << 3) | ((unsigned)((z >> 2) & 7) << 6);
    const unsigned vb = (unsigned)(x & 3) | ((unsigned)(y & 3) << 2) | ((unsigned)(z & 3) << 4);
    if (threadIdx.x == 0) {
        const unsigned wi = ci * 512u + bi;
        mats[(size_t)wi * 64u + vb] = (unsigned char)mat;
        if (mat) mask[wi] |= 1ull << vb;
        else mask[wi] &= ~(1ull << vb);
    }
    __syncthreads();
    const int any = __syncthreads_or(mask[ci * 512u + threadIdx.x] != 0ull);
    if (threadIdx.x == 0) {
        const unsigned long long bit = 1ull << (ci & 63u);
        if (any) atomicOr(coarse + (ci >> 6), bit);
        else atomicAnd(coarse + (ci >> 6), ~bit);
    }
}

// Empty-space distances, per direction octant.  For the octant with signs s,
// a weighted Chebyshev distance to the nearest occupied cell ahead is
// separable:
//     min over c' ahead of max(|dx|, w|dy|, |dz|)
//   = min_{dz ahead} max(|dz|, min_{dy ahead} max(w|dy|, min_{dx ahead} max(|dx|, occ(c')))),
// so each field is three one-sided 1-D min-max passes, x, then y, then z.
// The x pass depends on s_x only (2 fields), the y pass on s_x, s_y (4 fields),
// the z pass on all three (8 fields).  Cells outside the grid count as empty.
//
// Chunk level: chunks to chunks, "ahead" meaning 0 <= s_i * d_i <= kDistCap,
// capped at kDistCap + 1.  blockIdx.y is the output field v: bit i of v gives
// the direction of axis i (1: +) for axes 0..axis; the pass reads input field
// v & ((1 << axis) - 1) (pass 0 reads the coarse bits instead).  Fields are
// `stride` bytes apart.  The pass covers the whole chunk grid.
__global__ void k_dist_pass(const unsigned long long* __restrict__ coarse, const unsigned char* __restrict__ in,
                            unsigned char* __restrict__ out, int axis, int CX, int CY, int CZ, size_t stride) {
    const unsigned v = blockIdx.y;
    const bool fwd = ((v >> axis) & 1u) != 0u;
    if (axis > 0) in += (size_t)(v & ((1u << axis) - 1u)) * stride;
    out += (size_t)v * stride;
    const int dlo = fwd ? 0 : -kDistCap, dhi = fwd ? kDistCap : 0;
    const int g[3] = {CX, CY, CZ};
    const size_t total = (size_t)CX * CY * CZ;
    for (size_t lin = blockIdx.x * (size_t)blockDim.x + threadIdx.x; lin < total; lin += (size_t)gridDim.x * blockDim.x) {
        int p[3] = {(int)(lin % CX), (int)((lin / CX) % CY), (int)(lin / ((size_t)CX * CY))};
        const int u = p[axis];
        int best = kDistCap + 1;
        for (int dd = dlo; dd <= dhi; ++dd) {
            const int q = u + dd;
            if (q < 0 || q >= g[axis]) continue;
            p[axis] = q;
            const unsigned idx = (unsigned)p[0] + (unsigned)CX * ((unsigned)p[1] + (unsigned)CY * (unsigned)p[2]);
            const int val = axis == 0 ? (((coarse[idx >> 6] >> (idx & 63u)) & 1ull) ? 0 : kDistCap + 1) : (int)in[idx];
            best = min(best, max(abs(dd), val));
        }
        out[lin] = (unsigned char)best;
    }
}

// Brick level, in voxels.  With vertical weight w = 2^shape, brick b has
//     s_w = min(kVoxCap + 1, min over occupied voxels q ahead of b of max(dx, w*dy, dz)),
// where d_i is the number of voxel layers between b's far face on axis i and
// q (0 when q lies within b's extent on that axis) and "ahead" means q is not
// behind b's near face on any axis: b plus s_w - 1 layers beyond its far faces
// across and (s_w - 1) / w layers vertically holds no occupied voxel (s_w = 0:
// b is occupied).  Field o of b stores s_1 for the octants moving +y, and for
// those moving -y the s_w | shape << 6 of the shape with the largest box
// (box_score; the smallest weight on a tie).  Each pass coarsens one axis from
// voxels to bricks:
//   x: X(bx, qy, qz), 2 fields (x direction): layers from brick bx's far x face
//      to the first occupied voxel of row (qy, qz) (read from the mask words);
//   y: Y(bx, by, qz), kYFields fields (y_field: x and y direction, and for -y
//      the shape): min over qy of max(w*dy, X(bx, qy, qz));
//   z: the brick field, 8 fields: min over qz of max(dz, Y(bx, by, qz)), and
//      the shape choice.
// The intermediates are x-fastest arrays: X over (GX bricks, GY*4, GZ*4
// voxels), Y over (GX, GY bricks, GZ*4 voxels).  Each pass covers a box of
// its own output grid, [lo, lo + ext) clipped to the grid; with `d_cell`
// ({x, y, z, valid} of an edited voxel in device memory) the box is taken
// relative to that voxel's brick (brick axes) or the brick's first voxel
// (voxel axes), and skipped when !valid.
__device__ __forceinline__ unsigned brick_index(int bx, int by, int bz, int CX, int CY) {
    const unsigned ci = (unsigned)(bx >> 3) + (unsigned)CX * ((unsigned)(by >> 3) + (unsigned)CY * (unsigned)(bz >> 3));
    return ci * 512u + (unsigned)((bx & 7) | ((by & 7) << 3) | ((bz & 7) << 6));
}

struct BrickGrid {
    int CX, CY, CZ;   // chunks
    int GX, GY, GZ;   // bricks
};

// The y pass's fields: x direction xs, y direction ys (1: +y) and, for -y,
// the box shape.
constexpr int kYFields = 2 + 2 * kBoxShapes;
__host__ __device__ constexpr int y_field(int xs, int ys, int shape) { return ys ? xs : 2 + xs + 2 * shape; }

__device__ __forceinline__ bool box_cell(size_t lin, int3 lo, int3 ext, int3 g, int& x, int& y, int& z) {
    x = lo.x + (int)(lin % ext.x);
    y = lo.y + (int)((lin / ext.x) % ext.y);
    z = lo.z + (int)(lin / ((size_t)ext.x * ext.y));
    return x >= 0 && y >= 0 && z >= 0 && x < g.x && y < g.y && z < g.z;
}

__device__ __forceinline__ int3 edit_origin(int3 lo, const int* d_cell, bool vx, bool vy, bool vz) {
    const int bx = d_cell[0] >> 2, by = d_cell[1] >> 2, bz = d_cell[2] >> 2;
    lo.x += vx ? 4 * bx : bx;
    lo.y += vy ? 4 * by : by;
    lo.z += vz ? 4 * bz : bz;
    return lo;
}

__global__ void k_bdist_x(const unsigned long long* __restrict__ mask, unsigned char* __restrict__ xf, BrickGrid b,
                          int3 lo, int3 ext, const int* __restrict__ d_cell) {
    if (d_cell) {
        if (!d_cell[3]) return;
        lo = edit_origin(lo, d_cell, false, true, true);
    }
    const bool fwd = blockIdx.y != 0;
    const int3 g = make_int3(b.GX, b.GY * 4, b.GZ * 4);
    const size_t fsize = (size_t)g.x * g.y * g.z;
    xf += blockIdx.y * fsize;
    const size_t total = (size_t)ext.x * ext.y * ext.z;
    for (size_t lin = blockIdx.x * (size_t)blockDim.x + threadIdx.x; lin < total; lin += (size_t)gridDim.x * blockDim.x) {
        int bx, qy, qz;
        if (!box_cell(lin, lo, ext, g, bx, qy, qz)) continue;
        const unsigned row = 4u * (unsigned)(qy & 3) + 16u * (unsigned)(qz & 3);
        int best = kVoxCap + 1;
        for (int j = 0;; ++j) {
            const int nb = fwd ? bx + j : bx - j;
            // a voxel of brick nb lies at least 4j - 3 layers beyond bx's far face
            if (max(0, 4 * j - 3) >= best || nb < 0 || nb >= g.x) break;
            const unsigned bits = (unsigned)(mask[brick_index(nb, qy >> 2, qz >> 2, b.CX, b.CY)] >> row) & 15u;
            if (bits) {
                best = fwd ? max(0, 4 * j + (__ffs(bits) - 1) - 3) : max(0, 4 * j - (31 - __clz(bits)));
                break;
            }
        }
        xf[(size_t)bx + (size_t)g.x * ((size_t)qy + (size_t)g.y * qz)] = (unsigned char)min(best, kVoxCap + 1);
    }
}

__global__ void k_bdist_y(const unsigned char* __restrict__ xf, unsigned char* __restrict__ yf, BrickGrid b, int3 lo,
                          int3 ext, const int* __restrict__ d_cell) {
    if (d_cell) {
        if (!d_cell[3]) return;
        lo = edit_origin(lo, d_cell, false, false, true);
    }
    const int yi = (int)blockIdx.y;  // y_field(xs, ys, shape)
    const bool fwd = yi < 2;
    const int xs = fwd ? yi : (yi - 2) & 1, shape = fwd ? 0 : (yi - 2) >> 1;
    const int wy = 1 << shape;
    const int Y = b.GY * 4;
    const int3 g = make_int3(b.GX, b.GY, b.GZ * 4);
    xf += (size_t)xs * ((size_t)b.GX * Y * g.z);
    yf += (size_t)yi * ((size_t)g.x * g.y * g.z);
    const size_t total = (size_t)ext.x * ext.y * ext.z;
    for (size_t lin = blockIdx.x * (size_t)blockDim.x + threadIdx.x; lin < total; lin += (size_t)gridDim.x * blockDim.x) {
        int bx, by, qz;
        if (!box_cell(lin, lo, ext, g, bx, by, qz)) continue;
        int best = kVoxCap + 1;
        for (int t = 0;; ++t) {
            const int dy = max(0, t - 3);
            const int qy = fwd ? 4 * by + t : 4 * by + 3 - t;
            if (wy * dy >= best || qy < 0 || qy >= Y) break;
            best = min(best, max(wy * dy, (int)xf[(size_t)bx + (size_t)g.x * ((size_t)qy + (size_t)Y * qz)]));
        }
        yf[(size_t)bx + (size_t)g.x * ((size_t)by + (size_t)g.y * qz)] = (unsigned char)best;
    }
}

__global__ void k_bdist_z(const unsigned char* __restrict__ yf, unsigned char* __restrict__ out, BrickGrid b, int3 lo,
                          int3 ext, const int* __restrict__ d_cell, size_t stride) {
    if (d_cell) {
        if (!d_cell[3]) return;
        lo = edit_origin(lo, d_cell, false, false, false);
    }
    const unsigned v = blockIdx.y;   // the octant
    const bool fwd = (v & 4u) != 0u, up = (v & 2u) != 0u;
    const int xs = (int)(v & 1u);
    const int Z = b.GZ * 4;
    const int3 g = make_int3(b.GX, b.GY, b.GZ);
    const size_t yfield = (size_t)b.GX * b.GY * Z;
    out += (size_t)v * stride;
    const size_t total = (size_t)ext.x * ext.y * ext.z;
    for (size_t lin = blockIdx.x * (size_t)blockDim.x + threadIdx.x; lin < total; lin += (size_t)gridDim.x * blockDim.x) {
        int bx, by, bz;
        if (!box_cell(lin, lo, ext, g, bx, by, bz)) continue;
        const size_t col = (size_t)bx + (size_t)g.x * (size_t)by;
        unsigned char res = 0;
        int best_score = -1;
        for (int shape = 0; shape < (up ? 1 : kBoxShapes); ++shape) {
            const unsigned char* f = yf + (size_t)y_field(xs, up ? 1 : 0, shape) * yfield;
            int best = kVoxCap + 1;
            for (int t = 0;; ++t) {
                const int dz = max(0, t - 3);
                const int qz = fwd ? 4 * bz + t : 4 * bz + 3 - t;
                if (dz >= best || qz < 0 || qz >= Z) break;
                best = min(best, max(dz, (int)f[col + (size_t)g.x * g.y * qz]));
            }
            if (best == 0) break;   // the brick is occupied
            const int score = box_score(best, shape);
            if (score > best_score) {
                best_score = score;
                res = (unsigned char)(best | (shape << 6));
            }
        }
        out[brick_index(bx, by, bz, b.CX, b.CY)] = res;
    }
}

namespace {

constexpr int kDistThreads = 256;

unsigned dist_blocks(size_t n) {
    return (unsigned)std::min<size_t>((n + kDistThreads - 1) / kDistThreads, 65535u * 4u);
}

size_t volume(int3 e) { return (size_t)e.x * e.y * e.z; }

// The chunk level over the whole chunk grid (at most a few tens of thousands
// of cells: cheap enough to redo after any edit): x into 2 fields of tmp, y
// into the 4 fields after them, z into the 8 output fields.
void chunk_passes(vt_world* w, cudaStream_t st) {
    const int CX = w->cdim[0], CY = w->cdim[1], CZ = w->cdim[2];
    const size_t stride = cdist_stride((unsigned)w->nchunks);
    unsigned char* fx = w->d_ctmp;
    unsigned char* fy = w->d_ctmp + 2 * stride;
    const unsigned nb = dist_blocks(w->nchunks);
    k_dist_pass<<<dim3(nb, 2), kDistThreads, 0, st>>>(w->d_coarse, nullptr, fx, 0, CX, CY, CZ, stride);
    k_dist_pass<<<dim3(nb, 4), kDistThreads, 0, st>>>(w->d_coarse, fx, fy, 1, CX, CY, CZ, stride);
    k_dist_pass<<<dim3(nb, 8), kDistThreads, 0, st>>>(w->d_coarse, fy, w->d_cdist, 2, CX, CY, CZ, stride);
}

// The brick level, each pass over its own box (x: bricks x voxels x voxels,
// y: bricks x bricks x voxels, z: bricks).  The intermediates stay valid
// between calls, which is what lets an edit recompute only the boxes it can
// change.
void brick_passes(vt_world* w, cudaStream_t st, const int3 lo[3], const int3 ext[3], const int* d_cell) {
    const BrickGrid b = {w->cdim[0], w->cdim[1], w->cdim[2], w->cdim[0] * 8, w->cdim[1] * 8, w->cdim[2] * 8};
    const size_t nb = w->nchunks * kBricksPerChunk;
    unsigned char* xf = w->d_dtmp;             // 2 fields of 16 bytes per brick
    unsigned char* yf = w->d_dtmp + 32 * nb;   // kYFields fields of 4 bytes per brick
    if (volume(ext[0]))
        k_bdist_x<<<dim3(dist_blocks(volume(ext[0])), 2), kDistThreads, 0, st>>>(w->d_mask, xf, b, lo[0], ext[0], d_cell);
    if (volume(ext[1]))
        k_bdist_y<<<dim3(dist_blocks(volume(ext[1])), kYFields), kDistThreads, 0, st>>>(xf, yf, b, lo[1], ext[1],
                                                                                        d_cell);
    if (volume(ext[2]))
        k_bdist_z<<<dim3(dist_blocks(volume(ext[2])), 8), kDistThreads, 0, st>>>(yf, w->d_bdist, b, lo[2], ext[2],
                                                                                 d_cell, nb);
}

// After the bricks of box [blo, blo + bext) changed occupancy only these
// cells can change (R bricks: a pass stops before a layer kVoxCap + 1 beyond
// the far face, so it reads at most kVoxCap + 3 layers past the near face,
// which reaches R = (kVoxCap + 3) / 4 bricks away): the x pass in the box
// +- R bricks in x over the edited bricks' voxel rows, the y pass +- R bricks
// in x and y over their voxel layers in z, the z pass +- R bricks on every
// axis.  Recomputing those boxes, in pass order, from the current masks
// leaves every buffer equal to a full rebuild.
void edit_boxes(int3 blo, int3 bext, int3 lo[3], int3 ext[3]) {
    const int R = (kVoxCap + 3) / 4;
    lo[0] = make_int3(blo.x - R, 4 * blo.y, 4 * blo.z);
    ext[0] = make_int3(bext.x + 2 * R, 4 * bext.y, 4 * bext.z);
    lo[1] = make_int3(blo.x - R, blo.y - R, 4 * blo.z);
    ext[1] = make_int3(bext.x + 2 * R, bext.y + 2 * R, 4 * bext.z);
    lo[2] = make_int3(blo.x - R, blo.y - R, blo.z - R);
    ext[2] = make_int3(bext.x + 2 * R, bext.y + 2 * R, bext.z + 2 * R);
}

}  // namespace

vt_status rebuild_distances(vt_world* w, cudaStream_t st) {
    const int GX = w->cdim[0] * 8, GY = w->cdim[1] * 8, GZ = w->cdim[2] * 8;
    const int3 o = make_int3(0, 0, 0);
    const int3 lo[3] = {o, o, o};
    const int3 ext[3] = {make_int3(GX, 4 * GY, 4 * GZ), make_int3(GX, GY, 4 * GZ), make_int3(GX, GY, GZ)};
    brick_passes(w, st, lo, ext, nullptr);
    chunk_passes(w, st);
    VT_CUDA(w->ctx, cudaGetLastError());
    w->dist_dirty = false;
    w->dist_box = false;
    return VT_OK;
}

vt_status update_distances(vt_world* w, cudaStream_t st) {
    if (w->dist_dirty) return rebuild_distances(w, st);
    if (!w->dist_box) return VT_OK;
    const int3 blo = make_int3(w->box_lo[0], w->box_lo[1], w->box_lo[2]);
    const int3 bext = make_int3(w->box_hi[0] - w->box_lo[0] + 1, w->box_hi[1] - w->box_lo[1] + 1,
                                w->box_hi[2] - w->box_lo[2] + 1);
    int3 lo[3], ext[3];
    edit_boxes(blo, bext, lo, ext);
    if (volume(ext[2]) >= w->nchunks * kBricksPerChunk / 2) return rebuild_distances(w, st);
    brick_passes(w, st, lo, ext, nullptr);
    chunk_passes(w, st);
    VT_CUDA(w->ctx, cudaGetLastError());
    w->dist_box = false;
    return VT_OK;
}

vt_status update_distances_at(vt_world* w, const int* d_cell, cudaStream_t st) {
    vt_status s = update_distances(w, st);
    if (s || w->dist_dirty) return s;
    int3 lo[3], ext[3];
    edit_boxes(make_int3(0, 0, 0), make_int3(1, 1, 1), lo, ext);
    brick_passes(w, st, lo, ext, d_cell);
    chunk_passes(w, st);
    VT_CUDA(w->ctx, cudaGetLastError());
    return VT_OK;
}

// Records an edit of the bricks in [lo, hi] (inclusive brick coordinates):
// the distances near them are recomputed before the next use (unless a full
// rebuild is pending anyway).
static void note_edit(vt_world* w, const int lo[3], const int hi[3]) {
    if (w->dist_dirty) return;
    for (int i = 0; i < 3; ++i) {
        if (!w->dist_box || lo[i] < w->box_lo[i]) w->box_lo[i] = lo[i];
        if (!w->dist_box || hi[i] > w->box_hi[i]) w->box_hi[i] = hi[i];
    }
    w->dist_box = true;
}

vt_status world_stage(vt_world* w, size_t bytes, unsigned char** out) {
    if (bytes <= w->stage_bytes) {
        *out = w->d_stage;
        return VT_OK;
    }
    if (w->d_stage) {
        VT_CUDA(w->ctx, cudaDeviceSynchronize());
        vt::dev_free(w->d_stage);
        w->d_stage = nullptr;
        w->stage_bytes = 0;
    }
    VT_CUDA(w->ctx, vt::dev_alloc(&w->d_stage, bytes));
    w->stage_bytes = bytes;
    *out = w->d_stage;
    return VT_OK;
}

static void free_world(vt_world* w) {
    if (w->d_mask) vt::dev_free(w->d_mask);
    if (w->d_mats) vt::dev_free(w->d_mats);
    if (w->d_coarse) vt::dev_free(w->d_coarse);
    if (w->d_palette) vt::dev_free(w->d_palette);
    if (w->d_stage) vt::dev_free(w->d_stage);
    if (w->d_bdist) vt::dev_free(w->d_bdist);
    if (w->d_cdist) vt::dev_free(w->d_cdist);
    if (w->d_dtmp) vt::dev_free(w->d_dtmp);
    if (w->d_ctmp) vt::dev_free(w->d_ctmp);
    if (w->d_edit) vt::dev_free(w->d_edit);
    if (w->d_entities) vt::dev_free(w->d_entities);
    delete w;
}

}  // namespace vt

using namespace vt;

extern "C" {

vt_status vt_world_create(vt_ctx* ctx, const vt_world_desc* desc, vt_world** out) {
    if (!ctx) return VT_ERR_ARG;
    if (!desc || !out) return fail(ctx, VT_ERR_ARG, "null world descriptor or output");
    *out = nullptr;
    uint64_t cells = 1;
    for (int i = 0; i < 3; ++i) {
        if (desc->dims[i] < 1 || desc->dims[i] > 8192) return fail(ctx, VT_ERR_ARG, "world dims must be in [1, 8192]");
        cells *= (uint64_t)desc->dims[i];
    }
    if (cells >= (1ull << 32)) return fail(ctx, VT_ERR_ARG, "world must hold fewer than 2^32 voxels");
    vt_world* w = new (std::nothrow) vt_world();
    if (!w) return fail(ctx, VT_ERR_OOM, "host allocation failed");
    w->ctx = ctx;
    for (int i = 0; i < 3; ++i) {
        w->dims[i] = desc->dims[i];
        w->cdim[i] = (desc->dims[i] + kChunk - 1) / kChunk;
    }
    w->nchunks = (size_t)w->cdim[0] * w->cdim[1] * w->cdim[2];
    w->ncoarse = (w->nchunks + 63) / 64;
    cudaError_t e;
    if ((e = vt::dev_alloc(&w->d_mask, w->nchunks * kBricksPerChunk * 8)) != cudaSuccess ||
        (e = vt::dev_alloc(&w->d_mats, w->nchunks * (size_t)kChunkBytes)) != cudaSuccess ||
        (e = vt::dev_alloc(&w->d_coarse, w->ncoarse * 8)) != cudaSuccess ||
        (e = vt::dev_alloc(&w->d_palette, 256 * sizeof(unsigned))) != cudaSuccess ||
        (e = vt::dev_alloc(&w->d_bdist, kOctants * w->nchunks * kBricksPerChunk)) != cudaSuccess ||
        (e = vt::dev_alloc(&w->d_cdist, kOctants * (size_t)cdist_stride((unsigned)w->nchunks))) != cudaSuccess ||
        (e = vt::dev_alloc(&w->d_dtmp, (32 + 4 * kYFields) * w->nchunks * kBricksPerChunk)) != cudaSuccess ||
        (e = vt::dev_alloc(&w->d_ctmp, 6 * (size_t)cdist_stride((unsigned)w->nchunks))) != cudaSuccess ||
        (e = vt::dev_alloc(&w->d_edit, 4 * sizeof(int))) != cudaSuccess ||
        (e = vt::dev_alloc(&w->d_entities, kMaxEntities * 6 * sizeof(float))) != cudaSuccess ||
        (e = cudaMemset(w->d_edit, 0, 4 * sizeof(int))) != cudaSuccess ||
        (e = cudaMemset(w->d_mask, 0, w->nchunks * kBricksPerChunk * 8)) != cudaSuccess ||
        (e = cudaMemset(w->d_mats, 0, w->nchunks * (size_t)kChunkBytes)) != cudaSuccess ||
        (e = cudaMemset(w->d_coarse, 0, w->ncoarse * 8)) != cudaSuccess) {
        free_world(w);
        return check_cuda(ctx, e, "world allocation");
    }
    uint32_t pal[256];
    vt_default_palette(pal);
    if ((e = cudaMemcpy(w->d_palette, pal, sizeof(pal), cudaMemcpyHostToDevice)) != cudaSuccess) {
        free_world(w);
        return check_cuda(ctx, e, "palette upload");
    }
    *out = w;
    return VT_OK;
}

vt_status vt_world_destroy(vt_world* world) {
    if (!world) return VT_ERR_ARG;
    cudaDeviceSynchronize();
    free_world(world);
    return VT_OK;
}

vt_status vt_world_clear(vt_world* w, vt_stream stream) {
    if (!w) return VT_ERR_ARG;
    cudaStream_t s = (cudaStream_t)stream;
    VT_CUDA(w->ctx, cudaMemsetAsync(w->d_mask, 0, w->nchunks * kBricksPerChunk * 8, s));
    VT_CUDA(w->ctx, cudaMemsetAsync(w->d_mats, 0, w->nchunks * (size_t)kChunkBytes, s));
    VT_CUDA(w->ctx, cudaMemsetAsync(w->d_coarse, 0, w->ncoarse * 8, s));
    w->dist_dirty = true;
    return VT_OK;
}

vt_status vt_world_upload_dense(vt_world* w, const uint8_t* h_materials, size_t nbytes, vt_stream stream) {
    if (!w) return VT_ERR_ARG;
    const size_t need = (size_t)w->dims[0] * w->dims[1] * w->dims[2];
    if (!h_materials || nbytes != need) return fail(w->ctx, VT_ERR_ARG, "dense upload needs exactly X*Y*Z bytes");
    unsigned char* stage = nullptr;
    vt_status s = world_stage(w, need, &stage);
    if (s) return s;
    cudaStream_t st = (cudaStream_t)stream;
    VT_CUDA(w->ctx, cudaMemcpyAsync(w->d_stage, h_materials, need, cudaMemcpyHostToDevice, st));
    const int3 sdims = make_int3(w->dims[0], w->dims[1], w->dims[2]);
    k_build_chunks<<<(unsigned)w->nchunks, 512, 0, st>>>(w->view(), w->d_mask, w->d_mats, w->d_coarse, w->d_stage, sdims,
                                                        make_int3(0, 0, 0), make_int3(0, 0, 0),
                                                        make_int3(w->cdim[0], w->cdim[1], w->cdim[2]));
    VT_CUDA(w->ctx, cudaGetLastError());
    w->dist_dirty = true;
    // the staging buffer is reused by the next upload on any stream
    VT_CUDA(w->ctx, cudaStreamSynchronize(st));
    return VT_OK;
}

vt_status vt_world_upload_chunk(vt_world* w, int32_t cx, int32_t cy, int32_t cz, const uint8_t* h_chunk,
                                vt_stream stream) {
    if (!w) return VT_ERR_ARG;
    if (!h_chunk) return fail(w->ctx, VT_ERR_ARG, "null chunk");
    if (cx < 0 || cy < 0 || cz < 0 || cx >= w->cdim[0] || cy >= w->cdim[1] || cz >= w->cdim[2])
        return fail(w->ctx, VT_ERR_ARG, "chunk coordinate out of range");
    unsigned char* stage = nullptr;
    vt_status s = world_stage(w, kChunkBytes, &stage);
    if (s) return s;
    cudaStream_t st = (cudaStream_t)stream;
    VT_CUDA(w->ctx, cudaMemcpyAsync(w->d_stage, h_chunk, kChunkBytes, cudaMemcpyHostToDevice, st));
    k_build_chunks<<<1, 512, 0, st>>>(w->view(), w->d_mask, w->d_mats, w->d_coarse, w->d_stage, make_int3(32, 32, 32),
                                      make_int3(cx * 32, cy * 32, cz * 32), make_int3(cx, cy, cz), make_int3(1, 1, 1));
    VT_CUDA(w->ctx, cudaGetLastError());
    const int blo[3] = {cx * 8, cy * 8, cz * 8}, bhi[3] = {cx * 8 + 7, cy * 8 + 7, cz * 8 + 7};
    note_edit(w, blo, bhi);
    VT_CUDA(w->ctx, cudaStreamSynchronize(st));
    return VT_OK;
}

vt_status vt_world_set_voxel(vt_world* w, int32_t x, int32_t y, int32_t z, uint8_t material, vt_stream stream) {
    if (!w) return VT_ERR_ARG;
    if (x < 0 || y < 0 || z < 0 || x >= w->dims[0] || y >= w->dims[1] || z >= w->dims[2])
        return fail(w->ctx, VT_ERR_ARG, "voxel coordinate out of range");
    k_set_voxel<<<1, 512, 0, (cudaStream_t)stream>>>(w->view(), w->d_mask, w->d_mats, w->d_coarse, x, y, z, material);
    VT_CUDA(w->ctx, cudaGetLastError());
    const int b[3] = {x >> 2, y >> 2, z >> 2};
    note_edit(w, b, b);
    return VT_OK;
}

vt_status vt_world_get_voxel(vt_world* w, int32_t x, int32_t y, int32_t z, uint8_t* material) {
    if (!w) return VT_ERR_ARG;
    if (!material || x < 0 || y < 0 || z < 0 || x >= w->dims[0] || y >= w->dims[1] || z >= w->dims[2])
        return fail(w->ctx, VT_ERR_ARG, "voxel coordinate out of range");
    const unsigned ci = (unsigned)(x >> 5) + (unsigned)w->cdim[0] * ((unsigned)(y >> 5) + (unsigned)w->cdim[1] * (unsigned)(z >> 5));
    const unsigned bi = (unsigned)((x >> 2) & 7) | ((unsigned)((y >> 2) & 7) << 3) | ((unsigned)((z >> 2) & 7) << 6);
    const unsigned vb = (unsigned)(x & 3) | ((unsigned)(y & 3) << 2) | ((unsigned)(z & 3) << 4);
    VT_CUDA(w->ctx, cudaDeviceSynchronize());
    VT_CUDA(w->ctx, cudaMemcpy(material, w->d_mats + ((size_t)ci * 512u + bi) * 64u + vb, 1, cudaMemcpyDeviceToHost));
    return VT_OK;
}

vt_status vt_world_set_palette(vt_world* w, const uint32_t* h_rgba256) {
    if (!w) return VT_ERR_ARG;
    if (!h_rgba256) return fail(w->ctx, VT_ERR_ARG, "null palette");
    VT_CUDA(w->ctx, cudaMemcpy(w->d_palette, h_rgba256, 256 * sizeof(uint32_t), cudaMemcpyHostToDevice));
    return VT_OK;
}

vt_status vt_world_set_entities(vt_world* w, const float* h_boxes, int32_t n) {
    if (!w) return VT_ERR_ARG;
    if (n < 0 || n > kMaxEntities || (n > 0 && !h_boxes))
        return fail(w->ctx, VT_ERR_ARG, "entity count must be in [0, 1024] with a box list");
    for (int i = 0; i < 6 * n; ++i)
        if (!(h_boxes[i] == h_boxes[i])) return fail(w->ctx, VT_ERR_ARG, "entity box coordinates must not be NaN");
    if (n > 0) VT_CUDA(w->ctx, cudaMemcpy(w->d_entities, h_boxes, (size_t)n * 6 * sizeof(float), cudaMemcpyHostToDevice));
    w->n_entities = n;
    return VT_OK;
}

vt_status vt_world_get_info(const vt_world* w, vt_world_info* info) {
    if (!w || !info) return VT_ERR_ARG;
    std::memset(info, 0, sizeof(*info));
    for (int i = 0; i < 3; ++i) {
        info->dims[i] = w->dims[i];
        info->chunks[i] = w->cdim[i];
    }
    info->mask_bytes = (uint64_t)w->nchunks * kBricksPerChunk * 8;
    info->material_bytes = (uint64_t)w->nchunks * kChunkBytes;
    info->coarse_bytes = (uint64_t)w->ncoarse * 8;
    info->d_mask = w->d_mask;
    info->d_materials = w->d_mats;
    info->d_coarse = w->d_coarse;
    return VT_OK;
}

}  // extern "C"
