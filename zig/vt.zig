//! vt.zig -- the reference engine's world/camera/render objects over libvt.
//!
//! Mirrors the Zig API the reference's game loop uses, so that src/game.zig
//! keeps its shape when the OpenGL path is replaced:
//!
//!   VoxelBrickmap.init/clear/set/get   (src/engine/voxel.zig:25-82)
//!   Camera.rotate/set_pos/incrementFov (src/engine/graphics/camera.zig:5-44)
//!   Renderer.render                    (src/game.zig:232-256: primary + secondary dispatch)
//!   Renderer.pick / edit               (assets/shaders/terrain_edit.comp.glsl:11-24)
//!
//! Every call goes through include/vt.h by @cImport; errors come back as
//! error.VoxelTracer with the library's message in `lastError`.  Where the
//! reference panics (a failed buffer grow, gpu_block_allocator.zig:22) these
//! wrappers return the error instead.
const std = @import("std");
pub const c = @cImport(@cInclude("vt.h"));

pub const Error = error{VoxelTracer};

fn check(ctx: ?*c.vt_ctx, s: c.vt_status) Error!void {
    if (s == c.VT_OK) return;
    if (ctx) |cx| std.log.err("libvt: {s}", .{c.vt_last_error_string(cx)});
    return error.VoxelTracer;
}

/// One CUDA device (the GL context's role).
pub const Context = struct {
    handle: *c.vt_ctx,

    pub fn init(device: i32) Error!Context {
        var h: ?*c.vt_ctx = null;
        try check(null, c.vt_ctx_create(device, &h));
        return .{ .handle = h.? };
    }

    pub fn deinit(self: *Context) void {
        _ = c.vt_ctx_destroy(self.handle);
    }

    pub fn lastError(self: *const Context) [*:0]const u8 {
        return c.vt_last_error_string(self.handle);
    }
};

/// The reference's Voxel (voxel.zig:7-19).  A nonzero voxel is occupied
/// whatever its ty (procgen.zig:42 writes ty 0 voxels), so a voxel maps to
/// material ty + 1 (capped at 255) and material m reads back as ty m - 1.
pub const Voxel = packed struct(u32) {
    ty: u28 = 0,
    is_solid: bool = false,
    _pad: u3 = 0,

    pub const EMPTY = Voxel{};
};

/// VoxelBrickmap(dim, chsize) over a device world of dim^3 voxels.  The
/// chunk edge is the library's (32); chsize is accepted for source
/// compatibility with the reference's generic type.
pub fn VoxelBrickmap(comptime dim: comptime_int, comptime chsize: comptime_int) type {
    _ = chsize;
    return struct {
        ctx: *Context,
        world: *c.vt_world,

        pub fn init(ctx: *Context) Error!@This() {
            var w: ?*c.vt_world = null;
            const desc = c.vt_world_desc{ .dims = .{ dim, dim, dim } };
            try check(ctx.handle, c.vt_world_create(ctx.handle, &desc, &w));
            return .{ .ctx = ctx, .world = w.? };
        }

        pub fn deinit(self: *@This()) void {
            _ = c.vt_world_destroy(self.world);
        }

        pub fn clear(self: *@This(), _: u32) Error!void {
            try check(self.ctx.handle, c.vt_world_clear(self.world, null));
        }

        pub fn set(self: *@This(), x: usize, y: usize, z: usize, voxel: Voxel) Error!void {
            const m: u8 = if (@as(u32, @bitCast(voxel)) == 0) 0 else @intCast(@min(@as(u32, voxel.ty) + 1, 255));
            try check(self.ctx.handle, c.vt_world_set_voxel(self.world, @intCast(x), @intCast(y), @intCast(z), m, null));
        }

        pub fn get(self: *@This(), x: usize, y: usize, z: usize) Error!Voxel {
            var m: u8 = 0;
            try check(self.ctx.handle, c.vt_world_get_voxel(self.world, @intCast(x), @intCast(y), @intCast(z), &m));
            return if (m == 0) Voxel.EMPTY else .{ .ty = m - 1, .is_solid = true };
        }

        /// The whole grid at once (x fastest), instead of dim^3 set() calls.
        pub fn upload(self: *@This(), materials: []const u8) Error!void {
            try check(self.ctx.handle, c.vt_world_upload_dense(self.world, materials.ptr, materials.len, null));
        }

        /// The seeded scene generator on the device (procgen.zig's role).
        pub fn generate(self: *@This(), seed: u64, trees: i32) Error!void {
            var d: c.vt_gen_desc = undefined;
            c.vt_gen_desc_init(&d, dim, dim, dim, @as(f32, @floatFromInt(dim)) / 128.0, seed);
            d.trees = trees;
            try check(self.ctx.handle, c.vt_world_generate(self.world, &d, null));
        }
    };
}

/// Camera (camera.zig:5-44): yaw/pitch in radians, the reference's 0.001
/// mouse gain and pitch clamp.
pub const Camera = struct {
    fov: f32 = std.math.pi / 2.0,
    pitch: f32 = 0.0,
    yaw: f32 = 0.0,
    cam_pos: [3]f32 = .{ 0, 0, 0 },

    pub fn rotate(self: *Camera, pitch: f32, yaw: f32) void {
        self.pitch = std.math.clamp(self.pitch + pitch * 0.001, -std.math.pi / 2.0, std.math.pi / 2.0);
        self.yaw = self.yaw + yaw * 0.001;
    }

    pub fn set_pos(self: *Camera, pos: [3]f32) void {
        self.cam_pos = pos;
    }

    pub fn incrementFov(self: *Camera, increment: f32) void {
        self.fov = std.math.clamp(self.fov + increment * 0.1, 0.314, 2.4);
    }

    /// The library's camera record for a width x height frame (the uniform
    /// block of camera.glsl:2-6 plus the frame size).
    pub fn as_uniform_data(self: *const Camera, width: i32, height: i32) Error!c.vt_camera {
        var out: c.vt_camera = undefined;
        try check(null, c.vt_camera_look(&self.cam_pos, self.yaw, self.pitch, self.fov, width, height, &out));
        return out;
    }
};

/// Game.render's two dispatches as one call: primary + shadow rays, shaded,
/// one 16-byte vt_hit per pixel into `records` (host memory).
pub const Renderer = struct {
    ctx: *Context,
    params: c.vt_params,

    pub fn init(ctx: *Context) Renderer {
        var p: c.vt_params = undefined;
        c.vt_params_default(&p);
        return .{ .ctx = ctx, .params = p };
    }

    pub fn render(self: *Renderer, world: *c.vt_world, cam: *const c.vt_camera, records: []c.vt_hit) Error!void {
        std.debug.assert(records.len == @as(usize, @intCast(cam.width * cam.height)));
        try check(self.ctx.handle, c.vt_render_host(self.ctx.handle, world, cam, &self.params, records.ptr));
    }

    /// terrain_edit.comp.glsl's pick ray; the hit voxel comes back.
    pub fn pick(self: *Renderer, world: *c.vt_world, cam: *const c.vt_camera, max_steps: i32) Error!c.vt_hit {
        var h: c.vt_hit = undefined;
        try check(self.ctx.handle, c.vt_pick(self.ctx.handle, world, cam, max_steps, &h));
        return h;
    }

    /// Pick + edit on the device: edit_mode 0 removes the hit voxel, 1..255
    /// places that material in front of it.
    pub fn edit(self: *Renderer, world: *c.vt_world, cam: *const c.vt_camera, max_steps: i32, edit_mode: i32) Error!void {
        try check(self.ctx.handle, c.vt_edit(self.ctx.handle, world, cam, max_steps, edit_mode, null, null));
    }
};
