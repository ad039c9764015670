//! The reference's frame loop (game.zig:90-256) reduced to libvt calls:
//! generate a world, place a camera, render a frame, edit where it looks.
const std = @import("std");
const vt = @import("vt.zig");

pub fn main() !void {
    var ctx = try vt.Context.init(0);
    defer ctx.deinit();

    var world = try vt.VoxelBrickmap(512, 8).init(&ctx);
    defer world.deinit();
    try world.generate(1, 200);

    var cam = vt.Camera{};
    cam.set_pos(.{ 256.0, 80.0, 256.0 });
    cam.rotate(-300.0, 700.0);
    const ucam = try cam.as_uniform_data(1280, 720);

    var renderer = vt.Renderer.init(&ctx);
    const records = try std.heap.page_allocator.alloc(vt.c.vt_hit, 1280 * 720);
    defer std.heap.page_allocator.free(records);
    try renderer.render(world.world, &ucam, records);

    const hit = try renderer.pick(world.world, &ucam, 512);
    std.debug.print("centre voxel {d} material {d}\n", .{ hit.voxel, hit.material });
    try renderer.edit(world.world, &ucam, 512, 0);
}
