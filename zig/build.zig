//! Builds zig/example.zig against libvt (unnamed-voxel-tracer_gb300/lib/libvt.so).
//! In the reference's own build.zig the same three lines go on its `exe`.
const std = @import("std");

pub fn build(b: *std.Build) void {
    const target = b.standardTargetOptions(.{});
    const optimize = b.standardOptimizeOption(.{});
    const exe = b.addExecutable(.{
        .name = "vt-example",
        .root_source_file = b.path("example.zig"),
        .target = target,
        .optimize = optimize,
    });
    exe.addIncludePath(b.path("../include"));
    exe.addLibraryPath(b.path("../unnamed-voxel-tracer_gb300/lib"));
    exe.linkSystemLibrary("vt");
    exe.linkLibC();
    b.installArtifact(exe);
}
