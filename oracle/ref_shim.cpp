// ref_shim.cpp -- C entry points around the reference's own shader functions
// (TEST INFRASTRUCTURE).  oracle/build_ref.py extracts the function bodies from
// the reference's GLSL (map.glsl, camera.glsl, primary.comp.glsl) into
// oracle/_ref/*.inc and compiles this file with them; the resulting
// oracle/_ref/libref.so runs the reference's traversal on the CPU so that the
// C restatement in vt_oracle.c can be checked against it.
#include "glsl_compat.hpp"

// the shader's resources (map.glsl:11-19, camera.glsl:1-5)
static const uint* chunks = nullptr;  // binding 10
static uint* data = nullptr;          // binding 9
static image3D model;                 // binding 6
static vec4 C_position;
static mat4 C_view;
static float fov = 0.0f;

#include "ref_map.inc"
#include "ref_camera.inc"

extern "C" {

void ref_set_world(const uint32_t* chunk_table, uint32_t* bricks, const uint32_t* atlas) {
    chunks = chunk_table;
    data = bricks;
    model.texels = atlas;
}

static void put(const HitInfo& h, uint32_t* out_data, float hit_pos[3], float normal[3]) {
    *out_data = h.data;
    hit_pos[0] = h.hit_pos.x;
    hit_pos[1] = h.hit_pos.y;
    hit_pos[2] = h.hit_pos.z;
    normal[0] = h.normal.x;
    normal[1] = h.normal.y;
    normal[2] = h.normal.z;
}

void ref_trace_map(const float o[3], const float d[3], int32_t max_steps, uint32_t* out_data, float hit_pos[3],
                   float normal[3]) {
    put(traceMap(vec3(o[0], o[1], o[2]), vec3(d[0], d[1], d[2]), max_steps), out_data, hit_pos, normal);
}

void ref_trace_entities(const float o[3], const float d[3], float max_distance, uint32_t* out_data, float hit_pos[3],
                        float normal[3]) {
    put(traceEntities(vec3(o[0], o[1], o[2]), vec3(d[0], d[1], d[2]), max_distance), out_data, hit_pos, normal);
}

void ref_sky(const float ro[3], const float rd[3], float out[4]) {
    const vec4 c = SkyDome2(vec3(ro[0], ro[1], ro[2]), vec3(rd[0], rd[1], rd[2]));
    out[0] = c.x;
    out[1] = c.y;
    out[2] = c.z;
    out[3] = c.w;
}

// primary.comp.glsl:31-43 for one pixel: the ray and its traceMap result.
void ref_primary(const float cam_pos[4], const float view[16], float cam_fov, int32_t px, int32_t py, int32_t width,
                 int32_t height, float ray_dir[3], uint32_t* out_data, float hit_pos[3], float normal[3]) {
    C_position = vec4(cam_pos[0], cam_pos[1], cam_pos[2], cam_pos[3]);
    for (int i = 0; i < 16; ++i) C_view.m[i] = view[i];
    fov = cam_fov;
    ivec2 pixelCoords(px, py);
    ivec2 size(width, height);
#include "ref_primary.inc"
    ray_dir[0] = rayDir.x;
    ray_dir[1] = rayDir.y;
    ray_dir[2] = rayDir.z;
    put(inter, out_data, hit_pos, normal);
}

// terrain_edit.comp.glsl:11-17 (the pick ray) and map_setVoxel
// (map.glsl:49-55), the two pieces of the reference's editing pass.
void ref_pick(const float cam_pos[4], const float view[16], uint32_t* out_data, float hit_pos[3], float normal[3]) {
    C_position = vec4(cam_pos[0], cam_pos[1], cam_pos[2], cam_pos[3]);
    for (int i = 0; i < 16; ++i) C_view.m[i] = view[i];
#include "ref_edit.inc"
    put(inter, out_data, hit_pos, normal);
}

void ref_set_voxel(int32_t x, int32_t y, int32_t z, uint32_t voxel) { map_setVoxel(ivec3(x, y, z), voxel); }

}  // extern "C"
