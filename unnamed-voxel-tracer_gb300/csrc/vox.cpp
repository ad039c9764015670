// vox.cpp -- MagicaVoxel (.vox) reader for the reference-format model atlas.
//
// The reference loads block models with the zvox library (Game4all/zvox,
// deb43ad, build.zig.zon:27-30) and copies each model into its 8^3 atlas slot
// (VoxelModelAtlas.load_single_block_model, voxel.zig:94-112):
//     storage[x + 8 * (z + 8 * y)] = palette.colors[color - 1]
// i.e. the file's y and z axes swap, and only the first 8^3 entries of the
// storage are uploaded.  This reader follows the published file format:
// "VOX " + version, then chunks (id, content size, children size); the MAIN
// chunk's children hold SIZE/XYZI pairs (one per model, in order) and the
// RGBA palette (256 x r,g,b,a; colour index i in XYZI means entry i - 1).
#include <stdint.h>
#include <string.h>

#include <vector>

#include "../../include/vt.h"

namespace vt {

namespace {

uint32_t rd32(const uint8_t* p) { return (uint32_t)p[0] | ((uint32_t)p[1] << 8) | ((uint32_t)p[2] << 16) | ((uint32_t)p[3] << 24); }

}  // namespace

// Parses `bytes`; fills models (512 RGBA8 texels each, x + 8*(y + 8*z) in
// atlas order).  Returns VT_OK or VT_ERR_FORMAT.
vt_status parse_vox(const uint8_t* bytes, size_t n, std::vector<std::vector<uint32_t>>& models) {
    models.clear();
    if (n < 8 || memcmp(bytes, "VOX ", 4) != 0) return VT_ERR_FORMAT;
    size_t p = 8;
    // MAIN
    if (p + 12 > n || memcmp(bytes + p, "MAIN", 4) != 0) return VT_ERR_FORMAT;
    const uint32_t main_content = rd32(bytes + p + 4), main_children = rd32(bytes + p + 8);
    p += 12 + (size_t)main_content;
    const size_t end = p + (size_t)main_children;
    if (end > n) return VT_ERR_FORMAT;
    struct Raw {
        std::vector<uint8_t> xyzi;  // x, y, z, colour index per voxel
    };
    std::vector<Raw> raw;
    uint32_t palette[256];
    bool have_palette = false;
    bool expect_xyzi = false;
    while (p + 12 <= end) {
        const uint8_t* id = bytes + p;
        const uint32_t content = rd32(bytes + p + 4), children = rd32(bytes + p + 8);
        const size_t body = p + 12;
        if (body + (size_t)content + (size_t)children > end) return VT_ERR_FORMAT;
        if (memcmp(id, "SIZE", 4) == 0) {
            if (content < 12) return VT_ERR_FORMAT;
            expect_xyzi = true;
        } else if (memcmp(id, "XYZI", 4) == 0) {
            if (!expect_xyzi || content < 4) return VT_ERR_FORMAT;
            const uint32_t count = rd32(bytes + body);
            if ((size_t)count * 4 + 4 > content) return VT_ERR_FORMAT;
            Raw r;
            r.xyzi.assign(bytes + body + 4, bytes + body + 4 + (size_t)count * 4);
            raw.push_back(std::move(r));
            expect_xyzi = false;
        } else if (memcmp(id, "RGBA", 4) == 0) {
            if (content < 1024) return VT_ERR_FORMAT;
            for (int i = 0; i < 256; ++i) palette[i] = rd32(bytes + body + 4 * i);
            have_palette = true;
        }
        p = body + (size_t)content + (size_t)children;
    }
    if (!have_palette) return VT_ERR_FORMAT;
    for (const Raw& r : raw) {
        std::vector<uint32_t> m(512, 0u);
        for (size_t k = 0; k + 3 < r.xyzi.size(); k += 4) {
            const unsigned x = r.xyzi[k], y = r.xyzi[k + 1], z = r.xyzi[k + 2], ci = r.xyzi[k + 3];
            if (ci == 0) continue;  // colour indices start at 1
            const size_t idx = (size_t)x + 8u * ((size_t)z + 8u * (size_t)y);
            if (idx < 512) m[idx] = palette[ci - 1];
        }
        models.push_back(std::move(m));
    }
    return VT_OK;
}

}  // namespace vt

extern "C" vt_status vt_vox_decode(const uint8_t* h_bytes, size_t nbytes, uint32_t* h_texels, int32_t max_models,
                                   int32_t* models) {
    if (!h_bytes || !models || max_models < 0 || (max_models > 0 && !h_texels)) return VT_ERR_ARG;
    std::vector<std::vector<uint32_t>> m;
    const vt_status s = vt::parse_vox(h_bytes, nbytes, m);
    if (s) return s;
    *models = (int32_t)m.size();
    for (size_t i = 0; i < m.size() && (int32_t)i < max_models; ++i)
        memcpy(h_texels + i * 512, m[i].data(), 512 * sizeof(uint32_t));
    return VT_OK;
}
