/*
 * ref_gltf.cpp — runs gbizzotto/swegl's own glTF loader (src/data/gltf.cpp,
 * compiled unmodified from the reference sources by oracle/ref/Makefile
 * against the json.hpp stand-in in shim/) and writes the scene_t it builds as
 * text, so that tests can compare the library's loader with it.
 *
 * TEST INFRASTRUCTURE ONLY.  Built into oracle/_ref/libswegl_ref.so; nothing
 * in the product links it.
 *
 * Images: the reference decodes them with libpng / libjpeg
 * (src/misc/image.cpp), which are not available here.  The decoders below
 * stand in for read_image_file / read_png_file / read_jpeg_file and return a
 * 1x1 texture: the dump records how many images the loader read, and the
 * texel decoders are checked on their own.
 *
 * Dump (whitespace-separated; floats as C99 hex literals, exact):
 *   images N
 *   materials N, then per material: colour (BGRA as one uint32), metallic,
 *     roughness, texture index, double sided
 *   nodes N, then per node: scale xyz, translation xyz, rotation (16, row
 *     major), root flag, children count and indices, primitive count; per
 *     primitive: mode, material, vertex count, index count, then per vertex
 *     position xyz, normal xyz, texture coordinates xy, then the indices
 *   roots N and the root node indices
 *   animations N, then per animation: end time, channel count; per channel:
 *     node, path, step count; per step: time and value xyzw
 */
#include <cstdio>
#include <string>

#include <swegl/data/gltf.hpp>
#include <swegl/misc/image.hpp>

namespace swegl {

texture_t read_image_file(const std::string &, int) { return texture_t(0xFF000000u); }
texture_t read_png_file(const std::string &, int) { return texture_t(0xFF000000u); }
texture_t read_jpeg_file(const std::string &, int) { return texture_t(0xFF000000u); }

} // namespace swegl

namespace {

void hexf(FILE *f, float v) { std::fprintf(f, " %a", (double)v); }

} // namespace

extern "C" __attribute__((visibility("default"))) int ref_gltf_dump(const char *path, const char *out_path)
{
    FILE *f = std::fopen(out_path, "w");
    if (!f)
        return -1;
    swegl::scene_t s = swegl::load_scene(path);
    std::fprintf(f, "images %zu\n", s.images.size());
    std::fprintf(f, "materials %zu\n", s.materials.size());
    for (const auto &m : s.materials) {
        std::fprintf(f, "%u", (unsigned)m.color.to_int());
        hexf(f, m.metallic);
        hexf(f, m.roughness);
        std::fprintf(f, " %d %d\n", m.texture_idx, m.double_sided ? 1 : 0);
    }
    std::fprintf(f, "nodes %zu\n", s.nodes.size());
    for (const auto &n : s.nodes) {
        hexf(f, n.scale.x());
        hexf(f, n.scale.y());
        hexf(f, n.scale.z());
        hexf(f, n.translation.x());
        hexf(f, n.translation.y());
        hexf(f, n.translation.z());
        for (int r = 0; r < 4; r++)
            for (int c = 0; c < 4; c++)
                hexf(f, n.rotation[r][c]);
        std::fprintf(f, " %d %zu", n.root ? 1 : 0, n.children_idx.size());
        for (int c : n.children_idx)
            std::fprintf(f, " %d", c);
        std::fprintf(f, " %zu\n", n.primitives.size());
        for (const auto &p : n.primitives) {
            std::fprintf(f, "%d %d %zu %zu\n", (int)p.mode, p.material_id, p.vertices.size(), p.indices.size());
            for (const auto &v : p.vertices) {
                hexf(f, v.v.x());
                hexf(f, v.v.y());
                hexf(f, v.v.z());
                hexf(f, v.normal.x());
                hexf(f, v.normal.y());
                hexf(f, v.normal.z());
                hexf(f, v.tex_coords.x());
                hexf(f, v.tex_coords.y());
                std::fprintf(f, "\n");
            }
            for (auto i : p.indices)
                std::fprintf(f, " %u", (unsigned)i);
            std::fprintf(f, "\n");
        }
    }
    std::fprintf(f, "roots %zu", s.root_nodes.size());
    for (int r : s.root_nodes)
        std::fprintf(f, " %d", r);
    std::fprintf(f, "\nanimations %zu\n", s.animations.size());
    for (const auto &a : s.animations) {
        hexf(f, a.end_time);
        std::fprintf(f, " %zu\n", a.channels.size());
        for (const auto &c : a.channels) {
            std::fprintf(f, "%d %d %zu\n", c.node_idx, (int)c.path, c.steps.size());
            for (const auto &st : c.steps) {
                hexf(f, st.time);
                hexf(f, st.value.x());
                hexf(f, st.value.y());
                hexf(f, st.value.z());
                hexf(f, st.value.w());
                std::fprintf(f, "\n");
            }
        }
    }
    std::fclose(f);
    return 0;
}
