// sgl_gltf.cpp — glTF 2.0 (.gltf / .glb) scenes into sgl_scene_desc, and
// their animations, following swegl's loader (src/data/gltf.cpp:13-464) and
// scene_t::animate (swegl/data/model.hpp:146-177), quirks included:
//   * POSITION, NORMAL and TEXCOORD_0 are read as floats whatever the
//     accessor's component type, and TEXCOORD_0's two components are swapped
//     (gltf.cpp:178-186);
//   * indices are read as 16-bit values at the accessor's stride, whatever
//     their component type (gltf.cpp:196);
//   * a primitive without indices draws nothing; modes other than triangles,
//     strips and fans draw nothing (renderer.cpp:196-232);
//   * meshes without "primitives" are skipped when meshes are numbered, and
//     a mesh used by a second node gives that node no primitives (its
//     primitives were moved to the first, gltf.cpp:296);
//   * a material without pbrMetallicRoughness is white and single-sided
//     (gltf.cpp:121-125); base colour bytes are (uint8)(255 * factor);
//   * a node rotation quaternion [x, y, z, w] goes to
//     matrix44_t::from_quaternion(x, y, z, w), which takes its first
//     argument as the scalar part (swegl/projection/matrix44.hpp:34-43);
//   * a node matrix is split with scales from its rows' lengths, each
//     dividing a column (gltf.cpp:246-292).
// A .gltf's buffers and images are files next to it (as in the reference) or
// base64 data URIs (an addition).  The arithmetic is float, in the
// reference's order of operations.
#include <algorithm>
#include <array>
#include <cmath>
#include <cctype>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <string>
#include <utility>
#include <vector>

#include "sgl.h"
#include "sgl_image.h"

namespace sgl {
namespace json {

// A JSON value (RFC 8259); numbers are kept as doubles.
struct Value {
    enum Kind { Null, Bool, Number, String, Array, Object } kind = Null;
    bool b = false;
    double num = 0.0;
    std::string str;
    std::vector<Value> arr;
    std::vector<std::pair<std::string, Value>> obj;

    const Value *get(const char *key) const
    {
        if (kind != Object)
            return nullptr;
        for (const auto &kv : obj)
            if (kv.first == key)
                return &kv.second;
        return nullptr;
    }
    bool has(const char *key) const { return get(key) != nullptr; }
    size_t size() const { return kind == Array ? arr.size() : (kind == Object ? obj.size() : 0); }
    const Value *at(size_t i) const { return (kind == Array && i < arr.size()) ? &arr[i] : nullptr; }
};

struct Parser {
    const char *p, *end;
    std::string err;
    int depth = 0;

    void ws()
    {
        while (p < end && (*p == ' ' || *p == '\t' || *p == '\n' || *p == '\r'))
            p++;
    }
    bool bad(const char *m)
    {
        if (err.empty())
            err = m;
        return false;
    }
    static void put_utf8(std::string &s, uint32_t c)
    {
        if (c < 0x80) {
            s += (char)c;
        } else if (c < 0x800) {
            s += (char)(0xC0 | (c >> 6));
            s += (char)(0x80 | (c & 0x3F));
        } else if (c < 0x10000) {
            s += (char)(0xE0 | (c >> 12));
            s += (char)(0x80 | ((c >> 6) & 0x3F));
            s += (char)(0x80 | (c & 0x3F));
        } else {
            s += (char)(0xF0 | (c >> 18));
            s += (char)(0x80 | ((c >> 12) & 0x3F));
            s += (char)(0x80 | ((c >> 6) & 0x3F));
            s += (char)(0x80 | (c & 0x3F));
        }
    }
    bool hex4(uint32_t &v)
    {
        if (end - p < 4)
            return bad("JSON: short \\u escape");
        v = 0;
        for (int k = 0; k < 4; k++, p++) {
            const char c = *p;
            v <<= 4;
            if (c >= '0' && c <= '9') v |= (uint32_t)(c - '0');
            else if (c >= 'a' && c <= 'f') v |= (uint32_t)(c - 'a' + 10);
            else if (c >= 'A' && c <= 'F') v |= (uint32_t)(c - 'A' + 10);
            else return bad("JSON: bad \\u escape");
        }
        return true;
    }
    bool string(std::string &s)
    {
        if (p >= end || *p != '"')
            return bad("JSON: string expected");
        p++;
        while (p < end && *p != '"') {
            const char c = *p++;
            if (c != '\\') {
                s += c;
                continue;
            }
            if (p >= end)
                return bad("JSON: unterminated escape");
            const char e = *p++;
            switch (e) {
            case '"': s += '"'; break;
            case '\\': s += '\\'; break;
            case '/': s += '/'; break;
            case 'b': s += '\b'; break;
            case 'f': s += '\f'; break;
            case 'n': s += '\n'; break;
            case 'r': s += '\r'; break;
            case 't': s += '\t'; break;
            case 'u': {
                uint32_t c1;
                if (!hex4(c1))
                    return false;
                if (c1 >= 0xD800 && c1 < 0xDC00 && end - p >= 6 && p[0] == '\\' && p[1] == 'u') {
                    p += 2;
                    uint32_t c2;
                    if (!hex4(c2))
                        return false;
                    c1 = 0x10000 + ((c1 - 0xD800) << 10) + (c2 - 0xDC00);
                }
                put_utf8(s, c1);
                break;
            }
            default: return bad("JSON: unknown escape");
            }
        }
        if (p >= end)
            return bad("JSON: unterminated string");
        p++;
        return true;
    }
    bool number(double &v)
    {
        const char *s = p;
        if (p < end && *p == '-')
            p++;
        while (p < end && ((*p >= '0' && *p <= '9') || *p == '.' || *p == 'e' || *p == 'E' || *p == '+' || *p == '-'))
            p++;
        if (p == s)
            return bad("JSON: value expected");
        const std::string t(s, p);
        char *e = nullptr;
        v = std::strtod(t.c_str(), &e);
        if (!e || *e)
            return bad("JSON: bad number");
        return true;
    }
    bool value(Value &v)
    {
        if (++depth > 256)
            return bad("JSON: nested too deeply");
        ws();
        if (p >= end)
            return bad("JSON: unexpected end");
        bool ok = true;
        if (*p == '{') {
            v.kind = Value::Object;
            p++;
            ws();
            if (p < end && *p == '}') {
                p++;
            } else {
                for (;;) {
                    ws();
                    std::pair<std::string, Value> kv;
                    if (!string(kv.first))
                        return false;
                    ws();
                    if (p >= end || *p != ':')
                        return bad("JSON: ':' expected");
                    p++;
                    if (!value(kv.second))
                        return false;
                    v.obj.push_back(std::move(kv));
                    ws();
                    if (p < end && *p == ',') {
                        p++;
                        continue;
                    }
                    if (p < end && *p == '}') {
                        p++;
                        break;
                    }
                    return bad("JSON: ',' or '}' expected");
                }
            }
        } else if (*p == '[') {
            v.kind = Value::Array;
            p++;
            ws();
            if (p < end && *p == ']') {
                p++;
            } else {
                for (;;) {
                    Value e;
                    if (!value(e))
                        return false;
                    v.arr.push_back(std::move(e));
                    ws();
                    if (p < end && *p == ',') {
                        p++;
                        continue;
                    }
                    if (p < end && *p == ']') {
                        p++;
                        break;
                    }
                    return bad("JSON: ',' or ']' expected");
                }
            }
        } else if (*p == '"') {
            v.kind = Value::String;
            ok = string(v.str);
        } else if (end - p >= 4 && !std::strncmp(p, "true", 4)) {
            v.kind = Value::Bool;
            v.b = true;
            p += 4;
        } else if (end - p >= 5 && !std::strncmp(p, "false", 5)) {
            v.kind = Value::Bool;
            p += 5;
        } else if (end - p >= 4 && !std::strncmp(p, "null", 4)) {
            p += 4;
        } else {
            v.kind = Value::Number;
            ok = number(v.num);
        }
        depth--;
        return ok;
    }
};

bool parse(const char *data, size_t size, Value &out, std::string &err)
{
    Parser ps{data, data + size};
    if (!ps.value(out)) {
        err = ps.err;
        return false;
    }
    ps.ws();
    if (ps.p != ps.end) {
        err = "JSON: trailing characters";
        return false;
    }
    return true;
}

} // namespace json

namespace {

using json::Value;

struct Step {
    float time;
    float v[4];
};
enum Path { P_SCALE = 0, P_ROTATION = 1, P_TRANSLATION = 2, P_OTHER = 3 };
struct Channel {
    int node;
    int path;
    std::vector<Step> steps;
};
struct Animation {
    float end_time = 0.0f;
    std::vector<Channel> channels;
};

struct Bytes {
    std::shared_ptr<std::vector<uint8_t>> owner;
    const uint8_t *data = nullptr;
    size_t size = 0;
};

struct BufferView {
    Bytes bytes;
    int stride = 0;
};

struct Accessor {
    Bytes bytes; // from the accessor's byte offset to the end of its buffer view
    int stride = 0;
    int count = 0;
};

struct Error {
    std::string msg;
};

} // namespace

// The loaded scene and the state scene_t::animate edits.
struct GltfScene {
    std::vector<sgl_node_desc> nodes;
    std::vector<sgl_primitive_desc> prims;
    std::vector<float> pos, nrm, uv;
    std::vector<uint32_t> idx;
    std::vector<sgl_material_desc> mats;
    std::vector<Image> images;
    std::vector<sgl_texture_desc> texs;
    std::vector<Animation> anims;
    sgl_scene_desc desc{};

    void finish_desc()
    {
        desc = sgl_scene_desc{};
        desc.n_nodes = (int)nodes.size();
        desc.nodes = nodes.data();
        desc.n_primitives = (int)prims.size();
        desc.primitives = prims.data();
        desc.n_vertices = (uint32_t)(pos.size() / 3);
        desc.positions = pos.data();
        desc.normals = nrm.data();
        desc.uvs = uv.data();
        desc.n_indices = (uint32_t)idx.size();
        desc.indices = idx.data();
        desc.n_materials = (int)mats.size();
        desc.materials = mats.data();
        texs.clear();
        for (const Image &im : images)
            texs.push_back(sgl_texture_desc{im.texels.data(), im.width, im.height});
        desc.n_textures = (int)texs.size();
        desc.textures = texs.data();
        // a loaded scene_t carries no lights; the caller sets them
        desc.ambient = 0.0f;
        desc.sun_direction[0] = desc.sun_direction[1] = desc.sun_direction[2] = 0.0f;
        desc.sun_intensity = 0.0f;
        desc.default_material = sgl_material_desc{0xFFFFFFFFu, -1, 0, 32}; // material_t's defaults
    }
};

namespace {

bool read_file(const std::string &path, std::vector<uint8_t> &out)
{
    FILE *f = std::fopen(path.c_str(), "rb");
    if (!f)
        return false;
    std::fseek(f, 0, SEEK_END);
    const long n = std::ftell(f);
    std::fseek(f, 0, SEEK_SET);
    if (n < 0) {
        std::fclose(f);
        return false;
    }
    out.resize((size_t)n);
    const size_t got = n ? std::fread(out.data(), 1, (size_t)n, f) : 0;
    std::fclose(f);
    return got == (size_t)n;
}

bool base64(const std::string &s, size_t from, std::vector<uint8_t> &out)
{
    auto val = [](char c) -> int {
        if (c >= 'A' && c <= 'Z') return c - 'A';
        if (c >= 'a' && c <= 'z') return c - 'a' + 26;
        if (c >= '0' && c <= '9') return c - '0' + 52;
        if (c == '+') return 62;
        if (c == '/') return 63;
        return -1;
    };
    uint32_t acc = 0;
    int bits = 0;
    for (size_t i = from; i < s.size(); i++) {
        if (s[i] == '=')
            break;
        const int v = val(s[i]);
        if (v < 0)
            return false;
        acc = (acc << 6) | (uint32_t)v;
        bits += 6;
        if (bits >= 8) {
            bits -= 8;
            out.push_back((uint8_t)(acc >> bits));
        }
    }
    return true;
}

// A buffer or image named by a URI: a file relative to the scene's folder, or
// a base64 data URI.
bool load_uri(const std::string &dir, const std::string &uri, std::vector<uint8_t> &out)
{
    if (uri.compare(0, 5, "data:") == 0) {
        const size_t comma = uri.find(',');
        if (comma == std::string::npos || uri.find(";base64") > comma)
            return false;
        return base64(uri, comma + 1, out);
    }
    return read_file(dir.empty() ? uri : dir + "/" + uri, out);
}

// A JSON integer; non-numbers, NaN and values outside int give `dflt` or
// an out-of-range marker that every index check rejects.
int as_int(const Value *v, int dflt)
{
    if (!v || v->kind != Value::Number || !(v->num == v->num))
        return dflt;
    if (v->num >= 2147483647.0 || v->num <= -2147483648.0)
        return -2147483647;
    return (int)v->num;
}

float as_float(const Value *v, float dflt)
{
    return (v && v->kind == Value::Number) ? (float)v->num : dflt;
}

float rd_f32(const Bytes &b, size_t off)
{
    float f = 0.0f;
    if (off + 4 <= b.size)
        std::memcpy(&f, b.data + off, 4);
    return f;
}

uint32_t rd_u16(const Bytes &b, size_t off)
{
    uint32_t v = 0;
    if (off < b.size)
        v = b.data[off];
    if (off + 1 < b.size)
        v |= (uint32_t)b.data[off + 1] << 8;
    return v;
}

// matrix44_t::from_quaternion (swegl/projection/matrix44.hpp:34-43), row-major
void from_quaternion(float q0, float q1, float q2, float q3, float m[16])
{
    const float r[16] = {2 * (q0 * q0 + q1 * q1) - 1, 2 * (q1 * q2 - q0 * q3), 2 * (q1 * q3 + q0 * q2), 0.0f,
                         2 * (q1 * q2 + q0 * q3), 2 * (q0 * q0 + q2 * q2) - 1, 2 * (q2 * q3 - q0 * q1), 0.0f,
                         2 * (q1 * q3 - q0 * q2), 2 * (q2 * q3 + q0 * q1), 2 * (q0 * q0 + q3 * q3) - 1, 0.0f,
                         0.0f, 0.0f, 0.0f, 1.0f};
    std::memcpy(m, r, sizeof r);
}

float len3(float x, float y, float z) { return (float)std::sqrt(x * x + y * y + z * z); }

// (unsigned char)(255 * factor), the float-to-integer conversion then the low byte
uint32_t colour_byte(float f)
{
    const float v = 255 * f;
    if (!(v > -2147483648.0f && v < 2147483648.0f))
        return 0u;
    return (uint32_t)(uint8_t)(int32_t)v;
}

bool load_json_scene(GltfScene &g, const std::string &dir, const Value &j, std::vector<Bytes> &buffers,
                     const uint8_t *glb_file, size_t glb_size, std::string &err)
{
    (void)glb_file;
    (void)glb_size;
    auto fail = [&](const std::string &m) {
        err = "glTF: " + m;
        return false;
    };
    // buffer views (gltf.cpp:61-72)
    std::vector<BufferView> views;
    if (const Value *bvs = j.get("bufferViews")) {
        for (const Value &bv : bvs->arr) {
            const int b = as_int(bv.get("buffer"), -1);
            if (b < 0 || b >= (int)buffers.size())
                return fail("buffer view with a bad buffer index");
            const int off = as_int(bv.get("byteOffset"), 0), len = as_int(bv.get("byteLength"), -1);
            if (off < 0 || len < 0 || (size_t)off + (size_t)len > buffers[b].size)
                return fail("buffer view outside its buffer");
            BufferView v;
            v.bytes = buffers[b];
            v.bytes.data += off;
            v.bytes.size = (size_t)len;
            v.stride = as_int(bv.get("byteStride"), 0);
            views.push_back(v);
        }
    }
    // accessors (gltf.cpp:13-53)
    std::vector<Accessor> accessors;
    if (const Value *acs = j.get("accessors")) {
        for (const Value &a : acs->arr) {
            const int bvi = as_int(a.get("bufferView"), -1);
            if (bvi < 0 || bvi >= (int)views.size())
                return fail("accessor without a valid bufferView (sparse accessors are not read)");
            const BufferView &bv = views[bvi];
            Accessor ac;
            ac.count = as_int(a.get("count"), 0);
            ac.stride = bv.stride;
            if (ac.stride == 0) {
                const int ct = as_int(a.get("componentType"), 0);
                int cs = 0;
                switch (ct) {
                case 5120: case 5121: cs = 1; break;
                case 5122: case 5123: cs = 2; break;
                case 5125: case 5126: cs = 4; break;
                default: return fail("accessor with an unknown component type");
                }
                const Value *ty = a.get("type");
                const std::string t = ty ? ty->str : "";
                int nc = 0;
                if (t == "SCALAR") nc = 1;
                else if (t == "VEC2") nc = 2;
                else if (t == "VEC3") nc = 3;
                else if (t == "VEC4") nc = 4;
                else if (t == "MAT2") nc = 4;
                else if (t == "MAT3") nc = 9;
                else if (t == "MAT4") nc = 16;
                else return fail("accessor with an unknown type");
                ac.stride = cs * nc;
            }
            const int off = as_int(a.get("byteOffset"), 0);
            if (off < 0 || (size_t)off > bv.bytes.size || ac.count < 0)
                return fail("accessor outside its buffer view");
            ac.bytes = bv.bytes;
            ac.bytes.data += off;
            ac.bytes.size -= (size_t)off;
            accessors.push_back(ac);
        }
    }
    auto accessor = [&](const Value *v, Accessor *&out) {
        const int i = as_int(v, -1);
        if (i < 0 || i >= (int)accessors.size())
            return false;
        out = &accessors[i];
        return true;
    };
    // images (gltf.cpp:74-110)
    if (const Value *ims = j.get("images")) {
        for (const Value &im : ims->arr) {
            Image out;
            std::string ierr;
            if (const Value *uri = im.get("uri")) {
                std::vector<uint8_t> bytes;
                if (!load_uri(dir, uri->str, bytes))
                    return fail("cannot read image " + uri->str);
                const std::string name = uri->str.compare(0, 5, "data:") == 0
                                             ? (uri->str.find("image/png") != std::string::npos ? ".png" : ".jpg")
                                             : uri->str;
                if (!decode_by_name(name, bytes.data(), bytes.size(), out, ierr))
                    return fail(ierr);
            } else {
                const Value *mt = im.get("mimeType");
                const int bvi = as_int(im.get("bufferView"), -1);
                if (bvi < 0 || bvi >= (int)views.size())
                    return fail("image without a valid bufferView");
                const Bytes &b = views[bvi].bytes;
                const std::string mime = mt ? mt->str : "";
                bool ok;
                if (mime == "image/png")
                    ok = decode_png(b.data, b.size, out, ierr);
                else if (mime == "image/jpg" || mime == "image/jpeg")
                    ok = decode_jpeg(b.data, b.size, out, ierr);
                else
                    return fail("image of unknown mime type " + mime);
                if (!ok)
                    return fail(ierr);
            }
            g.images.push_back(std::move(out));
        }
    }
    // materials (gltf.cpp:112-154)
    if (const Value *ms = j.get("materials")) {
        for (const Value &m : ms->arr) {
            uint32_t b = 255, gg = 255, r = 255, a = 255;
            int img = -1;
            const Value *db = m.get("doubleSided");
            const bool double_sided = db && db->kind == Value::Bool && db->b;
            const Value *pbr = m.get("pbrMetallicRoughness");
            if (!pbr) {
                g.mats.push_back(sgl_material_desc{0xFFFFFFFFu, -1, 0, 32});
                continue;
            }
            if (const Value *f = pbr->get("baseColorFactor")) {
                b = colour_byte(as_float(f->at(2), 0.0f));
                gg = colour_byte(as_float(f->at(1), 0.0f));
                r = colour_byte(as_float(f->at(0), 0.0f));
                a = colour_byte(as_float(f->at(3), 0.0f));
            }
            if (const Value *t = pbr->get("baseColorTexture")) {
                const int ti = as_int(t->get("index"), -1);
                const Value *texs = j.get("textures");
                const Value *tex = texs ? texs->at((size_t)std::max(ti, 0)) : nullptr;
                if (ti < 0 || !tex)
                    return fail("material with a bad texture index");
                img = as_int(tex->get("source"), -1);
                if (img < 0 || img >= (int)g.images.size())
                    return fail("texture with a bad image index");
            }
            g.mats.push_back(sgl_material_desc{(a << 24) | (r << 16) | (gg << 8) | b, img, double_sided ? 1 : 0, 32});
        }
    }
    // meshes (gltf.cpp:156-203): per mesh with primitives, its primitives'
    // vertex and index data, staged until a node takes them
    struct Prim {
        int mode, material;
        std::vector<float> pos, nrm, uv;
        std::vector<uint32_t> idx;
    };
    std::vector<std::vector<Prim>> temp_meshes;
    if (const Value *meshes = j.get("meshes")) {
        for (const Value &mesh : meshes->arr) {
            const Value *prims = mesh.get("primitives");
            if (!prims)
                continue;
            std::vector<Prim> &out = temp_meshes.emplace_back();
            for (const Value &pv : prims->arr) {
                Prim pr;
                pr.material = as_int(pv.get("material"), -1);
                pr.mode = as_int(pv.get("mode"), 4);
                const Value *attrs = pv.get("attributes");
                Accessor *ap = nullptr;
                if (!attrs || !accessor(attrs->get("POSITION"), ap))
                    return fail("primitive without a valid POSITION accessor");
                const int n = ap->count;
                pr.pos.resize(3 * (size_t)n);
                pr.nrm.assign(3 * (size_t)n, 0.0f);
                pr.uv.assign(2 * (size_t)n, 0.0f);
                for (int i = 0; i < n; i++)
                    for (int c = 0; c < 3; c++)
                        pr.pos[3 * (size_t)i + c] = rd_f32(ap->bytes, 4 * (size_t)c + (size_t)i * ap->stride);
                Accessor *an = nullptr;
                if (attrs->has("NORMAL")) {
                    if (!accessor(attrs->get("NORMAL"), an))
                        return fail("bad NORMAL accessor");
                    for (int i = 0; i < std::min(n, an->count); i++)
                        for (int c = 0; c < 3; c++)
                            pr.nrm[3 * (size_t)i + c] = rd_f32(an->bytes, 4 * (size_t)c + (size_t)i * an->stride);
                }
                Accessor *at = nullptr;
                if (attrs->has("TEXCOORD_0")) {
                    if (!accessor(attrs->get("TEXCOORD_0"), at))
                        return fail("bad TEXCOORD_0 accessor");
                    for (int i = 0; i < std::min(n, at->count); i++) {
                        pr.uv[2 * (size_t)i] = rd_f32(at->bytes, 4 + (size_t)i * at->stride);
                        pr.uv[2 * (size_t)i + 1] = rd_f32(at->bytes, (size_t)i * at->stride);
                    }
                }
                if (pv.has("indices")) {
                    Accessor *ai = nullptr;
                    if (!accessor(pv.get("indices"), ai))
                        return fail("bad indices accessor");
                    pr.idx.resize((size_t)ai->count);
                    for (int i = 0; i < ai->count; i++) {
                        pr.idx[i] = rd_u16(ai->bytes, (size_t)i * ai->stride);
                        if (pr.idx[i] >= (uint32_t)n)
                            return fail("index outside its primitive's vertices (indices are read as 16-bit)");
                    }
                }
                out.push_back(std::move(pr));
            }
        }
    }
    // nodes (gltf.cpp:205-313)
    const Value *jnodes = j.get("nodes");
    const size_t n_nodes = jnodes ? jnodes->arr.size() : 0;
    std::vector<std::vector<int>> children(n_nodes);
    std::vector<bool> mesh_taken(temp_meshes.size(), false);
    for (size_t ni = 0; ni < n_nodes; ni++) {
        const Value &jn = jnodes->arr[ni];
        sgl_node_desc nd{};
        nd.scale[0] = nd.scale[1] = nd.scale[2] = 1.0f;
        float *m = nd.rotation;
        for (int k = 0; k < 16; k++)
            m[k] = (k % 5 == 0) ? 1.0f : 0.0f;
        nd.parent = -1;
        if (const Value *r = jn.get("rotation")) {
            if (r->size() != 4)
                return fail("node rotation must have 4 components");
            from_quaternion(as_float(r->at(0), 0), as_float(r->at(1), 0), as_float(r->at(2), 0), as_float(r->at(3), 0), m);
        }
        if (const Value *t = jn.get("translation")) {
            if (t->size() != 3)
                return fail("node translation must have 3 components");
            for (int c = 0; c < 3; c++)
                nd.translation[c] = as_float(t->at(c), 0);
        }
        if (const Value *s = jn.get("scale")) {
            if (s->size() != 3)
                return fail("node scale must have 3 components");
            for (int c = 0; c < 3; c++)
                nd.scale[c] = as_float(s->at(c), 0);
        }
        if (const Value *mm = jn.get("matrix")) {
            if (mm->size() != 16)
                return fail("node matrix must have 16 components");
            float a[16];
            for (int r = 0; r < 4; r++)
                for (int c = 0; c < 4; c++)
                    a[4 * r + c] = as_float(mm->at((size_t)(4 * c + r)), 0); // column-major to row-major
            nd.translation[0] = a[3];
            nd.translation[1] = a[7];
            nd.translation[2] = a[11];
            nd.scale[0] = len3(a[0], a[1], a[2]);
            nd.scale[1] = len3(a[4], a[5], a[6]);
            nd.scale[2] = len3(a[8], a[9], a[10]);
            a[3] = a[7] = a[11] = 0.0f;
            for (int c = 0; c < 3; c++)
                if (nd.scale[c] != 0)
                    for (int r = 0; r < 3; r++)
                        a[4 * r + c] /= nd.scale[c];
            std::memcpy(m, a, sizeof a);
        }
        g.nodes.push_back(nd);
        if (const Value *mi = jn.get("mesh")) {
            const int k = as_int(mi, -1);
            if (k < 0 || k >= (int)temp_meshes.size())
                return fail("node with a bad mesh index");
            if (!mesh_taken[k]) {
                mesh_taken[k] = true;
                for (Prim &pr : temp_meshes[k]) {
                    if (pr.mode != SGL_TRIANGLES && pr.mode != SGL_TRIANGLE_STRIP && pr.mode != SGL_TRIANGLE_FAN)
                        continue; // points and lines draw nothing
                    sgl_primitive_desc pd{};
                    pd.node = (int)ni;
                    pd.mode = pr.mode;
                    pd.material = pr.material;
                    pd.vertex_offset = (uint32_t)(g.pos.size() / 3);
                    pd.vertex_count = (uint32_t)(pr.pos.size() / 3);
                    pd.index_offset = (uint32_t)g.idx.size();
                    pd.index_count = (uint32_t)pr.idx.size();
                    g.pos.insert(g.pos.end(), pr.pos.begin(), pr.pos.end());
                    g.nrm.insert(g.nrm.end(), pr.nrm.begin(), pr.nrm.end());
                    g.uv.insert(g.uv.end(), pr.uv.begin(), pr.uv.end());
                    g.idx.insert(g.idx.end(), pr.idx.begin(), pr.idx.end());
                    g.prims.push_back(pd);
                }
            }
        }
        if (const Value *ch = jn.get("children"))
            for (const Value &c : ch->arr)
                children[ni].push_back(as_int(&c, -1));
    }
    for (size_t ni = 0; ni < n_nodes; ni++)
        for (int c : children[ni]) {
            if (c < 0 || c >= (int)n_nodes)
                return fail("node with a bad child index");
            g.nodes[c].parent = (int)ni;
        }
    for (const sgl_primitive_desc &pd : g.prims)
        if (pd.material >= (int)g.mats.size())
            return fail("primitive with a bad material index");
    // animations (gltf.cpp:322-385)
    if (const Value *anims = j.get("animations")) {
        for (const Value &ja : anims->arr) {
            Animation &an = g.anims.emplace_back();
            const Value *samplers = ja.get("samplers");
            const Value *channels = ja.get("channels");
            if (!samplers || !channels)
                return fail("animation without samplers or channels");
            for (const Value &jc : channels->arr) {
                const Value *target = jc.get("target");
                Channel ch;
                ch.node = as_int(target ? target->get("node") : nullptr, -1);
                const Value *pv = target ? target->get("path") : nullptr;
                const std::string path = pv ? pv->str : "";
                ch.path = path == "scale" ? P_SCALE : path == "rotation" ? P_ROTATION
                                                    : path == "translation" ? P_TRANSLATION : P_OTHER;
                if (ch.node < 0 || ch.node >= (int)n_nodes)
                    return fail("animation channel with a bad node");
                const Value *smp = samplers->at((size_t)std::max(as_int(jc.get("sampler"), -1), 0));
                if (!smp || as_int(jc.get("sampler"), -1) < 0)
                    return fail("animation channel with a bad sampler");
                Accessor *times = nullptr, *values = nullptr;
                if (!accessor(smp->get("input"), times) || !accessor(smp->get("output"), values))
                    return fail("animation sampler with bad accessors");
                for (int i = 0; i < times->count; i++) {
                    Step st{rd_f32(times->bytes, (size_t)i * times->stride), {0.0f, 0.0f, 0.0f, 1.0f}};
                    const int nc = ch.path == P_ROTATION ? 4 : (ch.path == P_OTHER ? 0 : 3);
                    for (int c = 0; c < nc; c++)
                        st.v[c] = rd_f32(values->bytes, 4 * (size_t)c + (size_t)i * values->stride);
                    ch.steps.push_back(st);
                }
                if (ch.steps.empty())
                    return fail("animation channel without keyframes");
                std::stable_sort(ch.steps.begin(), ch.steps.end(),
                                 [](const Step &a, const Step &b) { return a.time < b.time; });
                an.end_time = std::max(an.end_time, ch.steps.back().time);
                an.channels.push_back(std::move(ch));
            }
        }
    }
    g.finish_desc();
    return true;
}

} // namespace

// scene_t::animate (swegl/data/model.hpp:146-177) on the loaded nodes.
static void animate(GltfScene &g, float elapsed)
{
    for (Animation &an : g.anims) {
        const float rel = std::fmod(elapsed, an.end_time);
        for (Channel &ch : an.channels) {
            // animation_channel_t::get_steps (model.hpp:109-119)
            auto it = std::lower_bound(ch.steps.begin(), ch.steps.end(), rel,
                                       [](const Step &s, float t) { return s.time < t; });
            const Step *before, *after;
            if (it == ch.steps.end()) {
                before = after = &ch.steps.back();
            } else if (it == ch.steps.begin()) {
                before = after = &ch.steps.front();
            } else {
                before = &*std::prev(it);
                after = &*it;
            }
            float f[4];
            if (after->time == before->time) {
                std::memcpy(f, before->v, sizeof f);
            } else {
                const float wa = (after->time - rel) / (after->time - before->time);
                const float wb = (rel - before->time) / (after->time - before->time);
                for (int c = 0; c < 4; c++)
                    f[c] = before->v[c] * wa + after->v[c] * wb;
            }
            sgl_node_desc &nd = g.nodes[ch.node];
            if (ch.path == P_ROTATION) {
                // vec4f_t::normalize (swegl/projection/vec2f.hpp:67-77)
                const float len = (float)std::sqrt(f[0] * f[0] + f[1] * f[1] + f[2] * f[2] + f[3] * f[3]);
                if (len != 0) {
                    for (int c = 0; c < 4; c++)
                        f[c] = f[c] / len;
                }
                from_quaternion(f[0], f[1], f[2], f[3], nd.rotation);
            } else if (ch.path == P_TRANSLATION) {
                for (int c = 0; c < 3; c++)
                    nd.translation[c] = f[c];
            } else if (ch.path == P_SCALE) {
                for (int c = 0; c < 3; c++)
                    nd.scale[c] = f[c];
            }
        }
    }
}

static void put_error(char *buf, size_t size, const std::string &m)
{
    if (buf && size) {
        const size_t n = std::min(size - 1, m.size());
        std::memcpy(buf, m.data(), n);
        buf[n] = 0;
    }
}

static std::string dir_of(const std::string &path)
{
    const size_t s = path.find_last_of('/');
    return s == std::string::npos ? std::string() : path.substr(0, s);
}

static bool ends_with_ci(const std::string &s, const char *suf)
{
    const size_t k = std::strlen(suf);
    if (s.size() < k)
        return false;
    for (size_t i = 0; i < k; i++)
        if (std::tolower((unsigned char)s[s.size() - k + i]) != suf[i])
            return false;
    return true;
}

// load_scene_glb / load_scene_gltf (gltf.cpp:388-452)
static bool load_file(GltfScene &g, const std::string &path, std::string &err)
{
    auto file = std::make_shared<std::vector<uint8_t>>();
    if (!read_file(path, *file)) {
        err = "glTF: cannot read " + path;
        return false;
    }
    const std::string dir = dir_of(path);
    json::Value j;
    std::vector<Bytes> buffers;
    const uint8_t *bin = nullptr;
    size_t bin_size = 0;
    if (ends_with_ci(path, "glb")) {
        const std::vector<uint8_t> &f = *file;
        if (f.size() < 20 || std::memcmp(f.data(), "glTF", 4) != 0) {
            err = "glTF: not a GLB file";
            return false;
        }
        uint32_t total;
        std::memcpy(&total, f.data() + 8, 4);
        total = (uint32_t)std::min<size_t>(total, f.size());
        const uint8_t *jdata = nullptr;
        size_t jsize = 0;
        int k = 0;
        for (size_t at = 12; at + 8 <= total; k++) {
            uint32_t len;
            std::memcpy(&len, f.data() + at, 4);
            if (at + 8 + (size_t)len > total) {
                err = "glTF: GLB chunk overruns the file";
                return false;
            }
            if (k == 0) {
                jdata = f.data() + at + 8;
                jsize = len;
            } else if (k == 1) {
                bin = f.data() + at + 8;
                bin_size = len;
            }
            at += 8 + (size_t)len;
        }
        if (!jdata || !json::parse((const char *)jdata, jsize, j, err))
            return false;
    } else if (ends_with_ci(path, "gltf")) {
        if (!json::parse((const char *)file->data(), file->size(), j, err))
            return false;
    } else {
        err = "glTF: file name must end in .gltf or .glb";
        return false;
    }
    if (const Value *bufs = j.get("buffers")) {
        for (const Value &b : bufs->arr) {
            const int len = as_int(b.get("byteLength"), -1);
            Bytes by;
            if (const Value *uri = b.get("uri")) {
                auto data = std::make_shared<std::vector<uint8_t>>();
                if (!load_uri(dir, uri->str, *data)) {
                    err = "glTF: cannot read buffer " + uri->str;
                    return false;
                }
                by.owner = data;
                by.data = data->data();
                by.size = data->size();
            } else if (bin) {
                by.owner = file;
                by.data = bin;
                by.size = bin_size;
            } else {
                err = "glTF: buffer without a uri outside a GLB file";
                return false;
            }
            if (len < 0 || (size_t)len > by.size) {
                err = "glTF: buffer shorter than its byteLength";
                return false;
            }
            by.size = (size_t)len;
            buffers.push_back(by);
        }
    }
    return load_json_scene(g, dir, j, buffers, file->data(), file->size(), err);
}

} // namespace sgl

struct sgl_gltf {
    sgl::GltfScene scene;
};

extern "C" {

SGL_API sgl_status sgl_gltf_load(const char *path, sgl_gltf **out, char *error, size_t error_size)
{
    if (!path || !out)
        return SGL_ERR_INVALID;
    *out = nullptr;
    auto g = std::make_unique<sgl_gltf>();
    std::string err;
    try {
        if (!sgl::load_file(g->scene, path, err)) {
            sgl::put_error(error, error_size, err);
            return SGL_ERR_INVALID;
        }
    } catch (const std::bad_alloc &) {
        sgl::put_error(error, error_size, "glTF: out of host memory");
        return SGL_ERR_OOM;
    }
    *out = g.release();
    return SGL_OK;
}

SGL_API const sgl_scene_desc *sgl_gltf_scene(const sgl_gltf *g) { return g ? &g->scene.desc : nullptr; }

SGL_API int sgl_gltf_animation_count(const sgl_gltf *g) { return g ? (int)g->scene.anims.size() : 0; }

SGL_API sgl_status sgl_gltf_animate(sgl_gltf *g, float seconds, sgl_node_desc *nodes)
{
    if (!g)
        return SGL_ERR_INVALID;
    sgl::animate(g->scene, seconds);
    if (nodes)
        std::memcpy(nodes, g->scene.nodes.data(), sizeof(sgl_node_desc) * g->scene.nodes.size());
    return SGL_OK;
}

SGL_API void sgl_gltf_free(sgl_gltf *g) { delete g; }

SGL_API sgl_status sgl_image_load(const char *path, uint32_t **texels, int *width, int *height, char *error,
                                  size_t error_size)
{
    if (!path || !texels || !width || !height)
        return SGL_ERR_INVALID;
    *texels = nullptr;
    std::vector<uint8_t> bytes;
    if (!sgl::read_file(path, bytes)) {
        sgl::put_error(error, error_size, std::string("image: cannot read ") + path);
        return SGL_ERR_INVALID;
    }
    sgl::Image im;
    std::string err;
    if (!sgl::decode_by_name(path, bytes.data(), bytes.size(), im, err)) {
        sgl::put_error(error, error_size, err);
        return SGL_ERR_INVALID;
    }
    uint32_t *t = (uint32_t *)std::malloc(sizeof(uint32_t) * im.texels.size());
    if (!t)
        return SGL_ERR_OOM;
    std::memcpy(t, im.texels.data(), sizeof(uint32_t) * im.texels.size());
    *texels = t;
    *width = im.width;
    *height = im.height;
    return SGL_OK;
}

SGL_API void sgl_image_free(uint32_t *texels) { std::free(texels); }

} // extern "C"
