// Engine asset readers: .aemesh (Loader::MeshLoader::LoadMesh,
// src/engine/loader/MeshLoader.cpp:6-36, document layout of
// src/engine/mesh/MeshSerializer.cpp:7-156) and .aematerial
// (MeshSerializer.cpp:174-256), and the two steps the engine takes from them
// to the ray tracer's buffers: MeshData::BuildBVH's triangle assembly
// (src/engine/mesh/MeshData.cpp:89-155) and RayTracingWorld::UpdateMaterials'
// GPUMaterial flattening (src/engine/raytracing/RayTracingWorld.cpp:171-240).
//
// The engine writes meshes with nlohmann::json::to_msgpack (MeshLoader.cpp:47-58;
// ModelImporter.cpp:228-231 saves with binaryJson = true) and materials as
// JSON text.  Both decoders here are written from the MessagePack
// specification and RFC 8259; every length is checked against the bytes
// left, nesting is limited, and malformed input is an AE_RT_INVALID_ARG
// with a message (ae_asset_last_error), never a read past the buffer.
#include "atlas_rt.h"

#include <charconv>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <iterator>
#include <memory>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

namespace {

thread_local std::string g_asset_error;

struct AssetError : std::runtime_error {
    using std::runtime_error::runtime_error;
};

// A decoded document node.  Strings and binary blobs both keep their bytes
// in `bytes`.
struct Value {
    enum Kind { Nil, Bool, Int, Float, Str, Bin, Arr, Map } kind = Nil;
    bool b = false;
    int64_t i = 0;        // Int (unsigned values above INT64_MAX are rejected)
    double f = 0.0;       // Float
    std::string bytes;    // Str, Bin
    std::vector<Value> arr;
    std::vector<std::pair<std::string, Value>> map;

    const Value* find(const char* key) const {
        if (kind != Map) return nullptr;
        for (const auto& kv : map)
            if (kv.first == key) return &kv.second;
        return nullptr;
    }
    const Value& at(const char* key) const {
        const Value* v = find(key);
        if (!v) throw AssetError(std::string("missing field \"") + key + "\"");
        return *v;
    }
    bool is_number() const { return kind == Int || kind == Float; }
    double number(const char* what) const {
        if (kind == Int) return double(i);
        if (kind == Float) return f;
        if (kind == Bool) return b ? 1.0 : 0.0;
        throw AssetError(std::string("field \"") + what + "\" is not a number");
    }
    int64_t integer(const char* what) const {
        if (kind == Int) return i;
        if (kind == Float) return int64_t(f);
        if (kind == Bool) return b ? 1 : 0;
        throw AssetError(std::string("field \"") + what + "\" is not a number");
    }
    bool boolean(const char* what) const {
        if (kind == Bool) return b;
        if (kind == Int) return i != 0;
        throw AssetError(std::string("field \"") + what + "\" is not a boolean");
    }
    const std::string& string(const char* what) const {
        if (kind != Str) throw AssetError(std::string("field \"") + what + "\" is not a string");
        return bytes;
    }
};

constexpr int kMaxDepth = 64;

// ---------------------------------------------------------------------------
// MessagePack (big-endian lengths and scalars)
// ---------------------------------------------------------------------------

class MsgPackReader {
public:
    MsgPackReader(const uint8_t* p, size_t n) : p_(p), n_(n) {}

    Value Parse() {
        Value v = Read(0);
        if (pos_ != n_) throw AssetError("trailing bytes after the MessagePack document");
        return v;
    }

private:
    void Need(size_t k) const {
        if (k > n_ - pos_) throw AssetError("truncated MessagePack document");
    }
    uint64_t Be(int bytes) {
        Need(size_t(bytes));
        uint64_t v = 0;
        for (int k = 0; k < bytes; k++) v = (v << 8) | p_[pos_ + size_t(k)];
        pos_ += size_t(bytes);
        return v;
    }
    std::string Bytes(uint64_t len) {
        Need(len);
        std::string s(reinterpret_cast<const char*>(p_ + pos_), size_t(len));
        pos_ += size_t(len);
        return s;
    }
    Value Scalar(Value::Kind k) {
        Value v;
        v.kind = k;
        return v;
    }
    Value Array(uint64_t count, int depth) {
        Need(count);  // every element takes at least one byte
        Value v = Scalar(Value::Arr);
        v.arr.reserve(size_t(count));
        for (uint64_t k = 0; k < count; k++) v.arr.push_back(Read(depth + 1));
        return v;
    }
    Value Map(uint64_t count, int depth) {
        if (count > (n_ - pos_) / 2) throw AssetError("truncated MessagePack document");
        Value v = Scalar(Value::Map);
        v.map.reserve(size_t(count));
        for (uint64_t k = 0; k < count; k++) {
            Value key = Read(depth + 1);
            if (key.kind != Value::Str) throw AssetError("MessagePack map key is not a string");
            v.map.emplace_back(std::move(key.bytes), Read(depth + 1));
        }
        return v;
    }
    Value Ext(uint64_t len) {
        Be(1);  // the extension type: nlohmann stores a binary subtype there
        Value v = Scalar(Value::Bin);
        v.bytes = Bytes(len);
        return v;
    }

    Value Read(int depth) {
        if (depth > kMaxDepth) throw AssetError("MessagePack document nested too deeply");
        const uint8_t b = uint8_t(Be(1));
        Value v;
        if (b <= 0x7f) {
            v.kind = Value::Int;
            v.i = b;
            return v;
        }
        if (b >= 0xe0) {
            v.kind = Value::Int;
            v.i = int8_t(b);
            return v;
        }
        if ((b & 0xf0) == 0x80) return Map(b & 0x0f, depth);
        if ((b & 0xf0) == 0x90) return Array(b & 0x0f, depth);
        if ((b & 0xe0) == 0xa0) {
            v.kind = Value::Str;
            v.bytes = Bytes(b & 0x1f);
            return v;
        }
        switch (b) {
        case 0xc0: return Scalar(Value::Nil);
        case 0xc2: v.kind = Value::Bool; v.b = false; return v;
        case 0xc3: v.kind = Value::Bool; v.b = true; return v;
        case 0xc4: case 0xc5: case 0xc6: {
            const uint64_t len = Be(b == 0xc4 ? 1 : (b == 0xc5 ? 2 : 4));
            v.kind = Value::Bin;
            v.bytes = Bytes(len);
            return v;
        }
        case 0xc7: return Ext(Be(1));
        case 0xc8: return Ext(Be(2));
        case 0xc9: return Ext(Be(4));
        case 0xca: {
            const uint32_t bits = uint32_t(Be(4));
            float x;
            std::memcpy(&x, &bits, 4);
            v.kind = Value::Float;
            v.f = x;
            return v;
        }
        case 0xcb: {
            const uint64_t bits = Be(8);
            std::memcpy(&v.f, &bits, 8);
            v.kind = Value::Float;
            return v;
        }
        case 0xcc: case 0xcd: case 0xce: case 0xcf: {
            const uint64_t u = Be(1 << (b - 0xcc));
            if (u > uint64_t(INT64_MAX)) throw AssetError("MessagePack integer out of range");
            v.kind = Value::Int;
            v.i = int64_t(u);
            return v;
        }
        case 0xd0: v.kind = Value::Int; v.i = int8_t(Be(1)); return v;
        case 0xd1: v.kind = Value::Int; v.i = int16_t(Be(2)); return v;
        case 0xd2: v.kind = Value::Int; v.i = int32_t(Be(4)); return v;
        case 0xd3: v.kind = Value::Int; v.i = int64_t(Be(8)); return v;
        case 0xd4: return Ext(1);
        case 0xd5: return Ext(2);
        case 0xd6: return Ext(4);
        case 0xd7: return Ext(8);
        case 0xd8: return Ext(16);
        case 0xd9: v.kind = Value::Str; v.bytes = Bytes(Be(1)); return v;
        case 0xda: v.kind = Value::Str; v.bytes = Bytes(Be(2)); return v;
        case 0xdb: v.kind = Value::Str; v.bytes = Bytes(Be(4)); return v;
        case 0xdc: return Array(Be(2), depth);
        case 0xdd: return Array(Be(4), depth);
        case 0xde: return Map(Be(2), depth);
        case 0xdf: return Map(Be(4), depth);
        default: break;
        }
        throw AssetError("unknown MessagePack type byte " + std::to_string(int(b)));
    }

    const uint8_t* p_;
    size_t n_;
    size_t pos_ = 0;
};

// ---------------------------------------------------------------------------
// JSON text
// ---------------------------------------------------------------------------

class JsonReader {
public:
    JsonReader(const char* p, size_t n) : p_(p), n_(n) {}

    Value Parse() {
        Value v = Read(0);
        Skip();
        if (pos_ != n_) throw AssetError("trailing characters after the JSON document");
        return v;
    }

private:
    void Skip() {
        while (pos_ < n_ && (p_[pos_] == ' ' || p_[pos_] == '\t' || p_[pos_] == '\n' || p_[pos_] == '\r')) pos_++;
    }
    char Peek() {
        Skip();
        if (pos_ >= n_) throw AssetError("truncated JSON document");
        return p_[pos_];
    }
    void Expect(char c) {
        if (Peek() != c) throw AssetError(std::string("JSON: expected '") + c + "'");
        pos_++;
    }
    void Word(const char* w) {
        const size_t len = std::strlen(w);
        if (n_ - pos_ < len || std::memcmp(p_ + pos_, w, len) != 0) throw AssetError("JSON: bad literal");
        pos_ += len;
    }
    static void Utf8(uint32_t cp, std::string& out) {
        if (cp < 0x80) {
            out += char(cp);
        } else if (cp < 0x800) {
            out += char(0xc0 | (cp >> 6));
            out += char(0x80 | (cp & 0x3f));
        } else if (cp < 0x10000) {
            out += char(0xe0 | (cp >> 12));
            out += char(0x80 | ((cp >> 6) & 0x3f));
            out += char(0x80 | (cp & 0x3f));
        } else {
            out += char(0xf0 | (cp >> 18));
            out += char(0x80 | ((cp >> 12) & 0x3f));
            out += char(0x80 | ((cp >> 6) & 0x3f));
            out += char(0x80 | (cp & 0x3f));
        }
    }
    uint32_t Hex4() {
        if (n_ - pos_ < 4) throw AssetError("JSON: truncated \\u escape");
        uint32_t v = 0;
        for (int k = 0; k < 4; k++) {
            const char c = p_[pos_++];
            v <<= 4;
            if (c >= '0' && c <= '9') v |= uint32_t(c - '0');
            else if (c >= 'a' && c <= 'f') v |= uint32_t(c - 'a' + 10);
            else if (c >= 'A' && c <= 'F') v |= uint32_t(c - 'A' + 10);
            else throw AssetError("JSON: bad \\u escape");
        }
        return v;
    }
    std::string String() {
        Expect('"');
        std::string s;
        for (;;) {
            if (pos_ >= n_) throw AssetError("JSON: unterminated string");
            const char c = p_[pos_++];
            if (c == '"') return s;
            if (uint8_t(c) < 0x20) throw AssetError("JSON: control character in a string");
            if (c != '\\') {
                s += c;
                continue;
            }
            if (pos_ >= n_) throw AssetError("JSON: unterminated string");
            const char e = p_[pos_++];
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
                uint32_t cp = Hex4();
                if (cp >= 0xd800 && cp < 0xdc00 && n_ - pos_ >= 2 && p_[pos_] == '\\' && p_[pos_ + 1] == 'u') {
                    pos_ += 2;
                    const uint32_t lo = Hex4();
                    if (lo < 0xdc00 || lo >= 0xe000) throw AssetError("JSON: bad surrogate pair");
                    cp = 0x10000 + ((cp - 0xd800) << 10) + (lo - 0xdc00);
                }
                Utf8(cp, s);
                break;
            }
            default: throw AssetError("JSON: bad escape");
            }
        }
    }
    Value Number() {
        const size_t start = pos_;
        bool is_float = false;
        while (pos_ < n_) {
            const char c = p_[pos_];
            if ((c >= '0' && c <= '9') || c == '-' || c == '+') {
                pos_++;
            } else if (c == '.' || c == 'e' || c == 'E') {
                is_float = true;
                pos_++;
            } else {
                break;
            }
        }
        Value v;
        if (!is_float) {
            v.kind = Value::Int;
            const auto r = std::from_chars(p_ + start, p_ + pos_, v.i);
            if (r.ec == std::errc() && r.ptr == p_ + pos_) return v;
        }
        v.kind = Value::Float;
        const auto r = std::from_chars(p_ + start, p_ + pos_, v.f);
        if (r.ec != std::errc() || r.ptr != p_ + pos_) throw AssetError("JSON: bad number");
        return v;
    }
    Value Read(int depth) {
        if (depth > kMaxDepth) throw AssetError("JSON document nested too deeply");
        const char c = Peek();
        Value v;
        if (c == '{') {
            pos_++;
            v.kind = Value::Map;
            if (Peek() == '}') {
                pos_++;
                return v;
            }
            for (;;) {
                std::string key = String();
                Expect(':');
                v.map.emplace_back(std::move(key), Read(depth + 1));
                const char d = Peek();
                pos_++;
                if (d == '}') return v;
                if (d != ',') throw AssetError("JSON: expected ',' or '}'");
            }
        }
        if (c == '[') {
            pos_++;
            v.kind = Value::Arr;
            if (Peek() == ']') {
                pos_++;
                return v;
            }
            for (;;) {
                v.arr.push_back(Read(depth + 1));
                const char d = Peek();
                pos_++;
                if (d == ']') return v;
                if (d != ',') throw AssetError("JSON: expected ',' or ']'");
            }
        }
        if (c == '"') {
            v.kind = Value::Str;
            v.bytes = String();
            return v;
        }
        if (c == 't') {
            Word("true");
            v.kind = Value::Bool;
            v.b = true;
            return v;
        }
        if (c == 'f') {
            Word("false");
            v.kind = Value::Bool;
            return v;
        }
        if (c == 'n') {
            Word("null");
            return v;
        }
        if (c == '-' || (c >= '0' && c <= '9')) return Number();
        throw AssetError(std::string("JSON: unexpected character '") + c + "'");
    }

    const char* p_;
    size_t n_;
    size_t pos_ = 0;
};

// MessagePack documents begin with a map byte; JSON text with '{' after any
// whitespace.
Value ParseDocument(const void* bytes, size_t size) {
    if (!bytes || size == 0) throw AssetError("empty document");
    const auto* p = static_cast<const uint8_t*>(bytes);
    size_t k = 0;
    while (k < size && (p[k] == ' ' || p[k] == '\t' || p[k] == '\n' || p[k] == '\r')) k++;
    if (k < size && p[k] == '{') return JsonReader(reinterpret_cast<const char*>(p), size).Parse();
    return MsgPackReader(p, size).Parse();
}

std::string ReadFile(const char* path) {
    std::ifstream f(path, std::ios::binary);
    if (!f) throw AssetError(std::string("cannot open ") + path);
    return std::string(std::istreambuf_iterator<char>(f), std::istreambuf_iterator<char>());
}

// glm vec3 / AABB as the serialisation helpers write them
// (common/SerializationHelper.cpp:51-61, :141-150): {"x","y","z"}, {"min","max"}.
void Vec3(const Value& v, const char* what, float out[3]) {
    const char* keys[3] = { "x", "y", "z" };
    for (int c = 0; c < 3; c++) {
        const Value* e = v.find(keys[c]);
        if (!e || !e->is_number()) throw AssetError(std::string("field \"") + what + "\" is not a vec3");
        out[c] = float(e->number(what));
    }
}

void Aabb(const Value& v, const char* what, float out[6]) {
    Vec3(v.at("min"), what, out);
    Vec3(v.at("max"), what, out + 3);
}

// DataComponent<T> (MeshSerializer.h:29-72): {"format": int, "data": bytes},
// the bytes a MessagePack bin, a JSON array of byte values, or nlohmann's
// JSON form of a binary value ({"bytes": [...], "subtype": ...}).
std::string ComponentBytes(const Value& c, const char* what) {
    const Value& d = c.at("data");
    if (d.kind == Value::Bin) return d.bytes;
    const Value* arr = &d;
    if (d.kind == Value::Map) arr = &d.at("bytes");
    if (arr->kind != Value::Arr) throw AssetError(std::string("component \"") + what + "\" has no byte data");
    std::string out(arr->arr.size(), '\0');
    for (size_t k = 0; k < arr->arr.size(); k++) {
        const Value& e = arr->arr[k];
        if (e.kind != Value::Int || e.i < 0 || e.i > 255)
            throw AssetError(std::string("component \"") + what + "\" holds a non-byte value");
        out[k] = char(uint8_t(e.i));
    }
    return out;
}

template <class T>
std::vector<T> Component(const Value& data, const char* key, size_t width) {
    const std::string bytes = ComponentBytes(data.at(key), key);
    const size_t elem = sizeof(T) * width;
    if (bytes.size() % elem)
        throw AssetError(std::string("component \"") + key + "\" is not a whole number of elements");
    std::vector<T> out(bytes.size() / sizeof(T));
    if (!bytes.empty()) std::memcpy(out.data(), bytes.data(), bytes.size());
    return out;
}

ae_rt_status Fail(const std::string& msg) {
    g_asset_error = msg;
    return AE_RT_INVALID_ARG;
}

}  // namespace

struct ae_mesh_asset {
    std::string name;
    int32_t mobility = 0, usage = 0, cull_back_faces = 0, cast_shadow = 0, invert_uvs = 0, primitive_type = 0;
    float radius = 0.0f;
    float aabb[6] = {};
    uint32_t vertex_count = 0, index_count = 0;
    std::vector<uint32_t> indices;
    std::vector<float> vertices, tex_coords, normals, tangents, colors;  // 3, 2, 4, 4, 4 floats per vertex
    struct Sub {
        std::string name;
        uint32_t offset = 0, count = 0;
        int32_t material = 0;
        float aabb[6] = {};
    };
    std::vector<Sub> subs;
    std::vector<std::string> materials;
    uint32_t triangle_count = 0;
};

struct ae_material_asset {
    std::string name;
    float baseColor[3] = { 1, 1, 1 }, transmissiveColor[3] = {}, emissiveColor[3] = {};
    float emissiveIntensity = 1, opacity = 1, roughness = 1, metalness = 0, ao = 1, reflectance = 0.5f;
    float normalScale = 1, displacementScale = 0, tiling = 1;
    int32_t twoSided = 0, vertexColors = 0, uvChannel = 0;
    std::string maps[7];  // AE_MAP_* order
};

namespace {

const char* const kMapKeys[7] = { "baseColorMapPath", "opacityMapPath", "normalMapPath", "roughnessMapPath",
                                  "metalnessMapPath", "aoMapPath", "displacementMapPath" };

// Mesh::from_json + MeshData::from_json (MeshSerializer.cpp:32-134).
void ReadMesh(const Value& j, ae_mesh_asset& m) {
    m.name = j.at("name").string("name");
    if (const Value* v = j.find("mobility")) m.mobility = int32_t(v->integer("mobility"));
    if (const Value* v = j.find("usage")) m.usage = int32_t(v->integer("usage"));
    if (const Value* v = j.find("castShadow")) m.cast_shadow = v->boolean("castShadow") ? 1 : 0;
    m.cull_back_faces = j.at("cullBackFaces").boolean("cullBackFaces") ? 1 : 0;
    m.invert_uvs = j.at("invertUVs").boolean("invertUVs") ? 1 : 0;
    const Value& d = j.at("data");
    const int64_t ic = d.at("indexCount").integer("indexCount");
    const int64_t vc = d.at("vertexCount").integer("vertexCount");
    if (ic < 0 || vc < 0 || ic > INT32_MAX || vc > INT32_MAX) throw AssetError("negative or huge element counts");
    m.index_count = uint32_t(ic);
    m.vertex_count = uint32_t(vc);
    m.primitive_type = int32_t(d.at("primitiveType").integer("primitiveType"));
    m.radius = float(d.at("radius").number("radius"));
    Aabb(d.at("aabb"), "aabb", m.aabb);
    m.indices = Component<uint32_t>(d, "indices", 1);
    m.vertices = Component<float>(d, "vertices", 3);
    m.tex_coords = Component<float>(d, "texCoords", 2);
    m.normals = Component<float>(d, "normals", 4);
    m.tangents = Component<float>(d, "tangents", 4);
    m.colors = Component<float>(d, "colors", 4);
    const Value& subs = d.at("subData");
    if (subs.kind != Value::Arr) throw AssetError("field \"subData\" is not an array");
    uint64_t tris = 0;
    for (const Value& s : subs.arr) {
        ae_mesh_asset::Sub sub;
        if (const Value* v = s.find("name")) sub.name = v->kind == Value::Str ? v->bytes : std::string();
        const int64_t off = s.at("indicesOffset").integer("indicesOffset");
        const int64_t cnt = s.at("indicesCount").integer("indicesCount");
        if (off < 0 || cnt < 0 || off > UINT32_MAX || cnt > UINT32_MAX) throw AssetError("bad subData range");
        sub.offset = uint32_t(off);
        sub.count = uint32_t(cnt);
        sub.material = int32_t(s.at("materialIdx").integer("materialIdx"));
        Aabb(s.at("aabb"), "subData.aabb", sub.aabb);
        tris += sub.count / 3;
        m.subs.push_back(std::move(sub));
    }
    if (tris > UINT32_MAX / 3) throw AssetError("too many triangles");
    m.triangle_count = uint32_t(tris);
    if (const Value* mats = d.find("materials")) {
        if (mats->kind != Value::Arr) throw AssetError("field \"materials\" is not an array");
        for (const Value& p : mats->arr) m.materials.push_back(p.string("materials"));
    }
}

// Material from_json (MeshSerializer.cpp:212-256).
void ReadMaterial(const Value& j, ae_material_asset& m) {
    m.name = j.at("name").string("name");
    Vec3(j.at("baseColor"), "baseColor", m.baseColor);
    Vec3(j.at("transmissiveColor"), "transmissiveColor", m.transmissiveColor);
    Vec3(j.at("emissiveColor"), "emissiveColor", m.emissiveColor);
    m.emissiveIntensity = float(j.at("emissiveIntensity").number("emissiveIntensity"));
    m.opacity = float(j.at("opacity").number("opacity"));
    m.roughness = float(j.at("roughness").number("roughness"));
    m.metalness = float(j.at("metalness").number("metalness"));
    m.ao = float(j.at("ao").number("ao"));
    m.reflectance = float(j.at("reflectance").number("reflectance"));
    m.normalScale = float(j.at("normalScale").number("normalScale"));
    m.displacementScale = float(j.at("displacementScale").number("displacementScale"));
    m.tiling = float(j.at("tiling").number("tiling"));
    m.twoSided = j.at("twoSided").boolean("twoSided") ? 1 : 0;
    m.vertexColors = j.at("vertexColors").boolean("vertexColors") ? 1 : 0;
    m.uvChannel = int32_t(j.at("uvChannel").integer("uvChannel"));
    for (int k = 0; k < 7; k++)
        if (const Value* v = j.find(kMapKeys[k])) m.maps[k] = v->string(kMapKeys[k]);
}

}  // namespace

extern "C" {

const char* ae_asset_last_error(void) { return g_asset_error.c_str(); }

ae_rt_status ae_mesh_asset_load(const void* bytes, size_t size, ae_mesh_asset** out) {
    if (!out) return Fail("null output handle");
    *out = nullptr;
    try {
        auto m = std::make_unique<ae_mesh_asset>();
        ReadMesh(ParseDocument(bytes, size), *m);
        *out = m.release();
        g_asset_error.clear();
        return AE_RT_OK;
    } catch (const AssetError& e) {
        return Fail(std::string("mesh asset: ") + e.what());
    } catch (const std::bad_alloc&) {
        g_asset_error = "mesh asset: out of memory";
        return AE_RT_OUT_OF_MEMORY;
    }
}

ae_rt_status ae_mesh_asset_load_file(const char* path, ae_mesh_asset** out) {
    if (!path || !out) return Fail("null path or output handle");
    try {
        const std::string data = ReadFile(path);
        return ae_mesh_asset_load(data.data(), data.size(), out);
    } catch (const AssetError& e) {
        return Fail(e.what());
    }
}

void ae_mesh_asset_destroy(ae_mesh_asset* a) { delete a; }

ae_rt_status ae_mesh_asset_get_info(const ae_mesh_asset* a, ae_mesh_asset_info* info) {
    if (!a || !info) return Fail("null argument");
    std::memset(info, 0, sizeof(*info));
    info->vertex_count = uint32_t(a->vertices.size() / 3);
    info->index_count = uint32_t(a->indices.size());
    info->triangle_count = a->triangle_count;
    info->sub_count = uint32_t(a->subs.size());
    info->material_count = uint32_t(a->materials.size());
    info->tex_coord_count = uint32_t(a->tex_coords.size() / 2);
    info->normal_count = uint32_t(a->normals.size() / 4);
    info->tangent_count = uint32_t(a->tangents.size() / 4);
    info->color_count = uint32_t(a->colors.size() / 4);
    info->cull_back_faces = a->cull_back_faces;
    info->invert_uvs = a->invert_uvs;
    info->cast_shadow = a->cast_shadow;
    info->primitive_type = a->primitive_type;
    info->mobility = a->mobility;
    info->usage = a->usage;
    info->radius = a->radius;
    std::memcpy(info->aabb, a->aabb, sizeof(info->aabb));
    return AE_RT_OK;
}

const char* ae_mesh_asset_name(const ae_mesh_asset* a) { return a ? a->name.c_str() : ""; }

const char* ae_mesh_asset_material_path(const ae_mesh_asset* a, uint32_t i) {
    return a && i < a->materials.size() ? a->materials[i].c_str() : nullptr;
}

ae_rt_status ae_mesh_asset_get_sub(const ae_mesh_asset* a, uint32_t i, ae_mesh_sub* out) {
    if (!a || !out) return Fail("null argument");
    if (i >= a->subs.size()) return Fail("sub-mesh index out of range");
    out->indices_offset = a->subs[i].offset;
    out->indices_count = a->subs[i].count;
    out->material_idx = a->subs[i].material;
    std::memcpy(out->aabb, a->subs[i].aabb, sizeof(out->aabb));
    return AE_RT_OK;
}

ae_rt_status ae_mesh_asset_get_arrays(const ae_mesh_asset* a, uint32_t* indices, float* vertices, float* tex_coords,
                                      float* normals, float* tangents, float* colors) {
    if (!a) return Fail("null asset");
    auto copy = [](void* dst, const void* src, size_t bytes) {
        if (dst && bytes) std::memcpy(dst, src, bytes);
    };
    copy(indices, a->indices.data(), a->indices.size() * 4);
    copy(vertices, a->vertices.data(), a->vertices.size() * 4);
    copy(tex_coords, a->tex_coords.data(), a->tex_coords.size() * 4);
    copy(normals, a->normals.data(), a->normals.size() * 4);
    copy(tangents, a->tangents.data(), a->tangents.size() * 4);
    copy(colors, a->colors.data(), a->colors.size() * 4);
    return AE_RT_OK;
}

ae_rt_status ae_mesh_asset_triangles(const ae_mesh_asset* a, const ae_material* materials, uint32_t n_materials,
                                     float* verts, float* normals, float* uvs, float* colors, int32_t* material,
                                     float* opacity) {
    if (!a) return Fail("null asset");
    if (materials == nullptr && n_materials) return Fail("null material table");
    const size_t n_vert = a->vertices.size() / 3;
    const size_t n_nrm = a->normals.size() / 4, n_uv = a->tex_coords.size() / 2, n_col = a->colors.size() / 4;
    if (size_t(a->triangle_count) * 3 > a->indices.size())
        return Fail("the sub-meshes name " + std::to_string(a->triangle_count) + " triangles but the index buffer holds " +
                    std::to_string(a->indices.size()) + " indices");
    // materials are checked before anything is written
    for (const auto& s : a->subs)
        if (materials && s.count >= 3 && (s.material < 0 || uint32_t(s.material) >= n_materials))
            return Fail("sub-mesh material index " + std::to_string(s.material) + " out of range");
    for (size_t k = 0; k < size_t(a->triangle_count) * 3; k++) {
        const uint32_t idx = a->indices[k];
        if (idx >= n_vert) return Fail("index " + std::to_string(idx) + " out of range of the vertex buffer");
        if (n_nrm && idx >= n_nrm) return Fail("index out of range of the normal buffer");
        if (n_uv && idx >= n_uv) return Fail("index out of range of the texture-coordinate buffer");
        if (n_col && idx >= n_col) return Fail("index out of range of the colour buffer");
    }
    uint32_t k = 0;
    for (const auto& s : a->subs) {
        const uint32_t count = s.count / 3;
        for (uint32_t i = 0; i < count; i++, k++) {
            for (int c = 0; c < 3; c++) {
                const uint32_t idx = a->indices[size_t(k) * 3 + size_t(c)];
                if (verts)
                    for (int e = 0; e < 3; e++) verts[size_t(k) * 9 + size_t(c) * 3 + size_t(e)] = a->vertices[size_t(idx) * 3 + size_t(e)];
                if (normals)
                    for (int e = 0; e < 3; e++)
                        normals[size_t(k) * 9 + size_t(c) * 3 + size_t(e)] = n_nrm ? a->normals[size_t(idx) * 4 + size_t(e)] : 0.0f;
                if (uvs)
                    for (int e = 0; e < 2; e++)
                        uvs[size_t(k) * 6 + size_t(c) * 2 + size_t(e)] = n_uv ? a->tex_coords[size_t(idx) * 2 + size_t(e)] : 0.0f;
                if (colors)
                    for (int e = 0; e < 4; e++)
                        colors[size_t(k) * 12 + size_t(c) * 4 + size_t(e)] = n_col ? a->colors[size_t(idx) * 4 + size_t(e)] : 1.0f;
            }
            if (material) material[k] = s.material;
            if (opacity) {
                float o = 1.0f;
                if (materials) {
                    const ae_material& m = materials[s.material];
                    o = m.opacityTexture >= 0 ? -1.0f : m.opacity;
                }
                opacity[k] = o;
            }
        }
    }
    return AE_RT_OK;
}

ae_rt_status ae_material_asset_load(const void* bytes, size_t size, ae_material_asset** out) {
    if (!out) return Fail("null output handle");
    *out = nullptr;
    try {
        auto m = std::make_unique<ae_material_asset>();
        ReadMaterial(ParseDocument(bytes, size), *m);
        *out = m.release();
        g_asset_error.clear();
        return AE_RT_OK;
    } catch (const AssetError& e) {
        return Fail(std::string("material asset: ") + e.what());
    } catch (const std::bad_alloc&) {
        g_asset_error = "material asset: out of memory";
        return AE_RT_OUT_OF_MEMORY;
    }
}

ae_rt_status ae_material_asset_load_file(const char* path, ae_material_asset** out) {
    if (!path || !out) return Fail("null path or output handle");
    try {
        const std::string data = ReadFile(path);
        return ae_material_asset_load(data.data(), data.size(), out);
    } catch (const AssetError& e) {
        return Fail(e.what());
    }
}

void ae_material_asset_destroy(ae_material_asset* m) { delete m; }

const char* ae_material_asset_name(const ae_material_asset* m) { return m ? m->name.c_str() : ""; }

const char* ae_material_asset_map_path(const ae_material_asset* m, uint32_t which) {
    return m && which < 7 ? m->maps[which].c_str() : "";
}

ae_rt_status ae_material_asset_get_emissive(const ae_material_asset* m, float srgb[3], float* intensity) {
    if (!m || !srgb || !intensity) return Fail("null argument");
    std::memcpy(srgb, m->emissiveColor, sizeof(m->emissiveColor));
    *intensity = m->emissiveIntensity;
    return AE_RT_OK;
}

ae_rt_status ae_material_asset_to_gpu(const ae_material_asset* m, const ae_mesh_asset* mesh,
                                      const int32_t* texture_ids, int32_t id, ae_material* out) {
    if (!m || !out) return Fail("null argument");
    std::memset(out, 0, sizeof(*out));
    out->ID = id;
    for (int c = 0; c < 3; c++) {
        // ColorConverter::ConvertSRGBToLinear (common/ColorConverter.h:18-23): pow(c, 2.2)
        out->baseColor[c] = std::pow(m->baseColor[c], 2.2f);
        out->emissiveColor[c] = std::pow(m->emissiveColor[c], 2.2f) * m->emissiveIntensity;
    }
    out->opacity = m->opacity;
    out->roughness = m->roughness;
    out->metalness = m->metalness;
    out->ao = m->ao;
    out->reflectance = m->reflectance;
    out->normalScale = m->normalScale;
    out->invertUVs = mesh ? mesh->invert_uvs : 0;
    out->twoSided = m->twoSided;
    out->cullBackFaces = mesh ? mesh->cull_back_faces : 0;
    out->useVertexColors = m->vertexColors;
    int32_t* tex[6] = { &out->baseColorTexture, &out->opacityTexture, &out->normalTexture, &out->roughnessTexture,
                        &out->metalnessTexture, &out->aoTexture };
    for (int k = 0; k < 6; k++)
        *tex[k] = (!m->maps[k].empty() && texture_ids && texture_ids[k] >= 0) ? texture_ids[k] : -1;
    return AE_RT_OK;
}

}  // extern "C"
