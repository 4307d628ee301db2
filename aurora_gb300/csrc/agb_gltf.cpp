// glTF 2.0 scene loading and camera saving for the headless renderer (declarations and provenance
// in include/aurora_gb300_loaders.hpp).  The container handling restates what the reference takes
// from tinygltf: JSON text, binary .glb (12-byte header, JSON chunk, optional BIN chunk that backs a
// buffer without a uri), buffers from base64 data URIs or files beside the glTF file, accessors
// read through their buffer views (byteOffset, byteStride), node matrix or TRS.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <map>
#include <memory>
#include <sstream>

#include "../../include/aurora_gb300_loaders.hpp"

namespace agb_aurora
{
namespace
{

// ------------------------------------------------------------------------------------- JSON
struct Json
{
    enum Kind
    {
        Null,
        Bool,
        Number,
        String,
        Array,
        Object
    };
    Kind kind     = Null;
    bool b        = false;
    double n      = 0.0;
    std::string s;
    std::vector<Json> a;
    std::map<std::string, Json> o;

    const Json* get(const std::string& key) const
    {
        if (kind != Object)
            return nullptr;
        auto it = o.find(key);
        return it == o.end() ? nullptr : &it->second;
    }
    double num(const std::string& key, double def) const
    {
        const Json* v = get(key);
        return v && v->kind == Number ? v->n : def;
    }
    int integer(const std::string& key, int def) const
    {
        const Json* v = get(key);
        return v && v->kind == Number ? int(v->n) : def;
    }
    std::string str(const std::string& key) const
    {
        const Json* v = get(key);
        return v && v->kind == String ? v->s : std::string();
    }
    const std::vector<Json>& arr(const std::string& key) const
    {
        static const std::vector<Json> kEmpty;
        const Json* v = get(key);
        return v && v->kind == Array ? v->a : kEmpty;
    }
};

class JsonParser
{
public:
    JsonParser(const char* p, const char* end) : p_(p), end_(end) {}
    bool parse(Json& out, std::string& error)
    {
        if (!value(out, 0))
        {
            error = "invalid JSON near byte " + std::to_string(size_t(p_ - begin_)) + ": " + error_;
            return false;
        }
        ws();
        if (p_ != end_)
        {
            error = "trailing characters after the JSON document";
            return false;
        }
        return true;
    }
    void setBegin(const char* b) { begin_ = b; }

private:
    const char* p_;
    const char* end_;
    const char* begin_ = p_;
    std::string error_;

    void ws()
    {
        while (p_ < end_ && (*p_ == ' ' || *p_ == '\t' || *p_ == '\n' || *p_ == '\r'))
            p_++;
    }
    bool fail(const char* what)
    {
        error_ = what;
        return false;
    }
    bool literal(const char* word)
    {
        size_t n = std::strlen(word);
        if (size_t(end_ - p_) < n || std::memcmp(p_, word, n) != 0)
            return fail("unknown literal");
        p_ += n;
        return true;
    }
    static void utf8(uint32_t c, std::string& out)
    {
        if (c < 0x80)
            out += char(c);
        else if (c < 0x800)
        {
            out += char(0xC0 | (c >> 6));
            out += char(0x80 | (c & 0x3F));
        }
        else if (c < 0x10000)
        {
            out += char(0xE0 | (c >> 12));
            out += char(0x80 | ((c >> 6) & 0x3F));
            out += char(0x80 | (c & 0x3F));
        }
        else
        {
            out += char(0xF0 | (c >> 18));
            out += char(0x80 | ((c >> 12) & 0x3F));
            out += char(0x80 | ((c >> 6) & 0x3F));
            out += char(0x80 | (c & 0x3F));
        }
    }
    bool hex4(uint32_t& v)
    {
        if (end_ - p_ < 4)
            return fail("short \\u escape");
        v = 0;
        for (int k = 0; k < 4; k++)
        {
            char c = *p_++;
            v <<= 4;
            if (c >= '0' && c <= '9')
                v |= uint32_t(c - '0');
            else if (c >= 'a' && c <= 'f')
                v |= uint32_t(c - 'a' + 10);
            else if (c >= 'A' && c <= 'F')
                v |= uint32_t(c - 'A' + 10);
            else
                return fail("bad \\u escape");
        }
        return true;
    }
    bool string(std::string& out)
    {
        p_++; // opening quote
        while (p_ < end_ && *p_ != '"')
        {
            char c = *p_++;
            if (c != '\\')
            {
                out += c;
                continue;
            }
            if (p_ >= end_)
                return fail("unterminated escape");
            char e = *p_++;
            switch (e)
            {
            case '"': out += '"'; break;
            case '\\': out += '\\'; break;
            case '/': out += '/'; break;
            case 'b': out += '\b'; break;
            case 'f': out += '\f'; break;
            case 'n': out += '\n'; break;
            case 'r': out += '\r'; break;
            case 't': out += '\t'; break;
            case 'u':
            {
                uint32_t c1;
                if (!hex4(c1))
                    return false;
                if (c1 >= 0xD800 && c1 < 0xDC00 && end_ - p_ >= 6 && p_[0] == '\\' && p_[1] == 'u')
                {
                    p_ += 2;
                    uint32_t c2;
                    if (!hex4(c2))
                        return false;
                    c1 = 0x10000 + ((c1 - 0xD800) << 10) + (c2 - 0xDC00);
                }
                utf8(c1, out);
                break;
            }
            default: return fail("bad escape");
            }
        }
        if (p_ >= end_)
            return fail("unterminated string");
        p_++;
        return true;
    }
    bool value(Json& v, int depth)
    {
        if (depth > 256)
            return fail("nesting too deep");
        ws();
        if (p_ >= end_)
            return fail("unexpected end");
        char c = *p_;
        if (c == '{')
        {
            v.kind = Json::Object;
            p_++;
            ws();
            if (p_ < end_ && *p_ == '}')
            {
                p_++;
                return true;
            }
            for (;;)
            {
                ws();
                if (p_ >= end_ || *p_ != '"')
                    return fail("expected a key");
                std::string key;
                if (!string(key))
                    return false;
                ws();
                if (p_ >= end_ || *p_ != ':')
                    return fail("expected ':'");
                p_++;
                if (!value(v.o[key], depth + 1))
                    return false;
                ws();
                if (p_ < end_ && *p_ == ',')
                {
                    p_++;
                    continue;
                }
                if (p_ < end_ && *p_ == '}')
                {
                    p_++;
                    return true;
                }
                return fail("expected ',' or '}'");
            }
        }
        if (c == '[')
        {
            v.kind = Json::Array;
            p_++;
            ws();
            if (p_ < end_ && *p_ == ']')
            {
                p_++;
                return true;
            }
            for (;;)
            {
                v.a.emplace_back();
                if (!value(v.a.back(), depth + 1))
                    return false;
                ws();
                if (p_ < end_ && *p_ == ',')
                {
                    p_++;
                    continue;
                }
                if (p_ < end_ && *p_ == ']')
                {
                    p_++;
                    return true;
                }
                return fail("expected ',' or ']'");
            }
        }
        if (c == '"')
        {
            v.kind = Json::String;
            return string(v.s);
        }
        if (c == 't' || c == 'f')
        {
            v.kind = Json::Bool;
            v.b    = c == 't';
            return literal(v.b ? "true" : "false");
        }
        if (c == 'n')
        {
            v.kind = Json::Null;
            return literal("null");
        }
        // Number: strtod on a bounded copy (the text need not be NUL-terminated).
        const char* q = p_;
        while (q < end_ && (std::strchr("+-0123456789.eE", *q) != nullptr))
            q++;
        if (q == p_)
            return fail("unexpected character");
        std::string num(p_, q);
        char* stop = nullptr;
        v.kind     = Json::Number;
        v.n        = std::strtod(num.c_str(), &stop);
        if (!stop || *stop != '\0')
            return fail("bad number");
        p_ = q;
        return true;
    }
};

// ---------------------------------------------------------------------------- file helpers
bool readFile(const std::string& path, std::string& out)
{
    std::ifstream f(path, std::ios::binary);
    if (!f)
        return false;
    std::ostringstream s;
    s << f.rdbuf();
    out = s.str();
    return true;
}

std::string dirOf(const std::string& path)
{
    size_t k = path.find_last_of("/\\");
    return k == std::string::npos ? std::string() : path.substr(0, k + 1);
}

// %XX escapes of a relative uri.
std::string uriDecode(const std::string& u)
{
    std::string out;
    for (size_t i = 0; i < u.size(); i++)
    {
        if (u[i] == '%' && i + 2 < u.size())
        {
            char h[3] = { u[i + 1], u[i + 2], 0 };
            char* end = nullptr;
            long v    = std::strtol(h, &end, 16);
            if (end == h + 2)
            {
                out += char(v);
                i += 2;
                continue;
            }
        }
        out += u[i];
    }
    return out;
}

bool base64(const std::string& in, size_t start, std::string& out)
{
    auto val = [](char c) -> int {
        if (c >= 'A' && c <= 'Z')
            return c - 'A';
        if (c >= 'a' && c <= 'z')
            return c - 'a' + 26;
        if (c >= '0' && c <= '9')
            return c - '0' + 52;
        if (c == '+' || c == '-')
            return 62;
        if (c == '/' || c == '_')
            return 63;
        return -1;
    };
    uint32_t acc = 0;
    int bits     = 0;
    for (size_t i = start; i < in.size(); i++)
    {
        char c = in[i];
        if (c == '=')
            break;
        int v = val(c);
        if (v < 0)
            return false;
        acc = (acc << 6) | uint32_t(v);
        bits += 6;
        if (bits >= 8)
        {
            bits -= 8;
            out += char((acc >> bits) & 0xFF);
        }
    }
    return true;
}

uint32_t le32(const std::string& s, size_t at)
{
    uint32_t v;
    std::memcpy(&v, s.data() + at, 4);
    return v;
}

// ------------------------------------------------------------------------------- transforms
// Column-major 4x4 product in glm's order: column c = A[0] B[c][0] + A[1] B[c][1] + ...
mat4 mul(const mat4& A, const mat4& B)
{
    mat4 r{};
    for (int c = 0; c < 4; c++)
        for (int row = 0; row < 4; row++)
            r[c * 4 + row] = A[0 * 4 + row] * B[c * 4 + 0] + A[1 * 4 + row] * B[c * 4 + 1] +
                A[2 * 4 + row] * B[c * 4 + 2] + A[3 * 4 + row] * B[c * 4 + 3];
    return r;
}

// General inverse by cofactors (FP64, rounded to FP32); false when singular.
bool invert(const mat4& m, mat4& out)
{
    double a[16], inv[16];
    for (int k = 0; k < 16; k++)
        a[k] = m[k];
    inv[0] = a[5] * a[10] * a[15] - a[5] * a[11] * a[14] - a[9] * a[6] * a[15] + a[9] * a[7] * a[14] +
        a[13] * a[6] * a[11] - a[13] * a[7] * a[10];
    inv[4] = -a[4] * a[10] * a[15] + a[4] * a[11] * a[14] + a[8] * a[6] * a[15] - a[8] * a[7] * a[14] -
        a[12] * a[6] * a[11] + a[12] * a[7] * a[10];
    inv[8] = a[4] * a[9] * a[15] - a[4] * a[11] * a[13] - a[8] * a[5] * a[15] + a[8] * a[7] * a[13] +
        a[12] * a[5] * a[11] - a[12] * a[7] * a[9];
    inv[12] = -a[4] * a[9] * a[14] + a[4] * a[10] * a[13] + a[8] * a[5] * a[14] - a[8] * a[6] * a[13] -
        a[12] * a[5] * a[10] + a[12] * a[6] * a[9];
    inv[1] = -a[1] * a[10] * a[15] + a[1] * a[11] * a[14] + a[9] * a[2] * a[15] - a[9] * a[3] * a[14] -
        a[13] * a[2] * a[11] + a[13] * a[3] * a[10];
    inv[5] = a[0] * a[10] * a[15] - a[0] * a[11] * a[14] - a[8] * a[2] * a[15] + a[8] * a[3] * a[14] +
        a[12] * a[2] * a[11] - a[12] * a[3] * a[10];
    inv[9] = -a[0] * a[9] * a[15] + a[0] * a[11] * a[13] + a[8] * a[1] * a[15] - a[8] * a[3] * a[13] -
        a[12] * a[1] * a[11] + a[12] * a[3] * a[9];
    inv[13] = a[0] * a[9] * a[14] - a[0] * a[10] * a[13] - a[8] * a[1] * a[14] + a[8] * a[2] * a[13] +
        a[12] * a[1] * a[10] - a[12] * a[2] * a[9];
    inv[2] = a[1] * a[6] * a[15] - a[1] * a[7] * a[14] - a[5] * a[2] * a[15] + a[5] * a[3] * a[14] +
        a[13] * a[2] * a[7] - a[13] * a[3] * a[6];
    inv[6] = -a[0] * a[6] * a[15] + a[0] * a[7] * a[14] + a[4] * a[2] * a[15] - a[4] * a[3] * a[14] -
        a[12] * a[2] * a[7] + a[12] * a[3] * a[6];
    inv[10] = a[0] * a[5] * a[15] - a[0] * a[7] * a[13] - a[4] * a[1] * a[15] + a[4] * a[3] * a[13] +
        a[12] * a[1] * a[7] - a[12] * a[3] * a[5];
    inv[14] = -a[0] * a[5] * a[14] + a[0] * a[6] * a[13] + a[4] * a[1] * a[14] - a[4] * a[2] * a[13] -
        a[12] * a[1] * a[6] + a[12] * a[2] * a[5];
    inv[3] = -a[1] * a[6] * a[11] + a[1] * a[7] * a[10] + a[5] * a[2] * a[11] - a[5] * a[3] * a[10] -
        a[9] * a[2] * a[7] + a[9] * a[3] * a[6];
    inv[7] = a[0] * a[6] * a[11] - a[0] * a[7] * a[10] - a[4] * a[2] * a[11] + a[4] * a[3] * a[10] +
        a[8] * a[2] * a[7] - a[8] * a[3] * a[6];
    inv[11] = -a[0] * a[5] * a[11] + a[0] * a[7] * a[9] + a[4] * a[1] * a[11] - a[4] * a[3] * a[9] -
        a[8] * a[1] * a[7] + a[8] * a[3] * a[5];
    inv[15] = a[0] * a[5] * a[10] - a[0] * a[6] * a[9] - a[4] * a[1] * a[10] + a[4] * a[2] * a[9] +
        a[8] * a[1] * a[6] - a[8] * a[2] * a[5];
    double det = a[0] * inv[0] + a[1] * inv[4] + a[2] * inv[8] + a[3] * inv[12];
    if (det == 0.0 || !std::isfinite(det))
        return false;
    for (int k = 0; k < 16; k++)
        out[k] = float(inv[k] / det);
    return true;
}

// getNodeTransform (glTFLoader.cpp:26-54): the node's matrix, else translate * rotate * scale.
// With unit axes and zero off-diagonals the product T R S is exactly [R0 sx, R1 sy, R2 sz, t].
mat4 nodeTransform(const Json& node)
{
    const std::vector<Json>& m = node.arr("matrix");
    if (m.size() == 16)
    {
        mat4 r{};
        for (int k = 0; k < 16; k++)
            r[k] = float(m[k].n);
        return r;
    }
    float t[3] = { 0.f, 0.f, 0.f }, s[3] = { 1.f, 1.f, 1.f };
    float q[4] = { 0.f, 0.f, 0.f, 1.f }; // x y z w
    const std::vector<Json>& tj = node.arr("translation");
    const std::vector<Json>& rj = node.arr("rotation");
    const std::vector<Json>& sj = node.arr("scale");
    if (tj.size() == 3)
        for (int k = 0; k < 3; k++)
            t[k] = float(tj[k].n);
    if (rj.size() == 4)
        for (int k = 0; k < 4; k++)
            q[k] = float(rj[k].n);
    if (sj.size() == 3)
        for (int k = 0; k < 3; k++)
            s[k] = float(sj[k].n);
    // Rotation matrix of the unit quaternion (x, y, z, w), columns R0 R1 R2.
    float x = q[0], y = q[1], z = q[2], w = q[3];
    float xx = x * x, yy = y * y, zz = z * z, xz = x * z, xy = x * y, yz = y * z;
    float wx = w * x, wy = w * y, wz = w * z;
    float R[3][3] = { { 1.f - 2.f * (yy + zz), 2.f * (xy + wz), 2.f * (xz - wy) },
        { 2.f * (xy - wz), 1.f - 2.f * (xx + zz), 2.f * (yz + wx) },
        { 2.f * (xz + wy), 2.f * (yz - wx), 1.f - 2.f * (xx + yy) } };
    mat4 r{};
    for (int c = 0; c < 3; c++)
        for (int row = 0; row < 3; row++)
            r[c * 4 + row] = R[c][row] * s[c];
    r[12] = t[0];
    r[13] = t[1];
    r[14] = t[2];
    r[15] = 1.f;
    return r;
}

// -------------------------------------------------------------------------------- the model
enum : int
{
    kByte = 5120,
    kUnsignedByte,
    kShort,
    kUnsignedShort,
    kUnsignedInt = 5125,
    kFloat
};

struct Model
{
    Json doc;
    std::vector<std::string> buffers;
    std::string filePath;
    std::string warnings;

    int components(const std::string& type) const
    {
        if (type == "SCALAR")
            return 1;
        if (type == "VEC2")
            return 2;
        if (type == "VEC3")
            return 3;
        if (type == "VEC4" || type == "MAT2")
            return 4;
        if (type == "MAT3")
            return 9;
        if (type == "MAT4")
            return 16;
        return 0;
    }

    // The bytes of an accessor: base pointer, element stride, count; false when it does not fit
    // its buffer.
    bool view(int accessor, int elementSize, const uint8_t*& base, size_t& stride, size_t& count,
        const Json*& acc) const
    {
        const std::vector<Json>& accs = doc.arr("accessors");
        if (accessor < 0 || size_t(accessor) >= accs.size())
            return false;
        acc = &accs[size_t(accessor)];
        // Sizes as JSON numbers: refuse negative or absurd values before converting them.
        auto size = [](double v, size_t& out) {
            if (!(v >= 0.0 && v <= 4294967295.0))
                return false;
            out = size_t(v);
            return true;
        };
        if (!size(acc->num("count", 0), count))
            return false;
        int bvIdx = acc->integer("bufferView", -1);
        const std::vector<Json>& views = doc.arr("bufferViews");
        if (bvIdx < 0 || size_t(bvIdx) >= views.size())
            return false;
        const Json& bv = views[size_t(bvIdx)];
        int bIdx       = bv.integer("buffer", -1);
        if (bIdx < 0 || size_t(bIdx) >= buffers.size())
            return false;
        const std::string& buf = buffers[size_t(bIdx)];
        size_t bvOffset, bvLength, accOffset;
        if (!size(bv.num("byteOffset", 0), bvOffset) || !size(bv.num("byteLength", 0), bvLength) ||
            !size(acc->num("byteOffset", 0), accOffset) || !size(bv.num("byteStride", 0), stride))
            return false;
        if (!stride)
            stride = size_t(elementSize);
        if (bvOffset + bvLength > buf.size() || bvOffset + bvLength < bvOffset)
            return false;
        if (count && accOffset + (count - 1) * stride + size_t(elementSize) > bvLength)
            return false;
        base = reinterpret_cast<const uint8_t*>(buf.data()) + bvOffset + accOffset;
        return true;
    }

    // decodeFloatAccessor (glTFLoader.cpp:96-125): FLOAT components only.
    std::vector<float> floats(int accessor)
    {
        if (accessor < 0)
            return {};
        const std::vector<Json>& accs = doc.arr("accessors");
        if (size_t(accessor) >= accs.size())
        {
            warnings += "accessor " + std::to_string(accessor) + " does not exist\n";
            return {};
        }
        const Json& a = accs[size_t(accessor)];
        if (a.integer("componentType", 0) != kFloat)
        {
            warnings += "skipping accessor " + std::to_string(accessor) + " with component type " +
                std::to_string(a.integer("componentType", 0)) + " (only FLOAT is supported)\n";
            return {};
        }
        int comps = components(a.str("type"));
        const uint8_t* base;
        size_t stride, count;
        const Json* acc;
        if (!comps || !view(accessor, comps * 4, base, stride, count, acc))
        {
            warnings += "accessor " + std::to_string(accessor) + " is outside its buffer\n";
            return {};
        }
        std::vector<float> out(count * size_t(comps));
        for (size_t i = 0; i < count; i++)
            std::memcpy(&out[i * size_t(comps)], base + i * stride, size_t(comps) * 4);
        return out;
    }

    // decodeIndexAccessor (glTFLoader.cpp:128-177): unsigned 8, 16 or 32-bit.
    std::vector<uint32_t> indices(int accessor)
    {
        if (accessor < 0)
            return {};
        const std::vector<Json>& accs = doc.arr("accessors");
        if (size_t(accessor) >= accs.size())
        {
            warnings += "accessor " + std::to_string(accessor) + " does not exist\n";
            return {};
        }
        int type = accs[size_t(accessor)].integer("componentType", 0);
        int size = type == kUnsignedByte ? 1 : type == kUnsignedShort ? 2 : type == kUnsignedInt ? 4 : 0;
        if (!size)
        {
            warnings += "skipping index accessor with component type " + std::to_string(type) + "\n";
            return {};
        }
        const uint8_t* base;
        size_t stride, count;
        const Json* acc;
        if (!view(accessor, size, base, stride, count, acc))
        {
            warnings += "accessor " + std::to_string(accessor) + " is outside its buffer\n";
            return {};
        }
        std::vector<uint32_t> out(count);
        for (size_t i = 0; i < count; i++)
        {
            const uint8_t* e = base + i * stride;
            if (size == 1)
                out[i] = *e;
            else if (size == 2)
            {
                uint16_t v;
                std::memcpy(&v, e, 2);
                out[i] = v;
            }
            else
                std::memcpy(&out[i], e, 4);
        }
        return out;
    }
};

// Reads a .glb or .gltf file with its buffers.
bool loadModel(const std::string& path, Model& m, std::string& error)
{
    std::string data;
    if (!readFile(path, data))
    {
        error = "cannot read " + path;
        return false;
    }
    m.filePath = path;
    std::string bin;
    bool hasBin = false;
    const char* jsonBegin = data.data();
    const char* jsonEnd   = data.data() + data.size();
    if (data.size() >= 12 && le32(data, 0) == 0x46546C67u) // "glTF"
    {
        if (le32(data, 4) != 2)
        {
            error = "unsupported .glb version " + std::to_string(le32(data, 4));
            return false;
        }
        size_t total = std::min<size_t>(le32(data, 8), data.size());
        size_t at    = 12;
        bool hasJson = false;
        while (at + 8 <= total)
        {
            size_t len = le32(data, at);
            uint32_t type = le32(data, at + 4);
            if (at + 8 + len > total)
            {
                error = ".glb chunk runs past the end of the file";
                return false;
            }
            if (type == 0x4E4F534Au && !hasJson) // "JSON"
            {
                jsonBegin = data.data() + at + 8;
                jsonEnd   = jsonBegin + len;
                hasJson   = true;
            }
            else if (type == 0x004E4942u && !hasBin) // "BIN\0"
            {
                bin    = data.substr(at + 8, len);
                hasBin = true;
            }
            at += 8 + ((len + 3) & ~size_t(3));
        }
        if (!hasJson)
        {
            error = ".glb has no JSON chunk";
            return false;
        }
    }
    JsonParser parser(jsonBegin, jsonEnd);
    parser.setBegin(jsonBegin);
    if (!parser.parse(m.doc, error))
        return false;
    if (m.doc.kind != Json::Object)
    {
        error = "the glTF document is not a JSON object";
        return false;
    }
    const std::string dir = dirOf(path);
    for (const Json& b : m.doc.arr("buffers"))
    {
        std::string uri = b.str("uri"), bytes;
        if (uri.empty())
        {
            if (!hasBin)
            {
                error = "a buffer without uri needs the .glb BIN chunk";
                return false;
            }
            bytes = bin;
        }
        else if (uri.compare(0, 5, "data:") == 0)
        {
            size_t comma = uri.find(',');
            if (comma == std::string::npos || uri.find(";base64") == std::string::npos ||
                !base64(uri, comma + 1, bytes))
            {
                error = "unsupported data uri in buffer";
                return false;
            }
        }
        else if (!readFile(dir + uriDecode(uri), bytes))
        {
            error = "cannot read buffer " + uri;
            return false;
        }
        double lengthValue = b.num("byteLength", double(bytes.size()));
        if (!(lengthValue >= 0.0) || lengthValue > double(bytes.size()))
        {
            error = "buffer " + uri + " is shorter than its byteLength";
            return false;
        }
        m.buffers.push_back(std::move(bytes));
    }
    return true;
}

// loadCameras (glTFLoader.cpp:57-94), every node of the list and their children.
void loadCameras(const Model& m, const std::vector<Json>& nodes, SceneContents& contents, int depth)
{
    const std::vector<Json>& all  = m.doc.arr("nodes");
    const std::vector<Json>& cams = m.doc.arr("cameras");
    if (depth > 64)
        return;
    for (const Json& ni : nodes)
    {
        int idx = int(ni.n);
        if (ni.kind != Json::Number || idx < 0 || size_t(idx) >= all.size())
            continue;
        const Json& node = all[size_t(idx)];
        int ci           = node.integer("camera", -1);
        if (ci >= 0 && size_t(ci) < cams.size())
        {
            SceneCamera c;
            c.name = node.str("name");
            if (!invert(nodeTransform(node), c.viewMatrix))
                c.viewMatrix = nodeTransform(node);
            const Json& cam = cams[size_t(ci)];
            if (cam.str("type") == "perspective")
            {
                const Json* p = cam.get("perspective");
                c.type        = SceneCamera::Perspective;
                if (p)
                {
                    c.yfov        = float(p->num("yfov", 0));
                    c.aspectRatio = float(p->num("aspectRatio", 0));
                    c.znear       = float(p->num("znear", 0));
                    c.zfar        = float(p->num("zfar", 0));
                }
            }
            else if (cam.str("type") == "orthographic")
            {
                const Json* o = cam.get("orthographic");
                c.type        = SceneCamera::Orthographic;
                if (o)
                {
                    c.znear = float(o->num("znear", 0));
                    c.zfar  = float(o->num("zfar", 0));
                    c.xmag  = float(o->num("xmag", 0));
                    c.ymag  = float(o->num("ymag", 0));
                }
            }
            contents.cameras.push_back(c);
        }
        loadCameras(m, node.arr("children"), contents, depth + 1);
    }
}

// loadNode (glTFLoader.cpp:180-371).
void loadNode(Model& m, int nodeIdx, const mat4& parent, SceneContents& contents,
    const std::vector<Path>& materialPaths, int& geomCounter, bool& boundsSet, int depth)
{
    const std::vector<Json>& all = m.doc.arr("nodes");
    if (nodeIdx < 0 || size_t(nodeIdx) >= all.size() || depth > 64)
        return;
    const Json& node = all[size_t(nodeIdx)];
    const mat4 local = mul(parent, nodeTransform(node));
    int meshIdx      = node.integer("mesh", -1);
    const std::vector<Json>& meshes = m.doc.arr("meshes");
    if (meshIdx >= 0 && size_t(meshIdx) < meshes.size())
    {
        for (const Json& prim : meshes[size_t(meshIdx)].arr("primitives"))
        {
            if (prim.integer("mode", 4) != 4) // TRIANGLES
                continue;
            const Json* attrs = prim.get("attributes");
            const Json* pos   = attrs ? attrs->get("POSITION") : nullptr;
            if (!pos || pos->kind != Json::Number)
                continue;
            std::vector<float> positions = m.floats(int(pos->n));
            if (positions.empty())
                continue;
            std::vector<float> normals, texCoords;
            if (const Json* n = attrs->get("NORMAL"))
                normals = m.floats(int(n->n));
            if (const Json* t = attrs->get("TEXCOORD_0"))
                texCoords = m.floats(int(t->n));
            std::vector<uint32_t> idx = m.indices(prim.integer("indices", -1));
            uint32_t vertexCount      = uint32_t(positions.size() / 3);
            if (idx.empty())
            {
                idx.resize(vertexCount);
                for (uint32_t i = 0; i < vertexCount; i++)
                    idx[i] = i;
            }
            bool inRange = true;
            for (uint32_t i : idx)
                inRange = inRange && i < vertexCount;
            if (!inRange || idx.size() % 3 != 0)
            {
                m.warnings += "skipping a primitive with out-of-range or incomplete indices\n";
                continue;
            }
            if (normals.size() != positions.size())
            {
                normals.assign(positions.size(), 0.f);
                calculateNormals(vertexCount, positions.data(), idx.size() / 3, idx.data(), normals.data());
            }
            if (!texCoords.empty() && texCoords.size() != size_t(vertexCount) * 2)
                texCoords.clear();
            const Path geomPath = m.filePath + ":gltfGeom:" + std::to_string(geomCounter);
            const Path instPath = m.filePath + ":gltfInst:" + std::to_string(geomCounter);
            geomCounter++;
            SceneGeometryData& g = contents.geometry[geomPath];
            g.positions          = std::move(positions);
            g.normals            = std::move(normals);
            g.texCoords          = std::move(texCoords);
            g.indices            = std::move(idx);

            SceneInstanceData inst;
            inst.instance  = instPath;
            inst.geometry  = geomPath;
            inst.transform = local;
            // Priority 1: the node's AURORA_materials_materialX extension; 2: the glTF material.
            const Json* ext = node.get("extensions");
            const Json* mx  = ext ? ext->get("AURORA_materials_materialX") : nullptr;
            if (mx && mx->kind == Json::Object && !mx->str("materialXFile").empty())
            {
                const std::string file = dirOf(m.filePath) + mx->str("materialXFile");
                const Path path        = "AURORA_mtlx:" + file;
                bool known             = false;
                for (const SceneMaterialData& md : contents.materials)
                    known = known || md.path == path;
                if (known)
                    inst.material = path;
                else
                {
                    SceneMaterialData md;
                    md.path = path;
                    std::vector<MaterialXImage> imgs;
                    if (materialXFileToProperties(file, md.properties, m.warnings, &imgs))
                    {
                        for (const MaterialXImage& im : imgs)
                        {
                            bool have = false;
                            for (const SceneImageData& d : contents.images)
                                have = have || d.path == im.image;
                            if (!have)
                                contents.images.push_back(SceneImageData{ im.image, im.file, im.linearize });
                        }
                        contents.materials.push_back(md);
                        inst.material = path;
                    }
                    else
                        m.warnings += "node " + std::to_string(nodeIdx) + ": using the glTF material\n";
                }
            }
            int mi = prim.integer("material", -1);
            if (inst.material.empty() && mi >= 0 && size_t(mi) < materialPaths.size())
                inst.material = materialPaths[size_t(mi)];
            contents.instances.push_back(inst);
            contents.vertexCount += vertexCount;
            contents.triangleCount += uint32_t(g.indices.size() / 3);
            // Bounds of the transformed positions (glTFLoader.cpp:361-367).
            for (size_t v = 0; v + 2 < g.positions.size(); v += 3)
            {
                float x = g.positions[v], y = g.positions[v + 1], z = g.positions[v + 2];
                for (int r = 0; r < 3; r++)
                {
                    float p = local[0 * 4 + r] * x + local[1 * 4 + r] * y + local[2 * 4 + r] * z + local[3 * 4 + r];
                    if (!boundsSet || p < contents.boundsMin[r])
                        contents.boundsMin[r] = p;
                    if (!boundsSet || p > contents.boundsMax[r])
                        contents.boundsMax[r] = p;
                }
                boundsSet = true;
            }
        }
    }
    for (const Json& c : node.arr("children"))
        if (c.kind == Json::Number)
            loadNode(m, int(c.n), local, contents, materialPaths, geomCounter, boundsSet, depth + 1);
}

// JSON number text that reads back as the same double.
std::string number(double v)
{
    char buf[40];
    std::snprintf(buf, sizeof buf, "%.17g", v);
    return buf;
}

std::string quoted(const std::string& s)
{
    std::string out = "\"";
    for (char c : s)
    {
        if (c == '"' || c == '\\')
        {
            out += '\\';
            out += c;
        }
        else if (uint8_t(c) < 0x20)
        {
            char buf[8];
            std::snprintf(buf, sizeof buf, "\\u%04x", unsigned(uint8_t(c)));
            out += buf;
        }
        else
            out += c;
    }
    return out + "\"";
}

} // namespace

bool loadglTFFile(IScene* scene, const std::string& filePath, SceneContents& contents)
{
    contents.reset();
    Model m;
    std::string error;
    if (!loadModel(filePath, m, error))
    {
        contents.warnings = error;
        return false;
    }
    for (const Json& s : m.doc.arr("scenes"))
        loadCameras(m, s.arr("nodes"), contents, 0);
    // Materials (glTFLoader.cpp:403-425): base colour, metalness and roughness factors.
    std::vector<Path> materialPaths;
    const std::vector<Json>& mats = m.doc.arr("materials");
    for (size_t i = 0; i < mats.size(); i++)
    {
        float bc[4] = { 1.f, 1.f, 1.f, 1.f }, metallic = 1.f, roughness = 1.f;
        if (const Json* pbr = mats[i].get("pbrMetallicRoughness"))
        {
            const std::vector<Json>& f = pbr->arr("baseColorFactor");
            if (f.size() == 4)
                for (int k = 0; k < 4; k++)
                    bc[k] = float(f[size_t(k)].n);
            metallic  = float(pbr->num("metallicFactor", 1.0));
            roughness = float(pbr->num("roughnessFactor", 1.0));
        }
        SceneMaterialData md;
        md.path       = filePath + ":gltfMat:" + std::to_string(i);
        md.properties = { { "base_color", vec3{ bc[0], bc[1], bc[2] } }, { "metalness", metallic },
            { "specular_roughness", roughness } };
        contents.materials.push_back(md);
        materialPaths.push_back(md.path);
    }
    int geomCounter = 0;
    bool boundsSet  = false;
    const mat4 identity = { 1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1 };
    for (const Json& s : m.doc.arr("scenes"))
        for (const Json& n : s.arr("nodes"))
            if (n.kind == Json::Number)
                loadNode(m, int(n.n), identity, contents, materialPaths, geomCounter, boundsSet, 0);
    contents.warnings = m.warnings;
    addContentsToScene(scene, contents);
    return true;
}

bool saveglTFFile(const std::string& filePath, const SceneContents& contents)
{
    if (contents.cameras.empty())
        return false;
    std::string cams, nodes, sceneNodes;
    for (size_t i = 0; i < contents.cameras.size(); i++)
    {
        const SceneCamera& c = contents.cameras[i];
        std::string sep      = i ? "," : "";
        if (c.type == SceneCamera::Perspective)
            cams += sep + "{\"name\":" + quoted(c.name) + ",\"type\":\"perspective\",\"perspective\":{" +
                "\"yfov\":" + number(c.yfov) + ",\"aspectRatio\":" + number(c.aspectRatio) +
                ",\"znear\":" + number(c.znear) + ",\"zfar\":" + number(c.zfar) + "}}";
        else
            cams += sep + "{\"name\":" + quoted(c.name) + ",\"type\":\"orthographic\",\"orthographic\":{" +
                "\"xmag\":" + number(c.xmag) + ",\"ymag\":" + number(c.ymag) + ",\"znear\":" +
                number(c.znear) + ",\"zfar\":" + number(c.zfar) + "}}";
        // The node holds the inverse of the view matrix (glTFLoader.cpp:475-480).
        mat4 node;
        if (!invert(c.viewMatrix, node))
            return false;
        std::string mtx;
        for (int k = 0; k < 16; k++)
            mtx += (k ? "," : "") + number(double(node[size_t(k)]));
        nodes += sep + "{\"name\":" + quoted(c.name) + ",\"camera\":" + std::to_string(i) + ",\"matrix\":[" +
            mtx + "]}";
        sceneNodes += sep + std::to_string(i);
    }
    std::ofstream f(filePath, std::ios::binary);
    if (!f)
        return false;
    f << "{\"asset\":{\"version\":\"2.0\",\"generator\":\"agb_render\"},\"scene\":0,\"scenes\":[{\"nodes\":["
      << sceneNodes << "]}],\"nodes\":[" << nodes << "],\"cameras\":[" << cams << "]}\n";
    return bool(f);
}

} // namespace agb_aurora
