// File formats of the C++ scene API: the JSON scene file (SceneLoaderJson), OBJ meshes,
// Radiance .hdr images and tone-mapped .png output.
//
// The reference reads JSON with nlohmann-json, meshes with Assimp and images with stb
// (SceneLoader.cpp:17-297, Mesh.cpp:18-125, Texture2D.cpp:107-252); none of those
// libraries is part of this project, so each format has its own small reader/writer
// here, following the reference's use of the data: the same keys and defaults, the
// same camera call order, the same vertex defaults, and the same tone curve.
#include "petrichor_gb300/Petrichor.hpp"

#include <algorithm>
#include <cctype>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <fstream>
#include <iostream>
#include <iterator>
#include <map>
#include <sstream>

namespace Petrichor {
namespace Core {

namespace {

// ---------------------------------------------------------------- JSON (subset: RFC 8259
// values; numbers as double; \u escapes kept as '?')
struct Json {
    enum Kind { Null, Bool, Number, String, Array, Object } kind = Null;
    bool b = false;
    double num = 0.0;
    std::string str;
    std::vector<Json> arr;
    std::vector<std::pair<std::string, Json>> obj;

    const Json* Find(const std::string& key) const {
        if (kind != Object) return nullptr;
        for (const auto& kv : obj)
            if (kv.first == key) return &kv.second;
        return nullptr;
    }
    const Json& operator[](const std::string& key) const {
        static const Json kNull;
        const Json* j = Find(key);
        return j ? *j : kNull;
    }
};

class JsonParser {
public:
    explicit JsonParser(const std::string& text) : s_(text) {}
    bool Parse(Json* out) {
        Ws();
        if (!Value(out, 0)) return false;
        Ws();
        return i_ == s_.size();
    }

private:
    const std::string& s_;
    size_t i_ = 0;
    void Ws() {
        while (i_ < s_.size() && std::isspace((unsigned char)s_[i_])) i_++;
    }
    bool Lit(const char* w) {
        const size_t n = std::strlen(w);
        if (s_.compare(i_, n, w) != 0) return false;
        i_ += n;
        return true;
    }
    bool Str(std::string* out) {
        if (i_ >= s_.size() || s_[i_] != '"') return false;
        i_++;
        while (i_ < s_.size() && s_[i_] != '"') {
            char c = s_[i_++];
            if (c == '\\' && i_ < s_.size()) {
                const char e = s_[i_++];
                switch (e) {
                case 'n': c = '\n'; break;
                case 't': c = '\t'; break;
                case 'r': c = '\r'; break;
                case 'b': c = '\b'; break;
                case 'f': c = '\f'; break;
                case 'u': i_ = std::min(s_.size(), i_ + 4); c = '?'; break;
                default: c = e; break;
                }
            }
            out->push_back(c);
        }
        if (i_ >= s_.size()) return false;
        i_++;
        return true;
    }
    bool Value(Json* v, int depth) {
        if (depth > 256 || i_ >= s_.size()) return false;
        const char c = s_[i_];
        if (c == '{') {
            v->kind = Json::Object;
            i_++;
            Ws();
            if (i_ < s_.size() && s_[i_] == '}') return ++i_, true;
            for (;;) {
                std::string key;
                Ws();
                if (!Str(&key)) return false;
                Ws();
                if (i_ >= s_.size() || s_[i_++] != ':') return false;
                Ws();
                Json child;
                if (!Value(&child, depth + 1)) return false;
                v->obj.emplace_back(std::move(key), std::move(child));
                Ws();
                if (i_ < s_.size() && s_[i_] == ',') { i_++; continue; }
                if (i_ < s_.size() && s_[i_] == '}') return ++i_, true;
                return false;
            }
        }
        if (c == '[') {
            v->kind = Json::Array;
            i_++;
            Ws();
            if (i_ < s_.size() && s_[i_] == ']') return ++i_, true;
            for (;;) {
                Ws();
                Json child;
                if (!Value(&child, depth + 1)) return false;
                v->arr.push_back(std::move(child));
                Ws();
                if (i_ < s_.size() && s_[i_] == ',') { i_++; continue; }
                if (i_ < s_.size() && s_[i_] == ']') return ++i_, true;
                return false;
            }
        }
        if (c == '"') {
            v->kind = Json::String;
            return Str(&v->str);
        }
        if (Lit("true")) { v->kind = Json::Bool; v->b = true; return true; }
        if (Lit("false")) { v->kind = Json::Bool; v->b = false; return true; }
        if (Lit("null")) { v->kind = Json::Null; return true; }
        const char* begin = s_.c_str() + i_;
        char* end = nullptr;
        v->num = std::strtod(begin, &end);
        if (end == begin) return false;
        v->kind = Json::Number;
        i_ += (size_t)(end - begin);
        return true;
    }
};

void Error(const std::string& msg) { std::cerr << "[Error] " << msg << "\n"; }

// SceneLoader.cpp:35-59: a 3-vector, zero with an error message when absent
Math::Vector3f LoadVector3f(const Json& json, const char* name) {
    const Json* a = json.Find(name);
    if (!a) {
        Error(std::string("[SceneLoaderJson] '") + name + "' not found.");
        return Math::Vector3f::Zero();
    }
    if (a->kind != Json::Array || a->arr.size() != 3)
        Error(std::string("[SceneLoaderJson] '") + name + "' size != 3.");
    Math::Vector3f v;
    if (a->kind == Json::Array)
        for (int i = 0; i < std::min<int>(3, (int)a->arr.size()); i++) v[i] = (float)a->arr[i].num;
    return v;
}

// SceneLoader.cpp:61-78: keeps the default when absent
template <class T>
void LoadValue(T* out, const Json& json, const char* name) {
    const Json* v = json.Find(name);
    if (!v) {
        Error(std::string("[SceneLoaderJson] '") + name + "' not found.");
        return;
    }
    if constexpr (std::is_same_v<T, std::string>) {
        *out = v->str;
    } else {
        *out = (T)v->num;
    }
}

// ---------------------------------------------------------------- Radiance RGBE
bool ReadRgbeScanline(std::istream& f, int W, std::vector<uint8_t>& line) {
    line.assign((size_t)W * 4, 0);
    uint8_t head[4];
    if (!f.read((char*)head, 4)) return false;
    const bool rle = W >= 8 && W < 32768 && head[0] == 2 && head[1] == 2 && !(head[2] & 0x80) &&
                     ((head[2] << 8) | head[3]) == W;
    if (!rle) {  // flat scanline: the 4 bytes read are the first pixel
        std::memcpy(line.data(), head, 4);
        return (bool)f.read((char*)line.data() + 4, (std::streamsize)(W - 1) * 4);
    }
    for (int c = 0; c < 4; c++) {
        int x = 0;
        while (x < W) {
            int n = f.get();
            if (n == EOF) return false;
            if (n > 128) {  // run
                n -= 128;
                const int v = f.get();
                if (v == EOF || x + n > W) return false;
                for (int k = 0; k < n; k++) line[(size_t)(x++) * 4 + c] = (uint8_t)v;
            } else {
                if (n == 0 || x + n > W) return false;
                for (int k = 0; k < n; k++) {
                    const int v = f.get();
                    if (v == EOF) return false;
                    line[(size_t)(x++) * 4 + c] = (uint8_t)v;
                }
            }
        }
    }
    return true;
}

float RgbeComponent(uint8_t m, uint8_t e) {  // mantissa * 2^(e - 136); e = 0 is black
    return e ? std::ldexp((float)m, (int)e - 136) : 0.0f;
}

void ToRgbe(float r, float g, float b, uint8_t* out) {
    const float v = std::max(r, std::max(g, b));
    if (!(v >= 1e-32f)) {
        out[0] = out[1] = out[2] = out[3] = 0;
        return;
    }
    int e = 0;
    const float scale = std::frexp(v, &e) * 256.0f / v;
    out[0] = (uint8_t)std::min(255.0f, std::max(0.0f, r * scale));
    out[1] = (uint8_t)std::min(255.0f, std::max(0.0f, g * scale));
    out[2] = (uint8_t)std::min(255.0f, std::max(0.0f, b * scale));
    out[3] = (uint8_t)(e + 128);
}

// ---------------------------------------------------------------- PNG (stored deflate)
uint32_t Crc32(const uint8_t* p, size_t n, uint32_t crc = 0) {
    static uint32_t table[256];
    static bool init = false;
    if (!init) {
        for (uint32_t i = 0; i < 256; i++) {
            uint32_t c = i;
            for (int k = 0; k < 8; k++) c = (c & 1) ? 0xEDB88320u ^ (c >> 1) : c >> 1;
            table[i] = c;
        }
        init = true;
    }
    crc = ~crc;
    for (size_t i = 0; i < n; i++) crc = table[(crc ^ p[i]) & 0xff] ^ (crc >> 8);
    return ~crc;
}

void PutU32(std::vector<uint8_t>& v, uint32_t x) {
    for (int s = 24; s >= 0; s -= 8) v.push_back((uint8_t)(x >> s));
}

void Chunk(std::ofstream& f, const char* type, const std::vector<uint8_t>& data) {
    std::vector<uint8_t> c;
    PutU32(c, (uint32_t)data.size());
    c.insert(c.end(), type, type + 4);
    c.insert(c.end(), data.begin(), data.end());
    PutU32(c, Crc32(c.data() + 4, c.size() - 4));
    f.write((const char*)c.data(), (std::streamsize)c.size());
}

bool WritePng(const std::filesystem::path& path, int W, int H, const std::vector<uint8_t>& rgb) {
    std::ofstream f(path, std::ios::binary);
    if (!f) return false;
    static const uint8_t sig[8] = {137, 80, 78, 71, 13, 10, 26, 10};
    f.write((const char*)sig, 8);
    std::vector<uint8_t> ihdr;
    PutU32(ihdr, (uint32_t)W);
    PutU32(ihdr, (uint32_t)H);
    ihdr.insert(ihdr.end(), {8, 2, 0, 0, 0});  // 8-bit RGB, no interlace
    Chunk(f, "IHDR", ihdr);
    // zlib stream of stored deflate blocks over the filtered scanlines (filter 0)
    std::vector<uint8_t> raw;
    raw.reserve((size_t)H * (W * 3 + 1));
    for (int y = 0; y < H; y++) {
        raw.push_back(0);
        raw.insert(raw.end(), rgb.begin() + (size_t)y * W * 3, rgb.begin() + (size_t)(y + 1) * W * 3);
    }
    std::vector<uint8_t> z = {0x78, 0x01};
    size_t off = 0;
    do {
        const size_t n = std::min<size_t>(65535, raw.size() - off);
        z.push_back(off + n == raw.size() ? 1 : 0);
        z.push_back((uint8_t)(n & 0xff));
        z.push_back((uint8_t)(n >> 8));
        z.push_back((uint8_t)(~n & 0xff));
        z.push_back((uint8_t)((~n >> 8) & 0xff));
        z.insert(z.end(), raw.begin() + off, raw.begin() + off + n);
        off += n;
    } while (off < raw.size());
    uint32_t a = 1, b = 0;  // Adler-32
    for (uint8_t c : raw) {
        a = (a + c) % 65521;
        b = (b + a) % 65521;
    }
    PutU32(z, (b << 16) | a);
    Chunk(f, "IDAT", z);
    Chunk(f, "IEND", {});
    return (bool)f;
}

// Tone mapping of Texture2D::Save (Texture2D.cpp:15-91): ACES film curve, the
// reference's gamma-based contrast curve, then 1.1 / (1 / 2.2) power "degamma".
float AcesFilm(float x) {
    const float a = 2.51f, b = 0.03f, c = 2.43f, d = 0.59f, e = 0.14f;
    return (x * (a * x + b)) / (x * (c * x + d) + e);
}
float Gamma(float v, float g) { return (float)std::pow((double)v, (double)g); }
Color3f ToneMap(const Color3f& in) {
    Color3f c(AcesFilm(in.x), AcesFilm(in.y), AcesFilm(in.z));
    c = Color3f(Gamma(c.x, 1.2f), Gamma(c.y, 1.2f), Gamma(c.z, 1.2f));
    const float x0 = Gamma(0.05f, 2.2f), x1 = Gamma(0.9f, 2.2f);
    c = Color3f((c.x - x0) / (x1 - x0), (c.y - x0) / (x1 - x0), (c.z - x0) / (x1 - x0));
    c.y = Gamma(c.y, 1.3f);
    c.z = Gamma(c.z, 1.6f);
    return c;
}
float Degamma(float v) {
    v = (float)std::pow((double)v, 1.1);
    v = std::clamp(v, 0.0f, 1.0f);
    return (float)std::pow((double)v, (double)(1 / 2.2f));
}


// ---- PNG reading (what stbi_load(path, 3 channels) returns to Texture2D::Load,
// Texture2D.cpp:118-160). An own decoder written from the zlib / DEFLATE formats
// (RFC 1950, RFC 1951) and the PNG specification: all colour types and bit depths,
// Adam7 interlacing, the five scanline filters. The result is 8-bit RGB: grey is
// replicated, palette indices are looked up, alpha is dropped, 16-bit samples keep
// their high byte, and 1/2/4-bit grey is scaled to 0..255.

class BitStream {  // DEFLATE bit order: least significant bit of each byte first
public:
    BitStream(const uint8_t* p, size_t n) : m_p(p), m_n(n) {}
    bool Bits(int count, uint32_t* out) {
        uint32_t v = 0;
        for (int i = 0; i < count; i++) {
            if (m_byte >= m_n) return false;
            v |= (uint32_t)((m_p[m_byte] >> m_bit) & 1u) << i;
            if (++m_bit == 8) m_bit = 0, m_byte++;
        }
        *out = v;
        return true;
    }
    void AlignToByte() {
        if (m_bit) m_bit = 0, m_byte++;
    }
    bool Bytes(size_t count, const uint8_t** out) {
        if (m_byte + count > m_n) return false;
        *out = m_p + m_byte;
        m_byte += count;
        return true;
    }

private:
    const uint8_t* m_p;
    size_t m_n, m_byte = 0;
    int m_bit = 0;
};

// Canonical Huffman code given by its code lengths (RFC 1951 section 3.2.2), decoded
// one bit at a time: codes of each length are consecutive, ordered by symbol.
class Huffman {
public:
    bool Build(const uint8_t* lengths, int n) {
        std::fill(std::begin(m_count), std::end(m_count), 0);
        for (int i = 0; i < n; i++) m_count[lengths[i]]++;
        m_count[0] = 0;
        int left = 1;  // reject over-subscribed sets
        for (int len = 1; len < 16; len++) {
            left = 2 * left - m_count[len];
            if (left < 0) return false;
        }
        int offset[16] = {0};
        for (int len = 1; len < 15; len++) offset[len + 1] = offset[len] + m_count[len];
        m_symbol.assign(n, 0);
        for (int i = 0; i < n; i++)
            if (lengths[i]) m_symbol[offset[lengths[i]]++] = (uint16_t)i;
        return true;
    }
    int Decode(BitStream& in) const {
        int code = 0, first = 0, index = 0;
        for (int len = 1; len < 16; len++) {
            uint32_t b;
            if (!in.Bits(1, &b)) return -1;
            code |= (int)b;
            const int count = m_count[len];
            if (code - first < count) return m_symbol[index + code - first];
            index += count;
            first = (first + count) << 1;
            code <<= 1;
        }
        return -1;
    }

private:
    int m_count[16];
    std::vector<uint16_t> m_symbol;
};

// Length and distance codes (RFC 1951 section 3.2.5).
constexpr uint16_t kLenBase[29] = {3,  4,  5,  6,  7,  8,  9,  10, 11,  13,  15,  17,  19,  23, 27,
                                   31, 35, 43, 51, 59, 67, 83, 99, 115, 131, 163, 195, 227, 258};
constexpr uint8_t kLenExtra[29] = {0, 0, 0, 0, 0, 0, 0, 0, 1, 1, 1, 1, 2, 2, 2,
                                   2, 3, 3, 3, 3, 4, 4, 4, 4, 5, 5, 5, 5, 0};
constexpr uint16_t kDistBase[30] = {1,   2,   3,   4,   5,   7,    9,    13,   17,   25,
                                    33,  49,  65,  97,  129, 193,  257,  385,  513,  769,
                                    1025, 1537, 2049, 3073, 4097, 6145, 8193, 12289, 16385, 24577};
constexpr uint8_t kDistExtra[30] = {0, 0, 0, 0, 1, 1, 2, 2,  3,  3,  4,  4,  5,  5,  6,
                                    6, 7, 7, 8, 8, 9, 9, 10, 10, 11, 11, 12, 12, 13, 13};

bool InflateBlock(BitStream& in, const Huffman& lit, const Huffman& dist, std::vector<uint8_t>& out,
                  size_t limit) {
    for (;;) {
        const int sym = lit.Decode(in);
        if (sym < 0) return false;
        if (sym < 256) {
            if (out.size() >= limit) return false;
            out.push_back((uint8_t)sym);
            continue;
        }
        if (sym == 256) return true;
        const int li = sym - 257;
        if (li >= 29) return false;
        uint32_t e;
        if (!in.Bits(kLenExtra[li], &e)) return false;
        const size_t len = kLenBase[li] + e;
        const int di = dist.Decode(in);
        if (di < 0 || di >= 30) return false;
        if (!in.Bits(kDistExtra[di], &e)) return false;
        const size_t d = kDistBase[di] + e;
        if (d > out.size() || out.size() + len > limit) return false;
        for (size_t k = 0; k < len; k++) {
            const uint8_t v = out[out.size() - d];
            out.push_back(v);
        }
    }
}

// zlib stream -> bytes (at most `limit`); false on any malformed input.
bool Inflate(const std::vector<uint8_t>& z, std::vector<uint8_t>& out, size_t limit) {
    if (z.size() < 2 || (z[0] & 15) != 8 || ((z[0] << 8) | z[1]) % 31 != 0 || (z[1] & 32))
        return false;
    BitStream in(z.data() + 2, z.size() - 2);
    Huffman fixedLit, fixedDist;
    {
        uint8_t l[288], d[30];
        for (int i = 0; i < 288; i++) l[i] = i < 144 ? 8 : i < 256 ? 9 : i < 280 ? 7 : 8;
        std::fill(d, d + 30, 5);
        fixedLit.Build(l, 288);
        fixedDist.Build(d, 30);
    }
    uint32_t last = 0;
    while (!last) {
        uint32_t type;
        if (!in.Bits(1, &last) || !in.Bits(2, &type)) return false;
        if (type == 0) {  // stored
            in.AlignToByte();
            const uint8_t* h;
            if (!in.Bytes(4, &h)) return false;
            const uint32_t len = h[0] | (h[1] << 8), nlen = h[2] | (h[3] << 8);
            if ((len ^ 0xffffu) != nlen || out.size() + len > limit) return false;
            const uint8_t* p;
            if (!in.Bytes(len, &p)) return false;
            out.insert(out.end(), p, p + len);
        } else if (type == 1) {
            if (!InflateBlock(in, fixedLit, fixedDist, out, limit)) return false;
        } else if (type == 2) {  // dynamic codes
            uint32_t hlit, hdist, hclen;
            if (!in.Bits(5, &hlit) || !in.Bits(5, &hdist) || !in.Bits(4, &hclen)) return false;
            hlit += 257, hdist += 1, hclen += 4;
            if (hlit > 286 || hdist > 30) return false;
            static constexpr uint8_t kOrder[19] = {16, 17, 18, 0, 8, 7, 9, 6, 10, 5,
                                                   11, 4,  12, 3, 13, 2, 14, 1, 15};
            uint8_t cl[19] = {0};
            for (uint32_t i = 0; i < hclen; i++) {
                uint32_t v;
                if (!in.Bits(3, &v)) return false;
                cl[kOrder[i]] = (uint8_t)v;
            }
            Huffman clCode;
            if (!clCode.Build(cl, 19)) return false;
            uint8_t lens[286 + 30] = {0};
            for (uint32_t i = 0; i < hlit + hdist;) {
                const int sym = clCode.Decode(in);
                if (sym < 0) return false;
                if (sym < 16) {
                    lens[i++] = (uint8_t)sym;
                    continue;
                }
                uint32_t rep, v = 0;
                if (sym == 16) {
                    if (i == 0 || !in.Bits(2, &rep)) return false;
                    rep += 3, v = lens[i - 1];
                } else if (sym == 17) {
                    if (!in.Bits(3, &rep)) return false;
                    rep += 3;
                } else {
                    if (!in.Bits(7, &rep)) return false;
                    rep += 11;
                }
                if (i + rep > hlit + hdist) return false;
                while (rep--) lens[i++] = (uint8_t)v;
            }
            if (lens[256] == 0) return false;
            Huffman lit, dist;
            if (!lit.Build(lens, (int)hlit) || !dist.Build(lens + hlit, (int)hdist)) return false;
            if (!InflateBlock(in, lit, dist, out, limit)) return false;
        } else {
            return false;
        }
    }
    return true;
}

uint32_t BigEndian32(const uint8_t* p) {
    return ((uint32_t)p[0] << 24) | ((uint32_t)p[1] << 16) | ((uint32_t)p[2] << 8) | p[3];
}

int Paeth(int a, int b, int c) {
    const int p = a + b - c, pa = std::abs(p - a), pb = std::abs(p - b), pc = std::abs(p - c);
    return (pa <= pb && pa <= pc) ? a : (pb <= pc ? b : c);
}

// Reverses the scanline filters of one (sub)image in place; rows of `stride` bytes
// each preceded by their filter byte; bpp = bytes per complete pixel (at least 1).
bool Unfilter(uint8_t* data, int rows, size_t stride, int bpp, std::vector<uint8_t>& out) {
    out.assign((size_t)rows * stride, 0);
    for (int y = 0; y < rows; y++) {
        const uint8_t f = data[(size_t)y * (stride + 1)];
        const uint8_t* src = data + (size_t)y * (stride + 1) + 1;
        uint8_t* row = out.data() + (size_t)y * stride;
        const uint8_t* up = y ? row - stride : nullptr;
        for (size_t x = 0; x < stride; x++) {
            const int a = x >= (size_t)bpp ? row[x - bpp] : 0, b = up ? up[x] : 0;
            const int c = (up && x >= (size_t)bpp) ? up[x - bpp] : 0;
            int v = src[x];
            switch (f) {
            case 0: break;
            case 1: v += a; break;
            case 2: v += b; break;
            case 3: v += (a + b) >> 1; break;
            case 4: v += Paeth(a, b, c); break;
            default: return false;
            }
            row[x] = (uint8_t)v;
        }
    }
    return true;
}

bool ReadPng(const std::filesystem::path& path, int* W, int* H, std::vector<uint8_t>& rgb) {
    std::ifstream f(path, std::ios::binary);
    std::vector<uint8_t> file((std::istreambuf_iterator<char>(f)), std::istreambuf_iterator<char>());
    static constexpr uint8_t kSig[8] = {137, 80, 78, 71, 13, 10, 26, 10};
    if (file.size() < 8 || std::memcmp(file.data(), kSig, 8) != 0) return false;
    uint32_t width = 0, height = 0;
    int depth = 0, color = -1, interlace = 0;
    std::vector<uint8_t> idat, palette;
    for (size_t off = 8; off + 12 <= file.size();) {
        const uint32_t len = BigEndian32(&file[off]);
        if (len > file.size() - off - 12) return false;
        const char* type = (const char*)&file[off + 4];
        const uint8_t* d = &file[off + 8];
        if (std::memcmp(type, "IHDR", 4) == 0 && len >= 13) {
            width = BigEndian32(d), height = BigEndian32(d + 4);
            depth = d[8], color = d[9], interlace = d[12];
            if (d[10] != 0 || d[11] != 0) return false;
        } else if (std::memcmp(type, "PLTE", 4) == 0) {
            palette.assign(d, d + len);
        } else if (std::memcmp(type, "IDAT", 4) == 0) {
            idat.insert(idat.end(), d, d + len);
        } else if (std::memcmp(type, "IEND", 4) == 0) {
            break;
        }
        off += 12 + (size_t)len;
    }
    const int channels = color == 0 ? 1 : color == 2 ? 3 : color == 3 ? 1 : color == 4 ? 2 : color == 6 ? 4 : 0;
    const bool depthOk = (color == 0 && (depth == 1 || depth == 2 || depth == 4 || depth == 8 || depth == 16)) ||
                         (color == 3 && (depth == 1 || depth == 2 || depth == 4 || depth == 8)) ||
                         ((color == 2 || color == 4 || color == 6) && (depth == 8 || depth == 16));
    if (!channels || !depthOk || width == 0 || height == 0 || width > (1u << 24) || height > (1u << 24) ||
        (uint64_t)width * height > (1ull << 28) || interlace > 1 || (color == 3 && palette.size() < 3))
        return false;
    const int bitsPerPixel = channels * depth, bpp = std::max(1, bitsPerPixel / 8);
    auto stride = [&](uint32_t w) { return ((size_t)w * bitsPerPixel + 7) / 8; };
    // Adam7 passes (start and step in x and y); a non-interlaced image is one pass
    static constexpr int kX0[7] = {0, 4, 0, 2, 0, 1, 0}, kY0[7] = {0, 0, 4, 0, 2, 0, 1};
    static constexpr int kDX[7] = {8, 8, 4, 4, 2, 2, 1}, kDY[7] = {8, 8, 8, 4, 4, 2, 2};
    const int passes = interlace ? 7 : 1;
    size_t expected = 0;
    uint32_t pw[7], ph[7];
    for (int p = 0; p < passes; p++) {
        pw[p] = interlace ? (width > (uint32_t)kX0[p] ? (width - kX0[p] + kDX[p] - 1) / kDX[p] : 0) : width;
        ph[p] = interlace ? (height > (uint32_t)kY0[p] ? (height - kY0[p] + kDY[p] - 1) / kDY[p] : 0) : height;
        if (pw[p] && ph[p]) expected += (size_t)ph[p] * (stride(pw[p]) + 1);
    }
    std::vector<uint8_t> raw;
    if (!Inflate(idat, raw, expected) || raw.size() != expected) return false;
    rgb.assign((size_t)width * height * 3, 0);
    const int maxSample = (1 << depth) - 1;
    size_t pos = 0;
    std::vector<uint8_t> rows;
    for (int p = 0; p < passes; p++) {
        if (!pw[p] || !ph[p]) continue;
        const size_t st = stride(pw[p]);
        if (!Unfilter(raw.data() + pos, (int)ph[p], st, bpp, rows)) return false;
        pos += (size_t)ph[p] * (st + 1);
        for (uint32_t y = 0; y < ph[p]; y++) {
            const uint8_t* row = rows.data() + (size_t)y * st;
            // sample c of pixel x as 0..255 (or the raw index for palettes)
            auto sample = [&](uint32_t x, int c) -> int {
                const size_t bit = ((size_t)x * channels + c) * depth;
                if (depth == 16) return row[bit / 8];  // high byte
                if (depth == 8) return row[bit / 8];
                const int v = (row[bit / 8] >> (8 - depth - (int)(bit % 8))) & maxSample;
                return color == 3 ? v : v * (255 / maxSample);
            };
            for (uint32_t x = 0; x < pw[p]; x++) {
                const uint32_t ox = interlace ? kX0[p] + x * kDX[p] : x;
                const uint32_t oy = interlace ? kY0[p] + y * kDY[p] : y;
                uint8_t* o = &rgb[((size_t)oy * width + ox) * 3];
                if (color == 3) {
                    const int i = sample(x, 0);
                    if ((size_t)i * 3 + 2 >= palette.size()) return false;
                    o[0] = palette[3 * i], o[1] = palette[3 * i + 1], o[2] = palette[3 * i + 2];
                } else if (channels <= 2) {
                    o[0] = o[1] = o[2] = (uint8_t)sample(x, 0);
                } else {
                    for (int c = 0; c < 3; c++) o[c] = (uint8_t)sample(x, c);
                }
            }
        }
    }
    *W = (int)width;
    *H = (int)height;
    return true;
}
}  // namespace

// ---------------------------------------------------------------- Texture2D
bool Texture2D::Load(const std::filesystem::path& path, TextureColorType type) {
    std::ifstream f(path, std::ios::binary);
    if (!f) {
        Error("Texture not found. " + path.string());
        return false;
    }
    if (path.extension() == ".png") {  // Texture2D.cpp:118-160
        int W = 0, H = 0;
        std::vector<uint8_t> rgb;
        if (!ReadPng(path, &W, &H, rgb)) {
            Error("Could not read png file. [" + path.string() + "]");
            return false;
        }
        std::vector<float> px(rgb.size());
        for (size_t i = 0; i < rgb.size(); i++) {
            px[i] = static_cast<float>(rgb[i]) / static_cast<float>(255);
            // colour textures are linearised with ApplyGamma (std::pow(v, 2.2f))
            if (type == TextureColorType::Color) px[i] = std::pow(px[i], 2.2f);
        }
        m_width = W;
        m_height = H;
        m_pixels = std::move(px);
        m_isLoaded = true;
        return true;
    }
    char magic[8] = {};
    f.read(magic, 8);
    if (f && std::memcmp(magic, "PTRAWF32", 8) == 0) {
        uint32_t dims[2];
        if (!f.read((char*)dims, 8)) return false;
        std::vector<float> px((size_t)dims[0] * dims[1] * 3);
        if (!f.read((char*)px.data(), (std::streamsize)(px.size() * 4))) return false;
        m_width = (int)dims[0];
        m_height = (int)dims[1];
        m_pixels = std::move(px);
        m_isLoaded = true;
        return true;
    }
    if (path.extension() == ".hdr") {
        f.clear();
        f.seekg(0);
        std::string line;
        bool rgbe = false;
        while (std::getline(f, line) && !line.empty())
            if (line.rfind("FORMAT=32-bit_rle_rgbe", 0) == 0) rgbe = true;
        char ya[3] = {}, xa[3] = {};
        int H = 0, W = 0;
        if (!std::getline(f, line) ||
            std::sscanf(line.c_str(), "%2s %d %2s %d", ya, &H, xa, &W) != 4 ||
            std::strcmp(ya, "-Y") != 0 || std::strcmp(xa, "+X") != 0 || W <= 0 || H <= 0 ||
            (magic[0] != '#' && !rgbe)) {
            Error("Could not read hdr file. [" + path.string() + "]");
            return false;
        }
        std::vector<float> px((size_t)W * H * 3);
        std::vector<uint8_t> scan;
        for (int y = 0; y < H; y++) {
            if (!ReadRgbeScanline(f, W, scan)) {
                Error("Could not read hdr file. [" + path.string() + "]");
                return false;
            }
            for (int x = 0; x < W; x++) {
                const uint8_t* q = &scan[(size_t)x * 4];
                float* o = &px[((size_t)y * W + x) * 3];
                for (int c = 0; c < 3; c++) o[c] = RgbeComponent(q[c], q[3]);
            }
        }
        m_width = W;
        m_height = H;
        m_pixels = std::move(px);
        m_isLoaded = true;
        return true;
    }
    Error("Unsupported texture format. [" + path.string() + "]");
    return false;
}

void Texture2D::Save(const std::filesystem::path& path) const {
    const size_t n = (size_t)std::max(m_width, 0) * std::max(m_height, 0);
    if (path.extension() == ".png") {  // Texture2D.cpp:199-225
        std::vector<uint8_t> rgb(n * 3);
        for (size_t i = 0; i < n; i++) {
            const Color3f t = ToneMap(Color3f(m_pixels[3 * i], m_pixels[3 * i + 1], m_pixels[3 * i + 2]));
            const float v[3] = {Degamma(t.x), Degamma(t.y), Degamma(t.z)};
            for (int c = 0; c < 3; c++) rgb[3 * i + c] = (uint8_t)((255 - 1e-3f) * v[c]);
        }
        if (!WritePng(path, m_width, m_height, rgb)) Error("Could not write " + path.string());
        return;
    }
    if (path.extension() == ".hdr") {  // Texture2D.cpp:228-245, flat RGBE scanlines
        std::ofstream f(path, std::ios::binary);
        f << "#?RADIANCE\nFORMAT=32-bit_rle_rgbe\n\n-Y " << m_height << " +X " << m_width << "\n";
        std::vector<uint8_t> out(n * 4);
        for (size_t i = 0; i < n; i++) ToRgbe(m_pixels[3 * i], m_pixels[3 * i + 1], m_pixels[3 * i + 2], &out[4 * i]);
        f.write((const char*)out.data(), (std::streamsize)out.size());
        if (!f) Error("Could not write " + path.string());
        return;
    }
    Error("Unsupported image type. [" + path.string() + "]");
}

// ---------------------------------------------------------------- Mesh (OBJ)
void Mesh::Load(const std::filesystem::path& path, const MaterialBase* material, ShadingTypes shadingType) {
    std::ifstream f(path);
    if (!f) {
        Error("Fail to load mesh. [" + path.string() + "]");
        return;
    }
    std::vector<Math::Vector3f> P, N, T;
    struct Corner { int p, t, n; };
    std::vector<std::array<Corner, 3>> faces;
    std::string line;
    auto index = [](long v, size_t count) -> int {  // 1-based, negative = relative
        if (v > 0) return (int)(v - 1);
        if (v < 0) return (int)((long)count + v);
        return -1;
    };
    while (std::getline(f, line)) {
        std::istringstream in(line);
        std::string tag;
        in >> tag;
        if (tag == "v" || tag == "vn" || tag == "vt") {
            float x = 0.0f, y = 0.0f, z = 0.0f;
            in >> x >> y;
            if (tag != "vt") in >> z;
            (tag == "v" ? P : tag == "vn" ? N : T).emplace_back(x, y, z);
        } else if (tag == "f") {
            std::vector<Corner> poly;
            std::string tok;
            while (in >> tok) {
                long a = 0, b = 0, c = 0;
                const size_t s1 = tok.find('/');
                a = std::stol(tok.substr(0, s1));
                if (s1 != std::string::npos) {
                    const size_t s2 = tok.find('/', s1 + 1);
                    const std::string ts = tok.substr(s1 + 1, s2 == std::string::npos ? std::string::npos : s2 - s1 - 1);
                    if (!ts.empty()) b = std::stol(ts);
                    if (s2 != std::string::npos && s2 + 1 < tok.size()) c = std::stol(tok.substr(s2 + 1));
                }
                poly.push_back({index(a, P.size()), index(b, T.size()), index(c, N.size())});
            }
            // the reference imports without triangulation and reads three indices per face
            if (poly.size() >= 3) faces.push_back({poly[0], poly[1], poly[2]});
        }
    }
    m_vertices.clear();
    m_triangles.clear();
    m_vertices.reserve(faces.size() * 3);
    for (const auto& face : faces)
        for (const Corner& c : face) {
            Vertex v;  // normal defaults to +Z, uv to zero (Vertex.h)
            if (c.p >= 0 && c.p < (int)P.size()) v.pos = P[c.p];
            if (c.n >= 0 && c.n < (int)N.size()) v.normal = N[c.n].Normalized();
            if (c.t >= 0 && c.t < (int)T.size()) v.uv = Math::Vector3f(T[c.t].x, T[c.t].y, 0.0f);
            m_vertices.push_back(v);
        }
    m_triangles.reserve(faces.size());
    for (size_t k = 0; k < faces.size(); k++) {
        m_triangles.emplace_back(&m_vertices[3 * k], &m_vertices[3 * k + 1], &m_vertices[3 * k + 2], shadingType);
        m_triangles.back().SetMaterial(material);
    }
}

// ---------------------------------------------------------------- Scene
void Scene::LoadModel(const std::filesystem::path& path) { LoadModel(path, "default"); }

void Scene::LoadModel(const std::filesystem::path& path, std::string_view materialName) {
    auto mesh = std::make_unique<Mesh>();
    mesh->Load(path, GetMaterial(materialName), ShadingTypes::Smooth);
    AppendMesh(*mesh);
    m_meshes.push_back(std::move(mesh));
}

void Scene::LoadAssets(const std::filesystem::path& path) {
    Json root;
    {
        std::ifstream file(path, std::ios::in);
        if (file.fail()) {
            Error("Failed to read the scene file. [" + path.string() + "]");
        } else {
            std::stringstream ss;
            ss << file.rdbuf();
            const std::string text = ss.str();
            if (!JsonParser(text).Parse(&root)) Error("Invalid JSON. [" + path.string() + "]");
        }
    }
    const std::filesystem::path dir = path.parent_path();
    // ---- materials (SceneLoader.cpp:82-218)
    RegisterMaterial("default", std::make_unique<Lambert>(Color3f::One()));
    for (const Json& m : root["materials"].arr) {
        std::string type, name;
        LoadValue(&type, m, "type");
        if (type.empty()) continue;
        LoadValue(&name, m, "name");
        if (name.empty()) continue;
        if (type == "lambert") {
            auto mat = std::make_unique<Lambert>(LoadVector3f(m, "base_color"));
            std::string tex;
            LoadValue(&tex, m, "color_tex");
            if (!tex.empty()) {  // relative to the scene file, registered under that path
                const std::filesystem::path tp = dir / tex;
                Texture2D t;
                if (t.Load(tp, Texture2D::TextureColorType::Color))
                    mat->SetTexAlbedo(GetTexture(RegisterTexture(tp, t)));
            }
            RegisterMaterial(name, std::move(mat));
        } else if (type == "glass") {
            const Color3f color = LoadVector3f(m, "color");
            float ior = 1.0f;
            LoadValue(&ior, m, "ior");
            RegisterMaterial(name, std::make_unique<Glass>(color, ior));
        } else if (type == "glossy") {
            const Color3f color = LoadVector3f(m, "color");
            float roughness = 0.0f;
            LoadValue(&roughness, m, "roughness");
            auto mat = std::make_unique<GGX>(color, roughness);
            std::string tex;
            LoadValue(&tex, m, "color_tex");
            if (!tex.empty()) {  // read relative to the scene file, registered under the key as written
                Texture2D t;
                if (t.Load(dir / tex, Texture2D::TextureColorType::Color))
                    mat->SetF0Texture(GetTexture(RegisterTexture(tex, t)));
            }
            tex.clear();
            LoadValue(&tex, m, "roughness_tex");
            if (!tex.empty()) {  // the reference reads this one relative to the working directory
                Texture2D t;
                if (t.Load(tex, Texture2D::TextureColorType::NonColor))
                    mat->SetRoughnessMap(GetTexture(RegisterTexture(tex, t)));
            }
            RegisterMaterial(name, std::move(mat));
        } else if (type == "emission") {
            // the reference registers nothing for an emission entry (SceneLoader.cpp:189-191)
        } else if (type == "mix") {
            std::string n0, n1;
            LoadValue(&n0, m, "mat0_name");
            const MaterialBase* m0 = GetMaterial(n0);
            LoadValue(&n1, m, "mat1_name");
            const MaterialBase* m1 = GetMaterial(n1);
            float mix = 0.5f;
            LoadValue(&mix, m, "mix");
            RegisterMaterial(name, std::make_unique<MixMaterial>(m0, m1, mix));
        } else {
            std::cout << "[SceneLoaderJson] Invalid material type '" << type << "'.";
        }
    }
    // ---- camera (SceneLoader.cpp:221-253), in the reference's call order
    {
        const Json& c = root["camera"];
        auto camera = std::make_unique<Camera>();
        camera->SetPosition(LoadVector3f(c, "position"));
        camera->LookAt(LoadVector3f(c, "look_at"));
        camera->FocusTo(LoadVector3f(c, "focus_pos"));
        float fNumber = 2.8f;
        LoadValue(&fNumber, c, "f_number");
        camera->SetFNumber(fNumber);
        float focalLength = 55e-3f;
        LoadValue(&focalLength, c, "focal_length");
        camera->SetFocalLength(focalLength);
        SetMainCamera(std::move(camera));
    }
    // ---- environment (SceneLoader.cpp:256-277)
    {
        const Json& e = root["env"];
        Environment env;
        env.SetBaseColor(LoadVector3f(e, "base_color"));
        std::string tex;
        LoadValue(&tex, e, "texture");
        if (!tex.empty()) env.Load(dir / tex);
        SetEnvironment(env);
    }
    // ---- assets (SceneLoader.cpp:280-296)
    for (const Json& a : root["assets"].arr) {
        const std::filesystem::path p = dir / a["path"].str;
        if (a.Find("mat")) LoadModel(p, a["mat"].str);
        else LoadModel(p);
    }
}

}  // namespace Core
}  // namespace Petrichor
