// Image files for material textures (declarations in include/aurora_gb300_loaders.hpp): PNG
// decoding -- a zlib stream (RFC 1950) of DEFLATE blocks (RFC 1951: stored, fixed and dynamic
// Huffman), then the PNG scanline filters (None, Sub, Up, Average, Paeth) -- for grey, grey +
// alpha, RGB, RGBA and palette images at 1, 2, 4, 8 and 16 bits, non-interlaced; Radiance HDR
// through loadHDRFile.  Written from the two specifications.
#include <cstring>
#include <fstream>
#include <sstream>

#include "../../include/aurora_gb300_loaders.hpp"

namespace agb_aurora
{
namespace
{

// ---------------------------------------------------------------------------------- inflate
class BitReader
{
public:
    BitReader(const uint8_t* p, size_t n) : p_(p), n_(n) {}
    // Next `count` bits, least significant first; false past the end.
    bool bits(int count, uint32_t& v)
    {
        while (have_ < count)
        {
            if (pos_ >= n_)
                return false;
            acc_ |= uint64_t(p_[pos_++]) << have_;
            have_ += 8;
        }
        v = uint32_t(acc_ & ((uint64_t(1) << count) - 1));
        acc_ >>= count;
        have_ -= count;
        return true;
    }
    void alignByte()
    {
        acc_ >>= (have_ & 7);
        have_ -= (have_ & 7);
    }
    bool byte(uint8_t& b)
    {
        uint32_t v;
        if (!bits(8, v))
            return false;
        b = uint8_t(v);
        return true;
    }

private:
    const uint8_t* p_;
    size_t n_, pos_ = 0;
    uint64_t acc_ = 0;
    int have_     = 0;
};

// Canonical Huffman code from code lengths (RFC 1951 3.2.2), decoded bit by bit.
struct Huffman
{
    uint16_t count[16] = {};
    std::vector<uint16_t> symbols;
    bool build(const uint8_t* lengths, int n)
    {
        std::memset(count, 0, sizeof count);
        for (int i = 0; i < n; i++)
            count[lengths[i]]++;
        count[0] = 0;
        int left = 1;
        for (int len = 1; len < 16; len++)
        {
            left <<= 1;
            left -= count[len];
            if (left < 0)
                return false; // over-subscribed
        }
        uint16_t offs[16] = {};
        for (int len = 1; len < 15; len++)
            offs[len + 1] = uint16_t(offs[len] + count[len]);
        symbols.assign(size_t(n), 0);
        for (int i = 0; i < n; i++)
            if (lengths[i])
                symbols[offs[lengths[i]]++] = uint16_t(i);
        return true;
    }
    bool decode(BitReader& br, int& sym) const
    {
        int code = 0, first = 0, index = 0;
        for (int len = 1; len < 16; len++)
        {
            uint32_t b;
            if (!br.bits(1, b))
                return false;
            code |= int(b);
            int c = count[len];
            if (code - c < first)
            {
                sym = symbols[size_t(index + (code - first))];
                return true;
            }
            index += c;
            first += c;
            first <<= 1;
            code <<= 1;
        }
        return false;
    }
};

const uint16_t kLenBase[29]  = { 3, 4, 5, 6, 7, 8, 9, 10, 11, 13, 15, 17, 19, 23, 27, 31, 35, 43, 51, 59, 67, 83,
    99, 115, 131, 163, 195, 227, 258 };
const uint8_t kLenExtra[29]  = { 0, 0, 0, 0, 0, 0, 0, 0, 1, 1, 1, 1, 2, 2, 2, 2, 3, 3, 3, 3, 4, 4, 4, 4, 5, 5, 5, 5, 0 };
const uint16_t kDistBase[30] = { 1, 2, 3, 4, 5, 7, 9, 13, 17, 25, 33, 49, 65, 97, 129, 193, 257, 385, 513, 769, 1025,
    1537, 2049, 3073, 4097, 6145, 8193, 12289, 16385, 24577 };
const uint8_t kDistExtra[30] = { 0, 0, 0, 0, 1, 1, 2, 2, 3, 3, 4, 4, 5, 5, 6, 6, 7, 7, 8, 8, 9, 9, 10, 10, 11, 11, 12,
    12, 13, 13 };

bool inflateCodes(BitReader& br, const Huffman& lit, const Huffman& dist, std::vector<uint8_t>& out, size_t limit)
{
    for (;;)
    {
        int sym;
        if (!lit.decode(br, sym))
            return false;
        if (sym < 256)
        {
            if (out.size() >= limit)
                return false;
            out.push_back(uint8_t(sym));
        }
        else if (sym == 256)
            return true;
        else
        {
            sym -= 257;
            if (sym >= 29)
                return false;
            uint32_t e;
            if (!br.bits(kLenExtra[sym], e))
                return false;
            size_t len = kLenBase[sym] + e;
            int ds;
            if (!dist.decode(br, ds) || ds >= 30)
                return false;
            if (!br.bits(kDistExtra[ds], e))
                return false;
            size_t d = kDistBase[ds] + e;
            if (d > out.size() || out.size() + len > limit)
                return false;
            size_t from = out.size() - d;
            for (size_t k = 0; k < len; k++)
                out.push_back(out[from + k]);
        }
    }
}

// A zlib stream (2-byte header, DEFLATE blocks, Adler-32) into at most `limit` bytes.
bool zlibInflate(const uint8_t* p, size_t n, std::vector<uint8_t>& out, size_t limit, std::string& error)
{
    if (n < 6 || (p[0] & 0x0F) != 8 || ((uint32_t(p[0]) << 8) | p[1]) % 31 != 0 || (p[1] & 0x20))
    {
        error = "not a zlib stream";
        return false;
    }
    BitReader br(p + 2, n - 2);
    bool last = false;
    while (!last)
    {
        uint32_t hdr;
        if (!br.bits(3, hdr))
        {
            error = "truncated DEFLATE stream";
            return false;
        }
        last         = hdr & 1;
        uint32_t type = hdr >> 1;
        if (type == 0)
        {
            br.alignByte();
            uint8_t b[4];
            for (auto& x : b)
                if (!br.byte(x))
                {
                    error = "truncated stored block";
                    return false;
                }
            uint32_t len = b[0] | (uint32_t(b[1]) << 8), nlen = b[2] | (uint32_t(b[3]) << 8);
            if ((len ^ 0xFFFFu) != nlen || out.size() + len > limit)
            {
                error = "bad stored block";
                return false;
            }
            for (uint32_t k = 0; k < len; k++)
            {
                uint8_t x;
                if (!br.byte(x))
                {
                    error = "truncated stored block";
                    return false;
                }
                out.push_back(x);
            }
            continue;
        }
        Huffman lit, dist;
        if (type == 1)
        {
            uint8_t l[288], d[30];
            for (int i = 0; i < 144; i++)
                l[i] = 8;
            for (int i = 144; i < 256; i++)
                l[i] = 9;
            for (int i = 256; i < 280; i++)
                l[i] = 7;
            for (int i = 280; i < 288; i++)
                l[i] = 8;
            for (int i = 0; i < 30; i++)
                d[i] = 5;
            lit.build(l, 288);
            dist.build(d, 30);
        }
        else if (type == 2)
        {
            uint32_t hlit, hdist, hclen;
            if (!br.bits(5, hlit) || !br.bits(5, hdist) || !br.bits(4, hclen))
            {
                error = "truncated dynamic block";
                return false;
            }
            hlit += 257;
            hdist += 1;
            hclen += 4;
            static const uint8_t kOrder[19] = { 16, 17, 18, 0, 8, 7, 9, 6, 10, 5, 11, 4, 12, 3, 13, 2, 14, 1, 15 };
            uint8_t cl[19] = {};
            for (uint32_t i = 0; i < hclen; i++)
            {
                uint32_t v;
                if (!br.bits(3, v))
                {
                    error = "truncated dynamic block";
                    return false;
                }
                cl[kOrder[i]] = uint8_t(v);
            }
            Huffman clh;
            if (!clh.build(cl, 19))
            {
                error = "bad code-length code";
                return false;
            }
            uint8_t lens[320] = {};
            uint32_t i = 0;
            while (i < hlit + hdist)
            {
                int sym;
                if (!clh.decode(br, sym))
                {
                    error = "bad code lengths";
                    return false;
                }
                if (sym < 16)
                    lens[i++] = uint8_t(sym);
                else
                {
                    uint32_t rep, prev = 0, extra;
                    if (sym == 16)
                    {
                        if (i == 0 || !br.bits(2, extra))
                        {
                            error = "bad repeat";
                            return false;
                        }
                        prev = lens[i - 1];
                        rep  = 3 + extra;
                    }
                    else if (sym == 17)
                    {
                        if (!br.bits(3, extra))
                            return false;
                        rep = 3 + extra;
                    }
                    else
                    {
                        if (!br.bits(7, extra))
                            return false;
                        rep = 11 + extra;
                    }
                    if (i + rep > hlit + hdist)
                    {
                        error = "code lengths overrun";
                        return false;
                    }
                    while (rep--)
                        lens[i++] = uint8_t(prev);
                }
            }
            if (!lit.build(lens, int(hlit)) || !dist.build(lens + hlit, int(hdist)))
            {
                error = "bad Huffman code";
                return false;
            }
        }
        else
        {
            error = "reserved DEFLATE block type";
            return false;
        }
        if (!inflateCodes(br, lit, dist, out, limit))
        {
            error = "corrupt DEFLATE data";
            return false;
        }
    }
    return true;
}

uint32_t be32(const uint8_t* p) { return (uint32_t(p[0]) << 24) | (uint32_t(p[1]) << 16) | (uint32_t(p[2]) << 8) | p[3]; }

int paeth(int a, int b, int c)
{
    int p = a + b - c, pa = p > a ? p - a : a - p, pb = p > b ? p - b : b - p, pc = p > c ? p - c : c - p;
    return (pa <= pb && pa <= pc) ? a : (pb <= pc ? b : c);
}

} // namespace

bool decodePNG(const std::string& data, std::vector<uint8_t>& rgba, int& width, int& height, std::string& error)
{
    static const uint8_t kSig[8] = { 0x89, 'P', 'N', 'G', '\r', '\n', 0x1A, '\n' };
    const uint8_t* p = reinterpret_cast<const uint8_t*>(data.data());
    size_t n         = data.size();
    if (n < 8 || std::memcmp(p, kSig, 8) != 0)
    {
        error = "not a PNG file";
        return false;
    }
    uint32_t w = 0, h = 0;
    int depth = 0, color = -1;
    std::vector<uint8_t> idat, palette, trns;
    bool ihdr = false;
    for (size_t at = 8; at + 12 <= n;)
    {
        uint32_t len = be32(p + at);
        if (len > n - at - 12)
        {
            error = "PNG chunk runs past the end of the file";
            return false;
        }
        const uint8_t* type = p + at + 4;
        const uint8_t* body = p + at + 8;
        if (!std::memcmp(type, "IHDR", 4) && len >= 13)
        {
            w     = be32(body);
            h     = be32(body + 4);
            depth = body[8];
            color = body[9];
            if (body[10] != 0 || body[11] != 0)
            {
                error = "unknown PNG compression or filter method";
                return false;
            }
            if (body[12] != 0)
            {
                error = "interlaced PNG images are not supported";
                return false;
            }
            ihdr = true;
        }
        else if (!std::memcmp(type, "PLTE", 4))
            palette.assign(body, body + len);
        else if (!std::memcmp(type, "tRNS", 4))
            trns.assign(body, body + len);
        else if (!std::memcmp(type, "IDAT", 4))
            idat.insert(idat.end(), body, body + len);
        else if (!std::memcmp(type, "IEND", 4))
            break;
        at += 12 + size_t(len);
    }
    const int channels = color == 0 ? 1 : color == 2 ? 3 : color == 3 ? 1 : color == 4 ? 2 : color == 6 ? 4 : 0;
    bool depthOk = depth == 8 || depth == 16 || ((color == 0 || color == 3) && (depth == 1 || depth == 2 || depth == 4));
    if (!ihdr || !channels || !depthOk || w == 0 || h == 0 || w > (1u << 15) || h > (1u << 15) ||
        (color == 3 && palette.size() < 3))
    {
        error = "unsupported or invalid PNG header";
        return false;
    }
    const size_t bitsPerPixel = size_t(channels) * size_t(depth);
    const size_t stride       = (size_t(w) * bitsPerPixel + 7) / 8;
    const size_t bpp          = (bitsPerPixel + 7) / 8; // filter byte distance
    if ((stride + 1) * size_t(h) > (size_t(1) << 30))
    {
        error = "PNG image too large (more than 1 GiB of scanlines)";
        return false;
    }
    std::vector<uint8_t> raw;
    raw.reserve((stride + 1) * h);
    if (!zlibInflate(idat.data(), idat.size(), raw, (stride + 1) * h, error))
        return false;
    if (raw.size() != (stride + 1) * h)
    {
        error = "PNG image data has the wrong size";
        return false;
    }
    std::vector<uint8_t> prev(stride, 0), cur(stride);
    rgba.assign(size_t(w) * h * 4, 0);
    for (uint32_t y = 0; y < h; y++)
    {
        const uint8_t* line = raw.data() + size_t(y) * (stride + 1);
        uint8_t f           = line[0];
        for (size_t i = 0; i < stride; i++)
        {
            int x = line[1 + i], a = i >= bpp ? cur[i - bpp] : 0, b = prev[i], c = i >= bpp ? prev[i - bpp] : 0;
            switch (f)
            {
            case 0: break;
            case 1: x += a; break;
            case 2: x += b; break;
            case 3: x += (a + b) / 2; break;
            case 4: x += paeth(a, b, c); break;
            default: error = "unknown PNG filter type"; return false;
            }
            cur[i] = uint8_t(x);
        }
        // Samples to 8-bit RGBA (16-bit: the high byte; grey scaled to 0-255).
        auto sample = [&](size_t idx) -> uint32_t {
            if (depth == 8)
                return cur[idx];
            if (depth == 16)
                return cur[idx * 2];
            size_t bit = idx * size_t(depth);
            return (cur[bit / 8] >> (8 - depth - int(bit % 8))) & ((1u << depth) - 1);
        };
        for (uint32_t x = 0; x < w; x++)
        {
            uint8_t* o = &rgba[(size_t(y) * w + x) * 4];
            if (color == 3)
            {
                uint32_t idx = sample(x);
                if (size_t(idx) * 3 + 2 >= palette.size())
                {
                    error = "PNG palette index out of range";
                    return false;
                }
                o[0] = palette[idx * 3];
                o[1] = palette[idx * 3 + 1];
                o[2] = palette[idx * 3 + 2];
                o[3] = idx < trns.size() ? trns[idx] : 255;
                continue;
            }
            uint32_t s[4];
            for (int k = 0; k < channels; k++)
                s[k] = sample(size_t(x) * channels + k);
            if (color == 0 || color == 4)
            {
                uint32_t g = depth < 8 ? s[0] * 255u / ((1u << depth) - 1u) : s[0];
                o[0] = o[1] = o[2] = uint8_t(g);
                o[3] = color == 4 ? uint8_t(s[1]) : 255;
            }
            else
            {
                o[0] = uint8_t(s[0]);
                o[1] = uint8_t(s[1]);
                o[2] = uint8_t(s[2]);
                o[3] = color == 6 ? uint8_t(s[3]) : 255;
            }
        }
        std::swap(prev, cur);
    }
    width  = int(w);
    height = int(h);
    return true;
}

bool loadPNGFile(const std::string& path, std::vector<uint8_t>& rgba, int& width, int& height, std::string& error)
{
    std::ifstream f(path, std::ios::binary);
    if (!f)
    {
        error = "cannot read " + path;
        return false;
    }
    std::ostringstream s;
    s << f.rdbuf();
    return decodePNG(s.str(), rgba, width, height, error);
}

} // namespace agb_aurora
