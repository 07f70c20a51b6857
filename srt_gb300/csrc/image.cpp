// image.cpp — film images on disk (Image::save_to_file, src/scene/texture.cu:
// 219-230 with save_exr / save_hdr / save_ldr :69-168, and
// Image::load_from_file :170-217 for float images).  Host code only.
//
//   .png  8-bit RGBA, channels clamp(x, 0, 1) * 255 truncated (Image::f_to_u,
//         texture.cu:11-21); zlib stream of stored (uncompressed) deflate blocks
//   .bmp  24-bit BGR, same 8-bit conversion
//   .jpg  baseline JPEG at quality 100 (4:4:4), same 8-bit conversion
//   .hdr  Radiance RGBE, flat (not run-length encoded) scanlines
//   .pfm  float RGB
//   .exr  OpenEXR scanline file, channels B, G, R, A stored as half, no
//         compression: the layout the reference's tinyexr call writes
//         (save_exr), float-to-half rounding ties away from zero as it does
// With `flip` set the image is mirrored in x and in y before it is written,
// as the reference's save_to_file does (texture.cu:221); the film's row 0 is
// the bottom of the picture, so png / bmp / hdr / exr rows then run top to
// bottom.  PFM stores its rows bottom to top, so it is written unflipped in y.
//
// Reading (srt_image_read) takes float images: OpenEXR (single-part
// scanline; half / float / uint channels; no compression, RLE, ZIPS, ZIP),
// Radiance HDR (flat or run-length scanlines, converted like stbi_loadf)
// and PFM.  `flip` undoes the writer's flip, as the reference's
// load_from_file(path, true, true) does for the Measure pass.
#include <algorithm>
#include <cctype>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <cstdio>
#include <fstream>
#include <functional>
#include <string>
#include <vector>

#include "common.h"
#include "inflate.h"
#include "jpeg.h"

using namespace srt;

namespace {

std::string extension(const std::string& path)
{
    size_t dot = path.find_last_of('.');
    std::string e = dot == std::string::npos ? std::string() : path.substr(dot + 1);
    for (char& c : e) c = (char)std::tolower((unsigned char)c);
    return e;
}

uint8_t to_u8(float v)
{
    // clamp(v, 0, 1) * 255 converted like make_uchar4(float): truncation; NaN gives 0
    if (!(v > 0.0f)) return 0;
    if (v >= 1.0f) return 255;
    return (uint8_t)(v * 255.0f);
}

// CRC-32 (ISO-HDLC polynomial 0xEDB88320, as PNG chunks use), table built once
uint32_t crc32(const uint8_t* p, size_t n)
{
    static uint32_t table[256];
    static bool init = false;
    if (!init) {
        for (uint32_t i = 0; i < 256; ++i) {
            uint32_t r = i;
            for (int k = 0; k < 8; ++k) r = (r & 1u) ? 0xEDB88320u ^ (r >> 1) : r >> 1;
            table[i] = r;
        }
        init = true;
    }
    uint32_t c = 0xffffffffu;
    for (size_t i = 0; i < n; ++i) c = table[(c ^ p[i]) & 0xffu] ^ (c >> 8);
    return c ^ 0xffffffffu;
}

void put_be32(std::vector<uint8_t>& v, uint32_t x)
{
    v.push_back((uint8_t)(x >> 24));
    v.push_back((uint8_t)(x >> 16));
    v.push_back((uint8_t)(x >> 8));
    v.push_back((uint8_t)x);
}

void png_chunk(std::vector<uint8_t>& out, const char* type, const std::vector<uint8_t>& data)
{
    put_be32(out, (uint32_t)data.size());
    std::vector<uint8_t> td(type, type + 4);
    td.insert(td.end(), data.begin(), data.end());
    out.insert(out.end(), td.begin(), td.end());
    put_be32(out, crc32(td.data(), td.size()));
}

std::vector<uint8_t> encode_png(int w, int h, const std::vector<uint8_t>& rgba_rows)
{
    // raw scanlines: filter byte 0 then w * 4 bytes
    std::vector<uint8_t> raw;
    raw.reserve((size_t)h * (w * 4 + 1));
    for (int y = 0; y < h; ++y) {
        raw.push_back(0);
        raw.insert(raw.end(), rgba_rows.begin() + (size_t)y * w * 4, rgba_rows.begin() + (size_t)(y + 1) * w * 4);
    }
    // zlib: CMF/FLG, stored deflate blocks of at most 65535 bytes, Adler-32
    std::vector<uint8_t> z = {0x78, 0x01};
    size_t pos = 0;
    do {
        const size_t len = std::min<size_t>(65535, raw.size() - pos);
        const bool last = pos + len == raw.size();
        z.push_back(last ? 1 : 0);
        z.push_back((uint8_t)(len & 0xff));
        z.push_back((uint8_t)(len >> 8));
        z.push_back((uint8_t)(~len & 0xff));
        z.push_back((uint8_t)((~len >> 8) & 0xff));
        z.insert(z.end(), raw.begin() + pos, raw.begin() + pos + len);
        pos += len;
    } while (pos < raw.size());
    uint32_t a = 1, b = 0;
    for (uint8_t x : raw) {
        a = (a + x) % 65521u;
        b = (b + a) % 65521u;
    }
    put_be32(z, (b << 16) | a);
    std::vector<uint8_t> out = {0x89, 'P', 'N', 'G', '\r', '\n', 0x1a, '\n'};
    std::vector<uint8_t> ihdr;
    put_be32(ihdr, (uint32_t)w);
    put_be32(ihdr, (uint32_t)h);
    ihdr.insert(ihdr.end(), {8, 6, 0, 0, 0});  // 8-bit RGBA, deflate, adaptive filters (all 0), no interlace
    png_chunk(out, "IHDR", ihdr);
    png_chunk(out, "IDAT", z);
    png_chunk(out, "IEND", {});
    return out;
}

// Radiance RGBE of one pixel (G. Ward, "Real Pixels", Graphics Gems II, 1991)
void rgbe(float r, float g, float b, uint8_t* out)
{
    const float v = std::max(r, std::max(g, b));
    if (!(v >= 1e-32f)) {
        out[0] = out[1] = out[2] = out[3] = 0;
        return;
    }
    int e;
    const float scale = std::frexp(v, &e) * 256.0f / v;
    out[0] = (uint8_t)std::max(0.0f, r * scale);
    out[1] = (uint8_t)std::max(0.0f, g * scale);
    out[2] = (uint8_t)std::max(0.0f, b * scale);
    out[3] = (uint8_t)(e + 128);
}

// ---- half floats -----------------------------------------------------------

// float -> IEEE binary16 with ties rounded away from zero (what the
// reference's EXR writer does; CUDA's __float2half_rn would round ties to
// even), overflow to infinity, float denormals to signed zero, NaN to the
// quiet NaN 0x7e00 with its sign.
uint16_t f32_to_f16(float f)
{
    uint32_t x;
    std::memcpy(&x, &f, 4);
    const uint16_t sign = (uint16_t)((x >> 16) & 0x8000u);
    const uint32_t e = (x >> 23) & 0xffu, m = x & 0x7fffffu;
    if (e == 0xffu) return sign | 0x7c00u | (m ? 0x200u : 0u);
    if (e == 0) return sign;
    const int he = (int)e - 127 + 15;
    if (he >= 31) return sign | 0x7c00u;
    if (he <= 0) {
        // subnormal half: the 24-bit significand shifted into units of 2^-24
        const int shift = 14 - he;
        if (shift > 24) return sign;
        const uint32_t mant = m | 0x800000u;
        uint32_t h = mant >> shift;
        if ((mant >> (shift - 1)) & 1u) ++h;
        return sign | (uint16_t)h;
    }
    uint32_t h = ((uint32_t)he << 10) | (m >> 13);
    if (m & 0x1000u) ++h;  // a carry into the exponent is the correct result (up to infinity)
    return sign | (uint16_t)h;
}

float f16_to_f32(uint16_t h)
{
    const uint32_t sign = (uint32_t)(h & 0x8000u) << 16;
    const uint32_t e = (h >> 10) & 0x1fu, m = h & 0x3ffu;
    uint32_t x;
    if (e == 0) {
        if (m == 0) {
            x = sign;
        } else {  // subnormal: renormalise
            int k = 0;
            uint32_t mm = m;
            while (!(mm & 0x400u)) {
                mm <<= 1;
                ++k;
            }
            x = sign | ((uint32_t)(127 - 15 - k + 1) << 23) | ((mm & 0x3ffu) << 13);
        }
    } else if (e == 31) {
        x = sign | 0x7f800000u | (m << 13);
    } else {
        x = sign | ((e - 15 + 127) << 23) | (m << 13);
    }
    float f;
    std::memcpy(&f, &x, 4);
    return f;
}

// ---- OpenEXR ------------------------------------------------------------------
// File layout from the OpenEXR file-format description: magic 20000630,
// version 2 with flags, attributes (name, type, size, value) ending in a
// zero byte, a table of 64-bit chunk offsets, then chunks (y, packed size,
// data); inside a scanline block the lines follow each other and each line
// holds every channel's row in channel-list order.

void put_le32(std::vector<uint8_t>& v, uint32_t x)
{
    for (int k = 0; k < 4; ++k) v.push_back((uint8_t)(x >> (8 * k)));
}

void put_attr(std::vector<uint8_t>& v, const char* name, const char* type, const std::vector<uint8_t>& value)
{
    v.insert(v.end(), name, name + std::strlen(name) + 1);
    v.insert(v.end(), type, type + std::strlen(type) + 1);
    put_le32(v, (uint32_t)value.size());
    v.insert(v.end(), value.begin(), value.end());
}

// header + offsets + uncompressed one-line chunks; `row(y)` gives the film
// row shown as image line y (top first), `col(x)` the film column
std::vector<uint8_t> encode_exr(int w, int h, const std::function<const float*(int, int)>& px)
{
    std::vector<uint8_t> f = {0x76, 0x2f, 0x31, 0x01, 2, 0, 0, 0};
    std::vector<uint8_t> ch;
    for (const char* n : {"B", "G", "R", "A"}) {
        ch.push_back((uint8_t)n[0]);
        ch.push_back(0);
        put_le32(ch, 1);  // HALF
        put_le32(ch, 0);  // pLinear + reserved
        put_le32(ch, 1);  // x sampling
        put_le32(ch, 1);  // y sampling
    }
    ch.push_back(0);
    put_attr(f, "channels", "chlist", ch);
    put_attr(f, "compression", "compression", {0});
    std::vector<uint8_t> box;
    for (uint32_t x : {0u, 0u, (uint32_t)(w - 1), (uint32_t)(h - 1)}) put_le32(box, x);
    put_attr(f, "dataWindow", "box2i", box);
    put_attr(f, "displayWindow", "box2i", box);
    put_attr(f, "lineOrder", "lineOrder", {0});
    const std::vector<uint8_t> one = {0, 0, 0x80, 0x3f};
    put_attr(f, "pixelAspectRatio", "float", one);
    put_attr(f, "screenWindowCenter", "v2f", std::vector<uint8_t>(8, 0));
    put_attr(f, "screenWindowWidth", "float", one);
    f.push_back(0);
    const size_t line = (size_t)w * 4 * 2;
    const size_t table = f.size();
    for (int y = 0; y < h; ++y) {
        const uint64_t off = table + 8 * (uint64_t)h + (uint64_t)y * (8 + line);
        for (int k = 0; k < 8; ++k) f.push_back((uint8_t)(off >> (8 * k)));
    }
    f.reserve(f.size() + (size_t)h * (8 + line));
    const int order[4] = {2, 1, 0, 3};  // B, G, R, A
    for (int y = 0; y < h; ++y) {
        put_le32(f, (uint32_t)y);
        put_le32(f, (uint32_t)line);
        for (int c : order)
            for (int x = 0; x < w; ++x) {
                const uint16_t v = f32_to_f16(px(x, y)[c]);
                f.push_back((uint8_t)v);
                f.push_back((uint8_t)(v >> 8));
            }
    }
    return f;
}

struct Reader {
    const std::vector<uint8_t>& b;
    size_t pos = 0;
    bool bad = false;
    uint32_t u32()
    {
        if (pos + 4 > b.size()) {
            bad = true;
            return 0;
        }
        uint32_t x = b[pos] | (uint32_t)b[pos + 1] << 8 | (uint32_t)b[pos + 2] << 16 | (uint32_t)b[pos + 3] << 24;
        pos += 4;
        return x;
    }
    uint64_t u64()
    {
        uint64_t lo = u32(), hi = u32();
        return lo | hi << 32;
    }
    std::string cstr()
    {
        size_t e = pos;
        while (e < b.size() && b[e]) ++e;
        if (e >= b.size()) {
            bad = true;
            return std::string();
        }
        std::string s(b.begin() + pos, b.begin() + e);
        pos = e + 1;
        return s;
    }
};

// undo the EXR byte predictor and the two-half interleave (ZIP and RLE)
void exr_unpredict(std::vector<uint8_t>& t, std::vector<uint8_t>& out)
{
    for (size_t i = 1; i < t.size(); ++i) t[i] = (uint8_t)(t[i - 1] + t[i] - 128);
    out.resize(t.size());
    const size_t half = (t.size() + 1) / 2;
    for (size_t i = 0; i < t.size(); ++i) out[i] = (i & 1) ? t[half + i / 2] : t[i / 2];
}

bool exr_rle(const uint8_t* in, size_t n, std::vector<uint8_t>& out, size_t limit)
{
    size_t i = 0;
    while (i < n) {
        const int c = (int8_t)in[i++];
        if (c < 0) {
            const size_t k = (size_t)(-c);
            if (i + k > n || out.size() + k > limit) return false;
            out.insert(out.end(), in + i, in + i + k);
            i += k;
        } else {
            if (i >= n || out.size() + c + 1 > limit) return false;
            out.insert(out.end(), (size_t)c + 1, in[i++]);
        }
    }
    return true;
}

srt_status read_exr(const std::vector<uint8_t>& b, const std::string& path, int& w, int& h, std::vector<float>& rgba)
{
    auto bad = [&](const std::string& why) { return set_error(SRT_ERR_PARSE, path + ": " + why); };
    Reader r{b};
    if (r.u32() != 20000630u) return bad("not an OpenEXR file");
    const uint32_t ver = r.u32();
    if ((ver & 0xff) != 2) return bad("unknown OpenEXR version");
    if (ver & 0x200u) return set_error(SRT_ERR_UNSUPPORTED, path + ": tiled OpenEXR files are not read");
    if (ver & 0x1800u) return set_error(SRT_ERR_UNSUPPORTED, path + ": deep or multi-part OpenEXR files are not read");
    struct Chan {
        std::string name;
        int type;
        int xs, ys;
    };
    std::vector<Chan> chans;
    int comp = -1;
    int32_t dw[4] = {0, 0, -1, -1};
    bool have_dw = false;
    for (;;) {
        std::string name = r.cstr();
        if (r.bad) return bad("truncated header");
        if (name.empty()) break;
        std::string type = r.cstr();
        const uint32_t size = r.u32();
        if (r.bad || r.pos + size > b.size()) return bad("truncated header");
        const size_t end = r.pos + size;
        if (name == "channels" && type == "chlist") {
            while (r.pos < end && b[r.pos]) {
                Chan c;
                c.name = r.cstr();
                c.type = (int)r.u32();
                r.u32();
                c.xs = (int)r.u32();
                c.ys = (int)r.u32();
                chans.push_back(c);
            }
        } else if (name == "compression") {
            comp = size >= 1 ? b[r.pos] : -1;
        } else if (name == "dataWindow" && size == 16) {
            for (int k = 0; k < 4; ++k) dw[k] = (int32_t)r.u32();
            have_dw = true;
        }
        r.pos = end;
    }
    if (!have_dw || chans.empty()) return bad("no dataWindow or channels");
    const int64_t W = (int64_t)dw[2] - dw[0] + 1, H = (int64_t)dw[3] - dw[1] + 1;
    if (W <= 0 || H <= 0 || W > (1 << 16) || H > (1 << 16)) return bad("bad dataWindow");
    int lines;
    if (comp == 0 || comp == 1 || comp == 2)
        lines = 1;
    else if (comp == 3)
        lines = 16;
    else
        return set_error(SRT_ERR_UNSUPPORTED, path + ": OpenEXR compression " + std::to_string(comp) +
                                                  " (none, RLE, ZIPS and ZIP are read)");
    size_t line_bytes = 0;
    for (const Chan& c : chans) {
        if (c.type < 0 || c.type > 2) return bad("unknown channel type");
        if (c.xs != 1 || c.ys != 1) return set_error(SRT_ERR_UNSUPPORTED, path + ": subsampled channels");
        line_bytes += (size_t)W * (c.type == 1 ? 2 : 4);
    }
    // which channel fills R, G, B, A (a lone channel is grey)
    int src[4] = {-1, -1, -1, -1};
    for (size_t i = 0; i < chans.size(); ++i) {
        const std::string& n = chans[i].name;
        if (n == "R") src[0] = (int)i;
        if (n == "G") src[1] = (int)i;
        if (n == "B") src[2] = (int)i;
        if (n == "A") src[3] = (int)i;
    }
    if (chans.size() == 1) src[0] = src[1] = src[2] = 0;
    if (src[0] < 0 || src[1] < 0 || src[2] < 0) return set_error(SRT_ERR_UNSUPPORTED, path + ": no R, G, B channels");
    const int64_t nchunks = (H + lines - 1) / lines;
    std::vector<uint64_t> offs((size_t)nchunks);
    for (auto& o : offs) o = r.u64();
    if (r.bad) return bad("truncated offset table");
    w = (int)W;
    h = (int)H;
    rgba.assign((size_t)W * H * 4, 0.0f);
    for (size_t i = 0; i < (size_t)W * H; ++i) rgba[4 * i + 3] = 1.0f;
    std::vector<uint8_t> raw, tmp;
    for (int64_t k = 0; k < nchunks; ++k) {
        r.pos = (size_t)offs[(size_t)k];
        const int32_t y0 = (int32_t)r.u32();
        const uint32_t packed = r.u32();
        if (r.bad || r.pos + packed > b.size()) return bad("truncated chunk");
        if (y0 < dw[1] || y0 > dw[3]) return bad("chunk outside the dataWindow");
        const int nl = (int)std::min<int64_t>(lines, (int64_t)dw[3] - y0 + 1);
        const size_t want = line_bytes * nl;
        const uint8_t* d = b.data() + r.pos;
        raw.clear();
        if (comp == 0 || packed == want) {  // stored as is (also a block that did not compress)
            if (packed != want) return bad("chunk size");
            raw.assign(d, d + packed);
        } else {
            tmp.clear();
            const bool ok = comp == 1 ? exr_rle(d, packed, tmp, want) : inflate_zlib(d, packed, tmp, want);
            if (!ok || tmp.size() != want) return bad("corrupt compressed chunk");
            exr_unpredict(tmp, raw);
        }
        size_t at = 0;
        for (int l = 0; l < nl; ++l) {
            const int64_t row = (int64_t)y0 - dw[1] + l;
            for (size_t c = 0; c < chans.size(); ++c) {
                const int t = chans[c].type, sz = t == 1 ? 2 : 4;
                for (int64_t x = 0; x < W; ++x) {
                    const uint8_t* q = &raw[at + (size_t)x * sz];
                    float v;
                    if (t == 1) {
                        v = f16_to_f32((uint16_t)(q[0] | q[1] << 8));
                    } else {
                        uint32_t u = q[0] | (uint32_t)q[1] << 8 | (uint32_t)q[2] << 16 | (uint32_t)q[3] << 24;
                        if (t == 2)
                            std::memcpy(&v, &u, 4);
                        else
                            v = (float)u;
                    }
                    for (int o = 0; o < 4; ++o)
                        if (src[o] == (int)c) rgba[4 * ((size_t)row * W + x) + o] = v;
                }
                at += (size_t)W * sz;
            }
        }
    }
    return SRT_OK;
}

// ---- Radiance HDR (read) ------------------------------------------------------

srt_status read_hdr(const std::vector<uint8_t>& b, const std::string& path, int& w, int& h, std::vector<float>& rgba)
{
    auto bad = [&](const std::string& why) { return set_error(SRT_ERR_PARSE, path + ": " + why); };
    size_t pos = 0;
    auto line = [&]() {
        std::string s;
        while (pos < b.size() && b[pos] != '\n') s.push_back((char)b[pos++]);
        ++pos;
        return s;
    };
    std::string first = line();
    if (first != "#?RADIANCE" && first != "#?RGBE") return bad("not a Radiance HDR file");
    for (;;) {
        if (pos >= b.size()) return bad("truncated header");
        std::string l = line();
        if (l.empty()) break;
        if (l.compare(0, 7, "FORMAT=") == 0 && l != "FORMAT=32-bit_rle_rgbe") return bad("unsupported " + l);
    }
    std::string res = line();
    int hh = 0, ww = 0;
    char ys[3] = {}, xs[3] = {};
    if (std::sscanf(res.c_str(), "%2s %d %2s %d", ys, &hh, xs, &ww) != 4 || std::string(ys) != "-Y" ||
        std::string(xs) != "+X")
        return set_error(SRT_ERR_UNSUPPORTED, path + ": HDR orientation other than -Y +X");
    if (ww <= 0 || hh <= 0 || ww > (1 << 16) || hh > (1 << 16)) return bad("bad size");
    w = ww;
    h = hh;
    rgba.assign((size_t)w * h * 4, 1.0f);
    std::vector<uint8_t> sl((size_t)w * 4);
    for (int y = 0; y < h; ++y) {
        const bool rle = w >= 8 && w < 32768 && pos + 4 <= b.size() && b[pos] == 2 && b[pos + 1] == 2 &&
                         (b[pos + 2] << 8 | b[pos + 3]) == w;
        if (rle) {
            pos += 4;
            for (int c = 0; c < 4; ++c) {
                int x = 0;
                while (x < w) {
                    if (pos >= b.size()) return bad("truncated scanline");
                    int n = b[pos++];
                    if (n > 128) {
                        n -= 128;
                        if (pos >= b.size() || x + n > w) return bad("bad run");
                        for (int k = 0; k < n; ++k) sl[4 * (x + k) + c] = b[pos];
                        ++pos;
                    } else {
                        if (n == 0 || x + n > w || pos + n > b.size()) return bad("bad run");
                        for (int k = 0; k < n; ++k) sl[4 * (x + k) + c] = b[pos + k];
                        pos += n;
                    }
                    x += n;
                }
            }
        } else {
            if (pos + sl.size() > b.size()) return bad("truncated scanline");
            std::memcpy(sl.data(), &b[pos], sl.size());
            pos += sl.size();
        }
        for (int x = 0; x < w; ++x) {
            const uint8_t* e = &sl[4 * (size_t)x];
            float* o = &rgba[4 * ((size_t)y * w + x)];
            // RGBE to float as stbi_loadf does: mantissa * 2^(exponent - 136), no half-unit offset
            const float f = e[3] ? std::ldexp(1.0f, (int)e[3] - 136) : 0.0f;
            for (int c = 0; c < 3; ++c) o[c] = e[c] * f;
        }
    }
    return SRT_OK;
}

// ---- PFM (read) ---------------------------------------------------------------

srt_status read_pfm(const std::vector<uint8_t>& b, const std::string& path, int& w, int& h, std::vector<float>& rgba)
{
    auto bad = [&](const std::string& why) { return set_error(SRT_ERR_PARSE, path + ": " + why); };
    std::string head(b.begin(), b.begin() + std::min<size_t>(b.size(), 256));
    char magic[3] = {};
    int ww = 0, hh = 0, used = 0;
    double scale = 0.0;
    if (std::sscanf(head.c_str(), "%2s %d %d %lf%n", magic, &ww, &hh, &scale, &used) != 4) return bad("bad PFM header");
    const int ch = std::string(magic) == "PF" ? 3 : std::string(magic) == "Pf" ? 1 : 0;
    if (!ch || ww <= 0 || hh <= 0 || ww > (1 << 16) || hh > (1 << 16)) return bad("bad PFM header");
    const size_t start = (size_t)used + 1;  // one whitespace byte after the scale
    const size_t n = (size_t)ww * hh * ch;
    if (start + 4 * n > b.size()) return bad("truncated PFM data");
    w = ww;
    h = hh;
    rgba.assign((size_t)w * h * 4, 1.0f);
    const bool big = scale > 0.0;
    for (size_t i = 0; i < (size_t)w * h; ++i)
        for (int c = 0; c < 3; ++c) {
            const uint8_t* q = &b[start + 4 * (i * ch + (ch == 3 ? c : 0))];
            uint32_t u = big ? ((uint32_t)q[0] << 24 | (uint32_t)q[1] << 16 | (uint32_t)q[2] << 8 | q[3])
                             : (q[0] | (uint32_t)q[1] << 8 | (uint32_t)q[2] << 16 | (uint32_t)q[3] << 24);
            std::memcpy(&rgba[4 * i + c], &u, 4);
        }
    return SRT_OK;
}

// ---- PNG (read, 8 bits per channel out) -----------------------------------------
// From the PNG specification: chunks, zlib-compressed scanlines with one
// filter byte each (None, Sub, Up, Average, Paeth), Adam7 interlacing, and
// the conversions to 8-bit RGBA that stbi_load(..., 4) makes: low bit depths
// scaled to 0..255, 16-bit samples cut to their high byte, palette and tRNS
// transparency applied.

uint32_t be32(const uint8_t* p) { return (uint32_t)p[0] << 24 | (uint32_t)p[1] << 16 | (uint32_t)p[2] << 8 | p[3]; }

int paeth(int a, int b, int c)
{
    const int p = a + b - c, pa = std::abs(p - a), pb = std::abs(p - b), pc = std::abs(p - c);
    return (pa <= pb && pa <= pc) ? a : (pb <= pc ? b : c);
}

srt_status read_png(const std::vector<uint8_t>& b, const std::string& path, int& w, int& h, std::vector<uint8_t>& rgba)
{
    auto bad = [&](const std::string& why) { return set_error(SRT_ERR_PARSE, path + ": " + why); };
    static const uint8_t sig[8] = {0x89, 'P', 'N', 'G', '\r', '\n', 0x1a, '\n'};
    if (b.size() < 8 || std::memcmp(b.data(), sig, 8) != 0) return bad("not a PNG file");
    size_t pos = 8;
    int depth = 0, ctype = -1, interlace = 0;
    std::vector<uint8_t> idat, plte, trns;
    bool ihdr = false;
    while (pos + 12 <= b.size()) {
        const uint32_t len = be32(&b[pos]);
        const std::string type(b.begin() + pos + 4, b.begin() + pos + 8);
        if (pos + 12 + (size_t)len > b.size()) return bad("truncated chunk");
        const uint8_t* d = &b[pos + 8];
        if (type == "IHDR") {
            if (len < 13) return bad("short IHDR");
            w = (int)be32(d);
            h = (int)be32(d + 4);
            depth = d[8];
            ctype = d[9];
            interlace = d[12];
            ihdr = true;
            if (d[10] != 0 || d[11] != 0 || interlace > 1) return bad("unknown compression, filter or interlace");
        } else if (type == "PLTE") {
            plte.assign(d, d + len);
        } else if (type == "tRNS") {
            trns.assign(d, d + len);
        } else if (type == "IDAT") {
            idat.insert(idat.end(), d, d + len);
        } else if (type == "IEND") {
            break;
        }
        pos += 12 + (size_t)len;
    }
    if (!ihdr || w <= 0 || h <= 0 || w > (1 << 16) || h > (1 << 16)) return bad("bad IHDR");
    int ch;
    switch (ctype) {
    case 0: ch = 1; break;
    case 2: ch = 3; break;
    case 3: ch = 1; break;
    case 4: ch = 2; break;
    case 6: ch = 4; break;
    default: return bad("unknown colour type");
    }
    const bool depth_ok = (ctype == 0 && (depth == 1 || depth == 2 || depth == 4 || depth == 8 || depth == 16)) ||
                          (ctype == 3 && (depth == 1 || depth == 2 || depth == 4 || depth == 8)) ||
                          ((ctype == 2 || ctype == 4 || ctype == 6) && (depth == 8 || depth == 16));
    if (!depth_ok) return bad("bad bit depth");
    if (ctype == 3 && (plte.empty() || plte.size() % 3)) return bad("missing palette");
    const int bits_px = ch * depth, bpp = std::max(1, bits_px / 8);
    // raw size over the (one or seven) passes
    static const int ax0[7] = {0, 4, 0, 2, 0, 1, 0}, ay0[7] = {0, 0, 4, 0, 2, 0, 1};
    static const int adx[7] = {8, 8, 4, 4, 2, 2, 1}, ady[7] = {8, 8, 8, 4, 4, 2, 2};
    const int passes = interlace ? 7 : 1;
    size_t need = 0;
    int pw[7], ph[7];
    for (int p = 0; p < passes; ++p) {
        pw[p] = interlace ? (w - ax0[p] + adx[p] - 1) / adx[p] : w;
        ph[p] = interlace ? (h - ay0[p] + ady[p] - 1) / ady[p] : h;
        if (pw[p] > 0 && ph[p] > 0) need += (size_t)ph[p] * (1 + ((size_t)pw[p] * bits_px + 7) / 8);
    }
    std::vector<uint8_t> raw;
    if (!inflate_zlib(idat.data(), idat.size(), raw, need) || raw.size() != need) return bad("corrupt image data");
    // samples of the whole image, as 16-bit values before the 8-bit cut
    std::vector<uint16_t> smp((size_t)w * h * ch);
    size_t at = 0;
    for (int p = 0; p < passes; ++p) {
        if (pw[p] <= 0 || ph[p] <= 0) continue;
        const size_t stride = ((size_t)pw[p] * bits_px + 7) / 8;
        std::vector<uint8_t> prev(stride, 0), cur(stride);
        for (int y = 0; y < ph[p]; ++y) {
            const int ft = raw[at++];
            for (size_t i = 0; i < stride; ++i) {
                const int x = raw[at + i];
                const int a = i >= (size_t)bpp ? cur[i - bpp] : 0, up = prev[i], c = i >= (size_t)bpp ? prev[i - bpp] : 0;
                int v;
                switch (ft) {
                case 0: v = x; break;
                case 1: v = x + a; break;
                case 2: v = x + up; break;
                case 3: v = x + ((a + up) >> 1); break;
                case 4: v = x + paeth(a, up, c); break;
                default: return bad("unknown filter type");
                }
                cur[i] = (uint8_t)v;
            }
            at += stride;
            const int iy = interlace ? ay0[p] + y * ady[p] : y;
            for (int x = 0; x < pw[p]; ++x) {
                const int ix = interlace ? ax0[p] + x * adx[p] : x;
                for (int c = 0; c < ch; ++c) {
                    uint16_t v;
                    if (depth == 16) {
                        const size_t o = ((size_t)x * ch + c) * 2;
                        v = (uint16_t)(cur[o] << 8 | cur[o + 1]);
                    } else if (depth == 8) {
                        v = cur[(size_t)x * ch + c];
                    } else {
                        const size_t bit = (size_t)x * depth;  // one channel
                        v = (uint16_t)((cur[bit / 8] >> (8 - depth - bit % 8)) & ((1 << depth) - 1));
                    }
                    smp[((size_t)iy * w + ix) * ch + c] = v;
                }
            }
            std::swap(prev, cur);
        }
    }
    rgba.assign((size_t)w * h * 4, 255);
    const int scale = depth == 1 ? 255 : depth == 2 ? 85 : depth == 4 ? 17 : 1;
    for (size_t i = 0; i < (size_t)w * h; ++i) {
        const uint16_t* s = &smp[i * ch];
        uint8_t* o = &rgba[4 * i];
        auto to8 = [&](uint16_t v) { return (uint8_t)(depth == 16 ? v >> 8 : v * scale); };
        if (ctype == 3) {
            const size_t k = s[0];
            if (3 * k + 2 >= plte.size()) return bad("palette index out of range");
            o[0] = plte[3 * k];
            o[1] = plte[3 * k + 1];
            o[2] = plte[3 * k + 2];
            o[3] = k < trns.size() ? trns[k] : 255;
            continue;
        }
        if (ch <= 2) {
            o[0] = o[1] = o[2] = to8(s[0]);
            if (ch == 2) o[3] = to8(s[1]);
        } else {
            for (int c = 0; c < ch; ++c) o[c] = to8(s[c]);
        }
        // a tRNS key colour makes matching pixels transparent (compared before the 8-bit cut)
        if (ctype == 0 && trns.size() >= 2 && s[0] == (uint16_t)(trns[0] << 8 | trns[1])) o[3] = 0;
        if (ctype == 2 && trns.size() >= 6 && s[0] == (uint16_t)(trns[0] << 8 | trns[1]) &&
            s[1] == (uint16_t)(trns[2] << 8 | trns[3]) && s[2] == (uint16_t)(trns[4] << 8 | trns[5]))
            o[3] = 0;
    }
    return SRT_OK;
}

// ---- BMP (read): uncompressed 24- and 32-bit --------------------------------------

srt_status read_bmp(const std::vector<uint8_t>& b, const std::string& path, int& w, int& h, std::vector<uint8_t>& rgba)
{
    auto bad = [&](const std::string& why) { return set_error(SRT_ERR_PARSE, path + ": " + why); };
    auto le32 = [&](size_t o) { return (uint32_t)b[o] | (uint32_t)b[o + 1] << 8 | (uint32_t)b[o + 2] << 16 | (uint32_t)b[o + 3] << 24; };
    if (b.size() < 54 || b[0] != 'B' || b[1] != 'M') return bad("not a BMP file");
    const uint32_t off = le32(10);
    const int32_t bw = (int32_t)le32(18), bh = (int32_t)le32(22);
    const int bitc = b[28] | b[29] << 8;
    const uint32_t comp = le32(30);
    if ((bitc != 24 && bitc != 32) || (comp != 0 && !(comp == 3 && bitc == 32)))
        return set_error(SRT_ERR_UNSUPPORTED, path + ": only uncompressed 24- and 32-bit BMP files are read");
    if (bw <= 0 || bh == 0 || bw > (1 << 16) || std::abs(bh) > (1 << 16)) return bad("bad size");
    w = bw;
    h = std::abs(bh);
    const size_t row = ((size_t)w * (bitc / 8) + 3) & ~(size_t)3;
    if (off + row * h > b.size()) return bad("truncated pixel data");
    rgba.assign((size_t)w * h * 4, 255);
    for (int y = 0; y < h; ++y) {
        const int sy = bh > 0 ? h - 1 - y : y;  // positive height: rows stored bottom to top
        const uint8_t* r = &b[off + (size_t)sy * row];
        for (int x = 0; x < w; ++x) {
            const uint8_t* q = r + (size_t)x * (bitc / 8);
            uint8_t* o = &rgba[4 * ((size_t)y * w + x)];
            o[0] = q[2];
            o[1] = q[1];
            o[2] = q[0];
            if (bitc == 32) o[3] = q[3];
        }
    }
    return SRT_OK;
}

}  // namespace

extern "C" srt_status srt_image_write(const char* path, int32_t w, int32_t h, const float* rgba, int32_t flip)
{
    clear_error();
    if (!path || !rgba || w <= 0 || h <= 0) return set_error(SRT_ERR_ARG, "bad image arguments");
    const std::string ext = extension(path);
    if (ext != "png" && ext != "bmp" && ext != "jpg" && ext != "jpeg" && ext != "hdr" && ext != "pfm" && ext != "exr")
        return set_error(SRT_ERR_UNSUPPORTED, "unsupported image format: " + ext + " (png, bmp, jpg, hdr, pfm, exr)");
    // film pixel of the image's pixel (x, y), y counted from the first stored
    // row; mirror_y: the format stores rows top to bottom
    auto src = [&](int x, int y, bool mirror_y) -> const float* {
        const int sx = flip ? w - 1 - x : x;
        const int sy = (flip && mirror_y) ? h - 1 - y : y;
        return rgba + 4 * ((size_t)sy * w + sx);
    };
    std::ofstream f(path, std::ios::binary);
    if (!f) return set_error(SRT_ERR_ARG, std::string("cannot open ") + path);
    if (ext == "exr") {
        std::vector<uint8_t> exr = encode_exr(w, h, [&](int x, int y) { return src(x, y, true); });
        f.write(reinterpret_cast<const char*>(exr.data()), (std::streamsize)exr.size());
    } else if (ext == "png" || ext == "bmp" || ext == "jpg" || ext == "jpeg") {
        std::vector<uint8_t> px((size_t)w * h * 4);
        for (int y = 0; y < h; ++y)
            for (int x = 0; x < w; ++x) {
                const float* p = src(x, y, true);
                uint8_t* q = &px[4 * ((size_t)y * w + x)];
                for (int c = 0; c < 4; ++c) q[c] = to_u8(p[c]);
            }
        if (ext == "png") {
            std::vector<uint8_t> png = encode_png(w, h, px);
            f.write(reinterpret_cast<const char*>(png.data()), (std::streamsize)png.size());
        } else if (ext == "jpg" || ext == "jpeg") {
            // stbi_write_jpg(..., 100) in save_ldr (texture.cu:157-158)
            std::vector<uint8_t> jpg = jpeg_encode(w, h, px.data(), 100);
            f.write(reinterpret_cast<const char*>(jpg.data()), (std::streamsize)jpg.size());
        } else {
            const int row = (w * 3 + 3) & ~3;
            const uint32_t size = 54u + (uint32_t)row * (uint32_t)h;
            uint8_t hd[54] = {'B', 'M'};
            auto le32 = [&](int o, uint32_t v) {
                for (int k = 0; k < 4; ++k) hd[o + k] = (uint8_t)(v >> (8 * k));
            };
            le32(2, size);
            le32(10, 54);
            le32(14, 40);
            le32(18, (uint32_t)w);
            le32(22, (uint32_t)h);  // positive height: rows stored bottom to top
            hd[26] = 1;
            hd[28] = 24;
            le32(34, (uint32_t)row * (uint32_t)h);
            f.write(reinterpret_cast<const char*>(hd), 54);
            std::vector<uint8_t> line((size_t)row, 0);
            for (int y = h - 1; y >= 0; --y) {
                for (int x = 0; x < w; ++x) {
                    const uint8_t* q = &px[4 * ((size_t)y * w + x)];
                    line[3 * x] = q[2];
                    line[3 * x + 1] = q[1];
                    line[3 * x + 2] = q[0];
                }
                f.write(reinterpret_cast<const char*>(line.data()), row);
            }
        }
    } else if (ext == "hdr") {
        f << "#?RADIANCE\nFORMAT=32-bit_rle_rgbe\n\n-Y " << h << " +X " << w << "\n";
        std::vector<uint8_t> line((size_t)w * 4);
        for (int y = 0; y < h; ++y) {
            for (int x = 0; x < w; ++x) {
                const float* p = src(x, y, true);
                rgbe(p[0], p[1], p[2], &line[4 * (size_t)x]);
            }
            f.write(reinterpret_cast<const char*>(line.data()), (std::streamsize)line.size());
        }
    } else {
        f << "PF\n" << w << " " << h << "\n-1.0\n";
        std::vector<float> line((size_t)w * 3);
        for (int y = 0; y < h; ++y) {
            for (int x = 0; x < w; ++x) {
                const float* p = src(x, y, false);
                for (int c = 0; c < 3; ++c) line[3 * (size_t)x + c] = p[c];
            }
            f.write(reinterpret_cast<const char*>(line.data()), (std::streamsize)(line.size() * 4));
        }
    }
    return f ? SRT_OK : set_error(SRT_ERR_ARG, std::string("write failed: ") + path);
}

extern "C" srt_status srt_image_read(const char* path, int32_t* width, int32_t* height, float* rgba, int32_t flip)
{
    clear_error();
    if (!path || !width || !height) return set_error(SRT_ERR_ARG, "NULL argument");
    std::ifstream f(path, std::ios::binary);
    if (!f) return set_error(SRT_ERR_ARG, std::string("Failed to open file: ") + path);
    std::vector<uint8_t> b((std::istreambuf_iterator<char>(f)), std::istreambuf_iterator<char>());
    int w = 0, h = 0;
    std::vector<float> px;
    bool bottom_up = false;  // PFM rows run bottom to top, like the film's
    if (b.size() >= 4 && b[0] == 0x76 && b[1] == 0x2f && b[2] == 0x31 && b[3] == 0x01) {
        SRT_TRY(read_exr(b, path, w, h, px));
    } else if (b.size() >= 2 && b[0] == '#' && b[1] == '?') {
        SRT_TRY(read_hdr(b, path, w, h, px));
    } else if (b.size() >= 2 && b[0] == 'P' && (b[1] == 'F' || b[1] == 'f')) {
        SRT_TRY(read_pfm(b, path, w, h, px));
        bottom_up = true;
    } else {
        return set_error(SRT_ERR_UNSUPPORTED, std::string(path) + ": not a float image (exr, hdr, pfm)");
    }
    *width = w;
    *height = h;
    if (!rgba) return SRT_OK;
    // Image::flip(flip_x, flip_y) for the top-to-bottom formats; PFM rows
    // already run bottom to top, so its y flip is the identity
    const bool fx = flip == SRT_FLIP_XY, fy = (flip == SRT_FLIP_XY || flip == SRT_FLIP_Y) && !bottom_up;
    for (int y = 0; y < h; ++y)
        for (int x = 0; x < w; ++x) {
            const int sx = fx ? w - 1 - x : x;
            const int sy = fy ? h - 1 - y : y;
            std::memcpy(rgba + 4 * ((size_t)y * w + x), &px[4 * ((size_t)sy * w + sx)], 16);
        }
    return SRT_OK;
}

extern "C" srt_status srt_image_read_rgba8(const char* path, int32_t* width, int32_t* height, uint8_t* rgba,
                                           int32_t flip)
{
    clear_error();
    if (!path || !width || !height) return set_error(SRT_ERR_ARG, "NULL argument");
    std::ifstream f(path, std::ios::binary);
    if (!f) return set_error(SRT_ERR_ARG, std::string("Failed to open file: ") + path);
    std::vector<uint8_t> b((std::istreambuf_iterator<char>(f)), std::istreambuf_iterator<char>());
    int w = 0, h = 0;
    std::vector<uint8_t> px;
    if (b.size() >= 8 && b[0] == 0x89 && b[1] == 'P' && b[2] == 'N' && b[3] == 'G') {
        SRT_TRY(read_png(b, path, w, h, px));
    } else if (b.size() >= 2 && b[0] == 'B' && b[1] == 'M') {
        SRT_TRY(read_bmp(b, path, w, h, px));
    } else if (b.size() >= 3 && b[0] == 0xFF && b[1] == 0xD8 && b[2] == 0xFF) {
        SRT_TRY(jpeg_decode(b, path, w, h, px));
    } else {
        return set_error(SRT_ERR_UNSUPPORTED, std::string(path) + ": not an 8-bit image this library reads (png, bmp, jpg)");
    }
    *width = w;
    *height = h;
    if (!rgba) return SRT_OK;
    // Image::flip(flip_x, flip_y): SRT_FLIP_XY mirrors both, SRT_FLIP_Y rows only
    const bool fx = flip == SRT_FLIP_XY, fy = flip == SRT_FLIP_XY || flip == SRT_FLIP_Y;
    for (int y = 0; y < h; ++y)
        for (int x = 0; x < w; ++x) {
            const int sx = fx ? w - 1 - x : x, sy = fy ? h - 1 - y : y;
            std::memcpy(rgba + 4 * ((size_t)y * w + x), &px[4 * ((size_t)sy * w + sx)], 4);
        }
    return SRT_OK;
}
