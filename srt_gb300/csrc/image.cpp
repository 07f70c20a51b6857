// image.cpp — film images on disk (Image::save_to_file, src/scene/texture.cu:
// 219-230 with save_ldr / save_hdr :132-168).  Host code only.
//
//   .png  8-bit RGBA, channels clamp(x, 0, 1) * 255 truncated (Image::f_to_u,
//         texture.cu:11-21); zlib stream of stored (uncompressed) deflate blocks
//   .bmp  24-bit BGR, same 8-bit conversion
//   .hdr  Radiance RGBE, flat (not run-length encoded) scanlines
//   .pfm  float RGB
// With `flip` set the image is mirrored in x and in y before it is written,
// as the reference's save_to_file does (texture.cu:221); the film's row 0 is
// the bottom of the picture, so png / bmp / hdr rows then run top to bottom.
// PFM stores its rows bottom to top, so it is written unflipped in y.
#include <algorithm>
#include <cctype>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <fstream>
#include <string>
#include <vector>

#include "common.h"

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

}  // namespace

using namespace srt;

extern "C" srt_status srt_image_write(const char* path, int32_t w, int32_t h, const float* rgba, int32_t flip)
{
    clear_error();
    if (!path || !rgba || w <= 0 || h <= 0) return set_error(SRT_ERR_ARG, "bad image arguments");
    const std::string ext = extension(path);
    if (ext != "png" && ext != "bmp" && ext != "hdr" && ext != "pfm")
        return set_error(SRT_ERR_UNSUPPORTED, "unsupported image format: " + ext + " (png, bmp, hdr, pfm)");
    // film pixel of the image's pixel (x, y), y counted from the first stored
    // row; mirror_y: the format stores rows top to bottom
    auto src = [&](int x, int y, bool mirror_y) -> const float* {
        const int sx = flip ? w - 1 - x : x;
        const int sy = (flip && mirror_y) ? h - 1 - y : y;
        return rgba + 4 * ((size_t)sy * w + sx);
    };
    std::ofstream f(path, std::ios::binary);
    if (!f) return set_error(SRT_ERR_ARG, std::string("cannot open ") + path);
    if (ext == "png" || ext == "bmp") {
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
