// jpeg.cpp — baseline JPEG written from ITU-T T.81: marker parsing, Huffman
// entropy coding (Annex C / F), the 8x8 DCT by its defining sums, JFIF
// YCbCr colour, and for chroma upsampling the triangle ("fancy") filter.
// Host code.
#include "jpeg.h"

#include <algorithm>
#include <cmath>
#include <cstring>

namespace srt {
namespace {

// natural (row-major) index of the k-th coefficient in zigzag order
const int kZigzag[64] = {0,  1,  8,  16, 9,  2,  3,  10, 17, 24, 32, 25, 18, 11, 4,  5,  12, 19, 26, 33, 40, 48,
                         41, 34, 27, 20, 13, 6,  7,  14, 21, 28, 35, 42, 49, 56, 57, 50, 43, 36, 29, 22, 15, 23,
                         30, 37, 44, 51, 58, 59, 52, 45, 38, 31, 39, 46, 53, 60, 61, 54, 47, 55, 62, 63};

// cos((2x + 1) u pi / 16) * C(u) / 2, the separable DCT basis
struct DctBasis {
    double c[8][8];  // [u][x]
    DctBasis()
    {
        for (int u = 0; u < 8; ++u)
            for (int x = 0; x < 8; ++x)
                c[u][x] = (u == 0 ? std::sqrt(0.5) : 1.0) * 0.5 * std::cos((2 * x + 1) * u * M_PI / 16.0);
    }
};
const DctBasis& basis()
{
    static const DctBasis b;
    return b;
}

uint8_t clamp8(double v)
{
    const double r = std::floor(v + 0.5);
    return (uint8_t)std::min(255.0, std::max(0.0, r));
}

// ---- decoding --------------------------------------------------------------------------

struct Huff {
    int mincode[17], maxcode[18], valptr[17];
    uint8_t vals[256];
    bool present = false;
    bool build(const uint8_t* bits, const uint8_t* v, int nv)
    {
        int code = 0, k = 0;
        for (int l = 1; l <= 16; ++l) {
            valptr[l] = k;
            mincode[l] = code;
            code += bits[l - 1];
            k += bits[l - 1];
            maxcode[l] = bits[l - 1] ? code - 1 : -1;
            if (code > (1 << l)) return false;  // over-subscribed
            code <<= 1;
        }
        maxcode[17] = 0x7fffffff;
        if (k != nv || nv > 256) return false;
        std::memcpy(vals, v, (size_t)nv);
        present = true;
        return true;
    }
};

struct Component {
    int id, h, v, tq;
    int td = 0, ta = 0;
    int bw = 0, bh = 0;          // blocks per line / column, padded to whole MCUs
    std::vector<uint8_t> plane;  // bw*8 x bh*8 samples
    int pred = 0;
};

struct BitIn {
    const std::vector<uint8_t>& b;
    size_t pos;
    uint32_t acc = 0;
    int n = 0;
    bool marker = false;  // a marker was met: further bits are zeros
    int getbit()
    {
        if (n == 0) {
            uint32_t byte = 0;
            if (!marker && pos < b.size()) {
                byte = b[pos];
                if (byte == 0xFF) {
                    const uint8_t nx = pos + 1 < b.size() ? b[pos + 1] : 0;
                    if (nx == 0x00) {
                        pos += 2;
                    } else {
                        marker = true;
                        byte = 0;
                    }
                } else {
                    ++pos;
                }
            }
            acc = byte;
            n = 8;
        }
        --n;
        return (int)((acc >> n) & 1u);
    }
    int getbits(int s)
    {
        int v = 0;
        for (int i = 0; i < s; ++i) v = (v << 1) | getbit();
        return v;
    }
    void reset()  // byte-align and step over an RSTn marker
    {
        n = 0;
        marker = false;
        if (pos + 1 < b.size() && b[pos] == 0xFF && b[pos + 1] >= 0xD0 && b[pos + 1] <= 0xD7) pos += 2;
    }
};

int huff_decode(BitIn& in, const Huff& h)
{
    int code = 0;
    for (int l = 1; l <= 16; ++l) {
        code = (code << 1) | in.getbit();
        if (code <= h.maxcode[l]) return h.vals[h.valptr[l] + code - h.mincode[l]];
    }
    return -1;
}

int extend(int v, int s) { return s == 0 ? 0 : (v < (1 << (s - 1)) ? v - (1 << s) + 1 : v); }

// inverse DCT of one dequantised block (natural order) into 8x8 samples
void idct_block(const int* coef, uint8_t* out, int stride)
{
    const DctBasis& B = basis();
    double tmp[8][8];
    for (int v = 0; v < 8; ++v)  // rows of coefficients -> spatial x
        for (int x = 0; x < 8; ++x) {
            double s = 0.0;
            for (int u = 0; u < 8; ++u) s += B.c[u][x] * coef[v * 8 + u];
            tmp[v][x] = s;
        }
    for (int x = 0; x < 8; ++x)
        for (int y = 0; y < 8; ++y) {
            double s = 0.0;
            for (int v = 0; v < 8; ++v) s += B.c[v][y] * tmp[v][x];
            out[y * stride + x] = clamp8(s + 128.0);
        }
}

}  // namespace

srt_status jpeg_decode(const std::vector<uint8_t>& b, const std::string& path, int& w, int& h, std::vector<uint8_t>& rgba)
{
    auto bad = [&](const std::string& why) { return set_error(SRT_ERR_PARSE, path + ": " + why); };
    auto unsupported = [&](const std::string& why) { return set_error(SRT_ERR_UNSUPPORTED, path + ": " + why); };
    if (b.size() < 4 || b[0] != 0xFF || b[1] != 0xD8) return bad("not a JPEG file");
    uint16_t qt[4][64];
    bool qt_ok[4] = {false, false, false, false};
    Huff dc[4], ac[4];
    std::vector<Component> comps;
    int hmax = 1, vmax = 1, mcux = 0, mcuy = 0, restart = 0;
    bool frame = false, scanned = false;
    size_t pos = 2;
    auto u16 = [&](size_t p) { return (int)b[p] << 8 | b[p + 1]; };
    while (pos + 4 <= b.size()) {
        if (b[pos] != 0xFF) return bad("marker expected");
        const int m = b[pos + 1];
        if (m == 0xFF) {  // fill byte
            ++pos;
            continue;
        }
        if (m == 0xD9) break;  // EOI
        if (m == 0xD8 || (m >= 0xD0 && m <= 0xD7)) {
            pos += 2;
            continue;
        }
        const int len = u16(pos + 2);
        if (len < 2 || pos + 2 + (size_t)len > b.size()) return bad("truncated segment");
        const size_t s0 = pos + 4, s1 = pos + 2 + (size_t)len;
        if (m == 0xDB) {  // DQT
            size_t p = s0;
            while (p < s1) {
                const int pq = b[p] >> 4, tq = b[p] & 15;
                if (tq > 3 || pq > 1) return bad("bad quantisation table");
                ++p;
                if (p + (pq ? 128 : 64) > s1) return bad("truncated quantisation table");
                for (int k = 0; k < 64; ++k) qt[tq][k] = pq ? (uint16_t)u16(p + 2 * k) : b[p + k];
                p += pq ? 128 : 64;
                qt_ok[tq] = true;
            }
        } else if (m == 0xC4) {  // DHT
            size_t p = s0;
            while (p < s1) {
                if (p + 17 > s1) return bad("truncated Huffman table");
                const int tc = b[p] >> 4, th = b[p] & 15;
                if (tc > 1 || th > 3) return bad("bad Huffman table");
                int nv = 0;
                for (int l = 0; l < 16; ++l) nv += b[p + 1 + l];
                if (p + 17 + (size_t)nv > s1) return bad("truncated Huffman table");
                if (!(tc ? ac[th] : dc[th]).build(&b[p + 1], &b[p + 17], nv)) return bad("bad Huffman table");
                p += 17 + (size_t)nv;
            }
        } else if (m == 0xDD) {  // DRI
            restart = u16(s0);
        } else if (m == 0xC0 || m == 0xC1) {  // SOF0 / SOF1: sequential, Huffman
            if (b[s0] != 8) return unsupported("only 8-bit JPEG samples are read");
            h = u16(s0 + 1);
            w = u16(s0 + 3);
            const int nc = b[s0 + 5];
            if (w <= 0 || h <= 0) return bad("bad size");
            if (nc != 1 && nc != 3) return unsupported("JPEG with " + std::to_string(nc) + " components (grey and YCbCr are read)");
            for (int i = 0; i < nc; ++i) {
                Component c;
                c.id = b[s0 + 6 + 3 * i];
                c.h = b[s0 + 7 + 3 * i] >> 4;
                c.v = b[s0 + 7 + 3 * i] & 15;
                c.tq = b[s0 + 8 + 3 * i];
                if (c.h < 1 || c.h > 4 || c.v < 1 || c.v > 4 || c.tq > 3) return bad("bad component");
                comps.push_back(c);
                hmax = std::max(hmax, c.h);
                vmax = std::max(vmax, c.v);
            }
            mcux = (w + 8 * hmax - 1) / (8 * hmax);
            mcuy = (h + 8 * vmax - 1) / (8 * vmax);
            for (Component& c : comps) {
                c.bw = mcux * c.h;
                c.bh = mcuy * c.v;
                c.plane.assign((size_t)c.bw * 8 * c.bh * 8, 0);
            }
            frame = true;
        } else if (m >= 0xC2 && m <= 0xCF && m != 0xC4 && m != 0xC8 && m != 0xCC) {
            return unsupported("progressive, lossless or arithmetic-coded JPEG (baseline is read)");
        } else if (m == 0xDA) {  // SOS
            if (!frame) return bad("scan before frame");
            const int ns = b[s0];
            std::vector<int> sc;
            for (int i = 0; i < ns; ++i) {
                const int cid = b[s0 + 1 + 2 * i];
                int k = -1;
                for (size_t j = 0; j < comps.size(); ++j)
                    if (comps[j].id == cid) k = (int)j;
                if (k < 0) return bad("scan of an unknown component");
                comps[k].td = b[s0 + 2 + 2 * i] >> 4;
                comps[k].ta = b[s0 + 2 + 2 * i] & 15;
                if (comps[k].td > 3 || comps[k].ta > 3 || !dc[comps[k].td].present || !ac[comps[k].ta].present ||
                    !qt_ok[comps[k].tq])
                    return bad("scan references a missing table");
                sc.push_back(k);
            }
            BitIn in{b, s1};
            for (Component& c : comps) c.pred = 0;
            int coef[64];
            auto block = [&](Component& c, int bx, int by) -> bool {
                std::fill(coef, coef + 64, 0);
                const int t = huff_decode(in, dc[c.td]);
                if (t < 0 || t > 11) return false;
                c.pred += extend(in.getbits(t), t);
                coef[0] = c.pred * qt[c.tq][0];
                for (int k = 1; k < 64;) {
                    const int rs = huff_decode(in, ac[c.ta]);
                    if (rs < 0) return false;
                    const int r = rs >> 4, s = rs & 15;
                    if (s == 0) {
                        if (r != 15) break;  // end of block
                        k += 16;
                        continue;
                    }
                    k += r;
                    if (k > 63) return false;
                    coef[kZigzag[k]] = extend(in.getbits(s), s) * qt[c.tq][k];
                    ++k;
                }
                idct_block(coef, &c.plane[(size_t)by * 8 * c.bw * 8 + (size_t)bx * 8], c.bw * 8);
                return true;
            };
            if (sc.size() == 1) {
                // non-interleaved: the component's own blocks in raster order
                Component& c = comps[sc[0]];
                const int cw = (w * c.h + hmax - 1) / hmax, ch = (h * c.v + vmax - 1) / vmax;
                const int nbx = (cw + 7) / 8, nby = (ch + 7) / 8;
                int count = 0;
                for (int by = 0; by < nby; ++by)
                    for (int bx = 0; bx < nbx; ++bx) {
                        if (restart && count > 0 && count % restart == 0) {
                            in.reset();
                            c.pred = 0;
                        }
                        if (!block(c, bx, by)) return bad("corrupt entropy-coded data");
                        ++count;
                    }
            } else {
                int count = 0;
                for (int my = 0; my < mcuy; ++my)
                    for (int mx = 0; mx < mcux; ++mx) {
                        if (restart && count > 0 && count % restart == 0) {
                            in.reset();
                            for (Component& c : comps) c.pred = 0;
                        }
                        for (int k : sc) {
                            Component& c = comps[k];
                            for (int v = 0; v < c.v; ++v)
                                for (int u = 0; u < c.h; ++u)
                                    if (!block(c, mx * c.h + u, my * c.v + v)) return bad("corrupt entropy-coded data");
                        }
                        ++count;
                    }
            }
            // continue after the entropy-coded segment: the next marker that is not RSTn
            size_t p = in.pos;
            while (p + 1 < b.size() && !(b[p] == 0xFF && b[p + 1] != 0x00 && !(b[p + 1] >= 0xD0 && b[p + 1] <= 0xD7)))
                ++p;
            pos = p;
            scanned = true;
            continue;
        }
        pos = s1;
    }
    if (!frame || !scanned) return bad("no image data");
    // upsampling to full resolution: the triangle filter in each direction
    // (sample centres of a subsampled plane sit between full-resolution ones)
    std::vector<std::vector<float>> full(comps.size());
    for (size_t ci = 0; ci < comps.size(); ++ci) {
        const Component& c = comps[ci];
        const int sx = hmax / c.h, sy = vmax / c.v;
        const int pw = c.bw * 8, ph = c.bh * 8;
        std::vector<float>& f = full[ci];
        f.resize((size_t)w * h);
        for (int y = 0; y < h; ++y)
            for (int x = 0; x < w; ++x) {
                // position of this pixel's centre in the plane's sample grid
                const float fx = (x + 0.5f) / sx - 0.5f, fy = (y + 0.5f) / sy - 0.5f;
                int x0 = (int)std::floor(fx), y0 = (int)std::floor(fy);
                const float ax = sx == 1 ? 0.0f : fx - x0, ay = sy == 1 ? 0.0f : fy - y0;
                if (sx == 1) x0 = x;
                if (sy == 1) y0 = y;
                auto at = [&](int xx, int yy) {
                    xx = std::min(std::max(xx, 0), pw - 1);
                    yy = std::min(std::max(yy, 0), ph - 1);
                    return (float)c.plane[(size_t)yy * pw + xx];
                };
                f[(size_t)y * w + x] = (1 - ax) * (1 - ay) * at(x0, y0) + ax * (1 - ay) * at(x0 + 1, y0) +
                                       (1 - ax) * ay * at(x0, y0 + 1) + ax * ay * at(x0 + 1, y0 + 1);
            }
    }
    rgba.assign((size_t)w * h * 4, 255);
    for (size_t i = 0; i < (size_t)w * h; ++i) {
        uint8_t* o = &rgba[4 * i];
        if (comps.size() == 1) {
            o[0] = o[1] = o[2] = clamp8(full[0][i]);
        } else {
            const double Y = full[0][i], cb = full[1][i] - 128.0, cr = full[2][i] - 128.0;
            o[0] = clamp8(Y + 1.402 * cr);
            o[1] = clamp8(Y - 0.344136 * cb - 0.714136 * cr);
            o[2] = clamp8(Y + 1.772 * cb);
        }
    }
    return SRT_OK;
}

// ---- encoding --------------------------------------------------------------------------

namespace {

// ITU-T T.81 Annex K: quantisation tables (natural order) and Huffman tables
const uint8_t kStdLum[64] = {16, 11, 10, 16, 24,  40,  51,  61,  12, 12, 14, 19, 26,  58,  60,  55,
                             14, 13, 16, 24, 40,  57,  69,  56,  14, 17, 22, 29, 51,  87,  80,  62,
                             18, 22, 37, 56, 68,  109, 103, 77,  24, 35, 55, 64, 81,  104, 113, 92,
                             49, 64, 78, 87, 103, 121, 120, 101, 72, 92, 95, 98, 112, 100, 103, 99};
const uint8_t kStdChr[64] = {17, 18, 24, 47, 99, 99, 99, 99, 18, 21, 26, 66, 99, 99, 99, 99, 24, 26, 56, 99, 99, 99,
                             99, 99, 47, 66, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99,
                             99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99};
const uint8_t kDcLumBits[16] = {0, 1, 5, 1, 1, 1, 1, 1, 1, 0, 0, 0, 0, 0, 0, 0};
const uint8_t kDcChrBits[16] = {0, 3, 1, 1, 1, 1, 1, 1, 1, 1, 1, 0, 0, 0, 0, 0};
const uint8_t kDcVals[12] = {0, 1, 2, 3, 4, 5, 6, 7, 8, 9, 10, 11};
const uint8_t kAcLumBits[16] = {0, 2, 1, 3, 3, 2, 4, 3, 5, 5, 4, 4, 0, 0, 1, 0x7d};
const uint8_t kAcLumVals[162] = {
    0x01, 0x02, 0x03, 0x00, 0x04, 0x11, 0x05, 0x12, 0x21, 0x31, 0x41, 0x06, 0x13, 0x51, 0x61, 0x07, 0x22, 0x71, 0x14,
    0x32, 0x81, 0x91, 0xa1, 0x08, 0x23, 0x42, 0xb1, 0xc1, 0x15, 0x52, 0xd1, 0xf0, 0x24, 0x33, 0x62, 0x72, 0x82, 0x09,
    0x0a, 0x16, 0x17, 0x18, 0x19, 0x1a, 0x25, 0x26, 0x27, 0x28, 0x29, 0x2a, 0x34, 0x35, 0x36, 0x37, 0x38, 0x39, 0x3a,
    0x43, 0x44, 0x45, 0x46, 0x47, 0x48, 0x49, 0x4a, 0x53, 0x54, 0x55, 0x56, 0x57, 0x58, 0x59, 0x5a, 0x63, 0x64, 0x65,
    0x66, 0x67, 0x68, 0x69, 0x6a, 0x73, 0x74, 0x75, 0x76, 0x77, 0x78, 0x79, 0x7a, 0x83, 0x84, 0x85, 0x86, 0x87, 0x88,
    0x89, 0x8a, 0x92, 0x93, 0x94, 0x95, 0x96, 0x97, 0x98, 0x99, 0x9a, 0xa2, 0xa3, 0xa4, 0xa5, 0xa6, 0xa7, 0xa8, 0xa9,
    0xaa, 0xb2, 0xb3, 0xb4, 0xb5, 0xb6, 0xb7, 0xb8, 0xb9, 0xba, 0xc2, 0xc3, 0xc4, 0xc5, 0xc6, 0xc7, 0xc8, 0xc9, 0xca,
    0xd2, 0xd3, 0xd4, 0xd5, 0xd6, 0xd7, 0xd8, 0xd9, 0xda, 0xe1, 0xe2, 0xe3, 0xe4, 0xe5, 0xe6, 0xe7, 0xe8, 0xe9, 0xea,
    0xf1, 0xf2, 0xf3, 0xf4, 0xf5, 0xf6, 0xf7, 0xf8, 0xf9, 0xfa};
const uint8_t kAcChrBits[16] = {0, 2, 1, 2, 4, 4, 3, 4, 7, 5, 4, 4, 0, 1, 2, 0x77};
const uint8_t kAcChrVals[162] = {
    0x00, 0x01, 0x02, 0x03, 0x11, 0x04, 0x05, 0x21, 0x31, 0x06, 0x12, 0x41, 0x51, 0x07, 0x61, 0x71, 0x13, 0x22, 0x32,
    0x81, 0x08, 0x14, 0x42, 0x91, 0xa1, 0xb1, 0xc1, 0x09, 0x23, 0x33, 0x52, 0xf0, 0x15, 0x62, 0x72, 0xd1, 0x0a, 0x16,
    0x24, 0x34, 0xe1, 0x25, 0xf1, 0x17, 0x18, 0x19, 0x1a, 0x26, 0x27, 0x28, 0x29, 0x2a, 0x35, 0x36, 0x37, 0x38, 0x39,
    0x3a, 0x43, 0x44, 0x45, 0x46, 0x47, 0x48, 0x49, 0x4a, 0x53, 0x54, 0x55, 0x56, 0x57, 0x58, 0x59, 0x5a, 0x63, 0x64,
    0x65, 0x66, 0x67, 0x68, 0x69, 0x6a, 0x73, 0x74, 0x75, 0x76, 0x77, 0x78, 0x79, 0x7a, 0x82, 0x83, 0x84, 0x85, 0x86,
    0x87, 0x88, 0x89, 0x8a, 0x92, 0x93, 0x94, 0x95, 0x96, 0x97, 0x98, 0x99, 0x9a, 0xa2, 0xa3, 0xa4, 0xa5, 0xa6, 0xa7,
    0xa8, 0xa9, 0xaa, 0xb2, 0xb3, 0xb4, 0xb5, 0xb6, 0xb7, 0xb8, 0xb9, 0xba, 0xc2, 0xc3, 0xc4, 0xc5, 0xc6, 0xc7, 0xc8,
    0xc9, 0xca, 0xd2, 0xd3, 0xd4, 0xd5, 0xd6, 0xd7, 0xd8, 0xd9, 0xda, 0xe2, 0xe3, 0xe4, 0xe5, 0xe6, 0xe7, 0xe8, 0xe9,
    0xea, 0xf2, 0xf3, 0xf4, 0xf5, 0xf6, 0xf7, 0xf8, 0xf9, 0xfa};

struct HuffEnc {
    uint16_t code[256];
    uint8_t size[256];
    HuffEnc(const uint8_t* bits, const uint8_t* vals)
    {
        std::memset(size, 0, sizeof(size));
        int c = 0, k = 0;
        for (int l = 1; l <= 16; ++l) {
            for (int i = 0; i < bits[l - 1]; ++i, ++k) {
                code[vals[k]] = (uint16_t)c++;
                size[vals[k]] = (uint8_t)l;
            }
            c <<= 1;
        }
    }
};

struct BitOut {
    std::vector<uint8_t>& out;
    uint32_t acc = 0;
    int n = 0;
    void put(uint32_t bits, int len)
    {
        for (int i = len - 1; i >= 0; --i) {
            acc = (acc << 1) | ((bits >> i) & 1u);
            if (++n == 8) {
                out.push_back((uint8_t)acc);
                if (acc == 0xFF) out.push_back(0x00);  // byte stuffing
                acc = 0;
                n = 0;
            }
        }
    }
    void flush()
    {
        while (n) put(1, 1);  // pad with ones
    }
};

int bit_size(int v)
{
    v = std::abs(v);
    int s = 0;
    while (v) {
        ++s;
        v >>= 1;
    }
    return s;
}

void encode_block(BitOut& bo, const float* samples, int stride, const uint8_t* q, int& pred, const HuffEnc& dc,
                  const HuffEnc& ac)
{
    const DctBasis& B = basis();
    double tmp[8][8], F[64];
    for (int y = 0; y < 8; ++y)
        for (int u = 0; u < 8; ++u) {
            double s = 0.0;
            for (int x = 0; x < 8; ++x) s += B.c[u][x] * (samples[y * stride + x] - 128.0);
            tmp[y][u] = s;
        }
    for (int u = 0; u < 8; ++u)
        for (int v = 0; v < 8; ++v) {
            double s = 0.0;
            for (int y = 0; y < 8; ++y) s += B.c[v][y] * tmp[y][u];
            F[v * 8 + u] = s;
        }
    int zz[64];
    for (int k = 0; k < 64; ++k) zz[k] = (int)std::lround(F[kZigzag[k]] / q[k]);
    const int diff = zz[0] - pred;
    pred = zz[0];
    const int s0 = bit_size(diff);
    bo.put(dc.code[s0], dc.size[s0]);
    if (s0) bo.put((uint32_t)(diff < 0 ? diff + (1 << s0) - 1 : diff), s0);
    int run = 0;
    for (int k = 1; k < 64; ++k) {
        if (zz[k] == 0) {
            ++run;
            continue;
        }
        while (run > 15) {
            bo.put(ac.code[0xF0], ac.size[0xF0]);  // sixteen zeros
            run -= 16;
        }
        const int s = bit_size(zz[k]);
        const int rs = (run << 4) | s;
        bo.put(ac.code[rs], ac.size[rs]);
        bo.put((uint32_t)(zz[k] < 0 ? zz[k] + (1 << s) - 1 : zz[k]), s);
        run = 0;
    }
    if (run) bo.put(ac.code[0x00], ac.size[0x00]);  // end of block
}

}  // namespace

std::vector<uint8_t> jpeg_encode(int w, int h, const uint8_t* rgba, int quality)
{
    quality = std::min(100, std::max(1, quality));
    const int scale = quality < 50 ? 5000 / quality : 200 - 2 * quality;
    uint8_t ql[64], qc[64];  // zigzag order, as stored
    for (int k = 0; k < 64; ++k) {
        ql[k] = (uint8_t)std::min(255, std::max(1, (kStdLum[kZigzag[k]] * scale + 50) / 100));
        qc[k] = (uint8_t)std::min(255, std::max(1, (kStdChr[kZigzag[k]] * scale + 50) / 100));
    }
    const bool sub = quality <= 90;  // 4:2:0
    const int mcu = sub ? 16 : 8;
    const int pw = (w + mcu - 1) / mcu * mcu, ph = (h + mcu - 1) / mcu * mcu;
    std::vector<float> Y((size_t)pw * ph), Cb((size_t)pw * ph), Cr((size_t)pw * ph);
    for (int y = 0; y < ph; ++y)
        for (int x = 0; x < pw; ++x) {
            const uint8_t* p = rgba + 4 * ((size_t)std::min(y, h - 1) * w + std::min(x, w - 1));  // edge replication
            const float r = p[0], g = p[1], b = p[2];
            const size_t i = (size_t)y * pw + x;
            Y[i] = 0.299f * r + 0.587f * g + 0.114f * b;
            Cb[i] = -0.168736f * r - 0.331264f * g + 0.5f * b + 128.0f;
            Cr[i] = 0.5f * r - 0.418688f * g - 0.081312f * b + 128.0f;
        }
    std::vector<uint8_t> out = {0xFF, 0xD8};
    auto seg = [&](uint8_t m, const std::vector<uint8_t>& body) {
        out.push_back(0xFF);
        out.push_back(m);
        out.push_back((uint8_t)((body.size() + 2) >> 8));
        out.push_back((uint8_t)(body.size() + 2));
        out.insert(out.end(), body.begin(), body.end());
    };
    seg(0xE0, {'J', 'F', 'I', 'F', 0, 1, 1, 0, 0, 1, 0, 1, 0, 0});
    std::vector<uint8_t> dqt = {0x00};
    dqt.insert(dqt.end(), ql, ql + 64);
    dqt.push_back(0x01);
    dqt.insert(dqt.end(), qc, qc + 64);
    seg(0xDB, dqt);
    const uint8_t ys = sub ? 0x22 : 0x11;
    seg(0xC0, {8, (uint8_t)(h >> 8), (uint8_t)h, (uint8_t)(w >> 8), (uint8_t)w, 3, 1, ys, 0, 2, 0x11, 1, 3, 0x11, 1});
    std::vector<uint8_t> dht;
    auto table = [&](uint8_t cls, const uint8_t* bits, const uint8_t* vals, int nv) {
        dht.push_back(cls);
        dht.insert(dht.end(), bits, bits + 16);
        dht.insert(dht.end(), vals, vals + nv);
    };
    table(0x00, kDcLumBits, kDcVals, 12);
    table(0x10, kAcLumBits, kAcLumVals, 162);
    table(0x01, kDcChrBits, kDcVals, 12);
    table(0x11, kAcChrBits, kAcChrVals, 162);
    seg(0xC4, dht);
    seg(0xDA, {3, 1, 0x00, 2, 0x11, 3, 0x11, 0, 63, 0});
    const HuffEnc dcl(kDcLumBits, kDcVals), acl(kAcLumBits, kAcLumVals);
    const HuffEnc dcc(kDcChrBits, kDcVals), acc(kAcChrBits, kAcChrVals);
    BitOut bo{out};
    int py = 0, pcb = 0, pcr = 0;
    float cb8[64], cr8[64];
    for (int my = 0; my < ph; my += mcu)
        for (int mx = 0; mx < pw; mx += mcu) {
            if (!sub) {
                encode_block(bo, &Y[(size_t)my * pw + mx], pw, ql, py, dcl, acl);
                encode_block(bo, &Cb[(size_t)my * pw + mx], pw, qc, pcb, dcc, acc);
                encode_block(bo, &Cr[(size_t)my * pw + mx], pw, qc, pcr, dcc, acc);
                continue;
            }
            for (int by = 0; by < 2; ++by)
                for (int bx = 0; bx < 2; ++bx)
                    encode_block(bo, &Y[(size_t)(my + 8 * by) * pw + mx + 8 * bx], pw, ql, py, dcl, acl);
            for (int y = 0; y < 8; ++y)  // chroma: mean of each 2x2
                for (int x = 0; x < 8; ++x) {
                    const size_t i = (size_t)(my + 2 * y) * pw + mx + 2 * x;
                    cb8[y * 8 + x] = 0.25f * (Cb[i] + Cb[i + 1] + Cb[i + pw] + Cb[i + pw + 1]);
                    cr8[y * 8 + x] = 0.25f * (Cr[i] + Cr[i + 1] + Cr[i + pw] + Cr[i + pw + 1]);
                }
            encode_block(bo, cb8, 8, qc, pcb, dcc, acc);
            encode_block(bo, cr8, 8, qc, pcr, dcc, acc);
        }
    bo.flush();
    out.push_back(0xFF);
    out.push_back(0xD9);
    return out;
}

}  // namespace srt
