// inflate.cpp — DEFLATE decoder written from RFC 1951 (block types 0, 1, 2;
// canonical Huffman codes decoded one bit at a time, which is plenty for
// image headers and scanline blocks) and the zlib wrapper of RFC 1950.
#include "inflate.h"

namespace srt {
namespace {

struct BitReader {
    const uint8_t* p;
    size_t n;
    size_t pos = 0;  // in bits
    bool bad = false;
    uint32_t bit()
    {
        if ((pos >> 3) >= n) {
            bad = true;
            return 0;
        }
        const uint32_t b = (p[pos >> 3] >> (pos & 7)) & 1u;
        ++pos;
        return b;
    }
    uint32_t bits(int k)  // k <= 16, least significant bit first
    {
        uint32_t v = 0;
        for (int i = 0; i < k; ++i) v |= bit() << i;
        return v;
    }
};

// Canonical Huffman code: number of codes of each length and the symbols
// ordered by (length, symbol), RFC 1951 3.2.2.
struct Huffman {
    uint16_t count[16] = {};
    std::vector<uint16_t> symbol;
    bool build(const uint8_t* lengths, int n)
    {
        for (int i = 0; i < 16; ++i) count[i] = 0;
        for (int s = 0; s < n; ++s) ++count[lengths[s]];
        count[0] = 0;
        int left = 1;  // over-subscribed sets are rejected; incomplete ones are allowed
        for (int len = 1; len < 16; ++len) {
            left = (left << 1) - count[len];
            if (left < 0) return false;
        }
        uint16_t offs[16] = {};
        for (int len = 1; len < 15; ++len) offs[len + 1] = offs[len] + count[len];
        symbol.assign(n, 0);
        for (int s = 0; s < n; ++s)
            if (lengths[s]) symbol[offs[lengths[s]]++] = (uint16_t)s;
        return true;
    }
    int decode(BitReader& br) const
    {
        int code = 0, first = 0, index = 0;
        for (int len = 1; len < 16; ++len) {
            code |= (int)br.bit();
            const int c = count[len];
            if (code - first < c) return symbol[index + code - first];
            index += c;
            first = (first + c) << 1;
            code <<= 1;
            if (br.bad) return -1;
        }
        return -1;
    }
};

// length codes 257..285 and distance codes 0..29 (RFC 1951 3.2.5)
const uint16_t kLenBase[29] = {3, 4, 5, 6, 7, 8, 9, 10, 11, 13, 15, 17, 19, 23, 27, 31,
                               35, 43, 51, 59, 67, 83, 99, 115, 131, 163, 195, 227, 258};
const uint8_t kLenExtra[29] = {0, 0, 0, 0, 0, 0, 0, 0, 1, 1, 1, 1, 2, 2, 2, 2, 3, 3, 3, 3, 4, 4, 4, 4, 5, 5, 5, 5, 0};
const uint16_t kDistBase[30] = {1, 2, 3, 4, 5, 7, 9, 13, 17, 25, 33, 49, 65, 97, 129,
                                193, 257, 385, 513, 769, 1025, 1537, 2049, 3073, 4097, 6145, 8193, 12289, 16385, 24577};
const uint8_t kDistExtra[30] = {0, 0, 0, 0, 1, 1, 2, 2, 3, 3, 4, 4, 5, 5, 6, 6, 7, 7, 8, 8, 9, 9, 10, 10, 11, 11, 12, 12, 13, 13};
// order of the code-length code lengths in a dynamic block header
const uint8_t kClOrder[19] = {16, 17, 18, 0, 8, 7, 9, 6, 10, 5, 11, 4, 12, 3, 13, 2, 14, 1, 15};

bool inflate_codes(BitReader& br, const Huffman& lit, const Huffman& dist, std::vector<uint8_t>& out, size_t limit)
{
    for (;;) {
        const int sym = lit.decode(br);
        if (sym < 0 || br.bad) return false;
        if (sym < 256) {
            if (out.size() >= limit) return false;
            out.push_back((uint8_t)sym);
        } else if (sym == 256) {
            return true;
        } else {
            const int li = sym - 257;
            if (li >= 29) return false;
            const size_t len = kLenBase[li] + br.bits(kLenExtra[li]);
            const int ds = dist.decode(br);
            if (ds < 0 || ds >= 30) return false;
            const size_t d = kDistBase[ds] + br.bits(kDistExtra[ds]);
            if (br.bad || d > out.size() || out.size() + len > limit) return false;
            const size_t from = out.size() - d;
            for (size_t k = 0; k < len; ++k) out.push_back(out[from + k]);  // copies may overlap
        }
    }
}

}  // namespace

bool inflate_raw(const uint8_t* in, size_t n, std::vector<uint8_t>& out, size_t limit)
{
    BitReader br{in, n};
    for (;;) {
        const uint32_t last = br.bit();
        const uint32_t type = br.bits(2);
        if (br.bad) return false;
        if (type == 0) {
            br.pos = (br.pos + 7) & ~(size_t)7;  // stored: byte aligned LEN, NLEN, data
            const size_t at = br.pos >> 3;
            if (at + 4 > n) return false;
            const uint32_t len = in[at] | (uint32_t)in[at + 1] << 8;
            const uint32_t nlen = in[at + 2] | (uint32_t)in[at + 3] << 8;
            if ((len ^ 0xffffu) != nlen || at + 4 + len > n || out.size() + len > limit) return false;
            out.insert(out.end(), in + at + 4, in + at + 4 + len);
            br.pos = (at + 4 + len) << 3;
        } else if (type == 1) {
            uint8_t l[288 + 30];
            for (int s = 0; s < 288; ++s) l[s] = s < 144 ? 8 : s < 256 ? 9 : s < 280 ? 7 : 8;
            for (int s = 0; s < 30; ++s) l[288 + s] = 5;
            Huffman lit, dist;
            lit.build(l, 288);
            dist.build(l + 288, 30);
            if (!inflate_codes(br, lit, dist, out, limit)) return false;
        } else if (type == 2) {
            const int hlit = (int)br.bits(5) + 257, hdist = (int)br.bits(5) + 1, hclen = (int)br.bits(4) + 4;
            if (hlit > 286 || hdist > 30) return false;
            uint8_t cl[19] = {};
            for (int i = 0; i < hclen; ++i) cl[kClOrder[i]] = (uint8_t)br.bits(3);
            Huffman clh;
            if (!clh.build(cl, 19)) return false;
            uint8_t l[286 + 30] = {};
            int i = 0;
            while (i < hlit + hdist) {
                const int sym = clh.decode(br);
                if (sym < 0 || br.bad) return false;
                if (sym < 16) {
                    l[i++] = (uint8_t)sym;
                    continue;
                }
                int rep = 0;
                uint8_t val = 0;
                if (sym == 16) {
                    if (i == 0) return false;
                    val = l[i - 1];
                    rep = 3 + (int)br.bits(2);
                } else if (sym == 17) {
                    rep = 3 + (int)br.bits(3);
                } else {
                    rep = 11 + (int)br.bits(7);
                }
                if (i + rep > hlit + hdist) return false;
                while (rep--) l[i++] = val;
            }
            if (l[256] == 0) return false;  // a block needs its end code
            Huffman lit, dist;
            if (!lit.build(l, hlit) || !dist.build(l + hlit, hdist)) return false;
            if (!inflate_codes(br, lit, dist, out, limit)) return false;
        } else {
            return false;
        }
        if (last) return !br.bad;
    }
}

bool inflate_zlib(const uint8_t* in, size_t n, std::vector<uint8_t>& out, size_t limit)
{
    if (n < 6) return false;
    const uint32_t cmf = in[0], flg = in[1];
    if ((cmf & 0x0f) != 8 || ((cmf << 8) | flg) % 31 != 0 || (flg & 0x20)) return false;  // deflate, no dictionary
    const size_t start = out.size();
    if (!inflate_raw(in + 2, n - 6, out, limit)) return false;
    uint32_t a = 1, b = 0;
    for (size_t i = start; i < out.size(); ++i) {
        a = (a + out[i]) % 65521u;
        b = (b + a) % 65521u;
    }
    const uint32_t want = (uint32_t)in[n - 4] << 24 | (uint32_t)in[n - 3] << 16 | (uint32_t)in[n - 2] << 8 | in[n - 1];
    return ((b << 16) | a) == want;
}

}  // namespace srt
