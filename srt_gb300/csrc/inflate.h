// inflate.h — DEFLATE (RFC 1951) and zlib (RFC 1950) decoding for the image
// readers (ZIP-compressed EXR scanline blocks).  Host code.
#pragma once

#include <cstddef>
#include <cstdint>
#include <vector>

namespace srt {

// Raw DEFLATE stream -> bytes appended to `out`.  `limit` caps the output
// size (a corrupt or hostile stream cannot grow it past that).  Returns
// false on a malformed stream or when the cap is reached.
bool inflate_raw(const uint8_t* in, size_t n, std::vector<uint8_t>& out, size_t limit);

// zlib stream (2-byte header, DEFLATE data, Adler-32 of the output).
bool inflate_zlib(const uint8_t* in, size_t n, std::vector<uint8_t>& out, size_t limit);

}  // namespace srt
