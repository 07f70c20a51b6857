// jpeg.h — baseline JPEG (ITU-T T.81) decoding and encoding for film and
// texture images.  Host code.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

#include "common.h"

namespace srt {

// Baseline / extended-sequential Huffman JPEG, 8-bit samples, one
// (grey) or three (YCbCr) components, any sampling factors up to 4,
// restart intervals, interleaved and single-component scans -> RGBA8
// (alpha 255).  Progressive, arithmetic-coded, 12-bit and CMYK files are
// SRT_ERR_UNSUPPORTED; malformed ones SRT_ERR_PARSE.
srt_status jpeg_decode(const std::vector<uint8_t>& b, const std::string& path, int& w, int& h,
                       std::vector<uint8_t>& rgba);

// Baseline JPEG of RGBA8 rows (alpha dropped): JFIF YCbCr, 4:4:4 above
// quality 90 and 4:2:0 at or below it, the Annex K tables scaled by
// `quality` (1..100) and the Annex K Huffman tables.
std::vector<uint8_t> jpeg_encode(int w, int h, const uint8_t* rgba, int quality);

}  // namespace srt
