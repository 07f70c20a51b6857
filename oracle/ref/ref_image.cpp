// Reference image I/O built for the host (test infrastructure only).
//
// Compiles the image libraries the reference vendors (extensions/tinyexr,
// extensions/stb_image) with the steps of the reference's Image class
// (src/scene/texture.cu: save_exr :69-130, save_hdr :132-143, save_ldr
// :145-168, load_from_file :170-217, flip :44-66) so the tests can check
// our writers and readers against what the reference itself writes and
// reads.  tinyexr is built over the system zlib (TINYEXR_USE_MINIZ 0): the
// reference tree does not vendor miniz.  The library lands in oracle/_ref/
// and is git-ignored.
#include <zlib.h>

#define TINYEXR_USE_MINIZ 0
#define TINYEXR_USE_THREAD 0
#define TINYEXR_USE_OPENMP 0
#define TINYEXR_IMPLEMENTATION
#include "tinyexr.h"

#define STB_IMAGE_IMPLEMENTATION
#include "stb_image.h"
#define STB_IMAGE_WRITE_IMPLEMENTATION
#include "stb_image_write.h"

#include <cstdlib>
#include <cstring>
#include <vector>

extern "C" {

// Image::save_exr: channels B, G, R, A given as FLOAT, stored as HALF;
// `compression` is a TINYEXR_COMPRESSIONTYPE_* (the reference leaves
// InitEXRHeader's 0 = none).
int ref_save_exr(const char* path, int w, int h, const float* rgba, int compression)
{
    EXRHeader header;
    InitEXRHeader(&header);
    EXRImage image;
    InitEXRImage(&image);
    std::vector<float> ch[4];
    for (int c = 0; c < 4; ++c) {
        ch[c].resize((size_t)w * h);
        for (size_t i = 0; i < (size_t)w * h; ++i) ch[c][i] = rgba[4 * i + c];
    }
    float* ptr[4] = {ch[2].data(), ch[1].data(), ch[0].data(), ch[3].data()};
    image.num_channels = 4;
    image.images = (unsigned char**)ptr;
    image.width = w;
    image.height = h;
    header.num_channels = 4;
    header.compression_type = compression;
    header.channels = (EXRChannelInfo*)malloc(sizeof(EXRChannelInfo) * 4);
    const char* names[4] = {"B", "G", "R", "A"};
    for (int c = 0; c < 4; ++c) {
        std::strncpy(header.channels[c].name, names[c], 255);
        header.channels[c].name[1] = '\0';
    }
    header.pixel_types = (int*)malloc(sizeof(int) * 4);
    header.requested_pixel_types = (int*)malloc(sizeof(int) * 4);
    for (int c = 0; c < 4; ++c) {
        header.pixel_types[c] = TINYEXR_PIXELTYPE_FLOAT;
        header.requested_pixel_types[c] = TINYEXR_PIXELTYPE_HALF;
    }
    const char* err = nullptr;
    int ret = SaveEXRImageToFile(&image, &header, path, &err);
    if (err) FreeEXRErrorMessage(err);
    free(header.channels);
    free(header.pixel_types);
    free(header.requested_pixel_types);
    return ret;
}

// Image::save_hdr / save_ldr (stb_image_write), 4 channels.
int ref_save_stb(const char* path, int kind, int w, int h, const float* rgba)
{
    if (kind == 0) return stbi_write_hdr(path, w, h, 4, rgba) ? 0 : -1;
    std::vector<unsigned char> u((size_t)w * h * 4);
    for (size_t i = 0; i < u.size(); ++i) {
        float v = rgba[i] < 0.0f ? 0.0f : (rgba[i] > 1.0f ? 1.0f : rgba[i]);  // Image::f_to_u
        u[i] = (unsigned char)(v * 255.0f);
    }
    if (kind == 1) return stbi_write_png(path, w, h, 4, u.data(), 0) ? 0 : -1;
    return stbi_write_bmp(path, w, h, 4, u.data()) ? 0 : -1;
}

// Image::load_from_file without the flip: EXR through LoadEXR, else
// stbi_loadf for Radiance HDR; RGBA float.  Call with out == nullptr for
// the size.  Returns 0 on success.
int ref_load_float_image(const char* path, int* w, int* h, float* out)
{
    float* data = nullptr;
    if (IsEXR(path) == TINYEXR_SUCCESS) {
        const char* err = nullptr;
        if (LoadEXR(&data, w, h, path, &err) != TINYEXR_SUCCESS) {
            if (err) FreeEXRErrorMessage(err);
            return -1;
        }
    } else if (stbi_is_hdr(path)) {
        data = stbi_loadf(path, w, h, nullptr, STBI_rgb_alpha);
        if (!data) return -2;
    } else {
        return -3;
    }
    if (out) std::memcpy(out, data, (size_t)(*w) * (*h) * 16);
    free(data);
    return 0;
}

// stbi_write_jpg of 8-bit pixels (the reference's save_ldr uses quality 100)
int ref_save_jpg(const char* path, int w, int h, int comp, const unsigned char* px, int quality)
{
    return stbi_write_jpg(path, w, h, comp, px, quality) ? 0 : -1;
}

// Image::load_from_file's 8-bit branch without the flip: stbi_load(.., 4).
int ref_load_u8_image(const char* path, int* w, int* h, unsigned char* out)
{
    unsigned char* data = stbi_load(path, w, h, nullptr, STBI_rgb_alpha);
    if (!data) return -1;
    if (out) std::memcpy(out, data, (size_t)(*w) * (*h) * 4);
    stbi_image_free(data);
    return 0;
}

}  // extern "C"
