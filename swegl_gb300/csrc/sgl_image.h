// sgl_image.h — host image decoders for textures (swegl's image readers,
// src/misc/image.cpp:20-265), producing 0xAARRGGBB texels, row 0 first.
#pragma once

#include <cstddef>
#include <cstdint>
#include <string>
#include <vector>

namespace sgl {

struct Image {
    int width = 0, height = 0;
    std::vector<uint32_t> texels;
};

// read_bmp_file (image.cpp:29-83): a 54-byte header, then 24-bit BGR rows
// bottom-up with (width * 3) % 4 bytes skipped after each row.
bool decode_bmp(const uint8_t *data, size_t size, Image &out, std::string &err);
// read_png_file (image.cpp:92-172): every PNG colour type and bit depth
// expanded to 8-bit RGBA (16-bit samples keep their high byte, tRNS becomes
// alpha, grey is replicated), Adam7 interlacing included.
bool decode_png(const uint8_t *data, size_t size, Image &out, std::string &err);
// The zlib stream inflater the PNG decoder uses (RFC 1950/1951).
bool zlib_inflate(const uint8_t *data, size_t size, std::vector<uint8_t> &out, std::string &err);
// read_jpeg_file (image.cpp:183-255): baseline JPEG.
bool decode_jpeg(const uint8_t *data, size_t size, Image &out, std::string &err);
// read_image_file (image.cpp:20-27): the decoder chosen by the file name's
// extension (png, jpg, jpeg, bmp; case-insensitive).
bool decode_by_name(const std::string &name, const uint8_t *data, size_t size, Image &out, std::string &err);

} // namespace sgl
