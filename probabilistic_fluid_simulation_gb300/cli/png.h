// PNG reading and writing for the command-line driver, self-contained (no
// libpng, no zlib): the reference reads its inputs and writes one PNG per step
// through libpng's simplified API (includes/utils.hpp:31-150), which is not on
// the machines this library targets.
//
// Reading yields 8-bit RGBA, as libpng's png_image_finish_read with
// PNG_FORMAT_RGBA does for 8-bit and lower bit depths: gray expanded to
// R = G = B (low bit depths scaled by 255 / (2^d - 1)), palettes looked up,
// tRNS turned into alpha, alpha 255 where the file has none. Both interlace
// methods are read. Not supported: 16-bit samples (libpng would convert them
// from linear light to sRGB), and gamma / colour-space chunks are ignored
// (libpng would convert files whose gAMA differs from sRGB).
//
// Writing produces 8-bit RGBA, non-interlaced, each row filtered with the
// filter of least absolute sum, deflated with LZ77 (32 KiB window, hash
// chains) and the fixed Huffman codes.
#pragma once

#include <cstddef>
#include <cstdint>
#include <string>
#include <vector>

namespace pfs {
namespace png {

struct Image {
    int width = 0, height = 0;
    std::vector<uint8_t> rgba;  // height * width * 4, row-major
};

bool decode(const uint8_t *data, size_t size, Image &out, std::string &err);
bool read_file(const std::string &path, Image &out, std::string &err);
std::vector<uint8_t> encode(const uint8_t *rgba, int width, int height);
bool write_file(const std::string &path, const uint8_t *rgba, int width, int height, std::string &err);

// zlib stream (RFC 1950 / 1951) decoder and encoder, exposed for tests.
bool inflate_zlib(const uint8_t *data, size_t size, std::vector<uint8_t> &out, std::string &err);
std::vector<uint8_t> deflate_zlib(const uint8_t *data, size_t size);

}  // namespace png
}  // namespace pfs
