// Round trips of the PNG encoder (cli/png.cpp) on images of many sizes and
// kinds of content (noise, long runs, gradients, zeros), meant to be built
// with AddressSanitizer and UndefinedBehaviorSanitizer: the encoder's
// word-wise match compares and table-driven bit output must stay inside their
// buffers, and every file must decode to the image encoded.
//
//   png_encode_asan_main <images> <rng seed>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

#include "png.h"

int main(int argc, char **argv)
{
    if (argc != 3) return 2;
    const int images = std::atoi(argv[1]);
    uint64_t s = std::strtoull(argv[2], nullptr, 10);
    auto next = [&]() {
        s += 0x9E3779B97F4A7C15ull;
        uint64_t z = s;
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        return z ^ (z >> 31);
    };
    for (int k = 0; k < images; ++k) {
        const int w = 1 + (int)(next() % 300), h = 1 + (int)(next() % 40), kind = (int)(next() % 4);
        std::vector<uint8_t> rgba((size_t)w * h * 4);
        for (size_t i = 0; i < rgba.size(); ++i) {
            switch (kind) {
            case 0: rgba[i] = (uint8_t)next(); break;                        // noise
            case 1: rgba[i] = (uint8_t)((i / (1 + next() % 3 + 300)) * 37); break;  // long runs
            case 2: rgba[i] = (uint8_t)(i % 4 == 3 ? 255 : (i / 4) % (size_t)w); break;  // gradient
            default: rgba[i] = 0; break;
            }
        }
        const std::vector<uint8_t> png = pfs::png::encode(rgba.data(), w, h);
        pfs::png::Image img;
        std::string err;
        if (!pfs::png::decode(png.data(), png.size(), img, err) || img.width != w || img.height != h ||
            img.rgba != rgba) {
            std::fprintf(stderr, "image %d (%dx%d kind %d): round trip failed %s\n", k, w, h, kind, err.c_str());
            return 1;
        }
    }
    std::printf("ok %d\n", images);
    return 0;
}
