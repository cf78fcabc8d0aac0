// Mutation fuzzing of the PNG decoder (cli/png.cpp), meant to be built with
// AddressSanitizer and UndefinedBehaviorSanitizer: every seed file is
// mutated many times (bytes flipped, set or inserted, runs duplicated,
// chunk lengths rewritten, the file truncated; half the mutants get their
// chunk CRCs rewritten, so the corrupted contents reach the inflater and the
// row filters) and decoded. A mutated file
// must give either an error message or an image of its stated size; any
// memory error or undefined behaviour aborts the program under the
// sanitizers.
//
//   png_fuzz_main <iterations per seed> <rng seed> <seed.png>...
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <iterator>
#include <string>
#include <vector>

#include "png.h"

namespace {

struct Rng {
    uint64_t s;
    uint64_t next()
    {
        s += 0x9E3779B97F4A7C15ull;
        uint64_t z = s;
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        return z ^ (z >> 31);
    }
    size_t below(size_t n) { return n ? (size_t)(next() % n) : 0; }
};

void mutate(std::vector<uint8_t> &d, Rng &r)
{
    const int edits = 1 + (int)r.below(6);
    for (int e = 0; e < edits && !d.empty(); ++e) {
        switch (r.below(6)) {
        case 0: d[r.below(d.size())] ^= (uint8_t)(1u << r.below(8)); break;
        case 1: d[r.below(d.size())] = (uint8_t)r.next(); break;
        case 2: d.insert(d.begin() + (long)r.below(d.size() + 1), (uint8_t)r.next()); break;
        case 3: {  // duplicate a run
            const size_t a = r.below(d.size()), n = 1 + r.below(64);
            std::vector<uint8_t> run(d.begin() + (long)a, d.begin() + (long)std::min(d.size(), a + n));
            d.insert(d.begin() + (long)r.below(d.size() + 1), run.begin(), run.end());
            break;
        }
        case 4: {  // a chunk length field (after the signature, 4 bytes big-endian)
            if (d.size() > 12) {
                const size_t at = 8 + r.below(d.size() - 12);
                const uint32_t v = (uint32_t)r.next() >> (r.below(32));
                for (int k = 0; k < 4; ++k) d[at + k] = (uint8_t)(v >> (24 - 8 * k));
            }
            break;
        }
        default: d.resize(r.below(d.size() + 1)); break;  // truncate
        }
    }
}

uint32_t crc32(const uint8_t *p, size_t n)
{
    static uint32_t t[256];
    static bool ready = false;
    if (!ready) {
        for (uint32_t k = 0; k < 256; ++k) {
            uint32_t c = k;
            for (int j = 0; j < 8; ++j) c = (c & 1u) ? 0xEDB88320u ^ (c >> 1) : c >> 1;
            t[k] = c;
        }
        ready = true;
    }
    uint32_t c = 0xFFFFFFFFu;
    for (size_t i = 0; i < n; ++i) c = t[(c ^ p[i]) & 0xFFu] ^ (c >> 8);
    return c ^ 0xFFFFFFFFu;
}

// Rewrites the CRC of every whole chunk, so mutated chunk contents (IHDR
// fields, compressed image data) get past the CRC check and reach the header
// checks, the inflater and the row filters.
void fix_crcs(std::vector<uint8_t> &d)
{
    size_t pos = 8;
    while (pos + 12 <= d.size()) {
        const uint32_t len = ((uint32_t)d[pos] << 24) | ((uint32_t)d[pos + 1] << 16) | ((uint32_t)d[pos + 2] << 8) | d[pos + 3];
        if ((size_t)len > d.size() - pos - 12) break;
        const uint32_t c = crc32(d.data() + pos + 4, 4 + (size_t)len);
        for (int k = 0; k < 4; ++k) d[pos + 8 + len + k] = (uint8_t)(c >> (24 - 8 * k));
        pos += 12 + (size_t)len;
    }
}

}  // namespace

int main(int argc, char **argv)
{
    if (argc < 4) return 2;
    const long iters = std::atol(argv[1]);
    Rng r{(uint64_t)std::strtoull(argv[2], nullptr, 10)};
    long ok = 0, rejected = 0;
    for (int f = 3; f < argc; ++f) {
        std::ifstream in(argv[f], std::ios::binary);
        const std::vector<uint8_t> seed((std::istreambuf_iterator<char>(in)), std::istreambuf_iterator<char>());
        if (seed.empty()) return 2;
        for (long i = 0; i < iters; ++i) {
            std::vector<uint8_t> d = seed;
            mutate(d, r);
            if (r.below(2)) fix_crcs(d);
            pfs::png::Image img;
            std::string err;
            if (pfs::png::decode(d.data(), d.size(), img, err)) {
                if (img.width <= 0 || img.height <= 0 || img.rgba.size() != (size_t)img.width * img.height * 4) {
                    std::fprintf(stderr, "decoded image with inconsistent size\n");
                    return 1;
                }
                ++ok;
            } else {
                if (err.empty()) {
                    std::fprintf(stderr, "rejected without a message\n");
                    return 1;
                }
                ++rejected;
            }
        }
    }
    std::printf("decoded %ld rejected %ld\n", ok, rejected);
    return 0;
}
