// Drives the command-line driver's frame writer pool (cli/fluidsim.cpp) on
// the host: frames taken from the pool, filled with a pattern, submitted, and
// after finish() every file is read back and compared with the byte
// conversion of its frame. Needs no GPU.
//
//   png_writers_main <dir> <frames> <width> <height> <threads> <queue>
#define main fluidsim_cli_main
#include "../../probabilistic_fluid_simulation_gb300/cli/fluidsim.cpp"
#undef main

int main(int argc, char **argv)
{
    if (argc != 7) return 2;
    const std::string dir = argv[1];
    const int frames = std::atoi(argv[2]), w = std::atoi(argv[3]), h = std::atoi(argv[4]);
    const int threads = std::atoi(argv[5]), queue = std::atoi(argv[6]);
    const size_t n = (size_t)w * h * 4;
    auto value = [&](int f, size_t k) {
        // values in [-0.25, 1.25): both clamps of the byte conversion occur
        return (float)((double)((k * 2654435761u + (size_t)f * 40503u) % 1500u) / 1000.0 - 0.25);
    };
    {
        PngWriters writers(w, h, threads, (size_t)queue);
        for (int f = 0; f < frames; ++f) {
            std::vector<float> frame = writers.take_buffer(n);
            for (size_t k = 0; k < n; ++k) frame[k] = value(f, k);
            writers.submit(dir + "/" + std::to_string(f) + ".png", std::move(frame));
        }
        const std::string err = writers.finish();
        if (!err.empty()) {
            std::fprintf(stderr, "%s\n", err.c_str());
            return 1;
        }
    }
    for (int f = 0; f < frames; ++f) {
        pfs::png::Image img;
        std::string err;
        if (!pfs::png::read_file(dir + "/" + std::to_string(f) + ".png", img, err)) {
            std::fprintf(stderr, "frame %d: %s\n", f, err.c_str());
            return 1;
        }
        if (img.width != w || img.height != h || img.rgba.size() != n) return 1;
        for (size_t k = 0; k < n; ++k)
            if (img.rgba[k] != to_byte(value(f, k))) {
                std::fprintf(stderr, "frame %d byte %zu differs\n", f, k);
                return 1;
            }
    }
    std::printf("ok %d frames\n", frames);
    return 0;
}
