// Command-line driver with the reference's interface (src/main.cpp):
//
//   fluidsim_gb300 <n_timesteps> <delta_t> <viscosity> <input_image> <velocity_field> [output_dir]
//
// Same arguments, checks and messages (src/main.cpp:40-42,110-126); the same
// input conversion: PNG samples as RGBA / 255 (includes/utils.hpp:81-83), the
// velocity field rescaled to v * VP_RANGE - VP_RANGE / 2 with VP_RANGE = 2 on
// all four channels (src/main.cpp:171-179), the temporary velocity buffer
// filled with (-1, -1, -1, 1) (src/main.cpp:186-195); the same loop
// (simulate_fluid_step then advect_color_step, src/main.cpp:219-246) with the
// image written after every step as <output_dir>/<step>.png, each sample as
// (byte)(x * 255) (includes/utils.hpp:128-131); without output_dir the run is
// timed only. The steps run in a session that keeps the state on the GPU
// (include/pfs.h); NUM_JACOBI_ITERS (includes/fluid.hpp:11) is taken from the
// environment variable PFS_JACOBI_ITERS (default 30).
//
// Differences from the reference, on purpose: the elapsed time is taken after
// the device has finished and every frame is written (src/main.cpp:247-254
// reads the clock before its cudaDeviceSynchronize); frames are compressed
// and written by worker threads while the steps go on; a missing output
// directory is created; a failing read, write or CUDA call ends the run with
// a message and exit status 1. The library's kernels are loaded when the CUDA
// context is created (CUDA_MODULE_LOADING=EAGER unless the environment sets
// it), so the clock measures the steps, not the first-use loading of kernels
// that lazy loading would put inside the timed loop.
#include <sys/stat.h>

#include <algorithm>
#include <cerrno>
#include <chrono>
#include <condition_variable>
#include <cstdio>
#include <cstdlib>
#include <deque>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "pfs.h"
#include "png.h"

namespace {

constexpr double kVpRange = 2.0;

void usage(const char *prog)
{
    std::fprintf(stderr, "Usage: %s <n_timesteps> <delta_t> <viscosity> <input_image> <velocity_field> [output_dir]\n",
                 prog);
}

int fail_api(const char *what)
{
    std::fprintf(stderr, "%s failed: %s\n", what, pfs_last_error());
    return 1;
}

std::vector<float> to_float(const pfs::png::Image &img)
{
    std::vector<float> x(img.rgba.size());
    for (size_t i = 0; i < x.size(); ++i) x[i] = (float)((double)(float)img.rgba[i] / 255.0);
    return x;
}

uint8_t to_byte(float x)
{
    const double v = (double)x * 255.0;
    if (!(v > 0.0)) return 0;  // (-1, 0] truncates to 0; below that the reference's cast is undefined
    if (v >= 255.0) return 255;
    return (uint8_t)v;  // truncation, as the reference's cast
}

// Converts, encodes and writes the per-step PNGs on worker threads, so the
// steps go on while earlier frames are compressed (the frames are
// independent). The queue is bounded; the first failure is kept and reported
// by finish().
class PngWriters {
  public:
    PngWriters(int width, int height, int threads, size_t max_queued)
        : w_(width), h_(height), max_queued_(max_queued), max_buffers_(max_queued + 2)
    {
        for (int k = 0; k < threads; ++k) pool_.emplace_back([this] { run(); });
    }
    ~PngWriters() { finish(); }
    // A frame buffer of n floats: one the workers have finished with, or a new
    // one while fewer than max_queued + 2 exist (else wait for one: a worker
    // hands its frame back as soon as it has converted it to bytes).
    std::vector<float> take_buffer(size_t n)
    {
        std::unique_lock<std::mutex> lk(mu_);
        buf_.wait(lk, [this] { return !free_.empty() || allocated_ < max_buffers_; });
        if (!free_.empty()) {
            std::vector<float> b = std::move(free_.back());
            free_.pop_back();
            b.resize(n);
            return b;
        }
        ++allocated_;
        lk.unlock();
        return std::vector<float>(n);
    }
    // `image`: the step's image as floats, converted to bytes on the worker
    void submit(std::string path, std::vector<float> image)
    {
        std::unique_lock<std::mutex> lk(mu_);
        room_.wait(lk, [this] { return jobs_.size() < max_queued_; });
        jobs_.push_back({std::move(path), std::move(image)});
        work_.notify_one();
    }
    // Waits for every frame; returns the first error message ("" if none).
    std::string finish()
    {
        {
            std::lock_guard<std::mutex> lk(mu_);
            closing_ = true;
        }
        work_.notify_all();
        for (auto &t : pool_)
            if (t.joinable()) t.join();
        pool_.clear();
        return error_;
    }

  private:
    struct Job {
        std::string path;
        std::vector<float> image;
    };
    void run()
    {
        for (;;) {
            Job j;
            {
                std::unique_lock<std::mutex> lk(mu_);
                work_.wait(lk, [this] { return closing_ || !jobs_.empty(); });
                if (jobs_.empty()) return;
                j = std::move(jobs_.front());
                jobs_.pop_front();
                room_.notify_one();
            }
            std::vector<uint8_t> rgba(j.image.size());
            for (size_t k = 0; k < rgba.size(); ++k) rgba[k] = to_byte(j.image[k]);
            {
                std::lock_guard<std::mutex> lk(mu_);
                free_.push_back(std::move(j.image));  // for the next step's frame
            }
            buf_.notify_one();
            std::string err;
            if (!pfs::png::write_file(j.path, rgba.data(), w_, h_, err)) {
                std::lock_guard<std::mutex> lk(mu_);
                if (error_.empty()) error_ = err;
            }
        }
    }
    int w_, h_;
    size_t max_queued_, max_buffers_, allocated_ = 0;
    std::vector<std::thread> pool_;
    std::deque<Job> jobs_;
    std::vector<std::vector<float>> free_;
    std::mutex mu_;
    std::condition_variable work_, room_, buf_;
    bool closing_ = false;
    std::string error_;
};

bool make_dir(const std::string &dir)
{
    struct stat st;
    if (stat(dir.c_str(), &st) == 0) return S_ISDIR(st.st_mode);
    return mkdir(dir.c_str(), 0755) == 0 || errno == EEXIST;
}

}  // namespace

int main(int argc, char *argv[])
{
    setenv("CUDA_MODULE_LOADING", "EAGER", 0);  // before the first CUDA call; a user's setting wins
    if (argc != 6 && argc != 7) {
        usage(argv[0]);
        return 1;
    }
    const bool write = argc == 7;
    const int n_timesteps = std::atoi(argv[1]);
    const float delta_t = (float)std::atof(argv[2]);
    const float viscosity = (float)std::atof(argv[3]);
    if (n_timesteps <= 0) {
        std::fprintf(stderr, "Timesteps must be greater than 0.\n");
        return 1;
    }
    if (delta_t <= 0) {
        std::fprintf(stderr, "Delta T must be greater than 0.\n");
        return 1;
    }
    int iters = 30;
    if (const char *e = std::getenv("PFS_JACOBI_ITERS")) iters = std::atoi(e);
    if (iters < 1) {
        std::fprintf(stderr, "PFS_JACOBI_ITERS must be at least 1.\n");
        return 1;
    }

    pfs::png::Image input, velocity;
    std::string err;
    if (!pfs::png::read_file(argv[4], input, err)) {
        std::fprintf(stderr, "Something went wrong reading the input image... (%s)\n", err.c_str());
        return 1;
    }
    if (!pfs::png::read_file(argv[5], velocity, err)) {
        std::fprintf(stderr, "Something went wrong reading the initial velocity field... (%s)\n", err.c_str());
        return 1;
    }
    if (write && !make_dir(argv[6])) {
        std::fprintf(stderr, "Cannot create the output directory %s\n", argv[6]);
        return 1;
    }

    std::vector<float> image = to_float(input), vp = to_float(velocity);
    for (float &v : vp) v = (float)((double)v * kVpRange - kVpRange / 2.0);
    std::vector<float> vtmp(vp.size());
    for (size_t i = 0; i < vtmp.size(); ++i) vtmp[i] = (i % 4) == 3 ? 1.0f : -1.0f;

    pfs_params p;
    pfs_params_default(&p);
    p.dt = delta_t;
    p.viscosity = viscosity;
    p.diffuse_iters = iters;
    p.max_iters = iters;
    p.tol = 0.0;
    pfs_session *s = nullptr;
    if (pfs_session_create(&s, velocity.width, velocity.height, input.width, input.height, 4, &p, nullptr) != PFS_OK)
        return fail_api("pfs_session_create");
    if (pfs_session_upload(s, vp.data(), vtmp.data(), image.data(), PFS_HOST) != PFS_OK)
        return fail_api("pfs_session_upload");

    std::printf("Simulating [%d x %d] domain for %d timesteps at dt=%g...\n", velocity.height, velocity.width,
                n_timesteps, (double)delta_t);
    const int nthreads = (int)std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
    // frames waiting for a writer: up to two per thread, and about 512 MB of them at most
    const size_t frame_bytes = std::max<size_t>(1, image.size() * sizeof(float));
    const size_t queue = std::max<size_t>(1, std::min<size_t>(2 * (size_t)nthreads, (512u << 20) / frame_bytes));
    PngWriters writers(input.width, input.height, write ? nthreads : 0, queue);
    const auto t0 = std::chrono::high_resolution_clock::now();
    for (int i = 0; i < n_timesteps; ++i) {
        if (pfs_session_step(s, 1) != PFS_OK) return fail_api("pfs_session_step");
        if (write) {
            std::vector<float> frame = writers.take_buffer(image.size());
            if (pfs_session_download(s, nullptr, nullptr, frame.data(), PFS_HOST) != PFS_OK)
                return fail_api("pfs_session_download");
            std::string path = std::string(argv[6]) + "/" + std::to_string(i) + ".png";
            std::printf("[%d] Writing to : %s\n", i, path.c_str());
            writers.submit(std::move(path), std::move(frame));
        }
    }
    if (pfs_session_sync(s) != PFS_OK) return fail_api("pfs_session_sync");
    const std::string werr = writers.finish();  // every frame on disk before the clock stops
    if (!werr.empty()) {
        std::fprintf(stderr, "%s\n", werr.c_str());
        return 1;
    }
    const auto t1 = std::chrono::high_resolution_clock::now();
    std::printf("%d timesteps took %lld us.\n", n_timesteps,
                (long long)std::chrono::duration_cast<std::chrono::microseconds>(t1 - t0).count());
    pfs_session_destroy(s);
    return 0;
}
