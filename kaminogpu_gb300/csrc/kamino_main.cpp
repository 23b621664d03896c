// kamino_main.cpp — the `kamino` executable: `kamino configKamino.txt`.
//
// Drop-in for the reference's main (KaminoGPU/kernel/main.cu:4-59) and
// Kamino::run (KaminoCore.cu:860-912), written over the C ABI only: parse the
// positional config, build the solver with the reference's FBM velocity and
// particle placement, write frame 0, then for every frame take the
// reference's steps and write the grid and particle .bgeo files.  A frame's
// files are written while the GPU runs the next frame's steps.
//
// Image inputs (density and colour images, read with OpenCV by the
// reference) are not supported: a non-empty path is reported and ignored,
// which is what the reference does when the image cannot be read
// (KaminoSolver.cu:250-254, KaminoParticles.cu:8-11).
#include <chrono>
#include <cstdio>
#include <string>

#include "../../include/kamino_gb300.h"

namespace {

int fail(const char* what)
{
    std::fprintf(stderr, "kamino: %s: %s\n", what, kamino_last_error());
    return 1;
}

}  // namespace

int main(int argc, char** argv)
{
    if (argc != 2) {
        std::printf("Please provide the path to configKamino.txt as an argument.\n");
        std::printf("Usage example: ./kamino ./configKamino.txt\n");
        std::printf("Configuration file was missing, exiting.\n");
        return 255;
    }
    kamino_config cfg;
    if (kamino_parse_config(argv[1], &cfg)) return fail("config");
    if (cfg.density_image[0])
        std::fprintf(stderr, "kamino: density image '%s' ignored (image input is not supported)\n",
                     cfg.density_image);
    if (cfg.color_image[0])
        std::fprintf(stderr, "kamino: colour image '%s' ignored (image input is not supported)\n", cfg.color_image);
    kamino_handle h = nullptr;
    if (kamino_create(&cfg, &h)) return fail("create");
    int rc = 0;
    const std::string grid = cfg.grid_path, part = cfg.particle_path;
    const bool want[2] = {!grid.empty(), !part.empty() && kamino_particle_count(&cfg) > 0};
    const std::string* base[2] = {&grid, &part};
    const auto t0 = std::chrono::steady_clock::now();
    auto write = [&](int frame) {
        for (int k = 0; k < 2; k++) {
            if (!want[k]) continue;
            const std::string file = *base[k] + std::to_string(frame) + ".bgeo";
            std::printf("Writing to: %s\n", file.c_str());
            if (kamino_frame_write(h, k, file.c_str(), nullptr, 0)) return fail("write");
        }
        return 0;
    };
    auto capture = [&]() {
        for (int k = 0; k < 2; k++)
            if (want[k] && kamino_frame_capture(h, k)) return fail("capture");
        return 0;
    };
    if (kamino_init_fbm(h)) {
        rc = fail("velocity");
    } else if (kamino_init_particles(h, 1)) {
        rc = fail("particles");
    } else if (!(rc = capture())) {
        for (int i = 1; i <= cfg.frames && !rc; i++) {
            const int64_t n = kamino_frame_steps(cfg.dt, cfg.frame_dt, i) - kamino_frame_steps(cfg.dt, cfg.frame_dt, i - 1);
            if (n < 1 || n > 0x7fffffff || kamino_step_n(h, (int)n)) {
                rc = fail("step");
                break;
            }
            if ((rc = capture())) break;
            if ((rc = write(i - 1))) break;  // frame i-1's files while frame i runs
            std::printf("Frame %d is ready\n", i);
        }
        if (!rc) rc = write(cfg.frames);
    }
    if (!rc && kamino_synchronize(h)) rc = fail("synchronize");
    const double ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    kamino_destroy(h);
    if (rc) return rc;
    std::printf("Time spent: %gms\n", ms);
    std::printf("Performance: %g frames per second\n", 1000.0 * cfg.frames / ms);
    return 0;
}
