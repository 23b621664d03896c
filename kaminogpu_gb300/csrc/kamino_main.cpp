// kamino_main.cpp — the `kamino` executable: `kamino configKamino.txt`.
//
// Drop-in for the reference's main (KaminoGPU/kernel/main.cu:4-59) and
// Kamino::run (KaminoCore.cu:860-912), written over the C ABI only: parse the
// positional config, build the solver with the reference's FBM velocity and
// particle placement, write frame 0, then for every frame take the
// reference's steps and write the grid and particle .bgeo files.  A frame's
// files are written while the GPU runs the next frame's steps.
//
// Image inputs: the reference reads the density and colour images with
// OpenCV (KaminoSolver.cu:243-277, KaminoParticles.cu:6-17); here binary PPM
// (P6, 8-bit) files are read and handed to the library's image entry points.
// Other formats are reported and ignored, which is what the reference does
// when it cannot read an image (KaminoSolver.cu:250-254, KaminoParticles.cu:
// 8-11).
#include <cctype>
#include <chrono>
#include <cstdint>
#include <cstdio>
#include <string>
#include <vector>

#include "../../include/kamino_gb300.h"

namespace {

int fail(const char* what)
{
    std::fprintf(stderr, "kamino: %s: %s\n", what, kamino_last_error());
    return 1;
}

// A binary PPM (P6, maxval 255) as B, G, R pixels (OpenCV's order).
bool read_ppm(const std::string& path, std::vector<uint8_t>& bgr, int& w, int& h)
{
    FILE* fp = std::fopen(path.c_str(), "rb");
    if (!fp) return false;
    auto next_int = [fp](long& v) {
        int c = std::fgetc(fp);
        while (c != EOF && (std::isspace(c) || c == '#')) {
            if (c == '#')
                while (c != EOF && c != '\n') c = std::fgetc(fp);
            c = std::fgetc(fp);
        }
        if (c == EOF || !std::isdigit(c)) return false;
        v = 0;
        while (c != EOF && std::isdigit(c) && v < (1L << 30)) {
            v = 10 * v + (c - '0');
            c = std::fgetc(fp);
        }
        return c != EOF && std::isspace(c);  // one whitespace byte ends the header
    };
    long W = 0, H = 0, maxval = 0;
    bool ok = std::fgetc(fp) == 'P' && std::fgetc(fp) == '6' && next_int(W) && next_int(H) && next_int(maxval) &&
              maxval == 255 && W > 0 && H > 0 && W * H <= (1L << 28);
    if (ok) {
        bgr.resize((size_t)W * H * 3);
        ok = std::fread(bgr.data(), 1, bgr.size(), fp) == bgr.size();
        for (size_t k = 0; ok && k < bgr.size(); k += 3) std::swap(bgr[k], bgr[k + 2]);  // RGB -> BGR
        w = (int)W;
        h = (int)H;
    }
    std::fclose(fp);
    return ok;
}

// Loads an image path of the config; false (with a message) when it is not a
// readable P6 PPM.
bool load_image(const char* path, const char* what, std::vector<uint8_t>& bgr, int& w, int& h)
{
    if (!path[0]) return false;
    if (read_ppm(path, bgr, w, h)) return true;
    std::fprintf(stderr, "kamino: %s image '%s' ignored (not a readable binary PPM)\n", what, path);
    return false;
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
    std::vector<uint8_t> dimg, cimg;
    int dw = 0, dh = 0, cw = 0, ch = 0;
    const bool have_density = load_image(cfg.density_image, "density", dimg, dw, dh);
    const bool have_color = load_image(cfg.color_image, "colour", cimg, cw, ch);
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
    } else if (have_density && kamino_init_density_image(h, dimg.data(), dw, dh, 3 * (size_t)dw)) {
        rc = fail("density image");
    } else if (kamino_init_particles(h, 1)) {
        rc = fail("particles");
    } else if (have_color && kamino_init_particle_colors_image(h, cimg.data(), cw, ch, 3 * (size_t)cw)) {
        rc = fail("colour image");
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
