// kamino_init.cpp — host side of the C ABI that needs no GPU: config
// defaults and parsing (KaminoGPU/kernel/main.cu:17-45), the particle count
// rule (KaminoParticles.cu:20-26) and the seeded synthetic initial states.
//
// The reference initialises velocity from FBM curl noise
// (KaminoInitializer.cu:3-134), thickness from an image and particles from a
// jittered grid with unseeded rand() (KaminoParticles.cu:33-62); the last is
// kamino_reference_particles below.  The benchmark workloads are seeded
// instead: a spherical-harmonic stream function
// (plus an optional Gaussian vortex), thickness 1 + a*U(-1,1), particles
// uniform on the sphere.  Every draw comes from a splitmix64-seeded
// xoshiro256** stream, so the same seed gives the same state on any host.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <string>
#include <vector>

#include "../../include/kamino_gb300.h"
#include "kamino_common.h"

namespace {

struct Rng {
    uint64_t s[4];
    static uint64_t splitmix(uint64_t& x)
    {
        uint64_t z = (x += 0x9E3779B97F4A7C15ull);
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        return z ^ (z >> 31);
    }
    explicit Rng(uint64_t seed)
    {
        uint64_t x = seed;
        for (auto& w : s) w = splitmix(x);
    }
    static uint64_t rotl(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }
    uint64_t next()
    {
        uint64_t r = rotl(s[1] * 5, 7) * 9, t = s[1] << 17;
        s[2] ^= s[0];
        s[3] ^= s[1];
        s[1] ^= s[2];
        s[0] ^= s[3];
        s[2] ^= t;
        s[3] = rotl(s[3], 45);
        return r;
    }
    double uniform() { return (double)(next() >> 11) * (1.0 / 9007199254740992.0); } // [0,1)
    double normal()
    {
        double u1 = uniform(), u2 = uniform();
        if (u1 < 1e-300) u1 = 1e-300;
        return std::sqrt(-2.0 * std::log(u1)) * std::cos(2.0 * M_PI * u2);
    }
};

// Independent streams per quantity so that, e.g., adding particles does not
// change the velocity drawn from the same seed.
enum { STREAM_SH = 1, STREAM_THICK = 2, STREAM_PART = 3, STREAM_VORTEX = 4 };
uint64_t stream_seed(uint64_t seed, int stream) { return seed * 0x2545F4914F6CDD1Dull + 0x9E37u * (uint64_t)stream; }

void set_str(char* dst, const std::string& s)
{
    std::snprintf(dst, 256, "%s", s.c_str());
}

// Orthonormal associated Legendre functions Pbar_l^m(cos theta), l <= L, and
// their theta-derivatives, by the standard three-term recurrences.
void legendre(int L, double theta, std::vector<double>& P, std::vector<double>& dP)
{
    const int W = L + 1;
    P.assign((size_t)W * W, 0.0);
    dP.assign((size_t)W * W, 0.0);
    double x = std::cos(theta), s = std::sin(theta);
    P[0] = std::sqrt(1.0 / (4.0 * M_PI));
    for (int m = 1; m <= L; m++)
        P[(size_t)m * W + m] = std::sqrt((2.0 * m + 1.0) / (2.0 * m)) * s * P[(size_t)(m - 1) * W + m - 1];
    for (int m = 0; m < L; m++)
        P[(size_t)(m + 1) * W + m] = std::sqrt(2.0 * m + 3.0) * x * P[(size_t)m * W + m];
    for (int m = 0; m <= L; m++) {
        for (int l = m + 2; l <= L; l++) {
            double a = std::sqrt((4.0 * l * l - 1.0) / ((double)l * l - (double)m * m));
            double b = std::sqrt(((l - 1.0) * (l - 1.0) - (double)m * m) / (4.0 * (l - 1.0) * (l - 1.0) - 1.0));
            P[(size_t)l * W + m] = a * (x * P[(size_t)(l - 1) * W + m] - b * P[(size_t)(l - 2) * W + m]);
        }
    }
    // sin(theta) dPbar_l^m/dtheta = l cos(theta) Pbar_l^m
    //                               - sqrt((l^2-m^2)(2l+1)/(2l-1)) Pbar_{l-1}^m
    for (int l = 0; l <= L; l++) {
        for (int m = 0; m <= l; m++) {
            double v = l * x * P[(size_t)l * W + m];
            if (l > m) v -= std::sqrt(((double)l * l - (double)m * m) * (2.0 * l + 1.0) / (2.0 * l - 1.0)) *
                            P[(size_t)(l - 1) * W + m];
            dP[(size_t)l * W + m] = v / s;
        }
    }
}

} // namespace

extern "C" int kamino_config_default(kamino_config* cfg)
{
    if (!cfg) return kamino_fail(KAMINO_ERR_INVALID, "kamino_config_default: null config");
    std::memset(cfg, 0, sizeof(*cfg));
    // Kamino(...) defaults, KaminoGPU/include/KaminoGPU.cuh:40-44
    cfg->radius = 5.0;
    cfg->n_theta = 128;
    cfg->particle_density = 200.0;
    cfg->dt = 0.005;
    cfg->frame_dt = 1.0 / 24.0;
    cfg->frames = 1000;
    cfg->A = 0.0;
    cfg->B = cfg->C = cfg->D = cfg->E = 1;
    set_str(cfg->grid_path, "output/frame");
    set_str(cfg->particle_path, "particles/frame");
    cfg->n_particles = 0;
    cfg->flags = 0;
    cfg->fp64_modes = 4;
    cfg->device = 0;
    return KAMINO_OK;
}

extern "C" int kamino_parse_config(const char* path, kamino_config* cfg)
{
    if (!path || !cfg) return kamino_fail(KAMINO_ERR_INVALID, "kamino_parse_config: null argument");
    std::ifstream fin(path);
    if (!fin) return kamino_fail(KAMINO_ERR_IO, "cannot open config file '%s'", path);
    kamino_config c;
    kamino_config_default(&c);
    // The 16 positional fields of main.cu:17-45, in order.
    double radius, pdens, A;
    long long ntheta;
    float dt, DT;
    int frames, B, C, D, E;
    std::string gridPath, particlePath, densityImage, solidImage, colorImage;
    if (!(fin >> radius >> ntheta >> pdens >> dt >> DT >> frames >> A >> B >> C >> D >> E >> gridPath >>
          particlePath >> densityImage >> solidImage >> colorImage))
        return kamino_fail(KAMINO_ERR_IO, "config '%s': expected 16 whitespace-separated fields", path);
    if (ntheta <= 0 || ntheta > (1 << 30))
        return kamino_fail(KAMINO_ERR_IO, "config '%s': nTheta=%lld out of range", path, ntheta);
    c.radius = radius;
    c.n_theta = (int32_t)ntheta;
    c.particle_density = pdens;
    c.dt = dt;
    c.frame_dt = DT;
    c.frames = frames;
    c.A = A;
    c.B = B;
    c.C = C;
    c.D = D;
    c.E = E;
    auto nul = [](const std::string& s) { return s == "null" ? std::string() : s; };
    set_str(c.grid_path, gridPath);
    set_str(c.particle_path, particlePath);
    set_str(c.density_image, nul(densityImage));
    set_str(c.solid_image, nul(solidImage));
    set_str(c.color_image, nul(colorImage));
    c.n_particles = -1; // count from particle_density, as the reference does
    *cfg = c;
    return KAMINO_OK;
}

// The particle density as KaminoParticles receives it: the config's fReal
// value truncated to size_t by initParticlesfromPic, then back to fReal.
static float reference_density(double d)
{
    const float f = (float)d;
    return f > 0.0f ? (float)(size_t)f : 0.0f;
}

extern "C" int64_t kamino_particle_count(const kamino_config* cfg)
{
    if (!cfg) return -1;
    if (cfg->n_particles >= 0) return cfg->n_particles;
    // KaminoParticles.cu:20-26: linearDensity = sqrt(particleDensity) in
    // fReal; numTheta = (unsigned)(linearDensity * nTheta); numPhi = 2*numTheta.
    // The density reaches it through initParticlesfromPic's size_t parameter
    // (KaminoSolver.cu:278, called with the fReal density at KaminoCore.cu:865),
    // so its fraction is dropped first.
    float linearDensity = std::sqrt(reference_density(cfg->particle_density));
    unsigned numThetaParticles = (unsigned)(linearDensity * (float)(size_t)cfg->n_theta);
    unsigned numPhiParticles = 2 * numThetaParticles;
    return (int64_t)numThetaParticles * (int64_t)numPhiParticles;
}

// KaminoParticles::KaminoParticles (KaminoParticles.cu:20-62): a jittered
// grid of numPhi x numTheta particles, four rand() draws per particle (two
// signs, two offsets of up to half a spacing), in the reference's float
// arithmetic, particle index i * numTheta + j.  The draws come from the C
// library's random() generator seeded like srand(seed) (the reference never
// seeds it: seed 1), through the reentrant random_r so the caller's own
// rand() sequence is left alone; with the GNU C library that is the sequence
// the reference's rand() gives.
extern "C" int kamino_reference_particles(const kamino_config* cfg, uint32_t seed, float* out, int64_t n)
{
    if (!cfg || !out) return kamino_fail(KAMINO_ERR_INVALID, "kamino_reference_particles: null argument");
    kamino_config c = *cfg;
    c.n_particles = -1;
    const int64_t want = kamino_particle_count(&c);
    if (n != want)
        return kamino_fail(KAMINO_ERR_INVALID, "particle_density %g at nTheta %d makes %lld particles, not %lld",
                           cfg->particle_density, cfg->n_theta, (long long)want, (long long)n);
    const float linearDensity = std::sqrt(reference_density(cfg->particle_density));
    const size_t nTheta = (size_t)cfg->n_theta;
    const float delta = (float)(KAMINO_PI_D / (double)nTheta / (double)linearDensity);
    const float halfDelta = (float)((double)delta / 2.0);
    const unsigned numThetaParticles = (unsigned)(linearDensity * (float)nTheta);
    const unsigned numPhiParticles = 2 * numThetaParticles;
    char state[128];
    struct random_data rd;
    std::memset(&rd, 0, sizeof(rd));
    std::memset(state, 0, sizeof(state));
    if (initstate_r(seed, state, sizeof(state), &rd) != 0)
        return kamino_fail(KAMINO_ERR_INVALID, "initstate_r failed");
    auto draw = [&rd]() {
        int32_t r = 0;
        random_r(&rd, &r);
        return (float)r / (float)RAND_MAX;
    };
    for (unsigned i = 0; i < numPhiParticles; ++i) {
        for (unsigned j = 0; j < numThetaParticles; ++j) {
            float signPhi = draw();
            signPhi = signPhi >= 0.5f ? 1.0f : -1.0f;
            float signTheta = draw();
            signTheta = signTheta >= 0.5f ? 1.0f : -1.0f;
            int32_t r = 0;
            random_r(&rd, &r);
            const float randPhi = signPhi * halfDelta * (float)r / (float)RAND_MAX;
            random_r(&rd, &r);
            const float randTheta = signTheta * halfDelta * (float)r / (float)RAND_MAX;
            float phi = (float)i * delta + randPhi;
            float theta = (float)j * delta + randTheta;
            if (phi < 0.0f) phi = 0.0f;
            if (theta < 0.0f) theta = 0.0f;
            const size_t index = (size_t)i * numThetaParticles + j;
            out[2 * index] = phi;
            out[2 * index + 1] = theta;
        }
    }
    return KAMINO_OK;
}

extern "C" int kamino_init_spec_default(kamino_init_spec* spec)
{
    if (!spec) return kamino_fail(KAMINO_ERR_INVALID, "kamino_init_spec_default: null spec");
    std::memset(spec, 0, sizeof(*spec));
    spec->n_theta = 128;
    spec->lmax = 8;
    spec->seed = 1;
    spec->radius = 1.0;
    spec->thickness_noise = 0.05;
    spec->vortex = 0;
    spec->vortex_sigma = 0.1;
    spec->vortex_amplitude = 0.0;
    spec->velocity_scale = 1.0;
    spec->n_particles = 0;
    return KAMINO_OK;
}

extern "C" int kamino_make_initial_state(kamino_init_spec* spec, float* u_phi, float* u_theta,
                                         float* thickness, float* particles)
{
    if (!spec) return kamino_fail(KAMINO_ERR_INVALID, "kamino_make_initial_state: null spec");
    const int nt = spec->n_theta;
    if (nt < 4 || (nt & (nt - 1)))
        return kamino_fail(KAMINO_ERR_INVALID, "n_theta=%d must be a power of two >= 4", nt);
    if (spec->lmax < 1 || spec->lmax > 256)
        return kamino_fail(KAMINO_ERR_INVALID, "lmax=%d out of range [1, 256]", spec->lmax);
    if (!(spec->radius > 0)) return kamino_fail(KAMINO_ERR_INVALID, "radius must be > 0");
    const int np = 2 * nt, L = spec->lmax, W = L + 1;
    const double h = M_PI / nt, R = spec->radius;

    // stream-function coefficients, orthonormal real harmonics, l = 1..L
    std::vector<double> ca((size_t)W * W, 0.0), cb((size_t)W * W, 0.0);
    {
        Rng rng(stream_seed(spec->seed, STREAM_SH));
        for (int l = 1; l <= L; l++)
            for (int m = 0; m <= l; m++) {
                double s = m ? std::sqrt(2.0) : 1.0;
                ca[(size_t)l * W + m] = s * rng.normal();
                cb[(size_t)l * W + m] = m ? s * rng.normal() : 0.0;
            }
    }
    double vth = 0, vph = 0, vamp = 0, vsig = spec->vortex_sigma;
    if (spec->vortex) {
        Rng rng(stream_seed(spec->seed, STREAM_VORTEX));
        vth = std::acos(1.0 - 2.0 * rng.uniform());
        vph = 2.0 * M_PI * rng.uniform();
        double a = 0.5 + rng.uniform(); // peak swirl speed in [0.5, 1.5)
        if (rng.uniform() < 0.5) a = -a;
        // psi = A exp((cos d - 1)/sigma^2) has peak speed ~ A e^{-1/2}/sigma
        vamp = spec->vortex_amplitude != 0.0 ? spec->vortex_amplitude : a * vsig * std::exp(0.5);
        if (!(vsig > 0)) return kamino_fail(KAMINO_ERR_INVALID, "vortex_sigma must be > 0");
    }

    // d psi / d theta and d psi / d phi at (theta, phi)
    auto row_coeffs = [&](double theta, std::vector<double>& Ac, std::vector<double>& As,
                          std::vector<double>& dAc, std::vector<double>& dAs) {
        std::vector<double> P, dP;
        legendre(L, theta, P, dP);
        Ac.assign(W, 0.0);
        As.assign(W, 0.0);
        dAc.assign(W, 0.0);
        dAs.assign(W, 0.0);
        for (int m = 0; m <= L; m++)
            for (int l = std::max(m, 1); l <= L; l++) {
                size_t k = (size_t)l * W + m;
                Ac[m] += ca[k] * P[k];
                As[m] += cb[k] * P[k];
                dAc[m] += ca[k] * dP[k];
                dAs[m] += cb[k] * dP[k];
            }
    };
    auto vortex_grad = [&](double theta, double phi, double& dth, double& dph) {
        double ct = std::cos(theta), st = std::sin(theta);
        double cc = std::cos(vth), sc = std::sin(vth);
        double dp = phi - vph;
        double cosd = ct * cc + st * sc * std::cos(dp);
        double psi = vamp * std::exp((cosd - 1.0) / (vsig * vsig));
        dth = psi / (vsig * vsig) * (-st * cc + ct * sc * std::cos(dp));
        dph = psi / (vsig * vsig) * (-st * sc * std::sin(dp));
    };

    std::vector<double> up((size_t)nt * np), vt((size_t)(nt - 1) * np);
    // u_phi = -(1/R) d psi/d theta at (phi=(i-1/2)h, theta=(j+1/2)h)
    // u_theta = (1/(R sin theta)) d psi/d phi at (phi=i h, theta=(j+1)h)
#pragma omp parallel for schedule(dynamic)
    for (int j = 0; j < 2 * nt - 1; j++) {
        bool isu = j < nt;
        int row = isu ? j : j - nt;
        double theta = isu ? (row + 0.5) * h : (row + 1.0) * h;
        std::vector<double> Ac, As, dAc, dAs;
        row_coeffs(theta, Ac, As, dAc, dAs);
        for (int i = 0; i < np; i++) {
            double phi = isu ? (i - 0.5) * h : i * h;
            double dth = 0, dph = 0;
            for (int m = 0; m <= L; m++) {
                double cm = std::cos(m * phi), sm = std::sin(m * phi);
                dth += dAc[m] * cm + dAs[m] * sm;
                dph += m * (-Ac[m] * sm + As[m] * cm);
            }
            if (spec->vortex) {
                double a, b;
                vortex_grad(theta, phi, a, b);
                dth += a;
                dph += b;
            }
            if (isu)
                up[(size_t)row * np + i] = -dth / R;
            else
                vt[(size_t)row * np + i] = dph / (R * std::sin(theta));
        }
    }
    double scale = 1.0;
    if (spec->velocity_scale > 0) {
        double mx = 0;
        for (double x : up) mx = std::max(mx, std::fabs(x));
        for (double x : vt) mx = std::max(mx, std::fabs(x));
        if (mx > 0) scale = spec->velocity_scale / mx;
    }
    if (u_phi)
        for (size_t k = 0; k < up.size(); k++) u_phi[k] = (float)(up[k] * scale);
    if (u_theta)
        for (size_t k = 0; k < vt.size(); k++) u_theta[k] = (float)(vt[k] * scale);
    if (thickness) {
        Rng rng(stream_seed(spec->seed, STREAM_THICK));
        for (size_t k = 0; k < (size_t)nt * np; k++)
            thickness[k] = (float)(1.0 + spec->thickness_noise * (2.0 * rng.uniform() - 1.0));
    }
    if (particles && spec->n_particles > 0) {
        Rng rng(stream_seed(spec->seed, STREAM_PART));
        for (int64_t k = 0; k < spec->n_particles; k++) {
            double th = std::acos(1.0 - 2.0 * rng.uniform());
            double ph = 2.0 * M_PI * rng.uniform();
            particles[2 * k] = (float)ph;
            particles[2 * k + 1] = (float)th;
        }
    }
    spec->vortex_out[0] = vth;
    spec->vortex_out[1] = vph;
    spec->vortex_out[2] = vamp * scale;
    return KAMINO_OK;
}

// Steps Kamino::run takes for `frames` frames (KaminoCore.cu:886-895): per
// frame, while T < i*DT one step and T += dt, then one remainder step, all in
// float as the reference does.
extern "C" int64_t kamino_frame_steps(double dt, double frame_dt, int frames)
{
    const float fdt = (float)dt, DT = (float)frame_dt;
    if (!(fdt > 0) || !(DT > 0) || frames < 0) return -1;
    int64_t total = 0;
    float T = 0.0f;
    for (int i = 1; i <= frames; i++) {
        while (T < i * DT) {
            total++;
            T += fdt;
        }
        total++;
        T = i * DT;
    }
    return total;
}

// sizeof of the ABI structs, for binding checks: config, init spec, server
// config, server stats.
extern "C" int kamino_abi_sizes(size_t* out, int n)
{
    const size_t s[4] = {sizeof(kamino_config), sizeof(kamino_init_spec), sizeof(kamino_server_config),
                         sizeof(kamino_server_stats)};
    if (!out) return KAMINO_ERR_INVALID;
    for (int i = 0; i < n && i < 4; i++) out[i] = s[i];
    return KAMINO_OK;
}

// KaminoSolver::initParticlesfromPic without an image (KaminoSolver.cu:
// 278-281): the reference's particle placement, uploaded to the handle.
extern "C" int kamino_init_particles(kamino_handle h, uint32_t seed)
{
    kamino_config cfg;
    int rc = kamino_internal_config(h, &cfg);
    if (rc) return rc;
    const int64_t n = kamino_particle_count(&cfg);
    if (n == 0) return KAMINO_OK;
    std::vector<float> buf(2 * (size_t)n);
    if ((rc = kamino_reference_particles(&cfg, seed, buf.data(), n))) return rc;
    return kamino_set_state(h, KAMINO_PARTICLES, buf.data(), 0);
}

// ------------------------------------------------------- checkpoint / resume
// A raw dump of one sphere's state, for resuming a run; the reference has no
// counterpart (its .bgeo frames are write-only).  Layout, native little-endian:
//   char[8] "KAMINOS1", int32 n_theta, int32 flags, int64 n_particles,
//   double radius, double dt, int64 steps, double time,
//   float u_phi[nt][2nt], u_theta[nt-1][2nt], thickness[nt][2nt],
//   float particles[n][2], uint64 FNV-1a hash of every byte before it.
namespace {

struct StateHeader {
    char magic[8];
    int32_t n_theta;
    uint32_t flags;
    int64_t n_particles;
    double radius, dt;
    int64_t steps;
    double time;
};
static_assert(sizeof(StateHeader) == 56, "state header layout");

constexpr char kStateMagic[8] = {'K', 'A', 'M', 'I', 'N', 'O', 'S', '1'};

uint64_t fnv1a(const void* p, size_t n, uint64_t hsh)
{
    const unsigned char* c = (const unsigned char*)p;
    for (size_t k = 0; k < n; k++) hsh = (hsh ^ c[k]) * 0x100000001b3ull;
    return hsh;
}

constexpr uint64_t kFnvBasis = 0xcbf29ce484222325ull;

}  // namespace

extern "C" int kamino_save_state(kamino_handle h, const char* path)
{
    kamino_config cfg;
    int rc = kamino_internal_config(h, &cfg);
    if (rc) return rc;
    if (!path) return kamino_fail(KAMINO_ERR_INVALID, "kamino_save_state: null path");
    StateHeader hd;
    std::memcpy(hd.magic, kStateMagic, 8);
    hd.n_theta = cfg.n_theta;
    hd.flags = cfg.flags;
    hd.n_particles = kamino_particle_count(&cfg);
    hd.radius = cfg.radius;
    hd.dt = cfg.dt;
    int cu, cr;
    if ((rc = kamino_internal_get_counters(h, &cu, &cr, &hd.steps, &hd.time))) return rc;
    const size_t np = 2 * (size_t)cfg.n_theta, nt = (size_t)cfg.n_theta;
    std::vector<float> data(np * nt + np * (nt - 1) + np * nt + 2 * (size_t)hd.n_particles);
    float* p = data.data();
    if ((rc = kamino_get_state(h, KAMINO_U_PHI, p, 0)) || (rc = kamino_get_state(h, KAMINO_U_THETA, p + np * nt, 0)) ||
        (rc = kamino_get_state(h, KAMINO_THICKNESS, p + np * (2 * nt - 1), 0)))
        return rc;
    if (hd.n_particles && (rc = kamino_get_state(h, KAMINO_PARTICLES, p + np * (3 * nt - 1), 0))) return rc;
    const uint64_t sum = fnv1a(data.data(), sizeof(float) * data.size(), fnv1a(&hd, sizeof(hd), kFnvBasis));
    FILE* fp = std::fopen(path, "wb");
    if (!fp) return kamino_fail(KAMINO_ERR_IO, "cannot open %s for writing", path);
    bool ok = std::fwrite(&hd, sizeof(hd), 1, fp) == 1 &&
              std::fwrite(data.data(), sizeof(float), data.size(), fp) == data.size() &&
              std::fwrite(&sum, sizeof(sum), 1, fp) == 1;
    ok = (std::fclose(fp) == 0) && ok;
    if (!ok) return kamino_fail(KAMINO_ERR_IO, "short write to %s", path);
    return KAMINO_OK;
}

extern "C" int kamino_load_state(kamino_handle h, const char* path)
{
    kamino_config cfg;
    int rc = kamino_internal_config(h, &cfg);
    if (rc) return rc;
    if (!path) return kamino_fail(KAMINO_ERR_INVALID, "kamino_load_state: null path");
    FILE* fp = std::fopen(path, "rb");
    if (!fp) return kamino_fail(KAMINO_ERR_IO, "cannot open %s", path);
    StateHeader hd;
    const size_t np = 2 * (size_t)cfg.n_theta, nt = (size_t)cfg.n_theta;
    const int64_t npart = kamino_particle_count(&cfg);
    std::vector<float> data(np * nt + np * (nt - 1) + np * nt + 2 * (size_t)npart);
    uint64_t sum = 0;
    bool ok = std::fread(&hd, sizeof(hd), 1, fp) == 1 && std::memcmp(hd.magic, kStateMagic, 8) == 0;
    if (ok && (hd.n_theta != cfg.n_theta || hd.n_particles != npart)) {
        std::fclose(fp);
        return kamino_fail(KAMINO_ERR_INVALID, "%s holds nTheta %d with %lld particles; the handle has %d and %lld",
                           path, hd.n_theta, (long long)hd.n_particles, cfg.n_theta, (long long)npart);
    }
    ok = ok && std::fread(data.data(), sizeof(float), data.size(), fp) == data.size() &&
         std::fread(&sum, sizeof(sum), 1, fp) == 1 && std::fgetc(fp) == EOF;
    std::fclose(fp);
    if (!ok) return kamino_fail(KAMINO_ERR_IO, "%s is not a complete state file", path);
    if (sum != fnv1a(data.data(), sizeof(float) * data.size(), fnv1a(&hd, sizeof(hd), kFnvBasis)))
        return kamino_fail(KAMINO_ERR_IO, "%s: checksum mismatch", path);
    if (hd.radius != cfg.radius || hd.dt != cfg.dt)
        return kamino_fail(KAMINO_ERR_INVALID, "%s: radius %g, dt %g; the handle has radius %g, dt %g", path,
                           hd.radius, hd.dt, cfg.radius, cfg.dt);
    // the switches that change the trajectory must match too
    const uint32_t traj = KAMINO_F_PARTICLE_RK2 | KAMINO_F_POLE_SIGN_FLIP | KAMINO_F_HONOR_STEP_DT |
                          KAMINO_F_REFERENCE_ROUNDING;
    if ((hd.flags & traj) != (cfg.flags & traj))
        return kamino_fail(KAMINO_ERR_INVALID, "%s: saved with flags 0x%x; the handle has 0x%x", path,
                           hd.flags & traj, cfg.flags & traj);
    const float* p = data.data();
    if ((rc = kamino_set_state(h, KAMINO_U_PHI, p, 0)) || (rc = kamino_set_state(h, KAMINO_U_THETA, p + np * nt, 0)) ||
        (rc = kamino_set_state(h, KAMINO_THICKNESS, p + np * (2 * nt - 1), 0)))
        return rc;
    if (npart && (rc = kamino_set_state(h, KAMINO_PARTICLES, p + np * (3 * nt - 1), 0))) return rc;
    int cu, cr;
    if ((rc = kamino_internal_get_counters(h, &cu, &cr, nullptr, nullptr))) return rc;
    return kamino_internal_set_counters(h, cu, cr, hd.steps, hd.time);
}
